// rf_trace_accurate.cu — the ghost-path trace with its geometry in double precision.
//
// The reference's trace in FP32 (rf_trace, bit-identical to the reference's kernel) leaves
// ray positions a few units in the last place from the same trace evaluated exactly, and the
// rasteriser is discontinuous in them: it truncates positions to integer sample coordinates
// (rasterizing.cl:624) and special-cases zero cross products (rasterizing.cl:127-130), so a
// position one ulp away can move a quad corner across a sample and change whole pixels. On
// lenses of 16 and more strongly curved surfaces this puts the FP32 image about 1e-3
// (relative L2) from the image of the same algorithm in double. This trace evaluates
// everything that determines where a ray goes in double: the grid point, the light
// direction, intersect (raytracing.cl:123-175), refract and reflect (70-102), dispersion
// (107-120), the aperture position and rrel. Only the outputs are rounded to float, so
// positions equal those of the double evaluation rounded to float. The coating and Fresnel
// reflectances (1-59) stay in FP32: they scale intensities continuously and cannot move a
// pixel. Compiled without fused multiply-adds, the double arithmetic is the oracle's
// double build operation for operation (IEEE double division and square root).
//
// One thread per ray as in rf_trace; lens elements and the (wavelength, element) indices of
// the block's rows in shared memory (double). Double throughput on this part is a small
// fraction of FP32, so this is an opt-in mode.
#include <math.h>

#include "rf_trace_core.cuh"

namespace rf {
namespace {

constexpr int kAccRows = 8;  // wavelength rows of the per-block index table

struct AccParams {
    long long n_rays;
    int E, aperture, P, W, G, R;
    float cmin, layer_n0, layer_n1;
    float grid_length;
    double dir[3];  // normalize(-direction.xyz) in double
};

struct AccElement {
    double radius, center, height, ior;
    int coating, layers;
    float d0, d1;
};

struct AccHit {
    double px, py, pz, nx, ny, nz;
    bool hit;
};

// intersect (raytracing.cl:123-175) in double, the incident angle left to the caller
__device__ __forceinline__ AccHit intersect_d(double px, double py, double pz, double dx, double dy, double dz,
                                              const AccElement& e) {
    AccHit h;
    h.px = h.py = h.pz = h.nx = h.ny = h.nz = 0.0;
    h.hit = false;
    if (dz == 0.0) return h;
    if (e.radius == 0.0) {
        const double t = (-e.center - pz) / dz;
        h.px = px + dx * t;
        h.py = py + dy * t;
        h.pz = pz + dz * t;
        h.nz = (dz < 0.0) ? 1.0 : -1.0;
        h.hit = true;
        return h;
    }
    const double r = fabs(e.radius);
    const double cz = -e.center;
    const double ux = 0.0 - px, uy = 0.0 - py, uz = cz - pz;
    const double proj = ux * dx + uy * dy + uz * dz;
    const double u1x = dx * proj, u1y = dy * proj, u1z = dz * proj;
    const double ex = ux - u1x, ey = uy - u1y, ez = uz - u1z;
    const double d = sqrt(ex * ex + ey * ey + ez * ez);
    if (d > r) return h;
    const double sgn = (e.radius * dz) > 0.0 ? -1.0 : 1.0;
    const double m = sqrt(r * r - d * d);
    h.px = (px + u1x) - (dx * m) * sgn;
    h.py = (py + u1y) - (dy * m) * sgn;
    h.pz = (pz + u1z) - (dz * m) * sgn;
    const double qx = h.px, qy = h.py, qz = h.pz - cz;
    const double inv = 1.0 / sqrt(qx * qx + qy * qy + qz * qz);
    h.nx = (qx * inv) * sgn;
    h.ny = (qy * inv) * sgn;
    h.nz = (qz * inv) * sgn;
    h.hit = true;
    return h;
}

// dispersion (raytracing.cl:107-120) in double
__device__ __forceinline__ double dispersion_d(float lambda, const float* c) {
    const double l = (double)lambda * 1e-3;
    const double l2 = l * l;
    const double d0 = ((double)c[0] * l2) / (l2 - (double)c[1]);
    const double d1 = ((double)c[2] * l2) / (l2 - (double)c[3]);
    const double d2 = ((double)c[4] * l2) / (l2 - (double)c[5]);
    return sqrt(1.0 + d0 + d1 + d2);
}

__global__ void __launch_bounds__(kTraceThreads) k_trace_accurate(const rf_lens_element* __restrict__ elements,
                                                                  const int2* __restrict__ paths,
                                                                  const float* __restrict__ wavelengths,
                                                                  const __grid_constant__ AccParams p,
                                                                  float* __restrict__ rays) {
    __shared__ AccElement se[kMaxElements];
    __shared__ double ior_tab[kAccRows * kMaxElements];
    const int E = p.E;
    const long long first = (long long)blockIdx.x * kTraceThreads;
    const long long last = min(first + kTraceThreads, p.n_rays) - 1;
    const long long pw_first = first / p.R, pw_last = last / p.R;
    const long long span_rows = pw_last - pw_first + 1;
    const int span = (int)(span_rows < (long long)p.W ? span_rows : (long long)p.W);
    const bool table = span <= kAccRows;
    const bool disperse = !isnan(__ldg(&elements[0].coefficients[0]));
    for (int i = threadIdx.x; i < E; i += kTraceThreads) {
        const rf_lens_element& e = elements[i];
        se[i].radius = e.radius;
        se[i].center = e.center;
        se[i].height = e.height;
        se[i].ior = e.ior;
        se[i].coating = e.coating;
        se[i].layers = e.coating_layers;
        se[i].d0 = e.coating_thickness[0];
        se[i].d1 = e.coating_thickness[1];
    }
    if (table) {
        for (int k = threadIdx.x; k < span * E; k += kTraceThreads) {
            const int row = k / E, el = k % E;
            const int wl = (int)((pw_first + row) % p.W);
            double n = elements[el].ior;
            if (disperse && n > 1.0) n = dispersion_d(wavelengths[wl], elements[el].coefficients);
            ior_tab[row * E + el] = n;
        }
    }
    __syncthreads();

    const long long idx = first + threadIdx.x;
    if (idx >= p.n_rays) return;
    const int ray_id = (int)(idx % p.R);
    const long long pw = idx / p.R;
    const int wl_id = (int)(pw % p.W);
    const int path_id = (int)(pw / p.W);
    const int row = (int)((pw - pw_first) % p.W);
    const float wavelength = __ldg(wavelengths + wl_id);
    const int2 path = __ldg(paths + path_id);
    auto ior_of = [&](int el) -> double {
        if (table) return ior_tab[row * E + el];
        double n = se[el].ior;
        if (disperse && n > 1.0) n = dispersion_d(wavelength, elements[el].coefficients);
        return n;
    };

    // init_ray (raytracing.cl:178-215): the grid point in double, as the reference's
    // double expression grid_length * (x / (G - 1) - 0.5) gives it before any rounding
    const int gy = (int)truncf((float)ray_id / (float)p.G);
    const int gx = ray_id - gy * p.G;
    const float fx = (float)gx / (float)(p.G - 1), fy = (float)gy / (float)(p.G - 1);
    double px = (double)p.grid_length * ((double)fx - 0.5);
    double py = (double)p.grid_length * (0.5 - (double)fy);
    double pz = 1.0;
    {
        const AccHit h0 = intersect_d(px, py, pz, 0.0, 0.0, -1.0, se[0]);
        px = h0.px;  // zero when the grid point misses element 0
        py = h0.py;
        pz = h0.pz;
    }
    double dx = p.dir[0], dy = p.dir[1], dz = p.dir[2];
    px = px - dx;
    py = py - dy;
    pz = pz - dz;
    double apt_x = 0.0, apt_y = 0.0, rrel = 0.0;
    float refl = 1.0f;

    int step = 0, delta = 1;
    int lens_id;
    for (lens_id = 0; lens_id >= 0 && lens_id < E; lens_id += delta) {
        const AccElement& e = se[lens_id];
        const AccHit h = intersect_d(px, py, pz, dx, dy, dz, e);
        if (!h.hit) break;
        px = h.px;
        py = h.py;
        pz = h.pz;
        if (lens_id == p.aperture) {
            apt_x = h.px / e.height;
            apt_y = h.py / e.height;
            continue;
        }
        rrel = fmax(rrel, sqrt(h.px * h.px + h.py * h.py) / e.height);
        if (lens_id == E - 1) continue;
        bool do_reflect = false;
        if ((step == 0 && lens_id == path.x) || (step == 1 && lens_id == path.y)) {
            do_reflect = true;
            step++;
            delta = -delta;
        }
        const int n_index = (dz < 0.0) ? lens_id - 1 : lens_id + 1;
        const double n1 = (0 <= n_index && n_index < E) ? ior_of(n_index) : 1.0;
        const double n2 = ior_of(lens_id);
        if (do_reflect) {
            double c = -dx * h.nx + -dy * h.ny + -dz * h.nz;
            c = fmin(fmax(c, -1.0), 1.0);
            const double theta_d = acos(c) + 1e-9;
            // reflect, raytracing.cl:96-102
            const double k = 2.0 * (h.nx * -dx + h.ny * -dy + h.nz * -dz);
            dx = dx + h.nx * k;
            dy = dy + h.ny * k;
            dz = dz + h.nz * k;
            const float theta = (float)theta_d, fn1 = (float)n1, fn2 = (float)n2;
            float reflectance;
            if (e.layers == 2) {
                reflectance = fresnel_two_layer(theta, wavelength, fn1, p.layer_n0, e.d0, p.layer_n1, e.d1, fn2);
            } else if (e.layers == 1 || e.coating > 0) {
                const float nc = fmaxf(sqrtf(fn1 * fn2), p.cmin);
                const float d1 = e.layers == 1 ? e.d0 : (float)e.coating / (4.0f * nc);
                reflectance = fresnel_ar(theta, wavelength, d1, fn1, nc, fn2);
            } else {
                reflectance = fresnel(theta, fn1, fn2);
            }
            if (reflectance > 0.0f) refl *= reflectance;
        } else {
            // refract, raytracing.cl:70-86
            const double o = n1 / n2;
            const double cost = -dx * h.nx + -dy * h.ny + -dz * h.nz;
            const double sint2 = (o * o) * (1.0 - cost * cost);
            const double k = o * cost - sqrt(fabs(1.0 - sint2));
            const double valid = (double)(sint2 < 1.0);
            dx = (dx * o + h.nx * k) * valid;
            dy = (dy * o + h.ny * k) * valid;
            dz = (dz * o + h.nz * k) * valid;
            if (dz == 0.0) break;
        }
    }
    if (lens_id >= 0 && lens_id < E) refl = __int_as_float(0x7fffffff);
    const long long n = p.n_rays;
    rays[0 * n + idx] = (float)px;
    rays[1 * n + idx] = (float)py;
    rays[2 * n + idx] = (float)apt_x;
    rays[3 * n + idx] = (float)apt_y;
    rays[4 * n + idx] = (float)rrel;
    rays[5 * n + idx] = refl;
}

}  // namespace
}  // namespace rf

extern "C" int rf_trace_accurate(const rf_lens_element* elements, const int32_t* paths, const float* wavelengths,
                                 const rf_trace_args* args, float* rays, void* stream) {
    using namespace rf;
    if (!elements || !paths || !wavelengths || !args || !rays) return RF_ERR_INVALID_ARG;
    const rf_trace_args& a = *args;
    if (a.element_count < 2 || a.element_count > kMaxElements || a.path_count < 0 || a.wavelength_count < 1 ||
        a.grid_count < 2 || a.grid_count > kMaxGrid || a.aperture_index < 0)
        return RF_ERR_INVALID_ARG;
    AccParams p;
    p.R = a.grid_count * a.grid_count;
    p.n_rays = (long long)a.path_count * a.wavelength_count * p.R;
    p.E = a.element_count;
    p.aperture = a.aperture_index;
    p.P = a.path_count;
    p.W = a.wavelength_count;
    p.G = a.grid_count;
    p.cmin = a.coating_min_ior;
    p.layer_n0 = a.coating_layer_ior[0];
    p.layer_n1 = a.coating_layer_ior[1];
    p.grid_length = a.grid_length;
    // normalize(direction.xyz * -1) in double: the reciprocal length, then three products
    const double vx = -(double)a.direction[0], vy = -(double)a.direction[1], vz = -(double)a.direction[2];
    const double inv = 1.0 / sqrt(vx * vx + vy * vy + vz * vz);
    p.dir[0] = vx * inv;
    p.dir[1] = vy * inv;
    p.dir[2] = vz * inv;
    if (p.n_rays == 0) return RF_OK;
    k_trace_accurate<<<blocks_for(p.n_rays, kTraceThreads), kTraceThreads, 0, (cudaStream_t)stream>>>(
        elements, (const int2*)paths, wavelengths, p, rays);
    return launch_status();
}
