// rf_trace_core.cuh — per-ray trace code shared by the trace (rf_trace.cu) and its adjoint
// (rf_adjoint.cu). Both translation units are compiled without floating-point contraction,
// so a ray recomputed by the adjoint follows the forward trace's arithmetic exactly.
//
// Follows realflare/api/tasks/cl/raytracing.cl: init_ray (178-215), the element loop of
// raytrace (218-359), intersect (123-175), refract / reflect (70-102), dispersion
// (107-120), fresnel (1-16) and fresnel_ar (18-59).
#pragma once

#include <math.h>

#include "rf_common.cuh"

namespace rf {
namespace {

constexpr int kTraceThreads = 256;
constexpr int kMaxElements = 128;
constexpr int kMaxGrid = 2048;  // (float)ray_id / G is exact enough for trunc() up to 2048
constexpr int kMaxTableWavelengths = 64;  // per block; larger spans fall back to global

struct TraceParams {
    long long n_rays;
    int E, aperture, P, W, G, R;
    float cmin, layer_n0, layer_n1;
    float dir[3];        // normalize(-direction.xyz), host-computed in FP32
    float grid[kMaxGrid];  // grid_length * ((float)i / (G - 1) - 0.5), rounded from double
};

struct SmemElement {
    float radius, center, height, ior;
    int coating, layers;
    float d0, d1;
};

struct Hit {
    float px, py, pz, nx, ny, nz, incident;
    bool hit;
};

// Inlining of the reflection-only functions (RF_CORE_COLD: the Fresnel variants) and of the
// sphere/plane intersection (RF_CORE_HOT); a unit may define them __noinline__ before
// including this file (same arithmetic either way: nothing is contracted across calls).
#ifndef RF_CORE_COLD
#define RF_CORE_COLD __forceinline__
#endif
#ifndef RF_CORE_HOT
#define RF_CORE_HOT __forceinline__
#endif
__device__ RF_CORE_HOT Hit intersect(float px, float py, float pz, float dx, float dy, float dz,
                                         const SmemElement& e) {
    Hit h;
    h.px = h.py = h.pz = h.nx = h.ny = h.nz = h.incident = 0.0f;
    h.hit = false;
    if (dz == 0.0f) return h;
    if (e.radius == 0.0f) {
        float t = (-e.center - pz) / dz;
        h.px = px + dx * t;
        h.py = py + dy * t;
        h.pz = pz + dz * t;
        h.nx = 0.0f;
        h.ny = 0.0f;
        h.nz = (dz < 0.0f) ? 1.0f : -1.0f;
        h.hit = true;
        h.incident = 0.0f;
        return h;
    }
    float r = fabsf(e.radius);
    float cz = -e.center;
    float ux = 0.0f - px, uy = 0.0f - py, uz = cz - pz;
    float proj = ux * dx + uy * dy + uz * dz;
    float u1x = dx * proj, u1y = dy * proj, u1z = dz * proj;
    float ex = ux - u1x, ey = uy - u1y, ez = uz - u1z;
    float d = sqrtf(ex * ex + ey * ey + ez * ez);
    if (d > r) return h;
    float sgn = (e.radius * dz) > 0.0f ? -1.0f : 1.0f;
    float m = sqrtf(r * r - d * d);
    h.px = (px + u1x) - (dx * m) * sgn;
    h.py = (py + u1y) - (dy * m) * sgn;
    h.pz = (pz + u1z) - (dz * m) * sgn;
    float qx = h.px, qy = h.py, qz = h.pz - cz;
    float inv = 1.0f / sqrtf(qx * qx + qy * qy + qz * qz);
    h.nx = (qx * inv) * sgn;
    h.ny = (qy * inv) * sgn;
    h.nz = (qz * inv) * sgn;
    h.incident = 0.0f;  // acos of the incidence cosine, needed only at reflections
    h.hit = true;
    return h;
}

__device__ __forceinline__ float incident_angle(float dx, float dy, float dz, const Hit& h) {
    float c = -dx * h.nx + -dy * h.ny + -dz * h.nz;
    return acosf(clampf(c, -1.0f, 1.0f));
}

__device__ RF_CORE_COLD float fresnel(float theta0, float n1, float n2) {
    float theta1 = asinf(sinf(theta0) * n1 / n2);
    float cosi = cosf(theta0);
    float cost = cosf(theta1);
    float rs = ((n1 * cosi) - (n2 * cost)) / ((n1 * cosi) + (n2 * cost));
    float rp = ((n1 * cost) - (n2 * cosi)) / ((n1 * cost) + (n2 * cosi));
    return (rs * rs + rp * rp) / 2.0f;
}

__device__ RF_CORE_COLD float fresnel_ar(float theta0, float lambda, float d1, float n0, float n1, float n2) {
    float s0 = sinf(theta0);
    float theta1 = asinf(s0 * n0 / n1);
    float theta2 = asinf(s0 * n0 / n2);
    float rs01 = -sinf(theta0 - theta1) / sinf(theta0 + theta1);
    float rp01 = tanf(theta0 - theta1) / tanf(theta0 + theta1);
    float ts01 = 2.0f * sinf(theta1) * cosf(theta0) / sinf(theta0 + theta1);
    float tp01 = ts01 * cosf(theta0 - theta1);
    float rs12 = -sinf(theta1 - theta2) / sinf(theta1 + theta2);
    float rp12 = tanf(theta1 - theta2) / tanf(theta1 + theta2);
    float ris = ts01 * ts01 * rs12;
    float rip = tp01 * tp01 * rp12;
    float dy = d1 * n1;
    float dx = tanf(theta1) * dy;
    float delay = sqrtf(dx * dx + dy * dy);
    float rel_phase = 4.0f * RF_MPI_F / lambda * (delay - dx * s0);
    float c = cosf(rel_phase);
    float out_s2 = rs01 * rs01 + ris * ris + 2.0f * rs01 * ris * c;
    float out_p2 = rp01 * rp01 + rip * rip + 2.0f * rp01 * rip * c;
    return (out_s2 + out_p2) / 2.0f;
}

// Exact two-layer thin-film reflectance (no reference counterpart; the same definition as
// the oracle): incident medium n0 | layer a | layer b | substrate n2, s/p averaged.
__device__ __forceinline__ void interface_r(float ni, float ci, float nj, float cj, float& rs, float& rp) {
    rs = (ni * ci - nj * cj) / (ni * ci + nj * cj);
    rp = (nj * ci - ni * cj) / (nj * ci + ni * cj);
}
__device__ __forceinline__ float stack_r2(float r01, float r12, float r23, float d1, float d2) {
    float s2, c2, s1, c1;
    sincosf(d2, &s2, &c2);
    sincosf(d1, &s1, &c1);
    float nre = r12 + r23 * c2, nim = r23 * s2;
    float dre = 1.0f + r12 * r23 * c2, dim = r12 * r23 * s2;
    float den = dre * dre + dim * dim;
    float ire = (nre * dre + nim * dim) / den;
    float iim = (nim * dre - nre * dim) / den;
    float ere = ire * c1 - iim * s1, eim = ire * s1 + iim * c1;
    float tre = r01 + ere, tim = eim;
    float bre = 1.0f + r01 * ere, bim = r01 * eim;
    return (tre * tre + tim * tim) / (bre * bre + bim * bim);
}
__device__ RF_CORE_COLD float fresnel_two_layer(float theta0, float lambda, float n0, float na, float da,
                                                   float nb, float db, float n2) {
    float s0, c0;
    sincosf(theta0, &s0, &c0);
    float sa = n0 * s0 / na, sb = n0 * s0 / nb, s2 = n0 * s0 / n2;
    float ca = sqrtf(1.0f - sa * sa), cb = sqrtf(1.0f - sb * sb), c2 = sqrtf(1.0f - s2 * s2);
    float rs01, rp01, rs12, rp12, rs23, rp23;
    interface_r(n0, c0, na, ca, rs01, rp01);
    interface_r(na, ca, nb, cb, rs12, rp12);
    interface_r(nb, cb, n2, c2, rs23, rp23);
    float phase = 4.0f * RF_MPI_F / lambda;
    float d1 = phase * na * da * ca;
    float d2 = phase * nb * db * cb;
    return (stack_r2(rs01, rs12, rs23, d1, d2) + stack_r2(rp01, rp12, rp23, d1, d2)) / 2.0f;
}

// dispersion, raytracing.cl:107-120 (lambda * 1e-3 is a double expression there)
__device__ __forceinline__ float dispersion(float lambda, const float* c) {
    float l = (float)((double)lambda * 1e-3);
    float l2 = l * l;
    float d0 = (c[0] * l2) / (l2 - c[1]);
    float d1 = (c[2] * l2) / (l2 - c[3]);
    float d2 = (c[4] * l2) / (l2 - c[5]);
    return sqrtf(1.0f + d0 + d1 + d2);
}

// reflect (raytracing.cl:96-102): d + n * 2 (n . -d)
__device__ __forceinline__ void reflect_dir(float& dx, float& dy, float& dz, const Hit& h) {
    float k = 2.0f * (h.nx * -dx + h.ny * -dy + h.nz * -dz);
    dx = dx + h.nx * k;
    dy = dy + h.ny * k;
    dz = dz + h.nz * k;
}

// refract (raytracing.cl:70-86) with o = n1 / n2; the direction is zeroed past total
// internal reflection
__device__ __forceinline__ void refract_dir(float& dx, float& dy, float& dz, const Hit& h, float n1, float n2) {
    const float o = n1 / n2;
    const float cost = -dx * h.nx + -dy * h.ny + -dz * h.nz;
    const float sint2 = (o * o) * (1.0f - cost * cost);
    const float k = o * cost - sqrtf(fabsf(1.0f - sint2));
    const float valid = (float)(sint2 < 1.0f);
    dx = (o * dx + k * h.nx) * valid;
    dy = (o * dy + k * h.ny) * valid;
    dz = (o * dz + k * h.nz) * valid;
}

// Per-frame constants of the trace.
struct TraceFrame {
    int E, aperture, W, G, R;
    float cmin, layer_n0, layer_n1;
    float dir[3];  // normalize(-direction.xyz), host-computed in FP32
};

// Observer of a traced ray: step() sees the ray entering each element (element index,
// position, direction), hit() each successful intersection (loop step index, the hit, the
// incoming direction, whether the element is flat), rrel() each candidate of the running
// maximum before it is taken, reflect() each reflection. The adjoint records steps, the
// intersection trace records hits; the forward trace uses NoRecord (inlined away).
struct NoRecord {
    __device__ __forceinline__ void step(int, float, float, float, float, float, float) {}
    __device__ __forceinline__ void hit(int, const Hit&, float, float, float, bool) {}
    __device__ __forceinline__ void rrel(float, float) {}
    __device__ __forceinline__ void reflect() {}
};

// One ray: init_ray (raytracing.cl:178-215) from grid point (grid_x, grid_y), then the
// element loop of raytrace (218-359). ior_row: this ray's wavelength row of the (wavelength,
// element) index table in shared memory, or nullptr to evaluate dispersion per element.
template <class Recorder>
__device__ __forceinline__ void trace_ray_rec(const SmemElement* __restrict__ se, const float* ior_row, bool disperse,
                                              const float* __restrict__ coef_base, float wavelength, int2 path,
                                              float grid_x, float grid_y, const TraceFrame& f, float out[6],
                                              Recorder& rec) {
    const int E = f.E;
    auto ior_of = [&](int el) -> float {
        if (ior_row) return ior_row[el];
        float n = se[el].ior;
        if (disperse && n > 1.0f) n = dispersion(wavelength, coef_base + (size_t)el * 16);
        return n;
    };

    float px = grid_x, py = -grid_y, pz = 1.0f;
    {
        Hit h0 = intersect(px, py, pz, 0.0f, 0.0f, -1.0f, se[0]);
        px = h0.px;  // zero when the grid point misses element 0
        py = h0.py;
        pz = h0.pz;
    }
    float dx = f.dir[0], dy = f.dir[1], dz = f.dir[2];
    px = px - dx;
    py = py - dy;
    pz = pz - dz;
    float apt_x = 0.0f, apt_y = 0.0f, rrel = 0.0f, refl = 1.0f;

    int step = 0, delta = 1;
    int lens_id, inter_id = 0;  // inter_id: loop steps so far (raytracing.cl:256)
    for (lens_id = 0; lens_id >= 0 && lens_id < E; lens_id += delta, inter_id++) {
        const SmemElement& e = se[lens_id];
        rec.step(lens_id, px, py, pz, dx, dy, dz);
        Hit h = intersect(px, py, pz, dx, dy, dz, e);
        if (!h.hit) break;
        rec.hit(inter_id, h, dx, dy, dz, e.radius == 0.0f);
        px = h.px;
        py = h.py;
        pz = h.pz;
        if (lens_id == f.aperture) {
            apt_x = h.px / e.height;
            apt_y = h.py / e.height;
            continue;
        }
        const float r_here = sqrtf(h.px * h.px + h.py * h.py) / e.height;
        rec.rrel(r_here, rrel);
        rrel = fmaxf(rrel, r_here);
        if (lens_id == E - 1) continue;
        bool do_reflect = false;
        if ((step == 0 && lens_id == path.x) || (step == 1 && lens_id == path.y)) {
            do_reflect = true;
            step++;
            delta = -delta;
        }
        const int n_index = (dz < 0.0f) ? lens_id - 1 : lens_id + 1;
        const float n1 = (0 <= n_index && n_index < E) ? ior_of(n_index) : 1.0f;
        const float n2 = ior_of(lens_id);
        if (do_reflect) {
            rec.reflect();
            const float incident = incident_angle(dx, dy, dz, h);
            reflect_dir(dx, dy, dz, h);
            // theta = incident + 1e-9 (a double sum there); only angles below 0.02 rad
            // are close enough to 1e-9 for the double sum to differ from `incident`
            float theta = incident < 0.02f ? (float)((double)incident + 1e-9) : incident;
            float reflectance;
            if (e.layers == 2) {
                reflectance = fresnel_two_layer(theta, wavelength, n1, f.layer_n0, e.d0, f.layer_n1, e.d1, n2);
            } else if (e.layers == 1 || e.coating > 0) {
                float nc = fmaxf(sqrtf(n1 * n2), f.cmin);
                float d1 = e.layers == 1 ? e.d0 : (float)e.coating / (4.0f * nc);
                reflectance = fresnel_ar(theta, wavelength, d1, n1, nc, n2);
            } else {
                reflectance = fresnel(theta, n1, n2);
            }
            if (reflectance > 0.0f) refl *= reflectance;
        } else {
            refract_dir(dx, dy, dz, h, n1, n2);
            if (dz == 0.0f) break;
        }
    }
    if (lens_id >= 0 && lens_id < E) refl = __int_as_float(0x7fffffff);
    out[0] = px;
    out[1] = py;
    out[2] = apt_x;
    out[3] = apt_y;
    out[4] = rrel;
    out[5] = refl;
}

__device__ __forceinline__ void trace_ray(const SmemElement* __restrict__ se, const float* ior_row, bool disperse,
                                          const float* __restrict__ coef_base, float wavelength, int2 path,
                                          float grid_x, float grid_y, const TraceFrame& f, float out[6]) {
    NoRecord none;
    trace_ray_rec(se, ior_row, disperse, coef_base, wavelength, path, grid_x, grid_y, f, out, none);
}

// Stage the lens elements and the refractive indices of wavelength rows [row0, row0 + span)
// (row r = wavelength (row0 + r) % W) in shared memory; table false: too many rows.
__device__ __forceinline__ void stage_lens(const rf_lens_element* __restrict__ elements, const float* __restrict__ wavelengths,
                                           int E, int W, long long row0, int span, bool table, bool disperse,
                                           SmemElement* se, float* ior_tab) {
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
            int row = k / E, el = k % E;
            int wl = (int)((row0 + row) % W);
            float n = elements[el].ior;
            if (disperse && n > 1.0f) n = dispersion(wavelengths[wl], elements[el].coefficients);
            ior_tab[row * E + el] = n;
        }
    }
}

// Kernel parameters of a trace (host): counts, coating constants, the light direction
// normalize(direction.xyz * -1) in FP32 without fused multiply-adds (the host code is
// compiled with -ffp-contract=off: the value the oracle computes) and the grid
// coordinates grid_length * (i / (G - 1) - 0.5), evaluated in double as the reference does.
inline bool trace_params(const rf_trace_args& a, TraceParams& p) {
    if (a.grid_count < 2 || a.grid_count > kMaxGrid) return false;
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
    float vx = -a.direction[0], vy = -a.direction[1], vz = -a.direction[2];
    float dd = vx * vx + vy * vy + vz * vz;
    float inv = 1.0f / sqrtf(dd);
    p.dir[0] = vx * inv;
    p.dir[1] = vy * inv;
    p.dir[2] = vz * inv;
    for (int i = 0; i < a.grid_count; i++) {
        float f = (float)i / (float)(a.grid_count - 1);
        p.grid[i] = (float)((double)a.grid_length * ((double)f - 0.5));
    }
    return true;
}

}  // namespace
}  // namespace rf
