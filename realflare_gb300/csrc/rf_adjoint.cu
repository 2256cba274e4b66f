// rf_adjoint.cu — reverse-mode derivative (adjoint) of the ghost ray trace.
//
// No reference counterpart: the reference has no differentiation. Given the gradient of a
// loss with respect to every traced ray's outputs (sensor position, aperture position,
// rrel, reflectance), rf_trace_adjoint returns the gradient with respect to every lens
// element's radius, center and coating thicknesses and to the (normalised) light direction.
//
// Rays whose outputs carry no gradient are skipped: each warp packs the others of its span
// of consecutive rays into full warps. Per ray, the thread re-traces the ray from its entry
// with the forward's own code
// (rf_trace_core.cuh, compiled like rf_trace.cu without floating-point contraction, so the
// re-trace takes the same path). It keeps only every kCheckpoint-th step's state (position
// and direction entering the element) and one byte per step (element, reflected or not);
// the reverse sweep goes back one segment of kCheckpoint steps at a time, re-tracing the
// segment from its checkpoint with the same step code to regenerate the states entering its
// elements, and recomputes each surface hit (point, normal) from them: no bounce is stored.
// The reverse sweep applies, element by element from the sensor back to the entry,
// the transposed Jacobians of intersect (sphere or plane), refract, reflect and the coating
// reflectance (the last by three-tangent forward-mode duals of the Fresnel formulas), then
// the entry ray (grid point hitting element 0, stepped back along the light direction).
// Rays that do not reach the sensor have no outputs and no gradient; the discrete choices
// (which element is hit, reflection or refraction, the rrel maximum) are those of the
// forward, i.e. the gradient is the derivative wherever they do not change.
// RF_ADJOINT_CALLS 1: the forward Fresnel variants out of line (the kernel's instruction
// fetches stall it more than anything else; 7.48 against 7.51 ms per forward+adjoint on the
// 16-surface differentiable workload); 2: the intersection too (7.54 ms)
#ifndef RF_ADJOINT_CALLS
#define RF_ADJOINT_CALLS 1
#endif
#if RF_ADJOINT_CALLS >= 1
#define RF_CORE_COLD __noinline__
#endif
#if RF_ADJOINT_CALLS >= 2
#define RF_CORE_HOT __noinline__
#endif
#include "rf_trace_core.cuh"

namespace rf {
namespace {

constexpr int kAdjThreads = 128;
// resident blocks per SM requested from the register allocator (8: 64 registers; the
// checkpoints and the segment's states live in local memory, and the spills cost less than
// the extra resident warps gain: 1.46 ms against 1.52 ms at 6 blocks and 1.67 ms at 4 on the
// 16-surface differentiable workload)
#ifndef RF_ADJOINT_MIN_BLOCKS
#define RF_ADJOINT_MIN_BLOCKS 8
#endif
constexpr int kAdjMaxElements = 32;
constexpr int kAdjMaxSteps = 3 * kAdjMaxElements;
// steps between stored states (segments re-traced in the reverse sweep)
#ifndef RF_ADJOINT_CHECKPOINT
#define RF_ADJOINT_CHECKPOINT 8
#endif
constexpr int kCheckpoint = RF_ADJOINT_CHECKPOINT;
constexpr int kMaxCheckpoints = (kAdjMaxSteps + kCheckpoint - 1) / kCheckpoint;
static_assert(kAdjMaxElements <= 128, "an element index and the reflection flag share one byte");
constexpr int kAdjTableRows = 4;
// consecutive rays a warp takes (a block: kAdjThreads / 32 such spans); the warp packs the
// rays whose outputs have a gradient into full warps before tracing them back
#ifndef RF_ADJOINT_WARP_RAYS
#define RF_ADJOINT_WARP_RAYS 128
#endif
constexpr int kAdjWarpRays = RF_ADJOINT_WARP_RAYS;
constexpr int kAdjBlockRays = kAdjThreads / 32 * kAdjWarpRays;
static_assert(kAdjWarpRays % 32 == 0, "whole warps of rays");
constexpr int kGradPerElement = 4;  // radius, center, coating thickness 0 and 1

// ---------------------------------------------------------------- three-tangent duals
struct D3 {
    float v, g0, g1, g2;
};
__device__ __forceinline__ D3 dconst(float v) { return {v, 0.f, 0.f, 0.f}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.v + b.v, a.g0 + b.g0, a.g1 + b.g1, a.g2 + b.g2}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.v - b.v, a.g0 - b.g0, a.g1 - b.g1, a.g2 - b.g2}; }
__device__ __forceinline__ D3 operator-(D3 a) { return {-a.v, -a.g0, -a.g1, -a.g2}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) {
    return {a.v * b.v, a.g0 * b.v + a.v * b.g0, a.g1 * b.v + a.v * b.g1, a.g2 * b.v + a.v * b.g2};
}
__device__ __forceinline__ D3 operator*(D3 a, float s) { return {a.v * s, a.g0 * s, a.g1 * s, a.g2 * s}; }
__device__ __forceinline__ D3 operator*(float s, D3 a) { return a * s; }
__device__ __forceinline__ D3 operator/(D3 a, D3 b) {
    const float q = a.v / b.v, ib = 1.0f / b.v;
    return {q, (a.g0 - q * b.g0) * ib, (a.g1 - q * b.g1) * ib, (a.g2 - q * b.g2) * ib};
}
__device__ __forceinline__ D3 operator/(D3 a, float s) { return a * (1.0f / s); }
__device__ __forceinline__ D3 chain(float v, float dv, D3 a) { return {v, dv * a.g0, dv * a.g1, dv * a.g2}; }
__device__ __forceinline__ D3 dsin(D3 a) { return chain(sinf(a.v), cosf(a.v), a); }
__device__ __forceinline__ D3 dcos(D3 a) { return chain(cosf(a.v), -sinf(a.v), a); }
__device__ __forceinline__ D3 dtan(D3 a) {
    const float t = tanf(a.v);
    return chain(t, 1.0f + t * t, a);
}
__device__ __forceinline__ D3 dasin(D3 a) { return chain(asinf(a.v), rsqrtf(fmaxf(1.0f - a.v * a.v, 1e-30f)), a); }
__device__ __forceinline__ D3 dsqrt(D3 a) {
    const float r = sqrtf(a.v);
    return chain(r, r > 0.0f ? 0.5f / r : 0.0f, a);
}

// the Fresnel formulas of rf_trace_core.cuh over duals (theta in tangent 0, the coating
// thicknesses in tangents 1 and 2)
__device__ __noinline__ D3 fresnel_d(D3 theta0, float n1, float n2) {
    D3 theta1 = dasin(dsin(theta0) * n1 / n2);
    D3 cosi = dcos(theta0), cost = dcos(theta1);
    D3 rs = (cosi * n1 - cost * n2) / (cosi * n1 + cost * n2);
    D3 rp = (cost * n1 - cosi * n2) / (cost * n1 + cosi * n2);
    return (rs * rs + rp * rp) / 2.0f;
}
__device__ __noinline__ D3 fresnel_ar_d(D3 theta0, float lambda, D3 d1, float n0, float n1, float n2) {
    D3 s0 = dsin(theta0);
    D3 theta1 = dasin(s0 * n0 / n1);
    D3 theta2 = dasin(s0 * n0 / n2);
    D3 rs01 = -dsin(theta0 - theta1) / dsin(theta0 + theta1);
    D3 rp01 = dtan(theta0 - theta1) / dtan(theta0 + theta1);
    D3 ts01 = 2.0f * dsin(theta1) * dcos(theta0) / dsin(theta0 + theta1);
    D3 tp01 = ts01 * dcos(theta0 - theta1);
    D3 rs12 = -dsin(theta1 - theta2) / dsin(theta1 + theta2);
    D3 rp12 = dtan(theta1 - theta2) / dtan(theta1 + theta2);
    D3 ris = ts01 * ts01 * rs12;
    D3 rip = tp01 * tp01 * rp12;
    D3 dy = d1 * n1;
    D3 dx = dtan(theta1) * dy;
    D3 delay = dsqrt(dx * dx + dy * dy);
    D3 rel_phase = (delay - dx * s0) * (4.0f * RF_MPI_F / lambda);
    D3 c = dcos(rel_phase);
    D3 out_s2 = rs01 * rs01 + ris * ris + 2.0f * rs01 * ris * c;
    D3 out_p2 = rp01 * rp01 + rip * rip + 2.0f * rp01 * rip * c;
    return (out_s2 + out_p2) / 2.0f;
}
__device__ void interface_r_d(float ni, D3 ci, float nj, D3 cj, D3& rs, D3& rp) {
    rs = (ci * ni - cj * nj) / (ci * ni + cj * nj);
    rp = (ci * nj - cj * ni) / (ci * nj + cj * ni);
}
__device__ D3 stack_r2_d(D3 r01, D3 r12, D3 r23, D3 d1, D3 d2) {
    D3 s2 = dsin(d2), c2 = dcos(d2), s1 = dsin(d1), c1 = dcos(d1);
    D3 nre = r12 + r23 * c2, nim = r23 * s2;
    D3 dre = dconst(1.0f) + r12 * r23 * c2, dim = r12 * r23 * s2;
    D3 den = dre * dre + dim * dim;
    D3 ire = (nre * dre + nim * dim) / den;
    D3 iim = (nim * dre - nre * dim) / den;
    D3 ere = ire * c1 - iim * s1, eim = ire * s1 + iim * c1;
    D3 tre = r01 + ere, tim = eim;
    D3 bre = dconst(1.0f) + r01 * ere, bim = r01 * eim;
    return (tre * tre + tim * tim) / (bre * bre + bim * bim);
}
__device__ __noinline__ D3 fresnel_two_layer_d(D3 theta0, float lambda, float n0, float na, D3 da, float nb, D3 db,
                                           float n2) {
    D3 s0 = dsin(theta0), c0 = dcos(theta0);
    D3 sa = s0 * (n0 / na), sb = s0 * (n0 / nb), s2 = s0 * (n0 / n2);
    D3 ca = dsqrt(dconst(1.0f) - sa * sa), cb = dsqrt(dconst(1.0f) - sb * sb), c2 = dsqrt(dconst(1.0f) - s2 * s2);
    D3 rs01, rp01, rs12, rp12, rs23, rp23;
    interface_r_d(n0, c0, na, ca, rs01, rp01);
    interface_r_d(na, ca, nb, cb, rs12, rp12);
    interface_r_d(nb, cb, n2, c2, rs23, rp23);
    const float phase = 4.0f * RF_MPI_F / lambda;
    D3 d1 = da * ca * (phase * na);
    D3 d2 = db * cb * (phase * nb);
    return (stack_r2_d(rs01, rs12, rs23, d1, d2) + stack_r2_d(rp01, rp12, rp23, d1, d2)) / 2.0f;
}

// ---------------------------------------------------------------- recording
// The state entering a loop step: position and direction.
struct State {
    float px, py, pz, dx, dy, dz;
};
struct CheckpointRecorder {
    State* checkpoints;  // the state entering steps 0, kCheckpoint, 2 kCheckpoint, ...
    unsigned char* tags;  // per step: element index | 0x80 when the ray reflects there
    int n;
    int argmax;  // step whose |xy| / height is the final rrel
    float best;
    __device__ __forceinline__ void step(int lens, float px, float py, float pz, float dx, float dy, float dz) {
        if (n < kAdjMaxSteps) {
            if (n % kCheckpoint == 0) checkpoints[n / kCheckpoint] = {px, py, pz, dx, dy, dz};
            tags[n] = (unsigned char)lens;
        }
        n++;
    }
    __device__ __forceinline__ void hit(int, const Hit&, float, float, float, bool) {}
    __device__ __forceinline__ void rrel(float r, float) {
        if (r > best) {
            best = r;
            argmax = n - 1;
        }
    }
    __device__ __forceinline__ void reflect() {
        if (n - 1 < kAdjMaxSteps) tags[n - 1] |= 0x80;
    }
};

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Reverse of intersect(p, d, e): given the adjoints of the hit point (gh) and of the normal
// (gn), adds the adjoints of p and d and returns those of the element's radius and center.
__device__ void intersect_adjoint(V3 p, V3 d, const SmemElement& e, V3 gh, V3 gn, V3& gp, V3& gd, float& gradius,
                                  float& gcenter) {
    if (e.radius == 0.0f) {  // plane z = -center: t = (-center - pz) / dz, hit = p + d t
        const float t = (-e.center - p.z) / d.z;
        const float gt = dot(gh, d);
        gp = gp + gh;
        gd = gd + gh * t;
        gcenter += -gt / d.z;
        gp.z += -gt / d.z;
        gd.z += -gt * t / d.z;
        return;
    }
    const float r = fabsf(e.radius), cz = -e.center;
    const V3 u = v3(0.0f - p.x, 0.0f - p.y, cz - p.z);
    const float proj = dot(u, d);
    const V3 u1 = d * proj;
    const V3 ev = u - u1;
    const float dist2 = dot(ev, ev);
    const float sgn = (e.radius * d.z) > 0.0f ? -1.0f : 1.0f;
    const float m = sqrtf(fmaxf(r * r - dist2, 0.0f));
    const V3 hit = (p + u1) - d * (m * sgn);
    const V3 q = v3(hit.x, hit.y, hit.z - cz);
    const float qn = sqrtf(dot(q, q));
    // n = sgn q / |q|
    const V3 qh = q * (1.0f / qn);
    const V3 gq = (gn - qh * dot(qh, gn)) * (sgn / qn);
    const V3 ghit = gh + gq;
    float gcz = -gq.z;
    // hit = p + u1 - sgn m d
    gp = gp + ghit;
    V3 gu1 = ghit;
    const float gm = -sgn * dot(ghit, d);
    gd = gd - ghit * (sgn * m);
    // m = sqrt(r^2 - |e|^2) (a ray grazing the sphere, m = 0, gets no gradient through m)
    V3 gu = v3(0.0f, 0.0f, 0.0f);
    if (m > 1e-12f) {
        const float gm2 = gm / (2.0f * m);
        gradius += gm2 * 2.0f * e.radius;
        const V3 ge = ev * (-2.0f * gm2);
        // e = u - u1
        gu = gu + ge;
        gu1 = gu1 - ge;
    }
    // u1 = d proj
    gd = gd + gu1 * proj;
    const float gproj = dot(gu1, d);
    // proj = u . d
    gu = gu + d * gproj;
    gd = gd + u * gproj;
    // u = (0, 0, cz) - p
    gcz += gu.z;
    gp = gp - gu;
    gcenter += -gcz;
}

__global__ void __launch_bounds__(kAdjThreads, RF_ADJOINT_MIN_BLOCKS) k_trace_adjoint(const rf_lens_element* __restrict__ elements,
                                                              const int2* __restrict__ paths,
                                                              const float* __restrict__ wavelengths,
                                                              const __grid_constant__ TraceParams p,
                                                              const float* __restrict__ grad_rays,
                                                              float* __restrict__ grad_elements,
                                                              float* __restrict__ grad_dir) {
    __shared__ SmemElement se[kAdjMaxElements];
    __shared__ float ior_tab[kAdjTableRows * kAdjMaxElements];
    __shared__ float acc[kAdjMaxElements * kGradPerElement + 3];
    __shared__ int queue[kAdjThreads / 32][64];  // per warp: ray offsets (in its span) still to trace
    const int E = p.E;
    const long long first = (long long)blockIdx.x * kAdjBlockRays;
    const long long last = min(first + kAdjBlockRays, p.n_rays) - 1;
    const long long pw_first = first / p.R, pw_last = last / p.R;
    const long long span_rows = pw_last - pw_first + 1;
    const int span = (int)(span_rows < (long long)p.W ? span_rows : (long long)p.W);
    const bool table = span <= kAdjTableRows;
    const bool disperse = !isnan(__ldg(&elements[0].coefficients[0]));
    for (int i = threadIdx.x; i < E; i += kAdjThreads) {
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
        for (int k = threadIdx.x; k < span * E; k += kAdjThreads) {
            int row = k / E, el = k % E;
            int wl = (int)((pw_first + row) % p.W);
            float n = elements[el].ior;
            if (disperse && n > 1.0f) n = dispersion(wavelengths[wl], elements[el].coefficients);
            ior_tab[row * E + el] = n;
        }
    }
    for (int i = threadIdx.x; i < E * kGradPerElement + 3; i += kAdjThreads) acc[i] = 0.0f;
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long n = p.n_rays;
    const float* coef_base = &elements[0].coefficients[0];
    TraceFrame f;
    f.E = E;
    f.aperture = p.aperture;
    f.W = p.W;
    f.G = p.G;
    f.R = p.R;
    f.cmin = p.cmin;
    f.layer_n0 = p.layer_n0;
    f.layer_n1 = p.layer_n1;
    f.dir[0] = p.dir[0];
    f.dir[1] = p.dir[1];
    f.dir[2] = p.dir[2];
    // The warp's span of consecutive rays; rays whose outputs have no gradient (rays that
    // miss, rays outside every covered pixel) contribute nothing and are not traced back.
    // The others are packed in order into full warps (a queue of up to 63 offsets), so
    // lanes are not left idle through a whole reverse sweep; rays of one span mostly share
    // their ghost path and wavelength (R = G^2 consecutive rays do).
    const long long span_first = first + (long long)warp * kAdjWarpRays;
    const long long span_end = min(span_first + kAdjWarpRays, n);
    int* q = queue[warp];
    int queued = 0;
    long long scan = span_first;
    for (;;) {
        while (queued < 32 && scan < span_end) {
            const long long i = scan + lane;
            bool has = false;
            if (i < span_end)
#pragma unroll
                for (int k = 0; k < 6; k++) has = has || grad_rays[k * n + i] != 0.0f;
            const unsigned m = __ballot_sync(0xffffffffu, has);
            if (has) q[queued + __popc(m & ((1u << lane) - 1u))] = (int)(i - span_first);
            queued += __popc(m);
            scan += 32;
        }
        __syncwarp();
        if (queued == 0) break;
        const int take = min(queued, 32), rest = queued - take;
        const int mine = lane < take ? q[lane] : -1;
        const int moved = lane < rest ? q[take + lane] : 0;
        __syncwarp();
        if (lane < rest) q[lane] = moved;
        queued = rest;
        // every lane runs the reverse sweep (lanes without a valid ray add zeros), so that the
        // warp can sum each step's gradient with shuffles when its rays share one ghost path
        // and wavelength (the same element sequence); otherwise lanes add to shared memory
        const bool in_range = mine >= 0;
        const long long idx = in_range ? span_first + mine : span_first;
        const int ray_id = (int)(idx % p.R);
        const long long pw = idx / p.R;
        const int wl_id = (int)(pw % p.W);
        const int path_id = (int)(pw / p.W);
        const int row = (int)((pw - pw_first) % p.W);
        const float* ior_row = table ? ior_tab + row * E : nullptr;
        const float wavelength = __ldg(wavelengths + wl_id);
        auto ior_of = [&](int el) -> float {
            if (ior_row) return ior_row[el];
            float nn = se[el].ior;
            if (disperse && nn > 1.0f) nn = dispersion(wavelength, coef_base + (size_t)el * 16);
            return nn;
        };
        const int gy = (int)truncf((float)ray_id / (float)p.G);
        const int gx = ray_id - gy * p.G;
        // a ray whose outputs have no gradient contributes nothing: it is not re-traced
        float g_out[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        bool needed = false;
        if (in_range) {
#pragma unroll
            for (int k = 0; k < 6; k++) {
                g_out[k] = grad_rays[k * n + idx];
                needed = needed || g_out[k] != 0.0f;
            }
        }
        State checkpoints[kMaxCheckpoints];
        unsigned char tags[kAdjMaxSteps];
        CheckpointRecorder rec{checkpoints, tags, 0, -1, 0.0f};
        float out[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (needed)
            trace_ray_rec(se, ior_row, disperse, coef_base, wavelength, __ldg(paths + path_id), p.grid[gx], p.grid[gy],
                          f, out, rec);
        const bool valid = needed && !isnan(out[5]) && rec.n <= kAdjMaxSteps && rec.n > 0;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        const int leader = vmask ? __ffs(vmask) - 1 : 0;
        const int key = path_id * p.W + wl_id;
        const int lead_key = __shfl_sync(0xffffffffu, key, leader);  // every lane takes part
        const bool uniform = __all_sync(0xffffffffu, !valid || key == lead_key);
        const int n_steps = __reduce_max_sync(0xffffffffu, valid ? (unsigned)rec.n : 0u);
        const float refl = out[5];
        V3 gp = v3(0.0f, 0.0f, 0.0f), gd = v3(0.0f, 0.0f, 0.0f);  // adjoint of the state leaving a step
        bool apt_pending = true;  // the last aperture crossing sets pos_apt
        // the states entering the steps of the current segment, regenerated from its checkpoint
        // by the forward's step (intersect, then reflect or refract; the stop and the sensor
        // keep the direction)
        State seg[kCheckpoint];
        for (int j = n_steps - 1; j >= 0; j--) {
            if (j == n_steps - 1 || (j + 1) % kCheckpoint == 0) {
                const int j0 = j - j % kCheckpoint;
                if (valid && j0 < rec.n) {
                    State st = checkpoints[j0 / kCheckpoint];
                    const int j1 = min(j + 1, rec.n);
                    for (int q = j0; q < j1; q++) {
                        seg[q - j0] = st;
                        if (q + 1 == j1) break;
                        const int i = tags[q] & 0x7f;
                        const Hit h = intersect(st.px, st.py, st.pz, st.dx, st.dy, st.dz, se[i]);
                        const State in = st;
                        st.px = h.px;
                        st.py = h.py;
                        st.pz = h.pz;
                        if (i == p.aperture || i == E - 1) continue;
                        const int n_index = (in.dz < 0.0f) ? i - 1 : i + 1;
                        if (tags[q] & 0x80) {
                            reflect_dir(st.dx, st.dy, st.dz, h);
                        } else {
                            const float n1 = (0 <= n_index && n_index < E) ? ior_of(n_index) : 1.0f;
                            refract_dir(st.dx, st.dy, st.dz, h, n1, ior_of(i));
                        }
                    }
                }
            }
            float g4[kGradPerElement] = {0.f, 0.f, 0.f, 0.f};
            int el = 0;
            if (valid && j < rec.n) {
                const State& st = seg[j % kCheckpoint];
                const int tag = tags[j];
                const int i = tag & 0x7f;
                el = i;
                const SmemElement& e = se[i];
                const V3 pin = v3(st.px, st.py, st.pz), din = v3(st.dx, st.dy, st.dz);
                const Hit h = intersect(pin.x, pin.y, pin.z, din.x, din.y, din.z, e);
                V3 gh = gp;  // adjoint of the hit point
                V3 gn = v3(0.0f, 0.0f, 0.0f);
                V3 gdin = v3(0.0f, 0.0f, 0.0f);
                if (j == rec.n - 1) gh = gh + v3(g_out[0], g_out[1], 0.0f);  // sensor position
                if (i == p.aperture) {
                    if (apt_pending) {
                        gh.x += g_out[2] / e.height;
                        gh.y += g_out[3] / e.height;
                        apt_pending = false;
                    }
                    gdin = gd;  // no change of direction at the stop
                } else {
                    if (j == rec.argmax) {
                        const float rxy = sqrtf(h.px * h.px + h.py * h.py);
                        if (rxy > 0.0f) {
                            const float sc = g_out[4] / (rxy * e.height);
                            gh.x += sc * h.px;
                            gh.y += sc * h.py;
                        }
                    }
                    const V3 nrm = v3(h.nx, h.ny, h.nz);
                    if (i == E - 1) {
                        gdin = gd;
                    } else {
                        const int n_index = (din.z < 0.0f) ? i - 1 : i + 1;
                        const float n1 = (0 <= n_index && n_index < E) ? ior_of(n_index) : 1.0f;
                        const float n2 = ior_of(i);
                        if (tag & 0x80) {
                            // d' = d - 2 (d.n) n
                            const float dn = dot(din, nrm), gdn = dot(gd, nrm);
                            gdin = gd - nrm * (2.0f * gdn);
                            gn = gn - (gd * dn + din * gdn) * 2.0f;
                            // reflectance factor R(theta, thicknesses), refl *= R when R > 0
                            const float c = -dn;
                            const float cc = clampf(c, -1.0f, 1.0f);
                            const float incident = acosf(cc);
                            const float theta = incident < 0.02f ? (float)((double)incident + 1e-9) : incident;
                            D3 th = {theta, 1.0f, 0.0f, 0.0f};
                            D3 R;
                            float gtheta = 0.0f;
                            if (e.layers == 2) {
                                R = fresnel_two_layer_d(th, wavelength, n1, p.layer_n0, D3{e.d0, 0.f, 1.f, 0.f},
                                                        p.layer_n1, D3{e.d1, 0.f, 0.f, 1.f}, n2);
                            } else if (e.layers == 1 || e.coating > 0) {
                                const float nc = fmaxf(sqrtf(n1 * n2), p.cmin);
                                const D3 d1 = e.layers == 1 ? D3{e.d0, 0.f, 1.f, 0.f}
                                                            : dconst((float)e.coating / (4.0f * nc));
                                R = fresnel_ar_d(th, wavelength, d1, n1, nc, n2);
                            } else {
                                R = fresnel_d(th, n1, n2);
                            }
                            if (R.v > 0.0f) {
                                const float gR = g_out[5] * refl / R.v;
                                gtheta = gR * R.g0;
                                g4[2] += gR * R.g1;
                                g4[3] += gR * R.g2;
                            }
                            if (fabsf(c) < 1.0f) {
                                const float gc = gtheta * (-rsqrtf(1.0f - c * c));
                                // c = -d.n
                                gdin = gdin - nrm * gc;
                                gn = gn - din * gc;
                            }
                        } else {
                            // d' = o d + k n, k = o c - sqrt(1 - o^2 (1 - c^2)), c = -d.n
                            const float o = n1 / n2;
                            const float c = -dot(din, nrm);
                            const float sint2 = (o * o) * (1.0f - c * c);
                            const float sq = sqrtf(fabsf(1.0f - sint2));
                            const float k = o * c - sq;
                            const float gk = dot(gd, nrm);
                            const float dk_dc = sq > 0.0f ? o - o * o * c / sq : o;
                            gdin = gd * o - nrm * (gk * dk_dc);
                            gn = gn + gd * k - din * (gk * dk_dc);
                        }
                    }
                }
                V3 gpin = v3(0.0f, 0.0f, 0.0f);
                intersect_adjoint(pin, din, e, gh, gn, gpin, gdin, g4[0], g4[1]);
                gp = gpin;
                gd = gdin;
            }
            if (uniform) {
                // the warp's four sums in one reduce-scatter: lanes exchange halves of their
                // values (lane bit 4 picks components 2-3 or 0-1, bit 3 one of those), then sum
                // within groups of 8; lanes 0, 8, 16, 24 end with components 0, 1, 2, 3
                static_assert(kGradPerElement == 4, "four gradient components per element");
                el = __shfl_sync(0xffffffffu, el, leader);
                const bool hi = (lane & 16) != 0, odd = (lane & 8) != 0;
                float a = hi ? g4[2] : g4[0], b = hi ? g4[3] : g4[1];
                a += __shfl_xor_sync(0xffffffffu, hi ? g4[0] : g4[2], 16);
                b += __shfl_xor_sync(0xffffffffu, hi ? g4[1] : g4[3], 16);
                float v = odd ? b : a;
                v += __shfl_xor_sync(0xffffffffu, odd ? a : b, 8);
                v += __shfl_xor_sync(0xffffffffu, v, 4);
                v += __shfl_xor_sync(0xffffffffu, v, 2);
                v += __shfl_xor_sync(0xffffffffu, v, 1);
                if ((lane & 7) == 0 && v != 0.0f) atomicAdd(&acc[el * kGradPerElement + (lane >> 3)], v);
            } else if (valid && j < rec.n) {
#pragma unroll
                for (int k = 0; k < kGradPerElement; k++)
                    if (g4[k] != 0.0f) atomicAdd(&acc[el * kGradPerElement + k], g4[k]);
            }
        }
        // entry ray: p_in = hit0 - dir, d_in = dir; hit0 = grid point hitting element 0
        V3 gdir = v3(0.0f, 0.0f, 0.0f);
        float g0r = 0.0f, g0c = 0.0f;
        if (valid) {
            gdir = gd - gp;
            const V3 g0 = v3(p.grid[gx], -p.grid[gy], 1.0f);
            const Hit h0 = intersect(g0.x, g0.y, g0.z, 0.0f, 0.0f, -1.0f, se[0]);
            if (h0.hit) {
                V3 gpg = v3(0.f, 0.f, 0.f), gdg = v3(0.f, 0.f, 0.f);
                intersect_adjoint(g0, v3(0.0f, 0.0f, -1.0f), se[0], gp, v3(0.f, 0.f, 0.f), gpg, gdg, g0r, g0c);
            }
        }
        const float tail[5] = {g0r, g0c, gdir.x, gdir.y, gdir.z};
#pragma unroll
        for (int k = 0; k < 5; k++) {
            float v = tail[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && v != 0.0f)
                atomicAdd(&acc[k < 2 ? k : E * kGradPerElement + (k - 2)], v);
        }
    }  // the warp's next 32 rays
    __syncthreads();
    for (int i = threadIdx.x; i < E * kGradPerElement; i += kAdjThreads)
        if (acc[i] != 0.0f) atomicAdd(&grad_elements[i], acc[i]);
    if (threadIdx.x < 3 && acc[E * kGradPerElement + threadIdx.x] != 0.0f)
        atomicAdd(&grad_dir[threadIdx.x], acc[E * kGradPerElement + threadIdx.x]);
}

}  // namespace
}  // namespace rf

extern "C" int rf_trace_adjoint(const rf_lens_element* elements, const int32_t* paths, const float* wavelengths,
                                const rf_trace_args* args, const float* grad_rays, float* grad_elements,
                                float* grad_direction, void* stream) {
    using namespace rf;
    if (!elements || !paths || !wavelengths || !args || !grad_rays || !grad_elements || !grad_direction)
        return RF_ERR_INVALID_ARG;
    const rf_trace_args& a = *args;
    if (a.element_count < 2 || a.element_count > kAdjMaxElements || a.path_count < 0 || a.wavelength_count < 1 ||
        a.grid_count < 2 || a.grid_count > kMaxGrid || a.aperture_index < 0)
        return RF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    RF_TRY(cuda_status(
        cudaMemsetAsync(grad_elements, 0, sizeof(float) * kGradPerElement * (size_t)a.element_count, s)));
    RF_TRY(cuda_status(cudaMemsetAsync(grad_direction, 0, sizeof(float) * 3, s)));
    TraceParams p;
    if (!trace_params(a, p)) return RF_ERR_INVALID_ARG;
    if (p.n_rays == 0) return RF_OK;
    k_trace_adjoint<<<blocks_for(p.n_rays, kAdjBlockRays), kAdjThreads, 0, s>>>(elements, (const int2*)paths,
                                                                           wavelengths, p, grad_rays, grad_elements,
                                                                           grad_direction);
    return launch_status();
}
