// rf_raster.cu — the ghost rasteriser.
//
// Per pixel the result is the reference's (realflare/api/tasks/cl/rasterizing.cl:524-663):
// the sum over visible primitives (in primitive order), wavelength pairs and sub-wavelength
// steps of XYZ(lambda) * fragment, where a fragment is the n-rook sample coverage of the
// integer quad (intersect_quad 55-93) times the mean-value interpolated ghost texture,
// housing falloff, area intensity and coating reflectance (compute_barycentric_quad
// 95-148, fragment_shader 471-506, mix_vertex 509-522), scaled and converted to AP1
// (color.cl:3-10) and written y-flipped.
//
// GB300 organisation (k_raster): one CTA per T x T tile, threads own pixels (T = 32: 256
// threads x 4 pixels). The tile's list from rf_bin_tiles holds (primitive, wavelength pair)
// entries in increasing order. Entries are expanded in batches into shared-memory records
// (one per sub-wavelength step): the mixed integer vertices, the five edge functions as
// wrapping-int32 plane coefficients with the top-left bias folded in, the integer bounds
// and the mixed attributes, set up once by one thread each. Every pixel then walks the
// records in order, so its sum runs in the reference's order; a pixel whose samples lie
// outside a record's integer bounds skips it (exact: with vertex and sample coordinates
// below 2^14 the edge functions cannot wrap, and the quad test then never accepts a
// sample outside the bounds; records beyond that range are tested at every pixel).
//
// k_raster_masks is the literal per-pixel loop over the reference's bin masks, used for
// parity checks of the binner and the rasteriser.
#include <stddef.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "rf_common.cuh"

namespace rf {
int tile_size_of(const rf_raster_args& a);

namespace {

// Tuning knobs (compile-time): records per shared-memory batch, resident blocks per SM
// requested from the register allocator, and where the half-angle tangents use the
// reference's exact FP32 operations (1: small angles, 0: only a_i == 0).
#ifndef RF_RASTER_BATCH
#define RF_RASTER_BATCH 64
#endif
#ifndef RF_RASTER_MIN_BLOCKS
#define RF_RASTER_MIN_BLOCKS 3
#endif
#ifndef RF_RASTER_MIN_BLOCKS_S1  // the one-sample kernel needs fewer registers
#define RF_RASTER_MIN_BLOCKS_S1 4
#endif
#ifndef RF_RASTER_CLASSIFY
#define RF_RASTER_CLASSIFY 1
#endif
#ifndef RF_RASTER_EXACT_SMALL_ANGLES
#define RF_RASTER_EXACT_SMALL_ANGLES 0
#endif
constexpr int kBatchRecords = RF_RASTER_BATCH;

#ifdef RF_RASTER_STATS
// Work counters of the statistics build (never compiled into the product library):
// record iterations per 8 x 4 block, those of whole-block records, fragments, fragments of
// whole-block records, block visits, fragments whose smoothstep factor is 0 (rrel >= 1),
// record iterations where that holds for every shaded pixel of the block (those two with
// more than one sample per pixel), warp steps of the one-sample shading loop.
constexpr int kRasterStats = 8;
__device__ unsigned long long g_raster_stats[kRasterStats];
#define RF_STAT(stmt) stmt
#else
#define RF_STAT(stmt)
#endif

// Every group the shading loop reads starts on a 16-byte boundary and is read with
// 16-byte shared-memory loads (ec[12..14] and flags as one vector). Records are 272 bytes
// apart (17 x 16): where the lanes of a warp read 32 different records at one offset (the
// block selection), each group of 8 lanes then reads 8 different 16-byte bank groups instead
// of one.
struct alignas(16) Rec {
    int bb[4];       // xmin, xmax, ymin, ymax
    float col[4];    // the record's XYZ weight (1, 1, 1 with one wavelength), pad
    float qf[8];     // q as floats (exact: |q| < 2^24)
    float uv[8];     // ghost texel coordinates of the corners (u0, v0, ..., u3, v3), see store_corner
    float rs[4];     // (rrel - 1) / (0.95 - 1): smoothstep(1, 0.95, rrel)'s ramp before clamping
    float inten[4], refl[4];
    int ec[15];      // edges 01, 12, 23, 30, 20: l = A * y + B * x + C (bias folded into C)
    int flags;       // 1: bounds rejection is exact; 2: adds nothing (collinear, or zero_record)
    int q[8];        // mixed vertex positions, sample space (x0, y0, ..., x3, y3)
    int color;       // w * WS + i
    int pad[4];      // the stride
};
static_assert(sizeof(Rec) == 272 && offsetof(Rec, bb) == 0 && offsetof(Rec, col) % 16 == 0 &&
                  offsetof(Rec, qf) % 16 == 0 && offsetof(Rec, uv) % 16 == 0 && offsetof(Rec, rs) % 16 == 0 &&
                  offsetof(Rec, inten) % 16 == 0 && offsetof(Rec, refl) % 16 == 0 &&
                  offsetof(Rec, ec) % 16 == 0 && offsetof(Rec, flags) == offsetof(Rec, ec) + 15 * sizeof(int),
              "records are read with 16-byte loads");
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ int4 ld4i(const int* p) { return *reinterpret_cast<const int4*>(p); }

struct RasterParams {
    int width, height, T, ntx, S, W, WS, G, maxW;
    float intensity, ghost_scale;
    int ghost_w, ghost_h;
    bool safe_screen;
    unsigned long long ghost_tex;  // texture object over the ghost texture (the kTex kernels)
};

__device__ __forceinline__ bool top_left(int ax, int ay, int bx, int by) {
    int ex = wsub(bx, ax), ey = wsub(by, ay);
    return (ey == 0 && ex > 0) || ey > 0;
}

__device__ __forceinline__ int32_t edge_i(int ax, int ay, int bx, int by, int cx, int cy) {
    return wsub(wmul(wsub(ax, bx), wsub(cy, ay)), wmul(wsub(ay, by), wsub(cx, ax)));
}

__device__ __forceinline__ void edge_coeffs(int ax, int ay, int bx, int by, int* e) {
    // (a.x - b.x) * (p.y - a.y) - (a.y - b.y) * (p.x - a.x) + bias, as A*p.y + B*p.x + C
    const int A = wsub(ax, bx);
    const int dy = wsub(ay, by);
    e[0] = A;
    e[1] = wsub(0, dy);
    e[2] = wadd(wsub(wmul(dy, ax), wmul(A, ay)), top_left(ax, ay, bx, by) ? 0 : -1);
}

// the 15 edge coefficients and the flags word, by four 16-byte loads
__device__ __forceinline__ void load_edges(const Rec& r, int e[16]) {
    const int4 a = ld4i(r.ec), b = ld4i(r.ec + 4), c = ld4i(r.ec + 8), d = ld4i(r.ec + 12);
    e[0] = a.x, e[1] = a.y, e[2] = a.z, e[3] = a.w, e[4] = b.x, e[5] = b.y, e[6] = b.z, e[7] = b.w;
    e[8] = c.x, e[9] = c.y, e[10] = c.z, e[11] = c.w, e[12] = d.x, e[13] = d.y, e[14] = d.z, e[15] = d.w;
}

// intersect_quad (rasterizing.cl:55-93) from plane coefficients
__device__ __forceinline__ bool inside(const Rec& r, int px, int py) {
    int e[16];
    load_edges(r, e);
    const bool w01 = wadd(wadd(wmul(e[0], py), wmul(e[1], px)), e[2]) >= 0;
    const bool w12 = wadd(wadd(wmul(e[3], py), wmul(e[4], px)), e[5]) >= 0;
    const bool w23 = wadd(wadd(wmul(e[6], py), wmul(e[7], px)), e[8]) >= 0;
    const bool w30 = wadd(wadd(wmul(e[9], py), wmul(e[10], px)), e[11]) >= 0;
    const bool w20 = wadd(wadd(wmul(e[12], py), wmul(e[13], px)), e[14]) >= 0;
    const bool front = (w20 && w01 && w12 && (w23 || w30)) || (!w20 && w23 && w30 && (w01 || w12));
    const bool back = (!w20 && !w01 && !w12 && (!w23 || !w30)) || (w20 && !w23 && !w30 && (!w01 || !w12));
    return front || back;
}

// Coverage of the sample rectangle [x0, x1] x [y0, y1] by a record whose coordinates
// keep every edge value exact (flags & 1): each edge value is linear in the sample, so
// its sign is constant over the rectangle when its minimum and maximum there (over the
// corners) agree, and then inside() is constant too. Returns 0 (no sample inside),
// 2 (every sample inside) or 1 (mixed or undecided).
__device__ __forceinline__ int rect_coverage(const Rec& r, int x0, int x1, int y0, int y1) {
    int ec[16];
    load_edges(r, ec);
    bool w[5];
#pragma unroll
    for (int e = 0; e < 5; e++) {
        const int A = ec[3 * e], B = ec[3 * e + 1], C = ec[3 * e + 2];
        const int ay0 = A * y0, ay1 = A * y1, bx0 = B * x0, bx1 = B * x1;
        const int lo = C + min(ay0, ay1) + min(bx0, bx1);
        const int hi = C + max(ay0, ay1) + max(bx0, bx1);
        if (lo < 0 && hi >= 0) return 1;
        w[e] = lo >= 0;
    }
    const bool w01 = w[0], w12 = w[1], w23 = w[2], w30 = w[3], w20 = w[4];
    const bool front = (w20 && w01 && w12 && (w23 || w30)) || (!w20 && w23 && w30 && (w01 || w12));
    const bool back = (!w20 && !w01 && !w12 && (!w23 || !w30)) || (w20 && !w23 && !w30 && (!w01 || !w12));
    return (front || back) ? 2 : 0;
}

// Mean-value weights (compute_barycentric_quad, rasterizing.cl:95-148) at the integer
// sample point (px, py). The coordinates s_i = q_i - p are exact floats; the products
// a_i, d_i, |s_i|^2 are exact integers wherever |s| < 4096, so fused multiply-adds give
// the reference's values there. Where a_i is 0 the reference divides the rounding residue
// of r_i r_j - d_i by 1e-3: that tangent is evaluated with the reference's exact FP32
// operations (correctly rounded square roots, product, difference, quotient). Elsewhere
// the tangents and the divisions by r_i and by the weight sum use reciprocal and
// reciprocal-square-root instructions (a few ulps).
__device__ __forceinline__ void barycentric_fast(const Rec& rec, float px, float py, float w[4]) {
    float sx[4], sy[4], a[4], d[4], r2[4];
    const float4 q01 = ld4(rec.qf), q23 = ld4(rec.qf + 4);
    sx[0] = q01.x - px, sy[0] = q01.y - py, sx[1] = q01.z - px, sy[1] = q01.w - py;
    sx[2] = q23.x - px, sy[2] = q23.y - py, sx[3] = q23.z - px, sy[3] = q23.w - py;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int j = (i + 1) & 3;
        a[i] = sx[i] * sy[j] - sx[j] * sy[i];
        d[i] = sx[i] * sx[j] + sy[i] * sy[j];
        r2[i] = sx[i] * sx[i] + sy[i] * sy[i];
    }
    // The common case first. a_i are integers (differences of products of integers): when
    // none is 0 each |a_i| >= 1 and every term below is finite, so the weight sum is finite.
    // An a_i of 0 makes t_i infinite or NaN, and a vertex on the sample point (r2_i = 0)
    // makes r_i NaN; either way the sum is not finite, and only then are the weights redone
    // with the reference's special cases (the rare path).
    static_assert(!RF_RASTER_EXACT_SMALL_ANGLES, "the rare path is entered only for a_i == 0 or r_i == 0");
    float ir[4], r[4], t[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        ir[i] = rsqrtf(r2[i]);
        r[i] = r2[i] * ir[i];
    }
#pragma unroll
    for (int i = 0; i < 4; i++) t[i] = (r[i] * r[(i + 1) & 3] - d[i]) * __fdividef(1.0f, a[i]);
#pragma unroll
    for (int i = 0; i < 4; i++) w[i] = (t[(i + 3) & 3] + t[i]) * ir[i];
    float sum = w[0] + w[1] + w[2] + w[3];
    if (!(fabsf(sum) <= 3.40282347e38f)) {
        bool zero = false;
#pragma unroll
        for (int i = 0; i < 4; i++) zero = zero || r2[i] == 0.0f;
        if (zero) {  // a vertex on the sample point: one-hot on the first such vertex
            int k = 0;
#pragma unroll
            for (int i = 3; i >= 0; i--)
                if (sx[i] == 0.0f && sy[i] == 0.0f) k = i;
#pragma unroll
            for (int i = 0; i < 4; i++) w[i] = i == k ? 1.0f : 0.0f;
            return;
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int j = (i + 1) & 3;
            const bool exact = RF_RASTER_EXACT_SMALL_ANGLES ? a[i] * a[i] < (1.0f / 4096.0f) * r2[i] * r2[j]
                                                            : a[i] == 0.0f;
            if (exact) {
                const float ai = a[i] == 0.0f ? 1e-3f : a[i];
                t[i] = __fdiv_rn(__fsub_rn(__fmul_rn(__fsqrt_rn(r2[i]), __fsqrt_rn(r2[j])), d[i]), ai);
            } else {
                t[i] = (r[i] * r[j] - d[i]) * __fdividef(1.0f, a[i]);
            }
        }
#pragma unroll
        for (int i = 0; i < 4; i++) w[i] = (t[(i + 3) & 3] + t[i]) * ir[i];
        sum = w[0] + w[1] + w[2] + w[3];
    }
    const float inv = __fdividef(1.0f, sum);
#pragma unroll
    for (int i = 0; i < 4; i++) w[i] *= inv;
}

// Bilinear ghost sample (read_imagef LINEAR, CLAMP -> border 0, rasterizing.cl:483-485)
// at texel coordinates (u, v) = uv * size - 0.5.
__device__ __forceinline__ float ghost_sample(const float* __restrict__ tex, int w, int h, float u, float v) {
    if (!(fabsf(u) + fabsf(v) < 2e9f)) return 0.0f;  // non-finite or far outside
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const int i0 = (int)fu, j0 = (int)fv;
    float t00, t10, t01, t11;
    if ((unsigned)i0 < (unsigned)(w - 1) && (unsigned)j0 < (unsigned)(h - 1)) {
        // all four texels inside (the common case)
        const float* q = tex + (j0 * w + i0);
        t00 = __ldg(q);
        t10 = __ldg(q + 1);
        t01 = __ldg(q + w);
        t11 = __ldg(q + w + 1);
    } else {
        const bool i0_in = (unsigned)i0 < (unsigned)w, i1_in = (unsigned)(i0 + 1) < (unsigned)w;
        const bool j0_in = (unsigned)j0 < (unsigned)h, j1_in = (unsigned)(j0 + 1) < (unsigned)h;
        // load from clamped (always valid) addresses, then zero the texels outside the image
        const int ia = min(max(i0, 0), w - 1), ib = min(max(i0 + 1, 0), w - 1);
        const float* row0 = tex + (size_t)min(max(j0, 0), h - 1) * w;
        const float* row1 = tex + (size_t)min(max(j0 + 1, 0), h - 1) * w;
        t00 = (i0_in && j0_in) ? __ldg(row0 + ia) : 0.0f;
        t10 = (i1_in && j0_in) ? __ldg(row0 + ib) : 0.0f;
        t01 = (i0_in && j1_in) ? __ldg(row1 + ia) : 0.0f;
        t11 = (i1_in && j1_in) ? __ldg(row1 + ib) : 0.0f;
    }
    // the specification's (1-a)(1-b) t00 + a(1-b) t10 + (1-a) b t01 + a b t11, as three
    // interpolations (the same value up to rounding)
    const float top = fmaf(a, t10 - t00, t00), bottom = fmaf(a, t11 - t01, t01);
    return fmaf(b, bottom - top, top);
}

// ghost_sample through a texture object over the same texels (float, pitch-linear, border
// address mode): tex2Dgather at the centre of the 2 x 2 footprint, (i0 + 1, j0 + 1), exactly
// half a texel from every footprint boundary, returns texels (i0, j0 + 1), (i0 + 1, j0 + 1),
// (i0 + 1, j0), (i0, j0) in x, y, z, w, and 0 for texels outside the image; one texture
// instruction instead of the bounds test, the address arithmetic and four loads. The values,
// and so the interpolation, are ghost_sample's.
__device__ __forceinline__ float ghost_sample_tex(unsigned long long tex, float u, float v) {
    if (!(fabsf(u) + fabsf(v) < 2e9f)) return 0.0f;  // non-finite or far outside
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const float4 g = tex2Dgather<float4>((cudaTextureObject_t)tex, fu + 1.0f, fv + 1.0f, 0);
    const float top = fmaf(a, g.z - g.w, g.w), bottom = fmaf(a, g.y - g.x, g.x);
    return fmaf(b, bottom - top, top);
}

// fragment_shader (rasterizing.cl:471-506) times the hit count. The texture coordinate
// ((uv / scale + 1) / 2) * size - 0.5 is evaluated as uv * tex_scale + tex_offset.
struct FragmentConsts {
    float tsx, tox, tsy, toy;  // texel coordinate scale and offset per axis
};
template <bool kTex = false>
__device__ __forceinline__ float fragment_fast(const Rec& r, const float w[4], const float* __restrict__ ghost,
                                               const RasterParams& p, const FragmentConsts& fc, int hits) {
    const float4 uv01 = ld4(r.uv), uv23 = ld4(r.uv + 4);
    const float u = w[0] * uv01.x + w[1] * uv01.z + w[2] * uv23.x + w[3] * uv23.z;
    const float v = w[0] * uv01.y + w[1] * uv01.w + w[2] * uv23.y + w[3] * uv23.w;
    const float gi = kTex ? ghost_sample_tex(p.ghost_tex, u, v) : ghost_sample(ghost, p.ghost_w, p.ghost_h, u, v);
    // smoothstep(1, 0.95, rrel): the ramp (rrel - 1) / (0.95 - 1) is linear in rrel, so the
    // corners' ramps interpolate to the fragment's (the weights sum to one)
    const float4 rl = ld4(r.rs);
    const float st = __saturatef(w[0] * rl.x + w[1] * rl.y + w[2] * rl.z + w[3] * rl.w);
    const float ri = st * st * (3.0f - 2.0f * st);
    const float4 in = ld4(r.inten), rf = ld4(r.refl);
    float ai = w[0] * in.x + w[1] * in.y + w[2] * in.z + w[3] * in.w;
    float ci = w[0] * rf.x + w[1] * rf.y + w[2] * rf.z + w[3] * rf.w;
    ai = fmaxf(ai, 0.0f);
    ci = fmaxf(ci, 0.0f);
    return gi * ri * ai * ci * (float)hits;
}

__host__ __device__ inline FragmentConsts fragment_consts(const RasterParams& p) {
    FragmentConsts fc;
    const double sx = 0.5 / p.ghost_scale * p.ghost_w, sy = 0.5 / p.ghost_scale * p.ghost_h;
    fc.tsx = (float)sx;
    fc.tsy = (float)sy;
    fc.tox = (float)(0.5 * p.ghost_w - 0.5);
    fc.toy = (float)(0.5 * p.ghost_h - 0.5);
    return fc;
}

// 1 / (0.95 - 1), the smoothstep ramp's slope (fragment_shader, rasterizing.cl:487-488)
constexpr float kRampScale = 1.0f / (0.95f - 1.0f);

// Corner k of entry `entry` at the pair's two wavelengths: vertex words a0, a1 (first
// wavelength) and b0, b1 (second).
struct CornerLoad {
    float4 a0, a1, b0, b1;
};
__device__ __forceinline__ void load_corner(const float4* __restrict__ vtx, uint32_t entry, int k,
                                            const RasterParams& p, CornerLoad& c) {
    const long long prim = entry / p.maxW;
    const int w = (int)(entry % p.maxW);
    const int Q = (p.G - 1) * (p.G - 1), VC = p.G * p.G;
    const long long path = prim / Q;
    const int quad = (int)(prim % Q);
    const int c0 = (quad / (p.G - 1)) * p.G + quad % (p.G - 1);
    const int corner = k == 0 ? c0 : (k == 1 ? c0 + 1 : (k == 2 ? c0 + 1 + p.G : c0 + p.G));
    const long long vi = (path * VC + corner) * p.W + w;
    c.a0 = __ldg(vtx + 2 * vi);
    c.a1 = __ldg(vtx + 2 * vi + 1);
    c.b0 = __ldg(vtx + 2 * vi + 2);
    c.b1 = __ldg(vtx + 2 * vi + 3);
}
// mix_vertex (rasterizing.cl:509-522) of one corner into record r. The texture coordinate
// is stored in texels, uv * tex_scale + tex_offset (fragment_fast): the weights sum to one,
// so interpolating texel coordinates is the fragment's ((uv / scale + 1) / 2) * size - 0.5.
__device__ __forceinline__ void store_corner(const CornerLoad& c, int k, float t, int S, const FragmentConsts& fc,
                                             Rec& r) {
    const float px = c.a0.x + (c.b0.x - c.a0.x) * t, py = c.a0.y + (c.b0.y - c.a0.y) * t;
    r.uv[2 * k] = (c.a0.z + (c.b0.z - c.a0.z) * t) * fc.tsx + fc.tox;
    r.uv[2 * k + 1] = (c.a0.w + (c.b0.w - c.a0.w) * t) * fc.tsy + fc.toy;
    r.rs[k] = ((c.a1.x + (c.b1.x - c.a1.x) * t) - 1.0f) * kRampScale;
    r.refl[k] = c.a1.y + (c.b1.y - c.a1.y) * t;
    r.inten[k] = c.a1.z + (c.b1.z - c.a1.z) * t;
    r.q[2 * k] = cvt_rz_sat(px * (float)S);
    r.q[2 * k + 1] = cvt_rz_sat(py * (float)S);
    r.qf[2 * k] = (float)r.q[2 * k];
    r.qf[2 * k + 1] = (float)r.q[2 * k + 1];
}
// Whether every fragment of a record is zero, so that shading it adds nothing:
//  - a corner's reflectance is NaN (a ray that failed, at either wavelength of the pair):
//    the coating term max(NaN, 0) is 0 (rasterizing.cl:495-497) and every other factor is
//    finite, so each fragment is exactly 0;
//  - one sample per pixel, every corner's rrel >= 1 (the ray left the lens housing) and the
//    quad strictly convex and counter-clockwise in sample space, with coordinates that keep
//    the edge functions exact and an extent below 4096: a covered pixel is then inside the
//    quad or on one of its edges or corners, where every cross product a_i is >= 0 (an
//    exact integer) and the tangents share its sign, so the mean-value weights are
//    non-negative up to rounding and their rrel is >= 1; smoothstep(1, 0.95, rrel) is 0
//    there, and at most a few units in the last place of 1 below it (a factor below 1e-9).
// Clockwise quads are left in: on an edge the reference divides by +1e-3 whatever the
// orientation, so the weights there mix signs.
__device__ __forceinline__ bool zero_record(const RasterParams& p, const Rec& r, bool safe) {
    const float4 rf = ld4(r.refl);
    if (isnan(rf.x) || isnan(rf.y) || isnan(rf.z) || isnan(rf.w)) return true;
    if (p.S != 1 || !safe || r.bb[1] - r.bb[0] >= 4096 || r.bb[3] - r.bb[2] >= 4096) return false;
    const float4 rl = ld4(r.rs);  // rrel >= 1 exactly when the ramp is <= 0
    if (!(rl.x <= 0.0f && rl.y <= 0.0f && rl.z <= 0.0f && rl.w <= 0.0f)) return false;
    const int* q = r.q;
    bool convex = true;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int j = (i + 1) & 3, k = (i + 2) & 3;
        // |differences| < 4096: the products are exact in 32 bits
        const int turn = (q[2 * j] - q[2 * i]) * (q[2 * k + 1] - q[2 * j + 1]) -
                         (q[2 * j + 1] - q[2 * i + 1]) * (q[2 * k] - q[2 * j]);
        convex = convex && turn > 0;
    }
    return convex;
}

// edges, bounds and flags of a record whose corners are stored
__device__ __forceinline__ void finish_record(const RasterParams& p, int w, int i, const float* xyz, Rec& r) {
    const int* q = r.q;
    edge_coeffs(q[0], q[1], q[2], q[3], r.ec + 0);
    edge_coeffs(q[2], q[3], q[4], q[5], r.ec + 3);
    edge_coeffs(q[4], q[5], q[6], q[7], r.ec + 6);
    edge_coeffs(q[6], q[7], q[0], q[1], r.ec + 9);
    edge_coeffs(q[4], q[5], q[0], q[1], r.ec + 12);
    r.bb[0] = min(min(q[0], q[2]), min(q[4], q[6]));
    r.bb[1] = max(max(q[0], q[2]), max(q[4], q[6]));
    r.bb[2] = min(min(q[1], q[3]), min(q[5], q[7]));
    r.bb[3] = max(max(q[1], q[3]), max(q[5], q[7]));
    // bounds rejection is exact while every coordinate stays below 2^14 - 1 in magnitude
    const int lim = 16382;
    bool safe = p.safe_screen;
#pragma unroll
    for (int k = 0; k < 8; k++) safe = safe && q[k] <= lim && q[k] >= -lim;
    int flags = safe ? 1 : 0;
    if (edge_i(q[0], q[1], q[2], q[3], q[4], q[5]) == 0 && edge_i(q[0], q[1], q[4], q[5], q[6], q[7]) == 0)
        flags |= 2;
    if (!(flags & 2) && zero_record(p, r, safe)) flags |= 2;
    r.flags = flags;
    r.color = w * p.WS + i;
    if (p.W > 1) {
        const float* c = xyz + 3 * r.color;
        r.col[0] = c[0];
        r.col[1] = c[1];
        r.col[2] = c[2];
    } else {  // rgb += frag (rasterizing.cl:648-650): a weight of exactly 1
        r.col[0] = r.col[1] = r.col[2] = 1.0f;
    }
    r.col[3] = 0.0f;
}

// A CTA of 8 warps shades one T x T tile (T = 32 or 16): the tile's T^2 / 32 blocks of
// 8 x 4 pixels (block b at column b % (T / 8), row b / (T / 8)) go to warps one at a time,
// so a record outside a block's sample bounds is skipped by the whole warp at once.
constexpr int kThreads = 256;

template <int T>
constexpr size_t raster_smem_bytes(int maxW, int WS) {
    return sizeof(Rec) * 2 * kBatchRecords + sizeof(float) * (3 * maxW * WS + ((WS + 3) & ~3)) +
           sizeof(float) * 96 * (T * T / 32);
}

// Tile (tx, ty), whose entries are tile_entries[begin, end). smem4 holds the dynamic shared
// memory (raster_smem_bytes), next_block two shared counters. kS: the anti-aliasing sample
// count when known at compile time (1), else 0 (p.S). kTex: sample the ghost texture through
// p.ghost_tex.
template <int T, int kS, bool kTex = false>
__device__ __forceinline__ void raster_tile(const float4* __restrict__ vtx, uint32_t begin, uint32_t end,
                                            const uint32_t* __restrict__ tile_entries,
                                            const float* __restrict__ ghost, const float* __restrict__ spectrum,
                                            const RasterParams& p, const FragmentConsts& fcs,
                                            float4* __restrict__ image, int tx, int ty, float4* smem4,
                                            int* next_block) {
    constexpr int kBlocks = T * T / 32;  // 8 x 4 pixel blocks per tile
    constexpr int kCols = T / 8;         // blocks per tile row
    Rec* recbuf = (Rec*)smem4;     // two batches of records
    float* xyz = (float*)(recbuf + 2 * kBatchRecords);  // [maxW * WS][3]
    float* blend = xyz + 3 * p.maxW * p.WS;       // [WS]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        const float sub_step = 1.0f / (float)p.WS;
        float b = 0.0f;
        for (int i = 0; i < p.WS; i++) {
            blend[i] = b;
            b += sub_step;
        }
    }
    if (p.W > 1) {
        const float sub_step = 1.0f / (float)p.WS;
        const float wl_step = sub_step / (float)p.W;
        for (int w = threadIdx.x; w < p.maxW; w += kThreads) {
            float pos = ((float)w + 0.5f) / (float)p.W;
            for (int i = 0; i < p.WS; i++) {
                for (int c = 0; c < 3; c++)
                    xyz[3 * (w * p.WS + i) + c] = sample_linear(spectrum, RF_SPECTRUM_WIDTH, 1, 4, c, pos, 0.0f, true);
                pos += wl_step;
            }
        }
    }

    const int S = kS ? kS : p.S;
    const FragmentConsts fc = fcs;
    RF_STAT(unsigned long long st_iter = 0; unsigned long long st_whole = 0; unsigned long long st_frag = 0;
            unsigned long long st_frag_whole = 0; unsigned long long st_blocks = 0; unsigned long long st_zero = 0;
            unsigned long long st_zero_iter = 0; unsigned long long st_steps = 0;)
    // accumulators of the pixel blocks, [block * 3 + channel][lane]
    float* acc = blend + ((p.WS + 3) & ~3);
#pragma unroll
    for (int i = threadIdx.x; i < kBlocks * 96; i += kThreads) acc[i] = 0.0f;

    const int per_batch = kBatchRecords / p.WS;  // entries per batch (WS <= kBatchRecords)
    // Batches of records are double-buffered: while warps shade batch t from one buffer,
    // warps that are done build batch t + 1 in the other, one barrier per batch. Thread j
    // loads corner j % 4 of entry j / 4 (the four corners of an entry sit in one warp), one
    // batch ahead, into registers.
    const int my_entry = threadIdx.x >> 2, my_corner = threadIdx.x & 3;
    constexpr int kLoads = (kBatchRecords + 63) / 64;
    CornerLoad next[kLoads];
    int next_w[kLoads];
    bool have_next[kLoads];
    auto prefetch = [&](uint32_t first) {
#pragma unroll
        for (int h = 0; h < kLoads; h++) {
            const int e = my_entry + 64 * h;
            have_next[h] = e < per_batch && first + e < end;
            if (have_next[h]) {
                const uint32_t entry = tile_entries[first + e];
                next_w[h] = (int)(entry % p.maxW);
                load_corner(vtx, entry, my_corner, p, next[h]);
            }
        }
    };
    // records of the prefetched batch into dst, then prefetch the batch after it
    auto build = [&](Rec* dst, uint32_t first) {
#pragma unroll
        for (int h = 0; h < kLoads; h++) {
            const int e = my_entry + 64 * h;
            if (have_next[h])
                for (int i = 0; i < p.WS; i++)
                    store_corner(next[h], my_corner, blend[i], S, fc, dst[e * p.WS + i]);
        }
        __syncwarp();  // the four corners of each record are stored
#pragma unroll
        for (int h = 0; h < kLoads; h++) {
            const int e = my_entry + 64 * h;
            if (have_next[h])
                for (int i = my_corner; i < p.WS; i += 4) finish_record(p, next_w[h], i, xyz, dst[e * p.WS + i]);
        }
        prefetch(first + per_batch);
    };
    if (threadIdx.x == 0) {
        next_block[0] = 0;
        next_block[1] = 0;
    }
    prefetch(begin);
    __syncthreads();  // blend weights and colours are set
    if (begin < end) build(recbuf, begin);
    __syncthreads();
    int cur = 0;
    for (uint32_t base = begin; base < end; base += per_batch, cur ^= 1) {
        const int n_rec = (int)min((uint32_t)per_batch, end - base) * p.WS;
        const Rec* recs = recbuf + cur * kBatchRecords;
        // Warps take the tile's 8 x 4 blocks one at a time (blocks differ widely in work);
        // a block is shaded by one warp per batch, batches in order, so every pixel still
        // adds its records in increasing order.
#pragma unroll 1
        for (;;) {
            int blk = 0;
            if (lane == 0) blk = atomicAdd(&next_block[cur], 1);
            blk = __shfl_sync(0xffffffffu, blk, 0);
            if (blk >= kBlocks) break;
            RF_STAT(st_blocks += lane == 0;)
            const int x0 = tx * T + (blk % kCols) * 8, y0 = ty * T + (blk / kCols) * 4;
            const int px = x0 + (lane & 7), py = y0 + (lane >> 3);
            const int bx0 = x0 * S, by0 = y0 * S, bx1 = bx0 + 8 * S - 1, by1 = by0 + 4 * S - 1;
            const bool in_image = px < p.width && py < p.height;
            const int sx0 = px * S, sy0 = py * S;
            // which records can touch this 8 x 4 block, and which cover all of it: lanes
            // test 32 records at a time
            unsigned sel[kBatchRecords / 32], whole[kBatchRecords / 32];
#pragma unroll
            for (int m = 0; m < kBatchRecords / 32; m++) {
                const int j = m * 32 + lane;
                bool take = false, all = false;
                if (j < n_rec) {
                    const Rec& r = recs[j];
                    const int flags = ld4i(r.ec + 12).w;  // with ec[12..14], which rect_coverage reads
                    if (!(flags & 2)) {  // collinear (intersect_quad rejects all) or all-zero
                        const int4 bb = *reinterpret_cast<const int4*>(r.bb);
                        take = !(flags & 1) || !(bx1 < bb.x || bx0 > bb.y || by1 < bb.z || by0 > bb.w);
#if RF_RASTER_CLASSIFY
                        if (take && (flags & 1)) {
                            const int cov = rect_coverage(r, bx0, bx1, by0, by1);
                            take = cov != 0;
                            all = cov == 2;
                        }
#endif
                    }
                }
                sel[m] = __ballot_sync(0xffffffffu, take);
                whole[m] = __ballot_sync(0xffffffffu, all);
            }
            float r0 = acc[(3 * blk) * 32 + lane];
            float r1 = acc[(3 * blk + 1) * 32 + lane];
            float r2 = acc[(3 * blk + 2) * 32 + lane];
            // (no warp-wide operation below: lanes outside the image skip the records)
            if constexpr (kS == 1) {
                // One sample per pixel: every lane first marks the selected records that cover
                // its pixel (whole-block records cover every pixel; the others are tested, in a
                // loop that is the same for all lanes), then shades its own covered records in
                // increasing order. A lane is not held up by records that miss its pixel, so a
                // warp takes about as many shading steps as its busiest pixel has fragments.
                static_assert(kBatchRecords <= 64, "one 64-bit coverage mask per lane");
                unsigned long long cov = 0;
#pragma unroll
                for (int m = 0; m < kBatchRecords / 32; m++) {
                    unsigned c = whole[m], part = sel[m] & ~whole[m];
                    while (part) {
                        const int b = __ffs(part) - 1;
                        part &= part - 1;
                        if (inside(recs[m * 32 + b], sx0, sy0)) c |= 1u << b;
                    }
                    cov |= (unsigned long long)c << (32 * m);
                    RF_STAT(if (lane == 0) { st_iter += __popc(sel[m]); st_whole += __popc(whole[m]); })
                }
                if (!in_image) cov = 0;
                const float fx = (float)sx0, fy = (float)sy0;
                while (cov) {
                    const int j = __ffsll(cov) - 1;
                    cov &= cov - 1;
                    const Rec& r = recs[j];
                    RF_STAT(st_frag++; st_frag_whole += (whole[j >> 5] >> (j & 31)) & 1u;
                            if (lane == __ffs(__activemask()) - 1) st_steps++;)
                    float wt[4];
                    barycentric_fast(r, fx, fy, wt);
                    const float f = fragment_fast<kTex>(r, wt, ghost, p, fc, 1);
                    const float4 col = *reinterpret_cast<const float4*>(r.col);
                    r0 += col.x * f;
                    r1 += col.y * f;
                    r2 += col.z * f;
                }
            }
#pragma unroll
            for (int m = 0; m < kBatchRecords / 32 && in_image && kS != 1; m++) {
                unsigned bits = sel[m];
                while (bits) {  // in increasing record order: the reference's summation order
                    const int b = __ffs(bits) - 1;
                    const int j = m * 32 + b;
                    const bool is_whole = (whole[m] >> b) & 1u;
                    bits &= bits - 1;
                    const Rec& r = recs[j];
                    RF_STAT(if (lane == 0) { st_iter++; st_whole += is_whole; })
                    int hits = S;
                    if (!is_whole) {
                        // (a bounds test first would save nothing: the block was selected
                        // because the bounds touch it, so some lane tests coverage anyway)
                        hits = 0;
                        for (int s = 0; s < S; s++) hits += inside(r, sx0 + s, sy0 + SUB_OFFSETS[S - 1 + s]) ? 1 : 0;
                        if (hits == 0) continue;
                    }
                    RF_STAT(st_frag++; st_frag_whole += is_whole;)
                    float wt[4];
                    barycentric_fast(r, (float)(sx0 + S / 2), (float)(sy0 + S / 2), wt);
                    RF_STAT({
                        const float4 rl = ld4(r.rs);
                        const bool z = wt[0] * rl.x + wt[1] * rl.y + wt[2] * rl.z + wt[3] * rl.w <= 0.0f;
                        st_zero += z;
                        const unsigned am = __activemask();
                        if (__all_sync(am, z) && lane == __ffs(am) - 1) st_zero_iter++;
                    })
                    const float f = fragment_fast<kTex>(r, wt, ghost, p, fc, kS == 1 ? 1 : hits);
                    const float4 col = *reinterpret_cast<const float4*>(r.col);
                    r0 += col.x * f;
                    r1 += col.y * f;
                    r2 += col.z * f;
                }
            }
            acc[(3 * blk) * 32 + lane] = r0;
            acc[(3 * blk + 1) * 32 + lane] = r1;
            acc[(3 * blk + 2) * 32 + lane] = r2;
        }
        if (base + per_batch < end) build(recbuf + (cur ^ 1) * kBatchRecords, base + per_batch);
        // the other counter was last used by the previous batch, behind the last barrier
        if (threadIdx.x == 0) next_block[cur ^ 1] = 0;
        __syncthreads();
    }

    RF_STAT(atomicAdd(&g_raster_stats[0], st_iter); atomicAdd(&g_raster_stats[1], st_whole);
            atomicAdd(&g_raster_stats[2], st_frag); atomicAdd(&g_raster_stats[3], st_frag_whole);
            atomicAdd(&g_raster_stats[4], st_blocks); atomicAdd(&g_raster_stats[5], st_zero);
            atomicAdd(&g_raster_stats[6], st_zero_iter); atomicAdd(&g_raster_stats[7], st_steps);)
    __syncthreads();  // every block's last batch is shaded
    const float scale = p.intensity / (float)(p.W * p.S * p.WS);
#pragma unroll
    for (int k = 0; k < kBlocks / 8; k++) {
        const int blk = warp + 8 * k;
        const int px = tx * T + (blk % kCols) * 8 + (lane & 7), py = ty * T + (blk / kCols) * 4 + (lane >> 3);
        if (px >= p.width || py >= p.height) continue;
        const float c0 = acc[(3 * blk) * 32 + lane], c1 = acc[(3 * blk + 1) * 32 + lane],
                    c2 = acc[(3 * blk + 2) * 32 + lane];
        float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c0 > 0.0f || c1 > 0.0f || c2 > 0.0f) out = xyz_to_ap1(c0 * scale, c1 * scale, c2 * scale);
        image[(size_t)(p.height - (py + 1)) * p.width + px] = out;
    }
}

// One CTA per tile of a frame: CTA k shades tile order[k], or tile k without an order.
// CTAs start in index order as slots free up, so an order by decreasing work starts the
// heaviest tiles first and ends the launch with light ones.
template <int T, int kS, bool kTex>
__global__ void __launch_bounds__(kThreads, kS == 1 ? RF_RASTER_MIN_BLOCKS_S1 : RF_RASTER_MIN_BLOCKS)
    k_raster(const float4* __restrict__ vtx, const uint32_t* __restrict__ tile_offsets,
             const uint32_t* __restrict__ tile_entries, const uint32_t* __restrict__ order,
             const float* __restrict__ ghost, const float* __restrict__ spectrum, RasterParams p, FragmentConsts fcs,
             float4* __restrict__ image) {
    extern __shared__ float4 smem4[];
    __shared__ int next_block[2];  // blocks of each buffer's batch handed out so far
    const int tile = order ? (int)order[blockIdx.x] : (int)blockIdx.x;
    raster_tile<T, kS, kTex>(vtx, tile_offsets[tile], tile_offsets[tile + 1], tile_entries, ghost, spectrum, p, fcs,
                             image, tile % p.ntx, tile / p.ntx, smem4, next_block);
}

__host__ __device__ inline bool make_params(const rf_raster_args& a, RasterParams& p);
__host__ __device__ inline FragmentConsts fragment_consts(const RasterParams& p);

// Every frame of a batch in one persistent launch: each CTA takes the next tile from the
// queue (tiles ordered by decreasing entry count) until none are left. kTex: every frame's
// ghost lookups go through its rf_frame.ghost_texture.
template <int T, int kS, bool kTex>
__global__ void __launch_bounds__(kThreads, kS == 1 ? RF_RASTER_MIN_BLOCKS_S1 : RF_RASTER_MIN_BLOCKS)
    k_raster_batch(const rf_frame* __restrict__ frames, int F, int tiles, const uint32_t* __restrict__ order,
                   unsigned* __restrict__ queue, const unsigned long long* __restrict__ entry_total,
                   long long capacity, const float4* __restrict__ vtx_all, const uint32_t* __restrict__ tile_offsets,
                   const uint32_t* __restrict__ tile_entries, const float* __restrict__ ghosts,
                   const float* __restrict__ spectrum, float4* __restrict__ images) {
    extern __shared__ float4 smem4[];
    __shared__ int next_block[2];
    // the current tile's frame settings, held in shared memory rather than registers
    __shared__ RasterParams sp;
    __shared__ FragmentConsts sfc;
    __shared__ int item, s_tile, s_gt;
    __shared__ long long s_vtx, s_ghost, s_image;
    if (*entry_total > (unsigned long long)capacity) return;  // incomplete lists: nothing is drawn
    for (;;) {
        if (threadIdx.x == 0) {
            item = (int)atomicAdd(queue, 1u);
            if (item < tiles) {
                const int gt = (int)order[item];
                const int f = find_frame(frames, F, gt, [](const rf_frame& fr) { return fr.tile_offset; });
                const rf_frame& fr = frames[f];
                RasterParams q;
                make_params(fr.raster, q);
                if (kTex) q.ghost_tex = fr.ghost_texture;
                q.T = T;
                q.ntx = (q.width + T - 1) / T;
                sp = q;
                sfc = fragment_consts(q);
                s_gt = gt;
                s_tile = gt - fr.tile_offset;
                s_vtx = fr.vertex_offset;
                s_ghost = fr.ghost_offset;
                s_image = fr.image_offset;
            }
        }
        __syncthreads();
        if (item >= tiles) break;
        const int gt = s_gt, tile = s_tile;
        raster_tile<T, kS, kTex>(vtx_all + 2 * s_vtx, tile_offsets[gt], tile_offsets[gt + 1], tile_entries,
                           ghosts + s_ghost, spectrum, sp, sfc, images + s_image, tile % sp.ntx, tile / sp.ntx, smem4,
                           next_block);
        __syncthreads();  // the tile's accumulators and `item` are free again
    }
}

// ---------------------------------------------------------------- adjoint
// ghost_sample with its derivatives with respect to the texel coordinates (u, v).
__device__ __forceinline__ float ghost_sample_grad(const float* __restrict__ tex, int w, int h, float u, float v,
                                                   float& du, float& dv) {
    du = dv = 0.0f;
    if (!(fabsf(u) < 1e9f) || !(fabsf(v) < 1e9f)) return 0.0f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const int i0 = (int)fu, j0 = (int)fv;
    const bool i0_in = (unsigned)i0 < (unsigned)w, i1_in = (unsigned)(i0 + 1) < (unsigned)w;
    const bool j0_in = (unsigned)j0 < (unsigned)h, j1_in = (unsigned)(j0 + 1) < (unsigned)h;
    const int ia = min(max(i0, 0), w - 1), ib = min(max(i0 + 1, 0), w - 1);
    const float* row0 = tex + (size_t)min(max(j0, 0), h - 1) * w;
    const float* row1 = tex + (size_t)min(max(j0 + 1, 0), h - 1) * w;
    const float t00 = (i0_in && j0_in) ? __ldg(row0 + ia) : 0.0f;
    const float t10 = (i1_in && j0_in) ? __ldg(row0 + ib) : 0.0f;
    const float t01 = (i0_in && j1_in) ? __ldg(row1 + ia) : 0.0f;
    const float t11 = (i1_in && j1_in) ? __ldg(row1 + ib) : 0.0f;
    du = (1.0f - b) * (t10 - t00) + b * (t11 - t01);
    dv = (1.0f - a) * (t01 - t00) + a * (t11 - t10);
    return (1.0f - a) * (1.0f - b) * t00 + a * (1.0f - b) * t10 + (1.0f - a) * b * t01 + a * b * t11;
}

// ghost_sample_grad with the four texels from one gather of the ghost texture's texture object
// (border mode: texels outside the texture read 0, as the loads' bounds checks give).
__device__ __forceinline__ float ghost_sample_grad_tex(unsigned long long tex, float u, float v, float& du,
                                                       float& dv) {
    du = dv = 0.0f;
    if (!(fabsf(u) < 1e9f) || !(fabsf(v) < 1e9f)) return 0.0f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const float4 g = tex2Dgather<float4>((cudaTextureObject_t)tex, fu + 1.0f, fv + 1.0f, 0);
    const float t00 = g.w, t10 = g.z, t01 = g.x, t11 = g.y;
    du = (1.0f - b) * (t10 - t00) + b * (t11 - t01);
    dv = (1.0f - a) * (t01 - t00) + a * (t11 - t10);
    return (1.0f - a) * (1.0f - b) * t00 + a * (1.0f - b) * t10 + (1.0f - a) * b * t01 + a * b * t11;
}

constexpr int kGradAttrs = 5;  // per corner: u, v, rrel, reflectance, intensity
// row stride of the backward's per-warp transpose buffers (floats)
constexpr int kRedStride = 36;
// rows of a warp's transpose buffer: the 5 attribute gradients and the 4 corner weights
constexpr int kRedRows = kGradAttrs + 4;
// vertex float of each attribute (pos.xy, uv.xy, rrel, reflectance, intensity, pad)
__device__ __constant__ static const int kGradSlot[kGradAttrs] = {2, 3, 4, 5, 6};

// Backward of k_raster (32 x 32 or 16 x 16 tiles): the same tiles, entry lists, records, coverage
// and mean-value weights as the forward (held fixed: they are piecewise constant in the
// vertex positions), differentiating each fragment with respect to the attributes its
// corners interpolate. Per record the warp sums its pixels' contributions through a
// shared-memory transpose; the CTA sums warps in shared memory and adds each record's totals to the two vertices
// (wavelength pair endpoints) of each corner once per tile. kTex: the ghost lookups gather
// from the texture object p.ghost_tex.
template <int T, int kS, bool kTex>
__global__ void __launch_bounds__(kThreads, kS == 1 ? 3 : 2)
    k_raster_backward(const float4* __restrict__ vtx, const uint32_t* __restrict__ tile_offsets,
                      const uint32_t* __restrict__ tile_entries, const float* __restrict__ ghost,
                      const float* __restrict__ spectrum, RasterParams p, FragmentConsts fc,
                      const float4* __restrict__ image, const float4* __restrict__ grad_image,
                      float* __restrict__ grad_vtx) {
    constexpr int kBlocks = T * T / 32, kCols = T / 8;
    extern __shared__ float4 smem4[];
    Rec* recbuf = (Rec*)smem4;  // two batches of records
    // Where each record's gradients go: the vertex index of corner 0 at the pair's first
    // wavelength and the sub-step's blend weight, set when the record is built and read by the
    // batch's flush. Three batches' worth: the build of batch t + 2 may run while slower warps
    // still flush batch t, and the build of t + 3 comes after the barrier of t + 1.
    long long* vbase_buf = (long long*)(recbuf + 2 * kBatchRecords);  // [3][kBatchRecords]
    float* tbuf = (float*)(vbase_buf + 3 * kBatchRecords);            // [3][kBatchRecords]
    // per-warp transpose buffers of each lane's 5 attribute gradients and 4 corner weights:
    // [row][lane], rows kRedStride floats apart (16-byte aligned, and the rows that lanes read
    // side by side fall in different bank groups)
    float* red = (tbuf + 3 * kBatchRecords) + (threadIdx.x >> 5) * (kRedRows * kRedStride);
    float* xyz = (tbuf + 3 * kBatchRecords) + 8 * kRedRows * kRedStride;
    float* blend = xyz + 3 * p.maxW * p.WS;
    float* grgb = blend + ((p.WS + 3) & ~3);          // [block * 3 + channel][lane]: dL / d(linear XYZ sum)
    float* rgrad_buf = grgb + 96 * kBlocks;            // two batches of [record][corner * 5 + attribute]
    __shared__ int next_block[2];
    const int tile = blockIdx.x;
    const int tx = tile % p.ntx, ty = tile / p.ntx;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        const float sub_step = 1.0f / (float)p.WS;
        float b = 0.0f;
        for (int i = 0; i < p.WS; i++) {
            blend[i] = b;
            b += sub_step;
        }
    }
    if (p.W > 1) {
        const float sub_step = 1.0f / (float)p.WS;
        const float wl_step = sub_step / (float)p.W;
        for (int w = threadIdx.x; w < p.maxW; w += kThreads) {
            float pos = ((float)w + 0.5f) / (float)p.W;
            for (int i = 0; i < p.WS; i++) {
                for (int c = 0; c < 3; c++)
                    xyz[3 * (w * p.WS + i) + c] = sample_linear(spectrum, RF_SPECTRUM_WIDTH, 1, 4, c, pos, 0.0f, true);
                pos += wl_step;
            }
        }
    }
    // out = AP1(rgb * scale) where any channel of rgb is positive, else 0
    const float scale = p.intensity / (float)(p.W * p.S * p.WS);
    const float4 m0 = xyz_to_ap1(1.0f, 0.0f, 0.0f), m1 = xyz_to_ap1(0.0f, 1.0f, 0.0f),
                 m2 = xyz_to_ap1(0.0f, 0.0f, 1.0f);
#pragma unroll
    for (int k = 0; k < kBlocks / 8; k++) {
        const int blk = warp + 8 * k;
        const int px = tx * T + (blk % kCols) * 8 + (lane & 7), py = ty * T + (blk / kCols) * 4 + (lane >> 3);
        float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f;
        if (px < p.width && py < p.height) {
            const size_t o = (size_t)(p.height - (py + 1)) * p.width + px;
            const float4 out = image[o], g = grad_image[o];
            if (out.x != 0.0f || out.y != 0.0f || out.z != 0.0f) {
                g0 = scale * (m0.x * g.x + m0.y * g.y + m0.z * g.z);
                g1 = scale * (m1.x * g.x + m1.y * g.y + m1.z * g.z);
                g2 = scale * (m2.x * g.x + m2.y * g.y + m2.z * g.z);
            }
        }
        grgb[(3 * blk) * 32 + lane] = g0;
        grgb[(3 * blk + 1) * 32 + lane] = g1;
        grgb[(3 * blk + 2) * 32 + lane] = g2;
    }
    for (int i = threadIdx.x; i < 2 * kBatchRecords * 4 * kGradAttrs; i += kThreads) rgrad_buf[i] = 0.0f;

    const int S = kS ? kS : p.S;
    const uint32_t begin = tile_offsets[tile], end = tile_offsets[tile + 1];
    const int per_batch = kBatchRecords / p.WS;
    const int my_entry = threadIdx.x >> 2, my_corner = threadIdx.x & 3;
    const int Q = (p.G - 1) * (p.G - 1), VC = p.G * p.G;
    // Records of the batch at `first` into buffer `dst`, as k_raster builds them: thread j
    // loads and mixes corner j % 4 of entry j / 4 (the four corners of an entry sit in one
    // warp), then one thread per record finishes it. Batches are double-buffered: warps that
    // are done shading batch t build batch t + 1 while the others shade, one barrier per
    // batch, and each batch sums its records' gradients in its own buffer.
    auto build = [&](Rec* dst, uint32_t first, int slot) {
        for (int h = 0; h < (kBatchRecords + 63) / 64; h++) {
            const int e = my_entry + 64 * h;
            if (e < per_batch && first + e < end) {
                const uint32_t entry = tile_entries[first + e];
                CornerLoad c;
                load_corner(vtx, entry, my_corner, p, c);
                for (int i = 0; i < p.WS; i++) store_corner(c, my_corner, blend[i], S, fc, dst[e * p.WS + i]);
                if (my_corner == 0) {  // where the record's gradients go (the batch's flush)
                    const long long prim = entry / p.maxW;
                    const int w = (int)(entry % p.maxW);
                    const int quad = (int)(prim % Q);
                    const long long v0 = ((prim / Q) * VC + (quad / (p.G - 1)) * p.G + quad % (p.G - 1)) * p.W + w;
                    for (int i = 0; i < p.WS; i++) {
                        vbase_buf[slot * kBatchRecords + e * p.WS + i] = v0;
                        tbuf[slot * kBatchRecords + e * p.WS + i] = blend[i];
                    }
                }
            }
        }
        __syncwarp();  // the four corners of each record are stored
        for (int h = 0; h < (kBatchRecords + 63) / 64; h++) {
            const int e = my_entry + 64 * h;
            if (e < per_batch && first + e < end) {
                const uint32_t entry = tile_entries[first + e];
                for (int i = my_corner; i < p.WS; i += 4) finish_record(p, (int)(entry % p.maxW), i, xyz, dst[e * p.WS + i]);
            }
        }
    };
    if (threadIdx.x == 0) {
        next_block[0] = 0;
        next_block[1] = 0;
    }
    __syncthreads();  // blend weights, colours and pixel gradients are set
    if (begin < end) build(recbuf, begin, 0);
    __syncthreads();
    int cur = 0, slot = 0;  // record buffer (batch parity) and flush slot (batch index mod 3)
    for (uint32_t base = begin; base < end; base += per_batch, cur ^= 1, slot = slot == 2 ? 0 : slot + 1) {
        const int n_rec = (int)min((uint32_t)per_batch, end - base) * p.WS;
        const Rec* recs = recbuf + cur * kBatchRecords;
        float* rgrad = rgrad_buf + cur * (kBatchRecords * 4 * kGradAttrs);
#pragma unroll 1
        for (;;) {
            int blk = 0;
            if (lane == 0) blk = atomicAdd(&next_block[cur], 1);
            blk = __shfl_sync(0xffffffffu, blk, 0);
            if (blk >= kBlocks) break;
            const int x0 = tx * T + (blk % kCols) * 8, y0 = ty * T + (blk / kCols) * 4;
            const int px = x0 + (lane & 7), py = y0 + (lane >> 3);
            const int bx0 = x0 * S, by0 = y0 * S, bx1 = bx0 + 8 * S - 1, by1 = by0 + 4 * S - 1;
            const bool in_image = px < p.width && py < p.height;
            const int sx0 = px * S, sy0 = py * S;
            const float g0 = grgb[(3 * blk) * 32 + lane], g1 = grgb[(3 * blk + 1) * 32 + lane],
                        g2 = grgb[(3 * blk + 2) * 32 + lane];
            const bool any_grad = __any_sync(0xffffffffu, g0 != 0.0f || g1 != 0.0f || g2 != 0.0f);
            if (!any_grad) continue;
            unsigned sel[kBatchRecords / 32], whole[kBatchRecords / 32];
#pragma unroll
            for (int m = 0; m < kBatchRecords / 32; m++) {
                const int j = m * 32 + lane;
                bool take = false, all = false;
                if (j < n_rec) {
                    const Rec& r = recs[j];
                    const int flags = ld4i(r.ec + 12).w;  // with ec[12..14], which rect_coverage reads
                    if (!(flags & 2)) {
                        const int4 bb = *reinterpret_cast<const int4*>(r.bb);
                        take = !(flags & 1) || !(bx1 < bb.x || bx0 > bb.y || by1 < bb.z || by0 > bb.w);
                        if (take && (flags & 1)) {
                            const int cov = rect_coverage(r, bx0, bx1, by0, by1);
                            take = cov != 0;
                            all = cov == 2;
                        }
                    }
                }
                sel[m] = __ballot_sync(0xffffffffu, take);
                whole[m] = __ballot_sync(0xffffffffu, all);
            }
#pragma unroll
            for (int m = 0; m < kBatchRecords / 32; m++) {
                unsigned bits = sel[m];
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    const int j = m * 32 + b;
                    bits &= bits - 1;
                    const Rec& r = recs[j];
                    int hits = 0;
                    if (in_image) {
                        if ((whole[m] >> b) & 1u) {
                            hits = S;
                        } else {
                            for (int s = 0; s < S; s++) hits += inside(r, sx0 + s, sy0 + SUB_OFFSETS[S - 1 + s]) ? 1 : 0;
                        }
                    }
                    if (!__any_sync(0xffffffffu, hits > 0)) continue;
                    float gw[kGradAttrs] = {0.f, 0.f, 0.f, 0.f, 0.f};
                    float wt[4] = {0.f, 0.f, 0.f, 0.f};
                    if (hits > 0) {
                        barycentric_fast(r, (float)(sx0 + S / 2), (float)(sy0 + S / 2), wt);
                        float dLdf;
                        if (p.W > 1) {
                            const float* c = xyz + 3 * r.color;
                            dLdf = g0 * c[0] + g1 * c[1] + g2 * c[2];
                        } else {
                            dLdf = g0 + g1 + g2;
                        }
                        const float4 uv01 = ld4(r.uv), uv23 = ld4(r.uv + 4);
                        const float u = wt[0] * uv01.x + wt[1] * uv01.z + wt[2] * uv23.x + wt[3] * uv23.z;
                        const float v = wt[0] * uv01.y + wt[1] * uv01.w + wt[2] * uv23.y + wt[3] * uv23.w;
                        float dgu, dgv;
                        const float gi = kTex ? ghost_sample_grad_tex(p.ghost_tex, u, v, dgu, dgv)
                                              : ghost_sample_grad(ghost, p.ghost_w, p.ghost_h, u, v, dgu, dgv);
                        const float4 rl = ld4(r.rs);
                        const float st = __saturatef(wt[0] * rl.x + wt[1] * rl.y + wt[2] * rl.z + wt[3] * rl.w);
                        const float ri = st * st * (3.0f - 2.0f * st);
                        const float dri = (st > 0.0f && st < 1.0f) ? 6.0f * st * (1.0f - st) * (1.0f / (0.95f - 1.0f))
                                                                  : 0.0f;
                        const float4 in = ld4(r.inten), rf = ld4(r.refl);
                        const float ai_raw = wt[0] * in.x + wt[1] * in.y + wt[2] * in.z + wt[3] * in.w;
                        const float ci_raw = wt[0] * rf.x + wt[1] * rf.y + wt[2] * rf.z + wt[3] * rf.w;
                        const float ai = fmaxf(ai_raw, 0.0f), ci = fmaxf(ci_raw, 0.0f);
                        const float H = (float)hits;
                        const float d = dLdf * H;
                        gw[0] = d * ri * ai * ci * dgu * fc.tsx;
                        gw[1] = d * ri * ai * ci * dgv * fc.tsy;
                        gw[2] = d * gi * ai * ci * dri;
                        gw[3] = ci_raw > 0.0f ? d * gi * ri * ai : 0.0f;
                        gw[4] = ai_raw > 0.0f ? d * gi * ri * ci : 0.0f;
                    }
                    // the warp's sum of each corner attribute's gradient, sum over lanes of
                    // gw[a] * wt[c]: every lane writes its 5 attribute gradients and 4 weights
                    // (rows 0-4 and 5-8), lane k < 20 forms column (a, c) = (k % 5, k / 5)
#pragma unroll
                    for (int a = 0; a < kGradAttrs; a++) red[a * kRedStride + lane] = gw[a];
#pragma unroll
                    for (int c = 0; c < 4; c++) red[(kGradAttrs + c) * kRedStride + lane] = wt[c];
                    __syncwarp();
                    if (lane < 4 * kGradAttrs) {
                        const int a = lane % kGradAttrs, c = lane / kGradAttrs;
                        const float4* ga = reinterpret_cast<const float4*>(red + a * kRedStride);
                        const float4* wc = reinterpret_cast<const float4*>(red + (kGradAttrs + c) * kRedStride);
                        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
#pragma unroll
                        for (int q = 0; q < 8; q++) {
                            const float4 g = ga[q], v = wc[q];
                            s0 = fmaf(g.x, v.x, s0);
                            s1 = fmaf(g.y, v.y, s1);
                            s2 = fmaf(g.z, v.z, s2);
                            s3 = fmaf(g.w, v.w, s3);
                        }
                        const float sum = (s0 + s1) + (s2 + s3);
                        if (sum != 0.0f) atomicAdd(&rgrad[j * 4 * kGradAttrs + lane], sum);
                    }
                    __syncwarp();
                }
            }
        }
        if (base + per_batch < end) build(recbuf + (cur ^ 1) * kBatchRecords, base + per_batch, slot == 2 ? 0 : slot + 1);
        // the other counter was last used by the previous batch, behind the last barrier
        if (threadIdx.x == 0) next_block[cur ^ 1] = 0;
        __syncthreads();  // every block of this batch is shaded and the next batch is built
        // each record's gradients to the two vertices of each corner (mix_vertex weights);
        // the buffer is cleared here and written again two batches later, behind the next
        // barrier
        for (int idx = threadIdx.x; idx < n_rec * 4 * kGradAttrs; idx += kThreads) {
            const float g = rgrad[idx];
            if (g == 0.0f) continue;
            rgrad[idx] = 0.0f;
            const int j = idx / (4 * kGradAttrs), rem = idx % (4 * kGradAttrs);
            const int corner = rem / kGradAttrs, a = rem % kGradAttrs;
            const float t = tbuf[slot * kBatchRecords + j];
            const int offset = corner == 0 ? 0 : (corner == 1 ? 1 : (corner == 2 ? 1 + p.G : p.G));
            const long long vi = vbase_buf[slot * kBatchRecords + j] + (long long)offset * p.W;
            atomicAdd(grad_vtx + 8 * vi + kGradSlot[a], g * (1.0f - t));
            atomicAdd(grad_vtx + 8 * (vi + 1) + kGradSlot[a], g * t);
        }
    }
}

// The reference's own loop: every pixel scans every mask of its bin (rasterizing.cl:573-654).
__global__ void __launch_bounds__(256) k_raster_masks(const float4* __restrict__ vtx,
                                                      const unsigned long long* __restrict__ masks, int batch_count,
                                                      int B, long long prim_total, const float* __restrict__ ghost,
                                                      const float* __restrict__ spectrum, RasterParams p,
                                                      FragmentConsts fc, float4* __restrict__ image) {
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= p.width || y >= p.height) return;
    const int bdx = (p.width + B - 1) / B;
    const int bin = (y / B) * bdx + (x / B);
    const int S = p.S;
    const int sx0 = x * S, sy0 = y * S;
    const float sub_step = 1.0f / (float)p.WS;
    const float wl_step = sub_step / (float)p.W;
    const int Q = (p.G - 1) * (p.G - 1), VC = p.G * p.G;
    float rgb[3] = {0.f, 0.f, 0.f};
    Rec r;
    for (int batch = 0; batch < batch_count; batch++) {
        const unsigned long long* q = masks + 4 * ((size_t)bin * batch_count + batch);
        if ((q[0] & 1ull) == 0) continue;
        for (int k = 0; k < RF_BATCH_PRIMITIVE_COUNT; k++) {
            const long long prim = (long long)batch * RF_BATCH_PRIMITIVE_COUNT + k;
            if (prim >= prim_total) continue;
            const int bit = k + 1;
            if (!((q[bit >> 6] >> (bit & 63)) & 1ull)) continue;
            const long long path = prim / Q;
            const int quad = (int)(prim % Q);
            const int row = quad / (p.G - 1), col = quad % (p.G - 1);
            const int c0 = row * p.G + col;
            const int corners[4] = {c0, c0 + 1, c0 + 1 + p.G, c0 + p.G};
            for (int w = 0; w < p.maxW; w++) {
                float sub_pos = 0.0f;
                float wl_pos = ((float)w + 0.5f) / (float)p.W;
                for (int i = 0; i < p.WS; i++) {
                    // the full record, no skipping of invalid endpoints
                    for (int c = 0; c < 4; c++) {
                        const long long vi = (path * VC + corners[c]) * p.W + w;
                        const float4 a0 = vtx[2 * vi], a1 = vtx[2 * vi + 1], b0 = vtx[2 * vi + 2], b1 = vtx[2 * vi + 3];
                        const float px = a0.x + (b0.x - a0.x) * sub_pos, py = a0.y + (b0.y - a0.y) * sub_pos;
                        r.uv[2 * c] = (a0.z + (b0.z - a0.z) * sub_pos) * fc.tsx + fc.tox;
                        r.uv[2 * c + 1] = (a0.w + (b0.w - a0.w) * sub_pos) * fc.tsy + fc.toy;
                        r.rs[c] = ((a1.x + (b1.x - a1.x) * sub_pos) - 1.0f) * kRampScale;
                        r.refl[c] = a1.y + (b1.y - a1.y) * sub_pos;
                        r.inten[c] = a1.z + (b1.z - a1.z) * sub_pos;
                        r.q[2 * c] = cvt_rz_sat(px * (float)S);
                        r.q[2 * c + 1] = cvt_rz_sat(py * (float)S);
                        r.qf[2 * c] = (float)r.q[2 * c];
                        r.qf[2 * c + 1] = (float)r.q[2 * c + 1];
                    }
                    const int* qq = r.q;
                    edge_coeffs(qq[0], qq[1], qq[2], qq[3], r.ec + 0);
                    edge_coeffs(qq[2], qq[3], qq[4], qq[5], r.ec + 3);
                    edge_coeffs(qq[4], qq[5], qq[6], qq[7], r.ec + 6);
                    edge_coeffs(qq[6], qq[7], qq[0], qq[1], r.ec + 9);
                    edge_coeffs(qq[4], qq[5], qq[0], qq[1], r.ec + 12);
                    const bool never = edge_i(qq[0], qq[1], qq[2], qq[3], qq[4], qq[5]) == 0 &&
                                       edge_i(qq[0], qq[1], qq[4], qq[5], qq[6], qq[7]) == 0;
                    int hits = 0;
                    if (!never)
                        for (int s = 0; s < S; s++) hits += inside(r, sx0 + s, sy0 + SUB_OFFSETS[S - 1 + s]) ? 1 : 0;
                    float f = 0.0f;
                    if (hits > 0) {
                        float wt[4];
                        barycentric_fast(r, (float)(sx0 + S / 2), (float)(sy0 + S / 2), wt);
                        f += fragment_fast(r, wt, ghost, p, fc, hits);
                    }
                    if (p.W > 1) {
                        for (int c = 0; c < 3; c++)
                            rgb[c] += sample_linear(spectrum, RF_SPECTRUM_WIDTH, 1, 4, c, wl_pos, 0.0f, true) * f;
                    } else {
                        rgb[0] += f;
                        rgb[1] += f;
                        rgb[2] += f;
                    }
                    sub_pos += sub_step;
                    wl_pos += wl_step;
                }
            }
        }
    }
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (rgb[0] > 0.0f || rgb[1] > 0.0f || rgb[2] > 0.0f) {
        const float scale = p.intensity / (float)(p.W * p.S * p.WS);
        out = xyz_to_ap1(rgb[0] * scale, rgb[1] * scale, rgb[2] * scale);
    }
    image[(size_t)(p.height - (y + 1)) * p.width + x] = out;
}

__host__ __device__ inline bool make_params(const rf_raster_args& a, RasterParams& p) {
    if (a.width < 1 || a.height < 1 || a.grid_count < 2 || a.wavelength_count < 1 || a.wavelength_sub_count < 1 ||
        a.path_count < 0 || a.ghost_width < 1 || a.ghost_height < 1)
        return false;
    if (a.sub_steps != 1 && a.sub_steps != 2 && a.sub_steps != 4 && a.sub_steps != 8) return false;
    p.width = a.width;
    p.height = a.height;
    p.S = a.sub_steps;
    p.W = a.wavelength_count;
    p.WS = a.wavelength_sub_count;
    p.G = a.grid_count;
    p.maxW = a.wavelength_count - 1 > 1 ? a.wavelength_count - 1 : 1;
    p.intensity = a.intensity;
    p.ghost_scale = a.ghost_scale;
    p.ghost_w = a.ghost_width;
    p.ghost_h = a.ghost_height;
    p.safe_screen = (float)a.width * a.sub_steps <= 16384.0f && (float)a.height * a.sub_steps <= 16384.0f;
    p.ghost_tex = 0;  // the texels are loaded unless a launcher sets a texture object
    return true;
}

// Raise a kernel's dynamic shared-memory limit once per device and size, so that later
// launches of it can be captured into a CUDA graph without further attribute calls.
constexpr int kMaxDevices = 64;
template <class K>
int allow_smem(K kernel, size_t bytes, std::atomic<size_t>* allowed) {
    if (bytes <= 48 * 1024) return RF_OK;
    int dev = 0;
    RF_TRY(cuda_status(cudaGetDevice(&dev)));
    if (dev < 0 || dev >= kMaxDevices) return RF_ERR_NOT_SUPPORTED;
    if (bytes <= allowed[dev].load()) return RF_OK;
    RF_TRY(cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes)));
    allowed[dev].store(bytes);
    return RF_OK;
}

// A texture object over a caller's ghost texture (float texels, pitch w * 4 bytes, border
// address mode, point filtering, unnormalised coordinates) for ghost_sample_tex, created once
// per device, address and size and kept (at most kMaxGhostTextures; rf_ghost_textures_forget
// drops a device's objects after a device reset). 0 when the address or the row pitch is not
// aligned as textures require, or past the cap; the raster then loads texels.
constexpr size_t kMaxGhostTextures = 4096;
struct GhostTextureEntry {
    int dev;
    const float* ptr;
    int w, h;
    cudaTextureObject_t obj;
};
std::mutex ghost_texture_mutex;
std::vector<GhostTextureEntry> ghost_texture_cache;

unsigned long long ghost_texture_object(const float* ghost, int w, int h) {
    using Entry = GhostTextureEntry;
    std::mutex& mutex = ghost_texture_mutex;
    std::vector<Entry>& cache = ghost_texture_cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::lock_guard<std::mutex> lock(mutex);
    for (const Entry& e : cache)
        if (e.dev == dev && e.ptr == ghost && e.w == w && e.h == h) return e.obj;
    // the row pitch must be a multiple of the texture pitch alignment, the base address a
    // multiple of the texture alignment
    int pitch_align = 0, base_align = 0;
    if (cudaDeviceGetAttribute(&pitch_align, cudaDevAttrTexturePitchAlignment, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&base_align, cudaDevAttrTextureAlignment, dev) != cudaSuccess || pitch_align <= 0 ||
        base_align <= 0)
        return 0;
    if (((size_t)w * sizeof(float)) % (size_t)pitch_align != 0 || (uintptr_t)ghost % (uintptr_t)base_align != 0)
        return 0;
    // Objects are kept for the life of the process (one per device, address and size; a
    // kernel in flight may still use any of them, and no synchronisation is allowed here:
    // a caller may be capturing a graph). Past the cap the raster loads the texels.
    if (cache.size() >= kMaxGhostTextures) return 0;
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypePitch2D;
    rd.res.pitch2D.devPtr = const_cast<float*>(ghost);
    rd.res.pitch2D.desc = cudaCreateChannelDesc<float>();
    rd.res.pitch2D.width = (size_t)w;
    rd.res.pitch2D.height = (size_t)h;
    rd.res.pitch2D.pitchInBytes = (size_t)w * sizeof(float);
    cudaTextureDesc td = {};
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    cudaTextureObject_t obj = 0;
    if (cudaCreateTextureObject(&obj, &rd, &td, nullptr) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    cache.push_back({dev, ghost, w, h, obj});
    return obj;
}

template <int T, int kS>
int launch_raster_s(const float* vertexes, const uint32_t* offsets, const uint32_t* entries, const uint32_t* order,
                    const float* ghost, const float* spectrum, RasterParams p, float* image, cudaStream_t s) {
    static std::atomic<size_t> allowed[kMaxDevices];
    static std::atomic<size_t> allowed_tex[kMaxDevices];
    p.T = T;
    p.ntx = (p.width + T - 1) / T;
    const int nty = (p.height + T - 1) / T;
    const size_t smem = raster_smem_bytes<T>(p.maxW, p.WS);
    p.ghost_tex = ghost_texture_object(ghost, p.ghost_w, p.ghost_h);
    if (p.ghost_tex) {
        RF_TRY(allow_smem(k_raster<T, kS, true>, smem, allowed_tex));
        k_raster<T, kS, true><<<p.ntx * nty, kThreads, smem, s>>>((const float4*)vertexes, offsets, entries, order,
                                                                 ghost, spectrum, p, fragment_consts(p),
                                                                 (float4*)image);
    } else {
        RF_TRY(allow_smem(k_raster<T, kS, false>, smem, allowed));
        k_raster<T, kS, false><<<p.ntx * nty, kThreads, smem, s>>>((const float4*)vertexes, offsets, entries, order,
                                                                  ghost, spectrum, p, fragment_consts(p),
                                                                  (float4*)image);
    }
    return launch_status();
}

template <int T>
int launch_raster(const float* vertexes, const uint32_t* offsets, const uint32_t* entries, const uint32_t* order,
                  const float* ghost, const float* spectrum, RasterParams p, float* image, cudaStream_t s) {
    if (p.S == 1) return launch_raster_s<T, 1>(vertexes, offsets, entries, order, ghost, spectrum, p, image, s);
    return launch_raster_s<T, 0>(vertexes, offsets, entries, order, ghost, spectrum, p, image, s);
}

template <int T, int kS, bool kTex>
int launch_raster_batch(const rf_frame* frames, const rf_batch_sizes& z, const float* vertexes,
                        const uint32_t* tile_offsets, const uint32_t* tile_entries, const float* ghosts,
                        const float* spectrum, const BatchWorkspace& w, long long capacity,
                        const uint64_t* entry_total, float* images, cudaStream_t s) {
    static std::atomic<size_t> allowed[kMaxDevices];
    static std::atomic<int> ctas_per_sm[kMaxDevices];
    // the largest frame layout: 3 * max(W-1,1) * WS colours, WS blend weights (rounded to 4)
    const size_t smem = sizeof(Rec) * 2 * kBatchRecords + sizeof(float) * (3 * z.max_colors + ((z.max_sub + 3) & ~3)) +
                        sizeof(float) * 96 * (T * T / 32);
    RF_TRY(allow_smem(k_raster_batch<T, kS, kTex>, smem, allowed));
    int dev = 0, sms = 0;
    RF_TRY(cuda_status(cudaGetDevice(&dev)));
    RF_TRY(cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)));
    int per_sm = ctas_per_sm[dev].load();
    if (per_sm == 0) {
        RF_TRY(cuda_status(
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_raster_batch<T, kS, kTex>, kThreads, smem)));
        per_sm = per_sm > 0 ? per_sm : 1;
        ctas_per_sm[dev].store(per_sm);
    }
    const long long ctas = std::min<long long>((long long)sms * per_sm, z.tiles);
    RF_TRY(cuda_status(cudaMemsetAsync(w.queue, 0, sizeof(uint32_t), s)));
    k_raster_batch<T, kS, kTex><<<(unsigned)ctas, kThreads, smem, s>>>(
        frames, z.frame_count, z.tiles, batch_tile_order(w, z), w.queue, (const unsigned long long*)entry_total,
        capacity, (const float4*)vertexes, tile_offsets, tile_entries, ghosts, spectrum, (float4*)images);
    return launch_status();
}

}  // namespace
}  // namespace rf

extern "C" int rf_raster_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const float* vertexes,
                               const uint32_t* tile_offsets, const uint32_t* tile_entries, const float* ghosts,
                               const float* spectrum, void* workspace, size_t workspace_bytes,
                               int64_t entry_capacity, const uint64_t* entry_total, float* images, void* stream) {
    using namespace rf;
    if (!frames || !sizes || !vertexes || !tile_offsets || !tile_entries || !ghosts || !spectrum || !workspace ||
        !entry_total || !images || entry_capacity < 1)
        return RF_ERR_INVALID_ARG;
    if (!aligned16(vertexes) || !aligned16(images) || !aligned16(workspace)) return RF_ERR_INVALID_ARG;
    const rf_batch_sizes& z = *sizes;
    if (z.tiles < 1) return RF_OK;
    if (z.max_sub < 1 || z.max_sub > kBatchRecords || z.max_colors > 4096) return RF_ERR_INVALID_ARG;
    BatchWorkspace w = batch_layout((char*)workspace, z, entry_capacity);
    if (w.bytes > workspace_bytes) return RF_ERR_INVALID_ARG;
    const bool one = z.max_sub_steps <= 1;  // every frame takes one sample per pixel
    cudaStream_t s = (cudaStream_t)stream;
#define RF_BATCH_LAUNCH(T, S, X)                                                                              \
    launch_raster_batch<T, S, X>(frames, z, vertexes, tile_offsets, tile_entries, ghosts, spectrum, w, entry_capacity, \
                                 entry_total, images, s)
    const bool tex = z.ghost_textures != 0;
    switch (z.tile_size) {
        case 32:
            return one ? (tex ? RF_BATCH_LAUNCH(32, 1, true) : RF_BATCH_LAUNCH(32, 1, false))
                       : (tex ? RF_BATCH_LAUNCH(32, 0, true) : RF_BATCH_LAUNCH(32, 0, false));
        case 16:
            return one ? (tex ? RF_BATCH_LAUNCH(16, 1, true) : RF_BATCH_LAUNCH(16, 1, false))
                       : (tex ? RF_BATCH_LAUNCH(16, 0, true) : RF_BATCH_LAUNCH(16, 0, false));
#undef RF_BATCH_LAUNCH
        default:
            return RF_ERR_NOT_SUPPORTED;
    }
}

extern "C" int rf_ghost_textures_forget(void) {
    using namespace rf;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return RF_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(ghost_texture_mutex);
    auto& c = ghost_texture_cache;
    c.erase(std::remove_if(c.begin(), c.end(), [dev](const GhostTextureEntry& e) { return e.dev == dev; }), c.end());
    return RF_OK;
}

extern "C" int rf_ghost_texture_object(const float* ghost, int32_t width, int32_t height, uint64_t* texture) {
    using namespace rf;
    if (!ghost || !texture || width < 1 || height < 1) return RF_ERR_INVALID_ARG;
    *texture = ghost_texture_object(ghost, width, height);
    return RF_OK;
}

namespace {
int raster_entry(const float* vertexes, const uint32_t* tile_offsets, const uint32_t* tile_entries,
                 const uint32_t* tile_order, const float* ghost, const float* spectrum, const rf_raster_args* args,
                 float* image, void* stream) {
    using namespace rf;
    if (!vertexes || !tile_offsets || !ghost || !spectrum || !args || !image) return RF_ERR_INVALID_ARG;
    if (!aligned16(vertexes) || !aligned16(image)) return RF_ERR_INVALID_ARG;
    RasterParams p;
    if (!make_params(*args, p)) return RF_ERR_INVALID_ARG;
    if (p.WS > kBatchRecords || p.maxW * p.WS > 4096) return RF_ERR_INVALID_ARG;
    switch (tile_size_of(*args)) {
        case 32:
            return launch_raster<32>(vertexes, tile_offsets, tile_entries, tile_order, ghost, spectrum, p, image,
                                     (cudaStream_t)stream);
        case 16:
            return launch_raster<16>(vertexes, tile_offsets, tile_entries, tile_order, ghost, spectrum, p, image,
                                     (cudaStream_t)stream);
        default:
            return RF_ERR_NOT_SUPPORTED;
    }
}
}  // namespace

extern "C" int rf_raster(const float* vertexes, const uint32_t* tile_offsets, const uint32_t* tile_entries,
                         const float* ghost, const float* spectrum, const rf_raster_args* args, float* image,
                         void* stream) {
    return raster_entry(vertexes, tile_offsets, tile_entries, nullptr, ghost, spectrum, args, image, stream);
}

extern "C" int rf_raster_ordered(const float* vertexes, const uint32_t* tile_offsets, const uint32_t* tile_entries,
                                 const uint32_t* tile_order, const float* ghost, const float* spectrum,
                                 const rf_raster_args* args, float* image, void* stream) {
    if (!tile_order) return RF_ERR_INVALID_ARG;
    return raster_entry(vertexes, tile_offsets, tile_entries, tile_order, ghost, spectrum, args, image, stream);
}

extern "C" int rf_raster_masks(const float* vertexes, const uint64_t* masks, int32_t batch_count, const float* ghost,
                               const float* spectrum, const rf_raster_args* args, float* image, void* stream) {
    using namespace rf;
    if (!vertexes || !masks || !ghost || !spectrum || !args || !image || batch_count < 0) return RF_ERR_INVALID_ARG;
    RasterParams p;
    if (!make_params(*args, p)) return RF_ERR_INVALID_ARG;
    const long long prim_total = (long long)args->path_count * (args->grid_count - 1) * (args->grid_count - 1);
    dim3 grid((p.width + 15) / 16, (p.height + 15) / 16);
    k_raster_masks<<<grid, 256, 0, (cudaStream_t)stream>>>((const float4*)vertexes, (const unsigned long long*)masks,
                                                           batch_count, args->bin_size, prim_total, ghost, spectrum,
                                                           p, fragment_consts(p), (float4*)image);
    return launch_status();
}

extern "C" int rf_raster_backward(const float* vertexes, const uint32_t* tile_offsets, const uint32_t* tile_entries,
                                  const float* ghost, const float* spectrum, const rf_raster_args* args,
                                  const float* image, const float* grad_image, float* grad_vertexes, void* stream) {
    using namespace rf;
    if (!vertexes || !tile_offsets || !ghost || !spectrum || !args || !image || !grad_image || !grad_vertexes)
        return RF_ERR_INVALID_ARG;
    if (!aligned16(vertexes) || !aligned16(image) || !aligned16(grad_image)) return RF_ERR_INVALID_ARG;
    RasterParams p;
    if (!make_params(*args, p)) return RF_ERR_INVALID_ARG;
    if (p.WS > kBatchRecords || p.maxW * p.WS > 4096) return RF_ERR_INVALID_ARG;
    const int T = tile_size_of(*args);
    if (T != 32 && T != 16) return RF_ERR_NOT_SUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    const long long n_vertices = (long long)args->path_count * args->grid_count * args->grid_count *
                                 args->wavelength_count + 1;
    RF_TRY(cuda_status(cudaMemsetAsync(grad_vertexes, 0, sizeof(float) * 8 * (size_t)n_vertices, s)));
    p.T = T;
    p.ntx = (p.width + T - 1) / T;
    const int nty = (p.height + T - 1) / T;
    const size_t smem = sizeof(Rec) * 2 * kBatchRecords + (sizeof(long long) + sizeof(float)) * 3 * kBatchRecords +
                        sizeof(float) * (3 * p.maxW * p.WS + ((p.WS + 3) & ~3)) +
                        sizeof(float) * (96 * (T * T / 32) + 2 * kBatchRecords * 4 * kGradAttrs +
                                         8 * kRedRows * kRedStride);
    const FragmentConsts fc = fragment_consts(p);
    const float4 *im = (const float4*)image, *gim = (const float4*)grad_image;
    const unsigned grid = (unsigned)(p.ntx * nty);
    p.ghost_tex = ghost_texture_object(ghost, p.ghost_w, p.ghost_h);
#define RF_BACKWARD_LAUNCH(TT, SS, X)                                                                         \
    do {                                                                                                      \
        static std::atomic<size_t> allowed[kMaxDevices];                                                      \
        RF_TRY(allow_smem(k_raster_backward<TT, SS, X>, smem, allowed));                                      \
        k_raster_backward<TT, SS, X><<<grid, kThreads, smem, s>>>((const float4*)vertexes, tile_offsets,       \
                                                                  tile_entries, ghost, spectrum, p, fc, im, gim, \
                                                                  grad_vertexes);                             \
    } while (0)
    const bool tex = p.ghost_tex != 0;
    if (T == 32 && p.S == 1) {
        if (tex) RF_BACKWARD_LAUNCH(32, 1, true); else RF_BACKWARD_LAUNCH(32, 1, false);
    } else if (T == 32) {
        if (tex) RF_BACKWARD_LAUNCH(32, 0, true); else RF_BACKWARD_LAUNCH(32, 0, false);
    } else if (p.S == 1) {
        if (tex) RF_BACKWARD_LAUNCH(16, 1, true); else RF_BACKWARD_LAUNCH(16, 1, false);
    } else {
        if (tex) RF_BACKWARD_LAUNCH(16, 0, true); else RF_BACKWARD_LAUNCH(16, 0, false);
    }
#undef RF_BACKWARD_LAUNCH
    return launch_status();
}

#ifdef RF_RASTER_STATS
// Statistics build only: read (and zero) the counters of the k_raster launches since the
// last call. out[8]: record iterations, whole-block record iterations, fragments, fragments
// of whole-block records, block visits, fragments with a zero smoothstep factor, record
// iterations where every shaded pixel has one (those two with more than one sample per
// pixel), warp steps of the one-sample shading loop.
extern "C" int rf_raster_stats(unsigned long long* out) {
    using namespace rf;
    if (!out) return RF_ERR_INVALID_ARG;
    RF_TRY(cuda_status(cudaMemcpyFromSymbol(out, g_raster_stats, sizeof(unsigned long long) * kRasterStats)));
    const unsigned long long zero[kRasterStats] = {};
    RF_TRY(cuda_status(cudaMemcpyToSymbol(g_raster_stats, zero, sizeof zero)));
    return RF_OK;
}
#endif
