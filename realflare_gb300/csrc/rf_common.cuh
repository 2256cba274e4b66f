// rf_common.cuh — shared device helpers and host-side error plumbing of the CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/realflare_gb300.h"

#define RF_MPI_F 3.14159274101257324f  // OpenCL M_PI_F

namespace rf {

// ---------------------------------------------------------------- host error plumbing
void set_cuda_error(cudaError_t e);
void set_error_text(const char* text);
void count_launch();
// Called after every kernel launch: counts it and reports a launch error.
inline int launch_status() {
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return RF_ERR_CUDA;
    }
    return RF_OK;
}
inline int cuda_status(cudaError_t e) {
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return RF_ERR_CUDA;
    }
    return RF_OK;
}
#define RF_TRY(expr)                  \
    do {                              \
        int rf_s_ = (expr);           \
        if (rf_s_ != RF_OK) return rf_s_; \
    } while (0)

inline unsigned blocks_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }
inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// ---------------------------------------------------------------- batched frames
// The frame owning work unit `unit` of a stage: the last frame whose first unit of that
// stage (first(frame), non-decreasing over the frames) is <= unit. Frames without units
// share their first unit with the next frame, so the last of equal starts owns it.
template <class First>
__device__ __forceinline__ int find_frame(const rf_frame* __restrict__ frames, int F, long long unit, First first) {
    int lo = 0, hi = F - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((long long)first(frames[mid]) <= unit) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------- integer semantics
// float -> int truncating toward zero, saturating, NaN -> 0 (cvt.rzi.s32.f32 semantics,
// the conversion the reference's convert_int2/convert_int4 compile to on NVIDIA GPUs).
__device__ __forceinline__ int32_t cvt_rz_sat(float x) { return __float2int_rz(x); }
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// read_imagef with CLK_FILTER_LINEAR | CLK_NORMALIZED_COORDS_TRUE, computed in FP32 from
// the OpenCL specification's formula on a w x h texture of `ch` floats per texel (channel
// c). edge: CLAMP_TO_EDGE, else CLAMP with border 0. Non-finite coordinates give 0.
__device__ __forceinline__ float sample_linear(const float* __restrict__ tex, int w, int h, int ch, int c,
                                               float s, float t, bool edge) {
    float u = s * (float)w - 0.5f, v = t * (float)h - 0.5f;
    if (!isfinite(u) || !isfinite(v)) return 0.0f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    long long i0 = cvt_rz_sat(fu), j0 = cvt_rz_sat(fv);
    long long is[2] = {i0, i0 + 1}, js[2] = {j0, j0 + 1};
    float T[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        long long i = is[k & 1], j = js[k >> 1];
        if (edge) {
            i = i < 0 ? 0 : (i >= w ? w - 1 : i);
            j = j < 0 ? 0 : (j >= h ? h - 1 : j);
            T[k] = __ldg(tex + ((size_t)j * w + i) * ch + c);
        } else {
            T[k] = (i < 0 || i >= w || j < 0 || j >= h) ? 0.0f : __ldg(tex + ((size_t)j * w + i) * ch + c);
        }
    }
    return (1.0f - a) * (1.0f - b) * T[0] + a * (1.0f - b) * T[1] + (1.0f - a) * b * T[2] + a * b * T[3];
}

// xyz_to_ap1 (realflare/api/tasks/cl/color.cl:3-10): the matrix literals are double in
// OpenCL C, so the products and sums are evaluated in double.
__device__ __forceinline__ float4 xyz_to_ap1(float x, float y, float z) {
    double dx = x, dy = y, dz = z;
    float4 o;
    o.x = (float)(1.6410233797 * dx + -0.3248032942 * dy + -0.2364246952 * dz);
    o.y = (float)(-0.6636628587 * dx + 1.6153315917 * dy + 0.0167563477 * dz);
    o.z = (float)(0.0117218943 * dx + -0.0082844420 * dy + 0.9883948585 * dz);
    o.w = 0.0f;
    return o;
}

// The n-rook sample offsets of realflare/api/tasks/rasterizing.py:78-87.
__device__ __constant__ static const unsigned char SUB_OFFSETS[15] = {0, 1, 0, 1, 2, 0, 3, 4, 1, 6, 2, 5, 0, 3, 7};

// ---------------------------------------------------------------- batch workspace
// Scratch of rf_bin_tiles_batch and rf_raster_batch (rf_bin.cu): pair counters and their
// scan, the entry sort's buffers, the raster's tile order and its queue head.
struct BatchWorkspace {
    uint32_t *counts, *scan_scratch, *keys_a, *keys_b, *vals_tmp, *radix_scratch;
    uint32_t *order_keys, *order_vals, *order_keys_b, *order_vals_b, *queue;
    size_t bytes;
};
BatchWorkspace batch_layout(char* base, const rf_batch_sizes& sizes, long long entry_capacity);
const uint32_t* batch_tile_order(const BatchWorkspace& w, const rf_batch_sizes& sizes);

// ---------------------------------------------------------------- scans / sorting
// Exclusive prefix sum of n uint32 values (in may equal out). scratch: scan_scratch_words(n)
// uint32 words. Values must not overflow 32 bits.
size_t scan_scratch_words(long long n);
int exclusive_scan_u32(const uint32_t* in, uint32_t* out, long long n, uint32_t* scratch, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs by the low key_bits bits of key.
// keys/vals hold the input; keys_alt/vals_alt are buffers of the same size. On return
// *result_in_alt tells which pair of buffers holds the sorted output.
size_t radix_scratch_words(long long n);
int radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, long long n,
                     int key_bits, uint32_t* scratch, bool* result_in_alt, cudaStream_t s);

}  // namespace rf
