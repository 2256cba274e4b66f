// cl_shim.hpp — an OpenCL C 1.2 environment in C++ for running the reference's kernels on
// the host (test infrastructure: used only to build oracle/_ref from the reference's own
// .cl sources, see oracle/build_ref.py).
//
// Provides what realflare's kernels use: the vector types (float3 occupies 16 bytes, as in
// OpenCL) with component access and the swizzles the kernels use, arithmetic operators,
// the math/geometric/common built-ins, convert_* (truncation toward zero, saturating;
// NaN -> 0, as NVIDIA hardware converts), vstore4, work-item ids (set by the harness per
// work-item), async_work_group_copy, and images with read_imagef implementing the OpenCL
// specification's CLK_FILTER_LINEAR formula in FP32 (CLAMP -> border 0, CLAMP_TO_EDGE).
// fmax/fmin/max/min/clamp follow fmaxf/fminf (a NaN operand yields the other operand).
// Unsuffixed floating literals in the kernels are double, as in OpenCL C with fp64.
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <string.h>

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;

#define __kernel
#define kernel
#define __global
#define global
#define __local
#define local
#define __constant const
#define __private
#define __read_only
#define __write_only
#define read_only
#define write_only
#define read_write

#define INFINITY (__builtin_inff())
#define NAN (__builtin_nanf(""))
#define FLT_MIN 1.17549435e-38f
#define M_PI_F 3.14159274101257324f
#define CLK_NORMALIZED_COORDS_TRUE 1
#define CLK_NORMALIZED_COORDS_FALSE 0
#define CLK_ADDRESS_CLAMP 2
#define CLK_ADDRESS_CLAMP_TO_EDGE 4
#define CLK_ADDRESS_REPEAT 8
#define CLK_ADDRESS_NONE 0
#define CLK_FILTER_LINEAR 16
#define CLK_FILTER_NEAREST 0
typedef int sampler_t;
typedef int event_t;

// ------------------------------------------------------------------ scalar math
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline double sqrt(double x) { return __builtin_sqrt(x); }
inline float fabs(float x) { return __builtin_fabsf(x); }
inline double fabs(double x) { return __builtin_fabs(x); }
inline float sin(float x) { return __builtin_sinf(x); }
inline float cos(float x) { return __builtin_cosf(x); }
inline float tan(float x) { return __builtin_tanf(x); }
inline float asin(float x) { return __builtin_asinf(x); }
inline float acos(float x) { return __builtin_acosf(x); }
inline float atan2(float y, float x) { return __builtin_atan2f(y, x); }
inline float pow(float x, float y) { return __builtin_powf(x, y); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float ceil(float x) { return __builtin_ceilf(x); }
inline float trunc(float x) { return __builtin_truncf(x); }
inline float fmod(float x, float y) { return __builtin_fmodf(x, y); }
inline float fmax(float a, float b) { return __builtin_fmaxf(a, b); }
inline float fmin(float a, float b) { return __builtin_fminf(a, b); }
inline float max(float a, float b) { return __builtin_fmaxf(a, b); }
inline float min(float a, float b) { return __builtin_fminf(a, b); }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline float clamp(float x, float lo, float hi) { return fmin(fmax(x, lo), hi); }
inline float mix(float a, float b, float t) { return a + (b - a) * t; }
inline float smoothstep(float e0, float e1, float x) {
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline float fract(float x, float* ip) {
    float f = floor(x);
    *ip = f;
    return fmin(x - f, 0x1.fffffep-1f);
}
inline int isnan(float x) { return x != x; }
inline int cvt_int_rz_sat(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int)0x80000000u;
    return (int)x;
}

// ------------------------------------------------------------------ vector types
template <class S, class V, int N, int A, int B>
struct Swz2 {
    S s[N];
    operator V() const { return V(s[A], s[B]); }
    Swz2& operator=(const V& v) { s[A] = v.x; s[B] = v.y; return *this; }
    Swz2& operator=(const Swz2&) = delete;
};
template <class S, class V, int N, int A, int B, int C>
struct Swz3 {
    S s[N];
    operator V() const { return V(s[A], s[B], s[C]); }
    Swz3& operator=(const V& v) { s[A] = v.x; s[B] = v.y; s[C] = v.z; return *this; }
    Swz3& operator+=(const V& v) { s[A] += v.x; s[B] += v.y; s[C] += v.z; return *this; }
    Swz3& operator=(const Swz3&) = delete;
};

#define RF_VEC2(V, S)                                                      \
    struct alignas(2 * sizeof(S)) V {                                      \
        union { S s[2]; struct { S x, y; }; };                             \
        V() { s[0] = 0; s[1] = 0; }                                        \
        V(S v) { s[0] = v; s[1] = v; }                                     \
        V(S a, S b) { s[0] = a; s[1] = b; }                                \
        V(const V& o) { s[0] = o.s[0]; s[1] = o.s[1]; }                    \
        V& operator=(const V& o) { s[0] = o.s[0]; s[1] = o.s[1]; return *this; } \
    };
#define RF_VEC3(V, S, V2)                                                  \
    struct alignas(4 * sizeof(S)) V {                                      \
        union { S s[4]; struct { S x, y, z, w_; }; Swz2<S, V2, 4, 0, 1> xy; Swz2<S, V2, 4, 2, 1> zy; Swz3<S, V, 4, 0, 1, 2> xyz; }; \
        V() { s[0] = 0; s[1] = 0; s[2] = 0; s[3] = 0; }                    \
        V(S v) { s[0] = v; s[1] = v; s[2] = v; s[3] = 0; }                 \
        V(S a, S b, S c) { s[0] = a; s[1] = b; s[2] = c; s[3] = 0; }       \
        V(const V& o) { memcpy(s, o.s, sizeof s); }                        \
        V& operator=(const V& o) { memcpy(s, o.s, sizeof s); return *this; } \
    };
#define RF_VEC4(V, S, V2, V3)                                              \
    struct alignas(4 * sizeof(S)) V {                                      \
        union {                                                            \
            S s[4];                                                        \
            struct { S x, y, z, w; };                                      \
            Swz2<S, V2, 4, 0, 1> xy;                                       \
            Swz2<S, V2, 4, 2, 3> zw;                                       \
            Swz2<S, V2, 4, 1, 0> yx;                                       \
            Swz3<S, V3, 4, 0, 1, 2> xyz;                                   \
        };                                                                 \
        V() { s[0] = 0; s[1] = 0; s[2] = 0; s[3] = 0; }                    \
        V(S v) { s[0] = v; s[1] = v; s[2] = v; s[3] = v; }                 \
        V(S a, S b, S c, S d) { s[0] = a; s[1] = b; s[2] = c; s[3] = d; } \
        V(const V& o) { memcpy(s, o.s, sizeof s); }                        \
        V& operator=(const V& o) { memcpy(s, o.s, sizeof s); return *this; } \
        V operator++(int) { V old = *this; for (int i = 0; i < 4; i++) s[i]++; return old; } \
    };

RF_VEC2(float2, float)
RF_VEC2(int2, int)
RF_VEC2(uint2, uint)
RF_VEC3(float3, float, float2)
RF_VEC3(int3, int, int2)
RF_VEC4(float4, float, float2, float3)
RF_VEC4(int4, int, int2, int3)
RF_VEC2(long2, long)
RF_VEC3(long3, long, long2)
RF_VEC4(long4, long, long2, long3)

struct alignas(32) float8 {
    union { float s[8]; struct { float s0, s1, s2, s3, s4, s5, s6, s7; }; struct { float x, y, z, w; }; };
    float8() { memset(s, 0, sizeof s); }
};

// element-wise operators over every vector type (vector op vector, vector op scalar,
// scalar op vector), and compound assignment.
#define RF_OPS(V, S, N)                                                                    \
    inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] + b.s[i]; return r; } \
    inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] - b.s[i]; return r; } \
    inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] * b.s[i]; return r; } \
    inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] / b.s[i]; return r; } \
    inline V operator+(const V& a, S b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] + b; return r; } \
    inline V operator-(const V& a, S b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] - b; return r; } \
    inline V operator*(const V& a, S b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] * b; return r; } \
    inline V operator/(const V& a, S b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] / b; return r; } \
    inline V operator+(S a, const V& b) { V r; for (int i = 0; i < N; i++) r.s[i] = a + b.s[i]; return r; } \
    inline V operator-(S a, const V& b) { V r; for (int i = 0; i < N; i++) r.s[i] = a - b.s[i]; return r; } \
    inline V operator*(S a, const V& b) { V r; for (int i = 0; i < N; i++) r.s[i] = a * b.s[i]; return r; } \
    inline V operator-(const V& a) { V r; for (int i = 0; i < N; i++) r.s[i] = -a.s[i]; return r; } \
    inline V& operator+=(V& a, const V& b) { for (int i = 0; i < N; i++) a.s[i] += b.s[i]; return a; } \
    inline V& operator-=(V& a, const V& b) { for (int i = 0; i < N; i++) a.s[i] -= b.s[i]; return a; } \
    inline V& operator*=(V& a, S b) { for (int i = 0; i < N; i++) a.s[i] *= b; return a; } \
    inline V& operator/=(V& a, S b) { for (int i = 0; i < N; i++) a.s[i] /= b; return a; }

RF_OPS(float2, float, 2)
RF_OPS(float3, float, 3)
RF_OPS(float4, float, 4)
RF_OPS(int2, int, 2)
RF_OPS(int4, int, 4)
RF_OPS(uint2, uint, 2)

inline float2 make_float2(float a, float b) { return float2(a, b); }
inline float3 make_float3(float a, float b, float c) { return float3(a, b, c); }
inline float3 make_float3(float2 a, float c) { return float3(a.x, a.y, c); }
inline float4 make_float4(float a, float b, float c, float d) { return float4(a, b, c, d); }
inline int2 make_int2(int a, int b) { return int2(a, b); }
inline int4 make_int4(int a, int b, int c, int d) { return int4(a, b, c, d); }
inline int4 make_int4(int2 a, int2 b) { return int4(a.x, a.y, b.x, b.y); }
inline uint2 make_uint2(uint a, uint b) { return uint2(a, b); }
inline long4 make_long4(long a, long b, long c, long d) { return long4(a, b, c, d); }

// geometric / common built-ins
inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(float2 a) { return sqrt(dot(a, a)); }
inline float length(float3 a) { return sqrt(dot(a, a)); }
inline float3 normalize(float3 a) { return a * (1.0f / sqrt(dot(a, a))); }
inline float2 min(float2 a, float2 b) { return float2(fmin(a.x, b.x), fmin(a.y, b.y)); }
inline float2 max(float2 a, float2 b) { return float2(fmax(a.x, b.x), fmax(a.y, b.y)); }
inline float2 fmax(float2 a, float b) { return float2(fmax(a.x, b), fmax(a.y, b)); }
inline float2 fmax(float2 a, float2 b) { return float2(fmax(a.x, b.x), fmax(a.y, b.y)); }
inline float2 fabs(float2 a) { return float2(fabs(a.x), fabs(a.y)); }
inline float2 fmod(float2 a, float m) { return float2(fmod(a.x, m), fmod(a.y, m)); }
inline float2 mix(float2 a, float2 b, float t) { return a + (b - a) * t; }
inline int2 convert_int2(float2 a) { return int2(cvt_int_rz_sat(a.x), cvt_int_rz_sat(a.y)); }
inline int4 convert_int4(float4 a) {
    return int4(cvt_int_rz_sat(a.x), cvt_int_rz_sat(a.y), cvt_int_rz_sat(a.z), cvt_int_rz_sat(a.w));
}
inline float2 convert_float2(int2 a) { return float2((float)a.x, (float)a.y); }
inline void vstore4(int4 v, size_t off, int* p) { memcpy(p + 4 * off, v.s, sizeof(int) * 4); }
inline void vstore4(long4 v, size_t off, long* p) { memcpy(p + 4 * off, v.s, sizeof(long) * 4); }

// ------------------------------------------------------------------ work-items
static thread_local size_t rf_gid[3], rf_gsz[3] = {1, 1, 1}, rf_lid[3], rf_lsz[3] = {1, 1, 1};
inline size_t get_global_id(int d) { return rf_gid[d]; }
inline size_t get_global_size(int d) { return rf_gsz[d]; }
inline size_t get_local_id(int d) { return rf_lid[d]; }
inline size_t get_local_size(int d) { return rf_lsz[d]; }
inline size_t get_group_id(int d) { return rf_gid[d] / rf_lsz[d]; }
inline size_t get_num_groups(int d) { return rf_gsz[d] / rf_lsz[d]; }
inline event_t async_work_group_copy(float4* dst, const float4* src, size_t n, event_t) {
    memcpy((void*)dst, (const void*)src, n * sizeof(float4));
    return 0;
}
inline void wait_group_events(int, event_t*) {}

// ------------------------------------------------------------------ images
struct rf_image {
    int width, height, channels;  // channels: 1 (INTENSITY: read returns (v, v, v, v)) or 4
    float* data;
};
typedef rf_image* image2d_t;

inline int2 get_image_dim(image2d_t im) { return int2(im->width, im->height); }
inline float rf_texel(image2d_t im, long i, long j, int c, int edge) {
    if (edge) {
        i = i < 0 ? 0 : (i >= im->width ? im->width - 1 : i);
        j = j < 0 ? 0 : (j >= im->height ? im->height - 1 : j);
    } else if (i < 0 || i >= im->width || j < 0 || j >= im->height) {
        return 0.0f;
    }
    return im->data[((size_t)j * im->width + i) * im->channels + (im->channels == 1 ? 0 : c)];
}
inline float4 read_imagef(image2d_t im, sampler_t smp, float2 st) {
    int edge = (smp & CLK_ADDRESS_CLAMP_TO_EDGE) != 0;
    float u = st.x * (float)im->width - 0.5f, v = st.y * (float)im->height - 0.5f;
    float4 r(0.0f);
    if (!(u - u == 0.0f) || !(v - v == 0.0f)) return r;  // non-finite coordinate -> 0
    float fu = floor(u), fv = floor(v);
    float a = u - fu, b = v - fv;
    long i0 = cvt_int_rz_sat(fu), j0 = cvt_int_rz_sat(fv);
    for (int c = 0; c < 4; c++) {
        float t00 = rf_texel(im, i0, j0, c, edge), t10 = rf_texel(im, i0 + 1, j0, c, edge);
        float t01 = rf_texel(im, i0, j0 + 1, c, edge), t11 = rf_texel(im, i0 + 1, j0 + 1, c, edge);
        r.s[c] = (1.0f - a) * (1.0f - b) * t00 + a * (1.0f - b) * t10 + (1.0f - a) * b * t01 + a * b * t11;
    }
    return r;
}
inline float4 read_imagef(image2d_t im, int2 p) {
    float4 r(0.0f);
    for (int c = 0; c < 4; c++) r.s[c] = rf_texel(im, p.x, p.y, c, 1);
    return r;
}
inline void write_imagef(image2d_t im, int2 p, float4 v) {
    if (p.x < 0 || p.y < 0 || p.x >= im->width || p.y >= im->height) return;
    float* d = im->data + ((size_t)p.y * im->width + p.x) * im->channels;
    if (im->channels == 1) d[0] = v.x;
    else memcpy(d, v.s, sizeof(float) * 4);
}
