// rf_image.cu — per-pixel image kernels: the starburst compositor, the aperture masks and
// the flare/starburst composite.
//
// k_starburst follows realflare/api/tasks/cl/starburst.cl:1-87 with noise.cl:1-5 and
// geometry.cl:1-48; k_aperture_shape / k_aperture_dust follow aperture.cl:5-47 / 139-174.
#include <math.h>

#include <cmath>

#include "rf_common.cuh"

namespace rf {
namespace {

__device__ __forceinline__ float fract1(float x) { return fminf(x - floorf(x), 0x1.fffffep-1f); }
// sin(x) for the noise hash. The hash's arguments reach 10^6, where sinf takes its slow
// reduction path; here x is reduced by pi/2 with the Cody-Waite method (W. J. Cody and
// W. Waite, Software Manual for the Elementary Functions, 1980) using a three-part split of
// pi/2 (C1 = fl(pi/2), C2 = fl(pi/2 - C1), C3 = fl(pi/2 - C1 - C2), which sum to pi/2 within
// 1e-23, computed in 200-bit arithmetic) and fused multiply-adds, then sin or cos of the
// remainder (|r| <= pi/4 + a rounding) by quadrant. Accurate to a few ulps for |x| < 2^22.
__device__ __forceinline__ float hash_sin(float x) {
    const float k = rintf(x * 0x1.45f306p-1f);  // x * 2 / pi
    float r = fmaf(-k, 0x1.921fb6p+0f, x);
    r = fmaf(-k, -0x1.777a5cp-25f, r);
    r = fmaf(-k, -0x1.ee59dap-50f, r);
    float sr, cr;
    sincosf(r, &sr, &cr);
    const int q = (int)k & 3;
    return q == 0 ? sr : (q == 1 ? cr : (q == 2 ? -sr : -cr));
}
// noise(x, y, z) of noise.cl:1-5
__device__ __forceinline__ float noise3(float x, float y, float z) {
    return fract1(hash_sin(x * 112.9898f + y * 179.233f + z * 237.212f) * 43758.5453f);
}
__device__ __forceinline__ void ndc_of(int px, int py, int w, int h, float& nx, float& ny) {
    nx = 2.0f * ((float)px / (float)(w - 1)) - 1.0f;
    ny = 2.0f * ((float)py / (float)(h - 1)) - 1.0f;
}
__device__ __forceinline__ void rot2(float& x, float& y, float angle) {
    float s, c;
    sincosf(angle, &s, &c);
    const float nx = x * c + y * s, ny = y * c - x * s;
    x = nx;
    y = ny;
}

// Per-sample terms of k_starburst that do not depend on the pixel, tabulated per CTA in
// chunks of kStarburstChunk samples: the light's XYZW weight at the sample's spectral
// position, the chromatic scale and the spectrum index.
constexpr int kStarburstChunk = 256;
struct StarburstSample {
    float4 light;
    float scale;
    int sidx;
};

__global__ void __launch_bounds__(256) k_starburst(const float* __restrict__ spectrum,
                                                   const float* __restrict__ light, rf_starburst_args a,
                                                   float4* __restrict__ image) {
    __shared__ StarburstSample tab[kStarburstChunk];
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    const bool inside = x < a.width && y < a.height;  // (every thread takes part in the table fills)
    float nx, ny;
    ndc_of(x, y, a.width, a.height, nx, ny);
    nx = (nx - a.offset[0]) / fmaxf(a.scale[0], 1.17549435e-38f);
    ny = (ny - a.offset[1]) / fmaxf(a.scale[1], 1.17549435e-38f);
    const size_t plane = (size_t)a.spectrum_width * a.spectrum_height;
    // With blur 0 the jitter radius is 0 * sqrt(noise) = 0 (noise in [0, 1)), and with
    // rotation 0 and a non-negative weight the angle is +-0 * (1 - noise^weight) = +-0: the
    // jitter and the rotation then leave the position unchanged and their noise is skipped.
    const bool jitter = a.blur != 0.0f;
    const bool rotate = a.rotation != 0.0f || !(a.rotation_weight >= 0.0f);
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const float fx = (float)x, fy = (float)y;
    for (int t0 = 0; t0 < a.samples; t0 += kStarburstChunk) {
        const int n = min(kStarburstChunk, a.samples - t0);
        __syncthreads();  // the previous chunk's table is no longer read
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int t = t0 + i;
            const float step = (float)t / (float)a.samples;
            // no contraction into an FMA: the spectrum index below rounds this value, and a
            // sample can fall exactly halfway between two spectra
            const float wavelength = __fadd_rn(__fmul_rn(step, (float)(RF_LAMBDA_MAX - RF_LAMBDA_MIN)),
                                               (float)RF_LAMBDA_MIN);
            StarburstSample e;
            // chromatic scale 1 - (1 - lambda / 560) (LAMBDA_MID is an int in starburst.cl)
            e.scale = fmaxf(1.0f - (1.0f - (wavelength / (float)RF_LAMBDA_MID)) * 1.0f, 1.17549435e-38f);
            int sidx = 0;
            if (a.spectrum_count > 1) {
                const int k = cvt_rz_sat(floorf(__fadd_rn(__fsub_rn(wavelength, a.lambda_first) / a.lambda_step, 0.5f)));
                sidx = k < 0 ? 0 : (k >= a.spectrum_count ? a.spectrum_count - 1 : k);
            }
            e.sidx = sidx;
            e.light = make_float4(sample_linear(light, RF_SPECTRUM_WIDTH, 1, 4, 0, step, 0.0f, false),
                                  sample_linear(light, RF_SPECTRUM_WIDTH, 1, 4, 1, step, 0.0f, false),
                                  sample_linear(light, RF_SPECTRUM_WIDTH, 1, 4, 2, step, 0.0f, false),
                                  sample_linear(light, RF_SPECTRUM_WIDTH, 1, 4, 3, step, 0.0f, false));
            tab[i] = e;
        }
        __syncthreads();
        if (!inside) continue;
        for (int i = 0; i < n; i++) {
            const int t = t0 + i;
            const StarburstSample e = tab[i];
            const float seed = (float)(t * 4);
            float px = nx, py = ny;
            if (jitter) {
                const float radius = a.blur * sqrtf(noise3(fx, fy, seed));
                const float alpha = noise3(fx, fy, seed + 1.0f) * 2.0f * RF_MPI_F;
                float sa, ca;
                sincosf(alpha, &sa, &ca);
                px += ca * radius;
                py += sa * radius;
            }
            px = px / e.scale;
            py = py / e.scale;
            if (rotate) {
                const float sign = noise3(fx, fy, seed + 2.0f) > 0.5f ? 1.0f : -1.0f;
                const float angle = sign * a.rotation * (1.0f - powf(noise3(fx, fy, seed + 3.0f), a.rotation_weight));
                rot2(px, py, angle);
            }
            const float u = px * 0.5f + 0.5f, v = py * 0.5f + 0.5f;
            const float fi = sample_linear(spectrum + e.sidx * plane, a.spectrum_width, a.spectrum_height, 1, 0, u, v,
                                           false);
            acc[0] += e.light.x * fi;
            acc[1] += e.light.y * fi;
            acc[2] += e.light.z * fi;
            acc[3] += e.light.w * fi;
        }
    }
    if (!inside) return;
#pragma unroll
    for (int c = 0; c < 4; c++) acc[c] = acc[c] / (float)a.samples;
    if (!isnan(a.vignetting[0])) {
        const float sdf = sqrtf(nx * nx + ny * ny) - 0.0f;
        const float f = smoothstepf(a.vignetting[1], a.vignetting[0], sdf);
#pragma unroll
        for (int c = 0; c < 4; c++) acc[c] *= f;
    }
#pragma unroll
    for (int c = 0; c < 4; c++) acc[c] *= a.intensity;
    image[(size_t)y * a.width + x] = xyz_to_ap1(acc[0], acc[1], acc[2]);
}

__global__ void __launch_bounds__(256) k_aperture_shape(float* __restrict__ image, int w, int h, float sx, float sy,
                                                        int blades, float rotation, float roundness, float softness) {
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= w || y >= h) return;
    float px, py;
    ndc_of(x, y, w, h, px, py);
    px = px / fmaxf(sx, 1.17549435e-38f);
    py = py / fmaxf(sy, 1.17549435e-38f);
    rot2(px, py, rotation);
    float sdf = 0.0f;
    for (int i = 0; i < blades; i++) {
        const float angle = ((float)i / (float)blades + 0.25f) * 2.0f * RF_MPI_F;
        float s, c;
        sincosf(angle, &s, &c);
        sdf = fmaxf(sdf, c * px + s * py);
    }
    const float cg = atan2f(-px, -py) / (2.0f * RF_MPI_F) + 0.5f;
    const float bg = fmodf(cg * (float)blades + 0.5f, 1.0f);
    sdf += sinf(bg * RF_MPI_F) * roundness;
    image[(size_t)y * w + x] = 1.0f - smoothstepf(1.0f - softness, 1.0f + softness, sdf);
}

__global__ void __launch_bounds__(256) k_aperture_dust(float* __restrict__ image, int w, int h, float sx, float sy,
                                                       float strength, int count, float radius, float par_x,
                                                       float par_y, float softness) {
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= w || y >= h) return;
    float px, py;
    ndc_of(x, y, w, h, px, py);
    px = px / fmaxf(sx, 1.17549435e-38f);
    py = py / fmaxf(sy, 1.17549435e-38f);
    float sdf = 1.0f;
    for (int i = 0; i < count; i++) {
        float cx = noise3((float)i, (float)count, 0.0f) + par_x;
        float cy = noise3((float)i, (float)count, 1.0f) + par_y;
        cx = fmodf(1.0f + fmodf(cx, 1.0f), 1.0f) * 2.0f - 1.0f;
        cy = fmodf(1.0f + fmodf(cy, 1.0f), 1.0f) * 2.0f - 1.0f;
        const float dx = px - cx, dy = py - cy;
        sdf = fminf(sdf, sqrtf(dx * dx + dy * dy) - radius);
    }
    float v = image[(size_t)y * w + x];
    v *= 1.0f - (strength * smoothstepf(softness, -softness, sdf));
    image[(size_t)y * w + x] = v;
}

// Separable Gaussian over the noise (no reference counterpart): pass 0 blurs rows into
// tmp, pass 1 blurs columns of tmp and multiplies the image by 1 - strength * blur.
struct BlurWeights {
    float w[513];
    int rad;
};

__global__ void __launch_bounds__(256) k_noise_blur(const float* __restrict__ src, float* __restrict__ dst,
                                                    float* __restrict__ image, int w, int h,
                                                    const __grid_constant__ BlurWeights bw, int pass, float strength) {
    const int rad = bw.rad;
    const float* weights = bw.w;
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= w || y >= h) return;
    float acc = 0.0f;
    for (int k = -rad; k <= rad; k++) {
        int xx = x, yy = y;
        if (pass == 0) xx = min(max(x + k, 0), w - 1);
        else yy = min(max(y + k, 0), h - 1);
        acc += weights[k + rad] * src[(size_t)yy * w + xx];
    }
    if (pass == 0) dst[(size_t)y * w + x] = acc;
    else image[(size_t)y * w + x] = image[(size_t)y * w + x] * (1.0f - strength * acc);
}

// Engine.image_flare's accumulation (realflare/api/engine.py:120-150): per light sample i,
// image += v_i0 * F_i + v_i1 * flip_y(F_i) + v_i2 * flip_yx(F_i) + v_i3 * flip_x(F_i) (per
// channel weights), in sample order, each product and sum rounded as in float32 numpy;
// then image /= count. One thread per output pixel (float4).
__global__ void k_accumulate_mirrored(const float4* __restrict__ frames, const float4* __restrict__ weights, int n,
                                      int w, int h, float divisor, float4* __restrict__ image) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)w * h) return;
    const int x = (int)(i % w), y = (int)(i / w);
    const long long frame = (long long)w * h;
    const long long src[4] = {(long long)y * w + x, (long long)(h - 1 - y) * w + x,
                              (long long)(h - 1 - y) * w + (w - 1 - x), (long long)y * w + (w - 1 - x)};
    float4 acc = image[i];
    for (int k = 0; k < n; k++) {
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const float4 f = frames[k * frame + src[m]];
            const float4 v = weights[4 * k + m];
            acc.x = __fadd_rn(acc.x, __fmul_rn(v.x, f.x));
            acc.y = __fadd_rn(acc.y, __fmul_rn(v.y, f.y));
            acc.z = __fadd_rn(acc.z, __fmul_rn(v.z, f.z));
            acc.w = __fadd_rn(acc.w, __fmul_rn(v.w, f.w));
        }
    }
    if (divisor > 0.0f) {
        acc.x = __fdiv_rn(acc.x, divisor);
        acc.y = __fdiv_rn(acc.y, divisor);
        acc.z = __fdiv_rn(acc.z, divisor);
        acc.w = __fdiv_rn(acc.w, divisor);
    }
    image[i] = acc;
}

__global__ void k_axpby(const float* __restrict__ a, float wa, const float* __restrict__ b, float wb,
                        float* __restrict__ out, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] * wa + b[i] * wb;
}

}  // namespace
}  // namespace rf

extern "C" int rf_starburst(const float* spectrum, const float* light_spectrum, const rf_starburst_args* args,
                            float* image, void* stream) {
    using namespace rf;
    if (!spectrum || !light_spectrum || !args || !image) return RF_ERR_INVALID_ARG;
    const rf_starburst_args& a = *args;
    if (a.width < 2 || a.height < 2 || a.samples < 1 || a.spectrum_width < 1 || a.spectrum_height < 1 ||
        a.spectrum_count < 1 || !aligned16(image))
        return RF_ERR_INVALID_ARG;
    dim3 grid((a.width + 15) / 16, (a.height + 15) / 16);
    k_starburst<<<grid, 256, 0, (cudaStream_t)stream>>>(spectrum, light_spectrum, a, (float4*)image);
    return launch_status();
}

extern "C" int rf_aperture_shape(float* image, int32_t width, int32_t height, float size_x, float size_y,
                                 int32_t blades, float rotation, float roundness, float softness, void* stream) {
    using namespace rf;
    if (!image || width < 2 || height < 2 || blades < 0) return RF_ERR_INVALID_ARG;
    dim3 grid((width + 15) / 16, (height + 15) / 16);
    k_aperture_shape<<<grid, 256, 0, (cudaStream_t)stream>>>(image, width, height, size_x, size_y, blades, rotation,
                                                             roundness, softness);
    return launch_status();
}

extern "C" int rf_aperture_dust(float* image, int32_t width, int32_t height, float size_x, float size_y,
                                float strength, float density, float radius, float parallax_x, float parallax_y,
                                float softness, void* stream) {
    using namespace rf;
    if (!image || width < 2 || height < 2) return RF_ERR_INVALID_ARG;
    // int count = fmin(density, 1) * 1000 (aperture.cl:160)
    const int count = (int)(fminf(density, 1.0f) * 1000.0f);
    dim3 grid((width + 15) / 16, (height + 15) / 16);
    k_aperture_dust<<<grid, 256, 0, (cudaStream_t)stream>>>(image, width, height, size_x, size_y, strength, count,
                                                            radius, parallax_x, parallax_y, softness);
    return launch_status();
}

extern "C" int rf_aperture_noise_dust(float* image, const float* noise, float* scratch, int32_t width,
                                      int32_t height, float strength, float sigma, void* stream) {
    using namespace rf;
    if (!image || !noise || !scratch || width < 1 || height < 1 || !(sigma >= 0.0f) || sigma > 64.0f)
        return RF_ERR_INVALID_ARG;
    // weights exp(-k^2 / (2 sigma^2)) normalised to 1 in FP32 (the oracle's values),
    // passed by value
    BlurWeights bw;
    bw.rad = (int)std::ceil((double)sigma * 4.0);
    float sum = 0.0f;
    for (int k = -bw.rad; k <= bw.rad; k++) {
        bw.w[k + bw.rad] = sigma > 0.0f ? expf(-(float)(k * k) / (2.0f * sigma * sigma)) : 1.0f;
        sum += bw.w[k + bw.rad];
    }
    for (int k = 0; k <= 2 * bw.rad; k++) bw.w[k] = bw.w[k] / sum;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 grid((width + 15) / 16, (height + 15) / 16);
    k_noise_blur<<<grid, 256, 0, s>>>(noise, scratch, image, width, height, bw, 0, strength);
    RF_TRY(launch_status());
    k_noise_blur<<<grid, 256, 0, s>>>(scratch, nullptr, image, width, height, bw, 1, strength);
    return launch_status();
}

extern "C" int rf_axpby(const float* a, float wa, const float* b, float wb, float* out, int64_t n, void* stream) {
    using namespace rf;
    if (!a || !b || !out || n < 0) return RF_ERR_INVALID_ARG;
    if (n == 0) return RF_OK;
    k_axpby<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(a, wa, b, wb, out, n);
    return launch_status();
}

extern "C" int rf_accumulate_mirrored(const float* frames, const float* weights, int32_t count, int32_t width,
                                      int32_t height, float divisor, float* image, void* stream) {
    using namespace rf;
    if (!frames || !weights || !image || count < 0 || width < 1 || height < 1) return RF_ERR_INVALID_ARG;
    if (!aligned16(frames) || !aligned16(weights) || !aligned16(image)) return RF_ERR_INVALID_ARG;
    const long long n = (long long)width * height;
    k_accumulate_mirrored<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        (const float4*)frames, (const float4*)weights, count, width, height, divisor, (float4*)image);
    return launch_status();
}
