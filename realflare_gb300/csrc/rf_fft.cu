// rf_fft.cu — 2-D FFTs for the diffraction stages.
//
// A 2-D transform of a [batch][h][w] complex64 array is two passes of the same kernel:
// each block loads one row into shared memory in bit-reversed order, runs the radix-2
// decimation-in-time butterflies in place (twiddles from a per-block sincospi table), and
// writes the row transposed ([batch][w][h]); the second pass transforms those rows and
// transposes back, applying the normalisation. Pre- and post-operations of the two
// callers are fused into the first load and the last store:
//  * the starburst power spectrum (realflare/api/tasks/starburst.py:45-81): load
//    A * exp(i pi (x^2 + y^2) / (lambda d)), store |F|^2 at the fftshift position;
//  * the ghost texture's fractional Fourier transform (realflare/api/tasks/ghost.py:13-36
//    and realflare/utils/frft.py:20-62, Ozaktas et al. 1996 chirp convolution), built from
//    the plain transform and element-wise chirp kernels.
// Rows whose length is a power of two run the radix-2 kernel below; any other length from
// 2 to 4096 runs Bluestein's chirp-z form (Bluestein 1970): with w_m = exp(d pi i m^2 / n),
// X_k = w_k sum_j (x_j w_j) conj(w_{k-j}), a linear convolution evaluated by radix-2
// transforms of a power-of-two length M >= 2n - 1, in shared memory, one row per block.
#include <complex>
#include <math.h>

#include "rf_common.cuh"

namespace rf {
namespace {

constexpr int kMaxN = 4096;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Load callbacks: produce element i of row `row` (row = batch * rows_per_batch + r).
struct LoadComplex {
    const float2* in;
    int n;
    __device__ float2 operator()(long long row, int i) const { return in[row * n + i]; }
};
struct LoadStarburst {  // aperture * chirp, batch = wavelength
    const float* aperture;
    int w, h;
    float phase_scale[256];  // per batch: 1 / (lambda d); the phase is pi * scale * r^2
    __device__ float2 operator()(long long row, int i) const {
        const int b = (int)(row / h), y = (int)(row % h);
        const float x0 = w > 1 ? -1.0f + (float)i * (2.0f / (float)(w - 1)) : -1.0f;
        const float y0 = h > 1 ? -1.0f + (float)y * (2.0f / (float)(h - 1)) : -1.0f;
        const float a = __ldg(aperture + (size_t)y * w + i);
        float s, c;
        sincospif(phase_scale[b] * (x0 * x0 + y0 * y0), &s, &c);
        return make_float2(a * c, a * s);
    }
};

// Store callbacks: receive the transformed element i of row `row`.
struct StoreTransposed {  // out[batch][i][r] (row = batch * rows + r), scaled
    float2* out;
    int n, rows;
    float scale;
    __device__ void operator()(long long row, int i, float2 v) const {
        const long long b = row / rows, r = row % rows;
        out[(b * n + i) * rows + r] = make_float2(v.x * scale, v.y * scale);
    }
};
struct StorePower {  // |v|^2 at the fftshift position of the [batch][rows][n] image
    float* out;
    int n, rows;
    __device__ void operator()(long long row, int i, float2 v) const {
        const long long b = row / rows, r = row % rows;  // r = original column, i = original row
        const int ys = (i + n / 2) % n, xs = (int)((r + rows / 2) % rows);
        out[(b * n + ys) * rows + xs] = v.x * v.x + v.y * v.y;
    }
};

template <class Load, class Store>
__global__ void k_fft_rows(Load load, Store store, int n, int log_n, float dir) {
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* tw = sm + n;
    const long long row = blockIdx.x;
    for (int k = threadIdx.x; k < n / 2; k += blockDim.x) {
        float s, c;
        sincospif(dir * 2.0f * (float)k / (float)n, &s, &c);  // exp(dir * 2 pi i k / n)
        tw[k] = make_float2(c, s);
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int rev = (int)(__brev((unsigned)i) >> (32 - log_n));
        x[rev] = load(row, i);
    }
    __syncthreads();
    for (int s = 1; s <= log_n; s++) {
        const int half = 1 << (s - 1);
        const int stride = n >> s;  // twiddle index step
        for (int k = threadIdx.x; k < n / 2; k += blockDim.x) {
            const int j = k & (half - 1);
            const int base = (k >> (s - 1)) << s;
            const float2 u = x[base + j];
            const float2 v = cmul(x[base + j + half], tw[j * stride]);
            x[base + j] = make_float2(u.x + v.x, u.y + v.y);
            x[base + j + half] = make_float2(u.x - v.x, u.y - v.y);
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) store(row, i, x[i]);
}

int log2_exact(int n) {
    if (n < 2 || n > 2 * kMaxN || (n & (n - 1))) return -1;
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

// lengths the row transforms accept: 2 to 4096, any factorisation
bool fft_length_ok(int n) { return n >= 2 && n <= kMaxN; }

// exp(d pi i m^2 / n), the phase reduced exactly: m^2 mod 2n
__device__ __forceinline__ float2 bluestein_chirp(int m, int n, float d) {
    const long long r = ((long long)m * m) % (2LL * n);
    float sn, cs;
    sincospif(d * (float)r / (float)n, &sn, &cs);
    return make_float2(cs, sn);
}

// the radix-2 butterflies of k_fft_rows over two arrays at once (input in bit-reversed order,
// output in natural order), twiddles tw[k] = exp(-2 pi i k / M)
__device__ __forceinline__ void butterflies2(float2* x, float2* y, const float2* tw, int M, int logM) {
    for (int s = 1; s <= logM; s++) {
        const int half = 1 << (s - 1);
        const int stride = M >> s;
        for (int k = threadIdx.x; k < M / 2; k += blockDim.x) {
            const int j = k & (half - 1);
            const int base = (k >> (s - 1)) << s;
            const float2 w = tw[j * stride];
            float2 u = x[base + j], v = cmul(x[base + j + half], w);
            x[base + j] = make_float2(u.x + v.x, u.y + v.y);
            x[base + j + half] = make_float2(u.x - v.x, u.y - v.y);
            if (y) {
                u = y[base + j];
                v = cmul(y[base + j + half], w);
                y[base + j] = make_float2(u.x + v.x, u.y + v.y);
                y[base + j + half] = make_float2(u.x - v.x, u.y - v.y);
            }
        }
        __syncthreads();
    }
}

// One row of any length n (Bluestein): a_j = x_j w_j and b_m = conj(w_m) for |m| < n
// (wrapped to M - m), A = FFT(a), B = FFT(b), conv = IFFT(A B) (as conj(FFT(conj(A B))) / M),
// X_k = w_k conv_k. Shared memory: a, b (M each) and the twiddles (M / 2).
template <class Load, class Store>
__global__ void k_fft_rows_bluestein(Load load, Store store, int n, int M, int logM, float dir) {
    extern __shared__ float2 sm[];
    float2* a = sm;
    float2* b = a + M;
    float2* tw = b + M;
    const long long row = blockIdx.x;
    for (int k = threadIdx.x; k < M / 2; k += blockDim.x) {
        float sn, cs;
        sincospif(-2.0f * (float)k / (float)M, &sn, &cs);
        tw[k] = make_float2(cs, sn);
    }
    for (int i = threadIdx.x; i < M; i += blockDim.x) {
        float2 av = make_float2(0.0f, 0.0f), bv = make_float2(0.0f, 0.0f);
        if (i < n) {
            const float2 w = bluestein_chirp(i, n, dir);
            av = cmul(load(row, i), w);
            bv = make_float2(w.x, -w.y);
        } else if (i > M - n) {
            const float2 w = bluestein_chirp(M - i, n, dir);
            bv = make_float2(w.x, -w.y);
        }
        const int rev = (int)(__brev((unsigned)i) >> (32 - logM));
        a[rev] = av;
        b[rev] = bv;
    }
    __syncthreads();
    butterflies2(a, b, tw, M, logM);
    for (int i = threadIdx.x; i < M; i += blockDim.x) a[i] = cmul(a[i], b[i]);
    __syncthreads();
    for (int i = threadIdx.x; i < M; i += blockDim.x) {
        const float2 v = a[i];
        b[(int)(__brev((unsigned)i) >> (32 - logM))] = make_float2(v.x, -v.y);
    }
    __syncthreads();
    butterflies2(b, nullptr, tw, M, logM);
    const float inv = 1.0f / (float)M;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const float2 c = make_float2(b[k].x * inv, -b[k].y * inv);
        store(row, k, cmul(bluestein_chirp(k, n, dir), c));
    }
}

template <class Load, class Store>
int launch_rows(Load load, Store store, long long rows, int n, float dir, cudaStream_t s) {
    if (!fft_length_ok(n)) return RF_ERR_NOT_SUPPORTED;
    if (n & (n - 1)) {
        int M = 1;
        while (M < 2 * n - 1) M <<= 1;
        const int logM = log2_exact(M);
        const size_t smem = sizeof(float2) * (2 * M + M / 2);
        auto kernel = k_fft_rows_bluestein<Load, Store>;
        if (smem > 48 * 1024)
            RF_TRY(cuda_status(
                cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)));
        kernel<<<(unsigned)rows, M / 2 < 256 ? (M / 2 < 32 ? 32 : M / 2) : 256, smem, s>>>(load, store, n, M, logM,
                                                                                            dir);
        return launch_status();
    }
    const int log_n = log2_exact(n);
    const int threads = n / 2 < 256 ? (n / 2 < 32 ? 32 : n / 2) : 256;
    const size_t smem = sizeof(float2) * (n + n / 2);
    auto kernel = k_fft_rows<Load, Store>;
    if (smem > 48 * 1024)
        RF_TRY(cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)));
    kernel<<<(unsigned)rows, threads, smem, s>>>(load, store, n, log_n, dir);
    return launch_status();
}

// 2-D transform of data [batch][h][w] in place (scratch of the same size).
int fft2(float2* data, float2* scratch, int batch, int w, int h, int direction, float scale, cudaStream_t s) {
    const float dir = direction < 0 ? -1.0f : 1.0f;
    RF_TRY(launch_rows(LoadComplex{data, w}, StoreTransposed{scratch, w, h, 1.0f}, (long long)batch * h, w, dir, s));
    return launch_rows(LoadComplex{scratch, h}, StoreTransposed{data, h, w, scale}, (long long)batch * w, h, dir, s);
}

// ---------------------------------------------------------------- FRFT helpers
// numpy's fftshift moves element i to (i + n / 2) mod n: output i reads (i + n - n / 2) mod n
__global__ void k_fftshift_real(const float* __restrict__ in, float2* __restrict__ out, int w, int h) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)w * h) return;
    const int y = (int)(i / w), x = (int)(i % w);
    out[i] = make_float2(in[(size_t)((y + h - h / 2) % h) * w + (x + w - w / 2) % w], 0.0f);
}

__global__ void k_flip(const float2* __restrict__ in, float2* __restrict__ out, int w, int h) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)w * h) return;
    const int y = (int)(i / w), x = (int)(i % w);
    out[i] = in[(size_t)(h - 1 - y) * w + (w - 1 - x)];
}

// chirp(shape) of frft.py:8-17: pi * (a^2 / h + b^2 / w), a/b = fftshift(arange(-n/2, n/2))
__device__ __forceinline__ float chirp_r(int y, int x, int w, int h) {
    const int a = y < h / 2 ? y : y - h;
    const int b = x < w / 2 ? x : x - w;
    return (float)(a * a) / (float)h + (float)(b * b) / (float)w;
}

// mode 0: data *= exp(i pi r c1); mode 1: data = exp(i pi r c2)
__global__ void k_chirp(float2* __restrict__ data, int w, int h, float c, int mode) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)w * h) return;
    const int y = (int)(i / w), x = (int)(i % w);
    float s, co;
    sincospif(chirp_r(y, x, w, h) * c, &s, &co);
    const float2 e = make_float2(co, s);
    data[i] = mode == 0 ? cmul(data[i], e) : e;
}

__global__ void k_cmul(float2* __restrict__ a, const float2* __restrict__ b, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = cmul(a[i], b[i]);
}

// out = |fftshift(scale * chirp1 * data)| * norm
__global__ void k_frft_finish(const float2* __restrict__ data, float* __restrict__ out, int w, int h, float c1,
                              float2 scale, float norm) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)w * h) return;
    const int y = (int)(i / w), x = (int)(i % w);
    const int ys = (y + h - h / 2) % h, xs = (x + w - w / 2) % w;  // fftshift source
    float s, co;
    sincospif(chirp_r(ys, xs, w, h) * c1, &s, &co);
    float2 v = cmul(cmul(scale, make_float2(co, s)), data[(size_t)ys * w + xs]);
    out[i] = sqrtf(v.x * v.x + v.y * v.y) * norm;
}

}  // namespace
}  // namespace rf

extern "C" int rf_fft2(float* data, float* scratch, int32_t batch, int32_t width, int32_t height, int32_t direction,
                       float scale, void* stream) {
    using namespace rf;
    if (!data || !scratch || batch < 1) return RF_ERR_INVALID_ARG;
    if (!fft_length_ok(width) || !fft_length_ok(height)) return RF_ERR_NOT_SUPPORTED;
    return fft2((float2*)data, (float2*)scratch, batch, width, height, direction, scale, (cudaStream_t)stream);
}

extern "C" int rf_starburst_spectrum(const float* aperture, int32_t width, int32_t height, const float* lambdas_mm,
                                     int32_t count, float distance_mm, float* scratch, float* spectrum,
                                     void* stream) {
    using namespace rf;
    if (!aperture || !lambdas_mm || !scratch || !spectrum || count < 1 || count > 256) return RF_ERR_INVALID_ARG;
    if (!fft_length_ok(width) || !fft_length_ok(height)) return RF_ERR_NOT_SUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    // phase = pi * (x^2 + y^2) / (lambda d): one factor per wavelength, passed by value
    LoadStarburst load;
    load.aperture = aperture;
    load.w = width;
    load.h = height;
    for (int b = 0; b < count; b++) load.phase_scale[b] = (float)(1.0 / ((double)lambdas_mm[b] * (double)distance_mm));
    float2* buf = (float2*)scratch;
    // rows: aperture * chirp -> transposed; columns: -> |F|^2 at the fftshift position
    RF_TRY(launch_rows(load, StoreTransposed{buf, width, height, 1.0f}, (long long)count * height, width, -1.0f, s));
    return launch_rows(LoadComplex{buf, height}, StorePower{spectrum, height, width}, (long long)count * width,
                       height, -1.0f, s);
}

extern "C" int rf_ghost_frft(const float* aperture, int32_t width, int32_t height, float alpha, float* scratch,
                             float* texture, void* stream) {
    using namespace rf;
    if (!aperture || !scratch || !texture) return RF_ERR_INVALID_ARG;
    if (!fft_length_ok(width) || !fft_length_ok(height)) return RF_ERR_NOT_SUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = (long long)width * height;
    float2* A = (float2*)scratch;
    float2* B = A + n;
    float2* T = B + n;
    const unsigned blocks = blocks_for(n, 256);
    const float ortho = (float)(1.0 / std::sqrt((double)n));
    k_fftshift_real<<<blocks, 256, 0, s>>>(aperture, A, width, height);
    RF_TRY(launch_status());
    // normalize() of frft.py:20-40, in double on the host
    double rel = std::fmod((double)alpha, 4.0);
    if (rel < 0) rel += 4.0;
    double a;
    if (rel < 0.5) {
        a = rel + 1;
        RF_TRY(fft2(A, T, 1, width, height, +1, ortho, s));
    } else if (rel < 1.5) {
        a = rel;
    } else if (rel < 2.5) {
        a = rel - 1;
        RF_TRY(fft2(A, T, 1, width, height, -1, ortho, s));
    } else if (rel < 3.5) {
        a = rel - 2;
        k_flip<<<blocks, 256, 0, s>>>(A, T, width, height);
        RF_TRY(launch_status());
        RF_TRY(cuda_status(cudaMemcpyAsync(A, T, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s)));
    } else {
        a = rel - 3;
        RF_TRY(fft2(A, T, 1, width, height, +1, ortho, s));
    }
    const double phi = a * M_PI / 2.0;
    const double cot = 1.0 / std::tan(phi);
    const double sq = std::sqrt(1.0 + cot * cot);
    const std::complex<double> scale = std::sqrt(std::complex<double>(1.0, -cot)) / std::sqrt((double)n);
    const float c1 = (float)(cot - sq), c2 = (float)sq;
    // fft2 = fftn(chirp1 * A); fft1 = fftn(chirp2); A = ifftn(fft1 * fft2)
    k_chirp<<<blocks, 256, 0, s>>>(A, width, height, c1, 0);
    RF_TRY(launch_status());
    RF_TRY(fft2(A, T, 1, width, height, -1, ortho, s));
    k_chirp<<<blocks, 256, 0, s>>>(B, width, height, c2, 1);
    RF_TRY(launch_status());
    RF_TRY(fft2(B, T, 1, width, height, -1, ortho, s));
    k_cmul<<<blocks, 256, 0, s>>>(A, B, n);
    RF_TRY(launch_status());
    RF_TRY(fft2(A, T, 1, width, height, +1, ortho, s));
    // |fftshift(scale * chirp1 * A)| * sqrt(w * h), ghost.py:33-35
    k_frft_finish<<<blocks, 256, 0, s>>>(A, texture, width, height, c1,
                                         make_float2((float)scale.real(), (float)scale.imag()),
                                         (float)std::sqrt((double)n));
    return launch_status();
}

// ---------------------------------------------------------------- no-allocation variant
//
// Some callers cannot allocate device memory at render time: a plugin inside a host
// application that owns every device allocation through its own pool (and forbids
// cudaMalloc in its render callback), or a real-time loop that must not allocate after
// start-up because an allocation can synchronise the device and stall a frame. For them,
// rf_ghost_frft_static keeps its scratch in this file-scope device array instead of a
// caller buffer. Every GPU that loads the library holds the array (6 MiB) until the
// process exits; all calls share it.
static __device__ __align__(256) float2 g_ghost_frft_scratch[3 * RF_GHOST_FRFT_STATIC_MAX_PIXELS];

namespace rf {
namespace {
// Device address of the static scratch on the current device. The host-side symbol is
// not a device address; the lookup runs on every call (it is cheap), so a pointer is
// never kept across a device reset, after which the module and its array are reloaded.
int static_scratch(float** out) {
    void* p = nullptr;
    RF_TRY(cuda_status(cudaGetSymbolAddress(&p, g_ghost_frft_scratch)));
    *out = (float*)p;
    return RF_OK;
}
}  // namespace
}  // namespace rf

extern "C" int rf_ghost_frft_static(const float* aperture, int32_t width, int32_t height, float alpha,
                                    float* texture, void* stream) {
    using namespace rf;
    if (!aperture || !texture || width < 1 || height < 1) return RF_ERR_INVALID_ARG;
    if ((long long)width * height > RF_GHOST_FRFT_STATIC_MAX_PIXELS) {
        set_error_text("rf_ghost_frft_static: width * height exceeds RF_GHOST_FRFT_STATIC_MAX_PIXELS (512 x 512)");
        return RF_ERR_INVALID_ARG;
    }
    float* scratch = nullptr;
    RF_TRY(static_scratch(&scratch));
    // every scratch plane is fully written before it is read, so the previous call's
    // contents never need clearing
    return rf_ghost_frft(aperture, width, height, alpha, scratch, texture, stream);
}
