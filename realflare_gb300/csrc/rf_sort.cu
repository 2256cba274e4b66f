// rf_sort.cu — device-wide exclusive scan and stable LSD radix sort of (key, value) pairs.
//
// Scan: reduce-then-scan over 2048-element chunks (256 threads x 8 items), recursing on
// the chunk sums. Radix sort: 8-bit digits; per pass a block histogram, a scan of the
// (digit, block) counts in digit-major order, and a stable scatter in which each warp
// ranks its items in input order with __match_any_sync and the warps' counts are
// prefixed per digit; the block stages its chunk in shared memory in (digit, input) order
// and writes each digit's run with consecutive threads. Stability makes the output ordered
// by (key, input position).
#include "rf_common.cuh"

namespace rf {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kChunk = kThreads * kItems;  // 2048
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < kWarps ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < kWarps; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kWarps) warp_sums[lane] = s;  // inclusive
    }
    __syncthreads();
    uint32_t before = warp == 0 ? 0u : warp_sums[warp - 1];
    if (total) *total = warp_sums[kWarps - 1];
    return before + x - v;
}

__global__ void __launch_bounds__(kThreads) k_scan_reduce(const uint32_t* __restrict__ in, long long n,
                                                          uint32_t* __restrict__ sums) {
    __shared__ uint32_t ws[kWarps];
    const long long base = (long long)blockIdx.x * kChunk;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + (long long)k * kThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kWarps; w++) t += ws[w];
        sums[blockIdx.x] = t;
    }
}

// Each thread owns kItems consecutive elements (blocked arrangement).
__global__ void __launch_bounds__(kThreads) k_scan_apply(const uint32_t* in, uint32_t* out, long long n,
                                                         const uint32_t* __restrict__ offsets) {
    __shared__ uint32_t ws[kWarps];
    const long long base = (long long)blockIdx.x * kChunk + (long long)threadIdx.x * kItems;
    uint32_t v[kItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + k;
        v[k] = i < n ? in[i] : 0u;
        s += v[k];
    }
    uint32_t run = block_exclusive_scan(s, ws, nullptr) + (offsets ? offsets[blockIdx.x] : 0u);
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

// ---------------------------------------------------------------- radix sort
__global__ void __launch_bounds__(kThreads) k_radix_hist(const uint32_t* __restrict__ keys, long long n, int shift,
                                                         int nblocks, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kChunk;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + (long long)k * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kThreads) k_radix_scatter(const uint32_t* __restrict__ keys,
                                                            const uint32_t* __restrict__ vals, long long n, int shift,
                                                            int nblocks, const uint32_t* __restrict__ offsets,
                                                            uint32_t* __restrict__ keys_out,
                                                            uint32_t* __restrict__ vals_out) {
    __shared__ uint32_t warp_count[kWarps][257];
    __shared__ uint32_t stage_k[kChunk], stage_v[kChunk];  // the chunk in (digit, input) order
    __shared__ uint32_t digit_start[256], digit_out[256], warp_sums[kWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarps * 257; i += kThreads) (&warp_count[0][0])[i] = 0;
    __syncthreads();
    // warp w owns items [base + w*256, base + (w+1)*256), processed in 8 rounds of 32 in
    // increasing index order
    const long long wbase = (long long)blockIdx.x * kChunk + (long long)warp * (kItems * 32);
    uint32_t key[kItems], val[kItems], rank[kItems];
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        long long i = wbase + (long long)r * 32 + lane;
        bool ok = i < n;
        key[r] = ok ? keys[i] : 0u;
        val[r] = ok ? vals[i] : 0u;
        uint32_t d = ok ? ((key[r] >> shift) & 255u) : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (lane == leader) {
            before = warp_count[warp][d];
            warp_count[warp][d] = before + __popc(peers);
        }
        before = __shfl_sync(0xffffffffu, before, leader);
        rank[r] = before + __popc(peers & lt_mask);
        __syncwarp();
    }
    __syncthreads();
    // per digit (thread d): prefix over warps, the block's count of the digit, and where its
    // run starts in the block (a scan over digits) and in the output (the global offset)
    {
        const int d = threadIdx.x;  // 256 threads = 256 digits
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kWarps; w++) {
            uint32_t c = warp_count[w][d];
            warp_count[w][d] = run;
            run += c;
        }
        const uint32_t start = block_exclusive_scan(run, warp_sums, nullptr);
        digit_start[d] = start;
        digit_out[d] = offsets[(size_t)d * nblocks + blockIdx.x];
    }
    __syncthreads();
    // stage every item at its place in the block's digit-ordered chunk ...
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        long long i = wbase + (long long)r * 32 + lane;
        if (i < n) {
            uint32_t d = (key[r] >> shift) & 255u;
            uint32_t lp = digit_start[d] + warp_count[warp][d] + rank[r];
            stage_k[lp] = key[r];
            stage_v[lp] = val[r];
        }
    }
    __syncthreads();
    // ... and write the chunk out with consecutive threads on consecutive places of each run
    const long long in_block = n - (long long)blockIdx.x * kChunk;
    const int count = in_block < kChunk ? (int)in_block : kChunk;
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        const int lp = r * kThreads + threadIdx.x;
        if (lp < count) {
            const uint32_t k = stage_k[lp];
            const uint32_t d = (k >> shift) & 255u;
            const uint32_t pos = digit_out[d] + (uint32_t)lp - digit_start[d];
            keys_out[pos] = k;
            vals_out[pos] = stage_v[lp];
        }
    }
}

}  // namespace

size_t scan_scratch_words(long long n) {
    size_t words = 0;
    long long m = n;
    while (m > kChunk) {
        m = (m + kChunk - 1) / kChunk;
        words += (size_t)m + 64;
    }
    return words + 64;
}

int exclusive_scan_u32(const uint32_t* in, uint32_t* out, long long n, uint32_t* scratch, cudaStream_t s) {
    if (n <= 0) return RF_OK;
    const long long nb = (n + kChunk - 1) / kChunk;
    if (nb == 1) {
        k_scan_apply<<<1, kThreads, 0, s>>>(in, out, n, nullptr);
        return launch_status();
    }
    uint32_t* sums = scratch;
    uint32_t* rest = scratch + nb + 64;
    k_scan_reduce<<<(unsigned)nb, kThreads, 0, s>>>(in, n, sums);
    RF_TRY(launch_status());
    RF_TRY(exclusive_scan_u32(sums, sums, nb, rest, s));
    k_scan_apply<<<(unsigned)nb, kThreads, 0, s>>>(in, out, n, sums);
    return launch_status();
}

size_t radix_scratch_words(long long n) {
    const long long nb = (n + kChunk - 1) / kChunk;
    return (size_t)(256 * nb) + scan_scratch_words(256 * nb) + 64;
}

int radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, long long n,
                     int key_bits, uint32_t* scratch, bool* result_in_alt, cudaStream_t s) {
    *result_in_alt = false;
    if (n <= 1 || key_bits <= 0) return RF_OK;
    const long long nb = (n + kChunk - 1) / kChunk;
    if (nb > 0x7fffffffLL) return RF_ERR_INVALID_ARG;
    uint32_t* hist = scratch;
    uint32_t* sscr = scratch + 256 * nb;
    uint32_t *ka = keys, *va = vals, *kb = keys_alt, *vb = vals_alt;
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_radix_hist<<<(unsigned)nb, kThreads, 0, s>>>(ka, n, shift, (int)nb, hist);
        RF_TRY(launch_status());
        RF_TRY(exclusive_scan_u32(hist, hist, 256 * nb, sscr, s));
        k_radix_scatter<<<(unsigned)nb, kThreads, 0, s>>>(ka, va, n, shift, (int)nb, hist, kb, vb);
        RF_TRY(launch_status());
        uint32_t* t = ka;
        ka = kb;
        kb = t;
        t = va;
        va = vb;
        vb = t;
        *result_in_alt = !*result_in_alt;
    }
    return RF_OK;
}

}  // namespace rf
