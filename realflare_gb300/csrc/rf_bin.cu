// rf_bin.cu — binning of ghost quads.
//
// The reference bins primitives into BIN_SIZE-pixel bins with 255-primitive bit masks
// (realflare/api/tasks/cl/rasterizing.cl:388-469) and then lets every pixel scan every
// mask of its bin. Here a primitive's reference bins form a rectangle, computed with the
// reference's exact integer test (convert_int4 truncation, integer res / 2, inclusive
// overlap on both ends), and:
//  * rf_bin_masks materialises the reference's mask layout from those rectangles (parity);
//  * rf_bin_tiles emits one entry per (primitive, wavelength pair, raster tile) where the
//    tile lies in the primitive's reference bins and in the conservative bounds of that
//    wavelength pair's quads, then orders every tile's entries by (primitive, pair) with a
//    stable radix sort keyed by tile. The raster then visits exactly the reference's
//    (pixel, primitive) candidates that can produce coverage, in the reference's order.
#include <algorithm>

#include "rf_common.cuh"

namespace rf {
namespace {

constexpr int kThreads = 256;
// Sample coordinates below this magnitude keep the reference's 32-bit edge functions
// free of overflow (|difference| < 2^15, |product| < 2^30), so a sample outside the
// integer bounds of a quad is never inside it.
constexpr float kSafeSamples = 16383.0f;

struct BinGeometry {
    int width, height, B, T, bdx, bdy, ntx, nty, S, W, G, maxW;
    float st;
    bool safe_screen;  // width * S and height * S fit the overflow-free range
};

__device__ __forceinline__ long long floor_div(long long a, long long b) {
    long long q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}

// Reference bins overlapped by a primitive's bounds (mm), rasterizing.cl:449-453.
// Returns false for culled primitives (bounds.x NaN) or empty rectangles.
__device__ __forceinline__ bool ref_bin_rect(float4 b, const BinGeometry& g, int& bx0, int& bx1, int& by0,
                                             int& by1) {
    if (isnan(b.x)) return false;
    int32_t sx0 = wadd(cvt_rz_sat(b.x * g.st), g.width / 2);
    int32_t sy0 = wadd(cvt_rz_sat(b.y * g.st), g.height / 2);
    int32_t sx1 = wadd(cvt_rz_sat(b.z * g.st), g.width / 2);
    int32_t sy1 = wadd(cvt_rz_sat(b.w * g.st), g.height / 2);
    // bin bx covers [bx*B, bx*B + B] inclusive: sx0 <= bx*B + B and sx1 >= bx*B
    long long lx = floor_div((long long)sx0 - 1, g.B), hx = floor_div((long long)sx1, g.B);
    long long ly = floor_div((long long)sy0 - 1, g.B), hy = floor_div((long long)sy1, g.B);
    lx = max(lx, 0LL);
    ly = max(ly, 0LL);
    hx = min(hx, (long long)g.bdx - 1);
    hy = min(hy, (long long)g.bdy - 1);
    if (lx > hx || ly > hy) return false;
    bx0 = (int)lx;
    bx1 = (int)hx;
    by0 = (int)ly;
    by1 = (int)hy;
    return true;
}

__global__ void __launch_bounds__(kThreads) k_bin_masks(const float4* __restrict__ bounds, int prim_count,
                                                        BinGeometry g, int batch_count,
                                                        unsigned long long* __restrict__ masks) {
    const int prim = blockIdx.x * kThreads + threadIdx.x;
    if (prim >= prim_count) return;
    int bx0, bx1, by0, by1;
    if (!ref_bin_rect(bounds[prim], g, bx0, bx1, by0, by1)) return;
    const int batch = prim / RF_BATCH_PRIMITIVE_COUNT;
    const int bit = prim % RF_BATCH_PRIMITIVE_COUNT + 1;
    for (int by = by0; by <= by1; by++)
        for (int bx = bx0; bx <= bx1; bx++) {
            unsigned long long* q = masks + 4 * ((size_t)(by * g.bdx + bx) * batch_count + batch);
            atomicOr(q + (bit >> 6), 1ull << (bit & 63));
            atomicOr(q, 1ull);
        }
}

// Tile rectangle of one (primitive, wavelength pair); false when it contributes nothing.
__device__ __forceinline__ bool pair_tile_rect(const float4* __restrict__ bounds, const float4* __restrict__ vtx,
                                               long long prim, int w, const BinGeometry& g, int& tx0, int& tx1,
                                               int& ty0, int& ty1) {
    int bx0, bx1, by0, by1;
    if (!ref_bin_rect(__ldg(bounds + prim), g, bx0, bx1, by0, by1)) return false;
    const int Q = (g.G - 1) * (g.G - 1), VC = g.G * g.G;
    const long long path = prim / Q;
    const int quad = (int)(prim % Q);
    const int row = quad / (g.G - 1), col = quad % (g.G - 1);
    const int c0 = row * g.G + col;
    const int corners[4] = {c0, c0 + 1, c0 + 1 + g.G, c0 + g.G};
    float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const long long vi = (path * VC + corners[k]) * g.W + w;
#pragma unroll
        for (int e = 0; e < 2; e++) {  // endpoints at pair wavelengths w and w + 1
            const float4 a = __ldg(vtx + 2 * (vi + e));
            const float refl = __ldg(&vtx[2 * (vi + e) + 1].y);
            if (isnan(refl)) return false;  // an invalid endpoint: the pair contributes 0
            finite = finite && isfinite(a.x) && isfinite(a.y);
            mnx = fminf(mnx, a.x);
            mxx = fmaxf(mxx, a.x);
            mny = fminf(mny, a.y);
            mxy = fmaxf(mxy, a.y);
        }
    }
    const int tpb = g.B / g.T;  // tiles per bin edge
    tx0 = bx0 * tpb;
    tx1 = min((bx1 + 1) * tpb - 1, g.ntx - 1);
    ty0 = by0 * tpb;
    ty1 = min((by1 + 1) * tpb - 1, g.nty - 1);
    const float S = (float)g.S;
    const bool safe = g.safe_screen && finite && fabsf(mnx * S) < kSafeSamples && fabsf(mxx * S) < kSafeSamples &&
                      fabsf(mny * S) < kSafeSamples && fabsf(mxy * S) < kSafeSamples;
    if (safe) {
        // pixels with a sample inside the quads lie within [min - 2, max + 2]
        tx0 = max(tx0, (int)floorf((mnx - 2.0f) / (float)g.T));
        tx1 = min(tx1, (int)floorf((mxx + 2.0f) / (float)g.T));
        ty0 = max(ty0, (int)floorf((mny - 2.0f) / (float)g.T));
        ty1 = min(ty1, (int)floorf((mxy + 2.0f) / (float)g.T));
    }
    return tx0 <= tx1 && ty0 <= ty1;
}

__global__ void __launch_bounds__(kThreads) k_pair_count(const float4* __restrict__ bounds,
                                                         const float4* __restrict__ vtx, long long n_pairs,
                                                         BinGeometry g, uint32_t* __restrict__ counts,
                                                         unsigned long long* __restrict__ total) {
    const long long j = (long long)blockIdx.x * kThreads + threadIdx.x;
    unsigned long long c = 0;
    if (j < n_pairs) {
        int tx0, tx1, ty0, ty1;
        if (pair_tile_rect(bounds, vtx, j / g.maxW, (int)(j % g.maxW), g, tx0, tx1, ty0, ty1))
            c = (unsigned long long)(tx1 - tx0 + 1) * (unsigned long long)(ty1 - ty0 + 1);
        counts[j] = (uint32_t)min(c, 0xffffffffull);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

__global__ void __launch_bounds__(kThreads) k_pair_emit(const float4* __restrict__ bounds,
                                                        const float4* __restrict__ vtx, long long n_pairs,
                                                        BinGeometry g, const uint32_t* __restrict__ offsets,
                                                        uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const long long j = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (j >= n_pairs) return;
    int tx0, tx1, ty0, ty1;
    if (!pair_tile_rect(bounds, vtx, j / g.maxW, (int)(j % g.maxW), g, tx0, tx1, ty0, ty1)) return;
    uint32_t o = offsets[j];
    for (int ty = ty0; ty <= ty1; ty++)
        for (int tx = tx0; tx <= tx1; tx++) {
            keys[o] = (uint32_t)(ty * g.ntx + tx);
            vals[o] = (uint32_t)j;
            o++;
        }
}

// tile_offsets[t] = first position of key >= t in the sorted keys
__global__ void k_tile_offsets(const uint32_t* __restrict__ keys, long long n, int ntiles,
                               uint32_t* __restrict__ tile_offsets) {
    const int t = blockIdx.x * kThreads + threadIdx.x;
    if (t > ntiles) return;
    long long lo = 0, hi = n;
    while (lo < hi) {
        long long mid = (lo + hi) >> 1;
        if (keys[mid] < (uint32_t)t) lo = mid + 1;
        else hi = mid;
    }
    tile_offsets[t] = (uint32_t)lo;
}

// Raster tiles are 32 x 32 (default) or 16 x 16 pixels (rf_raster.cu); bins must be
// multiples of the tile.
__host__ __device__ inline int auto_tile(const rf_raster_args& a) { return a.tile_size > 0 ? a.tile_size : 32; }

__host__ __device__ inline bool make_geometry(const rf_raster_args& a, BinGeometry& g) {
    if (a.width < 1 || a.height < 1 || a.bin_size < 1 || a.grid_count < 2 || a.wavelength_count < 1 ||
        a.path_count < 0)
        return false;
    g.width = a.width;
    g.height = a.height;
    g.B = a.bin_size;
    g.T = auto_tile(a);
    if ((g.T != 32 && g.T != 16) || g.B % g.T) return false;
    g.bdx = (a.width + g.B - 1) / g.B;
    g.bdy = (a.height + g.B - 1) / g.B;
    g.ntx = (a.width + g.T - 1) / g.T;
    g.nty = (a.height + g.T - 1) / g.T;
    g.S = a.sub_steps;
    g.W = a.wavelength_count;
    g.G = a.grid_count;
    g.maxW = a.wavelength_count - 1 > 1 ? a.wavelength_count - 1 : 1;
    g.st = a.screen_transform;
    g.safe_screen = (float)a.width * a.sub_steps <= 16384.0f && (float)a.height * a.sub_steps <= 16384.0f;
    return true;
}

// ---------------------------------------------------------------- batched frames
// Block b of a stage works for the frame whose first block is the largest one <= b; the
// frame's pairs, bounds and vertices are found through its offsets, and its tiles are
// numbered from tile_offset in the batch's tile numbering.
struct FramePairs {
    BinGeometry g;
    long long n_pairs, first;  // the frame's pair count and this thread's first local pair
    const float4* bounds;
    const float4* vtx;
    long long pair_offset;
    int tile_offset;
};

__device__ __forceinline__ bool frame_pairs(const rf_frame* __restrict__ frames, int F, const float4* bounds_all,
                                            const float4* vtx_all, int* frame_index, FramePairs& fp) {
    if (threadIdx.x == 0)
        *frame_index = find_frame(frames, F, blockIdx.x, [](const rf_frame& fr) { return fr.pair_block; });
    __syncthreads();
    const rf_frame& fr = frames[*frame_index];
    if (!make_geometry(fr.raster, fp.g)) return false;
    fp.n_pairs = (long long)fr.raster.path_count * (fp.g.G - 1) * (fp.g.G - 1) * fp.g.maxW;
    fp.first = (long long)(blockIdx.x - fr.pair_block) * kThreads + threadIdx.x;
    fp.bounds = bounds_all + fr.prim_offset;
    fp.vtx = vtx_all + 2 * fr.vertex_offset;
    fp.pair_offset = fr.pair_offset;
    fp.tile_offset = fr.tile_offset;
    return true;
}

__global__ void __launch_bounds__(kThreads) k_pair_count_batch(const rf_frame* __restrict__ frames, int F,
                                                               const float4* __restrict__ bounds_all,
                                                               const float4* __restrict__ vtx_all,
                                                               uint32_t* __restrict__ counts,
                                                               unsigned long long* __restrict__ total) {
    __shared__ int frame_index;
    FramePairs fp;
    const bool ok = frame_pairs(frames, F, bounds_all, vtx_all, &frame_index, fp);
    const long long j = fp.first;
    unsigned long long c = 0;
    if (ok && j < fp.n_pairs) {
        int tx0, tx1, ty0, ty1;
        if (pair_tile_rect(fp.bounds, fp.vtx, j / fp.g.maxW, (int)(j % fp.g.maxW), fp.g, tx0, tx1, ty0, ty1))
            c = (unsigned long long)(tx1 - tx0 + 1) * (unsigned long long)(ty1 - ty0 + 1);
        counts[fp.pair_offset + j] = (uint32_t)min(c, 0xffffffffull);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

__global__ void __launch_bounds__(kThreads) k_pair_emit_batch(const rf_frame* __restrict__ frames, int F,
                                                              const float4* __restrict__ bounds_all,
                                                              const float4* __restrict__ vtx_all,
                                                              const uint32_t* __restrict__ offsets,
                                                              long long capacity, uint32_t* __restrict__ keys,
                                                              uint32_t* __restrict__ vals) {
    __shared__ int frame_index;
    FramePairs fp;
    if (!frame_pairs(frames, F, bounds_all, vtx_all, &frame_index, fp)) return;
    const long long j = fp.first;
    if (j >= fp.n_pairs) return;
    int tx0, tx1, ty0, ty1;
    if (!pair_tile_rect(fp.bounds, fp.vtx, j / fp.g.maxW, (int)(j % fp.g.maxW), fp.g, tx0, tx1, ty0, ty1)) return;
    long long o = offsets[fp.pair_offset + j];
    for (int ty = ty0; ty <= ty1; ty++)
        for (int tx = tx0; tx <= tx1; tx++) {
            if (o < capacity) {  // an overflowing batch is reported through the entry total
                keys[o] = (uint32_t)(fp.tile_offset + ty * fp.g.ntx + tx);
                vals[o] = (uint32_t)j;
            }
            o++;
        }
}

// Entries [total, capacity) get the key `pad` (one past the last tile), so the sort over the
// whole capacity leaves them at the end.
__global__ void k_pad_entries(const unsigned long long* __restrict__ total, long long capacity, uint32_t pad,
                              uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= capacity || (unsigned long long)i < *total) return;
    keys[i] = pad;
    vals[i] = 0;
}

// Sort keys for the raster's tile order: 255 minus the tile's entry count as a tiny float
// (the position of its leading one bit and the three bits after it), so an ascending
// stable sort puts the heaviest tiles first, within 12.5 %, and ties in tile order; empty
// tiles, which still write their pixels, come last.
constexpr int kOrderKeyBits = 8;
__global__ void k_tile_order_keys(const uint32_t* __restrict__ tile_offsets, int tiles, uint32_t* __restrict__ keys,
                                  uint32_t* __restrict__ vals) {
    const int t = blockIdx.x * kThreads + threadIdx.x;
    if (t >= tiles) return;
    const uint32_t n = tile_offsets[t + 1] - tile_offsets[t];
    uint32_t key = 255;
    if (n > 0) {
        const int lz = __clz((int)n);
        const uint32_t e = 31 - lz, m = (n << lz) << 1 >> 29;  // the 3 bits after the leading one
        key = 255 - (e * 8 + m);
    }
    keys[t] = key;
    vals[t] = (uint32_t)t;
}

struct BinWorkspace {
    uint32_t *counts, *scan_scratch, *keys_a, *keys_b, *vals_tmp, *radix_scratch;
    unsigned long long* total;
    size_t bytes;
};

BinWorkspace layout(char* base, long long n_pairs, long long capacity) {
    BinWorkspace w;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    w.total = (unsigned long long*)take(sizeof(unsigned long long));
    w.counts = (uint32_t*)take(sizeof(uint32_t) * (size_t)(n_pairs + 1));
    w.scan_scratch = (uint32_t*)take(sizeof(uint32_t) * scan_scratch_words(n_pairs));
    w.keys_a = (uint32_t*)take(sizeof(uint32_t) * (size_t)capacity);
    w.keys_b = (uint32_t*)take(sizeof(uint32_t) * (size_t)capacity);
    w.vals_tmp = (uint32_t*)take(sizeof(uint32_t) * (size_t)capacity);
    w.radix_scratch = (uint32_t*)take(sizeof(uint32_t) * radix_scratch_words(capacity));
    w.bytes = off;
    return w;
}

}  // namespace

int tile_size_of(const rf_raster_args& a) { return auto_tile(a); }

BatchWorkspace batch_layout(char* base, const rf_batch_sizes& z, long long capacity) {
    BatchWorkspace w;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    const long long sort_n = capacity > z.tiles ? capacity : z.tiles;
    w.counts = (uint32_t*)take(sizeof(uint32_t) * (size_t)(z.pairs + 1));
    w.scan_scratch = (uint32_t*)take(sizeof(uint32_t) * scan_scratch_words(z.pairs));
    w.keys_a = (uint32_t*)take(sizeof(uint32_t) * (size_t)capacity);
    w.keys_b = (uint32_t*)take(sizeof(uint32_t) * (size_t)capacity);
    w.vals_tmp = (uint32_t*)take(sizeof(uint32_t) * (size_t)capacity);
    w.radix_scratch = (uint32_t*)take(sizeof(uint32_t) * radix_scratch_words(sort_n));
    w.order_keys = (uint32_t*)take(sizeof(uint32_t) * (size_t)z.tiles);
    w.order_vals = (uint32_t*)take(sizeof(uint32_t) * (size_t)z.tiles);
    w.order_keys_b = (uint32_t*)take(sizeof(uint32_t) * (size_t)z.tiles);
    w.order_vals_b = (uint32_t*)take(sizeof(uint32_t) * (size_t)z.tiles);
    w.queue = (uint32_t*)take(sizeof(uint32_t) * 4);
    w.bytes = off;
    return w;
}

// The tile order is sorted by 8-bit keys: one pass when there are two tiles or more, so it
// starts in the _b buffers and ends in order_vals; a single tile is never moved.
const uint32_t* batch_tile_order(const BatchWorkspace& w, const rf_batch_sizes& z) {
    return z.tiles > 1 ? w.order_vals : w.order_vals_b;
}

}  // namespace rf

extern "C" int rf_bin_masks(const float* bounds, int32_t prim_count, float screen_transform, int32_t width,
                            int32_t height, int32_t bin_size, uint64_t* masks, void* stream) {
    using namespace rf;
    if (!bounds || !masks || prim_count < 0 || width < 1 || height < 1 || bin_size < 1) return RF_ERR_INVALID_ARG;
    if (!aligned16(bounds)) return RF_ERR_INVALID_ARG;
    BinGeometry g = {};
    g.width = width;
    g.height = height;
    g.B = bin_size;
    g.bdx = (width + bin_size - 1) / bin_size;
    g.bdy = (height + bin_size - 1) / bin_size;
    g.st = screen_transform;
    const int batches = (prim_count + RF_BATCH_PRIMITIVE_COUNT - 1) / RF_BATCH_PRIMITIVE_COUNT;
    cudaStream_t s = (cudaStream_t)stream;
    RF_TRY(cuda_status(cudaMemsetAsync(masks, 0, sizeof(uint64_t) * 4 * (size_t)g.bdx * g.bdy * batches, s)));
    if (prim_count == 0) return RF_OK;
    k_bin_masks<<<blocks_for(prim_count, kThreads), kThreads, 0, s>>>((const float4*)bounds, prim_count, g, batches,
                                                                      (unsigned long long*)masks);
    return launch_status();
}

extern "C" int rf_raster_tiles(const rf_raster_args* args, int32_t* tile_size, int32_t* tile_count) {
    using namespace rf;
    if (!args) return RF_ERR_INVALID_ARG;
    BinGeometry g;
    if (!make_geometry(*args, g)) return RF_ERR_INVALID_ARG;
    if (tile_size) *tile_size = g.T;
    if (tile_count) *tile_count = g.ntx * g.nty;
    return RF_OK;
}

extern "C" int rf_bin_workspace_size(const rf_raster_args* args, int64_t entry_capacity, size_t* bytes) {
    using namespace rf;
    if (!args || !bytes || entry_capacity < 0) return RF_ERR_INVALID_ARG;
    BinGeometry g;
    if (!make_geometry(*args, g)) return RF_ERR_INVALID_ARG;
    const long long n_pairs = (long long)args->path_count * (g.G - 1) * (g.G - 1) * g.maxW;
    *bytes = layout(nullptr, n_pairs, entry_capacity).bytes;
    return RF_OK;
}

extern "C" int rf_bin_tiles(const float* bounds, const float* vertexes, const rf_raster_args* args, void* workspace,
                            size_t workspace_bytes, uint32_t* tile_offsets, uint32_t* tile_entries,
                            int64_t entry_capacity, int64_t* entry_count, void* stream) {
    using namespace rf;
    if (!bounds || !vertexes || !args || !workspace || !tile_offsets || !entry_count || entry_capacity < 0)
        return RF_ERR_INVALID_ARG;
    if (!aligned16(bounds) || !aligned16(vertexes) || !aligned16(workspace)) return RF_ERR_INVALID_ARG;
    BinGeometry g;
    if (!make_geometry(*args, g)) return RF_ERR_INVALID_ARG;
    const long long n_pairs = (long long)args->path_count * (g.G - 1) * (g.G - 1) * g.maxW;
    BinWorkspace w = layout((char*)workspace, n_pairs, entry_capacity);
    if (w.bytes > workspace_bytes) return RF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const int ntiles = g.ntx * g.nty;
    *entry_count = 0;
    RF_TRY(cuda_status(cudaMemsetAsync(w.total, 0, sizeof(unsigned long long), s)));
    if (n_pairs > 0) {
        k_pair_count<<<blocks_for(n_pairs, kThreads), kThreads, 0, s>>>((const float4*)bounds,
                                                                         (const float4*)vertexes, n_pairs, g,
                                                                         w.counts, w.total);
        RF_TRY(launch_status());
    }
    unsigned long long total = 0;
    RF_TRY(cuda_status(cudaMemcpyAsync(&total, w.total, sizeof(total), cudaMemcpyDeviceToHost, s)));
    RF_TRY(cuda_status(cudaStreamSynchronize(s)));
    *entry_count = (int64_t)total;
    if (total > 0xfffffff0ull) return RF_ERR_NOT_SUPPORTED;
    if ((long long)total > entry_capacity || (total > 0 && !tile_entries)) return RF_ERR_WORKSPACE;
    if (total == 0) return cuda_status(cudaMemsetAsync(tile_offsets, 0, sizeof(uint32_t) * (ntiles + 1), s));
    RF_TRY(exclusive_scan_u32(w.counts, w.counts, n_pairs, w.scan_scratch, s));
    int bits = 0;
    while ((1LL << bits) < ntiles) bits++;
    const int passes = (bits + 7) / 8;
    // arrange the ping-pong buffers so that the sorted values land in tile_entries
    uint32_t* vals_first = (passes % 2 == 0) ? tile_entries : w.vals_tmp;
    uint32_t* vals_alt = (passes % 2 == 0) ? w.vals_tmp : tile_entries;
    k_pair_emit<<<blocks_for(n_pairs, kThreads), kThreads, 0, s>>>((const float4*)bounds, (const float4*)vertexes,
                                                                    n_pairs, g, w.counts, w.keys_a, vals_first);
    RF_TRY(launch_status());
    bool in_alt = false;
    RF_TRY(radix_sort_pairs(w.keys_a, vals_first, w.keys_b, vals_alt, (long long)total, bits, w.radix_scratch,
                            &in_alt, s));
    const uint32_t* sorted_keys = in_alt ? w.keys_b : w.keys_a;
    k_tile_offsets<<<blocks_for(ntiles + 1, kThreads), kThreads, 0, s>>>(sorted_keys, (long long)total, ntiles,
                                                                          tile_offsets);
    return launch_status();
}

namespace rf {
namespace {
struct OrderWorkspace {
    uint32_t *keys, *keys_b, *vals_b, *radix_scratch;
    size_t bytes;
};
OrderWorkspace order_layout(char* base, int tiles) {
    OrderWorkspace w;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    w.keys = (uint32_t*)take(sizeof(uint32_t) * (size_t)tiles);
    w.keys_b = (uint32_t*)take(sizeof(uint32_t) * (size_t)tiles);
    w.vals_b = (uint32_t*)take(sizeof(uint32_t) * (size_t)tiles);
    w.radix_scratch = (uint32_t*)take(sizeof(uint32_t) * radix_scratch_words(tiles));
    w.bytes = off;
    return w;
}
}  // namespace
}  // namespace rf

extern "C" int rf_tile_order_workspace_size(int32_t tile_count, size_t* bytes) {
    if (!bytes || tile_count < 1) return RF_ERR_INVALID_ARG;
    *bytes = rf::order_layout(nullptr, tile_count).bytes;
    return RF_OK;
}

extern "C" int rf_tile_order(const uint32_t* tile_offsets, int32_t tile_count, void* workspace,
                             size_t workspace_bytes, uint32_t* tile_order, void* stream) {
    using namespace rf;
    if (!tile_offsets || !workspace || !tile_order || tile_count < 1) return RF_ERR_INVALID_ARG;
    if (!aligned16(workspace)) return RF_ERR_INVALID_ARG;
    OrderWorkspace w = order_layout((char*)workspace, tile_count);
    if (w.bytes > workspace_bytes) return RF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    k_tile_order_keys<<<blocks_for(tile_count, kThreads), kThreads, 0, s>>>(tile_offsets, tile_count, w.keys_b,
                                                                           w.vals_b);
    RF_TRY(launch_status());
    if (tile_count == 1) return cuda_status(cudaMemsetAsync(tile_order, 0, sizeof(uint32_t), s));
    // two or more tiles and 8 key bits: exactly one pass, so the sorted pairs land in the
    // alternate buffers (keys, tile_order)
    bool in_alt = false;
    return radix_sort_pairs(w.keys_b, w.vals_b, w.keys, tile_order, tile_count, kOrderKeyBits, w.radix_scratch,
                            &in_alt, s);
}

extern "C" int rf_batch_workspace_size(const rf_batch_sizes* sizes, int64_t entry_capacity, size_t* bytes) {
    using namespace rf;
    if (!sizes || !bytes || entry_capacity < 0) return RF_ERR_INVALID_ARG;
    *bytes = batch_layout(nullptr, *sizes, entry_capacity).bytes;
    return RF_OK;
}

extern "C" int rf_bin_tiles_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const float* bounds,
                                  const float* vertexes, void* workspace, size_t workspace_bytes,
                                  uint32_t* tile_offsets, uint32_t* tile_entries, int64_t entry_capacity,
                                  uint64_t* entry_total, void* stream) {
    using namespace rf;
    if (!frames || !sizes || !bounds || !vertexes || !workspace || !tile_offsets || !entry_total ||
        entry_capacity < 1 || !tile_entries)
        return RF_ERR_INVALID_ARG;
    if (!aligned16(bounds) || !aligned16(vertexes) || !aligned16(workspace)) return RF_ERR_INVALID_ARG;
    const rf_batch_sizes& z = *sizes;
    if (entry_capacity > 0xfffffff0LL || z.tiles < 1 || z.tiles > (1 << 30) || z.pair_blocks > 0x7fffffffLL)
        return RF_ERR_NOT_SUPPORTED;
    BatchWorkspace w = batch_layout((char*)workspace, z, entry_capacity);
    if (w.bytes > workspace_bytes) return RF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    RF_TRY(cuda_status(cudaMemsetAsync(entry_total, 0, sizeof(uint64_t), s)));
    if (z.pair_blocks > 0) {
        k_pair_count_batch<<<(unsigned)z.pair_blocks, kThreads, 0, s>>>(
            frames, z.frame_count, (const float4*)bounds, (const float4*)vertexes, w.counts,
            (unsigned long long*)entry_total);
        RF_TRY(launch_status());
        RF_TRY(exclusive_scan_u32(w.counts, w.counts, z.pairs, w.scan_scratch, s));
    }
    int bits = 0;
    while ((1LL << bits) <= z.tiles) bits++;  // keys 0 .. tiles (tiles = padding)
    const int passes = (entry_capacity > 1) ? (bits + 7) / 8 : 0;
    uint32_t* vals_first = (passes % 2 == 0) ? tile_entries : w.vals_tmp;
    uint32_t* vals_alt = (passes % 2 == 0) ? w.vals_tmp : tile_entries;
    if (z.pair_blocks > 0) {
        k_pair_emit_batch<<<(unsigned)z.pair_blocks, kThreads, 0, s>>>(
            frames, z.frame_count, (const float4*)bounds, (const float4*)vertexes, w.counts, entry_capacity,
            w.keys_a, vals_first);
        RF_TRY(launch_status());
    }
    k_pad_entries<<<blocks_for(entry_capacity, kThreads), kThreads, 0, s>>>(
        (const unsigned long long*)entry_total, entry_capacity, (uint32_t)z.tiles, w.keys_a, vals_first);
    RF_TRY(launch_status());
    bool in_alt = false;
    RF_TRY(radix_sort_pairs(w.keys_a, vals_first, w.keys_b, vals_alt, entry_capacity, bits, w.radix_scratch,
                            &in_alt, s));
    const uint32_t* sorted_keys = in_alt ? w.keys_b : w.keys_a;
    k_tile_offsets<<<blocks_for(z.tiles + 1, kThreads), kThreads, 0, s>>>(sorted_keys, entry_capacity, z.tiles,
                                                                          tile_offsets);
    RF_TRY(launch_status());
    // the raster's work queue: tiles by decreasing entry count
    k_tile_order_keys<<<blocks_for(z.tiles, kThreads), kThreads, 0, s>>>(tile_offsets, z.tiles, w.order_keys_b,
                                                                         w.order_vals_b);
    RF_TRY(launch_status());
    RF_TRY(radix_sort_pairs(w.order_keys_b, w.order_vals_b, w.order_keys, w.order_vals, z.tiles, kOrderKeyBits,
                            w.radix_scratch, &in_alt, s));
    return RF_OK;
}
