// rf_batch.cu — planning of batched frames (host code).
//
// rf_batch_plan validates every frame the way the single-frame entry points do and lays
// the frames out one after another in every buffer and in every stage's block range, so
// that each batched kernel finds its frame from its block index (find_frame) and then
// runs the single-frame code on the frame's slices.
#include <math.h>

#include "rf_common.cuh"

namespace rf {
namespace {

constexpr int kThreads = 256;       // block size of every batched stage
constexpr int kMaxElements = 128;   // rf_trace.cu
constexpr int kMaxGrid = 2048;      // rf_trace.cu
constexpr int kMaxSub = 64;         // records per raster batch (rf_raster.cu)

long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

bool valid_frame(const rf_frame& f, int tile) {
    const rf_trace_args& t = f.trace;
    const rf_raster_args& r = f.raster;
    if (t.element_count < 2 || t.element_count > kMaxElements || t.aperture_index < 0 || t.path_count < 0 ||
        t.wavelength_count < 1 || t.grid_count < 2 || t.grid_count > kMaxGrid)
        return false;
    if (r.path_count != t.path_count || r.wavelength_count != t.wavelength_count || r.grid_count != t.grid_count)
        return false;
    if (r.width < 1 || r.height < 1 || r.wavelength_sub_count < 1 || r.wavelength_sub_count > kMaxSub ||
        r.ghost_width < 1 || r.ghost_height < 1 || r.bin_size < 1 || r.bin_size % tile != 0)
        return false;
    if (r.sub_steps != 1 && r.sub_steps != 2 && r.sub_steps != 4 && r.sub_steps != 8) return false;
    const int maxW = t.wavelength_count - 1 > 1 ? t.wavelength_count - 1 : 1;
    if (maxW * r.wavelength_sub_count > 4096) return false;
    if (f.element_offset < 0 || f.path_offset < 0 || f.wavelength_offset < 0 || f.ghost_offset < 0) return false;
    return true;
}

}  // namespace
}  // namespace rf

extern "C" int rf_batch_plan(rf_frame* frames, int32_t frame_count, int32_t tile_size, int32_t rays_per_thread,
                             rf_batch_sizes* sizes) {
    using namespace rf;
    if (!frames || !sizes || frame_count < 1) return RF_ERR_INVALID_ARG;
    if (tile_size != 16 && tile_size != 32) return RF_ERR_NOT_SUPPORTED;
    if (rays_per_thread != 1 && rays_per_thread != 2 && rays_per_thread != 4) return RF_ERR_NOT_SUPPORTED;
    rf_batch_sizes z = {};
    z.frame_count = frame_count;
    z.tile_size = tile_size;
    z.rays_per_thread = rays_per_thread;
    long long tiles = 0;
    for (int i = 0; i < frame_count; i++) {
        rf_frame& f = frames[i];
        if (!valid_frame(f, tile_size)) {
            set_error_text("rf_batch_plan: a frame has settings outside the supported range");
            return RF_ERR_INVALID_ARG;
        }
        f.raster.tile_size = tile_size;
        const long long P = f.trace.path_count, W = f.trace.wavelength_count, G = f.trace.grid_count;
        const long long n_rays = P * W * G * G, Q = (G - 1) * (G - 1);
        const long long maxW = W - 1 > 1 ? W - 1 : 1;
        f.ray_offset = z.rays;
        f.prim_offset = z.prims;
        f.inten_offset = z.intensities;
        f.vertex_offset = z.vertices;
        f.pair_offset = z.pairs;
        f.trace_block = z.trace_blocks;
        f.quad_block = z.quad_blocks;
        f.vertex_block = z.vertex_blocks;
        f.pair_block = z.pair_blocks;
        f.image_offset = z.image_pixels;
        z.rays += n_rays;
        z.prims += P * Q;
        z.intensities += P * Q * W;
        z.vertices += n_rays + 1;
        z.pairs += P * Q * maxW;
        z.trace_blocks += ceil_div(n_rays, (long long)kThreads * rays_per_thread);
        z.quad_blocks += ceil_div(P * Q, kThreads);
        z.vertex_blocks += ceil_div(n_rays + 1, kThreads);
        z.pair_blocks += ceil_div(P * Q * maxW, kThreads);
        z.image_pixels += (long long)f.raster.width * f.raster.height;
        const long long ghost_end = f.ghost_offset + (long long)f.raster.ghost_width * f.raster.ghost_height;
        if (ghost_end > z.ghost_floats) z.ghost_floats = ghost_end;
        const int ntx = (f.raster.width + tile_size - 1) / tile_size, nty = (f.raster.height + tile_size - 1) / tile_size;
        f.tile_offset = (int32_t)tiles;
        f.tile_count = ntx * nty;
        tiles += (long long)ntx * nty;
        const int colors = (int)maxW * f.raster.wavelength_sub_count;
        if (colors > z.max_colors) z.max_colors = colors;
        if (f.raster.wavelength_sub_count > z.max_sub) z.max_sub = f.raster.wavelength_sub_count;
        if (f.raster.sub_steps > z.max_sub_steps) z.max_sub_steps = f.raster.sub_steps;
        // normalize(direction.xyz * -1) in FP32, the value rf_trace computes (this file is
        // compiled without floating-point contraction too)
        const float vx = -f.trace.direction[0], vy = -f.trace.direction[1], vz = -f.trace.direction[2];
        const float dd = vx * vx + vy * vy + vz * vz;
        const float inv = 1.0f / sqrtf(dd);
        f.direction_n[0] = vx * inv;
        f.direction_n[1] = vy * inv;
        f.direction_n[2] = vz * inv;
        f.pad1 = 0;
    }
    z.ghost_textures = 1;
    for (int i = 0; i < frame_count; i++) z.ghost_textures = z.ghost_textures && frames[i].ghost_texture != 0;
    if (tiles > (1LL << 30) || z.trace_blocks > 0x7fffffffLL || z.vertex_blocks > 0x7fffffffLL ||
        z.pair_blocks > 0x7fffffffLL || z.quad_blocks > 0x7fffffffLL) {
        set_error_text("rf_batch_plan: the batch exceeds 2^31 blocks or 2^30 tiles in one stage");
        return RF_ERR_NOT_SUPPORTED;
    }
    z.tiles = (int32_t)tiles;
    *sizes = z;
    return RF_OK;
}
