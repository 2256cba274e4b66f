// rf_trace.cu — the ghost-path spectral ray trace.
//
// One thread per ray (ghost path, wavelength, grid point), in the reference's ray order
// ((path * W + wavelength) * G^2 + ray). Follows realflare/api/tasks/cl/raytracing.cl:
// init_ray (178-215), the element loop of raytrace (218-359), intersect (123-175), refract
// / reflect (70-102), dispersion (107-120), fresnel (1-16) and fresnel_ar (18-59).
//
// GB300 layout:
//  * the lens elements (radius, center, height, ior, coating) and the refractive index of
//    every (wavelength, element) pair are staged in shared memory once per block; the
//    index table replaces the per-interaction Sellmeier evaluation with a lookup of the
//    same FP32 value (dispersion() depends only on the wavelength and the element);
//  * rays of a warp share path and wavelength (G^2 is a multiple of 32 for G >= 32 in
//    practice), so the element loop is warp-uniform up to rays that stop early;
//  * the grid coordinates grid_length * (x / (G - 1) - 0.5), which the reference evaluates
//    in double, are computed once on the host in double and passed as a kernel parameter;
//  * output is six coalesced float planes (pos.xy, pos_apt.xy, rrel, reflectance): the
//    fields the rasteriser reads (pos.z and dir are never read downstream).
#include <math.h>
#include <stdio.h>

#include "rf_trace_core.cuh"

namespace rf {
namespace {

__global__ void __launch_bounds__(kTraceThreads) k_trace(const rf_lens_element* __restrict__ elements,
                                                         const int2* __restrict__ paths,
                                                         const float* __restrict__ wavelengths,
                                                         const __grid_constant__ TraceParams p,
                                                         float* __restrict__ rays) {
    __shared__ SmemElement se[kMaxElements];
    __shared__ float ior_tab[kMaxTableWavelengths * kMaxElements];
    const int E = p.E;
    const long long first = (long long)blockIdx.x * kTraceThreads;
    // wavelength rows this block needs: the span of (first, last) ray indices
    const long long last = min(first + kTraceThreads, p.n_rays) - 1;
    const long long pw_first = first / p.R, pw_last = last / p.R;
    const long long span_rows = pw_last - pw_first + 1;
    const int span = (int)(span_rows < (long long)p.W ? span_rows : (long long)p.W);
    const bool table = span <= kMaxTableWavelengths;
    // dispersion is on unless coefficient 0 of element 0 is NaN (raytracing.cl:255)
    const bool disperse = !isnan(__ldg(&elements[0].coefficients[0]));
    stage_lens(elements, wavelengths, E, p.W, pw_first, span, table, disperse, se, ior_tab);
    __syncthreads();

    const long long idx = first + threadIdx.x;
    if (idx >= p.n_rays) return;
    const int ray_id = (int)(idx % p.R);
    const long long pw = idx / p.R;
    const int wl_id = (int)(pw % p.W);
    const int path_id = (int)(pw / p.W);
    const int row = (int)((pw - pw_first) % p.W);
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
    // init_ray grid point, raytracing.cl:178-215
    const int gy = (int)truncf((float)ray_id / (float)p.G);
    const int gx = ray_id - gy * p.G;
    float out[6];
    trace_ray(se, table ? ior_tab + row * E : nullptr, disperse, &elements[0].coefficients[0],
              __ldg(wavelengths + wl_id), __ldg(paths + path_id), p.grid[gx], p.grid[gy], f, out);
    const long long n = p.n_rays;
#pragma unroll
    for (int k = 0; k < 6; k++) rays[k * n + idx] = out[k];
}

// Every frame of a batch: block b traces rays_per_thread * 256 consecutive rays of the frame
// whose first trace block is the largest one <= b.
__global__ void __launch_bounds__(kTraceThreads) k_trace_batch(const rf_frame* __restrict__ frames, int F,
                                                               const rf_lens_element* __restrict__ elements_all,
                                                               const int2* __restrict__ paths_all,
                                                               const float* __restrict__ wavelengths_all,
                                                               float* __restrict__ rays_all, int rays_per_thread) {
    __shared__ SmemElement se[kMaxElements];
    __shared__ float ior_tab[kMaxTableWavelengths * kMaxElements];
    __shared__ float grid[kMaxGrid];
    __shared__ int frame_index;
    if (threadIdx.x == 0)
        frame_index = find_frame(frames, F, blockIdx.x, [](const rf_frame& fr) { return fr.trace_block; });
    __syncthreads();
    const rf_frame& fr = frames[frame_index];
    TraceFrame f;
    f.E = fr.trace.element_count;
    f.aperture = fr.trace.aperture_index;
    f.W = fr.trace.wavelength_count;
    f.G = fr.trace.grid_count;
    f.R = f.G * f.G;
    f.cmin = fr.trace.coating_min_ior;
    f.layer_n0 = fr.trace.coating_layer_ior[0];
    f.layer_n1 = fr.trace.coating_layer_ior[1];
    f.dir[0] = fr.direction_n[0];
    f.dir[1] = fr.direction_n[1];
    f.dir[2] = fr.direction_n[2];
    const long long n_rays = (long long)fr.trace.path_count * f.W * f.R;
    const rf_lens_element* elements = elements_all + fr.element_offset;
    const float* wavelengths = wavelengths_all + fr.wavelength_offset;
    const int2* paths = paths_all + fr.path_offset;
    float* rays = rays_all + 6 * fr.ray_offset;
    const long long chunk = kTraceThreads * (long long)rays_per_thread;
    const long long first = (blockIdx.x - fr.trace_block) * chunk;
    const long long last = min(first + chunk, n_rays) - 1;
    const long long pw_first = first / f.R, pw_last = last / f.R;
    const long long span_rows = pw_last - pw_first + 1;
    const int span = (int)(span_rows < (long long)f.W ? span_rows : (long long)f.W);
    const bool table = span <= kMaxTableWavelengths;
    const bool disperse = !isnan(__ldg(&elements[0].coefficients[0]));
    stage_lens(elements, wavelengths, f.E, f.W, pw_first, span, table, disperse, se, ior_tab);
    // grid_length * (x / (G - 1) - 0.5), in double as in the reference (and rf_trace's host table)
    for (int i = threadIdx.x; i < f.G; i += kTraceThreads) {
        const float t = (float)i / (float)(f.G - 1);
        grid[i] = (float)((double)fr.trace.grid_length * ((double)t - 0.5));
    }
    __syncthreads();
    for (int r = 0; r < rays_per_thread; r++) {
        const long long idx = first + r * kTraceThreads + threadIdx.x;
        if (idx > last) break;
        const int ray_id = (int)(idx % f.R);
        const long long pw = idx / f.R;
        const int wl_id = (int)(pw % f.W);
        const int path_id = (int)(pw / f.W);
        const int row = (int)((pw - pw_first) % f.W);
        const int gy = (int)truncf((float)ray_id / (float)f.G);
        const int gx = ray_id - gy * f.G;
        float out[6];
        trace_ray(se, table ? ior_tab + row * f.E : nullptr, disperse, &elements[0].coefficients[0],
                  __ldg(wavelengths + wl_id), __ldg(paths + path_id), grid[gx], grid[gy], f, out);
#pragma unroll
        for (int k = 0; k < 6; k++) rays[k * n_rays + idx] = out[k];
    }
}

}  // namespace
}  // namespace rf

extern "C" int rf_trace(const rf_lens_element* elements, const int32_t* paths, const float* wavelengths,
                        const rf_trace_args* args, float* rays, void* stream) {
    using namespace rf;
    if (!elements || !paths || !wavelengths || !args || !rays) return RF_ERR_INVALID_ARG;
    const rf_trace_args& a = *args;
    if (a.element_count < 2 || a.element_count > kMaxElements || a.path_count < 0 || a.wavelength_count < 1 ||
        a.grid_count < 2 || a.grid_count > kMaxGrid || a.aperture_index < 0)
        return RF_ERR_INVALID_ARG;
    TraceParams p;
    if (!trace_params(a, p)) return RF_ERR_INVALID_ARG;
    if (p.n_rays == 0) return RF_OK;
    k_trace<<<blocks_for(p.n_rays, kTraceThreads), kTraceThreads, 0, (cudaStream_t)stream>>>(
        elements, (const int2*)paths, wavelengths, p, rays);
    return launch_status();
}

extern "C" int rf_trace_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const rf_lens_element* elements,
                              const int32_t* paths, const float* wavelengths, float* rays, void* stream) {
    using namespace rf;
    if (!frames || !sizes || !elements || !paths || !wavelengths || !rays) return RF_ERR_INVALID_ARG;
    if (sizes->trace_blocks == 0) return RF_OK;
    if (sizes->trace_blocks > 0x7fffffffLL) return RF_ERR_NOT_SUPPORTED;
    k_trace_batch<<<(unsigned)sizes->trace_blocks, kTraceThreads, 0, (cudaStream_t)stream>>>(
        frames, sizes->frame_count, elements, (const int2*)paths, wavelengths, rays, sizes->rays_per_thread);
    return launch_status();
}
