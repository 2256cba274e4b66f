// rf_quad.cu — quad setup (prim_shader) and vertex setup (vertex_shader).
//
// Both follow realflare/api/tasks/cl/rasterizing.cl (prim_shader 233-320, vertex_shader
// 322-386, quad_vertexes 218-230, quad_neighbors 196-216). This file is compiled without
// fused multiply-add contraction, so for identical rays the bounds, intensities and
// vertex positions equal the oracle's bit for bit. Both kernels are memory-bound: one
// thread per primitive (reading its 4 corner rays per wavelength) and one thread per ray
// (coalesced plane reads, one 32-byte vertex store).
#include "rf_common.cuh"

namespace rf {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float edge_f(float ax, float ay, float bx, float by, float cx, float cy) {
    return (ax - bx) * (cy - ay) - (ay - by) * (cx - ax);
}

// Primitive pq = path * Q + quad of one frame.
__device__ __forceinline__ void quad_setup_one(const float* __restrict__ rays, int P, int W, int G, long long n_rays,
                                               float area_orig, float min_area, float4* __restrict__ bounds,
                                               float* __restrict__ inten, long long pq) {
    const int Q = (G - 1) * (G - 1), R = G * G;
    if (pq >= (long long)P * Q) return;
    const int path = (int)(pq / Q), quad = (int)(pq % Q);
    const int row = quad / (G - 1), col = quad % (G - 1);
    int v[4];
    v[0] = row * G + col;
    v[1] = v[0] + 1;
    v[2] = v[1] + G;
    v[3] = v[0] + G;
    const float* pos_x = rays;
    const float* pos_y = rays + n_rays;
    const float* rrel = rays + 4 * n_rays;
    const float* refl = rays + 5 * n_rays;
    float bx0 = INFINITY, by0 = INFINITY, bx1 = -INFINITY, by1 = -INFINITY;
    int invalid_rrel = 0;
    bool culled = false;
    for (int w = 0; w < W; w++) {
        const size_t prim_index = (size_t)pq * W + w;
        if (culled) {
            inten[prim_index] = 0.0f;  // the reference leaves these entries stale
            continue;
        }
        const size_t off = ((size_t)path * W + w) * R;
        float px[4], py[4], rr[4];
        int valid = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            rr[i] = __ldg(rrel + off + v[i]);
            float x = __ldg(pos_x + off + v[i]), y = __ldg(pos_y + off + v[i]);
            if (!isnan(__ldg(refl + off + v[i]))) {
                // compaction into the first free slot (valid <= i)
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (k == valid) {
                        px[k] = x;
                        py[k] = y;
                    }
                valid++;
            }
        }
        float area;
        if (valid == 4) {
            float a0 = edge_f(px[0], py[0], px[1], py[1], px[2], py[2]);
            float a1 = edge_f(px[0], py[0], px[2], py[2], px[3], py[3]);
            area = fabsf(a0 + a1) / 2.0f;
        } else if (valid == 3) {
            area = fabsf(edge_f(px[0], py[0], px[1], py[1], px[2], py[2]));
            px[3] = px[2];
            py[3] = py[2];
            rr[3] = rr[2];
        } else {
            culled = true;
            inten[prim_index] = 0.0f;
            continue;
        }
        if (rr[0] > 1.0f && rr[1] > 1.0f && rr[2] > 1.0f && rr[3] > 1.0f) invalid_rrel++;
        float area_actual = fmaxf(area, min_area);
        inten[prim_index] = area_actual > 0.0f ? area_orig / area_actual : 0.0f;
        bx0 = fminf(bx0, fminf(fminf(px[0], px[1]), fminf(px[2], px[3])));
        by0 = fminf(by0, fminf(fminf(py[0], py[1]), fminf(py[2], py[3])));
        bx1 = fmaxf(bx1, fmaxf(fmaxf(px[0], px[1]), fmaxf(px[2], px[3])));
        by1 = fmaxf(by1, fmaxf(fmaxf(py[0], py[1]), fmaxf(py[2], py[3])));
    }
    if (invalid_rrel == W) culled = true;
    bounds[pq] = make_float4(culled ? __int_as_float(0x7fffffff) : bx0, by0, bx1, by1);
}

__global__ void __launch_bounds__(kThreads) k_quad_setup(const float* __restrict__ rays, int P, int W, int G,
                                                         long long n_rays, float area_orig, float min_area,
                                                         float4* __restrict__ bounds, float* __restrict__ inten) {
    quad_setup_one(rays, P, W, G, n_rays, area_orig, min_area, bounds, inten,
                   (long long)blockIdx.x * kThreads + threadIdx.x);
}

// Vertex i (ray-plane order; i == n_rays is the trailing zero vertex) of one frame.
__device__ __forceinline__ void vertex_one(const float* __restrict__ rays, const float* __restrict__ inten, int P,
                                           int W, int G, long long n_rays, float st, float half_w, float half_h,
                                           float4* __restrict__ vertexes, long long i) {
    const int Q = (G - 1) * (G - 1), R = G * G;
    if (i > n_rays) return;
    if (i == n_rays) {  // the zero vertex after the last one
        vertexes[2 * n_rays] = make_float4(0.f, 0.f, 0.f, 0.f);
        vertexes[2 * n_rays + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const int ray_id = (int)(i % R);
    const long long pw = i / R;
    const int w = (int)(pw % W);
    const int path = (int)(pw / W);
    const long long vi = ((long long)path * R + ray_id) * W + w;  // the reference's order
    const float refl = __ldg(rays + 5 * n_rays + i);
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = make_float4(0.f, refl, 0.f, 0.f);
    if (!isnan(refl)) {
        const int x = ray_id % G, y = ray_id / G;
        int nb[4];
        nb[0] = (y - 1) * (G - 1) + (x - 1);
        nb[1] = nb[0] + 1;
        nb[2] = y * (G - 1) + (x - 1);
        nb[3] = nb[2] + 1;
        float s = 0.0f;
        int count = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (nb[k] < 0 || nb[k] >= Q) continue;
            float v = __ldg(inten + ((size_t)path * Q + nb[k]) * W + w);
            if (v > 0.0f) {
                s += v;
                ++count;
            }
        }
        s /= (float)(count > 1 ? count : 1);
        a.x = __fadd_rn(__fmul_rn(__ldg(rays + i), st), half_w);
        a.y = __fadd_rn(__fmul_rn(__ldg(rays + n_rays + i), st), half_h);
        a.z = __ldg(rays + 2 * n_rays + i);
        a.w = __ldg(rays + 3 * n_rays + i);
        b.x = __ldg(rays + 4 * n_rays + i);
        b.z = s;
    }
    vertexes[2 * vi] = a;
    vertexes[2 * vi + 1] = b;
}

__global__ void __launch_bounds__(kThreads) k_vertex(const float* __restrict__ rays, const float* __restrict__ inten,
                                                     int P, int W, int G, long long n_rays, float st, float half_w,
                                                     float half_h, float4* __restrict__ vertexes) {
    vertex_one(rays, inten, P, W, G, n_rays, st, half_w, half_h, vertexes,
               (long long)blockIdx.x * kThreads + threadIdx.x);
}

// ---------------------------------------------------------------- adjoints
// Vertex i (ray-plane order): the aperture position, rrel and reflectance gradients pass to
// the ray unchanged; the intensity gradient goes to the neighbour quads whose positive
// intensities the vertex averaged (vertex_shader, rasterizing.cl:362-369).
__global__ void __launch_bounds__(kThreads) k_vertex_backward(const float* __restrict__ rays,
                                                              const float* __restrict__ inten, int W, int G,
                                                              long long n_rays, const float* __restrict__ grad_vtx,
                                                              float* __restrict__ grad_rays,
                                                              float* __restrict__ grad_inten) {
    const int Q = (G - 1) * (G - 1), R = G * G;
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n_rays) return;
    const int ray_id = (int)(i % R);
    const long long pw = i / R;
    const int w = (int)(pw % W);
    const long long path = pw / W;
    const long long vi = (path * R + ray_id) * W + w;
    const float refl = __ldg(rays + 5 * n_rays + i);
    const float* g = grad_vtx + 8 * vi;
    const bool valid = !isnan(refl);
    grad_rays[2 * n_rays + i] = valid ? g[2] : 0.0f;
    grad_rays[3 * n_rays + i] = valid ? g[3] : 0.0f;
    grad_rays[4 * n_rays + i] = valid ? g[4] : 0.0f;
    grad_rays[5 * n_rays + i] = valid ? g[5] : 0.0f;
    const float gi = g[6];
    if (!valid || gi == 0.0f) return;
    const int x = ray_id % G, y = ray_id / G;
    int nb[4];
    nb[0] = (y - 1) * (G - 1) + (x - 1);
    nb[1] = nb[0] + 1;
    nb[2] = y * (G - 1) + (x - 1);
    nb[3] = nb[2] + 1;
    int count = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (nb[k] >= 0 && nb[k] < Q && __ldg(inten + ((size_t)path * Q + nb[k]) * W + w) > 0.0f) ++count;
    const float share = gi / (float)(count > 1 ? count : 1);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (nb[k] < 0 || nb[k] >= Q) continue;
        const size_t qi = ((size_t)path * Q + nb[k]) * W + w;
        if (__ldg(inten + qi) > 0.0f) atomicAdd(grad_inten + qi, share);
    }
}

// d edge_f(a, b, c) / d(ax, ay, bx, by, cx, cy), scaled by s and added to g[2 * slot]
__device__ __forceinline__ void edge_grad(const float* x, const float* y, int a, int b, int c, float s, float* gx,
                                          float* gy) {
    gx[a] += s * (y[c] - y[b]);
    gy[a] += s * (x[b] - x[c]);
    gx[b] += s * (y[a] - y[c]);
    gy[b] += s * (x[c] - x[a]);
    gx[c] += s * (y[b] - y[a]);
    gy[c] += s * (x[a] - x[b]);
}

// Primitive pq: intensity = area_orig / max(area, min_area) (prim_shader,
// rasterizing.cl:271-301) passes its gradient to the sensor positions of the corner rays.
__global__ void __launch_bounds__(kThreads) k_quad_setup_backward(const float* __restrict__ rays, int P, int W, int G,
                                                                  long long n_rays, float area_orig, float min_area,
                                                                  const float* __restrict__ grad_inten,
                                                                  float* __restrict__ grad_rays) {
    const int Q = (G - 1) * (G - 1), R = G * G;
    const long long pq = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (pq >= (long long)P * Q) return;
    const int path = (int)(pq / Q), quad = (int)(pq % Q);
    const int row = quad / (G - 1), col = quad % (G - 1);
    int v[4];
    v[0] = row * G + col;
    v[1] = v[0] + 1;
    v[2] = v[1] + G;
    v[3] = v[0] + G;
    for (int w = 0; w < W; w++) {
        const size_t off = ((size_t)path * W + w) * R;
        float px[4], py[4];
        int src[4];
        int valid = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if (!isnan(__ldg(rays + 5 * n_rays + off + v[i]))) {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (k == valid) {
                        px[k] = __ldg(rays + off + v[i]);
                        py[k] = __ldg(rays + n_rays + off + v[i]);
                        src[k] = v[i];
                    }
                valid++;
            }
        }
        if (valid < 3) break;  // the forward culls this and every later wavelength
        const float g = __ldg(grad_inten + (size_t)pq * W + w);
        if (g == 0.0f) continue;
        float area, sa;
        float gx[4] = {0.f, 0.f, 0.f, 0.f}, gy[4] = {0.f, 0.f, 0.f, 0.f};
        if (valid == 4) {
            const float a0 = edge_f(px[0], py[0], px[1], py[1], px[2], py[2]);
            const float a1 = edge_f(px[0], py[0], px[2], py[2], px[3], py[3]);
            area = fabsf(a0 + a1) / 2.0f;
            sa = (a0 + a1 >= 0.0f ? 0.5f : -0.5f);
        } else {
            const float a0 = edge_f(px[0], py[0], px[1], py[1], px[2], py[2]);
            area = fabsf(a0);
            sa = a0 >= 0.0f ? 1.0f : -1.0f;
        }
        if (!(area > min_area)) continue;  // max(area, min_area) holds min_area: no gradient
        const float g_area = -area_orig / (area * area) * g;
        edge_grad(px, py, 0, 1, 2, g_area * sa, gx, gy);
        if (valid == 4) edge_grad(px, py, 0, 2, 3, g_area * sa, gx, gy);
        for (int k = 0; k < valid; k++) {
            atomicAdd(grad_rays + off + src[k], gx[k]);
            atomicAdd(grad_rays + n_rays + off + src[k], gy[k]);
        }
    }
}

// Batched forms: block b works for the frame whose first block of the stage is the largest
// one <= b.
__global__ void __launch_bounds__(kThreads) k_quad_setup_batch(const rf_frame* __restrict__ frames, int F,
                                                               const float* __restrict__ rays_all,
                                                               float4* __restrict__ bounds_all,
                                                               float* __restrict__ inten_all) {
    __shared__ int frame_index;
    if (threadIdx.x == 0)
        frame_index = find_frame(frames, F, blockIdx.x, [](const rf_frame& fr) { return fr.quad_block; });
    __syncthreads();
    const rf_frame& fr = frames[frame_index];
    const int P = fr.trace.path_count, W = fr.trace.wavelength_count, G = fr.trace.grid_count;
    const long long n_rays = (long long)P * W * G * G;
    quad_setup_one(rays_all + 6 * fr.ray_offset, P, W, G, n_rays, fr.area_orig, fr.min_area,
                   bounds_all + fr.prim_offset, inten_all + fr.inten_offset,
                   (long long)(blockIdx.x - fr.quad_block) * kThreads + threadIdx.x);
}

__global__ void __launch_bounds__(kThreads) k_vertex_batch(const rf_frame* __restrict__ frames, int F,
                                                           const float* __restrict__ rays_all,
                                                           const float* __restrict__ inten_all,
                                                           float4* __restrict__ vertexes_all) {
    __shared__ int frame_index;
    if (threadIdx.x == 0)
        frame_index = find_frame(frames, F, blockIdx.x, [](const rf_frame& fr) { return fr.vertex_block; });
    __syncthreads();
    const rf_frame& fr = frames[frame_index];
    const int P = fr.trace.path_count, W = fr.trace.wavelength_count, G = fr.trace.grid_count;
    const long long n_rays = (long long)P * W * G * G;
    const float half_w = (float)fr.raster.width / 2.0f, half_h = (float)fr.raster.height / 2.0f;
    vertex_one(rays_all + 6 * fr.ray_offset, inten_all + fr.inten_offset, P, W, G, n_rays,
               fr.raster.screen_transform, half_w, half_h, vertexes_all + 2 * fr.vertex_offset,
               (long long)(blockIdx.x - fr.vertex_block) * kThreads + threadIdx.x);
}

}  // namespace
}  // namespace rf

extern "C" int rf_quad_setup(const float* rays, int32_t path_count, int32_t wavelength_count, int32_t grid_count,
                             float area_orig, float min_area, float* bounds, float* intensities, void* stream) {
    using namespace rf;
    if (!rays || !bounds || !intensities || path_count < 0 || wavelength_count < 1 || grid_count < 2)
        return RF_ERR_INVALID_ARG;
    if (!aligned16(bounds)) return RF_ERR_INVALID_ARG;
    const long long Q = (long long)(grid_count - 1) * (grid_count - 1);
    const long long n = (long long)path_count * Q;
    if (n == 0) return RF_OK;
    const long long n_rays = (long long)path_count * wavelength_count * grid_count * grid_count;
    k_quad_setup<<<blocks_for(n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        rays, path_count, wavelength_count, grid_count, n_rays, area_orig, min_area, (float4*)bounds, intensities);
    return launch_status();
}

extern "C" int rf_vertex(const float* rays, const float* intensities, int32_t path_count, int32_t wavelength_count,
                         int32_t grid_count, float screen_transform, int32_t width, int32_t height, float* vertexes,
                         void* stream) {
    using namespace rf;
    if (!rays || !intensities || !vertexes || path_count < 0 || wavelength_count < 1 || grid_count < 2 ||
        width < 1 || height < 1)
        return RF_ERR_INVALID_ARG;
    if (!aligned16(vertexes)) return RF_ERR_INVALID_ARG;
    const long long n_rays = (long long)path_count * wavelength_count * grid_count * grid_count;
    // convert_float2(resolution) / 2 (rasterizing.cl:374)
    const float half_w = (float)width / 2.0f, half_h = (float)height / 2.0f;
    k_vertex<<<blocks_for(n_rays + 1, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        rays, intensities, path_count, wavelength_count, grid_count, n_rays, screen_transform, half_w, half_h,
        (float4*)vertexes);
    return launch_status();
}

extern "C" int rf_quad_setup_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const float* rays,
                                   float* bounds, float* intensities, void* stream) {
    using namespace rf;
    if (!frames || !sizes || !rays || !bounds || !intensities) return RF_ERR_INVALID_ARG;
    if (!aligned16(bounds)) return RF_ERR_INVALID_ARG;
    if (sizes->quad_blocks == 0) return RF_OK;
    if (sizes->quad_blocks > 0x7fffffffLL) return RF_ERR_NOT_SUPPORTED;
    k_quad_setup_batch<<<(unsigned)sizes->quad_blocks, kThreads, 0, (cudaStream_t)stream>>>(
        frames, sizes->frame_count, rays, (float4*)bounds, intensities);
    return launch_status();
}

extern "C" int rf_vertex_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const float* rays,
                               const float* intensities, float* vertexes, void* stream) {
    using namespace rf;
    if (!frames || !sizes || !rays || !intensities || !vertexes) return RF_ERR_INVALID_ARG;
    if (!aligned16(vertexes)) return RF_ERR_INVALID_ARG;
    if (sizes->vertex_blocks == 0) return RF_OK;
    if (sizes->vertex_blocks > 0x7fffffffLL) return RF_ERR_NOT_SUPPORTED;
    k_vertex_batch<<<(unsigned)sizes->vertex_blocks, kThreads, 0, (cudaStream_t)stream>>>(
        frames, sizes->frame_count, rays, intensities, (float4*)vertexes);
    return launch_status();
}

extern "C" int rf_vertex_backward(const float* rays, const float* intensities, int32_t path_count,
                                  int32_t wavelength_count, int32_t grid_count, const float* grad_vertexes,
                                  float* grad_rays, float* grad_intensities, void* stream) {
    using namespace rf;
    if (!rays || !intensities || !grad_vertexes || !grad_rays || !grad_intensities || path_count < 0 ||
        wavelength_count < 1 || grid_count < 2)
        return RF_ERR_INVALID_ARG;
    const long long n_rays = (long long)path_count * wavelength_count * grid_count * grid_count;
    const long long n_inten = (long long)path_count * (grid_count - 1) * (grid_count - 1) * wavelength_count;
    cudaStream_t s = (cudaStream_t)stream;
    RF_TRY(cuda_status(cudaMemsetAsync(grad_intensities, 0, sizeof(float) * (size_t)n_inten, s)));
    RF_TRY(cuda_status(cudaMemsetAsync(grad_rays, 0, sizeof(float) * 2 * (size_t)n_rays, s)));
    if (n_rays == 0) return RF_OK;
    k_vertex_backward<<<blocks_for(n_rays, kThreads), kThreads, 0, s>>>(
        rays, intensities, wavelength_count, grid_count, n_rays, grad_vertexes, grad_rays, grad_intensities);
    return launch_status();
}

extern "C" int rf_quad_setup_backward(const float* rays, int32_t path_count, int32_t wavelength_count,
                                      int32_t grid_count, float area_orig, float min_area,
                                      const float* grad_intensities, float* grad_rays, void* stream) {
    using namespace rf;
    if (!rays || !grad_intensities || !grad_rays || path_count < 0 || wavelength_count < 1 || grid_count < 2)
        return RF_ERR_INVALID_ARG;
    const long long n = (long long)path_count * (grid_count - 1) * (grid_count - 1);
    if (n == 0) return RF_OK;
    const long long n_rays = (long long)path_count * wavelength_count * grid_count * grid_count;
    k_quad_setup_backward<<<blocks_for(n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        rays, path_count, wavelength_count, grid_count, n_rays, area_orig, min_area, grad_intensities, grad_rays);
    return launch_status();
}
