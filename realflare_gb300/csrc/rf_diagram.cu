// rf_diagram.cu — the lens diagram: the trace with every surface hit stored, and the
// cross-section image drawn from the lens and those hits.
//
// rf_trace_intersections follows the trace kernel built with STORE_INTERSECTIONS
// (realflare/api/tasks/cl/raytracing.cl:218-359 with 229-271): the shared per-ray trace
// (rf_trace_core.cuh) with a recorder that stores each hit, so the rays equal rf_trace's.
// rf_diagram fuses the kernels lenses and intersections of
// realflare/api/tasks/cl/diagram.cl:21-138 into one pass per pixel. This unit is compiled
// without floating-point contraction (like the trace), so the drawing tests evaluate the
// products and sums the kernels write in FP32, operation by operation.
#include "rf_trace_core.cuh"

namespace rf {
namespace {

constexpr int kDiagramBlock = 16;  // 16 x 16 pixels per block

// Stores hit k of one ray at out[k] (k < count): the reference's Intersection record.
struct IntersectionRecorder {
    rf_intersection* out;
    int count;
    __device__ __forceinline__ void step(int, float, float, float, float, float, float) {}
    __device__ __forceinline__ void hit(int k, const Hit& h, float dx, float dy, float dz, bool flat) {
        if (k >= count) return;
        rf_intersection r;
        r.pos[0] = h.px;
        r.pos[1] = h.py;
        r.pos[2] = h.pz;
        r.normal[0] = h.nx;
        r.normal[1] = h.ny;
        r.normal[2] = h.nz;
        // intersect's incidence angle, raytracing.cl:167 (0 on flat elements, :140)
        r.incident = flat ? 0.0f : incident_angle(dx, dy, dz, h);
        r.hit = 1;
        out[k] = r;
    }
    __device__ __forceinline__ void rrel(float, float) {}
    __device__ __forceinline__ void reflect() {}
};

__global__ void __launch_bounds__(kTraceThreads) k_trace_intersections(const rf_lens_element* __restrict__ elements,
                                                                       const int2* __restrict__ paths,
                                                                       const float* __restrict__ wavelengths,
                                                                       const __grid_constant__ TraceParams p,
                                                                       float* __restrict__ rays,
                                                                       rf_intersection* __restrict__ inter,
                                                                       int count) {
    __shared__ SmemElement se[kMaxElements];
    const bool disperse = !isnan(__ldg(&elements[0].coefficients[0]));
    stage_lens(elements, wavelengths, p.E, p.W, 0, 0, false, disperse, se, nullptr);
    __syncthreads();
    const long long idx = (long long)blockIdx.x * kTraceThreads + threadIdx.x;
    if (idx >= p.n_rays) return;
    const int ray_id = (int)(idx % p.R);
    const long long pw = idx / p.R;
    const int wl_id = (int)(pw % p.W);
    const int path_id = (int)(pw / p.W);
    TraceFrame f;
    f.E = p.E;
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
    const int gy = (int)truncf((float)ray_id / (float)p.G);
    const int gx = ray_id - gy * p.G;
    IntersectionRecorder rec{inter + idx * count, count};
    float out[6];
    trace_ray_rec(se, nullptr, disperse, &elements[0].coefficients[0], __ldg(wavelengths + wl_id),
                  __ldg(paths + path_id), p.grid[gx], p.grid[gy], f, out, rec);
    const long long n = p.n_rays;
#pragma unroll
    for (int k = 0; k < 6; k++) rays[k * n + idx] = out[k];
}

// is_line (diagram.cl:1-19): pixel pos strictly between the segment's ends along it and
// within width / 2 of its line.
__device__ __forceinline__ bool is_line(float posx, float posy, float p0x, float p0y, float p1x, float p1y,
                                        float width) {
    const float vx = p1x - p0x, vy = p1y - p0y;
    const float ax = posx - p0x, ay = posy - p0y;
    const float bx = posx - p1x, by = posy - p1y;
    const bool between = (vx * ax + vy * ay) > 0.0f && (vx * bx + vy * by) < 0.0f;
    const float d = fabsf(vx * ay - ax * vy) / sqrtf(vx * vx + vy * vy);
    return between && d <= width / 2.0f;
}

struct DiagramArgs {
    int E, aperture, width, height, rays, count;
    float scale;
};

__global__ void __launch_bounds__(kDiagramBlock* kDiagramBlock) k_diagram(const rf_lens_element* __restrict__ elements,
                                                                           const rf_intersection* __restrict__ inter,
                                                                           DiagramArgs a, float4* __restrict__ image) {
    const int px = blockIdx.x * kDiagramBlock + threadIdx.x, py = blockIdx.y * kDiagramBlock + threadIdx.y;
    if (px >= a.width || py >= a.height) return;
    // lenses (diagram.cl:21-67)
    const float x = (float)px, y = (float)(a.height / 2 - py);
    float4 rgba = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if ((int)y == 0) rgba.x = 1.0f;  // the optical axis
    for (int i = 0; i < a.E; i++) {
        const float r = __ldg(&elements[i].radius) * a.scale;
        const float h = __ldg(&elements[i].height) * a.scale;
        const float c = __ldg(&elements[i].center) * a.scale;
        if (r == 0.0f && fabsf(y) < h && (int)x == (int)c) {
            // flat elements: the aperture and the sensor green, others blue
            if (i == a.aperture || i == a.E - 1)
                rgba.y = 1.0f;
            else
                rgba.z = 1.0f;
            break;
        }
        // pow(x - c, 2) + pow(y, 2), the squares as products
        const float ex = x - c;
        const float r_circle = sqrtf(ex * ex + y * y);
        const bool draw_half = (r > 0.0f) ? (x < c) : (x > c);
        if (draw_half && (int)fabsf(r) == (int)r_circle && fabsf(y) < h) rgba.z = 1.0f;
    }
    // intersections (diagram.cl:70-138): each ray's segments between consecutive hits and
    // each hit's normal, in the (-z, -y) plane at scale pixels per mm
    if (inter) {
        const long long total = (long long)a.rays * a.count;
        for (int ray = 0; ray < a.rays; ray++) {
            for (int k = 0; k < a.count; k++) {
                const long long i1 = (long long)ray * a.count + k;
                // the record after a ray's last one is the next ray's first (none after the last ray)
                if (i1 + 1 >= total || !__ldg(&inter[i1 + 1].hit)) break;
                const rf_intersection* s = inter + i1;
                const rf_intersection* t = inter + i1 + 1;
                const float p0x = (__ldg(&s->pos[2]) * a.scale) * -1.0f, p0y = (__ldg(&s->pos[1]) * a.scale) * -1.0f;
                const float p1x = (__ldg(&t->pos[2]) * a.scale) * -1.0f, p1y = (__ldg(&t->pos[1]) * a.scale) * -1.0f;
                const float nx = __ldg(&s->normal[2]) * a.scale, ny = __ldg(&s->normal[1]) * a.scale;
                // normal_length = 1
                if (is_line(x, y, p0x, p0y, p0x - nx * 1.0f, p0y - ny * 1.0f, 1.0f))
                    rgba = make_float4(0.25f, 0.0f, 0.0f, 0.0f);
                if (p1x == 0.0f) break;
                if (is_line(x, y, p0x, p0y, p1x, p1y, 1.0f)) {
                    rgba.x += 0.25f;
                    rgba.y += 0.25f;
                    rgba.z += 0.25f;
                }
            }
        }
    }
    image[(size_t)py * a.width + px] = rgba;
}

}  // namespace
}  // namespace rf

extern "C" int rf_trace_intersections(const rf_lens_element* elements, const int32_t* paths, const float* wavelengths,
                                      const rf_trace_args* args, float* rays, rf_intersection* intersections,
                                      int32_t intersection_count, void* stream) {
    using namespace rf;
    if (!elements || !paths || !wavelengths || !args || !rays || !intersections || intersection_count < 1)
        return RF_ERR_INVALID_ARG;
    const rf_trace_args& a = *args;
    if (a.element_count < 2 || a.element_count > kMaxElements || a.path_count < 0 || a.wavelength_count < 1 ||
        a.grid_count < 2 || a.grid_count > kMaxGrid || a.aperture_index < 0)
        return RF_ERR_INVALID_ARG;
    TraceParams p;
    if (!trace_params(a, p)) return RF_ERR_INVALID_ARG;
    if (p.n_rays == 0) return RF_OK;
    cudaStream_t s = (cudaStream_t)stream;
    RF_TRY(cuda_status(
        cudaMemsetAsync(intersections, 0, sizeof(rf_intersection) * (size_t)p.n_rays * intersection_count, s)));
    k_trace_intersections<<<blocks_for(p.n_rays, kTraceThreads), kTraceThreads, 0, s>>>(
        elements, (const int2*)paths, wavelengths, p, rays, intersections, intersection_count);
    return launch_status();
}

extern "C" int rf_diagram(const rf_lens_element* elements, int32_t element_count, int32_t aperture_index, float scale,
                          const rf_intersection* intersections, int32_t ray_count, int32_t intersection_count,
                          int32_t width, int32_t height, float* image, void* stream) {
    using namespace rf;
    if (!elements || !image || element_count < 0 || width < 1 || height < 1 || ray_count < 0 ||
        intersection_count < 0)
        return RF_ERR_INVALID_ARG;
    if (!aligned16(image)) return RF_ERR_INVALID_ARG;
    DiagramArgs a;
    a.E = element_count;
    a.aperture = aperture_index;
    a.width = width;
    a.height = height;
    a.rays = intersections ? ray_count : 0;
    a.count = intersection_count;
    a.scale = scale;
    const dim3 block(kDiagramBlock, kDiagramBlock);
    const dim3 grid((width + kDiagramBlock - 1) / kDiagramBlock, (height + kDiagramBlock - 1) / kDiagramBlock);
    k_diagram<<<grid, block, 0, (cudaStream_t)stream>>>(elements, intersections, a, (float4*)image);
    return launch_status();
}
