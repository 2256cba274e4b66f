/*
 * realflare_gb300 — C ABI of the GB300 flare render path.
 *
 * Every entry point takes plain device pointers (allocated and owned by the caller), sizes
 * and a CUDA stream handle (cudaStream_t passed as void*; NULL = legacy default stream).
 * Work is enqueued asynchronously on that stream; nothing is allocated inside the library
 * except where a function says so. Every function returns an rf_status; there are no
 * exceptions across the ABI. Device pointers must be 16-byte aligned.
 *
 * Each declaration names the reference interface it replaces (paths inside the
 * beatreichenbach/realflare project, v0.6.4).
 */
#ifndef REALFLARE_GB300_H
#define REALFLARE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RF_LAMBDA_MIN 390 /* realflare/api/tasks/opencl.py:14 */
#define RF_LAMBDA_MAX 730 /* realflare/api/tasks/opencl.py:15 */
#define RF_LAMBDA_MID 560 /* realflare/api/tasks/opencl.py:16 */
#define RF_BATCH_PRIMITIVE_COUNT 255 /* realflare/api/tasks/rasterizing.py:26 */
#define RF_RAY_PLANES 6  /* pos.x, pos.y, pos_apt.x, pos_apt.y, rrel, reflectance */
#define RF_VERTEX_FLOATS 8 /* pos.xy, uv.xy, rrel, reflectance, intensity, pad */
#define RF_SPECTRUM_WIDTH 340 /* CIE rows 390..729 nm */

typedef enum rf_status {
    RF_OK = 0,
    RF_ERR_INVALID_ARG = 1,     /* a size, pointer or setting outside the supported range */
    RF_ERR_OUT_OF_MEMORY = 2,   /* a device allocation requested by the caller failed */
    /* 3 is not used: no kernel of this library waits on another */
    RF_ERR_CUDA = 4,            /* a CUDA runtime call failed (see rf_last_cuda_error) */
    RF_ERR_WORKSPACE = 5,       /* workspace too small; the required size was written back */
    RF_ERR_NOT_SUPPORTED = 6    /* e.g. an FFT side above 4096 */
} rf_status;

/* One lens element (64 bytes). radius/ior/height/center/coating/coefficients carry the
 * meaning of the reference's lens_element_dtype (realflare/api/tasks/opencl.py:28-37,
 * filled by realflare/api/lens.py:40-86). coating_layers selects the coating model at a
 * reflection: 0 = the reference's single-layer quarter-wave rule (lambda0 = coating nm,
 * thickness lambda0 / (4 nc), realflare/api/tasks/cl/raytracing.cl:316-335); 1 = the same
 * single-layer formula with thickness coating_thickness[0] nm; 2 = an exact two-layer
 * thin-film stack with thicknesses coating_thickness[0..1] nm and layer indices
 * rf_trace_args.coating_layer_ior. coefficients[0..5] = Sellmeier B1,C1,B2,C2,B3,C3;
 * coefficients[0] = NaN on element 0 turns dispersion off. */
typedef struct rf_lens_element {
    float radius;
    float ior;
    float height;
    float center;
    int32_t coating;
    int32_t coating_layers;
    float coating_thickness[2];
    float coefficients[8];
} rf_lens_element;

typedef struct rf_trace_args {
    int32_t element_count;   /* lens elements including the appended sensor */
    int32_t aperture_index;
    int32_t path_count;
    int32_t wavelength_count;
    int32_t grid_count;
    float grid_length;
    float coating_min_ior;
    float coating_layer_ior[2];
    float direction[4];      /* realflare/api/tasks/raytracing.py:92-106 */
} rf_trace_args;

typedef struct rf_raster_args {
    int32_t width, height;
    int32_t bin_size;        /* the reference's BIN_SIZE (realflare/api/data.py:222) */
    int32_t tile_size;       /* raster tile edge in pixels; must divide bin_size; 0 = auto */
    int32_t path_count, wavelength_count, wavelength_sub_count, grid_count;
    int32_t sub_steps;       /* anti-aliasing 1, 2, 4 or 8 */
    float screen_transform;  /* realflare/api/tasks/rasterizing.py:158-167 */
    float intensity;         /* light intensity * 1e3 (rasterizing.py:415) */
    float ghost_scale;       /* 1 - fstop / 32 (rasterizing.py:393) */
    int32_t ghost_width, ghost_height;
} rf_raster_args;

/* ---- library ---------------------------------------------------------------------- */
const char* rf_version(void);
/* Text of the last CUDA error (or rejected argument, where a function says so) seen by
 * this thread; empty if none. */
const char* rf_last_cuda_error(void);
/* Number of kernels this library has launched in this process (all threads). */
long long rf_launch_count(void);

/* ---- ray trace ---------------------------------------------------------------------- */
/* Replaces RaytracingTask.raytrace's kernel launch (realflare/api/tasks/raytracing.py:
 * 140-221) and the raytrace kernel (realflare/api/tasks/cl/raytracing.cl:218-359).
 * elements: device rf_lens_element[element_count]; paths: device int32 pairs [path_count]
 * (bounce1, bounce2); wavelengths: device float nm [wavelength_count]; rays: device
 * float[RF_RAY_PLANES][path_count][wavelength_count][grid_count^2] (plane-major). Invalid
 * rays carry reflectance NaN and the state they had when they stopped. */
int rf_trace(const rf_lens_element* elements, const int32_t* paths, const float* wavelengths,
             const rf_trace_args* args, float* rays, void* stream);

/* rf_trace with the ray geometry in double precision (an opt-in accurate mode; the same
 * kernel of realflare/api/tasks/cl/raytracing.cl:218-359, the same arguments and layout).
 * Grid point, light direction, intersect (raytracing.cl:123-175), refract and reflect
 * (70-102), dispersion (107-120), aperture position and rrel are evaluated in double and
 * rounded to float on output; the coating and Fresnel reflectances (1-59) are FP32. The
 * reference's FP32 positions (rf_trace) differ from the same trace in double by a few ulps,
 * which the rasteriser's integer sample coordinates can turn into whole-pixel changes; this
 * mode's positions are those of the double evaluation. Several times slower than rf_trace
 * (double-precision throughput). */
int rf_trace_accurate(const rf_lens_element* elements, const int32_t* paths, const float* wavelengths,
                      const rf_trace_args* args, float* rays, void* stream);

/* One surface hit of a traced ray (the reference's Intersection, realflare/api/tasks/
 * opencl.py:18-25, without the float3 padding): position and unit normal at the surface,
 * the incidence angle acos(-dir . normal) (0 on flat elements), hit 1 (0 in an unused
 * record). */
typedef struct rf_intersection {
    float pos[3];
    float normal[3];
    float incident;
    int32_t hit;
} rf_intersection;

/* Replaces IntersectionsTask.raytrace (realflare/api/tasks/raytracing.py:250-348): the
 * trace kernel built with STORE_INTERSECTIONS (raytracing.cl:229-271). rf_trace into rays,
 * and every ray's hits into intersections: device rf_intersection[n_rays][intersection_count]
 * (rays in rf_trace's order), zeroed first; record k of a ray is the hit of its k-th loop
 * step (aperture and sensor included); steps past intersection_count are not stored. The
 * reference sizes intersection_count as 3 * element_count - 1. */
int rf_trace_intersections(const rf_lens_element* elements, const int32_t* paths, const float* wavelengths,
                           const rf_trace_args* args, float* rays, rf_intersection* intersections,
                           int32_t intersection_count, void* stream);

/* Replaces DiagramTask (realflare/api/tasks/diagram.py:24-228) and its kernels lenses and
 * intersections (realflare/api/tasks/cl/diagram.cl:21-138): the lens cross-section diagram.
 * image: device float[height][width][4] RGBA, written whole: the optical axis and the
 * elements' profiles at scale pixels per mm (lenses), then, when intersections is not
 * NULL, each ray's path between consecutive hits and each hit's normal (intersections).
 * intersections: device rf_intersection[ray_count][intersection_count], the rays of one
 * grid column (DiagramTask.update_intersection_slice); a ray's last record is followed by
 * the next ray's first, and the last ray's by an unused record. */
int rf_diagram(const rf_lens_element* elements, int32_t element_count, int32_t aperture_index, float scale,
               const rf_intersection* intersections, int32_t ray_count, int32_t intersection_count,
               int32_t width, int32_t height, float* image, void* stream);

/* ---- quad setup ------------------------------------------------------------------- */
/* Replaces the prim_shader kernel (realflare/api/tasks/cl/rasterizing.cl:233-320) and its
 * launch (realflare/api/tasks/rasterizing.py:210-221,321-344). bounds: device float4
 * [path_count][quads] in mm (x = NaN: culled); intensities: device float
 * [path_count][quads][wavelength_count]; entries after a degenerate wavelength are 0. */
int rf_quad_setup(const float* rays, int32_t path_count, int32_t wavelength_count,
                  int32_t grid_count, float area_orig, float min_area, float* bounds,
                  float* intensities, void* stream);

/* Replaces the vertex_shader kernel (realflare/api/tasks/cl/rasterizing.cl:322-386) and
 * its launch (realflare/api/tasks/rasterizing.py:223-235,348-362). vertexes: device
 * float[path_count * grid_count^2 * wavelength_count + 1][RF_VERTEX_FLOATS] in the
 * reference's (path, ray, wavelength) order; the extra trailing vertex is zero. Invalid
 * rays give reflectance NaN and zero elsewhere. */
int rf_vertex(const float* rays, const float* intensities, int32_t path_count,
              int32_t wavelength_count, int32_t grid_count, float screen_transform,
              int32_t width, int32_t height, float* vertexes, void* stream);

/* ---- binning ------------------------------------------------------------------------ */
/* Reference-layout bin masks: replaces the binner kernel (realflare/api/tasks/cl/
 * rasterizing.cl:388-469) and its launch (realflare/api/tasks/rasterizing.py:237-255,
 * 366-385). masks: device uint64[bin_count][batch_count][4], zeroed by this call, with
 * bit (i+1) of (bin, batch) set when primitive batch*255+i overlaps the bin and bit 0 set
 * when any is. Used for parity checks and by callers that consume the reference layout. */
int rf_bin_masks(const float* bounds, int32_t prim_count, float screen_transform,
                 int32_t width, int32_t height, int32_t bin_size, uint64_t* masks,
                 void* stream);

/* Scratch bytes rf_bin_tiles needs for the render settings in args and an entry
 * capacity (entries = (primitive, wavelength pair, tile) triples). */
int rf_bin_workspace_size(const rf_raster_args* args, int64_t entry_capacity, size_t* bytes);

/* Ordered per-tile work lists for rf_raster. An entry is one (primitive, wavelength pair)
 * of the reference's rasteriser loop (rasterizing.cl:573-653) on one raster tile. A tile
 * receives the entry when the primitive's reference bin (bin_size, exactly the test of
 * rasterizing.cl:449-453) contains the tile, and the conservative pixel bounds of the
 * pair's quads touch the tile (pairs whose vertices lie beyond +-(2^14-1) samples, where
 * the reference's 32-bit edge functions can wrap, go to every tile of the reference bin).
 * Pairs with an invalid ray among their endpoint vertices contribute nothing and get no
 * entry. Lists are in increasing (primitive, pair) order, the reference's per-pixel
 * summation order. bounds: rf_quad_setup output; vertexes: rf_vertex output;
 * tile_offsets: device uint32[tiles + 1]; tile_entries: device uint32[entry_capacity]
 * holding primitive * max(W - 1, 1) + pair. The entry count is copied to the host (one
 * stream synchronisation); if it exceeds entry_capacity the call returns RF_ERR_WORKSPACE
 * with the count in *entry_count and leaves the lists unfilled. */
int rf_bin_tiles(const float* bounds, const float* vertexes, const rf_raster_args* args,
                 void* workspace, size_t workspace_bytes, uint32_t* tile_offsets,
                 uint32_t* tile_entries, int64_t entry_capacity, int64_t* entry_count,
                 void* stream);

/* Raster tile grid of args: writes the tile edge (resolving tile_size 0) and tile count. */
int rf_raster_tiles(const rf_raster_args* args, int32_t* tile_size, int32_t* tile_count);

/* ---- raster ------------------------------------------------------------------------- */
/* Replaces the rasterizer kernel (realflare/api/tasks/cl/rasterizing.cl:524-663), its
 * launch with the preceding image clear (realflare/api/tasks/rasterizing.py:257-285,
 * 387-418) and fragment_shader / xyz_to_ap1 (rasterizing.cl:471-522, color.cl:3-10).
 * ghost: device float[ghost_height][ghost_width]; spectrum: device float[340][4] (CIE XYZ0
 * 390..729 nm); image: device float[height][width][4] RGBA (AP1, alpha 0, row 0 = top). */
int rf_raster(const float* vertexes, const uint32_t* tile_offsets, const uint32_t* tile_entries,
              const float* ghost, const float* spectrum, const rf_raster_args* args, float* image,
              void* stream);

/* Largest-first tile order for rf_raster_ordered: a stable sort of the tiles by decreasing
 * entry count (to 3 significant bits), from rf_bin_tiles' tile_offsets [tile_count + 1].
 * tile_order: device uint32[tile_count], a permutation of 0 .. tile_count - 1. Extends the
 * reference's row-major bin launch (rasterizing.py:257-285) with a work order; the image
 * does not depend on it. */
int rf_tile_order_workspace_size(int32_t tile_count, size_t* bytes);
int rf_tile_order(const uint32_t* tile_offsets, int32_t tile_count, void* workspace,
                  size_t workspace_bytes, uint32_t* tile_order, void* stream);

/* rf_raster with the tiles started in tile_order (a permutation of the tiles, e.g. from
 * rf_tile_order) instead of row-major order: heavy tiles first shorten the end of the
 * launch. The image equals rf_raster's bit for bit. */
int rf_raster_ordered(const float* vertexes, const uint32_t* tile_offsets,
                      const uint32_t* tile_entries, const uint32_t* tile_order, const float* ghost,
                      const float* spectrum, const rf_raster_args* args, float* image, void* stream);

/* Reference-order rasteriser over reference-layout masks (for parity checks). */
int rf_raster_masks(const float* vertexes, const uint64_t* masks, int32_t batch_count,
                    const float* ghost, const float* spectrum, const rf_raster_args* args,
                    float* image, void* stream);

/* ---- diffraction ------------------------------------------------------------------ */
/* In-place 2-D FFT of a batch of complex64 images [batch][height][width] (interleaved
 * re, im), width and height any length in [2, 4096] (powers of two by radix-2 passes, other
 * lengths by Bluestein's chirp-z convolution, as numpy accepts any length). direction -1 = forward
 * (exp(-i...)), +1 = inverse; scale multiplies the result (1/sqrt(wh) = numpy "ortho").
 * Replaces numpy.fft.fft2/fftn/ifftn in realflare/api/tasks/starburst.py:71 and
 * realflare/utils/frft.py:27-60. scratch: device complex64 buffer of the same size. */
int rf_fft2(float* data, float* scratch, int32_t batch, int32_t width, int32_t height,
            int32_t direction, float scale, void* stream);

/* Starburst power spectrum: |fftshift(fft2(A * exp(i pi (x^2+y^2) / (lambda d))))|^2 per
 * wavelength (realflare/api/tasks/starburst.py:45-81). aperture: device float[h][w];
 * lambdas_mm: host float[count]; spectrum: device float[count][h][w]; scratch: device
 * complex64[2][count][h][w]. distance_mm = max(1e-9, distance_m * 1e3). */
int rf_starburst_spectrum(const float* aperture, int32_t width, int32_t height,
                          const float* lambdas_mm, int32_t count, float distance_mm,
                          float* scratch, float* spectrum, void* stream);

typedef struct rf_starburst_args {
    int32_t width, height;           /* output image */
    int32_t spectrum_width, spectrum_height, spectrum_count;
    int32_t samples;
    float blur, rotation, rotation_weight;
    float vignetting[2];             /* NaN = off */
    float intensity;                 /* starburst intensity * 1e-6 */
    float offset[2], scale[2];
    float lambda_first, lambda_step; /* per-wavelength spectra: nm of spectrum 0 and step */
} rf_starburst_args;

/* Replaces the starburst kernel (realflare/api/tasks/cl/starburst.cl:1-87) and its launch
 * (realflare/api/tasks/starburst.py:83-153). spectrum_count 1 = the reference's single
 * 560 nm spectrum; > 1 = one spectrum per wavelength (nearest is sampled). image: device
 * float[height][width][4]. */
int rf_starburst(const float* spectrum, const float* light_spectrum, const rf_starburst_args* args,
                 float* image, void* stream);

/* Fractional Fourier transform ghost texture (realflare/api/tasks/ghost.py:13-36 with
 * realflare/utils/frft.py:20-62): |fftshift(frft(fftshift(A), alpha))| * sqrt(w h).
 * aperture: device float[h][w]; texture: device float[h][w]; scratch: device
 * complex64[3][h][w]. */
int rf_ghost_frft(const float* aperture, int32_t width, int32_t height, float alpha,
                  float* scratch, float* texture, void* stream);

/* Largest width * height that rf_ghost_frft_static accepts (512 x 512 pixels). */
#define RF_GHOST_FRFT_STATIC_MAX_PIXELS (512 * 512)

/* rf_ghost_frft for callers that cannot allocate device memory: it has no counterpart in
 * the reference. A plugin inside a host application that owns all device memory through
 * its own pool, or a render loop that must not allocate after start-up (an allocation can
 * synchronise the device and stall a frame), passes only the aperture and the texture;
 * the scratch is a static device array of 3 x RF_GHOST_FRFT_STATIC_MAX_PIXELS complex64
 * values (6 MiB) that every GPU loading this library holds until the process exits. Every
 * call looks up the array's device address on the current device (so no address outlives
 * a device reset); the first call on a device may load the library's device code, so make
 * that first call before any stream capture. All calls share the array: calls that overlap on the GPU
 * (other streams, other host threads on the same device) race. Sizes above the maximum
 * return RF_ERR_INVALID_ARG (text via rf_last_cuda_error). Allocates nothing. */
int rf_ghost_frft_static(const float* aperture, int32_t width, int32_t height, float alpha,
                         float* texture, void* stream);

/* ---- aperture masks ----------------------------------------------------------------- */
/* aperture_shape kernel (realflare/api/tasks/cl/aperture.cl:5-47): writes image[h][w]. */
int rf_aperture_shape(float* image, int32_t width, int32_t height, float size_x, float size_y,
                      int32_t blades, float rotation, float roundness, float softness,
                      void* stream);
/* aperture_dust kernel (realflare/api/tasks/cl/aperture.cl:139-174): multiplies image. */
int rf_aperture_dust(float* image, int32_t width, int32_t height, float size_x, float size_y,
                     float strength, float density, float radius, float parallax_x,
                     float parallax_y, float softness, void* stream);
/* Blurred-noise dust (no reference counterpart): image *= 1 - strength * G_sigma * noise,
 * a separable Gaussian of radius ceil(4 sigma), clamp-to-edge. noise: device float[h][w];
 * scratch: device float[h][w]. */
int rf_aperture_noise_dust(float* image, const float* noise, float* scratch, int32_t width,
                           int32_t height, float strength, float sigma, void* stream);

/* ---- batched frames ------------------------------------------------------------------ */
/* Many frames (lights, lenses, grids, wavelength sets) in one launch per stage, with no
 * host synchronisation, so the whole sequence can be captured into one CUDA graph. There
 * is no reference counterpart: the reference renders one light per Engine call, and its
 * only many-light path loops over lights in Python (realflare/api/engine.py:98-155). Each
 * frame's results equal those of the single-frame functions on the same inputs. */
typedef struct rf_frame {
    rf_trace_args trace;      /* as for rf_trace */
    rf_raster_args raster;    /* as for rf_raster; raster.tile_size is set by rf_batch_plan */
    float area_orig, min_area;  /* as for rf_quad_setup */
    int32_t element_offset;   /* first element in the concatenated rf_lens_element array */
    int32_t path_offset;      /* first path (int32 pair) in the concatenated paths */
    int32_t wavelength_offset;  /* first wavelength in the concatenated wavelengths */
    int64_t ghost_offset;     /* first float of the frame's ghost texture */
    int64_t image_offset;     /* first pixel (4 floats) of the frame's image */
    /* filled by rf_batch_plan */
    int64_t ray_offset;       /* the frame's rays: RF_RAY_PLANES planes of n_rays at rays + 6 * ray_offset */
    int64_t prim_offset;      /* the frame's bounds (float4) */
    int64_t inten_offset;     /* the frame's intensities (float) */
    int64_t vertex_offset;    /* the frame's vertices (n_rays + 1 of them) */
    int64_t pair_offset;      /* the frame's (primitive, wavelength pair) counters */
    int64_t trace_block, quad_block, vertex_block, pair_block;  /* first block of each stage */
    int32_t tile_offset, tile_count;  /* the frame's raster tiles in the batch's tile numbering */
    float direction_n[3];     /* normalize(-direction.xyz) in FP32, as rf_trace computes it */
    int32_t pad1;
    uint64_t ghost_texture;   /* rf_ghost_texture_object of the frame's ghost texture, or 0 */
} rf_frame;

typedef struct rf_batch_sizes {
    int32_t frame_count, tile_size, rays_per_thread, tiles;
    int64_t rays, prims, intensities, vertices, pairs;  /* element counts of the buffers */
    int64_t trace_blocks, quad_blocks, vertex_blocks, pair_blocks;
    int64_t image_pixels, ghost_floats;
    int32_t max_colors, max_sub;  /* largest max(W-1,1) * WS and WS over the frames */
    int32_t max_sub_steps;        /* largest anti-aliasing sample count over the frames */
    int32_t ghost_textures;       /* 1 when every frame has a ghost texture object */
} rf_batch_sizes;

/* Checks every frame and fills the derived fields of frames (host memory) and sizes.
 * tile_size: 16 or 32; rays_per_thread: 1, 2 or 4. The caller then copies frames to the
 * device and allocates rays float[6 * sizes.rays], bounds float4[sizes.prims],
 * intensities float[sizes.intensities], vertexes float[8 * sizes.vertices], images
 * float[4 * sizes.image_pixels]. */
int rf_batch_plan(rf_frame* frames, int32_t frame_count, int32_t tile_size, int32_t rays_per_thread,
                  rf_batch_sizes* sizes);

/* rf_trace of every frame: frames is the planned array in device memory; elements, paths
 * and wavelengths are the concatenated inputs the frames' offsets index. */
int rf_trace_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const rf_lens_element* elements,
                   const int32_t* paths, const float* wavelengths, float* rays, void* stream);

/* rf_quad_setup and rf_vertex of every frame. */
int rf_quad_setup_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const float* rays,
                        float* bounds, float* intensities, void* stream);
int rf_vertex_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const float* rays,
                    const float* intensities, float* vertexes, void* stream);

/* Scratch bytes of rf_bin_tiles_batch + rf_raster_batch for an entry capacity. */
int rf_batch_workspace_size(const rf_batch_sizes* sizes, int64_t entry_capacity, size_t* bytes);

/* rf_bin_tiles of every frame into one tile numbering (frame f's tiles are tile_offset ..
 * tile_offset + tile_count - 1), without host synchronisation: the entry total is written
 * to entry_total (device uint64). When it exceeds entry_capacity the lists are incomplete,
 * rf_raster_batch leaves the images untouched, and the caller retries with a larger
 * capacity. Also orders the tiles by decreasing entry count for rf_raster_batch.
 * tile_offsets: device uint32[tiles + 1]; tile_entries: device uint32[entry_capacity]. */
int rf_bin_tiles_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const float* bounds,
                       const float* vertexes, void* workspace, size_t workspace_bytes,
                       uint32_t* tile_offsets, uint32_t* tile_entries, int64_t entry_capacity,
                       uint64_t* entry_total, void* stream);

/* rf_raster of every frame in one persistent launch: CTAs take tiles from a device-side
 * queue (heaviest first) until it is empty. ghosts: the concatenated ghost textures;
 * images: float[4 * image_pixels]; workspace: the one given to rf_bin_tiles_batch. */
/* A texture object over a ghost texture (device float[height][width]) for the raster's ghost
 * lookups (no counterpart in the reference: its rasteriser reads an OpenCL image,
 * rasterizing.cl:483-485): created once per device, address and size and kept by the library.
 * *texture = 0 when the address or the row pitch (width * 4 bytes) is not aligned as the
 * device's textures require, or when the library already holds 4096 of them (it keeps
 * every object for the life of the process and never synchronises to release one); the
 * raster then loads the texels. rf_raster, rf_raster_ordered and rf_raster_backward use
 * it by themselves; a batch passes it per frame in rf_frame.ghost_texture. */
int rf_ghost_texture_object(const float* ghost, int32_t width, int32_t height, uint64_t* texture);

/* Forgets the library's ghost texture objects on the current device without destroying
 * them: for a host that reset the device (cudaDeviceReset ends the objects with the
 * context, and a later raster call must not be handed one of them). Call it after the reset
 * and before the next raster call; no CUDA work is issued. */
int rf_ghost_textures_forget(void);

int rf_raster_batch(const rf_frame* frames, const rf_batch_sizes* sizes, const float* vertexes,
                    const uint32_t* tile_offsets, const uint32_t* tile_entries, const float* ghosts,
                    const float* spectrum, void* workspace, size_t workspace_bytes,
                    int64_t entry_capacity, const uint64_t* entry_total, float* images, void* stream);

/* ---- differentiation ------------------------------------------------------------------- */
/* Adjoint (reverse-mode derivative) of rf_trace; no reference counterpart (the reference
 * has no derivatives). grad_rays: device float[RF_RAY_PLANES][n_rays], the gradient of a
 * loss with respect to rf_trace's outputs (sensor x, y; aperture x, y; rrel; reflectance).
 * Writes grad_elements: device float[element_count][4], the gradient with respect to each
 * element's radius, center, coating_thickness[0] and coating_thickness[1], and
 * grad_direction: device float[3], with respect to normalize(-direction.xyz). Rays that do
 * not reach the sensor contribute nothing; each ray's discrete choices (elements hit,
 * reflections, the element giving rrel) are held fixed. element_count <= 32. */
int rf_trace_adjoint(const rf_lens_element* elements, const int32_t* paths, const float* wavelengths,
                     const rf_trace_args* args, const float* grad_rays, float* grad_elements,
                     float* grad_direction, void* stream);

/* Adjoint of rf_raster (the same tile size and tile lists). Coverage and the mean-value
 * weights depend on the vertex positions only through integer sample coordinates, so they
 * are held fixed: the gradient flows to each vertex's interpolated attributes (aperture
 * position, rrel, reflectance, intensity), not to its screen position (the change of
 * covered pixels as quad edges move is not included). image: rf_raster's output; grad_image:
 * device float[height][width][4]; grad_vertexes: device float[n_vertices][8] (the vertex
 * layout; floats 2..6 receive the gradients), zeroed by this call. */
int rf_raster_backward(const float* vertexes, const uint32_t* tile_offsets, const uint32_t* tile_entries,
                       const float* ghost, const float* spectrum, const rf_raster_args* args,
                       const float* image, const float* grad_image, float* grad_vertexes, void* stream);

/* Adjoint of rf_vertex: writes grad_rays planes 2..5 (aperture x, y, rrel, reflectance)
 * from grad_vertexes, zeroes planes 0..1, and writes grad_intensities (device
 * float[path_count][quads][wavelength_count]) from the vertices' averaged intensities. */
int rf_vertex_backward(const float* rays, const float* intensities, int32_t path_count,
                       int32_t wavelength_count, int32_t grid_count, const float* grad_vertexes,
                       float* grad_rays, float* grad_intensities, void* stream);

/* Adjoint of rf_quad_setup's intensity area_orig / max(area, min_area): adds the gradient
 * of the quads' sensor-plane areas to grad_rays planes 0..1 (sensor x, y). */
int rf_quad_setup_backward(const float* rays, int32_t path_count, int32_t wavelength_count,
                           int32_t grid_count, float area_orig, float min_area,
                           const float* grad_intensities, float* grad_rays, void* stream);

/* ---- compositing ---------------------------------------------------------------------- */
/* Image-based light accumulation (realflare/api/engine.py:120-150): image (device
 * float[height][width][4], read and written) += for each light sample k, weights[k][m] *
 * (frame k mirrored: m = 0 as is, 1 flipped vertically, 2 both ways, 3 horizontally),
 * per channel, in sample order; then divided by divisor when it is > 0. frames: device
 * float[count][height][width][4]; weights: device float[count][4][4]. */
int rf_accumulate_mirrored(const float* frames, const float* weights, int32_t count, int32_t width,
                           int32_t height, float divisor, float* image, void* stream);

/* out = a * wa + b * wb elementwise over n floats (Engine.flare_starburst,
 * realflare/api/engine.py:174-187, uses wa = 2, wb = 1). */
int rf_axpby(const float* a, float wa, const float* b, float wb, float* out, int64_t n,
             void* stream);

#ifdef __cplusplus
}
#endif

#endif /* REALFLARE_GB300_H */
