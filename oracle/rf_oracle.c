/*
 * rf_oracle.c — CPU restatement of realflare's render hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker for the CUDA library: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it. The product path never
 * calls it.
 *
 * It restates, function by function, the OpenCL kernels of realflare v0.6.4 (paths below
 * are inside that project) in plain C. Built twice: RFO_REAL=float (the FP32 parity
 * target) and RFO_REAL=double (the FP64 oracle; rounding and discontinuities such as the
 * float->int truncations stay where the reference has them). Places where OpenCL C
 * evaluates an unsuffixed literal in double are evaluated in double here as well.
 *
 * Behaviour the reference leaves undefined is given one definition, shared with the CUDA
 * kernels:
 *  - float->int conversions truncate toward zero and saturate (NaN -> 0);
 *  - integer edge functions wrap in 32 bits;
 *  - max(NaN, 0) = 0 and clamp(NaN, lo, hi) = lo (fmax/fmin semantics);
 *  - fields of vertices of invalid rays are 0 (reflectance stays NaN);
 *  - intensities after a degenerate wavelength are 0;
 *  - bilinear sampling at a non-finite coordinate returns 0;
 *  - the vertex after the last one is all zeros;
 *  - a ray whose first intersection misses element 0 starts from the origin (the
 *    reference leaves that intersection uninitialised; zero is its zero-initialised value).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <tgmath.h>

#include "../include/realflare_gb300.h"

#ifndef RFO_REAL
#define RFO_REAL float
#endif
typedef RFO_REAL real;
#define K(x) ((real)(x))

static const real M_PI_R = (real)3.14159274101257324f; /* OpenCL M_PI_F */

/* ---------------------------------------------------------------- integer semantics */
static inline int32_t cvt_rz_sat(real x) {
    if (x != x) return 0;
    if (x >= (real)2147483647.0) return INT32_MAX;
    if (x <= (real)-2147483648.0) return INT32_MIN;
    return (int32_t)x;
}
static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

static inline real rmax(real a, real b) { return fmax(a, b); }
static inline real rmin(real a, real b) { return fmin(a, b); }
static inline real rclamp(real x, real lo, real hi) { return fmin(fmax(x, lo), hi); }
static inline real smoothstep_r(real e0, real e1, real x) {
    real t = rclamp((x - e0) / (e1 - e0), K(0), K(1));
    return t * t * (K(3) - K(2) * t);
}

/* ---------------------------------------------------------------- vectors */
typedef struct { real x, y, z; } v3;
static inline v3 mk3(real x, real y, real z) { v3 r = {x, y, z}; return r; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, real s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline v3 neg3(v3 a) { return mk3(-a.x, -a.y, -a.z); }
static inline real dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline real len3(v3 a) { return sqrt(dot3(a, a)); }
static inline v3 norm3(v3 a) { return mul3(a, K(1) / sqrt(dot3(a, a))); }

/* ---------------------------------------------------------------- trace
 * realflare/api/tasks/cl/raytracing.cl */

/* fresnel, raytracing.cl:1-16 */
static real fresnel(real theta0, real n1, real n2) {
    real theta1 = asin(sin(theta0) * n1 / n2);
    real cosi = cos(theta0);
    real cost = cos(theta1);
    real rs = ((n1 * cosi) - (n2 * cost)) / ((n1 * cosi) + (n2 * cost));
    real rp = ((n1 * cost) - (n2 * cosi)) / ((n1 * cost) + (n2 * cosi));
    return (rs * rs + rp * rp) / K(2);
}

/* fresnel_ar, raytracing.cl:18-59 (Ritschel et al. 2009, two-beam single layer) */
static real fresnel_ar(real theta0, real lambda, real d1, real n0, real n1, real n2) {
    real theta1 = asin(sin(theta0) * n0 / n1);
    real theta2 = asin(sin(theta0) * n0 / n2);
    real rs01 = -sin(theta0 - theta1) / sin(theta0 + theta1);
    real rp01 = tan(theta0 - theta1) / tan(theta0 + theta1);
    real ts01 = K(2) * sin(theta1) * cos(theta0) / sin(theta0 + theta1);
    real tp01 = ts01 * cos(theta0 - theta1);
    real rs12 = -sin(theta1 - theta2) / sin(theta1 + theta2);
    real rp12 = tan(theta1 - theta2) / tan(theta1 + theta2);
    real ris = ts01 * ts01 * rs12;
    real rip = tp01 * tp01 * rp12;
    real dy = d1 * n1;
    real dx = tan(theta1) * dy;
    real delay = sqrt(dx * dx + dy * dy);
    real rel_phase = K(4) * M_PI_R / lambda * (delay - dx * sin(theta0));
    real out_s2 = rs01 * rs01 + ris * ris + K(2) * rs01 * ris * cos(rel_phase);
    real out_p2 = rp01 * rp01 + rip * rip + K(2) * rp01 * rip * cos(rel_phase);
    return (out_s2 + out_p2) / K(2);
}

/* Two-layer thin-film stack (no reference counterpart): exact Airy reflectance of
 * incident medium n0 | layer a (na, da) | layer b (nb, db) | substrate n2, averaged over
 * s and p. Real cosines; a layer in total internal reflection yields NaN, which the
 * caller's "multiply only if > 0" rule skips like the reference's single-layer NaN. */
static void interface_r(real ni, real ci, real nj, real cj, real* rs, real* rp) {
    *rs = (ni * ci - nj * cj) / (ni * ci + nj * cj);
    *rp = (nj * ci - ni * cj) / (nj * ci + ni * cj);
}
static real stack_r2(real r01, real r12, real r23, real d1, real d2) {
    /* r_inner = (r12 + r23 e^{i d2}) / (1 + r12 r23 e^{i d2}); d = 2 delta */
    real c2 = cos(d2), s2 = sin(d2);
    real nre = r12 + r23 * c2, nim = r23 * s2;
    real dre = K(1) + r12 * r23 * c2, dim = r12 * r23 * s2;
    real den = dre * dre + dim * dim;
    real ire = (nre * dre + nim * dim) / den;
    real iim = (nim * dre - nre * dim) / den;
    /* r = (r01 + ri e^{i d1}) / (1 + r01 ri e^{i d1}) */
    real c1 = cos(d1), s1 = sin(d1);
    real ere = ire * c1 - iim * s1, eim = ire * s1 + iim * c1;
    real tre = r01 + ere, tim = eim;
    real bre = K(1) + r01 * ere, bim = r01 * eim;
    return (tre * tre + tim * tim) / (bre * bre + bim * bim);
}
static real fresnel_two_layer(real theta0, real lambda, real n0, real na, real da, real nb,
                              real db, real n2) {
    real s0 = sin(theta0);
    real c0 = cos(theta0);
    real sa = n0 * s0 / na, sb = n0 * s0 / nb, s2 = n0 * s0 / n2;
    real ca = sqrt(K(1) - sa * sa), cb = sqrt(K(1) - sb * sb), c2 = sqrt(K(1) - s2 * s2);
    real rs01, rp01, rs12, rp12, rs23, rp23;
    interface_r(n0, c0, na, ca, &rs01, &rp01);
    interface_r(na, ca, nb, cb, &rs12, &rp12);
    interface_r(nb, cb, n2, c2, &rs23, &rp23);
    real phase = K(4) * M_PI_R / lambda;
    real d1 = phase * na * da * ca;
    real d2 = phase * nb * db * cb;
    return (stack_r2(rs01, rs12, rs23, d1, d2) + stack_r2(rp01, rp12, rp23, d1, d2)) / K(2);
}

/* dispersion, raytracing.cl:107-120 (lambda * 1e-3 is a double expression there) */
static real dispersion(real lambda, const float* c) {
    real l = (real)((double)lambda * 1e-3);
    real l2 = l * l;
    real d0 = ((real)c[0] * l2) / (l2 - (real)c[1]);
    real d1 = ((real)c[2] * l2) / (l2 - (real)c[3]);
    real d2 = ((real)c[4] * l2) / (l2 - (real)c[5]);
    return sqrt(K(1) + d0 + d1 + d2);
}

typedef struct { v3 pos, normal; real incident; int hit; } hit_t;

/* intersect, raytracing.cl:123-175, with the element's radius and center given */
static hit_t intersect_rc(v3 pos, v3 dir, real radius, real center) {
    hit_t h;
    memset(&h, 0, sizeof(h));
    if (dir.z == 0) {
        h.hit = 0;
    } else if (radius == 0) {
        real dz = -center - pos.z;
        h.pos = add3(pos, mul3(dir, dz / dir.z));
        h.normal = (dir.z < 0) ? mk3(0, 0, 1) : mk3(0, 0, -1);
        h.hit = 1;
        h.incident = 0;
    } else {
        real r = fabs(radius);
        v3 C = mk3(0, 0, -center);
        v3 U = sub3(C, pos);
        v3 U1 = mul3(dir, dot3(U, dir));
        real d = len3(sub3(U, U1));
        if (d > r) {
            h.hit = 0;
            return h;
        }
        real sgn = (radius * dir.z) > 0 ? K(-1) : K(1);
        real m = sqrt(r * r - d * d);
        v3 p = sub3(add3(pos, U1), mul3(mul3(dir, m), sgn));
        v3 normal = mul3(norm3(sub3(p, C)), sgn);
        real incident = acos(rclamp(dot3(neg3(dir), normal), K(-1), K(1)));
        h.hit = 1;
        h.incident = incident;
        h.pos = p;
        h.normal = normal;
    }
    return h;
}

static hit_t intersect(v3 pos, v3 dir, const rf_lens_element* e) {
    return intersect_rc(pos, dir, (real)e->radius, (real)e->center);
}

/* reflect / refract, raytracing.cl:70-102 */
static v3 reflect3(v3 i, v3 n) { return add3(i, mul3(n, K(2) * dot3(n, neg3(i)))); }
static v3 refract3(v3 i, v3 n, real o) {
    real cost = dot3(neg3(i), n);
    real sint2 = (o * o) * (K(1) - cost * cost);
    v3 t = add3(mul3(i, o), mul3(n, o * cost - sqrt(fabs(K(1) - sint2))));
    return mul3(t, (real)(sint2 < K(1)));
}

/* Grid point of a ray, init_ray raytracing.cl:185-194 (the 0.5 literals are double). */
static void grid_point(int ray_id, int grid_count, real grid_length, real* px, real* py) {
    int y = (int)trunc((float)ray_id / (float)grid_count);
    int x = ray_id - y * grid_count;
    float fx = (float)x / (float)(grid_count - 1);
    float fy = (float)y / (float)(grid_count - 1);
    *px = (real)((double)grid_length * ((double)fx - 0.5));
    *py = (real)((double)grid_length * (0.5 - (double)fy));
}

/* raytrace kernel, raytracing.cl:178-359. rays: RF_RAY_PLANES planes of P*W*R floats. */
/* geom (optional, finite-difference checks): per element radius, center, coating
 * thickness 0 and 1 in double, replacing the element's float fields; dir3 (optional): the
 * light direction in double. inter (optional): the ray's hits as built with
 * STORE_INTERSECTIONS (raytracing.cl:229-271), inter_count records of 8 floats (pos xyz,
 * normal xyz, incident, hit as int32) per ray, record k = the hit of loop step k. */
static void trace_one(const rf_lens_element* el, const int32_t* paths, const float* wavelengths,
                      const rf_trace_args* a, size_t idx, float* rays, double* rays_d, size_t n_rays,
                      const double* geom, const double* dir3, float* inter, int inter_count) {
    const int E = a->element_count;
    const int R = a->grid_count * a->grid_count;
    const int ray_id = (int)(idx % (size_t)R);
    const int wl_id = (int)((idx / (size_t)R) % (size_t)a->wavelength_count);
    const int path_id = (int)(idx / ((size_t)R * (size_t)a->wavelength_count));
    const int px_bounce = paths[2 * path_id], py_bounce = paths[2 * path_id + 1];
    const real wavelength = (real)wavelengths[wl_id];

    real gx, gy;
    grid_point(ray_id, a->grid_count, (real)a->grid_length, &gx, &gy);
    v3 pos = mk3(gx, gy, 1), dir = mk3(0, 0, -1);
#define RFO_RADIUS(i) (geom ? (real)geom[4 * (i)] : (real)el[i].radius)
#define RFO_CENTER(i) (geom ? (real)geom[4 * (i) + 1] : (real)el[i].center)
#define RFO_T0(i) (geom ? (real)geom[4 * (i) + 2] : (real)el[i].coating_thickness[0])
#define RFO_T1(i) (geom ? (real)geom[4 * (i) + 3] : (real)el[i].coating_thickness[1])
    hit_t h0 = intersect_rc(pos, dir, RFO_RADIUS(0), RFO_CENTER(0));
    pos = h0.pos; /* zero when the grid point misses element 0 */
    v3 direction = dir3 ? norm3(neg3(mk3((real)dir3[0], (real)dir3[1], (real)dir3[2])))
                        : norm3(neg3(mk3((real)a->direction[0], (real)a->direction[1], (real)a->direction[2])));
    pos = sub3(pos, direction);
    dir = direction;
    real apt_x = 0, apt_y = 0, rrel = 0, refl = 1;

    int step = 0, delta = 1;
    const int disperse = !isnan(el[0].coefficients[0]);
    int lens_id, inter_id = 0;
    for (lens_id = 0; lens_id >= 0 && lens_id < E; lens_id += delta, inter_id++) {
        const rf_lens_element* e = &el[lens_id];
        hit_t h = intersect_rc(pos, dir, RFO_RADIUS(lens_id), RFO_CENTER(lens_id));
        if (!h.hit) break;
        if (inter && inter_id < inter_count) {
            float* o = inter + (idx * (size_t)inter_count + (size_t)inter_id) * 8;
            const int32_t one = 1;
            o[0] = (float)h.pos.x;
            o[1] = (float)h.pos.y;
            o[2] = (float)h.pos.z;
            o[3] = (float)h.normal.x;
            o[4] = (float)h.normal.y;
            o[5] = (float)h.normal.z;
            o[6] = (float)h.incident;
            memcpy(o + 7, &one, sizeof one);
        }
        pos = h.pos;
        if (lens_id == a->aperture_index) {
            apt_x = h.pos.x / (real)e->height;
            apt_y = h.pos.y / (real)e->height;
            continue;
        } else {
            rrel = rmax(rrel, sqrt(h.pos.x * h.pos.x + h.pos.y * h.pos.y) / (real)e->height);
        }
        if (lens_id == E - 1) continue;
        int do_reflect = 0;
        if ((step == 0 && lens_id == px_bounce) || (step == 1 && lens_id == py_bounce)) {
            do_reflect = 1;
            step++;
            delta = -delta;
        }
        int n_index = (dir.z < 0) ? lens_id - 1 : lens_id + 1;
        real n1 = (0 <= n_index && n_index < E) ? (real)el[n_index].ior : K(1);
        real n2 = (real)e->ior;
        if (disperse && n1 > 1) n1 = dispersion(wavelength, el[n_index].coefficients);
        if (disperse && n2 > 1) n2 = dispersion(wavelength, e->coefficients);
        if (do_reflect) {
            dir = reflect3(dir, h.normal);
            real theta = (real)((double)h.incident + 1e-9);
            real reflectance;
            if (e->coating_layers == 2) {
                reflectance = fresnel_two_layer(theta, wavelength, n1, (real)a->coating_layer_ior[0],
                                                RFO_T0(lens_id), (real)a->coating_layer_ior[1],
                                                RFO_T1(lens_id), n2);
            } else if (e->coating_layers == 1 || e->coating > 0) {
                real nc = rmax(sqrt(n1 * n2), (real)a->coating_min_ior);
                real d1 = e->coating_layers == 1 ? RFO_T0(lens_id) : (real)e->coating / (K(4) * nc);
                reflectance = fresnel_ar(theta, wavelength, d1, n1, nc, n2);
            } else {
                reflectance = fresnel(theta, n1, n2);
            }
            if (reflectance > 0) refl *= reflectance;
        } else {
            real ratio = n1 / n2;
            dir = refract3(dir, h.normal, ratio);
            if (dir.z == 0) break;
        }
    }
#undef RFO_RADIUS
#undef RFO_CENTER
#undef RFO_T0
#undef RFO_T1
    if (lens_id >= 0 && lens_id < E) refl = (real)NAN;
    if (rays_d) { /* unrounded outputs (finite-difference checks of the FP64 build) */
        rays_d[0 * n_rays + idx] = (double)pos.x;
        rays_d[1 * n_rays + idx] = (double)pos.y;
        rays_d[2 * n_rays + idx] = (double)apt_x;
        rays_d[3 * n_rays + idx] = (double)apt_y;
        rays_d[4 * n_rays + idx] = (double)rrel;
        rays_d[5 * n_rays + idx] = (double)refl;
        return;
    }
    rays[0 * n_rays + idx] = (float)pos.x;
    rays[1 * n_rays + idx] = (float)pos.y;
    rays[2 * n_rays + idx] = (float)apt_x;
    rays[3 * n_rays + idx] = (float)apt_y;
    rays[4 * n_rays + idx] = (float)rrel;
    rays[5 * n_rays + idx] = (float)refl;
}

int rfo_trace(const rf_lens_element* el, const int32_t* paths, const float* wavelengths,
              const rf_trace_args* a, float* rays) {
    const size_t R = (size_t)a->grid_count * (size_t)a->grid_count;
    const size_t n = (size_t)a->path_count * (size_t)a->wavelength_count * R;
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long i = 0; i < (long long)n; i++) trace_one(el, paths, wavelengths, a, (size_t)i, rays, NULL, n, NULL, NULL, NULL, 0);
    return 0;
}

/* rfo_trace with the element geometry (radius, center, coating thicknesses per element) and
 * the light direction given in double, outputs in double (finite-difference checks). */
int rfo_trace_geom_d(const rf_lens_element* el, const int32_t* paths, const float* wavelengths,
                     const rf_trace_args* a, const double* geom, const double* dir3, double* rays) {
    const size_t R = (size_t)a->grid_count * (size_t)a->grid_count;
    const size_t n = (size_t)a->path_count * (size_t)a->wavelength_count * R;
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long i = 0; i < (long long)n; i++) trace_one(el, paths, wavelengths, a, (size_t)i, NULL, rays, n, geom, dir3, NULL, 0);
    return 0;
}

/* rfo_trace with outputs in double, not rounded to float. */
int rfo_trace_d(const rf_lens_element* el, const int32_t* paths, const float* wavelengths,
                const rf_trace_args* a, double* rays) {
    const size_t R = (size_t)a->grid_count * (size_t)a->grid_count;
    const size_t n = (size_t)a->path_count * (size_t)a->wavelength_count * R;
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long i = 0; i < (long long)n; i++) trace_one(el, paths, wavelengths, a, (size_t)i, NULL, rays, n, NULL, NULL, NULL, 0);
    return 0;
}

/* rfo_trace that also stores every ray's hits (IntersectionsTask.raytrace,
 * raytracing.py:250-348): inter = n_rays * inter_count records of 8 floats, zeroed first
 * (update_intersections allocates zeros, raytracing.py:115-123). */
int rfo_trace_intersections(const rf_lens_element* el, const int32_t* paths, const float* wavelengths,
                            const rf_trace_args* a, float* rays, float* inter, int inter_count) {
    const size_t R = (size_t)a->grid_count * (size_t)a->grid_count;
    const size_t n = (size_t)a->path_count * (size_t)a->wavelength_count * R;
    memset(inter, 0, sizeof(float) * 8 * n * (size_t)inter_count);
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)n; i++)
        trace_one(el, paths, wavelengths, a, (size_t)i, rays, NULL, n, NULL, NULL, inter, inter_count);
    return 0;
}

/* Trace a subset of ray indices [first, first + count) (CPU baseline samples). */
int rfo_trace_range(const rf_lens_element* el, const int32_t* paths, const float* wavelengths,
                    const rf_trace_args* a, float* rays, long long first, long long count) {
    const size_t R = (size_t)a->grid_count * (size_t)a->grid_count;
    const size_t n = (size_t)a->path_count * (size_t)a->wavelength_count * R;
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long i = first; i < first + count; i++) trace_one(el, paths, wavelengths, a, (size_t)i, rays, NULL, n, NULL, NULL, NULL, 0);
    return 0;
}

/* ---------------------------------------------------------------- quad setup
 * prim_shader, realflare/api/tasks/cl/rasterizing.cl:233-320 */
static inline real edge_f(real ax, real ay, real bx, real by, real cx, real cy) {
    return (ax - bx) * (cy - ay) - (ay - by) * (cx - ax);
}

int rfo_quad_setup(const float* rays, int P, int W, int G, float area_orig, float min_area,
                   float* bounds, float* intensities) {
    const int R = G * G, Q = (G - 1) * (G - 1);
    const size_t n_rays = (size_t)P * W * R;
    const float* pos_x = rays;
    const float* pos_y = rays + n_rays;
    const float* rrel = rays + 4 * n_rays;
    const float* refl = rays + 5 * n_rays;
#pragma omp parallel for schedule(static)
    for (long long pq = 0; pq < (long long)P * Q; pq++) {
        int path = (int)(pq / Q), quad = (int)(pq % Q);
        int row = quad / (G - 1), col = quad % (G - 1);
        int v[4];
        v[0] = row * G + col;
        v[1] = v[0] + 1;
        v[2] = v[1] + G;
        v[3] = v[0] + G;
        real bx0 = INFINITY, by0 = INFINITY, bx1 = -INFINITY, by1 = -INFINITY;
        int invalid_rrel = 0;
        int culled = 0;
        for (int w = 0; w < W; w++) {
            size_t prim_index = ((size_t)path * Q + quad) * W + w;
            intensities[prim_index] = 0;
        }
        for (int w = 0; w < W; w++) {
            if (culled) continue;
            size_t off = ((size_t)path * W + w) * R;
            size_t prim_index = ((size_t)path * Q + quad) * W + w;
            real px[4], py[4], rr[4];
            int valid = 0;
            for (int i = 0; i < 4; i++) rr[i] = (real)rrel[off + v[i]];
            for (int i = 0; i < 4; i++) {
                if (!isnan(refl[off + v[i]])) {
                    px[valid] = (real)pos_x[off + v[i]];
                    py[valid] = (real)pos_y[off + v[i]];
                    valid++;
                }
            }
            real area;
            if (valid == 4) {
                real a0 = edge_f(px[0], py[0], px[1], py[1], px[2], py[2]);
                real a1 = edge_f(px[0], py[0], px[2], py[2], px[3], py[3]);
                area = fabs(a0 + a1) / K(2);
            } else if (valid == 3) {
                area = fabs(edge_f(px[0], py[0], px[1], py[1], px[2], py[2]));
                px[3] = px[2];
                py[3] = py[2];
                rr[3] = rr[2];
            } else {
                culled = 1;
                continue;
            }
            if (rr[0] > 1 && rr[1] > 1 && rr[2] > 1 && rr[3] > 1) invalid_rrel++;
            real area_actual = rmax(area, (real)min_area);
            intensities[prim_index] = (float)(area_actual > 0 ? (real)area_orig / area_actual : K(0));
            real mnx = rmin(rmin(px[0], px[1]), rmin(px[2], px[3]));
            real mny = rmin(rmin(py[0], py[1]), rmin(py[2], py[3]));
            real mxx = rmax(rmax(px[0], px[1]), rmax(px[2], px[3]));
            real mxy = rmax(rmax(py[0], py[1]), rmax(py[2], py[3]));
            bx0 = rmin(bx0, mnx);
            by0 = rmin(by0, mny);
            bx1 = rmax(bx1, mxx);
            by1 = rmax(by1, mxy);
        }
        if (invalid_rrel == W) culled = 1;
        float* b = bounds + 4 * pq;
        b[0] = culled ? NAN : (float)bx0;
        b[1] = (float)by0;
        b[2] = (float)bx1;
        b[3] = (float)by1;
    }
    return 0;
}

/* ---------------------------------------------------------------- vertex shader
 * rasterizing.cl:196-216 (quad_neighbors), 322-386 */
int rfo_vertex(const float* rays, const float* intensities, int P, int W, int G, float st,
               int width, int height, float* vertexes) {
    const int R = G * G, Q = (G - 1) * (G - 1);
    const size_t n_rays = (size_t)P * W * R;
    const real hw = (real)width / K(2), hh = (real)height / K(2);
#pragma omp parallel for schedule(static)
    for (long long vi = 0; vi < (long long)n_rays; vi++) {
        int w = (int)(vi % W);
        int ray_id = (int)((vi / W) % R);
        int path = (int)(vi / ((long long)W * R));
        size_t ray_index = ((size_t)path * W + w) * R + ray_id;
        float* out = vertexes + 8 * vi;
        for (int k = 0; k < 8; k++) out[k] = 0;
        real refl = (real)rays[5 * n_rays + ray_index];
        out[5] = (float)refl;
        if (isnan(refl)) continue;
        int x = ray_id % G, y = ray_id / G;
        int nb[4];
        nb[0] = (y - 1) * (G - 1) + (x - 1);
        nb[1] = nb[0] + 1;
        nb[2] = y * (G - 1) + (x - 1);
        nb[3] = nb[2] + 1;
        real inten = 0;
        int count = 0;
        for (int i = 0; i < 4; i++) {
            if (nb[i] < 0 || nb[i] >= Q) continue;
            real v = (real)intensities[((size_t)path * Q + nb[i]) * W + w];
            if (v > 0) {
                inten += v;
                ++count;
            }
        }
        inten /= (real)(count > 1 ? count : 1);
        out[0] = (float)((real)rays[ray_index] * (real)st + hw);
        out[1] = (float)((real)rays[n_rays + ray_index] * (real)st + hh);
        out[2] = rays[2 * n_rays + ray_index];
        out[3] = rays[3 * n_rays + ray_index];
        out[4] = rays[4 * n_rays + ray_index];
        out[6] = (float)inten;
    }
    /* the slot after the last vertex is all zero */
    for (int k = 0; k < 8; k++) vertexes[8 * n_rays + k] = 0;
    return 0;
}

/* ---------------------------------------------------------------- binner
 * rasterizing.cl:388-469: masks[bin][batch][4] uint64 */
static void screen_bounds(const float* b, real st, int width, int height, int32_t sb[4]) {
    sb[0] = wadd(cvt_rz_sat((real)b[0] * st), width / 2);
    sb[1] = wadd(cvt_rz_sat((real)b[1] * st), height / 2);
    sb[2] = wadd(cvt_rz_sat((real)b[2] * st), width / 2);
    sb[3] = wadd(cvt_rz_sat((real)b[3] * st), height / 2);
}

int rfo_bin_masks(const float* bounds, int prim_count, float st, int width, int height, int B,
                  uint64_t* masks) {
    const int bdx = (width + B - 1) / B, bdy = (height + B - 1) / B;
    const int bins = bdx * bdy;
    const int batches = (prim_count + RF_BATCH_PRIMITIVE_COUNT - 1) / RF_BATCH_PRIMITIVE_COUNT;
    memset(masks, 0, sizeof(uint64_t) * 4 * (size_t)bins * batches);
#pragma omp parallel for schedule(dynamic, 4)
    for (int batch = 0; batch < batches; batch++) {
        for (int bin = 0; bin < bins; bin++) {
            int bx = bin % bdx, by = bin / bdx;
            int32_t binr[4] = {bx * B, by * B, bx * B + B, by * B + B};
            uint64_t q[4] = {0, 0, 0, 0};
            int any = 0;
            int last = batch * RF_BATCH_PRIMITIVE_COUNT + RF_BATCH_PRIMITIVE_COUNT;
            if (last > prim_count) last = prim_count;
            for (int p = batch * RF_BATCH_PRIMITIVE_COUNT, c = 0; p < last; p++, c++) {
                const float* b = bounds + 4 * (size_t)p;
                if (isnan(b[0])) continue;
                int32_t sb[4];
                screen_bounds(b, (real)st, width, height, sb);
                if (sb[0] <= binr[2] && sb[2] >= binr[0] && sb[1] <= binr[3] && sb[3] >= binr[1]) {
                    int bit = c + 1;
                    q[bit >> 6] |= (uint64_t)1 << (bit & 63);
                    any = 1;
                }
            }
            if (any) q[0] |= 1;
            uint64_t* out = masks + 4 * ((size_t)bin * batches + batch);
            out[0] = q[0];
            out[1] = q[1];
            out[2] = q[2];
            out[3] = q[3];
        }
    }
    return 0;
}

/* ---------------------------------------------------------------- raster
 * rasterizing.cl:1-148 (edge functions, Hormann-Tarini quad test, mean value
 * coordinates), 471-663 (fragment shader, rasterizer), color.cl:3-10 */
static const unsigned char SUB_OFFSETS[15] = {0, 1, 0, 1, 2, 0, 3, 4, 1, 6, 2, 5, 0, 3, 7};

static inline int32_t edge_i(int32_t ax, int32_t ay, int32_t bx, int32_t by, int32_t cx, int32_t cy) {
    return wsub(wmul(wsub(ax, bx), wsub(cy, ay)), wmul(wsub(ay, by), wsub(cx, ax)));
}
static inline int top_left(int32_t ax, int32_t ay, int32_t bx, int32_t by) {
    int32_t ex = wsub(bx, ax), ey = wsub(by, ay);
    return (ey == 0 && ex > 0) || ey > 0;
}
static int intersect_quad(int32_t px, int32_t py, const int32_t* q /* x0 y0 .. x3 y3 */) {
    int32_t b01 = top_left(q[0], q[1], q[2], q[3]) ? 0 : -1;
    int32_t b12 = top_left(q[2], q[3], q[4], q[5]) ? 0 : -1;
    int32_t b23 = top_left(q[4], q[5], q[6], q[7]) ? 0 : -1;
    int32_t b30 = top_left(q[6], q[7], q[0], q[1]) ? 0 : -1;
    int32_t b20 = top_left(q[4], q[5], q[0], q[1]) ? 0 : -1;
    int32_t l01 = wadd(edge_i(q[0], q[1], q[2], q[3], px, py), b01);
    int32_t l12 = wadd(edge_i(q[2], q[3], q[4], q[5], px, py), b12);
    int32_t l23 = wadd(edge_i(q[4], q[5], q[6], q[7], px, py), b23);
    int32_t l30 = wadd(edge_i(q[6], q[7], q[0], q[1], px, py), b30);
    int32_t l20 = wadd(edge_i(q[4], q[5], q[0], q[1], px, py), b20);
    int w01 = l01 >= 0, w12 = l12 >= 0, w23 = l23 >= 0, w30 = l30 >= 0;
    if (edge_i(q[0], q[1], q[2], q[3], q[4], q[5]) == 0 && edge_i(q[0], q[1], q[4], q[5], q[6], q[7]) == 0)
        return 0;
    int w20 = l20 >= 0;
    int front = (w20 && w01 && w12 && (w23 || w30)) || (!w20 && w23 && w30 && (w01 || w12));
    int back = (!w20 && !w01 && !w12 && (!w23 || !w30)) || (w20 && !w23 && !w30 && (!w01 || !w12));
    return front || back;
}
static void barycentric_quad(int32_t px, int32_t py, const int32_t* q, real w[4]) {
    real sx[4], sy[4], a[4], d[4], r[4];
    for (int i = 0; i < 4; i++) {
        sx[i] = (real)wsub(q[2 * i], px);
        sy[i] = (real)wsub(q[2 * i + 1], py);
    }
    for (int i = 0; i < 4; i++) {
        int j = (i + 1) & 3;
        a[i] = sx[i] * sy[j] - sx[j] * sy[i];
        d[i] = sx[i] * sx[j] + sy[i] * sy[j];
        r[i] = sqrt(sx[i] * sx[i] + sy[i] * sy[i]);
    }
    for (int i = 0; i < 4; i++) {
        if (r[i] == 0) {
            for (int k = 0; k < 4; k++) w[k] = (k == i) ? K(1) : K(0);
            return;
        }
    }
    for (int i = 0; i < 4; i++)
        if (a[i] == 0) a[i] = (real)1e-3f;
    real t[4];
    for (int i = 0; i < 4; i++) {
        int j = (i + 1) & 3;
        t[i] = (r[i] * r[j] - d[i]) / a[i];
    }
    for (int i = 0; i < 4; i++) w[i] = (t[(i + 3) & 3] + t[i]) / r[i];
    real sum = w[0] + w[1] + w[2] + w[3];
    for (int i = 0; i < 4; i++) w[i] = w[i] / sum;
}

/* read_imagef with CLK_FILTER_LINEAR | CLK_NORMALIZED_COORDS_TRUE on a w x h image of
 * `ch`-float texels (channel c), per the OpenCL specification's filtering formula.
 * edge = 1: CLAMP_TO_EDGE; edge = 0: CLAMP (border 0). */
static real sample_linear(const float* tex, int w, int h, int ch, int c, real s, real t, int edge) {
    real u = s * (real)w - (real)0.5f, v = t * (real)h - (real)0.5f;
    if (!isfinite(u) || !isfinite(v)) return 0;
    real fu = floor(u), fv = floor(v);
    real a = u - fu, b = v - fv;
    long long i0 = cvt_rz_sat(fu), j0 = cvt_rz_sat(fv);
    long long i1 = i0 + 1, j1 = j0 + 1;
    real T[4];
    long long is[4] = {i0, i1, i0, i1}, js[4] = {j0, j0, j1, j1};
    for (int k = 0; k < 4; k++) {
        long long i = is[k], j = js[k];
        if (edge) {
            i = i < 0 ? 0 : (i >= w ? w - 1 : i);
            j = j < 0 ? 0 : (j >= h ? h - 1 : j);
            T[k] = (real)tex[((size_t)j * w + i) * ch + c];
        } else {
            T[k] = (i < 0 || i >= w || j < 0 || j >= h) ? K(0) : (real)tex[((size_t)j * w + i) * ch + c];
        }
    }
    return (K(1) - a) * (K(1) - b) * T[0] + a * (K(1) - b) * T[1] + (K(1) - a) * b * T[2] + a * b * T[3];
}

/* xyz_to_ap1, color.cl:3-10 (double literals: evaluated in double) */
static void xyz_to_ap1(const real in[3], float out[4]) {
    double x = (double)in[0], y = (double)in[1], z = (double)in[2];
    out[0] = (float)(1.6410233797 * x + -0.3248032942 * y + -0.2364246952 * z);
    out[1] = (float)(-0.6636628587 * x + 1.6153315917 * y + 0.0167563477 * z);
    out[2] = (float)(0.0117218943 * x + -0.0082844420 * y + 0.9883948585 * z);
    out[3] = 0.0f;
}

typedef struct { real px, py, ux, uy, rrel, refl, inten; } vtx_t;
static inline vtx_t load_vtx(const float* v) {
    vtx_t r = {(real)v[0], (real)v[1], (real)v[2], (real)v[3], (real)v[4], (real)v[5], (real)v[6]};
    return r;
}
static inline real mixr(real a, real b, real t) { return a + (b - a) * t; }

/* Contribution of one primitive to one pixel, rasterizing.cl:590-653. */
static void shade_prim(const float* vertexes, long long prim_id, const rf_raster_args* a,
                       const float* ghost, const float* spectrum, int x, int y, real rgb[3]) {
    const int G = a->grid_count, W = a->wavelength_count, WS = a->wavelength_sub_count;
    const int S = a->sub_steps;
    const int Q = (G - 1) * (G - 1), VC = G * G;
    const int maxW = W - 1 > 1 ? W - 1 : 1;
    const int32_t ppx = x * S, ppy = y * S;
    const int32_t pcx = ppx + S / 2, pcy = ppy + S / 2;
    const real sub_step = K(1) / (real)WS;
    const real wl_step = sub_step / (real)W;
    long long path = prim_id / Q;
    int quad = (int)(prim_id % Q);
    int row = quad / (G - 1), col = quad % (G - 1);
    long long vq[4];
    vq[0] = row * G + col;
    vq[1] = vq[0] + 1;
    vq[2] = vq[1] + G;
    vq[3] = vq[0] + G;
    long long vidx[4];
    for (int j = 0; j < 4; j++) vidx[j] = (path * VC + vq[j]) * W;
    vtx_t src[8];
    for (int j = 0; j < 4; j++) src[4 + j] = load_vtx(vertexes + 8 * vidx[j]);
    for (int j = 0; j < 4; j++) vidx[j]++;
    for (int w = 0; w < maxW; w++) {
        for (int j = 0; j < 4; j++) {
            src[j] = src[4 + j];
            src[4 + j] = load_vtx(vertexes + 8 * vidx[j]);
            vidx[j]++;
        }
        real sub_pos = 0;
        real wl_pos = ((real)w + (real)0.5f) / (real)W;
        for (int i = 0; i < WS; i++) {
            vtx_t v[4];
            int32_t q[8];
            for (int j = 0; j < 4; j++) {
                vtx_t s0 = src[j], s1 = src[j + 4];
                v[j].px = mixr(s0.px, s1.px, sub_pos);
                v[j].py = mixr(s0.py, s1.py, sub_pos);
                v[j].ux = mixr(s0.ux, s1.ux, sub_pos);
                v[j].uy = mixr(s0.uy, s1.uy, sub_pos);
                v[j].inten = mixr(s0.inten, s1.inten, sub_pos);
                v[j].rrel = mixr(s0.rrel, s1.rrel, sub_pos);
                v[j].refl = mixr(s0.refl, s1.refl, sub_pos);
                q[2 * j] = cvt_rz_sat(v[j].px * (real)S);
                q[2 * j + 1] = cvt_rz_sat(v[j].py * (real)S);
            }
            int hits = 0;
            for (int s = 0; s < S; s++) {
                if (intersect_quad(ppx + s, ppy + SUB_OFFSETS[S - 1 + s], q)) hits++;
            }
            real frag = 0;
            if (hits > 0) {
                real wt[4];
                barycentric_quad(pcx, pcy, q, wt);
                real u = wt[0] * v[0].ux + wt[1] * v[1].ux + wt[2] * v[2].ux + wt[3] * v[3].ux;
                real vv = wt[0] * v[0].uy + wt[1] * v[1].uy + wt[2] * v[2].uy + wt[3] * v[3].uy;
                u = (u / (real)a->ghost_scale + K(1)) / K(2);
                vv = (vv / (real)a->ghost_scale + K(1)) / K(2);
                real gi = sample_linear(ghost, a->ghost_width, a->ghost_height, 1, 0, u, vv, 0);
                real rr = wt[0] * v[0].rrel + wt[1] * v[1].rrel + wt[2] * v[2].rrel + wt[3] * v[3].rrel;
                real ri = smoothstep_r(K(1), (real)0.95f, rr);
                real ai = wt[0] * v[0].inten + wt[1] * v[1].inten + wt[2] * v[2].inten + wt[3] * v[3].inten;
                real ci = wt[0] * v[0].refl + wt[1] * v[1].refl + wt[2] * v[2].refl + wt[3] * v[3].refl;
                ai = rmax(ai, K(0));
                ci = rmax(ci, K(0));
                frag += gi * ri * ai * ci * (real)hits;
            }
            if (W > 1) {
                for (int c = 0; c < 3; c++)
                    rgb[c] += sample_linear(spectrum, RF_SPECTRUM_WIDTH, 1, 4, c, wl_pos, 0, 1) * frag;
            } else {
                for (int c = 0; c < 3; c++) rgb[c] += frag;
            }
            sub_pos += sub_step;
            wl_pos += wl_step;
        }
    }
}

static void finish_pixel(const rf_raster_args* a, int x, int y, const real rgb[3], float* image) {
    if (rgb[0] > 0 || rgb[1] > 0 || rgb[2] > 0) {
        const int total = a->wavelength_count * a->sub_steps * a->wavelength_sub_count;
        real scale = (real)a->intensity / (real)total;
        real v[3] = {rgb[0] * scale, rgb[1] * scale, rgb[2] * scale};
        float* out = image + 4 * ((size_t)(a->height - (y + 1)) * a->width + x);
        xyz_to_ap1(v, out);
    }
}

/* rfo_raster on a list of pixels (x, y pairs, unflipped) in one OpenMP region: each listed
 * pixel of the full-size image is cleared and shaded (sampled frames). */
int rfo_raster_pixels(const float* vertexes, const uint64_t* masks, int batch_count, const float* ghost,
                      const float* spectrum, const rf_raster_args* a, const int32_t* xy, long long count,
                      float* image) {
    const int B = a->bin_size;
    const int bdx = (a->width + B - 1) / B;
    const long long prim_total = (long long)a->path_count * (a->grid_count - 1) * (a->grid_count - 1);
#pragma omp parallel for schedule(dynamic, 1)
    for (long long i = 0; i < count; i++) {
        const int x = xy[2 * i], y = xy[2 * i + 1];
        const int bin = (y / B) * bdx + (x / B);
        real rgb[3] = {0, 0, 0};
        for (int batch = 0; batch < batch_count; batch++) {
            const uint64_t* q = masks + 4 * ((size_t)bin * batch_count + batch);
            if ((q[0] & 1u) == 0) continue;
            for (int k = 0; k < RF_BATCH_PRIMITIVE_COUNT; k++) {
                long long prim = (long long)batch * RF_BATCH_PRIMITIVE_COUNT + k;
                if (prim >= prim_total) continue;
                int bit = k + 1;
                if (!((q[bit >> 6] >> (bit & 63)) & 1u)) continue;
                shade_prim(vertexes, prim, a, ghost, spectrum, x, y, rgb);
            }
        }
        float* out = image + 4 * ((size_t)(a->height - (y + 1)) * a->width + x);
        out[0] = out[1] = out[2] = out[3] = 0;
        finish_pixel(a, x, y, rgb, image);
    }
    return 0;
}

/* Fragments (covered pixel x primitive x wavelength pair x sub-wavelength) of the
 * rasterizer, in its loop order, with their hit counts and mean-value weights: the frozen
 * coverage of finite-difference checks of the render's derivative. Writes at most capacity
 * fragments: pixel index y * width + x (unflipped), primitive, pair, sub-wavelength, hits and
 * 4 weights; returns the count. */
long long rfo_raster_fragments(const float* vertexes, const uint64_t* masks, int batch_count,
                               const rf_raster_args* a, long long capacity, int32_t* pixel, int64_t* prim_out,
                               int32_t* pair, int32_t* sub, int32_t* hits_out, double* weights) {
    const int B = a->bin_size;
    const int bdx = (a->width + B - 1) / B;
    const int G = a->grid_count, W = a->wavelength_count, WS = a->wavelength_sub_count, S = a->sub_steps;
    const int Q = (G - 1) * (G - 1), VC = G * G;
    const int maxW = W - 1 > 1 ? W - 1 : 1;
    const long long prim_total = (long long)a->path_count * Q;
    long long count = 0;
    for (int y = 0; y < a->height; y++) {
        for (int x = 0; x < a->width; x++) {
            int bin = (y / B) * bdx + (x / B);
            const int32_t ppx = x * S, ppy = y * S, pcx = ppx + S / 2, pcy = ppy + S / 2;
            for (int batch = 0; batch < batch_count; batch++) {
                const uint64_t* q = masks + 4 * ((size_t)bin * batch_count + batch);
                if ((q[0] & 1u) == 0) continue;
                for (int k = 0; k < RF_BATCH_PRIMITIVE_COUNT; k++) {
                    long long prim = (long long)batch * RF_BATCH_PRIMITIVE_COUNT + k;
                    if (prim >= prim_total) continue;
                    int bit = k + 1;
                    if (!((q[bit >> 6] >> (bit & 63)) & 1u)) continue;
                    long long path = prim / Q;
                    int quad = (int)(prim % Q), row = quad / (G - 1), col = quad % (G - 1);
                    long long vq[4] = {row * G + col, row * G + col + 1, row * G + col + 1 + G, row * G + col + G};
                    for (int w = 0; w < maxW; w++) {
                        real sub_pos = 0;
                        const real sub_step = K(1) / (real)WS;
                        for (int i = 0; i < WS; i++) {
                            int32_t qq[8];
                            for (int j = 0; j < 4; j++) {
                                const float* s0 = vertexes + 8 * ((path * VC + vq[j]) * W + w);
                                const float* s1 = s0 + 8;
                                qq[2 * j] = cvt_rz_sat(mixr((real)s0[0], (real)s1[0], sub_pos) * (real)S);
                                qq[2 * j + 1] = cvt_rz_sat(mixr((real)s0[1], (real)s1[1], sub_pos) * (real)S);
                            }
                            int hits = 0;
                            for (int s = 0; s < S; s++)
                                if (intersect_quad(ppx + s, ppy + SUB_OFFSETS[S - 1 + s], qq)) hits++;
                            if (hits > 0) {
                                if (count < capacity) {
                                    real wt[4];
                                    barycentric_quad(pcx, pcy, qq, wt);
                                    pixel[count] = y * a->width + x;
                                    prim_out[count] = prim;
                                    pair[count] = w;
                                    sub[count] = i;
                                    hits_out[count] = hits;
                                    for (int j = 0; j < 4; j++) weights[4 * count + j] = (double)wt[j];
                                }
                                count++;
                            }
                            sub_pos += sub_step;
                        }
                    }
                }
            }
        }
    }
    return count;
}

/* rasterizer kernel over the reference's bin masks, rasterizing.cl:524-663 */
int rfo_raster(const float* vertexes, const uint64_t* masks, int batch_count, const float* ghost,
               const float* spectrum, const rf_raster_args* a, float* image) {
    const int B = a->bin_size;
    const int bdx = (a->width + B - 1) / B;
    const long long prim_total = (long long)a->path_count * (a->grid_count - 1) * (a->grid_count - 1);
    memset(image, 0, sizeof(float) * 4 * (size_t)a->width * a->height);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < a->height; y++) {
        for (int x = 0; x < a->width; x++) {
            int bin = (y / B) * bdx + (x / B);
            real rgb[3] = {0, 0, 0};
            for (int batch = 0; batch < batch_count; batch++) {
                const uint64_t* q = masks + 4 * ((size_t)bin * batch_count + batch);
                if ((q[0] & 1u) == 0) continue;
                for (int k = 0; k < RF_BATCH_PRIMITIVE_COUNT; k++) {
                    long long prim = (long long)batch * RF_BATCH_PRIMITIVE_COUNT + k;
                    if (prim >= prim_total) continue;
                    int bit = k + 1;
                    if (!((q[bit >> 6] >> (bit & 63)) & 1u)) continue;
                    shade_prim(vertexes, prim, a, ghost, spectrum, x, y, rgb);
                }
            }
            finish_pixel(a, x, y, rgb, image);
        }
    }
    return 0;
}

/* Rasterise pixels [x0, x1) x [y0, y1) only (CPU baseline samples). */
int rfo_raster_rows(const float* vertexes, const uint64_t* masks, int batch_count, const float* ghost,
                    const float* spectrum, const rf_raster_args* a, float* image, int y0, int y1, int x0, int x1) {
    const int B = a->bin_size;
    const int bdx = (a->width + B - 1) / B;
    const long long prim_total = (long long)a->path_count * (a->grid_count - 1) * (a->grid_count - 1);
    if (x1 <= 0 || x1 > a->width) x1 = a->width;
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int y = y0; y < y1; y++) {
        for (int x = x0; x < x1; x++) {
            int bin = (y / B) * bdx + (x / B);
            real rgb[3] = {0, 0, 0};
            for (int batch = 0; batch < batch_count; batch++) {
                const uint64_t* q = masks + 4 * ((size_t)bin * batch_count + batch);
                if ((q[0] & 1u) == 0) continue;
                for (int k = 0; k < RF_BATCH_PRIMITIVE_COUNT; k++) {
                    long long prim = (long long)batch * RF_BATCH_PRIMITIVE_COUNT + k;
                    if (prim >= prim_total) continue;
                    int bit = k + 1;
                    if (!((q[bit >> 6] >> (bit & 63)) & 1u)) continue;
                    shade_prim(vertexes, prim, a, ghost, spectrum, x, y, rgb);
                }
            }
            float* out = image + 4 * ((size_t)(a->height - (y + 1)) * a->width + x);
            out[0] = out[1] = out[2] = out[3] = 0;
            finish_pixel(a, x, y, rgb, image);
        }
    }
    return 0;
}

/* ---------------------------------------------------------------- aperture / starburst
 * noise.cl:1-5, geometry.cl:1-48, aperture.cl:1-47,139-174, starburst.cl:1-87 */
static real fract_r(real x) { return fmin(x - floor(x), (real)0x1.fffffep-1f); }
static real noise3(real x, real y, real z) {
    return fract_r(sin(x * (real)112.9898f + y * (real)179.233f + z * (real)237.212f) * (real)43758.5453f);
}
static void ndc_of(int px, int py, int w, int h, real* nx, real* ny) {
    *nx = K(2) * ((real)px / (real)(w - 1)) - K(1);
    *ny = K(2) * ((real)py / (real)(h - 1)) - K(1);
}
static void rot2(real* x, real* y, real angle) {
    real s = sin(angle), c = cos(angle);
    real nx = *x * c + *y * s, ny = *y * c - *x * s;
    *x = nx;
    *y = ny;
}

int rfo_aperture_shape(float* image, int w, int h, float size_x, float size_y, int blades,
                       float rotation, float roundness, float softness) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            real px, py;
            ndc_of(x, y, w, h, &px, &py);
            px = px / rmax((real)size_x, (real)FLT_MIN);
            py = py / rmax((real)size_y, (real)FLT_MIN);
            rot2(&px, &py, (real)rotation);
            real sdf = 0;
            for (int i = 0; i < blades; i++) {
                real angle = ((real)i / (real)blades + (real)0.25f) * K(2) * M_PI_R;
                sdf = rmax(sdf, cos(angle) * px + sin(angle) * py);
            }
            real cg = atan2(-px, -py) / (K(2) * M_PI_R) + (real)0.5f;
            real bg = fmod(cg * (real)blades + (real)0.5f, K(1));
            real rg = sin(bg * M_PI_R);
            sdf += rg * (real)roundness;
            real s = (real)softness;
            image[(size_t)y * w + x] = (float)(K(1) - smoothstep_r(K(1) - s, K(1) + s, sdf));
        }
    }
    return 0;
}

static real wrap1(real v) { return fmod(K(1) + fmod(v, K(1)), K(1)); }

int rfo_aperture_dust(float* image, int w, int h, float size_x, float size_y, float strength,
                      float density, float radius, float par_x, float par_y, float softness) {
    int count = (int)(rmin((real)density, K(1)) * K(1000));
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            real px, py;
            ndc_of(x, y, w, h, &px, &py);
            px = px / rmax((real)size_x, (real)FLT_MIN);
            py = py / rmax((real)size_y, (real)FLT_MIN);
            real sdf = 1;
            for (int i = 0; i < count; i++) {
                real cx = noise3((real)i, (real)count, 0) + (real)par_x;
                real cy = noise3((real)i, (real)count, 1) + (real)par_y;
                cx = wrap1(cx) * K(2) - K(1);
                cy = wrap1(cy) * K(2) - K(1);
                real dx = px - cx, dy = py - cy;
                sdf = rmin(sdf, sqrt(dx * dx + dy * dy) - (real)radius);
            }
            real s = (real)softness;
            real inten = (real)image[(size_t)y * w + x];
            inten *= K(1) - ((real)strength * smoothstep_r(s, -s, sdf));
            image[(size_t)y * w + x] = (float)inten;
        }
    }
    return 0;
}

/* Blurred-noise dust (no reference counterpart), the definition rf_aperture_noise_dust
 * implements: separable Gaussian, radius ceil(4 sigma), weights exp(-k^2 / (2 sigma^2))
 * normalised to sum 1, clamp-to-edge; rows first, then columns. */
int rfo_aperture_noise_dust(float* image, const float* noise, int w, int h, float strength, float sigma) {
    int rad = (int)ceil((double)sigma * 4.0);
    if (rad < 0) rad = 0;
    real* wts = (real*)malloc(sizeof(real) * (2 * rad + 1));
    real sum = 0;
    for (int k = -rad; k <= rad; k++) {
        wts[k + rad] = sigma > 0 ? exp(-(real)(k * k) / (K(2) * (real)sigma * (real)sigma)) : K(1);
        sum += wts[k + rad];
    }
    for (int k = 0; k <= 2 * rad; k++) wts[k] = wts[k] / sum;
    real* tmp = (real*)malloc(sizeof(real) * (size_t)w * h);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            real acc = 0;
            for (int k = -rad; k <= rad; k++) {
                int xx = x + k;
                xx = xx < 0 ? 0 : (xx >= w ? w - 1 : xx);
                acc += wts[k + rad] * (real)noise[(size_t)y * w + xx];
            }
            tmp[(size_t)y * w + x] = acc;
        }
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            real acc = 0;
            for (int k = -rad; k <= rad; k++) {
                int yy = y + k;
                yy = yy < 0 ? 0 : (yy >= h ? h - 1 : yy);
                acc += wts[k + rad] * tmp[(size_t)yy * w + x];
            }
            image[(size_t)y * w + x] = (float)((real)image[(size_t)y * w + x] * (K(1) - (real)strength * acc));
        }
    free(tmp);
    free(wts);
    return 0;
}

/* starburst kernel, starburst.cl:1-87. spectrum: count x (sh x sw) floats. */
int rfo_starburst(const float* spectrum, const float* light_spectrum, const rf_starburst_args* a,
                  float* image, int y0, int y1) {
    const int w = a->width, h = a->height;
    if (y1 <= 0 || y1 > h) y1 = h;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = y0; y < y1; y++) {
        for (int x = 0; x < w; x++) {
            real nx, ny;
            ndc_of(x, y, w, h, &nx, &ny);
            nx = nx - (real)a->offset[0];
            ny = ny - (real)a->offset[1];
            nx = nx / rmax((real)a->scale[0], (real)FLT_MIN);
            ny = ny / rmax((real)a->scale[1], (real)FLT_MIN);
            real acc[4] = {0, 0, 0, 0};
            for (int t = 0; t < a->samples; t++) {
                real step = (real)t / (real)a->samples;
                real wavelength = step * (real)(RF_LAMBDA_MAX - RF_LAMBDA_MIN) + (real)RF_LAMBDA_MIN;
                real seed = (real)(t * 4);
                real px = nx, py = ny;
                real radius = (real)a->blur * sqrt(noise3((real)x, (real)y, seed));
                real alpha = noise3((real)x, (real)y, seed + K(1)) * K(2) * M_PI_R;
                px += cos(alpha) * radius;
                py += sin(alpha) * radius;
                real sc = K(1) - (K(1) - (wavelength / (real)RF_LAMBDA_MID)) * K(1);
                sc = rmax(sc, (real)FLT_MIN);
                px = px / sc;
                py = py / sc;
                real sign = (noise3((real)x, (real)y, seed + K(2)) > (real)0.5f) ? K(1) : K(-1);
                real angle = sign * (real)a->rotation *
                             (K(1) - pow(noise3((real)x, (real)y, seed + K(3)), (real)a->rotation_weight));
                rot2(&px, &py, angle);
                real u = px * (real)0.5f + (real)0.5f;
                real v = py * (real)0.5f + (real)0.5f;
                int sidx = 0;
                if (a->spectrum_count > 1) {
                    real f = (wavelength - (real)a->lambda_first) / (real)a->lambda_step;
                    int k = cvt_rz_sat(floor(f + (real)0.5f));
                    sidx = k < 0 ? 0 : (k >= a->spectrum_count ? a->spectrum_count - 1 : k);
                }
                const float* spec = spectrum + (size_t)sidx * a->spectrum_width * a->spectrum_height;
                real fi = sample_linear(spec, a->spectrum_width, a->spectrum_height, 1, 0, u, v, 0);
                for (int c = 0; c < 4; c++)
                    acc[c] += sample_linear(light_spectrum, RF_SPECTRUM_WIDTH, 1, 4, c, step, 0, 0) * fi;
            }
            for (int c = 0; c < 4; c++) acc[c] = acc[c] / (real)a->samples;
            if (!isnan(a->vignetting[0])) {
                real sdf = sqrt(nx * nx + ny * ny) - K(0);
                real f = smoothstep_r((real)a->vignetting[1], (real)a->vignetting[0], sdf);
                for (int c = 0; c < 4; c++) acc[c] *= f;
            }
            for (int c = 0; c < 4; c++) acc[c] *= (real)a->intensity;
            float* out = image + 4 * ((size_t)y * w + x);
            xyz_to_ap1(acc, out);
        }
    }
    return 0;
}

/* ---------------------------------------------------------------- lens diagram
 * DiagramTask (realflare/api/tasks/diagram.py:24-228): the kernels lenses
 * (realflare/api/tasks/cl/diagram.cl:21-67) and intersections (70-138) in FP32, one after
 * the other per pixel. pow(v, 2) is taken as v * v. inter: rays * count records of 8 floats
 * (rfo_trace_intersections); the record after the last one reads as unused. */
static int diagram_is_line(float posx, float posy, float p0x, float p0y, float p1x, float p1y, float width) {
    float vx = p1x - p0x, vy = p1y - p0y;
    float ax = posx - p0x, ay = posy - p0y;
    float bx = posx - p1x, by = posy - p1y;
    int between = (vx * ax + vy * ay) > 0.0f && (vx * bx + vy * by) < 0.0f;
    float d = fabsf(vx * ay - ax * vy) / sqrtf(vx * vx + vy * vy);
    return between && d <= width / 2.0f;
}

static int diagram_hit(const float* inter, long long i, long long total) {
    int32_t h = 0;
    if (i < total) memcpy(&h, inter + 8 * i + 7, sizeof h);
    return h != 0;
}

int rfo_diagram(const rf_lens_element* el, int E, int aperture, float scale, const float* inter, int rays,
                int count, int width, int height, float* image) {
    const long long total = inter ? (long long)rays * count : 0;
#pragma omp parallel for schedule(static)
    for (int py = 0; py < height; py++) {
        for (int px = 0; px < width; px++) {
            float x = (float)px, y = (float)(height / 2 - py);
            float rgba[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if ((int)y == 0) rgba[0] = 1.0f;
            for (int i = 0; i < E; i++) {
                float r = el[i].radius * scale, h = el[i].height * scale, c = el[i].center * scale;
                if (r == 0.0f && fabsf(y) < h && (int)x == (int)c) {
                    if (i == aperture || i == E - 1) rgba[1] = 1.0f;
                    else rgba[2] = 1.0f;
                    break;
                }
                float ex = x - c;
                float r_circle = sqrtf(ex * ex + y * y);
                int draw_half = (r > 0.0f) ? (x < c) : (x > c);
                if (draw_half && (int)fabsf(r) == (int)r_circle && fabsf(y) < h) rgba[2] = 1.0f;
            }
            for (int ray = 0; inter && ray < rays; ray++) {
                for (int k = 0; k < count; k++) {
                    long long i1 = (long long)ray * count + k;
                    if (!diagram_hit(inter, i1 + 1, total)) break;
                    const float* s = inter + 8 * i1;
                    const float* t = s + 8;
                    float p0x = (s[2] * scale) * -1.0f, p0y = (s[1] * scale) * -1.0f;
                    float p1x = (t[2] * scale) * -1.0f, p1y = (t[1] * scale) * -1.0f;
                    float nx = s[5] * scale, ny = s[4] * scale;
                    if (diagram_is_line(x, y, p0x, p0y, p0x - nx * 1.0f, p0y - ny * 1.0f, 1.0f)) {
                        rgba[0] = 0.25f;
                        rgba[1] = rgba[2] = rgba[3] = 0.0f;
                    }
                    if (p1x == 0.0f) break;
                    if (diagram_is_line(x, y, p0x, p0y, p1x, p1y, 1.0f)) {
                        rgba[0] += 0.25f;
                        rgba[1] += 0.25f;
                        rgba[2] += 0.25f;
                    }
                }
            }
            memcpy(image + 4 * ((size_t)py * width + px), rgba, sizeof rgba);
        }
    }
    return 0;
}
