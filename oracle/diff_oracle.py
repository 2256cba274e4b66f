"""FP64 finite-difference oracle of the differentiable render (test infrastructure only).

The render's gradient holds coverage fixed (which pixels each quad covers, its hit counts
and mean-value weights: piecewise constant in the vertex positions, which the reference
truncates to integer samples). The matching function to difference is the image with that
coverage frozen: ``FrozenRender`` takes the fragments of a base render (the C oracle's
rasteriser loop, ``rfo_raster_fragments``), and for any lens geometry and light direction
re-evaluates in FP64 the trace (``rfo_trace_geom_d`` of the FP64 build), the quad
intensities (prim_shader, rasterizing.cl:233-320), the vertex attributes (vertex_shader,
rasterizing.cl:322-386) and every frozen fragment's shading (fragment_shader,
rasterizing.cl:471-506, mix_vertex 509-522, the colour and output of 604-662).
"""
from __future__ import annotations

import ctypes

import numpy as np

from .oracle import Oracle, _c, _ptr

XYZ_TO_AP1 = np.array([[1.6410233797, -0.3248032942, -0.2364246952],
                       [-0.6636628587, 1.6153315917, 0.0167563477],
                       [0.0117218943, -0.0082844420, 0.9883948585]])


def _lib(variant):
    o = Oracle(variant)
    lib = o.lib
    if not hasattr(lib, '_diff_ready'):
        from realflare_gb300._abi import RasterArgs, TraceArgs

        P = ctypes.c_void_p
        lib.rfo_trace_geom_d.argtypes = [P, P, P, ctypes.POINTER(TraceArgs), P, P, P]
        lib.rfo_raster_fragments.argtypes = [P, P, ctypes.c_int, ctypes.POINTER(RasterArgs), ctypes.c_longlong,
                                             P, P, P, P, P, P]
        lib.rfo_raster_fragments.restype = ctypes.c_longlong
        lib._diff_ready = True
    return o


def trace_geom(elements, paths, wavelengths, args, geom: np.ndarray, dir3: np.ndarray) -> np.ndarray:
    """FP64 trace with geometry (E x 4: radius, center, thickness 0, 1) and the light
    direction in double; outputs (6, n) double."""
    o = _lib('f64')
    n = args.path_count * args.wavelength_count * args.grid_count ** 2
    out = np.zeros((6, n), np.float64)
    g = np.ascontiguousarray(geom, np.float64)
    d = np.ascontiguousarray(dir3, np.float64)
    o.lib.rfo_trace_geom_d(_ptr(_c(elements, elements.dtype)), _ptr(_c(paths, np.int32)),
                           _ptr(_c(wavelengths, np.float32)), ctypes.byref(args), _ptr(g), _ptr(d), _ptr(out))
    return out


def fragments(vertexes, masks, args) -> dict:
    """The rasteriser's fragments of a base render (FP32 oracle: the GPU's coverage)."""
    o = _lib('f32')
    v = _c(vertexes, np.float32)
    m = _c(masks, np.uint64)
    cap = 1 << 16
    while True:
        out = {'pixel': np.zeros(cap, np.int32), 'prim': np.zeros(cap, np.int64), 'pair': np.zeros(cap, np.int32),
               'sub': np.zeros(cap, np.int32), 'hits': np.zeros(cap, np.int32), 'w': np.zeros((cap, 4), np.float64)}
        n = o.lib.rfo_raster_fragments(_ptr(v), _ptr(m), masks.shape[1], ctypes.byref(args), cap,
                                       *[_ptr(out[k]) for k in ('pixel', 'prim', 'pair', 'sub', 'hits', 'w')])
        if n <= cap:
            return {k: a[:n] for k, a in out.items()}
        cap = int(n) + 1


def _sample_linear_edge(tex: np.ndarray, s: np.ndarray) -> np.ndarray:
    """read_imagef LINEAR, CLAMP_TO_EDGE on a 1-row texture (the CIE table), channels last."""
    w = tex.shape[0]
    u = s * w - 0.5
    fu = np.floor(u)
    a = u - fu
    i0 = np.clip(fu.astype(np.int64), 0, w - 1)
    i1 = np.clip(fu.astype(np.int64) + 1, 0, w - 1)
    return (1 - a)[..., None] * tex[i0] + a[..., None] * tex[i1]


def _bilinear_border(tex: np.ndarray, u: np.ndarray, v: np.ndarray) -> np.ndarray:
    h, w = tex.shape
    ok = np.isfinite(u) & np.isfinite(v) & (np.abs(u) < 1e9) & (np.abs(v) < 1e9)
    u = np.where(ok, u, 0.0)
    v = np.where(ok, v, 0.0)
    fu, fv = np.floor(u), np.floor(v)
    a, b = u - fu, v - fv
    i0, j0 = fu.astype(np.int64), fv.astype(np.int64)

    def t(i, j):
        inside = (i >= 0) & (i < w) & (j >= 0) & (j < h)
        return np.where(inside, tex[np.clip(j, 0, h - 1), np.clip(i, 0, w - 1)], 0.0)
    g = (1 - a) * (1 - b) * t(i0, j0) + a * (1 - b) * t(i0 + 1, j0) + (1 - a) * b * t(i0, j0 + 1) + a * b * t(i0 + 1, j0 + 1)
    return np.where(ok, g, 0.0)


class FrozenRender:
    """The image as a function of the lens geometry and light direction, coverage frozen."""

    def __init__(self, trace_inputs, raster_args, frags: dict, ghost: np.ndarray, spectrum: np.ndarray,
                 area_orig: float, min_area: float, lit: np.ndarray) -> None:
        self.ti = trace_inputs
        self.ra = raster_args
        self.f = frags
        self.ghost = np.asarray(ghost, np.float64)
        self.spectrum = np.asarray(spectrum, np.float64).reshape(-1, 4)[:, :3]
        self.area_orig, self.min_area = float(area_orig), float(min_area)
        self.lit = lit  # (h, w) bool: pixels the base render wrote (any channel > 0)

    def image(self, geom: np.ndarray, dir3: np.ndarray) -> np.ndarray:
        ti, ra = self.ti, self.ra
        P, W, G = ra.path_count, ra.wavelength_count, ra.grid_count
        R, Q, VC = G * G, (G - 1) ** 2, G * G
        rays = trace_geom(ti.elements, ti.paths, ti.wavelengths, ti.args, geom, dir3)
        px, py = rays[0].reshape(P, W, G, G), rays[1].reshape(P, W, G, G)
        refl = rays[5].reshape(P, W, G, G)
        ok = ~np.isnan(refl)
        # prim_shader intensities, rasterizing.cl:233-320 (compaction of valid corners)
        corner = lambda A: np.stack([A[:, :, :-1, :-1], A[:, :, :-1, 1:], A[:, :, 1:, 1:], A[:, :, 1:, :-1]], 0)
        cx, cy, cok = corner(px), corner(py), corner(ok)  # (4, P, W, G-1, G-1)
        order = np.argsort(~cok, axis=0, kind='stable')
        sx, sy = np.take_along_axis(cx, order, 0), np.take_along_axis(cy, order, 0)
        nval = cok.sum(0)

        def e(a, b, c):
            return (sx[a] - sx[b]) * (sy[c] - sy[a]) - (sy[a] - sy[b]) * (sx[c] - sx[a])
        with np.errstate(invalid='ignore'):
            area = np.where(nval == 4, np.abs(e(0, 1, 2) + e(0, 2, 3)) / 2, np.abs(e(0, 1, 2)))
        culled = np.cumsum(nval < 3, axis=1) > 0  # a degenerate wavelength culls the later ones
        area_actual = np.maximum(np.nan_to_num(area), self.min_area)
        inten = np.where(culled | (area_actual <= 0), 0.0, self.area_orig / np.where(area_actual > 0, area_actual, 1))
        inten = inten.reshape(P, W, Q)
        # vertex_shader, rasterizing.cl:322-386: mean of the positive neighbour intensities
        yy, xx = np.divmod(np.arange(R), G)
        nb = np.stack([(yy - 1) * (G - 1) + (xx - 1), (yy - 1) * (G - 1) + xx, yy * (G - 1) + (xx - 1),
                       yy * (G - 1) + xx], 0)  # (4, R)
        inr = (nb >= 0) & (nb < Q)
        vals = np.where(inr[None, None], inten[:, :, np.clip(nb, 0, Q - 1)], 0.0)  # (P, W, 4, R)
        pos = vals > 0
        cnt = pos.sum(2)
        vint = np.where(pos, vals, 0).sum(2) / np.maximum(cnt, 1)
        okr = ok.reshape(P, W, R)
        attrs = np.stack([rays[2].reshape(P, W, R), rays[3].reshape(P, W, R), rays[4].reshape(P, W, R),
                          rays[5].reshape(P, W, R), vint], -1)  # u, v, rrel, refl, inten
        attrs = np.where(okr[..., None], attrs, 0.0)
        attrs[..., 3] = np.where(okr, attrs[..., 3], np.nan)
        # vertex buffer order (path, ray, wavelength) + the zero vertex after the last
        vert = np.concatenate([attrs.transpose(0, 2, 1, 3).reshape(-1, 5), np.zeros((1, 5))], 0)
        # frozen fragments
        f = self.f
        prim = f['prim']
        path, quad = prim // Q, prim % Q
        row, col = quad // (G - 1), quad % (G - 1)
        c0 = row * G + col
        corners = np.stack([c0, c0 + 1, c0 + 1 + G, c0 + G], 1)  # (n, 4)
        vi = (path[:, None] * VC + corners) * W + f['pair'][:, None]
        t = f['sub'] / ra.wavelength_sub_count
        a0, a1 = vert[vi], vert[vi + 1]  # (n, 4, 5)
        mix = a0 + (a1 - a0) * t[:, None, None]
        wt = f['w']
        it = np.einsum('nk,nka->na', wt, mix)  # interpolated u, v, rrel, refl, inten
        tex_u = (it[:, 0] / ra.ghost_scale + 1) / 2 * ra.ghost_width - 0.5
        tex_v = (it[:, 1] / ra.ghost_scale + 1) / 2 * ra.ghost_height - 0.5
        gi = _bilinear_border(self.ghost, tex_u, tex_v)
        st = np.clip((it[:, 2] - 1.0) / (0.95 - 1.0), 0.0, 1.0)
        st = np.nan_to_num(st)
        ri = st * st * (3 - 2 * st)
        ai = np.where(it[:, 4] > 0, it[:, 4], 0.0)
        ci = np.where(it[:, 3] > 0, it[:, 3], 0.0)
        frag = gi * ri * ai * ci * f['hits']
        if W > 1:
            WS = ra.wavelength_sub_count
            pos_c = (f['pair'] + 0.5) / W + f['sub'] * (1.0 / WS / W)
            col = _sample_linear_edge(self.spectrum, pos_c)
        else:
            col = np.ones((len(frag), 3))
        rgb = np.zeros((ra.height * ra.width, 3))
        np.add.at(rgb, f['pixel'], col * frag[:, None])
        scale = ra.intensity / (W * ra.sub_steps * ra.wavelength_sub_count)
        out = (rgb * scale) @ XYZ_TO_AP1.T
        out = out.reshape(ra.height, ra.width, 3)[::-1]  # row 0 = top
        return np.where(self.lit[..., None], out, 0.0)
