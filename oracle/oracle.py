"""Python front-end of the oracles (test infrastructure only).

* ``Oracle('f32' | 'f64')``: the C restatement ``oracle/rf_oracle.c`` (float / double).
* ``Reference()``: the reference's own OpenCL kernels compiled for the host
  (``oracle/_ref``, see ``oracle/build_ref.py``), driven like the reference's Python tasks.
* ``fft_power_spectrum`` / ``ghost_frft``: numpy float64 restatements of
  ``realflare/api/tasks/starburst.py:45-81`` and ``realflare/api/tasks/ghost.py:13-36`` with
  ``realflare/utils/frft.py:8-62``.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use this.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from realflare_gb300._abi import RasterArgs, StarburstArgs, TraceArgs

from . import build_oracle, build_ref

_P = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_F = ctypes.c_float


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def _c(a, dtype) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


class Oracle:
    """The C restatement, FP32 (``'f32'``) or FP64 (``'f64'``)."""

    _libs: dict = {}

    def __init__(self, variant: str = 'f32') -> None:
        if variant not in self._libs:
            build_oracle.build()
            lib = ctypes.CDLL(build_oracle.lib_path(variant))
            lib.rfo_trace.argtypes = [_P, _P, _P, ctypes.POINTER(TraceArgs), _P]
            lib.rfo_trace_range.argtypes = [_P, _P, _P, ctypes.POINTER(TraceArgs), _P, _LL, _LL]
            lib.rfo_trace_d.argtypes = [_P, _P, _P, ctypes.POINTER(TraceArgs), _P]
            lib.rfo_quad_setup.argtypes = [_P, _I, _I, _I, _F, _F, _P, _P]
            lib.rfo_vertex.argtypes = [_P, _P, _I, _I, _I, _F, _I, _I, _P]
            lib.rfo_bin_masks.argtypes = [_P, _I, _F, _I, _I, _I, _P]
            lib.rfo_raster.argtypes = [_P, _P, _I, _P, _P, ctypes.POINTER(RasterArgs), _P]
            lib.rfo_raster_rows.argtypes = [_P, _P, _I, _P, _P, ctypes.POINTER(RasterArgs), _P, _I, _I, _I, _I]
            lib.rfo_raster_pixels.argtypes = [_P, _P, _I, _P, _P, ctypes.POINTER(RasterArgs), _P, _LL, _P]
            lib.rfo_aperture_shape.argtypes = [_P, _I, _I, _F, _F, _I, _F, _F, _F]
            lib.rfo_aperture_dust.argtypes = [_P, _I, _I, _F, _F, _F, _F, _F, _F, _F, _F]
            lib.rfo_aperture_noise_dust.argtypes = [_P, _P, _I, _I, _F, _F]
            lib.rfo_starburst.argtypes = [_P, _P, ctypes.POINTER(StarburstArgs), _P, _I, _I]
            lib.rfo_trace_intersections.argtypes = [_P, _P, _P, ctypes.POINTER(TraceArgs), _P, _P, _I]
            lib.rfo_diagram.argtypes = [_P, _I, _I, _F, _P, _I, _I, _I, _I, _P]
            self._libs[variant] = lib
        self.lib = self._libs[variant]

    def trace(self, elements, paths, wavelengths, args: TraceArgs, first=None, count=None):
        R = args.grid_count**2
        n = args.path_count * args.wavelength_count * R
        out = np.zeros((6, n), np.float32)
        el = _c(elements, elements.dtype)
        pa = _c(paths, np.int32)
        wl = _c(wavelengths, np.float32)
        if first is None:
            self.lib.rfo_trace(_ptr(el), _ptr(pa), _ptr(wl), ctypes.byref(args), _ptr(out))
        else:
            self.lib.rfo_trace_range(_ptr(el), _ptr(pa), _ptr(wl), ctypes.byref(args), _ptr(out), first, count)
        return out

    def trace_d(self, elements, paths, wavelengths, args: TraceArgs):
        """trace() with the outputs in double (for finite differences of the FP64 build)."""
        n = args.path_count * args.wavelength_count * args.grid_count**2
        out = np.zeros((6, n), np.float64)
        el = _c(elements, elements.dtype)
        self.lib.rfo_trace_d(_ptr(el), _ptr(_c(paths, np.int32)), _ptr(_c(wavelengths, np.float32)),
                             ctypes.byref(args), _ptr(out))
        return out

    def trace_intersections(self, elements, paths, wavelengths, args: TraceArgs, count: int):
        """(rays [6, n], hits [n, count, 8] float32: pos xyz, normal xyz, incident, hit as int32)."""
        n = args.path_count * args.wavelength_count * args.grid_count**2
        rays = np.zeros((6, n), np.float32)
        inter = np.zeros((n, count, 8), np.float32)
        self.lib.rfo_trace_intersections(_ptr(_c(elements, elements.dtype)), _ptr(_c(paths, np.int32)),
                                         _ptr(_c(wavelengths, np.float32)), ctypes.byref(args), _ptr(rays),
                                         _ptr(inter), count)
        return rays, inter

    def diagram(self, elements, aperture_index, scale, inter, width, height):
        """The lens diagram (height, width, 4); inter: [rays, count, 8] records or None."""
        image = np.zeros((height, width, 4), np.float32)
        el = _c(elements, elements.dtype)
        if inter is None:
            self.lib.rfo_diagram(_ptr(el), len(el), aperture_index, scale, None, 0, 0, width, height, _ptr(image))
        else:
            rec = _c(inter, np.float32)
            self.lib.rfo_diagram(_ptr(el), len(el), aperture_index, scale, _ptr(rec), rec.shape[0], rec.shape[1],
                                 width, height, _ptr(image))
        return image

    def quad_setup(self, rays, P, W, G, area_orig, min_area):
        Q = (G - 1) ** 2
        bounds = np.zeros((P * Q, 4), np.float32)
        inten = np.zeros(P * Q * W, np.float32)
        r = _c(rays, np.float32)
        self.lib.rfo_quad_setup(_ptr(r), P, W, G, area_orig, min_area, _ptr(bounds), _ptr(inten))
        return bounds, inten

    def vertex(self, rays, intensities, P, W, G, st, width, height):
        n = P * W * G * G
        out = np.zeros((n + 1, 8), np.float32)
        self.lib.rfo_vertex(_ptr(_c(rays, np.float32)), _ptr(_c(intensities, np.float32)), P, W, G, st,
                            width, height, _ptr(out))
        return out

    def bin_masks(self, bounds, st, width, height, bin_size):
        prims = bounds.shape[0]
        bins = ((width + bin_size - 1) // bin_size) * ((height + bin_size - 1) // bin_size)
        batches = (prims + 254) // 255
        masks = np.zeros((bins, batches, 4), np.uint64)
        self.lib.rfo_bin_masks(_ptr(_c(bounds, np.float32)), prims, st, width, height, bin_size, _ptr(masks))
        return masks

    def raster(self, vertexes, masks, ghost, spectrum, args: RasterArgs, rows=None, cols=(0, 0)):
        image = np.zeros((args.height, args.width, 4), np.float32)
        v = _c(vertexes, np.float32)
        m = _c(masks, np.uint64)
        g = _c(ghost, np.float32)
        s = _c(spectrum, np.float32)
        if rows is None:
            self.lib.rfo_raster(_ptr(v), _ptr(m), masks.shape[1], _ptr(g), _ptr(s), ctypes.byref(args), _ptr(image))
        else:
            self.lib.rfo_raster_rows(_ptr(v), _ptr(m), masks.shape[1], _ptr(g), _ptr(s), ctypes.byref(args),
                                     _ptr(image), rows[0], rows[1], cols[0], cols[1])
        return image

    def raster_pixels(self, vertexes, masks, ghost, spectrum, args: RasterArgs, xy, image=None):
        """raster() of the listed pixels only ((n, 2) int x, y, unflipped), one parallel
        region; returns the full-size image with those pixels set (others as given, or 0)."""
        if image is None:
            image = np.zeros((args.height, args.width, 4), np.float32)
        xy = _c(xy, np.int32)
        self.lib.rfo_raster_pixels(_ptr(_c(vertexes, np.float32)), _ptr(_c(masks, np.uint64)), masks.shape[1],
                                   _ptr(_c(ghost, np.float32)), _ptr(_c(spectrum, np.float32)), ctypes.byref(args),
                                   _ptr(xy), len(xy), _ptr(image))
        return image

    def aperture_shape(self, w, h, size, blades, rotation, roundness, softness):
        out = np.zeros((h, w), np.float32)
        self.lib.rfo_aperture_shape(_ptr(out), w, h, size[0], size[1], blades, rotation, roundness, softness)
        return out

    def aperture_dust(self, image, size, strength, density, radius, parallax, softness):
        out = _c(image, np.float32).copy()
        h, w = out.shape
        self.lib.rfo_aperture_dust(_ptr(out), w, h, size[0], size[1], strength, density, radius,
                                   parallax[0], parallax[1], softness)
        return out

    def aperture_noise_dust(self, image, noise, strength, sigma):
        out = _c(image, np.float32).copy()
        h, w = out.shape
        self.lib.rfo_aperture_noise_dust(_ptr(out), _ptr(_c(noise, np.float32)), w, h, strength, sigma)
        return out

    def starburst(self, spectrum, light_spectrum, args: StarburstArgs, rows=None):
        out = np.zeros((args.height, args.width, 4), np.float32)
        y0, y1 = rows if rows is not None else (0, args.height)
        self.lib.rfo_starburst(_ptr(_c(spectrum, np.float32)), _ptr(_c(light_spectrum, np.float32)),
                               ctypes.byref(args), _ptr(out), y0, y1)
        return out


class Reference:
    """The reference's own kernels compiled for the host (``oracle/_ref``)."""

    _lib = None

    @classmethod
    def available(cls) -> bool:
        try:
            cls()
            return True
        except (OSError, RuntimeError):
            return False

    def __init__(self) -> None:
        if Reference._lib is None:
            path = build_ref.build()
            if path is None:
                raise RuntimeError('reference kernels unavailable (no checkout and no generated sources)')
            lib = ctypes.CDLL(path)
            lib.ref_trace.argtypes = [_P, _I, _P, _I, _P, _I, _I, _F, _I, _F, _P, _P, _LL, _LL]
            lib.ref_prim_shader.argtypes = [_P, _I, _I, _I, _F, _F, _P, _P]
            lib.ref_vertex_shader.argtypes = [_P, _P, _I, _I, _I, _F, _I, _I, _P]
            lib.ref_binner.argtypes = [_P, _I, _F, _I, _I, _I, _I, _P]
            lib.ref_rasterizer.argtypes = [_P, _P, _I, _P, _I, _I, _P, _I, _I, _I, _I, _I, _F, _F, _I, _I, _I,
                                           _I, _I, _I, _I, _P]
            lib.ref_rasterizer_pixels.argtypes = [_P, _P, _I, _P, _I, _I, _P, _I, _I, _I, _I, _I, _F, _F, _I, _I,
                                                  _I, _P, _LL, _P]
            lib.ref_set_threads.argtypes = [_I]
            lib.ref_set_threads.restype = _I
            lib.ref_starburst.argtypes = [_P, _I, _I, _P, _I, _F, _F, _F, _P, _F, _P, _P, _I, _I, _I, _I, _P]
            lib.ref_aperture_shape.argtypes = [_P, _I, _I, _F, _F, _I, _F, _F, _F]
            lib.ref_aperture_dust.argtypes = [_P, _I, _I, _F, _F, _F, _F, _F, _F, _F, _F]
            lib.ref_trace_intersections.argtypes = [_P, _I, _P, _I, _P, _I, _I, _F, _I, _F, _P, _P, _P, _I]
            lib.ref_diagram.argtypes = [_P, _I, _I, _F, _P, _I, _I, _I, _I, _P]
            Reference._lib = lib
        self.lib = Reference._lib

    def trace(self, elements, paths, wavelengths_int, args: TraceArgs, first=0, count=-1):
        R = args.grid_count**2
        n = args.path_count * args.wavelength_count * R
        out = np.zeros((6, n), np.float32)
        el = _c(elements, elements.dtype)
        pa = _c(paths, np.int32)
        wl = _c(wavelengths_int, np.int32)
        d = np.array(list(args.direction), np.float32)
        self.lib.ref_trace(_ptr(el), args.element_count, _ptr(pa), args.path_count, _ptr(wl),
                           args.wavelength_count, args.aperture_index, args.coating_min_ior, args.grid_count,
                           args.grid_length, _ptr(d), _ptr(out), first, count)
        return out

    def trace_intersections(self, elements, paths, wavelengths_int, args: TraceArgs, count: int):
        n = args.path_count * args.wavelength_count * args.grid_count**2
        rays = np.zeros((6, n), np.float32)
        inter = np.zeros((n, count, 8), np.float32)
        d = np.array(list(args.direction), np.float32)
        self.lib.ref_trace_intersections(_ptr(_c(elements, elements.dtype)), args.element_count,
                                         _ptr(_c(paths, np.int32)), args.path_count,
                                         _ptr(_c(wavelengths_int, np.int32)), args.wavelength_count,
                                         args.aperture_index, args.coating_min_ior, args.grid_count,
                                         args.grid_length, _ptr(d), _ptr(rays), _ptr(inter), count)
        return rays, inter

    def diagram(self, elements, aperture_index, scale, inter, width, height):
        image = np.zeros((height, width, 4), np.float32)
        el = _c(elements, elements.dtype)
        if inter is None:
            self.lib.ref_diagram(_ptr(el), len(el), aperture_index, scale, None, 0, 0, width, height, _ptr(image))
        else:
            rec = _c(inter, np.float32)
            self.lib.ref_diagram(_ptr(el), len(el), aperture_index, scale, _ptr(rec), rec.shape[0], rec.shape[1],
                                 width, height, _ptr(image))
        return image

    def prim_shader(self, rays, P, W, G, area_orig, min_area):
        Q = (G - 1) ** 2
        bounds = np.zeros((P * Q, 4), np.float32)
        inten = np.zeros(P * Q * W, np.float32)
        self.lib.ref_prim_shader(_ptr(_c(rays, np.float32)), P, W, G, area_orig, min_area, _ptr(bounds),
                                 _ptr(inten))
        return bounds, inten

    def vertex_shader(self, rays, intensities, P, W, G, st, width, height):
        n = P * W * G * G
        out = np.zeros((n + 1, 8), np.float32)
        self.lib.ref_vertex_shader(_ptr(_c(rays, np.float32)), _ptr(_c(intensities, np.float32)), P, W, G, st,
                                   width, height, _ptr(out))
        return out

    def binner(self, bounds, st, width, height, bin_size, local_size=1024):
        prims = bounds.shape[0]
        bins = ((width + bin_size - 1) // bin_size) * ((height + bin_size - 1) // bin_size)
        batches = (prims + 254) // 255
        masks = np.zeros((bins, batches, 4), np.uint64)
        self.lib.ref_binner(_ptr(_c(bounds, np.float32)), prims, st, width, height, bin_size, local_size,
                            _ptr(masks))
        return masks

    def rasterizer(self, vertexes, masks, ghost, spectrum, args: RasterArgs, rows=None, cols=(0, 0)):
        image = np.zeros((args.height, args.width, 4), np.float32)
        y0, y1 = rows if rows is not None else (0, args.height)
        g = _c(ghost, np.float32)
        self.lib.ref_rasterizer(_ptr(_c(vertexes, np.float32)), _ptr(_c(masks, np.uint64)), masks.shape[1],
                                _ptr(g), g.shape[1], g.shape[0], _ptr(_c(spectrum, np.float32)), args.path_count,
                                args.wavelength_count, args.wavelength_sub_count, args.grid_count, args.sub_steps,
                                args.intensity, args.ghost_scale, args.width, args.height, args.bin_size, y0, y1,
                                cols[0], cols[1], _ptr(image))
        return image

    def rasterizer_pixels(self, vertexes, masks, ghost, spectrum, args: RasterArgs, xy, image=None):
        """The reference rasterizer on the listed pixels ((n, 2) int x, y, unflipped) in one
        parallel region; returns the full-size image with those pixels set."""
        if image is None:
            image = np.zeros((args.height, args.width, 4), np.float32)
        g = _c(ghost, np.float32)
        xy = _c(xy, np.int32)
        self.lib.ref_rasterizer_pixels(_ptr(_c(vertexes, np.float32)), _ptr(_c(masks, np.uint64)), masks.shape[1],
                                       _ptr(g), g.shape[1], g.shape[0], _ptr(_c(spectrum, np.float32)),
                                       args.path_count, args.wavelength_count, args.wavelength_sub_count,
                                       args.grid_count, args.sub_steps, args.intensity, args.ghost_scale, args.width,
                                       args.height, args.bin_size, _ptr(xy), len(xy), _ptr(image))
        return image

    def set_threads(self, threads: int) -> int:
        """OpenMP threads of the reference kernels (0 keeps the count); returns the previous."""
        return self.lib.ref_set_threads(threads)

    def starburst(self, fourier, spectrum, a: StarburstArgs, rows=None):
        out = np.zeros((a.height, a.width, 4), np.float32)
        y0, y1 = rows if rows is not None else (0, a.height)
        f = _c(fourier, np.float32)
        vig = np.array(list(a.vignetting), np.float32)
        off = np.array(list(a.offset), np.float32)
        sc = np.array(list(a.scale), np.float32)
        self.lib.ref_starburst(_ptr(f), f.shape[1], f.shape[0], _ptr(_c(spectrum, np.float32)), a.samples, a.blur,
                               a.rotation, a.rotation_weight, _ptr(vig), a.intensity, _ptr(off), _ptr(sc), a.width,
                               a.height, y0, y1, _ptr(out))
        return out

    def aperture_shape(self, w, h, size, blades, rotation, roundness, softness):
        out = np.zeros((h, w), np.float32)
        self.lib.ref_aperture_shape(_ptr(out), w, h, size[0], size[1], blades, rotation, roundness, softness)
        return out

    def aperture_dust(self, image, size, strength, density, radius, parallax, softness):
        out = _c(image, np.float32).copy()
        h, w = out.shape
        self.lib.ref_aperture_dust(_ptr(out), w, h, size[0], size[1], strength, density, radius, parallax[0],
                                   parallax[1], softness)
        return out


# ------------------------------------------------------------------ FFT stages (numpy FP64)
def fft_power_spectrum(aperture: np.ndarray, wavelength_mm: float, distance_mm: float) -> np.ndarray:
    """``StarburstTask.update_fourier_spectrum`` (``realflare/api/tasks/starburst.py:45-81``)."""
    h, w = aperture.shape[:2]
    x = np.linspace(-1, 1, w)
    y = np.linspace(-1, 1, h)
    xv, yv = np.meshgrid(x, y)
    phase = np.exp(1j * np.pi / (wavelength_mm * distance_mm) * (xv**2 + yv**2))
    f = np.fft.fftshift(np.fft.fft2(aperture.astype(np.float64) * phase))
    return f.real**2 + f.imag**2


def _chirp_arg(shape) -> np.ndarray:
    """``frft.chirp`` (``realflare/utils/frft.py:8-17``): i*pi*sum_k fftshift(n_k)^2 / N_k."""
    grids = np.meshgrid(*[np.arange(-n // 2, n // 2) for n in shape], indexing='ij')
    total = np.zeros(shape, np.float64)
    for i, g in enumerate(grids):
        total = total + np.fft.fftshift(g) ** 2 / shape[i]
    return 1j * np.pi * total


def frft(array: np.ndarray, alpha: float) -> np.ndarray:
    """Fractional Fourier transform (``realflare/utils/frft.py:20-62``, Ozaktas et al. 1996)."""
    rel = alpha % 4
    if rel < 0.5:
        alpha, array = rel + 1, np.fft.ifftn(array, norm='ortho')
    elif rel < 1.5:
        alpha = rel
    elif rel < 2.5:
        alpha, array = rel - 1, np.fft.fftn(array, norm='ortho')
    elif rel < 3.5:
        alpha, array = rel - 2, np.flip(array)
    else:
        alpha, array = rel - 3, np.fft.ifftn(array, norm='ortho')
    phi = alpha * np.pi / 2.0
    cot = 1.0 / np.tan(phi)
    sq = np.sqrt(1.0 + cot**2)
    scale = np.sqrt(1.0 - 1.0j * cot) / np.sqrt(np.prod(array.shape))
    c = _chirp_arg(array.shape)
    chirp1 = np.exp(c * (cot - sq))
    chirp2 = np.exp(c * sq)
    f1 = np.fft.fftn(chirp2, norm='ortho')
    f2 = np.fft.fftn(chirp1 * array, norm='ortho')
    return scale * chirp1 * np.fft.ifftn(f1 * f2, norm='ortho')


def ghost_texture(aperture: np.ndarray, fstop: float, resolution: tuple) -> np.ndarray:
    """``GhostTask.ghost`` (``realflare/api/tasks/ghost.py:13-36``); returns float64."""
    alpha = 0.15 * (560.0 / 400) * (fstop / 18)
    spectrum = np.fft.fftshift(aperture.astype(np.float64))
    spectrum = frft(spectrum, alpha)
    spectrum = np.fft.fftshift(spectrum)
    return np.abs(spectrum) * np.sqrt(resolution[0] * resolution[1])


def stratified_pixels(width: int, height: int, cells: int = 8, span: int = 16, seed: int = 0) -> np.ndarray:
    """(n, 2) int32 x, y of cells x cells horizontal spans of ``span`` pixels, one span at a
    seeded random place inside each cell of a cells x cells grid over the image (the pixel
    samples of the parity tests and of the timed CPU baseline)."""
    rng = np.random.default_rng(seed)
    xy = []
    for cy in range(cells):
        for cx in range(cells):
            y = int(rng.integers(cy * height // cells, (cy + 1) * height // cells))
            x_lo, x_hi = cx * width // cells, max(cx * width // cells + 1, (cx + 1) * width // cells - span)
            x0 = int(rng.integers(x_lo, x_hi))
            xy += [(min(x0 + i, width - 1), y) for i in range(span)]
    return np.unique(np.array(xy, np.int32), axis=0)


def reference_available() -> bool:
    return Reference.available()


ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
