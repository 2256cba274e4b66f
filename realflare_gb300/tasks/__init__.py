"""The render tasks: drop-in counterparts of the reference's OpenCL tasks.

Each class keeps the reference's name and ``run`` signature (``realflare/api/tasks/*.py``)
and calls the CUDA library through its C ABI on one torch CUDA stream (the reference's
command queue). Results stay on the device until ``.array`` is read.

* ``RaytracingTask.run(project, path_indexes) -> Rays | None``  (raytracing.py:223-247)
* ``RasterizingTask.run(project, rays, ghost) -> Image``        (rasterizing.py:423-439)
* ``GhostApertureTask.run(project) -> Image``, ``StarburstApertureTask.run(project)``
                                                                (aperture.py:189-219)
* ``GhostTask.run(project, aperture) -> Image``                 (ghost.py:38-43)
* ``StarburstTask.run(project, aperture) -> Image``             (starburst.py:155-168)
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from .. import prepare
from .._abi import (
    RF_ERR_WORKSPACE,
    RF_OK,
    SPECTRUM_WIDTH,
    StarburstArgs,
    check,
    lib,
)
from ..constants import LAMBDA_MID, light_spectrum
from ..data import Project, RealflareError
from ..device import Image, Rays, empty, ptr, require_cuda, stream_handle, to_device


class Task:
    """Common base: the stream ("queue") the task's kernels are enqueued on."""

    def __init__(self, queue: torch.cuda.Stream | None = None) -> None:
        require_cuda()
        self.queue = queue
        self.lib = lib()

    @property
    def stream(self) -> int:
        return stream_handle(self.queue)


class RaytracingTask(Task):
    """Spectral trace of every ghost path (``realflare/api/tasks/raytracing.py:37-247``)."""

    def __init__(self, queue=None, cache: bool = True) -> None:
        super().__init__(queue)
        self._cache = None
        self.use_cache = cache

    def raytrace(self, project: Project, path_indexes: tuple = (), paths=None) -> Rays | None:
        inputs = prepare.trace_inputs(project, paths=paths, path_indexes=path_indexes)
        if inputs is None:
            return None
        key = (inputs.elements.tobytes(), inputs.paths.tobytes(), inputs.wavelengths.tobytes(),
               bytes(inputs.args))
        if self.use_cache and self._cache is not None and self._cache[0] == key:
            return self._cache[1]
        a = inputs.args
        elements = to_device(inputs.elements.view(np.uint8))
        paths_t = to_device(inputs.paths)
        wl = to_device(inputs.wavelengths)
        rays = empty((6, inputs.ray_count))
        if inputs.ray_count:
            check(self.lib.rf_trace(ptr(elements), ptr(paths_t), ptr(wl), ctypes.byref(a), ptr(rays), self.stream),
                  'rf_trace')
        shape = (a.path_count, a.wavelength_count, a.grid_count**2)
        result = Rays(rays, shape, args=key)
        result.inputs = inputs
        self._cache = (key, result)
        return result

    def run(self, project: Project, path_indexes: tuple = (), paths=None) -> Rays | None:
        return self.raytrace(project, path_indexes, paths)


class RasterizingTask(Task):
    """Quad setup, binning and rasterisation (``realflare/api/tasks/rasterizing.py``)."""

    def __init__(self, queue=None) -> None:
        super().__init__(queue)
        self._spectrum = None
        self._entry_capacity = 0
        self._buffers: dict = {}
        self.last_entry_count = 0
        self.tile_size = 0

    def _buffer(self, name: str, numel: int, dtype=torch.float32) -> torch.Tensor:
        t = self._buffers.get(name)
        if t is None or t.numel() < numel or t.dtype != dtype:
            t = empty((max(numel, 1),), dtype)
            self._buffers[name] = t
        return t

    def spectrum(self) -> torch.Tensor:
        if self._spectrum is None:
            self._spectrum = to_device(light_spectrum())
        return self._spectrum

    def setup(self, project: Project, rays: Rays):
        """Quad setup and vertex setup: (bounds, intensities, vertexes) on the device."""
        P, W, R = rays.shape
        G = project.render.grid_count
        Q = (G - 1) ** 2
        area, min_area = prepare.quad_constants(project)
        bounds = self._buffer('bounds', P * Q * 4)
        inten = self._buffer('intensities', P * Q * W)
        check(self.lib.rf_quad_setup(ptr(rays.tensor), P, W, G, area, min_area, ptr(bounds), ptr(inten), self.stream),
              'rf_quad_setup')
        a = prepare.raster_args(project, P, W, (1, 1))
        vertexes = self._buffer('vertexes', (P * R * W + 1) * 8)
        check(self.lib.rf_vertex(ptr(rays.tensor), ptr(inten), P, W, G, a.screen_transform, a.width, a.height,
                                 ptr(vertexes), self.stream), 'rf_vertex')
        return bounds, inten, vertexes

    def bin(self, args, bounds, vertexes):
        """Ordered per-tile entry lists: (tile_offsets, tile_entries)."""
        tile_size = ctypes.c_int32()
        tile_count = ctypes.c_int32()
        check(self.lib.rf_raster_tiles(ctypes.byref(args), ctypes.byref(tile_size), ctypes.byref(tile_count)),
              'rf_raster_tiles')
        self.tile_size = tile_size.value
        offsets = self._buffer('tile_offsets', tile_count.value + 1, torch.int32)
        count = ctypes.c_int64()
        for _ in range(3):
            cap = self._entry_capacity
            ws_bytes = ctypes.c_size_t()
            check(self.lib.rf_bin_workspace_size(ctypes.byref(args), cap, ctypes.byref(ws_bytes)),
                  'rf_bin_workspace_size')
            ws = self._buffer('bin_workspace', (ws_bytes.value + 3) // 4, torch.int32)
            entries = self._buffer('tile_entries', cap, torch.int32)
            status = self.lib.rf_bin_tiles(ptr(bounds), ptr(vertexes), ctypes.byref(args), ptr(ws),
                                           ws.numel() * 4, ptr(offsets), ptr(entries) if cap else None, cap,
                                           ctypes.byref(count), self.stream)
            if status == RF_ERR_WORKSPACE:
                self._entry_capacity = int(count.value * 1.25) + 1024
                continue
            check(status, 'rf_bin_tiles')
            self.last_entry_count = count.value
            return offsets, entries
        raise RealflareError('rf_bin_tiles: workspace did not converge')

    def rasterize(self, project: Project, rays: Rays | None, ghost: Image) -> Image:
        render = project.render
        h, w = render.resolution.height(), render.resolution.width()
        image = empty((h, w, 4))
        if rays is None or rays.shape[0] == 0:
            image.zero_()
            return Image(tensor=image, args=(None, render.resolution))
        P, W, R = rays.shape
        gt = ghost.tensor
        a = prepare.raster_args(project, P, W, tuple(gt.shape[:2]))
        bounds, inten, vertexes = self.setup(project, rays)
        offsets, entries = self.bin(a, bounds, vertexes)
        check(self.lib.rf_raster(ptr(vertexes), ptr(offsets), ptr(entries), ptr(gt), ptr(self.spectrum()),
                                 ctypes.byref(a), ptr(image), self.stream), 'rf_raster')
        return Image(tensor=image, args=(rays.args, ghost.args, hash(render), hash(project.flare.lens)))

    def run(self, project: Project, rays: Rays | None, ghost: Image) -> Image:
        return self.rasterize(project, rays, ghost)


class ApertureTask(Task):
    """Procedural aperture masks (``realflare/api/tasks/aperture.py:21-186``)."""

    def aperture(self, aperture, resolution, scratches_parallax=(0.0, 0.0), dust_parallax=(0.0, 0.0)) -> Image:
        w, h = resolution.width(), resolution.height()
        image = empty((h, w))
        s = aperture.shape
        check(self.lib.rf_aperture_shape(ptr(image), w, h, s.size.width(), s.size.height(), s.blades,
                                         math.radians(s.rotation), s.roundness, s.softness / 10, self.stream),
              'rf_aperture_shape')
        if aperture.grating.strength > 0 or aperture.scratches.strength > 0 or (
                aperture.image.strength > 0 and aperture.image.file):
            raise RealflareError('aperture grating, scratches and image textures are not supported')
        d = aperture.dust
        if d.strength > 0:
            if d.blur_sigma > 0:
                rng = np.random.Generator(np.random.PCG64(d.seed))
                noise = to_device(rng.random((h, w), dtype=np.float32))
                scratch = empty((h, w))
                check(self.lib.rf_aperture_noise_dust(ptr(image), ptr(noise), ptr(scratch), w, h, d.strength,
                                                      d.blur_sigma, self.stream), 'rf_aperture_noise_dust')
            else:
                check(self.lib.rf_aperture_dust(ptr(image), w, h, s.size.width(), s.size.height(), d.strength,
                                                d.density, d.radius * 0.1, dust_parallax[0], dust_parallax[1],
                                                d.softness / 10, self.stream), 'rf_aperture_dust')
        return Image(tensor=image, args=(aperture, resolution, tuple(scratches_parallax), tuple(dust_parallax)))


class GhostApertureTask(ApertureTask):
    def run(self, project: Project) -> Image:
        return self.aperture(project.flare.ghost_aperture, project.render.ghost.resolution)


class StarburstApertureTask(ApertureTask):
    def run(self, project: Project) -> Image:
        position = project.flare.light.position
        sp = project.flare.starburst_aperture.scratches.parallax
        dp = project.flare.starburst_aperture.dust.parallax
        return self.aperture(
            project.flare.starburst_aperture,
            project.render.starburst.resolution,
            (position.x() * sp.width(), position.y() * sp.height()),
            (position.x() * dp.width(), position.y() * dp.height()),
        )


class GhostTask(Task):
    """Ghost ringing texture by fractional Fourier transform (``ghost.py:13-43``)."""

    def ghost(self, aperture: Image, fstop: float, resolution) -> Image:
        at = aperture.tensor
        h, w = at.shape[:2]
        alpha = 0.15 * (LAMBDA_MID / 400) * (fstop / 18)
        scratch = empty((3, h, w, 2))
        out = empty((h, w))
        check(self.lib.rf_ghost_frft(ptr(at), w, h, alpha, ptr(scratch), ptr(out), self.stream), 'rf_ghost_frft')
        return Image(tensor=out, args=(aperture.args, fstop, resolution))

    def run(self, project: Project, aperture: Image) -> Image:
        return self.ghost(aperture, project.flare.ghost.fstop, project.render.ghost.resolution)


class StarburstTask(Task):
    """Starburst diffraction (``realflare/api/tasks/starburst.py:16-168``)."""

    def __init__(self, queue=None) -> None:
        super().__init__(queue)
        self._light = None

    def light(self) -> torch.Tensor:
        if self._light is None:
            self._light = to_device(light_spectrum())
        return self._light

    def fourier_spectrum(self, aperture: Image, distance: float, wavelengths_nm) -> torch.Tensor:
        at = aperture.tensor
        h, w = at.shape[:2]
        count = len(wavelengths_nm)
        lam = (ctypes.c_float * count)(*[float(x) * 1e-6 for x in wavelengths_nm])
        distance_mm = max(1e-9, distance * 1e3)
        scratch = empty((2, count, h, w, 2))
        spectrum = empty((count, h, w))
        check(self.lib.rf_starburst_spectrum(ptr(at), w, h, lam, count, distance_mm, ptr(scratch), ptr(spectrum),
                                             self.stream), 'rf_starburst_spectrum')
        return spectrum

    def starburst(self, project: Project, aperture: Image) -> Image:
        config = project.flare.starburst
        resolution = project.render.resolution
        w, h = resolution.width(), resolution.height()
        if config.per_wavelength:
            from ..lens import render_wavelengths

            wl = [float(x) for x in render_wavelengths(project.render)]
        else:
            wl = [LAMBDA_MID]
        spectrum = self.fourier_spectrum(aperture, config.distance, wl)
        a = StarburstArgs()
        a.width, a.height = w, h
        a.spectrum_count, a.spectrum_height, a.spectrum_width = spectrum.shape
        a.samples = project.render.starburst.samples
        a.blur = config.blur / 100
        a.rotation = math.radians(config.rotation)
        a.rotation_weight = config.rotation_weight
        if config.vignetting_enabled:
            a.vignetting[0], a.vignetting[1] = config.vignetting.x(), config.vignetting.y()
        else:
            a.vignetting[0] = a.vignetting[1] = float('nan')
        a.intensity = config.intensity * 1e-6
        pos = project.flare.light.position
        a.offset[0], a.offset[1] = pos.x(), -pos.y()
        a.scale[0], a.scale[1] = config.scale.width(), config.scale.height() * w / h
        a.lambda_first = wl[0]
        a.lambda_step = (wl[-1] - wl[0]) / (len(wl) - 1) if len(wl) > 1 else 1.0
        image = empty((h, w, 4))
        check(self.lib.rf_starburst(ptr(spectrum), ptr(self.light()), ctypes.byref(a), ptr(image), self.stream),
              'rf_starburst')
        return Image(tensor=image, args=(aperture.args, hash(config), hash(resolution), a.samples, hash(pos)))

    def run(self, project: Project, aperture: Image) -> Image:
        return self.starburst(project, aperture)


__all__ = [
    'ApertureTask', 'GhostApertureTask', 'GhostTask', 'RasterizingTask', 'RaytracingTask',
    'StarburstApertureTask', 'StarburstTask', 'SPECTRUM_WIDTH', 'RF_OK',
]
