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

import copy
import ctypes
import math
import os

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
from ..data import Project, QPointF, QSize, RealflareError
from ..device import Image, MemoryObject, Rays, empty, ptr, require_cuda, stream_handle, to_device


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
    """Spectral trace of every ghost path (``realflare/api/tasks/raytracing.py:37-247``).

    ``accurate=True`` traces the ray geometry in double precision (``rf_trace_accurate``):
    positions equal the double evaluation of the reference's trace rounded to float, instead
    of the reference's FP32 values, at the cost of double-precision throughput."""

    def __init__(self, queue=None, cache: bool = True, accurate: bool = False) -> None:
        super().__init__(queue)
        self._cache = None
        self.use_cache = cache
        self.accurate = accurate

    def raytrace(self, project: Project, path_indexes: tuple = (), paths=None) -> Rays | None:
        inputs = prepare.trace_inputs(project, paths=paths, path_indexes=path_indexes)
        if inputs is None:
            return None
        key = (inputs.elements.tobytes(), inputs.paths.tobytes(), inputs.wavelengths.tobytes(),
               bytes(inputs.args), self.accurate)
        if self.use_cache and self._cache is not None and self._cache[0] == key:
            return self._cache[1]
        a = inputs.args
        elements = to_device(inputs.elements.view(np.uint8))
        paths_t = to_device(inputs.paths)
        wl = to_device(inputs.wavelengths)
        rays = empty((6, inputs.ray_count))
        if inputs.ray_count:
            trace = self.lib.rf_trace_accurate if self.accurate else self.lib.rf_trace
            check(trace(ptr(elements), ptr(paths_t), ptr(wl), ctypes.byref(a), ptr(rays), self.stream),
                  'rf_trace_accurate' if self.accurate else 'rf_trace')
        shape = (a.path_count, a.wavelength_count, a.grid_count**2)
        result = Rays(rays, shape, args=key)
        result.inputs = inputs
        self._cache = (key, result)
        return result

    def run(self, project: Project, path_indexes: tuple = (), paths=None) -> Rays | None:
        return self.raytrace(project, path_indexes, paths)


class IntersectionsTask(Task):
    """The trace with every surface hit stored, for the lens diagram
    (``realflare/api/tasks/raytracing.py:250-380``): the diagram's light position, grid and
    resolution, one wavelength. ``run`` returns a ``MemoryObject`` whose tensor is float32
    [paths, 1, grid, grid, 3 * elements - 1, 8] (rf_intersection records: pos xyz, normal
    xyz, incident, hit as int32), or None without a lens or without paths."""

    def run(self, project: Project, path_indexes: tuple) -> MemoryObject | None:
        p = prepare.diagram_project(project)
        inputs = prepare.trace_inputs(p, path_indexes=path_indexes)
        if inputs is None or inputs.ray_count == 0:
            return None
        a = inputs.args
        count = prepare.intersection_count(a.element_count)
        elements = to_device(inputs.elements.view(np.uint8))
        paths_t = to_device(inputs.paths)
        wl = to_device(inputs.wavelengths)
        rays = empty((6, inputs.ray_count))
        inter = empty((inputs.ray_count, count, 8))
        check(self.lib.rf_trace_intersections(ptr(elements), ptr(paths_t), ptr(wl), ctypes.byref(a), ptr(rays),
                                              ptr(inter), count, self.stream), 'rf_trace_intersections')
        G = a.grid_count
        result = MemoryObject(tensor=inter.view(a.path_count, a.wavelength_count, G, G, count, 8),
                              args=(bytes(a), inputs.paths.tobytes()))
        result.rays = rays
        return result


class DiagramTask(Task):
    """The lens cross-section with the traced rays (``realflare/api/tasks/diagram.py:24-228``):
    rf_diagram draws the optical axis and element profiles, then the paths and normals of
    one grid column of rays (column (grid - 1) // 2 + diagram.column_offset, sliced as the
    reference slices its array)."""

    def run(self, project: Project, intersections: MemoryObject | None) -> Image:
        r = project.diagram.resolution
        w, h = r.width(), r.height()
        image = empty((h, w, 4))
        inputs = prepare.trace_inputs(prepare.diagram_project(project), paths=np.zeros((0, 2), np.int32))
        if inputs is None:  # no lens: the reference's lenses kernel does not run
            image.zero_()
            return Image(tensor=image, args=(hash(project.diagram), None))
        elements = to_device(inputs.elements.view(np.uint8))
        scale = np.float32(prepare.diagram_scale(project))
        records, rays, count = None, 0, 0
        if intersections is not None:
            t = intersections.tensor
            column = int((t.shape[3] - 1) / 2) + project.diagram.column_offset
            part = t[:, :, :, column:column + 1].contiguous()  # DiagramTask.update_intersection_slice
            rays, count = part.shape[2] * part.shape[3], part.shape[4]
            if rays > 0 and part.shape[0] > 0:
                records = part[0, 0].reshape(rays, count, 8).contiguous()
            else:
                rays = 0
        check(self.lib.rf_diagram(ptr(elements), inputs.args.element_count, inputs.args.aperture_index, float(scale),
                                  ptr(records) if records is not None else None, rays, count, w, h, ptr(image),
                                  self.stream), 'rf_diagram')
        return Image(tensor=image, args=(hash(project.diagram), intersections.args if intersections else None))


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

    def order(self, offsets):
        """Tiles by decreasing entry count (rf_tile_order), for rf_raster_ordered."""
        tiles = offsets.numel() - 1
        ws_bytes = ctypes.c_size_t()
        check(self.lib.rf_tile_order_workspace_size(tiles, ctypes.byref(ws_bytes)), 'rf_tile_order_workspace_size')
        ws = self._buffer('order_workspace', (ws_bytes.value + 3) // 4, torch.int32)
        order = self._buffer('tile_order', tiles, torch.int32)
        check(self.lib.rf_tile_order(ptr(offsets), tiles, ptr(ws), ws.numel() * 4, ptr(order), self.stream),
              'rf_tile_order')
        return order

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
        order = self.order(offsets)
        check(self.lib.rf_raster_ordered(ptr(vertexes), ptr(offsets), ptr(entries), ptr(order), ptr(gt),
                                         ptr(self.spectrum()), ctypes.byref(a), ptr(image), self.stream),
              'rf_raster_ordered')
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


class PreprocessTask(Task):
    """Ghost culling (``realflare/api/tasks/preprocessing.py:22-103``): a 3 x 3 grid is
    traced at 1 % of the grid length with the light on axis and one wavelength; each path's
    "area" is |x| * |x| of its first ray's sensor position (the reference squares x; kept),
    and the paths with the largest areas are dropped up to ``cull_percentage``. Returns the
    kept path indexes in increasing-area order (the trace then keeps the paths' order)."""

    def __init__(self, queue=None) -> None:
        super().__init__(queue)
        self.raytracing_task = RaytracingTask(queue, cache=False)
        self._cache = None

    def preprocess(self, project: Project) -> tuple:
        p = copy.deepcopy(project)
        r = p.render
        r.grid_count = 3
        r.grid_length = project.render.grid_length * 0.01
        r.resolution = QSize(100, 100)
        r.wavelength_count = 1
        r.wavelengths = ()
        p.flare.light.position = QPointF(0, 0)
        rays = self.raytracing_task.run(p)
        if rays is None:
            return tuple()
        P, W, R = rays.shape
        x = rays.tensor[0].view(P, W, R)[:, 0, 0].cpu().numpy()
        areas = {path: np.abs(x[path]) * np.abs(x[path]) for path in range(P)}
        sorted_areas = sorted(areas.items(), key=lambda item: item[1])
        index_to_keep = int(len(sorted_areas) * (1 - project.render.cull_percentage))
        return tuple(int(k) for k, v in sorted_areas[:index_to_keep])

    def run(self, project: Project) -> tuple:
        lens, render = project.flare.lens, project.render
        key = (hash(lens), render.grid_length, render.cull_percentage)
        if self._cache is None or self._cache[0] != key:
            self._cache = (key, self.preprocess(project))
        return self._cache[1]


def resize_linear(array: np.ndarray, width: int, height: int) -> np.ndarray:
    """Bilinear resize with half-pixel centres and clamped edges (the documented behaviour of
    OpenCV's ``resize`` with ``INTER_LINEAR`` on float images, which the reference calls,
    ``preprocessing.py:136``): each output pixel interpolates the 2 x 2 nearest inputs."""
    h0, w0 = array.shape[:2]

    def axis(n_out, n_in):
        f = (np.arange(n_out, dtype=np.float64) + 0.5) * (n_in / n_out) - 0.5
        i = np.floor(f).astype(np.int64)
        t = (f - i).astype(np.float32)
        t = np.where(i < 0, 0.0, t)
        i = np.where(i < 0, 0, i)
        t = np.where(i >= n_in - 1, 0.0, t).astype(np.float32)
        i = np.minimum(i, n_in - 1)
        return i, np.minimum(i + 1, n_in - 1), t

    xi0, xi1, xt = axis(width, w0)
    yi0, yi1, yt = axis(height, h0)
    a = np.asarray(array, np.float32)
    rows = a[yi0] * (1 - yt)[:, None, None] + a[yi1] * yt[:, None, None]
    return (rows[:, xi0] * (1 - xt)[None, :, None] + rows[:, xi1] * xt[None, :, None]).astype(np.float32)


class ImageSamplingTask(Task):
    """Light image samples (``realflare/api/tasks/preprocessing.py:106-185``): the image is
    resized to ``image_sample_resolution`` (even width, height by the render's aspect ratio,
    even), and every pixel below the ``1 - samples / pixels`` percentile of its channel mean
    is zeroed; returns RGBA float32 (alpha 0). Files are ``.npy`` arrays (H, W, 3 or 4) of
    linear RGB: there is no image decoder in this package."""

    def __init__(self, queue=None) -> None:
        super().__init__(queue)
        self._cache = None

    @staticmethod
    def load_file(path: str) -> np.ndarray:
        path = os.path.expandvars(path)
        if not path.endswith('.npy') or not os.path.exists(path):
            raise RealflareError(f'Invalid Image path for flare light: {path}')
        array = np.load(path)
        if array.ndim != 3 or array.shape[2] < 3:
            raise RealflareError(f'Invalid Image path for flare light: {path}')
        array = array[..., :3]
        if array.dtype == np.uint8:
            array = np.divide(array, 255)
        return np.float32(array)

    @staticmethod
    def sample_data(array: np.ndarray, width: int, height: int, samples: int) -> np.ndarray:
        array = resize_linear(array, width, height)
        intensity = np.mean(array, axis=2, keepdims=True).ravel()
        try:
            threshold = 1 - (samples / len(intensity))
        except ZeroDivisionError:
            threshold = 0
        threshold = np.clip(threshold * 100, 0, 100)
        percentile = np.percentile(intensity, threshold)
        mask = intensity > percentile
        masked = np.reshape(array.copy(), (-1, 3))
        masked[~mask] = np.zeros((3,), np.float32)
        masked = masked.reshape(array.shape)
        return np.dstack((masked, np.zeros(masked.shape[:-1]))).astype(np.float32)

    def run(self, project: Project) -> np.ndarray:
        light = project.flare.light
        width = max(light.image_sample_resolution, 1)
        if width % 2 != 0:
            width += 1
        resolution = project.render.resolution
        ratio = resolution.height() / resolution.width()
        height = width * ratio
        if height % 2 != 0:
            height += 1
        height = int(height)
        key = (light.image_file, width, height, light.image_samples)
        if self._cache is None or self._cache[0] != key:
            array = self.load_file(light.image_file)
            self._cache = (key, self.sample_data(array, width, height, light.image_samples))
        return self._cache[1]


__all__ = [
    'ApertureTask', 'GhostApertureTask', 'GhostTask', 'ImageSamplingTask', 'PreprocessTask', 'RasterizingTask',
    'RaytracingTask',
    'StarburstApertureTask', 'StarburstTask', 'SPECTRUM_WIDTH', 'RF_OK',
]
