"""Batched frames: many lights, lenses, grids and wavelength sets per launch.

The reference renders one light per ``Engine`` call, and its only many-light path
(``Engine.image_flare``, ``realflare/api/engine.py:98-155``) loops over lights in Python,
tracing and rasterising each one. ``BatchRenderer`` renders a list of projects with one
launch per stage for all of them (trace, quad setup, vertices, binning into one tile
numbering, and one persistent raster launch whose CTAs take tiles from a device-side queue,
heaviest first) and no host synchronisation, so the sequence can be captured into one CUDA
graph and replayed. Each frame's image equals the single-frame path's image bit for bit
(the kernels share their per-ray, per-primitive and per-tile code).

Memory is bounded: frames are grouped so that no group's buffers exceed ``max_bytes``;
every group is one launch per stage (and one graph).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import prepare
from ._abi import BatchSizes, Frame, check, lib
from .constants import light_spectrum
from .data import Project, RealflareError
from .device import empty, ptr, require_cuda, to_device
from .lens import render_wavelengths

TILE_SIZES = (32, 16)
RAYS_PER_THREAD = (1, 2, 4)


def _ghost_key(project: Project) -> tuple:
    f, r = project.flare, project.render
    return (repr(f.ghost_aperture), f.ghost.fstop, r.ghost.resolution.width(), r.ghost.resolution.height())


# ghost texture starts in the batch buffer: multiples of 128 floats (512 bytes, the texture
# base alignment of current GPUs), so that every texture can get a texture object
GHOST_ALIGN_FLOATS = 128


def ghost_textures(projects: list, stream=None) -> tuple:
    """Ghost textures of the distinct ghost settings among the projects: (one float tensor of
    all textures, per-project float offset, per-project (height, width)). Each texture starts
    at a multiple of ``GHOST_ALIGN_FLOATS`` floats (zeros fill the gaps)."""
    from .tasks import GhostApertureTask, GhostTask

    aperture_task, ghost_task = GhostApertureTask(stream), GhostTask(stream)
    cache: dict = {}
    textures, offsets, shapes = [], [], []
    total = 0
    for p in projects:
        key = _ghost_key(p)
        if key not in cache:
            t = ghost_task.run(p, aperture_task.run(p)).tensor
            pad = -total % GHOST_ALIGN_FLOATS
            if pad:
                textures.append(torch.zeros(pad, dtype=t.dtype, device=t.device))
                total += pad
            cache[key] = (total, tuple(t.shape[:2]))
            textures.append(t.reshape(-1))
            total += t.numel()
        off, shape = cache[key]
        offsets.append(off)
        shapes.append(shape)
    return torch.cat(textures), offsets, shapes


@dataclass
class _Inputs:
    frames: ctypes.Array
    elements: np.ndarray
    paths: np.ndarray
    wavelengths: np.ndarray


def _frame_inputs(projects: list, ghost_offsets: list, ghost_shapes: list,
                  ghosts: torch.Tensor | None = None) -> _Inputs:
    """The frames' rf_frame records; with ``ghosts`` (the device buffer of the ghost textures)
    each frame also gets the texture object of its ghost texture."""
    frames = (Frame * len(projects))()
    elements, paths, wavelengths = [], [], []
    n_el = n_pa = n_wl = 0
    for i, p in enumerate(projects):
        ti = prepare.trace_inputs(p)
        if ti is None:
            raise RealflareError('a batched frame needs a lens with at least two elements')
        a = ti.args
        f = frames[i]
        f.trace = a
        f.raster = prepare.raster_args(p, a.path_count, a.wavelength_count, ghost_shapes[i])
        f.area_orig, f.min_area = prepare.quad_constants(p)
        f.element_offset, f.path_offset, f.wavelength_offset = n_el, n_pa, n_wl
        f.ghost_offset = ghost_offsets[i]
        if ghosts is not None:
            tex = ctypes.c_uint64()
            h, w = ghost_shapes[i]
            check(lib().rf_ghost_texture_object(ptr(ghosts) + 4 * int(ghost_offsets[i]), w, h, ctypes.byref(tex)),
                  'rf_ghost_texture_object')
            f.ghost_texture = tex.value
        elements.append(ti.elements)
        paths.append(ti.paths)
        wavelengths.append(ti.wavelengths)
        n_el += len(ti.elements)
        n_pa += len(ti.paths)
        n_wl += len(ti.wavelengths)
    return _Inputs(frames, np.concatenate(elements), np.concatenate(paths).astype(np.int32),
                   np.concatenate(wavelengths).astype(np.float32))


def frame_bytes(project: Project) -> int:
    """Device bytes one frame holds in a batch, before tile lists: rays (24 B), vertices
    (32 B), bounds and intensities, pair counters, image."""
    r = project.render
    P = len(project.flare.lens.ghost_paths)
    W, G = len(render_wavelengths(r)), r.grid_count
    rays = P * W * G * G
    prims = P * (G - 1) ** 2
    return rays * (24 + 32) + prims * (16 + 4 * W + 4 * max(W - 1, 1)) + r.resolution.width() * r.resolution.height() * 16


class BatchRenderer:
    """Renders ``projects`` (frames) together: ``run()`` enqueues every stage on the stream;
    ``capture()`` records the same sequence into a CUDA graph that ``replay()`` launches.
    ``images[i]`` is frame i's (height, width, 4) RGBA image on the device."""

    def __init__(self, projects: list, tile_size: int = 32, rays_per_thread: int = 1,
                 stream: torch.cuda.Stream | None = None, ghosts: tuple | None = None,
                 entry_capacity: int = 0) -> None:
        require_cuda()
        if tile_size not in TILE_SIZES or rays_per_thread not in RAYS_PER_THREAD:
            raise RealflareError('tile_size must be 16 or 32 and rays_per_thread 1, 2 or 4')
        self.lib = lib()
        self.projects = list(projects)
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self.sh = int(self.stream.cuda_stream)
        with torch.cuda.stream(self.stream):
            self.ghosts, ghost_offsets, ghost_shapes = ghosts if ghosts is not None else ghost_textures(
                self.projects, self.stream)
            inputs = _frame_inputs(self.projects, ghost_offsets, ghost_shapes, self.ghosts)
            self.sizes = BatchSizes()
            check(self.lib.rf_batch_plan(inputs.frames, len(self.projects), tile_size, rays_per_thread,
                                         ctypes.byref(self.sizes)), 'rf_batch_plan')
            z = self.sizes
            self.frames = inputs.frames
            self.frames_d = to_device(np.frombuffer(bytes(inputs.frames), np.uint8).copy())
            self.elements = to_device(inputs.elements.view(np.uint8))
            self.paths = to_device(inputs.paths)
            self.wavelengths = to_device(inputs.wavelengths)
            self.spectrum = to_device(light_spectrum())
            self.rays = empty((max(6 * z.rays, 1),))
            self.bounds = empty((max(4 * z.prims, 4),))
            self.inten = empty((max(z.intensities, 1),))
            self.vertexes = empty((8 * z.vertices,))
            self.tile_offsets = empty((z.tiles + 1,), torch.int32)
            self.entry_total = torch.zeros((1,), dtype=torch.int64, device=self.rays.device)
            self.image_buffer = empty((4 * z.image_pixels,))
        self.images = []
        for f in inputs.frames:
            h, w = f.raster.height, f.raster.width
            self.images.append(self.image_buffer[4 * f.image_offset: 4 * (f.image_offset + w * h)].view(h, w, 4))
        self.capacity = 0
        self._reserve(max(int(entry_capacity), 1 << 20))
        self.graph = None

    def _reserve(self, capacity: int) -> None:
        ws = ctypes.c_size_t()
        check(self.lib.rf_batch_workspace_size(ctypes.byref(self.sizes), capacity, ctypes.byref(ws)),
              'rf_batch_workspace_size')
        with torch.cuda.stream(self.stream):
            self.workspace = empty(((ws.value + 3) // 4,), torch.int32)
            self.entries = empty((capacity,), torch.int32)
        self.workspace_bytes = self.workspace.numel() * 4
        self.capacity = capacity
        self.graph = None

    def enqueue(self) -> None:
        """Every stage of every frame, on the stream, without host synchronisation."""
        L, z, s = self.lib, ctypes.byref(self.sizes), self.sh
        fd = ptr(self.frames_d)
        check(L.rf_trace_batch(fd, z, ptr(self.elements), ptr(self.paths), ptr(self.wavelengths), ptr(self.rays), s),
              'rf_trace_batch')
        check(L.rf_quad_setup_batch(fd, z, ptr(self.rays), ptr(self.bounds), ptr(self.inten), s),
              'rf_quad_setup_batch')
        check(L.rf_vertex_batch(fd, z, ptr(self.rays), ptr(self.inten), ptr(self.vertexes), s), 'rf_vertex_batch')
        check(L.rf_bin_tiles_batch(fd, z, ptr(self.bounds), ptr(self.vertexes), ptr(self.workspace),
                                   self.workspace_bytes, ptr(self.tile_offsets), ptr(self.entries), self.capacity,
                                   ptr(self.entry_total), s), 'rf_bin_tiles_batch')
        check(L.rf_raster_batch(fd, z, ptr(self.vertexes), ptr(self.tile_offsets), ptr(self.entries),
                                ptr(self.ghosts), ptr(self.spectrum), ptr(self.workspace), self.workspace_bytes,
                                self.capacity, ptr(self.entry_total), ptr(self.image_buffer), s), 'rf_raster_batch')

    def entry_count(self) -> int:
        self.stream.synchronize()
        return int(self.entry_total.item())

    def run(self) -> list:
        """Render eagerly, growing the tile-entry capacity until the lists fit."""
        for _ in range(4):
            self.enqueue()
            n = self.entry_count()
            if n <= self.capacity:
                return self.images
            self._reserve(int(n * 1.1) + 1024)
        raise RealflareError('rf_bin_tiles_batch: entry capacity did not converge')

    def capture(self) -> torch.cuda.CUDAGraph:
        """Record enqueue() into a CUDA graph (after a run() has sized the capacity)."""
        if self.capacity == 0 or self.entry_count() > self.capacity:
            self.run()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream):
            self.enqueue()
        self.graph = g
        return g

    def replay(self) -> None:
        if self.graph is None:
            self.capture()
        with torch.cuda.stream(self.stream):
            self.graph.replay()


def group_frames(projects: list, max_bytes: int) -> list:
    """Consecutive groups of frame indices whose buffers (``frame_bytes``, plus a share
    for tile lists) stay within max_bytes each."""
    groups, cur, cur_bytes = [], [], 0
    for i, p in enumerate(projects):
        b = 2 * frame_bytes(p)  # tile lists and sort buffers are of the same order
        if cur and cur_bytes + b > max_bytes:
            groups.append(cur)
            cur, cur_bytes = [], 0
        cur.append(i)
        cur_bytes += b
    if cur:
        groups.append(cur)
    return groups
