"""Autotuner of the batched path: picks the raster tile size and the rays per trace thread.

Both knobs change only the schedule (the images are bit-identical for every choice), so the
tuner renders a sample of the frames once per candidate, times each with CUDA events on
the renderer's stream, and keeps the fastest. Results are cached per device name and
sample signature in memory and, when ``cache_path`` is given, in a JSON file.
"""
from __future__ import annotations

import hashlib
import json
import os
from dataclasses import dataclass, field

import torch

from .batch import RAYS_PER_THREAD, TILE_SIZES, BatchRenderer, ghost_textures

CANDIDATES = tuple((t, r) for t in TILE_SIZES for r in RAYS_PER_THREAD)
_memory: dict = {}


@dataclass
class Choice:
    tile_size: int
    rays_per_thread: int
    timings_ms: dict = field(default_factory=dict)  # "tile x rays" -> best ms of the sample


def signature(projects: list) -> str:
    h = hashlib.sha256()
    h.update(torch.cuda.get_device_name().encode())
    for p in projects:
        r = p.render
        h.update(repr((len(p.flare.lens.ghost_paths), r.grid_count, r.wavelength_count, r.resolution.width(),
                       r.resolution.height(), r.anti_aliasing, r.wavelength_sub_count,
                       p.flare.lens.lens_model.name)).encode())
    return h.hexdigest()[:16]


def time_candidate(projects: list, tile: int, rpt: int, ghosts: tuple, repeats: int = 2) -> float:
    r = BatchRenderer(projects, tile_size=tile, rays_per_thread=rpt, ghosts=ghosts)
    r.run()  # sizes the tile lists and warms up
    best = float('inf')
    for _ in range(repeats):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(r.stream)
        r.enqueue()
        e1.record(r.stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del r
    return best


def autotune(projects: list, candidates=CANDIDATES, repeats: int = 2, cache_path: str | None = None) -> Choice:
    """The fastest (tile size, rays per thread) for rendering ``projects`` as one batch."""
    key = signature(projects)
    if key in _memory:
        return _memory[key]
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            stored = json.load(f).get(key)
        if stored:
            choice = Choice(**stored)
            _memory[key] = choice
            return choice
    ghosts = ghost_textures(projects)
    timings = {}
    for tile, rpt in candidates:
        timings[f'{tile}x{rpt}'] = time_candidate(projects, tile, rpt, ghosts, repeats)
    best = min(timings, key=timings.get)
    tile, rpt = (int(x) for x in best.split('x'))
    choice = Choice(tile, rpt, timings)
    _memory[key] = choice
    if cache_path:
        data = {}
        if os.path.exists(cache_path):
            with open(cache_path) as f:
                data = json.load(f)
        data[key] = choice.__dict__
        with open(cache_path, 'w') as f:
            json.dump(data, f, indent=1)
    return choice
