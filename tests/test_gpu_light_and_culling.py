"""Image-based lights and ghost culling through the Engine (the reference's
Engine.image_flare, engine.py:98-155, and PreprocessTask, preprocessing.py:22-103).

* image_flare renders every light sample's flare as one batch and accumulates the four
  mirrored copies on the device; it must equal the reference's loop (one single-light
  render per sample, float32 numpy accumulation in the same order) bit for bit;
* PreprocessTask's kept paths equal those computed from the oracle's trace of the probe
  grid, and a culled render equals the single-light render of the kept paths.
"""
from __future__ import annotations

import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from realflare_gb300 import prepare, synthetic  # noqa: E402
from realflare_gb300.data import QPointF, QSize  # noqa: E402


def small_project():
    w = synthetic.workload('plain-8')
    p = w.project
    p.render.resolution = QSize(128, 128)
    p.render.grid_count = 16
    return p


def test_image_flare_equals_the_reference_loop(tmp_path):
    from realflare_gb300.engine import Engine
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    rng = np.random.default_rng(3)
    yy, xx = np.mgrid[0:40, 0:40]
    light = np.zeros((40, 40, 3), np.float32)
    for _ in range(6):  # soft blobs: the bilinear downscale samples 2 x 2 pixels
        cy, cx = rng.uniform(0, 40, 2)
        light += (np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / 18.0)[..., None]
                  * rng.uniform(0.5, 4.0, 3)).astype(np.float32)
    path = tmp_path / 'light.npy'
    np.save(path, light)
    p = small_project()
    p.flare.light.image_file_enabled = True
    p.flare.light.image_file = str(path)
    p.flare.light.image_sample_resolution = 8
    p.flare.light.image_samples = 6
    engine = Engine(cache=False)
    engine._init()
    with torch.cuda.stream(engine.queue):
        got = engine.image_flare(p).array.copy()
        sample = engine.image_sampling_task.run(p)
        ghost = engine.ghost(p)
    engine.queue.synchronize()
    # the reference's loop, engine.py:118-150
    h, w, _ = sample.shape
    hw, hh = int(w / 2), int(h / 2)
    want = np.zeros((128, 128, 4), np.float32)
    trace, raster = RaytracingTask(cache=False), RasterizingTask()
    count = 0
    for y in range(hh):
        for x in range(hw):
            values = np.float32([sample[y, x], sample[h - y - 1, x], sample[h - y - 1, w - x - 1],
                                 sample[y, w - x - 1]])
            if np.sum(values) == 0:
                continue
            q = copy.deepcopy(p)
            q.flare.light.position = QPointF((x + 0.5) / hw - 1, 1 - (y + 0.5) / hh)
            flare = raster.run(q, trace.run(q), ghost).array.copy()
            want += values[0] * flare
            flare = np.flip(flare, 0)
            want += values[1] * flare
            flare = np.flip(flare, 1)
            want += values[2] * flare
            flare = np.flip(flare, 0)
            want += values[3] * flare
            count += 1
    want /= w * h
    assert count >= 2
    assert np.abs(want).sum() > 0
    assert np.array_equal(got, want)


def test_culling_keeps_the_smallest_ghosts():
    from oracle.oracle import Oracle
    from realflare_gb300.device import Image
    from realflare_gb300.engine import Engine
    from realflare_gb300.tasks import GhostApertureTask, GhostTask, PreprocessTask, RasterizingTask, RaytracingTask

    p = small_project()
    p.render.cull_percentage = 0.4
    kept = PreprocessTask().run(p)
    # the same probe with the oracle (bit-identical FP32 positions)
    q = copy.deepcopy(p)
    q.render.grid_count, q.render.grid_length = 3, p.render.grid_length * 0.01
    q.render.resolution, q.render.wavelength_count, q.render.wavelengths = QSize(100, 100), 1, ()
    q.flare.light.position = QPointF(0, 0)
    ti = prepare.trace_inputs(q)
    rays = Oracle('f32').trace(ti.elements, ti.paths, ti.wavelengths, ti.args)
    P = ti.args.path_count
    x = rays[0].reshape(P, 1, 9)[:, 0, 0]
    areas = {i: np.abs(x[i]) * np.abs(x[i]) for i in range(P)}
    order = [k for k, _ in sorted(areas.items(), key=lambda item: item[1])]
    assert kept == tuple(order[: int(P * (1 - 0.4))])
    assert 0 < len(kept) < P
    # a culled flare equals the single-light render of the kept paths
    engine = Engine(cache=False)
    assert engine.render(p)
    got = engine.image.array
    ghost = GhostTask().run(p, GhostApertureTask().run(p))
    want = RasterizingTask().run(p, RaytracingTask(cache=False).run(p, kept), Image(tensor=ghost.tensor)).array
    assert np.array_equal(got, want)
