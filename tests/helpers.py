"""Shared helpers of the parity tests: workloads reduced to sizes the CPU oracle finishes
in seconds, and error measures."""
from __future__ import annotations

import numpy as np

from realflare_gb300 import prepare, synthetic
from realflare_gb300.data import QSize


def reduced(name: str, grid: int | None = None, resolution: int | tuple | None = None, paths: int | None = None,
            wavelengths: int | None = None, integer_wavelengths: bool = True):
    """A named workload with optional smaller grid / image (side, or (width, height)) / path
    list / wavelength count."""
    w = synthetic.workload(name, integer_wavelengths=integer_wavelengths)
    p = w.project
    if grid:
        p.render.grid_count = grid
    if resolution:
        p.render.resolution = QSize(*resolution) if isinstance(resolution, tuple) else QSize(resolution, resolution)
    if paths:
        w.paths = w.paths[:paths]
        p.flare.lens.ghost_paths = tuple(tuple(x) for x in w.paths)
    if wavelengths:
        wl = np.linspace(p.render.wavelengths[0], p.render.wavelengths[-1], wavelengths)
        if integer_wavelengths:
            wl = np.round(wl)
        p.render.wavelengths = tuple(float(x) for x in wl)
        p.render.wavelength_count = wavelengths
    return w


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b|| / ||b|| over finite entries (NaN positions must agree separately)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    m = np.isfinite(a) & np.isfinite(b)
    den = np.linalg.norm(b[m])
    return float(np.linalg.norm((a - b)[m]) / (den if den > 0 else 1.0))


def ghost_texture(shape=(64, 64), seed=0) -> np.ndarray:
    return np.random.default_rng(seed).uniform(0.5, 1.5, shape).astype(np.float32)


def oracle_pipeline(o, w, ghost, spectrum):
    """Trace -> quad setup -> vertices -> bin masks -> raster with the C oracle."""
    ti = prepare.trace_inputs(w.project, w.paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    rays = o.trace(ti.elements, ti.paths, ti.wavelengths, a)
    area, min_area = prepare.quad_constants(w.project)
    bounds, inten = o.quad_setup(rays, P, W, G, area, min_area)
    ra = prepare.raster_args(w.project, P, W, ghost.shape)
    vtx = o.vertex(rays, inten, P, W, G, ra.screen_transform, ra.width, ra.height)
    masks = o.bin_masks(bounds, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    image = o.raster(vtx, masks, ghost, spectrum, ra)
    return dict(inputs=ti, rays=rays, bounds=bounds, inten=inten, vtx=vtx, masks=masks, image=image, raster_args=ra)


def stratified_pixels(width: int, height: int, cells: int = 8, span: int = 16, seed: int = 0) -> np.ndarray:
    """Seeded stratified spans of pixels (``oracle.oracle.stratified_pixels``)."""
    from oracle.oracle import stratified_pixels as sample

    return sample(width, height, cells, span, seed)


def at_pixels(image: np.ndarray, xy: np.ndarray) -> np.ndarray:
    """The RGBA values of the listed (unflipped x, y) pixels of a row-flipped image."""
    return image[image.shape[0] - 1 - xy[:, 1], xy[:, 0]]


def kept_paths(project, trace) -> tuple:
    """The ghost paths PreprocessTask keeps (``preprocessing.py:22-103``: a 3 x 3 probe grid
    over 1 % of the grid length, light at the centre, one wavelength; ghosts sorted by the
    reference's ``x * x`` "area" of the first probe ray; the smallest kept), with ``trace``
    (``Oracle.trace`` or ``Reference.trace`` with integer wavelengths) running the probe."""
    import copy

    from realflare_gb300.data import QPointF

    q = copy.deepcopy(project)
    q.render.grid_count, q.render.grid_length = 3, project.render.grid_length * 0.01
    q.render.resolution, q.render.wavelength_count, q.render.wavelengths = QSize(100, 100), 1, ()
    q.flare.light.position = QPointF(0, 0)
    ti = prepare.trace_inputs(q)
    rays = trace(ti.elements, ti.paths, ti.wavelengths.astype(np.int32), ti.args)
    P = ti.args.path_count
    x = rays[0].reshape(P, 1, 9)[:, 0, 0]
    areas = {i: np.abs(x[i]) * np.abs(x[i]) for i in range(P)}
    order = [k for k, _ in sorted(areas.items(), key=lambda item: item[1])]
    return tuple(order[: int(P * (1 - project.render.cull_percentage))])
