"""Generate the golden fixtures of tests/golden from the reference's own kernels.

The reference's OpenCL kernels, compiled for the host from the reference checkout by
oracle/build_ref.py, produce rays, primitive bounds and intensities, vertices, bin masks and
the rasterised image for two small workloads; the arrays are stored in
``tests/golden/<name>.npz`` with their SHA-256 in ``tests/golden/manifest.json``.

Usage: ``python tests/golden/make_golden.py`` (needs the reference checkout).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from helpers import ghost_texture, reduced  # noqa: E402

from realflare_gb300 import prepare  # noqa: E402
from realflare_gb300.constants import light_spectrum  # noqa: E402

CASES = {
    # name: (workload, grid, resolution, paths, wavelengths)
    'plain8_g12_96': ('plain-8', 12, 96, None, None),
    'spectral16_g10_64': ('spectral-16', 10, 64, 6, 4),
}


def case_project(name):
    wl, grid, res, paths, nwl = CASES[name]
    w = reduced(wl, grid=grid, resolution=res, paths=paths, wavelengths=nwl)
    return w


def generate(name) -> dict:
    from oracle.oracle import Reference

    ref = Reference()
    w = case_project(name)
    ti = prepare.trace_inputs(w.project, w.paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    rays = ref.trace(ti.elements, ti.paths, ti.wavelengths.astype(np.int32), a)
    area, min_area = prepare.quad_constants(w.project)
    bounds, inten = ref.prim_shader(rays, P, W, G, area, min_area)
    ghost = ghost_texture((32, 32), seed=7)
    ra = prepare.raster_args(w.project, P, W, ghost.shape)
    vtx = ref.vertex_shader(rays, inten, P, W, G, ra.screen_transform, ra.width, ra.height)
    masks = ref.binner(bounds, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    image = ref.rasterizer(vtx, masks, ghost, light_spectrum(), ra)
    return dict(rays=rays, bounds=bounds, intensities=inten, vertexes=vtx, masks=masks, ghost=ghost, image=image)


def main() -> None:
    manifest_path = os.path.join(HERE, 'manifest.json')
    with open(manifest_path) as f:
        manifest = json.load(f)  # other fixtures' entries (make_frft_golden.py) stay
    for name in CASES:
        arrays = generate(name)
        path = os.path.join(HERE, f'{name}.npz')
        np.savez_compressed(path, **arrays)
        manifest[name] = {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() for k, v in arrays.items()}
        print(name, {k: v.shape for k, v in arrays.items()}, os.path.getsize(path))
    with open(manifest_path, 'w') as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
        f.write('\n')


if __name__ == '__main__':
    main()
