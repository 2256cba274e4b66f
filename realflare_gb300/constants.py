"""Constants and wire layouts shared with the reference.

``LAMBDA_*`` follow ``realflare/api/tasks/opencl.py:14-16``; ``BATCH_PRIMITIVE_COUNT``
``realflare/api/tasks/rasterizing.py:26``; the n-rook sample offsets
``realflare/api/tasks/rasterizing.py:78-87``. The numpy dtypes are the reference's
``ray_dtype``/``vertex_dtype``/``lens_element_dtype`` (``opencl.py:28-61``) laid out as
OpenCL lays them out (``float3`` occupies 16 bytes), for exporting this library's compact
device buffers in the reference's own layout.
"""
from __future__ import annotations

import csv
import os

import numpy as np

LAMBDA_MIN = 390
LAMBDA_MAX = 730
LAMBDA_MID = (LAMBDA_MIN + LAMBDA_MAX) / 2

BATCH_PRIMITIVE_COUNT = 255

SUB_OFFSETS = (0, 1, 0, 1, 2, 0, 3, 4, 1, 6, 2, 5, 0, 3, 7)

RESOURCES = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'resources')

_f3 = np.dtype((np.float32, 4))  # OpenCL float3 is 16 bytes
ray_dtype = np.dtype(
    [
        ('pos', _f3),
        ('dir', _f3),
        ('pos_apt', np.float32, 2),
        ('rrel', np.float32),
        ('reflectance', np.float32),
    ]
)
vertex_dtype = np.dtype(
    {
        'names': ['pos', 'uv', 'rrel', 'reflectance', 'intensity'],
        'formats': [(np.float32, 2), (np.float32, 2), np.float32, np.float32, np.float32],
        'offsets': [0, 8, 16, 20, 24],
        'itemsize': 32,
    }
)

# Device layout of one lens element (64 bytes), the C struct ``rf_lens_element`` of
# include/realflare_gb300.h. The first five fields carry the reference's
# ``lens_element_dtype`` meaning; ``coating_layers``/``coating_thickness`` select the
# coating extensions (0 = the reference rule).
lens_element_dtype = np.dtype(
    [
        ('radius', np.float32),
        ('ior', np.float32),
        ('height', np.float32),
        ('center', np.float32),
        ('coating', np.int32),
        ('coating_layers', np.int32),
        ('coating_thickness', np.float32, 2),
        ('coefficients', np.float32, 8),
    ]
)
assert lens_element_dtype.itemsize == 64


def cie_xyz_table() -> np.ndarray:
    """The CIE 2006 10-degree table, rows (nm, X, Y, Z) (``realflare/utils/ciexyz.py``)."""
    rows = []
    with open(os.path.join(RESOURCES, 'ciexyz.csv'), encoding='utf-8') as f:
        for row in csv.reader(line for line in f if not line.startswith('#')):
            rows.append([float(v) for v in row])
    return np.array(rows, dtype=np.float64)


def light_spectrum() -> np.ndarray:
    """The spectrum texture: XYZ0 rows for LAMBDA_MIN <= nm < LAMBDA_MAX as float32 (340, 4).

    ``realflare/api/tasks/rasterizing.py:170-179`` and ``starburst.py:33-43``.
    """
    table = cie_xyz_table()
    keep = (table[:, 0] >= LAMBDA_MIN) & (table[:, 0] < LAMBDA_MAX)
    out = np.zeros((int(keep.sum()), 4), np.float32)
    out[:, :3] = table[keep, 1:4]
    return out
