"""Glass catalogue lookup (``realflare/api/glass.py``).

The catalogue is the Schott table extracted once into ``resources/schott.json``
(see ``resources/make_resources.py``). ``glasses_from_path`` accepts the reference's
``glasses_path`` values: ``'$GLASS/schott'``/``'$RES/glass/schott'``/a directory named
``schott``/an empty string select the bundled Schott table; a directory holding
refractiveindex.info YAML files is parsed like the reference parses it.
"""
from __future__ import annotations

import json
import math
import os
from functools import lru_cache

import numpy as np

from .constants import RESOURCES
from .data import Glass


@lru_cache(1)
def _bundled_schott() -> tuple:
    with open(os.path.join(RESOURCES, 'schott.json'), encoding='utf-8') as f:
        rows = json.load(f)
    return tuple(
        Glass(r['name'], r['manufacturer'], r['n'], r['v'], list(r['coefficients'])) for r in rows
    )


def manufacturers() -> dict:
    return {'schott': '$GLASS/schott'}


def glasses_from_path(dir_path: str = '$GLASS/schott') -> list:
    """Glasses of one manufacturer, in the catalogue's file-name order (``glass.py:32-70``)."""
    if dir_path is None:
        return []
    normalized = dir_path.replace('\\', '/').rstrip('/')
    if normalized in ('', '$GLASS/schott', '$RES/glass/schott') or (
        os.path.basename(normalized) == 'schott' and not os.path.isdir(dir_path)
    ):
        return list(_bundled_schott())
    if not os.path.isdir(dir_path):
        return []
    from .resources.make_resources import _parse_glass_yaml

    glasses = []
    for file_name in sorted(os.listdir(dir_path)):
        if not file_name.endswith(('.yml', '.yaml')):
            continue
        path = os.path.join(dir_path, file_name)
        if not os.path.isfile(path):
            continue
        with open(path, encoding='utf-8') as f:
            parsed = _parse_glass_yaml(f.read())
        if parsed is None:
            continue
        nd, vd, coefficients = parsed
        glasses.append(
            Glass(os.path.splitext(file_name)[0], os.path.basename(dir_path), nd, vd, coefficients)
        )
    return glasses


@lru_cache(64)
def closest_glass(glasses: tuple, n: float, v: float, v_offset: float = 0):
    """Nearest glass by relative (n, V) distance (``realflare/api/glass.py:73-87``)."""
    if n == 0 or v == 0 or not glasses:
        return None
    glass_array = np.array([(g.n, g.v) for g in glasses])
    differences = 1 - glass_array / np.array((n, v + v_offset))
    lengths = np.sum(np.power(differences, 2), axis=1)
    return glasses[int(np.argmin(lengths))]


def sellmeier(coefficients, wavelength: float) -> float:
    """n(lambda) with lambda in nm (``realflare/api/glass.py:90-99``)."""
    wavelength *= 1e-3
    l2 = wavelength * wavelength
    d0 = (coefficients[0] * l2) / (l2 - coefficients[1])
    d1 = (coefficients[2] * l2) / (l2 - coefficients[3])
    d2 = (coefficients[4] * l2) / (l2 - coefficients[5])
    return math.sqrt(1 + d0 + d1 + d2)
