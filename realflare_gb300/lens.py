"""Lens model → device lens elements, ghost paths, wavelengths and light direction.

Restates ``realflare/api/lens.py:25-113`` and the small host helpers of
``realflare/api/tasks/raytracing.py:28-34,92-106``.
"""
from __future__ import annotations

import json
import math
import os
from functools import lru_cache

import numpy as np

from . import glass
from .constants import LAMBDA_MAX, LAMBDA_MIN, RESOURCES, lens_element_dtype
from .data import LensElement, LensModel, RealflareError, cast


def model_from_path(lens_model_path: str) -> LensModel:
    """Load a lens model JSON file (``realflare/api/lens.py:25-37``)."""
    if not lens_model_path:
        raise RealflareError('No Lens Model')
    try:
        with open(lens_model_path, encoding='utf-8') as f:
            data = json.load(f)
        return cast(LensModel, data)
    except (OSError, ValueError, TypeError):
        raise RealflareError(f'Invalid Lens Model: {lens_model_path}') from None


def decode_path(path: str) -> str:
    """``$RES`` names the bundled resources (the reference's ``storage.decode_path``,
    ``realflare/storage.py:80,139-150``, maps it to its own resources directory); other
    variables expand from the environment."""
    normalized = path.replace('\\', '/')
    if normalized == '$RES' or normalized.startswith('$RES/'):
        path = os.path.join(RESOURCES, *normalized[len('$RES/'):].split('/'))
    return os.path.expandvars(path)


def resolve_model(lens) -> LensModel:
    """The lens model of a ``Flare.Lens``: a model object or a JSON path (``$RES/model/...``
    selects one of the bundled prescriptions)."""
    if lens.lens_model is not None:
        return lens.lens_model
    return model_from_path(decode_path(lens.lens_model_path))


@lru_cache(16)
def _catalogue(glasses_path: str) -> tuple:
    """The glasses of a catalogue directory, read once per path (the reference caches its
    lens elements per glasses path the same way, ``raytracing.py:54-73``)."""
    return tuple(glass.glasses_from_path(glasses_path))


@lru_cache(4096)
def _closest_coefficients(glasses_path: str, n: float, v: float, v_offset: float):
    """Sellmeier coefficients of the closest catalogue glass, or None; keyed by the
    catalogue's path rather than its glasses, which are costly to hash."""
    closest = glass.closest_glass(_catalogue(glasses_path), n, v, v_offset)
    return tuple(closest.coefficients[:6]) if closest else None


def elements(
    lens_model: LensModel,
    sensor_size: tuple,
    glasses_path: str,
    abbe_nr_adjustment: float,
    coating: tuple,
    coating_thickness: tuple = (),
) -> np.ndarray:
    """Device lens elements incl. the appended sensor (``realflare/api/lens.py:40-86``).

    ``center = sum(distance of previous elements) + radius``; the sensor is a flat element
    of height ``|sensor|/2``; the Sellmeier coefficients come from the closest catalogue
    glass; with an empty catalogue coefficient 0 of element 0 is NaN, which turns
    dispersion off in the trace. ``coating_thickness`` (extension): per element either a
    number (single layer with that thickness in nm) or a pair (two-layer stack).
    """
    lens_elements = list(lens_model.lens_elements)
    sensor_length = float(np.linalg.norm(sensor_size) / 2)
    lens_elements.append(LensElement(height=sensor_length))
    glasses = _catalogue(glasses_path)

    array = np.zeros(len(lens_elements), lens_element_dtype)
    if not glasses:
        array[0]['coefficients'][0] = np.nan
    offset = 0.0
    for i, element in enumerate(lens_elements):
        array[i]['radius'] = element.radius
        array[i]['ior'] = element.refractive_index
        array[i]['height'] = element.height
        array[i]['center'] = offset + element.radius
        if i < len(coating):
            array[i]['coating'] = coating[i]
        if i < len(coating_thickness) and coating_thickness[i] is not None:
            t = coating_thickness[i]
            if np.ndim(t) == 0:
                array[i]['coating_layers'] = 1
                array[i]['coating_thickness'][0] = t
            else:
                array[i]['coating_layers'] = 2
                array[i]['coating_thickness'][:] = t[:2]
        coefficients = _closest_coefficients(glasses_path, element.refractive_index, element.abbe_nr,
                                             abbe_nr_adjustment)
        if coefficients:
            array[i]['coefficients'][:6] = coefficients
        offset += element.distance
    return array


def ray_paths(lens_model: LensModel, path_indexes: tuple = ()) -> list:
    """Two-bounce ghost paths (``realflare/api/lens.py:89-113``).

    ``(bounce1, bounce2)`` with ``bounce2 < bounce1 <= n-2``, both on the same side of
    the aperture.
    """
    paths = []
    count = len(lens_model.lens_elements)
    index_min = 0
    for bounce1 in range(1, count - 1):
        if bounce1 == lens_model.aperture_index:
            index_min = bounce1 + 1
        for bounce2 in range(index_min, bounce1):
            paths.append((bounce1, bounce2))
    if path_indexes:
        paths = [p for i, p in enumerate(paths) if i in path_indexes]
    if tuple(path_indexes) == (-1,):
        paths = [(-1, -1)]
    return paths


def all_two_bounce_paths(lens_model: LensModel) -> list:
    """Every pair of reflecting surfaces (b1 > b2), the stop excluded.

    Unlike ``ray_paths`` this includes pairs on both sides of the stop; the trace accepts
    any pair.
    """
    surfaces = [i for i in range(len(lens_model.lens_elements)) if i != lens_model.aperture_index]
    return [(b1, b2) for ai, b1 in enumerate(surfaces) for b2 in surfaces[:ai]]


def wavelength_array(wavelength_count: int) -> list:
    """Bin-centre wavelengths over [390, 730) nm (``raytracing.py:28-34``)."""
    array = []
    for i in range(wavelength_count):
        step = (i + 0.5) / wavelength_count
        array.append(LAMBDA_MIN + step * (LAMBDA_MAX - LAMBDA_MIN))
    return array


def render_wavelengths(render) -> np.ndarray:
    """float32 wavelengths of a render: explicit ones, else the reference's int32 array."""
    if render.wavelengths:
        return np.asarray(render.wavelengths, np.float32)
    return np.int32(wavelength_array(render.wavelength_count)).astype(np.float32)


def direction(position: tuple, resolution, sensor_size: tuple, focal_length: float) -> np.ndarray:
    """Light direction float4 (``raytracing.py:92-106``)."""
    sensor_length = sensor_size[0] / 2
    ratio = resolution.height() / resolution.width()
    d = np.ones(4, np.float32)
    d[0] = position[0] * sensor_length
    d[1] = position[1] * ratio * sensor_length
    d[2] = focal_length
    return d


def screen_transform(resolution, sensor_size: tuple) -> float:
    """Pixels per mm along the half diagonal (``rasterizing.py:158-167``)."""
    sensor_length = float(np.linalg.norm((sensor_size[0], sensor_size[1])) / 2)
    try:
        return resolution.width() / sensor_length
    except ZeroDivisionError:
        return 0.0


def area_orig(grid_count: int, grid_length: float) -> float:
    """Area of one undistorted grid quad (``rasterizing.py:151-156``)."""
    grid_count = max(1, grid_count)
    quad_length = grid_length / (grid_count - 1)
    return quad_length**2


def paraxial(lens_model: LensModel, wavelength_ior=None):
    """(effective focal length, back focal distance) from ABCD ray-transfer matrices.

    Surfaces with radius 0 are flat. ``wavelength_ior`` optionally overrides the media
    indices. Used only to place the sensor and pick a focal length for synthetic lenses.
    """
    m = np.eye(2)
    n1 = 1.0
    elems = lens_model.lens_elements
    for i, e in enumerate(elems):
        n2 = e.refractive_index if wavelength_ior is None else wavelength_ior[i]
        power = 0.0 if e.radius == 0 else (n2 - n1) / e.radius
        refraction = np.array([[1.0, 0.0], [-power / n2, n1 / n2]])
        m = refraction @ m
        if i < len(elems) - 1:
            m = np.array([[1.0, e.distance], [0.0, 1.0]]) @ m
        n1 = n2
    a, b = m[0]
    c, d = m[1]
    if c == 0:
        return math.inf, math.inf
    efl = -1.0 / c
    bfd = -a / c
    return efl, bfd
