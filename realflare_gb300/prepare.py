"""Host-side argument preparation for the render path.

Restates the host halves of ``RaytracingTask.raytrace`` (``realflare/api/tasks/raytracing.py:
140-221``) and ``RasterizingTask.rasterize`` (``realflare/api/tasks/rasterizing.py:296-421``):
lens elements, ghost paths, wavelengths and light direction for the trace; screen transform,
quad area, bin sizes and scale factors for the raster.
"""
from __future__ import annotations

import copy
from dataclasses import dataclass

import numpy as np

from . import lens as lens_mod
from ._abi import RasterArgs, TraceArgs
from .data import Project, QPointF, QSize, RealflareError


@dataclass
class TraceInputs:
    elements: np.ndarray      # rf_lens_element[E]
    paths: np.ndarray         # int32 [P, 2]
    wavelengths: np.ndarray   # float32 [W]
    args: TraceArgs

    @property
    def ray_count(self) -> int:
        return self.args.path_count * self.args.wavelength_count * self.args.grid_count**2


def trace_inputs(project: Project, paths=None, path_indexes: tuple = ()) -> TraceInputs | None:
    """Inputs of one trace; None when the lens has fewer than two elements
    (``raytracing.py:164-165``). ``paths`` overrides the reference's ``ray_paths``."""
    lens = project.flare.lens
    model = lens_mod.resolve_model(lens)
    sensor_size = (lens.sensor_size.width(), lens.sensor_size.height())
    elements = lens_mod.elements(
        model, sensor_size, lens.glasses_path, lens.abbe_nr_adjustment, tuple(lens.coating),
        tuple(lens.coating_thickness),
    )
    if len(elements) <= 1:
        return None
    if paths is None and lens.ghost_paths:
        paths = list(lens.ghost_paths)
        if path_indexes:
            paths = [pp for i, pp in enumerate(paths) if i in path_indexes]
    if paths is None:
        paths = lens_mod.ray_paths(model, tuple(path_indexes))
    paths = np.asarray(paths, np.int32).reshape(-1, 2)
    wavelengths = lens_mod.render_wavelengths(project.render)
    render = project.render
    light = project.flare.light
    direction = lens_mod.direction(
        (light.position.x(), light.position.y()), render.resolution, sensor_size, model.focal_length
    )
    a = TraceArgs()
    a.element_count = len(elements)
    a.aperture_index = model.aperture_index
    a.path_count = len(paths)
    a.wavelength_count = len(wavelengths)
    a.grid_count = render.grid_count
    a.grid_length = render.grid_length
    a.coating_min_ior = lens.coating_min_ior
    a.coating_layer_ior[0] = lens.coating_layer_ior[0]
    a.coating_layer_ior[1] = lens.coating_layer_ior[1]
    for i in range(4):
        a.direction[i] = float(direction[i])
    if a.grid_count < 2:
        raise RealflareError('grid_count must be >= 2')
    return TraceInputs(elements, paths, wavelengths, a)


def raster_args(project: Project, path_count: int, wavelength_count: int, ghost_shape: tuple,
                tile_size: int = 0) -> RasterArgs:
    render = project.render
    lens = project.flare.lens
    sensor_size = (lens.sensor_size.width(), lens.sensor_size.height())
    a = RasterArgs()
    a.width = render.resolution.width()
    a.height = render.resolution.height()
    a.bin_size = max(render.bin_size, 1)
    a.tile_size = tile_size
    a.path_count = path_count
    a.wavelength_count = wavelength_count
    # rasterizing.py:390-392: sub-wavelengths only with more than one wavelength
    a.wavelength_sub_count = render.wavelength_sub_count if wavelength_count > 1 else 1
    a.grid_count = render.grid_count
    a.sub_steps = render.anti_aliasing
    a.screen_transform = lens_mod.screen_transform(render.resolution, sensor_size)
    a.intensity = float(np.float32(project.flare.light.intensity * 1e3))
    a.ghost_scale = 1 - lens.fstop / 32
    a.ghost_height, a.ghost_width = ghost_shape[0], ghost_shape[1]
    if a.sub_steps not in (1, 2, 4, 8):
        raise RealflareError('anti_aliasing must be 1, 2, 4 or 8')
    return a


def quad_constants(project: Project) -> tuple:
    """(area_orig, rel_min_area) of ``rasterizing.py:328-329``."""
    area = lens_mod.area_orig(project.render.grid_count, project.render.grid_length)
    return area, project.flare.lens.min_area * area


def diagram_project(project: Project) -> Project:
    """The project IntersectionsTask traces (``raytracing.py:362-380``): light at
    (0, diagram.light_position), the diagram's grid, grid length and resolution (which sets
    the light direction's aspect), one wavelength."""
    p = copy.deepcopy(project)
    d = project.diagram
    p.flare.light.position = QPointF(0.0, float(d.light_position))
    p.render.grid_count = d.grid_count
    p.render.grid_length = d.grid_length
    p.render.resolution = QSize(d.resolution.width(), d.resolution.height())
    p.render.wavelength_count = 1
    p.render.wavelengths = ()
    return p


def intersection_count(element_count: int) -> int:
    """Hit records per ray (``raytracing.py:326``): three per element, less one."""
    return element_count * 3 - 1


def diagram_scale(project: Project) -> float:
    """Pixels per mm of the diagram (``diagram.py:45-57``): the image width less 10 pixels of
    padding over the lens model's total element distance (1 when that is 0)."""
    model = lens_mod.resolve_model(project.flare.lens)
    distance = 0.0
    for e in model.lens_elements:
        distance += e.distance
    if distance == 0:
        return 1.0
    return (project.diagram.resolution.width() - 10) / distance
