"""Seeded synthetic lenses and the benchmark workloads built on them.

Lens recipe (n spherical surfaces, ``numpy.random.Generator(PCG64(seed))``):

* radii ``|r| ~ U[20, 120]`` mm with a random sign; axial gaps ``U[2, 12]`` mm;
* media alternate: glass after even-indexed surfaces, air after odd-indexed ones; glass
  ``n_d ~ U[1.50, 1.75]``, ``V_d ~ U[30, 60]``; Sellmeier coefficients then come from the
  closest Schott glass, as for any lens model;
* semi-heights 15 mm; a flat stop (radius 0, n 1, height 8 mm) is inserted as element
  ``n/2``, halving the air gap after surface ``n/2``;
* the last gap (to the sensor) is the paraxial back focal distance and ``focal_length`` is
  the paraxial focal length (fallbacks 50 mm when the paraxial values are unusable).

Draw order: magnitudes, signs, gaps, n_d, V_d (all n values each, gaps n-1), so a lens of
a given (n, seed) is fixed. Two-layer coating thicknesses use a second generator seeded
``seed + 1000`` so they do not move the geometry.

Lens acceptance: random radii with random signs often give a system that no ray survives
(at seed 0, 0.6 % of the 16-surface lens's ghost rays and 1.8 % of the 24-surface lens's
reach the sensor). The workloads therefore use, per surface count, the first seed
0, 1, 2, ... whose two-bounce ghost rays reach the sensor for at least
``ACCEPT_FRACTION`` of a 12 x 12 grid over ``GRID_LENGTH`` at 550 nm with the
workload's light position.
``LENS_SEEDS`` records the result of that rule (checked by the CPU tests); the 8-surface
lens is accepted at seed 0.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import lens as lens_mod
from .data import (
    Aperture,
    ApertureDust,
    ApertureShape,
    FlareLens,
    LensElement,
    LensModel,
    Project,
    QPointF,
    QSize,
    QSizeF,
)

SEMI_HEIGHT = 15.0
STOP_HEIGHT = 8.0
GRID_LENGTH = 30.0
ACCEPT_FRACTION = 0.4
LENS_SEEDS = {8: 0, 16: 10, 24: 11}


def make_lens(n_surfaces: int, seed: int = 0) -> LensModel:
    if n_surfaces < 2 or n_surfaces % 2:
        raise ValueError('n_surfaces must be even and >= 2')
    rng = np.random.Generator(np.random.PCG64(seed))
    magnitude = rng.uniform(20.0, 120.0, n_surfaces)
    sign = rng.choice(np.array([-1.0, 1.0]), n_surfaces)
    gaps = rng.uniform(2.0, 12.0, n_surfaces - 1)
    nd = rng.uniform(1.50, 1.75, n_surfaces)
    vd = rng.uniform(30.0, 60.0, n_surfaces)

    stop = n_surfaces // 2
    elements = []
    for i in range(n_surfaces):
        glass_after = i % 2 == 0
        gap = float(gaps[i]) if i < n_surfaces - 1 else 0.0
        if i == stop - 1:
            gap = gap / 2
        elements.append(
            LensElement(
                radius=float(magnitude[i] * sign[i]),
                distance=gap,
                refractive_index=float(nd[i]) if glass_after else 1.0,
                abbe_nr=float(vd[i]) if glass_after else 0.0,
                height=SEMI_HEIGHT,
            )
        )
        if i == stop - 1:
            elements.append(
                LensElement(radius=0.0, distance=gap, refractive_index=1.0, abbe_nr=0.0, height=STOP_HEIGHT)
            )
    model = LensModel(name=f'synthetic-{n_surfaces}-seed{seed}', aperture_index=stop, lens_elements=elements)
    efl, bfd = lens_mod.paraxial(model)
    if not (math.isfinite(bfd) and 5.0 <= bfd <= 500.0):
        bfd = 50.0
    if not (math.isfinite(efl) and 10.0 <= abs(efl) <= 1000.0):
        efl = 50.0
    elements[-1].distance = float(bfd)
    model.focal_length = float(abs(efl))
    return model


def two_layer_thickness(n_elements: int, seed: int = 0) -> tuple:
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    t = rng.uniform(80.0, 150.0, (n_elements, 2))
    return tuple((float(a), float(b)) for a, b in t)


@dataclass
class Workload:
    """One benchmark/parity workload: a project plus the explicit ghost path list."""

    name: str
    project: Project
    paths: list = field(default_factory=list)

    @property
    def model(self) -> LensModel:
        return self.project.flare.lens.lens_model


def _project(model, grid, wavelengths, light, resolution, coating, thickness=()) -> Project:
    p = Project()
    p.flare.lens = FlareLens(
        sensor_size=QSizeF(36, 24),
        lens_model=model,
        glasses_path='$GLASS/schott',
        coating=coating,
        coating_thickness=thickness,
        coating_min_ior=1.38,
        min_area=0.01,
    )
    p.flare.light.position = QPointF(*light)
    p.flare.light.intensity = 1.0
    p.render.resolution = QSize(resolution, resolution)
    p.render.grid_count = grid
    p.render.grid_length = GRID_LENGTH
    p.render.wavelength_count = len(wavelengths)
    p.render.wavelengths = tuple(float(w) for w in wavelengths)
    p.render.bin_size = 64
    p.render.anti_aliasing = 1
    p.render.wavelength_sub_count = 1
    return p


def workload(name: str, integer_wavelengths: bool = False) -> Workload:
    """Named workloads.

    * ``plain-8``: 8-surface lens, 28 ghosts, 32x32 grid, 550 nm, light (0.2, 0.1), 512x512.
    * ``spectral-16``: 16 surfaces, 120 ghosts, 64x64 grid, 8 wavelengths over 400-700 nm,
      light (0.35, -0.2), 1024x1024.
    * ``production-24``: 24 surfaces, 276 ghosts, 128x128 grid, 16 wavelengths over
      390-700 nm, two-layer coatings 80-150 nm, light (0.3, 0.2), 2048x2048, plus a 512x512
      8-blade starburst aperture with Gaussian-blurred (sigma 2 px) uniform dust.
    * ``differentiable-16``: the 16-surface lens at 512x512, 64x64 grid, 8 wavelengths,
      single-layer coatings with explicit thickness (lambda0/(4*1.38) at 550 nm).

    ``integer_wavelengths`` rounds wavelengths to whole nm (the reference's int32 buffer).
    """
    if name == 'plain-8':
        model = make_lens(8, LENS_SEEDS[8])
        wl = [550.0]
        p = _project(model, 32, wl, (0.2, 0.1), 512, (550,) * (len(model.lens_elements) + 1))
    elif name == 'spectral-16':
        model = make_lens(16, LENS_SEEDS[16])
        wl = np.linspace(400.0, 700.0, 8)
        p = _project(model, 64, wl, (0.35, -0.2), 1024, (550,) * (len(model.lens_elements) + 1))
    elif name == 'production-24':
        model = make_lens(24, LENS_SEEDS[24])
        wl = np.linspace(390.0, 700.0, 16)
        n_el = len(model.lens_elements) + 1
        p = _project(
            model, 128, wl, (0.3, 0.2), 2048, (550,) * n_el,
            two_layer_thickness(n_el, LENS_SEEDS[24]),
        )
        p.render.starburst.resolution = QSize(512, 512)
        p.flare.starburst_aperture = Aperture(
            shape=ApertureShape(size=QSizeF(0.75, 0.75), blades=8, softness=0.0),
            dust=ApertureDust(strength=1.0, blur_sigma=2.0, seed=0),
        )
    elif name == 'differentiable-16':
        model = make_lens(16, LENS_SEEDS[16])
        wl = np.linspace(400.0, 700.0, 8)
        n_el = len(model.lens_elements) + 1
        p = _project(
            model, 64, wl, (0.35, -0.2), 512, (550,) * n_el, (550.0 / (4 * 1.38),) * n_el
        )
    else:
        raise KeyError(name)
    if integer_wavelengths:
        p.render.wavelengths = tuple(float(int(round(w))) for w in p.render.wavelengths)
    paths = lens_mod.all_two_bounce_paths(model)
    p.flare.lens.ghost_paths = tuple(tuple(pp) for pp in paths)
    return Workload(name, p, paths)


BATCH_SURFACES = (8, 16, 24)
BATCH_GRIDS = (32, 64, 128)


def batched_projects(count: int = 256, seed: int = 0, resolution: int = 1024, surfaces: tuple = BATCH_SURFACES,
                     grids: tuple = BATCH_GRIDS, max_wavelengths: int = 16) -> list:
    """Frame requests of the batched form: per request a lens drawn from the 8-, 16- and
    24-surface workload lenses (all their two-bounce ghosts: 28 / 120 / 276), a grid of
    32^2, 64^2 or 128^2, 1-16 wavelengths spread over 390-700 nm (550 nm for one) and a
    light position uniform over the normalised field, rendered at resolution^2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    names = {8: 'plain-8', 16: 'spectral-16', 24: 'production-24'}
    lenses = {n: workload(names[n]) for n in surfaces}
    projects = []
    for _ in range(count):
        n = int(rng.choice(np.array(surfaces)))
        grid = int(rng.choice(np.array(grids)))
        w = int(rng.integers(1, max_wavelengths + 1))
        light = rng.uniform(-1.0, 1.0, 2)
        base = lenses[n].project
        wl = [550.0] if w == 1 else list(np.linspace(390.0, 700.0, w))
        p = _project(base.flare.lens.lens_model, grid, wl, (float(light[0]), float(light[1])), resolution,
                     base.flare.lens.coating, base.flare.lens.coating_thickness)
        p.flare.lens.ghost_paths = base.flare.lens.ghost_paths
        projects.append(p)
    return projects
