"""Configuration dataclasses with the reference's field names and defaults.

Mirrors ``realflare/api/data.py:10-249`` without Qt: the reference stores sizes and points
as ``QtCore.QSize``/``QSizeF``/``QPointF``/``QPoint`` and reads them with ``.width()``,
``.height()``, ``.x()``, ``.y()``. The small value classes below keep that call syntax, so
code written against the reference's ``Project`` tree reads the same here. All classes are
frozen-free but hashable by value (the reference hashes them for its ``lru_cache`` keys).
"""
from __future__ import annotations

import dataclasses
import enum
from dataclasses import dataclass, field
from typing import Any


class RealflareError(ValueError):
    """User-facing error (``realflare/api/data.py:10-11``)."""


@dataclass(eq=True, frozen=False)
class QSize:
    w: int = 0
    h: int = 0

    def width(self) -> int:
        return self.w

    def height(self) -> int:
        return self.h

    def __hash__(self) -> int:
        return hash((self.w, self.h))


@dataclass(eq=True)
class QSizeF:
    w: float = 0.0
    h: float = 0.0

    def width(self) -> float:
        return self.w

    def height(self) -> float:
        return self.h

    def __hash__(self) -> int:
        return hash((self.w, self.h))


@dataclass(eq=True)
class QPointF:
    px: float = 0.0
    py: float = 0.0

    def x(self) -> float:
        return self.px

    def y(self) -> float:
        return self.py

    def setX(self, value: float) -> None:  # noqa: N802 - Qt spelling
        self.px = value

    def setY(self, value: float) -> None:  # noqa: N802 - Qt spelling
        self.py = value

    def __hash__(self) -> int:
        return hash((self.px, self.py))


QPoint = QPointF


def _hashable(cls):
    """Dataclass whose hash is computed from its field values (lists become tuples)."""
    cls = dataclass(eq=True)(cls)

    def __hash__(self):
        values = []
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, list):
                v = tuple(v)
            values.append(v)
        return hash(tuple(values))

    cls.__hash__ = __hash__
    return cls


class AntiAliasing(enum.Enum):
    ONE = 1
    TWO = 2
    FOUR = 4
    EIGHT = 8


@enum.unique
class RenderElement(enum.Enum):
    STARBURST_APERTURE = enum.auto()
    STARBURST = enum.auto()
    GHOST_APERTURE = enum.auto()
    GHOST = enum.auto()
    FLARE = enum.auto()
    FLARE_STARBURST = enum.auto()
    DIAGRAM = enum.auto()


@_hashable
class Glass:
    name: str
    manufacturer: str
    n: float
    v: float
    coefficients: list = field(repr=False, default_factory=list)


@_hashable
class LensElement:
    radius: float = 0
    distance: float = 0
    refractive_index: float = 1
    abbe_nr: float = 0
    height: float = 0


@_hashable
class LensModel:
    name: str = 'New Model'
    year: int = 0
    patent_number: str = ''
    notes: str = ''
    focal_length: float = 0
    fstop: float = 0
    aperture_index: int = 0
    lens_elements: list = field(default_factory=list)

    LensElement = LensElement


@_hashable
class ApertureShape:
    size: QSizeF = field(default_factory=lambda: QSizeF(0.75, 0.75))
    blades: int = 6
    roundness: float = 0
    rotation: float = 0
    softness: float = 0


@_hashable
class ApertureGrating:
    strength: float = 0
    density: float = 0.5
    length: float = 0.5
    width: float = 0.25
    softness: float = 0


@_hashable
class ApertureScratches:
    strength: float = 0
    density: float = 0.5
    length: float = 0.5
    width: float = 0.25
    rotation: float = 0
    rotation_variation: float = 0
    softness: float = 0
    parallax: QSizeF = field(default_factory=lambda: QSizeF(0, 0))


@_hashable
class ApertureDust:
    strength: float = 0
    density: float = 0.5
    radius: float = 0.5
    softness: float = 0
    parallax: QSizeF = field(default_factory=lambda: QSizeF(0, 0))
    # Extension with no reference counterpart: uniform noise blurred by a Gaussian of this
    # standard deviation in pixels replaces the hash-placed circles when > 0.
    blur_sigma: float = 0
    seed: int = 0


@_hashable
class ApertureImage:
    strength: float = 0
    file: str = ''
    size: QSizeF = field(default_factory=lambda: QSizeF(0.75, 0.75))
    threshold: float = 1


@_hashable
class Aperture:
    shape: ApertureShape = field(default_factory=ApertureShape)
    grating: ApertureGrating = field(default_factory=ApertureGrating)
    scratches: ApertureScratches = field(default_factory=ApertureScratches)
    dust: ApertureDust = field(default_factory=ApertureDust)
    image: ApertureImage = field(default_factory=ApertureImage)

    Shape = ApertureShape
    Grating = ApertureGrating
    Scratches = ApertureScratches
    Dust = ApertureDust
    ApertureImage = ApertureImage


@_hashable
class FlareLight:
    intensity: float = 1
    position: QPointF = field(default_factory=lambda: QPointF(0, 0))
    image_file_enabled: bool = False
    image_file: str = ''
    image_sample_resolution: int = 256
    image_samples: int = 8
    show_image: bool = False


@_hashable
class FlareLens:
    sensor_size: QSizeF = field(default_factory=lambda: QSizeF(36, 24))
    fstop: float = 0
    lens_model_path: str = ''
    glasses_path: str = ''
    abbe_nr_adjustment: float = 0
    coating: tuple = field(default_factory=tuple)
    coating_range: QPoint = field(default_factory=lambda: QPointF(390, 730))
    coating_min_ior: float = 1.38
    min_area: float = 0.01
    # Extensions with no reference counterpart (default off): explicit coating
    # thicknesses in nm per element. One value per element selects the reference's
    # single-layer formula with that thickness instead of lambda0 / (4 nc); two values
    # select an exact two-layer thin-film stack with indices ``coating_layer_ior``.
    coating_thickness: tuple = field(default_factory=tuple)
    coating_layer_ior: tuple = (1.38, 1.65)
    # A lens model can be given directly instead of by path (synthetic lenses).
    lens_model: Any = None
    # Explicit ghost paths ((bounce1, bounce2) element pairs); empty = the reference's
    # ray_paths (same-side pairs).
    ghost_paths: tuple = field(default_factory=tuple)


@_hashable
class FlareStarburst:
    intensity: float = 1
    scale: QSizeF = field(default_factory=lambda: QSizeF(1, 1))
    distance: float = 1
    blur: float = 0
    rotation: float = 0
    rotation_weight: float = 1
    vignetting_enabled: bool = False
    vignetting: QPointF = field(default_factory=lambda: QPointF(0.75, 1))
    # Extension with no reference counterpart: one diffraction spectrum per render
    # wavelength instead of one at 560 nm scaled radially.
    per_wavelength: bool = False


@_hashable
class FlareGhost:
    fstop: float = 0


@_hashable
class Flare:
    light: FlareLight = field(default_factory=FlareLight)
    lens: FlareLens = field(default_factory=FlareLens)
    starburst_aperture: Aperture = field(default_factory=Aperture)
    starburst: FlareStarburst = field(default_factory=FlareStarburst)
    ghost_aperture: Aperture = field(default_factory=Aperture)
    ghost: FlareGhost = field(default_factory=FlareGhost)

    Light = FlareLight
    Lens = FlareLens
    Starburst = FlareStarburst
    Ghost = FlareGhost


@_hashable
class Output:
    element: RenderElement = RenderElement.FLARE
    path: str = ''
    colorspace: str = 'ACES - ACEScg'
    split_files: bool = True
    write: bool = False
    frame: int = 0


@_hashable
class Diagram:
    resolution: QSize = field(default_factory=lambda: QSize(2048, 1024))
    debug_ghost: int = 0
    light_position: float = 0
    grid_count: int = 8
    grid_length: float = 50
    column_offset: int = 0


@_hashable
class RenderStarburst:
    resolution: QSize = field(default_factory=lambda: QSize(256, 256))
    samples: int = 100


@_hashable
class RenderGhost:
    resolution: QSize = field(default_factory=lambda: QSize(256, 256))


@_hashable
class Render:
    resolution: QSize = field(default_factory=lambda: QSize(512, 512))
    bin_size: int = 64
    anti_aliasing: int = 1
    wavelength_count: int = 1
    wavelength_sub_count: int = 1
    grid_count: int = 33
    grid_length: float = 50
    cull_percentage: float = 0
    debug_ghost_enabled: bool = False
    debug_ghost: int = 0
    starburst: RenderStarburst = field(default_factory=RenderStarburst)
    ghost: RenderGhost = field(default_factory=RenderGhost)
    device: str = ''
    # Extension: explicit wavelengths in nm (floats). Empty = the reference's
    # ``wavelength_array(wavelength_count)`` truncated to int nm.
    wavelengths: tuple = field(default_factory=tuple)

    Starburst = RenderStarburst
    Ghost = RenderGhost


@_hashable
class Project:
    output: Output = field(default_factory=Output)
    flare: Flare = field(default_factory=Flare)
    render: Render = field(default_factory=Render)
    diagram: Diagram = field(default_factory=Diagram)


def _cast(cls, data):
    """Build a dataclass tree from JSON-like data (the reference uses qt_extensions.cast)."""
    if not dataclasses.is_dataclass(cls) or not isinstance(data, dict):
        return data
    kwargs = {}
    hints = {f.name: f for f in dataclasses.fields(cls)}
    defaults = cls()
    for key, value in data.items():
        if key not in hints:
            continue
        current = getattr(defaults, key)
        if dataclasses.is_dataclass(current):
            if isinstance(current, (QSize, QSizeF, QPointF)) and isinstance(value, (list, tuple)):
                kwargs[key] = type(current)(*value)
            else:
                kwargs[key] = _cast(type(current), value)
        elif key == 'lens_elements':
            kwargs[key] = [LensElement(**e) for e in value]
        elif isinstance(current, enum.Enum):
            kwargs[key] = type(current)[value] if isinstance(value, str) else type(current)(value)
        elif isinstance(current, tuple):
            kwargs[key] = tuple(value)
        else:
            kwargs[key] = value
    return cls(**kwargs)


def cast(cls, data):
    return _cast(cls, data)
