"""Animated renders: per-frame values applied to a project, frames rendered in batches.

The reference's command line renders frame_start..frame_end by setting
``project.output.frame`` and applying frame i's animation values to the same project
before each ``Engine.render`` (``realflare/cli/app.py:22-41,86-97``). ``frame_projects``
keeps those semantics (values persist until a later frame changes them);
``render_frames`` renders the frames. Single-light flare frames go through
``BatchRenderer`` (one launch per stage for a group of frames, images bit-identical to
``Engine.render``); any other frame (another render element, a light image, a debug
ghost, ghost culling) goes through ``Engine.render`` one frame at a time. Argument parsing
and file output (EXR) stay with the caller.
"""
from __future__ import annotations

import copy
import dataclasses
import enum
from typing import Any

import torch

from .data import Project, QPointF, QSize, QSizeF, RealflareError, RenderElement, cast


_PLAIN = {'float': float, 'int': int, 'bool': bool, 'str': str}


def cast_value(current: Any, value: Any, annotation: Any = None) -> Any:
    """``value`` converted to the attribute's type: the field's declared type when it is a
    plain one, else the type of its current value (the reference casts to the dataclass
    field's type with qt_extensions.cast)."""
    plain = _PLAIN.get(annotation) if isinstance(annotation, str) else (
        annotation if annotation in _PLAIN.values() else None)
    if plain is not None and isinstance(value, (int, float, bool, str)):
        return plain(value)
    if isinstance(current, (QSize, QSizeF, QPointF)) and isinstance(value, (list, tuple)):
        return type(current)(*value)
    if isinstance(current, enum.Enum):
        return type(current)[value] if isinstance(value, str) else type(current)(value)
    if dataclasses.is_dataclass(current) and isinstance(value, dict):
        return cast(type(current), value)
    if isinstance(current, tuple) and isinstance(value, list):
        return tuple(value)
    if isinstance(current, bool):
        return bool(value)
    if isinstance(current, (int, float)) and isinstance(value, (int, float)) and not isinstance(value, bool):
        return type(current)(value)
    return value


def apply_animation(obj: Any, animation: dict, index: int) -> None:
    """Set frame ``index``'s values on obj (cli/app.py:22-41). A list holds one value per
    frame; past its end the attribute keeps its value. A dict descends into the attribute
    of that name; names obj lacks are skipped."""
    for name, value in animation.items():
        if isinstance(value, list):
            try:
                current_value = value[index]
            except IndexError:
                continue
            if dataclasses.is_dataclass(obj):
                fields = {f.name: f.type for f in dataclasses.fields(obj)}
                if name in fields:
                    current_value = cast_value(getattr(obj, name), current_value, fields[name])
            setattr(obj, name, current_value)
        elif isinstance(value, dict):
            try:
                child = getattr(obj, name)
            except AttributeError:
                continue
            apply_animation(child, value, index)
        else:
            raise RealflareError(f'animation value of {name!r} must be a list of frame values or a dict')


def frame_projects(project: Project, animation: dict | None = None, frame_start: int = 1,
                   frame_end: int = 1) -> list:
    """The project of every frame of frame_start..frame_end (inclusive), as the command
    line's loop sets it before each render (cli/app.py:86-97)."""
    if frame_end < frame_start:
        raise RealflareError('frame_end must not be before frame_start')
    p = copy.deepcopy(project)
    frames = []
    for i, frame in enumerate(range(frame_start, frame_end + 1)):
        p.output.frame = frame
        if animation:
            apply_animation(p, animation, i)
        frames.append(copy.deepcopy(p))
    return frames


def _batchable(p: Project) -> bool:
    r, light = p.render, p.flare.light
    return (p.output.element == RenderElement.FLARE and not r.debug_ghost_enabled and r.cull_percentage <= 0
            and not light.image_file_enabled)


def render_frames(project: Project, animation: dict | None = None, frame_start: int = 1, frame_end: int = 1,
                  engine=None, max_bytes: int = 0) -> list:
    """Every frame's image (a (height, width, 4) RGBA device tensor), in frame order.
    Batched flare frames are grouped so that a group's buffers stay within max_bytes
    (0: 30 % of the free device memory)."""
    from .batch import BatchRenderer, group_frames
    from .engine import Engine

    projects = frame_projects(project, animation, frame_start, frame_end)
    images: list = [None] * len(projects)
    batched = [i for i, p in enumerate(projects) if _batchable(p)]
    if batched:
        if max_bytes <= 0:
            free, _ = torch.cuda.mem_get_info()
            max_bytes = int(0.3 * free)
        stream = torch.cuda.Stream()
        frames = [projects[i] for i in batched]
        for group in group_frames(frames, max_bytes):
            b = BatchRenderer([frames[k] for k in group], stream=stream)
            out = b.run()
            with torch.cuda.stream(stream):
                for k, img in zip(group, out):
                    images[batched[k]] = img.clone()
            del b
        stream.synchronize()
    rest = [i for i in range(len(projects)) if images[i] is None]
    if rest:
        engine = engine if engine is not None else Engine()
        for i in rest:
            if not engine.render(projects[i]):
                raise RealflareError(f'an error occurred while rendering frame {frame_start + i}')
            images[i] = engine.image.tensor.clone()  # the engine may reuse its buffers
    return images
