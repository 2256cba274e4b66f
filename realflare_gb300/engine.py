"""The render engine (``realflare/api/engine.py``): composes the tasks into render elements.

``Engine.render(project) -> bool`` renders ``project.output.element`` and keeps the result
in ``Engine.image``; ``flare``, ``starburst``, ``ghost``, ``flare_starburst`` and the two
aperture elements are available individually, as in the reference (engine.py:80-193).
User errors raise ``RealflareError`` inside and make ``render`` return False
(engine.py:195-223).
"""
from __future__ import annotations

import copy
import logging

import numpy as np
import torch

from . import prepare, tasks
from ._abi import check
from .data import Project, RealflareError, RenderElement
from .device import Image, empty, ptr

logger = logging.getLogger(__name__)


class Engine:
    """``accurate_trace=True`` selects the double-precision ray geometry of
    ``RaytracingTask(accurate=True)`` for the single-light flares this engine renders
    (image-based lights render through the batched path, whose trace is FP32)."""

    def __init__(self, device: str = '', cache: bool = True, accurate_trace: bool = False) -> None:
        self.cache = cache
        self.accurate_trace = accurate_trace
        self.queue = None
        self.image: Image | None = None
        self._device = device
        self._initialized = False

    def _init(self) -> None:
        # one stream plays the role of the reference's command queue (engine.py:44-75)
        self.queue = torch.cuda.Stream()
        self.ghost_aperture_task = tasks.GhostApertureTask(self.queue)
        self.starburst_aperture_task = tasks.StarburstApertureTask(self.queue)
        self.ghost_task = tasks.GhostTask(self.queue)
        self.starburst_task = tasks.StarburstTask(self.queue)
        self.raytracing_task = tasks.RaytracingTask(self.queue, cache=self.cache, accurate=self.accurate_trace)
        self.rasterizing_task = tasks.RasterizingTask(self.queue)
        self.preprocess_task = tasks.PreprocessTask(self.queue)
        self.image_sampling_task = tasks.ImageSamplingTask(self.queue)
        self.renderers = {
            RenderElement.STARBURST_APERTURE: self.starburst_aperture,
            RenderElement.GHOST_APERTURE: self.ghost_aperture,
            RenderElement.STARBURST: self.starburst,
            RenderElement.GHOST: self.ghost,
            RenderElement.FLARE: self.flare,
            RenderElement.FLARE_STARBURST: self.flare_starburst,
            RenderElement.DIAGRAM: self.diagram,
        }
        self.intersection_task = tasks.IntersectionsTask(self.queue)
        self.diagram_task = tasks.DiagramTask(self.queue)
        self._initialized = True

    def starburst_aperture(self, project: Project) -> Image:
        return self.starburst_aperture_task.run(project)

    def starburst(self, project: Project) -> Image:
        return self.starburst_task.run(project, self.starburst_aperture(project))

    def ghost_aperture(self, project: Project) -> Image:
        return self.ghost_aperture_task.run(project)

    def ghost(self, project: Project) -> Image:
        return self.ghost_task.run(project, self.ghost_aperture(project))

    def flare(self, project: Project) -> Image:
        # engine.py:157-172
        if project.render.debug_ghost_enabled:
            path_indexes = (project.render.debug_ghost,)
        elif project.render.cull_percentage > 0:
            path_indexes = self.preprocess_task.run(project)
        else:
            path_indexes = ()  # cull 0 keeps every path (preprocessing.py:86-89)
        if project.flare.light.image_file_enabled:
            return self.image_flare(project, path_indexes)
        ghost = self.ghost(project)
        rays = self.raytracing_task.run(project, path_indexes)
        return self.rasterizing_task.run(project, rays, ghost)

    def image_flare(self, project: Project, path_indexes: tuple = ()) -> Image:
        """A flare per light-image sample, mirrored into the four quadrants and weighted by
        the samples (engine.py:98-155). The samples' flares render as one batch (one
        launch per stage, realflare_gb300.batch) instead of one trace + raster each, and
        are accumulated on the device (rf_accumulate_mirrored) in the reference's order."""
        from .batch import BatchRenderer, group_frames

        ghost = self.ghost(project)
        sample_data = self.image_sampling_task.run(project)
        if project.flare.light.show_image:
            return Image(array=sample_data, args=(project.flare.light, project.render.resolution))
        height, width, _ = sample_data.shape
        half_width, half_height = int(width / 2), int(height / 2)
        # the paths the single-light trace would use (explicit ghost paths or ray_paths,
        # filtered by path_indexes), fixed for every sample's frame
        inputs = prepare.trace_inputs(project, path_indexes=path_indexes)
        paths = tuple(tuple(int(v) for v in pp) for pp in inputs.paths) if inputs is not None else ()
        frames, weights = [], []
        for y in range(half_height):
            for x in range(half_width):
                values = np.float32([sample_data[y, x], sample_data[height - y - 1, x],
                                     sample_data[height - y - 1, width - x - 1], sample_data[y, width - x - 1]])
                if np.sum(values) == 0:
                    continue
                p = copy.deepcopy(project)
                p.flare.light.position = type(p.flare.light.position)((x + 0.5) / half_width - 1,
                                                                      1 - (y + 0.5) / half_height)
                p.flare.lens.ghost_paths = paths
                frames.append(p)
                weights.append(values)
        r = project.render.resolution
        out = empty((r.height(), r.width(), 4))
        out.zero_()
        if frames and paths:
            tex = ghost.tensor
            gshape = tuple(tex.shape[:2])
            free, _ = torch.cuda.mem_get_info()
            for group in group_frames(frames, int(0.3 * free)):
                b = BatchRenderer([frames[i] for i in group], stream=self.queue,
                                  ghosts=(tex.reshape(-1), [0] * len(group), [gshape] * len(group)))
                b.run()
                w = torch.from_numpy(np.stack([weights[i] for i in group])).to(out.device)
                check(tasks.lib().rf_accumulate_mirrored(ptr(b.image_buffer), ptr(w), len(group), r.width(),
                                                         r.height(), 0.0, ptr(out), self.rasterizing_task.stream),
                      'rf_accumulate_mirrored')
                del b
        check(tasks.lib().rf_accumulate_mirrored(ptr(out), ptr(out), 0, r.width(), r.height(), float(width * height),
                                                 ptr(out), self.rasterizing_task.stream), 'rf_accumulate_mirrored')
        return Image(tensor=out, args=(project.flare.light, hash(project.render)))

    def flare_starburst(self, project: Project) -> Image:
        flare = self.flare(project)
        starburst = self.starburst(project)
        ft, st = flare.tensor, starburst.tensor
        out = empty(tuple(ft.shape))
        # array = flare.copy(); array += flare + starburst (engine.py:176-184)
        check(tasks.lib().rf_axpby(ptr(ft), 2.0, ptr(st), 1.0, ptr(out), ft.numel(),
                                   self.rasterizing_task.stream), 'rf_axpby')
        return Image(tensor=out, args=(flare.args, starburst.args))

    def diagram(self, project: Project) -> Image:
        # engine.py:189-193: the debug ghost's rays over the lens cross-section
        path_indexes = (project.diagram.debug_ghost,)
        intersections = self.intersection_task.run(project, path_indexes)
        return self.diagram_task.run(project, intersections)

    def render(self, project: Project) -> bool:
        if not self._initialized:
            self._init()
        try:
            renderer = self.renderers.get(project.output.element)
            if renderer is None:
                raise RealflareError(f'render element not supported: {project.output.element}')
            with torch.cuda.stream(self.queue):
                self.image = renderer(project)
            self.queue.synchronize()
        except RealflareError as e:
            logger.error(e)
            return False
        return True
