"""The render engine (``realflare/api/engine.py``): composes the tasks into render elements.

``Engine.render(project) -> bool`` renders ``project.output.element`` and keeps the result
in ``Engine.image``; ``flare``, ``starburst``, ``ghost``, ``flare_starburst`` and the two
aperture elements are available individually, as in the reference (engine.py:80-193).
User errors raise ``RealflareError`` inside and make ``render`` return False
(engine.py:195-223).
"""
from __future__ import annotations

import logging

import torch

from . import tasks
from ._abi import check
from .data import Project, RealflareError, RenderElement
from .device import Image, empty, ptr

logger = logging.getLogger(__name__)


class Engine:
    def __init__(self, device: str = '', cache: bool = True) -> None:
        self.cache = cache
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
        self.raytracing_task = tasks.RaytracingTask(self.queue, cache=self.cache)
        self.rasterizing_task = tasks.RasterizingTask(self.queue)
        self.renderers = {
            RenderElement.STARBURST_APERTURE: self.starburst_aperture,
            RenderElement.GHOST_APERTURE: self.ghost_aperture,
            RenderElement.STARBURST: self.starburst,
            RenderElement.GHOST: self.ghost,
            RenderElement.FLARE: self.flare,
            RenderElement.FLARE_STARBURST: self.flare_starburst,
        }
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
        if project.flare.light.image_file_enabled:
            raise RealflareError('image based flares are not supported')
        if project.render.debug_ghost_enabled:
            path_indexes = (project.render.debug_ghost,)
        elif project.render.cull_percentage > 0:
            raise RealflareError('ghost culling (cull_percentage > 0) is not supported')
        else:
            path_indexes = ()  # cull 0 keeps every path (preprocessing.py:86-89)
        ghost = self.ghost(project)
        rays = self.raytracing_task.run(project, path_indexes)
        return self.rasterizing_task.run(project, rays, ghost)

    def flare_starburst(self, project: Project) -> Image:
        flare = self.flare(project)
        starburst = self.starburst(project)
        ft, st = flare.tensor, starburst.tensor
        out = empty(tuple(ft.shape))
        # array = flare.copy(); array += flare + starburst (engine.py:176-184)
        check(tasks.lib().rf_axpby(ptr(ft), 2.0, ptr(st), 1.0, ptr(out), ft.numel(),
                                   self.rasterizing_task.stream), 'rf_axpby')
        return Image(tensor=out, args=(flare.args, starburst.args))

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
