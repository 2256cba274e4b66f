"""Lens and light recovery by gradient descent through the differentiable render.

A target image is rendered from perturbed parameters (curvature radii, gaps, coating
thicknesses, light position); starting from the unperturbed lens, Adam minimises the
distance of the render to the target. The free variables are normalised offsets (radii and
gaps relative, thicknesses in units of 10 nm, light in units of 0.05) so one learning rate
fits all of them.

The render's gradient holds coverage fixed (``diff.py``): where a ghost lands and how large
it is enters the image only through which pixels its quads cover, so an image loss alone
cannot steer the geometry (from the unperturbed lens, 200 steps of it lower the loss through
intensities and leave radii, gaps and thicknesses further from the truth than they started).
The recovery therefore runs in two stages:

1. coarse: per blur width in ``sigmas`` (wide to narrow), ``coarse_steps`` Adam steps on the
   distance between the Gaussian-blurred target and the blurred model (the three AP1
   channels, each image normalised to unit sum). The splat of the traced rays
   (``DifferentiableRenderer.splat``) is smooth in the ray positions, so its gradient
   (through ``rf_trace_adjoint``) moves ghosts towards where the target has them. With
   ``corrected`` (the default) the model is the blurred render with the splat's gradient:
   blur(render) + splat - detach(splat), so the loss and its residual are the blurred
   render's own and only the direction of descent comes from the splat; the true
   parameters are then a stationary point, which they are not for the splat alone (the
   blurred splat and the blurred render differ by the quads' shapes and the ghost
   texture's variation over them). Without ``corrected`` the model is the splat.
   ``views`` renders the lens at further known light offsets (normalised field units) as
   more targets of the same unknowns;
2. image: ``steps`` Adam steps on the L2 distance of the render to the target over the
   parameters in ``image_params`` (by default the coating thicknesses, which the image
   gradient determines through the reflectances; the geometry keeps the coarse stage's
   values), at learning rate ``lr`` (0.001: larger steps move the thicknesses to explain
   the residuals the geometry leaves, and the parameter error rises again).
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np
import torch

from .data import Project
from .diff import DifferentiableRenderer, gaussian_blur

# perturbation of the target: radii +-2 %, gaps +-5 %, thickness +-10 nm, light +-0.05
SCALE = {'radii': 0.02, 'gaps': 0.05, 'thickness': 10.0, 'light': 0.05}
NAMES = ('radii', 'gaps', 'thickness', 'light')


@dataclass
class Recovery:
    steps: int
    loss_start: float | None  # image loss before the image stage
    loss_end: float
    error_start: float  # RMS of the normalised parameter error
    error_end: float
    seconds: float
    coarse_steps: int = 0
    loss_initial: float | None = None  # image loss at the unperturbed start
    error_after_coarse: float | None = None
    error_groups_start: dict | None = None  # RMS per parameter group
    error_groups_end: dict | None = None
    views: int = 1


def _params(base: list, z: list, offset=(0.0, 0.0)) -> list:
    r0, g0, t0, l0 = base
    zr, zg, zt, zl = z
    light = l0 + SCALE['light'] * zl
    if offset != (0.0, 0.0):
        light = light + torch.tensor(offset, dtype=light.dtype, device=light.device)
    return [r0 * (1 + SCALE['radii'] * zr), g0 * (1 + SCALE['gaps'] * zg), t0 + SCALE['thickness'] * zt, light]


def recover(project: Project, ghost: torch.Tensor, steps: int = 200, lr: float = 0.001, seed: int = 0,
            sigmas: tuple = (8.0, 4.0, 2.0, 1.0), coarse_steps: int = 100, coarse_lr: float = 0.05,
            decay: float = 0.995, views: tuple = ((0.0, 0.0),), image_params: tuple = ('thickness',),
            accurate: bool = False, corrected: bool = True) -> Recovery:
    renderer = DifferentiableRenderer(project, ghost, accurate=accurate)
    base = [t.detach() for t in renderer.params.tensors()]
    rng = np.random.Generator(np.random.PCG64(seed))
    truth = [torch.tensor(rng.uniform(-1.0, 1.0, t.shape), dtype=t.dtype, device=t.device) for t in base]
    views = tuple(tuple(float(c) for c in v) for v in views)
    with torch.no_grad():
        targets = [renderer.render(*_params(base, truth, v)).clone() for v in views]
    target = targets[0]
    z = [torch.zeros_like(t, requires_grad=True) for t in base]

    def error() -> float:
        d = torch.cat([(a.detach() - b).reshape(-1) for a, b in zip(z, truth)])
        return float(torch.sqrt((d * d).mean()))

    def group_errors() -> dict:
        return {n: float(torch.sqrt(((a.detach() - b) ** 2).mean())) for n, a, b in zip(NAMES, z, truth)}

    def image_loss() -> torch.Tensor:
        return ((renderer.render(*_params(base, z, views[0])) - target)[..., :3] ** 2).sum()

    e0, g0 = error(), group_errors()
    with torch.no_grad():
        loss_initial = float(image_loss())
    t0 = time.perf_counter()
    # 1. coarse: blurred splats of the rays against the blurred targets, unit sums
    e_coarse = None
    if coarse_steps > 0 and sigmas:
        opt = torch.optim.Adam(z, lr=coarse_lr)
        sched = torch.optim.lr_scheduler.ExponentialLR(opt, decay)
        for sg in sigmas:
            with torch.no_grad():
                tbs = []
                for t in targets:
                    tb = torch.stack([gaussian_blur(t[..., c], sg) for c in range(3)])
                    tbs.append(tb / tb.sum())
            for _ in range(coarse_steps):
                opt.zero_grad()
                loss = 0.0
                for v, tb in zip(views, tbs):
                    pv = _params(base, z, v)
                    sp = renderer.splat(renderer.trace(*pv), sg, channels=True)
                    model = sp / sp.sum()
                    if corrected:
                        with torch.no_grad():
                            im = renderer.render(*[q.detach() for q in pv])
                            rb = torch.stack([gaussian_blur(im[..., c], sg) for c in range(3)])
                        model = rb / rb.sum() + (model - model.detach())
                    loss = loss + ((model - tb) ** 2).sum() * tb.numel()
                loss.backward()
                opt.step()
                sched.step()
        e_coarse = error()
    # 2. the image loss
    loss0 = None
    free = [q for n, q in zip(NAMES, z) if n in image_params]
    if steps > 0 and free:
        opt = torch.optim.Adam(free, lr=lr)
        for _ in range(steps):
            opt.zero_grad()
            loss = image_loss()
            loss.backward()
            if loss0 is None:
                loss0 = float(loss.detach())
            opt.step()
    torch.cuda.synchronize()
    seconds = time.perf_counter() - t0
    with torch.no_grad():
        final = float(image_loss())
    return Recovery(steps, loss0, final, e0, error(), seconds, coarse_steps * len(sigmas), loss_initial, e_coarse,
                    g0, group_errors(), len(views))
