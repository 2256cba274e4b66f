"""Lens and light recovery by gradient descent through the differentiable render.

A target image is rendered from perturbed parameters (curvature radii, gaps, coating
thicknesses, light position); starting from the unperturbed lens, Adam minimises the L2
distance of the render to the target. The free variables are normalised offsets (radii and
gaps relative, thicknesses in units of 10 nm, light in units of 0.05) so one learning rate
fits all of them.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np
import torch

from .data import Project
from .diff import DifferentiableRenderer

# perturbation of the target: radii +-2 %, gaps +-5 %, thickness +-10 nm, light +-0.05
SCALE = {'radii': 0.02, 'gaps': 0.05, 'thickness': 10.0, 'light': 0.05}


@dataclass
class Recovery:
    steps: int
    loss_start: float
    loss_end: float
    error_start: float  # RMS of the normalised parameter error
    error_end: float
    seconds: float


def _params(base: list, z: list) -> list:
    r0, g0, t0, l0 = base
    zr, zg, zt, zl = z
    return [r0 * (1 + SCALE['radii'] * zr), g0 * (1 + SCALE['gaps'] * zg), t0 + SCALE['thickness'] * zt,
            l0 + SCALE['light'] * zl]


def recover(project: Project, ghost: torch.Tensor, steps: int = 200, lr: float = 0.02, seed: int = 0) -> Recovery:
    renderer = DifferentiableRenderer(project, ghost)
    base = [t.detach() for t in renderer.params.tensors()]
    rng = np.random.Generator(np.random.PCG64(seed))
    truth = [torch.tensor(rng.uniform(-1.0, 1.0, t.shape), dtype=t.dtype, device=t.device) for t in base]
    with torch.no_grad():
        target = renderer.render(*_params(base, truth)).clone()
    z = [torch.zeros_like(t, requires_grad=True) for t in base]
    opt = torch.optim.Adam(z, lr=lr)

    def error() -> float:
        d = torch.cat([(a.detach() - b).reshape(-1) for a, b in zip(z, truth)])
        return float(torch.sqrt((d * d).mean()))

    e0 = error()
    loss0 = None
    t0 = time.perf_counter()
    for _ in range(steps):
        opt.zero_grad()
        image = renderer.render(*_params(base, z))
        loss = ((image - target)[..., :3] ** 2).sum()
        loss.backward()
        if loss0 is None:
            loss0 = float(loss)
        opt.step()
    torch.cuda.synchronize()
    seconds = time.perf_counter() - t0
    with torch.no_grad():
        final = float(((renderer.render(*_params(base, z)) - target)[..., :3] ** 2).sum())
    return Recovery(steps, loss0, final, e0, error(), seconds)
