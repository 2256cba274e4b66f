"""Parameter recovery on the differentiable workload (16 surfaces, 512 x 512, 64 x 64 grid,
8 wavelengths, 120 ghosts): the target is rendered from seeded perturbations of radii,
gaps, coating thicknesses and light position, and the recovery starts from the unperturbed
lens (realflare_gb300/recover.py)."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from realflare_gb300 import synthetic  # noqa: E402


@pytest.fixture(scope='module')
def workload():
    from realflare_gb300.tasks import GhostApertureTask, GhostTask

    p = synthetic.workload('differentiable-16').project
    ghost = GhostTask().run(p, GhostApertureTask().run(p)).tensor
    return p, ghost


def test_corrected_coarse_stage_is_stationary_at_the_truth(workload):
    """With the render's residual and the splat's gradient, the coarse loss and its gradient
    vanish at the true parameters (for the splat alone they do not)."""
    from realflare_gb300.diff import DifferentiableRenderer, gaussian_blur

    p, ghost = workload
    r = DifferentiableRenderer(p, ghost)
    params = [t.detach().clone().requires_grad_(True) for t in r.params.tensors()]
    with torch.no_grad():
        im = r.render(*params)
        tb = torch.stack([gaussian_blur(im[..., c], 4.0) for c in range(3)])
        tb = tb / tb.sum()
    grads = {}
    for corrected in (True, False):
        for q in params:
            q.grad = None
        sp = r.splat(r.trace(*params), 4.0, channels=True)
        model = sp / sp.sum()
        if corrected:
            model = tb + (model - model.detach())
        loss = ((model - tb) ** 2).sum()
        loss.backward()
        grads[corrected] = (float(loss.detach()), torch.cat([q.grad.reshape(-1) for q in params]))
    loss_c, g_c = grads[True]
    loss_s, g_s = grads[False]
    assert loss_c == 0.0 and float(g_c.abs().max()) == 0.0
    assert loss_s > 0.0 and float(g_s.abs().max()) > 0.0


def test_recovery_moves_the_parameters_towards_the_truth(workload):
    from realflare_gb300.recover import recover

    p, ghost = workload
    rec = recover(p, ghost, steps=200)
    # the coarse stage alone, and the whole recovery, end nearer the truth than the start
    assert rec.error_after_coarse < 0.9 * rec.error_start
    assert rec.error_end < 0.9 * rec.error_start
    # the light position is the best-determined group
    assert rec.error_groups_end['light'] < 0.5 * rec.error_groups_start['light']
    # the image stage lowers the image loss
    assert rec.loss_end < rec.loss_start < rec.loss_initial
