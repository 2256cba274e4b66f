"""Animated renders (realflare/cli/app.py:22-41,86-97): per-frame values on one project.

The CPU tests check apply_animation's semantics (per-frame lists, nested dicts, values that
persist past the end of their list, casts to the attribute's type, unknown names skipped).
The GPU test renders the frames with render_frames (batched flare frames, Engine.render for
the rest) and compares each with Engine.render of the same frame's project, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from realflare_gb300 import synthetic
from realflare_gb300.animation import apply_animation, frame_projects
from realflare_gb300.data import Project, QPointF, QSize, RealflareError, RenderElement

ANIMATION = {
    'flare': {'light': {'position': [[0.1, 0.2], [0.3, -0.1]], 'intensity': [2, 3, 4]}},
    'render': {'grid_count': [16, 24], 'resolution': [[256, 256]]},
    'output': {'element': ['FLARE', 'STARBURST']},
    'not_a_field': {'x': [1, 2]},
}


def test_frame_projects_follow_the_command_line_loop():
    p = Project()
    frames = frame_projects(p, ANIMATION, 5, 7)
    assert [f.output.frame for f in frames] == [5, 6, 7]
    f1, f2, f3 = frames
    assert f1.flare.light.position == QPointF(0.1, 0.2)
    assert f2.flare.light.position == QPointF(0.3, -0.1)
    assert f3.flare.light.position == QPointF(0.3, -0.1)  # past the end: the last value stays
    assert [f.flare.light.intensity for f in frames] == [2.0, 3.0, 4.0]
    assert all(isinstance(f.flare.light.intensity, float) for f in frames)
    assert [f.render.grid_count for f in frames] == [16, 24, 24]
    assert all(f.render.resolution == QSize(256, 256) for f in frames)
    assert [f.output.element for f in frames] == [RenderElement.FLARE, RenderElement.STARBURST,
                                                  RenderElement.STARBURST]
    # the input project is left as it was
    assert p.output.frame == 0 and p.render.grid_count == Project().render.grid_count


def test_apply_animation_in_place_and_errors():
    p = Project()
    apply_animation(p, {'render': {'anti_aliasing': [1, 4]}}, 1)
    assert p.render.anti_aliasing == 4
    apply_animation(p, {'render': {'anti_aliasing': [2]}}, 3)  # no value for frame 3
    assert p.render.anti_aliasing == 4
    with pytest.raises(RealflareError):
        apply_animation(p, {'render': {'anti_aliasing': 2}}, 0)
    with pytest.raises(RealflareError):
        frame_projects(p, None, 3, 2)


@pytest.mark.gpu
def test_render_frames_match_engine_render():
    import torch

    from realflare_gb300.animation import render_frames
    from realflare_gb300.engine import Engine

    p = synthetic.workload('plain-8').project
    p.render.resolution = QSize(256, 256)
    anim = {'flare': {'light': {'position': [[0.2, 0.1], [0.35, -0.2], [-0.3, 0.25], [0.0, 0.4]]}},
            'render': {'grid_count': [16, 24, 32]},
            'output': {'element': ['FLARE', 'FLARE', 'FLARE', 'STARBURST']}}
    images = render_frames(p, anim, 1, 4)
    torch.cuda.synchronize()
    engine = Engine()
    for q, img in zip(frame_projects(p, anim, 1, 4), images):
        assert engine.render(q)
        want = engine.image.tensor.cpu().numpy()
        got = img.cpu().numpy()
        assert got.shape == want.shape
        assert np.abs(want).sum() > 0
        np.testing.assert_array_equal(got, want)
