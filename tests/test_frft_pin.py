"""The FRFT ghost texture's oracle against the reference's own ``frft.py``.

``tests/golden/frft_ghost.npz`` holds ghost textures computed by the reference's
``realflare/utils/frft.py`` (run unchanged but for the numpy-2 ``chirp`` shim) through
``GhostTask.ghost``'s arithmetic (``realflare/api/tasks/ghost.py:13-36``), made by
``tests/golden/make_frft_golden.py``, for fstops covering all five branches of
``frft.normalize``. The numpy FP64 restatement (``oracle.oracle.ghost_texture``) must
reproduce them to FP32 output rounding. With ``REALFLARE_REFERENCE`` naming the checkout,
the reference module is also imported directly and compared at 512 x 512."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

from golden.make_frft_golden import CASES, key
from helpers import rel_l2

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')

# float64 restatement vs the reference's float64 arithmetic with a float32 output
ORACLE_RTOL = 1e-6


def load():
    with np.load(os.path.join(HERE, 'frft_ghost.npz')) as z:
        return {k: z[k] for k in z.files}


def test_frft_fixture_intact():
    with open(os.path.join(HERE, 'manifest.json')) as f:
        manifest = json.load(f)['frft_ghost']
    g = load()
    assert set(g) == set(manifest)
    for k, v in g.items():
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == manifest[k], k


@pytest.mark.parametrize('case', [c[0] for c in CASES])
def test_oracle_ghost_texture_matches_reference_frft(case):
    from oracle.oracle import ghost_texture

    g = load()
    _, h, w, _, _, fstops = next(c for c in CASES if c[0] == case)
    ap = g[f'{case}_aperture']
    for fstop in fstops:
        want = g[key(case, fstop)]
        got = ghost_texture(ap, fstop, (w, h))
        assert np.linalg.norm(want) > 0
        assert rel_l2(got, want) < ORACLE_RTOL, (case, fstop)


@pytest.mark.skipif(not os.environ.get('REALFLARE_REFERENCE'), reason='REALFLARE_REFERENCE not set')
@pytest.mark.parametrize('fstop', [0.0, 64.0, 275.0])
def test_oracle_matches_reference_module_at_512(fstop):
    from golden.make_frft_golden import load_reference_frft, polygon, reference_ghost
    from oracle.oracle import ghost_texture

    module = load_reference_frft(os.environ['REALFLARE_REFERENCE'])
    ap = polygon(512, 512, 8, 0.0)
    assert rel_l2(ghost_texture(ap, fstop, (512, 512)), reference_ghost(module, ap, fstop)) < ORACLE_RTOL
