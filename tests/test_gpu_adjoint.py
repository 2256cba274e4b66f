"""The trace adjoint against central finite differences of the FP64 oracle.

For a random linear function of the traced outputs L = sum v * rays (v scaled per output
plane), rf_trace_adjoint's gradient with respect to each element's radius, center and
coating thickness and to the light direction is compared with (L(x + h) - L(x - h)) / 2h
computed from the FP64 oracle's trace (outputs unrounded). Rays whose validity changes
within the step are left out of both sides (the derivative does not exist there): the
adjoint is evaluated with that parameter's ray mask.

The step is 1e-5 relative (lengths: of max(|x|, 10 mm)). At 1e-3 the central difference
is not yet converged on this lens: rays near the edge of their ghost bend strongly, and
the difference quotients at 1e-3, 1e-4 and 1e-5 differ by up to 60 % for some radii while
1e-4 and 1e-5 agree with each other (and with the adjoint) to about 1e-4.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from realflare_gb300 import prepare, synthetic  # noqa: E402
from realflare_gb300._abi import check, lib  # noqa: E402

STEP = 1e-5
# |adjoint - FD| / |FD| over all checked parameters (vector norm), and per parameter
RTOL_VECTOR = 1e-3
RTOL_EACH = 1e-2


@pytest.fixture(scope='module')
def case():
    from oracle.oracle import Oracle

    w = synthetic.workload('differentiable-16')
    p = w.project
    p.render.grid_count = 16
    p.render.wavelengths = (450.0, 610.0)
    p.render.wavelength_count = 2
    ti = prepare.trace_inputs(p, w.paths[::12])
    return ti, Oracle('f64')


def gpu_trace(ti):
    rays = torch.empty((6, ti.ray_count), device='cuda')
    el = torch.from_numpy(ti.elements.view(np.uint8).copy()).cuda()
    pa = torch.from_numpy(ti.paths).cuda()
    wl = torch.from_numpy(ti.wavelengths).cuda()
    check(lib().rf_trace(el.data_ptr(), pa.data_ptr(), wl.data_ptr(), ctypes.byref(ti.args), rays.data_ptr(),
                         int(torch.cuda.current_stream().cuda_stream)), 'rf_trace')
    return rays, (el, pa, wl)


def adjoint(ti, bufs, grad_rays):
    el, pa, wl = bufs
    g = torch.from_numpy(np.ascontiguousarray(grad_rays, np.float32)).cuda()
    ge = torch.empty((ti.args.element_count, 4), device='cuda')
    gd = torch.empty((3,), device='cuda')
    check(lib().rf_trace_adjoint(el.data_ptr(), pa.data_ptr(), wl.data_ptr(), ctypes.byref(ti.args), g.data_ptr(),
                                 ge.data_ptr(), gd.data_ptr(), int(torch.cuda.current_stream().cuda_stream)),
          'rf_trace_adjoint')
    torch.cuda.synchronize()
    return ge.cpu().numpy().astype(np.float64), gd.cpu().numpy().astype(np.float64)


def test_trace_adjoint_matches_fp64_finite_differences(case):
    ti, o = case
    rays, bufs = gpu_trace(ti)
    base = rays.cpu().numpy()
    valid = ~np.isnan(base[5])
    assert valid.mean() > 0.3
    rng = np.random.default_rng(7)
    scale = np.array([np.std(base[k][valid]) + 1e-12 for k in range(6)])
    v = rng.normal(size=base.shape) / scale[:, None]

    results = []  # (name, adjoint, fd)

    def check_param(name, setter, h, adj_pick):
        e_plus, e_minus = ti.elements.copy(), ti.elements.copy()
        a_plus, a_minus = prepare.TraceArgs.from_buffer_copy(ti.args), prepare.TraceArgs.from_buffer_copy(ti.args)
        x_plus = setter(e_plus, a_plus, +h)
        x_minus = setter(e_minus, a_minus, -h)
        r_p = o.trace_d(e_plus, ti.paths, ti.wavelengths, a_plus)
        r_m = o.trace_d(e_minus, ti.paths, ti.wavelengths, a_minus)
        mask = valid & ~np.isnan(r_p[5]) & ~np.isnan(r_m[5])
        lp = float(np.sum(np.where(mask, v * np.nan_to_num(r_p), 0.0)))
        lm = float(np.sum(np.where(mask, v * np.nan_to_num(r_m), 0.0)))
        fd = (lp - lm) / (x_plus - x_minus)
        ge, gd = adjoint(ti, bufs, np.where(mask, v, 0.0))
        results.append((name, adj_pick(ge, gd), fd))

    E = ti.args.element_count
    for i in range(E):
        r = float(ti.elements[i]['radius'])
        if r != 0.0:
            def set_r(e, a, d, i=i, r=r):
                e[i]['radius'] = np.float32(r * (1 + d))
                return float(e[i]['radius'])
            check_param(f'radius[{i}]', set_r, STEP, lambda ge, gd, i=i: ge[i, 0])
        c = float(ti.elements[i]['center'])

        def set_c(e, a, d, i=i, c=c):
            e[i]['center'] = np.float32(c + d * max(abs(c), 10.0))
            return float(e[i]['center'])
        check_param(f'center[{i}]', set_c, STEP, lambda ge, gd, i=i: ge[i, 1])
        if ti.elements[i]['coating_layers'] == 1 and i not in (ti.args.aperture_index, E - 1):
            t = float(ti.elements[i]['coating_thickness'][0])

            def set_t(e, a, d, i=i, t=t):
                e[i]['coating_thickness'][0] = np.float32(t * (1 + d))
                return float(e[i]['coating_thickness'][0])
            check_param(f'thickness[{i}]', set_t, STEP, lambda ge, gd, i=i: ge[i, 2])
    # light direction: the adjoint is with respect to n = normalize(-direction.xyz)
    d0 = np.array(ti.args.direction[:3], np.float64)
    for k in (0, 1):
        def set_d(e, a, d, k=k):
            a.direction[k] = np.float32(d0[k] + d * max(abs(d0[k]), 1.0))
            return float(a.direction[k])

        def pick(ge, gd, k=k):
            vv = np.array(ti.args.direction[:3], np.float64)
            nrm = np.linalg.norm(vv)
            n = vv / nrm
            # dn/dv for n = -v / |v|: -(I - n n^T) / |v|
            jac = -(np.eye(3) - np.outer(n, n)) / nrm
            return float((jac.T @ gd)[k])
        check_param(f'direction[{k}]', set_d, STEP, pick)

    adj = np.array([a for _, a, _ in results])
    fd = np.array([f for _, _, f in results])
    assert np.linalg.norm(fd) > 0
    rel = np.linalg.norm(adj - fd) / np.linalg.norm(fd)
    big = np.abs(fd) > 1e-3 * np.abs(fd).max()
    each = np.abs(adj - fd)[big] / np.abs(fd)[big]
    worst = [results[i][0] for i in np.flatnonzero(big)[np.argsort(-each)[:3]]]
    assert rel <= RTOL_VECTOR, (rel, worst, each.max())
    assert each.max() <= RTOL_EACH, (worst, each.max())
