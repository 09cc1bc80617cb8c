"""Adjoint gradient of a velocity misfit with respect to log-viscosity (steady VE Stokes step,
variable viscosity) against central finite differences of the forward solve, in 2D and 3D: the
differences agree with the adjoint gradient to 1e-6 of its largest value."""

import dataclasses

import numpy as np
import pytest

from chmy_gb300 import _abi
from chmy_gb300.configs import stokes2d_inclusions, stokes3d_grf
from chmy_gb300.solvers import StokesSolver

pytestmark = pytest.mark.gpu


def _sensor(nd, n):
    """Vertical velocity on its middle interior vertex plane, over the interior cells: padded
    index slices (the last velocity component). Logical index I is padded I + 1, and the
    interior of a Center dimension is 1..n."""
    mid = n // 2 + 1 + 1
    inner = slice(2, n + 2)
    return (mid, inner) if nd == 2 else (mid, inner, inner)


def _misfit(solver, nd, n, obs):
    v = solver.fields["V"][nd - 1].to_numpy()
    s = _sensor(nd, n)
    r = v[s] - obs
    dJ = np.zeros_like(v)
    dJ[s] = r
    return 0.5 * float(np.sum(r * r)), dJ


def _solve(arch, pb):
    s = StokesSolver(arch, pb)
    s.apply_bc()
    res = s.solve(precision=_abi.CG_F64)
    assert res.converged == 1, (res.iterations, list(res.err))
    s.last_result = res
    return s


def _check(arch, pb, cells, h=1e-3, tol=1e-6, top=4):
    """Central differences of J in log(eta) at `cells` and at the `top` cells of largest adjoint
    gradient; every difference agrees with the adjoint gradient to `tol` of the largest."""
    nd, n = pb.grid.ndim, pb.grid.dims[0]
    rng = np.random.default_rng(5)
    fwd = _solve(arch, pb)
    fwd_res = fwd.last_result
    v = fwd.fields["V"][nd - 1].to_numpy()
    obs = v[_sensor(nd, n)] + 0.1 * rng.standard_normal(v[_sensor(nd, n)].shape)
    J0, dJ = _misfit(fwd, nd, n, obs)
    dJdV = [None] * (nd - 1) + [dJ]
    grad, res = fwd.gradient_log_eta(dJdV, eps=pb.eps)
    assert res.converged == 1
    # the adjoint is one more Stokes solve of the same kind: at most 3 forward costs
    assert res.iterations <= 3 * fwd_res.iterations, (res.iterations, fwd_res.iterations)
    g = grad.to_numpy()
    gi = g[(slice(2, n + 2),) * nd]  # interior cells, logical 1..n
    gmax = max(np.abs(gi).max(), 1e-300)
    big = np.argsort(np.abs(gi).ravel())[-top:]
    cells = list(cells) + [tuple(reversed(np.unravel_index(q, gi.shape))) for q in big]
    eta = pb.host["eta"]
    rows = []
    for c in cells:
        idx = tuple(reversed([int(ci) + 2 for ci in c]))  # cell c (0-based interior) -> padded [z, y, x]
        Jpm = []
        for sgn in (1.0, -1.0):
            e = eta.copy()
            e[idx] = eta[idx] * np.exp(sgn * h)
            s = _solve(arch, dataclasses.replace(pb, host={**pb.host, "eta": e}))
            Jpm.append(_misfit(s, nd, n, obs)[0])
        rows.append((tuple(int(x) for x in c), float(g[idx]), (Jpm[0] - Jpm[1]) / (2 * h)))
    worst = max(abs(a - b) for _, a, b in rows) / gmax
    assert worst <= tol, (worst, gmax, rows)


def test_gradient_log_eta_2d_matches_finite_differences(arch):
    pb = stokes2d_inclusions(32, ncheck=8)
    pb = dataclasses.replace(pb, eps=1e-12, max_iter=2000 * 32)
    _check(arch, pb, [(5, 9), (16, 16), (25, 20), (0, 31), (12, 3)])


def test_gradient_log_eta_3d_matches_finite_differences(arch):
    pb = stokes3d_grf(16, ncheck=8)
    pb = dataclasses.replace(pb, eps=1e-12, max_iter=2000 * 16)
    _check(arch, pb, [(3, 4, 5), (8, 8, 8), (12, 2, 10), (0, 15, 7)])
