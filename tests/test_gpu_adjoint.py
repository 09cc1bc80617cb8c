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


def _ptdiff_problem(n, T=np.float64):
    from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
    from chmy_gb300.configs import box_smooth, padded_mesh, ptdiff_params
    from chmy_gb300.grids import Center, UniformGrid

    grid = UniformGrid(origin=(T(-0.5), T(-0.5)), extent=(T(1), T(1)), dims=(n, n), dtype=T)
    x, y = padded_mesh(grid, Center())
    rng = np.random.default_rng(2)
    D = np.exp(box_smooth(rng.standard_normal(x.shape))).astype(T)
    C0 = np.exp(-(x * x + y * y) / 0.01).astype(T)
    bc = to_cg_bc(2, {"x": Dirichlet(0.0), "y": Neumann()})
    return grid, D, C0, bc, ptdiff_params(grid, 1e-3, float(D.max()))


def test_ptdiff_gradient_D_matches_finite_differences(arch):
    """Implicit diffusion steps (config 2 form, 2D 24^2): the adjoint gradient of
    J = 1/2 |C^N - C_obs|^2 with respect to log(D) agrees with central differences; the
    checkpointed reverse sweep gives the same bits for 1, 2 and sqrt(N) steps per segment."""
    from chmy_gb300.adjoint import PTDiffusion

    n, nsteps, npt = 24, 6, 1500
    grid, D, C0, bc, p = _ptdiff_problem(n)
    inner = (slice(2, n + 2), slice(2, n + 2))
    rng = np.random.default_rng(9)
    pt = PTDiffusion(arch, grid, D, p, bc, npt)
    CN = pt.run(C0, nsteps)
    obs = CN[inner] + 0.01 * rng.standard_normal(CN[inner].shape)

    def J(c):
        r = c[inner] - obs
        return 0.5 * float(np.sum(r * r))

    def dJ(c):
        g = np.zeros_like(c)
        g[inner] = c[inner] - obs
        return g

    gD, gC0, CN2 = pt.gradient(C0, nsteps, dJ)
    assert np.array_equal(CN, CN2)
    for K in (1, 2):
        gD2, gC02, _ = pt.gradient(C0, nsteps, dJ, checkpoint_every=K)
        assert np.array_equal(gD, gD2) and np.array_equal(gC0, gC02)
    glog = gD * D  # dJ/d log(D)
    gi = glog[inner]
    gmax = np.abs(gi).max()
    big = np.argsort(np.abs(gi).ravel())[-4:]
    cells = [(3, 5), (12, 12), (20, 1)] + [tuple(int(v) for v in reversed(np.unravel_index(q, gi.shape))) for q in big]
    h = 1e-3
    rows = []
    for c in cells:
        idx = (c[1] + 2, c[0] + 2)
        Jpm = []
        for sgn in (1.0, -1.0):
            Dp = D.copy()
            Dp[idx] = D[idx] * np.exp(sgn * h)
            Jpm.append(J(PTDiffusion(arch, grid, Dp, p, bc, npt).run(C0, nsteps)))
        rows.append((c, float(glog[idx]), (Jpm[0] - Jpm[1]) / (2 * h)))
    worst = max(abs(a - b) for _, a, b in rows) / gmax
    assert worst <= 1e-6, (worst, gmax, rows)
    # the initial-state gradient against a difference in C0 at one interior cell
    idx = (n // 2 + 2, n // 2 + 2)
    Jpm = []
    for sgn in (1.0, -1.0):
        C0p = C0.copy()
        C0p[idx] += sgn * 1e-4
        Jpm.append(J(PTDiffusion(arch, grid, D, p, bc, npt).run(C0p, nsteps)))
    fd = (Jpm[0] - Jpm[1]) / 2e-4
    assert abs(gC0[idx] - fd) <= 1e-6 * max(abs(fd), np.abs(gC0[inner]).max()), (gC0[idx], fd)
