"""Adjoint gradients against central finite differences and forward-mode dual numbers:
- a velocity misfit of the steady VE Stokes step with respect to log-viscosity, 2D and 3D
  (differences to 1e-6 of the largest gradient; the dual-number tangents of the oracle's PT
  iterations to 1e-7 along random directions);
- implicit diffusion with respect to D and the initial state;
- the SIA time loop with respect to Gamma, ela and the initial thickness."""

import ctypes
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


def _check_dual(arch, pb, tol=1e-7):
    """The adjoint gradient's directional derivatives along two random log-viscosity
    directions (zero in the ghost cells) against forward-mode dual numbers run through the
    oracle's PT iterations to their fixed point (or_stokes_solve_tangent)."""
    from _oracle import stokes_tangent_solve

    nd, n = pb.grid.ndim, pb.grid.dims[0]
    fwd = _solve(arch, pb)
    rng = np.random.default_rng(7)
    v = fwd.fields["V"][nd - 1].to_numpy()
    obs = v[_sensor(nd, n)] + 0.1 * rng.standard_normal(v[_sensor(nd, n)].shape)
    _, dJ = _misfit(fwd, nd, n, obs)
    grad, res = fwd.gradient_log_eta([None] * (nd - 1) + [dJ], eps=pb.eps)
    assert res.converged == 1
    inner = (slice(2, n + 2),) * nd
    g = grad.to_numpy()[inner]
    shape = pb.host["eta"].shape
    dirs = []
    for _ in range(2):
        d = np.zeros(shape)
        d[inner] = rng.standard_normal((n,) * nd)
        dirs.append(d)
    _, tan, iters = stokes_tangent_solve(pb, dirs)
    for k in range(2):
        adj = float(np.sum(g * dirs[k][inner]))
        dual = float(np.sum(dJ * tan[k][nd - 1]))
        assert abs(adj - dual) <= tol * abs(dual), (k, adj, dual, iters)


def test_gradient_log_eta_2d_matches_dual_numbers(arch):
    pb = stokes2d_inclusions(32, ncheck=8)
    _check_dual(arch, dataclasses.replace(pb, eps=1e-12, max_iter=2000 * 32))


def test_gradient_log_eta_3d_matches_dual_numbers(arch):
    """The 32^3 copy of the 3D VE Stokes configuration (random log-viscosity field)."""
    pb = stokes3d_grf(32, ncheck=8)
    _check_dual(arch, dataclasses.replace(pb, eps=1e-12, max_iter=2000 * 32))


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
    """Implicit variable-diffusivity steps (2D 24^2): the adjoint gradient of
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


def test_ptdiff_gradient_D_matches_dual_numbers(arch):
    """Implicit diffusion steps (2D 24^2, 6 steps of 1500 PT iterations): the adjoint gradient's
    directional derivatives along two random log-diffusivity directions agree with the
    dual-number tangents of the oracle's restated loop (or_ptdiff_run_tangent) to 1e-7
    relative."""
    from _oracle import ptdiff_tangent_run

    from chmy_gb300.adjoint import PTDiffusion

    n, nsteps, npt = 24, 6, 1500
    grid, D, C0, bc, p = _ptdiff_problem(n)
    inner = (slice(2, n + 2), slice(2, n + 2))
    rng = np.random.default_rng(12)
    pt = PTDiffusion(arch, grid, D, p, bc, npt)
    CN = pt.run(C0, nsteps)
    obs = CN[inner] + 0.01 * rng.standard_normal(CN[inner].shape)

    def dJ(c):
        g = np.zeros_like(c)
        g[inner] = c[inner] - obs
        return g

    gD, _, _ = pt.gradient(C0, nsteps, dJ)
    glog = (gD * D)[inner]
    dirs = []
    for _ in range(2):
        d = np.zeros(D.shape)
        d[inner] = rng.standard_normal((n, n))
        dirs.append(d)
    CN_o, tan = ptdiff_tangent_run(grid, D, C0, p, bc, nsteps, npt, dirs)
    assert np.max(np.abs(CN_o[inner] - CN[inner])) <= 1e-12 * np.max(np.abs(CN[inner]))
    r = CN[inner] - obs
    for k in range(2):
        adj = float(np.sum(glog * dirs[k][inner]))
        dual = float(np.sum(r * tan[k][inner]))
        assert abs(adj - dual) <= 1e-7 * abs(dual), (k, adj, dual)


def _sia_problem(n=(48, 40), dt_max=0.5):
    from chmy_gb300.configs import gaussian_random_field, padded_mesh
    from chmy_gb300.grids import Center, UniformGrid

    T = np.float64
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=n, dtype=T)
    x, y = padded_mesh(grid, Center())
    bed = 0.4 + 0.3 * gaussian_random_field(x.shape, 0.25, 2.0 / n[0], 7)
    H0 = np.clip(0.35 - 0.25 * (x * x + y * y), 0.0, None)
    p = _abi.cg_sia_params()
    p.Gamma, p.As, p.n, p.beta, p.ela, p.m_max, p.dt_max, p.cfl = 1.0, 0.0, 3, 0.5, 0.55, 0.25, dt_max, 4.1
    return grid, bed.astype(T), H0.astype(T), p


@pytest.mark.parametrize("tape", [True, False], ids=["taped", "recomputing"])
@pytest.mark.parametrize("dt_max", [0.5, 1e-3])
def test_sia_gradient_gamma_ela_matches_finite_differences(arch, dt_max, tape):
    """SIA time loop (flux -Gamma H^5 |grad S|^2 grad S, ELA mass balance; 2D 48 x 40, 60 steps): the adjoint gradients of
    J = 1/2 |H^N - H_obs|^2 with respect to log(Gamma) and ela agree with central differences
    to 1e-6, with the adaptive time step (dt_max = 0.5: dt from max D) and with dt capped
    (dt_max = 1e-3), for the taped and the recomputing reverse sweeps. Recomputing with
    checkpoints every 1, 7 and sqrt(N) steps gives the same bits; taped segments of 1 and 7
    steps give the same dJ/dH0 bits and dJ/dGamma, dJ/dela to 1e-13 (the per-segment sums
    associate differently)."""
    from chmy_gb300.adjoint import SIA

    grid, bed, H0, p = _sia_problem(dt_max=dt_max)
    nsteps = 60
    inner = (slice(2, -2), slice(2, -2))
    sia = SIA(arch, grid, bed, p)
    HN = sia.run(H0, nsteps)
    rng = np.random.default_rng(3)
    obs = HN[inner] + 0.01 * rng.standard_normal(HN[inner].shape)

    def J(h):
        r = h[inner] - obs
        return 0.5 * float(np.sum(r * r))

    def dJ(h):
        g = np.zeros_like(h)
        g[inner] = h[inner] - obs
        return g

    gG, gE, gH0, HN2 = sia.gradient(H0, nsteps, dJ, tape=tape)
    assert np.array_equal(HN, HN2)
    for K in (1, 7):
        a, b, c, _ = sia.gradient(H0, nsteps, dJ, checkpoint_every=K, tape=tape)
        if tape:
            assert abs(a - gG) <= 1e-13 * abs(gG) and abs(b - gE) <= 1e-13 * abs(gE) and np.array_equal(c, gH0)
        else:
            assert (a, b) == (gG, gE) and np.array_equal(c, gH0)

    def J_at(H=H0, **kw):
        q = _abi.cg_sia_params()
        ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(q))
        for k, v in kw.items():
            setattr(q, k, v)
        return J(SIA(arch, grid, bed, q).run(H, nsteps))

    h = 1e-6
    fdG = (J_at(Gamma=p.Gamma * np.exp(h)) - J_at(Gamma=p.Gamma * np.exp(-h))) / (2 * h)
    fdE = (J_at(ela=p.ela + h) - J_at(ela=p.ela - h)) / (2 * h)
    assert abs(gG * p.Gamma - fdG) <= 1e-6 * abs(fdG), (gG * p.Gamma, fdG)
    assert abs(gE - fdE) <= 1e-6 * abs(fdE), (gE, fdE)
    # the initial thickness at an ice-covered interior cell
    idx = (H0.shape[0] // 2, H0.shape[1] // 2 + 3)
    Hp, Hm = H0.copy(), H0.copy()
    Hp[idx] += 1e-6
    Hm[idx] -= 1e-6
    fdH = (J_at(H=Hp) - J_at(H=Hm)) / 2e-6
    assert abs(gH0[idx] - fdH) <= 1e-6 * max(abs(fdH), float(np.abs(gH0).max())), (gH0[idx], fdH)


@pytest.mark.parametrize("glen_n", [3, 2, 4])
@pytest.mark.parametrize("tape", [True, False], ids=["taped", "recomputing"])
@pytest.mark.parametrize("dt_max", [0.5, 1e-3])
def test_sia_gradient_matches_dual_numbers(arch, dt_max, tape, glen_n):
    """The SIA adjoint gradients (GPU, reverse sweep) against forward-mode dual numbers run
    through the oracle's restated time loop (exact tangents of its arithmetic, including the
    adaptive dt through max D), for Glen exponents 3, 2 and 4: dJ/dGamma and dJ/dela agree
    to 1e-9 relative. The remaining difference is the rounding of two forward evaluations of
    the same discrete model."""
    from _oracle import NpField, desc_array, lib
    from chmy_gb300.adjoint import SIA
    from chmy_gb300.grids import Center, Vertex

    grid, bed, H0, p = _sia_problem(dt_max=dt_max)
    p.n = glen_n  # n = 2 and 4 reach the square-root forms of the derivatives of D
    nsteps = 60
    inner = (slice(2, -2), slice(2, -2))
    T = np.float64
    H = NpField(grid, Center(), T)
    H.a[...] = H0
    B = NpField(grid, Center(), T)
    B.a[...] = bed
    q = [NpField(grid, (Vertex(), Center()), T), NpField(grid, (Center(), Vertex()), T)]
    tG, tE = NpField(grid, Center(), T), NpField(grid, Center(), T)
    g = grid.desc()
    assert lib().or_sia_run_tangent(ctypes.byref(g), ctypes.byref(H.desc()), ctypes.byref(B.desc()), desc_array(q, 3),
                                    ctypes.byref(p), nsteps, ctypes.byref(tG.desc()), ctypes.byref(tE.desc())) == 0
    rng = np.random.default_rng(3)
    obs = H.a[inner] + 0.01 * rng.standard_normal(H.a[inner].shape)
    r = H.a[inner] - obs
    dual_G = float(np.sum(r * tG.a[inner]))
    dual_E = float(np.sum(r * tE.a[inner]))

    def dJ(h):
        out = np.zeros_like(h)
        out[inner] = h[inner] - obs
        return out

    sia = SIA(arch, grid, bed, p)
    gG, gE, _, HN = sia.gradient(H0, nsteps, dJ, tape=tape)
    assert np.max(np.abs(HN[inner] - H.a[inner])) <= 1e-12 * np.max(np.abs(H.a[inner]))
    assert abs(gG - dual_G) <= 1e-9 * abs(dual_G), (gG, dual_G)
    assert abs(gE - dual_E) <= 1e-9 * abs(dual_E), (gE, dual_E)


@pytest.mark.parametrize("T", [np.float32, np.float64])
def test_sia_taped_run_equals_plain_run_and_sweeps_agree(arch, T):
    """cg_sia_run_taped gives cg_sia_run's H and t bit for bit, and the taped reverse sweep
    (cg_sia_adjoint_run, nothing recomputed) agrees with the recomputing one
    (cg_sia_adjoint_step per step): dJ/dH0, dJ/dGamma and dJ/dela to 1e-12 (FP64) / 1e-4
    (FP32) relative. An odd step count ends the ping-pong in the work field."""
    import torch

    from chmy_gb300 import Field
    from chmy_gb300.adjoint import SIA
    from chmy_gb300.grids import Center, UniformGrid, Vertex

    grid0, bed, H0, p = _sia_problem(n=(45, 38))
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(45, 38), dtype=T)
    nsteps = 33
    C = Center()
    H, B = Field(arch, grid, C, T), Field(arch, grid, C, T)
    q = [Field(arch, grid, (Vertex(), C), T), Field(arch, grid, (C, Vertex()), T)]
    qd = (_abi.cg_field * 3)(q[0].desc(), q[1].desc(), _abi.cg_field())
    B.from_numpy(bed.astype(T))
    g = grid.desc()
    H.from_numpy(H0.astype(T))
    t_plain = ctypes.c_double()
    arch.call("cg_sia_run", ctypes.byref(g), ctypes.byref(H.desc()), ctypes.byref(B.desc()), qd, ctypes.byref(p), nsteps,
              ctypes.byref(t_plain))
    H_plain = H.to_numpy()
    nbytes = ctypes.c_size_t()
    assert arch.lib.cg_sia_tape_bytes(ctypes.byref(g), ctypes.byref(H.desc()), nsteps, ctypes.byref(nbytes)) == 0
    tape = torch.empty(nbytes.value, dtype=torch.uint8, device=H.data.device)
    H.from_numpy(H0.astype(T))
    t_taped = ctypes.c_double()
    arch.call("cg_sia_run_taped", ctypes.byref(g), ctypes.byref(H.desc()), ctypes.byref(B.desc()), qd, ctypes.byref(p), nsteps,
              ctypes.c_void_p(tape.data_ptr()), nbytes.value, ctypes.byref(t_taped))
    assert np.array_equal(H.to_numpy(), H_plain, equal_nan=True)
    assert t_taped.value == t_plain.value

    inner = (slice(2, -2), slice(2, -2))
    obs = H_plain[inner] * 0.9

    def dJ(h):
        out = np.zeros_like(h)
        out[inner] = h[inner] - obs
        return out

    sia = SIA(arch, grid, bed.astype(T), p, dtype=T)
    a = sia.gradient(H0.astype(T), nsteps, dJ, tape=True)
    b = sia.gradient(H0.astype(T), nsteps, dJ, tape=False, checkpoint_every=1)
    tol = 1e-12 if T == np.float64 else 1e-4
    assert abs(a[0] - b[0]) <= tol * abs(b[0]), (a[0], b[0])
    assert abs(a[1] - b[1]) <= tol * abs(b[1]), (a[1], b[1])
    ga, gb = a[2][2:-2, 2:-2].astype(np.float64), b[2][2:-2, 2:-2].astype(np.float64)
    assert np.max(np.abs(ga - gb)) <= tol * np.max(np.abs(gb))


def test_sia_adjoint_run_argument_errors(arch):
    """cg_sia_adjoint_run refuses a buffer without a tape header, parameters other than the taped
    run's, and aliased lambda and work."""
    import torch

    from chmy_gb300 import _abi as abi
    from chmy_gb300.adjoint import SIA

    grid, bed, H0, p = _sia_problem(n=(40, 32))
    sia = SIA(arch, grid, bed, p)
    sia.H.from_numpy(H0)
    sia._steps_taped(3)
    g = grid.desc()
    lam, work = sia.lam[0].desc(), sia.lam[1].desc()
    tp = ctypes.c_void_p(sia._tape.data_ptr())
    n = sia._tape.numel()
    blank = torch.zeros(4096, dtype=torch.uint8, device=sia.H.data.device)
    rc = arch.lib.cg_sia_adjoint_run(arch.ctx, ctypes.byref(g), ctypes.byref(p), ctypes.c_void_p(blank.data_ptr()), 4096,
                                     ctypes.byref(lam), ctypes.byref(work), None)
    assert rc == abi.CG_ERR_ARG
    q = abi.cg_sia_params()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(q))
    q.ela = p.ela + 0.1
    assert arch.lib.cg_sia_adjoint_run(arch.ctx, ctypes.byref(g), ctypes.byref(q), tp, n, ctypes.byref(lam), ctypes.byref(work), None) == abi.CG_ERR_ARG
    assert arch.lib.cg_sia_adjoint_run(arch.ctx, ctypes.byref(g), ctypes.byref(p), tp, n, ctypes.byref(lam), ctypes.byref(lam), None) == abi.CG_ERR_ARG
    assert arch.lib.cg_sia_adjoint_run(arch.ctx, ctypes.byref(g), ctypes.byref(p), tp, 100, ctypes.byref(lam), ctypes.byref(work), None) == abi.CG_ERR_ARG
    dJ = (ctypes.c_double * 2)()
    arch.call("cg_sia_adjoint_run", ctypes.byref(g), ctypes.byref(p), tp, n, ctypes.byref(lam), ctypes.byref(work), dJ)


def _ensemble_members(T=np.float64):
    """Three SIA members of uneven sizes (the 60-step problem above on each grid), with
    different ela and Gamma."""
    from chmy_gb300.grids import UniformGrid

    out = []
    for k, n in enumerate([(48, 40), (33, 57), (64, 64)]):
        g0, bed, H0, p = _sia_problem(n=n)
        grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=n, dtype=T)
        p.ela = 0.5 + 0.05 * k
        p.Gamma = 1.0 + 0.2 * k
        out.append((grid, bed.astype(T), H0.astype(T), p))
    return out


@pytest.mark.parametrize("T", [np.float32, np.float64])
def test_sia_ensemble_taped_run_equals_plain_run(arch, T):
    """cg_sia_ensemble_run_taped gives cg_sia_ensemble_run's H and t bit for bit."""
    from chmy_gb300.adjoint import SIAEnsemble

    mem = _ensemble_members(T)
    ens = SIAEnsemble(arch, [(g, b, p) for g, b, _, p in mem], dtype=T)
    H0s = [h for _, _, h, _ in mem]
    plain = ens.run(H0s, 25)
    ens._set(H0s)
    ens._steps_taped(25)
    for a, H in zip(plain, ens.H):
        assert np.array_equal(a, H.to_numpy(), equal_nan=True)


def test_sia_ensemble_gradient_matches_members_and_differences(arch):
    """The batched ensemble adjoint (cg_sia_ensemble_adjoint_run, all members per launch) against
    (a) each member's own taped gradient (cg_sia_adjoint_run): dJ/dGamma, dJ/dela and dJ/dH0 to
    1e-10 relative (the ensemble forward computes the same quantities in forms that differ in
    rounding); (b) segments of 7 steps: dJ/dH0 bit for bit, the sums to 1e-13; (c) central
    differences of one member's J in log(Gamma) and ela to 1e-6."""
    from chmy_gb300.adjoint import SIA, SIAEnsemble

    mem = _ensemble_members()
    nsteps = 60
    inner = (slice(2, -2), slice(2, -2))
    ens = SIAEnsemble(arch, [(g, b, p) for g, b, _, p in mem])
    H0s = [h for _, _, h, _ in mem]
    HN = ens.run(H0s, nsteps)
    rng = np.random.default_rng(4)
    obs = [h[inner] + 0.01 * rng.standard_normal(h[inner].shape) for h in HN]

    def dJ(m, h):
        g = np.zeros_like(h)
        g[inner] = h[inner] - obs[m]
        return g

    gG, gE, gH, HN2 = ens.gradient(H0s, nsteps, dJ)
    for a, b in zip(HN, HN2):
        assert np.array_equal(a, b)
    sG, sE, sH, _ = ens.gradient(H0s, nsteps, dJ, checkpoint_every=7)
    for m in range(len(mem)):
        assert np.array_equal(sH[m], gH[m])
        assert abs(sG[m] - gG[m]) <= 1e-13 * abs(gG[m]) and abs(sE[m] - gE[m]) <= 1e-13 * abs(gE[m])
    for m, (grid, bed, H0, p) in enumerate(mem):
        one = SIA(arch, grid, bed, p)
        a, b, c, _ = one.gradient(H0, nsteps, lambda h: dJ(m, h))
        assert abs(a - gG[m]) <= 1e-10 * abs(a), (m, a, gG[m])
        assert abs(b - gE[m]) <= 1e-10 * abs(b), (m, b, gE[m])
        assert np.max(np.abs(c[inner] - gH[m][inner])) <= 1e-10 * np.max(np.abs(c[inner]))

    m = 1
    grid, bed, H0, p = mem[m]

    def J_at(**kw):
        q = _abi.cg_sia_params()
        ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(q))
        for k, v in kw.items():
            setattr(q, k, v)
        e = SIAEnsemble(arch, [(g, b, q if i == m else pp) for i, (g, b, _, pp) in enumerate(mem)])
        r = e.run(H0s, nsteps)[m][inner] - obs[m]
        return 0.5 * float(np.sum(r * r))

    h = 1e-6
    fdG = (J_at(Gamma=p.Gamma * np.exp(h)) - J_at(Gamma=p.Gamma * np.exp(-h))) / (2 * h)
    fdE = (J_at(ela=p.ela + h) - J_at(ela=p.ela - h)) / (2 * h)
    assert abs(gG[m] * p.Gamma - fdG) <= 1e-6 * abs(fdG), (gG[m] * p.Gamma, fdG)
    assert abs(gE[m] - fdE) <= 1e-6 * abs(fdE), (gE[m], fdE)


def test_sia_ensemble_adjoint_run_argument_errors(arch):
    """cg_sia_ensemble_adjoint_run refuses a buffer without an ensemble tape header, parameters
    or members other than the taped run's (the header's hash), aliased lambda and work, and a
    tape shorter than its steps."""
    import torch

    from chmy_gb300.adjoint import SIAEnsemble

    mem = _ensemble_members()
    ens = SIAEnsemble(arch, [(g, b, p) for g, b, _, p in mem])
    ens._set([h for _, _, h, _ in mem])
    ens._steps_taped(3)
    tp, n = ctypes.c_void_p(ens._tape.data_ptr()), ens._tape.numel()

    def call(par=None, tape=tp, nbytes=n, lam=None, nm=None):
        return arch.lib.cg_sia_ensemble_adjoint_run(arch.ctx, nm or ens.nm, ens._mem, par or ens._par, tape, nbytes,
                                                    lam or ens._lam, ens._work, None)

    blank = torch.zeros(4096, dtype=torch.uint8, device=ens.H[0].data.device)
    assert call(tape=ctypes.c_void_p(blank.data_ptr()), nbytes=4096) == _abi.CG_ERR_ARG
    par = (_abi.cg_sia_params * ens.nm)(*ens.params)
    par[1].Gamma = par[1].Gamma * 1.5
    assert call(par=par) == _abi.CG_ERR_ARG
    assert call(nm=ens.nm - 1) == _abi.CG_ERR_ARG
    assert call(lam=ens._work) == _abi.CG_ERR_ARG
    assert call(nbytes=n // 2) == _abi.CG_ERR_ARG
    dJ = (ctypes.c_double * (2 * ens.nm))()
    arch.call("cg_sia_ensemble_adjoint_run", ens.nm, ens._mem, ens._par, tp, n, ens._lam, ens._work, dJ)


def _explicit_setup(nd, kinds, seed=7):
    from chmy_gb300.bcs import Dirichlet, Neumann, Periodic, to_cg_bc
    from chmy_gb300.configs import padded_mesh
    from chmy_gb300.grids import Center, UniformGrid

    T = np.float64
    dims = (20, 16) if nd == 2 else (12, 10, 9)
    grid = UniformGrid(origin=(T(-1),) * nd, extent=(T(2),) * nd, dims=dims, dtype=T)
    xs = padded_mesh(grid, Center())
    r2 = sum(x * x for x in xs)
    rng = np.random.default_rng(seed)
    C0 = np.exp(-r2 / 0.1) + 0.01 * rng.standard_normal(xs[0].shape)
    if kinds == "neumann_dirichlet":
        spec = {"x": Neumann(0.3), "y": Dirichlet(0.2)}
    else:
        spec = {"x": Periodic(), "y": Neumann()}
    if nd == 3:
        spec["z"] = (Dirichlet(0.1), Neumann())
    bc = to_cg_bc(nd, spec)
    h = float(min(grid.spacing()))
    dt = h * h / (2.05 * nd)
    inner = (slice(2, -2),) * nd
    w = np.zeros_like(C0)
    w[inner] = rng.standard_normal(w[inner].shape)
    dirv = np.zeros_like(C0)
    dirv[inner] = rng.standard_normal(dirv[inner].shape)
    return grid, C0, bc, dt, inner, w, dirv


@pytest.mark.parametrize("nd,kinds", [(2, "neumann_dirichlet"), (2, "periodic"), (3, "neumann_dirichlet")])
def test_explicit_diffusion_gradient_matches_dual_numbers_and_differences(arch, nd, kinds):
    """The explicit diffusion loop's adjoint (taped forward, one reverse sweep) for
    J = 1/2 sum w C^N^2 over the interior: dJ/dchi and the directional derivative of J along an
    initial-state direction agree with the dual-number tangents of the oracle's loop to 1e-9, and
    with central differences of the GPU's own forward runs to 1e-6. Segments of 7 steps give the
    same dJ/dC0 bits, and dJ/dchi to 1e-13."""
    from _oracle import diffusion_tangent_run

    from chmy_gb300.adjoint import ExplicitDiffusion

    grid, C0, bc, dt, inner, w, dirv = _explicit_setup(nd, kinds)
    chi, nsteps = 1.0, 30
    ed = ExplicitDiffusion(arch, grid, chi, dt, bc)

    def J(c):
        return 0.5 * float(np.sum(w[inner] * c[inner] ** 2))

    gchi, gC0, CN = ed.gradient(C0, nsteps, lambda c: w * c)
    CN_ref, dchi, ddir = diffusion_tangent_run(grid, C0, chi, dt, bc, nsteps, dirv)
    assert np.max(np.abs(CN[inner] - CN_ref[inner])) <= 1e-12 * nsteps * np.abs(CN_ref[inner]).max()
    dual_chi = float(np.sum(w[inner] * CN_ref[inner] * dchi[inner]))
    dual_dir = float(np.sum(w[inner] * CN_ref[inner] * ddir[inner]))
    adj_dir = float(np.sum(gC0[inner] * dirv[inner]))
    assert abs(gchi - dual_chi) <= 1e-9 * abs(dual_chi), (gchi, dual_chi)
    assert abs(adj_dir - dual_dir) <= 1e-9 * abs(dual_dir), (adj_dir, dual_dir)
    e = 1e-6
    fd_chi = (J(ExplicitDiffusion(arch, grid, chi + e, dt, bc).run(C0, nsteps))
              - J(ExplicitDiffusion(arch, grid, chi - e, dt, bc).run(C0, nsteps))) / (2 * e)
    assert abs(gchi - fd_chi) <= 1e-6 * abs(fd_chi), (gchi, fd_chi)
    cell = tuple(s.start + 3 for s in inner)
    bump = np.zeros_like(C0)
    bump[cell] = 1.0
    fd_cell = (J(ed.run(C0 + e * bump, nsteps)) - J(ed.run(C0 - e * bump, nsteps))) / (2 * e)
    assert abs(gC0[cell] - fd_cell) <= 1e-6 * np.abs(gC0[inner]).max(), (gC0[cell], fd_cell)
    gchi7, gC07, _ = ed.gradient(C0, nsteps, lambda c: w * c, checkpoint_every=7)
    np.testing.assert_array_equal(gC07[inner], gC0[inner])
    assert abs(gchi7 - gchi) <= 1e-13 * abs(gchi)


def test_explicit_diffusion_adjoint_checks_the_tape(arch):
    """The reverse sweep refuses a tape whose header does not match its arguments (another chi,
    another boundary kind), and a boundary side without a rule."""
    import ctypes as C

    import torch

    from chmy_gb300.adjoint import ExplicitDiffusion
    from chmy_gb300.bcs import Neumann, to_cg_bc

    grid, C0, bc, dt, inner, w, dirv = _explicit_setup(2, "neumann_dirichlet")
    ed = ExplicitDiffusion(arch, grid, 1.0, dt, bc)
    ed.C.from_numpy(C0)
    nb = ed.tape_bytes(4)
    tape = torch.empty(nb, dtype=torch.uint8, device=ed.C.data.device)
    g = grid.desc()
    arch.call("cg_diffusion_run_taped", C.byref(g), C.byref(ed.C.desc()), 1.0, dt, C.byref(bc), 4, C.c_void_p(tape.data_ptr()), nb)
    dJ = (C.c_double * 1)()
    args = (C.byref(g), C.c_void_p(tape.data_ptr()), nb, C.byref(ed.lam[0].desc()), C.byref(ed.lam[1].desc()))
    assert arch.lib.cg_diffusion_adjoint_run(arch.ctx, *args, 1.5, dt, C.byref(bc), dJ) == _abi.CG_ERR_ARG
    other = to_cg_bc(2, Neumann())
    assert arch.lib.cg_diffusion_adjoint_run(arch.ctx, *args, 1.0, dt, C.byref(other), dJ) == _abi.CG_ERR_ARG
    assert arch.lib.cg_diffusion_adjoint_run(arch.ctx, *args, 1.0, dt, C.byref(bc), dJ) == _abi.CG_OK
    none = to_cg_bc(2, {"x": Neumann()})
    assert arch.lib.cg_diffusion_adjoint_run(arch.ctx, *args, 1.0, dt, C.byref(none), dJ) == _abi.CG_ERR_UNSUPPORTED


@pytest.mark.parametrize("nd,kinds", [(2, "neumann_dirichlet"), (2, "periodic"), (3, "neumann_dirichlet")])
def test_thermal_step_adjoint_matches_dual_numbers(arch, nd, kinds):
    """The fused thermal step's vector-Jacobian product (cg_stokes_thermal_step_adjoint) against
    the dual-number tangents of the oracle's two-kernel step: for J = sum mu T_out over the
    interior, <dJ/dT, dT> + <dJ/dT_old, dT_old> + <dJ/dV, dV> equals the tangent along those
    directions, and dJ/dlambda the tangent along lambda_rhoCp, to 1e-11 (FP64); the FP32 kernel's
    gradients agree with the FP64 ones to 1e-4. dJ/dlambda also matches central differences of the
    GPU's forward step."""
    import ctypes as C

    from _oracle import thermal_problem, thermal_tangent_step
    from chmy_gb300.bcs import Dirichlet, Neumann, Periodic, to_cg_bc
    from chmy_gb300.grids import Center, UniformGrid
    from chmy_gb300.kernels import stokes_fields, stokes_params
    from gpu_helpers import to_gpu

    T = np.float64
    dims = (18, 14) if nd == 2 else (11, 9, 8)
    grid = UniformGrid(origin=(T(-1),) * nd, extent=(T(2),) * nd, dims=dims, dtype=T)
    spec = {"x": Neumann(0.2), "y": Dirichlet(0.5)} if kinds == "neumann_dirichlet" else {"x": Periodic(), "y": Neumann()}
    if nd == 3:
        spec["z"] = (Neumann(), Dirichlet(-0.1))
    bc_T = to_cg_bc(nd, spec)
    pr = thermal_problem(grid, 11, bc_T)
    p = stokes_params(G=1.0, dt=2e-3, lambda_rhoCp=0.3)
    _, tan = thermal_tangent_step(grid, pr, p, bc_T)
    inner, mu = pr["inner"], pr["mu"]

    def adjoint(dtype):
        def dev(arr, loc):
            from _oracle import NpField

            f = NpField(grid, loc, dtype)
            f.a[...] = arr.astype(dtype)
            return to_gpu(arch, f)

        Tg = dev(pr["T"].a, Center())
        Vg = [dev(v.a, l) for v, l in zip(pr["V"], pr["vlocs"])]
        mug = dev(mu, Center())
        gT = dev(np.zeros_like(mu), Center())
        gTo = dev(np.zeros_like(mu), Center())
        gV = [dev(np.zeros_like(v.a), l) for v, l in zip(pr["V"], pr["vlocs"])]
        f = stokes_fields(V=Vg, T=Tg)
        dl = (C.c_double * 1)(0.0)
        arch.call("cg_stokes_thermal_step_adjoint", C.byref(grid.desc()), C.byref(f), C.byref(p), C.byref(bc_T),
                  C.byref(mug.desc()), C.byref(gT.desc()), C.byref(gTo.desc()), (_abi.cg_field * 3)(*[g.desc() for g in gV]), dl)
        return gT.to_numpy(), gTo.to_numpy(), [g.to_numpy() for g in gV], dl[0]

    gT, gTo, gV, dlam = adjoint(np.float64)
    lhs = float(np.sum(gT[inner] * pr["dT"][inner]) + np.sum(gTo[inner] * pr["dT_old"][inner])
                + sum(np.sum(g * d) for g, d in zip(gV, pr["dV"])))
    dual_dir = float(np.sum(mu[inner] * tan[0][inner]))
    dual_lam = float(np.sum(mu[inner] * tan[1][inner]))
    assert abs(lhs - dual_dir) <= 1e-11 * abs(dual_dir), (lhs, dual_dir)
    assert abs(dlam - dual_lam) <= 1e-11 * abs(dual_lam), (dlam, dual_lam)
    np.testing.assert_array_equal(gTo[inner], mu[inner])
    # FP32 kernel
    gT32, _, gV32, dlam32 = adjoint(np.float32)
    assert np.max(np.abs(gT32[inner] - gT[inner])) <= 1e-4 * np.abs(gT[inner]).max()
    for a, b in zip(gV32, gV):
        assert np.max(np.abs(a - b)) <= 1e-4 * np.abs(b).max()
    assert abs(dlam32 - dlam) <= 1e-4 * abs(dlam)
    # central differences of the GPU's forward step in lambda_rhoCp
    from _oracle import NpField

    def J(lam):
        q = stokes_params(G=1.0, dt=2e-3, lambda_rhoCp=lam)
        Tg = to_gpu(arch, pr["T"])
        Tog = to_gpu(arch, pr["T_old"])
        Vg = [to_gpu(arch, v) for v in pr["V"]]
        out = to_gpu(arch, NpField(grid, Center(), np.float64))
        arch.call("cg_stokes_thermal_step", C.byref(grid.desc()), C.byref(stokes_fields(V=Vg, T=Tg, T_old=Tog)), C.byref(q),
                  C.byref(bc_T), C.byref(out.desc()))
        return float(np.sum(mu[inner] * out.to_numpy()[inner]))

    e = 1e-6
    fd = (J(0.3 + e) - J(0.3 - e)) / (2 * e)
    assert abs(dlam - fd) <= 1e-6 * abs(fd), (dlam, fd)
