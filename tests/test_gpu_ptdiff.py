"""GPU parity of the PT variable-coefficient diffusion kernels against the oracle."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, desc_array, lib
from chmy_gb300 import _abi
from chmy_gb300.bcs import Dirichlet, Neumann, Periodic, to_cg_bc
from chmy_gb300.configs import ptdiff_params
from chmy_gb300.grids import Center, UniformGrid, Vertex
from gpu_helpers import assert_close, random_field, rtol_for, to_gpu

pytestmark = pytest.mark.gpu
TYPES = [np.float32, np.float64]
C_, V_ = Center(), Vertex()


def fields(arch, dims, T, seed, pitch_align=0):
    nd = len(dims)
    rng = np.random.default_rng(seed)
    grid = UniformGrid(origin=(T(-0.5),) * nd, extent=(T(1),) * nd, dims=dims, dtype=T)
    h = {
        "C": random_field(grid, C_, T, rng),
        "C_old": random_field(grid, C_, T, rng),
        "D": NpField(grid, C_, T),
        "q": [random_field(grid, tuple(V_ if e == d else C_ for e in range(nd)), T, rng, 0.1) for d in range(nd)],
        "R": NpField(grid, C_, T),
    }
    h["D"].a[...] = np.exp(rng.uniform(-1, 1, h["D"].a.shape)).astype(T)
    # pitch_align: every array on one row pitch and (3D) plane height, as the fused path needs
    rows = dims[1] + 5 if nd == 3 else 0
    d = {k: ([to_gpu(arch, f, pitch_align, rows) for f in v] if isinstance(v, list) else to_gpu(arch, v, pitch_align, rows))
         for k, v in h.items()}
    return grid, h, d


def desc(fs):
    s = _abi.cg_ptdiff_fields()
    s.C, s.C_old, s.D, s.R = fs["C"].desc(), fs["C_old"].desc(), fs["D"].desc(), fs["R"].desc()
    s.q = desc_array(fs["q"], 3)
    return s


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(40,), (33, 21), (17, 12, 14)])
def test_kernels(arch, T, dims):
    grid, h, d = fields(arch, dims, T, 3)
    p = ptdiff_params(grid, dt=1e-3, Dmax=float(h["D"].a.max()))
    g = grid.desc()
    hd, dd = desc(h), desc(d)
    for name in ("update_q", "update_C"):
        assert getattr(lib(), "or_ptdiff_" + name)(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p)) == 0
        arch.call("cg_ptdiff_" + name, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p))
        arch.synchronize()
        for k in ("C", "R"):
            assert_close(d[k], h[k], rtol_for(T), f"{name} {k}")
        for a, b in zip(d["q"], h["q"]):
            assert_close(a, b, rtol_for(T), f"{name} q")


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(48, 40), (20, 18, 16)])
def test_run_matches_oracle_steps(arch, T, dims):
    grid, h, d = fields(arch, dims, T, 8)
    nd = len(dims)
    p = ptdiff_params(grid, dt=1e-3, Dmax=float(h["D"].a.max()))
    spec = {"x": Dirichlet(0.0)}
    for e in range(1, nd):
        spec["xyz"[e]] = Neumann()
    bc = to_cg_bc(nd, spec)
    g = grid.desc()
    hd = desc(h)
    nsteps, npt = 2, 12
    for _ in range(nsteps):
        h["C_old"].a[...] = h["C"].a
        for _ in range(npt):
            lib().or_ptdiff_update_q(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
            lib().or_ptdiff_update_C(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
            bc_apply(grid, [h["C"]], [bc])
    arch.call("cg_ptdiff_run", ctypes.byref(g), ctypes.byref(desc(d)), ctypes.byref(p), ctypes.byref(bc), nsteps, npt)
    arch.synchronize()
    assert_close(d["C"], h["C"], rtol_for(T) * nsteps * npt, "C")
    assert_close(d["C_old"], h["C_old"], rtol_for(T) * nsteps * npt, "C_old")


@pytest.mark.parametrize("dims", [(17, 12, 14), (31, 9, 40), (64, 33, 20), (30, 30, 30), (2, 2, 3)])
@pytest.mark.parametrize("npt", [7, 12])
def test_fused_run_bitwise(arch, dims, npt):
    """cg_ptdiff_run on a 3D FP32 grid with one shared layout and no residual output takes the
    fused single-pass iteration (ping-pong partners, bc! per iteration): C, C_old and q equal
    the oracle's update_q!/update_C!/bc! steps bit for bit, for odd and even iteration counts
    and for grids that do not fill the kernel's 32 x 8 tiles."""
    T = np.float32
    grid, h, d = fields(arch, dims, T, 8, pitch_align=128)
    p = ptdiff_params(grid, dt=1e-3, Dmax=float(h["D"].a.max()))
    bc = to_cg_bc(3, {"x": Dirichlet(0.25), "y": Neumann(0.5), "z": (Neumann(), Dirichlet(-0.5))})
    g = grid.desc()
    hd = desc(h)
    nsteps = 2
    for _ in range(nsteps):
        h["C_old"].a[...] = h["C"].a
        for _ in range(npt):
            lib().or_ptdiff_update_q(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
            lib().or_ptdiff_update_C(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
            bc_apply(grid, [h["C"]], [bc])
    dd = desc(d)
    dd.R = _abi.cg_field()  # no residual output: the fused path
    arch.call("cg_ptdiff_run", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(bc), nsteps, npt)
    arch.synchronize()
    for k in ("C", "C_old"):
        assert_close(d[k], h[k], 0.0, k, exact=True)
    for a, b in zip(d["q"], h["q"]):
        assert_close(a, b, 0.0, "q", exact=True)


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("dims", [(17, 12, 14), (64, 33, 20), (2, 2, 3), (70, 19, 41)])
def test_fused_run_every_layout_bitwise(arch, monkeypatch, variant, dims):
    """Every launch layout of the fused iteration, forced with CG_PTD_VARIANT — the register-fed
    ptd_march3d_kernel at four block shapes (0-3) and the TMA-fed ptd_tma_kernel with blocks of
    8, 16, 20 and 24 rows (4-7), whose inputs stream through a ring of shared-memory planes —
    gives the oracle's
    update_q!/update_C!/bc! states bit for bit. The caller's fields (first padded element 12
    bytes past a 16-byte boundary) and the library's partner buffers (aligned) take different
    tensor-map offsets."""
    monkeypatch.setenv("CG_PTD_VARIANT", str(variant))
    T = np.float32
    grid, h, d = fields(arch, dims, T, 8, pitch_align=128)
    p = ptdiff_params(grid, dt=1e-3, Dmax=float(h["D"].a.max()))
    bc = to_cg_bc(3, {"x": Dirichlet(0.25), "y": Neumann(0.5), "z": (Neumann(), Dirichlet(-0.5))})
    g = grid.desc()
    hd = desc(h)
    npt = 9
    h["C_old"].a[...] = h["C"].a
    for _ in range(npt):
        lib().or_ptdiff_update_q(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        lib().or_ptdiff_update_C(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        bc_apply(grid, [h["C"]], [bc])
    dd = desc(d)
    dd.R = _abi.cg_field()
    arch.call("cg_ptdiff_run", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(bc), 1, npt)
    arch.synchronize()
    for k in ("C", "C_old"):
        assert_close(d[k], h[k], 0.0, f"{k} variant {variant}", exact=True)
    for a, b in zip(d["q"], h["q"]):
        assert_close(a, b, 0.0, f"q variant {variant}", exact=True)


def test_tma_wait_runs_out_and_the_context_stays_usable(arch, monkeypatch):
    """Failure detection of the TMA-fed iteration without a GPU fault: the producing thread
    withholds the copies of one ring plane (CG_TMA_WITHHOLD_PLANE) and every wait is limited to
    20 ms (CG_TMA_WAIT_LIMIT_MS). The waits for that plane run out, the blocks stop (the
    producer first waits, bounded, for its copies in flight) and cg_ptdiff_run reports
    CG_ERR_TIMEOUT. The same context then runs the iteration to the oracle's bits."""
    import time

    T = np.float32
    monkeypatch.setenv("CG_PTD_VARIANT", "4")
    monkeypatch.setenv("CG_TMA_WAIT_LIMIT_MS", "20")
    monkeypatch.setenv("CG_TMA_WITHHOLD_PLANE", "5")
    dims = (40, 30, 24)
    grid, h, d = fields(arch, dims, T, 8, pitch_align=128)
    p = ptdiff_params(grid, dt=1e-3, Dmax=float(h["D"].a.max()))
    bc = to_cg_bc(3, {"x": Dirichlet(0.25), "y": Neumann(0.5), "z": Neumann()})
    g = grid.desc()
    dd = desc(d)
    dd.R = _abi.cg_field()
    t0 = time.perf_counter()
    rc = arch.lib.cg_ptdiff_run(arch.ctx, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(bc), 1, 4)
    waited = time.perf_counter() - t0
    assert rc == _abi.CG_ERR_TIMEOUT, (rc, arch.lib.cg_last_error(arch.ctx))
    assert b"timed out" in arch.lib.cg_last_error(arch.ctx)
    assert waited < 10.0, waited  # the 20 ms limits applied, not the 2 s default
    monkeypatch.delenv("CG_TMA_WITHHOLD_PLANE")
    monkeypatch.delenv("CG_TMA_WAIT_LIMIT_MS")
    grid, h, d = fields(arch, dims, T, 9, pitch_align=128)
    hd = desc(h)
    npt = 4
    h["C_old"].a[...] = h["C"].a
    for _ in range(npt):
        lib().or_ptdiff_update_q(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        lib().or_ptdiff_update_C(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        bc_apply(grid, [h["C"]], [bc])
    dd = desc(d)
    dd.R = _abi.cg_field()
    arch.call("cg_ptdiff_run", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(bc), 1, npt)
    arch.synchronize()
    assert_close(d["C"], h["C"], 0.0, "C after a timed-out run", exact=True)


def _np_residual(C, Co, D, idx, dt):
    """max |R| dt over the interior of the implicit step R = -(C - C_old)/dt - divg(q(C)),
    q(C) = -lerp(D) ∂C, on padded [z, y, x] arrays with halo 1 (logical I at padded I + 1)."""
    sl = slice(2, -2)
    c = C[sl, sl, sl]
    dv = np.zeros_like(c)
    for ax, h in zip((2, 1, 0), idx):  # x, y, z
        def sh(a, o):
            s = [sl, sl, sl]
            s[ax] = slice(2 + o, a.shape[ax] - 2 + o)
            return a[tuple(s)]
        dc = D[sl, sl, sl]
        ql = -(0.5 * (dc - sh(D, -1)) + sh(D, -1)) * ((c - sh(C, -1)) * h)
        qr = -(0.5 * (sh(D, 1) - dc) + dc) * ((sh(C, 1) - c) * h)
        dv += (qr - ql) * h
    R = -(c - Co[sl, sl, sl]) / dt - dv
    return float(np.max(np.abs(R))) * dt


def test_solve_fp64_and_fp32_defect_correction(arch):
    """cg_ptdiff_solve (one implicit step, 3D): the FP64 PT solve and the FP32 PT solve inside
    FP64 defect correction both reach err < eps, satisfy the implicit step's equation (numpy
    residual) and agree with the oracle's PT iterations run to convergence."""
    from chmy_gb300.configs import box_smooth, padded_mesh

    T = np.float64
    dims = (24, 20, 28)
    grid = UniformGrid(origin=(T(-0.5),) * 3, extent=(T(1),) * 3, dims=dims, dtype=T)
    x, y, z = padded_mesh(grid, C_)
    rng = np.random.default_rng(4)
    D0 = np.exp(box_smooth(rng.standard_normal(x.shape))).astype(T)
    C0 = np.exp(-(x * x + y * y + z * z) / 0.01).astype(T)
    bc = to_cg_bc(3, {"x": (Dirichlet(0.1), Dirichlet(-0.2)), "y": Neumann(0.3), "z": Neumann()})
    dt = 2e-3
    p = ptdiff_params(grid, dt=dt, Dmax=float(D0.max()))
    idx = [float(v) for v in grid.desc().inv_spacing[:3]]
    eps = 1e-11

    def field_set():
        h = {"C": NpField(grid, C_, T), "C_old": NpField(grid, C_, T), "D": NpField(grid, C_, T),
             "q": [NpField(grid, tuple(V_ if e == d else C_ for e in range(3)), T) for d in range(3)],
             "R": NpField(grid, C_, T)}
        h["C"].a[...] = C0
        bc_apply(grid, [h["C"]], [bc])
        h["C_old"].a[...] = h["C"].a
        h["D"].a[...] = D0
        return h

    # the oracle's PT iterations, run until the step's residual is far below eps
    h = field_set()
    g = grid.desc()
    hd = desc(h)
    for _ in range(40):
        for _ in range(250):
            lib().or_ptdiff_update_q(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
            lib().or_ptdiff_update_C(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
            bc_apply(grid, [h["C"]], [bc])
        if _np_residual(h["C"].a, h["C_old"].a, D0, idx, dt) < 1e-3 * eps:
            break
    ref = h["C"].a.copy()
    assert _np_residual(ref, h["C_old"].a, D0, idx, dt) < 1e-2 * eps

    results = {}
    for prec in (_abi.CG_F64, _abi.CG_F32):
        hs = field_set()
        d = {k: ([to_gpu(arch, f) for f in v] if isinstance(v, list) else to_gpu(arch, v)) for k, v in hs.items()}
        o = _abi.cg_solve_opts()
        o.max_iter, o.ncheck, o.eps, o.precision, o.max_outer, o.inner_rtol = 200000, 100, eps, prec, 20, 1e-4
        res = _abi.cg_solve_result()
        arch.call("cg_ptdiff_solve", ctypes.byref(g), ctypes.byref(desc(d)), ctypes.byref(p), ctypes.byref(bc), ctypes.byref(o), ctypes.byref(res))
        arch.synchronize()
        assert res.converged == 1 and res.err[0] < eps, (prec, res.err[0], res.iterations)
        C = d["C"].to_numpy()
        assert _np_residual(C, hs["C_old"].a, D0, idx, dt) < 2 * eps, prec
        err = float(np.max(np.abs(C - ref))) / float(np.max(np.abs(ref)))
        assert err < 1e-9, (prec, err)
        results[prec] = res
    # the defect correction needs at most a few FP64 cycles
    assert 1 <= results[_abi.CG_F32].outer <= 6


def test_solve_argument_errors(arch):
    T = np.float64
    grid, h, d = fields(arch, (8, 8, 8), T, 1)
    p = ptdiff_params(grid, dt=1e-3, Dmax=float(h["D"].a.max()))
    o = _abi.cg_solve_opts()
    o.max_iter, o.ncheck, o.eps, o.precision, o.max_outer, o.inner_rtol = 100, 10, 1e-8, _abi.CG_F64, 4, 1e-3
    res = _abi.cg_solve_result()
    g = grid.desc()
    periodic = to_cg_bc(3, {"x": Dirichlet(0.0), "y": Neumann(), "z": Periodic()})
    rc = arch.lib.cg_ptdiff_solve(arch.ctx, ctypes.byref(g), ctypes.byref(desc(d)), ctypes.byref(p), ctypes.byref(periodic),
                                  ctypes.byref(o), ctypes.byref(res))
    assert rc == _abi.CG_ERR_UNSUPPORTED
    o.precision = 7
    bc = to_cg_bc(3, {"x": Dirichlet(0.0), "y": Neumann(), "z": Neumann()})
    rc = arch.lib.cg_ptdiff_solve(arch.ctx, ctypes.byref(g), ctypes.byref(desc(d)), ctypes.byref(p), ctypes.byref(bc),
                                  ctypes.byref(o), ctypes.byref(res))
    assert rc == _abi.CG_ERR_ARG
