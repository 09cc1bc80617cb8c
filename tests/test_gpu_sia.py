"""GPU parity of the shallow-ice kernels (examples/sia.jl) against the oracle."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, desc_array, lib
from chmy_gb300 import _abi
from chmy_gb300.configs import padded_mesh
from chmy_gb300.grids import Center, UniformGrid, Vertex
from gpu_helpers import assert_close, rtol_for, to_gpu

pytestmark = pytest.mark.gpu
TYPES = [np.float32, np.float64]


def reference_params(As=0.5):
    p = _abi.cg_sia_params()
    p.Gamma, p.As, p.n, p.beta, p.ela, p.m_max, p.dt_max, p.cfl = 1.0, As, 3, 0.5, 0.3, 0.25, 0.5, 4.1
    return p


def bed(x, y):
    """The bed of examples/sia.jl:30-36."""
    b1 = 0.3 * np.exp(-(((x - 0.5) / 0.3) ** 2) - ((y - 0.0) / 0.5) ** 2)
    b2 = 0.3 * np.exp(-(((x + 0.5) / 0.3) ** 2) - ((y - 0.0) / 0.5) ** 2)
    b3 = 1.0 * np.exp(-((x / 0.5) ** 2) - ((y - 0.5) / 0.5) ** 2)
    return b1 + b2 + b3


def setup(T, n=(40, 33), seed=4):
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=n, dtype=T)
    rng = np.random.default_rng(seed)
    x, y = padded_mesh(grid, Center())
    B = NpField(grid, Center(), T)
    B.a[...] = bed(x, y).astype(T)
    H = NpField(grid, Center(), T)
    H.interior()[...] = (0.05 + 0.3 * rng.random(H.dims)).astype(T)
    q = [NpField(grid, (Vertex(), Center()), T), NpField(grid, (Center(), Vertex()), T)]
    return grid, H, B, q


@pytest.mark.parametrize("T", TYPES)
def test_update_q_and_H(arch, T):
    grid, H, B, q = setup(T)
    p = reference_params()
    Hg, Bg = to_gpu(arch, H), to_gpu(arch, B)
    qg = [to_gpu(arch, f) for f in q]
    g = grid.desc()
    dmax_ref, dmax = ctypes.c_double(), ctypes.c_double()
    assert lib().or_sia_update_q(ctypes.byref(g), desc_array(q, 3), ctypes.byref(H.desc()), ctypes.byref(B.desc()), ctypes.byref(p), ctypes.byref(dmax_ref)) == 0
    arch.call("cg_sia_update_q", ctypes.byref(g), desc_array(qg, 3), ctypes.byref(Hg.desc()), ctypes.byref(Bg.desc()), ctypes.byref(p), ctypes.byref(dmax))
    arch.synchronize()
    for a, b in zip(qg, q):
        assert_close(a, b, rtol_for(T), "q")
    assert abs(dmax.value - dmax_ref.value) <= rtol_for(T) * dmax_ref.value
    dt = 1e-3
    assert lib().or_sia_update_H(ctypes.byref(g), ctypes.byref(H.desc()), desc_array(q, 3), ctypes.byref(B.desc()), dt, ctypes.byref(p)) == 0
    arch.call("cg_sia_update_H", ctypes.byref(g), ctypes.byref(Hg.desc()), desc_array(qg, 3), ctypes.byref(Bg.desc()), dt, ctypes.byref(p))
    arch.synchronize()
    assert_close(Hg, H, rtol_for(T), "H")


@pytest.mark.parametrize("T", TYPES)
def test_run_matches_reference_time_loop(arch, T):
    """cg_sia_run (device Δt, graph) == the reference loop: update_q!, bc!, Δt from
    maximum(interior(D)), update_H!, bc! (examples/sia.jl:71-81)."""
    grid, H, B, q = setup(T, n=(48, 40), seed=9)
    p = reference_params()
    Hg, Bg = to_gpu(arch, H), to_gpu(arch, B)
    qg = [to_gpu(arch, f) for f in q]
    g = grid.desc()
    nsteps = 25
    dx = min(grid.spacing())
    t_ref = 0.0
    for _ in range(nsteps):
        dmax = ctypes.c_double()
        lib().or_sia_update_q(ctypes.byref(g), desc_array(q, 3), ctypes.byref(H.desc()), ctypes.byref(B.desc()), ctypes.byref(p), ctypes.byref(dmax))
        dt_diff = T(T(dx) * T(dx)) / T(dmax.value) / T(4.1)
        dt = min(float(dt_diff), 0.5)
        lib().or_sia_update_H(ctypes.byref(g), ctypes.byref(H.desc()), desc_array(q, 3), ctypes.byref(B.desc()), dt, ctypes.byref(p))
        t_ref += dt
    t = ctypes.c_double()
    arch.call("cg_sia_run", ctypes.byref(g), ctypes.byref(Hg.desc()), ctypes.byref(Bg.desc()), desc_array(qg, 3), ctypes.byref(p), nsteps, ctypes.byref(t))
    arch.synchronize()
    assert_close(Hg, H, rtol_for(T) * nsteps, "H after steps")
    assert abs(t.value - t_ref) <= rtol_for(T) * nsteps * t_ref
    # ice thickness stays non-negative
    assert (Hg.to_numpy() >= 0).all()


def test_ensemble_matches_members(arch):
    """cg_sia_ensemble_run (batched launches over members of uneven sizes, folded bc!) ==
    cg_sia_run per member, for H over the interior and the ghost layer."""
    from chmy_gb300.configs import sia_ensemble

    T = np.float64
    ens = sia_ensemble(members=5, nmin=40, nmax=130, seed=11)
    nsteps = 30
    rng = np.random.default_rng(1)
    singles, batch = [], []
    for grid, h, p in ens:
        H0 = NpField(grid, Center(), T)
        H0.interior()[...] = rng.random(H0.dims) * 0.3  # start with ice so that D > 0
        B = NpField(grid, Center(), T)
        B.a[...] = h["B"]
        q = [NpField(grid, (Vertex(), Center()), T), NpField(grid, (Center(), Vertex()), T)]
        for store in (singles, batch):
            store.append((grid, to_gpu(arch, H0), to_gpu(arch, B), [to_gpu(arch, f) for f in q], p))
    t_single = []
    for grid, Hg, Bg, qg, p in singles:
        t = ctypes.c_double()
        arch.call("cg_sia_run", ctypes.byref(grid.desc()), ctypes.byref(Hg.desc()), ctypes.byref(Bg.desc()), desc_array(qg, 3), ctypes.byref(p), nsteps, ctypes.byref(t))
        t_single.append(t.value)
    mem = (_abi.cg_sia_member * len(batch))()
    params = (_abi.cg_sia_params * len(batch))()
    for k, (grid, Hg, Bg, qg, p) in enumerate(batch):
        mem[k].grid = grid.desc()
        mem[k].H, mem[k].B = Hg.desc(), Bg.desc()
        mem[k].q[0], mem[k].q[1] = qg[0].desc(), qg[1].desc()
        params[k] = p
    ts = (ctypes.c_double * len(batch))()
    arch.call("cg_sia_ensemble_run", len(batch), mem, params, nsteps, ts)
    arch.synchronize()
    for k, ((grid, Ha, _, _, _), (_, Hb, _, _, _)) in enumerate(zip(singles, batch)):
        a, b = Ha.to_numpy()[1:-1, 1:-1], Hb.to_numpy()[1:-1, 1:-1]
        assert np.max(np.abs(a - b)) <= 1e-12 * nsteps * max(np.abs(a).max(), 1e-30), k
        assert abs(ts[k] - t_single[k]) <= 1e-12 * nsteps * t_single[k]


@pytest.mark.parametrize("T", TYPES)
def test_ensemble_persistent_launch_equals_phase_launches(arch, monkeypatch, T):
    """The ensemble's single persistent cooperative launch (grid barriers between phases) gives
    the same bits as one launch per phase (CG_SIA_PERSISTENT=0), for H, q and t."""
    from chmy_gb300.configs import sia_ensemble

    ens = sia_ensemble(members=7, nmin=33, nmax=150, seed=5, dtype=T)
    nsteps = 40
    rng = np.random.default_rng(2)
    start = []
    for grid, h, p in ens:
        H0 = NpField(grid, Center(), T)
        H0.interior()[...] = (rng.random(H0.dims) * 0.3).astype(T)
        B = NpField(grid, Center(), T)
        B.a[...] = h["B"].astype(T)
        start.append((grid, H0, B, p))

    def run(persistent):
        monkeypatch.setenv("CG_SIA_PERSISTENT", "1" if persistent else "0")
        mem = (_abi.cg_sia_member * len(start))()
        params = (_abi.cg_sia_params * len(start))()
        keep = []
        for k, (grid, H0, B, p) in enumerate(start):
            Hg, Bg = to_gpu(arch, H0), to_gpu(arch, B)
            qg = [to_gpu(arch, NpField(grid, (Vertex(), Center()), T)), to_gpu(arch, NpField(grid, (Center(), Vertex()), T))]
            keep.append((Hg, qg, Bg))
            mem[k].grid = grid.desc()
            mem[k].H, mem[k].B = Hg.desc(), Bg.desc()
            mem[k].q[0], mem[k].q[1] = qg[0].desc(), qg[1].desc()
            params[k] = p
        ts = (ctypes.c_double * len(start))()
        arch.call("cg_sia_ensemble_run", len(start), mem, params, nsteps, ts)
        arch.synchronize()
        return [(Hg.to_numpy(), qg[0].to_numpy(), qg[1].to_numpy()) for Hg, qg, _ in keep], list(ts)

    (fa, ta), (fb, tb) = run(True), run(False)
    assert ta == tb
    for k, (a, b) in enumerate(zip(fa, fb)):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y, err_msg=f"member {k}")


def test_ensemble_persistent_barrier_wait_runs_out(arch, monkeypatch):
    """Failure detection of the persistent launch's grid barriers, without a GPU fault: the host
    makes every barrier expect one arrival more than the grid has blocks (an arrival that never
    comes) and sets a 20 ms limit on each wait. Every block's wait runs out, the kernel returns,
    and the call reports CG_ERR_TIMEOUT. The context stays usable: the same run without the
    withheld arrival then matches the per-phase launches bit for bit."""
    import time

    from chmy_gb300.configs import sia_ensemble

    T = np.float64
    ens = sia_ensemble(members=3, nmin=40, nmax=80, seed=9, dtype=T)
    nsteps = 5
    rng = np.random.default_rng(4)
    start = []
    for grid, h, p in ens:
        H0 = NpField(grid, Center(), T)
        H0.interior()[...] = rng.random(H0.dims) * 0.3
        B = NpField(grid, Center(), T)
        B.a[...] = h["B"]
        start.append((grid, H0, B, p))

    def run():
        mem = (_abi.cg_sia_member * len(start))()
        params = (_abi.cg_sia_params * len(start))()
        keep = []
        for k, (grid, H0, B, p) in enumerate(start):
            Hg, Bg = to_gpu(arch, H0), to_gpu(arch, B)
            qg = [to_gpu(arch, NpField(grid, (Vertex(), Center()), T)), to_gpu(arch, NpField(grid, (Center(), Vertex()), T))]
            keep.append((Hg, qg, Bg))
            mem[k].grid = grid.desc()
            mem[k].H, mem[k].B = Hg.desc(), Bg.desc()
            mem[k].q[0], mem[k].q[1] = qg[0].desc(), qg[1].desc()
            params[k] = p
        ts = (ctypes.c_double * len(start))()
        rc = arch.lib.cg_sia_ensemble_run(arch.ctx, len(start), mem, params, nsteps, ts)
        arch.synchronize()
        return rc, [Hg.to_numpy() for Hg, _, _ in keep]

    monkeypatch.setenv("CG_SIA_PERSISTENT", "1")
    monkeypatch.setenv("CG_SIA_BARRIER_LIMIT_MS", "20")
    monkeypatch.setenv("CG_SIA_BARRIER_WITHHELD", "1")
    t0 = time.perf_counter()
    rc, _ = run()
    waited = time.perf_counter() - t0
    assert rc == _abi.CG_ERR_TIMEOUT, (rc, arch.lib.cg_last_error(arch.ctx))
    assert b"timed out" in arch.lib.cg_last_error(arch.ctx)
    assert waited < 1.5, waited  # the 20 ms limit applied, not the 2 s default
    monkeypatch.delenv("CG_SIA_BARRIER_WITHHELD")
    monkeypatch.delenv("CG_SIA_BARRIER_LIMIT_MS")
    rc, Hp = run()
    assert rc == _abi.CG_OK, arch.lib.cg_last_error(arch.ctx)
    monkeypatch.setenv("CG_SIA_PERSISTENT", "0")
    rc, Hg = run()
    assert rc == _abi.CG_OK
    for a, b in zip(Hp, Hg):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("T", TYPES)
def test_ensemble_tile_heights_give_the_same_bits(arch, monkeypatch, T):
    """The ensemble's tile height (rows of its 32-point tiles: 4, 8 or 16, CG_SIA_TILE_ROWS) is an
    autotuned launch choice: H, q and every member's time are the same bits under each height, and
    under the autotuner's choice, for 9 members of uneven sizes."""
    from chmy_gb300.configs import sia_ensemble

    ens = sia_ensemble(members=9, nmin=20, nmax=140, seed=12, dtype=T)
    nsteps = 25
    rng = np.random.default_rng(8)
    start = []
    for grid, h, p in ens:
        H0 = NpField(grid, Center(), T)
        H0.interior()[...] = (rng.random(H0.dims) * 0.3).astype(T)
        B = NpField(grid, Center(), T)
        B.a[...] = h["B"].astype(T)
        start.append((grid, H0, B, p))

    def run():
        mem = (_abi.cg_sia_member * len(start))()
        params = (_abi.cg_sia_params * len(start))()
        keep = []
        for k, (grid, H0, B, p) in enumerate(start):
            Hg, Bg = to_gpu(arch, H0), to_gpu(arch, B)
            qg = [to_gpu(arch, NpField(grid, (Vertex(), Center()), T)), to_gpu(arch, NpField(grid, (Center(), Vertex()), T))]
            keep.append((Hg, qg, Bg))
            mem[k].grid = grid.desc()
            mem[k].H, mem[k].B = Hg.desc(), Bg.desc()
            mem[k].q[0], mem[k].q[1] = qg[0].desc(), qg[1].desc()
            params[k] = p
        ts = (ctypes.c_double * len(start))()
        arch.call("cg_sia_ensemble_run", len(start), mem, params, nsteps, ts)
        arch.synchronize()
        return [(Hg.to_numpy(), qg[0].to_numpy(), qg[1].to_numpy()) for Hg, qg, _ in keep], list(ts)

    monkeypatch.setenv("CG_SIA_PERSISTENT", "0")
    results = []
    for rows in ("4", "8", "16", None):
        if rows is None:
            monkeypatch.delenv("CG_SIA_TILE_ROWS", raising=False)
        else:
            monkeypatch.setenv("CG_SIA_TILE_ROWS", rows)
        results.append(run())
    fa, ta = results[0]
    for fb, tb in results[1:]:
        assert ta == tb
        for k, (a, b) in enumerate(zip(fa, fb)):
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y, err_msg=f"member {k}")
