"""GPU parity: fused boundary conditions, max-norm reduction and explicit diffusion against the
CPU oracle, through the C ABI."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, desc_array, lib, vec_fields
from chmy_gb300 import _abi
from chmy_gb300.bcs import Dirichlet, Neumann, Periodic, to_cg_bc
from chmy_gb300.grids import Center, UniformGrid, Vertex
from gpu_helpers import assert_close, random_field, to_gpu

pytestmark = pytest.mark.gpu
TYPES = [np.float32, np.float64]
C_, V_ = Center(), Vertex()


def _grid(dims, T):
    nd = len(dims)
    return UniformGrid(origin=(T(-1),) * nd, extent=(T(2),) * nd, dims=dims, dtype=T)


def _rand_spec(rng, nd, allow_periodic=True):
    spec = {}
    kinds = [Dirichlet, Neumann, None] + ([Periodic] if allow_periodic else [])
    for d in range(nd):
        k = kinds[rng.integers(len(kinds))]
        if k is Periodic:
            spec["xyz"[d]] = Periodic()
        elif k is None:
            continue
        else:
            spec["xyz"[d]] = (
                k(float(rng.uniform(-2, 2))) if rng.random() < 0.5 else k(),
                [Dirichlet, Neumann][rng.integers(2)](float(rng.uniform(-2, 2))),
            )
    return spec


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(9,), (7, 6), (11, 5, 4), (5, 8, 6)])
def test_bc_batch_matches_oracle_bitwise(arch, T, dims):
    rng = np.random.default_rng(len(dims) * 100 + dims[0])
    grid = _grid(dims, T)
    nd = len(dims)
    for trial in range(6):
        fields, specs = [], []
        for _ in range(3):
            loc = tuple(V_ if rng.random() < 0.5 else C_ for _ in range(nd))
            fields.append(random_field(grid, loc, T, rng))
            specs.append(_rand_spec(rng, nd))
        gpu = [to_gpu(arch, f) for f in fields]
        bcs = [to_cg_bc(nd, s) for s in specs]
        bc_apply(grid, fields, bcs)
        g = grid.desc()
        arch.call("cg_bc_apply", ctypes.byref(g), len(gpu), desc_array(gpu), (_abi.cg_bc * len(bcs))(*bcs))
        arch.synchronize()
        for i, (a, b) in enumerate(zip(gpu, fields)):
            assert_close(a, b, 0, f"trial {trial} field {i} {specs[i]}", exact=True)


@pytest.mark.parametrize("T", TYPES)
def test_bc_pitched_layout(arch, T):
    """Same results on a pitched (row-aligned) allocation."""
    rng = np.random.default_rng(7)
    grid = _grid((13, 9), T)
    f = random_field(grid, (V_, C_), T, rng)
    g = to_gpu(arch, f, pitch_align=128)
    assert g.data.stride(0) != g.data.shape[1]
    spec = {"x": Dirichlet(0.5), "y": Neumann(-1.0)}
    bc_apply(grid, [f], [to_cg_bc(2, spec)])
    from chmy_gb300 import bc_

    bc_(arch, grid, (g, spec))
    arch.synchronize()
    assert_close(g, f, 0, "pitched", exact=True)


@pytest.mark.parametrize("T", TYPES)
def test_maxabs(arch, T):
    rng = np.random.default_rng(3)
    grid = _grid((37, 21, 9), T)
    fs = [random_field(grid, (V_, C_, C_), T, rng), random_field(grid, C_, T, rng, scale=3.0)]
    # poison the halo: it must not enter the interior max
    fs[1].a[0, 0, 0] = 1e6
    gs = [to_gpu(arch, f) for f in fs]
    out = (ctypes.c_double * 2)()
    bad = ctypes.c_int32(7)
    arch.call("cg_maxabs", 2, desc_array(gs), out, ctypes.byref(bad))
    for i, f in enumerate(fs):
        assert out[i] == float(np.max(np.abs(f.interior())))
    assert bad.value == 0
    fs[0].interior()[3, 2, 1] = np.nan
    gs[0].from_numpy(fs[0].a)
    arch.call("cg_maxabs", 2, desc_array(gs), out, ctypes.byref(bad))
    assert bad.value == 1 and np.isnan(out[0])


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(30,), (33, 17), (19, 12, 9)])
def test_diffusion_kernels(arch, T, dims):
    """compute_q! and update_C! (examples/diffusion_2d.jl:8-19) equal the oracle bit for bit."""
    rng = np.random.default_rng(11)
    grid = _grid(dims, T)
    nd = len(dims)
    Cf = random_field(grid, C_, T, rng)
    q = vec_fields(grid, T)
    Cg = to_gpu(arch, Cf)
    qg = [to_gpu(arch, f) for f in q]
    g = grid.desc()
    chi, dt = 1.0, 1e-3
    assert lib().or_diffusion_compute_q(ctypes.byref(g), desc_array(q, 3), ctypes.byref(Cf.desc()), chi) == 0
    arch.call("cg_diffusion_compute_q", ctypes.byref(g), desc_array(qg, 3), ctypes.byref(Cg.desc()), chi)
    arch.synchronize()
    for a, b in zip(qg, q):
        assert_close(a, b, 0.0, "q", exact=True)
    assert lib().or_diffusion_update_C(ctypes.byref(g), ctypes.byref(Cf.desc()), desc_array(q, 3), dt) == 0
    arch.call("cg_diffusion_update_C", ctypes.byref(g), ctypes.byref(Cg.desc()), desc_array(qg, 3), dt)
    arch.synchronize()
    assert_close(Cg, Cf, 0.0, "C", exact=True)


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(300,), (64, 48), (100, 37), (21, 18, 15), (70, 9, 13)])
def test_diffusion_fused_steps(arch, T, dims):
    """cg_diffusion_run (fused step + bc!, graph-replayed) == oracle compute_q!/update_C!/bc!
    with fresh q arrays, over several steps, bit for bit: the fused step computes the flux form
    with the oracle's rounding (grids whose rows end inside a warp and inside a block)."""
    rng = np.random.default_rng(5)
    grid = _grid(dims, T)
    nd = len(dims)
    Cf = NpField(grid, C_, T)
    Cf.interior()[...] = rng.random(Cf.dims).astype(T)
    spec = {"x": Dirichlet(0.25), "y": Neumann()} if nd == 2 else Neumann()
    bc = to_cg_bc(nd, spec)
    bc_apply(grid, [Cf], [bc])
    A = to_gpu(arch, Cf)
    B = to_gpu(arch, Cf)
    dx = min(grid.spacing())
    chi = 1.0
    dt = float(dx * dx / chi / 4.1 / nd)
    nsteps = 10
    g = grid.desc()
    for _ in range(nsteps):
        q = vec_fields(grid, T)
        lib().or_diffusion_compute_q(ctypes.byref(g), desc_array(q, 3), ctypes.byref(Cf.desc()), chi)
        lib().or_diffusion_update_C(ctypes.byref(g), ctypes.byref(Cf.desc()), desc_array(q, 3), dt)
        bc_apply(grid, [Cf], [bc])
    arch.call("cg_diffusion_run", ctypes.byref(g), ctypes.byref(A.desc()), ctypes.byref(B.desc()), chi, dt, ctypes.byref(bc), nsteps)
    arch.synchronize()
    res = A if nsteps % 2 == 0 else B
    assert_close(res, Cf, 0.0, "C after steps", exact=True)


def test_argument_errors(arch):
    """Mismatched locations and aliasing are rejected with CG_ERR_ARG, no launch."""
    grid = _grid((8, 8), np.float64)
    Cf = NpField(grid, V_)  # wrong location for C
    Cg = to_gpu(arch, Cf)
    g = grid.desc()
    rc = arch.lib.cg_diffusion_step(arch.ctx, ctypes.byref(g), ctypes.byref(Cg.desc()), ctypes.byref(Cg.desc()), 1.0, 1e-3, None)
    assert rc == _abi.CG_ERR_ARG
    assert b"location" in arch.lib.cg_last_error(arch.ctx)
    C2 = to_gpu(arch, NpField(grid, C_))
    rc = arch.lib.cg_diffusion_step(arch.ctx, ctypes.byref(g), ctypes.byref(C2.desc()), ctypes.byref(C2.desc()), 1.0, 1e-3, None)
    assert rc == _abi.CG_ERR_ARG


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(7, 6), (11, 5, 4)])
def test_bc_per_point_values_bitwise(arch, T, dims):
    """Per-point condition values (BoundaryFunctions, arrays) in one batch on the GPU equal the
    oracle's bit for bit; the arrays live on the device (cg_bc.values)."""
    from chmy_gb300 import bc_
    from chmy_gb300.bcs import BoundaryFunction, materialize_bc

    rng = np.random.default_rng(11)
    grid = _grid(dims, T)
    nd = len(dims)
    fx = BoundaryFunction(lambda *c: 0.5 + sum(ci * ci for ci in c))
    fields, specs = [], []
    for loc in [tuple(V_ if d == e else C_ for e in range(nd)) for d in range(nd)] + [C_]:
        spec = {}
        for d in range(nd):
            shape = tuple(grid.dims[t] + 3 for t in reversed([t for t in range(nd) if t != d]))
            arr = rng.standard_normal(shape).astype(T)
            spec["xyz"[d]] = (Dirichlet(fx), Neumann(arr)) if d % 2 == 0 else (Neumann(fx), Dirichlet(arr))
        fields.append(random_field(grid, loc, T, rng))
        specs.append(spec)
    gpu = [to_gpu(arch, f) for f in fields]
    host = [materialize_bc(grid, f.loc, T, s) for f, s in zip(fields, specs)]
    bc_apply(grid, fields, [b for b, _ in host])
    bc_(arch, grid, *[(g, s) for g, s in zip(gpu, specs)])
    arch.synchronize()
    for i, (a, b) in enumerate(zip(gpu, fields)):
        assert_close(a, b, 0, f"field {i}", exact=True)


def test_gather_interior_and_dump(arch, tmp_path):
    """gather! on one GPU: the interior of a (pitched) field as a host array, x fastest, and
    the same bytes as a headless dump."""
    from chmy_gb300 import gather

    rng = np.random.default_rng(2)
    grid = _grid((7, 5, 4), np.float64)
    f = random_field(grid, (V_, C_, C_), np.float64, rng)
    g = to_gpu(arch, f, pitch_align=128)
    path = tmp_path / "interior.bin"
    a = gather(g, path=str(path))
    ref = f.interior().transpose(2, 1, 0)  # [x, y, z] view -> stored [z, y, x]
    assert np.array_equal(a, ref)
    assert np.array_equal(np.fromfile(path, dtype=np.float64), np.ascontiguousarray(ref).ravel())
    dst = np.empty_like(a)
    gather(g, dst)
    assert np.array_equal(dst, a)


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(33, 21), (17, 12, 9)])
def test_masked_diffusion_matches_oracle(arch, T, dims):
    """Masked explicit diffusion (q.d = -chi ∂d(C, ω), C -= dt divg(q, ω)): the per-launch
    kernels and the graph-replayed fused steps equal the oracle's masked operators bit for bit."""
    from chmy_gb300.fields import FieldMask

    rng = np.random.default_rng(6)
    grid = _grid(dims, T)
    nd = len(dims)
    g = grid.desc()
    mask = FieldMask(arch, grid, T)
    host = {}
    hm = _abi.cg_mask()
    for bits, f in mask.fields.items():
        h = NpField(grid, f.loc, T)
        h.a[...] = rng.random(h.a.shape).astype(T)
        f.from_numpy(h.a)
        host[bits] = h
        hm.at[bits] = h.desc()
    dm = mask.desc()
    Cf = NpField(grid, C_, T)
    Cf.interior()[...] = rng.random(Cf.dims).astype(T)
    chi = 1.0
    dx = min(grid.spacing())
    dt = float(dx * dx / chi / 4.1 / nd)
    # per launch
    Cg = to_gpu(arch, Cf)
    qh, qg = vec_fields(grid, T), [to_gpu(arch, f) for f in vec_fields(grid, T)]
    assert lib().or_diffusion_compute_q_masked(ctypes.byref(g), desc_array(qh, 3), ctypes.byref(Cf.desc()), chi, ctypes.byref(hm)) == 0
    arch.call("cg_diffusion_compute_q_masked", ctypes.byref(g), desc_array(qg, 3), ctypes.byref(Cg.desc()), chi, ctypes.byref(dm))
    arch.synchronize()
    for a, b in zip(qg, qh):
        assert_close(a, b, 0.0, "masked q", exact=True)
    C1 = Cf.copy()
    assert lib().or_diffusion_update_C_masked(ctypes.byref(g), ctypes.byref(C1.desc()), desc_array(qh, 3), dt, ctypes.byref(hm)) == 0
    arch.call("cg_diffusion_update_C_masked", ctypes.byref(g), ctypes.byref(Cg.desc()), desc_array(qg, 3), dt, ctypes.byref(dm))
    arch.synchronize()
    assert_close(Cg, C1, 0.0, "masked C", exact=True)
    # fused steps with bc!, graph-replayed
    spec = {"x": Dirichlet(0.25), "y": Neumann()} if nd == 2 else Neumann()
    bc = to_cg_bc(nd, spec)
    bc_apply(grid, [Cf], [bc])
    A, B = to_gpu(arch, Cf), to_gpu(arch, Cf)
    nsteps = 8
    for _ in range(nsteps):
        q = vec_fields(grid, T)
        lib().or_diffusion_compute_q_masked(ctypes.byref(g), desc_array(q, 3), ctypes.byref(Cf.desc()), chi, ctypes.byref(hm))
        lib().or_diffusion_update_C_masked(ctypes.byref(g), ctypes.byref(Cf.desc()), desc_array(q, 3), dt, ctypes.byref(hm))
        bc_apply(grid, [Cf], [bc])
    arch.call("cg_diffusion_run_masked", ctypes.byref(g), ctypes.byref(A.desc()), ctypes.byref(B.desc()), chi, dt,
              ctypes.byref(bc), ctypes.byref(dm), nsteps)
    arch.synchronize()
    assert_close(A, Cf, 0.0, "masked steps", exact=True)
