"""The block-shape autotuner of the per-point kernels (explicit diffusion step, update_stress! and
update_velocity! in the PT loops, update_q! and update_C! of PT diffusion): every candidate
shape, forced with CG_BLOCK=<x>x<y>, gives the bits of the default 32 x 8 shape, since each
thread computes one point whatever the shape."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField
from chmy_gb300 import _abi
from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
from chmy_gb300.grids import Center, UniformGrid
from gpu_helpers import to_gpu
from test_gpu_stokes import StokesSet, _bc_V, pt_params

pytestmark = pytest.mark.gpu
SHAPES = ["32x4", "64x4", "128x2", "32x16", "64x8", "128x4"]


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("T", [np.float32, np.float64])
@pytest.mark.parametrize("dims", [(45, 37), (19, 13, 11)])
def test_diffusion_run_block_shapes(arch, monkeypatch, T, dims):
    nd = len(dims)
    grid = UniformGrid(origin=(T(-1),) * nd, extent=(T(2),) * nd, dims=dims, dtype=T)
    rng = np.random.default_rng(4)
    C0 = NpField(grid, Center(), T)
    C0.a[...] = rng.random(C0.a.shape).astype(T)
    spec = {"x": Neumann(0.1), "y": Dirichlet(0.3)}
    if nd == 3:
        spec["z"] = Neumann()
    bc = to_cg_bc(nd, spec)
    dt = float(min(grid.spacing())) ** 2 / (4.1 * nd)

    def run():
        A, B = to_gpu(arch, C0), to_gpu(arch, C0)
        arch.call("cg_diffusion_run", ctypes.byref(grid.desc()), ctypes.byref(A.desc()), ctypes.byref(B.desc()), 1.0, dt,
                  ctypes.byref(bc), 10)
        arch.synchronize()
        return A.to_numpy(), B.to_numpy()

    monkeypatch.setenv("CG_BLOCK", "32x8")
    ref = run()
    for shape in SHAPES:
        monkeypatch.setenv("CG_BLOCK", shape)
        got = run()
        assert _bits_equal(got[0], ref[0]) and _bits_equal(got[1], ref[1]), shape


@pytest.mark.parametrize("T", [np.float32, np.float64])
@pytest.mark.parametrize("dims", [(37, 29), (13, 12, 11)])
def test_stokes_pt_iterations_block_shapes(arch, monkeypatch, T, dims):
    def run():
        s = StokesSet(arch, dims, T, 43, True)
        p = pt_params(s.grid, True)
        barr = (_abi.cg_bc * 3)(*_bc_V(len(dims)))
        d = s.dev_desc()
        arch.call("cg_stokes_pt_iterations", ctypes.byref(s.grid.desc()), ctypes.byref(d), ctypes.byref(p), barr, 5)
        arch.synchronize()
        return [f.to_numpy() for _, f, _ in s.pairs()]

    monkeypatch.setenv("CG_BLOCK", "32x8")
    ref = run()
    for shape in SHAPES:
        monkeypatch.setenv("CG_BLOCK", shape)
        for a, b in zip(run(), ref):
            assert _bits_equal(a, b), shape


@pytest.mark.parametrize("dims", [(41, 35), (14, 12, 10)])
def test_ptdiff_run_block_shapes(arch, monkeypatch, dims):
    from chmy_gb300.configs import ptdiff_params
    from chmy_gb300.grids import Vertex

    T = np.float64
    nd = len(dims)
    grid = UniformGrid(origin=(-0.5,) * nd, extent=(1.0,) * nd, dims=dims, dtype=T)
    rng = np.random.default_rng(9)
    C0 = NpField(grid, Center(), T)
    C0.a[...] = rng.random(C0.a.shape)
    D = NpField(grid, Center(), T)
    D.a[...] = np.exp(rng.uniform(-1, 1, D.a.shape))
    p = ptdiff_params(grid, 1e-3, float(D.a.max()))
    bc = to_cg_bc(nd, {"x": Dirichlet(0.0), "y": Neumann()} if nd == 2 else {"x": Dirichlet(0.0), "y": Neumann(), "z": Neumann()})

    def run():
        C, Co, Dg = to_gpu(arch, C0), to_gpu(arch, C0), to_gpu(arch, D)
        locs = [tuple(Vertex() if e == d else Center() for e in range(nd)) for d in range(nd)]
        q = [to_gpu(arch, NpField(grid, l, T)) for l in locs]
        f = _abi.cg_ptdiff_fields()
        f.C, f.C_old, f.D = C.desc(), Co.desc(), Dg.desc()
        for d in range(nd):
            f.q[d] = q[d].desc()
        arch.call("cg_ptdiff_run", ctypes.byref(grid.desc()), ctypes.byref(f), ctypes.byref(p), ctypes.byref(bc), 2, 7)
        arch.synchronize()
        return [C.to_numpy()] + [x.to_numpy() for x in q]

    monkeypatch.setenv("CG_BLOCK", "32x8")
    ref = run()
    for shape in SHAPES:
        monkeypatch.setenv("CG_BLOCK", shape)
        for a, b in zip(run(), ref):
            assert _bits_equal(a, b), shape
