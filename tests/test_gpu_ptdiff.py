"""GPU parity of the PT variable-coefficient diffusion kernels against the oracle."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, desc_array, lib
from chmy_gb300 import _abi
from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
from chmy_gb300.configs import ptdiff_params
from chmy_gb300.grids import Center, UniformGrid, Vertex
from gpu_helpers import assert_close, random_field, rtol_for, to_gpu

pytestmark = pytest.mark.gpu
TYPES = [np.float32, np.float64]
C_, V_ = Center(), Vertex()


def fields(arch, dims, T, seed):
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
    d = {k: ([to_gpu(arch, f) for f in v] if isinstance(v, list) else to_gpu(arch, v)) for k, v in h.items()}
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
