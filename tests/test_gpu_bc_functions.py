"""BoundaryFunction values evaluated on the device (cg_bc_apply_fn; src/BoundaryConditions/
boundary_function.jl:11-44 with first_order_boundary_condition.jl:46-84) against the oracle's
batch with the same values materialised: the function evaluated by the oracle at the points the
condition writes (its location rule, reduced or full dimensions), bit for bit."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, lib
from chmy_gb300 import _abi
from chmy_gb300.bcs import BoundaryFunction, Dirichlet, Neumann, bc_
from chmy_gb300.functions import FunctionField, affine, ball, constant
from chmy_gb300.grids import Center, UniformGrid, Vertex
from gpu_helpers import to_gpu

pytestmark = pytest.mark.gpu


def _params(form, nargs, rng):
    if form is constant:
        return (float(rng.normal()),)
    if form is ball:
        return tuple(rng.uniform(-0.3, 0.3, nargs)) + (0.4, 1.5, -0.5)
    return tuple(rng.normal(size=nargs + 1))


def _oracle_plane(grid, loc, T, d, side, kind, form, params, reduce_dims):
    """The per-point values (tangential logical indices 0..n_t+2, [z, y, x] order without d)
    the oracle's evaluation of the form gives at the points the condition writes."""
    nd = grid.ndim
    vtx_d = isinstance(loc[d], Vertex)
    L = (Vertex() if vtx_d else Center()) if kind == "dirichlet" else (Center() if vtx_d else Vertex())
    ext = grid.dims[d] + (1 if vtx_d else 0)
    gi = (1 if side == 0 else ext) if (kind == "dirichlet" and vtx_d) else (0 if side == 0 else ext + 1)
    tdims = [t for t in range(nd) if t != d]
    if reduce_dims:
        sub = UniformGrid(origin=tuple(grid.axes[t].origin for t in tdims), extent=tuple(grid.axes[t].extent for t in tdims),
                          dims=tuple(grid.dims[t] for t in tdims), dtype=T)
        ff = FunctionField(form, sub, (L,) * (nd - 1), parameters=params)
        out = NpField(sub, (L,) * (nd - 1), T)
        assert lib().or_function_fill(ctypes.byref(sub.desc()), ctypes.byref(ff.desc()), ctypes.byref(out.desc())) == 0
        sl = tuple(slice(1, 1 + grid.dims[t] + 3) for t in reversed(tdims))
        return np.ascontiguousarray(out.a[sl])
    ff = FunctionField(form, grid, (L,) * nd, parameters=params)
    out = NpField(grid, (L,) * nd, T)
    assert lib().or_function_fill(ctypes.byref(grid.desc()), ctypes.byref(ff.desc()), ctypes.byref(out.desc())) == 0
    sl = []
    for t in reversed(range(nd)):
        sl.append(gi + 1 if t == d else slice(1, 1 + grid.dims[t] + 3))
    return np.ascontiguousarray(out.a[tuple(sl)])


CASES = [(form, kind, red) for form in (affine, ball, constant) for kind in ("dirichlet", "neumann") for red in (True, False)]


@pytest.mark.parametrize("T", [np.float64, np.float32])
@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("form,kind,reduce_dims", CASES, ids=lambda v: getattr(v, "__name__", str(v)))
def test_device_boundary_functions_match_oracle(arch, T, nd, form, kind, reduce_dims):
    """Every side of a Center field and of a Vertex-in-x field carries the function (both sides
    of every dimension, so edges and corners chain through the rules): the device evaluation
    equals the oracle's batch with the values the oracle computes, bit for bit."""
    dims = (13, 9) if nd == 2 else (9, 7, 6)
    grid = UniformGrid(origin=tuple(-0.6 + 0.1 * t for t in range(nd)), extent=(1.3,) * nd, dims=dims, dtype=T)
    rng = np.random.default_rng(11 + nd)
    nargs = nd - 1 if reduce_dims else nd
    params = _params(form, nargs, rng)
    Rule = Dirichlet if kind == "dirichlet" else Neumann
    bf = BoundaryFunction(form, parameters=params, reduce_dims=reduce_dims)
    for loc in ((Center(),) * nd, (Vertex(),) + (Center(),) * (nd - 1)):
        host = NpField(grid, loc, T)
        host.a[...] = rng.standard_normal(host.a.shape).astype(T)
        dev = to_gpu(arch, host)
        spec = {"xyz"[d]: Rule(bf) for d in range(nd)}
        bc_(arch, grid, (dev, spec))
        arch.synchronize()
        b = _abi.cg_bc()
        keep = []
        for d in range(nd):
            for s in range(2):
                b.kind[d][s] = _abi.CG_BC_DIRICHLET if kind == "dirichlet" else _abi.CG_BC_NEUMANN
                arr = _oracle_plane(grid, loc, T, d, s, kind, form, params, reduce_dims)
                keep.append(arr)
                b.values[d][s] = arr.ctypes.data
        bc_apply(grid, [host], [b])
        got = dev.to_numpy()
        assert np.array_equal(got.view(np.uint8), host.a.view(np.uint8)), (loc, np.max(np.abs(got - host.a)))


def test_device_and_host_boundary_functions_agree(arch):
    """The device path and the host path (the same function given as a Python callable, so
    that the batch evaluates it on the host) agree to rounding: the host computes coordinates
    without fused multiply-adds."""
    T = np.float64
    grid = UniformGrid(origin=(0.0, 0.0), extent=(2.0, 2.0), dims=(16, 12), dtype=T)
    host = NpField(grid, (Center(), Center()), T)
    host.a[...] = np.random.default_rng(2).standard_normal(host.a.shape)
    a, b = to_gpu(arch, host), to_gpu(arch, host)
    dev_fn = BoundaryFunction(affine, parameters=(0.5, 2.0))
    host_fn = BoundaryFunction(lambda y, a0, a1: a0 + a1 * y, parameters=(0.5, 2.0))
    bc_(arch, grid, (a, {"x": Dirichlet(dev_fn), "y": Neumann()}))
    bc_(arch, grid, (b, {"x": Dirichlet(host_fn), "y": Neumann()}))
    arch.synchronize()
    np.testing.assert_allclose(a.to_numpy(), b.to_numpy(), rtol=1e-13, atol=1e-13)


def test_bc_apply_fn_rejects_bad_functions(arch):
    T = np.float64
    grid = UniformGrid(origin=(0.0, 0.0), extent=(1.0, 1.0), dims=(8, 8), dtype=T)
    f = to_gpu(arch, NpField(grid, (Center(), Center()), T))
    fa = (_abi.cg_field * 1)(f.desc())
    b = (_abi.cg_bc * 1)()
    b[0].kind[0][0] = _abi.CG_BC_PERIODIC
    b[0].kind[0][1] = _abi.CG_BC_PERIODIC
    fn = (_abi.cg_bc_fn * 1)()
    fn[0].fn[0][0].kind = _abi.CG_FN_AFFINE
    L = arch.lib
    assert L.cg_bc_apply_fn(arch.ctx, ctypes.byref(grid.desc()), 1, fa, b, fn) == _abi.CG_ERR_ARG  # periodic side
    b[0].kind[0][0] = b[0].kind[0][1] = _abi.CG_BC_DIRICHLET
    fn[0].fn[0][0].kind = 7
    assert L.cg_bc_apply_fn(arch.ctx, ctypes.byref(grid.desc()), 1, fa, b, fn) == _abi.CG_ERR_ARG  # unknown kind
    fn[0].fn[0][0].kind = _abi.CG_FN_NONE
    fn[0].fn[2][0].kind = _abi.CG_FN_CONST
    assert L.cg_bc_apply_fn(arch.ctx, ctypes.byref(grid.desc()), 1, fa, b, fn) == _abi.CG_ERR_ARG  # dim beyond the grid
    fn[0].fn[2][0].kind = _abi.CG_FN_NONE
    assert L.cg_bc_apply_fn(arch.ctx, ctypes.byref(grid.desc()), 1, fa, b, fn) == _abi.CG_OK
    arch.synchronize()
