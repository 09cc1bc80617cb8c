"""Device FunctionFields (src/Fields/function_field.jl:49-59): the body force of the VE Stokes
kernels evaluated in the kernel from a cg_function, as the examples' FunctionField(init_incl, grid,
(Center(), Vertex()); parameters) (examples/stokes_2d_inc_ve_T.jl:106-107), against the same
values materialised in an array."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, lib
from chmy_gb300 import _abi
from chmy_gb300.configs import stokes2d_inclusions, stokes3d_grf
from chmy_gb300.functions import FunctionField, affine, ball, constant
from chmy_gb300.grids import Center, UniformGrid, Vertex
from chmy_gb300.solvers import StokesSolver
from gpu_helpers import to_gpu

pytestmark = pytest.mark.gpu


def _cases(nd):
    if nd == 2:
        return [(ball, dict(x0=0.1, y0=-0.05, r=0.2, in_=1.5, out=-0.25)), (affine, (0.5, 2.0, -1.0)), (constant, (3.0,))]
    return [(ball, dict(x0=0.0, y0=0.1, z0=-0.1, r=0.25, in_=1.0, out=0.0)), (affine, (0.5, 2.0, -1.0, 0.25)), (constant, (-2.0,))]


@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_function_fill_matches_oracle(arch, nd, T):
    """cg_function_fill (set!(f, grid, func) on the device) equals the oracle's evaluation of the
    same FunctionField at every padded point, bit for bit, at Center, Vertex and mixed locations."""
    dims = (20, 17) if nd == 2 else (12, 10, 9)
    grid = UniformGrid(origin=(-0.5,) * nd, extent=(1.0,) * nd, dims=dims, dtype=T)
    locs = [(Center(),) * nd, (Vertex(),) * nd, tuple(Vertex() if d == nd - 1 else Center() for d in range(nd))]
    for func, params in _cases(nd):
        for loc in locs:
            ff = FunctionField(func, grid, loc, parameters=params)
            fn = ff.desc()
            ref = NpField(grid, loc, T)
            assert lib().or_function_fill(ctypes.byref(grid.desc()), ctypes.byref(fn), ctypes.byref(ref.desc())) == 0
            dev = to_gpu(arch, NpField(grid, loc, T))
            arch.call("cg_function_fill", ctypes.byref(grid.desc()), ctypes.byref(fn), ctypes.byref(dev.desc()))
            np.testing.assert_array_equal(dev.to_numpy(), ref.a, err_msg=f"{func.__name__} {loc}")


def _example_problem(n, T=np.float64):
    """examples/stokes_2d_inc_ve_T.jl:62-107: scalar eta, buoyant disc rhogy as a FunctionField."""
    import math

    from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
    from chmy_gb300.configs import StokesProblem, padded_mesh
    from chmy_gb300.kernels import stokes_params

    lx = ly = 2.0
    eta, G, dt = 10.0, 1.0, 1e-2
    grid = UniformGrid(origin=(-lx / 2, -ly / 2), extent=(lx, ly), dims=(n, n), dtype=T)
    C_, V_ = Center(), Vertex()

    def z(loc):
        return np.zeros_like(padded_mesh(grid, loc)[0], dtype=T)

    tl = [(C_, C_), (C_, C_), (V_, V_)]
    host = {"V": [z((V_, C_)), z((C_, V_))], "r_V": [z((V_, C_)), z((C_, V_))], "P": z(C_), "divV": z(C_),
            "tau": [z(l) for l in tl], "tau_old": [z(l) for l in tl]}
    rhogy = FunctionField(ball, grid, (C_, V_), parameters=dict(x0=0.0, y0=0.0, r=0.1 * lx, in_=1.0, out=0.0))
    dx = float(grid.spacing()[0])
    re_m, r = 2.3 * math.pi, 0.5
    lt = min(lx, ly) / re_m
    vdt = dx / math.sqrt(2 * 1.1)
    th = lt * (r + 4.0 / 3.0) / vdt
    params = stokes_params(eta=eta, eta_ve=1.0 / (1.0 / eta + 1.0 / (G * dt)), G=G, dt=dt, dtau_Pr=r / th,
                           dtau_r=1.0 / (th + 1.0), nu_dtau=vdt * lt)
    bc_V = [to_cg_bc(2, {"x": Dirichlet(), "y": Neumann()}), to_cg_bc(2, {"x": Neumann(), "y": Dirichlet()})]
    pb = StokesProblem(grid=grid, host=host, params=params, bc_V=bc_V, eps=1e-8, tau_scale=eta / G, v_scale=ly / G,
                       ncheck=2 * n, max_iter=50 * n)
    return pb, rhogy


def _oracle_values(ff):
    """The FunctionField at every padded point, by the oracle's evaluation (coordinates by
    fused multiply-adds, like Chmy's muladd and the device)."""
    ref = NpField(ff.grid, ff.loc)
    assert lib().or_function_fill(ctypes.byref(ff.grid.desc()), ctypes.byref(ff.desc()), ctypes.byref(ref.desc())) == 0
    return ref.a


def _with_array(pb, ff):
    import dataclasses

    host = dict(pb.host)
    nd = pb.grid.ndim
    rho = [None] * nd
    rho[nd - 1] = _oracle_values(ff)
    host["rho_g"] = rho
    return dataclasses.replace(pb, host=host)


def _with_function(pb, ff):
    import dataclasses

    host = dict(pb.host)
    nd = pb.grid.ndim
    rho = [None] * nd
    rho[nd - 1] = ff
    host["rho_g"] = rho
    return dataclasses.replace(pb, host=host)


def _states_equal(a, b):
    for name in ("V", "tau"):
        for fa, fb in zip(a.fields[name], b.fields[name]):
            np.testing.assert_array_equal(fa.to_numpy(), fb.to_numpy(), err_msg=name)
    np.testing.assert_array_equal(a.fields["P"].to_numpy(), b.fields["P"].to_numpy())


@pytest.mark.parametrize("precision", [_abi.CG_F64, _abi.CG_F32])
def test_example_solve_with_function_body_force(arch, precision):
    """The example's PT solve (scalar eta, buoyant disc) with rhogy a device FunctionField equals
    the solve with rhogy materialised (by the oracle's fill) in an array: the same iteration count
    and the same bits, in FP64 PT and in FP32 PT inside FP64 defect correction."""
    pb, ff = _example_problem(48)
    a = StokesSolver(arch, _with_array(pb, ff))
    b = StokesSolver(arch, _with_function(pb, ff))
    assert b.fields["rho_g"][1] is None and b.params.rho_g_fn[1].kind == _abi.CG_FN_BALL
    ra, rb = [], []
    for s, r in ((a, ra), (b, rb)):
        s.apply_bc()
        res = s.solve(precision=precision)
        assert res.converged == 1, (res.iterations, list(res.err))
        r.append(res.iterations)
    assert ra == rb
    _states_equal(a, b)


def test_3d_solve_with_function_body_force(arch):
    """3D VE Stokes (random log-viscosity, free slip) at 16^3 with the buoyant sphere rhogz as a
    device FunctionField: the FP64 solve equals the one with the sphere in an array, bit for bit."""
    pb = stokes3d_grf(16, ncheck=16)
    ff = FunctionField(ball, pb.grid, (Center(), Center(), Vertex()), parameters=(0.0, 0.0, 0.0, 0.1, 1.0, 0.0))
    # the configuration's sphere (coordinates rounded once more on the host) up to boundary points
    assert np.mean(ff.values() != pb.host["rho_g"][2]) < 1e-3
    a = StokesSolver(arch, _with_array(pb, ff))
    b = StokesSolver(arch, _with_function(pb, ff))
    for s in (a, b):
        s.apply_bc()
        res = s.solve(precision=_abi.CG_F64)
        assert res.converged == 1
    _states_equal(a, b)


def test_launcher_update_velocity_with_function_field(arch):
    """launch(update_velocity! => (V, r_V, Pr, tau, rhogy, eta_ve, nu_dtau, grid)) with rhogy the
    example's FunctionField equals the same launch with the array, bit for bit."""
    from chmy_gb300 import Field, Launcher, TensorField, VectorField, update_velocity

    pb, ff = _example_problem(40)
    grid = pb.grid
    outs = []
    for use_fn in (False, True):
        V, r_V, tau = VectorField(arch, grid), VectorField(arch, grid), TensorField(arch, grid)
        Pr = Field(arch, grid, Center())
        r2 = np.random.default_rng(3)
        for f in list(V) + list(tau) + [Pr]:
            f.from_numpy(r2.standard_normal(f.data.shape))
        if use_fn:
            rho = ff
        else:
            rho = Field(arch, grid, ff.loc)
            arch.call("cg_function_fill", ctypes.byref(grid.desc()), ctypes.byref(ff.desc()), ctypes.byref(rho.desc()))
        Launcher(arch, grid)(arch, grid, (update_velocity, (V, r_V, Pr, tau, rho, pb.params.eta_ve, pb.params.nu_dtau, grid)))
        outs.append([f.to_numpy() for f in list(V) + list(r_V)])
    for x, y in zip(*outs):
        np.testing.assert_array_equal(x, y)


def test_function_body_force_argument_checks(arch):
    """A component with both an array and a function is rejected, and so is a function given to
    the fused ping-pong entry (it reads body-force arrays only)."""
    pb, ff = _example_problem(32)
    s = StokesSolver(arch, _with_array(pb, ff))
    p = _abi.cg_stokes_params()
    ctypes.memmove(ctypes.byref(p), ctypes.byref(s.params), ctypes.sizeof(p))
    p.rho_g_fn[1] = ff.desc()
    rc = arch.lib.cg_stokes_update_velocity(arch.ctx, ctypes.byref(s.grid_desc), ctypes.byref(s.desc), ctypes.byref(p))
    assert rc == _abi.CG_ERR_ARG
    assert b"both" in arch.lib.cg_last_error(arch.ctx)
    p.rho_g_fn[1].kind = 9
    rc = arch.lib.cg_stokes_update_velocity(arch.ctx, ctypes.byref(s.grid_desc), ctypes.byref(s.desc), ctypes.byref(p))
    assert rc == _abi.CG_ERR_ARG
    p.rho_g_fn[1] = ff.desc()
    rc = arch.lib.cg_stokes_pt_iterations_pp(arch.ctx, ctypes.byref(s.grid_desc), ctypes.byref(s.desc), ctypes.byref(s.desc),
                                             ctypes.byref(p), None, 2)
    assert rc == _abi.CG_ERR_UNSUPPORTED
