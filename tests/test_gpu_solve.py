"""PT solves to 1e-8 on the GPU: FP64 PT iteration counts against the oracle's, and FP32 PT
inside FP64 defect correction reaching the same FP64-measured tolerance."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, lib, stokes_desc
from chmy_gb300 import _abi
from chmy_gb300.bcs import Dirichlet, to_cg_bc
from chmy_gb300.configs import stokes2d_inclusions
from chmy_gb300.grids import Center, Vertex
from chmy_gb300.solvers import StokesSolver

pytestmark = pytest.mark.gpu


def oracle_solve(pb):
    """The reference PT loop (examples/stokes_2d_inc_ve_T.jl:144-163) on the oracle."""
    g = pb.grid
    Cl, Vl = Center(), Vertex()

    def mk(a, loc):
        f = NpField(g, loc)
        f.a[...] = a
        return f

    h = pb.host
    V = [mk(h["V"][0], (Vl, Cl)), mk(h["V"][1], (Cl, Vl))]
    rV = [mk(h["r_V"][0], (Vl, Cl)), mk(h["r_V"][1], (Cl, Vl))]
    tau = [mk(h["tau"][0], Cl), mk(h["tau"][1], Cl), mk(h["tau"][2], Vl)]
    tauo = [mk(h["tau_old"][0], Cl), mk(h["tau_old"][1], Cl), mk(h["tau_old"][2], Vl)]
    P, divV, eta = mk(h["P"], Cl), mk(h["divV"], Cl), mk(h["eta"], Cl)
    d = stokes_desc(V=V, r_V=rV, P=P, divV=divV, tau=tau, tau_old=tauo, eta=eta)
    gd = g.desc()
    p = pb.params
    bc_apply(g, V, pb.bc_V)
    rb = [to_cg_bc(2, {"x": Dirichlet()}), to_cg_bc(2, {"y": Dirichlet()})]
    for it in range(1, pb.max_iter + 1):
        lib().or_stokes_update_stress(ctypes.byref(gd), ctypes.byref(d), ctypes.byref(p))
        lib().or_stokes_update_velocity(ctypes.byref(gd), ctypes.byref(d), ctypes.byref(p))
        bc_apply(g, V, pb.bc_V)
        if it % pb.ncheck == 0:
            bc_apply(g, rV, rb)
            e = [np.abs(divV.interior()).max() * pb.tau_scale] + [np.abs(f.interior()).max() * pb.v_scale for f in rV]
            if max(e) < pb.eps:
                return it, e, V, P
    return None, e, V, P


@pytest.fixture(scope="module")
def problem64():
    return stokes2d_inclusions(64, ncheck=16)


@pytest.fixture(scope="module")
def oracle64(problem64):
    return oracle_solve(problem64)


def test_fp64_iteration_count_matches_oracle(arch, problem64, oracle64):
    it_ref, e_ref, V_ref, P_ref = oracle64
    assert it_ref is not None, "oracle did not converge"
    s = StokesSolver(arch, problem64, precompute_inv_eta=False)
    s.apply_bc()
    res = s.solve(precision=_abi.CG_F64)
    assert res.converged == 1
    assert abs(res.iterations - it_ref) <= max(0.01 * it_ref, problem64.ncheck), (res.iterations, it_ref)
    # converged states agree to the solver tolerance
    vx = s.fields["V"][0].to_numpy()
    scale = np.abs(V_ref[0].a).max()
    assert np.max(np.abs(vx - V_ref[0].a)) <= 1e-6 * scale


def test_fp64_with_precomputed_inverse_is_bitwise_same(arch, problem64):
    a = StokesSolver(arch, problem64, precompute_inv_eta=False)
    b = StokesSolver(arch, problem64, precompute_inv_eta=True)
    for s in (a, b):
        s.apply_bc()
        s.iterate(64)
    arch.synchronize()
    for fa, fb in zip(a.fields["tau"], b.fields["tau"]):
        assert np.array_equal(fa.to_numpy(), fb.to_numpy())


@pytest.mark.parametrize("n", [64, 128])
def test_fp32_defect_correction_reaches_fp64_tolerance(arch, n):
    pb = stokes2d_inclusions(n, ncheck=n // 4)
    ref = StokesSolver(arch, pb)
    ref.apply_bc()
    r64 = ref.solve(precision=_abi.CG_F64)
    assert r64.converged == 1
    dc = StokesSolver(arch, pb)
    dc.apply_bc()
    r32 = dc.solve(precision=_abi.CG_F32, max_outer=8, inner_rtol=1e-5)
    assert r32.converged == 1, (r32.outer, r32.iterations, list(r32.err))
    assert max(r32.err[i] for i in range(3)) < pb.eps
    assert r32.outer >= 1
    # the two converged FP64 states agree to well below the discretisation scale
    for name in ("V", "tau"):
        for fa, fb in zip(ref.fields[name], dc.fields[name]):
            a, b = fa.to_numpy(), fb.to_numpy()
            assert np.max(np.abs(a - b)) <= 1e-5 * max(np.abs(a).max(), 1.0), name
    # with normal velocity prescribed on every side the pressure is defined up to a constant,
    # which each PT path fixes differently: compare the interior pressure minus its mean
    pa, pb_ = ref.fields["P"].to_numpy()[2:-2, 2:-2], dc.fields["P"].to_numpy()[2:-2, 2:-2]
    pa, pb_ = pa - pa.mean(), pb_ - pb_.mean()
    assert np.max(np.abs(pa - pb_)) <= 1e-5 * np.abs(pa).max()


def _compare_states(ref, dc, nd, rtol=1e-5):
    for name in ("V", "tau"):
        for fa, fb in zip(ref.fields[name], dc.fields[name]):
            a, b = fa.to_numpy(), fb.to_numpy()
            assert np.max(np.abs(a - b)) <= rtol * max(np.abs(a).max(), 1.0), name
    sl = (slice(2, -2),) * nd
    pa, pb_ = ref.fields["P"].to_numpy()[sl], dc.fields["P"].to_numpy()[sl]
    pa, pb_ = pa - pa.mean(), pb_ - pb_.mean()
    assert np.max(np.abs(pa - pb_)) <= rtol * max(np.abs(pa).max(), 1.0)


def test_fp32_defect_correction_scalar_viscosity(arch):
    """Scalar eta (the examples' form) with a buoyant disc: the FP32 correction runs the fused
    kernel on a constant 1/eta and reaches the FP64 solve's tolerance and state."""
    import dataclasses

    from chmy_gb300.configs import padded_mesh

    pb = stokes2d_inclusions(64, ncheck=16)
    host = {k: v for k, v in pb.host.items() if k != "eta"}
    x, y = padded_mesh(pb.grid, (Center(), Vertex()))
    host["rho_g"] = [None, np.where(x**2 + y**2 < 0.1**2, 1.0, 0.0)]
    pb = dataclasses.replace(pb, host=host)
    ref = StokesSolver(arch, pb)
    ref.apply_bc()
    r64 = ref.solve(precision=_abi.CG_F64)
    assert r64.converged == 1
    dc = StokesSolver(arch, pb)
    dc.apply_bc()
    r32 = dc.solve(precision=_abi.CG_F32, max_outer=8, inner_rtol=1e-5)
    assert r32.converged == 1, (r32.outer, r32.iterations, list(r32.err))
    assert max(r32.err[i] for i in range(3)) < pb.eps
    _compare_states(ref, dc, 2)


def test_fp32_defect_correction_3d(arch):
    """3D VE Stokes (Gaussian random log-viscosity, buoyant sphere, free slip): FP32 PT in the
    z-marching fused kernel inside FP64 defect correction reaches the FP64 solve's tolerance
    and state."""
    from chmy_gb300.configs import stokes3d_grf

    pb = stokes3d_grf(24, ncheck=24)
    ref = StokesSolver(arch, pb)
    ref.apply_bc()
    r64 = ref.solve(precision=_abi.CG_F64)
    assert r64.converged == 1, (r64.iterations, list(r64.err))
    dc = StokesSolver(arch, pb)
    dc.apply_bc()
    r32 = dc.solve(precision=_abi.CG_F32, max_outer=8, inner_rtol=1e-5)
    assert r32.converged == 1, (r32.outer, r32.iterations, list(r32.err))
    assert max(r32.err[i] for i in range(4)) < pb.eps
    _compare_states(ref, dc, 3)


def test_fp32_solve_rejects_fp32_state(arch):
    pb = stokes2d_inclusions(32, dtype=np.float32)
    s = StokesSolver(arch, pb)
    o = _abi.cg_solve_opts(max_iter=64, ncheck=8, eps=1e-8, tau_scale=1.0, v_scale=1.0, precision=_abi.CG_F32)
    res = _abi.cg_solve_result()
    rc = arch.lib.cg_stokes_solve(arch.ctx, ctypes.byref(s.grid_desc), ctypes.byref(s.desc), ctypes.byref(pb.params), s.bc_arr, ctypes.byref(o), ctypes.byref(res))
    assert rc == _abi.CG_ERR_UNSUPPORTED
