"""PT solves to 1e-8 on the GPU: FP64 PT iteration counts against the oracle's, and FP32 PT
inside FP64 defect correction reaching the same FP64-measured tolerance."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, lib, stokes_desc, stokes_problem_fields
from chmy_gb300 import _abi
from chmy_gb300.bcs import Dirichlet, to_cg_bc
from chmy_gb300.configs import stokes2d_inclusions
from chmy_gb300.grids import Center, Vertex
from chmy_gb300.solvers import StokesSolver

pytestmark = pytest.mark.gpu


def oracle_solve(pb):
    """The reference PT loop (examples/stokes_2d_inc_ve_T.jl:144-163; 3D
    examples/stokes_3d_inc_ve_T.jl:163-183) on the oracle, in 2D or 3D: update_stress!,
    update_velocity!, bc!(V) per iteration; every ncheck iterations bc!(r_V.d => Dirichlet on
    dim d) and the measures max|divV|*tau_scale, max|r_V.d|*v_scale against eps."""
    g = pb.grid
    nd = g.ndim
    f = stokes_problem_fields(pb)
    d = f["desc"]
    gd = g.desc()
    p = pb.params
    V, rV, divV = f["V"], f["r_V"], f["divV"]
    bc_apply(g, V, pb.bc_V)
    rb = [to_cg_bc(nd, {"xyz"[k]: Dirichlet()}) for k in range(nd)]
    e = None
    for it in range(1, pb.max_iter + 1):
        lib().or_stokes_update_stress(ctypes.byref(gd), ctypes.byref(d), ctypes.byref(p))
        lib().or_stokes_update_velocity(ctypes.byref(gd), ctypes.byref(d), ctypes.byref(p))
        bc_apply(g, V, pb.bc_V)
        if it % pb.ncheck == 0:
            bc_apply(g, rV, rb)
            e = [np.abs(divV.interior()).max() * pb.tau_scale] + [np.abs(x.interior()).max() * pb.v_scale for x in rV]
            if max(e) < pb.eps:
                return it, e, V, f["P"]
    return None, e, V, f["P"]


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


def test_fp64_iteration_count_with_the_reference_pt_constants(arch):
    """The example's own PT constants (examples/stokes_2d_inc_ve_T.jl:84-93): re_m = 2.3 pi and a
    check every 2 nx iterations, on the 64^2 inclusion problem. The GPU's FP64 solve stops at
    the oracle's check, and the states agree."""
    pb = stokes2d_inclusions(64, ncheck=2 * 64, re_m_pi=2.3)
    it_ref, e_ref, V_ref, P_ref = oracle_solve(pb)
    assert it_ref is not None, ("oracle did not converge", e_ref)
    s = StokesSolver(arch, pb, precompute_inv_eta=False)
    s.apply_bc()
    res = s.solve(precision=_abi.CG_F64)
    assert res.converged == 1
    assert abs(res.iterations - it_ref) <= 0.01 * it_ref, (res.iterations, it_ref)
    for d in range(2):
        a = s.fields["V"][d].to_numpy()
        assert np.max(np.abs(a - V_ref[d].a)) <= 1e-6 * np.abs(V_ref[d].a).max()


def test_fp64_iteration_count_3d_matches_oracle(arch):
    """3D VE Stokes (random log-viscosity field, buoyant sphere, free slip) at 24^3: the GPU's
    FP64 PT solve and the oracle's PT loop stop within 1 % of each other's iteration count,
    and their velocities agree."""
    from chmy_gb300.configs import stokes3d_grf

    pb = stokes3d_grf(24, ncheck=24)
    it_ref, e_ref, V_ref, P_ref = oracle_solve(pb)
    assert it_ref is not None, ("oracle did not converge", e_ref)
    s = StokesSolver(arch, pb, precompute_inv_eta=False)
    s.apply_bc()
    res = s.solve(precision=_abi.CG_F64)
    assert res.converged == 1, (res.iterations, list(res.err))
    assert abs(res.iterations - it_ref) <= max(0.01 * it_ref, pb.ncheck), (res.iterations, it_ref)
    for d in range(3):
        a = s.fields["V"][d].to_numpy()
        assert np.max(np.abs(a - V_ref[d].a)) <= 1e-6 * max(np.abs(V_ref[d].a).max(), 1e-30), d


@pytest.mark.parametrize("precision", [_abi.CG_F64, _abi.CG_F32])
@pytest.mark.parametrize("nd", [2, 3])
def test_solve_reports_nonfinite_viscosity(arch, precision, nd):
    """A NaN viscosity in one interior cell: the solve returns CG_ERR_NONFINITE, as the
    reference loop raises on a non-finite residual (examples/stokes_2d_inc_ve_T.jl:161), and
    the context stays usable."""
    import dataclasses

    from chmy_gb300.configs import stokes3d_grf

    pb = stokes2d_inclusions(32, ncheck=8) if nd == 2 else stokes3d_grf(16, ncheck=16)
    eta = pb.host["eta"].copy()
    eta[(7,) * nd] = np.nan
    bad = dataclasses.replace(pb, host={**pb.host, "eta": eta})
    s = StokesSolver(arch, bad)
    s.apply_bc()
    with pytest.raises(_abi.ChmyError) as exc:
        s.solve(precision=precision, max_iter=4 * pb.ncheck)
    assert exc.value.code == _abi.CG_ERR_NONFINITE, str(exc.value)
    ok = StokesSolver(arch, pb)
    ok.apply_bc()
    assert ok.solve(precision=precision).converged == 1


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


@pytest.mark.parametrize("layout", ["0:2", "0:3"])
def test_fp32_defect_correction_3d_staged_layouts_bitwise(arch, monkeypatch, layout):
    """The defect-correction solve with its inner FP32 iteration in march3d_tma_kernel (inputs
    staged by TMA, with the continuity forcing and all three body-force components) gives the
    register-fed kernel's solve bit for bit: the same iteration count and the same state."""
    from chmy_gb300.configs import stokes3d_grf

    pb = stokes3d_grf(24, ncheck=24)
    out = {}
    for lay in ("0:0", layout):
        monkeypatch.setenv("CG_MARCH_LAYOUT", lay)
        s = StokesSolver(arch, pb)
        s.apply_bc()
        r = s.solve(precision=_abi.CG_F32, max_outer=8, inner_rtol=1e-5)
        assert r.converged == 1, (lay, r.outer, r.iterations, list(r.err))
        out[lay] = (r.iterations, r.outer, [f.to_numpy() for f in s.fields["V"]], s.fields["P"].to_numpy(),
                    [f.to_numpy() for f in s.fields["tau"]])
    a, b = out["0:0"], out[layout]
    assert a[:2] == b[:2]
    for x, y in zip(a[2] + [a[3]] + a[4], b[2] + [b[3]] + b[4]):
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8))


def test_fp32_solve_rejects_fp32_state(arch):
    pb = stokes2d_inclusions(32, dtype=np.float32)
    s = StokesSolver(arch, pb)
    o = _abi.cg_solve_opts(max_iter=64, ncheck=8, eps=1e-8, tau_scale=1.0, v_scale=1.0, precision=_abi.CG_F32)
    res = _abi.cg_solve_result()
    rc = arch.lib.cg_stokes_solve(arch.ctx, ctypes.byref(s.grid_desc), ctypes.byref(s.desc), ctypes.byref(pb.params), s.bc_arr, ctypes.byref(o), ctypes.byref(res))
    assert rc == _abi.CG_ERR_UNSUPPORTED


def _example_setup(nxy, T):
    """examples/stokes_2d_inc_ve_T.jl:62-110 (scalar eta = 10, buoyant disc, hot disc)."""
    from chmy_gb300.configs import padded_mesh
    from chmy_gb300.grids import UniformGrid

    lx = ly = 2.0
    eta, G = 10.0, 1.0
    psc, tsc = G, eta / G
    T0, Ta = 1.0, 0.1
    lam = 1e-4 * ly**2 / tsc
    grid = UniformGrid(origin=(-lx / 2, -ly / 2), extent=(lx, ly), dims=(nxy, nxy), dtype=T)
    C_, V_ = Center(), Vertex()
    r = 0.1 * lx
    xc, yc = padded_mesh(grid, C_)
    xv, yv = padded_mesh(grid, (C_, V_))

    def z(loc):
        return np.zeros_like(padded_mesh(grid, loc)[0], dtype=T)

    tl = [(C_, C_), (C_, C_), (V_, V_)]
    host = {
        "V": [z((V_, C_)), z((C_, V_))],
        "r_V": [z((V_, C_)), z((C_, V_))],
        "P": z(C_),
        "divV": z(C_),
        "tau": [z(l) for l in tl],
        "tau_old": [z(l) for l in tl],
        "T": np.where(xc**2 + yc**2 < r * r, T0, Ta).astype(T),
        "T_old": z(C_),
        "rho_g": [None, np.where(xv**2 + yv**2 < r * r, 1.0, 0.0).astype(T)],
        "qT": [z((V_, C_)), z((C_, V_))],  # the oracle's two-kernel form stores the fluxes
    }
    dx = float(grid.spacing()[0])
    re_m, rr = 2.3 * np.pi, 0.5
    lt = min(lx, ly) / re_m
    vdt = dx / np.sqrt(2 * 1.1)
    th = lt * (rr + 4.0 / 3.0) / vdt
    consts = dict(eta=eta, G=G, lam=lam, dtau_r=1.0 / (th + 1.0), nu_dtau=vdt * lt, dtau_Pr=rr / th, tsc=tsc,
                  vsc=ly / psc, dx=dx)
    return grid, host, consts


def test_example_time_loop_with_thermal_coupling(arch):
    """Two time steps of examples/stokes_2d_inc_ve_T.jl:134-164 at 62^2 in FP64: update_old!,
    dt from max|V|, the PT solve (with the thermal step from the second time step on), on the
    GPU through the library and on the oracle. Iteration counts agree and so does T."""
    from chmy_gb300.bcs import Neumann
    from chmy_gb300.fields import Field
    from chmy_gb300.kernels import stokes_fields, stokes_params

    T = np.float64
    nxy = 62
    grid, host, c = _example_setup(nxy, T)
    g = grid.desc()
    bc_V = [to_cg_bc(2, {"x": Dirichlet(), "y": Neumann()}), to_cg_bc(2, {"x": Neumann(), "y": Dirichlet()})]
    bcT = to_cg_bc(2, {"x": Neumann(), "y": Neumann()})
    eps = 1e-6
    C_, V_ = Center(), Vertex()
    locs = {"V": [(V_, C_), (C_, V_)], "r_V": [(V_, C_), (C_, V_)], "tau": [(C_, C_), (C_, C_), (V_, V_)],
            "tau_old": [(C_, C_), (C_, C_), (V_, V_)], "rho_g": [None, (C_, V_)], "qT": [(V_, C_), (C_, V_)]}
    dev, hst = {}, {}
    for k, v in host.items():
        if isinstance(v, list):
            dev[k], hst[k] = [], []
            for a, loc in zip(v, locs[k]):
                if a is None:
                    dev[k].append(None)
                    hst[k].append(None)
                    continue
                f = Field(arch, grid, loc, T)
                f.from_numpy(a)
                dev[k].append(f)
                h = NpField(grid, loc, T)
                h.a[...] = a
                hst[k].append(h)
        else:
            f = Field(arch, grid, C_, T)
            f.from_numpy(v)
            dev[k] = f
            h = NpField(grid, C_, T)
            h.a[...] = v
            hst[k] = h
    dd = stokes_fields(**dev)
    hd = stokes_desc(**hst)
    bc_apply(grid, [hst["T"]], [bcT])
    arch.call("cg_bc_apply", ctypes.byref(g), 1, ctypes.byref(dev["T"].desc()), ctypes.byref(bcT))
    rb = [to_cg_bc(2, {"x": Dirichlet()}), to_cg_bc(2, {"y": Dirichlet()})]
    dx = c["dx"]
    for it in (1, 2):
        arch.call("cg_stokes_update_old", ctypes.byref(g), ctypes.byref(dd))
        lib().or_stokes_update_old(ctypes.byref(g), ctypes.byref(hd))
        vmax = [max(np.abs(f.interior()).max(), 1e-300) for f in hst["V"]]
        dt_diff = dx * dx / c["lam"] / 2 / 2.1
        dt_adv = 0.1 * min(dx / vmax[0], dx / vmax[1]) / 2 / 2.1
        dt = min(dt_diff, dt_adv)
        eta_ve = 1.0 / (1.0 / c["eta"] + 1.0 / (c["G"] * dt))
        p = stokes_params(eta=c["eta"], eta_ve=eta_ve, G=c["G"], dt=dt, dtau_Pr=c["dtau_Pr"], dtau_r=c["dtau_r"],
                          nu_dtau=c["nu_dtau"], lambda_rhoCp=c["lam"])
        ncheck = 2 * nxy
        niter = 50 * nxy
        # oracle: the reference loop
        it_ref = None
        for k in range(1, niter + 1):
            lib().or_stokes_update_stress(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
            lib().or_stokes_update_velocity(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
            bc_apply(grid, hst["V"], bc_V)
            if it > 1:
                lib().or_stokes_update_thermal_flux(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
                lib().or_stokes_update_thermal(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
                bc_apply(grid, [hst["T"]], [bcT])
            if k % ncheck == 0:
                bc_apply(grid, hst["r_V"], rb)
                e = [np.abs(hst["divV"].interior()).max() * c["tsc"]] + [np.abs(f.interior()).max() * c["vsc"] for f in hst["r_V"]]
                if max(e) < eps:
                    it_ref = k
                    break
        assert it_ref is not None, f"oracle did not converge in time step {it}"
        o = _abi.cg_solve_opts(max_iter=niter, ncheck=ncheck, eps=eps, tau_scale=c["tsc"], v_scale=c["vsc"], precision=_abi.CG_F64)
        r = _abi.cg_solve_result()
        bcv = (_abi.cg_bc * 3)(*bc_V)
        if it == 1:
            arch.call("cg_stokes_solve", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), bcv, ctypes.byref(o), ctypes.byref(r))
        else:
            arch.call("cg_stokes_solve_thermal", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), bcv, ctypes.byref(bcT), ctypes.byref(o), ctypes.byref(r))
        arch.synchronize()
        assert r.converged == 1
        assert r.iterations == it_ref, (it, r.iterations, it_ref)
    scale = np.abs(hst["T"].a).max()
    err = np.abs(dev["T"].to_numpy() - hst["T"].a).max()
    assert err <= 1e-9 * scale, err
    assert np.abs(dev["T"].to_numpy() - host["T"]).max() > 0  # the second step moved T
    # FP32 is not offered with thermal coupling
    o.precision = _abi.CG_F32
    rc = arch.lib.cg_stokes_solve_thermal(arch.ctx, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), bcv, ctypes.byref(bcT), ctypes.byref(o), ctypes.byref(r))
    assert rc == _abi.CG_ERR_UNSUPPORTED


@pytest.mark.parametrize("n", [64, 130])
def test_fp32_defect_correction_two_iterations_per_pass(arch, monkeypatch, n):
    """The FP32 PT chunks of the defect-correction solve with two iterations per pass (variants 1
    and 2 of the 2D layout) and with one (variant 0): the same iteration and cycle counts and the
    same bits of every solution field."""
    pb = stokes2d_inclusions(n, ncheck=n // 4)
    out = []
    for layout in ("0:0", "0:1", "16:2"):
        monkeypatch.setenv("CG_MARCH_LAYOUT", layout)
        s = StokesSolver(arch, pb)
        s.apply_bc()
        r = s.solve(precision=_abi.CG_F32, max_outer=8, inner_rtol=1e-5)
        assert r.converged == 1
        out.append((r.iterations, r.outer, [f.to_numpy() for f in s.fields["V"] + s.fields["tau"]] + [s.fields["P"].to_numpy()]))
    for it, outer, arrays in out[1:]:
        assert (it, outer) == (out[0][0], out[0][1])
        for a, b in zip(arrays, out[0][2]):
            np.testing.assert_array_equal(a, b)
