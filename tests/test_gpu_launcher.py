"""Chmy's launch API on the GB300 path: `Launcher`, the example kernel objects and `batch`/`bc_`
(src/KernelLaunch.jl:105-126, src/BoundaryConditions/batch.jl:156-160) drive the time loop of
examples/diffusion_2d.jl:37-47 and PT iterations of examples/stokes_2d_inc_ve_T.jl:144-146 (and
its 3D form), written as in the reference, and match the oracle's restatement of the same loops."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, diffusion_run, lib, stokes_desc, tensor_fields, vec_fields
from chmy_gb300 import (
    Arch,
    CellViscosity,
    Dirichlet,
    Field,
    Launcher,
    Neumann,
    TensorField,
    VectorField,
    batch,
    bc_,
    compute_q,
    interior,
    set_,
    update_C,
    update_stress,
    update_velocity,
)
from chmy_gb300.bcs import to_cg_bc
from chmy_gb300.grids import Center, UniformGrid, Vertex
from chmy_gb300.kernels import stokes_params

pytestmark = pytest.mark.gpu


def test_diffusion_time_loop_through_launcher(arch):
    """examples/diffusion_2d.jl:37-47: set! from a function, bc!, then nt iterations of
    launch(compute_q! => (q, C, chi, grid)) and launch(update_C! => (C, q, dt, grid); bc=batch(C
    => Neumann())). The loop equals the oracle's kernels step for step, bit for bit."""
    grid = UniformGrid(origin=(-1.0, -1.0), extent=(2.0, 2.0), dims=(30, 26))
    launch = Launcher(arch, grid)
    C = Field(arch, grid, Center())
    q = VectorField(arch, grid)
    set_(C, lambda x, y: np.exp(-(x * x + y * y) / 0.1), grid)
    bc_(arch, grid, (C, Neumann()))
    C0 = C.to_numpy()
    chi = 1.0
    dt = float(min(grid.spacing())) ** 2 / chi / 2 / 2.1  # examples/diffusion_2d.jl:29
    nt = 40
    for _ in range(nt):
        launch(arch, grid, (compute_q, (q, C, chi, grid)))
        launch(arch, grid, (update_C, (C, q, dt, grid)), bc=batch(grid, (C, Neumann()), exchange=C))
    ref = diffusion_run(grid, C0, chi, dt, to_cg_bc(2, Neumann()), nt)
    got = C.to_numpy()
    assert np.array_equal(got, ref)
    # the interior view is Chmy's [x, y] order
    assert tuple(interior(C).shape) == grid.dims


def _stokes_setup(nd, variable, seed=1):
    T = np.float64
    n = (26, 22) if nd == 2 else (14, 12, 10)
    grid = UniformGrid(origin=(-0.5,) * nd, extent=(1.0,) * nd, dims=n, dtype=T)
    rng = np.random.default_rng(seed)
    dx = float(min(grid.spacing()))
    re_m, r = 2.3 * np.pi, 0.5
    lt = 1.0 / re_m
    vdt = dx / np.sqrt(nd * 1.1)
    th = lt * (r + 4.0 / 3.0) / vdt
    c = dict(G=1.0, dt=1e-2, eta=1.0, dtau_Pr=r / th, dtau_r=1.0 / (th + 1.0), nu_dtau=vdt * lt)
    c["eta_ve"] = 1.0 / (1.0 / c["eta"] + 1.0 / (c["G"] * c["dt"]))
    eta = np.exp(rng.uniform(-1.5, 1.5, NpField(grid, Center()).a.shape)) if variable else None
    return grid, rng, c, eta


@pytest.mark.parametrize("nd,variable", [(2, False), (2, True), (3, False)])
def test_stokes_pt_iterations_through_launcher(arch, nd, variable):
    """PT iterations written as in the reference: launch(update_stress! => (tau, Pr, divV, V,
    tau_old, eta, eta_ve, G, dt, dtau_Pr, dtau_r, grid)) and launch(update_velocity! => (V, r_V,
    Pr, tau, rho_g, eta_ve, nu_dtau, grid); bc=batch(V.x => ..., V.y => ...)), with the
    examples' scalar viscosity or a CellViscosity passed as eta and eta_ve. The fields match the
    oracle's kernels after every iteration's boundary conditions."""
    grid, rng, c, eta = _stokes_setup(nd, variable)
    launch = Launcher(arch, grid)
    V = VectorField(arch, grid)
    r_V = VectorField(arch, grid)
    tau = TensorField(arch, grid)
    tau_old = TensorField(arch, grid)
    Pr = Field(arch, grid, Center())
    divV = Field(arch, grid, Center())
    rho_loc = tuple(Vertex() if d == nd - 1 else Center() for d in range(nd))
    rho = Field(arch, grid, rho_loc)
    # host copies for the oracle, with the same random start
    hV, hrV = vec_fields(grid, np.float64), vec_fields(grid, np.float64)
    htau, htau_old = tensor_fields(grid, np.float64), tensor_fields(grid, np.float64)
    hP, hdiv = NpField(grid, Center()), NpField(grid, Center())
    hrho = NpField(grid, rho_loc)
    for dev, host in zip(list(V) + list(tau_old) + [Pr, rho], hV + htau_old + [hP, hrho]):
        host.a[...] = rng.standard_normal(host.a.shape)
        dev.from_numpy(host.a)
    if variable:
        etaf = Field(arch, grid, Center())
        etaf.from_numpy(eta)
        heta = NpField(grid, Center())
        heta.a[...] = eta
        eta_arg = CellViscosity(etaf, c["G"], c["dt"])
        eta_ve_arg = eta_arg
    else:
        heta = None
        eta_arg, eta_ve_arg = c["eta"], c["eta_ve"]
    names = "xyz"
    specs = []
    for d in range(nd):
        specs.append({names[e]: (Dirichlet(0.1 * (d + 1)) if e == d else Neumann()) for e in range(nd)})
    bcV = batch(grid, *[(V[d], specs[d]) for d in range(nd)], exchange=V)
    hbc = [to_cg_bc(nd, s) for s in specs]
    bc_(arch, grid, bcV)
    bc_apply(grid, hV, hbc)
    rho_arg = rho
    hd = stokes_desc(V=hV, r_V=hrV, P=hP, divV=hdiv, tau=htau, tau_old=htau_old, eta=heta,
                     rho_g=[None] * (nd - 1) + [hrho])
    if variable:
        p = stokes_params(G=c["G"], dt=c["dt"], dtau_Pr=c["dtau_Pr"], dtau_r=c["dtau_r"], nu_dtau=c["nu_dtau"])
    else:
        p = stokes_params(eta=c["eta"], eta_ve=c["eta_ve"], G=c["G"], dt=c["dt"], dtau_Pr=c["dtau_Pr"], dtau_r=c["dtau_r"],
                          nu_dtau=c["nu_dtau"])
    g = grid.desc()
    niter = 12
    for it in range(niter):
        launch(arch, grid, (update_stress, (tau, Pr, divV, V, tau_old, eta_arg, c["eta_ve"], c["G"], c["dt"], c["dtau_Pr"],
                                            c["dtau_r"], grid)))
        launch(arch, grid, (update_velocity, (V, r_V, Pr, tau, rho_arg, eta_ve_arg, c["nu_dtau"], grid)), bc=bcV)
        assert lib().or_stokes_update_stress(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p)) == 0
        assert lib().or_stokes_update_velocity(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p)) == 0
        bc_apply(grid, hV, hbc)
    tol = 1e-12 * niter
    for dev, host, what in zip(list(V) + list(tau) + [Pr], hV + htau + [hP], ["V"] * nd + ["tau"] * len(htau) + ["P"]):
        a, b = dev.to_numpy(), host.a
        assert np.max(np.abs(a - b)) <= tol * max(np.abs(b).max(), 1.0), what
    for dev, host in zip(r_V, hrV):
        a, b = dev.to_numpy()[(slice(2, -2),) * nd], host.a[(slice(2, -2),) * nd]
        assert np.max(np.abs(a - b)) <= tol * max(np.abs(b).max(), 1.0), "r_V"


def test_launcher_rejects_foreign_kernels(arch):
    grid = UniformGrid(origin=(0.0, 0.0), extent=(1.0, 1.0), dims=(8, 8))
    launch = Launcher(arch, grid)
    with pytest.raises(TypeError):
        launch(arch, grid, (lambda *a: None, ()))
