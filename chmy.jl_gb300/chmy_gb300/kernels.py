"""The example kernels of Chmy.jl as library launches, and Launcher.

Chmy's user kernels are KernelAbstractions `@kernel` functions JIT-compiled by CUDA.jl.
On GB300 each known kernel of the hot path is a hand-written sm_103a kernel exported by
libchmy_gb300; the kernel objects below carry the reference's argument lists
(examples/diffusion_2d.jl:8-19, examples/stokes_2d_inc_ve_T.jl:11-60,
examples/stokes_3d_inc_ve_T.jl:11-77) so that `launch(arch, grid, kernel => args; bc)`
reads as in the reference.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

from . import _abi
from .bcs import Batch, apply_batch
from .fields import Field


@dataclass
class CellViscosity:
    """Per-cell viscosity for the VE Stokes kernels (the examples use a scalar eta).

    eta_ve = 1/(1/eta + 1/(G dt)) per cell; shear components use eta linearly interpolated
    (Chmy `lerp`) to their location; the velocity PT step uses the larger eta_ve of the two
    cells beside each face. Pass it as `η` to update_stress and as `η_ve` to
    update_velocity."""

    eta: Field
    G: float
    dt: float


def _vec(fields, n=3):
    arr = (_abi.cg_field * n)()
    if fields is None:
        return arr
    for i, f in enumerate(fields):
        if f is not None:
            arr[i] = f.desc()
    return arr


def stokes_fields(
    V=None, r_V=None, P=None, divV=None, tau=None, tau_old=None, eta=None, inv_eta=None, rho_g=None, T=None, T_old=None, qT=None
) -> _abi.cg_stokes_fields:
    """Pack the VE Stokes field set into the library descriptor. `rho_g` is a sequence of
    per-component fields (None entries allowed)."""
    s = _abi.cg_stokes_fields()
    s.V = _vec(V)
    s.r_V = _vec(r_V)
    if P is not None:
        s.P = P.desc()
    if divV is not None:
        s.divV = divV.desc()
    s.tau = _vec(tau, 6)
    s.tau_old = _vec(tau_old, 6)
    if eta is not None:
        s.eta = eta.desc()
    if inv_eta is not None:
        s.inv_eta = inv_eta.desc()
    s.rho_g = _vec(rho_g)
    if T is not None:
        s.T = T.desc()
    if T_old is not None:
        s.T_old = T_old.desc()
    s.qT = _vec(qT)
    return s


def stokes_params(eta=0.0, eta_ve=0.0, G=1.0, dt=1.0, dtau_Pr=0.0, dtau_r=0.0, nu_dtau=0.0, lambda_rhoCp=0.0):
    p = _abi.cg_stokes_params()
    p.eta, p.eta_ve, p.G, p.dt = float(eta), float(eta_ve), float(G), float(dt)
    p.dtau_Pr, p.dtau_r, p.nu_dtau, p.lambda_rhoCp = float(dtau_Pr), float(dtau_r), float(nu_dtau), float(lambda_rhoCp)
    return p


class Kernel:
    name = "kernel"

    def launch(self, arch, grid, *args):  # pragma: no cover - abstract
        raise NotImplementedError

    def __repr__(self):
        return f"{self.name}!"


class _ComputeQ(Kernel):
    """compute_q!(q, C, χ, g) (examples/diffusion_2d.jl:8-13); with a trailing FieldMask ω, the
    masked form q.d = -χ ∂d(C, ω, g, I)."""

    name = "compute_q"

    def launch(self, arch, grid, q, C, chi, g=None, omega=None):
        qa = _vec(q)
        c = C.desc()
        if omega is not None:
            arch.call("cg_diffusion_compute_q_masked", ctypes.byref(grid.desc()), qa, ctypes.byref(c), float(chi),
                      ctypes.byref(omega.desc()))
            return
        arch.call("cg_diffusion_compute_q", ctypes.byref(grid.desc()), qa, ctypes.byref(c), float(chi))


class _UpdateC(Kernel):
    """update_C!(C, q, Δt, g) (examples/diffusion_2d.jl:15-19); with a trailing FieldMask ω, the
    masked form C -= Δt divg(q, ω, g, I)."""

    name = "update_C"

    def launch(self, arch, grid, C, q, dt, g=None, omega=None):
        qa = _vec(q)
        c = C.desc()
        if omega is not None:
            arch.call("cg_diffusion_update_C_masked", ctypes.byref(grid.desc()), ctypes.byref(c), qa, float(dt),
                      ctypes.byref(omega.desc()))
            return
        arch.call("cg_diffusion_update_C", ctypes.byref(grid.desc()), ctypes.byref(c), qa, float(dt))


class _UpdateOld(Kernel):
    """update_old!(T, τ, T_old, τ_old) (examples/stokes_2d_inc_ve_T.jl:11-18)."""

    name = "update_old"

    def launch(self, arch, grid, T, tau, T_old, tau_old):
        s = stokes_fields(tau=tau, tau_old=tau_old, T=T, T_old=T_old)
        arch.call("cg_stokes_update_old", ctypes.byref(grid.desc()), ctypes.byref(s))


class _UpdateStress(Kernel):
    """update_stress!(τ, Pr, ∇V, V, τ_old, η, η_ve, G, dt, dτ_Pr, dτ_r, g)
    (examples/stokes_2d_inc_ve_T.jl:20-34; 3D :23-46). A trailing FieldMask ω selects the form
    written with the masked operators: ∂(V.d, ω, g, I) for the strain rates and divg(V, ω, g, I)."""

    name = "update_stress"

    def launch(self, arch, grid, tau, Pr, divV, V, tau_old, eta, eta_ve, G, dt, dtau_Pr, dtau_r, g=None, omega=None):
        eta_f = eta.eta if isinstance(eta, CellViscosity) else None
        s = stokes_fields(V=V, P=Pr, divV=divV, tau=tau, tau_old=tau_old, eta=eta_f)
        p = stokes_params(
            eta=0.0 if eta_f is not None else eta,
            eta_ve=0.0 if eta_f is not None else eta_ve,
            G=G,
            dt=dt,
            dtau_Pr=dtau_Pr,
            dtau_r=dtau_r,
        )
        if omega is not None:
            arch.call("cg_stokes_update_stress_masked", ctypes.byref(grid.desc()), ctypes.byref(s), ctypes.byref(p),
                      ctypes.byref(omega.desc()))
            return
        arch.call("cg_stokes_update_stress", ctypes.byref(grid.desc()), ctypes.byref(s), ctypes.byref(p))


class _UpdateVelocity(Kernel):
    """update_velocity!(V, r_V, Pr, τ, ρg, η_ve, νdτ, g) (examples/stokes_2d_inc_ve_T.jl:36-43;
    3D :48-57). `ρg` is the body force of the last component (ρgy in 2D, ρgz in 3D): a Field, a
    FunctionField of a device form (evaluated in the kernel, as the example's
    FunctionField(init_incl, ...) of :107), or None. A trailing FieldMask ω selects the form
    written with the masked operators ∂(Pr, ω, g, I) and ∂(τ.c, ω, g, I)."""

    name = "update_velocity"

    def launch(self, arch, grid, V, r_V, Pr, tau, rho_g, eta_ve, nu_dtau, g=None, omega=None):
        from .functions import FunctionField

        nd = grid.ndim
        rho = [None] * 3
        fn = None
        if isinstance(rho_g, FunctionField):
            fn = rho_g.desc()  # evaluated by the kernel at every face (a device FunctionField)
        else:
            rho[nd - 1] = rho_g
        if isinstance(eta_ve, CellViscosity):
            s = stokes_fields(V=V, r_V=r_V, P=Pr, tau=tau, rho_g=rho, eta=eta_ve.eta)
            p = stokes_params(G=eta_ve.G, dt=eta_ve.dt, nu_dtau=nu_dtau)
        else:
            s = stokes_fields(V=V, r_V=r_V, P=Pr, tau=tau, rho_g=rho)
            p = stokes_params(eta_ve=eta_ve, nu_dtau=nu_dtau)
        if fn is not None:
            p.rho_g_fn[nd - 1] = fn
        if omega is not None:
            arch.call("cg_stokes_update_velocity_masked", ctypes.byref(grid.desc()), ctypes.byref(s), ctypes.byref(p),
                      ctypes.byref(omega.desc()))
            return
        arch.call("cg_stokes_update_velocity", ctypes.byref(grid.desc()), ctypes.byref(s), ctypes.byref(p))


class _UpdateThermalFlux(Kernel):
    """update_thermal_flux!(qT, T, V, λ_ρCp, g) (examples/stokes_2d_inc_ve_T.jl:45-54)."""

    name = "update_thermal_flux"

    def launch(self, arch, grid, qT, T, V, lam, g=None):
        s = stokes_fields(V=V, T=T, qT=qT)
        p = stokes_params(lambda_rhoCp=lam)
        arch.call("cg_stokes_update_thermal_flux", ctypes.byref(grid.desc()), ctypes.byref(s), ctypes.byref(p))


class _UpdateThermal(Kernel):
    """update_thermal!(T, T_old, qT, dt, g) (examples/stokes_2d_inc_ve_T.jl:56-60)."""

    name = "update_thermal"

    def launch(self, arch, grid, T, T_old, qT, dt, g=None):
        s = stokes_fields(T=T, T_old=T_old, qT=qT)
        p = stokes_params(dt=dt)
        arch.call("cg_stokes_update_thermal", ctypes.byref(grid.desc()), ctypes.byref(s), ctypes.byref(p))


compute_q = _ComputeQ()
update_C = _UpdateC()
update_old = _UpdateOld()
update_stress = _UpdateStress()
update_velocity = _UpdateVelocity()
update_thermal_flux = _UpdateThermalFlux()
update_thermal = _UpdateThermal()


class Launcher:
    """Launcher(arch, grid; outer_width) (src/KernelLaunch.jl:21-54,105-126,152-159).

    `launch(arch, grid, (kernel, args), bc=batch)` runs the kernel over Chmy's launch range
    [0, n+1]^N, then the batch's boundary conditions, then synchronizes like the reference
    (pass sync=False to keep the work stream-ordered). `outer_width` configured Chmy's
    compute/MPI overlap and has no effect on one GPU."""

    def __init__(self, arch, grid, outer_width=None, sync: bool = True):
        self.arch = arch
        self.grid = grid
        self.outer_width = outer_width
        self.sync = sync

    def __call__(self, arch, grid, kernel_and_args, bc: Batch | None = None):
        kernel, args = kernel_and_args
        if not isinstance(kernel, Kernel):
            raise TypeError(f"{kernel!r} is not a GB300 kernel of the hot path")
        kernel.launch(arch, grid, *args)
        if bc is not None:
            apply_batch(arch, grid, bc)
        if self.sync:
            arch.synchronize()
