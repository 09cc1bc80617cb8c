"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset exists for these problems; each builder returns host (numpy) arrays of the whole
padded fields so that the GPU path and the CPU oracle start from identical bits.

stokes2d_inclusions: 2D incompressible VE Stokes (examples/stokes_2d_inc_ve_T.jl form) on
  [-0.5, 0.5]^2 with background viscosity 1 and 8 circular inclusions (centres uniform,
  radius U[0.02, 0.08], log10 viscosity U[-3, 3], seed 3), pure shear eps = 1 imposed as
  Dirichlet normal velocity -eps*x (x faces) and +eps*y (y faces) with free slip
  (Neumann) tangentially, G = 1, dt = 1e-2, PT parameters of the example (:86-93).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .bcs import Dirichlet, Neumann, to_cg_bc
from .grids import Center, UniformGrid, Vertex, expand_loc
from .kernels import stokes_params


def padded_coords(grid: UniformGrid, loc, halo=1):
    """Coordinates of every padded index (logical 1-2H .. n+2H) per dim, in the grid type."""
    locs = expand_loc(grid.ndim, loc)
    out = []
    for d, (ax, l) in enumerate(zip(grid.axes, locs)):
        n = ax.size(l)
        idx = np.arange(1 - 2 * halo, n + 2 * halo + 1)
        o = ax.origin if isinstance(l, Vertex) else ax.origin + 0.5 * ax.spacing
        out.append((o + (idx - 1) * ax.spacing).astype(grid.dtype))
    return out


def padded_mesh(grid: UniformGrid, loc, halo=1):
    """[z, y, x] ordered meshes of the padded coordinates (matching the storage order)."""
    c = padded_coords(grid, loc, halo)
    mesh = np.meshgrid(*reversed(c), indexing="ij")
    return list(reversed(mesh))  # x, y[, z] arrays shaped [z, y, x]


@dataclass
class StokesProblem:
    grid: UniformGrid
    host: dict = field(default_factory=dict)  # name -> padded numpy array or list of them
    params: object = None
    bc_V: list = field(default_factory=list)
    eps: float = 1e-8
    tau_scale: float = 1.0
    v_scale: float = 1.0
    ncheck: int = 512
    max_iter: int = 0


def inclusions(seed=3, count=8):
    rng = np.random.default_rng(seed)
    cx = rng.uniform(-0.5, 0.5, count)
    cy = rng.uniform(-0.5, 0.5, count)
    r = rng.uniform(0.02, 0.08, count)
    leta = rng.uniform(-3.0, 3.0, count)
    return cx, cy, r, leta


def stokes2d_inclusions(n=2048, dtype=np.float64, seed=3, eps=1e-8, ncheck=None, max_iter=None, re_m_pi=4.0) -> StokesProblem:
    T = np.dtype(dtype).type
    lx = ly = 1.0
    grid = UniformGrid(origin=(T(-lx / 2), T(-ly / 2)), extent=(T(lx), T(ly)), dims=(n, n), dtype=T)
    C, V = Center(), Vertex()
    # viscosity at cell centres, evaluated over the whole padded array
    x, y = padded_mesh(grid, C)
    eta = np.ones_like(x)
    for cx, cy, r, le in zip(*inclusions(seed)):
        eta[(x - cx) ** 2 + (y - cy) ** 2 < r * r] = 10.0**le
    erate = 1.0
    xv, _ = padded_mesh(grid, (V, C))
    _, yv = padded_mesh(grid, (C, V))
    Vx = (-erate * xv).astype(T)
    Vy = (erate * yv).astype(T)

    def zeros(loc):
        m = padded_mesh(grid, loc)[0]
        return np.zeros_like(m, dtype=T)

    tau_locs = [(C, C), (C, C), (V, V)]
    host = {
        "V": [Vx, Vy],
        "r_V": [zeros((V, C)), zeros((C, V))],
        "P": zeros(C),
        "divV": zeros(C),
        "tau": [zeros(l) for l in tau_locs],
        "tau_old": [zeros(l) for l in tau_locs],
        "eta": eta.astype(T),
    }
    G, dt = 1.0, 1e-2
    dx = float(min(grid.spacing()))
    re_m, r = re_m_pi * math.pi, 0.5
    lt = min(lx, ly) / re_m
    vdt = dx / math.sqrt(2 * 1.1)
    th = lt * (r + 4.0 / 3.0) / vdt
    params = stokes_params(eta=1.0, eta_ve=1.0 / (1.0 + 1.0 / (G * dt)), G=G, dt=dt, dtau_Pr=r / th, dtau_r=1.0 / (th + 1.0), nu_dtau=vdt * lt)
    bc_V = [
        to_cg_bc(2, {"x": (Dirichlet(erate * lx / 2), Dirichlet(-erate * lx / 2)), "y": Neumann()}),
        to_cg_bc(2, {"x": Neumann(), "y": (Dirichlet(-erate * ly / 2), Dirichlet(erate * ly / 2))}),
    ]
    eta_bg, psc = 1.0, G
    return StokesProblem(
        grid=grid,
        host=host,
        params=params,
        bc_V=bc_V,
        eps=eps,
        tau_scale=eta_bg / psc,
        v_scale=ly / psc,
        ncheck=ncheck or max(n // 4, 1),
        max_iter=max_iter or 200 * n,
    )


def ptdiff_params(grid: UniformGrid, dt: float, Dmax: float, lx: float | None = None):
    """Accelerated-PT parameters of the implicit diffusion step (one PT iteration damps the
    flux with omega_q and relaxes C with dtau_C): vdtau = min(Δ)/sqrt(N 1.1), Re = pi +
    sqrt(pi^2 + l^2/(D_max dt)), theta = l/(Re vdtau), beta = Re D_max/(vdtau l)."""
    from ._abi import cg_ptdiff_params

    nd = grid.ndim
    dx = float(min(grid.spacing()))
    l = float(lx if lx is not None else min(float(ax.extent) for ax in grid.axes))
    vdt = dx / math.sqrt(nd * 1.1)
    re = math.pi + math.sqrt(math.pi**2 + l * l / (Dmax * dt))
    th = l / (re * vdt)
    beta = re * Dmax / (vdt * l)
    p = cg_ptdiff_params()
    p.dt, p.omega_q, p.dtau_C = float(dt), 1.0 / (1.0 + th), 1.0 / (beta + 1.0 / dt)
    return p


def box_smooth(g: np.ndarray, passes: int = 5) -> np.ndarray:
    """`passes` sweeps of the 3-point box filter along every axis (periodic wrap)."""
    for _ in range(passes):
        for ax in range(g.ndim):
            g = (np.roll(g, 1, ax) + g + np.roll(g, -1, ax)) / 3.0
    return g


def ptdiff3d_blob(n=512, dtype=np.float64, seed=2, sigma=1.0, dt=1e-3, width=0.1):
    """3D variable-coefficient diffusion: D = exp(sigma g) per cell with g seeded Gaussian
    noise smoothed by 5 passes of a 3-point box filter; Dirichlet C = 0 on the x faces,
    Neumann elsewhere; C0 = Gaussian blob of width 0.1 on [-0.5, 0.5]^3."""
    T = np.dtype(dtype).type
    grid = UniformGrid(origin=(T(-0.5),) * 3, extent=(T(1),) * 3, dims=(n, n, n), dtype=T)
    C = Center()
    x, y, z = padded_mesh(grid, C)
    rng = np.random.default_rng(seed)
    g = box_smooth(rng.standard_normal(x.shape))
    D = np.exp(sigma * g).astype(T)
    C0 = np.exp(-(x * x + y * y + z * z) / (width * width)).astype(T)
    bc = to_cg_bc(3, {"x": Dirichlet(0.0), "y": Neumann(), "z": Neumann()})
    return grid, {"C": C0, "C_old": C0.copy(), "D": D}, bc, ptdiff_params(grid, dt, float(D.max()))


def gaussian_random_field(shape, corr_len, spacing, seed, std=1.0):
    """Seeded isotropic Gaussian random field with a Gaussian covariance of correlation length
    `corr_len` (FFT filtering of white noise), rescaled to zero mean and standard deviation
    `std`."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    ks = [np.fft.fftfreq(n, d=spacing) * 2.0 * math.pi for n in shape]
    K2 = sum(k**2 for k in np.meshgrid(*ks, indexing="ij", sparse=True))
    f = np.real(np.fft.ifftn(np.fft.fftn(w) * np.exp(-K2 * corr_len * corr_len / 4.0)))
    f -= f.mean()
    return f * (std / f.std())


def stokes3d_grf(n=256, dtype=np.float64, seed=4, eps=1e-8, ncheck=None, max_iter=None, re_m_pi=4.0):
    """3D VE Stokes (examples/stokes_3d_inc_ve_T.jl form) on [-0.5, 0.5]^3: log-viscosity a
    seeded Gaussian random field (correlation length 0.1, std 1), buoyancy rho_g.z = 1 in a
    sphere of radius 0.1 at the centre, free slip (normal velocity 0, tangential Neumann) on
    every face, G = 1, dt = 1e-2."""
    T = np.dtype(dtype).type
    lx = 1.0
    grid = UniformGrid(origin=(T(-lx / 2),) * 3, extent=(T(lx),) * 3, dims=(n, n, n), dtype=T)
    C, V = Center(), Vertex()
    x, y, z = padded_mesh(grid, C)
    g = gaussian_random_field(x.shape, 0.1, lx / n, seed)
    eta = np.exp(g).astype(T)
    zc = padded_mesh(grid, (C, C, V))
    rho_z = np.where(zc[0] ** 2 + zc[1] ** 2 + zc[2] ** 2 < 0.1**2, 1.0, 0.0).astype(T)

    def zeros(loc):
        return np.zeros_like(padded_mesh(grid, loc)[0], dtype=T)

    vlocs = [(V, C, C), (C, V, C), (C, C, V)]
    tlocs = [(C, C, C), (C, C, C), (C, C, C), (V, V, C), (V, C, V), (C, V, V)]
    host = {
        "V": [zeros(l) for l in vlocs],
        "r_V": [zeros(l) for l in vlocs],
        "P": zeros(C),
        "divV": zeros(C),
        "tau": [zeros(l) for l in tlocs],
        "tau_old": [zeros(l) for l in tlocs],
        "eta": eta,
        "rho_g": [None, None, rho_z],
    }
    G, dt = 1.0, 1e-2
    dx = float(min(grid.spacing()))
    re_m, r = re_m_pi * math.pi, 0.5
    lt = lx / re_m
    vdt = dx / math.sqrt(3 * 1.1)
    th = lt * (r + 4.0 / 3.0) / vdt
    params = stokes_params(eta=1.0, eta_ve=1.0 / (1.0 + 1.0 / (G * dt)), G=G, dt=dt, dtau_Pr=r / th, dtau_r=1.0 / (th + 1.0), nu_dtau=vdt * lt)
    bc_V = []
    for d in range(3):
        spec = {"xyz"[e]: (Dirichlet() if e == d else Neumann()) for e in range(3)}
        bc_V.append(to_cg_bc(3, spec))
    return StokesProblem(grid=grid, host=host, params=params, bc_V=bc_V, eps=eps, tau_scale=1.0, v_scale=lx,
                         ncheck=ncheck or max(n // 4, 1), max_iter=max_iter or 200 * n)


def sia_ensemble(members=64, seed=6, nmin=128, nmax=1024, dtype=np.float64, multiple=1):
    """Ensemble of independent SIA solves (examples/sia.jl form, flux -Gamma H^(n+2)|∇S|^(n-1)∇S,
    n = 3): member sizes n x n drawn uniformly from [nmin, nmax] (seed `seed`), bed = 0.4 + 0.3 x
    a smooth Gaussian random field (correlation length 0.25, seed 7 + k) on [-1, 1]^2, linear
    mass balance min(0.5 (S - ELA), 0.25) with ELA ~ U[0.3, 0.7] (seed 8), H0 = 0.
    Returns a list of (grid, {"H", "B"}, cg_sia_params)."""
    from ._abi import cg_sia_params

    T = np.dtype(dtype).type
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, members)
    if multiple > 1:
        sizes = (sizes // multiple) * multiple
    elas = np.random.default_rng(8).uniform(0.3, 0.7, members)
    out = []
    for k, n in enumerate(sizes):
        n = int(n)
        grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(n, n), dtype=T)
        x, _ = padded_mesh(grid, Center())
        bed = 0.4 + 0.3 * gaussian_random_field(x.shape, 0.25, 2.0 / n, 7 + k)
        p = cg_sia_params()
        p.Gamma, p.As, p.n, p.beta, p.ela, p.m_max, p.dt_max, p.cfl = 1.0, 0.0, 3, 0.5, float(elas[k]), 0.25, 0.5, 4.1
        out.append((grid, {"H": np.zeros_like(x, dtype=T), "B": bed.astype(T)}, p))
    return out
