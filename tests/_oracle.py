"""Test-side access to the CPU oracle (oracle/liboracle.so) and numpy-backed fields.

Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""

from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "chmy.jl_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

from chmy_gb300 import _abi  # noqa: E402
from chmy_gb300.grids import Center, UniformGrid, Vertex, expand_loc  # noqa: E402

import build as _oracle_build  # noqa: E402  (oracle/build.py)

P = C.POINTER
_vp = C.c_void_p
_SIGS = {
    "or_num_threads": ([], C.c_int),
    "or_set_threads": ([C.c_int], None),
    "or_bc_apply": ([P(_abi.cg_grid), C.c_int, P(_abi.cg_field), P(_abi.cg_bc)], C.c_int),
    "or_maxabs": ([C.c_int, P(_abi.cg_field), P(C.c_double), P(C.c_int32)], C.c_int),
    "or_diffusion_compute_q": ([P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), C.c_double], C.c_int),
    "or_diffusion_update_C": ([P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), C.c_double], C.c_int),
    "or_sia_run_tangent": ([P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_sia_params), C.c_int,
                            P(_abi.cg_field), P(_abi.cg_field)], C.c_int),
    "or_stokes_solve_tangent": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields), P(_abi.cg_stokes_params), P(_abi.cg_bc),
                                 P(_abi.cg_field), C.c_double, C.c_int, C.c_int, P(_abi.cg_field), P(C.c_int)], C.c_int),
    "or_ptdiff_run_tangent": ([P(_abi.cg_grid), P(_abi.cg_ptdiff_fields), P(_abi.cg_ptdiff_params), P(_abi.cg_bc), C.c_int, C.c_int,
                               P(_abi.cg_field), P(_abi.cg_field)], C.c_int),
    "or_diffusion_run_tangent": ([P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), C.c_double, C.c_double, P(_abi.cg_bc), C.c_int,
                                  P(_abi.cg_field), P(_abi.cg_field)], C.c_int),
    "or_thermal_step_tangent": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields), P(_abi.cg_stokes_params), P(_abi.cg_bc), P(_abi.cg_field),
                                 P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_field)], C.c_int),
    "or_function_fill": ([P(_abi.cg_grid), P(_abi.cg_function), P(_abi.cg_field)], C.c_int),
    "or_diffusion_compute_q_masked": ([P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), C.c_double, P(_abi.cg_mask)], C.c_int),
    "or_diffusion_update_C_masked": ([P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), C.c_double, P(_abi.cg_mask)], C.c_int),
    "or_stokes_update_old": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields)], C.c_int),
    "or_stokes_update_stress": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields), P(_abi.cg_stokes_params)], C.c_int),
    "or_stokes_update_velocity": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields), P(_abi.cg_stokes_params)], C.c_int),
    "or_stokes_update_stress_masked": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields), P(_abi.cg_stokes_params), P(_abi.cg_mask)],
                                       C.c_int),
    "or_stokes_update_velocity_masked": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields), P(_abi.cg_stokes_params), P(_abi.cg_mask)],
                                         C.c_int),
    "or_stokes_update_thermal_flux": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields), P(_abi.cg_stokes_params)], C.c_int),
    "or_stokes_update_thermal": ([P(_abi.cg_grid), P(_abi.cg_stokes_fields), P(_abi.cg_stokes_params)], C.c_int),
    "or_ptdiff_update_q": ([P(_abi.cg_grid), P(_abi.cg_ptdiff_fields), P(_abi.cg_ptdiff_params)], C.c_int),
    "or_ptdiff_update_C": ([P(_abi.cg_grid), P(_abi.cg_ptdiff_fields), P(_abi.cg_ptdiff_params)], C.c_int),
    "or_sia_update_q": (
        [P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_sia_params), P(C.c_double)],
        C.c_int,
    ),
    "or_sia_update_H": (
        [P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_field), C.c_double, P(_abi.cg_sia_params)],
        C.c_int,
    ),
    "or_op_kernel": (
        [C.c_int, P(_abi.cg_grid), P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_field), P(_abi.cg_field)],
        C.c_int,
    ),
}

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = _oracle_build.build()
        L = C.CDLL(str(path))
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


_CODE = {np.float32: _abi.CG_F32, np.float64: _abi.CG_F64}


class NpField:
    """Host field with Chmy's padded layout, stored [z, y, x] in a numpy array."""

    def __init__(self, grid: UniformGrid, loc, dtype=None, halo=1, fill=0.0):
        nd = grid.ndim
        self.grid = grid
        self.loc = expand_loc(nd, loc)
        self.dtype = np.dtype(dtype if dtype is not None else grid.dtype).type
        self.halo = tuple(halo for _ in range(nd)) if isinstance(halo, int) else tuple(halo)
        self.dims = grid.size(self.loc)
        self.ext = tuple(n + 4 * h for n, h in zip(self.dims, self.halo))
        self.a = np.full(tuple(reversed(self.ext)), fill, dtype=self.dtype)

    @property
    def ndim(self):
        return len(self.dims)

    def desc(self) -> _abi.cg_field:
        strides = tuple(s // self.a.itemsize for s in reversed(self.a.strides))
        return _abi.make_field(
            self.a.ctypes.data, _CODE[self.dtype], self.dims, tuple(l.code for l in self.loc), self.halo, strides
        )

    def at(self, *I):
        """Value at 1-based logical index I (x, y, z)."""
        idx = tuple(i + 2 * h - 1 for i, h in zip(I, self.halo))
        return self.a[tuple(reversed(idx))]

    def interior(self, with_halo=False) -> np.ndarray:
        sl = []
        for n, h in zip(reversed(self.dims), reversed(self.halo)):
            lo = 2 * h - (h if with_halo else 0)
            hi = 2 * h + n + (h if with_halo else 0)
            sl.append(slice(lo, hi))
        return self.a[tuple(sl)].transpose(*reversed(range(self.ndim)))

    def copy(self) -> "NpField":
        g = NpField.__new__(NpField)
        g.__dict__.update(self.__dict__)
        g.a = self.a.copy()
        return g


def vec_fields(grid, dtype=None, fill=0.0):
    nd = grid.ndim
    return [NpField(grid, tuple(Vertex() if i == d else Center() for i in range(nd)), dtype, fill=fill) for d in range(nd)]


def tensor_fields(grid, dtype=None, fill=0.0):
    C_, V_ = Center(), Vertex()
    if grid.ndim == 2:
        locs = [(C_, C_), (C_, C_), (V_, V_)]
    else:
        locs = [(C_, C_, C_), (C_, C_, C_), (C_, C_, C_), (V_, V_, C_), (V_, C_, V_), (C_, V_, V_)]
    return [NpField(grid, l, dtype, fill=fill) for l in locs]


def desc_array(fields, n=None):
    n = n or max(len(fields), 1)
    arr = (_abi.cg_field * n)()
    for i, f in enumerate(fields):
        if f is not None:
            arr[i] = f.desc()
    return arr


def stokes_desc(V=None, r_V=None, P=None, divV=None, tau=None, tau_old=None, eta=None, inv_eta=None, rho_g=None, T=None, T_old=None, qT=None):
    s = _abi.cg_stokes_fields()
    if V is not None:
        s.V = desc_array(V, 3)
    if r_V is not None:
        s.r_V = desc_array(r_V, 3)
    if P is not None:
        s.P = P.desc()
    if divV is not None:
        s.divV = divV.desc()
    if tau is not None:
        s.tau = desc_array(tau, 6)
    if tau_old is not None:
        s.tau_old = desc_array(tau_old, 6)
    if eta is not None:
        s.eta = eta.desc()
    if inv_eta is not None:
        s.inv_eta = inv_eta.desc()
    if rho_g is not None:
        s.rho_g = desc_array(rho_g, 3)
    if T is not None:
        s.T = T.desc()
    if T_old is not None:
        s.T_old = T_old.desc()
    if qT is not None:
        s.qT = desc_array(qT, 3)
    return s


def bc_apply(grid, fields, bcs):
    g = grid.desc()
    fa = desc_array(fields)
    ba = (_abi.cg_bc * len(bcs))(*bcs)
    rc = lib().or_bc_apply(C.byref(g), len(fields), fa, ba)
    assert rc == 0


def op(opcode, grid, Cf=None, C1=None, C2=None, V=None, chi=None):
    g = grid.desc()

    def ref(f):
        return C.byref(f.desc()) if f is not None else None

    Va = desc_array(V, 3) if V is not None else None
    rc = lib().or_op_kernel(opcode, C.byref(g), ref(Cf), ref(C1), ref(C2), Va, ref(chi))
    assert rc == 0


def stokes_problem_fields(pb):
    """Host NpFields (FP64) of a StokesProblem's initial state, for the oracle: a dict with
    V, r_V, tau, tau_old (lists), P, divV, eta and rho_g (list, None where absent), and the
    cg_stokes_fields over them under "desc"."""
    grid = pb.grid
    nd = grid.ndim
    Cl, Vl = Center(), Vertex()
    vlocs = [tuple(Vl if e == d else Cl for e in range(nd)) for d in range(nd)]
    if nd == 2:
        tlocs = [(Cl, Cl), (Cl, Cl), (Vl, Vl)]
    else:
        tlocs = [(Cl, Cl, Cl)] * 3 + [(Vl, Vl, Cl), (Vl, Cl, Vl), (Cl, Vl, Vl)]

    def nf(loc, arr):
        f = NpField(grid, loc, np.float64)
        f.a[...] = arr
        return f

    h = pb.host
    out = {
        "V": [nf(l, a) for l, a in zip(vlocs, h["V"])],
        "r_V": [nf(l, a) for l, a in zip(vlocs, h["r_V"])],
        "tau": [nf(l, a) for l, a in zip(tlocs, h["tau"])],
        "tau_old": [nf(l, a) for l, a in zip(tlocs, h["tau_old"])],
        "P": nf(Cl, h["P"]),
        "divV": nf(Cl, h["divV"]),
        "eta": nf(Cl, h["eta"]),
        "rho_g": [None if a is None else nf(l, a) for l, a in zip(vlocs, list(h.get("rho_g", [])) + [None] * nd)],
    }
    rho = out["rho_g"] if any(r is not None for r in out["rho_g"]) else None
    s = stokes_desc(V=out["V"], r_V=out["r_V"], P=out["P"], divV=out["divV"], tau=out["tau"], tau_old=out["tau_old"],
                    eta=out["eta"])
    if rho is not None:
        for d, r in enumerate(rho):
            if r is not None:
                s.rho_g[d] = r.desc()
    out["desc"] = s
    out["vlocs"] = vlocs
    return out


def stokes_tangent_solve(pb, dirs, tol=1e-11, max_iter=400000, ncheck=100):
    """or_stokes_solve_tangent on pb's initial state along the two log-viscosity directions
    `dirs` (host arrays of eta's padded shape). Returns (fields dict with the converged value,
    tangents [k][d] as padded arrays, iterations)."""
    grid = pb.grid
    nd = grid.ndim
    fs = stokes_problem_fields(pb)
    dfields = []
    for a in dirs:
        f = NpField(grid, Center(), np.float64)
        f.a[...] = a
        dfields.append(f)
    dV = [NpField(grid, fs["vlocs"][d], np.float64) for _ in range(2) for d in range(nd)]
    it = C.c_int()
    bcs = (_abi.cg_bc * nd)(*pb.bc_V)
    rc = lib().or_stokes_solve_tangent(C.byref(grid.desc()), C.byref(fs["desc"]), C.byref(pb.params), bcs,
                                       desc_array(dfields), tol, max_iter, ncheck, desc_array(dV), C.byref(it))
    assert rc == 0, (rc, it.value)
    return fs, [[dV[k * nd + d].a for d in range(nd)] for k in range(2)], it.value


def ptdiff_tangent_run(grid, D, C0, params, bc, nsteps, npt, dirs):
    """or_ptdiff_run_tangent from C0 (flux starting at zero) with diffusivity D (host arrays,
    FP64, padded) along the two log-D directions `dirs`. Returns (C^N, [dC^N/d eps_k])."""
    nd = grid.ndim
    Cl, Vl = Center(), Vertex()

    def nf(loc, arr=None):
        f = NpField(grid, loc, np.float64)
        if arr is not None:
            f.a[...] = arr
        return f

    Cf, Co, Df = nf(Cl, C0), nf(Cl, C0), nf(Cl, D)
    q = [nf(tuple(Vl if e == d else Cl for e in range(nd))) for d in range(nd)]
    fs = _abi.cg_ptdiff_fields()
    fs.C, fs.C_old, fs.D = Cf.desc(), Co.desc(), Df.desc()
    fs.q = desc_array(q, 3)
    dfields = [nf(Cl, a) for a in dirs]
    dC = [nf(Cl), nf(Cl)]
    rc = lib().or_ptdiff_run_tangent(C.byref(grid.desc()), C.byref(fs), C.byref(params), C.byref(bc), int(nsteps), int(npt),
                                     desc_array(dfields), desc_array(dC))
    assert rc == 0, rc
    return Cf.a.copy(), [d.a.copy() for d in dC]


def diffusion_tangent_run(grid, C0, chi, dt, bc, nsteps, direction):
    """or_diffusion_run_tangent from C0 (FP64 padded host array; bc! is applied first): the
    explicit diffusion loop's final state and its derivatives along chi and along the
    initial-state direction `direction` (a padded host array). Returns (C^N, dC^N/dchi,
    dC^N/d direction)."""
    nd = grid.ndim
    Cl, Vl = Center(), Vertex()
    Cf = NpField(grid, Cl, np.float64)
    Cf.a[...] = C0
    w = NpField(grid, Cl, np.float64)
    w.a[...] = direction
    q = [NpField(grid, tuple(Vl if e == d else Cl for e in range(nd)), np.float64) for d in range(nd)]
    dC = [NpField(grid, Cl, np.float64), NpField(grid, Cl, np.float64)]
    rc = lib().or_diffusion_run_tangent(C.byref(grid.desc()), C.byref(Cf.desc()), desc_array(q, 3), float(chi), float(dt),
                                        C.byref(bc), int(nsteps), C.byref(w.desc()), desc_array(dC))
    assert rc == 0, rc
    return Cf.a.copy(), dC[0].a.copy(), dC[1].a.copy()


def diffusion_run(grid, C0, chi, dt, bc, nsteps):
    """The oracle's explicit diffusion loop (compute_q!, update_C!, bc!) from bc!(C0): C^N."""
    nd = grid.ndim
    Cl, Vl = Center(), Vertex()
    Cf = NpField(grid, Cl, np.float64)
    Cf.a[...] = C0
    q = [NpField(grid, tuple(Vl if e == d else Cl for e in range(nd)), np.float64) for d in range(nd)]
    g = grid.desc()
    bc_apply(grid, [Cf], [bc])
    for _ in range(nsteps):
        assert lib().or_diffusion_compute_q(C.byref(g), desc_array(q, 3), C.byref(Cf.desc()), float(chi)) == 0
        assert lib().or_diffusion_update_C(C.byref(g), C.byref(Cf.desc()), desc_array(q, 3), float(dt)) == 0
        bc_apply(grid, [Cf], [bc])
    return Cf.a.copy()


def thermal_problem(grid, seed, bc_T):
    """Host fields of one thermal step: T (random, bc_T applied), T_old, V (random at every face),
    zero flux storage qT, and random tangent directions of T (interior), T_old (interior) and V
    (every face). Returns a dict of NpFields and direction arrays."""
    nd = grid.ndim
    Cl, Vl = Center(), Vertex()
    rng = np.random.default_rng(seed)
    vlocs = [tuple(Vl if e == d else Cl for e in range(nd)) for d in range(nd)]
    Tf = NpField(grid, Cl, np.float64)
    Tf.a[...] = 1.0 + rng.standard_normal(Tf.a.shape)
    bc_apply(grid, [Tf], [bc_T])
    To = NpField(grid, Cl, np.float64)
    To.a[...] = rng.standard_normal(To.a.shape)
    V = [NpField(grid, l, np.float64) for l in vlocs]
    for v in V:
        v.a[...] = rng.standard_normal(v.a.shape)
    inner = (slice(2, -2),) * nd
    dT = np.zeros_like(Tf.a)
    dT[inner] = rng.standard_normal(dT[inner].shape)
    dTo = np.zeros_like(To.a)
    dTo[inner] = rng.standard_normal(dTo[inner].shape)
    dV = [rng.standard_normal(v.a.shape) for v in V]
    mu = np.zeros_like(Tf.a)
    mu[inner] = rng.standard_normal(mu[inner].shape)
    return {"T": Tf, "T_old": To, "V": V, "vlocs": vlocs, "dT": dT, "dT_old": dTo, "dV": dV, "mu": mu, "inner": inner}


def thermal_tangent_step(grid, pr, params, bc_T):
    """or_thermal_step_tangent on copies of a thermal_problem: (T_out, [dT_out along the
    directions, dT_out / d lambda_rhoCp])."""
    nd = grid.ndim
    T = pr["T"].copy()
    To = pr["T_old"].copy()
    V = [v.copy() for v in pr["V"]]
    qT = [NpField(grid, l, np.float64) for l in pr["vlocs"]]
    s = stokes_desc(V=V, T=T, T_old=To, qT=qT)

    def nf(arr, loc):
        f = NpField(grid, loc, np.float64)
        f.a[...] = arr
        return f

    dT = nf(pr["dT"], Center())
    dTo = nf(pr["dT_old"], Center())
    dV = [nf(a, l) for a, l in zip(pr["dV"], pr["vlocs"])]
    out = [NpField(grid, Center(), np.float64), NpField(grid, Center(), np.float64)]
    rc = lib().or_thermal_step_tangent(C.byref(grid.desc()), C.byref(s), C.byref(params), C.byref(bc_T), C.byref(dT.desc()),
                                       C.byref(dTo.desc()), desc_array(dV, 3), desc_array(out))
    assert rc == 0, rc
    return T.a.copy(), [out[0].a.copy(), out[1].a.copy()]


def thermal_step(grid, T0, T_old, V, params, bc_T):
    """The oracle's plain thermal step (update_thermal_flux!, update_thermal!, bc!(T)) on host
    arrays: T_out."""
    nd = grid.ndim
    Cl, Vl = Center(), Vertex()
    vlocs = [tuple(Vl if e == d else Cl for e in range(nd)) for d in range(nd)]

    def nf(arr, loc):
        f = NpField(grid, loc, np.float64)
        f.a[...] = arr
        return f

    T = nf(T0, Cl)
    To = nf(T_old, Cl)
    Vf = [nf(a, l) for a, l in zip(V, vlocs)]
    qT = [NpField(grid, l, np.float64) for l in vlocs]
    s = stokes_desc(V=Vf, T=T, T_old=To, qT=qT)
    g = grid.desc()
    bc_apply(grid, [T], [bc_T])
    assert lib().or_stokes_update_thermal_flux(C.byref(g), C.byref(s), C.byref(params)) == 0
    assert lib().or_stokes_update_thermal(C.byref(g), C.byref(s), C.byref(params)) == 0
    bc_apply(grid, [T], [bc_T])
    return T.a.copy()
