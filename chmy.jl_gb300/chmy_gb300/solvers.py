"""Device-resident PT solvers over the library (the PT loops of the reference examples).

StokesSolver holds a VE Stokes field set on the GPU and runs the PT loop of
examples/stokes_2d_inc_ve_T.jl:144-163 through the library: graph-replayed chunks of
`ncheck` iterations (update_stress!, update_velocity!, bc!(V)), then the convergence
measures of :154-157, until every measure is below eps.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from .configs import StokesProblem
from .fields import Field
from .functions import FunctionField
from .grids import Center, Vertex
from .kernels import stokes_fields


def _loc_of(arr_name: str, idx: int, nd: int):
    C, V = Center(), Vertex()
    if arr_name in ("V", "r_V", "rho_g", "qT"):
        return tuple(V if d == idx else C for d in range(nd))
    if arr_name in ("tau", "tau_old"):
        if nd == 2:
            return [(C, C), (C, C), (V, V)][idx]
        return [(C, C, C), (C, C, C), (C, C, C), (V, V, C), (V, C, V), (C, V, V)][idx]
    return tuple(C for _ in range(nd))


class StokesSolver:
    """VE Stokes state on the device plus the library's PT entry points."""

    def __init__(self, arch, problem: StokesProblem, pitch_align: int = 0, precompute_inv_eta: bool = True):
        self.arch = arch
        self.pb = problem
        g = problem.grid
        nd = g.ndim
        self.fields: dict = {}
        # body forces given as device FunctionFields are evaluated by the kernels, not stored
        self.params = _abi.cg_stokes_params()
        ctypes.memmove(ctypes.byref(self.params), ctypes.byref(problem.params), ctypes.sizeof(self.params))
        for name, val in problem.host.items():
            if isinstance(val, list):
                fs = []
                for i, a in enumerate(val):
                    if isinstance(a, FunctionField):
                        if name != "rho_g":
                            raise TypeError(f"{name}[{i}]: only body forces may be FunctionFields")
                        self.params.rho_g_fn[i] = a.desc()
                        a = None
                    if a is None:
                        fs.append(None)
                        continue
                    f = Field(arch, g, _loc_of(name, i, nd), a.dtype.type, pitch_align=pitch_align)
                    f.from_numpy(a)
                    fs.append(f)
                self.fields[name] = fs
            else:
                f = Field(arch, g, _loc_of(name, 0, nd), val.dtype.type, pitch_align=pitch_align)
                f.from_numpy(val)
                self.fields[name] = f
        if precompute_inv_eta and "eta" in self.fields:
            # 1/eta is an input of the kernels: prepared on the host, uploaded like eta
            inv = Field(arch, g, Center(), self.fields["eta"].dtype, pitch_align=pitch_align)
            inv.from_numpy(1.0 / np.asarray(problem.host["eta"]))
            self.fields["inv_eta"] = inv
        self.desc = stokes_fields(**self.fields)
        self.grid_desc = g.desc()
        self.bc_arr = (_abi.cg_bc * 3)(*problem.bc_V)
        self.iterations = 0

    def upload(self, host: dict) -> None:
        """Copy host arrays (same layout as problem.host) into the device fields."""
        for name, val in host.items():
            if isinstance(val, list):
                for f, a in zip(self.fields[name], val):
                    if f is not None and a is not None:
                        f.data.copy_(a if not isinstance(a, np.ndarray) else __import__("torch").from_numpy(a), non_blocking=True)
            else:
                f = self.fields[name]
                f.data.copy_(val if not isinstance(val, np.ndarray) else __import__("torch").from_numpy(val), non_blocking=True)

    def iterate(self, niter: int) -> None:
        """`niter` PT iterations (one CUDA graph replay)."""
        self.arch.call(
            "cg_stokes_pt_iterations",
            ctypes.byref(self.grid_desc),
            ctypes.byref(self.desc),
            ctypes.byref(self.params),
            self.bc_arr,
            int(niter),
        )
        self.iterations += niter

    def residual(self) -> list[float]:
        err = (ctypes.c_double * 4)()
        self.arch.call(
            "cg_stokes_residual",
            ctypes.byref(self.grid_desc),
            ctypes.byref(self.desc),
            float(self.pb.tau_scale),
            float(self.pb.v_scale),
            err,
        )
        return [err[i] for i in range(self.pb.grid.ndim + 1)]

    def solve(self, max_iter: int | None = None, precision: int = _abi.CG_F64, max_outer: int = 8, inner_rtol: float = 1e-5):
        o = _abi.cg_solve_opts()
        o.max_iter = int(max_iter or self.pb.max_iter)
        o.ncheck = int(self.pb.ncheck)
        o.eps = float(self.pb.eps)
        o.tau_scale = float(self.pb.tau_scale)
        o.v_scale = float(self.pb.v_scale)
        o.precision = precision
        o.max_outer = max_outer
        o.inner_rtol = inner_rtol
        res = _abi.cg_solve_result()
        rc = self.arch.lib.cg_stokes_solve(
            self.arch.ctx,
            ctypes.byref(self.grid_desc),
            ctypes.byref(self.desc),
            ctypes.byref(self.params),
            self.bc_arr,
            ctypes.byref(o),
            ctypes.byref(res),
        )
        if rc not in (_abi.CG_OK, _abi.CG_ERR_NOCONV):
            _abi.check(self.arch.lib, rc, "cg_stokes_solve", self.arch.ctx)
        return res

    def gradient_log_eta(self, dJdV, precision: int = _abi.CG_F64, eps: float | None = None, max_iter: int | None = None):
        """dJ/d log(eta) at every cell for a misfit J(V) of the converged state this solver holds
        (call solve() first). `dJdV` lists per velocity component a padded host array, or None.

        The adjoint velocity solves the same Stokes problem (the discrete operator is
        symmetric): body force -dJ/dV, tau_old = 0, zero initial state and the forward's
        boundary-condition kinds with zero values, by cg_stokes_solve in `precision`. The
        library then forms the gradient from the adjoint velocity and the forward stress
        (cg_stokes_gradient_log_eta). Returns (grad Field, adjoint solve result)."""
        import dataclasses

        pb = self.pb
        g = pb.grid
        nd = g.ndim
        if "eta" not in pb.host:
            raise ValueError("gradient_log_eta: the problem needs a viscosity field")
        zero = {}
        for name, val in pb.host.items():
            if name in ("eta", "T", "T_old", "qT", "rho_g"):
                continue
            if isinstance(val, list):
                zero[name] = [None if a is None else np.zeros_like(a) for a in val]
            else:
                zero[name] = np.zeros_like(val)
        zero["eta"] = pb.host["eta"]
        ref = pb.host["V"]
        zero["rho_g"] = [None if a is None else -np.asarray(a, dtype=ref[d].dtype) for d, a in enumerate(list(dJdV) + [None] * (3 - len(dJdV)))][:nd]
        # the adjoint's body force is -dJ/dV alone: the forward's body-force functions drop out
        adj_params = _abi.cg_stokes_params()
        ctypes.memmove(ctypes.byref(adj_params), ctypes.byref(self.params), ctypes.sizeof(adj_params))
        for d in range(3):
            adj_params.rho_g_fn[d] = _abi.cg_function()
        bcs = []
        for b in pb.bc_V:
            b0 = _abi.cg_bc()
            ctypes.memmove(ctypes.byref(b0), ctypes.byref(b), ctypes.sizeof(b0))
            for d in range(3):
                for side in range(2):
                    b0.value[d][side] = 0.0
            bcs.append(b0)
        adj_pb = dataclasses.replace(pb, host=zero, bc_V=bcs, eps=float(eps if eps is not None else pb.eps), params=adj_params)
        adj = StokesSolver(self.arch, adj_pb)
        adj.apply_bc()
        res = adj.solve(precision=precision, max_iter=max_iter)
        grad = Field(self.arch, g, Center(), self.fields["eta"].dtype)
        mu = (_abi.cg_field * 3)(*[f.desc() for f in adj.fields["V"]])
        self.arch.call(
            "cg_stokes_gradient_log_eta",
            ctypes.byref(self.grid_desc),
            ctypes.byref(self.desc),
            mu,
            ctypes.byref(self.params),
            ctypes.byref(grad.desc()),
        )
        return grad, res

    def apply_bc(self) -> None:
        fa = (_abi.cg_field * 3)(*[f.desc() for f in self.fields["V"]])
        self.arch.call("cg_bc_apply", ctypes.byref(self.grid_desc), self.pb.grid.ndim, fa, self.bc_arr)
