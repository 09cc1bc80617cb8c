"""ctypes mirror of include/chmy_gb300.h and the loader of libchmy_gb300.so.

The descriptors (cg_field, cg_grid, cg_bc, cg_stokes_fields, ...) are plain C structs; the
same structs describe host arrays when the test-suite hands them to the CPU oracle.
"""

from __future__ import annotations

import ctypes as C
import os
import re
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "lib" / "libchmy_gb300.so"
HEADER = PKG_DIR.parent.parent / "include" / "chmy_gb300.h"

ABI_VERSION = 3

# status codes
CG_OK = 0
CG_ERR_ARG = 1
CG_ERR_CUDA = 2
CG_ERR_NONFINITE = 3
CG_ERR_TIMEOUT = 4
CG_ERR_UNSUPPORTED = 5
CG_ERR_NOCONV = 6

STATUS_NAMES = {
    CG_OK: "CG_OK",
    CG_ERR_ARG: "CG_ERR_ARG",
    CG_ERR_CUDA: "CG_ERR_CUDA",
    CG_ERR_NONFINITE: "CG_ERR_NONFINITE",
    CG_ERR_TIMEOUT: "CG_ERR_TIMEOUT",
    CG_ERR_UNSUPPORTED: "CG_ERR_UNSUPPORTED",
    CG_ERR_NOCONV: "CG_ERR_NOCONV",
}

CG_F32 = 1
CG_F64 = 2
CG_CENTER = 0
CG_VERTEX = 1
CG_BC_NONE = 0
CG_BC_DIRICHLET = 1
CG_BC_NEUMANN = 2
CG_BC_PERIODIC = 3


class cg_field(C.Structure):
    _fields_ = [
        ("data", C.c_void_p),
        ("dtype", C.c_int32),
        ("ndim", C.c_int32),
        ("n", C.c_int32 * 3),
        ("loc", C.c_int32 * 3),
        ("halo", C.c_int32 * 3),
        ("pad_", C.c_int32),
        ("stride", C.c_int64 * 3),
    ]


class cg_grid(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32),
        ("n", C.c_int32 * 3),
        ("origin", C.c_double * 3),
        ("extent", C.c_double * 3),
        ("spacing", C.c_double * 3),
        ("inv_spacing", C.c_double * 3),
    ]


class cg_bc(C.Structure):
    _fields_ = [("kind", (C.c_int32 * 2) * 3), ("value", (C.c_double * 2) * 3), ("values", (C.c_void_p * 2) * 3)]


class cg_mask(C.Structure):
    _fields_ = [("at", cg_field * 8)]


class cg_stokes_fields(C.Structure):
    _fields_ = [
        ("V", cg_field * 3),
        ("r_V", cg_field * 3),
        ("P", cg_field),
        ("divV", cg_field),
        ("tau", cg_field * 6),
        ("tau_old", cg_field * 6),
        ("eta", cg_field),
        ("inv_eta", cg_field),
        ("rho_g", cg_field * 3),
        ("T", cg_field),
        ("T_old", cg_field),
        ("qT", cg_field * 3),
    ]


CG_FN_NONE, CG_FN_CONST, CG_FN_BALL, CG_FN_AFFINE = 0, 1, 2, 3


class cg_function(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad_", C.c_int32), ("p", C.c_double * 8)]


class cg_bc_fn(C.Structure):
    _fields_ = [("fn", (cg_function * 2) * 3), ("full_dims", (C.c_int32 * 2) * 3)]


class cg_stokes_params(C.Structure):
    _fields_ = [
        ("eta", C.c_double),
        ("eta_ve", C.c_double),
        ("G", C.c_double),
        ("dt", C.c_double),
        ("dtau_Pr", C.c_double),
        ("dtau_r", C.c_double),
        ("nu_dtau", C.c_double),
        ("lambda_rhoCp", C.c_double),
        ("rho_g_fn", cg_function * 3),
    ]


class cg_solve_opts(C.Structure):
    _fields_ = [
        ("max_iter", C.c_int32),
        ("ncheck", C.c_int32),
        ("eps", C.c_double),
        ("tau_scale", C.c_double),
        ("v_scale", C.c_double),
        ("precision", C.c_int32),
        ("max_outer", C.c_int32),
        ("inner_rtol", C.c_double),
    ]


class cg_solve_result(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("outer", C.c_int32),
        ("checks", C.c_int32),
        ("converged", C.c_int32),
        ("err", C.c_double * 4),
        ("seconds", C.c_double),
        ("err_tau", C.c_double),
    ]


class cg_ptdiff_fields(C.Structure):
    _fields_ = [("C", cg_field), ("C_old", cg_field), ("D", cg_field), ("q", cg_field * 3), ("R", cg_field)]


class cg_ptdiff_params(C.Structure):
    _fields_ = [("dt", C.c_double), ("omega_q", C.c_double), ("dtau_C", C.c_double)]


class cg_sia_params(C.Structure):
    _fields_ = [
        ("Gamma", C.c_double),
        ("As", C.c_double),
        ("n", C.c_int32),
        ("pad_", C.c_int32),
        ("beta", C.c_double),
        ("ela", C.c_double),
        ("m_max", C.c_double),
        ("dt_max", C.c_double),
        ("cfl", C.c_double),
    ]


class cg_sia_member(C.Structure):
    _fields_ = [("grid", cg_grid), ("H", cg_field), ("B", cg_field), ("q", cg_field * 2)]


P = C.POINTER
_vp = C.c_void_p

# name -> argtypes (restype is int unless listed in _RESTYPES)
SIGNATURES: dict[str, list] = {
    "cg_abi_version": [],
    "cg_init": [C.c_int, P(_vp)],
    "cg_destroy": [_vp],
    "cg_last_error": [_vp],
    "cg_set_stream": [_vp, _vp],
    "cg_sync": [_vp],
    "cg_field_alloc": [_vp, C.c_int, C.c_int, P(C.c_int32), P(C.c_int32), P(C.c_int32), C.c_int, P(cg_field)],
    "cg_field_free": [_vp, P(cg_field)],
    "cg_field_upload": [_vp, P(cg_field), _vp],
    "cg_field_download": [_vp, P(cg_field), _vp],
    "cg_bc_apply": [_vp, P(cg_grid), C.c_int, P(cg_field), P(cg_bc)],
    "cg_bc_apply_fn": [_vp, P(cg_grid), C.c_int, P(cg_field), P(cg_bc), P(cg_bc_fn)],
    "cg_maxabs": [_vp, C.c_int, P(cg_field), P(C.c_double), P(C.c_int32)],
    "cg_maxabs_noalloc": [C.c_int, _vp, C.c_int, P(cg_field), P(C.c_double), P(C.c_int32)],
    "cg_diffusion_compute_q": [_vp, P(cg_grid), P(cg_field), P(cg_field), C.c_double],
    "cg_diffusion_update_C": [_vp, P(cg_grid), P(cg_field), P(cg_field), C.c_double],
    "cg_diffusion_step": [_vp, P(cg_grid), P(cg_field), P(cg_field), C.c_double, C.c_double, P(cg_bc)],
    "cg_diffusion_run": [_vp, P(cg_grid), P(cg_field), P(cg_field), C.c_double, C.c_double, P(cg_bc), C.c_int],
    "cg_diffusion_compute_q_masked": [_vp, P(cg_grid), P(cg_field), P(cg_field), C.c_double, P(cg_mask)],
    "cg_diffusion_update_C_masked": [_vp, P(cg_grid), P(cg_field), P(cg_field), C.c_double, P(cg_mask)],
    "cg_diffusion_run_masked": [_vp, P(cg_grid), P(cg_field), P(cg_field), C.c_double, C.c_double, P(cg_bc), P(cg_mask), C.c_int],
    "cg_diffusion_tape_bytes": [P(cg_grid), P(cg_field), C.c_int, P(C.c_size_t)],
    "cg_diffusion_run_taped": [_vp, P(cg_grid), P(cg_field), C.c_double, C.c_double, P(cg_bc), C.c_int, _vp, C.c_size_t],
    "cg_diffusion_adjoint_run": [_vp, P(cg_grid), _vp, C.c_size_t, P(cg_field), P(cg_field), C.c_double, C.c_double, P(cg_bc),
                                 P(C.c_double)],
    "cg_function_fill": [_vp, P(cg_grid), P(cg_function), P(cg_field)],
    "cg_fp64_peak": [_vp, P(C.c_double)],
    "cg_stokes_update_old": [_vp, P(cg_grid), P(cg_stokes_fields)],
    "cg_stokes_update_stress": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params)],
    "cg_stokes_update_velocity": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params)],
    "cg_stokes_update_thermal_flux": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params)],
    "cg_stokes_update_thermal": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params)],
    "cg_stokes_pt_iterations": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params), P(cg_bc), C.c_int],
    "cg_stokes_update_stress_masked": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params), P(cg_mask)],
    "cg_stokes_update_velocity_masked": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params), P(cg_mask)],
    "cg_stokes_pt_iterations_masked": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params), P(cg_bc), P(cg_mask),
                                       C.c_int],
    "cg_stokes_pt_iterations_pp": [
        _vp,
        P(cg_grid),
        P(cg_stokes_fields),
        P(cg_stokes_fields),
        P(cg_stokes_params),
        P(cg_bc),
        C.c_int,
    ],
    "cg_stokes_residual": [_vp, P(cg_grid), P(cg_stokes_fields), C.c_double, C.c_double, P(C.c_double)],
    "cg_stokes_solve": [
        _vp,
        P(cg_grid),
        P(cg_stokes_fields),
        P(cg_stokes_params),
        P(cg_bc),
        P(cg_solve_opts),
        P(cg_solve_result),
    ],
    "cg_stokes_gradient_log_eta": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_field), P(cg_stokes_params), P(cg_field)],
    "cg_stokes_thermal_step": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params), P(cg_bc), P(cg_field)],
    "cg_stokes_thermal_step_adjoint": [_vp, P(cg_grid), P(cg_stokes_fields), P(cg_stokes_params), P(cg_bc), P(cg_field), P(cg_field),
                                       P(cg_field), P(cg_field), P(C.c_double)],
    "cg_stokes_pt_iterations_thermal": [
        _vp,
        P(cg_grid),
        P(cg_stokes_fields),
        P(cg_stokes_params),
        P(cg_bc),
        P(cg_bc),
        C.c_int,
    ],
    "cg_stokes_solve_thermal": [
        _vp,
        P(cg_grid),
        P(cg_stokes_fields),
        P(cg_stokes_params),
        P(cg_bc),
        P(cg_bc),
        P(cg_solve_opts),
        P(cg_solve_result),
    ],
    "cg_ptdiff_update_q": [_vp, P(cg_grid), P(cg_ptdiff_fields), P(cg_ptdiff_params)],
    "cg_ptdiff_update_C": [_vp, P(cg_grid), P(cg_ptdiff_fields), P(cg_ptdiff_params)],
    "cg_ptdiff_gradient_D": [_vp, P(cg_grid), P(cg_field), P(cg_field), C.c_double, P(cg_field)],
    "cg_ptdiff_run": [_vp, P(cg_grid), P(cg_ptdiff_fields), P(cg_ptdiff_params), P(cg_bc), C.c_int, C.c_int],
    "cg_ptdiff_solve": [_vp, P(cg_grid), P(cg_ptdiff_fields), P(cg_ptdiff_params), P(cg_bc), P(cg_solve_opts), P(cg_solve_result)],
    "cg_sia_update_q": [_vp, P(cg_grid), P(cg_field), P(cg_field), P(cg_field), P(cg_sia_params), P(C.c_double)],
    "cg_sia_update_H": [_vp, P(cg_grid), P(cg_field), P(cg_field), P(cg_field), C.c_double, P(cg_sia_params)],
    "cg_sia_ensemble_run": [_vp, C.c_int, P(cg_sia_member), P(cg_sia_params), C.c_int, P(C.c_double)],
    "cg_sia_ensemble_tape_bytes": [C.c_int, P(cg_sia_member), C.c_int, P(C.c_size_t)],
    "cg_sia_ensemble_run_taped": [_vp, C.c_int, P(cg_sia_member), P(cg_sia_params), C.c_int, _vp, C.c_size_t, P(C.c_double)],
    "cg_sia_ensemble_adjoint_run": [_vp, C.c_int, P(cg_sia_member), P(cg_sia_params), _vp, C.c_size_t, P(cg_field), P(cg_field),
                                    P(C.c_double)],
    "cg_sia_adjoint_step": [_vp, P(cg_grid), P(cg_field), P(cg_field), P(cg_sia_params), P(cg_field), P(cg_field), P(C.c_double)],
    "cg_sia_run": [_vp, P(cg_grid), P(cg_field), P(cg_field), P(cg_field), P(cg_sia_params), C.c_int, P(C.c_double)],
    "cg_sia_tape_bytes": [P(cg_grid), P(cg_field), C.c_int, P(C.c_size_t)],
    "cg_sia_run_taped": [_vp, P(cg_grid), P(cg_field), P(cg_field), P(cg_field), P(cg_sia_params), C.c_int, _vp, C.c_size_t,
                         P(C.c_double)],
    "cg_sia_adjoint_run": [_vp, P(cg_grid), P(cg_sia_params), _vp, C.c_size_t, P(cg_field), P(cg_field), P(C.c_double)],
}
_RESTYPES = {"cg_last_error": C.c_char_p}


def header_symbols(path: Path = HEADER) -> list[str]:
    """Every entry point declared in include/chmy_gb300.h."""
    text = path.read_text()
    return sorted(set(re.findall(r"^CG_API\s+(?:int|const char\*)\s+(cg_\w+)\s*\(", text, flags=re.M)))


class ChmyError(RuntimeError):
    """A libchmy_gb300 call returned a non-zero status."""

    def __init__(self, code: int, fn: str, message: str):
        self.code = code
        self.fn = fn
        super().__init__(f"{fn}: {STATUS_NAMES.get(code, code)}: {message}")


_LIB: C.CDLL | None = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libchmy_gb300.so (built in-tree by chmy_gb300._build). Raises if it is missing:
    there is no fallback implementation."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"libchmy_gb300.so not found at {p}; build it with `python -c \"import __graft_entry__ as g; g.build()\"`"
        )
    lib = C.CDLL(str(p))
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = _RESTYPES.get(name, C.c_int)
    if lib.cg_abi_version() != ABI_VERSION:
        raise RuntimeError(f"libchmy_gb300 ABI version {lib.cg_abi_version()} != {ABI_VERSION}")
    if path is None:
        _LIB = lib
    return lib


def check(lib: C.CDLL, rc: int, fn: str, ctx=None) -> None:
    if rc != CG_OK:
        msg = lib.cg_last_error(ctx)
        raise ChmyError(rc, fn, msg.decode() if msg else "")


# ---- descriptor helpers -------------------------------------------------------------------


def make_field(
    ptr: int,
    dtype_code: int,
    n: tuple[int, ...],
    loc: tuple[int, ...],
    halo: tuple[int, ...],
    strides: tuple[int, ...],
) -> cg_field:
    """Build a cg_field for memory at `ptr` (start of the padded allocation)."""
    nd = len(n)
    f = cg_field()
    f.data = ptr
    f.dtype = dtype_code
    f.ndim = nd
    for d in range(3):
        f.n[d] = n[d] if d < nd else 1
        f.loc[d] = loc[d] if d < nd else 0
        f.halo[d] = halo[d] if d < nd else 0
        f.stride[d] = strides[d] if d < nd else 0
    f.pad_ = 0
    return f


def empty_field() -> cg_field:
    return cg_field()


def make_grid(n, origin, extent, spacing, inv_spacing) -> cg_grid:
    g = cg_grid()
    nd = len(n)
    g.ndim = nd
    for d in range(3):
        g.n[d] = n[d] if d < nd else 1
        g.origin[d] = float(origin[d]) if d < nd else 0.0
        g.extent[d] = float(extent[d]) if d < nd else 0.0
        g.spacing[d] = float(spacing[d]) if d < nd else 1.0
        g.inv_spacing[d] = float(inv_spacing[d]) if d < nd else 1.0
    return g
