"""The CPU oracle against the known answers of Chmy.jl's own test-suite.

Ports test/test_grids.jl, test_fields.jl, test_grid_operators.jl, test_interpolations.jl
and test_boundary_conditions.jl (TEST_TYPES = [Float32, Float64], test/common.jl:9).
"""

import json
import math
from pathlib import Path

import numpy as np
import pytest

from _oracle import NpField, bc_apply, op, tensor_fields, vec_fields
from chmy_gb300 import _abi
from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
from chmy_gb300.fields import evaluate
from chmy_gb300.grids import Center, UniformGrid, Vertex

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())
TYPES = [np.float32, np.float64]


def approx(a, b, T):
    tol = 1e-5 if T == np.float32 else 1e-12
    return np.allclose(np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64), rtol=tol, atol=tol)


# ---- test/test_grids.jl -----------------------------------------------------------------------


@pytest.mark.parametrize("T", TYPES)
def test_grid_kats(T):
    g = KATS["grids"]
    nx, ny = g["nx"], g["ny"]
    grid = UniformGrid(origin=tuple(T(o) for o in g["origin"]), extent=tuple(T(e) for e in g["extent"]), dims=(nx, ny), dtype=T)
    assert grid.size(Center()) == (nx, ny)
    assert grid.size(Vertex()) == (nx + 1, ny + 1)
    assert grid.size((Center(), Vertex())) == (nx, ny + 1)
    assert grid.size((Vertex(), Center())) == (nx + 1, ny)
    locs = {"Vertex": Vertex(), "Center": Center()}
    for case in g["cases"]:
        loc, dim = locs[case["loc"]], case["dim"]
        fn = case["fn"]
        if fn == "bounds":
            got = grid.bounds(loc, dim)
        elif fn == "extent":
            got = grid.extent(loc, dim)
        elif fn == "origin":
            got = grid.origin(loc, dim)
        elif fn == "spacing":
            got = grid.spacing()[dim - 1]
        elif fn == "inv_spacing":
            got = grid.inv_spacing()[dim - 1]
        else:
            idx = eval(case["index"], {"nx": nx, "ny": ny})
            got = grid.coord(loc, dim, idx)
        assert approx(got, case["expected"], T), (case, got)
    assert grid.dtype == T


# ---- test/test_fields.jl ------------------------------------------------------------------------


@pytest.mark.parametrize("T", TYPES)
def test_field_set_kats(T):
    f = KATS["fields"]
    grid = UniformGrid(origin=(T(0),) * 3, extent=(T(1),) * 3, dims=(2, 2, 2), dtype=T)
    loc = (Center(), Vertex(), Center())
    dims = grid.size(loc)
    assert dims == (2, 3, 2)
    funs = [
        (lambda g, l, ix, iy, iz: g.coord(l, 2, iy), True, ()),
        (lambda g, l, ix, iy, iz: g.coord(l, 1, ix), True, ()),
        (lambda g, l, ix, iy, iz, sc: g.coord(l, 2, iy) * sc, True, (T(2.0),)),
        (lambda x, y, z: y, False, ()),
        (lambda x, y, z: x, False, ()),
        (lambda x, y, z, sc: y * sc, False, (T(2.0),)),
    ]
    for (fun, discrete, params), case in zip(funs, f["cases"]):
        got = evaluate(grid, loc, dims, fun, discrete, params, T)
        want = np.array(case["array_zyx"]).transpose(2, 1, 0)  # -> [x, y, z]
        assert np.array_equal(got, want.astype(T)), (case["line"], got, want)


# ---- test/test_grid_operators.jl ------------------------------------------------------------------


def _gauss(grid, f):
    val = evaluate(grid, f.loc, f.dims, lambda x, y, z: np.exp(-x**2 - y**2 - z**2), False, (), f.dtype)
    f.interior()[...] = val


@pytest.mark.parametrize("T", TYPES)
def test_divg_lapl_identities(T):
    grid = UniformGrid(origin=(T(-5),) * 3, extent=(T(10),) * 3, dims=(12, 10, 8), dtype=T)
    Ci, C1, C2 = (NpField(grid, Center()) for _ in range(3))
    V = vec_fields(grid)
    _gauss(grid, Ci)
    op(0, grid, Cf=Ci, V=V)  # divg1!
    op(1, grid, C1=C1, C2=C2, V=V)  # divg2!
    assert np.array_equal(C1.interior(), C2.interior())
    # independent restatement: V.x[i] = (C[i] - C[i-1]) * iΔx over i in 0..n+1
    a = Ci.a
    idx = grid.inv_spacing()
    vx = V[0].a  # [z, y, x] with halo 1: logical i at index i+1
    ref = (a[1:-1, 1:-1, 1:-1] - a[1:-1, 1:-1, :-2]) * idx[0]
    assert np.array_equal(vx[1:-1, 1:-1, 1:-2], ref.astype(T))
    C1.a[...] = 0
    C2.a[...] = 0
    op(2, grid, Cf=Ci, C1=C1, C2=C2)  # lapl!
    assert np.array_equal(C1.interior(), C2.interior())
    # ∂²x at Center: ((C[i+1]-C[i])iΔ - (C[i]-C[i-1])iΔ) iΔ
    c = a.astype(np.float64)
    lx = ((c[2:-2, 2:-2, 3:-1] - c[2:-2, 2:-2, 2:-2]) * idx[0] - (c[2:-2, 2:-2, 2:-2] - c[2:-2, 2:-2, 1:-3]) * idx[0]) * idx[0]
    ly = ((c[2:-2, 3:-1, 2:-2] - c[2:-2, 2:-2, 2:-2]) * idx[1] - (c[2:-2, 2:-2, 2:-2] - c[2:-2, 1:-3, 2:-2]) * idx[1]) * idx[1]
    lz = ((c[3:-1, 2:-2, 2:-2] - c[2:-2, 2:-2, 2:-2]) * idx[2] - (c[2:-2, 2:-2, 2:-2] - c[1:-3, 2:-2, 2:-2]) * idx[2]) * idx[2]
    assert approx(C1.interior().transpose(2, 1, 0), lx + ly + lz, T)


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("chi_loc", ["center", "vertex"])
def test_divg_grad_identity(T, chi_loc):
    grid = UniformGrid(origin=(T(-5),) * 3, extent=(T(10),) * 3, dims=(12, 10, 8), dtype=T)
    Ci, C1, C2 = (NpField(grid, Center()) for _ in range(3))
    chi = NpField(grid, Center() if chi_loc == "center" else Vertex())
    V = vec_fields(grid)
    _gauss(grid, Ci)
    _gauss(grid, chi)
    op(3, grid, Cf=Ci, V=V, chi=chi)  # divg_grad1!
    op(4, grid, Cf=Ci, C1=C1, C2=C2, V=V, chi=chi)  # divg_grad2!
    # the reference asserts ≈ (test_grid_operators.jl:98,110)
    assert approx(C1.interior(), C2.interior(), T)


@pytest.mark.parametrize("T", TYPES)
def test_vmag_kat(T):
    grid = UniformGrid(origin=(T(-5),) * 3, extent=(T(10),) * 3, dims=(12, 10, 8), dtype=T)
    V = vec_fields(grid)
    for v in V:
        v.interior()[...] = T(KATS["vmag"]["value"])
    C1 = NpField(grid, Center())
    op(5, grid, C1=C1, V=V)
    got = C1.interior().astype(np.float64)
    rounded = np.vectorize(lambda x: float(f"{x:.5g}"))(got)
    assert np.all(np.isclose(rounded, KATS["vmag"]["expected_sigdigits5"]))


# ---- test/test_interpolations.jl ------------------------------------------------------------------


def av4(A):
    return 0.25 * (A[:-1, :-1] + A[1:, :-1] + A[1:, 1:] + A[:-1, 1:])


def avx(A):
    return 0.5 * (A[:-1, :] + A[1:, :])


def avy(A):
    return 0.5 * (A[:, :-1] + A[:, 1:])


@pytest.mark.parametrize("T", TYPES)
def test_interpolation_kats(T):
    grid = UniformGrid(origin=(T(0), T(0)), extent=(T(1), T(1)), dims=(2, 2), dtype=T)
    C_, V_ = Center(), Vertex()
    f_c = NpField(grid, C_)
    f_c.interior()[...] = np.arange(1, 5).reshape(2, 2, order="F")
    fci = f_c.interior().astype(np.float64)

    def lerp_to(src, loc):
        dst = NpField(grid, loc)
        op(6, grid, Cf=src, C1=dst)
        return dst.interior().astype(np.float64)

    assert np.allclose(lerp_to(f_c, (V_, V_))[1:-1, 1:-1], av4(fci))
    assert np.allclose(lerp_to(f_c, (C_, C_)), fci)
    assert np.allclose(lerp_to(f_c, (C_, V_))[:, 1:-1], avy(fci))
    assert np.allclose(lerp_to(f_c, (V_, C_))[1:-1, :], avx(fci))
    f_v = NpField(grid, V_)
    f_v.interior()[...] = np.arange(1, 10).reshape(3, 3, order="F")
    fvi = f_v.interior().astype(np.float64)
    assert np.allclose(lerp_to(f_v, (C_, C_)), av4(fvi))
    assert np.allclose(lerp_to(f_v, (V_, V_)), fvi)
    assert np.allclose(lerp_to(f_v, (C_, V_)), avx(fvi))
    assert np.allclose(lerp_to(f_v, (V_, C_)), avy(fvi))


def test_harmonic_rule():
    # hlerp rule: 1/(1/a + t(1/b - 1/a)) (interpolation.jl:211,297)
    grid = UniformGrid(origin=(0.0,), extent=(1.0,), dims=(4,))
    f = NpField(grid, Center())
    f.interior()[...] = [1.0, 3.0, 2.0, 5.0]
    dst = NpField(grid, Vertex())
    op(7, grid, Cf=f, C1=dst)
    got = dst.interior()[1:-1]
    want = [1 / (0.5 * (1 / 1 + 1 / 3)), 1 / (0.5 * (1 / 3 + 1 / 2)), 1 / (0.5 * (1 / 2 + 1 / 5))]
    assert np.allclose(got, want, rtol=1e-15)


# ---- test/test_boundary_conditions.jl -------------------------------------------------------------


def _bc(grid, f, spec):
    bc_apply(grid, [f], [to_cg_bc(grid.ndim, spec)])
    return f.interior(with_halo=True).astype(np.float64)


@pytest.mark.parametrize("T", TYPES)
def test_bc_1d_center(T):
    grid = UniformGrid(origin=(T(-math.pi),), extent=(T(2 * math.pi),), dims=(8,), dtype=T)
    f = NpField(grid, Center())
    f.interior()[...] = 1
    fi = _bc(grid, f, Dirichlet())
    assert approx(fi[0], -fi[1], T) and approx(fi[-1], -fi[-2], T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Neumann())
    assert approx(fi[0], fi[1], T) and approx(fi[-1], fi[-2], T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Dirichlet(T(2.0)))
    assert approx(fi[0], -fi[1] + 4, T) and approx(fi[-1], -fi[-2] + 4, T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Neumann(T(2.0)))
    dx = grid.spacing()[0]
    assert approx((fi[1] - fi[0]) / dx, 2.0, T) and approx((fi[-1] - fi[-2]) / dx, 2.0, T)


@pytest.mark.parametrize("T", TYPES)
def test_bc_1d_vertex(T):
    grid = UniformGrid(origin=(T(-math.pi),), extent=(T(2 * math.pi),), dims=(8,), dtype=T)
    f = NpField(grid, Vertex())
    f.interior()[...] = 1
    fi = _bc(grid, f, Dirichlet())
    assert fi[1] == 0 and fi[-2] == 0
    f.interior()[...] = 1
    fi = _bc(grid, f, Neumann())
    assert approx(fi[0], fi[1], T) and approx(fi[-1], fi[-2], T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Dirichlet(T(2.0)))
    assert approx(fi[1], 2.0, T) and approx(fi[-2], 2.0, T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Neumann(T(2.0)))
    dx = grid.spacing()[0]
    assert approx((fi[1] - fi[0]) / dx, 2.0, T) and approx((fi[-1] - fi[-2]) / dx, 2.0, T)


@pytest.mark.parametrize("T", TYPES)
def test_bc_2d(T):
    grid = UniformGrid(origin=(T(-math.pi),) * 2, extent=(T(2 * math.pi),) * 2, dims=(8, 8), dtype=T)
    f = NpField(grid, (Center(), Vertex()))
    f.interior()[...] = 1
    fi = _bc(grid, f, Dirichlet())
    assert approx(fi[0, 1:-1], -fi[1, 1:-1], T) and approx(fi[-1, 1:-1], -fi[-2, 1:-1], T)
    assert np.all(fi[1:-1, 1] == 0) and np.all(fi[1:-1, -2] == 0)
    f.interior()[...] = 1
    fi = _bc(grid, f, Neumann())
    assert approx(fi[0, 1:-1], fi[1, 1:-1], T) and approx(fi[-1, 1:-1], fi[-2, 1:-1], T)
    assert approx(fi[1:-1, 0], fi[1:-1, 1], T) and approx(fi[1:-1, -1], fi[1:-1, -2], T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Dirichlet(T(2.0)))
    assert approx(fi[0, 1:-1], -fi[1, 1:-1] + 4, T) and approx(fi[-1, 1:-1], -fi[-2, 1:-1] + 4, T)
    assert approx(fi[1:-1, 1], 2.0, T) and approx(fi[1:-1, -2], 2.0, T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Neumann(T(2.0)))
    dx, dy = grid.spacing()
    assert approx((fi[1, 1:-1] - fi[0, 1:-1]) / dx, 2.0, T) and approx((fi[-1, 1:-1] - fi[-2, 1:-1]) / dx, 2.0, T)
    assert approx((fi[1:-1, 1] - fi[1:-1, 0]) / dy, 2.0, T) and approx((fi[1:-1, -1] - fi[1:-1, -2]) / dy, 2.0, T)


@pytest.mark.parametrize("T", TYPES)
def test_bc_3d(T):
    grid = UniformGrid(origin=(T(-math.pi),) * 3, extent=(T(2 * math.pi),) * 3, dims=(8, 8, 6), dtype=T)
    f = NpField(grid, (Center(), Vertex(), Center()))
    s = slice(1, -1)
    f.interior()[...] = 1
    fi = _bc(grid, f, Dirichlet())
    assert approx(fi[0, s, s], -fi[1, s, s], T) and approx(fi[-1, s, s], -fi[-2, s, s], T)
    assert np.all(fi[s, 1, s] == 0) and np.all(fi[s, -2, s] == 0)
    assert approx(fi[s, s, 0], -fi[s, s, 1], T) and approx(fi[s, s, -1], -fi[s, s, -2], T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Neumann(T(2.0)))
    dx, dy, dz = grid.spacing()
    assert approx((fi[1, s, s] - fi[0, s, s]) / dx, 2.0, T) and approx((fi[-1, s, s] - fi[-2, s, s]) / dx, 2.0, T)
    assert approx((fi[s, 1, s] - fi[s, 0, s]) / dy, 2.0, T) and approx((fi[s, -1, s] - fi[s, -2, s]) / dy, 2.0, T)
    assert approx((fi[s, s, 1] - fi[s, s, 0]) / dz, 2.0, T) and approx((fi[s, s, -1] - fi[s, s, -2]) / dz, 2.0, T)
    f.interior()[...] = 1
    fi = _bc(grid, f, Dirichlet(T(2.0)))
    assert approx(fi[s, 1, s], 2.0, T) and approx(fi[s, s, 0], -fi[s, s, 1] + 4, T)


def test_bc_order_corners():
    """Corners follow Chmy's order: Dim N -> 1, so the last dim's rule writes the corner
    (batch.jl:104-113), reading the value the earlier dims left one step inward."""
    grid = UniformGrid(origin=(0.0, 0.0), extent=(1.0, 1.0), dims=(4, 5))
    f = NpField(grid, Center())
    rng = np.random.default_rng(0)
    f.a[...] = rng.standard_normal(f.a.shape)
    before = f.copy()
    bc_apply(grid, [f], [to_cg_bc(2, {"x": Dirichlet(1.5), "y": Neumann(-0.5)})])
    # y phase first: f[i,0] = f[i,1] + Δy*0.5 for i in 0..n+2 ; then x: f[0,j] = 2*(1.5 - f[1,j]) + f[1,j]
    dy = grid.spacing()[1]
    y0 = before.at(1, 1) + dy * 0.5
    corner = math.fma(2.0, 1.5 - y0, y0) if hasattr(math, "fma") else 2.0 * (1.5 - y0) + y0
    assert np.isclose(f.at(0, 0), corner, rtol=0, atol=1e-15)


# ---- explicit diffusion restated independently ----------------------------------------------------


@pytest.mark.parametrize("T", TYPES)
def test_diffusion_oracle_matches_numpy(T):
    from _oracle import lib
    import ctypes as C

    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(14, 11), dtype=T)
    rng = np.random.default_rng(1)
    Cf = NpField(grid, Center())
    Cf.a[1:-1, 1:-1] = rng.random((Cf.a.shape[0] - 2, Cf.a.shape[1] - 2)).astype(T)
    q = vec_fields(grid)
    chi, dt = T(1.0), T(1e-4)
    c0 = Cf.a.copy()
    from _oracle import desc_array

    g = grid.desc()
    assert lib().or_diffusion_compute_q(C.byref(g), desc_array(q, 3), C.byref(Cf.desc()), float(chi)) == 0
    assert lib().or_diffusion_update_C(C.byref(g), C.byref(Cf.desc()), desc_array(q, 3), float(dt)) == 0
    idx, idy = grid.inv_spacing()
    # numpy: q.x[i] = -χ (C[i]-C[i-1]) iΔ for i in 0..n+1 (array index i+1); q.x[n+2] = 0
    qx = np.zeros_like(c0)
    qy = np.zeros((c0.shape[0], c0.shape[1] + 1), dtype=T)
    qx = np.zeros((c0.shape[0] + 1, c0.shape[1]), dtype=T)  # y-extent n+4, x-extent n+4 for Center in x
    qxv = np.zeros((c0.shape[0], c0.shape[1] + 1), dtype=T)  # V.x: Vertex in x -> x ext +1
    qyv = np.zeros((c0.shape[0] + 1, c0.shape[1]), dtype=T)
    ny, nx = grid.dims[1], grid.dims[0]
    for j in range(0, ny + 2):
        for i in range(0, nx + 2):
            qxv[j + 1, i + 1] = (-chi) * ((c0[j + 1, i + 1] - c0[j + 1, i]) * idx)
            qyv[j + 1, i + 1] = (-chi) * ((c0[j + 1, i + 1] - c0[j, i + 1]) * idy)
    assert np.array_equal(q[0].a, qxv) and np.array_equal(q[1].a, qyv)
    c1 = c0.copy()
    for j in range(0, ny + 2):
        for i in range(0, nx + 2):
            dv = (qxv[j + 1, i + 2] - qxv[j + 1, i + 1]) * idx + (qyv[j + 2, i + 1] - qyv[j + 1, i + 1]) * idy
            c1[j + 1, i + 1] = c0[j + 1, i + 1] - dt * dv
    assert np.array_equal(Cf.a, c1)


def test_cg_bc_struct_roundtrip():
    b = to_cg_bc(3, {"x": Dirichlet(1.0), "z": (Neumann(2.0), None)})
    assert b.kind[0][0] == _abi.CG_BC_DIRICHLET and b.value[0][1] == 1.0
    assert b.kind[1][0] == _abi.CG_BC_NONE and b.kind[2][1] == _abi.CG_BC_NONE
    assert b.kind[2][0] == _abi.CG_BC_NEUMANN and b.value[2][0] == 2.0


# ---- test/test_boundary_functions.jl and Field-valued conditions -----------------------------


@pytest.mark.parametrize("T", TYPES)
def test_boundary_function_kats(T):
    """BoundaryFunction values at grid points (the checks of test_boundary_functions.jl:13-95):
    continuous/discrete, reduced/full dimensions, with parameters, on an 8 x 8 grid over
    [-pi, pi]^2."""
    from chmy_gb300.bcs import BoundaryFunction, Dim, coord

    nx = ny = 8
    grid = UniformGrid(origin=(T(-math.pi),) * 2, extent=(T(2 * math.pi),) * 2, dims=(nx, ny), dtype=T)
    tol = 1e-6 if T == np.float32 else 1e-12
    V = Vertex()

    def close(a, b):
        return abs(float(a) - float(b)) <= tol * max(1.0, abs(float(b)))

    for bf in (BoundaryFunction(np.cos),
               BoundaryFunction(lambda g, loc, dim, i: np.cos(coord(g, loc, dim, i)), discrete=True)):
        assert close(bf(grid, V, Dim(1), 1, 1), -1.0) and close(bf(grid, V, Dim(1), 1, ny + 1), -1.0)
        assert close(bf(grid, V, Dim(1), 1, ny // 2 + 1), 1.0)
        assert close(bf(grid, V, Dim(2), 1, 1), -1.0) and close(bf(grid, V, Dim(2), nx + 1, 1), -1.0)
        assert close(bf(grid, V, Dim(2), nx // 2 + 1, 1), 1.0)
        # the index along the condition's own dimension does not matter
        assert close(bf(grid, V, Dim(1), ny + 1, 1), bf(grid, V, Dim(1), 1, 1))
        assert close(bf(grid, V, Dim(2), 1, ny // 2 + 1), bf(grid, V, Dim(2), 1, 1))
    full = (BoundaryFunction(lambda x, y: np.cos(x) * y, reduce_dims=False),
            BoundaryFunction(lambda g, loc, dim, ix, iy: np.cos(coord(g, loc, ix, iy)[0]) * coord(g, loc, ix, iy)[1],
                             discrete=True, reduce_dims=False))
    for bf in full:
        assert close(bf(grid, V, Dim(1), 1, 1), math.pi) and close(bf(grid, V, Dim(1), 1, ny + 1), -math.pi)
        assert abs(float(bf(grid, V, Dim(1), 1, ny // 2 + 1))) <= tol
        assert close(bf(grid, V, Dim(2), 1, 1), math.pi) and close(bf(grid, V, Dim(2), nx // 2 + 1, 1), -math.pi)
    for bf in (BoundaryFunction(lambda x, eta: np.cos(x) * eta, parameters=math.pi),
               BoundaryFunction(lambda g, loc, dim, i, eta: np.cos(coord(g, loc, dim, i)) * eta, discrete=True,
                                parameters=math.pi)):
        assert close(bf(grid, V, Dim(1), 1, 1), -math.pi) and close(bf(grid, V, Dim(1), 1, ny // 2 + 1), math.pi)
        assert close(bf(grid, V, Dim(2), nx + 1, 1), -math.pi) and close(bf(grid, V, Dim(2), nx // 2 + 1, 1), math.pi)


@pytest.mark.parametrize("T", TYPES)
def test_bc_per_point_values_oracle(T):
    """Per-point condition values (a BoundaryFunction and an array) through the oracle: the
    ghost and boundary planes follow the same rules as constants, with the value of each
    tangential index (a direct numpy evaluation of first_order_boundary_condition.jl:46-84)."""
    from chmy_gb300.bcs import BoundaryFunction, materialize_bc

    nx, ny = 9, 7
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(nx, ny), dtype=T)
    rng = np.random.default_rng(3)
    f = NpField(grid, (Vertex(), Center()))
    f.a[...] = rng.standard_normal(f.a.shape).astype(T)
    before = f.copy()
    arr = rng.standard_normal(nx + 3).astype(T)  # y-sides: values over x indices 0..nx+2
    bfun = BoundaryFunction(lambda y: 1.0 + y * y)
    spec = {"x": (Dirichlet(bfun), Neumann(bfun)), "y": (Dirichlet(arr), Neumann(T(0.5)))}
    b, keep = materialize_bc(grid, f.loc, T, spec)
    bc_apply(grid, [f], [b])
    a = before.a.copy()  # padded [y, x], logical I at I + 1
    dx, dy = (float(v) for v in grid.spacing())
    # y first: side 0 Dirichlet on a Center dimension (ghost row 0) from the array; side 1 Neumann
    for i in range(0, nx + 3):
        a[1, i + 1] = T(2) * (arr[i] - a[2, i + 1]) + a[2, i + 1]
        a[ny + 2, i + 1] = T(dy) * T(0.5) + a[ny + 1, i + 1]
    # then x: side 0 Dirichlet on a Vertex dimension (boundary node 1) = bfun(y of the Vertex point),
    # side 1 Neumann on the Vertex dimension (ghost n+2) from node n+1 with the flipped (Center) location
    for j in range(0, ny + 3):
        yv = grid.axes[1].coord(Vertex(), j)
        yc = grid.axes[1].coord(Center(), j)
        a[j + 1, 2] = T(1.0 + yv * yv)
        a[j + 1, nx + 3] = T(dx) * T(1.0 + yc * yc) + a[j + 1, nx + 2]
    assert approx(f.a, a, T)
    assert any(np.array_equal(k, arr) for k in keep)  # the array itself is what the library reads


def test_gather_blocks_cartesian_order():
    """gather! (src/Distributed/gather.jl:9-33) places rank r's interior at the Cartesian
    coordinates of r, row-major over the topology dims (the last dim fastest)."""
    from chmy_gb300.fields import gather_blocks

    rng = np.random.default_rng(1)
    for dims, local in (((2, 3), (4, 5)), ((2, 2, 3), (3, 4, 2))):
        nd = len(dims)
        glob = rng.standard_normal(tuple(n * d for n, d in zip(reversed(local), reversed(dims))))
        blocks = []
        for r in range(int(np.prod(dims))):
            c = np.unravel_index(r, dims)  # row-major rank -> coordinates (x first)
            sl = tuple(slice(c[d] * local[d], (c[d] + 1) * local[d]) for d in reversed(range(nd)))
            blocks.append(glob[sl].copy())
        assert np.array_equal(gather_blocks(blocks, dims), glob)


def _np_mask_set(grid, T, rng, ones=False):
    """Host mask fields at every location (the oracle's cg_mask), random in [0, 1] or ones."""
    nd = grid.ndim
    fields = {}
    for bits in range(1 << nd):
        loc = tuple(Vertex() if (bits >> d) & 1 else Center() for d in range(nd))
        f = NpField(grid, loc, T)
        f.a[...] = 1 if ones else rng.random(f.a.shape).astype(T)
        fields[bits] = f
    m = _abi.cg_mask()
    for bits, f in fields.items():
        m.at[bits] = f.desc()
    return fields, m


@pytest.mark.parametrize("T", TYPES)
def test_masked_diffusion_oracle(T):
    """Masked operators (masked_operators.jl:11-39) in the oracle's diffusion kernels: with
    ones they equal the unmasked kernels bit for bit; with random weights they equal a numpy
    evaluation of q.x = -chi ∂x(C, ω) and C -= dt divg(q, ω)."""
    import ctypes

    from _oracle import lib

    rng = np.random.default_rng(5)
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(9, 7), dtype=T)
    g = grid.desc()
    C0 = NpField(grid, Center(), T)
    C0.a[...] = rng.standard_normal(C0.a.shape).astype(T)
    chi, dt = 1.3, 1e-3

    def run(masked, m):
        C = C0.copy()
        q = vec_fields(grid, T)
        qa = (_abi.cg_field * 3)(q[0].desc(), q[1].desc(), _abi.cg_field())
        if masked:
            assert lib().or_diffusion_compute_q_masked(ctypes.byref(g), qa, ctypes.byref(C.desc()), chi, ctypes.byref(m)) == 0
            assert lib().or_diffusion_update_C_masked(ctypes.byref(g), ctypes.byref(C.desc()), qa, dt, ctypes.byref(m)) == 0
        else:
            assert lib().or_diffusion_compute_q(ctypes.byref(g), qa, ctypes.byref(C.desc()), chi) == 0
            assert lib().or_diffusion_update_C(ctypes.byref(g), ctypes.byref(C.desc()), qa, dt) == 0
        return C, q

    _, ones = _np_mask_set(grid, T, rng, ones=True)
    Cm, qm = run(True, ones)
    Cu, qu = run(False, None)
    assert np.array_equal(Cm.a, Cu.a) and np.array_equal(qm[0].a, qu[0].a) and np.array_equal(qm[1].a, qu[1].a)
    wf, wm = _np_mask_set(grid, T, rng)
    Cm, qm = run(True, wm)
    c, wc, wx, wy = C0.a, wf[0].a, wf[1].a, wf[2].a
    idx, idy = (float(v) for v in grid.inv_spacing())
    nx, ny = grid.dims
    qx = np.zeros_like(qm[0].a)
    qy = np.zeros_like(qm[1].a)
    for j in range(0, ny + 2):  # launch range [0, n+1], logical I at padded I + 1
        for i in range(0, nx + 2):
            J, Ip = j + 1, i + 1
            qx[J, Ip] = -chi * ((c[J, Ip] * wc[J, Ip] - c[J, Ip - 1] * wc[J, Ip - 1]) * idx)
            qy[J, Ip] = -chi * ((c[J, Ip] * wc[J, Ip] - c[J - 1, Ip] * wc[J - 1, Ip]) * idy)
    cn = c.copy()
    for j in range(0, ny + 2):
        for i in range(0, nx + 2):
            J, Ip = j + 1, i + 1
            dv = (qx[J, Ip + 1] * wx[J, Ip + 1] - qx[J, Ip] * wx[J, Ip]) * idx
            dv += (qy[J + 1, Ip] * wy[J + 1, Ip] - qy[J, Ip] * wy[J, Ip]) * idy
            cn[J, Ip] = c[J, Ip] - dt * dv
    assert approx(qm[0].a, qx, T) and approx(qm[1].a, qy, T) and approx(Cm.a, cn, T)


def test_masked_stokes_oracle_matches_numpy():
    """The oracle's Stokes kernels with the masked operators (update_stress! with ∂(V.d, ω) and
    divg(V, ω), update_velocity! with ∂(Pr, ω) and ∂(τ, ω); 2D, scalar η, FP64) equal a numpy
    evaluation of the example kernels (examples/stokes_2d_inc_ve_T.jl:20-43) with every
    derivative operand weighted by the mask at its location and index, bit for bit; with unit
    weights they equal the unmasked oracle kernels bit for bit."""
    import ctypes

    from _oracle import lib, stokes_desc
    from chmy_gb300.kernels import stokes_params

    T = np.float64
    rng = np.random.default_rng(21)
    nx, ny = 11, 8
    grid = UniformGrid(origin=(-1.0, -1.0), extent=(2.0, 1.5), dims=(nx, ny), dtype=T)
    g = grid.desc()
    C_, V_ = Center(), Vertex()

    def rnd(loc, scale=1.0):
        f = NpField(grid, loc, T)
        f.a[...] = scale * rng.standard_normal(f.a.shape)
        return f

    V0 = [rnd((V_, C_)), rnd((C_, V_))]
    P0 = rnd(C_)
    tl = [(C_, C_), (C_, C_), (V_, V_)]
    tau0 = [rnd(l, 0.1) for l in tl]
    tauo = [rnd(l, 0.1) for l in tl]
    rho = rnd((C_, V_))
    p = stokes_params(eta=1.3, eta_ve=1.0 / (1.0 / 1.3 + 1.0 / 0.02), G=2.0, dt=1e-2, dtau_Pr=0.3, dtau_r=0.2, nu_dtau=0.05)

    def run(m):
        V = [f.copy() for f in V0]
        rV = vec_fields(grid, T)
        P, divV = P0.copy(), NpField(grid, C_, T)
        tau = [f.copy() for f in tau0]
        d = stokes_desc(V=V, r_V=rV, P=P, divV=divV, tau=tau, tau_old=tauo, rho_g=[None, rho])
        if m is None:
            assert lib().or_stokes_update_stress(ctypes.byref(g), ctypes.byref(d), ctypes.byref(p)) == 0
            assert lib().or_stokes_update_velocity(ctypes.byref(g), ctypes.byref(d), ctypes.byref(p)) == 0
        else:
            assert lib().or_stokes_update_stress_masked(ctypes.byref(g), ctypes.byref(d), ctypes.byref(p), ctypes.byref(m)) == 0
            assert lib().or_stokes_update_velocity_masked(ctypes.byref(g), ctypes.byref(d), ctypes.byref(p), ctypes.byref(m)) == 0
        return V, rV, P, divV, tau

    _, ones = _np_mask_set(grid, T, rng, ones=True)
    for a, b in zip(run(ones), run(None)):
        for fa, fb in zip(a if isinstance(a, list) else [a], b if isinstance(b, list) else [b]):
            assert np.array_equal(fa.a, fb.a)
    wf, wm = _np_mask_set(grid, T, rng)
    V, rV, P, divV, tau = run(wm)
    # numpy: logical index I at padded I + 1; the launch range [0, n+1] is padded 1 .. n+2
    idx, idy = (float(v) for v in grid.inv_spacing())
    G, dt, eta, eve = p.G, p.dt, p.eta, p.eta_ve
    J, I = np.meshgrid(np.arange(1, ny + 3), np.arange(1, nx + 3), indexing="ij")
    vx, vy = V0[0].a * wf[1].a, V0[1].a * wf[2].a
    exx = (vx[J, I + 1] - vx[J, I]) * idx
    eyy = (vy[J + 1, I] - vy[J, I]) * idy
    dv = exx + eyy
    exy = 0.5 * ((vx[J, I] - vx[J - 1, I]) * idy + (vy[J, I] - vy[J, I - 1]) * idx)
    Pn = P0.a.copy()
    Pn[J, I] = P0.a[J, I] - dv * eve * p.dtau_Pr
    tn = [f.a.copy() for f in tau0]
    for c, e in ((0, exx - dv / 3.0), (1, eyy - dv / 3.0), (2, exy)):
        t, to = tau0[c].a[J, I], tauo[c].a[J, I]
        r = -(t - to) / (G * dt) - t / eta + 2.0 * e
        tn[c][J, I] = t + r * eve * p.dtau_r
    assert np.array_equal(divV.a[J, I], dv) and np.array_equal(P.a, Pn)
    for c in range(3):
        assert np.array_equal(tau[c].a, tn[c]), c
    pw, txx, tyy, txy = Pn * wf[0].a, tn[0] * wf[0].a, tn[1] * wf[0].a, tn[2] * wf[3].a
    rx = -((pw[J, I] - pw[J, I - 1]) * idx) + (txx[J, I] - txx[J, I - 1]) * idx
    rx = rx + (txy[J + 1, I] - txy[J, I]) * idy
    ry = -((pw[J, I] - pw[J - 1, I]) * idy) + (tyy[J, I] - tyy[J - 1, I]) * idy
    ry = ry + (txy[J, I + 1] - txy[J, I]) * idx
    ry = ry - rho.a[J, I]
    assert np.array_equal(rV[0].a[J, I], rx) and np.array_equal(rV[1].a[J, I], ry)
    assert np.array_equal(V[0].a[J, I], V0[0].a[J, I] + rx * p.nu_dtau / eve)
    assert np.array_equal(V[1].a[J, I], V0[1].a[J, I] + ry * p.nu_dtau / eve)


def test_sia_dual_tangents_match_oracle_differences():
    """The oracle's dual-number SIA loop (or_sia_run_tangent): its value equals the plain
    restated loop bit for bit, and its tangents along Gamma and ela agree with central
    differences of that loop."""
    import ctypes

    from _oracle import desc_array, lib

    T = np.float64
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(20, 16), dtype=T)
    x, y = np.meshgrid(*[np.array([grid.axes[d].coord(Center(), i) for i in range(-1, grid.dims[d] + 3)]) for d in (1, 0)], indexing="ij")
    y, x = x, y  # [y, x] meshes of the padded Center coordinates
    bed = 0.4 + 0.2 * np.sin(2 * x) * np.cos(3 * y)
    H0 = np.clip(0.35 - 0.25 * (x * x + y * y), 0.0, None)
    p = _abi.cg_sia_params()
    p.Gamma, p.As, p.n, p.beta, p.ela, p.m_max, p.dt_max, p.cfl = 1.0, 0.0, 3, 0.5, 0.55, 0.25, 0.5, 4.1
    g = grid.desc()
    nsteps = 20

    def plain(Gamma, ela):
        q_ = _abi.cg_sia_params()
        ctypes.memmove(ctypes.byref(q_), ctypes.byref(p), ctypes.sizeof(q_))
        q_.Gamma, q_.ela = Gamma, ela
        H = NpField(grid, Center(), T)
        H.a[...] = H0
        B = NpField(grid, Center(), T)
        B.a[...] = bed
        q = [NpField(grid, (Vertex(), Center()), T), NpField(grid, (Center(), Vertex()), T)]
        dx = min(grid.spacing())
        for _ in range(nsteps):
            dmax = ctypes.c_double()
            lib().or_sia_update_q(ctypes.byref(g), desc_array(q, 3), ctypes.byref(H.desc()), ctypes.byref(B.desc()), ctypes.byref(q_), ctypes.byref(dmax))
            qd = T(dx * dx) / T(dmax.value) / T(q_.cfl)
            dt = float(qd) if (dmax.value > 0 and qd < q_.dt_max) else q_.dt_max
            lib().or_sia_update_H(ctypes.byref(g), ctypes.byref(H.desc()), desc_array(q, 3), ctypes.byref(B.desc()), dt, ctypes.byref(q_))
        return H.a.copy()

    H = NpField(grid, Center(), T)
    H.a[...] = H0
    B = NpField(grid, Center(), T)
    B.a[...] = bed
    q = [NpField(grid, (Vertex(), Center()), T), NpField(grid, (Center(), Vertex()), T)]
    tG, tE = NpField(grid, Center(), T), NpField(grid, Center(), T)
    assert lib().or_sia_run_tangent(ctypes.byref(g), ctypes.byref(H.desc()), ctypes.byref(B.desc()), desc_array(q, 3),
                                    ctypes.byref(p), nsteps, ctypes.byref(tG.desc()), ctypes.byref(tE.desc())) == 0
    assert np.array_equal(H.a, plain(p.Gamma, p.ela))
    h = 1e-6
    fdG = (plain(p.Gamma + h, p.ela) - plain(p.Gamma - h, p.ela)) / (2 * h)
    fdE = (plain(p.Gamma, p.ela + h) - plain(p.Gamma, p.ela - h)) / (2 * h)
    assert np.max(np.abs(tG.a - fdG)) <= 1e-6 * np.max(np.abs(fdG))
    assert np.max(np.abs(tE.a - fdE)) <= 1e-6 * np.max(np.abs(fdE))


def test_stokes_dual_tangents_match_oracle_differences():
    """The oracle's dual-number VE Stokes solve (or_stokes_solve_tangent, 2D 16^2 with 8
    viscous inclusions): a zero direction leaves the tangents zero, and the tangent of a
    velocity misfit along a random log-viscosity direction agrees with central differences
    of the oracle's own converged solve to 1e-6."""
    import dataclasses

    from _oracle import stokes_tangent_solve

    from chmy_gb300.configs import stokes2d_inclusions

    pb = stokes2d_inclusions(16, ncheck=8)
    shape = pb.host["eta"].shape
    rng = np.random.default_rng(4)
    dirv = np.zeros(shape)
    dirv[2:-2, 2:-2] = rng.standard_normal((16, 16))
    zero = np.zeros(shape)
    fs, tan, iters = stokes_tangent_solve(pb, [dirv, zero])
    assert iters > 0 and not np.any(tan[1][0]) and not np.any(tan[1][1])
    vy = fs["V"][1].a
    sens = (slice(2, 18), 10)  # Vy on one interior vertex row
    obs = vy[sens] * 0.7
    dual = float(np.sum((vy[sens] - obs) * tan[0][1][sens]))

    def J(scale):
        e = pb.host["eta"] * np.exp(scale * dirv)
        f, _, _ = stokes_tangent_solve(dataclasses.replace(pb, host={**pb.host, "eta": e}), [zero, zero])
        r = f["V"][1].a[sens] - obs
        return 0.5 * float(np.sum(r * r))

    h = 1e-5
    fd = (J(h) - J(-h)) / (2 * h)
    assert abs(dual - fd) <= 1e-6 * abs(fd), (dual, fd)


def test_ptdiff_dual_tangents_match_oracle_differences():
    """The oracle's dual-number PT-diffusion loop (or_ptdiff_run_tangent, 2D 16^2, 3 implicit
    steps of 400 PT iterations): a zero direction leaves the tangent zero, and the tangent of a
    misfit of C^N along a random log-diffusivity direction agrees with central differences of
    the same loop to 1e-6."""
    from _oracle import ptdiff_tangent_run

    from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
    from chmy_gb300.configs import box_smooth, padded_mesh, ptdiff_params

    T = np.float64
    n, nsteps, npt = 16, 3, 400
    grid = UniformGrid(origin=(T(-0.5), T(-0.5)), extent=(T(1), T(1)), dims=(n, n), dtype=T)
    x, y = padded_mesh(grid, Center())
    rng = np.random.default_rng(2)
    D = np.exp(box_smooth(rng.standard_normal(x.shape)))
    C0 = np.exp(-(x * x + y * y) / 0.01)
    bc = to_cg_bc(2, {"x": Dirichlet(0.0), "y": Neumann()})
    p = ptdiff_params(grid, 1e-3, float(D.max()))
    dirv = np.zeros(x.shape)
    dirv[2:-2, 2:-2] = rng.standard_normal((n, n))
    zero = np.zeros(x.shape)
    CN, tan = ptdiff_tangent_run(grid, D, C0, p, bc, nsteps, npt, [dirv, zero])
    assert not np.any(tan[1])
    inner = (slice(2, n + 2), slice(2, n + 2))
    obs = CN[inner] * 0.8
    dual = float(np.sum((CN[inner] - obs) * tan[0][inner]))

    def J(scale):
        c, _ = ptdiff_tangent_run(grid, D * np.exp(scale * dirv), C0, p, bc, nsteps, npt, [zero, zero])
        r = c[inner] - obs
        return 0.5 * float(np.sum(r * r))

    h = 1e-5
    fd = (J(h) - J(-h)) / (2 * h)
    assert abs(dual - fd) <= 1e-6 * abs(fd), (dual, fd)


@pytest.mark.parametrize("kinds", ["neumann_dirichlet", "periodic"])
def test_explicit_diffusion_dual_tangents_match_oracle_differences(kinds):
    """The oracle's dual-number explicit diffusion loop (or_diffusion_run_tangent, 2D 20x16, 25
    steps): its value equals the plain oracle loop bit for bit, and the tangents of a misfit of
    C^N along chi and along an initial-state direction agree with central differences of the
    plain loop to 1e-6."""
    from _oracle import diffusion_run, diffusion_tangent_run

    from chmy_gb300.configs import padded_mesh

    T = np.float64
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(20, 16), dtype=T)
    x, y = padded_mesh(grid, Center())
    rng = np.random.default_rng(6)
    C0 = np.exp(-(x * x + y * y) / 0.1) + 0.01 * rng.standard_normal(x.shape)
    from chmy_gb300.bcs import Periodic

    spec = {"x": Neumann(0.3), "y": Dirichlet(0.2)} if kinds == "neumann_dirichlet" else {"x": Periodic(), "y": Neumann()}
    bc = to_cg_bc(2, spec)
    h = float(grid.spacing()[0])
    chi, dt, nsteps = 1.0, h * h / 4.1, 25
    dirv = np.zeros(x.shape)
    dirv[2:-2, 2:-2] = rng.standard_normal((16, 20))
    CN, dchi, ddir = diffusion_tangent_run(grid, C0, chi, dt, bc, nsteps, dirv)
    np.testing.assert_array_equal(CN, diffusion_run(grid, C0, chi, dt, bc, nsteps))
    inner = (slice(2, -2), slice(2, -2))
    w = rng.standard_normal(CN[inner].shape)

    def J(c):
        return 0.5 * float(np.sum(w * c[inner] ** 2))

    dual_chi = float(np.sum(w * CN[inner] * dchi[inner]))
    dual_dir = float(np.sum(w * CN[inner] * ddir[inner]))
    e = 1e-6
    fd_chi = (J(diffusion_run(grid, C0, chi + e, dt, bc, nsteps)) - J(diffusion_run(grid, C0, chi - e, dt, bc, nsteps))) / (2 * e)
    fd_dir = (J(diffusion_run(grid, C0 + e * dirv, chi, dt, bc, nsteps)) - J(diffusion_run(grid, C0 - e * dirv, chi, dt, bc, nsteps))) / (2 * e)
    assert abs(dual_chi - fd_chi) <= 1e-6 * abs(fd_chi), (dual_chi, fd_chi)
    assert abs(dual_dir - fd_dir) <= 1e-6 * abs(fd_dir), (dual_dir, fd_dir)


def test_thermal_step_dual_tangents_match_oracle_differences():
    """The oracle's dual-number thermal step (or_thermal_step_tangent, 2D 18x14): its value equals
    the plain two-kernel step bit for bit, and the tangents of sum mu T_out along (T, T_old, V)
    directions and along lambda_rhoCp agree with central differences of the plain step."""
    from _oracle import thermal_problem, thermal_step, thermal_tangent_step

    from chmy_gb300.kernels import stokes_params

    T = np.float64
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(18, 14), dtype=T)
    bc_T = to_cg_bc(2, {"x": Neumann(0.2), "y": Dirichlet(0.5)})
    pr = thermal_problem(grid, 3, bc_T)
    p = stokes_params(G=1.0, dt=2e-3, lambda_rhoCp=0.3)
    out, tan = thermal_tangent_step(grid, pr, p, bc_T)
    Vs = [v.a for v in pr["V"]]
    np.testing.assert_array_equal(out, thermal_step(grid, pr["T"].a, pr["T_old"].a, Vs, p, bc_T))
    inner, mu = pr["inner"], pr["mu"]

    def J(e_dir, e_lam):
        q = stokes_params(G=1.0, dt=2e-3, lambda_rhoCp=0.3 + e_lam)
        o = thermal_step(grid, pr["T"].a + e_dir * pr["dT"], pr["T_old"].a + e_dir * pr["dT_old"],
                         [v + e_dir * d for v, d in zip(Vs, pr["dV"])], q, bc_T)
        return float(np.sum(mu[inner] * o[inner]))

    e = 1e-6
    fd_dir = (J(e, 0.0) - J(-e, 0.0)) / (2 * e)
    fd_lam = (J(0.0, e) - J(0.0, -e)) / (2 * e)
    dual_dir = float(np.sum(mu[inner] * tan[0][inner]))
    dual_lam = float(np.sum(mu[inner] * tan[1][inner]))
    # the upwind kinks: no face velocity lies within e of zero here, so J is smooth at this point
    assert min(np.abs(v).min() for v in Vs) > 1e-4
    assert abs(dual_dir - fd_dir) <= 1e-6 * abs(fd_dir), (dual_dir, fd_dir)
    assert abs(dual_lam - fd_lam) <= 1e-6 * abs(fd_lam), (dual_lam, fd_lam)


def test_function_field_host_and_oracle_evaluations():
    """FunctionField.values() (numpy, coordinates as padded_mesh rounds them) and the oracle's
    or_function_fill (coordinates by fused multiply-adds, Chmy's muladd) agree: the affine form to
    rounding, the ball indicator except at points within rounding of its radius."""
    import ctypes as C

    from _oracle import lib
    from chmy_gb300.functions import FunctionField, affine, ball

    T = np.float64
    for nd, dims in ((2, (40, 33)), (3, (14, 12, 11))):
        grid = UniformGrid(origin=(T(-0.5),) * nd, extent=(T(1),) * nd, dims=dims, dtype=T)
        loc = tuple(Vertex() if d == 0 else Center() for d in range(nd))
        cases = [(ball, (0.1,) * nd + (0.3, 2.0, -1.0)), (affine, (0.25,) + tuple(float(d + 1) for d in range(nd)))]
        for func, params in cases:
            ff = FunctionField(func, grid, loc, parameters=params)
            ref = NpField(grid, loc, T)
            assert lib().or_function_fill(C.byref(grid.desc()), C.byref(ff.desc()), C.byref(ref.desc())) == 0
            host = ff.values()
            if func is ball:
                assert set(np.unique(ref.a)) <= {2.0, -1.0}
                assert np.mean(host != ref.a) < 1e-3
            else:
                np.testing.assert_allclose(host, ref.a, rtol=0, atol=1e-14)
