"""The VE Stokes kernels written with Chmy's masked operators (src/GridOperators/
masked_operators.jl:11-39, masked_field_operators.jl; the FieldMask usage of
docs/src/concepts/grid_operators.md "Masking") against the oracle's masked kernels, per launch
and over graph-replayed PT iterations, through the C ABI and through the Launcher."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, lib
from chmy_gb300 import _abi
from chmy_gb300.grids import Center, Vertex
from gpu_helpers import to_gpu
from test_gpu_stokes import StokesSet, _bc_V, _compare, pt_params

pytestmark = pytest.mark.gpu
TYPES = [np.float32, np.float64]


def _masks(arch, grid, T, rng, kind="random"):
    """Host and device weight fields at every location (cg_mask indexed by location bits):
    'random' weights in [0, 1] with about a fifth exactly 0 (masked-out points), or 'ones'.
    The descriptors point into the returned fields: keep those alive while the masks are used."""
    nd = grid.ndim
    host, dev = {}, {}
    hm, dm = _abi.cg_mask(), _abi.cg_mask()
    for bits in range(1 << nd):
        loc = tuple(Vertex() if (bits >> d) & 1 else Center() for d in range(nd))
        h = NpField(grid, loc, T)
        if kind == "ones":
            h.a[...] = 1
        else:
            w = rng.random(h.a.shape)
            w[rng.random(h.a.shape) < 0.2] = 0.0
            h.a[...] = w.astype(T)
        host[bits], dev[bits] = h, to_gpu(arch, h)
        hm.at[bits], dm.at[bits] = h.desc(), dev[bits].desc()
    return host, dev, hm, dm


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(33, 21), (12, 9, 10)])
@pytest.mark.parametrize("var_eta", [False, True])
def test_masked_stress_velocity_match_oracle(arch, T, dims, var_eta):
    """update_stress! with ∂(V.d, ω) and divg(V, ω), and update_velocity! with ∂(Pr, ω) and
    ∂(τ, ω), per launch: the GPU kernels equal the oracle's masked kernels (FMA contraction
    aside), with random weights that include masked-out points."""
    s = StokesSet(arch, dims, T, 29, var_eta)
    p = pt_params(s.grid, var_eta)
    g = s.grid.desc()
    keep_h, keep_d, hm, dm = _masks(arch, s.grid, T, np.random.default_rng(3))
    hd, dd = s.host_desc(), s.dev_desc()
    assert lib().or_stokes_update_stress_masked(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p), ctypes.byref(hm)) == 0
    arch.call("cg_stokes_update_stress_masked", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(dm))
    arch.synchronize()
    _compare(s, T, "update_stress masked")
    assert lib().or_stokes_update_velocity_masked(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p), ctypes.byref(hm)) == 0
    arch.call("cg_stokes_update_velocity_masked", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(dm))
    arch.synchronize()
    _compare(s, T, "update_velocity masked")


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(27, 19), (10, 11, 9)])
def test_unit_mask_equals_unmasked_kernels(arch, T, dims):
    """With every weight 1 the masked kernels give the unmasked kernels' bits (x * 1 == x)."""
    a = StokesSet(arch, dims, T, 31, True)
    b = StokesSet(arch, dims, T, 31, True)
    p = pt_params(a.grid, True)
    g = a.grid.desc()
    _, keep_d, _, dm = _masks(arch, a.grid, T, None, kind="ones")
    da, db = a.dev_desc(), b.dev_desc()
    arch.call("cg_stokes_update_stress_masked", ctypes.byref(g), ctypes.byref(da), ctypes.byref(p), ctypes.byref(dm))
    arch.call("cg_stokes_update_velocity_masked", ctypes.byref(g), ctypes.byref(da), ctypes.byref(p), ctypes.byref(dm))
    arch.call("cg_stokes_update_stress", ctypes.byref(g), ctypes.byref(db), ctypes.byref(p))
    arch.call("cg_stokes_update_velocity", ctypes.byref(g), ctypes.byref(db), ctypes.byref(p))
    arch.synchronize()
    for (name, fa, _), (_, fb, _) in zip(a.pairs(), b.pairs()):
        x, y = fa.to_numpy(), fb.to_numpy()
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), name


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(31, 26), (13, 12, 11)])
def test_masked_pt_iterations_match_oracle(arch, T, dims):
    """cg_stokes_pt_iterations_masked (graph-replayed: masked update_stress!, masked
    update_velocity!, bc!(V)) == niter x the same on the oracle."""
    s = StokesSet(arch, dims, T, 37, True)
    p = pt_params(s.grid, True)
    g = s.grid.desc()
    nd = len(dims)
    bcs = _bc_V(nd)
    keep_h, keep_d, hm, dm = _masks(arch, s.grid, T, np.random.default_rng(8))
    hd, dd = s.host_desc(), s.dev_desc()
    bc_apply(s.grid, s.h["V"], bcs)
    for f, d in zip(s.h["V"], s.d["V"]):
        d.from_numpy(f.a)
    niter = 6
    for _ in range(niter):
        lib().or_stokes_update_stress_masked(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p), ctypes.byref(hm))
        lib().or_stokes_update_velocity_masked(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p), ctypes.byref(hm))
        bc_apply(s.grid, s.h["V"], bcs)
    barr = (_abi.cg_bc * 3)(*bcs)
    arch.call("cg_stokes_pt_iterations_masked", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), barr, ctypes.byref(dm), niter)
    arch.synchronize()
    _compare(s, T, "pt_iterations masked", scale=niter * 10)


def test_masked_kernels_through_the_launcher(arch):
    """The docs' masked kernels written as in the reference: a FieldMask ω whose velocity weights
    are set! from an inclusion function (grid_operators.md "Masking") and ones elsewhere, passed
    as the kernels' last argument to launch(...). Equal to the direct masked entry points."""
    from chmy_gb300 import Field, FieldMask, Launcher, TensorField, VectorField, set_, update_stress, update_velocity
    from chmy_gb300.grids import UniformGrid

    T = np.float64
    grid = UniformGrid(origin=(-1.0, -1.0), extent=(2.0, 2.0), dims=(40, 36), dtype=T)
    omega = FieldMask(arch, grid, T)
    for bits, f in omega.fields.items():
        f.from_numpy(np.ones(f.data.shape))
    r = 0.5
    incl = lambda x, y: np.where(x * x + y * y < r * r, 1.0, 0.0)  # noqa: E731
    set_(omega.at((Vertex(), Center())), incl, grid)
    set_(omega.at((Center(), Vertex())), incl, grid)
    outs = []
    for direct in (False, True):
        V, r_V, tau, tau_old = VectorField(arch, grid), VectorField(arch, grid), TensorField(arch, grid), TensorField(arch, grid)
        Pr, divV = Field(arch, grid, Center()), Field(arch, grid, Center())
        rho = Field(arch, grid, (Center(), Vertex()))
        r2 = np.random.default_rng(12)
        for f in list(V) + list(tau) + list(tau_old) + [Pr, rho]:
            f.from_numpy(r2.standard_normal(f.data.shape))
        p = pt_params(grid, False)
        if direct:
            from chmy_gb300.kernels import stokes_fields

            sf = stokes_fields(V=V, r_V=r_V, P=Pr, divV=divV, tau=tau, tau_old=tau_old, rho_g=[None, rho])
            m = omega.desc()
            arch.call("cg_stokes_update_stress_masked", ctypes.byref(grid.desc()), ctypes.byref(sf), ctypes.byref(p), ctypes.byref(m))
            arch.call("cg_stokes_update_velocity_masked", ctypes.byref(grid.desc()), ctypes.byref(sf), ctypes.byref(p),
                      ctypes.byref(m))
        else:
            launch = Launcher(arch, grid)
            launch(arch, grid, (update_stress, (tau, Pr, divV, V, tau_old, p.eta, p.eta_ve, p.G, p.dt, p.dtau_Pr, p.dtau_r, grid,
                                                omega)))
            launch(arch, grid, (update_velocity, (V, r_V, Pr, tau, rho, p.eta_ve, p.nu_dtau, grid, omega)))
        arch.synchronize()
        outs.append([f.to_numpy() for f in list(V) + list(r_V) + list(tau) + [Pr, divV]])
    for x, y in zip(*outs):
        np.testing.assert_array_equal(x, y)
    # the inclusion weights reach the divergence: zero in a corner cell, whose faces lie outside
    # the disc, and not at the centre (padded index = logical index + 1)
    divV = outs[0][-1]
    assert divV[3, 3] == 0.0 and divV[19, 21] != 0.0


def test_masked_entry_points_check_the_mask(arch):
    """A NULL mask, a missing weight field the kernel reads, or one at the wrong location is
    rejected with CG_ERR_ARG before any launch."""
    s = StokesSet(arch, (20, 18), np.float64, 41, False)
    p = pt_params(s.grid, False)
    g = s.grid.desc()
    _, dev, _, dm = _masks(arch, s.grid, np.float64, np.random.default_rng(1))
    dd = s.dev_desc()
    L = arch.lib
    assert L.cg_stokes_update_stress_masked(arch.ctx, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), None) == _abi.CG_ERR_ARG
    bad = _abi.cg_mask()
    ctypes.memmove(ctypes.byref(bad), ctypes.byref(dm), ctypes.sizeof(bad))
    bad.at[1] = _abi.cg_field()
    assert L.cg_stokes_update_stress_masked(arch.ctx, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(bad)) \
        == _abi.CG_ERR_ARG
    # update_velocity! does not read the velocity-location weights
    assert L.cg_stokes_update_velocity_masked(arch.ctx, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(bad)) \
        == _abi.CG_OK
    ctypes.memmove(ctypes.byref(bad), ctypes.byref(dm), ctypes.sizeof(bad))
    bad.at[3] = dev[0].desc()  # a cell field where the shear weights belong
    assert L.cg_stokes_update_velocity_masked(arch.ctx, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), ctypes.byref(bad)) \
        == _abi.CG_ERR_ARG
    barr = (_abi.cg_bc * 3)(*_bc_V(2))
    assert L.cg_stokes_pt_iterations_masked(arch.ctx, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), barr, ctypes.byref(bad), 2) \
        == _abi.CG_ERR_ARG
    arch.synchronize()
