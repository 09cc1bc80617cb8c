"""GPU parity of the VE Stokes kernels (examples/stokes_{2,3}d_inc_ve_T.jl) against the oracle,
per launch and over graph-replayed PT iterations, through the C ABI."""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, bc_apply, lib, stokes_desc, tensor_fields, vec_fields
from chmy_gb300 import _abi
from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
from chmy_gb300.grids import Center, UniformGrid, Vertex
from chmy_gb300.kernels import stokes_params
from gpu_helpers import assert_close, random_field, rtol_for, to_gpu

pytestmark = pytest.mark.gpu
TYPES = [np.float32, np.float64]
C_, V_ = Center(), Vertex()


class StokesSet:
    """Seeded random VE Stokes state on host and device."""

    def __init__(self, arch, dims, T, seed, var_eta, rho=True, thermal=False, pitch_align=0, plane_rows=0):
        rng = np.random.default_rng(seed)
        nd = len(dims)
        self.grid = UniformGrid(origin=(T(-1),) * nd, extent=(T(2),) * nd, dims=dims, dtype=T)
        g = self.grid
        self.h = {}
        self.h["V"] = [random_field(g, f.loc, T, rng) for f in vec_fields(g, T)]
        self.h["r_V"] = vec_fields(g, T)
        self.h["P"] = random_field(g, C_, T, rng)
        self.h["divV"] = NpField(g, C_, T)
        self.h["tau"] = [random_field(g, f.loc, T, rng, 0.1) for f in tensor_fields(g, T)]
        self.h["tau_old"] = [random_field(g, f.loc, T, rng, 0.1) for f in tensor_fields(g, T)]
        if var_eta:
            e = NpField(g, C_, T)
            e.a[...] = np.exp(rng.uniform(-3, 3, e.a.shape)).astype(T)
            self.h["eta"] = e
        if rho:
            r = [None] * 3
            r[nd - 1] = random_field(g, vec_fields(g, T)[nd - 1].loc, T, rng)
            self.h["rho_g"] = r
        if thermal:
            self.h["T"] = random_field(g, C_, T, rng, 1.0, 1.0)
            self.h["T_old"] = random_field(g, C_, T, rng, 1.0, 1.0)
            self.h["qT"] = vec_fields(g, T)
        self.d = {}
        for k, v in self.h.items():
            if isinstance(v, list):
                self.d[k] = [to_gpu(arch, f, pitch_align, plane_rows) if f is not None else None for f in v]
            else:
                self.d[k] = to_gpu(arch, v, pitch_align, plane_rows)

    def host_desc(self):
        return stokes_desc(**self.h)

    def dev_desc(self):
        return stokes_desc(**self.d)

    def pairs(self):
        for k, v in self.h.items():
            if isinstance(v, list):
                for i, f in enumerate(v):
                    if f is not None:
                        yield f"{k}[{i}]", self.d[k][i], f
            else:
                yield k, self.d[k], v


def pt_params(grid, var_eta):
    nd = grid.ndim
    lx = 2.0
    dx = min(float(s) for s in grid.spacing())
    re_m, r = 2.3 * np.pi, 0.5
    lt = lx / re_m
    vdt = dx / np.sqrt(nd * 1.1)
    th = lt * (r + 4 / 3) / vdt
    eta, G, dt = 1.0, 1.0, 1e-2
    return stokes_params(
        eta=eta, eta_ve=1.0 / (1.0 / eta + 1.0 / (G * dt)), G=G, dt=dt, dtau_Pr=r / th, dtau_r=1.0 / (th + 1.0), nu_dtau=vdt * lt,
        lambda_rhoCp=1e-3,
    )


def _compare(s, T, what, scale=1.0):
    for name, a, b in s.pairs():
        assert_close(a, b, rtol_for(T) * scale, f"{what}: {name}")


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(23, 17), (12, 9, 10)])
@pytest.mark.parametrize("var_eta", [False, True])
def test_stress_velocity_kernels(arch, T, dims, var_eta):
    s = StokesSet(arch, dims, T, 17, var_eta)
    p = pt_params(s.grid, var_eta)
    g = s.grid.desc()
    hd, dd = s.host_desc(), s.dev_desc()
    assert lib().or_stokes_update_stress(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p)) == 0
    arch.call("cg_stokes_update_stress", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p))
    arch.synchronize()
    _compare(s, T, "update_stress")
    assert lib().or_stokes_update_velocity(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p)) == 0
    arch.call("cg_stokes_update_velocity", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p))
    arch.synchronize()
    _compare(s, T, "update_velocity")


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(20, 14), (9, 11, 8)])
def test_update_old_and_thermal(arch, T, dims):
    s = StokesSet(arch, dims, T, 23, False, thermal=True)
    p = pt_params(s.grid, False)
    g = s.grid.desc()
    hd, dd = s.host_desc(), s.dev_desc()
    for name in ("update_thermal_flux", "update_thermal", "update_old"):
        fo = getattr(lib(), "or_stokes_" + name)
        if name == "update_old":
            assert fo(ctypes.byref(g), ctypes.byref(hd)) == 0
            arch.call("cg_stokes_" + name, ctypes.byref(g), ctypes.byref(dd))
        else:
            assert fo(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p)) == 0
            arch.call("cg_stokes_" + name, ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p))
        arch.synchronize()
        _compare(s, T, name)


def _bc_V(nd):
    bcs = []
    for d in range(nd):
        spec = {"xyz"[e]: (Neumann() if e != d else (Dirichlet(0.5), Dirichlet(-0.5))) for e in range(nd)}
        bcs.append(to_cg_bc(nd, spec))
    return bcs


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(31, 26), (13, 12, 11)])
@pytest.mark.parametrize("var_eta", [False, True])
def test_pt_iterations_graph(arch, T, dims, var_eta):
    """cg_stokes_pt_iterations == niter x (update_stress!, update_velocity!, bc!(V)) on the oracle."""
    s = StokesSet(arch, dims, T, 29, var_eta, rho=True)
    nd = len(dims)
    p = pt_params(s.grid, var_eta)
    g = s.grid.desc()
    bcs = _bc_V(nd)
    bc_apply(s.grid, s.h["V"], bcs)
    for f, d in zip(s.h["V"], s.d["V"]):
        d.from_numpy(f.a)
    hd, dd = s.host_desc(), s.dev_desc()
    niter = 7
    for _ in range(niter):
        lib().or_stokes_update_stress(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        lib().or_stokes_update_velocity(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        bc_apply(s.grid, s.h["V"], bcs)
    barr = (_abi.cg_bc * 3)(*bcs)
    arch.call("cg_stokes_pt_iterations", ctypes.byref(g), ctypes.byref(dd), ctypes.byref(p), barr, niter)
    arch.synchronize()
    _compare(s, T, "pt_iterations", scale=niter * 10)
    # residual measures equal the oracle's max-norms after bc!(r_V => Dirichlet)
    err = (ctypes.c_double * 4)()
    arch.call("cg_stokes_residual", ctypes.byref(g), ctypes.byref(dd), 1.0, 2.0, err)
    rb = []
    for d in range(nd):
        spec = {"xyz"[d]: Dirichlet()}
        rb.append(to_cg_bc(nd, spec))
    bc_apply(s.grid, s.h["r_V"], rb)
    want = [np.max(np.abs(s.h["divV"].interior()))] + [2.0 * np.max(np.abs(f.interior())) for f in s.h["r_V"]]
    for i in range(nd + 1):
        assert abs(err[i] - want[i]) <= rtol_for(T) * niter * 10 * max(abs(want[i]), 1.0)


def _pp_run(arch, T, dims, bcs, niter, seed=31, pitch_align=0, plane_rows=0):
    """niter fused ping-pong iterations (cg_stokes_pt_iterations_pp) against niter x
    (update_stress!, update_velocity!, bc!(V)) on the oracle. Returns the set, the partner
    buffers and the oracle's V after niter - 1 iterations. pitch_align: the device fields' row
    alignment (bytes; 0 = Chmy's dense layout); plane_rows: 3D rows per plane (with
    pitch_align, one plane stride for every array)."""
    s = StokesSet(arch, dims, T, seed, True, rho=True, pitch_align=pitch_align, plane_rows=plane_rows)
    g2 = s.grid
    rho_full = [random_field(g2, f.loc, T, np.random.default_rng(5)) for f in vec_fields(g2, T)]
    s.h["rho_g"] = rho_full
    s.d["rho_g"] = [to_gpu(arch, f, pitch_align, plane_rows) for f in rho_full]
    ie = NpField(g2, C_, T)
    ie.a[...] = (1.0 / s.h["eta"].a).astype(T)
    s.h["inv_eta"] = ie
    s.d["inv_eta"] = to_gpu(arch, ie, pitch_align, plane_rows)
    p = pt_params(g2, True)
    g = g2.desc()
    bc_apply(g2, s.h["V"], bcs)
    for f, d in zip(s.h["V"], s.d["V"]):
        d.from_numpy(f.a)
    # partner buffers for V, P, tau hold the same initial state
    partner = {k: ([to_gpu(arch, f, pitch_align, plane_rows) for f in s.h[k]] if isinstance(s.h[k], list)
                   else to_gpu(arch, s.h[k], pitch_align, plane_rows))
               for k in ("V", "P", "tau")}
    hd, da = s.host_desc(), s.dev_desc()
    from _oracle import stokes_desc as sd

    db = sd(V=partner["V"], P=partner["P"], tau=partner["tau"])
    prev = None
    for it in range(niter):
        if it == niter - 1:
            prev = [f.a.copy() for f in s.h["V"]]
        lib().or_stokes_update_stress(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        lib().or_stokes_update_velocity(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        bc_apply(g2, s.h["V"], bcs)
    barr = (_abi.cg_bc * 3)(*bcs)
    arch.call("cg_stokes_pt_iterations_pp", ctypes.byref(g), ctypes.byref(da), ctypes.byref(db), ctypes.byref(p), barr, niter)
    arch.synchronize()
    return s, partner, prev, (g, da, db, p, barr)


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(45, 38), (70, 33), (33, 97), (257, 300), (13, 12, 11), (31, 20, 70), (61, 7, 33)])
def test_fused_pingpong_iterations(arch, T, dims):
    """cg_stokes_pt_iterations_pp (one fused launch per iteration, ping-pong buffers) ==
    niter x (update_stress!, update_velocity!, bc!(V)) on the oracle, bit for bit."""
    s, _, _, (g, da, db, p, barr) = _pp_run(arch, T, dims, _bc_V(len(dims)), 6)
    for name in ("V", "P", "tau", "divV", "r_V"):
        hv = s.h[name] if isinstance(s.h[name], list) else [s.h[name]]
        dv = s.d[name] if isinstance(s.d[name], list) else [s.d[name]]
        for a, b in zip(dv, hv):
            if b is not None:
                # the fused kernel rounds every operation as the oracle does: bitwise equal
                assert_close(a, b, 0.0, f"pp {name}", exact=True)
    # odd niter is rejected
    rc = arch.lib.cg_stokes_pt_iterations_pp(arch.ctx, ctypes.byref(g), ctypes.byref(da), ctypes.byref(db), ctypes.byref(p), barr, 3)
    assert rc == _abi.CG_ERR_ARG


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("layout", ["8:0", "16:0", "24:0", "32:0", "48:0", "64:0"])
@pytest.mark.parametrize("dims", [(70, 33), (33, 97)])
def test_fused_2d_autotuner_layouts_give_the_same_bits(arch, monkeypatch, T, layout, dims):
    """Every one-iteration candidate of the 2D autotuner (segment lengths 8..64 rows, forced with
    CG_MARCH_LAYOUT=<segment length>:0) leaves the oracle's states bit for bit."""
    monkeypatch.setenv("CG_MARCH_LAYOUT", layout)
    s, partner, prev, _ = _pp_run(arch, T, dims, _bc_V(2), 6, seed=37)
    for name in ("V", "P", "tau", "divV", "r_V"):
        hv = s.h[name] if isinstance(s.h[name], list) else [s.h[name]]
        dv = s.d[name] if isinstance(s.d[name], list) else [s.d[name]]
        for a, b in zip(dv, hv):
            if b is not None:
                assert_close(a, b, 0.0, f"layout {layout} {name}", exact=True)
    for a, b in zip(partner["V"], prev):
        assert np.array_equal(a.to_numpy().view(np.uint8), b.view(np.uint8)), f"layout {layout}: partner V"


@pytest.mark.parametrize("layout", ["16:0", "32:0", "64:0", "0:1", "16:1", "32:1", "64:1",
                                    "0:2", "16:2", "32:2", "64:2", "0:3", "16:3", "32:3"])
@pytest.mark.parametrize("dims", [(31, 20, 70), (61, 7, 33), (95, 23, 17)])
def test_fused_3d_autotuner_layouts_give_the_same_bits(arch, monkeypatch, layout, dims):
    """Every candidate of the 3D autotuner (z-segment lengths x block shapes; forced with
    CG_MARCH_LAYOUT): march3d_kernel with 12 rows at 2 blocks per SM (variant 0) or 8 rows at 3
    (variant 1), and march3d_tma_kernel, its inputs staged by TMA, with 12 rows (variant 2) or 8
    (variant 3). On FP32 fields that share one row and plane stride, as the defect-correction
    pool lays them out: the oracle's states bit for bit. The grids put the tiles' first columns
    at every offset from a 16-byte boundary that strips of 30 columns reach."""
    monkeypatch.setenv("CG_MARCH_LAYOUT", layout)
    rows = dims[1] + 5
    # rows padded to 512 bytes: Center and Vertex rows of these grids get one row stride
    s, partner, prev, _ = _pp_run(arch, np.float32, dims, _bc_V(3), 4, seed=41, pitch_align=512, plane_rows=rows)
    strides = {f.data.stride()[:2] for v in s.d.values() for f in (v if isinstance(v, list) else [v]) if f is not None}
    assert len(strides) == 1, strides
    for name in ("V", "P", "tau", "divV", "r_V"):
        hv = s.h[name] if isinstance(s.h[name], list) else [s.h[name]]
        dv = s.d[name] if isinstance(s.d[name], list) else [s.d[name]]
        for a, b in zip(dv, hv):
            if b is not None:
                assert_close(a, b, 0.0, f"layout {layout} {name}", exact=True)
    for a, b in zip(partner["V"], prev):
        assert np.array_equal(a.to_numpy().view(np.uint8), b.view(np.uint8)), f"layout {layout}: partner V"


def test_staged_3d_wait_runs_out_and_the_context_stays_usable(arch, monkeypatch):
    """Failure detection of the TMA-fed 3D iteration without a GPU fault: the producing warp
    withholds the copies of one ring plane (CG_TMA_WITHHOLD_PLANE) and every wait is limited to
    20 ms (CG_TMA_WAIT_LIMIT_MS). The compute warps' waits for that plane run out and they stop
    together at their barrier; the producing warp's wait for their release runs out in turn,
    it waits (bounded) for its copies in flight, and cg_stokes_pt_iterations_pp reports
    CG_ERR_TIMEOUT. The same context then runs the iterations to the oracle's bits."""
    import time

    monkeypatch.setenv("CG_MARCH_LAYOUT", "16:2")
    monkeypatch.setenv("CG_TMA_WAIT_LIMIT_MS", "20")
    monkeypatch.setenv("CG_TMA_WITHHOLD_PLANE", "5")
    dims = (31, 20, 70)
    rows = dims[1] + 5
    t0 = time.perf_counter()
    with pytest.raises(_abi.ChmyError) as err:
        _pp_run(arch, np.float32, dims, _bc_V(3), 4, seed=41, pitch_align=512, plane_rows=rows)
    waited = time.perf_counter() - t0
    assert err.value.code == _abi.CG_ERR_TIMEOUT, str(err.value)
    assert "timed out" in str(err.value)
    assert waited < 20.0, waited  # the 20 ms limits applied, not the 2 s default
    monkeypatch.delenv("CG_TMA_WITHHOLD_PLANE")
    monkeypatch.delenv("CG_TMA_WAIT_LIMIT_MS")
    s, partner, prev, _ = _pp_run(arch, np.float32, dims, _bc_V(3), 4, seed=41, pitch_align=512, plane_rows=rows)
    for name in ("V", "P", "tau", "divV", "r_V"):
        hv = s.h[name] if isinstance(s.h[name], list) else [s.h[name]]
        dv = s.d[name] if isinstance(s.d[name], list) else [s.d[name]]
        for a, b in zip(dv, hv):
            if b is not None:
                assert_close(a, b, 0.0, f"after a timed-out run: {name}", exact=True)


def _bc_mix(kind):
    """Velocity boundary conditions with every foldable rule: Dirichlet on a Vertex dimension
    (a constant plane), Dirichlet on a Center dimension (2v - interior), Neumann on either,
    and sides left untouched."""
    if kind == "neumann_vertex":
        return [to_cg_bc(2, {"x": (Neumann(0.3), Neumann(-0.2)), "y": (Dirichlet(0.7), Dirichlet(-0.1))}),
                to_cg_bc(2, {"x": (Dirichlet(0.25), Dirichlet(0.5)), "y": (Neumann(-0.4), Neumann(0.6))})]
    if kind == "one_sided":
        return [to_cg_bc(2, {"x": (Dirichlet(0.2), None), "y": (None, Neumann(0.4))}),
                to_cg_bc(2, {"x": (None, Neumann(-0.3)), "y": (Dirichlet(0.1), None)})]
    return [to_cg_bc(2, {"x": (Neumann(0.1), Dirichlet(-0.6)), "y": Neumann(0.2)}),
            to_cg_bc(2, {"x": Dirichlet(0.3), "y": (Dirichlet(0.9), Neumann(0.05))})]


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("kind", ["neumann_vertex", "one_sided", "mixed"])
@pytest.mark.parametrize("dims", [(28, 29), (29, 30), (30, 28), (58, 33), (59, 7), (60, 61), (2, 3)])
@pytest.mark.parametrize("niter", [2, 6])
def test_fused_pingpong_boundary_rules(arch, T, kind, dims, niter):
    """The fused iterations read the previous iteration's velocity through bc!(V) and patch the
    boundary planes once at the end: both ping-pong buffers equal the oracle's states after
    niter and niter - 1 iterations bit for bit, for every Dirichlet/Neumann rule and for grids
    whose boundary planes fall on the edges of the kernel's 30-column strips."""
    s, partner, prev, _ = _pp_run(arch, T, dims, _bc_mix(kind), niter, seed=37)
    for name in ("V", "P", "tau"):
        hv = s.h[name] if isinstance(s.h[name], list) else [s.h[name]]
        dv = s.d[name] if isinstance(s.d[name], list) else [s.d[name]]
        for a, b in zip(dv, hv):
            assert_close(a, b, 0.0, f"pp {kind} {name}", exact=True)
    for a, b in zip(partner["V"], prev):
        got = a.to_numpy()
        assert np.array_equal(got.view(np.uint8), b.view(np.uint8)), f"partner V {kind}: max diff {np.max(np.abs(got - b))}"


def _thermal_set(arch, dims, T, seed):
    s = StokesSet(arch, dims, T, seed, True, thermal=True)
    # qT starts as a fresh (zero) field on the oracle side: the fused step reads zero beyond
    # the flux kernel's launch range exactly as the two-kernel form reads this allocation
    for f in s.h["qT"]:
        f.a[...] = 0
    return s


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(37, 29), (13, 11, 9)])
def test_thermal_step_fused_bitwise(arch, T, dims):
    """cg_stokes_thermal_step == update_thermal_flux!, update_thermal!, bc!(T) on the oracle, bit
    for bit (fluxes with both signs of V)."""
    s = _thermal_set(arch, dims, T, 41)
    p = pt_params(s.grid, True)
    g = s.grid.desc()
    nd = len(dims)
    bcT = to_cg_bc(nd, {"xyz"[d]: Neumann() for d in range(nd)})
    T_out = to_gpu(arch, s.h["T"])  # starts as a copy of T: points outside the launch range agree
    T0 = s.h["T"].a.copy()
    hd = s.host_desc()
    assert lib().or_stokes_update_thermal_flux(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p)) == 0
    assert lib().or_stokes_update_thermal(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p)) == 0
    bc_apply(s.grid, [s.h["T"]], [bcT])
    arch.call("cg_stokes_thermal_step", ctypes.byref(g), ctypes.byref(s.dev_desc()), ctypes.byref(p), ctypes.byref(bcT), ctypes.byref(T_out.desc()))
    arch.synchronize()
    assert_close(T_out, s.h["T"], 0.0, "thermal step", exact=True)
    assert np.array_equal(s.d["T"].to_numpy(), T0), "T is read only"


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("dims", [(31, 26), (12, 10, 11)])
@pytest.mark.parametrize("niter", [4, 5])
def test_pt_iterations_thermal(arch, T, dims, niter):
    """cg_stokes_pt_iterations_thermal == niter x (update_stress!, update_velocity!, bc!(V),
    update_thermal_flux!, update_thermal!, bc!(T)) on the oracle (odd niter ends in the partner
    buffer and is copied back)."""
    s = _thermal_set(arch, dims, T, 43)
    p = pt_params(s.grid, True)
    g = s.grid.desc()
    nd = len(dims)
    bcs = _bc_V(nd)
    bcT = to_cg_bc(nd, {"xyz"[d]: Neumann() for d in range(nd)})
    hd = s.host_desc()
    for _ in range(niter):
        lib().or_stokes_update_stress(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        lib().or_stokes_update_velocity(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        bc_apply(s.grid, s.h["V"], bcs)
        lib().or_stokes_update_thermal_flux(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        lib().or_stokes_update_thermal(ctypes.byref(g), ctypes.byref(hd), ctypes.byref(p))
        bc_apply(s.grid, [s.h["T"]], [bcT])
    arch.call("cg_stokes_pt_iterations_thermal", ctypes.byref(g), ctypes.byref(s.dev_desc()), ctypes.byref(p), (_abi.cg_bc * 3)(*bcs), ctypes.byref(bcT), niter)
    arch.synchronize()
    for name in ("V", "P", "tau", "T"):
        hv = s.h[name] if isinstance(s.h[name], list) else [s.h[name]]
        dv = s.d[name] if isinstance(s.d[name], list) else [s.d[name]]
        for a, b in zip(dv, hv):
            assert_close(a, b, rtol_for(T) * niter * 10, f"thermal PT {name}")


@pytest.mark.parametrize("T", TYPES)
@pytest.mark.parametrize("layout", ["0:1", "0:2", "8:1", "40:2"])
@pytest.mark.parametrize("kind", ["neumann_vertex", "one_sided", "mixed"])
@pytest.mark.parametrize("dims", [(28, 29), (57, 30), (29, 61), (2, 3), (85, 9)])
@pytest.mark.parametrize("niter", [6, 10])
def test_fused_two_iterations_per_pass(arch, monkeypatch, T, layout, kind, dims, niter):
    """The two-iterations-per-pass kernel (march2d_x2_kernel, forced with CG_MARCH_LAYOUT: segment
    length : variant) in the ping-pong loop: both buffers equal the oracle's states after niter
    and niter - 1 iterations bit for bit, for every rule mix, strip edges of its 28-column strips
    (28, 56, 84) and segment edges."""
    monkeypatch.setenv("CG_MARCH_LAYOUT", layout)
    # rows padded to 512 bytes: every array of these grids shares one row stride, which the
    # two-iteration kernel needs
    s, partner, prev, _ = _pp_run(arch, T, dims, _bc_mix(kind), niter, seed=53, pitch_align=512)
    strides = {f.data.stride()[-2] for v in s.d.values() for f in (v if isinstance(v, list) else [v]) if f is not None}
    assert len(strides) == 1, strides
    for name in ("V", "P", "tau", "divV", "r_V"):
        hv = s.h[name] if isinstance(s.h[name], list) else [s.h[name]]
        dv = s.d[name] if isinstance(s.d[name], list) else [s.d[name]]
        for a, b in zip(dv, hv):
            if b is not None:
                assert_close(a, b, 0.0, f"x2 {layout} {kind} {name}", exact=True)
    for a, b in zip(partner["V"], prev):
        got = a.to_numpy()
        assert np.array_equal(got.view(np.uint8), b.view(np.uint8)), f"partner V {kind}: max diff {np.max(np.abs(got - b))}"
