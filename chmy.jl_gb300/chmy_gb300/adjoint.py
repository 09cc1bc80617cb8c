"""Adjoints of the time loops, by reverse time stepping over checkpoints.

PTDiffusion: the implicit variable-coefficient diffusion steps (cg_ptdiff_run). The gradient of
a misfit of the final state with respect to the per-cell diffusivity D and to the initial state.

One step is C' = S C with S = (I - dt L_D)^-1, L_D C = divg(lerp(D) d C). I - dt L_D is symmetric
on the interior cells (the boundary rules folded in), so the adjoint of a step is the same PT
step: lambda^n = S lambda^{n+1}. The gradient with respect to D sums one term per step,
cg_ptdiff_gradient_D(lambda^n, C^{n+1}, dt). The reverse sweep needs C^{n+1} in reverse order:
every `checkpoint_every`-th state (with the PT flux, the rest of the state) is kept during the
forward sweep, and each segment is recomputed from its checkpoint before it is swept back.
Memory: nsteps / checkpoint_every + checkpoint_every states.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _abi
from .fields import Field
from .grids import Center, Vertex


def _zero_bc(bc: _abi.cg_bc) -> _abi.cg_bc:
    b = _abi.cg_bc()
    ctypes.memmove(ctypes.byref(b), ctypes.byref(bc), ctypes.sizeof(b))
    for d in range(3):
        for s in range(2):
            b.value[d][s] = 0.0
            b.values[d][s] = None
    return b


class PTDiffusion:
    """Implicit diffusion steps on device fields (C, C_old, D, q) with their adjoint."""

    def __init__(self, arch, grid, D: np.ndarray, params, bc: _abi.cg_bc, npt: int, dtype=np.float64):
        self.arch, self.grid, self.params, self.bc, self.npt = arch, grid, params, bc, int(npt)
        self.bc0 = _zero_bc(bc)
        nd = grid.ndim
        self.nd = nd
        C = Center()
        qloc = [tuple(Vertex() if e == d else C for e in range(nd)) for d in range(nd)]

        def fset():
            return {
                "C": Field(arch, grid, C, dtype),
                "C_old": Field(arch, grid, C, dtype),
                "q": [Field(arch, grid, l, dtype) for l in qloc],
            }

        self.D = Field(arch, grid, C, dtype)
        self.D.from_numpy(D)
        self.fwd, self.adj = fset(), fset()
        self.gD = Field(arch, grid, C, dtype)

    def _desc(self, fs):
        s = _abi.cg_ptdiff_fields()
        s.C, s.C_old, s.D = fs["C"].desc(), fs["C_old"].desc(), self.D.desc()
        s.q = (_abi.cg_field * 3)(*[f.desc() for f in fs["q"]])
        return s

    def _steps(self, fs, bc, nsteps: int) -> None:
        if nsteps <= 0:
            return
        self.arch.call("cg_ptdiff_run", ctypes.byref(self.grid.desc()), ctypes.byref(self._desc(fs)), ctypes.byref(self.params),
                       ctypes.byref(bc), int(nsteps), self.npt)

    def _save(self):
        return [self.fwd["C"].data.clone()] + [f.data.clone() for f in self.fwd["q"]]

    def _restore(self, st) -> None:
        self.fwd["C"].data.copy_(st[0])
        for f, s in zip(self.fwd["q"], st[1:]):
            f.data.copy_(s)

    def run(self, C0: np.ndarray, nsteps: int) -> np.ndarray:
        """Forward: `nsteps` implicit steps from C0 (flux starting at zero); returns C^N."""
        self.fwd["C"].from_numpy(C0)
        for f in self.fwd["q"]:
            f.data.zero_()
        self._steps(self.fwd, self.bc, nsteps)
        return self.fwd["C"].to_numpy()

    def gradient(self, C0: np.ndarray, nsteps: int, misfit_grad, checkpoint_every: int | None = None):
        """Gradients of J(C^N) with respect to D (per cell) and to C0. `misfit_grad(CN)` returns
        dJ/dC^N as a padded host array (zero outside the interior). Returns (dJ/dD, dJ/dC0, C^N)
        as padded host arrays."""
        K = int(checkpoint_every or max(1, math.ceil(math.sqrt(nsteps))))
        self.fwd["C"].from_numpy(C0)
        for f in self.fwd["q"]:
            f.data.zero_()
        checkpoints = {}
        for n in range(nsteps):
            if n % K == 0:
                checkpoints[n] = self._save()
            self._steps(self.fwd, self.bc, 1)
        CN = self.fwd["C"].to_numpy()
        self.adj["C"].from_numpy(misfit_grad(CN))
        self.gD.data.zero_()
        dt = float(self.params.dt)
        g = self.grid.desc()
        for start in sorted(checkpoints, reverse=True):
            stop = min(start + K, nsteps)
            # recompute this segment's states C^{start+1} .. C^{stop}
            self._restore(checkpoints[start])
            states = []
            for _ in range(start, stop):
                self._steps(self.fwd, self.bc, 1)
                states.append(self.fwd["C"].data.clone())
            for n in range(stop - 1, start - 1, -1):
                # lambda^n = S lambda^{n+1}: one PT step with C_old = lambda^{n+1}, zero boundary values
                for f in self.adj["q"]:
                    f.data.zero_()
                self._steps(self.adj, self.bc0, 1)
                Cn1 = self.fwd["C"]
                Cn1.data.copy_(states[n - start])
                self.arch.call("cg_ptdiff_gradient_D", ctypes.byref(g), ctypes.byref(self.adj["C"].desc()), ctypes.byref(Cn1.desc()),
                               dt, ctypes.byref(self.gD.desc()))
            del states
        return self.gD.to_numpy(), self.adj["C"].to_numpy(), CN


class ExplicitDiffusion:
    """The explicit diffusion loop of examples/diffusion_2d.jl:43-47 (cg_diffusion_run: the fused
    flux + update step, then bc!(C)) and its adjoint: the gradient of a misfit J(C^N) with respect
    to the diffusivity chi and to the initial state, by reverse time stepping.

    cg_diffusion_run_taped records the states C^0 .. C^N (the reverse step needs C^n and C^{n+1}
    for dJ/dchi), and cg_diffusion_adjoint_run sweeps them back in one call. The whole run is one
    taped segment when its tape fits `tape_budget` bytes (default: half the free device memory).
    Otherwise a plain forward run keeps the start state of every segment of K steps, and each
    segment, from the last, is re-run taped from its checkpoint and swept back (checkpointed
    reverse time stepping with recomputation; K = the most steps whose tape fits)."""

    def __init__(self, arch, grid, chi: float, dt: float, bc: _abi.cg_bc, dtype=np.float64):
        self.arch, self.grid, self.chi, self.dt, self.bc = arch, grid, float(chi), float(dt), bc
        C = Center()
        self.C = Field(arch, grid, C, dtype)
        self.B = Field(arch, grid, C, dtype)
        self.lam = [Field(arch, grid, C, dtype), Field(arch, grid, C, dtype)]
        self._tape = None

    def tape_bytes(self, nsteps: int) -> int:
        """Device bytes of a tape of `nsteps` steps."""
        b = ctypes.c_size_t()
        rc = self.arch.lib.cg_diffusion_tape_bytes(ctypes.byref(self.grid.desc()), ctypes.byref(self.C.desc()), int(nsteps),
                                                   ctypes.byref(b))
        if rc != 0:
            raise ValueError("cg_diffusion_tape_bytes: bad arguments")
        return int(b.value)

    def _tape_buffer(self, nbytes: int):
        import torch

        if self._tape is None or self._tape.numel() < nbytes:
            self._tape = None
            # zeroed: the states' outer halo layer, which no step writes, then holds zeros
            self._tape = torch.zeros(nbytes, dtype=torch.uint8, device=self.C.data.device)
            if self._tape.data_ptr() % 256:
                raise RuntimeError("the tape allocation is not 256-byte aligned")
        return self._tape

    def _apply_bc(self) -> None:
        self.arch.call("cg_bc_apply", ctypes.byref(self.grid.desc()), 1, ctypes.byref(self.C.desc()), ctypes.byref(self.bc))

    def _steps(self, nsteps: int) -> None:
        """`nsteps` plain steps of C in place (ping-pong with B)."""
        if nsteps <= 0:
            return
        self.B.data.copy_(self.C.data)  # the partner's outer halo (never written) matches C's
        self.arch.call("cg_diffusion_run", ctypes.byref(self.grid.desc()), ctypes.byref(self.C.desc()), ctypes.byref(self.B.desc()),
                       self.chi, self.dt, ctypes.byref(self.bc), int(nsteps))
        if nsteps % 2:
            self.C.data.copy_(self.B.data)

    def run(self, C0: np.ndarray, nsteps: int) -> np.ndarray:
        """Forward: bc!(C0), then `nsteps` steps; returns C^N (padded)."""
        self.C.from_numpy(C0)
        self._apply_bc()
        self._steps(nsteps)
        return self.C.to_numpy()

    def _segment(self, nsteps: int) -> int:
        """`nsteps` taped steps of C in place; returns the tape's size."""
        nbytes = self.tape_bytes(nsteps)
        tape = self._tape_buffer(nbytes)
        self.arch.call("cg_diffusion_run_taped", ctypes.byref(self.grid.desc()), ctypes.byref(self.C.desc()), self.chi, self.dt,
                       ctypes.byref(self.bc), int(nsteps), ctypes.c_void_p(tape.data_ptr()), nbytes)
        return nbytes

    def gradient(self, C0: np.ndarray, nsteps: int, misfit_grad, checkpoint_every: int | None = None,
                 tape_budget: int | None = None):
        """(dJ/dchi, dJ/dC0, C^N). `misfit_grad(CN)` returns dJ/dC^N as a padded host array (its
        interior is used); dJ/dC0 is a padded host array whose interior holds the gradient with
        respect to the interior of C0 (the ghost cells follow it through bc!).
        `checkpoint_every` caps the taped segment length."""
        import torch

        if tape_budget is None:
            free, _ = torch.cuda.mem_get_info(self.C.data.device)
            tape_budget = free // 2
        per_step = self.tape_bytes(1) - self.tape_bytes(0)
        K = max(1, min(nsteps, (int(tape_budget) - self.tape_bytes(0)) // per_step))
        if checkpoint_every:
            K = min(K, int(checkpoint_every))
        self.C.from_numpy(C0)
        self._apply_bc()
        starts = list(range(0, nsteps, K))
        checkpoints = {}
        for start in starts[:-1]:  # plain forward up to the last segment, keeping its start states
            checkpoints[start] = self.C.data.clone()
            self._steps(K)
        last = starts[-1]
        nbytes = self._segment(nsteps - last)
        CN = self.C.to_numpy()
        self.lam[0].from_numpy(misfit_grad(CN))
        dJ = (ctypes.c_double * 1)(0.0)
        g = self.grid.desc()

        def sweep(nb):
            self.arch.call("cg_diffusion_adjoint_run", ctypes.byref(g), ctypes.c_void_p(self._tape.data_ptr()), nb,
                           ctypes.byref(self.lam[0].desc()), ctypes.byref(self.lam[1].desc()), self.chi, self.dt,
                           ctypes.byref(self.bc), dJ)

        sweep(nbytes)
        for start in reversed(starts[:-1]):
            self.C.data.copy_(checkpoints.pop(start))
            sweep(self._segment(K))
        return dJ[0], self.lam[0].to_numpy(), CN


class SIA:
    """The shallow-ice time loop of cg_sia_run (examples/sia.jl:71-81 with the flux
    -Gamma H^(n+2) |∇S|^(n-1) ∇S, adaptive Δt and linear mass balance capped at m_max) and its
    adjoint: the gradient of a misfit J(H^N) with respect to Gamma and ela, and to the initial
    thickness, by reverse time stepping over checkpoints.

    A step reads only H (the flux is recomputed from it), so a checkpoint is one copy of H.
    Two reverse sweeps:
    - taped (default): cg_sia_run_taped records, per step, what the reverse step needs (about
      9 arrays of H's size), and cg_sia_adjoint_run sweeps a whole segment in one call without
      recomputing anything. The whole run is one segment when its tape fits `tape_budget`
      bytes (default: half the free device memory), else segments of as many steps as fit,
      each re-run taped from its checkpoint.
    - recomputing (tape=False): the forward keeps every `checkpoint_every`-th state; the
      reverse recomputes each segment's states from its checkpoint and runs
      cg_sia_adjoint_step over them backwards. Memory: nsteps / checkpoint_every +
      checkpoint_every states."""

    def __init__(self, arch, grid, B: np.ndarray, params, dtype=np.float64):
        self.arch, self.grid, self.params = arch, grid, params
        C = Center()
        self.H = Field(arch, grid, C, dtype)
        self.B = Field(arch, grid, C, dtype)
        self.B.from_numpy(B)
        self.q = [Field(arch, grid, (Vertex(), C), dtype), Field(arch, grid, (C, Vertex()), dtype)]
        self.lam = [Field(arch, grid, C, dtype), Field(arch, grid, C, dtype)]
        self._q = (_abi.cg_field * 3)(self.q[0].desc(), self.q[1].desc(), _abi.cg_field())
        self._tape = None

    def tape_bytes(self, nsteps: int) -> int:
        """Device bytes of a tape of `nsteps` steps."""
        b = ctypes.c_size_t()
        rc = self.arch.lib.cg_sia_tape_bytes(ctypes.byref(self.grid.desc()), ctypes.byref(self.H.desc()), int(nsteps), ctypes.byref(b))
        if rc != 0:
            raise ValueError("cg_sia_tape_bytes: bad arguments")
        return int(b.value)

    def _tape_buffer(self, nbytes: int):
        import torch

        if self._tape is None or self._tape.numel() < nbytes:
            self._tape = None
            self._tape = torch.empty(nbytes, dtype=torch.uint8, device=self.H.data.device)
            if self._tape.data_ptr() % 256:
                raise RuntimeError("the tape allocation is not 256-byte aligned")
        return self._tape

    def _steps_taped(self, nsteps: int) -> None:
        nbytes = self.tape_bytes(nsteps)
        tape = self._tape_buffer(nbytes)
        self.arch.call("cg_sia_run_taped", ctypes.byref(self.grid.desc()), ctypes.byref(self.H.desc()), ctypes.byref(self.B.desc()),
                       self._q, ctypes.byref(self.params), int(nsteps), ctypes.c_void_p(tape.data_ptr()), nbytes, None)

    def _reverse_taped(self, dJ) -> None:
        """Reverse sweep over the tape of the last _steps_taped call: lam[0] in and out."""
        self.arch.call("cg_sia_adjoint_run", ctypes.byref(self.grid.desc()), ctypes.byref(self.params),
                       ctypes.c_void_p(self._tape.data_ptr()), self._tape.numel(), ctypes.byref(self.lam[0].desc()),
                       ctypes.byref(self.lam[1].desc()), dJ)

    def _steps(self, nsteps: int, timed: bool = False) -> float:
        """`nsteps` forward steps in one call; the model time (which synchronises) if `timed`."""
        t = ctypes.c_double()
        if nsteps > 0:
            self.arch.call("cg_sia_run", ctypes.byref(self.grid.desc()), ctypes.byref(self.H.desc()), ctypes.byref(self.B.desc()),
                           self._q, ctypes.byref(self.params), int(nsteps), ctypes.byref(t) if timed else None)
        return t.value

    def run(self, H0: np.ndarray, nsteps: int) -> np.ndarray:
        """Forward: `nsteps` steps from H0; returns H^N (padded)."""
        self.H.from_numpy(H0)
        self._steps(nsteps)
        return self.H.to_numpy()

    def reset_accumulators(self) -> None:
        """Drop dJ/dGamma and dJ/dela sums left on the device by an interrupted reverse sweep."""
        tmp = (ctypes.c_double * 2)()
        self.arch.call("cg_sia_adjoint_step", ctypes.byref(self.grid.desc()), ctypes.byref(self.H.desc()), ctypes.byref(self.B.desc()),
                       ctypes.byref(self.params), ctypes.byref(self.lam[0].desc()), ctypes.byref(self.lam[1].desc()), tmp)

    def gradient(self, H0: np.ndarray, nsteps: int, misfit_grad, checkpoint_every: int | None = None, tape: bool = True,
                 tape_budget: int | None = None):
        """(dJ/dGamma, dJ/dela, dJ/dH0, H^N). `misfit_grad(HN)` returns dJ/dH^N as a padded host
        array (its interior is used). With `tape`, `checkpoint_every` caps the segment length
        (default: the whole run if its tape fits `tape_budget`)."""
        if tape:
            return self._gradient_taped(H0, nsteps, misfit_grad, checkpoint_every, tape_budget)
        K = int(checkpoint_every or max(1, math.ceil(math.sqrt(nsteps))))
        self.H.from_numpy(H0)
        self.reset_accumulators()
        checkpoints = {}
        for n in range(0, nsteps, K):
            checkpoints[n] = self.H.data.clone()
            self._steps(min(K, nsteps - n))
        HN = self.H.to_numpy()
        self.lam[0].from_numpy(misfit_grad(HN))
        dJ = (ctypes.c_double * 2)(0.0, 0.0)
        g = self.grid.desc()
        cur = 0
        for start in sorted(checkpoints, reverse=True):
            stop = min(start + K, nsteps)
            self.H.data.copy_(checkpoints[start])
            states = [self.H.data.clone()]
            for _ in range(start + 1, stop):  # H^start+1 .. H^stop-1 (H^stop is not needed)
                self._steps(1)
                states.append(self.H.data.clone())
            for n in range(stop - 1, start - 1, -1):
                self.H.data.copy_(states[n - start])
                # dJ/dGamma and dJ/dela accumulate on the device; the last step reads them
                self.arch.call("cg_sia_adjoint_step", ctypes.byref(g), ctypes.byref(self.H.desc()), ctypes.byref(self.B.desc()),
                               ctypes.byref(self.params), ctypes.byref(self.lam[cur].desc()), ctypes.byref(self.lam[1 - cur].desc()),
                               dJ if n == 0 else None)
                cur = 1 - cur
            del states
        return dJ[0], dJ[1], self.lam[cur].to_numpy(), HN

    def _gradient_taped(self, H0, nsteps, misfit_grad, checkpoint_every, tape_budget):
        import torch

        if tape_budget is None:
            free, _ = torch.cuda.mem_get_info(self.H.data.device)
            tape_budget = free // 2
        per_step = self.tape_bytes(1) - self.tape_bytes(0)
        K = max(1, min(nsteps, (int(tape_budget) - self.tape_bytes(0)) // per_step))
        if checkpoint_every:
            K = min(K, int(checkpoint_every))
        self.H.from_numpy(H0)
        starts = list(range(0, nsteps, K))
        checkpoints = {}
        for start in starts[:-1]:  # plain forward up to the last segment, keeping its start states
            checkpoints[start] = self.H.data.clone()
            self._steps(K)
        last = starts[-1]
        self._steps_taped(nsteps - last)
        HN = self.H.to_numpy()
        self.lam[0].from_numpy(misfit_grad(HN))
        dJ = (ctypes.c_double * 2)(0.0, 0.0)
        self._reverse_taped(dJ)
        for start in reversed(starts[:-1]):
            self.H.data.copy_(checkpoints.pop(start))
            self._steps_taped(K)
            self._reverse_taped(dJ)
        return dJ[0], dJ[1], self.lam[0].to_numpy(), HN


class SIAEnsemble:
    """An ensemble of independent SIA solves of uneven sizes (cg_sia_ensemble_run: every phase of
    a step is one launch over all members) and its adjoint: per member, the gradient of a
    misfit J_m(H_m^N) with respect to Gamma_m, ela_m and the initial thickness.

    The reverse sweep is taped: cg_sia_ensemble_run_taped records every member's reverse-step
    quantities, and cg_sia_ensemble_adjoint_run sweeps them back, all members in each launch.
    The whole run is one segment when its tape fits `tape_budget` bytes (default: half the free
    device memory). Otherwise the forward keeps every member's H at the start of each segment
    of K steps, and each segment is re-run taped before it is swept back."""

    def __init__(self, arch, members, dtype=np.float64):
        """`members`: a list of (grid, B, cg_sia_params) with B a padded host array."""
        self.arch = arch
        self.nm = len(members)
        C = Center()
        self.grids, self.params, self.H, self.B, self.q, self.lam, self.work = [], [], [], [], [], [], []
        for grid, B, p in members:
            self.grids.append(grid)
            self.params.append(p)
            H = Field(arch, grid, C, dtype)
            Bf = Field(arch, grid, C, dtype)
            Bf.from_numpy(B)
            self.H.append(H)
            self.B.append(Bf)
            self.q.append([Field(arch, grid, (Vertex(), C), dtype), Field(arch, grid, (C, Vertex()), dtype)])
            self.lam.append(Field(arch, grid, C, dtype))
            self.work.append(Field(arch, grid, C, dtype))
        self._mem = (_abi.cg_sia_member * self.nm)()
        self._par = (_abi.cg_sia_params * self.nm)(*self.params)
        for k in range(self.nm):
            self._mem[k].grid = self.grids[k].desc()
            self._mem[k].H, self._mem[k].B = self.H[k].desc(), self.B[k].desc()
            self._mem[k].q[0], self._mem[k].q[1] = self.q[k][0].desc(), self.q[k][1].desc()
        self._lam = (_abi.cg_field * self.nm)(*[f.desc() for f in self.lam])
        self._work = (_abi.cg_field * self.nm)(*[f.desc() for f in self.work])
        self._tape = None

    def tape_bytes(self, nsteps: int) -> int:
        b = ctypes.c_size_t()
        if self.arch.lib.cg_sia_ensemble_tape_bytes(self.nm, self._mem, int(nsteps), ctypes.byref(b)) != 0:
            raise ValueError("cg_sia_ensemble_tape_bytes: bad arguments")
        return int(b.value)

    def _set(self, H0s) -> None:
        for H, h0 in zip(self.H, H0s):
            H.from_numpy(h0)

    def _steps(self, nsteps: int) -> None:
        if nsteps > 0:
            self.arch.call("cg_sia_ensemble_run", self.nm, self._mem, self._par, int(nsteps), None)

    def _steps_taped(self, nsteps: int) -> None:
        import torch

        nbytes = self.tape_bytes(nsteps)
        if self._tape is None or self._tape.numel() < nbytes:
            self._tape = None
            self._tape = torch.empty(nbytes, dtype=torch.uint8, device=self.H[0].data.device)
            if self._tape.data_ptr() % 256:
                raise RuntimeError("the tape allocation is not 256-byte aligned")
        self.arch.call("cg_sia_ensemble_run_taped", self.nm, self._mem, self._par, int(nsteps), ctypes.c_void_p(self._tape.data_ptr()),
                       nbytes, None)

    def _reverse(self, dJ) -> None:
        self.arch.call("cg_sia_ensemble_adjoint_run", self.nm, self._mem, self._par, ctypes.c_void_p(self._tape.data_ptr()),
                       self._tape.numel(), self._lam, self._work, dJ)

    def run(self, H0s, nsteps: int):
        """Forward: `nsteps` steps from the padded host arrays H0s; returns the H^N arrays."""
        self._set(H0s)
        self._steps(nsteps)
        return [H.to_numpy() for H in self.H]

    def gradient(self, H0s, nsteps: int, misfit_grad, checkpoint_every: int | None = None, tape_budget: int | None = None):
        """(dJ/dGamma [m], dJ/dela [m], dJ/dH0 [m], H^N [m]). `misfit_grad(m, HN_m)` returns
        dJ/dH_m^N as a padded host array (its interior is used)."""
        import torch

        if tape_budget is None:
            free, _ = torch.cuda.mem_get_info(self.H[0].data.device)
            tape_budget = free // 2
        per_step = self.tape_bytes(1) - self.tape_bytes(0)
        K = max(1, min(nsteps, (int(tape_budget) - self.tape_bytes(0)) // per_step))
        if checkpoint_every:
            K = min(K, int(checkpoint_every))
        self._set(H0s)
        starts = list(range(0, nsteps, K))
        checkpoints = {}
        for start in starts[:-1]:
            checkpoints[start] = [H.data.clone() for H in self.H]
            self._steps(K)
        self._steps_taped(nsteps - starts[-1])
        HN = [H.to_numpy() for H in self.H]
        for m in range(self.nm):
            self.lam[m].from_numpy(misfit_grad(m, HN[m]))
        dJ = (ctypes.c_double * (2 * self.nm))()
        self._reverse(dJ)
        for start in reversed(starts[:-1]):
            for H, c in zip(self.H, checkpoints.pop(start)):
                H.data.copy_(c)
            self._steps_taped(K)
            self._reverse(dJ)
        return ([dJ[2 * m] for m in range(self.nm)], [dJ[2 * m + 1] for m in range(self.nm)],
                [f.to_numpy() for f in self.lam], HN)
