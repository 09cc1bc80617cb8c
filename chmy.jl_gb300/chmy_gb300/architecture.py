"""Arch for the GB300 backend (Chmy.jl src/Architectures.jl:21-74, ext/ChmyCUDAExt).

`Arch(GB300Backend(); device_id=1)` binds the process to one CUDA device (1-based like
Chmy's device_id) and owns a libchmy_gb300 context. PyTorch only provides device memory
and streams; all computation goes through the library.
"""

from __future__ import annotations

import ctypes

import torch

from . import _abi


class GB300Backend:
    """Backend tag (the role CUDABackend() plays for Chmy's CUDA extension)."""

    def __repr__(self):
        return "GB300Backend()"


class Arch:
    """SingleDeviceArchitecture on a GB300 (src/Architectures.jl:21-28,46-49)."""

    def __init__(self, backend: GB300Backend | None = None, device_id: int = 1):
        if backend is None:
            backend = GB300Backend()
        if not isinstance(backend, GB300Backend):
            raise TypeError(f"unsupported backend {backend!r}: only GB300Backend() is implemented")
        if not torch.cuda.is_available():
            raise RuntimeError("Arch(GB300Backend()) needs a CUDA device; none is visible")
        self.backend = backend
        self.device_id = int(device_id)
        self.device = torch.device("cuda", self.device_id - 1)
        torch.cuda.set_device(self.device)
        self.lib = _abi.load_library()
        ctx = ctypes.c_void_p()
        _abi.check(self.lib, self.lib.cg_init(self.device_id - 1, ctypes.byref(ctx)), "cg_init", None)
        self.ctx = ctx
        self._bind_stream()

    def _bind_stream(self) -> None:
        # Run library work on torch's current stream so that torch copies/fills and library
        # kernels are ordered without extra synchronisation.
        s = torch.cuda.current_stream(self.device).cuda_stream
        _abi.check(self.lib, self.lib.cg_set_stream(self.ctx, ctypes.c_void_p(s) if s else None), "cg_set_stream", self.ctx)

    def activate(self, priority: str = "normal") -> None:
        """activate!(arch; priority) (src/Architectures.jl:71-74)."""
        torch.cuda.set_device(self.device)
        self._bind_stream()

    def call(self, name: str, *args) -> None:
        rc = getattr(self.lib, name)(self.ctx, *args)
        _abi.check(self.lib, rc, name, self.ctx)

    def synchronize(self) -> None:
        """KernelAbstractions.synchronize(backend) (src/KernelLaunch.jl:117)."""
        self.call("cg_sync")

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.cg_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __repr__(self):
        return f"Arch({self.backend!r}; device_id={self.device_id})"


def get_backend(arch: Arch) -> GB300Backend:
    return arch.backend


def get_device(arch: Arch) -> torch.device:
    return arch.device


def heuristic_groupsize(arch: Arch, ndim: int) -> tuple[int, ...]:
    """Block shape used by the library's generic launches (the CUDA extension's (32, 8))."""
    return {1: (256,), 2: (32, 8), 3: (32, 8, 1)}[ndim]
