"""chmy_gb300 — Chmy.jl's staggered-grid hot path on GB300 (sm_103a).

Host-side mirror of Chmy's API surface (Arch, UniformGrid, Field/interior/set!, bc! with
batches, Launcher and the example kernels) over the C ABI of libchmy_gb300.so. Every
computation runs in the library's CUDA kernels; there is no CPU fallback.

Julia-to-Python name map: `set!` -> `set_`, `bc!` -> `bc_`, `f => bc` -> `(f, bc)`,
`launch(arch, grid, k => args; bc)` -> `launch(arch, grid, (k, args), bc=...)`.
"""

from ._abi import ChmyError, header_symbols, load_library
from .architecture import Arch, GB300Backend, get_backend, get_device, heuristic_groupsize
from .bcs import Batch, Dirichlet, Neumann, Periodic, batch, bc_
from .fields import Field, FieldMask, TensorField, VectorField, gather, gather_blocks, interior, set_
from .functions import FunctionField
from .grids import Center, Dim, Side, UniformGrid, Vertex, flip
from .kernels import (
    CellViscosity,
    Launcher,
    compute_q,
    stokes_fields,
    stokes_params,
    update_C,
    update_old,
    update_stress,
    update_thermal,
    update_thermal_flux,
    update_velocity,
)

__all__ = [
    "Arch",
    "Batch",
    "CellViscosity",
    "Center",
    "ChmyError",
    "Dim",
    "Dirichlet",
    "Field",
    "GB300Backend",
    "Launcher",
    "Neumann",
    "Periodic",
    "Side",
    "TensorField",
    "UniformGrid",
    "VectorField",
    "Vertex",
    "batch",
    "bc_",
    "compute_q",
    "flip",
    "get_backend",
    "get_device",
    "header_symbols",
    "heuristic_groupsize",
    "interior",
    "gather",
    "FieldMask",
    "FunctionField",
    "gather_blocks",
    "load_library",
    "set_",
    "stokes_fields",
    "stokes_params",
    "update_C",
    "update_old",
    "update_stress",
    "update_thermal",
    "update_thermal_flux",
    "update_velocity",
]
