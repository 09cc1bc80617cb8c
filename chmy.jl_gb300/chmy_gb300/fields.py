"""Field, VectorField, TensorField, interior and set! (Chmy.jl src/Fields/field.jl).

A Field stores its padded array (extent n + 4H per dimension, x fastest) in a torch CUDA
tensor. The tensor is indexed [z, y, x] (C order, reversed dims); `interior(f)` returns a
view indexed [x, y, z] like Chmy's column-major `interior`.
"""

from __future__ import annotations

from collections import namedtuple

import numpy as np
import torch

from . import _abi
from .grids import Center, Location, UniformGrid, Vertex, expand_loc

_TORCH = {np.float32: torch.float32, np.float64: torch.float64}
_CODE = {np.float32: _abi.CG_F32, np.float64: _abi.CG_F64}


def _np_type(dtype) -> type:
    if dtype in (torch.float32, np.float32, "float32", "f32"):
        return np.float32
    if dtype in (torch.float64, np.float64, "float64", "f64", float):
        return np.float64
    if isinstance(dtype, np.dtype):
        return dtype.type
    raise TypeError(f"unsupported field type {dtype!r}")


class Field:
    """Field(arch, grid, loc, type=eltype(grid); halo=1) (src/Fields/field.jl:56-62).

    `pitch_align` (bytes, 0 = dense Chmy layout) pads x rows so that logical x index
    `align_index` (default 0; -1 = the first padded element) of each row is aligned. The fused
    kernels read every row from index -1: with `align_index=-1` a row of n + 4 elements spans the
    fewest 128-byte lines, which is what DRAM moves. `plane_rows` (3D, with `pitch_align`) pads
    every z plane to that many rows. Fields of different locations then share their row and
    plane strides, and the fused kernels address them all with one offset."""

    def __init__(self, arch, grid: UniformGrid, loc, dtype=None, halo=1, pitch_align: int = 0, plane_rows: int = 0,
                 align_index: int = 0):
        self.arch = arch
        self.grid = grid
        nd = grid.ndim
        self.loc = expand_loc(nd, loc)
        self.dtype = _np_type(dtype if dtype is not None else grid.dtype)
        self.halo = tuple(halo) if isinstance(halo, (tuple, list)) else tuple(int(halo) for _ in range(nd))
        if any(h < 1 for h in self.halo):
            raise ValueError("the GB300 kernels need halo >= 1 in every dimension")
        self.dims = grid.size(self.loc)
        self.ext = tuple(n + 4 * h for n, h in zip(self.dims, self.halo))
        tdt = _TORCH[self.dtype]
        esz = np.dtype(self.dtype).itemsize
        dev = arch.device
        if pitch_align:
            a = pitch_align // esz
            front = (a - (2 * self.halo[0] - 1 + align_index) % a) % a
            pitch = ((front + self.ext[0] + a - 1) // a) * a
            outer = list(reversed(self.ext[1:]))
            if nd == 3 and plane_rows:
                if plane_rows < self.ext[1]:
                    raise ValueError(f"plane_rows {plane_rows} < {self.ext[1]} rows of this field")
                outer[-1] = plane_rows
            storage = torch.zeros(tuple(outer) + (pitch,), dtype=tdt, device=dev)
            self._storage = storage
            self.data = storage[..., : self.ext[1], front : front + self.ext[0]] if nd == 3 else storage[..., front : front + self.ext[0]]
        else:
            self._storage = None
            self.data = torch.zeros(tuple(reversed(self.ext)), dtype=tdt, device=dev)

    @property
    def ndim(self) -> int:
        return len(self.dims)

    def location(self) -> tuple[Location, ...]:
        return self.loc

    def size(self) -> tuple[int, ...]:
        return self.dims

    def desc(self) -> _abi.cg_field:
        strides = tuple(reversed(self.data.stride()))
        return _abi.make_field(
            self.data.data_ptr(),
            _CODE[self.dtype],
            self.dims,
            tuple(l.code for l in self.loc),
            self.halo,
            strides,
        )

    # -- host transfer helpers (padded array, stored [z, y, x]) --
    def to_numpy(self) -> np.ndarray:
        return self.data.detach().cpu().numpy().copy()

    def from_numpy(self, arr: np.ndarray) -> None:
        arr = np.asarray(arr, dtype=self.dtype)
        if arr.shape != tuple(reversed(self.ext)):
            raise ValueError(f"expected padded shape {tuple(reversed(self.ext))}, got {arr.shape}")
        self.data.copy_(torch.from_numpy(np.ascontiguousarray(arr)))

    def __repr__(self):
        return f"Field(dims={self.dims}, loc={self.loc}, dtype={self.dtype.__name__}, halo={self.halo})"


def interior(f: Field, with_halo: bool = False) -> torch.Tensor:
    """interior(f; with_halo=false) (src/Fields/field.jl:33-37) as an [x, y, z] view."""
    sl = []
    for n, h in zip(reversed(f.dims), reversed(f.halo)):
        lo = 2 * h - (h if with_halo else 0)
        hi = 2 * h + n + (h if with_halo else 0)
        sl.append(slice(lo, hi))
    v = f.data[tuple(sl)]
    return v.permute(*reversed(range(f.ndim)))


class FieldMask:
    """FieldMask(arch, grid, type) (src/GridOperators/field_mask.jl:1-117): one weight field at
    each of the 2^N locations, read by the masked operators as at(ω, loc, I). `at(loc)` returns
    the field at a location; `desc()` is the library's cg_mask, indexed by location bits
    (Vertex along d = bit d)."""

    def __init__(self, arch, grid: UniformGrid, dtype=None, **field_kwargs):
        from .grids import Center, Vertex

        self.grid = grid
        nd = grid.ndim
        self.fields = {}
        for bits in range(1 << nd):
            loc = tuple(Vertex() if (bits >> d) & 1 else Center() for d in range(nd))
            self.fields[bits] = Field(arch, grid, loc, dtype, **field_kwargs)

    def at(self, loc) -> Field:
        from .grids import Vertex, expand_loc

        locs = expand_loc(self.grid.ndim, loc)
        return self.fields[sum(1 << d for d, l in enumerate(locs) if isinstance(l, Vertex))]

    def desc(self) -> _abi.cg_mask:
        m = _abi.cg_mask()
        for bits, f in self.fields.items():
            m.at[bits] = f.desc()
        return m


def gather(f: Field, dst: np.ndarray | None = None, path=None) -> np.ndarray:
    """gather!(arch, dst, src::Field) (src/Distributed/gather.jl:36-42) on one GPU: the interior
    of `f` in a host array, x fastest (Julia's column-major order of the [x, y, z] interior,
    stored here as a C-ordered [z, y, x] array). With `dst`, the values go there (its shape must
    match). With `path`, the bytes are also written as a headless dump in that order."""
    sl = tuple(slice(2 * h, 2 * h + n) for n, h in zip(reversed(f.dims), reversed(f.halo)))
    a = f.data[sl].detach().cpu().numpy()
    if dst is None:
        dst = np.ascontiguousarray(a)
    else:
        if dst.shape != a.shape:
            raise ValueError(f"gather: destination shape {dst.shape} != interior {a.shape}")
        dst[...] = a
    if path is not None:
        np.ascontiguousarray(dst).tofile(path)
    return dst


def gather_blocks(blocks, dims) -> np.ndarray:
    """The global array that gather! assembles from the local interiors of a Cartesian
    decomposition (src/Distributed/gather.jl:9-33). `blocks[r]` is rank r's interior ([z, y, x]
    stored, all of one shape). Rank r sits at the coordinates MPI_Cart_coords gives it for the
    topology `dims` (x first): row-major, so the last dimension varies fastest. This is the
    order of gather!'s displacements, which it builds over the reversed dims. The block at
    coordinates (cx, cy, cz) fills [cz*nz:(cz+1)*nz, cy*ny:..., cx*nx:...]."""
    dims = tuple(int(d) for d in dims)
    nd = len(dims)
    shp = blocks[0].shape
    if len(blocks) != int(np.prod(dims)) or any(b.shape != shp for b in blocks):
        raise ValueError("gather_blocks: one block of one shape per rank")
    out = np.empty(tuple(s * d for s, d in zip(shp, reversed(dims))), dtype=blocks[0].dtype)
    for r, b in enumerate(blocks):
        c, rem = [], r
        for d in reversed(range(nd)):  # row-major over (dims[0], ..., dims[N-1]): the last dim fastest
            c.append(rem % dims[d])
            rem //= dims[d]
        c = list(reversed(c))  # c[d] = coordinate along dimension d
        sl = tuple(slice(c[d] * shp[nd - 1 - d], (c[d] + 1) * shp[nd - 1 - d]) for d in reversed(range(nd)))
        out[sl] = b
    return out


def evaluate(grid: UniformGrid, loc, dims, fun, discrete: bool = False, parameters=(), dtype=np.float64) -> np.ndarray:
    """Values of `fun` on the interior points of a field at `loc`, [x, y, z] indexed: the
    continuous form calls fun(coords..., params...) (_set_continuous!, field.jl:121-124); the
    discrete form calls fun(grid, loc, I..., params...) (_set_discrete!, field.jl:126-129)."""
    if discrete:
        out = np.empty(dims, dtype=dtype)
        for idx in np.ndindex(*dims):
            I = tuple(i + 1 for i in idx)
            out[idx] = fun(grid, loc, *I, *parameters)
        return out
    axes = [grid.coords(loc, d + 1) for d in range(len(dims))]
    mesh = np.meshgrid(*axes, indexing="ij")
    out = np.asarray(fun(*mesh, *parameters), dtype=dtype)
    # a writable copy (broadcast_to returns a read-only view, even of a full-size array)
    return np.array(np.broadcast_to(out, dims), dtype=dtype, order="C")


def set_(f: Field, value, grid: UniformGrid | None = None, *, discrete: bool = False, parameters=()) -> None:
    """set!(f, val) / set!(f, A) / set!(f, grid, fun; discrete, parameters) (field.jl:87-142)."""
    dst = interior(f)
    if callable(value):
        g = grid if grid is not None else f.grid
        out = evaluate(g, f.loc, f.dims, value, discrete, parameters, f.dtype)
        dst.copy_(torch.from_numpy(out))
    elif isinstance(value, (int, float, np.floating, np.integer)):
        dst.fill_(float(value))
    else:
        src = value if isinstance(value, torch.Tensor) else torch.from_numpy(np.asarray(value, dtype=f.dtype))
        dst.copy_(src.to(dst.dtype))


def vector_location(dim: int, ndim: int):
    """vector_location(Val(dim), Val(N)) (field.jl:148): Vertex along `dim`, Center elsewhere."""
    return tuple(Vertex() if i == dim else Center() for i in range(ndim))


_VEC = {1: namedtuple("VectorField1", "x"), 2: namedtuple("VectorField2", "x y"), 3: namedtuple("VectorField3", "x y z")}
_TEN = {2: namedtuple("TensorField2", "xx yy xy"), 3: namedtuple("TensorField3", "xx yy zz xy xz yz")}


def VectorField(arch, grid: UniformGrid, dtype=None, halo=1, pitch_align: int = 0):
    """VectorField(backend, grid) (field.jl:161-169): component d at Vertex along d."""
    nd = grid.ndim
    return _VEC[nd](*[Field(arch, grid, vector_location(d, nd), dtype, halo, pitch_align) for d in range(nd)])


def TensorField(arch, grid: UniformGrid, dtype=None, halo=1, pitch_align: int = 0):
    """TensorField(backend, grid) (field.jl:182-206): diagonal at Center, shear on edges."""
    nd = grid.ndim
    C, V = Center(), Vertex()
    if nd == 2:
        locs = [(C, C), (C, C), (V, V)]
    elif nd == 3:
        locs = [(C, C, C), (C, C, C), (C, C, C), (V, V, C), (V, C, V), (C, V, V)]
    else:
        raise ValueError("TensorField needs a 2D or 3D grid")
    return _TEN[nd](*[Field(arch, grid, l, dtype, halo, pitch_align) for l in locs])
