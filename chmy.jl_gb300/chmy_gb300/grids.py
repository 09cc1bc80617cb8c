"""Locations and UniformGrid (Chmy.jl src/Grids/Grids.jl, uniform_axis.jl, structured_grid.jl)."""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi


class Location:
    code: int = -1

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self))

    def __repr__(self):
        return f"{type(self).__name__}()"


class Center(Location):
    """Cell centre along a dimension (src/Grids/Grids.jl:33)."""

    code = _abi.CG_CENTER


class Vertex(Location):
    """Cell vertex along a dimension (src/Grids/Grids.jl:40)."""

    code = _abi.CG_VERTEX


def flip(loc: Location) -> Location:
    """flip(Center()) == Vertex() and vice versa (src/Grids/Grids.jl:42-43)."""
    return Vertex() if isinstance(loc, Center) else Center()


def expand_loc(ndim: int, loc) -> tuple[Location, ...]:
    """expand_loc(Val(N), loc) (src/Grids/Grids.jl:59-60)."""
    if isinstance(loc, Location):
        return tuple(loc for _ in range(ndim))
    loc = tuple(loc)
    if len(loc) != ndim:
        raise ValueError(f"expected {ndim} locations, got {len(loc)}")
    return loc


class Bounded:
    """Bounded connectivity: the only one Chmy gives a FieldBatch (batch.jl:187-189)."""


@dataclass(frozen=True)
class Dim:
    d: int  # 1-based like Chmy's Dim{D}


@dataclass(frozen=True)
class Side:
    s: int  # 1 = left, 2 = right


_libm = ctypes.CDLL(None)
_libm.fma.restype = ctypes.c_double
_libm.fma.argtypes = [ctypes.c_double] * 3
_libm.fmaf.restype = ctypes.c_float
_libm.fmaf.argtypes = [ctypes.c_float] * 3


def muladd(x, y, z, dtype):
    """Julia muladd (fused) in the grid's element type."""
    if dtype == np.float32:
        return np.float32(_libm.fmaf(float(np.float32(x)), float(np.float32(y)), float(np.float32(z))))
    return np.float64(_libm.fma(float(x), float(y), float(z)))


class UniformAxis:
    """UniformAxis (src/Grids/uniform_axis.jl:1-31): spacing = extent/len, inv = inv(spacing)."""

    def __init__(self, origin, extent, length: int, dtype):
        self.dtype = dtype
        self.origin = dtype(origin)
        self.extent = dtype(extent)
        self.length = int(length)
        self.spacing = dtype(self.extent / dtype(length))
        self.inv_spacing = dtype(dtype(1) / self.spacing)

    def nvertices(self) -> int:
        return self.length + 1

    def ncenters(self) -> int:
        return self.length

    def size(self, loc: Location) -> int:
        return self.nvertices() if isinstance(loc, Vertex) else self.ncenters()

    def vertex(self, i: int):
        return muladd(i - 1, self.spacing, self.origin, self.dtype)

    def center(self, i: int):
        return muladd(i - 1, self.spacing, muladd(0.5, self.spacing, self.origin, self.dtype), self.dtype)

    def coord(self, loc: Location, i: int):
        return self.vertex(i) if isinstance(loc, Vertex) else self.center(i)

    def origin_at(self, loc: Location):
        return self.origin if isinstance(loc, Vertex) else muladd(0.5, self.spacing, self.origin, self.dtype)

    def extent_at(self, loc: Location):
        return self.extent if isinstance(loc, Vertex) else self.dtype(self.extent - self.spacing)

    def coords(self, loc: Location) -> np.ndarray:
        return np.array([self.coord(loc, i) for i in range(1, self.size(loc) + 1)], dtype=self.dtype)


class UniformGrid:
    """UniformGrid(arch; origin, extent, dims) (src/Grids/structured_grid.jl:27-39).

    `dtype` is the grid element type (Chmy promotes origin/extent; float64 by default).
    Connectivity is Bounded on every side, as in Chmy's default."""

    def __init__(self, arch=None, *, origin, extent, dims, dtype=np.float64):
        dims = tuple(int(n) for n in dims)
        if not (len(dims) == len(origin) == len(extent)) or not 1 <= len(dims) <= 3:
            raise ValueError("origin, extent and dims must have the same length (1..3)")
        self.arch = arch
        self.dtype = np.dtype(dtype).type
        self.axes = tuple(UniformAxis(o, e, n, self.dtype) for o, e, n in zip(origin, extent, dims))
        self.dims = dims

    @property
    def ndim(self) -> int:
        return len(self.dims)

    def size(self, loc) -> tuple[int, ...]:
        locs = expand_loc(self.ndim, loc)
        return tuple(ax.size(l) for ax, l in zip(self.axes, locs))

    def spacing(self) -> tuple:
        return tuple(ax.spacing for ax in self.axes)

    def inv_spacing(self) -> tuple:
        return tuple(ax.inv_spacing for ax in self.axes)

    def coord(self, loc, dim: int, i: int):
        locs = expand_loc(self.ndim, loc)
        return self.axes[dim - 1].coord(locs[dim - 1], i)

    def coords(self, loc, dim: int) -> np.ndarray:
        locs = expand_loc(self.ndim, loc)
        return self.axes[dim - 1].coords(locs[dim - 1])

    def centers(self) -> tuple[np.ndarray, ...]:
        return tuple(ax.coords(Center()) for ax in self.axes)

    def vertices(self) -> tuple[np.ndarray, ...]:
        return tuple(ax.coords(Vertex()) for ax in self.axes)

    def origin(self, loc, dim: int):
        locs = expand_loc(self.ndim, loc)
        return self.axes[dim - 1].origin_at(locs[dim - 1])

    def extent(self, loc, dim: int):
        locs = expand_loc(self.ndim, loc)
        return self.axes[dim - 1].extent_at(locs[dim - 1])

    def bounds(self, loc, dim: int):
        o = self.origin(loc, dim)
        return (o, self.dtype(o + self.extent(loc, dim)))

    def connectivity(self, dim: int, side: int):
        return Bounded()

    def desc(self) -> _abi.cg_grid:
        return _abi.make_grid(
            self.dims,
            [ax.origin for ax in self.axes],
            [ax.extent for ax in self.axes],
            [ax.spacing for ax in self.axes],
            [ax.inv_spacing for ax in self.axes],
        )

    def __repr__(self):
        return f"UniformGrid(dims={self.dims}, dtype={self.dtype.__name__})"
