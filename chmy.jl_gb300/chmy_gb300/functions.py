"""FunctionField on the GB300 path (src/Fields/function_field.jl): a field whose values are a
function of the point's coordinates, computed where they are used.

Chmy compiles the user's Julia function into the kernel that reads the field. A library of
hand-written kernels cannot compile host functions, so the functions a GB300 kernel evaluates
on the device are a fixed set of forms (`cg_function`): `constant`, `ball` (the examples'
`init_incl`, examples/stokes_2d_inc_ve_T.jl:106) and `affine`. A FunctionField over one of these
is passed to the kernels as a descriptor and never materialised; any other function (or the
discrete form) is evaluated on the host by `set_` like Chmy's `set!(f, grid, func)`.
"""

from __future__ import annotations

import numpy as np

from . import _abi
from .grids import UniformGrid, expand_loc


class DeviceFunction:
    """A function form the library's kernels evaluate at a point: func(x..., parameters...)."""

    def __init__(self, kind: int, name: str):
        self.kind = kind
        self.__name__ = name

    def pack(self, nd: int, parameters) -> list[float]:
        """The form's parameters as cg_function.p."""
        vals = list(parameters.values()) if isinstance(parameters, dict) else list(parameters or ())
        if self.kind == _abi.CG_FN_CONST:
            if len(vals) != 1:
                raise ValueError("constant takes one parameter (the value)")
            return [float(vals[0])]
        if self.kind == _abi.CG_FN_BALL:
            if len(vals) != nd + 3:
                raise ValueError(f"ball in {nd}D takes {nd + 3} parameters: centre ({nd}), r, in, out")
            centre = [float(v) for v in vals[:nd]] + [0.0] * (3 - nd)
            return centre + [float(v) for v in vals[nd:]]
        if self.kind == _abi.CG_FN_AFFINE:
            if len(vals) != nd + 1:
                raise ValueError(f"affine in {nd}D takes {nd + 1} parameters: a0, then one slope per dimension")
            return [float(v) for v in vals]
        raise ValueError(f"unknown function kind {self.kind}")

    def __call__(self, *args):
        """Host evaluation on coordinate arrays, with the kernels' operation order."""
        kind = self.kind
        if kind == _abi.CG_FN_CONST:
            x, c = args[:-1], args[-1]
            return np.full(np.shape(x[0]), c) if x else c
        if kind == _abi.CG_FN_BALL:
            n = len(args) - 3
            nd = n // 2
            xs, centre, (r, inside, outside) = args[:nd], args[nd:n], args[n:]
            r2 = (xs[0] - centre[0]) * (xs[0] - centre[0])
            for x, c in zip(xs[1:], centre[1:]):
                r2 = r2 + (x - c) * (x - c)
            return np.where(r2 < r * r, inside, outside)
        if kind == _abi.CG_FN_AFFINE:
            nd = (len(args) - 1) // 2
            xs, a = args[:nd], args[nd:]
            v = a[0]
            for x, s in zip(xs, a[1:]):
                v = v + s * x
            return v
        raise ValueError(f"unknown function kind {kind}")


constant = DeviceFunction(_abi.CG_FN_CONST, "constant")
# init_incl(x, y[, z], x0, y0[, z0], r, in, out) = ifelse(sum (x_d - x0_d)^2 < r^2, in, out)
ball = DeviceFunction(_abi.CG_FN_BALL, "ball")
init_incl = ball
affine = DeviceFunction(_abi.CG_FN_AFFINE, "affine")


class FunctionField:
    """FunctionField(func, grid, loc; discrete=false, parameters=nothing)
    (src/Fields/function_field.jl:25-31). With a DeviceFunction, `desc()` is the descriptor the
    kernels evaluate; `values()` evaluates it on the host over the padded points."""

    def __init__(self, func, grid: UniformGrid, loc, discrete: bool = False, parameters=None):
        self.func = func
        self.grid = grid
        self.loc = expand_loc(grid.ndim, loc)
        self.discrete = bool(discrete)
        self.parameters = parameters

    @property
    def on_device(self) -> bool:
        return isinstance(self.func, DeviceFunction) and not self.discrete

    def desc(self) -> _abi.cg_function:
        if not self.on_device:
            raise TypeError(f"{self.func!r} is not a function form the GB300 kernels evaluate")
        fn = _abi.cg_function()
        fn.kind = self.func.kind
        for q, v in enumerate(self.func.pack(self.grid.ndim, self.parameters)):
            fn.p[q] = v
        return fn

    def size(self):
        return self.grid.size(self.loc)

    def values(self, halo: int = 1) -> np.ndarray:
        """The function at every padded point (logical 1-2H .. n+2H), stored [z, y, x]."""
        from .configs import padded_mesh

        xs = padded_mesh(self.grid, self.loc, halo)
        vals = list(self.parameters.values()) if isinstance(self.parameters, dict) else list(self.parameters or ())
        return np.asarray(self.func(*xs, *vals), dtype=self.grid.dtype) * np.ones_like(xs[0])
