"""The allocation-free max-norm entry point, cg_maxabs_noalloc, against cg_maxabs.

cg_maxabs_noalloc serves callers that cannot allocate device memory (a host runtime that
owns all device memory, work issued during stream capture, fixed memory budgets): it takes
no context and keeps its reduction slots in a fixed device array. This file is collected
last so that a failure here cannot hide the results of the other tests.
"""

import ctypes

import numpy as np
import pytest

from _oracle import NpField, desc_array
from chmy_gb300 import _abi
from chmy_gb300.grids import Center, UniformGrid, Vertex
from gpu_helpers import random_field, to_gpu

pytestmark = pytest.mark.gpu


def _fields(arch, seed):
    rng = np.random.default_rng(seed)
    g2 = UniformGrid(origin=(0.0, 0.0), extent=(1.0, 1.0), dims=(130, 97))
    g3 = UniformGrid(origin=(0.0,) * 3, extent=(1.0,) * 3, dims=(21, 18, 15), dtype=np.float32)
    hs = [
        random_field(g2, (Vertex(), Center()), np.float64, rng, 2.0),
        random_field(g2, Center(), np.float64, rng, 0.5),
        random_field(g3, (Center(), Vertex(), Vertex()), np.float32, rng, 3.0),
    ]
    return [to_gpu(arch, f) for f in hs]


def test_noalloc_matches_context_reduction_twice(arch):
    lib = arch.lib
    dev = arch.device_id - 1
    for call, seed in enumerate((11, 12)):  # two calls in a row: stale slots must not leak
        gs = _fields(arch, seed)
        n = len(gs)
        ref = (ctypes.c_double * n)()
        bad_ref = ctypes.c_int32(-1)
        arch.call("cg_maxabs", n, desc_array(gs), ref, ctypes.byref(bad_ref))
        out = (ctypes.c_double * n)()
        bad = ctypes.c_int32(-1)
        rc = lib.cg_maxabs_noalloc(dev, None, n, desc_array(gs), out, ctypes.byref(bad))
        assert rc == _abi.CG_OK, lib.cg_last_error(None)
        # both are exact max-norms of the same values: equal bit for bit
        assert [out[i] for i in range(n)] == [ref[i] for i in range(n)], (call, list(out), list(ref))
        assert bad.value == bad_ref.value == 0
        host_max = [float(np.max(np.abs(g.to_numpy()[tuple(slice(2, -2) for _ in range(g.ndim))]))) for g in gs]
        assert [out[i] for i in range(n)] == host_max


def test_noalloc_rejects_too_many_fields(arch):
    gs = _fields(arch, 3)
    many = [gs[0]] * (_abi_max() + 1)
    out = (ctypes.c_double * len(many))()
    rc = arch.lib.cg_maxabs_noalloc(arch.device_id - 1, None, len(many), desc_array(many), out, None)
    assert rc == _abi.CG_ERR_ARG
    assert b"nfields" in arch.lib.cg_last_error(None)


def _abi_max():
    import re

    text = _abi.HEADER.read_text()
    return int(re.search(r"#define CG_MAXABS_NOALLOC_MAX_FIELDS (\d+)", text).group(1))
