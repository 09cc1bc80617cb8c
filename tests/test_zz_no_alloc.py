"""The allocation-free max-norm entry point, cg_maxabs_noalloc, against cg_maxabs.

cg_maxabs_noalloc serves callers that cannot allocate device memory: a host runtime whose own
pool owns all device memory and does not let a library call cudaMalloc, or a deployment with a
fixed device-memory budget. It takes no context and keeps its reduction slots in a fixed device
array shared by every call. This file is collected last so that a failure here cannot hide the
results of the other tests.
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


def test_noalloc_nonfinite_on_a_side_stream(arch):
    """NaN in an FP32 field and Inf in an FP64 field, reduced on a stream other than the
    context's: the flag is raised and the maxima carry the NaN and the Inf, as cg_maxabs
    reports them."""
    import torch

    gs = _fields(arch, 21)
    gs[2].data[3, 4, 5] = float("nan")  # an interior point of the 21x18x15 FP32 field
    gs[1].data[7, 9] = float("-inf")  # an interior point of the 2D FP64 field
    n = len(gs)
    ref = (ctypes.c_double * n)()
    bad_ref = ctypes.c_int32(-1)
    arch.call("cg_maxabs", n, desc_array(gs), ref, ctypes.byref(bad_ref))
    side = torch.cuda.Stream(device=arch.device)
    side.wait_stream(torch.cuda.current_stream(arch.device))
    out = (ctypes.c_double * n)()
    bad = ctypes.c_int32(-1)
    rc = arch.lib.cg_maxabs_noalloc(arch.device_id - 1, ctypes.c_void_p(side.cuda_stream), n, desc_array(gs), out,
                                    ctypes.byref(bad))
    assert rc == _abi.CG_OK, arch.lib.cg_last_error(None)
    assert bad.value == bad_ref.value == 1
    assert np.isnan(out[2]) and np.isnan(ref[2])
    assert out[1] == ref[1] == float("inf")
    assert out[0] == ref[0]
    # the next call on clean data starts from cleared slots
    gs = _fields(arch, 22)
    rc = arch.lib.cg_maxabs_noalloc(arch.device_id - 1, None, n, desc_array(gs), out, ctypes.byref(bad))
    assert rc == _abi.CG_OK and bad.value == 0
    arch.call("cg_maxabs", n, desc_array(gs), ref, ctypes.byref(bad_ref))
    assert [out[i] for i in range(n)] == [ref[i] for i in range(n)]


def test_noalloc_rejects_bad_arguments(arch):
    gs = _fields(arch, 4)
    out = (ctypes.c_double * len(gs))()
    lib = arch.lib
    assert lib.cg_maxabs_noalloc(-1, None, len(gs), desc_array(gs), out, None) == _abi.CG_ERR_ARG
    assert b"device" in lib.cg_last_error(None)
    assert lib.cg_maxabs_noalloc(arch.device_id - 1, None, len(gs), None, out, None) == _abi.CG_ERR_ARG
    assert lib.cg_maxabs_noalloc(arch.device_id - 1, None, 0, desc_array(gs), out, None) == _abi.CG_ERR_ARG


def _abi_max():
    import re

    text = _abi.HEADER.read_text()
    return int(re.search(r"#define CG_MAXABS_NOALLOC_MAX_FIELDS (\d+)", text).group(1))
