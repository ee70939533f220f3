"""pihm_gpu_nv_wrms_norm_noalloc, the WRMS norm for callers that cannot
allocate device memory (graph capture, frameworks that own every allocation,
per-call integrator callbacks), against the regular entry point
pihm_gpu_nv_wrms_norm.

The file name sorts last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13  # the reduction tolerance of tests/test_nvector_gpu.py


def _lib():
    from pihm_gpu import nvector
    lib = nvector.load()
    f = lib.pihm_gpu_nv_wrms_norm_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return lib, nvector


def test_noalloc_matches_regular_entry_point_twice():
    import torch
    lib, nvector = _lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(2024)
    # two calls in a row on the shared static workspace, different lengths
    for n in (3_060_000, 12_345):
        x = torch.from_numpy(rng.normal(size=n)).to(dev)
        w = torch.from_numpy(rng.uniform(1e3, 1e5, n)).to(dev)
        rc = lib.pihm_gpu_nv_wrms_norm_noalloc(x.data_ptr(), w.data_ptr(), n, stream.cuda_stream,
                                               out.data_ptr())
        assert rc == 0
        stream.synchronize()
        got = float(out.item())
        want = nvector.wrms_norm(x.data_ptr(), w.data_ptr(), n, stream.cuda_stream)
        assert abs(got - want) <= RTOL * abs(want), (n, got, want)


def test_noalloc_rejects_too_long():
    import torch
    lib, _ = _lib()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # the length check happens on the host before anything is launched
    rc = lib.pihm_gpu_nv_wrms_norm_noalloc(x.data_ptr(), x.data_ptr(), 33554432 + 1, None,
                                           out.data_ptr())
    assert rc == -7
