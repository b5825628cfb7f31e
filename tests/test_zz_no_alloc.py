"""hqs_probability_noalloc: the allocation-free probability entry point.

It exists for callers that cannot call cudaMalloc (code running under
another framework's device memory pool, or inside recorded launch
sequences); it keeps its scratch in a fixed __device__ array in libhqs.so.
This test calls it through the C ABI twice in a row on the same device and
checks each result against the allocating entry point hqs_probability. The
file sorts last so that a failure here never hides another test's result."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_probability_matches_allocating_entry_point(hqs, cuda):
    from hiqsimulator_gb300 import capi
    lib = capi.load()
    ws = capi.Workspace()
    rng = np.random.Generator(np.random.PCG64(77))
    for arith, n, tol in (("df", 21, 1e-13), ("f64", 9, 1e-13), ("f32", 18, 1e-6)):
        v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        v /= np.linalg.norm(v)
        host = v.astype(np.complex64 if arith == "f32" else np.complex128)
        state = cuda.from_numpy(host).cuda()
        out = cuda.zeros(1, dtype=cuda.float64, device="cuda")
        cuda.cuda.synchronize()
        for call in range(2):  # two calls in a row share the static scratch
            mask = int(rng.integers(0, 1 << n))
            val = int(rng.integers(0, 1 << n)) & mask
            out.fill_(-1.0)
            cuda.cuda.synchronize()
            rc = lib.hqs_probability_noalloc(ctypes.c_void_p(state.data_ptr()), n, capi.ARITH[arith], mask, val,
                                             ctypes.c_void_p(out.data_ptr()), None)
            assert rc == capi.HQS_OK, lib.hqs_last_error()
            cuda.cuda.synchronize()
            got = float(out.cpu()[0])
            want = ws.probability(ctypes.c_void_p(state.data_ptr()), n, arith, mask, val)
            assert abs(got - want) < tol, (arith, call, got, want)
    # a request beyond the static scratch is refused before any launch
    big = lib.hqs_probability_noalloc(ctypes.c_void_p(16), 33, capi.ARITH["df"], 0, 0, ctypes.c_void_p(16), None)
    assert big == capi.HQS_ERR_INVALID
    assert b"2^32" in lib.hqs_last_error()
    ws.close()
