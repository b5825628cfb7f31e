"""hqs_probability_noalloc: the allocation-free probability entry point.

It exists for callers that cannot call cudaMalloc (code running under
another framework's device memory pool, or inside recorded launch
sequences); it keeps its scratch in a fixed __device__ array in libhqs.so.
This test calls it through the C ABI on the same device, call after call,
in every arithmetic code, on the legacy stream and on a torch stream, with
queries that spread over many partial sums followed by ones that fill a
single slot, and checks each result against a numpy sum of |a|^2 and against
the allocating entry point hqs_probability. The file sorts last so that a
failure here never hides another test's result."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (arith, qubits, tolerance): complex128 codes hold ~48 significant bits in
# their reductions (double-float partial sums); complex64 states are summed
# in double-float from FP32 amplitudes.
CASES = (("f64", 22, 1e-13), ("df", 22, 1e-13), ("tc", 21, 1e-13),
         ("f32", 22, 1e-6), ("tf32", 20, 1e-6), ("tc64", 21, 1e-6))


def _numpy_probability(v, mask, val):
    idx = np.arange(v.size, dtype=np.uint64)
    sel = (idx & np.uint64(mask)) == np.uint64(val)
    a = v[sel].astype(np.complex128)
    return float(np.sum(a.real * a.real + a.imag * a.imag))


def test_noalloc_probability_matches_numpy_and_allocating_entry_point(hqs, cuda):
    from hiqsimulator_gb300 import capi
    lib = capi.load()
    ws = capi.Workspace()
    rng = np.random.Generator(np.random.PCG64(77))
    side = cuda.cuda.Stream()
    for arith, n, tol in CASES:
        v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        v /= np.linalg.norm(v)
        host = v.astype(np.complex64 if capi.ARITH[arith] in (3, 5, 6) else np.complex128)
        state = cuda.from_numpy(host).cuda()
        out = cuda.zeros(1, dtype=cuda.float64, device="cuda")
        cuda.cuda.synchronize()
        # the whole state (every CTA writes a partial), then a query with a
        # handful of matching amplitudes (one partial: a later, smaller call
        # reads only the slot it wrote), then random masks; alternately on
        # the legacy stream and on a torch stream
        queries = [(0, 0), ((1 << n) - 1 - 5, 3 & ((1 << n) - 1 - 5))]
        for _ in range(2):
            mask = int(rng.integers(0, 1 << n))
            queries.append((mask, int(rng.integers(0, 1 << n)) & mask))
        for call, (mask, val) in enumerate(queries):
            out.fill_(-1.0)
            cuda.cuda.synchronize()
            stream = side if call % 2 else None
            handle = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
            rc = lib.hqs_probability_noalloc(ctypes.c_void_p(state.data_ptr()), n, capi.ARITH[arith], mask, val,
                                             ctypes.c_void_p(out.data_ptr()), handle)
            assert rc == capi.HQS_OK, lib.hqs_last_error()
            cuda.cuda.synchronize()
            got = float(out.cpu()[0])
            want_np = _numpy_probability(host, mask, val)
            want_ws = ws.probability(ctypes.c_void_p(state.data_ptr()), n, arith, mask, val)
            assert abs(got - want_np) < tol, (arith, call, got, want_np)
            assert abs(got - want_ws) < tol, (arith, call, got, want_ws)
        del state
    # a state beyond the entry point's limit is refused before any launch
    big = lib.hqs_probability_noalloc(ctypes.c_void_p(16), 41, capi.ARITH["df"], 0, 0, ctypes.c_void_p(16), None)
    assert big == capi.HQS_ERR_INVALID
    assert b"2^40" in lib.hqs_last_error()
    ws.close()
