"""Builds and loads the C oracle (``liboracle.so``) with ctypes.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liboracle.so")
_SRCS = [os.path.join(_HERE, "sv_oracle.c"), os.path.join(_HERE, "sched_oracle.c")]
_lock = threading.Lock()
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i64p = ctypes.POINTER(ctypes.c_int64)
_ip = ctypes.POINTER(ctypes.c_int)
_uip = ctypes.POINTER(ctypes.c_uint)


def build_oracle_lib(force=False):
    """Compile the C oracle with gcc (+OpenMP) into oracle/_build/liboracle.so."""
    os.makedirs(_BUILD, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in _SRCS)
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= newest:
        return _SO
    tmp = _SO + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=gnu11", "-o", tmp] + _SRCS + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _SO)
    return _SO


def load_oracle_lib():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        lib = ctypes.CDLL(build_oracle_lib())
        lib.orc_apply.argtypes = [_dp, ctypes.c_uint64, ctypes.c_int, _uip, _dp, ctypes.c_uint64, ctypes.c_int]
        lib.orc_fill.argtypes = [_dp, ctypes.c_uint64, ctypes.c_double, ctypes.c_double]
        lib.orc_probability.argtypes = [_dp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        lib.orc_probability.restype = ctypes.c_double
        lib.orc_normalize.argtypes = [_dp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double]
        lib.orc_block_cdf.argtypes = [_dp, ctypes.c_uint64, ctypes.c_uint64, _dp]
        lib.orc_sample_index.argtypes = [_dp, ctypes.c_uint64, ctypes.c_double, _dp]
        lib.orc_sample_index.restype = ctypes.c_int64
        lib.orc_sample_many.argtypes = [_dp, ctypes.c_uint64, ctypes.c_int64, _dp, _i64p, _dp]
        lib.orc_bit_probs.argtypes = [_dp, ctypes.c_uint64, ctypes.c_uint, _dp]
        lib.orc_drop_bit.argtypes = [_dp, ctypes.c_uint64, ctypes.c_uint, ctypes.c_int]
        lib.orc_entropy.argtypes = [_dp, ctypes.c_uint64]
        lib.orc_entropy.restype = ctypes.c_double
        for f in (lib.orc_expectation, lib.orc_apply_pauli_sum):
            f.argtypes = [_dp, ctypes.c_uint64, ctypes.c_int, _u64p, _u64p, _u64p, _dp]
        lib.orc_expectation.restype = ctypes.c_double
        lib.orc_mt_size.restype = ctypes.c_size_t
        lib.orc_mt_seed.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        lib.orc_mt_next.argtypes = [ctypes.c_void_p]
        lib.orc_mt_next.restype = ctypes.c_uint32
        lib.orc_mt_uniform.argtypes = [ctypes.c_void_p]
        lib.orc_mt_uniform.restype = ctypes.c_double
        lib.orc_greedy_schedule.argtypes = [ctypes.c_int, _i64p, _ip, _i64p, _ip, ctypes.c_int, _i64p,
                                            ctypes.c_int, _ip, _ip]
        lib.orc_greedy_schedule.restype = ctypes.c_int
        _lib = lib
        return lib


def dptr(a):
    return a.ctypes.data_as(_dp)


class MT19937:
    """std::mt19937(seed) + std::uniform_real_distribution<double>(0, 1)."""

    def __init__(self, seed):
        self._lib = load_oracle_lib()
        self._state = ctypes.create_string_buffer(self._lib.orc_mt_size())
        self._lib.orc_mt_seed(self._state, ctypes.c_uint64(seed & 0xFFFFFFFFFFFFFFFF))

    def next_u32(self):
        return self._lib.orc_mt_next(self._state)

    def uniform(self):
        return self._lib.orc_mt_uniform(self._state)


def greedy_schedule(gates, ctrls, locals_, K):
    """Greedy clustering of a gate list (restates GreedyScheduler +
    ClusterScheduler). gates/ctrls: lists of target / control id lists.
    Returns a list of clusters, each a list of gate indices in emission order."""
    lib = load_oracle_lib()
    n = len(gates)
    toff = np.zeros(n + 1, dtype=np.int32)
    coff = np.zeros(n + 1, dtype=np.int32)
    for i in range(n):
        toff[i + 1] = toff[i] + len(gates[i])
        coff[i + 1] = coff[i] + len(ctrls[i])
    tgt = np.array([q for g in gates for q in g] or [0], dtype=np.int64)
    ctl = np.array([q for c in ctrls for q in c] or [0], dtype=np.int64)
    loc = np.array(list(locals_) or [0], dtype=np.int64)
    order = np.zeros(max(n, 1), dtype=np.int32)
    ends = np.zeros(max(n, 1), dtype=np.int32)
    nc = lib.orc_greedy_schedule(n, tgt.ctypes.data_as(_i64p), toff.ctypes.data_as(_ip), ctl.ctypes.data_as(_i64p),
                                 coff.ctypes.data_as(_ip), len(locals_), loc.ctypes.data_as(_i64p), K,
                                 order.ctypes.data_as(_ip), ends.ctypes.data_as(_ip))
    if nc < 0:
        raise RuntimeError("CalcPos(): scheduling with 64 or more qubits is not yet supported")
    out, start = [], 0
    for c in range(nc):
        out.append([int(x) for x in order[start:ends[c]]])
        start = ends[c]
    return out
