"""ctypes binding of libhqs.so (include/hqs.h).

This is the binding a C-ABI consumer would write; the parity tests and the
benchmark use it to reach the kernel-level entry points directly. Raises on
any non-zero status with the library's message.
"""
import ctypes
import os
import re

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libhqs.so")
HEADER = os.path.join(os.path.dirname(_PKG), "include", "hqs.h")

HQS_OK, HQS_ERR_RUNTIME, HQS_ERR_INVALID, HQS_ERR_CUDA, HQS_ERR_MEMORY = range(5)
HQS_C128, HQS_C64 = 0, 1
ARITH = {"auto": 0, "f64": 1, "df": 2, "f32": 3, "tc": 4, "tf32": 5, "tc64": 6}

_i = ctypes.c_int
_u64 = ctypes.c_uint64
_i64 = ctypes.c_int64
_sz = ctypes.c_size_t
_d = ctypes.c_double
_vp = ctypes.c_void_p
_P = ctypes.POINTER


class HQSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


_lib = None


def header_functions():
    """Names of every function declared in include/hqs.h."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hqs_\w+)\s*\(", src)))


def load():
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(LIB_PATH)
    lib.hqs_last_error.restype = ctypes.c_char_p
    lib.hqs_version.restype = ctypes.c_char_p
    lib.hqs_sim_last_error.restype = ctypes.c_char_p
    lib.hqs_sim_last_error.argtypes = [_vp]
    lib.hqs_sim_create.argtypes = [_u64, _i64, _i64, _i, _i, _P(_vp)]
    lib.hqs_sim_destroy.argtypes = [_vp]
    lib.hqs_sim_destroy.restype = None
    lib.hqs_sim_allocate_qureg.argtypes = [_vp, _P(_i64), _sz, _d, _d]
    lib.hqs_sim_apply_controlled_gate.argtypes = [_vp, _P(_d), _sz, _P(_i64), _sz, _P(_i64), _sz]
    lib.hqs_sim_run.argtypes = [_vp]
    lib.hqs_sim_cheat_local.argtypes = [_vp, _P(_d), _sz]
    lib.hqs_sim_num_qubits.argtypes = [_vp, _P(_sz)]
    lib.hqs_sim_get_qubits_ids.argtypes = [_vp, _P(_i64), _sz, _P(_sz)]
    lib.hqs_sim_synchronize.argtypes = [_vp]
    lib.hqs_sim_state_view.argtypes = [_vp, _P(_vp), _P(_u64), _P(_i)]
    lib.hqs_sim_sample.argtypes = [_vp, _u64, _P(_u64)]
    lib.hqs_sim_get_probability.argtypes = [_vp, _P(ctypes.c_uint8), _sz, _P(_i64), _sz, _P(_d)]
    lib.hqs_sim_measure_qubits.argtypes = [_vp, _P(_i64), _sz, _P(ctypes.c_uint8)]
    lib.hqs_sim_timer_start.argtypes = [_vp]
    lib.hqs_sim_timer_stop.argtypes = [_vp, _P(ctypes.c_float)]
    lib.hqs_sim_stats.argtypes = [_vp, _P(_u64)]
    lib.hqs_sim_set_pass_limits.argtypes = [_vp, _i, _i, _i]
    lib.hqs_sim_get_expectation_value.argtypes = [_vp, _sz, _P(_sz), _P(_i64), ctypes.c_char_p, _P(_d), _P(_i64),
                                                  _sz, _P(_d)]
    lib.hqs_greedy_schedule.argtypes = [_i, _P(_i64), _P(_i), _P(_i64), _P(_i), _i, _P(_i64), _i, _P(_i), _P(_i),
                                        _P(_i)]
    lib.hqs_ws_create.argtypes = [_P(_vp)]
    lib.hqs_ws_destroy.argtypes = [_vp]
    lib.hqs_ws_destroy.restype = None
    lib.hqs_apply_gates.argtypes = [_vp, _vp, _i, _i, _i, _P(_i), _P(_i), _P(_u64), _P(_i), _P(_d), _i, _i,
                                    _P(_u64), _P(_u64)]
    lib.hqs_probability.argtypes = [_vp, _vp, _i, _i, _u64, _u64, _P(_d)]
    lib.hqs_block_sums.argtypes = [_vp, _vp, _i, _i, _u64, _P(_d)]
    lib.hqs_collapse.argtypes = [_vp, _vp, _i, _i, _u64, _u64, _d]
    lib.hqs_permute_bits.argtypes = [_vp, _vp, _i, _i, _i, _P(ctypes.c_uint8), _P(ctypes.c_uint8)]
    lib.hqs_drop_bit.argtypes = [_vp, _vp, _i, _i, _i, _i]
    lib.hqs_probability_noalloc.argtypes = [_vp, _i, _i, _u64, _u64, _vp, _vp]
    lib.hqs_ws_synchronize.argtypes = [_vp]
    lib.hqs_ws_timer_start.argtypes = [_vp]
    lib.hqs_ws_timer_stop.argtypes = [_vp, _P(ctypes.c_float)]
    lib.hqs_plan_launches.argtypes = [_i, _i, _i, _P(_i), _P(_i), _P(_u64), _P(_i), _i, _i, _P(LaunchInfo), _sz,
                                      _P(_sz)]
    lib.hqs_plan_passes.argtypes = [_i, _i, _i, _P(_i), _P(_i), _P(_u64), _P(_i), _i, _i, _P(PassInfo), _sz,
                                    _P(_sz)]
    _lib = lib
    return lib


class PassInfo(ctypes.Structure):
    _fields_ = [("first_op", ctypes.c_uint32), ("nops", ctypes.c_uint32), ("q", ctypes.c_uint32),
                ("w", ctypes.c_uint32), ("prefetch", ctypes.c_uint32), ("tc_ops", ctypes.c_uint32),
                ("tile_mask", ctypes.c_uint64), ("fixed_mask", ctypes.c_uint64), ("smem_bytes", ctypes.c_uint64),
                ("pool_bytes", ctypes.c_uint64), ("sweep_bytes", ctypes.c_uint64)]


class LaunchInfo(ctypes.Structure):
    _fields_ = [("first_op", ctypes.c_uint32), ("nops", ctypes.c_uint32), ("umma", ctypes.c_uint32),
                ("tc_op", ctypes.c_uint32), ("tile_mask", ctypes.c_uint64), ("target_mask", ctypes.c_uint64),
                ("fixed_mask", ctypes.c_uint64), ("rank", ctypes.c_uint32), ("nextra", ctypes.c_uint32),
                ("box_bytes", ctypes.c_uint32), ("dim_kind", ctypes.c_int32 * 5), ("dim_pos", ctypes.c_int32 * 5),
                ("dim_bits", ctypes.c_int32 * 5), ("dim_box", ctypes.c_int32 * 5), ("pool_bytes", ctypes.c_uint64),
                ("sweep_bytes", ctypes.c_uint64)]


def plan_launches(n, arith, gates, max_tile_bits=0, max_ops=0):
    """The launches the engine makes for gates (k, positions, ctrl_mask,
    diag[, matrix]), computed on the host: a list of dicts (LaunchInfo
    fields, arrays as lists)."""
    lib = load()
    nops, k, pos, ctrl, diag = _gate_arrays(gates)
    cap = max(nops, 1)
    out = (LaunchInfo * cap)()
    nl = _sz()
    check_ws(lib.hqs_plan_launches(n, ARITH[arith], nops, _ptr(k, _i), _ptr(pos, _i), _ptr(ctrl, _u64),
                                   _ptr(diag, _i), max_tile_bits, max_ops, out, cap, ctypes.byref(nl)))
    res = []
    for i in range(nl.value):
        d = {}
        for f, _ in LaunchInfo._fields_:
            v = getattr(out[i], f)
            d[f] = list(v) if f.startswith("dim_") else v
        res.append(d)
    return res


def _gate_arrays(gates):
    """(k, positions, ctrl_mask, diag, ...) tuples as the C ABI's arrays."""
    nops = len(gates)
    k = np.array([g[0] for g in gates] or [0], dtype=np.int32)
    pos = np.zeros(max(nops, 1) * 5, dtype=np.int32)
    ctrl = np.array([g[2] for g in gates] or [0], dtype=np.uint64)
    diag = np.array([1 if g[3] else 0 for g in gates] or [0], dtype=np.int32)
    for i, g in enumerate(gates):
        pos[5 * i:5 * i + g[0]] = g[1]
    return nops, k, pos, ctrl, diag


def plan_passes(n, arith, gates, max_tile_bits=0, max_ops=0):
    """How the engine groups gates (k, positions, ctrl_mask, diag[, matrix])
    into tiled passes, computed on the host: a list of dicts (PassInfo fields)."""
    lib = load()
    nops, k, pos, ctrl, diag = _gate_arrays(gates)
    cap = max(nops, 1)
    out = (PassInfo * cap)()
    np_ = _sz()
    check_ws(lib.hqs_plan_passes(n, ARITH[arith], nops, _ptr(k, _i), _ptr(pos, _i), _ptr(ctrl, _u64),
                                 _ptr(diag, _i), max_tile_bits, max_ops, out, cap, ctypes.byref(np_)))
    return [{f: getattr(out[i], f) for f, _ in PassInfo._fields_} for i in range(np_.value)]


def _ptr(a, t):
    return a.ctypes.data_as(_P(t))


def check_ws(rc):
    if rc != HQS_OK:
        raise HQSError(rc, load().hqs_last_error().decode())


class Workspace:
    """Kernel-level handle (hqs_ws): a stream plus matrix/reduction buffers."""

    def __init__(self):
        self.lib = load()
        h = _vp()
        check_ws(self.lib.hqs_ws_create(ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.hqs_ws_destroy(self.h)
            self.h = None

    __del__ = close

    def apply_gates(self, state_ptr, n, arith, gates, max_tile_bits=0, max_ops=0):
        """gates: list of (k, positions, ctrl_mask, diag, matrix as complex ndarray)."""
        nops = len(gates)
        k = np.array([g[0] for g in gates] or [0], dtype=np.int32)
        pos = np.zeros(max(nops, 1) * 5, dtype=np.int32)
        ctrl = np.array([g[2] for g in gates] or [0], dtype=np.uint64)
        diag = np.array([1 if g[3] else 0 for g in gates] or [0], dtype=np.int32)
        mats = []
        for i, g in enumerate(gates):
            pos[5 * i:5 * i + g[0]] = g[1]
            m = np.asarray(g[4], dtype=np.complex128)
            mats.append(np.diag(m) if (g[3] and m.ndim == 2) else m.reshape(-1))
        flat = np.ascontiguousarray(np.concatenate(mats) if mats else np.zeros(1, np.complex128))
        by = _u64()
        ps = _u64()
        check_ws(self.lib.hqs_apply_gates(self.h, state_ptr, n, ARITH[arith], nops, _ptr(k, _i), _ptr(pos, _i),
                                          _ptr(ctrl, _u64), _ptr(diag, _i), _ptr(flat.view(np.float64), _d),
                                          max_tile_bits, max_ops, ctypes.byref(by), ctypes.byref(ps)))
        return by.value, ps.value

    def probability(self, state_ptr, n, arith, mask, val):
        out = _d()
        check_ws(self.lib.hqs_probability(self.h, state_ptr, n, ARITH[arith], mask, val, ctypes.byref(out)))
        return out.value

    def block_sums(self, state_ptr, n, arith, nblocks):
        out = np.zeros(nblocks, dtype=np.float64)
        check_ws(self.lib.hqs_block_sums(self.h, state_ptr, n, ARITH[arith], nblocks, _ptr(out, _d)))
        return out

    def collapse(self, state_ptr, n, arith, mask, val, scale):
        check_ws(self.lib.hqs_collapse(self.h, state_ptr, n, ARITH[arith], mask, val, scale))

    def permute_bits(self, state_ptr, n, arith, oldpos, newpos):
        o = np.array(oldpos or [0], dtype=np.uint8)
        p = np.array(newpos or [0], dtype=np.uint8)
        check_ws(self.lib.hqs_permute_bits(self.h, state_ptr, n, ARITH[arith], len(oldpos), _ptr(o, ctypes.c_uint8),
                                           _ptr(p, ctypes.c_uint8)))

    def drop_bit(self, state_ptr, n, arith, pos, keep):
        check_ws(self.lib.hqs_drop_bit(self.h, state_ptr, n, ARITH[arith], pos, keep))

    def synchronize(self):
        check_ws(self.lib.hqs_ws_synchronize(self.h))

    def timer_start(self):
        check_ws(self.lib.hqs_ws_timer_start(self.h))

    def timer_stop(self):
        ms = ctypes.c_float()
        check_ws(self.lib.hqs_ws_timer_stop(self.h, ctypes.byref(ms)))
        return ms.value


def fuse(gates):
    """Host FP64 fusion (hqs_fuse) of gates given as (matrix, ids, ctrls),
    inserted in order. Returns (matrix, ids, ctrls, diag) of the fused gate:
    matrix bit l <-> ids[l] (ascending), ctrls the controls every gate
    shared."""
    lib = load()
    n = len(gates)
    mats = [np.ascontiguousarray(g[0], dtype=np.complex128) for g in gates]
    dim = np.array([m.shape[0] for m in mats] or [0], dtype=np.uint64)
    ioff = np.zeros(n + 1, dtype=np.uint64)
    coff = np.zeros(n + 1, dtype=np.uint64)
    for i, g in enumerate(gates):
        ioff[i + 1] = ioff[i] + len(g[1])
        coff[i + 1] = coff[i] + len(g[2])
    m = np.concatenate([x.ravel() for x in mats]) if mats else np.zeros(1, dtype=np.complex128)
    ids = np.array([q for g in gates for q in g[1]] or [0], dtype=np.int64)
    ctl = np.array([q for g in gates for q in g[2]] or [0], dtype=np.int64)
    nq = len({q for g in gates for q in list(g[1]) + list(g[2])})  # the fused ids are among these
    cap = 1 << (2 * min(nq, 12))
    out = np.zeros(cap, dtype=np.complex128)
    oids = np.zeros(64, dtype=np.int64)
    octl = np.zeros(64, dtype=np.int64)
    nid, nct, dg = _sz(), _sz(), _i()
    check_ws(lib.hqs_fuse(n, _ptr(m.view(np.float64), _d), _ptr(dim, _sz), _ptr(ids, _i64), _ptr(ioff, _sz),
                          _ptr(ctl, _i64), _ptr(coff, _sz), _ptr(out.view(np.float64), _d), cap,
                          _ptr(oids, _i64), 64, ctypes.byref(nid), _ptr(octl, _i64), 64, ctypes.byref(nct),
                          ctypes.byref(dg)))
    d = 1 << nid.value
    return (out[:d * d].reshape(d, d).copy(), [int(x) for x in oids[:nid.value]],
            [int(x) for x in octl[:nct.value]], bool(dg.value))


def greedy_schedule(gates, ctrls, locals_, cluster_size):
    """Native greedy clustering (hqs_greedy_schedule). Returns a list of
    clusters, each a list of gate indices in emission order."""
    lib = load()
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
    nc = _i()
    check_ws(lib.hqs_greedy_schedule(n, _ptr(tgt, _i64), _ptr(toff, _i), _ptr(ctl, _i64), _ptr(coff, _i),
                                     len(locals_), _ptr(loc, _i64), cluster_size, _ptr(order, _i), _ptr(ends, _i),
                                     ctypes.byref(nc)))
    out, start = [], 0
    for c in range(nc.value):
        out.append([int(x) for x in order[start:ends[c]]])
        start = ends[c]
    return out
