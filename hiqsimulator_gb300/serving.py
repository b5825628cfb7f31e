"""Batched serving of many small circuits (hqs_server_* in include/hqs.h).

    srv = Server("c128", budget_bytes=150e9)
    rid = srv.submit(circuit)           # Circuit: n, flattened gates, result kind
    results = srv.step()                # one round: finish, admit, one pass each

`serve(circuits, arrivals, ...)` replays a Poisson arrival stream against a
server and reports circuits/s and p50/p99 latency; with max_active=1 the same
server runs one circuit per launch, the baseline the batched mode is set
against.
"""
import ctypes
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import capi

_P = ctypes.POINTER
_i, _u64, _d, _vp, _sz = ctypes.c_int, ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t

RESULT_AMPLITUDE0, RESULT_SAMPLE, RESULT_EXPECTATION = 0, 1, 2


class ServerResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("kind", ctypes.c_int), ("value_re", ctypes.c_double),
                ("value_im", ctypes.c_double), ("sample", ctypes.c_uint64), ("submit_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double), ("passes", ctypes.c_uint32)]


def _lib():
    lib = capi.load()
    if not getattr(lib, "_server_bound", False):
        lib.hqs_server_create.argtypes = [_i, _i, _u64, _i, _i, _P(_vp)]
        lib.hqs_server_destroy.argtypes = [_vp]
        lib.hqs_server_destroy.restype = None
        lib.hqs_server_last_error.argtypes = [_vp]
        lib.hqs_server_last_error.restype = ctypes.c_char_p
        lib.hqs_server_submit.argtypes = [_vp, _i, _i, _P(_i), _P(_i), _P(_i), _P(_i), _P(_d), _i, _d, _sz,
                                          _P(_u64), _P(_u64), _P(_u64), _P(_d), _P(_u64)]
        lib.hqs_server_step.argtypes = [_vp, _P(ServerResult), _sz, _P(_sz)]
        lib.hqs_server_info.argtypes = [_vp, _P(_u64)]
        lib.hqs_server_timing.argtypes = [_vp, _P(_d)]
        lib._server_bound = True
    return lib


@dataclass
class Circuit:
    """A circuit on qubits 0..n-1 in the C-ABI's flattened form."""
    n: int
    ntgt: np.ndarray
    tgt: np.ndarray
    nctl: np.ndarray
    ctl: np.ndarray
    mats: np.ndarray            # complex128, concatenated row-major matrices
    kind: int = RESULT_AMPLITUDE0
    rnd: float = 0.0
    pauli: list = field(default_factory=list)   # [(xmask, ymask, zmask, coef)]

    @property
    def ngates(self):
        return len(self.ntgt)

    @staticmethod
    def from_gates(n, gates, kind=RESULT_AMPLITUDE0, rnd=0.0, pauli=()):
        ntgt = np.array([len(g.ids) for g in gates], dtype=np.int32)
        nctl = np.array([len(g.ctrls) for g in gates], dtype=np.int32)
        tgt = np.array([q for g in gates for q in g.ids] or [0], dtype=np.int32)
        ctl = np.array([q for g in gates for q in g.ctrls] or [0], dtype=np.int32)
        mats = np.concatenate([np.asarray(g.matrix, dtype=np.complex128).reshape(-1) for g in gates]) \
            if gates else np.zeros(1, np.complex128)
        return Circuit(n, ntgt, tgt, nctl, ctl, mats, kind, rnd, list(pauli))


def pauli_masks(op):
    """[(term, coef)] with term [(qubit, 'X'|'Y'|'Z')] -> [(x, y, z, coef)]."""
    out = []
    for term, coef in op:
        x = y = z = 0
        for q, p in term:
            b = 1 << q
            if p == "X":
                x |= b
            elif p == "Y":
                x |= b
                y |= b
            else:
                z |= b
        out.append((x, y, z, complex(coef)))
    return out


class Server:
    def __init__(self, precision="c128", arith="auto", budget_bytes=150e9, max_active=4096, cluster_size=4):
        self.lib = _lib()
        h = _vp()
        rc = self.lib.hqs_server_create(capi.HQS_C64 if precision == "c64" else capi.HQS_C128, capi.ARITH[arith],
                                        int(budget_bytes), int(max_active), int(cluster_size), ctypes.byref(h))
        if rc:
            raise capi.HQSError(rc, self.lib.hqs_last_error().decode())
        self.h = h
        self._buf = (ServerResult * 4096)()

    def close(self):
        if getattr(self, "h", None):
            self.lib.hqs_server_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, rc):
        if rc:
            raise capi.HQSError(rc, self.lib.hqs_server_last_error(self.h).decode())

    def submit(self, c):
        T = len(c.pauli)
        px = np.array([p[0] for p in c.pauli] or [0], dtype=np.uint64)
        py = np.array([p[1] for p in c.pauli] or [0], dtype=np.uint64)
        pz = np.array([p[2] for p in c.pauli] or [0], dtype=np.uint64)
        co = np.array([[p[3].real, p[3].imag] for p in c.pauli] or [[0, 0]], dtype=np.float64)
        mats = np.ascontiguousarray(c.mats, dtype=np.complex128)
        rid = _u64()
        self._check(self.lib.hqs_server_submit(
            self.h, c.n, c.ngates, c.ntgt.ctypes.data_as(_P(_i)), c.tgt.ctypes.data_as(_P(_i)),
            c.nctl.ctypes.data_as(_P(_i)), c.ctl.ctypes.data_as(_P(_i)), mats.view(np.float64).ctypes.data_as(_P(_d)),
            c.kind, c.rnd, T, px.ctypes.data_as(_P(_u64)), py.ctypes.data_as(_P(_u64)),
            pz.ctypes.data_as(_P(_u64)), co.ctypes.data_as(_P(_d)), ctypes.byref(rid)))
        return rid.value

    def step(self):
        n = _sz()
        self._check(self.lib.hqs_server_step(self.h, self._buf, len(self._buf), ctypes.byref(n)))
        return [{f: getattr(self._buf[i], f) for f, _ in ServerResult._fields_} for i in range(n.value)]

    def info(self):
        out = (_u64 * 5)()
        self._check(self.lib.hqs_server_info(self.h, out))
        return dict(zip(("queued", "active", "bytes_in_use", "rounds", "launches"), list(out)))

    def timing(self):
        """Host seconds spent in step(), by phase."""
        out = (_d * 6)()
        self._check(self.lib.hqs_server_timing(self.h, out))
        return dict(zip(("batching", "staging_wait", "launch", "results", "admission", "step"), list(out)))

    def drain(self):
        res = []
        while True:
            r = self.step()
            res += r
            inf = self.info()
            if not r and inf["queued"] == 0 and inf["active"] == 0:
                return res


# ---------------------------------------------------------------- workload

def _haar_u2_batch(rng, count):
    g = (rng.standard_normal((count, 2, 2)) + 1j * rng.standard_normal((count, 2, 2))) / math.sqrt(2.0)
    a, b = g[:, :, 0], g[:, :, 1]
    q0 = a / np.linalg.norm(a, axis=1, keepdims=True)
    b = b - np.sum(np.conj(q0) * b, axis=1, keepdims=True) * q0
    q1 = b / np.linalg.norm(b, axis=1, keepdims=True)
    return np.stack([q0, q1], axis=2)  # columns q0, q1


def random_circuit(rng, n, layers):
    """Seeded random layers (Haar U(2) on every qubit, CNOTs on a random
    perfect matching, one controlled phase) in flattened form."""
    us = _haar_u2_batch(rng, layers * n)
    ntgt, tgt, nctl, ctl, mats = [], [], [], [], []
    X = np.array([0, 1, 1, 0], dtype=np.complex128)
    for l in range(layers):
        for q in range(n):
            ntgt.append(1); tgt.append(q); nctl.append(0); mats.append(us[l * n + q].reshape(-1))
        perm = rng.permutation(n)
        flips = rng.random(n // 2)
        for a in range(n // 2):
            c, t = int(perm[2 * a]), int(perm[2 * a + 1])
            if flips[a] < 0.5:
                c, t = t, c
            ntgt.append(1); tgt.append(t); nctl.append(1); ctl.append(c); mats.append(X)
        a, b = rng.choice(n, size=2, replace=False)
        th = rng.uniform(0, 2 * math.pi)
        ntgt.append(1); tgt.append(int(b)); nctl.append(1); ctl.append(int(a))
        mats.append(np.array([1, 0, 0, complex(math.cos(th), math.sin(th))]))
    return Circuit(n, np.array(ntgt, np.int32), np.array(tgt, np.int32), np.array(nctl, np.int32),
                   np.array(ctl or [0], np.int32), np.concatenate(mats))


def serving_workload(seed, count, nmin=10, nmax=22, dmin=10, dmax=60):
    """The serving mix: n ~ U{nmin..nmax}, depth ~ U{dmin..dmax} layers; 30%
    end in a full-register sample (seeded draw), 20% ask for <H> of an 8-term
    Pauli sum with N(0,1) coefficients, the rest for <0...0|psi>."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        d = int(rng.integers(dmin, dmax + 1))
        c = random_circuit(rng, n, d)
        u = rng.random()
        if u < 0.3:
            c.kind, c.rnd = RESULT_SAMPLE, float(rng.random())
        elif u < 0.5:
            c.kind = RESULT_EXPECTATION
            op = []
            for _t in range(8):
                w = int(rng.integers(1, min(n, 4) + 1))
                idx = sorted(int(i) for i in rng.choice(n, size=w, replace=False))
                op.append(([(i, "XYZ"[int(rng.integers(0, 3))]) for i in idx], float(rng.standard_normal())))
            c.pauli = pauli_masks(op)
        out.append(c)
    return out


def poisson_arrivals(seed, count, rate):
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    return np.cumsum(rng.exponential(1.0 / rate, size=count))


def serve(circuits, arrivals, precision="c128", arith="auto", budget_bytes=150e9, max_active=4096,
          cluster_size=4, server=None):
    """Replay arrivals (seconds from start) against a server. Returns
    (results by request index, stats)."""
    srv = server or Server(precision, arith, budget_bytes, max_active, cluster_size)
    id2idx = {}
    results = {}
    t0 = time.perf_counter()
    i = 0
    N = len(circuits)
    while len(results) < N:
        now = time.perf_counter() - t0
        while i < N and arrivals[i] <= now:
            id2idx[srv.submit(circuits[i])] = i
            i += 1
        for r in srv.step():
            k = id2idx[r["id"]]
            r["done_wall"] = time.perf_counter() - t0
            results[k] = r
        inf = srv.info()
        if inf["queued"] == 0 and inf["active"] == 0 and i < N and len(results) == i:
            wait = arrivals[i] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.05))
    lat = np.array([results[k]["done_wall"] - arrivals[k] for k in range(N)])
    span = max(r["done_wall"] for r in results.values()) - float(arrivals[0])
    stats = {"circuits": N, "circuits_per_s": N / span, "p50_ms": float(np.percentile(lat, 50) * 1e3),
             "p99_ms": float(np.percentile(lat, 99) * 1e3), "makespan_s": span,
             "rounds": srv.info()["rounds"], "launches": srv.info()["launches"]}
    if server is None:
        srv.close()
    return results, stats
