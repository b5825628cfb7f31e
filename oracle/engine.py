"""Python restatement of the reference SimulatorMPI engine on one rank.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py). Host logic follows
src/simulator-mpi/SimulatorMPI.cpp and src/simulator-mpi/fusion_mpi.hpp line
by line in behaviour (qubit positions, fusion rules, error messages); the state
sweeps run in the C oracle (sv_oracle.c). With one rank there are no global
qubits, so every global-qubit branch of the reference collapses to its local
case.
"""
import numpy as np

from .lib import MT19937, dptr, load_oracle_lib
import ctypes
import time


class Fusion:
    """fusion_mpi.hpp:61-234: collects gates and composes one dense matrix."""

    def __init__(self):
        self.set_ = set()
        self.items = []          # [matrix (np.ndarray), diag flag, ids list]
        self.ctrl_set = set()
        self.factor = 1.0 + 0j

    def num_qubits(self):
        return len(self.set_)

    @staticmethod
    def add_controls(matrix, ids, new_ctrls):
        """fusion_mpi.hpp:167-187: controls become the highest matrix bits;
        identity everywhere except the bottom-right block."""
        ids = list(ids) + list(new_ctrls)
        F = 1 << len(new_ctrls)
        d = matrix.shape[0]
        out = np.zeros((F * d, F * d), dtype=np.complex128)
        off = F * d - d
        for i in range(off):
            out[i, i] = 1.0
        out[off:, off:] = matrix
        return out, ids

    def insert(self, matrix, diag, ids, ctrls=()):
        """fusion_mpi.hpp:85-99."""
        if matrix.shape[0] == 1:
            self.factor *= matrix[0, 0]
            return
        ids = list(ids)
        for i in ids:
            self.set_.add(i)
        matrix, ids = self._handle_controls(matrix, ids, list(ctrls))
        self.items.append([matrix, diag, ids])

    def _handle_controls(self, matrix, ids, ctrls):
        """fusion_mpi.hpp:190-226."""
        unhandled = set(self.ctrl_set)
        for c in ctrls:
            if c not in self.ctrl_set:
                if self.items:
                    matrix, ids = self.add_controls(matrix, ids, [c])
                    self.set_.add(c)
                else:
                    self.ctrl_set.add(c)
            else:
                unhandled.discard(c)
        if unhandled:
            new = sorted(unhandled)
            for c in new:
                self.ctrl_set.discard(c)
                self.set_.add(c)
            for it in self.items:
                it[0], it[2] = self.add_controls(it[0], it[2], new)
        return matrix, ids

    def perform_fusion(self):
        """fusion_mpi.hpp:101-165: M = items[-1] ... items[0] * factor over the
        sorted id set; bit l of M <-> l-th smallest id."""
        ids = sorted(self.set_)
        N = len(ids)
        dim = 1 << N
        M = np.eye(dim, dtype=np.complex128) * self.factor
        self.factor = 1.0 + 0j
        diag = True
        rows = np.arange(dim)
        for mat, idiag, iids in self.items:
            if not idiag:
                diag = False
            pos = [ids.index(q) for q in iids]
            k = len(iids)
            # M <- (item (x) I) @ M: row i of the result mixes the rows of M whose
            # index differs from i only at the item's bits.
            local_i = np.zeros(dim, dtype=np.int64)
            for l, p in enumerate(pos):
                local_i |= ((rows >> p) & 1) << l
            base = rows.copy()
            for p in pos:
                base &= ~(1 << p)
            newM = np.zeros_like(M)
            for j in range(1 << k):
                src = base.copy()
                for l, p in enumerate(pos):
                    src |= ((j >> l) & 1) << p
                newM += mat[local_i, j][:, None] * M[src, :]
            M = newM
        ctrls = sorted(self.ctrl_set)
        return M, ids, ctrls, diag


def _is_diag(m):
    """funcs.hpp:325-337: exact test of every off-diagonal element."""
    off = m - np.diag(np.diag(m))
    return not np.any(off != 0)


class OracleSimulator:
    """SimulatorMPI(seed, max_local, max_cluster_size) on one rank."""

    MAX_FLOAT_ERROR = 1e-12

    def __init__(self, seed, max_local, max_cluster_size):
        self.lib = load_oracle_lib()
        self.rng = MT19937(seed)
        self.max_local = int(max_local)
        self.min_local = int(max_cluster_size)
        self.max_cluster = int(max_cluster_size)
        self.locals = []
        self.vec = np.ones(1, dtype=np.complex128)
        self.fusion = Fusion()
        self.last_margin = None

    # --- qubit map -------------------------------------------------------
    def _find_sure(self, v, val):
        if val not in v:
            raise RuntimeError("ArrayFindSure(): Can't find %d in " % val)
        return v.index(val)

    def allocate_qubit(self, qid):
        """SimulatorMPI.cpp:184-216 (one rank: always local)."""
        if len(self.locals) < self.min_local or len(self.locals) < self.max_local:
            self.locals.append(int(qid))
            self.vec = np.concatenate([self.vec, np.zeros_like(self.vec)])
        else:
            raise RuntimeError("AllocateQubit(): can't allocate more than %d qubits" % len(self.locals))

    def allocate_qureg(self, ids, init=0.0):
        """SimulatorMPI.cpp:218-251."""
        if init != 0.0 and self.locals:
            raise RuntimeError("AllocateQureg(): initialization of only first qureg is supported")
        for i in ids:
            self.allocate_qubit(i)
        if init != 0.0:
            self.lib.orc_fill(dptr(self.vec.view(np.float64)), len(self.vec), complex(init).real, complex(init).imag)

    def deallocate_qubit(self, qid):
        """SimulatorMPI.cpp:278-322 / 369-426."""
        pos = self._find_sure(self.locals, qid)
        p = np.zeros(2)
        self.lib.orc_bit_probs(dptr(self.vec.view(np.float64)), len(self.vec), pos, dptr(p))
        if not ((p[0] > self.MAX_FLOAT_ERROR) ^ (p[1] > self.MAX_FLOAT_ERROR)):
            raise RuntimeError("DeallocateLocalQubit(): qubit %d is entangled" % qid)
        keep = 0 if p[0] > self.MAX_FLOAT_ERROR else 1
        self.lib.orc_drop_bit(dptr(self.vec.view(np.float64)), len(self.vec), pos, keep)
        self.vec = self.vec[: len(self.vec) // 2].copy()
        del self.locals[pos]

    def get_qubits_ids(self):
        return list(self.locals)

    def set_qubits_perm(self, perm):
        self.locals = [int(x) for x in perm[: len(self.locals)]]

    # --- gates -------------------------------------------------------------
    def apply_controlled_gate(self, m, ids, ctrls):
        """SimulatorMPI.cpp:710-815 on one rank."""
        m = np.array(m, dtype=np.complex128)
        ids = [int(i) for i in ids]
        ctrls = [int(c) for c in ctrls]
        diag = _is_diag(m)
        local_ctrls = [c for c in ctrls if c in self.locals]
        if len(ids) + len(local_ctrls) > self.max_cluster:
            self.run()
            self.fusion.insert(m, diag, ids, ctrls)
            return
        m, ids = Fusion.add_controls(m, ids, local_ctrls)
        self.fusion.insert(m, diag, ids, [])

    def run(self):
        """SimulatorMPI.cpp:441-541."""
        self.run_timed()

    def run_timed(self):
        """run(), returning the seconds spent in the state sweep alone (the
        fusion of the queued gates is not timed)."""
        M, ids, ctrls, diag = self.fusion.perform_fusion()
        ctrl_mask = 0
        for c in ctrls:
            if c in self.locals:
                ctrl_mask |= 1 << self.locals.index(c)
        pos = [self._find_sure(self.locals, q) for q in ids]
        k = len(ids)
        if k > 5:
            # the reference throws before resetting its fusion queue
            raise RuntimeError("Run(): cannot apply %d qubits gate" % k)
        t0 = time.perf_counter()
        self.apply_matrix(M, pos, ctrl_mask, diag)
        dt = time.perf_counter() - t0
        self.fusion = Fusion()
        return dt

    def apply_matrix(self, M, pos, ctrl_mask=0, diag=False):
        M = np.ascontiguousarray(M, dtype=np.complex128)
        k = len(pos)
        parr = (ctypes.c_uint * max(k, 1))(*pos)
        self.lib.orc_apply(dptr(self.vec.view(np.float64)), len(self.vec), k, parr,
                           dptr(M.view(np.float64)), ctrl_mask, 1 if diag else 0)

    # --- queries -----------------------------------------------------------
    def _mask_val(self, ids, bits):
        msk = val = 0
        for q, b in zip(ids, bits):
            pos = self._find_sure(self.locals, q) if q in self.locals else self._find_sure([], q)
            msk |= 1 << pos
            if b:
                val |= 1 << pos
        return msk, val

    def get_probability(self, bits, ids):
        """SimulatorMPI.cpp:561-600."""
        if len(ids) != len(bits):
            raise RuntimeError("GetProbability(): ids.size() != bit_string.size()")
        msk, val = self._mask_val(ids, bits)
        return self.lib.orc_probability(dptr(self.vec.view(np.float64)), len(self.vec), msk, val)

    def get_amplitude(self, bits, ids):
        """SimulatorMPI.cpp:602-650."""
        if len(bits) != len(self.locals) or len(bits) != len(ids):
            raise RuntimeError("GetAmplitude(): ids.size() != number of qubits")
        num = check = 0
        for q, b in zip(ids, bits):
            pos = self._find_sure(self.locals, q) if q in self.locals else self._find_sure([], q)
            if b:
                num |= 1 << pos
            check |= 1 << pos
        if check != (1 << len(self.locals)) - 1:
            raise RuntimeError("GetAmplitude(): the second argument must be a permutation of all allocated qubits.")
        return complex(self.vec[num])

    def collapse_wavefunction(self, ids, values):
        """SimulatorMPI.cpp:1010-1058."""
        if len(ids) != len(values):
            raise RuntimeError("collapseWaveFunction(): ids.size() != values.size()")
        msk, val = self._mask_val(ids, values)
        p = self.lib.orc_probability(dptr(self.vec.view(np.float64)), len(self.vec), msk, val)
        if p < 1e-12:
            raise RuntimeError("collapseWaveFunction(): Invalid collapse! Probability is ~0.")
        self.lib.orc_normalize(dptr(self.vec.view(np.float64)), len(self.vec), msk, val, p)

    def sample_index(self, rnd):
        margin = ctypes.c_double(0)
        idx = self.lib.orc_sample_index(dptr(self.vec.view(np.float64)), len(self.vec), rnd, ctypes.byref(margin))
        self.last_margin = margin.value
        return idx

    def sample_many(self, rnds):
        """sample_index for every draw of rnds on the current state (one
        block CDF): (indices, margins) as int64 / float64 arrays."""
        r = np.ascontiguousarray(rnds, dtype=np.float64)
        idx = np.zeros(len(r), dtype=np.int64)
        mar = np.zeros(len(r), dtype=np.float64)
        self.lib.orc_sample_many(dptr(self.vec.view(np.float64)), len(self.vec), len(r), dptr(r),
                                 idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), dptr(mar))
        return idx, mar

    def measure_qubits(self, ids):
        """SimulatorMPI.cpp:897-1008."""
        rnd = self.rng.uniform()
        idx = self.sample_index(rnd)
        if idx < 0:
            raise RuntimeError("MeasureQubits(): Random number %.3f > norm partial sum" % rnd)
        res = []
        msk = val = 0
        for q in ids:
            pos = self._find_sure(self.locals, q)
            msk |= 1 << pos
            bit = (idx >> pos) & 1
            if bit:
                val |= 1 << pos
            res.append(bool(bit))
        p = self.lib.orc_probability(dptr(self.vec.view(np.float64)), len(self.vec), msk, val)
        self.lib.orc_normalize(dptr(self.vec.view(np.float64)), len(self.vec), msk, val, p)
        return res

    def entropy(self):
        return self.lib.orc_entropy(dptr(self.vec.view(np.float64)), len(self.vec))

    def cheat_local(self):
        return {q: p for p, q in enumerate(self.locals)}, self.vec.copy()

    # --- Pauli operators (documented semantics, _simulator_mpi.py:148-223) ---
    def _pauli_masks(self, op, ids):
        xm, ym, zm, co = [], [], [], []
        for term, coef in op:
            x = y = z = 0
            for idx, p in term:
                if idx >= len(ids):
                    raise RuntimeError("qubit_operator acts on more qubits than contained in the qureg.")
                pos = self._find_sure(self.locals, ids[idx])
                if p == 'X':
                    x |= 1 << pos
                elif p == 'Y':
                    x |= 1 << pos
                    y |= 1 << pos
                elif p == 'Z':
                    z |= 1 << pos
                else:
                    raise RuntimeError("unknown Pauli operator %r" % (p,))
            xm.append(x); ym.append(y); zm.append(z)
            c = complex(coef)
            co += [c.real, c.imag]
        return (np.array(xm, dtype=np.uint64), np.array(ym, dtype=np.uint64),
                np.array(zm, dtype=np.uint64), np.array(co, dtype=np.float64))

    def get_expectation_value(self, op, ids):
        xm, ym, zm, co = self._pauli_masks(op, ids)
        up = ctypes.POINTER(ctypes.c_uint64)
        return self.lib.orc_expectation(dptr(self.vec.view(np.float64)), len(self.vec), len(xm),
                                        xm.ctypes.data_as(up), ym.ctypes.data_as(up), zm.ctypes.data_as(up), dptr(co))

    def apply_qubit_operator(self, op, ids):
        xm, ym, zm, co = self._pauli_masks(op, ids)
        up = ctypes.POINTER(ctypes.c_uint64)
        self.lib.orc_apply_pauli_sum(dptr(self.vec.view(np.float64)), len(self.vec), len(xm),
                                     xm.ctypes.data_as(up), ym.ctypes.data_as(up), zm.ctypes.data_as(up), dptr(co))

    def set_wavefunction(self, wf, ids):
        wf = np.asarray(wf, dtype=np.complex128)
        if len(wf) != (1 << len(self.locals)) or sorted(ids) != sorted(self.locals):
            raise RuntimeError("set_wavefunction(): the qureg must contain all allocated qubits "
                               "and the wavefunction must have 2^n entries")
        self.locals = [int(i) for i in ids]
        self.vec = wf.copy()
