"""ctypes binding of the drop-in backend as a maintainer would add it next to
hiq/projectq/backends/_sim/_simulator_mpi.py. tests/test_boundary.py runs it
from the repository root: it loads libhqs.so, declares the calls it makes,
and raises RuntimeError with the library's message when a call fails."""
import ctypes, numpy as np
lib = ctypes.CDLL("hiqsimulator_gb300/libhqs.so")
lib.hqs_sim_last_error.restype = ctypes.c_char_p
lib.hqs_last_error.restype = ctypes.c_char_p

class SimulatorBackend:
    def __init__(self, seed, max_local, max_fused):
        self.h = ctypes.c_void_p()
        rc = lib.hqs_sim_create(ctypes.c_uint64(seed), ctypes.c_int64(max_local), ctypes.c_int64(max_fused),
                                0, 0, ctypes.byref(self.h))          # HQS_C128, HQS_ARITH_AUTO
        if rc: raise RuntimeError(lib.hqs_last_error().decode())
    def _check(self, rc):
        if rc: raise RuntimeError(lib.hqs_sim_last_error(self.h).decode())
    def allocate_qureg(self, ids, init=0j):
        a = np.asarray(ids, dtype=np.int64)
        self._check(lib.hqs_sim_allocate_qureg(self.h, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(len(a)),
                                               ctypes.c_double(complex(init).real), ctypes.c_double(complex(init).imag)))
    def apply_controlled_gate(self, m, ids, ctrls):
        m = np.ascontiguousarray(m, dtype=np.complex128); i = np.asarray(ids, np.int64); c = np.asarray(ctrls, np.int64)
        self._check(lib.hqs_sim_apply_controlled_gate(self.h, m.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(len(m)),
                    i.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(len(i)), c.ctypes.data_as(ctypes.c_void_p),
                    ctypes.c_size_t(len(c))))
    def run(self):
        self._check(lib.hqs_sim_run(self.h))
    # ... one wrapper per hqs_sim_* function, same pattern
