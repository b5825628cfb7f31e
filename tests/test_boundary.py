"""The C-ABI boundary without a GPU: libhqs.so loads, exports every function
include/hqs.h declares, rejects bad arguments before touching the device, and
its native greedy scheduler reproduces the reference's clusters."""
import ctypes
import json
import os

import pytest

from conftest import GOLDEN


def test_library_exports_every_header_symbol(hqs):
    from hiqsimulator_gb300 import capi
    lib = ctypes.CDLL(capi.LIB_PATH)
    names = capi.header_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_pybind_module_has_reference_methods(hqs):
    from hiqsimulator_gb300 import _cppsim_mpi
    ref_methods = ["get_qubits_ids", "get_local_qubits_ids", "get_global_qubits_ids", "set_qubits_perm",
                   "swap_qubits", "allocate_qureg", "allocate_qubit", "deallocate_qubit", "measure_qubits",
                   "apply_controlled_gate", "emulate_math", "get_amplitude", "get_probability", "run", "entropy",
                   "cheat_local", "collapse_wavefunction"]
    added = ["get_expectation_value", "apply_qubit_operator", "set_wavefunction"]
    extensions = ["cheat_local_numpy", "state_dlpack", "sample", "synchronize", "move_qubits"]
    for m in ref_methods + added + extensions:
        assert hasattr(_cppsim_mpi.SimulatorMPI, m), m


def test_invalid_arguments_rejected_without_device(hqs):
    from hiqsimulator_gb300 import capi
    lib = capi.load()
    h = ctypes.c_void_p()
    assert lib.hqs_sim_create(1, 20, 4, 7, 0, ctypes.byref(h)) == capi.HQS_ERR_INVALID
    assert b"precision" in lib.hqs_last_error()
    assert lib.hqs_sim_create(1, 20, 4, 0, 9, ctypes.byref(h)) == capi.HQS_ERR_INVALID
    assert lib.hqs_apply_gates(None, None, 3, 1, 0, None, None, None, None, None, 0, 0, None, None) == \
        capi.HQS_ERR_INVALID
    assert lib.hqs_sim_run(None) == capi.HQS_ERR_INVALID
    ptr, amps, dev = ctypes.c_void_p(), ctypes.c_uint64(), ctypes.c_int()
    assert lib.hqs_sim_state_view(None, ctypes.byref(ptr), ctypes.byref(amps), ctypes.byref(dev)) == \
        capi.HQS_ERR_INVALID
    assert b"null simulator" in lib.hqs_last_error()
    assert lib.hqs_version().startswith(b"hiqsimulator_gb300")


def test_native_scheduler_matches_reference_clusters(hqs):
    from hiqsimulator_gb300 import capi, circuits
    sch = json.load(open(os.path.join(GOLDEN, "ref_sched.json")))
    for name, c in sch.items():
        if name == "qft10_k5":
            gates = circuits.qft(list(range(10))) + circuits.random_layers(3, list(range(10)), 2)
            n, K = 10, 5
        else:
            gates = circuits.random_layers(c["seed"], list(range(c["n"])), c["layers"])
            n, K = c["n"], c["K"]
        got = capi.greedy_schedule([list(g.ids) for g in gates], [list(g.ctrls) for g in gates], list(range(n)), K)
        assert got == c["clusters"], name


@pytest.mark.parametrize("n,layers,K,seed", [(24, 2, 4, 11), (30, 2, 5, 12), (9, 10, 3, 13)])
def test_native_scheduler_matches_oracle_scheduler(hqs, n, layers, K, seed):
    from hiqsimulator_gb300 import capi, circuits
    from oracle.lib import greedy_schedule
    gates = circuits.qft(list(range(n)))[: 3 * n] + circuits.random_layers(seed, list(range(n)), layers)
    G = [list(g.ids) for g in gates]
    C = [list(g.ctrls) for g in gates]
    assert capi.greedy_schedule(G, C, list(range(n)), K) == greedy_schedule(G, C, list(range(n)), K)


def test_huge_gate_is_its_own_cluster(hqs):
    """A gate with more qubits than the cluster size is emitted alone
    (cluster_scheduler.cpp:69-73)."""
    from hiqsimulator_gb300 import capi
    gates = [[0], [1], [5], [2]]
    ctrls = [[], [], [0, 1, 2, 3, 4], []]
    cl = capi.greedy_schedule(gates, ctrls, list(range(6)), 4)
    flat = [i for c in cl for i in c]
    assert sorted(flat) == [0, 1, 2, 3]
    assert [2] in cl


def test_integration_ctypes_stub_runs(hqs, monkeypatch):
    """The ctypes binding printed for maintainers (tests/ctypes_stub.py) runs
    as written: it loads libhqs.so, declares the calls it makes, and turns a
    failed create (no CUDA device here) into RuntimeError with the library's
    message."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("checks the no-device error path")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    monkeypatch.chdir(root)
    ns = {}
    with open(os.path.join(root, "tests", "ctypes_stub.py")) as f:
        exec(compile(f.read(), "ctypes_stub.py", "exec"), ns)
    with pytest.raises(RuntimeError, match="CUDA"):
        ns["SimulatorBackend"](1, 20, 4)
