"""The oracle's restatement of the three methods the reference never
implemented (get_expectation_value, apply_qubit_operator, set_wavefunction;
semantics of hiq/projectq/backends/_sim/_simulator_mpi.py:148-306), checked on
the CPU: against dense Kronecker-product operators built independently in
numpy, and against the known answers of the reference's commented-out tests
(_simulator_mpi_test.py:382-425, 454-478, 540-566)."""
import math

import numpy as np
import pytest

from oracle.engine import OracleSimulator

PAULI = {"X": np.array([[0, 1], [1, 0]], dtype=complex), "Y": np.array([[0, -1j], [1j, 0]]),
         "Z": np.array([[1, 0], [0, -1]], dtype=complex)}
H = np.array([[1, 1], [1, -1]]) / math.sqrt(2)
X = PAULI["X"]
Z = PAULI["Z"]


def dense_term(term, ids, locals_):
    """The 2^n operator of one Pauli string; bit p of the index <-> locals_[p]."""
    per_pos = [np.eye(2, dtype=complex) for _ in locals_]
    for idx, p in term:
        per_pos[locals_.index(ids[idx])] = PAULI[p]
    op = np.eye(1, dtype=complex)
    for m in per_pos:  # position 0 is the least significant bit: kron high positions first
        op = np.kron(m, op)
    return op


def random_op(rng, nq):
    op = []
    for _ in range(int(rng.integers(1, 5))):
        k = int(rng.integers(0, 4))
        idx = [int(i) for i in rng.choice(nq, size=k, replace=False)]
        term = [(i, "XYZ"[int(rng.integers(0, 3))]) for i in idx]
        op.append((term, complex(rng.normal(), rng.normal())))
    return op


def random_sim(rng, n):
    sim = OracleSimulator(3, 16, 4)
    ids = [10 + i for i in range(n)]
    sim.allocate_qureg(ids, 0)
    order = [int(i) for i in rng.permutation(ids)]
    wf = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    sim.set_wavefunction(wf / np.linalg.norm(wf), order)
    assert sim.get_qubits_ids() == order
    return sim, order


@pytest.mark.parametrize("seed", range(6))
def test_expectation_matches_dense_operators(seed):
    rng = np.random.Generator(np.random.PCG64(500 + seed))
    n = 5
    sim, order = random_sim(rng, n)
    qureg = [int(i) for i in rng.permutation(order)]  # the operator's own index order
    for _ in range(5):
        op = random_op(rng, n)
        want = sum((c * np.vdot(sim.vec, dense_term(t, qureg, order) @ sim.vec)).real for t, c in op)
        assert abs(sim.get_expectation_value(op, qureg) - want) < 1e-12


@pytest.mark.parametrize("seed", range(6))
def test_apply_qubit_operator_matches_dense_operators(seed):
    rng = np.random.Generator(np.random.PCG64(600 + seed))
    n = 5
    sim, order = random_sim(rng, n)
    qureg = [int(i) for i in rng.permutation(order)]
    op = random_op(rng, n)
    want = sum(c * (dense_term(t, qureg, order) @ sim.vec) for t, c in op)
    sim.apply_qubit_operator(op, qureg)
    assert np.max(np.abs(sim.vec - want)) < 1e-12


def test_operator_on_more_qubits_than_the_qureg_raises():
    sim = OracleSimulator(1, 8, 4)
    sim.allocate_qureg([0, 1, 2], 0)
    with pytest.raises(RuntimeError, match="more qubits than contained in the qureg"):
        sim.get_expectation_value([([(3, "Z")], 1.0)], [0, 1, 2])
    with pytest.raises(RuntimeError):
        sim.apply_qubit_operator([([(1, "X")], 1.0)], [0])


def g1(sim, m, q):
    sim.apply_controlled_gate(np.asarray(m, dtype=complex).tolist(), [q], [])
    sim.run()


def test_expectation_known_answers():
    sim = OracleSimulator(1, 8, 4)
    q = [0, 1, 2]
    sim.allocate_qureg(q, 0)
    ev = sim.get_expectation_value
    assert abs(ev([([(0, "Z")], 1.0)], q) - 1) < 1e-12
    g1(sim, X, 0)
    assert abs(ev([([(0, "Z")], 1.0)], q) + 1) < 1e-12
    g1(sim, H, 0)
    assert abs(ev([([(0, "X")], 1.0)], q) + 1) < 1e-12
    g1(sim, Z, 0)
    assert abs(ev([([(0, "X")], 1.0)], q) - 1) < 1e-12
    for m in (X, [[1, 0], [0, 1j]], Z, X):
        g1(sim, m, 0)
    assert abs(ev([([(0, "Y")], 1.0)], q) - 1) < 1e-12
    g1(sim, Z, 0)
    assert abs(ev([([(0, "Y")], 1.0)], q) + 1) < 1e-12
    op_sum = [([(0, "Y"), (1, "X"), (2, "Z")], 1.0), ([(1, "X")], 1.0)]
    g1(sim, H, 1)
    g1(sim, X, 2)
    assert abs(ev(op_sum, q) - 2) < 1e-12
    g1(sim, X, 2)
    assert abs(ev(op_sum, q)) < 1e-12
    assert abs(ev([([], 0.4)], q) - 0.4) < 1e-12


def test_apply_qubit_operator_known_answers():
    sim = OracleSimulator(1, 8, 4)
    q = [0, 1, 2]
    sim.allocate_qureg(q, 0)
    sim.apply_qubit_operator([([(0, "X"), (1, "Y"), (2, "Z")], 1.0)], q)
    g1(sim, X, 0)
    g1(sim, PAULI["Y"], 1)
    g1(sim, Z, 2)
    assert abs(sim.get_amplitude([False] * 3, q) - 1.0) < 1e-12
    g1(sim, H, 0)
    s = 1 / math.sqrt(2)
    sim.apply_qubit_operator([([(0, "X")], s), ([(0, "Z")], s)], [0])
    assert abs(sim.get_amplitude([False] * 3, q) - 1.0) < 1e-12
    g1(sim, H, 0)
    sim.apply_qubit_operator([([], 0.5), ([(0, "Z")], 0.5)], [0])
    assert abs(sim.get_amplitude([False] * 3, q) - s) < 1e-12
    sim.apply_qubit_operator([([], 0.5), ([(0, "Z")], -0.5)], [0])
    assert abs(sim.get_amplitude([False] * 3, q)) < 1e-12


def test_set_wavefunction_known_answers():
    sim = OracleSimulator(1, 8, 4)
    wf = [0.0, 0.0, math.sqrt(0.2), math.sqrt(0.8)]
    with pytest.raises(RuntimeError):
        sim.set_wavefunction(wf, [0, 1])
    sim.allocate_qureg([0, 1], 0)
    sim.set_wavefunction(wf, [0, 1])
    assert abs(sim.get_probability([True], [0]) - 0.8) < 1e-12
    assert abs(sim.get_probability([False, True], [0, 1]) - 0.2) < 1e-12
    assert abs(sim.get_probability([True], [1]) - 1.0) < 1e-12
    sim2 = OracleSimulator(1, 8, 4)
    sim2.allocate_qubit(0)
    sim2.set_wavefunction([1.0, 0.0], [0])
    g1(sim2, PAULI["Y"], 0)
    assert abs(sim2.get_amplitude([True], [0]) - 1j) < 1e-12
