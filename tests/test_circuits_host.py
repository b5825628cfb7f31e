"""The seeded benchmark workloads on the host: each generator builds the
configuration it stands for (gate counts and structure of the 20q, 30q,
33q/34q capacity and 28q brickwork circuits; Haar samples are unitary; the
Grover iterations amplify the marked string)."""
import math

import numpy as np

from hiqsimulator_gb300 import circuits


def test_haar_samples_are_unitary():
    rng = circuits.rng_for(5)
    for d in (2, 4, 8):
        u = circuits.haar_unitary(rng, d)
        assert np.max(np.abs(u.conj().T @ u - np.eye(d))) < 1e-13


def test_random_layer_structure():
    n = 20
    gates = circuits.random_circuit_20q(seed=1234, n=n, layers=20)
    assert len(gates) == 20 * (n + n // 2 + 1)
    layer = gates[: n + n // 2 + 1]
    assert [len(g.matrix) for g in layer[:n]] == [2] * n and sorted(g.ids[0] for g in layer[:n]) == list(range(n))
    cnots = layer[n:n + n // 2]
    touched = sorted(q for g in cnots for q in g.ids + g.ctrls)
    assert touched == list(range(n))  # a perfect matching
    assert all(np.array_equal(g.matrix, circuits.X) and len(g.ctrls) == 1 for g in cnots)
    cp = layer[-1]
    assert len(cp.ctrls) == 1 and abs(cp.matrix[0, 0] - 1) == 0 and abs(abs(cp.matrix[1, 1]) - 1) < 1e-15


def test_qft_plus_layers_is_the_30_qubit_workload():
    gates = circuits.qft_random_layers(seed=4321, n=30, layers=10)
    qft = 30 + 30 * 29 // 2
    assert len(gates) == qft + 10 * (30 + 15 + 1) == 925
    assert sum(1 for g in gates[:qft] if not g.ctrls) == 30  # one H per qubit
    zz, shots = circuits.zz_pairs_and_shots(4321, 30)
    assert len(zz) == 64 and shots == 1024 and all(a != b for a, b in zz)


def test_capacity_circuit_structure_and_bias():
    n = 33
    gates, marked = circuits.capacity_circuit(seed=99, n=n, layers=8, grover=4)
    mcz = [g for g in gates if len(g.ctrls) == n - 1]
    assert len(mcz) == 8 and len(marked) == n  # oracle + diffusion per iteration
    top = set(range(n - 8, n))
    cnots = [g for g in gates[: 8 * (n + n // 2 + 1)] if len(g.ctrls) == 1 and np.array_equal(g.matrix, circuits.X)]
    mixed = [g for g in cnots if (g.ids[0] in top) != (g.ctrls[0] in top)]
    frac = sum(g.ids[0] in top for g in mixed) / len(mixed)
    assert frac > 0.7, frac  # 0.5 + 0.5 * 0.7 expected


def test_grover_iterations_amplify_the_marked_string():
    from oracle.engine import OracleSimulator
    n = 6
    qs = list(range(n))
    gates, marked = circuits.grover_iterations(7, qs, 4)
    sim = OracleSimulator(1, 10, 4)
    sim.allocate_qureg(qs, 0)
    for g in [circuits.Gate(circuits.H, [q], []) for q in qs] + gates:
        sim.apply_controlled_gate(g.matrix.tolist(), list(g.ids), list(g.ctrls))
        sim.run()
    p = sim.get_probability([bool(b) for b in marked], qs)
    theta = math.asin(1 / math.sqrt(2 ** n))
    assert abs(p - math.sin(9 * theta) ** 2) < 1e-12


def test_brickwork_28q_structure():
    gates = circuits.brickwork_28q(seed=2024, n=28, layers=40)
    assert len(gates) == 20 * 14 + 20 * 13
    assert [g.ids for g in gates[:2]] == [[0, 1], [2, 3]] and gates[14].ids == [1, 2]
    assert all(g.matrix.shape == (4, 4) for g in gates)
