"""Capacity states: 33 qubits in complex128 and 34 in complex64 (128 GiB each)
on one GPU, with a circuit of random layers (CNOT targets biased towards the
top 8 qubits) and Grover iterations whose multi-controlled Z spans every
qubit (a 1-target gate with n-1 controls, SimulatorMPI.cpp:730-756).

No host oracle holds these states, so the full-size check is a round trip:
the circuit, then its inverse, must return |0...0> (|<0|psi>|^2 >= 1 - tol)
with the norm kept at every stage. The same circuit family at 22 qubits is
compared with the oracle amplitude by amplitude."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_bytes():
    import torch
    free, _ = torch.cuda.mem_get_info()
    return free


@pytest.mark.parametrize("precision,n,tol", [("c128", 33, 1e-10), ("c64", 34, 2e-5)])
def test_capacity_round_trip(hqs, cuda, precision, n, tol):
    from hiqsimulator_gb300 import circuits
    elem = 16 if precision == "c128" else 8
    if _free_bytes() < (elem << n) + (8 << 30):
        pytest.skip("device memory below the %d-qubit %s state" % (n, precision))
    gates, _ = circuits.capacity_circuit(seed=99, n=n)
    qs = list(range(n))
    sim = hqs.SimulatorMPI(99, n, 5, precision)
    sim.allocate_qureg(qs, 0)
    circuits.replay(sim, circuits.fusion_off_stream(gates))
    norm = sim.get_probability([], [])
    assert abs(norm - 1.0) < tol, norm
    p_top = sim.get_probability([True], [n - 1])
    assert 0.0 <= p_top <= 1.0 + tol
    circuits.replay(sim, circuits.fusion_off_stream(circuits.inverse(gates)))
    amp0 = sim.get_amplitude([False] * n, qs)
    assert abs(amp0) ** 2 > 1.0 - tol, amp0
    assert abs(sim.get_probability([], []) - 1.0) < tol
    del sim


def test_capacity_circuit_family_matches_oracle(hqs, cuda):
    from hiqsimulator_gb300 import circuits
    from oracle.engine import OracleSimulator
    n = 22
    gates, _ = circuits.capacity_circuit(seed=99, n=n)
    qs = list(range(n))
    cmds = circuits.fusion_off_stream(gates)
    sim = hqs.SimulatorMPI(99, n, 5, "c128")
    ref = OracleSimulator(99, n, 5)
    for s in (sim, ref):
        s.allocate_qureg(qs, 0)
        circuits.replay(s, cmds)
    _, vec = sim.cheat_local_numpy()
    assert np.max(np.abs(vec - ref.vec)) < 1e-12
