"""Host FP64 fusion (hqs_fuse, the engine's Fusion class) against the oracle's
restatement of fusion_mpi.hpp:85-226 on the CPU: random gate streams with
targets, controls shared by some or all gates, diagonal gates and scalars."""
import numpy as np
import pytest

from hiqsimulator_gb300 import circuits


def _oracle_fuse(gates):
    from oracle.engine import Fusion, _is_diag
    f = Fusion()
    for m, ids, ctrls in gates:
        f.insert(np.asarray(m, dtype=np.complex128), _is_diag(m), list(ids), list(ctrls))
    return f.perform_fusion()


def _random_gate(rng, pool):
    k = int(rng.integers(0, 3))
    if k == 0:
        return (np.array([[np.exp(1j * rng.uniform(0, 6.3))]]), [], [])
    ids = [int(q) for q in rng.choice(pool, size=k, replace=False)]
    rest = [q for q in pool if q not in ids]
    ctrls = [int(q) for q in rng.choice(rest, size=int(rng.integers(0, 3)), replace=False)]
    if rng.random() < 0.4:
        m = np.diag(np.exp(1j * rng.uniform(0, 6.3, size=1 << k)))
    else:
        m = circuits.haar_unitary(rng, 1 << k)
    return (m, ids, ctrls)


@pytest.mark.parametrize("seed", range(12))
def test_fusion_matches_oracle(hqs, seed):
    from hiqsimulator_gb300 import capi
    rng = np.random.Generator(np.random.PCG64(900 + seed))
    pool = list(range(3, 3 + 5 + seed % 3))
    for _ in range(10):
        gates = [_random_gate(rng, pool) for _ in range(int(rng.integers(1, 6)))]
        want = _oracle_fuse(gates)
        if len(want[1]) > 10:
            continue
        M, ids, ctrls, diag = capi.fuse(gates)
        assert (ids, ctrls, diag) == (want[1], want[2], want[3])
        assert np.max(np.abs(M - want[0])) <= 1e-15


def test_fusion_known_cases(hqs):
    from hiqsimulator_gb300 import capi
    # a controlled phase alone keeps its control as a control of the fused gate
    M, ids, ctrls, diag = capi.fuse([(circuits.phase(0.5), [4], [7])])
    assert ids == [4] and ctrls == [7] and diag
    # a control shared by every gate stays a control; the fused gate is diagonal
    M, ids, ctrls, diag = capi.fuse([(circuits.Z, [1], [9]), (circuits.phase(0.3), [2], [9])])
    assert ids == [1, 2] and ctrls == [9] and diag
    assert np.allclose(M, np.diag([1, -1, np.exp(0.3j), -np.exp(0.3j)]), atol=1e-15)
    # a control not shared by a later gate folds into the matrices as a target
    M, ids, ctrls, diag = capi.fuse([(circuits.X, [1], [0]), (circuits.H, [2], [])])
    assert ids == [0, 1, 2] and ctrls == [] and not diag
    # scalars only scale
    M, ids, ctrls, diag = capi.fuse([(np.array([[1j]]), [], []), (circuits.H, [5], [])])
    assert ids == [5] and np.allclose(M, 1j * circuits.H, atol=1e-16)


def test_fusion_rejects_bad_gates(hqs):
    from hiqsimulator_gb300 import capi
    with pytest.raises(capi.HQSError):
        capi.fuse([(np.eye(4), [0], [])])  # 4x4 matrix on one qubit
    with pytest.raises(capi.HQSError):
        capi.fuse([(np.eye(2), [q], []) for q in range(13)])  # more than 12 fused qubits
