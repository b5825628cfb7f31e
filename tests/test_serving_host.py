"""Host-side pieces that need no GPU: the seeded serving workload mix and the
clustered inverse stream of the capacity report."""
import numpy as np


def test_serving_workload_is_seeded_and_well_formed():
    from hiqsimulator_gb300 import serving
    a = serving.serving_workload(5, 30)
    b = serving.serving_workload(5, 30)
    kinds = [c.kind for c in a]
    assert kinds == [c.kind for c in b]
    for c, d in zip(a, b):
        assert c.n == d.n and np.array_equal(c.mats, d.mats)
        assert 10 <= c.n <= 22
        assert c.ngates == len(c.nctl) and int(c.ntgt.sum()) <= len(c.tgt)
        k = 0
        for g in range(c.ngates):
            dim = 1 << int(c.ntgt[g])
            u = c.mats[k:k + dim * dim].reshape(dim, dim)
            assert np.allclose(u @ u.conj().T, np.eye(dim), atol=1e-12)
            k += dim * dim
    assert serving.RESULT_SAMPLE in kinds and serving.RESULT_EXPECTATION in kinds
    arr = serving.poisson_arrivals(5, 100, 50.0)
    assert np.all(np.diff(arr) > 0)


def test_clustered_inverse_stream_round_trips_on_the_oracle():
    """circuits.inverse_stream undoes a greedy-fused stream cluster by cluster
    (the capacity report's check), shown on the CPU oracle at 10 qubits."""
    import numpy as np

    from hiqsimulator_gb300 import circuits
    from oracle.engine import OracleSimulator
    n = 10
    gates, _ = circuits.capacity_circuit(seed=99, n=n)
    qs = list(range(n))
    clusters = circuits.greedy_clusters(gates, qs, 5)
    sim = OracleSimulator(99, n, 5)
    sim.allocate_qureg(qs, 0)
    circuits.replay(sim, circuits.greedy_stream(gates, qs, 5, clusters=clusters))
    assert abs(abs(np.asarray(sim.vec)[0]) ** 2 - 1.0) > 1e-3  # the circuit moved the state
    circuits.replay(sim, circuits.inverse_stream(gates, clusters))
    sim.run()
    assert abs(abs(np.asarray(sim.vec)[0]) ** 2 - 1.0) < 1e-12
