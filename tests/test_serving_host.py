"""Host-side pieces of serving that need no GPU: the seeded workload mix."""
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
