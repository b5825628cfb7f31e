"""Batched serving: results equal the same circuit run alone, match the
oracle, and respect the HBM admission budget."""
import pytest

pytestmark = pytest.mark.gpu


def _oracle_result(c):
    from oracle.engine import OracleSimulator
    sim = OracleSimulator(1, 26, 5)
    sim.allocate_qureg(list(range(c.n)), 0)
    off_t = off_c = off_m = 0
    for g in range(c.ngates):
        k, nc = int(c.ntgt[g]), int(c.nctl[g])
        tg = [int(x) for x in c.tgt[off_t:off_t + k]]
        cs = [int(x) for x in c.ctl[off_c:off_c + nc]]
        d = 1 << k
        m = c.mats[off_m:off_m + d * d].reshape(d, d)
        off_t += k; off_c += nc; off_m += d * d
        sim.apply_controlled_gate(m.tolist(), tg, cs)
        sim.run()
    return sim


def _mix(seed, count, nmax=14):
    from hiqsimulator_gb300 import serving
    return serving.serving_workload(seed, count, nmin=6, nmax=nmax, dmin=3, dmax=12)


@pytest.mark.parametrize("precision,arith", [("c128", "auto"), ("c64", "f32"), ("c64", "tc"), ("c64", "tf32")])
def test_result_alone_equals_result_in_mix(hqs, cuda, precision, arith):
    from hiqsimulator_gb300 import serving
    circuits = _mix(11, 24)
    alone = {}
    for idx in (0, 5, 9, 17):
        srv = serving.Server(precision, arith, budget_bytes=1 << 30)
        srv.submit(circuits[idx])
        alone[idx] = srv.drain()[0]
        srv.close()
    srv = serving.Server(precision, arith, budget_bytes=1 << 30)
    ids = {srv.submit(c): i for i, c in enumerate(circuits)}
    mixed = {ids[r["id"]]: r for r in srv.drain()}
    assert len(mixed) == len(circuits)
    for idx, r in alone.items():
        m = mixed[idx]
        assert (r["value_re"], r["value_im"], r["sample"]) == (m["value_re"], m["value_im"], m["sample"]), idx


def test_results_match_oracle(hqs, cuda, oracle_lib):
    from hiqsimulator_gb300 import serving
    circuits = _mix(12, 12, nmax=12)
    srv = serving.Server("c128", budget_bytes=1 << 30)
    ids = {srv.submit(c): i for i, c in enumerate(circuits)}
    res = {ids[r["id"]]: r for r in srv.drain()}
    for i, c in enumerate(circuits):
        sim = _oracle_result(c)
        r = res[i]
        if c.kind == serving.RESULT_AMPLITUDE0:
            assert abs(complex(r["value_re"], r["value_im"]) - sim.vec[0]) < 1e-12
        elif c.kind == serving.RESULT_SAMPLE:
            assert r["sample"] == sim.sample_index(c.rnd)
        else:
            op = []
            for x, y, z, coef in c.pauli:
                term = []
                for q in range(c.n):
                    b = 1 << q
                    if y & b:
                        term.append((q, "Y"))
                    elif x & b:
                        term.append((q, "X"))
                    elif z & b:
                        term.append((q, "Z"))
                op.append((term, coef))
            assert abs(r["value_re"] - sim.get_expectation_value(op, list(range(c.n)))) < 1e-11


def test_admission_respects_budget(hqs, cuda):
    from hiqsimulator_gb300 import serving
    circuits = _mix(13, 16, nmax=14)
    budget = 2 * (1 << 14) * 16  # two of the largest states at a time
    srv = serving.Server("c128", budget_bytes=budget)
    for c in circuits:
        srv.submit(c)
    done = []
    peak = 0
    while len(done) < len(circuits):
        done += srv.step()
        peak = max(peak, srv.info()["bytes_in_use"])
    assert peak <= budget
    ref = serving.Server("c128", budget_bytes=1 << 30)
    for c in circuits:
        ref.submit(c)
    a = sorted((r["id"], r["value_re"], r["sample"]) for r in done)
    b = sorted((r["id"], r["value_re"], r["sample"]) for r in ref.drain())
    assert a == b


def test_poisson_serving_reports_latency(hqs, cuda):
    from hiqsimulator_gb300 import serving
    circuits = _mix(14, 40, nmax=12)
    arr = serving.poisson_arrivals(14, len(circuits), rate=2000.0)
    res, st = serving.serve(circuits, arr, budget_bytes=1 << 30)
    assert st["circuits"] == 40 and st["p99_ms"] >= st["p50_ms"] > 0
    res1, st1 = serving.serve(circuits, arr, budget_bytes=1 << 30, max_active=1)
    for i in range(len(circuits)):
        assert (res[i]["value_re"], res[i]["sample"]) == (res1[i]["value_re"], res1[i]["sample"])


@pytest.mark.parametrize("precision", ["c128", "c64"])
def test_large_states_in_tensor_memory_launches(hqs, cuda, oracle_lib, precision):
    """complex128 states of 18 qubits or more run their dense gates as
    tensor-memory launches inside the rounds, next to the batched small
    states (complex64 states stay batched): results are the same alone and
    in the mix, and (complex128) match the oracle."""
    from hiqsimulator_gb300 import serving
    large = serving.serving_workload(21, 4, nmin=18, nmax=19, dmin=3, dmax=5)
    circuits = large + _mix(22, 8)
    alone = {}
    for idx in (0, 1):
        srv = serving.Server(precision, "auto", budget_bytes=1 << 32)
        srv.submit(circuits[idx])
        alone[idx] = srv.drain()[0]
        srv.close()
    srv = serving.Server(precision, "auto", budget_bytes=1 << 32)
    ids = {srv.submit(c): i for i, c in enumerate(circuits)}
    mixed = {ids[r["id"]]: r for r in srv.drain()}
    assert srv.info()["launches"] > 0
    for idx, r in alone.items():
        m = mixed[idx]
        assert (r["value_re"], r["value_im"], r["sample"]) == (m["value_re"], m["value_im"], m["sample"]), idx
    if precision != "c128":
        return
    for i in range(2):
        c = circuits[i]
        sim = _oracle_result(c)
        r = mixed[i]
        if c.kind == serving.RESULT_AMPLITUDE0:
            assert abs(complex(r["value_re"], r["value_im"]) - sim.vec[0]) < 1e-12
        elif c.kind == serving.RESULT_SAMPLE:
            assert r["sample"] == sim.sample_index(c.rnd)
        else:
            op = []
            for x, y, z, coef in c.pauli:
                term = []
                for q in range(c.n):
                    b = 1 << q
                    if y & b:
                        term.append((q, "Y"))
                    elif x & b:
                        term.append((q, "X"))
                    elif z & b:
                        term.append((q, "Z"))
                op.append((term, coef))
            assert abs(r["value_re"] - sim.get_expectation_value(op, list(range(c.n)))) < 1e-11
