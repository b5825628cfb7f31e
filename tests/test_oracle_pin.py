"""Pins the CPU oracle to the reference engine: every golden fixture under
tests/golden/ was produced by the unmodified reference modules
(tests/golden/make_golden.py); the oracle must reproduce them. Where the
reference oracle build (oracle/_ref) is present, it is also compared live."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from hiqsimulator_gb300 import circuits
from oracle.engine import OracleSimulator
from oracle.lib import greedy_schedule as oracle_schedule

TOL = 1e-12


def _stream(gates, n, mode, K):
    if mode == "off":
        return circuits.fusion_off_stream(gates)
    return circuits.greedy_stream(gates, list(range(n)), K, scheduler=oracle_schedule)


def _run_oracle(n, cmds, seed, K):
    sim = OracleSimulator(seed, 24, K)
    sim.allocate_qureg(list(range(n)), 0)
    circuits.replay(sim, cmds)
    sim.run()
    return sim


CASES = [("c0_n12_off", 12, 20, "off", 4, 101), ("c0_n12_greedy4", 12, 20, "greedy", 4, 102),
         ("c0_n14_greedy5", 14, 10, "greedy", 5, 103), ("qft10_greedy5", 10, 0, "qft", 5, 104)]


@pytest.mark.parametrize("name,n,layers,mode,K,seed", CASES)
def test_oracle_matches_reference_states(name, n, layers, mode, K, seed):
    g = np.load(os.path.join(GOLDEN, "ref_states.npz"))
    if mode == "qft":
        gates = circuits.qft(list(range(n))) + circuits.random_layers(seed, list(range(n)), 2)
        cmds = _stream(gates, n, "greedy", K)
    else:
        gates = circuits.random_layers(seed, list(range(n)), layers)
        cmds = _stream(gates, n, mode, K)
    sim = _run_oracle(n, cmds, seed, K)
    assert np.max(np.abs(sim.vec - g[name + "_state"])) < TOL
    p1 = [sim.get_probability([True], [q]) for q in range(n)]
    assert np.max(np.abs(np.array(p1) - g[name + "_p1"])) < TOL
    meas = sim.measure_qubits(list(range(n)))
    assert [int(b) for b in meas] == list(g[name + "_meas"])
    assert np.max(np.abs(sim.vec - g[name + "_after_meas"])) < TOL


@pytest.mark.parametrize("mode", ["off", "greedy"])
def test_oracle_matches_reference_random_layers_20q(mode):
    ref = json.load(open(os.path.join(GOLDEN, "ref_layers_20q.json")))[mode]
    n = 20
    gates = circuits.random_circuit_20q(seed=1234, n=n, layers=20)
    sim = _run_oracle(n, _stream(gates, n, mode, 4), 1234, 4)
    p1 = [sim.get_probability([True], [q]) for q in range(n)]
    assert np.max(np.abs(np.array(p1) - ref["p1"])) < TOL
    head = np.array([complex(*v) for v in ref["head"]])
    assert np.max(np.abs(sim.vec[:64] - head)) < TOL
    pick = np.array([complex(*v) for v in ref["pick"]])
    assert np.max(np.abs(sim.vec[ref["pick_idx"]] - pick)) < TOL
    assert abs(np.sum(np.abs(sim.vec) ** 2) - ref["norm"]) < TOL
    assert [int(b) for b in sim.measure_qubits(list(range(n)))] == ref["meas"]


def test_oracle_scheduler_matches_reference():
    sch = json.load(open(os.path.join(GOLDEN, "ref_sched.json")))
    for name, c in sch.items():
        if name == "qft10_k5":
            gates = circuits.qft(list(range(10))) + circuits.random_layers(3, list(range(10)), 2)
            n, K = 10, 5
        else:
            gates = circuits.random_layers(c["seed"], list(range(c["n"])), c["layers"])
            n, K = c["n"], c["K"]
        got = oracle_schedule([list(g.ids) for g in gates], [list(g.ctrls) for g in gates], list(range(n)), K)
        assert got == c["clusters"], name


def test_oracle_rng_matches_reference():
    """Measurement outcomes on |+>^16 expose the draws of std::mt19937(seed) +
    uniform_real_distribution<double>."""
    ref = json.load(open(os.path.join(GOLDEN, "ref_rng.json")))
    for seed, outs in ref.items():
        sim = OracleSimulator(int(seed), 24, 4)
        n = 16
        sim.allocate_qureg(list(range(n)), 0)
        got = []
        for _ in range(16):
            for q in range(n):
                sim.apply_controlled_gate(circuits.H.tolist(), [q], [])
                sim.run()
            bits = sim.measure_qubits(list(range(n)))
            got.append(sum(int(b) << q for q, b in enumerate(bits)))
            for q in range(n):
                if bits[q]:
                    sim.apply_controlled_gate(circuits.X.tolist(), [q], [])
                    sim.run()
        assert got == outs, seed


def test_oracle_sample_many_matches_single_draws():
    """One block CDF for many draws gives the index and margin of a
    separate sample_index per draw (the draws that decide measure_qubits),
    including draws on block boundaries and a draw above the total."""
    rng = np.random.default_rng(8)
    for n in (6, 17):
        sim = OracleSimulator(3, 24, 4)
        sim.allocate_qureg(list(range(n)), 0)
        v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        v[rng.random(1 << n) < 0.2] = 0
        sim.vec = v / np.linalg.norm(v)
        cdf = np.cumsum(np.abs(sim.vec) ** 2)
        rnds = np.concatenate([rng.random(200), cdf[[0, 5, len(cdf) // 3]], [1.5]])
        idx, mar = sim.sample_many(rnds)
        for r, i, m in zip(rnds, idx, mar):
            assert sim.sample_index(float(r)) == i
            if i >= 0:
                assert sim.last_margin == m


def test_oracle_errors_match_reference():
    ref = json.load(open(os.path.join(GOLDEN, "ref_errors.json")))
    sim = OracleSimulator(1, 20, 4)
    sim.allocate_qureg([0, 1], 0)
    sim.apply_controlled_gate(circuits.H.tolist(), [0], [])
    sim.run()
    checks = {
        "amp_short": lambda: sim.get_amplitude([True], [0]),
        "amp_not_perm": lambda: sim.get_amplitude([True, False], [0, 0]),
        "prob_unknown": lambda: sim.get_probability([True], [7]),
        "prob_len": lambda: sim.get_probability([True, False], [0]),
        "dealloc_entangled": lambda: sim.deallocate_qubit(0),
        "collapse_zero": lambda: sim.collapse_wavefunction([1], [True]),
        "collapse_len": lambda: sim.collapse_wavefunction([1], [True, False]),
        "dealloc_unknown": lambda: sim.deallocate_qubit(9),
        "measure_unknown": lambda: sim.measure_qubits([5]),
    }
    for key, f in checks.items():
        with pytest.raises(RuntimeError) as e:
            f()
        assert str(e.value) == ref[key][1], key


def test_oracle_matches_live_reference_when_present():
    ref_dir = os.path.join(ROOT, "oracle", "_ref")
    if not any(f.startswith("_cppsim_mpi") for f in (os.listdir(ref_dir) if os.path.isdir(ref_dir) else [])):
        pytest.skip("reference oracle build (oracle/_ref) not present on this machine")
    import importlib.util
    import glob
    path = glob.glob(os.path.join(ref_dir, "_cppsim_mpi*.so"))[0]
    spec = importlib.util.spec_from_file_location("_cppsim_mpi", path)
    REF = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(REF)
    n = 11
    gates = circuits.qft(list(range(n))) + circuits.random_layers(9, list(range(n)), 3)
    cmds = _stream(gates, n, "greedy", 5)
    r = REF.SimulatorMPI(3, 20, 5)
    r.allocate_qureg(list(range(n)), 0)
    circuits.replay(r, cmds)
    r.run()
    o = _run_oracle(n, cmds, 3, 5)
    assert np.max(np.abs(np.array(r.cheat_local()[1]) - o.vec)) < TOL
    assert r.measure_qubits(list(range(n))) == o.measure_qubits(list(range(n)))
    assert abs(r.entropy() - o.entropy()) < 1e-10


RELEASE_CHILD = r"""
import glob, importlib.util, sys
import numpy as np
sys.path.insert(0, {root!r})
from hiqsimulator_gb300 import circuits
path = glob.glob({rel!r} + "/_cppsim_mpi*.so")[0]
spec = importlib.util.spec_from_file_location("_cppsim_mpi", path)
REF = importlib.util.module_from_spec(spec)
spec.loader.exec_module(REF)
n = 12
qs = list(range(n))
gates = circuits.qft(qs) + circuits.random_layers(13, qs, 4)
r = REF.SimulatorMPI(3, 20, 4)
r.allocate_qureg(qs, 0)
circuits.replay(r, circuits.greedy_stream(gates, qs, 4))
r.run()
np.save({out!r}, np.array(r.cheat_local()[1], dtype=complex))
"""


def test_oracle_matches_release_build_when_present(tmp_path):
    """The reference built with its release flags (-O3 -ffast-math, by
    REF_VARIANT=release oracle/build_ref.sh) gives the oracle's state too; it
    loads in a child process (two builds of one pybind11 module cannot share
    a process)."""
    import glob
    import subprocess
    import sys
    rel = os.path.join(ROOT, "oracle", "_ref", "release")
    if not glob.glob(os.path.join(rel, "_cppsim_mpi*.so")):
        pytest.skip("release build of the reference (oracle/_ref/release) not present on this machine")
    out = str(tmp_path / "state.npy")
    r = subprocess.run([sys.executable, "-c", RELEASE_CHILD.format(root=ROOT, rel=rel, out=out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    n = 12
    qs = list(range(n))
    gates = circuits.qft(qs) + circuits.random_layers(13, qs, 4)
    o = _run_oracle(n, circuits.greedy_stream(gates, qs, 4), 3, 4)
    assert np.max(np.abs(np.load(out) - o.vec)) < TOL


def test_oracle_matches_reference_perm_and_fill():
    """The oracle's set_qubits_perm relabelling, qubit-id getters and
    allocate_qureg fill value against ref_perm_init.json."""
    fx = json.load(open(os.path.join(GOLDEN, "ref_perm_init.json")))
    p = fx["perm"]
    n = p["n"]
    gates = circuits.random_layers(p["seed"], list(range(n)), p["layers"])
    sim = OracleSimulator(p["seed"], 24, p["cluster"])
    sim.allocate_qureg(p["alloc_ids"], 0)
    circuits.replay(sim, _stream(gates, n, "greedy", p["cluster"]))
    sim.run()
    assert list(sim.get_qubits_ids()) == p["before"]["ids"]
    sim.set_qubits_perm(p["perm"])
    assert list(sim.get_qubits_ids()) == p["after"]["ids"]
    id2pos, vec = sim.cheat_local()
    assert {str(k): int(v) for k, v in id2pos.items()} == p["id2pos"]
    assert np.max(np.abs(np.asarray(vec) - np.array([complex(*v) for v in p["state"]]))) < TOL
    for bits, want in zip(p["amp_bits"], p["amps"]):
        assert abs(sim.get_amplitude(bits, p["amp_ids"]) - complex(*want)) < TOL
    for f in fx["fill"]:
        nq = f["n"]
        sim = OracleSimulator(7, 24, f["cluster"])
        sim.allocate_qureg(list(range(nq)), complex(*f["init"]))
        assert np.max(np.abs(sim.vec - np.array([complex(*v) for v in f["filled"]]))) == 0.0
        g = circuits.random_layers(f["layers_seed"], list(range(nq)), f["layers"])
        circuits.replay(sim, _stream(g, nq, "greedy", f["cluster"]))
        sim.run()
        assert np.max(np.abs(sim.vec - np.array([complex(*v) for v in f["after_gates"]]))) < TOL
