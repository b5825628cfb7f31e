"""Generates the golden fixtures in this directory from the reference engine.

Runs the unmodified reference modules built by oracle/build_ref.sh
(oracle/_ref/_cppsim_mpi, oracle/_ref/_sched_cpp) on seeded circuits from
hiqsimulator_gb300.circuits and stores what they return:

  ref_states.npz     final states, P(q=1) and measurement outcomes of small
                     circuits (fusion off and greedy fusion), cheat_local order
  ref_layers_20q.json   20-qubit random-layer circuit summaries (fusion off / greedy k<=4):
                     P(q=1) for all 20 qubits, the first 64 amplitudes, the
                     amplitudes at 64 seeded indices, sum |a|^2
  ref_sched.json     greedy cluster lists for several circuits
  ref_rng.json       first uniform draws of std::mt19937(seed) as used by
                     MeasureQubits (one draw per call, read back via outcomes)
  ref_errors.json    error messages of the reference for invalid calls
  ref_perm_init.json qubit-id getters before and after set_qubits_perm
                     relabelling, with the queries that follow it; states
                     after allocate_qureg with a nonzero fill value

Usage (needs the reference sources and a built oracle/_ref):
    bash oracle/build_ref.sh && python tests/golden/make_golden.py [--only perm_init]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))

import _cppsim_mpi as REF  # noqa: E402
import _sched_cpp  # noqa: E402

from hiqsimulator_gb300 import circuits  # noqa: E402


def ref_schedule(gates, ctrls, locals_, K):
    idx = list(range(len(gates)))
    out = []
    while True:
        g = [list(gates[i]) for i in idx]
        c = [list(ctrls[i]) for i in idx]
        avail = _sched_cpp.ClusterScheduler(g, c, [False] * len(g), list(locals_), [], K).ScheduleCluster()
        if not avail:
            break
        out.append([idx[i] for i in avail])
        for i in sorted(avail, reverse=True):
            del idx[i]
    return out


def run_ref(n, cmds, seed, K):
    sim = REF.SimulatorMPI(seed, 24, K)
    sim.allocate_qureg(list(range(n)), 0)
    circuits.replay(sim, cmds)
    sim.run()
    return sim


def stream(gates, n, mode, K):
    if mode == "off":
        return circuits.fusion_off_stream(gates)
    G = [list(g.ids) for g in gates]
    C = [list(g.ctrls) for g in gates]
    return circuits.greedy_stream(gates, list(range(n)), K, clusters=ref_schedule(G, C, list(range(n)), K))


def cplx_list(vec):
    return [[float(v.real), float(v.imag)] for v in vec]


def perm_init_fixture():
    """set_qubits_perm relabels positions without moving data
    (SimulatorMPI.cpp:661-667); the getters return locals_ ++ globals_
    (:652-679). allocate_qureg(ids, init) fills every amplitude with init
    (:218-251)."""
    out = {}
    n = 6
    gates = circuits.random_layers(55, list(range(n)), 3)
    cmds = stream(gates, n, "greedy", 4)
    sim = REF.SimulatorMPI(55, 24, 4)
    ids = [3, 0, 5, 1, 4, 2]
    sim.allocate_qureg(ids, 0)
    circuits.replay(sim, cmds)
    sim.run()
    before = {"ids": list(sim.get_qubits_ids()), "local": list(sim.get_local_qubits_ids()),
              "global": list(sim.get_global_qubits_ids())}
    perm = [2, 4, 0, 5, 1, 3]
    sim.set_qubits_perm(perm)
    id2pos, vec = sim.cheat_local()
    bits = [[bool((b >> j) & 1) for j in range(n)] for b in (0, 5, 22, 63)]
    out["perm"] = {"n": n, "alloc_ids": ids, "seed": 55, "layers": 3, "cluster": 4, "before": before,
                   "perm": perm,
                   "after": {"ids": list(sim.get_qubits_ids()), "local": list(sim.get_local_qubits_ids()),
                             "global": list(sim.get_global_qubits_ids())},
                   "id2pos": {str(k): int(v) for k, v in id2pos.items()},
                   "state": cplx_list(vec),
                   "p1": [sim.get_probability([True], [q]) for q in range(n)],
                   "amp_bits": bits,
                   "amp_ids": list(range(n)),
                   "amps": cplx_list([sim.get_amplitude(b, list(range(n))) for b in bits]),
                   "p_pair": sim.get_probability([True, False], [4, 1])}
    fills = []
    for init, nq in ((0.25, 4), (complex(0.25, -0.25), 3), (complex(0.0, 0.5), 2)):  # normalised states
        sim = REF.SimulatorMPI(7, 24, 4)
        sim.allocate_qureg(list(range(nq)), init)
        filled = cplx_list(sim.cheat_local()[1])
        g = circuits.random_layers(8, list(range(nq)), 2)
        circuits.replay(sim, stream(g, nq, "greedy", 4))
        sim.run()
        fills.append({"init": [init.real, init.imag] if isinstance(init, complex) else [init, 0.0], "n": nq,
                      "filled": filled, "layers_seed": 8, "layers": 2, "cluster": 4,
                      "after_gates": cplx_list(sim.cheat_local()[1]),
                      "p1": [sim.get_probability([True], [q]) for q in range(nq)]})
    out["fill"] = fills
    with open(os.path.join(HERE, "ref_perm_init.json"), "w") as f:
        json.dump(out, f)


def main():
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "perm_init":
        perm_init_fixture()
        return
    perm_init_fixture()
    small = {}
    cases = [("c0_n12_off", 12, 20, "off", 4, 101), ("c0_n12_greedy4", 12, 20, "greedy", 4, 102),
             ("c0_n14_greedy5", 14, 10, "greedy", 5, 103), ("qft10_greedy5", 10, 0, "qft", 5, 104)]
    for name, n, layers, mode, K, seed in cases:
        if mode == "qft":
            gates = circuits.qft(list(range(n))) + circuits.random_layers(seed, list(range(n)), 2)
            cmds = stream(gates, n, "greedy", K)
        else:
            gates = circuits.random_layers(seed, list(range(n)), layers)
            cmds = stream(gates, n, mode, K)
        sim = run_ref(n, cmds, seed, K)
        id2pos, vec = sim.cheat_local()
        small[name + "_state"] = np.array(vec, dtype=np.complex128)
        small[name + "_p1"] = np.array([sim.get_probability([True], [q]) for q in range(n)])
        small[name + "_meas"] = np.array([int(b) for b in sim.measure_qubits(list(range(n)))], dtype=np.int8)
        small[name + "_after_meas"] = np.array(sim.cheat_local()[1], dtype=np.complex128)
    np.savez_compressed(os.path.join(HERE, "ref_states.npz"), **small)

    # 20-qubit random-layer circuit summaries
    summ = {}
    n = 20
    gates = circuits.random_circuit_20q(seed=1234, n=n, layers=20)
    pick = circuits.rng_for(77).choice(1 << n, size=64, replace=False)
    for mode in ("off", "greedy"):
        cmds = stream(gates, n, mode, 4)
        sim = run_ref(n, cmds, 1234, 4)
        vec = np.array(sim.cheat_local()[1], dtype=np.complex128)
        summ[mode] = {
            "p1": [sim.get_probability([True], [q]) for q in range(n)],
            "head": [[v.real, v.imag] for v in vec[:64]],
            "pick_idx": [int(i) for i in pick],
            "pick": [[vec[i].real, vec[i].imag] for i in pick],
            "norm": float(np.sum(np.abs(vec) ** 2)),
            "meas": [int(b) for b in sim.measure_qubits(list(range(n)))],
        }
    with open(os.path.join(HERE, "ref_layers_20q.json"), "w") as f:
        json.dump(summ, f)

    # schedules
    sch = {}
    for name, n, layers, K, seed in [("n8_k3", 8, 4, 3, 1), ("n12_k4", 12, 6, 4, 2), ("n20_k4", 20, 3, 4, 3),
                                     ("n16_k5", 16, 4, 5, 5)]:
        gates = circuits.random_layers(seed, list(range(n)), layers)
        sch[name] = {"n": n, "layers": layers, "K": K, "seed": seed,
                     "clusters": ref_schedule([list(g.ids) for g in gates], [list(g.ctrls) for g in gates],
                                              list(range(n)), K)}
    gates = circuits.qft(list(range(10))) + circuits.random_layers(3, list(range(10)), 2)
    sch["qft10_k5"] = {"clusters": ref_schedule([list(g.ids) for g in gates], [list(g.ctrls) for g in gates],
                                                list(range(10)), 5)}
    with open(os.path.join(HERE, "ref_sched.json"), "w") as f:
        json.dump(sch, f)

    # RNG: with the state |+>^n, measuring all qubits returns the bits of
    # floor(rnd * 2^n) (up to the block CDF boundaries), so the draws show up
    # as outcomes; store outcomes of 16 successive measurements for 3 seeds.
    rng = {}
    H = circuits.H
    for seed in (0, 42, 4294967297):
        sim = REF.SimulatorMPI(seed, 24, 4)
        n = 16
        sim.allocate_qureg(list(range(n)), 0)
        outs = []
        for _ in range(16):
            for q in range(n):
                sim.apply_controlled_gate(H.tolist(), [q], [])
                sim.run()
            bits = sim.measure_qubits(list(range(n)))
            outs.append(sum(int(b) << q for q, b in enumerate(bits)))
            # return to |0...0>
            for q in range(n):
                if bits[q]:
                    sim.apply_controlled_gate(circuits.X.tolist(), [q], [])
                    sim.run()
        rng[str(seed)] = outs
    with open(os.path.join(HERE, "ref_rng.json"), "w") as f:
        json.dump(rng, f)

    # error messages
    errs = {}
    sim = REF.SimulatorMPI(1, 20, 4)
    sim.allocate_qureg([0, 1], 0)
    sim.apply_controlled_gate(H.tolist(), [0], [])
    sim.run()

    def grab(key, f):
        try:
            f()
            errs[key] = None
        except Exception as e:  # noqa: BLE001
            errs[key] = [type(e).__name__, str(e)]

    grab("amp_short", lambda: sim.get_amplitude([True], [0]))
    grab("amp_not_perm", lambda: sim.get_amplitude([True, False], [0, 0]))
    grab("prob_unknown", lambda: sim.get_probability([True], [7]))
    grab("prob_len", lambda: sim.get_probability([True, False], [0]))
    grab("dealloc_entangled", lambda: sim.deallocate_qubit(0))
    grab("collapse_zero", lambda: sim.collapse_wavefunction([1], [True]))
    grab("collapse_len", lambda: sim.collapse_wavefunction([1], [True, False]))
    grab("emulate_math", lambda: sim.emulate_math(lambda x: x, [[0]], []))
    grab("swap_pairs", lambda: sim.swap_qubits([0, 1]))
    grab("dealloc_unknown", lambda: sim.deallocate_qubit(9))
    grab("measure_unknown", lambda: sim.measure_qubits([5]))
    sim2 = REF.SimulatorMPI(1, 3, 2)
    sim2.allocate_qureg([0, 1, 2], 0)
    grab("alloc_too_many", lambda: sim2.allocate_qubit(3))
    grab("qureg_init_twice", lambda: sim2.allocate_qureg([5], 0.5))
    sim3 = REF.SimulatorMPI(1, 20, 4)
    sim3.allocate_qureg(list(range(6)), 0)
    sim3.apply_controlled_gate(np.eye(64).tolist(), list(range(6)), [])
    grab("run_too_big", lambda: sim3.run())
    with open(os.path.join(HERE, "ref_errors.json"), "w") as f:
        json.dump(errs, f, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
