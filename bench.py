#!/usr/bin/env python
"""Benchmark of the fused-pass hot path on the workload the headline metric
is quoted on: 30-qubit complex128 state (16 GiB), QFT on all 30 qubits
followed by 10 seeded random layers (Haar U(2) on every qubit, CNOTs on a
random perfect matching, one controlled phase), greedy fusion k <= 5.

A step applies the whole fused circuit to the resident state and then forces
one qubit permutation (the qubits at the top 5 positions move to positions
0-4: one in-HBM bit-permutation sweep, standing in for the reference's
global/local qubit swap). The metric is the reference-equivalent state
bandwidth: every fused gate of the greedy schedule is one sweep of the
reference engine (kernelK, 2 * 2^n * 16 bytes, halved per control) and the
permutation one more, so value = sum of those bytes / step time. Inputs are
larger than L2 (16 GiB state), so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own CPU algorithm (the oracle port of
the reference kernels, oracle/, with OpenMP on every host core) on a bounded
sample of the same workload: the first fused gates of the schedule on the
30-qubit state.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = 30  # overridden by --qubits for profiling runs on smaller states
CLUSTER = 5
SEED = 4321
METRIC = "30q c128 fused-pass state bandwidth (QFT30 + 10 random layers, greedy fusion k<=5)"
UNIT = "GB/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo", init_method="env://")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v):
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


def workload():
    from hiqsimulator_gb300 import circuits
    gates = circuits.qft_random_layers(seed=SEED, n=N_QUBITS, layers=10)
    t0 = time.time()
    clusters = circuits.greedy_clusters(gates, list(range(N_QUBITS)), CLUSTER)
    log("schedule: %d gates -> %d fused gates in %.1fs" % (len(gates), len(clusters), time.time() - t0))
    cmds = circuits.greedy_stream(gates, list(range(N_QUBITS)), CLUSTER, clusters=clusters)
    return gates, clusters, cmds


def cluster_bytes(gates, clusters, n=None, elem=16):
    """Reference-equivalent bytes: one read + one write of the state per fused
    gate; a lone controlled gate too large to fuse touches 2^-c of it."""
    n = N_QUBITS if n is None else n
    total = 0
    for cl in clusters:
        c = 0
        if len(cl) == 1:
            g = gates[cl[0]]
            if len(g.ids) + len(g.ctrls) > CLUSTER:
                c = len(g.ctrls)
        total += 2 * (1 << (n - c)) * elem
    return total


def cluster_flops(gates, clusters, n=None):
    """Reference FP64 flops of the fused gates: a dense k-qubit fused gate is
    8 * 2^k real flops per amplitude it acts on (4 multiplies + 4 adds per
    complex multiply-add), a diagonal one 6 (SimulatorMPI.cpp:441-541). The
    fused gate acts on 2^(n - c) amplitudes, c the controls every gate of the
    cluster shares; the other controls fold into the fused matrix
    (fusion_mpi.hpp:190-226) and count as targets."""
    n = N_QUBITS if n is None else n
    total = 0
    for cl in clusters:
        common = set(gates[cl[0]].ctrls)
        for i in cl[1:]:
            common &= set(gates[i].ctrls)
        qs, diag = set(), True
        for i in cl:
            g = gates[i]
            qs |= set(g.ids) | (set(g.ctrls) - common)
            m = np.asarray(g.matrix)
            diag = diag and not np.any(m - np.diag(np.diag(m)))
        total += (6 if diag else 8 << len(qs)) << (n - len(common))
    return total


# GB300's FP64 rate, measured with a DFMA loop: 0.5 T DFMA/s = 1.0 TFLOP/s
# (nominal 1.25 TFLOP/s).
FP64_PEAK_TFLOPS = 1.0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel):
    """DRAM bytes per launch of a kernel from the committed ncu summaries
    (profiles/kernel_traffic.json: bytes per amplitude of one launch,
    measured on a smaller state), scaled to the state's amplitudes."""
    p = os.path.join(ROOT, "profiles", "kernel_traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p)).get(kernel)
    if not d:
        return None
    return float(d["bytes_per_amplitude"]) * (1 << N_QUBITS)


def cpu_sample_sim():
    """The oracle port's state for the CPU legs: N_QUBITS qubits, allocated
    once and reused by every sample (a sweep's time does not depend on the
    amplitudes)."""
    from oracle.engine import OracleSimulator
    sim = OracleSimulator(SEED, N_QUBITS, CLUSTER)
    sim.allocate_qureg(list(range(N_QUBITS)), 0)
    return sim


def cpu_sample(sim, gates, clusters, n_dense=4, n_diag=3, budget_s=20.0):
    """The oracle port of the reference engine on the host cores: fused gates
    of the schedule in its own mix of dense and diagonal clusters (64 dense :
    48 diagonal per step, so 4 : 3), the first of each kind, one run() each;
    only the state sweeps are timed (the host fusion of the queued gates is
    not). Returns (GB/s, threads, description)."""
    picked, nd, ng = [], 0, 0
    for cl in clusters:
        diag = all(not np.any(np.asarray(gates[i].matrix) - np.diag(np.diag(gates[i].matrix))) for i in cl)
        if diag and ng < n_diag:
            picked.append(cl)
            ng += 1
        elif not diag and nd < n_dense:
            picked.append(cl)
            nd += 1
        if nd >= n_dense and ng >= n_diag:
            break
    done, dense_done, t_total = 0, 0, 0.0
    for cl in picked:
        for i in cl:
            g = gates[i]
            sim.apply_controlled_gate(g.matrix.tolist(), list(g.ids), list(g.ctrls))
        t_total += sim.run_timed()
        done += 1
        dense_done += any(np.any(np.asarray(gates[i].matrix) - np.diag(np.diag(gates[i].matrix))) for i in cl)
        if t_total > budget_s:
            break
    byts = done * 2 * (1 << N_QUBITS) * 16
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return byts / t_total / 1e9, threads, (
        "%d fused gates of the schedule (%d dense, %d diagonal: its 4:3 mix) on the %d-qubit state, sweeps "
        "only (%.1f s)" % (done, dense_done, done - dense_done, N_QUBITS, t_total))


def host_info():
    """The host the CPU legs ran on: core count, architecture and CPU model
    (lscpu's "Model name", else /proc/cpuinfo's)."""
    import platform
    info = {"nproc": os.cpu_count(), "machine": platform.machine(), "cpu_model": None}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                info["cpu_model"] = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if info["cpu_model"] is None:
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.lower().startswith("model name"):
                        info["cpu_model"] = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return info


def force_permutation(sim):
    """Move the qubits at the top 5 positions to positions 0-4 (one sweep)."""
    top = sim.get_qubits_ids()[-5:]
    sim.move_qubits(top, list(range(5)))


def capacity_report():
    """The largest states one GPU holds: 33 qubits complex128 and 34 qubits
    complex64 (128 GiB each). Random layers with CNOT targets biased to the
    top 8 qubits + 4 Grover iterations (multi-controlled Z over all qubits),
    greedy fusion k <= 5 (the multi-controlled Z gates stay single-gate
    clusters); timed forward, then the inverse stream must return |0...0>."""
    import hiqsimulator_gb300 as hqs
    from hiqsimulator_gb300 import circuits
    out = {}
    for prec, n in (("c128", 33), ("c64", 34)):
        gates, _ = circuits.capacity_circuit(seed=99, n=n)
        qs = list(range(n))
        clusters = circuits.greedy_clusters(gates, qs, 5)
        sim = hqs.SimulatorMPI(99, n, 5, prec)
        sim.allocate_qureg(qs, 0)
        sim.synchronize()
        sim.enable_pass_timing(True)
        sim.timer_start()
        circuits.replay(sim, circuits.greedy_stream(gates, qs, 5, clusters=clusters))
        ms = sim.timer_stop()
        pt = sim.pass_timing()
        sim.enable_pass_timing(False)
        norm = sim.get_probability([], [])
        circuits.replay(sim, circuits.inverse_stream(gates, clusters))
        p0 = abs(sim.get_amplitude([False] * n, qs)) ** 2
        out[prec] = {"qubits": n, "state_bytes": (16 if prec == "c128" else 8) << n, "gates": len(gates),
                     "fused_gates": len(clusters),
                     "ms": ms, "passes": pt["launches"], "pass_bytes": pt["bytes"],
                     "pass_GBs": pt["bytes"] / (pt["ms"] / 1e3) / 1e9 if pt["ms"] > 0 else None,
                     "norm_after_circuit": norm, "round_trip_p0": p0}
        log("capacity %s %dq: %d gates in %.0f ms (%d passes, %.0f GB/s in passes), norm-1 %.1e, "
            "1-p0 after inverse %.1e" % (prec, n, len(gates), ms, pt["launches"], out[prec]["pass_GBs"] or 0,
                                         norm - 1, 1 - p0))
        del sim
    return out


def table_report(cmds30, ref_bytes30):
    """Rows of the reference-against-GPU table. 20 qubits (random circuit,
    20 layers; fusion off and greedy k <= 4): the oracle port of the
    reference's algorithm on every host core, the GPU with one launch per
    fused gate (the reference's one sweep per run(), no pass fusion), and the
    GPU engine as shipped, with the max-abs error against the oracle.
    30 qubits (the benchmark workload): the GPU with one launch per fused gate."""
    import hiqsimulator_gb300 as hqs
    from hiqsimulator_gb300 import circuits
    from oracle.engine import OracleSimulator
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    out = {"host_threads": int(os.environ["OMP_NUM_THREADS"])}
    n = 20
    qs = list(range(n))
    gates = circuits.random_circuit_20q(seed=1234, n=n, layers=20)
    for mode, cmds in (("fusion_off", circuits.fusion_off_stream(gates)),
                       ("greedy_k4", circuits.greedy_stream(gates, qs, 4))):
        row = {}
        ref = OracleSimulator(1234, n, 4)
        ref.allocate_qureg(qs, 0)
        t0 = time.perf_counter()
        circuits.replay(ref, cmds)
        ref.run()
        row["cpu_oracle_ms"] = (time.perf_counter() - t0) * 1e3
        for label, limits in (("gpu_one_fused_gate_per_launch_ms", dict(max_ops=1, defer=1)), ("gpu_ms", {})):
            sim = hqs.SimulatorMPI(1234, n, 4, "c128")
            if limits:
                sim.set_pass_limits(**limits)
            sim.allocate_qureg(qs, 0)
            circuits.replay(sim, cmds)  # warm-up
            sim.synchronize()
            del sim
            sim = hqs.SimulatorMPI(1234, n, 4, "c128")
            if limits:
                sim.set_pass_limits(**limits)
            sim.allocate_qureg(qs, 0)
            sim.synchronize()
            sim.timer_start()
            circuits.replay(sim, cmds)
            sim.run()
            row[label] = sim.timer_stop()
            if not limits:
                _, vec = sim.cheat_local_numpy()
                row["max_abs_error_vs_oracle"] = float(np.max(np.abs(vec - ref.vec)))
            del sim
        out["random_20q_" + mode] = row
        log("table 20q %s: cpu %.0f ms, gpu one fused gate per launch %.1f ms, gpu %.1f ms, err %.1e" % (
            mode, row["cpu_oracle_ms"], row["gpu_one_fused_gate_per_launch_ms"], row["gpu_ms"], row["max_abs_error_vs_oracle"]))
    sim = hqs.SimulatorMPI(SEED, N_QUBITS, CLUSTER, "c128")
    sim.set_pass_limits(max_ops=1, defer=1)
    sim.allocate_qureg(list(range(N_QUBITS)), 0)
    sim.synchronize()
    sim.timer_start()
    circuits.replay(sim, cmds30)
    sim.run()
    ms = sim.timer_stop()
    del sim
    out["headline_one_fused_gate_per_launch"] = {"ms": ms, "GBs": ref_bytes30 / (ms / 1e3) / 1e9}
    log("table %dq one fused gate per launch: %.0f ms, %.1f GB/s" % (N_QUBITS, ms, ref_bytes30 / (ms / 1e3) / 1e9))
    return out


def serving_report(args):
    """Serving of many small circuits: Poisson arrivals of circuits with
    n ~ U{10..22}, depth ~ U{10..60} random layers; batched continuous
    serving in each precision, and (complex128, first rate) against the same
    server running one circuit per launch. The first rate saturates the
    server (throughput); the others are below its service rate, so their
    p50/p99 are service latency rather than queueing."""
    from hiqsimulator_gb300 import serving
    out = {"circuits": args.serve, "budget_bytes": int(150e9),
           "workload": "n~U{10..22}, depth~U{10..60} random layers; 30% sample, 20% 8-term <H>, 50% <0|psi>"}
    circuits = serving.serving_workload(2024, args.serve)
    for prec, arith, key in (("c128", "tc", "c128"), ("c64", "tc", "c64_tc"), ("c64", "f32", "c64_f32"),
                             ("c64", "tf32", "c64_tf32")):
        rep = {}
        for rate in (args.serve_rates if prec == "c128" else args.serve_rates64):
            arr = serving.poisson_arrivals(2024, len(circuits), rate)
            res_b, st_b = serving.serve(circuits, arr, precision=prec, arith=arith, budget_bytes=150e9,
                                        max_active=args.serve_slots)
            entry = {"batched": st_b}
            if prec == "c128" and rate == args.serve_rates[0]:
                res_p, st_p = serving.serve(circuits, arr, precision=prec, budget_bytes=150e9, max_active=1)
                same = all((res_b[i]["value_re"], res_b[i]["value_im"], res_b[i]["sample"]) ==
                           (res_p[i]["value_re"], res_p[i]["value_im"], res_p[i]["sample"]) for i in res_b)
                entry["one_circuit_per_launch"] = st_p
                entry["results_identical"] = bool(same)
                entry["speedup_circuits_per_s"] = st_b["circuits_per_s"] / st_p["circuits_per_s"]
            rep["rate_%g_per_s" % rate] = entry
            log("serving %s rate %g: %.0f circuits/s p50 %.1f ms p99 %.1f ms" % (
                key, rate, st_b["circuits_per_s"], st_b["p50_ms"], st_b["p99_ms"]))
        out[key] = rep
    return out


def precision_report(qubits=28, layers=40, cluster=5):
    """Precision workload: a brickwork of Haar U(4) on alternating pairs,
    greedy-fused into blocks of up to `cluster` qubits, run as complex128
    (tensor-core digit mode) and as complex64 in FP32, in two-digit
    tensor-core mode and in 3xTF32. Every state is compared with the
    oracle's FP64 state of the same circuit (the checker: oracle/, on the
    host cores): fidelity, normalized fidelity, norm and max amplitude
    error; device time of each mode (second replay) against complex128."""
    import hiqsimulator_gb300 as hqs
    from hiqsimulator_gb300 import circuits
    from oracle.engine import OracleSimulator
    qs = list(range(qubits))
    gates = circuits.brickwork(2024, qs, layers)
    cmds = circuits.greedy_stream(gates, qs, cluster)
    out = {"workload": "%dq brickwork, %d layers of Haar U(4), greedy fusion k<=%d" % (qubits, layers, cluster),
           "against": "oracle FP64 state of the same fused circuit"}
    states = {}
    modes = (("c128_tc", "c128", "tc"), ("c64_f32", "c64", "f32"), ("c64_tc", "c64", "tc"), ("c64_tf32", "c64", "tf32"))
    for key, prec, arith in modes:
        sim = hqs.SimulatorMPI(7, qubits, cluster, prec, arith)
        sim.set_pass_limits(defer=16)
        sim.allocate_qureg(qs, 0)
        sim.synchronize()
        times = []
        for rep in range(2):  # the state after the first replay is compared; the second is timed warm
            sim.timer_start()
            circuits.replay(sim, cmds)
            times.append(sim.timer_stop())
            if rep == 0:
                m, v = sim.cheat_local_numpy()
                ident = {q: q for q in qs}
                if dict(m) != ident:  # bring the state to the allocation order
                    v = np.ascontiguousarray(v.reshape((2,) * qubits).transpose(
                        relayout_axes(dict(m), ident, qubits))).reshape(-1)
                states[key] = v
        out[key + "_ms"] = min(times)
        del sim
    ref = OracleSimulator(7, qubits, cluster)
    ref.allocate_qureg(qs, 0)
    circuits.replay(ref, cmds)
    ref.run()
    a = ref.vec
    c128 = states.pop("c128_tc")
    out["c128_tc_max_abs_error"] = float(np.max(np.abs(c128 - a)))
    del c128
    for key, _, _ in modes[1:]:
        b = states.pop(key).astype(np.complex128)
        nb = float(np.vdot(b, b).real)
        ov = float(abs(np.vdot(a, b)) ** 2)
        ms = out.pop(key + "_ms")
        out[key] = {"ms": ms, "fidelity": ov, "fidelity_normalized": ov / nb, "norm": nb,
                    "max_abs_error": float(np.max(np.abs(a - b))), "speedup_over_c128": out["c128_tc_ms"] / ms}
        log("precision %s: fidelity %.3e below 1 (normalized %.3e), norm-1 %.2e, max err %.2e, %.0f ms vs c128 %.0f ms" % (
            key, 1 - ov, 1 - ov / nb, nb - 1, out[key]["max_abs_error"], out[key]["ms"], out["c128_tc_ms"]))
        del b
    log("precision c128_tc: max err vs oracle %.2e" % out["c128_tc_max_abs_error"])
    del ref, a
    return out


# ------------------------------------------------------------ parity legs
# The oracle (oracle/, the C restatement of the reference engine, OpenMP on
# the host cores) is the checker here: the product's states, expectation
# values and samples are compared with it on the configurations the metric
# is quoted on. Nothing measured above runs through it.

def relayout_axes(map_src, map_dst, n):
    """Axes that transpose a state stored in layout map_src (qubit id -> bit
    position), viewed as shape (2,)*n (axis k = bit n-1-k), into layout
    map_dst."""
    axes = [0] * n
    for q, pd in map_dst.items():
        axes[n - 1 - pd] = n - 1 - map_src[q]
    return axes


def max_abs_diff(a, map_a, b, map_b, n, chunk_axes=6):
    """max |a - b| over every amplitude; a in layout map_a, b in layout
    map_b, compared in 2^chunk_axes chunks of b's order."""
    A = a.reshape((2,) * n).transpose(relayout_axes(map_a, map_b, n))
    c = min(chunk_axes, n)
    B = b.reshape((1 << c, -1))
    worst = 0.0
    for k in range(1 << c):
        idx = tuple((k >> (c - 1 - t)) & 1 for t in range(c))
        blk = np.ascontiguousarray(A[idx]).reshape(-1)
        worst = max(worst, float(np.max(np.abs(blk - B[k]))))
    return worst


def remap_indices(idx, map_src, map_dst):
    """Basis indices in layout map_src rewritten for layout map_dst."""
    idx = np.asarray(idx, dtype=np.uint64)
    out = np.zeros_like(idx)
    for q, ps in map_src.items():
        out |= ((idx >> np.uint64(ps)) & np.uint64(1)) << np.uint64(map_dst[q])
    return out


def parity_headline(args, cmds, zz, shots):
    """The benchmark configuration at full size against the oracle: the
    fused circuit (QFT + 10 random layers, greedy k <= 5) on the GPU and on
    the oracle; every amplitude compared (max-abs <= 1e-12); the 1024 seeded
    full-register samples (same MT19937 draws; identical wherever the draw's
    distance to the deciding CDF boundary exceeds 1e-12, the others counted);
    the forced permutation (2^22 seeded amplitudes followed bit-exactly to
    their new positions, then every amplitude against the oracle again); the
    64 <Z_i Z_j> after it (<= 1e-11)."""
    import hiqsimulator_gb300 as hqs
    from hiqsimulator_gb300 import circuits
    from oracle.engine import OracleSimulator
    n = N_QUBITS
    ids = list(range(n))
    out = {"qubits": n, "tolerances": {"amplitudes_max_abs": 1e-12, "zz_abs": 1e-11, "sample_margin": 1e-12}}
    t0 = time.perf_counter()
    sim = hqs.SimulatorMPI(SEED, n, CLUSTER, "c128", args.arith)
    sim.set_pass_limits(defer=args.defer)
    sim.allocate_qureg(ids, 0)
    circuits.replay(sim, cmds)
    sim.run()
    sim.synchronize()
    ref = OracleSimulator(SEED, n, CLUSTER)
    ref.allocate_qureg(ids, 0)
    t1 = time.perf_counter()
    circuits.replay(ref, cmds)
    ref.run()
    out["oracle_seconds"] = time.perf_counter() - t1
    rmap, rvec = {q: p for p, q in enumerate(ref.get_qubits_ids())}, ref.vec
    gmap, gvec = sim.cheat_local_numpy()
    gmap = dict(gmap)
    out["layout_equal_before_permutation"] = gmap == rmap
    out["amplitudes_max_abs"] = max_abs_diff(gvec, gmap, rvec, rmap, n)
    # seeded amplitudes to follow through the permutation
    pick = np.random.default_rng(SEED).integers(0, 1 << n, size=1 << 22, dtype=np.uint64)
    before = gvec[pick.astype(np.int64)].copy()
    del gvec
    # samples: the same draws on both sides
    got = remap_indices(np.asarray(sim.sample(shots), dtype=np.uint64), gmap, rmap).astype(np.int64)
    rnds = np.array([ref.rng.uniform() for _ in range(shots)])
    want, margin = ref.sample_many(rnds)
    decided = margin > 1e-12
    out["samples"] = {"shots": shots, "compared": int(decided.sum()),
                      "mismatches": int(np.sum((got != want) & decided)),
                      "near_ties": int((~decided).sum()), "near_tie_mismatches": int(np.sum((got != want) & ~decided)),
                      "distinct": int(len(np.unique(got))), "min_margin": float(margin.min())}
    # the forced permutation
    force_permutation(sim)
    pmap, pvec = sim.cheat_local_numpy()
    pmap = dict(pmap)
    moved = remap_indices(pick, gmap, pmap).astype(np.int64)
    out["permutation"] = {"followed_amplitudes": int(len(pick)),
                          "bit_exact": bool(np.array_equal(pvec[moved].view(np.uint64), before.view(np.uint64))),
                          "layout_changed": pmap != gmap,
                          "amplitudes_max_abs_vs_oracle": max_abs_diff(pvec, pmap, rvec, rmap, n)}
    del pvec, before
    zg = sim.get_expectation_values([[([(a, "Z"), (b, "Z")], 1.0)] for a, b in zz], ids)
    zr = [ref.get_expectation_value([([(a, "Z"), (b, "Z")], 1.0)], ids) for a, b in zz]
    out["zz"] = {"pairs": len(zz), "max_abs": float(np.max(np.abs(np.array(zg) - np.array(zr)))),
                 "call": "get_expectation_values (the 64 pairs in one read of the state)"}
    out["norm_minus_1"] = sim.get_probability([], []) - 1.0
    out["pass"] = bool(out["amplitudes_max_abs"] <= 1e-12 and out["permutation"]["bit_exact"]
                       and out["permutation"]["amplitudes_max_abs_vs_oracle"] <= 1e-12
                       and out["samples"]["mismatches"] == 0 and out["zz"]["max_abs"] <= 1e-11)
    out["seconds"] = time.perf_counter() - t0
    del sim, ref, rvec
    log("parity %dq: amplitudes %.2e, permuted %.2e (bit-exact %s), samples %d/%d compared, %d mismatches, "
        "zz %.2e, oracle %.0f s -> %s" % (n, out["amplitudes_max_abs"], out["permutation"]["amplitudes_max_abs_vs_oracle"],
                                          out["permutation"]["bit_exact"], out["samples"]["compared"], shots,
                                          out["samples"]["mismatches"], out["zz"]["max_abs"], out["oracle_seconds"],
                                          "pass" if out["pass"] else "FAIL"))
    return out


def parity_20q():
    """The 20-qubit random circuit (20 layers as in the benchmark's random
    layers), fusion off and greedy k <= 4: all 2^20 amplitudes and the 20
    single-qubit P(1) against the oracle."""
    import hiqsimulator_gb300 as hqs
    from hiqsimulator_gb300 import circuits
    from oracle.engine import OracleSimulator
    n = 20
    qs = list(range(n))
    gates = circuits.random_circuit_20q(seed=1234, n=n, layers=20)
    out = {}
    for mode, cmds in (("fusion_off", circuits.fusion_off_stream(gates)),
                       ("greedy_k4", circuits.greedy_stream(gates, qs, 4))):
        ref = OracleSimulator(1234, n, 4)
        sim = hqs.SimulatorMPI(1234, n, 4, "c128")
        for s in (ref, sim):
            s.allocate_qureg(qs, 0)
            circuits.replay(s, cmds)
            s.run()
        gmap, gvec = sim.cheat_local_numpy()
        rmap = {q: p for p, q in enumerate(ref.get_qubits_ids())}
        p1 = max(abs(sim.get_probability([True], [q]) - ref.get_probability([True], [q])) for q in qs)
        out[mode] = {"amplitudes": 1 << n, "amplitudes_max_abs": max_abs_diff(gvec, dict(gmap), ref.vec, rmap, n),
                     "p1_max_abs": float(p1)}
        out[mode]["pass"] = bool(out[mode]["amplitudes_max_abs"] <= 1e-12 and p1 <= 1e-12)
        log("parity 20q %s: amplitudes %.2e, P(1) %.2e" % (mode, out[mode]["amplitudes_max_abs"], p1))
        del sim, ref
    return out


def parity_report(args, cmds, zz, shots):
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    out = {"checker": "oracle/ (C restatement of the reference engine, pinned to the reference's own outputs)",
           "host_threads": int(os.environ["OMP_NUM_THREADS"])}
    out["random_20q"] = parity_20q()
    out["headline_%dq" % N_QUBITS] = parity_headline(args, cmds, zz, shots)
    return out


def run_tour(args):
    """One launch or a few of every state-streaming kernel on an
    args.qubits-qubit state (the workload for the per-kernel ncu summaries):
    fused passes of the benchmark circuit in tensor-core digit mode and in
    double-float mode (complex128) and in the complex64 tensor-core mode, probability, the measurement block sums, Z-string and
    general Pauli expectation values, 64 <Z_a Z_b> in one call, the qubit
    permutation, collapse, the drop of a qubit and one batched serving run."""
    import hiqsimulator_gb300 as hqs
    from hiqsimulator_gb300 import circuits, serving
    n = N_QUBITS
    ids = list(range(n))
    gates = circuits.qft_random_layers(seed=SEED, n=n, layers=2)
    cmds = circuits.greedy_stream(gates, ids, CLUSTER)
    head = []
    runs = 0
    for c in cmds:
        head.append(c)
        runs += c[0] == "run"
        if runs == 24:
            break
    def replayed(arith):
        sim = hqs.SimulatorMPI(SEED, n, CLUSTER, "c128", arith)
        sim.allocate_qureg(ids, 0)
        circuits.replay(sim, head)
        sim.run()
        sim.synchronize()
        log("tour %s: %d fused gates" % (arith, runs))
        return sim

    sim = replayed("df")
    del sim
    # the complex64 tensor-memory pass on the last 24 fused gates (random layers: dense gates alone)
    run_at = [i for i, c in enumerate(cmds) if c[0] == "run"]
    tail = cmds[run_at[-25] + 1:] if len(run_at) > 25 else cmds
    c64 = hqs.SimulatorMPI(SEED, n, CLUSTER, "c64", "tc")
    c64.allocate_qureg(ids, 0)
    circuits.replay(c64, tail)
    c64.run()
    c64.synchronize()
    log("tour c64: %d fused gates" % runs)
    del c64
    sim = replayed("tc")
    p = sim.get_probability([True], [3])
    smp = sim.sample(64)
    zz = sim.get_expectation_value([([(2, "Z"), (n - 1, "Z")], 1.0)], ids)
    xy = sim.get_expectation_value([([(0, "X"), (5, "Y")], 0.5), ([(7, "Z")], 0.25)], ids)
    zz64 = sim.get_expectation_values([[([(a, "Z"), (b, "Z")], 1.0)] for a, b in circuits.zz_pairs_and_shots(SEED, n)[0]],
                                      ids)
    force_permutation(sim)
    low = sim.get_qubits_ids()[0]  # the qubit now at position 0: dropping it compacts the whole state
    p0 = sim.get_probability([True], [low])
    sim.collapse_wavefunction([low], [p0 > 0.5])
    sim.deallocate_qubit(low)
    sim.synchronize()
    log("tour queries: p %.3f, %d samples, zz %.3e, xy %.3e, 64 zz sum %.3e" % (p, len(smp), zz, xy, sum(zz64)))
    del sim
    work = serving.serving_workload(11, 24)
    res, st = serving.serve(work, np.zeros(len(work)), precision="c128", arith="tc", budget_bytes=8e9, max_active=24)
    log("tour serving: %d circuits, %d launches" % (len(res), st["launches"]))
    return 0


def run_reference(args, dist):
    if dist.rank != 0:
        return 0
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    os.environ.setdefault("OMP_PROC_BIND", "spread")
    gates, clusters, cmds = workload()
    sim = cpu_sample_sim()
    vals = []
    for s in range(args.warmup + args.steps):
        v, threads, desc = cpu_sample(sim, gates, clusters)
        if s >= args.warmup:
            vals.append(v)
        log("reference step %d: %.2f GB/s (%s)" % (s, v, desc))
    value = statistics.median(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded circuits)",
            "config": {"workload": "QFT%d + 10 random layers, greedy fusion k<=5, complex128, %d qubits" % (
                           N_QUBITS, N_QUBITS),
                       "sample": desc},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc,
                             "host": host_info()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, dist):
    import hiqsimulator_gb300 as hqs
    from hiqsimulator_gb300 import circuits
    gates, clusters, cmds = workload()
    pass_ref_bytes = cluster_bytes(gates, clusters)  # the reference's sweeps, one per fused gate
    ref_bytes = pass_ref_bytes + 2 * (16 << N_QUBITS)  # + the forced permutation
    zz, shots = circuits.zz_pairs_and_shots(SEED, N_QUBITS)
    ids = list(range(N_QUBITS))

    # ---- device-resident timing (value): state allocated once, steps replay the
    # fused circuit through the engine; CUDA events on the engine's stream.
    sim = hqs.SimulatorMPI(SEED, N_QUBITS, CLUSTER, "c128", args.arith)
    sim.set_pass_limits(defer=args.defer)
    sim.allocate_qureg(ids, 0)
    sim.synchronize()
    for _ in range(args.warmup):
        circuits.replay(sim, cmds)
        force_permutation(sim)
        sim.synchronize()
    clocks = ClockSampler(args.gpu_id)
    dist.barrier()
    clocks.start()
    s0 = sim.stats()
    sim.enable_pass_timing(True)
    sim.timer_start()
    for _ in range(args.steps):
        circuits.replay(sim, cmds)
        force_permutation(sim)
    ms = sim.timer_stop()
    pt = sim.pass_timing()
    sim.enable_pass_timing(False)
    clk = clocks.stop()
    if args.pass_log:
        for k, (kname, nops, byts, lms, copies, tmask) in enumerate(pt["log"]):
            log("launch %3d %-17s ops %2d  %7.2f ms  copies %2d  targets %s" % (
                k, kname, nops, lms, copies, [b for b in range(64) if (tmask >> b) & 1]))
    s1 = sim.stats()
    ms = dist.max(ms)
    dist.barrier()
    launches = s1["passes"] - s0["passes"] + args.steps  # fused passes + one permutation per step
    value = dist.ws * args.steps * ref_bytes / (ms / 1e3) / 1e9
    log("value: %.1f GB/s over %d steps (%.1f ms/step, %d launches)" % (value, args.steps, ms / args.steps, launches))

    # roofline of the dominant kernel (the fused pass): every launch sweeps
    # the state once, so its algorithmic bytes are one read and one write of
    # every amplitude it touches (2 * 2^n * 16 B, halved per control the
    # pass's gates share), over the pass kernels' own device time (CUDA
    # events on the engine stream). The reference-equivalent rate (one
    # reference sweep per fused gate; a launch applies several fused gates)
    # is reported beside it as work throughput, not as the HBM fraction.
    peak, peak_kind = measured_peak()
    nl = max(pt["launches"], 1)
    algo = args.steps * pass_ref_bytes
    kinds = {}
    for kname, nops, byts, lms, _, _ in pt["log"]:
        k = kinds.setdefault(kname, {"launches": 0, "bytes": 0, "ms": 0.0, "ops": 0})
        k["launches"] += 1
        k["bytes"] += byts
        k["ms"] += lms
        k["ops"] += nops
    for k in kinds.values():
        k["GBs"] = k["bytes"] / (k["ms"] / 1e3) / 1e9 if k["ms"] > 0 else 0.0
        k["frac"] = k["GBs"] / peak
        k["avg_launch_ms"] = k["ms"] / max(k["launches"], 1)
        k["share"] = k["ms"] / pt["ms"] if pt["ms"] > 0 else 0.0
    top = max(kinds, key=lambda x: kinds[x]["ms"]) if kinds else "pass_kernel"
    for kname, k in sorted(kinds.items()):
        log("kernel %s: %d launches, %.1f ms avg, %.0f GB/s sweep (%.3f of %s HBM), %.0f%% of pass time" % (
            kname, k["launches"], k["avg_launch_ms"], k["GBs"], k["frac"], peak_kind, 100 * k["share"]))
    sweep = pt["bytes"] / (pt["ms"] / 1e3) / 1e9 if pt["ms"] > 0 else 0.0
    refeq = algo / (pt["ms"] / 1e3) / 1e9 if pt["ms"] > 0 else 0.0
    traffic = profile_traffic(top)
    kt = kinds.get(top, {"GBs": sweep, "launches": nl, "bytes": pt["bytes"], "ms": pt["ms"]})
    roof = {"bound": "hbm", "achieved": kt["GBs"], "peak": peak, "unit": "GB/s", "frac": kt["GBs"] / peak,
            "traffic": traffic, "peak_source": peak_kind, "kernel": top,
            "launches": kt["launches"], "algorithmic_bytes_per_launch": kt["bytes"] / max(kt["launches"], 1),
            "avg_launch_ms": kt["ms"] / max(kt["launches"], 1),
            "all_pass_launches": {"launches": pt["launches"], "GBs": sweep, "frac": sweep / peak,
                                  "fused_gates_per_launch": args.steps * len(clusters) / nl},
            "kernels": kinds,
            "reference_equivalent_bytes_per_launch": algo / nl, "reference_equivalent_GBs": refeq,
            "reference_equivalent_frac": refeq / peak}
    # the same launches against GB300's FP64 rate: the reference's FP64 flops
    # of the fused gates over the pass kernels' device time
    flops = cluster_flops(gates, clusters)
    fp64 = flops * args.steps / (pt["ms"] / 1e3) / 1e12 if pt["ms"] > 0 else 0.0
    roof64 = {"bound": "fp64", "achieved": fp64, "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s",
              "frac": fp64 / FP64_PEAK_TFLOPS, "flops_per_step": flops,
              "peak_source": "measured FP64 DFMA loop on GB300 (0.5 T DFMA/s)",
              "note": "reference FP64 flops per second; above 1 means faster than native FP64 could run them"}
    del sim

    # ---- end to end through the drop-in API: fresh simulator, allocate, gates
    # from host lists, <Z_i Z_j> for 64 pairs and 1024 samples back to the host.
    def e2e_step():
        s = hqs.SimulatorMPI(SEED, N_QUBITS, CLUSTER, "c128", args.arith)
        s.set_pass_limits(defer=args.defer)
        s.allocate_qureg(ids, 0)
        circuits.replay(s, cmds)
        s.run()
        force_permutation(s)
        ev = s.get_expectation_values([[([(a, "Z"), (b, "Z")], 1.0)] for a, b in zz], ids)
        smp = s.sample(shots)
        return ev, smp

    e2e = None
    if not args.no_e2e:
        e2e_steps = max(1, min(args.steps, 3))
        e2e_step()
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        e2e_s = dist.max(time.perf_counter() - t0)
        h2d = sum(16 * len(c[1].matrix) ** 2 for c in cmds if c[0] == "gate")
        d2h = 8 * len(zz) + 8 * shots
        e2e = {"value": dist.ws * e2e_steps * ref_bytes / e2e_s / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s / e2e_steps}

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        v, threads, desc = cpu_sample(cpu_sample_sim(), gates, clusters)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc, "host": host_info()}

    serv = serving_report(args) if (dist.rank == 0 and args.serve > 0) else None
    prec = precision_report() if (dist.rank == 0 and not args.no_precision) else None
    par = parity_report(args, cmds, zz, shots) if (dist.rank == 0 and not args.no_parity) else None
    cap = capacity_report() if (dist.rank == 0 and args.capacity) else None
    table = table_report(cmds, pass_ref_bytes) if (dist.rank == 0 and args.table) else None

    if dist.rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "c128 (%s arithmetic)" % args.arith,
                "data": "synthetic (seeded circuits)",
                "config": {"workload": "QFT%d + 10 random layers, greedy fusion k<=5, complex128, %d qubits" % (
                               N_QUBITS, N_QUBITS),
                           "fused_gates_per_step": len(clusters), "gates_per_step": len(gates),
                           "forced_permutation": "top 5 qubits to positions 0-4 once per step",
                           "state_bytes": 16 << N_QUBITS, "l2": "inputs larger than L2 (%d MiB state)" % ((16 << N_QUBITS) >> 20),
                           "parallelism": "replicas" if dist.ws > 1 else "single GPU"},
                "roofline": roof, "fp64_roofline": roof64, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk, "parity": par, "serving": serv, "precision": prec, "capacity": cap, "table": table}
        print(json.dumps(line), flush=True)
    return 0


def bind_gpu():
    """One GPU per rank under torchrun: the rank's device becomes the only
    visible one (before any CUDA use in this process). Returns the physical
    GPU id for nvidia-smi."""
    ws, _, local = dist_env()
    vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    if ws <= 1:
        return vis[0] if vis else "0"
    dev = vis[local % len(vis)] if vis else str(local)
    os.environ["CUDA_VISIBLE_DEVICES"] = dev
    return dev


def main():
    gpu_id = bind_gpu()
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--arith", default="tc", choices=["tc", "df", "f64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--defer", type=int, default=8, help="fused gates queued before the engine launches")
    ap.add_argument("--qubits", type=int, default=30, help="state size (30 is the benchmark configuration)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--serve", type=int, default=400, help="circuits in the serving run (0 skips it)")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[4000.0, 100.0, 50.0, 25.0],
                    help="complex128 arrival rates (circuits/s); the first is also run one circuit per launch")
    ap.add_argument("--serve-rates64", type=float, nargs="+", default=[4000.0, 200.0, 100.0],
                    help="complex64 arrival rates (circuits/s)")
    ap.add_argument("--serve-slots", type=int, default=32, help="resident circuits at most while serving")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the comparisons with the oracle")
    ap.add_argument("--tour", action="store_true", help="launch every state-streaming kernel once (profiling)")
    ap.add_argument("--pass-log", action="store_true", help="print every timed pass launch")
    ap.add_argument("--capacity", action="store_true", help="also run the 33q c128 / 34q c64 capacity states")
    ap.add_argument("--table", action="store_true", help="also time the reference-against-GPU table rows")
    args = ap.parse_args()
    args.gpu_id = gpu_id
    global N_QUBITS
    N_QUBITS = args.qubits
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        if args.tour:
            return run_tour(args)
        return run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
