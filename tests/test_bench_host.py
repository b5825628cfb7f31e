"""The benchmark's algorithmic counts on the host: reference bytes and FP64
flops per fused gate, on hand-built clusters with known answers."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402
from hiqsimulator_gb300.circuits import H, X, Gate, phase  # noqa: E402


def test_cluster_flops_and_bytes_known_answers():
    n = 10
    cp = phase(0.3)
    gates = [
        Gate(H, [0], []),             # 0
        Gate(X, [1], [0]),            # 1  CNOT 0 -> 1
        Gate(cp, [2], [1]),           # 2  controlled phase, diagonal
        Gate(cp, [3], [4]),           # 3
        Gate(np.diag([1, 1j]), [5], [6]),  # 4
        Gate(X, [7], [8, 9]),         # 5  Toffoli
    ]
    # {H, CNOT, CP}: dense on qubits {0, 1, 2} (the controls fold into the matrix)
    assert bench.cluster_flops(gates, [[0, 1, 2]], n) == 8 * 8 * 2 ** n
    # a lone controlled phase: diagonal on half the state
    assert bench.cluster_flops(gates, [[3]], n) == 6 * 2 ** (n - 1)
    # two diagonal gates with different controls: every qubit a target
    assert bench.cluster_flops(gates, [[3, 4]], n) == 6 * 2 ** n
    # a Toffoli alone: a 1-qubit dense gate on a quarter of the state
    assert bench.cluster_flops(gates, [[5]], n) == 8 * 2 * 2 ** (n - 2)
    assert bench.cluster_flops(gates, [[0, 1, 2], [3], [5]], n) == (
        8 * 8 * 2 ** n + 6 * 2 ** (n - 1) + 16 * 2 ** (n - 2))
    # bytes: one read and one write of the state per fused gate; a lone gate
    # too large to fuse touches 2^-c of it
    assert bench.cluster_bytes(gates, [[0, 1, 2], [5]], n) == 2 * 2 * 16 * 2 ** n


def test_host_info_names_the_cpu():
    info = bench.host_info()
    assert info["nproc"] == os.cpu_count() and info["nproc"] >= 1
    assert info["machine"] in ("x86_64", "aarch64")
    assert info["cpu_model"] is None or isinstance(info["cpu_model"], str)


def test_reference_arm_prints_the_contract_line():
    """bench.py --impl reference (the CPU arm) prints one JSON line with the
    keys the benchmark contract needs; run here at 16 qubits."""
    import json
    import subprocess
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--qubits", "16",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, env=env,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GB/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 0
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["cores"] == 2 and cpu["kind"] == "port"
    assert "16-qubit state" in cpu["sample"] and cpu["host"]["nproc"] == os.cpu_count()
    assert line["e2e"] == {"value": line["value"], "unit": "GB/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "16 qubits" in line["config"]["workload"]


def test_relayout_helpers_follow_a_qubit_permutation():
    """The parity leg compares states stored in different qubit layouts:
    the chunked comparison and the index remap agree with an explicit
    permutation of a 10-qubit state, and a planted error is found."""
    import numpy as np
    rng = np.random.default_rng(1)
    n = 10
    a = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    ma = {q: q for q in range(n)}
    perm = rng.permutation(n)
    mb = {q: int(perm[q]) for q in range(n)}
    to_b = bench.remap_indices(np.arange(1 << n, dtype=np.uint64), ma, mb).astype(np.int64)
    b = np.zeros_like(a)
    b[to_b] = a
    assert bench.max_abs_diff(a, ma, b, mb, n, chunk_axes=3) == 0.0
    assert bench.max_abs_diff(a, ma, b, ma, n) > 0.1
    b[17] += 1e-9
    assert abs(bench.max_abs_diff(a, ma, b, mb, n) - 1e-9) < 1e-15
    back = bench.remap_indices(to_b.astype(np.uint64), mb, ma)
    assert np.array_equal(back, np.arange(1 << n, dtype=np.uint64))
