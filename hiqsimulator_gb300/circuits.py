"""Seeded synthetic circuits for the benchmark configurations and the parity
tests, and the command streams a ProjectQ front end would send to the engine.

All randomness comes from numpy Generator(PCG64(seed)); the unitary samplers
use explicit Gram-Schmidt so the matrices do not depend on a LAPACK build.
A circuit is a list of Gate(matrix, ids, ctrls); a command stream is a list of
("gate", Gate) and ("run",) entries, the latter being the FlushGate -> run()
calls of the backend (hiq/projectq/backends/_sim/_simulator_mpi.py:485-508).
"""
import math
from collections import namedtuple

import numpy as np

Gate = namedtuple("Gate", ["matrix", "ids", "ctrls"])

H = np.array([[1, 1], [1, -1]], dtype=np.complex128) / math.sqrt(2.0)
X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)


def rng_for(seed):
    return np.random.Generator(np.random.PCG64(seed))


def phase(theta):
    """R(theta) = diag(1, e^{i theta})."""
    return np.array([[1, 0], [0, complex(math.cos(theta), math.sin(theta))]], dtype=np.complex128)


def haar_unitary(rng, d):
    """Haar-random U(d): Gram-Schmidt QR of a complex Ginibre matrix with the
    phases of R's diagonal folded into Q (Mezzadri's recipe)."""
    g = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / math.sqrt(2.0)
    q = np.zeros((d, d), dtype=np.complex128)
    for j in range(d):
        v = g[:, j].copy()
        for i in range(j):
            v = v - np.vdot(q[:, i], v) * q[:, i]
        r = math.sqrt(float(np.sum(v.real * v.real + v.imag * v.imag)))
        q[:, j] = v / r
    return q


def random_layer(rng, qubits, cnot_target_pool=None, bias=0.0):
    """One layer: Haar U(2) on every qubit, CNOTs on a random perfect matching
    (random control/target order), one controlled phase on a random pair.
    With cnot_target_pool and bias, a pair's target is drawn from the pool with
    probability bias when the pair touches it."""
    gates = [Gate(haar_unitary(rng, 2), [q], []) for q in qubits]
    perm = list(rng.permutation(len(qubits)))
    for a in range(0, len(perm) - 1, 2):
        c, t = qubits[perm[a]], qubits[perm[a + 1]]
        if rng.random() < 0.5:
            c, t = t, c
        if cnot_target_pool is not None:
            in_c, in_t = c in cnot_target_pool, t in cnot_target_pool
            if in_c != in_t and rng.random() < bias and in_c:
                c, t = t, c
        gates.append(Gate(X, [t], [c]))
    if len(qubits) >= 2:
        a, b = rng.choice(len(qubits), size=2, replace=False)
        theta = rng.uniform(0.0, 2.0 * math.pi)
        gates.append(Gate(phase(theta), [qubits[int(b)]], [qubits[int(a)]]))
    return gates


def random_layers(seed, qubits, layers, **kw):
    rng = rng_for(seed)
    out = []
    for _ in range(layers):
        out += random_layer(rng, qubits, **kw)
    return out


def qft(qubits):
    """QFT without the final swaps: for the top qubit down, H then controlled
    phases pi/2^d from every lower qubit."""
    out = []
    n = len(qubits)
    for i in range(n - 1, -1, -1):
        out.append(Gate(H, [qubits[i]], []))
        for j in range(i - 1, -1, -1):
            out.append(Gate(phase(math.pi / (1 << (i - j))), [qubits[i]], [qubits[j]]))
    return out


def brickwork(seed, qubits, layers):
    """Haar U(4) on (0,1),(2,3),... then (1,2),(3,4),..., alternating."""
    rng = rng_for(seed)
    out = []
    for l in range(layers):
        start = l % 2
        for a in range(start, len(qubits) - 1, 2):
            out.append(Gate(haar_unitary(rng, 4), [qubits[a], qubits[a + 1]], []))
    return out


def grover_iterations(seed, qubits, iterations):
    """Each iteration: oracle = X on the zero bits of a seeded marked string,
    multi-controlled Z, X; diffusion = H-X-MCZ-X-H on every qubit."""
    rng = rng_for(seed)
    marked = [int(b) for b in rng.integers(0, 2, size=len(qubits))]
    out = []
    top, rest = qubits[-1], qubits[:-1]
    for _ in range(iterations):
        zeros = [q for q, b in zip(qubits, marked) if b == 0]
        out += [Gate(X, [q], []) for q in zeros]
        out.append(Gate(Z, [top], list(rest)))
        out += [Gate(X, [q], []) for q in zeros]
        out += [Gate(H, [q], []) for q in qubits]
        out += [Gate(X, [q], []) for q in qubits]
        out.append(Gate(Z, [top], list(rest)))
        out += [Gate(X, [q], []) for q in qubits]
        out += [Gate(H, [q], []) for q in qubits]
    return out, marked


# ----------------------------------------------------------------- streams

def fusion_off_stream(gates):
    """gate_fusion=False: run() after every gate."""
    cmds = []
    for g in gates:
        cmds.append(("gate", g))
        cmds.append(("run",))
    return cmds


def greedy_clusters(gates, locals_, cluster_size, scheduler=None):
    """Greedy clusters of gate indices (native scheduler unless given)."""
    if scheduler is None:
        from .capi import greedy_schedule as scheduler
    return scheduler([list(g.ids) for g in gates], [list(g.ctrls) for g in gates], list(locals_), cluster_size)


def greedy_stream(gates, locals_, cluster_size, scheduler=None, clusters=None):
    """GreedyScheduler: each cluster's gates, then run()."""
    if clusters is None:
        clusters = greedy_clusters(gates, locals_, cluster_size, scheduler)
    cmds = []
    for cl in clusters:
        for i in cl:
            cmds.append(("gate", gates[i]))
        cmds.append(("run",))
    return cmds


def replay(sim, cmds):
    """Send a command stream to anything with the SimulatorMPI method names."""
    for c in cmds:
        if c[0] == "gate":
            g = c[1]
            sim.apply_controlled_gate(g.matrix.tolist(), list(g.ids), list(g.ctrls))
        else:
            sim.run()


# ------------------------------------------------------------ configurations

def random_circuit_20q(seed=1234, n=20, layers=20):
    """20-qubit seeded random circuit (20 layers)."""
    return random_layers(seed, list(range(n)), layers)


def qft_random_layers(seed=4321, n=30, layers=10):
    """QFT on all n qubits followed by `layers` random layers."""
    qs = list(range(n))
    return qft(qs) + random_layers(seed, qs, layers)


def zz_pairs_and_shots(seed, n, pairs=64, shots=1024):
    """Seeded qubit pairs for <Z_i Z_j> and the number of full-register samples."""
    rng = rng_for(seed + 7)
    zz = []
    for _ in range(pairs):
        a, b = rng.choice(n, size=2, replace=False)
        zz.append((int(a), int(b)))
    return zz, shots


def capacity_circuit(seed=99, n=33, layers=8, grover=4):
    """Random layers with CNOT targets biased 70% towards the top 8 qubits,
    then Grover iterations (multi-controlled Z on all n qubits) for a seeded
    marked string. Returns (gates, marked)."""
    qs = list(range(n))
    top = set(qs[-8:])
    g = random_layers(seed, qs, layers, cnot_target_pool=top, bias=0.7)
    gr, marked = grover_iterations(seed + 1, qs, grover)
    return g + gr, marked


def brickwork_28q(seed=2024, n=28, layers=40):
    return brickwork(seed, list(range(n)), layers)


def inverse(gates):
    """The inverse circuit: reversed order, conjugate-transposed matrices."""
    return [Gate(np.conj(np.asarray(g.matrix)).T.copy(), list(g.ids), list(g.ctrls)) for g in reversed(gates)]


def inverse_stream(gates, clusters):
    """Command stream of the inverse circuit that undoes a clustered stream
    cluster by cluster: the clusters in reverse order, each cluster's gates
    reversed and inverted, then run()."""
    cmds = []
    for cl in reversed(clusters):
        for g in inverse([gates[i] for i in cl]):
            cmds.append(("gate", g))
        cmds.append(("run",))
    return cmds


def pauli_sum(seed, n, terms=8):
    """Random Pauli-string sum with real N(0,1) coefficients, in the backend's
    encoding [(term, coef)] with term = [(index, 'X'|'Y'|'Z'), ...]."""
    rng = rng_for(seed)
    out = []
    for _ in range(terms):
        w = int(rng.integers(1, min(n, 4) + 1))
        idx = sorted(int(i) for i in rng.choice(n, size=w, replace=False))
        term = [(i, "XYZ"[int(rng.integers(0, 3))]) for i in idx]
        out.append((term, float(rng.standard_normal())))
    return out
