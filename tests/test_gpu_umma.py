"""The tensor-memory pass (umma_pass.cu: tcgen05 MMAs with tensor-memory
accumulators, TMA tile copies) through the C ABI against the C oracle, for
complex128 states (tc) and complex64 states (tc64): dense 3-5 qubit gates
with their targets low, high and scattered (one or two TMA copies per tile),
widened gates (k < 5), controls inside and outside the tile, runs of
diagonal and scalar gates before and after the dense gate, and states from
one tile per SM to many (the copy pipeline). Tolerance: 1e-12 max-abs for
complex128 (as every complex128 path); for complex64 1e-6 of the largest
amplitude (FP32 rounding of the inputs, outputs and run factors; the
oracle runs in FP64 on the complex64-rounded input)."""
import numpy as np
import pytest

from test_gpu_kernels import Dev, oracle_apply, rand_state

pytestmark = pytest.mark.gpu

TOL = 1e-12
C64_REL = 1e-6
ARITHS = ["tc", "tc64"]


def dense(rng, pos, ctrl=0):
    d = 1 << len(pos)
    g = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    m, _ = np.linalg.qr(g)
    return (len(pos), list(pos), ctrl, False, m)


def diag(rng, pos, ctrl=0):
    d = 1 << len(pos)
    return (len(pos), list(pos), ctrl, True, np.diag(np.exp(1j * rng.uniform(0, 2 * np.pi, d))))


def scalar(rng):
    return (0, [], 0, False, np.array([[np.exp(1j * rng.uniform(0, 2 * np.pi))]]))


@pytest.fixture(scope="module")
def ws(hqs, cuda):
    from hiqsimulator_gb300 import capi
    w = capi.Workspace()
    yield w
    w.close()


def run_case(ws, cuda, oracle_lib, n, gates, rng, expect_umma=1, psi=None, arith="tc"):
    from hiqsimulator_gb300 import capi
    plan = capi.plan_launches(n, arith, [g[:4] for g in gates])
    assert sum(L["umma"] for L in plan) == expect_umma, plan
    if psi is None:
        psi = rand_state(rng, n)
    c64 = arith == "tc64"
    if c64:
        psi = psi.astype(np.complex64).astype(np.complex128)
    d = Dev(cuda, psi, c64=c64)
    ws.apply_gates(d.ptr, n, arith, gates)
    ws.synchronize()
    ref = psi.copy()
    for g in gates:
        oracle_apply(oracle_lib, ref, g)
    err = float(np.max(np.abs(d.host() - ref)))
    tol = C64_REL * float(np.max(np.abs(ref))) if c64 else TOL
    assert err < tol, (n, arith, [g[:4] for g in gates], err)
    return plan


TARGETS = [
    (12, [0, 1, 2, 3, 4]),          # low targets: groups above them
    (12, [7, 8, 9, 10, 11]),        # high targets: one box
    (16, [11, 12, 13, 14, 15]),
    (18, [0, 5, 9, 13, 17]),        # scattered: gaps between runs
    (20, [3, 7, 11, 15, 19]),       # more runs than dimensions: copies
    (22, [2, 9, 12, 16, 21]),
    (24, [1, 6, 13, 18, 23]),       # includes outputs just below a power of two
    (24, [0, 1, 2, 3, 4]),
    (24, [8, 10, 12, 17, 21]),      # six runs of tile positions: two copies per tile
    (20, [7, 9, 11, 13, 15]),       # runs next to the low run
]


@pytest.mark.parametrize("arith", ARITHS)
@pytest.mark.parametrize("n,pos", TARGETS)
def test_umma_dense_gate_target_layouts(ws, cuda, oracle_lib, n, pos, arith):
    rng = np.random.Generator(np.random.PCG64(n * 131 + sum(pos)))
    run_case(ws, cuda, oracle_lib, n, [dense(rng, pos)], rng, arith=arith)


@pytest.mark.parametrize("arith", ARITHS)
@pytest.mark.parametrize("k", [3, 4])
@pytest.mark.parametrize("n", [12, 19])
def test_umma_widened_gates(ws, cuda, oracle_lib, k, n, arith):
    rng = np.random.Generator(np.random.PCG64(700 + 10 * k + n))
    for trial in range(3):
        pos = [int(p) for p in rng.choice(n, size=k, replace=False)]
        run_case(ws, cuda, oracle_lib, n, [dense(rng, pos)], rng, arith=arith)


@pytest.mark.parametrize("arith", ARITHS)
def test_umma_controls_inside_and_outside_the_tile(ws, cuda, oracle_lib, arith):
    rng = np.random.Generator(np.random.PCG64(77))
    n = 18
    run_case(ws, cuda, oracle_lib, n, [dense(rng, [4, 9, 10, 12, 13], ctrl=(1 << 1))], rng, arith=arith)
    run_case(ws, cuda, oracle_lib, n, [dense(rng, [4, 9, 10, 12, 13], ctrl=(1 << 17))], rng, arith=arith)
    run_case(ws, cuda, oracle_lib, n, [dense(rng, [2, 3, 8], ctrl=(1 << 0) | (1 << 16))], rng, arith=arith)


@pytest.mark.parametrize("arith", ARITHS)
def test_umma_diagonal_runs_around_the_dense_gate(ws, cuda, oracle_lib, arith):
    rng = np.random.Generator(np.random.PCG64(91))
    n = 20
    gates = [diag(rng, [0, 5, 19]), scalar(rng), diag(rng, [15, 16], ctrl=1 << 3),
             dense(rng, [1, 6, 11, 14, 18]),
             diag(rng, [2, 4, 7, 8, 17]), diag(rng, [19]), scalar(rng)]
    plan = run_case(ws, cuda, oracle_lib, n, gates, rng, arith=arith)
    assert plan[0]["umma"] and plan[0]["nops"] == len(gates)


@pytest.mark.parametrize("arith", ARITHS)
@pytest.mark.parametrize("ctrl", [1 << 2, 1 << 19, (1 << 0) | (1 << 17)])
def test_umma_runs_around_a_controlled_dense_gate(ws, cuda, oracle_lib, ctrl, arith):
    """Runs before and after a dense gate whose controls sit inside the tile
    (groups that keep their inputs still take both runs), outside it (tiles
    the gate leaves alone) or both; the runs carry their own controls."""
    rng = np.random.Generator(np.random.PCG64(400 + ctrl % 97))
    n = 20
    gates = [diag(rng, [0, 2, 19]), scalar(rng), diag(rng, [3, 16], ctrl=1 << 9),
             dense(rng, [1, 6, 11, 14, 18], ctrl=ctrl),
             diag(rng, [2, 4, 7, 17]), diag(rng, [19, 0]), scalar(rng)]
    plan = run_case(ws, cuda, oracle_lib, n, gates, rng, arith=arith)
    assert plan[0]["umma"] and plan[0]["nops"] == len(gates)


@pytest.mark.parametrize("arith", ARITHS)
def test_umma_runs_only_before_or_only_after(ws, cuda, oracle_lib, arith):
    """Runs on one side of the dense gate; matrix blocks whose size is not a
    multiple of 16 bytes (one scalar gate: 8 bytes in complex64), also
    after a tiled pass in the same call."""
    rng = np.random.Generator(np.random.PCG64(402))
    n = 18
    run_case(ws, cuda, oracle_lib, n, [diag(rng, [0, 9, 17]), dense(rng, [2, 5, 8, 12, 15])], rng, arith=arith)
    run_case(ws, cuda, oracle_lib, n, [dense(rng, [2, 5, 8, 12, 15]), diag(rng, [1, 9, 16]), scalar(rng)], rng,
             arith=arith)
    run_case(ws, cuda, oracle_lib, n, [dense(rng, [2, 5, 8, 12, 15]), scalar(rng)], rng, arith=arith)
    two = (2, [3, 6], 0, False, np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))[0])
    run_case(ws, cuda, oracle_lib, n, [two, dense(rng, [0, 1, 8, 7]), scalar(rng)], rng, arith=arith)


@pytest.mark.parametrize("arith", ARITHS)
def test_umma_sequences_of_passes_on_a_larger_state(ws, cuda, oracle_lib, arith):
    """Many tiles per CTA (the two-buffer copy pipeline), several passes in
    a row, gates whose targets move between low and high positions."""
    rng = np.random.Generator(np.random.PCG64(123))
    n = 24
    gates = []
    for i in range(6):
        pos = sorted(int(p) for p in rng.choice(n, size=5, replace=False))
        gates.append(dense(rng, pos))
        if i % 2:
            gates.append(diag(rng, [int(p) for p in rng.choice(n, size=3, replace=False)]))
    run_case(ws, cuda, oracle_lib, n, gates, rng, expect_umma=6, arith=arith)


@pytest.mark.parametrize("arith", ARITHS)
def test_umma_wide_dynamic_range_and_zeros(ws, cuda, oracle_lib, arith):
    """Amplitudes spanning 10^-20 .. 1 inside one index group, and whole
    groups of zeros."""
    rng = np.random.Generator(np.random.PCG64(5))
    n = 16
    for trial in range(3):
        psi = rand_state(rng, n) * np.exp(rng.uniform(-46, 0, 1 << n))
        psi[rng.random(1 << n) < 0.3] = 0.0
        psi /= np.linalg.norm(psi)
        gate = dense(rng, [int(p) for p in rng.choice(n, size=5, replace=False)])
        run_case(ws, cuda, oracle_lib, n, [gate], rng, psi=psi, arith=arith)
