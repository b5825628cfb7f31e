"""Kernel-level parity through the C ABI (hqs_ws_* / hqs_apply_gates ...) on
device buffers, against the C oracle on the same seeded inputs."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C128_TOL = 1e-12   # max-abs, complex128 states (F64 and DF arithmetic)
C64_TOL = 2e-6     # max-abs, complex64 states of norm 1
C64_ARITH = ("f32", "tf32", "tc64")
TC64_REL = 2e-5    # two-digit tensor-core gates: max-abs error over the largest amplitude


def tol(arith, ref, scale=1.0):
    if arith == "tc64":
        return scale * TC64_REL * float(np.max(np.abs(ref)))
    return scale * (C64_TOL if arith in C64_ARITH else C128_TOL)


def rand_state(rng, n):
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    return (v / np.linalg.norm(v)).astype(np.complex128)


def rand_gate(rng, n, k, with_ctrl=True, diag=False):
    pos = [int(p) for p in rng.choice(n, size=k, replace=False)]
    free = [p for p in range(n) if p not in pos]
    ctrl = 0
    if with_ctrl and free and rng.random() < 0.5:
        for p in rng.choice(free, size=int(rng.integers(1, min(3, len(free)) + 1)), replace=False):
            ctrl |= 1 << int(p)
    d = 1 << k
    if diag:
        m = np.diag(np.exp(1j * rng.uniform(0, 2 * np.pi, d)))
    else:
        g = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
        m, _ = np.linalg.qr(g)
    return (k, pos, ctrl, diag, m)


class Dev:
    """A device copy of a host state (torch buffers are plumbing only)."""

    def __init__(self, torch, host, c64=False):
        self.torch = torch
        self.c64 = c64
        t = torch.from_numpy(host.astype(np.complex64 if c64 else np.complex128))
        self.t = t.cuda()
        torch.cuda.synchronize()

    @property
    def ptr(self):
        return ctypes.c_void_p(self.t.data_ptr())

    def host(self):
        self.torch.cuda.synchronize()
        return self.t.cpu().numpy().astype(np.complex128)


def oracle_apply(lib, vec, gate):
    from oracle.lib import dptr
    k, pos, ctrl, diag, m = gate
    mm = np.ascontiguousarray(m, dtype=np.complex128)
    parr = (ctypes.c_uint * max(k, 1))(*pos)
    lib.orc_apply(dptr(vec.view(np.float64)), len(vec), k, parr, dptr(mm.view(np.float64)), ctrl, 1 if diag else 0)


@pytest.fixture(scope="module")
def ws(hqs, cuda):
    from hiqsimulator_gb300 import capi
    w = capi.Workspace()
    yield w
    w.close()


@pytest.mark.parametrize("arith", ["f64", "df", "tc", "f32", "tf32", "tc64"])
@pytest.mark.parametrize("n", [1, 3, 6, 11, 14])
def test_single_gates_match_oracle(ws, cuda, oracle_lib, arith, n):
    rng = np.random.Generator(np.random.PCG64(1000 + n))
    for k in range(1, min(5, n) + 1):
        for diag in (False, True):
            gate = rand_gate(rng, n, k, diag=diag)
            psi = rand_state(rng, n)
            d = Dev(cuda, psi, c64=arith in C64_ARITH)
            ws.apply_gates(d.ptr, n, arith, [gate])
            ws.synchronize()
            ref = psi.copy()
            oracle_apply(oracle_lib, ref, gate)
            err = np.max(np.abs(d.host() - ref))
            assert err < tol(arith, ref), (arith, n, k, diag, err)


@pytest.mark.parametrize("arith", ["f64", "df", "tc", "f32", "tf32", "tc64"])
@pytest.mark.parametrize("n,tile", [(12, 11), (16, 11), (16, 8), (20, 12)])
def test_fused_passes_match_sequential_oracle(ws, cuda, oracle_lib, arith, n, tile):
    """Many gates planned into multi-gate tiled passes equal the gates applied
    one by one."""
    rng = np.random.Generator(np.random.PCG64(2000 + n + tile))
    gates = []
    for _ in range(40):
        k = int(rng.integers(0, 6))
        if k == 0:
            gates.append((0, [], 0, False, np.array([[np.exp(1j * rng.uniform(0, 6.28))]])))
        else:
            gates.append(rand_gate(rng, n, k, diag=bool(rng.random() < 0.3)))
    psi = rand_state(rng, n)
    d = Dev(cuda, psi, c64=arith in C64_ARITH)
    by, passes = ws.apply_gates(d.ptr, n, arith, gates, max_tile_bits=tile)
    ws.synchronize()
    assert 1 <= passes <= len(gates)
    ref = psi.copy()
    for g in gates:
        oracle_apply(oracle_lib, ref, g)
    err = np.max(np.abs(d.host() - ref))
    assert err < tol(arith, ref, 5.0 if arith in C64_ARITH else 1.0), (arith, n, err, passes)


@pytest.mark.parametrize("arith", ["f64", "df", "f32"])
def test_probability_block_sums_collapse(ws, cuda, oracle_lib, arith):
    from oracle.lib import dptr
    rng = np.random.Generator(np.random.PCG64(3))
    n = 15
    psi = rand_state(rng, n)
    c64 = arith == "f32"
    src = psi.astype(np.complex64).astype(np.complex128) if c64 else psi
    d = Dev(cuda, psi, c64=c64)
    tol = 1e-6 if c64 else 1e-13
    for _ in range(10):
        mask = int(rng.integers(0, 1 << n))
        val = int(rng.integers(0, 1 << n)) & mask
        got = ws.probability(d.ptr, n, arith, mask, val)
        want = oracle_lib.orc_probability(dptr(src.view(np.float64)), len(src), mask, val)
        assert abs(got - want) < tol
    for nb in (1, 64, 1 << 10, 1 << 15):
        got = ws.block_sums(d.ptr, n, arith, nb)
        cdf = np.zeros(nb)
        oracle_lib.orc_block_cdf(dptr(src.view(np.float64)), len(src), nb, dptr(cdf))
        want = np.diff(np.concatenate([[0.0], cdf]))
        assert np.max(np.abs(got - want)) < tol
    mask, val = 0b1010000011, 0b0010000001
    p = oracle_lib.orc_probability(dptr(src.view(np.float64)), len(src), mask, val)
    ws.collapse(d.ptr, n, arith, mask, val, 1.0 / np.sqrt(p))
    ref = src.copy()
    oracle_lib.orc_normalize(dptr(ref.view(np.float64)), len(ref), mask, val, p)
    assert np.max(np.abs(d.host() - ref)) < (C64_TOL if c64 else C128_TOL)


@pytest.mark.parametrize("arith", ["df", "f32"])
def test_permute_bits_is_exact(ws, cuda, arith):
    rng = np.random.Generator(np.random.PCG64(4))
    c64 = arith == "f32"
    top5 = list(range(12, 17))
    for n, oldpos, newpos in [(17, [0, 16], [16, 0]), (17, [1, 2, 3, 14, 15, 16], [14, 15, 16, 1, 2, 3]),
                              (17, [0, 5, 9, 12], [5, 9, 12, 0]), (17, list(range(12)), list(range(11, -1, -1))),
                              (17, top5 + [0, 1, 2, 3, 4], [0, 1, 2, 3, 4] + top5),   # the forced permutation
                              (20, [15, 16, 17, 18, 19, 0, 1, 2, 3, 4], [0, 1, 2, 3, 4, 15, 16, 17, 18, 19]),
                              (7, [0, 6], [6, 0]), (5, [0, 1, 4], [4, 0, 1])]:
        psi = rand_state(rng, n)
        src = psi.astype(np.complex64).astype(np.complex128) if c64 else psi
        d = Dev(cuda, psi, c64=c64)
        ws.permute_bits(d.ptr, n, arith, oldpos, newpos)
        idx = np.arange(1 << n)
        # new index: bit newpos[j] = old bit oldpos[j]
        newidx = idx.copy()
        for o, p in zip(oldpos, newpos):
            newidx &= ~(1 << p)
        for o, p in zip(oldpos, newpos):
            newidx |= ((idx >> o) & 1) << p
        want = np.zeros_like(src)
        want[newidx] = src
        assert np.array_equal(d.host(), want)   # pure data movement: bit-exact


@pytest.mark.parametrize("arith", ["df", "f32"])
@pytest.mark.parametrize("pos,keep", [(0, 0), (0, 1), (5, 0), (5, 1), (12, 0), (12, 1)])
def test_drop_bit_matches_oracle(ws, cuda, oracle_lib, arith, pos, keep):
    from oracle.lib import dptr
    rng = np.random.Generator(np.random.PCG64(5 + pos))
    n = 13
    psi = rand_state(rng, n)
    c64 = arith == "f32"
    src = psi.astype(np.complex64).astype(np.complex128) if c64 else psi
    d = Dev(cuda, psi, c64=c64)
    ws.drop_bit(d.ptr, n, arith, pos, keep)
    ref = src.copy()
    oracle_lib.orc_drop_bit(dptr(ref.view(np.float64)), len(ref), pos, keep)
    got = d.host()[: 1 << (n - 1)]
    assert np.array_equal(got, ref[: 1 << (n - 1)])


def test_df_arith_roundtrip_exactness(ws, cuda):
    """An identity gate through the double-float path returns each amplitude
    to within 2^-46 of its value (the split keeps ~48 bits)."""
    rng = np.random.Generator(np.random.PCG64(6))
    n = 10
    psi = rand_state(rng, n) * np.exp(rng.uniform(-30, 0, 1 << n))
    d = Dev(cuda, psi)
    ws.apply_gates(d.ptr, n, "df", [(1, [3], 0, False, np.eye(2))])
    rel = np.abs(d.host() - psi) / np.maximum(np.abs(psi), 1e-300)
    assert np.max(rel) < 2.0 ** -45


@pytest.mark.parametrize("k", [3, 4, 5])
def test_tensor_core_gates_on_wide_dynamic_range(ws, cuda, oracle_lib, k):
    """Dense gates on the tensor-core path (digit products) stay within the
    complex128 tolerance when amplitudes inside one index group differ by many
    orders of magnitude, and with controls inside and outside the tile."""
    rng = np.random.Generator(np.random.PCG64(50 + k))
    n = 16
    for trial in range(3):
        psi = rand_state(rng, n) * np.exp(rng.uniform(-25, 0, 1 << n))
        psi /= np.linalg.norm(psi)
        gate = rand_gate(rng, n, k, with_ctrl=True)
        d = Dev(cuda, psi)
        ws.apply_gates(d.ptr, n, "tc", [gate])
        ref = psi.copy()
        oracle_apply(oracle_lib, ref, gate)
        assert np.max(np.abs(d.host() - ref)) < C128_TOL
