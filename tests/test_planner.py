"""The pass planner on the host (hqs_plan_passes, no GPU): how fused gates are
grouped into tiled sweeps of the state, the tile each sweep uses, and the
shared-memory and pipelining decisions that come with it."""
import numpy as np
import pytest

from hiqsimulator_gb300 import capi

SMEM_PER_SM = 233472      # 228 KB
SMEM_PER_CTA = 232448     # 227 KB


def popc(x):
    return bin(x).count("1")


def rand_ops(rng, n, count):
    ops = []
    for _ in range(count):
        k = int(rng.integers(0, 6))
        if k == 0:
            ops.append((0, [], 0, False))
            continue
        pos = [int(p) for p in rng.choice(n, size=k, replace=False)]
        free = [p for p in range(n) if p not in pos]
        ctrl = 0
        if rng.random() < 0.3:
            for p in rng.choice(free, size=int(rng.integers(1, 3)), replace=False):
                ctrl |= 1 << int(p)
        ops.append((k, pos, ctrl, bool(rng.random() < 0.35)))
    return ops


@pytest.mark.parametrize("arith", ["tc", "df", "f64", "f32", "tc64", "tf32"])
@pytest.mark.parametrize("n,tile", [(12, 11), (20, 11), (26, 10), (30, 12)])
def test_passes_partition_ops_and_hold_their_targets(hqs, arith, n, tile):
    rng = np.random.Generator(np.random.PCG64(300 + n + tile))
    ops = rand_ops(rng, n, 60)
    plans = capi.plan_passes(n, arith, ops, max_tile_bits=tile)
    nxt = 0
    for p in plans:
        assert p["first_op"] == nxt and p["nops"] >= 1
        nxt += p["nops"]
        assert popc(p["tile_mask"]) == p["q"]
        assert p["tile_mask"] & ((1 << p["w"]) - 1) == (1 << p["w"]) - 1
        assert not (p["tile_mask"] >> p["w"]) & 1 or p["w"] == p["q"]
        assert p["smem_bytes"] <= SMEM_PER_CTA
        dense = 0
        for k, pos, ctrl, diag in ops[p["first_op"]:p["first_op"] + p["nops"]]:
            if not diag:
                for q in pos:
                    dense |= 1 << q
        assert dense & ~p["tile_mask"] == 0, "a dense target outside the tile"
        if p["nops"] > 1:
            assert popc(dense) + 4 <= tile or popc(dense) <= p["q"]
        assert p["fixed_mask"] & p["tile_mask"] == 0
        assert p["sweep_bytes"] == 2 * (1 << (n - popc(p["fixed_mask"]))) * (8 if arith in ("f32", "tc64", "tf32") else 16)
    assert nxt == len(ops)


def test_diagonal_gates_join_a_pass_with_targets_outside_the_tile(hqs):
    # a 5-qubit dense gate then the diagonal 5-qubit gates a QFT produces
    n = 30
    ops = [(5, [25, 26, 27, 28, 29], 0, False)]
    ops += [(5, [a, a + 1, a + 2, 28, 29], 0, True) for a in (19, 16, 13, 10)]
    plans = capi.plan_passes(n, "tc", ops)
    assert len(plans) == 1 and plans[0]["nops"] == len(ops)
    p = plans[0]
    assert p["tc_ops"] == 1 and p["prefetch"] == 2  # every gate in place, next tile into the free buffer
    outside = 0
    for k, pos, ctrl, diag in ops[1:]:
        for q in pos:
            outside |= (1 << q) & ~p["tile_mask"]
    assert outside, "the diagonal gates should not have needed tile bits"


def test_tensor_core_pass_keeps_three_ctas_per_sm(hqs):
    # many diagonal 5-qubit gates after a tensor-core gate: their matrices
    # would push the pass past the shared memory of three resident CTAs
    n = 30
    ops = [(5, [25, 26, 27, 28, 29], 0, False)] + [(5, [a, a + 1, a + 2, 28, 29], 0, True) for a in range(0, 15)]
    plans = capi.plan_passes(n, "tc", ops, max_ops=24)
    assert plans[0]["tc_ops"] == 1
    assert SMEM_PER_SM // (plans[0]["smem_bytes"] + 1024) >= 3
    assert sum(p["nops"] for p in plans) == len(ops)


def test_shared_outer_controls_skip_tiles(hqs):
    n = 24
    ctrl = 1 << 23
    ops = [(1, [q], ctrl, False) for q in range(4)]
    p = capi.plan_passes(n, "df", ops)[0]
    assert p["nops"] == 4 and p["fixed_mask"] == ctrl
    assert p["sweep_bytes"] == 2 * (1 << (n - 1)) * 16  # half the state


def test_prefetch_modes(hqs):
    n = 26
    # dense CUDA-core gates ping-pong between the tile buffers: staging buffer
    p = capi.plan_passes(n, "df", [(2, [0, 1], 0, False), (1, [2], 0, False)])[0]
    assert p["prefetch"] in (0, 1)
    # diagonal / scalar gates on raw FP32 tiles: in place
    p = capi.plan_passes(n, "f32", [(3, [20, 21, 22], 0, True), (0, [], 0, False)])[0]
    assert p["prefetch"] == 2


def test_invalid_gates_rejected(hqs):
    with pytest.raises(capi.HQSError):
        capi.plan_passes(10, "tc", [(2, [3, 3], 0, False)])
    with pytest.raises(capi.HQSError):
        capi.plan_passes(10, "tc", [(1, [12], 0, False)])
    with pytest.raises(capi.HQSError):
        capi.plan_passes(10, "tc", [(1, [2], 1 << 2, False)])
    with pytest.raises(capi.HQSError):
        capi.plan_passes(10, "auto", [(1, [2], 0, False)])


# ------------------------------------------------------- tensor-memory passes

def _check_umma_launch(n, L, gates, amp=16):
    tile = L["tile_mask"]
    assert bin(tile).count("1") == 12
    tmask = L["target_mask"]
    assert bin(tmask).count("1") == 5 and tmask & tile == tmask
    g = gates[L["first_op"] + L["tc_op"]]
    for p in g[1]:
        assert (tmask >> p) & 1
    assert tmask & g[2] == 0  # controls are never targets of the widened gate
    # TMA dimensions cover positions 0..n-1 in order; each starts with a run
    # of tile positions (the box, at most 256 elements) and holds no other
    # tile position above it, except the last dimension of a plan with extra
    # tile bits, whose tile positions above its run are the copies
    pos, tbits = 0, 0
    rank = L["rank"]
    assert 1 <= rank <= 5
    for i in range(rank):
        kind, p, b, bx = L["dim_kind"][i], L["dim_pos"][i], L["dim_bits"][i], L["dim_box"][i]
        assert p == pos and b >= 1 and 1 <= bx <= b
        run = ((1 << bx) - 1) << p
        above = ((1 << (b - bx)) - 1) << (p + bx)
        assert run & tile == run
        assert bx <= (7 if i == 0 else 8)
        tbits += bx
        if kind == 1:
            assert above & tile == 0
        else:
            assert kind == 2 and i == rank - 1
            assert bin(above & tile).count("1") == L["nextra"]
        pos += b
    assert pos == n
    assert tbits + L["nextra"] == 12
    assert L["box_bytes"] == amp << tbits
    assert L["sweep_bytes"] == 2 * amp << (n - bin(L["fixed_mask"]).count("1"))


@pytest.mark.parametrize("arith,amp", [("tc", 16), ("tc64", 8)])
def test_umma_launch_plans_cover_gates_and_tile(arith, amp):
    rng = np.random.default_rng(21)
    for trial in range(60):
        n = int(rng.integers(12, 35))
        gates = []
        for _ in range(int(rng.integers(1, 12))):
            kind = rng.integers(0, 4)
            k = int(rng.integers(1, 6))
            pos = [int(x) for x in rng.choice(n, size=k, replace=False)]
            ctrl = 0
            if rng.random() < 0.2:
                free = [b for b in range(n) if b not in pos]
                ctrl = 1 << int(rng.choice(free))
            gates.append((k, pos, ctrl, kind == 0))
        launches = capi.plan_launches(n, arith, gates)
        nxt = 0
        for L in launches:
            assert L["first_op"] == nxt
            nxt += L["nops"]
            if L["umma"]:
                _check_umma_launch(n, L, gates, amp)
                ops = gates[L["first_op"]:L["first_op"] + L["nops"]]
                dense = [i for i, g in enumerate(ops) if not g[3] and g[0] >= 3]
                assert dense == [L["tc_op"]]
                assert all(g[3] or g[0] == 0 or i == L["tc_op"] for i, g in enumerate(ops))
        assert nxt == len(gates)
        # every dense 3-5 qubit gate runs in a tensor-memory pass
        umma_gates = {L["first_op"] + L["tc_op"] for L in launches if L["umma"]}
        for i, g in enumerate(gates):
            if not g[3] and g[0] >= 3:
                assert i in umma_gates


def test_umma_not_used_below_twelve_qubits_or_other_arithmetic():
    gates = [(5, [0, 2, 4, 6, 8], 0, False)]
    assert not any(L["umma"] for L in capi.plan_launches(11, "tc", gates))
    for arith in ("df", "f64", "f32", "tf32"):
        assert not any(L["umma"] for L in capi.plan_launches(20, arith, gates))
    assert any(L["umma"] for L in capi.plan_launches(20, "tc", gates))
    assert any(L["umma"] for L in capi.plan_launches(20, "tc64", gates))
