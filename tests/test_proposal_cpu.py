"""CPU tests of the learned-proposal oracle (oracle/proposal_oracle.py), the FP64 statement the GPU
kernels of include/tdag_nn.h are checked against: block-mask layout, hand-derived gradients against
finite differences, the AdamW step against its definition, and the causal top-k; plus the host-side
orders and baselines of tdag.proposal."""
import numpy as np
import pytest

from oracle import proposal_oracle as PO

torch = pytest.importorskip("torch")


def random_words(n, level, seed, density=0.3):
    rng = np.random.default_rng(seed)
    R = 1 << level
    bits = rng.random((n, R * R * R)) < density
    words = np.packbits(bits.reshape(n, -1), axis=-1, bitorder="little").view("<u8").reshape(n, -1)
    return words, bits


@pytest.mark.parametrize("level", [2, 3, 4])
def test_block_masks_layout(level):
    words, bits = random_words(3, level, level)
    masks = PO.block_masks(words, level)
    R, b = 1 << level, (1 << level) // 4
    assert masks.shape == (3, b ** 3)
    rng = np.random.default_rng(1)
    for i in range(3):
        for _ in range(40):
            x, y, z = (int(v) for v in rng.integers(0, R, 3))
            blk = x // 4 + b * (y // 4) + b * b * (z // 4)
            local = x % 4 + 4 * (y % 4) + 16 * (z % 4)
            assert ((int(masks[i, blk]) >> local) & 1) == int(bits[i, x + R * y + R * R * z])


def _batch(seed=4, B=6, level=3):
    params = PO.init_params(seed)
    words, _ = random_words(2 * B, level, seed)
    masks = PO.block_masks(words, level)
    return params, masks[:B], masks[B:]


def test_gradients_match_finite_differences_fp64():
    params, mt, mp = _batch()
    tau = 0.07
    loss, grads = PO.grads_of(params, mt, mp, tau)
    assert np.isfinite(loss)
    rng = np.random.default_rng(7)
    eps = 1e-6
    for pi, p in enumerate(params):
        for _ in range(6):
            idx = tuple(int(rng.integers(s)) for s in p.shape)
            plus = [q.copy() for q in params]
            minus = [q.copy() for q in params]
            plus[pi][idx] += eps
            minus[pi][idx] -= eps
            fd = (PO.loss_of(plus, mt, mp, tau) - PO.loss_of(minus, mt, mp, tau)) / (2 * eps)
            assert abs(grads[pi][idx] - fd) <= 1e-6 + 1e-5 * abs(fd), (pi, idx, grads[pi][idx], fd)


def test_info_nce_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    ut = rng.normal(size=(5, 32))
    up = rng.normal(size=(5, 32))
    loss, gt, gp = PO.info_nce(ut, up, 0.1)
    eps = 1e-6
    for (arr, g) in ((ut, gt), (up, gp)):
        for _ in range(5):
            i, d = int(rng.integers(5)), int(rng.integers(32))
            arr[i, d] += eps
            lp = PO.info_nce(ut, up, 0.1)[0]
            arr[i, d] -= 2 * eps
            lm = PO.info_nce(ut, up, 0.1)[0]
            arr[i, d] += eps
            assert abs((lp - lm) / (2 * eps) - g[i, d]) < 1e-6


def test_adamw_step_definition():
    rng = np.random.default_rng(5)
    w, g = rng.normal(size=10), rng.normal(size=10)
    m1, m2 = np.zeros(10), np.zeros(10)
    w1, a, v = PO.adamw(w, g, m1, m2, 1, lr=1e-2, decay=0.1)
    # step 1: bias-corrected moments are g and g^2, so the step is lr * g / (|g| + eps) after the decay
    assert np.allclose(w1, w * (1 - 1e-3) - 1e-2 * g / (np.abs(g) + 1e-8))
    assert np.allclose(a, 0.1 * g) and np.allclose(v, 0.001 * g * g)


def test_topk_is_causal_and_best():
    rng = np.random.default_rng(2)
    e = rng.normal(size=(40, 32))
    sets, s = PO.topk(e, 4)
    assert sets[0] == set() and sets[1] == {0} and len(sets[3]) == 3
    for i in range(5, 40):
        assert all(j < i for j in sets[i]) and len(sets[i]) == 4
        worst_in = min(s[i, j] for j in sets[i])
        assert all(s[i, j] <= worst_in for j in range(i) if j not in sets[i])


def test_popcount_positions_order():
    from tdag import proposal as P
    words, bits = random_words(50, 2, 2)
    pos = P.popcount_positions(torch.from_numpy(words.view(np.int64))).numpy()
    pc = bits.sum(axis=1)
    order = sorted(range(50), key=lambda i: (-pc[i], i))
    assert [int(p) for p in pos[order]] == list(range(50))


def test_baseline_lists_only_propose_predecessors():
    from tdag import proposal as P
    words, _ = random_words(300, 3, 3)
    pos = P.popcount_positions(torch.from_numpy(words.view(np.int64)))
    for lists in (P.popcount_neighbour_lists(pos, 8), P.random_lists(pos, 8)):
        ok = lists >= 0
        src = lists.clamp(min=0)
        assert bool((pos[src][ok] < pos.unsqueeze(1).expand_as(lists)[ok]).all())
    assert P.sources_of(P.popcount_neighbour_lists(pos, 1)).numel() == 299  # every item but the last one


def test_transform_tables_match_the_library_layout():
    """The oracle's octant tables: transform 0 is the identity, the 48 transforms of a byte's orbit
    are distinct permutations of the octants, and canon_slots picks the first smallest image."""
    pos, byte_map = PO.transform_tables()
    assert list(pos[0]) == list(range(8))
    assert all(sorted(pos[t]) == list(range(8)) for t in range(48))
    assert len({tuple(pos[t]) for t in range(48)}) == 48
    occ = np.arange(256)
    slots = PO.canon_slots(occ)
    for b in (0, 1, 0x80, 0x5A, 0xFF, 0x37):
        t = min(range(48), key=lambda k: (byte_map[k, b], k))
        assert list(slots[b]) == list(pos[t])
        assert sum(1 << int(slots[b][o]) for o in range(8) if (b >> o) & 1) == byte_map[:, b].min()


def test_canonical_slots_are_transform_invariant():
    """Two items whose child occupancies are transforms of each other get the same canonical byte."""
    pos, byte_map = PO.transform_tables()
    rng = np.random.default_rng(2)
    for _ in range(30):
        b = int(rng.integers(1, 256))
        t = int(rng.integers(48))
        bt = int(byte_map[t, b])
        sb, st = PO.canon_slots(np.array([b, bt]))
        img = lambda byte, s: sum(1 << int(s[o]) for o in range(8) if (byte >> o) & 1)  # noqa: E731
        assert img(b, sb) == img(bt, st)


@pytest.mark.parametrize("level", [2, 3, 4])
def test_hierarchical_gradients_match_finite_differences_fp64(level):
    P = PO.init_hier_params(3)
    n = 5
    words, _ = random_words(2 * n, level, 10 + level, density=0.2 if level < 4 else 0.05)
    masks = PO.block_masks(words, level)
    mt, mp = masks[:n], masks[n:]
    tau = 0.1
    loss, grads = PO.hier_grads_of(P, mt, mp, level, tau)
    assert np.isfinite(loss)
    used = {2: ["leaf"], 3: ["leaf", "up3"], 4: ["leaf", "up3", "up4"]}[level]
    assert all(grads[g] is not None for g in used) and all(grads[g] is None for g in grads if g not in used)
    rng = np.random.default_rng(level)
    eps = 1e-6
    for g in used:
        for pi in range(6):
            p = P[g][pi]
            for _ in range(2):
                idx = tuple(int(rng.integers(s)) for s in p.shape)
                plus = {k: [q.copy() for q in v] for k, v in P.items()}
                minus = {k: [q.copy() for q in v] for k, v in P.items()}
                plus[g][pi][idx] += eps
                minus[g][pi][idx] -= eps
                fd = (PO.hier_loss_of(plus, mt, mp, level, tau) - PO.hier_loss_of(minus, mt, mp, level, tau)) / (2 * eps)
                assert abs(grads[g][pi][idx] - fd) <= 1e-6 + 1e-5 * abs(fd), (g, pi, idx, grads[g][pi][idx], fd)
