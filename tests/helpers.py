"""Test helpers: seeded inputs built with the oracle's SVO builder and toDAG."""
import numpy as np


def random_grid(res, density, seed):
    rng = np.random.default_rng(seed)
    return (rng.random((res, res, res)) < density).astype(np.uint8)


def blocky_grid(res, seed, n_boxes=12, max_side=None):
    """Union of random boxes plus mirrored/translated copies: many exact matches."""
    rng = np.random.default_rng(seed)
    g = np.zeros((res, res, res), np.uint8)
    max_side = max_side or max(2, res // 3)
    for _ in range(n_boxes):
        s = rng.integers(1, max_side + 1, size=3)
        o = [rng.integers(0, res - s[k] + 1) for k in range(3)]
        g[o[2]:o[2] + s[2], o[1]:o[1] + s[1], o[0]:o[0] + s[0]] = 1
    # copy an octant with a mirror and a shift, to create transform matches
    h = res // 2
    block = g[:h, :h, :h].copy()
    g[h:, h:, :h] |= block[:, ::-1, :]
    g[:h, h:, h:] |= np.transpose(block, (1, 0, 2))
    return g


def dag_svo_bytes(oracle, dense):
    return oracle.to_dag(oracle.svo_from_dense(dense))


def structure_from_svo(tdag_mod, svo_bytes):
    return tdag_mod.EditStructure.from_svo_bytes(svo_bytes)
