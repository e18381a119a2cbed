"""NumPy FP64 statement of the learned-proposal encoder and its training step (test infrastructure only).

The learned source proposal has no counterpart in the reference: it is the approximate mode the
library adds beside the exhaustive matcher (include/tdag_nn.h). This module states, in plain FP64
NumPy with hand-derived gradients, what the library's kernels compute:

- block_masks: the 64-bit occupancy mask of every 4^3 block of an item (tdag_nn_block_masks);
- forward: the block MLP 64 -> 256 -> 256 -> 32 (ReLU after the first two layers), the mean over an
  item's non-empty blocks and the L2 normalisation (tdag_nn_gemm + tdag_nn_pool_forward);
- info_nce: the symmetric InfoNCE loss over in-batch pairs and its gradient (tdag_nn_info_nce);
- backward: every parameter's gradient (tdag_nn_pool_backward, tdag_nn_gemm with gates,
  tdag_nn_column_sums);
- adamw: one AdamW step with decoupled weight decay (tdag_nn_adamw);
- topk: the causal top-k of dot products (tdag_nn_topk).

Only the tests, __graft_entry__.smoke() and bench.py's CPU legs may import it.
"""
from __future__ import annotations

import numpy as np

EMBED_DIM = 32
HIDDEN = 256


def block_masks(words: np.ndarray, level: int) -> np.ndarray:
    """(n, R^3/64) uint64 item words (bit x + R y + R^2 z) -> (n, (R/4)^3) uint64 block masks, block
    bx + (R/4) by + (R/4)^2 bz, mask bit dx + 4 dy + 16 dz."""
    R = 1 << level
    n = words.shape[0]
    bits = np.unpackbits(words.astype("<u8").view(np.uint8).reshape(n, -1), bitorder="little").reshape(n, R, R, R)  # [z][y][x]
    b = R // 4
    blk = bits.reshape(n, b, 4, b, 4, b, 4)  # [bz, dz, by, dy, bx, dx]
    blk = blk.transpose(0, 1, 3, 5, 2, 4, 6).reshape(n, b * b * b, 64)  # block (bz, by, bx), local (dz, dy, dx)
    return np.packbits(blk, axis=-1, bitorder="little").view("<u8").reshape(n, b * b * b)


def unpack(masks: np.ndarray) -> np.ndarray:
    """(..., ) uint64 masks -> (..., 64) float64 bits."""
    m = masks.astype("<u8")
    return np.unpackbits(m.view(np.uint8).reshape(m.shape + (8,)), axis=-1, bitorder="little").astype(np.float64)


def bf16(x):
    """Round to bf16 (nearest even) and back to float64: the storage format of the kernels'
    activations, backward operands and weight copies."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return b.view(np.float32).astype(np.float64)


def _noop(x):
    return x


def init_params(seed: int = 0):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases, FP64: [w1, b1, w2, b2, w3, b3]."""
    rng = np.random.default_rng(seed)
    out = []
    for o, i in ((HIDDEN, 64), (HIDDEN, HIDDEN), (EMBED_DIM, HIDDEN)):
        bound = 1.0 / np.sqrt(i)
        out.append(rng.uniform(-bound, bound, (o, i)))
        out.append(rng.uniform(-bound, bound, (o,)))
    return out


def forward(params, masks: np.ndarray, storage=_noop):
    """masks (n, B) -> (u (n, 32), cache). `storage` rounds what the kernels store between layers
    (bf16 for the kernels' numerics, identity for exact FP64)."""
    w1, b1, w2, b2, w3, b3 = params
    n, B = masks.shape
    x = unpack(masks.reshape(-1))  # (n B, 64)
    z1 = x @ w1.T + b1
    h1 = storage(np.maximum(z1, 0.0))
    z2 = h1 @ w2.T + b2
    h2 = storage(np.maximum(z2, 0.0))
    z3 = (h2 @ w3.T + b3).reshape(n, B, EMBED_DIM)
    ne = (masks != 0).astype(np.float64)
    cnt = np.maximum(ne.sum(axis=1), 1.0)
    e = (z3 * ne[..., None]).sum(axis=1) / cnt[:, None]
    norm = np.maximum(np.linalg.norm(e, axis=1), 1e-12)
    u = e / norm[:, None]
    return u, (x, h1, h2, ne, cnt, norm, u, storage)


def info_nce(ut: np.ndarray, up: np.ndarray, tau: float, storage=_noop):
    """Symmetric InfoNCE over logits ut up^T / tau: (loss, d loss / d ut, d loss / d up). With
    `storage` the embeddings and the logit gradient are rounded as the kernels store them."""
    b = ut.shape[0]
    ut, up = storage(ut), storage(up)
    logits = ut @ up.T / tau

    def softmax(z, axis):
        z = z - z.max(axis=axis, keepdims=True)
        ez = np.exp(z)
        return ez / ez.sum(axis=axis, keepdims=True)

    def lse(z, axis):
        mx = z.max(axis=axis, keepdims=True)
        return (mx + np.log(np.exp(z - mx).sum(axis=axis, keepdims=True))).squeeze(axis)

    diag = np.diag(logits)
    loss = 0.5 * (np.mean(lse(logits, 1) - diag) + np.mean(lse(logits, 0) - diag))
    dl = storage(0.5 / b * (softmax(logits, 1) + softmax(logits, 0) - 2.0 * np.eye(b)))
    return loss, dl @ up / tau, dl.T @ ut / tau


def backward(params, cache, du: np.ndarray):
    """Gradients [gw1, gb1, gw2, gb2, gw3, gb3] from d loss / d u."""
    w1, b1, w2, b2, w3, b3 = params
    x, h1, h2, ne, cnt, norm, u, storage = cache
    n, B = ne.shape
    dot = (du * u).sum(axis=1, keepdims=True)
    de = storage((du - u * dot) / norm[:, None] / cnt[:, None])
    dz3 = (de[:, None, :] * ne[..., None]).reshape(n * B, EMBED_DIM)
    gw3 = dz3.T @ h2
    gb3 = dz3.sum(axis=0)
    dz2 = storage((dz3 @ w3) * (h2 > 0))
    gw2 = dz2.T @ h1
    gb2 = dz2.sum(axis=0)
    dz1 = storage((dz2 @ w2) * (h1 > 0))
    gw1 = dz1.T @ x
    gb1 = dz1.sum(axis=0)
    return [gw1, gb1, gw2, gb2, gw3, gb3]


def loss_of(params, masks_t: np.ndarray, masks_p: np.ndarray, tau: float, storage=_noop) -> float:
    ut, _ = forward(params, masks_t, storage)
    up, _ = forward(params, masks_p, storage)
    return info_nce(ut, up, tau, storage)[0]


def grads_of(params, masks_t: np.ndarray, masks_p: np.ndarray, tau: float, storage=_noop):
    """(loss, gradients) of the InfoNCE loss of a batch of (target, parent) pairs; storage=bf16
    states the kernels' numerics, the default the exact FP64 values."""
    ut, ct = forward(params, masks_t, storage)
    up, cp = forward(params, masks_p, storage)
    loss, dut, dup = info_nce(ut, up, tau, storage)
    gt = backward(params, ct, dut)
    gp = backward(params, cp, dup)
    return loss, [a + b for a, b in zip(gt, gp)]


def adamw(w, g, m1, m2, step: int, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, decay: float = 1e-2):
    """One AdamW step (Loshchilov & Hutter, decoupled weight decay); returns (w, m1, m2)."""
    w = w * (1.0 - lr * decay)
    m1 = beta1 * m1 + (1.0 - beta1) * g
    m2 = beta2 * m2 + (1.0 - beta2) * g * g
    c1 = 1.0 - beta1 ** step
    c2 = 1.0 - beta2 ** step
    w = w - (lr / c1) * m1 / (np.sqrt(m2) / np.sqrt(c2) + eps)
    return w, m1, m2


def topk(emb: np.ndarray, k: int):
    """For every row i, the set of the k rows j < i with the largest dot products (fewer where i < k)."""
    s = emb.astype(np.float64) @ emb.astype(np.float64).T
    out = []
    for i in range(emb.shape[0]):
        if i == 0:
            out.append(set())
            continue
        row = s[i, :i]
        take = np.argsort(-row, kind="stable")[:k]
        out.append(set(int(j) for j in take))
    return out, s


# ------------------------------------------------------------------------------------------------
# Hierarchical encoder: a 4^3 item is embedded by the leaf MLP above (no pooling); an 8^3 or 16^3
# item by an MLP 256 -> 256 -> 256 -> 32 of its level over its eight children's 32-wide vectors
# placed in a canonical octant order (tdag_nn_canon_gather). Children of an 8^3 item are its 4^3
# blocks (leaf MLP outputs), children of a 16^3 item its 8^3 octants (outputs of the 8^3 MLP).
# ------------------------------------------------------------------------------------------------
PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))  # transform ID = sym | perm << 3


def transform_tables():
    """pos[t][o]: the octant child o moves to under transform t (the axes permuted, then the mirrored
    axes flipped); byte_map[t][b]: the image of occupancy byte b (bit o = child o)."""
    pos = np.zeros((48, 8), np.int64)
    for t in range(48):
        s, p = t & 7, t >> 3
        for o in range(8):
            q = 0
            for k in range(3):
                q |= ((o >> PERMS[p][k]) & 1) << k
            pos[t, o] = q ^ s
    byte_map = np.zeros((48, 256), np.int64)
    for t in range(48):
        for b in range(256):
            byte_map[t, b] = sum(1 << int(pos[t, o]) for o in range(8) if (b >> o) & 1)
    return pos, byte_map


_POS, _BYTE_MAP = transform_tables()


def canon_slots(occupancy: np.ndarray) -> np.ndarray:
    """(m,) occupancy bytes -> (m, 8) slot of every child: its octant under the first transform that
    maps the byte to the smallest image."""
    t = np.argmin(_BYTE_MAP[:, occupancy], axis=0)  # argmin takes the first of equal minima
    return _POS[t]


def init_hier_params(seed: int = 0):
    """{'leaf', 'up3', 'up4'}: six FP64 tensors each, uniform(-1/sqrt(fan_in), 1/sqrt(fan_in))."""
    rng = np.random.default_rng(seed)
    out = {}
    for g, k_in in (("leaf", 64), ("up3", 256), ("up4", 256)):
        ps = []
        for o, i in ((HIDDEN, k_in), (HIDDEN, HIDDEN), (EMBED_DIM, HIDDEN)):
            bound = 1.0 / np.sqrt(i)
            ps.append(rng.uniform(-bound, bound, (o, i)))
            ps.append(rng.uniform(-bound, bound, (o,)))
        out[g] = ps
    return out


def _mlp(params, x, storage):
    w1, b1, w2, b2, w3, b3 = params
    h1 = storage(np.maximum(x @ w1.T + b1, 0.0))
    h2 = storage(np.maximum(h1 @ w2.T + b2, 0.0))
    return h2 @ w3.T + b3, (x, h1, h2)


def _mlp_backward(params, cache, dz, storage):
    w1, b1, w2, b2, w3, b3 = params
    x, h1, h2 = cache
    dz2 = storage((dz @ w3) * (h2 > 0))
    dz1 = storage((dz2 @ w2) * (h1 > 0))
    grads = [dz1.T @ x, dz1.sum(axis=0), dz2.T @ h1, dz2.sum(axis=0), dz.T @ h2, dz.sum(axis=0)]
    return grads, dz1 @ w1


def _gather(child, present, slots):
    """(m, 8, 32) child vectors, (m, 8) presence, (m, 8) slots -> (m, 256) canonical rows."""
    m = child.shape[0]
    x = np.zeros((m, 8, EMBED_DIM))
    for o in range(8):
        x[np.arange(m), slots[:, o]] = child[:, o] * present[:, o, None]
    return x.reshape(m, 8 * EMBED_DIM)


def _scatter(dx, present, slots):
    """Gradient of _gather: (m, 256) -> (m, 8, 32)."""
    m = dx.shape[0]
    d = dx.reshape(m, 8, EMBED_DIM)
    return np.stack([d[np.arange(m), slots[:, o]] * present[:, o, None] for o in range(8)], axis=1)


def _octant_blocks():
    """blk[q][o]: the 4^3 block (bx + 4 by + 16 bz) of sub-octant o of octant q of a 16^3 item."""
    blk = np.zeros((8, 8), np.int64)
    for q in range(8):
        for o in range(8):
            bx = 2 * (q & 1) + (o & 1)
            by = 2 * ((q >> 1) & 1) + ((o >> 1) & 1)
            bz = 2 * ((q >> 2) & 1) + ((o >> 2) & 1)
            blk[q, o] = bx + 4 * by + 16 * bz
    return blk


def hier_forward(P, masks: np.ndarray, level: int, storage=_noop):
    """(n, B) block masks of level-`level` items -> (u (n, 32), cache)."""
    n, B = masks.shape
    z0, c0 = _mlp(P["leaf"], unpack(masks.reshape(-1)), storage)  # (n B, 32)
    ne0 = masks != 0
    cache = {"level": level, "n": n, "c0": c0, "storage": storage}
    if level == 2:
        e = z0 * ne0.reshape(n, 1)
    elif level == 3:
        slots = canon_slots((ne0 * (1 << np.arange(8))).sum(axis=1))
        x3 = storage(_gather(z0.reshape(n, 8, EMBED_DIM), ne0, slots))
        e, c3 = _mlp(P["up3"], x3, storage)
        cache.update(c3=c3, ne0=ne0, slots3=slots)
    else:
        blk = _octant_blocks()
        z0b = z0.reshape(n, 64, EMBED_DIM)[:, blk].reshape(n * 8, 8, EMBED_DIM)  # sub-item (i, q), child o
        ne0b = ne0[:, blk].reshape(n * 8, 8)
        slots3 = canon_slots((ne0b * (1 << np.arange(8))).sum(axis=1))
        x3 = storage(_gather(z0b, ne0b, slots3))
        z3, c3 = _mlp(P["up3"], x3, storage)
        ne3 = ne0b.any(axis=1).reshape(n, 8)
        slots4 = canon_slots((ne3 * (1 << np.arange(8))).sum(axis=1))
        x4 = storage(_gather(z3.reshape(n, 8, EMBED_DIM), ne3, slots4))
        e, c4 = _mlp(P["up4"], x4, storage)
        cache.update(c3=c3, c4=c4, ne0b=ne0b, slots3=slots3, ne3=ne3, slots4=slots4, blk=blk)
    norm = np.maximum(np.linalg.norm(e, axis=1), 1e-12)
    u = e / norm[:, None]
    cache.update(u=u, norm=norm)
    return u, cache


def hier_backward(P, cache, du: np.ndarray):
    """{'leaf', 'up3', 'up4'} gradients (None for groups the level does not use) from d loss / d u."""
    storage, n, level, u, norm = cache["storage"], cache["n"], cache["level"], cache["u"], cache["norm"]
    dot = (du * u).sum(axis=1, keepdims=True)
    de = storage((du - u * dot) / norm[:, None])
    out = {"leaf": None, "up3": None, "up4": None}
    if level == 2:
        dz0 = de
    elif level == 3:
        out["up3"], dx3 = _mlp_backward(P["up3"], cache["c3"], de, storage)
        dz0 = storage(_scatter(dx3, cache["ne0"], cache["slots3"]).reshape(n * 8, EMBED_DIM))
    else:
        out["up4"], dx4 = _mlp_backward(P["up4"], cache["c4"], de, storage)
        dz3 = storage(_scatter(dx4, cache["ne3"], cache["slots4"]).reshape(n * 8, EMBED_DIM))
        out["up3"], dx3 = _mlp_backward(P["up3"], cache["c3"], dz3, storage)
        dz0b = _scatter(dx3, cache["ne0b"], cache["slots3"]).reshape(n, 8, 8, EMBED_DIM)  # (i, q, o)
        dz0 = np.zeros((n, 64, EMBED_DIM))
        dz0[:, cache["blk"].reshape(-1)] = dz0b.reshape(n, 64, EMBED_DIM)
        dz0 = storage(dz0.reshape(n * 64, EMBED_DIM))
    out["leaf"], _ = _mlp_backward(P["leaf"], cache["c0"], dz0, storage)
    return out


def hier_grads_of(P, masks_t: np.ndarray, masks_p: np.ndarray, level: int, tau: float, storage=_noop):
    """(loss, gradient dict) of the InfoNCE loss of (target, parent) pairs under the hierarchical encoder."""
    ut, ct = hier_forward(P, masks_t, level, storage)
    up, cp = hier_forward(P, masks_p, level, storage)
    loss, dut, dup = info_nce(ut, up, tau, storage)
    gt, gp = hier_backward(P, ct, dut), hier_backward(P, cp, dup)
    return loss, {g: (None if gt[g] is None else [a + b for a, b in zip(gt[g], gp[g])]) for g in gt}


def hier_loss_of(P, masks_t, masks_p, level, tau, storage=_noop) -> float:
    ut, _ = hier_forward(P, masks_t, level, storage)
    up, _ = hier_forward(P, masks_p, level, storage)
    return info_nce(ut, up, tau, storage)[0]
