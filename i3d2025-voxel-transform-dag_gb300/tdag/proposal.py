"""Learned proposal of translation-matching sources (an approximate mode; no counterpart in the reference).

The exhaustive search lets every item of a translation level search as a source. Here an encoder
embeds every item, each target proposes the k most similar items that precede it in the popcount
order, and only the proposed items search. The library verifies every match exactly
(tdag_build_device_proposed, tdag_find_duplicates_level_device), so the result is always a valid
TDAG. Its node count can only grow against the exhaustive build: that growth is the "extra nodes"
this mode trades for speed.

Encoder: every 4^3 block of an item -- its 64-bit occupancy mask read as 64 bf16 inputs, bit
dx + 4 dy + 16 dz -- goes through an MLP 64 -> 256 -> 256 -> 32. An item's embedding is the mean
over its non-empty blocks ((R/4)^3 = 1, 8, 64 blocks at levels 2, 3, 4), L2-normalised. Training:
symmetric InfoNCE over (target, exhaustive parent) pairs from the exhaustive GPU matcher with
in-batch negatives, AdamW on FP32 master weights.

Every arithmetic step runs in the library's own kernels (include/tdag_nn.h): the dense layers
forward and backward, the InfoNCE logits and the candidate scoring are bf16 GEMMs on the tcgen05
tensor cores with FP32 accumulation (bias, ReLU and the ReLU gate fused into their epilogues); block
masks, pooling, the loss, bias gradients and AdamW are plain CUDA kernels. PyTorch only holds the
device memory and orders the items.
"""
from __future__ import annotations

import ctypes
import math
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _abi
from ._abi import lib

EMBED_DIM = 32
HIDDEN = 256
PTR_MASK = (1 << 37) - 1
LAYERS = ((HIDDEN, 64), (HIDDEN, HIDDEN), (EMBED_DIM, HIDDEN))  # (out, in) of every dense layer


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else t.data_ptr()


def _op(t, mode: int, ld: int = 0) -> _abi.NnOperand:
    return _abi.NnOperand(t.data_ptr(), mode, ld)


def _ctx(ctx):
    if ctx is None:
        from . import default_context
        ctx = default_context()
    return ctx


def gemm(ctx, a: _abi.NnOperand, b: _abi.NnOperand, m: int, n: int, k: int, out: torch.Tensor, alpha: float = 1.0,
         bias: Optional[torch.Tensor] = None, relu: bool = False, gate: Optional[torch.Tensor] = None) -> torch.Tensor:
    """out (m x n, FP32 or bf16) = epilogue(alpha * A B^T) on the tensor cores (tdag_nn_gemm)."""
    _abi.check(lib().tdag_nn_gemm(_ctx(ctx).handle, ctypes.byref(a), ctypes.byref(b), m, n, k, alpha, _ptr(bias), int(relu), _ptr(gate),
                                  n if gate is not None else 0, out.data_ptr(), out.stride(0), int(out.dtype == torch.bfloat16)))
    return out


def block_masks(ctx, words: torch.Tensor, level: int) -> torch.Tensor:
    """(n, (R/4)^3) int64 block masks of n items (tdag_nn_block_masks)."""
    n = words.shape[0]
    B = ((1 << level) // 4) ** 3
    masks = torch.empty((n, B), dtype=torch.int64, device=words.device)
    _abi.check(lib().tdag_nn_block_masks(_ctx(ctx).handle, words.contiguous().data_ptr(), n, level, masks.data_ptr()))
    return masks


class ProposalEncoder:
    """Leaf-block MLP 64 -> 256 -> 256 -> 32 with mean pooling over an item's non-empty 4^3 blocks,
    on the library's kernels. Parameters: FP32 master weights (out x in) and biases, their bf16
    copies (the GEMM operands) and the AdamW moments, all on one device."""

    def __init__(self, device=None, seed: int = 0, ctx=None):
        self.ctx = _ctx(ctx)
        self.device = torch.device("cuda", self.ctx.device) if device is None else torch.device(device)
        g = torch.Generator(device="cpu").manual_seed(seed)
        params = []
        for o, i in LAYERS:  # uniform(-1/sqrt(fan_in), 1/sqrt(fan_in))
            bound = 1.0 / math.sqrt(i)
            params.append((torch.rand((o, i), generator=g, dtype=torch.float64) * 2 - 1) * bound)
            params.append((torch.rand((o,), generator=g, dtype=torch.float64) * 2 - 1) * bound)
        self.load(params)

    def load(self, params: Sequence) -> "ProposalEncoder":
        """Set the six parameters [w1, b1, w2, b2, w3, b3] (any array type) and reset AdamW."""
        self.params = [torch.as_tensor(p).to(device=self.device, dtype=torch.float32).contiguous() for p in params]
        self.w16 = [self.params[2 * l].to(torch.bfloat16) for l in range(3)]
        self.m1 = [torch.zeros_like(p) for p in self.params]
        self.m2 = [torch.zeros_like(p) for p in self.params]
        self.step_count = 0
        return self

    def numpy_params(self):
        return [p.double().cpu().numpy() for p in self.params]

    # ---- forward / backward
    def forward(self, words: torch.Tensor, level: int, keep: bool = False):
        """u (n x 32, FP32, L2-normalised) of n items; with keep, also the cache for backward()."""
        masks = block_masks(self.ctx, words, level)
        return self.forward_masks(masks, keep)

    def _mlp(self, flat: torch.Tensor):
        """The block MLP over a padded column of masks: (h1, h2, z)."""
        ctx, dev = self.ctx, self.device
        rows_p = flat.shape[0]
        h1 = torch.empty((rows_p, HIDDEN), dtype=torch.bfloat16, device=dev)
        h2 = torch.empty((rows_p, HIDDEN), dtype=torch.bfloat16, device=dev)
        z = torch.empty((rows_p, EMBED_DIM), dtype=torch.float32, device=dev)
        gemm(ctx, _op(flat, _abi.NN_BITS), _op(self.w16[0], _abi.NN_KMAJOR, 64), rows_p, HIDDEN, 64, h1, bias=self.params[1], relu=True)
        gemm(ctx, _op(h1, _abi.NN_KMAJOR, HIDDEN), _op(self.w16[1], _abi.NN_KMAJOR, HIDDEN), rows_p, HIDDEN, HIDDEN, h2, bias=self.params[3],
             relu=True)
        gemm(ctx, _op(h2, _abi.NN_KMAJOR, HIDDEN), _op(self.w16[2], _abi.NN_KMAJOR, HIDDEN), rows_p, EMBED_DIM, HIDDEN, z, bias=self.params[5])
        return h1, h2, z

    @staticmethod
    def _padded(col: torch.Tensor) -> torch.Tensor:
        rows_p = max(16, (col.numel() + 15) // 16 * 16)  # the weight gradients contract over rows: a multiple of 16
        flat = torch.zeros(rows_p, dtype=torch.int64, device=col.device)
        flat[:col.numel()] = col.reshape(-1)
        return flat

    def forward_masks(self, masks: torch.Tensor, keep: bool = False):
        """u and its bf16 copy from (n, B) block masks. Without keep (inference) the MLP runs once per
        distinct mask -- its output depends on the mask alone -- and pooling gathers the rows."""
        ctx, dev = self.ctx, self.device
        n, B = masks.shape
        if keep:
            flat = self._padded(masks)
            row_of = None
        else:
            uniq, inv = torch.unique(masks.reshape(-1), return_inverse=True)
            flat = self._padded(uniq)
            row_of = inv.to(torch.int32).contiguous()
        h1, h2, z = self._mlp(flat)
        u = torch.empty((n, EMBED_DIM), dtype=torch.float32, device=dev)
        ub = torch.empty((n, EMBED_DIM), dtype=torch.bfloat16, device=dev)
        norm = torch.empty(n, dtype=torch.float32, device=dev)
        count = torch.empty(n, dtype=torch.float32, device=dev)
        mk = masks.contiguous()
        _abi.check(lib().tdag_nn_pool_forward(ctx.handle, z.data_ptr(), _ptr(row_of), mk.data_ptr(), n, B, u.data_ptr(), ub.data_ptr(),
                                              norm.data_ptr(), count.data_ptr()))
        if not keep:
            return u, ub
        return u, ub, {"masks": flat, "h1": h1, "h2": h2, "u": u, "norm": norm, "count": count, "n": n, "B": B, "rows_p": flat.shape[0]}

    def backward(self, cache: dict, du: torch.Tensor) -> List[torch.Tensor]:
        """FP32 gradients [gw1, gb1, gw2, gb2, gw3, gb3] from d loss / d u (n x 32, FP32)."""
        ctx, dev = self.ctx, self.device
        n, B, rows_p = cache["n"], cache["B"], cache["rows_p"]
        h1, h2, flat = cache["h1"], cache["h2"], cache["masks"]
        dz3 = torch.zeros((rows_p, EMBED_DIM), dtype=torch.bfloat16, device=dev)
        _abi.check(lib().tdag_nn_pool_backward(ctx.handle, du.contiguous().data_ptr(), cache["u"].data_ptr(), cache["norm"].data_ptr(),
                                               cache["count"].data_ptr(), flat.data_ptr(), n, B, dz3.data_ptr()))
        grads = [None] * 6
        grads[4] = gemm(ctx, _op(dz3, _abi.NN_MNMAJOR, EMBED_DIM), _op(h2, _abi.NN_MNMAJOR, HIDDEN), EMBED_DIM, HIDDEN, rows_p,
                        torch.empty((EMBED_DIM, HIDDEN), dtype=torch.float32, device=dev))
        grads[5] = self._column_sums(dz3)
        dz2 = gemm(ctx, _op(dz3, _abi.NN_KMAJOR, EMBED_DIM), _op(self.w16[2], _abi.NN_MNMAJOR, HIDDEN), rows_p, HIDDEN, EMBED_DIM,
                   torch.empty((rows_p, HIDDEN), dtype=torch.bfloat16, device=dev), gate=h2)
        grads[2] = gemm(ctx, _op(dz2, _abi.NN_MNMAJOR, HIDDEN), _op(h1, _abi.NN_MNMAJOR, HIDDEN), HIDDEN, HIDDEN, rows_p,
                        torch.empty((HIDDEN, HIDDEN), dtype=torch.float32, device=dev))
        grads[3] = self._column_sums(dz2)
        dz1 = gemm(ctx, _op(dz2, _abi.NN_KMAJOR, HIDDEN), _op(self.w16[1], _abi.NN_MNMAJOR, HIDDEN), rows_p, HIDDEN, HIDDEN,
                   torch.empty((rows_p, HIDDEN), dtype=torch.bfloat16, device=dev), gate=h1)
        grads[0] = gemm(ctx, _op(dz1, _abi.NN_MNMAJOR, HIDDEN), _op(flat, _abi.NN_BITS_T), HIDDEN, 64, rows_p,
                        torch.empty((HIDDEN, 64), dtype=torch.float32, device=dev))
        grads[1] = self._column_sums(dz1)
        return grads

    def _column_sums(self, x: torch.Tensor) -> torch.Tensor:
        out = torch.empty(x.shape[1], dtype=torch.float32, device=self.device)
        _abi.check(lib().tdag_nn_column_sums(self.ctx.handle, x.data_ptr(), x.shape[0], x.shape[1], x.stride(0), out.data_ptr()))
        return out

    # ---- training
    def loss_and_grads(self, words_t: torch.Tensor, words_p: torch.Tensor, level: int, tau: float):
        """(loss tensor on the device, gradients) of the symmetric InfoNCE of b (target, parent) pairs;
        b must be a multiple of 16."""
        b = words_t.shape[0]
        assert b % 16 == 0 and b == words_p.shape[0]
        dev = self.device
        u, ub, cache = self.forward(torch.cat([words_t, words_p]), level, keep=True)
        logits = torch.empty((b, b), dtype=torch.float32, device=dev)
        gemm(self.ctx, _op(ub[:b], _abi.NN_KMAJOR, EMBED_DIM), _op(ub[b:], _abi.NN_KMAJOR, EMBED_DIM), b, b, EMBED_DIM, logits, alpha=1.0 / tau)
        loss = torch.empty(1, dtype=torch.float32, device=dev)
        dl = torch.empty((b, b), dtype=torch.bfloat16, device=dev)
        _abi.check(lib().tdag_nn_info_nce(self.ctx.handle, logits.data_ptr(), b, loss.data_ptr(), dl.data_ptr()))
        du = torch.empty((2 * b, EMBED_DIM), dtype=torch.float32, device=dev)
        gemm(self.ctx, _op(dl, _abi.NN_KMAJOR, b), _op(ub[b:], _abi.NN_MNMAJOR, EMBED_DIM), b, EMBED_DIM, b, du[:b], alpha=1.0 / tau)
        gemm(self.ctx, _op(dl, _abi.NN_MNMAJOR, b), _op(ub[:b], _abi.NN_MNMAJOR, EMBED_DIM), b, EMBED_DIM, b, du[b:], alpha=1.0 / tau)
        return loss, self.backward(cache, du)

    def adamw_step(self, grads: Sequence[torch.Tensor], lr: float, weight_decay: float = 1e-2, beta1: float = 0.9, beta2: float = 0.999,
                   eps: float = 1e-8) -> None:
        self.step_count += 1
        for i, (p, g) in enumerate(zip(self.params, grads)):
            w16 = self.w16[i // 2] if i % 2 == 0 else None
            decay = weight_decay
            _abi.check(lib().tdag_nn_adamw(self.ctx.handle, p.data_ptr(), g.contiguous().data_ptr(), self.m1[i].data_ptr(), self.m2[i].data_ptr(),
                                           p.numel(), lr, beta1, beta2, eps, decay, self.step_count, _ptr(w16)))

    def sync(self) -> None:
        """Waits for the queued kernels; raises on a tensor-core wait past its bound."""
        _abi.check(lib().tdag_nn_sync(self.ctx.handle))


UP_LAYERS = ((HIDDEN, 8 * EMBED_DIM), (HIDDEN, HIDDEN), (EMBED_DIM, HIDDEN))  # the upper levels' MLPs
GROUPS = (("leaf", LAYERS), ("up3", UP_LAYERS), ("up4", UP_LAYERS))


def _octant_blocks(device) -> torch.Tensor:
    """(8, 8): the 4^3 block (bx + 4 by + 16 bz) of sub-octant o of octant q of a 16^3 item."""
    blk = torch.empty((8, 8), dtype=torch.int64)
    for q in range(8):
        for o in range(8):
            bx, by, bz = 2 * (q & 1) + (o & 1), 2 * ((q >> 1) & 1) + ((o >> 1) & 1), 2 * ((q >> 2) & 1) + ((o >> 2) & 1)
            blk[q, o] = bx + 4 * by + 16 * bz
    return blk.to(device)


class HierarchicalEncoder:
    """The configured encoder: a 4^3 item (level 2) is embedded by the leaf MLP 64 -> 256 -> 256 -> 32
    over its occupancy mask; an 8^3 or 16^3 item by an MLP 256 -> 256 -> 256 -> 32 of its level
    ('up3', 'up4') over its eight children's vectors in a canonical octant order
    (tdag_nn_canon_gather): the children of an 8^3 item are its 4^3 blocks (leaf MLP outputs), those of
    a 16^3 item its 8^3 octants (outputs of the 8^3 MLP). The embedding is L2-normalised. Same kernels,
    training loop and interface as ProposalEncoder; gradients of all three MLPs flow through the
    canonical gathers (tdag_nn_canon_scatter)."""

    def __init__(self, device=None, seed: int = 0, ctx=None):
        self.ctx = _ctx(ctx)
        self.device = torch.device("cuda", self.ctx.device) if device is None else torch.device(device)
        g = torch.Generator(device="cpu").manual_seed(seed)
        params = {}
        for name, layers in GROUPS:
            ps = []
            for o, i in layers:
                bound = 1.0 / math.sqrt(i)
                ps.append((torch.rand((o, i), generator=g, dtype=torch.float64) * 2 - 1) * bound)
                ps.append((torch.rand((o,), generator=g, dtype=torch.float64) * 2 - 1) * bound)
            params[name] = ps
        self.load(params)
        self._blk = _octant_blocks(self.device)

    def load(self, params: Dict[str, Sequence]) -> "HierarchicalEncoder":
        """Set every group's six parameters [w1, b1, w2, b2, w3, b3] and reset AdamW."""
        self.params = {g: [torch.as_tensor(p).to(device=self.device, dtype=torch.float32).contiguous() for p in ps] for g, ps in params.items()}
        self.w16 = {g: [ps[2 * l].to(torch.bfloat16) for l in range(3)] for g, ps in self.params.items()}
        self.m1 = {g: [torch.zeros_like(p) for p in ps] for g, ps in self.params.items()}
        self.m2 = {g: [torch.zeros_like(p) for p in ps] for g, ps in self.params.items()}
        self.step_count = 0
        return self

    def numpy_params(self):
        return {g: [p.double().cpu().numpy() for p in ps] for g, ps in self.params.items()}

    # ---- pieces
    def _mlp(self, g: str, op_in: _abi.NnOperand, rows_p: int, k_in: int):
        ctx, dev, P, W = self.ctx, self.device, self.params[g], self.w16[g]
        h1 = torch.empty((rows_p, HIDDEN), dtype=torch.bfloat16, device=dev)
        h2 = torch.empty((rows_p, HIDDEN), dtype=torch.bfloat16, device=dev)
        z = torch.empty((rows_p, EMBED_DIM), dtype=torch.float32, device=dev)
        gemm(ctx, op_in, _op(W[0], _abi.NN_KMAJOR, k_in), rows_p, HIDDEN, k_in, h1, bias=P[1], relu=True)
        gemm(ctx, _op(h1, _abi.NN_KMAJOR, HIDDEN), _op(W[1], _abi.NN_KMAJOR, HIDDEN), rows_p, HIDDEN, HIDDEN, h2, bias=P[3], relu=True)
        gemm(ctx, _op(h2, _abi.NN_KMAJOR, HIDDEN), _op(W[2], _abi.NN_KMAJOR, HIDDEN), rows_p, EMBED_DIM, HIDDEN, z, bias=P[5])
        return h1, h2, z

    def _mlp_backward(self, g: str, x_in: torch.Tensor, h1, h2, dz: torch.Tensor, rows_p: int, want_dx: bool):
        """Gradients of group g from dz (bf16, rows_p x 32); x_in: the masks (leaf) or the bf16 input
        rows (upper). With want_dx also d loss / d input (FP32, rows_p x 256)."""
        ctx, dev, W = self.ctx, self.device, self.w16[g]
        grads = [None] * 6
        grads[4] = gemm(ctx, _op(dz, _abi.NN_MNMAJOR, EMBED_DIM), _op(h2, _abi.NN_MNMAJOR, HIDDEN), EMBED_DIM, HIDDEN, rows_p,
                        torch.empty((EMBED_DIM, HIDDEN), dtype=torch.float32, device=dev))
        grads[5] = self._column_sums(dz)
        dz2 = gemm(ctx, _op(dz, _abi.NN_KMAJOR, EMBED_DIM), _op(W[2], _abi.NN_MNMAJOR, HIDDEN), rows_p, HIDDEN, EMBED_DIM,
                   torch.empty((rows_p, HIDDEN), dtype=torch.bfloat16, device=dev), gate=h2)
        grads[2] = gemm(ctx, _op(dz2, _abi.NN_MNMAJOR, HIDDEN), _op(h1, _abi.NN_MNMAJOR, HIDDEN), HIDDEN, HIDDEN, rows_p,
                        torch.empty((HIDDEN, HIDDEN), dtype=torch.float32, device=dev))
        grads[3] = self._column_sums(dz2)
        dz1 = gemm(ctx, _op(dz2, _abi.NN_KMAJOR, HIDDEN), _op(W[1], _abi.NN_MNMAJOR, HIDDEN), rows_p, HIDDEN, HIDDEN,
                   torch.empty((rows_p, HIDDEN), dtype=torch.bfloat16, device=dev), gate=h1)
        if g == "leaf":
            grads[0] = gemm(ctx, _op(dz1, _abi.NN_MNMAJOR, HIDDEN), _op(x_in, _abi.NN_BITS_T), HIDDEN, 64, rows_p,
                            torch.empty((HIDDEN, 64), dtype=torch.float32, device=dev))
        else:
            grads[0] = gemm(ctx, _op(dz1, _abi.NN_MNMAJOR, HIDDEN), _op(x_in, _abi.NN_MNMAJOR, 8 * EMBED_DIM), HIDDEN, 8 * EMBED_DIM, rows_p,
                            torch.empty((HIDDEN, 8 * EMBED_DIM), dtype=torch.float32, device=dev))
        grads[1] = self._column_sums(dz1)
        dx = None
        if want_dx:
            dx = gemm(ctx, _op(dz1, _abi.NN_KMAJOR, HIDDEN), _op(W[0], _abi.NN_MNMAJOR, 8 * EMBED_DIM), rows_p, 8 * EMBED_DIM, HIDDEN,
                      torch.empty((rows_p, 8 * EMBED_DIM), dtype=torch.float32, device=dev))
        return grads, dx

    def _column_sums(self, x: torch.Tensor) -> torch.Tensor:
        out = torch.empty(x.shape[1], dtype=torch.float32, device=self.device)
        _abi.check(lib().tdag_nn_column_sums(self.ctx.handle, x.data_ptr(), x.shape[0], x.shape[1], x.stride(0), out.data_ptr()))
        return out

    def _gather(self, child: torch.Tensor, child_row: torch.Tensor, m: int):
        """(pad16(m) x 256) bf16 canonical rows (zero padding) and the (m x 8) slots."""
        x = torch.zeros((max(16, (m + 15) // 16 * 16), 8 * EMBED_DIM), dtype=torch.bfloat16, device=self.device)
        slot = torch.empty((max(m, 1), 8), dtype=torch.uint8, device=self.device)
        cr = child_row.to(torch.int32).contiguous()
        _abi.check(lib().tdag_nn_canon_gather(self.ctx.handle, child.data_ptr(), child.shape[0], cr.data_ptr(), m, x.data_ptr(), slot.data_ptr()))
        return x, slot, cr

    def _scatter(self, dx: torch.Tensor, cr: torch.Tensor, slot: torch.Tensor, m: int, rows: int) -> torch.Tensor:
        """d loss / d child rows (bf16, rows x 32) from d loss / d canonical rows."""
        dchild = torch.zeros((rows, EMBED_DIM), dtype=torch.float32, device=self.device)
        _abi.check(lib().tdag_nn_canon_scatter(self.ctx.handle, dx.data_ptr(), 0, cr.data_ptr(), slot.data_ptr(), m, dchild.data_ptr(), rows))
        out = torch.empty((rows, EMBED_DIM), dtype=torch.bfloat16, device=self.device)
        _abi.check(lib().tdag_nn_to_bf16(self.ctx.handle, dchild.data_ptr(), dchild.numel(), out.data_ptr()))
        return out

    # ---- forward / backward
    def forward(self, words: torch.Tensor, level: int, keep: bool = False):
        """u (n x 32, FP32, L2-normalised) of n items of `level`; with keep, also the cache for backward()."""
        ctx, dev = self.ctx, self.device
        masks = block_masks(ctx, words, level)
        n, B = masks.shape
        if keep:  # one leaf row per block
            flat = ProposalEncoder._padded(masks)
            leaf_row = torch.arange(n * B, device=dev)
        else:  # the leaf MLP once per distinct mask
            uniq, inv = torch.unique(masks.reshape(-1), return_inverse=True)
            flat = ProposalEncoder._padded(uniq)
            leaf_row = inv
        h1, h2, z0 = self._mlp("leaf", _op(flat, _abi.NN_BITS), flat.shape[0], 64)
        cache = {"level": level, "n": n, "leaf": (flat, h1, h2)}
        present = (masks != 0).reshape(-1)
        child_row = torch.where(present, leaf_row, torch.full_like(leaf_row, -1))
        if level == 2:
            top = z0
            top_row = child_row.to(torch.int32)
        elif level == 3:
            x3, slot3, cr3 = self._gather(z0, child_row.reshape(n, 8), n)
            a1, a2, top = self._mlp("up3", _op(x3, _abi.NN_KMAJOR, 8 * EMBED_DIM), x3.shape[0], 8 * EMBED_DIM)
            cache.update(up3=(x3, a1, a2), g3=(cr3, slot3, n, z0.shape[0]))
            top_row = None
        else:
            cr = child_row.reshape(n, 64)[:, self._blk].reshape(n * 8, 8)  # sub-item (i, q), child o
            x3, slot3, cr3 = self._gather(z0, cr, n * 8)
            a1, a2, z3 = self._mlp("up3", _op(x3, _abi.NN_KMAJOR, 8 * EMBED_DIM), x3.shape[0], 8 * EMBED_DIM)
            sub = torch.arange(n * 8, device=dev)
            cr4 = torch.where((cr >= 0).any(dim=1), sub, torch.full_like(sub, -1)).reshape(n, 8)
            x4, slot4, cr4 = self._gather(z3, cr4, n)
            b1, b2, top = self._mlp("up4", _op(x4, _abi.NN_KMAJOR, 8 * EMBED_DIM), x4.shape[0], 8 * EMBED_DIM)
            cache.update(up3=(x3, a1, a2), g3=(cr3, slot3, n * 8, z0.shape[0]), up4=(x4, b1, b2), g4=(cr4, slot4, n, z3.shape[0]))
            top_row = None
        # L2 normalisation: a one-block pool over the top output's rows
        ones = torch.ones(n, dtype=torch.int64, device=dev) if top_row is None else masks.reshape(n).contiguous()
        u = torch.empty((n, EMBED_DIM), dtype=torch.float32, device=dev)
        ub = torch.empty((n, EMBED_DIM), dtype=torch.bfloat16, device=dev)
        norm = torch.empty(n, dtype=torch.float32, device=dev)
        count = torch.empty(n, dtype=torch.float32, device=dev)
        ro = None if top_row is None else top_row.clamp(min=0).contiguous()
        _abi.check(lib().tdag_nn_pool_forward(ctx.handle, top.data_ptr(), _ptr(ro), ones.data_ptr(), n, 1, u.data_ptr(), ub.data_ptr(),
                                              norm.data_ptr(), count.data_ptr()))
        if not keep:
            return u, ub
        cache.update(u=u, norm=norm, count=count, ones=ones, top_rows=top.shape[0])
        return u, ub, cache

    def backward(self, cache: dict, du: torch.Tensor) -> Dict[str, Optional[List[torch.Tensor]]]:
        """FP32 gradients per group from d loss / d u (n x 32, FP32); None for groups the level does not use."""
        ctx, dev, n, level = self.ctx, self.device, cache["n"], cache["level"]
        dz = torch.zeros((cache["top_rows"], EMBED_DIM), dtype=torch.bfloat16, device=dev)
        _abi.check(lib().tdag_nn_pool_backward(ctx.handle, du.contiguous().data_ptr(), cache["u"].data_ptr(), cache["norm"].data_ptr(),
                                               cache["count"].data_ptr(), cache["ones"].data_ptr(), n, 1, dz.data_ptr()))
        out = {"leaf": None, "up3": None, "up4": None}
        if level == 4:
            x4, b1, b2 = cache["up4"]
            out["up4"], dx4 = self._mlp_backward("up4", x4, b1, b2, dz, x4.shape[0], True)
            cr4, slot4, m4, rows4 = cache["g4"]
            dz = self._scatter(dx4, cr4, slot4, m4, rows4)
        if level >= 3:
            x3, a1, a2 = cache["up3"]
            out["up3"], dx3 = self._mlp_backward("up3", x3, a1, a2, dz, x3.shape[0], True)
            cr3, slot3, m3, rows3 = cache["g3"]
            dz = self._scatter(dx3, cr3, slot3, m3, rows3)
        flat, h1, h2 = cache["leaf"]
        out["leaf"], _ = self._mlp_backward("leaf", flat, h1, h2, dz, flat.shape[0], False)
        return out

    # ---- training (the interface of ProposalEncoder)
    def loss_and_grads(self, words_t: torch.Tensor, words_p: torch.Tensor, level: int, tau: float):
        b = words_t.shape[0]
        assert b % 16 == 0 and b == words_p.shape[0]
        dev = self.device
        u, ub, cache = self.forward(torch.cat([words_t, words_p]), level, keep=True)
        logits = torch.empty((b, b), dtype=torch.float32, device=dev)
        gemm(self.ctx, _op(ub[:b], _abi.NN_KMAJOR, EMBED_DIM), _op(ub[b:], _abi.NN_KMAJOR, EMBED_DIM), b, b, EMBED_DIM, logits, alpha=1.0 / tau)
        loss = torch.empty(1, dtype=torch.float32, device=dev)
        dl = torch.empty((b, b), dtype=torch.bfloat16, device=dev)
        _abi.check(lib().tdag_nn_info_nce(self.ctx.handle, logits.data_ptr(), b, loss.data_ptr(), dl.data_ptr()))
        du = torch.empty((2 * b, EMBED_DIM), dtype=torch.float32, device=dev)
        gemm(self.ctx, _op(dl, _abi.NN_KMAJOR, b), _op(ub[b:], _abi.NN_MNMAJOR, EMBED_DIM), b, EMBED_DIM, b, du[:b], alpha=1.0 / tau)
        gemm(self.ctx, _op(dl, _abi.NN_MNMAJOR, b), _op(ub[:b], _abi.NN_MNMAJOR, EMBED_DIM), b, EMBED_DIM, b, du[b:], alpha=1.0 / tau)
        return loss, self.backward(cache, du)

    def adamw_step(self, grads: Dict[str, Optional[Sequence[torch.Tensor]]], lr: float, weight_decay: float = 1e-2, beta1: float = 0.9,
                   beta2: float = 0.999, eps: float = 1e-8) -> None:
        """One AdamW step of the groups that have gradients (the others are left as they are)."""
        self.step_count += 1
        for gname, gs in grads.items():
            if gs is None:
                continue
            for i, (p, gr) in enumerate(zip(self.params[gname], gs)):
                w16 = self.w16[gname][i // 2] if i % 2 == 0 else None
                _abi.check(lib().tdag_nn_adamw(self.ctx.handle, p.data_ptr(), gr.contiguous().data_ptr(), self.m1[gname][i].data_ptr(),
                                               self.m2[gname][i].data_ptr(), p.numel(), lr, beta1, beta2, eps, weight_decay, self.step_count,
                                               _ptr(w16)))

    def sync(self) -> None:
        _abi.check(lib().tdag_nn_sync(self.ctx.handle))


def _on_lib_stream(ctx):
    """torch's current stream set to the library context's stream, so that allocations and the
    kernels of both are ordered."""
    sp = ctypes.c_void_p()
    _abi.check(lib().tdag_ctx_stream(ctx.handle, ctypes.byref(sp)))
    return torch.cuda.stream(torch.cuda.ExternalStream(sp.value, device=ctx.device))


def embed(encoder: ProposalEncoder, words: torch.Tensor, level: int, chunk: int = 16384) -> torch.Tensor:
    """(n, 32) FP32 embeddings of n items, in chunks of items."""
    out = []
    torch.cuda.synchronize(words.device)  # the items may come from another stream
    with _on_lib_stream(encoder.ctx):
        for a in range(0, words.shape[0], chunk):
            out.append(encoder.forward(words[a:a + chunk], level)[0])
        res = torch.cat(out) if out else torch.zeros((0, EMBED_DIM), device=words.device)
    encoder.sync()
    return res


# ------------------------------------------------------------------------------------------------
# orders, labels
# ------------------------------------------------------------------------------------------------
def popcount_positions(words: torch.Tensor) -> torch.Tensor:
    """Every item's position in the matcher's source order: popcount descending, index ascending."""
    n = words.shape[0]
    shifts = torch.arange(64, device=words.device, dtype=torch.int64)
    pc = ((words.unsqueeze(-1) >> shifts) & 1).sum(dim=(1, 2))
    key = (-pc) * (n + 1) + torch.arange(n, device=words.device)
    order = torch.argsort(key)
    pos = torch.empty_like(order)
    pos[order] = torch.arange(n, device=words.device)
    return pos


def exhaustive_parents(ctx, words: torch.Tensor, level: int, config) -> Tuple[torch.Tensor, int]:
    """parent[t] = the original index of t's parent in the exhaustive search (t itself when unique)."""
    from . import _config_struct
    n = words.shape[0]
    words = words.contiguous()
    mapping = torch.empty(n, dtype=torch.int64, device=words.device)
    uniques = torch.empty(max(n, 1), dtype=torch.int32, device=words.device)
    nu = ctypes.c_uint32()
    _abi.check(lib().tdag_find_duplicates_level_device(ctx.handle, level, words.data_ptr(), n, ctypes.byref(_config_struct(config)), None, 0,
                                                       mapping.data_ptr(), uniques.data_ptr(), ctypes.byref(nu), None))
    return uniques[(mapping & PTR_MASK).long()].long(), nu.value


def subset_parents(ctx, words: torch.Tensor, level: int, config, sources: torch.Tensor) -> Tuple[torch.Tensor, int]:
    """Like exhaustive_parents, when only `sources` (original indices) search."""
    from . import _config_struct
    n = words.shape[0]
    src = sources.to(torch.int32).contiguous()
    mapping = torch.empty(n, dtype=torch.int64, device=words.device)
    uniques = torch.empty(max(n, 1), dtype=torch.int32, device=words.device)
    nu = ctypes.c_uint32()
    _abi.check(lib().tdag_find_duplicates_level_device(ctx.handle, level, words.contiguous().data_ptr(), n, ctypes.byref(_config_struct(config)),
                                                       src.data_ptr(), src.numel(), mapping.data_ptr(), uniques.data_ptr(), ctypes.byref(nu), None))
    return uniques[(mapping & PTR_MASK).long()].long(), nu.value


# ------------------------------------------------------------------------------------------------
# proposals
# ------------------------------------------------------------------------------------------------
def propose_lists(embeddings: torch.Tensor, positions: torch.Tensor, k: int, encoder_ctx=None) -> torch.Tensor:
    """(n, k) original indices: for every target, the k items with the highest embedding dot product
    among those preceding it in the source order (-1 where fewer exist). Scored on the tensor cores
    with the top-k kept in registers (tdag_nn_topk; k is rounded up to 8, 16 or 32 and cut back)."""
    n = embeddings.shape[0]
    out = torch.full((n, k), -1, dtype=torch.int64, device=embeddings.device)
    if n == 0:
        return out
    ctx = _ctx(encoder_ctx)
    kk = 8 if k <= 8 else (16 if k <= 16 else 32)
    assert k <= 32
    torch.cuda.synchronize(embeddings.device)  # the inputs may come from another stream
    with _on_lib_stream(ctx):
        order = torch.argsort(positions)  # sorted position -> original index
        e = embeddings[order].to(torch.bfloat16).contiguous()
        idx = torch.empty((n, kk), dtype=torch.int32, device=e.device)
        score = torch.empty((n, kk), dtype=torch.float32, device=e.device)
        _abi.check(lib().tdag_nn_topk(ctx.handle, e.data_ptr(), n, kk, idx.data_ptr(), score.data_ptr()))
        if kk > k:  # keep the k best of the kk
            sel = torch.topk(score, k, dim=1).indices
            idx = torch.gather(idx, 1, sel)
        idx = idx.long()
        res = torch.where(idx >= 0, order[idx.clamp(min=0)], torch.full_like(idx, -1))
        out[order] = res
    _abi.check(lib().tdag_nn_sync(ctx.handle))
    return out


def popcount_neighbour_lists(positions: torch.Tensor, k: int) -> torch.Tensor:
    """The no-network baseline: every target's k nearest predecessors in the source order (the
    closest popcounts at or above its own)."""
    n = positions.shape[0]
    order = torch.argsort(positions)
    out = torch.full((n, k), -1, dtype=torch.int64, device=positions.device)
    p = positions.unsqueeze(1) - torch.arange(1, k + 1, device=positions.device).unsqueeze(0)  # (n, k) sorted positions
    ok = p >= 0
    out[ok] = order[p[ok]]
    return out


def random_lists(positions: torch.Tensor, k: int, seed: int = 0) -> torch.Tensor:
    """Random baseline: k uniformly drawn predecessors per target."""
    n = positions.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    order = torch.argsort(positions)
    r = torch.rand((n, k), generator=g).to(positions.device)
    p = (r * positions.unsqueeze(1).float()).long()
    out = torch.where(positions.unsqueeze(1) > 0, order[p.clamp(max=n - 1)], torch.full_like(p, -1))
    return out


def sources_of(lists: torch.Tensor) -> torch.Tensor:
    """The union of the proposal lists: the items that search."""
    n = lists.shape[0]
    chosen = torch.zeros(n, dtype=torch.bool, device=lists.device)
    v = lists[lists >= 0]
    chosen[v] = True
    return chosen.nonzero().squeeze(1)


def recall_at_k(lists: torch.Tensor, parent: torch.Tensor) -> float:
    """Share of non-unique targets whose exhaustive parent is in their own proposal list."""
    n = parent.shape[0]
    dup = (parent != torch.arange(n, device=parent.device)).nonzero().squeeze(1)
    if dup.numel() == 0:
        return 1.0
    return float((lists[dup] == parent[dup].unsqueeze(1)).any(dim=1).float().mean())


# ------------------------------------------------------------------------------------------------
# training
# ------------------------------------------------------------------------------------------------
def train(encoder: ProposalEncoder, sets: Sequence[Tuple[torch.Tensor, int, torch.Tensor]], steps: int = 600, batch: int = 2048,
          lr: float = 2e-3, weight_decay: float = 1e-2, tau: float = 0.07, seed: int = 0) -> List[float]:
    """sets: (grid words, level, exhaustive parent per item). Each step draws a batch of positive
    pairs (a multiple of 16) from one randomly chosen set; forward, InfoNCE, backward and AdamW run
    as the library's kernels."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    pairs = []
    for words, level, parent in sets:
        t = (parent != torch.arange(parent.shape[0], device=parent.device)).nonzero().squeeze(1)
        if t.numel() >= 16:
            pairs.append((words, level, t, parent[t]))
    losses = []
    if not pairs:
        return losses
    dev_losses = []
    with _on_lib_stream(encoder.ctx):
        for step in range(steps):
            words, level, t, p = pairs[int(torch.randint(len(pairs), (1,), generator=g))]
            b = min(batch, t.numel()) // 16 * 16
            idx = torch.randint(t.numel(), (b,), generator=g).to(t.device)
            loss, grads = encoder.loss_and_grads(words[t[idx]], words[p[idx]], level, tau)
            encoder.adamw_step(grads, lr, weight_decay)
            dev_losses.append(loss)
        losses = torch.cat(dev_losses).cpu().tolist()
    encoder.sync()
    return losses


# ------------------------------------------------------------------------------------------------
# build hook
# ------------------------------------------------------------------------------------------------
class ProposalHook:
    """A tdag_proposal_fn backed by an encoder: the build calls it at every translation level."""

    def __init__(self, ctx, encoder: ProposalEncoder, k: int, device: int = 0):
        self.ctx, self.encoder, self.k, self.device = ctx, encoder, k, device
        self.sources: Dict[int, Tuple[int, int]] = {}  # level -> (items, proposed sources)
        self.seconds: Dict[int, Tuple[float, float]] = {}  # level -> (embedding, scoring) wall seconds
        self.error: Optional[BaseException] = None
        self.fn = _abi.PROPOSAL_FN(self._call)

    def _call(self, user, level, d_grids, n, d_sources, num_sources):
        import time
        try:
            W = (1 << (3 * level)) // 64
            words = torch.empty((n, W), dtype=torch.int64, device=f"cuda:{self.device}")
            _abi.check(lib().tdag_device_copy(self.ctx.handle, words.data_ptr(), d_grids, n * W * 8))
            t0 = time.perf_counter()
            emb = embed(self.encoder, words, level)
            t1 = time.perf_counter()
            src = sources_of(propose_lists(emb, popcount_positions(words), self.k, self.encoder.ctx)).to(torch.int32)
            torch.cuda.synchronize(self.device)
            self.seconds[level] = (t1 - t0, time.perf_counter() - t1)
            if src.numel():
                _abi.check(lib().tdag_device_copy(self.ctx.handle, d_sources, src.data_ptr(), src.numel() * 4))
            num_sources[0] = src.numel()
            self.sources[level] = (n, src.numel())
            return 0
        except BaseException as e:  # reported to the caller after the build
            self.error = e
            return 1


class RecordingHook(ProposalHook):
    """Lets every item search (the exhaustive result) and keeps each level's items: training data."""

    def __init__(self, ctx, device: int = 0):
        super().__init__(ctx, None, 0, device)
        self.grids: Dict[int, torch.Tensor] = {}

    def _call(self, user, level, d_grids, n, d_sources, num_sources):
        try:
            W = (1 << (3 * level)) // 64
            words = torch.empty((n, W), dtype=torch.int64, device=f"cuda:{self.device}")
            _abi.check(lib().tdag_device_copy(self.ctx.handle, words.data_ptr(), d_grids, n * W * 8))
            src = torch.arange(n, dtype=torch.int32, device=words.device)
            torch.cuda.synchronize(self.device)
            if n:
                _abi.check(lib().tdag_device_copy(self.ctx.handle, d_sources, src.data_ptr(), n * 4))
            num_sources[0] = n
            self.grids[level] = words
            self.sources[level] = (n, n)
            return 0
        except BaseException as e:
            self.error = e
            return 1


def level_items(in_dag, config=None, ctx=None) -> Dict[int, torch.Tensor]:
    """Every translation level's items (flattened grids, device) of a build of in_dag."""
    from . import TransformDAGConfig, _config_struct, default_context
    ctx = ctx or default_context()
    config = config or TransformDAGConfig()
    hook = RecordingHook(ctx, device=torch.cuda.current_device())
    v = in_dag.view()
    rp = ctypes.POINTER(_abi.Result)()
    rc = lib().tdag_build_device_proposed(ctx.handle, ctypes.byref(v), ctypes.byref(_config_struct(config)), hook.fn, None, ctypes.byref(rp))
    if hook.error is not None:
        raise hook.error
    _abi.check(rc)
    lib().tdag_result_free(rp)
    return hook.grids


def construct_transform_dag_proposed(in_dag, encoder: ProposalEncoder, k: int, config=None, ctx=None):
    """constructTransformDAG with learned source proposals at every translation level
    (tdag_build_device_proposed). Returns (DeviceResult, per-level (items, sources))."""
    from . import DeviceResult, TransformDAGConfig, _config_struct, default_context
    ctx = ctx or default_context()
    config = config or TransformDAGConfig()
    hook = ProposalHook(ctx, encoder, k, device=torch.cuda.current_device())
    v = in_dag.view()
    rp = ctypes.POINTER(_abi.Result)()
    rc = lib().tdag_build_device_proposed(ctx.handle, ctypes.byref(v), ctypes.byref(_config_struct(config)), hook.fn, None, ctypes.byref(rp))
    if hook.error is not None:
        raise hook.error
    _abi.check(rc)
    construct_transform_dag_proposed.last_seconds = dict(hook.seconds)
    return DeviceResult(rp), hook.sources


class FixedSourcesHook(ProposalHook):
    """Lets a given set of items search at every level (original indices per level)."""

    def __init__(self, ctx, sources_by_level: Dict[int, torch.Tensor], device: int = 0):
        super().__init__(ctx, None, 0, device)
        self.fixed = {l: v.to(torch.int32).contiguous() for l, v in sources_by_level.items()}

    def _call(self, user, level, d_grids, n, d_sources, num_sources):
        try:
            src = self.fixed.get(level)
            if src is None:
                src = torch.arange(n, dtype=torch.int32, device=f"cuda:{self.device}")
            torch.cuda.synchronize(self.device)
            if src.numel():
                _abi.check(lib().tdag_device_copy(self.ctx.handle, d_sources, src.data_ptr(), src.numel() * 4))
            num_sources[0] = src.numel()
            self.sources[level] = (n, src.numel())
            return 0
        except BaseException as e:
            self.error = e
            return 1


class FractionHook(ProposalHook):
    """No-network selectors: a fraction `rho` of every level's items searches, either the first ones
    in the source order ("popcount": the items with the most voxels) or a seeded random draw
    ("random"). They bound what any selector gains from the number of sources alone."""

    def __init__(self, ctx, rule: str, rho: float, device: int = 0, seed: int = 0):
        super().__init__(ctx, None, 0, device)
        if rule not in ("popcount", "random"):
            raise ValueError(f"unknown selection rule {rule!r}")
        self.rule, self.rho, self.seed = rule, rho, seed

    def _call(self, user, level, d_grids, n, d_sources, num_sources):
        try:
            W = (1 << (3 * level)) // 64
            words = torch.empty((n, W), dtype=torch.int64, device=f"cuda:{self.device}")
            _abi.check(lib().tdag_device_copy(self.ctx.handle, words.data_ptr(), d_grids, n * W * 8))
            m = int(self.rho * n)
            if self.rule == "popcount":
                src = (popcount_positions(words) < m).nonzero().squeeze(1).to(torch.int32)
            else:
                g = torch.Generator(device="cpu").manual_seed(self.seed + level)
                src = torch.randperm(n, generator=g)[:m].to(words.device).to(torch.int32)
            torch.cuda.synchronize(self.device)
            if src.numel():
                _abi.check(lib().tdag_device_copy(self.ctx.handle, d_sources, src.data_ptr(), src.numel() * 4))
            num_sources[0] = src.numel()
            self.sources[level] = (n, src.numel())
            return 0
        except BaseException as e:
            self.error = e
            return 1


def construct_transform_dag_by_fraction(in_dag, rule: str, rho: float, config=None, ctx=None):
    """constructTransformDAG where a fraction of the items searches at every translation level, chosen
    without a network (FractionHook). Returns (DeviceResult, per-level (items, sources))."""
    from . import DeviceResult, TransformDAGConfig, _config_struct, default_context
    ctx = ctx or default_context()
    config = config or TransformDAGConfig()
    hook = FractionHook(ctx, rule, rho, device=torch.cuda.current_device())
    v = in_dag.view()
    rp = ctypes.POINTER(_abi.Result)()
    rc = lib().tdag_build_device_proposed(ctx.handle, ctypes.byref(v), ctypes.byref(_config_struct(config)), hook.fn, None, ctypes.byref(rp))
    if hook.error is not None:
        raise hook.error
    _abi.check(rc)
    return DeviceResult(rp), hook.sources


def exhaustive_parent_sets(in_dag, config=None, ctx=None) -> Dict[int, torch.Tensor]:
    """Per translation level, the items that are some other item's parent in the exhaustive build."""
    from . import TransformDAGConfig, default_context
    ctx = ctx or default_context()
    config = config or TransformDAGConfig()
    out = {}
    for level, words in level_items(in_dag, config, ctx=ctx).items():
        parent, _ = exhaustive_parents(ctx, words, level, config)
        dup = parent != torch.arange(parent.shape[0], device=parent.device)
        out[level] = torch.unique(parent[dup])
    return out


def construct_transform_dag_with_sources(in_dag, sources_by_level: Dict[int, torch.Tensor], config=None, ctx=None):
    """constructTransformDAG where only the given items search at each translation level. With the
    exhaustive result's parents (exhaustive_parent_sets) it yields the exhaustive TDAG with the fewest
    sources: the speed no proposal method can exceed."""
    from . import DeviceResult, TransformDAGConfig, _config_struct, default_context
    ctx = ctx or default_context()
    config = config or TransformDAGConfig()
    hook = FixedSourcesHook(ctx, sources_by_level, device=torch.cuda.current_device())
    v = in_dag.view()
    rp = ctypes.POINTER(_abi.Result)()
    rc = lib().tdag_build_device_proposed(ctx.handle, ctypes.byref(v), ctypes.byref(_config_struct(config)), hook.fn, None, ctypes.byref(rp))
    if hook.error is not None:
        raise hook.error
    _abi.check(rc)
    return DeviceResult(rp), hook.sources
