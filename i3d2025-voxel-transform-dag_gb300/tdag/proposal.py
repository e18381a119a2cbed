"""Learned proposal of translation-matching sources (an approximate mode; no counterpart in the reference).

The exhaustive search lets every item of a translation level search as a source. Here an encoder
embeds every item, each target proposes the k most similar items that precede it in the popcount
order (dot products of embeddings: bf16 GEMMs on the tensor cores through cuBLAS), and only the
proposed items search. The library verifies every match exactly (tdag_build_device_proposed,
tdag_find_duplicates_level_device), so the result is always a valid TDAG. Its node count can only
grow against the exhaustive build: that growth is the "extra nodes" this mode trades for speed.

Encoder: every 4^3 block of an item -- its 64-bit occupancy mask unpacked to 64 bf16 values, bit
dx + 4 dy + 16 dz -- goes through an MLP 64 -> 256 -> 256 -> 32 (bf16 GEMMs with FP32 accumulation).
An item's embedding is the mean over its non-empty blocks ((R/4)^3 = 1, 8, 64 blocks at levels 2, 3,
4), L2-normalised. Training: InfoNCE over (target, exhaustive parent) pairs from the exhaustive GPU
matcher with in-batch negatives, AdamW on FP32 master weights.
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Optional, Sequence, Tuple

import torch
import torch.nn.functional as F

from . import _abi
from ._abi import lib

EMBED_DIM = 32
HIDDEN = 256
PTR_MASK = (1 << 37) - 1


# ------------------------------------------------------------------------------------------------
# encoder
# ------------------------------------------------------------------------------------------------
class ProposalEncoder(torch.nn.Module):
    """Leaf-block MLP 64 -> 256 -> 256 -> 32 with mean pooling over an item's non-empty 4^3 blocks."""

    def __init__(self):
        super().__init__()
        self.l1 = torch.nn.Linear(64, HIDDEN)
        self.l2 = torch.nn.Linear(HIDDEN, HIDDEN)
        self.l3 = torch.nn.Linear(HIDDEN, EMBED_DIM)

    def blocks(self, x: torch.Tensor) -> torch.Tensor:
        return self.l3(F.relu(self.l2(F.relu(self.l1(x)))))

    def forward(self, words: torch.Tensor, level: int) -> torch.Tensor:
        x = unpack_blocks(words, level)  # (n, B, 64) in {0, 1}
        nonempty = (x.amax(dim=-1) > 0).to(torch.float32)  # (n, B)
        with torch.autocast(device_type=x.device.type, dtype=torch.bfloat16, enabled=x.is_cuda):
            h = self.blocks(x.to(torch.bfloat16 if x.is_cuda else torch.float32))
        h = h.float() * nonempty.unsqueeze(-1)
        e = h.sum(dim=1) / nonempty.sum(dim=1).clamp(min=1.0).unsqueeze(-1)
        return F.normalize(e, dim=-1)


def unpack_blocks(words: torch.Tensor, level: int) -> torch.Tensor:
    """(n, R^3/64) int64 grid words (bit x + R*y + R^2*z) -> (n, (R/4)^3, 64) float blocks."""
    R = 1 << level
    n = words.shape[0]
    shifts = torch.arange(64, device=words.device, dtype=torch.int64)
    bits = ((words.unsqueeze(-1) >> shifts) & 1).to(torch.float32)  # arithmetic shift: bit s is still bit s
    b = R // 4
    bits = bits.reshape(n, b, 4, b, 4, b, 4)  # [bz, dz, by, dy, bx, dx] from the flat index x + R y + R^2 z
    return bits.permute(0, 1, 3, 5, 2, 4, 6).reshape(n, b * b * b, 64)


def embed(encoder: ProposalEncoder, words: torch.Tensor, level: int, chunk: int = 16384) -> torch.Tensor:
    out = []
    with torch.no_grad():
        for a in range(0, words.shape[0], chunk):
            out.append(encoder(words[a:a + chunk], level))
    return torch.cat(out) if out else torch.zeros((0, EMBED_DIM), device=words.device)


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
def propose_lists(embeddings: torch.Tensor, positions: torch.Tensor, k: int, chunk: int = 4096) -> torch.Tensor:
    """(n, k) original indices: for every target, the k items with the highest embedding dot product
    among those preceding it in the source order (-1 where fewer exist)."""
    n = embeddings.shape[0]
    out = torch.full((n, k), -1, dtype=torch.int64, device=embeddings.device)
    if n == 0:
        return out
    order = torch.argsort(positions)  # sorted position -> original index
    e = embeddings[order].to(torch.bfloat16)
    for a in range(1, n, chunk):
        b = min(n, a + chunk)
        scores = (e[a:b] @ e[:b].T).float()  # (targets a..b) x (sources 0..b), tensor-core GEMM
        col = torch.arange(b, device=e.device)
        row = torch.arange(a, b, device=e.device).unsqueeze(1)
        scores.masked_fill_(col.unsqueeze(0) >= row, float("-inf"))  # sources strictly before the target
        kk = min(k, b)
        top = torch.topk(scores, kk, dim=1)
        idx = torch.where(torch.isfinite(top.values), order[top.indices], torch.full_like(top.indices, -1))
        out[order[a:b], :kk] = idx
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
def info_nce(e_t: torch.Tensor, e_p: torch.Tensor, tau: float) -> torch.Tensor:
    """Symmetric InfoNCE with in-batch negatives."""
    logits = (e_t @ e_p.T) / tau
    labels = torch.arange(e_t.shape[0], device=e_t.device)
    return 0.5 * (F.cross_entropy(logits, labels) + F.cross_entropy(logits.T, labels))


def train(encoder: ProposalEncoder, sets: Sequence[Tuple[torch.Tensor, int, torch.Tensor]], steps: int = 600, batch: int = 2048,
          lr: float = 2e-3, weight_decay: float = 1e-2, tau: float = 0.07, seed: int = 0) -> List[float]:
    """sets: (grid words, level, exhaustive parent per item). Each step draws a batch of positive
    pairs from one randomly chosen set."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    opt = torch.optim.AdamW(encoder.parameters(), lr=lr, weight_decay=weight_decay)  # FP32 master weights
    pairs = []
    for words, level, parent in sets:
        t = (parent != torch.arange(parent.shape[0], device=parent.device)).nonzero().squeeze(1)
        if t.numel() >= 2:
            pairs.append((words, level, t, parent[t]))
    losses = []
    if not pairs:
        return losses
    for step in range(steps):
        words, level, t, p = pairs[int(torch.randint(len(pairs), (1,), generator=g))]
        idx = torch.randint(t.numel(), (min(batch, t.numel()),), generator=g).to(t.device)
        loss = info_nce(encoder(words[t[idx]], level), encoder(words[p[idx]], level), tau)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        losses.append(loss.item())
    return losses


# ------------------------------------------------------------------------------------------------
# build hook
# ------------------------------------------------------------------------------------------------
class ProposalHook:
    """A tdag_proposal_fn backed by an encoder: the build calls it at every translation level."""

    def __init__(self, ctx, encoder: ProposalEncoder, k: int, device: int = 0):
        self.ctx, self.encoder, self.k, self.device = ctx, encoder, k, device
        self.sources: Dict[int, Tuple[int, int]] = {}  # level -> (items, proposed sources)
        self.error: Optional[BaseException] = None
        self.fn = _abi.PROPOSAL_FN(self._call)

    def _call(self, user, level, d_grids, n, d_sources, num_sources):
        try:
            W = (1 << (3 * level)) // 64
            words = torch.empty((n, W), dtype=torch.int64, device=f"cuda:{self.device}")
            _abi.check(lib().tdag_device_copy(self.ctx.handle, words.data_ptr(), d_grids, n * W * 8))
            src = sources_of(propose_lists(embed(self.encoder, words, level), popcount_positions(words), self.k)).to(torch.int32)
            torch.cuda.synchronize(self.device)
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
    return DeviceResult(rp), hook.sources
