"""CPU tests of the learned-proposal encoder (tdag.proposal): layout, order, forward and gradients
against a NumPy FP64 restatement of the encoder and its InfoNCE loss."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from tdag import proposal as P  # noqa: E402


def np_forward(params, x, tau):
    """NumPy FP64 restatement: blocks MLP -> mean over non-empty blocks -> L2 norm -> symmetric InfoNCE.
    x: (2B, nb, 64) with the first B rows the targets and the last B their parents."""
    w1, b1, w2, b2, w3, b3 = params
    h = np.maximum(x @ w1.T + b1, 0)
    h = np.maximum(h @ w2.T + b2, 0)
    h = h @ w3.T + b3
    ne = (x.max(axis=-1) > 0).astype(np.float64)
    e = (h * ne[..., None]).sum(axis=1) / np.maximum(ne.sum(axis=1), 1.0)[:, None]
    e = e / np.maximum(np.linalg.norm(e, axis=1, keepdims=True), 1e-12)
    B = x.shape[0] // 2
    logits = e[:B] @ e[B:].T / tau

    def ce(z):
        z = z - z.max(axis=1, keepdims=True)
        return -np.mean(np.diag(z) - np.log(np.exp(z).sum(axis=1)))

    return 0.5 * (ce(logits) + ce(logits.T))


def random_words(n, level, seed, density=0.3):
    rng = np.random.default_rng(seed)
    R = 1 << level
    bits = rng.random((n, R * R * R)) < density
    words = np.packbits(bits.reshape(n, -1, 64)[:, :, ::-1], axis=-1).view(">u8").reshape(n, -1).astype(np.uint64)
    return torch.from_numpy(words.view(np.int64).copy()), bits


def test_unpack_blocks_layout():
    words, bits = random_words(3, 4, 1)
    blocks = P.unpack_blocks(words, 4).numpy()  # (3, 64, 64)
    R = 16
    for i in range(3):
        for (x, y, z) in [(0, 0, 0), (5, 9, 14), (15, 15, 15), (3, 12, 7)]:
            b = (x // 4) + 4 * (y // 4) + 16 * (z // 4)
            local = (x % 4) + 4 * (y % 4) + 16 * (z % 4)
            assert blocks[i, b, local] == bits[i, x + R * y + R * R * z]


def test_popcount_positions_order():
    words, bits = random_words(50, 2, 2)
    pos = P.popcount_positions(words).numpy()
    pc = bits.sum(axis=1)
    order = sorted(range(50), key=lambda i: (-pc[i], i))
    assert [int(p) for p in pos[order]] == list(range(50))


def test_proposal_lists_only_propose_predecessors():
    torch.manual_seed(0)
    words, _ = random_words(300, 3, 3)
    enc = P.ProposalEncoder()
    e = P.embed(enc, words, 3)
    pos = P.popcount_positions(words)
    for lists in (P.propose_lists(e, pos, 8, chunk=64), P.popcount_neighbour_lists(pos, 8), P.random_lists(pos, 8)):
        ok = lists >= 0
        src = lists.clamp(min=0)
        assert bool((pos[src][ok] < pos.unsqueeze(1).expand_as(lists)[ok]).all())
    assert P.sources_of(P.popcount_neighbour_lists(pos, 1)).numel() == 299  # every item but the last one


def _setup(seed=4, B=6, level=3):
    torch.manual_seed(seed)
    enc = P.ProposalEncoder().double()
    words, _ = random_words(2 * B, level, seed)
    x = P.unpack_blocks(words, level).double()
    return enc, words, x


def _torch_loss(enc, x, tau):
    nonempty = (x.amax(dim=-1) > 0).double()
    h = enc.blocks(x)
    e = (h * nonempty.unsqueeze(-1)).sum(1) / nonempty.sum(1).clamp(min=1.0).unsqueeze(-1)
    e = torch.nn.functional.normalize(e, dim=-1)
    B = x.shape[0] // 2
    return P.info_nce(e[:B], e[B:], tau)


def test_forward_matches_numpy_fp64():
    enc, words, x = _setup()
    params = [p.detach().numpy() for p in (enc.l1.weight, enc.l1.bias, enc.l2.weight, enc.l2.bias, enc.l3.weight, enc.l3.bias)]
    ref = np_forward(params, x.numpy(), 0.07)
    got = _torch_loss(enc, x, 0.07).item()
    assert abs(got - ref) < 1e-10 * max(1.0, abs(ref))
    # the encoder's own forward (float32 on the CPU) agrees with the FP64 embedding to float32 precision
    e32 = P.ProposalEncoder()
    e32.load_state_dict({k: v.float() for k, v in enc.state_dict().items()})
    emb32 = e32(words, 3).detach().numpy()
    nonempty = (x.amax(dim=-1) > 0).double()
    e64 = (enc.blocks(x) * nonempty.unsqueeze(-1)).sum(1) / nonempty.sum(1).clamp(min=1.0).unsqueeze(-1)
    e64 = torch.nn.functional.normalize(e64, dim=-1).detach().numpy()
    assert np.abs(emb32 - e64).max() < 1e-5


def test_gradients_match_finite_differences_fp64():
    enc, words, x = _setup()
    tau = 0.07
    loss = _torch_loss(enc, x, tau)
    loss.backward()
    params = [enc.l1.weight, enc.l1.bias, enc.l2.weight, enc.l2.bias, enc.l3.weight, enc.l3.bias]
    base = [p.detach().numpy().copy() for p in params]
    rng = np.random.default_rng(7)
    eps = 1e-6
    for pi, p in enumerate(params):
        g = p.grad.detach().numpy()
        for _ in range(6):
            idx = tuple(int(rng.integers(s)) for s in base[pi].shape)
            plus = [b.copy() for b in base]
            minus = [b.copy() for b in base]
            plus[pi][idx] += eps
            minus[pi][idx] -= eps
            fd = (np_forward(plus, x.numpy(), tau) - np_forward(minus, x.numpy(), tau)) / (2 * eps)
            assert abs(g[idx] - fd) <= 1e-6 + 1e-5 * abs(fd), (pi, idx, g[idx], fd)
