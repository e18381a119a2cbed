"""GPU tests of the learned-proposal mode (tdag.proposal): a source subset equal to all items is the
exhaustive search, a proposed build is a valid lossless TDAG, and learned proposals beat the
no-network baselines."""
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _scene(tdaglib, gpu_ctx, res, seed, n=None):
    spec = tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=res, seed=seed, num_primitives=n or max(40, res // 2))
    return tdaglib.scene_svdag(spec, to_dag=True, ctx=gpu_ctx)


def test_all_items_as_sources_is_the_exhaustive_search(tdaglib, gpu_ctx):
    from tdag import proposal as P
    cfg = tdaglib.TransformDAGConfig()
    grids = P.level_items(_scene(tdaglib, gpu_ctx, 256, 3), cfg, ctx=gpu_ctx)
    assert set(grids) == {2, 3, 4}
    for level, words in grids.items():
        ex, nu = P.exhaustive_parents(gpu_ctx, words, level, cfg)
        perm = torch.randperm(words.shape[0], device=words.device)  # any order of the list
        sub, nu2 = P.subset_parents(gpu_ctx, words, level, cfg, perm)
        assert nu2 == nu and torch.equal(sub, ex)
        # a strict subset can only keep more items, and every parent it finds is a listed source
        half = perm[: words.shape[0] // 2]
        sub2, nu3 = P.subset_parents(gpu_ctx, words, level, cfg, half)
        assert nu3 >= nu
        listed = torch.zeros(words.shape[0], dtype=torch.bool, device=words.device)
        listed[half] = True
        dup = sub2 != torch.arange(words.shape[0], device=words.device)
        assert bool(listed[sub2[dup]].all())


def test_proposed_build_is_lossless(oracle, tdaglib, gpu_ctx):
    from tdag import proposal as P
    cfg = tdaglib.TransformDAGConfig()
    g = _scene(tdaglib, gpu_ctx, 128, 11, 150)
    enc = P.ProposalEncoder(seed=0, ctx=gpu_ctx)
    res, sources = P.construct_transform_dag_proposed(g, enc, 4, cfg, ctx=gpu_ctx)
    got = res.to_host(ctx=gpu_ctx)
    ex = tdaglib.construct_transform_dag_device(g, cfg, ctx=gpu_ctx).to_host(ctx=gpu_ctx)
    assert set(sources) == {2, 3, 4} and all(s <= n for n, s in sources.values())
    nodes = lambda s: sum(len(a) for a in s.nodes_per_level) + len(s.sub_grids)  # noqa: E731
    assert nodes(got) >= nodes(ex)
    dense_got = oracle.tdag_decode(tdaglib.write_tdag(got, cfg), 128)
    dense_ex = oracle.tdag_decode(tdaglib.write_tdag(ex, cfg), 128)
    assert (dense_got == dense_ex).all()


@pytest.mark.parametrize("encoder", ["block", "hierarchical"])
def test_learned_proposals_beat_no_network_baselines(tdaglib, gpu_ctx, encoder):
    from tdag import proposal as P
    cfg = tdaglib.TransformDAGConfig()
    train_sets = []
    for seed in (1, 2, 3, 4):
        for level, words in P.level_items(_scene(tdaglib, gpu_ctx, 256, seed), cfg, ctx=gpu_ctx).items():
            if level >= 3:
                train_sets.append((words, level, P.exhaustive_parents(gpu_ctx, words, level, cfg)[0]))
    enc = (P.ProposalEncoder if encoder == "block" else P.HierarchicalEncoder)(seed=0, ctx=gpu_ctx)
    losses = P.train(enc, train_sets, steps=400, batch=1024)
    assert losses[-1] < losses[0]
    held = P.level_items(_scene(tdaglib, gpu_ctx, 256, 9), cfg, ctx=gpu_ctx)
    for level in (3, 4):
        words = held[level]
        parent, _ = P.exhaustive_parents(gpu_ctx, words, level, cfg)
        pos = P.popcount_positions(words)
        learned = P.recall_at_k(P.propose_lists(P.embed(enc, words, level), pos, 8), parent)
        neighbours = P.recall_at_k(P.popcount_neighbour_lists(pos, 8), parent)
        rand = P.recall_at_k(P.random_lists(pos, 8), parent)
        print(f"{encoder} encoder, level {level}: recall@8 learned {learned:.3f} popcount-neighbours {neighbours:.3f} random {rand:.3f}")
        assert learned > neighbours and learned > rand


def test_parents_as_the_only_sources_give_the_exhaustive_tdag(tdaglib, gpu_ctx):
    """The exhaustive result's parents are the smallest source set that still finds every merge: a
    build where only they search is byte-identical to the exhaustive build (the speed ceiling of any
    proposal method, which bench.py --workload proposal reports)."""
    from tdag import proposal as P
    cfg = tdaglib.TransformDAGConfig()
    g = _scene(tdaglib, gpu_ctx, 256, 5)
    parents = P.exhaustive_parent_sets(g, cfg, ctx=gpu_ctx)
    res, sources = P.construct_transform_dag_with_sources(g, parents, cfg, ctx=gpu_ctx)
    got = tdaglib.write_tdag(res.to_host(ctx=gpu_ctx), cfg)
    want = tdaglib.write_tdag(tdaglib.construct_transform_dag_device(g, cfg, ctx=gpu_ctx).to_host(ctx=gpu_ctx), cfg)
    assert got == want
    assert all(s < n for n, s in sources.values())


def test_fraction_selectors(tdaglib, gpu_ctx):
    """The no-network selectors: the whole fraction is the exhaustive build byte for byte, a smaller
    one searches with that share of the items and still yields a TDAG no smaller than the exhaustive."""
    from tdag import proposal as P
    cfg = tdaglib.TransformDAGConfig()
    g = _scene(tdaglib, gpu_ctx, 256, 5)
    ex = tdaglib.construct_transform_dag_device(g, cfg, ctx=gpu_ctx).to_host(gpu_ctx)
    want = tdaglib.write_tdag(ex, cfg)
    nodes = lambda s: sum(len(a) for a in s.nodes_per_level) + len(s.sub_grids)
    for rule in ("popcount", "random"):
        r, src = P.construct_transform_dag_by_fraction(g, rule, 1.0, cfg, ctx=gpu_ctx)
        assert tdaglib.write_tdag(r.to_host(gpu_ctx), cfg) == want
        assert all(items == s for items, s in src.values())
        r, src = P.construct_transform_dag_by_fraction(g, rule, 0.3, cfg, ctx=gpu_ctx)
        assert all(s == int(0.3 * items) for items, s in src.values())
        assert nodes(r.to_host(gpu_ctx)) >= nodes(ex)
