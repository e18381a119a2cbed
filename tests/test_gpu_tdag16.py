"""GPU parity of the .tdag16 encoder (tdag_encode16) against the oracle's encoder, byte for byte.

Both tie orders are compared: the default (the reference's: libstdc++ std::sort and
std::unordered_map iteration, which the oracle reproduces and which is pinned to the reference's own
encoder by test_reference_pin_cpu.py) and the canonical one (ascending item index and pointer value).
Every encoding variant (plain, Huffman, pointer tables, both) is covered, on transform DAGs built by
the oracle and by the GPU, and on a synthetic DAG whose pointer table outgrows 16-bit indices.
"""
import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes, random_grid, synthetic_tdag

pytestmark = pytest.mark.gpu

ENCODINGS = [(False, False), (False, True), (True, False), (True, True)]


TIES = [("reference", 1), ("canonical", 0)]  # library tie_order, oracle tie mode


def _gpu_encode(tdaglib, gpu_ctx, tdag_bytes, pt, hf, tie="reference"):
    s, cfg = tdaglib.read_tdag(tdag_bytes)
    return tdaglib.construct_transform_dag16(s, cfg, tdaglib.TransformEncodingConfig(pt, hf, tie), ctx=gpu_ctx, return_stats=True)


CASES = [
    ("blocky64", lambda g: blocky_grid(64, 3), dict()),
    ("terrain64", lambda g: g.terrain(64, 1), dict()),
    ("random32", lambda g: random_grid(32, 0.25, 7), dict()),
    ("blocky128-sym", lambda g: blocky_grid(128, 5), dict(axis=False, translation=False)),
    ("blocky64-plain", lambda g: blocky_grid(64, 6), dict(symmetry=False, axis=False, translation=False)),
    ("terrain256", lambda g: g.terrain(256, 1), dict()),
]


@pytest.mark.parametrize("name,make,cfg", CASES, ids=[c[0] for c in CASES])
def test_encode16_matches_oracle(oracle, tdaglib, gpu_ctx, name, make, cfg):
    from oracle import generator
    dense = make(generator)
    t, _, _ = oracle.construct_tdag(dag_svo_bytes(oracle, dense), **cfg)
    for (pt, hf), (tie, otie) in [(e, t_) for e in ENCODINGS for t_ in TIES]:
        ref, ref_stats = oracle.encode_tdag16(t, pointer_tables=pt, huffman=hf, tie=otie)
        got, st = _gpu_encode(tdaglib, gpu_ctx, t, pt, hf, tie)
        assert got == ref, (name, pt, hf, tie)
        for l in range(2, len(ref_stats)):
            g, r = st["levels"][l], ref_stats[l]
            assert (g["num_nodes"], g["memory_in_bytes"], g["table_size"]) == (r["num_nodes"], r["memory_in_bytes"], r["table_size"])
            if l >= 3:
                assert g["unique_pointers"] == r["unique_pointers"]
                assert g["table_pointers"] == [r["table_u16"], r["table_u32"], r["table_u48"]]
                assert g["direct_pointers"] == [r["direct_u16"], r["direct_u32"], r["direct_u48"]]
        assert st["kernel_launches"] > 0


def test_encode16_pointer_table_widening(oracle, tdaglib, gpu_ctx):
    t, _ = synthetic_tdag(70000, 5, 1)
    for (pt, hf), (tie, otie) in [(e, t_) for e in [(True, True), (True, False)] for t_ in TIES]:
        ref, _ = oracle.encode_tdag16(t, pointer_tables=pt, huffman=hf, tie=otie)
        got, st = _gpu_encode(tdaglib, gpu_ctx, t, pt, hf, tie)
        assert got == ref, (pt, hf, tie)
        assert st["levels"][3]["table_pointers"][0] == 65536


def test_encode16_of_device_build(oracle, tdaglib, gpu_ctx):
    """GPU build (device-resident result) -> GPU encode equals the oracle's encode of the oracle build."""
    dense = blocky_grid(128, 8)
    cfg = tdaglib.TransformDAGConfig()
    t, _, _ = oracle.construct_tdag(dag_svo_bytes(oracle, dense))
    sv = tdaglib.svdag_from_dense(dense, ctx=gpu_ctx)
    dev = tdaglib.construct_transform_dag_device(sv, cfg, ctx=gpu_ctx)
    for pt, hf in ENCODINGS:
        got = tdaglib.construct_transform_dag16(dev, cfg, tdaglib.TransformEncodingConfig(pt, hf), ctx=gpu_ctx)
        ref, _ = oracle.encode_tdag16(t, pointer_tables=pt, huffman=hf)
        assert got == ref, (pt, hf)
        assert np.array_equal(oracle.decode_tdag16(got, 128), dense)


def test_encode16_rejects_dangling_child_pointers(tdaglib, gpu_ctx):
    """A child index past the level below is reported (TDAG_ERR_CORRUPT) and its count is skipped."""
    s, cfg = tdaglib.read_tdag(synthetic_tdag(64, 1, 2)[0])
    s.nodes_per_level[3][0, 0] = tdaglib.tp_create(64)  # 64 leaves: valid indices are 0..63
    with pytest.raises(tdaglib.TDagError) as e:
        tdaglib.construct_transform_dag16(s, cfg, tdaglib.TransformEncodingConfig(True, True), ctx=gpu_ctx)
    assert e.value.code == 6


# ---- queries on the encoded file (tdag16_upload / tdag16_get / tdag16_verify) ------------------
@pytest.mark.parametrize("pt,hf", ENCODINGS)
def test_get_matches_oracle_decoder(oracle, tdaglib, gpu_ctx, pt, hf):
    """Every voxel of a 64^3 grid, plus coordinates outside the grid."""
    dense = blocky_grid(64, 3)
    t, _, _ = oracle.construct_tdag(dag_svo_bytes(oracle, dense))
    data, _ = oracle.encode_tdag16(t, pointer_tables=pt, huffman=hf)
    dev = tdaglib.Tdag16Device(data, ctx=gpu_ctx)
    z, y, x = np.meshgrid(np.arange(64), np.arange(64), np.arange(64), indexing="ij")
    xyz = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.uint32)
    got = dev.get(xyz).reshape(64, 64, 64)
    assert np.array_equal(got, oracle.decode_tdag16(data, 64))
    assert np.array_equal(got, dense)
    assert list(dev.get(np.array([[64, 0, 0], [0, 0, 1 << 20], [63, 63, 63]], np.uint32))) == [0, 0, int(dense[63, 63, 63])]


@pytest.mark.parametrize("cfg", [dict(), dict(translation=False), dict(symmetry=False, axis=False, translation=False), dict(max_level=3)])
def test_verify_accepts_lossless_encodings(tdaglib, gpu_ctx, cfg):
    dense = blocky_grid(128, 11)
    c = tdaglib.TransformDAGConfig(cfg.get("symmetry", True), cfg.get("axis", True), cfg.get("translation", True), cfg.get("max_level", 4))
    sv = tdaglib.svdag_from_dense(dense, ctx=gpu_ctx)
    dev = tdaglib.construct_transform_dag_device(sv, c, ctx=gpu_ctx)
    for pt, hf in ENCODINGS:
        data = tdaglib.construct_transform_dag16(dev, c, tdaglib.TransformEncodingConfig(pt, hf), ctx=gpu_ctx)
        st = tdaglib.Tdag16Device(data, ctx=gpu_ctx).verify(sv)
        assert st["existence_mismatches"] == 0 and st["voxel_mismatches"] == 0, (cfg, pt, hf, st)
        assert st["boxes_compared"] > 0


def test_verify_reports_a_changed_leaf(tdaglib, gpu_ctx):
    """A .tdag16 whose leaf masks were altered (pointers untouched) fails the check."""
    import struct
    dense = blocky_grid(64, 12)
    c = tdaglib.TransformDAGConfig()
    sv = tdaglib.svdag_from_dense(dense, ctx=gpu_ctx)
    data = tdaglib.construct_transform_dag16(tdaglib.construct_transform_dag_device(sv, c, ctx=gpu_ctx), c)
    off = 10
    (nl,) = struct.unpack_from("<Q", data, off)
    off += 8
    for _ in range(nl):
        (n,) = struct.unpack_from("<Q", data, off)
        off += 8 + 2 * n
    (n_leaves,) = struct.unpack_from("<Q", data, off)
    assert n_leaves > 0
    bad = bytearray(data)
    (mask,) = struct.unpack_from("<Q", data, off + 8)
    assert mask != 0
    # clear a solid voxel of leaf 0: every pointer to the leaf keeps its solid voxels inside its box,
    # so the change is visible wherever the leaf is used
    struct.pack_into("<Q", bad, off + 8, mask & (mask - 1))
    st = tdaglib.Tdag16Device(bytes(bad), ctx=gpu_ctx).verify(sv)
    assert st["voxel_mismatches"] > 0
    assert tdaglib.Tdag16Device(data, ctx=gpu_ctx).verify(sv)["voxel_mismatches"] == 0


def _rays(res, n, seed):
    """Rays from around and inside the grid towards random points, some axis-aligned, some cut short."""
    rng = np.random.default_rng(seed)
    org = rng.uniform(-0.3 * res, 1.3 * res, (n, 3))
    org[: n // 8] = rng.uniform(0.01, res - 0.01, (n // 8, 3))  # starting inside
    tgt = rng.uniform(0, res, (n, 3))
    d = tgt - org
    axis = rng.integers(0, 3, n // 8)
    d[n // 8: n // 4] = 0.0
    d[np.arange(n // 8, n // 4), axis] = rng.choice([-1.0, 1.0], n // 8)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmax = np.full(n, 4.0 * res)
    tmax[n // 4: n // 4 + n // 16] = rng.uniform(0, res, n // 16)
    return np.concatenate([org, d, np.zeros((n, 1)), tmax[:, None]], axis=1).astype(np.float32)


@pytest.mark.parametrize("pt,hf", [(False, False), (True, True)])
@pytest.mark.parametrize("maker", ["blocky", "terrain"])
def test_raycast_matches_oracle_dda(oracle, tdaglib, gpu_ctx, maker, pt, hf):
    """First hit of 4096 rays: the GPU's box-skipping traversal against a voxel-by-voxel DDA over the
    oracle's decoder (both double precision, same tie rule)."""
    from oracle import generator
    dense = blocky_grid(128, 5) if maker == "blocky" else generator.terrain(128, 3)
    t, _, _ = oracle.construct_tdag(dag_svo_bytes(oracle, dense))
    data, _ = oracle.encode_tdag16(t, pointer_tables=pt, huffman=hf)
    rays = _rays(128, 4096, 7)
    t_ref, v_ref, h_ref = oracle.raycast_tdag16(data, rays)
    t_got, v_got, h_got, steps = tdaglib.Tdag16Device(data, ctx=gpu_ctx).raycast(rays)
    assert np.array_equal(h_got, h_ref)
    assert np.array_equal(v_got[h_ref == 1], v_ref[h_ref == 1])
    assert np.allclose(t_got, t_ref, rtol=0, atol=1e-3)
    assert 0.2 < h_ref.mean() < 0.95  # both hits and misses are exercised
    assert all(dense[z, y, x] for x, y, z in v_got[h_got == 1])


def test_device_entry_points_check_their_pointers(oracle, tdaglib, gpu_ctx):
    """tdag16_get with host (numpy) arrays: refused with TDAG_ERR_ARG where the GPU cannot read
    pageable memory, answered correctly where it can (cudaDevAttrPageableMemoryAccess, e.g. Grace)."""
    import ctypes
    dense = blocky_grid(64, 3)
    t, _, _ = oracle.construct_tdag(dag_svo_bytes(oracle, dense))
    data, _ = oracle.encode_tdag16(t)
    dev = tdaglib.Tdag16Device(data, ctx=gpu_ctx)
    xyz = np.array([[1, 2, 3], [40, 41, 42], [63, 0, 17]], np.uint32)
    out = np.full(3, 7, np.uint8)
    rc = tdaglib.lib().tdag16_get(gpu_ctx.handle, dev._h, ctypes.c_void_p(xyz.ctypes.data), 3, ctypes.c_void_p(out.ctypes.data))
    if rc == 0:
        assert list(out) == [int(dense[z, y, x]) for x, y, z in xyz]
    else:
        assert rc == 1 and b"device" in tdaglib.lib().tdag_last_error_message()
