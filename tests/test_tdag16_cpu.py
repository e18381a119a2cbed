"""CPU tests of the .tdag16 oracle (tools/svdag_encoding/src/transform_dag_encoding.cpp, huffman.cpp).

The Huffman functions are pinned by the reference's own known-answer tests (huffman.cpp:246-367:
Moffat 2019's worked examples); the encoder by lossless decoding of every voxel, and by the
properties that do not depend on how ties are ordered (Huffman tables, node counts, distinct
pointers) agreeing between the two tie orders.
"""
import struct

import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes, random_grid, synthetic_tdag

ENCODINGS = [(False, False), (False, True), (True, False), (True, True)]


# ---- Huffman: the reference's known-answer tests -------------------------------------------------
def test_length_limited_huffman_known_answer(oracle):
    """testCreateLengthLimitedHuffmanCodeTable (huffman.cpp:269-285): Moffat 2019, fig. 6, L = 5."""
    assert oracle.huffman_lengths([20, 17, 6, 3, 2, 2, 2, 1, 1, 1], 5) == [2, 2, 3, 4, 4, 4, 4, 5, 5, 4]


def test_assign_code_words_known_answer(oracle):
    """testAssignCodeWords (huffman.cpp:287-310): Moffat 2019, table 1."""
    codes = oracle.huffman_codes([1, 2, 4, 5, 5, 5, 5, 5, 6, 6])
    assert [b for _, b in codes] == [1, 2, 4, 5, 5, 5, 5, 5, 6, 6]
    assert [c for c, _ in codes] == [0b0, 0b10, 0b1100, 0b11010, 0b11011, 0b11100, 0b11101, 0b11110, 0b111110, 0b111111]


def test_convert_to_lsb_known_answer(oracle):
    """testConvertHuffmanToLSB (huffman.cpp:319-337)."""
    codes = oracle.huffman_codes([1, 2, 4, 5, 5, 5, 5, 5, 6, 6], lsb=True)
    assert [c for c, _ in codes] == [0b0, 0b01, 0b0011, 0b01011, 0b11011, 0b00111, 0b10111, 0b01111, 0b011111, 0b111111]


def test_decoder_lut_known_answer(oracle):
    """testHuffmanDecoderLUT (huffman.cpp:339-367)."""
    codes = oracle.huffman_codes([1, 2, 4, 5, 5, 5, 5, 5, 6, 6], lsb=True)
    assert oracle.huffman_decode(codes, 0b0) == (0, 1)
    assert oracle.huffman_decode(codes, 0b1101010) == (0, 1)
    assert oracle.huffman_decode(codes, 0b01) == (1, 2)
    assert oracle.huffman_decode(codes, 0b0011) == (2, 4)
    assert oracle.huffman_decode(codes, 0b1010011) == (2, 4)


def test_kraft_sum_of_table1_is_one():
    """testKraftSum (huffman.cpp:312-317), in exact arithmetic."""
    assert sum(2.0 ** -l for l in [1, 2, 4, 5, 5, 5, 5, 5, 6, 6]) == 1.0


@pytest.mark.parametrize("seed", range(6))
def test_length_limited_codes_are_prefix_free_and_limited(oracle, seed):
    """Zero frequencies and ties included, as the encoder's 384-type histograms have them."""
    rng = np.random.default_rng(seed)
    n = [6, 48, 384, 384, 64, 8][seed]
    freq = rng.integers(0, 5, size=n) * rng.integers(0, 2, size=n) * rng.integers(1, 1000, size=n)
    lengths = oracle.huffman_lengths(freq, 16)
    assert max(lengths) <= 16 and min(lengths) >= 1
    assert sum(2.0 ** -l for l in lengths) <= 1.0
    codes = oracle.huffman_codes(lengths, lsb=True)
    for s, (c, b) in enumerate(codes):  # every code decodes to itself whatever bits follow it
        for suffix in (0, 1, (1 << (16 - b)) - 1):
            assert oracle.huffman_decode(codes, (suffix << b) | c) == (s, b)


# ---- the encoder --------------------------------------------------------------------------------
def _tdag(oracle, dense, **cfg):
    return oracle.construct_tdag(dag_svo_bytes(oracle, dense), **cfg)[0]


def _huffman_tables(data):
    """The Huffman code lists at the end of a .tdag16 (after the pointer tables)."""
    off = 10
    (nl,) = struct.unpack_from("<Q", data, off)
    off += 8
    for _ in range(nl):
        (n,) = struct.unpack_from("<Q", data, off)
        off += 8 + 2 * n
    (n,) = struct.unpack_from("<Q", data, off)
    off += 8 + 8 * n + 8
    (nl2,) = struct.unpack_from("<Q", data, off)
    off += 8
    for _ in range(nl2):
        (n,) = struct.unpack_from("<Q", data, off)
        off += 8 + 8 * n
    return data[off:]


CASES = [
    ("blocky64", lambda: blocky_grid(64, 3), {}),
    ("blocky64-sym", lambda: blocky_grid(64, 4), dict(axis=False, translation=False)),
    ("random32", lambda: random_grid(32, 0.25, 7), {}),
    ("blocky128-L3", lambda: blocky_grid(128, 5), dict(max_level=3)),
    ("blocky64-plain", lambda: blocky_grid(64, 6), dict(symmetry=False, axis=False, translation=False)),
]


@pytest.mark.parametrize("name,make,cfg", CASES, ids=[c[0] for c in CASES])
def test_encoding_decodes_every_voxel(oracle, name, make, cfg):
    dense = make()
    t = _tdag(oracle, dense, **cfg)
    for pt, hf in ENCODINGS:
        per_tie = {}
        for tie in (oracle.TIE_CANONICAL, oracle.TIE_LIBSTDCXX):
            data, stats = oracle.encode_tdag16(t, pointer_tables=pt, huffman=hf, tie=tie)
            assert np.array_equal(oracle.decode_tdag16(data, dense.shape[0]), dense), (pt, hf, tie)
            per_tie[tie] = (data, stats)
        (a, sa), (b, sb) = per_tie[0], per_tie[1]
        # tie order moves items and pointers, nothing else
        assert [(s["num_nodes"], s["unique_pointers"]) for s in sa] == [(s["num_nodes"], s["unique_pointers"]) for s in sb]
        if hf:
            assert _huffman_tables(a) == _huffman_tables(b)


def test_file_layout_header(oracle):
    dense = blocky_grid(64, 3)
    t = _tdag(oracle, dense)
    data, stats = oracle.encode_tdag16(t, pointer_tables=True, huffman=True)
    assert data[:8] == bytes([1, 1, 1, 0, 4, 0, 0, 0])  # TransformDAGConfig, padding byte zero
    assert data[8:10] == bytes([1, 1])  # TransformEncodingConfig
    (nl,) = struct.unpack_from("<Q", data, 10)
    assert nl == 7  # root level 6 + 1
    assert [s["num_nodes"] for s in stats][:3] == [0, 0, stats[2]["num_nodes"]]


def test_pointer_table_index_widens_past_65535_entries(oracle):
    """More than 65536 pointers earn a table slot at one level: the table's index grows from 16 to
    32 bits there (transform_dag_encoding.cpp:404-414), and later pointers choose with that cost."""
    t, _ = synthetic_tdag(70000, 5, 1)
    data, stats = oracle.encode_tdag16(t, pointer_tables=True, huffman=True)
    lv3 = stats[3]
    assert lv3["unique_pointers"] == 70000
    # refcount 5: a 16-bit table index (5*1 + 4 = 9 u16) beats a 32-bit inline pointer (5*2 = 10); a
    # 32-bit index (5*2 + 4 = 14) beats only a 48-bit inline pointer (15)
    assert lv3["table_u16"] == 65536
    assert lv3["table_u32"] == lv3["table_size"] - 65536 and lv3["table_u48"] == 0
    assert lv3["direct_u32"] > 0 and lv3["direct_u48"] == 0
    assert lv3["table_size"] + lv3["direct_u32"] == 70000


# ---- the library's host Huffman builder (libtdag.so, no device needed) against the oracle --------
def test_library_huffman_known_answer(tdaglib):
    codes = tdaglib.create_length_limited_huffman_code_table([20, 17, 6, 3, 2, 2, 2, 1, 1, 1], 5)
    assert [b for _, b in codes] == [2, 2, 3, 4, 4, 4, 4, 5, 5, 4]


@pytest.mark.parametrize("seed", range(8))
def test_library_huffman_matches_oracle(oracle, tdaglib, seed):
    """Pointer-type histograms: 384 / 48 / 8 symbols with many zeros and ties."""
    rng = np.random.default_rng(seed)
    n = [384, 384, 48, 8, 384, 64, 6, 1][seed]
    freq = rng.integers(0, 4, size=n) * rng.integers(0, 2, size=n) * rng.integers(1, 50, size=n)
    for lsb in (False, True):
        want = oracle.huffman_codes(oracle.huffman_lengths(freq, 16), lsb=lsb)
        assert tdaglib.create_length_limited_huffman_code_table(freq, 16, lsb_first=lsb) == want


def test_encoding_stats_json_has_the_reference_shape(tdaglib):
    """encoding_stats_json writes the svdag_encoding tool's --stats document
    (transform_dag_encoding.cpp:58-82): one entry per level from 0, the file size and both configs."""
    lv = lambda n: {"num_nodes": n, "memory_in_bytes": 2 * n, "table_size": n // 2, "unique_pointers": n, "table_pointers": [n, 1, 0],  # noqa: E731
                    "direct_pointers": [0, 2, 0]}
    stats = {"levels": {2: lv(10), 3: lv(6), 4: lv(2)}}
    enc = tdaglib.TransformEncodingConfig(pointer_tables=True, huffman_code=False)
    cfg = tdaglib.TransformDAGConfig(True, False, True, 3)
    j = tdaglib.encoding_stats_json(stats, 1234, cfg, enc)
    assert set(j) == {"levels", "total_size_in_bytes", "pointer_tables", "huffman_code", "symmetry", "axis_permutation",
                      "enable_translation", "translation_level"}
    assert len(j["levels"]) == 5 and j["levels"][0]["num_nodes"] == 0
    assert set(j["levels"][3]) == {"num_table_pointers_of_size_u16", "num_direct_pointers_of_size_u16", "table_size_in_pointers",
                                   "pointer_size_in_table", "num_nodes", "memory_in_bytes"}
    assert j["levels"][3]["pointer_size_in_table"] == 8 and j["levels"][3]["table_size_in_pointers"] == 3
    assert j["levels"][2]["pointer_size_in_table"] == 0
    assert (j["total_size_in_bytes"], j["pointer_tables"], j["huffman_code"], j["axis_permutation"], j["translation_level"]) == (1234, True, False, False, 3)
    plain = tdaglib.encoding_stats_json(stats, 1, cfg, tdaglib.TransformEncodingConfig())
    assert plain["levels"][3]["pointer_size_in_table"] == 0 and plain["levels"][3]["table_size_in_pointers"] == 0
    import json
    json.dumps(j)
