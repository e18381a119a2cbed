"""Failure paths of the boundary formats, on the host (no GPU involved, nothing traps).

The reference asserts on a bad .svo (export_import_structure.cpp:30-31, assert_always, which throws)
and reads vectors with no bound; the library's reader turns every malformed input into
TDAG_ERR_CORRUPT instead: a wrong magic or version, a file cut at any byte, a level count or a
vector length larger than the bytes that follow, and trailing bytes."""
import struct

import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes

CORRUPT = 6


@pytest.fixture(scope="module")
def svo(oracle):
    return dag_svo_bytes(oracle, blocky_grid(16, 2))


def _code(tdaglib, buf):
    with pytest.raises(tdaglib.TDagError) as e:
        tdaglib.EditStructure.from_svo_bytes(buf)
    return e.value.code


def test_intact_file_parses(tdaglib, svo):
    s = tdaglib.EditStructure.from_svo_bytes(svo)
    assert s.to_svo_bytes() == svo


def test_bad_magic_and_version(tdaglib, svo):
    bad_magic = bytearray(svo)
    bad_magic[0] ^= 0xFF
    assert _code(tdaglib, bytes(bad_magic)) == CORRUPT
    bad_version = bytearray(svo)
    struct.pack_into("<I", bad_version, 4, 3)
    assert _code(tdaglib, bytes(bad_version)) == CORRUPT


def test_every_truncation_is_rejected(tdaglib, svo):
    for cut in range(len(svo)):
        assert _code(tdaglib, svo[:cut]) == CORRUPT, cut


def test_trailing_bytes_rejected(tdaglib, svo):
    assert _code(tdaglib, svo + b"\0") == CORRUPT


def test_oversized_counts_rejected(tdaglib, svo):
    huge_levels = bytearray(svo)
    struct.pack_into("<Q", huge_levels, 8, 1 << 40)  # level count
    assert _code(tdaglib, bytes(huge_levels)) == CORRUPT
    huge_vector = bytearray(svo)
    struct.pack_into("<Q", huge_vector, 16, (1 << 62) // 32)  # level 0's node count
    assert _code(tdaglib, bytes(huge_vector)) == CORRUPT


def test_random_corruption_never_crashes(tdaglib, svo):
    """Flipped bytes either still parse or are reported as corrupt; nothing else escapes."""
    rng = np.random.default_rng(3)
    for _ in range(300):
        b = bytearray(svo)
        for i in rng.integers(0, len(b), size=3):
            b[i] = int(rng.integers(0, 256))
        try:
            tdaglib.EditStructure.from_svo_bytes(bytes(b))
        except tdaglib.TDagError as e:
            assert e.code == CORRUPT
