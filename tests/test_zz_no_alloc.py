"""tdag_find_duplicates_level_noalloc: the matcher entry point for callers that cannot allocate
device memory (for example code running inside an application that owns all device memory, or a
memory-capped service where an allocation could fail at an arbitrary point).

Called through the C ABI with device buffers owned by the test, twice in a row per case (the shared
scratch array keeps the previous call's contents, so the second call checks that everything that
must start at zero is cleared), over several (symmetry, axis permutation, translation) settings.
Each call is compared with tdag_find_duplicates_level on the same grids and with the CPU oracle;
the results are integers, so the comparison is exact. Around every call the device memory pool's
used and reserved bytes and torch's allocated bytes must stay unchanged: the call allocates nothing.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIGS = [(True, True, True), (False, True, True), (True, False, True), (True, True, False), (False, False, True)]


def _grids(level, n, seed):
    rng = np.random.default_rng(seed)
    R = 1 << level
    dense = rng.random((n, R, R, R)) < 0.2
    base = max(1, n // 4)
    for i in range(base, n):  # clipped shifted + mirrored copies of earlier grids: real matches
        src = dense[rng.integers(0, base)]
        sh = np.zeros_like(src)
        sh[1:, :, :-1] = src[:-1, :, 1:]
        dense[i] = sh[:, ::-1, :] if rng.random() < 0.5 else sh
    return np.packbits(dense.reshape(n, -1).astype(np.uint8), axis=1, bitorder="little").view(np.uint64).reshape(n, -1)


def _pool_usage(lib, ctx):
    used, reserved = ctypes.c_uint64(), ctypes.c_uint64()
    from tdag import _abi
    _abi.check(lib.tdag_device_pool_usage(ctx.handle, ctypes.byref(used), ctypes.byref(reserved)))
    return used.value, reserved.value


@pytest.mark.parametrize("cfg_flags", CONFIGS, ids=lambda c: "s{}p{}t{}".format(*map(int, c)))
@pytest.mark.parametrize("level,n", [(2, 4096), (3, 1500), (4, 300)])
def test_noalloc_matches_allocating_entry_point_and_oracle(oracle, tdaglib, gpu_ctx, level, n, cfg_flags):
    import torch
    from tdag import _abi

    L = tdaglib.lib()
    sym, axis, trans = cfg_flags
    tcfg = tdaglib.TransformDAGConfig(sym, axis, trans)
    cfg = tdaglib._config_struct(tcfg)
    dev = torch.device("cuda", gpu_ctx.device)
    for call, seed in enumerate((level * 10 + 1, level * 10 + 2)):
        grids = _grids(level, n, seed)
        ref_unique, ref_mapping = tdaglib.find_duplicates_among_flattened_items(level, grids, tcfg, ctx=gpu_ctx)
        orc_mapping, orc_unique, _ = oracle.find_duplicates(level, grids, sym, axis, trans)
        assert np.array_equal(ref_mapping, orc_mapping) and np.array_equal(ref_unique, orc_unique)

        d_grids = torch.from_numpy(grids.view(np.int64)).to(dev)
        d_map = torch.full((n,), -1, dtype=torch.int64, device=dev)
        d_uniq = torch.full((n,), -1, dtype=torch.int32, device=dev)
        d_count = torch.full((1,), -1, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        pool_before = _pool_usage(L, gpu_ctx)
        torch_before = torch.cuda.memory_allocated(dev)
        rc = L.tdag_find_duplicates_level_noalloc(gpu_ctx.handle, level, d_grids.data_ptr(), n, ctypes.byref(cfg),
                                                  d_map.data_ptr(), d_uniq.data_ptr(), d_count.data_ptr())
        _abi.check(rc)
        assert _pool_usage(L, gpu_ctx) == pool_before, f"call {call}: the device pool changed"
        assert torch.cuda.memory_allocated(dev) == torch_before
        count = int(d_count.cpu().item())
        assert count == len(ref_unique), f"call {call}"
        assert np.array_equal(d_uniq.cpu().numpy()[:count].astype(np.uint32), ref_unique), f"call {call}"
        assert np.array_equal(d_map.cpu().numpy().view(np.uint64), ref_mapping), f"call {call}"


def test_noalloc_rejects_oversized_calls(tdaglib, gpu_ctx):
    import torch
    from tdag import _abi

    L = tdaglib.lib()
    cfg = tdaglib._config_struct(tdaglib.TransformDAGConfig())
    dev = torch.device("cuda", gpu_ctx.device)
    n = 4097
    d = torch.zeros((n,), dtype=torch.int64, device=dev)
    u = torch.zeros((n,), dtype=torch.int32, device=dev)
    c = torch.zeros((1,), dtype=torch.int32, device=dev)
    rc = L.tdag_find_duplicates_level_noalloc(gpu_ctx.handle, 2, d.data_ptr(), n, ctypes.byref(cfg), d.data_ptr(), u.data_ptr(), c.data_ptr())
    assert rc == _abi.TDAG_ERR_ARG
