"""Host logic of the batched-build autotuner (tdag.autotune), with the library calls replaced by fakes:
the descent finds the fastest configuration of a separable cost, the grid mode times the whole space,
and a configuration that changes the result is an error."""
import pytest


class _FakeResult:
    def __init__(self, payload):
        self.payload = payload

    def to_host(self, ctx):
        return self

    def to_bytes(self):
        return self.payload

    def free(self):
        pass


def _install(monkeypatch, cost, payload=lambda t: b"same"):
    import tdag
    from tdag import autotune

    class FakeContext:
        def __init__(self, device=0, tuning=None):
            self.tuning = dict(tuning or {})

        def close(self):
            pass

    def fake_build(dags, config, ctx=None):
        return [_FakeResult(payload(ctx.tuning))], {"total_ms": cost(ctx.tuning)}

    monkeypatch.setattr(tdag, "Context", FakeContext)
    monkeypatch.setattr(tdag, "construct_transform_dag_batched_device", fake_build)
    return autotune


def _cost(t):
    # separable, with its minimum at load 60, 32 bits, 3 CTAs, bulk copy 1, 8 lanes, tile 256
    t = dict({"table_load_percent": 60, "filter_bits_per_key": 32, "search_ctas_per_sm": 3, "probe_bulk_copy": 1, "verify_lanes": 8,
              "lookup_tile": 256}, **t)
    return (abs(t["table_load_percent"] - 60) + (t["filter_bits_per_key"] != 32) * 5 + (t["search_ctas_per_sm"] != 3) * 3
            + (t["probe_bulk_copy"] != 1) + abs(t["verify_lanes"] - 8) + abs(t["lookup_tile"] - 256) / 32 + 100.0)


def test_descent_finds_the_separable_minimum(monkeypatch):
    autotune = _install(monkeypatch, _cost)
    best, ms, table = autotune.autotune_batched([object()], None)
    assert best == {"table_load_percent": 60, "filter_bits_per_key": 32, "search_ctas_per_sm": 3, "probe_bulk_copy": 1,
                    "verify_lanes": 8, "lookup_tile": 256}
    assert ms == 100.0
    full = 1
    for v in autotune.DEFAULT_SPACE.values():
        full *= len(v)
    assert len(table) < full // 10  # far fewer timings than the product
    assert len({tuple(sorted(t.items())) for t, _ in table}) == len(table)  # none timed twice


def test_grid_mode_times_every_configuration(monkeypatch):
    autotune = _install(monkeypatch, _cost)
    space = {"table_load_percent": (50, 60), "verify_lanes": (4, 8, 32)}
    best, ms, table = autotune.autotune_batched([object()], None, space=space, mode="grid")
    assert len(table) == 6 and best == {"table_load_percent": 60, "verify_lanes": 8}


def test_a_tuning_that_changes_the_result_is_an_error(monkeypatch):
    autotune = _install(monkeypatch, _cost, payload=lambda t: b"x" if t["verify_lanes"] == 4 else b"same")
    with pytest.raises(RuntimeError, match="changed the result"):
        autotune.autotune_batched([object()], None)
