"""Autotuner host logic on the CPU: coordinate descent over the knobs with a
synthetic cost, the JSON cache keyed by workload signature, and knob values
the C ABI accepts."""
import json

import pytest

from pyre_gb300 import autotune as AT


@pytest.fixture()
def cache(tmp_path, monkeypatch):
    path = tmp_path / "autotune.json"
    monkeypatch.setenv("PYRE_AUTOTUNE_CACHE", str(path))
    return path


def _cost(target):
    """A separable cost, minimal at `target` (a value per knob)."""
    def run(knobs):
        ms = 10.0
        for name, values in AT.KNOBS.items():
            ms += abs(values.index(knobs[name]) - values.index(target[name]))
        return ms
    return run


def test_coordinate_descent_finds_a_separable_optimum(cache):
    target = {name: values[-1] for name, values in AT.KNOBS.items()}
    best, trials = AT.tune(_cost(target), "sep", use_cache=False)
    assert best == target
    # every distinct configuration is timed once
    seen = [json.dumps(t["knobs"], sort_keys=True) for t in trials]
    assert len(seen) == len(set(seen))
    # the defaults are the first trial
    assert trials[0]["knobs"] == AT.DEFAULT


def test_results_are_cached_by_key(cache):
    target = {name: values[0] for name, values in AT.KNOBS.items()}
    best, _ = AT.tune(_cost(target), "key-a", use_cache=True)
    data = json.loads(cache.read_text())
    assert data["key-a"]["best"] == best
    assert data["key-a"]["best_ms"] == 10.0

    def fail(knobs):
        raise AssertionError("a cached key must not be timed again")

    again, _ = AT.tune(fail, "key-a", use_cache=True)
    assert again == best
    # another key is tuned afresh and stored beside the first
    AT.tune(_cost(target), "key-b", use_cache=True)
    assert set(json.loads(cache.read_text())) == {"key-a", "key-b"}


def test_signature_is_deterministic_and_distinguishes_workloads():
    a = AT.signature("batch", [(0, 64, 64, 4, 8), (1, 128, 128, 16, 6)])
    assert a == AT.signature("batch", [(0, 64, 64, 4, 8), (1, 128, 128, 16, 6)])
    assert a != AT.signature("batch", [(0, 64, 64, 4, 8), (1, 128, 128, 16, 7)])
    assert a != AT.signature("render", [(0, 64, 64, 4, 8), (1, 128, 128, 16, 6)])


def test_knob_values_are_valid_render_parameters():
    assert set(AT.DEFAULT) == set(AT.KNOBS)
    for name, value in AT.DEFAULT.items():
        assert value in AT.KNOBS[name], name
    for b in AT.KNOBS["block_size"]:  # 0 = library defaults, else whole warps up to 256
        assert b == 0 or (b % 32 == 0 and 32 <= b <= 256)
    for r in AT.KNOBS["refill_lanes"]:
        assert 0 <= r <= 32
    assert set(AT.KNOBS["bvh_width"]) <= {2, 4, 8}
    assert set(AT.KNOBS["use_graph"]) <= {0, 1} and set(AT.KNOBS["sort_by_material"]) <= {0, 1, 2, 3}
    for w in AT.KNOBS["wave_paths"]:
        assert w == 0 or w >= 1 << 20
