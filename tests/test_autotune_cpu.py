"""The transport autotuner's search and cache, on a synthetic cost function."""
import json

from mocassin_xray_gb300 import autotune


def test_search_finds_the_best_along_each_knob(tmp_path):
    calls = []

    def run(L):
        calls.append(dict(L))
        # best at emit 16, grid_mult 2, block 128
        return (1.0 + abs(L["emit_batch"] - 16) * 0.1 + abs((L["grid_mult"] or 4) - 2) * 0.2
                + (0.3 if L["block_size"] == 256 else 0.0))

    out = autotune.tune_transport(run, reps=1)
    assert autotune.launch_of(out) == {"block_size": 128, "grid_mult": 2, "emit_batch": 16}
    assert out["speedup"] > 1.0 and out["ms"] == min(out["trials"].values())
    n = len(calls)
    assert n <= 1 + len(autotune.EMIT_BATCHES) + len(autotune.GRID_MULTS) + len(autotune.BLOCK_SIZES)
    # the cache answers a known key without timing
    cache = tmp_path / "tune.json"
    first = autotune.tune_transport(run, key="k", cache=cache, reps=1)
    calls.clear()
    again = autotune.tune_transport(run, key="k", cache=cache, reps=1)
    assert not calls and again == json.loads(json.dumps(first))
