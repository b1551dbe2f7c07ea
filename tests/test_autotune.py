"""The autotuner's choice logic on CPU: the device timing is replaced by a synthetic cost
model, so what is tested is which candidate wins, the tuning left set in the library
(through the C ABI, no device calls) and the cache."""
import json

from tay_gb300 import api, autotune
from tay_gb300 import models as M
from tay_gb300 import workloads as W


def _groups():
    sph = W.sph_dam(4, 4, 4)
    return [(M.sph_setup(), M.records(M.SPH_RECORD, sph.points.p, sph.points.v))]


def _measure(groups, tuning, steps=3):
    """Row order with quarter-support cells and x cells of half of them is fastest."""
    ms = 2.0 + abs(tuning["cell_multiple"] - 0.25) + abs(tuning["x_cell_factor"] - 0.5)
    return ms + 0.5 * tuning["stage"] + (0.0 if tuning["cell_order"] == 1 else 1.0)


def test_fastest_candidate_is_set_and_cached(built, monkeypatch, tmp_path):
    monkeypatch.setattr(autotune, "measure", _measure)
    monkeypatch.setenv("TAY_GB300_TUNING_CACHE", str(tmp_path / "tuning.json"))
    try:
        out = autotune.autotune(_groups())
        t = api.get_tuning()
        assert (t["cell_order"], t["cell_multiple"], t["x_cell_factor"], t["stage"]) == (1, 0.25, 0.5, 0)
        # pair lists are not a candidate: they stay at the library default
        assert t["pair_list_cap"] == 320
        assert not out["cached"] and out["ms_per_step"] == 2.0
        assert len(out["trials"]) == len(autotune.DEFAULT_CANDIDATES)
        cache = json.load(open(tmp_path / "tuning.json"))
        assert list(cache.values())[0]["tuning"]["cell_multiple"] == 0.25
        again = autotune.autotune(_groups())
        assert again["cached"] and again["tuning"] == out["tuning"]
    finally:
        api.set_tuning()
