"""The autotuner's choice logic on CPU: the device timing is replaced by a synthetic cost
model, so what is tested is which candidate wins, the pair-list twin of the winner, the
tuning left set in the library (through the C ABI, no device calls) and the cache."""
import json

import numpy as np

from tay_gb300 import api, autotune
from tay_gb300 import models as M
from tay_gb300 import workloads as W


def _groups():
    sph = W.sph_dam(4, 4, 4)
    return [(M.sph_setup(), M.records(M.SPH_RECORD, sph.points.p, sph.points.v))]


def _cost(lists_pay):
    """Row order with quarter-support cells and x cells of half of them is fastest; lists
    save 0.1 ms when `lists_pay`, else cost 0.1 ms."""
    def measure(groups, tuning, steps=3):
        ms = 2.0 + abs(tuning["cell_multiple"] - 0.25) + abs(tuning["x_cell_factor"] - 0.5)
        ms += 0.5 * tuning["stage"] + (0.0 if tuning["cell_order"] == 1 else 1.0)
        if tuning["pair_list_cap"] == 0:
            ms += 0.1 if lists_pay else -0.1
        return ms
    return measure


def _tune(monkeypatch, tmp_path, lists_pay):
    monkeypatch.setattr(autotune, "measure", _cost(lists_pay))
    monkeypatch.setenv("TAY_GB300_TUNING_CACHE", str(tmp_path / "tuning.json"))
    return autotune.autotune(_groups())


def test_winner_keeps_pair_lists_when_they_pay(built, monkeypatch, tmp_path):
    try:
        out = _tune(monkeypatch, tmp_path, lists_pay=True)
        t = api.get_tuning()
        assert (t["cell_order"], t["cell_multiple"], t["x_cell_factor"], t["stage"]) == (1, 0.25, 0.5, 0)
        assert t["pair_list_cap"] == 320
        assert not out["cached"]
        assert out["trials"][-1]["tuning"]["pair_list_cap"] == 0  # the twin was measured
        cache = json.load(open(tmp_path / "tuning.json"))
        assert list(cache.values())[0]["tuning"]["pair_list_cap"] == 320
        again = autotune.autotune(_groups())
        assert again["cached"] and again["tuning"] == out["tuning"]
    finally:
        api.set_tuning()


def test_winner_drops_pair_lists_when_they_cost(built, monkeypatch, tmp_path):
    try:
        out = _tune(monkeypatch, tmp_path, lists_pay=False)
        t = api.get_tuning()
        assert t["pair_list_cap"] == 0 and t["cell_multiple"] == 0.25
        assert np.isclose(out["ms_per_step"], 1.9)
    finally:
        api.set_tuning()
