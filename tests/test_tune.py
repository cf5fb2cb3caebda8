"""CPU: the launch-shape autotuner (search, cache) and the rt_tuning ABI."""
import json

import pytest

from rtxplay_gb300 import tune


def _bowl(best, weights=None):
    """Synthetic launch time: a separable bowl with its minimum at `best`
    (index distance in each knob's candidate list)."""
    weights = weights or {k: 1.0 for k in tune.SPACE}
    calls = []

    def measure(t):
        calls.append(dict(t))
        cost = 1.0
        for k, vals in tune.SPACE.items():
            cost += weights[k] * abs(vals.index(t[k]) - vals.index(best[k])) * 0.1
        return cost

    return measure, calls


def test_autotune_finds_the_minimum_of_a_separable_cost():
    best = {"wave_log2": 21, "shade_block": 128, "extend_blocks_per_sm": 3, "refill_below": 16,
            "steps_per_check": 8}
    measure, calls = _bowl(best)
    t, sec, trials = tune.autotune(measure)
    assert t == best and sec == pytest.approx(1.0)
    # memoised: no setting is timed twice
    keys = [tuple(sorted(c.items())) for c in calls]
    assert len(keys) == len(set(keys)) == len(trials)
    # coordinate descent, not the full grid (4 * 4 * 4 * 5 * 3 = 960 settings)
    assert len(trials) < 60


def test_autotune_keeps_the_start_without_a_real_gain():
    measure, _ = _bowl(dict(tune.DEFAULT))
    t, _, trials = tune.autotune(measure)
    assert t == tune.DEFAULT
    # only the first sweep runs: every knob's other values, plus the start
    assert len(trials) == 1 + sum(len(v) - 1 for v in tune.SPACE.values())
    flat = lambda t: 1.0 - (0.005 if t["wave_log2"] == 22 else 0.0)   # below min_gain
    t, _, _ = tune.autotune(flat)
    assert t == tune.DEFAULT


def test_autotune_rejects_bad_measurements_and_spaces():
    with pytest.raises(ValueError):
        tune.autotune(lambda t: float("nan"))
    with pytest.raises(ValueError):
        tune.autotune(lambda t: 1.0, space={"wave_log2": ()})


def test_workload_key_buckets():
    a = tune.workload_key("render", 1200 * 800 * 500, 7979008, 50)
    b = tune.workload_key("render", 1200 * 800 * 480, 7900000, 50)
    c = tune.workload_key("render", 1200 * 800 * 16, 7979008, 50)
    assert a == b and a != c
    assert a.startswith("render:scenes=1:layout=sah:depth=50")


def test_cache_round_trip_and_tuned(tmp_path, product, monkeypatch):
    path = tmp_path / "sub" / "tuning.json"
    cache = tune.TuneCache(str(path))
    assert cache.get("dev", "k") is None
    measure, calls = _bowl({**tune.DEFAULT, "refill_below": 8})
    t, src = tune.tuned("k", measure, cache=cache, device="dev", apply=False)
    assert src == "tuned" and t["refill_below"] == 8
    n = len(calls)
    data = json.loads(path.read_text())
    assert data["dev"]["k"]["tuning"] == t and data["dev"]["k"]["trials"] == n
    # a second lookup comes from the file and times nothing
    t2, src2 = tune.tuned("k", measure, cache=tune.TuneCache(str(path)), device="dev", apply=False)
    assert (t2, src2) == (t, "cache") and len(calls) == n
    # no entry and no measure: the defaults, applied as "no tuning"
    monkeypatch.delenv("RTX_WAVE", raising=False)
    t3, src3 = tune.tuned("other", None, cache=cache, device="dev")
    assert src3 == "default" and t3 == tune.DEFAULT
    assert product.tuning_get() == tune.DEFAULT
    # a cached entry is applied through rt_tuning_set
    tune.tuned("k", None, cache=cache, device="dev")
    assert product.tuning_get()["refill_below"] == 8
    product.tuning_set(None)


def test_package_cache_is_valid(product):
    cache = tune.TuneCache(tune.PACKAGE_CACHE)
    for dev, entries in cache.data.items():
        for key, e in entries.items():
            assert set(e["tuning"]) == set(product.TUNING_FIELDS), key
            product.tuning_set(e["tuning"])   # in range
    product.tuning_set(None)


def test_tuning_abi_set_get_and_validation(product):
    R = product
    R.tuning_set(None)
    d = R.tuning_get()
    assert d == {"wave_log2": 26, "shade_block": 512, "extend_blocks_per_sm": 0, "refill_below": 12,
                 "steps_per_check": 16}
    t = {"wave_log2": 16, "shade_block": 512, "extend_blocks_per_sm": 1, "refill_below": 31, "steps_per_check": 64}
    R.tuning_set(t)
    assert R.tuning_get() == t
    R.tuning_set({"refill_below": 3})   # other fields back to their defaults
    assert R.tuning_get() == {**d, "refill_below": 3}
    for bad in ({"wave_log2": 15}, {"wave_log2": 27}, {"shade_block": 64}, {"shade_block": 2048},
                {"extend_blocks_per_sm": 33}, {"refill_below": 32}, {"steps_per_check": 65}):
        with pytest.raises(R.RTError) as e:
            R.tuning_set(bad)
        assert e.value.status == R.RT_ERR_INVALID_ARG
        assert R.tuning_get()["refill_below"] == 3   # a refused setting changes nothing
    with pytest.raises(ValueError):
        R.tuning_set({"nosuch": 1})
    R.tuning_set(None)
    assert R.tuning_get() == d


def test_tuning_reports_the_wave_environment(product, monkeypatch):
    R = product
    R.tuning_set(None)
    monkeypatch.setenv("RTX_WAVE", str(3 << 20))
    assert R.tuning_get()["wave_log2"] == 21   # rounded down to a power of two
    monkeypatch.delenv("RTX_WAVE")
    assert R.tuning_get()["wave_log2"] == 26
