"""CPU tests of the autotuner's host logic: cache keys, the JSON cache and
the coordinate search (with a synthetic cost in place of GPU timings)."""
from __future__ import annotations

import importlib
import json
import math

import pytest


@pytest.fixture(scope="module")
def at(pkg):
    return importlib.import_module(pkg.__name__ + ".autotune")


def test_n_bucket(at):
    assert at.n_bucket(0) == 0 and at.n_bucket(1) == 0
    assert at.n_bucket(2) == 1 and at.n_bucket(3) == 1
    assert at.n_bucket(1 << 20) == 20 and at.n_bucket((1 << 21) - 1) == 20


def test_tuning_key_fields(at):
    k = at.tuning_key(4096, 32, 36, 4, 3_000_000, "f")
    assert k == "G4096-P32-s36-os4-N2^21-f"
    assert at.tuning_key(4096, 32, 36, 4, 3_000_000, "f", 64).endswith("-C64")
    # Same bucket, same key; different support, different key.
    assert at.tuning_key(4096, 32, 36, 4, 2_500_000) == k
    assert at.tuning_key(4096, 32, 35, 4, 3_000_000) != k


def test_cache_round_trip(at, tmp_path):
    p = tmp_path / "sub" / "tuning.json"
    c = at.TuningCache(str(p))
    assert c.get("GB300", "k") is None
    entry = dict(at.DEFAULT_TUNING, tile_u=16, ms=1.5)
    c.put("GB300", "k", entry)
    c.save()
    c2 = at.TuningCache(str(p))
    got = c2.get("GB300", "k")
    assert got == entry
    assert c2.get("other GPU", "k") is None
    assert json.loads(p.read_text())["version"] == at.CACHE_VERSION


@pytest.mark.parametrize("text", ["", "{not json", "[1, 2]",
                                  '{"version": 99, "devices": {}}'])
def test_cache_ignores_bad_files(at, tmp_path, text):
    p = tmp_path / "tuning.json"
    p.write_text(text)
    c = at.TuningCache(str(p))
    assert c.data["devices"] == {}
    c.put("d", "k", dict(at.DEFAULT_TUNING))
    c.save()
    assert at.TuningCache(str(p)).get("d", "k") == at.DEFAULT_TUNING


def test_cache_rejects_incomplete_entries(at, tmp_path):
    p = tmp_path / "tuning.json"
    p.write_text(json.dumps({"version": at.CACHE_VERSION, "devices": {
        "d": {"k": {"tile_u": 32}}}}))
    assert at.TuningCache(str(p)).get("d", "k") is None


def test_cache_path_from_env(at, monkeypatch, tmp_path):
    monkeypatch.setenv(at.CACHE_ENV, str(tmp_path / "x.json"))
    assert at.default_cache_path() == str(tmp_path / "x.json")


def test_search_finds_separable_optimum(at):
    """A cost with one best value per setting group: the coordinate search
    finds the joint optimum and times no configuration twice."""
    calls = []

    def cost(t):
        calls.append(t)
        c = 10.0
        c += 0 if (t["tile_u"], t["slice_staging"]) == (16, 1) else 3
        c += abs(t["items_per_cta"] - 8) * 0.1
        c += 0 if t["sort_detail"] == 1 else 0.5
        c += 0 if t["ctas_per_sm"] == 0 else 0.2
        return c

    best, ms, trials = at.search(cost)
    assert best == {"tile_u": 16, "slice_staging": 1, "items_per_cta": 8,
                    "sort_detail": 1, "ctas_per_sm": 0, "plane_group_mb": 0,
                    "tile_order": 0, "lane_groups": 0, "tile_phases": 0}
    assert math.isclose(ms, 10.0)
    keys = [json.dumps(t, sort_keys=True) for t in calls]
    assert len(keys) == len(set(keys)) == len(trials)


def test_search_sweeps_again_when_settings_interact(at):
    """The tile width that is fastest with the default plane groups loses
    with one plane group: the first sweep settles on it, the second sweep
    (from the one-group setting) finds the joint optimum."""
    def cost(t):
        one_group = t["plane_group_mb"] == 1 << 20
        best_u = 32 if one_group else 16
        c = 10.0 if one_group else 12.0
        return c + (0 if t["tile_u"] == best_u else 1.0)

    space = ((("tile_u", "slice_staging"), [(0, -1), (32, 0), (16, 0)]),
             (("plane_group_mb",), [(0,), (1 << 20,)]))
    one, _, _ = at.search(cost, space, sweeps=1)
    assert (one["tile_u"], one["plane_group_mb"]) == (16, 1 << 20)
    best, ms, _ = at.search(cost, space)
    assert (best["tile_u"], best["plane_group_mb"]) == (32, 1 << 20)
    assert ms == 10.0


def test_search_skips_failed_configurations(at):
    def cost(t):
        return math.inf if t["tile_u"] == 8 else 5.0 - 0.1 * (t["tile_u"] == 32)

    best, ms, _ = at.search(cost)
    assert best["tile_u"] == 32 and math.isfinite(ms)


def test_tuning_struct_round_trip(pkg):
    t = pkg.Tuning.from_dict({"tile_u": 8, "sort_detail": 0})
    assert t.as_dict() == {"tile_u": 8, "slice_staging": -1,
                           "items_per_cta": 4, "sort_detail": 0,
                           "ctas_per_sm": 0, "plane_group_mb": 0,
                           "tile_order": 0, "lane_groups": 0,
                           "tile_phases": 0}


def test_host_search_keeps_the_fastest(at):
    """autotune_host re-times the host calls over the tile order, the
    plane groups and the tile phases from the plan's settings and applies
    the fastest."""
    applied = []

    class FakePkg:
        @staticmethod
        def set_host_tuning(t):
            applied.append(dict(t))

    base = dict(at.DEFAULT_TUNING, plane_group_mb=64)
    got = at.autotune_host(FakePkg, lambda: None, base, steps=1)
    assert {k: got[k] for k in base} in applied
    assert applied[-1] == {k: got[k] for k in base}
    tried = {(t["tile_order"], t["plane_group_mb"]) for t in applied}
    assert (0, 64) in tried and (1, 64) in tried
    assert {t["tile_phases"] for t in applied} >= {0, 1, 2}
    assert got["ms"] >= 0
