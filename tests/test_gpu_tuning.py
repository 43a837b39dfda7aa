"""GPU tests of the plan's tuning settings and of the autotuner.

Every setting changes speed only: num_skipped and norm stay identical to
the default plan's, the grid stays within 1e-5 (max |err| / max |grid|) of
the FP64-accumulating oracle.  The autotuner applies what it found, stores
it in its cache and takes it from there on the next call.
"""
from __future__ import annotations

import importlib

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


@pytest.fixture(scope="module")
def wl(synthetic):
    """60,000 visibilities on a 1024^2 grid, 32 planes, support 2..16."""
    return synthetic.random_uniform_workload("tuning_1024", 60_000, 1024, 32,
                                             2, 16, seed=7)


@pytest.fixture(scope="module")
def fp64(oracle_mod, wl):
    return oracle_mod.grid_f_fp64acc(wl)


def _grid(pkg, torch, wl, plan, stack):
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    G = wl.grid_size
    grid = torch.zeros((G, G, 2), dtype=torch.float32, device="cuda")
    norm = torch.zeros(1, dtype=torch.float64, device="cuda")
    skip = torch.zeros(1, dtype=torch.int64, device="cuda")
    pkg.grid_wproj_device(plan, stack, dev(wl.uu), dev(wl.vv), dev(wl.ww),
                          dev(wl.vis), dev(wl.weight),
                          np.float32(wl.cell_size_rad), np.float32(wl.w_scale),
                          G, grid, norm, skip)
    torch.cuda.synchronize()
    return grid.cpu().numpy(), float(norm.item()), int(skip.item())


TUNINGS = [
    {"tile_u": 32, "slice_staging": 1, "items_per_cta": 1, "sort_detail": 2},
    {"tile_u": 16, "slice_staging": 0, "items_per_cta": 16, "sort_detail": 1},
    {"tile_u": 8, "slice_staging": 1, "items_per_cta": 64, "sort_detail": 0},
    {"tile_u": 0, "slice_staging": -1, "items_per_cta": 8, "ctas_per_sm": 1},
    {"tile_u": 32, "slice_staging": 0, "items_per_cta": 4, "plane_group_mb": 1},
    {"tile_u": 8, "slice_staging": 1, "items_per_cta": 2, "plane_group_mb": 1},
    {"tile_u": 32, "slice_staging": 0, "items_per_cta": 4, "tile_order": 1},
    {"tile_u": 16, "slice_staging": 0, "items_per_cta": 2, "plane_group_mb": 1,
     "tile_order": 1},
    {"tile_u": 32, "slice_staging": 0, "items_per_cta": 4, "lane_groups": 1},
    {"tile_u": 32, "slice_staging": 0, "items_per_cta": 2, "lane_groups": 2,
     "plane_group_mb": 1},
    {"tile_u": 32, "slice_staging": 0, "items_per_cta": 4, "tile_phases": 2},
    {"tile_u": 32, "slice_staging": 1, "items_per_cta": 8, "tile_phases": 4,
     "plane_group_mb": 1},
    {"tile_u": 16, "slice_staging": 0, "items_per_cta": 2, "tile_phases": 4},
    {"tile_u": 8, "slice_staging": 1, "items_per_cta": 4, "tile_phases": 2,
     "plane_group_mb": 1},
    {"tile_u": 32, "slice_staging": 0, "items_per_cta": 2, "lane_groups": 2,
     "tile_phases": 2},
    {"tile_u": 32, "slice_staging": 0, "items_per_cta": 4, "tile_phases": 8},
    {"tile_u": 8, "slice_staging": 0, "items_per_cta": 4, "tile_phases": 8,
     "plane_group_mb": 1},
]


@pytest.mark.parametrize("tuning", TUNINGS)
def test_tuning_changes_speed_only(pkg, torch, wl, fp64, tuning):
    stack = pkg.KernelStack.from_workload(wl, "f")
    base = _grid(pkg, torch, wl, pkg.Plan(), stack)
    plan = pkg.Plan()
    plan.set_tuning(tuning)
    got = _grid(pkg, torch, wl, plan, stack)
    st = plan.stats()
    if tuning["tile_u"]:
        assert st["tile_u"] == tuning["tile_u"]
    if tuning.get("plane_group_mb") == 1:
        assert st["num_plane_groups"] > 1
    else:
        assert st["num_plane_groups"] == 1
    if tuning.get("ctas_per_sm") == 1:
        assert st["num_ctas"] == torch.cuda.get_device_properties(
            0).multi_processor_count
    assert got[2] == base[2] == fp64[1]
    assert got[1] == base[1]
    assert max_rel(got[0], fp64[0]) <= 1e-5


def test_tuning_rejects_bad_values(pkg, torch):
    plan = pkg.Plan()
    before = plan.tuning()
    for bad in ({"tile_u": 12}, {"slice_staging": 2}, {"items_per_cta": 0},
                {"items_per_cta": 65}, {"sort_detail": 3},
                {"ctas_per_sm": -1}, {"tile_order": 2}, {"lane_groups": 3},
                {"tile_phases": 3}, {"tile_phases": 16}):
        with pytest.raises(pkg.GridError):
            plan.set_tuning(bad)
        assert plan.tuning() == before


def test_autotune_applies_and_caches(pkg, torch, wl, fp64, tmp_path):
    at = importlib.import_module(pkg.__name__ + ".autotune")
    cache = at.TuningCache(str(tmp_path / "tuning.json"))
    stack = pkg.KernelStack.from_workload(wl, "f")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    args = (dev(wl.uu), dev(wl.vv), dev(wl.ww), dev(wl.vis), dev(wl.weight),
            wl.cell_size_rad, wl.w_scale, wl.grid_size)
    plan = pkg.Plan()
    r1 = at.autotune(pkg, plan, stack, *args, cache=cache, steps=1)
    assert r1["cached"] is False and r1["trials"] >= 10
    applied = plan.tuning()
    assert applied == {k: r1[k] for k in at.DEFAULT_TUNING}
    got = _grid(pkg, torch, wl, plan, stack)
    assert got[2] == fp64[1]
    assert max_rel(got[0], fp64[0]) <= 1e-5
    plan2 = pkg.Plan()
    r2 = at.autotune(pkg, plan2, stack, *args,
                     cache=at.TuningCache(cache.path))
    assert r2["cached"] is True and plan2.tuning() == applied


def test_plane_groups_deterministic(pkg, torch, wl):
    """Gridding in several plane-group passes is reproducible bit for bit."""
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    plan.set_tuning({"plane_group_mb": 1})
    a = _grid(pkg, torch, wl, plan, stack)
    b = _grid(pkg, torch, wl, plan, stack)
    assert plan.stats()["num_plane_groups"] > 1
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))


def test_host_tuning_applies_to_dropin(pkg, torch, wl, fp64):
    """The host-pointer entry points take a tuning like a plan does: the
    getter returns it, results stay within the bars, and None restores the
    defaults."""
    default = pkg.host_tuning()
    tuned = {"tile_u": 16, "slice_staging": 0, "items_per_cta": 8,
             "sort_detail": 1, "ctas_per_sm": 0, "plane_group_mb": 1,
             "tile_order": 1, "lane_groups": 1, "tile_phases": 2}
    try:
        pkg.set_host_tuning(tuned)
        assert pkg.host_tuning() == tuned
        g, ns, nm = pkg.grid_f(wl)
        assert ns == fp64[1]
        assert max_rel(g, fp64[0]) <= 1e-5
        with pytest.raises(pkg.GridError):
            pkg.set_host_tuning({"items_per_cta": 0})
        assert pkg.host_tuning() == tuned
    finally:
        pkg.set_host_tuning(None)
    assert pkg.host_tuning() == default
    g2, ns2, nm2 = pkg.grid_f(wl)
    assert ns2 == ns and nm2 == nm
