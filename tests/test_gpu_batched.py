"""GPU tests of the batched (multi-channel) gridding call.

Every channel of a batched call must give what a single call on that
channel's visibilities gives: num_skipped exact, norm within 1e-12, grid
within 1e-5 (max |err| / max |grid|) of the single call and of the FP64
oracle.  Channels have uneven visibility counts, one channel is empty, and
two batched calls are bit-identical.
"""
from __future__ import annotations

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
def batch(synthetic):
    """Six channels of a small SKA-LOW-shaped array on 1024^2 grids, with
    the third channel emptied."""
    wl = synthetic.config4(num_channels=6, grid_size=1024, times=24,
                           stations=64)
    offs = wl.channel_offsets.copy()
    # Empty channel 2 by dropping its visibilities.
    a, b = int(offs[2]), int(offs[3])
    keep = np.ones(wl.num_points, bool)
    keep[a:b] = False
    for name in ("uu", "vv", "ww", "weight"):
        setattr(wl, name, getattr(wl, name)[keep])
    wl.vis = wl.vis[keep]
    offs[3:] -= b - a
    wl.channel_offsets = offs
    return wl


def _run_batched(pkg, torch, wl, plan, stack):
    C, G = wl.num_grids, wl.grid_size
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    grids = torch.zeros((C, G, G, 2), dtype=torch.float32, device="cuda")
    norms = torch.zeros(C, dtype=torch.float64, device="cuda")
    skips = torch.full((C,), -1, dtype=torch.int64, device="cuda")
    pkg.grid_wproj_batched_device(
        plan, stack, wl.channel_offsets, dev(wl.uu), dev(wl.vv), dev(wl.ww),
        dev(wl.vis), dev(wl.weight), np.float32(wl.cell_size_rad),
        np.float32(wl.w_scale), G, grids, norms, skips)
    torch.cuda.synchronize()
    return grids.cpu().numpy(), norms.cpu().numpy(), skips.cpu().numpy()


TUNINGS = [{"plane_group_mb": 1 << 20}, {"plane_group_mb": 1},
           {"plane_group_mb": 1, "tile_phases": 2}, {"tile_phases": 4}]


@pytest.mark.parametrize("tuning", TUNINGS)
def test_batched_equals_single_calls(pkg, oracle_mod, torch, batch, tuning):
    wl = batch
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    plan.set_tuning(tuning)
    grids, norms, skips = _run_batched(pkg, torch, wl, plan, stack)
    assert wl.num_grids == 6
    for c in range(wl.num_grids):
        ch = wl.channel(c)
        g1, ns1, nm1 = pkg.grid_f(ch)
        assert skips[c] == ns1, c
        assert abs(norms[c] - nm1) <= 1e-12 * max(abs(nm1), 1.0), c
        if ch.num_points == 0:
            assert not grids[c].any() and norms[c] == 0.0
            continue
        assert max_rel(grids[c], g1) <= 1e-5, c
        g64, ns64, _ = oracle_mod.grid_f_fp64acc(ch)
        assert ns64 == skips[c]
        assert max_rel(grids[c], g64) <= 1e-5, c


def test_batched_is_deterministic(pkg, torch, batch):
    stack = pkg.KernelStack.from_workload(batch, "f")
    plan = pkg.Plan()
    a = _run_batched(pkg, torch, batch, plan, stack)
    b = _run_batched(pkg, torch, batch, plan, stack)
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_batched_rejects_bad_offsets(pkg, torch, batch):
    stack = pkg.KernelStack.from_workload(batch, "f")
    plan = pkg.Plan()
    t = torch.zeros(8, device="cuda")
    with pytest.raises(pkg.GridError):
        pkg.grid_wproj_batched_device(
            plan, stack, [0, 5, 3], t, t, t, t, t, 1.0, 1.0, 64,
            torch.zeros((2, 64, 64, 2), device="cuda"),
            torch.zeros(2, dtype=torch.float64, device="cuda"),
            torch.zeros(2, dtype=torch.int64, device="cuda"))


def _replay(pkg, torch, plan, stack, vis, weight, C, G):
    grids = torch.zeros((C, G, G, 2), dtype=torch.float32, device="cuda")
    norms = torch.zeros(C, dtype=torch.float64, device="cuda")
    skips = torch.full((C,), -1, dtype=torch.int64, device="cuda")
    pkg.grid_wproj_batched_replay(plan, stack, vis, weight, grids, norms,
                                  skips)
    pkg.check_plan(plan)
    return grids.cpu().numpy(), norms.cpu().numpy(), skips.cpu().numpy()


def _same(a, b):
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def _new_values(wl, seed):
    rng = np.random.default_rng(seed)
    vis = rng.standard_normal(wl.vis.shape).astype(np.float32)
    weight = rng.uniform(0.5, 2.0, wl.num_points).astype(np.float32)
    return vis, weight


@pytest.mark.parametrize("tuning", TUNINGS)
def test_replay_matches_batched_calls(pkg, torch, batch, tuning):
    """A replay with the original amplitudes reproduces the batched call bit
    for bit; with new amplitudes and weights it matches a fresh batched call
    on them bit for bit (the geometry depends on (u, v, w) only)."""
    import copy
    wl = batch
    C, G = wl.num_grids, wl.grid_size
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    plan.set_tuning(tuning)
    ref = _run_batched(pkg, torch, wl, plan, stack)
    # 1 MiB per pass: several plane groups; 1 TiB: a single pass.
    assert (plan.stats()["num_plane_groups"] > 1) == (
        tuning.get("plane_group_mb") == 1)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    _same(_replay(pkg, torch, plan, stack, dev(wl.vis), dev(wl.weight), C, G),
          ref)
    vis2, w2 = _new_values(wl, 5)
    got = _replay(pkg, torch, plan, stack, dev(vis2), dev(w2), C, G)
    wl2 = copy.copy(wl)
    wl2.vis, wl2.weight = vis2, w2
    plan2 = pkg.Plan()
    plan2.set_tuning(tuning)
    _same(got, _run_batched(pkg, torch, wl2, plan2, stack))


def test_replay_in_cuda_graph(pkg, torch, batch):
    """The replay captured in a CUDA graph: launching the graph after the
    inputs change in place gives the direct replay's results."""
    wl = batch
    C, G = wl.num_grids, wl.grid_size
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    _run_batched(pkg, torch, wl, plan, stack)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    vis, weight = dev(wl.vis), dev(wl.weight)
    grids = torch.zeros((C, G, G, 2), dtype=torch.float32, device="cuda")
    norms = torch.zeros(C, dtype=torch.float64, device="cuda")
    skips = torch.full((C,), -1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        grids.zero_()
        norms.zero_()
        pkg.grid_wproj_batched_replay(plan, stack, vis, weight, grids, norms,
                                      skips)
    for seed in (11, 12):
        v2, w2 = _new_values(wl, seed)
        vis.copy_(dev(v2))
        weight.copy_(dev(w2))
        graph.replay()
        pkg.check_plan(plan)
        got = (grids.cpu().numpy(), norms.cpu().numpy(), skips.cpu().numpy())
        _same(got, _replay(pkg, torch, plan, stack, dev(v2), dev(w2), C, G))
    del graph


def test_replay_needs_kept_geometry(pkg, torch, batch):
    wl = batch
    C, G = wl.num_grids, wl.grid_size
    stack = pkg.KernelStack.from_workload(wl, "f")
    other = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    vis, weight = dev(wl.vis), dev(wl.weight)
    with pytest.raises(pkg.GridError):   # nothing kept yet
        _replay(pkg, torch, plan, stack, vis, weight, C, G)
    _run_batched(pkg, torch, wl, plan, stack)
    with pytest.raises(pkg.GridError):   # another kernel stack
        _replay(pkg, torch, plan, other, vis, weight, C, G)
    ch = wl.channel(0)
    g = torch.zeros((G, G, 2), dtype=torch.float32, device="cuda")
    pkg.grid_wproj_device(plan, stack, dev(ch.uu), dev(ch.vv), dev(ch.ww),
                          dev(ch.vis), dev(ch.weight),
                          np.float32(ch.cell_size_rad), np.float32(ch.w_scale),
                          G, g, torch.zeros(1, dtype=torch.float64,
                                            device="cuda"),
                          torch.zeros(1, dtype=torch.int64, device="cuda"))
    with pytest.raises(pkg.GridError):   # a single call discarded it
        _replay(pkg, torch, plan, stack, vis, weight, C, G)


def _split_limit(wl, per_sub):
    """A batch limit that holds at most per_sub of the largest channels."""
    sizes = np.diff(wl.channel_offsets)
    return int(sizes.max()) * per_sub


@pytest.mark.parametrize("per_sub", [1, 2])
def test_sub_batches_match_one_batch(pkg, oracle_mod, torch, batch, per_sub):
    """A batched call cut into sub-batches (gg_plan_set_batch_limit; the cut
    a call larger than one sort's 32-bit record indices takes): every grid
    as the uncut call gives it -- skips exact, norm 1e-12, grid 1e-6 of the
    uncut grid and 1e-5 of the FP64 oracle -- with the same MAC and
    visibility totals."""
    wl = batch
    stack = pkg.KernelStack.from_workload(wl, "f")
    whole = pkg.Plan()
    ref = _run_batched(pkg, torch, wl, whole, stack)
    plan = pkg.Plan()
    plan.set_batch_limit(_split_limit(wl, per_sub))
    got = _run_batched(pkg, torch, wl, plan, stack)
    assert np.array_equal(got[2], ref[2])
    assert np.all(np.abs(got[1] - ref[1]) <=
                  1e-12 * np.maximum(np.abs(ref[1]), 1.0))
    st, st_ref = plan.stats(), whole.stats()
    assert st["num_points"] == st_ref["num_points"] == wl.num_points
    assert st["num_macs"] == st_ref["num_macs"]
    for c in range(wl.num_grids):
        if not ref[0][c].any():
            assert not got[0][c].any()
            continue
        assert max_rel(got[0][c], ref[0][c]) <= 1e-6, c
        g64, _, _ = oracle_mod.grid_f_fp64acc(wl.channel(c))
        assert max_rel(got[0][c], g64) <= 1e-5, c


def test_sub_batch_replays_and_graph(pkg, torch, batch):
    """Replays of a call cut into sub-batches cover every grid: with the
    original amplitudes bit-identical to the call, with new ones to a
    fresh cut call on them, and captured in a CUDA graph."""
    import copy
    wl = batch
    C, G = wl.num_grids, wl.grid_size
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    plan.set_batch_limit(_split_limit(wl, 2))
    ref = _run_batched(pkg, torch, wl, plan, stack)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    _same(_replay(pkg, torch, plan, stack, dev(wl.vis), dev(wl.weight), C, G),
          ref)
    vis2, w2 = _new_values(wl, 9)
    got = _replay(pkg, torch, plan, stack, dev(vis2), dev(w2), C, G)
    wl2 = copy.copy(wl)
    wl2.vis, wl2.weight = vis2, w2
    plan2 = pkg.Plan()
    plan2.set_batch_limit(_split_limit(wl, 2))
    _same(got, _run_batched(pkg, torch, wl2, plan2, stack))
    vis, weight = dev(wl.vis), dev(wl.weight)
    grids = torch.zeros((C, G, G, 2), dtype=torch.float32, device="cuda")
    norms = torch.zeros(C, dtype=torch.float64, device="cuda")
    skips = torch.full((C,), -1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        grids.zero_()
        norms.zero_()
        pkg.grid_wproj_batched_replay(plan, stack, vis, weight, grids, norms,
                                      skips)
    vis.copy_(dev(vis2))
    weight.copy_(dev(w2))
    graph.replay()
    pkg.check_plan(plan)
    _same((grids.cpu().numpy(), norms.cpu().numpy(), skips.cpu().numpy()),
          got)
    del graph


def test_sub_batch_limit_refuses_a_larger_grid(pkg, torch, batch):
    wl = batch
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    plan.set_batch_limit(int(np.diff(wl.channel_offsets).max()) - 1)
    with pytest.raises(pkg.GridError) as e:
        _run_batched(pkg, torch, wl, plan, stack)
    assert e.value.code == 4
