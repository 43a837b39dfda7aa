"""GPU parity tests of the gridder (run with -m gpu on a GB300).

Bars (the tolerances are written in each assertion):
* cell, offset and plane assignment and num_skipped: bit-exact with the
  reference's FP32 (and FP64) rules;
* norm: relative 1e-12 (it is the same FP64 per-visibility sums, added in a
  different order);
* FP32 grid: max |err| / max |grid| <= 1e-5 against the FP64 oracle with
  the same placement; against the reference's _f output, max-rel within
  max(1e-5, err_f + 1e-6), err_f being _f's own max-rel error against the
  FP64 oracle (on the small golden cases err_f is far below 1e-5, so the
  bound is 1e-5);
* FP64 grid: relative 1e-12 against the reference's _d output.
"""
from __future__ import annotations

import contextlib
import dataclasses

import numpy as np
import pytest

from conftest import golden_names, load_golden, max_rel, rms_rel

pytestmark = pytest.mark.gpu

GRID_CASES = [n for n in golden_names() if not n.startswith("weights")]


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def _dev(torch, a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


@pytest.mark.parametrize("name", GRID_CASES)
def test_dropin_matches_reference_golden(pkg, oracle_mod, torch, name):
    wl, z = load_golden(name)
    grid = z["grid_in"].copy()
    if str(z["precision"]) == "f":
        ns, nm = pkg.oskar_grid_wproj_f(
            wl.num_w_planes, wl.support, wl.oversample, wl.conv_size_half,
            wl.conv_func, wl.num_points, wl.uu, wl.vv, wl.ww, wl.vis,
            wl.weight, np.float32(wl.cell_size_rad), np.float32(wl.w_scale),
            wl.grid_size, grid, float(z["norm_in"]))
        tol = 1e-5
    else:
        ns, nm = pkg.oskar_grid_wproj_d(
            wl.num_w_planes, wl.support, wl.oversample, wl.conv_size_half,
            wl.conv_func, wl.num_points, wl.uu, wl.vv, wl.ww, wl.vis,
            wl.weight, float(wl.cell_size_rad), float(wl.w_scale),
            wl.grid_size, grid, float(z["norm_in"]))
        tol = 1e-12
    assert ns == int(z["num_skipped"])
    assert abs(nm - float(z["norm_out"])) <= 1e-12 * abs(float(z["norm_out"]))
    assert max_rel(grid, z["grid_out"]) <= tol
    if str(z["precision"]) == "f":
        g64, _, _ = oracle_mod.grid_f_fp64acc(
            wl, z["grid_in"].astype(np.float64), float(z["norm_in"]))
        assert max_rel(grid, g64) <= 1e-5


@pytest.mark.parametrize("name", ["small_f", "small_d", "edges_f",
                                  "edges_d", "os1_f", "os3_f", "os8_f"])
def test_placement_bit_exact_golden(pkg, oracle_mod, torch, name):
    wl, z = load_golden(name)
    prec = str(z["precision"])
    dt = torch.float32 if prec == "f" else torch.float64
    stack = pkg.KernelStack.from_workload(wl, prec)
    cast = np.float32 if prec == "f" else float
    out = pkg.place_wproj_device(
        stack, _dev(torch, wl.uu, dt), _dev(torch, wl.vv, dt),
        _dev(torch, wl.ww, dt), cast(wl.cell_size_rad), cast(wl.w_scale),
        wl.grid_size).cpu().numpy()
    p = oracle_mod.place(wl, prec)
    skipped = out[:, 5] & 1
    assert np.array_equal(skipped, p["skipped"])
    assert np.array_equal(out[:, 5] >> 1, p["conj_neg"])
    keep = p["skipped"] == 0
    for col, key in enumerate(("gu", "gv", "ou", "ov", "plane")):
        assert np.array_equal(out[keep, col], p[key][keep]), key
    assert int(skipped.sum()) == int(z["num_skipped"])


@pytest.mark.parametrize("which", ["cfg0", "cfg1_sub", "skalow_small"])
def test_placement_bit_exact_synthetic(pkg, oracle_mod, synthetic, torch,
                                       which):
    if which == "cfg0":
        wl = synthetic.config0()
    elif which == "cfg1_sub":
        wl = synthetic.config1().subset(400_000)
    else:
        wl = _skalow_small(synthetic)
    for prec in ("f", "d"):
        dt = torch.float32 if prec == "f" else torch.float64
        stack = pkg.KernelStack.from_workload(wl, prec)
        cast = np.float32 if prec == "f" else float
        out = pkg.place_wproj_device(
            stack, _dev(torch, wl.uu, dt), _dev(torch, wl.vv, dt),
            _dev(torch, wl.ww, dt), cast(wl.cell_size_rad),
            cast(wl.w_scale), wl.grid_size).cpu().numpy()
        p = oracle_mod.place(wl, prec)
        assert np.array_equal(out[:, 5] & 1, p["skipped"])
        keep = p["skipped"] == 0
        for col, key in enumerate(("gu", "gv", "ou", "ov", "plane")):
            assert np.array_equal(out[keep, col], p[key][keep]), (prec, key)


def _skalow_small(synthetic):
    """SKA-LOW-shaped array at reduced size (64 stations, 60 times)."""
    rng = np.random.Generator(np.random.PCG64(3))
    u, v, w = synthetic.ska_low_uvw_metres(rng, num_stations=64,
                                           num_times=60)
    sc = 100e6 / synthetic.SPEED_OF_LIGHT
    u, v, w = u * sc, v * sc, w * sc
    G, planes, s_min, s_max = 2048, 96, 4, 24
    cell = synthetic._fit_cell_size(float(max(abs(u).max(), abs(v).max())),
                                    G, s_max)
    support = synthetic.linear_supports(planes, s_min, s_max)
    wl = synthetic._finish("skalow_small", rng, support, 4, G, cell, u, v, w,
                           float(abs(w).max()),
                           weight=np.ones(u.shape[0], np.float32))
    return dataclasses.replace(wl)


def test_cfg0_error_vs_fp64_oracle(pkg, oracle_mod, synthetic, torch):
    wl = synthetic.config0()
    g, ns, nm = pkg.grid_f(wl)
    g64, ns64, nm64 = oracle_mod.grid_f_fp64acc(wl)
    gref, nsr, nmr = oracle_mod.grid_f(wl)
    assert ns == ns64 == nsr
    assert abs(nm - nm64) <= 1e-12 * abs(nm64)
    err = max_rel(g, g64)
    err_ref = max_rel(gref, g64)
    print(f"cfg0 max-rel vs FP64: gpu {err:.3e} (reference _f {err_ref:.3e}); "
          f"rms gpu {rms_rel(g, g64):.3e} ref {rms_rel(gref, g64):.3e}")
    assert err <= 1e-5
    # Compensated accumulation is at least as accurate as the serial FP32.
    assert rms_rel(g, g64) <= rms_rel(gref, g64)
    assert max_rel(g, gref) <= 1e-5


def test_device_entry_equals_drop_in_and_is_deterministic(pkg, synthetic,
                                                          torch):
    wl = synthetic.config0().subset(50_000)
    g_host, ns_h, nm_h = pkg.grid_f(wl)
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    grids = []
    for _ in range(2):
        grid = torch.zeros((wl.grid_size, wl.grid_size, 2),
                           dtype=torch.float32, device="cuda")
        norm = torch.zeros(1, dtype=torch.float64, device="cuda")
        ns = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        pkg.grid_wproj_device(plan, stack, _dev(torch, wl.uu),
                              _dev(torch, wl.vv), _dev(torch, wl.ww),
                              _dev(torch, wl.vis), _dev(torch, wl.weight),
                              np.float32(wl.cell_size_rad),
                              np.float32(wl.w_scale), wl.grid_size, grid,
                              norm, ns)
        torch.cuda.synchronize()
        grids.append(grid.cpu().numpy())
        assert int(ns.item()) == ns_h
        assert norm.item() == nm_h
    assert np.array_equal(grids[0].view(np.uint32), grids[1].view(np.uint32))
    assert np.array_equal(grids[0].view(np.uint32), g_host.view(np.uint32))
    st = plan.stats()
    assert st["num_points"] == wl.num_points and st["num_macs"] > 0


@pytest.mark.parametrize("which", ["cfg0", "skalow_small"])
def test_every_tile_shape_matches_fp64_oracle(pkg, oracle_mod, synthetic,
                                              torch, which):
    """Each tile width (32, 16, 8) grids to within 1e-5 of the FP64 oracle;
    the automatic choice equals one of them bit for bit."""
    wl = synthetic.config0() if which == "cfg0" else _skalow_small(synthetic)
    g64, ns64, nm64 = oracle_mod.grid_f_fp64acc(wl)
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    grids = {}
    for tu in (32, 16, 8, 0):
        plan.set_tile_shape(tu)
        grid = torch.zeros((wl.grid_size, wl.grid_size, 2),
                           dtype=torch.float32, device="cuda")
        norm = torch.zeros(1, dtype=torch.float64, device="cuda")
        ns = torch.zeros(1, dtype=torch.int64, device="cuda")
        pkg.grid_wproj_device(plan, stack, _dev(torch, wl.uu),
                              _dev(torch, wl.vv), _dev(torch, wl.ww),
                              _dev(torch, wl.vis), _dev(torch, wl.weight),
                              np.float32(wl.cell_size_rad),
                              np.float32(wl.w_scale), wl.grid_size, grid,
                              norm, ns)
        torch.cuda.synchronize()
        st = plan.stats()
        g = grid.cpu().numpy()
        assert int(ns.item()) == ns64
        assert abs(norm.item() - nm64) <= 1e-12 * abs(nm64)
        if tu:
            assert st["tile_u"] == tu and st["tile_u"] * st["tile_v"] == 2048
            assert max_rel(g, g64) <= 1e-5, tu
        grids[tu if tu else ("auto", st["tile_u"])] = g
    auto_key = next(k for k in grids if isinstance(k, tuple))
    assert np.array_equal(grids[auto_key].view(np.uint32),
                          grids[auto_key[1]].view(np.uint32))


@pytest.mark.parametrize("which", ["cfg0", "skalow_small"])
def test_slice_staging_is_bit_identical(pkg, synthetic, torch, which):
    """Staging kernel slices in shared memory changes only where taps are
    read from: the grids with staging on and off are bit-identical."""
    wl = synthetic.config0() if which == "cfg0" else _skalow_small(synthetic)
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    out = []
    for mode in (0, 1):
        plan.set_slice_staging(mode)
        grid = torch.zeros((wl.grid_size, wl.grid_size, 2),
                           dtype=torch.float32, device="cuda")
        norm = torch.zeros(1, dtype=torch.float64, device="cuda")
        ns = torch.zeros(1, dtype=torch.int64, device="cuda")
        pkg.grid_wproj_device(plan, stack, _dev(torch, wl.uu),
                              _dev(torch, wl.vv), _dev(torch, wl.ww),
                              _dev(torch, wl.vis), _dev(torch, wl.weight),
                              np.float32(wl.cell_size_rad),
                              np.float32(wl.w_scale), wl.grid_size, grid,
                              norm, ns)
        torch.cuda.synchronize()
        out.append(grid.cpu().numpy())
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_accumulate_semantics(pkg, synthetic, torch):
    """grid and norm accumulate across calls, num_skipped is set."""
    wl = synthetic.config0().subset(20_000)
    g1, ns1, nm1 = pkg.grid_f(wl)
    g2, ns2, nm2 = pkg.grid_f(wl, g1.copy(), nm1)
    assert ns2 == ns1
    assert abs(nm2 - 2 * nm1) <= 1e-12 * abs(nm2)
    assert max_rel(g2, 2 * g1) <= 1e-6


def test_linearity_exact_full_cfg1(pkg, oracle_mod, synthetic, torch):
    """Scaling visibilities by 2 scales the grid by exactly 2 (every
    operation on the path is exact under a power-of-two scale)."""
    wl = synthetic.config1()
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    outs = []
    for scale in (1.0, 2.0):
        grid = torch.zeros((wl.grid_size, wl.grid_size, 2),
                           dtype=torch.float32, device="cuda")
        norm = torch.zeros(1, dtype=torch.float64, device="cuda")
        ns = torch.zeros(1, dtype=torch.int64, device="cuda")
        pkg.grid_wproj_device(plan, stack, _dev(torch, wl.uu),
                              _dev(torch, wl.vv), _dev(torch, wl.ww),
                              _dev(torch, wl.vis * np.float32(scale)),
                              _dev(torch, wl.weight),
                              np.float32(wl.cell_size_rad),
                              np.float32(wl.w_scale), wl.grid_size, grid,
                              norm, ns)
        torch.cuda.synchronize()
        outs.append((grid, int(ns.item()), norm.item()))
    assert torch.equal(outs[1][0], 2 * outs[0][0])
    assert outs[0][1] == outs[1][1] == oracle_mod.place(wl)["num_skipped"]
    assert plan.stats()["num_macs"] == oracle_mod.mac_count(wl)


def test_cfg1_vs_reference_rules(pkg, oracle_mod, synthetic, torch):
    """Full synthetic-challenge shape against the host-parallel oracle,
    which is bit-identical to the reference's serial _f."""
    wl = synthetic.config1()
    g, ns, nm = pkg.grid_f(wl)
    gref, nsr, nmr = oracle_mod.grid_f_mt(wl)
    g64, _, _ = oracle_mod.grid_f_fp64acc_mt(wl)
    assert ns == nsr
    assert abs(nm - nmr) <= 1e-12 * abs(nmr)
    err = max_rel(g, gref)
    err_f = max_rel(gref, g64)
    tol_f = max(1e-5, err_f + 1e-6)
    print(f"cfg1 max-rel vs reference _f: {err:.3e} (bound {tol_f:.3e}); "
          f"vs FP64 {max_rel(g, g64):.3e}, _f vs FP64 {err_f:.3e}")
    assert err <= tol_f
    assert max_rel(g, g64) <= 1e-5


def test_fp64_path_vs_reference_d(pkg, oracle_mod, synthetic, torch):
    wl = synthetic.config0().subset(30_000)
    g, ns, nm = pkg.grid_d(wl)
    gr, nsr, nmr = oracle_mod.grid_d(wl)
    assert ns == nsr
    assert abs(nm - nmr) <= 1e-12 * abs(nmr)
    assert max_rel(g, gr) <= 1e-12


def test_empty_and_all_skipped_device(pkg, synthetic, torch):
    wl = synthetic.config0().subset(0)
    g, ns, nm = pkg.grid_f(wl, norm=3.5)
    assert ns == 0 and nm == 3.5 and not g.any()
    wl = synthetic.config0().subset(100)
    wl.uu = np.full(100, 1e9, np.float32)
    g, ns, nm = pkg.grid_f(wl, norm=1.0)
    assert ns == 100 and nm == 1.0 and not g.any()


@pytest.mark.parametrize("oversample,s_max,prec", [
    (4, 72, "f"), (2, 30, "f"), (8, 40, "f"), (4, 60, "d"), (14, 72, "f")])
def test_tap_sums_bit_exact_per_visibility(pkg, oracle_mod, synthetic,
                                           oversample, s_max, prec):
    """The per-(plane, offset class) tap sums of the norm: with one
    visibility per call the norm is that visibility's sum times its weight,
    so it must equal the reference's serial sum bit for bit, on every plane
    up to the largest support, for oversampling 2 to 14 (the last case's row
    window exceeds the block-per-plane kernel's and takes the per-sum
    kernel)."""
    wl = synthetic.random_uniform_workload(
        "taps", 40, 1024, 6, max(1, s_max // 3), s_max,
        oversample=oversample, seed=41 + oversample, cell_size_rad=1e-4)
    grid_fn = pkg.grid_f if prec == "f" else pkg.grid_d
    oracle_fn = oracle_mod.grid_f if prec == "f" else oracle_mod.grid_d
    planes = set()
    for i in range(wl.num_points):
        one = dataclasses.replace(
            wl, uu=wl.uu[i:i + 1], vv=wl.vv[i:i + 1], ww=wl.ww[i:i + 1],
            vis=wl.vis[i:i + 1], weight=wl.weight[i:i + 1])
        g, ns, nm = grid_fn(one)
        gr, nsr, nmr = oracle_fn(one)
        assert ns == nsr and nm == nmr, i
        if not ns:
            planes.add(int(oracle_mod.place(one, prec)["plane"][0]))
    assert wl.num_w_planes - 1 in planes      # the largest support


def test_nonfinite_kernel_tap_stays_in_its_footprints(pkg, oracle_mod,
                                                      synthetic, torch):
    """A NaN kernel tap reaches exactly the grid cells whose footprints use
    it, as in the reference: the kernel never reads a tap for a lane
    outside a footprint when the stack holds a non-finite value."""
    wl = synthetic.config0().subset(50_000)
    cf = wl.conv_func.copy()
    cf[3, 2, 1, 0] = np.nan     # plane 3, quadrant row 2, column 1, real
    wl.conv_func = cf
    g, ns, _ = pkg.grid_f(wl)
    gr, nsr, _ = oracle_mod.grid_f(wl)
    assert ns == nsr
    assert np.isnan(gr).any()
    assert np.array_equal(np.isnan(g), np.isnan(gr))
    fin = ~np.isnan(gr)
    assert max_rel(np.where(fin, g, 0), np.where(fin, gr, 0)) <= 1e-5


@pytest.mark.parametrize("os_,G,s_min,s_max", [(5, 255, 0, 6), (14, 301, 1, 5),
                                                (1, 128, 0, 9), (2, 97, 0, 3)])
def test_unusual_parameters_vs_oracle(pkg, oracle_mod, synthetic, torch, os_,
                                      G, s_min, s_max):
    """Odd and extreme oversampling (the column-residue split of the slab
    stack, offsets up to (os+1)/2), zero supports and odd grid sizes:
    skips and norm as the reference, FP32 grid within 1e-5 of the FP64
    oracle, FP64 grid within 1e-12 of the reference _d."""
    wl = synthetic.random_uniform_workload(
        f"odd_os{os_}", 6000, G, 7, s_min, s_max, oversample=os_, seed=os_,
        cell_size_rad=4.0 / (G * 300.0), w_max=400.0, sigma_frac=0.2,
        clip_frac=0.48)
    g, ns, nm = pkg.grid_f(wl)
    g64, ns64, nm64 = oracle_mod.grid_f_fp64acc(wl)
    _, nsr, nmr = oracle_mod.grid_f(wl)
    assert ns == ns64 == nsr
    assert abs(nm - nmr) <= 1e-12 * max(abs(nmr), 1.0)
    assert max_rel(g, g64) <= 1e-5
    gd, nsd, nmd = pkg.grid_d(wl)
    gr, nsdr, nmdr = oracle_mod.grid_d(wl)
    assert nsd == nsdr
    assert max_rel(gd, gr) <= 1e-12


@contextlib.contextmanager
def _access(pkg, mode):
    """Grid access mode of the host calls for the duration of a block."""
    old = pkg.host_grid_access()
    pkg.set_host_grid_access(mode)
    try:
        yield
    finally:
        pkg.set_host_grid_access(old)


def _pinned_like(a, torch):
    t = torch.empty(a.shape, dtype=getattr(torch, a.dtype.name),
                    pin_memory=True)
    t.numpy()[...] = a
    return t.numpy()


def _start_grid(G, seed, pinned=False, dtype=np.float32, torch=None):
    """Random starting grid; pinned=True puts it in page-locked memory (the
    drop-in's copies then run asynchronously on the copy engines)."""
    g = np.random.default_rng(seed).standard_normal((G, G, 2)).astype(dtype)
    if not pinned:
        return g
    t = torch.empty((G, G, 2), dtype=getattr(torch, np.dtype(dtype).name),
                    pin_memory=True)
    t.numpy()[...] = g
    return t.numpy()


@pytest.mark.parametrize("phases", [0, 4])
@pytest.mark.parametrize("mode", ["copy", "in_place"])
@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("where", ["disk", "patch_centre", "patch_corner"])
def test_dropin_copies_back_touched_spans(pkg, oracle_mod, synthetic, torch,
                                          where, pinned, mode, phases):
    """The host-pointer call copies back only the tile rows' spans that
    hold records (or, in place, reads and writes only the tiles that hold
    records), also with four tile phases (spans and host accesses in
    strips of a quarter tile).  With a random starting grid the result
    must be start + the contributions everywhere, and bit-for-bit the start
    wherever nothing was added (cells outside every footprint)."""
    G = 1800
    if where == "disk":
        wl = synthetic.random_uniform_workload(
            "spans_disk", 40_000, G, 32, 2, 12, seed=17, cell_size_rad=3e-5)
    else:
        wl = synthetic.random_uniform_workload(
            "spans_patch", 20_000, G, 32, 2, 12, seed=18, cell_size_rad=3e-5,
            sigma_frac=0.01, clip_frac=0.03)
        if where == "patch_corner":   # shift the patch towards a corner
            extent = 1.0 / wl.cell_size_rad
            wl = dataclasses.replace(
                wl, uu=(wl.uu + np.float32(0.4 * extent)).astype(np.float32),
                vv=(wl.vv - np.float32(0.4 * extent)).astype(np.float32))
    start = _start_grid(G, 3)
    pkg.set_host_tuning({"tile_phases": phases})
    try:
        with _access(pkg, pkg.GRID_ACCESS_COPY if mode == "copy"
                     else pkg.GRID_ACCESS_PAGEABLE):
            g0, ns0, nm0 = pkg.grid_f(wl)
            g1, ns1, nm1 = pkg.grid_f(
                wl, _start_grid(G, 3, pinned, torch=torch), 2.0)
    finally:
        pkg.set_host_tuning(None)
    assert ns1 == ns0 < wl.num_points
    assert abs(nm1 - (nm0 + 2.0)) <= 1e-12 * abs(nm1)
    assert max_rel(g1, start + g0) <= 1e-6
    untouched = g0 == 0
    assert untouched.any()
    assert np.array_equal(g1[untouched], start[untouched])
    gr, nsr, _ = oracle_mod.grid_f(wl)
    assert ns0 == nsr
    assert max_rel(g0, gr) <= 1e-5


@pytest.mark.parametrize("G", [4096, 4099])
@pytest.mark.parametrize("tuning", [{"plane_group_mb": 0},
                                    {"plane_group_mb": 1},
                                    {"plane_group_mb": 1, "tile_phases": 4},
                                    {"tile_phases": 2}])
@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("prec", ["f", "d"])
def test_dropin_split_passes(pkg, oracle_mod, synthetic, torch, prec, pinned,
                             tuning, G):
    """On grids of 128 MiB and more the host-pointer call uploads the grid
    in two halves by rows and grids the first and last plane groups (or
    the only one) in two passes by tile rows, the upper rows first, and
    copies the upper rows back while the lower ones are gridded.  A random
    starting grid must still come back as start + contributions, bit for
    bit where nothing was added, with the reference's placement; with one
    plane group and with several (1 MiB groups), with tile phases, on an
    even grid and on an odd one (ragged last tiles; the split row a
    multiple of 256)."""
    wl = synthetic.random_uniform_workload(
        "split", 60_000, G, 64, 2, 16, seed=23, cell_size_rad=1.2e-5,
        sigma_frac=0.15, clip_frac=0.45)
    dt = np.float32 if prec == "f" else np.float64
    grid_fn = pkg.grid_f if prec == "f" else pkg.grid_d
    start = _start_grid(G, 8, dtype=dt)
    pkg.set_host_tuning(tuning)
    try:
        with _access(pkg, pkg.GRID_ACCESS_COPY):
            g0, ns0, nm0 = grid_fn(wl)
            g1, ns1, nm1 = grid_fn(wl, _start_grid(G, 8, pinned, dt, torch),
                                   1.5)
    finally:
        pkg.set_host_tuning(None)
    assert ns1 == ns0 < wl.num_points
    assert max_rel(g1, start + g0) <= (1e-6 if prec == "f" else 1e-14)
    untouched = g0 == 0
    assert untouched.any() and (~untouched).any()
    assert np.array_equal(g1[untouched], start[untouched])
    if prec == "f":
        gr, nsr, _ = oracle_mod.grid_f(wl)
        assert ns0 == nsr
        assert max_rel(g0, gr) <= 1e-5
    else:
        gr, nsr, _ = oracle_mod.grid_d(wl)
        assert ns0 == nsr
        assert max_rel(g0, gr) <= 1e-12


@pytest.mark.parametrize("G", [1800, 4099])
@pytest.mark.parametrize("tuning", [{}, {"plane_group_mb": 1},
                                    {"plane_group_mb": 1, "items_per_cta": 16},
                                    {"tile_phases": 2},
                                    {"plane_group_mb": 1, "items_per_cta": 16,
                                     "tile_phases": 4}])
@pytest.mark.parametrize("prec", ["f", "d"])
def test_dropin_grid_access_modes(pkg, synthetic, torch, prec, tuning, G):
    """The caller's grid read and written in place by the gridding kernels
    (page-locked, and pageable where the device addresses it) gives the
    device-pointer call's grid, skip count and norm bit for bit, with one
    plane group and with several (a tile's first group reads the host grid,
    its last writes it back), with split heavy tiles (their partial sums
    reduced into the host grid) and with ragged edge tiles.  The copied
    grid agrees bit for bit below 128 MiB; above, its split passes size
    their work items per pass, which changes only the rounding.  With tile
    phases the host grid is read and written per strip of a phase's
    tiles."""
    wl = synthetic.random_uniform_workload(
        "access", 40_000, G, 48, 2, 14, seed=31, cell_size_rad=2.4e-5,
        sigma_frac=0.12, clip_frac=0.45)
    dt = np.float32 if prec == "f" else np.float64
    grid_fn = pkg.grid_f if prec == "f" else pkg.grid_d
    mode = pkg.host_grid_access()
    results = {}
    pkg.set_host_tuning(tuning)
    try:
        for name, m, pinned in (("copy", pkg.GRID_ACCESS_COPY, True),
                                ("pinned", pkg.GRID_ACCESS_PINNED, True),
                                ("pageable", pkg.GRID_ACCESS_PAGEABLE, False)):
            pkg.set_host_grid_access(m)
            g = _start_grid(G, 3, pinned, dt, torch)
            # A page-locked cube is gathered by a kernel in place too.
            w = dataclasses.replace(wl, conv_func=_pinned_like(
                wl.conv_func.astype(dt), torch)) if pinned else wl
            results[name] = grid_fn(w, g, 0.25) + pkg.host_last_transfer()
    finally:
        pkg.set_host_tuning(None)
        pkg.set_host_grid_access(mode)
    # The device-pointer call with the same settings.
    dev = torch.device("cuda", 0)
    tt = torch.float32 if prec == "f" else torch.float64
    plan = pkg.Plan()
    plan.set_tuning(tuning)
    stack = pkg.KernelStack.from_workload(wl, prec)
    d = {k: torch.from_numpy(np.ascontiguousarray(getattr(wl, k), dt)).to(dev)
         for k in ("uu", "vv", "ww", "vis", "weight")}
    grid = torch.from_numpy(_start_grid(G, 3, dtype=dt)).to(dev)
    norm = torch.full((1,), 0.25, dtype=torch.float64, device=dev)
    nskip = torch.zeros(1, dtype=torch.int64, device=dev)
    pkg.grid_wproj_device(plan, stack, d["uu"], d["vv"], d["ww"], d["vis"],
                          d["weight"], dt(wl.cell_size_rad), dt(wl.w_scale), G,
                          grid, norm, nskip)
    torch.cuda.synchronize()
    gd = grid.cpu().numpy()
    assert grid.dtype == tt
    full = G * G * 2 * np.dtype(dt).itemsize
    assert results["copy"][3] > full         # the copy uploads the grid
    assert results["pinned"][3] < results["copy"][3]  # in place: tiles only
    for name in ("pinned", "pageable"):
        g, ns, nm = results[name][:3]
        assert ns == int(nskip.item()) and nm == float(norm.item()), name
        assert np.array_equal(g.view(np.uint8), gd.view(np.uint8)), name
    g, ns, nm = results["copy"][:3]
    assert ns == int(nskip.item())
    if full < (128 << 20):
        assert nm == float(norm.item())
        assert np.array_equal(g.view(np.uint8), gd.view(np.uint8))
    else:
        start = _start_grid(G, 3, dtype=dt)
        assert max_rel(g - start, gd - start) <= (
            1e-6 if prec == "f" else 1e-14)
        assert abs(nm - float(norm.item())) <= 1e-12 * abs(nm)


@pytest.mark.parametrize("pinned", [False, True])
def test_dropin_stack_reuse_follows_the_cube(pkg, synthetic, torch, pinned):
    """The host calls re-lay the kernel stack only when the cube differs
    from the one it was made from.  Gridding with cube A, A again, then B
    (A with one row of taps scaled, in place in the same array), then B
    again must give exactly what fresh stacks give, in every grid access
    mode; a call with another geometry in between forces a fresh stack."""
    wl = synthetic.random_uniform_workload(
        "reuse", 20_000, 1024, 16, 4, 16, seed=43, cell_size_rad=4e-5)
    other = synthetic.random_uniform_workload("other", 200, 512, 8, 2, 8,
                                              seed=44)
    cube_a = wl.conv_func.copy()
    cube_b = cube_a.copy()
    cube_b[:, 1, :, 0] *= np.float32(1.25)
    arr = _pinned_like(cube_a, torch) if pinned else cube_a.copy()
    w = dataclasses.replace(wl, conv_func=arr)
    mode = pkg.host_grid_access()
    try:
        for m in (pkg.GRID_ACCESS_COPY, pkg.GRID_ACCESS_PINNED,
                  pkg.GRID_ACCESS_PAGEABLE):
            pkg.set_host_grid_access(m)
            fresh = {}
            for name, cube in (("a", cube_a), ("b", cube_b)):
                pkg.grid_f(other)                 # another geometry
                arr[...] = cube
                fresh[name] = pkg.grid_f(w)
            arr[...] = cube_a
            pkg.grid_f(other)
            seq = [pkg.grid_f(w), pkg.grid_f(w)]
            arr[...] = cube_b
            seq += [pkg.grid_f(w), pkg.grid_f(w)]
            for got, name in zip(seq, "aabb"):
                g, ns, nm = got
                assert (ns, nm) == fresh[name][1:], (m, name)
                assert np.array_equal(g.view(np.uint8),
                                      fresh[name][0].view(np.uint8)), (m, name)
            assert fresh["a"][2] != fresh["b"][2]
    finally:
        pkg.set_host_grid_access(mode)


def test_dropin_fresh_pageable_grid_is_copied(pkg, synthetic):
    """A freshly allocated pageable grid (np.zeros: its pages not yet
    touched) is copied rather than used in place, where the device would
    fault every page in; once its pages exist it is used in place.  Both
    give the copy's result."""
    G = 2048
    wl = synthetic.random_uniform_workload(
        "fresh", 30_000, G, 32, 2, 12, seed=37, cell_size_rad=3e-5)
    with _access(pkg, pkg.GRID_ACCESS_COPY):
        g0, ns0, nm0 = pkg.grid_f(wl)
        h2d_copy = pkg.host_last_transfer()[0]
    with _access(pkg, pkg.GRID_ACCESS_PAGEABLE):
        g1, ns1, nm1 = pkg.grid_f(wl)       # np.zeros inside grid_f
        h2d_fresh = pkg.host_last_transfer()[0]
        g2 = np.zeros((G, G, 2), np.float32)
        g2[...] = 0.0                        # pages touched
        g2, ns2, nm2 = pkg.grid_f(wl, g2)
        h2d_touched = pkg.host_last_transfer()[0]
    assert h2d_fresh == h2d_copy             # the whole grid went up
    assert h2d_touched < h2d_copy            # in place: touched tiles only
    for g, ns, nm in ((g1, ns1, nm1), (g2, ns2, nm2)):
        assert (ns, nm) == (ns0, nm0)
        assert np.array_equal(g.view(np.uint8), g0.view(np.uint8))


def test_host_phase_times(pkg, synthetic):
    """With profiling on, a host call's phase times are there, its device
    phases add up to about its duration and its host-clock marks are in
    order; off, none are recorded; a call without visibilities leaves
    nothing to report."""
    import time
    wl = synthetic.random_uniform_workload("phases", 50_000, 1024, 16, 2, 8,
                                           seed=47, cell_size_rad=6e-5)
    pkg.grid_f(wl)
    pkg.set_host_profiling(True)
    try:
        t0 = time.perf_counter()
        pkg.grid_f(wl)
        wall = (time.perf_counter() - t0) * 1e3
        ph = pkg.host_phase_ms()
        assert set(ph) == set(pkg.HOST_PHASES)
        assert all(v >= 0.0 for v in ph.values())
        assert ph["grid_tiles"] > 0.0
        device = sum(v for k, v in ph.items() if not k.startswith("host_"))
        assert 0.0 < device <= wall * 1.05 + 0.1
        assert (ph["host_first_work"] <= ph["host_synchronised"]
                <= ph["host_return"] <= wall)
        assert device <= ph["host_synchronised"] * 1.05 + 0.1
        marks = pkg.host_last_call_ms()
        assert marks["return"] == pytest.approx(ph["host_return"], abs=1e-3)
        empty = dataclasses.replace(wl, uu=wl.uu[:0], vv=wl.vv[:0],
                                    ww=wl.ww[:0], vis=wl.vis[:0],
                                    weight=wl.weight[:0])
        pkg.grid_f(empty)
        with pytest.raises(pkg.GridError):
            pkg.host_phase_ms()
    finally:
        pkg.set_host_profiling(False)
    t0 = time.perf_counter()
    pkg.grid_f(wl)
    wall = (time.perf_counter() - t0) * 1e3
    with pytest.raises(pkg.GridError):
        pkg.host_phase_ms()
    # The host-clock marks are kept without profiling too.
    marks = pkg.host_last_call_ms()
    assert 0.0 <= marks["first_work"] <= marks["synchronised"] \
        <= marks["return"] <= wall


def test_grid_access_mode_setting(pkg):
    mode = pkg.host_grid_access()
    assert mode == pkg.GRID_ACCESS_PAGEABLE   # the default
    try:
        for m in (pkg.GRID_ACCESS_COPY, pkg.GRID_ACCESS_PINNED):
            pkg.set_host_grid_access(m)
            assert pkg.host_grid_access() == m
        with pytest.raises(pkg.GridError):
            pkg.set_host_grid_access(3)
    finally:
        pkg.set_host_grid_access(mode)


def test_dropin_transfer_bytes(pkg, synthetic, torch):
    """The drop-in reports what it copied: everything up, and only the
    touched spans of the grid down (a centre patch here)."""
    G = 1024
    wl = synthetic.random_uniform_workload(
        "xfer", 10_000, G, 16, 2, 8, seed=9, cell_size_rad=6e-5,
        sigma_frac=0.01, clip_frac=0.03)
    with _access(pkg, pkg.GRID_ACCESS_COPY):
        pkg.grid_f(wl)
        h2d, d2h = pkg.host_last_transfer()
    n = wl.num_points
    # Of the cube only each plane's square up to the last row and column
    # the stack preparation reads goes up.
    omax = (wl.oversample + 1) // 2
    ext = np.minimum(wl.conv_size_half,
                     1 + np.maximum(wl.support * wl.oversample + omax,
                                    (wl.support + 1 + (omax >= wl.oversample))
                                    * wl.oversample - 1))
    cube = int((ext.astype(np.int64) ** 2).sum()) * 8
    assert cube < wl.conv_func.nbytes
    stack_and_inputs = cube + wl.num_w_planes * 20 + 24 * n + 8
    assert h2d == stack_and_inputs + 8 * G * G
    assert 0 < d2h < G * G * 8 // 10
    # A pinned grid copied moves the same bytes; addressed in place, only
    # the tiles that hold records cross the link, once each way (no more
    # than the spans the copy brings back, which cover those tiles).
    pinned = _start_grid(G, 1, True, torch=torch)
    with _access(pkg, pkg.GRID_ACCESS_COPY):
        pkg.grid_f(wl, pinned)
        assert pkg.host_last_transfer() == (h2d, d2h)
    with _access(pkg, pkg.GRID_ACCESS_PINNED):
        pkg.grid_f(wl, pinned)
        h2d_p, d2h_p = pkg.host_last_transfer()
    tiles = h2d_p - stack_and_inputs
    assert 0 < tiles <= d2h - 8 - 8 - 4 - 4 * 7 - 8 - 8
    assert tiles % 8 == 0 and tiles % (32 * 8) == 0
    assert d2h_p == tiles + 8 + 8 + 4 + 4 * 7 + 8 + 8
    empty = dataclasses.replace(wl, uu=wl.uu[:0], vv=wl.vv[:0],
                                ww=wl.ww[:0], vis=wl.vis[:0],
                                weight=wl.weight[:0])
    for m in (pkg.GRID_ACCESS_COPY, pkg.GRID_ACCESS_PAGEABLE):
        with _access(pkg, m):
            pkg.grid_f(empty)
            h2d, d2h = pkg.host_last_transfer()
        assert h2d == cube + wl.num_w_planes * 20 + 8
        assert d2h == 8 + 8 + 4


@pytest.mark.parametrize("mode", ["copy", "in_place"])
def test_dropin_nothing_gridded_leaves_grid(pkg, synthetic, torch, mode):
    """Every visibility off the grid (all skipped), and no visibilities at
    all: the grid comes back bit-for-bit unchanged and the norm as given."""
    with _access(pkg, pkg.GRID_ACCESS_COPY if mode == "copy"
                 else pkg.GRID_ACCESS_PAGEABLE):
        _nothing_gridded(pkg, synthetic, torch)


def _nothing_gridded(pkg, synthetic, torch):
    G = 512
    wl = synthetic.random_uniform_workload("off_grid", 5_000, G, 8, 2, 6,
                                           seed=5)
    far = np.float32(10.0 / wl.cell_size_rad)
    wl = dataclasses.replace(wl, uu=(wl.uu + far).astype(np.float32))
    start = _start_grid(G, 4)
    g, ns, nm = pkg.grid_f(wl, start.copy(), 3.5)
    assert ns == wl.num_points
    assert nm == 3.5
    assert np.array_equal(g, start)
    g, ns, nm = pkg.grid_f(wl, _start_grid(G, 4, True, torch=torch), 3.5)
    assert ns == wl.num_points and nm == 3.5
    assert np.array_equal(g, start)
    empty = dataclasses.replace(wl, uu=wl.uu[:0], vv=wl.vv[:0], ww=wl.ww[:0],
                                vis=wl.vis[:0], weight=wl.weight[:0])
    g, ns, nm = pkg.grid_f(empty, start.copy(), 1.25)
    assert ns == 0 and nm == 1.25
    assert np.array_equal(g, start)


def test_dropin_concurrent_threads(pkg, synthetic, torch):
    """Host-pointer calls from several threads at once (ctypes releases the
    GIL, so they really overlap) are serialised per device and give the
    same results, bit for bit, as the same calls made one after another."""
    from concurrent.futures import ThreadPoolExecutor
    wls = [synthetic.random_uniform_workload(f"thr{i}", 20_000 + 5_000 * i,
                                             512 + 128 * i, 16, 2, 8,
                                             seed=30 + i, cell_size_rad=1e-4)
           for i in range(4)]
    serial = [pkg.grid_f(wl) for wl in wls]
    with ThreadPoolExecutor(max_workers=4) as ex:
        futures = [ex.submit(pkg.grid_f, wl) for wl in wls * 2]
        results = [f.result() for f in futures]
    for i, (g, ns, nm) in enumerate(results):
        g0, ns0, nm0 = serial[i % 4]
        assert ns == ns0 and nm == nm0
        assert np.array_equal(g.view(np.uint32), g0.view(np.uint32))


def test_wide_support_table_takes_the_64_bit_record_count(pkg, oracle_mod,
                                                          synthetic, torch):
    """A call whose support table could make more records than 32-bit
    indices hold (2 M visibilities x up to 2268 records each with a plane
    of support 1000) counts its records in 64 bits before sizing the sort;
    here every visibility lies in the support-4 plane, so the call proceeds
    and grids as the FP64 oracle says."""
    wl = synthetic.random_uniform_workload("wide", 2_000_000, 4096, 2, 4,
                                           1000, seed=21,
                                           cell_size_rad=2.0e-5)
    wl.ww = np.zeros_like(wl.ww)
    assert int(wl.support.max()) == 1000
    g, ns, nm = pkg.grid_f(wl)
    g64, ns64, nm64 = oracle_mod.grid_f_fp64acc_mt(wl)
    assert ns == ns64
    assert abs(nm - nm64) <= 1e-12 * abs(nm64)
    assert max_rel(g, g64) <= 1e-5
