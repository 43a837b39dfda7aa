"""GPU tests of uniform weighting and of host-pointer degridding.

Uniform weighting (reference utils/oskar_grid_weights.c:38-172) is integer
placement plus serial FP32/FP64 additions and a division, so the GPU result
must be bit-identical to the reference's: density grid, re-weighted
visibilities and skip counts, on the reference's golden vectors and on
synthetic cases (many points per cell, off-grid and NaN coordinates,
accumulation onto an existing grid, empty input).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden, max_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.dtype == b.dtype and a.shape == b.shape
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("name", ["weights_f", "weights_d"])
def test_weights_match_reference_golden(pkg, torch, name):
    _, z = load_golden(name)
    real = z["uu"].dtype.type
    G = int(z["grid_size"])
    cell = real(z["cell_size_rad"])
    dens, ns = pkg.grid_weights_write(z["uu"], z["vv"], z["weight"], cell, G)
    assert ns == int(z["num_skipped_write"])
    _same(dens, z["density"])
    out = np.full(z["uu"].shape[0], -7.0, real)
    ns = pkg.grid_weights_read(z["uu"], z["vv"], z["weight"], out, cell, G,
                               dens)
    assert ns == int(z["num_skipped_read"])
    _same(out, z["weight_out"])


def _points(n, G, cell, dtype, seed):
    """Radially concentrated uv (many points share cells near the centre),
    some off the grid."""
    rng = np.random.default_rng(seed)
    r = np.abs(rng.normal(0.0, 0.15, n)) * (G / 2) / (G * cell)
    th = rng.uniform(0, 2 * np.pi, n)
    uu = (r * np.cos(th)).astype(dtype)
    vv = (r * np.sin(th)).astype(dtype)
    uu[: n // 50] *= 8.0                      # off the grid
    w = rng.uniform(0.5, 1.5, n).astype(dtype)
    return uu, vv, w


def test_weights_nan_coordinates_are_skipped(pkg, torch):
    """A NaN coordinate has no cell: the point is counted as skipped and
    changes neither the density nor its weight_out entry.  (The reference's
    int conversion of NaN is platform-dependent: INT_MIN, hence skipped, on
    x86.)"""
    G, cell = 64, np.float32(1e-3)
    uu, vv, w = _points(2000, G, cell, np.float32, 5)
    base, ns0 = pkg.grid_weights_write(uu, vv, w, cell, G)
    uu2, vv2, w2 = uu.copy(), vv.copy(), w.copy()
    uu2[100:110] = np.nan
    vv2[200:205] = np.nan
    g, ns = pkg.grid_weights_write(uu2, vv2, w2, cell, G)
    keep = np.ones(2000, bool)
    keep[100:110] = keep[200:205] = False
    ref, _ = pkg.grid_weights_write(uu[keep], vv[keep], w[keep], cell, G)
    assert ns == ns0 + 15
    _same(g, ref)
    out = np.full(2000, 3.0, np.float32)
    assert pkg.grid_weights_read(uu2, vv2, w2, out, cell, G, g) == ns
    assert (out[100:110] == 3.0).all() and (out[200:205] == 3.0).all()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_weights_match_oracle_synthetic(pkg, oracle_mod, torch, dtype):
    G, cell = 512, dtype(2.0e-4)
    uu, vv, w = _points(300_000, G, cell, dtype, 3)
    start = np.random.default_rng(4).uniform(0, 3, (G, G)).astype(dtype)
    g_ref, ns_ref = oracle_mod.weights_write(uu, vv, w, cell, G,
                                             start.copy())
    g, ns = pkg.grid_weights_write(uu, vv, w, cell, G, start.copy())
    assert ns == ns_ref > 0
    _same(g, g_ref)
    out_ref = np.full_like(w, 9.0)
    out = np.full_like(w, 9.0)
    nr = oracle_mod.weights_read(uu, vv, w, out_ref, cell, G, g_ref)
    assert pkg.grid_weights_read(uu, vv, w, out, cell, G, g) == nr == ns
    _same(out, out_ref)


def test_weights_one_crowded_cell(pkg, oracle_mod, torch):
    """100,000 points in one cell: the run is added in point order."""
    n, G, cell = 100_000, 64, np.float32(1e-3)
    rng = np.random.default_rng(8)
    uu = rng.uniform(-0.2, 0.2, n).astype(np.float32)
    vv = rng.uniform(-0.2, 0.2, n).astype(np.float32)
    w = rng.uniform(0.0, 1.0, n).astype(np.float32)
    g_ref, _ = oracle_mod.weights_write(uu, vv, w, cell, G)
    g, ns = pkg.grid_weights_write(uu, vv, w, cell, G)
    assert ns == 0 and np.count_nonzero(g) == 1
    _same(g, g_ref)


def test_weights_empty_and_all_off_grid(pkg, torch):
    G, cell = 32, np.float32(1e-3)
    e = np.zeros(0, np.float32)
    g, ns = pkg.grid_weights_write(e, e, e, cell, G)
    assert ns == 0 and not g.any()
    far = np.full(10, 1e9, np.float32)
    g, ns = pkg.grid_weights_write(far, far, np.ones(10, np.float32), cell, G)
    assert ns == 10 and not g.any()
    out = np.full(10, 5.0, np.float32)
    assert pkg.grid_weights_read(far, far, np.ones(10, np.float32), out, cell,
                                 G, g) == 10
    assert (out == 5.0).all()


def test_weights_device_equals_host(pkg, torch):
    G, cell = 256, np.float32(3e-4)
    uu, vv, w = _points(50_000, G, cell, np.float32, 11)
    g_host, ns_host = pkg.grid_weights_write(uu, vv, w, cell, G)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    plan = pkg.Plan()
    g = torch.zeros((G, G), dtype=torch.float32, device="cuda")
    ns = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    pkg.grid_weights_write_device(plan, dev(uu), dev(vv), dev(w), cell, G, g,
                                  ns)
    torch.cuda.synchronize()
    assert int(ns.item()) == ns_host
    _same(g.cpu().numpy(), g_host)
    out = torch.full((uu.shape[0],), 2.0, dtype=torch.float32, device="cuda")
    pkg.grid_weights_read_device(plan, dev(uu), dev(vv), dev(w), out, cell, G,
                                 g, ns)
    out_host = np.full_like(w, 2.0)
    pkg.grid_weights_read(uu, vv, w, out_host, cell, G, g_host)
    torch.cuda.synchronize()
    _same(out.cpu().numpy(), out_host)


def test_degrid_host_equals_device_and_oracle(pkg, oracle_mod, synthetic,
                                              torch):
    wl = synthetic.config0().subset(20_000)
    rng = np.random.default_rng(2)
    grid = rng.standard_normal((wl.grid_size, wl.grid_size, 2)) \
        .astype(np.float32)
    host = pkg.degrid_f(wl, grid)
    stack = pkg.KernelStack.from_workload(wl, "f")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    out = torch.zeros((wl.num_points, 2), dtype=torch.float32, device="cuda")
    pkg.degrid_wproj_device(pkg.Plan(), stack, dev(wl.uu), dev(wl.vv),
                            dev(wl.ww), np.float32(wl.cell_size_rad),
                            np.float32(wl.w_scale), wl.grid_size, dev(grid),
                            out)
    torch.cuda.synchronize()
    _same(host, out.cpu().numpy())
    ref = oracle_mod.degrid_fp64(wl, grid)
    assert max_rel(host, ref) <= 1e-5


@pytest.mark.parametrize("prec", ["f", "d"])
def test_degrid_host_grid_access_modes(pkg, synthetic, torch, prec):
    """The host degridding call reads a grid the device addresses in place
    (page-locked, or resident pageable memory) and copies any other; the
    visibilities are the same bit for bit in every mode and tile order."""
    wl = synthetic.config0().subset(20_000)
    dt = np.float32 if prec == "f" else np.float64
    rng = np.random.default_rng(5)
    grid = rng.standard_normal((wl.grid_size, wl.grid_size, 2)).astype(dt)
    pinned = torch.empty(grid.shape, dtype=getattr(torch, grid.dtype.name),
                         pin_memory=True).numpy()
    pinned[...] = grid
    args = (wl.num_w_planes, wl.support, wl.oversample, wl.conv_size_half,
            wl.conv_func, np.asarray(wl.uu, dt), np.asarray(wl.vv, dt),
            np.asarray(wl.ww, dt), dt(wl.cell_size_rad), dt(wl.w_scale),
            wl.grid_size)
    mode = pkg.host_grid_access()
    outs = []
    try:
        for m, g in ((pkg.GRID_ACCESS_COPY, grid),
                     (pkg.GRID_ACCESS_PINNED, pinned),
                     (pkg.GRID_ACCESS_PAGEABLE, grid)):
            pkg.set_host_grid_access(m)
            for order in (0, 1):
                pkg.set_host_tuning({"tile_order": order})
                outs.append(pkg.degrid_wproj(*args, g))
    finally:
        pkg.set_host_tuning(None)
        pkg.set_host_grid_access(mode)
    for o in outs[1:]:
        assert np.array_equal(o.view(np.uint8), outs[0].view(np.uint8))
