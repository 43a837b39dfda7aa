"""GPU parity tests on the SKA-LOW-shaped configuration (run with -m gpu).

The workload is the SKA-LOW EL56-82 array of the benchmark's default
configuration (512 stations, 601 w-planes, supports 4..72, an 8192^2 grid)
sampled at 60 time steps instead of 240: 7,848,960 visibilities with the
same uv density, w distribution and support table.  Its largest footprints
are 145 x 145 cells, so they span five to nineteen tile columns (with the
32-, 16- and 8-wide tile shapes) and three to five tile rows, and its slab
rows use the widest pitch the stack holds.

Bars (written in each assertion):
* cell, offset, plane and skip assignment: bit-exact with the reference's
  FP32 rules (and FP64 rules for the FP64 placement);
* num_skipped exact; norm relative 1e-12 + N * 2^-53 against the oracle's
  FP64 norm (the oracle adds N = 7.8 M positive terms serially, whose own
  rounding can reach N * 2^-53 relative; the GPU adds them by a fixed tree);
* grid max |err| / max |grid| <= 1e-5 against the FP64-accumulation oracle
  with the FP32 placement (the metric's bound);
* grid against the reference's own FP32 gridder _f: max-rel within
  max(1e-5, err_f + 1e-6), where err_f is _f's own max-rel error against
  the FP64 oracle.  The reference's FP32 sums drift past 1e-5 from the
  FP64 answer at this size (about 1.1e-5 here, 3e-5 on the 240-sample
  workload), so a flat 1e-5 against _f would test _f's rounding rather
  than this gridder; the stated bound is that drift plus 1e-6.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import max_rel, rms_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


@pytest.fixture(scope="module")
def skalow(synthetic, oracle_mod):
    """The workload, its FP32 placement and the two host oracles."""
    wl = synthetic.WORKLOADS["cfg2s"]()
    place = oracle_mod.place(wl, "f")
    g64, ns64, nm64 = oracle_mod.grid_f_fp64acc_mt(wl)
    gf, nsf, nmf = oracle_mod.grid_f_mt(wl)
    return dict(wl=wl, place=place, g64=g64, ns64=ns64, nm64=nm64, gf=gf,
                nsf=nsf, nmf=nmf, err_f=max_rel(gf, g64))


def _norm_tol(n):
    """Relative bound between two FP64 sums of n positive terms taken in
    different orders: 1e-12 plus the serial sum's own rounding bound."""
    return 1e-12 + n * 2.0 ** -53


def _dev(torch, a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def test_skalow_covers_supports_to_72(skalow):
    """The case reaches the large-support regime it is here for."""
    wl, p = skalow["wl"], skalow["place"]
    s = wl.support[p["plane"]][p["skipped"] == 0]
    assert s.max() == 72
    assert (s > 36).sum() > 10_000
    assert (s >= 60).sum() > 0


@pytest.mark.parametrize("prec", ["f", "d"])
def test_skalow_placement_bit_exact(pkg, oracle_mod, skalow, torch, prec):
    wl = skalow["wl"]
    dt = torch.float32 if prec == "f" else torch.float64
    cast = np.float32 if prec == "f" else float
    stack = pkg.KernelStack.from_workload(wl, prec)
    out = pkg.place_wproj_device(
        stack, _dev(torch, wl.uu, dt), _dev(torch, wl.vv, dt),
        _dev(torch, wl.ww, dt), cast(wl.cell_size_rad), cast(wl.w_scale),
        wl.grid_size).cpu().numpy()
    p = skalow["place"] if prec == "f" else oracle_mod.place(wl, "d")
    assert np.array_equal(out[:, 5] & 1, p["skipped"])
    keep = p["skipped"] == 0
    for col, key in enumerate(("gu", "gv", "ou", "ov", "plane")):
        assert np.array_equal(out[keep, col], p[key][keep]), key


@pytest.mark.parametrize("tile_u,phases", [(0, 0), (32, 0), (16, 0), (8, 0),
                                           (32, 2), (32, 4), (32, 8)])
def test_skalow_grid_vs_oracles(pkg, skalow, torch, tile_u, phases):
    """Device-pointer call, automatic and forced tile shapes, one, two, four
    and eight tile phases."""
    wl = skalow["wl"]
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    plan.set_tuning({"tile_u": tile_u, "tile_phases": phases})
    G = wl.grid_size
    grid = torch.zeros((G, G, 2), dtype=torch.float32, device="cuda")
    norm = torch.zeros(1, dtype=torch.float64, device="cuda")
    ns = torch.zeros(1, dtype=torch.int64, device="cuda")
    pkg.grid_wproj_device(plan, stack, _dev(torch, wl.uu), _dev(torch, wl.vv),
                          _dev(torch, wl.ww), _dev(torch, wl.vis),
                          _dev(torch, wl.weight),
                          np.float32(wl.cell_size_rad),
                          np.float32(wl.w_scale), G, grid, norm, ns)
    torch.cuda.synchronize()
    g = grid.cpu().numpy()
    assert int(ns.item()) == skalow["ns64"] == skalow["nsf"]
    assert abs(norm.item() - skalow["nm64"]) <= \
        _norm_tol(wl.num_points) * abs(skalow["nm64"])
    err = max_rel(g, skalow["g64"])
    err_rms = rms_rel(g, skalow["g64"])
    tol_f = max(1e-5, skalow["err_f"] + 1e-6)
    err_vs_f = max_rel(g, skalow["gf"])
    print(f"tile_u {tile_u} phases {phases}: vs FP64 max {err:.3e} rms {err_rms:.3e}; "
          f"vs _f {err_vs_f:.3e} (bound {tol_f:.3e}, _f vs FP64 "
          f"{skalow['err_f']:.3e})")
    assert err <= 1e-5
    assert err_rms <= err
    assert err_vs_f <= tol_f
    st = plan.stats()
    if tile_u:
        assert st["tile_u"] == tile_u


def test_skalow_dropin_host_call(pkg, skalow, torch):
    """The drop-in oskar_grid_wproj_f on host arrays, accumulating into a
    non-zero grid and norm."""
    wl = skalow["wl"]
    rng = np.random.default_rng(11)
    G = wl.grid_size
    grid0 = np.zeros((G, G, 2), np.float32)
    rows = rng.integers(0, G, 64)
    grid0[rows, rows] = rng.standard_normal((64, 2)).astype(np.float32)
    grid = grid0.copy()
    ns, nm = pkg.oskar_grid_wproj_f(
        wl.num_w_planes, wl.support, wl.oversample, wl.conv_size_half,
        wl.conv_func, wl.num_points, wl.uu, wl.vv, wl.ww, wl.vis, wl.weight,
        np.float32(wl.cell_size_rad), np.float32(wl.w_scale), G, grid, 2.5)
    assert ns == skalow["nsf"]
    assert abs(nm - (2.5 + skalow["nm64"])) <= \
        _norm_tol(wl.num_points) * abs(skalow["nm64"])
    expect = skalow["g64"] + grid0
    assert max_rel(grid, expect) <= 1e-5


@pytest.fixture(scope="module")
def skalow_full(synthetic):
    """The benchmark's default workload itself: 31,395,840 visibilities."""
    return synthetic.WORKLOADS["cfg2"]()


def test_full_skalow_linearity_skips_and_macs(pkg, oracle_mod, skalow_full,
                                              torch):
    """Properties that hold at any size, on the full SKA-LOW workload:
    doubling the amplitudes doubles the grid exactly (every operation on
    the path is exact under a power-of-two scale), the skip count equals
    the oracle's FP32 placement count and the complex-MAC count its
    sum of (2 s + 1)^2 over the gridded visibilities."""
    wl = skalow_full
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    G = wl.grid_size
    uu, vv, ww = _dev(torch, wl.uu), _dev(torch, wl.vv), _dev(torch, wl.ww)
    weight = _dev(torch, wl.weight)
    outs = []
    for scale in (1.0, 2.0):
        grid = torch.zeros((G, G, 2), dtype=torch.float32, device="cuda")
        norm = torch.zeros(1, dtype=torch.float64, device="cuda")
        ns = torch.zeros(1, dtype=torch.int64, device="cuda")
        pkg.grid_wproj_device(plan, stack, uu, vv, ww,
                              _dev(torch, wl.vis * np.float32(scale)), weight,
                              np.float32(wl.cell_size_rad),
                              np.float32(wl.w_scale), G, grid, norm, ns)
        torch.cuda.synchronize()
        outs.append((grid, int(ns.item())))
    assert torch.equal(outs[1][0], 2 * outs[0][0])
    assert outs[0][1] == outs[1][1] == oracle_mod.place(wl)["num_skipped"]
    assert plan.stats()["num_macs"] == oracle_mod.mac_count(wl)


def test_full_skalow_adjoint_dot_product(pkg, skalow_full, torch):
    """<G x, y> = <x, G^H y> on the full SKA-LOW workload with random
    complex x and y, FP32 forward and adjoint: relative 1e-6."""
    wl = skalow_full
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    G = wl.grid_size
    uu, vv, ww = _dev(torch, wl.uu), _dev(torch, wl.vv), _dev(torch, wl.ww)
    gen = torch.Generator(device="cuda").manual_seed(17)
    x = torch.randn((wl.num_points, 2), generator=gen, device="cuda")
    y = torch.randn((G, G, 2), generator=gen, device="cuda")
    gx = torch.zeros((G, G, 2), dtype=torch.float32, device="cuda")
    pkg.grid_wproj_device(plan, stack, uu, vv, ww, x,
                          torch.ones(wl.num_points, device="cuda"),
                          np.float32(wl.cell_size_rad),
                          np.float32(wl.w_scale), G, gx,
                          torch.zeros(1, dtype=torch.float64, device="cuda"),
                          torch.zeros(1, dtype=torch.int64, device="cuda"))
    ghy = torch.empty((wl.num_points, 2), dtype=torch.float32, device="cuda")
    pkg.degrid_wproj_device(plan, stack, uu, vv, ww,
                            np.float32(wl.cell_size_rad),
                            np.float32(wl.w_scale), G, y, ghy)
    torch.cuda.synchronize()

    def cdot(a, b):
        a, b = a.double(), b.double()
        re = (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]).sum()
        im = (a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]).sum()
        return complex(re.item(), im.item())

    lhs, rhs = cdot(gx, y), cdot(x, ghy)
    rel = abs(lhs - rhs) / abs(lhs)
    print(f"full SKA-LOW dot-product test: relative mismatch {rel:.2e}")
    assert rel <= 1e-6
