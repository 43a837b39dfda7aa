"""CPU tests: the oracle is pinned to the reference.

The oracle (oracle/oskar_grid_oracle.c) restates the reference's serial
gridder.  It must reproduce the reference's golden outputs bit for bit
(num_skipped, norm and every grid word), and -- where the reference source
tree is present -- the compiled reference itself on fresh inputs.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import golden_names, load_golden, max_rel


@pytest.mark.parametrize("name", [n for n in golden_names()
                                  if not n.startswith("weights")])
def test_oracle_matches_golden_bit_exact(oracle_mod, name):
    wl, z = load_golden(name)
    if str(z["precision"]) == "f":
        g, ns, nm = oracle_mod.grid_f(wl, z["grid_in"].copy(),
                                      float(z["norm_in"]))
    else:
        g, ns, nm = oracle_mod.grid_d(wl, z["grid_in"].copy(),
                                      float(z["norm_in"]))
    assert ns == int(z["num_skipped"])
    assert nm == float(z["norm_out"])          # bit-exact FP64
    assert np.array_equal(g.view(np.uint8), z["grid_out"].view(np.uint8))


@pytest.mark.parametrize("name", ["small_f", "edges_f", "os3_f"])
def test_multithreaded_oracle_bit_exact(oracle_mod, name):
    wl, z = load_golden(name)
    g, ns, nm = oracle_mod.grid_f_mt(wl, z["grid_in"].copy(),
                                     float(z["norm_in"]), threads=4)
    assert ns == int(z["num_skipped"])
    assert nm == float(z["norm_out"])
    assert np.array_equal(g.view(np.uint8), z["grid_out"].view(np.uint8))


@pytest.mark.parametrize("name", ["weights_f", "weights_d"])
def test_weights_oracle_matches_golden(oracle_mod, name):
    _, z = load_golden(name)
    real = z["uu"].dtype.type
    suffix = "f" if real == np.float32 else "d"
    L = oracle_mod.lib()
    G = int(z["grid_size"])
    dens = np.zeros((G, G), real)
    ns = ctypes.c_size_t(0)
    n = z["uu"].shape[0]
    getattr(L, f"oracle_grid_weights_write_{suffix}")(
        n, z["uu"], z["vv"], z["weight"], real(z["cell_size_rad"]), G,
        ctypes.byref(ns), dens.reshape(-1))
    assert ns.value == int(z["num_skipped_write"])
    assert np.array_equal(dens.view(np.uint8), z["density"].view(np.uint8))
    out = np.full(n, -7.0, real)
    getattr(L, f"oracle_grid_weights_read_{suffix}")(
        n, z["uu"], z["vv"], z["weight"], out, real(z["cell_size_rad"]), G,
        ctypes.byref(ns), dens.reshape(-1))
    assert ns.value == int(z["num_skipped_read"])
    assert np.array_equal(out.view(np.uint8), z["weight_out"].view(np.uint8))


def test_placement_matches_serial_skip_count(oracle_mod):
    wl, z = load_golden("small_f")
    p = oracle_mod.place(wl, "f")
    assert p["num_skipped"] == int(z["num_skipped"])
    assert p["ou"].min() >= -2 and p["ou"].max() <= 2
    assert p["plane"].max() == wl.num_w_planes - 1   # clamp exercised


def test_fp64_yardstick_close_to_reference_f(oracle_mod):
    """The FP64-accumulation oracle agrees with the reference _f to FP32
    rounding, with identical placement (same skip count, same norm)."""
    wl, z = load_golden("small_f")
    g64, ns, nm = oracle_mod.grid_f_fp64acc(
        wl, z["grid_in"].astype(np.float64), float(z["norm_in"]))
    assert ns == int(z["num_skipped"])
    assert nm == float(z["norm_out"])
    assert max_rel(z["grid_out"], g64) < 1e-5


@pytest.mark.parametrize("name", ["small_f", "edges_f", "os3_f"])
def test_multithreaded_fp64_yardstick_bit_exact(oracle_mod, name):
    """The host-threaded FP64 yardstick (the benchmark's error check) gives
    the serial one's grid, norm and skip count bit for bit."""
    wl, z = load_golden(name)
    g1, ns1, nm1 = oracle_mod.grid_f_fp64acc(
        wl, z["grid_in"].astype(np.float64), float(z["norm_in"]))
    g4, ns4, nm4 = oracle_mod.grid_f_fp64acc_mt(
        wl, z["grid_in"].astype(np.float64), float(z["norm_in"]), threads=4)
    assert ns4 == ns1 == int(z["num_skipped"])
    assert nm4 == nm1
    assert np.array_equal(g4.view(np.uint8), g1.view(np.uint8))


def test_adjoint_oracle_dot_product(oracle_mod):
    """<G x, y> = <x, G^H y> for the FP64 oracle pair."""
    wl, _ = load_golden("small_f")
    rng = np.random.default_rng(5)
    x = rng.standard_normal((wl.num_points, 2))
    y = rng.standard_normal((wl.grid_size, wl.grid_size, 2))
    wl1 = wl.subset(wl.num_points)
    wl1.vis = x.astype(np.float32)
    wl1.weight = np.ones(wl.num_points, np.float32)
    gx, _, _ = oracle_mod.grid_f_fp64acc(wl1)
    # Use the float32-rounded x on both sides.
    xs = wl1.vis.astype(np.float64)
    aty = oracle_mod.degrid_fp64(wl1, y)
    lhs = (gx[..., 0] * y[..., 0] + gx[..., 1] * y[..., 1]).sum()
    rhs = (xs[:, 0] * aty[:, 0] + xs[:, 1] * aty[:, 1]).sum()
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


def test_adjoint_oracle_dot_product_fp64(oracle_mod, synthetic):
    """<G x, y> = <x, G^H y> for the FP64 gridding map and its FP64
    adjoint (FP64 placement and cube)."""
    wl = synthetic.random_uniform_workload("adj_d", 1500, 256, 12, 1, 8,
                                           seed=8, cell_size_rad=1.5e-4)
    rng = np.random.default_rng(6)
    x = rng.standard_normal((wl.num_points, 2)).astype(np.float32)
    y = rng.standard_normal((wl.grid_size, wl.grid_size, 2))
    wl1 = wl.subset(wl.num_points)
    wl1.vis = x
    wl1.weight = np.ones(wl.num_points, np.float32)
    gx, ns, _ = oracle_mod.grid_d(wl1)
    assert ns < wl.num_points
    aty = oracle_mod.degrid_d(wl1, y)
    xs = x.astype(np.float64)
    lhs = (gx[..., 0] * y[..., 0] + gx[..., 1] * y[..., 1]).sum()
    rhs = (xs[:, 0] * aty[:, 0] + xs[:, 1] * aty[:, 1]).sum()
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.skipif("not __import__('oracle').ref_available()",
                    reason="reference source tree not present")
@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_matches_compiled_reference(oracle_mod, synthetic, seed):
    wl = synthetic.random_uniform_workload(
        "fresh", 4000, 192, 12, 1, 9, seed=seed, cell_size_rad=6e-4,
        w_max=500.0, sigma_frac=0.18, clip_frac=0.55)
    a, nsa, nma = oracle_mod.grid_f(wl, use_reference=True)
    b, nsb, nmb = oracle_mod.grid_f(wl)
    assert (nsa, nma) == (nsb, nmb)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    a, nsa, nma = oracle_mod.grid_d(wl, use_reference=True)
    b, nsb, nmb = oracle_mod.grid_d(wl)
    assert (nsa, nma) == (nsb, nmb)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("name", ["small_f", "edges_f", "os3_f"])
def test_promoted_fp64_oracle_is_the_serial_d(oracle_mod, name):
    """The host-threaded FP64 oracle on promoted FP32 inputs (the error
    report's `_d` column) equals the serial oskar_grid_wproj_d restatement
    on the promoted arrays bit for bit -- and the compiled reference's _d
    where it is built."""
    wl, _ = load_golden(name)
    g, ns, nm = oracle_mod.grid_d_promoted_mt(wl, threads=3)
    g2, ns2, nm2 = oracle_mod.grid_d(wl)
    assert ns == ns2 and nm == nm2
    assert np.array_equal(g.view(np.uint8), g2.view(np.uint8))
    if oracle_mod.ref_available():
        g3, ns3, nm3 = oracle_mod.grid_d(wl, use_reference=True)
        assert ns == ns3 and nm == nm3
        assert np.array_equal(g.view(np.uint8), g3.view(np.uint8))


def test_placement_disagreement_count(oracle_mod, synthetic):
    """The count of visibilities placed differently by the FP32 and the
    FP64 rules matches an element-wise comparison of the two placements,
    and is zero where FP32 placement is exact (integer cell positions)."""
    wl = synthetic.config0().subset(30_000)
    n, n_gridded = oracle_mod.placement_disagreements(wl)
    pf, pd = oracle_mod.place(wl, "f"), oracle_mod.place(wl, "d")
    ref = sum(int(np.any([pf[k][i] != pd[k][i] for k in
                          ("gu", "gv", "ou", "ov", "plane", "skipped")]))
              for i in range(wl.num_points))
    assert n == ref and 0 <= n_gridded <= n
    # Coordinates that place on exact cell centres with w on exact plane
    # squares: both rule sets agree everywhere.
    G, cell = wl.grid_size, wl.cell_size_rad
    rng = np.random.default_rng(3)
    k = rng.integers(-200, 200, (2, 1000))
    scale = np.float32(G * np.float32(cell))
    exact = synthetic.Workload(**{**wl.__dict__,
        "uu": (k[0] / scale).astype(np.float32),
        "vv": (k[1] / scale).astype(np.float32),
        "ww": np.zeros(1000, np.float32), "vis": wl.vis[:1000],
        "weight": wl.weight[:1000]})
    assert oracle_mod.placement_disagreements(exact) == (0, 0)
