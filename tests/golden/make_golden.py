"""Generates the golden vectors in this folder from the reference itself.

Runs the reference's own serial gridder and uniform-weighting functions
(oskar_grid_wproj.c and utils/oskar_grid_weights.c of the reference,
compiled from its source into oracle/_ref/libref.so by oracle/Makefile) on
small seeded inputs, and stores inputs and outputs as compressed .npz files.
The reference has no golden vectors or known-answer tests of its own for this
path, so these fixtures are how the oracle and the GPU library are pinned
without the reference tree present.

Usage (where the reference source is available):
    make -C oracle all ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402

synthetic = importlib.import_module("gpu-gridding_gb300.synthetic")


def _ref_grid(wl, real, grid0, norm0):
    grid = grid0.copy()
    if real == np.float32:
        g, ns, nm = oracle.grid_f(wl, grid, norm0, use_reference=True)
    else:
        g, ns, nm = oracle.grid_d(wl, grid, norm0, use_reference=True)
    return g, ns, nm


def _save(name, wl, real, seed, grid0_scale=0.5, norm0=1.25):
    rng = np.random.Generator(np.random.PCG64(seed))
    grid0 = (rng.standard_normal((wl.grid_size, wl.grid_size, 2)) *
             grid0_scale).astype(real)
    g, ns, nm = _ref_grid(wl, real, grid0, norm0)
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"),
        precision=np.array("f" if real == np.float32 else "d"),
        num_w_planes=wl.num_w_planes, support=wl.support,
        oversample=wl.oversample, conv_size_half=wl.conv_size_half,
        conv_func=wl.conv_func.astype(real), uu=wl.uu.astype(real),
        vv=wl.vv.astype(real), ww=wl.ww.astype(real),
        vis=wl.vis.astype(real), weight=wl.weight.astype(real),
        cell_size_rad=np.array(wl.cell_size_rad, dtype=real),
        w_scale=np.array(wl.w_scale, dtype=real), grid_size=wl.grid_size,
        grid_in=grid0, norm_in=norm0, grid_out=g, num_skipped=ns, norm_out=nm)
    print(f"{name}: N={wl.num_points} G={wl.grid_size} P={wl.num_w_planes} "
          f"os={wl.oversample} skipped={ns} norm={nm!r}")


def _small(name, n, G, P, s_min, s_max, os_, seed, w_over=1.25, sigma=0.2,
           clip=0.56):
    wl = synthetic.random_uniform_workload(
        name, n, G, P, s_min, s_max, oversample=os_, seed=seed,
        cell_size_rad=1.0e-3, w_max=1000.0, sigma_frac=sigma, clip_frac=clip)
    # Some |w| beyond the last plane (clamped to it).
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    wl.ww = (rng.uniform(-w_over, w_over, n) * 1000.0).astype(np.float32)
    return wl


def _edge_case():
    """Hand-placed visibilities on rounding ties and grid borders."""
    G, P, os_ = 101, 6, 4
    support = synthetic.linear_supports(P, 1, 4)
    csh = (int(support.max()) + 1) * os_
    cell = 1.0 / 128.0                     # grid_scale = 101/128, exact
    gs = np.float32(G) * np.float32(cell)
    w_scale = np.float32(1.0)
    pos_u, pos_v, wws = [], [], []
    # Exact half-cell positions (roundf ties away from zero) and exact
    # quarter-cell offsets (offset ties).
    for p in (0.5, -0.5, 1.5, -2.5, 10.125, -10.375, 7.0, 0.0, 3.625):
        for q in (0.5, -1.5, 0.25, -0.75, 4.0):
            pos_u.append(p); pos_v.append(q); wws.append(0.0)
    # Footprints touching the border exactly (kept) and one cell beyond
    # (skipped), for the support of plane 0.
    s0 = int(support[0])
    c = G // 2
    for edge in (G - 1 - s0, G - s0, s0, s0 - 1):
        pos_u.append(float(edge - c)); pos_v.append(0.0); wws.append(0.0)
        pos_u.append(0.0); pos_v.append(float(edge - c)); wws.append(0.0)
    # w on plane ties: sqrt(|w * w_scale|) = k + 0.5 exactly, signs, zeros,
    # and beyond the last plane.
    for k in range(P + 2):
        for sgn in (1.0, -1.0):
            pos_u.append(3.0); pos_v.append(-2.0)
            wws.append(sgn * (k + 0.5) ** 2)
    for w in (0.0, -0.0, 1e-30, -1e-30, 1e6):
        pos_u.append(-4.0); pos_v.append(5.0); wws.append(w)
    pos_u = np.array(pos_u, np.float64)
    pos_v = np.array(pos_v, np.float64)
    # uu = -pos_u / grid_scale and vv = pos_v / grid_scale, chosen so the
    # FP32 products give back the intended positions where representable.
    uu = (-pos_u / float(gs)).astype(np.float32)
    vv = (pos_v / float(gs)).astype(np.float32)
    n = uu.shape[0]
    rng = np.random.Generator(np.random.PCG64(99))
    wl = synthetic.Workload(
        name="edges", num_w_planes=P, support=support, oversample=os_,
        conv_size_half=csh,
        conv_func=synthetic.make_kernel_stack(support, os_, csh),
        uu=uu, vv=vv, ww=np.array(wws, np.float32),
        vis=rng.standard_normal((n, 2)).astype(np.float32),
        weight=np.concatenate([np.zeros(1, np.float32),
                               (1.5 - rng.random(n - 1)).astype(np.float32)]),
        cell_size_rad=float(np.float32(cell)), w_scale=float(w_scale),
        grid_size=G)
    return wl


def _weights_case(name, real, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    n, G = 5000, 64
    cell = 1.0 / 70.0
    uu = rng.normal(0, 20, n).astype(real)
    vv = rng.normal(0, 20, n).astype(real)
    w = (1.5 - rng.random(n)).astype(real)
    R = oracle.ref()
    suffix = "f" if real == np.float32 else "d"
    dens = np.zeros((G, G), real)
    ns = ctypes.c_size_t(0)
    getattr(R, f"oskar_grid_weights_write_{suffix}")(
        n, uu, vv, w, real(cell), G, ctypes.byref(ns), dens.reshape(-1))
    ns_w = int(ns.value)
    out = np.full(n, -7.0, real)     # untouched for skipped points
    getattr(R, f"oskar_grid_weights_read_{suffix}")(
        n, uu, vv, w, out, real(cell), G, ctypes.byref(ns), dens.reshape(-1))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), uu=uu, vv=vv,
                        weight=w, cell_size_rad=np.array(cell, real),
                        grid_size=G, density=dens, num_skipped_write=ns_w,
                        weight_out=out, num_skipped_read=int(ns.value))
    print(f"{name}: N={n} G={G} skipped={ns_w}")


def main():
    if not oracle.ref_available():
        oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference library not built (needs the reference "
                         "source tree)")
    wl = _small("small", 3000, 128, 8, 1, 6, 4, seed=11)
    _save("small_f", wl, np.float32, seed=12)
    _save("small_d", wl, np.float64, seed=13)
    for os_ in (1, 2, 3, 8):
        s_max = 6 if os_ < 8 else 4
        wl = _small(f"os{os_}", 1500, 96, 5, 1, s_max, os_, seed=20 + os_)
        _save(f"os{os_}_f", wl, np.float32, seed=30 + os_)
    _save("edges_f", _edge_case(), np.float32, seed=41)
    _save("edges_d", _edge_case(), np.float64, seed=42)
    empty = _small("empty", 0, 32, 3, 1, 2, 4, seed=50)
    _save("empty_f", empty, np.float32, seed=51)
    # All points off the grid.
    off = _small("off", 200, 32, 3, 1, 2, 4, seed=60, sigma=3.0, clip=3.0)
    off.uu = (off.uu * 0 + 1e5).astype(np.float32)
    _save("offgrid_f", off, np.float32, seed=61)
    _weights_case("weights_f", np.float32, 70)
    _weights_case("weights_d", np.float64, 71)


if __name__ == "__main__":
    main()
