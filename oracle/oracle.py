"""ctypes access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/_build/liboracle.so`` (the C restatement of the reference's
serial gridder, oskar_grid_wproj.c:37-212) and, where it was built,
``oracle/_ref/libref.so`` (the reference's own oskar_grid_wproj.c compiled
from its source).  Only tests, the smoke check and the benchmark's CPU
baseline use this module, as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_sz = ctypes.c_size_t
_szp = ctypes.POINTER(ctypes.c_size_t)
_dp = ctypes.POINTER(ctypes.c_double)


def build(reference_dir: str | None = None) -> None:
    """Compile liboracle.so, and libref.so when the reference tree exists.

    The reference tree's location is the Makefile's REFERENCE variable,
    overridden by reference_dir or $GG_REFERENCE_DIR; the `ref-if-present`
    target skips the build where the tree is absent."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    ref = reference_dir or os.environ.get("GG_REFERENCE_DIR")
    extra = [f"REFERENCE={ref}"] if ref else []
    subprocess.check_call(["make", "-s", "-C", HERE, "ref-if-present"] +
                          extra)


def _grid_sig(fn, real):
    p = _f32p if real == np.float32 else _f64p
    c = ctypes.c_float if real == np.float32 else ctypes.c_double
    fn.argtypes = [_sz, _i32p, ctypes.c_int, ctypes.c_int, p, _sz, p, p, p,
                   p, p, c, c, ctypes.c_int, _szp, _dp, p]
    fn.restype = None


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.isfile(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        _grid_sig(L.oracle_grid_wproj_f, np.float32)
        _grid_sig(L.oracle_grid_wproj_d, np.float64)
        for name, real in (("oracle_place_f", np.float32),
                           ("oracle_place_d", np.float64)):
            p = _f32p if real == np.float32 else _f64p
            c = ctypes.c_float if real == np.float32 else ctypes.c_double
            fn = getattr(L, name)
            fn.argtypes = [_sz, _i32p, ctypes.c_int, _sz, p, p, p, c, c,
                           ctypes.c_int] + [_i32p] * 7
            fn.restype = _sz
        L.oracle_grid_wproj_f_fp64acc.argtypes = [
            _sz, _i32p, ctypes.c_int, ctypes.c_int, _f32p, _sz, _f32p, _f32p,
            _f32p, _f32p, _f32p, ctypes.c_float, ctypes.c_float, ctypes.c_int,
            _szp, _dp, _f64p]
        L.oracle_grid_wproj_f_fp64acc.restype = None
        L.oracle_grid_wproj_f_mt.argtypes = [ctypes.c_int] + \
            L.oracle_grid_wproj_f.argtypes
        L.oracle_grid_wproj_f_mt.restype = ctypes.c_int
        L.oracle_grid_wproj_f_fp64acc_mt.argtypes = [ctypes.c_int] + \
            L.oracle_grid_wproj_f_fp64acc.argtypes
        L.oracle_grid_wproj_f_fp64acc_mt.restype = ctypes.c_int
        L.oracle_grid_wproj_d_promoted_mt.argtypes = \
            L.oracle_grid_wproj_f_fp64acc_mt.argtypes
        L.oracle_grid_wproj_d_promoted_mt.restype = ctypes.c_int
        L.oracle_degrid_wproj_f_fp64.argtypes = [
            _sz, _i32p, ctypes.c_int, ctypes.c_int, _f32p, _sz, _f32p, _f32p,
            _f32p, ctypes.c_float, ctypes.c_float, ctypes.c_int, _f64p, _f64p]
        L.oracle_degrid_wproj_f_fp64.restype = None
        L.oracle_degrid_wproj_d.argtypes = [
            _sz, _i32p, ctypes.c_int, ctypes.c_int, _f64p, _sz, _f64p, _f64p,
            _f64p, ctypes.c_double, ctypes.c_double, ctypes.c_int, _f64p,
            _f64p]
        L.oracle_degrid_wproj_d.restype = None
        for suffix, p, c in (("f", _f32p, ctypes.c_float),
                             ("d", _f64p, ctypes.c_double)):
            w = getattr(L, f"oracle_grid_weights_write_{suffix}")
            w.argtypes = [_sz, p, p, p, c, ctypes.c_int, _szp, p]
            w.restype = None
            r = getattr(L, f"oracle_grid_weights_read_{suffix}")
            r.argtypes = [_sz, p, p, p, p, c, ctypes.c_int, _szp, p]
            r.restype = None
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.isfile(REF_SO)


def ref():
    """The reference's own compiled serial gridder (None if not built)."""
    global _ref
    if _ref is None and ref_available():
        L = ctypes.CDLL(REF_SO)
        _grid_sig(L.oskar_grid_wproj_f, np.float32)
        _grid_sig(L.oskar_grid_wproj_d, np.float64)
        for suffix, p, c in (("f", _f32p, ctypes.c_float),
                             ("d", _f64p, ctypes.c_double)):
            w = getattr(L, f"oskar_grid_weights_write_{suffix}")
            w.argtypes = [_sz, p, p, p, c, ctypes.c_int, _szp, p]
            w.restype = None
            r = getattr(L, f"oskar_grid_weights_read_{suffix}")
            r.argtypes = [_sz, p, p, p, p, c, ctypes.c_int, _szp, p]
            r.restype = None
        _ref = L
    return _ref


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _grid_call(fn, wl, grid, norm, real, extra=()):
    ns = ctypes.c_size_t(0)
    nm = ctypes.c_double(norm)
    cast = np.float32 if real == np.float32 else np.float64
    fn(*extra, wl.num_w_planes, _c(wl.support, np.int32), wl.oversample,
       wl.conv_size_half, _c(wl.conv_func, real).reshape(-1), wl.num_points,
       _c(wl.uu, real), _c(wl.vv, real), _c(wl.ww, real),
       _c(wl.vis, real).reshape(-1), _c(wl.weight, real),
       cast(wl.cell_size_rad), cast(wl.w_scale), wl.grid_size,
       ctypes.byref(ns), ctypes.byref(nm), grid.reshape(-1))
    return int(ns.value), float(nm.value)


def new_grid(wl, dtype=np.float32):
    return np.zeros((wl.grid_size, wl.grid_size, 2), dtype=dtype)


def grid_f(wl, grid=None, norm=0.0, use_reference=False):
    """Serial FP32 gridding (oskar_grid_wproj_f semantics); grid in/out."""
    grid = new_grid(wl) if grid is None else grid
    assert grid.dtype == np.float32 and grid.flags.c_contiguous
    fn = ref().oskar_grid_wproj_f if use_reference else \
        lib().oracle_grid_wproj_f
    ns, nm = _grid_call(fn, wl, grid, norm, np.float32)
    return grid, ns, nm


def grid_f_mt(wl, grid=None, norm=0.0, threads=None):
    """Host-parallel FP32 gridding, bit-identical to grid_f."""
    grid = new_grid(wl) if grid is None else grid
    threads = threads or os.cpu_count() or 1
    ns, nm = _grid_call(lib().oracle_grid_wproj_f_mt, wl, grid, norm,
                        np.float32, extra=(threads,))
    return grid, ns, nm


def grid_d(wl, grid=None, norm=0.0, use_reference=False):
    """Serial FP64 gridding (oskar_grid_wproj_d semantics) on the workload's
    arrays promoted to float64; grid in/out (float64)."""
    grid = new_grid(wl, np.float64) if grid is None else grid
    assert grid.dtype == np.float64 and grid.flags.c_contiguous
    fn = ref().oskar_grid_wproj_d if use_reference else \
        lib().oracle_grid_wproj_d
    ns, nm = _grid_call(fn, wl, grid, norm, np.float64)
    return grid, ns, nm


def grid_f_fp64acc(wl, grid=None, norm=0.0):
    """FP64 accumulation with FP32 placement: the error yardstick for the
    FP32 path.  grid is float64 (in/out)."""
    grid = new_grid(wl, np.float64) if grid is None else grid
    ns = ctypes.c_size_t(0)
    nm = ctypes.c_double(norm)
    lib().oracle_grid_wproj_f_fp64acc(
        wl.num_w_planes, _c(wl.support, np.int32), wl.oversample,
        wl.conv_size_half, _c(wl.conv_func, np.float32).reshape(-1),
        wl.num_points, _c(wl.uu, np.float32), _c(wl.vv, np.float32),
        _c(wl.ww, np.float32), _c(wl.vis, np.float32).reshape(-1),
        _c(wl.weight, np.float32), np.float32(wl.cell_size_rad),
        np.float32(wl.w_scale), wl.grid_size, ctypes.byref(ns),
        ctypes.byref(nm), grid.reshape(-1))
    return grid, int(ns.value), float(nm.value)


def grid_f_fp64acc_mt(wl, grid=None, norm=0.0, threads=None):
    """grid_f_fp64acc on host threads; bit-identical to it."""
    grid = new_grid(wl, np.float64) if grid is None else grid
    assert grid.dtype == np.float64 and grid.flags.c_contiguous
    threads = threads or os.cpu_count() or 1
    ns = ctypes.c_size_t(0)
    nm = ctypes.c_double(norm)
    rc = lib().oracle_grid_wproj_f_fp64acc_mt(
        threads, wl.num_w_planes, _c(wl.support, np.int32), wl.oversample,
        wl.conv_size_half, _c(wl.conv_func, np.float32).reshape(-1),
        wl.num_points, _c(wl.uu, np.float32), _c(wl.vv, np.float32),
        _c(wl.ww, np.float32), _c(wl.vis, np.float32).reshape(-1),
        _c(wl.weight, np.float32), np.float32(wl.cell_size_rad),
        np.float32(wl.w_scale), wl.grid_size, ctypes.byref(ns),
        ctypes.byref(nm), grid.reshape(-1))
    if rc != 0:
        raise MemoryError("oracle_grid_wproj_f_fp64acc_mt: no scratch memory")
    return grid, int(ns.value), float(nm.value)


def grid_d_promoted_mt(wl, grid=None, norm=0.0, threads=None):
    """The reference's FP64 gridder (oskar_grid_wproj_d semantics: FP64
    placement and sums) on the FP32 workload promoted to FP64, on host
    threads; bit-identical to grid_d on the promoted arrays."""
    grid = new_grid(wl, np.float64) if grid is None else grid
    assert grid.dtype == np.float64 and grid.flags.c_contiguous
    threads = threads or os.cpu_count() or 1
    ns = ctypes.c_size_t(0)
    nm = ctypes.c_double(norm)
    rc = lib().oracle_grid_wproj_d_promoted_mt(
        threads, wl.num_w_planes, _c(wl.support, np.int32), wl.oversample,
        wl.conv_size_half, _c(wl.conv_func, np.float32).reshape(-1),
        wl.num_points, _c(wl.uu, np.float32), _c(wl.vv, np.float32),
        _c(wl.ww, np.float32), _c(wl.vis, np.float32).reshape(-1),
        _c(wl.weight, np.float32), np.float32(wl.cell_size_rad),
        np.float32(wl.w_scale), wl.grid_size, ctypes.byref(ns),
        ctypes.byref(nm), grid.reshape(-1))
    if rc != 0:
        raise MemoryError("oracle_grid_wproj_d_promoted_mt: no scratch "
                          "memory")
    return grid, int(ns.value), float(nm.value)


def placement_disagreements(wl):
    """Visibilities whose cell, offsets, plane or skip differ between the
    FP32 rules (oskar_grid_wproj_f) and the FP64 rules on the promoted
    coordinates (oskar_grid_wproj_d): (count, count among visibilities
    gridded by either)."""
    pf, pd = place(wl, "f"), place(wl, "d")
    diff = np.zeros(wl.num_points, bool)
    for k in ("gu", "gv", "ou", "ov", "plane", "skipped"):
        diff |= pf[k] != pd[k]
    either = (pf["skipped"] == 0) | (pd["skipped"] == 0)
    return int(diff.sum()), int((diff & either).sum())


def place(wl, precision="f"):
    """Per-visibility placement dict: gu, gv, ou, ov, plane, conj_neg,
    skipped (int32 arrays) and the skip count."""
    n = wl.num_points
    outs = {k: np.zeros(n, np.int32) for k in
            ("gu", "gv", "ou", "ov", "plane", "conj_neg", "skipped")}
    real = np.float32 if precision == "f" else np.float64
    fn = lib().oracle_place_f if precision == "f" else lib().oracle_place_d
    ns = fn(wl.num_w_planes, _c(wl.support, np.int32), wl.oversample, n,
            _c(wl.uu, real), _c(wl.vv, real), _c(wl.ww, real),
            real(wl.cell_size_rad), real(wl.w_scale), wl.grid_size,
            *[outs[k] for k in ("gu", "gv", "ou", "ov", "plane", "conj_neg",
                                "skipped")])
    outs["num_skipped"] = int(ns)
    return outs


def degrid_fp64(wl, grid):
    """Adjoint of the FP32 gridding map in FP64: float64[N, 2]."""
    g = _c(grid, np.float64)
    out = np.zeros((wl.num_points, 2), np.float64)
    lib().oracle_degrid_wproj_f_fp64(
        wl.num_w_planes, _c(wl.support, np.int32), wl.oversample,
        wl.conv_size_half, _c(wl.conv_func, np.float32).reshape(-1),
        wl.num_points, _c(wl.uu, np.float32), _c(wl.vv, np.float32),
        _c(wl.ww, np.float32), np.float32(wl.cell_size_rad),
        np.float32(wl.w_scale), wl.grid_size, g.reshape(-1), out.reshape(-1))
    return out


def degrid_d(wl, grid):
    """Adjoint of the FP64 gridding map (FP64 placement and cube)."""
    g = _c(grid, np.float64)
    out = np.zeros((wl.num_points, 2), np.float64)
    lib().oracle_degrid_wproj_d(
        wl.num_w_planes, _c(wl.support, np.int32), wl.oversample,
        wl.conv_size_half, _c(wl.conv_func, np.float64).reshape(-1),
        wl.num_points, _c(wl.uu, np.float64), _c(wl.vv, np.float64),
        _c(wl.ww, np.float64), float(wl.cell_size_rad), float(wl.w_scale),
        wl.grid_size, g.reshape(-1), out.reshape(-1))
    return out


def weights_write(uu, vv, weight, cell_size_rad, grid_size, grid=None):
    """Serial uniform-weighting density (oskar_grid_weights_write_{f,d}
    semantics, precision from uu's dtype); grid [G, G] in/out.  Returns
    (grid, num_skipped)."""
    real = np.asarray(uu).dtype.type
    sfx = "f" if real == np.float32 else "d"
    grid = np.zeros((grid_size, grid_size), real) if grid is None else grid
    ns = ctypes.c_size_t(0)
    getattr(lib(), f"oracle_grid_weights_write_{sfx}")(
        len(uu), _c(uu, real), _c(vv, real), _c(weight, real),
        real(cell_size_rad), grid_size, ctypes.byref(ns), grid.reshape(-1))
    return grid, int(ns.value)


def weights_read(uu, vv, weight_in, weight_out, cell_size_rad, grid_size,
                 grid):
    """Serial uniform re-weighting (oskar_grid_weights_read_{f,d});
    weight_out updated in place.  Returns num_skipped."""
    real = np.asarray(uu).dtype.type
    sfx = "f" if real == np.float32 else "d"
    ns = ctypes.c_size_t(0)
    getattr(lib(), f"oracle_grid_weights_read_{sfx}")(
        len(uu), _c(uu, real), _c(vv, real), _c(weight_in, real), weight_out,
        real(cell_size_rad), grid_size, ctypes.byref(ns),
        _c(grid, real).reshape(-1))
    return int(ns.value)


def mac_count(wl, precision="f"):
    """Algorithmic complex MACs: sum of (2 s + 1)^2 over gridded points."""
    p = place(wl, precision)
    s = np.asarray(wl.support, np.int64)[p["plane"]]
    keep = p["skipped"] == 0
    return int(((2 * s[keep] + 1) ** 2).sum())
