"""GB300 W-projection gridder -- Python host interface.

A thin ctypes layer over ``libgpugrid.so`` (C ABI in include/gpugrid.h):

* ``oskar_grid_wproj_f`` / ``oskar_grid_wproj_d`` -- the reference's serial
  gridding functions (oskar_grid_wproj.h:69-86, :114-131 of the reference),
  same argument names and meaning, host (numpy) arrays.  ``grid`` is updated
  in place; the function returns ``(num_skipped, norm)`` where the reference
  writes them through pointers.
* ``KernelStack``, ``Plan``, ``grid_wproj_device``, ``degrid_wproj_device``
  -- device-resident inputs (torch CUDA tensors) on a CUDA stream.
* ``GridWproj`` -- torch.autograd.Function whose backward pass is the
  hand-written adjoint (degridding) kernel.

There is no CPU fallback: if the library is missing or no GPU is present the
calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

GG_OK = 0
_ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of memory",
           4: "unsupported", 5: "capacity"}

# Every entry point declared in include/gpugrid.h and include/gpugrid_io.h.
EXPORTED_SYMBOLS = (
    "oskar_grid_wproj_d", "oskar_grid_wproj_f", "gg_grid_wproj_d",
    "gg_grid_wproj_f", "gg_last_error", "gg_version", "gg_kernels_create_f",
    "gg_kernels_create_d", "gg_kernels_generate_f", "gg_kernels_generate_d",
    "gg_kernels_destroy", "gg_plan_create",
    "gg_plan_destroy", "gg_plan_last_stats", "gg_plan_set_tile_shape",
    "gg_plan_set_slice_staging", "gg_plan_set_tuning", "gg_plan_get_tuning",
    "gg_host_set_tuning", "gg_host_get_tuning", "gg_host_last_transfer",
    "gg_host_last_call_ms",
    "gg_host_set_grid_access", "gg_host_get_grid_access",
    "gg_host_set_profiling", "gg_host_phase_ms",
    "gg_plan_probe_bounded_wait", "gg_plan_set_batch_limit",
    "gg_plan_set_profiling",
    "gg_plan_phase_ms", "gg_measure_fp32_fma_tflops", "gg_grid_wproj_f_device",
    "gg_grid_wproj_f_device_noalloc", "gg_noalloc_probe_bounded_wait",
    "gg_grid_wproj_f_batched_device",
    "gg_grid_wproj_d_batched_device", "gg_grid_wproj_f_batched_replay",
    "gg_grid_wproj_d_batched_replay", "gg_plan_check",
    "gg_grid_wproj_d_device", "gg_place_wproj_f_device",
    "gg_place_wproj_d_device", "gg_degrid_wproj_f_device",
    "gg_degrid_wproj_d_device", "gg_degrid_wproj_f", "gg_degrid_wproj_d",
    "oskar_degrid_wproj_f", "oskar_degrid_wproj_d",
    "oskar_grid_weights_write_f", "oskar_grid_weights_write_d",
    "oskar_grid_weights_read_f", "oskar_grid_weights_read_d",
    "gg_grid_weights_write_f", "gg_grid_weights_write_d",
    "gg_grid_weights_read_f", "gg_grid_weights_read_d",
    "gg_grid_weights_write_f_device", "gg_grid_weights_write_d_device",
    "gg_grid_weights_read_f_device", "gg_grid_weights_read_d_device",
    # include/gpugrid_io.h: the dataset loaders.
    "oskar_binary_create", "oskar_binary_free", "oskar_binary_num_tags",
    "oskar_binary_query", "oskar_binary_read_block", "oskar_binary_read",
    "oskar_binary_read_int", "oskar_binary_read_double",
    "gg_vis_read_coords", "gg_vis_scale_coords", "gg_read_kernel",
)


class GridError(RuntimeError):
    """A gg_* call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERRORS.get(code, code)}: {message}")
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("num_points", ctypes.c_ulonglong),
                ("num_skipped", ctypes.c_ulonglong),
                ("num_records", ctypes.c_ulonglong),
                ("num_macs", ctypes.c_ulonglong),
                ("num_launches", ctypes.c_ulonglong),
                ("tile_u", ctypes.c_int), ("tile_v", ctypes.c_int),
                ("slice_staging", ctypes.c_int), ("num_ctas", ctypes.c_int),
                ("chunk_records", ctypes.c_ulonglong),
                ("num_plane_groups", ctypes.c_int)]


class Tuning(ctypes.Structure):
    """gg_tuning: launch and decomposition parameters of a plan."""
    _fields_ = [("tile_u", ctypes.c_int), ("slice_staging", ctypes.c_int),
                ("items_per_cta", ctypes.c_int), ("sort_detail", ctypes.c_int),
                ("ctas_per_sm", ctypes.c_int), ("plane_group_mb", ctypes.c_int),
                ("tile_order", ctypes.c_int), ("lane_groups", ctypes.c_int),
                ("tile_phases", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}

    @classmethod
    def from_dict(cls, d: dict) -> "Tuning":
        t = cls(0, -1, 4, 2, 0, 0, 0, 0, 0)
        for k, _ in cls._fields_:
            if k in d:
                setattr(t, k, int(d[k]))
        return t


_lib = None
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t


def _declare(L):
    f32, f64 = ctypes.c_float, ctypes.c_double
    for suffix, real in (("f", f32), ("d", f64)):
        grid_args = [_sz, _vp, ctypes.c_int, ctypes.c_int, _vp, _sz, _vp, _vp,
                     _vp, _vp, _vp, real, real, ctypes.c_int, _vp, _vp, _vp]
        fn = getattr(L, f"gg_grid_wproj_{suffix}")
        fn.argtypes = grid_args
        fn.restype = ctypes.c_int
        fn = getattr(L, f"oskar_grid_wproj_{suffix}")
        fn.argtypes = grid_args
        fn.restype = None
        fn = getattr(L, f"gg_kernels_create_{suffix}")
        fn.argtypes = [ctypes.POINTER(_vp), _sz, _vp, ctypes.c_int,
                       ctypes.c_int, _vp, ctypes.c_int, _vp]
        fn.restype = ctypes.c_int
        fn = getattr(L, f"gg_kernels_generate_{suffix}")
        fn.argtypes = [ctypes.POINTER(_vp), _sz, _vp, ctypes.c_int,
                       ctypes.c_int, _vp, _vp, _vp]
        fn.restype = ctypes.c_int
        fn = getattr(L, f"gg_grid_wproj_{suffix}_device")
        fn.argtypes = [_vp, _vp, _sz, _vp, _vp, _vp, _vp, _vp, real, real,
                       ctypes.c_int, _vp, _vp, _vp, _vp]
        fn.restype = ctypes.c_int
        fn = getattr(L, f"gg_grid_wproj_{suffix}_batched_device")
        fn.argtypes = [_vp, _vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp,
                       real, real, ctypes.c_int, _vp, _vp, _vp, _vp]
        fn.restype = ctypes.c_int
        fn = getattr(L, f"gg_grid_wproj_{suffix}_batched_replay")
        fn.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
        fn.restype = ctypes.c_int
        fn = getattr(L, f"gg_place_wproj_{suffix}_device")
        fn.argtypes = [_vp, _sz, _vp, _vp, _vp, real, real, ctypes.c_int,
                       _vp, _vp]
        fn.restype = ctypes.c_int
        degrid_args = [_sz, _vp, ctypes.c_int, ctypes.c_int, _vp, _sz, _vp,
                       _vp, _vp, real, real, ctypes.c_int, _vp, _vp]
        fn = getattr(L, f"gg_degrid_wproj_{suffix}")
        fn.argtypes = degrid_args
        fn.restype = ctypes.c_int
        fn = getattr(L, f"oskar_degrid_wproj_{suffix}")
        fn.argtypes = degrid_args
        fn.restype = None
        w_args = [_sz, _vp, _vp, _vp, real, ctypes.c_int, _vp, _vp]
        r_args = [_sz, _vp, _vp, _vp, _vp, real, ctypes.c_int, _vp, _vp]
        for name, args in (("write", w_args), ("read", r_args)):
            fn = getattr(L, f"gg_grid_weights_{name}_{suffix}")
            fn.argtypes = args
            fn.restype = ctypes.c_int
            fn = getattr(L, f"oskar_grid_weights_{name}_{suffix}")
            fn.argtypes = args
            fn.restype = None
        fn = getattr(L, f"gg_grid_weights_write_{suffix}_device")
        fn.argtypes = [_vp, _sz, _vp, _vp, _vp, real, ctypes.c_int, _vp, _vp,
                       _vp]
        fn.restype = ctypes.c_int
        fn = getattr(L, f"gg_grid_weights_read_{suffix}_device")
        fn.argtypes = [_vp, _sz, _vp, _vp, _vp, _vp, real, ctypes.c_int, _vp,
                       _vp, _vp]
        fn.restype = ctypes.c_int
        fn = getattr(L, f"gg_degrid_wproj_{suffix}_device")
        fn.argtypes = [_vp, _vp, _sz, _vp, _vp, _vp, real, real, ctypes.c_int,
                       _vp, _vp, _vp]
        fn.restype = ctypes.c_int
    L.gg_last_error.restype = ctypes.c_char_p
    L.gg_last_error.argtypes = []
    L.gg_version.restype = ctypes.c_char_p
    L.gg_version.argtypes = []
    L.gg_kernels_destroy.argtypes = [_vp]
    L.gg_kernels_destroy.restype = ctypes.c_int
    L.gg_plan_create.argtypes = [ctypes.POINTER(_vp)]
    L.gg_plan_create.restype = ctypes.c_int
    L.gg_plan_destroy.argtypes = [_vp]
    L.gg_plan_destroy.restype = ctypes.c_int
    L.gg_plan_last_stats.argtypes = [_vp, ctypes.POINTER(Stats)]
    L.gg_plan_last_stats.restype = ctypes.c_int
    L.gg_plan_set_tile_shape.argtypes = [_vp, ctypes.c_int]
    L.gg_plan_set_tile_shape.restype = ctypes.c_int
    L.gg_plan_set_slice_staging.argtypes = [_vp, ctypes.c_int]
    L.gg_plan_set_slice_staging.restype = ctypes.c_int
    L.gg_plan_set_tuning.argtypes = [_vp, ctypes.POINTER(Tuning)]
    L.gg_plan_set_tuning.restype = ctypes.c_int
    L.gg_plan_get_tuning.argtypes = [_vp, ctypes.POINTER(Tuning)]
    L.gg_plan_get_tuning.restype = ctypes.c_int
    L.gg_host_set_tuning.argtypes = [ctypes.POINTER(Tuning)]
    L.gg_host_set_tuning.restype = ctypes.c_int
    L.gg_host_get_tuning.argtypes = [ctypes.POINTER(Tuning)]
    L.gg_host_get_tuning.restype = ctypes.c_int
    L.gg_host_last_transfer.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)] * 2
    L.gg_host_last_transfer.restype = ctypes.c_int
    L.gg_host_last_call_ms.argtypes = [ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_int]
    L.gg_host_last_call_ms.restype = ctypes.c_int
    L.gg_host_set_grid_access.argtypes = [ctypes.c_int]
    L.gg_host_set_grid_access.restype = ctypes.c_int
    L.gg_host_get_grid_access.argtypes = [ctypes.POINTER(ctypes.c_int)]
    L.gg_host_get_grid_access.restype = ctypes.c_int
    L.gg_host_set_profiling.argtypes = [ctypes.c_int]
    L.gg_host_set_profiling.restype = ctypes.c_int
    L.gg_host_phase_ms.argtypes = [ctypes.POINTER(ctypes.c_float),
                                   ctypes.c_int]
    L.gg_host_phase_ms.restype = ctypes.c_int
    L.gg_plan_probe_bounded_wait.argtypes = [_vp, ctypes.c_uint, _vp]
    L.gg_plan_probe_bounded_wait.restype = ctypes.c_int
    L.gg_plan_set_batch_limit.argtypes = [_vp, ctypes.c_ulonglong]
    L.gg_plan_set_batch_limit.restype = ctypes.c_int
    L.gg_plan_check.argtypes = [_vp, _vp]
    L.gg_plan_check.restype = ctypes.c_int
    L.gg_plan_set_profiling.argtypes = [_vp, ctypes.c_int]
    L.gg_plan_set_profiling.restype = ctypes.c_int
    L.gg_plan_phase_ms.argtypes = [_vp, ctypes.POINTER(ctypes.c_float),
                                   ctypes.c_int]
    L.gg_plan_phase_ms.restype = ctypes.c_int
    L.gg_measure_fp32_fma_tflops.argtypes = [ctypes.POINTER(ctypes.c_double)]
    L.gg_measure_fp32_fma_tflops.restype = ctypes.c_int


def lib():
    """The loaded libgpugrid.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "__graft_entry__.build() (or python gpu-gridding_gb300/build.py)")
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def build(force: bool = False) -> str:
    """Compile libgpugrid.so for sm_103a (in-tree)."""
    return _build.build(force=force)


def last_error() -> str:
    return lib().gg_last_error().decode()


def _check(code: int) -> None:
    if code != GG_OK:
        raise GridError(code, last_error())


def _ptr(a) -> int:
    if a is None:
        return 0
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def _host(a, dtype):
    a = np.asarray(a)
    if a.dtype != dtype or not a.flags.c_contiguous:
        a = np.ascontiguousarray(a, dtype=dtype)
    return a


# ---------------------------------------------------------------------------
# Drop-in (host arrays)
# ---------------------------------------------------------------------------
def _dropin(suffix, dtype, num_w_planes, support, oversample, conv_size_half,
            conv_func, num_points, uu, vv, ww, vis, weight, cell_size_rad,
            w_scale, grid_size, grid, norm):
    if not (isinstance(grid, np.ndarray) and grid.dtype == dtype and
            grid.flags.c_contiguous):
        raise TypeError(f"grid must be a C-contiguous {np.dtype(dtype)} array")
    if grid.size != 2 * grid_size * grid_size:
        raise ValueError("grid must hold grid_size^2 complex values")
    arrs = [_host(support, np.int32), _host(conv_func, dtype), _host(uu, dtype),
            _host(vv, dtype), _host(ww, dtype), _host(vis, dtype),
            _host(weight, dtype)]
    ns = ctypes.c_size_t(0)
    nm = ctypes.c_double(norm)
    _check(getattr(lib(), f"gg_grid_wproj_{suffix}")(
        num_w_planes, _ptr(arrs[0]), oversample, conv_size_half, _ptr(arrs[1]),
        num_points, _ptr(arrs[2]), _ptr(arrs[3]), _ptr(arrs[4]), _ptr(arrs[5]),
        _ptr(arrs[6]), cell_size_rad, w_scale, grid_size,
        ctypes.addressof(ns), ctypes.addressof(nm), _ptr(grid)))
    return int(ns.value), float(nm.value)


def oskar_grid_wproj_f(num_w_planes, support, oversample, conv_size_half,
                       conv_func, num_points, uu, vv, ww, vis, weight,
                       cell_size_rad, w_scale, grid_size, grid, norm=0.0):
    """GPU drop-in for oskar_grid_wproj_f (reference oskar_grid_wproj.c:
    126-212).  grid (float32, grid_size^2 complex) is accumulated in place;
    returns (num_skipped, norm + this call's normalisation)."""
    return _dropin("f", np.float32, num_w_planes, support, oversample,
                   conv_size_half, conv_func, num_points, uu, vv, ww, vis,
                   weight, cell_size_rad, w_scale, grid_size, grid, norm)


def oskar_grid_wproj_d(num_w_planes, support, oversample, conv_size_half,
                       conv_func, num_points, uu, vv, ww, vis, weight,
                       cell_size_rad, w_scale, grid_size, grid, norm=0.0):
    """GPU drop-in for oskar_grid_wproj_d (reference oskar_grid_wproj.c:
    37-123), FP64 throughout."""
    return _dropin("d", np.float64, num_w_planes, support, oversample,
                   conv_size_half, conv_func, num_points, uu, vv, ww, vis,
                   weight, cell_size_rad, w_scale, grid_size, grid, norm)


def grid_f(wl, grid=None, norm=0.0):
    """oskar_grid_wproj_f on a synthetic.Workload; returns
    (grid, num_skipped, norm) like the oracle's helper of the same name."""
    if grid is None:
        grid = np.zeros((wl.grid_size, wl.grid_size, 2), np.float32)
    ns, nm = oskar_grid_wproj_f(
        wl.num_w_planes, wl.support, wl.oversample, wl.conv_size_half,
        wl.conv_func, wl.num_points, wl.uu, wl.vv, wl.ww, wl.vis, wl.weight,
        np.float32(wl.cell_size_rad), np.float32(wl.w_scale), wl.grid_size,
        grid, norm)
    return grid, ns, nm


def grid_d(wl, grid=None, norm=0.0):
    """oskar_grid_wproj_d on a workload promoted to float64."""
    if grid is None:
        grid = np.zeros((wl.grid_size, wl.grid_size, 2), np.float64)
    ns, nm = oskar_grid_wproj_d(
        wl.num_w_planes, wl.support, wl.oversample, wl.conv_size_half,
        wl.conv_func, wl.num_points, wl.uu, wl.vv, wl.ww, wl.vis, wl.weight,
        float(wl.cell_size_rad), float(wl.w_scale), wl.grid_size, grid, norm)
    return grid, ns, nm


# ---------------------------------------------------------------------------
# Device API (torch tensors)
# ---------------------------------------------------------------------------
def _stream_ptr(stream):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class KernelStack:
    """Device-resident, re-laid kernel stack (gg_kernels handle)."""

    def __init__(self, num_w_planes, support, oversample, conv_size_half,
                 conv_func, precision="f", stream=None):
        self.precision = precision
        self.num_w_planes = int(num_w_planes)
        self.oversample = int(oversample)
        self.conv_size_half = int(conv_size_half)
        self.support = _host(support, np.int32)
        h = ctypes.c_void_p(0)
        on_device = 0 if isinstance(conv_func, np.ndarray) else 1
        if on_device == 0:
            conv_func = _host(conv_func, np.float32 if precision == "f"
                              else np.float64)
        self._keep = conv_func
        _check(getattr(lib(), f"gg_kernels_create_{precision}")(
            ctypes.byref(h), self.num_w_planes, _ptr(self.support),
            self.oversample, self.conv_size_half, _ptr(conv_func), on_device,
            _stream_ptr(stream) if on_device else None))
        self._keep = None
        self.handle = h

    @classmethod
    def generate(cls, num_w_planes, support, oversample, conv_size_half,
                 w_planes, precision="f", cube_out=None, stream=None):
        """Kernel stack generated on the device (gg_kernels_generate_*):
        the taper x chirp recipe with chirp parameters w_planes[p]; the
        cube also goes to cube_out (a CUDA tensor [P, csh, csh, 2]) when
        given."""
        self = cls.__new__(cls)
        self.precision = precision
        self.num_w_planes = int(num_w_planes)
        self.oversample = int(oversample)
        self.conv_size_half = int(conv_size_half)
        self.support = _host(support, np.int32)
        self._keep = None
        w = _host(w_planes, np.float64)
        if w.shape[0] != self.num_w_planes:
            raise ValueError("w_planes needs one value per plane")
        h = ctypes.c_void_p(0)
        _check(getattr(lib(), f"gg_kernels_generate_{precision}")(
            ctypes.byref(h), self.num_w_planes, _ptr(self.support),
            self.oversample, self.conv_size_half, _ptr(w),
            _ptr(cube_out) if cube_out is not None else None,
            _stream_ptr(stream)))
        self.handle = h
        return self

    @classmethod
    def from_workload(cls, wl, precision="f", stream=None):
        return cls(wl.num_w_planes, wl.support, wl.oversample,
                   wl.conv_size_half, wl.conv_func, precision, stream)

    def close(self):
        if self.handle and self.handle.value:
            lib().gg_kernels_destroy(self.handle)
            self.handle = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """Device workspace (gg_plan handle); one call at a time."""

    def __init__(self):
        h = ctypes.c_void_p(0)
        _check(lib().gg_plan_create(ctypes.byref(h)))
        self.handle = h

    PHASES = ("placement", "binning", "work_items", "grid_tiles",
              "reduce_partials")

    def stats(self) -> dict:
        s = Stats()
        _check(lib().gg_plan_last_stats(self.handle, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def set_tile_shape(self, tile_u: int = 0) -> None:
        """Force the tile width (32, 16 or 8); 0 = chosen per call."""
        _check(lib().gg_plan_set_tile_shape(self.handle, int(tile_u)))

    def set_slice_staging(self, mode: int = -1) -> None:
        """Kernel-slice staging in shared memory: -1 auto, 0 off, 1 on."""
        _check(lib().gg_plan_set_slice_staging(self.handle, int(mode)))

    def set_batch_limit(self, max_points: int = 0) -> None:
        """Most visibilities per sub-batch of a batched call (0 = only as
        the 32-bit record indices require); see gg_plan_set_batch_limit."""
        _check(lib().gg_plan_set_batch_limit(self.handle, int(max_points)))

    def set_tuning(self, tuning) -> None:
        """Apply a Tuning (or a dict of its fields; missing fields take the
        defaults)."""
        t = tuning if isinstance(tuning, Tuning) else Tuning.from_dict(tuning)
        _check(lib().gg_plan_set_tuning(self.handle, ctypes.byref(t)))

    def tuning(self) -> dict:
        t = Tuning()
        _check(lib().gg_plan_get_tuning(self.handle, ctypes.byref(t)))
        return t.as_dict()

    def probe_bounded_wait(self, iterations: int = 1000, stream=None) -> None:
        """Run the failure-path probe (gg_plan_probe_bounded_wait): raises
        GridError, and the plan reports the error from then on."""
        _check(lib().gg_plan_probe_bounded_wait(
            self.handle, int(iterations), _stream_ptr(stream)))

    def set_profiling(self, enable: bool = True) -> None:
        _check(lib().gg_plan_set_profiling(self.handle, int(enable)))

    def phase_ms(self) -> dict:
        """CUDA-event time of each phase of the last call (stream must be
        synchronised; profiling must be enabled)."""
        arr = (ctypes.c_float * len(self.PHASES))()
        _check(lib().gg_plan_phase_ms(self.handle, arr, len(self.PHASES)))
        return dict(zip(self.PHASES, list(arr)))

    def close(self):
        if self.handle and self.handle.value:
            lib().gg_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def measure_fp32_fma_tflops() -> float:
    """Measured FP32 FMA throughput of the current GPU (TFLOP/s)."""
    out = ctypes.c_double(0)
    _check(lib().gg_measure_fp32_fma_tflops(ctypes.byref(out)))
    return float(out.value)


def _require_cuda(*tensors):
    for t in tensors:
        if not t.is_cuda or not t.is_contiguous():
            raise TypeError("device entry points take contiguous CUDA tensors")


def set_host_tuning(tuning=None) -> None:
    """Tuning of the host-pointer entry points on the current device (a
    Tuning or a dict of its fields; None restores the defaults)."""
    if tuning is None:
        _check(lib().gg_host_set_tuning(None))
        return
    t = tuning if isinstance(tuning, Tuning) else Tuning.from_dict(tuning)
    _check(lib().gg_host_set_tuning(ctypes.byref(t)))


def host_last_transfer() -> tuple:
    """(host->device, device->host) bytes of the last host-pointer gridding
    call on the current device."""
    a, b = ctypes.c_ulonglong(0), ctypes.c_ulonglong(0)
    _check(lib().gg_host_last_transfer(ctypes.byref(a), ctypes.byref(b)))
    return int(a.value), int(b.value)


def host_last_call_ms() -> dict:
    """Host-clock marks (ms from entry) of the last host-pointer gridding
    call on the current device: first queued work, final synchronisation,
    return."""
    ms = (ctypes.c_double * 3)()
    _check(lib().gg_host_last_call_ms(ms, 3))
    return dict(zip(("first_work", "synchronised", "return"),
                    (float(x) for x in ms)))


# How the host-pointer gridding calls reach the caller's grid and cube (see
# gg_host_set_grid_access): copied, used in place when page-locked, or (the
# default) in place also when pageable, on devices that read pageable memory
# through the host's page tables.
GRID_ACCESS_COPY, GRID_ACCESS_PINNED, GRID_ACCESS_PAGEABLE = 0, 1, 2


def set_host_grid_access(mode: int) -> None:
    _check(lib().gg_host_set_grid_access(int(mode)))


def host_grid_access() -> int:
    m = ctypes.c_int(0)
    _check(lib().gg_host_get_grid_access(ctypes.byref(m)))
    return int(m.value)


HOST_PHASES = ("staging", "placement", "binning", "work_items", "grid_tiles",
               "finish", "host_first_work", "host_synchronised",
               "host_return")


def set_host_profiling(enable: bool) -> None:
    """Phase events in the host-pointer gridding calls on this device."""
    _check(lib().gg_host_set_profiling(1 if enable else 0))


def host_phase_ms() -> dict:
    """Phase times (ms) of the last profiled host-pointer gridding call."""
    ms = (ctypes.c_float * len(HOST_PHASES))()
    _check(lib().gg_host_phase_ms(ms, len(HOST_PHASES)))
    return dict(zip(HOST_PHASES, (float(x) for x in ms)))


def host_tuning() -> dict:
    t = Tuning()
    _check(lib().gg_host_get_tuning(ctypes.byref(t)))
    return t.as_dict()


def grid_wproj_device(plan, stack, uu, vv, ww, vis, weight, cell_size_rad,
                      w_scale, grid_size, grid, norm, num_skipped,
                      stream=None):
    """Grid device-resident visibilities onto a device grid.

    uu, vv, ww, weight: [N]; vis: [N, 2]; grid: [G, G, 2] (accumulated);
    norm: float64 [1] (accumulated); num_skipped: int64 [1] (set).  dtype
    float32 with a precision "f" stack, float64 with "d"."""
    import torch  # noqa: F401
    _require_cuda(uu, vv, ww, vis, weight, grid, norm, num_skipped)
    n = int(uu.shape[0])
    fn = getattr(lib(), f"gg_grid_wproj_{stack.precision}_device")
    _check(fn(plan.handle, stack.handle, n, _ptr(uu), _ptr(vv), _ptr(ww),
              _ptr(vis), _ptr(weight), cell_size_rad, w_scale, grid_size,
              _ptr(num_skipped), _ptr(norm), _ptr(grid), _stream_ptr(stream)))


def grid_wproj_batched_device(plan, stack, offsets, uu, vv, ww, vis, weight,
                              cell_size_rad, w_scale, grid_size, grids, norms,
                              num_skipped, stream=None):
    """Grid several channels in one call.  offsets: int sequence of
    num_grids + 1 (channel g = visibilities offsets[g]:offsets[g+1] of the
    concatenated uu, vv, ww, vis, weight); grids: [num_grids, G, G, 2]
    (accumulated); norms: float64 [num_grids] (accumulated); num_skipped:
    int64 [num_grids] (set)."""
    _require_cuda(uu, vv, ww, vis, weight, grids, norms, num_skipped)
    offs = np.ascontiguousarray(offsets, dtype=np.uint64)
    num_grids = int(offs.shape[0] - 1)
    if grids.shape[0] != num_grids or norms.shape[0] != num_grids:
        raise ValueError("grids and norms need one entry per channel")
    fn = getattr(lib(), f"gg_grid_wproj_{stack.precision}_batched_device")
    _check(fn(plan.handle, stack.handle, num_grids, _ptr(offs), _ptr(uu),
              _ptr(vv), _ptr(ww), _ptr(vis), _ptr(weight), cell_size_rad,
              w_scale, grid_size, _ptr(num_skipped), _ptr(norms), _ptr(grids),
              _stream_ptr(stream)))


def grid_wproj_batched_replay(plan, stack, vis, weight, grids, norms,
                              num_skipped, stream=None):
    """Grid new amplitudes and weights on the geometry kept by the plan's
    last batched call (same channel layout and visibility count).  Enqueues
    kernels only -- no allocation, no host synchronisation -- so it can be
    captured in a CUDA graph (pass the capturing stream, or call it inside
    ``torch.cuda.graph``, whose stream is then the current one)."""
    _require_cuda(vis, weight, grids, norms, num_skipped)
    fn = getattr(lib(), f"gg_grid_wproj_{stack.precision}_batched_replay")
    _check(fn(plan.handle, stack.handle, _ptr(vis), _ptr(weight),
              _ptr(num_skipped), _ptr(norms), _ptr(grids),
              _stream_ptr(stream)))


def check_plan(plan, stream=None):
    """Synchronise the stream and raise GridError if a gridding kernel of
    the plan flagged a failure (for replays, which do not check)."""
    _check(lib().gg_plan_check(plan.handle, _stream_ptr(stream)))


def place_wproj_device(stack, uu, vv, ww, cell_size_rad, w_scale, grid_size,
                       stream=None):
    """Per-visibility placement as the gridder computes it: int32 [N, 6] =
    (cell u, cell v, off_u, off_v, plane, flags); flags bit 0 = skipped,
    bit 1 = conjugated kernel (ww > 0)."""
    import torch
    _require_cuda(uu, vv, ww)
    n = int(uu.shape[0])
    out = torch.empty((n, 6), dtype=torch.int32, device=uu.device)
    fn = getattr(lib(), f"gg_place_wproj_{stack.precision}_device")
    _check(fn(stack.handle, n, _ptr(uu), _ptr(vv), _ptr(ww), cell_size_rad,
              w_scale, grid_size, _ptr(out), _stream_ptr(stream)))
    return out


def degrid_wproj_device(plan, stack, uu, vv, ww, cell_size_rad, w_scale,
                        grid_size, grid, out_vis, stream=None):
    """Adjoint of grid_wproj_device: out_vis[N, 2] = G^H grid."""
    _require_cuda(uu, vv, ww, grid, out_vis)
    n = int(uu.shape[0])
    fn = getattr(lib(), f"gg_degrid_wproj_{stack.precision}_device")
    _check(fn(plan.handle, stack.handle, n, _ptr(uu), _ptr(vv), _ptr(ww),
              cell_size_rad, w_scale, grid_size, _ptr(grid), _ptr(out_vis),
              _stream_ptr(stream)))


def _suffix(a):
    dt = np.asarray(a).dtype if not hasattr(a, "dtype") else a.dtype
    name = str(dt).replace("torch.", "")
    if name == "float32":
        return "f", np.float32
    if name == "float64":
        return "d", np.float64
    raise TypeError(f"float32 or float64 arrays expected, got {dt}")


# ---------------------------------------------------------------------------
# Uniform weighting (reference utils/oskar_grid_weights.c)
# ---------------------------------------------------------------------------
def grid_weights_write(uu, vv, weight, cell_size_rad, grid_size, grid=None):
    """Density grid of uniform weighting (oskar_grid_weights_write_{f,d}):
    grid[gv, gu] += weight for every point on the grid.  float32 or float64
    host arrays; grid ([G, G], accumulated) is created when None.  Returns
    (grid, num_skipped)."""
    suffix, dt = _suffix(uu)
    if grid is None:
        grid = np.zeros((grid_size, grid_size), dt)
    if not (isinstance(grid, np.ndarray) and grid.dtype == dt and
            grid.flags.c_contiguous and grid.size == grid_size * grid_size):
        raise TypeError("grid must be a C-contiguous [G, G] array of the "
                        "coordinates' dtype")
    a = [_host(uu, dt), _host(vv, dt), _host(weight, dt)]
    ns = ctypes.c_size_t(0)
    _check(getattr(lib(), f"gg_grid_weights_write_{suffix}")(
        a[0].shape[0], _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), cell_size_rad,
        grid_size, ctypes.addressof(ns), _ptr(grid)))
    return grid, int(ns.value)


def grid_weights_read(uu, vv, weight_in, weight_out, cell_size_rad,
                      grid_size, grid):
    """Uniform re-weighting (oskar_grid_weights_read_{f,d}): weight_out =
    weight_in / density for points on the grid (0 where the density is 0);
    other entries of weight_out (updated in place) are left alone.  Returns
    num_skipped."""
    suffix, dt = _suffix(uu)
    if not (isinstance(weight_out, np.ndarray) and weight_out.dtype == dt and
            weight_out.flags.c_contiguous):
        raise TypeError("weight_out must be a C-contiguous array of the "
                        "coordinates' dtype")
    a = [_host(uu, dt), _host(vv, dt), _host(weight_in, dt), _host(grid, dt)]
    ns = ctypes.c_size_t(0)
    _check(getattr(lib(), f"gg_grid_weights_read_{suffix}")(
        a[0].shape[0], _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(weight_out),
        cell_size_rad, grid_size, ctypes.addressof(ns), _ptr(a[3])))
    return int(ns.value)


def grid_weights_write_device(plan, uu, vv, weight, cell_size_rad, grid_size,
                              grid, num_skipped, stream=None):
    """Device form of grid_weights_write: torch CUDA tensors; grid [G, G]
    accumulated, num_skipped int64 [1] set."""
    _require_cuda(uu, vv, weight, grid, num_skipped)
    suffix, _ = _suffix(uu)
    _check(getattr(lib(), f"gg_grid_weights_write_{suffix}_device")(
        plan.handle, int(uu.shape[0]), _ptr(uu), _ptr(vv), _ptr(weight),
        cell_size_rad, grid_size, _ptr(num_skipped), _ptr(grid),
        _stream_ptr(stream)))


def grid_weights_read_device(plan, uu, vv, weight_in, weight_out,
                             cell_size_rad, grid_size, grid, num_skipped,
                             stream=None):
    """Device form of grid_weights_read."""
    _require_cuda(uu, vv, weight_in, weight_out, grid, num_skipped)
    suffix, _ = _suffix(uu)
    _check(getattr(lib(), f"gg_grid_weights_read_{suffix}_device")(
        plan.handle, int(uu.shape[0]), _ptr(uu), _ptr(vv), _ptr(weight_in),
        _ptr(weight_out), cell_size_rad, grid_size, _ptr(num_skipped),
        _ptr(grid), _stream_ptr(stream)))


# ---------------------------------------------------------------------------
# Degridding with host arrays
# ---------------------------------------------------------------------------
def degrid_wproj(num_w_planes, support, oversample, conv_size_half,
                 conv_func, uu, vv, ww, cell_size_rad, w_scale, grid_size,
                 grid):
    """Host form of the adjoint (gg_degrid_wproj_{f,d}): returns the
    [N, 2] visibilities G^H grid, in the coordinates' precision."""
    suffix, dt = _suffix(uu)
    a = [_host(support, np.int32), _host(conv_func, dt), _host(uu, dt),
         _host(vv, dt), _host(ww, dt), _host(grid, dt)]
    if a[5].size != 2 * grid_size * grid_size:
        raise ValueError("grid must hold grid_size^2 complex values")
    n = a[2].shape[0]
    out = np.zeros((n, 2), dt)
    _check(getattr(lib(), f"gg_degrid_wproj_{suffix}")(
        num_w_planes, _ptr(a[0]), oversample, conv_size_half, _ptr(a[1]), n,
        _ptr(a[2]), _ptr(a[3]), _ptr(a[4]), cell_size_rad, w_scale,
        grid_size, _ptr(a[5]), _ptr(out)))
    return out


def degrid_f(wl, grid):
    """degrid_wproj on a Workload in FP32."""
    return degrid_wproj(wl.num_w_planes, wl.support, wl.oversample,
                        wl.conv_size_half, wl.conv_func,
                        np.asarray(wl.uu, np.float32),
                        np.asarray(wl.vv, np.float32),
                        np.asarray(wl.ww, np.float32),
                        np.float32(wl.cell_size_rad), np.float32(wl.w_scale),
                        wl.grid_size, np.asarray(grid, np.float32))


from .autograd import GridWproj  # noqa: E402,F401
