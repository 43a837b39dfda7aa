"""GPU test of the allocation-free gridding entry point.

gg_grid_wproj_f_device_noalloc serves callers that cannot allocate device
memory while they grid (a real-time loop that must not stall on cudaMalloc,
or code running under another framework's memory pool): all its scratch is
a fixed 32 MiB device array inside the library.  This test calls it through
the C ABI twice in a row and checks each result against the allocating entry
point gg_grid_wproj_f_device on the same inputs, with the tolerances of the
other GPU tests (num_skipped exact, norm 1e-12, grid max-rel 1e-5), and
checks that inputs beyond its limits are rejected.  The file is named to be
collected last, so a run that stops at the first failure has already run
every other test.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu

_vp = ctypes.c_void_p


def _noalloc_fn(lib):
    fn = lib.gg_grid_wproj_f_device_noalloc
    fn.argtypes = [_vp, ctypes.c_size_t, _vp, _vp, _vp, _vp, _vp,
                   ctypes.c_float, ctypes.c_float, ctypes.c_int, _vp, _vp,
                   _vp, _vp]
    fn.restype = ctypes.c_int
    return fn


def test_noalloc_matches_allocating_entry_point(pkg, synthetic):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    lib = pkg.lib()
    fn = _noalloc_fn(lib)
    wl = synthetic.config0().subset(100_000)
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    uu, vv, ww = dev(wl.uu), dev(wl.vv), dev(wl.ww)
    vis, weight = dev(wl.vis), dev(wl.weight)
    G = wl.grid_size
    cell, wsc = np.float32(wl.cell_size_rad), np.float32(wl.w_scale)
    stream = torch.cuda.current_stream()

    def outputs():
        return (torch.zeros((G, G, 2), dtype=torch.float32, device="cuda"),
                torch.zeros(1, dtype=torch.float64, device="cuda"),
                torch.full((1,), -1, dtype=torch.int64, device="cuda"))

    ref_grid, ref_norm, ref_skip = outputs()
    pkg.grid_wproj_device(plan, stack, uu, vv, ww, vis, weight, cell, wsc, G,
                          ref_grid, ref_norm, ref_skip, stream)
    torch.cuda.synchronize()
    ref_g = ref_grid.cpu().numpy()

    for call in range(2):
        grid, norm, skip = outputs()
        rc = fn(stack.handle, wl.num_points, uu.data_ptr(), vv.data_ptr(),
                ww.data_ptr(), vis.data_ptr(), weight.data_ptr(), cell, wsc,
                G, skip.data_ptr(), norm.data_ptr(), grid.data_ptr(),
                stream.cuda_stream)
        assert rc == 0, pkg.last_error()
        torch.cuda.synchronize()
        assert int(skip.item()) == int(ref_skip.item()), call
        assert abs(norm.item() - ref_norm.item()) <= \
            1e-12 * abs(ref_norm.item()), call
        assert max_rel(grid.cpu().numpy(), ref_g) <= 1e-5, call


def test_noalloc_rejects_inputs_beyond_its_limits(pkg, synthetic):
    import torch
    lib = pkg.lib()
    fn = _noalloc_fn(lib)
    wl = synthetic.config0().subset(10)
    stack = pkg.KernelStack.from_workload(wl, "f")
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    # More visibilities than the array holds: rejected before any work.
    rc = fn(stack.handle, (1 << 17) + 1, p, p, p, p, p, 1.0, 1.0, 2048, p, p,
            p, None)
    assert rc == 5 and "131072" in pkg.last_error()
    # A grid side beyond the limit.
    rc = fn(stack.handle, 10, p, p, p, p, p, 1.0, 1.0, 16384, p, p, p, None)
    assert rc == 5 and "8192" in pkg.last_error()
