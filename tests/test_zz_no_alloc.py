"""GPU test of the allocation-free gridding entry point.

gg_grid_wproj_f_device_noalloc serves callers that cannot allocate device
memory while they grid (a real-time loop that must not stall on cudaMalloc,
or code running under another framework's memory pool): all its scratch is
a fixed 32 MiB device array inside the library.  These tests call it through
the C ABI:

* twice in a row, each result against the FP64 oracle and against the
  allocating entry point gg_grid_wproj_f_device on the same inputs, with
  the tolerances of the other GPU tests (num_skipped exact, norm 1e-12,
  grid max-rel 1e-5), with the device's free memory unchanged by the calls;
* inputs beyond its limits (visibilities, grid side, and a call whose
  (visibility, tile) records exceed the array) are rejected with
  GG_ERR_CAPACITY and leave the grid, norm and num_skipped untouched; a
  call with no visibilities sets num_skipped to 0 and nothing else;
* a bounded wait run out on purpose (the safe probe, no fault) is reported
  by the next call, which leaves its outputs untouched, and the call after
  it succeeds.

The file is named to be collected last, so a run that stops at the first
failure has already run every other test.
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


def _outputs(G, torch):
    """A grid with a few non-zero cells, a norm of 1.25 and a skip count of
    -1, so an untouched output is recognisable."""
    grid = torch.zeros((G, G, 2), dtype=torch.float32, device="cuda")
    grid[3, 5] = torch.tensor([1.0, -2.0])
    grid[G - 1, 0] = torch.tensor([0.5, 0.25])
    return (grid, torch.full((1,), 1.25, dtype=torch.float64, device="cuda"),
            torch.full((1,), -1, dtype=torch.int64, device="cuda"))


def _call(fn, stack, n, arrs, cell, wsc, G, outs, stream):
    uu, vv, ww, vis, weight = arrs
    grid, norm, skip = outs
    return fn(stack.handle, n, uu.data_ptr(), vv.data_ptr(), ww.data_ptr(),
              vis.data_ptr(), weight.data_ptr(), cell, wsc, G,
              skip.data_ptr(), norm.data_ptr(), grid.data_ptr(),
              stream.cuda_stream)


def _untouched(outs, torch):
    grid, norm, skip = outs
    torch.cuda.synchronize()
    G = grid.shape[0]
    ref = _outputs(G, torch)
    return (torch.equal(grid, ref[0]) and norm.item() == 1.25 and
            int(skip.item()) == -1)


def test_noalloc_matches_allocating_entry_point(pkg, synthetic, oracle_mod):
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
    g64, ns64, nm64 = oracle_mod.grid_f_fp64acc(wl)

    free = []
    for call in range(3):
        if call == 1:
            # The first call on the device may load the library's module
            # holding the array; from then on the calls allocate nothing.
            torch.cuda.synchronize()
            free.append(torch.cuda.mem_get_info()[0])
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
        assert int(skip.item()) == ns64, call
        assert abs(norm.item() - nm64) <= 1e-12 * abs(nm64), call
        assert max_rel(grid.cpu().numpy(), g64) <= 1e-5, call
        del grid, norm, skip
    torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info()[0])
    assert free[0] == free[1], free


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


def test_noalloc_record_capacity_and_empty_calls(pkg, synthetic):
    """A call whose footprints need more (visibility, tile) records than
    the array holds (131,072 visibilities of support 60 on a 2048^2 grid:
    about 1.8 M records) is rejected after placement with its outputs
    untouched; the next call on the device works."""
    import torch
    fn = _noalloc_fn(pkg.lib())
    wl = synthetic.random_uniform_workload("cap", 1 << 17, 2048, 8, 60, 60,
                                           seed=5)
    stack = pkg.KernelStack.from_workload(wl, "f")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    arrs = (dev(wl.uu), dev(wl.vv), dev(wl.ww), dev(wl.vis), dev(wl.weight))
    cell, wsc = np.float32(wl.cell_size_rad), np.float32(wl.w_scale)
    stream = torch.cuda.current_stream()
    outs = _outputs(wl.grid_size, torch)
    rc = _call(fn, stack, wl.num_points, arrs, cell, wsc, wl.grid_size, outs,
               stream)
    assert rc == 5 and "1048576" in pkg.last_error()
    assert _untouched(outs, torch)
    # No visibilities: num_skipped = 0, grid and norm untouched.
    outs = _outputs(wl.grid_size, torch)
    rc = _call(fn, stack, 0, arrs, cell, wsc, wl.grid_size, outs, stream)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(outs[2].item()) == 0 and outs[1].item() == 1.25
    assert torch.equal(outs[0], _outputs(wl.grid_size, torch)[0])
    # A call within the limits right after: accepted and correct.
    n = 4096
    part = tuple(a[:n] for a in arrs)
    outs = _outputs(wl.grid_size, torch)
    start = outs[0].clone()
    rc = _call(fn, stack, n, part, cell, wsc, wl.grid_size, outs, stream)
    assert rc == 0, pkg.last_error()
    plan = pkg.Plan()
    ref = _outputs(wl.grid_size, torch)
    pkg.grid_wproj_device(plan, stack, *part, cell, wsc, wl.grid_size, *ref,
                          stream)
    torch.cuda.synchronize()
    assert int(outs[2].item()) == int(ref[2].item()) == 0
    assert abs(outs[1].item() - ref[1].item()) <= 1e-12 * abs(ref[1].item())
    assert max_rel((outs[0] - start).cpu().numpy(),
                   (ref[0] - start).cpu().numpy()) <= 1e-5


def test_noalloc_reports_an_earlier_bounded_wait_failure(pkg, synthetic):
    """The failure of an earlier call's bounded wait, made safely by the
    probe (a wait on a barrier nothing arrives at, bounded to ~1000 probes),
    is returned by the next call, which leaves its outputs untouched; the
    flag is then cleared and the following call succeeds."""
    import torch
    lib = pkg.lib()
    fn = _noalloc_fn(lib)
    probe = lib.gg_noalloc_probe_bounded_wait
    probe.argtypes = [ctypes.c_uint, _vp]
    probe.restype = ctypes.c_int
    wl = synthetic.config0().subset(20_000)
    stack = pkg.KernelStack.from_workload(wl, "f")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    arrs = (dev(wl.uu), dev(wl.vv), dev(wl.ww), dev(wl.vis), dev(wl.weight))
    cell, wsc = np.float32(wl.cell_size_rad), np.float32(wl.w_scale)
    stream = torch.cuda.current_stream()
    assert probe(1000, stream.cuda_stream) == 0, pkg.last_error()
    outs = _outputs(wl.grid_size, torch)
    rc = _call(fn, stack, wl.num_points, arrs, cell, wsc, wl.grid_size, outs,
               stream)
    assert rc == 2 and "bounded wait" in pkg.last_error()
    assert _untouched(outs, torch)
    rc = _call(fn, stack, wl.num_points, arrs, cell, wsc, wl.grid_size, outs,
               stream)
    assert rc == 0, pkg.last_error()
    torch.cuda.synchronize()
    assert int(outs[2].item()) == 0
    assert probe(0, None) == 1   # iterations outside 1..1048576
