"""GPU test of the failure path, without a GPU fault.

Every mbarrier wait of the gridding kernels is bounded; when one runs out
the kernel sets its plan's error flag and returns, and the plan reports it.
The probe kernel makes such a wait run out on purpose (a barrier that
nothing arrives at, a few thousand probes) and the test checks that the
status reaches the host, that the plan keeps refusing work, and that the
device and a fresh plan still grid correctly.
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


def _grid(pkg, torch, wl, plan, stack):
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    G = wl.grid_size
    grid = torch.zeros((G, G, 2), dtype=torch.float32, device="cuda")
    norm = torch.zeros(1, dtype=torch.float64, device="cuda")
    skip = torch.zeros(1, dtype=torch.int64, device="cuda")
    pkg.grid_wproj_device(plan, stack, dev(wl.uu), dev(wl.vv), dev(wl.ww),
                          dev(wl.vis), dev(wl.weight),
                          np.float32(wl.cell_size_rad),
                          np.float32(wl.w_scale), G, grid, norm, skip)
    torch.cuda.synchronize()
    return grid.cpu().numpy(), int(skip.item())


def test_bounded_wait_runs_out_and_is_reported(pkg, oracle_mod, synthetic,
                                               torch):
    wl = synthetic.config0().subset(20_000)
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    with pytest.raises(pkg.GridError, match="bounded wait"):
        plan.probe_bounded_wait(2000)
    with pytest.raises(pkg.GridError, match="bounded wait"):
        pkg.check_plan(plan)
    with pytest.raises(pkg.GridError, match="bounded wait"):
        _grid(pkg, torch, wl, plan, stack)
    with pytest.raises(pkg.GridError):
        plan.probe_bounded_wait(0)           # argument checked first
    # The context is intact: a fresh plan grids as before.
    g, ns = _grid(pkg, torch, wl, pkg.Plan(), stack)
    gr, nsr, _ = oracle_mod.grid_f(wl)
    assert ns == nsr
    assert max_rel(g, gr) <= 1e-5
