"""GPU tests of W-kernel generation on the device.

The generated cube follows the taper x chirp recipe of synthetic.py's
make_kernel_stack (computed in FP64, rounded once to FP32), so it must
agree with the host recipe to FP32 rounding (the two use different exp /
sincos implementations and summation orders for the normalisation), and a
kernel stack generated on the device must grid like one built from the
host cube: same placement and skips, norm to 1e-6, grid within 1e-5.
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


def _recipe_w(num_planes):
    return 8.0 * np.arange(num_planes) / max(num_planes - 1, 1)


@pytest.mark.parametrize("planes,s_min,s_max,os_", [(16, 1, 12, 4),
                                                   (5, 0, 6, 3), (3, 2, 4, 1)])
def test_generated_cube_matches_host_recipe(pkg, synthetic, torch, planes,
                                            s_min, s_max, os_):
    support = synthetic.linear_supports(planes, s_min, s_max)
    csh = (int(support.max()) + 1) * os_
    host = synthetic.make_kernel_stack(support, os_, csh)
    cube = torch.zeros(host.shape, dtype=torch.float32, device="cuda")
    stack = pkg.KernelStack.generate(planes, support, os_, csh,
                                     _recipe_w(planes), "f", cube_out=cube)
    torch.cuda.synchronize()
    got = cube.cpu().numpy()
    scale = np.abs(host).max()
    assert np.abs(got - host).max() <= 1e-6 * scale
    stack.close()


def test_generated_stack_grids_like_host_stack(pkg, synthetic, torch):
    wl = synthetic.config0().subset(50_000)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    gen = pkg.KernelStack.generate(wl.num_w_planes, wl.support, wl.oversample,
                                   wl.conv_size_half,
                                   _recipe_w(wl.num_w_planes), "f")
    host = pkg.KernelStack.from_workload(wl, "f")
    out = []
    for stack in (gen, host):
        G = wl.grid_size
        grid = torch.zeros((G, G, 2), dtype=torch.float32, device="cuda")
        norm = torch.zeros(1, dtype=torch.float64, device="cuda")
        skip = torch.zeros(1, dtype=torch.int64, device="cuda")
        pkg.grid_wproj_device(pkg.Plan(), stack, dev(wl.uu), dev(wl.vv),
                              dev(wl.ww), dev(wl.vis), dev(wl.weight),
                              np.float32(wl.cell_size_rad),
                              np.float32(wl.w_scale), G, grid, norm, skip)
        torch.cuda.synchronize()
        out.append((grid.cpu().numpy(), float(norm.item()), int(skip.item())))
    assert out[0][2] == out[1][2]
    assert abs(out[0][1] - out[1][1]) <= 1e-6 * abs(out[1][1])
    assert max_rel(out[0][0], out[1][0]) <= 1e-5


def test_generate_rejects_bad_arguments(pkg, torch):
    with pytest.raises(pkg.GridError):        # conv_size_half too small
        pkg.KernelStack.generate(2, [4, 4], 4, 10, [0.0, 1.0], "f")
    with pytest.raises(ValueError):
        pkg.KernelStack.generate(2, [1, 1], 4, 16, [0.0], "f")
