"""GPU tests of the adjoint (degridding) kernel and the autograd binding.

* dot-product identity <G x, y> = <x, G^H y>: relative 1e-6 in FP32,
  1e-12 in FP64;
* degridding against the FP64 oracle adjoint: max-rel 1e-5 (FP32);
* torch.autograd.gradcheck in FP64 on a small case, and FP64 central
  finite differences of L = ||grid - target||^2 along a random direction on
  a 20,000-visibility subset of the synthetic-challenge shape: relative 1e-6.
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


def _setup(pkg, torch, wl, prec):
    dt = torch.float32 if prec == "f" else torch.float64
    cast = np.float32 if prec == "f" else float
    d = dict(
        stack=pkg.KernelStack.from_workload(wl, prec), plan=pkg.Plan(),
        uu=torch.from_numpy(wl.uu).to(dt).cuda(),
        vv=torch.from_numpy(wl.vv).to(dt).cuda(),
        ww=torch.from_numpy(wl.ww).to(dt).cuda(),
        cell=cast(wl.cell_size_rad), ws=cast(wl.w_scale), G=wl.grid_size,
        dt=dt)
    return d


def _forward(pkg, torch, s, vis, weight):
    G = s["G"]
    grid = torch.zeros((G, G, 2), dtype=s["dt"], device="cuda")
    norm = torch.zeros(1, dtype=torch.float64, device="cuda")
    ns = torch.zeros(1, dtype=torch.int64, device="cuda")
    pkg.grid_wproj_device(s["plan"], s["stack"], s["uu"], s["vv"], s["ww"],
                          vis.contiguous(), weight.contiguous(), s["cell"],
                          s["ws"], G, grid, norm, ns)
    return grid


def _adjoint(pkg, torch, s, grid):
    out = torch.empty((s["uu"].shape[0], 2), dtype=s["dt"], device="cuda")
    pkg.degrid_wproj_device(s["plan"], s["stack"], s["uu"], s["vv"], s["ww"],
                            s["cell"], s["ws"], s["G"], grid.contiguous(),
                            out)
    return out


def _cdot(a, b):
    """Complex inner product sum(conj(a) * b) of (.., 2) real tensors."""
    re = (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]).sum()
    im = (a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]).sum()
    return complex(re.item(), im.item())


@pytest.mark.parametrize("prec,tol,phases", [("f", 1e-6, 0), ("d", 1e-12, 0),
                                             ("f", 1e-6, 2), ("d", 1e-12, 4)])
def test_dot_product_identity(pkg, synthetic, torch, prec, tol, phases):
    """<G x, y> = <x, G^H y>, also with the gridding and the degridding on
    two and four tile phases."""
    wl = synthetic.config0().subset(60_000)
    s = _setup(pkg, torch, wl, prec)
    s["plan"].set_tuning({"tile_phases": phases})
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.randn((wl.num_points, 2), generator=g, device="cuda",
                    dtype=s["dt"])
    y = torch.randn((wl.grid_size, wl.grid_size, 2), generator=g,
                    device="cuda", dtype=s["dt"])
    ones = torch.ones(wl.num_points, dtype=s["dt"], device="cuda")
    gx = _forward(pkg, torch, s, x, ones)
    ghy = _adjoint(pkg, torch, s, y)
    lhs = _cdot(gx.double(), y.double())
    rhs = _cdot(x.double(), ghy.double())
    rel = abs(lhs - rhs) / abs(lhs)
    print(f"dot-product test ({prec}): relative mismatch {rel:.2e}")
    assert rel <= tol


def test_dot_product_identity_cfg1_shape(pkg, synthetic, torch):
    """The FP32 dot-product identity on the whole synthetic-challenge shape
    the gridding/degridding pair is stated on (2,152,800 visibilities,
    8192^2 grid, 714 w-planes, support 4..36): relative 1e-6."""
    wl = synthetic.config1()
    s = _setup(pkg, torch, wl, "f")
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn((wl.num_points, 2), generator=g, device="cuda",
                    dtype=torch.float32)
    y = torch.randn((wl.grid_size, wl.grid_size, 2), generator=g,
                    device="cuda", dtype=torch.float32)
    ones = torch.ones(wl.num_points, dtype=torch.float32, device="cuda")
    gx = _forward(pkg, torch, s, x, ones)
    ghy = _adjoint(pkg, torch, s, y)
    lhs = _cdot(gx.double(), y.double())
    rhs = _cdot(x.double(), ghy.double())
    rel = abs(lhs - rhs) / abs(lhs)
    print(f"dot-product test (cfg1 shape, FP32): relative mismatch "
          f"{rel:.2e}")
    assert rel <= 1e-6


@pytest.mark.parametrize("phases", [0, 1, 2, 4])
def test_degrid_matches_fp64_oracle(pkg, oracle_mod, torch, phases):
    wl, _ = load_golden("small_f")
    s = _setup(pkg, torch, wl, "f")
    s["plan"].set_tuning({"tile_phases": phases})
    rng = np.random.default_rng(3)
    y = rng.standard_normal((wl.grid_size, wl.grid_size, 2))
    out = _adjoint(pkg, torch, s, torch.from_numpy(
        y.astype(np.float32)).cuda()).cpu().numpy()
    ref = oracle_mod.degrid_fp64(wl, y.astype(np.float32).astype(np.float64))
    assert max_rel(out, ref) <= 1e-5
    p = oracle_mod.place(wl)
    assert not out[p["skipped"] == 1].any()   # skipped points get 0


def test_gradcheck_fp64_small(pkg, synthetic, torch):
    wl = synthetic.random_uniform_workload("gc", 40, 48, 6, 1, 4, seed=9,
                                           cell_size_rad=4e-3)
    s = _setup(pkg, torch, wl, "d")
    vis = torch.from_numpy(wl.vis).double().cuda().requires_grad_(True)
    w = torch.from_numpy(wl.weight).double().cuda().requires_grad_(True)

    def fn(v, ww):
        return pkg.GridWproj.apply(v, ww, s["uu"], s["vv"], s["ww"],
                                   s["stack"], s["plan"], s["cell"], s["ws"],
                                   s["G"])

    assert torch.autograd.gradcheck(fn, (vis, w), eps=1e-6, atol=1e-8,
                                    rtol=1e-6, fast_mode=True)


def test_finite_differences_fp64_cfg1_subset(pkg, synthetic, torch):
    """Central differences of L = ||grid - target||^2 along a random
    direction in (vis, weight) on 20,000 visibilities of the
    synthetic-challenge shape, against the autograd gradient."""
    wl = synthetic.config1().subset(20_000)
    s = _setup(pkg, torch, wl, "d")
    gen = torch.Generator(device="cuda").manual_seed(4)
    vis0 = torch.from_numpy(wl.vis).double().cuda()
    w0 = torch.from_numpy(wl.weight).double().cuda()
    target = torch.randn((wl.grid_size, wl.grid_size, 2), generator=gen,
                         device="cuda", dtype=torch.float64) * 1e-3
    dv = torch.randn(vis0.shape, generator=gen, device="cuda",
                     dtype=torch.float64)
    dw = torch.randn(w0.shape, generator=gen, device="cuda",
                     dtype=torch.float64)

    def loss(v, w):
        g = pkg.GridWproj.apply(v, w, s["uu"], s["vv"], s["ww"], s["stack"],
                                s["plan"], s["cell"], s["ws"], s["G"])
        return ((g - target) ** 2).sum()

    v = vis0.clone().requires_grad_(True)
    w = w0.clone().requires_grad_(True)
    L = loss(v, w)
    L.backward()
    analytic = (v.grad * dv).sum().item() + (w.grad * dw).sum().item()
    h = 1e-4
    with torch.no_grad():
        lp = loss(vis0 + h * dv, w0 + h * dw).item()
        lm = loss(vis0 - h * dv, w0 - h * dw).item()
    numeric = (lp - lm) / (2 * h)
    rel = abs(numeric - analytic) / abs(analytic)
    print(f"finite differences: analytic {analytic:.9e} numeric "
          f"{numeric:.9e} rel {rel:.2e}")
    assert rel <= 1e-6


def test_degrid_fp64_matches_fp64_oracle(pkg, oracle_mod, synthetic, torch):
    """FP64 degridding against the FP64 adjoint (FP64 placement and cube)."""
    wl = synthetic.random_uniform_workload("degrid_d", 3_000, 512, 16, 2, 10,
                                           seed=21, cell_size_rad=8e-5)
    s = _setup(pkg, torch, wl, "d")
    rng = np.random.default_rng(5)
    y = rng.standard_normal((wl.grid_size, wl.grid_size, 2))
    out = _adjoint(pkg, torch, s, torch.from_numpy(y).cuda()).cpu().numpy()
    ref = oracle_mod.degrid_d(wl, y)
    assert max_rel(out, ref) <= 1e-12
    p = oracle_mod.place(wl, "d")
    assert p["num_skipped"] < wl.num_points
    assert not out[p["skipped"] == 1].any()


DEGRID_TUNINGS = [{"plane_group_mb": 1}, {"items_per_cta": 1},
                  {"items_per_cta": 64}, {"sort_detail": 0},
                  {"sort_detail": 1, "ctas_per_sm": 1}]


def test_degrid_bit_identical_across_tunings(pkg, synthetic, torch):
    """Each record's partial result is formed the same way whichever CTA
    takes it, and each visibility adds its records in emission order, so
    plane groups, work-item splitting, record order and CTA count leave
    the output bit for bit unchanged (tile phases change which tiles a
    visibility's sum is cut into, so they are held at the default)."""
    wl = synthetic.config0().subset(40_000)
    s = _setup(pkg, torch, wl, "f")
    g = torch.Generator(device="cuda").manual_seed(7)
    y = torch.randn((wl.grid_size, wl.grid_size, 2), generator=g,
                    device="cuda", dtype=torch.float32)
    base = _adjoint(pkg, torch, s, y).cpu().numpy()
    again = _adjoint(pkg, torch, s, y).cpu().numpy()
    assert np.array_equal(base.view(np.uint32), again.view(np.uint32))
    for t in DEGRID_TUNINGS:
        plan = pkg.Plan()
        plan.set_tuning(t)
        s2 = dict(s, plan=plan)
        got = _adjoint(pkg, torch, s2, y).cpu().numpy()
        if t.get("plane_group_mb") == 1:
            assert plan.stats()["num_plane_groups"] > 1
        assert np.array_equal(got.view(np.uint32), base.view(np.uint32)), t
