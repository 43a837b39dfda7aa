"""CPU tests of the C ABI: the library loads, exports exactly what
include/gpugrid.h declares, and rejects invalid arguments with a status and
a message before touching the GPU (so these run without one)."""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

HEADER = os.path.join(ROOT, "include", "gpugrid.h")
HEADERS = [os.path.join(ROOT, "include", h) for h in
           sorted(os.listdir(os.path.join(ROOT, "include")))
           if h.endswith(".h")]


def declared_symbols():
    text = "".join(open(h).read() for h in HEADERS)
    return sorted(set(re.findall(r"GG_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


def test_header_declarations_match_python_binding(pkg):
    assert declared_symbols() == sorted(pkg.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(pkg):
    L = pkg.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", pkg.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = sorted(line.split()[-1] for line in out.splitlines()
                      if " T " in line)
    # Nothing else leaks out of the library (static CUDA runtime included).
    assert exported == declared_symbols()


def test_drop_in_signature_is_the_references():
    """The two drop-ins keep oskar_grid_wproj.h's parameter list."""
    text = open(HEADER).read()
    for suffix, real in (("d", "double"), ("f", "float")):
        m = re.search(r"void oskar_grid_wproj_%s\((.*?)\);" % suffix, text,
                      re.S)
        params = [p.strip() for p in m.group(1).replace("\n", " ").split(",")]
        names = [re.findall(r"(\w+)$", p)[0] for p in params]
        assert names == ["num_w_planes", "support", "oversample",
                         "conv_size_half", "conv_func", "num_points", "uu",
                         "vv", "ww", "vis", "weight", "cell_size_rad",
                         "w_scale", "grid_size", "num_skipped", "norm",
                         "grid"]
        assert params[16].startswith(f"{real}* grid")
        assert params[15] == "double* norm"


def _call_f(pkg, wl, **over):
    args = dict(num_w_planes=wl.num_w_planes, support=wl.support,
                oversample=wl.oversample, conv_size_half=wl.conv_size_half,
                conv_func=wl.conv_func, num_points=wl.num_points, uu=wl.uu,
                vv=wl.vv, ww=wl.ww, vis=wl.vis, weight=wl.weight,
                cell_size_rad=np.float32(wl.cell_size_rad),
                w_scale=np.float32(wl.w_scale), grid_size=wl.grid_size,
                grid=np.zeros((wl.grid_size, wl.grid_size, 2), np.float32))
    args.update(over)
    return pkg.oskar_grid_wproj_f(**args)


@pytest.mark.parametrize("over,needle", [
    (dict(num_w_planes=0), "num_w_planes"),
    (dict(oversample=0), "oversample"),
    (dict(oversample=15), "oversample"),
    (dict(conv_size_half=4), "conv_size_half"),
    (dict(support=np.full(8, -1, np.int32)), "support"),
])
def test_invalid_arguments_rejected_before_gpu(pkg, over, needle):
    wl, _ = load_golden("small_f")
    with pytest.raises(pkg.GridError) as e:
        _call_f(pkg, wl, **over)
    assert e.value.code == 1
    assert needle in str(e.value)


def test_grid_size_limit(pkg):
    wl, _ = load_golden("small_f")
    L = pkg.lib()
    g = np.zeros(2, np.float32)
    ns = ctypes.c_size_t(0)
    nm = ctypes.c_double(0)
    r = L.gg_grid_wproj_f(wl.num_w_planes, wl.support.ctypes.data,
                          wl.oversample, wl.conv_size_half,
                          wl.conv_func.ctypes.data, 0, None, None, None, None,
                          None, 1.0, 1.0, 70000, ctypes.addressof(ns),
                          ctypes.addressof(nm), g.ctypes.data)
    assert r == 4 and "grid_size" in pkg.last_error()


def test_null_outputs_rejected(pkg):
    wl, _ = load_golden("small_f")
    L = pkg.lib()
    r = L.gg_grid_wproj_f(wl.num_w_planes, wl.support.ctypes.data,
                          wl.oversample, wl.conv_size_half,
                          wl.conv_func.ctypes.data, 0, None, None, None, None,
                          None, 1.0, 1.0, 64, None, None, None)
    assert r == 1
    # The void drop-in reports through gg_last_error and leaves outputs.
    L.oskar_grid_wproj_f(wl.num_w_planes, wl.support.ctypes.data,
                         wl.oversample, 2, wl.conv_func.ctypes.data, 0, None,
                         None, None, None, None, 1.0, 1.0, 64, None, None,
                         None)
    assert pkg.last_error() != ""


def test_kernel_stack_validation(pkg):
    wl, _ = load_golden("small_f")
    L = pkg.lib()
    h = ctypes.c_void_p(0)
    r = L.gg_kernels_create_f(ctypes.byref(h), wl.num_w_planes,
                              wl.support.ctypes.data, 0, wl.conv_size_half,
                              wl.conv_func.ctypes.data, 0, None)
    assert r == 1 and not h.value
