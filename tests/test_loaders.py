"""CPU tests of the dataset loaders (include/gpugrid_io.h).

* OSKAR binary visibility files written by the reference's own container
  library (tests/golden/loaders/vis_small_{f,d}.vis,
  made by tests/golden/loaders/make_loader_fixtures.py): every header value, block
  dimension, coordinate and amplitude read back bit for bit; a named
  (extended) chunk between the blocks is skipped; a flipped payload byte
  fails the CRC-32C check; missing tags, short buffers, truncated files,
  bad magic and write mode fail with the reference's status codes; and,
  where the reference's reader is built here, the chunk index and every
  payload equal the reference reader's.
* FITS W-kernel cubes (tests/golden/loaders/kernel_small_{re,im}.fits): the cube,
  the four header keys and the per-plane supports, for FP32 pixels with an
  int32 support column and for 16-bit pixels with BSCALE/BZERO and an FP32
  support column of repeat 2; missing keys and wrong dimensionality fail.
* load_challenge assembles both into a gridding workload as the reference's
  driver does.
"""
from __future__ import annotations

import ctypes
import importlib
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

LOADERS = os.path.join(GOLDEN, "loaders")

OSKAR_ERR = {"open": -100, "read": -102, "file_invalid": -106,
             "memory": -114, "not_found": -115, "crc": -118}


@pytest.fixture(scope="module")
def ld(pkg):
    return importlib.import_module(pkg.__name__ + ".loaders")


@pytest.fixture(scope="module")
def expected():
    return dict(np.load(os.path.join(LOADERS, "expected.npz")))


def _path(name):
    return os.path.join(LOADERS, name)


@pytest.mark.parametrize("key", ["f", "d"])
def test_vis_file_reads_back_exactly(ld, expected, key):
    with ld.BinaryFile(_path(f"vis_small_{key}.vis")) as f:
        # 9 header chunks, 2 blocks of 5, one named chunk.
        assert f.num_tags == 9 + 2 * 5 + 1
        h = f.header()
        for tag, v in expected[f"{key}_header_ints"]:
            name = [k for k, t in ld.HEADER_TAGS.items() if t == tag][0]
            assert h[name] == v, name
        assert h["freq_start_hz"] == float(expected[f"{key}_freq"])
        prec = h["coord_precision"]
        for b in range(2):
            dims = f.read(ld.OSKAR_INT, ld.GROUP_VIS_BLOCK, ld.BLOCK_DIMS, b)
            assert np.array_equal(dims, expected[f"{key}_b{b}_dims"])
            n = int(dims[2]) * int(dims[4])
            uu, vv, ww = f.coords(b, prec, n)
            for name, a in (("uu", uu), ("vv", vv), ("ww", ww)):
                e = expected[f"{key}_b{b}_{name}"]
                assert a.dtype == e.dtype
                assert np.array_equal(a.view(np.uint8), e.view(np.uint8))
            vis = f.read(h["amp_type"], ld.GROUP_VIS_BLOCK, ld.BLOCK_VIS, b)
            assert np.array_equal(vis, expected[f"{key}_b{b}_vis"])


def test_scale_coords_matches_the_reference_rule(ld, expected):
    """utils/read_vis.c:49-73: scale = freq / c in FP64, FP32 arrays take
    the FP32-rounded scale."""
    freq = 1.234567e8
    for key, t in (("f", np.float32), ("d", np.float64)):
        uu = expected[f"{key}_b0_uu"].copy()
        vv = expected[f"{key}_b0_vv"].copy()
        ww = expected[f"{key}_b0_ww"].copy()
        ld.scale_coords(freq, uu, vv, ww)
        s = t(freq / 299792458.0)
        for a, name in ((uu, "uu"), (vv, "vv"), (ww, "ww")):
            e = expected[f"{key}_b0_{name}"] * s
            assert a.dtype == t and np.array_equal(a, e.astype(t))


def test_vis_file_errors(ld, tmp_path):
    src = _path("vis_small_f.vis")
    with ld.BinaryFile(src) as f:
        with pytest.raises(ld.LoaderError) as e:
            f.read(ld.OSKAR_SINGLE, ld.GROUP_VIS_BLOCK, ld.BLOCK_UU, 7)
        assert e.value.status == OSKAR_ERR["not_found"]
        L = ld.lib()
        st = ctypes.c_int(0)
        i, nbytes = f.query(ld.OSKAR_SINGLE, ld.GROUP_VIS_BLOCK,
                            ld.BLOCK_UU, 0)
        small = np.empty(nbytes // 4 - 1, np.float32)
        L.oskar_binary_read_block(f.handle, i, small.nbytes,
                                  small.ctypes.data, ctypes.byref(st))
        assert st.value == OSKAR_ERR["memory"]
    # One flipped payload byte: the chunk's CRC-32C no longer matches.
    bad = tmp_path / "crc.vis"
    shutil.copy(src, bad)
    with ld.BinaryFile(src) as f:
        L = ld.lib()
        i, _ = f.query(ld.OSKAR_SINGLE, ld.GROUP_VIS_BLOCK, ld.BLOCK_UU, 1)
    raw = bytearray(bad.read_bytes())
    # The payload of chunk i starts after the tag; find it through the
    # reader's own index by flipping a byte in the uu payload of block 1.
    uu1 = np.load(os.path.join(LOADERS, "expected.npz"))["f_b1_uu"]
    pos = bytes(raw).find(uu1.tobytes())
    assert pos > 0
    raw[pos + 5] ^= 0x10
    bad.write_bytes(bytes(raw))
    with ld.BinaryFile(bad) as f:
        with pytest.raises(ld.LoaderError) as e:
            f.read(ld.OSKAR_SINGLE, ld.GROUP_VIS_BLOCK, ld.BLOCK_UU, 1)
        assert e.value.status == OSKAR_ERR["crc"]
        f.read(ld.OSKAR_SINGLE, ld.GROUP_VIS_BLOCK, ld.BLOCK_UU, 0)  # intact
    # Cut short inside the last payload: indexed, fails when read.
    cut = tmp_path / "cut.vis"
    data = open(src, "rb").read()
    cut.write_bytes(data[:-30])
    with pytest.raises(ld.LoaderError) as e:
        with ld.BinaryFile(cut) as f:
            f.read(ld.OSKAR_SINGLE, ld.GROUP_VIS_BLOCK, ld.BLOCK_WW, 1)
    assert e.value.status in (OSKAR_ERR["read"], OSKAR_ERR["file_invalid"])
    # Not an OSKAR file; write mode; missing file.
    junk = tmp_path / "junk.vis"
    junk.write_bytes(b"NOTOSKAR" + bytes(100))
    with pytest.raises(ld.LoaderError) as e:
        ld.BinaryFile(junk)
    assert e.value.status == OSKAR_ERR["file_invalid"]
    st = ctypes.c_int(0)
    assert not ld.lib().oskar_binary_create(str(junk).encode(), b"w",
                                            ctypes.byref(st))
    assert st.value == OSKAR_ERR["open"]
    with pytest.raises(ld.LoaderError) as e:
        ld.BinaryFile(tmp_path / "absent.vis")
    assert e.value.status == OSKAR_ERR["open"]


def test_vis_index_matches_the_reference_reader(ld):
    """Chunk count, and for every standard chunk the same index and payload
    as the reference's own reader (built here from its source)."""
    so = os.path.join(ROOT, "oracle", "_ref", "libref_binary.so")
    if not os.path.isfile(so):
        pytest.skip("the reference's container library is not built here")
    R = ctypes.CDLL(so)
    R.oskar_binary_create.restype = ctypes.c_void_p
    R.oskar_binary_create.argtypes = [ctypes.c_char_p, ctypes.c_char,
                                      ctypes.POINTER(ctypes.c_int)]
    R.oskar_binary_num_tags.argtypes = [ctypes.c_void_p]
    R.oskar_binary_query.argtypes = [
        ctypes.c_void_p, ctypes.c_ubyte, ctypes.c_ubyte, ctypes.c_ubyte,
        ctypes.c_int, ctypes.POINTER(ctypes.c_size_t),
        ctypes.POINTER(ctypes.c_int)]
    R.oskar_binary_read_block.argtypes = [
        ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
        ctypes.POINTER(ctypes.c_int)]
    R.oskar_binary_free.argtypes = [ctypes.c_void_p]
    for name in ("vis_small_f.vis", "vis_small_d.vis"):
        st = ctypes.c_int(0)
        r = R.oskar_binary_create(_path(name).encode(), b"r",
                                  ctypes.byref(st))
        assert r and st.value == 0
        with ld.BinaryFile(_path(name)) as f:
            assert f.num_tags == R.oskar_binary_num_tags(r)
            for group, tags in ((11, (2, 5, 6, 7, 8, 9, 10, 11, 23)),
                                (12, (1, 3, 4, 5, 6))):
                for tag in tags:
                    for b in ((0,) if group == 11 else (0, 1)):
                        size = ctypes.c_size_t(0)
                        st = ctypes.c_int(0)
                        ri = R.oskar_binary_query(r, 0, group, tag, b,
                                                  ctypes.byref(size),
                                                  ctypes.byref(st))
                        mi, msize = f.query(0, group, tag, b)
                        assert (ri, size.value) == (mi, msize)
                        ref = np.empty(msize, np.uint8)
                        R.oskar_binary_read_block(r, ri, msize,
                                                  ref.ctypes.data,
                                                  ctypes.byref(st))
                        assert st.value == 0
                        mine = np.empty(msize, np.uint8)
                        st2 = ctypes.c_int(0)
                        ld.lib().oskar_binary_read_block(
                            f.handle, mi, msize, mine.ctypes.data,
                            ctypes.byref(st2))
                        assert st2.value == 0
                        assert np.array_equal(ref, mine)
        R.oskar_binary_free(r)


@pytest.mark.parametrize("part", ["re", "im"])
@pytest.mark.parametrize("precision", [0x04, 0x08])
def test_fits_kernel_reads_back(ld, expected, part, precision):
    cube, info = ld.read_kernel(_path(f"kernel_small_{part}.fits"),
                                precision)
    e = expected[f"kernel_{part}"]
    assert cube.shape == e.shape
    assert cube.dtype == (np.float64 if precision == 0x08 else np.float32)
    tol = 0 if part == "re" else 1e-12
    # 16-bit pixels: BZERO + BSCALE * stored, exact in FP64, FP32-rounded.
    ref = e.astype(np.float64) if precision == 0x08 else e.astype(np.float32)
    assert np.allclose(cube, ref, rtol=0, atol=tol if precision == 0x08 else
                       1e-7)
    assert np.array_equal(info["support"], expected["kernel_support"])
    assert (info["oversample"], info["grid_size"]) == tuple(
        expected["kernel_keys"])
    assert (info["cellsize_rad"], info["w_scale"]) == tuple(
        expected["kernel_cell_wscale"])
    assert info["conv_size_half"] == e.shape[1]
    assert info["num_w_planes"] == e.shape[0]


def test_fits_kernel_errors(ld, tmp_path):
    src = open(_path("kernel_small_re.fits"), "rb").read()
    # Without the OVERSAMP card.
    i = src.find(b"OVERSAMP")
    bad = bytearray(src)
    bad[i:i + 8] = b"OVERSAMX"
    p = tmp_path / "nokey.fits"
    p.write_bytes(bytes(bad))
    with pytest.raises(ld.LoaderError) as e:
        ld.read_kernel(p)
    assert "OVERSAMP" in str(e.value)
    # A 2-D image.
    i = src.find(b"NAXIS   =")
    bad = bytearray(src)
    bad[i + 29] = ord("2")
    p = tmp_path / "naxis.fits"
    p.write_bytes(bytes(bad))
    with pytest.raises(ld.LoaderError) as e:
        ld.read_kernel(p)
    assert "3D" in str(e.value)
    # No W_KERNELS table.
    bad = src.replace(b"'W_KERNELS'", b"'W_OTHER  '")
    p = tmp_path / "notable.fits"
    p.write_bytes(bad)
    with pytest.raises(ld.LoaderError) as e:
        ld.read_kernel(p)
    assert "W_KERNELS" in str(e.value)


def test_load_challenge_assembles_a_workload(ld, expected):
    wl = ld.load_challenge(_path("vis_small_f.vis"),
                           _path("kernel_small_re.fits"),
                           _path("kernel_small_im.fits"))
    s = np.float32(1.234567e8 / 299792458.0)
    uu = np.concatenate([expected["f_b0_uu"], expected["f_b1_uu"]]) * s
    assert np.array_equal(wl.uu, uu.astype(np.float32))
    vis = np.concatenate([expected["f_b0_vis"], expected["f_b1_vis"]])
    assert np.array_equal(wl.vis, vis)
    assert wl.conv_func.shape == (3, 12, 12, 2)
    assert np.array_equal(wl.conv_func[..., 0], expected["kernel_re"])
    assert np.array_equal(wl.support, expected["kernel_support"])
    assert wl.grid_size == 2048 and wl.oversample == 4
    assert np.all(wl.weight == 1)


@pytest.mark.gpu
def test_loaded_dataset_grids_on_the_gpu(ld, pkg, oracle_mod):
    """A workload read by the loaders grids through the drop-in as the FP64
    oracle says (skips exact, grid max-rel 1e-5, norm 1e-12)."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    wl = ld.load_challenge(_path("vis_small_f.vis"),
                           _path("kernel_small_re.fits"),
                           _path("kernel_small_im.fits"))
    g, ns, nm = pkg.grid_f(wl)
    g64, ns64, nm64 = oracle_mod.grid_f_fp64acc(wl)
    assert ns == ns64
    assert abs(nm - nm64) <= 1e-12 * abs(nm64)
    err = np.abs(g.astype(np.float64) - g64).max() / np.abs(g64).max()
    assert err <= 1e-5
