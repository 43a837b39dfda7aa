"""Generates the loader fixtures in this folder.

* ``vis_small_f.vis``, ``vis_small_d.vis``: OSKAR binary visibility files
  written by the reference's own container library (utils/binary/src of the
  reference, compiled into oracle/_ref/libref_binary.so by
  ``make -C oracle ref-binary``), with the header tags and the per-block
  coordinate and amplitude tags the reference's driver reads
  (main.cpp:108-125, :261-272; utils/read_vis.c:31-47), two blocks each, an
  extended (named) tag between them, FP32 and FP64 coordinates.
* ``kernel_small_re.fits``, ``kernel_small_im.fits``: W-kernel cubes in the
  layout the reference's read_kernel expects (utils/read_kernel.c:36-118):
  a 3-D primary image [planes][csh][csh] with the keys OVERSAMP, GRIDSIZE,
  CELLSIZE and W_SCALE, and the per-plane supports in column 1 of a
  binary-table extension W_KERNELS.  Written here from the FITS standard
  (cfitsio, which the reference uses, is not built); the real part as FP32
  pixels with a 32-bit integer support column, the imaginary part as 16-bit
  integers with BSCALE/BZERO and an FP32 support column of repeat 2.
* ``expected.npz``: every array and value the files hold.

Usage (where the reference source is available):
    make -C oracle ref-binary
    python tests/golden/loaders/make_loader_fixtures.py
"""
from __future__ import annotations

import ctypes
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_binary.so")

CHAR, INT, SINGLE, DOUBLE, COMPLEX = 0x01, 0x02, 0x04, 0x08, 0x20
G_HEADER, G_BLOCK = 11, 12


def _writer():
    L = ctypes.CDLL(LIB)
    L.oskar_binary_create.restype = ctypes.c_void_p
    L.oskar_binary_create.argtypes = [ctypes.c_char_p, ctypes.c_char,
                                      ctypes.POINTER(ctypes.c_int)]
    L.oskar_binary_write.argtypes = [
        ctypes.c_void_p, ctypes.c_ubyte, ctypes.c_ubyte, ctypes.c_ubyte,
        ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
        ctypes.POINTER(ctypes.c_int)]
    L.oskar_binary_write_ext.argtypes = [
        ctypes.c_void_p, ctypes.c_ubyte, ctypes.c_char_p, ctypes.c_char_p,
        ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
        ctypes.POINTER(ctypes.c_int)]
    L.oskar_binary_free.argtypes = [ctypes.c_void_p]
    return L


def write_vis(path, precision, seed, exp, key):
    L = _writer()
    st = ctypes.c_int(0)
    h = L.oskar_binary_create(path.encode(), b"w", ctypes.byref(st))
    assert h and st.value == 0, st.value

    def put(dtype, group, tag, index, arr):
        a = np.ascontiguousarray(arr)
        L.oskar_binary_write(h, dtype, group, tag, index, a.nbytes,
                             a.ctypes.data, ctypes.byref(st))
        assert st.value == 0, st.value

    rng = np.random.default_rng(seed)
    real = np.float32 if precision == SINGLE else np.float64
    n_st, n_times = 12, 3
    n_bl = n_st * (n_st - 1) // 2
    freq = 1.234567e8
    ints = {2: 5, 5: SINGLE | COMPLEX, 6: precision, 7: n_times, 8: 2 * n_times,
            9: 1, 10: 1, 11: n_st}
    for tag, v in ints.items():
        put(INT, G_HEADER, tag, 0, np.array([v], np.int32))
    put(DOUBLE, G_HEADER, 23, 0, np.array([freq]))
    exp[f"{key}_header_ints"] = np.array(sorted(ints.items()), np.int64)
    exp[f"{key}_freq"] = np.array(freq)
    for b in range(2):
        n = n_times * n_bl
        dims = np.array([b * n_times, 0, n_times, 1, n_bl, n_st], np.int32)
        uu = rng.normal(0, 500, n).astype(real)
        vv = rng.normal(0, 500, n).astype(real)
        ww = rng.normal(0, 50, n).astype(real)
        vis = rng.standard_normal((n, 2)).astype(np.float32)
        put(INT, G_BLOCK, 1, b, dims)
        put(SINGLE | COMPLEX, G_BLOCK, 3, b, vis)
        put(precision, G_BLOCK, 4, b, uu)
        put(precision, G_BLOCK, 5, b, vv)
        put(precision, G_BLOCK, 6, b, ww)
        if b == 0:
            # A named (extended) chunk between the blocks.
            note = np.frombuffer(b"challenge block notes\0", np.uint8)
            L.oskar_binary_write_ext(h, CHAR, b"notes", b"text", 0,
                                     note.nbytes, note.ctypes.data,
                                     ctypes.byref(st))
            assert st.value == 0
        for name, a in (("dims", dims), ("vis", vis), ("uu", uu),
                        ("vv", vv), ("ww", ww)):
            exp[f"{key}_b{b}_{name}"] = a
    L.oskar_binary_free(h)


# ---- FITS (written from the standard) -------------------------------------
def _card(key, value=None, comment=""):
    if value is None:
        return f"{key:<8}".ljust(80)[:80]
    if isinstance(value, bool):
        v = f"{'T' if value else 'F':>20}"
    elif isinstance(value, str):
        v = f"'{value:<8}'".ljust(20)
    elif isinstance(value, int):
        v = f"{value:>20d}"
    else:
        v = f"{value:>20.15E}"
    text = f"{key:<8}= {v}" + (f" / {comment}" if comment else "")
    return text.ljust(80)[:80]


def _header(cards):
    text = "".join(cards) + _card("END")
    text += " " * (-len(text) % 2880)
    return text.encode("ascii")


def _pad(data: bytes) -> bytes:
    return data + b"\0" * (-len(data) % 2880)


def write_fits(path, cube, keys, support, bitpix, bscale=None, bzero=None,
               col_form="1J"):
    planes, csh, _ = cube.shape
    cards = [_card("SIMPLE", True), _card("BITPIX", bitpix),
             _card("NAXIS", 3), _card("NAXIS1", csh), _card("NAXIS2", csh),
             _card("NAXIS3", planes), _card("EXTEND", True)]
    if bscale is not None:
        cards += [_card("BSCALE", float(bscale)), _card("BZERO", float(bzero))]
    cards += [_card(k, v) for k, v in keys.items()]
    if bitpix == -32:
        data = cube.astype(">f4").tobytes()
    elif bitpix == 16:
        data = np.rint((cube - bzero) / bscale).astype(">i2").tobytes()
    else:
        raise ValueError(bitpix)
    # Binary table of the supports, column 1.
    repeat = int(col_form[:-1] or 1)
    code = col_form[-1]
    dt = {"J": ">i4", "E": ">f4", "I": ">i2", "D": ">f8"}[code]
    rows = -(-planes // repeat)
    col = np.zeros(rows * repeat, dt)
    col[:planes] = support
    row_bytes = np.dtype(dt).itemsize * repeat
    tcards = [_card("XTENSION", "BINTABLE"), _card("BITPIX", 8),
              _card("NAXIS", 2), _card("NAXIS1", row_bytes),
              _card("NAXIS2", rows), _card("PCOUNT", 0), _card("GCOUNT", 1),
              _card("TFIELDS", 1), _card("TFORM1", col_form),
              _card("TTYPE1", "SUPPORT"), _card("EXTNAME", "W_KERNELS")]
    # An unrelated extension first, which the reader must skip.
    other = [_card("XTENSION", "IMAGE"), _card("BITPIX", 8), _card("NAXIS", 1),
             _card("NAXIS1", 3), _card("PCOUNT", 0), _card("GCOUNT", 1),
             _card("EXTNAME", "OTHER")]
    with open(path, "wb") as f:
        f.write(_header(cards))
        f.write(_pad(data))
        f.write(_header(other))
        f.write(_pad(b"abc"))
        f.write(_header(tcards))
        f.write(_pad(col.tobytes()))


def main():
    if not os.path.isfile(LIB):
        raise SystemExit("reference container library not built: run "
                         "`make -C oracle ref-binary` where the reference "
                         "source is available")
    exp = {}
    write_vis(os.path.join(HERE, "vis_small_f.vis"), SINGLE, 1, exp, "f")
    write_vis(os.path.join(HERE, "vis_small_d.vis"), DOUBLE, 2, exp, "d")
    rng = np.random.default_rng(3)
    planes, csh = 3, 12
    re = rng.standard_normal((planes, csh, csh)).astype(np.float32)
    im = rng.standard_normal((planes, csh, csh)).astype(np.float32)
    keys = {"OVERSAMP": 4, "GRIDSIZE": 2048, "CELLSIZE": 1.9e-5,
            "W_SCALE": 0.03125}
    support = np.array([1, 2, 2], np.int32)
    write_fits(os.path.join(HERE, "kernel_small_re.fits"), re, keys, support,
               -32, col_form="1J")
    bscale, bzero = 1.0 / 4096.0, 0.5
    im_q = (np.rint((im - bzero) / bscale) * bscale + bzero)
    write_fits(os.path.join(HERE, "kernel_small_im.fits"), im_q, keys,
               support, 16, bscale, bzero, col_form="2E")
    exp["kernel_re"] = re
    exp["kernel_im"] = im_q
    exp["kernel_support"] = support
    exp["kernel_keys"] = np.array([4, 2048], np.int64)
    exp["kernel_cell_wscale"] = np.array([1.9e-5, 0.03125])
    np.savez_compressed(os.path.join(HERE, "expected.npz"), **exp)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    sys.exit(main())
