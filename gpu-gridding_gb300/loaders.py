"""Dataset loaders: OSKAR binary visibility files and FITS W-kernel cubes.

Thin ctypes layer over the loader entry points of libgpugrid.so
(include/gpugrid_io.h): the OSKAR binary reader that keeps the reference's
oskar_binary_* interface (utils/binary/ of the reference project), the
coordinate helpers of utils/read_vis.c:31-73 and a FITS kernel reader with
read_kernel's arguments (utils/read_kernel.c:36-118).  ``load_challenge``
strings them together as the reference's driver does (main.cpp:99-272):
one visibility file plus the real and imaginary kernel cubes become a
``synthetic.Workload`` ready for the gridder.
"""
from __future__ import annotations

import ctypes
import importlib

import numpy as np

OSKAR_CHAR, OSKAR_INT, OSKAR_SINGLE, OSKAR_DOUBLE = 0x01, 0x02, 0x04, 0x08
OSKAR_COMPLEX, OSKAR_MATRIX = 0x20, 0x40
GROUP_VIS_HEADER, GROUP_VIS_BLOCK = 11, 12
HEADER_TAGS = {"num_tags_per_block": 2, "amp_type": 5, "coord_precision": 6,
               "max_times_per_block": 7, "num_times_total": 8,
               "max_channels_per_block": 9, "num_channels_total": 10,
               "num_stations": 11}
TAG_FREQ_START_HZ = 23
BLOCK_DIMS, BLOCK_VIS, BLOCK_UU, BLOCK_VV, BLOCK_WW = 1, 3, 4, 5, 6

_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_declared = False


class LoaderError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: status {status}")
        self.status = status


def _pkg():
    return importlib.import_module(__name__.rsplit(".", 1)[0])


def lib():
    """libgpugrid.so with the loader entry points declared."""
    global _declared
    L = _pkg().lib()
    if not _declared:
        u8 = ctypes.c_ubyte
        L.oskar_binary_create.restype = _vp
        L.oskar_binary_create.argtypes = [ctypes.c_char_p, ctypes.c_char, _ip]
        L.oskar_binary_free.argtypes = [_vp]
        L.oskar_binary_free.restype = None
        L.oskar_binary_num_tags.argtypes = [_vp]
        L.oskar_binary_num_tags.restype = ctypes.c_int
        L.oskar_binary_query.argtypes = [_vp, u8, u8, u8, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_size_t), _ip]
        L.oskar_binary_query.restype = ctypes.c_int
        L.oskar_binary_read_block.argtypes = [_vp, ctypes.c_int,
                                              ctypes.c_size_t, _vp, _ip]
        L.oskar_binary_read_block.restype = None
        L.oskar_binary_read.argtypes = [_vp, u8, u8, u8, ctypes.c_int,
                                        ctypes.c_size_t, _vp, _ip]
        L.oskar_binary_read.restype = None
        L.oskar_binary_read_int.argtypes = [_vp, u8, u8, ctypes.c_int, _ip,
                                            _ip]
        L.oskar_binary_read_int.restype = None
        L.oskar_binary_read_double.argtypes = [
            _vp, u8, u8, ctypes.c_int, ctypes.POINTER(ctypes.c_double), _ip]
        L.oskar_binary_read_double.restype = None
        L.gg_vis_read_coords.argtypes = [_vp, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_size_t, _vp, _vp, _vp, _ip]
        L.gg_vis_read_coords.restype = None
        L.gg_vis_scale_coords.argtypes = [ctypes.c_double, ctypes.c_int,
                                          ctypes.c_size_t, _vp, _vp, _vp]
        L.gg_vis_scale_coords.restype = None
        L.gg_read_kernel.restype = _vp
        L.gg_read_kernel.argtypes = [
            ctypes.c_char_p, ctypes.c_int, _ip, _ip,
            ctypes.POINTER(ctypes.POINTER(ctypes.c_int)), _ip, _ip,
            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
            _ip]
        _declared = True
    return L


def _np_type(data_type: int):
    base = data_type & 0x0F
    t = {OSKAR_CHAR: np.uint8, OSKAR_INT: np.int32, OSKAR_SINGLE: np.float32,
         OSKAR_DOUBLE: np.float64}[base]
    width = (2 if data_type & OSKAR_COMPLEX else 1) * \
        (4 if data_type & OSKAR_MATRIX else 1)
    return t, width


class BinaryFile:
    """An OSKAR binary file opened for reading (oskar_binary_create 'r')."""

    def __init__(self, path: str):
        self._L = lib()
        st = ctypes.c_int(0)
        self.handle = self._L.oskar_binary_create(str(path).encode(), b"r",
                                                  ctypes.byref(st))
        if not self.handle:
            raise LoaderError(st.value, f"cannot open {path}")

    def close(self):
        if self.handle:
            self._L.oskar_binary_free(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    @property
    def num_tags(self) -> int:
        return self._L.oskar_binary_num_tags(self.handle)

    def query(self, data_type, group, tag, index=0):
        """(chunk index, payload bytes); LoaderError if absent."""
        st = ctypes.c_int(0)
        size = ctypes.c_size_t(0)
        i = self._L.oskar_binary_query(self.handle, data_type, group, tag,
                                       index, ctypes.byref(size),
                                       ctypes.byref(st))
        if st.value:
            raise LoaderError(st.value, f"tag ({group}, {tag}, {index})")
        return i, size.value

    def read(self, data_type, group, tag, index=0):
        """The payload as a numpy array of the chunk's type (complex and
        matrix elements as trailing axes of 2 and 4 reals)."""
        _, nbytes = self.query(data_type, group, tag, index)
        t, width = _np_type(data_type)
        out = np.empty(nbytes // np.dtype(t).itemsize, t)
        st = ctypes.c_int(0)
        self._L.oskar_binary_read(self.handle, data_type, group, tag, index,
                                  out.nbytes, out.ctypes.data,
                                  ctypes.byref(st))
        if st.value:
            raise LoaderError(st.value, f"tag ({group}, {tag}, {index})")
        return out.reshape(-1, width) if width > 1 else out

    def read_int(self, group, tag, index=0) -> int:
        st = ctypes.c_int(0)
        v = ctypes.c_int(0)
        self._L.oskar_binary_read_int(self.handle, group, tag, index,
                                      ctypes.byref(v), ctypes.byref(st))
        if st.value:
            raise LoaderError(st.value, f"int tag ({group}, {tag}, {index})")
        return v.value

    def read_double(self, group, tag, index=0) -> float:
        st = ctypes.c_int(0)
        v = ctypes.c_double(0)
        self._L.oskar_binary_read_double(self.handle, group, tag, index,
                                         ctypes.byref(v), ctypes.byref(st))
        if st.value:
            raise LoaderError(st.value,
                              f"double tag ({group}, {tag}, {index})")
        return v.value

    def header(self) -> dict:
        """The visibility header values the reference's driver reads."""
        h = {k: self.read_int(GROUP_VIS_HEADER, t)
             for k, t in HEADER_TAGS.items()}
        h["freq_start_hz"] = self.read_double(GROUP_VIS_HEADER,
                                              TAG_FREQ_START_HZ)
        return h

    def coords(self, block: int, precision: int, num_coords: int):
        """(uu, vv, ww) of one block in metres (gg_vis_read_coords)."""
        t = np.float64 if precision == OSKAR_DOUBLE else np.float32
        uu, vv, ww = (np.empty(num_coords, t) for _ in range(3))
        st = ctypes.c_int(0)
        self._L.gg_vis_read_coords(self.handle, block, precision, num_coords,
                                   uu.ctypes.data, vv.ctypes.data,
                                   ww.ctypes.data, ctypes.byref(st))
        if st.value:
            raise LoaderError(st.value, f"coordinates of block {block}")
        return uu, vv, ww


def scale_coords(freq_hz: float, uu, vv, ww) -> None:
    """Metres to wavelengths in place (gg_vis_scale_coords)."""
    prec = OSKAR_DOUBLE if uu.dtype == np.float64 else OSKAR_SINGLE
    for a in (uu, vv, ww):
        assert a.flags.c_contiguous and a.dtype == uu.dtype
    lib().gg_vis_scale_coords(freq_hz, prec, uu.shape[0], uu.ctypes.data,
                              vv.ctypes.data, ww.ctypes.data)


def read_kernel(path: str, precision: int = OSKAR_SINGLE) -> tuple:
    """(cube [planes, csh, csh], info dict) of a FITS kernel file."""
    L = lib()
    csh, planes, os_, gs = (ctypes.c_int(0) for _ in range(4))
    cell, wsc = ctypes.c_double(0), ctypes.c_double(0)
    sup = ctypes.POINTER(ctypes.c_int)()
    st = ctypes.c_int(0)
    p = L.gg_read_kernel(str(path).encode(), precision, ctypes.byref(csh),
                         ctypes.byref(planes), ctypes.byref(sup),
                         ctypes.byref(os_), ctypes.byref(gs),
                         ctypes.byref(cell), ctypes.byref(wsc),
                         ctypes.byref(st))
    libc = ctypes.CDLL(None)
    libc.free.argtypes = [_vp]
    if st.value or not p:
        raise LoaderError(st.value, f"{path}: {_pkg().last_error()}")
    t = ctypes.c_double if precision == OSKAR_DOUBLE else ctypes.c_float
    n = csh.value * csh.value * planes.value
    cube = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(t)),
                                 (n,)).copy()
    support = np.ctypeslib.as_array(sup, (planes.value,)).copy()
    libc.free(p)
    libc.free(ctypes.cast(sup, _vp))
    info = {"conv_size_half": csh.value, "num_w_planes": planes.value,
            "support": support.astype(np.int32), "oversample": os_.value,
            "grid_size": gs.value, "cellsize_rad": cell.value,
            "w_scale": wsc.value}
    return cube.reshape(planes.value, csh.value, csh.value), info


def load_challenge(vis_path: str, kernel_re: str, kernel_im: str):
    """A visibility file and its kernel cubes as one gridding workload, the
    way the reference's driver assembles them (main.cpp:159-189, :261-286):
    every block's coordinates scaled to wavelengths at the start frequency,
    the single-channel single-polarisation amplitudes, unit weights (the
    driver's uniform weighting is a separate step) and the complex cube
    interleaved from the two files."""
    synthetic = importlib.import_module(__name__.rsplit(".", 1)[0] +
                                        ".synthetic")
    re, info = read_kernel(kernel_re)
    im, info_im = read_kernel(kernel_im)
    if re.shape != im.shape:
        raise ValueError("real and imaginary kernel cubes differ in shape")
    conv = np.stack([re, im], axis=-1).astype(np.float32)
    with BinaryFile(vis_path) as f:
        h = f.header()
        if h["num_channels_total"] != 1 or (h["amp_type"] & OSKAR_MATRIX):
            raise ValueError("needs single-channel, single-polarisation data")
        prec = h["coord_precision"]
        parts = {k: [] for k in ("uu", "vv", "ww", "vis")}
        b = 0
        while True:
            try:
                dims = f.read(OSKAR_INT, GROUP_VIS_BLOCK, BLOCK_DIMS, b)
            except LoaderError:
                break
            n = int(dims[2]) * int(dims[4])   # times x baselines
            uu, vv, ww = f.coords(b, prec, n)
            scale_coords(h["freq_start_hz"], uu, vv, ww)
            vis = f.read(h["amp_type"], GROUP_VIS_BLOCK, BLOCK_VIS, b)
            for k, a in (("uu", uu), ("vv", vv), ("ww", ww), ("vis", vis)):
                parts[k].append(a)
            b += 1
    arr = {k: np.concatenate(v) if v else np.zeros(0) for k, v in
           parts.items()}
    n = arr["uu"].shape[0]
    return synthetic.Workload(
        name=str(vis_path), num_w_planes=info["num_w_planes"],
        support=info["support"], oversample=info["oversample"],
        conv_size_half=info["conv_size_half"], conv_func=conv,
        uu=arr["uu"].astype(np.float32), vv=arr["vv"].astype(np.float32),
        ww=arr["ww"].astype(np.float32),
        vis=np.ascontiguousarray(arr["vis"].reshape(n, 2), np.float32),
        weight=np.ones(n, np.float32),
        cell_size_rad=float(np.float32(info["cellsize_rad"])),
        w_scale=float(np.float32(info["w_scale"])),
        grid_size=info["grid_size"])
