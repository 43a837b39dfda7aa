"""Seeded synthetic gridding workloads.

The reference's challenge datasets (OSKAR ``.vis`` files plus FITS kernel
cubes, README:122-134 of the reference) are not available, so these
generators build shape-matched stand-ins: the same visibility counts,
w-plane counts, supports, oversampling and grid sizes, with the value
distributions stated per workload below.  Every array is produced by numpy's
PCG64 generator from a fixed seed, so a workload is reproducible bit for bit.

Arrays follow the reference's gridder contract (oskar_grid_wproj.h:114-131):
``uu, vv, ww, weight`` are float32[N], ``vis`` is float32[N, 2] (re, im
interleaved), ``support`` is int32[P] and ``conv_func`` is
float32[P, conv_size_half, conv_size_half, 2], the first quadrant of each
oversampled kernel with rows indexed by |v offset| and columns by |u offset|.

Kernel recipe (all workloads): plane p has support s_p rising linearly with
p (so linearly in sqrt|w|, since the plane index is round(sqrt(|w| w_scale)));
its taps are a Gaussian taper exp(-2 (r / s_p)^2), r in grid cells, times a
chirp exp(i pi w_p r_os^2 / conv_size_half^2), r_os in oversampled pixels and
w_p = 8 p / (P - 1), normalised so the taps at zero offset sum to 1.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SPEED_OF_LIGHT = 299792458.0


@dataclasses.dataclass
class Workload:
    """One gridding problem in the reference's argument layout."""

    name: str
    num_w_planes: int
    support: np.ndarray          # int32[P]
    oversample: int
    conv_size_half: int
    conv_func: np.ndarray        # float32[P, csh, csh, 2]
    uu: np.ndarray               # float32[N]
    vv: np.ndarray               # float32[N]
    ww: np.ndarray               # float32[N]
    vis: np.ndarray              # float32[N, 2]
    weight: np.ndarray           # float32[N]
    cell_size_rad: float         # float32-representable
    w_scale: float               # float32-representable
    grid_size: int
    # Per-channel offsets into the visibility arrays for batched workloads
    # (None for single-grid workloads).
    channel_offsets: np.ndarray | None = None

    @property
    def num_points(self) -> int:
        return int(self.uu.shape[0])

    @property
    def num_grids(self) -> int:
        if self.channel_offsets is None:
            return 1
        return int(self.channel_offsets.shape[0] - 1)

    def channel(self, c: int) -> "Workload":
        """The single-grid workload of channel c of a batched workload."""
        if self.channel_offsets is None:
            if c != 0:
                raise IndexError(c)
            return self
        a, b = int(self.channel_offsets[c]), int(self.channel_offsets[c + 1])
        return dataclasses.replace(
            self, name=f"{self.name}[ch{c}]", uu=self.uu[a:b], vv=self.vv[a:b],
            ww=self.ww[a:b], vis=self.vis[a:b], weight=self.weight[a:b],
            channel_offsets=None)

    def strided(self, k: int) -> "Workload":
        """Every k-th visibility (same kernels and grid): a sample with the
        workload's own uv, w and support distribution."""
        if k <= 1:
            return self
        return dataclasses.replace(
            self, name=f"{self.name}[::{k}]", uu=self.uu[::k].copy(),
            vv=self.vv[::k].copy(), ww=self.ww[::k].copy(),
            vis=self.vis[::k].copy(), weight=self.weight[::k].copy(),
            channel_offsets=None)

    def subset(self, n: int) -> "Workload":
        """The first n visibilities (same kernels and grid)."""
        return dataclasses.replace(
            self, name=f"{self.name}[:{n}]", uu=self.uu[:n], vv=self.vv[:n],
            ww=self.ww[:n], vis=self.vis[:n], weight=self.weight[:n],
            channel_offsets=None)


def linear_supports(num_w_planes: int, s_min: int, s_max: int) -> np.ndarray:
    """Support rising linearly with the plane index from s_min to s_max."""
    if num_w_planes == 1:
        return np.array([s_max], dtype=np.int32)
    p = np.arange(num_w_planes, dtype=np.float64)
    return np.rint(s_min + (s_max - s_min) * p / (num_w_planes - 1)).astype(
        np.int32)


def make_kernel_stack(support: np.ndarray, oversample: int,
                      conv_size_half: int) -> np.ndarray:
    """Taper x chirp kernel quadrants, float32[P, csh, csh, 2]."""
    num_planes = int(support.shape[0])
    out = np.zeros((num_planes, conv_size_half, conv_size_half, 2),
                   dtype=np.float32)
    idx = np.arange(conv_size_half, dtype=np.float64)
    r2_os = idx[:, None] ** 2 + idx[None, :] ** 2          # oversampled px^2
    r2_cells = r2_os / float(oversample * oversample)
    for p in range(num_planes):
        s = max(int(support[p]), 1)
        w_p = 8.0 * p / max(num_planes - 1, 1)
        taper = np.exp(-2.0 * r2_cells / float(s * s))
        phase = math.pi * w_p * r2_os / float(conv_size_half ** 2)
        k = taper * np.exp(1j * phase)
        # Normalise so the zero-offset taps over the full footprint sum to 1.
        taps = np.abs(np.arange(-s, s + 1)) * oversample
        taps = taps[taps < conv_size_half]
        total = k[np.ix_(taps, taps)].sum()
        k = k / total
        out[p, :, :, 0] = k.real
        out[p, :, :, 1] = k.imag
    return out


def _radial_uv(rng, n, grid_size, cell_size_rad, sigma_frac=0.12,
               clip_frac=0.45):
    """Radially concentrated (u, v) in wavelengths: radius |N(0, sigma)| of
    the grid extent, clipped to clip_frac of it, uniform angle."""
    extent = 1.0 / cell_size_rad                  # full grid width in lambda
    r = np.abs(rng.normal(0.0, sigma_frac, n)) * extent
    r = np.minimum(r, clip_frac * extent)
    theta = rng.uniform(0.0, 2.0 * math.pi, n)
    return r * np.cos(theta), r * np.sin(theta)


def _finish(name, rng, support, oversample, grid_size, cell_size_rad, uu, vv,
            ww, w_max, weight=None, channel_offsets=None):
    num_w_planes = int(support.shape[0])
    conv_size_half = (int(support.max()) + 1) * oversample
    n = uu.shape[0]
    if weight is None:
        weight = (1.5 - rng.random(n)).astype(np.float32)      # (0.5, 1.5]
    vis = rng.standard_normal((n, 2)).astype(np.float32)
    w_scale = np.float32((num_w_planes - 1) ** 2 / w_max)
    return Workload(
        name=name, num_w_planes=num_w_planes, support=support,
        oversample=oversample, conv_size_half=conv_size_half,
        conv_func=make_kernel_stack(support, oversample, conv_size_half),
        uu=np.ascontiguousarray(uu, dtype=np.float32),
        vv=np.ascontiguousarray(vv, dtype=np.float32),
        ww=np.ascontiguousarray(ww, dtype=np.float32),
        vis=np.ascontiguousarray(vis), weight=np.ascontiguousarray(weight),
        cell_size_rad=float(np.float32(cell_size_rad)),
        w_scale=float(w_scale), grid_size=grid_size,
        channel_offsets=channel_offsets)


def random_uniform_workload(name: str, num_points: int, grid_size: int,
                            num_w_planes: int, s_min: int, s_max: int,
                            oversample: int = 4, seed: int = 0,
                            cell_size_rad: float = 2.0e-5,
                            w_max: float = 5000.0,
                            sigma_frac: float = 0.12,
                            clip_frac: float = 0.45) -> Workload:
    """Configs 0, 1 and 3: radially concentrated uv, uniform w in +-w_max."""
    rng = np.random.Generator(np.random.PCG64(seed))
    support = linear_supports(num_w_planes, s_min, s_max)
    uu, vv = _radial_uv(rng, num_points, grid_size, cell_size_rad,
                        sigma_frac, clip_frac)
    ww = rng.uniform(-w_max, w_max, num_points)
    return _finish(name, rng, support, oversample, grid_size, cell_size_rad,
                   uu, vv, ww, w_max)


def config0(seed: int = 20240) -> Workload:
    """200,000 visibilities, 2048^2 grid, 128 planes, support 4..24, os 4."""
    return random_uniform_workload("cfg0_plain_2048", 200_000, 2048, 128, 4,
                                   24, seed=seed)


def config1(seed: int = 20241) -> Workload:
    """Synthetic-challenge shape: 2,152,800 visibilities, 8192^2 grid,
    714 planes, support 4..36, os 4."""
    return random_uniform_workload("cfg1_synthetic_8192", 2_152_800, 8192,
                                   714, 4, 36, seed=seed)


# --------------------------------------------------------------------------
# SKA-LOW-shaped array (configs 2 and 4)
# --------------------------------------------------------------------------

SKA_LOW_LATITUDE_DEG = -26.82


def ska_low_stations(rng, num_stations=512, median_m=1000.0,
                     frac_within_2km=0.70, max_m=65000.0):
    """Station (east, north) in metres: log-normal radius with the given
    median and P(r < 2 km), truncated at max_m; uniform azimuth."""
    sigma = math.log(2000.0 / median_m) / _norm_ppf(frac_within_2km)
    r = np.empty(0)
    while r.shape[0] < num_stations:
        cand = np.exp(rng.normal(math.log(median_m), sigma, num_stations))
        r = np.concatenate([r, cand[cand <= max_m]])
    r = r[:num_stations]
    az = rng.uniform(0.0, 2.0 * math.pi, num_stations)
    return r * np.sin(az), r * np.cos(az)


def _norm_ppf(p):
    # Inverse of the standard normal CDF by bisection (no scipy dependency).
    lo, hi = -10.0, 10.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if 0.5 * (1.0 + math.erf(mid / math.sqrt(2.0))) < p:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def ska_low_uvw_metres(rng, num_stations=512, num_times=240,
                       track_hours=4.0, dec_deg=-27.0):
    """Baseline (u, v, w) in metres, time-major [t * n_baselines + b], for an
    Earth-rotation track of track_hours centred on transit."""
    e, n = ska_low_stations(rng, num_stations)
    lat = math.radians(SKA_LOW_LATITUDE_DEG)
    # Local (east, north, up=0) -> equatorial (X towards H=0, Y east, Z pole).
    X = -math.sin(lat) * n
    Y = e
    Z = math.cos(lat) * n
    i, j = np.triu_indices(num_stations, k=1)
    bx, by, bz = X[j] - X[i], Y[j] - Y[i], Z[j] - Z[i]
    nb = bx.shape[0]
    dec = math.radians(dec_deg)
    ha = np.linspace(-0.5, 0.5, num_times) * track_hours * (math.pi / 12.0)
    u = np.empty((num_times, nb), dtype=np.float64)
    v = np.empty_like(u)
    w = np.empty_like(u)
    for t, h in enumerate(ha):
        sh, ch = math.sin(h), math.cos(h)
        u[t] = sh * bx + ch * by
        v[t] = -math.sin(dec) * ch * bx + math.sin(dec) * sh * by + \
            math.cos(dec) * bz
        w[t] = math.cos(dec) * ch * bx - math.cos(dec) * sh * by + \
            math.sin(dec) * bz
    return u.reshape(-1), v.reshape(-1), w.reshape(-1)


def _fit_cell_size(u_max_lambda, grid_size, s_max):
    # Longest baseline lands s_max + 2 cells inside the grid edge.
    return float(np.float32(
        (grid_size / 2 - s_max - 2) / (grid_size * u_max_lambda)))


def config2(variant: str = "EL56-82", seed: int = 20242,
            freq_hz: float = 100e6, num_times: int = 240) -> Workload:
    """SKA-LOW-shaped snapshot: 512 stations, 130,816 baselines x 240 times
    = 31,395,840 visibilities on an 8192^2 grid, unit weights.  Variant
    "EL56-82": 601 planes, support 4..72; "EL82-70": 339 planes, 8..44.
    num_times < 240 samples the same 4 h track more coarsely (a smaller
    problem with the same uv density structure)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if variant == "EL56-82":
        planes, s_min, s_max = 601, 4, 72
    elif variant == "EL82-70":
        planes, s_min, s_max = 339, 8, 44
    else:
        raise ValueError(variant)
    grid_size = 8192
    u, v, w = ska_low_uvw_metres(rng, num_times=num_times)
    scale = freq_hz / SPEED_OF_LIGHT
    u *= scale; v *= scale; w *= scale
    u_max = float(max(np.abs(u).max(), np.abs(v).max()))
    cell = _fit_cell_size(u_max, grid_size, s_max)
    w_max = float(np.abs(w).max())
    n = u.shape[0]
    weight = np.ones(n, dtype=np.float32)
    support = linear_supports(planes, s_min, s_max)
    return _finish(f"cfg2_skalow_{variant}", rng, support, 4, grid_size, cell,
                   u, v, w, w_max, weight=weight)


def config4(num_channels: int = 64, seed: int = 20244,
            grid_size: int = 4096, times: int = 240,
            stations: int = 512, threads: int | None = None) -> Workload:
    """Batched multi-channel: the config-2 array at num_channels frequencies
    in 100-200 MHz, each channel with 0-60% of visibilities flagged
    (removed), onto num_channels separate grid_size^2 grids; 339 planes,
    support 8..44, unit weights, complex N(0, 1) amplitudes.  Channels are
    concatenated; channel_offsets[c] is the first visibility of channel c.

    Each channel draws from its own PCG64 stream (spawned from the seed), so
    the channels are generated on `threads` host threads (default: all) and
    the arrays do not depend on the thread count.  At the default size this
    is 64 x 31,395,840 x (0.4..1) ~ 1.4e9 visibilities (about 34 GB)."""
    import concurrent.futures
    import os
    ss = np.random.SeedSequence(seed)
    base_ss, *chan_ss = ss.spawn(1 + num_channels)
    rng = np.random.Generator(np.random.PCG64(base_ss))
    planes, s_min, s_max = 339, 8, 44
    u_m, v_m, w_m = ska_low_uvw_metres(rng, num_stations=stations,
                                       num_times=times)
    freqs = np.linspace(100e6, 200e6, num_channels)
    u_max = float(max(np.abs(u_m).max(), np.abs(v_m).max())) * \
        freqs[-1] / SPEED_OF_LIGHT
    w_max = float(np.abs(w_m).max()) * freqs[-1] / SPEED_OF_LIGHT
    cell = _fit_cell_size(u_max, grid_size, s_max)
    n_base = u_m.shape[0]

    def keep_mask(c):
        r = np.random.Generator(np.random.PCG64(chan_ss[c]))
        keep_frac = 1.0 - r.uniform(0.0, 0.6)
        return r, r.random(n_base, dtype=np.float32) < np.float32(keep_frac)

    workers = threads or min(16, os.cpu_count() or 1)
    with concurrent.futures.ThreadPoolExecutor(workers) as ex:
        counts = list(ex.map(lambda c: int(keep_mask(c)[1].sum()),
                             range(num_channels)))
    offs = np.zeros(num_channels + 1, dtype=np.int64)
    offs[1:] = np.cumsum(counts)
    n = int(offs[-1])
    uu = np.empty(n, np.float32)
    vv = np.empty(n, np.float32)
    ww = np.empty(n, np.float32)
    vis = np.empty((n, 2), np.float32)

    def fill(c):
        r, keep = keep_mask(c)
        a, b = int(offs[c]), int(offs[c + 1])
        sc = freqs[c] / SPEED_OF_LIGHT
        uu[a:b] = u_m[keep] * sc
        vv[a:b] = v_m[keep] * sc
        ww[a:b] = w_m[keep] * sc
        r.standard_normal((b - a, 2), dtype=np.float32, out=vis[a:b])

    with concurrent.futures.ThreadPoolExecutor(workers) as ex:
        list(ex.map(fill, range(num_channels)))
    support = linear_supports(planes, s_min, s_max)
    conv_size_half = (int(support.max()) + 1) * 4
    return Workload(
        name=f"cfg4_batched_{num_channels}x{grid_size}", num_w_planes=planes,
        support=support, oversample=4, conv_size_half=conv_size_half,
        conv_func=make_kernel_stack(support, 4, conv_size_half), uu=uu, vv=vv,
        ww=ww, vis=vis, weight=np.ones(n, dtype=np.float32),
        cell_size_rad=float(np.float32(cell)),
        w_scale=float(np.float32((planes - 1) ** 2 / w_max)),
        grid_size=grid_size, channel_offsets=offs)


WORKLOADS = {
    "cfg0": config0,
    "cfg1": config1,
    "cfg2": config2,
    "cfg2b": lambda: config2("EL82-70"),
    "cfg2s": lambda: config2("EL56-82", num_times=60),
    "cfg4": config4,
    # Config-4 structure at a reduced size: 64 channels (100-200 MHz, 0-60%
    # flagged) of a 128-station array, 120 times.
    "cfg4s": lambda: config4(num_channels=64, grid_size=4096, times=120,
                             stations=128),
}
