"""Seeded synthetic ROFEX-style scans: ellipse phantoms, analytic line integrals,
Poisson-distributed uint16 detector counts, dark/reference frames and planted
detector defects.

The reference ships no sample data (its config points at empty paths), so every
benchmark and test input is generated here. Geometry conventions follow the
reference's rebinning (Fan2Para.cu:286-309, 366-390):
  * source position j sits at angle theta_j = j*360/Pf - sourceOffset on the
    source ring of radius sourceDiameter/2;
  * fan detector i sits at physical angle gamma_i + 90 degrees,
    gamma_i = i*360/Df, on the detector ring of radius detectorDiameter/2;
  * the parallel ray (alpha, s) is the line {p : p . (sin a, -cos a) = s}, so
    the backprojection's angle theta = alpha - 90 degrees sees
    s = x cos(theta) + y sin(theta);
  * image pixel (x, y) of an N x N image over imageWidth mm sits at
    ((x - (N-1)/2) * W/N, (y - (N-1)/2) * W/N).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Ellipse:
    cx: float
    cy: float
    a: float
    b: float
    phi: float
    mu: float


def random_phantom(seed: int, n: int = 8, fov: float = 200.0, axes=(5.0, 60.0),
                   mu=(0.005, 0.05)) -> list[Ellipse]:
    """n ellipses with seeded centres inside the field of view (diameter fov, mm),
    semi-axes U(axes) mm and attenuation U(mu) /mm; every ellipse lies inside the FOV."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        a, b = rng.uniform(*axes, size=2)
        r_max = max(fov / 2.0 - max(a, b), 0.0)
        rr = r_max * np.sqrt(rng.uniform())
        ang = rng.uniform(0, 2 * np.pi)
        out.append(Ellipse(rr * np.cos(ang), rr * np.sin(ang), a, b, rng.uniform(0, np.pi),
                           rng.uniform(*mu)))
    return out


def segment_integrals(ellipses, p0, p1) -> np.ndarray:
    """Sum over ellipses of mu * (chord length inside the segment p0 -> p1).
    p0, p1: arrays [..., 2] in mm."""
    p0 = np.asarray(p0, np.float64)
    p1 = np.asarray(p1, np.float64)
    d = p1 - p0
    seg_len = np.sqrt((d ** 2).sum(-1))
    out = np.zeros(p0.shape[:-1], np.float64)
    for e in ellipses:
        c, s = np.cos(e.phi), np.sin(e.phi)
        q0x = ((p0[..., 0] - e.cx) * c + (p0[..., 1] - e.cy) * s) / e.a
        q0y = (-(p0[..., 0] - e.cx) * s + (p0[..., 1] - e.cy) * c) / e.b
        dx = (d[..., 0] * c + d[..., 1] * s) / e.a
        dy = (-d[..., 0] * s + d[..., 1] * c) / e.b
        A = dx * dx + dy * dy
        B = q0x * dx + q0y * dy
        C = q0x * q0x + q0y * q0y - 1.0
        disc = B * B - A * C
        ok = disc > 0
        sq = np.sqrt(np.where(ok, disc, 0.0))
        t1 = np.clip((-B - sq) / A, 0.0, 1.0)
        t2 = np.clip((-B + sq) / A, 0.0, 1.0)
        out += np.where(ok, (t2 - t1) * seg_len * e.mu, 0.0)
    return out


def line_integrals_parallel(ellipses, thetas, s) -> np.ndarray:
    """Radon transform on the infinite lines x cos(theta) + y sin(theta) = s.
    thetas [A] rad, s [S] mm -> [A, S]."""
    th = np.asarray(thetas, np.float64)[:, None]
    s = np.asarray(s, np.float64)[None, :]
    out = np.zeros((th.shape[0], s.shape[1]), np.float64)
    for e in ellipses:
        # shift to the ellipse centre, rotate into its frame
        sp = s - (e.cx * np.cos(th) + e.cy * np.sin(th))
        ang = th - e.phi
        a2 = (e.a * np.cos(ang)) ** 2 + (e.b * np.sin(ang)) ** 2
        inside = a2 - sp ** 2
        out += np.where(inside > 0, 2.0 * e.a * e.b * np.sqrt(np.maximum(inside, 0.0)) / a2, 0.0) * e.mu
    return out


def rasterize(ellipses, n_pixels: int, width: float, supersample: int = 4) -> np.ndarray:
    """Attenuation image [N, N] (image[y, x]) in /mm, area-averaged."""
    ss = supersample
    px = width / n_pixels
    off = (np.arange(n_pixels * ss) + 0.5) / ss - 0.5  # pixel-centre coordinates
    coord = (off - (n_pixels - 1) / 2.0) * px
    X, Y = np.meshgrid(coord, coord)
    img = np.zeros_like(X)
    for e in ellipses:
        c, s = np.cos(e.phi), np.sin(e.phi)
        u = ((X - e.cx) * c + (Y - e.cy) * s) / e.a
        v = (-(X - e.cx) * s + (Y - e.cy) * c) / e.b
        img += np.where(u * u + v * v <= 1.0, e.mu, 0.0)
    return img.reshape(n_pixels, ss, n_pixels, ss).mean(axis=(1, 3))


def fan_line_integrals(ellipses, n_fan_proj: int, n_fan_det: int, source_radius: float,
                       detector_radius: float, source_offset_deg: float = 0.0) -> np.ndarray:
    """[Pf, Df] line integrals from source j to detector i (segment integrals)."""
    th = np.deg2rad(np.arange(n_fan_proj) * 360.0 / n_fan_proj - source_offset_deg)
    ga = np.deg2rad(np.arange(n_fan_det) * 360.0 / n_fan_det) + np.pi / 2.0
    S = np.stack([source_radius * np.cos(th), source_radius * np.sin(th)], -1)[:, None, :]
    D = np.stack([detector_radius * np.cos(ga), detector_radius * np.sin(ga)], -1)[None, :, :]
    S, D = np.broadcast_arrays(S, D)
    return segment_integrals(ellipses, S, D)


def counts(line_integrals: np.ndarray, rng, i0: float = 40000.0, dark_level: float = 200.0) -> np.ndarray:
    """Poisson(I0 exp(-integral)) + Poisson(dark), clamped to uint16."""
    lam = i0 * np.exp(-line_integrals)
    v = rng.poisson(lam) + rng.poisson(dark_level, size=lam.shape)
    return np.clip(v, 0, 65535).astype(np.uint16)


def plant_defects(frame: np.ndarray, dead, flicker, rng, dead_value: int = 200) -> np.ndarray:
    """Dead columns read a constant; flickering columns vary by +-50% per projection."""
    out = frame.astype(np.float64)
    for c in dead:
        out[:, c] = dead_value
    for c in flicker:
        out[:, c] *= 1.0 + rng.uniform(-0.5, 0.5, size=out.shape[0])
    return np.clip(np.round(out), 0, 65535).astype(np.uint16)


def choose_defects(n_det: int, fraction: float, seed: int):
    """Seeded defect columns (~fraction of detectors), split into dead and flickering."""
    if fraction <= 0:
        return [], []
    rng = np.random.default_rng(seed)
    n = max(1, int(round(fraction * n_det)))
    cols = rng.choice(n_det, size=n, replace=False)
    kinds = rng.uniform(size=n) < 0.5
    return sorted(int(c) for c, k in zip(cols, kinds) if k), sorted(int(c) for c, k in zip(cols, kinds) if not k)


@dataclass
class Scan:
    raw: np.ndarray        # [n_frames*L, Pf, Df] uint16, frame-major, planes interleaved
    planes: np.ndarray     # [n_frames*L] plane of each frame
    ref: np.ndarray        # [1*L, Pf, Df] uint16 reference (empty scanner) frames
    dark: np.ndarray       # [1*L, Pf, Df] uint16 dark frames
    phantoms: list         # ellipse list per distinct frame
    dead: list
    flicker: list


def make_scan(n_frames: int, n_planes: int, n_fan_proj: int, n_fan_det: int, source_radius: float,
              detector_radius: float, source_offset: float = 0.0, seed: int = 0, n_ellipses: int = 8,
              fov: float = 200.0, i0: float = 40000.0, dark_level: float = 200.0,
              defect_fraction: float = 0.0, distinct: int | None = None) -> Scan:
    """A seeded scan. With `distinct` < n_frames, only that many distinct frames are
    generated per plane and cycled (each distinct frame has its own phantom and noise)."""
    rng = np.random.default_rng(seed)
    dead, flicker = choose_defects(n_fan_det, defect_fraction, seed + 7)
    nd = n_frames if distinct is None else max(1, min(distinct, n_frames))
    pool = []
    phantoms = []
    for j in range(nd):
        ph = random_phantom(seed * 1000 + j, n=n_ellipses, fov=fov)
        phantoms.append(ph)
        li = fan_line_integrals(ph, n_fan_proj, n_fan_det, source_radius, detector_radius, source_offset)
        per_plane = []
        for _ in range(n_planes):
            per_plane.append(plant_defects(counts(li, rng, i0, dark_level), dead, flicker, rng))
        pool.append(per_plane)
    raw = np.empty((n_frames * n_planes, n_fan_proj, n_fan_det), np.uint16)
    planes = np.empty(n_frames * n_planes, np.int32)
    for f in range(n_frames):
        for k in range(n_planes):
            raw[f * n_planes + k] = pool[f % nd][k]
            planes[f * n_planes + k] = k
    zero = np.zeros((n_fan_proj, n_fan_det))
    ref = np.stack([plant_defects(counts(zero, rng, i0, dark_level), dead, flicker, rng)
                    for _ in range(n_planes)])
    dark = np.stack([np.clip(rng.poisson(dark_level, size=(n_fan_proj, n_fan_det)), 0, 65535).astype(np.uint16)
                     for _ in range(n_planes)])
    return Scan(raw=raw, planes=planes, ref=ref, dark=dark, phantoms=phantoms, dead=dead, flicker=flicker)


def parallel_sinograms(n_slices: int, n_par_proj: int, n_par_det: int, width: float, seed: int = 0,
                       n_ellipses: int = 8, bin_centred: bool = True):
    """[n, Pp, Dp] float32 analytic parallel sinograms (angles i*pi/Pp) and their phantoms."""
    th = np.arange(n_par_proj) * np.pi / n_par_proj
    k = np.arange(n_par_det)
    s = (k + (0.5 if bin_centred else 0.0) - n_par_det / 2.0) * width / n_par_det
    out = np.empty((n_slices, n_par_proj, n_par_det), np.float32)
    phs = []
    for i in range(n_slices):
        ph = random_phantom(seed * 1000 + i, n=n_ellipses, fov=width)
        phs.append(ph)
        out[i] = line_integrals_parallel(ph, th, s)
    return out, phs


def sweep_instances(n: int, seed: int = 5, n_min: int = 128, n_max: int = 1024, pp_min: int = 180,
                    pp_max: int = 1440, defect_max: float = 0.02, ref_level: float = 40200.0,
                    dark_level: float = 200.0):
    """Seeded instance list of the uneven sweep: image side log-uniform in
    [n_min, n_max], angles uniform in [pp_min, pp_max], rays = 1.25 x the side
    rounded to a multiple of 32, 0..defect_max defective detector columns, a
    ramp or Hann filter, circular mask. Dicts as risa_gb300.Sweep takes them."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        side = int(round(float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))))
        pp = int(rng.integers(pp_min, pp_max + 1))
        dp = max(32, 32 * int(round(1.25 * side / 32.0)))
        k = int(round(rng.uniform(0.0, defect_max) * dp))
        dmap = np.zeros(dp, np.uint8)
        if k:
            cols = rng.choice(dp, size=k, replace=False)
            dmap[cols] = 1
        out.append(dict(n_pixels=side, n_par_proj=pp, n_par_det=dp,
                        filter_type="ramp" if rng.uniform() < 0.5 else "hanning", cutoff=1.0,
                        rotation_offset=0.0, ref_level=ref_level, dark_level=dark_level, masking=True,
                        masking_value=0.0, defect_map=dmap))
    return out


def sweep_counts(inst: dict, seed: int, width: float = 200.0, i0: float = 40000.0) -> np.ndarray:
    """uint16 parallel-beam counts [Pp][Dp] of one sweep instance: seeded 8-ellipse
    phantom, Poisson(I0 exp(-integral)) + dark, defective columns dead (= dark)
    or flickering (+-50%)."""
    pp, dp = inst["n_par_proj"], inst["n_par_det"]
    rng = np.random.default_rng(seed)
    ph = random_phantom(seed, n=8, fov=width)
    th = np.arange(pp) * np.pi / pp
    s = (np.arange(dp) + 0.5 - dp / 2.0) * width / dp
    raw = counts(line_integrals_parallel(ph, th, s), rng, i0, inst.get("dark_level", 200.0))
    dmap = inst.get("defect_map")
    if dmap is not None:
        for col in np.flatnonzero(dmap):
            if rng.uniform() < 0.5:
                raw[:, col] = int(inst.get("dark_level", 200.0))
            else:
                f = rng.uniform(0.5, 1.5, size=pp)
                raw[:, col] = np.clip(raw[:, col] * f, 0, 65535).astype(np.uint16)
    return raw
