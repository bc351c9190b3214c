"""Shared test helpers: geometries of the benchmark configurations and small
parity cases, and conversions between the product's and the oracle's tables."""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np

import risa_gb300 as rg

# Small geometry in the shape of the "plain single-plane FBP" configuration:
# source ring radius 215 mm, detector ring radius 240 mm, 432 detectors,
# 500 projections, 200 mm field of view.
SMALL = dict(n_planes=1, n_fan_det=432, n_fan_proj=500, n_par_proj=64, n_par_det=64, n_pixels=64,
             source_offset=0.0, detector_diameter=480.0, image_width=200.0, source_diameter=[430.0],
             delta_x=[0.0], delta_z=[1417.0], source_angle=[360.0])

# The reference's example geometry (two tilted planes, limited source arc).
ROFEX = dict(n_planes=2, n_fan_det=432, n_fan_proj=500, n_par_proj=64, n_par_det=64, n_pixels=64,
             source_offset=23.2, detector_diameter=216.0, image_width=190.0, source_diameter=[365.0, 370.0],
             delta_x=[815.0, 815.0], delta_z=[1417.0, 1430.0], source_angle=[240.0, 240.0])

CFG1 = dict(n_planes=1, n_fan_det=432, n_fan_proj=500, n_par_proj=256, n_par_det=256, n_pixels=256,
            source_offset=0.0, detector_diameter=480.0, image_width=200.0, source_diameter=[430.0],
            delta_x=[0.0], delta_z=[1417.0], source_angle=[360.0])

CFG2 = dict(n_planes=2, n_fan_det=1152, n_fan_proj=1000, n_par_proj=1024, n_par_det=1024, n_pixels=512,
            source_offset=0.0, detector_diameter=480.0, image_width=200.0, source_diameter=[430.0, 430.0],
            delta_x=[0.0, 0.0], delta_z=[1417.0, 1430.0], source_angle=[360.0, 360.0])


def geom(d: dict, **over) -> rg.Geometry:
    dd = dict(d)
    dd.update(over)
    return rg.make_geometry(**dd)


def ns(d: dict, **over):
    dd = dict(d)
    dd.update(over)
    dd.setdefault("image_center_x", 0.0)
    dd.setdefault("image_center_y", 0.0)
    dd.setdefault("rotation_offset", 0.0)
    return SimpleNamespace(**dd)


def oracle_gather(rec, plane: int, n_par_proj: int, n_par_det: int):
    """Oracle rebinning records -> the product's per-output gather layout."""
    Pp, Dp = n_par_proj, n_par_det
    valid = rec.valid[plane]
    tb, gb, u, v = rec.tb[plane], rec.gb[plane], rec.u[plane], rec.v[plane]
    packed = np.zeros((4, Pp * Dp), np.uint32)
    uu = np.zeros((4, Pp * Dp), np.float32)
    vv = np.zeros((4, Pp * Dp), np.float32)
    jo = np.repeat(np.arange(Pp), Dp)
    io = np.tile(np.arange(Dp), Pp)
    rows = (jo, jo + Pp)
    cols = (io, Dp - 1 - io)
    for s in range(2):
        for r in range(2):
            slot = 2 * s + r
            vm = valid[rows[s], cols[s], r].astype(bool)
            pk = (np.uint32(1) << np.uint32(31)) | (tb[rows[s], cols[s], r].astype(np.uint32) << np.uint32(16)) \
                | gb[rows[s], cols[s], r].astype(np.uint32)
            packed[slot] = np.where(vm, pk, 0).astype(np.uint32)
            uu[slot] = np.where(vm, u[rows[s], cols[s], r], 0).astype(np.float32)
            vv[slot] = np.where(vm, v[rows[s], cols[s], r], 0).astype(np.float32)
    return packed, uu, vv


def rel_err(got, ref):
    """(max |got - ref| / max |ref|, ||got - ref||_2 / ||ref||_2) in FP64."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    d = got - ref
    mx = np.abs(ref).max()
    return float(np.abs(d).max() / mx if mx else np.abs(d).max()), \
        float(np.linalg.norm(d) / max(np.linalg.norm(ref), 1e-300))
