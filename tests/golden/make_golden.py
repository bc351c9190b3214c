"""Generate the golden fixtures in this directory by running the reference's own
host-side code (compiled from the reference tree by oracle/ref_harness/build_ref.sh).

The reference ships no golden vectors, no tests and no sample data, so these
fixtures are made here: seeded inputs are fed to the reference's functions and
their exact outputs are stored. They pin the oracle (tests/test_oracle_golden.py).

    python tests/golden/make_golden.py            # needs the reference checkout

Reference functions exercised (paths within the reference project):
  Fan2Para::computeFan2ParaTransp / computeAngles   RISA/risaLib/src/Fan2Para/Fan2Para.cu:251-480
  findDefectDetectors / interpolateDefectDetectors  RISA/risaLib/src/DetectorInterpolation/interpolationFunctions.h:28-97
  Attenuation::computeAverage / computeDarkAverage  RISA/risaLib/src/Attenuation/Attenuation.cu:219-251
  Attenuation::relevantAreaMask                     RISA/risaLib/src/Attenuation/Attenuation.cu:327-381
  Filter::designFilter                              RISA/risaLib/src/Filter/Filter.cu:169-191
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "librisa_ref_host.so")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Geometries for the table fixtures. "rofex" is the reference's example
# configuration (RISA/example/config.cfg:29-45) at reduced parallel sampling.
F2P_CASES = {
    "rofex": dict(n_planes=2, n_fan_det=432, n_fan_proj=500, n_par_proj=32, n_par_det=48,
                  source_offset=23.2, detector_diameter=216.0, image_center_x=0.0,
                  image_center_y=0.0, image_width=190.0, source_diameter=[365.0, 370.0],
                  delta_x=[815.0, 815.0], delta_z=[1417.0, 1430.0], source_angle=[240.0, 240.0]),
    "synthetic": dict(n_planes=1, n_fan_det=432, n_fan_proj=500, n_par_proj=32, n_par_det=64,
                      source_offset=0.0, detector_diameter=480.0, image_center_x=0.0,
                      image_center_y=0.0, image_width=200.0, source_diameter=[430.0],
                      delta_x=[0.0], delta_z=[1417.0], source_angle=[360.0]),
    "offcentre": dict(n_planes=1, n_fan_det=96, n_fan_proj=120, n_par_proj=24, n_par_det=40,
                      source_offset=-10.5, detector_diameter=216.0, image_center_x=3.5,
                      image_center_y=-2.25, image_width=150.0, source_diameter=[365.0],
                      delta_x=[815.0], delta_z=[1417.0], source_angle=[300.0]),
}


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def load_ref():
    if not os.path.exists(REF_LIB):
        subprocess.check_call([os.path.join(ROOT, "oracle", "ref_harness", "build_ref.sh")])
    lib = ctypes.CDLL(REF_LIB)
    i, f, d, vp, u = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p, ctypes.c_uint
    lib.risa_ref_fan2para_tables.argtypes = [i] * 5 + [f] * 5 + [vp] * 10
    lib.risa_ref_relevant_area_mask.argtypes = [i, i, d, d, d] + [u] * 6 + [vp]
    lib.risa_ref_reference_average.argtypes = [vp, i, i, i, i, vp]
    lib.risa_ref_dark_average.argtypes = [vp, i, i, i, i, vp]
    lib.risa_ref_find_defects.argtypes = [vp, i, i, d, d, vp]
    lib.risa_ref_interpolate_defects.argtypes = [vp, vp, i, i]
    lib.risa_ref_design_filter.argtypes = [i, i, f, vp]
    return lib


def make_f2p(lib, out):
    for name, g in F2P_CASES.items():
        L, Pf, Df, Pp2, Dp = g["n_planes"], g["n_fan_proj"], g["n_fan_det"], 2 * g["n_par_proj"], g["n_par_det"]
        n = L * Pp2 * Dp
        theta = np.zeros(Pf, np.float32); gamma = np.zeros(Df, np.float32)
        s = np.zeros(Dp, np.float32); alpha = np.zeros(Pp2, np.float32)
        itab = np.zeros(10 * n, np.int32); ftab = np.zeros(4 * n, np.float32)
        arr = lambda key: np.array(g[key], np.float32)
        sd, dx, dz, sa = arr("source_diameter"), arr("delta_x"), arr("delta_z"), arr("source_angle")
        rc = lib.risa_ref_fan2para_tables(L, Df, Pf, g["n_par_proj"], Dp, g["source_offset"],
                                          g["detector_diameter"], g["image_center_x"],
                                          g["image_center_y"], g["image_width"], _p(sd), _p(dx),
                                          _p(dz), _p(sa), _p(theta), _p(gamma), _p(s), _p(alpha),
                                          _p(itab), _p(ftab))
        assert rc == 0
        np.savez_compressed(os.path.join(out, f"f2p_{name}.npz"), theta=theta, gamma=gamma, s=s,
                            alpha=alpha, itab=itab.reshape(10, n), ftab=ftab.reshape(4, n))


def planted_frame(rng, P, D, dead, flicker, base=30000):
    """A smooth u16 frame with planted dead (constant) and flickering columns."""
    x = np.arange(D)[None, :]
    y = np.arange(P)[:, None]
    f = base + 4000 * np.sin(2 * np.pi * x / D * 3 + y / P * 2.0) + rng.normal(0, 30, (P, D))
    f = np.clip(f, 0, 65535)
    for c in dead:
        f[:, c] = 1234.0
    for c in flicker:
        f[:, c] *= 1.0 + rng.uniform(-0.5, 0.5, P)
    return np.clip(np.round(f), 0, 65535).astype(np.uint16)


DEFECT_CASES = {
    # D, P, dead columns, flickering columns, thresh_min, thresh_max
    "mid": (432, 40, [17, 18, 19, 200, 300], [100, 250], 0.67, 1.5),
    "wrap": (432, 30, [0, 1, 431, 215, 216], [3], 0.67, 1.5),
    "all_edges": (96, 24, [0, 95, 47, 48], [94, 1], 0.33, 2.0),
    "clean": (96, 16, [], [], 0.67, 1.5),
}


def make_defects(lib, out):
    rng = np.random.default_rng(1234)
    data = {}
    for name, (D, P, dead, flick, tmin, tmax) in DEFECT_CASES.items():
        frame = planted_frame(rng, P, D, dead, flick)
        flags = np.zeros(D + 1, np.int32)
        assert lib.risa_ref_find_defects(_p(frame), D, P, tmin, tmax, _p(flags)) == 0
        repaired = frame.copy()
        assert lib.risa_ref_interpolate_defects(_p(repaired), _p(flags), D, P) == 0
        # interpolation with hand-made flags, including a run through column 0
        hand = np.zeros(D + 1, np.int32)
        for c in (0, 1, 2, D - 1, D // 2, D // 2 + 1):
            hand[c] = 1
        hand_out = frame.copy()
        assert lib.risa_ref_interpolate_defects(_p(hand_out), _p(hand), D, P) == 0
        data[f"{name}_frame"] = frame
        data[f"{name}_flags"] = flags
        data[f"{name}_repaired"] = repaired
        data[f"{name}_hand_flags"] = hand
        data[f"{name}_hand_out"] = hand_out
        data[f"{name}_thresh"] = np.array([tmin, tmax])
    np.savez_compressed(os.path.join(out, "defects.npz"), **data)


def make_averages(lib, out):
    rng = np.random.default_rng(99)
    n_frames, L, P, D = 3, 2, 20, 48
    vals = rng.integers(100, 60000, size=(n_frames * L, P, D), dtype=np.uint16)
    avg = np.zeros(L * P * D, np.float32)
    dark = np.zeros(L * D, np.float32)
    assert lib.risa_ref_reference_average(_p(vals), n_frames, L, D, P, _p(avg)) == 0
    assert lib.risa_ref_dark_average(_p(vals), n_frames, L, D, P, _p(dark)) == 0
    np.savez_compressed(os.path.join(out, "averages.npz"), values=vals, n_frames=n_frames,
                        n_planes=L, avg=avg.reshape(L, P, D), dark=dark.reshape(L, D))


def make_mask(lib, out):
    # RISA/example/config.cfg:36,63-70 with 500 projections x 432 detectors
    P, D = 500, 432
    mask = np.zeros(P * D, np.float32)
    assert lib.risa_ref_relevant_area_mask(D, P, 23.2, 47.0, 313.0, 43, 285, 175, 362, 0, 431, _p(mask)) == 0
    np.savez_compressed(os.path.join(out, "relevant_mask.npz"), mask=mask.reshape(P, D).astype(np.uint8),
                        params=np.array([D, P, 23.2, 47.0, 313.0, 43, 285, 175, 362, 0, 431]))


def make_filters(lib, out):
    data = {}
    for dp in (64, 256, 1024, 2048):
        for t in range(5):
            for cutoff in (1.0, 0.75):
                h = np.zeros(dp // 2 + 1, np.float32)
                assert lib.risa_ref_design_filter(dp, t, cutoff, _p(h)) == 0
                data[f"h_{dp}_{t}_{cutoff}"] = h
    np.savez_compressed(os.path.join(out, "filters.npz"), **data)


def main():
    import oracle

    if not os.path.isdir(oracle.reference_root()):
        print("make_golden: the reference checkout is not available; nothing to do")
        return 0
    lib = load_ref()
    make_f2p(lib, HERE)
    make_defects(lib, HERE)
    make_averages(lib, HERE)
    make_mask(lib, HERE)
    make_filters(lib, HERE)
    print("make_golden: fixtures written to", HERE)
    return 0


if __name__ == "__main__":
    sys.exit(main())
