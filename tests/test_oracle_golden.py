"""Pin the CPU oracle to fixtures produced by the reference's own host code.

Every comparison here is bit-exact: index tables, flags, u16 frames and the
float tables the reference stores (tests/golden/make_golden.py made them).
"""
import os

import numpy as np
import pytest

import oracle
from tests.golden.make_golden import DEFECT_CASES, F2P_CASES


class G:
    def __init__(self, d):
        self.__dict__.update(d)
        self.n_pixels = 64
        self.rotation_offset = 0.0


@pytest.mark.parametrize("name", sorted(F2P_CASES))
def test_f2p_tables_match_reference(golden_dir, name):
    ref = np.load(os.path.join(golden_dir, f"f2p_{name}.npz"))
    got = oracle.f2p_tables_risa(G(F2P_CASES[name]))
    for key in ("theta", "gamma", "s", "alpha"):
        np.testing.assert_array_equal(got[key].view(np.uint32), ref[key].view(np.uint32), err_msg=key)
    np.testing.assert_array_equal(got["itab"], ref["itab"])
    np.testing.assert_array_equal(got["ftab"].view(np.uint32), ref["ftab"].view(np.uint32))
    # the reference's quirk: alpha[0] stays 0 instead of pi/2
    assert got["alpha"][0] == 0.0


@pytest.mark.parametrize("name", sorted(DEFECT_CASES))
def test_defects_match_reference(golden_dir, name):
    d = np.load(os.path.join(golden_dir, "defects.npz"))
    frame = d[f"{name}_frame"]
    tmin, tmax = d[f"{name}_thresh"]
    flags = oracle.find_defects(frame, tmin, tmax, oracle.QUIRK_RISA)
    np.testing.assert_array_equal(flags, d[f"{name}_flags"])
    rep = oracle.interpolate_defects(frame, flags, oracle.QUIRK_RISA)
    np.testing.assert_array_equal(rep, d[f"{name}_repaired"])
    hand = oracle.interpolate_defects(frame, d[f"{name}_hand_flags"], oracle.QUIRK_RISA)
    np.testing.assert_array_equal(hand, d[f"{name}_hand_out"])


def test_planted_defects_are_found(golden_dir):
    d = np.load(os.path.join(golden_dir, "defects.npz"))
    D, P, dead, flick, _, _ = DEFECT_CASES["mid"]
    flags = d["mid_flags"][:D]
    for c in dead + flick:
        assert flags[c] == 1


def test_averages_match_reference(golden_dir):
    a = np.load(os.path.join(golden_dir, "averages.npz"))
    n, L = int(a["n_frames"]), int(a["n_planes"])
    avg = oracle.reference_average(a["values"], n, L, oracle.QUIRK_RISA)
    np.testing.assert_array_equal(avg.view(np.uint32), a["avg"].view(np.uint32))
    dark = oracle.dark_average(a["values"], n, L, oracle.QUIRK_RISA)
    np.testing.assert_array_equal(dark.view(np.uint32), a["dark"].view(np.uint32))


def test_relevant_mask_matches_reference(golden_dir):
    m = np.load(os.path.join(golden_dir, "relevant_mask.npz"))
    D, P, so, lo, up, xa, xb, xc, xd, xe, xf = m["params"]
    got = oracle.relevant_area_mask(int(D), int(P), so, lo, up, int(xa), int(xb), int(xc), int(xd),
                                    int(xe), int(xf))
    np.testing.assert_array_equal(got.astype(np.uint8), m["mask"])
    assert 0 < m["mask"].mean() < 1


def test_filters_match_reference(golden_dir):
    f = np.load(os.path.join(golden_dir, "filters.npz"))
    for key in f.files:
        _, dp, t, cutoff = key.split("_")
        got = oracle.design_filter(int(dp), int(t), float(cutoff), oracle.QUIRK_RISA)
        np.testing.assert_array_equal(got.astype(np.float32).view(np.uint32), f[key].view(np.uint32),
                                      err_msg=key)
        assert np.all(got == got.astype(np.float32))
