"""Host-built tables of the product against the oracle, bit for bit (no GPU)."""
import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from tests.golden.make_golden import F2P_CASES
from tests.helpers import CFG1, ROFEX, SMALL, geom, ns, oracle_gather


def _case(name):
    d = dict(F2P_CASES[name])
    d["n_pixels"] = 64
    return d


@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
@pytest.mark.parametrize("case", ["rofex", "synthetic", "offcentre", "small"])
def test_fan2para_gather_tables_bit_exact(case, quirk):
    d = SMALL if case == "small" else _case(case)
    g = geom(d)
    p = rg.make_params(quirks=quirk)
    rec = oracle.f2p_records(ns(d), quirk)
    for plane in range(d["n_planes"]):
        pk, u, v = rg.fan2para_tables_host(g, p, plane)
        opk, ou, ov = oracle_gather(rec, plane, d["n_par_proj"], d["n_par_det"])
        np.testing.assert_array_equal(pk, opk)
        np.testing.assert_array_equal(u.view(np.uint32), ou.view(np.uint32))
        np.testing.assert_array_equal(v.view(np.uint32), ov.view(np.uint32))
        assert (pk >> 31).sum() > 0


def test_fan2para_tables_rofex_limited_arc():
    # the 240-degree source arc invalidates some rays; both rays remain for most samples
    g = geom(ROFEX)
    pk, _, _ = rg.fan2para_tables_host(g, rg.make_params(quirks=rg.QUIRKS_NONE), 0)
    valid = (pk >> 31).astype(bool)
    assert 0.2 < valid.mean() < 1.0


def test_fan2para_odd_rays_rejected_in_risa_mode():
    g = geom(SMALL, n_par_det=63)
    with pytest.raises(rg.RisaError) as e:
        rg.fan2para_tables_host(g, rg.make_params(quirks=rg.QUIRKS_RISA), 0)
    assert e.value.status == -2
    # the corrected fold handles odd ray counts
    pk, _, _ = rg.fan2para_tables_host(g, rg.make_params(quirks=rg.QUIRKS_NONE), 0)
    assert pk.shape == (4, 64 * 63)


@pytest.mark.parametrize("ftype", list(rg.FILTERS))
@pytest.mark.parametrize("cutoff", [1.0, 0.6])
def test_filter_design_matches_oracle(ftype, cutoff):
    for quirk, dp, pad in [(rg.QUIRKS_RISA, 256, 0), (rg.QUIRKS_NONE, 256, 0), (rg.QUIRKS_NONE, 200, 1024)]:
        g = geom(CFG1, n_par_det=dp)
        p = rg.make_params(quirks=quirk, filter_type=ftype, cutoff=cutoff, pad=pad)
        n, h = rg.filter_design_host(g, p)
        on = oracle.filter_length(dp, pad, quirk)
        assert n == on
        oh = oracle.design_filter(on, rg.FILTERS[ftype], cutoff, quirk).astype(np.float32)
        np.testing.assert_array_equal(h.view(np.uint32), oh.view(np.uint32))


def test_filter_lengths():
    assert rg.filter_design_host(geom(CFG1, n_par_det=1024), rg.make_params())[0] == 2048
    assert rg.filter_design_host(geom(CFG1, n_par_det=256), rg.make_params())[0] == 512
    assert rg.filter_design_host(geom(CFG1, n_par_det=1280), rg.make_params())[0] == 4096
    with pytest.raises(rg.RisaError):
        rg.filter_design_host(geom(CFG1, n_par_det=200), rg.make_params(quirks=rg.QUIRKS_RISA))
