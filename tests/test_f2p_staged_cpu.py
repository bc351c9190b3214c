"""The batched engine's staged rebinning tables, host side (no GPU): every
valid output's four bilinear taps, followed through its tile's staged boxes
the way the kernel stages them (entry -> box row and column -> fan row and
column, both circular), land on the fan samples of the gather table; every
tile's boxes fit the stage; a tile marked mirrored (boxes (0, 0, 0, -1) for
slots 2 and 3, staged and blended with two slots) has slots 2 and 3 equal to
slots 1 and 0 bit for bit in every output; geometries whose boxes are too
large are left to the global-memory gather."""
import numpy as np
import pytest

import risa_gb300 as rg
from tests.helpers import SMALL, geom


def pitch_of(nc):
    nc = np.asarray(nc)
    return np.where(nc <= 0, 0, nc + ((12 - (nc & 7)) & 7))


def check_staged(g, p):
    L, Pf, Df, Pp, Dp = g.n_planes, g.n_fan_proj, g.n_fan_det, g.n_par_proj, g.n_par_det
    boxes, rel, se = rg.fan2para_staged_tables_host(g, p)
    assert 0 < se <= 1024
    tiles_s = (Dp + 31) // 32
    th, sr = np.divmod(np.arange(Pp * Dp), Dp)
    tile = (th // 8) * tiles_s + sr // 32
    pitches = pitch_of(boxes[..., 3])                                       # [L, tiles, 4]
    base = np.concatenate([np.zeros(boxes.shape[:2] + (1,), np.int64),
                           np.cumsum(boxes[..., 2] * pitches, axis=2)], axis=2)  # [L, tiles, 5]
    assert (base[..., 4] <= se).all()
    mirror = (boxes[:, :, 2, 3] < 0) & (boxes[:, :, 3, 3] < 0)                 # [L, tiles]
    assert ((boxes[:, :, 2:, 3] < 0) == mirror[..., None]).all()
    checked = 0
    for k in range(L):
        pk, uu, vv = rg.fan2para_tables_host(g, p, k)
        mo = mirror[k][tile]  # outputs of mirrored tiles
        for s in (0, 1):
            assert np.array_equal(pk[3 - s][mo], pk[s][mo])
            assert np.array_equal(uu[3 - s][mo].view(np.uint32), uu[s][mo].view(np.uint32))
            assert np.array_equal(vv[3 - s][mo].view(np.uint32), vv[s][mo].view(np.uint32))
        for s in range(4):
            valid = (pk[s] >> 31).astype(bool)
            if s >= 2:
                assert (rel[k, s][mo] == 0).all()
                valid = valid & ~mo
            assert np.array_equal(valid, (rel[k, s] >> 31).astype(bool))
            o = np.flatnonzero(valid)
            tb = ((pk[s][o] >> 16) & 0x7FFF).astype(np.int64)
            gb = (pk[s][o] & 0xFFFF).astype(np.int64)
            ta, ga = (tb + 1) % Pf, (gb + 1) % Df
            r = rel[k, s][o]
            off, pitch = (r & 0xFFFF).astype(np.int64), ((r >> 20) & 0xFF).astype(np.int64)
            t = tile[o]
            box = boxes[k, t, s].astype(np.int64)
            assert np.array_equal(pitch, pitch_of(box[:, 3]))
            b0, b1 = base[k, t, s], base[k, t, s + 1]
            for e, want_r, want_c in ((off, tb, gb), (off + 1, tb, ga), (off + pitch, ta, gb),
                                      (off + pitch + 1, ta, ga)):
                assert ((e >= b0) & (e < b1)).all()
                row, col = np.divmod(e - b0, pitch)
                assert (row < box[:, 2]).all() and (col < box[:, 3]).all()
                assert np.array_equal((box[:, 0] + row) % Pf, want_r)
                assert np.array_equal((box[:, 1] + col) % Df, want_c)
                checked += len(o)
    return checked


@pytest.mark.parametrize("Pp,Dp,L", [(404, 344, 2), (512, 512, 1)])
def test_staged_boxes_cover_every_tap(Pp, Dp, L):
    d = dict(SMALL, n_planes=L, source_diameter=[430.0] * L, delta_x=[0.0] * L,
             delta_z=[1417.0 + 13 * k for k in range(L)], source_angle=[360.0] * L,
             n_par_proj=Pp, n_par_det=Dp, n_pixels=128)
    assert check_staged(geom(d), rg.make_params()) > 0


def test_staged_full_circle_boxes():
    """A fan of 12 projections x 16 detectors: a tile's taps wrap the whole
    ring, so the box holds one extra row or column for the +1 taps."""
    d = dict(SMALL, n_fan_proj=12, n_fan_det=16, n_par_proj=16, n_par_det=32, n_pixels=16)
    assert check_staged(geom(d), rg.make_params()) > 0


def test_full_circle_tiles_are_mirrored():
    """The full-rate streaming geometry (NONE mode): nearly every tile is
    mirrored, RISA mode's reference steps break the symmetry."""
    from tests.helpers import CFG2

    none_boxes, _, se = rg.fan2para_staged_tables_host(geom(CFG2), rg.make_params())
    assert se > 0 and (none_boxes[:, :, 2, 3] < 0).mean() > 0.99
    risa_boxes, _, _ = rg.fan2para_staged_tables_host(geom(CFG2), rg.make_params(quirks=rg.QUIRKS_RISA))
    assert (risa_boxes[:, :, 2, 3] < 0).mean() < 0.5


def test_coarse_sampling_is_not_staged():
    _, _, se = rg.fan2para_staged_tables_host(geom(dict(SMALL)), rg.make_params())
    assert se == 0
