"""GPU parity: every stage through the C ABI against the CPU oracle.

Index work (defect flags, repaired uint16 frames, averaged tables) must match
bit for bit. FP32 outputs are compared with
    max_rel = max|gpu - oracle| / max|oracle|      (<= 1e-5, the FP32 bar)
    rel_l2  = ||gpu - oracle||_2 / ||oracle||_2
against the FP64 oracle run on the same inputs.
"""
import os

import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from risa_gb300 import phantom
from tests.helpers import ROFEX, SMALL, geom, ns, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_REL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


# ------------------------------------------------------------------------------ defects
@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
def test_defects_bit_exact(golden_dir, quirk):
    d = np.load(os.path.join(golden_dir, "defects.npz"))
    for name in ("mid", "wrap", "all_edges", "clean"):
        frame = d[f"{name}_frame"]
        P, D = frame.shape
        tmin, tmax = d[f"{name}_thresh"]
        g = rg.make_geometry(n_fan_det=D, n_fan_proj=P)
        p = rg.make_params(quirks=quirk, thresh_min=tmin, thresh_max=tmax)
        h = rg.Defects(g, p, max_batch=3)
        frames = np.stack([frame, frame[::-1].copy(), frame])
        t = dev(frames.view(np.int16))
        ws = torch.empty(h.workspace_bytes(3), dtype=torch.uint8, device="cuda")
        flags = torch.zeros((3, D), dtype=torch.int32, device="cuda")
        h.enqueue(t, 3, ws, flags_out=flags)
        got = host(t).view(np.uint16)
        gf = host(flags)
        for b in range(3):
            of = oracle.find_defects(frames[b], tmin, tmax, quirk)
            np.testing.assert_array_equal(gf[b], of[:D], err_msg=f"{name} flags {b}")
            np.testing.assert_array_equal(got[b], oracle.interpolate_defects(frames[b], of, quirk),
                                          err_msg=f"{name} frame {b}")
        if quirk == rg.QUIRKS_RISA:  # and against the reference's own output
            np.testing.assert_array_equal(got[0], d[f"{name}_repaired"])


def _column_var_and_threshold(frame, quirk):
    """The reference's per-column variance and 17-tap threshold in FP64, in its
    operation order (interpolationFunctions.h:36-57), separate roundings."""
    x = frame.astype(np.int64)
    P, D = x.shape
    tv = np.abs(np.diff(x, axis=0)).sum(axis=0)
    rng = x[:-1].max(axis=0) - x[:-1].min(axis=0)
    var = [float(np.float64(tv[d]) * np.float64(rng[d] * rng[d])) for d in range(D)]
    raw = [0.5, 1.0, 1.0, 1.0, 1.5, 2.0, 3.0, 3.5, 2.0, 3.5, 3.0, 2.0, 1.5, 1.0, 1.0, 1.0, 0.5]
    tot = 0.0
    for r in raw:
        tot += r
    inv = 1.0 / tot
    f = [inv * raw[j] for j in range(9)]
    H = D // 2
    th = np.zeros(D)
    for t in range(2 * H):
        seg, i = divmod(t, H)
        acc = 0.0
        for j in range(9):
            i1 = ((i - j) & 0xFFFFFFFF) % H if quirk == rg.QUIRKS_RISA else (i - j) % H
            acc = acc + f[j] * var[i1 + seg * H]
            acc = acc + f[j] * var[(i + j) % H + seg * H]
        th[seg * H + i] = acc
    return np.array(var), th


@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
def test_defect_thresholds_on_the_boundary(golden_dir, quirk):
    """Thresholds set to var/th of chosen columns put those columns on the
    comparison's boundary, where the FP32 screen of the flagging kernel cannot
    decide and the FP64 sequence must; flags match the oracle bit for bit."""
    frame = np.load(os.path.join(golden_dir, "defects.npz"))["mid_frame"]
    P, D = frame.shape
    var, th = _column_var_and_threshold(frame, quirk)
    cols = [d for d in range(0, D, 37) if var[d] > 0 and th[d] > 0][:6]
    assert len(cols) >= 4
    g = rg.make_geometry(n_fan_det=D, n_fan_proj=P)
    t = dev(np.stack([frame] * 2).view(np.int16))
    for d in cols:
        ratio = var[d] / th[d]
        for tmin, tmax in ((ratio, 1e30), (1e-30, ratio), (np.nextafter(ratio, 0), np.nextafter(ratio, 2 * ratio))):
            h = rg.Defects(g, rg.make_params(quirks=quirk, thresh_min=tmin, thresh_max=tmax), max_batch=2)
            ws = torch.empty(h.workspace_bytes(2), dtype=torch.uint8, device="cuda")
            flags = torch.zeros((2, D), dtype=torch.int32, device="cuda")
            h.enqueue(t.clone(), 2, ws, flags_out=flags)
            exp = oracle.find_defects(frame, tmin, tmax, quirk)[:D]
            got = host(flags)
            np.testing.assert_array_equal(got[0], exp, err_msg=f"column {d}, thresholds {tmin!r}, {tmax!r}")
            np.testing.assert_array_equal(got[1], exp)


def test_defects_on_scan_frames():
    sc = phantom.make_scan(2, 1, 200, 432, 215.0, 240.0, seed=3, defect_fraction=0.02, distinct=2)
    g = rg.make_geometry(n_fan_det=432, n_fan_proj=200)
    for quirk in (rg.QUIRKS_RISA, rg.QUIRKS_NONE):
        h = rg.Defects(g, rg.make_params(quirks=quirk), max_batch=2)
        t = dev(sc.raw.view(np.int16))
        ws = torch.empty(h.workspace_bytes(2), dtype=torch.uint8, device="cuda")
        h.enqueue(t, 2, ws)
        got = host(t).view(np.uint16)
        for b in range(2):
            of = oracle.find_defects(sc.raw[b], 0.67, 1.5, quirk)
            assert of[sc.dead].all()
            np.testing.assert_array_equal(got[b], oracle.interpolate_defects(sc.raw[b], of, quirk))


# ------------------------------------------------------------------------------ attenuation
@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
def test_attenuation(quirk):
    d = dict(SMALL, n_planes=2, source_diameter=[430.0, 430.0], delta_x=[0, 0], delta_z=[1417, 1430],
             source_angle=[360, 360])
    sc = phantom.make_scan(3, 2, 500, 432, 215.0, 240.0, seed=5, defect_fraction=0.01, distinct=3)
    g = geom(d)
    p = rg.make_params(quirks=quirk)
    att = rg.Attenuation(g, p, sc.ref, 1, sc.dark, 1)
    ref_t, dark_t = att.tables()
    oref, odark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, quirk)
    np.testing.assert_array_equal(ref_t.view(np.uint32), oref.view(np.uint32))
    np.testing.assert_array_equal(dark_t.view(np.uint32), odark.view(np.uint32))
    raw = dev(sc.raw.view(np.int16))
    out = torch.empty(sc.raw.shape, dtype=torch.float32, device="cuda")
    att.enqueue(raw, out, rg.PLANES_INTERLEAVED, sc.raw.shape[0])
    got = host(out)
    for b in range(sc.raw.shape[0]):
        k = b % 2
        exp = oracle.attenuation(sc.raw[b], oref[k], odark[k])
        mr, _ = rel_err(got[b], exp)
        assert mr < MAX_REL, (b, mr)


def test_attenuation_relevant_mask():
    g = geom(ROFEX)
    p = rg.make_params(quirks=rg.QUIRKS_RISA, relevant_mask=True, lower_lim_offset=47.0,
                       upper_lim_offset=313.0, fix_points=(43, 285, 175, 362, 0, 431))
    rng = np.random.default_rng(0)
    ref = rng.integers(30000, 40000, size=(2, 500, 432)).astype(np.uint16)
    raw = rng.integers(1000, 30000, size=(2, 500, 432)).astype(np.uint16)
    att = rg.Attenuation(g, p, ref, 1, None, 0)
    oref, odark = oracle.attenuation_init(ref, None, 2, 0.67, 1.5, True, rg.QUIRKS_RISA)
    mask = oracle.relevant_area_mask(432, 500, 23.2, 47.0, 313.0, 43, 285, 175, 362, 0, 431)
    out = torch.empty((2, 500, 432), dtype=torch.float32, device="cuda")
    att.enqueue(dev(raw.view(np.int16)), out, 1, 2)
    got = host(out)
    for b in range(2):
        exp = oracle.attenuation(raw[b], oref[1], odark[1], mask)
        assert np.all(got[b][mask == 0] == 0)
        assert rel_err(got[b], exp)[0] < MAX_REL


# ------------------------------------------------------------------------------ fan2para
@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
@pytest.mark.parametrize("gname", ["small", "rofex"])
def test_fan2para(quirk, gname):
    d = SMALL if gname == "small" else ROFEX
    g = geom(d)
    f2p = rg.Fan2Para(g, rg.make_params(quirks=quirk))
    rec = oracle.f2p_records(ns(d), quirk)
    L = d["n_planes"]
    B = 5
    rng = np.random.default_rng(1)
    fan = rng.standard_normal((B, d["n_fan_proj"], d["n_fan_det"])).astype(np.float32)
    par = torch.empty((B, d["n_par_proj"], d["n_par_det"]), dtype=torch.float32, device="cuda")
    for plane in ([rg.PLANES_INTERLEAVED] if L > 1 else []) + list(range(L)):
        f2p.enqueue(dev(fan), par, plane, B)
        got = host(par)
        for b in range(B):
            k = plane if plane >= 0 else b % L
            exp = oracle.f2p_apply(rec, k, quirk, fan[b])
            mr, _ = rel_err(got[b], exp)
            assert mr < MAX_REL, (plane, b, mr)


# ------------------------------------------------------------------------------ filter
@pytest.mark.parametrize("dp,pad,quirk,ftype", [
    (64, 0, rg.QUIRKS_RISA, "ramp"), (256, 0, rg.QUIRKS_NONE, "sheppLogan"),
    (1024, 0, rg.QUIRKS_NONE, "sheppLogan"), (160, 0, rg.QUIRKS_NONE, "hanning"),
    (1024, 0, rg.QUIRKS_RISA, "hamming"), (768, 0, rg.QUIRKS_NONE, "ramp"),
    (2048, 0, rg.QUIRKS_NONE, "cosine"), (4000, 0, rg.QUIRKS_NONE, "ramp")])
def test_filter(dp, pad, quirk, ftype):
    rows = 37
    g = rg.make_geometry(n_par_proj=rows, n_par_det=dp, n_pixels=64)
    p = rg.make_params(quirks=quirk, filter_type=ftype, pad=pad, cutoff=0.9)
    filt = rg.Filter(g, p)
    n, h = filt.response()
    rng = np.random.default_rng(dp)
    x = np.abs(rng.standard_normal((2, rows, dp))).astype(np.float32)
    t = dev(x)
    filt.enqueue(t, 2)
    got = host(t)
    ho = oracle.design_filter(n, rg.FILTERS[ftype], 0.9, quirk)
    for b in range(2):
        exp = oracle.filter_rows(x[b], n, ho)
        mr, l2 = rel_err(got[b], exp)
        assert mr < MAX_REL, (b, mr)


# ------------------------------------------------------------------------------ backprojection
@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
@pytest.mark.parametrize("interp", [rg.INTERP_LINEAR, rg.INTERP_NEAREST, rg.INTERP_NEAREST_TRUNC])
def test_backprojection(quirk, interp):
    Pp, Dp, N = 90, 128, 96
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N, rotation_offset=-7.5)
    p = rg.make_params(quirks=quirk, interp=interp)
    bp = rg.Backprojection(g, p)
    bp.reserve(4)  # pair buffer, so the staged variants run as themselves
    sino, _ = phantom.parallel_sinograms(2, Pp, Dp, 200.0, seed=4)
    img = torch.empty((2, N, N), dtype=torch.float32, device="cuda")
    for v in range(rg.Backprojection.variant_count()):
        bp.set_variant(v)
        bp.enqueue(dev(sino), img, 2)
        got = host(img)
        for b in range(2):
            exp = oracle.backproject(sino[b], N, -7.5, interp, quirk)
            mr, _ = rel_err(got[b], exp)
            tol = MAX_REL if interp == rg.INTERP_LINEAR else 2e-3  # nearest: exact .5 ties may round apart
            assert mr < tol, (v, b, mr)
    bp.check()


def test_backprojection_masking_and_autotune():
    Pp, Dp, N = 128, 160, 128
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N)
    p = rg.make_params(masking=True, masking_value=-1.0)
    bp = rg.Backprojection(g, p)
    bp.reserve(4)  # pair buffer, so the staged variants run as themselves
    sino, _ = phantom.parallel_sinograms(3, Pp, Dp, 200.0, seed=9)
    img = torch.empty((3, N, N), dtype=torch.float32, device="cuda")
    exps = [oracle.mask(oracle.backproject(sino[b], N), -1.0) for b in range(3)]
    yy, xx = np.mgrid[:N, :N]
    out = (xx - (N - 1) / 2) ** 2 + (yy - (N - 1) / 2) ** 2 > N * N / 4
    # every variant with the fused mask (tiles outside the circle skipped)
    for v in list(range(rg.Backprojection.variant_count())) + ["autotuned"]:
        if v == "autotuned":
            assert 0 <= bp.autotune(dev(sino), img, 3) < rg.Backprojection.variant_count()
        else:
            bp.set_variant(v)
        img.fill_(np.nan)
        bp.enqueue(dev(sino), img, 3)
        got = host(img)
        bp.check()
        for b in range(3):
            assert rel_err(got[b], exps[b])[0] < MAX_REL, (v, b)
            assert np.all(got[b][out] == -1.0), (v, b)


def test_masking_normalisation():
    N = 64
    g = rg.make_geometry(n_pixels=N, n_par_proj=8, n_par_det=8)
    m = rg.Masking(g, rg.make_params(masking=True, normalize=True, masking_value=0.5))
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, N, N)).astype(np.float32)
    t = dev(x)
    ws = torch.empty(m.workspace_bytes(2), dtype=torch.uint8, device="cuda")
    m.enqueue(t, 2, ws)
    got = host(t)
    for b in range(2):
        assert rel_err(got[b], oracle.mask(x[b], 0.5, True))[0] < 1e-6


# ------------------------------------------------------------------------------ whole chain
def _fbp_case(quirk, defects, masking, L=1, frames=3):
    # the reference's unpadded filter needs a power-of-two ray count
    dp = 128 if quirk == rg.QUIRKS_RISA else 96
    d = dict(SMALL, n_planes=L, source_diameter=[430.0] * L, delta_x=[0.0] * L,
             delta_z=[1417.0 + 13 * k for k in range(L)], source_angle=[360.0] * L,
             n_par_proj=96, n_par_det=dp, n_pixels=96)
    sc = phantom.make_scan(frames, L, 500, 432, 215.0, 240.0, seed=11, defect_fraction=0.01 if defects else 0,
                           distinct=frames)
    ftype = "sheppLogan"
    g = geom(d)
    p = rg.make_params(quirks=quirk, filter_type=ftype, defects=defects, masking=masking)
    op = oracle.make_params(quirk=quirk, filter_type=ftype, defects=defects, masking=masking)
    return d, sc, g, p, op


@pytest.mark.parametrize("quirk", [rg.QUIRKS_NONE, rg.QUIRKS_RISA])
@pytest.mark.parametrize("defects", [False, True])
def test_fbp_chain_vs_oracle(quirk, defects):
    d, sc, g, p, op = _fbp_case(quirk, defects, masking=True, L=2)
    n = sc.raw.shape[0]
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    img = torch.empty((n, d["n_pixels"], d["n_pixels"]), dtype=torch.float32, device="cuda")
    fbp.enqueue(dev(sc.raw.view(np.int16)), img, rg.PLANES_INTERLEAVED, n)
    got = host(img)
    oref, odark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, quirk)
    rec = oracle.f2p_records(ns(d), quirk)
    exp = oracle.fbp(ns(d), op, rec, oref, odark, sc.raw, sc.planes)
    for b in range(n):
        mr, l2 = rel_err(got[b], exp[b])
        assert mr < MAX_REL and l2 < MAX_REL, (b, mr, l2)


@pytest.mark.parametrize("Pp,Dp", [(93, 96), (96, 90)])
def test_fbp_rebinning_tiles(Pp, Dp):
    """The engine's rebinning from frame quads on shapes that end in partial
    blocks: an odd angle count (93) and a ray count that is not a multiple of
    32 (90)."""
    d, sc, g, p, op = _fbp_case(rg.QUIRKS_NONE, False, masking=True, L=2, frames=3)
    d.update(n_par_proj=Pp, n_par_det=Dp)
    g = geom(d)
    n = sc.raw.shape[0]
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    img = torch.empty((n, d["n_pixels"], d["n_pixels"]), dtype=torch.float32, device="cuda")
    fbp.enqueue(dev(sc.raw.view(np.int16)), img, rg.PLANES_INTERLEAVED, n)
    got = host(img)
    oref, odark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, rg.QUIRKS_NONE)
    exp = oracle.fbp(ns(d), op, oracle.f2p_records(ns(d), rg.QUIRKS_NONE), oref, odark, sc.raw, sc.planes)
    for b in range(n):
        mr, l2 = rel_err(got[b], exp[b])
        assert mr < MAX_REL and l2 < MAX_REL, (Pp, Dp, b, mr, l2)


def test_fbp_staged_rebinning():
    """A parallel sampling fine enough for the engine to stage each output
    tile's fan boxes in shared memory (404 angles x 344 rays from 500 x 432:
    partial angle and ray tiles), two planes, interleaved and fixed-plane
    batches, 3 frames per plane (a partly filled frame quad)."""
    d, sc, g, p, op = _fbp_case(rg.QUIRKS_NONE, True, masking=True, L=2, frames=3)
    d.update(n_par_proj=404, n_par_det=344, n_pixels=128)
    g = geom(d)
    n = sc.raw.shape[0]
    oref, odark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, rg.QUIRKS_NONE)
    rec = oracle.f2p_records(ns(d), rg.QUIRKS_NONE)
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    raw = sc.raw.view(np.int16)
    N = d["n_pixels"]
    plane1 = np.flatnonzero(sc.planes == 1)
    for plane, idx in ((rg.PLANES_INTERLEAVED, np.arange(n)), (1, plane1)):
        exp = oracle.fbp(ns(d), op, rec, oref, odark, sc.raw[idx], sc.planes[idx])
        img = torch.empty((len(idx), N, N), dtype=torch.float32, device="cuda")
        fbp.enqueue(dev(raw[idx]), img, plane, len(idx))
        got = host(img)
        for b in range(len(idx)):
            mr, l2 = rel_err(got[b], exp[b])
            assert mr < MAX_REL and l2 < MAX_REL, (plane, b, mr, l2)


def test_fbp_long_filter_rows():
    """Filter length 2048 (1024 rays zero padded, the benchmark's length):
    the engine's filter pass with one row pair per 128-thread CTA writing the
    pair records; an even and an odd batch (the last pair without its second
    slice), both plane modes."""
    d, sc, g, p, op = _fbp_case(rg.QUIRKS_NONE, True, masking=True, L=2, frames=3)
    d.update(n_par_proj=96, n_par_det=1024, n_pixels=128)
    g = geom(d)
    n = sc.raw.shape[0]
    oref, odark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, rg.QUIRKS_NONE)
    rec = oracle.f2p_records(ns(d), rg.QUIRKS_NONE)
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    raw = sc.raw.view(np.int16)
    N = d["n_pixels"]
    plane0 = np.flatnonzero(sc.planes == 0)
    for plane, idx in ((rg.PLANES_INTERLEAVED, np.arange(n)), (rg.PLANES_INTERLEAVED, np.arange(n - 2)),
                       (0, plane0)):
        exp = oracle.fbp(ns(d), op, rec, oref, odark, sc.raw[idx], sc.planes[idx])
        img = torch.empty((len(idx), N, N), dtype=torch.float32, device="cuda")
        fbp.enqueue(dev(raw[idx]), img, plane, len(idx))
        got = host(img)
        for b in range(len(idx)):
            mr, l2 = rel_err(got[b], exp[b])
            assert mr < MAX_REL and l2 < MAX_REL, (plane, len(idx), b, mr, l2)


@pytest.mark.parametrize("dp,pad,n_pix", [
    (200, 512, 64),     # rows at most half the FFT length: the pass skips the zero half; one warp per row pair
    (256, 512, 96),     # exactly half
    (300, 512, 96),     # more than half: the general pass
    (600, 1024, 128),   # general pass, two warps per row pair
    (600, 0, 128),      # default padding (2048), four warps per row pair
    (1500, 0, 128),     # 4096, eight warps per row pair
])
def test_fbp_filter_lengths(dp, pad, n_pix):
    """The engine's filter pass writing the backprojection's pair records, at
    every radix-16 length, with rows at most half, exactly half and more than
    half the FFT length, an odd batch (the last pair without its second
    slice), against the FP64 oracle."""
    d, sc, g, p, op = _fbp_case(rg.QUIRKS_NONE, True, masking=True, L=2, frames=3)
    d.update(n_par_proj=64, n_par_det=dp, n_pixels=n_pix)
    g = geom(d)
    p = rg.make_params(filter_type="sheppLogan", defects=True, masking=True, pad=pad)
    op = oracle.make_params(quirk=oracle.QUIRK_NONE, filter_type="sheppLogan", defects=True, masking=True, pad=pad)
    n = sc.raw.shape[0] - 1  # 5 frames
    oref, odark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, rg.QUIRKS_NONE)
    rec = oracle.f2p_records(ns(d), rg.QUIRKS_NONE)
    exp = oracle.fbp(ns(d), op, rec, oref, odark, sc.raw[:n], sc.planes[:n])
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    names = [rg.Backprojection.variant_name(v) for v in range(rg.Backprojection.variant_count())]
    raw = dev(sc.raw[:n].view(np.int16))
    for variant in ("staged_cp_s4_a8_p4", "staged_s2_a16_p4"):  # 4 and 2 slices per pair-record group
        fbp.backprojection().set_variant(names.index(variant))
        img = torch.full((n, n_pix, n_pix), float("nan"), dtype=torch.float32, device="cuda")
        fbp.enqueue(raw, img, rg.PLANES_INTERLEAVED, n)
        got = host(img)
        for b in range(n):
            mr, l2 = rel_err(got[b], exp[b])
            assert mr < MAX_REL and l2 < MAX_REL, (variant, b, mr, l2)
    fbp.backprojection().check()


def test_fbp_fused_filter_staging():
    """Staged backprojection variants with a radix-16 filter length: the filter
    writes the pair records itself (no staging pass); an odd batch leaves the
    second slice of its last pair empty."""
    d, sc, g, p, op = _fbp_case(rg.QUIRKS_NONE, True, masking=True, L=2, frames=3)
    d.update(n_par_det=256, n_pixels=128)  # filter length 512: the radix-16 path
    g = geom(d)
    n = sc.raw.shape[0]  # 6 frames
    oref, odark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, rg.QUIRKS_NONE)
    rec = oracle.f2p_records(ns(d), rg.QUIRKS_NONE)
    cases = [(rg.PLANES_INTERLEAVED, n, oracle.fbp(ns(d), op, rec, oref, odark, sc.raw, sc.planes)),
             (0, n - 1, oracle.fbp(ns(d), op, rec, oref, odark, sc.raw[: n - 1], np.zeros(n - 1, np.int64)))]
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    bp = fbp.backprojection()
    raw = dev(sc.raw.view(np.int16))
    N = d["n_pixels"]
    staged = [v for v in range(rg.Backprojection.variant_count())
              if rg.Backprojection.variant_name(v).startswith("staged")]
    assert staged
    for v in staged:
        bp.set_variant(v)
        for plane, batch, exp in cases:
            img = torch.zeros((batch, N, N), dtype=torch.float32, device="cuda")
            fbp.enqueue(raw[:batch], img, plane, batch)
            got = host(img)
            for b in range(batch):
                mr, l2 = rel_err(got[b], exp[b])
                assert mr < MAX_REL and l2 < MAX_REL, (rg.Backprojection.variant_name(v), plane, b, mr, l2)
        st = fbp.time_stages(raw, img, 0, n - 1, 1)
        assert st["bp_staging"] < 0.05, st
    bp.check()


def test_graph_replay_and_host_path_match_enqueue():
    d, sc, g, p, op = _fbp_case(rg.QUIRKS_NONE, True, True, L=2, frames=8)
    n = sc.raw.shape[0]  # 16 frames: host-path chunks 2, 2, 4, 4, 2, 2 (ramp, two graph replays, ramp)
    B = 4
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=B)
    N = d["n_pixels"]
    raw = dev(sc.raw.view(np.int16))
    ref_img = torch.empty((n, N, N), dtype=torch.float32, device="cuda")
    for c in range(0, n, B):
        fbp.enqueue(raw[c:c + B], ref_img[c:c + B], rg.PLANES_INTERLEAVED, B)
    expect = host(ref_img)
    s = torch.cuda.Stream()  # not ordered with the default stream: synchronise at the hand-over
    img = torch.zeros((n, N, N), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    graph = fbp.graph_capture(raw, img, rg.PLANES_INTERLEAVED, n, s)
    assert graph.kernel_count >= 2 * 5  # two chunks of the chain
    graph.replay(s)
    s.synchronize()
    np.testing.assert_array_equal(img.cpu().numpy(), expect)
    hraw = torch.from_numpy(sc.raw.view(np.int16)).pin_memory()
    himg = torch.zeros((n, N, N), dtype=torch.float32).pin_memory()
    fbp.run_host(hraw, himg, n, rg.PLANES_INTERLEAVED)
    np.testing.assert_array_equal(himg.numpy(), expect)
    # a ragged tail (n not a multiple of the batch) goes through the direct path
    himg2 = torch.zeros((n - 2, N, N), dtype=torch.float32).pin_memory()
    fbp.run_host(hraw[: n - 2], himg2, n - 2, rg.PLANES_INTERLEAVED)
    np.testing.assert_array_equal(himg2.numpy(), expect[: n - 2])
    # an odd frame count: the last chunk takes the plane-0 frame left over, which
    # the filter transforms without a partner slice (so not the same bits)
    himg3 = torch.zeros((n - 1, N, N), dtype=torch.float32).pin_memory()
    fbp.run_host(hraw[: n - 1], himg3, n - 1, rg.PLANES_INTERLEAVED)
    got3 = himg3.numpy()
    np.testing.assert_array_equal(got3[: n - 2], expect[: n - 2])
    assert rel_err(got3[n - 2], expect[n - 2])[0] < MAX_REL


@pytest.mark.parametrize("variant", ["staged_cp_s4_a8_p4", "staged_s2_a16_p4", "pairs_s2_a32"])
def test_two_lanes_match_one_lane(variant):
    """Graphs and the host path with one chunk's backprojection beside the next
    chunk's streaming stages (two lanes, two pair buffers) give the same bits
    as every stage in sequence; variants whose backprojection reads the
    rebinned sinogram itself run on one lane either way."""
    L = 2
    d = dict(SMALL, n_planes=L, source_diameter=[430.0] * L, delta_x=[0.0] * L, delta_z=[1417.0, 1430.0],
             source_angle=[360.0] * L, n_par_proj=128, n_par_det=256, n_pixels=128)
    sc = phantom.make_scan(8, L, 500, 432, 215.0, 240.0, seed=31, defect_fraction=0.01, distinct=8)
    n, N, B = sc.raw.shape[0], d["n_pixels"], 4  # 4 graph chunks; host chunks 2, 2, 4, 4, 2, 2
    g = geom(d)
    p = rg.make_params(filter_type="sheppLogan", defects=True, masking=True)
    v = [rg.Backprojection.variant_name(i) for i in range(rg.Backprojection.variant_count())].index(variant)
    raw = dev(sc.raw.view(np.int16))
    hraw = torch.from_numpy(sc.raw.view(np.int16)).pin_memory()
    out = {}
    for lanes in (1, 2):
        fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=B)
        fbp.backprojection().set_variant(v)
        fbp.set_lanes(lanes)
        direct = torch.empty((n, N, N), dtype=torch.float32, device="cuda")
        for c in range(0, n, B):
            fbp.enqueue(raw[c:c + B], direct[c:c + B], rg.PLANES_INTERLEAVED, B)
        s = torch.cuda.Stream()
        img = torch.full((n, N, N), float("nan"), dtype=torch.float32, device="cuda")
        # the enqueues and the fill ran on the default stream, which does not
        # order torch's streams: the graph must not start before they finish
        # (it uses the same engine buffers)
        torch.cuda.synchronize()
        graph = fbp.graph_capture(raw, img, rg.PLANES_INTERLEAVED, n, s)
        for _ in range(2):
            graph.replay(s)
        s.synchronize()
        himg = torch.full((n, N, N), float("nan"), dtype=torch.float32).pin_memory()
        fbp.run_host(hraw, himg, n, rg.PLANES_INTERLEAVED)
        fbp.backprojection().check()
        out[lanes] = (host(direct), img.cpu().numpy(), himg.numpy())
    ref = out[1][0]
    for lanes in (1, 2):
        for what, got in zip(("enqueue", "graph", "host path"), out[lanes]):
            np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32), err_msg=f"{lanes} lanes, {what}")
    ref_o, dark_o = oracle.attenuation_init(sc.ref, sc.dark, L, 0.67, 1.5, True, oracle.QUIRK_NONE)
    op = oracle.make_params(quirk=oracle.QUIRK_NONE, filter_type="sheppLogan", defects=True, masking=True)
    exp = oracle.fbp(ns(d), op, oracle.f2p_records(ns(d), oracle.QUIRK_NONE), ref_o, dark_o, sc.raw[:4], sc.planes[:4])
    for i in range(4):
        assert rel_err(ref[i], exp[i])[0] < MAX_REL, i


def test_errors_are_reported():
    g = rg.make_geometry(n_par_proj=16, n_par_det=16, n_pixels=16)
    bp = rg.Backprojection(g, rg.make_params())
    with pytest.raises(rg.RisaError) as e:
        bp.enqueue(0, 0, 1)
    assert e.value.status == -1
    with pytest.raises(rg.RisaError):
        rg.Fan2Para(rg.make_geometry(n_planes=0), rg.make_params())


# ------------------------------------------------------------------------------ adjoints
def test_backprojection_adjoint_dot_product():
    Pp, Dp, N = 60, 80, 64
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N)
    bp = rg.Backprojection(g, rg.make_params())
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2, Pp, Dp)).astype(np.float32)
    y = rng.standard_normal((2, N, N)).astype(np.float32)
    ax = torch.empty((2, N, N), dtype=torch.float32, device="cuda")
    aty = torch.empty((2, Pp, Dp), dtype=torch.float32, device="cuda")
    bp.enqueue(dev(x), ax, 2)
    bp.enqueue_adjoint(dev(y), aty, 2)
    lhs = float((host(ax).astype(np.float64) * y).sum())
    rhs = float((x.astype(np.float64) * host(aty)).sum())
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))


def test_backprojection_adjoint_fast_path():
    """The reserved slice-interleaved adjoint agrees with the direct gather and
    passes the dot test; a batch that is not a multiple of 8 and an image side
    that is not a multiple of 32 exercise the padded slices and tiles."""
    Pp, Dp, N, n = 90, 100, 72, 11
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N)
    direct = rg.Backprojection(g, rg.make_params())
    fast = rg.Backprojection(g, rg.make_params())
    fast.reserve_adjoint(n)
    rng = np.random.default_rng(5)
    x = rng.standard_normal((n, Pp, Dp)).astype(np.float32)
    y = rng.standard_normal((n, N, N)).astype(np.float32)
    a0 = torch.zeros((n, Pp, Dp), dtype=torch.float32, device="cuda")
    a1 = torch.zeros((n, Pp, Dp), dtype=torch.float32, device="cuda")
    direct.enqueue_adjoint(dev(y), a0, n)
    fast.enqueue_adjoint(dev(y), a1, n)
    r0, r1 = host(a0), host(a1)
    assert np.abs(r1 - r0).max() <= 1e-5 * np.abs(r0).max()
    ax = torch.empty((n, N, N), dtype=torch.float32, device="cuda")
    fast.enqueue(dev(x), ax, n)
    lhs = float((host(ax).astype(np.float64) * y).sum())
    rhs = float((x.astype(np.float64) * r1).sum())
    terms = float(np.abs(host(ax).astype(np.float64) * y).sum())
    assert abs(lhs - rhs) <= 1e-6 * terms


def test_fan2para_adjoint_dot_product():
    g = geom(SMALL)
    f2p = rg.Fan2Para(g, rg.make_params())
    rng = np.random.default_rng(4)
    x = rng.standard_normal((1, 500, 432)).astype(np.float32)
    y = rng.standard_normal((1, 64, 64)).astype(np.float32)
    ax = torch.empty((1, 64, 64), dtype=torch.float32, device="cuda")
    aty = torch.empty((1, 500, 432), dtype=torch.float32, device="cuda")
    f2p.enqueue(dev(x), ax, 0, 1)
    f2p.enqueue_adjoint(dev(y), aty, 0, 1)
    lhs = float((host(ax).astype(np.float64) * y).sum())
    rhs = float((x.astype(np.float64) * host(aty)).sum())
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))
