"""The benchmark configurations end to end on the GPU, against the FP64 oracle.

Plain single-plane: 64 frames of 500 x 432 uint16 counts (8-ellipse
phantoms, I0 40000, dark 200, Poisson), one dark and one reference frame,
rebinned to 256 angles x 256 rays, zero padded to 512, Ram-Lak,
backprojected to 256^2 -- through the reference-style per-stage path (one
frame per stage call) and through the batched engine, and the two paths
against each other.

Full-rate streaming, at its real geometry: 2 interleaved planes of 1000 x 1152
frames with 1% defective detector columns, rebinned to 1024 x 1024, zero
padded to 2048, Shepp-Logan, 512^2 with the circular mask -- through the
engine with the autotuned backprojection variant (and every other variant),
and through a captured graph replay, which must give the same bits.

The FP32 bar is max|gpu - oracle| / max|oracle| <= 1e-5 and
||gpu - oracle||_2 / ||oracle||_2 <= 1e-5 per image."""
import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from risa_gb300 import phantom
from tests.helpers import CFG1, CFG2, geom, ns, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_REL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def test_plain_small_configuration():
    d = dict(CFG1)
    g = geom(d)
    n = 64
    sc = phantom.make_scan(n, 1, 500, 432, 215.0, 240.0, seed=101, distinct=8)
    p = rg.make_params(filter_type="ramp")
    op = oracle.make_params(quirk=oracle.QUIRK_NONE, filter_type="ramp")
    # the reference frames are repaired before averaging (repair_reference defaults on)
    ref, dark = oracle.attenuation_init(sc.ref, sc.dark, 1, 0.67, 1.5, True, oracle.QUIRK_NONE)
    exp = oracle.fbp(ns(d), op, oracle.f2p_records(ns(d), oracle.QUIRK_NONE), ref, dark, sc.raw, sc.planes)
    N, Pp, Dp = d["n_pixels"], d["n_par_proj"], d["n_par_det"]
    raw = torch.from_numpy(np.ascontiguousarray(sc.raw.view(np.int16))).cuda()

    # per-stage path, one frame per call (the reference's structure)
    att = rg.Attenuation(g, p, sc.ref, 1, sc.dark, 1)
    f2p, filt, bp = rg.Fan2Para(g, p), rg.Filter(g, p), rg.Backprojection(g, p)
    fan = torch.empty((1, 500, 432), dtype=torch.float32, device="cuda")
    par = torch.empty((1, Pp, Dp), dtype=torch.float32, device="cuda")
    plain = torch.empty((n, N, N), dtype=torch.float32, device="cuda")
    for i in range(n):
        att.enqueue(raw[i:i + 1], fan, 0, 1)
        f2p.enqueue(fan, par, 0, 1)
        filt.enqueue(par, 1)
        bp.enqueue(par, plain[i:i + 1], 1)
    # batched engine, all frames in one enqueue
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    batched = torch.empty((n, N, N), dtype=torch.float32, device="cuda")
    fbp.enqueue(raw, batched, 0, n)
    torch.cuda.synchronize()
    got_p, got_b = plain.cpu().numpy(), batched.cpu().numpy()
    for i in range(n):
        for name, got in (("plain", got_p[i]), ("batched", got_b[i])):
            mr, l2 = rel_err(got, exp[i])
            assert mr < MAX_REL and l2 < MAX_REL, (name, i, mr, l2)
        assert rel_err(got_b[i], got_p[i])[0] < MAX_REL, i


def test_full_rate_streaming_configuration():
    d = dict(CFG2)
    L, Pf, Df, N = d["n_planes"], d["n_fan_proj"], d["n_fan_det"], d["n_pixels"]
    g = geom(d)
    frames_per_plane = 8
    sc = phantom.make_scan(frames_per_plane, L, Pf, Df, 215.0, 240.0, seed=2026, defect_fraction=0.01,
                           distinct=frames_per_plane)
    n = sc.raw.shape[0]
    assert len(sc.dead) + len(sc.flicker) >= Df // 100
    p = rg.make_params(filter_type="sheppLogan", defects=True, masking=True)
    op = oracle.make_params(quirk=oracle.QUIRK_NONE, filter_type="sheppLogan", defects=True, masking=True)
    ref, dark = oracle.attenuation_init(sc.ref, sc.dark, L, 0.67, 1.5, True, oracle.QUIRK_NONE)
    exp = oracle.fbp(ns(d), op, oracle.f2p_records(ns(d), oracle.QUIRK_NONE), ref, dark, sc.raw, sc.planes)

    raw = torch.from_numpy(np.ascontiguousarray(sc.raw.view(np.int16))).cuda()
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    img = torch.empty((n, N, N), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    fbp.enqueue(raw, img, rg.PLANES_INTERLEAVED, n, stream)
    stream.synchronize()
    bp = fbp.backprojection()
    _, par_buf = fbp.intermediates()
    chosen = bp.autotune(par_buf, img.data_ptr(), n, stream)

    def check(got, what):
        for i in range(n):
            mr, l2 = rel_err(got[i], exp[i])
            assert mr < MAX_REL and l2 < MAX_REL, (what, i, mr, l2)

    # the autotuned variant (the benchmark's choice), enqueue and graph replay
    bp.set_variant(chosen)
    img.fill_(float("nan"))
    torch.cuda.synchronize()  # the fill ran on the default stream, the engine runs on `stream`
    fbp.enqueue(raw, img, rg.PLANES_INTERLEAVED, n, stream)
    stream.synchronize()
    bp.check()
    direct = img.cpu().numpy()
    check(direct, f"enqueue, {rg.Backprojection.variant_name(chosen)}")
    graph = fbp.graph_capture(raw, img, rg.PLANES_INTERLEAVED, n, stream)
    for _ in range(2):
        img.fill_(float("nan"))
        torch.cuda.synchronize()
        graph.replay(stream)
        stream.synchronize()
        np.testing.assert_array_equal(img.cpu().numpy().view(np.uint32), direct.view(np.uint32))
    # every other backprojection variant on the same frames (a variant whose
    # staging does not fit the geometry is refused before any launch)
    ran = [chosen]
    for v in range(rg.Backprojection.variant_count()):
        if v == chosen:
            continue
        bp.set_variant(v)
        img.fill_(float("nan"))
        torch.cuda.synchronize()
        try:
            fbp.enqueue(raw, img, rg.PLANES_INTERLEAVED, n, stream)
        except rg.RisaError:
            continue
        stream.synchronize()
        bp.check()
        check(img.cpu().numpy(), rg.Backprojection.variant_name(v))
        ran.append(v)
    print("variants checked:", [rg.Backprojection.variant_name(v) for v in ran])
    assert len(ran) >= rg.Backprojection.variant_count() // 2
