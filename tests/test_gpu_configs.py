"""The plain single-plane configuration end to end on the GPU: 64 frames of
500 x 432 uint16 counts (8-ellipse phantoms, I0 40000, dark 200, Poisson),
one dark and one reference frame, rebinned to 256 angles x 256 rays, zero
padded to 512, Ram-Lak, backprojected to 256^2 -- through the reference-style
per-stage path (one frame per stage call) and through the batched engine,
both against the FP64 oracle at the FP32 bar (max-rel 1e-5), and the two
paths against each other."""
import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from risa_gb300 import phantom
from tests.helpers import CFG1, geom, ns, rel_err

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
