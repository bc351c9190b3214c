"""Uneven sweep (many reconstructions of different shapes in one persistent
launch) against the FP64 oracle chain, instance by instance:

    repair (interpolateDefectDetectors run rule, NONE mode) -> attenuation with
    a flat field -> filter (zero padded to a power of two >= 2 Dp) ->
    linear backprojection (NONE sampling) -> circular mask

FP32 bar: max|gpu - oracle| / max|oracle| <= 1e-5 per instance.
"""
import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from risa_gb300 import phantom
from tests.helpers import SMALL, ns, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_REL = 1e-5


def _defects(dp, cols):
    m = np.zeros(dp, np.uint8)
    m[list(cols)] = 1
    return m


CASES = [
    # (N, Pp, Dp, filter, cutoff, rotation, masking, defect columns)
    (128, 180, 160, "ramp", 1.0, 0.0, True, [0, 159, 70]),         # run wrapping through column 0
    (200, 361, 256, "hanning", 0.8, -7.5, False, [10, 11, 200]),    # 2-wide run, no mask
    (300, 500, 384, "ramp", 1.0, 0.0, True, []),                    # FFT 1024, no defects
    (256, 1440, 640, "hanning", 1.0, 0.0, True, [320, 321, 322]),  # FFT 2048, 2.5 bins per pixel
    (160, 250, 1280, "ramp", 1.0, 3.0, True, [5, 900]),             # FFT 4096, 8 bins per pixel
    (500, 720, 640, "ramp", 1.0, 0.0, True, [1, 2, 639]),           # ragged tiles (500 = 15 x 32 + 20)
    (1024, 180, 1280, "hanning", 1.0, 0.0, True, [100]),            # largest image
]


def _oracle(inst, raw):
    pp, dp, n = inst["n_par_proj"], inst["n_par_det"], inst["n_pixels"]
    flags = np.zeros(dp + 1, np.int32)
    if inst.get("defect_map") is not None:
        flags[:dp] = inst["defect_map"]
    rep = oracle.interpolate_defects(raw, flags, oracle.QUIRK_NONE)
    ref = np.full((pp, dp), inst["ref_level"], np.float32)
    dark = np.full(dp, inst["dark_level"], np.float32)
    att = oracle.attenuation(rep, ref, dark)
    g = ns(SMALL, n_par_proj=pp, n_par_det=dp, n_pixels=n, rotation_offset=inst["rotation_offset"])
    p = oracle.make_params(filter_type=inst["filter_type"], cutoff=inst["cutoff"], masking=inst["masking"],
                           masking_value=inst["masking_value"])
    return oracle.fbp_parallel(g, p, att[None])[0]


def _run(instances, seed):
    sw = rg.Sweep(instances)
    ro, io, rt, it = sw.layout()
    raws = [phantom.sweep_counts(d, seed + i) for i, d in enumerate(instances)]
    packed = np.concatenate([r.ravel() for r in raws])
    assert packed.size == rt
    t_raw = torch.from_numpy(packed.view(np.int16)).cuda()
    t_img = torch.full((it,), float("nan"), dtype=torch.float32, device="cuda")
    sw.enqueue(t_raw, t_img)
    sw.check()
    img = t_img.cpu().numpy()
    return sw, raws, img, io


def test_sweep_matches_oracle_per_instance():
    instances = [dict(n_pixels=n, n_par_proj=pp, n_par_det=dp, filter_type=f, cutoff=c, rotation_offset=rot,
                      ref_level=40200.0, dark_level=200.0, masking=m, masking_value=-1.0 if m else 0.0,
                      defect_map=_defects(dp, cols) if cols else None)
                 for (n, pp, dp, f, c, rot, m, cols) in CASES]
    sw, raws, img, io = _run(instances, seed=100)
    for i, d in enumerate(instances):
        n = d["n_pixels"]
        got = img[io[i]:io[i] + n * n].reshape(n, n)
        exp = _oracle(d, raws[i])
        assert np.isfinite(got).all(), i
        mr, l2 = rel_err(got, exp)
        assert mr < MAX_REL, (i, mr, l2)
    first, done, launch = sw.times()
    assert launch > 0 and np.all(done > 0) and np.all(first >= launch) and np.all(done > first)


def test_sweep_seeded_config_and_repeat():
    instances = phantom.sweep_instances(6, seed=3, n_max=384, pp_max=600)
    sw, raws, img, io = _run(instances, seed=7)
    for i, d in enumerate(instances):
        n = d["n_pixels"]
        got = img[io[i]:io[i] + n * n].reshape(n, n)
        assert rel_err(got, _oracle(d, raws[i]))[0] < MAX_REL, i
    # a second launch of the same work gives the same bits (no atomics on data)
    t_raw = torch.from_numpy(np.concatenate([r.ravel() for r in raws]).view(np.int16)).cuda()
    t_img = torch.empty(img.size, dtype=torch.float32, device="cuda")
    sw.enqueue(t_raw, t_img)
    sw.check()
    np.testing.assert_array_equal(t_img.cpu().numpy().view(np.uint32), img.view(np.uint32))
    # the same launch captured as a CUDA graph and replayed twice
    s = torch.cuda.Stream()
    t_img.fill_(float("nan"))
    graph = sw.graph_capture(t_raw, t_img, s)
    for _ in range(2):
        t_img.fill_(float("nan"))
        torch.cuda.synchronize()  # the fill ran on the default stream
        graph.replay(s)
        s.synchronize()
        sw.check()
        np.testing.assert_array_equal(t_img.cpu().numpy().view(np.uint32), img.view(np.uint32))
    first, done, launch = sw.times()
    assert (done >= first).all() and (first >= launch).all()
