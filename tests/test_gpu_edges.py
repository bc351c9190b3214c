"""GPU edge cases through the C ABI: empty batches, image sides that are not a
multiple of the 32-pixel tile with the fused circular mask (ragged tiles and
the edge-warp skipping together), and the largest geometry of the uneven
sweep on the staged backprojection. FP32 bar as everywhere: max-rel 1e-5
against the FP64 oracle."""
import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from risa_gb300 import phantom
from tests.helpers import SMALL, geom, rel_err

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


def test_empty_batches_touch_nothing():
    d = dict(SMALL)
    g = geom(d)
    p = rg.make_params(defects=True, masking=True)
    sc = phantom.make_scan(2, 1, 500, 432, 215.0, 240.0, seed=3)
    raw = dev(sc.raw.view(np.int16))
    N, Pp, Dp = d["n_pixels"], d["n_par_proj"], d["n_par_det"]
    fan = torch.full((1, 500, 432), np.nan, dtype=torch.float32, device="cuda")
    par = torch.full((1, Pp, Dp), np.nan, dtype=torch.float32, device="cuda")
    img = torch.full((1, N, N), np.nan, dtype=torch.float32, device="cuda")
    rg.Attenuation(g, p, sc.ref, 1, sc.dark, 1).enqueue(raw, fan, 0, 0)
    rg.Fan2Para(g, p).enqueue(fan, par, 0, 0)
    rg.Filter(g, p).enqueue(par, 0)
    bp = rg.Backprojection(g, p)
    bp.enqueue(par, img, 0)
    bp.enqueue_adjoint(img, par, 0)
    rg.Masking(g, p).enqueue(img, 0)
    rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=2).enqueue(raw, img, 0, 0)
    for t in (fan, par, img):
        assert np.isnan(host(t)).all()


@pytest.mark.parametrize("N", [100, 101])
def test_masked_backprojection_ragged_tiles(N):
    """N not a multiple of 32: partial tiles at the right and bottom edges, and
    circle-edge warps skipped inside them; every pixel must still be written."""
    Pp, Dp = 120, 2 * N + 6
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N, rotation_offset=3.0)
    p = rg.make_params(masking=True, masking_value=-2.0)
    bp = rg.Backprojection(g, p)
    bp.reserve(5)
    sino, _ = phantom.parallel_sinograms(5, Pp, Dp, 200.0, seed=12)
    exps = [oracle.mask(oracle.backproject(sino[b], N, 3.0), -2.0) for b in range(5)]
    img = torch.empty((5, N, N), dtype=torch.float32, device="cuda")
    for v in range(rg.Backprojection.variant_count()):
        bp.set_variant(v)
        img.fill_(np.nan)
        bp.enqueue(dev(sino), img, 5)
        got = host(img)
        assert not np.isnan(got).any(), rg.Backprojection.variant_name(v)
        for b in range(5):
            mr, _ = rel_err(got[b], exps[b])
            assert mr < MAX_REL, (rg.Backprojection.variant_name(v), b, mr)
    bp.check()


def test_largest_sweep_geometry_staged():
    """1440 angles x 1280 rays -> 1024^2 (the largest instance the uneven sweep
    draws), one slice, through the autotuned staged backprojection."""
    Pp, Dp, N = 1440, 1280, 1024
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N)
    p = rg.make_params(masking=True)
    bp = rg.Backprojection(g, p)
    sino, _ = phantom.parallel_sinograms(1, Pp, Dp, 200.0, seed=31)
    img = torch.empty((1, N, N), dtype=torch.float32, device="cuda")
    v = bp.autotune(dev(sino), img, 1)
    img.fill_(np.nan)
    bp.enqueue(dev(sino), img, 1)
    got = host(img)
    bp.check()
    exp = oracle.mask(oracle.backproject(sino[0], N), 0.0)
    mr, l2 = rel_err(got[0], exp)
    assert mr < MAX_REL and l2 < MAX_REL, (rg.Backprojection.variant_name(v), mr, l2)


def test_constant_parameter_variants_refuse_many_angles():
    """The staged variants that take the angle coefficients from their kernel
    parameters hold at most 2048 angles: with 2100 they refuse before any
    launch (an error, the context stays usable) and the autotuner picks
    another variant, whose output matches the oracle."""
    Pp, Dp, N = 2100, 96, 64
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N)
    bp = rg.Backprojection(g, rg.make_params(masking=True))
    bp.reserve(1)
    names = [rg.Backprojection.variant_name(v) for v in range(rg.Backprojection.variant_count())]
    cp = [v for v, name in enumerate(names) if name.startswith("staged_cp")]
    assert cp
    sino, _ = phantom.parallel_sinograms(1, Pp, Dp, 200.0, seed=5)
    img = torch.empty((1, N, N), dtype=torch.float32, device="cuda")
    for v in cp:
        bp.set_variant(v)
        with pytest.raises(rg.RisaError):
            bp.enqueue(dev(sino), img, 1)
    v = bp.autotune(dev(sino), img, 1)
    assert v not in cp
    img.fill_(np.nan)
    bp.enqueue(dev(sino), img, 1)
    got = host(img)
    bp.check()
    exp = oracle.mask(oracle.backproject(sino[0], N), 0.0)
    mr, l2 = rel_err(got[0], exp)
    assert mr < MAX_REL and l2 < MAX_REL, (names[v], mr, l2)
