"""Differentiation through the C ABI: test-only torch.autograd.Functions over
the hand-written kernels (taps filter, its transpose and taps gradient, the
backprojection and its adjoint -- the ray-driven forward projector -- and the
fan-to-parallel rebinning and its transpose).

FBP(s; h) = BP(F_h(s)) for parallel sinograms s [n, Pp, Dp] and real filter
taps h, and FanFBP(f; h) = BP(F_h(R f)) for fan sinograms f [n, Pf, Df] with
the rebinning R. Checked: adjoint identities <Ax, y> = <x, A^T y> to 1e-5 (of
the sum of the terms' magnitudes) for the filter, the backprojection and both
whole maps; the taps filter against the FP64 oracle's direct convolution; and
gradients of L = ||map - x_true||^2 against FP64 central finite differences
(step 1e-4) of the oracle: on the differentiation configuration (16 slices,
720 angles x 768 rays -> 512^2, 1024 taps, 10-ellipse phantom) for 32 random
taps and 32 random sinogram entries, and on a small fan geometry for 16 taps
and 16 fan-sinogram entries. The FP32 gradients meet 1e-4 of the largest
finite difference (the printed errors are the measured ones).
"""
import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from risa_gb300 import phantom

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


class FBPFunction(torch.autograd.Function):
    """y = BP(F_h(s)); backward works in slice chunks (bounded memory: only one
    chunk's backprojected gradient is alive at a time; nothing of the forward
    pass but s and h is kept)."""

    @staticmethod
    def forward(ctx, s, h, geom, params, chunk):
        n = s.shape[0]
        N = geom.n_pixels
        filt = rg.Filter(geom, params, taps=h.detach().cpu().numpy())
        bp = rg.Backprojection(geom, params)
        out = torch.empty((n, N, N), dtype=torch.float32, device=s.device)
        for c in range(0, n, chunk):
            nb = min(chunk, n - c)
            q = s[c:c + nb].detach().clone().contiguous()
            filt.enqueue(q, nb)
            bp.enqueue(q, out[c:c + nb], nb)
        ctx.save_for_backward(s, h)
        ctx.geom, ctx.params, ctx.chunk = geom, params, chunk
        return out

    @staticmethod
    def backward(ctx, gy):
        s, h = ctx.saved_tensors
        geom, params, chunk = ctx.geom, ctx.params, ctx.chunk
        n, Pp, Dp = s.shape
        filt = rg.Filter(geom, params, taps=h.detach().cpu().numpy())
        bp = rg.Backprojection(geom, params)
        bp.reserve_adjoint(chunk)
        gs = torch.empty_like(s)
        gh = torch.zeros(h.shape[0], dtype=torch.float64, device=s.device)
        part = torch.empty(h.shape[0], dtype=torch.float32, device=s.device)
        ws = torch.empty(filt.taps_grad_workspace_bytes(chunk), dtype=torch.uint8, device=s.device)
        gy = gy.contiguous()
        for c in range(0, n, chunk):
            nb = min(chunk, n - c)
            gq = torch.empty((nb, Pp, Dp), dtype=torch.float32, device=s.device)
            bp.enqueue_adjoint(gy[c:c + nb], gq, nb)
            filt.taps_grad(s[c:c + nb].contiguous(), gq, part, nb, ws)
            gh += part.double()
            filt.enqueue_adjoint(gq, nb)
            gs[c:c + nb] = gq
        return gs, gh.float(), None, None, None


class FanFBPFunction(torch.autograd.Function):
    """y = BP(F_h(R f)) for fan sinograms f of one plane; the backward pass runs
    the rebinning transpose R^T (risa_gb_fan2para_enqueue_adjoint) after the
    transposed filter. Slice chunks as in FBPFunction; R f is recomputed per
    chunk in the backward pass (it feeds the taps gradient)."""

    @staticmethod
    def forward(ctx, f, h, geom, params, chunk):
        n = f.shape[0]
        N, Pp, Dp = geom.n_pixels, geom.n_par_proj, geom.n_par_det
        rebin = rg.Fan2Para(geom, params)
        filt = rg.Filter(geom, params, taps=h.detach().cpu().numpy())
        bp = rg.Backprojection(geom, params)
        out = torch.empty((n, N, N), dtype=torch.float32, device=f.device)
        q = torch.empty((chunk, Pp, Dp), dtype=torch.float32, device=f.device)
        for c in range(0, n, chunk):
            nb = min(chunk, n - c)
            rebin.enqueue(f[c:c + nb].detach().contiguous(), q, 0, nb)
            filt.enqueue(q, nb)
            bp.enqueue(q, out[c:c + nb], nb)
        ctx.save_for_backward(f, h)
        ctx.geom, ctx.params, ctx.chunk = geom, params, chunk
        return out

    @staticmethod
    def backward(ctx, gy):
        f, h = ctx.saved_tensors
        geom, params, chunk = ctx.geom, ctx.params, ctx.chunk
        n = f.shape[0]
        Pp, Dp = geom.n_par_proj, geom.n_par_det
        rebin = rg.Fan2Para(geom, params)
        filt = rg.Filter(geom, params, taps=h.detach().cpu().numpy())
        bp = rg.Backprojection(geom, params)
        bp.reserve_adjoint(chunk)
        gf = torch.empty_like(f)
        gh = torch.zeros(h.shape[0], dtype=torch.float64, device=f.device)
        part = torch.empty(h.shape[0], dtype=torch.float32, device=f.device)
        ws = torch.empty(filt.taps_grad_workspace_bytes(chunk), dtype=torch.uint8, device=f.device)
        q = torch.empty((chunk, Pp, Dp), dtype=torch.float32, device=f.device)
        gq = torch.empty((chunk, Pp, Dp), dtype=torch.float32, device=f.device)
        gy = gy.contiguous()
        for c in range(0, n, chunk):
            nb = min(chunk, n - c)
            rebin.enqueue(f[c:c + nb].detach().contiguous(), q, 0, nb)
            bp.enqueue_adjoint(gy[c:c + nb], gq, nb)
            filt.taps_grad(q, gq, part, nb, ws)
            gh += part.double()
            filt.enqueue_adjoint(gq, nb)
            rebin.enqueue_adjoint(gq, gf[c:c + nb], 0, nb)
        return gf, gh.float(), None, None, None


def _geom(Pp, Dp, N, width=200.0):
    return rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N, image_width=width)


def _ramp_taps(n_taps, rng, jitter=0.05):
    """Spatial ramp kernel (1/4 at 0, -1/(pi n)^2 at odd n) plus a seeded perturbation."""
    c = n_taps // 2
    k = np.arange(n_taps) - c
    h = np.zeros(n_taps)
    h[k == 0] = 0.25
    odd = (k % 2) != 0
    h[odd] = -1.0 / (np.pi * k[odd]) ** 2
    return (h + jitter * rng.standard_normal(n_taps) / n_taps).astype(np.float32)


def test_taps_filter_matches_oracle_and_is_adjoint():
    rng = np.random.default_rng(0)
    Pp, Dp, n_taps = 33, 200, 64
    g = _geom(Pp, Dp, 64)
    taps = rng.standard_normal(n_taps).astype(np.float32)
    filt = rg.Filter(g, rg.make_params(), taps=taps)
    x = rng.standard_normal((2, Pp, Dp)).astype(np.float32)
    y = rng.standard_normal((2, Pp, Dp)).astype(np.float32)
    tx = torch.from_numpy(x).cuda()
    filt.enqueue(tx, 2)
    fx = tx.cpu().numpy()
    for b in range(2):
        exp = oracle.filter_rows_taps(x[b], taps)
        assert np.abs(fx[b] - exp).max() / np.abs(exp).max() < 1e-5
    ty = torch.from_numpy(y).cuda()
    filt.enqueue_adjoint(ty, 2)
    fty = ty.cpu().numpy()
    lhs = float((fx.astype(np.float64) * y).sum())
    rhs = float((x.astype(np.float64) * fty).sum())
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))


def test_taps_gradient_matches_direct_correlation():
    rng = np.random.default_rng(1)
    Pp, Dp, n_taps = 17, 96, 48
    g = _geom(Pp, Dp, 32)
    taps = rng.standard_normal(n_taps).astype(np.float32)
    filt = rg.Filter(g, rg.make_params(), taps=taps)
    x = rng.standard_normal((3, Pp, Dp)).astype(np.float32)
    gout = rng.standard_normal((3, Pp, Dp)).astype(np.float32)
    ws = torch.empty(filt.taps_grad_workspace_bytes(3), dtype=torch.uint8, device="cuda")
    grad = torch.empty(n_taps, dtype=torch.float32, device="cuda")
    filt.taps_grad(torch.from_numpy(x).cuda(), torch.from_numpy(gout).cuda(), grad, 3, ws)
    c = n_taps // 2
    exp = np.zeros(n_taps)
    xs = x.astype(np.float64).reshape(-1, Dp)
    gs = gout.astype(np.float64).reshape(-1, Dp)
    for j in range(n_taps):
        sh = j - c  # y[n] += h[j] x[n - sh]
        if sh >= 0:
            exp[j] = (gs[:, sh:] * xs[:, :Dp - sh]).sum()
        else:
            exp[j] = (gs[:, :Dp + sh] * xs[:, -sh:]).sum()
    got = grad.cpu().numpy()
    assert np.abs(got - exp).max() / np.abs(exp).max() < 1e-5


def test_whole_map_adjoint():
    rng = np.random.default_rng(2)
    Pp, Dp, N, n_taps = 60, 96, 64, 32
    g = _geom(Pp, Dp, N)
    p = rg.make_params()
    h = torch.from_numpy(rng.standard_normal(n_taps).astype(np.float32)).cuda()
    x = torch.from_numpy(rng.standard_normal((3, Pp, Dp)).astype(np.float32)).cuda().requires_grad_(True)
    y = torch.from_numpy(rng.standard_normal((3, N, N)).astype(np.float32)).cuda()
    ax = FBPFunction.apply(x, h, g, p, 2)
    (aty,) = torch.autograd.grad(ax, x, grad_outputs=y)
    # Dot-product test <Ax, y> == <x, A^T y>. Both sums cancel heavily (random
    # signs), so the FP32 rounding of A x and A^T y is measured against the
    # sum of the magnitudes of the terms, not against the cancelled total.
    t_l = ax.detach().double() * y.double()
    t_r = x.detach().double() * aty.double()
    lhs, rhs = float(t_l.sum()), float(t_r.sum())
    scale = max(float(t_l.abs().sum()), float(t_r.abs().sum()))
    assert abs(lhs - rhs) <= 1e-5 * scale, (lhs, rhs, scale)


def test_differentiation_configuration_fd_gradients():
    # 16 slices at 512^2 from 720 angles x 768 rays, 1024 taps, 10-ellipse phantoms
    n, Pp, Dp, N, n_taps, W = 16, 720, 768, 512, 1024, 200.0
    rng = np.random.default_rng(2024)
    sino, phs = phantom.parallel_sinograms(n, Pp, Dp, W, seed=77, n_ellipses=10)
    # with the spatial ramp taps (unit sample spacing) and the backprojection's
    # normalisation pi / Pp * N / Dp, the reconstruction is mu * (W / Dp) * (N / Dp)
    x_true = np.stack([phantom.rasterize(ph, N, W) for ph in phs]) * (W / Dp) * (N / Dp)
    taps = _ramp_taps(n_taps, rng)
    g = _geom(Pp, Dp, N, W)
    p = rg.make_params()
    s = torch.from_numpy(sino).cuda().requires_grad_(True)
    h = torch.from_numpy(taps).cuda().requires_grad_(True)
    xt = torch.from_numpy(x_true.astype(np.float32)).cuda()
    y = FBPFunction.apply(s, h, g, p, 4)
    loss = ((y.double() - xt.double()) ** 2).sum()
    loss.backward()
    gh = h.grad.detach().cpu().numpy().astype(np.float64)
    assert s.grad is not None and torch.isfinite(s.grad).all()

    # FP64 central differences of L on 32 random taps. L is quadratic in h and
    # the oracle's FBP is linear in h, so L(h +- eps e_j) = ||r +- eps A e_j||^2
    # with r = A h - x_true and A e_j the FP64 reconstruction with tap j alone.
    og = type("G", (), dict(n_planes=1, n_fan_det=4, n_fan_proj=2, n_par_proj=Pp, n_par_det=Dp, n_pixels=N,
                            source_offset=0.0, detector_diameter=1.0, image_width=W, image_center_x=0.0,
                            image_center_y=0.0, rotation_offset=0.0, source_diameter=[1.0], delta_x=[0.0],
                            delta_z=[1.0], source_angle=[360.0]))()
    op = oracle.make_params()
    ah = oracle.fbp_parallel_taps(og, op, sino, taps.astype(np.float64))
    r = ah - x_true
    eps = 1e-4
    idx = rng.choice(n_taps, size=32, replace=False)
    fd = np.zeros(32)
    for i, j in enumerate(idx):
        e = np.zeros(n_taps)
        e[j] = 1.0
        aj = oracle.fbp_parallel_taps(og, op, sino, e)
        lp = ((r + eps * aj) ** 2).sum()
        lm = ((r - eps * aj) ** 2).sum()
        fd[i] = (lp - lm) / (2 * eps)
    err = np.abs(gh[idx] - fd).max() / np.abs(fd).max()

    # FP64 central differences on 32 random sinogram entries (slice b, angle a,
    # ray k): only slice b's term of L moves, by A e_(a,k), the FP64
    # reconstruction of a sinogram holding a single 1 (32 of them in one call).
    gs = s.grad.detach().cpu().numpy().astype(np.float64)
    picks = [(int(rng.integers(n)), int(rng.integers(Pp)), int(rng.integers(Dp))) for _ in range(32)]
    unit = np.zeros((32, Pp, Dp))
    for i, (b, a, k) in enumerate(picks):
        unit[i, a, k] = 1.0
    au = oracle.fbp_parallel_taps(og, op, unit, taps.astype(np.float64))
    fd_s = np.zeros(32)
    for i, (b, a, k) in enumerate(picks):
        lp = ((r[b] + eps * au[i]) ** 2).sum()
        lm = ((r[b] - eps * au[i]) ** 2).sum()
        fd_s[i] = (lp - lm) / (2 * eps)
    got_s = np.array([gs[b, a, k] for b, a, k in picks])
    err_s = np.abs(got_s - fd_s).max() / np.abs(fd_s).max()
    print(f"config-4 gradients vs FP64 central differences: taps {err:.2e}, sinogram entries {err_s:.2e}")
    assert err < 1e-4, err
    assert err_s < 1e-4, err_s


# A small fan geometry for the rebinning chain: 500 x 432 fan frames -> 96 x 128
# parallel -> 96^2, 48 taps.
FAN = dict(n_planes=1, n_fan_det=432, n_fan_proj=500, n_par_proj=96, n_par_det=128, n_pixels=96,
           source_offset=0.0, detector_diameter=480.0, image_width=200.0, source_diameter=[430.0],
           delta_x=[0.0], delta_z=[1417.0], source_angle=[360.0])


def _fan_oracle_map(f, taps):
    """FP64 FanFBP of fan sinograms f [n, Pf, Df] (one plane) with taps."""
    from tests.helpers import ns

    og = ns(FAN)
    rec = oracle.f2p_records(og, oracle.QUIRK_NONE)
    par = np.stack([oracle.f2p_apply(rec, 0, oracle.QUIRK_NONE, f[i]) for i in range(f.shape[0])])
    return oracle.fbp_parallel_taps(og, oracle.make_params(), par, taps)


def test_fan_map_adjoint():
    """<A f, y> = <f, A^T y> through rebinning, taps filter and backprojection."""
    rng = np.random.default_rng(5)
    g = rg.make_geometry(**FAN)
    p = rg.make_params()
    h = torch.from_numpy(rng.standard_normal(48).astype(np.float32)).cuda()
    f = torch.from_numpy(rng.standard_normal((3, 500, 432)).astype(np.float32)).cuda().requires_grad_(True)
    y = torch.from_numpy(rng.standard_normal((3, 96, 96)).astype(np.float32)).cuda()
    af = FanFBPFunction.apply(f, h, g, p, 2)
    (aty,) = torch.autograd.grad(af, f, grad_outputs=y)
    t_l = af.detach().double() * y.double()
    t_r = f.detach().double() * aty.double()
    lhs, rhs = float(t_l.sum()), float(t_r.sum())
    scale = max(float(t_l.abs().sum()), float(t_r.abs().sum()))
    print(f"fan map dot test: {abs(lhs - rhs) / scale:.2e} of the terms' magnitudes")
    assert abs(lhs - rhs) <= 1e-5 * scale, (lhs, rhs, scale)


def test_fan_map_fd_gradients():
    """L = ||FanFBP(f; h) - x_true||^2: gradients with respect to 16 random taps
    and 16 random fan-sinogram entries against FP64 central differences."""
    from risa_gb300 import phantom as ph_mod

    rng = np.random.default_rng(6)
    n, n_taps, W = 2, 48, 200.0
    sc = ph_mod.make_scan(n, 1, 500, 432, 215.0, 240.0, seed=12, distinct=n)
    ref = np.full((500, 432), 40200.0)
    fan = np.log((ref - 200.0) / np.maximum(sc.raw.astype(np.float64) - 200.0, 1.0)).astype(np.float32)
    taps = _ramp_taps(n_taps, rng)
    x_true = np.stack([ph_mod.rasterize(ph, 96, W) for ph in sc.phantoms]) * (W / 128) * (96 / 128)
    g = rg.make_geometry(**FAN)
    p = rg.make_params()
    f = torch.from_numpy(fan).cuda().requires_grad_(True)
    h = torch.from_numpy(taps).cuda().requires_grad_(True)
    y = FanFBPFunction.apply(f, h, g, p, 2)
    loss = ((y.double() - torch.from_numpy(x_true).cuda()) ** 2).sum()
    loss.backward()
    r = _fan_oracle_map(fan, taps.astype(np.float64)) - x_true
    eps = 1e-4
    # taps: L is quadratic in h
    idx = rng.choice(n_taps, size=16, replace=False)
    gh = h.grad.detach().cpu().numpy().astype(np.float64)
    fd = np.zeros(16)
    for i, j in enumerate(idx):
        e = np.zeros(n_taps)
        e[j] = 1.0
        aj = _fan_oracle_map(fan, e)
        fd[i] = (((r + eps * aj) ** 2).sum() - ((r - eps * aj) ** 2).sum()) / (2 * eps)
    err_h = np.abs(gh[idx] - fd).max() / np.abs(fd).max()
    # fan entries inside the rebinned field: L is quadratic in f
    gf = f.grad.detach().cpu().numpy().astype(np.float64)
    cand = np.argwhere(np.abs(gf) > 0.1 * np.abs(gf).max())
    picks = cand[rng.choice(len(cand), size=16, replace=False)]
    fd_f = np.zeros(16)
    for i, (b, a, k) in enumerate(picks):
        unit = np.zeros((1, 500, 432))
        unit[0, a, k] = 1.0
        au = _fan_oracle_map(unit, taps.astype(np.float64))[0]
        fd_f[i] = (((r[b] + eps * au) ** 2).sum() - ((r[b] - eps * au) ** 2).sum()) / (2 * eps)
    got_f = np.array([gf[b, a, k] for b, a, k in picks])
    err_f = np.abs(got_f - fd_f).max() / np.abs(fd_f).max()
    print(f"fan map gradients vs FP64 central differences: taps {err_h:.2e}, fan entries {err_f:.2e}")
    assert err_h < 1e-4, err_h
    assert err_f < 1e-4, err_f
