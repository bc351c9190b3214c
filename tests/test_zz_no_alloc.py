"""The allocation-free defect entry point, risa_gb_defects_enqueue_noalloc.

It serves callers that cannot allocate device memory while running (a
detector front-end that must not touch the CUDA allocator during acquisition,
or a plug-in whose host framework owns all device memory): its scratch is a
fixed 4 MiB array inside the library instead of a caller workspace. This test
calls it through the C ABI twice in a row, with different frames, and checks
flags and repaired frames bit for bit against risa_gb_defects_enqueue, the
workspace-taking entry point. It lives in its own file, collected last.
"""
import ctypes
import os

import numpy as np
import pytest

import risa_gb300 as rg

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "defects.npz")


def _frames(seed, P=200, D=432, batch=3):
    data = np.load(GOLDEN)
    base = [data["mid_frame"], data["wrap_frame"]]
    rng = np.random.default_rng(seed)
    out = []
    for b in range(batch):
        f = base[b % 2]
        f = np.resize(f, (P, D)).astype(np.int64)
        f = f + rng.integers(-40, 40, size=f.shape)
        out.append(np.clip(f, 0, 65535).astype(np.uint16))
    return np.stack(out)


@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
def test_noalloc_matches_workspace_entry_point(quirk):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = rg.lib()
    P, D, B = 200, 432, 3
    g = rg.make_geometry(n_fan_det=D, n_fan_proj=P)
    p = rg.make_params(quirks=quirk)
    ref_h = rg.Defects(g, p, max_batch=B)
    ws = torch.empty(ref_h.workspace_bytes(B), dtype=torch.uint8, device="cuda")
    for call, seed in enumerate((11, 12)):  # two calls in a row share the fixed scratch
        frames = _frames(seed, P, D, B)
        a = torch.from_numpy(frames.view(np.int16)).cuda()
        b = a.clone()
        fa = torch.zeros((B, D), dtype=torch.int32, device="cuda")
        fb = torch.full((B, D), -7, dtype=torch.int32, device="cuda")
        ref_h.enqueue(a, B, ws, flags_out=fa)
        st = lib.risa_gb_defects_enqueue_noalloc(ctypes.byref(g), ctypes.byref(p), b.data_ptr(), B,
                                                 fb.data_ptr(), None)
        assert st == 0, rg.last_error()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(fb.cpu().numpy(), fa.cpu().numpy(), err_msg=f"flags, call {call}")
        np.testing.assert_array_equal(b.cpu().numpy(), a.cpu().numpy(), err_msg=f"frames, call {call}")
        assert fa.cpu().numpy().any()


def test_noalloc_rejects_batches_beyond_the_fixed_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = rg.lib()
    g = rg.make_geometry(n_fan_det=1152, n_fan_proj=1000)
    p = rg.make_params()
    frames = torch.zeros((1,), dtype=torch.int16, device="cuda")
    st = lib.risa_gb_defects_enqueue_noalloc(ctypes.byref(g), ctypes.byref(p), frames.data_ptr(), 100000,
                                             None, None)
    assert st == -1 and "limit" in rg.last_error()
