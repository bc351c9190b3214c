"""The allocation-free defect entry point, risa_gb_defects_enqueue_noalloc.

It serves callers that cannot allocate device memory while running (a
detector front-end that must not touch the CUDA allocator during acquisition,
or a plug-in whose host framework owns all device memory): its scratch is a
fixed 4 MiB array inside the library instead of a caller workspace. These tests
call it through the C ABI twice in a row, with different frames, and check
flags and repaired frames bit for bit against risa_gb_defects_enqueue, the
workspace-taking entry point: contiguous and module-major frames, with and
without a flags output, and the largest batch the array holds. A child
process (no torch) repeats the comparison after a cudaDeviceReset, when the
library must set the new context up again. This file is collected last.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import risa_gb300 as rg

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "defects.npz")
SCRATCH_BYTES = 4 << 20


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


def _wide_frames(seed, P, D, batch):
    """Counts with dead (constant) columns and two flickering ones."""
    rng = np.random.default_rng(seed)
    base = 20000 + 8000 * np.sin(np.linspace(0, 6, D))[None, None, :] * np.cos(np.linspace(0, 3, P))[None, :, None]
    f = base.astype(np.float32) + 150 * rng.standard_normal((batch, P, D), dtype=np.float32)
    f[:, :, rng.choice(D, size=D // 100, replace=False)] = 17000
    flick = rng.choice(D, size=2, replace=False)
    f[:, :, flick] *= rng.uniform(0.3, 1.7, size=(batch, P, 2))
    return np.clip(f, 0, 65535).astype(np.uint16)


def _compare_two_calls(g, p, B, make, with_flags=True):
    lib = rg.lib()
    D = g.n_fan_det
    ref_h = rg.Defects(g, p, max_batch=B)
    ws = torch.empty(ref_h.workspace_bytes(B), dtype=torch.uint8, device="cuda")
    for call, seed in enumerate((11, 12)):  # two calls in a row share the fixed scratch
        frames = make(seed)
        a = torch.from_numpy(frames.view(np.int16)).cuda()
        b = a.clone()
        fa = torch.zeros((B, D), dtype=torch.int32, device="cuda")
        fb = torch.full((B, D), -7, dtype=torch.int32, device="cuda")
        ref_h.enqueue(a, B, ws, flags_out=fa)
        st = lib.risa_gb_defects_enqueue_noalloc(ctypes.byref(g), ctypes.byref(p), b.data_ptr(), B,
                                                 fb.data_ptr() if with_flags else None, None)
        assert st == 0, rg.last_error()
        torch.cuda.synchronize()
        if with_flags:
            np.testing.assert_array_equal(fb.cpu().numpy(), fa.cpu().numpy(), err_msg=f"flags, call {call}")
        np.testing.assert_array_equal(b.cpu().numpy(), a.cpu().numpy(), err_msg=f"frames, call {call}")
        assert fa.cpu().numpy().any()
        assert (a.cpu().numpy() != frames.view(np.int16)).any(), "nothing was repaired"


@pytest.fixture(autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
def test_noalloc_matches_workspace_entry_point(quirk):
    P, D, B = 200, 432, 3
    _compare_two_calls(rg.make_geometry(n_fan_det=D, n_fan_proj=P), rg.make_params(quirks=quirk), B,
                       lambda s: _frames(s, P, D, B))


@pytest.mark.parametrize("quirk", [rg.QUIRKS_RISA, rg.QUIRKS_NONE])
def test_noalloc_module_major_frames(quirk):
    """Module-major frames (27 modules of 16 detectors) take the scalar statistics kernel."""
    P, D, B = 200, 432, 3
    g = rg.make_geometry(n_fan_det=D, n_fan_proj=P, n_modules=27)
    _compare_two_calls(g, rg.make_params(quirks=quirk, module_major=True), B,
                       lambda s: rg.to_module_major(_frames(s, P, D, B), 27))


def test_noalloc_without_flags_output():
    P, D, B = 200, 432, 3
    _compare_two_calls(rg.make_geometry(n_fan_det=D, n_fan_proj=P), rg.make_params(), B,
                       lambda s: _frames(s, P, D, B), with_flags=False)


def test_noalloc_largest_batch_that_fits():
    """1000 x 1152 frames: the largest batch whose scratch fits the 4 MiB array."""
    P, D = 1000, 1152
    g = rg.make_geometry(n_fan_det=D, n_fan_proj=P)
    p = rg.make_params()
    h = rg.Defects(g, p, max_batch=4096)
    B = 1
    while h.workspace_bytes(B + 1) <= SCRATCH_BYTES:
        B += 1
    assert B >= 150, B
    _compare_two_calls(g, p, B, lambda s: _wide_frames(s, P, D, B))
    lib = rg.lib()
    frames = torch.zeros((B + 1, P, D), dtype=torch.int16, device="cuda")
    st = lib.risa_gb_defects_enqueue_noalloc(ctypes.byref(g), ctypes.byref(p), frames.data_ptr(), B + 1,
                                             None, None)
    assert st == -1 and "limit" in rg.last_error()


def test_noalloc_rejects_batches_beyond_the_fixed_scratch():
    lib = rg.lib()
    g = rg.make_geometry(n_fan_det=1152, n_fan_proj=1000)
    p = rg.make_params()
    frames = torch.zeros((1,), dtype=torch.int16, device="cuda")
    st = lib.risa_gb_defects_enqueue_noalloc(ctypes.byref(g), ctypes.byref(p), frames.data_ptr(), 100000,
                                             None, None)
    assert st == -1 and "limit" in rg.last_error()


def test_noalloc_after_device_reset():
    """The set-up is redone in the context the runtime builds after cudaDeviceReset
    (a pipeline's main may reset the device between scans); checked in a child
    process that holds no torch memory."""
    env = dict(os.environ)
    env.pop("CUDA_LAUNCH_BLOCKING", None)
    res = subprocess.run([sys.executable, os.path.join(HERE, "noalloc_reset_child.py")], capture_output=True,
                         text=True, timeout=300, env=env)
    assert res.returncode == 0 and res.stdout.strip().endswith("ok"), res.stdout + res.stderr
