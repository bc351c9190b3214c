"""Child process of test_zz_no_alloc.py: the allocation-free defect entry point
across a device reset.

It runs without torch (a process whose torch allocator holds device memory
must not reset the device) and drives the CUDA runtime the library links
through ctypes. In each of two CUDA contexts -- the first one and the one the
runtime builds after cudaDeviceReset -- it calls
risa_gb_defects_enqueue_noalloc first and only then creates a
risa_gb_defects handle, so the allocation-free call depends on its own
per-context set-up (array address, threshold constants, the flagging kernel's
shared-memory limit), and compares flags and repaired frames bit for bit.
Between the reset and those calls it checks that a call needing set-up while
its stream is capturing is refused without launching anything. Prints "ok".
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import risa_gb300 as rg  # noqa: E402

H2D, D2H = 1, 2
CAPTURE_RELAXED = 2


def cudart():
    rg.lib()  # loads the runtime the library links; open the same file
    for line in open("/proc/self/maps"):
        path = line.split()[-1]
        if "libcudart.so" in path:
            return ctypes.CDLL(path)
    raise RuntimeError("libcudart not mapped")


RT = None


def ck(rc, what):
    if rc != 0:
        RT.cudaGetErrorString.restype = ctypes.c_char_p
        raise RuntimeError(f"{what}: {RT.cudaGetErrorString(rc).decode()}")


def dmalloc(n):
    p = ctypes.c_void_p()
    ck(RT.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(n)), "cudaMalloc")
    return p.value


def upload(a):
    d = dmalloc(a.nbytes)
    ck(RT.cudaMemcpy(ctypes.c_void_p(d), a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes), H2D),
       "cudaMemcpy H2D")
    return d


def download(d, shape, dtype):
    out = np.empty(shape, dtype)
    ck(RT.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(d), ctypes.c_size_t(out.nbytes), D2H),
       "cudaMemcpy D2H")
    return out


def frames(seed, P, D, B):
    """Counts with dead (constant) and flickering columns, so both kinds of flag occur."""
    rng = np.random.default_rng(seed)
    base = 20000 + 8000 * np.sin(np.linspace(0, 6, D))[None, None, :] * np.cos(np.linspace(0, 3, P))[None, :, None]
    f = base + rng.normal(0, 150, size=(B, P, D))
    dead = rng.choice(D, size=max(2, D // 100), replace=False)
    f[:, :, dead] = 17000
    flick = rng.choice(D, size=2, replace=False)
    f[:, :, flick] *= rng.uniform(0.3, 1.7, size=(B, P, 2))
    return np.clip(f, 0, 65535).astype(np.uint16)


def compare(P, D, B, quirk, seed):
    lib = rg.lib()
    g = rg.make_geometry(n_fan_det=D, n_fan_proj=P)
    p = rg.make_params(quirks=quirk)
    fr = frames(seed, P, D, B)
    da, db = upload(fr), upload(fr)
    fa, fb = dmalloc(B * D * 4), dmalloc(B * D * 4)
    st = lib.risa_gb_defects_enqueue_noalloc(ctypes.byref(g), ctypes.byref(p), db, B, fb, None)
    if st != 0:
        raise RuntimeError(f"noalloc call failed: {rg.last_error()}")
    ck(RT.cudaDeviceSynchronize(), "sync after noalloc")
    got_f, got_x = download(fb, (B, D), np.int32), download(db, fr.shape, np.uint16)
    h = rg.Defects(g, p, max_batch=B)
    ws = dmalloc(max(1, h.workspace_bytes(B)))
    h.enqueue(da, B, ws, flags_out=fa)
    ck(RT.cudaDeviceSynchronize(), "sync after handle path")
    exp_f, exp_x = download(fa, (B, D), np.int32), download(da, fr.shape, np.uint16)
    np.testing.assert_array_equal(got_f, exp_f, err_msg=f"flags P={P} D={D}")
    np.testing.assert_array_equal(got_x, exp_x, err_msg=f"frames P={P} D={D}")
    assert exp_f.any(), "no defect flagged: the case does not exercise the thresholds"
    assert (got_x != fr).any(), "nothing repaired"
    del h
    for d in (da, db, fa, fb, ws):
        ck(RT.cudaFree(ctypes.c_void_p(d)), "cudaFree")


def refused_while_capturing():
    """After a reset the set-up is due; a call on a capturing stream must refuse."""
    lib = rg.lib()
    P, D, B = 64, 432, 1
    g = rg.make_geometry(n_fan_det=D, n_fan_proj=P)
    p = rg.make_params()
    d = upload(frames(5, P, D, B))
    s = ctypes.c_void_p()
    ck(RT.cudaStreamCreate(ctypes.byref(s)), "cudaStreamCreate")
    ck(RT.cudaStreamBeginCapture(s, CAPTURE_RELAXED), "cudaStreamBeginCapture")
    st = lib.risa_gb_defects_enqueue_noalloc(ctypes.byref(g), ctypes.byref(p), d, B, None, s)
    graph = ctypes.c_void_p()
    ck(RT.cudaStreamEndCapture(s, ctypes.byref(graph)), "cudaStreamEndCapture")
    n = ctypes.c_size_t(99)
    ck(RT.cudaGraphGetNodes(graph, None, ctypes.byref(n)), "cudaGraphGetNodes")
    ck(RT.cudaGraphDestroy(graph), "cudaGraphDestroy")
    ck(RT.cudaStreamDestroy(s), "cudaStreamDestroy")
    ck(RT.cudaFree(ctypes.c_void_p(d)), "cudaFree")
    assert st == -2 and "capturing" in rg.last_error(), (st, rg.last_error())
    assert n.value == 0, f"{n.value} nodes captured by a refused call"


def main():
    global RT
    RT = cudart()
    ck(RT.cudaSetDevice(0), "cudaSetDevice")
    cases = [(200, 432, 3, rg.QUIRKS_RISA, 1), (64, 4608, 2, rg.QUIRKS_NONE, 2)]
    for c in cases:
        compare(*c)
    ck(RT.cudaDeviceReset(), "cudaDeviceReset")
    ck(RT.cudaSetDevice(0), "cudaSetDevice after reset")
    refused_while_capturing()
    for P, D, B, q, seed in cases:
        compare(P, D, B, q, seed + 10)
    print("ok")


if __name__ == "__main__":
    main()
