"""TEST INFRASTRUCTURE: the reference's own CUDA kernels on the GPU.

oracle/ref_harness/build_ref.sh compiles the reference's stage sources
(RISA/risaLib/src/{Attenuation,Fan2Para,Filter,Backprojection,Masking,
Reordering}/*.cu) to sm_103a cubins in oracle/_ref/; build_launch.sh builds
ref_launch.c, which loads them with the driver API and launches each kernel
with the grid, block and __constant__ set-up of the reference's processor()
loop. The GPU tests run these kernels and this library's kernels on the same
device buffers. Only tests import this module.

Arguments are torch CUDA tensors (device pointers are taken from them).
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "librisa_ref_launch.so")
CUBINS = ("risa_attenuation", "risa_fan2para", "risa_filter", "risa_backprojection", "risa_masking",
          "risa_reordering")

_lib: Optional[ctypes.CDLL] = None


def unavailable() -> Optional[str]:
    """Why the reference kernels cannot run here, or None."""
    missing = [c for c in CUBINS if not os.path.exists(os.path.join(REF_DIR, c + ".cubin"))]
    if missing:
        return "reference cubins not built (oracle/ref_harness/build_ref.sh needs the reference tree)"
    if not os.path.exists(LIB):
        return "launcher not built (oracle/ref_harness/build_launch.sh)"
    return None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        why = unavailable()
        if why:
            raise RuntimeError(why)
        l = ctypes.CDLL(LIB)
        vp, i, f, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint64
        l.rr_error.restype = ctypes.c_char_p
        l.rr_init.argtypes = [ctypes.c_char_p]
        l.rr_attenuation.argtypes = [u64] * 5 + [i] * 4 + [vp]
        l.rr_fan2para.argtypes = [i] + [u64] * 6 + [ctypes.POINTER(u64), u64, i, i, i, vp]
        l.rr_filter.argtypes = [u64, u64, u64, i, i, i, vp]
        l.rr_bp_constants.argtypes = [vp, vp, i, f, f, f]
        l.rr_backproject.argtypes = [i, u64, u64, i, i, i, i, vp]
        l.rr_mask.argtypes = [u64, f, i, vp]
        l.rr_reorder.argtypes = [u64, u64, u64, i, i, vp]
        if l.rr_init(REF_DIR.encode()) != 0:
            raise RuntimeError("reference kernels: " + l.rr_error().decode())
        _lib = l
    return _lib


def bp_setup(n_proj: int, n_det: int, n_pixels: int, rotation_offset: float = 0.0):
    """The host set-up of Backprojection::processor (Backprojection.cu:118-138):
    (sin table, cos table, norm, scale, center) with the reference's float steps."""
    import numpy as np

    sin_t = np.zeros(n_proj, np.float32)
    cos_t = np.zeros(n_proj, np.float32)
    for i in range(n_proj):
        th = np.float32(i * np.pi / float(np.float32(n_proj)) + float(np.float32(rotation_offset)) / 180.0 * np.pi)
        while th < 0.0:
            th = np.float32(float(th) + 2.0 * np.pi)
        sin_t[i] = np.float32(np.sin(np.float64(th)))
        cos_t[i] = np.float32(np.cos(np.float64(th)))
    scale = np.float32(n_det / float(np.float32(n_pixels)))
    norm = np.float32(np.pi / n_proj / float(scale))
    center = np.float32((n_pixels - 1.0) * 0.5)
    return sin_t, cos_t, float(norm), float(scale), float(center)


def fan2para_inputs(geom: dict, z: dict, block: int = 16) -> dict:
    """Device inputs of the reference's interpolation kernel for a geometry and its
    reference-layout tables z (theta, gamma, s, alpha, itab[10], ftab[4], as the
    reference's computeFan2ParaTransp writes them). The kernel reads the tables
    without bounds checks and its own bounds test lets threads past the edge
    run unless the grid covers the sinogram exactly, so both are checked here
    on the CPU before anything reaches the GPU."""
    import numpy as np
    import torch

    L, Pf, Df = geom["n_planes"], geom["n_fan_proj"], geom["n_fan_det"]
    Pp2, Dp = 2 * geom["n_par_proj"], geom["n_par_det"]
    itab, ftab = z["itab"], z["ftab"]
    if itab.shape != (10, L * Pp2 * Dp) or ftab.shape != (4, L * Pp2 * Dp):
        raise ValueError("fan2para tables do not match the geometry")
    if Dp % block or Pp2 % block:
        raise ValueError("the reference kernel's grid must cover the sinogram exactly")
    if not (len(z["gamma"]) == Df and len(z["theta"]) == Pf and len(z["s"]) == Dp and len(z["alpha"]) == Pp2):
        raise ValueError("fan2para axis tables do not match the geometry")
    for r in (0, 1):
        on = itab[8 + r] != 0
        for row, lim in ((0 + r, Pf), (2 + r, Pf), (4 + r, Df), (6 + r, Df)):
            v = itab[row][on]
            if v.size and (v.min() < 0 or v.max() >= lim):
                raise ValueError("fan2para table index out of range")

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    order = [itab[0], itab[1], itab[2], itab[3], itab[6], itab[7], itab[4], itab[5],
             ftab[0], ftab[1], ftab[2], ftab[3], itab[8], itab[9]]
    params = np.zeros(11, np.int32)
    params[:5] = (L, Df, Pf, Pp2, Dp)
    params[5:].view(np.float32)[:] = (geom["source_offset"], geom["detector_diameter"],
                                      geom["detector_diameter"] / 2.0, geom.get("image_center_x", 0.0),
                                      geom.get("image_center_y", 0.0), geom["image_width"])
    return dict(tables=[dev(t) for t in order], params=dev(params), gamma=dev(z["gamma"]), theta=dev(z["theta"]),
                alpha=dev(z["alpha"]), s=dev(z["s"]), n_par_det=Dp, n_par_proj360=Pp2, block=block)


def fan2para_run(plane: int, fan, par, inp: dict):
    """One launch of the reference's interpolation kernel with fan2para_inputs();
    par ([2 Pp][Dp] floats) must be zeroed first, as the reference's setValue does."""
    fan2para(plane, fan, par, inp["gamma"], inp["theta"], inp["alpha"], inp["s"], inp["tables"], inp["params"],
             inp["n_par_det"], inp["n_par_proj360"], inp["block"])


def _ck(rc: int):
    if rc != 0:
        raise RuntimeError("reference kernels: " + lib().rr_error().decode())


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def attenuation(raw, mask, out, ref_avg, dark_avg, n_det: int, n_proj: int, plane: int, block: int = 16):
    _ck(lib().rr_attenuation(raw.data_ptr(), mask.data_ptr(), out.data_ptr(), ref_avg.data_ptr(),
                             dark_avg.data_ptr(), n_det, n_proj, plane, block, _stream()))


def fan2para(plane: int, fan, par, gamma, theta, alpha, s, tables, params, n_par_det: int,
             n_par_proj360: int, block: int = 16):
    """tables: 14 tensors in the kernel's argument order (ref_launch.c)."""
    arr = (ctypes.c_uint64 * 14)(*[t.data_ptr() for t in tables])
    _ck(lib().rr_fan2para(plane, fan.data_ptr(), par.data_ptr(), gamma.data_ptr(), theta.data_ptr(),
                          alpha.data_ptr(), s.data_ptr(), arr, params.data_ptr(), n_par_det, n_par_proj360,
                          block, _stream()))


def filter_rows(sino, freq, filt, n_det: int, n_rows: int, block: int = 16):
    _ck(lib().rr_filter(sino.data_ptr(), freq.data_ptr(), filt.data_ptr(), n_det, n_rows, block, _stream()))


def bp_constants(sin_tab, cos_tab, n_proj: int, norm: float, scale: float, center: float):
    import numpy as np

    s = np.ascontiguousarray(sin_tab, np.float32)
    c = np.ascontiguousarray(cos_tab, np.float32)
    _ck(lib().rr_bp_constants(s.ctypes.data, c.ctypes.data, n_proj, norm, scale, center))


def backproject(nearest: bool, sino, img, n_pixels: int, n_proj: int, n_det: int, block: int = 16):
    _ck(lib().rr_backproject(int(nearest), sino.data_ptr(), img.data_ptr(), n_pixels, n_proj, n_det, block,
                             _stream()))


def mask(img, value: float, n_pixels: int):
    _ck(lib().rr_mask(img.data_ptr(), value, n_pixels, _stream()))


def reorder(inp, out, table, n_proj: int, n_det: int):
    _ck(lib().rr_reorder(inp.data_ptr(), out.data_ptr(), table.data_ptr(), n_proj, n_det, _stream()))
