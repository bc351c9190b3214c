"""CPU oracle for the streaming FBP chain -- TEST INFRASTRUCTURE ONLY.

This package is the checker: only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may import it. It wraps the FP64 C
restatement in ``risa_oracle.c`` (see that file's header for the reference
functions it follows, file:line) through ctypes.

Parity is pinned by ``tests/golden``: fixtures produced by running the
reference's own host-side code (``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "librisa_oracle.so")

QUIRK_NONE = 0
QUIRK_RISA = 1
FILTERS = {"ramp": 0, "sheppLogan": 1, "cosine": 2, "hamming": 3, "hanning": 4}
BP_LINEAR, BP_NEAREST, BP_NEAREST_TRUNC = 0, 1, 2
MAX_PLANES = 4


def reference_root() -> str:
    """Where the reference checkout is looked for by the reference-side harness
    (oracle/ref_harness): RISA_REF_ROOT if set, else the path written in
    oracle/ref_harness/reference_root, the one place that names it."""
    env = os.environ.get("RISA_REF_ROOT")
    if env:
        return env
    with open(os.path.join(HERE, "ref_harness", "reference_root")) as f:
        return f.readline().strip()


def build(force: bool = False) -> str:
    """Compile risa_oracle.c into oracle/_build/librisa_oracle.so (gcc, no FMA contraction)."""
    src = os.path.join(HERE, "risa_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "risa_oracle.h"))
    ):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-o", tmp, src, "-lm", "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Geometry(ctypes.Structure):
    _fields_ = [
        ("n_planes", ctypes.c_int), ("n_fan_det", ctypes.c_int), ("n_fan_proj", ctypes.c_int),
        ("n_par_proj", ctypes.c_int), ("n_par_det", ctypes.c_int), ("n_pixels", ctypes.c_int),
        ("source_offset", ctypes.c_double), ("detector_diameter", ctypes.c_double),
        ("image_width", ctypes.c_double), ("image_center_x", ctypes.c_double),
        ("image_center_y", ctypes.c_double), ("rotation_offset", ctypes.c_double),
        ("source_diameter", ctypes.c_double * MAX_PLANES), ("delta_x", ctypes.c_double * MAX_PLANES),
        ("delta_z", ctypes.c_double * MAX_PLANES), ("source_angle", ctypes.c_double * MAX_PLANES),
    ]


class FbpParams(ctypes.Structure):
    _fields_ = [
        ("quirk", ctypes.c_int), ("filter_type", ctypes.c_int), ("cutoff", ctypes.c_double),
        ("pad", ctypes.c_int), ("interp", ctypes.c_int), ("defects", ctypes.c_int),
        ("thresh_min", ctypes.c_double), ("thresh_max", ctypes.c_double),
        ("masking", ctypes.c_int), ("masking_value", ctypes.c_double), ("normalize", ctypes.c_int),
    ]


class Records(ctypes.Structure):
    _fields_ = [
        ("n_planes", ctypes.c_int), ("n_rows360", ctypes.c_int), ("n_par_det", ctypes.c_int),
        ("n_fan_proj", ctypes.c_int), ("n_fan_det", ctypes.c_int),
        ("valid", ctypes.POINTER(ctypes.c_uint8)), ("tb", ctypes.POINTER(ctypes.c_int32)),
        ("gb", ctypes.POINTER(ctypes.c_int32)), ("u", ctypes.POINTER(ctypes.c_double)),
        ("v", ctypes.POINTER(ctypes.c_double)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        sig = {
            "orc_find_defects": (i, [vp, i, i, d, d, i, vp]),
            "orc_interpolate_defects": (i, [vp, vp, i, i, i]),
            "orc_reference_average": (None, [vp, i, i, i, i, i, vp]),
            "orc_dark_average": (None, [vp, i, i, i, i, i, vp]),
            "orc_attenuation_init": (i, [vp, i, vp, i, i, i, i, d, d, i, i, vp, vp]),
            "orc_relevant_area_mask": (None, [i, i, d, d, d] + [ctypes.c_uint] * 6 + [vp]),
            "orc_attenuation": (None, [vp, vp, vp, vp, i, i, vp]),
            "orc_f2p_tables_risa": (i, [vp] * 7),
            "orc_f2p_records_alloc": (i, [vp, vp]),
            "orc_f2p_records_free": (None, [vp]),
            "orc_f2p_records_build": (i, [vp, i, vp]),
            "orc_f2p_apply": (None, [vp, i, i, vp, vp]),
            "orc_filter_length": (i, [i, i, i]),
            "orc_design_filter": (i, [i, i, d, i, vp]),
            "orc_filter_rows": (i, [vp, i, i, i, vp]),
            "orc_backproject": (i, [vp, i, i, i, d, i, i, vp]),
            "orc_mask": (None, [vp, i, d, i]),
            "orc_fbp": (i, [vp, vp, vp, vp, vp, vp, vp, vp, i, vp, i]),
            "orc_fbp_parallel": (i, [vp, vp, vp, i, vp, i]),
            "orc_filter_rows_taps": (i, [vp, i, i, vp, i]),
            "orc_fbp_parallel_taps": (i, [vp, vp, vp, i, vp, i, vp, i]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def make_geometry(g) -> Geometry:
    """Build the ctypes geometry from any object with the geometry attributes."""
    out = Geometry()
    for name in ("n_planes", "n_fan_det", "n_fan_proj", "n_par_proj", "n_par_det", "n_pixels"):
        setattr(out, name, int(getattr(g, name)))
    for name in ("source_offset", "detector_diameter", "image_width", "image_center_x",
                 "image_center_y", "rotation_offset"):
        setattr(out, name, float(getattr(g, name)))
    for name in ("source_diameter", "delta_x", "delta_z", "source_angle"):
        vals = list(getattr(g, name))
        arr = getattr(out, name)
        for k in range(MAX_PLANES):
            arr[k] = float(vals[k] if k < len(vals) else vals[-1])
    return out


# ---------------------------------------------------------------------------- defects
def find_defects(frame: np.ndarray, thresh_min: float, thresh_max: float, quirk: int) -> np.ndarray:
    frame = np.ascontiguousarray(frame, dtype=np.uint16)
    P, D = frame.shape
    flags = np.zeros(D + 1, np.int32)
    _check(lib().orc_find_defects(_p(frame), P, D, thresh_min, thresh_max, quirk, _p(flags)), "find_defects")
    return flags


def interpolate_defects(frame: np.ndarray, flags: np.ndarray, quirk: int) -> np.ndarray:
    out = np.array(frame, dtype=np.uint16, copy=True, order="C")
    P, D = out.shape
    fl = np.zeros(D + 1, np.int32)
    fl[: min(len(flags), D + 1)] = flags[: D + 1]
    fl[D] = 0
    _check(lib().orc_interpolate_defects(_p(out), _p(fl), P, D, quirk), "interpolate_defects")
    return out


# ---------------------------------------------------------------------------- attenuation
def reference_average(frames: np.ndarray, n_frames: int, n_planes: int, quirk: int) -> np.ndarray:
    frames = np.ascontiguousarray(frames, dtype=np.uint16)
    P, D = frames.shape[-2:]
    avg = np.zeros((n_planes, P, D), np.float32)
    lib().orc_reference_average(_p(frames), n_frames, n_planes, P, D, quirk, _p(avg))
    return avg


def dark_average(frames: np.ndarray, n_frames: int, n_planes: int, quirk: int) -> np.ndarray:
    frames = np.ascontiguousarray(frames, dtype=np.uint16)
    P, D = frames.shape[-2:]
    dark = np.zeros((n_planes, D), np.float32)
    lib().orc_dark_average(_p(frames), n_frames, n_planes, P, D, quirk, _p(dark))
    return dark


def attenuation_init(ref_frames, dark_frames, n_planes, thresh_min, thresh_max, repair, quirk):
    """ref_frames: [n_ref*L, P, D] u16 (copied, then repaired); dark: [n_dark*L, P, D] or None."""
    ref = np.array(ref_frames, dtype=np.uint16, copy=True, order="C")
    P, D = ref.shape[-2:]
    n_ref = ref.shape[0] // n_planes
    dark = None if dark_frames is None else np.ascontiguousarray(dark_frames, dtype=np.uint16)
    n_dark = 0 if dark is None else dark.shape[0] // n_planes
    avg_ref = np.zeros((n_planes, P, D), np.float32)
    avg_dark = np.zeros((n_planes, D), np.float32)
    _check(lib().orc_attenuation_init(_p(ref), n_ref, _p(dark), n_dark, n_planes, P, D, thresh_min,
                                      thresh_max, int(repair), quirk, _p(avg_ref), _p(avg_dark)),
           "attenuation_init")
    return avg_ref, avg_dark


def relevant_area_mask(n_det, n_proj, source_offset, lower, upper, xa, xb, xc, xd, xe, xf):
    mask = np.zeros((n_proj, n_det), np.float32)
    lib().orc_relevant_area_mask(n_det, n_proj, source_offset, lower, upper, xa, xb, xc, xd, xe, xf, _p(mask))
    return mask


def attenuation(raw, ref_plane, dark_plane, mask=None) -> np.ndarray:
    raw = np.ascontiguousarray(raw, dtype=np.uint16)
    P, D = raw.shape
    ref_plane = np.ascontiguousarray(ref_plane, dtype=np.float32)
    dark_plane = np.ascontiguousarray(dark_plane, dtype=np.float32)
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    out = np.zeros((P, D), np.float64)
    lib().orc_attenuation(_p(raw), _p(ref_plane), _p(dark_plane), _p(m), P, D, _p(out))
    return out


# ---------------------------------------------------------------------------- fan2para
def f2p_tables_risa(geom):
    g = make_geometry(geom)
    L, Pf, Df, Pp2, Dp = g.n_planes, g.n_fan_proj, g.n_fan_det, 2 * g.n_par_proj, g.n_par_det
    n = L * Pp2 * Dp
    theta = np.zeros(Pf, np.float32); gamma = np.zeros(Df, np.float32)
    s = np.zeros(Dp, np.float32); alpha = np.zeros(Pp2, np.float32)
    itab = np.zeros(10 * n, np.int32); ftab = np.zeros(4 * n, np.float32)
    _check(lib().orc_f2p_tables_risa(ctypes.byref(g), _p(theta), _p(gamma), _p(s), _p(alpha),
                                     _p(itab), _p(ftab)), "f2p_tables_risa")
    return dict(theta=theta, gamma=gamma, s=s, alpha=alpha, itab=itab.reshape(10, n),
                ftab=ftab.reshape(4, n))


@dataclass
class F2PRecords:
    """Oracle rebinning records; arrays shaped [L, 2*Pp, Dp, 2]."""
    valid: np.ndarray
    tb: np.ndarray
    gb: np.ndarray
    u: np.ndarray
    v: np.ndarray
    _c: Records = field(repr=False, default=None)
    _g: Geometry = field(repr=False, default=None)

    def __del__(self):
        if self._c is not None and _lib is not None:
            _lib.orc_f2p_records_free(ctypes.byref(self._c))
            self._c = None


def f2p_records(geom, quirk) -> F2PRecords:
    g = make_geometry(geom)
    rec = Records()
    _check(lib().orc_f2p_records_alloc(ctypes.byref(rec), ctypes.byref(g)), "records_alloc")
    rc = lib().orc_f2p_records_build(ctypes.byref(g), quirk, ctypes.byref(rec))
    if rc != 0:
        lib().orc_f2p_records_free(ctypes.byref(rec))
        raise RuntimeError(f"oracle f2p_records_build failed with status {rc}")
    shape = (g.n_planes, 2 * g.n_par_proj, g.n_par_det, 2)
    n = int(np.prod(shape))

    def view(ptr, dt):
        return np.ctypeslib.as_array(ptr, shape=(n,)).view(dt).reshape(shape)

    return F2PRecords(valid=view(rec.valid, np.uint8), tb=view(rec.tb, np.int32),
                      gb=view(rec.gb, np.int32), u=view(rec.u, np.float64),
                      v=view(rec.v, np.float64), _c=rec, _g=g)


def f2p_apply(rec: F2PRecords, plane: int, quirk: int, fan: np.ndarray) -> np.ndarray:
    fan = np.ascontiguousarray(fan, dtype=np.float64)
    Pp = rec._c.n_rows360 // 2
    par = np.zeros((Pp, rec._c.n_par_det), np.float64)
    lib().orc_f2p_apply(ctypes.byref(rec._c), plane, quirk, _p(fan), _p(par))
    return par


# ---------------------------------------------------------------------------- filter
def filter_length(n_par_det: int, pad: int, quirk: int) -> int:
    n = lib().orc_filter_length(n_par_det, pad, quirk)
    if n < 0:
        raise ValueError(f"unsupported filter length for Dp={n_par_det}, pad={pad}")
    return n


def design_filter(length: int, filter_type: int, cutoff: float, quirk: int) -> np.ndarray:
    h = np.zeros(length // 2 + 1, np.float64)
    _check(lib().orc_design_filter(length, filter_type, cutoff, quirk, _p(h)), "design_filter")
    return h


def filter_rows(rows: np.ndarray, length: int, h: np.ndarray) -> np.ndarray:
    out = np.array(rows, dtype=np.float64, copy=True, order="C")
    R, Dp = out.shape
    h = np.ascontiguousarray(h, dtype=np.float64)
    _check(lib().orc_filter_rows(_p(out), R, Dp, length, _p(h)), "filter_rows")
    return out


# ---------------------------------------------------------------------------- backprojection
def backproject(sino: np.ndarray, n_pixels: int, rotation_offset: float = 0.0,
                interp: int = BP_LINEAR, quirk: int = QUIRK_NONE) -> np.ndarray:
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    Pp, Dp = sino.shape
    img = np.zeros((n_pixels, n_pixels), np.float64)
    _check(lib().orc_backproject(_p(sino), Pp, Dp, n_pixels, rotation_offset, interp, quirk, _p(img)),
           "backproject")
    return img


def mask(img: np.ndarray, value: float = 0.0, normalize: bool = False) -> np.ndarray:
    out = np.array(img, dtype=np.float64, copy=True, order="C")
    lib().orc_mask(_p(out), out.shape[0], value, int(normalize))
    return out


# ---------------------------------------------------------------------------- full chain
def make_params(quirk=QUIRK_NONE, filter_type="ramp", cutoff=1.0, pad=0, interp=BP_LINEAR,
                defects=False, thresh_min=0.67, thresh_max=1.5, masking=False,
                masking_value=0.0, normalize=False) -> FbpParams:
    p = FbpParams()
    p.quirk = quirk
    p.filter_type = FILTERS[filter_type] if isinstance(filter_type, str) else int(filter_type)
    p.cutoff = cutoff
    p.pad = pad
    p.interp = interp
    p.defects = int(defects)
    p.thresh_min = thresh_min
    p.thresh_max = thresh_max
    p.masking = int(masking)
    p.masking_value = masking_value
    p.normalize = int(normalize)
    return p


def fbp(geom, params: FbpParams, rec: F2PRecords, ref, dark, raw, planes, relevant_mask=None,
        n_threads: int = 0) -> np.ndarray:
    g = make_geometry(geom)
    raw = np.ascontiguousarray(raw, dtype=np.uint16)
    n = raw.shape[0]
    planes = np.ascontiguousarray(planes, dtype=np.int32)
    ref = np.ascontiguousarray(ref, dtype=np.float32)
    dark = np.ascontiguousarray(dark, dtype=np.float32)
    m = None if relevant_mask is None else np.ascontiguousarray(relevant_mask, dtype=np.float32)
    out = np.zeros((n, g.n_pixels, g.n_pixels), np.float64)
    _check(lib().orc_fbp(ctypes.byref(g), ctypes.byref(params), ctypes.byref(rec._c), _p(ref),
                         _p(dark), _p(m), _p(raw), _p(planes), n, _p(out), n_threads), "fbp")
    return out


def filter_rows_taps(rows: np.ndarray, taps: np.ndarray) -> np.ndarray:
    out = np.array(rows, dtype=np.float64, copy=True, order="C")
    R, Dp = out.shape
    t = np.ascontiguousarray(taps, dtype=np.float64)
    _check(lib().orc_filter_rows_taps(_p(out), R, Dp, _p(t), len(t)), "filter_rows_taps")
    return out


def fbp_parallel_taps(geom, params: FbpParams, sino: np.ndarray, taps: np.ndarray,
                      n_threads: int = 0) -> np.ndarray:
    """Filter by taps, backproject (and mask per params) parallel sinograms [n, Pp, Dp], FP64."""
    g = make_geometry(geom)
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    t = np.ascontiguousarray(taps, dtype=np.float64)
    n = sino.shape[0]
    out = np.zeros((n, g.n_pixels, g.n_pixels), np.float64)
    _check(lib().orc_fbp_parallel_taps(ctypes.byref(g), ctypes.byref(params), _p(sino), n, _p(t), len(t),
                                       _p(out), n_threads), "fbp_parallel_taps")
    return out


def fbp_parallel(geom, params: FbpParams, sino: np.ndarray, n_threads: int = 0) -> np.ndarray:
    g = make_geometry(geom)
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    n = sino.shape[0]
    out = np.zeros((n, g.n_pixels, g.n_pixels), np.float64)
    _check(lib().orc_fbp_parallel(ctypes.byref(g), ctypes.byref(params), _p(sino), n, _p(out),
                                  n_threads), "fbp_parallel")
    return out
