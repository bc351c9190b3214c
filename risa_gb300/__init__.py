"""GB300-native streaming FBP chain (the reference's Attenuation -> DetectorInterpolation
-> Fan2Para -> Filter -> Backprojection -> Masking stages), Python access to the C ABI.

The compute lives in ``_build/librisa_gb300.so`` (sm_103a kernels behind the
C ABI declared in ``include/risa_gb300.h``). This module only marshals
geometry/parameter structs and device pointers (``int`` addresses or
objects with ``data_ptr()``, e.g. torch tensors) through ctypes. There is no
CPU fallback: if the library is missing, importing the stage classes fails.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "librisa_gb300.so")

QUIRKS_NONE, QUIRKS_RISA = 0, 1
FILTER_RAMP, FILTER_SHEPP_LOGAN, FILTER_COSINE, FILTER_HAMMING, FILTER_HANNING = range(5)
FILTERS = {"ramp": 0, "sheppLogan": 1, "cosine": 2, "hamming": 3, "hanning": 4}
INTERP_LINEAR, INTERP_NEAREST, INTERP_NEAREST_TRUNC = 0, 1, 2
PLANES_INTERLEAVED = -1
SPLIT_BF16X3, SPLIT_F16X3 = 0, 1
MAX_PLANES = 4

STATUS = {0: "ok", -1: "invalid argument", -2: "unsupported", -3: "CUDA error", -4: "timed out",
          -5: "out of memory", -6: "configuration error"}


class RisaError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str):
        super().__init__(f"{what}: {STATUS.get(status, status)} ({detail})")
        self.status = status


class Geometry(ctypes.Structure):
    """Mirror of risa_gb_geometry (config keys of the reference's config.cfg)."""
    _fields_ = [
        ("struct_size", ctypes.c_uint32), ("n_planes", ctypes.c_int32), ("n_fan_det", ctypes.c_int32),
        ("n_fan_proj", ctypes.c_int32), ("n_par_proj", ctypes.c_int32), ("n_par_det", ctypes.c_int32),
        ("n_pixels", ctypes.c_int32), ("n_modules", ctypes.c_int32),
        ("source_offset", ctypes.c_double), ("detector_diameter", ctypes.c_double),
        ("image_width", ctypes.c_double), ("image_center_x", ctypes.c_double),
        ("image_center_y", ctypes.c_double), ("rotation_offset", ctypes.c_double),
        ("source_diameter", ctypes.c_double * MAX_PLANES), ("delta_x", ctypes.c_double * MAX_PLANES),
        ("delta_z", ctypes.c_double * MAX_PLANES), ("source_angle", ctypes.c_double * MAX_PLANES),
    ]


class SweepInstance(ctypes.Structure):
    """Mirror of risa_gb_sweep_instance."""
    _fields_ = [
        ("n_pixels", ctypes.c_int32), ("n_par_proj", ctypes.c_int32), ("n_par_det", ctypes.c_int32),
        ("filter_type", ctypes.c_int32), ("cutoff", ctypes.c_double), ("rotation_offset", ctypes.c_double),
        ("ref_level", ctypes.c_double), ("dark_level", ctypes.c_double), ("masking", ctypes.c_int32),
        ("masking_value", ctypes.c_double), ("defect_map", ctypes.c_void_p),
    ]


class Params(ctypes.Structure):
    """Mirror of risa_gb_params."""
    _fields_ = [
        ("struct_size", ctypes.c_uint32), ("quirks", ctypes.c_int32), ("filter_type", ctypes.c_int32),
        ("cutoff", ctypes.c_double), ("pad", ctypes.c_int32), ("interp", ctypes.c_int32),
        ("defects", ctypes.c_int32), ("thresh_min", ctypes.c_double), ("thresh_max", ctypes.c_double),
        ("relevant_mask", ctypes.c_int32), ("lower_lim_offset", ctypes.c_double),
        ("upper_lim_offset", ctypes.c_double),
        ("xa", ctypes.c_uint32), ("xb", ctypes.c_uint32), ("xc", ctypes.c_uint32),
        ("xd", ctypes.c_uint32), ("xe", ctypes.c_uint32), ("xf", ctypes.c_uint32),
        ("masking", ctypes.c_int32), ("masking_value", ctypes.c_double), ("normalize", ctypes.c_int32),
        ("repair_reference", ctypes.c_int32), ("module_major", ctypes.c_int32),
    ]


# Every exported symbol of include/risa_gb300.h with its ctypes signature.
_vp, _i, _sz, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_double
_pp = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "risa_gb_params_init": (_i, [_vp]),
    "risa_gb_geometry_init": (_i, [_vp]),
    "risa_gb_last_error": (ctypes.c_char_p, []),
    "risa_gb_version": (ctypes.c_char_p, []),
    "risa_gb_config_load": (_i, [ctypes.c_char_p, _vp, _vp]),
    "risa_gb_config_lookup": (_i, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _sz]),
    "risa_gb_reorder_enqueue": (_i, [_vp, _vp, _i, _i, _i, _i, _vp]),
    "risa_gb_defects_create": (_i, [_vp, _vp, _i, _pp]),
    "risa_gb_defects_workspace_bytes": (_sz, [_vp, _i]),
    "risa_gb_defects_enqueue": (_i, [_vp, _vp, _i, _vp, _vp, _vp]),
    "risa_gb_defects_destroy": (_i, [_vp]),
    "risa_gb_defects_enqueue_noalloc": (_i, [_vp, _vp, _vp, _i, _vp, _vp]),
    "risa_gb_attenuation_create": (_i, [_vp, _vp, _vp, _i, _vp, _i, _pp]),
    "risa_gb_attenuation_enqueue": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "risa_gb_attenuation_tables": (_i, [_vp, _vp, _vp]),
    "risa_gb_attenuation_destroy": (_i, [_vp]),
    "risa_gb_fan2para_create": (_i, [_vp, _vp, _pp]),
    "risa_gb_fan2para_enqueue": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "risa_gb_fan2para_enqueue_adjoint": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "risa_gb_fan2para_destroy": (_i, [_vp]),
    "risa_gb_fan2para_tables_host": (_i, [_vp, _vp, _i, _vp, _vp, _vp]),
    "risa_gb_fan2para_staged_tables_host": (_i, [_vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_int)]),
    "risa_gb_filter_create": (_i, [_vp, _vp, _pp]),
    "risa_gb_filter_enqueue": (_i, [_vp, _vp, _i, _vp]),
    "risa_gb_filter_response": (_i, [_vp, ctypes.POINTER(ctypes.c_int), _vp]),
    "risa_gb_filter_destroy": (_i, [_vp]),
    "risa_gb_filter_design_host": (_i, [_vp, _vp, ctypes.POINTER(ctypes.c_int), _vp]),
    "risa_gb_filter_create_taps": (_i, [_vp, _vp, _vp, _i, _pp]),
    "risa_gb_filter_enqueue_adjoint": (_i, [_vp, _vp, _i, _vp]),
    "risa_gb_filter_taps_grad_workspace_bytes": (_sz, [_vp, _i]),
    "risa_gb_filter_taps_grad": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _vp]),
    "risa_gb_toeplitz_create": (_i, [_vp, _vp, _pp]),
    "risa_gb_toeplitz_workspace_bytes": (_sz, [_vp, _i]),
    "risa_gb_toeplitz_enqueue": (_i, [_vp, _vp, _i, _vp, _vp]),
    "risa_gb_toeplitz_check": (_i, [_vp]),
    "risa_gb_toeplitz_destroy": (_i, [_vp]),
    "risa_gb_toeplitz_set_precision": (_i, [_vp, _i]),
    "risa_gb_backprojection_create": (_i, [_vp, _vp, _pp]),
    "risa_gb_backprojection_enqueue": (_i, [_vp, _vp, _vp, _i, _vp]),
    "risa_gb_backprojection_enqueue_adjoint": (_i, [_vp, _vp, _vp, _i, _vp]),
    "risa_gb_backprojection_autotune": (_i, [_vp, _vp, _vp, _i, _vp, ctypes.POINTER(ctypes.c_int)]),
    "risa_gb_backprojection_set_variant": (_i, [_vp, _i]),
    "risa_gb_backprojection_variant_count": (_i, []),
    "risa_gb_backprojection_check": (_i, [_vp]),
    "risa_gb_backprojection_reserve": (_i, [_vp, _i]),
    "risa_gb_backprojection_reserve_adjoint": (_i, [_vp, _i]),
    "risa_gb_backprojection_variant_name": (ctypes.c_char_p, [_i]),
    "risa_gb_backprojection_window": (_i, [_vp, _i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "risa_gb_backprojection_time": (_i, [_vp, _vp, _vp, _i, _i, _vp, ctypes.POINTER(ctypes.c_float),
                                         ctypes.POINTER(ctypes.c_float)]),
    "risa_gb_backprojection_destroy": (_i, [_vp]),
    "risa_gb_masking_create": (_i, [_vp, _vp, _pp]),
    "risa_gb_masking_workspace_bytes": (_sz, [_vp, _i]),
    "risa_gb_masking_enqueue": (_i, [_vp, _vp, _i, _vp, _vp]),
    "risa_gb_masking_destroy": (_i, [_vp]),
    "risa_gb_fbp_create": (_i, [_vp, _vp, _vp, _i, _vp, _i, _i, _pp]),
    "risa_gb_fbp_enqueue": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "risa_gb_fbp_graph_capture": (_i, [_vp, _vp, _vp, _i, _i, _vp, _pp]),
    "risa_gb_graph_replay": (_i, [_vp, _vp]),
    "risa_gb_graph_kernel_count": (_i, [_vp]),
    "risa_gb_graph_destroy": (_i, [_vp]),
    "risa_gb_fbp_run_host": (_i, [_vp, _vp, _vp, _i, _i]),
    "risa_gb_fbp_intermediates": (_i, [_vp, _pp, _pp]),
    "risa_gb_fbp_backprojection": (_vp, [_vp]),
    "risa_gb_fbp_destroy": (_i, [_vp]),
    "risa_gb_fbp_time_stages": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp, _vp]),
    "risa_gb_sweep_create": (_i, [_vp, _i, _pp]),
    "risa_gb_sweep_layout": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "risa_gb_sweep_enqueue": (_i, [_vp, _vp, _vp, _vp]),
    "risa_gb_sweep_times": (_i, [_vp, _vp, _vp, _vp]),
    "risa_gb_sweep_check": (_i, [_vp]),
    "risa_gb_sweep_grid": (_i, [_vp]),
    "risa_gb_measure_peak": (_i, [_i, _i, _vp, ctypes.POINTER(ctypes.c_double)]),
    "risa_gb_fbp_set_lanes": (_i, [_vp, _i]),
    "risa_gb_sweep_graph_capture": (_i, [_vp, _vp, _vp, _vp, _pp]),
    "risa_gb_assembler_create": (_i, [_vp, _vp, _i, _i, _pp]),
    "risa_gb_assembler_ingest": (_i, [_vp, _i, ctypes.c_char_p, _sz]),
    "risa_gb_assembler_next": (_i, [_vp, _d, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int)]),
    "risa_gb_assembler_release": (_i, [_vp, ctypes.c_uint64]),
    "risa_gb_assembler_finish": (_i, [_vp]),
    "risa_gb_assembler_stats": (_i, [_vp, _vp, _vp, _vp]),
    "risa_gb_assembler_destroy": (_i, [_vp]),
    "risa_gb_sweep_destroy": (_i, [_vp]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load librisa_gb300.so (built by ``__graft_entry__.build()`` / ``risa_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m risa_gb300.build` "
                              "(there is no CPU fallback)")
        _lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def last_error() -> str:
    return lib().risa_gb_last_error().decode()


def _check(status: int, what: str):
    if status != 0:
        raise RisaError(status, what, last_error())


def _nbytes(x) -> Optional[int]:
    """Bytes reachable from the address of a tensor or array (None for raw addresses)."""
    if hasattr(x, "untyped_storage"):  # torch: from this view's start to its storage's end
        return x.untyped_storage().nbytes() - x.storage_offset() * x.element_size()
    if hasattr(x, "nbytes"):
        return int(x.nbytes)
    return None


def _need(x, nbytes: int, what: str):
    """Raise before a launch that would read or write past a tensor or array."""
    have = None if x is None or isinstance(x, int) else _nbytes(x)
    if have is not None and have < nbytes:
        raise RisaError(-1, what, f"buffer holds {have} bytes, the call needs {nbytes}")


def ptr(x) -> Optional[int]:
    """Device/host address of an int, a torch tensor, a numpy array or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)}")


def stream_ptr(stream) -> Optional[int]:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def make_geometry(n_planes=1, n_fan_det=432, n_fan_proj=500, n_par_proj=256, n_par_det=256,
                  n_pixels=256, n_modules=27, source_offset=0.0, detector_diameter=480.0,
                  image_width=200.0, image_center_x=0.0, image_center_y=0.0, rotation_offset=0.0,
                  source_diameter: Sequence[float] = (430.0,), delta_x: Sequence[float] = (0.0,),
                  delta_z: Sequence[float] = (1417.0,), source_angle: Sequence[float] = (360.0,)) -> Geometry:
    g = Geometry()
    lib().risa_gb_geometry_init(ctypes.byref(g))
    g.n_planes, g.n_fan_det, g.n_fan_proj = n_planes, n_fan_det, n_fan_proj
    g.n_par_proj, g.n_par_det, g.n_pixels, g.n_modules = n_par_proj, n_par_det, n_pixels, n_modules
    g.source_offset, g.detector_diameter, g.image_width = source_offset, detector_diameter, image_width
    g.image_center_x, g.image_center_y, g.rotation_offset = image_center_x, image_center_y, rotation_offset
    for name, vals in (("source_diameter", source_diameter), ("delta_x", delta_x),
                       ("delta_z", delta_z), ("source_angle", source_angle)):
        arr = getattr(g, name)
        vals = list(vals)
        for k in range(MAX_PLANES):
            arr[k] = float(vals[min(k, len(vals) - 1)])
    return g


def make_params(quirks=QUIRKS_NONE, filter_type="ramp", cutoff=1.0, pad=0, interp=INTERP_LINEAR,
                defects=False, thresh_min=0.67, thresh_max=1.5, relevant_mask=False,
                lower_lim_offset=0.0, upper_lim_offset=0.0, fix_points=(0, 0, 0, 0, 0, 0),
                masking=False, masking_value=0.0, normalize=False, repair_reference=True,
                module_major=False) -> Params:
    p = Params()
    lib().risa_gb_params_init(ctypes.byref(p))
    p.quirks = quirks
    p.filter_type = FILTERS[filter_type] if isinstance(filter_type, str) else int(filter_type)
    p.cutoff, p.pad, p.interp = cutoff, pad, interp
    p.defects, p.thresh_min, p.thresh_max = int(defects), thresh_min, thresh_max
    p.relevant_mask = int(relevant_mask)
    p.lower_lim_offset, p.upper_lim_offset = lower_lim_offset, upper_lim_offset
    p.xa, p.xb, p.xc, p.xd, p.xe, p.xf = (int(v) for v in fix_points)
    p.masking, p.masking_value, p.normalize = int(masking), masking_value, int(normalize)
    p.repair_reference = int(repair_reference)
    p.module_major = int(module_major)
    return p


def load_config(path: str):
    g, p = Geometry(), Params()
    _check(lib().risa_gb_config_load(path.encode(), ctypes.byref(g), ctypes.byref(p)), "config_load")
    return g, p


def config_lookup(path: str, key: str) -> str:
    """One setting of a config file as text (arrays comma-separated)."""
    buf = ctypes.create_string_buffer(4096)
    _check(lib().risa_gb_config_lookup(path.encode(), key.encode(), buf, len(buf)), "config_lookup")
    return buf.value.decode()


def reorder(inp, out, n_modules: int, n_fan_proj: int, n_fan_det: int, batch: int, stream=None):
    """Module-major -> detector-major raw frames on the device (the Reordering stage)."""
    _check(lib().risa_gb_reorder_enqueue(ptr(inp), ptr(out), n_modules, n_fan_proj, n_fan_det, batch,
                                         stream_ptr(stream)), "reorder_enqueue")


def to_module_major(frames, n_modules: int):
    """Host helper: detector-major [..., P, D] -> module-major [..., modules, P, D/modules]."""
    import numpy as np
    *lead, P, D = frames.shape
    w = D // n_modules
    return np.ascontiguousarray(frames.reshape(*lead, P, n_modules, w).swapaxes(-3, -2))


def geometry_dict(g: Geometry) -> dict:
    out = {f: getattr(g, f) for f, _ in Geometry._fields_ if f != "struct_size"}
    for k in ("source_diameter", "delta_x", "delta_z", "source_angle"):
        out[k] = list(out[k])[: g.n_planes]
    return out


class _Handle:
    _destroy = None

    def __init__(self):
        self._h = ctypes.c_void_p()

    @property
    def handle(self) -> int:
        return self._h.value

    def close(self):
        if self._h and self._h.value and self._destroy:
            getattr(lib(), self._destroy)(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Defects(_Handle):
    """DetectorInterpolation stage: defect detection + in-place repair of u16 frames."""
    _destroy = "risa_gb_defects_destroy"

    def __init__(self, geom: Geometry, params: Params, max_batch: int):
        super().__init__()
        _check(lib().risa_gb_defects_create(ctypes.byref(geom), ctypes.byref(params), max_batch,
                                            ctypes.byref(self._h)), "defects_create")

    def workspace_bytes(self, batch: int) -> int:
        return lib().risa_gb_defects_workspace_bytes(self._h, batch)

    def enqueue(self, frames, batch: int, workspace, flags_out=None, stream=None):
        _check(lib().risa_gb_defects_enqueue(self._h, ptr(frames), batch, ptr(flags_out), ptr(workspace),
                                             stream_ptr(stream)), "defects_enqueue")


class Attenuation(_Handle):
    _destroy = "risa_gb_attenuation_destroy"

    def __init__(self, geom: Geometry, params: Params, ref_frames, n_ref: int, dark_frames=None,
                 n_dark: int = 0):
        """ref_frames/dark_frames: host arrays [n][L][Pf][Df] uint16 (numpy)."""
        super().__init__()
        _check(lib().risa_gb_attenuation_create(ctypes.byref(geom), ctypes.byref(params), ptr(ref_frames),
                                                n_ref, ptr(dark_frames), n_dark, ctypes.byref(self._h)),
               "attenuation_create")
        self.geom = geom

    def enqueue(self, raw, out, plane: int, batch: int, stream=None):
        _check(lib().risa_gb_attenuation_enqueue(self._h, ptr(raw), ptr(out), plane, batch,
                                                 stream_ptr(stream)), "attenuation_enqueue")

    def tables(self):
        import numpy as np
        g = self.geom
        ref = np.zeros((g.n_planes, g.n_fan_proj, g.n_fan_det), np.float32)
        dark = np.zeros((g.n_planes, g.n_fan_det), np.float32)
        _check(lib().risa_gb_attenuation_tables(self._h, ptr(ref), ptr(dark)), "attenuation_tables")
        return ref, dark


class Fan2Para(_Handle):
    _destroy = "risa_gb_fan2para_destroy"

    def __init__(self, geom: Geometry, params: Params):
        super().__init__()
        _check(lib().risa_gb_fan2para_create(ctypes.byref(geom), ctypes.byref(params), ctypes.byref(self._h)),
               "fan2para_create")

    def enqueue(self, fan, par, plane: int, batch: int, stream=None):
        _check(lib().risa_gb_fan2para_enqueue(self._h, ptr(fan), ptr(par), plane, batch, stream_ptr(stream)),
               "fan2para_enqueue")

    def enqueue_adjoint(self, par, fan, plane: int, batch: int, stream=None):
        _check(lib().risa_gb_fan2para_enqueue_adjoint(self._h, ptr(par), ptr(fan), plane, batch,
                                                      stream_ptr(stream)), "fan2para_enqueue_adjoint")


def fan2para_tables_host(geom: Geometry, params: Params, plane: int = 0):
    """Host-built gather table of one plane: (packed u32, u f32, v f32), each [4, Pp*Dp]."""
    import numpy as np
    n = 4 * geom.n_par_proj * geom.n_par_det
    pk = np.zeros(n, np.uint32)
    u = np.zeros(n, np.float32)
    v = np.zeros(n, np.float32)
    _check(lib().risa_gb_fan2para_tables_host(ctypes.byref(geom), ctypes.byref(params), plane, ptr(pk),
                                              ptr(u), ptr(v)), "fan2para_tables_host")
    return pk.reshape(4, -1), u.reshape(4, -1), v.reshape(4, -1)


def fan2para_staged_tables_host(geom: Geometry, params: Params):
    """The engine's staged rebinning tables (host build, no GPU): (boxes
    [L, tiles, 4 slots, 4] as (first row, first column, rows, columns), rel
    [L, 4, Pp*Dp], stage_entries); stage_entries 0 when not staged."""
    import numpy as np
    L, Pp, Dp = geom.n_planes, geom.n_par_proj, geom.n_par_det
    tiles = ((Pp + 7) // 8) * ((Dp + 31) // 32)
    boxes = np.zeros((L, tiles, 4, 4), np.int32)
    rel = np.zeros((L, 4, Pp * Dp), np.uint32)
    se = ctypes.c_int(0)
    _check(lib().risa_gb_fan2para_staged_tables_host(ctypes.byref(geom), ctypes.byref(params), ptr(boxes),
                                                     ptr(rel), ctypes.byref(se)), "fan2para_staged_tables_host")
    return boxes, rel, se.value


class Filter(_Handle):
    _destroy = "risa_gb_filter_destroy"

    def __init__(self, geom: Geometry, params: Params, taps=None):
        """Window-designed filter from params, or (taps: host float32 array) a taps-defined one."""
        super().__init__()
        if taps is None:
            _check(lib().risa_gb_filter_create(ctypes.byref(geom), ctypes.byref(params), ctypes.byref(self._h)),
                   "filter_create")
        else:
            import numpy as np
            t = np.ascontiguousarray(taps, dtype=np.float32)
            _check(lib().risa_gb_filter_create_taps(ctypes.byref(geom), ctypes.byref(params), ptr(t), len(t),
                                                    ctypes.byref(self._h)), "filter_create_taps")
            self.n_taps = len(t)

    def enqueue(self, sino, batch: int, stream=None):
        _check(lib().risa_gb_filter_enqueue(self._h, ptr(sino), batch, stream_ptr(stream)), "filter_enqueue")

    def enqueue_adjoint(self, sino, batch: int, stream=None):
        _check(lib().risa_gb_filter_enqueue_adjoint(self._h, ptr(sino), batch, stream_ptr(stream)),
               "filter_enqueue_adjoint")

    def taps_grad_workspace_bytes(self, batch: int) -> int:
        return lib().risa_gb_filter_taps_grad_workspace_bytes(self._h, batch)

    def taps_grad(self, x, g, grad, batch: int, workspace, stream=None):
        _check(lib().risa_gb_filter_taps_grad(self._h, ptr(x), ptr(g), ptr(grad), batch, ptr(workspace),
                                              stream_ptr(stream)), "filter_taps_grad")

    def response(self):
        import numpy as np
        n = ctypes.c_int()
        _check(lib().risa_gb_filter_response(self._h, ctypes.byref(n), None), "filter_response")
        h = np.zeros(n.value // 2 + 1, np.float32)
        _check(lib().risa_gb_filter_response(self._h, ctypes.byref(n), ptr(h)), "filter_response")
        return n.value, h


class Toeplitz(_Handle):
    """The window-designed filter as a split-bf16 tensor-core Toeplitz GEMM (tcgen05)."""
    _destroy = "risa_gb_toeplitz_destroy"

    def __init__(self, geom: Geometry, params: Params):
        super().__init__()
        _check(lib().risa_gb_toeplitz_create(ctypes.byref(geom), ctypes.byref(params), ctypes.byref(self._h)),
               "toeplitz_create")

    def workspace_bytes(self, batch: int) -> int:
        return lib().risa_gb_toeplitz_workspace_bytes(self._h, batch)

    def enqueue(self, sino, batch: int, workspace, stream=None):
        _check(lib().risa_gb_toeplitz_enqueue(self._h, ptr(sino), batch, ptr(workspace), stream_ptr(stream)),
               "toeplitz_enqueue")

    def check(self):
        _check(lib().risa_gb_toeplitz_check(self._h), "toeplitz_check")

    def set_precision(self, split: int):
        """SPLIT_BF16X3 (default) or SPLIT_F16X3."""
        _check(lib().risa_gb_toeplitz_set_precision(self._h, split), "toeplitz_set_precision")


def filter_design_host(geom: Geometry, params: Params):
    import numpy as np
    n = ctypes.c_int()
    _check(lib().risa_gb_filter_design_host(ctypes.byref(geom), ctypes.byref(params), ctypes.byref(n), None),
           "filter_design_host")
    h = np.zeros(n.value // 2 + 1, np.float32)
    _check(lib().risa_gb_filter_design_host(ctypes.byref(geom), ctypes.byref(params), ctypes.byref(n), ptr(h)),
           "filter_design_host")
    return n.value, h


class Backprojection(_Handle):
    _destroy = "risa_gb_backprojection_destroy"

    def __init__(self, geom: Geometry, params: Params, handle: Optional[int] = None):
        super().__init__()
        if handle is not None:  # borrowed from an FBP engine
            self._h = ctypes.c_void_p(handle)
            self._destroy = None
            return
        _check(lib().risa_gb_backprojection_create(ctypes.byref(geom), ctypes.byref(params),
                                                   ctypes.byref(self._h)), "backprojection_create")

    def enqueue(self, sino, img, batch: int, stream=None):
        _check(lib().risa_gb_backprojection_enqueue(self._h, ptr(sino), ptr(img), batch, stream_ptr(stream)),
               "backprojection_enqueue")

    def enqueue_adjoint(self, img, sino, batch: int, stream=None):
        _check(lib().risa_gb_backprojection_enqueue_adjoint(self._h, ptr(img), ptr(sino), batch,
                                                            stream_ptr(stream)), "backprojection_adjoint")

    def autotune(self, sino, img, batch: int, stream=None) -> int:
        v = ctypes.c_int()
        _check(lib().risa_gb_backprojection_autotune(self._h, ptr(sino), ptr(img), batch, stream_ptr(stream),
                                                     ctypes.byref(v)), "backprojection_autotune")
        return v.value

    def set_variant(self, v: int):
        _check(lib().risa_gb_backprojection_set_variant(self._h, v), "backprojection_set_variant")

    def check(self):
        """Synchronises; raises RisaError if a bounded device-side wait ran out."""
        _check(lib().risa_gb_backprojection_check(self._h), "backprojection_check")

    def reserve(self, max_batch: int):
        """Device buffer for the staged variants at batches up to max_batch (set-up call)."""
        _check(lib().risa_gb_backprojection_reserve(self._h, max_batch), "backprojection_reserve")

    def reserve_adjoint(self, max_batch: int):
        """Scratch of the adjoint's fast path at batches up to max_batch (set-up call)."""
        _check(lib().risa_gb_backprojection_reserve_adjoint(self._h, max_batch), "backprojection_reserve_adjoint")

    def window(self, fused_mask: bool = True):
        """(win_lo, win_len) of the staged variants' padded pair sinogram."""
        lo, n = ctypes.c_int(), ctypes.c_int()
        _check(lib().risa_gb_backprojection_window(self._h, int(fused_mask), ctypes.byref(lo), ctypes.byref(n)),
               "backprojection_window")
        return lo.value, n.value

    def time(self, sino, img, batch: int, reps: int = 5, stream=None):
        """(staging ms, backprojection kernel ms), CUDA-event means over `reps` launches."""
        a, b = ctypes.c_float(), ctypes.c_float()
        _check(lib().risa_gb_backprojection_time(self._h, ptr(sino), ptr(img), batch, reps, stream_ptr(stream),
                                                 ctypes.byref(a), ctypes.byref(b)), "backprojection_time")
        return a.value, b.value

    @staticmethod
    def variant_count() -> int:
        return lib().risa_gb_backprojection_variant_count()

    @staticmethod
    def variant_name(v: int) -> str:
        return lib().risa_gb_backprojection_variant_name(v).decode()


class Masking(_Handle):
    _destroy = "risa_gb_masking_destroy"

    def __init__(self, geom: Geometry, params: Params):
        super().__init__()
        _check(lib().risa_gb_masking_create(ctypes.byref(geom), ctypes.byref(params), ctypes.byref(self._h)),
               "masking_create")

    def workspace_bytes(self, batch: int) -> int:
        return lib().risa_gb_masking_workspace_bytes(self._h, batch)

    def enqueue(self, img, batch: int, workspace=None, stream=None):
        _check(lib().risa_gb_masking_enqueue(self._h, ptr(img), batch, ptr(workspace), stream_ptr(stream)),
               "masking_enqueue")


class Graph(_Handle):
    """A captured whole-job CUDA graph (risa_gb_graph)."""
    _destroy = "risa_gb_graph_destroy"
    owner = None

    def replay(self, stream=None):
        _check(lib().risa_gb_graph_replay(self._h, stream_ptr(stream)), "graph_replay")

    @property
    def kernel_count(self) -> int:
        return lib().risa_gb_graph_kernel_count(self._h)


class FBP(_Handle):
    """Whole chain, raw u16 fan frames -> images, batched, graph-capturable."""
    _destroy = "risa_gb_fbp_destroy"

    def __init__(self, geom: Geometry, params: Params, ref_frames, n_ref: int, dark_frames=None,
                 n_dark: int = 0, max_batch: int = 1):
        super().__init__()
        _check(lib().risa_gb_fbp_create(ctypes.byref(geom), ctypes.byref(params), ptr(ref_frames), n_ref,
                                        ptr(dark_frames), n_dark, max_batch, ctypes.byref(self._h)),
               "fbp_create")
        self.geom, self.params, self.max_batch = geom, params, max_batch

    def _check_sizes(self, raw, img, n: int, what: str):
        g = self.geom
        _need(raw, 2 * n * g.n_fan_proj * g.n_fan_det, what + " (raw frames)")
        _need(img, 4 * n * g.n_pixels * g.n_pixels, what + " (images)")

    def enqueue(self, raw, img, plane: int, batch: int, stream=None):
        self._check_sizes(raw, img, batch, "fbp_enqueue")
        _check(lib().risa_gb_fbp_enqueue(self._h, ptr(raw), ptr(img), plane, batch, stream_ptr(stream)),
               "fbp_enqueue")

    def graph_capture(self, raw, img, plane: int, n_frames: int, stream) -> "Graph":
        """One CUDA graph reconstructing n_frames device frames (chunked by max_batch)."""
        self._check_sizes(raw, img, n_frames, "fbp_graph_capture")
        gr = Graph()
        _check(lib().risa_gb_fbp_graph_capture(self._h, ptr(raw), ptr(img), plane, n_frames,
                                               stream_ptr(stream), ctypes.byref(gr._h)), "fbp_graph_capture")
        gr.owner = self
        return gr

    def run_host(self, host_raw, host_img, n_frames: int, plane: int):
        self._check_sizes(host_raw, host_img, n_frames, "fbp_run_host")
        _check(lib().risa_gb_fbp_run_host(self._h, ptr(host_raw), ptr(host_img), n_frames, plane),
               "fbp_run_host")

    def set_lanes(self, lanes: int):
        """1 (default): every stage of a chunk in sequence; 2: one chunk's
        backprojection beside the next chunk's streaming stages, in graphs and
        the host path (same results)."""
        _check(lib().risa_gb_fbp_set_lanes(self._h, lanes), "fbp_set_lanes")

    def intermediates(self):
        fan, par = ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib().risa_gb_fbp_intermediates(self._h, ctypes.byref(fan), ctypes.byref(par)),
               "fbp_intermediates")
        return fan.value, par.value

    def time_stages(self, raw, img, plane: int, batch: int, reps: int = 5, stream=None) -> dict:
        """Mean ms of the engine's stages on one batch (CUDA events on the stream)."""
        import numpy as np

        self._check_sizes(raw, img, batch, "fbp_time_stages")
        ms = np.zeros(6, np.float32)
        _check(lib().risa_gb_fbp_time_stages(self._h, ptr(raw), ptr(img), plane, batch, reps, stream_ptr(stream),
                                             ms.ctypes.data), "fbp_time_stages")
        keys = ("defect_detect", "attenuation_repair", "rebinning", "filter", "bp_staging", "bp_kernel")
        return {k: float(v) for k, v in zip(keys, ms)}

    def backprojection(self) -> Backprojection:
        return Backprojection(self.geom, self.params, handle=lib().risa_gb_fbp_backprojection(self._h))


PEAK_SMEM_READ, PEAK_FP32_FMA = 0, 1
COMPLETION_EXACT, COMPLETION_LAST_PART = 0, 1
INGEST_ACCEPTED, INGEST_DUPLICATE, INGEST_MALFORMED, INGEST_STALE, INGEST_RING_FULL = range(5)


class PacketLayout(ctypes.Structure):
    """Mirror of risa_gb_packet_layout."""
    _fields_ = [("struct_size", ctypes.c_uint32), ("modules", ctypes.c_int32), ("det_per_module", ctypes.c_int32),
                ("proj", ctypes.c_int32), ("proj_per_packet", ctypes.c_int32), ("ring", ctypes.c_int32)]


def packet_layout(modules: int, det_per_module: int, proj: int, proj_per_packet: int, ring: int) -> PacketLayout:
    return PacketLayout(ctypes.sizeof(PacketLayout), modules, det_per_module, proj, proj_per_packet, ring)


def encode_packet(index: int, part: int, payload) -> bytes:
    """[uint64 frame index][uint16 part][payload uint16] in native byte order."""
    import struct

    return struct.pack("=QH", index, part) + payload.tobytes()


class Assembler(_Handle):
    """Online input: module packets -> whole module-major frames in a caller ring
    (risa_gb_assembler_*). `ring` is a uint16/int16 buffer of layout.ring frames
    that outlives this object (pinned host memory for one-copy uploads)."""
    _destroy = "risa_gb_assembler_destroy"

    def __init__(self, layout: PacketLayout, ring, skip_lag: int = 0, completion: int = COMPLETION_EXACT):
        super().__init__()
        self.layout, self.ring = layout, ring
        _check(lib().risa_gb_assembler_create(ctypes.byref(layout), ptr(ring), skip_lag, completion,
                                              ctypes.byref(self._h)), "assembler_create")

    def ingest(self, module: int, packet: bytes) -> int:
        r = lib().risa_gb_assembler_ingest(self._h, module, packet, len(packet))
        if r < 0:
            raise RisaError(r, "assembler_ingest", last_error())
        return r

    def next(self, timeout_s: float):
        """(frame index, ring slot), or None on timeout / when finished and drained."""
        idx, slot = ctypes.c_uint64(), ctypes.c_int()
        r = lib().risa_gb_assembler_next(self._h, timeout_s, ctypes.byref(idx), ctypes.byref(slot))
        if r < 0:
            raise RisaError(r, "assembler_next", last_error())
        return (idx.value, slot.value) if r == 1 else None

    def release(self, index: int):
        _check(lib().risa_gb_assembler_release(self._h, index), "assembler_release")

    def finish(self):
        _check(lib().risa_gb_assembler_finish(self._h), "assembler_finish")

    def stats(self) -> dict:
        v = [ctypes.c_uint64() for _ in range(3)]
        _check(lib().risa_gb_assembler_stats(self._h, *[ctypes.byref(x) for x in v]), "assembler_stats")
        return dict(zip(("skipped", "abandoned", "duplicates"), (x.value for x in v)))


def measure_peak(kind: int, reps: int = 5, stream=None) -> dict:
    """Measured shared-memory read bandwidth (kind PEAK_SMEM_READ) or FP32 FMA
    throughput (PEAK_FP32_FMA) of the current GPU; see risa_gb_measure_peak."""
    out = (ctypes.c_double * 4)()
    _check(lib().risa_gb_measure_peak(kind, reps, stream_ptr(stream), out), "measure_peak")
    unit = "GB/s" if kind == PEAK_SMEM_READ else "TFLOP/s"
    per = "B/clk/SM" if kind == PEAK_SMEM_READ else "FLOP/clk/SM"
    return {"value": out[0], "unit": unit, "per_sm_per_clk": out[1], "per_sm_per_clk_unit": per,
            "sm_mhz": out[2], "sms": int(out[3])}


class Sweep(_Handle):
    """Many parallel-beam reconstructions of different shapes in one persistent launch.

    instances: sequence of dicts with keys n_pixels, n_par_proj, n_par_det and
    optionally filter_type ("ramp", ...), cutoff, rotation_offset, ref_level,
    dark_level, masking, masking_value, defect_map (uint8 array [n_par_det]).
    Inputs and outputs are packed device buffers (see layout()).
    """
    _destroy = "risa_gb_sweep_destroy"

    def __init__(self, instances):
        super().__init__()
        import numpy as np

        n = len(instances)
        arr = (SweepInstance * n)()
        self._maps = []
        for i, d in enumerate(instances):
            s = arr[i]
            s.n_pixels, s.n_par_proj, s.n_par_det = d["n_pixels"], d["n_par_proj"], d["n_par_det"]
            ft = d.get("filter_type", "ramp")
            s.filter_type = FILTERS[ft] if isinstance(ft, str) else int(ft)
            s.cutoff = d.get("cutoff", 1.0)
            s.rotation_offset = d.get("rotation_offset", 0.0)
            s.ref_level = d.get("ref_level", 40200.0)
            s.dark_level = d.get("dark_level", 200.0)
            s.masking = int(d.get("masking", True))
            s.masking_value = d.get("masking_value", 0.0)
            m = d.get("defect_map")
            if m is not None:
                m = np.ascontiguousarray(m, dtype=np.uint8)
                self._maps.append(m)
                s.defect_map = m.ctypes.data
            else:
                s.defect_map = None
        self.n = n
        _check(lib().risa_gb_sweep_create(arr, n, ctypes.byref(self._h)), "sweep_create")

    def layout(self):
        """(raw offsets, image offsets, raw total, image total) in elements."""
        import numpy as np

        ro = np.zeros(self.n, np.uint64)
        io = np.zeros(self.n, np.uint64)
        rt, it = ctypes.c_size_t(), ctypes.c_size_t()
        _check(lib().risa_gb_sweep_layout(self._h, ro.ctypes.data, io.ctypes.data, ctypes.byref(rt),
                                          ctypes.byref(it)), "sweep_layout")
        return ro.astype(np.int64), io.astype(np.int64), rt.value, it.value

    def enqueue(self, raw, img, stream=None):
        _check(lib().risa_gb_sweep_enqueue(self._h, ptr(raw), ptr(img), stream_ptr(stream)), "sweep_enqueue")

    def graph_capture(self, raw, img, stream) -> "Graph":
        """The enqueue (counter resets + the persistent launch) as one CUDA graph."""
        gr = Graph()
        _check(lib().risa_gb_sweep_graph_capture(self._h, ptr(raw), ptr(img), stream_ptr(stream),
                                                 ctypes.byref(gr._h)), "sweep_graph_capture")
        gr.owner = self
        return gr

    def times(self):
        """(first_ns[n], done_ns[n], launch_ns) of the last enqueue (%globaltimer)."""
        import numpy as np

        f = np.zeros(self.n, np.uint64)
        d = np.zeros(self.n, np.uint64)
        t = ctypes.c_uint64()
        _check(lib().risa_gb_sweep_times(self._h, f.ctypes.data, d.ctypes.data, ctypes.byref(t)), "sweep_times")
        return f, d, t.value

    def check(self):
        _check(lib().risa_gb_sweep_check(self._h), "sweep_check")

    def grid(self) -> int:
        return lib().risa_gb_sweep_grid(self._h)
