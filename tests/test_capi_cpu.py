"""The C ABI library loads, exports every symbol the public header declares,
and its host-only entry points (init, config parsing, validation) behave."""
import ctypes
import os
import re

import pytest

import risa_gb300 as rg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(risa_gb_\w+)\s*\(", text))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "risa_gb_fbp_create" in names and "risa_gb_backprojection_enqueue" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol():
    lib = rg.lib()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    assert declared_symbols() <= set(rg.SIGNATURES)


def test_struct_sizes_match():
    g = rg.make_geometry()
    assert g.struct_size == ctypes.sizeof(rg.Geometry)
    p = rg.make_params()
    assert p.struct_size == ctypes.sizeof(rg.Params)
    assert rg.lib().risa_gb_version().decode().startswith("risa_gb300")


def test_config_file_parsing():
    g, p = rg.load_config(os.path.join(ROOT, "tests", "configs", "rofex_like.cfg"))
    assert (g.n_planes, g.n_fan_det, g.n_fan_proj) == (2, 432, 500)  # 1e6 * 1 / 2000
    assert (g.n_par_proj, g.n_par_det, g.n_pixels) == (512, 256, 256)
    assert list(g.source_diameter)[:2] == [365.0, 370.0]
    assert list(g.delta_z)[:2] == [1417.0, 1430.0]
    assert g.source_offset == pytest.approx(23.2)
    assert p.filter_type == rg.FILTER_SHEPP_LOGAN
    assert p.quirks == rg.QUIRKS_RISA and p.defects == 1 and p.masking == 1
    assert (p.xa, p.xd, p.xf) == (43, 362, 431)
    assert p.thresh_min == pytest.approx(0.67)


def test_config_errors(tmp_path):
    with pytest.raises(rg.RisaError) as e:
        rg.load_config(str(tmp_path / "missing.cfg"))
    assert e.value.status == -6
    bad = tmp_path / "bad.cfg"
    bad.write_text("numberOfFanDetectors = 432;\nscanRate = \n")
    with pytest.raises(rg.RisaError) as e:
        rg.load_config(str(bad))
    assert e.value.status == -6
    incomplete = tmp_path / "inc.cfg"
    incomplete.write_text("numberOfFanDetectors = 432;\n")
    with pytest.raises(rg.RisaError) as e:
        rg.load_config(str(incomplete))
    assert "missing" in str(e.value)


def test_invalid_geometry_rejected_without_gpu():
    g = rg.make_geometry(n_planes=7)
    with pytest.raises(rg.RisaError) as e:
        rg.fan2para_tables_host(g, rg.make_params(), 0)
    assert e.value.status == -1
    p = rg.make_params()
    p.struct_size = 3
    with pytest.raises(rg.RisaError):
        rg.filter_design_host(rg.make_geometry(), p)


def test_fbp_binding_rejects_short_buffers():
    """The binding checks tensor and array sizes before a launch that would read
    or write past them (raw frames and images of `batch` frames)."""
    import types

    import numpy as np
    import pytest

    import risa_gb300 as rg

    h = types.SimpleNamespace(geom=rg.make_geometry(n_fan_proj=10, n_fan_det=8, n_pixels=4))
    raw, img = np.zeros((4, 10, 8), np.uint16), np.zeros((4, 4, 4), np.float32)
    rg.FBP._check_sizes(h, raw, img, 4, "fbp_enqueue")
    with pytest.raises(rg.RisaError):
        rg.FBP._check_sizes(h, raw[:3], img, 4, "fbp_enqueue")
    with pytest.raises(rg.RisaError):
        rg.FBP._check_sizes(h, raw, img[:2], 4, "fbp_enqueue")
    rg.FBP._check_sizes(h, 12345, 67890, 4, "fbp_enqueue")  # raw addresses: the caller's responsibility
