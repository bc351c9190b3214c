"""The configuration-driven C++ pipeline (loader -> H2D -> Reordering ->
DetectorInterpolation -> Attenuation -> Fan2Para -> Filter -> Backprojection ->
Masking -> D2H -> TIFF) on synthetic module files, in its thread-per-stage
and batched forms, against the FP64 oracle; plus the fused module-major path
of the engine against the detector-major one."""
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from risa_gb300 import build as rb
from risa_gb300 import phantom
from tests.helpers import SMALL, geom, ns, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MODULES = 27


def read_float_tiff(path):
    """Pages of a little-endian 32-bit float TIFF written by the pipeline."""
    data = open(path, "rb").read()
    assert data[:4] == b"II*\x00"
    (off,) = struct.unpack_from("<I", data, 4)
    pages = []
    while off:
        (n,) = struct.unpack_from("<H", data, off)
        tags = {}
        for e in range(n):
            tag, typ, cnt, val = struct.unpack_from("<HHII", data, off + 2 + 12 * e)
            tags[tag] = val
        w, h, so = tags[256], tags[257], tags[273]
        assert tags[339] == 3 and tags[258] == 32
        pages.append(np.frombuffer(data, np.float32, w * h, so).reshape(h, w))
        (off,) = struct.unpack_from("<I", data, off + 2 + 12 * n)
    return np.stack(pages)


def write_module_files(prefix, frames, modules):
    """frames [n, P, D] detector-major -> modules files prefix<i>.fx (i from 1)."""
    n, P, D = frames.shape
    w = D // modules
    for m in range(modules):
        frames[:, :, m * w:(m + 1) * w].astype("<u2").tofile(f"{prefix}{m + 1}.fx")


def make_case(tmp_path, frames=3):
    d = dict(SMALL, n_planes=2, source_diameter=[430.0, 430.0], delta_x=[0.0, 0.0], delta_z=[1417.0, 1430.0],
             source_angle=[360.0, 360.0], n_par_proj=96, n_par_det=128, n_pixels=96)
    sc = phantom.make_scan(frames, 2, 500, 432, 215.0, 240.0, seed=21, defect_fraction=0.01, distinct=frames)
    data = tmp_path / "data"
    data.mkdir()
    write_module_files(str(data / "scan_DetModNr_"), sc.raw, MODULES)
    write_module_files(str(data / "ref_empty_tomograph_repaired_DetModNr_"), sc.ref, MODULES)
    write_module_files(str(data / "dark_192.168.100_DetModNr_"), sc.dark, MODULES)
    out = tmp_path / "reco"
    out.mkdir()
    cfg = tmp_path / "scan.cfg"
    cfg.write_text(f"""
numberOfDetectorModules = {MODULES}
numberOfFanDetectors = 432
samplingRate = 1
scanRate = 2000
numberOfPlanes = 2
numberOfDataFrames = {frames}
numberOfReferenceFrames = 1
numberOfDarkFrames = 1
dataInputPath = "{data}"
dataFileName = "scan_DetModNr_"
dataFileEnding = ".fx"
referenceInputPath = "{data}"
darkInputPath = "{data}"
outputPath = "{out}"
outputFileName = "reco"
sourceOffset = 0.0
detectorDiameter = 480.0
imageWidth = 200.0
imageCenterX = 0.0
imageCenterY = 0.0
sourceDiameter = [430.0, 430.0]
deltaX = [0.0, 0.0]
deltaZ = [1417.0, 1430.0]
sourceAngle = [360.0, 360.0]
filterType = "sheppLogan"
cutoffFraction = 1.0
numberOfParallelProjections = 96
numberOfParallelDetectors = 128
numberOfPixels = 96
rotationOffset = 0.0
interpolationType = "linear"
useTextureMemory = false
normalization = false
maskingValue = 0.0
thresh_min = 0.67
thresh_max = 1.5
memPoolSize_H2D = 4
memPoolSize_attenuation = 4
gb_quirks = "none"
gb_defects = true
gb_masking = true
gb_batch = 4
""")
    return d, sc, cfg, out


def oracle_images(d, sc):
    op = oracle.make_params(quirk=oracle.QUIRK_NONE, filter_type="sheppLogan", defects=True, masking=True)
    ref, dark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, oracle.QUIRK_NONE)
    rec = oracle.f2p_records(ns(d), oracle.QUIRK_NONE)
    return oracle.fbp(ns(d), op, rec, ref, dark, sc.raw, sc.planes)


@pytest.mark.parametrize("mode", ["stages", "batched"])
def test_config_driven_pipeline(tmp_path, mode):
    d, sc, cfg, out = make_case(tmp_path)
    exe = rb.PIPELINE
    assert os.path.exists(exe), "build() must compile the pipeline example"
    args = [exe, str(cfg)] + (["--batched"] if mode == "batched" else [])
    res = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert f'"mode": "{mode}"' in res.stdout and '"images": 6' in res.stdout
    exp = oracle_images(d, sc)
    for k in range(2):
        pages = read_float_tiff(str(out / f"reco_plane{k}.tif"))
        assert pages.shape == (3, 96, 96)
        for f in range(3):
            mr, l2 = rel_err(pages[f], exp[f * 2 + k])
            assert mr < 1e-5, (mode, k, f, mr)


def test_module_major_engine_matches_detector_major():
    d = dict(SMALL, n_planes=2, source_diameter=[430.0, 430.0], delta_x=[0.0, 0.0], delta_z=[1417.0, 1430.0],
             source_angle=[360.0, 360.0], n_modules=MODULES)
    sc = phantom.make_scan(2, 2, 500, 432, 215.0, 240.0, seed=8, defect_fraction=0.02, distinct=2)
    n = sc.raw.shape[0]
    outs = []
    for mm in (False, True):
        p = rg.make_params(filter_type="ramp", defects=True, masking=True, module_major=mm)
        fbp = rg.FBP(geom(d), p, sc.ref, 1, sc.dark, 1, max_batch=n)
        raw = rg.to_module_major(sc.raw, MODULES) if mm else sc.raw
        t = torch.from_numpy(np.ascontiguousarray(raw).view(np.int16)).cuda()
        img = torch.empty((n, 64, 64), dtype=torch.float32, device="cuda")
        fbp.enqueue(t, img, rg.PLANES_INTERLEAVED, n)
        torch.cuda.synchronize()
        outs.append(img.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    # the standalone reordering stage
    src = torch.from_numpy(rg.to_module_major(sc.raw, MODULES).view(np.int16)).cuda()
    dst = torch.empty_like(src)
    rg.reorder(src, dst, MODULES, 500, 432, n)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dst.cpu().numpy().view(np.uint16).reshape(sc.raw.shape), sc.raw)
