"""The detector modules' packet format and frame assembly (online input side)
on the CPU: packets in any order from concurrent module threads, lost,
duplicate, malformed and stale packets, ring back-pressure, the reference's
last-part completion rule; and the same assembler through the C ABI."""
import os
import subprocess

import numpy as np
import pytest

import risa_gb300 as rg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_frame_assembler(tmp_path):
    exe = tmp_path / "test_packets_cpu"
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-pthread", "-Wall", "-I", os.path.join(ROOT, "risa_gb300", "cpp"),
                           os.path.join(ROOT, "tests", "cpp", "test_packets_cpu.cpp"), "-o", str(exe)])
    for _ in range(5):  # the concurrent cases run several times
        out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "packets: failures=0" in out.stdout


def _packets(frame_mm, index, ppp):
    m_, p_, w = frame_mm.shape
    return [[rg.encode_packet(index, part, frame_mm[m, part * ppp:(part + 1) * ppp]) for part in range(p_ // ppp)]
            for m in range(m_)]


def test_assembler_c_abi():
    M, W, P, PPP, RING = 3, 4, 20, 5, 3
    layout = rg.packet_layout(M, W, P, PPP, RING)
    ring = np.zeros((RING, M, P, W), np.uint16)
    rng = np.random.default_rng(1)
    frames = rng.integers(0, 65535, size=(6, M, P, W), dtype=np.uint16)
    a = rg.Assembler(layout, ring, skip_lag=1)
    for f in range(3):
        for m, pk in enumerate(_packets(frames[f], f, PPP)):
            for part, b in enumerate(pk):
                if (f, m, part) != (1, 2, 3):  # lost packet: frame 1 never completes
                    assert a.ingest(m, b) == rg.INGEST_ACCEPTED
    assert a.ingest(0, _packets(frames[0], 0, PPP)[0][0]) == rg.INGEST_DUPLICATE
    assert a.ingest(0, b"short") == rg.INGEST_MALFORMED
    assert a.ingest(7, _packets(frames[0], 0, PPP)[0][0]) == rg.INGEST_MALFORMED
    got = []
    while (nx := a.next(0.05)) is not None:
        idx, slot = nx
        np.testing.assert_array_equal(ring[slot], frames[idx])
        got.append(idx)
        a.release(idx)
    assert got == [0, 2]
    assert a.ingest(0, _packets(frames[1], 1, PPP)[2][3]) == rg.INGEST_STALE
    assert a.stats() == {"skipped": 1, "abandoned": 0, "duplicates": 1}
    a.finish()
    assert a.next(0.05) is None
    # the reference's rule: frame 0 never handed out, the newest common frame is
    b = rg.Assembler(layout, np.zeros_like(ring), completion=rg.COMPLETION_LAST_PART)
    for f in range(3):
        for m, pk in enumerate(_packets(frames[f], f, PPP)):
            for part, pkt in enumerate(pk):
                assert b.ingest(m, pkt) == (rg.INGEST_STALE if f == 0 else rg.INGEST_ACCEPTED)
    assert b.next(0.05)[0] == 2 and b.stats()["skipped"] == 1
    with pytest.raises(rg.RisaError):
        rg.Assembler(rg.packet_layout(M, W, P, 7, RING), ring)  # 7 does not divide 20
