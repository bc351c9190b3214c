"""The detector modules' packet format and frame assembly (online input side)
on the CPU: packets in any order from concurrent module threads, lost,
duplicate, malformed and stale packets, ring back-pressure."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_frame_assembler(tmp_path):
    exe = tmp_path / "test_packets_cpu"
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-pthread", "-Wall", "-I", os.path.join(ROOT, "risa_gb300", "cpp"),
                           os.path.join(ROOT, "tests", "cpp", "test_packets_cpu.cpp"), "-o", str(exe)])
    for _ in range(5):  # the concurrent cases run several times
        out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "packets: failures=0" in out.stdout
