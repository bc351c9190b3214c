"""The C++ stage runtime (pooled images, bounded queues, thread-per-stage
pipeline, end-of-stream sentinel) on the CPU, without a GPU."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_glados_runtime(tmp_path):
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = tmp_path / "test_glados_cpu"
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-pthread", "-I", os.path.join(ROOT, "risa_gb300", "cpp"),
                           "-I", os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "test_glados_cpu.cpp"),
                           "-o", str(exe), "-L", os.path.join(cuda, "lib64"), "-lcudart",
                           "-Wl,-rpath," + os.path.join(cuda, "lib64")])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "seen=200 errors=0 pools_full=1" in out.stdout
