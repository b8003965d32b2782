"""Builds and runs the C++ tests of the AutoPas-facing mirror (tests/cpp/test_mirror.cpp) with g++."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def binary():
    from autopas_gb300.build import build, LIBDIR
    build()
    out_dir = os.path.join(ROOT, "tests", "cpp", "build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "test_mirror")
    src = os.path.join(ROOT, "tests", "cpp", "test_mirror.cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
           "-L", LIBDIR, "-lpairengine", f"-Wl,-rpath,{LIBDIR}"]
    subprocess.run(cmd, check=True)
    return exe


def test_mirror_host_logic(binary):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("the host-only mode expects no GPU")
    except Exception:
        pass
    r = subprocess.run([binary, "cpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_mirror_reference_known_answers_on_gpu(binary):
    r = subprocess.run([binary, "gpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failure(s)" in r.stdout
