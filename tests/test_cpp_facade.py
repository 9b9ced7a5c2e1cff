"""The C++ facade (include/oslg.hpp): a renderer-style program compiles
against it and the C ABI library; on the CPU it builds and optimizes a group
(and a batch wider than W is refused); on the GPU it shades W-lane batches
(4, 8, 16, ragged) and an N-point device batch, checking every result."""
import os
import shutil
import subprocess

import pytest

from helpers import ROOT

CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build(tmp_path, native):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = str(tmp_path / "batched_facade")
    libdir = os.path.dirname(native)
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", "batched_facade.cpp"),
           "-L", libdir, "-loslg_gb300", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
           "-Wl,-rpath," + libdir, "-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_facade_builds_and_lowers(tmp_path, native):
    exe = build(tmp_path, native)
    r = subprocess.run([exe, "lower"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "lowered" in r.stdout


@pytest.mark.gpu
def test_facade_shades_batches(tmp_path, native):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = build(tmp_path, native)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
