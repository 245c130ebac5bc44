"""Per-device kernel set-up (kernel attributes, persistent grid sizes) on the
host: once per device ordinal across threads, failures retried, ordinals kept
apart.  The logic is CUDA-free (csrc/per_device.h) and runs here without a GPU."""
import pathlib
import shutil
import subprocess

import pytest

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE.parent / "mpres-blas_gb300" / "csrc"


def test_per_device_once(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "per_device_check"
    subprocess.run([gxx, "-std=c++17", "-O1", "-pthread", "-I", str(CSRC), str(HERE / "native" / "per_device_check.cpp"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
