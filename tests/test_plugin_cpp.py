"""The C++ plugin FFT_CUDA<float> (include/FFT_CUDA.h) behind ESTL's factory
API, driven by tests/cpp/test_plugin.cpp (the semantics of the reference's
tests/Test.cpp).

* not gpu: the driver compiles against the reference's own plugin headers when
  they are available (drop-in proof) and against the interface-compatible
  headers in tests/cpp/compat; without a GPU it fails cleanly through
  EstlException.
* gpu: the driver runs the known-answer sweep, FFT2D and backward checks.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_plugin.cpp")
# Directory holding the reference's plugin headers (FFT.h, DataInterface.h,
# Complex.h); the drop-in compile check is skipped when it is unset or absent.
REFERENCE_HEADERS = os.environ.get("ESTL_REFERENCE_DIR", "")


CONV2D_SRC = os.path.join(ROOT, "tests", "cpp", "test_conv2d_plugin.cpp")


def compile_driver(include_dir, out, src=SRC):
    from estl_gb300 import build
    build.build()
    pkg = os.path.join(ROOT, "estl_gb300")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", include_dir, src,
           "-L", pkg, "-lestl_cuda", f"-Wl,-rpath,{pkg}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(not REFERENCE_HEADERS or not os.path.exists(os.path.join(REFERENCE_HEADERS, "FFT.h")),
                    reason="ESTL_REFERENCE_DIR unset or without the reference's FFT.h")
def test_compiles_against_reference_headers(tmp_path):
    exe = compile_driver(REFERENCE_HEADERS, str(tmp_path / "plugin_ref"))
    if not has_gpu():
        r = subprocess.run([exe, "0", "2"], capture_output=True, text=True, timeout=60)
        assert r.returncode == 2 and "estl_init" in r.stdout


def test_compiles_against_compat_headers(tmp_path):
    exe = compile_driver(os.path.join(ROOT, "tests", "cpp", "compat"), str(tmp_path / "plugin_compat"))
    if not has_gpu():
        r = subprocess.run([exe, "0", "2"], capture_output=True, text=True, timeout=60)
        assert r.returncode == 2 and "EstlException" not in r.stdout and "estl_init" in r.stdout


@pytest.mark.gpu
def test_plugin_driver_on_gpu(tmp_path):
    exe = compile_driver(os.path.join(ROOT, "tests", "cpp", "compat"), str(tmp_path / "plugin"))
    r = subprocess.run([exe, "4", "16"], capture_output=True, text=True, timeout=900)
    print(r.stdout[-4000:])
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "PASSED" in r.stdout


def test_conv2d_plugin_compiles(tmp_path):
    """Convolution2D_FFT_CUDA<float> (include/Convolution2D_CUDA.h) behind the
    Data2D / Convolution2D interfaces (the reference's Convolution.h pulls in
    every backend, OpenCL included, so the interface subset in tests/cpp/compat
    stands in for it); without a GPU it fails cleanly through EstlException."""
    exe = compile_driver(os.path.join(ROOT, "tests", "cpp", "compat"), str(tmp_path / "conv2d_plugin"), CONV2D_SRC)
    if not has_gpu():
        r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
        assert r.returncode == 2 and "estl_init" in r.stdout


@pytest.mark.gpu
def test_conv2d_plugin_on_gpu(tmp_path):
    exe = compile_driver(os.path.join(ROOT, "tests", "cpp", "compat"), str(tmp_path / "conv2d_plugin"), CONV2D_SRC)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout[-4000:])
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "PASSED" in r.stdout
