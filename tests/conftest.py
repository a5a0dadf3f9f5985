import ctypes
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


EMU_DIR = os.path.join(ROOT, "tests", "emu")
EMU_LIB = os.path.join(EMU_DIR, "_build", "libestl_emu.so")


def build_emulator():
    """Compile the host emulator of the tile kernels (g++, C++20)."""
    srcs = [os.path.join(EMU_DIR, "emu.cpp"), os.path.join(ROOT, "estl_gb300", "csrc", "planner.cpp"),
            os.path.join(ROOT, "estl_gb300", "csrc", "conv_plan.cpp"),
            os.path.join(ROOT, "estl_gb300", "csrc", "packed_plan.cpp")]
    deps = srcs + [os.path.join(ROOT, "estl_gb300", "csrc", f) for f in os.listdir(os.path.join(ROOT, "estl_gb300", "csrc"))]
    if os.path.exists(EMU_LIB) and os.path.getmtime(EMU_LIB) >= max(os.path.getmtime(d) for d in deps):
        return EMU_LIB
    os.makedirs(os.path.dirname(EMU_LIB), exist_ok=True)
    cmd = ["g++", "-std=c++20", "-O2", "-DESTL_EMU", "-fPIC", "-shared", "-pthread",
           "-I", os.path.join(ROOT, "estl_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
           "-x", "c++"] + srcs + ["-o", EMU_LIB]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return EMU_LIB


@pytest.fixture(scope="session")
def emu():
    lib = ctypes.CDLL(build_emulator())
    P = ctypes.c_void_p
    lib.emu_plan_run.argtypes = [ctypes.c_longlong, ctypes.c_longlong, P, ctypes.c_int, P, P, ctypes.c_char_p, ctypes.c_int]
    lib.emu_plan_run.restype = ctypes.c_int
    lib.emu_plan2d_run.argtypes = [ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int, P, P,
                                   ctypes.c_char_p, ctypes.c_int]
    lib.emu_plan2d_run.restype = ctypes.c_int
    lib.emu_bluestein_run.argtypes = [ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int, P, P, ctypes.c_char_p,
                                      ctypes.c_int]
    lib.emu_bluestein_run.restype = ctypes.c_int
    lib.emu_plan_describe.argtypes = [ctypes.c_longlong, ctypes.c_longlong, P, ctypes.c_char_p, ctypes.c_int]
    lib.emu_plan_candidates.argtypes = [ctypes.c_longlong, ctypes.c_longlong, P, ctypes.c_int]
    lib.emu_conv_run.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, ctypes.c_char_p, ctypes.c_int]
    lib.emu_conv_run.restype = ctypes.c_int
    L = ctypes.c_longlong
    lib.emu_conv2d_run.argtypes = [L, L, L, L, L, ctypes.c_int, P, P, P, ctypes.c_char_p, ctypes.c_int]
    lib.emu_conv2d_run.restype = ctypes.c_int
    lib.emu_packed_run.argtypes = [P, P, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_char_p,
                                   ctypes.c_int]
    lib.emu_packed_run.restype = ctypes.c_int
    lib.emu_packed_run_launches.argtypes = [P, P, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int,
                                            ctypes.c_char_p, ctypes.c_int]
    lib.emu_packed_run_launches.restype = ctypes.c_int
    lib.emu_cluster_barrier_selftest.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.emu_cluster_barrier_selftest.restype = ctypes.c_int
    lib.emu_packed_bucketed_run.argtypes = [P, P, ctypes.c_longlong, ctypes.c_int, P, P, ctypes.c_char_p, ctypes.c_int]
    lib.emu_packed_bucketed_run.restype = ctypes.c_int
    lib.emu_packed_mixed_run.argtypes = [P, P, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, P, P, P,
                                         ctypes.c_longlong, ctypes.c_int, P, P, P, ctypes.c_char_p, ctypes.c_int]
    lib.emu_packed_mixed_run.restype = ctypes.c_int
    lib.emu_bank.argtypes = [P]
    lib.emu_bank.restype = ctypes.c_longlong
    return lib


@pytest.fixture(scope="session")
def engine():
    """The CUDA engine, initialised on device 0 (GPU tests only)."""
    import estl_gb300 as estl
    estl.init(0)
    return estl
