"""The C++ drop-in classes (whatprot_gb300/cpp) without a GPU.

* They and their test driver compile and link against the library's own
  data types, and a call with no CUDA device surfaces as the library's
  error (exit status 3 and its message), not a crash.
* Where the reference sources are present, oracle/Makefile compiles the
  same files against the reference's own headers and data-type objects
  (-DWHATPROT_GPU_WITH_REFERENCE), which checks that the constructors and
  methods have the reference's signatures.
The GPU test (test_gpu_cpp_dropin.py) runs them on the reference's fixtures."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CPP = os.path.join(REPO, "whatprot_gb300", "cpp")


def _libdir():
    from whatprot_gb300 import capi
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("CUDA library not built")
    return os.path.dirname(capi.LIB_PATH)


def test_dropin_builds_and_reports_missing_device(tmp_path):
    libdir = _libdir()
    exe = str(tmp_path / "dropin_driver")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", CPP,
                    os.path.join(HERE, "cpp", "dropin_driver.cc"), os.path.join(CPP, "whatprot_gpu.cc"),
                    "-L", libdir, "-lwhatprot_gb300", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present: the GPU test covers the driver")
    inp = tmp_path / "in.txt"
    inp.write_text("1 2 max\n0.06 0.05 0 0 0 0\n0.05 0.07 0.00667 1 0.16\n1\n7 1 0.0\n0\n0 0 0\n1\n1.0 0.9\n")
    r = subprocess.run([exe, "hmm", str(inp)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "no context on device" in r.stderr


def test_dropin_builds_against_reference_headers():
    _libdir()
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "dropin-ref-if-present"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = os.path.join(REPO, "oracle", "_ref", "dropin_driver_ref")
    if not os.path.exists(exe):
        pytest.skip("reference sources absent: nothing to compile against")
    assert os.path.getmtime(exe) >= os.path.getmtime(os.path.join(CPP, "whatprot_gpu.cc"))
