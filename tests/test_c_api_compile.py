"""Drop-in at the source level: a C program and a C++ program written
against sFFT 0.1's API (tests/c_api/drop_in.c, drop_in.cc) compile against
include/sfft.h, link against libsfft.so and run.  Without a GPU the plan is
refused with a message; with one the transform runs."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_api")


def _build_and_run(tmp_path, src, compiler, extra):
    from sfft_gb300 import build
    lib = build.build()
    exe = str(tmp_path / (os.path.basename(src) + ".bin"))
    libdir = os.path.dirname(lib)
    cmd = [compiler, os.path.join(SRC, src), "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lsfft",
           "-Wl,-rpath," + libdir, "-o", exe] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    return out.stdout


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


@pytest.mark.parametrize("src,compiler,extra", [("drop_in.c", "gcc", ["-std=gnu99", "-lm"]),
                                                ("drop_in.cc", "g++", ["-std=c++17"])])
def test_reference_style_callers_compile_and_run(tmp_path, src, compiler, extra):
    out = _build_and_run(tmp_path, src, compiler, extra)
    if _has_gpu():
        assert out.startswith("plan v"), out
    else:
        assert "no plan" in out and "CUDA" in out, out


@pytest.mark.gpu
@pytest.mark.parametrize("src,compiler,extra", [("drop_in.c", "gcc", ["-std=gnu99", "-lm"]),
                                                ("drop_in.cc", "g++", ["-std=c++17"])])
def test_reference_style_callers_run_on_the_gpu(tmp_path, src, compiler, extra):
    if not _has_gpu():
        pytest.skip("no CUDA device")
    out = _build_and_run(tmp_path, src, compiler, extra)
    assert out.startswith("plan v"), out
    if src.endswith(".cc"):          # an impulse: v1 finds... a flat spectrum's entries
        assert int(out.split("entries=")[1]) >= 0
