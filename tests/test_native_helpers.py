"""Host build of the refinement step's float-float helpers
(meshoid_gb300/csrc/mg_refine.cuh): tests/native/refine_check.cu compiles the
header into a CPU program that checks sep1_ff / wrap1_ff against the first
pass's separations bit for bit and against FP64, and scaled_sep_lo /
refine_residual against FP64 bounds.  Needs nvcc (host code only; no GPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_refinement_helpers_on_the_host(tmp_path):
    from meshoid_gb300 import build
    try:
        nvcc = build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "refine_check")
    cmd = [nvcc, "-std=c++17", "-O2", *build.ARCH, "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "meshoid_gb300", "csrc"), "-o", exe,
           os.path.join(ROOT, "tests", "native", "refine_check.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout
