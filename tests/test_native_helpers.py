"""Host builds of device code shared through headers, run on the CPU (nvcc
for host code only; no GPU):

* tests/native/refine_check.cu: the refinement step's float-float helpers
  (meshoid_gb300/csrc/mg_refine.cuh) -- sep1_ff / wrap1_ff against the first
  pass's separations bit for bit and against FP64, scaled_sep_lo /
  refine_residual against FP64 bounds.
* tests/native/chol_check.cu: the sweep's FP32 Cholesky, solve and condition
  estimate (meshoid_gb300/csrc/mg_chol.cuh) on flattened neighbourhoods'
  moment matrices against FP64 -- the estimate that routes rows to the FP64
  re-solve stays near or above the true condition number.
* tests/native/cube_check.cu: the 3-D deposits' float-reciprocal decode of a
  node index (meshoid_gb300/csrc/mg_cube.cuh) against integer division, at
  every index of small cubes and at the column boundaries of large ones.
* tests/native/group_bound_check.cu: the first search pass's distance error
  bound e2 (k_knn_group), with the box, centre, offsets and FP32 squared
  distances restated from the kernel's arithmetic, on adversarial block
  geometries against FP64 distances.
* tests/native/band_check.cu: the warp-per-query search's FP32 squared
  distances from the hi/lo split against its 1e-5 FP64 re-decision band.
* tests/native/grad2_check.cu: the float-float order-2 derivative arithmetic
  (meshoid_gb300/csrc/mg_grad2.cuh, mg_ff.cuh) -- smoothing-length polish,
  float-float moments, right-hand sides and iterative refinement, the FP64
  factor / solve of re-solved rows -- against FP64 on balls, flattened
  neighbourhoods and tight clusters far from the origin.
* tests/native/spline_check.cu: spline_w_half (meshoid_gb300/csrc/mg_common.cuh),
  which the map tile kernels evaluate against a doubled coefficient, equal
  to spline_w / 2 bit for bit over every float in [1/4, 1.0625] and a
  stride below.
* tests/native/trunc_check.cu: trunc_pair32 (meshoid_gb300/csrc/mg_common.cuh),
  the FP32 decision behind the maps' footprints and the 3-D deposits' node
  ranges, equal to the reference's FP64 truncations whenever it decides, on
  random, near-integer and far-offset footprints.
* tests/native/sd_cull_check.cu: the large-footprint map kernel's skips
  (sd_block_skips, meshoid_gb300/csrc/mg_maps.cuh) change no pixel -- every
  node of a skipped sub-block evaluates q > 1 under the kernel's FP32
  arithmetic, its rsqrtf modelled to 2^-21 -- and nodes outside a
  footprint box weigh at most 1e-18 of the peak.
* tests/native/hsml_check.cu: the smoothing-length solver hsml_newton
  (meshoid_gb300/csrc/mg_hsml.cuh) on adversarial rows (clustered,
  coincident, equal and lattice-shell distances, six-decade ranges, k from 2
  to 128, 1-3 dimensions) against an FP64 bisection restating HsmlIter
  (src/meshoid/kernel_density.py:15-56), and for k <= 32 the float-float
  path (the early-stopping solve, then hsml_polish_ff) within 1e-10."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_and_run(tmp_path, name, defines=()):
    from meshoid_gb300 import build
    try:
        nvcc = build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / name)
    cmd = [nvcc, "-std=c++17", "-O2", *build.ARCH, "--expt-relaxed-constexpr", "-Xcompiler", "-ffp-contract=off",
           *defines, "-I", os.path.join(ROOT, "meshoid_gb300", "csrc"), "-o", exe,
           os.path.join(ROOT, "tests", "native", name + ".cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout


def test_refinement_helpers_on_the_host(tmp_path):
    _build_and_run(tmp_path, "refine_check")


def test_sweep_factor_and_condition_estimate_on_the_host(tmp_path):
    _build_and_run(tmp_path, "chol_check")


def test_first_pass_distance_bound_on_the_host(tmp_path):
    _build_and_run(tmp_path, "group_bound_check")


def test_warp_path_band_on_the_host(tmp_path):
    _build_and_run(tmp_path, "band_check")


def test_order2_float_float_on_the_host(tmp_path):
    _build_and_run(tmp_path, "grad2_check")


def test_deposit_node_decode_on_the_host(tmp_path):
    _build_and_run(tmp_path, "cube_check")


@pytest.mark.parametrize("compensated", [0, 1])
def test_hsml_solver_on_the_host(tmp_path, compensated):
    """The solver as built into the library (plain FP32 sum of n), and with
    the compensated sum staged behind MG_HSML_COMPENSATED."""
    _build_and_run(tmp_path, "hsml_check", [f"-DMG_HSML_COMPENSATED={compensated}"])


def test_half_spline_weight_on_the_host(tmp_path):
    _build_and_run(tmp_path, "spline_check")


def test_map_block_skips_on_the_host(tmp_path):
    _build_and_run(tmp_path, "sd_cull_check")


def test_footprint_truncations_on_the_host(tmp_path):
    _build_and_run(tmp_path, "trunc_check")
