"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/meshoid_gb300.h (no GPU needed: no compute calls)."""
import ctypes
import os
import re

import pytest

from meshoid_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "meshoid_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return ctypes.CDLL(build.LIB)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("mg_build_cells", "mg_knn_hsml", "mg_grad_sweep", "mg_kernel_average", "mg_surface_density",
                 "mg_nn_query", "mg_seed_plain", "mg_seed_features", "mg_mlp_forward", "mg_mlp_train_step"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_binding_table_matches_header():
    names = set(declared_functions())
    assert set(_native.SIGNATURES) <= names


def test_host_only_calls(lib):
    L = _native.load()
    assert L.mg_version() >= 100
    assert L.mg_status_string(0) == b"ok"
    assert 1 <= L.mg_default_grid_level(65536) <= 9
    assert L.mg_build_cells_workspace_bytes(1 << 20, 7) > 0
    assert L.mg_knn_hsml_workspace_bytes(1000, 32) > 0
    # process-wide switches: each call returns the previous setting
    import meshoid_gb300
    assert meshoid_gb300.set_order2_refinement(True) is False  # off by default
    assert meshoid_gb300.set_order2_refinement(False) is True
    assert L.mg_knn_set_group_pass(1) == 1 and L.mg_knn_set_group_pass(1) == 1
    assert L.mg_knn_set_persistent_passes(1) == 0 and L.mg_knn_set_persistent_passes(0) == 1  # off by default
    # argument validation happens before any device work
    c = _native.MgCells()
    c.n = 0
    assert L.mg_build_cells(None, ctypes.byref(c), None, 0, None) == _native.MG_ERR_ARG


def test_product_path_refuses_without_gpu(monkeypatch):
    import torch

    import meshoid_gb300
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(RuntimeError):
        meshoid_gb300.Meshoid([[0.0, 0.0, 0.0]] * 40)
