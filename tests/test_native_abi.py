"""The C-ABI library builds, loads without a GPU and exports every entry point of include/holodeck_gb300.h."""

import ctypes
import os
import re

from conftest import ROOT


def header_functions():
    text = open(os.path.join(ROOT, "include", "holodeck_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hgb_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = header_functions()
    for required in ["hgb_static_density", "hgb_find_2pwl_hardening_norm", "hgb_dbn_2pwl", "hgb_dbn_gw",
                     "hgb_integrate_3dx1d", "hgb_char_strain_sq", "hgb_number_and_strain", "hgb_argsort_f0_desc",
                     "hgb_loudest_hc_from_sorted", "hgb_sam_poisson_gwb"]:
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    from holodeck_gb300 import _native
    lib = ctypes.CDLL(_native.LIB_PATH)
    missing = [nn for nn in header_functions() if not hasattr(lib, nn)]
    assert not missing, f"declared but not exported: {missing}"
    assert sorted(_native.exported_symbols()) == header_functions()


def test_library_answers_without_a_gpu(built_lib):
    from holodeck_gb300 import _native
    assert built_lib.hgb_version() >= 1
    assert built_lib.hgb_error_string(_native.HGB_ERR_INVALID_ARGUMENT) == b"invalid argument"
    # argument errors are caught on the host before any CUDA call
    rc = built_lib.hgb_integrate_3dx1d(None, 0, None, 0, None, 0, None, 0, None, None, None)
    assert rc == _native.HGB_ERR_INVALID_ARGUMENT
    rc = built_lib.hgb_loudest_hc_from_sorted(None, None, 10, 2, 3, 1, None, 0, 0, None, None, None, None, 0, None,
                                              None)
    assert rc == _native.HGB_ERR_INVALID_ARGUMENT


def test_product_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "holodeck_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(dirpath, fn)).read()
                assert "oracle" not in re.sub(r"#.*|//.*", "", text).replace("the oracle", ""), fn
