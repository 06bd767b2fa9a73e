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


def test_schedule_knob_and_mlp_descriptions_checked_on_the_host(built_lib):
    """The realization kernels' waves knob and the MLP entry points validate their arguments before
    any CUDA call."""
    from holodeck_gb300 import _native as N
    lib = N.load()
    before = lib.hgb_get_bulk_waves()
    assert 1 <= before <= 16
    for bad in (0, -1, 17):
        assert lib.hgb_set_bulk_waves(bad) == N.HGB_ERR_INVALID_ARGUMENT
    assert lib.hgb_get_bulk_waves() == before
    assert lib.hgb_set_bulk_waves(before) == N.HGB_OK

    net = N.HgbMlp()
    net.n_layers, net.n_members = 5, 4
    for ii, d in enumerate([16, 256, 256, 256, 256, 160]):
        net.dims[ii] = d
    ref = ctypes.byref(net)
    # widths 16 -> 4 x 256 -> 160: W then b per layer
    assert lib.hgb_mlp_param_count(ref) == 16 * 256 + 256 + 3 * (256 * 256 + 256) + 256 * 160 + 160
    assert lib.hgb_mlp_weight_count(ref) == 16 * 256 + 3 * 256 * 256 + 256 * 160
    assert lib.hgb_mlp_backward_workspace_bytes(ref, 512) > 0
    # no parameter buffers: rejected before any launch
    assert lib.hgb_mlp_forward(ref, ctypes.c_void_p(16), 0, 8, ctypes.c_void_p(16), None, ctypes.c_void_p(16), None,
                               None) == N.HGB_ERR_INVALID_ARGUMENT
    for bad_dims in ([6, 256, 160], [16, 272, 160], [16, 8, 160]):   # widths must be multiples of 16 in [16, 256]
        bad = N.HgbMlp()
        bad.n_layers, bad.n_members = 2, 1
        for ii, d in enumerate(bad_dims):
            bad.dims[ii] = d
        assert lib.hgb_mlp_param_count(ctypes.byref(bad)) == -1
    none = N.HgbMlp()
    none.n_layers, none.n_members = 0, 1
    assert lib.hgb_mlp_param_count(ctypes.byref(none)) == -1


def test_batch_and_query_entry_points_check_arguments_on_the_host(built_lib):
    """The multi-sample realization launch, the fused forward and the native emulator query reject
    bad arguments before any CUDA call (no device pointer is dereferenced here)."""
    from holodeck_gb300 import _native as N
    lib = N.load()
    p = 256   # a non-null address that is never dereferenced: the checks return first
    ok = N.HgbLoudestSample(p, p, p, 100, 10, 1, p, p, p, 1 << 30, None)
    arr = (N.HgbLoudestSample * 1)(ok)
    bad = N.HgbLoudestSample(None, p, p, 100, 10, 1, p, p, p, 1 << 30, None)   # no number
    rc = lib.hgb_loudest_hc_batch((N.HgbLoudestSample * 1)(bad), 1, 4, 2, 0, p, 1 << 20, None)
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    rc = lib.hgb_loudest_hc_batch(arr, 1, 4, 2, 7, p, 1 << 20, None)           # blocks_per_sm above 6
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    rc = lib.hgb_loudest_hc_batch(arr, 1, 4, 256, 0, p, 1 << 20, None)         # nloud above 255
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    small = N.HgbLoudestSample(p, p, p, 100, 10, 1, p, p, p, 16, None)          # workspace too small
    rc = lib.hgb_loudest_hc_batch((N.HgbLoudestSample * 1)(small), 1, 4, 2, 0, p, 1 << 20, None)
    assert rc == N.HGB_ERR_WORKSPACE
    rc = lib.hgb_loudest_hc_batch(arr, 1, 4, 2, 0, p, 16, None)                 # batch workspace too small
    assert rc == N.HGB_ERR_WORKSPACE
    assert lib.hgb_loudest_batch_workspace_bytes(arr, 1, 4) > 0
    net = N.HgbMlp()
    net.n_layers, net.n_members = 2, 2
    for ii, d in enumerate((16, 32, 16)):
        net.dims[ii] = d
    net.params, net.weights = p, p
    rc = lib.hgb_mlp_forward_fused(ctypes.byref(net), p, 0, N.MLP_FUSED_MAX_BATCH + 1, p, None, None)
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    net.weights = p + 8                                                        # not 16-byte aligned
    rc = lib.hgb_mlp_forward_fused(ctypes.byref(net), p, 0, 1, p, None, None)
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    net.weights = p
    rc = lib.hgb_emulator_query(ctypes.byref(net), p, N.MLP_FUSED_MAX_BATCH + 1, 6, p, p, p, p, 10, p, p, p, p, None)
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    rc = lib.hgb_emulator_query(ctypes.byref(net), p, 1, 17, p, p, p, p, 10, p, p, p, p, None)   # > dims[0]
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    rc = lib.hgb_emulator_query(ctypes.byref(net), p, 1, 6, p, p, p, p, 17, p, p, p, p, None)    # > dims[L]
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    assert lib.hgb_error_string(N.HGB_ERR_DEVICE_LIMIT).startswith(b"a bounded device wait gave up")
