"""ctypes binding of the C ABI in ``include/holodeck_gb300.h`` (``_build/libholodeck_gb300.so``).

Every product function goes through here.  There is no CPU fallback: if the library cannot be
loaded, or no CUDA device is present, calls raise :class:`NativeUnavailable`.
"""

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libholodeck_gb300.so")
#: the same library built with -DHGB_BOUNDS_CHECK (holodeck_gb300.build.build(checked=True)); loaded
#: instead of LIB_PATH when HOLODECK_GB300_CHECKED=1 is set in the environment
CHECKED_LIB_PATH = os.path.join(_HERE, "_build_checked", "libholodeck_gb300.so")

HGB_OK = 0
HGB_ERR_INVALID_ARGUMENT = 1
HGB_ERR_CUDA = 2
HGB_ERR_WORKSPACE = 3
HGB_ERR_CAPACITY = 4
HGB_ERR_DEVICE_LIMIT = 5

STATUS_ITERATION_LIMIT = 1
STATUS_INVALID_REDSHIFT = 2
STATUS_TABLE_RANGE = 4
STATUS_GRADIENT_NOT_CONVERGED = 8
STATUS_BOUNDS = 16

RNG_PHILOX = 0
RNG_REPLAY = 1

GSMF_SCHECHTER = 0
GSMF_DOUBLE_SCHECHTER = 1
RATE_GPF_GMT = 0
RATE_GMR = 1

_d = ctypes.c_double
_i = ctypes.c_int
_l = ctypes.c_long
_p = ctypes.c_void_p
_sz = ctypes.c_size_t
_u64 = ctypes.c_uint64


class NativeUnavailable(RuntimeError):
    """The CUDA extension is missing or cannot run here."""


class HgbCosmo(ctypes.Structure):
    _fields_ = [
        ("H0", _d), ("Om0", _d), ("Ode0", _d), ("age_pref", _d), ("age_c1", _d), ("tz_c2", _d),
        ("age_limit", _d), ("hubble_distance", _d),
        ("grid_z", _p), ("grid_age", _p), ("grid_dcom", _p), ("grid_size", _i),
        ("dc_val", _p), ("dc_der", _p), ("dc_n", _i), ("dcg_val", _p), ("dcg_der", _p),
    ]


class HgbSamModel(ctypes.Structure):
    _fields_ = [
        ("gsmf_kind", _i), ("gsmf", _d * 11), ("rate_kind", _i), ("use_gmt", _i),
        ("gpf", _d * 6), ("gmt", _d * 5), ("gmr", _d * 11), ("mmb", _d * 4),
        ("gsmf_uses_mtot", _i), ("gpf_uses_mtot", _i), ("gmt_uses_mtot", _i),
    ]


class HgbScatterSizes(ctypes.Structure):
    _fields_ = [("n_pts", _i), ("n_tri", _i), ("n_nbr", _i), ("n_grid", _i), ("n_levels", _i)]


_SCATTER_ARRAYS = ["pts", "tri", "tri_kappa", "vtx_qinv", "nbr_ptr", "nbr_idx", "nbr_w", "level_ptr", "level_vtx",
                   "grid_tri", "grid_bary", "grid_near", "grid_axis", "weights", "back_idx", "back_t", "back_w",
                   "lv_nbr_ptr", "lv_nbr", "lv_nbr_w", "lv_qinv"]


class HgbScatterHostPlan(ctypes.Structure):
    _fields_ = [(name, _p) for name in _SCATTER_ARRAYS]


class HgbScatterPlan(ctypes.Structure):
    _fields_ = ([("n_mtot", _i), ("n_mrat", _i), ("n_grid", _i), ("n_tri", _i), ("n_levels", _i)] +
                [(name, _p) for name in _SCATTER_ARRAYS if name != "grid_axis"] +
                [("grad_tol", _d), ("grad_maxiter", _i)])


class HgbLoudestSample(ctypes.Structure):
    _fields_ = [("number", _p), ("h2fdf", _p), ("order", _p), ("n_bins", _l), ("nreals", _i), ("seed", _u64),
                ("hc2ss", _p), ("hc2bg", _p), ("workspace", _p), ("workspace_bytes", _sz), ("d_status", _p)]


MLP_MAX_LAYERS = 8       # HGB_MLP_MAX_LAYERS
MLP_SPLIT_ROWS = 128     # HGB_MLP_SPLIT_ROWS
MLP_FUSED_MAX_BATCH = 16 # HGB_MLP_FUSED_MAX_BATCH


class HgbMlp(ctypes.Structure):
    _fields_ = [("n_layers", _i), ("n_members", _i), ("dims", _i * (MLP_MAX_LAYERS + 1)), ("params", _p),
                ("weights", _p)]


#: (name, restype, argtypes) for every exported entry point
SIGNATURES = [
    ("hgb_version", _i, []),
    ("hgb_error_string", ctypes.c_char_p, [_i]),
    ("hgb_last_cuda_error", ctypes.c_char_p, []),
    ("hgb_static_density", _i, [ctypes.POINTER(HgbSamModel), ctypes.POINTER(HgbCosmo), _p, _i, _p, _i, _p, _i,
                                _p, _p, _p, _p, _p]),
    ("hgb_zero_stalled", _i, [_p, _p, _l, _p]),
    ("hgb_find_2pwl_hardening_norm", _i, [_d, _p, _p, _i, _d, _d, _d, _d, _i, _p, _p, _p, _p]),
    ("hgb_sqrt_inplace", _i, [_p, _l, _p]),
    ("hgb_scatter_plan_bounds", _i, [_i, _i, _i, ctypes.POINTER(HgbScatterSizes)]),
    ("hgb_scatter_plan_build", _i, [_p, _i, _p, _i, _i, _d, ctypes.POINTER(HgbScatterHostPlan),
                                    ctypes.POINTER(HgbScatterSizes)]),
    ("hgb_scatter_workspace_bytes", _sz, [_i, _i, _i, _i]),
    ("hgb_add_scatter_to_masses", _i, [ctypes.POINTER(HgbScatterPlan), _p, _i, _p, _sz, _p, _p]),
    ("hgb_dbn_2pwl", _i, [_p, _i, _i, _d, _i, _p, _d, _d, _d, _p, _p, _i, _p, _i, _p, _i, _p,
                          ctypes.POINTER(HgbCosmo), _p, _p, _p]),
    ("hgb_dbn_2pwl_phase", _i, [_p, _i, _i, _d, _i, _p, _d, _d, _d, _p, _p, _i, _p, _i, _p, _i, _p,
                                ctypes.POINTER(HgbCosmo), _p, _p, _i, _p]),
    ("hgb_dbn_2pwl_phase_f32", _i, [_p, _i, _i, _d, _i, _p, _d, _d, _d, _p, _p, _i, _p, _i, _p, _i, _p,
                                    ctypes.POINTER(HgbCosmo), _p, _p, _i, _p]),
    ("hgb_dbn_gw", _i, [_p, _i, _p, _p, _i, _p, _i, _i, _p, ctypes.POINTER(HgbCosmo), _p, _p, _p]),
    ("hgb_integrate_3dx1d", _i, [_p, _i, _p, _i, _p, _i, _p, _i, _p, _p, _p]),
    ("hgb_char_strain_sq", _i, [_p, _i, _p, _i, _i, _p, _i, _p, _d, ctypes.POINTER(HgbCosmo), _p, _p, _p]),
    ("hgb_number_and_strain", _i, [_p, _p, _i, _p, _i, _p, _i, _p, _p, _i, _p, _p, _d, ctypes.POINTER(HgbCosmo),
                                   _p, _p, _p, _p]),
    ("hgb_number_and_strain_f32", _i, [_p, _p, _i, _p, _i, _p, _i, _p, _p, _i, _p, _p, _d, ctypes.POINTER(HgbCosmo),
                                       _p, _p, _p, _p]),
    ("hgb_sort_workspace_bytes", _sz, [_l]),
    ("hgb_argsort_f0_desc", _i, [_p, _l, _i, _p, _p, _sz, _p]),
    ("hgb_argsort_f0_desc_static", _i, [_p, _l, _i, _p, _p]),
    ("hgb_loudest_workspace_bytes", _sz, [_l, _i, _i, _i, _i]),
    ("hgb_loudest_hc_from_sorted", _i, [_p, _p, _l, _i, _i, _i, _p, _i, _u64, _p, _p, _p, _p, _sz, _p, _p]),
    ("hgb_loudest_hc_from_sorted_ex", _i, [_p, _p, _l, _i, _i, _i, _p, _i, _u64, _p, _p, _p, _p, _sz, _p, _p, _i]),
    ("hgb_loudest_batch_workspace_bytes", _sz, [ctypes.POINTER(HgbLoudestSample), _i, _i]),
    ("hgb_loudest_hc_batch", _i, [ctypes.POINTER(HgbLoudestSample), _i, _i, _i, _i, _p, _sz, _p]),
    ("hgb_param_grids", _i, [_p, _i, _i, _i, _p, _i, _p, _d, ctypes.POINTER(HgbCosmo), _p, _p, _p, _p, _p, _p,
                             _p]),
    ("hgb_loudest_par_workspace_bytes", _sz, [_l, _i, _i, _i, _i]),
    ("hgb_loudest_hc_and_par_from_sorted", _i, [_p, _p, _i, _i, _i, _i, _i, _i, _p, _i, _u64, _p, _p, _p, _p, _p,
                                                _p, _p, _p, _p, _p, _p, _p, _p, _p, _sz, _p, _p]),
    ("hgb_model_details", _i, [_p, _p, _p, _p, _i, _i, _i, _i] + [_p] * 12),
    ("hgb_bulk_timing", _i, [_i]),
    ("hgb_bulk_last_ms", ctypes.c_float, []),
    ("hgb_set_bulk_waves", _i, [_i]),
    ("hgb_get_bulk_waves", _i, []),
    ("hgb_mlp_param_count", _l, [ctypes.POINTER(HgbMlp)]),
    ("hgb_mlp_weight_count", _l, [ctypes.POINTER(HgbMlp)]),
    ("hgb_mlp_forward", _i, [ctypes.POINTER(HgbMlp), _p, _l, _i, _p, _p, _p, _p, _p]),
    ("hgb_mlp_forward_fused", _i, [ctypes.POINTER(HgbMlp), _p, _l, _i, _p, _p, _p]),
    ("hgb_emulator_query", _i, [ctypes.POINTER(HgbMlp), _p, _i, _i, _p, _p, _p, _p, _i, _p, _p, _p, _p, _p]),
    ("hgb_mlp_backward_workspace_bytes", _sz, [ctypes.POINTER(HgbMlp), _i]),
    ("hgb_mlp_backward", _i, [ctypes.POINTER(HgbMlp), _p, _l, _i, _p, _p, _p, _p, _l, _p, _p, _p, _sz, _p, _p]),
    ("hgb_mlp_adamw", _i, [ctypes.POINTER(HgbMlp), _p, _p, _p, _p, _p, _i, ctypes.c_float, ctypes.c_float,
                           ctypes.c_float, ctypes.c_float, ctypes.c_float, _p]),
    ("hgb_mlp_pack_weights", _i, [ctypes.POINTER(HgbMlp), _p, _p, _p]),
    ("hgb_sam_poisson_gwb_workspace_bytes", _sz, [_l, _i, _i]),
    ("hgb_sam_poisson_gwb", _i, [_p, _p, _l, _i, _i, _i, _u64, _p, _p, _p, _sz, _p, _p]),
]

_LIB = None


def lib_path():
    return LIB_PATH


def load(path=None):
    """Load (once) and return the shared library; raises :class:`NativeUnavailable` if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if path is None:
        path = CHECKED_LIB_PATH if os.environ.get("HOLODECK_GB300_CHECKED") == "1" else LIB_PATH
    if not os.path.exists(path):
        raise NativeUnavailable(
            f"holodeck_gb300 CUDA extension not built ({path} missing); run holodeck_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def exported_symbols():
    return [name for name, _, _ in SIGNATURES]


class NativeError(RuntimeError):
    pass


def check_bounds(code, what):
    """Raise when a bounds-checked build flagged an index outside its array (HGB_STATUS_BOUNDS)."""
    if code & STATUS_BOUNDS:
        raise NativeError(f"{what}: an index left its array (device status HGB_STATUS_BOUNDS)")


def check(rc, what):
    if rc == HGB_OK:
        return
    lib = load()
    msg = lib.hgb_error_string(rc).decode()
    if rc == HGB_ERR_CUDA:
        msg += ": " + lib.hgb_last_cuda_error().decode()
    if rc == HGB_ERR_INVALID_ARGUMENT:
        raise ValueError(f"{what}: {msg}")
    raise NativeError(f"{what}: {msg} (code {rc})")


#: kernels each entry point launches (the radix argsort: a key gather, then a count, a scan and a
#: scatter per 8 key bits); used to report the launch count of a timed region
KERNELS_PER_CALL = {
    "hgb_static_density": 1, "hgb_zero_stalled": 1, "hgb_add_scatter_to_masses": 5,
    "hgb_find_2pwl_hardening_norm": 1, "hgb_sqrt_inplace": 1, "hgb_dbn_2pwl": 2, "hgb_dbn_2pwl_phase": 1, "hgb_dbn_2pwl_phase_f32": 1, "hgb_dbn_gw": 1,
    "hgb_integrate_3dx1d": 1, "hgb_char_strain_sq": 1, "hgb_number_and_strain": 1, "hgb_number_and_strain_f32": 1, "hgb_argsort_f0_desc": 25, "hgb_argsort_f0_desc_static": 25,
    "hgb_loudest_hc_from_sorted": 7, "hgb_loudest_hc_from_sorted_ex": 7, "hgb_sam_poisson_gwb": 3, "hgb_param_grids": 1, "hgb_model_details": 9,
    "hgb_loudest_hc_and_par_from_sorted": 6, "hgb_mlp_adamw": 1, "hgb_mlp_pack_weights": 1, "hgb_mlp_forward_fused": 1, "hgb_emulator_query": 1,
}
_launches = [0]
_launch_lock = threading.Lock()


def reset_launch_count():
    _launches[0] = 0


def launch_count():
    return _launches[0]


def add_launches(n):
    """Count kernels of a call whose launch count depends on its arguments."""
    with _launch_lock:
        _launches[0] += int(n)


def call(name, *args):
    """Call an entry point and raise on a non-zero return code."""
    fn = getattr(load(), name)
    check(fn(*args), name)
    with _launch_lock:
        _launches[0] += KERNELS_PER_CALL.get(name, 0)


def ptr(t):
    """Device pointer of a torch tensor (or None -> NULL)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def double_array(vals, n):
    arr = (ctypes.c_double * n)()
    vals = np.asarray(vals, dtype=np.float64).ravel()
    for ii, vv in enumerate(vals[:n]):
        arr[ii] = float(vv)
    return arr
