"""M-Mbulge scatter of the binary density on the GPU (holodeck/sams/sam.py:1291-1394).

The grid geometry (triangulation, interpolation stencils, redistribution matrix) is built once per
(mtot, mrat, refine, scatter) by the native plan builder ``hgb_scatter_plan_build`` and cached on
the device; every call then runs the per-slice kernels of ``csrc/hgb_scatter.cu``.
"""

import collections
import ctypes
import logging
import threading
import warnings

import numpy as np

from .. import _device as D
from .. import _native as N

log = logging.getLogger("holodeck_gb300")

GRAD_TOL = 1e-6        # CloughTocher2DInterpolator default tolerance
GRAD_MAXITER = 400     # CloughTocher2DInterpolator default sweep limit

_DTYPES = dict(pts=np.float64, tri=np.int32, tri_kappa=np.float64, vtx_qinv=np.float64, nbr_ptr=np.int32,
               nbr_idx=np.int32, nbr_w=np.float64, level_ptr=np.int32, level_vtx=np.int32, grid_tri=np.int32,
               grid_bary=np.float64, grid_near=np.int32, grid_axis=np.float64, weights=np.float64,
               back_idx=np.int32, back_t=np.float64, back_w=np.float64, lv_nbr_ptr=np.int32, lv_nbr=np.int32,
               lv_nbr_w=np.float64, lv_qinv=np.float64)

_PLANS = collections.OrderedDict()   # least recently used first
_PLAN_CACHE_MAX = 8                   # plans kept per process (a 91 x 81 plan holds about 60 MB)
_PLAN_LOCK = threading.Lock()


def host_plan(mtot, mrat, scatter, refine=4):
    """Build the geometry on the host; returns (dict of numpy arrays trimmed to size, sizes)."""
    lib = N.load()
    mtot = np.ascontiguousarray(mtot, dtype=np.float64)
    mrat = np.ascontiguousarray(mrat, dtype=np.float64)
    b = N.HgbScatterSizes()
    N.check(lib.hgb_scatter_plan_bounds(mtot.size, mrat.size, int(refine), ctypes.byref(b)), "hgb_scatter_plan_bounds")
    npts, ntri, nnbr, ngrid, nlev = b.n_pts, b.n_tri, b.n_nbr, b.n_grid, b.n_levels
    shapes = dict(pts=(npts, 2), tri=(ntri, 3), tri_kappa=(ntri, 3), vtx_qinv=(npts, 4), nbr_ptr=(npts + 1,),
                  nbr_idx=(nnbr,), nbr_w=(nnbr, 4), level_ptr=(nlev + 1,), level_vtx=(npts,),
                  grid_tri=(ngrid * ngrid,), grid_bary=(ngrid * ngrid, 3), grid_near=(ngrid * ngrid,),
                  grid_axis=(ngrid,), weights=(ngrid, ngrid), back_idx=(npts, 2), back_t=(npts, 2),
                  back_w=(npts, 2, ngrid), lv_nbr_ptr=(npts + 1,), lv_nbr=(nnbr,), lv_nbr_w=(nnbr, 4), lv_qinv=(npts, 4))
    arrs = {kk: np.zeros(shapes[kk], dtype=_DTYPES[kk]) for kk in N._SCATTER_ARRAYS}
    hp = N.HgbScatterHostPlan(**{kk: arrs[kk].ctypes.data_as(ctypes.c_void_p) for kk in N._SCATTER_ARRAYS})
    sz = N.HgbScatterSizes()
    N.check(lib.hgb_scatter_plan_build(mtot.ctypes.data_as(ctypes.c_void_p), mtot.size,
                                       mrat.ctypes.data_as(ctypes.c_void_p), mrat.size, int(refine), float(scatter),
                                       ctypes.byref(hp), ctypes.byref(sz)), "hgb_scatter_plan_build")
    arrs["tri"] = arrs["tri"][:sz.n_tri]
    arrs["tri_kappa"] = arrs["tri_kappa"][:sz.n_tri]
    arrs["nbr_idx"] = arrs["nbr_idx"][:sz.n_nbr]
    arrs["nbr_w"] = arrs["nbr_w"][:sz.n_nbr]
    arrs["lv_nbr"] = arrs["lv_nbr"][:sz.n_nbr]
    arrs["lv_nbr_w"] = arrs["lv_nbr_w"][:sz.n_nbr]
    arrs["level_ptr"] = arrs["level_ptr"][:sz.n_levels + 1]
    return arrs, sz


class DevicePlan:
    """Device copy of a scatter plan and its ``hgb_scatter_plan`` struct."""

    def __init__(self, mtot, mrat, scatter, refine=4, dev=None):
        arrs, sz = host_plan(mtot, mrat, scatter, refine)
        t = D.torch()
        self.sizes = sz
        self.host = arrs
        self.dev = {kk: D.as_device(vv, dev, dtype=t.int32 if vv.dtype == np.int32 else t.float64)
                    for kk, vv in arrs.items()}
        s = N.HgbScatterPlan()
        s.n_mtot = int(np.size(mtot))
        s.n_mrat = int(np.size(mrat))
        s.n_grid = sz.n_grid
        s.n_tri = sz.n_tri
        s.n_levels = sz.n_levels
        for kk in N._SCATTER_ARRAYS:
            if kk != "grid_axis":
                setattr(s, kk, N.ptr(self.dev[kk]))
        s.grad_tol = GRAD_TOL
        s.grad_maxiter = GRAD_MAXITER
        self.struct = s
        # the copies ran on this thread's stream; the plan is shared through the cache with workers on
        # other streams, so it is complete before anyone can find it there
        t.cuda.current_stream(D.device(dev)).synchronize()


def device_plan(mtot, mrat, scatter, refine=4):
    key = (np.asarray(mtot, dtype=np.float64).tobytes(), np.asarray(mrat, dtype=np.float64).tobytes(),
           float(scatter), int(refine), str(D.device()))
    with _PLAN_LOCK:
        plan = _PLANS.get(key)
        if plan is not None:
            _PLANS.move_to_end(key)
            return plan
    # built outside the lock (the native builder releases the GIL), so workers build plans concurrently;
    # a caller keeps its plan alive until its kernels have run, whatever the cache evicts
    plan = DevicePlan(mtot, mrat, scatter, refine)
    with _PLAN_LOCK:
        plan = _PLANS.setdefault(key, plan)
        _PLANS.move_to_end(key)
        while len(_PLANS) > _PLAN_CACHE_MAX:
            _PLANS.popitem(last=False)
    return plan


def clear_plan_cache():
    """Drop the cached plans (their device memory is freed once no call holds them)."""
    with _PLAN_LOCK:
        _PLANS.clear()


def add_scatter_to_masses_device(mtot, mrat, dens, scatter, refine=4, tol=GRAD_TOL, maxiter=GRAD_MAXITER):
    """Scatter the device density tensor ``dens`` (M, Q, Z) in place.  ``tol`` / ``maxiter`` are the
    gradient solve's stopping rule and sweep limit (CloughTocher2DInterpolator's arguments of those
    names; the reference uses their defaults).  Running out of sweeps warns, as scipy does."""
    plan = device_plan(mtot, mrat, scatter, refine)
    struct = plan.struct
    if tol != GRAD_TOL or maxiter != GRAD_MAXITER:
        if not (tol > 0.0 and int(maxiter) >= 1):
            raise ValueError(f"tol must be > 0 and maxiter >= 1, got {tol=} {maxiter=}")
        struct = N.HgbScatterPlan.from_buffer_copy(plan.struct)   # the cached plan stays as built
        struct.grad_tol = float(tol)
        struct.grad_maxiter = int(maxiter)
    nz = int(dens.shape[2])
    lib = N.load()
    ws_bytes = lib.hgb_scatter_workspace_bytes(plan.struct.n_mtot, plan.struct.n_mrat, nz, plan.sizes.n_grid)
    ws = D.workspace(ws_bytes, dens.device)
    st = D.StatusWord(dens.device)
    N.call("hgb_add_scatter_to_masses", ctypes.byref(struct), N.ptr(dens), nz, N.ptr(ws), int(ws_bytes), st.ptr,
           N.stream_handle())
    code = st.read()
    N.check_bounds(code, "M-Mbulge scatter")
    if code & N.STATUS_GRADIENT_NOT_CONVERGED:
        warnings.warn("Gradient estimation did not converge, the results may be inaccurate")
    return dens


def add_scatter_to_masses(mtot, mrat, dens, scatter, refine=4, log=None, tol=GRAD_TOL, maxiter=GRAD_MAXITER):
    """Same arguments and result as holodeck.sams.sam.add_scatter_to_masses (numpy in, numpy out);
    ``tol`` / ``maxiter`` as in :func:`add_scatter_to_masses_device`."""
    assert np.ndim(dens) == 3
    assert np.shape(dens)[:2] == (np.size(mtot), np.size(mrat))
    like_torch = D.is_torch(dens)
    out = D.as_device(dens).clone()
    add_scatter_to_masses_device(mtot, mrat, out, scatter, refine, tol=tol, maxiter=maxiter)
    return out if like_torch else D.to_host(out)
