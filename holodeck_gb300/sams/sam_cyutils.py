"""GPU versions of holodeck/sams/sam_cyutils.pyx (same names and arguments).

Arrays may be numpy arrays (results come back as numpy, like the reference) or CUDA tensors
(results stay on the device).
"""

import numpy as np

from .. import _device as D
from .. import _native as N
from ..cosmology import cosmo as _cosmo


def _out(t, like_torch):
    return t if like_torch else D.to_host(t)


def find_2pwl_hardening_norm(time, mtot, mrat, sepa_init, rchar, gamma_inner, gamma_outer, nsteps,
                             return_norm=False):
    """log10 hardening normalisation per cell (sam_cyutils.pyx:289-321); ``mtot``/``mrat`` are 1-D."""
    assert np.ndim(time) == 0
    assert np.ndim(mtot) == 1
    assert np.shape(mtot) == np.shape(mrat)
    like_torch = D.is_torch(mtot)
    mt = D.as_device(mtot)
    mr = D.as_device(mrat)
    t = D.torch()
    nl = t.empty_like(mt)
    norm = t.empty_like(mt)
    st = D.StatusWord()
    N.call("hgb_find_2pwl_hardening_norm", float(time), N.ptr(mt), N.ptr(mr), int(mt.numel()), float(sepa_init),
           float(rchar), float(gamma_inner), float(gamma_outer), int(nsteps), N.ptr(nl), N.ptr(norm), st.ptr,
           N.stream_handle())
    if return_norm:
        return _out(nl, like_torch), _out(norm, like_torch)
    return _out(nl, like_torch)


def dynamic_binary_number_at_fobs(fobs_orb, sam, hard, cosmo=None):
    """(redz_final, diff_num), each (M, Q, Z, F); sam_cyutils.pyx:421-504."""
    like_torch = D.is_torch(fobs_orb)
    redz_final, diff_num = sam._dbn_device(hard, fobs_orb, cosmo=cosmo)
    return _out(redz_final, like_torch), _out(diff_num, like_torch)


PRECISIONS = ("fp64", "fp32")


def check_precision(precision):
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {precision!r}")
    return precision


def dbn_2pwl_device(fobs_orb, hard, dens, mtot, mrat, redz, gmt_time, cosmo=None, phase=3, out=None,
                    precision="fp64"):
    """Device arrays in, device (redz_final, diff_num) out (sam_cyutils.pyx:510-781).

    ``phase`` 1 runs only the separation-step walk (``dens`` may be None; the outputs then hold the
    bracketing step and time, see hgb_dbn_2pwl_phase), 2 only the evaluation into ``out`` from
    phase 1, 3 both.  ``precision="fp32"`` evaluates the residence time in FP32 (the walk and the
    age -> redshift inversion stay FP64; hgb_dbn_2pwl_phase_f32).
    """
    t = D.torch()
    cosmo = _cosmo if cosmo is None else cosmo
    dc = D.device_cosmology(cosmo)
    fo = D.as_device(fobs_orb)
    nf = int(fo.numel())
    if D.is_torch(fobs_orb):
        sorted_ok = int(bool(t.all(fo[1:] >= fo[:-1]).item())) if nf > 1 else 1
    else:   # host input: decide on the host, no device round trip
        fh = np.asarray(fobs_orb, dtype=np.float64).ravel()
        sorted_ok = int(bool(np.all(fh[1:] >= fh[:-1])))
    if out is None:
        grid = (int(mtot.numel()), int(mrat.numel()), int(redz.numel()))
        redz_final = t.empty(grid + (nf,), dtype=t.float64, device=mtot.device)
        diff_num = t.empty(grid + (nf,), dtype=t.float64, device=mtot.device)
    else:
        redz_final, diff_num = out
    norm = D.as_device(hard._norm_device())
    fn = "hgb_dbn_2pwl_phase" if check_precision(precision) == "fp64" else "hgb_dbn_2pwl_phase_f32"
    N.call(fn, N.ptr(fo), nf, sorted_ok, float(hard._sepa_init), int(hard._num_steps),
           N.ptr(norm), float(hard._rchar), float(hard._gamma_inner), float(hard._gamma_outer), N.ptr(dens),
           N.ptr(mtot), int(mtot.numel()), N.ptr(mrat), int(mrat.numel()), N.ptr(redz), int(redz.numel()),
           N.ptr(gmt_time), dc.ref, N.ptr(redz_final), N.ptr(diff_num), int(phase), N.stream_handle())
    return redz_final, diff_num


def dbn_gw_device(fobs_orb, dens, mtot, mrat, redz_prime, cosmo=None):
    """Device arrays in, device (redz_final, diff_num) out (sam_cyutils.pyx:788-899)."""
    t = D.torch()
    cosmo = _cosmo if cosmo is None else cosmo
    dc = D.device_cosmology(cosmo)
    fo = D.as_device(fobs_orb)
    nf = int(fo.numel())
    shape = tuple(dens.shape) + (nf,)
    redz_final = t.empty(shape, dtype=t.float64, device=dens.device)
    diff_num = t.empty(shape, dtype=t.float64, device=dens.device)
    N.call("hgb_dbn_gw", N.ptr(fo), nf, N.ptr(dens), N.ptr(mtot), int(mtot.numel()), N.ptr(mrat),
           int(mrat.numel()), int(dens.shape[2]), N.ptr(redz_prime), dc.ref, N.ptr(redz_final), N.ptr(diff_num),
           N.stream_handle())
    return redz_final, diff_num


def integrate_differential_number_3dx1d(edges, dnum):
    """number (M-1, Q-1, Z-1, F) from dnum (M, Q, Z, F) (sam_cyutils.pyx:115-167)."""
    shape = [len(ee) for ee in edges]
    err = f"Shape of edges={shape} does not match dnum={tuple(dnum.shape)}"
    shape[-1] -= 1
    assert tuple(dnum.shape) == tuple(shape), err
    like_torch = D.is_torch(dnum)
    number = integrate_device(edges, D.as_device(dnum))
    return _out(number, like_torch)


def _axis_host(edges):
    """The axis arrays the reference's Python wrapper prepares (sam_cyutils.pyx:163-165)."""
    e0 = np.asarray(edges[0].cpu() if D.is_torch(edges[0]) else edges[0], dtype=np.float64)
    e3 = np.asarray(edges[3].cpu() if D.is_torch(edges[3]) else edges[3], dtype=np.float64)
    return np.log10(e0), np.diff(np.log(e3))


def integrate_device(edges, dnum):
    t = D.torch()
    lm, dlnf = _axis_host(edges)
    lm, mr, rz, dlnf = D.as_device(lm), D.as_device(edges[1]), D.as_device(edges[2]), D.as_device(dlnf)
    out = t.empty((lm.numel() - 1, mr.numel() - 1, rz.numel() - 1, dlnf.numel()), dtype=t.float64,
                  device=dnum.device)
    N.call("hgb_integrate_3dx1d", N.ptr(lm), int(lm.numel()), N.ptr(mr), int(mr.numel()), N.ptr(rz),
           int(rz.numel()), N.ptr(dlnf), int(dlnf.numel()), N.ptr(dnum), N.ptr(out), N.stream_handle())
    return out
