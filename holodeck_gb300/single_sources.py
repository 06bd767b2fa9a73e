"""GPU version of holodeck.single_sources.ss_gws_redz (single_sources.py:40-174)."""

import numpy as np

from . import _device as D
from . import _native as N
from . import constants as C
from . import cyutils, gravwaves, utils
from .cosmology import cosmo as _cosmo


def sort_order_device(h2fdf):
    """int32 loudest-first bin order at the first frequency (single_sources.py:89)."""
    t = D.torch()
    nf = int(h2fdf.shape[-1])
    nb = int(h2fdf.numel() // nf)
    order = t.empty(nb, dtype=t.int32, device=h2fdf.device)
    lib = N.load()
    ws_bytes = lib.hgb_sort_workspace_bytes(nb)
    ws = D.workspace(ws_bytes, h2fdf.device)
    N.call("hgb_argsort_f0_desc", N.ptr(h2fdf), nb, nf, N.ptr(order), N.ptr(ws), int(ws_bytes), N.stream_handle())
    return order


def check_redshift_status(st):
    code = st.read()
    N.check_bounds(code, "number and strain")
    if code & N.STATUS_INVALID_REDSHIFT:
        raise ValueError("redz < 0 and !=-1 found in redz, in ss_gws_redz()")


def ss_realize_device(number, h2fdf, realize, loudest, seed=None, replay=None, order=None):
    """Device (hc_ss[F, R, L], hc_bg[F, R]) from device number / h2fdf (M-1, Q-1, Z-1, F)."""
    nf = int(number.shape[-1])
    num = number.reshape(-1, nf)
    hh = h2fdf.reshape(-1, nf)
    if order is None:
        order = sort_order_device(h2fdf)
    else:
        order = cyutils.checked_order(order, h2fdf.numel() // h2fdf.shape[-1], h2fdf.device)
    st = D.StatusWord(number.device)
    hc2ss, hc2bg = cyutils.loudest_device(num, hh, int(realize), int(loudest), order, seed=seed, replay=replay,
                                          status=st)
    lib = N.load()
    N.call("hgb_sqrt_inplace", N.ptr(hc2ss), int(hc2ss.numel()), N.stream_handle())
    N.call("hgb_sqrt_inplace", N.ptr(hc2bg), int(hc2bg.numel()), N.stream_handle())
    cyutils._raise_status(st)
    return hc2ss, hc2bg


def ss_realize_batch_device(samples, loudest, blocks_per_sm=0):
    """:func:`ss_realize_device` (Philox draws) for many samples, their bulk backgrounds in one launch.
    ``samples``: list of (number, h2fdf, realize, seed), number / h2fdf (M_i-1, Q_i-1, Z_i-1, F) on
    the current device with one F.  Returns one entry per sample: (hc_ss[F, R, L], hc_bg[F, R]), or
    the exception that sample's status word raised (the others are unaffected)."""
    items = []
    for number, h2fdf, realize, seed in samples:
        nf = int(number.shape[-1])
        items.append(dict(number=number.reshape(-1, nf), h2fdf=h2fdf.reshape(-1, nf), order=sort_order_device(h2fdf),
                          nreals=int(realize), seed=seed, status=D.StatusWord(number.device)))
    outs = cyutils.loudest_batch_device(items, int(loudest), blocks_per_sm=blocks_per_sm)
    res = []
    for smp, (hc2ss, hc2bg) in zip(items, outs):
        N.call("hgb_sqrt_inplace", N.ptr(hc2ss), int(hc2ss.numel()), N.stream_handle())
        N.call("hgb_sqrt_inplace", N.ptr(hc2bg), int(hc2bg.numel()), N.stream_handle())
    for smp, (hc2ss, hc2bg) in zip(items, outs):
        try:
            cyutils._raise_status(smp["status"])
            res.append((hc2ss, hc2bg))
        except RuntimeError as exc:
            res.append(exc)
    return res


def param_grids_device(edges, redz, h2fdf=None, cosmo=None):
    """Device (redz_mid, dcom, sepa, angs), each (M-1, Q-1, Z-1, F), and the int32[4] frexp exponents of
    their largest finite magnitudes over the bins with nonzero strain (single_sources.py:117-143)."""
    t = D.torch()
    cosmo = _cosmo if cosmo is None else cosmo
    dc = D.device_cosmology(cosmo)
    mt = D.as_device(utils.midpoints(np.asarray(D.to_host(edges[0]) if D.is_torch(edges[0]) else edges[0])))
    fc = D.as_device(utils.midpoints(np.asarray(D.to_host(edges[3]) if D.is_torch(edges[3]) else edges[3])))
    nm, nq, nz, nf = int(np.size(edges[0])), int(np.size(edges[1])), int(redz.shape[2]), int(fc.numel())
    shape = (nm - 1, nq - 1, nz - 1, nf)
    grids = [t.empty(shape, dtype=t.float64, device=redz.device) for _ in range(4)]
    scales = t.empty(4, dtype=t.int32, device=redz.device)
    N.call("hgb_param_grids", N.ptr(mt), nm, nq, nz, N.ptr(fc), nf, N.ptr(redz), C.NWTG, dc.ref, N.ptr(h2fdf),
           *[N.ptr(g) for g in grids], N.ptr(scales), N.stream_handle())
    return grids, scales


def ss_params_device(edges, redz, number, h2fdf, realize, loudest, seed=None, replay=None, order=None, cosmo=None):
    """Device (hc_ss, hc_bg, sspar, bgpar) of the params=True branch (single_sources.py:102-161)."""
    grids, scales = param_grids_device(edges, redz, h2fdf=h2fdf, cosmo=cosmo)
    if order is None:
        order = sort_order_device(h2fdf)
    else:
        order = cyutils.checked_order(order, h2fdf.numel() // h2fdf.shape[-1], h2fdf.device)
    host = [np.asarray(D.to_host(e) if D.is_torch(e) else e, dtype=np.float64) for e in edges[:3]]
    mt, mr, rz = (utils.midpoints(e) for e in host)
    st = D.StatusWord(number.device)
    hc2ss, hc2bg, sspar, bgpar = cyutils.loudest_par_device(number, h2fdf, int(realize), int(loudest), order, mt, mr,
                                                            rz, grids, scales, seed=seed, replay=replay, status=st)
    N.call("hgb_sqrt_inplace", N.ptr(hc2ss), int(hc2ss.numel()), N.stream_handle())
    N.call("hgb_sqrt_inplace", N.ptr(hc2bg), int(hc2bg.numel()), N.stream_handle())
    cyutils._raise_status(st)
    z3 = sspar[3]
    bad = int(((z3 < 0) & (z3 != -1)).sum().item())
    if bad:
        raise ValueError(f"check 1: {bad} out of {z3.numel()} sspar[3] are negative and not -1 in sings.ss_gws_redz()")
    return hc2ss, hc2bg, sspar, bgpar


def ss_gws_redz(edges, redz, number, realize, loudest=1, params=False, seed=None, replay=None, order=None,
                cosmo=None):
    """Strain of the loudest single sources and of the background (single_sources.py:40-174).

    Returns ``hc_ss`` (F, R, L) and ``hc_bg`` (F, R), and with ``params=True`` also ``sspar``
    (4, F, R, L) and ``bgpar`` (7, F, R).  ``seed`` keys the Philox draws; ``replay`` (R, F, B) and
    ``order`` (B,) replay an externally drawn stream (see :mod:`holodeck_gb300.cyutils`).
    """
    like_torch = D.is_torch(number)
    rz = D.as_device(redz)
    st = D.StatusWord(rz.device)
    h2fdf = gravwaves.char_strain_sq_device(edges, rz, cosmo=cosmo, status=st)
    check_redshift_status(st)
    if not utils.isinteger(realize):
        raise Exception("`realize` ({}) must be an integer!")
    if params:
        out = ss_params_device(edges, rz, D.as_device(number), h2fdf, realize, loudest, seed=seed, replay=replay,
                               order=order, cosmo=cosmo)
        return out if like_torch else tuple(D.to_host(x) for x in out)
    hc_ss, hc_bg = ss_realize_device(D.as_device(number), h2fdf, realize, loudest, seed=seed, replay=replay,
                                     order=order)
    if like_torch:
        return hc_ss, hc_bg
    return D.to_host(hc_ss), D.to_host(hc_bg)
