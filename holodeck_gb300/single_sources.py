"""GPU version of holodeck.single_sources.ss_gws_redz (single_sources.py:40-174)."""

import numpy as np

from . import _device as D
from . import _native as N
from . import cyutils, gravwaves, utils


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
        order = D.as_device(order, dtype=D.torch().int32)
    st = D.StatusWord(number.device)
    hc2ss, hc2bg = cyutils.loudest_device(num, hh, int(realize), int(loudest), order, seed=seed, replay=replay,
                                          status=st)
    lib = N.load()
    N.call("hgb_sqrt_inplace", N.ptr(hc2ss), int(hc2ss.numel()), N.stream_handle())
    N.call("hgb_sqrt_inplace", N.ptr(hc2bg), int(hc2bg.numel()), N.stream_handle())
    cyutils._raise_status(st)
    return hc2ss, hc2bg


def ss_gws_redz(edges, redz, number, realize, loudest=1, params=False, seed=None, replay=None, order=None,
                cosmo=None):
    """Strain of the loudest single sources and of the background (single_sources.py:40-174).

    Returns ``hc_ss`` (F, R, L) and ``hc_bg`` (F, R).  ``seed`` keys the Philox draws; ``replay``
    (R, F, B) and ``order`` (B,) replay an externally drawn stream (see :mod:`holodeck_gb300.cyutils`).
    """
    if params:
        raise NotImplementedError("params=True (sspar/bgpar) is not on the GPU path yet")
    if not utils.isinteger(realize):
        raise Exception("`realize` ({}) must be an integer!")
    like_torch = D.is_torch(number)
    rz = D.as_device(redz)
    st = D.StatusWord(rz.device)
    h2fdf = gravwaves.char_strain_sq_device(edges, rz, cosmo=cosmo, status=st)
    check_redshift_status(st)
    hc_ss, hc_bg = ss_realize_device(D.as_device(number), h2fdf, realize, loudest, seed=seed, replay=replay,
                                     order=order)
    if like_torch:
        return hc_ss, hc_bg
    return D.to_host(hc_ss), D.to_host(hc_bg)
