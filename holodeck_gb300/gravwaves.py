"""GPU versions of the holodeck/gravwaves.py functions on the SAM path."""

import numpy as np

from . import _device as D
from . import _native as N
from . import constants as C
from . import cyutils
from .cosmology import cosmo as _cosmo


def _host(a):
    return np.asarray(D.to_host(a) if D.is_torch(a) else a, dtype=np.float64)


def char_strain_sq_device(edges, redz, cosmo=None, status=None):
    """Device h2fdf (M-1, Q-1, Z-1, F) from device redz_final (M, Q, Z, F)."""
    t = D.torch()
    cosmo = _cosmo if cosmo is None else cosmo
    dc = D.device_cosmology(cosmo)
    mt, mr, fe = D.as_device(edges[0]), D.as_device(edges[1]), D.as_device(edges[3])
    nm, nq, nz, nf = int(mt.numel()), int(mr.numel()), int(redz.shape[2]), int(fe.numel()) - 1
    out = t.empty((nm - 1, nq - 1, nz - 1, nf), dtype=t.float64, device=redz.device)
    st = status if status is not None else D.StatusWord(redz.device)
    N.call("hgb_char_strain_sq", N.ptr(mt), nm, N.ptr(mr), nq, nz, N.ptr(fe), nf, N.ptr(redz), C.GW_SRC_CONST,
           dc.ref, N.ptr(out), st.ptr, N.stream_handle())
    return out


def char_strain_sq_from_bin_edges_redz(edges, redz, cosmo=None):
    """h_s^2 f/df per bin and frequency; gravwaves.py:694-724."""
    assert len(edges) == 4
    assert np.all([np.ndim(ee) == 1 for ee in edges])
    like_torch = D.is_torch(redz)
    out = char_strain_sq_device(edges, D.as_device(redz), cosmo=cosmo)
    return out if like_torch else D.to_host(out)


def _gws_from_number_grid_integrated_redz(edges, redz, number, realize, sum=True, seed=None, replay=None,
                                          cosmo=None):
    """GWB characteristic strain of the whole grid (gravwaves.py:470-542): the `gwb` of the library runs."""
    like_torch = D.is_torch(number)
    hc2 = char_strain_sq_device(edges, D.as_device(redz), cosmo=cosmo)
    num = D.as_device(number)
    if realize is True:
        realize = 1
    if realize in [None, False]:
        out = hc2 * num
        if sum:
            out = out.sum(dim=(0, 1, 2))
    elif isinstance(realize, (int, np.integer)) and not isinstance(realize, bool):
        if not sum:
            raise NotImplementedError("per-bin realizations (sum=False) are not on the GPU path")
        out = cyutils.sam_poisson_gwb(num, hc2, int(realize), seed=seed, replay=replay)
    else:
        raise ValueError(f"`realize` ({realize}) must be one of {{True, False, integer}}!")
    lib = N.load()
    out = out.contiguous()
    N.call("hgb_sqrt_inplace", N.ptr(out), int(out.numel()), N.stream_handle())
    return out if like_torch else D.to_host(out)
