"""GPU versions of holodeck/librarian/lib_tools.py:714-943 (``run_model``, ``_calc_model_details``)
and a writer of the combined library (librarian/combine.py:86-260) as ``.npz``, or HDF5 when h5py
is importable."""

import numpy as np

from .. import _device as D
from .. import _native as N
from .. import gravwaves, hardening, single_sources, utils
from ..constants import YR
from . import DEF_NUM_FBINS, DEF_NUM_LOUDEST, DEF_NUM_REALS, DEF_PTA_DUR


def _calc_model_details_device(edges, redz_final, number, h2fdf=None, cosmo=None):
    """Device version of :func:`_calc_model_details`; ``redz_final`` / ``number`` / ``h2fdf`` are
    device tensors.  Returns (gwb_pars, num_pars, gwb_mtot_redz_final, num_mtot_redz_final)."""
    t = D.torch()
    if h2fdf is None:
        h2fdf = gravwaves.char_strain_sq_device(edges, redz_final, cosmo=cosmo)
    nm, nq, nz = (int(np.size(e)) for e in edges[:3])
    nf = int(number.shape[-1])
    dev = number.device

    def new(*shape):
        return t.empty(shape, dtype=t.float64, device=dev)

    gwb_m, gwb_q, gwb_z, gwb_rz = new(nm - 1, nz - 1, nf), new(nq - 1, nz - 1, nf), new(nz - 1, nf), new(nz - 1, nf)
    num_m, num_q, num_z, num_rz = new(nm - 1, nz - 1, nf), new(nq - 1, nz - 1, nf), new(nz - 1, nf), new(nz - 1, nf)
    gwb_mrz, num_mrz, denom = new(nm - 1, nz - 1, nf), new(nm - 1, nz - 1, nf), new(nf)
    zedges = D.as_device(np.asarray(D.to_host(edges[2]) if D.is_torch(edges[2]) else edges[2], dtype=np.float64), dev)
    N.call("hgb_model_details", N.ptr(number.contiguous()), N.ptr(h2fdf.contiguous()), N.ptr(redz_final.contiguous()),
           N.ptr(zedges), nm, nq, nz, nf, N.ptr(gwb_m), N.ptr(gwb_q), N.ptr(gwb_z), N.ptr(gwb_rz), N.ptr(num_m),
           N.ptr(num_q), N.ptr(num_z), N.ptr(num_rz), N.ptr(gwb_mrz), N.ptr(num_mrz), N.ptr(denom),
           N.stream_handle())
    return [gwb_m, gwb_q, gwb_z, gwb_rz], [num_m, num_q, num_z, num_rz], gwb_mrz, num_mrz


def _calc_model_details(edges, redz_final, number):
    """Derived properties of a population (lib_tools.py:845-943): strain-weighted marginals of mtot,
    mrat and redz and of the final redshift, and the matching number marginals.

    Returns ``gwb_pars`` = [(M-1, Z-1, F), (Q-1, Z-1, F), (Z-1, F), (Z-1, F)], ``num_pars`` (same
    shapes), ``gwb_mtot_redz_final`` and ``num_mtot_redz_final`` (M-1, Z-1, F), as numpy arrays (or
    tensors when ``number`` is one).
    """
    like_torch = D.is_torch(number)
    out = _calc_model_details_device(edges, D.as_device(redz_final), D.as_device(number))
    if like_torch:
        return out
    gwb_pars, num_pars, gm, nmr = out
    return [D.to_host(x) for x in gwb_pars], [D.to_host(x) for x in num_pars], D.to_host(gm), D.to_host(nmr)


def run_model(sam, hard, pta_dur=DEF_PTA_DUR, nfreqs=DEF_NUM_FBINS, nreals=DEF_NUM_REALS, nloudest=DEF_NUM_LOUDEST,
              gwb_flag=True, singles_flag=True, details_flag=False, params_flag=False, log=None, seed=None):
    """One library sample (lib_tools.py:714-842): the dict a library simulation file holds.

    Keys: ``fobs_cents``, ``fobs_edges``; with ``details_flag`` ``static_binary_density``, ``number``,
    ``redz_final``, ``gwb_params``, ``num_params``, ``gwb_mtot_redz_final``, ``num_mtot_redz_final``;
    with ``params_flag`` ``sspar``, ``bgpar``; with ``singles_flag`` ``hc_ss``, ``hc_bg``; with
    ``gwb_flag`` ``gwb``.  ``seed`` (added) keys the Philox draws of the realizations.
    """
    if not any([gwb_flag, details_flag, singles_flag, params_flag]):
        err = f"No flags set!  {gwb_flag=} {details_flag=} {singles_flag=} {params_flag=}"
        if log is not None:
            log.exception(err)
        raise RuntimeError(err)
    data = {}
    fobs_cents, fobs_edges = utils.pta_freqs(dur=pta_dur * YR, num=nfreqs)
    fobs_orb_cents = fobs_cents / 2.0
    fobs_orb_edges = fobs_edges / 2.0
    data['fobs_cents'] = fobs_cents
    data['fobs_edges'] = fobs_edges
    if not isinstance(hard, (hardening.Fixed_Time_2PL_SAM, hardening.Hard_GW)):
        err = f"`holo.hardening.Fixed_Time_2PL_SAM` must be used here!  Not {hard}!"
        if log is not None:
            log.exception(err)
        raise RuntimeError(err)
    redz_final, diff_num = sam._dbn_device(hard, fobs_orb_cents)
    edges = [sam.mtot, sam.mrat, sam.redz, fobs_orb_edges]
    number, h2fdf = sam._number_and_strain(fobs_orb_edges, diff_num, redz_final)
    if details_flag:
        data['static_binary_density'] = sam.static_binary_density
        data['number'] = D.to_host(number)
        data['redz_final'] = D.to_host(redz_final)
        gwb_pars, num_pars, gm, nmr = _calc_model_details_device(edges, redz_final, number, h2fdf=h2fdf)
        data['gwb_params'] = [D.to_host(x) for x in gwb_pars]
        data['num_params'] = [D.to_host(x) for x in num_pars]
        data['gwb_mtot_redz_final'] = D.to_host(gm)
        data['num_mtot_redz_final'] = D.to_host(nmr)
    if singles_flag or params_flag:
        nloudest = nloudest if singles_flag else 1
        s1 = None if seed is None else int(seed)
        if params_flag:
            hc_ss, hc_bg, sspar, bgpar = single_sources.ss_params_device(edges, redz_final, number, h2fdf, nreals,
                                                                         nloudest, seed=s1, cosmo=sam._cosmo)
            data['sspar'] = D.to_host(sspar)
            data['bgpar'] = D.to_host(bgpar)
        else:
            hc_ss, hc_bg = single_sources.ss_realize_device(number, h2fdf, nreals, nloudest, seed=s1)
        if singles_flag:
            data['hc_ss'] = D.to_host(hc_ss)
            data['hc_bg'] = D.to_host(hc_bg)
    if gwb_flag:
        s2 = None if seed is None else (int(seed) ^ 0x5DEECE66D) & 0xFFFFFFFFFFFFFFFF
        gwb = gravwaves._gws_from_number_grid_integrated_redz(edges, redz_final, number, nreals, seed=s2,
                                                              cosmo=sam._cosmo)
        data['gwb'] = D.to_host(gwb)
    return data


def write_library(path, samples, sample_params, param_names, parameter_space_class_name="", gwb_only=False):
    """Combine per-sample :func:`run_model` dicts into one library file (combine.py:212-260 layout):
    ``fobs_cents``, ``fobs_edges``, ``sample_params`` (S, P), and stacked ``gwb`` (S, F, R),
    ``hc_ss`` (S, F, R, L), ``hc_bg`` (S, F, R), ``sspar`` (S, 4, F, R, L), ``bgpar`` (S, 7, F, R)
    where the samples have them; attributes ``param_names`` and ``parameter_space_class_name``.
    A missing sample (``None``) gives NaN rows and NaN parameters, as failed simulations do.
    Writes HDF5 when ``path`` ends in ``.hdf5`` / ``.h5`` (h5py required), else ``.npz``.
    """
    ok = [s for s in samples if s is not None]
    if not ok:
        raise ValueError("no sample results to combine")
    first = ok[0]
    sample_params = np.array(sample_params, dtype=np.float64, copy=True)
    keys = ['gwb'] if gwb_only else ['gwb', 'hc_ss', 'hc_bg', 'sspar', 'bgpar']
    out = {'fobs_cents': first['fobs_cents'], 'fobs_edges': first['fobs_edges']}
    for kk in keys:
        if kk not in first:
            continue
        arr = np.full((len(samples),) + np.shape(first[kk]), np.nan)
        for ii, res in enumerate(samples):
            if res is not None:
                arr[ii] = res[kk]
        out[kk] = arr
    for ii, res in enumerate(samples):
        if res is None:
            sample_params[ii] = np.nan
    out['sample_params'] = sample_params
    attrs = {'param_names': np.array(param_names).astype('S'), 'parameter_space_class_name': parameter_space_class_name}
    path = str(path)
    if path.endswith(('.hdf5', '.h5')):
        import h5py
        with h5py.File(path, 'w') as h5:
            for kk, vv in out.items():
                h5.create_dataset(kk, data=vv)
            for kk, vv in attrs.items():
                h5.attrs[kk] = vv
    else:
        np.savez(path, **out, **{f"attr_{kk}": vv for kk, vv in attrs.items()})
    return path
