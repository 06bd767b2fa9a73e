"""GPU versions of holodeck/librarian/lib_tools.py:714-943 (``run_model``, ``_calc_model_details``),
the parameter-space classes that feed library runs (lib_tools.py:34-711: ``_Param_Space``,
``PD_Uniform``, ``PD_Normal``), and a writer of the combined library (librarian/combine.py:86-260) as
``.npz``, or HDF5 when h5py is importable."""

import abc
import logging

import numpy as np
import scipy as sp
import scipy.stats  # noqa: F401  (sp.stats.qmc, sp.stats.norm)

from .. import _device as D
from .. import _native as N
from .. import gravwaves, hardening, single_sources, utils
from ..constants import YR
from . import DEF_NUM_FBINS, DEF_NUM_LOUDEST, DEF_NUM_REALS, DEF_PTA_DUR


class _Param_Space(abc.ABC):
    """A library's parameter space (lib_tools.py:34-464): named parameter distributions, a Latin
    hypercube of ``nsamples`` draws over them, and the model (SAM + hardening) of any sample.

    The draws are scipy's ``LatinHypercube(d=P, strength=1, seed=seed)`` mapped through each
    distribution, exactly as lib_tools.py:136-141 makes them.  Subclasses set ``DEFAULTS`` and
    implement ``_init_sam(sam_shape, params)`` and ``_init_hard(sam, params)``.
    """

    DEFAULTS = {}

    def __init__(self, parameters, log=None, nsamples=None, sam_shape=None, seed=None, random_state=None):
        log = logging.getLogger("holodeck_gb300") if log is None else log
        try:
            nparameters = len(parameters)
            assert nparameters > 0
        except (TypeError, AssertionError) as err:
            log.exception("`parameters` must be a list of `_Param_Dist` subclasses!")
            raise err
        for param in parameters:
            if not isinstance(param, _Param_Dist):
                err = f"{param.name}: {param} is not a `_Param_Dist` object!"
                log.exception(err)
                raise ValueError(err)
        if nsamples is None:
            uniform_samples = None
            param_samples = None
        else:
            lhc = sp.stats.qmc.LatinHypercube(d=nparameters, strength=1, seed=seed)
            uniform_samples = lhc.random(n=nsamples)     # (S, P)
            param_samples = np.zeros_like(uniform_samples)
            for ii, param in enumerate(parameters):
                param_samples[:, ii] = param(uniform_samples[:, ii])
        self._log = log
        self._nparameters = nparameters
        self._nsamples = nsamples
        self._seed = seed
        self._random_state = random_state
        self.sam_shape = sam_shape
        self.param_names = [param.name for param in parameters]
        self.param_samples = param_samples
        self._parameters = parameters
        self._uniform_samples = uniform_samples

    def model_for_params(self, params, sam_shape=None):
        """(sam, hard) for a dict of parameter values; unnamed settings take ``DEFAULTS`` (lib_tools.py:156-213)."""
        if sam_shape is None:
            sam_shape = self.sam_shape
        settings = self.DEFAULTS.copy()
        for name, value in params.items():
            settings[name] = value
        sam = self._init_sam(sam_shape, settings)
        hard = self._init_hard(sam, settings)
        return sam, hard

    def param_dict(self, samp_num):
        return {nn: pp for nn, pp in zip(self.param_names, self.param_samples[samp_num])}

    @property
    def extrema(self):
        return np.asarray([dd.extrema for dd in self._parameters])

    @property
    def name(self):
        return self.__class__.__name__

    @property
    def lib_shape(self):
        return self.param_samples.shape

    @property
    def nsamples(self):
        return self._nsamples

    @property
    def nparameters(self):
        return self._nparameters

    def model_for_sample_number(self, samp_num, sam_shape=None):
        return self.model_for_params(self.param_dict(samp_num), sam_shape)

    def normalized_params(self, vals):
        """Parameters for fractional coordinates in [0, 1] (``None`` takes the default), lib_tools.py:409-451."""
        if np.ndim(vals) == 0:
            vals = self.nparameters * [vals]
        assert len(vals) == self.nparameters
        assert np.all([(vv is None) or np.isfinite(vv) for vv in vals]), f"Not all `vals` are finite!  {vals}"
        return {pname: (param.default if vv is None else param(vv))
                for pname, param, vv in zip(self.param_names, self._parameters, vals)}

    def default_params(self):
        return {param.name: param.default for param in self._parameters}

    @abc.abstractmethod
    def _init_sam(self, sam_shape, params):
        pass

    @abc.abstractmethod
    def _init_hard(self, sam, params):
        pass


class _Param_Dist(abc.ABC):
    """A parameter distribution: maps uniform [0, 1] draws to parameter values (lib_tools.py:467-517)."""

    def __init__(self, name, default=None, clip=None):
        if clip is not None:
            assert len(clip) == 2
        self._clip = clip
        self._name = name
        self._default = default

    def __call__(self, xx):
        rv = self._dist_func(xx)
        if self._clip is not None:
            rv = np.clip(rv, *self._clip)
        return rv

    @abc.abstractmethod
    def _dist_func(self, xx):
        pass

    @property
    def extrema(self):
        return self(np.asarray([0.0, 1.0]))

    @property
    def name(self):
        return self._name

    @property
    def default(self):
        return self._default if self._default is not None else self(0.5)


class PD_Uniform(_Param_Dist):
    """Uniform on [lo, hi] (lib_tools.py:520-530)."""

    def __init__(self, name, lo, hi, **kwargs):
        super().__init__(name, **kwargs)
        self._lo = lo
        self._hi = hi

    def _dist_func(self, xx):
        return self._lo + (self._hi - self._lo) * xx


class PD_Normal(_Param_Dist):
    """Normal(mean, stdev) through its inverse CDF (lib_tools.py:547-578)."""

    def __init__(self, name, mean, stdev, clip=None, **kwargs):
        assert stdev > 0.0
        super().__init__(name, clip=clip, **kwargs)
        self._mean = mean
        self._stdev = stdev
        self._dist = sp.stats.norm(loc=mean, scale=stdev)

    def _dist_func(self, xx):
        return self._dist.ppf(xx)


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
              gwb_flag=True, singles_flag=True, details_flag=False, params_flag=False, log=None, seed=None,
              precision="fp64"):
    """One library sample (lib_tools.py:714-842): the dict a library simulation file holds.

    Keys: ``fobs_cents``, ``fobs_edges``; with ``details_flag`` ``static_binary_density``, ``number``,
    ``redz_final``, ``gwb_params``, ``num_params``, ``gwb_mtot_redz_final``, ``num_mtot_redz_final``;
    with ``params_flag`` ``sspar``, ``bgpar``; with ``singles_flag`` ``hc_ss``, ``hc_bg``; with
    ``gwb_flag`` ``gwb``.  ``seed`` (added) keys the Philox draws of the realizations; ``precision``
    (added) selects the grid arithmetic as in :meth:`Semi_Analytic_Model.gwb`.
    """
    data, edges, number, h2fdf = run_model_grids(sam, hard, pta_dur=pta_dur, nfreqs=nfreqs, nreals=nreals,
                                                 gwb_flag=gwb_flag, singles_flag=singles_flag,
                                                 details_flag=details_flag, params_flag=params_flag, log=log,
                                                 seed=seed, precision=precision)
    if singles_flag or params_flag:
        nloudest = nloudest if singles_flag else 1
        s1 = None if seed is None else int(seed)
        if params_flag:
            hc_ss, hc_bg, sspar, bgpar = single_sources.ss_params_device(edges, data.pop('_redz_final_device'), number,
                                                                         h2fdf, nreals, nloudest, seed=s1,
                                                                         cosmo=sam._cosmo)
            data['sspar'] = D.to_host(sspar)
            data['bgpar'] = D.to_host(bgpar)
        else:
            hc_ss, hc_bg = single_sources.ss_realize_device(number, h2fdf, nreals, nloudest, seed=s1)
        if singles_flag:
            data['hc_ss'] = D.to_host(hc_ss)
            data['hc_bg'] = D.to_host(hc_bg)
    data.pop('_redz_final_device', None)
    return data


def run_model_grids(sam, hard, pta_dur=DEF_PTA_DUR, nfreqs=DEF_NUM_FBINS, nreals=DEF_NUM_REALS, gwb_flag=True,
                    singles_flag=True, details_flag=False, params_flag=False, log=None, seed=None, precision="fp64"):
    """Everything of :func:`run_model` but the single-source realizations: returns (data, edges,
    number, h2fdf) with ``data`` holding the frequencies, the details (``details_flag``) and ``gwb``
    (``gwb_flag``), and number / h2fdf the device grids the realizations draw from.  With
    ``params_flag`` data also carries the device redz_final under '_redz_final_device'."""
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
    redz_final, diff_num = sam._dbn_scheduled(hard, fobs_orb_cents, precision=precision)
    edges = [sam.mtot, sam.mrat, sam.redz, fobs_orb_edges]
    number, h2fdf = sam._number_and_strain(fobs_orb_edges, diff_num, redz_final, precision=precision)
    if details_flag:
        data['static_binary_density'] = sam.static_binary_density
        data['number'] = D.to_host(number)
        data['redz_final'] = D.to_host(redz_final)
        gwb_pars, num_pars, gm, nmr = _calc_model_details_device(edges, redz_final, number, h2fdf=h2fdf)
        data['gwb_params'] = [D.to_host(x) for x in gwb_pars]
        data['num_params'] = [D.to_host(x) for x in num_pars]
        data['gwb_mtot_redz_final'] = D.to_host(gm)
        data['num_mtot_redz_final'] = D.to_host(nmr)
    if gwb_flag:
        s2 = None if seed is None else (int(seed) ^ 0x5DEECE66D) & 0xFFFFFFFFFFFFFFFF
        gwb = gravwaves._gws_from_number_grid_integrated_redz(edges, redz_final, number, nreals, seed=s2,
                                                              cosmo=sam._cosmo)
        data['gwb'] = D.to_host(gwb)
    if params_flag:
        data['_redz_final_device'] = redz_final
    return data, edges, number, h2fdf


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
