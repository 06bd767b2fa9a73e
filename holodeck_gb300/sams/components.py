"""SAM components: GSMF, galaxy pair fraction, merger time and merger rate (holodeck/sams/components.py).

Parameter holders with holodeck's names and defaults; the formulas run in the density kernel
(``csrc/hgb_density.cu``).
"""

import numpy as np

from .. import constants as C
from .. import utils
from ..cosmology import cosmo as _cosmo


class _Galaxy_Stellar_Mass_Function:
    pass


class _Galaxy_Pair_Fraction:
    pass


class _Galaxy_Merger_Time:
    pass


class _Galaxy_Merger_Rate:
    pass


class GSMF_Schechter(_Galaxy_Stellar_Mass_Function):
    """Single Schechter function, components.py:110-172."""

    def __init__(self, phi0=-2.77, phiz=-0.27, mchar0_log10=11.24, mchar0=None, mcharz=0.0, alpha0=-1.24,
                 alphaz=-0.03):
        mchar0, _ = utils._parse_val_log10_val_pars(mchar0, mchar0_log10, val_units=C.MSOL, name="mchar0",
                                                     only_one=True)
        self._phi0 = phi0
        self._phiz = phiz
        self._mchar0 = mchar0
        self._mcharz = mcharz
        self._alpha0 = alpha0
        self._alphaz = alphaz

    def _pack(self, model):
        from .._native import GSMF_SCHECHTER
        model.gsmf_kind = GSMF_SCHECHTER
        for ii, vv in enumerate([self._phi0, self._phiz, self._mchar0, self._mcharz, self._alpha0, self._alphaz]):
            model.gsmf[ii] = vv


class GSMF_Double_Schechter(_Galaxy_Stellar_Mass_Function):
    """Sum of two Schechter functions with quadratic redshift terms, components.py:276-330."""

    def __init__(self, log10_phi1=(-2.383, -0.264, -0.107), log10_phi2=(-2.818, -0.368, +0.046),
                 log10_mstar=(+10.767, +0.124, -0.033), alpha1=-0.28, alpha2=-1.48):
        self._log10_phi1 = list(log10_phi1)
        self._log10_phi2 = list(log10_phi2)
        self._log10_mstar = list(log10_mstar)
        self._alpha1 = alpha1
        self._alpha2 = alpha2

    def _pack(self, model):
        from .._native import GSMF_DOUBLE_SCHECHTER
        model.gsmf_kind = GSMF_DOUBLE_SCHECHTER
        vals = self._log10_phi1 + self._log10_phi2 + self._log10_mstar + [self._alpha1, self._alpha2]
        for ii, vv in enumerate(vals):
            model.gsmf[ii] = vv


class GPF_Power_Law(_Galaxy_Pair_Fraction):
    """Single power-law pair fraction, components.py:520-586."""

    def __init__(self, frac_norm_allq=0.025, frac_norm=None, mref=None, mref_log10=11.0, malpha=0.0, zbeta=0.8,
                 qgamma=0.0, obs_conv_qlo=0.25, max_frac=1.0):
        mref, _ = utils._parse_val_log10_val_pars(mref, mref_log10, val_units=C.MSOL, name="mref", only_one=True)
        if frac_norm is None:
            if frac_norm_allq is None:
                raise ValueError("If `frac_norm` is not given, `frac_norm_allq` is requried!")
            pw = qgamma + 1.0
            pair_norm = (1.00 ** pw - obs_conv_qlo ** pw) / pw
            frac_norm = frac_norm_allq / pair_norm
        if (max_frac < 0.0) or (1.0 < max_frac):
            raise ValueError(f"Given `max_frac`={max_frac:.4f} must be between [0.0, 1.0]!")
        self._frac_norm = frac_norm
        self._malpha = malpha
        self._zbeta = zbeta
        self._qgamma = qgamma
        self._max_frac = max_frac
        self._mref = mref

    def _pack(self, model):
        for ii, vv in enumerate([self._frac_norm, self._mref, self._malpha, self._zbeta, self._qgamma,
                                 self._max_frac]):
            model.gpf[ii] = vv


class GMT_Power_Law(_Galaxy_Merger_Time):
    """Power-law galaxy merger time, components.py:629-675 (mref = mref0 * 0.4 / h)."""

    def __init__(self, time_norm=0.55 * C.GYR, mref0=1.0e11 * C.MSOL, malpha=0.0, zbeta=-0.5, qgamma=0.0,
                 cosmo=None):
        cosmo = _cosmo if cosmo is None else cosmo
        self._time_norm = time_norm
        self._malpha = malpha
        self._zbeta = zbeta
        self._qgamma = qgamma
        self._mref = mref0 * (0.4 / cosmo.h)

    def _pack(self, model):
        for ii, vv in enumerate([self._time_norm, self._mref, self._malpha, self._zbeta, self._qgamma]):
            model.gmt[ii] = vv


class GMR_Illustris(_Galaxy_Merger_Rate):
    """Illustris galaxy merger rate (Rodriguez-Gomez+2015 Table 1), components.py:380-483."""

    def __init__(self, norm0_log10=None, normz=None, malpha0=None, malphaz=None, mdelta0=None, mdeltaz=None,
                 qgamma0=None, qgammaz=None, qgammam=None):
        dflt = dict(norm0_log10=-2.2287, normz=+2.4644, malpha0=+0.2241, malphaz=-1.1759, mdelta0=+0.7668,
                    mdeltaz=-0.4695, qgamma0=-1.2595, qgammaz=+0.0611, qgammam=-0.0477)
        vals = dict(norm0_log10=norm0_log10, normz=normz, malpha0=malpha0, malphaz=malphaz, mdelta0=mdelta0,
                    mdeltaz=mdeltaz, qgamma0=qgamma0, qgammaz=qgammaz, qgammam=qgammam)
        vals = {kk: (dflt[kk] if vv is None else vv) for kk, vv in vals.items()}
        self._norm0 = (10.0 ** vals["norm0_log10"]) / C.GYR
        self._normz = vals["normz"]
        self._malpha0 = vals["malpha0"]
        self._malphaz = vals["malphaz"]
        self._mdelta0 = vals["mdelta0"]
        self._mdeltaz = vals["mdeltaz"]
        self._qgamma0 = vals["qgamma0"]
        self._qgammaz = vals["qgammaz"]
        self._qgammam = vals["qgammam"]
        self._mref_delta = 2.0e11 * C.MSOL
        self._mref = 1.0e10 * C.MSOL

    def _pack(self, model):
        vals = [self._norm0, self._normz, self._malpha0, self._malphaz, self._mdelta0, self._mdeltaz,
                self._qgamma0, self._qgammaz, self._qgammam, self._mref_delta, self._mref]
        for ii, vv in enumerate(vals):
            model.gmr[ii] = vv
