"""Host-side helpers of the SAM path, mirroring the holodeck.utils functions it uses.

These act on the small 1-D axis arrays (grid edges, frequency bins) or on scalars, exactly where
holodeck's Python glue does; every grid-sized computation runs in the CUDA kernels.
"""

import numbers

import numpy as np

from . import constants as C


def pta_freqs(dur=16.03 * C.YR, num=40, cad=None):
    """Fourier bin centres and edges, utils.py:835-874: centres (i+1)/dur, edges (i+1/2)/dur."""
    fmin = 1.0 / dur
    if cad is not None:
        num = int(np.floor(dur / (2.0 * cad)))
    cents = np.arange(1, num + 2) * fmin
    edges = cents - fmin / 2.0
    return cents[:-1], edges


def midpoints(arr, axis=-1):
    """Arithmetic mean of neighbouring entries along ``axis`` (kalepy.utils.midpoints, linear)."""
    arr = np.moveaxis(np.asarray(arr), axis, -1)
    return np.moveaxis(0.5 * (arr[..., 1:] + arr[..., :-1]), -1, axis)


def isinteger(val):
    """utils.isinteger: integral scalar of an integer type."""
    return isinstance(val, (numbers.Integral, np.integer)) and not isinstance(val, bool)


def m1m2_from_mtmr(mt, mr):
    """utils.py:1620-1642"""
    mt = np.asarray(mt)
    mr = np.asarray(mr)
    m1 = mt / (1.0 + mr)
    return np.array([m1, mt - m1])


def chirp_mass_mtmr(mt, mr):
    """utils.py:1978-1997"""
    return mt * np.power(mr, 3.0 / 5.0) / np.power(1 + mr, 6.0 / 5.0)


def chirp_mass(m1, m2):
    """utils.py:1956-1975"""
    return np.power(np.asarray(m1) * np.asarray(m2), 3.0 / 5.0) / np.power(np.asarray(m1) + np.asarray(m2), 1.0 / 5.0)


def frst_from_fobs(fobs, redz):
    """utils.py:1645-1662"""
    return fobs * (1.0 + redz)


def gw_strain_source(mchirp, dcom, freq_rest_orb):
    """utils.py:2260-2285, [Sesana2004] Eq.36"""
    mchirp, dcom, freq_rest_orb = [np.asarray(v) for v in (mchirp, dcom, freq_rest_orb)]
    return C.GW_SRC_CONST * mchirp * np.power(2 * mchirp * freq_rest_orb, 2 / 3) / dcom


def _parse_val_log10_val_pars(val, val_log10, val_units=1.0, name="value", only_one=True):
    """utils.py:1299-1337"""
    if only_one and ((val_log10 is not None) == (val is not None)):
        raise ValueError(f"One of {name} OR {name}_log10 must be provided!  {name}={val}, {name}_log10={val_log10}")
    if val is None:
        val = val_units * np.power(10.0, val_log10)
    if val_log10 is None:
        val_log10 = np.log10(val / val_units)
    return val, val_log10


def get_subclass_instance(value, default, superclass, allow_none=False):
    """utils.get_subclass_instance: accept an instance, a subclass (instantiated) or None (default)."""
    import inspect
    if value is None:
        value = default
    if value is None:
        if allow_none:
            return None
        raise ValueError(f"A {superclass} instance is required!")
    if inspect.isclass(value):
        value = value()
    if not isinstance(value, superclass):
        raise ValueError(f"`value` ({value}) must be an instance of {superclass}!")
    return value
