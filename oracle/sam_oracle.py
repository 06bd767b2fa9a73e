"""CPU oracle for the holodeck SAM gravitational-wave-background path.

TEST INFRASTRUCTURE ONLY.  This module restates the reference algorithm on
the CPU (numpy/scipy here, the loops in ``oracle_loops.c``).  Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use it, as the checker.  The ``holodeck_gb300`` product never
imports it.

It is pinned against the golden fixtures in ``tests/golden`` that the
reference itself produced (``tests/golden/make_golden.py``); the CPU tests
check every function below against them.

Parameter sets are plain dicts (see :func:`default_params`), so the oracle
shares no code with the product beyond the cosmology definition
(``holodeck_gb300.cosmology``), which is an input of both.
"""

import ctypes
import os
import subprocess

import numpy as np
import scipy.interpolate
import scipy.optimize
import scipy.stats

from holodeck_gb300 import constants as C
from holodeck_gb300.cosmology import cosmo as _cosmo

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

NORMAL_THRESHOLD = 1e10


def build(force=False):
    """Compile ``oracle_loops.c`` into ``oracle/_build/liboracle.so`` (gcc, no fused multiply-add)."""
    out_dir = os.path.join(_HERE, "_build")
    so = os.path.join(out_dir, "liboracle.so")
    src = os.path.join(_HERE, "oracle_loops.c")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        os.makedirs(out_dir, exist_ok=True)
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
                        "-o", so, src, "-lm"], check=True)
    return so


def lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build())
        d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        _LIB.orc_lifetime_2pwl.restype = d
        _LIB.orc_lifetime_2pwl.argtypes = [d, d, d, d, d, d, d, d, i]
        _LIB.orc_integrate_3dx1d.argtypes = [p, i, p, i, p, i, p, i, p, p]
        _LIB.orc_dbn_2pwl.argtypes = [p, i, d, i, p, d, d, d, p, p, i, p, i, p, i, p, p, p, p, i, p, p]
        _LIB.orc_dbn_gw.argtypes = [p, i, p, p, i, p, i, i, p, p, p, i, p, p]
        _LIB.orc_fill_loudest.argtypes = [i, p, p, i, p, p]
        _LIB.orc_fill_loudest_par.argtypes = [i, p, p, p, i, p, p, ctypes.c_long, p, p, ctypes.c_long]
        _LIB.orc_hard_func_2pwl_gw.argtypes = [i, p, p, p, p, d, d, d, p]
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---------------------------------------------------------------------------------------------
# Parameters
# ---------------------------------------------------------------------------------------------

def default_params(phi0=-2.77, phiz=-0.27, mchar0_log10=11.24, mcharz=0.0, alpha0=-1.24, alphaz=-0.03,
                   mamp_log10=8.69, mplaw=1.17, mref=1.0e11 * C.MSOL, scatter_dex=0.28, bulge_frac=0.615,
                   gpf_frac_norm_allq=0.025, gpf_mref_log10=11.0, gpf_malpha=0.0, gpf_zbeta=0.8,
                   gpf_qgamma=0.0, gpf_obs_conv_qlo=0.25, gpf_max_frac=1.0,
                   gmt_time_norm=0.55 * C.GYR, gmt_mref0=1.0e11 * C.MSOL, gmt_malpha=0.0, gmt_zbeta=-0.5,
                   gmt_qgamma=0.0, cosmo=None):
    """Parameters of GSMF_Schechter / GPF_Power_Law / GMT_Power_Law / MMBulge_KH2013 (their defaults)."""
    cosmo = _cosmo if cosmo is None else cosmo
    pw = gpf_qgamma + 1.0
    pair_norm = (1.0 ** pw - gpf_obs_conv_qlo ** pw) / pw                 # components.py:529-536
    return dict(
        phi0=phi0, phiz=phiz, mchar0=C.MSOL * np.power(10.0, mchar0_log10), mcharz=mcharz, alpha0=alpha0, alphaz=alphaz,
        mamp=C.MSOL * np.power(10.0, mamp_log10), mplaw=mplaw, mref=mref, scatter_dex=scatter_dex,
        bulge_frac=bulge_frac,
        gpf_frac_norm=gpf_frac_norm_allq / pair_norm, gpf_mref=C.MSOL * np.power(10.0, gpf_mref_log10),
        gpf_malpha=gpf_malpha, gpf_zbeta=gpf_zbeta, gpf_qgamma=gpf_qgamma, gpf_max_frac=gpf_max_frac,
        gmt_time_norm=gmt_time_norm, gmt_mref=gmt_mref0 * (0.4 / cosmo.h), gmt_malpha=gmt_malpha,
        gmt_zbeta=gmt_zbeta, gmt_qgamma=gmt_qgamma, cosmo=cosmo,
    )


def grid_edges(shape, mtot=(1.0e4 * C.MSOL, 1.0e12 * C.MSOL), mrat=(1e-3, 1.0), redz=(1e-3, 10.0)):
    """sam.py:195-218: log-spaced grid edges."""
    if np.isscalar(shape):
        shape = (shape,) * 3
    return [np.logspace(*np.log10(lim), nn) for lim, nn in zip([mtot, mrat, redz], shape)]


def pta_freqs(dur, num):
    """utils.py:835-874"""
    fmin = 1.0 / dur
    cents = np.arange(1, num + 2) * fmin
    edges = cents - fmin / 2.0
    return cents[:-1], edges


def midpoints(arr, axis=-1):
    arr = np.moveaxis(np.asarray(arr), axis, -1)
    return np.moveaxis(0.5 * (arr[..., 1:] + arr[..., :-1]), -1, axis)


# ---------------------------------------------------------------------------------------------
# Static binary density (a2 - a7)
# ---------------------------------------------------------------------------------------------

def mstar_from_mbh(mbh, p):
    """host_relations.py:768-771 -> _log10_relation_reverse (:1137-1178) -> BF_Constant (:190-192)"""
    xx = np.log10(mbh / p["mamp"])
    xx = (1.0 / p["mplaw"]) * xx
    mbulge = p["mref"] * np.power(10.0, xx)
    return mbulge / p["bulge_frac"]


def dmstar_dmbh(mstar, p):
    """host_relations.py:483-512 with MMBulge_Standard.dmbulge_dmbh (:718-741)"""
    mbulge = mstar * p["bulge_frac"]
    dmstar_dmbulge = 1.0 / p["bulge_frac"]
    yy = np.log10(mbulge / p["mref"]) * p["mplaw"]
    mbh = p["mamp"] * np.power(10.0, yy)
    return dmstar_dmbulge * (mbulge / (p["mplaw"] * mbh))


def mass_stellar(mtot, mrat, redz, p):
    """sam.py:250-278"""
    m1 = mtot[:, None] / (1.0 + mrat[None, :])
    m2 = mtot[:, None] - m1
    shape = (mtot.size, mrat.size, redz.size)
    mbh_pri = np.broadcast_to(m1[..., None], shape)
    mbh_sec = np.broadcast_to(m2[..., None], shape)
    mstar_pri = mstar_from_mbh(mbh_pri, p)
    mstar_sec = mstar_from_mbh(mbh_sec, p)
    return mstar_pri, mstar_sec / mstar_pri, mstar_pri + mstar_sec, np.broadcast_to(redz[None, None, :], shape)


def gsmf_schechter(mstar, redz, p):
    """components.py:132-172"""
    phi = np.power(10.0, p["phi0"] + p["phiz"] * redz)
    mchar = p["mchar0"] + p["mcharz"] * redz
    alpha = p["alpha0"] + p["alphaz"] * redz
    xx = mstar / mchar
    return np.log(10.0) * phi * np.power(xx, 1.0 + alpha) * np.exp(-xx)


def gpf_power_law(mass, mrat, redz, p):
    """components.py:556-586"""
    rv = p["gpf_frac_norm"] * np.power(mass / p["gpf_mref"], p["gpf_malpha"]) * \
        np.power(1.0 + redz, p["gpf_zbeta"]) * np.power(mrat, p["gpf_qgamma"])
    return np.clip(rv, None, p["gpf_max_frac"])


def gmt_power_law(mass, mrat, redz, p):
    """components.py:646-675"""
    return p["gmt_time_norm"] * np.power(mass / p["gmt_mref"], p["gmt_malpha"]) * \
        np.power(1.0 + redz, p["gmt_zbeta"]) * np.power(mrat, p["gmt_qgamma"])


def redz_after(time, redz, cosmo):
    """utils.py:1772-1808 (``_AGE_UNIVERSE_GYR`` round trip of utils.py:46 kept)"""
    age = cosmo.age(redz)
    new_age = age + time
    age_limit = (cosmo.age(0.0) / C.GYR) * C.GYR
    new_redz = -1.0 * np.ones_like(new_age)
    idx = new_age < age_limit
    new_redz[idx] = cosmo.tage_to_z(new_age[idx])
    return new_redz


def static_binary_density(mtot, mrat, redz, p, return_parts=False):
    """sam.py:280-398 for the GSMF / GPF / GMT / MMBulge combination."""
    cosmo = p["cosmo"]
    mstar_pri, mstar_rat, mstar_tot, rz = mass_stellar(mtot, mrat, redz, p)
    gmt_time = gmt_power_law(mstar_pri, mstar_rat, rz, p)
    zprime = redz_after(gmt_time, rz, cosmo)
    stalled = zprime < 0.0
    rate = gpf_power_law(mstar_pri, mstar_rat, rz, p) / gmt_time
    dens = gsmf_schechter(mstar_pri, rz, p) * rate * cosmo.dtdz(rz)
    mplaw = p["mplaw"]
    dqbh_dqgal = mplaw * np.power(mstar_rat, mplaw - 1.0)
    dmstar_dmbh_pri = dmstar_dmbh(mstar_pri, p)
    qterm = (1.0 + mstar_rat) / (1.0 + mrat[None, :, None])
    dens = dens * ((mtot[:, None, None] / mstar_tot) * (dmstar_dmbh_pri * qterm / dqbh_dqgal))
    dens_noscatter = dens.copy()
    if p["scatter_dex"] > 0.0:
        dens = add_scatter_to_masses(mtot, mrat, dens, p["scatter_dex"])
    dens[stalled] = 0.0
    if return_parts:
        return dict(density=dens, gmt_time=gmt_time, redz_prime=zprime, density_noscatter=dens_noscatter)
    return dens


def scatter_weights(log_cents, scatter):
    """utils.py:410-488: (N, N) redistribution matrix with rows = source bins."""
    num = log_cents.size
    dx = np.diff(log_cents)[0]
    dx = dx / 2.0 + np.arange(num) * dx
    dx = np.concatenate([-dx[::-1], dx])
    dm = np.diff(scipy.stats.norm(loc=0.0, scale=scatter).cdf(dx))
    # weights[i, k] = dm[(k - i) + num - 1]
    idx = np.arange(num)[None, :] - np.arange(num)[:, None] + num - 1
    return dm[idx]


def add_scatter_to_masses(mtot, mrat, dens, scatter, refine=4):
    """sam.py:1291-1394 with the same scipy interpolants."""
    output = np.zeros_like(dens)
    m1 = mtot[:, None] / (1.0 + mrat[None, :])
    m2 = mtot[:, None] - m1
    points = (np.log10(m1.flatten()), np.log10(m2.flatten()))
    grid_size = m1.shape[0] * refine
    lo = 0.9 * mtot[0] * mrat[0] / (1.0 + mrat[0])
    hi = mtot[-1] * (1.0 + mrat[0]) / mrat[0]
    mextr = [min(lo, hi), max(lo, hi)]
    mgrid_log10 = np.log10(np.logspace(*np.log10(mextr), grid_size))
    m1m2_grid = np.meshgrid(mgrid_log10, mgrid_log10, indexing="ij")
    weights = scatter_weights(mgrid_log10, scatter)
    tri = None
    for ii in range(dens.shape[2]):
        vals = dens[:, :, ii].flatten()
        interp = scipy.interpolate.CloughTocher2DInterpolator(points if tri is None else tri, vals)
        tri = interp.tri if tri is None else tri
        grid = interp(tuple(m1m2_grid))
        bads = np.isnan(grid) | (grid < 0.0)
        if np.any(bads):
            near = scipy.interpolate.NearestNDInterpolator(tri if False else points, vals)(tuple(m1m2_grid))
            grid[bads] = near[bads]
        grid = np.einsum("j...,jk...", grid, weights)
        grid = np.moveaxis(np.einsum("j...,jk...", np.moveaxis(grid, 1, 0), weights), 0, 1)
        back = scipy.interpolate.RegularGridInterpolator((mgrid_log10, mgrid_log10), grid)
        output[:, :, ii] = back(points, method="linear").reshape(m1.shape)
    return output


# ---------------------------------------------------------------------------------------------
# Hardening normalisation (a8) and differential number (a9, a10)
# ---------------------------------------------------------------------------------------------

def find_2pwl_hardening_norm(time, mtot, mrat, sepa_init, rchar, gamma_inner, gamma_outer, nsteps):
    """sam_cyutils.pyx:289-353: one Brent root per cell on [-20, 20], xtol 1e-3, rtol 1e-5, 100 iterations."""
    L = lib()
    mtot, mrat = np.asarray(mtot, float).ravel(), np.asarray(mrat, float).ravel()
    out = np.zeros(mtot.size)
    for ii in range(mtot.size):
        fn = lambda x, mt=mtot[ii], mr=mrat[ii]: L.orc_lifetime_2pwl(
            x, time, mt, mr, sepa_init, rchar, gamma_inner, gamma_outer, nsteps)
        out[ii] = scipy.optimize.brentq(fn, -20.0, 20.0, xtol=1e-3, rtol=1e-5, maxiter=100, disp=False)
    return out


def hard_func_2pwl_gw(mtot, mrat, sepa, norm, rchar, gamma_inner, gamma_outer):
    args = [_c64(a).ravel() for a in np.broadcast_arrays(mtot, mrat, sepa, norm)]
    out = np.zeros(args[0].size)
    lib().orc_hard_func_2pwl_gw(out.size, *[_ptr(a) for a in args], rchar, gamma_inner, gamma_outer, _ptr(out))
    return out.reshape(np.broadcast(mtot, mrat, sepa, norm).shape)


def dbn_2pwl(fobs_orb, sepa_init, num_steps, norm, rchar, gamma_inner, gamma_outer, dens, mtot, mrat, redz,
             gmt_time, cosmo=None):
    """sam_cyutils.pyx:510-781"""
    cosmo = _cosmo if cosmo is None else cosmo
    fobs_orb, norm, dens, mtot, mrat, redz, gmt_time = map(_c64, [fobs_orb, norm, dens, mtot, mrat, redz, gmt_time])
    zg, dg, ag = map(_c64, [cosmo._grid_z, cosmo._grid_dcom, cosmo._grid_age])
    shape = dens.shape + (fobs_orb.size,)
    redz_final = -1.0 * np.ones(shape)
    dnum = np.zeros(shape)
    rc = lib().orc_dbn_2pwl(_ptr(fobs_orb), fobs_orb.size, sepa_init, int(num_steps), _ptr(norm), rchar,
                            gamma_inner, gamma_outer, _ptr(dens), _ptr(mtot), mtot.size, _ptr(mrat), mrat.size,
                            _ptr(redz), redz.size, _ptr(gmt_time), _ptr(zg), _ptr(dg), _ptr(ag), zg.size,
                            _ptr(redz_final), _ptr(dnum))
    assert rc == 0
    return redz_final, dnum


def dbn_gw(fobs_orb, dens, mtot, mrat, redz_prime, cosmo=None):
    """sam_cyutils.pyx:788-899"""
    cosmo = _cosmo if cosmo is None else cosmo
    fobs_orb, dens, mtot, mrat, redz_prime = map(_c64, [fobs_orb, dens, mtot, mrat, redz_prime])
    zg, dg = map(_c64, [cosmo._grid_z, cosmo._grid_dcom])
    shape = dens.shape + (fobs_orb.size,)
    redz_final = -1.0 * np.ones(shape)
    dnum = np.zeros(shape)
    lib().orc_dbn_gw(_ptr(fobs_orb), fobs_orb.size, _ptr(dens), _ptr(mtot), mtot.size, _ptr(mrat), mrat.size,
                     dens.shape[2], _ptr(redz_prime), _ptr(zg), _ptr(dg), zg.size, _ptr(redz_final), _ptr(dnum))
    return redz_final, dnum


# ---------------------------------------------------------------------------------------------
# Integration (a11), strain (a12), realizations (a13, a14)
# ---------------------------------------------------------------------------------------------

def integrate_differential_number_3dx1d(edges, dnum):
    """sam_cyutils.pyx:115-216"""
    dnum = _c64(dnum)
    lm, mr, rz = _c64(np.log10(edges[0])), _c64(edges[1]), _c64(edges[2])
    dlnf = _c64(np.diff(np.log(edges[3])))
    assert dnum.shape == (lm.size, mr.size, rz.size, dlnf.size)
    out = np.zeros((lm.size - 1, mr.size - 1, rz.size - 1, dlnf.size))
    lib().orc_integrate_3dx1d(_ptr(lm), lm.size, _ptr(mr), mr.size, _ptr(rz), rz.size, _ptr(dlnf), dlnf.size,
                              _ptr(dnum), _ptr(out))
    return out


def chirp_mass_mtmr(mt, mr):
    """utils.py:1978-1997"""
    return mt * np.power(mr, 3.0 / 5.0) / np.power(1 + mr, 6.0 / 5.0)


def char_strain_sq_from_bin_edges_redz(edges, redz, cosmo=None):
    """gravwaves.py:694-724"""
    cosmo = _cosmo if cosmo is None else cosmo
    foo = edges[-1]
    df = np.diff(foo)
    fc = midpoints(foo)
    for dd in range(3):
        redz = midpoints(redz, axis=dd)
    mc = chirp_mass_mtmr(midpoints(edges[0])[:, None], midpoints(edges[1])[None, :])[:, :, None, None]
    dc = np.inf * np.ones_like(redz)
    sel = redz > 0.0
    dc[sel] = cosmo.comoving_distance(redz[sel])
    fr = fc[None, None, None, :] * (1.0 + redz)
    hs = C.GW_SRC_CONST * mc * np.power(2 * mc * fr, 2 / 3) / dc
    return (hs ** 2) * (fc / df)


def sort_order(h2fdf):
    """single_sources.py:89: argsort of -h2fdf at the first frequency."""
    return np.argsort(-h2fdf[..., 0].flatten())


def draw_counts(rng, lam_sorted, thresh=NORMAL_THRESHOLD):
    """The numpy draws ``_loudest_hc_from_sorted`` makes for one (realization, frequency)
    (cyutils.pyx:1326-1332): Poisson below the threshold, Normal above, in bin order."""
    big = np.flatnonzero(lam_sorted > thresh)
    if big.size == 0:
        return rng.poisson(lam_sorted).astype(np.float64)
    out = np.empty(lam_sorted.size)
    start = 0
    for jj in big:
        out[start:jj] = rng.poisson(lam_sorted[start:jj])
        out[jj] = rng.normal(lam_sorted[jj], np.sqrt(lam_sorted[jj]))
        start = jj + 1
    out[start:] = rng.poisson(lam_sorted[start:])
    return out


def replay_counts(number, order, nreals, seed):
    """All counts in the reference's draw order, shaped (R, F, B) in sorted-bin order."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nf = number.shape[-1]
    lam = number.reshape(-1, nf)[order]                  # (B, F)
    out = np.empty((nreals, nf, lam.shape[0]))
    for rr in range(nreals):
        for ff in range(nf):
            out[rr, ff] = draw_counts(rng, lam[:, ff])
    return out


def loudest_hc_from_sorted(number, h2fdf, nreals, nloudest, order, seed=None, counts=None):
    """cyutils.pyx:1220-1344: returns (hc2ss[F, R, L], hc2bg[F, R])."""
    L = lib()
    nf = number.shape[-1]
    lam = _c64(number.reshape(-1, nf)[order].T)          # (F, B)
    hh = _c64(h2fdf.reshape(-1, nf)[order].T)
    nb = lam.shape[1]
    hc2ss = np.zeros((nf, nreals, nloudest))
    hc2bg = np.zeros((nf, nreals))
    rng = None if counts is not None else np.random.Generator(np.random.PCG64(seed))
    ss = np.zeros(nloudest)
    bg = np.zeros(1)
    for rr in range(nreals):
        for ff in range(nf):
            num = _c64(counts[rr, ff] if counts is not None else draw_counts(rng, lam[ff]))
            ss[:] = 0.0
            L.orc_fill_loudest(nb, _ptr(hh[ff]), _ptr(num), nloudest, _ptr(ss), _ptr(bg))
            hc2ss[ff, rr] = ss
            hc2bg[ff, rr] = bg[0]
    return hc2ss, hc2bg


def ss_gws_redz(edges, redz, number, realize, loudest=1, seed=None, counts=None, cosmo=None):
    """single_sources.py:40-174 (params=False branch)."""
    h2fdf = char_strain_sq_from_bin_edges_redz(edges, redz, cosmo=cosmo)
    order = sort_order(h2fdf)
    if np.any(np.logical_and(redz < 0, redz != -1)):
        raise ValueError(f"{np.sum(np.logical_and(redz < 0, redz != -1))} redz < 0 and !=-1 found in redz")
    if not isinstance(realize, (int, np.integer)):
        raise Exception("`realize` must be an integer!")
    hc2ss, hc2bg = loudest_hc_from_sorted(number, h2fdf, realize, loudest, order, seed=seed, counts=counts)
    return np.sqrt(hc2ss), np.sqrt(hc2bg)


def param_grids(edges, redz, cosmo=None):
    """single_sources.py:117-143: bin-centre final redshift (-1 where <= 0), comoving distance
    (+inf there), Kepler separation at the rest-frame orbital frequency, angular separation."""
    cosmo = _cosmo if cosmo is None else cosmo
    mt = midpoints(edges[0])
    for dd in range(3):
        redz = midpoints(redz, axis=dd)
    redz = np.array(redz)
    dcom = np.inf * np.ones_like(redz)
    sel = redz > 0.0
    redz[~sel] = -1.0
    redz[redz < 0] = -1.0
    dcom[sel] = cosmo.comoving_distance(redz[sel])
    fobs_orb_cents = midpoints(edges[-1])
    frst = fobs_orb_cents[np.newaxis, np.newaxis, np.newaxis, :] * (1.0 + redz)
    with np.errstate(divide="ignore", invalid="ignore"):
        sepa = np.power(C.NWTG * mt[:, np.newaxis, np.newaxis, np.newaxis] / np.square(2.0 * np.pi * frst), 1.0 / 3.0)
        angs = sepa / (dcom / (1.0 + redz))
    return redz, dcom, sepa, angs


def loudest_hc_and_par_from_sorted(number, h2fdf, nreals, nloudest, order, pars, seed=None, counts=None):
    """cyutils.pyx:1541-1770: (hc2ss[F,R,L], hc2bg[F,R], sspar[4,F,R,L], bgpar[7,F,R]); ``pars`` is the
    list of the seven (B, F) parameter grids (mt, mr, rz broadcast, redz, dcom, sepa, angs)."""
    L = lib()
    nf = number.shape[-1]
    lam = _c64(number.reshape(-1, nf)[order].T)
    hh = _c64(h2fdf.reshape(-1, nf)[order].T)
    pp = _c64(np.stack([np.broadcast_to(p, number.shape).reshape(-1, nf)[order].T for p in pars], axis=1))  # (F,7,B)
    nb = lam.shape[1]
    hc2ss = np.zeros((nf, nreals, nloudest))
    hc2bg = np.zeros((nf, nreals))
    sspar = np.zeros((4, nf, nreals, nloudest))
    bgpar = np.zeros((7, nf, nreals))
    rng = None if counts is not None else np.random.Generator(np.random.PCG64(seed))
    ss = np.zeros(nloudest)
    sp = np.zeros((4, nloudest))
    bg = np.zeros(1)
    bp = np.zeros(7)
    with np.errstate(divide="ignore", invalid="ignore"):
        for rr in range(nreals):
            for ff in range(nf):
                num = _c64(counts[rr, ff] if counts is not None else draw_counts(rng, lam[ff]))
                ss[:] = 0.0
                sp[:] = 0.0
                par = _c64(pp[ff])
                L.orc_fill_loudest_par(nb, _ptr(hh[ff]), _ptr(num), _ptr(par), nloudest, _ptr(ss), _ptr(sp),
                                       nloudest, _ptr(bg), _ptr(bp), 1)
                hc2ss[ff, rr] = ss
                hc2bg[ff, rr] = bg[0]
                sspar[:, ff, rr] = sp
                bgpar[:, ff, rr] = bp
    return hc2ss, hc2bg, sspar, bgpar


def ss_gws_redz_params(edges, redz, number, realize, loudest=1, seed=None, counts=None, cosmo=None):
    """single_sources.py:40-174 (params=True branch): (hc_ss, hc_bg, sspar, bgpar)."""
    h2fdf = char_strain_sq_from_bin_edges_redz(edges, redz, cosmo=cosmo)
    order = sort_order(h2fdf)
    if np.any(np.logical_and(redz < 0, redz != -1)):
        raise ValueError(f"{np.sum(np.logical_and(redz < 0, redz != -1))} redz < 0 and !=-1 found in redz")
    rz_m, dcom, sepa, angs = param_grids(edges, redz, cosmo=cosmo)
    mt, mr, rz = midpoints(edges[0]), midpoints(edges[1]), midpoints(edges[2])
    pars = [mt[:, None, None, None], mr[None, :, None, None], rz[None, None, :, None], rz_m, dcom, sepa, angs]
    hc2ss, hc2bg, sspar, bgpar = loudest_hc_and_par_from_sorted(number, h2fdf, realize, loudest, order, pars,
                                                                seed=seed, counts=counts)
    return np.sqrt(hc2ss), np.sqrt(hc2bg), sspar, bgpar


def calc_model_details(edges, redz_final, number, cosmo=None):
    """lib_tools.py:845-943: strain-weighted and number marginals of mtot, mrat, redz and of the final
    redshift at bin centres (binned on the redz edges with scipy.stats.binned_statistic)."""
    redz = edges[2]
    nm, nz, nf = len(edges[0]) - 1, len(redz) - 1, len(edges[3]) - 1
    w = char_strain_sq_from_bin_edges_redz(edges, redz_final, cosmo=cosmo) * number
    denom = np.sum(w, axis=(0, 1, 2))
    gwb_pars, num_pars = [], []
    for axes in [(1,), (0,), (0, 1)]:
        gwb_pars.append(np.sum(w, axis=axes) / denom)
        num_pars.append(np.sum(number, axis=axes))
    rz = redz_final.copy()
    for ii in range(3):
        rz = midpoints(rz, axis=ii)
    g_m, n_m = np.zeros((nm, nz, nf)), np.zeros((nm, nz, nf))
    g_rz, n_rz = np.zeros((nz, nf)), np.zeros((nz, nf))
    for ff in range(nf):
        flat = rz[..., ff].flatten()
        g_rz[:, ff] = scipy.stats.binned_statistic(flat, w[..., ff].flatten(), bins=redz, statistic='sum')[0] / denom[ff]
        n_rz[:, ff] = scipy.stats.binned_statistic(flat, number[..., ff].flatten(), bins=redz, statistic='sum')[0]
        for mm in range(nm):
            flat = rz[mm, :, :, ff].flatten()
            g_m[mm, :, ff] = scipy.stats.binned_statistic(flat, w[mm, :, :, ff].flatten(), bins=redz,
                                                          statistic='sum')[0] / denom[ff]
            n_m[mm, :, ff] = scipy.stats.binned_statistic(flat, number[mm, :, :, ff].flatten(), bins=redz,
                                                          statistic='sum')[0]
    gwb_pars.append(g_rz)
    num_pars.append(n_rz)
    return gwb_pars, num_pars, g_m, n_m


def sam_poisson_gwb(number, hc2, nreals, seed, thresh=NORMAL_THRESHOLD):
    """cyutils.pyx:854-897: loop order M, Q, Z, F outer and R inner, no loudest split."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nf = number.shape[-1]
    lam = number.reshape(-1, nf)
    hh = hc2.reshape(-1, nf)
    gwb = np.zeros((nf, nreals))
    for bb in range(lam.shape[0]):
        for ff in range(nf):
            bn = lam[bb, ff]
            if bn > thresh:
                num = rng.normal(bn, np.sqrt(bn), size=nreals)
            else:
                num = rng.poisson(bn, size=nreals).astype(np.float64)
            for rr in range(nreals):
                gwb[ff, rr] += num[rr] * hh[bb, ff]
    return gwb


def gwb(fobs_gw_edges, mtot, mrat, redz, p, hard, realize, loudest, seed, counts=None):
    """sam.py:872-947.  ``hard`` is None (GW-only) or a dict with the Fixed_Time_2PL_SAM parameters."""
    parts = static_binary_density(mtot, mrat, redz, p, return_parts=True)
    fobs_gw_cents = midpoints(fobs_gw_edges)
    fobs_orb_edges = fobs_gw_edges / 2.0
    fobs_orb_cents = fobs_gw_cents / 2.0
    if hard is None:
        redz_final, dnum = dbn_gw(fobs_orb_cents, parts["density"], mtot, mrat, parts["redz_prime"], p["cosmo"])
    else:
        mt, mr = np.meshgrid(mtot, mrat, indexing="ij")
        norm = 10.0 ** find_2pwl_hardening_norm(hard["time"], mt.ravel(), mr.ravel(), hard["sepa_init"],
                                                hard["rchar"], hard["gamma_inner"], hard["gamma_outer"],
                                                hard["num_steps"]).reshape(mt.shape)
        redz_final, dnum = dbn_2pwl(fobs_orb_cents, hard["sepa_init"], hard["num_steps"], norm, hard["rchar"],
                                    hard["gamma_inner"], hard["gamma_outer"], parts["density"], mtot, mrat,
                                    redz, parts["gmt_time"], p["cosmo"])
    edges = [mtot, mrat, redz, fobs_orb_edges]
    number = integrate_differential_number_3dx1d(edges, dnum)
    hc_ss, hc_bg = ss_gws_redz(edges, redz_final, number, realize, loudest, seed=seed, counts=counts,
                               cosmo=p["cosmo"])
    return hc_ss, hc_bg
