"""The GPU path against the reference at the three plain-SAM workloads it is measured on:

* the 30^3 grid, 20 frequencies, 100 realizations, 5 loudest (``ref_cfg1.npz``);
* the default 91x81x101 grid, 40 frequencies, 10 loudest, 2 seeded realizations (``ref_cfg2.npz``);
* the 181x161x201 grid, 100 frequencies (``ref_cfg5.npz``, expectations only).

Every fixture was made by running the reference (``tests/golden/make_golden.py``).  Grids and their
per-frequency sums are compared at RTOL_GRID; the strains of replayed realizations (numpy PCG64
draws fed in the reference's visiting order) at RTOL_HC.  The FP64 contract is 1e-6 relative; the
measured agreement is far tighter, so the tests hold the tighter bounds.
"""

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import sam_oracle as O

pytestmark = pytest.mark.gpu

RTOL_GRID = 1e-9
RTOL_HC = 1e-8


def _model(g, scatter=0.28):
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    gsmf = H.sams.GSMF_Schechter(phi0=-2.77, mchar0_log10=11.24, alpha0=-1.24)
    mmb = H.host_relations.MMBulge_KH2013(mamp_log10=8.69, mplaw=1.17, scatter_dex=scatter)
    shape = (g["mtot"].size, g["mrat"].size, g["redz"].size)
    sam = H.sams.Semi_Analytic_Model(gsmf=gsmf, gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=mmb, shape=shape)
    sam.mtot, sam.mrat, sam.redz = g["mtot"], g["mrat"], g["redz"]
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5)
    return sam, hard


def _grids(sam, hard, fobs_gw_edges):
    """Device (redz_final, dnum, number, h2fdf) of gwb()'s grid stages."""
    fo_c = 0.5 * (fobs_gw_edges[1:] + fobs_gw_edges[:-1]) / 2.0
    redz_final, dnum = sam._dbn_device(hard, fo_c)
    number, h2fdf = sam._number_and_strain(fobs_gw_edges / 2.0, dnum, redz_final)
    return redz_final, dnum, number, h2fdf


def _strided(t, step):
    return t[::step, ::step, ::step, :].cpu().numpy()


def _check_slices(g, redz_final, dnum, number=None, h2fdf=None, step=None):
    rf = _strided(redz_final, step)
    assert np.array_equal(rf == -1.0, g["redz_final_slice"] == -1.0)
    assert rel_err(rf, g["redz_final_slice"]) < RTOL_GRID
    assert rel_err(_strided(dnum, step), g["dnum_slice"]) < RTOL_GRID
    if number is not None:
        assert rel_err(_strided(number, step), g["number_slice"]) < RTOL_GRID
        hh = _strided(h2fdf, step)
        assert np.array_equal(hh == 0.0, g["h2fdf_slice"] == 0.0)
        assert rel_err(hh, g["h2fdf_slice"]) < RTOL_GRID


def _sums(dnum, number, h2fdf):
    return (dnum.sum((0, 1, 2)).cpu().numpy(), number.sum((0, 1, 2)).cpu().numpy(),
            (number * h2fdf).sum((0, 1, 2)).cpu().numpy())


def test_cfg1_end_to_end(built_lib):
    """30^3 grid: the grids, their sums, the loudest-first order and the strain of the reference's
    100 seeded realizations (its PCG64(0) draws replayed through gwb())."""
    g = load_golden("ref_cfg1.npz")
    sam, hard = _model(g)
    fe = g["fobs_gw_edges"]
    assert rel_err(hard._norm, g["norm"]) < RTOL_GRID
    assert rel_err(sam.static_binary_density, g["density"]) < RTOL_GRID
    redz_final, dnum, number, h2fdf = _grids(sam, hard, fe)
    _check_slices(g, redz_final, dnum, step=7)
    d_sum, n_sum, hc2_sum = _sums(dnum, number, h2fdf)
    assert rel_err(d_sum, g["dnum_sum_f"]) < RTOL_GRID
    assert rel_err(n_sum, g["number_sum_f"]) < RTOL_GRID
    assert rel_err(hc2_sum, g["mean_hc2_f"]) < RTOL_GRID
    from holodeck_gb300 import single_sources
    order = single_sources.sort_order_device(h2fdf).cpu().numpy()
    key = h2fdf[..., 0].reshape(-1).cpu().numpy()
    head = g["order_head"]
    untied = np.concatenate([[True], np.diff(key[head]) != 0]) & np.concatenate([np.diff(key[head]) != 0, [True]])
    assert np.array_equal(order[:head.size][untied], head[untied])
    # the reference's draws: numpy PCG64(0) Poisson draws in the reference's visiting order, from the
    # oracle's expectations (bit-identical to the reference's on the machine that made the fixture;
    # numpy's argsort orders tied keys differently across machines, hence the stored order)
    mtot, mrat, redz = g["mtot"], g["mrat"], g["redz"]
    p = O.default_params(scatter_dex=0.28)
    hard_o = dict(time=float(hard._target_time), sepa_init=float(hard._sepa_init), rchar=float(hard._rchar),
                  gamma_inner=-1.0, gamma_outer=2.5, num_steps=int(hard._num_steps))
    parts = O.static_binary_density(mtot, mrat, redz, p, return_parts=True)
    rf_o, dn_o = O.dbn_2pwl(0.25 * (fe[1:] + fe[:-1]), hard_o["sepa_init"], hard_o["num_steps"], g["norm"],
                            hard_o["rchar"], -1.0, 2.5, parts["density"], mtot, mrat, redz, parts["gmt_time"])
    edges_o = [mtot, mrat, redz, fe / 2.0]
    number_o = O.integrate_differential_number_3dx1d(edges_o, dn_o)
    assert rel_err(number_o.sum((0, 1, 2)), g["number_sum_f"]) < 1e-13
    ref_order = g["order"].astype(np.int64)
    assert np.array_equal(ref_order[:head.size], head)
    counts = O.replay_counts(number_o, ref_order, int(g["nreals"]), int(g["seed"]))
    hc_ss, hc_bg = sam.gwb(fe, hard=hard, realize=int(g["nreals"]), loudest=int(g["nloud"]), replay=counts,
                           order=ref_order)
    assert np.array_equal(hc_ss == 0.0, g["hc_ss"] == 0.0)
    assert rel_err(hc_ss, g["hc_ss"]) < RTOL_HC
    assert rel_err(hc_bg, g["hc_bg"]) < RTOL_HC


def test_cfg2_default_grid(built_lib):
    """91x81x101 grid, 40 frequencies: norm, density, the grids (strided slices), per-frequency sums,
    the order wherever its key has no ties, and 2 seeded realizations replayed in the reference's
    order."""
    g = load_golden("ref_cfg2.npz")
    sam, hard = _model(g)
    fe = g["fobs_gw_edges"]
    assert rel_err(hard._norm, g["norm"]) < RTOL_GRID
    dens = sam._density_device()[0][::5, ::5, ::5].cpu().numpy()
    assert np.array_equal(dens == 0.0, g["density_slice"] == 0.0)
    assert rel_err(dens, g["density_slice"]) < RTOL_GRID
    redz_final, dnum, number, h2fdf = _grids(sam, hard, fe)
    _check_slices(g, redz_final, dnum, number, h2fdf, step=9)
    d_sum, n_sum, hc2_sum = _sums(dnum, number, h2fdf)
    assert rel_err(d_sum, g["dnum_sum_f"]) < RTOL_GRID
    assert rel_err(n_sum, g["number_sum_f"]) < RTOL_GRID
    assert rel_err(hc2_sum, g["mean_hc2_f"]) < RTOL_GRID
    assert rel_err(h2fdf.amax((0, 1, 2)).cpu().numpy(), g["h2fdf_max_f"]) < RTOL_GRID
    del redz_final, dnum
    from holodeck_gb300 import single_sources
    order = single_sources.sort_order_device(h2fdf).cpu().numpy()
    ref_order = g["order"].astype(np.int64)
    key = h2fdf[..., 0].reshape(-1).cpu().numpy()
    ks = key[ref_order]
    assert np.all(np.diff(ks) <= 0.0)
    untied = np.concatenate([[True], np.diff(ks) != 0]) & np.concatenate([np.diff(ks) != 0, [True]])
    assert untied.sum() > 100000
    assert np.array_equal(order[untied], ref_order[untied])
    counts = O.replay_counts(number.cpu().numpy(), ref_order, int(g["nreals"]), int(g["seed"]))
    hc_ss, hc_bg = sam.gwb(fe, hard=hard, realize=int(g["nreals"]), loudest=int(g["nloud"]), replay=counts,
                           order=ref_order)
    assert np.array_equal(hc_ss == 0.0, g["hc_ss"] == 0.0)
    assert rel_err(hc_ss, g["hc_ss"]) < RTOL_HC
    assert rel_err(hc_bg, g["hc_bg"]) < RTOL_HC


def test_cfg5_high_resolution_grid(built_lib):
    """181x161x201 grid, 100 frequencies: norm, the grids (strided slices), the per-frequency and
    per-(redshift, frequency) expected number and mean hc^2."""
    import os
    from conftest import GOLDEN
    if not os.path.exists(os.path.join(GOLDEN, "ref_cfg5.npz")):
        pytest.fail("ref_cfg5.npz is missing (tests/golden/make_golden.py case_cfg5)")
    g = load_golden("ref_cfg5.npz")
    sam, hard = _model(g)
    fe = g["fobs_gw_edges"]
    assert rel_err(hard._norm, g["norm"]) < RTOL_GRID
    redz_final, dnum, number, h2fdf = _grids(sam, hard, fe)
    _check_slices(g, redz_final, dnum, number, h2fdf, step=17)
    assert rel_err(dnum.sum((0, 1, 2)).cpu().numpy(), g["dnum_sum_f"]) < RTOL_GRID
    del redz_final, dnum
    w = number * h2fdf
    assert rel_err(number.sum((0, 1, 2)).cpu().numpy(), g["number_sum_f"]) < RTOL_GRID
    assert rel_err(w.sum((0, 1, 2)).cpu().numpy(), g["mean_hc2_f"]) < RTOL_GRID
    assert rel_err(number.sum((0, 1)).cpu().numpy(), g["number_zf"]) < RTOL_GRID
    assert rel_err(w.sum((0, 1)).cpu().numpy(), g["mean_hc2_zf"]) < RTOL_GRID


RTOL_FP32 = 1e-4     # the production mode's contract on hc and the expectation sums against FP64
RTOL_FP32_GRID = 2e-5


def _significant_rel(a, b, floor=1e-25):
    """Largest relative difference over values above floor * max (the FP32 mode flushes values below
    FLT_MIN, far below anything that reaches the strain)."""
    a, b = np.asarray(a), np.asarray(b)
    m = np.abs(b) > floor * np.abs(b).max()
    return float((np.abs(a[m] - b[m]) / np.abs(b[m])).max())


@pytest.mark.parametrize("name, step", [("ref_cfg1.npz", 7), ("ref_cfg2.npz", 9)])
def test_fp32_production_mode(built_lib, name, step):
    """The FP32 production mode against the reference's FP64 results: grids, the per-frequency
    expected number and mean hc^2, and the strain of the reference's seeded realizations replayed in
    its order, each within the mode's stated tolerance; the redshifts (an FP64 island) stay FP64-exact."""
    g = load_golden(name)
    sam, hard = _model(g)
    fe = g["fobs_gw_edges"]
    fo_c = 0.5 * (fe[1:] + fe[:-1]) / 2.0
    redz_final, dnum = sam._dbn_device(hard, fo_c, precision="fp32")
    number, h2fdf = sam._number_and_strain(fe / 2.0, dnum, redz_final, precision="fp32")
    rf = _strided(redz_final, step)
    assert np.array_equal(rf == -1.0, g["redz_final_slice"] == -1.0)
    assert rel_err(rf, g["redz_final_slice"]) < RTOL_GRID
    assert _significant_rel(_strided(dnum, step), g["dnum_slice"]) < RTOL_FP32_GRID
    if "number_slice" in g:
        assert _significant_rel(_strided(number, step), g["number_slice"]) < RTOL_FP32_GRID
        hh = _strided(h2fdf, step)
        assert np.array_equal(hh == 0.0, g["h2fdf_slice"] == 0.0)
        assert _significant_rel(hh, g["h2fdf_slice"]) < RTOL_FP32_GRID
    d_sum, n_sum, hc2_sum = _sums(dnum, number, h2fdf)
    assert rel_err(d_sum, g["dnum_sum_f"]) < RTOL_FP32_GRID
    assert rel_err(n_sum, g["number_sum_f"]) < RTOL_FP32_GRID
    assert rel_err(hc2_sum, g["mean_hc2_f"]) < RTOL_FP32_GRID
    del redz_final, dnum, number, h2fdf
    # the reference's draws come from FP64 expectations: the oracle's (cfg-1) or the FP64 mode's (cfg-2,
    # 1e-11 from the reference's), never the FP32 ones, whose 1e-7 offsets move large-lambda draws
    if name == "ref_cfg2.npz":
        lam = _grids(sam, hard, fe)[2].cpu().numpy()
    else:
        lam = _oracle_number(g)
    ref_order = g["order"].astype(np.int64)
    counts = O.replay_counts(lam, ref_order, int(g["nreals"]), int(g["seed"]))
    hc_ss, hc_bg = sam.gwb(fe, hard=hard, realize=int(g["nreals"]), loudest=int(g["nloud"]), replay=counts,
                           order=ref_order, precision="fp32")
    assert np.array_equal(hc_ss == 0.0, g["hc_ss"] == 0.0)
    for f in range(hc_bg.shape[0]):       # the contract is stated per frequency
        assert rel_err(hc_ss[f], g["hc_ss"][f]) < RTOL_FP32, f
        assert rel_err(hc_bg[f], g["hc_bg"][f]) < RTOL_FP32, f


def _oracle_number(g):
    """The oracle's expected numbers on a fixture's grid (bit-identical to the reference's where the
    fixture was made), for drawing the reference's Poisson counts."""
    from holodeck_gb300 import constants as C
    mtot, mrat, redz, fe = g["mtot"], g["mrat"], g["redz"], g["fobs_gw_edges"]
    p = O.default_params(scatter_dex=0.28)
    parts = O.static_binary_density(mtot, mrat, redz, p, return_parts=True)
    rf, dn = O.dbn_2pwl(0.25 * (fe[1:] + fe[:-1]), 1.0e3 * C.PC, 300, g["norm"], 100.0 * C.PC, -1.0, 2.5,
                        parts["density"], mtot, mrat, redz, parts["gmt_time"])
    return O.integrate_differential_number_3dx1d([mtot, mrat, redz, fe / 2.0], dn)
