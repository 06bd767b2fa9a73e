"""The params=True path on the GPU (single_sources.py:102-161, cyutils.pyx:1541-1770): loudest-source
parameters sspar (4, F, R, L) and background-weighted mean parameters bgpar (7, F, R).

Replay mode is bit-exact against the oracle (itself bit-exact against the reference fixture) when both
get the same strain, parameter grids and draws; the GPU parameter grids agree with the oracle's to
1e-12; Philox realizations match numpy-Poisson realizations of the oracle statistically.
"""

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import sam_oracle as O

pytestmark = pytest.mark.gpu


def _inputs(g):
    edges = [g["mtot"], g["mrat"], g["redz"], g["fobs_orb_edges"]]
    h2 = O.char_strain_sq_from_bin_edges_redz(edges, g["redz_final"])
    return edges, h2, O.sort_order(h2)


def test_param_grids_match_oracle(built_lib):
    import torch
    from holodeck_gb300 import single_sources
    g = load_golden("ref_params.npz")
    edges, h2, _ = _inputs(g)
    rz = torch.as_tensor(g["redz_final"], device="cuda")
    grids, scales = single_sources.param_grids_device(edges, rz, h2fdf=torch.as_tensor(h2, device="cuda"))
    ref = O.param_grids(edges, g["redz_final"])
    for got, exp, name in zip(grids, ref, ["redz_mid", "dcom", "sepa", "angs"]):
        got = got.cpu().numpy()
        assert np.array_equal(np.isfinite(got), np.isfinite(exp)), name
        assert np.array_equal(np.isnan(got), np.isnan(exp)), name
        fin = np.isfinite(exp)
        assert rel_err(got[fin], exp[fin]) < 1e-12, name
        e = int(scales[["redz_mid", "dcom", "sepa", "angs"].index(name)].item())
        sel = fin & (h2 != 0) & (exp != 0)
        assert e == int(np.frexp(np.abs(exp[sel]).max())[1]), name


def test_params_replay_bit_exact(built_lib):
    """Replayed PCG64 draws give the oracle's hc_ss, hc_bg, sspar and bgpar bit for bit (the oracle
    equals the reference bit for bit on its fixture; both sides here use this machine's strain,
    order and draws, which may differ in the last bits from the machine that made the fixture)."""
    from holodeck_gb300 import cyutils
    g = load_golden("ref_params.npz")
    edges, h2, order = _inputs(g)
    rz_m, dcom, sepa, angs = O.param_grids(edges, g["redz_final"])
    mt, mr, rz = (O.midpoints(e) for e in edges[:3])
    pars = [mt[:, None, None, None], mr[None, :, None, None], rz[None, None, :, None], rz_m, dcom, sepa, angs]
    ms, qs, zs = np.unravel_index(order, g["number"].shape[:3])
    for ii in range(int(g["ncases"])):
        nreals, nloud, seed = int(g[f"c{ii}_nreals"]), int(g[f"c{ii}_nloud"]), int(g[f"c{ii}_seed"])
        counts = O.replay_counts(g["number"], order, nreals, seed)
        exp = O.loudest_hc_and_par_from_sorted(g["number"], h2, nreals, nloud, order, pars, counts=counts)
        got = cyutils.loudest_hc_and_par_from_sorted_redz(
            g["number"], h2, nreals, nloud, mt, mr, rz, rz_m, dcom, sepa, angs, ms, qs, zs, replay=counts)
        for a, b, name in zip(got, exp, ["hc2ss", "hc2bg", "sspar", "bgpar"]):
            assert np.array_equal(a, b, equal_nan=True), (ii, name)


def test_ss_gws_redz_params_end_to_end(built_lib):
    """ss_gws_redz(params=True) through the GPU strain and grids against the oracle, same draws."""
    from holodeck_gb300 import single_sources
    g = load_golden("ref_params.npz")
    edges, h2, order = _inputs(g)
    nreals, nloud, seed = int(g["c0_nreals"]), int(g["c0_nloud"]), int(g["c0_seed"])
    counts = O.replay_counts(g["number"], order, nreals, seed)
    got = single_sources.ss_gws_redz(edges, g["redz_final"], g["number"], nreals, nloud, params=True,
                                     replay=counts, order=order)
    exp = O.ss_gws_redz_params(edges, g["redz_final"], g["number"], nreals, nloud, counts=counts)
    for a, b, name in zip(got, exp, ["hc_ss", "hc_bg", "sspar", "bgpar"]):
        assert rel_err(a, b) < 1e-9, name


def test_params_philox_statistics(built_lib):
    """Philox realizations of sspar / bgpar against numpy-Poisson realizations of the oracle."""
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    shape = (12, 11, 10)
    nreals, nloud = 3000, 2
    sam = H.sams.Semi_Analytic_Model(shape=shape, gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=0.0))
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5)
    _, fe = H.utils.pta_freqs(16.0 * C.YR, 3)
    hc_ss, hc_bg, sspar, bgpar = sam.gwb(fe, hard=hard, realize=nreals, loudest=nloud, params=True, seed=77)
    assert hc_ss.shape == (3, nreals, nloud) and sspar.shape == (4, 3, nreals, nloud) and bgpar.shape == (7, 3, nreals)
    fo_c = H.utils.midpoints(fe) / 2.0
    redz_final, diff_num = sam._dbn_device(hard, fo_c)
    number, _ = sam._number_and_strain(fe / 2.0, diff_num, redz_final)
    edges = [sam.mtot, sam.mrat, sam.redz, fe / 2.0]
    o_ss, o_bg, o_sspar, o_bgpar = O.ss_gws_redz_params(edges, redz_final.cpu().numpy(), number.cpu().numpy(),
                                                        nreals, nloud, seed=9)
    for ff in range(3):
        a, b = hc_bg[ff] ** 2, o_bg[ff] ** 2
        assert abs(a.mean() / b.mean() - 1.0) < 5 * np.sqrt(a.var() / nreals + b.var() / nreals) / b.mean()
        for kk in range(7):
            x, y = bgpar[kk, ff], o_bgpar[kk, ff]
            se = np.sqrt(x.var() / nreals + y.var() / nreals)
            assert abs(x.mean() - y.mean()) < 5 * se + 1e-12 * abs(y.mean()), (ff, kk, x.mean(), y.mean())
        for kk in range(4):
            x, y = sspar[kk, ff, :, 0], o_sspar[kk, ff, :, 0]
            se = np.sqrt(x.var() / nreals + y.var() / nreals)
            assert abs(x.mean() - y.mean()) < 5 * se + 1e-12 * abs(y.mean()), (ff, kk, x.mean(), y.mean())
