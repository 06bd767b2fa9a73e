"""The CPU oracle against the golden fixtures the holodeck reference produced (bit-exact)."""

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import sam_oracle as O


@pytest.mark.parametrize("tag", ["noscatter", "scatter"])
def test_density_and_merger(tag):
    g = load_golden(f"ref_small_2pwl_{tag}.npz")
    p = O.default_params(scatter_dex=0.0 if tag == "noscatter" else 0.28)
    parts = O.static_binary_density(g["mtot"], g["mrat"], g["redz"], p, return_parts=True)
    assert np.array_equal(parts["density"], g["density"])
    assert np.array_equal(parts["gmt_time"], g["gmt_time"])
    assert np.array_equal(parts["redz_prime"], g["redz_prime"])


def test_scatter_shapes():
    g = load_golden("ref_scatter.npz")
    for ii, scat in enumerate([0.28, 0.6]):
        p = O.default_params(scatter_dex=scat)
        parts = O.static_binary_density(g[f"s{ii}_mtot"], g[f"s{ii}_mrat"], g[f"s{ii}_redz"], p, return_parts=True)
        assert np.array_equal(parts["density"], g[f"s{ii}_density"])
        assert np.array_equal(parts["density_noscatter"], g[f"s{ii}_density_noscatter"])


def test_hardening_norm_sweep():
    g = load_golden("ref_norm_sweep.npz")
    for ii in range(int(g["nparams"])):
        nl = O.find_2pwl_hardening_norm(float(g[f"p{ii}_time"]), g["mtot"], g["mrat"], float(g[f"p{ii}_sepa_init"]),
                                        float(g[f"p{ii}_rchar"]), float(g[f"p{ii}_gamma_inner"]),
                                        float(g[f"p{ii}_gamma_outer"]), int(g[f"p{ii}_nsteps"]))
        assert np.array_equal(nl, g[f"p{ii}_norm_log10"])


@pytest.mark.parametrize("tag", ["noscatter", "scatter"])
def test_dbn_integrate_strain_realize_2pwl(tag):
    g = load_golden(f"ref_small_2pwl_{tag}.npz")
    rf, dn = O.dbn_2pwl(g["fobs_orb_cents"], float(g["sepa_init"]), int(g["num_steps"]), g["norm"], float(g["rchar"]),
                        float(g["gamma_inner"]), float(g["gamma_outer"]), g["density"], g["mtot"], g["mrat"],
                        g["redz"], g["gmt_time"])
    assert np.array_equal(rf, g["redz_final"])
    assert np.array_equal(dn, g["dnum"])
    edges = [g["mtot"], g["mrat"], g["redz"], g["fobs_orb_edges"]]
    assert np.array_equal(O.integrate_differential_number_3dx1d(edges, g["dnum"]), g["number"])
    h = O.char_strain_sq_from_bin_edges_redz(edges, g["redz_final"])
    assert np.array_equal(h, g["h2fdf"])
    assert np.array_equal(O.sort_order(h), g["order"])
    ss, bg = O.ss_gws_redz(edges, g["redz_final"], g["number"], int(g["nreals"]), int(g["nloud"]), seed=int(g["seed"]))
    assert np.array_equal(ss, g["hc_ss"]) and np.array_equal(bg, g["hc_bg"])


@pytest.mark.parametrize("tag", ["noscatter", "scatter"])
def test_dbn_gw_and_realize(tag):
    g = load_golden(f"ref_small_gw_{tag}.npz")
    rf, dn = O.dbn_gw(g["fobs_orb_cents"], g["density"], g["mtot"], g["mrat"], g["redz_prime"])
    assert np.array_equal(rf, g["redz_final"])
    assert np.array_equal(dn, g["dnum"])
    edges = [g["mtot"], g["mrat"], g["redz"], g["fobs_orb_edges"]]
    ss, bg = O.ss_gws_redz(edges, g["redz_final"], g["number"], int(g["nreals"]), int(g["nloud"]), seed=int(g["seed"]))
    assert np.array_equal(ss, g["hc_ss"]) and np.array_equal(bg, g["hc_bg"])


def test_loudest_edge_cases_and_second_pass():
    g = load_golden("ref_loudest_edges.npz")
    for ii in range(int(g["ncases"])):
        ss, bg = O.loudest_hc_from_sorted(g["number"], g["h2fdf"], int(g[f"c{ii}_nreals"]), int(g[f"c{ii}_nloud"]),
                                          g["order"], seed=int(g[f"c{ii}_seed"]))
        assert np.array_equal(ss, g[f"c{ii}_hc2ss"]) and np.array_equal(bg, g[f"c{ii}_hc2bg"])
    gw = O.sam_poisson_gwb(g["number"], g["h2fdf"], int(g["gwb_nreals"]), int(g["gwb_seed"]))
    assert np.array_equal(gw, g["gwb_hc2"])


def test_cfg1_end_to_end():
    """The reference's CPU workload (shape 30, F=20, R=100, L=5, scatter 0.28, seed 0), end to end."""
    g = load_golden("ref_cfg1.npz")
    p = O.default_params(scatter_dex=0.28)
    from holodeck_gb300 import constants as C
    hard = dict(time=3.0 * C.GYR, sepa_init=1.0e3 * C.PC, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5,
                num_steps=300)
    ss, bg = O.gwb(g["fobs_gw_edges"], g["mtot"], g["mrat"], g["redz"], p, hard, int(g["nreals"]), int(g["nloud"]),
                   seed=int(g["seed"]))
    assert np.array_equal(ss, g["hc_ss"]) and np.array_equal(bg, g["hc_bg"])


def test_known_answer_strain():
    """The reference's own known-answer values for the strain formula (holodeck/tests/test_utils.py:52-96)."""
    g = load_golden("ref_known_answers.npz")
    from holodeck_gb300 import utils
    mc = utils.chirp_mass(g["m1"], g["m2"])
    assert rel_err(mc, g["mc"]) < 1e-8
    hs = utils.gw_strain_source(g["mc"], g["dc"], g["freq"])
    assert rel_err(hs, g["hs"]) < 1e-8
    assert np.allclose(hs, g["check_hs"], rtol=1e-14, atol=0)


def test_oracle_params_path_bit_exact():
    """ss_gws_redz(params=True): loudest-source parameters and background-weighted means
    (single_sources.py:102-161, cyutils.pyx:1541-1770), replaying the reference's PCG64 stream."""
    g = load_golden("ref_params.npz")
    edges = [g["mtot"], g["mrat"], g["redz"], g["fobs_orb_edges"]]
    h2 = O.char_strain_sq_from_bin_edges_redz(edges, g["redz_final"])
    order = O.sort_order(h2)
    for ii in range(int(g["ncases"])):
        nreals, nloud, seed = int(g[f"c{ii}_nreals"]), int(g[f"c{ii}_nloud"]), int(g[f"c{ii}_seed"])
        counts = O.replay_counts(g["number"], order, nreals, seed)
        assert np.array_equal(counts, g[f"c{ii}_counts"])
        out = O.ss_gws_redz_params(edges, g["redz_final"], g["number"], nreals, nloud, counts=counts)
        for got, name in zip(out, ["hc_ss", "hc_bg", "sspar", "bgpar"]):
            assert np.array_equal(got, g[f"c{ii}_{name}"], equal_nan=True), (ii, name)


def test_oracle_model_details_bit_exact():
    """_calc_model_details (librarian/lib_tools.py:845-943) on the reference's run_model output."""
    g = load_golden("ref_details.npz")
    fe = g["fobs_edges"] / 2.0
    edges = [g["mtot"], g["mrat"], g["redz"], fe]
    gwb_pars, num_pars, gm, nm = O.calc_model_details(edges, g["redz_final"], g["number"])
    for ii in range(4):
        assert np.array_equal(gwb_pars[ii], g[f"gwb_params_{ii}"]), ii
        assert np.array_equal(num_pars[ii], g[f"num_params_{ii}"]), ii
    assert np.array_equal(gm, g["gwb_mtot_redz_final"])
    assert np.array_equal(nm, g["num_mtot_redz_final"])
