"""The reference's own Cython kernels as built by oracle/ref_build.py (the reference arm of bench.py
and its CPU baseline) reproduce the reference's fixtures bit for bit: the build and the import
stand-in change nothing in the reference's arithmetic."""

import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def ref_modules():
    from oracle import ref_build
    if not ref_build.generated():
        pytest.skip("oracle/_ref/gen holds no generated C (oracle/ref_build.py generate)")
    return ref_build.load()


def test_loudest_hc_from_sorted(ref_modules):
    cyutils, _ = ref_modules
    g = load_golden("ref_loudest_edges.npz")
    ms, qs, zs = np.unravel_index(g["order"], g["number"].shape[:3])
    for ii in range(int(g["ncases"])):
        seed = int(g[f"c{ii}_seed"])
        cyutils.PCG64 = lambda s=seed: np.random.PCG64(s)
        ss, bg = cyutils.loudest_hc_from_sorted(g["number"], g["h2fdf"], int(g[f"c{ii}_nreals"]),
                                                int(g[f"c{ii}_nloud"]), ms, qs, zs)
        assert np.array_equal(ss, g[f"c{ii}_hc2ss"]) and np.array_equal(bg, g[f"c{ii}_hc2bg"])


def test_hardening_norm_dbn_and_integration(ref_modules):
    from oracle import ref_stub
    from oracle import sam_oracle as O
    import holodeck
    _, sam_cyutils = ref_modules
    g = load_golden("ref_norm_sweep.npz")
    for ii in range(int(g["nparams"])):
        nl = sam_cyutils.find_2pwl_hardening_norm(float(g[f"p{ii}_time"]), g["mtot"], g["mrat"],
                                                  float(g[f"p{ii}_sepa_init"]), float(g[f"p{ii}_rchar"]),
                                                  float(g[f"p{ii}_gamma_inner"]), float(g[f"p{ii}_gamma_outer"]),
                                                  int(g[f"p{ii}_nsteps"]))
        assert np.array_equal(np.asarray(nl), g[f"p{ii}_norm_log10"])
    s = load_golden("ref_small_2pwl_noscatter.npz")
    hard = holodeck.hardening.Fixed_Time_2PL_SAM()
    hard._norm, hard._sepa_init, hard._num_steps = s["norm"], float(s["sepa_init"]), int(s["num_steps"])
    hard._rchar, hard._gamma_inner, hard._gamma_outer = (float(s["rchar"]), float(s["gamma_inner"]),
                                                         float(s["gamma_outer"]))
    sam = ref_stub._Sam(s["mtot"], s["mrat"], s["redz"], s["density"], s["gmt_time"])
    rf, dn = sam_cyutils.dynamic_binary_number_at_fobs(s["fobs_orb_cents"], sam, hard, O.default_params()["cosmo"])
    assert np.array_equal(rf, s["redz_final"]) and np.array_equal(dn, s["dnum"])
    number = sam_cyutils.integrate_differential_number_3dx1d([s["mtot"], s["mrat"], s["redz"], s["fobs_orb_edges"]],
                                                            dn)
    assert np.array_equal(number, s["number"])
