"""GPU kernels against the reference fixtures and the CPU oracle (run on a GB300).

Tolerances: the FP64 grid stages differ from the reference only through the last-ulp behaviour
of pow / log10 / exp on the device, so they are held to 1e-9 relative (the target is 1e-6);
integration, sorting and the replayed realizations are bit-exact.
"""

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import sam_oracle as O

pytestmark = pytest.mark.gpu

RTOL_GRID = 1e-9


def _sam(g, scatter):
    import holodeck_gb300 as H
    gsmf = H.sams.GSMF_Schechter(phi0=-2.77, mchar0_log10=11.24, alpha0=-1.24)
    mmb = H.host_relations.MMBulge_KH2013(mamp_log10=8.69, mplaw=1.17, scatter_dex=scatter)
    shape = (g["mtot"].size, g["mrat"].size, g["redz"].size)
    sam = H.sams.Semi_Analytic_Model(gsmf=gsmf, gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=mmb, shape=shape)
    # np.logspace may differ in the last bit between hosts: use the reference's own edges
    sam.mtot, sam.mrat, sam.redz = g["mtot"], g["mrat"], g["redz"]
    return sam


def _hard(sam, g):
    import holodeck_gb300 as H
    return H.hardening.Fixed_Time_2PL_SAM(sam, float(g["hard_time"]), sepa_init=float(g["sepa_init"]),
                                          rchar=float(g["rchar"]), gamma_inner=float(g["gamma_inner"]),
                                          gamma_outer=float(g["gamma_outer"]), num_steps=int(g["num_steps"]))


def test_static_density_noscatter(built_lib):
    g = load_golden("ref_small_2pwl_noscatter.npz")
    sam = _sam(g, 0.0)
    dens = sam.static_binary_density
    assert rel_err(dens, g["density"]) < 1e-12
    assert np.array_equal(dens == 0.0, g["density"] == 0.0)
    assert rel_err(sam._gmt_time, g["gmt_time"]) < 1e-12
    assert np.array_equal(sam._redz_prime < 0, g["redz_prime"] < 0)
    assert rel_err(sam._redz_prime, g["redz_prime"]) < 1e-12


def test_static_density_other_components(built_lib):
    """GMR_Illustris (the default rate) and GSMF_Double_Schechter against the oracle formulas."""
    import holodeck_gb300 as H
    sam = H.sams.Semi_Analytic_Model(shape=(9, 8, 7), mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=0.0))
    dens = sam.static_binary_density
    assert sam._gmt_time is None and sam._redz_prime is None
    p = O.default_params(scatter_dex=0.0)
    mstar_pri, mstar_rat, mstar_tot, rz = O.mass_stellar(sam.mtot, sam.mrat, sam.redz, p)
    gm = H.sams.GMR_Illustris()
    zp1 = 1.0 + rz
    rate = gm._norm0 * zp1 ** gm._normz * (mstar_tot / gm._mref) ** (gm._malpha0 * zp1 ** gm._malphaz) * \
        (1.0 + mstar_tot / gm._mref_delta) ** (gm._mdelta0 * zp1 ** gm._mdeltaz) * \
        mstar_rat ** (gm._qgamma0 * zp1 ** gm._qgammaz + gm._qgammam * np.log10(mstar_tot / gm._mref))
    ref = O.gsmf_schechter(mstar_pri, rz, p) * rate * p["cosmo"].dtdz(rz)
    jac = (sam.mtot[:, None, None] / mstar_tot) * (O.dmstar_dmbh(mstar_pri, p) * (1.0 + mstar_rat) /
                                                    (1.0 + sam.mrat[None, :, None]) /
                                                    (p["mplaw"] * mstar_rat ** (p["mplaw"] - 1.0)))
    assert rel_err(dens, ref * jac) < 1e-11


def test_hardening_norm_sweep(built_lib):
    from holodeck_gb300.sams import sam_cyutils
    g = load_golden("ref_norm_sweep.npz")
    for ii in range(int(g["nparams"])):
        nl = sam_cyutils.find_2pwl_hardening_norm(float(g[f"p{ii}_time"]), g["mtot"], g["mrat"],
                                                  float(g[f"p{ii}_sepa_init"]), float(g[f"p{ii}_rchar"]),
                                                  float(g[f"p{ii}_gamma_inner"]), float(g[f"p{ii}_gamma_outer"]),
                                                  int(g[f"p{ii}_nsteps"]))
        np.testing.assert_allclose(nl, g[f"p{ii}_norm_log10"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("tag", ["noscatter"])
def test_dbn_2pwl(built_lib, tag):
    g = load_golden(f"ref_small_2pwl_{tag}.npz")
    sam = _sam(g, 0.0)
    hard = _hard(sam, g)
    assert rel_err(hard._norm, g["norm"]) < 1e-9
    from holodeck_gb300.sams import sam_cyutils
    rf, dn = sam_cyutils.dynamic_binary_number_at_fobs(g["fobs_orb_cents"], sam, hard)
    assert np.array_equal(rf == -1.0, g["redz_final"] == -1.0)
    assert rel_err(rf, g["redz_final"]) < RTOL_GRID
    assert rel_err(dn, g["dnum"]) < RTOL_GRID


@pytest.mark.parametrize("tag", ["noscatter"])
def test_dbn_gw(built_lib, tag):
    import holodeck_gb300 as H
    from holodeck_gb300.sams import sam_cyutils
    g = load_golden(f"ref_small_gw_{tag}.npz")
    sam = _sam(g, 0.0)
    rf, dn = sam_cyutils.dynamic_binary_number_at_fobs(g["fobs_orb_cents"], sam, H.hardening.Hard_GW())
    assert np.array_equal(rf == -1.0, g["redz_final"] == -1.0)
    assert rel_err(rf, g["redz_final"]) < RTOL_GRID
    assert rel_err(dn, g["dnum"]) < RTOL_GRID


@pytest.mark.parametrize("name", ["ref_small_2pwl_noscatter.npz", "ref_small_gw_scatter.npz"])
def test_integrate_bit_exact_and_strain(built_lib, name):
    from holodeck_gb300.sams import sam_cyutils
    from holodeck_gb300 import gravwaves
    g = load_golden(name)
    edges = [g["mtot"], g["mrat"], g["redz"], g["fobs_orb_edges"]]
    number = sam_cyutils.integrate_differential_number_3dx1d(edges, g["dnum"])
    assert np.array_equal(number, g["number"])
    h2fdf = gravwaves.char_strain_sq_from_bin_edges_redz(edges, g["redz_final"])
    assert rel_err(h2fdf, g["h2fdf"]) < 1e-10
    assert np.array_equal(h2fdf == 0.0, g["h2fdf"] == 0.0)


def test_sort_order(built_lib):
    import torch
    from holodeck_gb300 import single_sources
    g = load_golden("ref_small_2pwl_noscatter.npz")
    h = torch.as_tensor(g["h2fdf"], device="cuda")
    order = single_sources.sort_order_device(h).cpu().numpy()
    key = g["h2fdf"][..., 0].ravel()
    assert np.all(np.diff(key[order]) <= 0.0)
    # identical to numpy's argsort wherever the key has no ties
    uniq = np.unique(key, return_counts=True)
    tied = np.isin(key[g["order"]], uniq[0][uniq[1] > 1])
    assert np.array_equal(order[~tied], g["order"][~tied])


@pytest.mark.parametrize("nb", [1, 2, 255, 2048, 2049, 100003, 1 << 20])
def test_sort_order_edge_values(built_lib, nb):
    """The radix argsort equals numpy's stable argsort of the negated first-frequency keys: ties in
    ascending bin order, -0.0 tied with +0.0, NaNs last; ragged tile ends and a strided frequency axis."""
    import torch
    from holodeck_gb300 import single_sources
    rng = np.random.default_rng(nb)
    nf = 3
    h = rng.lognormal(-40.0, 3.0, size=(nb, nf))
    pick = rng.random(nb)
    h[pick < 0.2, 0] = 0.0
    h[(pick >= 0.2) & (pick < 0.25), 0] = -0.0
    h[(pick >= 0.25) & (pick < 0.3), 0] = 1.5e-30   # a tie run
    h[(pick >= 0.3) & (pick < 0.31), 0] = np.nan
    h[(pick >= 0.31) & (pick < 0.32), 0] = -rng.random(int(((pick >= 0.31) & (pick < 0.32)).sum()))
    h[(pick >= 0.32) & (pick < 0.33), 0] = np.inf
    h[(pick >= 0.33) & (pick < 0.34), 0] = 5e-324
    key = h[:, 0]
    want = np.argsort(-key, kind="stable")
    got = single_sources.sort_order_device(torch.as_tensor(h, device="cuda")).cpu().numpy()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name", ["ref_small_2pwl_noscatter.npz", "ref_small_2pwl_scatter.npz",
                                  "ref_small_gw_noscatter.npz"])
def test_loudest_replay_bit_exact(built_lib, name):
    """Poisson counts replayed from numpy's PCG64 stream give the reference's hc bit for bit."""
    from holodeck_gb300 import single_sources
    import torch
    g = load_golden(name)
    nreals, nloud, seed = int(g["nreals"]), int(g["nloud"]), int(g["seed"])
    counts = O.replay_counts(g["number"], g["order"], nreals, seed)
    num = torch.as_tensor(g["number"], device="cuda")
    h2 = torch.as_tensor(g["h2fdf"], device="cuda")
    ss, bg = single_sources.ss_realize_device(num, h2, nreals, nloud, replay=counts, order=g["order"])
    assert np.array_equal(ss.cpu().numpy(), g["hc_ss"])
    assert np.array_equal(bg.cpu().numpy(), g["hc_bg"])


def test_loudest_replay_edge_cases(built_lib):
    """Zero bins, tied keys, Normal-branch bins (> 1e10), L larger than the sources, L = 1."""
    from holodeck_gb300 import cyutils
    g = load_golden("ref_loudest_edges.npz")
    shape = g["number"].shape
    ms, qs, zs = np.unravel_index(g["order"], shape[:3])
    for ii in range(int(g["ncases"])):
        nreals, nloud, seed = int(g[f"c{ii}_nreals"]), int(g[f"c{ii}_nloud"]), int(g[f"c{ii}_seed"])
        counts = O.replay_counts(g["number"], g["order"], nreals, seed)
        ss, bg = cyutils.loudest_hc_from_sorted(g["number"], g["h2fdf"], nreals, nloud, ms, qs, zs, replay=counts)
        assert np.array_equal(ss, g[f"c{ii}_hc2ss"])
        assert np.array_equal(bg, g[f"c{ii}_hc2bg"])


def test_second_pass_gwb_replay(built_lib):
    from holodeck_gb300 import cyutils
    g = load_golden("ref_loudest_edges.npz")
    nreals, seed = int(g["gwb_nreals"]), int(g["gwb_seed"])
    rng = np.random.Generator(np.random.PCG64(seed))
    lam = g["number"].reshape(-1, g["number"].shape[-1])
    rep = np.zeros(lam.shape + (nreals,))
    for bb in range(lam.shape[0]):
        for ff in range(lam.shape[1]):
            if lam[bb, ff] > 1e10:
                rep[bb, ff] = rng.normal(lam[bb, ff], np.sqrt(lam[bb, ff]), size=nreals)
            else:
                rep[bb, ff] = rng.poisson(lam[bb, ff], size=nreals)
    gw = cyutils.sam_poisson_gwb(g["number"], g["h2fdf"], nreals, replay=rep)
    assert np.array_equal(gw, g["gwb_hc2"])


def test_ss_gws_redz_invalid_redshift_raises(built_lib):
    from holodeck_gb300 import single_sources
    g = load_golden("ref_small_gw_noscatter.npz")
    edges = [g["mtot"], g["mrat"], g["redz"], g["fobs_orb_edges"]]
    bad = g["redz_final"].copy()
    bad[1, 1, 1, 0] = -0.5
    with pytest.raises(ValueError):
        single_sources.ss_gws_redz(edges, bad, g["number"], 3, 2)
    with pytest.raises(Exception):
        single_sources.ss_gws_redz(edges, g["redz_final"], g["number"], 3.5, 2)


def test_gwb_end_to_end_noscatter_vs_oracle(built_lib):
    """Full gwb(): grids within 1e-9 of the oracle, and hc of a replayed stream equal to the oracle's."""
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    shape = (16, 15, 14)
    p = O.default_params(scatter_dex=0.0)
    mtot, mrat, redz = O.grid_edges(shape)
    _, fe = O.pta_freqs(16.0 * C.YR, 6)
    sam = H.sams.Semi_Analytic_Model(gsmf=H.sams.GSMF_Schechter(), gpf=H.sams.GPF_Power_Law(),
                                     gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=0.0), shape=shape)
    sam.mtot, sam.mrat, sam.redz = mtot, mrat, redz
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5)
    hd = dict(time=3.0 * C.GYR, sepa_init=1.0e3 * C.PC, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5,
              num_steps=300)
    # grids
    parts = O.static_binary_density(mtot, mrat, redz, p, return_parts=True)
    assert rel_err(sam.static_binary_density, parts["density"]) < 1e-12
    fo_c = O.midpoints(fe) / 2.0
    mt, mr = np.meshgrid(mtot, mrat, indexing="ij")
    norm = 10.0 ** O.find_2pwl_hardening_norm(hd["time"], mt.ravel(), mr.ravel(), hd["sepa_init"], hd["rchar"],
                                              hd["gamma_inner"], hd["gamma_outer"], 300).reshape(mt.shape)
    rf_o, dn_o = O.dbn_2pwl(fo_c, hd["sepa_init"], 300, norm, hd["rchar"], -1.0, 2.5, parts["density"], mtot, mrat,
                            redz, parts["gmt_time"])
    edges = [mtot, mrat, redz, fe / 2.0]
    num_o = O.integrate_differential_number_3dx1d(edges, dn_o)
    h2_o = O.char_strain_sq_from_bin_edges_redz(edges, rf_o)
    redz_final, diff_num = sam._dbn_device(hard, fo_c)
    number, h2fdf = sam._number_and_strain(fe / 2.0, diff_num, redz_final)
    assert rel_err(number.cpu().numpy(), num_o) < 1e-9
    assert rel_err(h2fdf.cpu().numpy(), h2_o) < 1e-9
    mean_hc2_gpu = (number * h2fdf).sum(dim=(0, 1, 2)).cpu().numpy()
    mean_hc2_orc = (num_o * h2_o).sum(axis=(0, 1, 2))
    assert rel_err(mean_hc2_gpu, mean_hc2_orc) < 1e-9
    # realizations: replay the oracle's draws in the oracle's order
    order = O.sort_order(h2_o)
    counts = O.replay_counts(num_o, order, 4, 123)
    ss, bg = sam.gwb(fe, hard=hard, realize=4, loudest=3, replay=counts, order=order)
    ss_o, bg_o = O.ss_gws_redz(edges, rf_o, num_o, 4, 3, counts=counts)
    assert rel_err(bg, bg_o) < 1e-9
    assert rel_err(ss, ss_o) < 1e-9


def test_philox_poisson_statistics(built_lib):
    """Counts of the Philox sampler follow Poisson(lambda) across all sampler regimes."""
    from holodeck_gb300 import cyutils
    from scipy import stats
    # sampler boundaries: sparse 0.1, alias 10, inversion tables up to 47000 (one warp builds a table of
    # up to 2048 entries, lambda about 21200, the whole block above), PTRS32 above, PTRS64 beyond 2^22
    lams = np.array([1e-7, 0.03, 0.099, 0.1, 0.12, 0.16, 0.7, 3.0, 9.99, 10.0, 37.5, 412.0, 1500.0, 2000.0, 2100.0,
                     3000.0, 1.15e4, 1.16e4, 2.1e4, 2.2e4, 4.69e4, 4.71e4, 6.0e4, 9.1e4, 5.0e6])
    nreals = 20000
    # one bin per lambda, one frequency; L=0 so every source goes to the background sum
    number = lams.reshape(-1, 1, 1, 1)
    h2fdf = np.ones_like(number)
    ms, qs, zs = np.unravel_index(np.arange(lams.size), number.shape[:3])
    rows = []
    for jj, lam in enumerate(lams):
        num = np.zeros_like(number)
        num[jj] = lam
        _, bg = cyutils.loudest_hc_from_sorted(num, h2fdf, nreals, 0, ms, qs, zs, seed=99 + jj)
        cnt = bg[0]
        assert np.all(cnt == np.round(cnt)) and np.all(cnt >= 0)
        mean, var = cnt.mean(), cnt.var()
        se = np.sqrt(lam / nreals)
        assert abs(mean - lam) < 5 * se + 1e-12, (lam, mean)
        if lam > 0.01:
            assert abs(var / lam - 1.0) < 5 * np.sqrt(2.0 / nreals) * max(1.0, 1.0 / np.sqrt(lam)) + 0.02, (lam, var)
        if 0.02 < lam <= 0.5:   # geometric skipping and the small tables near their boundary
            obs = np.array([(cnt == 0).sum(), (cnt == 1).sum(), (cnt >= 2).sum()])
            exp = np.array([stats.poisson.pmf(0, lam), stats.poisson.pmf(1, lam), stats.poisson.sf(1, lam)]) * nreals
            chi2 = ((obs - exp) ** 2 / exp).sum()
            assert stats.chi2.sf(chi2, 2) > 1e-4, (lam, obs, exp)
        if 0.5 < lam < 1e5:
            lo, hi = int(stats.poisson.ppf(1e-4, lam)), int(stats.poisson.ppf(1 - 1e-4, lam))
            ks = np.arange(lo, hi + 1)
            obs = np.array([(cnt == k).sum() for k in ks])
            exp = stats.poisson.pmf(ks, lam) * nreals
            keep = exp > 5
            chi2 = ((obs[keep] - exp[keep]) ** 2 / exp[keep]).sum()
            assert stats.chi2.sf(chi2, keep.sum() - 1) > 1e-4, (lam, chi2)
        rows.append((lam, mean, var))


def test_philox_deterministic_and_seeded(built_lib):
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    sam = H.sams.Semi_Analytic_Model(shape=(12, 11, 10), gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=0.0))
    _, fe = H.utils.pta_freqs(16.0 * C.YR, 5)
    a = sam.gwb(fe, realize=300, loudest=4, seed=7)
    b = sam.gwb(fe, realize=300, loudest=4, seed=7)
    c = sam.gwb(fe, realize=300, loudest=4, seed=8)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[1], c[1])
    assert a[0].shape == (5, 300, 4) and a[1].shape == (5, 300)
    # loudest slots are non-increasing in the sort order of the first frequency
    assert np.all(np.diff(a[0][0], axis=-1) <= 0)


def test_philox_matches_oracle_statistics(built_lib):
    """hc_bg of Philox realizations vs numpy-Poisson realizations of the oracle: mean, variance, percentiles."""
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    shape = (14, 13, 12)
    nreals = 4000
    sam = H.sams.Semi_Analytic_Model(shape=shape, gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=0.0))
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5)
    _, fe = H.utils.pta_freqs(16.0 * C.YR, 4)
    ss, bg = sam.gwb(fe, hard=hard, realize=nreals, loudest=2, seed=2024)
    fo_c = H.utils.midpoints(fe) / 2.0
    redz_final, diff_num = sam._dbn_device(hard, fo_c)
    number, h2fdf = sam._number_and_strain(fe / 2.0, diff_num, redz_final)
    edges = [sam.mtot, sam.mrat, sam.redz, fe / 2.0]
    ss_o, bg_o = O.ss_gws_redz(edges, redz_final.cpu().numpy(), number.cpu().numpy(), nreals, 2, seed=5)
    hc2, hc2_o = bg ** 2, bg_o ** 2
    for ff in range(hc2.shape[0]):
        a, b = hc2[ff], hc2_o[ff]
        se = np.sqrt(a.var() / nreals + b.var() / nreals)
        assert abs(a.mean() - b.mean()) < 5 * se
        for q in (5, 50, 95):
            pa, pb = np.percentile(np.sqrt(a), q), np.percentile(np.sqrt(b), q)
            assert abs(pa / pb - 1.0) < 0.03, (ff, q, pa, pb)
        assert abs(a.var() / b.var() - 1.0) < 0.25


def test_philox_loudest_slots_distribution(built_lib):
    """Which bins fill the loudest slots, and the background left over, follow the reference's
    in-order walk: Philox realizations vs numpy-Poisson realizations of the oracle, two-sample
    chi-square over the slot tuples and moments of the background."""
    from holodeck_gb300 import cyutils
    from scipy import stats
    # sorted by h at the first frequency: bin k is the k-th loudest; lambdas cover every sampler
    lams = np.array([0.2, 1e-3, 1.5, 0.01, 3.0, 0.6, 25.0, 7.0, 400.0])
    hs = np.linspace(9.0, 1.0, lams.size) * 1e-30
    number = lams.reshape(-1, 1, 1, 1)
    h2fdf = hs.reshape(-1, 1, 1, 1)
    ms, qs, zs = np.unravel_index(np.arange(lams.size), number.shape[:3])
    nreals, nloud = 100_000, 3
    ss, bg = cyutils.loudest_hc_from_sorted(number, h2fdf, nreals, nloud, ms, qs, zs, seed=31337)
    ss_o, bg_o = O.loudest_hc_from_sorted(number, h2fdf, nreals, nloud, np.arange(lams.size), seed=4242)

    def tuples(s):
        idx = np.rint(s[0] / 1e-30).astype(np.int64)   # slot value -> 9..1, 0 when empty
        return idx[:, 0] * 100 + idx[:, 1] * 10 + idx[:, 2]

    ta, tb = tuples(ss), tuples(ss_o)
    cats = np.union1d(ta, tb)
    ca = np.array([(ta == c).sum() for c in cats])
    cb = np.array([(tb == c).sum() for c in cats])
    keep = (ca + cb) >= 20
    chi2, p, _, _ = stats.chi2_contingency(np.stack([ca[keep], cb[keep]]))
    assert p > 1e-4, (chi2, p, cats[keep], ca[keep], cb[keep])
    # background: mean and variance against the oracle; total mean against sum(lambda h)
    a, b = bg[0], bg_o[0]
    se = np.sqrt(a.var() / nreals + b.var() / nreals)
    assert abs(a.mean() - b.mean()) < 5 * se
    assert abs(a.var() / b.var() - 1.0) < 0.05
    tot = a + ss[0].sum(axis=-1)
    assert abs(tot.mean() / (lams * hs).sum() - 1.0) < 5 * tot.std() / np.sqrt(nreals) / (lams * hs).sum()
