"""Generate the golden fixtures in this directory from the holodeck reference.

Run in a container that holds the reference sources (see ``ref_env.py``)::

    HOLODECK_REF_SRC=<holodeck checkout> HOLODECK_REF_BUILD=<scratch dir> \
        python tests/golden/make_golden.py [case_name]

``case_cfg2`` (the default 91x81x101 grid) takes about two minutes of one core and ``case_cfg5`` (the
181x161x201 grid, 100 frequencies) about half an hour and 30 GB of memory; both are summaries, so
their fixtures stay small.

Every fixture is produced by the unmodified reference code path (plus the
one-token Cython-3 fix and import stand-ins described in ``ref_env.py``),
with ``holodeck.cyutils.PCG64`` replaced by a seeded ``np.random.PCG64`` so
that realizations are reproducible.  The tests never import the reference:
they read these ``.npz`` files.
"""

import ast
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
warnings.filterwarnings("ignore")

import ref_env  # noqa: E402

holo = ref_env.import_reference()
holo.log.setLevel(40)
from holodeck.constants import PC, YR, GYR  # noqa: E402
import holodeck.cyutils as cyutils  # noqa: E402
import holodeck.sams.sam_cyutils as sam_cyutils  # noqa: E402
from holodeck import single_sources, gravwaves  # noqa: E402


def seed_rng(seed):
    cyutils.PCG64 = lambda: np.random.PCG64(seed)


def make_sam(shape, scatter_dex, phi0=-2.77, mchar0_log10=11.24, alpha0=-1.24, mamp_log10=8.69, mplaw=1.17):
    gsmf = holo.sams.GSMF_Schechter(phi0=phi0, mchar0_log10=mchar0_log10, alpha0=alpha0)
    gpf = holo.sams.GPF_Power_Law()
    gmt = holo.sams.GMT_Power_Law()
    mmb = holo.host_relations.MMBulge_KH2013(mamp_log10=mamp_log10, mplaw=mplaw, scatter_dex=scatter_dex)
    return holo.sams.Semi_Analytic_Model(gsmf=gsmf, gpf=gpf, gmt=gmt, mmbulge=mmb, shape=shape)


def run_path(sam, hard, fobs_gw_edges, nreals, nloud, seed):
    """The body of ``Semi_Analytic_Model.gwb`` (sam.py:918-947), keeping intermediates."""
    fobs_gw_cents = 0.5 * (fobs_gw_edges[1:] + fobs_gw_edges[:-1])
    fobs_orb_edges = fobs_gw_edges / 2.0
    fobs_orb_cents = fobs_gw_cents / 2.0
    redz_final, dnum = sam_cyutils.dynamic_binary_number_at_fobs(fobs_orb_cents, sam, hard, holo.cosmo)
    edges = [sam.mtot, sam.mrat, sam.redz, fobs_orb_edges]
    number = sam_cyutils.integrate_differential_number_3dx1d(edges, dnum)
    h2fdf = gravwaves.char_strain_sq_from_bin_edges_redz(edges, redz_final)
    order = np.argsort(-h2fdf[..., 0].flatten())
    seed_rng(seed)
    hc_ss, hc_bg = single_sources.ss_gws_redz(edges, redz_final, number, realize=nreals, loudest=nloud)
    # the full gwb() call must give the same answer with the same seed
    seed_rng(seed)
    hc_ss2, hc_bg2 = sam.gwb(fobs_gw_edges, hard=hard, realize=nreals, loudest=nloud)
    assert np.array_equal(hc_ss, hc_ss2) and np.array_equal(hc_bg, hc_bg2)
    return dict(
        fobs_gw_edges=fobs_gw_edges, fobs_orb_edges=fobs_orb_edges, fobs_orb_cents=fobs_orb_cents,
        redz_final=redz_final, dnum=dnum, number=number, h2fdf=h2fdf, order=order,
        hc_ss=hc_ss, hc_bg=hc_bg,
    )


def sam_arrays(sam):
    dens = sam.static_binary_density
    out = dict(mtot=sam.mtot, mrat=sam.mrat, redz=sam.redz, density=dens,
               gmt_time=sam._gmt_time, redz_prime=sam._redz_prime)
    if getattr(sam, "_dens_bef", None) is not None:
        out["density_noscatter"] = sam._dens_bef
    return out


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({os.path.getsize(path)/1024:.1f} KiB)")


def case_small(scatter, tag):
    shape = (10, 11, 12)
    sam = make_sam(shape, scatter)
    base = sam_arrays(sam)
    fobs_gw_cents, fobs_gw_edges = holo.utils.pta_freqs(16.0 * YR, 5)
    hard = holo.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * GYR, rchar=100.0 * PC, gamma_inner=-1.0, gamma_outer=2.5)
    res = run_path(sam, hard, fobs_gw_edges, nreals=7, nloud=3, seed=0)
    save(f"ref_small_2pwl_{tag}.npz", **base, **res, norm=hard._norm, hard_time=3.0 * GYR,
         sepa_init=hard._sepa_init, rchar=hard._rchar, gamma_inner=hard._gamma_inner,
         gamma_outer=hard._gamma_outer, num_steps=hard._num_steps, nreals=7, nloud=3, seed=0)
    res = run_path(sam, holo.hardening.Hard_GW(), fobs_gw_edges, nreals=7, nloud=3, seed=1)
    save(f"ref_small_gw_{tag}.npz", **base, **res, nreals=7, nloud=3, seed=1)


def case_cfg1():
    """The reference's CPU-runnable workload: shape 30, 20 frequencies, 100 realizations, 5 loudest."""
    sam = make_sam(30, 0.28)
    base = sam_arrays(sam)
    fobs_gw_cents, fobs_gw_edges = holo.utils.pta_freqs(16.0 * YR, 20)
    hard = holo.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * GYR, rchar=100.0 * PC, gamma_inner=-1.0, gamma_outer=2.5)
    res = run_path(sam, hard, fobs_gw_edges, nreals=100, nloud=5, seed=0)
    number, h2fdf = res["number"], res["h2fdf"]
    keep = dict(
        fobs_gw_edges=res["fobs_gw_edges"], hc_ss=res["hc_ss"], hc_bg=res["hc_bg"],
        # size-independent summaries of the large grids
        number_sum_f=number.sum(axis=(0, 1, 2)), mean_hc2_f=(number * h2fdf).sum(axis=(0, 1, 2)),
        dnum_sum_f=res["dnum"].sum(axis=(0, 1, 2)), redz_final_slice=res["redz_final"][::7, ::7, ::7, :],
        dnum_slice=res["dnum"][::7, ::7, ::7, :], order_head=res["order"][:2000],
        # the whole visiting order: numpy's argsort orders the tied (zero) keys differently on other
        # machines, so a replay of the reference's draws needs the reference's own order
        order=res["order"].astype(np.int32),
    )
    save("ref_cfg1.npz", **base, **keep, norm=hard._norm, nreals=100, nloud=5, seed=0)


def _strided(arr, step):
    return np.ascontiguousarray(arr[::step, ::step, ::step, :])


def case_cfg2():
    """The default-grid workload: 91x81x101 grid, 40 frequencies, 10 loudest, with a seeded run of 2
    realizations.  The (M, Q, Z, F) grids are kept as per-frequency sums and strided slices; the
    loudest-first order is kept whole (int32), because numpy's argsort does not order the bins whose
    first-frequency strain ties (the zeros), and replaying the reference's draws needs its order."""
    sam = make_sam((91, 81, 101), 0.28)
    fobs_gw_cents, fobs_gw_edges = holo.utils.pta_freqs(16.0 * YR, 40)
    hard = holo.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * GYR, rchar=100.0 * PC, gamma_inner=-1.0, gamma_outer=2.5)
    res = run_path(sam, hard, fobs_gw_edges, nreals=2, nloud=10, seed=0)
    number, h2fdf, dnum, redz_final = res["number"], res["h2fdf"], res["dnum"], res["redz_final"]
    dens = sam.static_binary_density
    keep = dict(
        mtot=sam.mtot, mrat=sam.mrat, redz=sam.redz, fobs_gw_edges=fobs_gw_edges, norm=hard._norm,
        hc_ss=res["hc_ss"], hc_bg=res["hc_bg"],
        density_slice=np.ascontiguousarray(dens[::5, ::5, ::5]),
        number_sum_f=number.sum(axis=(0, 1, 2)), mean_hc2_f=(number * h2fdf).sum(axis=(0, 1, 2)),
        dnum_sum_f=dnum.sum(axis=(0, 1, 2)), h2fdf_max_f=h2fdf.max(axis=(0, 1, 2)),
        redz_final_slice=_strided(redz_final, 9), dnum_slice=_strided(dnum, 9),
        number_slice=_strided(number, 9), h2fdf_slice=_strided(h2fdf, 9),
        order=res["order"].astype(np.int32),
    )
    save("ref_cfg2.npz", **keep, nreals=2, nloud=10, seed=0)


def case_cfg5():
    """The high-resolution grid: 181x161x201, 100 frequencies (no realizations: 10^4 of them would take
    the reference days).  Keeps the per-frequency expected number and mean hc^2 = sum_b number h2fdf,
    their sums over redshift bins, and strided slices of the grids.  The integration and the strain
    are element-local, so they run through the reference's functions on slabs of the mtot axis (the
    strain function's whole-grid temporaries would need more than 64 GB); the values are the same."""
    sam = make_sam((181, 161, 201), 0.28)
    fobs_gw_cents, fobs_gw_edges = holo.utils.pta_freqs(16.0 * YR, 100)
    hard = holo.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * GYR, rchar=100.0 * PC, gamma_inner=-1.0, gamma_outer=2.5)
    fobs_orb_edges = fobs_gw_edges / 2.0
    fobs_orb_cents = 0.5 * (fobs_gw_edges[1:] + fobs_gw_edges[:-1]) / 2.0
    redz_final, dnum = sam_cyutils.dynamic_binary_number_at_fobs(fobs_orb_cents, sam, hard, holo.cosmo)
    keep = dict(redz_final_slice=_strided(redz_final, 17), dnum_slice=_strided(dnum, 17),
                dnum_sum_f=dnum.sum(axis=(0, 1, 2)))
    nm, nq, nz, nf = dnum.shape
    number_zf = np.zeros((nz - 1, nf))
    hc2_zf = np.zeros((nz - 1, nf))
    number_slice = np.zeros(((nm - 2) // 17 + 1, (nq - 2) // 17 + 1, (nz - 2) // 17 + 1, nf))
    h2fdf_slice = np.zeros_like(number_slice)
    slab = 17                       # a multiple of the slice stride, so slices align with slabs
    for m0 in range(0, nm - 1, slab):
        m1 = min(m0 + slab, nm - 1)
        edges = [sam.mtot[m0:m1 + 1], sam.mrat, sam.redz, fobs_orb_edges]
        num = sam_cyutils.integrate_differential_number_3dx1d(edges, dnum[m0:m1 + 1])
        h2 = gravwaves.char_strain_sq_from_bin_edges_redz(edges, redz_final[m0:m1 + 1])
        number_zf += num.sum(axis=(0, 1))
        hc2_zf += (num * h2).sum(axis=(0, 1))
        number_slice[m0 // 17] = num[0, ::17, ::17, :]
        h2fdf_slice[m0 // 17] = h2[0, ::17, ::17, :]
    keep.update(mtot=sam.mtot, mrat=sam.mrat, redz=sam.redz, fobs_gw_edges=fobs_gw_edges, norm=hard._norm,
                number_sum_f=number_zf.sum(axis=0), mean_hc2_f=hc2_zf.sum(axis=0), mean_hc2_zf=hc2_zf,
                number_zf=number_zf, number_slice=number_slice, h2fdf_slice=h2fdf_slice)
    save("ref_cfg5.npz", **keep)


def case_scatter_shapes():
    """Density with M-Mbulge scatter on two non-cubic grids (sam.py:1291-1394)."""
    out = {}
    for ii, shape in enumerate([(14, 13, 6), (25, 17, 5)]):
        sam = make_sam(shape, 0.28 if ii == 0 else 0.6)
        arr = sam_arrays(sam)
        for kk, vv in arr.items():
            out[f"s{ii}_{kk}"] = vv
    save("ref_scatter.npz", **out)


def case_norm_sweep():
    """Hardening normalisations over the library parameter box (sam_cyutils.pyx:289-398)."""
    sam = make_sam((12, 9, 3), 0.0)
    mt, mr = [mm.flatten() for mm in np.meshgrid(sam.mtot, sam.mrat, indexing="ij")]
    rows = []
    for time_gyr, gin, gout, rchar_pc, sepa_pc, nsteps in [
        (3.0, -1.0, 2.5, 100.0, 1e3, 300), (0.1, -1.5, 2.5, 100.0, 1e3, 300), (11.0, 0.0, 2.5, 100.0, 1e4, 300),
        (1.0, -0.5, 1.5, 10.0, 1e3, 100), (6.0, -1.2, 2.5, 100.0, 1e4, 300),
    ]:
        nl = sam_cyutils.find_2pwl_hardening_norm(time_gyr * GYR, mt, mr, sepa_pc * PC, rchar_pc * PC, gin, gout, nsteps)
        rows.append(dict(time=time_gyr * GYR, gamma_inner=gin, gamma_outer=gout, rchar=rchar_pc * PC,
                         sepa_init=sepa_pc * PC, nsteps=nsteps, norm_log10=np.asarray(nl)))
    out = dict(mtot=mt, mrat=mr)
    for ii, row in enumerate(rows):
        for kk, vv in row.items():
            out[f"p{ii}_{kk}"] = vv
    save("ref_norm_sweep.npz", **out, nparams=len(rows))


def case_loudest_edges():
    """``loudest_hc_from_sorted`` edge cases: zero bins, ties, huge expectation (Normal branch), L > sources."""
    rng = np.random.default_rng(7)
    shape = (4, 3, 5, 3)
    number = rng.lognormal(-1.0, 2.0, size=shape)
    number[0, 0, :, :] = 0.0
    number[1, 2, 3, :] = 3.0e10       # above the 1e10 Normal threshold
    number[2, 1, 1, 1] = 5.0e9        # large Poisson (PTRS branch)
    h2fdf = rng.lognormal(-60.0, 3.0, size=shape)
    h2fdf[3, :, :, 0] = h2fdf[3, 0, 0, 0]   # ties in the sort key
    h2fdf[0, 1, 2, :] = 0.0
    order = np.argsort(-h2fdf[..., 0].flatten())
    ms, qs, zs = np.unravel_index(order, shape[:3])
    out = dict(number=number, h2fdf=h2fdf, order=order)
    for ii, (nreals, nloud, seed) in enumerate([(5, 4, 3), (3, 40, 4), (1, 1, 5)]):
        seed_rng(seed)
        ss, bg = cyutils.loudest_hc_from_sorted(number, h2fdf, nreals, nloud, ms, qs, zs)
        out.update({f"c{ii}_nreals": nreals, f"c{ii}_nloud": nloud, f"c{ii}_seed": seed,
                    f"c{ii}_hc2ss": ss, f"c{ii}_hc2bg": bg})
    # second-pass GWB (gravwaves.py:518-522 -> cyutils.pyx:854-897)
    seed_rng(11)
    out["gwb_nreals"] = 6
    out["gwb_seed"] = 11
    out["gwb_hc2"] = np.asarray(cyutils.sam_poisson_gwb(number, h2fdf, 6))
    save("ref_loudest_edges.npz", **out, ncases=3)


def case_params():
    """``ss_gws_redz(params=True)`` (single_sources.py:102-161 -> cyutils.pyx:1541-1770): loudest-source
    parameters and background-weighted means, through ``gwb(params=True)`` as well."""
    sam = make_sam((10, 11, 12), 0.0)
    fobs_gw_cents, fobs_gw_edges = holo.utils.pta_freqs(16.0 * YR, 5)
    hard = holo.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * GYR, rchar=100.0 * PC, gamma_inner=-1.0, gamma_outer=2.5)
    fobs_orb_edges = fobs_gw_edges / 2.0
    fobs_orb_cents = 0.5 * (fobs_gw_edges[1:] + fobs_gw_edges[:-1]) / 2.0
    redz_final, dnum = sam_cyutils.dynamic_binary_number_at_fobs(fobs_orb_cents, sam, hard, holo.cosmo)
    edges = [sam.mtot, sam.mrat, sam.redz, fobs_orb_edges]
    number = sam_cyutils.integrate_differential_number_3dx1d(edges, dnum)
    out = dict(mtot=sam.mtot, mrat=sam.mrat, redz=sam.redz, fobs_gw_edges=fobs_gw_edges,
               fobs_orb_edges=fobs_orb_edges, redz_final=redz_final, number=number)
    h2fdf = gravwaves.char_strain_sq_from_bin_edges_redz(edges, redz_final)
    order = np.argsort(-h2fdf[..., 0].flatten())
    lam = number.reshape(-1, number.shape[-1])[order]   # (B, F) in the reference's visiting order
    for ii, (nreals, nloud, seed) in enumerate([(6, 3, 21), (2, 40, 22)]):
        seed_rng(seed)
        hc_ss, hc_bg, sspar, bgpar = single_sources.ss_gws_redz(edges, redz_final, number, realize=nreals,
                                                                loudest=nloud, params=True)
        # the draws the reference made (numpy's PCG64 stream in its visiting order; no Normal bins here),
        # kept so that a replay does not depend on the numpy build of the machine that runs the test
        assert np.all(lam <= 1e10)
        rng = np.random.Generator(np.random.PCG64(seed))
        counts = np.array([[rng.poisson(lam[:, ff]) for ff in range(lam.shape[1])] for _ in range(nreals)],
                          dtype=np.float64)
        out.update({f"c{ii}_nreals": nreals, f"c{ii}_nloud": nloud, f"c{ii}_seed": seed, f"c{ii}_hc_ss": hc_ss,
                    f"c{ii}_hc_bg": hc_bg, f"c{ii}_sspar": sspar, f"c{ii}_bgpar": bgpar, f"c{ii}_counts": counts})
    seed_rng(21)
    g = sam.gwb(fobs_gw_edges, hard=hard, realize=6, loudest=3, params=True)
    assert all(np.array_equal(a, b, equal_nan=True) for a, b in
               zip(g, (out["c0_hc_ss"], out["c0_hc_bg"], out["c0_sspar"], out["c0_bgpar"])))
    save("ref_params.npz", **out, ncases=2, hard_time=3.0 * GYR)


def case_param_space():
    """Latin-hypercube library samples of ``PS_Classic_Phenom_Uniform`` (lib_tools.py:49-154,
    param_spaces_classic.py:12-107) and the grids of two of its models at a small shape, which pin the
    mapping from library parameters to SAM and hardening settings."""
    from holodeck.librarian import param_spaces_classic as psc
    space = psc.PS_Classic_Phenom_Uniform(nsamples=8, sam_shape=(10, 11, 12), seed=0)
    out = dict(param_samples=space.param_samples, uniform_samples=space._uniform_samples,
               param_names=np.array(space.param_names), extrema=space.extrema)
    fobs_gw_cents, fobs_gw_edges = holo.utils.pta_freqs(16.03 * YR, 4)
    fobs_orb_edges = fobs_gw_edges / 2.0
    for ii in (0, 5):
        sam, hard = space.model_for_sample_number(ii)
        redz_final, dnum = sam_cyutils.dynamic_binary_number_at_fobs(fobs_gw_cents / 2.0, sam, hard, holo.cosmo)
        number = sam_cyutils.integrate_differential_number_3dx1d([sam.mtot, sam.mrat, sam.redz, fobs_orb_edges], dnum)
        out.update({f"s{ii}_mtot": sam.mtot, f"s{ii}_mrat": sam.mrat, f"s{ii}_redz": sam.redz,
                    f"s{ii}_density": sam.static_binary_density, f"s{ii}_norm": hard._norm,
                    f"s{ii}_redz_final": redz_final, f"s{ii}_number": number})
    out["fobs_gw_edges"] = fobs_gw_edges
    save("ref_param_space.npz", **out)


def case_details():
    """``_calc_model_details`` (librarian/lib_tools.py:845-943) and ``run_model``'s deterministic keys."""
    from holodeck.librarian import lib_tools
    sam = make_sam((10, 11, 12), 0.0)
    hard = holo.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * GYR, rchar=100.0 * PC, gamma_inner=-1.0, gamma_outer=2.5)
    seed_rng(31)
    data = lib_tools.run_model(sam, hard, nfreqs=6, nreals=4, nloudest=2, gwb_flag=False, singles_flag=True,
                               details_flag=True, params_flag=False)
    out = dict(mtot=sam.mtot, mrat=sam.mrat, redz=sam.redz, fobs_cents=data['fobs_cents'],
               fobs_edges=data['fobs_edges'], number=data['number'], redz_final=data['redz_final'],
               gwb_mtot_redz_final=data['gwb_mtot_redz_final'], num_mtot_redz_final=data['num_mtot_redz_final'])
    for ii in range(4):
        out[f"gwb_params_{ii}"] = data['gwb_params'][ii]
        out[f"num_params_{ii}"] = data['num_params'][ii]
    save("ref_details.npz", **out, hard_time=3.0 * GYR)


def case_known_answers():
    """Known-answer values the reference pins for the strain formula (holodeck/tests/test_utils.py:52-96)."""
    path = os.path.join(ref_env.REF_SRC, "holodeck", "tests", "test_utils.py")
    tree = ast.parse(open(path).read())
    vals = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == "test_with_fixed_values":
            for stmt in node.body:
                if isinstance(stmt, ast.Assign) and isinstance(stmt.value, ast.List):
                    try:
                        vals[stmt.targets[0].id] = np.array(ast.literal_eval(stmt.value), dtype=float)
                    except (ValueError, TypeError):
                        pass
    assert {"m1", "m2", "dc", "mc", "hs"} <= set(vals)
    freq = 1.0 / YR
    save("ref_known_answers.npz", m1=vals["m1"], m2=vals["m2"], dc=vals["dc"], mc=vals["mc"], hs=vals["hs"],
         freq=freq, check_mc=holo.utils.chirp_mass(vals["m1"], vals["m2"]),
         check_hs=holo.utils.gw_strain_source(vals["mc"], vals["dc"], freq))


def main(only=None):
    if only:
        globals()[only]()
        return
    case_known_answers()
    case_loudest_edges()
    case_norm_sweep()
    case_small(0.0, "noscatter")
    case_small(0.28, "scatter")
    case_scatter_shapes()
    case_cfg1()
    case_params()
    case_details()
    case_param_space()


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
