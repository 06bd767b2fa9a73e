"""Library parameter spaces and batched library runs.

The Latin-hypercube samples and the parameter -> model mapping of PS_Classic_Phenom_Uniform
(librarian/lib_tools.py:34-541, librarian/param_spaces_classic.py:12-107) against the reference's own
output (``ref_param_space.npz``); the batched runner against one run_model call per sample.
"""

import numpy as np
import pytest

from conftest import load_golden, rel_err


def _significant_rel(a, b, floor=1e-12):
    a, b = np.asarray(a), np.asarray(b)
    m = np.abs(b) > floor * np.abs(b).max()
    return float((np.abs(a[m] - b[m]) / np.abs(b[m])).max())


def test_param_space_samples_match_reference():
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform
    g = load_golden("ref_param_space.npz")
    space = PS_Classic_Phenom_Uniform(nsamples=8, sam_shape=(10, 11, 12), seed=0)
    assert list(space.param_names) == [str(x) for x in g["param_names"]]
    assert np.array_equal(space._uniform_samples, g["uniform_samples"])
    assert np.array_equal(space.param_samples, g["param_samples"])
    assert np.array_equal(space.extrema, g["extrema"])
    assert space.lib_shape == (8, 6) and space.nparameters == 6
    p = space.normalized_params([0.5, None, 0.0, 1.0, 0.25, 0.5])
    assert p["gsmf_phi0_log10"] == -2.5 and p["mmb_mamp_log10"] == 7.6 and p["mmb_scatter_dex"] == 0.9
    assert p["gsmf_mchar0_log10"] == 11.5   # default = the distribution at 0.5


def test_param_space_models_on_the_host():
    """A sample's SAM (built without a device) carries the sample's parameters and the reference's
    grid edges; the hardening settings the space passes on are the reference's defaults and units."""
    from holodeck_gb300 import constants as C
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform
    g = load_golden("ref_param_space.npz")
    space = PS_Classic_Phenom_Uniform(nsamples=8, sam_shape=(10, 11, 12), seed=0)
    for ii in (0, 5):
        pars = {**space.DEFAULTS, **space.param_dict(ii)}
        sam = space._init_sam(space.sam_shape, pars)
        for name in ("mtot", "mrat", "redz"):
            assert rel_err(getattr(sam, name), g[f"s{ii}_{name}"]) < 1e-14, name
        assert sam._gsmf._phi0 == pars["gsmf_phi0_log10"] and sam._gsmf._alpha0 == pars["gsmf_alpha0"]
        assert rel_err(sam._gsmf._mchar0, C.MSOL * 10.0 ** pars["gsmf_mchar0_log10"]) < 1e-15
        assert rel_err(sam._mmbulge._mamp, C.MSOL * 10.0 ** pars["mmb_mamp_log10"]) < 1e-15
        assert sam._mmbulge._scatter_dex == pars["mmb_scatter_dex"] and sam._mmbulge._mplaw == 1.10
        assert sam._gmt._time_norm == 0.5 * C.GYR and sam._gpf._frac_norm > 0.0
    assert space.DEFAULTS["hard_sepa_init"] == 1e4 and space.DEFAULTS["hard_rchar"] == 100.0


def test_jobs_seeds_and_shapes():
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch
    shapes, nreals = batch.random_shapes(512, seed=0)
    arr = np.array(shapes)
    assert arr.min() >= 40 and arr.max() <= 91 and min(nreals) >= 100 and max(nreals) <= 1000
    assert batch.random_shapes(512, seed=0) == (shapes, nreals)
    space = PS_Classic_Phenom_Uniform(nsamples=5, seed=1)
    jobs = batch.make_jobs(space, shapes[:5], nreals[:5], seed=3)
    again = batch.make_jobs(space, shapes[:5], nreals[:5], seed=3, indices=[4, 2, 0, 1, 3])
    by_index = {j.index: j.seed for j in again}
    assert [j.seed for j in jobs] == [by_index[i] for i in range(5)]
    assert len({j.seed for j in jobs}) == 5
    m, q, z = shapes[0]
    assert jobs[0].cost(40) == (m - 1) * (q - 1) * (z - 1) * 40 * nreals[0]
    one = batch.make_jobs(space, (12, 13, 14), 7)
    assert all(j.shape == (12, 13, 14) and j.nreals == 7 for j in one)


@pytest.mark.gpu
def test_param_space_models_match_reference(built_lib):
    """Two library samples (with M-Mbulge scatter) built from their parameters: density, hardening
    normalisation, final redshifts and bin numbers against the reference's own models."""
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform
    from holodeck_gb300.sams import sam_cyutils
    g = load_golden("ref_param_space.npz")
    space = PS_Classic_Phenom_Uniform(nsamples=8, sam_shape=(10, 11, 12), seed=0)
    fe = g["fobs_gw_edges"]
    fc = 0.5 * (fe[1:] + fe[:-1])
    for ii in (0, 5):
        k = f"s{ii}_"
        settings = {**space.DEFAULTS, **space.param_dict(ii)}
        sam = space._init_sam(space.sam_shape, settings)
        assert sam._mmbulge._scatter_dex > 0.0
        # np.logspace may differ in the last bit between hosts: use the reference's own edges
        sam.mtot, sam.mrat, sam.redz = g[k + "mtot"], g[k + "mrat"], g[k + "redz"]
        hard = space._init_hard(sam, settings)
        assert rel_err(hard._norm, g[k + "norm"]) < 1e-9, ii
        dens = sam.static_binary_density
        assert np.array_equal(dens == 0.0, g[k + "density"] == 0.0), ii
        assert _significant_rel(dens, g[k + "density"]) < 1e-9, ii
        rf, dn = sam_cyutils.dynamic_binary_number_at_fobs(fc / 2.0, sam, hard)
        assert np.array_equal(rf == -1.0, g[k + "redz_final"] == -1.0), ii
        assert rel_err(rf, g[k + "redz_final"]) < 1e-9, ii
        number = sam_cyutils.integrate_differential_number_3dx1d(
            [sam.mtot, sam.mrat, sam.redz, fe / 2.0], dn)
        assert _significant_rel(number, g[k + "number"]) < 1e-9, ii


@pytest.mark.gpu
def test_batched_library_equals_per_sample_runs(built_lib):
    """run_library on several workers gives each sample's run_model result bit for bit; the waves knob
    moves hc_bg in the last bits only."""
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch, lib_tools
    space = PS_Classic_Phenom_Uniform(nsamples=6, seed=2)
    shapes, nreals = batch.random_shapes(6, lo=10, hi=16, reals_lo=5, reals_hi=20, seed=4)
    stats = {}
    out = batch.run_library(space, shapes, nreals, nfreqs=5, nloudest=3, seed=11, workers=3, waves=2,
                            gwb_flag=True, stats=stats)
    assert stats["samples"] == 6 and stats["failed"] == 0 and stats["workers"] == 3
    assert stats["realizations"] == sum(nreals)
    for ii in range(6):
        sam, hard = space.model_for_sample_number(ii, sam_shape=shapes[ii])
        ref = lib_tools.run_model(sam, hard, nfreqs=5, nreals=nreals[ii], nloudest=3, gwb_flag=True,
                                  seed=batch.sample_seed(11, ii))
        for key in ("hc_ss", "hc_bg", "gwb", "fobs_edges"):
            assert np.array_equal(out[ii][key], ref[key]), (ii, key)
    one = batch.run_library(space, shapes, nreals, nfreqs=5, nloudest=3, seed=11, workers=1, waves=1)
    for ii in range(6):
        assert np.array_equal(one[ii]["hc_ss"], out[ii]["hc_ss"])
        assert rel_err(one[ii]["hc_bg"], out[ii]["hc_bg"]) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("blocks_per_sm", [0, 4])
def test_batched_realizations_equal_per_sample_calls(built_lib, blocks_per_sm):
    """One bulk launch over several samples' work items gives every sample's own loudest_device result
    bit for bit: expectations from 1e-4 to 1e8 (every sampler regime, FP64 wide bins included),
    different bin counts, realization counts across several groups of 1024."""
    import torch
    from holodeck_gb300 import cyutils, single_sources
    from holodeck_gb300 import _device as D
    rng = np.random.default_rng(21)
    nf, nl = 3, 4
    samples = []
    for nb, nr in ((5000, 7), (20011, 1030), (777, 2100), (3, 1)):
        lam = 10.0 ** rng.uniform(-4.0, 8.0, size=(nb, nf))
        lam[rng.random((nb, nf)) < 0.3] = 0.0
        h = 10.0 ** rng.uniform(-32.0, -26.0, size=(nb, nf))
        num = torch.as_tensor(lam, device="cuda")
        hh = torch.as_tensor(h, device="cuda")
        samples.append(dict(number=num, h2fdf=hh, order=single_sources.sort_order_device(hh), nreals=nr,
                            seed=1000 + nb, status=D.StatusWord()))
    got = cyutils.loudest_batch_device(samples, nl, blocks_per_sm=blocks_per_sm)
    for smp, (ss, bg) in zip(samples, got):
        ref_ss, ref_bg = cyutils.loudest_device(smp["number"], smp["h2fdf"], smp["nreals"], nl, smp["order"],
                                                seed=smp["seed"])
        assert torch.equal(ss, ref_ss) and torch.equal(bg, ref_bg), smp["number"].shape
        assert smp["status"].read() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("blocks_per_sm", [0, 3])
def test_device_batched_library_equals_per_sample_runs(built_lib, blocks_per_sm):
    """run_library with the realizations of up to four samples per launch gives each sample's
    run_model result bit for bit (two launches for six samples)."""
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch, lib_tools
    space = PS_Classic_Phenom_Uniform(nsamples=6, seed=2)
    shapes, nreals = batch.random_shapes(6, lo=10, hi=18, reals_lo=5, reals_hi=1500, seed=4)
    stats = {}
    out = batch.run_library(space, shapes, nreals, nfreqs=5, nloudest=3, seed=11, workers=3, waves=2,
                            gwb_flag=True, stats=stats, batch=4, blocks_per_sm=blocks_per_sm)
    assert stats["failed"] == 0 and stats["batch"] == 4
    for ii in range(6):
        sam, hard = space.model_for_sample_number(ii, sam_shape=shapes[ii])
        ref = lib_tools.run_model(sam, hard, nfreqs=5, nreals=nreals[ii], nloudest=3, gwb_flag=True,
                                  seed=batch.sample_seed(11, ii))
        for key in ("hc_ss", "hc_bg", "gwb", "fobs_edges"):
            assert np.array_equal(out[ii][key], ref[key]), (ii, key)


@pytest.mark.gpu
def test_autotune_times_every_candidate(built_lib):
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch
    from holodeck_gb300 import _native as N
    space = PS_Classic_Phenom_Uniform(nsamples=4, seed=5)
    shapes, nreals = batch.random_shapes(4, lo=12, hi=18, reals_lo=10, reals_hi=30, seed=6)
    jobs = batch.make_jobs(space, shapes, nreals)
    before = N.load().hgb_get_bulk_waves()
    res = batch.autotune(space, jobs, nfreqs=4, nloudest=2, candidates=((1, 2), (2, 1)), probe=3, use_cache=False)
    assert set(res["table"]) == {"1,2", "2,1"} and all(v > 0 for v in res["table"].values())
    assert (res["workers"], res["waves"]) in ((1, 2), (2, 1))
    assert N.load().hgb_get_bulk_waves() == before
    assert batch.autotune(space, jobs, nfreqs=4, nloudest=2, candidates=((1, 2),), probe=3)["workers"] in (1, 2)


def test_resume_loads_finished_samples_without_running_them(tmp_path):
    """A rerun skips every sample whose file holds a result (gen_lib.py:288-300): with all files
    present nothing is run, so no device is needed; a failure file does not count as finished."""
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch
    space = PS_Classic_Phenom_Uniform(nsamples=4, seed=3)
    jobs = batch.make_jobs(space, (12, 12, 12), 5)
    fake = {}
    for job in jobs:
        res = dict(fobs_cents=np.arange(3.0), fobs_edges=np.arange(4.0), hc_ss=np.full((3, 5, 2), job.index + 1.0),
                   hc_bg=np.full((3, 5), job.index + 0.5))
        batch._save_sim_file(batch.sim_fname(tmp_path, job.index), space, job, res, None)
        fake[job.index] = res
    stats = {}
    out = batch.run_library(space, (12, 12, 12), 5, nfreqs=3, nloudest=2, output_dir=tmp_path, stats=stats)
    assert stats["skipped"] == 4 and stats["failed"] == 0 and stats["realizations"] == 0
    for ii, res in enumerate(out):
        assert np.array_equal(res["hc_ss"], fake[ii]["hc_ss"]) and np.array_equal(res["hc_bg"], fake[ii]["hc_bg"])
        assert np.array_equal(res["params"], [space.param_dict(ii)[pn] for pn in space.param_names])
    batch._save_sim_file(batch.sim_fname(tmp_path, 9), space, jobs[0], None, RuntimeError("boom"))
    assert batch.load_sim_file(batch.sim_fname(tmp_path, 9)) is None
    with np.load(batch.sim_fname(tmp_path, 9)) as z:
        assert list(z.files) == ["fail"] and "boom" in str(z["fail"])


class _FailingSpace:
    """A parameter space whose model for one sample raises (a host-side injected failure)."""

    def __init__(self, space, bad):
        self._space, self._bad = space, bad

    def __getattr__(self, name):
        return getattr(self._space, name)

    def model_for_params(self, params, sam_shape=None):
        if params == self._space.param_dict(self._bad):
            raise RuntimeError("injected failure")
        return self._space.model_for_params(params, sam_shape)


@pytest.mark.gpu
def test_failed_sample_is_isolated_and_resumed(built_lib, tmp_path):
    """An exception in one sample marks that sample failed (a 'fail' file, None result, NaN rows in
    the written library) and leaves the others intact; a rerun runs only the failed sample; more
    failures than max_failures raise."""
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch, lib_tools
    space = PS_Classic_Phenom_Uniform(nsamples=5, seed=2)
    shapes, _ = batch.random_shapes(5, lo=10, hi=14, seed=8)
    nreals = [7] * 5     # one realization count, as a combined library file holds
    kw = dict(nfreqs=4, nloudest=2, seed=13, workers=2, waves=2)
    stats = {}
    out = batch.run_library(_FailingSpace(space, 2), shapes, nreals, output_dir=tmp_path, stats=stats, **kw)
    assert stats["failed"] == 1 and 2 in stats["errors"] and out[2] is None
    assert batch.load_sim_file(batch.sim_fname(tmp_path, 2)) is None
    clean = batch.run_library(space, shapes, nreals, **kw)
    for ii in (0, 1, 3, 4):
        assert np.array_equal(out[ii]["hc_ss"], clean[ii]["hc_ss"]) and np.array_equal(out[ii]["hc_bg"], clean[ii]["hc_bg"])
    lib = lib_tools.write_library(str(tmp_path / "lib.npz"), out, space.param_samples, space.param_names)
    with np.load(lib) as z:
        assert np.all(np.isnan(z["hc_bg"][2])) and np.all(np.isnan(z["sample_params"][2]))
        assert np.all(np.isfinite(z["hc_bg"][[0, 1, 3, 4]]))
    stats = {}
    again = batch.run_library(space, shapes, nreals, output_dir=tmp_path, stats=stats, **kw)
    assert stats["skipped"] == 4 and stats["failed"] == 0 and stats["realizations"] == nreals[2]
    assert np.array_equal(again[2]["hc_ss"], clean[2]["hc_ss"]) and np.array_equal(again[2]["hc_bg"], clean[2]["hc_bg"])
    with pytest.raises(RuntimeError, match="max_failures"):
        batch.run_library(_FailingSpace(space, 1), shapes, nreals, max_failures=0, **kw)


@pytest.mark.gpu
def test_failing_reduce_fails_only_its_sample(built_lib, monkeypatch):
    """A caller's ``reduce`` that raises for one sample marks that sample failed; the others finish
    (the worker thread survives)."""
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch
    space = PS_Classic_Phenom_Uniform(nsamples=5, seed=4)

    def fake_run_model(sam, hard, nreals=1, **kw):
        return dict(hc_bg=np.full((2, nreals), 1.0))

    monkeypatch.setattr(batch, "run_model", fake_run_model)
    monkeypatch.setattr(space, "model_for_params", lambda params, shape: (None, None))

    def reduce(res):
        if res["hc_bg"].shape[1] == 3:
            raise ValueError("bad sample")
        return float(res["hc_bg"].sum())

    jobs = batch.make_jobs(space, (10, 10, 10), [1, 2, 3, 4, 5])
    results, errors = batch._run_jobs(space, jobs, 2, 2, 1, 16.0, dict(singles_flag=True), reduce=reduce)
    assert set(errors) == {2} and isinstance(errors[2], ValueError)
    assert results[2] is None and [results[i] for i in (0, 1, 3, 4)] == [2.0, 4.0, 8.0, 10.0]
