"""Benchmark: SAM GWB realizations/s on one GB300 (plain GPU SAM).

Workload (the default-grid configuration): Semi_Analytic_Model on the 91 (mtot) x 81 (mrat) x 101 (redz)
grid with GSMF_Schechter(phi0=-2.77, mchar0_log10=11.24, alpha0=-1.24), GPF_Power_Law, GMT_Power_Law and
MMBulge_KH2013(mamp_log10=8.69, mplaw=1.17, scatter 0.28 dex); Fixed_Time_2PL_SAM(3 Gyr, rchar=100 pc,
gamma_inner=-1, gamma_outer=+2.5, sepa_init=1 kpc); 40 harmonics of 1/(16 yr); 1000 realizations,
10 loudest.  One step = one full model evaluation: build the SAM (density with M-Mbulge scatter),
find the hardening normalisation, and gwb() (dynamic binary number, integration, strain, sort,
Poisson realizations with the loudest split).  value = realizations / s.

The line also carries ``batched``: a whole library of 512 Latin-hypercube samples of
PS_Classic_Phenom_Uniform, each on its own grid (40-91 per axis) with its own realization count
(100-1000), run through the batched library API (realizations/s over the library); ``warm``: the
same workload on a reused model instance (density, scatter and hardening norm cached); ``highres``:
the 181x161x201, 100-frequency, 10^4-realization workload; and ``emulator``: the MLP ensemble trained on a GPU-SAM library of the same space at the default grid,
its held-out accuracy and query time against the plain GPU SAM's time for the same query.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --stages        # per-stage device times
    python bench.py --batched       # only the batched-library measurement
    python bench.py --emulator [--emulator-samples 20000]   # only the emulator measurement
    python bench.py --highres --steps 2   # the 181x161x201, 100-frequency, 10^4-realization workload
    python bench.py --profile --nfreqs K   # one untimed evaluation (the program ncu captures)

--impl reference times the CPU restatement of the reference path (the oracle) on the host cores.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPE = (91, 81, 101)
NFREQ = 40
NREALS = 1000
NLOUD = 10
METRIC = "SAM GWB realizations/s on 1 GB300: plain vs batched vs emulator at stated hc error"
UNIT = "realizations/s"
CONFIG_NAME = "plain SAM, 91x81x101 grid, 40 harmonics of 1/(16 yr), 1000 realizations, 10 loudest"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------

def make_model(H, C, shape=SHAPE, edges=None):
    """The bench model (SAM + hardening); ``edges`` replaces the grid's (mtot, mrat, redz) edges."""
    gsmf = H.sams.GSMF_Schechter(phi0=-2.77, mchar0_log10=11.24, alpha0=-1.24)
    mmb = H.host_relations.MMBulge_KH2013(mamp_log10=8.69, mplaw=1.17, scatter_dex=0.28)
    sam = H.sams.Semi_Analytic_Model(gsmf=gsmf, gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=mmb, shape=shape)
    if edges is not None:
        sam.mtot, sam.mrat, sam.redz = (np.asarray(e, dtype=np.float64) for e in edges)
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, sepa_init=1.0e3 * C.PC, rchar=100.0 * C.PC,
                                          gamma_inner=-1.0, gamma_outer=2.5)
    return sam, hard


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def issue_roofline(instr, t_launch, clk, n_sm=152, schedulers=4):
    """Warp-instruction issue rate of a launch against the GPU's peak (one instruction per clock per
    SM sub-partition at the sampled maximum SM clock)."""
    mhz = (clk or {}).get("sm_max_mhz") or 2070.0
    if not instr or not t_launch:
        return None
    peak = n_sm * schedulers * mhz * 1e6
    achieved = instr / t_launch
    return {"achieved": achieved, "peak": peak, "unit": "warp instructions/s", "frac": achieved / peak,
            "instructions_per_launch": instr, "sm_mhz_for_peak": mhz}


def run_gpu(args):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    from holodeck_gb300 import _native as N
    from holodeck_gb300 import single_sources

    _, fe = H.utils.pta_freqs(16.0 * C.YR, NFREQ)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")   # > 129 MB of L2
    seed0 = 1000 * (rank + 1)
    N.reset_launch_count()

    def step(i, keep_on_device=True):
        sam, hard = make_model(H, C)
        if keep_on_device:
            return sam.gwb(fe, hard=hard, realize=NREALS, loudest=NLOUD, seed=seed0 + i, return_torch=True,
                           precision=args.precision)
        return sam.gwb(fe, hard=hard, realize=NREALS, loudest=NLOUD, seed=seed0 + i, precision=args.precision)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()

    # ---- value: device-resident results, K steps between events
    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    N.reset_launch_count()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for i in range(args.steps):
        flush.zero_()
        step(args.warmup + i)
    t1.record()
    barrier()
    launches = N.launch_count()
    clk = clocks.stop()
    ms = t0.elapsed_time(t1) / args.steps
    if world > 1:
        tt = torch.tensor([ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    value = world * NREALS / (ms / 1e3)

    # ---- warm: the same model instance again (density, scatter and hardening norm cached on it, as
    # the reference caches static_binary_density); dbn, integration, strain, sort and realizations
    # recomputed every step
    warm_sam, warm_hard = make_model(H, C)
    warm_sam.gwb(fe, hard=warm_hard, realize=NREALS, loudest=NLOUD, seed=seed0, return_torch=True,
                 precision=args.precision)
    barrier()
    w0 = torch.cuda.Event(enable_timing=True)
    w1 = torch.cuda.Event(enable_timing=True)
    w0.record()
    for i in range(args.steps):
        flush.zero_()
        warm_sam.gwb(fe, hard=warm_hard, realize=NREALS, loudest=NLOUD, seed=seed0 + 7919 + i, return_torch=True,
                     precision=args.precision)
    w1.record()
    barrier()
    warm_ms = w0.elapsed_time(w1) / args.steps
    del warm_sam, warm_hard

    # ---- e2e: the public numpy API (results copied to host every step)
    barrier()
    te0 = time.perf_counter()
    for i in range(args.steps):
        hc_ss, hc_bg = step(args.warmup + args.steps + i, keep_on_device=False)
    barrier()
    e2e_ms = (time.perf_counter() - te0) * 1e3 / args.steps
    if world > 1:
        tt = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_ms = float(tt.item())
    h2d = 8 * (sum(SHAPE) + NFREQ + 1)
    d2h = int(hc_ss.nbytes + hc_bg.nbytes)

    # ---- roofline of the realization kernel (CUDA events on the launching stream)
    sam, hard = make_model(H, C)
    fo_c = H.utils.midpoints(fe) / 2.0
    rf, dn = sam._dbn_device(hard, fo_c)
    number, h2fdf = sam._number_and_strain(fe / 2.0, dn, rf)
    order = single_sources.sort_order_device(h2fdf)
    from holodeck_gb300 import cyutils
    nb = int(number.numel() // NFREQ)
    lib = N.load()
    N.check(lib.hgb_bulk_timing(1), "hgb_bulk_timing")
    times = []
    for i in range(3):
        flush.zero_()
        cyutils.loudest_device(number.reshape(-1, NFREQ), h2fdf.reshape(-1, NFREQ), NREALS, NLOUD, order, seed=i)
        torch.cuda.synchronize()
        times.append(float(lib.hgb_bulk_last_ms()) / 1e3)
    N.check(lib.hgb_bulk_timing(0), "hgb_bulk_timing")
    t_real = sum(times) / len(times)
    draws = nb * NFREQ * NREALS
    # algorithmic bytes of one k_bulk launch, per realization group: every bin's expectation and the
    # strain of the bins with a nonzero expectation (8 B each), each realization's first bulk
    # position read, the per-chunk partials written
    n_rgroups = -(-NREALS // 1024)
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    nchunk = max(1, -(-n_sm * 6 * lib.hgb_get_bulk_waves() // (NFREQ * n_rgroups)))
    n_pos = int((number > 0).sum().item())
    alg_bytes = (8 * nb * NFREQ + 8 * n_pos) * n_rgroups + 4 * NFREQ * NREALS + 8 * nchunk * NFREQ * NREALS
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg_bytes / t_real / 1e9
    traffic = None
    instr = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            prof = json.load(fh)
            traffic = prof.get("k_bulk_bytes_per_launch")
            instr = prof.get("k_bulk_warp_instructions_per_launch")
    except (OSError, ValueError):
        pass

    batched = run_batched(args, rank, world) if args.batched_samples > 0 else None
    highres = None
    if args.highres_steps > 0 and rank == 0:
        hargs = argparse.Namespace(**vars(args))
        hargs.steps = args.highres_steps
        highres = run_highres(hargs)
        torch.cuda.empty_cache()
    emulator = run_emulator(args) if (args.emulator_samples > 0 and rank == 0) else None
    cpu = hc_error = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, keep = cpu_baseline_sample(args)
        hc_error = hc_error_vs_oracle(keep)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 grids / f32+int32 realizations",
            "data": "synthetic (analytic model parameters; no dataset)",
            "config": {"workload": CONFIG_NAME, "grid": list(SHAPE), "nfreqs": NFREQ, "nreals": NREALS,
                       "nloudest": NLOUD, "rng": "philox4x32-10", "l2": "flushed (256 MB write) before every step",
                       "parallelism": f"replicas x{world}",
                       "note": "scatter geometry plan cached per grid; every other stage recomputed each step"},
            "e2e": {"value": world * NREALS / (e2e_ms / 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": {"kernel": "k_bulk", "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                         "launch_s": t_real, "draws_per_s": draws / t_real,
                         "issue": issue_roofline(instr, t_real, clk),
                         "note": ("issue-bound sampler: the HBM fraction is shown for the contract; the "
                                  "issue object is the bound that applies (warp instructions per launch "
                                  "from ncu, see profiles/)")},
            "clocks": clk,
            "cpu_baseline": cpu,
            "hc_error": hc_error,
            "warm": {"value": world * NREALS / (warm_ms / 1e3), "unit": UNIT, "ms_per_step": warm_ms,
                     "note": "same model instance each step: density, M-Mbulge scatter and hardening "
                             "normalisation cached on it; everything from the dbn stage on recomputed"},
            "batched": batched,
            "highres": highres,
            "emulator": emulator,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


BATCH_CONFIG = ("batched library: Latin-hypercube samples (seed 0) of PS_Classic_Phenom_Uniform (gsmf_phi0, "
                "gsmf_mchar0_log10, mmb_mamp_log10, mmb_scatter_dex, hard_time, hard_gamma_inner), per-sample grid "
                "uniform integers in [40, 91] per axis and realizations in [100, 1000] (default_rng(0)), "
                "40 frequencies, 10 loudest")


def run_batched(args, rank=0, world=1):
    """The batched-library workload through the public library API (host parameters in, host arrays
    out): samples rank, rank + world, ... of the library on this rank's GPU.  Returns the object the
    bench line carries (on rank 0; the wall time is the max over ranks)."""
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch
    n = args.batched_samples
    space = PS_Classic_Phenom_Uniform(nsamples=n, seed=0)
    shapes, nreals = batch.random_shapes(n, seed=0)
    stats = {}
    out = batch.run_library(space, shapes, nreals, nfreqs=NFREQ, nloudest=NLOUD, seed=1,
                            indices=batch.shard_indices(n, rank, world), stats=stats)
    job = batch.reduce_stats(stats)                       # max wall time, summed work over the replicas
    wall, reals, draws = job["seconds"], job["realizations"], job["draws"]
    d2h = sum(sum(v.nbytes for k, v in r.items() if isinstance(v, np.ndarray)) for r in out if r is not None)
    tuning = stats.get("tuning") or {}
    table = tuning.get("table", {})
    ones = [v for k, v in table.items() if k.split(",")[0] == "1"]
    one = max(ones) if ones else None
    best = table.get(f"{stats['workers']},{stats['waves']}")
    return {"workload": BATCH_CONFIG, "samples": n, "failed": job["failed"], "seconds": wall,
            "value": reals / wall, "unit": UNIT, "samples_per_s": n / wall, "draws_per_s": draws / wall,
            "realizations": int(reals), "schedule": {"workers": stats["workers"], "waves": stats["waves"]},
            "autotune_draws_per_s": table,
            "speedup_vs_one_worker_in_probe": (best / one) if (best and one) else None,
            "e2e": "host parameters in, host hc_ss / hc_bg out; per-sample scatter plans built on the host "
                   "inside the timed region", "d2h_bytes": int(d2h)}


EMU_CONFIG = ("learned emulator: 4-member ensemble of MLPs 6 -> 4x256 (SiLU) -> 40 x (5/50/95th percentile "
              "log10 hc, median log10 loudest-source hc), bf16 weights and activations, fp32 accumulation on "
              "tcgen05, AdamW; trained on Latin-hypercube samples (seed 0) of PS_Classic_Phenom_Uniform at the "
              "91x81x101 grid with 500 realizations, tested on held-out samples (seed 1)")


def run_emulator(args):
    """Train the emulator on a GPU-SAM library and measure it against the plain GPU SAM: held-out
    accuracy (and the nearest-library-sample answer a user has without the network, and the
    realization-noise floor of the held-out truth), query latency through the CUDA-graph path, and
    the plain GPU SAM's time for the same query."""
    import torch
    from holodeck_gb300 import emulator as EM
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform
    n_tr = args.emulator_samples
    n_te = max(64, n_tr // 10)
    sp_tr = PS_Classic_Phenom_Uniform(nsamples=n_tr, seed=0)
    sp_te = PS_Classic_Phenom_Uniform(nsamples=n_te, seed=1)
    lib_stats = {}
    cache = args.emulator_cache
    if cache and os.path.exists(cache):
        with np.load(cache) as z:
            assert np.array_equal(z["params_train"], sp_tr.param_samples), "cache holds another library"
            y_tr, y_te, y_te2 = z["y_train"], z["y_test"], z["y_test2"]
            lib_stats["seconds"] = float(z["library_seconds"])
    else:
        y_tr = EM.training_library(sp_tr, seed=2, stats=lib_stats)
        y_te = EM.training_library(sp_te, seed=3)
        y_te2 = EM.training_library(sp_te, seed=4)         # same held-out models, other realizations
        if cache:
            np.savez(cache, params_train=sp_tr.param_samples, params_test=sp_te.param_samples, y_train=y_tr,
                     y_test=y_te, y_test2=y_te2, library_seconds=lib_stats["seconds"])
    ok = np.all(np.isfinite(y_tr), axis=(1, 2))
    emu = EM.Emulator(sp_tr, nfreqs=NFREQ, members=4, width=256, depth=4, seed=0)
    steps_per_epoch = max(1, int(ok.sum()) // 512)
    epochs = max(50, -(-args.emulator_steps // steps_per_epoch))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = emu.fit(sp_tr.param_samples[ok], y_tr[ok], epochs=epochs, batch=512, lr=2e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    mean, spread, inside = emu.predict(sp_te.param_samples)
    spread_p50 = emu.predict(sp_te.param_samples, spread_stats=("log10_hc_p50",))[1]
    spread_hc = emu.predict(sp_te.param_samples, spread_stats=("log10_hc_p05", "log10_hc_p50", "log10_hc_p95"))[1]
    good = np.all(np.isfinite(y_te), axis=(1, 2)) & np.all(np.isfinite(y_te2), axis=(1, 2))
    err = np.abs(mean - y_te)[good]
    u_tr, u_te = emu.unit(sp_tr.param_samples[ok]), emu.unit(sp_te.param_samples)
    nn = np.argmin(((u_te[:, None, :] - u_tr[None, :, :]) ** 2).sum(-1), axis=1)
    err_nn = np.abs(y_tr[ok][nn] - y_te)[good]
    noise = np.abs(y_te - y_te2)[good] / np.sqrt(2.0)
    g1, gb = emu.graphed(1), emu.graphed(1024)
    q1 = sp_te.param_samples[:1]
    qb = np.resize(sp_te.param_samples, (1024, sp_te.param_samples.shape[1]))
    t_q1 = EM.timed(g1, q1, repeat=50)
    t_qb = EM.timed(gb, qb, repeat=20)
    solve = EM.sam_fallback(sp_tr, sam_shape=SHAPE, nreals=500, nfreqs=NFREQ, seed=5)
    t_plain = EM.timed(solve, q1[0], repeat=3)
    names = list(EM.STATS)

    def med(a):
        return {nm: float(np.median(a[..., k])) for k, nm in enumerate(names)}

    return {"workload": EMU_CONFIG, "train_samples": int(ok.sum()), "test_samples": int(good.sum()),
            "library_seconds": lib_stats.get("seconds"), "library_samples_per_s": n_tr / lib_stats["seconds"],
            "train_seconds": t_train, "train_steps": epochs * steps_per_epoch, "final_loss": hist[-1],
            "median_abs_dlog10": med(err), "p95_abs_dlog10": {nm: float(np.percentile(err[..., k], 95))
                                                             for k, nm in enumerate(names)},
            "nearest_sample_median_abs_dlog10": med(err_nn), "realization_noise_median_dlog10": med(noise),
            "ensemble_spread_median_dex": float(np.median(spread)),
            "flagged_fraction_at_0.05dex": float(np.mean(spread > 0.05)),
            "flagged_fraction_at_0.05dex_by_criterion": {
                "all_outputs": float(np.mean(spread > 0.05)),
                "hc_percentiles": float(np.mean(spread_hc > 0.05)),
                "median_hc": float(np.mean(spread_p50 > 0.05))},
            "query_s_batch1": t_q1, "query_s_per_sample_batch1024": t_qb / 1024,
            "plain_gpu_sam_s": t_plain, "speedup_vs_plain_batch1": t_plain / t_q1,
            "speedup_vs_plain_batch1_with_fallbacks": {
                nm: t_plain / (t_q1 + float(np.mean(sv > 0.05)) * t_plain)
                for nm, sv in (("all_outputs", spread), ("hc_percentiles", spread_hc), ("median_hc", spread_p50))},
            "speedup_vs_plain_batch1024": t_plain / (t_qb / 1024)}


# ------------------------------------------------------------------------------------------------
# CPU restatement (oracle): bounded sample, extrapolated to the full workload
# ------------------------------------------------------------------------------------------------

SAMPLE_Z = 11
SAMPLE_R = 3


def _oracle_sample(seed, nreals, keep=None):
    """Times the oracle path on the sample grid (91 x 81 x 11): stage seconds.  With ``keep`` (a
    dict) it also receives the sample's edges, frequency edges, grids and loudest-first order."""
    from oracle import sam_oracle as O
    from holodeck_gb300 import constants as C
    shape = (SHAPE[0], SHAPE[1], SAMPLE_Z)
    mtot, mrat, redz = O.grid_edges(shape)
    p = O.default_params(scatter_dex=0.28)
    t = {}
    t0 = time.perf_counter()
    parts = O.static_binary_density(mtot, mrat, redz, p, return_parts=True)
    t["density"] = time.perf_counter() - t0
    mt, mr = np.meshgrid(mtot, mrat, indexing="ij")
    t0 = time.perf_counter()
    norm = 10.0 ** O.find_2pwl_hardening_norm(3.0 * C.GYR, mt.ravel(), mr.ravel(), 1.0e3 * C.PC, 100.0 * C.PC,
                                              -1.0, 2.5, 300).reshape(mt.shape)
    t["norm"] = time.perf_counter() - t0
    _, fe = O.pta_freqs(16.0 * C.YR, NFREQ)
    fo_c = O.midpoints(fe) / 2.0
    t0 = time.perf_counter()
    rf, dn = O.dbn_2pwl(fo_c, 1.0e3 * C.PC, 300, norm, 100.0 * C.PC, -1.0, 2.5, parts["density"], mtot, mrat, redz,
                        parts["gmt_time"])
    t["dbn"] = time.perf_counter() - t0
    edges = [mtot, mrat, redz, fe / 2.0]
    t0 = time.perf_counter()
    number = O.integrate_differential_number_3dx1d(edges, dn)
    h2fdf = O.char_strain_sq_from_bin_edges_redz(edges, rf)
    order = O.sort_order(h2fdf)
    t["integrate_strain"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.loudest_hc_from_sorted(number, h2fdf, nreals, NLOUD, order, seed=seed)
    t["realize"] = time.perf_counter() - t0
    if keep is not None:
        keep.update(edges=[mtot, mrat, redz], fobs_gw_edges=fe, number=number, h2fdf=h2fdf, order=order,
                    redz_final=rf)
    return t


def _extrapolate(t, nreals_sampled):
    """Full-workload seconds per model: the Z-sliced stages scale with the redshift bins, the
    hardening normalisation is Z-independent, realizations scale with bins and count."""
    zscale = (SHAPE[2] - 1) / (SAMPLE_Z - 1)
    grid = zscale * (t["density"] + t["dbn"] + t["integrate_strain"]) + t["norm"]
    per_real = zscale * t["realize"] / nreals_sampled
    return grid + NREALS * per_real, grid, per_real


def cpu_baseline_sample(args):
    keep = {}
    t = _oracle_sample(seed=7, nreals=SAMPLE_R, keep=keep)
    total, grid, per_real = _extrapolate(t, SAMPLE_R)
    return {"value": NREALS / total, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": (f"oracle on grid 91x81x{SAMPLE_Z} with {SAMPLE_R} realizations, extrapolated linearly in "
                       f"redshift bins and realizations: grid stages {grid:.1f} s + {per_real:.2f} s/realization "
                       f"({', '.join(f'{k} {v:.2f}s' for k, v in t.items())})")}, keep


def hc_error_vs_oracle(keep, nreals=8):
    """The GPU path's strain against the FP64 oracle on the CPU baseline's sample model (the bench
    model on a 91 x 81 x 11 grid, 40 frequencies): the oracle's grids and numpy-PCG64 Poisson counts
    replayed through the public gwb(); max relative error of hc_ss and hc_bg, and of the number and
    strain grids."""
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    from oracle import sam_oracle as O
    sam, hard = make_model(H, C, shape=tuple(len(e) for e in keep["edges"]), edges=keep["edges"])
    fe = keep["fobs_gw_edges"]
    counts = O.replay_counts(keep["number"], keep["order"], nreals, 11)
    ss_o, bg_o = O.ss_gws_redz(keep["edges"] + [fe / 2.0], keep["redz_final"], keep["number"], nreals, NLOUD,
                               counts=counts)
    ss, bg = sam.gwb(fe, hard=hard, realize=nreals, loudest=NLOUD, replay=counts, order=keep["order"])
    rf, dn = sam._dbn_device(hard, O.midpoints(fe) / 2.0)
    number, h2fdf = sam._number_and_strain(fe / 2.0, dn, rf)

    def rel(a, b):
        a, b = np.asarray(a), np.asarray(b)
        scale = np.maximum(np.abs(a), np.abs(b))
        m = scale > 0
        return float((np.abs(a - b)[m] / scale[m]).max()) if m.any() else 0.0

    return {"case": (f"bench model on the 91x81x{SAMPLE_Z} grid, {NFREQ} frequencies, {nreals} realizations replayed "
                     "from numpy PCG64 Poisson draws, against the FP64 CPU oracle"),
            "hc_ss_max_rel": rel(ss, ss_o), "hc_bg_max_rel": rel(bg, bg_o),
            "hc_bg_max_rel_per_freq": [rel(bg[f], bg_o[f]) for f in range(bg.shape[0])],
            "number_max_rel": rel(number.cpu().numpy(), keep["number"]),
            "h2fdf_max_rel": rel(h2fdf.cpu().numpy(), keep["h2fdf"])}


def _worker(args):
    seed, nreals = args
    return _oracle_sample(seed, nreals)


def run_reference(args):
    """Reference arm: the CPU restatement on all host cores (one sample model per worker process)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    ncores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    results = []
    with ctx.Pool(ncores) as pool:
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_worker, [(1000 * i + k, SAMPLE_R) for k in range(ncores)])
            wall = time.perf_counter() - t0
            if i >= args.warmup:
                results.append((wall, res))
    # each worker ran the same sample model; the pool finishes ncores samples per wall time
    per_model = []
    for wall, res in results:
        cpu_total = sum(_extrapolate(t, SAMPLE_R)[0] for t in res) / len(res)
        cpu_sample = sum(sum(t.values()) for t in res) / len(res)
        per_model.append(cpu_total * (wall / cpu_sample) / ncores)   # wall-clock seconds per full model
    sec = statistics.median(per_model)
    value = NREALS / sec
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": CONFIG_NAME, "grid": list(SHAPE), "nfreqs": NFREQ, "nreals": NREALS,
                       "nloudest": NLOUD},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": (f"{ncores} processes, each the oracle on grid 91x81x{SAMPLE_Z} with "
                                        f"{SAMPLE_R} realizations per step, extrapolated linearly to the full "
                                        "workload")},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_profile(args):
    """One model evaluation of the bench workload with ``--nfreqs`` frequencies, no timing: the
    program the ncu captures run (a smaller frequency count keeps a full capture short)."""
    import torch
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    _, fe = H.utils.pta_freqs(16.0 * C.YR, NFREQ)
    fe = fe[:args.nfreqs + 1]
    for i in range(args.warmup + 1):
        sam, hard = make_model(H, C)
        sam.gwb(fe, hard=hard, realize=NREALS, loudest=NLOUD, seed=i, return_torch=True, precision=args.precision)
    torch.cuda.synchronize()
    print(json.dumps({"profile": CONFIG_NAME, "nfreqs": args.nfreqs, "evaluations": args.warmup + 1,
                      "precision": args.precision}))


HIRES_SHAPE = (181, 161, 201)
HIRES_NFREQ, HIRES_NREALS = 100, 10000


def run_highres(args):
    """The high-resolution workload: 181 x 161 x 201 grid, 100 harmonics of 1/(16 yr), 10^4
    realizations, 10 loudest (about 5.8e12 draws per evaluation), one untimed and ``--steps`` timed
    evaluations (device-resident results), and the check of the realization mean of the total
    characteristic strain against its FP64 expectation sum_b number_b h2fdf_b per frequency (the
    z-score with the Poisson variance sum_b number_b h2fdf_b^2)."""
    import torch
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    gsmf = H.sams.GSMF_Schechter(phi0=-2.77, mchar0_log10=11.24, alpha0=-1.24)
    mmb = H.host_relations.MMBulge_KH2013(mamp_log10=8.69, mplaw=1.17, scatter_dex=0.28)
    _, fe = H.utils.pta_freqs(16.0 * C.YR, HIRES_NFREQ)

    def model():
        sam = H.sams.Semi_Analytic_Model(shape=HIRES_SHAPE, gsmf=gsmf, gpf=H.sams.GPF_Power_Law(),
                                         gmt=H.sams.GMT_Power_Law(), mmbulge=mmb)
        hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, sepa_init=1.0e3 * C.PC, rchar=100.0 * C.PC,
                                              gamma_inner=-1.0, gamma_outer=2.5)
        return sam, hard

    sam, hard = model()
    sam.gwb(fe, hard=hard, realize=HIRES_NREALS, loudest=NLOUD, seed=1, return_torch=True)
    times = []
    for i in range(args.steps):
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        sam, hard = model()
        ss, bg = sam.gwb(fe, hard=hard, realize=HIRES_NREALS, loudest=NLOUD, seed=2 + i, return_torch=True)
        t1.record()
        torch.cuda.synchronize()
        times.append(t0.elapsed_time(t1) / 1e3)
    redz_final, diff_num = sam._dbn_device(hard, H.utils.midpoints(fe) / 2.0)
    number, h2fdf = sam._number_and_strain(fe / 2.0, diff_num, redz_final)
    del redz_final, diff_num
    lam, h = number.reshape(-1, HIRES_NFREQ), h2fdf.reshape(-1, HIRES_NFREQ)
    s1 = (lam * h).sum(0).cpu().numpy()
    s2 = (lam * h * h).sum(0).cpu().numpy()
    nb = int(lam.shape[0])
    del number, h2fdf, lam, h
    total = (bg ** 2 + (ss ** 2).sum(-1)).cpu().numpy()
    z = (total.mean(1) - s1) / np.sqrt(s2 / HIRES_NREALS)
    sec = statistics.median(times)
    return {"workload": (f"high-resolution plain SAM: grid {HIRES_SHAPE[0]}x{HIRES_SHAPE[1]}x{HIRES_SHAPE[2]}, "
                         f"{HIRES_NFREQ} harmonics of 1/(16 yr), {HIRES_NREALS} realizations, {NLOUD} loudest"),
            "value": HIRES_NREALS / sec, "unit": UNIT, "seconds_per_evaluation": sec, "evaluations": len(times),
            "draws_per_s": nb * HIRES_NFREQ * HIRES_NREALS / sec,
            "peak_device_memory_gb": torch.cuda.max_memory_allocated() / 1e9,
            "mean_total_hc2_vs_expectation": {"z_min": float(z.min()), "z_median": float(np.median(z)),
                                              "z_max": float(z.max()),
                                              "rel_median": float(np.median(np.abs(total.mean(1) / s1 - 1.0)))}}


def run_mlp_profile(args):
    """The emulator network's kernels at a fixed size, untimed (the program the MLP ncu captures run):
    a 4-member 16 -> 4x256 -> 160 ensemble, one forward of 1024 queries, then one training step
    (forward, backward, AdamW) on a batch of 512."""
    import torch
    from holodeck_gb300.emulator import MLPEnsemble
    net = MLPEnsemble([16, 256, 256, 256, 256, 160], members=4, seed=0)
    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.uniform(-1, 1, size=(1024, 16)).astype(np.float32), device="cuda").to(torch.bfloat16)
    for _ in range(args.warmup + 1):
        net.forward(x)
    t = torch.as_tensor(rng.normal(size=(512, 160)).astype(np.float32), device="cuda")
    net.train_step(x[:512].contiguous(), t, lr=1e-3)
    torch.cuda.synchronize()
    net.check_status()
    print(json.dumps({"profile": "emulator MLP 16-4x256-160, 4 members", "forward_batch": 1024, "train_batch": 512}))


def run_stages(args):
    """Device time of each stage of one model evaluation (CUDA events on the current stream), median
    over ``--steps`` evaluations after ``--warmup``: the breakdown behind the headline number.  The
    hardening normalisation starts on a side stream when the hardening model is built and overlaps
    the density; hardening_norm_wait is what is left of it afterwards."""
    import torch
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    from holodeck_gb300 import single_sources
    _, fe = H.utils.pta_freqs(16.0 * C.YR, NFREQ)
    fo_c = H.utils.midpoints(fe) / 2.0
    names = ["density_and_scatter", "hardening_norm_wait", "dbn", "number_and_strain", "sort", "realizations"]
    rows = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
        ev[0].record()
        sam, hard = make_model(H, C)
        sam._density_device()
        ev[1].record()
        hard._norm_device()
        ev[2].record()
        redz_final, diff_num = sam._dbn_device(hard, fo_c, precision=args.precision)
        ev[3].record()
        number, h2fdf = sam._number_and_strain(fe / 2.0, diff_num, redz_final, precision=args.precision)
        ev[4].record()
        order = single_sources.sort_order_device(h2fdf)
        ev[5].record()
        single_sources.ss_realize_device(number, h2fdf, NREALS, NLOUD, seed=i, order=order)
        ev[6].record()
        torch.cuda.synchronize()
        if i >= args.warmup:
            rows.append([ev[k].elapsed_time(ev[k + 1]) for k in range(len(names))])
    med = [statistics.median(r[k] for r in rows) for k in range(len(names))]
    print(json.dumps({"stages_ms": dict(zip(names, [round(m, 3) for m in med])), "sum_ms": round(sum(med), 3),
                      "config": {"workload": CONFIG_NAME, "precision": args.precision}, "evaluations": args.steps}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"],
                    help="grid arithmetic of the timed steps (fp32: the production mode; fp64: the parity mode)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true", help="run warmup + 1 untimed evaluations (for ncu)")
    ap.add_argument("--nfreqs", type=int, default=NFREQ, help="frequencies of a --profile run")
    ap.add_argument("--stages", action="store_true", help="per-stage device times of one model evaluation")
    ap.add_argument("--batched-samples", type=int, default=512,
                    help="library samples of the batched measurement carried by the bench line (0: skip)")
    ap.add_argument("--batched", action="store_true", help="only the batched-library measurement")
    ap.add_argument("--emulator-samples", type=int, default=2048,
                    help="training samples of the emulator measurement carried by the bench line (0: skip)")
    ap.add_argument("--emulator-steps", type=int, default=6000, help="emulator training steps (batch 512)")
    ap.add_argument("--emulator", action="store_true", help="only the emulator measurement")
    ap.add_argument("--mlp-profile", action="store_true", help="untimed emulator-network kernels (for ncu)")
    ap.add_argument("--highres-steps", type=int, default=1,
                    help="timed evaluations of the high-resolution measurement carried by the bench line (0: skip)")
    ap.add_argument("--highres", action="store_true",
                    help="only the high-resolution workload (181x161x201, 100 frequencies, 10^4 realizations)")
    ap.add_argument("--emulator-cache", default=None,
                    help=".npz holding the emulator's training library statistics (written when absent)")
    args = ap.parse_args()
    if args.batched and args.impl != "reference":
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps({"metric": METRIC, "batched": run_batched(args)}))
    elif args.emulator and args.impl != "reference":
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps({"metric": METRIC, "emulator": run_emulator(args)}))
    elif args.highres:
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps({"metric": METRIC, "highres": run_highres(args)}))
    elif args.mlp_profile:
        run_mlp_profile(args)
    elif args.profile:
        run_profile(args)
    elif args.stages:
        run_stages(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
