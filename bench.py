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


# ---- algorithmic cost of the realization stage, in thread instructions, declared from the
# algorithms (not measured); the issue roofline is draws/s against (issue peak / ops per draw)
OPS_UNIFORM = 10                 # Philox4x32-10: 10 rounds x (2 wide multiplies + 2 three-input XORs) / 4 words
OPS_ACCUM = 5                    # count to float, times strain, Kahan add
OPS_ALIAS = OPS_UNIFORM + 4 + OPS_ACCUM          # 0.1 <= lambda < 10: column, row word, compare, select
OPS_TABLE = OPS_UNIFORM + 5 + OPS_ACCUM          # 10 <= lambda <= 47000: guide cell, flags, one compare
OPS_TABLE_ENTRY = 4              # per table entry and realization group: recursion, to fixed point, prefix, store
OPS_PTRS_ATTEMPT = 2 * OPS_UNIFORM + 25          # lambda > 47000: one transformed-rejection attempt
PTRS_ATTEMPTS = 1.15             # expected attempts per draw (Hormann 1993)
OPS_SPARSE_EVENT = 2 * OPS_UNIFORM + 6 + 5 + OPS_ACCUM   # lambda < 0.1, per event: gap, zero-truncated count
OPS_STAGE = 10                   # per bin and frequency per realization group: load, classify


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except OSError:
        return {}


def realization_roofline(number, nreals, t_launch, n_sm, sm_mhz, waves):
    """The realization kernel (k_bulk) against its issue roofline: every SM sub-partition issues one
    warp instruction (32 thread instructions) per clock, and the workload needs ops_per_draw thread
    instructions per (bin, frequency, realization) draw by the declared costs above, weighted by the
    expectation histogram of this model.  The HBM view (algorithmic bytes over the launch time) is
    kept as a sub-object; the kernel is not HBM-bound."""
    import torch
    lam = number.reshape(-1)
    groups = -(-nreals // 1024)
    sparse = (lam > 0) & (lam < 0.1)
    alias = (lam >= 0.1) & (lam < 10.0)
    table = (lam >= 10.0) & (lam <= 47000.0)
    ptrs = lam > 47000.0
    lt = lam[table]
    sd = torch.sqrt(lt)
    entries = float((torch.ceil(lt + 7.0 * sd + 6.0) - torch.clamp(torch.floor(lt - 7.0 * sd - 2.0), min=0.0)
                     + 1.0).sum().item())
    n_alias, n_table, n_ptrs = (int(m.sum().item()) for m in (alias, table, ptrs))
    sparse_events = float(lam[sparse].sum().item())
    ops = (nreals * (OPS_ALIAS * n_alias + OPS_TABLE * n_table + (OPS_PTRS_ATTEMPT * PTRS_ATTEMPTS + OPS_ACCUM) * n_ptrs)
           + OPS_SPARSE_EVENT * nreals * sparse_events + OPS_TABLE_ENTRY * groups * entries
           + OPS_STAGE * groups * lam.numel())
    draws = lam.numel() * nreals
    ops_per_draw = ops / draws
    issue_peak = n_sm * 4 * 32 * sm_mhz * 1e6          # thread instructions / s
    achieved = draws / t_launch
    peak = issue_peak / ops_per_draw
    # HBM view: every bin's expectation and the strain of the bins with a nonzero one (8 B each) per
    # realization group, each realization's first bulk position, the per-chunk partial sums
    nf = int(number.shape[-1])
    nb = lam.numel() // nf
    nchunk = max(1, -(-n_sm * 6 * waves // (nf * groups)))
    n_pos = int((lam > 0).sum().item())
    alg_bytes = (8 * nb * nf + 8 * n_pos) * groups + 4 * nf * nreals + 8 * nchunk * nf * nreals
    hbm_peak = float(_peaks().get("hbm_gbs", 6800.0))
    hbm = alg_bytes / t_launch / 1e9
    n = lam.numel()
    return {"kernel": "k_bulk", "bound": "issue", "unit": "draws/s", "achieved": achieved, "peak": peak,
            "frac": achieved / peak, "launch_s": t_launch, "ops_per_draw": ops_per_draw,
            "peak_issue_thread_instructions_per_s": issue_peak, "sm_mhz_for_peak": sm_mhz,
            "draw_regimes": {"zero": int((lam <= 0).sum().item()) / n, "sparse_lt_0.1": int(sparse.sum().item()) / n,
                             "alias_lt_10": n_alias / n, "table_le_47000": n_table / n, "ptrs_gt_47000": n_ptrs / n,
                             "sparse_events_per_draw": sparse_events / n,
                             "table_entries_per_bin_frequency": entries / n},
            "traffic": 357620480,
            "traffic_source": ("DRAM bytes read + written by one k_bulk launch of this workload, one ncu capture "
                               "(profiles/k_bulk_91x81x101_f4_r1000.md)"),
            "hbm": {"achieved": hbm, "peak": hbm_peak, "unit": "GB/s", "frac": hbm / hbm_peak,
                    "algorithmic_bytes": alg_bytes},
            "note": ("ops_per_draw from the costs declared in bench.py (OPS_*), weighted by this model's "
                     "expectation histogram; the HBM floor of the launch is far below its time")}


# per-element FP64 lane operations of the grid stages with a fixed per-element cost (additions and
# multiplications are separate instructions: the parity mode is built without fused multiply-add)
FP64_OPS_CELLS = {"fp64": 45, "fp32": 0}   # per (bin, frequency): 8-vertex sum and scale 11, midpoints 14,
                                           # distance 12, (1+z)^(2/3) 2, strain product 6; FP32 mode: FP32
                                           # arithmetic (FP64 only in sentinel-mixed midpoints)
FP64_OPS_EVAL = {"fp64": 27, "fp32": 7}    # per bracketed element: redshift / distance interpolation 5, the
                                           # rest of the residence time 22; FP32 mode: interpolation and the
                                           # density products only


def grid_stage_rooflines(H, C, fe, precision, n_sm, sm_mhz):
    """One more model evaluation, stage by stage on one stream with CUDA events: the device time of
    each grid stage, and for the dbn evaluation and number + strain stages (fixed per-element work)
    their algorithmic FP64 and HBM fractions."""
    import torch
    from holodeck_gb300 import single_sources
    from holodeck_gb300.sams import sam_cyutils
    fp64_peak = 2.0 * n_sm * sm_mhz * 1e6   # FP64 lane operations / s (two per clock per SM)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(8)]
    ev[0].record()
    sam, hard = make_model(H, C)
    torch.cuda.current_stream().wait_event(hard._norm_ready)   # the normalisation runs on a side stream
    ev[1].record()
    dens, gmt_time, redz_prime = sam._static_density_launch()
    ev[2].record()
    sam._scatter_finish(dens, gmt_time, redz_prime)
    ev[3].record()
    mt, mr, rz = sam._edges_device()
    fo_c = H.utils.midpoints(fe) / 2.0
    rf, dn = sam_cyutils.dbn_2pwl_device(fo_c, hard, None, mt, mr, rz, gmt_time, phase=1)
    ev[4].record()
    rf, dn = sam_cyutils.dbn_2pwl_device(fo_c, hard, dens, mt, mr, rz, gmt_time, phase=2, out=(rf, dn),
                                         precision=precision)
    ev[5].record()
    number, h2fdf = sam._number_and_strain(fe / 2.0, dn, rf, precision=precision)
    ev[6].record()
    single_sources.sort_order_device(h2fdf)
    ev[7].record()
    torch.cuda.synchronize()
    ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(7)]
    nm, nq, nz = sam.shape
    nf = int(number.shape[-1])
    n_vf = nm * nq * nz * nf
    n_bf = int(number.numel())
    n_brk = int((rf >= 0).sum().item())
    bytes_eval = 32 * n_brk + 8 * nm * nq * nz    # hint + time in, redshift + number out; the density
    bytes_cells = 16 * n_vf + 16 * n_bf           # vertices in (each once from DRAM), number + strain out
    hbm_peak = float(_peaks().get("hbm_gbs", 6800.0)) * 1e9

    def fr(ops, nbytes, t_ms):
        return {"ms": t_ms, "fp64_ops": ops, "fp64_frac": ops / (t_ms * 1e-3) / fp64_peak,
                "hbm_bytes": nbytes, "hbm_frac": nbytes / (t_ms * 1e-3) / hbm_peak}

    return {"precision": precision,
            "stages_ms": {"model_build_and_hardening_norm": ms[0], "static_density": ms[1], "mbulge_scatter": ms[2],
                          "dbn_step_walk": ms[3], "dbn_evaluation": ms[4], "number_and_strain": ms[5], "sort": ms[6]},
            "dbn_evaluation": fr(FP64_OPS_EVAL[precision] * n_brk, bytes_eval, ms[4]),
            "number_and_strain": fr(FP64_OPS_CELLS[precision] * n_bf, bytes_cells, ms[5]),
            "fp64_peak_lane_ops_per_s": fp64_peak,
            "note": ("stages run one after another here (gwb() overlaps the normalisation and the step walk with "
                     "the density and scatter); FP64 ops per element declared in bench.py (FP64_OPS_*); the "
                     "FP64-pipe utilisation of the iterative grid kernels is in profiles/")}


def emit(args, obj):
    """Print one result line (the bench contract) and, with --json-out, append it to that file."""
    text = json.dumps(obj)
    print(text, flush=True)
    if getattr(args, "json_out", None):
        with open(args.json_out, "a") as fh:
            fh.write(text + "\n")


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
    rf, dn = sam._dbn_device(hard, fo_c, precision=args.precision)
    number, h2fdf = sam._number_and_strain(fe / 2.0, dn, rf, precision=args.precision)
    del rf, dn
    order = single_sources.sort_order_device(h2fdf)
    from holodeck_gb300 import cyutils
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
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = (clk or {}).get("sm_max_mhz") or 2070.0
    roofline = realization_roofline(number, NREALS, t_real, n_sm, sm_mhz, lib.hgb_get_bulk_waves())
    del number, h2fdf, order
    grid_stages = grid_stage_rooflines(H, C, fe, args.precision, n_sm, sm_mhz)

    batched = run_batched(args, rank, world) if args.batched_samples > 0 else None
    # the single-GPU legs (high-resolution model, emulator) run at N = 1 only: under torchrun the
    # other GPUs would wait idle for them
    highres = None
    if args.highres_steps > 0 and world == 1:
        hargs = argparse.Namespace(**vars(args))
        hargs.steps = args.highres_steps
        highres = run_highres(hargs)
        torch.cuda.empty_cache()
    emulator = run_emulator(args) if (args.emulator_samples > 0 and world == 1) else None
    cpu = hc_error = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, keep = cpu_baseline_sample(args)
        hc_error = hc_error_vs_reference(keep, args.precision)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": ("f64 grids / f32+int32 realizations" if args.precision == "fp64" else
                      "f32 grid arithmetic (f64 density, hardening integral, age->redshift inversion) / "
                      "f32+int32 realizations"),
            "data": "synthetic (analytic model parameters; no dataset)",
            "config": {"workload": CONFIG_NAME, "grid": list(SHAPE), "nfreqs": NFREQ, "nreals": NREALS,
                       "nloudest": NLOUD, "precision": args.precision, "rng": "philox4x32-10",
                       "l2": "flushed (256 MB write) before every step",
                       "parallelism": f"replicas x{world}",
                       "note": "scatter geometry plan cached per grid; every other stage recomputed each step"},
            "e2e": {"value": world * NREALS / (e2e_ms / 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": roofline,
            "grid_stages": grid_stages,
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
        emit(args, line)
    if world > 1:
        dist.destroy_process_group()


DEVICE_BATCH = 16
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
                            indices=batch.shard_indices(n, rank, world), stats=stats, precision=args.precision)
    job = batch.reduce_stats(stats)                       # max wall time, summed work over the replicas
    wall, reals, draws = job["seconds"], job["realizations"], job["draws"]
    # the same library with the realizations of DEVICE_BATCH samples per kernel launch, on the
    # schedule found above (the results are identical; only the wall time is compared)
    dstats = {}
    batch.run_library(space, shapes, nreals, nfreqs=NFREQ, nloudest=NLOUD, seed=1,
                      indices=batch.shard_indices(n, rank, world), stats=dstats, precision=args.precision,
                      workers=stats["workers"], waves=stats["waves"], tune=False, batch=DEVICE_BATCH,
                      reduce=lambda r: None)
    djob = batch.reduce_stats(dstats)
    d2h = sum(sum(v.nbytes for k, v in r.items() if isinstance(v, np.ndarray)) for r in out if r is not None)
    tuning = stats.get("tuning") or {}
    table = tuning.get("table", {})
    ones = [v for k, v in table.items() if k.split(",")[0] == "1"]
    one = max(ones) if ones else None
    best = table.get(f"{stats['workers']},{stats['waves']}")
    return {"workload": BATCH_CONFIG, "precision": args.precision, "samples": n, "failed": job["failed"], "seconds": wall,
            "value": reals / wall, "unit": UNIT, "samples_per_s": n / wall, "draws_per_s": draws / wall,
            "realizations": int(reals), "schedule": {"workers": stats["workers"], "waves": stats["waves"]},
            "autotune_draws_per_s": table,
            "speedup_vs_one_worker_in_probe": (best / one) if (best and one) else None,
            "e2e": "host parameters in, host hc_ss / hc_bg out; per-sample scatter plans built on the host "
                   "inside the timed region", "d2h_bytes": int(d2h),
            "errors": dict(list(stats.get("errors", {}).items())[:3]),
            "device_batched": {"batch": DEVICE_BATCH, "blocks_per_sm": 0, "seconds": djob["seconds"],
                               "draws_per_s": djob["draws"] / djob["seconds"], "failed": djob["failed"],
                               "note": "realizations of up to batch samples per k_bulk_multi launch (one block "
                                       "per work item), grid stages on the same worker pool"}}


NOISE_SAMPLES = 512
EMU_CONFIG = ("learned emulator: 4-member ensemble of MLPs 6 -> 4x256 (SiLU) -> 40 x (5/50/95th percentile "
              "log10 hc, median log10 loudest-source hc), bf16 weights and activations, fp32 accumulation on "
              "tcgen05, AdamW; trained on 20,000 Latin-hypercube samples (seed 0) of PS_Classic_Phenom_Uniform "
              "at the 91x81x101 grid with 500 realizations (FP32 production mode), tested on 2,000 held-out "
              "samples (seed 1); single queries through the one-launch fused forward")


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
    n_bd = args.emulator_boundary_samples
    sp_bd = EM.boundary_space(PS_Classic_Phenom_Uniform, n_bd, seed=2) if n_bd > 0 else None
    lib_stats = {}
    cache = args.emulator_cache
    if cache and os.path.exists(cache):
        with np.load(cache) as z:
            assert np.array_equal(z["params_train"], sp_tr.param_samples), "cache holds another library"
            y_tr, y_te, y_te2 = z["y_train"], z["y_test"], z["y_test2"]
            lib_stats["seconds"] = float(z["library_seconds"])
            cached = {kk: z[kk] for kk in z.files}
        if sp_bd is None:
            y_bd, bd_seconds = np.zeros((0,) + y_tr.shape[1:]), 0.0
        elif "y_boundary" in cached and np.array_equal(cached.get("params_boundary"), sp_bd.param_samples):
            y_bd, bd_seconds = cached["y_boundary"], float(cached["boundary_seconds"])
        else:
            bd_stats = {}
            y_bd = EM.training_library(sp_bd, seed=6, stats=bd_stats, precision=args.precision)
            bd_seconds = bd_stats["seconds"]
            np.savez(cache, **dict(cached, params_boundary=sp_bd.param_samples, y_boundary=y_bd,
                                   boundary_seconds=bd_seconds))
    else:
        y_tr = EM.training_library(sp_tr, seed=2, stats=lib_stats, precision=args.precision)
        y_te = EM.training_library(sp_te, seed=3, precision=args.precision)
        # the first NOISE_SAMPLES held-out models again with other realizations: the noise floor
        y_te2 = EM.training_library(sp_te, seed=4, precision=args.precision,
                                    indices=list(range(min(NOISE_SAMPLES, n_te))))
        y_bd, bd_seconds, extra = np.zeros((0,) + y_tr.shape[1:]), 0.0, {}
        if sp_bd is not None:
            bd_stats = {}
            y_bd = EM.training_library(sp_bd, seed=6, stats=bd_stats, precision=args.precision)
            bd_seconds = bd_stats["seconds"]
            extra = dict(params_boundary=sp_bd.param_samples, y_boundary=y_bd, boundary_seconds=bd_seconds)
        if cache:
            np.savez(cache, params_train=sp_tr.param_samples, params_test=sp_te.param_samples, y_train=y_tr,
                     y_test=y_te, y_test2=y_te2, library_seconds=lib_stats["seconds"], **extra)
    # the training set: the Latin hypercube, plus any points on the box's faces
    x_bd = sp_bd.param_samples if sp_bd is not None else np.zeros((0, sp_tr.param_samples.shape[1]))
    x_fit = np.concatenate([sp_tr.param_samples, x_bd])
    y_fit = np.concatenate([y_tr, y_bd])
    ok_fit = np.all(np.isfinite(y_fit), axis=(1, 2))
    ok = np.all(np.isfinite(y_tr), axis=(1, 2))
    emu = EM.Emulator(sp_tr, nfreqs=NFREQ, members=args.emulator_members, width=256, depth=4, seed=0)
    steps_per_epoch = max(1, int(ok_fit.sum()) // 512)
    epochs = max(50, -(-args.emulator_steps // steps_per_epoch))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = emu.fit(x_fit[ok_fit], y_fit[ok_fit], epochs=epochs, batch=512, lr=2e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    mean, spread, inside = emu.predict(sp_te.param_samples)
    spread_p50 = emu.predict(sp_te.param_samples, spread_stats=("log10_hc_p50",))[1]
    spread_hc = emu.predict(sp_te.param_samples, spread_stats=("log10_hc_p05", "log10_hc_p50", "log10_hc_p95"))[1]
    spread_rs = emu.predict(sp_te.param_samples, residual_scaled=True)[1]
    criteria = (("all_outputs", spread), ("hc_percentiles", spread_hc), ("median_hc", spread_p50),
                ("residual_scaled", spread_rs))
    good = np.all(np.isfinite(y_te), axis=(1, 2))
    err = np.abs(mean - y_te)[good]
    u_tr, u_te = emu.unit(sp_tr.param_samples[ok]), emu.unit(sp_te.param_samples)
    nn = np.array([np.argmin(((u_tr - u) ** 2).sum(-1)) for u in u_te])
    err_nn = np.abs(y_tr[ok][nn] - y_te)[good]
    n2 = len(y_te2)
    good2 = good[:n2] & np.all(np.isfinite(y_te2), axis=(1, 2))
    noise = np.abs(y_te[:n2] - y_te2)[good2] / np.sqrt(2.0)
    g1, gb = emu.graphed(1), emu.graphed(1024)
    q1 = sp_te.param_samples[:1]
    qb = np.resize(sp_te.param_samples, (1024, sp_te.param_samples.shape[1]))
    t_q1_graph = EM.timed(g1, q1, repeat=200)
    t_q1 = EM.timed(emu.native(1), q1, repeat=500)
    t_q1_tc = EM.timed(emu.graphed(1, fused=False), q1, repeat=200)
    # the fused kernel alone: 200 launches back to back between CUDA events (weights L2-resident)
    x1 = emu.inputs(q1)
    for _ in range(20):
        emu.net.forward_fused(x1)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(200):
        emu.net.forward_fused(x1)
    ev1.record()
    torch.cuda.synchronize()
    emu.net.check_status()
    t_fused_kernel = ev0.elapsed_time(ev1) / 200 * 1e-3
    t_qb = EM.timed(gb, qb, repeat=20)
    solve = EM.sam_fallback(sp_tr, sam_shape=SHAPE, nreals=500, nfreqs=NFREQ, seed=5, precision=args.precision)
    t_plain = EM.timed(solve, q1[0], repeat=3)
    names = list(EM.STATS)

    def med(a):
        return {nm: float(np.median(a[..., k])) for k, nm in enumerate(names)}

    return {"workload": EMU_CONFIG.replace("4-member", f"{args.emulator_members}-member"),
            "train_samples": int(ok.sum()), "boundary_samples": int(ok_fit.sum() - ok.sum()),
            "test_samples": int(good.sum()),
            "library_seconds": lib_stats.get("seconds"), "library_samples_per_s": n_tr / lib_stats["seconds"],
            "boundary_library_seconds": bd_seconds,
            "train_seconds": t_train, "train_steps": epochs * steps_per_epoch, "final_loss": hist[-1],
            "median_abs_dlog10": med(err), "p95_abs_dlog10": {nm: float(np.percentile(err[..., k], 95))
                                                             for k, nm in enumerate(names)},
            "nearest_sample_median_abs_dlog10": med(err_nn), "realization_noise_median_dlog10": med(noise),
            "ensemble_spread_median_dex": float(np.median(spread)),
            "flagged_fraction_at_0.05dex": float(np.mean(spread > 0.05)),
            "flagged_fraction_at_0.05dex_by_criterion": {nm: float(np.mean(sv > 0.05)) for nm, sv in criteria},
            "accepted_median_abs_dlog10_by_criterion": {
                nm: med(np.abs(mean - y_te)[good & (sv <= 0.05)]) for nm, sv in criteria},
            "training_residual_scatter_median_dex": float(np.median(emu.residual_scatter)),
            "query_s_batch1": t_q1, "query_s_batch1_paths": {
                "native (one hgb_emulator_query call)": t_q1, "graph, fused kernel, pinned I/O": t_q1_graph,
                "graph, tensor-core layers and copy nodes": t_q1_tc},
            "query_s_batch1_tensor_core_layers": t_q1_tc,
            "fused_kernel_s_back_to_back": t_fused_kernel,
            "query_s_per_sample_batch1024": t_qb / 1024,
            "plain_gpu_sam_s": t_plain, "speedup_vs_plain_batch1": t_plain / t_q1,
            "speedup_vs_plain_batch1_with_fallbacks": {
                "target": 100.0,
                **{nm: t_plain / (t_q1 + float(np.mean(sv > 0.05)) * t_plain) for nm, sv in criteria}},
            "criteria": "a query falls back to the plain GPU SAM when the 4 members' standard deviation of any "
                        "output exceeds 0.05 dex: over all outputs, over the hc percentiles, over the median hc; "
                        "residual_scaled: all outputs, each against max(0.05 dex, that output's training-residual "
                        "scatter, the emulator's typical error over its training library)",
            "speedup_vs_plain_batch1024": t_plain / (t_qb / 1024)}


# ------------------------------------------------------------------------------------------------
# The reference on the host cores: its compiled Cython kernels (oracle/ref_build.py) driven by the
# oracle's restatement of its Python glue (oracle/ref_stub.py), on bounded samples
# ------------------------------------------------------------------------------------------------

SAMPLE_Z = 11   # the GPU line's single-core sample: the 91 x 81 x 11 grid
SAMPLE_R = 3    # realizations drawn per sample (the rest is extrapolated linearly in R)
REF_SAMPLE_R = 3


def _ref_per_model(t, nreals_sampled, zscale=1.0):
    """Seconds of one full model (the 91 x 81 x 101 grid, NREALS realizations) from the stage
    seconds of a sample: the redshift-sliced stages scale with the redshift bins (zscale), the
    hardening normalisation does not, realizations scale with bins and count."""
    grid = zscale * sum(v for k, v in t.items() if k not in ("hardening_norm", "realizations"))
    grid += t["hardening_norm"]
    per_real = zscale * t["realizations"] / nreals_sampled
    return grid + NREALS * per_real, grid, per_real


def cpu_baseline_sample(args):
    """The reference's path on one host core on the 91 x 81 x 11 sample (about 10 s), extrapolated
    to the bench workload; also keeps the sample's FP64 grids for the hc error of the GPU path."""
    from oracle import ref_stub
    keep = {}
    t = ref_stub.reference_gwb_stages((SHAPE[0], SHAPE[1], SAMPLE_Z), NFREQ, SAMPLE_R, NLOUD, seed=7, keep=keep)
    total, grid, per_real = _ref_per_model(t, SAMPLE_R, zscale=(SHAPE[2] - 1) / (SAMPLE_Z - 1))
    return {"value": NREALS / total, "unit": UNIT, "cores": 1, "kind": "reference",
            "sample": (f"the reference's compiled Cython kernels (cyutils.pyx, sam_cyutils.pyx built from its "
                       f"sources) with the oracle's restatement of its Python glue, one process, on grid "
                       f"91x81x{SAMPLE_Z} with {SAMPLE_R} realizations, extrapolated linearly in redshift bins and "
                       f"realizations: grid stages {grid:.1f} s + {per_real:.2f} s/realization "
                       f"({', '.join(f'{k} {v:.2f}s' for k, v in t.items())})")}, keep


def hc_error_vs_reference(keep, precision, nreals=8):
    """The GPU path (in ``precision``) against the reference's FP64 kernels on the CPU baseline's
    sample model (the bench model on the 91 x 81 x 11 grid, 40 frequencies): numpy-PCG64 Poisson
    counts drawn from the reference's expectations and replayed in its visiting order through the
    public gwb(); relative errors of hc_ss and hc_bg (max, and per frequency), of the expected hc^2
    sum_b number h2fdf per frequency, and of the number and strain grids."""
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    from oracle import sam_oracle as O
    sam, hard = make_model(H, C, shape=tuple(len(e) for e in keep["edges"]), edges=keep["edges"])
    fe = keep["fobs_gw_edges"]
    counts = O.replay_counts(keep["number"], keep["order"], nreals, 11)
    ss_o, bg_o = O.ss_gws_redz(keep["edges"] + [fe / 2.0], keep["redz_final"], keep["number"], nreals, NLOUD,
                               counts=counts)
    ss, bg = sam.gwb(fe, hard=hard, realize=nreals, loudest=NLOUD, replay=counts, order=keep["order"],
                     precision=precision)
    rf, dn = sam._dbn_device(hard, O.midpoints(fe) / 2.0, precision=precision)
    number, h2fdf = sam._number_and_strain(fe / 2.0, dn, rf, precision=precision)
    number, h2fdf = number.cpu().numpy(), h2fdf.cpu().numpy()
    nf = number.shape[-1]
    mean_o = (keep["number"] * keep["h2fdf"]).reshape(-1, nf).sum(0)
    mean_g = (number * h2fdf).reshape(-1, nf).sum(0)

    def rel(a, b):
        a, b = np.asarray(a), np.asarray(b)
        scale = np.maximum(np.abs(a), np.abs(b))
        m = scale > 0
        return float((np.abs(a - b)[m] / scale[m]).max()) if m.any() else 0.0

    def sig_rel(a, b, floor=1e-25):   # over values that can reach the strain (FP32 flushes below FLT_MIN)
        a, b = np.asarray(a), np.asarray(b)
        m = np.abs(b) > floor * np.abs(b).max()
        return float((np.abs(a[m] - b[m]) / np.abs(b[m])).max())

    return {"case": (f"bench model on the 91x81x{SAMPLE_Z} grid, {NFREQ} frequencies, {nreals} realizations replayed "
                     f"from numpy PCG64 Poisson draws, GPU path in {precision} against the reference's FP64 kernels"),
            "precision": precision,
            "hc_ss_max_rel": rel(ss, ss_o), "hc_bg_max_rel": rel(bg, bg_o),
            "hc_ss_max_rel_per_freq": [rel(ss[f], ss_o[f]) for f in range(nf)],
            "hc_bg_max_rel_per_freq": [rel(bg[f], bg_o[f]) for f in range(nf)],
            "mean_hc2_rel_per_freq": [float(abs(mean_g[f] / mean_o[f] - 1.0)) for f in range(nf)],
            "number_max_rel": sig_rel(number, keep["number"]), "h2fdf_max_rel": sig_rel(h2fdf, keep["h2fdf"])}


def _ref_worker(seed):
    from oracle import ref_stub
    return ref_stub.reference_gwb_stages(SHAPE, NFREQ, REF_SAMPLE_R, NLOUD, seed=seed)


def run_reference(args):
    """Reference arm: the reference's path (its compiled Cython kernels with the oracle's restatement of
    its Python glue) on every host core, each worker one evaluation of the full 91 x 81 x 101 grid with
    REF_SAMPLE_R realizations, extrapolated linearly in the realization count.  The reference is
    serial, so the cores run independent model evaluations, as its MPI library driver does."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import ref_build
    if not ref_build.generated():
        print(json.dumps({"impl": "reference", "unavailable": "the reference's Cython kernels were not generated "
                          "(oracle/ref_build.py generate needs the reference sources and Cython)"}))
        return
    ref_build.compile()
    ncores = os.cpu_count() or 1
    nsamples = args.warmup + args.steps
    nproc = min(ncores, nsamples)
    ctx = mp.get_context("spawn")
    t_wall = time.perf_counter()
    with ctx.Pool(nproc) as pool:
        res = pool.map(_ref_worker, [1000 + k for k in range(nsamples)], chunksize=1)
    t_wall = time.perf_counter() - t_wall
    timed = res[args.warmup:]
    per_model = [_ref_per_model(t, REF_SAMPLE_R)[0] for t in timed]
    sec = statistics.median(per_model)   # one core's seconds per full model, measured with every core busy
    value = nproc * NREALS / sec
    stages = {k: round(statistics.median(t[k] for t in timed), 3) for k in timed[0]}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_wall * 1e3 / nsamples,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": CONFIG_NAME, "grid": list(SHAPE), "nfreqs": NFREQ, "nreals": NREALS,
                       "nloudest": NLOUD},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nproc, "kind": "reference",
                             "sample": (f"{nproc} processes, each step one evaluation of the full 91x81x101 grid "
                                        f"through the reference's compiled Cython kernels (cyutils.pyx, "
                                        f"sam_cyutils.pyx, built from its sources) and the oracle's restatement of "
                                        f"its Python glue, with {REF_SAMPLE_R} realizations, extrapolated linearly "
                                        f"in the realization count; {nsamples} evaluations in {t_wall:.0f} s"),
                             "stage_seconds_median": stages,
                             "seconds_per_model_one_core": sec,
                             "note": ("ms_per_step is the wall time per sampled evaluation with every core busy; "
                                      "value extrapolates each sample to the workload's 1000 realizations")},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    emit(args, line)


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
    (forward, backward, AdamW) on a batch of 512, then the fused forward of single queries
    (``--warmup`` + 1 launches)."""
    import torch
    from holodeck_gb300.emulator import MLPEnsemble
    net = MLPEnsemble([16, 256, 256, 256, 256, 160], members=4, seed=0)
    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.uniform(-1, 1, size=(1024, 16)).astype(np.float32), device="cuda").to(torch.bfloat16)
    for _ in range(args.warmup + 1):
        net.forward(x)
    t = torch.as_tensor(rng.normal(size=(512, 160)).astype(np.float32), device="cuda")
    net.train_step(x[:512].contiguous(), t, lr=1e-3)
    for _ in range(args.warmup + 1):
        net.forward_fused(x[:1].contiguous())
    torch.cuda.synchronize()
    net.check_status()
    print(json.dumps({"profile": "emulator MLP 16-4x256-160, 4 members", "forward_batch": 1024, "train_batch": 512,
                      "fused_forward_batch": 1}))


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
    ap.add_argument("--emulator-samples", type=int, default=20000,
                    help="training samples of the emulator measurement carried by the bench line (0: skip)")
    ap.add_argument("--emulator-steps", type=int, default=60000, help="emulator training steps (batch 512)")
    ap.add_argument("--emulator-members", type=int, default=4, help="ensemble members of the emulator")
    ap.add_argument("--emulator-boundary-samples", type=int, default=0,
                    help="training points on the faces of the parameter box, added to the Latin hypercube")
    ap.add_argument("--emulator", action="store_true", help="only the emulator measurement")
    ap.add_argument("--mlp-profile", action="store_true", help="untimed emulator-network kernels (for ncu)")
    ap.add_argument("--highres-steps", type=int, default=1,
                    help="timed evaluations of the high-resolution measurement carried by the bench line (0: skip)")
    ap.add_argument("--highres", action="store_true",
                    help="only the high-resolution workload (181x161x201, 100 frequencies, 10^4 realizations)")
    ap.add_argument("--json-out", default=None, help="also append each result line to this file")
    ap.add_argument("--emulator-cache", default=None,
                    help=".npz holding the emulator's training library statistics (written when absent)")
    args = ap.parse_args()
    if args.batched and args.impl != "reference":
        import torch
        torch.cuda.set_device(dist_env()[2])
        emit(args, {"metric": METRIC, "batched": run_batched(args)})
    elif args.emulator and args.impl != "reference":
        import torch
        torch.cuda.set_device(dist_env()[2])
        emit(args, {"metric": METRIC, "emulator": run_emulator(args)})
    elif args.highres:
        import torch
        torch.cuda.set_device(dist_env()[2])
        emit(args, {"metric": METRIC, "highres": run_highres(args)})
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
