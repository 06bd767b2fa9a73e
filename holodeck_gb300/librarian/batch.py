"""Batched library runs on one GPU.

A library is many independent model evaluations: the samples of a parameter space, each on its own
(mtot, mrat, redz) grid shape and with its own realization count (the per-sample work of
librarian/gen_lib.py:run_sam_at_pspace_num, which the reference spreads over MPI ranks).  Here one
process drives one GPU with a pool of host workers.  Each worker owns a CUDA stream (and the side
streams paired with it) and runs whole samples through :func:`lib_tools.run_model`, so the
latency-bound FP64 grid stages of one sample overlap the realization kernels of another, and the
host work of a sample (its scatter-plan geometry, which the native builder computes with the GIL
released) overlaps the device work of the others.  Samples are handed out longest first (their
cost is bins x frequencies x realizations), so the pool drains evenly.

The schedule (number of workers, and the waves of resident blocks the realization kernel's chunk
count aims for) is picked by :func:`autotune`, which times a probe subset of the library at each
candidate and caches the winner per device and workload class in ``_build/tuning.json``.

Every sample's Philox key is derived from the library seed and the sample index alone, and every
draw is keyed by (bin, realization, frequency), so the number of workers and the order in which they
take samples change nothing: a batched run equals one :func:`lib_tools.run_model` call per sample with
the same key, bit for bit.  The waves knob changes how the background sum is grouped into per-chunk
partials, so it moves hc_bg in the last bits only (the draws and the loudest sources are unchanged).
"""

import json
import os
import queue
import threading
import time

import numpy as np

from .. import _device as D
from .. import _native as N
from . import DEF_NUM_FBINS, DEF_NUM_LOUDEST, DEF_PTA_DUR
from .. import single_sources
from .lib_tools import run_model, run_model_grids

_TUNING_PATH = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_build", "tuning.json")
_TUNING_LOCK = threading.Lock()

#: (workers, waves) schedules the autotuner tries
CANDIDATES = ((1, 12), (2, 12), (4, 12), (6, 12), (8, 12), (10, 12), (12, 12), (8, 8), (8, 16))


def sample_seed(seed, index):
    """Philox key of library sample ``index`` (independent of the schedule)."""
    return int(np.random.SeedSequence([int(seed), int(index)]).generate_state(1, np.uint64)[0])


def random_shapes(nsamples, lo=40, hi=91, reals_lo=100, reals_hi=1000, seed=0):
    """Per-sample grid shapes (uniform integers in [lo, hi] per axis) and realization counts
    (uniform integers in [reals_lo, reals_hi]) from ``np.random.default_rng(seed)``."""
    rng = np.random.default_rng(seed)
    shapes = rng.integers(lo, hi + 1, size=(nsamples, 3))
    nreals = rng.integers(reals_lo, reals_hi + 1, size=nsamples)
    return [tuple(int(v) for v in s) for s in shapes], [int(r) for r in nreals]


class Job:
    """One library sample: its index, parameters, grid shape, realization count and Philox key."""

    __slots__ = ("index", "params", "shape", "nreals", "seed")

    def __init__(self, index, params, shape, nreals, seed):
        self.index, self.params, self.shape, self.nreals, self.seed = index, params, shape, nreals, seed

    def cost(self, nfreqs):
        m, q, z = self.shape
        return (m - 1) * (q - 1) * (z - 1) * nfreqs * self.nreals


def make_jobs(space, shapes=None, nreals=None, seed=0, indices=None):
    """Jobs for the samples of ``space`` (all, or ``indices``).  ``shapes`` / ``nreals`` are per-sample
    lists, or one value for every sample (default: the space's ``sam_shape`` and 100 realizations)."""
    n = space.nsamples
    indices = range(n) if indices is None else indices
    jobs = []
    for ii in indices:
        shp = space.sam_shape if shapes is None else (shapes[ii] if np.ndim(shapes) == 2 else shapes)
        if shp is None or np.isscalar(shp):
            shp = (91, 81, 101) if shp is None else (int(shp),) * 3
        nr = 100 if nreals is None else (nreals[ii] if np.ndim(nreals) == 1 else nreals)
        jobs.append(Job(ii, space.param_dict(ii), tuple(int(v) for v in shp), int(nr), sample_seed(seed, ii)))
    return jobs


def shard_indices(nsamples, rank, world):
    """The samples replica ``rank`` of ``world`` runs: round robin, so every sample runs exactly once
    and the replicas' mixes of grid shapes are alike.  Sample keys depend on the index only, so the
    union of the shards equals a one-GPU run."""
    if not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside world of {world}")
    return list(range(rank, int(nsamples), world))


def reduce_stats(stats, device=None):
    """Whole-job view of the ``stats`` of one replica's :func:`run_library` under torch.distributed:
    the longest wall time, and the summed samples, failures, realizations and draws.  Without an
    initialised process group (or with one rank) the stats are returned unchanged."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return dict(stats)
    if device is None:
        device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    longest = torch.tensor([float(stats["seconds"])], dtype=torch.float64, device=device)
    sums = torch.tensor([stats["samples"], stats["failed"], stats["realizations"], stats["draws"]],
                        dtype=torch.float64, device=device)
    dist.all_reduce(longest, op=dist.ReduceOp.MAX)
    dist.all_reduce(sums, op=dist.ReduceOp.SUM)
    out = dict(stats)
    sums = sums.cpu().tolist()
    out.update(seconds=float(longest.item()), samples=int(sums[0]), failed=int(sums[1]), realizations=int(sums[2]),
               draws=float(sums[3]), ranks=dist.get_world_size())
    return out


#: per-sample file name in a library's output directory (librarian/__init__.py:56)
FNAME_LIBRARY_SIM_FILE = "library__p{pnum:06d}.npz"


def sim_fname(output_dir, index):
    """Path of sample ``index``'s file in ``output_dir`` (lib_tools.py:1018-1026)."""
    return os.path.join(str(output_dir), FNAME_LIBRARY_SIM_FILE.format(pnum=int(index)))


def load_sim_file(path):
    """A sample file's contents as a dict, or None when the file records a failure (a 'fail' key) or
    cannot be read; list-valued keys written from lists come back as arrays."""
    try:
        with np.load(path, allow_pickle=False) as z:
            if "fail" in z.files:
                return None
            return {kk: z[kk] for kk in z.files}
    except (OSError, ValueError):
        return None


def _save_sim_file(path, space, job, res, err):
    """Write a sample's result (with its parameters, as gen_lib.py:313-315 adds them) or, for a failed
    sample, a file holding only 'fail' (gen_lib.py:316-323).  The file appears under its final name
    only once complete."""
    if err is not None:
        data = dict(fail=str(err))
    else:
        data = {kk: vv for kk, vv in res.items() if not isinstance(vv, list)}
        for kk, vv in res.items():
            if isinstance(vv, list):
                for ii, arr in enumerate(vv):
                    data[f"{kk}_{ii}"] = arr
        data["params"] = np.array([job.params[pn] for pn in space.param_names])
        data["param_names"] = np.array(space.param_names)
    tmp = path + ".part.npz"
    np.savez(tmp, **data)
    os.replace(tmp, path)


def _run_jobs(space, jobs, workers, nfreqs, nloudest, pta_dur, flags, reduce=None, output_dir=None,
              max_failures=None, batch=0, blocks_per_sm=0):
    """Run ``jobs`` on ``workers`` host threads, one CUDA stream each; returns {index: result or None}
    and {index: exception} for samples that failed.  A result is run_model's dict, or ``reduce`` of it.
    With ``output_dir`` every sample also writes its file there as it finishes.  With ``max_failures``
    the workers stop taking samples once more than that many have failed, and RuntimeError is raised
    (gen_lib.py:213-218).

    ``batch`` > 0 (single-source realizations without parameters only): the workers run each
    sample's grid stages (:func:`lib_tools.run_model_grids`) and hand the finished grids to one
    realization thread, which launches the bulk backgrounds of up to ``batch`` samples at a time as
    one kernel (:func:`single_sources.ss_realize_batch_device`, ``blocks_per_sm`` as there).  The
    results equal run_model's, bit for bit."""
    t = D.torch()
    dev = D.device()
    order = sorted(jobs, key=lambda j: -j.cost(nfreqs))
    q = queue.Queue()
    for job in order:
        q.put(job)
    results, errors = {}, {}
    lock = threading.Lock()
    stop = threading.Event()
    streams = [t.cuda.Stream(device=dev) for _ in range(workers)]
    batched = batch > 0 and flags.get("singles_flag", True) and not flags.get("params_flag", False)
    ready = queue.Queue(maxsize=max(2 * batch, 1)) if batched else None
    _DONE = object()

    def finish(job, res, err):
        if output_dir is not None:
            try:
                _save_sim_file(sim_fname(output_dir, job.index), space, job, res, err)
            except OSError as exc:
                err = err or exc
        value = None
        if err is None:
            try:   # a failing reduce fails its sample, not the thread that runs it
                value = res if reduce is None else reduce(res)
            except Exception as exc:
                err = exc
        with lock:
            results[job.index] = value
            if err is not None:
                errors[job.index] = err
                if max_failures is not None and len(errors) > max_failures:
                    stop.set()

    def work(stream):
        with t.cuda.stream(stream):
            while not stop.is_set():
                try:
                    job = q.get_nowait()
                except queue.Empty:
                    break
                res = err = None
                try:
                    with D.nvtx(f"hgb:sample {job.index}"):
                        sam, hard = space.model_for_params(job.params, job.shape)
                        if batched:
                            data, _, number, h2fdf = run_model_grids(sam, hard, pta_dur=pta_dur, nfreqs=nfreqs,
                                                                     nreals=job.nreals, seed=job.seed, **flags)
                            ev = t.cuda.Event()
                            ev.record(stream)
                            ready.put((job, data, number, h2fdf, ev))
                            continue
                        res = run_model(sam, hard, pta_dur=pta_dur, nfreqs=nfreqs, nreals=job.nreals,
                                        nloudest=nloudest, seed=job.seed, **flags)
                except Exception as exc:   # a failed sample gives NaN rows, as in the reference's libraries
                    err = exc
                finish(job, res, err)
        if batched:
            ready.put(_DONE)

    def realize():
        rstream = t.cuda.Stream(device=dev)
        live = workers
        with t.cuda.stream(rstream):
            while live > 0:
                group = []
                while len(group) < batch and live > 0:
                    item = ready.get()
                    if item is _DONE:
                        live -= 1
                    else:
                        group.append(item)
                if not group:
                    continue
                done = set()
                try:
                    for _, _, number, h2fdf, ev in group:
                        rstream.wait_event(ev)
                        number.record_stream(rstream)   # made on a worker's stream, read on this one
                        h2fdf.record_stream(rstream)
                    outs = single_sources.ss_realize_batch_device(
                        [(number, h2fdf, job.nreals, job.seed) for job, _, number, h2fdf, _ in group], nloudest,
                        blocks_per_sm=blocks_per_sm)
                    for (job, data, _, _, _), out in zip(group, outs):
                        if isinstance(out, Exception):
                            res, err = None, out
                        else:
                            res, err = dict(data, hc_ss=D.to_host(out[0]), hc_bg=D.to_host(out[1])), None
                        done.add(job.index)
                        finish(job, res, err)
                except Exception as exc:   # the whole group fails; the workers keep going
                    for job, *_ in group:
                        if job.index not in done:
                            finish(job, None, exc)
        rstream.synchronize()

    threads = [threading.Thread(target=work, args=(s,), daemon=True) for s in streams]
    if batched:
        threads.append(threading.Thread(target=realize, daemon=True))
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for s in streams:
        s.synchronize()
    if stop.is_set():
        first = min(errors)
        raise RuntimeError(f"{len(errors)} library samples failed, more than max_failures={max_failures}; "
                           f"first: sample {first}: {errors[first]!r}") from errors[first]
    if errors and len(errors) == len(jobs):
        raise next(iter(errors.values()))
    return results, errors


def _workload_class(jobs, nfreqs):
    """A coarse key for the tuning cache: log2 of the mean per-sample cost and of the sample count."""
    mean_cost = float(np.mean([j.cost(nfreqs) for j in jobs]))
    return f"c{int(np.log2(max(mean_cost, 1.0)))}_n{int(np.log2(max(len(jobs), 1)))}"


def _tuning_key(jobs, nfreqs):
    t = D.torch()
    return f"{t.cuda.get_device_name(D.device())}|{_workload_class(jobs, nfreqs)}"


def _load_tuning():
    try:
        with open(_TUNING_PATH) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_tuning(key, entry):
    with _TUNING_LOCK:
        table = _load_tuning()
        table[key] = entry
        try:
            os.makedirs(os.path.dirname(_TUNING_PATH), exist_ok=True)
            with open(_TUNING_PATH, "w") as fh:
                json.dump(table, fh, indent=1, sort_keys=True)
        except OSError:
            pass


def autotune(space, jobs, nfreqs=DEF_NUM_FBINS, nloudest=DEF_NUM_LOUDEST, pta_dur=DEF_PTA_DUR, flags=None,
             candidates=CANDIDATES, probe=8, use_cache=True):
    """Pick (workers, waves) for ``jobs`` by timing ``probe`` of them, spread over the cost range, at
    each candidate schedule (after one untimed pass).  The scatter-plan cache is cleared before every
    timed pass, so each candidate pays the per-sample host work a real library run pays.  Returns
    ``dict(workers=, waves=, table={"w,v": draws/s})``; the winner is cached per device and workload
    class."""
    from ..sams import scatter
    flags = dict(singles_flag=True) if flags is None else flags
    key = _tuning_key(jobs, nfreqs)
    if use_cache:
        hit = _load_tuning().get(key)
        if hit is not None:
            return hit
    ranked = sorted(jobs, key=lambda j: -j.cost(nfreqs))
    pick = np.unique(np.linspace(0, len(ranked) - 1, min(probe, len(ranked))).round().astype(int))
    probe_jobs = [ranked[i] for i in pick]
    draws = float(sum(j.cost(nfreqs) for j in probe_jobs))
    lib = N.load()
    old_waves = lib.hgb_get_bulk_waves()
    _run_jobs(space, probe_jobs, 1, nfreqs, nloudest, pta_dur, flags)   # untimed: lazy setup, allocator warm-up
    table = {}
    try:
        for workers, waves in candidates:
            N.check(lib.hgb_set_bulk_waves(int(waves)), "hgb_set_bulk_waves")
            scatter.clear_plan_cache()
            D.torch().cuda.synchronize()
            t0 = time.perf_counter()
            _run_jobs(space, probe_jobs, workers, nfreqs, nloudest, pta_dur, flags)
            D.torch().cuda.synchronize()
            table[f"{workers},{waves}"] = draws / (time.perf_counter() - t0)
    finally:
        N.check(lib.hgb_set_bulk_waves(old_waves), "hgb_set_bulk_waves")
    best = max(table, key=table.get)
    workers, waves = (int(v) for v in best.split(","))
    entry = dict(workers=workers, waves=waves, table=table, probe=len(probe_jobs))
    _store_tuning(key, entry)
    return entry


def run_library(space, shapes=None, nreals=None, nfreqs=DEF_NUM_FBINS, nloudest=DEF_NUM_LOUDEST,
                pta_dur=DEF_PTA_DUR, seed=0, singles_flag=True, gwb_flag=False, params_flag=False,
                details_flag=False, workers=None, waves=None, tune=True, indices=None, stats=None, reduce=None,
                output_dir=None, recreate=False, max_failures=None, precision="fp64", batch=0, blocks_per_sm=0):
    """Evaluate the samples of ``space`` (all, or ``indices``) on this GPU; returns the list of
    per-sample :func:`lib_tools.run_model` dicts in sample order (``None`` for a failed sample), the
    input that :func:`lib_tools.write_library` takes.

    ``shapes`` / ``nreals``: per-sample lists or one value each (see :func:`make_jobs`).  ``seed``
    keys every sample's realizations (:func:`sample_seed`).  ``workers`` / ``waves`` fix the
    schedule; otherwise it comes from :func:`autotune` (``tune=True``) or defaults to (6, 12).
    ``stats``, when a dict, receives the schedule, wall time, sample count, realizations and draws.
    ``reduce``, when given, maps each sample's dict to what is kept (on the worker, as soon as the
    sample is done), so large libraries need not hold every realization in host memory.

    ``output_dir``: every sample writes ``library__p{index:06d}.npz`` there as it finishes (its
    run_model dict plus ``params`` / ``param_names``; list-valued keys as ``key_0``, ``key_1``, ...), or
    a file holding only ``fail`` when it fails (gen_lib.py:236-323).  A rerun resumes: samples whose
    file exists and is not a failure are loaded instead of run (unless ``recreate``), failed ones are
    attempted again (gen_lib.py:288-300).  ``max_failures``: raise RuntimeError once more samples than
    this have failed (gen_lib.py:42, :213-218).  ``precision``: the grid arithmetic of every sample
    (see :meth:`Semi_Analytic_Model.gwb`).  ``batch`` / ``blocks_per_sm``: run the single-source
    realizations of up to ``batch`` samples as one kernel launch (see :func:`_run_jobs`); the results
    do not change.
    """
    flags = dict(singles_flag=singles_flag, gwb_flag=gwb_flag, params_flag=params_flag, details_flag=details_flag,
                 precision=precision)
    jobs = make_jobs(space, shapes, nreals, seed, indices)
    done = {}
    if output_dir is not None:
        os.makedirs(str(output_dir), exist_ok=True)
        if not recreate:
            for job in jobs:
                path = sim_fname(output_dir, job.index)
                if os.path.exists(path):
                    res = load_sim_file(path)
                    if res is not None:
                        done[job.index] = res if reduce is None else reduce(res)
        jobs_all, jobs = jobs, [j for j in jobs if j.index not in done]
    else:
        jobs_all = jobs
    if stats is not None:
        stats.update(skipped=len(done))
    if not jobs:
        if stats is not None:
            stats.update(workers=0, waves=None, seconds=0.0, samples=len(jobs_all), failed=0, realizations=0,
                         draws=0.0, tuning=None, errors={})
        return [done.get(j.index) for j in sorted(jobs_all, key=lambda j: j.index)]
    tuned = None
    if workers is None or waves is None:
        if tune:
            tuned = autotune(space, jobs, nfreqs, nloudest, pta_dur, flags)
            workers = tuned["workers"] if workers is None else workers
            waves = tuned["waves"] if waves is None else waves
        else:
            workers = 6 if workers is None else workers
            waves = 12 if waves is None else waves
    lib = N.load()
    old_waves = lib.hgb_get_bulk_waves()
    N.check(lib.hgb_set_bulk_waves(int(waves)), "hgb_set_bulk_waves")
    try:
        D.torch().cuda.synchronize()
        t0 = time.perf_counter()
        results, errors = _run_jobs(space, jobs, int(workers), nfreqs, nloudest, pta_dur, flags, reduce,
                                    output_dir=output_dir, max_failures=max_failures, batch=int(batch),
                                    blocks_per_sm=int(blocks_per_sm))
        D.torch().cuda.synchronize()
        wall = time.perf_counter() - t0
    finally:
        N.check(lib.hgb_set_bulk_waves(old_waves), "hgb_set_bulk_waves")
    if stats is not None:
        stats.update(workers=int(workers), waves=int(waves), batch=int(batch), blocks_per_sm=int(blocks_per_sm),
                     seconds=wall, samples=len(jobs_all),
                     failed=len(errors), realizations=int(sum(j.nreals for j in jobs)),
                     draws=float(sum(j.cost(nfreqs) for j in jobs)), tuning=tuned,
                     errors={k: repr(v) for k, v in errors.items()})
    results.update(done)
    return [results.get(j.index) for j in sorted(jobs_all, key=lambda j: j.index)]
