"""Entry points called from several host threads at once (the batched library's worker pool).

The kernels whose dynamic shared memory depends on the input (the scatter's gradient solve, the
hardening normalisation, the dbn step walk) share one per-function cap on the device; threads
working on grids of different sizes must never see a launch refused because another thread lowered
that cap between its own set and launch (cudaErrorLaunchOutOfResources).
"""

import threading

import numpy as np
import pytest

from conftest import rel_err


def _scatter_case(n):
    mtot = np.logspace(10, 12, n) * 2e33
    mrat = np.logspace(-2, 0, n - 3)
    rng = np.random.default_rng(n)
    dens = rng.lognormal(-8.0, 2.0, size=(mtot.size, mrat.size, 6))
    return mtot, mrat, dens


@pytest.mark.gpu
def test_concurrent_scatter_on_different_grids(built_lib):
    import torch
    from holodeck_gb300.sams import scatter
    cases = [_scatter_case(n) for n in (24, 61)]   # gradient-solve shared memory well apart
    want = []
    for mtot, mrat, dens in cases:
        d = torch.as_tensor(dens, device="cuda")
        scatter.add_scatter_to_masses_device(mtot, mrat, d, 0.3)
        want.append(d.cpu().numpy())
    errors = []

    def run(k):
        mtot, mrat, dens = cases[k]
        try:
            with torch.cuda.stream(torch.cuda.Stream()):
                for _ in range(25):
                    d = torch.as_tensor(dens, device="cuda")
                    scatter.add_scatter_to_masses_device(mtot, mrat, d, 0.3)
                    got = d.cpu().numpy()
                    if not np.array_equal(got, want[k]):
                        errors.append((k, rel_err(got, want[k])))
        except Exception as exc:   # a refused launch surfaces here as NativeError
            errors.append((k, repr(exc)))

    threads = [threading.Thread(target=run, args=(k,)) for k in (0, 1, 0, 1)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors[:3]


@pytest.mark.gpu
def test_concurrent_hardening_norm_on_different_step_counts(built_lib):
    import torch
    from holodeck_gb300.sams import sam_cyutils
    mt = torch.as_tensor(np.logspace(43, 45, 300), device="cuda")
    mr = torch.as_tensor(np.linspace(0.01, 1.0, 300), device="cuda")
    args = dict(time=3e16, mtot=mt, mrat=mr, sepa_init=3e21, rchar=3e19, gamma_inner=-1.0, gamma_outer=1.5)
    want = {ns: sam_cyutils.find_2pwl_hardening_norm(nsteps=ns, **args).cpu().numpy() for ns in (100, 300, 2000)}
    errors = []

    def run(ns):
        try:
            with torch.cuda.stream(torch.cuda.Stream()):
                for _ in range(20):
                    got = sam_cyutils.find_2pwl_hardening_norm(nsteps=ns, **args).cpu().numpy()
                    if not np.array_equal(got, want[ns]):
                        errors.append((ns, "differs"))
        except Exception as exc:
            errors.append((ns, repr(exc)))

    threads = [threading.Thread(target=run, args=(ns,)) for ns in (100, 2000, 300, 2000)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors[:3]
