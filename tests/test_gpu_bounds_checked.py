"""The bounds-checked build (``build(checked=True)``: -DHGB_BOUNDS_CHECK) on small shapes.

Every instrumented index (caller orders in the gather, the loudest-slot search, the sampler's
inversion-table and guide entries, the chunk partials) stays inside its array, and the results equal
the production build's bit for bit.  Each library runs in its own subprocess (the loader picks the
checked one when HOLODECK_GB300_CHECKED=1); a flagged index raises there (HGB_STATUS_BOUNDS).
"""

import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = r'''
import json, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
import holodeck_gb300 as H
from holodeck_gb300 import constants as C
from holodeck_gb300 import cyutils, single_sources
from holodeck_gb300 import _device as D
from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch
out = {}
_, fe = H.utils.pta_freqs(16.0 * C.YR, 7)
for n, scatter in ((5, 0.0), (8, 0.3), (12, 0.3)):
    sam = H.sams.Semi_Analytic_Model(shape=(n, n + 1, n + 2), gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=scatter))
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5)
    for prec in ("fp64", "fp32"):
        ss, bg = sam.gwb(fe, hard=hard, realize=1100, loudest=3, seed=7 + n, precision=prec)
        out[f"gwb_{n}_{prec}_ss"], out[f"gwb_{n}_{prec}_bg"] = np.asarray(ss).tolist(), np.asarray(bg).tolist()
    ss, bg, sspar, bgpar = sam.gwb(fe, hard=hard, realize=9, loudest=2, seed=3, params=True)
    for name, x in zip(("ss", "bg", "sspar", "bgpar"), (ss, bg, sspar, bgpar)):
        out[f"params_{n}_{name}"] = np.asarray(x).tolist()
# realizations over all sampler regimes, one call and the multi-sample launch
rng = np.random.default_rng(1)
items = []
for nb, nr in ((300, 5), (2000, 1030)):
    lam = 10.0 ** rng.uniform(-4.0, 8.0, size=(nb, 3))
    num = torch.as_tensor(lam, device="cuda")
    hh = torch.as_tensor(10.0 ** rng.uniform(-32.0, -26.0, size=(nb, 3)), device="cuda")
    items.append(dict(number=num, h2fdf=hh, order=single_sources.sort_order_device(hh), nreals=nr, seed=nb,
                      status=D.StatusWord()))
for k, (ss, bg) in enumerate(cyutils.loudest_batch_device(items, 4, blocks_per_sm=2)):
    out[f"batch_{k}_ss"], out[f"batch_{k}_bg"] = ss.cpu().numpy().tolist(), bg.cpu().numpy().tolist()
    cyutils._raise_status(items[k]["status"])
space = PS_Classic_Phenom_Uniform(nsamples=3, seed=2)
res = batch.run_library(space, [(9, 10, 11)] * 3, [40, 7, 1025], nfreqs=4, nloudest=2, seed=5, workers=2, waves=2,
                        tune=False)
for k, r in enumerate(res):
    out[f"library_{k}_ss"], out[f"library_{k}_bg"] = r["hc_ss"].tolist(), r["hc_bg"].tolist()
print("RESULT " + json.dumps(out))
'''


def _run(checked):
    env = dict(os.environ)
    env.pop("HOLODECK_GB300_CHECKED", None)
    if checked:
        env["HOLODECK_GB300_CHECKED"] = "1"
    res = subprocess.run([sys.executable, "-c", CASES, ROOT], capture_output=True, text=True, env=env, timeout=900)
    assert res.returncode == 0, res.stderr[-4000:]
    line = [ln for ln in res.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    return json.loads(line[len("RESULT "):])


@pytest.mark.gpu
def test_bounds_checked_build_on_small_shapes(built_lib):
    from holodeck_gb300 import build as B
    B.build(checked=True)
    got = _run(checked=True)
    ref = _run(checked=False)
    assert got.keys() == ref.keys()
    for key in ref:   # one array per key
        assert np.array_equal(np.asarray(got[key], dtype=float), np.asarray(ref[key], dtype=float),
                              equal_nan=True), key
