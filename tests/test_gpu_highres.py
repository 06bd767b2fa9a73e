"""The high-resolution grid (181 x 161 x 201 edges, 100 harmonics of 1/(16 yr)) end to end, at 1000
realizations instead of 10^4 to keep the test short: the largest sizes the path is specified for,
checked through properties that hold at any size.

- The expectation of the total characteristic strain per frequency, E[hc_bg^2 + sum_l hc_ss^2], is
  sum_b number_b h2fdf_b (every source is either a loudest slot or background), with variance
  sum_b number_b h2fdf_b^2; the realization mean may not fall more than five standard errors
  below it (the upper side, heavy-tailed, gets a loose bound).
- The same seed gives the same realizations bit for bit.
- Outputs are finite, and at the first frequency (whose strain orders the bins) hc_ss is
  non-increasing along the slots.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_high_resolution_grid_properties(built_lib):
    import torch
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    gsmf = H.sams.GSMF_Schechter(phi0=-2.77, mchar0_log10=11.24, alpha0=-1.24)
    mmb = H.host_relations.MMBulge_KH2013(mamp_log10=8.69, mplaw=1.17, scatter_dex=0.28)
    sam = H.sams.Semi_Analytic_Model(shape=(181, 161, 201), gsmf=gsmf, gpf=H.sams.GPF_Power_Law(),
                                     gmt=H.sams.GMT_Power_Law(), mmbulge=mmb)
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5)
    _, fe = H.utils.pta_freqs(16.0 * C.YR, 100)
    R, L = 1000, 10
    ss, bg = sam.gwb(fe, hard=hard, realize=R, loudest=L, seed=5, return_torch=True)
    ss2, bg2 = sam.gwb(fe, hard=hard, realize=R, loudest=L, seed=5, return_torch=True)
    torch.cuda.synchronize()
    assert torch.equal(ss, ss2) and torch.equal(bg, bg2)
    del ss2, bg2
    assert ss.shape == (100, R, L) and bg.shape == (100, R)
    assert bool(torch.isfinite(ss).all()) and bool(torch.isfinite(bg).all())
    assert bool((ss[0, :, 1:] <= ss[0, :, :-1]).all())   # slots follow the first frequency's order
    redz_final, diff_num = sam._dbn_device(hard, H.utils.midpoints(fe) / 2.0)
    number, h2fdf = sam._number_and_strain(fe / 2.0, diff_num, redz_final)
    del redz_final, diff_num
    lam, h = number.reshape(-1, 100), h2fdf.reshape(-1, 100)
    s1 = (lam * h).sum(0).cpu().numpy()               # E[total]
    s2 = (lam * h * h).sum(0).cpu().numpy()           # Var[total] (Poisson: Var[n h] = lambda h^2)
    del number, h2fdf, lam, h
    total = (bg ** 2 + (ss ** 2).sum(-1)).cpu().numpy()   # (F, R)
    z = (total.mean(1) - s1) / np.sqrt(s2 / R)
    # The variance is dominated by rare, loud bins, so the realization mean is heavy-tailed upwards
    # (a rare source lifts it by many standard errors) but light-tailed downwards (a sum of
    # non-negative terms): a tight lower bound and a loose upper one.
    assert np.all(z > -5.0), (np.argmin(z), z.min())
    assert np.all(z < 50.0), (np.argmax(z), z.max())
