"""hgb_loudest_hc_from_sorted_ex: realizations of a run of frequencies that starts at a global
frequency index (cyutils.pyx:1220-1264 split over several calls).

Philox draws are keyed by the global frequency, so frequency chunks realized by separate calls give
the loudest-source strains of one call over the whole band bit for bit; the background strains
differ only in FP32 summation order (the bulk kernel's bin chunking depends on the frequency count).
"""

import numpy as np
import pytest


def test_freq_offset_checked_on_the_host(built_lib):
    """Offsets beyond the counter range return HGB_ERR_INVALID_ARGUMENT before any CUDA call."""
    import ctypes
    from holodeck_gb300 import _native as N
    lib = N.load()
    fake = ctypes.c_void_p(256)   # never dereferenced: the argument checks come first
    args = [fake, fake, 10, 4, 8, 1, fake, N.RNG_PHILOX, 1, None, fake, fake, fake, 1 << 20, fake, None]
    assert lib.hgb_loudest_hc_from_sorted_ex(*args, -1) == N.HGB_ERR_INVALID_ARGUMENT
    assert lib.hgb_loudest_hc_from_sorted_ex(*args, 65532) == N.HGB_ERR_INVALID_ARGUMENT


@pytest.mark.gpu
def test_frequency_chunks_match_one_call(built_lib):
    import torch
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    from holodeck_gb300 import cyutils, single_sources
    sam = H.sams.Semi_Analytic_Model(shape=(20, 21, 22), gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=0.0))
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5)
    _, fe = H.utils.pta_freqs(16.0 * C.YR, 11)
    F, R, L, seed = 11, 96, 3, 1234
    redz_final, diff_num = sam._dbn_device(hard, H.utils.midpoints(fe) / 2.0)
    number, h2fdf = sam._number_and_strain(fe / 2.0, diff_num, redz_final)
    num, hh = number.reshape(-1, F), h2fdf.reshape(-1, F)
    order = single_sources.sort_order_device(h2fdf)
    ss1, bg1 = cyutils.loudest_device(num, hh, R, L, order, seed=seed)
    ss = torch.empty_like(ss1)
    bg = torch.empty_like(bg1)
    for f0, f1 in [(0, 2), (2, 7), (7, 11)]:
        cyutils.loudest_device(num[:, f0:f1].contiguous(), hh[:, f0:f1].contiguous(), R, L, order, seed=seed,
                               freq_offset=f0, out=(ss[f0:f1], bg[f0:f1]))
    torch.cuda.synchronize()
    ss, bg, ss1, bg1 = (x.cpu().numpy() for x in (ss, bg, ss1, bg1))
    assert np.array_equal(ss, ss1)
    assert np.all(np.abs(bg - bg1) <= 1e-5 * np.abs(bg1))
    assert np.all(bg > 0)


@pytest.mark.gpu
def test_overlapped_dbn_matches_sequential(built_lib):
    """gwb() on a fresh model walks the separation steps on a second stream while the scatter runs;
    the results equal the sequential stages bit for bit."""
    import torch
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    from holodeck_gb300 import single_sources

    def model():
        sam = H.sams.Semi_Analytic_Model(shape=(16, 15, 14), gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                         mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=0.3))
        hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0,
                                              gamma_outer=2.5)
        return sam, hard

    _, fe = H.utils.pta_freqs(16.0 * C.YR, 6)
    R, L, seed = 64, 2, 99
    sam, hard = model()
    ss, bg = sam.gwb(fe, hard=hard, realize=R, loudest=L, seed=seed, return_torch=True)
    sam2, hard2 = model()
    rf, dn = sam2._dbn_device(hard2, H.utils.midpoints(fe) / 2.0)
    number, h2fdf = sam2._number_and_strain(fe / 2.0, dn, rf)
    ss2, bg2 = single_sources.ss_realize_device(number, h2fdf, R, L, seed=seed)
    torch.cuda.synchronize()
    assert torch.equal(ss, ss2) and torch.equal(bg, bg2)


@pytest.mark.gpu
def test_sparse_sums_are_order_independent(built_lib):
    """Many sparse bins per tile (expectations 1e-4 .. 0.1, events of one realization from different
    threads): repeated calls with one seed agree bit for bit."""
    import torch
    from holodeck_gb300 import cyutils
    rng = np.random.default_rng(3)
    nb, nf, R, L = 60_000, 3, 2048, 2
    lam = torch.as_tensor(10.0 ** rng.uniform(-4, -1, size=(nb, nf)), device="cuda")
    h = torch.as_tensor(10.0 ** rng.uniform(-32, -26, size=(nb, nf)), device="cuda")
    order = torch.argsort(h[:, 0], descending=True).to(torch.int32)
    runs = [cyutils.loudest_device(lam, h, R, L, order, seed=11) for _ in range(3)]
    torch.cuda.synchronize()
    for ss, bg in runs[1:]:
        assert torch.equal(ss, runs[0][0]) and torch.equal(bg, runs[0][1])
