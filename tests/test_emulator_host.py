"""Host-side pieces of the emulator that need no GPU: the statistics a library sample is reduced to,
and the bfloat16 rounding of the graphed query path's inputs."""

import numpy as np


def test_strain_statistics_against_direct_formulas():
    from holodeck_gb300.emulator import STATS, strain_statistics
    rng = np.random.default_rng(0)
    F, R, L = 5, 301, 3
    hc_ss = np.sort(rng.lognormal(-35.0, 1.0, size=(F, R, L)), axis=-1)[..., ::-1]
    hc_bg = rng.lognormal(-33.0, 0.5, size=(F, R))
    hc_ss[2, :10, :] = 0.0                    # realizations without a resolved loudest source
    st = strain_statistics(hc_ss, hc_bg)
    assert st.shape == (F, len(STATS))
    for f in range(F):
        tot = np.log10(np.sqrt(hc_bg[f] ** 2 + (hc_ss[f] ** 2).sum(-1)))
        assert np.allclose(st[f, :3], np.percentile(tot, [5, 50, 95]), rtol=0, atol=1e-12)
        loud = np.log10(np.where(hc_ss[f, :, 0] > 0, hc_ss[f, :, 0], 1e-40))
        assert np.isclose(st[f, 3], np.median(loud), rtol=0, atol=1e-12)
    assert np.all(st[:, 0] <= st[:, 1]) and np.all(st[:, 1] <= st[:, 2])


def test_library_statistics_accepts_dicts_reduced_rows_and_failures():
    from holodeck_gb300.emulator import library_statistics, sample_statistics
    rng = np.random.default_rng(1)
    res = dict(hc_ss=rng.lognormal(-35, 1, size=(4, 50, 1)), hc_bg=rng.lognormal(-33, 1, size=(4, 50)))
    out = library_statistics([res, None, sample_statistics(res)])
    assert out.shape == (3, 4, 4)
    assert np.array_equal(out[0], out[2]) and np.all(np.isnan(out[1]))


def test_bf16_rounding_matches_torch():
    import torch
    from holodeck_gb300.emulator import bf16_bits
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(-1, 1, 10000), rng.normal(0, 1e3, 1000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.01171875, -1.00390625]]).astype(np.float32)
    ref = torch.as_tensor(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(bf16_bits(x), ref)
