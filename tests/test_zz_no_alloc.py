"""hgb_argsort_f0_desc_static: the allocation-free variant of the f0 argsort.

Collected last (file name) so that it also runs after every other test has used the library; it
passes alone as well.  The GPU test compares two consecutive calls with the workspace entry point
hgb_argsort_f0_desc on the same inputs, including tied keys.
"""

import ctypes

import numpy as np
import pytest

from conftest import load_golden


def test_static_sort_rejects_oversize_on_the_host(built_lib):
    """n_bins above the static capacity returns HGB_ERR_CAPACITY before any CUDA call."""
    from holodeck_gb300 import _native as N
    lib = N.load()
    fake = ctypes.c_void_p(256)   # never dereferenced: the size check comes first
    rc = lib.hgb_argsort_f0_desc_static(fake, (1 << 20) + 1, 1, fake, None)
    assert rc == N.HGB_ERR_CAPACITY
    assert lib.hgb_error_string(rc) == b"input exceeds the static scratch capacity"
    assert lib.hgb_argsort_f0_desc_static(None, 10, 1, fake, None) == N.HGB_ERR_INVALID_ARGUMENT


def _static_order(h):
    import torch
    from holodeck_gb300 import _native as N
    nb, nf = int(h.shape[0]), int(h.shape[1])
    out = torch.full((nb,), -1, dtype=torch.int32, device=h.device)
    N.check(N.load().hgb_argsort_f0_desc_static(N.ptr(h), nb, nf, N.ptr(out), N.stream_handle()),
            "hgb_argsort_f0_desc_static")
    return out


@pytest.mark.gpu
def test_static_sort_matches_workspace_entry_point(built_lib):
    import torch
    from holodeck_gb300 import single_sources
    rng = np.random.default_rng(7)
    g = load_golden("ref_small_2pwl_noscatter.npz")
    golden = torch.as_tensor(g["h2fdf"].reshape(-1, g["h2fdf"].shape[-1]), device="cuda")
    # a large case with many exact ties and zeros (stable order among equal keys)
    big = rng.choice(np.array([0.0, 1e-30, 2e-30, 3e-28]), size=(700_000, 3)) * rng.integers(1, 4, size=(700_000, 3))
    big = torch.as_tensor(big, device="cuda")
    # the capacity itself: 2^20 bins
    full = torch.as_tensor(rng.lognormal(-40.0, 3.0, size=(1 << 20, 2)), device="cuda")
    for h in (golden, big, full, golden):   # consecutive calls, sizes changing between them
        ref = single_sources.sort_order_device(h).cpu().numpy()
        first = _static_order(h).cpu().numpy()
        second = _static_order(h).cpu().numpy()
        assert np.array_equal(first, ref)
        assert np.array_equal(second, ref)
        assert np.array_equal(first, np.argsort(-h[:, 0].cpu().numpy(), kind="stable"))
    torch.cuda.synchronize()
