"""GPU versions of the holodeck/cyutils.pyx functions on the SAM path.

``loudest_hc_from_sorted`` (cyutils.pyx:1220-1264), ``loudest_hc_and_par_from_sorted_redz``
(cyutils.pyx:1541-1770) and ``sam_poisson_gwb`` (cyutils.pyx:854-897) keep the reference's argument
lists.  Two keyword arguments are added:

* ``seed``   -- 64-bit key of the Philox draws (default: fresh entropy, like the reference's
               unseeded ``PCG64()``);
* ``replay`` -- the draws themselves, to reproduce a numpy PCG64 stream bit for bit:
               (R, F, B) in the sorted-bin order for ``loudest_hc_from_sorted`` and (B, F, R)
               for ``sam_poisson_gwb`` (the reference's draw order in both cases).
"""

import os

import numpy as np

from . import _device as D
from . import _native as N

NORMAL_THRESHOLD = 1e10


def new_seed():
    return int.from_bytes(os.urandom(8), "little")


def _check_threshold(normal_threshold):
    if int(normal_threshold) != int(NORMAL_THRESHOLD):
        raise ValueError(f"normal_threshold={normal_threshold}: only the reference default 1e10 is supported")


def checked_order(order, n_bins, dev=None):
    """A caller-supplied loudest-first order as a device int32 tensor, after checking that it is a
    permutation of range(n_bins): the realization kernels index the grids with it, so a short array
    or an out-of-range index must stop here, as numpy's indexing stops the reference."""
    t = D.torch()
    n_bins = int(n_bins)
    if D.is_torch(order):
        flat = order.reshape(-1).to(t.int64)       # checked where it lives
        lo_hi = (lambda: (int(flat.min().item()), int(flat.max().item())))
        once = (lambda: int(t.bincount(flat, minlength=n_bins).max().item()) == 1)
    else:
        flat = np.asarray(order).reshape(-1)       # host data: checked before any device work
        if flat.size and not np.issubdtype(flat.dtype, np.integer):
            raise ValueError(f"order must hold integer bin indices, got {flat.dtype}")
        flat = flat.astype(np.int64)
        lo_hi = (lambda: (int(flat.min()), int(flat.max())))
        once = (lambda: int(np.bincount(flat, minlength=n_bins).max()) == 1)
    if int(flat.shape[0]) != n_bins:
        raise ValueError(f"order holds {flat.shape[0]} indices; the grid has {n_bins} bins")
    if n_bins:
        lo, hi = lo_hi()
        if lo < 0 or hi >= n_bins:
            raise ValueError(f"order indices must lie in [0, {n_bins}); got [{lo}, {hi}]")
        if not once():
            raise ValueError("order must visit every bin exactly once")
    return D.as_device(flat, dev, dtype=t.int32)


def loudest_device(number, h2fdf, nreals, nloudest, order, seed=None, replay=None, status=None, freq_offset=0,
                   out=None):
    """Device (hc2ss[F, R, L], hc2bg[F, R]) from device number/h2fdf (B, F) and order (B,) int32.

    ``freq_offset``: the global index of column 0 in a frequency chunk of a wider run; Philox draws
    are keyed by the global frequency, so chunk results equal the same frequencies' results of one
    call over the whole band.  ``out``: preallocated contiguous (hc2ss, hc2bg) to write into.
    """
    t = D.torch()
    nf = int(number.shape[-1])
    nb = int(number.numel() // nf)
    dev = number.device
    if out is None:
        hc2ss = t.empty((nf, nreals, nloudest), dtype=t.float64, device=dev)
        hc2bg = t.empty((nf, nreals), dtype=t.float64, device=dev)
    else:
        hc2ss, hc2bg = out
        if (tuple(hc2ss.shape) != (nf, nreals, nloudest) or tuple(hc2bg.shape) != (nf, nreals)
                or not (hc2ss.is_contiguous() and hc2bg.is_contiguous())):
            raise ValueError("out must be contiguous (F, R, L) and (F, R) float64 tensors")
    if freq_offset and replay is not None:
        raise ValueError("freq_offset applies to Philox draws only")
    if order.dtype != t.int32 or int(order.numel()) != nb or order.device != dev:
        raise ValueError(f"order must be an int32 tensor of {nb} bin indices on {dev} (see checked_order)")
    mode = N.RNG_PHILOX if replay is None else N.RNG_REPLAY
    rep = None
    if replay is not None:
        rep = D.as_device(replay)
        if tuple(rep.shape) != (nreals, nf, nb):
            raise ValueError(f"replay must be shaped (R, F, B)=({nreals}, {nf}, {nb}), got {tuple(rep.shape)}")
    lib = N.load()
    ws_bytes = lib.hgb_loudest_workspace_bytes(nb, nf, int(nreals), int(nloudest), mode)
    ws = D.workspace(ws_bytes, dev)
    st = status if status is not None else D.StatusWord(dev)
    seed = new_seed() if seed is None else int(seed) & 0xFFFFFFFFFFFFFFFF
    N.call("hgb_loudest_hc_from_sorted_ex", N.ptr(number), N.ptr(h2fdf), nb, nf, int(nreals), int(nloudest),
           N.ptr(order), mode, seed, N.ptr(rep), N.ptr(hc2ss), N.ptr(hc2bg), N.ptr(ws), int(ws_bytes), st.ptr,
           N.stream_handle(), int(freq_offset))
    return hc2ss, hc2bg


def loudest_batch_device(samples, nloudest, blocks_per_sm=0):
    """:func:`loudest_device` (Philox draws) for many samples in one bulk-background launch
    (``hgb_loudest_hc_batch``).  ``samples``: list of dicts with ``number`` and ``h2fdf`` (B_i, F)
    device tensors (F shared), ``order`` (B_i,) int32, ``nreals``, ``seed`` and ``status`` (a
    :class:`_device.StatusWord` or None).  Returns [(hc2ss (F, R_i, L), hc2bg (F, R_i))], each equal
    to that sample's own :func:`loudest_device` result with the same seed, bit for bit.
    ``blocks_per_sm``: 0 = one block per work item, 1..6 = a persistent grid (see the C header)."""
    t = D.torch()
    if not samples:
        return []
    nf = int(samples[0]["number"].shape[-1])
    dev = samples[0]["number"].device
    arr = (N.HgbLoudestSample * len(samples))()
    outs, keep = [], []
    lib = N.load()
    for ii, smp in enumerate(samples):
        num, hh, order = smp["number"], smp["h2fdf"], smp["order"]
        nr = int(smp["nreals"])
        if int(num.shape[-1]) != nf or tuple(hh.shape) != tuple(num.shape) or num.device != dev:
            raise ValueError("every sample's number / h2fdf must be (B, F) on one device with the same F")
        nb = int(num.numel() // nf)
        if order.dtype != t.int32 or int(order.numel()) != nb or order.device != dev:
            raise ValueError(f"order must be an int32 tensor of {nb} bin indices on {dev} (see checked_order)")
        hc2ss = t.empty((nf, nr, int(nloudest)), dtype=t.float64, device=dev)
        hc2bg = t.empty((nf, nr), dtype=t.float64, device=dev)
        ws_bytes = lib.hgb_loudest_workspace_bytes(nb, nf, nr, int(nloudest), N.RNG_PHILOX)
        ws = D.workspace(ws_bytes, dev)
        st = smp.get("status")
        seed = new_seed() if smp.get("seed") is None else int(smp["seed"]) & 0xFFFFFFFFFFFFFFFF
        arr[ii] = N.HgbLoudestSample(num.data_ptr(), hh.data_ptr(), order.data_ptr(), nb, nr, seed,
                                     hc2ss.data_ptr(), hc2bg.data_ptr(), ws.data_ptr(), int(ws_bytes),
                                     st.t.data_ptr() if st is not None else None)
        outs.append((hc2ss, hc2bg))
        keep.append(ws)
    bw_bytes = lib.hgb_loudest_batch_workspace_bytes(arr, len(samples), nf)
    bw = D.workspace(bw_bytes, dev)
    N.call("hgb_loudest_hc_batch", arr, len(samples), nf, int(nloudest), int(blocks_per_sm), N.ptr(bw),
           int(bw_bytes), N.stream_handle())
    N.add_launches(5 * len(samples) + 2)
    del keep   # the caching allocator reuses the workspaces only after this stream's work
    return outs


def loudest_hc_from_sorted(number, h2fdf, nreals, nloudest, msort, qsort, zsort, normal_threshold=1e10,
                           seed=None, replay=None):
    """hc^2 of the loudest sources (F, R, L) and of the background (F, R); cyutils.pyx:1220-1264."""
    _check_threshold(normal_threshold)
    like_torch = D.is_torch(number)
    shape = tuple(number.shape)
    num = D.as_device(number).reshape(-1, shape[-1])
    hh = D.as_device(h2fdf).reshape(-1, shape[-1])
    ms, qs, zs = [np.asarray(D.to_host(v) if D.is_torch(v) else v, dtype=np.int64) for v in (msort, qsort, zsort)]
    order_t = checked_order(np.ravel_multi_index((ms, qs, zs), shape[:3]), num.shape[0], num.device)
    st = D.StatusWord()
    ss, bg = loudest_device(num, hh, int(nreals), int(nloudest), order_t, seed=seed, replay=replay, status=st)
    _raise_status(st)
    if like_torch:
        return ss, bg
    return D.to_host(ss), D.to_host(bg)


def sam_poisson_gwb(dist, hc2, nreals, normal_threshold=1e10, seed=None, replay=None):
    """hc^2 of the whole population per (F, R), bins in grid order (cyutils.pyx:854-897)."""
    _check_threshold(normal_threshold)
    like_torch = D.is_torch(dist)
    t = D.torch()
    nf = int(dist.shape[-1])
    num = D.as_device(dist).reshape(-1, nf)
    hh = D.as_device(hc2).reshape(-1, nf)
    nb = int(num.shape[0])
    gwb = t.empty((nf, int(nreals)), dtype=t.float64, device=num.device)
    mode = N.RNG_PHILOX if replay is None else N.RNG_REPLAY
    rep = None
    if replay is not None:
        rep = D.as_device(replay)
        if tuple(rep.shape) != (nb, nf, int(nreals)):
            raise ValueError(f"replay must be shaped (B, F, R)=({nb}, {nf}, {nreals}), got {tuple(rep.shape)}")
    st = D.StatusWord()
    seed = new_seed() if seed is None else int(seed) & 0xFFFFFFFFFFFFFFFF
    lib = N.load()
    ws_bytes = lib.hgb_sam_poisson_gwb_workspace_bytes(nb, nf, int(nreals))
    ws = D.workspace(ws_bytes, num.device)
    N.call("hgb_sam_poisson_gwb", N.ptr(num), N.ptr(hh), nb, nf, int(nreals), mode, seed, N.ptr(rep), N.ptr(gwb),
           N.ptr(ws), int(ws_bytes), st.ptr, N.stream_handle())
    _raise_status(st)
    return gwb if like_torch else D.to_host(gwb)


def _frexp_exponent(values):
    """frexp exponent of max |finite, nonzero value| (0 when there is none)."""
    v = np.abs(np.asarray(values, dtype=np.float64))
    v = v[np.isfinite(v) & (v > 0)]
    return int(np.frexp(v.max())[1]) if v.size else 0


def loudest_par_device(number, h2fdf, nreals, nloudest, order, mt, mr, rz, grids, grid_scales, seed=None,
                       replay=None, status=None):
    """Device (hc2ss, hc2bg, sspar, bgpar) of the parameter path (cyutils.pyx:1541-1770).

    number / h2fdf / the four ``grids`` (redz_mid, dcom, sepa, angs) are device (M-1, Q-1, Z-1, F)
    tensors, ``mt`` / ``mr`` / ``rz`` the bin centres (host arrays), ``order`` the int32 loudest-first
    bin order and ``grid_scales`` a device int32[4] of the grids' frexp exponents (hgb_param_grids).
    """
    t = D.torch()
    shape = tuple(number.shape)
    nf = int(shape[-1])
    nb = int(number.numel() // nf)
    dev = number.device
    hc2ss = t.empty((nf, nreals, nloudest), dtype=t.float64, device=dev)
    hc2bg = t.empty((nf, nreals), dtype=t.float64, device=dev)
    sspar = t.empty((4, nf, nreals, nloudest), dtype=t.float64, device=dev)
    bgpar = t.empty((7, nf, nreals), dtype=t.float64, device=dev)
    if order.dtype != t.int32 or int(order.numel()) != nb or order.device != dev:
        raise ValueError(f"order must be an int32 tensor of {nb} bin indices on {dev} (see checked_order)")
    mode = N.RNG_PHILOX if replay is None else N.RNG_REPLAY
    rep = None
    if replay is not None:
        rep = D.as_device(replay)
        if tuple(rep.shape) != (nreals, nf, nb):
            raise ValueError(f"replay must be shaped (R, F, B)=({nreals}, {nf}, {nb}), got {tuple(rep.shape)}")
    mt_d, mr_d, rz_d = (D.as_device(np.ascontiguousarray(x, dtype=np.float64), dev) for x in (mt, mr, rz))
    scales = t.cat([t.tensor([_frexp_exponent(x) for x in (mt, mr, rz)], dtype=t.int32, device=dev),
                    grid_scales.to(t.int32)])
    lib = N.load()
    ws_bytes = lib.hgb_loudest_par_workspace_bytes(nb, nf, int(nreals), int(nloudest), mode)
    ws = D.workspace(ws_bytes, dev)
    st = status if status is not None else D.StatusWord(dev)
    seed = new_seed() if seed is None else int(seed) & 0xFFFFFFFFFFFFFFFF
    N.call("hgb_loudest_hc_and_par_from_sorted", N.ptr(number), N.ptr(h2fdf), int(shape[0]), int(shape[1]),
           int(shape[2]), nf, int(nreals), int(nloudest), N.ptr(order), mode, seed, N.ptr(rep), N.ptr(mt_d),
           N.ptr(mr_d), N.ptr(rz_d), *[N.ptr(g) for g in grids], N.ptr(scales), N.ptr(hc2ss), N.ptr(hc2bg),
           N.ptr(sspar), N.ptr(bgpar), N.ptr(ws), int(ws_bytes), st.ptr, N.stream_handle())
    return hc2ss, hc2bg, sspar, bgpar


def loudest_hc_and_par_from_sorted_redz(number, h2fdf, nreals, nloudest, mt, mr, rz, redz_final, dcom_final, sepa,
                                        angs, msort, qsort, zsort, normal_threshold=1e10, seed=None, replay=None):
    """(hc2ss (F, R, L), hc2bg (F, R), sspar (4, F, R, L), bgpar (7, F, R)); cyutils.pyx:1541-1770.

    Same arguments as the reference (the (M, Q, Z, F) grids as numpy arrays or device tensors);
    ``seed`` / ``replay`` as in :func:`loudest_hc_from_sorted`.
    """
    _check_threshold(normal_threshold)
    like_torch = D.is_torch(number)
    shape = tuple(number.shape)
    num = D.as_device(number)
    hh = D.as_device(h2fdf)
    grids = [D.as_device(np.broadcast_to(np.asarray(D.to_host(g) if D.is_torch(g) else g), shape).copy()
                         if not D.is_torch(g) else g).contiguous() for g in (redz_final, dcom_final, sepa, angs)]
    t = D.torch()
    scales = t.tensor([_frexp_exponent(D.to_host(g)[D.to_host(hh) != 0]) for g in grids], dtype=t.int32,
                      device=num.device)
    ms, qs, zs = [np.asarray(D.to_host(v) if D.is_torch(v) else v, dtype=np.int64) for v in (msort, qsort, zsort)]
    order = checked_order(np.ravel_multi_index((ms, qs, zs), shape[:3]), num.numel() // shape[-1], num.device)
    st = D.StatusWord()
    out = loudest_par_device(num, hh, int(nreals), int(nloudest), order, D.to_host(mt) if D.is_torch(mt) else mt,
                             D.to_host(mr) if D.is_torch(mr) else mr, D.to_host(rz) if D.is_torch(rz) else rz,
                             grids, scales, seed=seed, replay=replay, status=st)
    _raise_status(st)
    return out if like_torch else tuple(D.to_host(x) for x in out)


def _raise_status(st):
    code = st.read()
    N.check_bounds(code, "realizations")
    if code & N.STATUS_ITERATION_LIMIT:
        raise RuntimeError("a Poisson sampler exhausted its attempt budget (device status ITERATION_LIMIT)")
