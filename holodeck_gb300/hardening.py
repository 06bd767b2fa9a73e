"""Binary hardening models of the SAM path (holodeck/hardening.py): Hard_GW and Fixed_Time_2PL_SAM."""

import numpy as np

from . import _device as D
from . import constants as C


class _Hardening:
    CONSISTENT = None


class Hard_GW(_Hardening):
    """GW-driven hardening (hardening.py:87-212); used by the Hard_GW branch of the dbn kernel."""

    CONSISTENT = False

    @property
    def consistent(self):
        return False


class Fixed_Time_2PL_SAM(_Hardening):
    """Two-power-law hardening normalised to a fixed total lifetime (hardening.py:1371-1457).

    The per-cell normalisation is found on the GPU (Brent root of the trapezoid lifetime,
    ``csrc/hgb_hardening.cu``) when the instance is built, as the reference does.
    """

    CONSISTENT = True

    def __init__(self, sam, time, sepa_init=1.0e3 * C.PC, rchar=10.0 * C.PC, gamma_inner=-1.0, gamma_outer=+1.5,
                 num_steps=300):
        from .sams import sam_cyutils
        assert np.ndim(time) == 0
        assert np.ndim(rchar) == 0
        assert np.ndim(gamma_inner) == 0
        assert np.ndim(gamma_outer) == 0
        t = D.torch()
        mt_d, mr_d = sam._edges_device()[:2]
        # The root finding depends only on the mass grid: it runs on a side stream, concurrently with the
        # density and scatter stages that the next gwb() call enqueues, and the dbn stage waits on it.
        main = t.cuda.current_stream(mt_d.device)
        side = D.side_stream("hardening_norm", mt_d.device)
        side.wait_stream(main)
        with t.cuda.stream(side), D.nvtx("hgb:hardening_norm"):
            mtot, mrat = t.meshgrid(mt_d, mr_d, indexing="ij")
            shape = tuple(mtot.shape)
            nl, norm = sam_cyutils.find_2pwl_hardening_norm(time, mtot.reshape(-1), mrat.reshape(-1), sepa_init,
                                                            rchar, gamma_inner, gamma_outer, num_steps,
                                                            return_norm=True)
            self._norm_ready = t.cuda.Event()
            self._norm_ready.record(side)
        for x in (nl, norm):
            x.record_stream(main)   # freed memory is not reused before the main stream is done with it
        self._norm_t = norm.reshape(shape)
        self._norm_log10_t = nl.reshape(shape)
        self._norm_host = None
        self._target_time = time
        self._num_steps = num_steps
        self._sepa_init = sepa_init
        self._rchar = rchar
        self._gamma_inner = gamma_inner
        self._gamma_outer = gamma_outer

    @property
    def _norm(self):
        """Hardening-rate normalisation per (mtot, mrat) cell (numpy, like hardening.py:1416)."""
        if self._norm_host is None:
            self._norm_host = D.to_host(self._norm_device())
        return self._norm_host

    def _norm_device(self):
        """The device normalisation, ordered before the work enqueued next on the current stream."""
        D.torch().cuda.current_stream(self._norm_t.device).wait_event(self._norm_ready)
        return self._norm_t

    def __str__(self):
        return (f"Fixed_Time_2PL_SAM :: target_time/Gyr={self._target_time/C.GYR:.2e} num_steps={self._num_steps} "
                f"sepa_init/pc={self._sepa_init/C.PC:.2e} rchar/pc={self._rchar/C.PC:.2e} "
                f"gamma_inner={self._gamma_inner:.2e} gamma_outer={self._gamma_outer:.2e} ")
