"""Semi-analytic model (holodeck/sams/sam.py) with every grid stage on the GPU.

:class:`Semi_Analytic_Model` keeps holodeck's constructor, attributes and ``gwb()`` signature.
Grid-sized arrays live on the device as float64 tensors (``(M, Q, Z)`` and ``(M, Q, Z, F)``,
C order like the reference's numpy arrays); the numpy-facing attributes (``static_binary_density``,
``_gmt_time``, ``_redz_prime``) copy them to the host on first access.
"""

import logging

import numpy as np

from .. import _device as D
from .. import _native as N
from .. import constants as C
from .. import cyutils, gravwaves, hardening, host_relations, single_sources, utils
from ..cosmology import cosmo as _cosmo
from . import sam_cyutils
from .components import (_Galaxy_Merger_Rate, _Galaxy_Merger_Time, _Galaxy_Pair_Fraction,
                         _Galaxy_Stellar_Mass_Function, GMR_Illustris, GMT_Power_Law, GPF_Power_Law, GSMF_Schechter)

log = logging.getLogger("holodeck_gb300")

GSMF_USES_MTOT = False       #: sam.py:57
GPF_USES_MTOT = False        #: sam.py:58
GMT_USES_MTOT = False        #: sam.py:59


class Semi_Analytic_Model:
    """Semi-analytic model of MBH-binary populations on an (mtot, mrat, redz) grid (sam.py:66-234)."""

    def __init__(self, mtot=(1.0e4 * C.MSOL, 1.0e12 * C.MSOL, 91), mrat=(1e-3, 1.0, 81), redz=(1e-3, 10.0, 101),
                 shape=None, log=None, gsmf=GSMF_Schechter, gpf=None, gmt=None, gmr=None,
                 mmbulge=host_relations.MMBulge_KH2013, cosmo=None, **kwargs):
        self._log = logging.getLogger("holodeck_gb300") if log is None else log
        deprecated_keys = ["ZERO_DYNAMIC_STALLED_SYSTEMS", "ZERO_GMT_STALLED_SYSTEMS"]
        for key, val in kwargs.items():
            if key in deprecated_keys:
                self._log.error(f"Using deprecated kwarg: {key}: {val}!  In the future this will raise an error.")
            else:
                raise ValueError(f"Unexpected kwarg {key=}: {val=}!")

        gsmf = utils.get_subclass_instance(gsmf, None, _Galaxy_Stellar_Mass_Function)
        mmbulge = utils.get_subclass_instance(mmbulge, None, host_relations._MMBulge_Relation)
        if gpf is None:
            gmr = utils.get_subclass_instance(gmr, GMR_Illustris, _Galaxy_Merger_Rate)
            gmt = utils.get_subclass_instance(gmt, None, _Galaxy_Merger_Time, allow_none=True)
        else:
            if gmr is not None:
                raise ValueError("Can only use one of `gpf` and `gmr`!")
            gmt = utils.get_subclass_instance(gmt, GMT_Power_Law, _Galaxy_Merger_Time)
            gpf = utils.get_subclass_instance(gpf, GPF_Power_Law, _Galaxy_Pair_Fraction)
        self._gsmf = gsmf
        self._gmr = gmr
        self._gpf = gpf
        self._gmt = gmt
        self._mmbulge = mmbulge
        self._cosmo = _cosmo if cosmo is None else cosmo

        if shape is not None and np.isscalar(shape):
            shape = [shape for ii in range(3)]
        params = [mtot, mrat, redz]
        for ii, (par, name) in enumerate(zip(params, ["mtot", "mrat", "redz"])):
            if not isinstance(par, tuple) and (len(par) == 3):
                raise ValueError(f"{name} (type={type(par)}, len={len(par)}) must be a (3,) tuple specifying a "
                                 "log-spacing, or ndarray of grid edges!")
            par = [pp for pp in par]
            if shape is not None and shape[ii] is not None:
                par[2] = shape[ii]
            params[ii] = np.logspace(*np.log10(par[:2]), par[2])
        self.mtot, self.mrat, self.redz = params

        self._density = None
        self._shape = None
        self._density_t = None
        self._gmt_time_t = None
        self._redz_prime_t = None
        self._gmt_time_host = None
        self._redz_prime_host = None
        self._edges_t = None

    # ---- grid

    @property
    def edges(self):
        return [self.mtot, self.mrat, self.redz]

    @property
    def shape(self):
        if self._shape is None:
            self._shape = tuple([len(ee) for ee in self.edges])
        return self._shape

    def _edges_device(self):
        if self._edges_t is None:
            self._edges_t = [D.as_device(ee) for ee in self.edges]
        return self._edges_t

    # ---- static binary density (sam.py:280-398)

    def _model_struct(self):
        m = N.HgbSamModel()
        self._gsmf._pack(m)
        self._mmbulge._pack(m)
        if self._gmr is None:
            m.rate_kind = N.RATE_GPF_GMT
            self._gpf._pack(m)
        else:
            m.rate_kind = N.RATE_GMR
            self._gmr._pack(m)
        m.use_gmt = int(self._gmt is not None)
        if self._gmt is not None:
            self._gmt._pack(m)
        m.gsmf_uses_mtot = int(GSMF_USES_MTOT)
        m.gpf_uses_mtot = int(GPF_USES_MTOT)
        m.gmt_uses_mtot = int(GMT_USES_MTOT)
        return m

    def _density_device(self):
        """Device (density, gmt_time or None, redz_prime or None), computed once per instance."""
        if self._density_t is not None:
            return self._density_t, self._gmt_time_t, self._redz_prime_t
        dens, gmt_time, redz_prime = self._static_density_launch()
        self._scatter_finish(dens, gmt_time, redz_prime)
        return dens, gmt_time, redz_prime

    def _static_density_launch(self):
        """The static density before the M-Mbulge scatter, with gmt_time and redz_prime."""
        import ctypes
        t = D.torch()
        mt, mr, rz = self._edges_device()
        dev = mt.device
        dc = D.device_cosmology(self._cosmo, dev)
        dens = t.empty(self.shape, dtype=t.float64, device=dev)
        gmt_time = redz_prime = None
        if self._gmt is not None:
            gmt_time = t.empty(self.shape, dtype=t.float64, device=dev)
            redz_prime = t.empty(self.shape, dtype=t.float64, device=dev)
        model = self._model_struct()
        st = D.StatusWord(dev)
        N.call("hgb_static_density", ctypes.byref(model), dc.ref, N.ptr(mt), mt.numel(), N.ptr(mr), mr.numel(),
               N.ptr(rz), rz.numel(), N.ptr(dens), N.ptr(gmt_time), N.ptr(redz_prime), st.ptr, N.stream_handle())
        return dens, gmt_time, redz_prime

    def _scatter_finish(self, dens, gmt_time, redz_prime):
        """Scatter and stalled-bin zeroing in place; caches the final density on the instance."""
        scatter = self._mmbulge._scatter_dex
        if scatter > 0.0:
            from . import scatter as _scatter
            _scatter.add_scatter_to_masses_device(self.mtot, self.mrat, dens, scatter)
        if redz_prime is not None:
            N.call("hgb_zero_stalled", N.ptr(dens), N.ptr(redz_prime), int(dens.numel()), N.stream_handle())
        self._density_t, self._gmt_time_t, self._redz_prime_t = dens, gmt_time, redz_prime
        return dens

    @property
    def static_binary_density(self):
        """d^3 n / [dlog10 M dq dz] at the grid edges, (M, Q, Z) [Mpc^-3] (numpy copy)."""
        if self._density is None:
            self._density = D.to_host(self._density_device()[0])
        return self._density

    @property
    def _gmt_time(self):
        if self._gmt_time_host is None:
            g = self._density_device()[1]
            self._gmt_time_host = None if g is None else D.to_host(g)
        return self._gmt_time_host

    @property
    def _redz_prime(self):
        if self._redz_prime_host is None:
            z = self._density_device()[2]
            self._redz_prime_host = None if z is None else D.to_host(z)
        return self._redz_prime_host

    # ---- differential number at target frequencies (sam.py:400-466, sam_cyutils.pyx:421-504)

    def _dbn_device(self, hard, fobs_orb, cosmo=None, precision="fp64"):
        t = D.torch()
        cosmo = self._cosmo if cosmo is None else cosmo
        dens, gmt_time, redz_prime = self._density_device()
        mt, mr, rz = self._edges_device()
        if isinstance(hard, hardening.Fixed_Time_2PL_SAM):
            if gmt_time is None:
                gmt_time = t.zeros(self.shape, dtype=t.float64, device=dens.device)
            return sam_cyutils.dbn_2pwl_device(fobs_orb, hard, dens, mt, mr, rz, gmt_time, cosmo=cosmo,
                                               precision=precision)
        if isinstance(hard, hardening.Hard_GW) or (isinstance(hard, type) and issubclass(hard, hardening.Hard_GW)):
            if redz_prime is None:
                redz_prime = rz[None, None, :].expand(self.shape).contiguous()
            return sam_cyutils.dbn_gw_device(fobs_orb, dens, mt, mr, redz_prime, cosmo=cosmo)
        raise ValueError(f"Unexpected `hard` value {hard}!")

    def _dbn_2pwl_overlapped(self, hard, fobs_orb, precision="fp64"):
        """_dbn_device for Fixed_Time_2PL_SAM on a fresh instance, with the separation-step walk (which
        needs gmt_time but not the density) on a second stream while a high-priority third stream
        applies the M-Mbulge scatter; the evaluation, which needs the final density, follows on the
        current stream.  Same results as _dbn_device."""
        t = D.torch()
        dens, gmt_time, redz_prime = self._static_density_launch()
        mt, mr, rz = self._edges_device()
        main = t.cuda.current_stream()
        side = D.side_stream("dbn_walk", main.device)
        static_done = t.cuda.Event()
        static_done.record(main)
        side.wait_event(static_done)
        with t.cuda.stream(side), D.nvtx("hgb:dbn_step_walk"):
            redz_final, diff_num = sam_cyutils.dbn_2pwl_device(fobs_orb, hard, None, mt, mr, rz, gmt_time,
                                                               cosmo=self._cosmo, phase=1)
            walk_done = t.cuda.Event()
            walk_done.record(side)
        gmt_time.record_stream(side)
        # the scatter's gradient solve is one latency-bound block per redshift slice: on a
        # high-priority stream its blocks take SMs as the hardening normalisation's blocks retire,
        # and the normalisation and the walk fill the rest
        hi = D.side_stream("mbulge_scatter", main.device, priority=-1)
        hi.wait_event(static_done)
        with t.cuda.stream(hi), D.nvtx("hgb:mbulge_scatter"):
            self._scatter_finish(dens, gmt_time, redz_prime)
            scatter_done = t.cuda.Event()
            scatter_done.record(hi)
        for x in (dens, gmt_time, redz_prime):
            if x is not None:
                x.record_stream(hi)
        main.wait_event(scatter_done)
        main.wait_event(walk_done)
        redz_final.record_stream(main)
        diff_num.record_stream(main)
        return sam_cyutils.dbn_2pwl_device(fobs_orb, hard, dens, mt, mr, rz, gmt_time, cosmo=self._cosmo, phase=2,
                                           out=(redz_final, diff_num), precision=precision)

    def _dbn_scheduled(self, hard, fobs_orb, precision="fp64"):
        """_dbn_device, overlapping the separation-step walk with the scatter where that applies."""
        if (self._density_t is None and self._gmt is not None and isinstance(hard, hardening.Fixed_Time_2PL_SAM)
                and self._mmbulge._scatter_dex > 0.0):
            return self._dbn_2pwl_overlapped(hard, fobs_orb, precision=precision)
        return self._dbn_device(hard, fobs_orb, precision=precision)

    def dynamic_binary_number_at_fobs(self, hard, fobs_orb, use_cython=True, **kwargs):
        """(grid, dnum, redz_final) like sam.py:400-466 (``use_cython`` is accepted and ignored)."""
        redz_final, dnum = self._dbn_device(hard, fobs_orb)
        grid = [self.mtot, self.mrat, self.redz, np.asarray(fobs_orb)]
        return grid, D.to_host(dnum), D.to_host(redz_final)

    # ---- GWB (sam.py:872-947)

    def gwb_device(self, fobs_gw_edges, hard=None, realize=100, loudest=1, seed=None, replay=None, order=None,
                   params=False, precision="fp64"):
        """Device (hc_ss[F, R, L], hc_bg[F, R]) tensors, plus (sspar, bgpar) with ``params``; see :meth:`gwb`."""
        hard = hardening.Hard_GW() if hard is None else hard
        sam_cyutils.check_precision(precision)
        if not isinstance(hard, (hardening.Fixed_Time_2PL_SAM, hardening.Hard_GW)):
            raise ValueError("`sam_cyutils` methods only work with `Fixed_Time_2PL_SAM` or `Hard_GW` hardening "
                             "models!  Use `gwb_only` for alternative classes!")
        if not utils.isinteger(realize):
            raise Exception("`realize` ({}) must be an integer!")
        fobs_gw_edges = np.asarray(fobs_gw_edges, dtype=np.float64)
        fobs_gw_cents = utils.midpoints(fobs_gw_edges)
        fobs_orb_edges = fobs_gw_edges / 2.0
        fobs_orb_cents = fobs_gw_cents / 2.0
        with D.nvtx("hgb:density_scatter_dbn"):
            redz_final, diff_num = self._dbn_scheduled(hard, fobs_orb_cents, precision=precision)
        with D.nvtx("hgb:number_and_strain"):
            number, h2fdf = self._number_and_strain(fobs_orb_edges, diff_num, redz_final, precision=precision)
        with D.nvtx("hgb:realizations"):
            if params:
                edges = [self.mtot, self.mrat, self.redz, fobs_orb_edges]
                return single_sources.ss_params_device(edges, redz_final, number, h2fdf, realize, loudest,
                                                       seed=seed, replay=replay, order=order, cosmo=self._cosmo)
            return single_sources.ss_realize_device(number, h2fdf, realize, loudest, seed=seed, replay=replay,
                                                    order=order)

    def _number_and_strain(self, fobs_orb_edges, diff_num, redz_final, status=None, precision="fp64"):
        """Device (number, h2fdf) on the (M-1, Q-1, Z-1, F) bins.  With ``status`` the redshift check
        is left to the caller (no host read here).  ``precision="fp32"``: hgb_number_and_strain_f32."""
        t = D.torch()
        mt, mr, rz = self._edges_device()
        lm = D.as_device(np.log10(self.mtot))
        fe = D.as_device(fobs_orb_edges)
        dlnf = D.as_device(np.diff(np.log(fobs_orb_edges)))
        dc = D.device_cosmology(self._cosmo, mt.device)
        nm, nq, nz = self.shape
        nf = int(dlnf.numel())
        number = t.empty((nm - 1, nq - 1, nz - 1, nf), dtype=t.float64, device=mt.device)
        h2fdf = t.empty_like(number)
        st = D.StatusWord(mt.device) if status is None else status
        fn = "hgb_number_and_strain" if sam_cyutils.check_precision(precision) == "fp64" else "hgb_number_and_strain_f32"
        N.call(fn, N.ptr(mt), N.ptr(lm), nm, N.ptr(mr), nq, N.ptr(rz), nz, N.ptr(fe),
               N.ptr(dlnf), nf, N.ptr(diff_num), N.ptr(redz_final), C.GW_SRC_CONST, dc.ref, N.ptr(number),
               N.ptr(h2fdf), st.ptr, N.stream_handle())
        if status is None:
            single_sources.check_redshift_status(st)
        return number, h2fdf

    def gwb(self, fobs_gw_edges, hard=None, realize=100, loudest=1, params=False, seed=None, replay=None,
            order=None, return_torch=False, precision="fp64"):
        """Characteristic strain of the L loudest sources (F, R, L) and of the background (F, R), and
        with ``params=True`` the loudest sources' (M, q, z, z_final) (4, F, R, L) and the background's
        weighted-mean parameters (7, F, R).

        Same arguments and results as sam.py:872-947.  Added keywords: ``seed`` (Philox key; default
        fresh entropy), ``replay``/``order`` (replay an externally drawn Poisson stream bit for bit),
        ``return_torch`` (keep the results on the device), ``precision``: "fp64" (default, the parity
        mode: every grid stage in FP64) or "fp32" (the production mode: the residence-time evaluation,
        the cell integration and the strain in FP32 with compensated sums; the hardening integral, the
        age -> redshift inversion and the static density stay FP64; relative error of the grids about
        1e-6, see hgb_number_and_strain_f32 / hgb_dbn_2pwl_phase_f32).
        """
        out = self.gwb_device(fobs_gw_edges, hard=hard, realize=realize, loudest=loudest, seed=seed,
                              replay=replay, order=order, params=params, precision=precision)
        if return_torch:
            return out
        return tuple(D.to_host(x) for x in out)
