"""Import stand-in for the package around the reference's compiled Cython modules.

TEST INFRASTRUCTURE ONLY.  ``oracle/ref_build.py`` writes :data:`PACKAGE_INIT` as the ``holodeck``
package ``__init__`` next to the modules it compiles.  The compiled ``sam_cyutils`` looks up two
names in its package at run time (sam_cyutils.pyx:465, :483: the isinstance dispatch on the
hardening model); everything else the reference's Cython code needs comes in through arguments.
:func:`reference_gwb_stages` then drives those compiled kernels with the oracle's restatement of
the reference's Python glue (sam.py:872-947, single_sources.py:40-174).
"""

import time

import numpy as np

PACKAGE_INIT = '''"""Import stand-in (oracle/ref_stub.py): the names the compiled holodeck modules look up."""
import types


class Fixed_Time_2PL_SAM:
    """Carrier of the hardening parameters sam_cyutils.dynamic_binary_number_at_fobs reads."""


class Hard_GW:
    """GW-only hardening marker."""


hardening = types.SimpleNamespace(Fixed_Time_2PL_SAM=Fixed_Time_2PL_SAM, Hard_GW=Hard_GW)
'''


class _Sam:
    """The attributes of a Semi_Analytic_Model that sam_cyutils.dynamic_binary_number_at_fobs reads."""

    def __init__(self, mtot, mrat, redz, density, gmt_time):
        self.mtot, self.mrat, self.redz = mtot, mrat, redz
        self.static_binary_density = density
        self._gmt_time = gmt_time
        self._redz_prime = None
        self.shape = (mtot.size, mrat.size, redz.size)


def reference_gwb_stages(shape, nfreqs, nreals, nloudest, seed, scatter_dex=0.28, keep=None):
    """One evaluation of the plain-SAM workload through the reference's compiled kernels: the static
    density with M-Mbulge scatter (the oracle's restatement of sam.py:280-398, which runs scipy's
    interpolators as the reference does), the hardening normalisation
    (``sam_cyutils.find_2pwl_hardening_norm``), the differential number
    (``sam_cyutils.dynamic_binary_number_at_fobs``), the integration
    (``sam_cyutils.integrate_differential_number_3dx1d``), the strain (the oracle's
    gravwaves.py:694-724), numpy's loudest-first argsort and ``nreals`` realizations
    (``cyutils.loudest_hc_from_sorted`` with a seeded PCG64).  Returns the seconds per stage; ``keep``
    (a dict) receives the edges, frequency edges, redz_final, number, h2fdf and order."""
    from holodeck_gb300 import constants as C
    from oracle import ref_build
    from oracle import sam_oracle as O
    cyutils, sam_cyutils = ref_build.load()
    import holodeck
    t = {}
    t0 = time.perf_counter()
    mtot, mrat, redz = O.grid_edges(shape)
    p = O.default_params(scatter_dex=scatter_dex)
    parts = O.static_binary_density(mtot, mrat, redz, p, return_parts=True)
    t["density_and_scatter"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    mt, mr = np.meshgrid(mtot, mrat, indexing="ij")
    norm_log10 = sam_cyutils.find_2pwl_hardening_norm(3.0 * C.GYR, mt.ravel(), mr.ravel(), 1.0e3 * C.PC,
                                                      100.0 * C.PC, -1.0, 2.5, 300)
    t["hardening_norm"] = time.perf_counter() - t0
    hard = holodeck.hardening.Fixed_Time_2PL_SAM()
    hard._norm = 10.0 ** np.asarray(norm_log10).reshape(mt.shape)
    hard._sepa_init, hard._num_steps, hard._rchar = 1.0e3 * C.PC, 300, 100.0 * C.PC
    hard._gamma_inner, hard._gamma_outer = -1.0, 2.5
    _, fe = O.pta_freqs(16.0 * C.YR, nfreqs)
    fo_c = O.midpoints(fe) / 2.0
    sam = _Sam(mtot, mrat, redz, parts["density"], parts["gmt_time"])
    t0 = time.perf_counter()
    redz_final, dnum = sam_cyutils.dynamic_binary_number_at_fobs(fo_c, sam, hard, p["cosmo"])
    t["dbn"] = time.perf_counter() - t0
    edges = [mtot, mrat, redz, fe / 2.0]
    t0 = time.perf_counter()
    number = sam_cyutils.integrate_differential_number_3dx1d(edges, dnum)
    t["integrate"] = time.perf_counter() - t0
    del dnum
    t0 = time.perf_counter()
    h2fdf = O.char_strain_sq_from_bin_edges_redz(edges, redz_final, cosmo=p["cosmo"])
    t["strain"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    order = np.argsort(-h2fdf[..., 0].flatten())
    msort, qsort, zsort = np.unravel_index(order, number.shape[:3])
    t["sort"] = time.perf_counter() - t0
    cyutils.PCG64 = lambda: np.random.PCG64(seed)
    t0 = time.perf_counter()
    cyutils.loudest_hc_from_sorted(number, h2fdf, nreals, nloudest, msort, qsort, zsort)
    t["realizations"] = time.perf_counter() - t0
    if keep is not None:
        keep.update(edges=[mtot, mrat, redz], fobs_gw_edges=fe, redz_final=redz_final, number=number, h2fdf=h2fdf,
                    order=order)
    return t
