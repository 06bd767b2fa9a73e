"""M_bh - M_bulge relations and bulge fractions of the SAM path (holodeck/host_relations.py).

The classes hold parameters with holodeck's names and defaults; the arithmetic that uses them
(mstar_from_mbh, dmstar_dmbh, the density Jacobian) runs in the density kernel
(``csrc/hgb_density.cu``).
"""

import numpy as np

from . import constants as C


class _Bulge_Frac:
    pass


class BF_Constant(_Bulge_Frac):
    """Constant stellar-bulge mass fraction, host_relations.py:166-195."""

    def __init__(self, bulge_frac=0.69):
        if not (0.0 < bulge_frac <= 1.0):
            raise AssertionError("bulge_frac must be in (0, 1]")
        self._bulge_mass_frac = bulge_frac

    def bulge_frac(self, *args, **kwargs):
        return self._bulge_mass_frac


class _MMBulge_Relation:
    BULGE_MASS_FRAC = 0.615

    def __init__(self, bulge_frac=None, bulge_mfrac=None):
        if bulge_mfrac is not None:
            if bulge_frac is not None:
                raise ValueError("Cannot provide both a ``bulge_mfrac`` and ``bulge_frac``!")
            bulge_frac = BF_Constant(bulge_mfrac)
        if bulge_frac is None:
            bulge_frac = BF_Constant(self.BULGE_MASS_FRAC)
        if not isinstance(bulge_frac, BF_Constant):
            raise NotImplementedError("Only a constant bulge fraction (BF_Constant) is on the GPU SAM path")
        self._bulge_frac = bulge_frac


class MMBulge_Standard(_MMBulge_Relation):
    """Single power-law M_bh - M_bulge relation, host_relations.py:624-771."""

    MASS_AMP_LOG10 = 8.17
    MASS_PLAW = 1.01
    MASS_REF = 1.0e11 * C.MSOL
    SCATTER_DEX = 0.3
    BULGE_MASS_FRAC = 0.615

    def __init__(self, mamp_log10=None, mplaw=None, mref=None, scatter_dex=None, bulge_frac=None,
                 bulge_mfrac=None, **kwargs):
        if "mamp" in kwargs:
            if mamp_log10 is not None:
                raise ValueError("Both `mamp` (deprecated!) and `mamp_log10` have been given!  Cannot correct.")
            mamp_log10 = np.log10(kwargs.pop("mamp") / C.MSOL)
        super().__init__(bulge_frac=bulge_frac, bulge_mfrac=bulge_mfrac)
        if mamp_log10 is None:
            mamp_log10 = self.MASS_AMP_LOG10
        self._mamp = C.MSOL * np.power(10.0, mamp_log10)
        self._mplaw = self.MASS_PLAW if mplaw is None else mplaw
        self._mref = self.MASS_REF if mref is None else mref
        self._scatter_dex = self.SCATTER_DEX if scatter_dex is None else scatter_dex

    def _pack(self, model):
        model.mmb[0] = self._mamp
        model.mmb[1] = self._mplaw
        model.mmb[2] = self._mref
        model.mmb[3] = self._bulge_frac.bulge_frac()


class MMBulge_KH2013(MMBulge_Standard):
    """Kormendy & Ho 2013 Eq.10 values, host_relations.py:774-784."""

    MASS_AMP_LOG10 = 8.69
    MASS_REF = C.MSOL * 1e11
    MASS_PLAW = 1.17
    SCATTER_DEX = 0.28


class MMBulge_MM2013(MMBulge_Standard):
    """McConnell & Ma 2013 values, host_relations.py:787-797."""

    MASS_AMP_LOG10 = 8.46
    MASS_REF = C.MSOL * 1e11
    MASS_PLAW = 1.05
    SCATTER_DEX = 0.34
