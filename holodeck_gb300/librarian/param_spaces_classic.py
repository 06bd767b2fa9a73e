"""The classic phenomenological parameter spaces of holodeck/librarian/param_spaces_classic.py.

``_PS_Classic_Phenom`` holds the default settings and the mapping from library parameters to a SAM
(GSMF_Schechter, GPF_Power_Law, GMT_Power_Law, MMBulge_KH2013) and a Fixed_Time_2PL_SAM hardening
(param_spaces_classic.py:12-84); ``PS_Classic_Phenom_Uniform`` is its 6-parameter uniform box
(param_spaces_classic.py:87-107).  Times are given in Gyr and lengths in pc, as in the reference.
"""

from .. import hardening, host_relations, sams
from ..constants import GYR, PC
from .lib_tools import PD_Uniform, _Param_Space


class _PS_Classic_Phenom(_Param_Space):
    """Defaults and model construction of the classic phenomenological spaces."""

    DEFAULTS = dict(
        hard_time=3.0,          # [Gyr]
        hard_sepa_init=1e4,     # [pc]
        hard_rchar=100.0,       # [pc]
        hard_gamma_inner=-1.0,
        hard_gamma_outer=+2.5,
        gsmf_phi0_log10=-2.77,
        gsmf_phiz=-0.6,
        gsmf_mchar0_log10=11.24,
        gsmf_mcharz=0.11,
        gsmf_alpha0=-1.21,
        gsmf_alphaz=-0.03,
        gpf_frac_norm_allq=0.025,
        gpf_malpha=0.0,
        gpf_qgamma=0.0,
        gpf_zbeta=1.0,
        gpf_max_frac=1.0,
        gmt_norm=0.5,           # [Gyr]
        gmt_malpha=0.0,
        gmt_qgamma=-1.0,
        gmt_zbeta=-0.5,
        mmb_mamp_log10=8.69,
        mmb_plaw=1.10,
        mmb_scatter_dex=0.3,
    )

    @classmethod
    def _init_sam(cls, sam_shape, params):
        gsmf = sams.GSMF_Schechter(phi0=params['gsmf_phi0_log10'], phiz=params['gsmf_phiz'],
                                   mchar0_log10=params['gsmf_mchar0_log10'], mcharz=params['gsmf_mcharz'],
                                   alpha0=params['gsmf_alpha0'], alphaz=params['gsmf_alphaz'])
        gpf = sams.GPF_Power_Law(frac_norm_allq=params['gpf_frac_norm_allq'], malpha=params['gpf_malpha'],
                                 qgamma=params['gpf_qgamma'], zbeta=params['gpf_zbeta'],
                                 max_frac=params['gpf_max_frac'])
        gmt = sams.GMT_Power_Law(time_norm=params['gmt_norm'] * GYR, malpha=params['gmt_malpha'],
                                 qgamma=params['gmt_qgamma'], zbeta=params['gmt_zbeta'])
        mmbulge = host_relations.MMBulge_KH2013(mamp_log10=params['mmb_mamp_log10'], mplaw=params['mmb_plaw'],
                                                scatter_dex=params['mmb_scatter_dex'])
        return sams.Semi_Analytic_Model(gsmf=gsmf, gpf=gpf, gmt=gmt, mmbulge=mmbulge, shape=sam_shape)

    @classmethod
    def _init_hard(cls, sam, params):
        return hardening.Fixed_Time_2PL_SAM(sam, params['hard_time'] * GYR, sepa_init=params['hard_sepa_init'] * PC,
                                            rchar=params['hard_rchar'] * PC,
                                            gamma_inner=params['hard_gamma_inner'],
                                            gamma_outer=params['hard_gamma_outer'])


class PS_Classic_Phenom_Uniform(_PS_Classic_Phenom):
    """The 6-parameter uniform box of the 15-year analysis ('phenom-uniform')."""

    def __init__(self, log=None, nsamples=None, sam_shape=None, seed=None):
        parameters = [
            PD_Uniform("gsmf_phi0_log10", -3.5, -1.5),
            PD_Uniform("gsmf_mchar0_log10", 10.5, 12.5),   # [log10(Msol)]
            PD_Uniform("mmb_mamp_log10", +7.6, +9.0),      # [log10(Msol)]
            PD_Uniform("mmb_scatter_dex", +0.0, +0.9),
            PD_Uniform("hard_time", 0.1, 11.0),            # [Gyr]
            PD_Uniform("hard_gamma_inner", -1.5, +0.0),
        ]
        super().__init__(parameters, log=log, nsamples=nsamples, sam_shape=sam_shape, seed=seed)


param_spaces_dict = {
    "PS_Classic_Phenom_Uniform": PS_Classic_Phenom_Uniform,
}
