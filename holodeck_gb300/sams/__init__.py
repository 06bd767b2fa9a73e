"""Semi-analytic models (holodeck.sams) on the GPU."""

from . import components, sam, sam_cyutils  # noqa
from .sam import Semi_Analytic_Model  # noqa
from .components import (GSMF_Schechter, GSMF_Double_Schechter, GPF_Power_Law, GMT_Power_Law,  # noqa
                         GMR_Illustris)
