"""holodeck_gb300: GB300-native (sm_103a) semi-analytic-model gravitational-wave background.

A drop-in for holodeck's ``Semi_Analytic_Model.gwb()`` / ``single_sources.ss_gws_redz()`` path:
the same classes, arguments and returned arrays, computed by hand-written CUDA kernels behind the
C ABI of ``include/holodeck_gb300.h``.  There is no CPU fallback; without the built extension or a
CUDA device the compute calls raise.
"""

import logging

from . import constants  # noqa
from .cosmology import cosmo, Cosmology  # noqa

log = logging.getLogger("holodeck_gb300")

from . import utils  # noqa: E402
from . import host_relations, hardening  # noqa: E402
from . import cyutils, gravwaves, single_sources  # noqa: E402
from . import sams  # noqa: E402
from . import librarian  # noqa: E402

__version__ = "0.1.0"
