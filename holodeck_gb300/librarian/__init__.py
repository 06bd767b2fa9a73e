"""Library runs of the SAM on the GPU (holodeck/librarian): one model evaluation with every output
a library file holds (:func:`lib_tools.run_model`), the model details (:func:`lib_tools._calc_model_details`),
the parameter spaces that define a library (:mod:`lib_tools`, :mod:`param_spaces_classic`), batched
runs of a whole library on one GPU (:func:`batch.run_library`) and a writer for the combined-library
layout (:func:`lib_tools.write_library`)."""

DEF_NUM_REALS = 100     #: realizations per library sample (librarian/__init__.py:48)
DEF_NUM_FBINS = 40      #: frequency bins (librarian/__init__.py:49)
DEF_NUM_LOUDEST = 5     #: loudest binaries per frequency bin (librarian/__init__.py:50)
DEF_PTA_DUR = 16.03     #: PTA duration setting the Nyquist frequency bins [yr] (librarian/__init__.py:51)

from . import lib_tools  # noqa: E402,F401
from .lib_tools import PD_Normal, PD_Uniform, run_model, write_library  # noqa: E402,F401
from . import param_spaces_classic  # noqa: E402,F401
from .param_spaces_classic import PS_Classic_Phenom_Uniform, param_spaces_dict  # noqa: E402,F401
from . import batch  # noqa: E402,F401
from .batch import run_library  # noqa: E402,F401
