"""Library runs of the SAM on the GPU (holodeck/librarian): one model evaluation with every output
a library file holds (:func:`lib_tools.run_model`), the model details (:func:`lib_tools._calc_model_details`)
and a writer for the combined-library layout (:func:`lib_tools.write_library`)."""

DEF_NUM_REALS = 100     #: realizations per library sample (librarian/__init__.py:48)
DEF_NUM_FBINS = 40      #: frequency bins (librarian/__init__.py:49)
DEF_NUM_LOUDEST = 5     #: loudest binaries per frequency bin (librarian/__init__.py:50)
DEF_PTA_DUR = 16.03     #: PTA duration setting the Nyquist frequency bins [yr] (librarian/__init__.py:51)

from . import lib_tools  # noqa: E402,F401
from .lib_tools import run_model, write_library  # noqa: E402,F401
