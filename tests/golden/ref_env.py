"""Build and import the holodeck reference for generating golden fixtures.

This helper runs only in a development container that holds the holodeck
sources.  Two environment variables are required: ``HOLODECK_REF_SRC``, the
root of the holodeck source tree (it holds ``holodeck/`` and ``setup.py``),
and ``HOLODECK_REF_BUILD``, a scratch directory outside this repository for
the patched copy and its build.  It is not used by the tests: they read the
committed ``.npz`` fixtures.

Steps, all in a scratch directory outside the repository:

1. copy ``holodeck/`` plus ``setup.py``/``README.md``/``requirements.txt``;
2. apply the one-token Cython-3 fix ``long(normal_threshold)`` ->
   ``int(normal_threshold)`` (holodeck/cyutils.pyx:855; Cython 3 has no
   ``long`` builtin and Cython<3 is not installable offline);
3. ``python setup.py build_ext -i`` (the reference's own extension recipe);
4. put import stand-ins on ``sys.path`` for packages the SAM path imports but
   that are not installed: ``cosmopy`` (backed by
   :mod:`holodeck_gb300.cosmology`, so reference and GPU share one cosmology),
   ``astropy`` (constants only), ``kalepy`` (``utils.midpoints`` as the
   arithmetic mean of neighbours), and import-only ``h5py``/``numba``/
   ``matplotlib``.
"""

import os
import shutil
import subprocess
import sys

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))


def _required_dir(name):
    val = os.environ.get(name)
    if not val:
        raise RuntimeError(f"set {name} (see the module docstring of tests/golden/ref_env.py)")
    return os.path.abspath(val)


REF_SRC = _required_dir("HOLODECK_REF_SRC")
BUILD_DIR = _required_dir("HOLODECK_REF_BUILD")
if os.path.commonpath([BUILD_DIR, REPO]) == REPO:
    raise RuntimeError("HOLODECK_REF_BUILD must lie outside the repository")

_STUBS = {
    "cosmopy/__init__.py": '''
import numpy as np
from holodeck_gb300.cosmology import Cosmology as _Base
from holodeck_gb300 import constants as _C

_TO_SEC = {"s": 1.0, "Gyr": _C.GYR, "yr": _C.YR, "Myr": _C.MYR}
_TO_CM = {"cm": 1.0, "Mpc": _C.MPC, "kpc": _C.KPC, "pc": _C.PC}


class _Q:
    """Minimal stand-in for an astropy Quantity holding a value in base cgs units."""

    def __init__(self, value, kind):
        self._v = np.asarray(value) if np.ndim(value) else float(value)
        self._kind = kind

    def to(self, unit):
        table = _TO_SEC if self._kind == "time" else _TO_CM
        return _Q(self._v / table[unit], "plain")

    @property
    def value(self):
        return self._v

    @property
    def cgs(self):
        return _Q(self._v, "plain")


class Cosmology(_Base):
    def age(self, z):
        return _Q(super().age(z), "time")

    def comoving_distance(self, z):
        return _Q(super().comoving_distance(z), "dist")

    def tage_to_z(self, age):
        return _Base.tage_to_z(self, age)
''',
    "astropy/__init__.py": '''
from . import constants, units  # noqa
''',
    "astropy/constants.py": '''
class _C:
    def __init__(self, v):
        self.value = v
        self.cgs = self
        self.gauss = self

G = _C(6.6743e-08)
c = _C(29979245800.0)
m_e = _C(9.1093837015e-28)
m_p = _C(1.67262192369e-24)
e = _C(4.803204712570263e-10)
k_B = _C(1.380649e-16)
h = _C(6.62607015e-27)
sigma_sb = _C(5.6703744191844314e-05)
sigma_T = _C(6.6524587321e-25)
M_sun = _C(1.988409870698051e+33)
L_sun = _C(3.828e+33)
R_sun = _C(69570000000.0)
pc = _C(3.085677581491367e+18)
au = _C(14959787070000.0)
''',
    "astropy/units.py": '''
class _U:
    def __init__(self, s):
        self.s = s
        self.scale = s
        self.cgs = self
    def to(self, other):
        return self.s / other.s
    def __truediv__(self, o):
        return _U(self.s / o.s)
    def __mul__(self, o):
        return _U(self.s * o.s)
    def __pow__(self, p):
        return _U(self.s ** p)

s = _U(1.0)
cm = _U(1.0)
km = _U(1.0e5)
g = _U(1.0)
erg = _U(1.0)
arcsec = _U(4.84813681109536e-06)
year = _U(31557600.0)
eV = _U(1.602176634e-12)
jansky = _U(1.0e-23)
''',
    "kalepy/__init__.py": '''
from . import utils  # noqa
def sample_grid(*a, **k):
    raise NotImplementedError
def sample_outliers(*a, **k):
    raise NotImplementedError
''',
    "kalepy/utils.py": '''
import numpy as np
def midpoints(arr, axis=-1, **kwargs):
    arr = np.moveaxis(np.asarray(arr), axis, -1)
    mid = 0.5 * (arr[..., 1:] + arr[..., :-1])
    return np.moveaxis(mid, -1, axis)
''',
    "h5py/__init__.py": "",
    "numba/__init__.py": '''
def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f
jit = njit
''',
    "matplotlib/__init__.py": '''
import types as _t
class _Any:
    def __getattr__(self, k):
        if k[:1].isupper():
            return type(k, (), {"__init__": lambda self, *a, **kw: None})
        return _Any()
    def __call__(self, *a, **k):
        return _Any()
    def __setitem__(self, k, v):
        pass
    def __getitem__(self, k):
        return _Any()
rcParams = _Any()
style = _Any()
colors = _Any()
def __getattr__(name):
    return _Any()
''',
    "matplotlib/pyplot.py": '''
from matplotlib import _Any
rcParams = _Any()
def __getattr__(name):
    return _Any()
''',
    "matplotlib/cm.py": '''
from matplotlib import _Any
def __getattr__(name):
    return _Any()
''',
}


def _write_stubs(root):
    for rel, text in _STUBS.items():
        path = os.path.join(root, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as fh:
            fh.write(text)


def build():
    """Copy, patch and build the reference; return the directory to put on ``sys.path``."""
    src = os.path.join(BUILD_DIR, "src")
    stamp = os.path.join(BUILD_DIR, ".built")
    if not os.path.exists(stamp):
        if os.path.isdir(BUILD_DIR):
            shutil.rmtree(BUILD_DIR)
        os.makedirs(src)
        shutil.copytree(os.path.join(REF_SRC, "holodeck"), os.path.join(src, "holodeck"))
        for fn in ["setup.py", "README.md", "requirements.txt"]:
            shutil.copy(os.path.join(REF_SRC, fn), os.path.join(src, fn))
        pyx = os.path.join(src, "holodeck", "cyutils.pyx")
        for fn in [pyx]:
            os.chmod(fn, 0o644)
        text = open(pyx).read()
        assert text.count("long(normal_threshold)") == 1
        text = text.replace("long(normal_threshold)", "int(normal_threshold)")
        with open(pyx, "w") as fh:
            fh.write(text)
        for dirpath, dirnames, filenames in os.walk(src):
            os.chmod(dirpath, 0o755)
            for fn in filenames:
                os.chmod(os.path.join(dirpath, fn), 0o644)
        subprocess.run([sys.executable, "setup.py", "build_ext", "-i"], cwd=src, check=True,
                       stdout=subprocess.DEVNULL)
        open(stamp, "w").close()
    stubs = os.path.join(BUILD_DIR, "stubs")
    _write_stubs(stubs)
    return src, stubs


def import_reference():
    """Build if needed and import ``holodeck`` from the scratch copy."""
    src, stubs = build()
    for p in [REPO, stubs, src]:
        if p not in sys.path:
            sys.path.insert(0, p)
    import holodeck  # noqa
    import holodeck.sams  # noqa
    import holodeck.hardening  # noqa
    import holodeck.single_sources  # noqa
    import holodeck.cyutils  # noqa
    import holodeck.sams.sam_cyutils  # noqa
    return holodeck
