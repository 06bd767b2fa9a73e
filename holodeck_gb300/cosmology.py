"""Flat Lambda-CDM cosmology used by the SAM path (host side).

holodeck takes its cosmology from the third-party ``cosmopy`` package
(holodeck/__init__.py:81-85: ``cosmopy.Cosmology(h=0.6933, Om0=0.2880,
Ob0=0.0472, size=200)``).  ``cosmopy`` is not vendored in holodeck and its
version is not pinned (requirements.txt:2), so its exact arithmetic is not
available.  This module restates the quantities the SAM path reads from it,
for a flat universe with matter + Lambda and no radiation (astropy's
``FlatLambdaCDM`` default ``Tcmb0=0``):

* ``age(z)``             closed form  t(z) = 2/(3 H0 sqrt(OL)) asinh(sqrt(OL/Om) (1+z)^-3/2)
* ``tage_to_z(t)``       the exact inverse of ``age``
* ``dtdz(z)``            |dt/dz| = 1 / (H0 (1+z) E(z)),  E(z) = sqrt(Om (1+z)^3 + OL)
* ``comoving_distance``  D_C = (c/H0) int_{sqrt(a)}^1 2 du / sqrt(Om + OL u^6),  a = 1/(1+z),
  evaluated by 32-point Gauss-Legendre quadrature (the integrand is analytic
  on [0, 1], so the rule is accurate to ~1e-15 relative).
* ``_grid_z`` / ``_grid_age`` / ``_grid_dcom``: the 200-entry interpolation
  tables that the Cython kernels consume (sam_cyutils.pyx:476, :494).  The
  redshift grid is decreasing (sam_cyutils.pyx:567-570 rely on that) and ends
  at z=0 so that the last age is the age of the Universe.

The same tables, constants and quadrature nodes are handed to the CUDA
kernels, so host and device evaluate one definition.
"""

import numpy as np

from . import constants as C

_GL_ORDER = 32


class Cosmology:
    """Flat matter + Lambda cosmology with the interpolation tables the SAM kernels use."""

    def __init__(self, h=0.6933, Om0=0.2880, Ob0=0.0472, size=200, zmax=1.0e4, zmin_log=1.0e-4):
        if size < 3:
            raise ValueError(f"`size`={size} must be at least 3")
        self.h = float(h)
        self.Om0 = float(Om0)
        self.Ob0 = float(Ob0)
        self.Ode0 = 1.0 - self.Om0
        #: Hubble constant [1/s]
        self.H0 = self.h * 100.0 * C.KMPERSEC / C.MPC
        #: Hubble distance c/H0 [cm]
        self.hubble_distance = C.SPLC / self.H0
        nodes, weights = np.polynomial.legendre.leggauss(_GL_ORDER)
        self.gl_nodes = nodes.astype(np.float64)
        self.gl_weights = weights.astype(np.float64)

        grid_z = np.concatenate([np.logspace(np.log10(zmax), np.log10(zmin_log), size - 1), [0.0]])
        self._grid_z = grid_z
        self._grid_age = Cosmology.age(self, grid_z)
        self._grid_dcom = Cosmology.comoving_distance(self, grid_z)
        self._age_universe = float(Cosmology.age(self, 0.0))

    # ---- closed forms

    def efunc(self, z):
        zp1 = 1.0 + np.asarray(z, dtype=np.float64)
        return np.sqrt(self.Om0 * zp1 ** 3 + self.Ode0)

    def age(self, z):
        """Age of the Universe at redshift ``z`` [s]."""
        zp1 = 1.0 + np.asarray(z, dtype=np.float64)
        pref = 2.0 / (3.0 * self.H0 * np.sqrt(self.Ode0))
        return pref * np.arcsinh(np.sqrt(self.Ode0 / self.Om0) * np.power(zp1, -1.5))

    def tage_to_z(self, age):
        """Redshift at which the Universe has age ``age`` [s] (inverse of :meth:`age`)."""
        age = np.asarray(age, dtype=np.float64)
        arg = 1.5 * self.H0 * np.sqrt(self.Ode0) * age
        return np.power(np.sqrt(self.Ode0 / self.Om0) / np.sinh(arg), 2.0 / 3.0) - 1.0

    def dtdz(self, z):
        """|dt/dz| [s]."""
        zp1 = 1.0 + np.asarray(z, dtype=np.float64)
        return 1.0 / (self.H0 * zp1 * np.sqrt(self.Om0 * zp1 ** 3 + self.Ode0))

    def comoving_distance(self, z):
        """Line-of-sight comoving distance [cm]."""
        z = np.asarray(z, dtype=np.float64)
        u0 = np.sqrt(1.0 / (1.0 + z))
        half = 0.5 * (1.0 - u0)
        mid = 0.5 * (1.0 + u0)
        uu = mid[..., np.newaxis] + half[..., np.newaxis] * self.gl_nodes
        integ = 2.0 / np.sqrt(self.Om0 + self.Ode0 * uu ** 6)
        return self.hubble_distance * half * np.sum(integ * self.gl_weights, axis=-1)

    # ---- packed parameters for the device kernels

    def device_params(self):
        """Scalars the CUDA kernels need, in the order of ``hgb_cosmo`` (include/holodeck_gb300.h)."""
        return dict(H0=self.H0, Om0=self.Om0, Ode0=self.Ode0, hubble_distance=self.hubble_distance)

    def __repr__(self):
        return f"Cosmology(h={self.h}, Om0={self.Om0}, Ob0={self.Ob0}, size={self._grid_z.size})"


#: module-level instance with holodeck's WMAP9 parameters (holodeck/__init__.py:48-53)
cosmo = Cosmology(h=0.6933, Om0=0.2880, Ob0=0.0472, size=200)
