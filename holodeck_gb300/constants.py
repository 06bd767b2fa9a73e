"""CGS constants used on the SAM gravitational-wave-background path.

Two constant sets exist on this path and each stage uses the same set as the
holodeck stage it replaces:

* The Python stages (grid construction, components, chirp-mass / strain
  formula) use astropy's CODATA-2018 / IAU-2015 values
  (holodeck/constants.py:23-55, holodeck/utils.py:40).
* The Cython kernels hard-code an older set (holodeck/sams/sam_cyutils.pyx:30-42,
  holodeck/cyutils.pyx:40-45).  Those are mirrored in ``CY_*`` below and in
  ``csrc/hgb_constants.cuh``.
"""

import numpy as np

# ---- astropy (CODATA 2018 / IAU 2015) values, cgs
NWTG = 6.6743e-08                      #: Newton's constant [cm^3/g/s^2]
SPLC = 29979245800.0                   #: speed of light [cm/s]
MSOL = 1.988409870698051e+33           #: solar mass [g]
PC = 3.085677581491367e+18             #: parsec [cm]
YR = 31557600.0                        #: Julian year [s]
DAY = 86400.0
KPC = 1.0e3 * PC
MPC = 1.0e6 * PC
GPC = 1.0e9 * PC
MYR = 1.0e6 * YR
GYR = 1.0e9 * YR
SCHW = 2 * NWTG / (SPLC * SPLC)        #: Schwarzschild constant 2G/c^2 [cm/g]
KMPERSEC = 1.0e5

#: strain prefactor of a circular source, [Sesana2004] Eq.36 (holodeck/utils.py:40)
GW_SRC_CONST = 8 * np.power(NWTG, 5 / 3) * np.power(np.pi, 2 / 3) / np.sqrt(10) / np.power(SPLC, 4)

# ---- constants hard-coded in the Cython kernels (sam_cyutils.pyx:30-42)
CY_NWTG = 6.6742999e-08
CY_SPLC = 29979245800.0
CY_MPC = 3.08567758e+24
CY_MSOL = 1.988409870698051e+33
CY_YR = 31557600.0
CY_SCHW = 1.4852320538237328e-28
