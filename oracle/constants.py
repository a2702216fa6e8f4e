"""Physical constants of the reference (constants.py:5-11).

G is astropy's CODATA-2018 gravitational constant expressed in
kpc^3 / Msun / Gyr^2; KPCGYR_TO_KMS = kpc/km / (Gyr/s) with the Julian year.
"""
import math

# astropy: G=6.6743e-11 m^3 kg^-1 s^-2, M_sun=1.988409870698051e30 kg,
# kpc=3.0856775814913673e19 m, Gyr=3.15576e16 s.
_KPC_M = 3.0856775814913673e19
_MSUN_KG = 1.988409870698051e30
_GYR_S = 3.15576e16
G = 6.6743e-11 * _MSUN_KG * _GYR_S ** 2 / _KPC_M ** 3
KPC_TO_KM = _KPC_M / 1e3
GYR_TO_S = _GYR_S
KMS_TO_KPCGYR = GYR_TO_S / KPC_TO_KM
KPCGYR_TO_KMS = KPC_TO_KM / GYR_TO_S
EPSILON = 1e-12
TWOPI = 2 * math.pi
