"""Physical constants used by the polarisation path.

Same names, values and formulas as ``muspinsim/constants.py:12-108``:
gyromagnetic ratios in MHz/T (a frequency, not a pulsation), quadrupole
moments in barn-scaled units that combine with ``EFG_2_MHZ``, spins in hbar.
"""

import numpy as np
from scipy import constants as cnst

from muspinsim_gb300.isotopes import isotope_data

# CODATA values (muspinsim/constants.py:12-14)
ELEC_GAMMA = -28024.9514242  # electron gyromagnetic ratio, MHz/T
MU_GAMMA = -(ELEC_GAMMA / 206.7669883)  # muon gyromagnetic ratio, MHz/T
MU_TAU = 2.19703  # muon lifetime, microseconds

# Electric field gradient (atomic units) times quadrupole moment (millibarn)
# to MHz; 1e-37 = 1e-6 (to MHz) * 1e-28 (barn to m^2) * 1e-3 (milli)
# (muspinsim/constants.py:20-25)
EFG_2_MHZ = (
    cnst.physical_constants["atomic unit of electric field gradient"][0]
    * cnst.e
    * 1e-37
    / cnst.h
)


def gyromagnetic_ratio(elem="mu", iso=None):
    """Gyromagnetic ratio in MHz/T of 'e', 'mu' or a nucleus
    (muspinsim/constants.py:28-53)."""
    if elem == "e":
        return ELEC_GAMMA
    elif elem == "mu":
        return MU_GAMMA
    try:
        val = isotope_data(elem, "gamma", iso)
    except RuntimeError as exc:
        raise ValueError(f"Invalid isotope {iso} for element {elem}") from exc
    return val / (2e6 * np.pi)


def quadrupole_moment(elem="mu", iso=None):
    """Quadrupole moment of a particle, 0 for 'e' and 'mu'
    (muspinsim/constants.py:56-77)."""
    if elem in ("e", "mu"):
        return 0
    try:
        val = isotope_data(elem, "Q", iso)
    except RuntimeError as exc:
        raise ValueError(f"Invalid isotope {iso} for element {elem}") from exc
    return val


def spin(elem="mu", iso=None):
    """Spin in units of hbar; for 'e' the isotope is a multiplicity of
    strongly coupled electrons (muspinsim/constants.py:80-108)."""
    if elem == "mu":
        return 0.5
    elif elem == "e":
        iso = iso or 1
        if iso < 1 or int(iso) != iso:
            raise ValueError(f"Invalid multiplicity {iso} for electron")
        return 0.5 * int(iso)
    try:
        val = isotope_data(elem, "I", iso)
    except RuntimeError as exc:
        raise ValueError(f"Invalid isotope {iso} for element {elem}") from exc
    return val
