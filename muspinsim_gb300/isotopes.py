"""Nuclear isotope data: spin I, gyromagnetic ratio and quadrupole moment.

The reference looks these up through a third-party NMR library
(``muspinsim/constants.py:8, 49, 73, 104`` call
``soprano.nmr.utils._get_isotope_data``), which returns gamma in rad/(s T),
the quadrupole moment in millibarn and the spin in units of hbar; the element
alone selects its most abundant isotope.  That library is not a dependency
here, so this module holds its own table, written from published NMR tables
(IUPAC recommendations, Harris et al. 2001; CODATA 2018 for the proton).  The
same table feeds the CPU oracle, so the two sides agree exactly on every
constant even where a value differs in the last digits from other tables.

Each entry is ``(I, gamma_MHz_per_T, Q_millibarn)``; ``GAMMA_RAD`` gives gamma
in rad/(s T) the way the reference receives it, so that
``gamma_rad / (2e6 * pi)`` reproduces the MHz/T figure the reference uses.
"""

import numpy as np

# element -> {mass number: (spin I, gamma / 2pi in MHz/T, Q in millibarn)}
_TABLE = {
    "H": {1: (0.5, 42.577478518, 0.0), 2: (1.0, 6.535903, 2.860), 3: (0.5, 45.414836, 0.0)},
    "He": {3: (0.5, -32.43410, 0.0), 4: (0.0, 0.0, 0.0)},
    "Li": {6: (1.0, 6.265884, -0.808), 7: (1.5, 16.546, -40.1)},
    "Be": {9: (1.5, -5.9834, 52.88)},
    "B": {10: (3.0, 4.5751, 84.59), 11: (1.5, 13.6630, 40.59)},
    "C": {12: (0.0, 0.0, 0.0), 13: (0.5, 10.7084, 0.0)},
    "N": {14: (1.0, 3.077706, 20.44), 15: (0.5, -4.316, 0.0)},
    "O": {16: (0.0, 0.0, 0.0), 17: (2.5, -5.7742, -25.58)},
    "F": {19: (0.5, 40.0776, 0.0)},
    "Ne": {20: (0.0, 0.0, 0.0), 21: (1.5, -3.3631, 101.55)},
    "Na": {23: (1.5, 11.2688, 104.0)},
    "Mg": {24: (0.0, 0.0, 0.0), 25: (2.5, -2.6083, 199.4)},
    "Al": {27: (2.5, 11.1031, 146.6)},
    "Si": {28: (0.0, 0.0, 0.0), 29: (0.5, -8.4655, 0.0)},
    "P": {31: (0.5, 17.2515, 0.0)},
    "S": {32: (0.0, 0.0, 0.0), 33: (1.5, 3.2717, -67.8)},
    "Cl": {35: (1.5, 4.1765, -81.65), 37: (1.5, 3.4765, -64.35)},
    "K": {39: (1.5, 1.9894, 58.5), 41: (1.5, 1.0920, 71.1)},
    "Ca": {40: (0.0, 0.0, 0.0), 43: (3.5, -2.8688, -40.8)},
    "Ti": {48: (0.0, 0.0, 0.0), 47: (2.5, -2.4040, 302.0), 49: (3.5, -2.4047, 247.0)},
    "V": {51: (3.5, 11.2133, -52.0)},
    "Cr": {52: (0.0, 0.0, 0.0), 53: (1.5, -2.4115, -150.0)},
    "Mn": {55: (2.5, 10.5763, 330.0)},
    "Fe": {56: (0.0, 0.0, 0.0), 57: (0.5, 1.3816, 0.0)},
    "Co": {59: (3.5, 10.077, 420.0)},
    "Ni": {58: (0.0, 0.0, 0.0), 61: (1.5, -3.8113, 162.0)},
    "Cu": {63: (1.5, 11.319, -220.0), 65: (1.5, 12.103, -204.0)},
    "Zn": {64: (0.0, 0.0, 0.0), 67: (2.5, 2.6693, 150.0)},
    "Ga": {69: (1.5, 10.2475, 171.0), 71: (1.5, 13.0204, 107.0)},
    "Ge": {74: (0.0, 0.0, 0.0), 73: (4.5, -1.4897, -196.0)},
    "As": {75: (1.5, 7.3150, 314.0)},
    "Se": {80: (0.0, 0.0, 0.0), 77: (0.5, 8.1571, 0.0)},
    "Br": {79: (1.5, 10.7042, 313.0), 81: (1.5, 11.5384, 262.0)},
    "Rb": {85: (2.5, 4.1253, 276.0), 87: (1.5, 13.9807, 133.5)},
    "Sr": {88: (0.0, 0.0, 0.0)},
    "Y": {89: (0.5, -2.0949, 0.0)},
    "Nb": {93: (4.5, 10.4523, -320.0)},
    "Mo": {98: (0.0, 0.0, 0.0)},
    "Ag": {107: (0.5, -1.7331, 0.0), 109: (0.5, -1.9924, 0.0)},
    "Cd": {114: (0.0, 0.0, 0.0), 111: (0.5, -9.0689, 0.0)},
    "In": {115: (4.5, 9.3856, 770.0)},
    "Sn": {120: (0.0, 0.0, 0.0), 119: (0.5, -15.9680, 0.0)},
    "Sb": {121: (2.5, 10.2552, -360.0)},
    "Te": {130: (0.0, 0.0, 0.0), 125: (0.5, -13.5454, 0.0)},
    "I": {127: (2.5, 8.5782, -696.0)},
    "Cs": {133: (3.5, 5.6234, -3.43)},
    "Ba": {138: (0.0, 0.0, 0.0)},
    "La": {139: (3.5, 6.0614, 200.0)},
    "Pt": {195: (0.5, 9.2921, 0.0)},
    "Au": {197: (1.5, 0.7406, 547.0)},
    "Hg": {202: (0.0, 0.0, 0.0), 199: (0.5, 7.7123, 0.0)},
    "Tl": {205: (0.5, 24.8624, 0.0)},
    "Pb": {208: (0.0, 0.0, 0.0), 207: (0.5, 9.0340, 0.0)},
    "Bi": {209: (4.5, 6.9630, -516.0)},
}

# Most abundant isotope of each element (used when no mass number is given)
_DEFAULT = {
    "H": 1, "He": 4, "Li": 7, "Be": 9, "B": 11, "C": 12, "N": 14, "O": 16,
    "F": 19, "Ne": 20, "Na": 23, "Mg": 24, "Al": 27, "Si": 28, "P": 31,
    "S": 32, "Cl": 35, "K": 39, "Ca": 40, "Ti": 48, "V": 51, "Cr": 52,
    "Mn": 55, "Fe": 56, "Co": 59, "Ni": 58, "Cu": 63, "Zn": 64, "Ga": 69,
    "Ge": 74, "As": 75, "Se": 80, "Br": 79, "Rb": 85, "Sr": 88, "Y": 89,
    "Nb": 93, "Mo": 98, "Ag": 107, "Cd": 114, "In": 115, "Sn": 120, "Sb": 121,
    "Te": 130, "I": 127, "Cs": 133, "Ba": 138, "La": 139, "Pt": 195,
    "Au": 197, "Hg": 202, "Tl": 205, "Pb": 208, "Bi": 209,
}


def isotope_data(element, prop, isotope=None):
    """Return one property of an isotope: ``"I"``, ``"gamma"`` (rad/(s T)) or
    ``"Q"`` (millibarn).

    Raises RuntimeError for an unknown element or isotope, which is the
    error the reference's constants module turns into
    ``ValueError("Invalid isotope ...")`` (``muspinsim/constants.py:48-51``).
    """
    try:
        entries = _TABLE[element]
    except KeyError as exc:
        raise RuntimeError(f"No data for element {element}") from exc
    iso = _DEFAULT[element] if isotope is None else isotope
    try:
        I, gmhz, q = entries[iso]
    except KeyError as exc:
        raise RuntimeError(f"No data for isotope {iso} of {element}") from exc
    if prop == "I":
        return I
    if prop == "gamma":
        return gmhz * 2e6 * np.pi
    if prop == "Q":
        return q
    raise ValueError(f"Unknown isotope property {prop}")
