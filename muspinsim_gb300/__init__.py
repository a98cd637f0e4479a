"""muspinsim_gb300: GB300-native muon spin polarisation path.

Drop-in replacement for MuSpinSim's polarisation hot path: spin systems and
Hamiltonians built on the host exactly as the reference builds them, and
every diagonalisation, time evolution, decaying integral and powder average
executed by hand-written sm_103a CUDA kernels (``libmspgpu.so``) through a
C ABI.  There is no CPU fallback.
"""

from muspinsim_gb300.constants import ELEC_GAMMA, MU_GAMMA, MU_TAU, EFG_2_MHZ  # noqa: F401
from muspinsim_gb300.spinop import SpinOperator, DensityOperator, Operator  # noqa: F401
from muspinsim_gb300.hamiltonian import Hamiltonian  # noqa: F401
from muspinsim_gb300.spinsys import SpinSystem, MuonSpinSystem  # noqa: F401
from muspinsim_gb300.powder import powder_average  # noqa: F401

__version__ = "0.1.0"
