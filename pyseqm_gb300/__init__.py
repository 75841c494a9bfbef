"""pyseqm_gb300: GB300-native batched MNDO/AM1/PM3/PM6_SP SCF behind PYSEQM's seqm API.

The compute path is hand-written sm_103a CUDA in ``csrc/`` behind the C ABI of
``include/pyseqm_gb300.h``; this package is the host side.
"""

__version__ = "0.1.0"

from .api import single_point  # noqa: E402,F401
from .basics import (  # noqa: E402,F401
    Constants,
    Electronic_Structure,
    Energy,
    Force,
    Hamiltonian,
    Molecule,
    Pack_Parameters,
    Parser,
    SCFEnergyFunction,
    EnergyXL,
    ForceXL,
    NACConfig,
    active_state_tensor,
    resolve_nac_config,
)
from .io import read_xyz, read_xyz_trajectory, save_xyz  # noqa: E402,F401
from .optimization import geomeTRIC_optimization, geometric_optimization  # noqa: E402,F401
from .dynamics import KSA_XL_BOMD, XL_BOMD, Geometry_Optimization_SD, Molecular_Dynamics_Basic, Molecular_Dynamics_Langevin  # noqa: E402,F401
