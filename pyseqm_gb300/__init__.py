"""pyseqm_gb300: GB300-native batched MNDO/AM1/PM3 SCF behind PYSEQM's seqm API.

The compute path is hand-written sm_103a CUDA in ``csrc/`` behind the C ABI of
``include/pyseqm_gb300.h``; this package is the host side.
"""

__version__ = "0.1.0"
