"""GB300-native (sm_103a) NEGF transport engine for the phinfortran hot path.

The compute lives in the in-tree C-ABI library built from ``csrc/``
(``include/phinfortran_gb300.h``).  Importing the package does not need a
GPU; calling an entry point does, and fails loudly without the library.
"""
from . import _abi
from .transport import TdbBlocks, transport_tdb, DeviceTransport, fortran_block

__all__ = ["TdbBlocks", "transport_tdb", "DeviceTransport", "fortran_block", "_abi"]
