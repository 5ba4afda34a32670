"""pyqcm_gb300: GB300 (sm_103a) engine for pyqcm's exact-diagonalization hot
path -- the factorized Hubbard Hamiltonian-vector product inside Lanczos and
band Lanczos, and the Lehmann Green function and k x omega lattice integrals
built on it.  The compute runs in libqcmg (CUDA, C ABI in include/qcmg.h);
this package is the host-side mirror of pyqcm's interface for that path.
"""
from ._lib import QcmgError, lib  # noqa: F401
from .ed import (GLOBAL, ClusterModel, Hamiltonian, ModelInstance, Sector,  # noqa: F401
                 apply_c, green_function, halfbasis, halfbasis_rank, lanczos_batch,
                 set_global_parameter, streamline)

__all__ = ["QcmgError", "lib", "GLOBAL", "ClusterModel", "Hamiltonian", "ModelInstance",
           "Sector", "apply_c", "green_function", "halfbasis", "halfbasis_rank", "lanczos_batch",
           "set_global_parameter", "streamline"]
