"""tenetgb — GB300 (sm_103a) implementation of Tenet.jl's tensor-network hot path.

All arithmetic runs in libtenetgb.so (hand-written CUDA for sm_103a, C ABI in
include/tenet_gb300.h).  This package is the host-side mirror of the reference's
interface for that path: Muscle-level tensor operations (``core``) and the device-resident
MPS with Tenet's canonical-form operations (``mps``).
"""

from . import _lib
from .core import (
    Context,
    DeviceTensor,
    binary_einsum,
    default_context,
    hadamard,
    norm as tensor_norm,
    permute,
    simple_update,
    tensor_qr_thin,
    tensor_svd_thin,
)
from .dmrg import Dmrg1, Dmrg2, dmrg, dmrg_, ising_1d_mpo
from .dmrg import last_stats as dmrg_last_stats
from .mpo import MPO
from .mps import (
    MPS,
    BondCanonical,
    MixedCanonical,
    NonCanonical,
    canonize,
    canonize_,
    compress,
    compress_,
    entropy_vonneumann,
    entropy_vonneumann_,
    evolve_,
    evolve_mpo,
    evolve_mpo_,
    normalize,
    normalize_,
    norm,
    overlap,
    sample,
    schmidt_values,
    schmidt_values_,
    simple_update_,
    truncate,
    truncate_,
)

__all__ = [n for n in dir() if not n.startswith("__")]
