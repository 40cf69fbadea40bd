"""muscle_gb300 — a GB300 (sm_103a) backend for Muscle.jl's tensor contractions.

Host-side mirror of Muscle.jl's operation API (``binary_einsum``,
``binary_einsum!``, ``unary_einsum``, ``unary_einsum!`` on labelled
``Tensor``s, backend dispatch with ``with_backend``) over the C ABI of
libmuscle_gb300.so. Compute runs only in the library's CUDA kernels; there is
no CPU path, and operations on host arrays raise.
"""
from ._lib import (
    ArgumentError,
    DeviceTimeout,
    DimensionMismatch,
    MuscleError,
    OutOfBudget,
    UnsupportedError,
)
from .backend import (
    Backend,
    BackendBase,
    Domain,
    DomainCUDA,
    DomainHost,
    choose_backend,
    choose_backend_rule,
    domain,
    with_backend,
)
from .ops import (
    BackendGB300,
    binary_einsum,
    binary_einsum_,
    contract_into,
    contraction_plan,
    device_status,
    hadamard,
    hadamard_,
    simple_update,
    tensor_svd_thin,
    permutedims,
    promote_eltype,
    unary_einsum,
    unary_einsum_,
    unary_plan,
)
from .blocks import BlockContraction, BlockPlan, block_einsum
from .grouped import Group, batched_contract
from .serve import Request, Server
from .tensor import (
    Index,
    Tensor,
    empty_colmajor,
    findperm,
    inds,
    isapprox,
    nonunique,
    parent,
    zeros_colmajor,
)

__all__ = [n for n in dir() if not n.startswith("_")]


def library():
    """Loads (building in-tree if needed) and returns the ctypes library."""
    from ._lib import load

    return load()
