"""Backend selection mirroring src/Backend.jl and src/Domain.jl.

``choose_backend(f, *tensors)`` returns the scoped override when one is set
(``with_backend``, src/Backend.jl:16-18, 28-36) and otherwise looks the
operation up by the memory domain of every array, as the
``choose_backend_rule`` tables of src/Operations/binary_einsum.jl:20-31 and
src/Operations/unary_einsum.jl:20-24 do. This package registers exactly one
backend, ``BackendGB300``, for device-resident operands; host arrays have no
rule here (they belong to Muscle.jl's own BackendBase), so they raise.
"""
from __future__ import annotations

import contextlib
import contextvars

import torch

from ._lib import ArgumentError


class Domain:
    pass


class DomainHost(Domain):
    def __eq__(self, o):
        return isinstance(o, DomainHost)

    def __hash__(self):
        return hash("DomainHost")


class DomainCUDA(Domain):
    def __eq__(self, o):
        return isinstance(o, DomainCUDA)

    def __hash__(self):
        return hash("DomainCUDA")


def domain(x) -> Domain:
    """Memory domain of an array or Tensor (src/Domain.jl:11-14)."""
    data = getattr(x, "data", x)
    if isinstance(data, torch.Tensor) and data.is_cuda:
        return DomainCUDA()
    return DomainHost()


class Backend:
    """Operations raise until a backend implements them
    (src/Operations/binary_einsum.jl:53-55, 72-74; unary_einsum.jl:38-50)."""

    def binary_einsum(self, inds_c, a, b):
        raise ArgumentError(f"`binary_einsum` not implemented or not loaded for backend {type(self).__name__}")

    def binary_einsum_(self, c, a, b):
        raise ArgumentError(f"`binary_einsum!` not implemented or not loaded for backend {type(self).__name__}")

    def unary_einsum(self, inds_y, x):
        raise ArgumentError(f"`unary_einsum` not implemented or not loaded for backend {type(self).__name__}")

    def unary_einsum_(self, y, x):
        raise ArgumentError(f"`unary_einsum!` not implemented or not loaded for backend {type(self).__name__}")

    def hadamard(self, a, b):
        raise ArgumentError(f"`hadamard` not implemented or not loaded for backend {type(self).__name__}")

    def hadamard_(self, c, a, b):
        raise ArgumentError(f"`hadamard!` not implemented or not loaded for backend {type(self).__name__}")

    def __eq__(self, o):
        return type(self) is type(o) and self.__dict__ == o.__dict__

    def __hash__(self):
        return hash((type(self).__name__, tuple(sorted(self.__dict__.items()))))

    def __repr__(self):
        args = ", ".join(f"{k}={v!r}" for k, v in self.__dict__.items())
        return f"{type(self).__name__}({args})"


class BackendBase(Backend):
    """Muscle.jl's host backend; not provided by this package."""


_CURRENT = contextvars.ContextVar("muscle_gb300_backend", default=None)
_RULES: dict = {}


def choose_backend_rule(f, *domains):
    key = (f.__name__,) + tuple(type(d).__name__ for d in domains)
    if key in _RULES:
        return _RULES[key]()
    names = ", ".join(type(d).__name__ for d in domains)
    raise ArgumentError(f"no backend rule for {f.__name__}({names}) in muscle_gb300")


def register_rule(fname: str, domains: tuple, factory) -> None:
    _RULES[(fname,) + tuple(d.__name__ for d in domains)] = factory


def choose_backend(f, *arrays) -> Backend:
    cur = _CURRENT.get()
    if cur is not None:
        return cur
    return choose_backend_rule(f, *(domain(a) for a in arrays))


@contextlib.contextmanager
def _scoped(backend: Backend):
    tok = _CURRENT.set(backend)
    try:
        yield backend
    finally:
        _CURRENT.reset(tok)


def with_backend(*args):
    """``with_backend(backend)`` as a context manager, or
    ``with_backend(f, backend)`` calling ``f()`` under the override."""
    if len(args) == 1:
        return _scoped(args[0])
    f, backend = args
    with _scoped(backend):
        return f()
