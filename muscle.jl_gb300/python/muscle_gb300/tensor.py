"""Index / Tensor data model mirroring Muscle.jl's src/Index.jl and src/Tensor.jl.

A ``Tensor`` pairs an array (a torch tensor; on the device for this backend)
with one ``Index`` label per dimension. Arrays created by this package are
column-major like Julia arrays (first dimension fastest); any strides are
accepted on input.
"""
from __future__ import annotations

from typing import Iterable, Sequence

import torch

from ._lib import ArgumentError, DimensionMismatch


class Index:
    """A dimension label (src/Index.jl:3-5). Equality and hashing by tag;
    ``Index("x")`` and ``Index(Index("x"))`` are the same label."""

    __slots__ = ("tag",)

    def __init__(self, tag):
        self.tag = tag.tag if isinstance(tag, Index) else tag

    def __eq__(self, other):
        return isinstance(other, Index) and self.tag == other.tag

    def __hash__(self):
        return hash(("Index", self.tag))

    def __repr__(self):
        return f"index<{self.tag}>"


def _as_index(i) -> Index:
    return i if isinstance(i, Index) else Index(i)


def nonunique(xs: Sequence) -> list:
    """Repeated elements, each once, in order of their second appearance
    (src/Utils/Utils.jl:5-25)."""
    seen, rep = [], []
    for x in xs:
        if x in seen:
            if x not in rep:
                rep.append(x)
        else:
            seen.append(x)
    return rep


def unique(xs: Iterable) -> list:
    out = []
    for x in xs:
        if x not in out:
            out.append(x)
    return out


def setdiff(xs: Iterable, ys: Iterable) -> list:
    """Julia's setdiff: unique elements of xs not in ys, in xs order."""
    ys = list(ys)
    return [x for x in unique(xs) if x not in ys]


def intersect(*seqs) -> list:
    """Julia's ∩: unique elements of the first sequence present in all others."""
    first, rest = seqs[0], [list(s) for s in seqs[1:]]
    return [x for x in unique(first) if all(x in r for r in rest)]


def union(*seqs) -> list:
    out = []
    for s in seqs:
        for x in s:
            if x not in out:
                out.append(x)
    return out


def empty_colmajor(shape: Sequence[int], dtype, device) -> torch.Tensor:
    """An uninitialised column-major (Julia-order) array."""
    shape = list(shape)
    if not shape:
        return torch.empty((), dtype=dtype, device=device)
    rev = torch.empty(list(reversed(shape)), dtype=dtype, device=device)
    return rev.permute(*reversed(range(len(shape))))


def zeros_colmajor(shape: Sequence[int], dtype, device) -> torch.Tensor:
    t = empty_colmajor(shape, dtype, device)
    t.zero_()
    return t


class Tensor:
    """Array with named dimensions (src/Tensor.jl:11-32)."""

    __slots__ = ("data", "_inds")

    def __init__(self, data, inds: Sequence | None = None):
        if isinstance(data, Tensor):
            raise ArgumentError("Can't wrap a `Tensor` with another `Tensor`")
        if not isinstance(data, torch.Tensor):
            data = torch.as_tensor(data)
        inds = [] if inds is None else [_as_index(i) for i in inds]
        if len(inds) != data.dim():
            raise ArgumentError(
                f"ndims(data) [{data.dim()}] must be equal to length(inds) [{len(inds)}]"
            )
        for i in nonunique(inds):
            sizes = {data.shape[d] for d, j in enumerate(inds) if j == i}
            if len(sizes) != 1:
                raise DimensionMismatch("nonuniform size of repeated indices")
        self.data = data
        self._inds = tuple(inds)

    # --- accessors mirroring Muscle.jl -------------------------------------
    @property
    def inds(self) -> list:
        return list(self._inds)

    def parent(self) -> torch.Tensor:
        return self.data

    @property
    def ndim(self) -> int:
        return self.data.dim()

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def device(self):
        return self.data.device

    def size(self, i=None):
        if i is None:
            return tuple(self.data.shape)
        if isinstance(i, int):
            return self.data.shape[i]
        return self.data.shape[self.dim(i)]

    def dim(self, i) -> int:
        i = _as_index(i)
        for d, j in enumerate(self._inds):
            if j == i:
                return d
        raise ArgumentError(f"index {i} not in tensor")

    def __repr__(self):
        return f"Tensor({tuple(self.data.shape)}, {self.dtype}, inds={list(self._inds)})"


def inds(t: Tensor) -> list:
    return t.inds


def parent(t: Tensor) -> torch.Tensor:
    return t.data


def findperm(frm: Sequence[Index], to: Sequence[Index]) -> list[int]:
    """Positions in ``to`` of each label of ``frm``, consuming repeated labels
    one by one (src/Index.jl:20-34)."""
    pool = list(to)
    perm = []
    for i in frm:
        k = pool.index(i)
        pool[k] = None
        perm.append(k)
    return perm


def isapprox(a: Tensor, b: Tensor, rtol: float | None = None, atol: float = 0.0) -> bool:
    """Approximate equality up to a permutation of labels (src/Tensor.jl:117-121),
    with Julia's default ``rtol = sqrt(eps)`` of the wider element type."""
    if sorted(map(repr, a.inds)) != sorted(map(repr, b.inds)):
        return False
    perm = findperm(a.inds, b.inds)
    bd = b.data.permute(*perm) if perm else b.data
    x = a.data.to(torch.promote_types(a.dtype, b.dtype))
    y = bd.to(x.dtype).to(x.device)
    if rtol is None:
        rtol = torch.finfo(x.dtype).eps ** 0.5
    diff = torch.linalg.vector_norm((x - y).flatten()).item()
    scale = max(torch.linalg.vector_norm(x.flatten()).item(), torch.linalg.vector_norm(y.flatten()).item())
    return diff <= max(atol, rtol * scale)
