"""Block-partitioned contraction, the decomposition of Muscle's Dagger
backend (ext/MuscleDaggerExt/binary_einsum.jl:64-119) on device tensors.

The operands are split into blocks along the labels of ``blocksize`` (the
Dagger partitioning; every block size must divide its extent, as the
reference's ``÷`` does). Every output block is the sum, over the blocks of
the contracted labels, of the contractions of one block of A with one block
of B (the reference spawns one task per block pair and reduces them with
``treereduce(AddComputeOp, ...)``, :100-115). Here:

  * blocks are views of the operands and of the output: nothing is copied;
  * every block pair of every output block runs as one ``Group`` (pairs of
    equal shapes share a plan and run as one batched launch);
  * an output block with more than one contracted-block pair gets its partial
    results stacked along one extra label, and ``unary_einsum`` sums them into
    the output block (the tree reduction); with one pair the contraction
    writes into the output block directly.

``rank`` / ``world`` restrict the work to the output blocks one replica
owns: blocks are dealt, largest work first, to the replica with the least
work so far, so replicas sharding by output blocks need no collective (their
blocks are disjoint); with contracted-label blocks the reduction stays inside
one replica. The planning is pure host logic (``BlockPlan``), independent of
the device, so it can be checked without one.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import torch

from ._lib import ArgumentError, DimensionMismatch
from .tensor import Index, Tensor, empty_colmajor, setdiff, union, zeros_colmajor


def _idx(i):
    return i if isinstance(i, Index) else Index(i)


@dataclass
class BlockTask:
    out_block: tuple                      # block coordinates along the output labels
    pairs: list = field(default_factory=list)  # [(slices of A, slices of B)] per contracted-block combination
    flops: float = 0.0


class BlockPlan:
    """Blocks of C[ic] = sum A[ia] B[ib] for a partitioning {label: block size}.

    Labels absent from ``blocksize`` are one block. Output labels follow the
    reference's rule (:51-60): a label's block size comes from whichever
    operand holds it."""

    def __init__(self, ia, shape_a, ib, shape_b, ic, blocksize: dict):
        self.ia, self.ib, self.ic = [_idx(i) for i in ia], [_idx(i) for i in ib], [_idx(i) for i in ic]
        if len(set(self.ia)) != len(self.ia) or len(set(self.ib)) != len(self.ib) or len(set(self.ic)) != len(self.ic):
            raise ArgumentError("block contraction: labels must be unique per tensor")
        if any(i not in self.ia and i not in self.ib for i in self.ic):
            raise ArgumentError("block contraction: ic must be a subset of ia ∪ ib")
        ext = {}
        for labs, shp in ((self.ia, shape_a), (self.ib, shape_b)):
            for i, e in zip(labs, shp):
                if i in ext and ext[i] != int(e):
                    raise DimensionMismatch(f"label {i} has different extents")
                ext[i] = int(e)
        self.ext = ext
        want = {_idx(k): int(v) for k, v in blocksize.items()}
        if any(k not in ext for k in want):
            raise ArgumentError("block contraction: block size given for a label of neither operand")
        self.bs = {}
        for i in union(self.ia, self.ib):
            b = want.get(i, ext[i])
            if b <= 0 or ext[i] % b != 0:
                raise ArgumentError(f"block size {b} of label {i} must divide its extent {ext[i]}")
            self.bs[i] = b
        self.nblocks = {i: self.ext[i] // self.bs[i] for i in self.bs}
        self.sum_labels = setdiff(union(self.ia, self.ib), self.ic)

    def _slices(self, labels, coords: dict):
        return tuple(slice(coords[i] * self.bs[i], (coords[i] + 1) * self.bs[i]) if i in coords else slice(None)
                     for i in labels)

    def tasks(self) -> list:
        """Every output block with its block pairs, in output-block order."""
        out = []
        ranges_c = [range(self.nblocks[i]) for i in self.ic]
        ranges_k = [range(self.nblocks[i]) for i in self.sum_labels]
        for oc in itertools.product(*ranges_c):
            co = dict(zip(self.ic, oc))
            t = BlockTask(oc)
            for kc in itertools.product(*ranges_k):
                c = dict(co)
                c.update(zip(self.sum_labels, kc))
                t.pairs.append((self._slices(self.ia, c), self._slices(self.ib, c)))
            m = 1.0
            for i in union(self.ia, self.ib):
                m *= self.bs[i]
            t.flops = 2.0 * m * len(t.pairs)
            out.append(t)
        return out

    def assign(self, rank: int = 0, world: int = 1) -> list:
        """The tasks of replica `rank` of `world`: dealt largest first to the
        replica with the least work so far (ties to the lowest rank)."""
        if world < 1 or not 0 <= rank < world:
            raise ArgumentError("block contraction: rank out of range")
        tasks = self.tasks()
        order = sorted(range(len(tasks)), key=lambda k: (-tasks[k].flops, k))
        load = [0.0] * world
        mine = []
        for k in order:
            r = min(range(world), key=lambda x: (load[x], x))
            load[r] += tasks[k].flops
            if r == rank:
                mine.append(k)
        return [tasks[k] for k in sorted(mine)]


class BlockContraction:
    """A block-partitioned contraction prepared once and executed any number
    of times: the Group of every block pair this replica owns, the stacked
    partial-result buffers and their reductions. ``execute`` runs on the
    current stream; the operands and the output keep their storage."""

    def __init__(self, a: Tensor, b: Tensor, blocksize: dict, out=None, rank: int = 0, world: int = 1,
                 form: str = "auto", c: Tensor | None = None):
        from .grouped import Group
        from .ops import binary_inds_c

        ia, ib = list(a.inds), list(b.inds)
        if out is not None:
            ic = [_idx(i) for i in out]
        elif c is not None:
            ic = list(c.inds)
        else:
            ic = binary_inds_c(ia, ib)
        self.plan = plan = BlockPlan(ia, a.data.shape, ib, b.data.shape, ic, blocksize)
        dt = torch.promote_types(a.dtype, b.dtype)
        dev = a.data.device
        if c is None:
            alloc = zeros_colmajor if world > 1 else empty_colmajor
            c = Tensor(alloc([plan.ext[i] for i in ic], dt, dev), ic)
        elif list(c.inds) != ic or list(c.data.shape) != [plan.ext[i] for i in ic]:
            raise DimensionMismatch("block contraction: output labels or extents do not match")
        self.c = c
        self.tasks = plan.assign(rank, world)
        items, self.reductions = [], []
        part = Index("__block_part")
        for t in self.tasks:
            cview = c.data[plan._slices(ic, dict(zip(ic, t.out_block)))]
            if len(t.pairs) == 1:
                sa, sb = t.pairs[0]
                items.append((Tensor(cview, ic), Tensor(a.data[sa], ia), Tensor(b.data[sb], ib)))
                continue
            # partial results stacked along one more label, summed afterwards
            P = empty_colmajor([plan.bs[i] for i in ic] + [len(t.pairs)], dt, dev)
            for k, (sa, sb) in enumerate(t.pairs):
                items.append((Tensor(P[..., k], ic), Tensor(a.data[sa], ia), Tensor(b.data[sb], ib)))
            self.reductions.append((Tensor(cview, ic), Tensor(P, ic + [part])))
        self.group = Group(items, form) if items else None

    @property
    def flops(self) -> float:
        return self.group.flops if self.group is not None else 0.0

    def execute(self) -> Tensor:
        from .ops import unary_einsum_

        if self.group is not None:
            self.group.execute()
            for y, x in self.reductions:  # the tree reduction of the partial results
                unary_einsum_(y, x)
        return self.c


def block_einsum(a: Tensor, b: Tensor, blocksize: dict, out=None, rank: int = 0, world: int = 1, form: str = "auto",
                 c: Tensor | None = None) -> Tensor:
    """Contracts a and b block by block (the Dagger decomposition of
    ext/MuscleDaggerExt/binary_einsum.jl:64-119) on the device. ``out``: the
    output labels (default: those of ``c`` if given, else Muscle's: a's free
    labels then b's); ``c``: an output tensor to write (default: a new one).
    With ``world`` > 1 only the output blocks of ``rank`` are written (a new
    output starts at zero, so the replicas' outputs add up to the whole
    result)."""
    return BlockContraction(a, b, blocksize, out, rank, world, form, c).execute()
