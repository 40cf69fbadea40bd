"""Grouped contractions (the batching form): thousands of independent
contractions, e.g. the site pairs of a PEPS sweep, in a few batched launches.

Members whose operands have identical shapes and strides share a plan
(plans are cached by descriptor), and the library runs every such bucket as
one batched launch per kernel. ``Group.capture()`` records the whole group in
one CUDA graph; ``Group.update()`` swaps operand pointers for a replay on new
data. The per-bucket schedule (arithmetic form and rasterisation band) can be
chosen by ``autotune.Autotuner``.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import torch

from . import _lib
from ._lib import ArgumentError, check
from .ops import _require_cuda, contraction_plan
from .tensor import Tensor


class Group:
    """A fixed set of contractions C_i[ic] = A_i[ia] * B_i[ib].

    items: sequence of (C, A, B) Tensors (device-resident, labels define the
    contraction). forms: one form per item, or a single form for all.
    """

    def __init__(self, items: Sequence[tuple], forms="auto", slices: int = 0, bands=None):
        if not items:
            raise ArgumentError("empty group")
        self.items = list(items)
        n = len(self.items)
        self.forms = [forms] * n if isinstance(forms, str) else list(forms)
        if len(self.forms) != n:
            raise ArgumentError("one form per item")
        self.slices = slices
        self.plans = []
        for (c, a, b), form in zip(self.items, self.forms):
            _require_cuda(a.data, b.data, c.data)
            self.plans.append(contraction_plan(a.data, a.inds, b.data, b.inds, c.data, c.inds, form, slices))
        self.device = self.items[0][0].data.device
        lib = _lib.load()
        handles = (ctypes.c_void_p * n)(*[p.handle for p in self.plans])
        A, B, C = self._pointer_arrays()
        self.handle = ctypes.c_void_p()
        check(lib.mgb_group_create(ctypes.byref(self.handle), handles, n, A, B, C), lib)
        ws = ctypes.c_uint64(0)
        check(lib.mgb_group_workspace_size(self.handle, ctypes.byref(ws)), lib)
        self.workspace_bytes = int(ws.value)
        self.workspace = torch.empty(max(self.workspace_bytes, 1), dtype=torch.uint8, device=self.device)
        if bands is not None:
            self.set_bands(bands)
        # default schedule of capture(): every bucket's own launches on four
        # parallel branches (the autotuner measures and replaces it)
        self.schedule = (4, False)

    def _pointer_arrays(self):
        n = len(self.items)
        A = (ctypes.c_void_p * n)(*[a.data.data_ptr() for (_, a, _) in self.items])
        B = (ctypes.c_void_p * n)(*[b.data.data_ptr() for (_, _, b) in self.items])
        C = (ctypes.c_void_p * n)(*[c.data.data_ptr() for (c, _, _) in self.items])
        return A, B, C

    @property
    def flops(self) -> float:
        return sum(p.flops for p in self.plans)

    def set_bands(self, bands):
        """Rasterisation band index (0..5 -> 1,2,3,4,8,16 row tiles) per item."""
        n = len(self.items)
        arr = (ctypes.c_int32 * n)(*bands)
        lib = _lib.load()
        check(lib.mgb_group_set_tiles(self.handle, arr), lib)

    def update(self, items: Sequence[tuple]):
        """New operand/output tensors with the same shapes as at creation."""
        if len(items) != len(self.items):
            raise ArgumentError("update must keep the member count")
        for (c, a, b), (c0, a0, b0) in zip(items, self.items):
            if c.data.shape != c0.data.shape or a.data.shape != a0.data.shape or b.data.shape != b0.data.shape:
                raise ArgumentError("update must keep the member shapes")
        self.items = list(items)
        lib = _lib.load()
        check(lib.mgb_group_update(self.handle, *self._pointer_arrays()), lib)

    def execute(self, stream: torch.cuda.Stream | None = None, parts: int = 1, persistent: bool = True):
        """Runs every member on `stream` (default: the current stream).

        persistent: the emulated buckets' tensor-core work runs as one
        persistent launch per kernel variant (after all pre-passes);
        otherwise every bucket runs its own launches. With parts > 1 the
        pre-passes (persistent) or whole buckets (not persistent) are split
        into that many parts of about equal work, run on side streams forked
        from and joined back into `stream` (the parts write disjoint outputs
        and workspace slices)."""
        lib = _lib.load()
        main = stream if stream is not None else torch.cuda.current_stream(self.device)
        ws, wsb = self.workspace.data_ptr(), self.workspace_bytes
        if parts <= 1:
            if persistent:
                check(lib.mgb_group_execute(self.handle, ws, wsb, main.cuda_stream), lib)
            else:
                check(lib.mgb_group_execute_part(self.handle, 0, 1, ws, wsb, main.cuda_stream), lib)
            return
        side = self._side_streams(parts)
        for ss in side:
            ss.wait_stream(main)
        fn = lib.mgb_group_prepare_part if persistent else lib.mgb_group_execute_part
        for i, ss in enumerate(side):
            check(fn(self.handle, i, parts, ws, wsb, ss.cuda_stream), lib)
        for ss in side:
            main.wait_stream(ss)
        if persistent:
            check(lib.mgb_group_finish(self.handle, ws, wsb, main.cuda_stream), lib)

    def _side_streams(self, parts):
        cache = getattr(self, "_side", None)
        if cache is None or len(cache) != parts:
            cache = [torch.cuda.Stream(self.device) for _ in range(parts)]
            self._side = cache
        return cache

    def capture(self, parts: int | None = None, persistent: bool | None = None) -> torch.cuda.CUDAGraph:
        """Warm up once (which also uploads the persistent launches' job
        tables), then record execute() into a CUDA graph (with parts > 1 the
        parts become parallel branches of the graph).

        On a 4096-member PEPS batch, parts=4 or 8 with persistent=False was
        the fastest schedule on GB300 (ComplexF64 97.8 ms against 109.6 ms
        for one persistent launch per kernel variant after all pre-passes):
        the HBM-bound pre-passes of some buckets then overlap the
        tensor-core work of others, which a persistent launch, holding every
        SM, leaves no room for. Without arguments the group's `schedule` is
        used (set by ``Autotuner.schedule``)."""
        if parts is None:
            parts = self.schedule[0]
        if persistent is None:
            persistent = self.schedule[1]
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.execute(s, parts, persistent)
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.execute(torch.cuda.current_stream(self.device), parts, persistent)
        return g

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                _lib.load().mgb_group_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def batched_contract(items: Sequence[tuple], forms="auto", slices: int = 0) -> Group:
    """Builds a Group for (C, A, B) items and executes it once."""
    g = Group(items, forms, slices)
    g.execute()
    return g
