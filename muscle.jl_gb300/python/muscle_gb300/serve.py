"""Serving form: a request loop for contractions of mixed sizes.

``Server`` wraps the library's native scheduler (mgb_server_*): requests are
admitted against an HBM byte budget and batched continuously onto several
streams, so requests that arrive while others run overlap with them on the
device. Operands stay device-resident; each request gets its own output
Tensor. ``submit`` returns a ``Request`` whose ``result()`` blocks until the
contraction finished.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import ArgumentError, check
from .ops import BackendGB300, binary_inds_c, contraction_plan, promote_eltype
from .tensor import Index, Tensor, empty_colmajor


class Request:
    __slots__ = ("server", "ticket", "out", "plan", "keep", "_status")

    def __init__(self, server, ticket, out, plan, keep):
        self.server, self.ticket, self.out, self.plan, self.keep = server, ticket, out, plan, keep
        self._status = None

    def wait(self, timeout: float = -1.0) -> int:
        if self._status is None:
            lib = _lib.load()
            st = ctypes.c_int32(0)
            check(lib.mgb_server_wait(self.server.handle, self.ticket, timeout, ctypes.byref(st)), lib)
            self._status = int(st.value)
            self.keep = None
        return self._status

    def result(self, timeout: float = -1.0) -> Tensor:
        status = self.wait(timeout)
        if status != _lib.OK:
            _lib.check(status)
        return self.out


class Server:
    """budget_bytes: HBM admission budget; streams: concurrent batches;
    max_batch: requests per launch batch; form / slices: arithmetic form of
    every request (BackendGB300 semantics)."""

    def __init__(self, budget_bytes: int = 120 * 10**9, streams: int = 4, max_batch: int = 256,
                 form: str = "auto", slices: int = 0, device=None):
        self.device = torch.device(device if device is not None else torch.cuda.current_device())
        if self.device.type != "cuda":
            raise ArgumentError("the server runs on a CUDA device")
        self.backend = BackendGB300(form, slices)
        lib = _lib.load()
        self.handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(lib.mgb_server_create(ctypes.byref(self.handle), int(budget_bytes), int(streams), int(max_batch)), lib)

    def submit(self, a: Tensor, b: Tensor, dims=None, out=None, wait_for_stream: bool = True) -> Request:
        """Queues C = binary_einsum(a, b; dims, out); returns a Request."""
        inds_c = binary_inds_c(a.inds, b.inds, dims, out)
        sizes = {}
        for t in (a, b):
            for d, i in enumerate(t.inds):
                sizes.setdefault(i, t.data.shape[d])
        for i in inds_c:
            if i not in sizes:
                raise ArgumentError(f"output index {i} is in neither operand")
        c = empty_colmajor([sizes[i] for i in inds_c], promote_eltype(a.dtype, b.dtype), a.data.device)
        C = Tensor(c, inds_c)
        plan = contraction_plan(a.data, a.inds, b.data, b.inds, c, inds_c, self.backend.form, self.backend.slices)
        resident = a.data.numel() * a.data.element_size() + b.data.numel() * b.data.element_size() + \
            c.numel() * c.element_size()
        dep = torch.cuda.current_stream(self.device).cuda_stream if wait_for_stream else None
        ticket = ctypes.c_int64(0)
        lib = _lib.load()
        check(lib.mgb_server_submit(self.handle, plan.handle, a.data.data_ptr(), b.data.data_ptr(), c.data_ptr(),
                                    resident, dep, ctypes.byref(ticket)), lib)
        return Request(self, int(ticket.value), C, plan, (a, b))

    def submit_planned(self, plan, a: Tensor, b: Tensor, c: Tensor, wait_for_stream: bool = False) -> Request:
        """Low-overhead submission of a contraction whose plan and output the
        caller prepared (``contraction_plan`` on the same tensors)."""
        resident = a.data.numel() * a.data.element_size() + b.data.numel() * b.data.element_size() + \
            c.data.numel() * c.data.element_size()
        dep = torch.cuda.current_stream(self.device).cuda_stream if wait_for_stream else None
        ticket = ctypes.c_int64(0)
        lib = _lib.load()
        check(lib.mgb_server_submit(self.handle, plan.handle, a.data.data_ptr(), b.data.data_ptr(),
                                    c.data.data_ptr(), resident, dep, ctypes.byref(ticket)), lib)
        return Request(self, int(ticket.value), c, plan, (a, b))

    def stats(self) -> dict:
        s = _lib.ServerStats()
        lib = _lib.load()
        check(lib.mgb_server_get_stats(self.handle, ctypes.byref(s)), lib)
        return {f: getattr(s, f) for f, _ in _lib.ServerStats._fields_}

    def reset_stats(self):
        lib = _lib.load()
        check(lib.mgb_server_reset_stats(self.handle), lib)

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().mgb_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
