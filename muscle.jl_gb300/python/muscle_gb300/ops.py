"""binary_einsum / unary_einsum front-ends and the GB300 backend.

Front-ends restate the label algebra of src/Operations/binary_einsum.jl:33-51
and src/Operations/unary_einsum.jl:26-46; ``BackendGB300`` is the one backend
this package adds, taken for (DomainCUDA, DomainCUDA) operands, and calls the
C ABI of libmuscle_gb300.so (include/muscle_gb300.h). Label -> integer mode
mapping follows ext/MuscleCUDAExt.jl:24-27 (first appearance in a, then b).
"""
from __future__ import annotations

import ctypes
import threading
from collections import OrderedDict

import torch

from . import _lib
from ._lib import ArgumentError, check
from .backend import Backend, DomainCUDA, choose_backend, register_rule
from .tensor import Index, Tensor, empty_colmajor, intersect, nonunique, setdiff, union

_DT = {torch.float32: _lib.F32, torch.float64: _lib.F64, torch.complex64: _lib.C32, torch.complex128: _lib.C64}
_TORCH = {v: k for k, v in _DT.items()}


def mgb_dtype(t: torch.dtype) -> int:
    try:
        return _DT[t]
    except KeyError:
        raise ArgumentError(f"element type {t} is not supported (Float32/64, ComplexF32/64)") from None


def promote_eltype(a: torch.dtype, b: torch.dtype) -> torch.dtype:
    return torch.promote_types(a, b)


# ---------------------------------------------------------------------------
# plans
class Plan:
    """Owns an mgb_plan handle."""

    __slots__ = ("handle", "info", "__weakref__")

    def __init__(self, handle):
        self.handle = handle
        info = _lib.PlanInfo()
        check(_lib.load().mgb_plan_info_get(handle, ctypes.byref(info)))
        self.info = info

    @property
    def workspace_bytes(self) -> int:
        return int(self.info.workspace_bytes)

    @property
    def flops(self) -> float:
        return float(self.info.flops)

    @property
    def adaptive(self) -> bool:
        """True for an OZAKI plan whose slice count is chosen per call."""
        return self.info.form == _lib.FORM_OZAKI and self.info.slices == 0

    @property
    def operands_swapped(self) -> bool:
        """True when the library computes C^T = B^T A^T for this plan (an
        emulated form with few rows in A and many columns in B)."""
        v = ctypes.c_int32(0)
        check(_lib.load().mgb_plan_operands_swapped(self.handle, ctypes.byref(v)))
        return bool(v.value)

    def set_tolerance(self, tol: float) -> None:
        """Target relative Frobenius error of an adaptive plan's choice."""
        check(_lib.load().mgb_plan_set_tolerance(self.handle, float(tol)))

    def report(self, workspace, stream=None) -> dict:
        """The adaptive choice of the last call that ran with ``workspace``
        (a device tensor or pointer): ``slices`` (0: the plain form ran),
        ``estimate`` per candidate slice count, ``nonfinite``, ``tolerance``."""
        lib = _lib.load()
        r = _lib.AdaptiveReport()
        wp = workspace.data_ptr() if hasattr(workspace, "data_ptr") else int(workspace)
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib.mgb_plan_adaptive_report(self.handle, wp, st, ctypes.byref(r)), lib)
        return {"slices": int(r.slices), "nonfinite": bool(r.nonfinite), "tolerance": float(r.tolerance),
                "estimate": {S: float(r.estimate[S]) for S in range(9) if r.estimate[S] > 0 or S == r.slices}}

    def __del__(self):
        try:
            if self.handle:
                _lib.load().mgb_plan_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


class _PlanCache:
    def __init__(self, capacity=4096):
        self.cap = capacity
        self.d: OrderedDict = OrderedDict()
        self.lock = threading.Lock()

    def get(self, key, make):
        with self.lock:
            p = self.d.get(key)
            if p is not None:
                self.d.move_to_end(key)
                return p
        p = make()
        with self.lock:
            self.d[key] = p
            while len(self.d) > self.cap:
                self.d.popitem(last=False)
        return p


_PLANS = _PlanCache()


def _modes_for(*label_lists) -> dict:
    m = {}
    for labels in label_lists:
        for i in labels:
            if i not in m:
                m[i] = len(m)
    return m


def _desc_args(t: torch.Tensor, labels, modes: dict):
    return (mgb_dtype(t.dtype), tuple(modes[i] for i in labels), tuple(t.shape), tuple(t.stride()))


def contraction_plan(a: torch.Tensor, ia, b: torch.Tensor, ib, c: torch.Tensor, ic, form: str = "auto",
                     slices: int = 0) -> Plan:
    modes = _modes_for(ia, ib, ic)
    da, db, dc = _desc_args(a, ia, modes), _desc_args(b, ib, modes), _desc_args(c, ic, modes)
    f = _lib.FORMS[form]
    key = ("c", da, db, dc, f, int(slices))

    def make():
        lib = _lib.load()
        (ad, ka), (bd, kb), (cd, kc) = (_lib.make_desc(*da), _lib.make_desc(*db), _lib.make_desc(*dc))
        h = ctypes.c_void_p()
        check(lib.mgb_contraction_plan(ctypes.byref(h), ctypes.byref(ad), ctypes.byref(bd), ctypes.byref(cd),
                                       f, int(slices)), lib)
        return Plan(h)

    return _PLANS.get(key, make)


def unary_plan(x: torch.Tensor, ix, y: torch.Tensor, iy) -> Plan:
    modes = _modes_for(ix, iy)
    dx, dy = _desc_args(x, ix, modes), _desc_args(y, iy, modes)
    key = ("u", dx, dy)

    def make():
        lib = _lib.load()
        (xd, kx), (yd, ky) = _lib.make_desc(*dx), _lib.make_desc(*dy)
        h = ctypes.c_void_p()
        check(lib.mgb_unary_plan(ctypes.byref(h), ctypes.byref(xd), ctypes.byref(yd)), lib)
        return Plan(h)

    return _PLANS.get(key, make)


def _stream_handle(dev) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


def _require_cuda(*ts):
    for t in ts:
        if not t.is_cuda:
            raise ArgumentError("BackendGB300 needs device-resident (CUDA) arrays")


def _workspace(nbytes: int, dev):
    if nbytes == 0:
        return None, 0
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    return ws, ws.data_ptr()


def contract_into(c: torch.Tensor, ic, a: torch.Tensor, ia, b: torch.Tensor, ib, form="auto", slices=0,
                  workspace: torch.Tensor | None = None) -> torch.Tensor:
    """C[ic] = sum A[ia] * B[ib] on the current stream (cuTENSOR semantics)."""
    _require_cuda(a, b, c)
    plan = contraction_plan(a, ia, b, ib, c, ic, form, slices)
    need = plan.workspace_bytes
    if workspace is not None and workspace.numel() >= need:
        ws, wp = workspace, workspace.data_ptr()
    else:
        ws, wp = _workspace(need, c.device)
    lib = _lib.load()
    check(lib.mgb_contract(plan.handle, a.data_ptr(), b.data_ptr(), c.data_ptr(), wp, need,
                           _stream_handle(c.device)), lib)
    return c


# ---------------------------------------------------------------------------
class BackendGB300(Backend):
    """The GB300 backend. ``form`` is one of "auto" (Ozaki for Float64 /
    ComplexF64 results, BF16x3 for Float32 / ComplexF32), "plain" (native
    FP64 DMMA / FP32 FFMA), "ozaki" or "bf16x3"; ``slices`` is the Ozaki
    slice count (3..8), or 0 (the default): chosen on the device for every
    call, the smallest count whose estimated relative error is within 1e-13,
    else the plain FP64 form."""

    def __init__(self, form: str = "auto", slices: int = 0):
        if form not in _lib.FORMS:
            raise ArgumentError(f"unknown form {form!r}")
        self.form = form
        self.slices = int(slices)

    # binary_einsum(::BackendGB300, inds_c, a, b)  (called at binary_einsum.jl:50)
    def binary_einsum(self, inds_c, a: Tensor, b: Tensor) -> Tensor:
        inds_c = [i if isinstance(i, Index) else Index(i) for i in inds_c]
        sizes = {}
        for t in (a, b):
            for d, i in enumerate(t.inds):
                sizes.setdefault(i, t.data.shape[d])
        for i in inds_c:
            if i not in sizes:
                raise ArgumentError(f"output index {i} is in neither operand")
        dt = promote_eltype(a.dtype, b.dtype)
        c = empty_colmajor([sizes[i] for i in inds_c], dt, a.data.device)
        C = Tensor(c, inds_c)
        self.binary_einsum_(C, a, b)
        return C

    # binary_einsum!(::BackendGB300, c, a, b)  (called at binary_einsum.jl:68)
    def binary_einsum_(self, c: Tensor, a: Tensor, b: Tensor) -> Tensor:
        contract_into(c.data, c.inds, a.data, a.inds, b.data, b.inds, self.form, self.slices)
        return c

    # unary_einsum(::BackendGB300, inds_y, x)  (called at unary_einsum.jl:35)
    def unary_einsum(self, inds_y, x: Tensor) -> Tensor:
        inds_y = [i if isinstance(i, Index) else Index(i) for i in inds_y]
        for i in inds_y:
            if i not in x.inds:
                raise ArgumentError("Output indices must be a subset of input indices")
        y = empty_colmajor([x.size(i) for i in inds_y], x.dtype, x.data.device)
        Y = Tensor(y, inds_y)
        self.unary_einsum_(Y, x)
        return Y

    # unary_einsum!(::BackendGB300, y, x)  (called at unary_einsum.jl:44)
    def unary_einsum_(self, y: Tensor, x: Tensor) -> Tensor:
        _require_cuda(x.data, y.data)
        if x.dtype != y.dtype:
            raise ArgumentError("unary_einsum!: X and Y must share the element type")
        plan = unary_plan(x.data, x.inds, y.data, y.inds)
        lib = _lib.load()
        check(lib.mgb_unary(plan.handle, x.data.data_ptr(), y.data.data_ptr(), None, 0,
                            _stream_handle(y.data.device)), lib)
        return y


    # hadamard(::BackendBase, a, b) (src/Operations/hadamard.jl:34-40): the
    # result has a's labels and a's element type
    def hadamard(self, a: Tensor, b: Tensor) -> Tensor:
        if a.ndim < b.ndim:
            a, b = b, a
        c = empty_colmajor(list(a.data.shape), a.dtype, a.data.device)
        C = Tensor(c, list(a.inds))
        self.hadamard_(C, a, b)
        return C

    # hadamard!(::BackendBase, c, a, b) (src/Operations/hadamard.jl:42-77)
    def hadamard_(self, c: Tensor, a: Tensor, b: Tensor) -> Tensor:
        if a.ndim < b.ndim:
            a, b = b, a
        _require_cuda(a.data, b.data, c.data)
        if list(c.inds) != list(a.inds):
            raise ArgumentError("hadamard!: inds(c) must equal inds(a)")
        if any(i not in a.inds for i in b.inds):
            raise ArgumentError("hadamard: inds(b) must be a subset of inds(a)")
        modes = _modes_for(a.inds)
        lib = _lib.load()
        (ad, ka), (bd, kb), (cd, kc) = (_lib.make_desc(*_desc_args(a.data, a.inds, modes)),
                                        _lib.make_desc(*_desc_args(b.data, b.inds, modes)),
                                        _lib.make_desc(*_desc_args(c.data, c.inds, modes)))
        check(lib.mgb_hadamard(ctypes.byref(ad), ctypes.byref(bd), ctypes.byref(cd), a.data.data_ptr(),
                               b.data.data_ptr(), c.data.data_ptr(), _stream_handle(c.data.device)), lib)
        return c


    # tensor_svd_thin (src/Operations/tensor_svd.jl:98-125) on the device
    def tensor_svd_thin(self, x: Tensor, inds_u, inds_v, ind_s, keep: int = 0, normalize: bool = False,
                        sqrt_s: bool = False):
        """U (inds_u..., ind_s), s (ind_s), conj(V) (inds_v..., ind_s) of the
        thin SVD of x matricised as [inds_u; inds_v]; keep > 0 keeps the
        largest `keep` triplets; normalize scales the kept s to unit norm;
        sqrt_s returns sqrt(s) (for an equal absorb)."""
        _require_cuda(x.data)
        inds_u = [i if isinstance(i, Index) else Index(i) for i in inds_u]
        inds_v = [i if isinstance(i, Index) else Index(i) for i in inds_v]
        ind_s = ind_s if isinstance(ind_s, Index) else Index(ind_s)
        if sorted(map(repr, inds_u + inds_v)) != sorted(map(repr, x.inds)):
            raise ArgumentError("tensor_svd_thin: inds_u and inds_v must split inds(x)")
        if x.dtype not in (torch.float64, torch.complex128):
            raise _lib.UnsupportedError("tensor_svd_thin on the device: Float64 or ComplexF64")
        dense = True
        acc = 1
        for d in range(x.data.dim()):
            dense = dense and (x.data.shape[d] == 1 or x.data.stride(d) == acc)
            acc *= x.data.shape[d]
        # the matrix must be dense column-major: permute (copy) otherwise
        xm = x if (list(x.inds) == inds_u + inds_v and dense) else permutedims(x, inds_u + inds_v)
        su = [x.size(i) for i in inds_u]
        sv = [x.size(i) for i in inds_v]
        m, n = int(torch.tensor(su, dtype=torch.int64).prod()), int(torch.tensor(sv, dtype=torch.int64).prod())
        k = min(m, n)
        keep = k if keep <= 0 else min(keep, k)
        dev = x.data.device
        lib = _lib.load()
        wsb = ctypes.c_uint64(0)
        dt = mgb_dtype(x.dtype)
        check(lib.mgb_svd_workspace_size(dt, m, n, ctypes.byref(wsb)), lib)
        ws = torch.empty(max(int(wsb.value), 1), dtype=torch.uint8, device=dev)
        U = empty_colmajor(su + [keep], x.dtype, dev)
        S = torch.empty(keep, dtype=torch.float64, device=dev)
        V = empty_colmajor(sv + [keep], x.dtype, dev)
        flags = _lib.SVD_CONJ_V | (_lib.SVD_NORMALIZE if normalize else 0) | (_lib.SVD_SQRT_S if sqrt_s else 0)
        src = xm.data
        check(lib.mgb_svd(dt, m, n, src.data_ptr(), max(m, 1), U.data_ptr(), S.data_ptr(), V.data_ptr(), keep, flags,
                          ws.data_ptr(), ws.numel(), _stream_handle(dev)), lib)
        return Tensor(U, inds_u + [ind_s]), Tensor(S, [ind_s]), Tensor(V, inds_v + [ind_s])

    # simple_update (src/Operations/simple_update.jl:35-82) on the device
    def simple_update(self, A: Tensor, ind_physical_a, B: Tensor, ind_physical_b, ind_bond_ab, G: Tensor,
                      ind_physical_g_a, ind_physical_g_b, normalize: bool = False, absorb=None, maxdim=None):
        idx = lambda i: i if isinstance(i, Index) else Index(i)
        pa, pb, bond, ga, gb = map(idx, (ind_physical_a, ind_physical_b, ind_bond_ab, ind_physical_g_a,
                                         ind_physical_g_b))
        AB = self.binary_einsum(binary_inds_c(A.inds, B.inds, dims=[bond]), A, B)
        theta = self.binary_einsum(binary_inds_c(AB.inds, G.inds, dims=[pa, pb]), AB, G)
        theta = Tensor(theta.data, [pa if i == ga else pb if i == gb else i for i in theta.inds])
        inds_u, inds_v = setdiff(A.inds, [bond]), setdiff(B.inds, [bond])
        keep = 0 if maxdim is None else int(maxdim)
        U, S, V = self.tensor_svd_thin(theta, inds_u, inds_v, bond, keep, normalize, sqrt_s=absorb == "equally")
        if absorb is None:
            return U, S, V
        if absorb in ("u", "equally"):
            self.hadamard_(U, U, S)
        if absorb in ("v", "equally"):
            self.hadamard_(V, V, S)
        if absorb not in ("u", "v", "equally"):
            raise ArgumentError(f"unknown absorb behaviour {absorb!r}")
        return U, V


for _f, _doms in (("binary_einsum", (DomainCUDA, DomainCUDA)), ("binary_einsum_", (DomainCUDA, DomainCUDA, DomainCUDA)),
                  ("unary_einsum", (DomainCUDA,)), ("unary_einsum_", (DomainCUDA, DomainCUDA)),
                  ("hadamard", (DomainCUDA, DomainCUDA)), ("hadamard_", (DomainCUDA, DomainCUDA, DomainCUDA)),
                  ("simple_update", (DomainCUDA, DomainCUDA, DomainCUDA)), ("tensor_svd_thin", (DomainCUDA,))):
    register_rule(_f, _doms, BackendGB300)


# ---------------------------------------------------------------------------
# front-ends
def _labels(xs) -> list:
    if isinstance(xs, (Index, str)):
        xs = [xs]
    return [x if isinstance(x, Index) else Index(x) for x in xs]


def binary_inds_c(ia, ib, dims=None, out=None) -> list:
    """Output labels of binary_einsum(a, b; dims, out)
    (src/Operations/binary_einsum.jl:33-40)."""
    if out is not None:
        return _labels(out)
    dims = intersect(ia, ib) if dims is None else _labels(dims)
    inds_sum = intersect(dims, ia, ib)
    return setdiff(union(ia, ib), inds_sum)


def unary_inds_y(ix, dims=None, out=None) -> list:
    """Output labels of unary_einsum(x; dims, out) (src/Operations/unary_einsum.jl:26-32)."""
    if out is not None:
        return _labels(out)
    dims = nonunique(ix) if dims is None else _labels(dims)
    return setdiff(ix, intersect(dims, ix))


def binary_einsum(a: Tensor, b: Tensor, dims=None, out=None) -> Tensor:
    """Contract ``a`` and ``b`` (src/Operations/binary_einsum.jl:33-51).

    dims: labels to contract (default: the shared labels);
    out:  output labels (default: a's free labels, then b's, in order)."""
    inds_c = binary_inds_c(a.inds, b.inds, dims, out)
    backend = choose_backend(binary_einsum, a.data, b.data)
    return backend.binary_einsum(inds_c, a, b)


def binary_einsum_(c: Tensor, a: Tensor, b: Tensor) -> Tensor:
    """In-place contraction into ``c`` (src/Operations/binary_einsum.jl:57-70)."""
    backend = choose_backend(binary_einsum_, c.data, a.data, b.data)
    backend.binary_einsum_(c, a, b)
    return c


def unary_einsum(x: Tensor, dims=None, out=None) -> Tensor:
    """Trace / diagonal / partial sum (src/Operations/unary_einsum.jl:26-36).

    dims: labels summed over (default: the repeated labels);
    out:  output labels (default: the remaining unique labels)."""
    inds_y = unary_inds_y(x.inds, dims, out)
    backend = choose_backend(unary_einsum, x.data)
    return backend.unary_einsum(inds_y, x)


def unary_einsum_(y: Tensor, x: Tensor) -> Tensor:
    """In-place unary contraction into ``y`` (src/Operations/unary_einsum.jl:42-46)."""
    backend = choose_backend(unary_einsum_, y.data, x.data)
    backend.unary_einsum_(y, x)
    return y


def hadamard(a: Tensor, b: Tensor) -> Tensor:
    """Broadcast element-wise product (src/Operations/hadamard.jl:7-13): the
    operand of lower rank is broadcast along the other's labels; its labels
    must be a subset of the other's."""
    if a.ndim < b.ndim:
        a, b = b, a
    if any(i not in a.inds for i in b.inds):
        raise ArgumentError("hadamard: inds(b) must be a subset of inds(a)")
    backend = choose_backend(hadamard, a.data, b.data)
    return backend.hadamard(a, b)


def hadamard_(c: Tensor, a: Tensor, b: Tensor) -> Tensor:
    """In-place broadcast product into ``c`` (src/Operations/hadamard.jl:19-28):
    inds(c) == inds(a), inds(b) a subset of inds(a)."""
    if a.ndim < b.ndim:
        a, b = b, a
    if list(c.inds) != list(a.inds):
        raise ArgumentError("hadamard!: inds(c) must equal inds(a)")
    if any(i not in a.inds for i in b.inds):
        raise ArgumentError("hadamard!: inds(b) must be a subset of inds(a)")
    backend = choose_backend(hadamard_, c.data, a.data, b.data)
    backend.hadamard_(c, a, b)
    return c


def permutedims(t: Tensor, perm) -> Tensor:
    """Device permutation by labels (src/Tensor.jl:316-319) through the
    permutation kernel; ``perm`` is a list of Index labels or positions."""
    if t.ndim == 0:
        return t
    labels = [t.inds[p] if isinstance(p, int) else (p if isinstance(p, Index) else Index(p)) for p in perm]
    if sorted(map(repr, labels)) != sorted(map(repr, t.inds)):
        raise ArgumentError("permutation must use every label once")
    _require_cuda(t.data)
    y = empty_colmajor([t.size(i) for i in labels], t.dtype, t.data.device)
    modes = _modes_for(t.inds)
    (xd, kx) = _lib.make_desc(*_desc_args(t.data, t.inds, modes))
    (yd, ky) = _lib.make_desc(*_desc_args(y, labels, modes))
    lib = _lib.load()
    check(lib.mgb_permute(ctypes.byref(xd), ctypes.byref(yd), t.data.data_ptr(), y.data_ptr(),
                          _stream_handle(y.device)), lib)
    return Tensor(y, labels)


def device_status(device=None) -> int:
    """Reads and clears the device status word (0 = no timeout recorded)."""
    lib = _lib.load()
    st = ctypes.c_int32(0)
    check(lib.mgb_device_status(_stream_handle(device or torch.cuda.current_device()), ctypes.byref(st)), lib)
    return int(st.value)


def tensor_svd_thin(x: Tensor, inds_u=None, inds_v=None, ind_s=None):
    """Thin SVD of a tensor (src/Operations/tensor_svd.jl:66-69,98-125):
    U (inds_u..., ind_s), s (ind_s) and conj(V) (inds_v..., ind_s); either
    inds_u or inds_v may be omitted (the other labels of x)."""
    if inds_u is None and inds_v is None:
        raise ArgumentError("tensor_svd_thin: give inds_u or inds_v")
    if inds_u is None:
        inds_u = setdiff(x.inds, _labels(inds_v))
    if inds_v is None:
        inds_v = setdiff(x.inds, _labels(inds_u))
    ind_s = Index("svd") if ind_s is None else ind_s
    backend = choose_backend(tensor_svd_thin, x.data)
    return backend.tensor_svd_thin(x, _labels(inds_u), _labels(inds_v), ind_s)


def simple_update(A: Tensor, ind_physical_a, B: Tensor, ind_physical_b, ind_bond_ab, G: Tensor, ind_physical_g_a,
                  ind_physical_g_b, normalize: bool = False, absorb=None, maxdim=None):
    """Muscle's simple_update (src/Operations/simple_update.jl:16-82): apply
    the gate G to the pair A, B joined by ind_bond_ab and refactor it: returns
    (U, s, V), or (U, V) with s absorbed (absorb = "u", "v" or "equally",
    the reference's AbsorbU / AbsorbV / AbsorbEqually)."""
    backend = choose_backend(simple_update, A.data, B.data, G.data)
    return backend.simple_update(A, ind_physical_a, B, ind_physical_b, ind_bond_ab, G, ind_physical_g_a,
                                 ind_physical_g_b, normalize=normalize, absorb=absorb, maxdim=maxdim)
