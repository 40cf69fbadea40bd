"""Seeded random contraction structures against the CPU oracle (96 single
calls in every form, and 32 as one group and through the serving loop): every
combination of free, contracted and batch labels (none to three of each, so
scalars, inner, outer and batched products all occur), labels in random
order in A, B and C, extents from 1 to 40, operands as permuted and strided
device views, same-type and real x complex operands, in every form. The
tolerances are those of the parity tests: 1e-13 relative Frobenius for
Float64 / ComplexF64 results and 1e-5 for Float32 / ComplexF32, with exact
output label order and result type."""
import numpy as np
import pytest
import torch

from oracle import muscle_ref as ref
from tests.gpu_util import TOL, to_np

pytestmark = pytest.mark.gpu

DTYPES = [
    (np.float64, np.float64),
    (np.complex128, np.complex128),
    (np.float32, np.float32),
    (np.complex64, np.complex64),
    (np.float64, np.complex128),
    (np.complex128, np.float64),
    (np.float32, np.complex64),
    (np.complex64, np.float32),
]
NCASES = 96


def structure(rng):
    """Labels and extents of one random contraction."""
    counts = {g: int(rng.integers(0, 4)) for g in ("a", "b", "k")}
    counts["l"] = int(rng.integers(0, 3))  # batch labels (in A, B and C)
    labels = {g: [f"{g}{i}" for i in range(n)] for g, n in counts.items()}
    ext = {}
    for lab in sum(labels.values(), []):
        ext[lab] = int(rng.integers(1, 8))
    big = list(ext)
    if big:  # one larger extent crosses the tile edges
        ext[big[int(rng.integers(0, len(big)))]] = int(rng.integers(20, 41))
    ia = labels["a"] + labels["k"] + labels["l"]
    ib = labels["k"] + labels["b"] + labels["l"]
    ic = labels["a"] + labels["b"] + labels["l"]
    ia, ib, ic = ([str(v) for v in rng.permutation(x)] if x else [] for x in (ia, ib, ic))
    return ia, ib, ic, ext


def values(rng, shape, dtype):
    x = rng.standard_normal(shape)
    if np.issubdtype(dtype, np.complexfloating):
        x = x + 1j * rng.standard_normal(shape)
    return np.array(x.astype(dtype), order="F")


def device_view(rng, x):
    """x on the device as a view with permuted and (for one mode) doubled
    strides: column-major storage of x permuted, every other element along
    one mode, then indexed back to x's own mode order."""
    if x.ndim == 0:
        return torch.from_numpy(np.asarray(x)).cuda()
    perm = rng.permutation(x.ndim)
    xp = np.transpose(x, perm)
    stride_mode = int(rng.integers(0, x.ndim))
    shape = list(xp.shape)
    shape[stride_mode] *= 2
    buf = np.zeros(shape, dtype=x.dtype, order="F")
    sl = [slice(None)] * x.ndim
    sl[stride_mode] = slice(0, None, 2)
    buf[tuple(sl)] = xp
    dev = torch.from_numpy(buf).cuda()[tuple(sl)]
    view = dev.permute(*np.argsort(perm).tolist())
    assert tuple(view.shape) == x.shape
    return view


@pytest.mark.parametrize("case", range(NCASES))
def test_random_structure(case):
    import muscle_gb300 as m

    rng = np.random.default_rng(5000 + case)
    ia, ib, ic, ext = structure(rng)
    ta, tb = DTYPES[case % len(DTYPES)]
    a = values(rng, [ext[x] for x in ia], ta)
    b = values(rng, [ext[x] for x in ib], tb)
    want = ref.contract(a, ia, b, ib, ic)
    rt = np.result_type(ta, tb).type
    if rt in (np.float64, np.complex128):
        forms = [("plain", 0), ("ozaki", 0), ("ozaki", 7), ("auto", 0)]
    else:
        forms = [("plain", 0), ("bf16x3", 0), ("auto", 0)]
    views = rng.random() < 0.5
    A = m.Tensor(device_view(rng, a) if views else torch.from_numpy(a).cuda(), ia)
    B = m.Tensor(device_view(rng, b) if views else torch.from_numpy(b).cuda(), ib)
    for form, slices in forms:
        with m.with_backend(m.BackendGB300(form, slices)):
            C = m.binary_einsum(A, B, out=ic)
        torch.cuda.synchronize()
        got = to_np(C.data)
        assert [i.tag for i in C.inds] == ic, (case, form)
        assert got.dtype == want.dtype, (case, form)
        err = ref.rel_fro(got, want)
        assert err <= TOL[rt], (case, form, slices, ia, ib, ic, err)
    assert m.device_status() == 0


TORCH = {np.float64: torch.float64, np.complex128: torch.complex128, np.float32: torch.float32,
         np.complex64: torch.complex64}


def test_random_structures_grouped_and_served():
    """32 random structures as one group, under every schedule (one
    persistent launch per kernel variant, or every bucket's own launches, on
    one stream or three parallel parts), then through the serving loop."""
    import muscle_gb300 as m

    items, wants, tols = [], [], []
    for i in range(32):
        rng = np.random.default_rng(7000 + i)
        ia, ib, ic, ext = structure(rng)
        ta, tb = DTYPES[i % len(DTYPES)]
        a = values(rng, [ext[x] for x in ia], ta)
        b = values(rng, [ext[x] for x in ib], tb)
        rt = np.result_type(ta, tb).type
        wants.append(ref.contract(a, ia, b, ib, ic))
        tols.append(TOL[rt])
        views = i % 2 == 1
        A = m.Tensor(device_view(rng, a) if views else torch.from_numpy(a).cuda(), ia)
        B = m.Tensor(device_view(rng, b) if views else torch.from_numpy(b).cuda(), ib)
        C = m.Tensor(m.zeros_colmajor([ext[x] for x in ic], TORCH[rt], "cuda"), ic)
        items.append((C, A, B))
    forms = ["ozaki" if np.dtype(w.dtype).type in (np.float64, np.complex128) else "bf16x3" for w in wants]
    g = m.Group(items, forms)
    for parts, persistent in ((1, True), (1, False), (3, True), (3, False)):
        for C, _, _ in items:
            C.data.fill_(float("nan"))
        g.execute(parts=parts, persistent=persistent)
        torch.cuda.synchronize()
        for j, ((C, _, _), want, tol) in enumerate(zip(items, wants, tols)):
            err = ref.rel_fro(to_np(C.data), want)
            assert err <= tol, (parts, persistent, j, err)
    with m.Server(budget_bytes=1 << 30, streams=2, max_batch=16, form="auto") as srv:
        pending = [srv.submit(A, B, out=[i.tag for i in C.inds]) for C, A, B in items]
        outs = [p.result(timeout=120) for p in pending]
    for j, (C, want, tol) in enumerate(zip(outs, wants, tols)):
        assert ref.rel_fro(to_np(C.data), want) <= tol, ("served", j)
    assert m.device_status() == 0
