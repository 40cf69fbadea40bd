"""CPU oracle for Muscle.jl's tensor contractions — TEST INFRASTRUCTURE ONLY.

This module restates, in numpy, the algorithm of Muscle.jl's host backend so
that the GPU library can be checked against it. It is imported only by
``tests/``, ``__graft_entry__.smoke()`` (as the checker) and ``bench.py``'s
CPU-baseline / reference arm; the product (``muscle.jl_gb300``) never calls it.

Followed reference code (paths inside the Muscle.jl repository, v0.3.20):
  * label algebra of the front-end ......... src/Operations/binary_einsum.jl:33-51
  * BackendBase: permute -> GEMM -> permute . src/Operations/binary_einsum.jl:76-96
  * in-place variant (inds(c) == [left; right]) src/Operations/binary_einsum.jl:98-121
  * permutedims by labels .................. src/Tensor.jl:316-319
  * findperm (label order comparison) ...... src/Index.jl:20-34
  * batch (hyper) labels kept in the output  test/integration/cuda.jl:126-145,170-180
                                             (cuTENSOR semantics, ext/MuscleCUDAExt.jl:10-41)
  * unary trace / diagonal / sums .......... src/Operations/unary_einsum.jl:26-46,
                                             test/integration/omeinsum.jl:6-100
  * simple_update (contract, SVD, absorb) .. src/Operations/simple_update.jl:35-82,
                                             src/Operations/tensor_svd.jl:98-125
The GEMM is numpy's matmul, i.e. OpenBLAS (scipy-openblas), the same BLAS
family Julia's LinearAlgebra uses. Julia arrays are column-major: reshapes
here use order="F" so that the folded matrices are the same as Julia's.

Parity status: the reference is Julia and no Julia exists in this build
environment, so this restatement cannot be run side by side with it. It is
pinned against every known-answer assertion of the reference's own tests for
this path (tests/golden/kat_cases.json, generated by tests/golden/make_kat.py);
bit-level parity with Julia's BLAS is unpinned (and not expected: BLAS
summation order is unspecified). Floating-point parity is asserted at the
stated tolerances (1e-13 / 1e-5 relative Frobenius).
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np


class ArgumentError(ValueError):
    pass


class DimensionMismatch(ValueError):
    pass


# ---------------------------------------------------------------- label algebra
def _unique(xs):
    out = []
    for x in xs:
        if x not in out:
            out.append(x)
    return out


def setdiff(xs, ys):
    ys = list(ys)
    return [x for x in _unique(xs) if x not in ys]


def intersect(*seqs):
    first, rest = seqs[0], [list(s) for s in seqs[1:]]
    return [x for x in _unique(first) if all(x in r for r in rest)]


def union(*seqs):
    out = []
    for s in seqs:
        for x in s:
            if x not in out:
                out.append(x)
    return out


def nonunique(xs):
    seen, rep = [], []
    for x in xs:
        if x in seen:
            if x not in rep:
                rep.append(x)
        else:
            seen.append(x)
    return rep


def front_inds_c(ia, ib, dims=None, out=None):
    """Output labels chosen by binary_einsum(a, b; dims, out)
    (src/Operations/binary_einsum.jl:33-40)."""
    if dims is None:
        dims = intersect(ia, ib)
    inds_sum = intersect(dims, ia, ib)
    return list(out) if out is not None else setdiff(union(ia, ib), inds_sum)


def front_inds_y(ix, dims=None, out=None):
    """Output labels chosen by unary_einsum(x; dims, out)
    (src/Operations/unary_einsum.jl:26-32)."""
    if dims is None:
        dims = nonunique(ix)
    inds_sum = intersect(dims, ix)
    return list(out) if out is not None else setdiff(ix, inds_sum)


# ---------------------------------------------------------------- contractions
def _permute(x, labels, to):
    """permutedims by labels (src/Tensor.jl:316-319)."""
    return np.transpose(x, [labels.index(i) for i in to]) if to else x


def _prod(xs):
    p = 1
    for x in xs:
        p *= int(x)
    return p


def backend_base(inds_c, a, ia, b, ib):
    """BackendBase binary_einsum (src/Operations/binary_einsum.jl:76-96)."""
    ia, ib, inds_c = list(ia), list(ib), list(inds_c)
    inds_contract = intersect(ia, ib)
    inds_left = setdiff(ia, inds_contract)
    inds_right = setdiff(ib, inds_contract)
    if any(i in inds_contract for i in inds_c) or sorted(map(repr, inds_c)) != sorted(
        map(repr, setdiff(union(ia, ib), inds_contract))
    ):
        raise ArgumentError("`BackendBase` can't deal with hyperindices. Load OMEinsum and use `BackendOMEinsum` instead.")
    sl = [a.shape[ia.index(i)] for i in inds_left]
    sr = [b.shape[ib.index(i)] for i in inds_right]
    sk = [a.shape[ia.index(i)] for i in inds_contract]
    a_mat = _permute(a, ia, inds_left + inds_contract).reshape(_prod(sl), _prod(sk), order="F")
    b_mat = _permute(b, ib, inds_contract + inds_right).reshape(_prod(sk), _prod(sr), order="F")
    c_mat = a_mat @ b_mat
    c = c_mat.reshape(sl + sr, order="F")
    return _permute(c, inds_left + inds_right, inds_c)


def contract(a, ia, b, ib, ic):
    """Contraction with cuTENSOR label semantics, as expected of the CUDA path
    by test/integration/cuda.jl:126-145,170-180: labels of A and B absent from C
    are summed; labels in A, B and C are batch labels. Computed as BackendBase
    (permute -> BLAS GEMM -> permute) once per batch entry."""
    ia, ib, ic = list(ia), list(ib), list(ic)
    for x, lx in ((a, ia), (b, ib)):
        if len(set(map(repr, lx))) != len(lx):
            raise ArgumentError("repeated label in a binary contraction operand")
    size = {}
    for x, lx in ((a, ia), (b, ib)):
        for d, i in enumerate(lx):
            if i in size and size[i] != x.shape[d]:
                raise DimensionMismatch(f"label {i} has different extents")
            size[i] = x.shape[d]
    for i in ic:
        if i not in size:
            raise ArgumentError(f"output label {i} is in neither operand")
    batch = [i for i in ia if i in ib and i in ic]
    contr = [i for i in ia if i in ib and i not in ic]
    left = [i for i in ia if i not in ib]
    right = [i for i in ib if i not in ia]
    for i in left + right:
        if i not in ic:
            raise ArgumentError(f"label {i} appears in one operand only and not in the output")
    dt = np.result_type(a.dtype, b.dtype)
    M, N, K, L = (_prod(size[i] for i in g) for g in (left, right, contr, batch))
    am = _permute(a, ia, left + contr + batch).astype(dt, copy=False).reshape(M, K, L, order="F")
    bm = _permute(b, ib, contr + right + batch).astype(dt, copy=False).reshape(K, N, L, order="F")
    cm = np.empty((M, N, L), dtype=dt, order="F")
    for l in range(L):
        cm[:, :, l] = am[:, :, l] @ bm[:, :, l]
    c = cm.reshape([size[i] for i in left + right + batch], order="F")
    return _permute(c, left + right + batch, ic)


def unary(x, ix, iy):
    """unary_einsum with OMEinsum semantics (ext/MuscleOMEinsumExt.jl:25-38):
    repeated labels of X take the diagonal, labels absent from Y are summed."""
    ix, iy = list(ix), list(iy)
    for i in iy:
        if i not in ix:
            raise ArgumentError("Output indices must be a subset of input indices")
    labels = _unique(ix)
    letters = {lab: chr(ord("a") + n) for n, lab in enumerate(labels)}
    spec = "".join(letters[i] for i in ix) + "->" + "".join(letters[i] for i in iy)
    return np.einsum(spec, x)


def hadamard(a, ia, b, ib):
    """BackendBase hadamard (src/Operations/hadamard.jl:34-77): c = a .* b with
    the operand of lower rank broadcast along the other's labels; c has a's
    labels and a's element type (c = copy(a), then c .= a .* b), so a complex
    product into a real a is an error (Julia's InexactError).

    b is brought into a's label order by labels. The reference does this with
    permutedims(b, findperm(inds(b), inds(a) ∩ inds(b))) (hadamard.jl:66-69),
    which equals the label-wise order whenever that permutation is its own
    inverse (every case of its tests: rank(b) <= 2); for a 3-cycle of labels it
    would use the inverse permutation."""
    ia, ib = list(ia), list(ib)
    if a.ndim < b.ndim:
        a, ia, b, ib = b, ib, a, ia
    if any(i not in ia for i in ib):
        raise ArgumentError("hadamard: inds(b) must be a subset of inds(a)")
    if b.ndim == 0:
        prod = a * b
    else:
        order = [i for i in ia if i in ib]
        bb = np.transpose(b, [ib.index(i) for i in order])
        shape = [a.shape[d] if ia[d] in ib else 1 for d in range(len(ia))]
        prod = a * bb.reshape(shape, order="F")
    if np.iscomplexobj(prod) and not np.iscomplexobj(a) and np.any(np.imag(prod) != 0):
        raise ArgumentError("hadamard: InexactError (complex product into a real array)")
    return np.array(np.real(prod) if not np.iscomplexobj(a) else prod, dtype=a.dtype, order="F"), ia


def tensor_svd_thin(x, ix, inds_u, inds_v):
    """tensor_svd_thin of BackendBase (src/Operations/tensor_svd.jl:98-125):
    permute to [inds_u; inds_v], reshape to a matrix (column-major), thin SVD
    (numpy's LAPACK, as Julia's LinearAlgebra.svd), and the factors as tensors:
    U (inds_u..., s), s, and conj(V) (inds_v..., s)."""
    ix, inds_u, inds_v = list(ix), list(inds_u), list(inds_v)
    su = [x.shape[ix.index(i)] for i in inds_u]
    sv = [x.shape[ix.index(i)] for i in inds_v]
    xm = _permute(x, ix, inds_u + inds_v).reshape(_prod(su), _prod(sv), order="F")
    u, s, vh = np.linalg.svd(xm, full_matrices=False)
    k = s.shape[0]
    U = np.array(u.reshape(su + [k], order="F"), order="F")
    Vt = np.array(vh.T.reshape(sv + [k], order="F"), order="F")  # conj(V) = (V^H)^T
    return U, s, Vt


def simple_update(a, ia, phys_a, b, ib, phys_b, bond, g, ig, g_a, g_b, normalize=False, absorb=None, maxdim=None):
    """simple_update of Muscle (src/Operations/simple_update.jl:35-82): contract
    A and B over the bond, then with the gate G over the physical labels,
    rename G's output labels back, thin SVD with the bond as the new label,
    truncate to maxdim, normalise, absorb. absorb: None, "u", "v" or
    "equally". Returns (U, s, Vt) or (U, Vt), each an (array, labels) pair."""
    ia, ib, ig = list(ia), list(ib), list(ig)
    l1 = setdiff(union(ia, ib), [bond])
    t1 = contract(a, ia, b, ib, l1)
    l2 = setdiff(union(l1, ig), [phys_a, phys_b])
    theta = contract(t1, l1, g, ig, l2)
    l2 = [phys_a if i == g_a else phys_b if i == g_b else i for i in l2]
    inds_u, inds_v = setdiff(ia, [bond]), setdiff(ib, [bond])
    U, s, Vt = tensor_svd_thin(theta, l2, inds_u, inds_v)
    if maxdim is not None:
        k = min(maxdim, s.shape[0])
        U, s, Vt = U[..., :k], s[:k], Vt[..., :k]
    if normalize:
        s = s / np.linalg.norm(s)
    lu, lv = inds_u + [bond], inds_v + [bond]
    if absorb is None:
        return (U, lu), (s, [bond]), (Vt, lv)
    if absorb == "u":
        U = U * s
    elif absorb == "v":
        Vt = Vt * s
    elif absorb == "equally":
        U, Vt = U * np.sqrt(s), Vt * np.sqrt(s)
    return (np.array(U, order="F"), lu), (np.array(Vt, order="F"), lv)


def exact_entries(a, ia, b, ib, ic, positions):
    """Exact (rational) values of selected output entries, used to bound the
    oracle's own rounding error. positions: list of index tuples of C."""
    ia, ib, ic = list(ia), list(ib), list(ic)
    contr = [i for i in ia if i in ib and i not in ic]
    size = {i: a.shape[d] for d, i in enumerate(ia)}
    size.update({i: b.shape[d] for d, i in enumerate(ib)})
    out = []
    cx = np.iscomplexobj(a) or np.iscomplexobj(b)
    for pos in positions:
        fixed = dict(zip(ic, pos))
        re, im = Fraction(0), Fraction(0)
        for kidx in np.ndindex(*[size[i] for i in contr]):
            lab = dict(fixed)
            lab.update(zip(contr, kidx))
            av = a[tuple(lab[i] for i in ia)]
            bv = b[tuple(lab[i] for i in ib)]
            ar, ai = Fraction(float(np.real(av))), Fraction(float(np.imag(av)))
            br, bi = Fraction(float(np.real(bv))), Fraction(float(np.imag(bv)))
            re += ar * br - ai * bi
            im += ar * bi + ai * br
        out.append(complex(float(re), float(im)) if cx else float(re))
    return out


def _veltkamp(x):
    """x = hi + lo with hi, lo of at most 26 significant bits each, so that
    every product of two halves is exact in float64 (Dekker 1971)."""
    c = 134217729.0 * x  # 2^27 + 1
    hi = c - (c - x)
    return hi, x - hi


def _exact_products(x, y):
    xh, xl = _veltkamp(np.ascontiguousarray(x, dtype=np.float64).ravel())
    yh, yl = _veltkamp(np.ascontiguousarray(y, dtype=np.float64).ravel())
    return [xh * yh, xh * yl, xl * yh, xl * yl]


def exact_dot(x, y):
    """Correctly rounded sum_k x_k y_k of two float64 or complex128 vectors:
    every product is split into exact float64 parts (Veltkamp/Dekker) and the
    parts are summed with math.fsum (Shewchuk's exact summation)."""
    x = np.asarray(x)
    y = np.asarray(y)
    if not (np.iscomplexobj(x) or np.iscomplexobj(y)):
        return math.fsum(np.concatenate(_exact_products(x, y)))
    xr, xi, yr, yi = x.real, x.imag, y.real, y.imag
    re = np.concatenate(_exact_products(xr, yr) + _exact_products(-xi, yi))
    im = np.concatenate(_exact_products(xr, yi) + _exact_products(xi, yr))
    return complex(math.fsum(re), math.fsum(im))


def exact_entries_fast(a, ia, b, ib, ic, positions):
    """Correctly rounded values of selected entries of C = contract(a, b),
    for checking results (and the FP64 oracle itself) at full problem sizes.
    The contracted set follows the same rule as ``contract``: labels of both
    operands that are not in ``ic``. positions: list of index tuples of C."""
    ia, ib, ic = list(ia), list(ib), list(ic)
    contr = [i for i in ia if i in ib and i not in ic]
    out = []
    for pos in positions:
        fixed = dict(zip(ic, pos))

        def vec(x, ix):
            sel = tuple(fixed[i] if i in fixed else slice(None) for i in ix)
            rest = [i for i in ix if i not in fixed]
            sub = x[sel]
            return np.transpose(sub, [rest.index(i) for i in contr]).ravel(order="F")

        out.append(exact_dot(vec(a, ia), vec(b, ib)))
    return out


def rel_fro(x, ref):
    """Relative Frobenius error ||x - ref|| / ||ref||."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    den = np.linalg.norm(ref.ravel())
    num = np.linalg.norm((x - ref).ravel())
    return float(num / den) if den else float(num)
