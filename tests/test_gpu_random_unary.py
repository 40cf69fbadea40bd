"""Seeded random unary structures and permutations against the CPU oracle.

unary_einsum: labels repeated two or three times in X (diagonals), kept
labels in random order, summed labels, extents from 1 to 40, X as a permuted
and strided device view, four element types; 1e-13 / 1e-5 relative
Frobenius. permutedims: ranks 1 to 6, strided views, four element types
(Float64 and ComplexF64 go through the TMA-staged transpose whenever their
strides allow it); bit-exact."""
import numpy as np
import pytest
import torch

from oracle import muscle_ref as ref
from tests.gpu_util import TOL, to_np
from tests.test_gpu_random_structures import device_view, values

pytestmark = pytest.mark.gpu

DTYPES = [np.float64, np.complex128, np.float32, np.complex64]


def unary_structure(rng):
    """X's labels (some repeated) and extents, and Y's labels."""
    n = int(rng.integers(1, 5))
    labels = [f"u{i}" for i in range(n)]
    ext = {lab: int(rng.integers(1, 8)) for lab in labels}
    ext[labels[int(rng.integers(0, n))]] = int(rng.integers(20, 41))
    ix = []
    for lab in labels:
        reps = 1 + (rng.random() < 0.3) + (rng.random() < 0.1)
        ix += [lab] * reps
    ix = [str(v) for v in rng.permutation(ix)]
    kept = [lab for lab in labels if rng.random() < 0.5]
    iy = [str(v) for v in rng.permutation(kept)] if kept else []
    return ix, iy, ext


@pytest.mark.parametrize("case", range(48))
def test_random_unary(case):
    import muscle_gb300 as m

    rng = np.random.default_rng(9000 + case)
    ix, iy, ext = unary_structure(rng)
    dtype = DTYPES[case % len(DTYPES)]
    x = values(rng, [ext[lab] for lab in ix], dtype)
    want = ref.unary(x, ix, iy)
    X = m.Tensor(device_view(rng, x) if case % 2 else torch.from_numpy(x).cuda(), ix)
    Y = m.unary_einsum(X, out=iy)
    torch.cuda.synchronize()
    assert [i.tag for i in Y.inds] == iy
    assert ref.rel_fro(to_np(Y.data), want) <= TOL[dtype], (case, ix, iy)
    assert m.device_status() == 0


@pytest.mark.parametrize("case", range(48))
def test_random_permutation_bit_exact(case):
    import muscle_gb300 as m

    rng = np.random.default_rng(11000 + case)
    nd = int(rng.integers(1, 7))
    shape = [int(rng.integers(1, 6)) for _ in range(nd)]
    shape[int(rng.integers(0, nd))] = int(rng.integers(20, 200))
    dtype = DTYPES[case % len(DTYPES)]
    x = values(rng, shape, dtype)
    ix = [f"p{i}" for i in range(nd)]
    perm = [int(v) for v in rng.permutation(nd)]
    X = m.Tensor(device_view(rng, x) if case % 2 else torch.from_numpy(x).cuda(), ix)
    Y = m.permutedims(X, [ix[p] for p in perm])
    torch.cuda.synchronize()
    assert [i.tag for i in Y.inds] == [ix[p] for p in perm]
    assert np.array_equal(to_np(Y.data), np.transpose(x, perm)), (case, shape, perm)
    assert m.device_status() == 0
