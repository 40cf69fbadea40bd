"""Permutations through the C ABI (mgb_permute) with arbitrary strided source
and destination views, bit-exact against torch's own copy. The cases cover
the TMA-staged transpose of same-type 8- and 16-byte elements (tiles of 32
or 64 rows, ragged edges, zero to three outer modes in any stride order,
destination columns of odd length) and the shapes that it hands back to the
register-tiled kernels (four outer modes, 8-byte sources that start off a
16-byte boundary or have odd row strides)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DTYPES = [torch.float64, torch.complex64, torch.complex128]


def _rand(n, dtype, gen):
    return torch.randn(n, dtype=dtype, generator=gen)


def _view(buf, offset, shape, strides):
    return buf.as_strided(tuple(shape), tuple(strides), offset)


def _permute_abi(x, ix, y, iy):
    """Y[iy] = X[ix] through mgb_permute; x and y are torch views on cuda."""
    from muscle_gb300 import _lib
    from muscle_gb300.ops import _desc_args, _modes_for

    modes = _modes_for(ix, iy)
    xd, kx = _lib.make_desc(*_desc_args(x, ix, modes))
    yd, ky = _lib.make_desc(*_desc_args(y, iy, modes))
    lib = _lib.load()
    st = lib.mgb_permute(ctypes.byref(xd), ctypes.byref(yd), x.data_ptr(), y.data_ptr(),
                         torch.cuda.current_stream().cuda_stream)
    _lib.check(st, lib)
    torch.cuda.synchronize()


def _dense_strides(shape, pad_first=0):
    """Column-major strides; the first stride after mode 0 padded by pad_first."""
    s, acc = [], 1
    for d, e in enumerate(shape):
        s.append(acc)
        acc *= e + (pad_first if d == 0 else 0)
    return s, acc


# (X extents by label, X label order, Y label order, pad of X's mode-0 row, pad of Y's, X offset)
CASES = [
    ({"a": 96, "b": 64}, "ba", "ab", 0, 0, 0),                     # 32-row tiles (a = 96), no outer mode
    ({"a": 128, "b": 50}, "ba", "ab", 0, 0, 0),                    # 64-row tiles, ragged b
    ({"a": 33, "b": 17}, "ba", "ab", 1, 1, 0),                     # ragged both ways, odd a with padded Y
    ({"a": 7, "b": 3, "c": 5}, "bca", "acb", 1, 1, 0),             # one outer mode
    ({"a": 65, "b": 40, "c": 3, "d": 4}, "bcda", "adcb", 0, 1, 0),  # two outer modes
    ({"a": 40, "b": 16, "c": 3, "d": 2, "e": 5}, "bdeca", "acdbe", 0, 2, 0),  # three, X strides unsorted
    ({"a": 9, "b": 16, "c": 2, "d": 3, "e": 2, "f": 2}, "bcdefa", "afedcb", 0, 0, 0),  # four: fallback
    ({"a": 64, "b": 33}, "ba", "ab", 0, 0, 1),                     # source off a 16-byte boundary
    ({"a": 64, "b": 33}, "ba", "ab", 0, 0, 0),                     # odd source row stride
]


@pytest.mark.parametrize("dtype", DTYPES, ids=str)
@pytest.mark.parametrize("case", range(len(CASES)))
def test_permute_views(dtype, case):
    ext, xl, yl, padx, pady, xoff = CASES[case]
    gen = torch.Generator().manual_seed(17 + case)
    xshape = [ext[c] for c in xl]
    yshape = [ext[c] for c in yl]
    xs, xn = _dense_strides(xshape, padx)
    ys, yn = _dense_strides(yshape, pady)
    xbuf = _rand(xn + xoff, dtype, gen).cuda()
    X = _view(xbuf, xoff, xshape, xs)
    ybuf = torch.full((yn,), 7, dtype=dtype, device="cuda")
    Y = _view(ybuf, 0, yshape, ys)
    _permute_abi(X, list(xl), Y, list(yl))
    want = X.permute(*[xl.index(c) for c in yl])
    assert torch.equal(Y, want), (dtype, case)
    # the padding of Y stays untouched
    mask = torch.ones(yn, dtype=torch.bool, device="cuda")
    mask[_view(torch.arange(yn, device="cuda"), 0, yshape, ys).flatten()] = False
    assert torch.all(ybuf[mask] == 7)


def test_permute_full_tiles_many_outer():
    """Many tiles per CTA of the persistent grid (every stage of the ring
    reused several times), 64-row and 32-row tiles, each element type."""
    gen = torch.Generator().manual_seed(3)
    for dtype in DTYPES:
        for shape, perm in (([64, 96, 64, 12, 8], [1, 3, 0, 2, 4]), ([96, 64, 30, 20], [1, 0, 3, 2])):
            x = _rand(int(np.prod(shape)), dtype, gen).cuda().reshape(list(reversed(shape)))
            x = x.permute(*reversed(range(len(shape))))  # column-major view with shape `shape`
            labels = [f"m{d}" for d in range(len(shape))]
            ylab = [labels[p] for p in perm]
            ys, yn = _dense_strides([shape[p] for p in perm])
            y = torch.empty(yn, dtype=dtype, device="cuda").as_strided([shape[p] for p in perm], ys)
            _permute_abi(x, labels, y, ylab)
            assert torch.equal(y, x.permute(*perm)), (dtype, shape)
