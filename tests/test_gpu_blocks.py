"""Block-partitioned contraction on the device (the Dagger decomposition of
ext/MuscleDaggerExt/binary_einsum.jl:64-119): every block pair through one
grouped launch set, partial results of contracted-label blocks summed by the
unary kernel, against the oracle's whole contraction."""
import numpy as np
import pytest
import torch

import muscle_gb300 as m
from oracle import muscle_ref as ref
from tests.gpu_util import TOL, to_dev, to_np
from tests.test_blocks import CASES

pytestmark = pytest.mark.gpu


def _data(case, dtype, seed=0):
    ia, sa, ib, sb, ic, bs = case
    rng = np.random.default_rng(seed)
    cx = np.dtype(dtype).kind == "c"
    mk = lambda s: np.asfortranarray((rng.standard_normal(s) + (1j * rng.standard_normal(s) if cx else 0))
                                     .astype(dtype))
    return mk(sa), mk(sb)


@pytest.mark.parametrize("dtype", [np.complex128, np.float64, np.complex64, np.float32])
@pytest.mark.parametrize("case", CASES)
def test_blocks_against_the_oracle(case, dtype):
    ia, sa, ib, sb, ic, bs = case
    a, b = _data(case, dtype)
    A, B = m.Tensor(to_dev(a), ia), m.Tensor(to_dev(b), ib)
    C = m.block_einsum(A, B, bs, out=ic)
    torch.cuda.synchronize()
    assert [i.tag for i in C.inds] == ic
    want = ref.contract(a, ia, b, ib, ic)
    assert ref.rel_fro(to_np(C.data), want) <= TOL[dtype]


@pytest.mark.parametrize("form", ["plain", "ozaki", "auto"])
def test_forms_and_given_output(form):
    ia, sa, ib, sb, ic, bs = CASES[1]
    a, b = _data(CASES[1], np.complex128, seed=1)
    A, B = m.Tensor(to_dev(a), ia), m.Tensor(to_dev(b), ib)
    C = m.Tensor(m.empty_colmajor([{"n": 5, "i": 4, "m": 3, "j": 6}[x] for x in ic], torch.complex128, "cuda"), ic)
    C.data.fill_(float("nan"))  # every element is written
    out = m.block_einsum(A, B, bs, c=C, form=form)
    torch.cuda.synchronize()
    assert out is C
    assert ref.rel_fro(to_np(C.data), ref.contract(a, ia, b, ib, ic)) <= 1e-13


def test_replicas_add_up_to_the_whole():
    """Two replicas (ranks 0 and 1 of 2) each write their own output blocks
    into a zero output; the sum of the two is the whole contraction and they
    share no block."""
    case = (["i", "k"], (256, 384), ["k", "j"], (384, 192), ["i", "j"], {"i": 64, "k": 128, "j": 64})
    ia, sa, ib, sb, ic, bs = case
    a, b = _data(case, np.complex128, seed=2)
    A, B = m.Tensor(to_dev(a), ia), m.Tensor(to_dev(b), ib)
    parts = [m.block_einsum(A, B, bs, rank=r, world=2) for r in range(2)]
    torch.cuda.synchronize()
    p0, p1 = to_np(parts[0].data), to_np(parts[1].data)
    assert not np.any((p0 != 0) & (p1 != 0))
    want = ref.contract(a, ia, b, ib, ic)
    assert ref.rel_fro(p0 + p1, want) <= 1e-13


def test_large_contracted_split():
    """A 1024 x 2048 by 2048 x 768 ComplexF64 product with the contracted label
    in eight blocks and both output labels in two: 4 output blocks of 8
    partial products each."""
    ia, ib, ic = ["i", "k"], ["k", "j"], ["i", "j"]
    a, b = _data((ia, (1024, 2048), ib, (2048, 768), ic, {}), np.complex128, seed=4)
    A, B = m.Tensor(to_dev(a), ia), m.Tensor(to_dev(b), ib)
    C = m.block_einsum(A, B, {"i": 512, "k": 256, "j": 384})
    torch.cuda.synchronize()
    assert ref.rel_fro(to_np(C.data), a @ b) <= 1e-13


def test_block_pairs_share_plans():
    """Equal block shapes share one plan: a 4 x 4 x 4 split of a square
    product makes 64 members over a single plan signature."""
    a, b = _data((["i", "k"], (512, 512), ["k", "j"], (512, 512), ["i", "j"], {}), np.float64, seed=5)
    A, B = m.Tensor(to_dev(a), ["i", "k"]), m.Tensor(to_dev(b), ["k", "j"])
    bc = m.BlockContraction(A, B, {"i": 128, "j": 128, "k": 128})
    assert len(bc.group.items) == 64 and len(bc.reductions) == 16
    assert len({p.handle.value for p in bc.group.plans}) == 1
    for _ in range(2):  # prepared once, executed twice
        C = bc.execute()
    torch.cuda.synchronize()
    assert ref.rel_fro(to_np(C.data), a @ b) <= 1e-13
