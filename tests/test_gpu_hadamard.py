"""hadamard / hadamard! on the device (src/Operations/hadamard.jl): the known
answers of the reference's tests, seeded random broadcasts in every element
type against the oracle (real products bit-exact, complex within rounding),
strided views, in-place aliasing and the errors."""
import numpy as np
import pytest
import torch

import muscle_gb300 as m
from oracle import muscle_ref as ref
from tests.gpu_util import to_dev, to_np
from tests.kat_util import expected_hadamard, make_array

pytestmark = pytest.mark.gpu


def rand(rng, shape, dtype):
    x = rng.standard_normal(shape)
    if np.issubdtype(dtype, np.complexfloating):
        x = x + 1j * rng.standard_normal(shape)
    return np.array(x.astype(dtype), order="F")


def test_kat_hadamard(kat_cases):
    hs = [c for c in kat_cases if c["kind"] == "hadamard"]
    assert hs
    for case in hs:
        a, b = make_array(case["a"]), make_array(case["b"])
        A = m.Tensor(to_dev(a), case["a"]["inds"])
        B = m.Tensor(to_dev(b), case["b"]["inds"])
        exp = case["expect"]
        want = expected_hadamard(exp, b, case["b"]["inds"])
        if case["inplace"]:
            C = m.hadamard_(A, A, B)
            assert C is A
        else:
            C = m.hadamard(A, B)
            C2 = m.hadamard(B, A)  # the operand of lower rank is broadcast
            assert [i.tag for i in C2.inds] == exp["inds"]
            assert np.array_equal(to_np(C2.data), want), case["name"]
        torch.cuda.synchronize()
        assert [i.tag for i in C.inds] == exp["inds"], case["name"]
        assert list(C.data.shape) == exp["shape"]
        assert np.array_equal(to_np(C.data), want), case["name"]


CASES = [
    # (A labels, A extents, B labels)
    (["i", "j", "k"], [33, 70, 9], ["k", "i"]),      # B permuted against A
    (["i", "j", "k"], [300, 4, 5], ["j"]),           # vector along a middle label
    (["a", "b", "c", "d"], [5, 6, 7, 8], ["d", "b", "a"]),  # 3-label B, permutation of order 3
    (["x", "y"], [1000, 3], ["x", "y"]),             # same labels
    (["x", "y"], [1000, 3], []),                     # scalar
    (["l"], [4097], ["l"]),
]


@pytest.mark.parametrize("dta,dtb", [(np.float64, np.float64), (np.float32, np.float32), (np.complex128, np.complex128),
                                     (np.complex64, np.complex64), (np.complex128, np.float64),
                                     (np.float32, np.float64), (np.complex64, np.float32)])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_random_broadcasts(case, dta, dtb):
    ia, ea, ib = CASES[case]
    rng = np.random.default_rng(300 + case)
    a = rand(rng, ea, dta)
    eb = [ea[ia.index(i)] for i in ib]
    b = rand(rng, eb, dtb)
    want, iw = ref.hadamard(a, ia, b, ib)
    C = m.hadamard(m.Tensor(to_dev(a), ia), m.Tensor(to_dev(b), ib))
    got = to_np(C.data)
    assert [i.tag for i in C.inds] == iw and got.dtype == want.dtype
    if np.iscomplexobj(want):
        tol = 1e-15 if want.dtype == np.complex128 else 1e-6
        assert np.max(np.abs(got - want)) <= tol * max(1.0, np.max(np.abs(want)))
    else:
        assert np.array_equal(got, want)


def test_strided_views_and_inplace():
    rng = np.random.default_rng(9)
    big = torch.from_numpy(rng.standard_normal((40, 60))).cuda()
    before = big.clone()
    av = big[::2, 1::3]  # 20 x 20 strided view
    bv = torch.from_numpy(rng.standard_normal(40)).cuda()[::2]
    want, _ = ref.hadamard(to_np(av), ["i", "j"], to_np(bv), ["i"])
    A = m.Tensor(av, ["i", "j"])
    C = m.hadamard(A, m.Tensor(bv, ["i"]))
    assert np.array_equal(to_np(C.data), want)
    # hadamard!(a, a, b) writes into the view itself
    m.hadamard_(A, A, m.Tensor(bv, ["i"]))
    torch.cuda.synchronize()
    assert np.array_equal(to_np(av), want)
    # elements outside the view are untouched
    mask = torch.ones_like(big, dtype=torch.bool)
    mask[::2, 1::3] = False
    assert torch.equal(big[mask], before[mask])


def test_errors():
    A = m.Tensor(torch.ones(2, 3, dtype=torch.float64, device="cuda"), ["i", "j"])
    with pytest.raises(m.ArgumentError):
        m.hadamard(A, m.Tensor(torch.ones(4, dtype=torch.float64, device="cuda"), ["k"]))
    with pytest.raises(m.ArgumentError):
        m.hadamard_(m.Tensor(torch.ones(3, 2, dtype=torch.float64, device="cuda"), ["j", "i"]), A,
                    m.Tensor(torch.ones(3, dtype=torch.float64, device="cuda"), ["j"]))
    with pytest.raises(m.ArgumentError):  # complex product into a real array
        m.hadamard(A, m.Tensor(torch.ones(3, dtype=torch.complex128, device="cuda"), ["j"]))
    with pytest.raises(m.DimensionMismatch):
        m.hadamard(A, m.Tensor(torch.ones(5, dtype=torch.float64, device="cuda"), ["j"]))


def test_large_bandwidth_case():
    """A 2^28-element ComplexF64 array scaled by a vector along its last label:
    every element checked on the device against torch's broadcast product."""
    n0, n1 = 1 << 16, 1 << 12
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    a = torch.randn(n1, n0, dtype=torch.complex128, device="cuda", generator=g).t()  # column-major (n0, n1)
    b = torch.randn(n1, dtype=torch.complex128, device="cuda", generator=g)
    C = m.hadamard(m.Tensor(a, ["x", "y"]), m.Tensor(b, ["y"]))
    want = a * b[None, :]
    err = (C.data - want).abs().max().item()
    assert err <= 1e-15 * want.abs().max().item()
