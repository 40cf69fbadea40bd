"""Seeded random contractions: GPU (every form) against the CPU oracle at the
stated tolerances — 1e-13 relative Frobenius for Float64/ComplexF64, 1e-5 for
Float32/ComplexF32 — with exact output label order; permutations and unary
reductions bit-exact / at 1e-13."""
import numpy as np
import pytest
import torch

from oracle import muscle_ref as ref
from muscle_gb300 import workloads as wl
from tests.gpu_util import TOL, forms_for, run, to_dev, to_np

pytestmark = pytest.mark.gpu

F64_TOL = 1e-13
F32_TOL = 1e-5


def rand(rng, shape, dtype):
    x = rng.standard_normal(shape)
    if np.issubdtype(dtype, np.complexfloating):
        x = x + 1j * rng.standard_normal(shape)
    return np.array(x.astype(dtype), order="F")


CASES = [
    # (A labels, A extents, B labels, B extents, C labels)
    (["i", "j", "k", "l"], [5, 6, 7, 3], ["k", "m", "l", "n"], [7, 4, 3, 9], ["i", "j", "m", "n"]),  # config-1 pattern
    (["a", "b", "c", "d", "e"], [16, 24, 16, 12, 8], ["e", "c", "f", "a"], [8, 16, 32, 16], ["b", "d", "f"]),  # 2a / 4
    (["l", "p", "r"], [128, 4, 128], ["r", "q", "s"], [128, 4, 128], ["l", "p", "q", "s"]),  # 2b / 4
    (["i", "k1", "k2"], [200, 16, 8], ["k2", "j", "k1"], [8, 136, 16], ["i", "j"]),  # config-3 pattern
    (["i", "k1", "k2"], [200, 16, 8], ["k2", "j", "k1"], [8, 136, 16], ["j", "i"]),  # transposed output
    (["x", "y"], [130, 257], ["y", "z"], [257, 3], ["z", "x"]),  # ragged tiles, N < tile
    (["i", "j", "b"], [9, 33, 5], ["j", "k", "b"], [33, 17, 5], ["k", "b", "i"]),  # batch label
    (["i"], [1000], ["i"], [1000], []),  # inner product (M = N = 1)
    (["i", "j"], [37, 41], ["k"], [23], ["k", "i", "j"]),  # outer product (K = 1)
    ([], [], ["i", "j"], [7, 5], ["j", "i"]),  # scale by a scalar
]


@pytest.mark.parametrize("dtype", [np.float64, np.complex128, np.float32, np.complex64])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_random_contractions(case, dtype):
    ia, ea, ib, eb, ic = CASES[case]
    rng = np.random.default_rng(1000 + case)
    a, b = rand(rng, ea, dtype), rand(rng, eb, dtype)
    want = ref.contract(a, ia, b, ib, ic)
    for form, slices in forms_for(dtype):
        got, C = run(a, ia, b, ib, ic, form, slices)
        assert [i.tag for i in C.inds] == ic
        assert got.dtype == want.dtype
        err = ref.rel_fro(got, want)
        assert err <= TOL[dtype], (form, err)


def test_mixed_precision_promotion():
    rng = np.random.default_rng(7)
    a = rand(rng, [20, 30], np.float64)
    b = rand(rng, [30, 11], np.complex128)
    want = ref.contract(a, ["i", "j"], b, ["j", "k"], ["i", "k"])
    for form in ("plain", "ozaki"):
        got, _ = run(a, ["i", "j"], b, ["j", "k"], ["i", "k"], form)
        assert got.dtype == np.complex128 and ref.rel_fro(got, want) <= F64_TOL
    got, _ = run(b.T.copy(order="F"), ["k", "j"], a.T.copy(order="F"), ["j", "i"], ["i", "k"], "ozaki")
    assert ref.rel_fro(got, want) <= F64_TOL
    a32 = rand(rng, [20, 30], np.float32)
    got, _ = run(a32, ["i", "j"], b, ["j", "k"], ["i", "k"], "plain")  # F32 x C64 -> C64
    assert got.dtype == np.complex128
    assert ref.rel_fro(got, ref.contract(a32, ["i", "j"], b, ["j", "k"], ["i", "k"])) <= F64_TOL


def test_strided_views():
    """Non-contiguous operands (views of larger arrays, src/Tensor.jl:287-356)."""
    import muscle_gb300 as m

    rng = np.random.default_rng(11)
    big_a = torch.from_numpy(rand(rng, [40, 50, 6], np.complex128)).cuda()
    big_b = torch.from_numpy(rand(rng, [60, 30], np.complex128)).cuda()
    av = big_a[3:35:2, ::3, 1]  # (16, 17) strided
    bv = big_b[5:22, 2:30:3].transpose(0, 1)  # (10, 17)
    want = ref.contract(to_np(av), ["i", "j"], to_np(bv), ["k", "j"], ["k", "i"])
    for form in ("plain", "ozaki"):
        with m.with_backend(m.BackendGB300(form)):
            C = m.binary_einsum(m.Tensor(av, ["i", "j"]), m.Tensor(bv, ["k", "j"]), out=["k", "i"])
        assert ref.rel_fro(to_np(C.data), want) <= F64_TOL


def test_edge_sizes():
    import muscle_gb300 as m

    # contracted extent 0: empty sum -> zeros
    a = torch.zeros(3, 0, dtype=torch.float64, device="cuda")
    b = torch.zeros(0, 4, dtype=torch.float64, device="cuda")
    for form in ("plain", "ozaki"):
        with m.with_backend(m.BackendGB300(form)):
            C = m.binary_einsum(m.Tensor(a, ["i", "j"]), m.Tensor(b, ["j", "k"]))
        assert np.array_equal(to_np(C.data), np.zeros((3, 4)))
    # free extent 0: empty result
    a = torch.zeros(0, 5, dtype=torch.complex128, device="cuda")
    b = torch.ones(5, 4, dtype=torch.complex128, device="cuda")
    C = m.binary_einsum(m.Tensor(a, ["i", "j"]), m.Tensor(b, ["j", "k"]))
    assert tuple(C.data.shape) == (0, 4)
    # rank-0 x rank-0
    for form in ("plain", "ozaki"):
        with m.with_backend(m.BackendGB300(form)):
            C = m.binary_einsum(m.Tensor(torch.tensor(3.0, dtype=torch.float64, device="cuda")),
                                m.Tensor(torch.tensor(-2.5, dtype=torch.float64, device="cuda")))
        assert C.data.item() == -7.5
    # zero operand rows / columns (scale exponent of an all-zero row)
    rng = np.random.default_rng(3)
    x = rand(rng, [70, 40], np.float64)
    x[5, :] = 0.0
    y = rand(rng, [40, 90], np.float64)
    y[:, 7] = 0.0
    want = ref.contract(x, ["i", "j"], y, ["j", "k"], ["i", "k"])
    got, _ = run(x, ["i", "j"], y, ["j", "k"], ["i", "k"], "ozaki")
    assert ref.rel_fro(got, want) <= F64_TOL and np.all(got[5, :] == 0) and np.all(got[:, 7] == 0)


def test_errors_from_device_path():
    import muscle_gb300 as m

    a = m.Tensor(torch.ones(2, 3, device="cuda", dtype=torch.float64), ["i", "j"])
    b = m.Tensor(torch.ones(4, 5, device="cuda", dtype=torch.float64), ["j", "k"])
    with pytest.raises(m.DimensionMismatch):
        m.binary_einsum(a, b)
    with pytest.raises(m.ArgumentError):
        m.binary_einsum(a, a, out=["i", "q"])
    with pytest.raises(m.UnsupportedError):
        with m.with_backend(m.BackendGB300("ozaki")):
            m.binary_einsum(m.Tensor(torch.ones(2, 3, device="cuda"), ["i", "j"]),
                            m.Tensor(torch.ones(3, 2, device="cuda"), ["j", "k"]))


def test_ozaki_exact_on_integer_data():
    """Integer data whose products and sums are exact in float64: every digit
    product is exact in bf16 and every float32 TMEM partial sum must be an
    exact integer, so the emulated result must equal the exact one bit for bit.
    Entries near 2^20 make the leading digits large, pushing the chunk sums of
    the first digit group towards the 2^24 bound."""
    rng = np.random.default_rng(17)
    a = rng.integers(2**20 - 2**12, 2**20, size=(256, 4096)).astype(np.float64)
    b = rng.integers(2**20 - 2**12, 2**20, size=(4096, 192)).astype(np.float64)
    a[:, ::7] *= -1.0
    want = a @ b  # |sum| < 2^52: exact in float64 (each partial sum too)
    assert np.abs(want).max() < 2.0**52
    got, _ = run(np.asfortranarray(a), ["i", "j"], np.asfortranarray(b), ["j", "k"], ["i", "k"], "ozaki", 7)
    assert np.array_equal(got, want)
    a, b = a[:, :2048], b[:2048]  # complex sums stay below 2^52 too
    ac, bc = (a + 1j * a[::-1]).copy(order="F"), (b - 1j * b[:, ::-1]).copy(order="F")
    wantc = ac @ bc
    gotc, _ = run(ac, ["i", "j"], bc, ["j", "k"], ["i", "k"], "ozaki", 7)
    assert np.array_equal(gotc, wantc)


@pytest.mark.parametrize("slices", range(3, 9))
def test_ozaki_every_slice_count_exact_on_16_bit_integers(slices):
    """Integers below 2^16 need two 8-bit (or three 7-bit) digits after the
    row and column scaling, so every slice count from 3 up must reproduce the
    exact product bit for bit, real and complex, including ragged tiles."""
    rng = np.random.default_rng(40 + slices)
    a = rng.integers(-(2**16) + 1, 2**16, size=(200, 1100)).astype(np.float64)
    b = rng.integers(-(2**16) + 1, 2**16, size=(1100, 70)).astype(np.float64)
    want = a @ b  # |sum| < 2^43
    got, _ = run(np.asfortranarray(a), ["i", "j"], np.asfortranarray(b), ["j", "k"], ["i", "k"], "ozaki", slices)
    assert np.array_equal(got, want), slices
    ac = (a + 1j * a[::-1]).copy(order="F")
    bc = (b - 1j * b[:, ::-1]).copy(order="F")
    gotc, _ = run(ac, ["i", "j"], bc, ["j", "k"], ["i", "k"], "ozaki", slices)
    assert np.array_equal(gotc, ac @ bc), slices


def test_ozaki_slice_sweep_and_loguniform_spread():
    """Config-3 pattern (log-uniform magnitudes over 2^-20..2^20) at a reduced
    size: error falls with the slice count and S >= 7 meets 1e-13."""
    (a, ia), (b, ib), ic = wl.gen_config3(seed=0, n=512, k1=32, k2=16)
    want = ref.contract(a, ia, b, ib, ic)
    errs = {}
    for s in range(3, 9):
        got, _ = run(a, ia, b, ib, ic, "ozaki", s)
        errs[s] = ref.rel_fro(got, want)
    # 8-bit digits for S <= 6, 7-bit digits for S >= 7: monotone within each width
    assert all(errs[s + 1] < errs[s] for s in range(3, 6)), errs
    assert errs[8] < errs[7], errs
    assert errs[6] <= F64_TOL and errs[7] <= F64_TOL and errs[8] <= F64_TOL, errs
    got, _ = run(a, ia, b, ib, ic, "plain")
    assert ref.rel_fro(got, want) <= F64_TOL


def test_permute_bit_exact():
    import muscle_gb300 as m

    rng = np.random.default_rng(2)
    for dtype in (np.float32, np.float64, np.complex64, np.complex128):
        for shape, perm in (([33, 65, 7], [2, 0, 1]), ([64, 96, 64, 3], [1, 3, 0, 2]), ([130, 70], [1, 0]),
                            ([5, 6, 7], [0, 1, 2]), ([300, 2, 5], [0, 2, 1])):
            x = rand(rng, shape, dtype)
            labels = [f"m{d}" for d in range(len(shape))]
            X = m.Tensor(to_dev(x), labels)
            Y = m.permutedims(X, [labels[p] for p in perm])
            assert np.array_equal(to_np(Y.data), np.transpose(x, perm)), (dtype, shape, perm)
    # strided (non-contiguous) source
    big = torch.arange(0, 4000, dtype=torch.float64, device="cuda").reshape(40, 100)
    v = big[::2, 1::3]
    Y = m.permutedims(m.Tensor(v, ["a", "b"]), ["b", "a"])
    assert np.array_equal(to_np(Y.data), to_np(v).T)


def test_unary_random():
    import muscle_gb300 as m

    rng = np.random.default_rng(4)
    for dtype in (np.float64, np.complex128, np.float32):
        x = rand(rng, [6, 50, 6, 300], dtype)
        X = m.Tensor(to_dev(x), ["i", "j", "i", "k"])
        for out in (["j"], ["k", "i"], [], ["i", "j", "k"]):
            Y = m.unary_einsum(X, out=out)
            want = ref.unary(x, ["i", "j", "i", "k"], out)
            tol = 1e-13 if np.dtype(dtype) in (np.float64, np.complex128) else 1e-5
            assert ref.rel_fro(to_np(Y.data), want) <= tol, (dtype, out)


def test_ozaki_subnormal_results_correctly_rounded():
    """Exact-form results below the smallest normal float64 go through the
    epilogue's general conversion, normal ones through its straight-line
    path; both must be the correctly rounded value of the exact sum. Integer
    data scaled by powers of two make the exact sum known: C = (Ai Bi) 2^e
    with e = -1080 (subnormal) except column 0 (e = -480, normal)."""
    from fractions import Fraction

    rng = np.random.default_rng(21)
    ai = rng.integers(-100, 101, size=(8, 16))
    bi = rng.integers(-100, 101, size=(16, 8))
    a = np.asfortranarray(ai * 2.0**-540)
    bscale = np.full(8, 2.0**-540)
    bscale[0] = 2.0**60
    b = np.asfortranarray(bi * bscale[None, :])
    x = ai.astype(object).dot(bi.astype(object))  # exact integers
    want = np.empty((8, 8))
    for i in range(8):
        for j in range(8):
            e = -480 if j == 0 else -1080
            want[i, j] = float(Fraction(int(x[i, j])) * Fraction(2) ** e)
    assert np.any((want != 0) & (np.abs(want) < 2.0**-1022))  # subnormal results present
    for S in (6, 7):
        got, _ = run(a, ["i", "k"], b, ["k", "j"], ["i", "j"], "ozaki", S)
        assert np.array_equal(got.view(np.int64), want.view(np.int64)), S
