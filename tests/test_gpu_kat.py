"""Known answers of Muscle.jl's tests through the product API on the GPU, in
every arithmetic form (exact where the reference asserts `==`)."""
import numpy as np
import pytest
import torch

from tests.gpu_util import forms_for, to_dev, to_np
from tests.kat_util import expected_binary, make_array

pytestmark = pytest.mark.gpu


def test_kat_binary_all_forms(kat_cases):
    import muscle_gb300 as m

    checked = 0
    for case in kat_cases:
        if case["kind"] != "binary":
            continue
        a, b = make_array(case["a"]), make_array(case["b"])
        rdt = np.result_type(a, b)
        exp = case["expect_gpu"]
        want = expected_binary(case, exp, a, b)
        for form, slices in forms_for(rdt):
            A = m.Tensor(to_dev(a), case["a"]["inds"])
            B = m.Tensor(to_dev(b), case["b"]["inds"])
            with m.with_backend(m.BackendGB300(form, slices)):
                C = m.binary_einsum(A, B, dims=case["dims"], out=case["out"])
            got = to_np(C.data)
            tag = f"{case['name']} [{form}]"
            assert [i.tag for i in C.inds] == exp["inds"], tag
            assert list(got.shape) == exp["shape"], tag
            assert got.dtype == rdt, tag
            if "fill" in exp:
                assert np.array_equal(got, want.astype(rdt)), tag
            else:
                assert np.allclose(got, want, rtol=1e-12, atol=0), tag
            checked += 1
    assert checked >= 90
    assert m.device_status() == 0


def test_kat_binary_inplace(kat_cases):
    """binary_einsum! into a preallocated C (src/Operations/binary_einsum.jl:57-70)."""
    import muscle_gb300 as m

    case = [c for c in kat_cases if c["name"] == "matmul out permuted"][0]
    a, b = make_array(case["a"]), make_array(case["b"])
    for form in ("plain", "ozaki", "auto"):
        C = m.Tensor(m.zeros_colmajor([4, 2], torch.float64, "cuda"), ["k", "i"])
        with m.with_backend(m.BackendGB300(form)):
            m.binary_einsum_(C, m.Tensor(to_dev(a), ["i", "j"]), m.Tensor(to_dev(b), ["j", "k"]))
        assert np.array_equal(to_np(C.data), np.full((4, 2), 3.0))


def test_kat_unary(kat_cases):
    import muscle_gb300 as m

    for case in kat_cases:
        if case["kind"] != "unary":
            continue
        x = make_array(case["x"])
        X = m.Tensor(to_dev(x), case["x"]["inds"])
        exp = case["expect"]
        if case["inplace"] is not None:
            Y = m.Tensor(m.zeros_colmajor(exp["shape"], torch.float64, "cuda"), case["inplace"])
            m.unary_einsum_(Y, X)
        else:
            Y = m.unary_einsum(X, dims=case["dims"], out=case["out"])
        assert [i.tag for i in Y.inds] == exp["inds"], case["name"]
        assert np.array_equal(to_np(Y.data), np.full(exp["shape"], exp["fill"])), case["name"]


def test_kat_permute(kat_cases):
    import muscle_gb300 as m

    case = [c for c in kat_cases if c["kind"] == "permute"][0]
    x = make_array(case["x"])
    X = m.Tensor(to_dev(x), case["x"]["inds"])
    for perm in (case["perm"], [2, 0, 1]):
        Y = m.permutedims(X, perm)
        assert [i.tag for i in Y.inds] == case["expect"]["inds"]
        assert np.array_equal(to_np(Y.data), np.transpose(x, (2, 0, 1)))
