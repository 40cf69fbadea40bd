"""Emulated plans that compute C^T = B^T A^T (A with few rows, B with many
columns): results against the CPU oracle at the stated tolerances through a
single call, a group and the server, with strided views, permuted output
labels, batch labels and mixed real x complex operands; the exact form gives
the same bits as the plain-orientation arithmetic would (exact sums), which
the integer-data case checks bit for bit."""
import numpy as np
import pytest
import torch

from oracle import muscle_ref as ref
from tests.gpu_util import to_dev

pytestmark = pytest.mark.gpu


def rand(rng, shape, dtype):
    x = rng.standard_normal(shape)
    if np.issubdtype(dtype, np.complexfloating):
        x = x + 1j * rng.standard_normal(shape)
    return np.array(x.astype(dtype), order="F")


# (A labels, A extents, A dtype, B labels, B extents, B dtype, C labels)
CASES = [
    (["i", "k"], [8, 40], np.float64, ["k", "j"], [40, 500], np.float64, ["i", "j"]),
    (["k", "i"], [33, 5], np.complex128, ["j", "k"], [700, 33], np.complex128, ["j", "i"]),
    (["i", "k", "b"], [8, 30, 3], np.float64, ["k", "j", "b"], [30, 300, 3], np.complex128, ["i", "j", "b"]),
    (["p", "i", "k"], [2, 6, 17], np.complex128, ["k", "q", "j"], [17, 3, 200], np.complex128, ["q", "i", "j", "p"]),
    (["i", "k"], [20, 64], np.complex64, ["k", "j"], [64, 900], np.complex64, ["i", "j"]),
]


def _plan_swapped(A, B, C, form):
    import muscle_gb300 as m

    p = m.contraction_plan(A.data, A.inds, B.data, B.inds, C.data, C.inds, form, 0)
    return p.operands_swapped


@pytest.mark.parametrize("case", range(len(CASES)))
def test_swapped_single_calls(case):
    import muscle_gb300 as m

    ia, ea, ta, ib, eb, tb, ic = CASES[case]
    rng = np.random.default_rng(100 + case)
    a, b = rand(rng, ea, ta), rand(rng, eb, tb)
    want = ref.contract(a, ia, b, ib, ic)
    single = np.result_type(ta, tb) == np.complex64
    forms = ["bf16x3", "auto"] if single else ["ozaki", "auto"]
    tol = 1e-5 if single else 1e-13
    # a strided view of A: every other element of a larger buffer
    big = np.zeros([2 * ea[0]] + ea[1:], dtype=ta, order="F")
    big[::2] = a
    Abig = torch.from_numpy(big).cuda()
    for form in forms:
        for A in (m.Tensor(to_dev(a), ia), m.Tensor(Abig[::2], ia)):
            B = m.Tensor(to_dev(b), ib)
            with m.with_backend(m.BackendGB300(form)):
                C = m.binary_einsum(A, B, out=ic)
            torch.cuda.synchronize()
            assert [i.tag for i in C.inds] == ic
            assert _plan_swapped(A, B, C, form), (case, form)
            assert ref.rel_fro(C.data.cpu().numpy(), want) <= tol, (case, form)
    assert m.device_status() == 0


def test_swapped_exact_form_is_bit_exact_on_integers():
    """Integer operands: every digit product is exact, so the exact form must
    reproduce the integer result bit for bit in either orientation."""
    import muscle_gb300 as m

    rng = np.random.default_rng(9)
    a = np.asfortranarray(rng.integers(-1000, 1001, size=(6, 50)).astype(np.float64))
    b = np.asfortranarray(rng.integers(-1000, 1001, size=(50, 400)).astype(np.float64))
    want = a @ b  # exact: |entries| < 2^53
    A, B = m.Tensor(to_dev(a), ["i", "k"]), m.Tensor(to_dev(b), ["k", "j"])
    for slices in (5, 7):
        with m.with_backend(m.BackendGB300("ozaki", slices)):
            C = m.binary_einsum(A, B, out=["i", "j"])
        torch.cuda.synchronize()
        assert np.array_equal(C.data.cpu().numpy(), want), slices


def test_swapped_plans_in_group_and_server():
    import muscle_gb300 as m

    rng = np.random.default_rng(31)
    items, wants = [], []
    for t in range(12):
        m_, n_, k_ = 4 + t, 300 + 17 * t, 24 + t
        a = rand(rng, [m_, k_], np.complex128)
        b = rand(rng, [k_, n_], np.complex128)
        wants.append(ref.contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"]))
        A, B = m.Tensor(to_dev(a), ["i", "k"]), m.Tensor(to_dev(b), ["k", "j"])
        C = m.Tensor(m.zeros_colmajor([m_, n_], torch.complex128, "cuda"), ["i", "j"])
        items.append((C, A, B))
    assert all(_plan_swapped(A, B, C, "ozaki") for C, A, B in items)
    g = m.Group(items, "ozaki")
    g.execute()
    torch.cuda.synchronize()
    for (C, _, _), want in zip(items, wants):
        assert ref.rel_fro(C.data.cpu().numpy(), want) <= 1e-13
    with m.Server(budget_bytes=1 << 30, streams=2, max_batch=8, form="auto") as srv:
        pending = [srv.submit(A, B, out=["i", "j"]) for _, A, B in items]
        outs = [p.result(timeout=120) for p in pending]
    for C, want in zip(outs, wants):
        assert ref.rel_fro(C.data.cpu().numpy(), want) <= 1e-13
    assert m.device_status() == 0
