"""Thin SVD on the device (mgb_svd, one-sided Jacobi) and simple_update
(src/Operations/simple_update.jl:35-82) against the CPU oracle: singular
values, reconstruction, orthonormality (singular vectors are unique only up
to phases, so the tests compare what is invariant), the reference's own
known answers, truncation, normalisation and every absorb behaviour."""
import ctypes

import numpy as np
import pytest
import torch

import muscle_gb300 as m
from oracle import muscle_ref as ref
from tests.gpu_util import to_dev, to_np

pytestmark = pytest.mark.gpu


def _svd(a, keep=0, flags=0):
    from muscle_gb300 import _lib

    lib = _lib.load()
    mm, nn = a.shape
    dt = _lib.C64 if np.iscomplexobj(a) else _lib.F64
    k = min(mm, nn)
    kk = k if keep <= 0 else min(keep, k)
    A = to_dev(np.asfortranarray(a))
    tdt = torch.complex128 if np.iscomplexobj(a) else torch.float64
    U = m.empty_colmajor([mm, kk], tdt, "cuda")
    V = m.empty_colmajor([nn, kk], tdt, "cuda")
    S = torch.empty(kk, dtype=torch.float64, device="cuda")
    wsb = ctypes.c_uint64(0)
    _lib.check(lib.mgb_svd_workspace_size(dt, mm, nn, ctypes.byref(wsb)), lib)
    ws = torch.empty(wsb.value, dtype=torch.uint8, device="cuda")
    _lib.check(lib.mgb_svd(dt, mm, nn, A.data_ptr(), mm, U.data_ptr(), S.data_ptr(), V.data_ptr(), keep, flags,
                           ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream), lib)
    torch.cuda.synchronize()
    return to_np(U), to_np(S), to_np(V)


def _rand(rng, shape, cx):
    x = rng.standard_normal(shape)
    return x + 1j * rng.standard_normal(shape) if cx else x


@pytest.mark.parametrize("shape", [(64, 64), (200, 37), (37, 200), (1, 9), (300, 300), (128, 1)])
@pytest.mark.parametrize("cx", [False, True])
def test_svd_against_lapack(shape, cx):
    rng = np.random.default_rng(shape[0] * 1000 + shape[1] + cx)
    a = _rand(rng, shape, cx)
    U, s, V = _svd(a)
    want = np.linalg.svd(a, compute_uv=False)
    assert np.allclose(s, want, rtol=1e-13, atol=1e-13 * want[0])
    k = min(shape)
    assert np.linalg.norm(U @ np.diag(s) @ V.conj().T - a) <= 1e-13 * np.linalg.norm(a)
    assert np.linalg.norm(U.conj().T @ U - np.eye(k)) <= 1e-13 * k
    assert np.linalg.norm(V.conj().T @ V - np.eye(k)) <= 1e-13 * k


def test_svd_rank_deficient_and_flags():
    rng = np.random.default_rng(3)
    x, y = _rand(rng, (90, 3), True), _rand(rng, (3, 50), True)
    a = x @ y  # rank 3
    U, s, V = _svd(a)
    assert np.all(s[3:] <= 1e-13 * s[0]) and np.allclose(s[:3], np.linalg.svd(a, compute_uv=False)[:3], rtol=1e-13)
    assert np.linalg.norm(U.conj().T @ U - np.eye(50)) <= 1e-12  # completed to an orthonormal set
    assert np.linalg.norm(U @ np.diag(s) @ V.conj().T - a) <= 1e-13 * np.linalg.norm(a)
    z = np.zeros((6, 4))  # the zero matrix: orthonormal factors, zero values
    U, s, V = _svd(z)
    assert np.all(s == 0) and np.allclose(U.T @ U, np.eye(4)) and np.allclose(V.T @ V, np.eye(4))
    from muscle_gb300 import _lib

    b = _rand(rng, (40, 30), True)
    U, s, V = _svd(b, keep=7, flags=_lib.SVD_NORMALIZE | _lib.SVD_CONJ_V)
    want = np.linalg.svd(b, compute_uv=False)[:7]
    assert U.shape == (40, 7) and np.allclose(s, want / np.linalg.norm(want), rtol=1e-13)
    Uf, sf, Vf = _svd(b)
    assert np.allclose(np.abs(V), np.abs(Vf[:, :7])) and np.allclose(V, Vf[:, :7].conj())
    _, ss, _ = _svd(b, keep=7, flags=_lib.SVD_NORMALIZE | _lib.SVD_SQRT_S)
    assert np.allclose(ss, np.sqrt(want / np.linalg.norm(want)), rtol=1e-13)


_OP_ID = np.eye(4)
_OP_CX = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]


def _ref_case(op):
    I2 = np.eye(2)
    g = np.array(op, dtype=float).reshape(2, 2, 2, 2, order="F")
    return (m.Tensor(to_dev(I2), ["s1", "b"]), m.Tensor(to_dev(I2), ["s2", "b"]),
            m.Tensor(to_dev(np.asfortranarray(g)), ["s1", "s2", "g1", "g2"]))


def _su_dev(A, B, G, **kw):
    return m.simple_update(A, "s1", B, "s2", "b", G, "g1", "g2", **kw)


def _psi_norm2(U, s, V):
    us = m.hadamard(U, s)
    psi = m.binary_einsum(us, V)
    return float(np.vdot(to_np(psi.data), to_np(psi.data)).real)


def test_simple_update_reference_known_answers():
    """test/unit/operations/simple_update.jl:32-172 on the device."""
    A, B, G = _ref_case(_OP_ID)
    U, s, V = _su_dev(A, B, G)
    assert [i.tag for i in U.inds] == ["s1", "b"] and [i.tag for i in V.inds] == ["s2", "b"]
    assert np.array_equal(to_np(s.data), [1.0, 1.0])
    assert np.allclose(np.abs(to_np(U.data)), np.eye(2)) and np.allclose(np.abs(to_np(V.data)), np.eye(2))
    assert np.isclose(_psi_norm2(U, s, V), 2.0)
    A, B, G = _ref_case(_OP_CX)
    U, s, V = _su_dev(A, B, G)
    assert np.allclose(to_np(s.data), [np.sqrt(2), 0.0], atol=1e-15)
    assert np.allclose(np.abs(to_np(U.data)), np.eye(2))
    assert np.allclose(np.abs(to_np(V.data)[:, 0]), [1 / np.sqrt(2)] * 2)
    assert np.isclose(_psi_norm2(U, s, V), 2.0)
    U, s, V = _su_dev(A, B, G, normalize=True)
    assert np.allclose(to_np(s.data), [1.0, 0.0], atol=1e-15) and np.isclose(_psi_norm2(U, s, V), 1.0)
    U, s, V = _su_dev(A, B, G, maxdim=1)
    assert U.data.shape == (2, 1) and np.allclose(to_np(s.data), [np.sqrt(2)])
    assert np.allclose(np.abs(to_np(V.data)), np.ones((2, 1)) / np.sqrt(2))
    A, B, G = _ref_case(_OP_ID)
    nrm = np.sqrt(2.0)
    U, V = _su_dev(A, B, G, absorb="u")
    assert np.isclose(np.linalg.norm(to_np(U.data)), nrm)
    U, V = _su_dev(A, B, G, absorb="v")
    assert np.isclose(np.linalg.norm(to_np(V.data)), nrm)
    U, V = _su_dev(A, B, G, absorb="equally")
    assert np.allclose(np.abs(to_np(U.data)), np.eye(2)) and np.allclose(np.abs(to_np(V.data)), np.eye(2))


@pytest.mark.parametrize("cx", [False, True])
@pytest.mark.parametrize("chi", [8, 32])
def test_simple_update_random_mps_pair(cx, chi):
    """A(p1, l, b) and B(p2, b, r) of an MPS with bond chi, a random two-site
    gate: the device result against the oracle (singular values, the
    reconstructed two-site tensor, orthonormal factors), with truncation to
    chi and every absorb."""
    rng = np.random.default_rng(100 * chi + cx)
    a = np.asfortranarray(_rand(rng, (2, chi, chi), cx))
    b = np.asfortranarray(_rand(rng, (2, chi, chi), cx))
    g = np.asfortranarray(_rand(rng, (2, 2, 2, 2), cx))
    ia, ib, ig = ["p1", "l", "b"], ["p2", "b", "r"], ["p1", "p2", "q1", "q2"]
    A, B, G = m.Tensor(to_dev(a), ia), m.Tensor(to_dev(b), ib), m.Tensor(to_dev(g), ig)
    (Uo, lu), (so, _), (Vo, lv) = ref.simple_update(a, ia, "p1", b, ib, "p2", "b", g, ig, "q1", "q2", maxdim=chi)
    U, s, V = m.simple_update(A, "p1", B, "p2", "b", G, "q1", "q2", maxdim=chi)
    assert [i.tag for i in U.inds] == lu and [i.tag for i in V.inds] == lv
    got_s = to_np(s.data)
    assert np.allclose(got_s, so, rtol=1e-13, atol=1e-13 * so[0])
    rec = lambda u, ss, v: ref.contract(u * ss, lu, v, lv, ["p1", "l", "p2", "r"])
    want = rec(Uo, so, Vo)
    assert ref.rel_fro(rec(to_np(U.data), got_s, to_np(V.data)), want) <= 1e-13
    um = to_np(U.data).reshape(-1, chi, order="F")
    assert np.linalg.norm(um.conj().T @ um - np.eye(chi)) <= 1e-12
    for absorb in ("u", "v", "equally"):
        (Uo2, _), (Vo2, _) = ref.simple_update(a, ia, "p1", b, ib, "p2", "b", g, ig, "q1", "q2", maxdim=chi,
                                               absorb=absorb)
        U2, V2 = m.simple_update(A, "p1", B, "p2", "b", G, "q1", "q2", maxdim=chi, absorb=absorb)
        got = ref.contract(to_np(U2.data), lu, to_np(V2.data), lv, ["p1", "l", "p2", "r"])
        assert ref.rel_fro(got, ref.contract(Uo2, lu, Vo2, lv, ["p1", "l", "p2", "r"])) <= 1e-13, absorb
