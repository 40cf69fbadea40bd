"""The oracle against the known answers of Muscle.jl's own tests (CPU only)."""
import numpy as np
import pytest

from oracle import muscle_ref as ref
from muscle_gb300 import workloads as wl
from tests.kat_util import expected_binary, make_array


def test_kat_binary_base_and_gpu_semantics(kat_cases):
    n = 0
    for case in kat_cases:
        if case["kind"] != "binary":
            continue
        a, b = make_array(case["a"]), make_array(case["b"])
        ia, ib = case["a"]["inds"], case["b"]["inds"]
        ic = ref.front_inds_c(ia, ib, case["dims"], case["out"])
        eb = case["expect_base"]
        if "raises" in eb:
            with pytest.raises(ref.ArgumentError):
                ref.backend_base(ic, a, ia, b, ib)
        else:
            c = ref.backend_base(ic, a, ia, b, ib)
            assert list(ic) == eb["inds"], case["name"]
            assert list(np.shape(c)) == eb["shape"], case["name"]
            want = expected_binary(case, eb, a, b)
            if "fill" in eb:
                assert np.array_equal(c, want), case["name"]
            else:
                assert np.allclose(c, want, rtol=1e-12), case["name"]
        eg = case["expect_gpu"]
        c = ref.contract(a, ia, b, ib, ic)
        assert list(ic) == eg["inds"], case["name"]
        assert list(np.shape(c)) == eg["shape"], case["name"]
        want = expected_binary(case, eg, a, b)
        if "fill" in eg:
            assert np.array_equal(c, want), case["name"]
        else:
            assert np.allclose(c, want, rtol=1e-12), case["name"]
        n += 1
    assert n >= 30


def test_kat_unary(kat_cases):
    for case in kat_cases:
        if case["kind"] != "unary":
            continue
        x = make_array(case["x"])
        ix = case["x"]["inds"]
        iy = case["inplace"] if case["inplace"] is not None else ref.front_inds_y(ix, case["dims"], case["out"])
        y = ref.unary(x, ix, iy)
        assert list(iy) == case["expect"]["inds"], case["name"]
        assert np.array_equal(y, np.full(case["expect"]["shape"], case["expect"]["fill"])), case["name"]


def test_kat_hadamard(kat_cases):
    from tests.kat_util import expected_hadamard

    hs = [c for c in kat_cases if c["kind"] == "hadamard"]
    assert len(hs) == 12
    for case in hs:
        a, b = make_array(case["a"]), make_array(case["b"])
        c, ic = ref.hadamard(a, case["a"]["inds"], b, case["b"]["inds"])
        exp = case["expect"]
        assert ic == exp["inds"] and list(c.shape) == exp["shape"], case["name"]
        assert np.array_equal(c, expected_hadamard(exp, b, case["b"]["inds"])), case["name"]
        # operand order does not matter: the operand of lower rank is broadcast
        c2, ic2 = ref.hadamard(b, case["b"]["inds"], a, case["a"]["inds"])
        assert ic2 == ic and np.array_equal(c2, c)


def test_hadamard_errors_and_types():
    a = np.ones((2, 3))
    with pytest.raises(ref.ArgumentError):
        ref.hadamard(a, ["i", "j"], np.ones(4), ["k"])
    c, _ = ref.hadamard(a.astype(np.float32), ["i", "j"], np.full(3, 0.5), ["j"])
    assert c.dtype == np.float32 and np.all(c == 0.5)
    with pytest.raises(ref.ArgumentError):
        ref.hadamard(a, ["i", "j"], np.full(3, 1j), ["j"])


def test_kat_permute(kat_cases):
    case = [c for c in kat_cases if c["kind"] == "permute"][0]
    x = make_array(case["x"])
    y = ref._permute(x, case["x"]["inds"], case["perm"])
    assert list(y.shape) == case["expect"]["shape"]
    assert np.array_equal(y, np.transpose(x, (2, 0, 1)))


def test_contract_matches_exact_rational():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((3, 4, 5)) + 1j * rng.standard_normal((3, 4, 5))
    b = rng.standard_normal((5, 2, 4)) + 1j * rng.standard_normal((5, 2, 4))
    c = ref.contract(a, ["i", "k", "l"], b, ["l", "j", "k"], ["j", "i"])
    pos = [(0, 0), (1, 2), (0, 1)]
    ex = ref.exact_entries(a, ["i", "k", "l"], b, ["l", "j", "k"], ["j", "i"], pos)
    for p, e in zip(pos, ex):
        assert abs(c[p] - e) <= 1e-14 * max(1.0, abs(e))


def test_exact_dot_matches_rational():
    """The fast exact entries (Veltkamp split + fsum) equal the rational
    ones bit for bit, also over a 2^-20..2^20 magnitude spread."""
    rng = np.random.default_rng(8)
    a = wl.loguniform_complex(rng, (6, 40, 7))
    b = wl.loguniform_complex(rng, (7, 5, 40))
    ia, ib, ic = ["i", "k1", "k2"], ["k2", "j", "k1"], ["j", "i"]
    pos = [(0, 0), (4, 5), (2, 3)]
    assert ref.exact_entries_fast(a, ia, b, ib, ic, pos) == ref.exact_entries(a, ia, b, ib, ic, pos)
    x = rng.standard_normal(300) * np.exp2(rng.uniform(-20, 20, 300))
    y = rng.standard_normal(300)
    assert ref.exact_dot(x, y) == ref.exact_entries(x, ["k"], y, ["k"], [], [()])[0]
    # batch labels stay fixed
    ab = rng.standard_normal((6, 7, 2))
    bb = rng.standard_normal((7, 6, 2))
    p2 = [(1, 2, 0), (5, 0, 1)]
    lab = (["i", "k", "b"], ["k", "j", "b"], ["i", "j", "b"])
    assert ref.exact_entries_fast(ab, lab[0], bb, lab[1], lab[2], p2) == ref.exact_entries(
        ab, lab[0], bb, lab[1], lab[2], p2)


def test_front_end_defaults():
    assert ref.front_inds_c(["i", "j"], ["j", "k"]) == ["i", "k"]
    assert ref.front_inds_c(["i", "j", "b"], ["j", "k", "b"], dims=["j"]) == ["i", "b", "k"]
    assert ref.front_inds_y(["i", "j", "i"]) == ["j"]
    assert ref.nonunique(["i", "j", "i", "j", "i"]) == ["i", "j"]


def test_generators_are_seeded():
    (a1, _), (b1, _), _ = wl.gen_config1(seed=0, dim=4)
    (a2, _), (b2, _), _ = wl.gen_config1(seed=0, dim=4)
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
    (a, ia), (b, ib), ic = wl.gen_config3(seed=0, n=64, k1=8, k2=4)
    mags = np.log2(np.abs(a))
    assert mags.min() >= -20 and mags.max() <= 20
    for s in range(20):
        (pa, pia), (pb, pib), pic, tries = wl.peps_instance(100 + s)
        n = pa.size + pb.size + int(np.prod([dict(zip(pia + pib, pa.shape + pb.shape))[i] for i in pic]))
        assert n <= wl.PEPS_CAP


def _su_case(op):
    """The reference's simple_update test set-up (test/unit/operations/simple_update.jl:5-30):
    an MPS of |00> + |01> + |10> + |11> (identity site tensors) and a two-site gate."""
    I2 = np.eye(2)
    g = np.array(op, dtype=float).reshape(2, 2, 2, 2, order="F")
    return I2, ["s1", "b"], I2, ["s2", "b"], g, ["s1", "s2", "g1", "g2"]


_OP_ID = np.eye(4)
_OP_CX = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]


def _su(op, **kw):
    a, ia, b, ib, g, ig = _su_case(op)
    return ref.simple_update(a, ia, "s1", b, ib, "s2", "b", g, ig, "g1", "g2", **kw)


def test_simple_update_restatement_matches_reference_asserts():
    """The known answers of test/unit/operations/simple_update.jl:32-172."""
    (U, lu), (s, ls), (V, lv) = _su(_OP_ID)  # apply identity
    assert lu == ["s1", "b"] and lv == ["s2", "b"] and ls == ["b"]
    assert np.allclose(U, np.eye(2)) and np.allclose(V, np.eye(2)) and np.array_equal(s, [1.0, 1.0])
    (U, _), (s, _), (V, _) = _su(_OP_CX)  # apply cx
    assert np.allclose(U, np.eye(2)) and np.allclose(V, np.array([[1, -1], [1, 1]]) / np.sqrt(2))
    assert np.allclose(s, [np.sqrt(2), 0.0])
    psi = ref.contract(U * s, ["s1", "b"], V, ["s2", "b"], ["s1", "s2"])
    assert np.isclose(np.vdot(psi, psi).real, 2.0)
    (U, _), (s, _), (V, _) = _su(_OP_ID, normalize=True)
    assert np.allclose(s, [1 / np.sqrt(2)] * 2)
    (U, _), (s, _), (V, _) = _su(_OP_CX, normalize=True)
    assert np.allclose(s, [1.0, 0.0])
    (U, _), (s, _), (V, _) = _su(_OP_ID, maxdim=1)
    assert U.shape == (2, 1) and np.allclose(U, np.eye(2)[:, :1]) and np.allclose(s, [1.0])
    (U, _), (s, _), (V, _) = _su(_OP_CX, maxdim=1)
    assert np.allclose(V, np.ones((2, 1)) / np.sqrt(2)) and np.allclose(s, [np.sqrt(2)])
    nrm = np.linalg.norm(ref.contract(np.eye(2), ["s1", "b"], np.eye(2), ["s2", "b"], ["s1", "s2"]))
    (U, _), (V, _) = _su(_OP_ID, absorb="u")
    assert np.isclose(np.linalg.norm(U), nrm)
    (U, _), (V, _) = _su(_OP_ID, absorb="v")
    assert np.isclose(np.linalg.norm(V), nrm)
    (U, _), (V, _) = _su(_OP_ID, absorb="equally")
    assert np.allclose(U, np.eye(2)) and np.allclose(V, np.eye(2))
