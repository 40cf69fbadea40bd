"""Adaptive slice count of the emulated FP64 form (slices = 0, the default of
the "auto" and "ozaki" forms): results within 1e-13 of the CPU oracle
whatever the spread of the data, the device's choice and estimate against
the host restatement (tests/ozaki_model.py), the plain fallback, and a CUDA
graph that chooses again on every replay."""
import numpy as np
import pytest
import torch

import muscle_gb300 as m
from muscle_gb300 import workloads as wl
from oracle import muscle_ref as ref
from tests import ozaki_model as oz
from tests.gpu_util import to_dev, to_np

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _contract(a, ia, b, ib, ic, form="auto", slices=0, tol=None):
    """One contraction through the C ABI; returns (result, report)."""
    A, B = to_dev(a), to_dev(b)
    I = lambda xs: [m.Index(x) for x in xs]
    ext = dict(zip(ia + ib, list(a.shape) + list(b.shape)))
    dt = torch.promote_types(A.dtype, B.dtype)
    C = m.empty_colmajor([ext[x] for x in ic], dt, "cuda")
    p = m.contraction_plan(A, I(ia), B, I(ib), C, I(ic), form, slices)
    if tol is not None:
        p.set_tolerance(tol)
    ws = torch.empty(max(p.workspace_bytes, 1), dtype=torch.uint8, device="cuda")
    _run(p, A, B, C, ws)
    rep = p.report(ws) if p.adaptive else None
    torch.cuda.synchronize()
    if tol is not None:
        p.set_tolerance(1e-13)  # plans are cached by descriptor: leave the default behind
    return to_np(C), rep


def _run(p, A, B, C, ws):
    from muscle_gb300 import _lib

    lib = _lib.load()
    _lib.check(lib.mgb_contract(p.handle, A.data_ptr(), B.data_ptr(), C.data_ptr(), ws.data_ptr(), ws.numel(),
                                torch.cuda.current_stream().cuda_stream), lib)


def _logu(rng, shape, lo, hi, cx=True):
    return np.asfortranarray(wl.loguniform_complex(rng, shape, np.complex128 if cx else np.float64, lo, hi))


def test_config1_at_its_stated_size():
    """A(i,j,k,l) x B(k,m,l,n), every extent 32, ComplexF64 N(0,1) from PCG64
    seed 0: the adaptive form against the oracle."""
    (a, ia), (b, ib), ic = wl.gen_config1(seed=0)
    want = ref.contract(a, ia, b, ib, ic)
    got, rep = _contract(a, ia, b, ib, ic)
    assert ref.rel_fro(got, want) <= TOL
    assert rep["slices"] in (5, 6), rep
    got_plain, _ = _contract(a, ia, b, ib, ic, "plain")
    assert ref.rel_fro(got_plain, want) <= TOL


@pytest.mark.parametrize("spread", [20, 40, 60])
@pytest.mark.parametrize("cx", [True, False])
def test_wide_exponent_spread_meets_tolerance(spread, cx):
    """Log-uniform magnitudes over 2^-spread..2^spread (the precision
    workload's distribution, widened): "auto" stays within 1e-13."""
    rng = np.random.default_rng(spread + (100 if cx else 0))
    a, b = _logu(rng, (300, 24, 40), -spread, spread, cx), _logu(rng, (40, 260, 24), -spread, spread, cx)
    ia, ib, ic = ["i", "k1", "k2"], ["k2", "j", "k1"], ["i", "j"]
    want = ref.contract(a, ia, b, ib, ic)
    got, rep = _contract(a, ia, b, ib, ic)
    err = ref.rel_fro(got, want)
    assert err <= TOL, (err, rep)
    assert rep["slices"] >= 6 and rep["estimate"][rep["slices"]] <= TOL, rep


def test_choice_follows_the_data():
    """A dominant column of A needs more slices than the same Gaussian data
    without it; inversely scaled columns of A and rows of B defeat per-row
    scaling, so the plain form runs; every result meets 1e-13."""
    rng = np.random.default_rng(8)
    a = np.asfortranarray(rng.standard_normal((200, 700)))
    b = np.asfortranarray(rng.standard_normal((700, 150)))
    _, plain_rep = _contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"])
    a[:, 3] *= 1e6
    want = ref.contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"])
    got, rep = _contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"])
    assert rep["slices"] == oz.choose(a, b) and rep["slices"] > plain_rep["slices"], (rep, plain_rep)
    assert ref.rel_fro(got, want) <= TOL, rep
    s = np.exp2(rng.uniform(-20, 20, 700))
    a2 = np.asfortranarray(rng.standard_normal((200, 700)) * s[None, :])
    b2 = np.asfortranarray(rng.standard_normal((700, 150)) / s[:, None])
    want = ref.contract(a2, ["i", "k"], b2, ["k", "j"], ["i", "j"])
    got, rep = _contract(a2, ["i", "k"], b2, ["k", "j"], ["i", "j"])
    assert rep["slices"] == 0 and ref.rel_fro(got, want) <= TOL, rep


@pytest.mark.parametrize("case", ["normal", "loguniform", "dominant", "complex"])
def test_device_estimate_matches_host_restatement(case):
    rng = np.random.default_rng(77)
    if case == "loguniform":
        a, b = _logu(rng, (96, 512), -20, 20, False), _logu(rng, (512, 80), -20, 20, False)
    elif case == "complex":
        a, b = _logu(rng, (96, 512), -30, 30), _logu(rng, (512, 80), -30, 30)
    else:
        a = np.asfortranarray(rng.standard_normal((96, 512)))
        b = np.asfortranarray(rng.standard_normal((512, 80)))
        if case == "dominant":
            b[7, :] *= 1e5
    _, rep = _contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"])
    for S, est in rep["estimate"].items():
        want = oz.estimate(a, b, S)
        assert abs(est - want) <= 1e-3 * want, (S, est, want)
    assert rep["slices"] == oz.choose(a, b), rep


def test_tolerance_setting():
    """A looser target picks fewer slices and still meets it."""
    rng = np.random.default_rng(5)
    a = np.asfortranarray(rng.standard_normal((128, 256)) + 1j * rng.standard_normal((128, 256)))
    b = np.asfortranarray(rng.standard_normal((256, 64)) + 1j * rng.standard_normal((256, 64)))
    want = ref.contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"])
    got, rep = _contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"], "ozaki", 0, tol=1e-8)
    assert rep["tolerance"] == 1e-8 and rep["slices"] in (3, 4), rep
    assert ref.rel_fro(got, want) <= 1e-8
    with pytest.raises(m.ArgumentError):
        p = m.contraction_plan(to_dev(a), [m.Index("i"), m.Index("k")], to_dev(b), [m.Index("k"), m.Index("j")],
                               m.empty_colmajor([128, 64], torch.complex128, "cuda"),
                               [m.Index("i"), m.Index("j")], "ozaki", 7)
        p.set_tolerance(1e-8)  # fixed slice count: no tolerance to set


def test_nonfinite_and_zero_operands():
    rng = np.random.default_rng(6)
    a = np.asfortranarray(rng.standard_normal((64, 100)))
    b = np.asfortranarray(rng.standard_normal((100, 48)))
    a[3, 5] = np.inf
    b[9, 2] = np.nan
    got, rep = _contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"])
    assert rep["slices"] == 0 and rep["nonfinite"], rep
    plain, _ = _contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"], "plain")
    assert np.array_equal(np.isnan(got), np.isnan(plain)) and np.array_equal(got[~np.isnan(got)], plain[~np.isnan(plain)])
    z = np.zeros((64, 100), order="F")
    b[9, 2] = 1.0  # finite again: the zero operand alone decides
    got, rep = _contract(z, ["i", "k"], b, ["k", "j"], ["i", "j"])
    assert np.all(got == 0) and rep["slices"] == 5 and rep["estimate"][5] == 0.0, rep


def test_graph_replay_chooses_again():
    """The choice is made on the device: a CUDA graph captured once picks more
    slices when a dominant column is copied into the same buffers than for
    the Gaussian data before and after, and each result meets 1e-13."""
    rng = np.random.default_rng(9)
    a1 = np.asfortranarray(rng.standard_normal((256, 600)))
    b1 = np.asfortranarray(rng.standard_normal((600, 192)))
    a2 = a1.copy(order="F")
    a2[:, 11] *= 1e6
    A, B = to_dev(a1), to_dev(b1)
    C = m.empty_colmajor([256, 192], torch.float64, "cuda")
    I = lambda xs: [m.Index(x) for x in xs]
    p = m.contraction_plan(A, I("ik"), B, I("kj"), C, I("ij"), "auto", 0)
    ws = torch.empty(p.workspace_bytes, dtype=torch.uint8, device="cuda")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        _run(p, A, B, C, ws)  # warm-up outside the capture
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        _run(p, A, B, C, ws)
    seen = []
    for a in (a1, a2, a1):
        A.copy_(to_dev(a))
        g.replay()
        torch.cuda.synchronize()
        rep = p.report(ws)
        assert rep["slices"] == oz.choose(a, b1), rep
        seen.append(rep["slices"])
        assert ref.rel_fro(to_np(C), ref.contract(a, ["i", "k"], b1, ["k", "j"], ["i", "j"])) <= TOL
    assert seen[1] > seen[0] == seen[2], seen
