"""Serving form: mixed-size contractions submitted as they arrive, admitted
against an HBM byte budget and batched onto several streams. Each result is
the same alone and in the mix (bit for bit: the same kernels run on the same
data), and matches the CPU oracle at 1e-13 (Float64/ComplexF64) or 1e-5
(ComplexF32)."""
import threading

import numpy as np
import pytest
import torch

from muscle_gb300 import workloads as wl
from oracle import muscle_ref as ref

pytestmark = pytest.mark.gpu


def make_requests(n, seed, flops_hi=1e8):
    import muscle_gb300 as m

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        req = wl.serve_request(rng, 1e4, flops_hi)
        a, b = wl.serve_arrays(rng, req)
        sa, ia, sb, ib, ic, dtype, _ = req
        out.append((m.Tensor(torch.from_numpy(a).cuda(), ia), m.Tensor(torch.from_numpy(b).cuda(), ib), ic, a, b))
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("form", ["auto", "plain"])
def test_served_results_equal_alone_and_oracle(form):
    import muscle_gb300 as m

    reqs = make_requests(120, 7)
    with m.Server(budget_bytes=2 << 30, streams=4, max_batch=16, form=form) as srv:
        pending = [srv.submit(A, B, out=ic) for A, B, ic, _, _ in reqs]
        outs = [p.result(timeout=120) for p in pending]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["rejected"] == 0 and st["batches"] >= 2
    for (A, B, ic, a, b), C in zip(reqs, outs):
        with m.with_backend(m.BackendGB300(form)):
            alone = m.binary_einsum(A, B, out=ic)
        got = C.data.cpu().numpy()
        assert np.array_equal(alone.data.cpu().numpy(), got)
        tol = 1e-5 if got.dtype == np.complex64 else 1e-13
        assert ref.rel_fro(got, ref.contract(a, [i.tag for i in A.inds], b, [i.tag for i in B.inds], ic)) <= tol


def test_budget_admission_and_rejection():
    import muscle_gb300 as m

    reqs = make_requests(40, 11, flops_hi=1e7)
    sizes = [A.data.nbytes + B.data.nbytes for A, B, *_ in reqs]
    budget = max(sizes) * 4 + (64 << 20)
    with m.Server(budget_bytes=budget, streams=3, max_batch=4, form="auto") as srv:
        pending = [srv.submit(A, B, out=ic) for A, B, ic, _, _ in reqs]
        peak = 0
        for p in pending:
            p.wait(timeout=120)
            peak = max(peak, srv.stats()["used_bytes"])
        assert peak <= budget
        assert all(p.wait() == 0 for p in pending)
        # a request larger than the whole budget is rejected with OutOfBudget
        big = m.Tensor(torch.zeros(4096, 4096, dtype=torch.complex128, device="cuda"), ["i", "j"])
        bigb = m.Tensor(torch.zeros(4096, 64, dtype=torch.complex128, device="cuda"), ["j", "k"])
        with pytest.raises(m.OutOfBudget):
            srv.submit(big, bigb).result(timeout=60)


def test_concurrent_clients():
    import muscle_gb300 as m

    reqs = make_requests(64, 13, flops_hi=1e7)
    results = [None] * len(reqs)
    with m.Server(budget_bytes=1 << 30, streams=4, max_batch=8) as srv:
        def client(lo):
            for i in range(lo, len(reqs), 4):
                A, B, ic, _, _ = reqs[i]
                results[i] = srv.submit(A, B, out=ic).result(timeout=120)

        threads = [threading.Thread(target=client, args=(k,)) for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    for (A, B, ic, a, b), C in zip(reqs, results):
        tol = 1e-5 if C.dtype == torch.complex64 else 1e-13
        assert ref.rel_fro(C.data.cpu().numpy(), ref.contract(a, [i.tag for i in A.inds], b, [i.tag for i in B.inds], ic)) <= tol


def test_one_batch_with_every_kind_of_request():
    """One batch of Gaussian ComplexF64 requests, Float64 requests with a
    dominant column (more slices), Float64 requests whose inversely scaled
    columns and rows defeat row scaling (the device chooses the plain form and
    the server runs them again), and ComplexF32 requests (BF16x3): every
    result equals the same contraction run alone and meets the oracle."""
    import muscle_gb300 as m

    rng = np.random.default_rng(21)
    arrays = []
    for kind in ["gauss"] * 6 + ["dominant"] * 2 + ["kscaled"] * 2 + ["c32"] * 3:
        M, K, N = (int(x) for x in rng.integers(40, 300, size=3))
        if kind in ("gauss", "c32"):
            dt = np.complex128 if kind == "gauss" else np.complex64
            a = (rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))).astype(dt)
            b = (rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))).astype(dt)
        else:
            a, b = rng.standard_normal((M, K)), rng.standard_normal((K, N))
            if kind == "dominant":
                a[:, 1] *= 1e6
            else:
                s = np.exp2(rng.uniform(-20, 20, K))
                a, b = a * s[None, :], b / s[:, None]
        arrays.append((np.asfortranarray(a), np.asfortranarray(b), kind))
    tens = [(m.Tensor(torch.from_numpy(a).cuda(), ["i", "k"]), m.Tensor(torch.from_numpy(b).cuda(), ["k", "j"]))
            for a, b, _ in arrays]
    torch.cuda.synchronize()
    with m.Server(budget_bytes=4 << 30, streams=2, max_batch=64, form="auto") as srv:
        pending = [srv.submit(A, B, out=["i", "j"]) for A, B in tens]
        outs = [p.result(timeout=120) for p in pending]
        st = srv.stats()
    assert st["completed"] == len(arrays) and st["rejected"] == 0
    for (a, b, kind), (A, B), C in zip(arrays, tens, outs):
        got = C.data.cpu().numpy()
        alone = m.binary_einsum(A, B, out=["i", "j"]).data.cpu().numpy()
        assert np.array_equal(got, alone), kind
        tol = 1e-5 if kind == "c32" else 1e-13
        assert ref.rel_fro(got, ref.contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"])) <= tol, kind
