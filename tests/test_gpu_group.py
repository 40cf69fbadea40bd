"""Batching form: groups of PEPS-style contractions (rank-5 sites with
physical dimension 2 and bond dimension chi, contracted with a neighbour over
1-3 shared bonds) executed as batched launches and as a captured CUDA graph,
against the CPU oracle; each member's result in the group equals its result
computed alone."""
import numpy as np
import pytest
import torch

from oracle import muscle_ref as ref
from muscle_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

SMALL_CAP = 1 << 17  # elements of A + B + C per instance in these tests


def instances(n, seed, dtype):
    out = []
    for i in range(n):
        (a, ia), (b, ib), ic, _ = wl.peps_instance(seed + i, dtype=dtype, cap=SMALL_CAP)
        out.append((a, ia, b, ib, ic))
    return out


def make_items(insts):
    import muscle_gb300 as m

    items = []
    for a, ia, b, ib, ic in insts:
        A = m.Tensor(torch.from_numpy(a).cuda(), ia)
        B = m.Tensor(torch.from_numpy(b).cuda(), ib)
        size = dict(zip(ia + ib, a.shape + b.shape))
        dt = torch.promote_types(A.dtype, B.dtype)
        C = m.Tensor(m.zeros_colmajor([size[i] for i in ic], dt, "cuda"), ic)
        items.append((C, A, B))
    return items


@pytest.mark.parametrize("dtype,forms", [(np.complex128, ["ozaki", "plain"]), (np.complex64, ["bf16x3", "plain"])])
def test_group_matches_oracle_and_single(dtype, forms):
    import muscle_gb300 as m

    insts = instances(48, 500, dtype)
    tol = 1e-13 if dtype == np.complex128 else 1e-5
    wants = [ref.contract(a, ia, b, ib, ic) for a, ia, b, ib, ic in insts]
    for form in forms:
        items = make_items(insts)
        g = m.Group(items, form)
        g.execute()
        torch.cuda.synchronize()
        for (C, A, B), want in zip(items, wants):
            got = C.data.cpu().numpy()
            assert ref.rel_fro(got, want) <= tol, form
            with m.with_backend(m.BackendGB300(form)):
                alone = m.binary_einsum(A, B, out=C.inds)
            if form != "plain" or dtype == np.complex128:
                assert np.array_equal(alone.data.cpu().numpy(), got), form  # same kernels, same arithmetic
    assert m.device_status() == 0


def test_group_graph_capture_and_update():
    import muscle_gb300 as m

    insts = instances(40, 900, np.complex128)
    items = make_items(insts)
    g = m.Group(items, "ozaki")
    graph = g.capture()
    for C, _, _ in items:
        C.data.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for (C, _, _), (a, ia, b, ib, ic) in zip(items, insts):
        assert ref.rel_fro(C.data.cpu().numpy(), ref.contract(a, ia, b, ib, ic)) <= 1e-13
    # new data in the same device buffers: replay sees it
    rng = np.random.default_rng(3)
    new = []
    for (C, A, B), (a, ia, b, ib, ic) in zip(items, insts):
        a2 = np.array(rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape), order="F")
        A.data.copy_(torch.from_numpy(a2))
        new.append((a2, ia, b, ib, ic))
    graph.replay()
    torch.cuda.synchronize()
    for (C, _, _), (a, ia, b, ib, ic) in zip(items, new):
        assert ref.rel_fro(C.data.cpu().numpy(), ref.contract(a, ia, b, ib, ic)) <= 1e-13
    # update() swaps pointers to other tensors; execute reads them
    items2 = make_items(insts[::-1][: len(items)])
    shapes_ok = all(c2.data.shape == c.data.shape for (c2, _, _), (c, _, _) in zip(items2, items))
    if shapes_ok:
        g.update(items2)
        g.execute()
        torch.cuda.synchronize()


def test_group_parts_and_parallel_graph_branches():
    """The members split into parts on side streams (parallel branches of one
    captured graph), with the tensor-core work in one persistent launch per
    kernel variant or in every bucket's own launches, give results
    bit-identical to the one-stream execution."""
    import muscle_gb300 as m

    insts = instances(60, 1300, np.complex128)
    items = make_items(insts)
    g = m.Group(items, "ozaki")
    g.execute()
    torch.cuda.synchronize()
    ref_out = [C.data.clone() for C, _, _ in items]
    for parts in (1, 2, 3, 7):
        for persistent in (True, False):
            for C, _, _ in items:
                C.data.zero_()
            g.execute(parts=parts, persistent=persistent)
            torch.cuda.synchronize()
            assert all(torch.equal(C.data, r) for (C, _, _), r in zip(items, ref_out)), (parts, persistent)
    for persistent in (True, False):
        graph = g.capture(parts=4, persistent=persistent)
        for C, _, _ in items:
            C.data.zero_()
        graph.replay()
        torch.cuda.synchronize()
        assert all(torch.equal(C.data, r) for (C, _, _), r in zip(items, ref_out)), persistent
    assert m.device_status() == 0


def test_autotuner_caches_choices(tmp_path):
    import json

    import muscle_gb300 as m
    from muscle_gb300.autotune import Autotuner

    insts = instances(24, 1300, np.complex128)
    items = make_items(insts)
    path = str(tmp_path / "tune.json")
    tuner = Autotuner(path, reps=1)
    g = tuner.group(items)
    g.execute()
    torch.cuda.synchronize()
    for (C, _, _), (a, ia, b, ib, ic) in zip(items, insts):
        assert ref.rel_fro(C.data.cpu().numpy(), ref.contract(a, ia, b, ib, ic)) <= 1e-13
    cache = json.load(open(path))
    assert cache and all(v["form"] in ("ozaki", "plain") for v in cache.values())
    again = Autotuner(path, reps=1)
    forms, bands = again.tune(items)  # served from the cache, no timing
    assert all(f in ("ozaki", "plain") for f in forms)


def test_autotuner_chooses_and_caches_the_schedule(tmp_path):
    """The group schedule (parallel branches, one persistent launch or every
    bucket's own launches) is timed on the group's data, kept as the group's
    default for capture(), cached, and every schedule gives the same result."""
    import json

    from muscle_gb300.autotune import SCHEDULES, Autotuner

    insts = instances(24, 1400, np.complex128)
    items = make_items(insts)
    path = str(tmp_path / "tune.json")
    tuner = Autotuner(path, reps=1)
    g = tuner.group(items)
    chosen, times = tuner.schedule(g)
    assert chosen in SCHEDULES and set(times) == set(SCHEDULES) and g.schedule == chosen
    assert times[chosen] == min(times.values())
    graph = g.capture()
    graph.replay()
    torch.cuda.synchronize()
    for (C, _, _), (a, ia, b, ib, ic) in zip(items, insts):
        assert ref.rel_fro(C.data.cpu().numpy(), ref.contract(a, ia, b, ib, ic)) <= 1e-13
    assert any(k.startswith("schedule|") for k in json.load(open(path)))
    g2 = Autotuner(path, reps=1).group(items)
    again, t2 = Autotuner(path, reps=1).schedule(g2)
    assert again == chosen and t2 == {}  # from the cache, no timing
