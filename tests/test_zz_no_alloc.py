"""mgb_contract_noalloc: the contraction entry point that allocates nothing.

It serves callers that cannot allocate device memory (their own allocator
owns a fixed byte budget, or a cudaMalloc's implicit synchronisation is not
acceptable on their path); its workspace is a fixed-size scratch array the
library holds on each GPU. This file is collected last so that a failure here
cannot stop the rest of the GPU suite.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import muscle_ref as ref

pytestmark = pytest.mark.gpu


def _call_plan(a, ia, b, ib, c, ic, form, slices):
    import muscle_gb300 as m

    I = lambda xs: [m.Index(x) for x in xs]
    return m.contraction_plan(a, I(ia), b, I(ib), c, I(ic), form, slices)


def test_noalloc_matches_workspace_entry_point_twice():
    import muscle_gb300 as m
    from muscle_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(31)
    a = np.array(rng.standard_normal((96, 40, 12)) + 1j * rng.standard_normal((96, 40, 12)), order="F")
    b = np.array(rng.standard_normal((12, 70, 40)) + 1j * rng.standard_normal((12, 70, 40)), order="F")
    ia, ib, ic = ["i", "k1", "k2"], ["k2", "j", "k1"], ["i", "j"]
    A, B = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for form, slices in (("ozaki", 7), ("plain", 0)):
        C_ws = m.empty_colmajor([96, 70], torch.complex128, "cuda")
        plan = _call_plan(A, ia, B, ib, C_ws, ic, form, slices)
        assert plan.workspace_bytes <= _lib_max()
        ws = torch.empty(max(plan.workspace_bytes, 1), dtype=torch.uint8, device="cuda")
        _lib.check(lib.mgb_contract(plan.handle, A.data_ptr(), B.data_ptr(), C_ws.data_ptr(), ws.data_ptr(),
                                    plan.workspace_bytes, stream), lib)
        want = C_ws.cpu().numpy()
        assert ref.rel_fro(want, ref.contract(a, ia, b, ib, ic)) <= 1e-13
        for _ in range(2):  # the scratch keeps the previous call's contents
            C_na = m.zeros_colmajor([96, 70], torch.complex128, "cuda")
            _lib.check(lib.mgb_contract_noalloc(plan.handle, A.data_ptr(), B.data_ptr(), C_na.data_ptr(), stream), lib)
            got = C_na.cpu().numpy()
            assert ref.rel_fro(got, want) <= 1e-13, form
    assert m.device_status() == 0


def _lib_max():
    from muscle_gb300 import _lib

    return _lib.NOALLOC_SCRATCH_BYTES


def test_noalloc_rejects_plans_larger_than_its_scratch():
    import muscle_gb300 as m
    from muscle_gb300 import _lib

    lib = _lib.load()
    A = torch.zeros(1024, 1024, dtype=torch.complex128, device="cuda")
    B = torch.zeros(1024, 1024, dtype=torch.complex128, device="cuda")
    C = m.empty_colmajor([1024, 1024], torch.complex128, "cuda")
    plan = _call_plan(A, ["i", "k"], B, ["k", "j"], C, ["i", "j"], "ozaki", 7)
    assert plan.workspace_bytes > _lib_max()
    st = lib.mgb_contract_noalloc(plan.handle, A.data_ptr(), B.data_ptr(), C.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream)
    assert st == _lib.ERR_WORKSPACE
    assert b"at most" in lib.mgb_last_error()
