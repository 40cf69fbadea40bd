"""Failure detection on the device without a fault: every wait in the
library's kernels has a limit (about a second); when it runs out the kernel
records MGB_ERR_DEVICE_TIMEOUT in the device status word and returns, so the
context stays usable. The self-test kernel waits on an mbarrier that nothing
completes, through the same wait routine the contraction kernels use."""
import time

import numpy as np
import pytest
import torch

import muscle_gb300 as m
from muscle_gb300 import _lib
from oracle import muscle_ref as ref
from tests.gpu_util import run

pytestmark = pytest.mark.gpu

MGB_ERR_DEVICE_TIMEOUT = 6


def test_wait_timeout_is_reported_and_context_survives():
    lib = _lib.load()
    assert m.device_status() == 0
    t0 = time.perf_counter()
    _lib.check(lib.mgb_selftest_wait_timeout(torch.cuda.current_stream().cuda_stream), lib)
    status = m.device_status()  # synchronises the stream
    elapsed = time.perf_counter() - t0
    assert status == MGB_ERR_DEVICE_TIMEOUT
    assert 0.2 < elapsed < 30.0
    assert m.device_status() == 0  # reading clears the word
    # the context is intact: contractions in every form still match the oracle
    rng = np.random.default_rng(17)
    a = np.array(rng.standard_normal((40, 33)) + 1j * rng.standard_normal((40, 33)), order="F")
    b = np.array(rng.standard_normal((33, 21)) + 1j * rng.standard_normal((33, 21)), order="F")
    want = ref.contract(a, ["i", "k"], b, ["k", "j"], ["i", "j"])
    for form, slices in (("ozaki", 6), ("ozaki", 7), ("plain", 0)):
        got, _ = run(a, ["i", "k"], b, ["k", "j"], ["i", "j"], form, slices)
        assert ref.rel_fro(got, want) <= 1e-13, form
    assert m.device_status() == 0
