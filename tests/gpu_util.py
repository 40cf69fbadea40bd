"""Helpers for GPU tests: numpy <-> device tensors (layout preserved) and a
call through the product API."""
import numpy as np
import torch

TOL = {np.float64: 1e-13, np.complex128: 1e-13, np.float32: 1e-5, np.complex64: 1e-5}


def to_dev(x: np.ndarray) -> torch.Tensor:
    t = torch.from_numpy(np.asarray(x))
    return t.to("cuda")


def to_np(t: torch.Tensor) -> np.ndarray:
    return t.detach().cpu().numpy()


def run(a, ia, b, ib, ic, form="auto", slices=0):
    import muscle_gb300 as m

    A = m.Tensor(to_dev(a), ia)
    B = m.Tensor(to_dev(b), ib)
    with m.with_backend(m.BackendGB300(form, slices)):
        C = m.binary_einsum(A, B, out=ic)
    torch.cuda.synchronize()
    return to_np(C.data), C


def forms_for(dtype):
    if np.dtype(dtype) in (np.float64, np.complex128):
        return [("plain", 0), ("ozaki", 7), ("auto", 0)]
    return [("plain", 0), ("bf16x3", 0), ("auto", 0)]
