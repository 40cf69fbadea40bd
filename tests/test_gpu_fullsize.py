"""Full-size cases of the benchmark workloads on the device, checked where the
CPU oracle cannot follow at full size:
  * sampled output entries against their correctly rounded values (every
    product split exactly, summed with math.fsum) -- this also bounds the
    error of the FP64 plain form that the benchmark uses as its reference;
  * size-independent properties: scaling an operand by a power of two scales
    the result bit-exactly (every form), and the permutation is bit-exact.
Workloads: the precision form (ComplexF64 A(i,k1,k2) = 8192x128x64,
B(k2,j,k1) = 64x8192x128, log-uniform magnitudes 2^-20..2^20), the permuting
plain shapes A(a,b,c,d,e) = 64x96x64x48x32, B(e,c,f,a) = 32x64x128x64 and the
MPS bond A(l,p,r) = B(r,q,s) = 512x4x512."""
import math

import numpy as np
import pytest
import torch

import muscle_gb300 as m
from muscle_gb300 import workloads as wl
from oracle import muscle_ref as ref

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

F64_TOL = 1e-13
F32_TOL = 1e-5


def contract(A, ia, B, ib, ic, form, slices=0):
    with m.with_backend(m.BackendGB300(form, slices)):
        C = m.binary_einsum(m.Tensor(A, ia), m.Tensor(B, ib), out=ic)
    torch.cuda.synchronize()
    return C.data


def positions(rng, shape, n):
    return [tuple(int(rng.integers(0, s)) for s in shape) for _ in range(n)]


def sampled_rel(got, pos, exact):
    g = np.array([complex(got[p].item()) for p in pos])
    e = np.array(exact, dtype=np.complex128)
    return float(np.linalg.norm(g - e) / np.linalg.norm(e))


def colmajor_randn(gen, shape, dtype):
    t = torch.randn(list(reversed(shape)), dtype=dtype, device="cuda", generator=gen)
    return t.permute(*reversed(range(len(shape))))


def full_rel(x, y):
    return (torch.linalg.vector_norm((x - y).flatten()) / torch.linalg.vector_norm(y.flatten())).item()


@pytest.fixture(scope="module")
def precision_workload():
    (a, ia), (b, ib), ic = wl.gen_config3(seed=0)
    A = torch.from_numpy(a).cuda()
    B = torch.from_numpy(b).cuda()
    yield a, ia, b, ib, ic, A, B
    del A, B
    torch.cuda.empty_cache()


def test_precision_form_sampled_exact(precision_workload):
    a, ia, b, ib, ic, A, B = precision_workload
    rng = np.random.default_rng(3)
    pos = positions(rng, (a.shape[0], b.shape[1]), 48)
    exact = ref.exact_entries_fast(a, ia, b, ib, ic, pos)
    plain = contract(A, ia, B, ib, ic, "plain")
    e_plain = sampled_rel(plain, pos, exact)
    print(f"plain FP64 sampled rel err {e_plain:.3e}")
    assert e_plain <= 1e-14  # the FP64 reference is two orders inside the tolerance
    for s in (6, 7, 8):
        oz = contract(A, ia, B, ib, ic, "ozaki", s)
        e_oz = sampled_rel(oz, pos, exact)
        e_full = full_rel(oz, plain)
        print(f"ozaki S={s}: sampled rel err {e_oz:.3e}, full rel err vs plain {e_full:.3e}")
        assert e_oz <= F64_TOL and e_full <= F64_TOL, (s, e_oz, e_full)
        del oz
    del plain
    torch.cuda.empty_cache()


def test_precision_form_float32_variant(precision_workload):
    a, ia, b, ib, ic, A, B = precision_workload
    a32, b32 = a.astype(np.complex64), b.astype(np.complex64)
    rng = np.random.default_rng(4)
    pos = positions(rng, (a.shape[0], b.shape[1]), 32)
    exact = ref.exact_entries_fast(a32.astype(np.complex128), ia, b32.astype(np.complex128), ib, ic, pos)
    A32, B32 = A.to(torch.complex64), B.to(torch.complex64)
    got = contract(A32, ia, B32, ib, ic, "bf16x3")
    e = sampled_rel(got, pos, exact)
    print(f"bf16x3 sampled rel err {e:.3e}")
    assert e <= F32_TOL
    # the result is a power-of-two-scaled copy when an operand is scaled
    got2 = contract(A32 * 0.125, ia, B32, ib, ic, "bf16x3")
    assert torch.equal(got2, got * 0.125)


def test_precision_form_power_of_two_linearity(precision_workload):
    a, ia, b, ib, ic, A, B = precision_workload
    for form, s in (("ozaki", 7), ("ozaki", 6), ("plain", 0)):
        c1 = contract(A, ia, B, ib, ic, form, s)
        c2 = contract(A, ia, B * 0.25, ib, ic, form, s)
        assert torch.equal(c2, c1 * 0.25), form
        del c1, c2
    torch.cuda.empty_cache()


@pytest.mark.parametrize("dtype", [torch.complex128, torch.float64])
def test_permuting_shapes_sampled_exact(dtype):
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    ia, ea = ["a", "b", "c", "d", "e"], [64, 96, 64, 48, 32]
    ib, eb = ["e", "c", "f", "a"], [32, 64, 128, 64]
    ic = ["b", "d", "f"]
    A = colmajor_randn(gen, ea, dtype)
    B = colmajor_randn(gen, eb, dtype)
    rng = np.random.default_rng(5)
    pos = positions(rng, (96, 48, 128), 12)
    exact = []
    for bb, dd, ff in pos:
        x = A[:, bb, :, dd, :].cpu().numpy()  # (a, c, e)
        y = B[:, :, ff, :].cpu().numpy()  # (e, c, a)
        exact.append(ref.exact_dot(x.ravel(order="F"), np.transpose(y, (2, 1, 0)).ravel(order="F")))
    forms = [("plain", 0), ("ozaki", 7)]
    res = {}
    for form, s in forms:
        got = contract(A, ia, B, ib, ic, form, s)
        res[form] = got
        e = sampled_rel(got, pos, exact)
        print(f"{dtype} {form}: sampled rel err {e:.3e}")
        assert e <= F64_TOL, (form, e)
    assert full_rel(res["ozaki"], res["plain"]) <= F64_TOL
    del res
    # the permutation BackendBase stages for this pair, bit-exact at full size
    Y = m.permutedims(m.Tensor(A, ia), ["b", "d", "a", "c", "e"])
    torch.cuda.synchronize()
    assert torch.equal(Y.data, A.permute(1, 3, 0, 2, 4))
    del Y, A, B
    torch.cuda.empty_cache()


@pytest.mark.parametrize("dtype", [torch.complex128, torch.float64])
def test_mps_bond_sampled_exact(dtype):
    gen = torch.Generator(device="cuda")
    gen.manual_seed(12)
    ia, ib, ic = ["l", "p", "r"], ["r", "q", "s"], ["l", "p", "q", "s"]
    A = colmajor_randn(gen, [512, 4, 512], dtype)
    B = colmajor_randn(gen, [512, 4, 512], dtype)
    a, b = A.cpu().numpy(), B.cpu().numpy()
    rng = np.random.default_rng(6)
    pos = positions(rng, (512, 4, 4, 512), 64)
    exact = ref.exact_entries_fast(a, ia, b, ib, ic, pos)
    for form, s in (("plain", 0), ("ozaki", 7), ("ozaki", 6)):
        got = contract(A, ia, B, ib, ic, form, s)
        e = sampled_rel(got, pos, exact)
        assert e <= F64_TOL, (form, s, e)
        assert math.isfinite(e)
