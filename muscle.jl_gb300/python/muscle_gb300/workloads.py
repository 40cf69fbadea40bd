"""Seeded synthetic workloads for the benchmark configurations.

Shapes, label orders and value distributions of the workloads Muscle.jl's
contractions are measured on (no public dataset is involved; PCG64 seeds make
every array reproducible, so the CPU oracle and the GPU see identical bytes).
Arrays are numpy, column-major like Julia arrays.
"""
from __future__ import annotations

import numpy as np


def _cnormal(rng, shape, dtype, scale=1.0):
    if np.issubdtype(dtype, np.complexfloating):
        re = rng.standard_normal(shape)
        im = rng.standard_normal(shape)
        return (scale * (re + 1j * im)).astype(dtype)
    return (scale * rng.standard_normal(shape)).astype(dtype)


def colmajor(x):
    return np.array(x, order="F")  # keeps 0-d arrays 0-d


def gen_config1(seed=0, dtype=np.complex128, dim=32):
    """Plain C64: A(i,j,k,l), B(k,m,l,n), all extents ``dim`` (32 in the
    benchmark), re/im iid N(0,1), PCG64(seed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = colmajor(_cnormal(rng, (dim,) * 4, dtype))
    b = colmajor(_cnormal(rng, (dim,) * 4, dtype))
    return (a, ["i", "j", "k", "l"]), (b, ["k", "m", "l", "n"]), ["i", "j", "m", "n"]


def gen_config2a(seed=0, dtype=np.complex128, scale=1):
    """A(a,b,c,d,e) = 64x96x64x48x32, B(e,c,f,a) = 32x64x128x64 -> (b,d,f);
    ``scale`` divides every extent (for CPU-sized parity cases)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ea = [64 // scale, 96 // scale, 64 // scale, 48 // scale, 32 // scale]
    eb = [32 // scale, 64 // scale, 128 // scale, 64 // scale]
    a = colmajor(_cnormal(rng, ea, dtype))
    b = colmajor(_cnormal(rng, eb, dtype))
    return (a, ["a", "b", "c", "d", "e"]), (b, ["e", "c", "f", "a"]), ["b", "d", "f"]


def gen_config2b(seed=0, dtype=np.complex128, scale=1):
    """MPS bond: A(l,p,r) = 512x4x512, B(r,q,s) = 512x4x512 -> (l,p,q,s)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = colmajor(_cnormal(rng, (512 // scale, 4, 512 // scale), dtype))
    b = colmajor(_cnormal(rng, (512 // scale, 4, 512 // scale), dtype))
    return (a, ["l", "p", "r"]), (b, ["r", "q", "s"]), ["l", "p", "q", "s"]


def loguniform_complex(rng, shape, dtype=np.complex128, lo=-20.0, hi=20.0):
    """|z| = 2^U(lo,hi), arg z = U(0, 2 pi) (real dtypes: random sign)."""
    mag = np.exp2(rng.uniform(lo, hi, size=shape))
    if np.issubdtype(dtype, np.complexfloating):
        ph = rng.uniform(0.0, 2 * np.pi, size=shape)
        return (mag * np.exp(1j * ph)).astype(dtype)
    sgn = np.where(rng.uniform(size=shape) < 0.5, -1.0, 1.0)
    return (mag * sgn).astype(dtype)


def gen_config3(seed=0, dtype=np.complex128, n=8192, k1=128, k2=64):
    """Precision form: A(i,k1,k2) = n x k1 x k2, B(k2,j,k1) = k2 x n x k1
    (M = N = n, K = k1 k2), log-uniform magnitudes over 2^-20..2^20."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = colmajor(loguniform_complex(rng, (n, k1, k2), dtype))
    b = colmajor(loguniform_complex(rng, (k2, n, k1), dtype))
    return (a, ["i", "k1", "k2"]), (b, ["k2", "j", "k1"]), ["i", "j"]


PEPS_CHI = (8, 12, 16, 24, 32, 48, 64)
PEPS_CAP = 1 << 24  # elements of A + B + C per instance


def peps_instance(seed, dtype=np.complex128, cap=PEPS_CAP, max_tries=1000):
    """One batching-form instance: a rank-5 site (physical dim 2, four bonds of
    one bond dimension chi drawn from PEPS_CHI) contracted with a neighbour
    over 1-3 shared bonds; entries iid complex N(0, 1/chi). Instances whose
    A + B + C exceed ``cap`` elements are redrawn from the same stream.
    Returns ((a, ia), (b, ib), ic, tries)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    for tries in range(1, max_tries + 1):
        chi = int(rng.choice(PEPS_CHI))
        nsh = int(rng.integers(1, 4))
        bonds = ["u", "r", "d", "l"]
        shared = list(rng.choice(bonds, size=nsh, replace=False))
        ia = ["p"] + bonds
        ib = ["q"] + shared + [f"x{t}" for t in range(4 - nsh)]
        ea = [2] + [chi] * 4
        eb = [2] + [chi] * 4
        ic = ["p"] + [b for b in bonds if b not in shared] + ["q"] + [f"x{t}" for t in range(4 - nsh)]
        na, nb = 2 * chi**4, 2 * chi**4
        nc = 4 * chi ** (2 * (4 - nsh))
        if na + nb + nc > cap:
            continue
        sc = 1.0 / np.sqrt(2.0 * chi)  # complex N(0, 1/chi): re, im ~ N(0, 1/(2 chi))
        a = colmajor(_cnormal(rng, ea, dtype, sc))
        b = colmajor(_cnormal(rng, eb, dtype, sc))
        return (a, ia), (b, ib), ic, tries
    raise RuntimeError("no instance under the cap")


SERVE_DTYPES = (np.complex128, np.float64, np.complex64)


def serve_request(rng, flops_lo=1e4, flops_hi=1e10, dtypes=SERVE_DTYPES):
    """One serving-form request: a random binary contraction with ranks 3-6,
    1-3 contracted labels, extents drawn so that its algorithmic flops are
    log-uniform in [flops_lo, flops_hi], labels in random orders, element type
    drawn from ``dtypes``. Returns (shape_a, ia, shape_b, ib, ic, dtype, flops)."""
    dtype = dtypes[int(rng.integers(len(dtypes)))]
    cx = np.issubdtype(dtype, np.complexfloating)
    target = float(np.exp(rng.uniform(np.log(flops_lo), np.log(flops_hi))))
    mnk = max(target / (8.0 if cx else 2.0), 1.0)
    while True:
        ra, rb = int(rng.integers(3, 7)), int(rng.integers(3, 7))
        nc = int(rng.integers(1, 4))
        if nc < ra and nc < rb:
            break
    fa, fb = ra - nc, rb - nc
    frac = rng.dirichlet([4.0, 4.0, 4.0])  # share of log(MNK) for M, N, K

    def split(total, parts):
        if parts == 0:
            return []
        w = rng.dirichlet([2.0] * parts)
        return [max(1, int(round(total ** wi))) for wi in w]

    em, en, ek = split(mnk ** frac[0], fa), split(mnk ** frac[1], fb), split(mnk ** frac[2], nc)
    names = [f"x{i}" for i in range(fa + fb + nc)]
    rng.shuffle(names)
    lm, ln, lk = names[:fa], names[fa:fa + fb], names[fa + fb:]
    ext = dict(zip(lm + ln + lk, em + en + ek))
    ia = list(lm + lk)
    ib = list(lk + ln)
    ic = list(lm + ln)
    for lab in (ia, ib, ic):
        rng.shuffle(lab)
    flops = (8.0 if cx else 2.0) * np.prod(em) * np.prod(en) * np.prod(ek)
    return [ext[i] for i in ia], ia, [ext[i] for i in ib], ib, ic, dtype, float(flops)


def serve_arrays(rng, req):
    """Seeded operands (iid N(0,1), complex parts independent) for a request."""
    sa, ia, sb, ib, ic, dtype, _ = req
    return _cnormal(rng, sa, dtype), _cnormal(rng, sb, dtype)
