"""Numpy model of the emulated FP64 form, for tests.

``emulate`` restates the digit scheme of the tensor-core kernel: per-row
(per-column for B) power-of-two scales from the largest exponent, S signed
digits of W bits taken most significant first with round-to-nearest, the
products of digit pairs i + j <= S - 1 (0-based) summed exactly, and the
result scaled back. ``estimate`` restates the device's a-priori error
estimate that picks the slice count of an adaptive plan (the same sums in
float64 instead of float32). Together they let CPU tests check that the
estimate bounds the scheme's actual error, and GPU tests check the device's
estimate against this restatement.
"""
from __future__ import annotations

import math

import numpy as np


def digit_bits(S: int) -> int:
    return 8 if S <= 6 else 7


def _biased_exp(x: np.ndarray) -> np.ndarray:
    """IEEE biased exponent of every float64 (0 for zero and subnormals)."""
    return ((np.abs(x).astype(np.float64).view(np.int64) >> 52) & 0x7FF).astype(np.int64)


def row_exponents(x: np.ndarray) -> np.ndarray:
    """Largest biased exponent of each row of a matrix (real and imaginary
    parts together), as the exponent scan computes it."""
    parts = [x.real, x.imag] if np.iscomplexobj(x) else [x]
    return np.max(np.stack([_biased_exp(p) for p in parts]), axis=0).max(axis=1)


def _digits(v: np.ndarray, S: int) -> list:
    """Balanced digits as the slicer forms them: Q + B with B = half a unit of
    the last digit plus 2^(W-1) at every digit position after the first;
    digit s >= 1 is the W-bit window minus 2^(W-1), the leading digit all the
    bits above its position."""
    W = digit_bits(S)
    Q = np.trunc(np.ldexp(v, 62)).astype(np.int64)
    B = np.int64(1) << np.int64(62 - W * S - 1)
    for s in range(1, S):
        B += np.int64(1) << np.int64(62 - W * (s + 1) + W - 1)
    Qb = Q + B
    out = []
    for s in range(S):
        sh = np.int64(62 - W * (s + 1))
        if s == 0:
            d = Qb >> sh
        else:
            d = ((Qb >> sh) & np.int64((1 << W) - 1)) - np.int64(1 << (W - 1))
        out.append(d.astype(np.float64))
    return out


def emulate(A: np.ndarray, B: np.ndarray, S: int) -> np.ndarray:
    """C = A @ B (A: M x K, B: K x N) through the digit scheme with S slices."""
    W = digit_bits(S)
    cx = np.iscomplexobj(A) or np.iscomplexobj(B)
    ea = np.maximum(row_exponents(A), 1) - 1022  # |a_ik| < 2^ea_i
    eb = np.maximum(row_exponents(B.T), 1) - 1022
    An = A * np.ldexp(1.0, -ea)[:, None]
    Bn = B * np.ldexp(1.0, -eb)[None, :]
    if cx:
        Ar, Ai = _digits(np.real(An), S), _digits(np.imag(An), S)
        Br, Bi = _digits(np.real(Bn), S), _digits(np.imag(Bn), S)
    else:
        Ar, Br = _digits(An, S), _digits(Bn, S)
    M, N = A.shape[0], B.shape[1]
    Cr, Ci = np.zeros((M, N)), np.zeros((M, N))
    for i in range(S):
        for j in range(S - i):
            w = 2.0 ** (-W * (i + 1) - W * (j + 1))
            if cx:
                Cr += w * (Ar[i] @ Br[j] - Ai[i] @ Bi[j])
                Ci += w * (Ar[i] @ Bi[j] + Ai[i] @ Br[j])
            else:
                Cr += w * (Ar[i] @ Br[j])
    C = Cr + 1j * Ci if cx else Cr
    return C * np.ldexp(1.0, ea)[:, None] * np.ldexp(1.0, eb)[None, :]


def estimate(A: np.ndarray, B: np.ndarray, S: int, margin: bool = True) -> float:
    """The adaptive form's estimate of ||C_S - C||_F / ||C||_F.

    With u = 2^-(W S), row scales 2^e_i of A, column scales 2^f_j of B,
    P = sum of squared scales and q[k] the squared norms of A's columns and
    B's rows (everything relative to the operand's largest exponent):
      digit truncation  u^2/12 (P_A sum q_B + P_B sum q_A)      (x2 complex)
      dropped pairs     (S - 1) u^2/144 K P_A P_B                 (x4 complex)
      ||C||^2           sum_k q_A[k] q_B[k]
    times 1 + 2 / sqrt(#outputs) for the fluctuation of a small norm."""
    W = digit_bits(S)
    u = 2.0 ** (-W * S)
    cx = np.iscomplexobj(A) or np.iscomplexobj(B)
    bea, beb = row_exponents(A), row_exponents(B.T)
    ma, mb = int(bea.max()), int(beb.max())
    Pa = float(np.sum(np.where(bea > 0, 4.0 ** (bea - ma), 0.0)))
    Pb = float(np.sum(np.where(beb > 0, 4.0 ** (beb - mb), 0.0)))
    # |x|^2 4^-(be_max + 1 - 1023), scaled before squaring (no overflow)
    qa = np.sum(np.ldexp(np.abs(A), -(ma + 1 - 1023)) ** 2, axis=0)
    qb = np.sum(np.ldexp(np.abs(B), -(mb + 1 - 1023)) ** 2, axis=1)
    K = A.shape[1]
    f1, f2 = (2.0, 4.0) if cx else (1.0, 1.0)
    num = u * u * (f1 / 12.0 * (Pa * qb.sum() + Pb * qa.sum()) + f2 * (S - 1) / 144.0 * K * Pa * Pb)
    den = float(np.sum(qa * qb))
    if num == 0.0:
        return 0.0
    if den == 0.0:
        return math.inf
    e = math.sqrt(num / den)
    if margin:
        e *= 1.0 + 2.0 / math.sqrt(A.shape[0] * B.shape[1])
    return e


def choose(A: np.ndarray, B: np.ndarray, tol: float = 1e-13, candidates=(5, 6, 7, 8)) -> int:
    """Smallest candidate slice count whose estimate is within tol, else 0."""
    if not (np.all(np.isfinite(A)) and np.all(np.isfinite(B))):
        return 0
    for S in sorted(candidates):
        if estimate(A, B, S) <= tol:
            return S
    return 0
