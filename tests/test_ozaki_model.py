"""CPU checks of the error estimate behind the adaptive slice count.

The estimate (tests/ozaki_model.py, restating the device's chooser) must not
fall below the actual error of the digit scheme (emulated exactly in numpy)
on data of very different shapes, and the count it chooses must meet the
tolerance. The reference product is evaluated in extended precision."""
import numpy as np
import pytest

from tests import ozaki_model as oz

M, N, K = 40, 36, 1536


def _logu(rng, shape, lo, hi, cx):
    mag = np.exp2(rng.uniform(lo, hi, size=shape))
    if cx:
        return mag * np.exp(1j * rng.uniform(0, 2 * np.pi, size=shape))
    return mag * np.where(rng.uniform(size=shape) < 0.5, -1.0, 1.0)


def _normal(rng, shape, cx):
    x = rng.standard_normal(shape)
    return x + 1j * rng.standard_normal(shape) if cx else x


def _cases(cx):
    rng = np.random.default_rng(123 if cx else 321)
    out = {
        "normal": (_normal(rng, (M, K), cx), _normal(rng, (K, N), cx)),
        "loguniform 2^-20..2^20": (_logu(rng, (M, K), -20, 20, cx), _logu(rng, (K, N), -20, 20, cx)),
        "loguniform 2^-60..2^60": (_logu(rng, (M, K), -60, 60, cx), _logu(rng, (K, N), -60, 60, cx)),
    }
    a, b = _normal(rng, (M, K), cx), _normal(rng, (K, N), cx)
    a[:, 0] *= 1e6  # one dominant column of A
    out["dominant column"] = (a, b)
    s = np.exp2(rng.uniform(-20, 20, K))  # A's columns and B's rows scaled inversely
    out["k-scaled"] = (_normal(rng, (M, K), cx) * s[None, :], _normal(rng, (K, N), cx) / s[:, None])
    out["row-scaled"] = (_normal(rng, (M, K), cx) * np.exp2(rng.uniform(-30, 30, M))[:, None],
                         _normal(rng, (K, N), cx))
    return out


def _exact(a, b):
    ld = np.clongdouble if np.iscomplexobj(a) or np.iscomplexobj(b) else np.longdouble
    return a.astype(ld) @ b.astype(ld)


def _rel(x, ref):
    ref = np.asarray(ref)
    return float(np.linalg.norm((x - ref).astype(np.complex128 if np.iscomplexobj(ref) else np.float64)) /
                 np.linalg.norm(ref.astype(np.complex128 if np.iscomplexobj(ref) else np.float64)))


@pytest.mark.parametrize("cx", [False, True])
def test_estimate_bounds_the_emulated_error(cx):
    for name, (a, b) in _cases(cx).items():
        ref = _exact(a, b)
        for S in (5, 6, 7, 8):
            err = _rel(oz.emulate(a, b, S), ref)
            if err < 2e-15:  # at the float64 rounding of the final combination
                continue
            est = oz.estimate(a, b, S, margin=False)
            assert est >= 0.9 * err, (name, S, est, err)
            assert est <= 20 * err, (name, S, est, err)  # and not uselessly loose


@pytest.mark.parametrize("cx", [False, True])
def test_chosen_count_meets_the_tolerance(cx):
    chosen = {}
    for name, (a, b) in _cases(cx).items():
        S = oz.choose(a, b)
        chosen[name] = S
        if S:
            assert _rel(oz.emulate(a, b, S), _exact(a, b)) <= 1e-13, (name, S)
    # the choice follows the data: well-scaled data needs fewer slices than a
    # dominant column, and inversely scaled columns defeat row scaling
    assert chosen["normal"] in (5, 6) and chosen["dominant column"] == 8 and chosen["k-scaled"] == 0, chosen


def test_estimate_edge_cases():
    z = np.zeros((4, 8))
    b = np.ones((8, 3))
    assert oz.estimate(z, b, 5) == 0.0  # an all-zero operand: every form is exact
    a = np.zeros((4, 8))
    a[:, 0] = 1.0
    b = np.zeros((8, 3))
    b[1, :] = 1.0  # no k where both are nonzero: C = 0, nothing to rest a relative bound on
    assert oz.estimate(a, b, 8) == float("inf")
    a = np.ones((4, 8))
    a[2, 3] = np.inf
    assert oz.choose(a, np.ones((8, 3))) == 0
