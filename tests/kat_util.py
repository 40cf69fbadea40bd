"""Helpers that turn kat_cases.json entries into arrays and expected values."""
import numpy as np

NP = {"float32": np.float32, "float64": np.float64, "complex64": np.complex64, "complex128": np.complex128}


def fill_value(f):
    return complex(f[0], f[1]) if isinstance(f, list) else f


def make_array(spec):
    dt = NP[spec["dtype"]]
    if "values" in spec:
        return np.array(np.array(spec["values"], dtype=dt).reshape(spec["shape"], order="F"), order="F")
    if spec.get("iota"):
        n = int(np.prod(spec["shape"]))
        return np.array(np.arange(1, n + 1, dtype=dt).reshape(spec["shape"], order="F"), order="F")
    return np.array(np.full(spec["shape"], fill_value(spec["fill"]), dtype=dt), order="F")


def expected_binary(case, exp, a, b):
    """Expected array of a binary case (fill or the test's own formula)."""
    if "fill" in exp:
        return np.full(exp["shape"], fill_value(exp["fill"]))
    if exp["formula"].startswith("reshape"):
        a_mat = a.reshape(2, 12, order="F")
        b_mat = np.transpose(b, (2, 0, 1)).reshape(12, 5, order="F")
        return a_mat @ b_mat
    c = np.zeros((2, 4, 5), dtype=np.result_type(a, b))
    for i in range(2):
        for j in range(3):
            for k in range(4):
                for l in range(5):
                    c[i, k, l] += a[i, j, k] * b[k, l, j]
    return c


def expected_hadamard(exp, b, ib):
    """Expected c of a hadamard case on a = ones: a fill, or b broadcast along
    c's labels (each slice of c at b's coordinates equals b's entry there)."""
    if "fill" in exp:
        return np.full(exp["shape"], fill_value(exp["fill"]))
    c = np.zeros(exp["shape"], dtype=b.dtype)
    for idx in np.ndindex(*exp["shape"]):
        pos = dict(zip(exp["inds"], idx))
        c[idx] = b[tuple(pos[i] for i in ib)]
    return c
