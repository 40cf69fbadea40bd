"""Host-side checks that need no GPU: the C ABI library loads and exports
every declared symbol, plan construction (label algebra, errors, workspace
sizes), and the Python mirror of Muscle.jl's data model and dispatch."""
import ctypes
import os
import re

import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(mgb_\w+)\s*\(", src, re.M))
    return names


def test_library_exports_every_declared_symbol():
    import muscle_gb300
    from muscle_gb300 import _lib

    lib = muscle_gb300.library()
    names = declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, n
    assert lib.mgb_version().startswith(b"muscle_gb300")


def _plan(a, b, c, form=0, slices=0):
    from muscle_gb300 import _lib

    lib = _lib.load()
    da, ka = _lib.make_desc(*a)
    db, kb = _lib.make_desc(*b)
    dc, kc = _lib.make_desc(*c)
    h = ctypes.c_void_p()
    st = lib.mgb_contraction_plan(ctypes.byref(h), ctypes.byref(da), ctypes.byref(db), ctypes.byref(dc), form, slices)
    info = _lib.PlanInfo()
    if st == 0:
        assert lib.mgb_plan_info_get(h, ctypes.byref(info)) == 0
        lib.mgb_plan_destroy(h)
    return st, info, lib.mgb_last_error().decode()


def colmajor(shape):
    s, out = 1, []
    for e in shape:
        out.append(s)
        s *= e
    return out


def desc(dtype, modes, shape):
    return (dtype, modes, shape, colmajor(shape))


def test_plan_config1_folds_to_gemm():
    from muscle_gb300 import _lib

    st, info, _ = _plan(desc(_lib.C64, [0, 1, 2, 3], [32] * 4), desc(_lib.C64, [2, 4, 3, 5], [32] * 4),
                        desc(_lib.C64, [0, 1, 4, 5], [32] * 4), _lib.FORM_OZAKI, 7)
    assert st == 0
    assert (info.m, info.n, info.k, info.batch) == (1024, 1024, 1024, 1)
    assert info.flops == 8.0 * 1024**3
    assert info.slices == 7 and info.form == _lib.FORM_OZAKI
    # A and B slices (7 x M x 2K and 7 x 2N x 2K bf16) + scales
    assert info.workspace_bytes >= 7 * 1024 * 2048 * 2 + 7 * 2048 * 2048 * 2


def test_plan_errors_map_to_julia_exceptions():
    from muscle_gb300 import _lib

    # extent mismatch of a shared label -> DimensionMismatch
    st, _, msg = _plan(desc(_lib.F64, [0, 1], [2, 3]), desc(_lib.F64, [1, 2], [4, 5]), desc(_lib.F64, [0, 2], [2, 5]))
    assert st == _lib.ERR_DIMENSION_MISMATCH and "extent" in msg
    # output label absent from the operands -> ArgumentError
    st, _, _ = _plan(desc(_lib.F64, [0, 1], [2, 3]), desc(_lib.F64, [1, 2], [3, 5]), desc(_lib.F64, [0, 7], [2, 5]))
    assert st == _lib.ERR_ARGUMENT
    # wrong result element type -> ArgumentError
    st, _, _ = _plan(desc(_lib.F64, [0, 1], [2, 3]), desc(_lib.C64, [1, 2], [3, 5]), desc(_lib.F64, [0, 2], [2, 5]))
    assert st == _lib.ERR_ARGUMENT
    # a free label dropped from the output -> ArgumentError
    st, _, _ = _plan(desc(_lib.F64, [0, 1], [2, 3]), desc(_lib.F64, [1, 2], [3, 5]), desc(_lib.F64, [0], [2]))
    assert st == _lib.ERR_ARGUMENT
    # Ozaki on a Float32 result -> unsupported
    st, _, _ = _plan(desc(_lib.F32, [0, 1], [2, 3]), desc(_lib.F32, [1, 2], [3, 5]), desc(_lib.F32, [0, 2], [2, 5]),
                     _lib.FORM_OZAKI)
    assert st == _lib.ERR_UNSUPPORTED
    # slice count out of range
    st, _, _ = _plan(desc(_lib.F64, [0, 1], [2, 3]), desc(_lib.F64, [1, 2], [3, 5]), desc(_lib.F64, [0, 2], [2, 5]),
                     _lib.FORM_OZAKI, 12)
    assert st == _lib.ERR_ARGUMENT


def test_plan_band_setting():
    """The rasterisation band is a schedule knob: 0 (default) .. 64 row tiles,
    rejected outside that range and on a null plan."""
    from muscle_gb300 import _lib

    lib = _lib.load()
    da, _ = _lib.make_desc(*desc(_lib.C64, [0, 1], [300, 40]))
    db, _ = _lib.make_desc(*desc(_lib.C64, [1, 2], [40, 70]))
    dc, _ = _lib.make_desc(*desc(_lib.C64, [0, 2], [300, 70]))
    h = ctypes.c_void_p()
    assert lib.mgb_contraction_plan(ctypes.byref(h), ctypes.byref(da), ctypes.byref(db), ctypes.byref(dc),
                                    _lib.FORM_OZAKI, 6) == 0
    try:
        for band in (0, 1, 2, 64):
            assert lib.mgb_plan_set_band(h, band) == 0, band
        for band in (-1, 65):
            assert lib.mgb_plan_set_band(h, band) == _lib.ERR_ARGUMENT, band
            assert b"band" in lib.mgb_last_error()
    finally:
        lib.mgb_plan_destroy(h)
    assert lib.mgb_plan_set_band(None, 1) == _lib.ERR_ARGUMENT


def test_plan_batch_and_scalar():
    from muscle_gb300 import _lib

    st, info, _ = _plan(desc(_lib.F64, [0, 1, 9], [2, 3, 6]), desc(_lib.F64, [1, 2, 9], [3, 4, 6]),
                        desc(_lib.F64, [9, 0, 2], [6, 2, 4]), _lib.FORM_PLAIN)
    assert st == 0 and (info.m, info.n, info.k, info.batch) == (2, 4, 3, 6)
    st, info, _ = _plan(desc(_lib.F64, [], []), desc(_lib.F64, [0, 1], [2, 3]), desc(_lib.F64, [1, 0], [3, 2]),
                        _lib.FORM_PLAIN)
    assert st == 0 and (info.m, info.n, info.k) == (1, 6, 1)


def test_plan_folds_config2a_groups():
    from muscle_gb300 import _lib

    # A(a,b,c,d,e) B(e,c,f,a) -> C(b,d,f): M = b*d, N = f, K = a*c*e
    st, info, _ = _plan(desc(_lib.C64, [0, 1, 2, 3, 4], [64, 96, 64, 48, 32]), desc(_lib.C64, [4, 2, 5, 0], [32, 64, 128, 64]),
                        desc(_lib.C64, [1, 3, 5], [96, 48, 128]), _lib.FORM_PLAIN)
    assert st == 0 and (info.m, info.n, info.k) == (96 * 48, 128, 64 * 64 * 32)
    assert abs(info.flops - 6.18e11) / 6.18e11 < 0.01


def test_data_model_and_dispatch():
    import muscle_gb300 as m

    i, j = m.Index("i"), m.Index("j")
    assert m.Index(i) == i and hash(m.Index("i")) == hash(i)
    with pytest.raises(m.ArgumentError):
        m.Tensor(torch.ones(2, 3), [i])
    with pytest.raises(m.DimensionMismatch):
        m.Tensor(torch.ones(2, 3), [i, i])
    t = m.Tensor(torch.ones(2, 3, 2), [i, j, i])
    assert m.nonunique(t.inds) == [i]
    assert t.size(j) == 3
    # host arrays have no rule in this package (they belong to Muscle's BackendBase)
    with pytest.raises(m.ArgumentError):
        m.binary_einsum(m.Tensor(torch.ones(2, 3), ["i", "j"]), m.Tensor(torch.ones(3), ["j"]))
    with pytest.raises(m.ArgumentError):
        m.unary_einsum(t)
    # scoped override wins over the rule table and is restored afterwards
    with m.with_backend(m.BackendGB300("plain")) as be:
        assert m.choose_backend(m.binary_einsum, t.data, t.data) == be
    assert m.with_backend(lambda: m.choose_backend(m.unary_einsum, t.data), m.BackendGB300("ozaki", 6)) == m.BackendGB300("ozaki", 6)
    with pytest.raises(m.ArgumentError):
        m.choose_backend(m.binary_einsum, t.data, t.data)
    # a backend that lacks the method raises like the reference's fallback methods
    with pytest.raises(m.ArgumentError):
        m.BackendBase().binary_einsum([], t, t)


def test_column_major_allocation():
    import muscle_gb300 as m

    x = m.empty_colmajor([2, 3, 4], torch.float64, "cpu")
    assert x.shape == (2, 3, 4) and x.stride() == (1, 2, 6)
    assert m.empty_colmajor([], torch.float64, "cpu").dim() == 0


def test_front_end_label_algebra_matches_oracle(kat_cases):
    """The product's label algebra equals the oracle's on every KAT case,
    with labels given as plain tags or as Index objects."""
    import muscle_gb300 as m
    from muscle_gb300.ops import binary_inds_c, unary_inds_y
    from oracle import muscle_ref as ref

    for case in kat_cases:
        if case["kind"] == "binary":
            ia = [m.Index(x) for x in case["a"]["inds"]]
            ib = [m.Index(x) for x in case["b"]["inds"]]
            want = ref.front_inds_c(case["a"]["inds"], case["b"]["inds"], case["dims"], case["out"])
            for wrap in (lambda v: v, lambda v: None if v is None else [m.Index(x) for x in v]):
                got = binary_inds_c(ia, ib, wrap(case["dims"]), wrap(case["out"]))
                assert [i.tag for i in got] == want, case["name"]
                assert [i.tag for i in got] == case["expect_gpu"]["inds"], case["name"]
        elif case["kind"] == "unary" and case["inplace"] is None:
            ix = [m.Index(x) for x in case["x"]["inds"]]
            got = unary_inds_y(ix, case["dims"], case["out"])
            assert [i.tag for i in got] == case["expect"]["inds"], case["name"]


def test_noalloc_scratch_constant_matches_header():
    """The Python constant the no-allocation tests size against is the
    header's MGB_NOALLOC_SCRATCH_BYTES."""
    import re

    from muscle_gb300 import _lib

    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "muscle_gb300.h")).read()
    m = re.search(r"#define MGB_NOALLOC_SCRATCH_BYTES \((\d+)u << (\d+)\)", hdr)
    assert m, "MGB_NOALLOC_SCRATCH_BYTES not found"
    assert _lib.NOALLOC_SCRATCH_BYTES == int(m.group(1)) << int(m.group(2))


def test_adaptive_plan():
    """slices = 0: an adaptive OZAKI plan (plan info reports slice count 0),
    its workspace sized for the largest candidate, and a tolerance setter
    that only adaptive plans accept."""
    from muscle_gb300 import _lib

    a, b, c = desc(_lib.C64, [0, 1], [512, 700]), desc(_lib.C64, [1, 2], [700, 300]), desc(_lib.C64, [0, 2], [512, 300])
    st, info, _ = _plan(a, b, c, _lib.FORM_AUTO, 0)
    assert st == 0 and info.form == _lib.FORM_OZAKI and info.slices == 0
    assert info.workspace_bytes >= 8 * 512 * 1400 * 2 + 8 * 600 * 1400 * 2  # eight slices of A and B
    st, fixed, _ = _plan(a, b, c, _lib.FORM_OZAKI, 6)
    assert st == 0 and fixed.slices == 6 and fixed.workspace_bytes < info.workspace_bytes
    lib = _lib.load()
    da, ka = _lib.make_desc(*a)
    db, kb = _lib.make_desc(*b)
    dc, kc = _lib.make_desc(*c)
    for slices, ok in ((0, True), (6, False)):
        h = ctypes.c_void_p()
        assert lib.mgb_contraction_plan(ctypes.byref(h), ctypes.byref(da), ctypes.byref(db), ctypes.byref(dc),
                                        _lib.FORM_OZAKI, slices) == 0
        assert (lib.mgb_plan_set_tolerance(h, 1e-10) == 0) == ok
        if ok:
            assert lib.mgb_plan_set_tolerance(h, 0.0) == _lib.ERR_ARGUMENT
            assert lib.mgb_plan_set_tolerance(h, -1.0) == _lib.ERR_ARGUMENT
        lib.mgb_plan_destroy(h)
    # mixed element types need no workspace in the plain form
    st, info, _ = _plan(desc(_lib.F64, [0, 1], [40, 50]), desc(_lib.C64, [1, 2], [50, 30]),
                        desc(_lib.C64, [0, 2], [40, 30]), _lib.FORM_PLAIN, 0)
    assert st == 0 and info.workspace_bytes == 0 and info.permute_a == 0


def test_emulated_plans_put_the_long_side_on_the_tile_rows():
    """An emulated plan whose A has few rows and whose B has many columns
    computes C^T = B^T A^T (the tensor-core tile is 128 rows by 32 or 64
    embedded columns); plan info keeps the caller's view of M and N, and
    plain plans keep their orientation."""
    from muscle_gb300 import _lib

    lib = _lib.load()

    def swapped(dt, m, n, k, form, slices=0):
        a, b, c = desc(dt, [0, 1], [m, k]), desc(dt, [1, 2], [k, n]), desc(dt, [0, 2], [m, n])
        da, ka = _lib.make_desc(*a)
        db, kb = _lib.make_desc(*b)
        dc, kc = _lib.make_desc(*c)
        h = ctypes.c_void_p()
        assert lib.mgb_contraction_plan(ctypes.byref(h), ctypes.byref(da), ctypes.byref(db), ctypes.byref(dc),
                                        form, slices) == 0
        v, info = ctypes.c_int32(-1), _lib.PlanInfo()
        assert lib.mgb_plan_operands_swapped(h, ctypes.byref(v)) == 0
        assert lib.mgb_plan_info_get(h, ctypes.byref(info)) == 0
        assert (info.m, info.n, info.k) == (m, n, k)
        lib.mgb_plan_destroy(h)
        return v.value

    assert swapped(_lib.F64, 8, 500, 40, _lib.FORM_OZAKI, 6) == 1
    assert swapped(_lib.C64, 8, 500, 40, _lib.FORM_AUTO, 0) == 1
    assert swapped(_lib.C32, 20, 900, 64, _lib.FORM_BF16X3) == 1
    assert swapped(_lib.F64, 500, 8, 40, _lib.FORM_OZAKI, 6) == 0
    assert swapped(_lib.C64, 48, 48, 4096, _lib.FORM_AUTO, 0) == 0  # square: same tile count
    assert swapped(_lib.F64, 8, 500, 40, _lib.FORM_PLAIN) == 0
    v = ctypes.c_int32(0)
    assert lib.mgb_plan_operands_swapped(None, ctypes.byref(v)) == _lib.ERR_ARGUMENT
