"""Writes kat_cases.json: the known-answer assertions of Muscle.jl's own tests
for binary_einsum / unary_einsum / permutedims / hadamard, restated as data.

Every case records where its assertion lives in the Muscle.jl test suite.
Inputs in those tests are `ones`/`fill` arrays, so expected results are exact
constants ("fill"), explicit permutations of the input ("permute"), or the
test's own reference formula ("formula"). `expect_base` is the host backend's
behaviour (test/unit/...), `expect_gpu` the CUDA backend's
(test/integration/cuda.jl, omeinsum.jl).

Run: python tests/golden/make_kat.py  (no dependencies beyond the stdlib).
"""
import json
import os

U = "test/unit/operations/binary_einsum.jl"
G = "test/integration/cuda.jl"
O = "test/integration/omeinsum.jl"


def arr(shape, inds, fill=1.0, dtype="float64"):
    return {"shape": shape, "inds": inds, "fill": fill, "dtype": dtype}


def res(inds, shape, fill):
    return {"inds": inds, "shape": shape, "fill": fill}


cases = []


def add(name, ref, a, b, expect_base, expect_gpu=None, dims=None, out=None):
    cases.append({"kind": "binary", "name": name, "ref": ref, "a": a, "b": b, "dims": dims, "out": out,
                  "expect_base": expect_base, "expect_gpu": expect_gpu if expect_gpu is not None else expect_base})


A, B = arr([2, 3], ["i", "j"]), arr([3, 4], ["j", "k"])
add("matmul default", f"{U}:4-11", A, B, res(["i", "k"], [2, 4], 3.0))
add("matmul out", f"{U}:13-17", A, B, res(["i", "k"], [2, 4], 3.0), out=["i", "k"])
add("matmul out permuted", f"{U}:19-23", A, B, res(["k", "i"], [4, 2], 3.0), out=["k", "i"])
add("matmul dims", f"{U}:25-29", A, B, res(["i", "k"], [2, 4], 3.0), dims=["j"])
# GPU matmul with CUDA.ones: Float32 must be exact too (test/integration/cuda.jl:8-33)
A32, B32 = arr([2, 3], ["i", "j"], 1.0, "float32"), arr([3, 4], ["j", "k"], 1.0, "float32")
add("matmul float32", f"{G}:8-14", A32, B32, res(["i", "k"], [2, 4], 3.0))
add("matmul float32 out permuted", f"{G}:22-26", A32, B32, res(["k", "i"], [4, 2], 3.0), out=["k", "i"])

A, B = arr([3, 4], ["i", "j"]), arr([4, 3], ["j", "i"])
add("inner default", f"{U}:32-39", A, B, res([], [], 12.0))
add("inner out", f"{U}:41-45", A, B, res([], [], 12.0), out=[])
add("inner dims", f"{U}:47-51", A, B, res([], [], 12.0), dims=["i", "j"])
add("inner dims permuted", f"{U}:53-57", A, B, res([], [], 12.0), dims=["j", "i"])

A, B = arr([2, 3], ["i", "j"]), arr([4, 5], ["k", "l"])
add("outer default", f"{U}:60-67", A, B, res(["i", "j", "k", "l"], [2, 3, 4, 5], 1.0))
for out, shape, lines in ((["i", "j", "k", "l"], [2, 3, 4, 5], "69-72"), (["k", "l", "i", "j"], [4, 5, 2, 3], "74-78"),
                          (["l", "k", "j", "i"], [5, 4, 3, 2], "79-82"), (["l", "i", "k", "j"], [5, 2, 4, 3], "84-87"),
                          (["j", "i", "k", "l"], [3, 2, 4, 5], "89-92")):
    add("outer out " + "".join(out), f"{U}:{lines}", A, B, res(out, shape, 1.0), out=out)

A, alpha = arr([2, 3], ["i", "j"]), arr([], [], 2.0)
add("scale right", f"{U}:96-104", A, alpha, res(["i", "j"], [2, 3], 2.0))
add("scale left", f"{U}:106-109", alpha, A, res(["i", "j"], [2, 3], 2.0))
add("scale right transposed", f"{U}:111-114", A, alpha, res(["j", "i"], [3, 2], 2.0), out=["j", "i"])
add("scale left transposed", f"{U}:116-119", alpha, A, res(["j", "i"], [3, 2], 2.0), out=["j", "i"])
# mixed ComplexF64 x Float64 promotion (test/integration/cuda.jl:100-123, src/Muscle.jl:47-55)
Ac = arr([2, 3], ["i", "j"], [1.0, 0.0], "complex128")
add("scale complex x real", f"{G}:100-108", Ac, alpha, res(["i", "j"], [2, 3], [2.0, 0.0]))
add("scale real x complex transposed", f"{G}:120-123", alpha, Ac, res(["j", "i"], [3, 2], [2.0, 0.0]), out=["j", "i"])
for ta, tb in (("float64", "complex128"), ("complex128", "float64")):
    fa = [1.0, 0.0] if ta == "complex128" else 1.0
    fb = [1.0, 0.0] if tb == "complex128" else 1.0
    add(f"precompile {ta} x {tb} rank2", "src/Muscle.jl:47-51", arr([2, 2], ["i", "j"], fa, ta),
        arr([2, 2], ["j", "k"], fb, tb), res(["i", "k"], [2, 2], [2.0, 0.0]))
    add(f"precompile {ta} x {tb} rank3", "src/Muscle.jl:53-55", arr([2, 2, 2], ["i", "j", "k"], fa, ta),
        arr([2, 2, 2], ["j", "k", "l"], fb, tb), res(["i", "l"], [2, 2], [4.0, 0.0]))

A, B = arr([2, 3, 6], ["i", "j", "batch"]), arr([3, 4, 6], ["j", "k", "batch"])
err = {"raises": "ArgumentError"}
add("batch out ikb", f"{U}:127 / {G}:130-133", A, B, err, res(["i", "k", "batch"], [2, 4, 6], 3.0), out=["i", "k", "batch"])
add("batch out kib", f"{U}:128 / {G}:135-138", A, B, err, res(["k", "i", "batch"], [4, 2, 6], 3.0), out=["k", "i", "batch"])
add("batch out bik", f"{U}:129 / {G}:140-143", A, B, err, res(["batch", "i", "k"], [6, 2, 4], 3.0), out=["batch", "i", "k"])
# dims=[j] keeps `batch` as a hyperindex; the CUDA test marks the [i,k,batch]
# order broken (test/integration/cuda.jl:147-150): the front-end order is [i,batch,k]
add("batch dims j", f"{U}:132 / {G}:146-150", A, B, err, res(["i", "batch", "k"], [2, 6, 4], 3.0), dims=["j"])

for t, f in (("float64", 1.0), ("complex128", [1.0, 0.0])):
    A, B = arr([2, 3, 4], ["i", "j", "k"], f, t), arr([4, 5, 3], ["k", "l", "j"], f, t)
    add(f"manual {t} dims jk", f"{U}:135-149 / {G}:158-168", A, B,
        {"inds": ["i", "l"], "shape": [2, 5], "formula": "reshape(A,2,12)*reshape(permutedims(B,[3,1,2]),12,5)"},
        dims=["j", "k"])
    add(f"manual {t} dims j", f"{U}:151-152 / {G}:170-180", A, B, err,
        {"inds": ["i", "k", "l"], "shape": [2, 4, 5], "formula": "C[i,k,l] += A[i,j,k]*B[k,l,j]"}, dims=["j"])


def uadd(name, ref, x, expect, dims=None, out=None, inplace=None):
    cases.append({"kind": "unary", "name": name, "ref": ref, "x": x, "dims": dims, "out": out,
                  "inplace": inplace, "expect": expect})


X = arr([2, 3, 4], ["i", "j", "k"])
uadd("axis sum dims", f"{O}:9-11", X, res(["j", "k"], [3, 4], 2.0), dims=["i"])
uadd("axis sum out", f"{O}:13-14", X, res(["j", "k"], [3, 4], 2.0), out=["j", "k"])
uadd("axis sum inplace", f"{O}:16-18", X, res(["j", "k"], [3, 4], 2.0), inplace=["j", "k"])
uadd("full sum dims", f"{O}:22-25", X, res([], [], 24.0), dims=["i", "j", "k"])
uadd("full sum out", f"{O}:27-29", X, res([], [], 24.0), out=[])
uadd("full sum inplace", f"{O}:31-33", X, res([], [], 24.0), inplace=[])
X = arr([2, 2], ["i", "i"])
uadd("diagonal ii->i", f"{O}:40-43", X, res(["i"], [2], 1.0), out=["i"])
uadd("diagonal ii->i inplace", f"{O}:45-47", X, res(["i"], [2], 1.0), inplace=["i"])
uadd("trace ii-> default", f"{O}:66-69", X, res([], [], 2.0))
uadd("trace ii-> dims", f"{O}:71-73", X, res([], [], 2.0), dims=["i"])
uadd("trace ii-> out", f"{O}:75-77", X, res([], [], 2.0), out=[])
uadd("trace ii-> inplace", f"{O}:79-81", X, res([], [], 2.0), inplace=[])
X = arr([2, 3, 2], ["i", "j", "i"])
uadd("diagonal iji->ij", f"{O}:51-54", X, res(["i", "j"], [2, 3], 1.0), out=["i", "j"])
uadd("diagonal iji->ij inplace", f"{O}:56-58", X, res(["i", "j"], [2, 3], 1.0), inplace=["i", "j"])
uadd("partial trace iji->j default", f"{O}:85-88", X, res(["j"], [3], 2.0))
uadd("partial trace iji->j dims", f"{O}:90-92", X, res(["j"], [3], 2.0), dims=["i"])
uadd("partial trace iji->j out", f"{O}:94-96", X, res(["j"], [3], 2.0), out=["j"])
uadd("partial trace iji->j inplace", f"{O}:98-100", X, res(["j"], [3], 2.0), inplace=["j"])

# permutedims by position and by labels on 1:24 reshaped (test/unit/tensor.jl:447-465)
cases.append({"kind": "permute", "name": "permutedims 1:24", "ref": "test/unit/tensor.jl:447-465",
              "x": {"shape": [2, 3, 4], "inds": ["i", "j", "k"], "iota": True, "dtype": "float64"},
              "perm": ["k", "i", "j"], "expect": {"inds": ["k", "i", "j"], "shape": [4, 2, 3]}})

# hadamard / hadamard! on ones(2, 3, 4) (test/unit/operations/hadamard.jl). "b_broadcast":
# the test asserts that every slice of c along b's labels equals b's entry there.
H = "test/unit/operations/hadamard.jl"
A = arr([2, 3, 4], ["i", "j", "k"])


def hadd(name, lines, b, expect):
    for inplace in (False, True):
        cases.append({"kind": "hadamard", "name": name + (" inplace" if inplace else ""), "ref": f"{H}:{lines}",
                      "a": A, "b": b, "inplace": inplace, "expect": expect})


hadd("tensor - scalar", "4-19", arr([], [], 2.0), res(["i", "j", "k"], [2, 3, 4], 2.0))
for lab, vals, lines in (("i", [1.0, 2.0], "24-40"), ("j", [1.0, 2.0, 3.0], "42-58"), ("k", [1.0, 2.0, 3.0, 4.0], "60-76")):
    hadd(f"tensor - vector {lab}", lines, {"shape": [len(vals)], "inds": [lab], "values": vals, "dtype": "float64"},
         {"inds": ["i", "j", "k"], "shape": [2, 3, 4], "formula": "b_broadcast"})
# Float64[1 2 3; 4 5 6] in column-major order
hadd("tensor - matrix bcast", "79-101", {"shape": [2, 3], "inds": ["i", "j"], "values": [1.0, 4.0, 2.0, 5.0, 3.0, 6.0],
                                         "dtype": "float64"},
     {"inds": ["i", "j", "k"], "shape": [2, 3, 4], "formula": "b_broadcast"})
hadd("tensor - tensor", "103-117", arr([2, 3, 4], ["i", "j", "k"], 2.0), res(["i", "j", "k"], [2, 3, 4], 2.0))

path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat_cases.json")
with open(path, "w") as f:
    json.dump({"source": "Muscle.jl v0.3.20 test suite", "cases": cases}, f, indent=1)
print(f"wrote {len(cases)} cases to {path}")
