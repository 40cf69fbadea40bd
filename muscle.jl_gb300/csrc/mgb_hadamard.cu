// Hadamard (broadcast element-wise) product C = A .* B on device arrays
// (hadamard / hadamard! of src/Operations/hadamard.jl:34-77).
//
// The labels of A (which C shares) are folded into one ModeGroup with the
// strides of A, B (0 along the labels B lacks: the broadcast) and C; mode 0
// is C's fastest. HBM-bound: algorithmic bytes = numel(C) * (sizeof A +
// sizeof C) + numel(B) * sizeof B.
//  * row kernel  — C's fastest mode is long (>= 64): one block walks rows of
//                  it, so loads and stores of A and C are coalesced (with four
//                  loads in flight per thread when all types agree);
//  * flat kernel — every element decodes its own offsets.
// Element types: the product is formed in T = promote(A, B) (float, double,
// float2 or double2) from operands of any narrower type, and stored in C's.
#include <algorithm>

#include "mgb_internal.h"

namespace mgb {

template <typename T>
struct HVal;
template <>
struct HVal<float> {
    __device__ static float mul(float a, float b) { return a * b; }
};
template <>
struct HVal<double> {
    __device__ static double mul(double a, double b) { return a * b; }
};
template <>
struct HVal<float2> {
    __device__ static float2 mul(float2 a, float2 b) {
        return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    }
};
template <>
struct HVal<double2> {
    __device__ static double2 mul(double2 a, double2 b) {
        return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    }
};

// element `i` of an array of element type `dt`, widened to T
template <typename T>
__device__ __forceinline__ T hload(const void *p, int dt, int64_t i);
template <>
__device__ __forceinline__ float hload<float>(const void *p, int, int64_t i) {
    return __ldg((const float *)p + i);
}
template <>
__device__ __forceinline__ double hload<double>(const void *p, int dt, int64_t i) {
    return dt == MGB_F32 ? (double)__ldg((const float *)p + i) : __ldg((const double *)p + i);
}
template <>
__device__ __forceinline__ float2 hload<float2>(const void *p, int dt, int64_t i) {
    return dt == MGB_F32 ? make_float2(__ldg((const float *)p + i), 0.f) : __ldg((const float2 *)p + i);
}
template <>
__device__ __forceinline__ double2 hload<double2>(const void *p, int dt, int64_t i) {
    switch (dt) {
    case MGB_F32: return make_double2((double)__ldg((const float *)p + i), 0.0);
    case MGB_F64: return make_double2(__ldg((const double *)p + i), 0.0);
    case MGB_C32: {
        float2 v = __ldg((const float2 *)p + i);
        return make_double2((double)v.x, (double)v.y);
    }
    default: return __ldg((const double2 *)p + i);
    }
}

// store v (type T) into an array of element type `dt` (narrowing allowed,
// complex into real never requested)
template <typename T>
__device__ __forceinline__ void hstore(void *p, int dt, int64_t i, T v);
template <>
__device__ __forceinline__ void hstore<float>(void *p, int dt, int64_t i, float v) {
    switch (dt) {
    case MGB_F32: ((float *)p)[i] = v; break;
    case MGB_F64: ((double *)p)[i] = (double)v; break;
    case MGB_C32: ((float2 *)p)[i] = make_float2(v, 0.f); break;
    default: ((double2 *)p)[i] = make_double2((double)v, 0.0); break;
    }
}
template <>
__device__ __forceinline__ void hstore<double>(void *p, int dt, int64_t i, double v) {
    switch (dt) {
    case MGB_F32: ((float *)p)[i] = (float)v; break;
    case MGB_F64: ((double *)p)[i] = v; break;
    case MGB_C32: ((float2 *)p)[i] = make_float2((float)v, 0.f); break;
    default: ((double2 *)p)[i] = make_double2(v, 0.0); break;
    }
}
template <>
__device__ __forceinline__ void hstore<float2>(void *p, int dt, int64_t i, float2 v) {
    if (dt == MGB_C32) ((float2 *)p)[i] = v;
    else ((double2 *)p)[i] = make_double2((double)v.x, (double)v.y);
}
template <>
__device__ __forceinline__ void hstore<double2>(void *p, int dt, int64_t i, double2 v) {
    if (dt == MGB_C64) ((double2 *)p)[i] = v;
    else ((float2 *)p)[i] = make_float2((float)v.x, (float)v.y);
}

template <typename T>
struct HDtype;
template <>
struct HDtype<float> {
    static constexpr int code = MGB_F32;
};
template <>
struct HDtype<double> {
    static constexpr int code = MGB_F64;
};
template <>
struct HDtype<float2> {
    static constexpr int code = MGB_C32;
};
template <>
struct HDtype<double2> {
    static constexpr int code = MGB_C64;
};

struct HArgs {
    const void *A, *B;
    void *C;
    int ta, tb, tc;  // element types
};

// rows of mode 0; the other modes enumerate the rows
template <typename T>
__global__ void __launch_bounds__(256) k_hadamard_rows(HArgs a, ModeGroup outer, int64_t len, int64_t sa,
                                                       int64_t sb, int64_t sc, int64_t rows) {
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const int64_t oa = group_offset(outer, 0, r), ob = group_offset(outer, 1, r),
                      oc = group_offset(outer, 2, r);
        for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
            T x = hload<T>(a.A, a.ta, oa + i * sa);
            T y = hload<T>(a.B, a.tb, ob + i * sb);
            hstore<T>(a.C, a.tc, oc + i * sc, HVal<T>::mul(x, y));
        }
    }
}

// Same element type everywhere and A, C unit-stride along the row: four
// independent loads in flight per thread, and a broadcast B (stride 0 along
// the row) read once per row.
// Work items are (row, chunk of HCHUNK elements) so that the grid balances
// even when the rows are few and long.
constexpr int64_t HCHUNK = 4096;

template <typename T>
__global__ void __launch_bounds__(256) k_hadamard_rows_same(const T *__restrict__ A, const T *__restrict__ B,
                                                            T *__restrict__ C, ModeGroup outer, int64_t len,
                                                            int64_t sb, int64_t rows) {
    constexpr int U = 4;  // measured: 8 in flight per thread was slower for 8-byte types
    const int64_t chunks = (len + HCHUNK - 1) / HCHUNK;
    for (int64_t w = blockIdx.x; w < rows * chunks; w += gridDim.x) {
        const int64_t r = w / chunks, lo = (w - r * chunks) * HCHUNK, hi = min(len, lo + HCHUNK);
        const T *a = A + group_offset(outer, 0, r);
        const T *b = B + group_offset(outer, 1, r);
        T *c = C + group_offset(outer, 2, r);
        const T y0 = __ldg(b);
        for (int64_t i0 = lo + threadIdx.x; i0 < hi; i0 += (int64_t)U * blockDim.x) {
            T x[U], y[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t i = i0 + (int64_t)u * blockDim.x;
                if (i < hi) {
                    x[u] = __ldg(a + i);
                    y[u] = sb == 0 ? y0 : __ldg(b + i * sb);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t i = i0 + (int64_t)u * blockDim.x;
                if (i < hi) c[i] = HVal<T>::mul(x[u], y[u]);
            }
        }
    }
}

// The same with 16-byte vectors (V elements each) when every row of A and C
// (and of B, unless it is broadcast along the row) starts on a 16-byte
// boundary: a quarter (4-byte types) or half (8-byte types) of the memory
// instructions, each moving a full 16 bytes.
template <typename T, int V>
__global__ void __launch_bounds__(256, 4) k_hadamard_rows_vec(const T *__restrict__ A, const T *__restrict__ B,
                                                           T *__restrict__ C, ModeGroup outer, int64_t len,
                                                           int64_t sb, int64_t rows) {
    constexpr int U = 4;
    static_assert(sizeof(T) * V == 16, "16-byte vectors");
    struct alignas(16) Vec {
        T v[V];
    };
    const int64_t chunks = (len + HCHUNK - 1) / HCHUNK;
    for (int64_t w = blockIdx.x; w < rows * chunks; w += gridDim.x) {
        const int64_t r = w / chunks, lo = (w - r * chunks) * HCHUNK, hi = min(len, lo + HCHUNK);
        const T *a = A + group_offset(outer, 0, r) + lo;
        const T *b = B + group_offset(outer, 1, r);
        T *c = C + group_offset(outer, 2, r) + lo;
        const T y0 = __ldg(b);
        const int64_t nv = (hi - lo) / V;  // whole vectors of this chunk (lo is a multiple of V)
        const Vec *av = reinterpret_cast<const Vec *>(a);
        const Vec *bv = reinterpret_cast<const Vec *>(b + lo);
        Vec *cv = reinterpret_cast<Vec *>(c);
        for (int64_t i0 = threadIdx.x; i0 < nv; i0 += (int64_t)U * blockDim.x) {
            Vec x[U], y[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t i = i0 + (int64_t)u * blockDim.x;
                if (i < nv) {
                    x[u] = av[i];
                    if (sb != 0) y[u] = bv[i];
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t i = i0 + (int64_t)u * blockDim.x;
                if (i < nv) {
                    Vec z;
#pragma unroll
                    for (int e = 0; e < V; ++e) z.v[e] = HVal<T>::mul(x[u].v[e], sb != 0 ? y[u].v[e] : y0);
                    cv[i] = z;
                }
            }
        }
        for (int64_t i = nv * V + threadIdx.x; i < hi - lo; i += blockDim.x)
            c[i] = HVal<T>::mul(__ldg(a + i), sb != 0 ? __ldg(b + lo + i) : y0);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_hadamard_flat(HArgs a, ModeGroup g, int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        T x = hload<T>(a.A, a.ta, group_offset(g, 0, i));
        T y = hload<T>(a.B, a.tb, group_offset(g, 1, i));
        hstore<T>(a.C, a.tc, group_offset(g, 2, i), HVal<T>::mul(x, y));
    }
}

template <typename T>
static int run_hadamard(const ModeGroup &g, const HArgs &a, cudaStream_t s) {
    const int64_t total = g.size();
    if (total == 0) return MGB_OK;
    const int64_t cap = 152 * 16;  // resident blocks of 256 threads on 152 SMs, x 2
    if (g.n > 0 && g.ext[0] >= 64 && g.str[2][0] == 1) {
        ModeGroup outer;
        outer.n = g.n - 1;
        for (int i = 1; i < g.n; ++i) {
            outer.ext[i - 1] = g.ext[i];
            for (int t = 0; t < 3; ++t) outer.str[t][i - 1] = g.str[t][i];
        }
        const int64_t rows = outer.size();
        const int dt = HDtype<T>::code;
        const int64_t items = rows * ((g.ext[0] + HCHUNK - 1) / HCHUNK);
        const bool same = a.ta == dt && a.tb == dt && a.tc == dt && g.str[0][0] == 1;
        // 16-byte vectors: every row of A and C (and of B unless broadcast)
        // starts on a 16-byte boundary
        bool vec = same && sizeof(T) < 16 && (g.str[1][0] == 0 || g.str[1][0] == 1);
        if (vec) {
            auto al = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
            vec = al(a.A) && al(a.C) && (g.str[1][0] == 0 || al(a.B));
            for (int i = 0; i < outer.n && vec; ++i)
                vec = (outer.str[0][i] * (int64_t)sizeof(T)) % 16 == 0 && (outer.str[2][i] * (int64_t)sizeof(T)) % 16 == 0 &&
                      (g.str[1][0] == 0 || (outer.str[1][i] * (int64_t)sizeof(T)) % 16 == 0);
        }
        const unsigned grid = (unsigned)std::min(items, cap * 4);
        if (vec)
            k_hadamard_rows_vec<T, 16 / sizeof(T)><<<grid, 256, 0, s>>>((const T *)a.A, (const T *)a.B, (T *)a.C, outer,
                                                                        g.ext[0], g.str[1][0], rows);
        else if (same)
            k_hadamard_rows_same<T><<<grid, 256, 0, s>>>((const T *)a.A, (const T *)a.B, (T *)a.C, outer, g.ext[0],
                                                        g.str[1][0], rows);
        else
            k_hadamard_rows<T><<<(unsigned)std::min(rows, cap * 4), 256, 0, s>>>(a, outer, g.ext[0], g.str[0][0],
                                                                               g.str[1][0], g.str[2][0], rows);
    } else {
        k_hadamard_flat<T><<<(unsigned)std::min((total + 255) / 256, cap), 256, 0, s>>>(a, g, total);
    }
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

int launch_hadamard(const ModeGroup &g, int ta, int tb, int tc, const void *A, const void *B, void *C,
                    cudaStream_t s) {
    HArgs a{A, B, C, ta, tb, tc};
    switch (promote(ta, tb)) {
    case MGB_F32: return run_hadamard<float>(g, a, s);
    case MGB_F64: return run_hadamard<double>(g, a, s);
    case MGB_C32: return run_hadamard<float2>(g, a, s);
    default: return run_hadamard<double2>(g, a, s);
    }
}

}  // namespace mgb

using namespace mgb;

extern "C" int mgb_hadamard(const mgb_tensor_desc *a, const mgb_tensor_desc *b, const mgb_tensor_desc *c,
                            const void *A, const void *B, void *C, void *stream) {
    Desc da, db, dc;
    int st;
    if ((st = read_desc(a, da, "A")) || (st = read_desc(b, db, "B")) || (st = read_desc(c, dc, "C"))) return st;
    if (has_repeats(da) || has_repeats(db)) return fail(MGB_ERR_ARGUMENT, "hadamard: repeated labels");
    if (dc.rank != da.rank) return fail(MGB_ERR_ARGUMENT, "hadamard: C must carry the labels of A");
    for (int i = 0; i < da.rank; ++i) {
        if (dc.modes[i] != da.modes[i]) return fail(MGB_ERR_ARGUMENT, "hadamard: C must carry the labels of A in order");
        if (dc.ext[i] != da.ext[i]) return fail(MGB_ERR_DIMENSION_MISMATCH, "hadamard: C and A differ in size");
    }
    std::vector<ModeRec> modes;
    for (int i = 0; i < da.rank; ++i) {
        ModeRec r;
        r.label = da.modes[i];
        r.ext = da.ext[i];
        r.str[0] = da.str[i];
        r.str[2] = dc.str[i];
        const int j = find_mode(db, da.modes[i]);
        if (j >= 0 && db.ext[j] != da.ext[i]) return fail(MGB_ERR_DIMENSION_MISMATCH, "hadamard: B and A differ in size");
        r.str[1] = j >= 0 ? db.str[j] : 0;
        modes.push_back(r);
    }
    for (int i = 0; i < db.rank; ++i)
        if (find_mode(da, db.modes[i]) < 0) return fail(MGB_ERR_ARGUMENT, "hadamard: labels of B must be a subset of A's");
    if (is_complex(promote(da.dtype, db.dtype)) && !is_complex(dc.dtype))
        return fail(MGB_ERR_ARGUMENT, "hadamard: a complex product cannot be stored in a real array");
    const bool present[3] = {true, true, true};
    ModeGroup g = fold_group(modes, present, 2);
    if (g.size() == 0) return MGB_OK;
    if (!A || !B || !C) return fail(MGB_ERR_ARGUMENT, "null operand pointer");
    return launch_hadamard(g, da.dtype, db.dtype, dc.dtype, A, B, C, (cudaStream_t)stream);
}
