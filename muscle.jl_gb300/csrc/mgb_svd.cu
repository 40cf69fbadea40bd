// Thin singular value decomposition on the device, for the factorisation step
// of simple_update (src/Operations/simple_update.jl:56-60), whose host path is
// LinearAlgebra.svd in tensor_svd_thin (src/Operations/tensor_svd.jl:98-125)
// and whose CUDA path is cuTensorNet (:34).
//
// One-sided Jacobi (Hestenes) rotations in one thread block: the columns of
// W (A, or A^H when A is wide, so that W has at least as many rows as
// columns) are rotated in pairs until every pair is orthogonal to within
// `tol` relative to their norms; V accumulates the rotations. Each sweep visits
// every pair once, in n - 1 rounds of disjoint pairs (the circle method), the
// pairs of a round spread over the warps. The singular values are the final
// column norms, with high relative accuracy. A second pass sorts them in
// descending order, normalises the columns into singular vectors, and
// completes the left vectors of exactly zero singular values to an
// orthonormal set (Gram-Schmidt on unit vectors). Sweeps are bounded
// (kMaxSweeps), so the kernel always ends; the sweep count is reported.
#include <algorithm>
#include <cmath>

#include "mgb_internal.h"

namespace mgb {

constexpr int kSvdThreads = 1024;
constexpr int kMaxSweeps = 60;
constexpr int64_t kSvdMaxCols = 1024;  // min(m, n)

__device__ __forceinline__ double sconj(double x) { return x; }
__device__ __forceinline__ double2 sconj(double2 x) { return make_double2(x.x, -x.y); }
__device__ __forceinline__ double abs2(double x) { return x * x; }
__device__ __forceinline__ double abs2(double2 x) { return x.x * x.x + x.y * x.y; }
__device__ __forceinline__ double smul(double a, double b) { return a * b; }
__device__ __forceinline__ double2 smul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double sadd(double a, double b) { return a + b; }
__device__ __forceinline__ double2 sadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double sscale(double a, double c) { return a * c; }
__device__ __forceinline__ double2 sscale(double2 a, double c) { return make_double2(a.x * c, a.y * c); }
__device__ __forceinline__ double zero_of(double) { return 0.0; }
__device__ __forceinline__ double2 zero_of(double2) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double one_of(double) { return 1.0; }
__device__ __forceinline__ double2 one_of(double2) { return make_double2(1.0, 0.0); }
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}
__device__ __forceinline__ double2 warp_sum(double2 v) { return make_double2(warp_sum(v.x), warp_sum(v.y)); }
__device__ __forceinline__ double phase_of(double g, double gabs) { return g / gabs; }
__device__ __forceinline__ double2 phase_of(double2 g, double gabs) { return make_double2(g.x / gabs, g.y / gabs); }
__device__ __forceinline__ double abs_of(double g) { return fabs(g); }
__device__ __forceinline__ double abs_of(double2 g) { return hypot(g.x, g.y); }

// Position `i` of round `r` in the circle method over nn (even) players:
// player 0 stays, the others rotate.
__device__ __forceinline__ int circle(int i, int r, int nn) { return i == 0 ? 0 : (i - 1 + r) % (nn - 1) + 1; }

// W: M x N (column-major, M >= N), V: N x N. info[0] = sweeps used.
// A round has three phases: the warps compute the inner products of their
// pairs; one thread per pair computes its rotation (the scalar square roots
// and divisions run once per pair, not once per lane: on a GPU whose FP64
// pipe retires under two operations per clock per SM they cost more than
// the vector work of small matrices); the warps apply the rotations.
template <typename T>
__global__ void __launch_bounds__(kSvdThreads) k_svd_jacobi(T *__restrict__ W, int M, int N, T *__restrict__ V,
                                                            double tol, int32_t *info) {
    constexpr int kPairs = kSvdMaxCols / 2;
    __shared__ int rotated;
    __shared__ double pa[kPairs], pb[kPairs], pc[kPairs];
    __shared__ T pg[kPairs], pse[kPairs], psec[kPairs];
    __shared__ unsigned char pdo[kPairs];
    const int nn = N + (N & 1);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
    for (int64_t i = threadIdx.x; i < (int64_t)N * N; i += blockDim.x)
        V[i] = (i % (N + 1) == 0) ? one_of(T()) : zero_of(T());
    auto pair = [&](int pi, int r, int &p, int &q) {
        p = circle(pi, r, nn);
        q = circle(nn - 1 - pi, r, nn);
        if (p > q) {
            const int t = p;
            p = q;
            q = t;
        }
    };
    int sweep = 0;
    for (; sweep < kMaxSweeps; ++sweep) {
        __syncthreads();  // every thread has read the previous sweep's flag
        if (threadIdx.x == 0) rotated = 0;
        __syncthreads();
        for (int r = 0; r + 1 < nn; ++r) {
            // inner products of the round's pairs
            for (int pi = warp; pi < nn / 2; pi += nw) {
                int p, q;
                pair(pi, r, p, q);
                if (q >= N) {  // the padding player of an odd N
                    if (lane == 0) pg[pi] = zero_of(T());
                    continue;
                }
                const T *wp = W + (int64_t)p * M, *wq = W + (int64_t)q * M;
                double a = 0.0, b = 0.0;
                T g = zero_of(T());
                for (int i = lane; i < M; i += 32) {
                    const T x = wp[i], y = wq[i];
                    a += abs2(x);
                    b += abs2(y);
                    g = sadd(g, smul(sconj(x), y));
                }
                a = warp_sum(a);
                b = warp_sum(b);
                g = warp_sum(g);
                if (lane == 0) {
                    pa[pi] = a;
                    pb[pi] = b;
                    pg[pi] = g;
                }
            }
            __syncthreads();
            // rotations, one thread per pair
            for (int pi = threadIdx.x; pi < nn / 2; pi += blockDim.x) {
                const double a = pa[pi], b = pb[pi];
                const T g = pg[pi];
                const double gabs = abs_of(g);
                if (!(gabs > tol * sqrt(a * b)) || gabs == 0.0) {  // orthogonal (or the padding pair)
                    pdo[pi] = 0;
                    continue;
                }
                // [w_p, w_q] <- [w_p, w_q] J, J = [[c, s e], [-s conj(e), c]], e = g / |g|:
                // makes w_p^H w_q vanish (c, s from the smaller root of t^2 + 2 zeta t - 1)
                const double zeta = (b - a) / (2.0 * gabs);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
                const T e = phase_of(g, gabs);
                pc[pi] = c;
                pse[pi] = sscale(e, s);
                psec[pi] = sscale(sconj(e), -s);
                pdo[pi] = 1;
                rotated = 1;
            }
            __syncthreads();
            // apply them to the columns of W and V
            for (int pi = warp; pi < nn / 2; pi += nw) {
                if (!pdo[pi]) continue;
                int p, q;
                pair(pi, r, p, q);
                const double c = pc[pi];
                const T se = pse[pi], sec = psec[pi];
                T *wp = W + (int64_t)p * M, *wq = W + (int64_t)q * M;
                for (int i = lane; i < M; i += 32) {
                    const T x = wp[i], y = wq[i];
                    wp[i] = sadd(sscale(x, c), smul(sec, y));
                    wq[i] = sadd(smul(se, x), sscale(y, c));
                }
                T *vp = V + (int64_t)p * N, *vq = V + (int64_t)q * N;
                for (int i = lane; i < N; i += 32) {
                    const T x = vp[i], y = vq[i];
                    vp[i] = sadd(sscale(x, c), smul(sec, y));
                    vq[i] = sadd(smul(se, x), sscale(y, c));
                }
            }
            __syncthreads();
        }
        if (!rotated) break;  // read by every thread after the round's barrier
    }
    if (threadIdx.x == 0) info[0] = sweep;
}

// Sorting, normalisation and output. uw: the normalised columns of W (left
// vectors of W), vw: the columns of V. For a wide A (trans) the roles swap:
// A = W^H = V S Uw^H. Writes the first `keep` triplets; flags as mgb_svd.
template <typename T>
__global__ void __launch_bounds__(kSvdThreads) k_svd_finish(T *__restrict__ W, int M, int N, const T *__restrict__ V,
                                                            int trans, int keep, int flags, T *__restrict__ U_out,
                                                            double *__restrict__ s_out, T *__restrict__ V_out) {
    __shared__ double sv[kSvdMaxCols];
    __shared__ int rank[kSvdMaxCols];
    __shared__ int col_of_rank[kSvdMaxCols];
    __shared__ double norm2;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
    for (int j = warp; j < N; j += nw) {
        double a = 0.0;
        for (int i = lane; i < M; i += 32) a += abs2(W[(int64_t)j * M + i]);
        a = warp_sum(a);
        if (lane == 0) sv[j] = sqrt(a);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) {  // descending, ties by column
        int rk = 0;
        for (int k = 0; k < N; ++k) rk += (sv[k] > sv[j] || (sv[k] == sv[j] && k < j)) ? 1 : 0;
        rank[j] = rk;
        col_of_rank[rk] = j;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s2 = 0.0;
        for (int r = 0; r < keep; ++r) s2 += sv[col_of_rank[r]] * sv[col_of_rank[r]];
        norm2 = s2;
    }
    // normalise the columns of W with a nonzero norm
    for (int j = warp; j < N; j += nw) {
        const double sj = sv[j];
        if (sj > 0.0)
            for (int i = lane; i < M; i += 32) W[(int64_t)j * M + i] = sscale(W[(int64_t)j * M + i], 1.0 / sj);
    }
    __syncthreads();
    // complete the left vectors of zero singular values (they come last):
    // Gram-Schmidt of unit vectors against the columns before them, by warp 0
    if (warp == 0) {
        for (int r = 0; r < N; ++r) {
            const int j = col_of_rank[r];
            if (sv[j] > 0.0) continue;
            T *wj = W + (int64_t)j * M;
            for (int cand = 0; cand < M; ++cand) {
                for (int i = lane; i < M; i += 32) wj[i] = (i == cand) ? one_of(T()) : zero_of(T());
                __syncwarp();
                for (int pass = 0; pass < 2; ++pass)
                    for (int rr = 0; rr < r; ++rr) {
                        const T *u = W + (int64_t)col_of_rank[rr] * M;
                        T d = zero_of(T());
                        for (int i = lane; i < M; i += 32) d = sadd(d, smul(sconj(u[i]), wj[i]));
                        d = warp_sum(d);
                        __syncwarp();
                        for (int i = lane; i < M; i += 32) wj[i] = sadd(wj[i], sscale(smul(u[i], d), -1.0));
                        __syncwarp();
                    }
                double a = 0.0;
                for (int i = lane; i < M; i += 32) a += abs2(wj[i]);
                a = warp_sum(a);
                if (a > 0.25) {
                    for (int i = lane; i < M; i += 32) wj[i] = sscale(wj[i], 1.0 / sqrt(a));
                    __syncwarp();
                    break;
                }
            }
        }
    }
    __syncthreads();
    // outputs: rank r of `keep`; U_out is (rows of A) x keep, V_out (columns of A) x keep
    const int mA = trans ? N : M, nA = trans ? M : N;
    const double scale = (flags & MGB_SVD_NORMALIZE) && norm2 > 0.0 ? 1.0 / sqrt(norm2) : 1.0;
    for (int r = warp; r < keep; r += nw) {
        const int j = col_of_rank[r];
        const T *uw = W + (int64_t)j * M;  // length M
        const T *vw = V + (int64_t)j * N;  // length N
        const T *ucol = trans ? vw : uw, *vcol = trans ? uw : vw;
        for (int i = lane; i < mA; i += 32) U_out[(int64_t)r * mA + i] = ucol[i];
        for (int i = lane; i < nA; i += 32) {
            const T v = vcol[i];
            V_out[(int64_t)r * nA + i] = (flags & MGB_SVD_CONJ_V) ? sconj(v) : v;
        }
        if (lane == 0) {
            double sj = sv[j] * scale;
            s_out[r] = (flags & MGB_SVD_SQRT_S) ? sqrt(sj) : sj;
        }
    }
}

// W = A (M >= N) or A^H, from A with leading dimension lda
template <typename T>
__global__ void k_svd_load(const T *__restrict__ A, int64_t lda, int m, int n, int trans, T *__restrict__ W) {
    const int M = trans ? n : m, N = trans ? m : n;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)M * N;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % M, j = idx / M;
        W[idx] = trans ? sconj(A[i * lda + j]) : A[j * lda + i];
    }
}

static uint64_t svd_ws(int dtype, int64_t m, int64_t n) {
    const int64_t M = std::max(m, n), N = std::min(m, n);
    const uint64_t eb = dtype == MGB_C64 ? 16 : 8;
    return 256 + ((M * N * eb + 255) & ~uint64_t(255)) + N * N * eb;
}

}  // namespace mgb

using namespace mgb;

extern "C" int mgb_svd_workspace_size(int32_t dtype, int64_t m, int64_t n, uint64_t *bytes) {
    if (!bytes || (dtype != MGB_F64 && dtype != MGB_C64) || m < 0 || n < 0)
        return fail(MGB_ERR_ARGUMENT, "svd: Float64 or ComplexF64, nonnegative sizes");
    *bytes = svd_ws(dtype, m, n);
    return MGB_OK;
}

extern "C" int mgb_svd(int32_t dtype, int64_t m, int64_t n, const void *A, int64_t lda, void *U, void *s, void *V,
                       int32_t keep, int32_t flags, void *workspace, uint64_t workspace_bytes, void *stream) {
    if ((dtype != MGB_F64 && dtype != MGB_C64) || m < 0 || n < 0 || lda < std::max<int64_t>(m, 1))
        return fail(MGB_ERR_ARGUMENT, "svd: Float64 or ComplexF64, nonnegative sizes, lda >= m");
    const int64_t M = std::max(m, n), N = std::min(m, n);
    if (N == 0) return MGB_OK;
    if (N > kSvdMaxCols || M * N > (int64_t)1 << 28)
        return fail(MGB_ERR_UNSUPPORTED, "svd: min(m, n) above 1024 or m n above 2^28 (one thread block)");
    if (keep <= 0 || keep > N) keep = (int32_t)N;
    if (flags & ~(MGB_SVD_NORMALIZE | MGB_SVD_CONJ_V | MGB_SVD_SQRT_S))
        return fail(MGB_ERR_ARGUMENT, "svd: unknown flags");
    if (!A || !U || !s || !V) return fail(MGB_ERR_ARGUMENT, "svd: null pointer");
    if (!workspace || workspace_bytes < svd_ws(dtype, m, n))
        return fail(MGB_ERR_WORKSPACE, "svd: workspace smaller than mgb_svd_workspace_size");
    if (((uintptr_t)workspace & 255) != 0) return fail(MGB_ERR_WORKSPACE, "svd: workspace must be 256-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    const int trans = m < n ? 1 : 0;
    const uint64_t eb = dtype == MGB_C64 ? 16 : 8;
    uint8_t *w = (uint8_t *)workspace;
    int32_t *info = (int32_t *)w;
    void *W = w + 256;
    void *Vw = w + 256 + ((M * N * eb + 255) & ~uint64_t(255));
    // relative orthogonality at which a pair is left alone
    const double tol = 4.0 * 1.1102230246251565e-16 * std::sqrt((double)M);
    const unsigned lb = (unsigned)std::min<int64_t>((M * N + 255) / 256, 152 * 8);
    if (dtype == MGB_C64) {
        k_svd_load<double2><<<lb, 256, 0, st>>>((const double2 *)A, lda, (int)m, (int)n, trans, (double2 *)W);
        k_svd_jacobi<double2><<<1, kSvdThreads, 0, st>>>((double2 *)W, (int)M, (int)N, (double2 *)Vw, tol, info);
        k_svd_finish<double2><<<1, kSvdThreads, 0, st>>>((double2 *)W, (int)M, (int)N, (const double2 *)Vw, trans, keep,
                                                        flags, (double2 *)U, (double *)s, (double2 *)V);
    } else {
        k_svd_load<double><<<lb, 256, 0, st>>>((const double *)A, lda, (int)m, (int)n, trans, (double *)W);
        k_svd_jacobi<double><<<1, kSvdThreads, 0, st>>>((double *)W, (int)M, (int)N, (double *)Vw, tol, info);
        k_svd_finish<double><<<1, kSvdThreads, 0, st>>>((double *)W, (int)M, (int)N, (const double *)Vw, trans, keep,
                                                       flags, (double *)U, (double *)s, (double *)V);
    }
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}
