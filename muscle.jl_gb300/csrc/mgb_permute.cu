// Index permutation (Base.permutedims via src/Tensor.jl:316-319) with optional
// widening element conversion (real -> complex, Float32 -> Float64).
//
// After folding, the copy is one of:
//  * row copy   — the fastest mode of Y is also unit-stride in X: contiguous
//                 rows, copied with 128-bit vectors when aligned;
//  * transpose  — X and Y have different unit-stride modes. Same-type 8- and
//                 16-byte elements whose strides TMA can address (at most
//                 three other modes, strides in multiples of 16 bytes) go
//                 through TMA-staged tiles (k_transpose_tma); the rest use
//                 register-staged shared-memory tiles with edges of 32 or 64
//                 elements (32 x 32 for 16-byte types), coalesced on both
//                 sides, other modes enumerated by the grid;
//  * gather     — strided views without a unit-stride mode: element-wise.
// HBM-bound: algorithmic bytes = numel * (sizeof(src) + sizeof(dst)).
#include <algorithm>
#include <cuComplex.h>
#include <type_traits>

#include "mgb_internal.h"
#include "mgb_ptx.h"

namespace mgb {

template <typename TS, typename TD>
struct Conv;
template <typename T>
struct Conv<T, T> {
    __device__ static T f(T v) { return v; }
};
template <>
struct Conv<float, double> {
    __device__ static double f(float v) { return (double)v; }
};
template <>
struct Conv<float, float2> {
    __device__ static float2 f(float v) { return make_float2(v, 0.f); }
};
template <>
struct Conv<float, double2> {
    __device__ static double2 f(float v) { return make_double2((double)v, 0.0); }
};
template <>
struct Conv<double, double2> {
    __device__ static double2 f(double v) { return make_double2(v, 0.0); }
};
template <>
struct Conv<float2, double2> {
    __device__ static double2 f(float2 v) { return make_double2((double)v.x, (double)v.y); }
};

struct PermGeom {
    ModeGroup g;    // folded modes, tensor 0 = X, 1 = Y; mode 0 = Y's fastest
    int a = -1;     // Y unit-stride mode (0) or -1
    int b = -1;     // X unit-stride mode or -1
};

// ---- row copy --------------------------------------------------------------
constexpr int kRowChunk = 4096;

template <typename TS, typename TD>
__global__ void k_rowcopy(const TS *__restrict__ x, TD *__restrict__ y, ModeGroup outer,
                          int64_t rowlen, int64_t chunks_per_row, int vec) {
    int64_t blk = blockIdx.x;
    int64_t row = blk / chunks_per_row;
    int64_t chunk = blk - row * chunks_per_row;
    const TS *xr = x + group_offset(outer, 0, row);
    TD *yr = y + group_offset(outer, 1, row);
    int64_t begin = chunk * kRowChunk;
    int64_t end = min(begin + (int64_t)kRowChunk, rowlen);
    if (vec) {
        // same type, 16-byte aligned rows: copy 16-byte vectors
        constexpr int per = 16 / sizeof(TD);
        const uint4 *xs = reinterpret_cast<const uint4 *>(xr + begin);
        uint4 *ys = reinterpret_cast<uint4 *>(yr + begin);
        int64_t nv = (end - begin) / per;
        for (int64_t i = threadIdx.x; i < nv; i += blockDim.x) ys[i] = __ldg(xs + i);
        for (int64_t i = begin + nv * per + threadIdx.x; i < end; i += blockDim.x)
            yr[i] = Conv<TS, TD>::f(xr[i]);
        return;
    }
    for (int64_t i = begin + threadIdx.x; i < end; i += blockDim.x) yr[i] = Conv<TS, TD>::f(xr[i]);
}

// ---- tiled transpose ------------------------------------------------------------
// TA x TB tiles: TA elements along a (Y's unit-stride mode) by TB along b
// (X's unit-stride mode); loads walk b and stores walk a, 32 consecutive
// elements per warp on both sides.
template <typename TS, typename TD, int TA, int TB>
__global__ void k_transpose(const TS *__restrict__ x, TD *__restrict__ y, ModeGroup outer,
                            int64_t ea, int64_t eb, int64_t sxa, int64_t syb, int64_t tiles_a,
                            int64_t tiles_b) {
    __shared__ TD tile[TA][TB + 1];
    int64_t blk = blockIdx.x;
    int64_t tb = blk % tiles_b;
    blk /= tiles_b;
    int64_t ta = blk % tiles_a;
    int64_t o = blk / tiles_a;
    const TS *xo = x + group_offset(outer, 0, o);
    TD *yo = y + group_offset(outer, 1, o);
    int64_t a0 = ta * TA, b0 = tb * TB;
    int tx = threadIdx.x % 32, ty = threadIdx.x / 32;  // 32 x 8
#pragma unroll
    for (int bb = 0; bb < TB; bb += 32) {
#pragma unroll
        for (int r = ty; r < TA; r += 8) {
            int64_t ia = a0 + r, ib = b0 + bb + tx;
            if (ia < ea && ib < eb) tile[r][bb + tx] = Conv<TS, TD>::f(__ldg(xo + ia * sxa + ib));
        }
    }
    __syncthreads();
#pragma unroll
    for (int aa = 0; aa < TA; aa += 32) {
#pragma unroll
        for (int r = ty; r < TB; r += 8) {
            int64_t ib = b0 + r, ia = a0 + aa + tx;
            if (ia < ea && ib < eb) yo[ia + ib * syb] = tile[aa + tx][r];
        }
    }
}

// Same-type 8-byte elements (Float64, ComplexF32) with 16-byte vectors on both
// sides: 64 x 64 tiles, each lane loads two consecutive elements of X's
// unit-stride mode and stores two consecutive elements of Y's, so every
// global access moves 16 bytes (scalar accesses only at ragged edges). Used
// when every tile row starts on a 16-byte boundary in X and in Y.
template <typename T>
__global__ void __launch_bounds__(256) k_transpose_v2(const T *__restrict__ x, T *__restrict__ y, ModeGroup outer,
                                                      int64_t ea, int64_t eb, int64_t sxa, int64_t syb,
                                                      int64_t tiles_a, int64_t tiles_b) {
    static_assert(sizeof(T) == 8, "8-byte elements");
    struct alignas(16) P2 {
        T v[2];
    };
    __shared__ T tile[64][65];
    int64_t blk = blockIdx.x;
    const int64_t tb = blk % tiles_b;
    blk /= tiles_b;
    const int64_t ta = blk % tiles_a;
    const int64_t o = blk / tiles_a;
    const T *xo = x + group_offset(outer, 0, o);
    T *yo = y + group_offset(outer, 1, o);
    const int64_t a0 = ta * 64, b0 = tb * 64;
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
    const int c = 2 * lane;  // this lane's pair within a tile row
#pragma unroll
    for (int r = w; r < 64; r += 8) {
        const int64_t ia = a0 + r, ib = b0 + c;
        if (ia >= ea) continue;
        const T *src = xo + ia * sxa + ib;
        if (ib + 1 < eb) {
            const P2 v = *reinterpret_cast<const P2 *>(src);
            tile[r][c] = v.v[0];
            tile[r][c + 1] = v.v[1];
        } else if (ib < eb) {
            tile[r][c] = __ldg(src);
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = w; r < 64; r += 8) {
        const int64_t ib = b0 + r, ia = a0 + c;
        if (ib >= eb) continue;
        T *dst = yo + ia + ib * syb;
        if (ia + 1 < ea) {
            P2 v;
            v.v[0] = tile[c][r];
            v.v[1] = tile[c + 1][r];
            *reinterpret_cast<P2 *>(dst) = v;
        } else if (ia < ea) {
            *dst = tile[c][r];
        }
    }
}

// ---- TMA-staged transpose (same-type 8- and 16-byte elements) -----------------
// A tile is 32 R rows of a (Y's unit-stride mode; R = 1..4, whichever pads
// a's extent least) by 128 bytes of b (X's unit-stride mode: 16 Float64 /
// ComplexF32 or 8 ComplexF64 elements). One 5-D TMA box per tile (b, a and
// up to three outer modes, X's own strides) lands in a ring of stages with
// the 128-byte swizzle: 16-byte chunk j of tile row r sits at
// r * 128 + ((j ^ (r % 8)) * 16), so the 8 lanes of a quarter warp, reading
// one chunk of 8 consecutive rows, hit 8 different bank groups.
// A persistent grid walks the tiles t = b, b + grid, ...; the producer
// thread steps the tile coordinates by the grid size in mixed radix (one
// add and compare per digit, no division), issues the load and publishes
// the tile's Y offset beside the stage. Four warps read each tile
// column-wise:
//  * 16-byte elements: lane l reads row l of a chunk (one element) and the
//    warp stores 32 consecutive elements of a Y column, 512 bytes;
//  * 8-byte elements: lane l reads row l of a chunk (elements b, b + 1);
//    lanes l and l ^ 1 swap one element by a shuffle, so that the even lane
//    holds column b and the odd lane column b + 1 for rows (l & ~1, l | 1),
//    and every lane stores one 16-byte pair of a Y column.
// Loads never wait for stores, so each SM keeps several tiles of reads in
// flight while it writes the previous ones. Rows past a's extent arrive
// zero-filled from the TMA box and are not stored.
static ModeGroup drop_mode(const ModeGroup &g, int a, int b);

constexpr int kTmaConsumers = 4;  // warps
constexpr int kTmaThreads = 32 * (kTmaConsumers + 1);

struct TmaPermArgs {
    int64_t ext[5];   // tiles along b, tiles along a, outer extents (1 past n)
    int64_t ystr[3];  // Y strides of the outer modes
    int64_t ea, eb, syb;
    int64_t tiles;
};
struct TmaTileInfo {
    int64_t yoff;  // Y offset (elements) of the tile's first row and column
    int32_t rows, cols;  // rows of a and columns of b inside the tensor
};

__host__ __device__ constexpr int tma_stages(int R) { return R == 1 ? 8 : R == 2 ? 4 : R == 3 ? 3 : 2; }
__host__ __device__ constexpr int tma_tile_bytes(int R) { return 32 * R * 128; }
__host__ __device__ constexpr int tma_smem_bytes(int R) {
    return tma_stages(R) * (tma_tile_bytes(R) + (int)sizeof(TmaTileInfo) + 16) + 1024 /*align*/ + 16;
}

template <int ES, int R>
__global__ void __launch_bounds__(kTmaThreads) k_transpose_tma(const __grid_constant__ CUtensorMap tm,
                                                               unsigned char *__restrict__ y, const TmaPermArgs p,
                                                               int32_t *status) {
    static_assert(ES == 8 || ES == 16, "8- or 16-byte elements");
    constexpr int NST = tma_stages(R);
    constexpr int TB = tma_tile_bytes(R);
    constexpr int BI = 128 / ES;  // elements of b per tile
    extern __shared__ unsigned char smem_raw[];
    unsigned char *ring = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    TmaTileInfo *info = (TmaTileInfo *)(ring + NST * TB);
    uint64_t *full = (uint64_t *)(info + NST);
    uint64_t *empty = full + NST;
    volatile int *abort_flag = (volatile int *)(empty + NST);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(smem_u32(full + s), 1);
            mbar_init(smem_u32(empty + s), kTmaConsumers);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    if (warp == kTmaConsumers) {
        // ---------------- TMA producer ----------------
        if (lane != 0) return;
        // coordinates of tile blockIdx.x and of the step gridDim.x, mixed radix
        int64_t c[5], st[5];
        int64_t u = blockIdx.x, v = gridDim.x;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            const int64_t qu = u / p.ext[i], qv = v / p.ext[i];
            c[i] = u - qu * p.ext[i];
            st[i] = v - qv * p.ext[i];
            u = qu;
            v = qv;
        }
        uint32_t g = 0;  // tiles issued by this CTA
        for (int64_t t = blockIdx.x; t < p.tiles; t += gridDim.x, ++g) {
            const int s = (int)(g % NST);
            const uint32_t round = g / NST;
            if (!mbar_wait(smem_u32(empty + s), (round & 1) ^ 1, abort_flag, status)) break;
            const int64_t a0 = c[1] * 32 * R, b0 = c[0] * BI;
            TmaTileInfo ti;
            ti.yoff = c[2] * p.ystr[0] + c[3] * p.ystr[1] + c[4] * p.ystr[2] + a0 + b0 * p.syb;
            ti.rows = (int32_t)min(p.ea - a0, (int64_t)(32 * R));
            ti.cols = (int32_t)min(p.eb - b0, (int64_t)BI);
            info[s] = ti;
            const uint32_t fb = smem_u32(full + s);
            mbar_expect_tx(fb, TB);  // release: the consumers see info[s] after their wait
            // x coordinate in 8-byte units: c[0] * 16, a multiple of 16 bytes
            tma_load_5d(smem_u32(ring + s * TB), &tm, (int)(c[0] * 16), (int)a0, (int)c[2], (int)c[3], (int)c[4],
                        fb);
            // next tile: add the step digit by digit with carries
            int64_t carry = 0;
#pragma unroll
            for (int i = 0; i < 5; ++i) {
                c[i] += st[i] + carry;
                carry = c[i] >= p.ext[i];
                if (carry) c[i] -= p.ext[i];
            }
        }
        // no bulk copy may still be writing into shared memory at exit
        for (uint32_t gg = g > (uint32_t)NST ? g - NST : 0u; gg < g; ++gg)
            mbar_drain(smem_u32(full + gg % NST), (gg / NST) & 1);
        return;
    }

    // ---------------- consumers ----------------
    // Warp w reads the (row block, chunk) pairs q = w + 4 i, i < 2 R:
    // row block q % R, 16-byte chunk q / R.
    uint32_t g = 0;
    for (int64_t t = blockIdx.x; t < p.tiles; t += gridDim.x, ++g) {
        const int s = (int)(g % NST);
        const uint32_t round = g / NST;
        if (!__all_sync(0xffffffffu, mbar_wait(smem_u32(full + s), round & 1, abort_flag, status))) break;
        const TmaTileInfo ti = info[s];
        const unsigned char *tile = ring + s * TB;
#pragma unroll
        for (int i = 0; i < 2 * R; ++i) {
            const int q = warp + 4 * i;
            const int row = (q % R) * 32 + lane;
            const int j = q / R;
            const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(tile + row * 128 + ((j ^ (row & 7)) << 4));
            if constexpr (ES == 16) {
                if (row < ti.rows && j < ti.cols)
                    *reinterpret_cast<ulonglong2 *>(y + (ti.yoff + row + j * p.syb) * ES) = v;
            } else {
                const bool odd = lane & 1;
                const unsigned long long got = __shfl_xor_sync(0xffffffffu, odd ? v.x : v.y, 1);
                const int r0 = row & ~1, col = 2 * j + (odd ? 1 : 0);
                if (r0 < ti.rows && col < ti.cols) {
                    unsigned char *dst = y + (ti.yoff + r0 + col * p.syb) * ES;
                    if (r0 + 1 < ti.rows)
                        *reinterpret_cast<ulonglong2 *>(dst) = odd ? make_ulonglong2(got, v.y)
                                                                   : make_ulonglong2(v.x, got);
                    else
                        *reinterpret_cast<unsigned long long *>(dst) = odd ? got : v.x;
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(empty + s));
    }
}

// Tries the TMA-staged transpose; returns 1 when it does not apply (the
// caller then uses the register-tiled kernels), else an mgb_status.
template <int ES>
static int try_transpose_tma(const ModeGroup &g, int bmode, const void *x, void *y, cudaStream_t s) {
    const int64_t ea = g.ext[0], eb = g.ext[bmode];
    const int64_t sxa = g.str[0][0], syb = g.str[1][bmode];
    ModeGroup outer = drop_mode(g, 0, bmode);
    if (outer.n > 3) return 1;
    if ((uintptr_t)x % 16 || (uintptr_t)y % 16) return 1;
    if (ea >= INT32_MAX || eb * (ES / 8) >= INT32_MAX) return 1;
    // box strides: positive multiples of 16 bytes below 2^40; Y pairs 16-byte aligned
    auto ok_x = [](int64_t st) { return st > 0 && (st * ES) % 16 == 0 && st * ES < (1ll << 40); };
    auto ok_y = [](int64_t st) { return st > 0 && (st * ES) % 16 == 0; };
    if (!ok_x(sxa) || !ok_y(syb)) return 1;
    for (int i = 0; i < outer.n; ++i)
        if (!ok_x(outer.str[0][i]) || !ok_y(outer.str[1][i]) || outer.ext[i] >= INT32_MAX) return 1;
    // outer modes by increasing X stride
    std::vector<int> ord(outer.n);
    for (int i = 0; i < outer.n; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](int u, int v) { return outer.str[0][u] < outer.str[0][v]; });
    // 32 R rows per tile, R = 1..4: the least padding of a's extent, the
    // larger tile on ties
    int R = 4;
    for (int r = 3; r >= 1; --r)
        if ((ea + 32 * r - 1) / (32 * r) * (32 * r) < (ea + 32 * R - 1) / (32 * R) * (32 * R)) R = r;
    TmaPermArgs a;
    a.ext[0] = (eb + 128 / ES - 1) / (128 / ES);
    a.ext[1] = (ea + 32 * R - 1) / (32 * R);
    for (int i = 0; i < 3; ++i) {
        a.ext[2 + i] = i < outer.n ? outer.ext[ord[i]] : 1;
        a.ystr[i] = i < outer.n ? outer.str[1][ord[i]] : 0;
    }
    a.ea = ea;
    a.eb = eb;
    a.syb = syb;
    a.tiles = a.ext[0] * a.ext[1] * a.ext[2] * a.ext[3] * a.ext[4];

    PFN_encodeTiled_t enc = tensor_map_encoder();
    if (!enc) return 1;
    cuuint64_t dims[5], strides[4];
    dims[0] = (cuuint64_t)(eb * (ES / 8));  // 8-byte units
    dims[1] = (cuuint64_t)ea;
    strides[0] = (cuuint64_t)(sxa * ES);
    for (int i = 0; i < 3; ++i) {
        dims[2 + i] = (cuuint64_t)a.ext[2 + i];
        strides[1 + i] = i < outer.n ? (cuuint64_t)(outer.str[0][ord[i]] * ES) : strides[i];
    }
    cuuint32_t box[5] = {16, (cuuint32_t)(32 * R), 1, 1, 1};
    cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUtensorMap tm;
    if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, const_cast<void *>(x), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return 1;
    int32_t *status = device_status_ptr();
    if (!status) return fail(MGB_ERR_CUDA, "device status word unavailable");

    auto launch = [&](auto kern, int smem) -> int {
        int dev = 0, sms = 0, per_sm = 0;
        MGB_CUDA_CHECK(cudaGetDevice(&dev));
        MGB_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        MGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTmaThreads, smem));
        const int64_t grid = std::min<int64_t>(a.tiles, (int64_t)sms * std::max(per_sm, 1));
        kern<<<(unsigned)grid, kTmaThreads, smem, s>>>(tm, (unsigned char *)y, a, status);
        MGB_CUDA_CHECK(cudaGetLastError());
        return MGB_OK;
    };
    static_assert(tma_smem_bytes(1) <= 48 * 1024 && tma_smem_bytes(2) <= 48 * 1024 &&
                      tma_smem_bytes(3) <= 48 * 1024 && tma_smem_bytes(4) <= 48 * 1024,
                  "default dynamic shared memory limit");
    switch (R) {
    case 1: return launch(k_transpose_tma<ES, 1>, tma_smem_bytes(1));
    case 2: return launch(k_transpose_tma<ES, 2>, tma_smem_bytes(2));
    case 3: return launch(k_transpose_tma<ES, 3>, tma_smem_bytes(3));
    default: return launch(k_transpose_tma<ES, 4>, tma_smem_bytes(4));
    }
}

// ---- gather (no unit-stride mode) ---------------------------------------------
template <typename TS, typename TD>
__global__ void k_gather(const TS *__restrict__ x, TD *__restrict__ y, ModeGroup g, int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t idx = i, ox = 0, oy = 0;
        for (int m = 0; m < g.n; ++m) {
            int64_t e = g.ext[m];
            int64_t q = idx / e;
            int64_t r = idx - q * e;
            ox += r * g.str[0][m];
            oy += r * g.str[1][m];
            idx = q;
        }
        y[oy] = Conv<TS, TD>::f(x[ox]);
    }
}

static ModeGroup drop_mode(const ModeGroup &g, int a, int b) {
    ModeGroup o;
    o.n = 0;
    for (int i = 0; i < g.n; ++i) {
        if (i == a || i == b) continue;
        o.ext[o.n] = g.ext[i];
        for (int t = 0; t < 3; ++t) o.str[t][o.n] = g.str[t][i];
        ++o.n;
    }
    return o;
}

template <typename TS, typename TD>
static int run_permute(const PermGeom &pg, const TS *x, TD *y, cudaStream_t s) {
    const ModeGroup &g = pg.g;
    int64_t total = g.size();
    if (total == 0) return MGB_OK;
    if (pg.a == 0 && pg.b == 0) {
        ModeGroup outer = drop_mode(g, 0, 0);
        int64_t rowlen = g.ext[0];
        int64_t nrows = outer.size();
        int64_t cpr = (rowlen + kRowChunk - 1) / kRowChunk;
        int vec = 0;
        if (sizeof(TS) == sizeof(TD) && std::is_same<TS, TD>::value && sizeof(TD) <= 16) {
            bool al = ((uintptr_t)x % 16 == 0) && ((uintptr_t)y % 16 == 0);
            for (int i = 0; i < outer.n; ++i)
                al = al && ((outer.str[0][i] * (int64_t)sizeof(TS)) % 16 == 0) &&
                     ((outer.str[1][i] * (int64_t)sizeof(TD)) % 16 == 0);
            al = al && ((kRowChunk * sizeof(TD)) % 16 == 0);
            vec = al ? 1 : 0;
        }
        int64_t blocks = nrows * cpr;
        if (blocks > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "permute: too many rows");
        k_rowcopy<TS, TD><<<(unsigned)blocks, 256, 0, s>>>(x, y, outer, rowlen, cpr, vec);
    } else if (pg.a == 0 && pg.b > 0) {
        ModeGroup outer = drop_mode(g, 0, pg.b);
        int64_t ea = g.ext[0], eb = g.ext[pg.b];
        int64_t sxa = g.str[0][0], syb = g.str[1][pg.b];
        // Tile edges of 32 or 64 elements, each chosen to pad its extent
        // least (a 96-wide panel is three 32-row tiles, not one and a half
        // 64-row ones whose second half idles), larger on ties; 16-byte
        // types stay at 32 x 32 (16 KB of shared memory).
        if constexpr (std::is_same<TS, TD>::value && (sizeof(TD) == 8 || sizeof(TD) == 16)) {
            const int rc = try_transpose_tma<(int)sizeof(TD)>(g, pg.b, x, y, s);
            if (rc != 1) return rc;
        }
        if constexpr (std::is_same<TS, TD>::value && sizeof(TD) == 8) {
            // 16-byte vectors: every tile row starts on a 16-byte boundary in
            // X (row stride sxa, tile columns from an even b) and in Y
            bool al = ((uintptr_t)x % 16 == 0) && ((uintptr_t)y % 16 == 0) && sxa % 2 == 0 && syb % 2 == 0;
            for (int i = 0; i < outer.n && al; ++i) al = outer.str[0][i] % 2 == 0 && outer.str[1][i] % 2 == 0;
            if (al) {
                const int64_t tiles_a = (ea + 63) / 64, tiles_b = (eb + 63) / 64;
                const int64_t blocks = tiles_a * tiles_b * outer.size();
                if (blocks > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "permute: too many tiles");
                k_transpose_v2<TD><<<(unsigned)blocks, 256, 0, s>>>((const TD *)x, y, outer, ea, eb, sxa, syb, tiles_a,
                                                                     tiles_b);
                MGB_CUDA_CHECK(cudaGetLastError());
                return MGB_OK;
            }
        }
        auto pad = [](int64_t e, int64_t t) { return (e + t - 1) / t * t; };
        const bool wide = sizeof(TD) <= 8;
        const int ta_ = (wide && pad(ea, 64) <= pad(ea, 32)) ? 64 : 32;
        const int tb_ = (wide && pad(eb, 64) <= pad(eb, 32)) ? 64 : 32;
        int64_t tiles_a = (ea + ta_ - 1) / ta_, tiles_b = (eb + tb_ - 1) / tb_;
        int64_t blocks = tiles_a * tiles_b * outer.size();
        if (blocks > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "permute: too many tiles");
        const unsigned nb = (unsigned)blocks;
        if (ta_ == 64 && tb_ == 64)
            k_transpose<TS, TD, 64, 64><<<nb, 256, 0, s>>>(x, y, outer, ea, eb, sxa, syb, tiles_a, tiles_b);
        else if (ta_ == 64)
            k_transpose<TS, TD, 64, 32><<<nb, 256, 0, s>>>(x, y, outer, ea, eb, sxa, syb, tiles_a, tiles_b);
        else if (tb_ == 64)
            k_transpose<TS, TD, 32, 64><<<nb, 256, 0, s>>>(x, y, outer, ea, eb, sxa, syb, tiles_a, tiles_b);
        else
            k_transpose<TS, TD, 32, 32><<<nb, 256, 0, s>>>(x, y, outer, ea, eb, sxa, syb, tiles_a, tiles_b);
    } else {
        int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 32);
        k_gather<TS, TD><<<(unsigned)blocks, 256, 0, s>>>(x, y, g, total);
    }
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

int launch_permute(const Desc &x, const Desc &y, const void *X, void *Y, cudaStream_t s) {
    // modes in Y's order with their X strides; fold with Y as the primary tensor
    ModeGroup g;
    g.n = 0;
    bool empty = false;
    struct R {
        int64_t e, sx, sy;
    };
    std::vector<R> ms;
    for (int i = 0; i < y.rank; ++i) {
        int j = 0;
        while (j < x.rank && x.modes[j] != y.modes[i]) ++j;
        if (y.ext[i] == 0) empty = true;
        if (y.ext[i] == 1) continue;
        ms.push_back({y.ext[i], x.str[j], y.str[i]});
    }
    if (empty) return MGB_OK;
    std::stable_sort(ms.begin(), ms.end(),
                     [](const R &p, const R &q) { return std::llabs(p.sy) < std::llabs(q.sy); });
    std::vector<R> f;
    for (auto &m : ms) {
        if (!f.empty() && m.sx == f.back().sx * f.back().e && m.sy == f.back().sy * f.back().e) {
            f.back().e *= m.e;
            continue;
        }
        f.push_back(m);
    }
    PermGeom pg;
    g.n = (int)f.size();
    for (int i = 0; i < g.n; ++i) {
        g.ext[i] = f[i].e;
        g.str[0][i] = f[i].sx;
        g.str[1][i] = f[i].sy;
        g.str[2][i] = 0;
    }
    if (g.n == 0) {  // single element
        g.n = 1;
        g.ext[0] = 1;
        g.str[0][0] = g.str[1][0] = 1;
        g.str[2][0] = 0;
    }
    pg.g = g;
    if (g.str[1][0] == 1) pg.a = 0;
    for (int i = 0; i < g.n; ++i)
        if (g.str[0][i] == 1) {
            pg.b = i;
            break;
        }
    if (pg.a != 0) pg.b = -1;
    if (pg.b < 0) pg.a = -1;

#define MGB_PERM_CASE(SD, DD, TS, TD) \
    if (x.dtype == SD && y.dtype == DD) return run_permute<TS, TD>(pg, (const TS *)X, (TD *)Y, s);
    MGB_PERM_CASE(MGB_F32, MGB_F32, float, float)
    MGB_PERM_CASE(MGB_F64, MGB_F64, double, double)
    MGB_PERM_CASE(MGB_C32, MGB_C32, float2, float2)
    MGB_PERM_CASE(MGB_C64, MGB_C64, double2, double2)
    MGB_PERM_CASE(MGB_F32, MGB_F64, float, double)
    MGB_PERM_CASE(MGB_F32, MGB_C32, float, float2)
    MGB_PERM_CASE(MGB_F32, MGB_C64, float, double2)
    MGB_PERM_CASE(MGB_F64, MGB_C64, double, double2)
    MGB_PERM_CASE(MGB_C32, MGB_C64, float2, double2)
#undef MGB_PERM_CASE
    return fail(MGB_ERR_ARGUMENT, "permute: unsupported conversion");
}

// ---- zero fill for K == 0 contractions (sum over an empty range) ----------------
template <typename T>
__global__ void k_fill_zero(T *y, ModeGroup g, int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t idx = i, off = 0;
        for (int m = 0; m < g.n; ++m) {
            int64_t e = g.ext[m];
            int64_t q = idx / e;
            off += (idx - q * e) * g.str[0][m];
            idx = q;
        }
        T z;
        memset(&z, 0, sizeof(T));
        y[off] = z;
    }
}

int launch_fill_zero(void *p, int64_t count, int dtype, const Desc &d, cudaStream_t s) {
    ModeGroup g;
    g.n = d.rank;
    for (int i = 0; i < d.rank; ++i) {
        g.ext[i] = d.ext[i];
        g.str[0][i] = d.str[i];
        g.str[1][i] = g.str[2][i] = 0;
    }
    if (g.n == 0) {
        g.n = 1;
        g.ext[0] = 1;
        g.str[0][0] = 1;
    }
    int64_t blocks = std::min<int64_t>((count + 255) / 256, 152 * 16);
    switch (dtype) {
    case MGB_F32: k_fill_zero<float><<<(unsigned)blocks, 256, 0, s>>>((float *)p, g, count); break;
    case MGB_F64: k_fill_zero<double><<<(unsigned)blocks, 256, 0, s>>>((double *)p, g, count); break;
    case MGB_C32: k_fill_zero<float2><<<(unsigned)blocks, 256, 0, s>>>((float2 *)p, g, count); break;
    default: k_fill_zero<double2><<<(unsigned)blocks, 256, 0, s>>>((double2 *)p, g, count); break;
    }
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

}  // namespace mgb
