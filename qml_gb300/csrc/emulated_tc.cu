// Emulated-FP64 products on the tcgen05 tensor cores (sm_103a).
//
//   C[i][j]  -=  sum_k P[i][k] * Q[j][k]        (mode SUBTRACT, C row-major, FP64)
//
// for an (i, j) region, where the rows of P and Q were cut into S base-128 digit
// planes by slice_rows_kernel (|digit| <= 64, exact in bf16) with one power-of-two
// scale per row.  Level l = s + t of the digit products is accumulated exactly in
// FP32 in tensor memory:
//   TMEM lane   = j (128 per tile; the contiguous index of C, so stores coalesce)
//   TMEM column = b * 8 TN + l * TN + (i - i0)   (TN per level, 8 levels)
// Every mode takes TN = 64 by default (8 levels fill the 512 columns, one accumulator
// b = 0, handed back once the levels are merged, so the next tile's MMAs run under the
// rest of the epilogue); TN = 32 gives two accumulators, so one tile's MMAs run while
// the epilogue drains the previous tile.  A tile runs kchunks 64-deep K
// chunks.  Per chunk the 8 digit planes of the TN i-rows are loaded once
// (double-buffered) and the 8 planes of the 128 j-rows stream through a ring; each
// j-plane s meets the i-planes t <= S-1-s in MMAs of N = TN cnt <= 256.
// Exactness: a level sums at most 8 * (64*kchunks) * 4096 products, so kchunks <= 8
// keeps every partial sum below 2^24.
//
// Warp roles (576 threads): warp 0 issues TMA loads, warp 1 owns TMEM and issues
// the MMAs from one thread, warps 2-17 run the epilogue, four per TMEM lane quarter
// (one per quarter of the TN columns, four columns per step, so each scheduler
// interleaves four epilogue warps): the levels are merged in 64-bit integers,
// converted once to FP64, scaled by 2^(e_i + e_j) and subtracted from C.  Waits are
// bounded; a timeout sets *err.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "rsqrt.cuh"
#include "common.cuh"
#include "emulated_gemm.cuh"
#include "tc_ptx.cuh"
#include "exp_fixed.cuh"

namespace {

using namespace qmlg::tc;

constexpr int TM = 128;         // TMEM lanes per tile (j)
constexpr int KC = 64;          // K chunk: one 128-byte swizzled row of bf16
constexpr int S_MAX = 8;
constexpr int EPI_WARPS = 16;   // four per TMEM lane quarter
constexpr int THREADS = 64 + 32 * EPI_WARPS;  // producer + MMA warps, then the epilogue
constexpr int EPI_THREADS = 32 * EPI_WARPS;
constexpr int EG = 4;           // columns per epilogue step
constexpr int A_BYTES = TM * KC * 2;  // 16 KB

// kLinear: the linear kernel matrix K = A B^T (the kKernelMatrix tiles, stores and
// symmetric mirror with the dot product itself as the entry).  kMatern: the Matern
// L2 kernel of order 1 or 2 on the same tiles, from d^2 = |a|^2 + |b|^2 - 2 a.b.
enum Mode { kSyrk = 0, kKernelMatrix = 1, kPredict = 2, kLinear = 3, kMatern = 4 };

// Tile shapes.  TN = 64 i-columns per level: 8 levels fill TMEM's 512 columns, one
// accumulator, so the next tile's MMAs wait for the epilogue's level merge; each A
// tile (128 rows x 8 planes) feeds 64 columns.  TN = 32: two accumulators, one
// tile's MMAs run while the epilogue drains the other, the B buffers are half as
// large (room for a deeper A ring), but each A tile feeds half as many outputs.
// The trailing update takes 64 (at 39488^2 x 512: 1501 TF/s against 1083 with 32,
// where the operand feed sets the pace), and so do the Gaussian kernel matrix (4.53
// against 4.98 ms at 20000^2) and the prediction.  Grouped updates can take either
// (a batch autotuner chooses).
template <int MODE, int TN_ = 64>
struct Shape {
    static constexpr int TN = TN_;                  // i columns per level
    static constexpr int NBUF = TN_ == 64 ? 1 : 2;  // accumulators in TMEM
    static constexpr int A_STAGES = TN_ == 64 ? 5 : 9;
    static constexpr int B_BYTES = TN * KC * 2;
    static constexpr int TBUF = 8 * TN;             // TMEM columns per accumulator
};
constexpr int RED_BYTES = 4 * 64 * 8;  // predict: per-warp column sums
constexpr int SMEM_BYTES = 2 * S_MAX * Shape<kSyrk>::B_BYTES + Shape<kSyrk>::A_STAGES * A_BYTES +
                           1024 /*align*/ + 256 /*barriers*/ + RED_BYTES;
static_assert(2 * S_MAX * Shape<kKernelMatrix>::B_BYTES + Shape<kKernelMatrix>::A_STAGES * A_BYTES +
                      1024 + 256 + RED_BYTES <= SMEM_BYTES,
              "shared memory of the Gaussian tile shape");

struct TileArgs {
    int ntiles;        // tiles in the (lower-triangular or full) tile list
    int tj;            // tiles along j
    double *C;         // kSyrk: row-major C; kKernelMatrix: column-major K
    int64_t ldc;
    int jbase, jend;   // lanes: contiguous index range of C / K
    int ibase, iend;   // TMEM columns
    int a_row0;        // digit row of j = jbase
    int b_row0;        // digit row of i = ibase
    int kchunks;
    int slices;
    const int *expA;   // per digit row
    const int *expB;
    int lower;         // kSyrk: update only j <= i; kKernelMatrix: symmetric (A is B)
    int *err;
    // Gaussian epilogues
    const double *normA;  // |x|^2 per digit row
    const double *normB;
    double scale;         // -0.5 / sigma^2 (kMatern: 1, the FMA then gives d^2)
    double diag_shift;
    int order;            // kMatern: 1 or 2
    double s1, s2;        // kMatern: -sqrt(2 order + 1) / sigma, 5 / (3 sigma^2)
    const double *alpha;  // kPredict: weights of the j rows
    double *partial;      // kPredict: [tiles along j][iend - ibase] partial sums
};

// Walks the tile list in increasing order.  With `lower`, row-block it (TN rows of
// i) holds the j-blocks jt with jbase + 128 jt <= ibase + TN it + TN - 1 (the tiles
// that reach the lower triangle); otherwise every jt.  The list runs in bands of
// kBand row-blocks (1024 rows of i): inside a band j-block by j-block, each across
// the band's row-blocks that hold it.  The CTAs working at the same time then share
// one band's i-planes and a few j-planes, which stay in L2.
template <int TN>
struct TileCursor {
    static constexpr int kBand = 1024 / TN;
    int band = 0, jt = 0, base = 0, rows = -1;
    __device__ __forceinline__ int count(const TileArgs &p, int r) const
    {
        if (!p.lower) return p.tj;
        const int lim = p.ibase - p.jbase + TN * r + TN - 1;
        return lim < 0 ? 0 : min(p.tj, lim / TM + 1);
    }
    // first row-block that holds j-block j (count(it) > j from there on)
    __device__ __forceinline__ int first_it(const TileArgs &p, int j) const
    {
        if (!p.lower) return 0;
        const int need = j * TM - (p.ibase - p.jbase) - TN + 1;
        return need <= 0 ? 0 : (need + TN - 1) / TN;
    }
    // t < ntiles; successive calls take nondecreasing t
    __device__ __forceinline__ void locate(const TileArgs &p, int t, int &jto, int &itl)
    {
        const int ti = (p.iend - p.ibase + TN - 1) / TN;
        if (!p.lower) {
            // every band holds tj rows of its width: found directly, so a CTA that
            // takes one tile (one CTA per tile) does not walk the list
            const int b = t / (p.tj * kBand);
            const int b0 = b * kBand, len = min(kBand, ti - b0);
            const int rem = t - b * (p.tj * kBand);
            jto = rem / len;
            itl = b0 + rem % len;
            return;
        }
        for (;;) {
            const int b0 = band * kBand, b1 = min(b0 + kBand, ti);
            if (b0 >= ti) {  // past the list: not reached for t < ntiles
                jto = 0;
                itl = 0;
                return;
            }
            if (rows < 0) {
                // entering a band: skip it whole when t lies beyond it (its size
                // summed over rows or over row-blocks, whichever are fewer)
                const int nr = count(p, b1 - 1);
                int tot = 0;
                if (nr <= b1 - b0) {
                    for (int j = 0; j < nr; ++j) tot += b1 - max(b0, first_it(p, j));
                } else {
                    for (int it = b0; it < b1; ++it) tot += count(p, it);
                }
                if (base + tot <= t) {
                    base += tot;
                    ++band;
                    continue;
                }
                rows = nr;
            }
            if (jt < rows) {
                const int i0 = max(b0, first_it(p, jt));
                const int len = b1 - i0;
                if (base + len > t) {
                    jto = jt;
                    itl = i0 + (t - base);
                    return;
                }
                base += len;
                ++jt;
            } else {
                ++band;
                jt = 0;
                rows = -1;
            }
        }
    }
};

__device__ __forceinline__ double pow2i(int e)
{
    if (e >= -1022 && e <= 1023) return __longlong_as_double((long long)(e + 1023) << 52);
    return ldexp(1.0, e);
}

__global__ void epilogue_exp_kernel(const double *__restrict__ x, double *__restrict__ y, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = exp_nonpos(x[i]);
}

// Grouped launches: the tiles of up to kMaxGroup independent problems in one
// persistent launch.  The problems share the two tensor maps (their digit rows lie at
// different offsets of one plane buffer), K width, plane count and the per-row
// arrays; each has its own output, ranges, digit-row offsets and Gaussian scale.
// Problem g owns tiles [tile_base, tile_base + its count) of the launch's list, in
// the order of its own tile cursor.
constexpr int kMaxGroup = 128;

struct GroupEntry {
    double *C;
    int64_t ldc;
    double scale;
    int jbase, jend, ibase, iend;
    int a_row0, b_row0;
    int tj, tile_base;
};

struct TileGroup {
    int count, pad;
    GroupEntry e[kMaxGroup];
};

// Maps a tile index to (jt, itl) and returns the arguments that hold for that tile:
// the launch's own, or (grouped) a copy with its problem's fields.  A CTA visits its
// tiles in increasing order, so the problem index only grows and each problem's
// cursor starts fresh.
template <int TN, bool GROUPED>
struct TileWalker;

template <int TN>
struct TileWalker<TN, false> {
    TileCursor<TN> cur;
    __device__ __forceinline__ const TileArgs &locate(const TileArgs &p, const TileGroup *, int t,
                                                      int &jt, int &itl)
    {
        cur.locate(p, t, jt, itl);
        return p;
    }
};

template <int TN>
struct TileWalker<TN, true> {
    TileCursor<TN> cur;
    int g = -1;
    TileArgs q;
    __device__ __forceinline__ const TileArgs &locate(const TileArgs &p, const TileGroup *grp, int t,
                                                      int &jt, int &itl)
    {
        int gg = g < 0 ? 0 : g;
        while (gg + 1 < grp->count && grp->e[gg + 1].tile_base <= t) ++gg;
        if (gg != g) {
            const GroupEntry &e = grp->e[gg];
            g = gg;
            cur = TileCursor<TN>();
            q = p;
            q.C = e.C;
            q.ldc = e.ldc;
            q.scale = e.scale;
            q.jbase = e.jbase;
            q.jend = e.jend;
            q.ibase = e.ibase;
            q.iend = e.iend;
            q.a_row0 = e.a_row0;
            q.b_row0 = e.b_row0;
            q.tj = e.tj;
        }
        cur.locate(q, t - grp->e[g].tile_base, jt, itl);
        return q;
    }
};

template <int MODE, bool GROUPED, int TNX = Shape<MODE>::TN>
__device__ __forceinline__ void emu_tc_body(const CUtensorMap &mapA, const CUtensorMap &mapB,
                                            const TileArgs &p, const TileGroup *grp)
{
    using SH = Shape<MODE, TNX>;
    constexpr int TN = SH::TN, A_STAGES = SH::A_STAGES, B_BYTES = SH::B_BYTES, TBUF = SH::TBUF;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *base =
        (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *Bbuf = base;                               // [2][S_MAX][B_BYTES]
    unsigned char *Aring = base + 2 * S_MAX * B_BYTES;        // [A_STAGES][A_BYTES]
    uint64_t *bars = (uint64_t *)(Aring + A_STAGES * A_BYTES);
    uint64_t *bFull = bars, *bEmpty = bars + 2, *aFull = bars + 4, *aEmpty = bars + 4 + A_STAGES,
             *tFull = bars + 4 + 2 * A_STAGES, *tEmpty = tFull + 2;
    uint32_t *tmem_holder = (uint32_t *)(tEmpty + 2);
    double(*red)[TN] = (double(*)[TN])(bars + 32);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int S = p.slices;

    if (threadIdx.x == 0) {
        for (int k = 0; k < 2; ++k) {
            mbar_init(&bFull[k], 1);
            mbar_init(&bEmpty[k], 1);
        }
        for (int k = 0; k < A_STAGES; ++k) {
            mbar_init(&aFull[k], 1);
            mbar_init(&aEmpty[k], 1);
        }
        for (int k = 0; k < 2; ++k) {
            mbar_init(&tFull[k], 1);
            mbar_init(&tEmpty[k], EPI_THREADS);
        }
        fence_barrier_init();
    }
    if (warp == 0 && lane == 0) {
        prefetch_tensormap(&mapA);
        prefetch_tensormap(&mapB);
    }
    if (warp == 1) tmem_alloc(tmem_holder, 512);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_holder;

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- TMA producer: runs ahead across tiles.  The i-planes of
            // chunk g+1 are requested halfway through the j-planes of chunk g, so they
            // are in flight while chunk g's MMAs run.
            TileWalker<TN, GROUPED> cur, nxt;
            int g = 0, it = 0;
            bool ok = true;
            int b_issued = -1;  // highest chunk index whose i-planes are requested
            auto issue_b = [&](int gg, int brow_g, int cc) -> bool {
                const int bb = gg & 1;
                if (gg >= 2 && !mbar_wait(&bEmpty[bb], ((gg >> 1) - 1) & 1)) return false;
                mbar_expect_tx(&bFull[bb], (uint32_t)(S * B_BYTES));
                for (int u = 0; u < S; ++u)
                    tma_load_3d(Bbuf + (bb * S_MAX + u) * B_BYTES, &mapB, &bFull[bb], cc * KC, brow_g, u);
                b_issued = gg;
                return true;
            };
            for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
                int jt, itl;
                const TileArgs &pt = cur.locate(p, grp, t, jt, itl);
                const int arow = pt.a_row0 + jt * TM, brow = pt.b_row0 + itl * TN;
                // the chunk after this tile's last one belongs to the next tile
                int brow_next = -1;
                if (t + (int)gridDim.x < p.ntiles) {
                    int jt2, it2;
                    nxt = cur;
                    const TileArgs &pn = nxt.locate(p, grp, t + gridDim.x, jt2, it2);
                    brow_next = pn.b_row0 + it2 * TN;
                }
                for (int c = 0; c < p.kchunks && ok; ++c, ++g) {
                    if (b_issued < g && !issue_b(g, brow, c)) {
                        ok = false;
                        break;
                    }
                    for (int s = 0; s < S; ++s, ++it) {
                        if (s == S / 2) {
                            // next chunk's i-planes (this tile, or the next tile's first)
                            if (c + 1 < p.kchunks) {
                                if (!issue_b(g + 1, brow, c + 1)) ok = false;
                            } else if (brow_next >= 0) {
                                if (!issue_b(g + 1, brow_next, 0)) ok = false;
                            }
                            if (!ok) break;
                        }
                        const int st = it % A_STAGES, round = it / A_STAGES;
                        if (round >= 1 && !mbar_wait(&aEmpty[st], (round - 1) & 1)) {
                            ok = false;
                            break;
                        }
                        mbar_expect_tx(&aFull[st], (uint32_t)A_BYTES);
                        tma_load_3d(Aring + st * A_BYTES, &mapA, &aFull[st], c * KC, arow, s);
                    }
                }
            }
            if (!ok) atomicOr(p.err, 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer
            int g = 0, it = 0, u = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x, ++u) {
                // accumulator tb, its use-th use: wait for the epilogue to have
                // drained the previous one
                const int tb = SH::NBUF == 2 ? (u & 1) : 0, use = SH::NBUF == 2 ? (u >> 1) : u;
                if (use >= 1 && !mbar_wait(&tEmpty[tb], (use - 1) & 1)) {
                    ok = false;
                    break;
                }
                fence_after_sync();
                for (int c = 0; c < p.kchunks && ok; ++c, ++g) {
                    const int bb = g & 1;
                    if (!mbar_wait(&bFull[bb], (g >> 1) & 1)) {
                        ok = false;
                        break;
                    }
                    fence_after_sync();
                    for (int s = 0; s < S; ++s, ++it) {
                        const int st = it % A_STAGES, round = it / A_STAGES;
                        if (!mbar_wait(&aFull[st], round & 1)) {
                            ok = false;
                            break;
                        }
                        fence_after_sync();
                        const uint64_t da = desc_sw128(Aring + st * A_BYTES);
                        // the i-planes v .. v+cnt-1 sit back to back in shared memory, so
                        // one MMA with N = TN cnt (<= 256) accumulates levels s+v ..
                        // s+v+cnt-1, each into its own TN TMEM columns
                        for (int v = 0; v + s < S;) {
                            const int cnt = min(256 / TN, S - s - v);
                            const uint32_t idn = idesc_bf16_f32(TM, TN * cnt);
                            const uint64_t db = desc_sw128(Bbuf + (bb * S_MAX + v) * B_BYTES);
                            const uint32_t dst = tmem + (uint32_t)(tb * TBUF + (s + v) * TN);
#pragma unroll
                            for (int kk = 0; kk < KC / 16; ++kk) {
                                const uint32_t acc = (c > 0 || s > 0 || kk > 0) ? 1u : 0u;
                                mma_bf16(dst, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idn, acc);
                            }
                            v += cnt;
                        }
                        mma_commit(&aEmpty[st]);
                    }
                    mma_commit(&bEmpty[bb]);
                }
                mma_commit(&tFull[tb]);
            }
            if (!ok) atomicOr(p.err, 2);
        }
    } else {
        // ---------------- epilogue: warps 2..9 -> TMEM lane quarter q = warp & 3,
        // columns HC h .. HC h + HC-1 of each level with h = (warp - 2) / 4
        constexpr int HC = TN / (EPI_WARPS / 4);
        const int q = warp & 3, h = (warp - 2) >> 2;
        const int jl = q * 32 + lane;
        const int H = (S + 1) / 2;
        const int lo_levels = S - H;
        const int shift = lo_levels >= 2 ? 12 : 0;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        TileWalker<TN, GROUPED> cur;
        int u = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < p.ntiles; t += gridDim.x, ++u) {
            int jt, itl;
            const TileArgs &pt = cur.locate(p, grp, t, jt, itl);
            const int j0 = pt.jbase + jt * TM, i0 = pt.ibase + itl * TN;
            const int arow = pt.a_row0 + jt * TM, brow = pt.b_row0 + itl * TN;
            const int j = j0 + jl;
            const int tb = SH::NBUF == 2 ? (u & 1) : 0, use = SH::NBUF == 2 ? (u >> 1) : u;
            const uint32_t tbuf = lane_base + (uint32_t)(tb * TBUF);  // this tile's accumulator
            // every (j, i) of the tile is inside the updated range
            const bool interior = j0 + TM <= pt.jend && i0 + TN <= pt.iend &&
                                  (!p.lower || j0 + TM - 1 <= i0);
            if (MODE == kSyrk && j < pt.jend) {
                // while the MMAs run, pull this thread's part of C into L2 so the
                // read-modify-write below does not wait on DRAM
                const int ilo = i0 + h * HC, ilim = min(ilo + HC, pt.iend);
                for (int i = ilo; i < ilim; ++i)
                    if (interior || !p.lower || j <= i)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(pt.C + (int64_t)i * pt.ldc + j));
            }
            if (ok && !mbar_wait(&tFull[tb], use & 1)) {
                ok = false;
                if (lane == 0) atomicOr(p.err, 4);
            }
            fence_after_sync();
            const bool jvalid = j < pt.jend;
            const int ej = jvalid ? p.expA[arow + jl] : 0;
            double aj = 0.0, aw = 0.0;
            if (MODE != kSyrk && MODE != kLinear && jvalid) {
                aj = pt.scale * p.normA[arow + jl];
                if (MODE == kPredict) aw = p.alpha[j];
            }
            // Levels of eight columns -> exact integers (value in units of 2^(shift -
            // 7(S+1)) relative to the row scales).
            auto merge8 = [&](const uint32_t (&v)[S_MAX][EG], long long *out) {
                if (S == 8) {
                    // K <= 512 bounds level l by (l+1) 2^21, so two adjacent levels
                    // combine exactly in 32 bits (d6 * 128 + d7 < 1.9e9)
#pragma unroll
                    for (int col = 0; col < EG; ++col) {
                        int d[8];
#pragma unroll
                        for (int l = 0; l < 8; ++l) d[l] = __float2int_rn(__uint_as_float(v[l][col]));
                        const long long hi = (long long)(d[0] * 128 + d[1]) * 16384 + (d[2] * 128 + d[3]);
                        const long long lo = (long long)(d[4] * 128 + d[5]) * 16384 + (d[6] * 128 + d[7]);
                        out[col] = (hi << (28 - 12)) + (lo >> 12);
                    }
                } else {
#pragma unroll
                    for (int col = 0; col < EG; ++col) {
                        long long hi = 0, lo = 0;
#pragma unroll
                        for (int l = 0; l < S_MAX; ++l) {
                            if (l >= S) break;
                            const long long d = (long long)__float2int_rn(__uint_as_float(v[l][col]));
                            if (l < H) hi = hi * 128 + d;
                            else lo = lo * 128 + d;
                        }
                        // value = hi * 128^lo_levels + lo, kept in 62 bits by dropping the
                        // lowest `shift` bits of lo (far below FP64 resolution of the value)
                        out[col] = (hi << (7 * lo_levels - shift)) + (lo >> shift);
                    }
                }
            };
            if (MODE == kSyrk) {
                // (1) merge all HC of this warp's columns, then hand the accumulator
                // back, then (2) the read-modify-write of C
                long long v64[HC];
#pragma unroll
                for (int gq = 0; gq < HC / EG; ++gq) {
                    uint32_t v[S_MAX][EG];
#pragma unroll
                    for (int l = 0; l < S_MAX; ++l)
                        if (l < S) tmem_ld4(tbuf + (uint32_t)(l * TN + h * HC + gq * EG), v[l]);
                    tmem_ld_wait();
                    merge8(v, v64 + gq * EG);
                }
                fence_before_sync();
                mbar_arrive(&tEmpty[tb]);
                if (ok) {
#pragma unroll
                    for (int gq = 0; gq < HC / EG; ++gq) {
                        const int cb = h * HC + gq * EG;
                        double cv[EG];
#pragma unroll
                        for (int col = 0; col < EG; ++col) {
                            const int i = i0 + cb + col;
                            cv[col] = (interior || (jvalid && i < pt.iend && (!p.lower || j <= i)))
                                          ? pt.C[(int64_t)i * pt.ldc + j] : 0.0;
                        }
#pragma unroll
                        for (int col = 0; col < EG; ++col) {
                            const int il = cb + col;
                            const int i = i0 + il;
                            if (interior || (jvalid && i < pt.iend && (!p.lower || j <= i))) {
                                const double sc = pow2i(p.expB[brow + il] + ej + shift - 7 * (S + 1));
                                pt.C[(int64_t)i * pt.ldc + j] = fma(-(double)v64[gq * EG + col], sc, cv[col]);
                            }
                        }
                    }
                }
            } else {
                // Gaussian epilogues.  The per-column terms (scale |b|^2, b's exponent)
                // are loaded once per tile by the lane of that column and broadcast;
                // -2 scale 2^e is formed on the bits.
                const int ibl = i0 + h * HC + lane;
                const bool ilv = lane < HC && ibl < pt.iend;
                const double sBl = ilv ? pt.scale * p.normB[brow + h * HC + lane] : 0.0;
                const int eBl = ilv ? p.expB[brow + h * HC + lane] : 0;
                const double m2s = -2.0 * pt.scale;
                const long long m2s_bits = __double_as_longlong(m2s);
                const int m2s_exp = (int)((m2s_bits >> 52) & 0x7ff);
                double cs[HC];  // kPredict: this thread's k(a_j, b_i) alpha_j, i = column
#pragma unroll
                for (int k = 0; k < HC; ++k) cs[k] = 0.0;
                // one accumulator (TN = 64): merge every column's levels first and hand
                // the accumulator back, so the next tile's MMAs run under the exps;
                // two (TN = 32): drain and compute eight columns at a time
                constexpr bool EARLY = SH::NBUF == 1;
                long long v64all[EARLY ? HC : 1];
                if constexpr (EARLY) {
#pragma unroll
                    for (int gq = 0; gq < HC / EG; ++gq) {
                        uint32_t v[S_MAX][EG];
#pragma unroll
                        for (int l = 0; l < S_MAX; ++l)
                            if (l < S) tmem_ld4(tbuf + (uint32_t)(l * TN + h * HC + gq * EG), v[l]);
                        tmem_ld_wait();
                        merge8(v, v64all + gq * EG);
                    }
                    fence_before_sync();
                    mbar_arrive(&tEmpty[tb]);
                }
#pragma unroll
                for (int gq = 0; gq < HC / EG; ++gq) {
                    const int cb = h * HC + gq * EG;
                    long long v64[EG];
                    if constexpr (EARLY) {
                        if (!ok) continue;
#pragma unroll
                        for (int col = 0; col < EG; ++col) v64[col] = v64all[gq * EG + col];
                    } else {
                        uint32_t v[S_MAX][EG];
#pragma unroll
                        for (int l = 0; l < S_MAX; ++l)
                            if (l < S) tmem_ld4(tbuf + (uint32_t)(l * TN + cb), v[l]);
                        tmem_ld_wait();
                        if (gq == HC / EG - 1) {
                            fence_before_sync();
                            mbar_arrive(&tEmpty[tb]);
                        }
                        if (!ok) continue;
                        merge8(v, v64);
                    }
#pragma unroll
                    for (int col = 0; col < EG; ++col) {
                        const int il = cb + col;
                        const int i = i0 + il;
                        const double sb = __shfl_sync(0xffffffffu, sBl, gq * EG + col);
                        const int eb = __shfl_sync(0xffffffffu, eBl, gq * EG + col);
                        const bool valid = jvalid && i < pt.iend;
                        double kv = 0.0;
                        if (valid) {
                            const int ew = eb + ej + shift - 7 * (S + 1);
                            if constexpr (MODE == kLinear) {
                                // a.b = v 2^ew: one rounding, in the integer-to-double step
                                kv = (double)v64[col] * pow2i(ew);
                                if (p.lower && i == j) kv += p.diag_shift;
                            } else {
                                // x = scale * (|a|^2 + |b|^2 - 2 a.b)
                                const int ef = m2s_exp + ew;
                                const double w = (m2s_exp > 0 && ef > 0 && ef < 2047)
                                                     ? __longlong_as_double(m2s_bits + ((long long)ew << 52))
                                                     : m2s * pow2i(ew);
                                const double x = fma((double)v64[col], w, aj + sb);
                                if constexpr (MODE == kMatern) {
                                    // d^2 rounds below 0 only for (near) equal rows; the
                                    // sign and zero tests are on the bits, and d = d^2 /
                                    // sqrt(d^2) comes from rsqrt_halley (within 2 ulp)
                                    const bool pos = __double_as_longlong(x) > 0;
                                    const double d2 = pos ? x : 0.0;
                                    const double dd = pos ? d2 * rsqrt_halley(d2) : 0.0;
                                    double poly = 1.0 - p.s1 * dd;
                                    if (p.order == 2) poly += p.s2 * d2;
                                    kv = exp_nonpos(p.s1 * dd) * poly;
                                } else {
                                    kv = exp_nonpos(x);
                                }
                                if ((MODE == kKernelMatrix || MODE == kMatern) && p.lower && i == j)
                                    kv = 1.0 + p.diag_shift;
                            }
                        }
                        if (MODE == kKernelMatrix || MODE == kLinear || MODE == kMatern) {
                            if (valid && (!p.lower || j <= i)) {
                                pt.C[(int64_t)i * pt.ldc + j] = kv;
                                if (p.lower && j < i) pt.C[(int64_t)j * pt.ldc + i] = kv;
                            }
                        } else {
                            cs[gq * EG + col] = valid ? kv * aw : 0.0;
                        }
                    }
                    if constexpr (MODE == kPredict) {
                        if ((gq + 1) * EG % 8 == 0) {
                            // eight columns complete: their sums over the warp's 32 rows
                            // by recursive halving.  Each step a lane keeps half of its
                            // columns and adds its partner's values for them (9 FP64
                            // adds for 8 columns, not 5 per column); lanes 4m end with
                            // the sum of column (lane bits 4, 3, 2).  The lanes are
                            // paired by distance 16, 8, 4, 2, 1 for every column.
                            const int hb = (gq + 1) * EG - 8;  // first column of the eight
                            const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0,
                                       h4 = (lane & 4) != 0;
                            double v4[4], v2[2];
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                v4[k] = (h16 ? cs[hb + k + 4] : cs[hb + k]) +
                                        __shfl_xor_sync(0xffffffffu, h16 ? cs[hb + k] : cs[hb + k + 4], 16);
#pragma unroll
                            for (int k = 0; k < 2; ++k)
                                v2[k] = (h8 ? v4[k + 2] : v4[k]) +
                                        __shfl_xor_sync(0xffffffffu, h8 ? v4[k] : v4[k + 2], 8);
                            double v1 = (h4 ? v2[1] : v2[0]) +
                                        __shfl_xor_sync(0xffffffffu, h4 ? v2[0] : v2[1], 4);
                            v1 += __shfl_xor_sync(0xffffffffu, v1, 2);
                            v1 += __shfl_xor_sync(0xffffffffu, v1, 1);
                            if ((lane & 3) == 0)
                                red[q][h * HC + hb + (h16 ? 4 : 0) + (h8 ? 2 : 0) + (h4 ? 1 : 0)] = v1;
                        }
                    }
                }
            }
            if (MODE == kPredict) {
                // the four quarters' column sums are added in a fixed order
                asm volatile("bar.sync 1, %0;" ::"n"(EPI_THREADS) : "memory");
                const int tt = threadIdx.x - 64;
                if (ok && tt < TN && i0 + tt < pt.iend)
                    p.partial[(int64_t)jt * (pt.iend - pt.ibase) + (i0 - pt.ibase) + tt] =
                        ((red[0][tt] + red[1][tt]) + red[2][tt]) + red[3][tt];
                asm volatile("bar.sync 1, %0;" ::"n"(EPI_THREADS) : "memory");
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, 512);
}

template <int MODE>
__global__ void __launch_bounds__(THREADS, 1)
emu_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
              const __grid_constant__ TileArgs p)
{
    emu_tc_body<MODE, false>(mapA, mapB, p, nullptr);
}

template <int MODE, int TNX = Shape<MODE>::TN>
__global__ void __launch_bounds__(THREADS, 1)
emu_tc_group_kernel(const __grid_constant__ CUtensorMap mapA,
                    const __grid_constant__ CUtensorMap mapB, const __grid_constant__ TileArgs p,
                    const __grid_constant__ TileGroup grp)
{
    emu_tc_body<MODE, true, TNX>(mapA, mapB, p, &grp);
}

// One warp per row: power-of-two row scale over the K-range and S digit planes.
// src rows r0 .. r0+nrows-1, columns c0 .. c0+kw-1 of the row-major matrix;
// digits [S][rpad][kp] bf16 (zero beyond kw and beyond nrows), expo [rpad].
// Each value is rounded once to the fixed-point integer q = round(x * 2^(7S-e))
// (|q| <= 2^(7S-1)), then split into balanced base-128 digits with integer shifts,
// least significant first: d = ((q + 64) mod 128) - 64, q <- (q - d) / 128; the most
// significant digit takes what is left, which is at most 64 in magnitude.
__device__ __forceinline__ void slice_row(const double *__restrict__ A, int64_t lda, int r0,
                                          int nrows, int c0, int kw, int kp, int rpad, int slices,
                                          __nv_bfloat16 *__restrict__ digits,
                                          int *__restrict__ expo, double *__restrict__ norms,
                                          const int *__restrict__ info, int warp)
{
    if (info != nullptr && *info != 0) return;
    const int lane = threadIdx.x & 31;
    if (warp >= rpad) return;
    const bool live = warp < nrows;
    const double *row = A + (int64_t)(r0 + warp) * lda + c0;
    // max |x| on the bits (the integer order of non-negative doubles is their order;
    // an infinity or NaN comes out non-finite), and the sum of squares only if asked
    unsigned long long mb = 0ull;
    double sq = 0.0;
    if (live)
        for (int k = lane; k < kw; k += 32) {
            const double v = row[k];
            const unsigned long long bv =
                (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
            mb = bv > mb ? bv : mb;
            if (norms != nullptr) sq = fma(v, v, sq);
        }
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, mb, off);
        mb = o > mb ? o : mb;
        if (norms != nullptr) sq += __shfl_xor_sync(0xffffffffu, sq, off);
    }
    if (norms != nullptr && lane == 0) norms[warp] = sq;
    const double m = __longlong_as_double((long long)mb);
    int e = 0;
    if (m > 0.0 && isfinite(m)) {
        frexp(m, &e);
        e += 1;  // |x| * 2^-e < 1/2
    }
    // x * 2^ks on the exponent bits (exact; |x * 2^ks| < 2^(7S-1)); a result below
    // 2^-1022 rounds to 0, and a subnormal x takes the FP64 multiply
    const int ks = 7 * slices - e;
    const double scale = pow2i(ks);
    const int64_t plane = (int64_t)rpad * kp;
    __nv_bfloat16 *dst = digits + (int64_t)warp * kp;
    for (int k0 = lane * 8; k0 < kp; k0 += 256) {
        long long q[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int k = k0 + u;
            long long qv = 0;
            if (live && k < kw) {
                const double v = row[k];
                const unsigned long long bv = (unsigned long long)__double_as_longlong(v);
                const int E = (int)((bv >> 52) & 0x7ff);
                if (E == 0) {
                    if ((bv & 0x000fffffffffffffull) != 0ull) qv = __double2ll_rn(v * scale);
                } else if (E + ks > 0) {
                    qv = __double2ll_rn(__longlong_as_double(
                        (long long)(bv + ((unsigned long long)(long long)ks << 52))));
                }
            }
            q[u] = qv;
        }
        for (int s = slices - 1; s >= 0; --s) {
            __align__(16) __nv_bfloat16 b[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                // the most significant digit keeps the remainder (|q| <= 64 there)
                const long long d = s > 0 ? ((q[u] + 64) & 127) - 64 : q[u];
                q[u] = (q[u] - d) >> 7;
                b[u] = __int2bfloat16_rn((int)d);
            }
            *reinterpret_cast<uint4 *>(dst + (int64_t)s * plane + k0) =
                *reinterpret_cast<const uint4 *>(b);
        }
    }
    if (lane == 0) expo[warp] = e;
}

__global__ void slice_rows_kernel(const double *__restrict__ A, int64_t lda, int r0, int nrows,
                                  int c0, int kw, int kp, int rpad, int slices,
                                  __nv_bfloat16 *__restrict__ digits, int *__restrict__ expo,
                                  double *__restrict__ norms, const int *__restrict__ info)
{
    slice_row(A, lda, r0, nrows, c0, kw, kp, rpad, slices, digits, expo, norms, info,
              (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5));
}

// Rows of many problems sliced into one shared plane buffer in one launch: problem g
// owns warps [warp_base, warp_base + its rows padded to 128) and its digit rows start
// at row0 (the plane stride is the shared buffer's row count).
struct SliceEntry {
    const double *A;
    int64_t lda;
    int r0, nrows, c0, kw;
    int row0, warp_base;
    const int *info;
};

struct SliceGroup {
    int count, pad;
    SliceEntry e[kMaxGroup];
};

__global__ void slice_rows_group_kernel(const __grid_constant__ SliceGroup g, int kp, int rows_total,
                                        int slices, __nv_bfloat16 *__restrict__ digits,
                                        int *__restrict__ expo)
{
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lo = 0, hi = g.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (g.e[mid].warp_base <= warp) lo = mid;
        else hi = mid - 1;
    }
    const SliceEntry &e = g.e[lo];
    const int w = warp - e.warp_base;
    if (w < 0 || w >= (e.nrows + 127) / 128 * 128) return;
    slice_row(e.A, e.lda, e.r0, e.nrows, e.c0, e.kw, kp, rows_total, slices,
              digits + (int64_t)e.row0 * kp, expo + e.row0, nullptr, e.info, w);
}

typedef CUresult (*EncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                             const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                             const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                             CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn()
{
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    });
    return fn;
}

int make_plane_map(CUtensorMap *map, const __nv_bfloat16 *digits, int kp, int rpad, int slices,
                   int box_rows)
{
    EncodeFn fn = encode_fn();
    if (fn == nullptr) return QMLG_E_CUDA;
    cuuint64_t dims[3] = {(cuuint64_t)kp, (cuuint64_t)rpad, (cuuint64_t)slices};
    cuuint64_t strides[2] = {(cuuint64_t)kp * 2, (cuuint64_t)rpad * kp * 2};
    cuuint32_t box[3] = {(cuuint32_t)KC, (cuuint32_t)box_rows, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)digits, dims, strides, box,
                    es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? QMLG_OK : QMLG_E_CUDA;
}


// Largest |x| over a row-major block (bit pattern of a non-negative double, so the
// integer maximum is the floating-point maximum).
__global__ void max_abs_kernel(const double *__restrict__ X, int64_t ldx, int rows, int cols,
                               unsigned long long *__restrict__ out)
{
    unsigned long long m = 0;
    const int64_t total = (int64_t)rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const double v = fabs(X[(e / cols) * ldx + e % cols]);
        const unsigned long long b = (unsigned long long)__double_as_longlong(v);
        if (b > m) m = b;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, m, off);
        if (o > m) m = o;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void reduce_partial_rows_kernel(const double *__restrict__ partial, int nparts, int n,
                                           double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += partial[(int64_t)p * n + i];
    y[i] = s;
}

int sm_count()
{
    static int n = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            n = 148;
    });
    return qmlg::sm_limit(n);
}

// Persistent CTAs (one per SM, looping over tiles) or, when the calling thread
// turned persistence off, one CTA per tile so that the block scheduler spreads
// the work over whatever SMs are free.
int tile_grid(int ntiles)
{
    return qmlg::persistent_tiles() ? std::min(ntiles, sm_count()) : ntiles;
}

// Same tile list as TileCursor on the device.
int count_tiles(int jbase, int jend, int ibase, int iend, int lower, int TN, int &tj)
{
    tj = (int)qmlg::ceil_div(jend - jbase, TM);
    const int ti = (int)qmlg::ceil_div(iend - ibase, TN);
    if (!lower) return tj * ti;
    int total = 0;
    for (int r = 0; r < ti; ++r) {
        const int lim = ibase - jbase + TN * r + TN - 1;
        total += lim < 0 ? 0 : std::min(tj, lim / TM + 1);
    }
    return total;
}

void set_smem_attrs()
{
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(emu_tc_kernel<kSyrk>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SMEM_BYTES);
        cudaFuncSetAttribute(emu_tc_kernel<kKernelMatrix>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        cudaFuncSetAttribute(emu_tc_kernel<kLinear>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        cudaFuncSetAttribute(emu_tc_kernel<kMatern>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        cudaFuncSetAttribute(emu_tc_kernel<kPredict>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    });
}

// Gaussian path: feature width padded to a multiple of the 64-element chunk.
int feature_pad(int d) { return (int)qmlg::ceil_div(d < 1 ? 1 : d, KC) * KC; }
int rows_pad(int n) { return (int)qmlg::ceil_div(n < 1 ? 1 : n, TM) * TM; }

// Smallest S whose worst-case error bound on K keeps the relative error below
// 0.5e-12: |dot error| <= 2^(eA + eB - 7S) * kp * (S + 1) / 4 (truncated digit
// levels plus the rounding of the fixed-point values), and the relative error of
// K = exp(-d^2 / (2 sigma^2)) is that error / sigma^2.  0 if no S <= 8 reaches it.
int choose_slices(double maxA, double maxB, int kp, double sigma, double gain = 1.0)
{
    int ea = 0, eb = 0;
    if (maxA > 0.0) std::frexp(maxA, &ea);
    if (maxB > 0.0) std::frexp(maxB, &eb);
    ea += 1;
    eb += 1;
    for (int S = 4; S <= S_MAX; ++S) {
        const double bound = std::ldexp(1.0, ea + eb - 7 * S) * kp * (S + 1) / 4.0;
        if (gain * bound / (sigma * sigma) <= 0.5e-12) return S;
    }
    return 0;
}

int read_max(const double *X, int64_t ldx, int rows, int cols, unsigned long long *dbuf,
             double &out, cudaStream_t s)
{
    out = 0.0;
    if (rows == 0 || cols == 0) return QMLG_OK;
    cudaError_t e = cudaMemsetAsync(dbuf, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    const int64_t total = (int64_t)rows * cols;
    const int blocks = (int)std::min<int64_t>(qmlg::ceil_div(total, 256), 1216);
    max_abs_kernel<<<blocks, 256, 0, s>>>(X, ldx, rows, cols, dbuf);
    qmlg::count_launches(1);
    unsigned long long h = 0;
    const int st = qmlg::read_back(&h, dbuf, sizeof(h), s);
    if (st != QMLG_OK) return st;
    std::memcpy(&out, &h, sizeof(out));
    return QMLG_OK;
}

}  // namespace

namespace qmlg {

int slice_rows(const double *A, int64_t lda, int r0, int nrows, int c0, int kw, int kp, int rpad,
               int slices, __nv_bfloat16 *digits, int *expo, const int *d_info, cudaStream_t s,
               double *norms)
{
    if (slices < 1 || slices > S_MAX || kp % KC != 0 || kw > kp || nrows > rpad) return QMLG_E_ARG;
    // Tiles read digit rows below ceil128(nrows) only: rows up to there are written
    // (zeros past nrows), the rest of the buffer is left as it is.
    const int rows = std::min(rpad, (int)ceil_div(nrows, 128) * 128);
    if (rows == 0) return QMLG_OK;
    slice_rows_kernel<<<(unsigned)ceil_div((int64_t)rows * 32, 256), 256, 0, s>>>(
        A, lda, r0, nrows, c0, kw, kp, rpad, slices, digits, expo, norms, d_info);
    count_launches(1);
    return check_launch();
}

int emu_tc_update(double *C, int64_t ldc, int jbase, int jend, int ibase, int iend,
                  const __nv_bfloat16 *digits, const int *expo, int kp, int rpad, int slices,
                  int a_row0, int b_row0, int lower, int *d_err, cudaStream_t s, int max_ctas)
{
    if (jend <= jbase || iend <= ibase) return QMLG_OK;
    if (slices < 1 || slices > S_MAX || kp % KC != 0 || kp / KC > 8) return QMLG_E_ARG;
    CUtensorMap mA, mB;
    int st = make_plane_map(&mA, digits, kp, rpad, slices, TM);
    if (st == QMLG_OK) st = make_plane_map(&mB, digits, kp, rpad, slices, Shape<kSyrk>::TN);
    if (st != QMLG_OK) return st;
    set_smem_attrs();
    TileArgs a{};
    a.ntiles = count_tiles(jbase, jend, ibase, iend, lower, Shape<kSyrk>::TN, a.tj);
    if (a.ntiles == 0) return QMLG_OK;
    a.C = C;
    a.ldc = ldc;
    a.jbase = jbase;
    a.jend = jend;
    a.ibase = ibase;
    a.iend = iend;
    a.a_row0 = a_row0;
    a.b_row0 = b_row0;
    a.kchunks = kp / KC;
    a.slices = slices;
    a.expA = expo;
    a.expB = expo;
    a.lower = lower;
    a.err = d_err;
    // max_ctas > 0: persistent grid of at most that many CTAs (leaves SMs free for
    // work on another stream); max_ctas < 0: one CTA per tile; 0: the thread default
    int grid = tile_grid(a.ntiles);
    if (max_ctas > 0) grid = std::min(a.ntiles, max_ctas);
    if (max_ctas < 0) grid = a.ntiles;
    emu_tc_kernel<kSyrk><<<grid, THREADS, SMEM_BYTES, s>>>(mA, mB, a);
    count_launches(1);
    return check_launch();
}

int tc_sm_count() { return sm_count(); }

}  // namespace qmlg

// ------------------------------------------------------------------ C ABI --

namespace {

struct GaussPlan {
    int kp, rpa, rpb;
};

void plan_gauss(qmlg::WorkspacePlan &p, int na, int nb, int d, bool share_b, bool predict)
{
    const int kp = feature_pad(d), rpa = rows_pad(na), rpb = rows_pad(nb);
    p.add<__nv_bfloat16>((size_t)S_MAX * rpa * kp);
    p.add<int>((size_t)rpa);
    p.add<double>((size_t)rpa);
    if (!share_b) {
        p.add<__nv_bfloat16>((size_t)S_MAX * rpb * kp);
        p.add<int>((size_t)rpb);
        p.add<double>((size_t)rpb);
    }
    if (predict) p.add<double>((size_t)qmlg::ceil_div(na < 1 ? 1 : na, TM) * (size_t)nb);
    p.add<unsigned long long>(2);
    p.add<int>(4);
}

struct GaussBufs {
    __nv_bfloat16 *dA = nullptr, *dB = nullptr;
    int *eA = nullptr, *eB = nullptr;
    double *nA = nullptr, *nB = nullptr, *partial = nullptr;
    unsigned long long *maxbuf = nullptr;
    int *err = nullptr;
};

bool take_gauss(qmlg::Workspace &ws, int na, int nb, int d, bool share_b, bool predict,
                GaussBufs &b)
{
    const int kp = feature_pad(d), rpa = rows_pad(na), rpb = rows_pad(nb);
    b.dA = ws.take<__nv_bfloat16>((size_t)S_MAX * rpa * kp);
    b.eA = ws.take<int>((size_t)rpa);
    b.nA = ws.take<double>((size_t)rpa);
    if (share_b) {
        b.dB = b.dA;
        b.eB = b.eA;
        b.nB = b.nA;
    } else {
        b.dB = ws.take<__nv_bfloat16>((size_t)S_MAX * rpb * kp);
        b.eB = ws.take<int>((size_t)rpb);
        b.nB = ws.take<double>((size_t)rpb);
    }
    if (predict) b.partial = ws.take<double>((size_t)qmlg::ceil_div(na, TM) * (size_t)nb);
    b.maxbuf = ws.take<unsigned long long>(2);
    b.err = ws.take<int>(4);
    return b.dA && b.eA && b.nA && b.dB && b.eB && b.nB && b.maxbuf && b.err &&
           (!predict || b.partial);
}

// Slices A (and B), picks S; returns S, 0 when the bound cannot be met.
int prepare_gauss(const double *A, int64_t lda, int na, const double *B, int64_t ldb, int nb,
                  int d, double sigma, bool share_b, GaussBufs &b, int &S, cudaStream_t s,
                  double gain = 1.0)
{
    const int kp = feature_pad(d), rpa = rows_pad(na), rpb = rows_pad(nb);
    double ma = 0.0, mb = 0.0;
    int st = read_max(A, lda, na, d, b.maxbuf, ma, s);
    if (st == QMLG_OK && !share_b) st = read_max(B, ldb, nb, d, b.maxbuf, mb, s);
    if (st != QMLG_OK) return st;
    if (share_b) mb = ma;
    if (!std::isfinite(ma) || !std::isfinite(mb)) {
        S = 0;
        return QMLG_OK;
    }
    S = choose_slices(ma, mb, kp, sigma, gain);
    if (S == 0) return QMLG_OK;
    cudaError_t e = cudaMemsetAsync(b.err, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    st = qmlg::slice_rows(A, lda, 0, na, 0, d, kp, rpa, S, b.dA, b.eA, nullptr, s, b.nA);
    if (st == QMLG_OK && !share_b)
        st = qmlg::slice_rows(B, ldb, 0, nb, 0, d, kp, rpb, S, b.dB, b.eB, nullptr, s, b.nB);
    return st;
}

int launch_gauss(int mode, const GaussBufs &b, int na, int nb, int d, int S, double sigma,
                 double *K, int64_t ldk, bool sym, double diag_shift, const double *alpha,
                 double *yhat, cudaStream_t s, int order = 0)
{
    const int kp = feature_pad(d), rpa = rows_pad(na), rpb = rows_pad(nb);
    CUtensorMap mA, mB;
    int st = make_plane_map(&mA, b.dA, kp, rpa, S, TM);
    const int TNm = mode == kPredict ? Shape<kPredict>::TN : Shape<kKernelMatrix>::TN;
    static_assert(Shape<kLinear>::TN == Shape<kKernelMatrix>::TN &&
                      Shape<kMatern>::TN == Shape<kKernelMatrix>::TN, "kernel-matrix tiles");
    if (st == QMLG_OK) st = make_plane_map(&mB, b.dB, kp, rpb, S, TNm);
    if (st != QMLG_OK) return st;
    set_smem_attrs();
    TileArgs a{};
    a.ntiles = count_tiles(0, na, 0, nb, sym ? 1 : 0, TNm, a.tj);
    a.C = K;
    a.ldc = ldk;
    a.jbase = 0;
    a.jend = na;
    a.ibase = 0;
    a.iend = nb;
    a.kchunks = kp / KC;
    a.slices = S;
    a.expA = b.eA;
    a.expB = b.eB;
    a.lower = sym ? 1 : 0;
    a.err = b.err;
    a.normA = b.nA;
    a.normB = b.nB;
    a.scale = -0.5 / (sigma * sigma);
    a.diag_shift = diag_shift;
    a.alpha = alpha;
    a.partial = b.partial;
    if (mode == kMatern) {
        a.scale = 1.0;
        a.order = order;
        a.s1 = -std::sqrt(2.0 * order + 1.0) / sigma;
        a.s2 = 5.0 / (3.0 * sigma * sigma);
    }
    const int grid = tile_grid(a.ntiles);
    if (mode == kKernelMatrix)
        emu_tc_kernel<kKernelMatrix><<<grid, THREADS, SMEM_BYTES, s>>>(mA, mB, a);
    else if (mode == kLinear)
        emu_tc_kernel<kLinear><<<grid, THREADS, SMEM_BYTES, s>>>(mA, mB, a);
    else if (mode == kMatern)
        emu_tc_kernel<kMatern><<<grid, THREADS, SMEM_BYTES, s>>>(mA, mB, a);
    else
        emu_tc_kernel<kPredict><<<grid, THREADS, SMEM_BYTES, s>>>(mA, mB, a);
    qmlg::count_launches(1);
    st = qmlg::check_launch();
    if (st == QMLG_OK && mode == kPredict) {
        reduce_partial_rows_kernel<<<(int)qmlg::ceil_div(nb, 256), 256, 0, s>>>(
            b.partial, (int)qmlg::ceil_div(na, TM), nb, yhat);
        qmlg::count_launches(1);
        st = qmlg::check_launch();
    }
    if (st == QMLG_OK) st = qmlg::read_device_flag(b.err, s);
    return st;
}

}  // namespace

extern "C" size_t qmlg_gaussian_kernel_emulated_workspace_size(int na, int nb, int d, int flags)
{
    qmlg::WorkspacePlan p;
    plan_gauss(p, na, nb, d, (flags & QMLG_KERNEL_SYMMETRIC) != 0, false);
    return p.total();
}

extern "C" int qmlg_gaussian_kernel_emulated(const double *A, int64_t lda, int na, const double *B,
                                             int64_t ldb, int nb, int d, double sigma, double *K,
                                             int64_t ldk, int flags, double diag_shift,
                                             void *workspace, size_t ws_bytes, void *stream)
{
    const bool sym = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (na < 0 || nb < 0 || d < 0 || !(sigma > 0.0) || !std::isfinite(sigma)) return QMLG_E_ARG;
    if ((na > 0 && (A == nullptr || lda < d)) || (nb > 0 && (B == nullptr || ldb < d)))
        return QMLG_E_ARG;
    if (K == nullptr || ldk < na) return QMLG_E_ARG;
    if (sym && (na != nb || A != B || lda != ldb)) return QMLG_E_ARG;
    if (na == 0 || nb == 0) return QMLG_OK;
    if (ws_bytes < qmlg_gaussian_kernel_emulated_workspace_size(na, nb, d, flags))
        return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    GaussBufs b;
    if (!take_gauss(ws, na, nb, d, sym, false, b)) return QMLG_E_WORKSPACE;
    int S = 0;
    int st = prepare_gauss(A, lda, na, B, ldb, nb, d, sigma, sym, b, S, s);
    if (st != QMLG_OK) return st;
    if (S == 0)  // sigma too small for the digit bound: the FP64 kernel
        return qmlg_gaussian_kernel(A, lda, na, B, ldb, nb, d, sigma, K, ldk, flags, diag_shift,
                                    stream);
    return launch_gauss(kKernelMatrix, b, na, nb, d, S, sigma, K, ldk, sym, diag_shift, nullptr,
                        nullptr, s);
}

extern "C" size_t qmlg_linear_kernel_emulated_workspace_size(int na, int nb, int d, int flags)
{
    return qmlg_gaussian_kernel_emulated_workspace_size(na, nb, d, flags);
}

// The linear kernel on the Gaussian tiles: every row sliced into S_MAX digit planes
// (the most the tiles hold), the merged integer dot product scaled to K once.
// |K - A B^T| <= 2^(eA + eB - 56) * kp * 9/4 entry by entry, 2^eA > max|a_j|,
// 2^eB > max|b_i| of the two rows.  Non-finite input takes the FP64 kernel.
extern "C" int qmlg_linear_kernel_emulated(const double *A, int64_t lda, int na, const double *B,
                                           int64_t ldb, int nb, int d, double *K, int64_t ldk,
                                           int flags, double diag_shift, void *workspace,
                                           size_t ws_bytes, void *stream)
{
    const bool sym = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (na < 0 || nb < 0 || d < 0) return QMLG_E_ARG;
    if ((na > 0 && (A == nullptr || lda < d)) || (nb > 0 && (B == nullptr || ldb < d)))
        return QMLG_E_ARG;
    if (K == nullptr || ldk < na) return QMLG_E_ARG;
    if (sym && (na != nb || A != B || lda != ldb)) return QMLG_E_ARG;
    if (na == 0 || nb == 0) return QMLG_OK;
    if (ws_bytes < qmlg_linear_kernel_emulated_workspace_size(na, nb, d, flags))
        return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    GaussBufs b;
    if (!take_gauss(ws, na, nb, d, sym, false, b)) return QMLG_E_WORKSPACE;
    double ma = 0.0, mb = 0.0;
    int st = read_max(A, lda, na, d, b.maxbuf, ma, s);
    if (st == QMLG_OK && !sym) st = read_max(B, ldb, nb, d, b.maxbuf, mb, s);
    if (st != QMLG_OK) return st;
    if (sym) mb = ma;
    if (!std::isfinite(ma) || !std::isfinite(mb))
        return qmlg_linear_kernel(A, lda, na, B, ldb, nb, d, K, ldk, flags, diag_shift, stream);
    const int kp = feature_pad(d), rpa = rows_pad(na), rpb = rows_pad(nb);
    cudaError_t e = cudaMemsetAsync(b.err, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    st = qmlg::slice_rows(A, lda, 0, na, 0, d, kp, rpa, S_MAX, b.dA, b.eA, nullptr, s, b.nA);
    if (st == QMLG_OK && !sym)
        st = qmlg::slice_rows(B, ldb, 0, nb, 0, d, kp, rpb, S_MAX, b.dB, b.eB, nullptr, s, b.nB);
    if (st != QMLG_OK) return st;
    return launch_gauss(kLinear, b, na, nb, d, S_MAX, 1.0, K, ldk, sym, diag_shift, nullptr,
                        nullptr, s);
}

extern "C" size_t qmlg_matern_kernel_l2_emulated_workspace_size(int na, int nb, int d, int flags)
{
    return qmlg_gaussian_kernel_emulated_workspace_size(na, nb, d, flags);
}

// Matern orders 1 and 2 on the Gaussian tiles.  Both are flat at d = 0, so the error
// of d^2 passes into K like the Gaussian's: |dK|/K <= 1.5 |d(d^2)| / sigma^2 (order
// 1; 5/6 for order 2).  The digit count is chosen with three times the Gaussian's
// margin on |d(d^2)| / sigma^2, which keeps |dK|/K below 0.25e-12; where no count
// meets it, and for order 0 (whose slope at d = 0 is not 0), the FP64 kernel runs.
extern "C" int qmlg_matern_kernel_l2_emulated(const double *A, int64_t lda, int na, const double *B,
                                              int64_t ldb, int nb, int d, double sigma, int order,
                                              double *K, int64_t ldk, int flags, double diag_shift,
                                              void *workspace, size_t ws_bytes, void *stream)
{
    const bool sym = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (na < 0 || nb < 0 || d < 0 || !(sigma > 0.0) || !std::isfinite(sigma)) return QMLG_E_ARG;
    if (order < 0 || order > 2) return QMLG_E_ARG;
    if ((na > 0 && (A == nullptr || lda < d)) || (nb > 0 && (B == nullptr || ldb < d)))
        return QMLG_E_ARG;
    if (K == nullptr || ldk < na) return QMLG_E_ARG;
    if (sym && (na != nb || A != B || lda != ldb)) return QMLG_E_ARG;
    if (na == 0 || nb == 0) return QMLG_OK;
    if (order == 0)
        return qmlg_matern_kernel_l2(A, lda, na, B, ldb, nb, d, sigma, order, K, ldk, flags,
                                     diag_shift, stream);
    if (ws_bytes < qmlg_matern_kernel_l2_emulated_workspace_size(na, nb, d, flags))
        return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    GaussBufs b;
    if (!take_gauss(ws, na, nb, d, sym, false, b)) return QMLG_E_WORKSPACE;
    int S = 0;
    int st = prepare_gauss(A, lda, na, B, ldb, nb, d, sigma, sym, b, S, s, 3.0);
    if (st != QMLG_OK) return st;
    if (S == 0)
        return qmlg_matern_kernel_l2(A, lda, na, B, ldb, nb, d, sigma, order, K, ldk, flags,
                                     diag_shift, stream);
    return launch_gauss(kMatern, b, na, nb, d, S, sigma, K, ldk, sym, diag_shift, nullptr, nullptr,
                        s, order);
}

extern "C" size_t qmlg_predict_emulated_workspace_size(int ntrain, int ntest, int d)
{
    qmlg::WorkspacePlan p;
    plan_gauss(p, ntrain, ntest, d, false, true);
    p.add<char>(qmlg_predict_workspace_size(ntrain, ntest));  // FP64 fallback
    return p.total();
}

extern "C" int qmlg_predict_emulated(const double *Xtrain, int64_t ldtrain, int ntrain,
                                     const double *Xtest, int64_t ldtest, int ntest, int d,
                                     double sigma, const double *alpha, double *yhat,
                                     void *workspace, size_t ws_bytes, void *stream)
{
    if (ntrain < 0 || ntest < 0 || d < 0 || !(sigma > 0.0) || !std::isfinite(sigma))
        return QMLG_E_ARG;
    if ((ntrain > 0 && (Xtrain == nullptr || ldtrain < d || alpha == nullptr)) ||
        (ntest > 0 && (Xtest == nullptr || ldtest < d || yhat == nullptr)))
        return QMLG_E_ARG;
    if (ntest == 0) return QMLG_OK;
    cudaStream_t s = qmlg::as_stream(stream);
    if (ntrain == 0) {
        cudaError_t e = cudaMemsetAsync(yhat, 0, sizeof(double) * (size_t)ntest, s);
        return e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
    }
    if (ws_bytes < qmlg_predict_emulated_workspace_size(ntrain, ntest, d)) return QMLG_E_WORKSPACE;
    qmlg::Workspace ws(workspace, ws_bytes);
    GaussBufs b;
    if (!take_gauss(ws, ntrain, ntest, d, false, true, b)) return QMLG_E_WORKSPACE;
    int S = 0;
    int st = prepare_gauss(Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, sigma, false, b, S, s);
    if (st != QMLG_OK) return st;
    if (S == 0) {
        const size_t fb = qmlg_predict_workspace_size(ntrain, ntest);
        char *p = ws.take<char>(fb);
        if (p == nullptr) return QMLG_E_WORKSPACE;
        return qmlg_predict_fused(QMLG_KIND_GAUSSIAN, Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest,
                                  d, sigma, alpha, yhat, p, fb, stream);
    }
    return launch_gauss(kPredict, b, ntrain, ntest, d, S, sigma, nullptr, 0, false, 0.0, alpha,
                        yhat, s);
}

extern "C" size_t qmlg_syrk_emulated_workspace_size(int n, int k)
{
    qmlg::WorkspacePlan p;
    const int kp = feature_pad(k), rp = rows_pad(n);
    p.add<__nv_bfloat16>((size_t)S_MAX * rp * kp);
    p.add<int>((size_t)rp);
    p.add<int>(4);
    return p.total();
}

extern "C" int qmlg_syrk_emulated(double *C, int64_t ldc, int n, const double *P, int64_t ldp,
                                  int k, void *workspace, size_t ws_bytes, void *stream)
{
    if (n < 0 || k < 0 || k > 512 || ldc < n || ldp < k) return QMLG_E_ARG;
    if (n == 0 || k == 0) return QMLG_OK;
    if (C == nullptr || P == nullptr) return QMLG_E_ARG;
    if (ws_bytes < qmlg_syrk_emulated_workspace_size(n, k)) return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    const int kp = feature_pad(k), rp = rows_pad(n);
    __nv_bfloat16 *dig = ws.take<__nv_bfloat16>((size_t)S_MAX * rp * kp);
    int *ex = ws.take<int>((size_t)rp);
    int *err = ws.take<int>(4);
    if (dig == nullptr || ex == nullptr || err == nullptr) return QMLG_E_WORKSPACE;
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    int st = qmlg::slice_rows(P, ldp, 0, n, 0, k, kp, rp, S_MAX, dig, ex, nullptr, s);
    if (st == QMLG_OK)
        st = qmlg::emu_tc_update(C, ldc, 0, n, 0, n, dig, ex, kp, rp, S_MAX, 0, 0, 1, err, s, 0);
    return st;
}

// ------------------------------------------------ asynchronous prediction --

namespace {

// Sets *flag when 8 digit planes cannot keep the kernel within 1e-12 for the
// maxima in maxbits[0..1] (the host-side choose_slices bound, evaluated on device).
__global__ void bound_check_kernel(const unsigned long long *__restrict__ maxbits, int kp,
                                   double sigma, int *__restrict__ flag)
{
    const double ma = __longlong_as_double((long long)maxbits[0]);
    const double mb = __longlong_as_double((long long)maxbits[1]);
    if (!isfinite(ma) || !isfinite(mb)) {
        atomicOr(flag, 8);
        return;
    }
    int ea = 0, eb = 0;
    if (ma > 0.0) frexp(ma, &ea);
    if (mb > 0.0) frexp(mb, &eb);
    const double bound = ldexp(1.0, ea + 1 + eb + 1 - 7 * S_MAX) * kp * (S_MAX + 1) / 4.0;
    if (bound / (sigma * sigma) > 0.5e-12) atomicOr(flag, 8);
}

}  // namespace

extern "C" int qmlg_predict_emulated_async(const double *Xtrain, int64_t ldtrain, int ntrain,
                                           const double *Xtest, int64_t ldtest, int ntest, int d,
                                           double sigma, const double *alpha, double *yhat,
                                           int *d_flag, void *workspace, size_t ws_bytes,
                                           void *stream)
{
    if (ntrain < 0 || ntest < 0 || d < 0 || !(sigma > 0.0) || !std::isfinite(sigma))
        return QMLG_E_ARG;
    if ((ntrain > 0 && (Xtrain == nullptr || ldtrain < d || alpha == nullptr)) ||
        (ntest > 0 && (Xtest == nullptr || ldtest < d || yhat == nullptr)) || d_flag == nullptr)
        return QMLG_E_ARG;
    if (ntest == 0) return QMLG_OK;
    cudaStream_t s = qmlg::as_stream(stream);
    if (ntrain == 0) {
        cudaError_t e = cudaMemsetAsync(yhat, 0, sizeof(double) * (size_t)ntest, s);
        return e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
    }
    if (ws_bytes < qmlg_predict_emulated_workspace_size(ntrain, ntest, d)) return QMLG_E_WORKSPACE;
    qmlg::Workspace ws(workspace, ws_bytes);
    GaussBufs b;
    if (!take_gauss(ws, ntrain, ntest, d, false, true, b)) return QMLG_E_WORKSPACE;
    b.err = d_flag;  // timeouts and the accuracy bound share the caller's flag
    const int kp = feature_pad(d), rpa = rows_pad(ntrain), rpb = rows_pad(ntest);
    cudaError_t e = cudaMemsetAsync(b.maxbuf, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    const int ba = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)ntrain * d, 256), 1216);
    const int bb = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)ntest * d, 256), 1216);
    max_abs_kernel<<<ba, 256, 0, s>>>(Xtrain, ldtrain, ntrain, d, b.maxbuf);
    max_abs_kernel<<<bb, 256, 0, s>>>(Xtest, ldtest, ntest, d, b.maxbuf + 1);
    bound_check_kernel<<<1, 1, 0, s>>>(b.maxbuf, kp, sigma, d_flag);
    qmlg::count_launches(3);
    int st = qmlg::slice_rows(Xtrain, ldtrain, 0, ntrain, 0, d, kp, rpa, S_MAX, b.dA, b.eA, nullptr,
                              s, b.nA);
    if (st == QMLG_OK)
        st = qmlg::slice_rows(Xtest, ldtest, 0, ntest, 0, d, kp, rpb, S_MAX, b.dB, b.eB, nullptr, s,
                              b.nB);
    if (st != QMLG_OK) return st;
    // launch without the trailing flag read (launch_gauss reads it synchronously)
    CUtensorMap mA, mB;
    st = make_plane_map(&mA, b.dA, kp, rpa, S_MAX, TM);
    if (st == QMLG_OK) st = make_plane_map(&mB, b.dB, kp, rpb, S_MAX, Shape<kPredict>::TN);
    if (st != QMLG_OK) return st;
    set_smem_attrs();
    TileArgs a{};
    a.ntiles = count_tiles(0, ntrain, 0, ntest, 0, Shape<kPredict>::TN, a.tj);
    a.jend = ntrain;
    a.iend = ntest;
    a.kchunks = kp / KC;
    a.slices = S_MAX;
    a.expA = b.eA;
    a.expB = b.eB;
    a.err = d_flag;
    a.normA = b.nA;
    a.normB = b.nB;
    a.scale = -0.5 / (sigma * sigma);
    a.alpha = alpha;
    a.partial = b.partial;
    emu_tc_kernel<kPredict><<<tile_grid(a.ntiles), THREADS, SMEM_BYTES, s>>>(mA, mB, a);
    reduce_partial_rows_kernel<<<(int)qmlg::ceil_div(ntest, 256), 256, 0, s>>>(
        b.partial, (int)qmlg::ceil_div(ntrain, TM), ntest, yhat);
    qmlg::count_launches(2);
    return qmlg::check_launch();
}

// Capture-safe Gaussian kernel: 8 digit planes always, no host synchronisation;
// the accuracy bound (and any bounded-wait timeout) is reported in *d_flag.
extern "C" int qmlg_gaussian_kernel_emulated_async(const double *A, int64_t lda, int na,
                                                   const double *B, int64_t ldb, int nb, int d,
                                                   double sigma, double *K, int64_t ldk, int flags,
                                                   double diag_shift, int *d_flag, void *workspace,
                                                   size_t ws_bytes, void *stream)
{
    const bool sym = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (na < 0 || nb < 0 || d < 0 || !(sigma > 0.0) || !std::isfinite(sigma) || d_flag == nullptr)
        return QMLG_E_ARG;
    if ((na > 0 && (A == nullptr || lda < d)) || (nb > 0 && (B == nullptr || ldb < d)))
        return QMLG_E_ARG;
    if (K == nullptr || ldk < na) return QMLG_E_ARG;
    if (sym && (na != nb || A != B || lda != ldb)) return QMLG_E_ARG;
    if (na == 0 || nb == 0) return QMLG_OK;
    if (ws_bytes < qmlg_gaussian_kernel_emulated_workspace_size(na, nb, d, flags))
        return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    GaussBufs b;
    if (!take_gauss(ws, na, nb, d, sym, false, b)) return QMLG_E_WORKSPACE;
    b.err = d_flag;
    const int kp = feature_pad(d), rpa = rows_pad(na), rpb = rows_pad(nb);
    cudaError_t e = cudaMemsetAsync(b.maxbuf, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    const int ba = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)na * d, 256), 1216);
    const int bb = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)nb * d, 256), 1216);
    max_abs_kernel<<<ba, 256, 0, s>>>(A, lda, na, d, b.maxbuf);
    max_abs_kernel<<<bb, 256, 0, s>>>(B, ldb, nb, d, b.maxbuf + 1);
    bound_check_kernel<<<1, 1, 0, s>>>(b.maxbuf, kp, sigma, d_flag);
    qmlg::count_launches(3);
    int st = qmlg::slice_rows(A, lda, 0, na, 0, d, kp, rpa, S_MAX, b.dA, b.eA, nullptr, s, b.nA);
    if (st == QMLG_OK && !sym)
        st = qmlg::slice_rows(B, ldb, 0, nb, 0, d, kp, rpb, S_MAX, b.dB, b.eB, nullptr, s, b.nB);
    if (st != QMLG_OK) return st;
    CUtensorMap mA, mB;
    st = make_plane_map(&mA, b.dA, kp, rpa, S_MAX, TM);
    if (st == QMLG_OK) st = make_plane_map(&mB, b.dB, kp, rpb, S_MAX, Shape<kKernelMatrix>::TN);
    if (st != QMLG_OK) return st;
    set_smem_attrs();
    TileArgs a{};
    a.ntiles = count_tiles(0, na, 0, nb, sym ? 1 : 0, Shape<kKernelMatrix>::TN, a.tj);
    a.C = K;
    a.ldc = ldk;
    a.jend = na;
    a.iend = nb;
    a.kchunks = kp / KC;
    a.slices = S_MAX;
    a.expA = b.eA;
    a.expB = b.eB;
    a.lower = sym ? 1 : 0;
    a.err = d_flag;
    a.normA = b.nA;
    a.normB = b.nB;
    a.scale = -0.5 / (sigma * sigma);
    a.diag_shift = diag_shift;
    emu_tc_kernel<kKernelMatrix><<<tile_grid(a.ntiles), THREADS, SMEM_BYTES, s>>>(mA, mB, a);
    qmlg::count_launches(1);
    return qmlg::check_launch();
}

// -------------------------------------------------------- grouped launches --

namespace {

// The 1e-12 bound of a symmetric Gaussian K from the one max |x| of its rows.
__global__ void bound_check_sym_kernel(const unsigned long long *__restrict__ maxbits, int kp,
                                       double sigma, int *__restrict__ flag)
{
    const double m = __longlong_as_double((long long)maxbits[0]);
    if (!isfinite(m)) {
        atomicOr(flag, 8);
        return;
    }
    int e = 0;
    if (m > 0.0) frexp(m, &e);
    const double bound = ldexp(1.0, 2 * (e + 1) - 7 * S_MAX) * kp * (S_MAX + 1) / 4.0;
    if (bound / (sigma * sigma) > 0.5e-12) atomicOr(flag, 8);
}

void set_group_smem_attrs()
{
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(emu_tc_group_kernel<kSyrk>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        cudaFuncSetAttribute(emu_tc_group_kernel<kSyrk, 32>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        cudaFuncSetAttribute(emu_tc_group_kernel<kKernelMatrix>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    });
}

// Launches the items' tiles in groups of at most kMaxGroup problems.
template <int MODE, int TN = Shape<MODE>::TN>
int launch_group(const qmlg::GroupItem *items, int count, const CUtensorMap &mA,
                 const CUtensorMap &mB, const TileArgs &base, cudaStream_t s)
{
    set_group_smem_attrs();
    static TileGroup grp;  // host staging of the kernel parameter (copied at launch)
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    for (int first = 0; first < count; first += kMaxGroup) {
        const int m = std::min(kMaxGroup, count - first);
        int total = 0;
        grp.count = m;
        for (int k = 0; k < m; ++k) {
            const qmlg::GroupItem &it = items[first + k];
            GroupEntry &e = grp.e[k];
            int tj = 0;
            const int nt = (it.jend > it.jbase && it.iend > it.ibase)
                               ? count_tiles(it.jbase, it.jend, it.ibase, it.iend, 1, TN, tj)
                               : 0;
            e.C = it.C;
            e.ldc = it.ldc;
            e.scale = it.scale;
            e.jbase = it.jbase;
            e.jend = it.jend;
            e.ibase = it.ibase;
            e.iend = it.iend;
            e.a_row0 = it.a_row0;
            e.b_row0 = it.b_row0;
            e.tj = tj;
            e.tile_base = total;
            total += nt;
        }
        if (total == 0) continue;
        TileArgs a = base;
        a.ntiles = total;
        emu_tc_group_kernel<MODE, TN><<<tile_grid(total), THREADS, SMEM_BYTES, s>>>(mA, mB, a, grp);
        qmlg::count_launches(1);
        const int st = qmlg::check_launch();
        if (st != QMLG_OK) return st;
    }
    return QMLG_OK;
}

}  // namespace

namespace qmlg {

int emu_tc_group_update(const GroupItem *items, int count, const __nv_bfloat16 *digits,
                        const int *expo, int kp, int rows_total, int slices, int *d_err,
                        cudaStream_t s, int tile_cols)
{
    if (count <= 0) return QMLG_OK;
    if (items == nullptr || slices < 1 || slices > S_MAX || kp % KC != 0 || kp / KC > 8 ||
        rows_total < 1 || (tile_cols != 32 && tile_cols != 64))
        return QMLG_E_ARG;
    CUtensorMap mA, mB;
    int st = make_plane_map(&mA, digits, kp, rows_total, slices, TM);
    if (st == QMLG_OK) st = make_plane_map(&mB, digits, kp, rows_total, slices, tile_cols);
    if (st != QMLG_OK) return st;
    TileArgs a{};
    a.kchunks = kp / KC;
    a.slices = slices;
    a.expA = expo;
    a.expB = expo;
    a.lower = 1;
    a.err = d_err;
    return tile_cols == 32 ? launch_group<kSyrk, 32>(items, count, mA, mB, a, s)
                           : launch_group<kSyrk, 64>(items, count, mA, mB, a, s);
}

int slice_rows_group(const SliceItem *items, int count, int kp, int rows_total, int slices,
                     __nv_bfloat16 *digits, int *expo, cudaStream_t s)
{
    if (count <= 0) return QMLG_OK;
    if (items == nullptr || slices < 1 || slices > S_MAX || kp % KC != 0 || rows_total < 1)
        return QMLG_E_ARG;
    static SliceGroup g;  // host staging of the kernel parameter (copied at launch)
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    for (int first = 0; first < count; first += kMaxGroup) {
        const int m = std::min(kMaxGroup, count - first);
        int warps = 0, used = 0;
        for (int k = 0; k < m; ++k) {
            const SliceItem &it = items[first + k];
            if (it.nrows <= 0) continue;
            if (it.kw > kp || it.row0 < 0 || it.row0 + plane_rows(it.nrows) > rows_total)
                return QMLG_E_ARG;
            SliceEntry &e = g.e[used++];
            e.A = it.A;
            e.lda = it.lda;
            e.r0 = it.r0;
            e.nrows = it.nrows;
            e.c0 = it.c0;
            e.kw = it.kw;
            e.row0 = it.row0;
            e.warp_base = warps;
            e.info = it.info;
            warps += plane_rows(it.nrows);
        }
        if (used == 0) continue;
        g.count = used;
        slice_rows_group_kernel<<<(unsigned)ceil_div((int64_t)warps * 32, 256), 256, 0, s>>>(
            g, kp, rows_total, slices, digits, expo);
        count_launches(1);
        const int st = check_launch();
        if (st != QMLG_OK) return st;
    }
    return QMLG_OK;
}

int gauss_group_kernel_matrix(const GaussItem *items, int count, int d, __nv_bfloat16 *digits,
                              int *expo, double *norms, unsigned long long *maxbuf,
                              int rows_total, int *d_err, cudaStream_t s)
{
    if (count <= 0) return QMLG_OK;
    if (items == nullptr || d < 1 || rows_total < 1) return QMLG_E_ARG;
    const int kp = feature_pad(d);
    std::vector<GroupItem> g((size_t)count);
    for (int k = 0; k < count; ++k) {
        const GaussItem &it = items[k];
        if (it.n < 0 || it.row0 < 0 || it.row0 + rows_pad(it.n) > rows_total || it.ldx < d ||
            !(it.sigma > 0.0))
            return QMLG_E_ARG;
        if (it.n == 0) {
            g[(size_t)k] = GroupItem{it.K, it.ldk, 0, 0, 0, 0, it.row0, it.row0, 0.0};
            continue;
        }
        // the plane count is fixed at 8; a K that the bound says may be less accurate
        // than 1e-12 is still formed and flagged (8) for the caller
        cudaError_t e = cudaMemsetAsync(maxbuf + k, 0, sizeof(unsigned long long), s);
        if (e != cudaSuccess) return set_cuda_error(e);
        const int64_t total = (int64_t)it.n * d;
        const int blocks = (int)std::min<int64_t>(ceil_div(total, 256), 1216);
        max_abs_kernel<<<blocks, 256, 0, s>>>(it.X, it.ldx, it.n, d, maxbuf + k);
        bound_check_sym_kernel<<<1, 1, 0, s>>>(maxbuf + k, kp, it.sigma, it.flag);
        count_launches(2);
        // rpad = rows_total keeps the planes' stride; the rows start at row0
        const int st = slice_rows(it.X, it.ldx, 0, it.n, 0, d, kp, rows_total, S_MAX,
                                  digits + (size_t)it.row0 * kp, expo + it.row0, nullptr, s,
                                  norms + it.row0);
        if (st != QMLG_OK) return st;
        g[(size_t)k] = GroupItem{it.K, it.ldk, 0, it.n, 0, it.n, it.row0, it.row0,
                                 -0.5 / (it.sigma * it.sigma)};
    }
    CUtensorMap mA, mB;
    int st = make_plane_map(&mA, digits, kp, rows_total, S_MAX, TM);
    if (st == QMLG_OK) st = make_plane_map(&mB, digits, kp, rows_total, S_MAX, Shape<kKernelMatrix>::TN);
    if (st != QMLG_OK) return st;
    TileArgs a{};
    a.kchunks = kp / KC;
    a.slices = S_MAX;
    a.expA = expo;
    a.expB = expo;
    a.normA = norms;
    a.normB = norms;
    a.lower = 1;
    a.diag_shift = 0.0;
    a.err = d_err;
    return launch_group<kKernelMatrix>(g.data(), count, mA, mB, a, s);
}

}  // namespace qmlg

extern "C" int qmlg_epilogue_exp(const double *x, double *y, int n, void *stream)
{
    if (n < 0 || (n > 0 && (x == nullptr || y == nullptr))) return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    const int blocks = (int)std::min<int64_t>(qmlg::ceil_div(n, 256), 152 * 16);
    epilogue_exp_kernel<<<blocks, 256, 0, qmlg::as_stream(stream)>>>(x, y, n);
    qmlg::count_launches(1);
    return qmlg::check_launch();
}
