// Block one-sided Jacobi on the tcgen05 tensor cores: the split-precision
// ("mixed") form of the truncated SVD of mps_apply_2q_batch.
//
// Replaces the same computation as the FP32 SIMT sweep kernel (jacobi.cu):
// TensorNetwork's split_node_full_svd (mpsim/core.py:1132-1137; LAPACK
// gesdd underneath) for the left-canonical tall jobs, whose left factor is
// U = X/S from the final columns and whose right factor is formed afterwards
// as U^H theta.
//
// Storage.  For the sweeps, X (FP32, the L factor of theta or theta) is held
// as three bf16 piece planes P0, P1, P2 per job, laid out like X, with
// x = p0 + p1 + p2 exactly (p0 = bf16(x), p1 = bf16(x - p0), p2 =
// bf16(x - p0 - p1); both subtractions are exact, and the last residual has
// at most 8 significant bits, so it is p2 itself, barring underflow).
// tc_split_kernel writes the planes before the first sweep and tc_merge_kernel
// sums them back into X after the last one; in between the visits read and
// write pieces only (12 bytes a complex element instead of 8 + 12, and the
// planes of a 32-job chi=256 call, 96 MB, mostly stay in L2).
//
// The C columns are split into blocks of 32.  A sweep visits every pair of
// blocks once (circle-method rounds, as in the SIMT form, over the L factor's
// own column order: unlike the SIMT form's, these jobs are not re-sorted by
// norm before each sweep, which measured a sweep fewer).  One visit of blocks
// (I, J), Y = [X_I X_J] (L x 64 complex), by one 256-thread CTA:
//   1. Gram:     G = Y^H Y (64 x 64 complex) on the tensor cores.  Real form:
//                rows 0..63 of the operand tile are the columns of Y as
//                interleaved (re, im) vectors of length 2L, rows 64..127 are
//                T = -i Y; D[m, q] = sum over the 2L reals of tile row m times
//                tile row q gives Re G (m < 64) and -Im G (m >= 64).  T's
//                pieces are Y's with each packed (re, im) pair turned into
//                (im, -re): a half-word swap and a sign flip.  K-major
//                operands, K = 2L in chunks of 64 reals (the six piece
//                products of order <= 2 per K step), two tile buffers so that
//                the stores of chunk c + 1 overlap the MMAs of chunk c.  Each
//                chunk accumulates into its own TMEM buffer and the chunks are
//                summed in FP32 registers with round-to-nearest: tcgen05's
//                FP32 accumulation truncates toward zero, and one accumulator
//                over all 2L reals left Gram errors of ~1e-6 |y_p||y_q|, the
//                size of the convergence tolerance, which cost sweeps.
//   2. Convergence test and rotations on G.  The off-diagonal test runs
//                first, in FP64 on the fresh Gram: a visit none of whose
//                pairs has |G_pq|^2 > tol^2 G_pp G_qq changes nothing and
//                skips the rest.  Otherwise two-sided Jacobi on G held in
//                registers, 32 disjoint pairs per step (the 32 x 32
//                inter-block pairs in 32 steps, or all 2016 pairs in 63 steps
//                on a block's first visit of a sweep), accumulating E = Q - I;
//                every pair over kInnerTol2 tol^2 rotates.  Every warp
//                computes the 32 rotations of a step (lane k: pair k, the FP32
//                parameters of rot.cuh), so a step where no pair rotates is
//                skipped by all warps alike.  Ring visits hold G as 2 x 2
//                blocks (row pair x column pair) and apply R^H B R in the
//                thread, one barrier a step; full visits hold rows w, w + 8,
//                ... and lane k's two columns and take G' = R^H G R in two
//                passes (H = G R written conjugate-transposed, then G' = H^H R;
//                G is Hermitian), two barriers a step.  E takes R with the
//                column layout in both.
//   3. Update:   Y <- Y + Y E, skipped when the visit rotated nothing.  Per
//                64 rows, the tensor cores form D1 = Y Re E and D2 = Y Im E
//                from the rows' piece tiles read as an MN-major A operand
//                (M = the 128 interleaved reals, K = the 64 visit columns)
//                times a K-major B holding Re E and Im E (N = 128); the
//                epilogue combines the two reals of a row (adjacent TMEM
//                lanes, one shuffle), adds the result to Y (summed from its
//                pieces) in FP32 with round-to-nearest and writes the new
//                pieces.  The update form keeps the truncation small: D = Y E
//                is small once the rotations are (accumulating Y Q in full
//                shrank every singular value by ~5e-5 over a chi=256 SVD).
//                The piece products are issued smallest first.
// The new squared column norms (the diagonal of Q^H G Q) go to cnrm, the
// column-norm record the SIMT form sorts by.
//
// Shared memory (96 KB + the small arrays: two CTAs per SM):
//   [0, 96K)   step 1: two tile buffers, each three 16 KB piece tiles
//              (128 rows x 128 B, 128-byte swizzle)
//   [0, 32K)   step 2: G (64 x 64 complex, columns XOR-swizzled by the row),
//              read into registers at the start
//   [32K, 64K) step 2: H^H, the first pass's output (full visits, same
//              layout); the ring visits' Q-row exchange (8 KB)
//   [64K, 96K) step 2: E = Q - I (64 x 64 complex, row-major)
//   [0, 48K)   step 3: the three B-operand pieces of E (16 KB each)
//   [48K, 96K) step 3: the three A piece tiles of 64 rows (two 8 KB M-groups
//              each), filled by cp.async
#include "rot.cuh"
#include "tc.cuh"
#include "twoq.cuh"

namespace mps {
namespace {

constexpr int TJ_T = 256;                  // threads per CTA
constexpr int TJ_BC = 32;                  // columns per block
constexpr int TJ_W = 2 * TJ_BC;            // columns per visit
constexpr uint32_t TJ_PIECE = 16384;       // 128 rows x 128 B
constexpr uint32_t TJ_GTILE = 3 * TJ_PIECE;         // one Gram tile buffer (48 KB)
constexpr uint32_t TJ_GBUF = TJ_W * TJ_W * 8;       // one 64 x 64 complex buffer (32 KB)
constexpr uint32_t TJ_HOFF = TJ_GBUF;               // H^H at 32 KB
constexpr uint32_t TJ_EOFF = 2 * TJ_GBUF;           // E at 64 KB
constexpr uint32_t TJ_AOFF = 3 * TJ_PIECE;          // the update's A tiles at 48 KB
constexpr uint32_t TJ_MGRP = 8192;                  // one 64-real M-group of an A tile
constexpr uint32_t TJ_AUX = 2 * TJ_GTILE;           // 96 KB: small arrays
constexpr uint32_t TJ_TMEM_COLS = 128;              // two 64-column Gram accumulators
constexpr int TJ_WAIT_LIMIT = 1 << 14;
// Inside a visit that has work (some pair over the tolerance by the FP64
// test), every pair whose squared cosine exceeds kInnerTol2 tol^2 rotates:
// pairs that the visit's rounding would leave just over the tolerance are
// settled now instead of bringing their blocks back a sweep later (per job
// about one sweep fewer; the convergence record keeps the FP64 test at tol).
constexpr float kInnerTol2 = 0.25f;
static_assert(TJ_EOFF + TJ_GBUF <= TJ_AUX, "E overlaps the small arrays");
static_assert(TJ_AOFF + 3 * TJ_PIECE <= TJ_AUX, "the update's A tiles overlap the small arrays");

// Cycles spent in the three steps of a visit, summed over the CTAs of every
// visit since the last reset: [0] Gram, [1] rotations on G, [2] Y <- Y + Y E,
// [3] visits, [4] visits that rotated, [5] inner steps that rotated, [6]
// pairs rotated, [7] cycles spent waiting for the blocks' previous round,
// [8] CTA lifetimes of the sweep kernel, [9] its CTAs.  Read with
// mps_tc_profile.
__device__ unsigned long long g_tj_cycles[10];

struct Aux {
    uint64_t bar[2];      // MMA completion, one per Gram tile buffer
    uint32_t tmem;
    int item, abort, skip;   // the claimed visit, the stop flag, its skip decision
    int rotated;          // some pair of this visit needs a rotation
    int col[TJ_W];        // physical column of each visit column (-1: zero padding)
    float diag[TJ_W];     // diagonal of G (squared column norms)
    cf gam[TJ_W];         // G[cP][cQ] of the 32 pairs of the next inner step (the ring
                          // visit double-buffers it: [step parity][pair])
    float cmax;           // largest squared cosine of the visit's pairs
};
constexpr size_t TJ_SMEM = TJ_AUX + sizeof(Aux) + 1024;

// Element (r, c) of a 64 x 64 complex buffer; the column is XOR-swizzled by
// the row, so that lanes reading or writing one column of different rows
// (the transposed writes of the first pass) spread over the banks.
__device__ __forceinline__ int gidx(int r, int c) { return r * TJ_W + (c ^ (r & 31)); }

__device__ __forceinline__ bool wait_mma(uint64_t* bar, unsigned& phase) {
    const bool ok = tc::mbar_wait_bounded(bar, phase, TJ_WAIT_LIMIT);
    phase ^= 1u;
    return ok;
}

// Columns x (p) and y (q) of a row times R = [[1 - tp, conj(s)], [-s, 1 - tp]]
// in the tau form of rot.cuh: x' = x - (tp x + s y), y' = y + (conj(s) x -
// tp y).  Twelve FMAs; each output starts from fma(-tp, x, x), which rounds
// x - tp x once (an explicit c = 1 - tp would round to 1 for small angles and
// inflate the norms).
__device__ __forceinline__ void rotate_cols(cf& x, cf& y, float tp, cf sg) {
    const float xr = x.x, xi = x.y, yr = y.x, yi = y.y;
    x.x = fmaf(-sg.x, yr, fmaf(sg.y, yi, fmaf(-tp, xr, xr)));
    x.y = fmaf(-sg.x, yi, fmaf(-sg.y, yr, fmaf(-tp, xi, xi)));
    y.x = fmaf(sg.x, xr, fmaf(sg.y, xi, fmaf(-tp, yr, yr)));
    y.y = fmaf(sg.x, xi, fmaf(-sg.y, xr, fmaf(-tp, yi, yi)));
}

__device__ __forceinline__ cf shfl_cf(cf v, int src) {
    return cmake(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// One step of the circle method over the 32 lanes' (top, bottom) slots:
// top of lane 0 stays, top of lane 1 <- bottom of lane 0, top of lane k <-
// top of lane k - 1 (k >= 2), bottom of lane k <- bottom of lane k + 1
// (k <= 30), bottom of lane 31 <- top of lane 31.
__device__ __forceinline__ float circle_top(float t, float b, int lane) {
    const float up = __shfl_up_sync(0xffffffffu, t, 1);
    const float b0 = __shfl_sync(0xffffffffu, b, 0);
    return lane == 0 ? t : (lane == 1 ? b0 : up);
}
__device__ __forceinline__ float circle_bottom(float t, float b, int lane) {
    const float dn = __shfl_down_sync(0xffffffffu, b, 1);
    return lane == 31 ? t : dn;
}
__device__ __forceinline__ void circle_move(cf& t, cf& b, int lane) {
    const cf nt = cmake(circle_top(t.x, b.x, lane), circle_top(t.y, b.y, lane));
    const cf nb = cmake(circle_bottom(t.x, b.x, lane), circle_bottom(t.y, b.y, lane));
    t = nt;
    b = nb;
}
// (top, bottom) of one lane packed as (x, y).
__device__ __forceinline__ void circle_move_pair(cf& tb, int lane) {
    const float nt = circle_top(tb.x, tb.y, lane), nb = circle_bottom(tb.x, tb.y, lane);
    tb = cmake(nt, nb);
}
__device__ __forceinline__ void circle_move_idx(int& t, int& b, int lane) {
    const int up = __shfl_up_sync(0xffffffffu, t, 1);
    const int b0 = __shfl_sync(0xffffffffu, b, 0);
    const int dn = __shfl_down_sync(0xffffffffu, b, 1);
    const int nt = lane == 0 ? t : (lane == 1 ? b0 : up);
    b = lane == 31 ? t : dn;
    t = nt;
}

// gamma = G[cP][cQ] of this lane's pair, written by the warp holding row cP
// (row warp + 8h of gQ).  A masked sum, not an indexed read: an index that
// depends on the lane would move the array to local memory.
__device__ __forceinline__ void publish_gamma(const cf (&gQ)[8], int warp, int cP, cf* dst) {
    cf v = cmake(0.f, 0.f);
#pragma unroll
    for (int h = 0; h < 8; ++h) {
        const float m = (warp + 8 * h == cP) ? 1.f : 0.f;
        v.x = fmaf(m, gQ[h].x, v.x);
        v.y = fmaf(m, gQ[h].y, v.y);
    }
    if (warp == (cP & 7)) *dst = v;
}

// T = -i Y on 8 packed bf16 (four (re, im) pairs, re in the low half of each
// word): (re, im) -> (im, -re).  Exact: the split is odd-symmetric.
__device__ __forceinline__ uint4 twist_packed(uint4 w) {
    const uint32_t sign = 0x80000000u;
    w.x = __byte_perm(w.x, 0, 0x1032) ^ sign;
    w.y = __byte_perm(w.y, 0, 0x1032) ^ sign;
    w.z = __byte_perm(w.z, 0, 0x1032) ^ sign;
    w.w = __byte_perm(w.w, 0, 0x1032) ^ sign;
    return w;
}

// Two reals -> their three bf16 pieces, packed in pairs (a in the low half),
// with the paired round-to-nearest conversion: the same pieces as
// tc::split3, in three conversions instead of six.
struct Pieces2 {
    uint32_t w0, w1, w2;
};
__device__ __forceinline__ Pieces2 split3x2(float a, float b) {
    const __nv_bfloat162 p0 = __floats2bfloat162_rn(a, b);
    const float2 f0 = __bfloat1622float2(p0);
    const float ra = a - f0.x, rb = b - f0.y;            // exact
    const __nv_bfloat162 p1 = __floats2bfloat162_rn(ra, rb);
    const float2 f1 = __bfloat1622float2(p1);
    const __nv_bfloat162 p2 = __floats2bfloat162_rn(ra - f1.x, rb - f1.y);
    Pieces2 r;
    r.w0 = *reinterpret_cast<const uint32_t*>(&p0);
    r.w1 = *reinterpret_cast<const uint32_t*>(&p1);
    r.w2 = *reinterpret_cast<const uint32_t*>(&p2);
    return r;
}

// 8 reals -> the 16-byte chunks of all three pieces, in buffers `stride`
// bytes apart.
__device__ __forceinline__ void put_pieces(uint8_t* base, size_t stride, uint32_t off,
                                           const float* v) {
    uint32_t w[3][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const Pieces2 q = split3x2(v[2 * e], v[2 * e + 1]);
        w[0][e] = q.w0;
        w[1][e] = q.w1;
        w[2][e] = q.w2;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
        *reinterpret_cast<uint4*>(base + i * stride + off) =
            make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

__device__ __forceinline__ float bf16_bits(uint16_t u) {
    return __uint_as_float((uint32_t)u << 16);
}

// The Gram's per-thread tasks, fixed for a visit: task t = tid + 256 h
// (0..1535) = (column p, piece i, 16-byte chunk g of the 128 bytes a piece
// column holds for 32 rows).  soff: its Y row's offset in a tile buffer (the
// T row is 8 KB further: rows 64 + p share p's swizzle); goff: its source in
// the planes, less the chunk's 64 c (~0u: a padding column).
__device__ __forceinline__ void gram_tasks(uint32_t (&soff)[6], uint32_t (&goff)[6],
                                           const int* col, int lslot, size_t pplane, int tid) {
#pragma unroll
    for (int h = 0; h < 6; ++h) {
        const int t = tid + TJ_T * h;
        const int p = t / 24, rem = t - 24 * (t / 24);
        const int i = rem >> 3, g = rem & 7;
        soff[h] = (uint32_t)i * TJ_PIECE + tc::sw128_off(p, g * 8);
        const int cc = col[p];
        goff[h] = cc >= 0 ? (uint32_t)((size_t)i * pplane + (size_t)cc * 2 * lslot + g * 8) : ~0u;
    }
}

// Step-1 loads of rows 32c..32c+31: 6 16-byte chunks a thread.
__device__ __forceinline__ void load_gram_pieces(uint4 (&v)[6], const uint16_t* P,
                                                 const uint32_t (&goff)[6], int c) {
#pragma unroll
    for (int h = 0; h < 6; ++h)
        v[h] = goff[h] != ~0u ? __ldcg(reinterpret_cast<const uint4*>(P + goff[h] + (size_t)c * 64))
                              : make_uint4(0u, 0u, 0u, 0u);
}

// Step-3 loads of rows 64cp..64cp+63 (128 reals, 256 bytes a piece column)
// straight into the A tiles by cp.async: task t (0..3071) = (piece i, column
// p, 16-byte chunk g), 12 a thread; zero padding for absent columns.
__device__ __forceinline__ void load_update_pieces(uint8_t* At, const uint16_t* P, size_t pplane,
                                                   const int* col, int lslot, int cp, int tid) {
#pragma unroll
    for (int h = 0; h < 12; ++h) {
        const int t = tid + TJ_T * h;
        const int i = t >> 10, p = (t >> 4) & 63, g = t & 15;
        const int cc = col[p];
        const uint16_t* src = P + i * pplane + (size_t)(cc >= 0 ? cc : 0) * 2 * lslot +
                              (size_t)cp * 128 + g * 8;
        uint8_t* dst = At + i * TJ_PIECE + (uint32_t)(g >> 3) * TJ_MGRP + tc::sw128_off(p, (g & 7) * 8);
        tc::cp_async16(dst, src, cc >= 0 ? 16u : 0u);
    }
    tc::cp_async_commit();
}

// Adds the 32 TMEM columns at taddr (this thread's lane) into acc.
__device__ __forceinline__ void tmem_accumulate(uint32_t taddr, float (&acc)[32]) {
    float v[32];
    tc::tmem_ld32(taddr, v);
#pragma unroll
    for (int e = 0; e < 32; ++e) acc[e] += v[e];
}

// One visit of blocks (I, J) of job j (see the file comment).  All threads
// call it; returns whether it rotated anything and clears ok when a bounded
// MMA wait expired (the outputs are then invalid).
__device__ __forceinline__ bool visit(const TwoQGeom& g, int j, int I, int J, bool full,
                                      double tol2d, float tol2, uint8_t* smem, Aux& ax,
                                      uint32_t tmem, unsigned& ph0, unsigned& ph1, bool& ok) {
    cf* const G = reinterpret_cast<cf*>(smem);
    cf* const H = reinterpret_cast<cf*>(smem + TJ_HOFF);
    cf* const E = reinterpret_cast<cf*>(smem + TJ_EOFF);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int lslot = g.lslot;
    const size_t pplane = g.pplane;
    uint16_t* P = g.P + (size_t)j * 3 * pplane;
    // this thread's TMEM lane quarter and its 32 accumulator columns
    const uint32_t tlane = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 32u * (uint32_t)(warp >> 2);

    if (tid < TJ_W) {
        const int pos = (tid < TJ_BC ? I * TJ_BC : J * TJ_BC - TJ_BC) + tid;
        ax.col[tid] = pos < g.cslot ? __ldcg(g.cmap + (size_t)j * g.cslot + pos) : -1;
    }
    if (tid == 0) {
        ax.rotated = 0;
        ax.cmax = 0.f;
    }
    __syncthreads();
    const long long c0 = clock64();

    // ---- 1. Gram -------------------------------------------------------
    {
        const int nchunk = lslot / 32;
        constexpr uint32_t IDESC_G = tc::idesc_bf16(128, 64, false, false);
        float acc[32];
#pragma unroll
        for (int e = 0; e < 32; ++e) acc[e] = 0.f;
        uint32_t soff[6], goff[6];
        gram_tasks(soff, goff, ax.col, lslot, pplane, tid);
        uint4 pre[6];
        load_gram_pieces(pre, P, goff, 0);
        int waited = -1;                  // chunks <= waited are summed into acc
        for (int c = 0; c < nchunk; ++c) {
            const int b = c & 1;
            if (c >= 2) {
                // tile buffer b and accumulator b were used by chunk c - 2
                ok = __syncthreads_and(b ? wait_mma(&ax.bar[1], ph1) : wait_mma(&ax.bar[0], ph0)) != 0;
                if (!ok) break;
                tc::fence_after_sync();
                tmem_accumulate(tlane + 64u * b, acc);
                tc::fence_before_sync();
                waited = c - 2;
            }
            uint8_t* tile = smem + b * TJ_GTILE;
#pragma unroll
            for (int h = 0; h < 6; ++h) {
                *reinterpret_cast<uint4*>(tile + soff[h]) = pre[h];
                *reinterpret_cast<uint4*>(tile + soff[h] + TJ_W * 128) = twist_packed(pre[h]);
            }
            // the next chunk's loads overlap this chunk's MMAs and the next
            // accumulator read
            if (c + 1 < nchunk) load_gram_pieces(pre, P, goff, c + 1);
            tc::fence_async_smem();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint64_t d0 = tc::sdesc(tc::smem_u32(tile), 16, 1024);
                // piece products smallest first: (2,0) (1,1) (0,2) (1,0) (0,1) (0,0)
                const int pa[6] = {2, 1, 0, 1, 0, 0};
                const int pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
                for (int ks = 0; ks < 4; ++ks)
#pragma unroll
                    for (int q = 0; q < 6; ++q)
                        tc::mma_bf16(tmem + 64u * b,
                                     tc::sdesc_add(d0, pa[q] * TJ_PIECE + ks * 32),
                                     tc::sdesc_add(d0, pb[q] * TJ_PIECE + ks * 32), IDESC_G,
                                     (ks | q) != 0);
                tc::mma_commit(&ax.bar[b]);
            }
        }
        // the last one or two chunks (every phase is waited on, so the
        // barriers' parities stay in step)
        for (int c = waited + 1; ok && c < nchunk; ++c) {
            const int b = c & 1;
            ok = __syncthreads_and(b ? wait_mma(&ax.bar[1], ph1) : wait_mma(&ax.bar[0], ph0)) != 0;
            if (!ok) break;
            tc::fence_after_sync();
            tmem_accumulate(tlane + 64u * b, acc);
        }
        if (!ok) return false;
        // acc -> G: D rows 0..63 are Re G, rows 64..127 are -Im G
        tc::fence_before_sync();
        __syncthreads();                                   // the tile buffers are dead
        const int mrow = 32 * (warp & 3) + lane;
        const int q0 = 32 * (warp >> 2);
        if (mrow < TJ_W) {
#pragma unroll
            for (int e = 0; e < 32; ++e) G[gidx(mrow, q0 + e)].x = acc[e];
        } else {
#pragma unroll
            for (int e = 0; e < 32; ++e) G[gidx(mrow - TJ_W, q0 + e)].y = -acc[e];
        }
    }
    for (int e = tid; e < TJ_W * TJ_W; e += TJ_T) E[e] = cmake(0.f, 0.f);
    __syncthreads();
    if (tid < TJ_W) {
        G[gidx(tid, tid)].y = 0.f;
        ax.diag[tid] = G[gidx(tid, tid)].x;
    }
    __syncthreads();
    const long long c1 = clock64();

    // ---- 2. convergence test (FP64) and rotations on G ----------------------
    // The visit's pairs (the 32 x 32 inter-block pairs, or all 2016 on a full
    // visit) with |G_pq|^2 > tol^2 G_pp G_qq; the largest squared cosine goes
    // to the job's convergence record.
    {
        float cmax = 0.f;
        int any = 0;
        for (int e = tid; e < TJ_W * TJ_W; e += TJ_T) {
            const int p = e / TJ_W, q = e % TJ_W;
            if (q <= p || (!full && (p >= TJ_BC || q < TJ_BC))) continue;
            const float a = ax.diag[p], b = ax.diag[q];
            const cf gam = G[gidx(p, q)];
            const double g2 = (double)gam.x * gam.x + (double)gam.y * gam.y;
            const double ab = (double)a * (double)b;
            if (a > 0.f && b > 0.f && g2 > tol2d * ab) {
                any = 1;
                cmax = fmaxf(cmax, (float)g2 / (float)ab);
            }
        }
        cmax = warp_max(cmax);
        any = __any_sync(0xffffffffu, any);
        if (lane == 0 && any) {
            atomicMax(reinterpret_cast<int*>(&ax.cmax), __float_as_int(fmaxf(cmax, tol2 * 1.0001f)));
            ax.rotated = 1;
        }
        __syncthreads();
    }
    const bool work = ax.rotated != 0;
    const int nsteps = TJ_W - 1;           // the full visit's steps
    int rsteps = 0, rpairs = 0;
    if (work && !full) {
        // Ring visit (the 32 x 32 inter-block pairs), 2 x 2 blocks: step s
        // pairs index k with 32 + (k + s) % 32 on both sides of G, so row
        // pair i and column pair k span a 2 x 2 block of G that the step
        // changes as R_i^H B R_k.  Thread (warp w, lane k) holds the blocks
        // of column pair k and row pairs i = 4w + h (h < 4): PP = G[i][k],
        // PQ = G[i][q_k], QP = G[q_i][k], QQ = G[q_i][q_k] -- all of a step's
        // arithmetic on G is local.  Between steps the Q columns move one
        // lane down (shuffles) and the Q rows one row pair down: row pair
        // i + 1's, in the same thread but for h = 3, which takes row pair
        // 4(w + 1)'s through a double-buffered shared array in the H area; a
        // step has one barrier.  E (Y <- Y + Y E) keeps the column layout of
        // the full visit: rows w + 8h (h < 8), columns k and q_k.
        const int cP = lane;
        int cQ = TJ_BC + lane;
        cf bPP[4], bPQ[4], bQP[4], bQQ[4], eP[8], eQ[8];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int i = 4 * warp + h;
            bPP[h] = G[gidx(i, cP)];
            bPQ[h] = G[gidx(i, cQ)];
            bQP[h] = G[gidx(TJ_BC + i, cP)];
            bQQ[h] = G[gidx(TJ_BC + i, cQ)];
        }
#pragma unroll
        for (int h = 0; h < 8; ++h) {
            eP[h] = cmake(0.f, 0.f);
            eQ[h] = cmake(0.f, 0.f);
        }
        float4* const xq = reinterpret_cast<float4*>(smem + TJ_HOFF);   // [2][8 warps][32]
        {
            // gamma of pair k = G[k][q_k] = PQ of row pair k (warp k / 4)
            cf v = cmake(0.f, 0.f);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const float m = (4 * warp + h == cP) ? 1.f : 0.f;
                v.x = fmaf(m, bPQ[h].x, v.x);
                v.y = fmaf(m, bPQ[h].y, v.y);
            }
            if (warp == (cP >> 2)) ax.gam[lane] = v;
        }
        float dP = ax.diag[cP], dQ = ax.diag[cQ];
        __syncthreads();
        for (int s = 0; s < TJ_BC; ++s) {
            const int b = s & 1;
            if (s > 0) {
                // the last row pair's Q row: row pair 4(w + 1)'s of the previous step
                const float4 q = xq[((b ^ 1) * 8 + ((warp + 1) & 7)) * 32 + lane];
                bQP[3] = cmake(q.x, q.y);
                bQQ[3] = cmake(q.z, q.w);
            }
            float tp = 0.f, na = 0.f, nb = 0.f;
            cf sg = cmake(0.f, 0.f);
            bool rot;
            {
                const float a = dP, bb = dQ;
                const cf gam = ax.gam[(b * 32) + lane];
                rot = pair_cos2(gam, cabs2(gam), a, bb) > kInnerTol2 * tol2;
                if (rot) {
                    const Rot r = make_rot(a, bb, gam);
                    tp = r.tp;
                    sg = r.sigma;
                    na = a - r.dn;
                    nb = bb + r.dn;
                }
            }
            const unsigned rmask = __ballot_sync(0xffffffffu, rot);
            if (rmask) {
                ++rsteps;
                rpairs += __popc(rmask);
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    // the rotation of row pair i = 4w + h, from lane i
                    const int i = 4 * warp + h;
                    const float tpi = __shfl_sync(0xffffffffu, tp, i);
                    const cf sgi = cmake(__shfl_sync(0xffffffffu, sg.x, i),
                                         -__shfl_sync(0xffffffffu, sg.y, i));   // conj
                    rotate_cols(bPP[h], bPQ[h], tp, sg);
                    rotate_cols(bQP[h], bQQ[h], tp, sg);
                    rotate_cols(bPP[h], bQP[h], tpi, sgi);
                    rotate_cols(bPQ[h], bQQ[h], tpi, sgi);
                }
#pragma unroll
                for (int h = 0; h < 8; ++h) {
                    const int r = warp + 8 * h;
                    rotate_cols(eP[h], eQ[h], tp, sg);
                    const float mp = r == cP ? 1.f : 0.f, mq = r == cQ ? 1.f : 0.f;
                    eP[h].x = fmaf(-mp, tp, fmaf(-mq, sg.x, eP[h].x));
                    eP[h].y = fmaf(-mq, sg.y, eP[h].y);
                    eQ[h].x = fmaf(mp, sg.x, fmaf(-mq, tp, eQ[h].x));
                    eQ[h].y = fmaf(-mp, sg.y, eQ[h].y);
                }
                if (rot) {
                    dP = na;
                    dQ = nb;
                }
            }
            if (s + 1 < TJ_BC) {
                // the Q columns move to the lane of their next pair
                const int src = (lane + 1) & 31;
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    bPQ[h] = shfl_cf(bPQ[h], src);
                    bQQ[h] = shfl_cf(bQQ[h], src);
                }
#pragma unroll
                for (int h = 0; h < 8; ++h) eQ[h] = shfl_cf(eQ[h], src);
                cQ = __shfl_sync(0xffffffffu, cQ, src);
                dQ = __shfl_sync(0xffffffffu, dQ, src);
                // the Q rows move one row pair down: row pair 4w's goes to
                // warp w - 1 (for its row pair 4w - 1) through shared memory,
                // the others within the thread
                xq[(b * 8 + warp) * 32 + lane] = make_float4(bQP[0].x, bQP[0].y, bQQ[0].x, bQQ[0].y);
#pragma unroll
                for (int h = 0; h < 3; ++h) {
                    bQP[h] = bQP[h + 1];
                    bQQ[h] = bQQ[h + 1];
                }
                // the next step's gamma of pair k: PQ of row pair k
                cf v = cmake(0.f, 0.f);
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const float m = (4 * warp + h == cP) ? 1.f : 0.f;
                    v.x = fmaf(m, bPQ[h].x, v.x);
                    v.y = fmaf(m, bPQ[h].y, v.y);
                }
                if (warp == (cP >> 2)) ax.gam[((b ^ 1) * 32) + lane] = v;
            }
            __syncthreads();
        }
        if (warp == 0) {
            ax.diag[cP] = dP;
            ax.diag[cQ] = dQ;
        }
        __syncthreads();                  // the diagonal is read below
#pragma unroll
        for (int h = 0; h < 8; ++h) {
            const int r = warp + 8 * h;
            E[r * TJ_W + cP] = eP[h];
            E[r * TJ_W + cQ] = eQ[h];
        }
    } else if (work) {
        // Full visit (all 2016 pairs of the 64 columns, 63 steps).
        // Register-resident: warp w holds rows w, w + 8, ... of G and E, lane
        // k the two columns of pair k (visit columns cP, cQ).  The column
        // rotations of both passes are then local; between the passes H goes
        // through shared memory conjugate-transposed, and between the steps
        // the columns move to the lanes of their next pairs by shuffles in the
        // circle method (cP of lane 0 fixed, the other 63 columns moving
        // along t1 -> t2 -> ... -> t31 -> b31 -> ... -> b0 -> t1).  The angle
        // inputs of a step, diag and gamma = G[cP][cQ], come from the warps
        // holding those rows, through the small arrays.
        int cP = lane, cQ = TJ_W - 1 - lane;
        cf gP[8], gQ[8], eP[8], eQ[8];
#pragma unroll
        for (int h = 0; h < 8; ++h) {
            const int r = warp + 8 * h;
            gP[h] = G[gidx(r, cP)];
            gQ[h] = G[gidx(r, cQ)];
            eP[h] = cmake(0.f, 0.f);
            eQ[h] = cmake(0.f, 0.f);
        }
        publish_gamma(gQ, warp, cP, ax.gam + lane);
        // the diagonal of this lane's columns, kept in every warp alike
        float dP = ax.diag[cP], dQ = ax.diag[cQ];
        __syncthreads();
        for (int s = 0; s < nsteps; ++s) {
            // this warp's copy of the step's 32 rotations: lane k holds pair k
            // (tp = sigma = 0 for a pair that does not rotate: the rotation
            // below is then exactly the identity)
            float tp = 0.f, na = 0.f, nb = 0.f;
            cf sg = cmake(0.f, 0.f);
            bool rot;
            {
                const float a = dP, b = dQ;
                const cf gam = ax.gam[lane];
                // per-step rotation decision in FP32 (kInnerTol2 above)
                rot = pair_cos2(gam, cabs2(gam), a, b) > kInnerTol2 * tol2;
                if (rot) {
                    const Rot r = make_rot(a, b, gam);
                    tp = r.tp;
                    sg = r.sigma;
                    na = a - r.dn;        // the norm transfer of rot.cuh
                    nb = b + r.dn;
                }
            }
            // every warp holds the same 32 decisions: a step without a
            // rotation changes nothing
            const unsigned rmask = __ballot_sync(0xffffffffu, rot);
            if (rmask) {
                ++rsteps;
                rpairs += __popc(rmask);
                // pass 1: H = G R on this warp's rows, stored as H^H
#pragma unroll
                for (int h = 0; h < 8; ++h) {
                    const int r = warp + 8 * h;
                    rotate_cols(gP[h], gQ[h], tp, sg);
                    H[gidx(cP, r)] = cconj(gP[h]);
                    H[gidx(cQ, r)] = cconj(gQ[h]);
                }
                __syncthreads();
                if (rot) {
                    dP = na;
                    dQ = nb;
                }
                // pass 2: G' = H^H R (= R^H G R) and E <- (I + E) R - I =
                // E R + (R - I), whose identity part adds -tp, -sigma to
                // column cP and conj(sigma), -tp to column cQ in rows cP, cQ.
                // (The rotated pair's own entry G'[cP][cQ] keeps its rounding
                // residue: the pair is not met again in this visit.)
#pragma unroll
                for (int h = 0; h < 8; ++h) {
                    const int r = warp + 8 * h;
                    cf x = H[gidx(r, cP)], y = H[gidx(r, cQ)];
                    rotate_cols(x, y, tp, sg);
                    gP[h] = x;
                    gQ[h] = y;
                    rotate_cols(eP[h], eQ[h], tp, sg);
                    const float mp = r == cP ? 1.f : 0.f, mq = r == cQ ? 1.f : 0.f;
                    eP[h].x = fmaf(-mp, tp, fmaf(-mq, sg.x, eP[h].x));
                    eP[h].y = fmaf(-mq, sg.y, eP[h].y);
                    eQ[h].x = fmaf(mp, sg.x, fmaf(-mq, tp, eQ[h].x));
                    eQ[h].y = fmaf(-mp, sg.y, eQ[h].y);
                }
            }
            if (s + 1 < nsteps) {
                // the columns move to the lanes of the next step's pairs
#pragma unroll
                for (int h = 0; h < 8; ++h) {
                    circle_move(gP[h], gQ[h], lane);
                    circle_move(eP[h], eQ[h], lane);
                }
                circle_move_idx(cP, cQ, lane);
                cf d = cmake(dP, dQ);
                circle_move_pair(d, lane);
                dP = d.x;
                dQ = d.y;
                publish_gamma(gQ, warp, cP, ax.gam + lane);
            }
            __syncthreads();
        }
        if (warp == 0) {
            ax.diag[cP] = dP;
            ax.diag[cQ] = dQ;
        }
        __syncthreads();                  // the diagonal is read below
        // E (row-major) for the update's B operand
#pragma unroll
        for (int h = 0; h < 8; ++h) {
            const int r = warp + 8 * h;
            E[r * TJ_W + cP] = eP[h];
            E[r * TJ_W + cQ] = eQ[h];
        }
    }
    const long long c2 = clock64();
    const bool rotated = work && rsteps > 0;

    // new squared norms for the next sweep's sort, and this visit's largest
    // cosine (a pair over the FP64 test that the FP32 step test does not
    // rotate is on the tolerance's edge: it counts as converged, or the job
    // would see the same Gram again every sweep)
    if (rotated && tid < TJ_W) {
        const int col = ax.col[tid];
        if (col >= 0) g.cnrm[(size_t)j * g.cslot + col] = ax.diag[tid];
    }
    if (rotated && tid == 0) atomicMax(reinterpret_cast<int*>(g.offmax + j), __float_as_int(ax.cmax));

    // ---- 3. Y <- Y + Y E ---------------------------------------------------
    // Real form without the -i Y rows: D1 = Y Re E and D2 = Y Im E (M = the
    // 128 interleaved reals of 64 rows, N = 128: Re E's columns then Im E's,
    // K = the 64 visit columns), then Re y' = Re y + D1(re) - D2(im) and
    // Im y' = Im y + D2(re) + D1(im): the two reals of a row are adjacent
    // TMEM lanes, one shuffle apart.  All three pieces of a chunk's A tile fit
    // beside B, so one step (24 MMAs) per 64 rows; the chunk's pieces arrive
    // by cp.async while the previous chunk's epilogue runs.
    if (rotated) {
        __syncthreads();                                   // the diagonal above is read
        // B pieces at [0, 48K): row n of piece i at i*16K + sw128_off(n, k),
        // k = the visit column; n < 64: Re E[k][n], n >= 64: Im E[k][n-64].
        // Task (n, k-group of 8): 128 x 8 = 1024 tasks, 4 a thread.
#pragma unroll 1
        for (int h = 0; h < 4; ++h) {
            const int task = tid + TJ_T * h;
            const int n = task & 127, kg = task >> 7;      // kg in 0..7
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const cf x = E[(kg * 8 + e) * TJ_W + (n & 63)];
                v[e] = n < 64 ? x.x : x.y;
            }
            put_pieces(smem, TJ_PIECE, tc::sw128_off(n, kg * 8), v);
        }
        __syncthreads();                                   // E is dead
        uint8_t* At = smem + TJ_AOFF;                      // piece i at At + i*16K
        constexpr uint32_t IDESC_U = tc::idesc_bf16(128, 128, true, false);
        const int npair = lslot / 64;
        const int mreal = 32 * (warp & 3) + lane;          // TMEM lane: real of the chunk
        const int q0 = 32 * (warp >> 2);
        const uint32_t xoff = (uint32_t)(mreal >> 6) * TJ_MGRP;
        const bool re_lane = (mreal & 1) == 0;
        load_update_pieces(At, P, pplane, ax.col, lslot, 0, tid);
        for (int cp = 0; cp < npair; ++cp) {
            tc::cp_async_wait_all();
            tc::fence_async_smem();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint64_t da = tc::sdesc(tc::smem_u32(At), TJ_MGRP, 1024);
                const uint64_t db = tc::sdesc(tc::smem_u32(smem), 16, 1024);
                // piece products smallest first: (2,0) (1,1) (0,2) (1,0) (0,1) (0,0)
                const int pa[6] = {2, 1, 0, 1, 0, 0};
                const int pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
                for (int q = 0; q < 6; ++q)
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks)
                        tc::mma_bf16(tmem, tc::sdesc_add(da, pa[q] * TJ_PIECE + ks * 2048),
                                     tc::sdesc_add(db, pb[q] * TJ_PIECE + ks * 32), IDESC_U,
                                     (q | ks) != 0);
                tc::mma_commit(&ax.bar[0]);
            }
            // Y of this thread's elements (real mreal, columns q0..q0+31),
            // summed from the three pieces in the tile (exact)
            float xr[32];
#pragma unroll
            for (int e = 0; e < 32; ++e) {
                const uint32_t o = xoff + tc::sw128_off(q0 + e, mreal & 63);
                xr[e] = bf16_bits(*reinterpret_cast<const uint16_t*>(At + o)) +
                        (bf16_bits(*reinterpret_cast<const uint16_t*>(At + TJ_PIECE + o)) +
                         bf16_bits(*reinterpret_cast<const uint16_t*>(At + 2 * TJ_PIECE + o)));
            }
            ok = __syncthreads_and(wait_mma(&ax.bar[0], ph0)) != 0;
            if (!ok) break;
            tc::fence_after_sync();
            // the tile is free: the next chunk's pieces load during the epilogue
            if (cp + 1 < npair) load_update_pieces(At, P, pplane, ax.col, lslot, cp + 1, tid);
            // Per 16 columns: y of this lane's real, then the two lanes of a
            // row swap halves so that each holds (re, im) of 8 columns and
            // writes one 4-byte word per piece plane and column.
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                float d1[16], d2[16];
                const uint32_t tl = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + q0 + 16 * half;
                tc::tmem_ld16(tl, d1);
                tc::tmem_ld16(tl + 64, d2);
                float y[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const float d2p = __shfl_xor_sync(0xffffffffu, d2[e], 1);
                    y[e] = xr[16 * half + e] + (re_lane ? d1[e] - d2p : d2p + d1[e]);
                }
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    // even lane: columns e (its re, the partner's im); odd
                    // lane: columns 8 + e (the partner's re, its im)
                    const float send = re_lane ? y[8 + e] : y[e];
                    const float got = __shfl_xor_sync(0xffffffffu, send, 1);
                    const float vr = re_lane ? y[e] : got, vi = re_lane ? got : y[8 + e];
                    const int col = ax.col[q0 + 16 * half + (re_lane ? e : 8 + e)];
                    if (col >= 0) {
                        const size_t off = (size_t)col * 2 * lslot + (size_t)cp * 128 + (mreal & ~1);
                        const Pieces2 pc = split3x2(vr, vi);
                        *reinterpret_cast<uint32_t*>(P + off) = pc.w0;
                        *reinterpret_cast<uint32_t*>(P + pplane + off) = pc.w1;
                        *reinterpret_cast<uint32_t*>(P + 2 * pplane + off) = pc.w2;
                    }
                }
            }
            tc::fence_before_sync();
        }
        __syncthreads();
    }
    if (tid == 0) {
        const long long c3 = clock64();
        atomicAdd(&g_tj_cycles[0], (unsigned long long)(c1 - c0));
        atomicAdd(&g_tj_cycles[1], (unsigned long long)(c2 - c1));
        atomicAdd(&g_tj_cycles[2], (unsigned long long)(c3 - c2));
        atomicAdd(&g_tj_cycles[3], 1ull);
        if (rotated) {
            atomicAdd(&g_tj_cycles[4], 1ull);
            atomicAdd(&g_tj_cycles[5], (unsigned long long)rsteps);
            atomicAdd(&g_tj_cycles[6], (unsigned long long)rpairs);
        }
    }
    return rotated;
}

// One persistent launch per sweep: CTAs claim the visits (round, job, block
// pair) in round-major order from one counter, wait (bounded) until both
// blocks have finished the previous round, run the visit and publish the
// round -- the protocol of the SIMT sweep kernel, so visits of different
// rounds and jobs overlap and the two CTAs on an SM are seldom in the same
// step.  A visit whose pairs were all below the tolerance when it last ran,
// and whose blocks have not changed since (no rotation touched them and the
// sort kept their sets of columns), is skipped.  tbase = sweep * (rounds + 1).
__global__ void __launch_bounds__(TJ_T, 2)
tc_sweep_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, double tol2d, float tol2,
                int njobs, int rounds, int pairs, SweepSync sync, int tbase) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    Aux& ax = *reinterpret_cast<Aux*>(smem + TJ_AUX);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        mbar_init(&ax.bar[0], 1);
        mbar_init(&ax.bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tc::tmem_alloc(&ax.tmem, TJ_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const long long t_start = clock64();
    const uint32_t tmem = ax.tmem;
    unsigned ph0 = 0u, ph1 = 0u;     // phases of bar[0], bar[1], kept across visits
    const int per_round = njobs * pairs;
    const int total = rounds * per_round;
    for (;;) {
        if (tid == 0) {
            ax.item = atomicAdd(sync.next_item, 1);
            ax.abort = *reinterpret_cast<volatile int*>(sync.error);
        }
        __syncthreads();
        const int item = ax.item;
        if (item >= total || ax.abort) break;
        const int r = item / per_round, rem = item - r * per_round;
        const int j = rem / pairs, p = rem - (rem / pairs) * pairs;
        bool active = !g.done[j];
        int I = 0, J = 0, nb = 2;
        if (active) {
            const mps_2q_job job = jobs[j];
            const int m = job.chi_l * g.d, n = job.chi_r * g.d;
            const int C = min(m, n);
            if (!tc_job(m, n, job.keep_left_canonical)) {
                active = false;           // the SIMT sweep kernel's job
            } else {
                nb = (C + TJ_BC - 1) / TJ_BC;
                nb += nb & 1;
                active = r < nb - 1 && p < nb / 2;
                if (active) tournament_pair(nb, r, p, I, J);
            }
        }
        if (active) {
            // a job of one block pair has one visit per sweep, and a visit
            // that rotates nothing ends it: no stamps
            const bool track = nb > 2;
            volatile int* vst = g.vstamp + (size_t)j * g.nbmax;
            volatile int* qst = g.qstamp + (size_t)j * g.qstride + r * pairs + p;
            if (tid == 0) {
                // qstamp of this (round, pair) changes only when this item
                // runs, so it is read before the wait; the block stamps after it
                const int q = track ? *qst : -1;
                ax.skip = 0;
                if (r > 0) {
                    const long long w0 = clock64();
                    volatile int* fl = sync.block_round + (size_t)j * sync.nbmax;
                    volatile int* err = sync.error;
                    int polls = 0;
                    while ((fl[I] < r - 1 || fl[J] < r - 1) && *err == 0) {
                        if (++polls > sync.wait_limit) {
                            atomicExch(sync.error, 1);
                            break;
                        }
                        __nanosleep(64);
                    }
                    ax.abort = *err;
                    __threadfence();
                    atomicAdd(&g_tj_cycles[7], (unsigned long long)(clock64() - w0));
                }
                if (track) ax.skip = (q >= 0 && q > vst[I] && q > vst[J]) ? 1 : 0;
            }
            __syncthreads();
            if (ax.abort) break;
            bool rot = false;
            if (!ax.skip) {
                bool ok = true;
                rot = visit(g, j, I, J, r == 0, tol2d, tol2, smem, ax, tmem, ph0, ph1, ok);
                if (!ok) {
                    // an MMA wait expired: stop every CTA (the call reports it)
                    if (tid == 0) {
                        atomicExch(g.counter + 3, 1);
                        atomicExch(sync.error, 1);
                    }
                    break;
                }
            }
            __syncthreads();
            if (tid == 0) {
                if (track && !ax.skip) {
                    const int now = tbase + r + 1;
                    if (rot) {
                        vst[I] = now;
                        vst[J] = now;
                    } else {
                        *qst = now;
                    }
                }
                __threadfence();
                atomicExch(sync.block_round + (size_t)j * sync.nbmax + I, r);
                atomicExch(sync.block_round + (size_t)j * sync.nbmax + J, r);
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        atomicAdd(&g_tj_cycles[8], (unsigned long long)(clock64() - t_start));
        atomicAdd(&g_tj_cycles[9], 1ull);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TJ_TMEM_COLS);
}

// X <-> its three bf16 piece planes, every element of every job's slot, 8
// reals a thread (a slot holds 2 lslot cslot reals, a multiple of 64).
__device__ __forceinline__ bool tc_job_at(const mps_2q_job* jobs, size_t j, int d) {
    return tc_job(jobs[j].chi_l * d, jobs[j].chi_r * d, jobs[j].keep_left_canonical);
}

__global__ void __launch_bounds__(256)
tc_split_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int njobs) {
    const size_t per8 = g.pplane / 8;
    const size_t total8 = per8 * (size_t)njobs;
    const float4* X = reinterpret_cast<const float4*>(g.X);
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total8;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t jj = e / per8, off = (e - jj * per8) * 8;
        if (!tc_job_at(jobs, jj, g.d)) continue;
        const float4 lo = __ldcs(X + 2 * e), hi = __ldcs(X + 2 * e + 1);
        const float v[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        uint8_t* base = reinterpret_cast<uint8_t*>(g.P + jj * 3 * g.pplane + off);
        put_pieces(base, g.pplane * sizeof(uint16_t), 0u, v);
    }
}

__global__ void __launch_bounds__(256)
tc_merge_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int njobs) {
    const size_t per8 = g.pplane / 8;
    const size_t total8 = per8 * (size_t)njobs;
    float4* X = reinterpret_cast<float4*>(g.X);
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total8;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t jj = e / per8, off = (e - jj * per8) * 8;
        if (!tc_job_at(jobs, jj, g.d)) continue;
        const uint16_t* base = g.P + jj * 3 * g.pplane + off;
        const uint4 w0 = __ldcs(reinterpret_cast<const uint4*>(base));
        const uint4 w1 = __ldcs(reinterpret_cast<const uint4*>(base + g.pplane));
        const uint4 w2 = __ldcs(reinterpret_cast<const uint4*>(base + 2 * g.pplane));
        const uint32_t a0[4] = {w0.x, w0.y, w0.z, w0.w};
        const uint32_t a1[4] = {w1.x, w1.y, w1.z, w1.w};
        const uint32_t a2[4] = {w2.x, w2.y, w2.z, w2.w};
        float v[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            // the sum is exact: p1 + p2 is the first residual, p0 + it is x
            v[2 * k] = __uint_as_float(a0[k] << 16) +
                       (__uint_as_float(a1[k] << 16) + __uint_as_float(a2[k] << 16));
            v[2 * k + 1] = __uint_as_float(a0[k] & 0xffff0000u) +
                           (__uint_as_float(a1[k] & 0xffff0000u) + __uint_as_float(a2[k] & 0xffff0000u));
        }
        __stcs(X + 2 * e, make_float4(v[0], v[1], v[2], v[3]));
        __stcs(X + 2 * e + 1, make_float4(v[4], v[5], v[6], v[7]));
    }
}

int split_grid(const TwoQGeom& g, int njobs) {
    const size_t total8 = g.pplane / 8 * (size_t)njobs;
    return (int)std::min<size_t>((total8 + 255) / 256, 152 * 8);
}

}  // namespace

int tc_split_launch(const mps_2q_job* jobs, int njobs, const TwoQGeom& g, cudaStream_t s) {
    if (!g.P) return fail(MPS_ERR_ARG, "tc sweeps: the workspace has no piece planes");
    if (g.pplane % 64 != 0) return fail(MPS_ERR_ARG, "tc sweeps: unsupported slot size");
    tc_split_kernel<<<split_grid(g, njobs), 256, 0, s>>>(jobs, g, njobs);
    MPS_LAUNCH_CHECK("tc_split_kernel");
    return MPS_OK;
}

int tc_merge_launch(const mps_2q_job* jobs, int njobs, const TwoQGeom& g, cudaStream_t s) {
    if (!g.P) return fail(MPS_ERR_ARG, "tc sweeps: the workspace has no piece planes");
    if (g.pplane % 64 != 0) return fail(MPS_ERR_ARG, "tc sweeps: unsupported slot size");
    tc_merge_kernel<<<split_grid(g, njobs), 256, 0, s>>>(jobs, g, njobs);
    MPS_LAUNCH_CHECK("tc_merge_kernel");
    return MPS_OK;
}

int tc_sweep_launch(const mps_2q_job* jobs, int njobs, int rounds, int pairs, const TwoQGeom& g,
                    float tol2, const SweepSync& sync, int tbase, cudaStream_t s) {
    static KernelSetup ks;
    int dev = 0;
    MPS_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(MPS_ERR_ARG, "device index beyond 63");
    std::call_once(ks.once[dev], [&] {
        int rc = MPS_OK;
        cudaError_t e = cudaFuncSetAttribute(tc_sweep_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)TJ_SMEM);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaFuncSetAttribute(tc_sweep_kernel)");
        // all of the unified L1 as shared memory: two CTAs of ~100 KB per SM
        // (with the default split the occupancy is one)
        if (rc == MPS_OK) {
            e = cudaFuncSetAttribute(tc_sweep_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared);
            if (e != cudaSuccess) rc = cuda_fail(e, "carveout of tc_sweep_kernel");
        }
        int sms = 0, per_sm = 0;
        if (rc == MPS_OK) {
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_sweep_kernel, TJ_T, TJ_SMEM);
            if (e != cudaSuccess) rc = cuda_fail(e, "resident CTAs of tc_sweep_kernel");
        }
        // The occupancy query answers 1 for this kernel even without dynamic
        // shared memory; by its registers and shared memory two CTAs fit (and
        // do run side by side).  A larger grid is safe either way: a visit
        // only waits for visits that running CTAs claimed before it.
        if (rc == MPS_OK) {
            cudaFuncAttributes fa;
            e = cudaFuncGetAttributes(&fa, tc_sweep_kernel);
            if (e != cudaSuccess) rc = cuda_fail(e, "attributes of tc_sweep_kernel");
            int regs_per_sm = 0, smem_per_sm = 0, smem_reserved = 0;
            if (rc == MPS_OK) {
                cudaDeviceGetAttribute(&regs_per_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
                cudaDeviceGetAttribute(&smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
                cudaDeviceGetAttribute(&smem_reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
                const int by_regs = regs_per_sm / std::max(1, ((fa.numRegs * 32 + 255) / 256) * 256 * (TJ_T / 32));
                const int by_smem = smem_per_sm / (int)(TJ_SMEM + fa.sharedSizeBytes + smem_reserved);
                per_sm = std::max(per_sm, std::min(by_regs, by_smem));
            }
        }
        // every CTA allocates TMEM_COLS of the SM's 512 TMEM columns
        per_sm = std::min(per_sm, (int)(512 / TJ_TMEM_COLS));
        ks.ctas[dev] = sms * (per_sm > 0 ? per_sm : 1);
        ks.rc[dev] = rc;
    });
    if (ks.rc[dev] != MPS_OK) return ks.rc[dev];
    if (g.lslot % 64 != 0) return fail(MPS_ERR_ARG, "tc sweeps: slot rows must be a multiple of 64");
    if (!g.P) return fail(MPS_ERR_ARG, "tc sweeps: the workspace has no piece planes");
    if (!g.vstamp || !g.qstamp) return fail(MPS_ERR_ARG, "tc sweeps: no visit stamps");
    const int total = rounds * njobs * pairs;
    if (total <= 0) return MPS_OK;
    // co-resident CTAs only: a visit waits for visits claimed before it
    const int grid = std::min(total, ks.ctas[dev]);
    tc_sweep_kernel<<<grid, TJ_T, TJ_SMEM, s>>>(jobs, g, (double)tol2, tol2, njobs, rounds, pairs,
                                                sync, tbase);
    MPS_LAUNCH_CHECK("tc_sweep_kernel");
    return MPS_OK;
}

}  // namespace mps

// Counters of the tensor-core visits (g_tj_cycles), reset after reading when
// reset != 0.  Blocks.
extern "C" int mps_tc_profile(unsigned long long* out10, int reset) {
    unsigned long long v[10] = {0};
    MPS_CUDA_CHECK(cudaMemcpyFromSymbol(v, mps::g_tj_cycles, sizeof(v)));
    if (reset) {
        const unsigned long long z[10] = {0};
        MPS_CUDA_CHECK(cudaMemcpyToSymbol(mps::g_tj_cycles, z, sizeof(z)));
    }
    if (out10)
        for (int i = 0; i < 10; ++i) out10[i] = v[i];
    return MPS_OK;
}
