// Block one-sided Jacobi on the tcgen05 tensor cores: the split-precision
// ("mixed") form of the truncated SVD of mps_apply_2q_batch.
//
// Replaces the same computation as the FP32 SIMT sweep kernel (jacobi.cu):
// TensorNetwork's split_node_full_svd (mpsim/core.py:1132-1137; LAPACK
// gesdd underneath) for the left-canonical tall jobs, whose left factor is
// U = X/S from the final columns and whose right factor is formed afterwards
// as U^H theta.
//
// The C columns of X (the L factor of theta, or theta) are split into blocks
// of 32.  A sweep visits every pair of blocks once (circle-method rounds over
// the norm-sorted column order, as in the SIMT form).  One visit of blocks
// (I, J), Y = [X_I X_J] (L x 64 complex), by one 256-thread CTA:
//   1. Gram:     G = Y^H Y (64 x 64 complex) on the tensor cores.  Real form:
//                rows 0..63 of the operand tile are the columns of Y as
//                interleaved (re, im) vectors of length 2L, rows 64..127 are
//                T = -i Y; D[m, q] = sum over the 2L reals of tile row m times
//                tile row q gives Re G (m < 64) and -Im G (m >= 64).
//                K-major operands, K = 2L in chunks of 64 reals.
//   2. Rotations on G in shared memory: two-sided Jacobi, 32 disjoint pairs
//                per step (the 32 x 32 inter-block pairs in 32 steps, or all
//                2016 pairs in 63 steps on a block's first visit of a
//                sweep), accumulating the 64 x 64 unitary Q.  The convergence
//                test runs first, in FP64 on the fresh Gram: a visit none of
//                whose pairs has |G_pq|^2 > tol^2 G_pp G_qq changes nothing and
//                skips steps 2 and 3.  The per-step rotation test and the
//                rotation parameters are the FP32 ones of rot.cuh.
//   3. Rotation: Y <- Y + Y E with E = Q - I, skipped when the visit rotated
//                nothing.  The tensor cores form D = Y E; the epilogue adds
//                Y + D in FP32 with round-to-nearest.  Real form:
//                D[(r, c), q] = sum_p Y[(r, c), p] Re E_pq + T[(r, c), p]
//                (-Im E_pq): the SAME shared-memory tile as step 1, now read
//                as an MN-major A operand (M = the 2L reals, 64 per swizzle
//                row; K = the 128 tile rows), times a K-major B operand holding
//                (Re E, -Im E).  M = 128 reals per MMA.
// Why the update form: the tensor core's FP32 accumulation truncates toward
// zero (it does not round to nearest), so a product accumulated over many
// MMAs comes out slightly small.  Y Q re-accumulates all of Y in every visit
// and shrank every singular value by ~5e-5 over a chi=256 SVD; D = Y E is
// small once the rotations are (after the first sweeps), and its bias goes
// with it.  The piece products are also issued smallest first, so the
// accumulator is small for all but the last eight MMAs.
// Every FP32 value is split into three bf16 pieces and each product sums
// the six piece products of order <= 2 (tc.cuh): FP32-grade Gram entries
// and rotations, with the tensor pipe doing the O(L) work that the SIMT form
// does with FMAs.  The new squared column norms (the diagonal of Q^H G Q) go
// to cnrm for the next sweep's sort.
//
// Shared memory (about 82 KB, two CTAs per SM):
//   R0 [0, 48K):   step 1: three 16 KB bf16 piece tiles (128 rows x 128 B);
//                  step 2: G (64 x 65 complex, padded rows);
//                  step 3: the three B-operand pieces of Q (16 KB each).
//   R1 [48K, 80K): step 2: E = Q - I (64 x 64 complex);
//                  step 3: one A piece tile (2 x 16 KB M-groups).
#include "rot.cuh"
#include "tc.cuh"
#include "twoq.cuh"

namespace mps {
namespace {

constexpr int TJ_T = 256;                  // threads per CTA
constexpr int TJ_BC = 32;                  // columns per block
constexpr int TJ_W = 2 * TJ_BC;            // columns per visit
constexpr uint32_t TJ_PIECE = 16384;       // 128 rows x 128 B
constexpr uint32_t TJ_R1 = 3 * TJ_PIECE;   // 48 KB
constexpr uint32_t TJ_AUX = TJ_R1 + 2 * TJ_PIECE;   // 80 KB: small arrays
constexpr int TJ_GS = TJ_W + 1;            // padded row stride of G (complex): column reads
constexpr int TJ_QS = TJ_W;                // row stride of Q (its accesses are row-contiguous)
constexpr uint32_t TJ_TMEM_COLS = 64;
constexpr int TJ_WAIT_LIMIT = 1 << 14;

// Cycles spent in the three steps of a visit, summed over the CTAs of every
// visit since the last reset: [0] Gram, [1] rotations on G, [2] Y <- Y + Y E,
// [3] visits.  Read with mps_tc_profile.
__device__ unsigned long long g_tj_cycles[4];

struct Aux {
    uint64_t bar;
    uint32_t tmem;
    int rotated;          // any pair of this visit rotated
    int col[TJ_W];        // physical column of each visit column (-1: zero padding)
    float tp[TJ_W / 2];   // rotation parameters of the current step
    cf sigma[TJ_W / 2];
    int pp[TJ_W / 2], pq[TJ_W / 2];
    float cmax;           // largest squared cosine of a rotated pair
};
constexpr size_t TJ_SMEM = TJ_AUX + sizeof(Aux) + 1024;

// Two FP32 values -> piece `which` of each, packed as one 32-bit word.
__device__ __forceinline__ uint32_t pack_piece(float a, float b, int which) {
    const tc::Split3 sa = tc::split3(a), sb = tc::split3(b);
    const __nv_bfloat16 xa = which == 0 ? sa.p0 : (which == 1 ? sa.p1 : sa.p2);
    const __nv_bfloat16 xb = which == 0 ? sb.p0 : (which == 1 ? sb.p1 : sb.p2);
    return (uint32_t)__bfloat16_as_ushort(xa) | ((uint32_t)__bfloat16_as_ushort(xb) << 16);
}

// 8 reals -> the 16-byte chunk of piece `which` at off (registers only: a
// runtime-indexed local array would live in local memory).
__device__ __forceinline__ void put_piece(uint8_t* base, uint32_t off, const float* v, int which) {
    uint4 w;
    w.x = pack_piece(v[0], v[1], which);
    w.y = pack_piece(v[2], v[3], which);
    w.z = pack_piece(v[4], v[5], which);
    w.w = pack_piece(v[6], v[7], which);
    *reinterpret_cast<uint4*>(base + off) = w;
}

// 8 reals -> the 16-byte chunks of all three pieces, in tiles `stride` apart.
__device__ __forceinline__ void put_pieces(uint8_t* base, uint32_t stride, uint32_t off,
                                           const float* v) {
    uint32_t w[3][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const tc::Split3 a = tc::split3(v[2 * e]), b = tc::split3(v[2 * e + 1]);
        w[0][e] = (uint32_t)__bfloat16_as_ushort(a.p0) | ((uint32_t)__bfloat16_as_ushort(b.p0) << 16);
        w[1][e] = (uint32_t)__bfloat16_as_ushort(a.p1) | ((uint32_t)__bfloat16_as_ushort(b.p1) << 16);
        w[2][e] = (uint32_t)__bfloat16_as_ushort(a.p2) | ((uint32_t)__bfloat16_as_ushort(b.p2) << 16);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
        *reinterpret_cast<uint4*>(base + i * stride + off) = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

// T = -i Y: (re, im) -> (im, -re).
__device__ __forceinline__ void twist8(const float* v, float* t) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        t[2 * e] = v[2 * e + 1];
        t[2 * e + 1] = -v[2 * e];
    }
}

__device__ __forceinline__ bool wait_mma(uint64_t* bar, unsigned& phase) {
    const bool ok = tc::mbar_wait_bounded(bar, phase, TJ_WAIT_LIMIT);
    phase ^= 1u;
    return ok;
}

// Pair k of inner step s: the 32 x 32 inter-block pairs (ring) or the
// circle-method pairs of all 64 columns (full).
__device__ __forceinline__ void inner_pair(bool full, int s, int k, int& p, int& q) {
    if (full) {
        tournament_pair(TJ_W, s, k, p, q);
    } else {
        p = k;
        q = TJ_BC + ((k + s) & (TJ_BC - 1));
    }
}

// Phase-1 loads of rows 32c..32c+31: task (p, grp) = 8 reals of column p.
__device__ __forceinline__ void load_gram_chunk(float (&pre)[2][8], const float* X, const int* col,
                                                int lslot, int c, int tid) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int task = tid + TJ_T * h;
        const int p = task >> 3, grp = task & 7;
        const int cc = col[p];
        if (cc >= 0) {
            const float4* src = reinterpret_cast<const float4*>(
                X + ((size_t)cc * lslot + (size_t)c * 32) * 2 + grp * 8);
            const float4 a = __ldcg(src), b = __ldcg(src + 1);
            pre[h][0] = a.x; pre[h][1] = a.y; pre[h][2] = a.z; pre[h][3] = a.w;
            pre[h][4] = b.x; pre[h][5] = b.y; pre[h][6] = b.z; pre[h][7] = b.w;
        } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) pre[h][e] = 0.f;
        }
    }
}

// Phase-3 loads of rows 64cp..64cp+63: task (p, grp) = 8 reals of column p.
__device__ __forceinline__ void load_rot_chunk(float (&y)[4][8], const float* X, const int* col,
                                               int lslot, int cp, int tid) {
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        const int task = tid + TJ_T * h;
        const int p = task >> 4, grp = task & 15;
        const int cc = col[p];
        if (cc >= 0) {
            const float4* src = reinterpret_cast<const float4*>(
                X + ((size_t)cc * lslot + (size_t)cp * 64) * 2 + grp * 8);
            const float4 a = __ldcg(src), b = __ldcg(src + 1);
            y[h][0] = a.x; y[h][1] = a.y; y[h][2] = a.z; y[h][3] = a.w;
            y[h][4] = b.x; y[h][5] = b.y; y[h][6] = b.z; y[h][7] = b.w;
        } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) y[h][e] = 0.f;
        }
    }
}

__global__ void __launch_bounds__(TJ_T, 2)
tc_visit_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int round, double tol2d,
                float tol2) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    Aux& ax = *reinterpret_cast<Aux*>(smem + TJ_AUX);
    uint8_t* R0 = smem;
    uint8_t* R1 = smem + TJ_R1;
    cf* G = reinterpret_cast<cf*>(R0);
    cf* Q = reinterpret_cast<cf*>(R1);

    const int j = blockIdx.y;
    if (__ldg(g.done + j)) return;
    const mps_2q_job job = jobs[j];
    const int m = job.chi_l * g.d, n = job.chi_r * g.d;
    const int C = min(m, n);
    if (job_tracks_v(m, n, job.keep_left_canonical) || C < TJ_W) {
        // only left-canonical tall jobs of 64+ columns take these sweeps
        if (threadIdx.x == 0 && blockIdx.x == 0 && round == 0) atomicExch(g.counter + 2, 1);
        return;
    }
    int nb = (C + TJ_BC - 1) / TJ_BC;
    if (nb < 2) nb = 2;
    nb += nb & 1;
    if (round >= nb - 1 || (int)blockIdx.x >= nb / 2) return;
    int I, J;
    tournament_pair(nb, round, blockIdx.x, I, J);
    const bool full = round == 0;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int lslot = g.lslot;
    float* X = reinterpret_cast<float*>(g.X + (size_t)j * lslot * g.cslot);

    if (tid < TJ_W) {
        const int pos = (tid < TJ_BC ? I * TJ_BC : J * TJ_BC - TJ_BC) + tid;
        ax.col[tid] = pos < g.cslot ? __ldcg(g.cmap + (size_t)j * g.cslot + pos) : -1;
    }
    if (tid == 0) {
        mbar_init(&ax.bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        ax.rotated = 0;
        ax.cmax = 0.f;
    }
    if (warp == 0) {
        tc::tmem_alloc(&ax.tmem, TJ_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = ax.tmem;
    unsigned phase = 0;
    bool ok = true;

    const long long c0 = clock64();
    // ---- 1. Gram -------------------------------------------------------
    // chunk c: rows 32c..32c+31 (64 reals); task (p, grp): 8 reals of column p
    const int nchunk = lslot / 32;
    float pre[2][8];
    constexpr uint32_t IDESC_G = tc::idesc_bf16(128, 64, false, false);
    load_gram_chunk(pre, X, ax.col, lslot, 0, tid);
    for (int c = 0; c < nchunk; ++c) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int task = tid + TJ_T * h;
            const int p = task >> 3, grp = task & 7;
            float t[8];
            twist8(pre[h], t);
            put_pieces(R0, TJ_PIECE, tc::sw128_off(p, grp * 8), pre[h]);
            put_pieces(R0, TJ_PIECE, tc::sw128_off(TJ_W + p, grp * 8), t);
        }
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t s0 = tc::smem_u32(R0);
            const int pa[6] = {2, 1, 0, 1, 0, 0};
            const int pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
#pragma unroll
                for (int q = 0; q < 6; ++q)
                    tc::mma_bf16(tmem, tc::sdesc(s0 + pa[q] * TJ_PIECE + ks * 32, 16, 1024),
                                 tc::sdesc(s0 + pb[q] * TJ_PIECE + ks * 32, 16, 1024), IDESC_G,
                                 (c | ks | q) != 0);
            tc::mma_commit(&ax.bar);
        }
        if (c + 1 < nchunk) load_gram_chunk(pre, X, ax.col, lslot, c + 1, tid);  // overlaps the MMAs
        ok = __syncthreads_and(wait_mma(&ax.bar, phase)) != 0;
        if (!ok) break;
    }
    tc::fence_after_sync();

    // ---- TMEM -> G (R0), E = Q - I = 0 (R1) --------------------------------
    if (ok) {
        const int mrow = 32 * (warp & 3) + lane;           // tile row of this lane
        const int q0 = 32 * (warp >> 2);
        float v[32];
        tc::tmem_ld32(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + q0, v);
        __syncthreads();                                   // R0 pieces are dead
        if (mrow < TJ_W) {
#pragma unroll
            for (int e = 0; e < 32; ++e) G[mrow * TJ_GS + q0 + e].x = v[e];
        } else {
#pragma unroll
            for (int e = 0; e < 32; ++e) G[(mrow - TJ_W) * TJ_GS + q0 + e].y = -v[e];
        }
        for (int e = tid; e < TJ_W * TJ_W; e += TJ_T) {
            const int r = e / TJ_W, c = e % TJ_W;
            Q[r * TJ_QS + c] = cmake(0.f, 0.f);
        }
        __syncthreads();
        if (tid < TJ_W) G[tid * TJ_GS + tid].y = 0.f;
        __syncthreads();
    }

    const long long c1 = clock64();
    // ---- 2. rotations on G -------------------------------------------------
    // The off-diagonal convergence test, in FP64 on the fresh Gram: the
    // visit's pairs (the 32 x 32 inter-block pairs, or all 2016 on a full
    // visit) with |G_pq|^2 > tol^2 G_pp G_qq.  None: the visit changes nothing
    // and steps 2 and 3 are skipped.  The largest squared cosine goes to the
    // job's convergence record.
    if (ok) {
        float cmax = 0.f;
        int any = 0;
        for (int e = tid; e < TJ_W * TJ_W; e += TJ_T) {
            const int p = e / TJ_W, q = e % TJ_W;
            if (q <= p || (!full && (p >= TJ_BC || q < TJ_BC))) continue;
            const float a = G[p * TJ_GS + p].x, b = G[q * TJ_GS + q].x;
            const cf gam = G[p * TJ_GS + q];
            const double g2 = (double)gam.x * gam.x + (double)gam.y * gam.y;
            const double ab = (double)a * (double)b;
            if (a > 0.f && b > 0.f && g2 > tol2d * ab) {
                any = 1;
                cmax = fmaxf(cmax, (float)(g2 / ab));
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
    const bool work = ok && ax.rotated;
    const int nsteps = full ? TJ_W - 1 : TJ_BC;
    for (int s = 0; work && s < nsteps; ++s) {
        if (warp == 0) {
            int p, q;
            inner_pair(full, s, lane, p, q);
            const float a = G[p * TJ_GS + p].x, b = G[q * TJ_GS + q].x;
            const cf gam = G[p * TJ_GS + q];
            // per-step rotation decision in FP32 (the SIMT form's test)
            const bool rot = pair_cos2(gam, cabs2(gam), a, b) > tol2;
            float tp = 0.f;
            cf sg = cmake(0.f, 0.f);
            if (rot) {
                const Rot r = make_rot(a, b, gam);
                tp = r.tp;
                sg = r.sigma;
            }
            ax.tp[lane] = tp;
            ax.sigma[lane] = sg;
            ax.pp[lane] = p;
            ax.pq[lane] = q;
        }
        __syncthreads();
        // G <- R^H G R on the 2x2 blocks (pair a, pair b): 1024 blocks, 4 each
#pragma unroll 1
        for (int h = 0; h < 4; ++h) {
            const int a = tid >> 3, b = (tid & 7) * 4 + h;
            const int pa = ax.pp[a], qa = ax.pq[a], pb = ax.pp[b], qb = ax.pq[b];
            const float ta = ax.tp[a], tb = ax.tp[b];
            const cf sa = ax.sigma[a], sb = ax.sigma[b];
            if (ta == 0.f && tb == 0.f && sa.x == 0.f && sa.y == 0.f && sb.x == 0.f && sb.y == 0.f)
                continue;
            cf m00 = G[pa * TJ_GS + pb], m01 = G[pa * TJ_GS + qb];
            cf m10 = G[qa * TJ_GS + pb], m11 = G[qa * TJ_GS + qb];
            // Both sides in the implicit-c ("tau") form of rot.cuh, R = I + D
            // with D = [[-tp, conj(s)], [-s, -tp]]: an explicit c = 1 - tp
            // rounds to 1 for small angles and every such rotation would
            // inflate the norms.  M <- M R_b, then M <- R_a^H M.
            const cf n00 = csub(m00, cadd(cscale(m00, tb), cmul(m01, sb)));
            const cf n01 = cadd(m01, csub(cmul(m00, cconj(sb)), cscale(m01, tb)));
            const cf n10 = csub(m10, cadd(cscale(m10, tb), cmul(m11, sb)));
            const cf n11 = cadd(m11, csub(cmul(m10, cconj(sb)), cscale(m11, tb)));
            m00 = csub(n00, cadd(cscale(n00, ta), cmul(cconj(sa), n10)));
            m01 = csub(n01, cadd(cscale(n01, ta), cmul(cconj(sa), n11)));
            m10 = cadd(n10, csub(cmul(sa, n00), cscale(n10, ta)));
            m11 = cadd(n11, csub(cmul(sa, n01), cscale(n11, ta)));
            if (a == b) {                 // the rotated pair's own block
                m00.y = 0.f;
                m11.y = 0.f;
                if (ta != 0.f || sa.x != 0.f || sa.y != 0.f) {
                    m01 = cmake(0.f, 0.f);
                    m10 = cmake(0.f, 0.f);
                }
            }
            G[pa * TJ_GS + pb] = m00;
            G[pa * TJ_GS + qb] = m01;
            G[qa * TJ_GS + pb] = m10;
            G[qa * TJ_GS + qb] = m11;
        }
        // Q <- Q R kept as E = Q - I: rows r, pair b (2048 tasks, 8 each)
#pragma unroll 2
        for (int h = 0; h < 8; ++h) {
            const int task = tid + TJ_T * h;
            const int b = task & 31, r = task >> 5;
            const float tb = ax.tp[b];
            const cf sb = ax.sigma[b];
            if (tb == 0.f && sb.x == 0.f && sb.y == 0.f) continue;
            const int pb = ax.pp[b], qb = ax.pq[b];
            const cf ex = Q[r * TJ_QS + pb], ey = Q[r * TJ_QS + qb];
            // tau form, as for G, on Q's columns x = e_pb + E[:, pb],
            // y = e_qb + E[:, qb]; the identity is added back here only
            const cf x = cmake(ex.x + (r == pb ? 1.f : 0.f), ex.y);
            const cf y = cmake(ey.x + (r == qb ? 1.f : 0.f), ey.y);
            Q[r * TJ_QS + pb] = csub(ex, cadd(cscale(x, tb), cmul(y, sb)));
            Q[r * TJ_QS + qb] = cadd(ey, csub(cmul(x, cconj(sb)), cscale(y, tb)));
        }
        __syncthreads();
    }

    const long long c2 = clock64();
    // new squared norms for the next sweep's sort (a visit with nothing to
    // rotate leaves them as they were), and this visit's largest cosine
    if (work && tid < TJ_W) {
        const int col = ax.col[tid];
        if (col >= 0) g.cnrm[(size_t)j * g.cslot + col] = G[tid * TJ_GS + tid].x;
    }
    if (ok && tid == 0 && ax.rotated)
        atomicMax(reinterpret_cast<int*>(g.offmax + j), __float_as_int(ax.cmax));

    // ---- 3. Y <- Y + Y E ---------------------------------------------------
    if (work) {
        // B pieces in R0: element (q, k) of piece i at i*16K + (k/64)*8K +
        // sw128_off(q, k % 64); k < 64: Re E[k][q], k >= 64: -Im E[k-64][q].
        // Task (q, k-group of 8): 64 x 16 = 1024 tasks, 4 each.
        __syncthreads();
#pragma unroll 1
        for (int h = 0; h < 4; ++h) {
            const int task = tid + TJ_T * h;
            const int q = task & 63, kg = task >> 6;       // kg in 0..15
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int k = kg * 8 + e;
                const cf x = Q[(k & 63) * TJ_QS + q];
                v[e] = k < 64 ? x.x : -x.y;
            }
            put_pieces(R0, TJ_PIECE, (uint32_t)(kg >> 3) * 8192u + tc::sw128_off(q, (kg & 7) * 8), v);
        }
        __syncthreads();                                   // E (R1) is dead
        constexpr uint32_t IDESC_R = tc::idesc_bf16(128, 64, true, false);
        const int npair = lslot / 64;
        float y[4][8];
        load_rot_chunk(y, X, ax.col, lslot, 0, tid);
        for (int cp = 0; ok && cp < npair; ++cp) {
            // piece products smallest first: A2 B0 | A1 B1, A1 B0 | A0 B2, A0 B1,
            // A0 B0, each over all eight K steps, so that only the last eight
            // MMAs see a full-size accumulator
            for (int step = 0; step < 3 && ok; ++step) {
                const int ia = 2 - step;
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const int task = tid + TJ_T * h;
                    const int p = task >> 4, grp = task & 15;
                    const uint32_t mo = (uint32_t)(grp >> 3) * TJ_PIECE;
                    float t[8];
                    twist8(y[h], t);
                    put_piece(R1, mo + tc::sw128_off(p, (grp & 7) * 8), y[h], ia);
                    put_piece(R1, mo + tc::sw128_off(TJ_W + p, (grp & 7) * 8), t, ia);
                }
                tc::fence_async_smem();
                __syncthreads();
                if (tid == 0) {
                    tc::fence_after_sync();
                    const uint32_t sa = tc::smem_u32(R1), sb = tc::smem_u32(R0);
                    for (int ib = 2 - ia; ib >= 0; --ib)
#pragma unroll 1
                        for (int ks = 0; ks < 8; ++ks)
                            tc::mma_bf16(tmem, tc::sdesc(sa + ks * 2048, TJ_PIECE, 1024),
                                         tc::sdesc(sb + ib * TJ_PIECE + (ks >> 2) * 8192 +
                                                       (ks & 3) * 32, 16, 1024),
                                         IDESC_R, (step | ks | (ib != 2 - ia)) != 0);
                    tc::mma_commit(&ax.bar);
                }
                if (step == 2 && cp + 1 < npair) {
                    // the current values were written for the last time: the
                    // next chunk's loads overlap the last MMAs
                    load_rot_chunk(y, X, ax.col, lslot, cp + 1, tid);
                }
                ok = __syncthreads_and(wait_mma(&ax.bar, phase)) != 0;
            }
            if (!ok) break;
            tc::fence_after_sync();
            // epilogue: lane = real index within the 128 reals of rows 64cp..;
            // Y + D with FP32 round-to-nearest
            {
                const int mreal = 32 * (warp & 3) + lane;
                const int q0 = 32 * (warp >> 2);
                float v[32];
                tc::tmem_ld32(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + q0, v);
#pragma unroll
                for (int e = 0; e < 32; ++e) {
                    const int col = ax.col[q0 + e];
                    if (col >= 0) {
                        float* dst = X + ((size_t)col * lslot + (size_t)cp * 64) * 2 + mreal;
                        *dst = __ldcg(dst) + v[e];
                    }
                }
            }
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
        }
    }
    if (!ok && tid == 0) atomicExch(g.counter + 3, 1);     // an MMA wait expired
    if (tid == 0) {
        const long long c3 = clock64();
        atomicAdd(&g_tj_cycles[0], (unsigned long long)(c1 - c0));
        atomicAdd(&g_tj_cycles[1], (unsigned long long)(c2 - c1));
        atomicAdd(&g_tj_cycles[2], (unsigned long long)(c3 - c2));
        atomicAdd(&g_tj_cycles[3], 1ull);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TJ_TMEM_COLS);
}

}  // namespace

int tc_sweep_launch(const mps_2q_job* jobs, int njobs, int rounds, int pairs, const TwoQGeom& g,
                    float tol2, cudaStream_t s) {
    static KernelSetup ks;
    int dev = 0;
    MPS_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(MPS_ERR_ARG, "device index beyond 63");
    std::call_once(ks.once[dev], [&] {
        cudaError_t e = cudaFuncSetAttribute(tc_visit_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)TJ_SMEM);
        ks.rc[dev] = e == cudaSuccess ? MPS_OK : cuda_fail(e, "cudaFuncSetAttribute(tc_visit_kernel)");
    });
    if (ks.rc[dev] != MPS_OK) return ks.rc[dev];
    if (g.lslot % 64 != 0) return fail(MPS_ERR_ARG, "tc sweeps: slot rows must be a multiple of 64");
    for (int r = 0; r < rounds; ++r) {
        tc_visit_kernel<<<dim3(pairs, njobs), TJ_T, TJ_SMEM, s>>>(jobs, g, r, (double)tol2, tol2);
        MPS_LAUNCH_CHECK("tc_visit_kernel");
    }
    return MPS_OK;
}

}  // namespace mps

// Per-step cycle totals of the tensor-core visits (see g_tj_cycles); reset
// after reading when reset != 0.  Blocks.
extern "C" int mps_tc_profile(unsigned long long* out4, int reset) {
    unsigned long long v[4] = {0, 0, 0, 0};
    MPS_CUDA_CHECK(cudaMemcpyFromSymbol(v, mps::g_tj_cycles, sizeof(v)));
    if (reset) {
        const unsigned long long z[4] = {0, 0, 0, 0};
        MPS_CUDA_CHECK(cudaMemcpyToSymbol(mps::g_tj_cycles, z, sizeof(z)));
    }
    if (out4)
        for (int i = 0; i < 4; ++i) out4[i] = v[i];
    return MPS_OK;
}
