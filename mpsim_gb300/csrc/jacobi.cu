// Truncated SVD of the merged two-site matrix by block one-sided (Hestenes)
// Jacobi, with an in-kernel descending sort, truncation to k values and the
// regauge that places the singular values left or right.
//
// Replaces TensorNetwork's split_node_full_svd(..., max_singular_values=k)
// (mpsim/core.py:1132-1137; LAPACK gesdd underneath) and the contraction of
// S into one side (core.py:1139-1145).
//
// Algorithm.  The C columns of X are split into nb blocks of BC columns
// (zero-padded).  A sweep is nb-1 rounds of nb/2 disjoint block pairs
// (circle-method round robin), so every pair of columns is rotated exactly
// once per sweep.  One persistent launch runs a whole sweep: CTAs take
// (round, job, block pair) items in round-major order and wait (bounded) for
// the two blocks' previous round.
//  * round 0 ("full" visit): the CTA stages its 2*BC columns in shared memory
//    and rotates all pairs among them -- the intra-block pairs of every block
//    (round 0's pairs cover each block once) and the first inter-block pairs;
//  * rounds 1..nb-2 ("ring" visit): only the BC*BC inter-block pairs.  Warp w
//    keeps home column I*BC+w in registers and meets the J columns in turn;
//    in the sweep kernel the J columns stay in shared memory and pass from
//    warp to warp through per-column mbarriers (visit_ring_handoff); the
//    per-round kernels pass them through double-buffered slots (visit_ring).
// For a pair (x, q) with gamma = x^H q, alpha = |x|^2, beta = |q|^2 the
// rotation zeroes gamma:
//   zeta = (beta - alpha) / (2|gamma|), t = sign(zeta)/(|zeta| + sqrt(1+zeta^2)),
//   c = 1/sqrt(1+t^2), s = c t, sigma = s conj(gamma)/|gamma|, tp = s^2/(1+c),
//   x <- x - (tp x + sigma q),   q <- q + (conj(sigma) x - tp q).
// Keeping c implicit as 1 - tp matters: with an explicit c, tiny angles round
// c up to exactly 1 and every such rotation grows the column norms; over
// thousands of rotations that biases every singular value.  A pair is rotated
// only when |gamma|^2 > tol^2 alpha beta (tol = 2^-24 max(8, sqrt(L)) by
// default); a sweep with no rotation in a job marks the job converged.
// Column norms are recomputed from the data at every visit, so they do not
// drift.
//
// V.  A job that is tall (m >= n) and left-canonical -- the default of
// apply_two_qudit_gate -- needs only U = X_k / S: one Newton-Schulz step makes
// U an isometry to rounding, and its right site S V^H equals U^H theta, one
// GEMM against a copy of theta, so such jobs never accumulate V.  Other jobs accumulate the 2BC x 2BC rotation of each visit in
// shared memory and apply V <- V Q.
//
// Afterwards sigma_c = |X_c|, sorted descending (ties by column index); the
// first k are kept.  Where the isometric factor would divide by an exact-zero
// singular value, an orthonormal completion (classical Gram-Schmidt, twice) is
// written instead -- LAPACK also returns orthonormal singular vectors for zero
// singular values, and which ones it returns does not change any later
// singular value of the state.
#include <mutex>
#include <string>

#include "rot.cuh"
#include "twoq.cuh"

namespace mps {

namespace {

struct JobShape {
    int m, n, L, C, nb;
    bool tall, track_v;
};

template <int BC>
__device__ __forceinline__ JobShape job_shape(const mps_2q_job* jobs, int j, int d) {
    JobShape s;
    s.m = jobs[j].chi_l * d;
    s.n = jobs[j].chi_r * d;
    s.L = max(s.m, s.n);
    s.C = min(s.m, s.n);
    s.tall = s.m >= s.n;
    s.track_v = job_tracks_v(s.m, s.n, jobs[j].keep_left_canonical);
    int nb = (s.C + BC - 1) / BC;
    if (nb < 2) nb = 2;
    s.nb = nb + (nb & 1);
    return s;
}

__device__ __forceinline__ int block_col(int c, int I, int J, int BC) {
    return (c < BC) ? I * BC + c : J * BC + (c - BC);
}

// Physical column of job j at sorted position c.  The columns are never
// moved: the per-sweep norm sort rewrites this map instead (positions >= C,
// the zero padding, always map to themselves).
__device__ __forceinline__ int phys_col(const TwoQGeom& g, int j, int c) {
    return __ldcg(g.cmap + (size_t)j * g.cslot + c);
}

// V <- V Q for the 2*BC columns of this visit (rows < C).
template <int BC>
__device__ __forceinline__ void update_v(const TwoQGeom& g, int j, int C, int I, int J,
                                         const cf* Qs) {
    constexpr int W = 2 * BC;
    const int cslot = g.cslot;
    cf* V = g.V + (size_t)j * cslot * cslot;
    for (int r = threadIdx.x; r < C; r += BC * 32) {
        cf v[W];
#pragma unroll
        for (int c = 0; c < W; ++c)
            v[c] = __ldcg(V + (size_t)phys_col(g, j, block_col(c, I, J, BC)) * cslot + r);
#pragma unroll 4
        for (int c2 = 0; c2 < W; ++c2) {
            cf acc = cmake(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < W; ++c) cfma(acc, v[c], Qs[c2 * W + c]);
            V[(size_t)phys_col(g, j, block_col(c2, I, J, BC)) * cslot + r] = acc;
        }
    }
}

__device__ __forceinline__ void publish_offmax(float offmax, float* s_off, int nwarps, float* dst) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    offmax = warp_max(offmax);
    if (lane == 0) s_off[warp] = offmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        float o = 0.f;
        for (int w = 0; w < nwarps; ++w) o = fmaxf(o, s_off[w]);
        atomicMax(reinterpret_cast<int*>(dst), __float_as_int(o));
    }
}

// ---------------------------------------------------------------------------
// Round 0: all pairs among the 2*BC staged columns.  ROWS = rows per lane
// held in registers (working column length Lw <= 32*ROWS).
// Loads of X and V use __ldcg (L2, bypassing L1): inside the persistent
// sweep kernel another CTA may have rewritten a column since this SM last
// cached it.
// Returns whether any pair rotated (the same on every thread).
template <int BC, int ROWS>
__device__ __forceinline__ bool visit_full(const mps_2q_job* __restrict__ jobs, const TwoQGeom& g,
                                           int j, int round, int pair, float tol2, float2* smem,
                                           float* s_off) {
    if (g.done[j]) return false;
    const JobShape sh = job_shape<BC>(jobs, j, g.d);
    if (sh.C < 2) return false;
    if (round >= sh.nb - 1 || pair >= sh.nb / 2) return false;
    int I, J;
    tournament_pair(sh.nb, round, pair, I, J);
    const int Lw = (sh.L + 31) & ~31;
    constexpr int W = 2 * BC;
    cf* X = g.X + (size_t)j * g.lslot * g.cslot;
    cf* Xs = smem;                              // [W][Lw]
    cf* Qs = smem + (size_t)W * Lw;             // [W][W], column-major
    float* nrm = reinterpret_cast<float*>(Qs + W * W);   // [W]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = warp; c < W; c += BC) {
        const cf* src = X + (size_t)phys_col(g, j, block_col(c, I, J, BC)) * g.lslot;
        for (int r = lane; r < Lw; r += 32) Xs[(size_t)c * Lw + r] = __ldcg(src + r);
    }
    if (sh.track_v)
        for (int e = tid; e < W * W; e += BC * 32)
            Qs[e] = (e % W == e / W) ? cmake(1.f, 0.f) : cmake(0.f, 0.f);
    __syncthreads();
    for (int c = warp; c < W; c += BC) {
        float s = 0.f;
        for (int r = lane; r < Lw; r += 32) s += cabs2(Xs[(size_t)c * Lw + r]);
        s = warp_sum(s);
        if (lane == 0) nrm[c] = s;
    }
    __syncthreads();

    float offmax = 0.f;
    bool rotated = false;
    for (int step = 0; step < W - 1; ++step) {
        int p, q;
        tournament_pair(W, step, warp, p, q);
        cf* cp = Xs + (size_t)p * Lw;
        cf* cq = Xs + (size_t)q * Lw;
        const float a = nrm[p], b = nrm[q];
        cf xp[ROWS], xq[ROWS];
        cf gam = cmake(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < ROWS; ++i) {
            const int r = lane + 32 * i;
            xp[i] = r < Lw ? cp[r] : cmake(0.f, 0.f);
            xq[i] = r < Lw ? cq[r] : cmake(0.f, 0.f);
            cfma_conj(gam, xp[i], xq[i]);
        }
        gam.x = warp_sum(gam.x);
        gam.y = warp_sum(gam.y);
        const float g2 = cabs2(gam);
        const float r2 = pair_cos2(gam, g2, a, b);
        offmax = fmaxf(offmax, r2);
        if (r2 > tol2) {                        // warp-uniform (butterfly sums)
            const Rot R = make_rot(a, b, gam);
            float na = 0.f, nq = 0.f;
#pragma unroll
            for (int i = 0; i < ROWS; ++i) {
                const int r = lane + 32 * i;
                apply_rot(R, xp[i], xq[i]);
                if (r < Lw) {
                    cp[r] = xp[i];
                    cq[r] = xq[i];
                }
                na += cabs2(xp[i]);
                nq += cabs2(xq[i]);
            }
            na = warp_sum(na);
            nq = warp_sum(nq);
            rotated = true;
            if (sh.track_v && lane < W) {
                cf qa = Qs[p * W + lane], qb = Qs[q * W + lane];
                apply_rot(R, qa, qb);
                Qs[p * W + lane] = qa;
                Qs[q * W + lane] = qb;
            }
            __syncwarp();
            if (lane == 0) {
                nrm[p] = na;
                nrm[q] = nq;
            }
        }
        __syncthreads();
    }
    const bool any = __syncthreads_or(rotated ? 1 : 0) != 0;
    for (int c = warp; c < W; c += BC) {
        const int pc = phys_col(g, j, block_col(c, I, J, BC));
        if (any) {
            cf* dst = X + (size_t)pc * g.lslot;
            for (int r = lane; r < Lw; r += 32) dst[r] = Xs[(size_t)c * Lw + r];
        }
        if (lane == 0) g.cnrm[(size_t)j * g.cslot + pc] = nrm[c];
    }
    if (sh.track_v && any) update_v<BC>(g, j, sh.C, I, J, Qs);
    publish_offmax(offmax, s_off, BC, g.offmax + j);
    return any;
}

template <int BC, int ROWS>
__global__ void __launch_bounds__(BC * 32)
full_visit_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int round, float tol2) {
    extern __shared__ float2 smem[];
    __shared__ float s_off[BC];
    visit_full<BC, ROWS>(jobs, g, blockIdx.y, round, blockIdx.x, tol2, smem, s_off);
}

// ---------------------------------------------------------------------------
// Rounds >= 1: the BC*BC pairs between block I (home, warp w holds column
// I*BC+w) and block J (visitors, passed to warp w+1 after every step).
template <int BC, int ROWS>
__device__ __forceinline__ void visit_ring(const mps_2q_job* __restrict__ jobs, const TwoQGeom& g,
                                           int j, int round, int pair, float tol2, float2* smem,
                                           float* s_off) {
    // Every slot column has exactly 32*ROWS rows (lslot == 32*ROWS) and rows
    // past the job's length are zero, so no row is predicated: zero rows stay
    // zero under every rotation.
    if (g.done[j]) return;
    const JobShape sh = job_shape<BC>(jobs, j, g.d);
    if (sh.C < 2) return;
    if (round >= sh.nb - 1 || pair >= sh.nb / 2) return;
    int I, J;
    tournament_pair(sh.nb, round, pair, I, J);
    constexpr int LW = 32 * ROWS;
    constexpr int W = 2 * BC;
    cf* X = g.X + (size_t)j * g.lslot * g.cslot;
    cf* ring = smem;                            // [2][BC][LW], double-buffered
    cf* Qs = smem + (size_t)2 * BC * LW;        // [W][W], column-major
    float* ringn = reinterpret_cast<float*>(Qs + W * W);  // [2][BC]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    cf hx[ROWS], vx[ROWS];
    float hn = 0.f, vn = 0.f;
    {
        const cf* hs = X + (size_t)phys_col(g, j, I * BC + warp) * g.lslot;
        const cf* vs = X + (size_t)phys_col(g, j, J * BC + warp) * g.lslot;
#pragma unroll
        for (int i = 0; i < ROWS; ++i) {
            hx[i] = __ldcg(hs + lane + 32 * i);
            vx[i] = __ldcg(vs + lane + 32 * i);
            hn += cabs2(hx[i]);
            vn += cabs2(vx[i]);
        }
        hn = warp_sum(hn);
        vn = warp_sum(vn);
    }
    if (sh.track_v) {
        for (int e = tid; e < W * W; e += BC * 32)
            Qs[e] = (e % W == e / W) ? cmake(1.f, 0.f) : cmake(0.f, 0.f);
        __syncthreads();
    }
    float offmax = 0.f;
    int vid = warp;                             // J-local index of the visitor held
    for (int step = 0; step < BC; ++step) {
        cf gam = cmake(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < ROWS; ++i) cfma_conj(gam, hx[i], vx[i]);
        gam.x = warp_sum(gam.x);
        gam.y = warp_sum(gam.y);
        const float g2 = cabs2(gam);
        const float r2 = pair_cos2(gam, g2, hn, vn);
        offmax = fmaxf(offmax, r2);
        if (r2 > tol2) {
            const Rot R = make_rot(hn, vn, gam);
#pragma unroll
            for (int i = 0; i < ROWS; ++i) apply_rot(R, hx[i], vx[i]);
            // closed-form norm update (Hestenes): |x'|^2 = |x|^2 - t|gamma|,
            // |q'|^2 = |q|^2 + t|gamma|; recompute when cancellation leaves
            // less than 1/16 of a norm (warp-uniform decision)
            const float dn = R.dn;
            float na = hn - dn, nq = vn + dn;
            if (na < 0.0625f * hn || nq < 0.0625f * vn) {
                na = 0.f;
                nq = 0.f;
#pragma unroll
                for (int i = 0; i < ROWS; ++i) {
                    na += cabs2(hx[i]);
                    nq += cabs2(vx[i]);
                }
                na = warp_sum(na);
                nq = warp_sum(nq);
            }
            hn = na;
            vn = nq;
            if (sh.track_v && lane < W) {
                cf qa = Qs[warp * W + lane], qb = Qs[(BC + vid) * W + lane];
                apply_rot(R, qa, qb);
                Qs[warp * W + lane] = qa;
                Qs[(BC + vid) * W + lane] = qb;
            }
        }
        if (step + 1 < BC) {
            // Pass the visitor to warp+1 through buffer (step & 1).  One
            // barrier per step suffices: a warp writes buffer b again only
            // two steps later, after the next barrier, by which time every
            // warp has read its slot of b.
            const int buf = step & 1;
            const int to = (warp + 1) % BC;
            cf* dst = ring + ((size_t)buf * BC + to) * LW;
#pragma unroll
            for (int i = 0; i < ROWS; ++i) dst[lane + 32 * i] = vx[i];
            if (lane == 0) ringn[buf * BC + to] = vn;
            __syncthreads();
            const cf* src = ring + ((size_t)buf * BC + warp) * LW;
#pragma unroll
            for (int i = 0; i < ROWS; ++i) vx[i] = src[lane + 32 * i];
            vn = ringn[buf * BC + warp];
            vid = (vid + BC - 1) % BC;
        }
    }
    {
        const int ph = phys_col(g, j, I * BC + warp), pv = phys_col(g, j, J * BC + vid);
        cf* hd = X + (size_t)ph * g.lslot;
        cf* vd = X + (size_t)pv * g.lslot;
#pragma unroll
        for (int i = 0; i < ROWS; ++i) {
            hd[lane + 32 * i] = hx[i];
            vd[lane + 32 * i] = vx[i];
        }
        if (lane == 0) {
            g.cnrm[(size_t)j * g.cslot + ph] = hn;
            g.cnrm[(size_t)j * g.cslot + pv] = vn;
        }
    }
    if (sh.track_v) {
        __syncthreads();
        update_v<BC>(g, j, sh.C, I, J, Qs);
    }
    publish_offmax(offmax, s_off, BC, g.offmax + j);
}

// Two adjacent rows (2k, 2k+1) of a column as one 16-byte access: global
// through L2 only (another CTA may have rewritten the column), or shared.
__device__ __forceinline__ void ld_pair(const cf* col, int k, cf& a, cf& b) {
    const float4 t = __ldcg(reinterpret_cast<const float4*>(col) + k);
    a = cmake(t.x, t.y);
    b = cmake(t.z, t.w);
}
__device__ __forceinline__ void lds_pair(const cf* col, int k, cf& a, cf& b) {
    const float4 t = reinterpret_cast<const float4*>(col)[k];
    a = cmake(t.x, t.y);
    b = cmake(t.z, t.w);
}
__device__ __forceinline__ void st_pair(cf* col, int k, cf a, cf b) {
    reinterpret_cast<float4*>(col)[k] = make_float4(a.x, a.y, b.x, b.y);
}

// The same BC*BC pairs for the persistent sweep kernel, with the J columns
// kept in shared memory instead of travelling warp to warp: at step s warp w
// takes visitor (w - s) mod BC (the order of visit_ring), so visitor v passes
// from warp w-1 (step s-1) to warp w (step s).  The hand-off is one
// mbarrier per (step, visitor), bars[s * BC + v] with arrival count 1: the
// owner at step s arrives after its last access and the owner at step s+1
// waits on it, suspended in hardware rather than spinning, so a warp waits
// only for its neighbour instead of for the whole CTA every step and the
// warps' dot-product, angle and rotation phases overlap.  (One barrier per
// visitor would not do: a warp may reach step s while the visitor's step s-2
// arrival is still missing, and a parity wait cannot tell that phase from the
// awaited one.)  Each barrier completes exactly one phase per visit, so the
// phase awaited is the parity of the number of ring visits this CTA has made,
// which the caller keeps in `parity` and this function flips.  A visitor that
// was not rotated is not written back to shared memory, and a visit that
// rotated nothing writes nothing back to global memory.  Each wait gives up after kHandoffTries suspended tries;
// then it sets *err and goes on without waiting (the call reports a timeout
// and its results are not used), so every warp still reaches the CTA
// barriers.
constexpr int kHandoffTries = 1 << 18;
constexpr unsigned kHandoffSuspendNs = 1000;

template <int BC, int ROWS>
__device__ __forceinline__ bool visit_ring_handoff(const mps_2q_job* __restrict__ jobs,
                                                   const TwoQGeom& g, int j, int round, int pair,
                                                   float tol2, float2* smem, float* s_off,
                                                   uint64_t* bars, unsigned& parity, int* err) {
    if (g.done[j]) return false;
    const JobShape sh = job_shape<BC>(jobs, j, g.d);
    if (sh.C < 2) return false;
    if (round >= sh.nb - 1 || pair >= sh.nb / 2) return false;
    int I, J;
    tournament_pair(sh.nb, round, pair, I, J);
    constexpr int LW = 32 * ROWS;
    constexpr int W = 2 * BC;
    static_assert((BC & (BC - 1)) == 0, "BC must be a power of two");
    cf* X = g.X + (size_t)j * g.lslot * g.cslot;
    cf* vis = smem;                             // [BC][LW]
    cf* Qs = smem + (size_t)BC * LW;            // [W][W], column-major
    float* visn = reinterpret_cast<float*>(Qs + W * W);   // [BC]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    cf hx[ROWS], vx[ROWS];
    float hn = 0.f;
    {
        const cf* hs = X + (size_t)phys_col(g, j, I * BC + warp) * g.lslot;
        const cf* vs = X + (size_t)phys_col(g, j, J * BC + warp) * g.lslot;
        cf* vd = vis + (size_t)warp * LW;
        float vn = 0.f;
#pragma unroll
        for (int i = 0; i < ROWS / 2; ++i) {
            ld_pair(hs, lane + 32 * i, hx[2 * i], hx[2 * i + 1]);
            ld_pair(vs, lane + 32 * i, vx[2 * i], vx[2 * i + 1]);
            st_pair(vd, lane + 32 * i, vx[2 * i], vx[2 * i + 1]);
        }
#pragma unroll
        for (int i = 0; i < ROWS; ++i) {
            hn += cabs2(hx[i]);
            vn += cabs2(vx[i]);
        }
        hn = warp_sum(hn);
        vn = warp_sum(vn);
        if (lane == 0) visn[warp] = vn;
    }
    if (sh.track_v)
        for (int e = tid; e < W * W; e += BC * 32)
            Qs[e] = (e % W == e / W) ? cmake(1.f, 0.f) : cmake(0.f, 0.f);
    __syncthreads();
    float offmax = 0.f;
    bool expired = false, rotated = false;
    for (int step = 0; step < BC; ++step) {
        const int v = (warp + BC - step) & (BC - 1);
        cf* vcol = vis + (size_t)v * LW;
        if (step > 0) {
            // visitor v was processed by warp-1 at step-1; the vote keeps
            // the try count, and so the expiry, uniform across the warp
            uint64_t* bar = bars + (step - 1) * BC + v;
            int tries = 0;
            while (!expired &&
                   !__all_sync(0xffffffffu, mbar_try_wait(bar, parity, kHandoffSuspendNs))) {
                if (++tries > kHandoffTries) expired = true;
            }
#pragma unroll
            for (int i = 0; i < ROWS / 2; ++i) lds_pair(vcol, lane + 32 * i, vx[2 * i], vx[2 * i + 1]);
        }
        const float vn = visn[v];
        cf gam = cmake(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < ROWS; ++i) cfma_conj(gam, hx[i], vx[i]);
        gam.x = warp_sum(gam.x);
        gam.y = warp_sum(gam.y);
        const float g2 = cabs2(gam);
        const float r2 = pair_cos2(gam, g2, hn, vn);
        offmax = fmaxf(offmax, r2);
        if (r2 > tol2) {                        // warp-uniform (butterfly sums)
            const Rot R = make_rot(hn, vn, gam);
#pragma unroll
            for (int i = 0; i < ROWS; ++i) apply_rot(R, hx[i], vx[i]);
#pragma unroll
            for (int i = 0; i < ROWS / 2; ++i) st_pair(vcol, lane + 32 * i, vx[2 * i], vx[2 * i + 1]);
            // closed-form norm update, recomputed on cancellation (as in
            // visit_ring)
            const float dn = R.dn;
            float na = hn - dn, nq = vn + dn;
            if (na < 0.0625f * hn || nq < 0.0625f * vn) {
                na = 0.f;
                nq = 0.f;
#pragma unroll
                for (int i = 0; i < ROWS; ++i) {
                    na += cabs2(hx[i]);
                    nq += cabs2(vx[i]);
                }
                na = warp_sum(na);
                nq = warp_sum(nq);
            }
            hn = na;
            rotated = true;
            if (lane == 0) visn[v] = nq;
            if (sh.track_v && lane < W) {
                cf qa = Qs[warp * W + lane], qb = Qs[(BC + v) * W + lane];
                apply_rot(R, qa, qb);
                Qs[warp * W + lane] = qa;
                Qs[(BC + v) * W + lane] = qb;
            }
        }
        __syncwarp();
        if (lane == 0 && step + 1 < BC) mbar_arrive(bars + step * BC + v);
    }
    parity ^= 1u;
    if (expired && lane == 0) atomicExch(err, 1);
    const bool any = __syncthreads_or(rotated ? 1 : 0) != 0;
    const int ph = phys_col(g, j, I * BC + warp), pv = phys_col(g, j, J * BC + warp);
    if (any) {
        cf* hd = X + (size_t)ph * g.lslot;
        cf* vd = X + (size_t)pv * g.lslot;
        const cf* vsrc = vis + (size_t)warp * LW;
#pragma unroll
        for (int i = 0; i < ROWS / 2; ++i) {
            st_pair(hd, lane + 32 * i, hx[2 * i], hx[2 * i + 1]);
            reinterpret_cast<float4*>(vd)[lane + 32 * i] =
                reinterpret_cast<const float4*>(vsrc)[lane + 32 * i];
        }
    }
    if (lane == 0) {       // the norms the next sweep's sort reads
        g.cnrm[(size_t)j * g.cslot + ph] = hn;
        g.cnrm[(size_t)j * g.cslot + pv] = visn[warp];
    }
    if (sh.track_v && any) update_v<BC>(g, j, sh.C, I, J, Qs);
    publish_offmax(offmax, s_off, BC, g.offmax + j);
    return any;
}

template <int BC, int ROWS>
__global__ void __launch_bounds__(BC * 32)
ring_visit_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int round, float tol2) {
    extern __shared__ float2 smem[];
    __shared__ float s_off[BC];
    visit_ring<BC, ROWS>(jobs, g, blockIdx.y, round, blockIdx.x, tol2, smem, s_off);
}

// ---------------------------------------------------------------------------
// One whole sweep in one launch.  Persistent CTAs take items (round, job,
// block pair) in round-major order from an atomic counter; an item of round
// r > 0 first waits until both of its blocks have finished round r-1.  All
// items of round r-1 are handed out before any item of round r and a CTA
// holds one item at a time, so every awaited item is held by a running CTA:
// no deadlock, whatever number of CTAs is resident.  The wait polls a flag
// at most wait_limit times (with __nanosleep backoff); on expiry it raises
// the error flag and the CTA leaves, as do the others once they see it.
//
// A visit is skipped when it would rotate nothing for certain: its last run
// (the same round and pair in an earlier sweep, at time qstamp) rotated
// nothing, and neither block has changed since (vstamp older than qstamp:
// no visit rotated it and the per-sweep sort kept its set of columns).  Its
// pairs then hold the same bits that were checked, so the visit would find
// every one below the threshold again.  A skipped item still waits for its
// blocks and publishes its round.  tbase = sweep * (rounds + 1).
template <int BC, int ROWS>
__global__ void __launch_bounds__(BC * 32)
sweep_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, float tol2, int njobs, int rounds,
             int pairs, SweepSync sync, int tbase) {
    extern __shared__ float2 smem[];
    __shared__ float s_off[BC];
    __shared__ int s_item, s_abort, s_skip;
    // a mixed call whose jobs all take the tensor-core sweeps: nothing to claim
    if (g.tc_mode && __ldcg(g.counter + 6) == 0) return;
    // ring hand-off barriers, one per (step < BC-1, visitor); see
    // visit_ring_handoff
    __shared__ __align__(8) uint64_t s_bar[(BC - 1) * BC];
    unsigned parity = 0;
    const int per_round = njobs * pairs;
    const int total = rounds * per_round;
    // the loop's first barrier orders the initialisation before any use
    for (int b = threadIdx.x; b < (BC - 1) * BC; b += blockDim.x) mbar_init(&s_bar[b], 1);
    for (;;) {
        if (threadIdx.x == 0) {
            s_item = atomicAdd(sync.next_item, 1);
            s_abort = *reinterpret_cast<volatile int*>(sync.error);
        }
        __syncthreads();
        const int item = s_item;
        if (item >= total || s_abort) return;
        const int r = item / per_round, rem = item - r * per_round;
        const int j = rem / pairs, p = rem - (rem / pairs) * pairs;
        bool active = !g.done[j];
        int I = 0, J = 0, nb = 2;
        if (active) {
            const JobShape sh = job_shape<BC>(jobs, j, g.d);
            nb = sh.nb;
            active = sh.C >= 2 && r < sh.nb - 1 && p < sh.nb / 2 &&
                     !(g.tc_mode && tc_job(sh.m, sh.n, jobs[j].keep_left_canonical));
            if (active) tournament_pair(sh.nb, r, p, I, J);
        }
        if (active) {
            // a job of one block pair has one visit per sweep, and a visit
            // that rotates nothing ends it: no stamps (and r > 0 implies nb > 2)
            const bool track = nb > 2;
            volatile int* vst = g.vstamp + (size_t)j * g.nbmax;
            volatile int* qst = g.qstamp + (size_t)j * g.qstride + r * pairs + p;
            if (track && threadIdx.x == 0) {
                // qstamp of this (round, pair) changes only when this item
                // runs, so it is read before the wait; the block stamps only
                // after it, and only when the visit was once quiet
                const int q = *qst;
                if (r > 0) {
                    volatile int* fl = sync.block_round + (size_t)j * sync.nbmax;
                    volatile int* err = sync.error;
                    // the test hook waits for a round no block ever reaches
                    const int need = (sync.stall_test && item == per_round) ? rounds + 1 : r - 1;
                    int polls = 0;
                    while ((fl[I] < need || fl[J] < need) && *err == 0) {
                        if (++polls > sync.wait_limit) {
                            atomicExch(sync.error, 1);
                            break;
                        }
                        __nanosleep(64);
                    }
                    s_abort = *err;
                    __threadfence();
                }
                s_skip = (q >= 0 && q > vst[I] && q > vst[J]) ? 1 : 0;
            }
            if (track) {
                __syncthreads();
                if (s_abort) return;
            }
            const bool skip = track && s_skip != 0;
            bool rot = false;
            if (!skip) {
                if (r == 0) rot = visit_full<BC, ROWS>(jobs, g, j, r, p, tol2, smem, s_off);
                else rot = visit_ring_handoff<BC, ROWS>(jobs, g, j, r, p, tol2, smem, s_off, s_bar,
                                                        parity, sync.error);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                if (track && !skip) {
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
}

__global__ void sweep_end_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int njobs,
                                 float tol2, const int* wait_error) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    // an expired round-dependency wait also marks every job's status (for
    // calls that do not read the error word back: stream capture)
    if (j == 0 && wait_error && *wait_error) atomicOr(g.counter + 3, 1);
    if (j >= njobs) return;
    if (!g.done[j]) {
        const float o = g.offmax[j];
        if (o > tol2) {
            atomicAdd(g.counter, 1);
            // mixed calls: jobs left for each sweep kernel (the host skips a
            // kernel with none)
            if (g.tc_mode)
                atomicAdd(g.counter + (tc_job(jobs[j].chi_l * g.d, jobs[j].chi_r * g.d,
                                              jobs[j].keep_left_canonical) ? 4 : 5), 1);
        } else {
            g.done[j] = 1;
        }
    }
    g.offmax[j] = 0.f;
}

__global__ void init_slots_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int njobs) {
    // V = identity for jobs that track V, identity column maps, bookkeeping
    // cleared
    const size_t per = (size_t)g.cslot * g.cslot;
    const size_t total = per * njobs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(e / per);
        if (!job_tracks_v(jobs[j].chi_l * g.d, jobs[j].chi_r * g.d, jobs[j].keep_left_canonical))
            continue;
        const size_t w = e % per;
        const int r = (int)(w % g.cslot), c = (int)(w / g.cslot);
        const cf v = (r == c) ? cmake(1.f, 0.f) : cmake(0.f, 0.f);
        g.V[e] = v;
    }
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)njobs * g.cslot;
         e += (size_t)gridDim.x * blockDim.x)
        g.cmap[e] = (int)(e % g.cslot);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < njobs) {
        g.done[t] = 0;
        g.offmax[t] = 0.f;
        g.need[t] = 0;
    }
    if (t < 8) g.counter[t] = 0;
}

// counter[6] = the jobs of a mixed call that take the SIMT sweeps (counted
// once, after init_slots_kernel cleared the counters; nothing resets it)
__global__ void count_simt_jobs_kernel(const mps_2q_job* __restrict__ jobs, int d, int njobs,
                                       int* counter) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < njobs && !tc_job(jobs[t].chi_l * d, jobs[t].chi_r * d, jobs[t].keep_left_canonical))
        atomicAdd(counter + 6, 1);
}

// ---------------------------------------------------------------------------
// Per-sweep reordering: columns sorted by descending norm before each sweep
// (de Rijk's ordering), which cuts the sweep count.  The columns stay where
// they are; presort_kernel sorts the squared norms the previous sweep's visits
// left in cnrm (theta_norm_kernel's before the first sweep) and rewrites the
// job's column map.  Converged jobs keep theirs, and so do the tensor-core
// jobs of a mixed call (see below).
constexpr int PRESORT_T = 512;

__global__ void __launch_bounds__(PRESORT_T)
presort_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int npow2, int bc, int tpre) {
    extern __shared__ float2 sm1[];
    float* key = reinterpret_cast<float*>(sm1);
    int* idx = reinterpret_cast<int*>(key + npow2);
    const int j = blockIdx.x;
    if (__ldg(g.done + j)) return;
    const int m = jobs[j].chi_l * g.d, n = jobs[j].chi_r * g.d;
    const int C = min(m, n);
    if (C < 2) return;
    // The tensor-core sweeps keep their columns in place: measured, their jobs
    // converge about a sweep sooner unsorted (the LQ factor's own column order,
    // and blocks that keep their columns keep their visits skippable), while
    // the SIMT sweeps gain from the sort.
    if (g.tc_mode && tc_job(m, n, jobs[j].keep_left_canonical)) return;
    const int tid = threadIdx.x;
    const float* cn = g.cnrm + (size_t)j * g.cslot;
    for (int i = tid; i < npow2; i += PRESORT_T) {
        float k = -1.f;
        if (i < C) {
            k = cn[i];
            if (!(k == k)) k = 0.f;                  // NaN sorts as zero
        }
        key[i] = k;
        idx[i] = i;
    }
    __syncthreads();
    for (int size = 2; size <= npow2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = tid; i < npow2; i += PRESORT_T) {
                const int pj = i ^ stride;
                if (pj > i) {
                    const bool desc = (i & size) == 0;
                    const float ki = key[i], kj = key[pj];
                    const int ii = idx[i], ij = idx[pj];
                    const bool i_first = (ki > kj) || (ki == kj && ii < ij);
                    if (i_first != desc) {
                        key[i] = kj; key[pj] = ki;
                        idx[i] = ij; idx[pj] = ii;
                    }
                }
            }
            __syncthreads();
        }
    }
    if (g.vstamp) {
        // a block whose set of columns changes counts as changed (its pairs
        // are not the ones last checked); moves inside a block do not
        int* oldpos = reinterpret_cast<int*>(key);     // the keys are no longer needed
        for (int i = tid; i < C; i += PRESORT_T) oldpos[__ldcg(g.cmap + (size_t)j * g.cslot + i)] = i;
        __syncthreads();
        int* vst = g.vstamp + (size_t)j * g.nbmax;
        for (int c = tid; c < C; c += PRESORT_T) {
            const int ob = oldpos[idx[c]] / bc, nb = c / bc;
            if (ob != nb) {
                vst[ob] = tpre;
                vst[nb] = tpre;
            }
        }
    }
    for (int i = tid; i < C; i += PRESORT_T) g.cmap[(size_t)j * g.cslot + i] = idx[i];
}

// ---------------------------------------------------------------------------
// Norms, descending sort, svals / discarded weight / status.  One CTA per job.
constexpr int SORT_T = 512;

__global__ void __launch_bounds__(SORT_T)
sort_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int npow2) {
    extern __shared__ float2 sm2[];
    float* key = reinterpret_cast<float*>(sm2);
    int* idx = reinterpret_cast<int*>(key + npow2);
    __shared__ double s_red[SORT_T / 32];
    __shared__ int s_bad;
    const int j = blockIdx.x;
    const mps_2q_job job = jobs[j];
    const int m = job.chi_l * g.d, n = job.chi_r * g.d;
    const int L = max(m, n), C = min(m, n);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const cf* X = g.X + (size_t)j * g.lslot * g.cslot;
    if (tid == 0) s_bad = 0;
    for (int i = tid; i < npow2; i += SORT_T) {
        key[i] = -1.f;
        idx[i] = i;
    }
    __syncthreads();
    for (int c = warp; c < C; c += SORT_T / 32) {
        float s = 0.f;
        for (int r = lane; r < L; r += 32) s += cabs2(X[(size_t)c * g.lslot + r]);
        s = warp_sum(s);
        if (lane == 0) {
            const float sg = sqrtf(s);
            if (!isfinite(sg)) atomicOr(&s_bad, 1);
            key[c] = isfinite(sg) ? sg : 0.f;
        }
    }
    __syncthreads();
    // bitonic sort: descending key, ascending index on ties
    for (int size = 2; size <= npow2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = tid; i < npow2; i += SORT_T) {
                const int pj = i ^ stride;
                if (pj > i) {
                    const bool desc = (i & size) == 0;
                    const float ki = key[i], kj = key[pj];
                    const int ii = idx[i], ij = idx[pj];
                    const bool i_first = (ki > kj) || (ki == kj && ii < ij);
                    if (i_first != desc) {
                        key[i] = kj; key[pj] = ki;
                        idx[i] = ij; idx[pj] = ii;
                    }
                }
            }
            __syncthreads();
        }
    }
    const int k = job.k;
    const float thr = kZeroSigma * fmaxf(C > 0 ? key[0] : 0.f, 1.f);
    for (int i = tid; i < C; i += SORT_T) {
        g.sig[(size_t)j * g.cslot + i] = key[i];
        g.perm[(size_t)j * g.cslot + i] = idx[i];
        if (job.svals) job.svals[i] = key[i];
    }
    double part = 0.0;
    for (int i = k + tid; i < C; i += SORT_T) part += (double)key[i] * (double)key[i];
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) s_red[warp] = part;
    __syncthreads();
    if (tid == 0) {
        double tot = 0.0;
        for (int w = 0; w < SORT_T / 32; ++w) tot += s_red[w];
        if (job.discarded) *job.discarded = tot;
        const bool tall = m >= n;
        const bool divides = tall ? (job.keep_left_canonical != 0) : (job.keep_left_canonical == 0);
        int need = 0;
        if (divides)
            for (int i = 0; i < k; ++i) need += (key[i] <= thr) ? 1 : 0;
        g.need[j] = need;
        int st = 0;
        if (!g.done[j]) st |= MPS_STATUS_NOT_CONVERGED;
        if (__ldcg(g.counter + 3)) st |= MPS_STATUS_TIMEOUT;
        if (s_bad) {
            st |= MPS_STATUS_NONFINITE;
            atomicAdd(g.counter + 1, 1);
        }
        if (job.status) *job.status = st;
    }
}

// a_out (m x k, row-major): a_out[row*k + i] = scale_i * src[perm_i * ld + row]
//   tall: src = X (U S columns), scale = 1/s (left-canonical) or 1
//   wide: src = V,               scale = 1 (left-canonical) or s
__global__ void regauge_a_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g) {
    __shared__ cf tile[32][33];
    const int j = blockIdx.z;
    const mps_2q_job job = jobs[j];
    const int m = job.chi_l * g.d, n = job.chi_r * g.d;
    const int k = job.k;
    const int i0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    if (i0 >= k || r0 >= m) return;
    const bool tall = m >= n;
    const bool lc = job.keep_left_canonical != 0;
    const cf* src;
    int ld;
    if (tall) { src = g.X + (size_t)j * g.lslot * g.cslot; ld = g.lslot; }
    else { src = g.V + (size_t)j * g.cslot * g.cslot; ld = g.cslot; }
    const float* sig = g.sig + (size_t)j * g.cslot;
    const int* perm = g.perm + (size_t)j * g.cslot;
    const float thr = kZeroSigma * fmaxf(sig[0], 1.f);
    const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
    for (int ii = ty; ii < 32; ii += 8) {
        const int i = i0 + ii, row = r0 + tx;
        cf v = cmake(0.f, 0.f);
        if (i < k && row < m) {
            const float s = sig[i];
            float sc;
            if (tall) sc = lc ? (s > thr ? 1.f / s : 0.f) : 1.f;
            else sc = lc ? 1.f : s;
            v = cscale(src[(size_t)perm[i] * ld + row], sc);
        }
        tile[ii][tx] = v;
    }
    __syncthreads();
    cf* out = reinterpret_cast<cf*>(job.a_out);
    for (int rr = ty; rr < 32; rr += 8) {
        const int row = r0 + rr, i = i0 + tx;
        if (row < m && i < k) out[(size_t)row * k + i] = tile[tx][rr];
    }
}

// b_out (k x n, row-major) for jobs that track V:
//   tall (right-canonical): b_out[i, :] = conj(V[:, perm_i])
//   wide: b_out[i, :] = scale_i * conj(X[:, perm_i]), scale = 1 (lc) or 1/s
__global__ void regauge_b_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g) {
    const int j = blockIdx.z;
    const mps_2q_job job = jobs[j];
    const int m = job.chi_l * g.d, n = job.chi_r * g.d;
    const int i = blockIdx.y;
    if (i >= job.k) return;
    if (!job_tracks_v(m, n, job.keep_left_canonical)) return;
    const bool tall = m >= n;
    const bool lc = job.keep_left_canonical != 0;
    const cf* src;
    int ld;
    if (tall) { src = g.V + (size_t)j * g.cslot * g.cslot; ld = g.cslot; }
    else { src = g.X + (size_t)j * g.lslot * g.cslot; ld = g.lslot; }
    const float* sig = g.sig + (size_t)j * g.cslot;
    const float thr = kZeroSigma * fmaxf(sig[0], 1.f);
    const float s = sig[i];
    float sc;
    if (tall) sc = 1.f;
    else sc = lc ? 1.f : (s > thr ? 1.f / s : 0.f);
    const cf* col = src + (size_t)g.perm[(size_t)j * g.cslot + i] * ld;
    cf* out = reinterpret_cast<cf*>(job.b_out) + (size_t)i * n;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        out[c] = cscale(cconj(col[c]), sc);
}

// Post-processing GEMMs for tall left-canonical jobs (the V-free path), all
// 64x64 output tiles, K in chunks of 16, 256 threads x 4x4 outputs:
//   POST_GRAM : G = U^H U          (k x k, into the job's V slot), U = a_out
//   POST_APPLY: U' = U (3I - G)/2  (m x k, into the job's X slot): one
//               Newton-Schulz step, which squares U's distance from an
//               isometry (the Jacobi tolerance) so U U^H is a projector to
//               rounding, as LAPACK's U would give
//   POST_UH   : S V^H = U'^H theta (k x n, into b_out), theta = the T copy
//   POST_COPY : a_out = U'
enum PostMode { POST_GRAM = 0, POST_APPLY = 1, POST_UH = 2 };

template <int MODE>
__global__ void __launch_bounds__(256)
post_gemm_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g) {
    __shared__ cf As[16][64];
    __shared__ cf Bs[16][64];
    const int j = blockIdx.z;
    const mps_2q_job job = jobs[j];
    const int m = job.chi_l * g.d, n = job.chi_r * g.d, k = job.k;
    if (job_tracks_v(m, n, job.keep_left_canonical)) return;
    int M, N, K;
    if (MODE == POST_GRAM) { M = k; N = k; K = m; }
    else if (MODE == POST_APPLY) { M = m; N = k; K = k; }
    else { M = k; N = n; K = m; }
    const int i0 = blockIdx.y * 64, c0 = blockIdx.x * 64;
    if (i0 >= M || c0 >= N) return;
    const cf* U = reinterpret_cast<const cf*>(job.a_out);          // m x k row-major
    cf* Gm = g.V + (size_t)j * g.cslot * g.cslot;                   // k x k row-major
    cf* Up = g.X + (size_t)j * g.lslot * g.cslot;                   // m x k row-major
    const cf* T = g.T + (size_t)j * g.lslot * g.cslot;              // theta, column-major
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    cf acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = cmake(0.f, 0.f);
    for (int l0 = 0; l0 < K; l0 += 16) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int idx = tid + q * 256;
            int ti, kk;
            if (MODE == POST_APPLY) { kk = idx & 15; ti = idx >> 4; }   // U rows: l contiguous
            else { ti = idx & 63; kk = idx >> 6; }                     // U^H: i contiguous
            const int i = i0 + ti, l = l0 + kk;
            cf v = cmake(0.f, 0.f);
            if (i < M && l < K) {
                if (MODE == POST_GRAM) v = cconj(U[(size_t)l * k + i]);
                else if (MODE == POST_APPLY) v = U[(size_t)i * k + l];
                else v = cconj(Up[(size_t)l * k + i]);
            }
            As[kk][ti] = v;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int idx = tid + q * 256;
            int tc, kk;
            if (MODE == POST_UH) { kk = idx & 15; tc = idx >> 4; }      // theta column-major
            else { tc = idx & 63; kk = idx >> 6; }
            const int c = c0 + tc, l = l0 + kk;
            cf v = cmake(0.f, 0.f);
            if (c < N && l < K) {
                if (MODE == POST_GRAM) v = U[(size_t)l * k + c];
                else if (MODE == POST_APPLY) {
                    const cf gl = Gm[(size_t)l * k + c];
                    v = cmake((l == c ? 1.5f : 0.f) - 0.5f * gl.x, -0.5f * gl.y);
                } else v = T[(size_t)c * g.lslot + l];
            }
            Bs[kk][tc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            cf av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = As[kk][ty + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) cfma(acc[a][b], av[a], bv[b]);
        }
        __syncthreads();
    }
    cf* out;
    size_t ld;
    if (MODE == POST_GRAM) { out = Gm; ld = (size_t)k; }
    else if (MODE == POST_APPLY) { out = Up; ld = (size_t)k; }
    else { out = reinterpret_cast<cf*>(job.b_out); ld = (size_t)n; }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int i = i0 + ty + 16 * a, c = c0 + tx + 16 * b;
            if (i < M && c < N) out[(size_t)i * ld + c] = acc[a][b];
        }
}

// a_out = U' (the X slot) for tall left-canonical jobs.
__global__ void post_copy_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g) {
    const int j = blockIdx.y;
    const mps_2q_job job = jobs[j];
    const int m = job.chi_l * g.d, n = job.chi_r * g.d;
    if (job_tracks_v(m, n, job.keep_left_canonical)) return;
    const size_t total = (size_t)m * job.k;
    const cf* src = g.X + (size_t)j * g.lslot * g.cslot;
    cf* dst = reinterpret_cast<cf*>(job.a_out);
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x)
        dst[e] = src[e];
}

int launch_post(const mps_2q_job* jobs, int njobs, int max_m, int max_n, int kmax,
                const TwoQGeom& g, cudaStream_t s) {
    post_gemm_kernel<POST_GRAM><<<dim3((kmax + 63) / 64, (kmax + 63) / 64, njobs), 256, 0, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("post_gemm_kernel<gram>");
    post_gemm_kernel<POST_APPLY><<<dim3((kmax + 63) / 64, (max_m + 63) / 64, njobs), 256, 0, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("post_gemm_kernel<apply>");
    post_gemm_kernel<POST_UH><<<dim3((max_n + 63) / 64, (kmax + 63) / 64, njobs), 256, 0, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("post_gemm_kernel<uh>");
    const size_t total = (size_t)max_m * kmax;
    int blocks = (int)((total + 255) / 256 < 1024 ? (total + 255) / 256 : 1024);
    post_copy_kernel<<<dim3(blocks > 0 ? blocks : 1, njobs), 256, 0, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("post_copy_kernel");
    return MPS_OK;
}

// Orthonormal completion of the isometric factor where sigma is an exact
// zero.  Vectors u_i (i < k): tall -> columns of a_out (R = m, element
// stride k); wide -> rows of b_out (R = n, element stride 1).  The columns
// needing completion are a suffix of the kept set (sigma sorted).
constexpr int COMP_T = 256;

__global__ void __launch_bounds__(COMP_T)
complete_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g) {
    extern __shared__ float2 sm3[];
    const int j = blockIdx.x;
    const int need = g.need[j];
    if (need == 0) return;
    const mps_2q_job job = jobs[j];
    const int m = job.chi_l * g.d, n = job.chi_r * g.d;
    const bool tall = m >= n;
    const int k = job.k;
    const int R = tall ? m : n;
    cf* base = reinterpret_cast<cf*>(tall ? job.a_out : job.b_out);
    const size_t es = tall ? (size_t)k : 1;     // element stride
    const size_t vs = tall ? 1 : (size_t)n;     // vector stride
    cf* v = sm3;                                // [R]
    cf* h = sm3 + R;                            // [k]
    __shared__ float s_nrm[COMP_T / 32];
    __shared__ int s_ok;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int cand = 0;
    for (int i = k - need; i < k; ++i) {
        for (;;) {
            if (cand >= R) return;              // unreachable: see the threshold below
            for (int e = tid; e < R; e += COMP_T) v[e] = cmake(e == cand ? 1.f : 0.f, 0.f);
            __syncthreads();
            for (int pass = 0; pass < 2; ++pass) {
                for (int t = warp; t < i; t += COMP_T / 32) {
                    cf acc = cmake(0.f, 0.f);
                    for (int e = lane; e < R; e += 32)
                        cfma_conj(acc, base[t * vs + e * es], v[e]);
                    acc.x = warp_sum(acc.x);
                    acc.y = warp_sum(acc.y);
                    if (lane == 0) h[t] = acc;
                }
                __syncthreads();
                for (int e = tid; e < R; e += COMP_T) {
                    cf acc = v[e];
                    for (int t = 0; t < i; ++t) acc = csub(acc, cmul(h[t], base[t * vs + e * es]));
                    v[e] = acc;
                }
                __syncthreads();
            }
            float s = 0.f;
            for (int e = tid; e < R; e += COMP_T) s += cabs2(v[e]);
            s = warp_sum(s);
            if (lane == 0) s_nrm[warp] = s;
            __syncthreads();
            if (tid == 0) {
                float tot = 0.f;
                for (int w = 0; w < COMP_T / 32; ++w) tot += s_nrm[w];
                s_nrm[0] = tot;
                // the residuals of all R candidates sum to R - i >= 1, so
                // some candidate always clears 0.5 / R
                s_ok = tot > 0.5f / (float)R;
            }
            __syncthreads();
            const float nv = s_nrm[0];
            const int ok = s_ok;
            ++cand;
            __syncthreads();
            if (ok) {
                const float inv = rsqrtf(nv);
                for (int e = tid; e < R; e += COMP_T) base[i * vs + e * es] = cscale(v[e], inv);
                __syncthreads();
                break;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Exact power-of-two scaling of every job's theta to a Frobenius norm in
// [1, 2) before the SVD, undone on the outputs afterwards.  A state whose norm
// has decayed through truncation (to 1e-9 at the end of a 64-qubit, depth-40,
// maxsvals=256 circuit) gives squared column norms near 1e-19 and |gamma|^2
// below the smallest normal float, where FP32 keeps only a few bits; LAPACK,
// which the reference uses, scales for the same reason.  Multiplying by a
// power of two changes no bit of the relative arithmetic.

// Warp per column: squared column norms (FP64 sums) into cnrm, for the first
// sweep's norm sort, and |theta|_F^2 into nrm2.
__global__ void __launch_bounds__(256) theta_norm_kernel(TwoQGeom g) {
    const int j = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (c >= g.cslot) return;
    const cf* col = g.X + (size_t)j * g.lslot * g.cslot + (size_t)c * g.lslot;
    double acc = 0.0;
    for (int r = lane; r < g.lslot; r += 32) {
        const cf x = col[r];
        acc += (double)x.x * x.x + (double)x.y * x.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
        g.cnrm[(size_t)j * g.cslot + c] = (float)acc;
        if (acc != 0.0) atomicAdd(g.nrm2 + j, acc);
    }
}

__device__ __forceinline__ int theta_scale_exponent(double n2) {
    if (!(n2 > 0.0) || !isfinite(n2)) return 0;       // zero or NaN/Inf: leave as is
    int ex;
    frexp(sqrt(n2), &ex);                             // |theta| = f 2^ex, f in [0.5, 1)
    int e = 1 - ex;
    return e < -120 ? -120 : (e > 120 ? 120 : e);
}

__global__ void __launch_bounds__(256) theta_scale_kernel(const mps_2q_job* __restrict__ jobs,
                                                          TwoQGeom g) {
    const int j = blockIdx.y;
    const double n2 = g.nrm2[j];
    const int e = theta_scale_exponent(n2);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        g.scale[j] = e;
        // a NaN/Inf element makes |theta|^2 non-finite; the scaled Jacobi
        // arithmetic cannot create one, so this is the call's whole check
        if (!isfinite(n2)) atomicAdd(g.counter + 1, 1);
    }
    if (e == 0) return;
    const float f = ldexpf(1.f, e);
    const size_t count = (size_t)g.lslot * g.cslot;
    cf* X = g.X + (size_t)j * count;
    const mps_2q_job job = jobs[j];
    cf* T = job_tracks_v(job.chi_l * g.d, g.d * job.chi_r, job.keep_left_canonical)
                ? nullptr : g.T + (size_t)j * count;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
         t += (size_t)gridDim.x * blockDim.x) {
        X[t] = cscale(X[t], f);
        if (T) T[t] = cscale(T[t], f);
    }
}

// The singular values, the discarded weight and the site that carries S
// (the right one for keep_left_canonical, else the left) back to theta's scale.
__global__ void __launch_bounds__(256) unscale_kernel(const mps_2q_job* __restrict__ jobs,
                                                      TwoQGeom g) {
    const int j = blockIdx.y;
    const int e = g.scale[j];
    if (e == 0) return;
    const mps_2q_job job = jobs[j];
    const float f = ldexpf(1.f, -e);
    const size_t m = (size_t)job.chi_l * g.d, n = (size_t)g.d * job.chi_r;
    const size_t r = m < n ? m : n, k = (size_t)job.k;
    cf* out = reinterpret_cast<cf*>(job.keep_left_canonical ? job.b_out : job.a_out);
    const size_t count = out ? (job.keep_left_canonical ? k * n : m * k) : 0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
         t += (size_t)gridDim.x * blockDim.x)
        out[t] = cscale(out[t], f);
    if (blockIdx.x == 0) {
        if (job.svals)
            for (size_t t = threadIdx.x; t < r; t += blockDim.x) job.svals[t] *= f;
        if (job.discarded && threadIdx.x == 0) *job.discarded = ldexp(*job.discarded, -2 * e);
    }
}

int scale_theta(const mps_2q_job* jobs, int njobs, const TwoQGeom& g, cudaStream_t s) {
    MPS_CUDA_CHECK(cudaMemsetAsync(g.nrm2, 0, (size_t)njobs * sizeof(double), s));
    theta_norm_kernel<<<dim3((g.cslot + 7) / 8, njobs), 256, 0, s>>>(g);
    MPS_LAUNCH_CHECK("theta_norm_kernel");
    const size_t count = (size_t)g.lslot * g.cslot;
    const int bx = (int)((count + 256 * 32 - 1) / (256 * 32));
    dim3 grid(bx < 1 ? 1 : bx, njobs);
    theta_scale_kernel<<<grid, 256, 0, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("theta_scale_kernel");
    return MPS_OK;
}

int unscale_outputs(const mps_2q_job* jobs, int njobs, int max_m, int max_n, const TwoQGeom& g,
                    cudaStream_t s) {
    const size_t count = (size_t)max_m * max_n;
    const int bx = (int)((count + 256 * 16 - 1) / (256 * 16));
    unscale_kernel<<<dim3(bx < 1 ? 1 : bx, njobs), 256, 0, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("unscale_kernel");
    return MPS_OK;
}

// ---------------------------------------------------------------------------
// Launch helpers.

// Largest dynamic shared memory a kernel may request on the current device:
// the per-block opt-in limit minus the kernel's own static shared memory.
template <typename K>
int dynamic_smem_limit(K kernel, int* limit) {
    int dev = 0, optin = 0;
    MPS_CUDA_CHECK(cudaGetDevice(&dev));
    MPS_CUDA_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    MPS_CUDA_CHECK(cudaFuncGetAttributes(&fa, kernel));
    *limit = optin - (int)fa.sharedSizeBytes;
    return MPS_OK;
}

// Sets the kernel's dynamic shared-memory opt-in to the device's limit, once
// per device; with threads > 0 also counts the CTAs of (threads, smem) that
// fit on the whole device.
template <typename K>
int prepare_kernel(K kernel, KernelSetup& ks, int* limit, int threads = 0, size_t smem = 0,
                   int* ctas = nullptr) {
    int dev = 0;
    MPS_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(MPS_ERR_ARG, "device index beyond 63");
    std::call_once(ks.once[dev], [&] {
        ks.ctas[dev] = 0;
        int rc = dynamic_smem_limit(kernel, &ks.limit[dev]);
        if (rc == MPS_OK) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 ks.limit[dev]);
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaFuncSetAttribute(jacobi visit)");
        }
        if (rc == MPS_OK && threads > 0) {
            int sms = 0, per_sm = 0;
            cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
            if (e != cudaSuccess) rc = cuda_fail(e, "resident CTAs of the sweep kernel");
            ks.ctas[dev] = sms * (per_sm > 0 ? per_sm : 1);
        }
        ks.rc[dev] = rc;
    });
    *limit = ks.limit[dev];
    if (ctas) *ctas = ks.ctas[dev];
    return ks.rc[dev];
}

template <int BC>
size_t full_smem(int lw) {
    return (size_t)2 * BC * lw * sizeof(cf) + (size_t)4 * BC * BC * sizeof(cf) +
           (size_t)2 * BC * sizeof(float);
}

template <int BC>
size_t ring_smem(int lw) {
    return (size_t)2 * BC * lw * sizeof(cf) + (size_t)4 * BC * BC * sizeof(cf) +
           (size_t)2 * BC * sizeof(float);
}

template <int BC, int ROWS>
int launch_visit(const mps_2q_job* jobs, int njobs, int pairs, const TwoQGeom& g, int round,
                 float tol2, int lw, cudaStream_t s) {
    dim3 grid(pairs, njobs);
    if (round == 0) {
        static KernelSetup ks;
        int limit = 0;
        if (int rc = prepare_kernel(full_visit_kernel<BC, ROWS>, ks, &limit)) return rc;
        const size_t smem = full_smem<BC>(lw);
        if (smem > (size_t)limit) return fail(MPS_ERR_ARG, "jacobi: merged matrix too long for shared memory");
        full_visit_kernel<BC, ROWS><<<grid, BC * 32, smem, s>>>(jobs, g, round, tol2);
        MPS_LAUNCH_CHECK("full_visit_kernel");
    } else {
        static KernelSetup ks;
        int limit = 0;
        if (int rc = prepare_kernel(ring_visit_kernel<BC, ROWS>, ks, &limit)) return rc;
        const size_t smem = ring_smem<BC>(lw);
        if (smem > (size_t)limit) return fail(MPS_ERR_ARG, "jacobi: merged matrix too long for shared memory");
        ring_visit_kernel<BC, ROWS><<<grid, BC * 32, smem, s>>>(jobs, g, round, tol2);
        MPS_LAUNCH_CHECK("ring_visit_kernel");
    }
    return MPS_OK;
}

template <int BC, int ROWS>
int launch_sweep(const mps_2q_job* jobs, int njobs, int rounds, int pairs, const TwoQGeom& g,
                 float tol2, int lw, const SweepSync& sync, int tbase, cudaStream_t s) {
    static KernelSetup ks;
    const size_t smem = ring_smem<BC>(lw);
    int limit = 0, ctas = 0;
    if (int rc = prepare_kernel(sweep_kernel<BC, ROWS>, ks, &limit, BC * 32, smem, &ctas)) return rc;
    if (smem > (size_t)limit) return fail(MPS_ERR_ARG, "jacobi: merged matrix too long for shared memory");
    const int items = rounds * njobs * pairs;
    const int grid = items < ctas ? items : ctas;
    if (grid <= 0) return MPS_OK;
    sweep_kernel<BC, ROWS><<<grid, BC * 32, smem, s>>>(jobs, g, tol2, njobs, rounds, pairs, sync,
                                                       tbase);
    MPS_LAUNCH_CHECK("sweep_kernel");
    return MPS_OK;
}

typedef int (*sweep_fn)(const mps_2q_job*, int, int, int, const TwoQGeom&, float, int,
                        const SweepSync&, int, cudaStream_t);

sweep_fn pick_sweep(int lw, int block_request) {
    if (block_request == 8 && lw > 256 && lw <= 576)
        return lw <= 512 ? launch_sweep<8, 16> : launch_sweep<8, 18>;
    if (lw <= 576) {
        if (lw <= 64) return launch_sweep<16, 2>;
        if (lw <= 128) return launch_sweep<16, 4>;
        if (lw <= 256) return launch_sweep<16, 8>;
        if (lw <= 512) return launch_sweep<16, 16>;
        return launch_sweep<16, 18>;
    }
    if (lw <= 1024) return launch_sweep<8, 32>;
    return launch_sweep<8, 56>;
}

typedef int (*visit_fn)(const mps_2q_job*, int, int, const TwoQGeom&, int, float, int, cudaStream_t);

// Block width and register rows for a working column length lw (<= 1792).
visit_fn pick_visit(int lw, int* bc) {
    if (lw <= 576) {
        *bc = 16;
        if (lw <= 64) return launch_visit<16, 2>;
        if (lw <= 128) return launch_visit<16, 4>;
        if (lw <= 256) return launch_visit<16, 8>;
        if (lw <= 512) return launch_visit<16, 16>;
        return launch_visit<16, 18>;
    }
    *bc = 8;
    if (lw <= 1024) return launch_visit<8, 32>;
    return launch_visit<8, 56>;
}

struct Layout {
    int lslot, cslot;
    size_t off_X, off_V, off_T, off_sig, off_perm, off_cmap, off_cnrm, off_off, off_done, off_need,
        off_counter, off_scale, off_nrm2, off_sync, off_vst, off_qst, off_P, total;
    int nbmax, qstride;
};

// Column length of a slot: the ring kernel reads exactly 32*ROWS rows, so
// the slot is padded up to the ROWS step pick_visit chooses for it.
int slot_rows(int L) {
    const int steps[] = {64, 128, 256, 512, 576, 1024, 1792};
    for (int r : steps)
        if (L <= r) return r;
    return (int)align_up((size_t)L, 32);
}

Layout make_layout(int njobs, int max_m, int max_n, bool pieces = false) {
    Layout lo;
    const int L = max(max_m, max_n), C = min(max_m, max_n);
    lo.lslot = slot_rows(max(L, 1));
    lo.cslot = (int)align_up((size_t)max(C, 1), 32);
    size_t o = 0;
    const size_t nj = (size_t)max(njobs, 1);
    lo.off_X = o; o = align_up(o + nj * lo.lslot * lo.cslot * sizeof(cf), 256);
    lo.off_V = o; o = align_up(o + nj * lo.cslot * lo.cslot * sizeof(cf), 256);
    lo.off_T = o; o = align_up(o + nj * lo.lslot * lo.cslot * sizeof(cf), 256);
    lo.off_sig = o; o = align_up(o + nj * lo.cslot * sizeof(float), 256);
    lo.off_perm = o; o = align_up(o + nj * lo.cslot * sizeof(int), 256);
    lo.off_cmap = o; o = align_up(o + nj * lo.cslot * sizeof(int), 256);
    lo.off_cnrm = o; o = align_up(o + nj * lo.cslot * sizeof(float), 256);
    lo.off_off = o; o = align_up(o + nj * sizeof(float), 256);
    lo.off_done = o; o = align_up(o + nj * sizeof(int), 256);
    lo.off_need = o; o = align_up(o + nj * sizeof(int), 256);
    lo.off_counter = o; o = align_up(o + 8 * sizeof(int), 256);
    lo.off_scale = o; o = align_up(o + nj * sizeof(int), 256);
    lo.off_nrm2 = o; o = align_up(o + nj * sizeof(double), 256);
    // sweep sync: next_item, error, then block_round[njobs][nbmax] (nbmax
    // for the smallest block width, 8 columns)
    lo.nbmax = (int)align_up((size_t)(lo.cslot + 7) / 8, 2);
    lo.off_sync = o; o = align_up(o + (2 + nj * lo.nbmax) * sizeof(int), 256);
    // visit skipping: a stamp per column block and per (round, pair)
    lo.qstride = lo.nbmax * (lo.nbmax / 2);
    lo.off_vst = o; o = align_up(o + nj * lo.nbmax * sizeof(int), 256);
    lo.off_qst = o; o = align_up(o + nj * lo.qstride * sizeof(int), 256);
    // the mixed form's bf16 piece planes of X (3 per job)
    lo.off_P = o;
    if (pieces) o = align_up(o + nj * 3 * 2 * (size_t)lo.lslot * lo.cslot * sizeof(uint16_t), 256);
    lo.total = o;
    return lo;
}

thread_local int* t_pinned = nullptr;

}  // namespace

}  // namespace mps

using namespace mps;

extern "C" size_t mps_2q_workspace_bytes(int njobs, int max_m, int max_n, int d) {
    (void)d;
    if (njobs <= 0 || max_m <= 0 || max_n <= 0) return 0;
    return make_layout(njobs, max_m, max_n).total;
}

extern "C" size_t mps_2q_workspace_bytes_mixed(int njobs, int max_m, int max_n, int d) {
    (void)d;
    if (njobs <= 0 || max_m <= 0 || max_n <= 0) return 0;
    return make_layout(njobs, max_m, max_n, true).total;
}

extern "C" int mps_apply_2q_batch(void* stream, const mps_2q_job* jobs, int njobs,
                                  int max_m, int max_n, int d, void* workspace,
                                  size_t workspace_bytes, mps_svd_params* params) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (njobs == 0) return MPS_OK;
    // Under stream capture (a CUDA graph) the call may not read anything back:
    // it queues max_sweeps sweeps, in which converged jobs return at once, and
    // leaves non-convergence, NaN/Inf and expired waits to the per-job status
    // words (MPS_STATUS_*) for the caller to read after the replay.
    cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
    MPS_CUDA_CHECK(cudaStreamIsCapturing(s, &cst));
    const bool capturing = cst != cudaStreamCaptureStatusNone;
    if (njobs < 0 || njobs > 65535 || !jobs) return fail(MPS_ERR_ARG, "mps_apply_2q_batch: bad job list");
    if (d < 1 || d > 64) return fail(MPS_ERR_ARG, "mps_apply_2q_batch: qudit dimension must be 1..64");
    if (max_m <= 0 || max_n <= 0)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch: max_m/max_n must be positive");
    const bool mixed_req = params && params->precision == MPS_PRECISION_MIXED;
    const Layout lo = make_layout(njobs, max_m, max_n, mixed_req);
    if (lo.lslot > 1792)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch: merged matrix longer than 1792 rows "
                                 "is beyond this build's shared-memory Jacobi kernel");
    if (!workspace || workspace_bytes < lo.total)
        return fail(MPS_ERR_WORKSPACE, "mps_apply_2q_batch: workspace too small");
    if ((reinterpret_cast<uintptr_t>(workspace) & 255) != 0)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch: workspace must be 256-byte aligned");

    char* ws = static_cast<char*>(workspace);
    TwoQGeom g;
    g.d = d;
    g.lslot = lo.lslot;
    g.cslot = lo.cslot;
    g.X = reinterpret_cast<cf*>(ws + lo.off_X);
    g.V = reinterpret_cast<cf*>(ws + lo.off_V);
    g.T = reinterpret_cast<cf*>(ws + lo.off_T);
    g.sig = reinterpret_cast<float*>(ws + lo.off_sig);
    g.perm = reinterpret_cast<int*>(ws + lo.off_perm);
    g.offmax = reinterpret_cast<float*>(ws + lo.off_off);
    g.done = reinterpret_cast<int*>(ws + lo.off_done);
    g.need = reinterpret_cast<int*>(ws + lo.off_need);
    g.counter = reinterpret_cast<int*>(ws + lo.off_counter);
    g.cmap = reinterpret_cast<int*>(ws + lo.off_cmap);
    g.cnrm = reinterpret_cast<float*>(ws + lo.off_cnrm);
    g.scale = reinterpret_cast<int*>(ws + lo.off_scale);
    g.nrm2 = reinterpret_cast<double*>(ws + lo.off_nrm2);
    g.vstamp = reinterpret_cast<int*>(ws + lo.off_vst);
    g.qstamp = reinterpret_cast<int*>(ws + lo.off_qst);
    g.nbmax = lo.nbmax;
    g.qstride = lo.qstride;
    g.P = mixed_req ? reinterpret_cast<uint16_t*>(ws + lo.off_P) : nullptr;
    g.pplane = (size_t)2 * lo.lslot * lo.cslot;

    int max_sweeps = 40;
    float tol = 0.f;
    if (params) {
        if (params->max_sweeps > 0) max_sweeps = params->max_sweeps;
        tol = params->tol;
    }
    // The computed x_p^H x_q carries a rounding error of a few 2^-24
    // sum_r |x_r||q_r|, growing slowly with the length L; the default
    // threshold 2^-24 max(8, sqrt(L)) stays above that noise (no sweep keeps
    // rotating noise) while the kept subspace -- whose error is about
    // tol s_k / gap at the truncation cut -- stays close to what a
    // backward-stable complex64 SVD gives.
    if (!(tol > 0.f)) tol = 5.9604645e-8f * fmaxf(8.f, sqrtf((float)lo.lslot));
    const float tol2 = tol * tol;     // the kernels compare squared cosines
    const bool mixed = params && params->precision == MPS_PRECISION_MIXED;
    if (params && params->precision != MPS_PRECISION_PLAIN && !mixed)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch: unknown precision");
    const int lw = lo.lslot;
    int bc = 16;
    (void)pick_visit(lw, &bc);
    const int block_request = params ? params->block_request : 0;
    if (block_request != 0 && block_request != 8 && block_request != 16)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch: block_request must be 0, 8 or 16");
    sweep_fn sweep = pick_sweep(lw, block_request);
    if (block_request == 8 && lw > 256 && lw <= 576) bc = 8;
    // MPS_PRECISION_MIXED: the left-canonical tall jobs of 64+ columns take
    // the tensor-core sweeps (32-column blocks), the others the SIMT ones, in
    // the same sweep loop
    g.tc_mode = mixed ? 1 : 0;
    constexpr int kTcBlock = 32;
    if (params) params->block_cols = mixed ? kTcBlock : bc;
    SweepSync sync;
    sync.next_item = reinterpret_cast<int*>(ws + lo.off_sync);
    sync.error = sync.next_item + 1;
    sync.block_round = sync.next_item + 2;
    sync.nbmax = lo.nbmax;
    sync.wait_limit = (params && params->wait_limit > 0) ? params->wait_limit : (1 << 22);
    sync.stall_test = params ? params->stall_test : 0;
    // padding rows and columns of X must be zero; no block has a stamp yet
    MPS_CUDA_CHECK(cudaMemsetAsync(g.X, 0, lo.off_V - lo.off_X, s));
    MPS_CUDA_CHECK(cudaMemsetAsync(g.vstamp, 0xff, lo.off_qst - lo.off_vst +
                                                       (size_t)njobs * lo.qstride * sizeof(int), s));
    {
        const size_t total = (size_t)njobs * lo.cslot * lo.cslot;
        int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
        blocks = max(blocks, (njobs + 255) / 256);
        init_slots_kernel<<<blocks, 256, 0, s>>>(jobs, g, njobs);
        MPS_LAUNCH_CHECK("init_slots_kernel");
        if (mixed) {
            count_simt_jobs_kernel<<<(njobs + 255) / 256, 256, 0, s>>>(jobs, d, njobs, g.counter);
            MPS_LAUNCH_CHECK("count_simt_jobs_kernel");
        }
    }
    const int max_chil = (max_m + d - 1) / d, max_chir = (max_n + d - 1) / d;
    int rc = merge_gate_launch(jobs, njobs, max_chil, max_chir, g, s);
    if (rc) return rc;
    if (mixed) {
        rc = merge_tc_launch(jobs, njobs, max_m, max_n, g, s);
        if (rc) return rc;
    }
    rc = scale_theta(jobs, njobs, g, s);
    if (rc) return rc;
    if (!(params && params->lq_off)) rc = lq_precondition(jobs, njobs, max_m, max_n, g, s);
    if (rc) return rc;

    const int cmax = min(max_m, max_n);
    auto block_count = [&](int width) {
        int nb = (cmax + width - 1) / width;
        if (nb < 2) nb = 2;
        return nb + (nb & 1);
    };
    const int nbmax = block_count(bc);
    const int rounds = nbmax - 1, pairs = nbmax / 2;
    const int nb_tc = block_count(kTcBlock);
    const int rounds_tc = nb_tc - 1, pairs_tc = nb_tc / 2;
    // stamps of every sweep lie above those of the sweeps before it
    const int tbase_stride = rounds + 1;

    if (!t_pinned && !capturing) {
        MPS_CUDA_CHECK(cudaHostAlloc(reinterpret_cast<void**>(&t_pinned), 8 * sizeof(int),
                                     cudaHostAllocDefault));
    }
    int npow2 = 1;
    while (npow2 < lo.cslot) npow2 <<= 1;
    const size_t sort_smem = (size_t)npow2 * (sizeof(float) + sizeof(int));
    int sweeps = 0;
    bool converged = false;
    if (cmax >= 2) {
        // mixed calls: whether the last sweep left jobs for each sweep kernel
        // (unknown, so both run, before the first read and under capture)
        bool tc_left = true, simt_left = true;
        for (sweeps = 1; sweeps <= max_sweeps; ++sweeps) {
            MPS_CUDA_CHECK(cudaMemsetAsync(g.counter, 0, sizeof(int), s));
            if (mixed) MPS_CUDA_CHECK(cudaMemsetAsync(g.counter + 4, 0, 2 * sizeof(int), s));
            if (cmax > 2 * bc) {
                presort_kernel<<<njobs, PRESORT_T, sort_smem, s>>>(jobs, g, npow2, bc,
                                                                   sweeps * tbase_stride);
                MPS_LAUNCH_CHECK("presort_kernel");
            }
            MPS_CUDA_CHECK(cudaMemsetAsync(sync.block_round, 0xff,
                                           (size_t)njobs * lo.nbmax * sizeof(int), s));
            if (mixed) {
                // the tensor-core jobs: one persistent launch per sweep with
                // the same round flags and visit stamps as the SIMT form (its
                // own item counter, counter[2]); X is split into its bf16
                // pieces before the first sweep.  An expired wait stays in
                // sync.error until the call returns.
                if (sweeps == 1) {
                    MPS_CUDA_CHECK(cudaMemsetAsync(sync.error, 0, sizeof(int), s));
                    if (int e = tc_split_launch(jobs, njobs, g, s)) return e;
                }
                if (tc_left) {
                    SweepSync tsync = sync;
                    tsync.next_item = g.counter + 2;
                    MPS_CUDA_CHECK(cudaMemsetAsync(tsync.next_item, 0, sizeof(int), s));
                    rc = tc_sweep_launch(jobs, njobs, rounds_tc, pairs_tc, g, tol2, tsync,
                                         sweeps * tbase_stride, s);
                    if (rc) return rc;
                }
                MPS_CUDA_CHECK(cudaMemsetAsync(sync.next_item, 0, sizeof(int), s));
            } else {
                MPS_CUDA_CHECK(cudaMemsetAsync(sync.next_item, 0, 2 * sizeof(int), s));
            }
            // the SIMT jobs (all of them in the plain form): one persistent
            // launch runs every round of the sweep
            if (simt_left) {
                rc = sweep(jobs, njobs, rounds, pairs, g, tol2, lw, sync, sweeps * tbase_stride, s);
                if (rc) return rc;
            }
            sweep_end_kernel<<<(njobs + 255) / 256, 256, 0, s>>>(jobs, g, njobs, tol2, sync.error);
            MPS_LAUNCH_CHECK("sweep_end_kernel");
            if (capturing) {
                converged = true;            // reported through the status words
                continue;
            }
            // counter[0..5] (jobs left, NaN count, -, expired MMA wait, jobs
            // left per kind) and the round-flag error word
            MPS_CUDA_CHECK(cudaMemcpyAsync(t_pinned, g.counter, 6 * sizeof(int),
                                           cudaMemcpyDeviceToHost, s));
            MPS_CUDA_CHECK(cudaMemcpyAsync(t_pinned + 6, sync.error, sizeof(int),
                                           cudaMemcpyDeviceToHost, s));
            MPS_CUDA_CHECK(cudaStreamSynchronize(s));
            if (t_pinned[6] != 0)
                return fail(MPS_ERR_TIMEOUT, "mps_apply_2q_batch: a round-dependency wait inside the "
                                             "sweep kernel expired; results are invalid");
            if (mixed && t_pinned[3] != 0)
                return fail(MPS_ERR_TIMEOUT, "mps_apply_2q_batch: a tensor-core MMA wait "
                                             "expired; results are invalid");
            if (mixed) {
                tc_left = t_pinned[4] != 0;
                simt_left = t_pinned[5] != 0;
            }
            if (t_pinned[0] == 0) {
                converged = true;
                break;
            }
        }
        if (sweeps > max_sweeps) sweeps = max_sweeps;
        if (mixed) {
            // the tensor-core sweeps kept their jobs' columns in the piece planes
            rc = tc_merge_launch(jobs, njobs, g, s);
            if (rc) return rc;
        }
    } else {
        converged = true;
        // single-column (or empty) jobs: nothing to rotate
        MPS_CUDA_CHECK(cudaMemsetAsync(g.done, 0xff, (size_t)njobs * sizeof(int), s));
    }
    if (params) params->sweeps_out = sweeps;

    if (sort_smem > 48 * 1024) {
        MPS_CUDA_CHECK(cudaFuncSetAttribute(sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)sort_smem));
    }
    sort_kernel<<<njobs, SORT_T, sort_smem, s>>>(jobs, g, npow2);
    MPS_LAUNCH_CHECK("sort_kernel");
    {
        const int kmax = cmax;
        dim3 ga((kmax + 31) / 32, (max_m + 31) / 32, njobs);
        regauge_a_kernel<<<ga, dim3(32, 8), 0, s>>>(jobs, g);
        MPS_LAUNCH_CHECK("regauge_a_kernel");
        dim3 gb((max_n + 255) / 256, kmax, njobs);
        regauge_b_kernel<<<gb, 256, 0, s>>>(jobs, g);
        MPS_LAUNCH_CHECK("regauge_b_kernel");
        const size_t comp_smem = (size_t)(max(max_m, max_n) + kmax) * sizeof(cf);
        if (comp_smem > 48 * 1024) {
            MPS_CUDA_CHECK(cudaFuncSetAttribute(complete_kernel,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)comp_smem));
        }
        complete_kernel<<<njobs, COMP_T, comp_smem, s>>>(jobs, g);
        MPS_LAUNCH_CHECK("complete_kernel");
        rc = launch_post(jobs, njobs, max_m, max_n, kmax, g, s);
        if (rc) return rc;
        rc = unscale_outputs(jobs, njobs, max_m, max_n, g, s);
        if (rc) return rc;
    }
    // The non-finite count is complete before the first sweep (see
    // theta_scale_kernel) and came back with every convergence read, so the
    // call returns without waiting for its last kernels and the host can
    // prepare the next call meanwhile.  Jobs of one column have no sweep: read
    // the count here.
    if (capturing) return MPS_OK;
    if (cmax < 2) {
        MPS_CUDA_CHECK(cudaMemcpyAsync(t_pinned + 1, g.counter + 1, sizeof(int),
                                       cudaMemcpyDeviceToHost, s));
        MPS_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    if (t_pinned[1] != 0) return fail(MPS_ERR_NONFINITE, "mps_apply_2q_batch: NaN/Inf singular value");
    if (!converged)
        return fail(MPS_ERR_NOT_CONVERGED, "mps_apply_2q_batch: Jacobi SVD hit its sweep cap");
    return MPS_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of mps_apply_2q_batch.
//
// Some callers cannot allocate device memory: an application whose memory
// pool owns the whole GPU and forbids allocations outside it, a plugin host
// that hands its plugins no allocator, or a latency-critical loop that must
// never enter the allocator.  This entry point takes its scratch from the
// fixed array below instead of from a caller-provided workspace, and makes
// no allocation of its own (no cudaMalloc/cudaFree, no pinned host buffer:
// the per-sweep convergence count is read into a stack variable).
//
// The array is a static __device__ object: every GPU that loads this library
// holds MPS_NOALLOC_SCRATCH_BYTES of it until the process exits.  In host code
// its name is only a host-side stand-in, never a device address; the device
// address is looked up with cudaGetSymbolAddress once per device, with that
// device current, on the first call made on that device -- so make that first
// call before any stream capture.  All calls share the one array and it keeps
// the previous call's contents: the driver clears everything that must start
// at zero, and calls that overlap on the GPU (two streams, two threads) race
// on it and must be serialised by the caller.
static __device__ __align__(256) unsigned char g_noalloc_scratch[MPS_NOALLOC_SCRATCH_BYTES];

namespace mps {
namespace {

std::once_flag g_noalloc_once[kMaxDevices];
void* g_noalloc_ptr[kMaxDevices];
cudaError_t g_noalloc_err[kMaxDevices];

int noalloc_scratch(void** ptr) {
    int dev = 0;
    MPS_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(MPS_ERR_ARG, "mps_apply_2q_batch_noalloc: device index out of range");
    std::call_once(g_noalloc_once[dev], [dev] {
        g_noalloc_err[dev] = cudaGetSymbolAddress(&g_noalloc_ptr[dev], g_noalloc_scratch);
    });
    if (g_noalloc_err[dev] != cudaSuccess)
        return cuda_fail(g_noalloc_err[dev], "cudaGetSymbolAddress(g_noalloc_scratch)");
    *ptr = g_noalloc_ptr[dev];
    return MPS_OK;
}

}  // namespace
}  // namespace mps

extern "C" int mps_apply_2q_batch_noalloc(void* stream, const mps_2q_job* jobs, int njobs,
                                          int max_m, int max_n, int d,
                                          mps_svd_params* params) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (njobs == 0) return MPS_OK;
    if (njobs < 0 || njobs > 65535 || !jobs)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch_noalloc: bad job list");
    if (d < 1 || d > 64) return fail(MPS_ERR_ARG, "mps_apply_2q_batch_noalloc: qudit dimension must be 1..64");
    if (max_m <= 0 || max_n <= 0)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch_noalloc: max_m/max_n must be positive");
    const Layout lo = make_layout(njobs, max_m, max_n, false);
    if (lo.lslot > 1792)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch_noalloc: merged matrix longer than 1792 rows "
                                 "is beyond this build's shared-memory Jacobi kernel");
    if (lo.total > (size_t)MPS_NOALLOC_SCRATCH_BYTES)
        return fail(MPS_ERR_WORKSPACE,
                    "mps_apply_2q_batch_noalloc: these jobs need " + std::to_string(lo.total) +
                        " bytes of scratch, more than the fixed " +
                        std::to_string((size_t)MPS_NOALLOC_SCRATCH_BYTES) +
                        "; use mps_apply_2q_batch with a workspace, or fewer/smaller jobs per call");
    void* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;

    char* ws = static_cast<char*>(scratch);
    TwoQGeom g;
    g.d = d;
    g.lslot = lo.lslot;
    g.cslot = lo.cslot;
    g.X = reinterpret_cast<cf*>(ws + lo.off_X);
    g.V = reinterpret_cast<cf*>(ws + lo.off_V);
    g.T = reinterpret_cast<cf*>(ws + lo.off_T);
    g.sig = reinterpret_cast<float*>(ws + lo.off_sig);
    g.perm = reinterpret_cast<int*>(ws + lo.off_perm);
    g.offmax = reinterpret_cast<float*>(ws + lo.off_off);
    g.done = reinterpret_cast<int*>(ws + lo.off_done);
    g.need = reinterpret_cast<int*>(ws + lo.off_need);
    g.counter = reinterpret_cast<int*>(ws + lo.off_counter);
    g.cmap = reinterpret_cast<int*>(ws + lo.off_cmap);
    g.cnrm = reinterpret_cast<float*>(ws + lo.off_cnrm);
    g.scale = reinterpret_cast<int*>(ws + lo.off_scale);
    g.nrm2 = reinterpret_cast<double*>(ws + lo.off_nrm2);
    // the per-round visit kernels of this entry point do not skip visits
    g.vstamp = nullptr;
    g.qstamp = nullptr;
    g.nbmax = lo.nbmax;
    g.qstride = lo.qstride;
    g.P = nullptr;
    g.pplane = 0;
    g.tc_mode = 0;

    int max_sweeps = 40;
    float tol = 0.f;
    if (params) {
        if (params->max_sweeps > 0) max_sweeps = params->max_sweeps;
        tol = params->tol;
    }
    if (!(tol > 0.f)) tol = 5.9604645e-8f * fmaxf(8.f, sqrtf((float)lo.lslot));
    const float tol2 = tol * tol;     // the kernels compare squared cosines
    const int lw = lo.lslot;
    int bc = 16;
    visit_fn visit = pick_visit(lw, &bc);
    if (params) params->block_cols = bc;

    // the array keeps the last call's contents: clear X (padding must be
    // zero), set V to I, the column maps to identity and reset the per-job
    // flags and counters
    MPS_CUDA_CHECK(cudaMemsetAsync(g.X, 0, lo.off_V - lo.off_X, s));
    {
        const size_t total = (size_t)njobs * lo.cslot * lo.cslot;
        int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
        blocks = max(blocks, (njobs + 255) / 256);
        init_slots_kernel<<<blocks, 256, 0, s>>>(jobs, g, njobs);
        MPS_LAUNCH_CHECK("init_slots_kernel");
    }
    const int max_chil = (max_m + d - 1) / d, max_chir = (max_n + d - 1) / d;
    rc = merge_gate_launch(jobs, njobs, max_chil, max_chir, g, s);
    if (rc) return rc;
    rc = scale_theta(jobs, njobs, g, s);
    if (rc) return rc;
    rc = lq_precondition(jobs, njobs, max_m, max_n, g, s);
    if (rc) return rc;

    const int cmax = min(max_m, max_n);
    int nbmax = (cmax + bc - 1) / bc;
    if (nbmax < 2) nbmax = 2;
    nbmax += nbmax & 1;
    const int rounds = nbmax - 1, pairs = nbmax / 2;
    int npow2 = 1;
    while (npow2 < lo.cslot) npow2 <<= 1;
    const size_t sort_smem = (size_t)npow2 * (sizeof(float) + sizeof(int));
    int host_counter[2] = {0, 0};   // pageable stack memory: no pinned buffer
    int sweeps = 0;
    bool converged = false;
    if (cmax >= 2) {
        for (sweeps = 1; sweeps <= max_sweeps; ++sweeps) {
            MPS_CUDA_CHECK(cudaMemsetAsync(g.counter, 0, sizeof(int), s));
            if (cmax > 2 * bc) {
                presort_kernel<<<njobs, PRESORT_T, sort_smem, s>>>(jobs, g, npow2, bc, 0);
                MPS_LAUNCH_CHECK("presort_kernel");
            }
            for (int r = 0; r < rounds; ++r) {
                rc = visit(jobs, njobs, pairs, g, r, tol2, lw, s);
                if (rc) return rc;
            }
            sweep_end_kernel<<<(njobs + 255) / 256, 256, 0, s>>>(jobs, g, njobs, tol2, nullptr);
            MPS_LAUNCH_CHECK("sweep_end_kernel");
            MPS_CUDA_CHECK(cudaMemcpyAsync(host_counter, g.counter, sizeof(int),
                                           cudaMemcpyDeviceToHost, s));
            MPS_CUDA_CHECK(cudaStreamSynchronize(s));
            if (host_counter[0] == 0) {
                converged = true;
                break;
            }
        }
        if (sweeps > max_sweeps) sweeps = max_sweeps;
    } else {
        converged = true;
        MPS_CUDA_CHECK(cudaMemsetAsync(g.done, 0xff, (size_t)njobs * sizeof(int), s));
    }
    if (params) params->sweeps_out = sweeps;

    if (sort_smem > 48 * 1024) {
        MPS_CUDA_CHECK(cudaFuncSetAttribute(sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)sort_smem));
    }
    sort_kernel<<<njobs, SORT_T, sort_smem, s>>>(jobs, g, npow2);
    MPS_LAUNCH_CHECK("sort_kernel");
    {
        const int kmax = cmax;
        dim3 ga((kmax + 31) / 32, (max_m + 31) / 32, njobs);
        regauge_a_kernel<<<ga, dim3(32, 8), 0, s>>>(jobs, g);
        MPS_LAUNCH_CHECK("regauge_a_kernel");
        dim3 gb((max_n + 255) / 256, kmax, njobs);
        regauge_b_kernel<<<gb, 256, 0, s>>>(jobs, g);
        MPS_LAUNCH_CHECK("regauge_b_kernel");
        const size_t comp_smem = (size_t)(max(max_m, max_n) + kmax) * sizeof(cf);
        if (comp_smem > 48 * 1024) {
            MPS_CUDA_CHECK(cudaFuncSetAttribute(complete_kernel,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)comp_smem));
        }
        complete_kernel<<<njobs, COMP_T, comp_smem, s>>>(jobs, g);
        MPS_LAUNCH_CHECK("complete_kernel");
        rc = launch_post(jobs, njobs, max_m, max_n, kmax, g, s);
        if (rc) return rc;
        rc = unscale_outputs(jobs, njobs, max_m, max_n, g, s);
        if (rc) return rc;
    }
    MPS_CUDA_CHECK(cudaMemcpyAsync(host_counter + 1, g.counter + 1, sizeof(int),
                                   cudaMemcpyDeviceToHost, s));
    MPS_CUDA_CHECK(cudaStreamSynchronize(s));
    if (host_counter[1] != 0)
        return fail(MPS_ERR_NONFINITE, "mps_apply_2q_batch_noalloc: NaN/Inf singular value");
    if (!converged)
        return fail(MPS_ERR_NOT_CONVERGED, "mps_apply_2q_batch_noalloc: Jacobi SVD hit its sweep cap");
    return MPS_OK;
}
