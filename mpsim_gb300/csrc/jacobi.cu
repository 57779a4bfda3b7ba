// Truncated SVD of the merged two-site matrix by block one-sided (Hestenes)
// Jacobi, with an in-kernel descending sort, truncation to k values and the
// regauge that places the singular values left or right.
//
// Replaces TensorNetwork's split_node_full_svd(..., max_singular_values=k)
// (mpsim/core.py:1132-1137; LAPACK gesdd underneath) and the contraction of
// S into one side (core.py:1139-1145).
//
// Algorithm.  The C columns of X are split into nb blocks of BC columns
// (zero-padded).  One sweep visits every pair of blocks once, in nb-1 rounds
// of nb/2 disjoint block pairs (circle-method round robin); each round is one
// launch with one CTA per (block pair, job).  A CTA copies its 2*BC columns
// to shared memory and runs one inner sweep of Hestenes rotations over all
// pairs of those columns (2*BC-1 steps of BC disjoint pairs, one warp per
// pair), accumulating the 2BC x 2BC rotation Q; it writes the columns back and
// applies V <- V Q.  For a pair (p, q) with gamma = x_p^H x_q,
// alpha = |x_p|^2, beta = |x_q|^2, the rotation zeroes gamma:
//   zeta = (beta - alpha) / (2|gamma|), t = sign(zeta)/(|zeta| + sqrt(1+zeta^2)),
//   c = 1/sqrt(1+t^2), s = c t, e = conj(gamma)/|gamma|,
//   x_p <- c x_p - s e x_q,  x_q <- s x_p + c e x_q.
// A pair is rotated only when |gamma| > tol sqrt(alpha beta); a sweep with no
// rotation in a job marks the job converged.  Column norms are recomputed
// from the rotated data (not updated by formula), so they do not drift.
//
// Afterwards sigma_c = |X_c|, sorted descending (ties by column index);
// the first k are kept.  U and V factors are read from X/sigma or V as the
// tall/wide orientation requires (see twoq.cuh); where the isometric factor
// would divide by an exact-zero singular value, an orthonormal completion
// (classical Gram-Schmidt, twice) is written instead -- LAPACK also returns
// orthonormal singular vectors for zero singular values, and which ones it
// returns does not change any later singular value of the state.
#include <mutex>
#include <vector>

#include "twoq.cuh"

namespace mps {

namespace {

constexpr int kMaxSmem = 227 * 1024;

// ---------------------------------------------------------------------------
// One round: CTA (pair index, job).  ROWS = rows per lane kept in registers
// (the working column length Lw <= 32*ROWS).
template <int BC, int ROWS>
__global__ void __launch_bounds__(BC * 32)
jacobi_round_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int round, float tol) {
    extern __shared__ float2 smem[];
    const int j = blockIdx.y;
    if (g.done[j]) return;
    const int chil = jobs[j].chi_l, chir = jobs[j].chi_r;
    const int m = chil * g.d, n = chir * g.d;
    const int L = max(m, n), C = min(m, n);
    if (C < 2) return;
    int nb = (C + BC - 1) / BC;
    if (nb < 2) nb = 2;
    nb += nb & 1;
    if (round >= nb - 1 || (int)blockIdx.x >= nb / 2) return;
    int I, J;
    tournament_pair(nb, round, blockIdx.x, I, J);
    const int Lw = (L + 31) & ~31;
    constexpr int W = 2 * BC;                   // columns in shared memory
    cf* X = g.X + (size_t)j * g.lslot * g.cslot;
    cf* Xs = smem;                              // [W][Lw]
    cf* Qs = smem + (size_t)W * Lw;             // [W][W], column-major
    float* nrm = reinterpret_cast<float*>(Qs + W * W);   // [W]
    __shared__ float s_off[BC];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = warp; c < W; c += BC) {
        const int gc = (c < BC) ? I * BC + c : J * BC + (c - BC);
        const cf* src = X + (size_t)gc * g.lslot;
        for (int r = lane; r < Lw; r += 32) Xs[(size_t)c * Lw + r] = src[r];
    }
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
    for (int step = 0; step < W - 1; ++step) {
        int p, q;
        tournament_pair(W, step, warp, p, q);
        cf* cp = Xs + (size_t)p * Lw;
        cf* cq = Xs + (size_t)q * Lw;
        cf xp[ROWS], xq[ROWS];
        cf gam = cmake(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < ROWS; ++i) {
            const int r = lane + 32 * i;
            if (r < Lw) {
                xp[i] = cp[r];
                xq[i] = cq[r];
            } else {
                xp[i] = cmake(0.f, 0.f);
                xq[i] = cmake(0.f, 0.f);
            }
            cfma_conj(gam, xp[i], xq[i]);
        }
        gam.x = warp_sum(gam.x);
        gam.y = warp_sum(gam.y);
        const float a = nrm[p], b = nrm[q];
        const float ag = sqrtf(cabs2(gam));
        const float den = sqrtf(a) * sqrtf(b);
        const float rel = den > 0.f ? ag / den : 0.f;
        offmax = fmaxf(offmax, rel);
        if (rel > tol) {                        // warp-uniform (butterfly sums)
            const float zeta = (b - a) / (2.f * ag);
            const float az = fabsf(zeta);
            float t = az > 1e10f ? 0.5f / zeta
                                 : copysignf(1.f, zeta) / (az + sqrtf(fmaf(zeta, zeta, 1.f)));
            const float c = rsqrtf(fmaf(t, t, 1.f));
            const float s = c * t;
            const cf e = cmake(gam.x / ag, -gam.y / ag);
            float na = 0.f, nq = 0.f;
#pragma unroll
            for (int i = 0; i < ROWS; ++i) {
                const int r = lane + 32 * i;
                const cf y = cmul(e, xq[i]);
                const cf np = csub(cscale(xp[i], c), cscale(y, s));
                const cf nn = cadd(cscale(xp[i], s), cscale(y, c));
                if (r < Lw) {
                    cp[r] = np;
                    cq[r] = nn;
                }
                na += cabs2(np);
                nq += cabs2(nn);
            }
            na = warp_sum(na);
            nq = warp_sum(nq);
            if (lane < W) {
                cf* qp = Qs + p * W;
                cf* qq = Qs + q * W;
                const cf a0 = qp[lane];
                const cf y = cmul(e, qq[lane]);
                qp[lane] = csub(cscale(a0, c), cscale(y, s));
                qq[lane] = cadd(cscale(a0, s), cscale(y, c));
            }
            __syncwarp();
            if (lane == 0) {
                nrm[p] = na;
                nrm[q] = nq;
            }
        }
        __syncthreads();
    }

    // write the rotated columns back
    for (int c = warp; c < W; c += BC) {
        const int gc = (c < BC) ? I * BC + c : J * BC + (c - BC);
        cf* dst = X + (size_t)gc * g.lslot;
        for (int r = lane; r < Lw; r += 32) dst[r] = Xs[(size_t)c * Lw + r];
    }
    // V <- V Q on the 2*BC columns (rows < C; the rest stay as they are)
    cf* V = g.V + (size_t)j * g.cslot * g.cslot;
    for (int r = tid; r < C; r += BC * 32) {
        cf v[W];
#pragma unroll
        for (int c = 0; c < W; ++c) {
            const int gc = (c < BC) ? I * BC + c : J * BC + (c - BC);
            v[c] = V[(size_t)gc * g.cslot + r];
        }
#pragma unroll 4
        for (int c2 = 0; c2 < W; ++c2) {
            cf acc = cmake(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < W; ++c) cfma(acc, v[c], Qs[c2 * W + c]);
            const int gc = (c2 < BC) ? I * BC + c2 : J * BC + (c2 - BC);
            V[(size_t)gc * g.cslot + r] = acc;
        }
    }
    offmax = warp_max(offmax);
    if (lane == 0) s_off[warp] = offmax;
    __syncthreads();
    if (tid == 0) {
        float o = 0.f;
        for (int w = 0; w < BC; ++w) o = fmaxf(o, s_off[w]);
        atomicMax(reinterpret_cast<int*>(g.offmax + j), __float_as_int(o));
    }
}

__global__ void sweep_end_kernel(TwoQGeom g, int njobs, float tol) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    if (!g.done[j]) {
        const float o = g.offmax[j];
        if (o > tol) atomicAdd(g.counter, 1);
        else g.done[j] = 1;
    }
    g.offmax[j] = 0.f;
}

__global__ void init_slots_kernel(TwoQGeom g, int njobs) {
    // V = identity, bookkeeping cleared
    const size_t per = (size_t)g.cslot * g.cslot;
    const size_t total = per * njobs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t w = e % per;
        const int r = (int)(w % g.cslot), c = (int)(w / g.cslot);
        g.V[e] = (r == c) ? cmake(1.f, 0.f) : cmake(0.f, 0.f);
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < njobs) {
        g.done[t] = 0;
        g.offmax[t] = 0.f;
        g.need[t] = 0;
    }
    if (t < 4) g.counter[t] = 0;
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
        if (s_bad) {
            st |= MPS_STATUS_NONFINITE;
            atomicAdd(g.counter + 1, 1);
        }
        if (job.status) *job.status = st;
    }
}

// out (R x k, row-major): out[row*k + i] = scale_i * src[perm_i * ld + row]
// out (k x R, row-major): out[i*R + col] = scale_i * conj?(src[perm_i*ld + col])
// which = 0 -> a_out, which = 1 -> b_out.
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

__global__ void regauge_b_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g) {
    const int j = blockIdx.z;
    const mps_2q_job job = jobs[j];
    const int m = job.chi_l * g.d, n = job.chi_r * g.d;
    const int i = blockIdx.y;
    if (i >= job.k) return;
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
    if (tall) sc = lc ? s : 1.f;
    else sc = lc ? 1.f : (s > thr ? 1.f / s : 0.f);
    const cf* col = src + (size_t)g.perm[(size_t)j * g.cslot + i] * ld;
    cf* out = reinterpret_cast<cf*>(job.b_out) + (size_t)i * n;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        out[c] = cscale(cconj(col[c]), sc);
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
                // h_t = u_t^H v for t < i
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
                    for (int t = 0; t < i; ++t) {
                        const cf u = base[t * vs + e * es];
                        acc = csub(acc, cmul(h[t], u));
                    }
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

template <int BC, int ROWS>
int launch_round(const mps_2q_job* jobs, int njobs, int pairs, const TwoQGeom& g,
                 int round, float tol, int lw, cudaStream_t s) {
    const size_t smem = (size_t)2 * BC * lw * sizeof(cf) + (size_t)4 * BC * BC * sizeof(cf) +
                        (size_t)2 * BC * sizeof(float);
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(jacobi_round_kernel<BC, ROWS>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    });
    if (attr_err != cudaSuccess) return cuda_fail(attr_err, "cudaFuncSetAttribute(jacobi_round)");
    dim3 grid(pairs, njobs);
    jacobi_round_kernel<BC, ROWS><<<grid, BC * 32, smem, s>>>(jobs, g, round, tol);
    MPS_LAUNCH_CHECK("jacobi_round_kernel");
    return MPS_OK;
}

typedef int (*round_fn)(const mps_2q_job*, int, int, const TwoQGeom&, int, float, int, cudaStream_t);

template <int BC>
round_fn pick_rows(int lw) {
    if (lw <= 64) return launch_round<BC, 2>;
    if (lw <= 128) return launch_round<BC, 4>;
    if (lw <= 256) return launch_round<BC, 8>;
    if (lw <= 512) return launch_round<BC, 16>;
    if (lw <= 576) return launch_round<BC, 18>;
    if (lw <= 1024) return launch_round<BC, 32>;
    return launch_round<BC, 56>;
}

struct Layout {
    int lslot, cslot;
    size_t off_X, off_V, off_sig, off_perm, off_off, off_done, off_need, off_counter, total;
};

Layout make_layout(int njobs, int max_m, int max_n) {
    Layout lo;
    const int L = max(max_m, max_n), C = min(max_m, max_n);
    lo.lslot = (int)align_up((size_t)max(L, 1), 32);
    lo.cslot = (int)align_up((size_t)max(C, 1), 32);
    size_t o = 0;
    const size_t nj = (size_t)max(njobs, 1);
    lo.off_X = o; o = align_up(o + nj * lo.lslot * lo.cslot * sizeof(cf), 256);
    lo.off_V = o; o = align_up(o + nj * lo.cslot * lo.cslot * sizeof(cf), 256);
    lo.off_sig = o; o = align_up(o + nj * lo.cslot * sizeof(float), 256);
    lo.off_perm = o; o = align_up(o + nj * lo.cslot * sizeof(int), 256);
    lo.off_off = o; o = align_up(o + nj * sizeof(float), 256);
    lo.off_done = o; o = align_up(o + nj * sizeof(int), 256);
    lo.off_need = o; o = align_up(o + nj * sizeof(int), 256);
    lo.off_counter = o; o = align_up(o + 4 * sizeof(int), 256);
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

extern "C" int mps_apply_2q_batch(void* stream, const mps_2q_job* jobs, int njobs,
                                  int max_m, int max_n, int d, void* workspace,
                                  size_t workspace_bytes, mps_svd_params* params) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (njobs == 0) return MPS_OK;
    if (njobs < 0 || njobs > 65535 || !jobs) return fail(MPS_ERR_ARG, "mps_apply_2q_batch: bad job list");
    if (d < 1 || d > 64) return fail(MPS_ERR_ARG, "mps_apply_2q_batch: qudit dimension must be 1..64");
    if (max_m <= 0 || max_n <= 0)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch: max_m/max_n must be positive");
    const Layout lo = make_layout(njobs, max_m, max_n);
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
    g.sig = reinterpret_cast<float*>(ws + lo.off_sig);
    g.perm = reinterpret_cast<int*>(ws + lo.off_perm);
    g.offmax = reinterpret_cast<float*>(ws + lo.off_off);
    g.done = reinterpret_cast<int*>(ws + lo.off_done);
    g.need = reinterpret_cast<int*>(ws + lo.off_need);
    g.counter = reinterpret_cast<int*>(ws + lo.off_counter);

    int max_sweeps = 40, bc = 16;
    float tol = 0.f;
    if (params) {
        if (params->max_sweeps > 0) max_sweeps = params->max_sweeps;
        if (params->block_cols == 8) bc = 8;
        tol = params->tol;
    }
    if (!(tol > 0.f)) tol = fmaxf(sqrtf((float)lo.lslot) * 5.9604645e-8f, 1.1920929e-7f);
    const int lw = lo.lslot;
    size_t need_smem = (size_t)2 * bc * lw * sizeof(cf) + (size_t)4 * bc * bc * sizeof(cf) + 256;
    if (need_smem > (size_t)kMaxSmem) bc = 8;
    need_smem = (size_t)2 * bc * lw * sizeof(cf) + (size_t)4 * bc * bc * sizeof(cf) + 256;
    if (need_smem > (size_t)kMaxSmem)
        return fail(MPS_ERR_ARG, "mps_apply_2q_batch: merged matrix too long for shared memory");

    MPS_CUDA_CHECK(cudaMemsetAsync(g.X, 0, (size_t)njobs * lo.lslot * lo.cslot * sizeof(cf), s));
    {
        const size_t total = (size_t)njobs * lo.cslot * lo.cslot;
        int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
        blocks = max(blocks, (njobs + 255) / 256);
        init_slots_kernel<<<blocks, 256, 0, s>>>(g, njobs);
        MPS_LAUNCH_CHECK("init_slots_kernel");
    }
    const int max_chil = (max_m + d - 1) / d, max_chir = (max_n + d - 1) / d;
    int rc = merge_gate_launch(jobs, njobs, max_chil, max_chir, g, s);
    if (rc) return rc;

    const int cmax = min(max_m, max_n);
    int nbmax = (cmax + bc - 1) / bc;
    if (nbmax < 2) nbmax = 2;
    nbmax += nbmax & 1;
    const int rounds = nbmax - 1, pairs = nbmax / 2;
    round_fn fn = (bc == 16) ? pick_rows<16>(lw) : pick_rows<8>(lw);

    if (!t_pinned) {
        MPS_CUDA_CHECK(cudaHostAlloc(reinterpret_cast<void**>(&t_pinned), 4 * sizeof(int),
                                     cudaHostAllocDefault));
    }
    int sweeps = 0;
    bool converged = false;
    if (cmax >= 2) {
        for (sweeps = 1; sweeps <= max_sweeps; ++sweeps) {
            MPS_CUDA_CHECK(cudaMemsetAsync(g.counter, 0, sizeof(int), s));
            for (int r = 0; r < rounds; ++r) {
                rc = fn(jobs, njobs, pairs, g, r, tol, lw, s);
                if (rc) return rc;
            }
            sweep_end_kernel<<<(njobs + 255) / 256, 256, 0, s>>>(g, njobs, tol);
            MPS_LAUNCH_CHECK("sweep_end_kernel");
            MPS_CUDA_CHECK(cudaMemcpyAsync(t_pinned, g.counter, sizeof(int),
                                           cudaMemcpyDeviceToHost, s));
            MPS_CUDA_CHECK(cudaStreamSynchronize(s));
            if (t_pinned[0] == 0) {
                converged = true;
                break;
            }
        }
        if (sweeps > max_sweeps) sweeps = max_sweeps;
    } else {
        converged = true;
        // single-column (or empty) jobs: nothing to rotate
        MPS_CUDA_CHECK(cudaMemsetAsync(g.done, 0xff, (size_t)njobs * sizeof(int), s));
    }
    if (params) params->sweeps_out = sweeps;

    int npow2 = 1;
    while (npow2 < lo.cslot) npow2 <<= 1;
    const size_t sort_smem = (size_t)npow2 * (sizeof(float) + sizeof(int));
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
    }
    MPS_CUDA_CHECK(cudaMemcpyAsync(t_pinned + 1, g.counter + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPS_CUDA_CHECK(cudaStreamSynchronize(s));
    if (t_pinned[1] != 0) return fail(MPS_ERR_NONFINITE, "mps_apply_2q_batch: NaN/Inf singular value");
    if (!converged)
        return fail(MPS_ERR_NOT_CONVERGED, "mps_apply_2q_batch: Jacobi SVD hit its sweep cap");
    return MPS_OK;
}
