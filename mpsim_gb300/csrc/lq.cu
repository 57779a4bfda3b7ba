// lq.cu -- LQ preconditioning of the Jacobi SVD (sm_103a).
//
// For a job whose left factor is read off the final Jacobi columns (theta
// tall or square, keep_left_canonical: X = theta, L x C, column-major in the
// X slot), X is replaced by its L factor before the sweeps:
//
//     X = L Q,  Q (C x C) unitary,  L (L x C) lower trapezoidal.
//
// Q changes neither the singular values nor the left singular vectors, so
// the sweeps' final columns L V = U S still give U, and S V^H is formed as
// U'^H theta from the untouched copy of theta in g.T, exactly as without the
// factorisation.  One-sided Jacobi needs markedly fewer sweeps on the
// triangular factor than on theta itself: the QR-preconditioned Jacobi SVD
// of Drmac and Veselic (SIAM J. Matrix Anal. Appl. 29, 2008), here applied to
// the rows (theta^H = Q^H L^H is the QR factorisation of theta^H).  On the
// chi=256 brickwork layers the sorted ring needs about 10 sweeps on L
// against 14-15 on theta.
//
// Algorithm: blocked Householder reflectors applied from the right.  For
// each panel of LQ_B rows k0 .. k0+kb-1:
//   lq_panel_kernel (one CTA per job): the panel (kb x (C-k0)) in shared
//     memory; for row i the reflector H_i = I - tau_i v_i v_i^H with
//     x_i H_i = beta_i e_i (x_i the row, beta_i real; the textbook complex
//     Householder vector of y = x_i^H: beta = -sign(Re y0) |y|,
//     tau = (beta - y0) / beta, v = (1, y_1.. / (y0 - beta))), applied at once
//     to the panel rows below; then the compact WY factor
//     H_0 ... H_{kb-1} = I - V T V^H (T upper triangular,
//     T[0:i, i] = -tau_i T[0:i, 0:i] V[:, 0:i]^H v_i).
//   lq_trail_kernel (job x 64-row tiles): the rows below the panel,
//     R <- R (I - V T V^H) = R - ((R V) T) V^H.
// V (nc x LQ_B) and T (LQ_B x LQ_B) of the current panel live in the job's
// V slot, which jobs of this kind do not otherwise use before the Gram step
// after the sweeps.
#include <mutex>

#include "twoq.cuh"

namespace mps {
namespace {

constexpr int LQ_B = 32;        // rows per panel
constexpr int LQ_T = 1024;      // threads of the panel kernel: a warp per panel row
constexpr int LQ_NW = LQ_T / 32;
constexpr int LQ_TR = 64;       // rows per trailing-update CTA
constexpr int LQ_MIN_C = 64;    // narrower jobs converge in a few cheap sweeps anyway
constexpr int LQ_MAX_C = 768;   // the panel (LQ_B x (C+1)) must fit in shared memory
// V (C x LQ_B) and T (LQ_B x LQ_B, at offset LQ_B * cslot) must fit in the
// job's cslot x cslot V slot; cslot >= C >= LQ_MIN_C
static_assert(LQ_MIN_C * LQ_MIN_C >= LQ_B * (LQ_MIN_C + LQ_B), "V slot too small for V and T");

// Jobs that are factorised, and their shape (X is L x C).
__device__ __forceinline__ bool lq_job(const mps_2q_job& job, int d, int& L, int& C) {
    const int m = job.chi_l * d, n = job.chi_r * d;
    if (job_tracks_v(m, n, job.keep_left_canonical)) return false;
    L = m;
    C = n;
    return C >= LQ_MIN_C && C <= LQ_MAX_C;
}

__device__ __forceinline__ cf cinv(cf a) {
    const float s = 1.f / cabs2(a);
    return cmake(a.x * s, -a.y * s);
}

__global__ void __launch_bounds__(LQ_T)
lq_panel_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int k0) {
    extern __shared__ float2 lq_sm[];
    const int j = blockIdx.x;
    int L, C;
    if (!lq_job(jobs[j], g.d, L, C) || k0 >= C) return;
    const int kb = min(LQ_B, C - k0), nc = C - k0, ps = nc + 1;
    cf* P = lq_sm;                              // [kb][ps]: the panel, row-major
    cf* zz = P + (size_t)LQ_B * ps;             // [LQ_B][LQ_B]: (V^H V)[a][b], a < b
    cf* Ts = zz + LQ_B * LQ_B;                  // [LQ_B][LQ_B]: T, row-major
    cf* tau = Ts + LQ_B * LQ_B;                 // [LQ_B]
    cf* invs = tau + LQ_B;                      // [LQ_B]: 1 / (y0 - beta)
    float* betas = reinterpret_cast<float*>(invs + LQ_B);   // [LQ_B]
    float* tail = betas + LQ_B;                 // [2]: |row i|^2 beyond its diagonal
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    cf* X = g.X + (size_t)j * g.lslot * g.cslot;

#pragma unroll 4
    for (int e = tid; e < kb * nc; e += LQ_T) {
        const int r = e % kb, c = e / kb;
        P[r * ps + c] = X[(size_t)(k0 + c) * g.lslot + k0 + r];
    }
    __syncthreads();
    if (warp == 0) {
        float s = 0.f;
        for (int c = 1 + lane; c < nc; c += 32) s += cabs2(P[c]);
        s = warp_sum(s);
        if (lane == 0) tail[0] = s;
    }
    __syncthreads();

    // One barrier per reflector.  Every thread derives H_i from row i's
    // diagonal entry and tail norm (left by the warp that updated row i in the
    // step before); the rows below use row i unscaled (v = conj(x) inv), and
    // row i becomes (beta, v) only after the loop.
    for (int i = 0; i < kb; ++i) {
        const cf* x = P + (size_t)i * ps;
        const cf y0 = cconj(x[i]);
        const float s = tail[i & 1];
        cf t = cmake(0.f, 0.f), inv = cmake(0.f, 0.f);
        float beta = y0.x;
        if (s > 0.f || y0.y != 0.f) {
            const float nrm = sqrtf(cabs2(y0) + s);
            beta = y0.x >= 0.f ? -nrm : nrm;
            t = cmake((beta - y0.x) / beta, -y0.y / beta);
            inv = cinv(cmake(y0.x - beta, y0.y));
        }
        if (tid == 0) {
            tau[i] = t;
            invs[i] = inv;
            betas[i] = beta;
        }
        // z <- z H_i: d = z v = z[i] + inv sum_c z[c] conj(x[c]);
        // z[i] -= tau d, z[c] -= tau d conj(inv) x[c]
        for (int r = i + 1 + warp; r < kb; r += LQ_NW) {
            cf* z = P + (size_t)r * ps;
            const cf zi = z[i];
            cf acc = cmake(0.f, 0.f);
            for (int c = i + 1 + lane; c < nc; c += 32) cfma_conj(acc, x[c], z[c]);
            acc.x = warp_sum(acc.x);
            acc.y = warp_sum(acc.y);
            const cf td = cmul(t, cadd(zi, cmul(inv, acc)));
            const cf kx = cmul(td, cconj(inv));
            if (lane == 0) z[i] = csub(zi, td);
            float nn = 0.f;
            for (int c = i + 1 + lane; c < nc; c += 32) {
                const cf zc = csub(z[c], cmul(kx, x[c]));
                z[c] = zc;
                if (c > i + 1) nn += cabs2(zc);
            }
            if (r == i + 1) {
                nn = warp_sum(nn);
                if (lane == 0) tail[(i + 1) & 1] = nn;
            }
        }
        __syncthreads();
    }
    for (int e = tid; e < kb * nc; e += LQ_T) {
        const int i = e / nc, c = e - (e / nc) * nc;
        if (c > i) P[(size_t)i * ps + c] = cmul(cconj(P[(size_t)i * ps + c]), invs[i]);
        else if (c == i) P[(size_t)i * ps + c] = cmake(betas[i], 0.f);
    }
    __syncthreads();

    // (V^H V)[a][b] for a < b, with V[c][a] = 0 (c < a), 1 (c = a), P[a][c] (c > a)
    for (int pi = warp; pi < kb * kb; pi += LQ_NW) {
        const int a = pi / kb, b = pi - (pi / kb) * kb;
        if (a >= b) continue;
        const cf* va = P + (size_t)a * ps;
        const cf* vb = P + (size_t)b * ps;
        cf s = lane == 0 ? cconj(va[b]) : cmake(0.f, 0.f);
        for (int c = b + 1 + lane; c < nc; c += 32) cfma_conj(s, va[c], vb[c]);
        s.x = warp_sum(s.x);
        s.y = warp_sum(s.y);
        if (lane == 0) zz[a * LQ_B + b] = s;
    }
    __syncthreads();
    if (warp == 0) {
        for (int i = 0; i < kb; ++i) {
            cf val = cmake(0.f, 0.f);
            if (lane < i) {
                cf s = cmake(0.f, 0.f);
                for (int b = lane; b < i; ++b) cfma(s, Ts[lane * LQ_B + b], zz[b * LQ_B + i]);
                const cf ts = cmul(tau[i], s);
                val = cmake(-ts.x, -ts.y);
            } else if (lane == i) {
                val = tau[i];
            }
            __syncwarp();
            Ts[lane * LQ_B + i] = val;
            __syncwarp();
        }
    }
    __syncthreads();

    // V (nc x LQ_B, zero beyond kb) and T (LQ_B x LQ_B) to the V slot
    cf* Vg = g.V + (size_t)j * g.cslot * g.cslot;
    cf* Tg = Vg + (size_t)LQ_B * g.cslot;
    for (int e = tid; e < nc * LQ_B; e += LQ_T) {
        const int c = e / LQ_B, b = e % LQ_B;
        cf v = cmake(0.f, 0.f);
        if (b < kb) v = c < b ? cmake(0.f, 0.f) : (c == b ? cmake(1.f, 0.f) : P[(size_t)b * ps + c]);
        Vg[e] = v;
    }
    for (int e = tid; e < LQ_B * LQ_B; e += LQ_T) {
        const int a = e / LQ_B, b = e % LQ_B;
        Tg[e] = (a < kb && b < kb && b >= a) ? Ts[e] : cmake(0.f, 0.f);
    }
    // the panel's rows of L: left of the diagonal as transformed, beta on it,
    // zero right of it
    for (int e = tid; e < kb * nc; e += LQ_T) {
        const int r = e % kb, c = e / kb;
        const cf v = c <= r ? P[r * ps + c] : cmake(0.f, 0.f);
        X[(size_t)(k0 + c) * g.lslot + k0 + r] = v;
    }
}

// Rows k0+kb .. L-1 of the job: R <- R - ((R V) T) V^H, 64 rows per CTA,
// in 32-column chunks; each chunk's global loads are issued while the
// previous chunk is being multiplied.
__global__ void __launch_bounds__(256)
lq_trail_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int k0) {
    // phase 1: Xs [32][LQ_TR] and Bs [32][LQ_B] (a V chunk, then T);
    // phase 2: Vt [LQ_B][33] (a conjugated V chunk, transposed) over Xs
    __shared__ cf sm[32 * LQ_TR + 32 * LQ_B + LQ_B * LQ_TR];
    cf (*Xs)[LQ_TR] = reinterpret_cast<cf (*)[LQ_TR]>(sm);
    cf (*Vt)[33] = reinterpret_cast<cf (*)[33]>(sm);
    cf (*Bs)[LQ_B] = reinterpret_cast<cf (*)[LQ_B]>(sm + 32 * LQ_TR);
    cf (*Ws)[LQ_TR] = reinterpret_cast<cf (*)[LQ_TR]>(sm + 32 * LQ_TR + 32 * LQ_B);
    const int j = blockIdx.y;
    int L, C;
    if (!lq_job(jobs[j], g.d, L, C) || k0 >= C) return;
    const int kb = min(LQ_B, C - k0), nc = C - k0;
    const int row0 = k0 + kb + blockIdx.x * LQ_TR;
    if (row0 >= L) return;
    const int tid = threadIdx.x, rr = tid & (LQ_TR - 1), q = tid / LQ_TR;   // q: 0..3
    const int r = row0 + rr;
    const bool live = r < L;
    cf* X = g.X + (size_t)j * g.lslot * g.cslot;
    const cf* Vg = g.V + (size_t)j * g.cslot * g.cslot;
    const cf* Tg = Vg + (size_t)LQ_B * g.cslot;
    const cf zero = cmake(0.f, 0.f);

    // W[r][b] = sum_c X[r][k0 + c] V[c][b]; this thread: b = q*8 .. q*8+7.
    // Staging: element q2*256 + tid of a chunk is X column q2*4 + q, row rr,
    // and V row (q2*256+tid)/32, column tid % 32.
    cf xr[8], vr[4];
    auto fetch1 = [&](int c0) {
#pragma unroll
        for (int q2 = 0; q2 < 8; ++q2) {
            const int c = c0 + q2 * 4 + q;
            xr[q2] = (c < nc && live) ? X[(size_t)(k0 + c) * g.lslot + r] : zero;
        }
#pragma unroll
        for (int q2 = 0; q2 < 4; ++q2) {
            const int e = q2 * 256 + tid, c = c0 + e / LQ_B;
            vr[q2] = c < nc ? Vg[(size_t)c * LQ_B + (e % LQ_B)] : zero;
        }
    };
    cf acc[8];
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[b] = zero;
    fetch1(0);
    for (int c0 = 0; c0 < nc; c0 += 32) {
#pragma unroll
        for (int q2 = 0; q2 < 8; ++q2) Xs[q2 * 4 + q][rr] = xr[q2];
#pragma unroll
        for (int q2 = 0; q2 < 4; ++q2) {
            const int e = q2 * 256 + tid;
            Bs[e / LQ_B][e % LQ_B] = vr[q2];
        }
        __syncthreads();
        if (c0 + 32 < nc) fetch1(c0 + 32);
#pragma unroll 4
        for (int cc = 0; cc < 32; ++cc) {
            const cf x = Xs[cc][rr];
#pragma unroll
            for (int b = 0; b < 8; ++b) cfma(acc[b], x, Bs[cc][q * 8 + b]);
        }
        __syncthreads();
    }
    // W <- W T (T upper triangular)
#pragma unroll
    for (int b = 0; b < 8; ++b) Ws[q * 8 + b][rr] = acc[b];
#pragma unroll
    for (int q2 = 0; q2 < 4; ++q2) {
        const int e = q2 * 256 + tid;
        Bs[e / LQ_B][e % LQ_B] = Tg[e];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int bb = q * 8 + b;
        cf w = zero;
        for (int a = 0; a <= bb; ++a) cfma(w, Ws[a][rr], Bs[a][bb]);
        acc[b] = w;
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < 8; ++b) Ws[q * 8 + b][rr] = acc[b];

    // X[r][k0 + c] -= sum_b W[r][b] conj(V[c][b]); this thread: columns
    // q*8 .. q*8+7 of each chunk (its row's entries fetched a chunk ahead)
    cf zr[8];
    auto fetch2 = [&](int c0) {
#pragma unroll
        for (int q2 = 0; q2 < 4; ++q2) {
            const int e = q2 * 256 + tid, c = c0 + e / LQ_B;
            vr[q2] = c < nc ? Vg[(size_t)c * LQ_B + (e % LQ_B)] : zero;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int c = c0 + q * 8 + k;
            zr[k] = (live && c < nc) ? X[(size_t)(k0 + c) * g.lslot + r] : zero;
        }
    };
    fetch2(0);
    for (int c0 = 0; c0 < nc; c0 += 32) {
#pragma unroll
        for (int q2 = 0; q2 < 4; ++q2) {
            const int e = q2 * 256 + tid;
            Vt[e % LQ_B][e / LQ_B] = cconj(vr[q2]);
        }
        cf z[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) z[k] = zr[k];
        __syncthreads();
        if (c0 + 32 < nc) fetch2(c0 + 32);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int cc = q * 8 + k, c = c0 + cc;
            cf s = cmake(0.f, 0.f);
#pragma unroll 8
            for (int b = 0; b < LQ_B; ++b) cfma(s, Ws[b][rr], Vt[b][cc]);
            if (live && c < nc) X[(size_t)(k0 + c) * g.lslot + r] = csub(z[k], s);
        }
        __syncthreads();
    }
}

// Column norms of the factorised jobs for the first sweep's sort.
__global__ void __launch_bounds__(256) lq_norm_kernel(const mps_2q_job* __restrict__ jobs,
                                                      TwoQGeom g) {
    const int j = blockIdx.y;
    int L, C;
    if (!lq_job(jobs[j], g.d, L, C)) return;
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (c >= C) return;
    const cf* col = g.X + (size_t)j * g.lslot * g.cslot + (size_t)c * g.lslot;
    float acc = 0.f;
    for (int r = lane; r < L; r += 32) acc += cabs2(col[r]);
    acc = warp_sum(acc);
    if (lane == 0) g.cnrm[(size_t)j * g.cslot + c] = acc;
}

}  // namespace

int lq_precondition(const mps_2q_job* jobs, int njobs, int max_m, int max_n, const TwoQGeom& g,
                    cudaStream_t s) {
    const int cmax = min(min(max_m, max_n), LQ_MAX_C);
    if (cmax < LQ_MIN_C) return MPS_OK;
    // the shared-memory opt-in is per device: set it once on every device used
    static std::once_flag once[kMaxDevices];
    static cudaError_t attr[kMaxDevices];
    const size_t smem_max = ((size_t)LQ_B * (LQ_MAX_C + 1) + 2 * LQ_B * LQ_B + 3 * LQ_B) * sizeof(cf);
    int dev = 0;
    MPS_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(MPS_ERR_ARG, "lq_precondition: device index beyond 63");
    std::call_once(once[dev], [&] {
        attr[dev] = cudaFuncSetAttribute(lq_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_max);
    });
    if (attr[dev] != cudaSuccess) return cuda_fail(attr[dev], "cudaFuncSetAttribute(lq_panel_kernel)");
    const size_t smem = ((size_t)LQ_B * (cmax + 1) + 2 * LQ_B * LQ_B + 3 * LQ_B) * sizeof(cf);
    for (int k0 = 0; k0 < cmax; k0 += LQ_B) {
        lq_panel_kernel<<<njobs, LQ_T, smem, s>>>(jobs, g, k0);
        MPS_LAUNCH_CHECK("lq_panel_kernel");
        const int rows = max_m - k0;     // covers every job's rows below its panel
        if (rows > 0) {
            lq_trail_kernel<<<dim3((rows + LQ_TR - 1) / LQ_TR, njobs), 256, 0, s>>>(jobs, g, k0);
            MPS_LAUNCH_CHECK("lq_trail_kernel");
        }
    }
    lq_norm_kernel<<<dim3((cmax + 7) / 8, njobs), 256, 0, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("lq_norm_kernel");
    return MPS_OK;
}

}  // namespace mps
