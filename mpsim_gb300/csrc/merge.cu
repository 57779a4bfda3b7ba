// Two-site merge with the gate fused into the epilogue (FP32 SIMT form).
//
// theta[(l,a'),(b',r)] = sum_{a,b} G[(a'b'),(ab)] sum_c A[l,a,c] B[c,b,r]
//
// mpsim computes this as two TensorNetwork contractions (mpsim/core.py:
// 1059-1062 merge, 1064-1068 gate).  Here one CTA computes a 64x64 tile of
// M = A.B whose rows are (l, a) for TL = 64/d values of l and all a, and whose
// columns are (b, r) for TR = 64/d values of r and all b -- exactly the
// entries the gate needs for the same theta tile -- then mixes the tile with
// the gate in shared memory and writes theta straight into the Jacobi working
// matrix X (column-major; conjugate-transposed for wide theta).
//
// A job flagged MPS_JOB_THETA_GIVEN carries theta itself: a points to the
// (chi_l*d) x (d*chi_r) matrix, row-major, and the same CTAs copy their tile
// of it into X (the plain truncated SVD of a given matrix, which
// from_wavefunction and the orthonormalisation of one site use).
#include "twoq.cuh"

namespace mps {

namespace {

constexpr int TILE = 64;
constexpr int KC = 16;
constexpr int NT = 256;

__global__ void __launch_bounds__(NT)
merge_gate_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g) {
    const mps_2q_job job = jobs[blockIdx.z];
    const int d = g.d;
    const int chil = job.chi_l, chim = job.chi_m, chir = job.chi_r;
    const int TL = TILE / d, TR = TILE / d;
    const int TM = TL * d, TN = TR * d;
    const int l0 = blockIdx.y * TL, r0 = blockIdx.x * TR;
    if (l0 >= chil || r0 >= chir) return;
    const int m = chil * d, n = d * chir;
    const bool tall = m >= n;
    const bool given = (job.flags & MPS_JOB_THETA_GIVEN) != 0;   // block-uniform
    if (g.tc_mode && merge_on_tensor_cores(job, d)) return;       // merge_tc_kernel's job

    __shared__ union {
        struct { cf a[KC][TILE]; cf b[KC][TILE]; } ld;
        cf mt[TILE][TILE + 1];
    } sh;

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    cf acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cmake(0.f, 0.f);

    const cf* A = reinterpret_cast<const cf*>(job.a);
    const cf* B = reinterpret_cast<const cf*>(job.b);
    const int row0 = l0 * d;
    for (int k0 = 0; k0 < (given ? 0 : chim); k0 += KC) {
#pragma unroll
        for (int q = 0; q < (KC * TILE) / NT; ++q) {
            const int idx = tid + q * NT;
            const int kk = idx % KC, tr = idx / KC;
            const int row = row0 + tr, k = k0 + kk;
            cf v = cmake(0.f, 0.f);
            if (tr < TM && row < m && k < chim) v = A[(size_t)row * chim + k];
            sh.ld.a[kk][tr] = v;
        }
#pragma unroll
        for (int q = 0; q < (KC * TILE) / NT; ++q) {
            const int idx = tid + q * NT;
            const int tc = idx % TILE, kk = idx / TILE;
            const int bb = tc / TR, r = r0 + tc % TR, k = k0 + kk;
            cf v = cmake(0.f, 0.f);
            if (tc < TN && r < chir && k < chim) v = B[(size_t)k * n + (size_t)bb * chir + r];
            sh.ld.b[kk][tc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < KC; ++kk) {
            cf av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = sh.ld.a[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = sh.ld.b[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) cfma(acc[i][j], av[i], bv[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) sh.mt[ty + 16 * i][tx + 16 * j] = acc[i][j];
    __syncthreads();

    const cf* G = reinterpret_cast<const cf*>(job.gate);
    cf* X = g.X + (size_t)blockIdx.z * g.lslot * g.cslot;
    cf* T = g.T + (size_t)blockIdx.z * g.lslot * g.cslot;
    const bool track_v = job_tracks_v(m, n, job.keep_left_canonical);
    const int dd = d * d;
    for (int e = tid; e < TILE * TILE; e += NT) {
        int tr, tc;
        if (tall) { tr = e % TILE; tc = e / TILE; } else { tc = e % TILE; tr = e / TILE; }
        if (tr >= TM || tc >= TN) continue;
        const int l = l0 + tr / d, ap = tr % d;
        const int bp = tc / TR, rr = tc % TR, r = r0 + rr;
        if (l >= chil || r >= chir) continue;
        const int trow = l * d + ap;              // theta row
        const int tcol = bp * chir + r;           // theta column
        cf th = cmake(0.f, 0.f);
        if (given) {
            th = A[(size_t)trow * n + tcol];
        } else {
            const cf* grow = G + (size_t)(ap * d + bp) * dd;
            const int rbase = tr - ap;            // tile row of (l, a=0)
            for (int a = 0; a < d; ++a)
                for (int b = 0; b < d; ++b)
                    cfma(th, __ldg(reinterpret_cast<const float2*>(grow + a * d + b)),
                         sh.mt[rbase + a][b * TR + rr]);
        }
        if (tall) {
            X[(size_t)tcol * g.lslot + trow] = th;
            if (!track_v) T[(size_t)tcol * g.lslot + trow] = th;
        } else {
            X[(size_t)trow * g.lslot + tcol] = cconj(th);
        }
    }
}

}  // namespace

int merge_gate_launch(const mps_2q_job* jobs, int njobs, int max_chil, int max_chir,
                      const TwoQGeom& g, cudaStream_t s) {
    if (njobs <= 0) return MPS_OK;
    const int TL = TILE / g.d, TR = TILE / g.d;
    dim3 grid((max_chir + TR - 1) / TR, (max_chil + TL - 1) / TL, njobs);
    if (grid.x == 0 || grid.y == 0) return MPS_OK;
    merge_gate_kernel<<<grid, NT, 0, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("merge_gate_kernel");
    return MPS_OK;
}

}  // namespace mps
