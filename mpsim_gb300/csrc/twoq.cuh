// Workspace geometry shared by the two-qudit kernels (merge, Jacobi SVD,
// sort, regauge).  One slot per job; every job's slot has the same shape.
//
// For a job with theta of m x n (m = chi_l*d, n = d*chi_r):
//   tall (m >= n): the Jacobi matrix X is theta itself, column-major,
//                  C = n columns of length L = m.  X V = U S.
//   wide (m <  n): X is theta^H (conjugate transpose), C = m columns of
//                  length L = n.  theta = V S (X/S)^H.
// X: lslot x cslot complex64, column-major (column c at X + c*lslot).
// V: cslot x cslot complex64, column-major, starts as the identity.
#pragma once

#include "common.cuh"

namespace mps {

struct TwoQGeom {
    int d;
    int lslot;        // rows per slot, multiple of 32
    int cslot;        // columns per slot, multiple of 32
    cf* X;            // njobs * lslot * cslot
    cf* V;            // njobs * cslot * cslot (only jobs that track V use theirs)
    cf* T;            // njobs * lslot * cslot: copy of theta for jobs that form
                      // S V^H as U^H theta instead of tracking V
    float* sig;       // njobs * cslot: sorted singular values
    int* perm;        // njobs * cslot: source column of each sorted value
    float* offmax;    // njobs: max relative off-diagonal seen this sweep
    int* done;        // njobs: 1 once a sweep made no rotation
    int* need;        // njobs: kept columns that need an orthonormal completion
    int* counter;     // [0] jobs still rotating, [1] jobs with NaN/Inf, [2] the tensor-core
                      // sweep's item counter, [3] an expired wait (MMA or round flag),
                      // [4] / [5] tensor-core / SIMT jobs left after a sweep (mixed
                      // calls), [6] SIMT jobs of a mixed call
    int* cmap;        // njobs * cslot: physical column at each sorted position
    float* cnrm;      // njobs * cslot: squared norm of each physical column
    int* scale;       // njobs: theta was multiplied by 2^scale[j] before the SVD
    double* nrm2;     // njobs: |theta|_F^2 (scratch of the scaling)
    // Visit skipping of the sweep kernel (null where unused).  Times count
    // t = sweep * (rounds + 1) + round + 1, and sweep * (rounds + 1) for the
    // sort before a sweep.
    int* vstamp;      // njobs * nbmax: last time a column block changed
    int* qstamp;      // njobs * qstride: last time visit (round, pair) rotated nothing
    int nbmax, qstride;
    // MPS_PRECISION_MIXED only (null otherwise): X split into three bf16
    // piece planes per job, plane i of job j at P + (3 j + i) * pplane, each
    // laid out like X (column c = 2 lslot bf16 at c * 2 lslot); during the
    // tensor-core sweeps the planes, not X, hold the columns
    uint16_t* P;
    size_t pplane;
    // 1 in MPS_PRECISION_MIXED calls: the jobs tc_job() accepts take the
    // tensor-core sweeps, the SIMT sweep kernel the others
    int tc_mode;
};

// Work distribution of the persistent sweep kernel.
struct SweepSync {
    int* next_item;   // atomic item counter (reset to 0 before each sweep)
    int* error;       // set to 1 when a dependency wait expires
    int* block_round; // [njobs][nbmax]: last round each block finished (-1)
    int nbmax;
    int wait_limit;
    int stall_test;
};

// A job tracks the right rotations V unless it is tall (m >= n) and left-
// canonical: then U = X/S is all the Jacobi iteration must produce, and the
// right site S V^H = U^H theta comes from one GEMM against a copy of theta.
__host__ __device__ __forceinline__ bool job_tracks_v(int m, int n, int keep_left_canonical) {
    return !(m >= n && keep_left_canonical != 0);
}

// The jobs of a mixed call that take the tensor-core sweeps: left-canonical,
// tall, 64+ columns (their left factor comes from the final columns).
__host__ __device__ __forceinline__ bool tc_job(int m, int n, int keep_left_canonical) {
    return !job_tracks_v(m, n, keep_left_canonical) && (m < n ? m : n) >= 64;
}

// ... and whose merge runs on the tensor cores as well (theta not given;
// qudits of up to 4 levels: the gate step keeps a d^2 block in registers).
__host__ __device__ __forceinline__ bool merge_on_tensor_cores(const mps_2q_job& job, int d) {
    return d <= 4 && tc_job(job.chi_l * d, job.chi_r * d, job.keep_left_canonical) &&
           (job.flags & MPS_JOB_THETA_GIVEN) == 0;
}

// Singular values at or below this (relative to max(s_0, 1)) are treated as
// exact zeros: the isometric factor gets an orthonormal completion there.
constexpr float kZeroSigma = 1e-30f;

// Replaces X by its L factor (X = L Q) for the jobs whose left factor comes
// from the final columns (lq.cu); the sweeps then need fewer passes.
int lq_precondition(const mps_2q_job* jobs, int njobs, int max_m, int max_n, const TwoQGeom& g,
                    cudaStream_t s);

// Tensor-core block sweeps (tcjacobi.cu): one persistent launch runs every
// round of one sweep of the tc_job() jobs, 32-column blocks, with the sweep
// kernel's round flags (sync, with its own item counter) and visit stamps
// (tbase).  counter[3] (and sync.error) is set when a bounded MMA wait
// expired.
int tc_sweep_launch(const mps_2q_job* jobs, int njobs, int rounds, int pairs, const TwoQGeom& g,
                    float tol2, const SweepSync& sync, int tbase, cudaStream_t s);
// X -> its bf16 piece planes (before the first tensor-core sweep), and the
// planes summed back into X (after the last one), for the tc_job() jobs.
int tc_split_launch(const mps_2q_job* jobs, int njobs, const TwoQGeom& g, cudaStream_t s);
int tc_merge_launch(const mps_2q_job* jobs, int njobs, const TwoQGeom& g, cudaStream_t s);

// The mixed form's merge of the merge_on_tensor_cores() jobs (tcgemm.cu): M =
// A B on tcgen05 (split bf16, FP32-grade) into X, then the gate mixed in
// place and copied to T.  The SIMT merge skips those jobs in such a call.
int merge_tc_launch(const mps_2q_job* jobs, int njobs, int max_m, int max_n, const TwoQGeom& g,
                    cudaStream_t s);
int merge_gate_launch(const mps_2q_job* jobs, int njobs, int max_chil, int max_chir,
                      const TwoQGeom& g, cudaStream_t s);

}  // namespace mps
