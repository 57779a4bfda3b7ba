/*
 * mpsim_gb300.h -- C ABI of the GB300 (sm_103a) MPS gate-application core.
 *
 * All tensor pointers are DEVICE pointers to interleaved complex64 (two
 * floats, the layout of numpy.complex64 / torch.complex64).  Every call takes
 * an explicit cudaStream_t (passed as void*) and enqueues its kernels on it.
 * Functions return MPS_OK (0) or a nonzero MPS_ERR_* code; mps_last_error()
 * gives a message for the most recent failure on the calling thread.
 *
 * Site tensors use the layout (chi_left, d, chi_right), row-major: element
 * (l, a, r) at ((l * d) + a) * chi_right + r.  A gate acting on one qudit is a
 * d x d matrix U[a', a]; a gate acting on two qudits is a (d*d) x (d*d)
 * matrix G[(a' b'), (a b)] where a is the qudit of the LEFT site.
 *
 * The reference (grmlarose/mpsim) is pure Python and has no native
 * interface; each entry point names the Python method of mpsim/core.py whose
 * arithmetic it replaces.  The Python package mpsim_gb300 binds these through
 * ctypes and keeps mpsim's method names and error behaviour.
 */
#ifndef MPSIM_GB300_H
#define MPSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPS_OK 0
#define MPS_ERR_ARG 1          /* invalid argument (shape, pointer, size)   */
#define MPS_ERR_CUDA 2         /* a CUDA runtime call failed                */
#define MPS_ERR_WORKSPACE 3    /* workspace too small                       */
#define MPS_ERR_NOT_CONVERGED 4/* Jacobi SVD hit its sweep cap              */
#define MPS_ERR_NONFINITE 5    /* NaN/Inf met in a singular value           */
#define MPS_ERR_TIMEOUT 6      /* a bounded in-kernel wait expired          */

/* Per-job status bits written by mps_apply_2q_batch (the only report of a
 * call made under stream capture, which reads nothing back). */
#define MPS_STATUS_NOT_CONVERGED 1
#define MPS_STATUS_NONFINITE 2
#define MPS_STATUS_TIMEOUT 4

typedef struct { float re, im; } mps_c64;

/* mps_2q_job.flags: the job is the truncated SVD of a given matrix (a points
 * to theta itself, (chi_l*d) x (d*chi_r) row-major; b, gate and chi_m are
 * unused).  The plain SVD that from_wavefunction and the orthonormalisation
 * of one site need (mpsim/core.py:245-328, 847-937). */
#define MPS_JOB_THETA_GIVEN 1

/* One two-qudit gate on adjacent sites (left site a, right site b).
 * 88 bytes, naturally aligned; the Python side mirrors it field by field. */
typedef struct {
    const mps_c64* a;      /* (chi_l, d, chi_m), or theta (see flags)      */
    const mps_c64* b;      /* (chi_m, d, chi_r)                            */
    const mps_c64* gate;   /* (d*d, d*d) row-major G[(a'b'),(ab)]          */
    mps_c64* a_out;        /* (chi_l, d, k): new left site                 */
    mps_c64* b_out;        /* (k, d, chi_r): new right site                */
    float* svals;          /* optional: min(m,n) singular values, descending */
    double* discarded;     /* optional: sum of squares of dropped values   */
    int32_t* status;       /* optional: MPS_STATUS_* bits for this job     */
    int32_t chi_l, chi_m, chi_r;
    int32_t k;             /* kept count, 0 <= k <= min(chi_l*d, d*chi_r)  */
    int32_t keep_left_canonical; /* 1: left=U, right=S.V^H; 0: U.S, V^H   */
    int32_t flags;         /* MPS_JOB_* bits; 0 for a gate on two sites    */
} mps_2q_job;

/* Solver controls for the Jacobi SVD (zero fields take the defaults). */
typedef struct {
    int32_t max_sweeps;    /* default 40                                   */
    float tol;             /* relative off-diagonal threshold; default
                              2^-24 * max(8, sqrt(rows))                   */
    int32_t block_cols;    /* out: columns per block the kernel used       */
    int32_t sweeps_out;    /* out: sweeps taken by the slowest job         */
    int32_t wait_limit;    /* max polls of a round-dependency wait inside a
                              sweep (default 1<<22, ~0.3 s); on expiry the
                              call returns MPS_ERR_TIMEOUT                 */
    int32_t stall_test;    /* test hook: nonzero makes one wait target a
                              round that never completes, so the wait must
                              expire (with a small wait_limit)             */
    int32_t precision;     /* MPS_PRECISION_PLAIN (default) or
                              MPS_PRECISION_MIXED                          */
    int32_t lq_off;        /* nonzero: no LQ preconditioning (the sweeps run
                              on theta itself)                              */
    int32_t block_request; /* Jacobi block width of the plain form for slots
                              of 512 / 576 rows: 0 (default) = 16, or 8     */
} mps_svd_params;

/* mps_svd_params.precision.
 * PLAIN: complex64 with FP32 SIMT arithmetic throughout.
 * MIXED: the Jacobi sweeps run as 32-column block pairs whose Gram matrices
 *   G = Y^H Y and rotations Y <- Y Q are tcgen05 tensor-core GEMMs on bf16
 *   operands (every FP32 value split into three bf16 pieces, six piece
 *   products accumulated in FP32 in TMEM: FP32-grade products); the rotation
 *   parameters come from G in shared memory, the off-diagonal test is FP64.
 *   This form covers the tall (m >= n), left-canonical jobs of 64+ columns;
 *   the call's other jobs take the PLAIN sweeps in the same sweep loop. */
#define MPS_PRECISION_PLAIN 0
#define MPS_PRECISION_MIXED 1

/* Library version and build description. */
int mps_version(void);
const char* mps_last_error(void);
/* Kernel launches this library has issued in the process so far. */
unsigned long long mps_kernel_launches(void);

/* One-qudit gate in place: site[l,a',r] = sum_a U[a',a] site[l,a,r].
 * Replaces MPS.apply_one_qudit_gate, unitary branch (mpsim/core.py:753-826). */
int mps_apply_1q(void* stream, mps_c64* site, int chi_l, int d, int chi_r,
                 const mps_c64* gate);

/* One-qudit gates on many sites (of one or many states) in one launch.
 * 24 bytes; the Python side mirrors it field by field. */
typedef struct {
    mps_c64* site;         /* (chi_l, d, chi_r), updated in place           */
    const mps_c64* gate;   /* (d, d) row-major U[a', a]                     */
    int32_t chi_l, chi_r;
} mps_1q_job;

/* mps_apply_1q for njobs (site, gate) pairs in a device array; sites must not
 * alias.  Same arithmetic as MPS.apply_one_qudit_gate, unitary branch
 * (mpsim/core.py:820-826), batched over states for the multi-circuit form. */
int mps_apply_1q_batch(void* stream, const mps_1q_job* jobs_dev, int njobs, int d);

/* Workspace bytes mps_apply_2q_batch needs for njobs jobs whose merged
 * matrices are at most max_m x max_n (m = chi_l*d, n = d*chi_r). */
size_t mps_2q_workspace_bytes(int njobs, int max_m, int max_n, int d);

/* The same for a call with params->precision == MPS_PRECISION_MIXED, whose
 * workspace also holds every job's matrix split into three bf16 piece planes
 * (12 more bytes per complex element); such a call with a smaller workspace
 * returns MPS_ERR_WORKSPACE. */
size_t mps_2q_workspace_bytes_mixed(int njobs, int max_m, int max_n, int d);

/* Applies njobs independent two-qudit gates (jobs_dev: a device array of
 * mps_2q_job; the sites of different jobs must not alias).  Per job: merge
 * A.B with the gate fused in (theta = (chi_l*d) x (d*chi_r)), block one-sided
 * Jacobi SVD, descending sort, truncation to k values, and the regauge with
 * the singular values placed as keep_left_canonical asks.  max_m/max_n bound
 * every job's theta; the host must know them.  Left-canonical jobs with
 * m >= n and 64 <= n <= 768 run the Jacobi sweeps on the L factor of theta
 * (theta = L Q, Householder from the right), which needs fewer sweeps and
 * leaves the singular values and left vectors unchanged; the right factor
 * is then formed as U^H theta.  Blocks the calling thread
 * once per Jacobi sweep to test convergence, and returns after the last
 * sweep with the sort, regauge and output kernels still queued on the stream
 * (the outputs are stream-ordered like any kernel's).  Under stream capture
 * (cudaStreamIsCapturing) it never blocks: it queues params->max_sweeps
 * sweeps (default 40; converged jobs return at once from each) and reports
 * only through each job's status word, so a whole circuit can be captured
 * into one CUDA graph.
 * Replaces MPS.apply_two_qudit_gate for adjacent sites (mpsim/core.py:
 * 1059-1152: merge 1059-1062, gate 1064-1068, truncated SVD 1132-1137 via
 * TensorNetwork split_node_full_svd, S placement 1139-1145). */
int mps_apply_2q_batch(void* stream, const mps_2q_job* jobs_dev, int njobs,
                       int max_m, int max_n, int d, void* workspace,
                       size_t workspace_bytes, mps_svd_params* params);

/* Size of the fixed device scratch array behind mps_apply_2q_batch_noalloc. */
#define MPS_NOALLOC_SCRATCH_BYTES (32u << 20)

/* mps_apply_2q_batch for callers that cannot allocate device memory (an
 * application whose own pool owns the GPU's memory, a plugin host that gives
 * its plugins no allocator, a loop that must never enter the allocator).
 * No counterpart in the reference (it has no native interface at all).
 * Same jobs, same results; scratch comes from a static __device__ array of
 * MPS_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until
 * exit, and the call allocates nothing.  Jobs whose slots need more scratch
 * than that are rejected with MPS_ERR_WORKSPACE (at theta 512x512 about five
 * jobs fit per call).  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current: make it before any
 * stream capture.  Calls share the array: calls that overlap on the GPU race
 * and must be serialised by the caller.  The call returns only when its work
 * on the stream has finished: it reads the convergence and non-finite counts
 * back into host memory (always the plain form, whatever params->precision). */
int mps_apply_2q_batch_noalloc(void* stream, const mps_2q_job* jobs_dev, int njobs,
                               int max_m, int max_n, int d, mps_svd_params* params);

/* Workspace bytes for the contractions below (sites of at most max_chi). */
size_t mps_sweep_workspace_bytes(int max_chi, int d);

/* <a|b>-style overlap, reference convention: sum_x a(x) * conj(b(x)).
 * a_sites/b_sites: host arrays of n device pointers; chis: host array of
 * n+1 bond dimensions for a (chi_0 = chi_n = 1), chis_b likewise for b.
 * Writes the complex result to *result_host (blocks until done).
 * Replaces MPS.inner_product / MPS.norm (mpsim/core.py:507-565). */
int mps_inner_product(void* stream, const mps_c64* const* a_sites,
                      const int* chis_a, const mps_c64* const* b_sites,
                      const int* chis_b, int n, int d, void* workspace,
                      size_t workspace_bytes, double* result_host);

/* Full state vector psi[x_0 ... x_{n-1}] (qudit 0 most significant) into
 * out_dev (d**n elements).  workspace: 2 * d**n complex64 plus slack.
 * Replaces MPS.wavefunction (mpsim/core.py:483-500). */
int mps_wavefunction(void* stream, const mps_c64* const* sites,
                     const int* chis, int n, int d, mps_c64* out_dev,
                     void* workspace, size_t workspace_bytes);

/* Amplitudes <x|psi> for nbits bitstrings (bits_dev: nbits x n int8,
 * row-major) into out_dev (nbits complex64).  workspace:
 * 2 * nbits * d * max_chi complex64. */
int mps_amplitudes(void* stream, const mps_c64* const* sites, const int* chis,
                   int n, int d, const int8_t* bits_dev, int nbits,
                   mps_c64* out_dev, void* workspace, size_t workspace_bytes);

/* site[i] = alpha * (conj ? conj(site[i]) : site[i]) for count elements.
 * Used by MPS.renormalize (mpsim/core.py:567-594, scale every site by
 * (to/norm)^(1/n)) and MPS.dagger (core.py:502-505, conj every site). */
int mps_scale(void* stream, mps_c64* site, size_t count, float alpha_re,
              float alpha_im, int conj);

/* Strided batched complex GEMM on the device: for z < max(batch, 1),
 *   C[z](i, j) = sum_t opA(i, t) opB(t, j),  0 <= i < m, 0 <= j < n, t < k,
 * with opA(i, t) = a[z*bsa + i*sam + t*sak] (conjugated when conj_a) and
 * likewise b (sbk, sbn, conj_b) and c (scm, scn; overwritten).  The
 * contractions the reference performs with TensorNetwork for the
 * environment sweeps of MPS.reduced_density_matrix (mpsim/core.py:596-653)
 * and for folding S.V^H or U.S into a neighbour after
 * orthonormalize_right_edge_of / orthonormalize_left_edge_of
 * (core.py:884-887, 933-937) use this. */
int mps_cgemm(void* stream, int m, int n, int k, const mps_c64* a, long long sam,
              long long sak, int conj_a, const mps_c64* b, long long sbk,
              long long sbn, int conj_b, mps_c64* c, long long scm, long long scn,
              int batch, long long bsa, long long bsb, long long bsc);

/* mps_cgemm on the tcgen05 tensor cores: same arguments and result, computed
 * as a real GEMM on the complex embedding with every FP32 operand split into
 * three bf16 pieces and the six piece products of order <= 2 accumulated in
 * FP32 in TMEM (as accurate as FP32 arithmetic).  The overlap, wavefunction
 * and reduced-density-matrix sweeps (mpsim/core.py:483-565, 596-653) use it
 * where their contractions are compute-bound. */
int mps_cgemm_tc(void* stream, int m, int n, int k, const mps_c64* a, long long sam,
                 long long sak, int conj_a, const mps_c64* b, long long sbk,
                 long long sbn, int conj_b, mps_c64* c, long long scm, long long scn,
                 int batch, long long bsa, long long bsb, long long bsc);

/* Reads and clears the flag the tensor-core kernels set when one of their
 * bounded mbarrier waits expired (their outputs are then invalid).  Blocks. */
int mps_tc_error(int* flag_out);

/* Profiling counters of the tensor-core Jacobi visits (MPS_PRECISION_MIXED),
 * since the last reset: out10[0..2] = SM cycles summed over visits in the
 * Gram, rotation and Y-update steps, out10[3] = visits, out10[4] = visits
 * that rotated, out10[5] = inner steps that rotated, out10[6] = pairs
 * rotated, out10[7] = cycles visits waited for their blocks' previous round,
 * out10[8] = summed lifetimes of the sweep kernel's CTAs, out10[9] = those
 * CTAs.  Blocks. */
int mps_tc_profile(unsigned long long* out10, int reset);

/* Workspace for mps_site_marginals: every left environment plus two
 * right environments and two (chi, d, chi) scratch tensors. */
size_t mps_marginals_workspace_bytes(const int* chis, int n, int d);

/* The diagonal of every single-site reduced density matrix,
 * probs_host[i*d + x] = <psi| (|x><x| on site i) |psi> (not normalised), in
 * one pass of left environments and one of right environments.  Blocks until
 * done.  Replaces reduced_density_matrix(i).diagonal().real as
 * MPS._sample uses it (mpsim/core.py:655-667, 596-653). */
int mps_site_marginals(void* stream, const mps_c64* const* sites, const int* chis,
                       int n, int d, void* workspace, size_t workspace_bytes,
                       float* probs_host);

#ifdef __cplusplus
}
#endif
#endif /* MPSIM_GB300_H */
