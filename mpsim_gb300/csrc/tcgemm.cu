// Complex GEMM on the tcgen05 tensor cores in split precision.
//
// C[z] = opA(A[z]) opB(B[z]) with arbitrary element strides (the contract of
// mps_cgemm), computed as a real GEMM on the complex embedding
//   Areal[i, (t, c')]       = (Re a_it, Im a_it)                 (K-major)
//   Breal[(j, re), (t, c')] = (Re b_tj, -Im b_tj) = conj(b_tj)
//   Breal[(j, im), (t, c')] = (Im b_tj,  Re b_tj) = i conj(b_tj)
// so that D[i, (j, c)] = sum_(t,c') Areal Breal^T is C interleaved: the 4M
// form of the complex product, 8 m n k real flops.  Every FP32 operand value
// is split into three bf16 pieces in shared memory and D accumulates the six
// piece products of order <= 2 (tc.cuh), which makes the product as accurate
// as FP32 SIMT arithmetic.
//
// Tile: 128 rows of C (M = 128, one TMEM lane each) by 64 complex columns
// (N = 128 real accumulator columns), K in chunks of 32 complex (64 reals:
// one 128-byte swizzle row).  Two shared-memory stages: 128 threads split
// chunk c + 1 while the tensor core multiplies chunk c; one elected thread
// issues the MMAs and commits them to the stage's mbarrier.  The epilogue
// reads TMEM with tcgen05.ld (warp w owns lanes 32w..32w+31) and stores C.
//
// Used by the environment sweeps (overlap / norm, wavefunction, reduced
// density matrices) at bond dimensions where they are compute-bound: the
// contractions of MPS.inner_product / norm (mpsim/core.py:507-565).
#include "tc.cuh"
#include "twoq.cuh"

namespace mps {
namespace {

constexpr int TC_BM = 128;           // rows of C per CTA
constexpr int TC_BN = 64;            // complex columns of C per CTA
constexpr int TC_BK = 32;            // complex K per chunk
constexpr int TC_THREADS = 128;
constexpr uint32_t TC_PIECE = 128u * 128u;            // one 128-row SW128 tile (bytes)
constexpr uint32_t TC_STAGE = 6u * TC_PIECE;          // A pieces + B pieces
constexpr size_t TC_SMEM = 2 * (size_t)TC_STAGE + 1024 + 64;
constexpr uint32_t TC_TMEM_COLS = 128;
constexpr int TC_WAIT_LIMIT = 1 << 14;   // x up to 20 us suspended per poll

__device__ int g_tc_error = 0;

struct GemmArgs {
    int m, n, k;
    const cf* a;
    long long sam, sak;
    int conj_a;
    const cf* b;
    long long sbk, sbn;
    int conj_b;
    cf* c;
    long long scm, scn;
    long long bsa, bsb, bsc;
};

__device__ __forceinline__ void store_split8(uint8_t* base, uint32_t off, const float* v) {
    // v: 8 reals -> 16 bytes per piece at the same offset of three piece tiles
    // (the paired round-to-nearest conversion: the pieces of tc::split3)
    uint32_t w[3][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const __nv_bfloat162 p0 = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
        const float2 f0 = __bfloat1622float2(p0);
        const float ra = v[2 * e] - f0.x, rb = v[2 * e + 1] - f0.y;
        const __nv_bfloat162 p1 = __floats2bfloat162_rn(ra, rb);
        const float2 f1 = __bfloat1622float2(p1);
        const __nv_bfloat162 p2 = __floats2bfloat162_rn(ra - f1.x, rb - f1.y);
        w[0][e] = *reinterpret_cast<const uint32_t*>(&p0);
        w[1][e] = *reinterpret_cast<const uint32_t*>(&p1);
        w[2][e] = *reinterpret_cast<const uint32_t*>(&p2);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
        *reinterpret_cast<uint4*>(base + i * TC_PIECE + off) =
            make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

// Fills one stage with K chunk kc: A rows i0..i0+127, B columns j0..j0+63.
__device__ __forceinline__ void fill_stage(uint8_t* st, const GemmArgs& p, const cf* a,
                                           const cf* b, int i0, int j0, int kc) {
    const int tid = threadIdx.x;
    const int t0 = kc * TC_BK;
    // A: thread tid owns row tid; 8 groups of 4 complex along K.
    {
        const int i = i0 + tid;
#pragma unroll 2
        for (int grp = 0; grp < 8; ++grp) {
            float v[8];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int t = t0 + grp * 4 + e;
                cf x = cmake(0.f, 0.f);
                if (i < p.m && t < p.k) x = a[(long long)i * p.sam + (long long)t * p.sak];
                if (p.conj_a) x.y = -x.y;
                v[2 * e] = x.x;
                v[2 * e + 1] = x.y;
            }
            store_split8(st, tc::sw128_off(tid, grp * 8), v);
        }
    }
    // B: 64 columns x 8 groups = 512 items, 4 per thread (column fastest).
    uint8_t* sb = st + 3 * TC_PIECE;
#pragma unroll 1
    for (int it = 0; it < 4; ++it) {
        const int g = tid + TC_THREADS * it;
        const int jl = g & 63, grp = g >> 6;
        const int j = j0 + jl;
        float vr[8], vi[8];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int t = t0 + grp * 4 + e;
            cf x = cmake(0.f, 0.f);
            if (j < p.n && t < p.k) x = b[(long long)t * p.sbk + (long long)j * p.sbn];
            if (p.conj_b) x.y = -x.y;
            vr[2 * e] = x.x;       // row (j, re): conj(b)
            vr[2 * e + 1] = -x.y;
            vi[2 * e] = x.y;       // row (j, im): i conj(b)
            vi[2 * e + 1] = x.x;
        }
        store_split8(sb, tc::sw128_off(2 * jl, grp * 8), vr);
        store_split8(sb, tc::sw128_off(2 * jl + 1, grp * 8), vi);
    }
}

// One 128 x 64 tile of C = opA(A) opB(B) (rows i0.., columns j0..) for the
// operands at a, b, c.  All 128 threads call it; returns false when a
// bounded MMA wait expired (the tile is then not written).
__device__ __forceinline__ bool cgemm_tile(const GemmArgs& p, const cf* a, const cf* b, cf* c,
                                           int i0, int j0) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * TC_STAGE);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, TC_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    constexpr uint32_t IDESC = tc::idesc_bf16(128, 128, false, false);
    const int nchunks = (p.k + TC_BK - 1) / TC_BK;
    bool ok = true;
    for (int kc = 0; kc < nchunks; ++kc) {
        const int s = kc & 1;
        uint8_t* st = smem + s * TC_STAGE;
        if (kc >= 2) {
            const bool w = tc::mbar_wait_bounded(&bar[s], ((kc - 2) >> 1) & 1, TC_WAIT_LIMIT);
            ok = __syncthreads_and(w) != 0;
            if (!ok) break;
        }
        fill_stage(st, p, a, b, i0, j0, kc);
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t sa = tc::smem_u32(st), sbase = sa + 3 * TC_PIECE;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                // piece products of order <= 2, smallest first
                const int pa[6] = {2, 1, 0, 1, 0, 0};
                const int pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const uint64_t ad = tc::sdesc(sa + pa[q] * TC_PIECE + ks * 32, 16, 1024);
                    const uint64_t bd = tc::sdesc(sbase + pb[q] * TC_PIECE + ks * 32, 16, 1024);
                    tc::mma_bf16(tmem, ad, bd, IDESC, (kc | ks | q) != 0);
                }
            }
            tc::mma_commit(&bar[s]);
        }
    }
    if (ok && nchunks > 0) {
        const bool w = tc::mbar_wait_bounded(&bar[(nchunks - 1) & 1], ((nchunks - 1) >> 1) & 1,
                                             TC_WAIT_LIMIT);
        ok = __syncthreads_and(w) != 0;
    }
    tc::fence_after_sync();

    if (!ok) {
        if (lane == 0) atomicExch(&g_tc_error, 1);
    } else {
        const int i = i0 + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int cc = 0; cc < 4; ++cc) {
            float v[32];
            if (nchunks > 0) {
                tc::tmem_ld32(trow + cc * 32, v);
            } else {
#pragma unroll
                for (int e = 0; e < 32; ++e) v[e] = 0.f;
            }
            if (i < p.m) {
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const int j = j0 + cc * 16 + e;
                    if (j < p.n) c[(long long)i * p.scm + (long long)j * p.scn] = cmake(v[2 * e], v[2 * e + 1]);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
    return ok;
}

__global__ void __launch_bounds__(TC_THREADS) tc_cgemm_kernel(GemmArgs p) {
    const int z = blockIdx.z;
    (void)cgemm_tile(p, p.a + (long long)z * p.bsa, p.b + (long long)z * p.bsb,
                     p.c + (long long)z * p.bsc, blockIdx.y * TC_BM, blockIdx.x * TC_BN);
}

// The two-site merge of the mixed form's tensor-core jobs (tc_job, theta not
// given): M = A B per job, A = (chi_l d) x chi_m row-major, B = chi_m x
// (d chi_r) row-major, written column-major into the job's Jacobi matrix X
// (leading dimension lslot); merge_gate_tc_kernel then mixes M with the gate
// in place.  Grid: (column tiles, row tiles, jobs) of the largest job.
__global__ void __launch_bounds__(TC_THREADS)
merge_tc_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g) {
    const mps_2q_job job = jobs[blockIdx.z];
    const int d = g.d;
    const int m = job.chi_l * d, n = d * job.chi_r;
    if (!merge_on_tensor_cores(job, d)) return;
    const int i0 = blockIdx.y * TC_BM, j0 = blockIdx.x * TC_BN;
    if (i0 >= m || j0 >= n) return;
    GemmArgs p;
    p.m = m; p.n = n; p.k = job.chi_m;
    p.a = reinterpret_cast<const cf*>(job.a); p.sam = job.chi_m; p.sak = 1; p.conj_a = 0;
    p.b = reinterpret_cast<const cf*>(job.b); p.sbk = n; p.sbn = 1; p.conj_b = 0;
    cf* X = g.X + (size_t)blockIdx.z * g.lslot * g.cslot;
    p.c = X; p.scm = 1; p.scn = g.lslot;
    p.bsa = p.bsb = p.bsc = 0;
    if (!cgemm_tile(p, p.a, p.b, X, i0, j0) && threadIdx.x == 0) atomicOr(g.counter + 3, 1);
}

// theta[(l,a'),(b',r)] = sum_{a,b} G[(a'b'),(ab)] M[(l,a),(b,r)] in place in
// X for the jobs merge_tc_kernel took, and its copy in T (their right factor
// comes from U^H theta).  One thread per (job, l, r).
template <int D>
__device__ __forceinline__ void gate_block(cf* X, cf* T, const cf* G, int l, int r, int chir,
                                           int lslot) {
    cf mloc[D * D];
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
        for (int b = 0; b < D; ++b) mloc[a * D + b] = X[(size_t)(b * chir + r) * lslot + (l * D + a)];
#pragma unroll
    for (int ap = 0; ap < D; ++ap)
#pragma unroll
        for (int bp = 0; bp < D; ++bp) {
            const cf* grow = G + (size_t)(ap * D + bp) * D * D;
            cf th = cmake(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < D * D; ++q)
                cfma(th, __ldg(reinterpret_cast<const float2*>(grow + q)), mloc[q]);
            const size_t off = (size_t)(bp * chir + r) * lslot + (l * D + ap);
            X[off] = th;
            T[off] = th;
        }
}

__global__ void __launch_bounds__(256)
merge_gate_tc_kernel(const mps_2q_job* __restrict__ jobs, TwoQGeom g, int max_lr) {
    const mps_2q_job job = jobs[blockIdx.y];
    const int d = g.d;
    if (!merge_on_tensor_cores(job, d)) return;
    const int chil = job.chi_l, chir = job.chi_r;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= max_lr || e >= chil * chir) return;
    const int l = e / chir, r = e - (e / chir) * chir;
    cf* X = g.X + (size_t)blockIdx.y * g.lslot * g.cslot;
    cf* T = g.T + (size_t)blockIdx.y * g.lslot * g.cslot;
    const cf* G = reinterpret_cast<const cf*>(job.gate);
    if (d == 2) gate_block<2>(X, T, G, l, r, chir, g.lslot);
    else if (d == 3) gate_block<3>(X, T, G, l, r, chir, g.lslot);
    else gate_block<4>(X, T, G, l, r, chir, g.lslot);
}

}  // namespace
}  // namespace mps

using namespace mps;

namespace mps {

int merge_tc_launch(const mps_2q_job* jobs, int njobs, int max_m, int max_n, const TwoQGeom& g,
                    cudaStream_t s) {
    if (njobs <= 0 || g.d > 4) return MPS_OK;   // (the SIMT merge takes d > 4)
    static KernelSetup ks;
    int dev = 0;
    MPS_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(MPS_ERR_ARG, "device index beyond 63");
    std::call_once(ks.once[dev], [&] {
        cudaError_t e = cudaFuncSetAttribute(merge_tc_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)TC_SMEM);
        ks.rc[dev] = e == cudaSuccess ? MPS_OK : cuda_fail(e, "cudaFuncSetAttribute(merge_tc_kernel)");
    });
    if (ks.rc[dev] != MPS_OK) return ks.rc[dev];
    dim3 grid((max_n + TC_BN - 1) / TC_BN, (max_m + TC_BM - 1) / TC_BM, njobs);
    merge_tc_kernel<<<grid, TC_THREADS, TC_SMEM, s>>>(jobs, g);
    MPS_LAUNCH_CHECK("merge_tc_kernel");
    const int max_lr = (max_m / g.d) * (max_n / g.d);
    dim3 gg((max_lr + 255) / 256, njobs);
    merge_gate_tc_kernel<<<gg, 256, 0, s>>>(jobs, g, max_lr);
    MPS_LAUNCH_CHECK("merge_gate_tc_kernel");
    return MPS_OK;
}

}  // namespace mps

extern "C" int mps_cgemm_tc(void* stream, int m, int n, int k, const mps_c64* a, long long sam,
                            long long sak, int conj_a, const mps_c64* b, long long sbk,
                            long long sbn, int conj_b, mps_c64* c, long long scm, long long scn,
                            int batch, long long bsa, long long bsb, long long bsc) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (m < 0 || n < 0 || k < 0 || batch < 0)
        return fail(MPS_ERR_ARG, "mps_cgemm_tc: negative size");
    if (m == 0 || n == 0) return MPS_OK;
    if (!a || !b || !c) return fail(MPS_ERR_ARG, "mps_cgemm_tc: null pointer");
    const int nb = batch < 1 ? 1 : batch;
    if (nb > 65535 || (m + TC_BM - 1) / TC_BM > 65535)
        return fail(MPS_ERR_ARG, "mps_cgemm_tc: grid too large");
    // the shared-memory opt-in is a per-device attribute: set it on every
    // device this process uses (setting it twice is harmless)
    static bool configured[64] = {};
    int dev = 0;
    MPS_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(MPS_ERR_ARG, "mps_cgemm_tc: device index beyond 63");
    if (!configured[dev]) {
        MPS_CUDA_CHECK(cudaFuncSetAttribute(tc_cgemm_kernel,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)TC_SMEM));
        configured[dev] = true;
    }
    GemmArgs p;
    p.m = m; p.n = n; p.k = k;
    p.a = reinterpret_cast<const cf*>(a); p.sam = sam; p.sak = sak; p.conj_a = conj_a;
    p.b = reinterpret_cast<const cf*>(b); p.sbk = sbk; p.sbn = sbn; p.conj_b = conj_b;
    p.c = reinterpret_cast<cf*>(c); p.scm = scm; p.scn = scn;
    p.bsa = bsa; p.bsb = bsb; p.bsc = bsc;
    dim3 grid((n + TC_BN - 1) / TC_BN, (m + TC_BM - 1) / TC_BM, nb);
    tc_cgemm_kernel<<<grid, TC_THREADS, TC_SMEM, s>>>(p);
    MPS_LAUNCH_CHECK("tc_cgemm_kernel");
    return MPS_OK;
}

// Reads and clears the tensor-core kernels' wait-expiry flag (blocks).
extern "C" int mps_tc_error(int* flag_out) {
    int v = 0, zero = 0;
    MPS_CUDA_CHECK(cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int)));
    MPS_CUDA_CHECK(cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int)));
    if (flag_out) *flag_out = v;
    return MPS_OK;
}
