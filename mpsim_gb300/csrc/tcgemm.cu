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
    __align__(16) __nv_bfloat16 p0[8], p1[8], p2[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const tc::Split3 s = tc::split3(v[e]);
        p0[e] = s.p0;
        p1[e] = s.p1;
        p2[e] = s.p2;
    }
    *reinterpret_cast<uint4*>(base + off) = *reinterpret_cast<const uint4*>(p0);
    *reinterpret_cast<uint4*>(base + TC_PIECE + off) = *reinterpret_cast<const uint4*>(p1);
    *reinterpret_cast<uint4*>(base + 2 * TC_PIECE + off) = *reinterpret_cast<const uint4*>(p2);
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

__global__ void __launch_bounds__(TC_THREADS) tc_cgemm_kernel(GemmArgs p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * TC_STAGE);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 2);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int z = blockIdx.z;
    const int i0 = blockIdx.y * TC_BM, j0 = blockIdx.x * TC_BN;
    const cf* a = p.a + (long long)z * p.bsa;
    const cf* b = p.b + (long long)z * p.bsb;
    cf* c = p.c + (long long)z * p.bsc;

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
}

}  // namespace
}  // namespace mps

using namespace mps;

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
