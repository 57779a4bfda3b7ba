// One-qudit gate, left-to-right contraction sweeps (overlap/norm,
// wavefunction, sampled amplitudes, single-site marginals), a strided batched
// complex GEMM and elementwise scale/conjugate.
//
// mpsim performs these with TensorNetwork contractions on the host:
//   apply_one_qudit_gate   mpsim/core.py:820-826
//   wavefunction           mpsim/core.py:483-500
//   inner_product / norm   mpsim/core.py:543-565
//   renormalize / dagger   mpsim/core.py:567-594, 502-505
//   marginals for sample   mpsim/core.py:655-667 (reduced_density_matrix(i)
//                          diagonal, core.py:596-653)
#include <atomic>
#include <string>

#include "common.cuh"

namespace mps {

thread_local std::string t_error;
static std::atomic<unsigned long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const std::string& msg) { t_error = msg; }

int fail(int code, const std::string& msg) {
    t_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    t_error = std::string(what) + ": " + cudaGetErrorString(e);
    return MPS_ERR_CUDA;
}

namespace {

// ---------------------------------------------------------------------------
// One-qudit gate: one thread per (l, r); consecutive threads take consecutive
// r, so every load/store of a (l, a, :) row is coalesced.  HBM-bound:
// 2 * chi_l * d * chi_r * 8 bytes per call.
template <int DMAX>
__global__ void apply_1q_kernel(cf* __restrict__ site, int chil, int d, int chir,
                                const cf* __restrict__ gate) {
    __shared__ cf U[DMAX * DMAX];
    for (int e = threadIdx.x; e < d * d; e += blockDim.x) U[e] = gate[e];
    __syncthreads();
    const size_t total = (size_t)chil * chir;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t l = t / chir, r = t % chir;
        cf* base = site + l * d * chir + r;
        cf v[DMAX];
#pragma unroll
        for (int a = 0; a < DMAX; ++a)
            if (a < d) v[a] = base[(size_t)a * chir];
#pragma unroll
        for (int ap = 0; ap < DMAX; ++ap) {
            if (ap < d) {
                cf acc = cmake(0.f, 0.f);
#pragma unroll
                for (int a = 0; a < DMAX; ++a)
                    if (a < d) cfma(acc, U[ap * d + a], v[a]);
                base[(size_t)ap * chir] = acc;
            }
        }
    }
}

// Batched one-qudit gates: blockIdx.y selects the (site, gate) job.  A job
// whose chi_r is even and whose site is 16-byte aligned (every torch
// allocation is) runs the vectorised form: each thread owns two adjacent r
// and moves them as one 16-byte load and store per a; the 128 threads of a
// CTA form rows of rpw = next power of two of (chi_r / 2), capped at 128,
// lanes, so (l, r) comes from shifts and masks, never from an integer divide.
// Other jobs take the scalar form (one thread per (l, r)).
constexpr int ONEQ_T = 128;

template <int DMAX>
__global__ void __launch_bounds__(ONEQ_T) apply_1q_batch_kernel(const mps_1q_job* __restrict__ jobs,
                                                                int d) {
    __shared__ cf U[DMAX * DMAX];
    const mps_1q_job job = jobs[blockIdx.y];
    const cf* gate = reinterpret_cast<const cf*>(job.gate);
    for (int e = threadIdx.x; e < d * d; e += blockDim.x) U[e] = gate[e];
    __syncthreads();
    const int chil = job.chi_l, chir = job.chi_r;
    cf* site = reinterpret_cast<cf*>(job.site);
    if ((chir & 1) == 0 && (reinterpret_cast<uintptr_t>(site) & 15) == 0) {
        const int rp = chir >> 1;                       // r pairs per row
        int sh = 0;
        while ((1 << sh) < rp && sh < 7) ++sh;          // rpw = 2^sh lanes per row
        const int rows = ONEQ_T >> sh;                  // rows per pass of the CTA
        const int ly = threadIdx.x >> sh, qx = threadIdx.x & ((1 << sh) - 1);
        const size_t rs = (size_t)d * chir;             // complex per l row
        const int step = gridDim.x * rows;
        // two rows per iteration, every load issued before any arithmetic:
        // 2 d 16-byte loads in flight per thread (the kernel is bound by
        // load latency, not by instructions)
        for (int l = blockIdx.x * rows + ly; l < chil; l += 2 * step) {
            const int l2 = l + step;
            const bool two = l2 < chil;
            float4* row = reinterpret_cast<float4*>(site + (size_t)l * rs);
            float4* row2 = reinterpret_cast<float4*>(site + (size_t)(two ? l2 : l) * rs);
            for (int q = qx; q < rp; q += 1 << sh) {
                float4 v[DMAX], w[DMAX];
#pragma unroll
                for (int a = 0; a < DMAX; ++a) {
                    if (a < d) {
                        v[a] = __ldcs(row + (size_t)a * rp + q);
                        if (two) w[a] = __ldcs(row2 + (size_t)a * rp + q);
                    }
                }
#pragma unroll
                for (int ap = 0; ap < DMAX; ++ap) {
                    if (ap < d) {
                        cf a0 = cmake(0.f, 0.f), a1 = cmake(0.f, 0.f);
                        cf b0 = cmake(0.f, 0.f), b1 = cmake(0.f, 0.f);
#pragma unroll
                        for (int a = 0; a < DMAX; ++a) {
                            if (a < d) {
                                const cf u = U[ap * d + a];
                                cfma(a0, u, cmake(v[a].x, v[a].y));
                                cfma(a1, u, cmake(v[a].z, v[a].w));
                                if (two) {
                                    cfma(b0, u, cmake(w[a].x, w[a].y));
                                    cfma(b1, u, cmake(w[a].z, w[a].w));
                                }
                            }
                        }
                        __stcs(row + (size_t)ap * rp + q, make_float4(a0.x, a0.y, a1.x, a1.y));
                        if (two) __stcs(row2 + (size_t)ap * rp + q, make_float4(b0.x, b0.y, b1.x, b1.y));
                    }
                }
            }
        }
        return;
    }
    const size_t total = (size_t)chil * chir;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t l = t / chir, r = t % chir;
        cf* base = site + l * d * chir + r;
        cf v[DMAX];
#pragma unroll
        for (int a = 0; a < DMAX; ++a)
            if (a < d) v[a] = base[(size_t)a * chir];
#pragma unroll
        for (int ap = 0; ap < DMAX; ++ap) {
            if (ap < d) {
                cf acc = cmake(0.f, 0.f);
#pragma unroll
                for (int a = 0; a < DMAX; ++a)
                    if (a < d) cfma(acc, U[ap * d + a], v[a]);
                base[(size_t)ap * chir] = acc;
            }
        }
    }
}

__global__ void scale_kernel(cf* __restrict__ x, size_t count, cf alpha, int conj) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
         t += (size_t)gridDim.x * blockDim.x) {
        cf v = x[t];
        if (conj) v = cconj(v);
        x[t] = cmul(alpha, v);
    }
}

// ---------------------------------------------------------------------------
// Generic complex GEMM C = op(A) op(B) with arbitrary element strides and
// optional conjugation, batched over blockIdx.z with element strides bsa,
// bsb, bsc between batches (zero: the same matrix for every batch).  64x64
// tile, K chunks of 16, 256 threads, each thread 4x4 outputs at
// (ty + 16i, tx + 16j).
struct GemmArgs {
    int M, N, K;
    const cf* A;
    long long sam, sak;
    int conjA;
    const cf* B;
    long long sbk, sbn;
    int conjB;
    cf* C;
    long long scm, scn;
    int batch;                  // 0 or 1: one product
    long long bsa, bsb, bsc;
};

__global__ void __launch_bounds__(256) cgemm_kernel(GemmArgs g) {
    __shared__ cf As[16][64];
    __shared__ cf Bs[16][64];
    g.A += blockIdx.z * g.bsa;
    g.B += blockIdx.z * g.bsb;
    g.C += blockIdx.z * g.bsc;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    cf acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cmake(0.f, 0.f);
    const bool a_kfast = g.sak == 1;
    const bool b_nfast = g.sbn == 1;
    for (int k0 = 0; k0 < g.K; k0 += 16) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int idx = tid + q * 256;
            int kk, tr;
            if (a_kfast) { kk = idx & 15; tr = idx >> 4; } else { tr = idx & 63; kk = idx >> 6; }
            const int row = m0 + tr, k = k0 + kk;
            cf v = cmake(0.f, 0.f);
            if (row < g.M && k < g.K) {
                v = g.A[row * g.sam + k * g.sak];
                if (g.conjA) v = cconj(v);
            }
            As[kk][tr] = v;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int idx = tid + q * 256;
            int kk, tc;
            if (b_nfast) { tc = idx & 63; kk = idx >> 6; } else { kk = idx & 15; tc = idx >> 4; }
            const int col = n0 + tc, k = k0 + kk;
            cf v = cmake(0.f, 0.f);
            if (col < g.N && k < g.K) {
                v = g.B[k * g.sbk + col * g.sbn];
                if (g.conjB) v = cconj(v);
            }
            Bs[kk][tc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            cf av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
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
        for (int j = 0; j < 4; ++j) {
            const int row = m0 + ty + 16 * i, col = n0 + tx + 16 * j;
            if (row < g.M && col < g.N) g.C[row * g.scm + col * g.scn] = acc[i][j];
        }
}

int cgemm(const GemmArgs& a, cudaStream_t s) {
    if (a.M <= 0 || a.N <= 0 || a.batch < 0) return MPS_OK;
    dim3 grid((a.N + 63) / 64, (a.M + 63) / 64, a.batch > 1 ? a.batch : 1);
    if (grid.y > 65535) return fail(MPS_ERR_ARG, "cgemm: too many rows");
    if (grid.z > 65535) return fail(MPS_ERR_ARG, "cgemm: batch above 65535");
    cgemm_kernel<<<grid, 256, 0, s>>>(a);
    MPS_LAUNCH_CHECK("cgemm_kernel");
    return MPS_OK;
}

// env'[s, r] = full[s, x_s * chir + r]
__global__ void select_kernel(const cf* __restrict__ full, cf* __restrict__ env, int nbits,
                              int chir, int d, const int8_t* __restrict__ bits, int n, int site) {
    const size_t total = (size_t)nbits * chir;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t sidx = t / chir, r = t % chir;
        const int x = bits[sidx * n + site];
        env[t] = (x >= 0 && x < d) ? full[sidx * (size_t)d * chir + (size_t)x * chir + r]
                                   : cmake(0.f, 0.f);
    }
}

// probs[x] = Re sum_{l, r} conj(A[l, x, r]) W[l, x, r]: block x, FP64 sum.
__global__ void __launch_bounds__(256) marginal_kernel(const cf* __restrict__ A,
                                                       const cf* __restrict__ W, int chil,
                                                       int d, int chir, float* __restrict__ probs) {
    __shared__ double part[256];
    const int x = blockIdx.x;
    const size_t total = (size_t)chil * chir;
    double acc = 0.0;
    for (size_t t = threadIdx.x; t < total; t += blockDim.x) {
        const size_t l = t / chir, r = t % chir;
        const size_t o = (l * d + x) * chir + r;
        const cf a = A[o], w = W[o];
        acc += (double)a.x * w.x + (double)a.y * w.y;
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) probs[x] = (float)part[0];
}

__global__ void fill_one_kernel(cf* x, size_t count) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
         t += (size_t)gridDim.x * blockDim.x)
        x[t] = cmake(1.f, 0.f);
}

int grid_for(size_t total) {
    size_t b = (total + 255) / 256;
    if (b < 1) b = 1;
    if (b > 8192) b = 8192;
    return (int)b;
}

}  // namespace
}  // namespace mps

using namespace mps;

extern "C" int mps_version(void) { return 100; }

extern "C" const char* mps_last_error(void) { return t_error.c_str(); }

extern "C" unsigned long long mps_kernel_launches(void) { return g_launches.load(); }

extern "C" int mps_apply_1q(void* stream, mps_c64* site, int chi_l, int d, int chi_r,
                            const mps_c64* gate) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (chi_l < 0 || chi_r < 0 || d < 1 || d > 64) return fail(MPS_ERR_ARG, "mps_apply_1q: bad shape");
    const size_t total = (size_t)chi_l * chi_r;
    if (total == 0) return MPS_OK;
    if (!site || !gate) return fail(MPS_ERR_ARG, "mps_apply_1q: null pointer");
    cf* x = reinterpret_cast<cf*>(site);
    const cf* u = reinterpret_cast<const cf*>(gate);
    const int blocks = grid_for(total);
    if (d <= 2) apply_1q_kernel<2><<<blocks, 256, 0, s>>>(x, chi_l, d, chi_r, u);
    else if (d <= 4) apply_1q_kernel<4><<<blocks, 256, 0, s>>>(x, chi_l, d, chi_r, u);
    else if (d <= 8) apply_1q_kernel<8><<<blocks, 256, 0, s>>>(x, chi_l, d, chi_r, u);
    else if (d <= 16) apply_1q_kernel<16><<<blocks, 256, 0, s>>>(x, chi_l, d, chi_r, u);
    else apply_1q_kernel<64><<<blocks, 256, 0, s>>>(x, chi_l, d, chi_r, u);
    MPS_LAUNCH_CHECK("apply_1q_kernel");
    return MPS_OK;
}

extern "C" int mps_apply_1q_batch(void* stream, const mps_1q_job* jobs, int njobs, int d) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (njobs == 0) return MPS_OK;
    if (njobs < 0 || njobs > 65535 || !jobs) return fail(MPS_ERR_ARG, "mps_apply_1q_batch: bad job list");
    if (d < 1 || d > 64) return fail(MPS_ERR_ARG, "mps_apply_1q_batch: bad qudit dimension");
    // 16 CTAs per job, two rows per thread per iteration: a 64-site chi=256
    // layer is 1024 CTAs of 128 threads, ~27 warps and ~55 KB of loads in
    // flight per SM
    dim3 grid(16, njobs);
    if (d <= 2) apply_1q_batch_kernel<2><<<grid, ONEQ_T, 0, s>>>(jobs, d);
    else if (d <= 4) apply_1q_batch_kernel<4><<<grid, ONEQ_T, 0, s>>>(jobs, d);
    else if (d <= 8) apply_1q_batch_kernel<8><<<grid, ONEQ_T, 0, s>>>(jobs, d);
    else if (d <= 16) apply_1q_batch_kernel<16><<<grid, ONEQ_T, 0, s>>>(jobs, d);
    else apply_1q_batch_kernel<64><<<grid, ONEQ_T, 0, s>>>(jobs, d);
    MPS_LAUNCH_CHECK("apply_1q_batch_kernel");
    return MPS_OK;
}

extern "C" int mps_scale(void* stream, mps_c64* site, size_t count, float alpha_re,
                         float alpha_im, int conj) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (count == 0) return MPS_OK;
    if (!site) return fail(MPS_ERR_ARG, "mps_scale: null pointer");
    scale_kernel<<<grid_for(count), 256, 0, s>>>(reinterpret_cast<cf*>(site), count,
                                                 cmake(alpha_re, alpha_im), conj);
    MPS_LAUNCH_CHECK("scale_kernel");
    return MPS_OK;
}

extern "C" size_t mps_sweep_workspace_bytes(int max_chi, int d) {
    if (max_chi < 1) max_chi = 1;
    const size_t c = (size_t)max_chi;
    return align_up((2 * c * c + (size_t)d * c * c) * sizeof(cf) + 1024, 256);
}

extern "C" int mps_inner_product(void* stream, const mps_c64* const* a_sites, const int* chis_a,
                                 const mps_c64* const* b_sites, const int* chis_b, int n, int d,
                                 void* workspace, size_t workspace_bytes, double* result_host) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n < 1 || d < 1 || !a_sites || !b_sites || !chis_a || !chis_b || !result_host)
        return fail(MPS_ERR_ARG, "mps_inner_product: bad arguments");
    if (chis_a[0] != 1 || chis_b[0] != 1 || chis_a[n] != 1 || chis_b[n] != 1)
        return fail(MPS_ERR_ARG, "mps_inner_product: end bonds must be 1");
    int maxchi = 1;
    for (int i = 0; i <= n; ++i) maxchi = max(maxchi, max(chis_a[i], chis_b[i]));
    if (workspace_bytes < mps_sweep_workspace_bytes(maxchi, d) || !workspace)
        return fail(MPS_ERR_WORKSPACE, "mps_inner_product: workspace too small");
    const size_t cc = (size_t)maxchi * maxchi;
    cf* E0 = static_cast<cf*>(workspace);
    cf* E1 = E0 + cc;
    cf* T = E1 + cc;
    fill_one_kernel<<<1, 32, 0, s>>>(E0, 1);
    MPS_LAUNCH_CHECK("fill_one_kernel");
    for (int i = 0; i < n; ++i) {
        const int al = chis_a[i], ar = chis_a[i + 1], bl = chis_b[i], br = chis_b[i + 1];
        const cf* A = reinterpret_cast<const cf*>(a_sites[i]);
        const cf* B = reinterpret_cast<const cf*>(b_sites[i]);
        // T[l, (x, r')] = sum_l' E[l, l'] conj(B[l', x, r'])
        GemmArgs g1{al, d * br, bl, E0, bl, 1, 0, B, (long long)d * br, 1, 1, T, (long long)d * br, 1};
        int rc = cgemm(g1, s);
        if (rc) return rc;
        // E'[r, r'] = sum_(l,x) A[(l,x), r] T[(l,x), r']
        GemmArgs g2{ar, br, al * d, A, 1, ar, 0, T, br, 1, 0, E1, br, 1};
        if (ar > 0 && br > 0 && al * d == 0) {
            MPS_CUDA_CHECK(cudaMemsetAsync(E1, 0, (size_t)ar * br * sizeof(cf), s));
        } else {
            rc = cgemm(g2, s);
            if (rc) return rc;
        }
        cf* t = E0; E0 = E1; E1 = t;
    }
    float2 res;
    MPS_CUDA_CHECK(cudaMemcpyAsync(&res, E0, sizeof(float2), cudaMemcpyDeviceToHost, s));
    MPS_CUDA_CHECK(cudaStreamSynchronize(s));
    result_host[0] = res.x;
    result_host[1] = res.y;
    return MPS_OK;
}

extern "C" int mps_wavefunction(void* stream, const mps_c64* const* sites, const int* chis,
                                int n, int d, mps_c64* out_dev, void* workspace,
                                size_t workspace_bytes) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n < 1 || d < 1 || !sites || !chis || !out_dev)
        return fail(MPS_ERR_ARG, "mps_wavefunction: bad arguments");
    size_t need = 1, p = 1;
    for (int i = 0; i < n; ++i) {
        p *= (size_t)d;
        need = max(need, p * (size_t)max(chis[i + 1], 1));
    }
    if (!workspace || workspace_bytes < 2 * need * sizeof(cf))
        return fail(MPS_ERR_WORKSPACE, "mps_wavefunction: workspace too small");
    cf* buf[2] = {static_cast<cf*>(workspace), static_cast<cf*>(workspace) + need};
    fill_one_kernel<<<1, 32, 0, s>>>(buf[0], 1);
    MPS_LAUNCH_CHECK("fill_one_kernel");
    size_t P = 1;
    int cur = 0;
    for (int i = 0; i < n; ++i) {
        const int cl = chis[i], cr = chis[i + 1];
        cf* dst = (i == n - 1) ? reinterpret_cast<cf*>(out_dev) : buf[cur ^ 1];
        const size_t rows = P;
        if (rows > 0x7fffffff) return fail(MPS_ERR_ARG, "mps_wavefunction: state too large");
        if (cl == 0) {
            MPS_CUDA_CHECK(cudaMemsetAsync(dst, 0, rows * d * cr * sizeof(cf), s));
        } else {
            GemmArgs g{(int)rows, d * cr, cl, buf[cur], cl, 1, 0,
                       reinterpret_cast<const cf*>(sites[i]), (long long)d * cr, 1, 0,
                       dst, (long long)d * cr, 1};
            // cgemm tiles rows in grid.y (<= 65535 * 64 rows); split larger ones
            const long long chunk = 65535LL * 64;
            for (long long r0 = 0; r0 < (long long)rows; r0 += chunk) {
                GemmArgs gc = g;
                gc.M = (int)(((long long)rows - r0) < chunk ? ((long long)rows - r0) : chunk);
                gc.A = buf[cur] + r0 * cl;
                gc.C = dst + r0 * (long long)d * cr;
                int rc = cgemm(gc, s);
                if (rc) return rc;
            }
        }
        P = rows * d;
        cur ^= 1;
    }
    return MPS_OK;
}

extern "C" int mps_amplitudes(void* stream, const mps_c64* const* sites, const int* chis, int n,
                              int d, const int8_t* bits_dev, int nbits, mps_c64* out_dev,
                              void* workspace, size_t workspace_bytes) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n < 1 || d < 1 || nbits < 0 || !sites || !chis || (nbits > 0 && (!bits_dev || !out_dev)))
        return fail(MPS_ERR_ARG, "mps_amplitudes: bad arguments");
    if (nbits == 0) return MPS_OK;
    int maxchi = 1;
    for (int i = 0; i <= n; ++i) maxchi = max(maxchi, chis[i]);
    const size_t full_sz = (size_t)nbits * d * maxchi, env_sz = (size_t)nbits * maxchi;
    if (!workspace || workspace_bytes < (full_sz + 2 * env_sz) * sizeof(cf))
        return fail(MPS_ERR_WORKSPACE, "mps_amplitudes: workspace too small");
    cf* full = static_cast<cf*>(workspace);
    cf* env[2] = {full + full_sz, full + full_sz + env_sz};
    fill_one_kernel<<<grid_for(nbits), 256, 0, s>>>(env[0], nbits);
    MPS_LAUNCH_CHECK("fill_one_kernel");
    int cur = 0;
    for (int i = 0; i < n; ++i) {
        const int cl = chis[i], cr = chis[i + 1];
        cf* dst = (i == n - 1) ? reinterpret_cast<cf*>(out_dev) : env[cur ^ 1];
        if (cl == 0) {
            MPS_CUDA_CHECK(cudaMemsetAsync(full, 0, (size_t)nbits * d * cr * sizeof(cf), s));
        } else {
            GemmArgs g{nbits, d * cr, cl, env[cur], cl, 1, 0, reinterpret_cast<const cf*>(sites[i]),
                       (long long)d * cr, 1, 0, full, (long long)d * cr, 1};
            int rc = cgemm(g, s);
            if (rc) return rc;
        }
        select_kernel<<<grid_for((size_t)nbits * cr), 256, 0, s>>>(full, dst, nbits, cr, d,
                                                                    bits_dev, n, i);
        MPS_LAUNCH_CHECK("select_kernel");
        cur ^= 1;
    }
    return MPS_OK;
}

extern "C" int mps_cgemm(void* stream, int m, int n, int k, const mps_c64* a, long long sam,
                         long long sak, int conj_a, const mps_c64* b, long long sbk,
                         long long sbn, int conj_b, mps_c64* c, long long scm, long long scn,
                         int batch, long long bsa, long long bsb, long long bsc) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (m < 0 || n < 0 || k < 0 || batch < 0 || (m > 0 && n > 0 && (!c || (k > 0 && (!a || !b)))))
        return fail(MPS_ERR_ARG, "mps_cgemm: bad arguments");
    GemmArgs g{m, n, k, reinterpret_cast<const cf*>(a), sam, sak, conj_a ? 1 : 0,
               reinterpret_cast<const cf*>(b), sbk, sbn, conj_b ? 1 : 0,
               reinterpret_cast<cf*>(c), scm, scn, batch, bsa, bsb, bsc};
    return cgemm(g, s);
}

extern "C" size_t mps_marginals_workspace_bytes(const int* chis, int n, int d) {
    if (!chis || n < 1 || d < 1) return 0;
    size_t envs = 0, maxchi = 1;
    for (int i = 0; i < n; ++i) envs += (size_t)chis[i] * chis[i];
    for (int i = 0; i <= n; ++i) maxchi = max(maxchi, (size_t)chis[i]);
    const size_t cells = envs + 2 * maxchi * maxchi + 2 * maxchi * d * maxchi;
    return align_up(cells * sizeof(cf) + (size_t)n * d * sizeof(float) + 1024, 256);
}

extern "C" int mps_site_marginals(void* stream, const mps_c64* const* sites, const int* chis,
                                  int n, int d, void* workspace, size_t workspace_bytes,
                                  float* probs_host) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n < 1 || d < 1 || !sites || !chis || !probs_host)
        return fail(MPS_ERR_ARG, "mps_site_marginals: bad arguments");
    if (chis[0] != 1 || chis[n] != 1) return fail(MPS_ERR_ARG, "mps_site_marginals: end bonds must be 1");
    if (!workspace || workspace_bytes < mps_marginals_workspace_bytes(chis, n, d))
        return fail(MPS_ERR_WORKSPACE, "mps_site_marginals: workspace too small");
    size_t maxchi = 1;
    for (int i = 0; i <= n; ++i) maxchi = max(maxchi, (size_t)chis[i]);
    // left environments L_i (ket, bra), i = 0..n-1, packed
    cf* base = static_cast<cf*>(workspace);
    size_t off = 0;
    cf* R[2];
    cf* U;
    cf* W;
    {
        size_t envs = 0;
        for (int i = 0; i < n; ++i) envs += (size_t)chis[i] * chis[i];
        R[0] = base + envs;
        R[1] = R[0] + maxchi * maxchi;
        U = R[1] + maxchi * maxchi;
        W = U + maxchi * d * maxchi;
    }
    float* probs_dev = reinterpret_cast<float*>(W + maxchi * d * maxchi);
    fill_one_kernel<<<1, 32, 0, s>>>(base, 1);
    MPS_LAUNCH_CHECK("fill_one_kernel");
    for (int i = 0; i + 1 < n; ++i) {
        const int cl = chis[i], cr = chis[i + 1];
        const cf* A = reinterpret_cast<const cf*>(sites[i]);
        cf* L = base + off;
        cf* Ln = L + (size_t)cl * cl;
        // U[l, (x, r')] = sum_l' L[l, l'] conj(A[l', x, r'])
        GemmArgs g1{cl, d * cr, cl, L, cl, 1, 0, A, (long long)d * cr, 1, 1, U, (long long)d * cr, 1};
        int rc = cgemm(g1, s);
        if (rc) return rc;
        // L'[r, r'] = sum_(l,x) A[(l,x), r] U[(l,x), r']
        if (cr > 0 && cl == 0) {
            MPS_CUDA_CHECK(cudaMemsetAsync(Ln, 0, (size_t)cr * cr * sizeof(cf), s));
        } else {
            GemmArgs g2{cr, cr, cl * d, A, 1, cr, 0, U, cr, 1, 0, Ln, cr, 1};
            rc = cgemm(g2, s);
            if (rc) return rc;
        }
        off += (size_t)cl * cl;
    }
    // right-to-left: p_i(x) = sum L_i[l,l'] A[l,x,r] conj(A[l',x,r']) R_i[r,r']
    fill_one_kernel<<<1, 32, 0, s>>>(R[0], 1);
    MPS_LAUNCH_CHECK("fill_one_kernel");
    int cur = 0;
    for (int i = n - 1; i >= 0; --i) {
        const int cl = chis[i], cr = chis[i + 1];
        const cf* A = reinterpret_cast<const cf*>(sites[i]);
        cf* L = base + off;
        // U[(l, x), r'] = sum_r A[(l, x), r] R[r, r']
        GemmArgs g1{cl * d, cr, cr, A, cr, 1, 0, R[cur], cr, 1, 0, U, cr, 1};
        int rc = cgemm(g1, s);
        if (rc) return rc;
        // W[l', (x, r')] = sum_l L[l, l'] U[l, (x, r')]
        GemmArgs g2{cl, d * cr, cl, L, 1, cl, 0, U, (long long)d * cr, 1, 0, W, (long long)d * cr, 1};
        rc = cgemm(g2, s);
        if (rc) return rc;
        marginal_kernel<<<d, 256, 0, s>>>(A, W, cl, d, cr, probs_dev + (size_t)i * d);
        MPS_LAUNCH_CHECK("marginal_kernel");
        if (i > 0) {
            // R'[l, l'] = sum_(x, r') U[l, (x, r')] conj(A[l', (x, r')])
            GemmArgs g3{cl, cl, d * cr, U, (long long)d * cr, 1, 0, A, 1, (long long)d * cr, 1,
                        R[cur ^ 1], cl, 1};
            rc = cgemm(g3, s);
            if (rc) return rc;
            cur ^= 1;
            off -= (size_t)chis[i - 1] * chis[i - 1];
        }
    }
    MPS_CUDA_CHECK(cudaMemcpyAsync(probs_host, probs_dev, (size_t)n * d * sizeof(float),
                                   cudaMemcpyDeviceToHost, s));
    MPS_CUDA_CHECK(cudaStreamSynchronize(s));
    return MPS_OK;
}
