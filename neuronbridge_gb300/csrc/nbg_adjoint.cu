// nbg_adjoint.cu -- forward and adjoint step kernels of the differentiable
// recurrent LIF (C ABI and equations in include/nbg_adjoint.h).  The dense
// products (x W_in, s W_rec, dI W_rec^T and the weight gradients) are plain
// library GEMMs issued by the caller; everything elementwise of a step --
// leak, jump, threshold, surrogate, reset, refractory, readout weighting and
// the parameter gradients -- is one fused kernel each way.

#include <cuda_runtime.h>

#include "nbg_adjoint.h"
#include "nbg_lif_grad.cuh"
#include "nbg_common.cuh"

namespace {


__global__ void __launch_bounds__(256) k_lif_fwd(const float *__restrict__ I, float *__restrict__ v,
                                                 int *__restrict__ ref, float *__restrict__ s_out,
                                                 float *__restrict__ u_rec, unsigned char *__restrict__ m_rec,
                                                 float *__restrict__ vprev_rec, float *__restrict__ z, float c_t,
                                                 const float *__restrict__ alpha, const float *__restrict__ theta,
                                                 nbg_lif_grad_params p, int N, int total) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int j = idx % N;
    const float vp = v[idx];
    const int rf = p.smooth ? 0 : ref[idx];
    const bool m = rf == 0;
    const float a = alpha[j], th = theta[j];
    const float u = m ? vp + a * (p.v_rest - vp) + I[idx] : p.v_reset;
    float s;
    if (p.smooth) s = 1.0f / (1.0f + expf(-p.slope * (u - th)));
    else s = u > th ? 1.0f : 0.0f;
    v[idx] = u - s * (u - p.v_reset);
    if (!p.smooth) ref[idx] = s > 0.0f ? p.t_ref : (rf > 0 ? rf - 1 : 0);
    s_out[idx] = s;
    if (u_rec) u_rec[idx] = u;
    if (m_rec) m_rec[idx] = m ? 1 : 0;
    if (vprev_rec) vprev_rec[idx] = vp;
    if (z) z[idx] = z[idx] + c_t * s;
}

__global__ void __launch_bounds__(256) k_lif_adj(const float *__restrict__ g_ext, const float *__restrict__ g_read,
                                                 float c_t, const float *__restrict__ u, const float *__restrict__ s,
                                                 const unsigned char *__restrict__ m, const float *__restrict__ vprev,
                                                 float *__restrict__ lam_v, float *__restrict__ dI,
                                                 float *__restrict__ g_theta, float *__restrict__ g_alpha,
                                                 const float *__restrict__ alpha, const float *__restrict__ theta,
                                                 nbg_lif_grad_params p, int N, int total) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int j = idx % N;
    const float uu = u[idx], ss = s[idx], lv = lam_v[idx];
    const float th = theta[j];
    const float dsdu = p.smooth ? p.slope * ss * (1.0f - ss) : surrogate(uu - th, p.slope);
    // dL/ds_t: recurrent path + readout + the reset's dependence on s
    float gs = c_t * g_read[idx] - lv * (uu - p.v_reset);
    if (g_ext) gs = gs + g_ext[idx];
    // dL/du_t through the spike and through v_t = u - s (u - V_reset)
    const float gu = gs * dsdu + lv * (1.0f - ss);
    const float gm = m[idx] ? gu : 0.0f;
    dI[idx] = gm;
    lam_v[idx] = gm * (1.0f - alpha[j]);
    g_theta[idx] = g_theta[idx] - gs * dsdu;
    g_alpha[idx] = g_alpha[idx] + gm * (p.v_rest - vprev[idx]);
}

// Spike-driven forward step (spiking mode, binary s): one CTA per instance
// row b.  I = xi + the sum of the W_rec rows of the previous step's spikes in
// ascending neuron order (the spike list of row b), then the same update as
// k_lif_fwd, then the row's new spike list in ascending order (block-wide
// ballot prefix).  Each thread owns columns j = threadIdx.x + q * blockDim.x.
constexpr int kSparseThreads = 256;
constexpr int kSparseCols = 8; // columns per thread: N <= 2048

__global__ void __launch_bounds__(kSparseThreads) k_lif_fwd_sparse(
    const float *__restrict__ xi, const float *__restrict__ w, const int *__restrict__ idx_in,
    const int *__restrict__ cnt_in, int *__restrict__ idx_out, int *__restrict__ cnt_out, float *__restrict__ v,
    int *__restrict__ ref, float *__restrict__ s_out, float *__restrict__ u_rec, unsigned char *__restrict__ m_rec,
    float *__restrict__ vprev_rec, float *__restrict__ z, float c_t, const float *__restrict__ alpha,
    const float *__restrict__ theta, nbg_lif_grad_params p, int N) {
    __shared__ int warp_base[kSparseThreads / 32 + 1];
    const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const size_t row = (size_t)b * N;
    const int nq = (N + kSparseThreads - 1) / kSparseThreads;
    float acc[kSparseCols];
#pragma unroll
    for (int q = 0; q < kSparseCols; ++q) {
        const int j = tid + q * kSparseThreads;
        acc[q] = (q < nq && j < N) ? xi[row + j] : 0.0f;
    }
    const int cnt = cnt_in[b];
    const int *list = idx_in + row;
    for (int k = 0; k < cnt; ++k) {
        const float *wr = w + (size_t)__ldg(&list[k]) * N;
#pragma unroll
        for (int q = 0; q < kSparseCols; ++q) {
            const int j = tid + q * kSparseThreads;
            if (q < nq && j < N) acc[q] = acc[q] + __ldg(&wr[j]);
        }
    }
    int base = 0; // spikes of this row in earlier column chunks
    for (int q = 0; q < nq; ++q) {
        const int j = tid + q * kSparseThreads;
        bool spk = false;
        if (j < N) {
            const size_t i = row + j;
            const float vp = v[i];
            const int rf = ref[i];
            const bool m = rf == 0;
            float a_q = acc[0];
#pragma unroll
            for (int r = 1; r < kSparseCols; ++r)
                if (q == r) a_q = acc[r];
            const float u = m ? vp + alpha[j] * (p.v_rest - vp) + a_q : p.v_reset;
            const float sv = u > theta[j] ? 1.0f : 0.0f;
            v[i] = u - sv * (u - p.v_reset);
            ref[i] = sv > 0.0f ? p.t_ref : (rf > 0 ? rf - 1 : 0);
            s_out[i] = sv;
            if (u_rec) u_rec[i] = u;
            if (m_rec) m_rec[i] = m ? 1 : 0;
            if (vprev_rec) vprev_rec[i] = vp;
            if (z) z[i] = z[i] + c_t * sv;
            spk = sv > 0.0f;
        }
        // ordered compaction of this chunk's spikes
        const unsigned bal = __ballot_sync(0xffffffffu, spk);
        if (lane == 0) warp_base[wid] = __popc(bal);
        __syncthreads();
        if (tid == 0) {
            int sum = 0;
            for (int k = 0; k < kSparseThreads / 32; ++k) {
                const int c = warp_base[k];
                warp_base[k] = sum;
                sum += c;
            }
            warp_base[kSparseThreads / 32] = sum;
        }
        __syncthreads();
        if (spk) idx_out[row + base + warp_base[wid] + __popc(bal & ((1u << lane) - 1u))] = j;
        base += warp_base[kSparseThreads / 32];
        __syncthreads();
    }
    if (tid == 0) cnt_out[b] = base;
}

// A whole checkpoint segment of the spike-driven forward: L steps of
// k_lif_fwd_sparse in one launch.  Rows are independent (row b's input at
// step t is x_t W_in plus the W_rec rows of row b's own spikes of step t-1),
// so each CTA runs its row through all L steps with v and ref in registers
// and the spike list in shared memory: no launch per step and no exchange
// between CTAs.  The arithmetic is k_lif_fwd_sparse's, in the same order.
//
// acc[q] (column tid + q * kSparseThreads) += the rows idx[0..n) of w (N
// columns), in ascending k, each scaled by val[k] when kScaled.  The rows are
// fetched kRowBatch at a time before any is added, so a batch costs one L2
// round trip instead of one per row; the additions keep their order.
constexpr int kRowBatch = 4;
template <bool kScaled>
__device__ __forceinline__ void gather_rows(float (&acc)[kSparseCols], const float *__restrict__ w,
                                            const int *idx, const float *val, int n, int tid, int nq, int N) {
    for (int k0 = 0; k0 < n; k0 += kRowBatch) {
        float x[kRowBatch][kSparseCols];
#pragma unroll
        for (int r = 0; r < kRowBatch; ++r) {
            const float *wr = w + (size_t)(k0 + r < n ? idx[k0 + r] : 0) * N;
#pragma unroll
            for (int q = 0; q < kSparseCols; ++q) {
                const int j = tid + q * kSparseThreads;
                x[r][q] = (k0 + r < n && q < nq && j < N) ? __ldg(&wr[j]) : 0.0f;
            }
        }
#pragma unroll
        for (int r = 0; r < kRowBatch; ++r) {
            if (k0 + r >= n) break;
            const float v = kScaled ? val[k0 + r] : 1.0f;
#pragma unroll
            for (int q = 0; q < kSparseCols; ++q) {
                const int j = tid + q * kSparseThreads;
                if (q < nq && j < N) acc[q] = kScaled ? acc[q] + v * x[r][q] : acc[q] + x[r][q];
            }
        }
    }
}

//
// kGather: the input term too is a gather instead of a precomputed xi.  At
// every step the CTA lists row b's nonzero inputs x_t[b][c] (ascending c,
// with their values) in shared memory and starts the sum from them:
// I_t = (sum over listed c of x_t[b][c] * W_in[c]) + (the W_rec rows of the
// previous step's spikes), each term added in ascending order.  With spike
// inputs (x in {0, 1}) the products are exact and the step costs a few rows
// of W_in instead of a GEMM of the segment's inputs.
template <bool kGather>
__global__ void __launch_bounds__(kSparseThreads) k_lif_fwd_segment(
    const float *__restrict__ xi, const float *__restrict__ x, const float *__restrict__ w_in, int C,
    const float *__restrict__ w, int *__restrict__ spk, int *__restrict__ cnt,
    float *__restrict__ v, int *__restrict__ ref, float *__restrict__ s_out, float *__restrict__ s_last,
    float *__restrict__ u_rec, unsigned char *__restrict__ m_rec, float *__restrict__ vprev_rec,
    float *__restrict__ z, const float *__restrict__ c, const float *__restrict__ alpha,
    const float *__restrict__ theta, nbg_lif_grad_params p, int L, int B, int N) {
    extern __shared__ int seg_lists[]; // [2][N], then (kGather) in_idx[C], in_val[C]
    __shared__ int warp_base[kSparseThreads / 32 + 1];
    __shared__ int list_cnt[2];
    int *in_idx = seg_lists + 2 * N;
    float *in_val = reinterpret_cast<float *>(in_idx + C);
    const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const size_t row = (size_t)b * N, plane = (size_t)B * N;
    const int nq = (N + kSparseThreads - 1) / kSparseThreads;
    float vv[kSparseCols], zz[kSparseCols];
    int rr[kSparseCols];
#pragma unroll
    for (int q = 0; q < kSparseCols; ++q) {
        const int j = tid + q * kSparseThreads;
        vv[q] = zz[q] = 0.0f;
        rr[q] = 0;
        if (q < nq && j < N) {
            vv[q] = v[row + j];
            rr[q] = ref[row + j];
            if (z) zz[q] = z[row + j];
        }
    }
    if (tid == 0) list_cnt[0] = cnt[b];
    __syncthreads();
    for (int k = tid; k < list_cnt[0]; k += kSparseThreads) seg_lists[k] = spk[row + k];
    __syncthreads();
    int cur = 0;
    for (int step = 0; step < L; ++step) {
        float acc[kSparseCols];
        if constexpr (kGather) {
            // row b's nonzero inputs of this step, ascending
            const float *xr = x + ((size_t)step * B + b) * C;
            int nin = 0;
            for (int c0 = 0; c0 < C; c0 += kSparseThreads) {
                const int ch = c0 + tid;
                const float xv = ch < C ? xr[ch] : 0.0f;
                const bool nz = xv != 0.0f;
                const unsigned bal = __ballot_sync(0xffffffffu, nz);
                if (lane == 0) warp_base[wid] = __popc(bal);
                __syncthreads();
                if (tid == 0) {
                    int sum = 0;
                    for (int k = 0; k < kSparseThreads / 32; ++k) {
                        const int cc = warp_base[k];
                        warp_base[k] = sum;
                        sum += cc;
                    }
                    warp_base[kSparseThreads / 32] = sum;
                }
                __syncthreads();
                if (nz) {
                    const int at = nin + warp_base[wid] + __popc(bal & ((1u << lane) - 1u));
                    in_idx[at] = ch;
                    in_val[at] = xv;
                }
                nin += warp_base[kSparseThreads / 32];
                __syncthreads();
            }
#pragma unroll
            for (int q = 0; q < kSparseCols; ++q) acc[q] = 0.0f;
            gather_rows<true>(acc, w_in, in_idx, in_val, nin, tid, nq, N);
        } else {
            const float *xs = xi + (size_t)step * plane + row;
#pragma unroll
            for (int q = 0; q < kSparseCols; ++q) {
                const int j = tid + q * kSparseThreads;
                acc[q] = (q < nq && j < N) ? xs[j] : 0.0f;
            }
        }
        const int *list = seg_lists + cur * N;
        gather_rows<false>(acc, w, list, nullptr, list_cnt[cur], tid, nq, N);
        int *out_list = seg_lists + (cur ^ 1) * N;
        int base = 0;
        const float ct = z ? c[step] : 0.0f;
#pragma unroll
        for (int q = 0; q < kSparseCols; ++q) {
            if (q >= nq) break;
            const int j = tid + q * kSparseThreads;
            bool sp = false;
            if (j < N) {
                const size_t i = row + j, o = (size_t)step * plane + i;
                const float vp = vv[q];
                const int rf = rr[q];
                const bool m = rf == 0;
                const float u = m ? vp + alpha[j] * (p.v_rest - vp) + acc[q] : p.v_reset;
                const float sv = u > theta[j] ? 1.0f : 0.0f;
                vv[q] = u - sv * (u - p.v_reset);
                rr[q] = sv > 0.0f ? p.t_ref : (rf > 0 ? rf - 1 : 0);
                if (s_out) s_out[o] = sv;
                if (s_last && step == L - 1) s_last[i] = sv;
                if (u_rec) u_rec[o] = u;
                if (m_rec) m_rec[o] = m ? 1 : 0;
                if (vprev_rec) vprev_rec[o] = vp;
                if (z) zz[q] = zz[q] + ct * sv;
                sp = sv > 0.0f;
            }
            // ordered compaction of this chunk's spikes into the next list
            const unsigned bal = __ballot_sync(0xffffffffu, sp);
            if (lane == 0) warp_base[wid] = __popc(bal);
            __syncthreads();
            if (tid == 0) {
                int sum = 0;
                for (int k = 0; k < kSparseThreads / 32; ++k) {
                    const int cc = warp_base[k];
                    warp_base[k] = sum;
                    sum += cc;
                }
                warp_base[kSparseThreads / 32] = sum;
            }
            __syncthreads();
            if (sp) out_list[base + warp_base[wid] + __popc(bal & ((1u << lane) - 1u))] = j;
            base += warp_base[kSparseThreads / 32];
            __syncthreads();
        }
        if (tid == 0) list_cnt[cur ^ 1] = base;
        __syncthreads();
        cur ^= 1;
    }
#pragma unroll
    for (int q = 0; q < kSparseCols; ++q) {
        const int j = tid + q * kSparseThreads;
        if (q < nq && j < N) {
            v[row + j] = vv[q];
            ref[row + j] = rr[q];
            if (z) z[row + j] = zz[q];
        }
    }
    const int nl = list_cnt[cur];
    for (int k = tid; k < nl; k += kSparseThreads) spk[row + k] = seg_lists[cur * N + k];
    if (tid == 0) cnt[b] = nl;
}

// Ascending spike list of each row of a 0/1 matrix (segment restarts).
__global__ void __launch_bounds__(kSparseThreads) k_spike_list(const float *__restrict__ s, int *__restrict__ idx,
                                                               int *__restrict__ cnt, int N) {
    __shared__ int warp_base[kSparseThreads / 32 + 1];
    const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const size_t row = (size_t)b * N;
    int base = 0;
    for (int c0 = 0; c0 < N; c0 += kSparseThreads) {
        const int j = c0 + tid;
        const bool spk = j < N && s[row + j] > 0.0f;
        const unsigned bal = __ballot_sync(0xffffffffu, spk);
        if (lane == 0) warp_base[wid] = __popc(bal);
        __syncthreads();
        if (tid == 0) {
            int sum = 0;
            for (int k = 0; k < kSparseThreads / 32; ++k) {
                const int c = warp_base[k];
                warp_base[k] = sum;
                sum += c;
            }
            warp_base[kSparseThreads / 32] = sum;
        }
        __syncthreads();
        if (spk) idx[row + base + warp_base[wid] + __popc(bal & ((1u << lane) - 1u))] = j;
        base += warp_base[kSparseThreads / 32];
        __syncthreads();
    }
    if (tid == 0) cnt[b] = base;
}

__global__ void k_poisson(float *__restrict__ x, const float *__restrict__ rates, int T, int B, int C, float dt,
                          int seed, long long total) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int c = (int)(idx % C);
    const int bc = (int)(idx % ((long long)B * C));
    const int t = (int)(idx / ((long long)B * C));
    float r = rates[c];
    r = r > 0.0f ? r : 0.0f;
    float prob = r * dt * 0.001f;
    prob = prob < 1.0f ? prob : 1.0f;
    x[idx] = nbg_hash_uniform01(bc + seed, t) < prob ? 1.0f : 0.0f;
}

} // namespace

// C[i][j] = sum over k of A[i][k] B[k][j] (element (r, c) of A at
// A[r * a_rs + c * a_cs], likewise B), for the readout's small products
// (B x N by N x O and the like).  Short sums (K < kSmallGemmWarpK): one
// thread per output, k ascending.  Long ones: one warp per output, lane l
// adding k = l, l + 32, ... in order, then the 32 lane sums in a fixed tree.
// Either way the order depends only on K, so the result does not depend on
// the launch.
constexpr int kSmallGemmWarpK = 64;

__global__ void k_small_gemm(const float *__restrict__ A, int a_rs, int a_cs, const float *__restrict__ Bm, int b_rs,
                             int b_cs, float *__restrict__ Cm, int M, int N, int K) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= (long long)M * N) return;
    const int i = (int)(o / N), j = (int)(o % N);
    float acc = 0.0f;
    for (int k = 0; k < K; ++k) acc = acc + A[(size_t)i * a_rs + (size_t)k * a_cs] * Bm[(size_t)k * b_rs + (size_t)j * b_cs];
    Cm[o] = acc;
}

__global__ void k_small_gemm_warp(const float *__restrict__ A, int a_rs, int a_cs, const float *__restrict__ Bm,
                                  int b_rs, int b_cs, float *__restrict__ Cm, int M, int N, int K) {
    const long long o = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (o >= (long long)M * N) return; // whole warps: o is the same for all 32 lanes
    const int i = (int)(o / N), j = (int)(o % N);
    float acc = 0.0f;
    for (int k = lane; k < K; k += 32)
        acc = acc + A[(size_t)i * a_rs + (size_t)k * a_cs] * Bm[(size_t)k * b_rs + (size_t)j * b_cs];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc = acc + __shfl_down_sync(0xffffffffu, acc, d);
    if (lane == 0) Cm[o] = acc;
}

extern "C" {

nbg_status nbg_small_gemm(const float *A, int a_rs, int a_cs, const float *B, int b_rs, int b_cs, float *C, int M,
                          int N, int K, void *stream) {
    if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0) return nbg_fail(NBG_ERR_INVALID, "nbg_small_gemm: bad arguments");
    const long long total = (long long)M * N;
    if (K >= kSmallGemmWarpK)
        k_small_gemm_warp<<<(unsigned)((total + 3) / 4), 128, 0, (cudaStream_t)stream>>>(A, a_rs, a_cs, B, b_rs, b_cs,
                                                                                         C, M, N, K);
    else
        k_small_gemm<<<(unsigned)((total + 127) / 128), 128, 0, (cudaStream_t)stream>>>(A, a_rs, a_cs, B, b_rs, b_cs,
                                                                                       C, M, N, K);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_lif_forward_step(const float *I, float *v, int32_t *ref, float *s_out, float *u_rec, uint8_t *m_rec,
                                float *vprev_rec, float *z, float c_t, const float *alpha, const float *theta,
                                const nbg_lif_grad_params *p, int B, int N, void *stream) {
    if (!I || !v || !ref || !s_out || !alpha || !theta || !p || B <= 0 || N <= 0)
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_forward_step: bad arguments");
    const int total = B * N;
    k_lif_fwd<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(I, v, ref, s_out, u_rec, m_rec, vprev_rec, z,
                                                                      c_t, alpha, theta, *p, N, total);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_lif_adjoint_step(const float *g_ext, const float *g_read, float c_t, const float *u, const float *s,
                                const uint8_t *m, const float *vprev, float *lam_v, float *dI, float *g_theta,
                                float *g_alpha, const float *alpha, const float *theta, const nbg_lif_grad_params *p,
                                int B, int N, void *stream) {
    if (!g_read || !u || !s || !m || !vprev || !lam_v || !dI || !g_theta || !g_alpha || !alpha || !theta || !p ||
        B <= 0 || N <= 0)
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_adjoint_step: bad arguments");
    const int total = B * N;
    k_lif_adj<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(g_ext, g_read, c_t, u, s, m, vprev, lam_v, dI,
                                                                      g_theta, g_alpha, alpha, theta, *p, N, total);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_lif_forward_step_sparse(const float *xi, const float *w_rec, const int32_t *spk_in,
                                       const int32_t *cnt_in, int32_t *spk_out, int32_t *cnt_out, float *v,
                                       int32_t *ref, float *s_out, float *u_rec, uint8_t *m_rec, float *vprev_rec,
                                       float *z, float c_t, const float *alpha, const float *theta,
                                       const nbg_lif_grad_params *p, int B, int N, void *stream) {
    if (!xi || !w_rec || !spk_in || !cnt_in || !spk_out || !cnt_out || !v || !ref || !s_out || !alpha || !theta ||
        !p || B <= 0 || N <= 0)
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_forward_step_sparse: bad arguments");
    if (p->smooth) return nbg_fail(NBG_ERR_UNSUPPORTED, "the spike-driven step needs binary spikes (smooth = 0)");
    if (N > kSparseThreads * kSparseCols)
        return nbg_fail(NBG_ERR_UNSUPPORTED, "the spike-driven step supports up to %d neurons",
                        kSparseThreads * kSparseCols);
    k_lif_fwd_sparse<<<B, kSparseThreads, 0, (cudaStream_t)stream>>>(xi, w_rec, spk_in, cnt_in, spk_out, cnt_out, v,
                                                                      ref, s_out, u_rec, m_rec, vprev_rec, z, c_t,
                                                                      alpha, theta, *p, N);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_lif_forward_segment_sparse(const float *xi, const float *w_rec, int32_t *spk, int32_t *cnt, float *v,
                                          int32_t *ref, float *s_out, float *s_last, float *u_rec, uint8_t *m_rec,
                                          float *vprev_rec, float *z, const float *c, const float *alpha,
                                          const float *theta, const nbg_lif_grad_params *p, int L, int B, int N,
                                          void *stream) {
    if (!xi || !w_rec || !spk || !cnt || !v || !ref || !alpha || !theta || !p || (z && !c) || L <= 0 || B <= 0 ||
        N <= 0)
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_forward_segment_sparse: bad arguments");
    if (p->smooth) return nbg_fail(NBG_ERR_UNSUPPORTED, "the spike-driven step needs binary spikes (smooth = 0)");
    if (N > kSparseThreads * kSparseCols)
        return nbg_fail(NBG_ERR_UNSUPPORTED, "the spike-driven step supports up to %d neurons",
                        kSparseThreads * kSparseCols);
    k_lif_fwd_segment<false><<<B, kSparseThreads, 2 * N * sizeof(int), (cudaStream_t)stream>>>(
        xi, nullptr, nullptr, 0, w_rec, spk, cnt, v, ref, s_out, s_last, u_rec, m_rec, vprev_rec, z, c, alpha,
        theta, *p, L, B, N);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_lif_forward_segment_gather(const float *x, const float *w_in, int C, const float *w_rec, int32_t *spk,
                                          int32_t *cnt, float *v, int32_t *ref, float *s_out, float *s_last,
                                          float *u_rec, uint8_t *m_rec, float *vprev_rec, float *z, const float *c,
                                          const float *alpha, const float *theta, const nbg_lif_grad_params *p,
                                          int L, int B, int N, void *stream) {
    if (!x || !w_in || C <= 0 || !w_rec || !spk || !cnt || !v || !ref || !alpha || !theta || !p || (z && !c) ||
        L <= 0 || B <= 0 || N <= 0)
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_forward_segment_gather: bad arguments");
    if (p->smooth) return nbg_fail(NBG_ERR_UNSUPPORTED, "the spike-driven step needs binary spikes (smooth = 0)");
    if (N > kSparseThreads * kSparseCols)
        return nbg_fail(NBG_ERR_UNSUPPORTED, "the spike-driven step supports up to %d neurons",
                        kSparseThreads * kSparseCols);
    const size_t smem = (2 * (size_t)N + 2 * (size_t)C) * sizeof(int);
    if (smem > 200 * 1024) return nbg_fail(NBG_ERR_UNSUPPORTED, "too many inputs for the gather form (C = %d)", C);
    if (smem > 48 * 1024)
        NBG_CUDA(cudaFuncSetAttribute(k_lif_fwd_segment<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    k_lif_fwd_segment<true><<<B, kSparseThreads, smem, (cudaStream_t)stream>>>(
        nullptr, x, w_in, C, w_rec, spk, cnt, v, ref, s_out, s_last, u_rec, m_rec, vprev_rec, z, c, alpha, theta,
        *p, L, B, N);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_spike_lists(const float *s, int32_t *spk, int32_t *cnt, int B, int N, void *stream) {
    if (!s || !spk || !cnt || B <= 0 || N <= 0) return nbg_fail(NBG_ERR_INVALID, "nbg_spike_lists: bad arguments");
    k_spike_list<<<B, kSparseThreads, 0, (cudaStream_t)stream>>>(s, spk, cnt, N);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_poisson_inputs(float *x, const float *rates_hz, int T, int B, int C, float dt_ms, int seed,
                              void *stream) {
    if (!x || !rates_hz || T <= 0 || B <= 0 || C <= 0) return nbg_fail(NBG_ERR_INVALID, "nbg_poisson_inputs: bad arguments");
    const long long total = (long long)T * B * C;
    k_poisson<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, rates_hz, T, B, C, dt_ms, seed,
                                                                                  total);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

} // extern "C"
