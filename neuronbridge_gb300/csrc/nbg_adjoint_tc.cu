// nbg_adjoint_tc.cu -- the recurrent product of the adjoint on tcgen05
// (C ABI in include/nbg_adjoint.h).
//
// Each adjoint step needs g_ext[b][i] = sum_j dI[b][j] W_rec[i][j], a GEMM of
// B = 128 rows by N by N.  As cuBLAS FP32 it takes about 24 us at N = 1024;
// here it runs on the tensor cores in split BF16:
//   x = x_hi + x_lo,  x_hi = bf16(x),  x_lo = bf16(x - x_hi)
//   dI W^T ~= dI_hi W_hi^T + dI_hi W_lo^T + dI_lo W_hi^T      (FP32 accumulation)
// which keeps about 16 mantissa bits of each operand (the dropped term
// dI_lo W_lo^T is below 2^-16 of the product).
//
// Operands use the UMMA blocked K-major layout of nbg_umma.cuh: A = W (rows
// i, K = j), tiled once per backward by nbg_adjoint_rec_prepare; B = dI
// (rows b, K = j), written tiled by the adjoint step itself
// (nbg_lif_adjoint_step_split).  One CTA owns 128 rows i and all 128 batch
// rows (UMMA M = N = 128, a 128-column TMEM accumulator) over one K range;
// the split-K partials go to g_parts[ks] and the next adjoint step adds them
// in a fixed order, so the backward stays deterministic.
//
// The weight gradients of a checkpoint segment, dW_rec = sum_t S_{t-1}^T dI_t
// and dW_in = sum_t X_t^T dI_t, are the same kind of product with K = the
// segment's (step, batch row) pairs: D[j][n] = sum_K dI^T[j][K] B[n][K] with
// dI^T split (two products) and B = S^T or X^T exact in BF16 (spikes are 0 or
// 1).  nbg_adjoint_blocked_t lays the [L][B][R] FP32 arrays out transposed
// and blocked, nbg_adjoint_wgrad runs the tcgen05 product (UMMA M = 128 rows
// j, N = 256 columns n, split-K partials stored as [split][n][j] so the
// stores are coalesced along j), and nbg_adjoint_reduce_add adds the
// partials into the gradient in a fixed order.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "nbg_adjoint.h"
#include "nbg_common.cuh"
#include "nbg_lif_grad.cuh"
#include "nbg_umma.cuh"

namespace {

using namespace umma;

constexpr int kAdjM = 128, kAdjN = 128;
constexpr int kAdjStages = 3;
constexpr int kAdjBlockA = kAdjM * kKChunk * 2; // 16 KiB per operand block
constexpr int kAdjBlockB = kAdjN * kKChunk * 2;
constexpr int kAdjStageBytes = 2 * kAdjBlockA + 2 * kAdjBlockB; // A_hi A_lo B_hi B_lo
constexpr int kAdjSmemBytes = kAdjStages * kAdjStageBytes + 1024 + 256;
constexpr int kAdjTmemCols = 128;

// kind::f16 instruction descriptor: BF16 x BF16 -> F32, K-major, M = N = 128.
constexpr uint32_t kAdjIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kAdjN >> 3) << 17) |
                               ((uint32_t)(kAdjM >> 4) << 24);

// Element (r, c) of a rows x cols matrix in the blocked layout of 128-row x
// 64-column blocks, block (r / 128, c / 64) at ((r / 128) * (cols / 64) +
// c / 64) blocks.
__device__ __forceinline__ size_t blocked_index(int r, int c, int cols) {
    const size_t blk = (size_t)(r >> 7) * (size_t)(cols >> 6) + (size_t)(c >> 6);
    return blk * (size_t)(kAdjM * kKChunk) + block_offset(r & 127, c & 63) / 2;
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
    hi = __float2bfloat16_rn(x);
    lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

__global__ void k_split_blocked(const float *__restrict__ x, __nv_bfloat16 *__restrict__ hi,
                                __nv_bfloat16 *__restrict__ lo, int rows, int cols) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)rows * cols) return;
    const int r = (int)(idx / cols), c = (int)(idx % cols);
    const size_t o = blocked_index(r, c, cols);
    split_bf16(x[idx], hi[o], lo[o]);
}

// The adjoint step of k_lif_adj (nbg_adjoint.cu) with g_ext the fixed-order
// sum of the split-K partials, writing dI also as the split BF16 B operand.
__global__ void __launch_bounds__(256) k_lif_adj_split(
    const float *__restrict__ g_parts, int n_parts, const float *__restrict__ g_read, float c_t,
    const float *__restrict__ u, const float *__restrict__ s, const unsigned char *__restrict__ m,
    const float *__restrict__ vprev, float *__restrict__ lam_v, float *__restrict__ dI,
    __nv_bfloat16 *__restrict__ dI_hi, __nv_bfloat16 *__restrict__ dI_lo, float *__restrict__ g_theta,
    float *__restrict__ g_alpha, const float *__restrict__ alpha, const float *__restrict__ theta,
    nbg_lif_grad_params p, int N, int total) {
    // programmatic dependent launch: the product that follows may start its
    // prologue (and its W tiles) while this step runs; this step reads
    // g_parts and lam_v only after the product before it has finished
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int j = idx % N;
    const float uu = u[idx], ss = s[idx], lv = lam_v[idx];
    const float th = theta[j];
    const float dsdu = p.smooth ? p.slope * ss * (1.0f - ss) : surrogate(uu - th, p.slope);
    float gs = c_t * g_read[idx] - lv * (uu - p.v_reset);
    if (g_parts) {
        float ge = g_parts[idx];
        for (int q = 1; q < n_parts; ++q) ge = ge + g_parts[(size_t)q * total + idx];
        gs = gs + ge;
    }
    const float gu = gs * dsdu + lv * (1.0f - ss);
    const float gm = m[idx] ? gu : 0.0f;
    dI[idx] = gm;
    const size_t o = blocked_index(idx / N, j, N);
    split_bf16(gm, dI_hi[o], dI_lo[o]);
    lam_v[idx] = gm * (1.0f - alpha[j]);
    g_theta[idx] = g_theta[idx] - gs * dsdu;
    g_alpha[idx] = g_alpha[idx] + gm * (p.v_rest - vprev[idx]);
}

// g_parts[ks][b][i] = sum over the K chunks of split ks of the three split
// products.  Grid (N / 128, split), 256 threads: warp 0 lane 0 produces
// (bulk copies into kAdjStages stages), warp 1 lane 0 issues the MMAs, warp 2
// owns the TMEM allocation, all 8 warps run the epilogue.  Every mbarrier
// wait is bounded; on expiry the CTA records kUmmaTimeout in *err, stops,
// frees its TMEM and returns.
__global__ void __launch_bounds__(kThreads, 1)
    k_adj_umma(const __nv_bfloat16 *__restrict__ w_hi, const __nv_bfloat16 *__restrict__ w_lo,
               const __nv_bfloat16 *__restrict__ d_hi, const __nv_bfloat16 *__restrict__ d_lo,
               float *__restrict__ g_parts, int n, int split, int *__restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *stages = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(stages + kAdjStages * kAdjStageBytes);
    uint64_t *empty = full + kAdjStages;
    uint64_t *done = empty + kAdjStages;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    volatile int *abort = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = blockIdx.x, ks = blockIdx.y;
    const int kchunks = n / kKChunk;
    const int per = kchunks / split;
    const int kc0 = ks * per;
    const int iters = (ks == split - 1) ? kchunks - kc0 : per;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kAdjStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kAdjTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    // Programmatic dependent launch: W does not change during the backward,
    // so the first stages' W tiles are requested before the wait for the
    // adjoint step that writes dI (a no-op without a programmatic launch).
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (warp == 0 && lane == 0) { // producer
        const int pre = iters < kAdjStages ? iters : kAdjStages;
        for (int it = 0; it < pre; ++it) {
            uint8_t *st = stages + it * kAdjStageBytes;
            const size_t a_blk = (size_t)mt * kchunks + kc0 + it;
            mbar_expect_tx(&full[it], kAdjStageBytes);
            bulk_copy(st, (const uint8_t *)w_hi + a_blk * kAdjBlockA, kAdjBlockA, &full[it]);
            bulk_copy(st + kAdjBlockA, (const uint8_t *)w_lo + a_blk * kAdjBlockA, kAdjBlockA, &full[it]);
        }
        asm volatile("griddepcontrol.wait;" ::: "memory");
        for (int it = 0; it < pre; ++it) {
            uint8_t *st = stages + it * kAdjStageBytes;
            const int kc = kc0 + it;
            bulk_copy(st + 2 * kAdjBlockA, (const uint8_t *)d_hi + (size_t)kc * kAdjBlockB, kAdjBlockB, &full[it]);
            bulk_copy(st + 2 * kAdjBlockA + kAdjBlockB, (const uint8_t *)d_lo + (size_t)kc * kAdjBlockB, kAdjBlockB,
                      &full[it]);
        }
        for (int it = pre; it < iters; ++it) {
            const int s = it % kAdjStages;
            if (!mbar_wait(&empty[s], ((it / kAdjStages) & 1) ^ 1, abort)) break;
            uint8_t *st = stages + s * kAdjStageBytes;
            const int kc = kc0 + it;
            const size_t a_blk = (size_t)mt * kchunks + kc;
            mbar_expect_tx(&full[s], kAdjStageBytes);
            bulk_copy(st, (const uint8_t *)w_hi + a_blk * kAdjBlockA, kAdjBlockA, &full[s]);
            bulk_copy(st + kAdjBlockA, (const uint8_t *)w_lo + a_blk * kAdjBlockA, kAdjBlockA, &full[s]);
            bulk_copy(st + 2 * kAdjBlockA, (const uint8_t *)d_hi + (size_t)kc * kAdjBlockB, kAdjBlockB, &full[s]);
            bulk_copy(st + 2 * kAdjBlockA + kAdjBlockB, (const uint8_t *)d_lo + (size_t)kc * kAdjBlockB, kAdjBlockB,
                      &full[s]);
        }
    } else if (warp == 1 && lane == 0) { // MMA issuer
        for (int it = 0; it < iters; ++it) {
            const int s = it % kAdjStages;
            if (!mbar_wait(&full[s], (it / kAdjStages) & 1, abort)) break;
            fence_after();
            const uint32_t a_hi = smem_addr(stages + s * kAdjStageBytes);
            const uint32_t a_lo = a_hi + kAdjBlockA;
            const uint32_t b_hi = a_hi + 2 * kAdjBlockA;
            const uint32_t b_lo = b_hi + kAdjBlockB;
#pragma unroll
            for (int k = 0; k < kKChunk / 16; ++k) {
                mma(tmem, make_desc(a_hi + 256 * k), make_desc(b_hi + 256 * k), kAdjIdesc, (it | k) != 0);
                mma(tmem, make_desc(a_lo + 256 * k), make_desc(b_hi + 256 * k), kAdjIdesc, 1u);
                mma(tmem, make_desc(a_hi + 256 * k), make_desc(b_lo + 256 * k), kAdjIdesc, 1u);
            }
            commit(&empty[s]);
        }
        commit(done);
    }
    __syncwarp();
    asm volatile("griddepcontrol.wait;" ::: "memory"); // the previous adjoint step has read g_parts
    // epilogue: warp w reads TMEM lanes 32*(w%4).. (rows i) and columns
    // 64*(w/4).. (batch rows b)
    mbar_wait(done, 0, abort);
    __syncthreads();
    fence_after();
    const int q = warp & 3, h = warp >> 2;
    const int i = mt * kAdjM + 32 * q + lane;
    if (!*abort) {
        float *out = g_parts + (size_t)ks * kAdjN * n;
#pragma unroll
        for (int c16 = 0; c16 < 4; ++c16) {
            float acc[16];
            tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * h + 16 * c16), acc);
#pragma unroll
            for (int c = 0; c < 16; ++c) out[(size_t)(64 * h + 16 * c16 + c) * n + i] = acc[c];
        }
    }
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && *abort) atomicOr(err, kUmmaTimeout);
    if (warp == 2) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kAdjTmemCols)
                     : "memory");
    }
}

// One adjoint step in one launch: the recurrent product of step t + 1 and
// the adjoint step t that consumes it.  Grid (N / 128, kAdjCluster) in
// clusters of kAdjCluster CTAs along y: the CTAs of a cluster split the K
// range of one 128-row tile of W exactly as k_adj_umma's split-K does
// (cluster rank = split index) and run the same three split products into
// TMEM.  Rank r owns batch rows [16 r, 16 r + 16) of the tile: every CTA
// stores its partial of those rows straight into rank r's receive buffer
// ([source rank][row][i], 64 KiB) through distributed shared memory, which
// waits for nothing.  After one cluster barrier rank r adds the partials of
// ranks 0..7 in order from its own shared memory -- the sum k_lif_adj_split
// forms from g_parts, so the result is the same bit for bit -- and runs the
// adjoint step on those elements, writing dI_t as the split
// BF16 operand of the next step's product into the other of two buffers
// (the next launch reads this one while writing its own), in FP32 (when dI
// is given) and as the split BF16 operand of the weight gradients (when dT_hi
// is given: dI^T, row i, column k_off + b of a k_cols-column blocked matrix,
// eight consecutive b of one i per 16-byte store).  No CTA reads another's
// shared memory, so none waits for its peers before it exits.  Waits on
// mbarriers are bounded as in k_adj_umma; a CTA that gives up still takes
// part in the cluster barrier, and the error word marks the step's results
// invalid.  Two pipeline stages (a CTA has two K chunks at N = 1024) leave
// room for the receive buffer.
constexpr int kAdjCluster = 8;
constexpr int kAdjFusedStages = 2;
constexpr int kAdjRecvBytes = kAdjN * kAdjM * 4;
constexpr int kAdjFusedSmemBytes = kAdjFusedStages * kAdjStageBytes + kAdjRecvBytes + 1024 + 256;

__global__ void __cluster_dims__(1, kAdjCluster, 1) __launch_bounds__(kThreads, 1) k_adj_step_umma(
    const __nv_bfloat16 *__restrict__ w_hi, const __nv_bfloat16 *__restrict__ w_lo,
    const __nv_bfloat16 *__restrict__ d_hi_in, const __nv_bfloat16 *__restrict__ d_lo_in,
    __nv_bfloat16 *__restrict__ d_hi_out, __nv_bfloat16 *__restrict__ d_lo_out, const float *__restrict__ g_read,
    float c_t, const float *__restrict__ u, const float *__restrict__ s, const unsigned char *__restrict__ m,
    const float *__restrict__ vprev, float *__restrict__ lam_v, float *__restrict__ dI, float *__restrict__ g_theta,
    float *__restrict__ g_alpha, const float *__restrict__ alpha, const float *__restrict__ theta,
    nbg_lif_grad_params p, int n, __nv_bfloat16 *__restrict__ dT_hi, __nv_bfloat16 *__restrict__ dT_lo,
    long long k_off, long long k_cols, int *__restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *stages = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *recv = reinterpret_cast<float *>(stages + kAdjFusedStages * kAdjStageBytes); // [rank][row][i]
    uint64_t *full = (uint64_t *)((uint8_t *)recv + kAdjRecvBytes);
    uint64_t *empty = full + kAdjFusedStages;
    uint64_t *done = empty + kAdjFusedStages;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    volatile int *abort = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t rank;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
    const int mt = blockIdx.x, ks = (int)rank;
    const int kchunks = n / kKChunk;
    const int per = kchunks / kAdjCluster;
    const int kc0 = ks * per;
    const int iters = (ks == kAdjCluster - 1) ? kchunks - kc0 : per;

    if (threadIdx.x == 0) {
        for (int st = 0; st < kAdjFusedStages; ++st) {
            mbar_init(&full[st], 1);
            mbar_init(&empty[st], 1);
        }
        mbar_init(done, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kAdjTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    // Programmatic dependent launch: W is constant during the backward, so
    // the first stages' W tiles are requested before the wait for the
    // previous step (which writes dI_{t+1}, lam_v and the gradients).
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (warp == 0 && lane == 0) { // producer
        const int pre = iters < kAdjFusedStages ? iters : kAdjFusedStages;
        for (int it = 0; it < pre; ++it) {
            uint8_t *st = stages + it * kAdjStageBytes;
            const size_t a_blk = (size_t)mt * kchunks + kc0 + it;
            mbar_expect_tx(&full[it], kAdjStageBytes);
            bulk_copy(st, (const uint8_t *)w_hi + a_blk * kAdjBlockA, kAdjBlockA, &full[it]);
            bulk_copy(st + kAdjBlockA, (const uint8_t *)w_lo + a_blk * kAdjBlockA, kAdjBlockA, &full[it]);
        }
        asm volatile("griddepcontrol.wait;" ::: "memory");
        for (int it = 0; it < pre; ++it) {
            uint8_t *st = stages + it * kAdjStageBytes;
            const int kc = kc0 + it;
            bulk_copy(st + 2 * kAdjBlockA, (const uint8_t *)d_hi_in + (size_t)kc * kAdjBlockB, kAdjBlockB, &full[it]);
            bulk_copy(st + 2 * kAdjBlockA + kAdjBlockB, (const uint8_t *)d_lo_in + (size_t)kc * kAdjBlockB,
                      kAdjBlockB, &full[it]);
        }
        for (int it = pre; it < iters; ++it) {
            const int st_i = it % kAdjFusedStages;
            if (!mbar_wait(&empty[st_i], ((it / kAdjFusedStages) & 1) ^ 1, abort)) break;
            uint8_t *st = stages + st_i * kAdjStageBytes;
            const int kc = kc0 + it;
            const size_t a_blk = (size_t)mt * kchunks + kc;
            mbar_expect_tx(&full[st_i], kAdjStageBytes);
            bulk_copy(st, (const uint8_t *)w_hi + a_blk * kAdjBlockA, kAdjBlockA, &full[st_i]);
            bulk_copy(st + kAdjBlockA, (const uint8_t *)w_lo + a_blk * kAdjBlockA, kAdjBlockA, &full[st_i]);
            bulk_copy(st + 2 * kAdjBlockA, (const uint8_t *)d_hi_in + (size_t)kc * kAdjBlockB, kAdjBlockB, &full[st_i]);
            bulk_copy(st + 2 * kAdjBlockA + kAdjBlockB, (const uint8_t *)d_lo_in + (size_t)kc * kAdjBlockB,
                      kAdjBlockB, &full[st_i]);
        }
    } else if (warp == 1 && lane == 0) { // MMA issuer
        for (int it = 0; it < iters; ++it) {
            const int st_i = it % kAdjFusedStages;
            if (!mbar_wait(&full[st_i], (it / kAdjFusedStages) & 1, abort)) break;
            fence_after();
            const uint32_t a_hi = smem_addr(stages + st_i * kAdjStageBytes);
            const uint32_t a_lo = a_hi + kAdjBlockA;
            const uint32_t b_hi = a_hi + 2 * kAdjBlockA;
            const uint32_t b_lo = b_hi + kAdjBlockB;
#pragma unroll
            for (int k = 0; k < kKChunk / 16; ++k) {
                mma(tmem, make_desc(a_hi + 256 * k), make_desc(b_hi + 256 * k), kAdjIdesc, (it | k) != 0);
                mma(tmem, make_desc(a_lo + 256 * k), make_desc(b_hi + 256 * k), kAdjIdesc, 1u);
                mma(tmem, make_desc(a_hi + 256 * k), make_desc(b_lo + 256 * k), kAdjIdesc, 1u);
            }
            commit(&empty[st_i]);
        }
        commit(done);
    }
    __syncwarp();
    // this thread's share of the adjoint step: batch rows 16 ks + 8 bsub + k
    // of column i (eight consecutive rows: one 16-byte store of dI^T).  Its
    // operands are loaded while the products run: first those no adjoint
    // step writes (the forward's record, g_read and the parameters, all
    // complete before the first step of the sweep), before the wait for the
    // previous step, then the accumulators that step updated.
    const int il = threadIdx.x & 127, bsub = threadIdx.x >> 7;
    const int i = mt * kAdjM + il;
    constexpr int kRows = 8;
    float op_u[kRows], op_s[kRows], op_lv[kRows], op_gr[kRows], op_gt[kRows], op_ga[kRows], op_vp[kRows];
    unsigned char op_m[kRows];
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
        const size_t idx = (size_t)(16 * ks + 8 * bsub + k) * n + i;
        op_u[k] = u[idx];
        op_s[k] = s[idx];
        op_gr[k] = g_read[idx];
        op_vp[k] = vprev[idx];
        op_m[k] = m[idx];
    }
    const float th = theta[i], al = alpha[i];
    asm volatile("griddepcontrol.wait;" ::: "memory"); // the previous step's writes are visible
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
        const size_t idx = (size_t)(16 * ks + 8 * bsub + k) * n + i;
        op_lv[k] = lam_v[idx];
        op_gt[k] = g_theta[idx];
        op_ga[k] = g_alpha[idx];
    }
    mbar_wait(done, 0, abort);
    __syncthreads();
    fence_after();
    // the partial accumulator to the rows' owners: warp w holds rows
    // i = 32 (w % 4) + lane and batch columns b = 64 (w / 4) + 16 c16 + c,
    // which rank 4 (w / 4) + c16 owns; they land in its receive buffer at
    // [this rank][c][i]
    {
        const int q = warp & 3, h = warp >> 2;
        const int il = 32 * q + lane;
        if (!*abort) {
            const uint32_t mine = smem_addr(recv) + (uint32_t)((ks * 16 * kAdjM + il) * 4);
#pragma unroll
            for (int c16 = 0; c16 < 4; ++c16) {
                float acc[16];
                tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * h + 16 * c16), acc);
                uint32_t ra;
                asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(mine), "r"(4 * h + c16));
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(ra + (uint32_t)(c * kAdjM * 4)), "f"(acc[c])
                                 : "memory");
            }
        }
    }
    fence_before();
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    // reduce this rank's batch rows over the cluster's partials, in rank
    // order, and run the adjoint step on them
    {
        // every partial of the thread's rows, loaded back to back, then added
        // in rank order
        float x[kRows][kAdjCluster];
#pragma unroll
        for (int k = 0; k < kRows; ++k)
#pragma unroll
            for (int r = 0; r < kAdjCluster; ++r) x[k][r] = recv[(r * 16 + 8 * bsub + k) * kAdjM + il];
        uint32_t t_hi[kRows / 2], t_lo[kRows / 2]; // dI^T of the eight rows, split, packed in pairs
#pragma unroll
        for (int k = 0; k < kRows; ++k) {
            const int b = 16 * ks + 8 * bsub + k;
            float ge = x[k][0];
#pragma unroll
            for (int r = 1; r < kAdjCluster; ++r) ge = ge + x[k][r];
            const size_t idx = (size_t)b * n + i;
            const float uu = op_u[k], ss = op_s[k], lv = op_lv[k];
            const float dsdu = p.smooth ? p.slope * ss * (1.0f - ss) : surrogate(uu - th, p.slope);
            float gs = c_t * op_gr[k] - lv * (uu - p.v_reset);
            gs = gs + ge;
            const float gu = gs * dsdu + lv * (1.0f - ss);
            const float gm = op_m[k] ? gu : 0.0f;
            if (dI) dI[idx] = gm;
            const size_t o = blocked_index(b, i, n);
            __nv_bfloat16 h, l;
            split_bf16(gm, h, l);
            d_hi_out[o] = h;
            d_lo_out[o] = l;
            const uint32_t hb = __bfloat16_as_ushort(h), lb = __bfloat16_as_ushort(l);
            if (k & 1) {
                t_hi[k >> 1] |= hb << 16;
                t_lo[k >> 1] |= lb << 16;
            } else {
                t_hi[k >> 1] = hb;
                t_lo[k >> 1] = lb;
            }
            lam_v[idx] = gm * (1.0f - al);
            g_theta[idx] = op_gt[k] - gs * dsdu;
            g_alpha[idx] = op_ga[k] + gm * (p.v_rest - op_vp[k]);
        }
        if (dT_hi) {
            const size_t o = blocked_index(i, (int)(k_off + 16 * ks + 8 * bsub), (int)k_cols);
            reinterpret_cast<uint4 *>(dT_hi + o)[0] = make_uint4(t_hi[0], t_hi[1], t_hi[2], t_hi[3]);
            reinterpret_cast<uint4 *>(dT_lo + o)[0] = make_uint4(t_lo[0], t_lo[1], t_lo[2], t_lo[3]);
        }
    }
    if (threadIdx.x == 0 && *abort) atomicOr(err, kUmmaTimeout);
    if (warp == 2) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kAdjTmemCols)
                     : "memory");
    }
}

// [L][B][R] FP32 -> the R x (L*B) matrix (row r, K = l*B + b) in the blocked
// layout, split into hi and lo (lo may be null: the values are exact in BF16).
// [L][B][R] FP32 -> the R_pad x (L*B) matrix (row r, K = l*B + b) in the
// blocked layout, split into hi and lo (lo may be null: the values are exact
// in BF16); rows R .. R_pad - 1 are zero (padding to the product's tile).
// One CTA per 128-row x 64-K output block: the 64 x 128 source tile is read
// with coalesced loads into shared memory, and the block -- 16 KiB,
// contiguous in the blocked layout -- is written one 16-byte core-matrix row
// (8 K values of one row) per store.
constexpr int kBtThreads = 256;
__global__ void __launch_bounds__(kBtThreads) k_blocked_t(const float *__restrict__ src, int L, int B, int R,
                                                          int R_pad, __nv_bfloat16 *__restrict__ hi,
                                                          __nv_bfloat16 *__restrict__ lo) {
    __shared__ float tile[kKChunk][kAdjM + 1];
    const int rb = blockIdx.x, kb = blockIdx.y, KK = L * B;
    for (int e = threadIdx.x; e < kKChunk * kAdjM; e += kBtThreads) {
        const int kk = e / kAdjM, rr = e % kAdjM; // r fastest: coalesced along the source row
        const int r = rb * kAdjM + rr;
        tile[kk][rr] = r < R ? src[(size_t)(kb * kKChunk + kk) * R + r] : 0.0f;
    }
    __syncthreads();
    const size_t blk = ((size_t)rb * (size_t)(KK / kKChunk) + (size_t)kb) * (size_t)(kAdjM * kKChunk);
    // 1,024 core-matrix rows of 8 values; element e of the block:
    //   k & 7 = e & 7, row & 7 = (e >> 3) & 7, k >> 3 = (e >> 6) & 7, row >> 3 = e >> 9
    for (int c = threadIdx.x; c < kAdjM * kKChunk / 8; c += kBtThreads) {
        const int e0 = c * 8;
        const int row = ((e0 >> 9) << 3) | ((e0 >> 3) & 7), k0 = ((e0 >> 6) & 7) << 3;
        __align__(16) __nv_bfloat16 h[8], l[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float v = tile[k0 + q][row];
            if (lo) split_bf16(v, h[q], l[q]);
            else h[q] = __float2bfloat16_rn(v);
        }
        reinterpret_cast<uint4 *>(hi + blk)[c] = *reinterpret_cast<const uint4 *>(h);
        if (lo) reinterpret_cast<uint4 *>(lo + blk)[c] = *reinterpret_cast<const uint4 *>(l);
    }
}

constexpr int kWgN = 256; // UMMA N of the weight-gradient product
constexpr int kWgBlockB = kWgN * kKChunk * 2; // 32 KiB
// stages: 3 of A_hi A_lo B (64 KiB), or 2 of A_hi A_lo B_hi B_lo (96 KiB)
template <bool kSplitB> struct WgShape {
    static constexpr int stages = kSplitB ? 2 : 3;
    static constexpr int stage_bytes = 2 * kAdjBlockA + (kSplitB ? 2 : 1) * kWgBlockB;
    static constexpr int smem_bytes = stages * stage_bytes + 1024 + 256;
};
constexpr int kWgTmemCols = 256;
constexpr uint32_t kWgIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kWgN >> 3) << 17) |
                              ((uint32_t)(kAdjM >> 4) << 24);

// part[ks][n][j] = sum over the K chunks of split ks of (a_hi + a_lo)[j][K]
// (b_hi + b_lo)[n][K], the lo x lo product dropped (b_lo absent when b is
// exact in BF16).  a: M x K blocked (128-row tiles), b: Nc x K blocked (its
// 256-row tile n0 = blockIdx.y * 256 is two 128-row block rows).  Grid
// (M / 128, Nc / 256, split); roles as in k_adj_umma.
template <bool kSplitB>
__global__ void __launch_bounds__(kThreads, 1)
    k_wgrad_umma(const __nv_bfloat16 *__restrict__ a_hi, const __nv_bfloat16 *__restrict__ a_lo,
                 const __nv_bfloat16 *__restrict__ b, const __nv_bfloat16 *__restrict__ b_lo,
                 float *__restrict__ part, int M, int Nc, int K, int split, int *__restrict__ err) {
    constexpr int kWgStages = WgShape<kSplitB>::stages;
    constexpr int kWgStageBytes = WgShape<kSplitB>::stage_bytes;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *stages = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(stages + kWgStages * kWgStageBytes);
    uint64_t *empty = full + kWgStages;
    uint64_t *done = empty + kWgStages;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    volatile int *abort = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = blockIdx.x, nt = blockIdx.y, ks = blockIdx.z;
    const int kchunks = K / kKChunk;
    const int per = kchunks / split;
    const int kc0 = ks * per;
    const int iters = (ks == split - 1) ? kchunks - kc0 : per;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kWgStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kWgTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) { // producer
        for (int it = 0; it < iters; ++it) {
            const int s = it % kWgStages;
            if (it >= kWgStages && !mbar_wait(&empty[s], ((it / kWgStages) & 1) ^ 1, abort)) break;
            uint8_t *st = stages + s * kWgStageBytes;
            const int kc = kc0 + it;
            const size_t a_blk = (size_t)mt * kchunks + kc;
            const size_t b_blk0 = (size_t)(2 * nt) * kchunks + kc, b_blk1 = (size_t)(2 * nt + 1) * kchunks + kc;
            mbar_expect_tx(&full[s], kWgStageBytes);
            bulk_copy(st, (const uint8_t *)a_hi + a_blk * kAdjBlockA, kAdjBlockA, &full[s]);
            bulk_copy(st + kAdjBlockA, (const uint8_t *)a_lo + a_blk * kAdjBlockA, kAdjBlockA, &full[s]);
            // the two 128-row halves of the B tile, one after the other: rows
            // 128..255 continue the 8-row core-matrix groups at byte 16384
            bulk_copy(st + 2 * kAdjBlockA, (const uint8_t *)b + b_blk0 * kAdjBlockA, kAdjBlockA, &full[s]);
            bulk_copy(st + 3 * kAdjBlockA, (const uint8_t *)b + b_blk1 * kAdjBlockA, kAdjBlockA, &full[s]);
            if constexpr (kSplitB) {
                bulk_copy(st + 4 * kAdjBlockA, (const uint8_t *)b_lo + b_blk0 * kAdjBlockA, kAdjBlockA, &full[s]);
                bulk_copy(st + 5 * kAdjBlockA, (const uint8_t *)b_lo + b_blk1 * kAdjBlockA, kAdjBlockA, &full[s]);
            }
        }
    } else if (warp == 1 && lane == 0) { // MMA issuer
        for (int it = 0; it < iters; ++it) {
            const int s = it % kWgStages;
            if (!mbar_wait(&full[s], (it / kWgStages) & 1, abort)) break;
            fence_after();
            const uint32_t ah = smem_addr(stages + s * kWgStageBytes);
            const uint32_t al = ah + kAdjBlockA;
            const uint32_t bb = ah + 2 * kAdjBlockA;
#pragma unroll
            for (int k = 0; k < kKChunk / 16; ++k) {
                mma(tmem, make_desc(ah + 256 * k), make_desc(bb + 256 * k), kWgIdesc, (it | k) != 0);
                mma(tmem, make_desc(al + 256 * k), make_desc(bb + 256 * k), kWgIdesc, 1u);
                if constexpr (kSplitB)
                    mma(tmem, make_desc(ah + 256 * k), make_desc(bb + kWgBlockB + 256 * k), kWgIdesc, 1u);
            }
            commit(&empty[s]);
        }
        commit(done);
    }
    __syncwarp();
    mbar_wait(done, 0, abort);
    __syncthreads();
    fence_after();
    // epilogue: warp w reads TMEM lanes 32*(w%4).. (rows j) and columns
    // 128*(w/4).. (n); stores are coalesced along j
    const int q = warp & 3, h = warp >> 2;
    const int j = mt * kAdjM + 32 * q + lane;
    if (!*abort) {
        float *out = part + (size_t)ks * Nc * M;
        for (int c16 = 0; c16 < 8; ++c16) {
            float acc[16];
            tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(128 * h + 16 * c16), acc);
            const int n0 = nt * kWgN + 128 * h + 16 * c16;
#pragma unroll
            for (int c = 0; c < 16; ++c) out[(size_t)(n0 + c) * M + j] = acc[c];
        }
    }
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && *abort) atomicOr(err, kUmmaTimeout);
    if (warp == 2) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kWgTmemCols)
                     : "memory");
    }
}

__global__ void k_reduce_add(float *__restrict__ g, const float *__restrict__ part, int split, long long count,
                             long long stride) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count) return;
    float acc = part[idx];
    for (int q = 1; q < split; ++q) acc = acc + part[(size_t)q * stride + idx];
    g[idx] = g[idx] + acc;
}

bool adj_shape_ok(int B, int N) { return B == kAdjN && N > 0 && N % kAdjM == 0; }

} // namespace

extern "C" {

nbg_status nbg_adjoint_rec_prepare(const float *w_rec, void *w_hi, void *w_lo, int N, void *stream) {
    if (!w_rec || !w_hi || !w_lo || N <= 0 || N % kAdjM)
        return nbg_fail(NBG_ERR_INVALID, "nbg_adjoint_rec_prepare: N must be a positive multiple of %d", kAdjM);
    const long long total = (long long)N * N;
    k_split_blocked<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        w_rec, (__nv_bfloat16 *)w_hi, (__nv_bfloat16 *)w_lo, N, N);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_lif_adjoint_step_split(const float *g_parts, int n_parts, const float *g_read, float c_t,
                                      const float *u, const float *s, const uint8_t *m, const float *vprev,
                                      float *lam_v, float *dI, void *dI_hi, void *dI_lo, float *g_theta,
                                      float *g_alpha, const float *alpha, const float *theta,
                                      const nbg_lif_grad_params *p, int B, int N, void *stream) {
    if (!g_read || !u || !s || !m || !vprev || !lam_v || !dI || !dI_hi || !dI_lo || !g_theta || !g_alpha || !alpha ||
        !theta || !p || (g_parts && n_parts <= 0) || !adj_shape_ok(B, N))
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_adjoint_step_split: bad arguments (B must be %d, N a multiple of %d)",
                        kAdjN, kAdjM);
    const int total = B * N;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((total + 255) / 256);
    cfg.blockDim = dim3(256);
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    NBG_CUDA(cudaLaunchKernelEx(&cfg, k_lif_adj_split, g_parts, n_parts, g_read, c_t, u, s, m, vprev, lam_v, dI,
                                (__nv_bfloat16 *)dI_hi, (__nv_bfloat16 *)dI_lo, g_theta, g_alpha, alpha, theta, *p,
                                N, total));
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_adjoint_rec_grad(const void *w_hi, const void *w_lo, const void *dI_hi, const void *dI_lo,
                                float *g_parts, int split, int B, int N, int *err, void *stream) {
    if (!w_hi || !w_lo || !dI_hi || !dI_lo || !g_parts || !err || !adj_shape_ok(B, N) || split <= 0 ||
        split > N / kKChunk)
        return nbg_fail(NBG_ERR_INVALID, "nbg_adjoint_rec_grad: bad arguments (B must be %d, N a multiple of %d, "
                        "1 <= split <= N / %d)", kAdjN, kAdjM, kKChunk);
    static bool attr_set = false;
    if (!attr_set) {
        NBG_CUDA(cudaFuncSetAttribute(k_adj_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, kAdjSmemBytes));
        attr_set = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(N / kAdjM, split);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = kAdjSmemBytes;
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    NBG_CUDA(cudaLaunchKernelEx(&cfg, k_adj_umma, (const __nv_bfloat16 *)w_hi, (const __nv_bfloat16 *)w_lo,
                                (const __nv_bfloat16 *)dI_hi, (const __nv_bfloat16 *)dI_lo, g_parts, N, split, err));
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_lif_adjoint_step_fused(const void *w_hi, const void *w_lo, const void *dI_hi_in, const void *dI_lo_in,
                                      void *dI_hi_out, void *dI_lo_out, const float *g_read, float c_t,
                                      const float *u, const float *s, const uint8_t *m, const float *vprev,
                                      float *lam_v, float *dI, float *g_theta, float *g_alpha, const float *alpha,
                                      const float *theta, const nbg_lif_grad_params *p, int B, int N, void *dT_hi,
                                      void *dT_lo, int64_t k_off, int64_t k_cols, int *err, void *stream) {
    if (!w_hi || !w_lo || !dI_hi_in || !dI_lo_in || !dI_hi_out || !dI_lo_out || !g_read || !u || !s || !m ||
        !vprev || !lam_v || !g_theta || !g_alpha || !alpha || !theta || !p || !err || !adj_shape_ok(B, N) ||
        N / kKChunk < kAdjCluster || dI_hi_in == dI_hi_out || dI_lo_in == dI_lo_out)
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_adjoint_step_fused: bad arguments (B must be %d, N a multiple of %d "
                        "and at least %d, distinct in and out operand buffers)", kAdjN, kAdjM,
                        kAdjCluster * kKChunk);
    if (dT_hi && (!dT_lo || k_off < 0 || k_off % kAdjN || k_cols % kKChunk || k_off + kAdjN > k_cols ||
                  k_cols > 0x7fffffff))
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_adjoint_step_fused: dT needs dT_lo, k_off a multiple of %d with "
                        "k_off + %d <= k_cols, k_cols a multiple of %d below 2^31", kAdjN, kAdjN, kKChunk);
    static bool attr_set = false;
    if (!attr_set) {
        NBG_CUDA(cudaFuncSetAttribute(k_adj_step_umma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kAdjFusedSmemBytes));
        attr_set = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(N / kAdjM, kAdjCluster);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = kAdjFusedSmemBytes;
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    NBG_CUDA(cudaLaunchKernelEx(&cfg, k_adj_step_umma, (const __nv_bfloat16 *)w_hi, (const __nv_bfloat16 *)w_lo,
                                (const __nv_bfloat16 *)dI_hi_in, (const __nv_bfloat16 *)dI_lo_in,
                                (__nv_bfloat16 *)dI_hi_out, (__nv_bfloat16 *)dI_lo_out, g_read, c_t, u, s, m, vprev,
                                lam_v, dI, g_theta, g_alpha, alpha, theta, *p, N, (__nv_bfloat16 *)dT_hi,
                                (__nv_bfloat16 *)dT_lo, (long long)k_off, (long long)k_cols, err));
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_adjoint_blocked_t(const float *src, int L, int B, int R, int R_pad, void *hi, void *lo,
                                 void *stream) {
    if (!src || !hi || L <= 0 || B <= 0 || R <= 0 || R_pad < R || R_pad % kAdjM || ((long long)L * B) % kKChunk)
        return nbg_fail(NBG_ERR_INVALID, "nbg_adjoint_blocked_t: R_pad must be >= R and a multiple of %d, L*B a "
                        "multiple of %d", kAdjM, kKChunk);
    const dim3 grid(R_pad / kAdjM, (unsigned)(((long long)L * B) / kKChunk));
    k_blocked_t<<<grid, kBtThreads, 0, (cudaStream_t)stream>>>(src, L, B, R, R_pad, (__nv_bfloat16 *)hi,
                                                               (__nv_bfloat16 *)lo);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_adjoint_wgrad(const void *a_hi, const void *a_lo, const void *b, const void *b_lo, int M, int Nc,
                             int K, float *part, int split, int *err, void *stream) {
    if (!a_hi || !a_lo || !b || !part || !err || M <= 0 || M % kAdjM || Nc <= 0 || Nc % kWgN || K <= 0 ||
        K % kKChunk || split <= 0 || split > K / kKChunk)
        return nbg_fail(NBG_ERR_INVALID, "nbg_adjoint_wgrad: M must be a multiple of %d, Nc of %d, K of %d, "
                        "1 <= split <= K / %d", kAdjM, kWgN, kKChunk, kKChunk);
    static bool attr_set[2] = {false, false};
    const dim3 grid(M / kAdjM, Nc / kWgN, split);
    const __nv_bfloat16 *ah = (const __nv_bfloat16 *)a_hi, *al = (const __nv_bfloat16 *)a_lo;
    if (b_lo) {
        if (!attr_set[1]) {
            NBG_CUDA(cudaFuncSetAttribute(k_wgrad_umma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          WgShape<true>::smem_bytes));
            attr_set[1] = true;
        }
        k_wgrad_umma<true><<<grid, kThreads, WgShape<true>::smem_bytes, (cudaStream_t)stream>>>(
            ah, al, (const __nv_bfloat16 *)b, (const __nv_bfloat16 *)b_lo, part, M, Nc, K, split, err);
    } else {
        if (!attr_set[0]) {
            NBG_CUDA(cudaFuncSetAttribute(k_wgrad_umma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          WgShape<false>::smem_bytes));
            attr_set[0] = true;
        }
        k_wgrad_umma<false><<<grid, kThreads, WgShape<false>::smem_bytes, (cudaStream_t)stream>>>(
            ah, al, (const __nv_bfloat16 *)b, nullptr, part, M, Nc, K, split, err);
    }
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_adjoint_reduce_add(float *g, const float *part, int split, int64_t count, int64_t stride,
                                  void *stream) {
    if (!g || !part || split <= 0 || count <= 0 || stride < count)
        return nbg_fail(NBG_ERR_INVALID, "nbg_adjoint_reduce_add: bad arguments");
    k_reduce_add<<<(unsigned)((count + 255) / 256), 256, 0, (cudaStream_t)stream>>>(g, part, split, (long long)count,
                                                                                 (long long)stride);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

} // extern "C"
