// nbg_dense.cu -- dense all-to-all spike delivery for many LIF populations
// sharing one weight matrix (C ABI in include/nbg_dense.h).
//
// Per step t (instances B = 64, neurons N):
//   delivery   I_t = S_{t-1} W          S binary, W N x N FP32
//   update     voltage-jump LIF over B x N neurons, writes S_t
//
// Delivery paths:
//   * NBG_DENSE_SPLIT_BF16 -- tcgen05 (nbg_umma.cuh): the same split-K GEMM
//     with the accumulator in tensor memory and operands in the UMMA blocked
//     layout, moved by bulk copies; W is tiled once at create time and the
//     update kernel writes S blocked.
//   * NBG_DENSE_SPLIT_BF16_SYNC -- the legacy mma.sync tensor path.  W = W_hi + W_lo with both parts
//     BF16 (W_hi = bf16(W), W_lo = bf16(W - W_hi)); a binary spike is exact in
//     BF16, so S W_hi + S W_lo accumulated in FP32 carries ~16 mantissa bits
//     of W.  The GEMM is "swap-AB": M = post-synaptic neurons (128 per CTA),
//     N = the 64 instances, K = pre-synaptic neurons, with W stored transposed
//     (K-major) so that both operands stream K-contiguous.  Split-K = 2 gives
//     128 CTAs; the two partial sums are added in a fixed order by the update
//     kernel, so results are deterministic.  At M = 64 instances the GEMM
//     streams 2 x N^2 BF16 per step and is HBM-bound.
//   * NBG_DENSE_FP32 -- CUDA cores: each post neuron sums W[i][j] over the
//     spiking pre-synaptic i of its instance in ascending i, in FP32, which is
//     the exact sequential sum the CPU oracle computes.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "nbg_common.cuh"
#include "nbg_dense.h"
#include "nbg_umma.cuh"

namespace {

constexpr int kInstances = 64; // GEMM N
constexpr int kBM = 128;       // post neurons per CTA (GEMM M)
constexpr int kBK = 64;        // pre neurons per pipeline stage
constexpr int kStages = 4;
constexpr int kSplitK = 2;
constexpr int kGemmThreads = 256;
constexpr int kStageA = kBM * kBK;              // bf16 elements of one A (W^T) tile
constexpr int kStageB = kInstances * kBK;       // bf16 elements of the S tile
constexpr int kStageElems = 2 * kStageA + kStageB;
constexpr size_t kGemmSmem = (size_t)kStages * kStageElems * sizeof(__nv_bfloat16); // 160 KiB

// ------------------------------------------------------------ preprocessing

// W (pre x post, FP32) -> W_hi^T, W_lo^T (post x pre, BF16): 32 x 32 tiles
// transposed through shared memory.
__global__ void k_split_transpose(const float *__restrict__ w, __nv_bfloat16 *__restrict__ hi,
                                  __nv_bfloat16 *__restrict__ lo, int n) {
    __shared__ float tile[32][33];
    const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) tile[r][threadIdx.x] = w[(size_t)(i0 + r) * n + j0 + threadIdx.x];
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const float x = tile[threadIdx.x][r]; // W[i0 + tx][j0 + r]
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
        const size_t o = (size_t)(j0 + r) * n + i0 + threadIdx.x;
        hi[o] = h;
        lo[o] = l;
    }
}

// W (pre x post, FP32) -> W_hi^T, W_lo^T in the UMMA blocked layout: block
// (m tile, k chunk) of 128 post x 64 pre at ((mt * kchunks + kc) * 16 KiB).
__global__ void k_split_tile(const float *__restrict__ w, __nv_bfloat16 *__restrict__ hi,
                             __nv_bfloat16 *__restrict__ lo, int n) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n * n) return;
    const int k = (int)(idx / n), j = (int)(idx % n); // W[k][j]: pre k, post j
    const float x = w[idx];
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    const int kchunks = n / umma::kKChunk;
    const size_t byte = ((size_t)(j / umma::kM) * kchunks + k / umma::kKChunk) * umma::kBlockA +
                        umma::block_offset(j % umma::kM, k % umma::kKChunk);
    hi[byte / 2] = h;
    lo[byte / 2] = l;
}

// offset (elements) of S[b][k] in the blocked S of the tcgen05 path
__device__ __host__ __forceinline__ size_t s_blocked(int b, int k) {
    return ((size_t)(k / umma::kKChunk) * umma::kBlockB + umma::block_offset(b, k % umma::kKChunk)) / 2;
}

// ------------------------------------------------------------- GEMM (mma.sync)

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}

// element offset of (row, col) in a [rows][64] BF16 tile whose 16-byte chunks
// are XOR-swizzled by row so that ldmatrix reads are bank-conflict free
__device__ __forceinline__ int swz(int row, int col) {
    return row * kBK + ((((col >> 3) ^ (row & 7)) << 3) | (col & 7));
}

__device__ __forceinline__ void ldsm_x4(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3, const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float *c, const unsigned *a, unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One stage: W_hi^T rows [m0, m0+128) x K [k0, k0+64), W_lo^T likewise, and
// S rows [0, 64) x K [k0, k0+64).  16-byte cp.async chunks, 10 per thread.
__device__ __forceinline__ void load_stage(__nv_bfloat16 *st, const __nv_bfloat16 *__restrict__ whi,
                                           const __nv_bfloat16 *__restrict__ wlo,
                                           const __nv_bfloat16 *__restrict__ s, int n, int m0, int k0) {
    const int tid = threadIdx.x;
    // A tiles: 128 rows x 8 chunks = 1024 chunks each
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = tid + q * kGemmThreads;
        const int row = c >> 3, ch = c & 7;
        const size_t g = (size_t)(m0 + row) * n + k0 + ch * 8;
        cp_async16(st + swz(row, ch * 8), whi + g);
        cp_async16(st + kStageA + swz(row, ch * 8), wlo + g);
    }
    // B tile: 64 rows x 8 chunks = 512 chunks
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int c = tid + q * kGemmThreads;
        const int row = c >> 3, ch = c & 7;
        cp_async16(st + 2 * kStageA + swz(row, ch * 8), s + (size_t)row * n + k0 + ch * 8);
    }
}

// partial[ks][b][j] = sum over k in split ks of S[b][k] * (W_hi[k][j] + W_lo[k][j])
__global__ void __launch_bounds__(kGemmThreads, 1)
    k_dense_gemm(const __nv_bfloat16 *__restrict__ whi, const __nv_bfloat16 *__restrict__ wlo,
                 const __nv_bfloat16 *__restrict__ s, float *__restrict__ partial, int n) {
    extern __shared__ __align__(128) __nv_bfloat16 smem[];
    const int m0 = blockIdx.x * kBM;
    const int ks = blockIdx.y;
    const int kper = n / kSplitK;
    const int kbeg = ks * kper;
    const int iters = kper / kBK;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    float acc[8][4];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;

#pragma unroll
    for (int p = 0; p < kStages - 1; ++p) {
        if (p < iters) load_stage(smem + p * kStageElems, whi, wlo, s, n, m0, kbeg + p * kBK);
        asm volatile("cp.async.commit_group;\n");
    }
    for (int it = 0; it < iters; ++it) {
        asm volatile("cp.async.wait_group %0;\n" ::"n"(kStages - 2));
        __syncthreads();
        // prefetch stage it + kStages - 1 into the buffer freed by iteration it-1
        const int nx = it + kStages - 1;
        if (nx < iters) load_stage(smem + (nx % kStages) * kStageElems, whi, wlo, s, n, m0, kbeg + nx * kBK);
        asm volatile("cp.async.commit_group;\n");

        const __nv_bfloat16 *st = smem + (it % kStages) * kStageElems;
        const __nv_bfloat16 *sa_hi = st, *sa_lo = st + kStageA, *sb = st + 2 * kStageA;
#pragma unroll
        for (int kk = 0; kk < kBK; kk += 16) {
            unsigned ahi[4], alo[4];
            {
                const int row = warp * 16 + (lane & 7) + 8 * ((lane >> 3) & 1);
                const int col = kk + 8 * (lane >> 4);
                ldsm_x4(ahi[0], ahi[1], ahi[2], ahi[3], sa_hi + swz(row, col));
                ldsm_x4(alo[0], alo[1], alo[2], alo[3], sa_lo + swz(row, col));
            }
#pragma unroll
            for (int nt = 0; nt < 8; nt += 2) {
                unsigned b0, b1, b2, b3;
                const int row = nt * 8 + (lane & 7) + 8 * (lane >> 4);
                const int col = kk + 8 * ((lane >> 3) & 1);
                ldsm_x4(b0, b1, b2, b3, sb + swz(row, col));
                mma_bf16(acc[nt], ahi, b0, b1);
                mma_bf16(acc[nt], alo, b0, b1);
                mma_bf16(acc[nt + 1], ahi, b2, b3);
                mma_bf16(acc[nt + 1], alo, b2, b3);
            }
        }
    }
    asm volatile("cp.async.wait_group 0;\n");
    // D[j][b] fragments -> partial[ks][b][j]
    const int g = lane >> 2, t4 = lane & 3;
    float *out = partial + (size_t)ks * kInstances * n;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int b = nt * 8 + 2 * t4;
        const int j = m0 + warp * 16 + g;
        out[(size_t)b * n + j] = acc[nt][0];
        out[(size_t)(b + 1) * n + j] = acc[nt][1];
        out[(size_t)b * n + j + 8] = acc[nt][2];
        out[(size_t)(b + 1) * n + j + 8] = acc[nt][3];
    }
}

// --------------------------------------------------------- FP32 CUDA cores

// cur[b][j] = sum over i ascending with bit i of S_b set of W[i][j]
__global__ void __launch_bounds__(256) k_dense_fp32(const float *__restrict__ w, const unsigned *__restrict__ sbits,
                                                    float *__restrict__ cur, int n) {
    extern __shared__ unsigned bits[];
    const int b = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int nw = n / 32;
    for (int k = threadIdx.x; k < nw; k += blockDim.x) bits[k] = sbits[(size_t)b * nw + k];
    __syncthreads();
    float sum = 0.0f;
    for (int k = 0; k < nw; ++k) {
        unsigned word = bits[k];
        while (word) {
            const int i = k * 32 + __ffs(word) - 1;
            word &= word - 1u;
            sum = sum + w[(size_t)i * n + j];
        }
    }
    cur[(size_t)b * n + j] = sum;
}

// -------------------------------------------------------------- LIF update

struct LifParams {
    float v_rest, tau, v_th, r, v_reset, i_ext, dt, drive_w, drive_p;
    int t_ref;
};

// One update of every (instance, neuron): summed arrival, refractory-gated
// voltage jump, forward-Euler voltage-jump LIF (TimeDrivenLIF_Voltage_jump.cpp
// :49-86), spike -> S_t (BF16 0/1 for the tensor path, bit words for FP32).
// One neuron's update (state vv, ls in registers) given its summed arrival
// `a`; idx = the element of the instance-major state (the drive's hash index).
__device__ __forceinline__ bool lif_apply(const LifParams &P, float a, float &vv, int &ls, int t, int idx) {
    if (t >= 1 && nbg_hash_uniform01(idx, t - 1) < P.drive_p) a = a + P.drive_w;
    if (ls > P.t_ref) vv = vv + a;
    float cur = 0.0f;
    cur = cur + P.r * P.i_ext / P.tau;
    const float aux = (ls > P.t_ref) ? cur + (P.v_rest - vv) / P.tau : 0.0f;
    vv = vv + aux * P.dt;
    ls += 1;
    bool spk = false;
    if (vv > P.v_th) {
        vv = P.v_reset;
        ls = 0;
        spk = true;
    }
    return spk;
}

__global__ void __launch_bounds__(256) k_dense_lif(LifParams P, const float *__restrict__ partial, int nparts,
                                                   float *__restrict__ v, int *__restrict__ last,
                                                   __nv_bfloat16 *__restrict__ s_out, int s_blocked_layout,
                                                   unsigned *__restrict__ bits_out, int *__restrict__ counts, int t,
                                                   int n, int total) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    bool spk = false;
    if (idx < total) {
        float a = partial[idx];
        for (int k = 1; k < nparts; ++k) a = a + partial[(size_t)k * total + idx];
        float vv = v[idx];
        int ls = last[idx];
        spk = lif_apply(P, a, vv, ls, t, idx);
        v[idx] = vv;
        last[idx] = ls;
        if (s_out) {
            const __nv_bfloat16 one = __float2bfloat16_rn(spk ? 1.0f : 0.0f);
            if (s_blocked_layout) s_out[s_blocked(idx / n, idx % n)] = one;
            else s_out[idx] = one;
        }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, spk);
    if ((threadIdx.x & 31) == 0) {
        if (bits_out && idx < total) bits_out[idx >> 5] = bal; // n % 32 == 0: a warp is one word
        if (bal) atomicAdd(&counts[0], __popc(bal));
    }
}

// The step's neuron update fused into the tcgen05 delivery: the same update
// as k_dense_lif for the elements of the tile a CTA completes, with their
// state loads batched ahead of the updates; S_t is written in the blocked
// layout the next delivery reads.
struct LifFinish {
    static constexpr bool kActive = true;
    LifParams P;
    float *v;
    int *last;
    __nv_bfloat16 *s_out;
    int *counts;
    int t;
    __device__ void load(int idx, float &vv, int &ls) const {
        vv = v[idx];
        ls = last[idx];
    }
    __device__ bool update(int b, int j, int idx, float a, float vv, int ls) const {
        const bool spk = lif_apply(P, a, vv, ls, t, idx);
        v[idx] = vv;
        last[idx] = ls;
        s_out[s_blocked(b, j)] = __float2bfloat16_rn(spk ? 1.0f : 0.0f);
        return spk;
    }
    __device__ void count(int k) const {
        if (k) atomicAdd(counts, k);
    }
};

} // namespace

struct nbg_dense {
    int device = 0, B = 64, N = 0, precision = 0;
    LifParams P{};
    DevBuf<float> w, partial, v;
    DevBuf<__nv_bfloat16> whi, wlo, s[2];
    DevBuf<unsigned> bits[2];
    DevBuf<int> last, err;
    DevBuf<unsigned int> tile_cnt; // fused-update arrivals per tile (zero between launches)
    std::vector<cudaEvent_t> dev_pool; // delivery start/stop events, 2 per step
    int next_t = 0;
    bool ran = false;
    std::vector<int> counts_host;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evd0 = nullptr, evd1 = nullptr;
    double last_ms = 0.0, last_delivery_ms = 0.0;
    int64_t last_launches = 0;
};

namespace {

nbg_status dense_reset(nbg_dense *d) {
    const size_t tot = (size_t)d->B * d->N;
    std::vector<float> v0(tot, d->P.v_reset); // V_reset + random_mu (legacy init)
    NBG_CUDA(cudaMemcpy(d->v.p, v0.data(), tot * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<int> l0(tot, 10000);
    NBG_CUDA(cudaMemcpy(d->last.p, l0.data(), tot * sizeof(int), cudaMemcpyHostToDevice));
    for (int k = 0; k < 2; ++k) {
        NBG_CUDA(d->s[k].zero());
        NBG_CUDA(d->bits[k].zero());
    }
    if (d->tile_cnt.p) NBG_CUDA(d->tile_cnt.zero());
    d->next_t = 0;
    d->ran = false;
    d->counts_host.clear();
    return NBG_OK;
}

// delivery of S (buffer `par`) into d->partial (parts, instance-major)
nbg_status launch_delivery(nbg_dense *d, int par) {
    if (d->precision == NBG_DENSE_SPLIT_BF16) {
        dim3 grid(d->N / umma::kM, kSplitK);
        umma::k_dense_umma<umma::NoFinish><<<grid, umma::kThreads, umma::kSmemBytes, d->stream>>>(
            d->whi.p, d->wlo.p, d->s[par].p, d->partial.p, d->N, kSplitK, 0, d->err.p, d->tile_cnt.p,
            umma::NoFinish{});
    } else if (d->precision == NBG_DENSE_SPLIT_BF16_SYNC) {
        dim3 grid(d->N / kBM, kSplitK);
        k_dense_gemm<<<grid, kGemmThreads, kGemmSmem, d->stream>>>(d->whi.p, d->wlo.p, d->s[par].p, d->partial.p,
                                                                   d->N);
    } else {
        dim3 grid(d->N / 256, d->B);
        k_dense_fp32<<<grid, 256, (d->N / 32) * sizeof(unsigned), d->stream>>>(d->w.p, d->bits[par].p,
                                                                                d->partial.p, d->N);
    }
    return NBG_OK;
}

} // namespace

extern "C" {

nbg_status nbg_dense_create(int instances, int neurons, const float *w, const nbg_layer_desc *lif,
                            float drive_rate_hz, float drive_weight, float dt_ms, int precision, int device,
                            nbg_dense **out) {
    if (!out || !w || !lif) return nbg_fail(NBG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (instances != kInstances) return nbg_fail(NBG_ERR_UNSUPPORTED, "instances must be %d", kInstances);
    if (neurons <= 0 || neurons % kBM != 0 || (neurons / kSplitK) % kBK != 0)
        return nbg_fail(NBG_ERR_INVALID, "neurons must be a positive multiple of %d", kBM);
    if (lif->model != NBG_MODEL_LIF_VJ) return nbg_fail(NBG_ERR_UNSUPPORTED, "the dense engine runs the voltage-jump LIF");
    if (precision != NBG_DENSE_SPLIT_BF16 && precision != NBG_DENSE_FP32 && precision != NBG_DENSE_SPLIT_BF16_SYNC)
        return nbg_fail(NBG_ERR_INVALID, "unknown precision %d", precision);
    if (!(dt_ms > 0.0f) || !(lif->f[1] != 0.0f)) return nbg_fail(NBG_ERR_INVALID, "dt and tau must be non-zero");
    auto *d = new nbg_dense();
    auto bail = [&](nbg_status st) {
        delete d;
        return st;
    };
    d->device = device;
    d->B = instances;
    d->N = neurons;
    d->precision = precision;
    d->P.v_rest = lif->f[0];
    d->P.tau = lif->f[1];
    d->P.v_th = lif->f[2];
    d->P.r = lif->f[3];
    d->P.v_reset = lif->f[4] + lif->f[5];
    d->P.i_ext = lif->f[6];
    d->P.t_ref = lif->ip[0];
    d->P.dt = dt_ms;
    d->P.drive_w = drive_weight;
    {
        float rate = drive_rate_hz > 0.0f ? drive_rate_hz : 0.0f;
        float p = rate * dt_ms * 0.001f;
        d->P.drive_p = p < 1.0f ? p : 1.0f;
    }
    if (cudaSetDevice(device) != cudaSuccess) return bail(nbg_fail(NBG_ERR_CUDA, "cudaSetDevice(%d) failed", device));
    const size_t nn = (size_t)neurons * neurons, tot = (size_t)instances * neurons;
    cudaError_t ce = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (ce == cudaSuccess) ce = x;
    };
    chk(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking));
    chk(cudaEventCreate(&d->ev0));
    chk(cudaEventCreate(&d->ev1));
    chk(cudaEventCreate(&d->evd0));
    chk(cudaEventCreate(&d->evd1));
    chk(d->v.alloc(tot));
    chk(d->last.alloc(tot));
    chk(d->err.alloc(1));
    chk(d->err.zero());
    chk(d->partial.alloc((size_t)kSplitK * tot));
    for (int k = 0; k < 2; ++k) {
        chk(d->s[k].alloc(tot));
        chk(d->bits[k].alloc(tot / 32));
    }
    if (precision == NBG_DENSE_FP32) {
        chk(d->w.alloc(nn));
        if (ce == cudaSuccess) chk(cudaMemcpy(d->w.p, w, nn * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        DevBuf<float> tmp;
        chk(tmp.alloc(nn));
        chk(d->whi.alloc(nn));
        chk(d->wlo.alloc(nn));
        if (ce == cudaSuccess) chk(cudaMemcpy(tmp.p, w, nn * sizeof(float), cudaMemcpyHostToDevice));
        if (ce == cudaSuccess && precision == NBG_DENSE_SPLIT_BF16) {
            k_split_tile<<<(unsigned)((nn + 255) / 256), 256>>>(tmp.p, d->whi.p, d->wlo.p, neurons);
            chk(cudaGetLastError());
            chk(cudaDeviceSynchronize());
            if (ce == cudaSuccess)
                chk(cudaFuncSetAttribute(umma::k_dense_umma<umma::NoFinish>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, umma::kSmemBytes));
            if (ce == cudaSuccess)
                chk(cudaFuncSetAttribute(umma::k_dense_umma<LifFinish>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         umma::kSmemBytes));
            if (ce == cudaSuccess) chk(d->tile_cnt.alloc((size_t)neurons / umma::kM));
            if (ce == cudaSuccess) chk(d->tile_cnt.zero());
        } else if (ce == cudaSuccess) {
            dim3 grid(neurons / 32, neurons / 32), block(32, 8);
            k_split_transpose<<<grid, block>>>(tmp.p, d->whi.p, d->wlo.p, neurons);
            chk(cudaGetLastError());
            chk(cudaDeviceSynchronize());
        }
        if (ce == cudaSuccess)
            chk(cudaFuncSetAttribute(k_dense_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem));
    }
    if (ce != cudaSuccess)
        return bail(nbg_fail(ce == cudaErrorMemoryAllocation ? NBG_ERR_OOM : NBG_ERR_CUDA, "dense create: %s",
                             cudaGetErrorString(ce)));
    nbg_status st = dense_reset(d);
    if (st != NBG_OK) return bail(st);
    *out = d;
    return NBG_OK;
}

nbg_status nbg_dense_destroy(nbg_dense *d) {
    if (!d) return NBG_OK;
    cudaSetDevice(d->device);
    if (d->stream) cudaStreamSynchronize(d->stream);
    for (cudaEvent_t e : {d->ev0, d->ev1, d->evd0, d->evd1})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : d->dev_pool) cudaEventDestroy(e);
    if (d->stream) cudaStreamDestroy(d->stream);
    delete d;
    return NBG_OK;
}

nbg_status nbg_dense_reset(nbg_dense *d) {
    if (!d) return nbg_fail(NBG_ERR_INVALID, "null engine");
    NBG_CUDA(cudaSetDevice(d->device));
    NBG_CUDA(cudaStreamSynchronize(d->stream));
    return dense_reset(d);
}

nbg_status nbg_dense_run(nbg_dense *d, int steps) {
    if (!d) return nbg_fail(NBG_ERR_INVALID, "null engine");
    if (steps <= 0) return nbg_fail(NBG_ERR_INVALID, "steps must be positive");
    NBG_CUDA(cudaSetDevice(d->device));
    const int count = d->ran ? steps : steps + 1;
    const int total = d->B * d->N;
    std::vector<int> cnt((size_t)count, 0);
    DevBuf<int> dcnt;
    NBG_CUDA(dcnt.alloc((size_t)count));
    NBG_CUDA(cudaMemsetAsync(dcnt.p, 0, count * sizeof(int), d->stream));
    // event pairs bracketing every delivery launch (reused across calls)
    const int chunk = 256;
    while ((int)d->dev_pool.size() < 2 * chunk) {
        cudaEvent_t ev;
        NBG_CUDA(cudaEventCreate(&ev));
        d->dev_pool.push_back(ev);
    }
    double dms = 0.0;
    NBG_CUDA(cudaEventRecord(d->ev0, d->stream));
    const bool tensor = d->precision != NBG_DENSE_FP32;
    const int blocked = d->precision == NBG_DENSE_SPLIT_BF16;
    for (int k0 = 0; k0 < count; k0 += chunk) {
        const int k1 = std::min(count, k0 + chunk);
        for (int k = k0; k < k1; ++k) {
            const int t = d->next_t + k;
            const int in = (t + 1) & 1, outp = t & 1; // S_{t-1} lives in buffer (t-1)&1
            if (blocked) { // tcgen05: delivery and update in one launch, back to back (PDL)
                const LifFinish fin{d->P, d->v.p, d->last.p, d->s[outp].p, dcnt.p + k, t};
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(d->N / umma::kM, kSplitK);
                cfg.blockDim = dim3(umma::kThreads);
                cfg.dynamicSmemBytes = umma::kSmemBytes;
                cfg.stream = d->stream;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
                attr[0].val.programmaticStreamSerializationAllowed = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                NBG_CUDA(cudaLaunchKernelEx(&cfg, umma::k_dense_umma<LifFinish>, (const __nv_bfloat16 *)d->whi.p,
                                            (const __nv_bfloat16 *)d->wlo.p, (const __nv_bfloat16 *)d->s[in].p,
                                            d->partial.p, d->N, (int)kSplitK, t & 1, d->err.p, d->tile_cnt.p, fin));
                continue;
            }
            NBG_CUDA(cudaEventRecord(d->dev_pool[2 * (k - k0)], d->stream));
            launch_delivery(d, in);
            NBG_CUDA(cudaEventRecord(d->dev_pool[2 * (k - k0) + 1], d->stream));
            k_dense_lif<<<(total + 255) / 256, 256, 0, d->stream>>>(
                d->P, d->partial.p, tensor ? kSplitK : 1, d->v.p, d->last.p, tensor ? d->s[outp].p : nullptr, blocked,
                tensor ? nullptr : d->bits[outp].p, dcnt.p + k, t, d->N, total);
        }
        NBG_CUDA(cudaGetLastError());
        if (blocked) continue; // one launch per step, no per-step events (they would break the overlap)
        NBG_CUDA(cudaEventSynchronize(d->dev_pool[2 * (k1 - 1 - k0) + 1]));
        for (int k = k0; k < k1; ++k) {
            float x = 0.0f;
            NBG_CUDA(cudaEventElapsedTime(&x, d->dev_pool[2 * (k - k0)], d->dev_pool[2 * (k - k0) + 1]));
            dms += x;
        }
    }
    NBG_CUDA(cudaEventRecord(d->ev1, d->stream));
    NBG_CUDA(cudaStreamSynchronize(d->stream));
    float ms = 0.0f;
    NBG_CUDA(cudaEventElapsedTime(&ms, d->ev0, d->ev1));
    d->last_ms = ms;
    d->last_delivery_ms = blocked ? ms : dms; // tcgen05: the whole step is the delivery launch
    d->last_launches = (blocked ? 1LL : 2LL) * count;
    NBG_CUDA(cudaMemcpy(cnt.data(), dcnt.p, count * sizeof(int), cudaMemcpyDeviceToHost));
    int errv = 0;
    NBG_CUDA(cudaMemcpy(&errv, d->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (errv) return nbg_fail(NBG_ERR_TIMEOUT, "tensor-core delivery gave up waiting on a pipeline barrier");
    d->counts_host.insert(d->counts_host.end(), cnt.begin(), cnt.end());
    d->next_t += count;
    d->ran = true;
    return NBG_OK;
}

nbg_status nbg_dense_get_state(nbg_dense *d, float *v, int32_t *last) {
    if (!d) return nbg_fail(NBG_ERR_INVALID, "null engine");
    NBG_CUDA(cudaSetDevice(d->device));
    NBG_CUDA(cudaStreamSynchronize(d->stream));
    const size_t tot = (size_t)d->B * d->N;
    if (v) NBG_CUDA(cudaMemcpy(v, d->v.p, tot * sizeof(float), cudaMemcpyDeviceToHost));
    if (last) NBG_CUDA(cudaMemcpy(last, d->last.p, tot * sizeof(int), cudaMemcpyDeviceToHost));
    return NBG_OK;
}

nbg_status nbg_dense_num_steps(nbg_dense *d, int64_t *n) {
    if (!d || !n) return nbg_fail(NBG_ERR_INVALID, "null argument");
    *n = (int64_t)d->counts_host.size();
    return NBG_OK;
}

nbg_status nbg_dense_spike_counts(nbg_dense *d, int32_t *counts) {
    if (!d || !counts) return nbg_fail(NBG_ERR_INVALID, "null argument");
    if (!d->counts_host.empty())
        std::memcpy(counts, d->counts_host.data(), d->counts_host.size() * sizeof(int32_t));
    return NBG_OK;
}

nbg_status nbg_dense_get_spikes(nbg_dense *d, uint8_t *s) {
    if (!d || !s) return nbg_fail(NBG_ERR_INVALID, "null argument");
    NBG_CUDA(cudaSetDevice(d->device));
    NBG_CUDA(cudaStreamSynchronize(d->stream));
    const size_t tot = (size_t)d->B * d->N;
    const int par = (d->next_t - 1) & 1;
    if (d->next_t == 0) {
        std::memset(s, 0, tot);
        return NBG_OK;
    }
    if (d->precision != NBG_DENSE_FP32) {
        std::vector<__nv_bfloat16> h(tot);
        NBG_CUDA(cudaMemcpy(h.data(), d->s[par].p, tot * sizeof(__nv_bfloat16), cudaMemcpyDeviceToHost));
        const bool blocked = d->precision == NBG_DENSE_SPLIT_BF16;
        for (size_t i = 0; i < tot; ++i) {
            const size_t src = blocked ? s_blocked((int)(i / d->N), (int)(i % d->N)) : i;
            s[i] = __bfloat162float(h[src]) != 0.0f;
        }
    } else {
        std::vector<unsigned> h(tot / 32);
        NBG_CUDA(cudaMemcpy(h.data(), d->bits[par].p, (tot / 32) * sizeof(unsigned), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < tot; ++i) s[i] = (h[i >> 5] >> (i & 31)) & 1u;
    }
    return NBG_OK;
}

nbg_status nbg_dense_deliver(nbg_dense *d, const uint8_t *s, float *out) {
    if (!d || !s || !out) return nbg_fail(NBG_ERR_INVALID, "null argument");
    NBG_CUDA(cudaSetDevice(d->device));
    NBG_CUDA(cudaStreamSynchronize(d->stream));
    const size_t tot = (size_t)d->B * d->N;
    // stage S into the buffer of the next step's input, deliver, restore nothing:
    // use a scratch parity-independent copy so the simulation state is untouched
    DevBuf<__nv_bfloat16> sb;
    DevBuf<unsigned> bb;
    DevBuf<float> part;
    NBG_CUDA(part.alloc((size_t)kSplitK * tot));
    if (d->precision == NBG_DENSE_SPLIT_BF16) {
        std::vector<__nv_bfloat16> h(tot);
        for (size_t i = 0; i < tot; ++i)
            h[s_blocked((int)(i / d->N), (int)(i % d->N))] = __float2bfloat16_rn(s[i] ? 1.0f : 0.0f);
        NBG_CUDA(sb.upload(h));
        dim3 grid(d->N / umma::kM, kSplitK);
        umma::k_dense_umma<umma::NoFinish><<<grid, umma::kThreads, umma::kSmemBytes, d->stream>>>(
            d->whi.p, d->wlo.p, sb.p, part.p, d->N, kSplitK, 0, d->err.p, d->tile_cnt.p, umma::NoFinish{});
    } else if (d->precision == NBG_DENSE_SPLIT_BF16_SYNC) {
        std::vector<__nv_bfloat16> h(tot);
        for (size_t i = 0; i < tot; ++i) h[i] = __float2bfloat16_rn(s[i] ? 1.0f : 0.0f);
        NBG_CUDA(sb.upload(h));
        dim3 grid(d->N / kBM, kSplitK);
        k_dense_gemm<<<grid, kGemmThreads, kGemmSmem, d->stream>>>(d->whi.p, d->wlo.p, sb.p, part.p, d->N);
    } else {
        std::vector<unsigned> h(tot / 32, 0u);
        for (size_t i = 0; i < tot; ++i)
            if (s[i]) h[i >> 5] |= 1u << (i & 31);
        NBG_CUDA(bb.upload(h));
        dim3 grid(d->N / 256, d->B);
        k_dense_fp32<<<grid, 256, (d->N / 32) * sizeof(unsigned), d->stream>>>(d->w.p, bb.p, part.p, d->N);
    }
    NBG_CUDA(cudaGetLastError());
    NBG_CUDA(cudaStreamSynchronize(d->stream));
    const bool split = d->precision != NBG_DENSE_FP32;
    std::vector<float> h((size_t)(split ? kSplitK : 1) * tot);
    NBG_CUDA(cudaMemcpy(h.data(), part.p, h.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < tot; ++i) {
        float a = h[i];
        if (split)
            for (int k = 1; k < kSplitK; ++k) a = a + h[(size_t)k * tot + i];
        out[i] = a;
    }
    int errv = 0;
    NBG_CUDA(cudaMemcpy(&errv, d->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (errv) return nbg_fail(NBG_ERR_TIMEOUT, "tensor-core delivery gave up waiting on a pipeline barrier");
    return NBG_OK;
}

nbg_status nbg_dense_profile(nbg_dense *d, double *total_ms, double *delivery_ms, int64_t *launches) {
    if (!d) return nbg_fail(NBG_ERR_INVALID, "null engine");
    if (total_ms) *total_ms = d->last_ms;
    if (delivery_ms) *delivery_ms = d->last_delivery_ms;
    if (launches) *launches = d->last_launches;
    return NBG_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Delivery without allocation (nbg_dense_deliver_noalloc): the split-K
// partial sums go to a file-scope device array instead of a buffer the
// library allocates.  Host code must not use `g_noalloc_partial` as a device
// address: it is a host-side stand-in for the symbol.  The real address is
// looked up once per device with cudaGetSymbolAddress.

static __device__ __align__(256) float g_noalloc_partial[kSplitK * kInstances * NBG_DENSE_NOALLOC_MAX_NEURONS];

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
float *g_noalloc_scratch[kNoAllocMaxDevices] = {};

// out = partial[0] + partial[1]: the same fixed order as the update kernel
__global__ void k_sum_split_partials(const float *__restrict__ part, float *__restrict__ out, int total) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < total) out[idx] = part[idx] + part[(size_t)total + idx];
}

} // namespace

extern "C" nbg_status nbg_dense_deliver_noalloc(const void *w_hi_t, const void *w_lo_t, const void *spikes,
                                                float *out, int neurons, void *stream) {
    if (!w_hi_t || !w_lo_t || !spikes || !out) return nbg_fail(NBG_ERR_INVALID, "null argument");
    // the GEMM reads all three inputs with 16-byte cp.async copies
    if (((uintptr_t)w_hi_t | (uintptr_t)w_lo_t | (uintptr_t)spikes) & 15u)
        return nbg_fail(NBG_ERR_INVALID, "w_hi_t, w_lo_t and spikes must be 16-byte aligned");
    if ((uintptr_t)out & 3u) return nbg_fail(NBG_ERR_INVALID, "out must be 4-byte aligned");
    if (neurons <= 0 || neurons % kBM != 0 || (neurons / kSplitK) % kBK != 0)
        return nbg_fail(NBG_ERR_INVALID, "neurons must be a positive multiple of %d", kBM);
    if (neurons > NBG_DENSE_NOALLOC_MAX_NEURONS)
        return nbg_fail(NBG_ERR_INVALID, "neurons = %d exceeds the no-allocation limit of %d", neurons,
                        NBG_DENSE_NOALLOC_MAX_NEURONS);
    int dev = 0;
    NBG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return nbg_fail(NBG_ERR_UNSUPPORTED, "device ordinal %d too large", dev);
    float *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_scratch[dev]) { // first call on this device: set-up, with `dev` current
            void *p = nullptr;
            NBG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_partial));
            NBG_CUDA(cudaFuncSetAttribute(k_dense_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem));
            g_noalloc_scratch[dev] = static_cast<float *>(p);
        }
        scratch = g_noalloc_scratch[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dim3 grid(neurons / kBM, kSplitK);
    k_dense_gemm<<<grid, kGemmThreads, kGemmSmem, st>>>(static_cast<const __nv_bfloat16 *>(w_hi_t),
                                                         static_cast<const __nv_bfloat16 *>(w_lo_t),
                                                         static_cast<const __nv_bfloat16 *>(spikes), scratch, neurons);
    const int total = kInstances * neurons;
    k_sum_split_partials<<<(total + 255) / 256, 256, 0, st>>>(scratch, out, total);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}
