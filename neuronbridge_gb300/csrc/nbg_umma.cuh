// nbg_umma.cuh -- Blackwell (sm_103a) tensor-core GEMM for split-precision
// dense spike delivery: tcgen05.mma with the accumulator in tensor memory,
// operands staged in shared memory by bulk (TMA) copies, an mbarrier
// producer/consumer pipeline.  Included by nbg_dense.cu.
//
//   D[j][b] = sum_k W_hi^T[j][k] S[b][k] + W_lo^T[j][k] S[b][k]
//
// One CTA owns 128 post-synaptic neurons (UMMA M = 128) and all 64 instances
// (UMMA N = 64) over one K range (split-K).  Per 64-wide K chunk it copies
// three pre-tiled blocks (W_hi^T 16 KiB, W_lo^T 16 KiB, S 8 KiB) with
// cp.async.bulk into one of kUStages stages; one elected thread issues
// 4 k-steps x 2 (hi, lo) tcgen05.mma of K = 16 into the same TMEM
// accumulator and commits the stage back to the producer.  The epilogue
// reads the 128 x 64 FP32 accumulator with tcgen05.ld.
//
// Operand layout (both operands K-major, no swizzle): an operand block of R
// rows x 64 K is made of 8-row x 16-byte core matrices; core matrix (row
// group i, K chunk c) sits at byte c * 128 + i * 1024, row r of it at r * 16.
// So the leading-dimension (K) byte offset is 128 and the stride-dimension
// (M/N) byte offset is 1024; k-step s of a chunk starts at byte 256 * s.
// W is stored in HBM already in this blocked order (nbg_dense.cu tiles it
// once at create time) and the update kernel writes S in it, so every stage
// is three contiguous bulk copies.
//
// Every wait on an mbarrier is bounded (clock64 deadline); on expiry the CTA
// records kUmmaTimeout in the error word, stops issuing, waits (bounded) for
// the MMAs it already issued, frees its TMEM and returns.
//
// Fused step (split = 2): with an active `Finish` functor, the CTA that
// completes a tile (the second of its two split-K contributors to arrive,
// found with one atomic per CTA on a per-tile counter after every thread's
// release fence; nothing waits) adds the other CTA's partial to the
// accumulator it still holds in registers (two-term float addition is
// commutative, so the sum equals partial 0 + partial 1 whichever CTA
// finishes) and runs the functor on each of its elements -- the neuron
// update of the step -- then rearms the counter for the next launch.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace umma {

constexpr int kM = 128, kN = 64, kKChunk = 64;
constexpr int kUStages = 4;
constexpr int kBlockA = kM * kKChunk * 2;  // 16 KiB
constexpr int kBlockB = kN * kKChunk * 2;  // 8 KiB
constexpr int kStageBytes = 2 * kBlockA + kBlockB;
// stages (aligned up to 1024 B inside the allocation) + barrier block
constexpr int kSmemBytes = kUStages * kStageBytes + 1024 + 256;
constexpr int kThreads = 256;
constexpr int kTmemCols = 64;
constexpr int kUmmaTimeout = 4;
constexpr long long kWaitCycles = 2000000000ll; // ~1 s at 2 GHz

// byte offset of element (row, k) inside a blocked R x 64 operand block
__host__ __device__ __forceinline__ uint32_t block_offset(int row, int k) {
    return (uint32_t)((k >> 3) * 128 + (row >> 3) * 1024 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// UMMA shared-memory descriptor: K-major, no swizzle, sm100 version bits.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);          // start address
    d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;     // leading-dimension byte offset (K)
    d |= (uint64_t)((1024u >> 4) & 0x3FFF) << 32;    // stride-dimension byte offset (M/N)
    d |= (uint64_t)1 << 46;                          // descriptor version for sm100
    return d;                                        // base offset 0, layout type 0 = no swizzle
}

// UMMA instruction descriptor, kind::f16: BF16 x BF16 -> F32, K-major A/B.
__host__ __device__ constexpr uint32_t make_idesc() {
    return (1u << 4)                 // D format F32
           | (1u << 7)               // A format BF16
           | (1u << 10)              // B format BF16
           | ((uint32_t)(kN >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Bounded wait: true when the phase with `parity` completed, false on timeout
// or when another role of the CTA already gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort) {
    const long long t0 = clock64();
    while (!mbar_test(bar, parity)) {
        if (*abort) return false;
        if (clock64() - t0 > kWaitCycles) {
            *abort = 1;
            return false;
        }
        __nanosleep(64);
    }
    return true;
}

__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// partial[ks][b][j] for the CTA's 128 post neurons and K range (split ks).
// wt_hi / wt_lo: blocked W^T, block (m tile, k chunk) at ((mt * kchunks + kc) * kBlockA);
// s_blk: blocked S, block kc at kc * kBlockB.
// No fused update: the partial sums are the result.
struct NoFinish {
    static constexpr bool kActive = false;
    __device__ void load(int, float &, int &) const {}
    __device__ bool update(int, int, int, float, float, int) const { return false; }
    __device__ void count(int) const {}
};

template <class Finish>
__global__ void __launch_bounds__(kThreads, 1)
    k_dense_umma(const __nv_bfloat16 *__restrict__ wt_hi, const __nv_bfloat16 *__restrict__ wt_lo,
                 const __nv_bfloat16 *__restrict__ s_blk, float *__restrict__ partial, int n, int split,
                 int reverse, int *__restrict__ err, unsigned int *__restrict__ tile_cnt, const Finish fin) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *stages = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(stages + kUStages * kStageBytes);
    uint64_t *empty = full + kUStages;
    uint64_t *done = empty + kUStages;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    volatile int *abort = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = blockIdx.x, ks = blockIdx.y;
    const int kchunks = n / kKChunk;
    const int per = kchunks / split;
    const int kc0 = ks * per;
    const int iters = (ks == split - 1) ? kchunks - kc0 : per;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kUStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    // Programmatic dependent launch: the next step's grid may be scheduled
    // as soon as every CTA of this one has started; W does not depend on the
    // previous step, so its first stages are requested before the grid
    // dependency wait (a no-op without a programmatic launch), and S and all
    // state after it.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    // K chunks in ascending order, or descending when `reverse`: the chunks a
    // step streams last are still in L2 when the next step, run in the other
    // direction, streams them first
    auto chunk = [&](int it) { return reverse ? kc0 + iters - 1 - it : kc0 + it; };
    if (warp == 0 && lane == 0) { // producer: bulk copies into free stages
        const int pre = iters < kUStages ? iters : kUStages;
        for (int it = 0; it < pre; ++it) {
            uint8_t *st = stages + it * kStageBytes;
            const size_t blk = (size_t)mt * kchunks + chunk(it);
            mbar_expect_tx(&full[it], kStageBytes);
            bulk_copy(st, (const uint8_t *)wt_hi + blk * kBlockA, kBlockA, &full[it]);
            bulk_copy(st + kBlockA, (const uint8_t *)wt_lo + blk * kBlockA, kBlockA, &full[it]);
        }
        asm volatile("griddepcontrol.wait;" ::: "memory");
        for (int it = 0; it < pre; ++it)
            bulk_copy(stages + it * kStageBytes + 2 * kBlockA, (const uint8_t *)s_blk + (size_t)chunk(it) * kBlockB,
                      kBlockB, &full[it]);
        for (int it = pre; it < iters; ++it) {
            const int s = it % kUStages;
            if (!mbar_wait(&empty[s], ((it / kUStages) & 1) ^ 1, abort)) break;
            uint8_t *st = stages + s * kStageBytes;
            const int kc = chunk(it);
            const size_t blk = (size_t)mt * kchunks + kc;
            mbar_expect_tx(&full[s], kStageBytes);
            bulk_copy(st, (const uint8_t *)wt_hi + blk * kBlockA, kBlockA, &full[s]);
            bulk_copy(st + kBlockA, (const uint8_t *)wt_lo + blk * kBlockA, kBlockA, &full[s]);
            bulk_copy(st + 2 * kBlockA, (const uint8_t *)s_blk + (size_t)kc * kBlockB, kBlockB, &full[s]);
        }
    } else if (warp == 1 && lane == 0) { // MMA issuer
        constexpr uint32_t idesc = make_idesc();
        int issued = 0;
        for (int it = 0; it < iters; ++it) {
            const int s = it % kUStages;
            if (!mbar_wait(&full[s], (it / kUStages) & 1, abort)) break;
            fence_after();
            const uint32_t a_hi = smem_addr(stages + s * kStageBytes);
            const uint32_t a_lo = a_hi + kBlockA;
            const uint32_t b = a_hi + 2 * kBlockA;
#pragma unroll
            for (int k = 0; k < kKChunk / 16; ++k) {
                mma(tmem, make_desc(a_hi + 256 * k), make_desc(b + 256 * k), idesc, (it | k) != 0);
                mma(tmem, make_desc(a_lo + 256 * k), make_desc(b + 256 * k), idesc, 1u);
            }
            commit(&empty[s]); // frees the stage once these MMAs have read it
            ++issued;
        }
        commit(done); // arrives when every MMA issued above has completed
        (void)issued;
    }
    __syncwarp();
    asm volatile("griddepcontrol.wait;" ::: "memory"); // before touching anything the previous step wrote
    // epilogue: warp w reads TMEM lanes 32*(w%4).. (post neurons) and
    // columns 32*(w/4).. (instances).  The abort decision is made uniform
    // across the block before the warp-collective tcgen05.ld.
    mbar_wait(done, 0, abort);
    __syncthreads();
    fence_after();
    const int q = warp & 3, h = warp >> 2;
    const int j = mt * kM + 32 * q + lane;
    float acc[2][16];
    if (!*abort) {
        float *out = partial + (size_t)ks * kN * n;
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * h), acc[0]);
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * h + 16), acc[1]);
#pragma unroll
        for (int c = 0; c < 32; ++c) out[(size_t)(32 * h + c) * n + j] = acc[c >> 4][c & 15];
    }
    fence_before();
    if constexpr (Finish::kActive) __threadfence(); // this thread's partial before the CTA's arrival
    __syncthreads();
    if (threadIdx.x == 0 && *abort) atomicOr(err, kUmmaTimeout);
    if (warp == 2) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
    if constexpr (Finish::kActive) {
        __shared__ int finisher;
        if (threadIdx.x == 0)
            finisher = !*abort && atomicAdd(&tile_cnt[mt], 1u) == (unsigned int)(split - 1);
        __syncthreads();
        if (finisher) {
            __threadfence(); // the other contributor's partial is visible after its arrival
            const float *other = partial + (size_t)(ks ^ 1) * kN * n;
            int spikes = 0;
#pragma unroll
            for (int half = 0; half < 2; ++half) { // loads of 16 elements in flight, then their updates
                float oth[16], vv[16];
                int ls[16];
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    const int idx = (32 * h + 16 * half + c) * n + j;
                    oth[c] = __ldcg(other + idx);
                    fin.load(idx, vv[c], ls[c]);
                }
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    const int b = 32 * h + 16 * half + c;
                    spikes += fin.update(b, j, b * n + j, acc[half][c] + oth[c], vv[c], ls[c]) ? 1 : 0;
                }
            }
            for (int o = 16; o > 0; o >>= 1) spikes += __shfl_down_sync(0xffffffffu, spikes, o);
            if (lane == 0) fin.count(spikes);
            if (threadIdx.x == 0) tile_cnt[mt] = 0u;
        }
    }
}

} // namespace umma
