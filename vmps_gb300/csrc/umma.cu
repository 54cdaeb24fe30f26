// tcgen05 (UMMA) engine of the split-precision grouped GEMM (sm_103a).
//
// Same work lists and operand layout as gg_split_kernel in kernels.cu: every
// operand is pre-split into bf16 hi and lo arrays, stored K-contiguous (rows of
// A, columns of B) with rows padded to 8 elements and zero padding.  One CTA
// owns one output tile of up to 128 x 64 and walks its segments' K ranges in
// steps of 64:
//
//   * all 128 threads stage the step's four 64-wide slices (A hi/lo: 128 rows,
//     B hi/lo: 64 rows) with cp.async into a 4-deep ring of shared-memory
//     stages, in the 128-byte-swizzled K-major layout the UMMA descriptors
//     describe (16-byte chunk c of row r stored at chunk c ^ (r % 8));
//   * one thread issues, per 16-wide K slice, tcgen05.mma lo*hi, hi*lo, hi*hi
//     (kind::f16, bf16 inputs, FP32 accumulator of 128 lanes x 64 columns in
//     tensor memory) and tcgen05.commit to the stage's mbarrier, which tells
//     the producers when the stage may be refilled;
//   * the epilogue reads the accumulator with tcgen05.ld (each warp its 32
//     lanes) and writes FP64, or bf16 hi/lo for the next phase.
//
// Every mbarrier wait is bounded by a clock budget; a wait that runs out sets
// the error word, the kernel skips the remaining MMAs, releases its tensor
// memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.hpp"

namespace vmps {
namespace um {
constexpr int BM = 128, BN = 64, BK = 64, NT = 128, STAGES = 4;
constexpr int A_BYTES = BM * BK * 2;                       // one of A hi / A lo: 16 KB
constexpr int B_BYTES = BN * BK * 2;                       // one of B hi / B lo: 8 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;     // 48 KB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 128;
constexpr uint32_t TMEM_COLS = 64;
// kind::f16 instruction descriptor: D FP32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);
constexpr long long WAIT_BUDGET = 4000000000LL;           // clock cycles (~2 s) per mbarrier wait
}  // namespace um

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);   // start address >> 4
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset between 8-row groups
    d |= (uint64_t)1 << 46;                    // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;                    // 128-byte swizzle
    return d;
}
// byte offset of (row, 16-byte chunk) inside a swizzled K-major tile
__device__ __forceinline__ uint32_t swz(int r, int c) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

__device__ __forceinline__ void cp16(uint32_t dst, const void* src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ uint32_t mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok;
}
// bounded wait: false when the clock budget ran out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_test(bar, parity))
        if (clock64() - t0 > um::WAIT_BUDGET) return false;
    return true;
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(um::IDESC), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// 32 lanes x 16 consecutive 32-bit columns of tensor memory
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int OUT_SPLIT>
__global__ void __launch_bounds__(um::NT, 1) gg_umma_kernel(GGArgs g) {
    using namespace um;
    extern __shared__ __align__(1024) unsigned char smraw[];
    // 1024-byte aligned stage ring (the swizzle pattern is anchored to 1024-byte boundaries)
    const uint32_t raw = su32(smraw);
    const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
    unsigned char* ring = smraw + pad;
    const uint32_t ring_s = raw + pad;
    uint64_t* bars = reinterpret_cast<uint64_t*>(ring + STAGES * STAGE_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + STAGES);
    __shared__ int s_fail;

    const GTile tile = g.tiles[blockIdx.x];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int mrem = tile.tm, nrem = tile.tn;
    const __nv_bfloat16* __restrict__ Ah = (const __nv_bfloat16*)g.A;
    const __nv_bfloat16* __restrict__ Al = (const __nv_bfloat16*)g.A2;
    const __nv_bfloat16* __restrict__ Bh = (const __nv_bfloat16*)g.B;
    const __nv_bfloat16* __restrict__ Bl = (const __nv_bfloat16*)g.B2;

    if (tid == 0) {
        s_fail = 0;
        for (int s = 0; s < STAGES; ++s) mbar_init(su32(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    int nsteps = 0;
    for (int s = tile.seg_begin; s < tile.seg_end; ++s) nsteps += (g.segs[s].K + BK - 1) / BK;

    // producer cursor (segment, k offset)
    int lseg = tile.seg_begin, lk0 = 0;
    GSeg lsg{};
    int64_t laoff = 0;
    if (lseg < tile.seg_end) { lsg = g.segs[lseg]; laoff = g.terms[lsg.term_begin].off; }
    // 3072 16-byte chunks per stage: A hi, A lo (128 rows x 8), B hi, B lo (64 rows x 8)
    auto load_step = [&](int stage) {
        const uint32_t sb = ring_s + stage * STAGE_BYTES;
#pragma unroll 4
        for (int i = 0; i < 24; ++i) {
            const int cid = tid + NT * i;
            int part, r, c;
            if (cid < 2048) { part = cid >> 10; r = (cid >> 3) & 127; c = cid & 7; }
            else { const int c2 = cid - 2048; part = 2 + (c2 >> 9); r = (c2 >> 3) & 63; c = c2 & 7; }
            const int k = lk0 + c * 8;
            const bool isA = part < 2;
            const bool ok = (isA ? r < mrem : r < nrem) && k < lsg.K;
            const __nv_bfloat16* src;
            uint32_t dst;
            if (isA) {
                src = (part == 0 ? Ah : Al) + laoff + (int64_t)(tile.row0 + (ok ? r : 0)) * lsg.lda + (ok ? k : 0);
                dst = sb + part * A_BYTES + swz(r, c);
            } else {
                src = (part == 2 ? Bh : Bl) + lsg.b_off + (int64_t)(tile.col0 + (ok ? r : 0)) * lsg.ldb + (ok ? k : 0);
                dst = sb + 2 * A_BYTES + (part - 2) * B_BYTES + swz(r, c);
            }
            cp16(dst, src, ok ? 16 : 0);
        }
        lk0 += BK;
        if (lk0 >= lsg.K) {
            lk0 = 0;
            if (++lseg < tile.seg_end) { lsg = g.segs[lseg]; laoff = g.terms[lsg.term_begin].off; }
        }
    };

#pragma unroll 1
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < nsteps) load_step(s);
        cp_commit();
    }
    // Per step: (A) the step's slices have landed in every thread -> thread 0
    // queues the step's MMAs and commits them to the stage barrier, then waits
    // (bounded) for the previous step's MMAs, whose stage is refilled next ->
    // (B) everyone refills that stage.  The wait comes after the new MMAs are
    // queued, so the tensor pipe never drains between steps.
#pragma unroll 1
    for (int step = 0; step < nsteps; ++step) {
        const int st = step % STAGES;
        const int nxt = step + STAGES - 1;
        cp_wait<STAGES - 2>();
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");   // cp.async data -> async proxy
        __syncthreads();                                                  // (A)
        if (tid == 0) {
            tc_fence_after();
            const uint32_t sb = ring_s + st * STAGE_BYTES;
            const uint64_t ah = sw128_desc(sb), al = sw128_desc(sb + A_BYTES);
            const uint64_t bh = sw128_desc(sb + 2 * A_BYTES), bl = sw128_desc(sb + 2 * A_BYTES + B_BYTES);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint64_t adv = (uint64_t)(kk * 32) >> 4;   // 16 bf16 = 32 bytes along K
                umma_bf16(tmem, al + adv, bh + adv, (step | kk) != 0);
                umma_bf16(tmem, ah + adv, bl + adv, 1);
                umma_bf16(tmem, ah + adv, bh + adv, 1);
            }
            umma_commit(su32(&bars[st]));
            if (step >= 1 && nxt < nsteps) {
                const int ps = (step - 1) % STAGES;
                if (!mbar_wait(su32(&bars[ps]), (uint32_t)(((step - 1) / STAGES) & 1))) s_fail = 1;
            }
        }
        __syncthreads();                                                  // (B)
        if (s_fail) break;
        if (nxt < nsteps) load_step(nxt % STAGES);
        cp_commit();
    }
    if (tid == 0 && nsteps > 0 && !s_fail) {
        const int ls = (nsteps - 1) % STAGES;
        if (!mbar_wait(su32(&bars[ls]), (uint32_t)(((nsteps - 1) / STAGES) & 1))) s_fail = 1;
    }
    cp_wait<0>();
    __syncthreads();
    tc_fence_after();
    const bool bad = s_fail != 0;
    if (bad && tid == 0 && g.err) atomicOr(g.err, 1);

    // epilogue: warp w owns accumulator lanes (rows) 32w .. 32w+31
    const int r = warp * 32 + lane;
#pragma unroll 1
    for (int j0 = 0; j0 < BN; j0 += 16) {
        float v[16];
        if (nsteps > 0 && !bad) {
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)j0, v);
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = 0.f;
        }
        if (r >= mrem || j0 >= nrem) continue;
        const int64_t gr = tile.row0 + r;
        if (OUT_SPLIT) {
            __nv_bfloat16* Ch = (__nv_bfloat16*)g.C;
            __nv_bfloat16* Cl = (__nv_bfloat16*)g.C2;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int c = j0 + i;
                if (c >= nrem) break;
                const int64_t gc = tile.col0 + c;
                const int64_t e = g.transC ? (gc + gr * tile.ldc) : (gr + gc * tile.ldc);
                const __nv_bfloat16 h = __float2bfloat16_rn(v[i]);
                Ch[tile.c_off + e] = h;
                Cl[tile.c_off + e] = __float2bfloat16_rn(v[i] - __bfloat162float(h));
            }
        } else {
            double* C = (double*)g.C;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int c = j0 + i;
                if (c >= nrem) break;
                const int64_t gc = tile.col0 + c;
                const int64_t e = g.transC ? (gc + gr * tile.ldc) : (gr + gc * tile.ldc);
                C[tile.c_off + e] = (double)v[i];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS));
}

cudaError_t umma_init() {
    cudaError_t e = cudaFuncSetAttribute(gg_umma_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, um::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(gg_umma_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, um::SMEM_BYTES);
}

cudaError_t launch_gg_umma(int out_split, const GGArgs& a, cudaStream_t st) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (out_split) gg_umma_kernel<1><<<a.ntiles, um::NT, um::SMEM_BYTES, st>>>(a);
    else gg_umma_kernel<0><<<a.ntiles, um::NT, um::SMEM_BYTES, st>>>(a);
    return cudaGetLastError();
}

}  // namespace vmps
