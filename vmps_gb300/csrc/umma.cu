// tcgen05 (UMMA) engine of the split-precision grouped GEMM (sm_103a).
//
// Same work lists as gg_split_kernel in kernels.cu.  Operands are pre-split
// into bf16 hi and lo halves of one arena ([hi | lo]), stored K-contiguous
// (rows of A, columns of B, row stride a multiple of 8 elements).  Every
// prepared block has a TMA descriptor (K, rows, hi/lo) built on the host, so a
// K step of one operand is one 3-d box copy that lands both halves in the
// 128-byte-swizzled K-major layout the UMMA shared-memory descriptors read,
// with zeros outside the block.  Tiles are up to 128 x 64 (UMMA M = 128,
// N = 64, K = 16 per instruction), accumulated in FP32 in tensor memory.
//
// Every barrier wait is bounded by a clock budget; when one runs out the
// kernel records it in the error word, the roles leave their loops, the tensor
// memory is released and the kernel returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.hpp"

namespace vmps {
namespace um {
constexpr int BM = 128, BN = 64, BK = 64, STAGES = 4;
constexpr int NT = 192;                                    // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr int A_BYTES = BM * BK * 2;                       // one of A hi / A lo: 16 KB
constexpr int B_BYTES = BN * BK * 2;                       // one of B hi / B lo: 8 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;     // 48 KB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr uint32_t ACC_COLS = 64;                          // one FP32 accumulator: 128 lanes x 64 columns
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;               // two, so an epilogue overlaps the next tile
// kind::f16 instruction descriptor: D FP32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);
constexpr long long WAIT_BUDGET = 4000000000LL;           // clock cycles (~2 s) per barrier wait
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
// wait for the phase of the given parity, bounded by the clock budget only
// (used to drain copies and MMAs in flight before the CTA exits)
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity, volatile int* fail) {
    const long long t0 = clock64();
    while (!mbar_test(bar, parity))
        if (clock64() - t0 > um::WAIT_BUDGET) { *fail = 1; return; }
}
// bounded wait on the phase of the given parity; false when the clock budget ran
// out or another role has already given up (the failure word is then set)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* fail) {
    const long long t0 = clock64();
    while (!mbar_test(bar, parity)) {
        if (*fail) return false;
        if (clock64() - t0 > um::WAIT_BUDGET) { *fail = 1; return false; }
    }
    return true;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
// 3-d tile copy (K, rows, hi/lo) global -> shared, completion counted on an mbarrier
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const void* tmap, int x, int y, int z, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(dst),
        "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// descriptors are written to global memory by the host, and a later plan may reuse
// an address: acquire the current contents for the tensor-map proxy before use
__device__ __forceinline__ void tmap_acquire(const void* tmap) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(tmap) : "memory");
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

__device__ __forceinline__ int tile_steps(const GGArgs& g, const GTile& t) {
    int n = 0;
    for (int s = t.seg_begin; s < t.seg_end; ++s) n += (g.segs[s].K + um::BK - 1) / um::BK;
    return n;
}

// Persistent, warp-specialised grouped GEMM on pre-split operands.
//   warp 0 (one lane): TMA loads of each 64-wide K step -- one 3-d box (K, rows,
//     hi/lo) per operand, 128-byte swizzle, zero fill outside the block -- into
//     a 4-deep ring of stages ("full" barriers carry the byte count);
//   warp 1 (one lane): per K step 4 x (lo*hi, hi*lo, hi*hi) tcgen05.mma into one
//     of two TMEM accumulators, commit to the stage's "empty" barrier, and at
//     the end of a tile to the accumulator's "full" barrier;
//   warps 2-5: epilogue -- tcgen05.ld of their 32 accumulator lanes, store,
//     release the accumulator -- overlapping the next tile's main loop.
// CTAs take tiles b, b + gridDim.x, ... (tiles are sorted by descending work).
template <int OUT_SPLIT>
__global__ void __launch_bounds__(um::NT, 1) gg_umma_kernel(GGArgs g) {
    using namespace um;
    extern __shared__ __align__(1024) unsigned char smraw[];
    const uint32_t raw = su32(smraw);
    const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
    const uint32_t ring = raw + pad;   // 1024-aligned: the swizzle pattern is anchored to 1024-byte boundaries
    uint64_t* bars = reinterpret_cast<uint64_t*>(smraw + pad + STAGES * STAGE_BYTES);
    // bars[0..S) full, [S..2S) empty, [2S..2S+2) accumulator full, [2S+2..2S+4) accumulator empty,
    // [2S+4] drain of the MMAs issued
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
    __shared__ volatile int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    auto bar = [&](int i) { return su32(&bars[i]); };

    if (tid == 0) {
        s_fail = 0;
        for (int s = 0; s < STAGES; ++s) { mbar_init(bar(s), 1); mbar_init(bar(STAGES + s), 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(bar(2 * STAGES + b), 1); mbar_init(bar(2 * STAGES + 2 + b), 4); }
        mbar_init(bar(2 * STAGES + 4), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int G = gridDim.x;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        const char* amaps = (const char*)g.amaps;
        const char* bmaps = (const char*)g.bmaps;
        int it = 0;
        const void* last_a = nullptr;
        const void* last_b = nullptr;
        for (int t = blockIdx.x; t < g.ntiles && !s_fail; t += G) {
            const GTile tile = g.tiles[t];
            for (int s = tile.seg_begin; s < tile.seg_end && !s_fail; ++s) {
                const int K = g.segs[s].K;
                const void* am = amaps + (size_t)g.seg_amap[s] * 128;
                const void* bm = bmaps + (size_t)g.seg_bmap[s] * 128;
                if (am != last_a) { tmap_acquire(am); last_a = am; }
                if (bm != last_b) { tmap_acquire(bm); last_b = bm; }
                for (int k0 = 0; k0 < K; k0 += BK, ++it) {
                    const int st = it % STAGES, use = it / STAGES;
                    if (use >= 1 && !mbar_wait(bar(STAGES + st), (uint32_t)((use - 1) & 1), &s_fail)) break;
                    const uint32_t sb = ring + st * STAGE_BYTES;
                    mbar_expect_tx(bar(st), STAGE_BYTES);
                    tma_load_3d(sb, am, k0, tile.row0, 0, bar(st));
                    tma_load_3d(sb + 2 * A_BYTES, bm, k0, tile.col0, 0, bar(st));
                }
            }
        }
        // copies still in flight land before the CTA exits (a no-op when the MMA warp consumed them)
        for (int i = it - 1; i >= 0 && i >= it - STAGES; --i)
            mbar_drain(bar(i % STAGES), (uint32_t)((i / STAGES) & 1), &s_fail);
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        int it = 0, lt = 0;
        for (int t = blockIdx.x; t < g.ntiles && !s_fail; t += G, ++lt) {
            const GTile tile = g.tiles[t];
            const int buf = lt & 1, buse = lt >> 1;
            if (buse >= 1 && !mbar_wait(bar(2 * STAGES + 2 + buf), (uint32_t)((buse - 1) & 1), &s_fail)) break;
            tc_fence_after();
            const uint32_t dacc = tmem + (uint32_t)buf * ACC_COLS;
            bool first = true;
            const int nsteps = tile_steps(g, tile);
            for (int k = 0; k < nsteps; ++k, ++it) {
                const int st = it % STAGES, use = it / STAGES;
                if (!mbar_wait(bar(st), (uint32_t)(use & 1), &s_fail)) break;
                tc_fence_after();
                const uint32_t sb = ring + st * STAGE_BYTES;
                const uint64_t ah = sw128_desc(sb), al = sw128_desc(sb + A_BYTES);
                const uint64_t bh = sw128_desc(sb + 2 * A_BYTES), bl = sw128_desc(sb + 2 * A_BYTES + B_BYTES);
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
                    const uint64_t adv = (uint64_t)(kk * 32) >> 4;   // 16 bf16 = 32 bytes along K
                    umma_bf16(dacc, al + adv, bh + adv, first ? 0u : 1u);
                    first = false;
                    umma_bf16(dacc, ah + adv, bl + adv, 1);
                    umma_bf16(dacc, ah + adv, bh + adv, 1);
                }
                umma_commit(bar(STAGES + st));
            }
            umma_commit(bar(2 * STAGES + buf));
        }
        umma_commit(bar(2 * STAGES + 4));
        mbar_drain(bar(2 * STAGES + 4), 0, &s_fail);
    } else if (warp >= 2) {
        // ---------------- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31
        const int sp = warp & 3;
        const int r = sp * 32 + lane;
        int lt = 0;
        for (int t = blockIdx.x; t < g.ntiles; t += G, ++lt) {
            const GTile tile = g.tiles[t];
            const int buf = lt & 1, buse = lt >> 1;
            // warp-uniform outcome: the tensor-memory loads below are warp-collective
            const bool ok = __all_sync(0xffffffffu, mbar_wait(bar(2 * STAGES + buf), (uint32_t)(buse & 1), &s_fail));
            if (!ok) break;
            tc_fence_after();
            const bool any = tile.seg_end > tile.seg_begin;
            const int mrem = tile.tm, nrem = tile.tn;
            const int64_t gr = tile.row0 + r;
#pragma unroll 1
            for (int j0 = 0; j0 < BN; j0 += 16) {
                float v[16];
                if (any) tmem_ld16(tmem + ((uint32_t)(sp * 32) << 16) + (uint32_t)(buf * ACC_COLS + j0), v);
                else {
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = 0.f;
                }
                if (r >= mrem || j0 >= nrem) continue;
                const int64_t gc0 = tile.col0 + j0;
                if (OUT_SPLIT) {
                    __nv_bfloat16* Ch = (__nv_bfloat16*)g.C;
                    __nv_bfloat16* Cl = (__nv_bfloat16*)g.C2;
                    if (g.transC && j0 + 16 <= nrem) {   // 16 consecutive elements of one row: two 16-byte stores
                        uint32_t h[8], l[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * i]), h1 = __float2bfloat16_rn(v[2 * i + 1]);
                            const __nv_bfloat16 l0 = __float2bfloat16_rn(v[2 * i] - __bfloat162float(h0));
                            const __nv_bfloat16 l1 = __float2bfloat16_rn(v[2 * i + 1] - __bfloat162float(h1));
                            h[i] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
                            l[i] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
                        }
                        const int64_t e = tile.c_off + gc0 + gr * tile.ldc;
                        uint4* ph = reinterpret_cast<uint4*>(Ch + e);
                        uint4* pl = reinterpret_cast<uint4*>(Cl + e);
                        ph[0] = make_uint4(h[0], h[1], h[2], h[3]);
                        ph[1] = make_uint4(h[4], h[5], h[6], h[7]);
                        pl[0] = make_uint4(l[0], l[1], l[2], l[3]);
                        pl[1] = make_uint4(l[4], l[5], l[6], l[7]);
                    } else {
#pragma unroll
                        for (int i = 0; i < 16; ++i) {
                            if (j0 + i >= nrem) break;
                            const int64_t gc = gc0 + i;
                            const int64_t e = tile.c_off + (g.transC ? (gc + gr * tile.ldc) : (gr + gc * tile.ldc));
                            const __nv_bfloat16 hh = __float2bfloat16_rn(v[i]);
                            Ch[e] = hh;
                            Cl[e] = __float2bfloat16_rn(v[i] - __bfloat162float(hh));
                        }
                    }
                } else {
                    double* C = (double*)g.C;
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        if (j0 + i >= nrem) break;
                        const int64_t gc = gc0 + i;
                        C[tile.c_off + (g.transC ? (gc + gr * tile.ldc) : (gr + gc * tile.ldc))] = (double)v[i];
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(2 * STAGES + 2 + buf));
        }
    }
    __syncthreads();
    if (s_fail && tid == 0 && g.err) atomicOr(g.err, 1);
    tc_fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS));
}

static int g_num_sms = 0;

cudaError_t umma_init() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(gg_umma_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, um::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(gg_umma_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, um::SMEM_BYTES);
}

cudaError_t launch_gg_umma(int out_split, const GGArgs& a, cudaStream_t st) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (!a.amaps || !a.bmaps || !a.seg_amap || !a.seg_bmap) return cudaErrorInvalidValue;
    const int grid = a.ntiles < g_num_sms ? a.ntiles : (g_num_sms > 0 ? g_num_sms : 148);
    if (out_split) gg_umma_kernel<1><<<grid, um::NT, um::SMEM_BYTES, st>>>(a);
    else gg_umma_kernel<0><<<grid, um::NT, um::SMEM_BYTES, st>>>(a);
    return cudaGetLastError();
}

}  // namespace vmps
