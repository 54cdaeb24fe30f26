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

#include "convert.hpp"
#include "kernels.hpp"

namespace vmps {
namespace um {
constexpr int BM = kUmmaTileM, BN = kUmmaTileN, BK = kUmmaBK, STAGES = 4;   // 128 x (<= 256) x 32
constexpr int NT = 192;                                    // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr int ROW_BYTES = BK * 2;                          // one K step of one row: 64 bytes
constexpr int A_BYTES = BM * ROW_BYTES;                    // one of A hi / A lo: 8 KB
constexpr int B_BYTES = BN * ROW_BYTES;                    // one of B hi / B lo, at most: 16 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;     // 48 KB
constexpr int STAGE_OUT_BYTES = 4 * 8192;                  // split-output epilogue: 32 rows x 64 cols x hi/lo per warp
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + STAGE_OUT_BYTES + 1024 + 256;
constexpr uint32_t ACC_COLS = BN;                          // one FP32 accumulator: 128 lanes x 256 columns
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;               // two (all of TMEM), so an epilogue overlaps the next tile
// kind::f16 instruction descriptor: D FP32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22 (per tile), M >> 4 in bits 24-28
constexpr uint32_t IDESC_BASE = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BM >> 4) << 24);
constexpr long long WAIT_BUDGET = 4000000000LL;           // clock cycles (~2 s) per barrier wait
constexpr int LOOKAHEAD = STAGES;                          // descriptors acquired this many steps ahead
}  // namespace um

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 64-byte swizzle (rows of one 32-element
// K step), 8-row groups 512 B apart
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);   // start address >> 4
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;           // stride byte offset between 8-row groups
    d |= (uint64_t)1 << 46;                    // descriptor version (tcgen05)
    d |= (uint64_t)4 << 61;                    // 64-byte swizzle
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

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// 32 lanes x 16 consecutive 32-bit columns of tensor memory (completion: tmem_wait_ld)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
// registers loaded by tmem_ld16 are read only after tmem_wait_ld: this empty
// statement redefines them in program order after the wait
__device__ __forceinline__ void reg_fence16(uint32_t* r) {
    asm volatile(""
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]));
}

__device__ __forceinline__ void tmap_prefetch(const void* tmap) {
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(tmap) : "memory");
}
// first use of a descriptor by this CTA: acquire it for the tensor-map proxy and
// start fetching it
__device__ __forceinline__ void acquire_step(const GGArgs& g, int j) {
    const TStep s = g.steps[j];
    if (s.flags & 1) {
        const void* m = (const char*)g.amaps + (size_t)s.amap * 128;
        tmap_acquire(m);
        tmap_prefetch(m);
    }
    if (s.flags & 2) {
        const void* m = (const char*)g.bmaps + (size_t)s.bmap * 128;
        tmap_acquire(m);
        tmap_prefetch(m);
    }
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}

// Persistent, warp-specialised grouped GEMM on pre-split operands.  CTA b runs
// tiles[cta_tiles[b] .. cta_tiles[b+1]) (a host-side longest-first schedule),
// whose K steps are steps[tiles[.].step0 ...], contiguous per CTA.
//   warp 0 (one lane): per step one TMA 3-d box (K, rows, hi/lo) of A and one
//     of B -- 128-byte swizzle, zero fill outside the block -- into a 4-deep
//     ring of stages ("full" barriers count the bytes); descriptors are
//     acquired and prefetched LOOKAHEAD steps ahead of their first use;
//   warp 1 (one lane): per step 4 x (lo*hi, hi*lo, hi*hi) tcgen05.mma into one
//     of two TMEM accumulators, commit to the stage's "empty" barrier, and at
//     the end of a tile to the accumulator's "full" barrier;
//   warps 2-5: epilogue of their 32 accumulator lanes, overlapping the next
//     tile's main loop.  A split (bf16 hi/lo, row-major) output is staged
//     through swizzled shared memory so that global stores are whole rows.
template <int OUT_SPLIT>
__global__ void __launch_bounds__(um::NT, 1) gg_umma_kernel(GGArgs g) {
    using namespace um;
    extern __shared__ __align__(1024) unsigned char smraw[];
    const uint32_t raw = su32(smraw);
    const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
    const uint32_t ring = raw + pad;   // 1024-aligned: the swizzle pattern is anchored to 1024-byte boundaries
    unsigned char* stage_out = smraw + pad + STAGES * STAGE_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(stage_out + STAGE_OUT_BYTES);
    // bars[0..S) full, [S..2S) empty, [2S..2S+2) accumulator full, [2S+2..2S+4) accumulator empty,
    // [2S+4] drain of the MMAs issued
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
    volatile int* s_fail = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    auto bar = [&](int i) { return su32(&bars[i]); };

    if (tid == 0) {
        *s_fail = 0;
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
    const int t0 = g.cta_tiles[blockIdx.x], t1 = g.cta_tiles[blockIdx.x + 1];

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        const char* amaps = (const char*)g.amaps;
        const char* bmaps = (const char*)g.bmaps;
        int S0 = 0, S1 = 0;
        if (t0 < t1) {
            S0 = g.tiles[t0].step0;
            S1 = g.tiles[t1 - 1].step0 + g.tiles[t1 - 1].nsteps;
        }
        for (int j = S0; j < S1 && j < S0 + LOOKAHEAD; ++j) acquire_step(g, j);
        int it = 0;
        for (int j = S0; j < S1 && !*s_fail; ++j, ++it) {
            if (j + LOOKAHEAD < S1) acquire_step(g, j + LOOKAHEAD);
            const TStep s = g.steps[j];
            const int st = it % STAGES, use = it / STAGES;
            if (use >= 1 && !mbar_wait(bar(STAGES + st), (uint32_t)((use - 1) & 1), s_fail)) break;
            const uint32_t sb = ring + st * STAGE_BYTES;
            mbar_expect_tx(bar(st), (uint32_t)(2 * A_BYTES + 2 * s.brows * ROW_BYTES));
            tma_load_3d(sb, amaps + (size_t)s.amap * 128, s.k0, s.row0, 0, bar(st));
            tma_load_3d(sb + 2 * A_BYTES, bmaps + (size_t)s.bmap * 128, s.k0, s.col0, 0, bar(st));
        }
        // copies still in flight land before the CTA exits (a no-op when the MMA warp consumed them)
        for (int i = it - 1; i >= 0 && i >= it - STAGES; --i)
            mbar_drain(bar(i % STAGES), (uint32_t)((i / STAGES) & 1), s_fail);
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        int it = 0, lt = 0;
        for (int t = t0; t < t1 && !*s_fail; ++t, ++lt) {
            const GTile tile = g.tiles[t];
            const int nsteps = tile.nsteps;
            const int brows = nsteps > 0 ? g.steps[tile.step0].brows : 16;
            const uint32_t idesc = IDESC_BASE | ((uint32_t)(((tile.tn + 15) & ~15) >> 3) << 17);   // N = round16(tn)
            const int buf = lt & 1, buse = lt >> 1;
            if (buse >= 1 && !mbar_wait(bar(2 * STAGES + 2 + buf), (uint32_t)((buse - 1) & 1), s_fail)) break;
            tc_fence_after();
            const uint32_t dacc = tmem + (uint32_t)buf * ACC_COLS;
            for (int k = 0; k < nsteps; ++k, ++it) {
                const int st = it % STAGES, use = it / STAGES;
                if (!mbar_wait(bar(st), (uint32_t)(use & 1), s_fail)) break;
                tc_fence_after();
                const uint32_t sb = ring + st * STAGE_BYTES;
                const uint64_t ah = sw64_desc(sb), al = sw64_desc(sb + A_BYTES);
                const uint64_t bh = sw64_desc(sb + 2 * A_BYTES), bl = sw64_desc(sb + 2 * A_BYTES + brows * ROW_BYTES);
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
                    const uint64_t adv = (uint64_t)(kk * 32) >> 4;   // 16 bf16 = 32 bytes along K
                    umma_bf16(dacc, al + adv, bh + adv, idesc, (k | kk) != 0 ? 1u : 0u);
                    umma_bf16(dacc, ah + adv, bl + adv, idesc, 1);
                    umma_bf16(dacc, ah + adv, bh + adv, idesc, 1);
                }
                umma_commit(bar(STAGES + st));
            }
            umma_commit(bar(2 * STAGES + buf));
        }
        umma_commit(bar(2 * STAGES + 4));
        mbar_drain(bar(2 * STAGES + 4), 0, s_fail);
    } else if (warp >= 2) {
        // ---------------- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31
        const int sp = warp & 3;
        const int rl = sp * 32 + lane;   // tile row of this lane
        unsigned char* so = stage_out + (warp - 2) * 8192;   // this warp's staging: hi rows, then lo rows
        int lt = 0;
        for (int t = t0; t < t1; ++t, ++lt) {
            const GTile tile = g.tiles[t];
            const int buf = lt & 1, buse = lt >> 1;
            // warp-uniform outcome: the tensor-memory loads below are warp-collective
            const bool ok = __all_sync(0xffffffffu, mbar_wait(bar(2 * STAGES + buf), (uint32_t)(buse & 1), s_fail));
            if (!ok) break;
            tc_fence_after();
            const int ncols = tile.tn;
#pragma unroll 1
            for (int c0 = 0; c0 < ncols; c0 += 64) {
                uint32_t v[64];
                if (tile.nsteps > 0) {
                    const uint32_t ta = tmem + ((uint32_t)(sp * 32) << 16) + (uint32_t)(buf * ACC_COLS + c0);
                    tmem_ld16(ta, v);
                    tmem_ld16(ta + 16, v + 16);
                    tmem_ld16(ta + 32, v + 32);
                    tmem_ld16(ta + 48, v + 48);
                    tmem_wait_ld();
                    reg_fence16(v);
                    reg_fence16(v + 16);
                    reg_fence16(v + 32);
                    reg_fence16(v + 48);
                } else {
#pragma unroll
                    for (int i = 0; i < 64; ++i) v[i] = 0u;
                }
                if (c0 + 64 >= ncols) {
                    // the accumulator is free once its last columns sit in registers
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(bar(2 * STAGES + 2 + buf));
                }
                const int tn = ncols - c0 < 64 ? ncols - c0 : 64;   // columns of this chunk
                const int col0 = tile.col0 + c0;
                if (OUT_SPLIT) {
                    // row-major bf16 hi / lo: stage 32 rows x 64 columns (chunk c of row r at
                    // r*128 + ((c ^ (r & 7)) << 4)), then store 4 whole 128-byte rows per instruction
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        uint32_t h[4], l[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const float a = __uint_as_float(v[c * 8 + 2 * i]), b = __uint_as_float(v[c * 8 + 2 * i + 1]);
                            const float ha = __bfloat162float(__float2bfloat16_rn(a));
                            const float hb = __bfloat162float(__float2bfloat16_rn(b));
                            h[i] = pack_bf16x2(a, b);
                            l[i] = pack_bf16x2(a - ha, b - hb);
                        }
                        const int off = lane * 128 + ((c ^ (lane & 7)) << 4);
                        *reinterpret_cast<uint4*>(so + off) = make_uint4(h[0], h[1], h[2], h[3]);
                        *reinterpret_cast<uint4*>(so + 4096 + off) = make_uint4(l[0], l[1], l[2], l[3]);
                    }
                    __syncwarp();
                    __nv_bfloat16* Ch = (__nv_bfloat16*)g.C;
                    __nv_bfloat16* Cl = (__nv_bfloat16*)g.C2;
                    const int c = lane & 7;
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int row = i * 4 + (lane >> 3);
                        const int off = row * 128 + ((c ^ (row & 7)) << 4);
                        const uint4 hv = *reinterpret_cast<const uint4*>(so + off);
                        const uint4 lv = *reinterpret_cast<const uint4*>(so + 4096 + off);
                        if (sp * 32 + row < tile.tm && c * 8 < tn) {
                            const int64_t e = tile.c_off + (int64_t)(tile.row0 + sp * 32 + row) * tile.ldc + col0 + c * 8;
                            *reinterpret_cast<uint4*>(Ch + e) = hv;
                            *reinterpret_cast<uint4*>(Cl + e) = lv;
                        }
                    }
                    __syncwarp();   // the staging area is rewritten by the next chunk
                } else {
                    double* C = (double*)g.C;
                    if (rl < tile.tm) {
                        const int64_t gr = tile.row0 + rl;
#pragma unroll
                        for (int j = 0; j < 64; ++j) {
                            if (j < tn) {
                                const int64_t gc = col0 + j;
                                C[tile.c_off + (g.transC ? (gc + gr * tile.ldc) : (gr + gc * tile.ldc))] =
                                    f32_to_f64(__uint_as_float(v[j]));
                            }
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    if (*s_fail && tid == 0 && g.err) atomicOr(g.err, 1);
    tc_fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS));
}

cudaError_t umma_init() {
    cudaError_t e = cudaFuncSetAttribute(gg_umma_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, um::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(gg_umma_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, um::SMEM_BYTES);
}

cudaError_t launch_gg_umma(int out_split, const GGArgs& a, cudaStream_t st) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (!a.amaps || !a.bmaps || !a.steps || !a.cta_tiles || a.ncta <= 0) return cudaErrorInvalidValue;
    if (out_split && !a.transC) return cudaErrorInvalidValue;   // the staged epilogue writes row-major tiles
    const int grid = a.ncta;
    if (out_split) gg_umma_kernel<1><<<grid, um::NT, um::SMEM_BYTES, st>>>(a);
    else gg_umma_kernel<0><<<grid, um::NT, um::SMEM_BYTES, st>>>(a);
    return cudaGetLastError();
}

}  // namespace vmps
