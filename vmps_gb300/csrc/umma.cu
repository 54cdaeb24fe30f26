// tcgen05 (UMMA) engine of the split-precision (BF16x3) grouped GEMM (sm_103a).
//
// Operands live in bf16 panels (engine.hpp): rows of A / of B, each 128-byte
// row segment holding the hi and lo halves of one 32-wide K step.  A K step of
// an operand is one 2-d TMA box of that panel (x = 2*k0, y = panel row, box
// 64 elements x 16..256 rows) landing in the 128-byte-swizzled K-major layout
// the UMMA shared-memory descriptors read: hi at K slices 0-1 of each row, lo
// at K slices 2-3.  TMA descriptors, one per (panel class, box height), are a
// grid-constant kernel parameter.  Tiles are up to 128 x 256 (UMMA M = 128,
// N = round16(tile width), K = 16 per instruction), accumulated in FP32 in
// tensor memory; per K step the products lo*hi + hi*lo + hi*hi.
//
// Panel rows next to a block belong to other blocks: they only reach rows or
// columns of the accumulator the epilogue never stores, and the split epilogue
// writes zeros past the tile width, so panel padding stays zero.
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
// warp 0 TMA, warp 1 MMA, then the epilogue warps: four for split (panel) outputs, whose
// staging takes 8 KB of shared memory per warp, eight (two per tensor-memory lane quadrant,
// alternate 64-column chunks) for FP32 / FP64 outputs
constexpr int epi_warps(int out_split) { return out_split == 1 ? 4 : 8; }
constexpr int nt_of(int out_split) { return 64 + 32 * epi_warps(out_split); }
constexpr int ROW_BYTES = 128;                             // one K step of one row: 32 hi + 32 lo
constexpr int A_BYTES = BM * ROW_BYTES;                    // A region: 16 KB
constexpr int B_BYTES = BN * ROW_BYTES;                    // B region, at most: 32 KB
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;             // 48 KB
constexpr int STAGE_OUT_BYTES = 4 * 8192;                  // split-output epilogue: 32 rows x 256 B per warp
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + STAGE_OUT_BYTES + 1024 + 256;
static_assert((2 * STAGES + 5) * 8 + 4 * (2 + STAGES) <= 256, "barrier area overflow");
constexpr uint32_t ACC_COLS = BN;                          // one FP32 accumulator: 128 lanes x 256 columns
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;               // two (all of TMEM), so an epilogue overlaps the next tile
// kind::f16 instruction descriptor: D FP32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22 (per tile), M >> 4 in bits 24-28
constexpr uint32_t IDESC_BASE = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BM >> 4) << 24);
// kind::tf32: the same with A and B TF32 (format 2 in bits 7-9 and 10-12)
constexpr uint32_t IDESC_BASE_TF32 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BM >> 4) << 24);
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
// out or another role has already given up (the failure word is then set).
// budget: clock cycles (the main loops pass the kernel's budget; drains use WAIT_BUDGET)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* fail, long long budget) {
    const long long t0 = clock64();
    while (!mbar_test(bar, parity)) {
        if (*fail) return false;
        if (clock64() - t0 > budget) { *fail = 1; return false; }
    }
    return true;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
// 2-d tile copy (panel columns, panel rows) global -> shared, completion counted on an mbarrier
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void* tmap, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(dst),
        "l"(tmap), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
// TF32 operands (FP32 storage): K = 8 per instruction, 32 bytes along K like a bf16 K16 slice
__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ float to_tf32_rna(float v) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
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

__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];\n" ::"l"(p));
}
// one 32-byte step record through the read-only path
__device__ __forceinline__ TStep load_step(const TStep* p) {
    const int4 a = __ldg(reinterpret_cast<const int4*>(p));
    const int4 b = __ldg(reinterpret_cast<const int4*>(p) + 1);
    TStep s;
    s.amap = a.x; s.bmap = a.y; s.x = a.z; s.ay = a.w;
    s.by = b.x; s.arows = b.y; s.brows = b.z; s.xa = b.w;
    return s;
}
__device__ __forceinline__ void tmap_prefetch(const void* tmap) {
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(tmap) : "memory");
}

// Persistent, warp-specialised grouped GEMM on panel operands.  CTA b runs
// tiles[cta_tiles[b] .. cta_tiles[b+1]) (a host-side longest-first schedule),
// whose K steps are steps[tiles[.].step0 ...], contiguous per CTA.
//   warp 0, lane 0: per step one TMA box of A and one of B into a 4-deep ring of
//     stages ("full" barriers count the bytes), the step records read through L1
//     and prefetched ahead;
//   warp 1 (one lane): per step 2 x (lo*hi, hi*lo, hi*hi) tcgen05.mma into one
//     of two TMEM accumulators, commit to the stage's "empty" barrier, and at
//     the end of a tile to the accumulator's "full" barrier;
//   warps 2..: epilogue of their 32 accumulator lanes in 64-column chunks,
//     overlapping the next tile's main loop.  A split output (T panels) is
//     staged through swizzled shared memory so that each panel row segment is
//     one 256-byte store (four warps); FP32 / FP64 outputs have two warps per
//     lane quadrant, taking alternate chunks (eight warps).
// TF32: the operands are 3xTF32 panels (FP32 [16 hi | 16 lo] per 128-byte row segment, a K step
// of 16), the MMAs kind::tf32 with K = 8; the shared-memory layout of a stage is the same bytes.
template <int OUT_SPLIT, bool MULTI, bool TF32 = false>
__global__ void __launch_bounds__(um::nt_of(OUT_SPLIT), 1)
    gg_umma_kernel(const GGArgs g, const __grid_constant__ TmaMaps maps) {
    using namespace um;
    constexpr int EPI = epi_warps(OUT_SPLIT);
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
        for (int b = 0; b < 2; ++b) { mbar_init(bar(2 * STAGES + b), 1); mbar_init(bar(2 * STAGES + 2 + b), EPI); }
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
    // main-loop waits give up after wb cycles; the drains before exit keep the full budget
    const long long wb = g.wait_budget > 0 ? g.wait_budget : WAIT_BUDGET;

    if (warp == 0) {
        // ---------------- TMA producer: one lane walks the CTA's K steps; their records
        // come through L1, each 128-byte line prefetched 16 steps ahead
        for (int i = lane; i < kMaxMapsA; i += 32) tmap_prefetch(&maps.a[i]);
        for (int i = lane; i < kMaxMapsB; i += 32) tmap_prefetch(&maps.b[i]);
        if (lane == 0) {
            int S0 = 0, S1 = 0;
            if (t0 < t1) {
                S0 = g.tiles[t0].step0;
                S1 = g.tiles[t1 - 1].step0 + g.tiles[t1 - 1].nsteps;
            }
            for (int j = S0 & ~3; j < S0 + 16 && j < S1; j += 4) prefetch_l1(g.steps + j);
            int it = 0;
            for (int j = S0; j < S1; ++j, ++it) {
                if (((j + 16) & 3) == 0 && j + 16 < S1) prefetch_l1(g.steps + j + 16);
                const TStep r = load_step(g.steps + j);
                const int st = it % STAGES, use = it / STAGES;
                if (use >= 1 && !mbar_wait(bar(STAGES + st), (uint32_t)((use - 1) & 1), s_fail, wb)) break;
                const uint32_t sb = ring + st * STAGE_BYTES;
                mbar_expect_tx(bar(st), (uint32_t)((r.arows + r.brows) * ROW_BYTES));
                tma_load_2d(sb, &maps.a[r.amap], r.xa, r.ay, bar(st));
                // bit 0 of x flags a step whose second K16 slice is padding
                tma_load_2d(sb + A_BYTES, &maps.b[r.bmap], r.x & ~1, r.by, bar(st));
            }
            // copies still in flight land before the CTA exits (a no-op when the MMA warp consumed them)
            for (int i = it - 1; i >= 0 && i >= it - STAGES; --i)
                mbar_drain(bar(i % STAGES), (uint32_t)((i / STAGES) & 1), s_fail);
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer (the next tile's record is fetched one tile ahead)
        int it = 0, lt = 0;
        GTile tile{};
        if (t0 < t1) tile = g.tiles[t0];
        for (int t = t0; t < t1 && !*s_fail; ++t, ++lt) {
            GTile next{};
            if (t + 1 < t1) next = g.tiles[t + 1];
            const int nsteps = tile.nsteps;
            const uint32_t idesc = (TF32 ? IDESC_BASE_TF32 : IDESC_BASE) |
                                   ((uint32_t)(((tile.tn + 15) & ~15) >> 3) << 17);   // N = round16(tn)
            const int buf = lt & 1, buse = lt >> 1;
            if (buse >= 1 && !mbar_wait(bar(2 * STAGES + 2 + buf), (uint32_t)((buse - 1) & 1), s_fail, wb)) break;
            tc_fence_after();
            const uint32_t dacc = tmem + (uint32_t)buf * ACC_COLS;
            for (int k = 0; k < nsteps; ++k, ++it) {
                const int st = it % STAGES, use = it / STAGES;
                if (!mbar_wait(bar(st), (uint32_t)(use & 1), s_fail, wb)) break;
                tc_fence_after();
                const uint32_t sb = ring + st * STAGE_BYTES;
                const uint64_t a = sw128_desc(sb), b = sw128_desc(sb + A_BYTES);
                // a padding half (zeros in A and B) adds nothing: its three MMAs are skipped
                const int nk16 = (__ldg(&g.steps[tile.step0 + k].x) & 1) ? 1 : BK / 16;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
                    if (kk >= nk16) break;
                    // 16 bf16 (or 8 tf32) = 32 bytes along K; the lo halves sit 64 bytes after the hi halves
                    const uint64_t hi = (uint64_t)(kk * 32) >> 4, lo = (uint64_t)(64 + kk * 32) >> 4;
                    if (TF32) {
                        umma_tf32(dacc, a + lo, b + hi, idesc, (k | kk) != 0 ? 1u : 0u);
                        umma_tf32(dacc, a + hi, b + lo, idesc, 1);
                        umma_tf32(dacc, a + hi, b + hi, idesc, 1);
                    } else {
                        umma_bf16(dacc, a + lo, b + hi, idesc, (k | kk) != 0 ? 1u : 0u);
                        umma_bf16(dacc, a + hi, b + lo, idesc, 1);
                        umma_bf16(dacc, a + hi, b + hi, idesc, 1);
                    }
                }
                umma_commit(bar(STAGES + st));
            }
            umma_commit(bar(2 * STAGES + buf));
            tile = next;
        }
        umma_commit(bar(2 * STAGES + 4));
        mbar_drain(bar(2 * STAGES + 4), 0, s_fail);
    } else if (warp >= 2) {
        // ---------------- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31
        const int sp = warp & 3;
        const int rl = sp * 32 + lane;   // tile row of this lane
        // chunks c0 = cfirst, cfirst + cstride, ... of every tile are this warp's
        const int cfirst = EPI == 8 ? ((warp - 2) >> 2) * 64 : 0, cstride = EPI == 8 ? 128 : 64;
        unsigned char* so = stage_out + (warp - 2) * 8192;   // this warp's staging: 32 rows x 256 B (split output)
        int lt = 0;
        for (int t = t0; t < t1; ++t, ++lt) {
            const GTile tile = g.tiles[t];
            const int buf = lt & 1, buse = lt >> 1;
            // warp-uniform outcome: the tensor-memory loads below are warp-collective
            const bool ok = __all_sync(0xffffffffu, mbar_wait(bar(2 * STAGES + buf), (uint32_t)(buse & 1), s_fail, wb));
            if (!ok) break;
            tc_fence_after();
            const int ncols = tile.tn;
            if (cfirst >= ncols) {
                // no chunk of this tile for this warp: its share of the accumulator is free
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(2 * STAGES + 2 + buf));
                continue;
            }
#pragma unroll 1
            for (int c0 = cfirst; c0 < ncols; c0 += cstride) {
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
                if (c0 + cstride >= ncols) {
                    // the accumulator is free once this warp's last columns sit in registers
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(bar(2 * STAGES + 2 + buf));
                }
                const int tn = ncols - c0 < 64 ? ncols - c0 : 64;   // columns of this chunk
                if (OUT_SPLIT == 1 && TF32) {
                    // 3xTF32 T panel rows: columns col0+c0 .. +63 are four 16-wide K steps, the
                    // 512-byte row segment [hi 0-15 | lo 0-15 | hi 16-31 | lo 16-31 | ...]; columns
                    // past the tile inside a written step are zeros.  Each lane writes its own row.
                    if (rl < tile.tm) {
                        float* C = (float*)g.C;
                        float* row = C + tile.c_off + (int64_t)(tile.row0 + rl) * tile.ldc +
                                     (int64_t)((tile.col0 + c0) >> 4) * 32;
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            // K steps past the tile are not written: they may lie beyond the
                            // panel row (its padded width is the block's K rounded up to 32)
                            if (q * 16 >= tn) break;
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                float h[4], l[4];
#pragma unroll
                                for (int i = 0; i < 4; ++i) {
                                    const int j = q * 16 + u * 4 + i;
                                    const float x = j < tn ? __uint_as_float(v[j]) : 0.f;
                                    h[i] = to_tf32_rna(x);
                                    l[i] = to_tf32_rna(x - h[i]);
                                }
                                *reinterpret_cast<float4*>(row + q * 32 + u * 4) = make_float4(h[0], h[1], h[2], h[3]);
                                *reinterpret_cast<float4*>(row + q * 32 + 16 + u * 4) =
                                    make_float4(l[0], l[1], l[2], l[3]);
                            }
                        }
                    }
                } else if (OUT_SPLIT == 1) {
                    // T panel rows: columns col0+c0 .. +63 are two 32-wide K steps, i.e. the
                    // 256-byte row segment [hi 0-31 | lo 0-31 | hi 32-63 | lo 32-63] (16-byte
                    // units u = 8q + 4h + g: K step q, half h, columns 8g..8g+7).  Columns past
                    // the tile are written as zeros.  Stage row r's unit u at r*256 + ((u ^ (r & 15)) << 4).
#pragma unroll
                    for (int cg = 0; cg < 8; ++cg) {
                        uint32_t h[4], l[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const int j = cg * 8 + 2 * i;
                            const float a = j < tn ? __uint_as_float(v[j]) : 0.f;
                            const float b = j + 1 < tn ? __uint_as_float(v[j + 1]) : 0.f;
                            // hi = bf16(x), lo = bf16(x - hi), two elements per conversion
                            const __nv_bfloat162 hv = __floats2bfloat162_rn(a, b);
                            const float2 hf = __bfloat1622float2(hv);
                            const __nv_bfloat162 lv = __floats2bfloat162_rn(a - hf.x, b - hf.y);
                            h[i] = *reinterpret_cast<const uint32_t*>(&hv);
                            l[i] = *reinterpret_cast<const uint32_t*>(&lv);
                        }
                        const int q = cg >> 2, gq = cg & 3;
                        const int uh = q * 8 + gq, ul = q * 8 + 4 + gq;
                        *reinterpret_cast<uint4*>(so + lane * 256 + ((uh ^ (lane & 15)) << 4)) = make_uint4(h[0], h[1], h[2], h[3]);
                        *reinterpret_cast<uint4*>(so + lane * 256 + ((ul ^ (lane & 15)) << 4)) = make_uint4(l[0], l[1], l[2], l[3]);
                    }
                    __syncwarp();
                    __nv_bfloat16* C = (__nv_bfloat16*)g.C;
                    const int u = lane & 15;
                    const int ucol = (u >> 3) * 32 + (u & 3) * 8;   // first column of unit u in the chunk
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int row = i * 2 + (lane >> 4);
                        const uint4 val = *reinterpret_cast<const uint4*>(so + row * 256 + ((u ^ (row & 15)) << 4));
                        if (sp * 32 + row < tile.tm && ucol < tn) {
                            // (col0 + c0) is a multiple of 32: the chunk starts a panel K step
                            int64_t e;
                            if (MULTI) {
                                // multi-RHS: column n = k * rstride + c goes to panel row R*i + k, K step c/32
                                const int n = tile.col0 + c0 + (u >> 3) * 32;
                                const int k = n / tile.rstride, c = n - k * tile.rstride;
                                e = tile.c_off + ((int64_t)(tile.row0 + sp * 32 + row) * tile.nrhs + k) * tile.ldc +
                                    (int64_t)(c >> 5) * 64 + (u & 7) * 8;
                            } else {
                                e = tile.c_off + (int64_t)(tile.row0 + sp * 32 + row) * tile.ldc +
                                    (int64_t)((tile.col0 + c0) >> 5) * 64 + u * 8;
                            }
                            *reinterpret_cast<uint4*>(C + e) = val;
                        }
                    }
                    __syncwarp();   // the staging area is rewritten by the next chunk
                } else {
                    // FP32 (OUT_SPLIT 2) or FP64 output, column-major (transC = 0) or row-major;
                    // multi-RHS tiles: tile row R*i + k is row i of vector k (at k * vstride)
                    if (rl < tile.tm) {
                        int64_t gr = tile.row0 + rl, base = tile.c_off;
                        if (MULTI) {
                            const int64_t i = gr / tile.nrhs;
                            base += (gr - i * tile.nrhs) * g.vstride;
                            gr = i;
                        }
                        // element (gr, gc) at base + gr * rs + gc * cs
                        const int64_t rs = g.transC ? tile.ldc : 1, cs = g.transC ? 1 : tile.ldc;
                        const int64_t e0 = base + gr * rs + (int64_t)(tile.col0 + c0) * cs;
#pragma unroll
                        for (int j = 0; j < 64; ++j) {
                            if (j < tn) {
                                if (OUT_SPLIT == 2) ((float*)g.C)[e0 + j * cs] = __uint_as_float(v[j]);
                                else ((double*)g.C)[e0 + j * cs] = (double)__uint_as_float(v[j]);   // exact widening
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
    cudaError_t e;
#define UMMA_ATTR(O, M)                                                                                     \
    if ((e = cudaFuncSetAttribute(gg_umma_kernel<O, M>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                                  um::SMEM_BYTES)) != cudaSuccess)                                          \
        return e;
    UMMA_ATTR(0, false) UMMA_ATTR(1, false) UMMA_ATTR(2, false) UMMA_ATTR(0, true) UMMA_ATTR(1, true)
#undef UMMA_ATTR
#define UMMA_ATTR_TF32(O)                                                                                   \
    if ((e = cudaFuncSetAttribute(gg_umma_kernel<O, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                  um::SMEM_BYTES)) != cudaSuccess)                                          \
        return e;
    UMMA_ATTR_TF32(0) UMMA_ATTR_TF32(1) UMMA_ATTR_TF32(2)
#undef UMMA_ATTR_TF32
    return cudaSuccess;
}

// multi: the plan's tiles interleave nrhs right-hand sides (separate instances, so
// that the single-vector epilogues keep their register budget)
cudaError_t launch_gg_umma(int out_mode, bool multi, const GGArgs& a, const TmaMaps& maps, cudaStream_t st,
                           bool tf32) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (!a.steps || !a.cta_tiles || a.ncta <= 0 || !a.C) return cudaErrorInvalidValue;
    if (out_mode == 1 && !a.transC) return cudaErrorInvalidValue;   // the staged epilogue writes panel rows
    if (multi && (out_mode == 2 || (out_mode == 0 && a.vstride <= 0))) return cudaErrorInvalidValue;
    if (tf32) {
        if (multi) return cudaErrorInvalidValue;   // 3xTF32 plans have one right-hand side
        if (out_mode == 1) gg_umma_kernel<1, false, true><<<a.ncta, um::nt_of(out_mode), um::SMEM_BYTES, st>>>(a, maps);
        else if (out_mode == 2) gg_umma_kernel<2, false, true><<<a.ncta, um::nt_of(out_mode), um::SMEM_BYTES, st>>>(a, maps);
        else if (out_mode == 0) gg_umma_kernel<0, false, true><<<a.ncta, um::nt_of(out_mode), um::SMEM_BYTES, st>>>(a, maps);
        else return cudaErrorInvalidValue;
        return cudaGetLastError();
    }
    if (out_mode == 1 && !multi) gg_umma_kernel<1, false><<<a.ncta, um::nt_of(out_mode), um::SMEM_BYTES, st>>>(a, maps);
    else if (out_mode == 1) gg_umma_kernel<1, true><<<a.ncta, um::nt_of(out_mode), um::SMEM_BYTES, st>>>(a, maps);
    else if (out_mode == 2) gg_umma_kernel<2, false><<<a.ncta, um::nt_of(out_mode), um::SMEM_BYTES, st>>>(a, maps);
    else if (out_mode == 0 && !multi) gg_umma_kernel<0, false><<<a.ncta, um::nt_of(out_mode), um::SMEM_BYTES, st>>>(a, maps);
    else if (out_mode == 0) gg_umma_kernel<0, true><<<a.ncta, um::nt_of(out_mode), um::SMEM_BYTES, st>>>(a, maps);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

}  // namespace vmps
