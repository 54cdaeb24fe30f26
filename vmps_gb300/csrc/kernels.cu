// CUDA kernels of the GB300 effective-Hamiltonian engine (sm_103a).
//
// gg_fp64  : grouped GEMM, FP64 operands, DMMA (mma.sync m8n8k4 f64) -- the
//            plain drop-in form, bit-for-bit the same arithmetic type as the
//            Eigen path of pivot/DmrgPivotMatrix1.h:236-262.
// gg_split : grouped GEMM, operands split into bf16 hi/lo on the fly while
//            staging to shared memory, hi*hi + hi*lo + lo*hi products on the
//            tensor cores (mma.sync m16n8k16 bf16, FP32 accumulate).
//
// Work layout (planned on the host, engine.hpp): every CTA owns one output tile
// and loops over that tile's segments; a segment is one GEMM of K columns
// whose A operand is a linear combination of up to several same-shape blocks
// (sum_t c_t A_t).  Output tiles are written exactly once, so no atomics are
// needed and results are deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "kernels.hpp"

namespace vmps {

// ---------------------------------------------------------------------------
// operand access helpers
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Operand staging.  Device blocks are column-major with ld a multiple of 8,
// start offsets aligned to 32 elements and zero padding, and tile origins are
// multiples of 16 (rows) / 8 (columns), so every 4-element group read below is
// 16-byte aligned and stays inside its block's padded storage.  Groups whose
// first element lies outside the tile are replaced by zeros; elements past the
// block edge inside a group are either zero padding or rows/columns that only
// reach output entries the epilogue masks off.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void ldg4(const float* p, float (&v)[4]) {
    const float4 x = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
__device__ __forceinline__ void ldg4(const double* p, float (&v)[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    v[0] = (float)a.x; v[1] = (float)a.y; v[2] = (float)b.x; v[3] = (float)b.y;
}
__device__ __forceinline__ void ldg2(const double* p, double (&v)[2]) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p));
    v[0] = a.x; v[1] = a.y;
}

// ===========================================================================
// FP64 grouped GEMM: tile <= 64x64, 128 threads (2x2 warps of 32x32), BK = 16,
// DMMA m8n8k4.  Shared layouts follow the contiguous global dimension:
//   A row-contiguous  -> As[k][m] (stride 68)   A k-contiguous -> As[m][k] (stride 20)
//   B k-contiguous    -> Bs[n][k] (stride 20)   B col-contiguous -> Bs[k][n] (stride 68)
// (strides keep every half-warp of fragment reads on distinct banks).
// ===========================================================================
namespace f64k {
constexpr int BM = 64, BN = 64, BK = 16, NT = 128;
constexpr int SMN = 68;   // [k][m] / [k][n] row stride (doubles)
constexpr int SKK = 20;   // [m][k] / [n][k] row stride (doubles)
constexpr int OP_ELEMS = BM * SKK > BK * SMN ? BM * SKK : BK * SMN;   // 1280 vs 1088
}

__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(f64k::NT, 3) gg_fp64_kernel(GGArgs g) {
    using namespace f64k;
    __shared__ __align__(16) double As[2][OP_ELEMS];
    __shared__ __align__(16) double Bs[2][OP_ELEMS];
    const GTile tile = g.tiles[blockIdx.x];
    const double* __restrict__ A = (const double*)g.A;
    const double* __restrict__ B = (const double*)g.B;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int mrem = tile.tm, nrem = tile.tn;
    const bool tA = g.transA, tB = g.transB;

    double acc[4][4][2];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = 0.0;

    // each thread stages 4 double2 of A and 4 of B per BK step
    double ra[4][2], rb[4][2];
    auto stage = [&](int s, int k0) {
        const GSeg sg = g.segs[s];
        const int krem = sg.K - k0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int v = tid + NT * r;   // 512 pairs per operand tile
            int i, k;
            if (!tA) { i = (v & 31) * 2; k = v >> 5; }      // m-pairs along rows, 16 k columns
            else     { k = (v & 7) * 2;  i = v >> 3; }      // k-pairs, 64 rows
            ra[r][0] = ra[r][1] = 0.0;
            if (i < mrem && k < krem) {
                const int64_t e = tA ? ((int64_t)(k0 + k) + (int64_t)(tile.row0 + i) * sg.lda)
                                     : ((int64_t)(tile.row0 + i) + (int64_t)(k0 + k) * sg.lda);
                for (int t = 0; t < sg.term_count; ++t) {
                    const GTerm tm = g.terms[sg.term_begin + t];
                    double x[2];
                    ldg2(A + tm.off + e, x);
                    ra[r][0] = fma(tm.coef, x[0], ra[r][0]);
                    ra[r][1] = fma(tm.coef, x[1], ra[r][1]);
                }
            }
            int j, kb;
            if (!tB) { kb = (v & 7) * 2;  j = v >> 3; }
            else     { j = (v & 31) * 2;  kb = v >> 5; }
            rb[r][0] = rb[r][1] = 0.0;
            if (j < nrem && kb < krem) {
                const int64_t e = tB ? ((int64_t)(tile.col0 + j) + (int64_t)(k0 + kb) * sg.ldb)
                                     : ((int64_t)(k0 + kb) + (int64_t)(tile.col0 + j) * sg.ldb);
                ldg2(B + sg.b_off + e, rb[r]);
            }
        }
    };
    auto commit = [&](int buf) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int v = tid + NT * r;
            if (!tA) { const int i = (v & 31) * 2, k = v >> 5;
                       *reinterpret_cast<double2*>(&As[buf][k * SMN + i]) = make_double2(ra[r][0], ra[r][1]); }
            else     { const int k = (v & 7) * 2, i = v >> 3;
                       *reinterpret_cast<double2*>(&As[buf][i * SKK + k]) = make_double2(ra[r][0], ra[r][1]); }
            if (!tB) { const int kb = (v & 7) * 2, j = v >> 3;
                       *reinterpret_cast<double2*>(&Bs[buf][j * SKK + kb]) = make_double2(rb[r][0], rb[r][1]); }
            else     { const int j = (v & 31) * 2, kb = v >> 5;
                       *reinterpret_cast<double2*>(&Bs[buf][kb * SMN + j]) = make_double2(rb[r][0], rb[r][1]); }
        }
    };

    int seg = tile.seg_begin, k0 = 0;
    // warps whose 32x32 sub-tile is entirely outside the tile skip the MMAs
    const bool warp_live = wm < mrem && wn < nrem;
    if (seg < tile.seg_end) {
        stage(seg, k0);
        int buf = 0;
        while (true) {
            commit(buf);
            __syncthreads();
            int ns = seg, nk = k0 + BK;
            if (nk >= g.segs[seg].K) { nk = 0; ++ns; }
            const bool more = ns < tile.seg_end;
            if (more) stage(ns, nk);
            if (warp_live) {
                const int g4 = lane >> 2, t4 = lane & 3;
#pragma unroll
                for (int kq = 0; kq < BK; kq += 4) {
                    double af[4], bf[4];
#pragma unroll
                    for (int mi = 0; mi < 4; ++mi) {
                        const int m = wm + mi * 8 + g4, k = kq + t4;
                        af[mi] = tA ? As[buf][m * SKK + k] : As[buf][k * SMN + m];
                    }
#pragma unroll
                    for (int ni = 0; ni < 4; ++ni) {
                        const int n = wn + ni * 8 + g4, k = kq + t4;
                        bf[ni] = tB ? Bs[buf][k * SMN + n] : Bs[buf][n * SKK + k];
                    }
#pragma unroll
                    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                        for (int ni = 0; ni < 4; ++ni) dmma(acc[mi][ni][0], acc[mi][ni][1], af[mi], bf[ni]);
                }
            }
            if (!more) break;
            seg = ns; k0 = nk;
            buf ^= 1;
        }
    }
    double* __restrict__ C = (double*)g.C;
    const int g4 = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = wm + mi * 8 + g4, c = wn + ni * 8 + t4 * 2 + h;
                if (r < mrem && c < nrem) {
                    const int64_t gr = tile.row0 + r, gc = tile.col0 + c;
                    const int64_t e = g.transC ? (gc + gr * tile.ldc) : (gr + gc * tile.ldc);
                    C[tile.c_off + e] = acc[mi][ni][h];
                }
            }
}

// ===========================================================================
// BF16x3 split-precision grouped GEMM: tile <= 64x64, 128 threads (2x2 warps
// of 32x32), BK = 32, mma.sync m16n8k16 bf16 -> f32.  Operands are read as
// fp32/fp64 16-byte groups, scaled and summed over the segment's terms in
// fp32, split into hi/lo bf16 and stored in shared memory in the layout that
// matches the contiguous global dimension; fragments come from ldmatrix
// (k-contiguous layouts) or ldmatrix.trans (row-/column-contiguous layouts).
// ===========================================================================
namespace spk {
constexpr int BM = 64, BN = 64, BK = 32, NT = 128;
constexpr int SMN = BM + 8;   // [k][m] / [k][n] row stride (bf16): 144 B, conflict-free ldmatrix
constexpr int SKK = BK + 8;   // [m][k] / [n][k] row stride (bf16): 80 B
constexpr int OP_ELEMS = BM * SKK > BK * SMN ? BM * SKK : BK * SMN;   // 2560
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// split four fp32 values into packed hi and lo bf16 quadruples
__device__ __forceinline__ void split4(const float (&x)[4], uint2& hi, uint2& lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const __nv_bfloat16 bh = __float2bfloat16_rn(x[i]);
        const __nv_bfloat16 bl = __float2bfloat16_rn(x[i] - __bfloat162float(bh));
        h[i] = __bfloat16_as_ushort(bh);
        l[i] = __bfloat16_as_ushort(bl);
    }
    hi = make_uint2(h[0] | (h[1] << 16), h[2] | (h[3] << 16));
    lo = make_uint2(l[0] | (l[1] << 16), l[2] | (l[3] << 16));
}

template <typename TA, typename TB, typename TC>
__global__ void __launch_bounds__(spk::NT, 4) gg_split_kernel(GGArgs g) {
    using namespace spk;
    // [stage][Ahi, Alo, Bhi, Blo]
    __shared__ __align__(128) __nv_bfloat16 sm[2][4][OP_ELEMS];
    const GTile tile = g.tiles[blockIdx.x];
    const TA* __restrict__ A = (const TA*)g.A;
    const TB* __restrict__ B = (const TB*)g.B;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int mrem = tile.tm, nrem = tile.tn;
    const bool tA = g.transA, tB = g.transB;

    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;

    // 512 groups of 4 per operand tile (64 x 32): 4 per thread
    float ra[4][4], rb[4][4];
    auto stage = [&](int s, int k0) {
        const GSeg sg = g.segs[s];
        const int krem = sg.K - k0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int v = tid + NT * r;
            int i, k;
            if (!tA) { i = (v & 15) * 4; k = v >> 4; }     // row quads, 32 k columns
            else     { k = (v & 7) * 4;  i = v >> 3; }     // k quads, 64 rows
#pragma unroll
            for (int q = 0; q < 4; ++q) ra[r][q] = 0.f;
            if (i < mrem && k < krem) {
                const int64_t e = tA ? ((int64_t)(k0 + k) + (int64_t)(tile.row0 + i) * sg.lda)
                                     : ((int64_t)(tile.row0 + i) + (int64_t)(k0 + k) * sg.lda);
                for (int t = 0; t < sg.term_count; ++t) {
                    const GTerm tm = g.terms[sg.term_begin + t];
                    const float c = (float)tm.coef;
                    float x[4];
                    ldg4(A + tm.off + e, x);
#pragma unroll
                    for (int q = 0; q < 4; ++q) ra[r][q] = fmaf(c, x[q], ra[r][q]);
                }
            }
            int j, kb;
            if (!tB) { kb = (v & 7) * 4;  j = v >> 3; }    // k quads, 64 columns
            else     { j = (v & 15) * 4;  kb = v >> 4; }   // column quads, 32 k rows
#pragma unroll
            for (int q = 0; q < 4; ++q) rb[r][q] = 0.f;
            if (j < nrem && kb < krem) {
                const int64_t e = tB ? ((int64_t)(tile.col0 + j) + (int64_t)(k0 + kb) * sg.ldb)
                                     : ((int64_t)(k0 + kb) + (int64_t)(tile.col0 + j) * sg.ldb);
                ldg4(B + sg.b_off + e, rb[r]);
            }
        }
    };
    auto commit = [&](int st) {
        __nv_bfloat16 *Ah = sm[st][0], *Al = sm[st][1], *Bh = sm[st][2], *Bl = sm[st][3];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int v = tid + NT * r;
            uint2 hi, lo;
            split4(ra[r], hi, lo);
            int ia;
            if (!tA) { const int i = (v & 15) * 4, k = v >> 4; ia = k * SMN + i; }
            else     { const int k = (v & 7) * 4, i = v >> 3;  ia = i * SKK + k; }
            *reinterpret_cast<uint2*>(Ah + ia) = hi;
            *reinterpret_cast<uint2*>(Al + ia) = lo;
            split4(rb[r], hi, lo);
            int ib;
            if (!tB) { const int kb = (v & 7) * 4, j = v >> 3; ib = j * SKK + kb; }
            else     { const int j = (v & 15) * 4, kb = v >> 4; ib = kb * SMN + j; }
            *reinterpret_cast<uint2*>(Bh + ib) = hi;
            *reinterpret_cast<uint2*>(Bl + ib) = lo;
        }
    };

    const bool warp_live = wm < mrem && wn < nrem;
    int seg = tile.seg_begin, k0 = 0;
    if (seg < tile.seg_end) {
        stage(seg, k0);
        int st = 0;
        while (true) {
            commit(st);
            __syncthreads();
            int ns = seg, nk = k0 + BK;
            if (nk >= g.segs[seg].K) { nk = 0; ++ns; }
            const bool more = ns < tile.seg_end;
            if (more) stage(ns, nk);
            if (warp_live) {
                const __nv_bfloat16 *Ah = sm[st][0], *Al = sm[st][1], *Bh = sm[st][2], *Bl = sm[st][3];
#pragma unroll
                for (int kk = 0; kk < BK; kk += 16) {
                    uint32_t ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
                    for (int mi = 0; mi < 2; ++mi) {
                        const int mb = wm + mi * 16;
                        if (tA) {   // [m][k]: plain ldmatrix
                            const int off = (mb + (lane & 15)) * SKK + kk + (lane >> 4) * 8;
                            ldsm_x4(ah[mi][0], ah[mi][1], ah[mi][2], ah[mi][3], smem_u32(Ah + off));
                            ldsm_x4(al[mi][0], al[mi][1], al[mi][2], al[mi][3], smem_u32(Al + off));
                        } else {    // [k][m]: transposing ldmatrix
                            const int off = (kk + (lane & 7) + ((lane >> 4) & 1) * 8) * SMN + mb + ((lane >> 3) & 1) * 8;
                            ldsm_x4_t(ah[mi][0], ah[mi][1], ah[mi][2], ah[mi][3], smem_u32(Ah + off));
                            ldsm_x4_t(al[mi][0], al[mi][1], al[mi][2], al[mi][3], smem_u32(Al + off));
                        }
                    }
#pragma unroll
                    for (int np = 0; np < 2; ++np) {
                        const int nb = wn + np * 16;
                        if (!tB) {  // [n][k]: plain ldmatrix
                            const int off = (nb + (lane & 7) + ((lane >> 4) << 3)) * SKK + kk + ((lane >> 3) & 1) * 8;
                            ldsm_x4(bh[2 * np][0], bh[2 * np][1], bh[2 * np + 1][0], bh[2 * np + 1][1], smem_u32(Bh + off));
                            ldsm_x4(bl[2 * np][0], bl[2 * np][1], bl[2 * np + 1][0], bl[2 * np + 1][1], smem_u32(Bl + off));
                        } else {    // [k][n]: transposing ldmatrix
                            const int off = (kk + (lane & 7) + ((lane >> 3) & 1) * 8) * SMN + nb + (lane >> 4) * 8;
                            ldsm_x4_t(bh[2 * np][0], bh[2 * np][1], bh[2 * np + 1][0], bh[2 * np + 1][1], smem_u32(Bh + off));
                            ldsm_x4_t(bl[2 * np][0], bl[2 * np][1], bl[2 * np + 1][0], bl[2 * np + 1][1], smem_u32(Bl + off));
                        }
                    }
#pragma unroll
                    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                        for (int ni = 0; ni < 4; ++ni) {
                            mma_bf16(acc[mi][ni], al[mi], bh[ni][0], bh[ni][1]);
                            mma_bf16(acc[mi][ni], ah[mi], bl[ni][0], bl[ni][1]);
                            mma_bf16(acc[mi][ni], ah[mi], bh[ni][0], bh[ni][1]);
                        }
                }
            }
            if (!more) break;
            seg = ns; k0 = nk;
            st ^= 1;
        }
    }
    // epilogue: c0,c1 -> (g, 2t..2t+1), c2,c3 -> (g+8, 2t..2t+1)
    TC* __restrict__ C = (TC*)g.C;
    const int g4 = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const int r = wm + mi * 16 + g4 + (h >> 1) * 8, c = wn + ni * 8 + t4 * 2 + (h & 1);
                if (r < mrem && c < nrem) {
                    const int64_t gr = tile.row0 + r, gc = tile.col0 + c;
                    const int64_t e = g.transC ? (gc + gr * tile.ldc) : (gr + gc * tile.ldc);
                    C[tile.c_off + e] = (TC)acc[mi][ni][h];
                }
            }
}

// ===========================================================================
// layout conversion, vector algebra
// ===========================================================================
// dst (padded) <- scale * src (compact), or the reverse
__global__ void pack_kernel(const PackBlock* blocks, int nb, const double* __restrict__ src, double* __restrict__ dst,
                            int to_padded) {
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        const PackBlock pb = blocks[b];
        const int64_t n = pb.rows * pb.cols;
        for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
            const int64_t r = e % pb.rows, c = e / pb.rows;
            if (to_padded) dst[pb.doff + r + c * pb.ld] = pb.scale * src[pb.coff + e];
            else dst[pb.coff + e] = src[pb.doff + r + c * pb.ld] / pb.scale;
        }
    }
}

__global__ void to_f32_kernel(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

// partial dot products: fixed chunking -> deterministic two-pass reduction
constexpr int kDotThreads = 256;
__global__ void dot_partial_kernel(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                                   int64_t chunk, double* __restrict__ part) {
    __shared__ double red[kDotThreads];
    const int64_t b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    double s = 0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += kDotThreads) s = fma(x[i], y[i], s);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kDotThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
__global__ void sum_partial_kernel(const double* __restrict__ part, int np, double* __restrict__ out) {
    __shared__ double red[kDotThreads];
    double s = 0;
    for (int i = threadIdx.x; i < np; i += kDotThreads) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kDotThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}
// many dots at once: out[j] = <V_j, w> for j < nv (V row-major [nv][n]); partials [nv][nchunk]
__global__ void mdot_partial_kernel(const double* __restrict__ V, int64_t n, const double* __restrict__ w,
                                    int64_t chunk, int nchunk, double* __restrict__ part) {
    __shared__ double red[kDotThreads];
    const int j = blockIdx.y;
    const int64_t b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    const double* v = V + (int64_t)j * n;
    double s = 0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += kDotThreads) s = fma(v[i], w[i], s);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int ww = kDotThreads / 2; ww > 0; ww >>= 1) {
        if (threadIdx.x < ww) red[threadIdx.x] += red[threadIdx.x + ww];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(int64_t)j * nchunk + blockIdx.x] = red[0];
}
__global__ void msum_partial_kernel(const double* __restrict__ part, int nchunk, double* __restrict__ out) {
    __shared__ double red[kDotThreads];
    const int j = blockIdx.x;
    double s = 0;
    for (int i = threadIdx.x; i < nchunk; i += kDotThreads) s += part[(int64_t)j * nchunk + i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kDotThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[j] = red[0];
}
// w -= sum_j coef[j] V_j
__global__ void mgs_update_kernel(const double* __restrict__ V, int nv, int64_t n, const double* __restrict__ coef,
                                  double* __restrict__ w) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = w[i];
        for (int j = 0; j < nv; ++j) s = fma(-coef[j], V[(int64_t)j * n + i], s);
        w[i] = s;
    }
}
__global__ void axpy_kernel(double a, const double* __restrict__ x, double* __restrict__ y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], y[i]);
}
__global__ void scale_kernel(double a, double* __restrict__ x, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= a;
}
// y = sum_j c[j] V_j  (Ritz vector assembly)
__global__ void combine_kernel(const double* __restrict__ V, int nv, int64_t n, const double* __restrict__ c,
                               double* __restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0;
        for (int j = 0; j < nv; ++j) s = fma(c[j], V[(int64_t)j * n + i], s);
        y[i] = s;
    }
}
__global__ void finite_kernel(const double* __restrict__ x, int64_t n, int* __restrict__ bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!isfinite(x[i])) { atomicOr(bad, 1); return; }
}

// ===========================================================================
// launchers
// ===========================================================================
static int grid_for(int64_t n, int threads, int cap) {
    int64_t g = (n + threads - 1) / threads;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// opt the split kernels into their dynamic shared memory size (once per process,
// before any launch or stream capture)
cudaError_t kernels_init() {
    // all grouped-GEMM kernels use static shared memory below 48 KB
    return cudaSuccess;
}

cudaError_t launch_gg(int prec, int ta, int tb, int tc, const GGArgs& a, cudaStream_t st) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (prec == VMPS_PREC_FP64) {
        gg_fp64_kernel<<<a.ntiles, f64k::NT, 0, st>>>(a);
        return cudaGetLastError();
    }
    // split precision: type codes 0 = double, 1 = float
    const int code = ta * 4 + tb * 2 + tc;
    switch (code) {
        case 0: gg_split_kernel<double, double, double><<<a.ntiles, spk::NT, 0, st>>>(a); break;
        case 1: gg_split_kernel<double, double, float><<<a.ntiles, spk::NT, 0, st>>>(a); break;
        case 2: gg_split_kernel<double, float, double><<<a.ntiles, spk::NT, 0, st>>>(a); break;
        case 3: gg_split_kernel<double, float, float><<<a.ntiles, spk::NT, 0, st>>>(a); break;
        case 4: gg_split_kernel<float, double, double><<<a.ntiles, spk::NT, 0, st>>>(a); break;
        case 5: gg_split_kernel<float, double, float><<<a.ntiles, spk::NT, 0, st>>>(a); break;
        case 6: gg_split_kernel<float, float, double><<<a.ntiles, spk::NT, 0, st>>>(a); break;
        case 7: gg_split_kernel<float, float, float><<<a.ntiles, spk::NT, 0, st>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_pack(const PackBlock* blocks, int nb, const double* src, double* dst, int to_padded, cudaStream_t st) {
    if (nb <= 0) return cudaSuccess;
    if (!blocks || !src || !dst) return cudaErrorInvalidValue;   // never launch on an unallocated buffer
    pack_kernel<<<min(nb, 4096), 256, 0, st>>>(blocks, nb, src, dst, to_padded);
    return cudaGetLastError();
}
cudaError_t launch_to_f32(const double* src, float* dst, int64_t n, cudaStream_t st) {
    to_f32_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}
// chunked dot: part must hold nchunk doubles
int64_t dot_chunk(int64_t n) {
    const int64_t c = (n + 2047) / 2048;
    return c > 8192 ? c : 8192;
}
int dot_nchunk(int64_t n) { return (int)((n + dot_chunk(n) - 1) / dot_chunk(n)); }
cudaError_t launch_dot(const double* x, const double* y, int64_t n, double* part, double* out, cudaStream_t st) {
    const int64_t ch = dot_chunk(n);
    const int nc = dot_nchunk(n);
    dot_partial_kernel<<<nc, kDotThreads, 0, st>>>(x, y, n, ch, part);
    sum_partial_kernel<<<1, kDotThreads, 0, st>>>(part, nc, out);
    return cudaGetLastError();
}
cudaError_t launch_mdot(const double* V, int nv, int64_t n, const double* w, double* part, double* out,
                        cudaStream_t st) {
    if (nv <= 0) return cudaSuccess;
    const int64_t ch = dot_chunk(n);
    const int nc = dot_nchunk(n);
    mdot_partial_kernel<<<dim3(nc, nv), kDotThreads, 0, st>>>(V, n, w, ch, nc, part);
    msum_partial_kernel<<<nv, kDotThreads, 0, st>>>(part, nc, out);
    return cudaGetLastError();
}
cudaError_t launch_mgs(const double* V, int nv, int64_t n, const double* coef, double* w, cudaStream_t st) {
    if (nv <= 0) return cudaSuccess;
    mgs_update_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(V, nv, n, coef, w);
    return cudaGetLastError();
}
cudaError_t launch_axpy(double a, const double* x, double* y, int64_t n, cudaStream_t st) {
    axpy_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(a, x, y, n);
    return cudaGetLastError();
}
cudaError_t launch_scale(double a, double* x, int64_t n, cudaStream_t st) {
    scale_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(a, x, n);
    return cudaGetLastError();
}
cudaError_t launch_combine(const double* V, int nv, int64_t n, const double* c, double* y, cudaStream_t st) {
    combine_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(V, nv, n, c, y);
    return cudaGetLastError();
}
cudaError_t launch_finite(const double* x, int64_t n, int* bad, cudaStream_t st) {
    finite_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(x, n, bad);
    return cudaGetLastError();
}

}  // namespace vmps
