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
template <typename T> __device__ __forceinline__ double ld_d(const T* p) { return (double)__ldg(p); }
template <typename T> __device__ __forceinline__ float ld_f(const T* p) { return (float)__ldg(p); }

// A(i,k) of the segment, summed over its terms; (i,k) relative to the block
template <typename TA, typename Acc>
__device__ __forceinline__ Acc load_A(const TA* A, const GTerm* terms, int tb, int tc, int lda, bool trans, int i,
                                      int k) {
    Acc v = 0;
    const int64_t e = trans ? ((int64_t)k + (int64_t)i * lda) : ((int64_t)i + (int64_t)k * lda);
    for (int t = 0; t < tc; ++t) {
        const GTerm tm = terms[tb + t];
        v += (Acc)tm.coef * (Acc)__ldg(A + tm.off + e);
    }
    return v;
}
template <typename TB, typename Acc>
__device__ __forceinline__ Acc load_B(const TB* B, int64_t off, int ldb, bool trans, int k, int j) {
    const int64_t e = trans ? ((int64_t)j + (int64_t)k * ldb) : ((int64_t)k + (int64_t)j * ldb);
    return (Acc)__ldg(B + off + e);
}

// ===========================================================================
// FP64 grouped GEMM, 64x64 tile, 128 threads (2x2 warps of 32x32), BK = 16
// ===========================================================================
namespace f64k {
constexpr int BM = 64, BN = 64, BK = 16, NT = 128;
constexpr int SA = BM + 4, SB = BN + 4;   // padded strides: conflict-free fragment reads
}

__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(f64k::NT) gg_fp64_kernel(GGArgs g) {
    using namespace f64k;
    __shared__ double As[2][BK][SA];
    __shared__ double Bs[2][BK][SB];
    const GTile tile = g.tiles[blockIdx.x];
    const double* __restrict__ A = (const double*)g.A;
    const double* __restrict__ B = (const double*)g.B;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int mrem = min(BM, tile.m - tile.row0), nrem = min(BN, tile.n - tile.col0);

    double acc[4][4][2];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = 0.0;

    double ra[8], rb[8];
    int seg = tile.seg_begin, k0 = 0;
    // staged load of (seg, k0) into registers
    auto stage = [&](int s, int kk0) {
        const GSeg sg = g.segs[s];
        const int krem = sg.K - kk0;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            int i, k;
            if (!g.transA) { i = tid & 63; k = (tid >> 6) + 2 * r; }
            else { k = tid & 15; i = (tid >> 4) + 8 * r; }
            ra[r] = (i < mrem && k < krem)
                        ? load_A<double, double>(A, g.terms, sg.term_begin, sg.term_count, sg.lda, g.transA,
                                                 tile.row0 + i, kk0 + k)
                        : 0.0;
            int j, kb;
            if (!g.transB) { kb = tid & 15; j = (tid >> 4) + 8 * r; }
            else { j = tid & 63; kb = (tid >> 6) + 2 * r; }
            rb[r] = (j < nrem && kb < krem) ? load_B<double, double>(B, sg.b_off, sg.ldb, g.transB, kk0 + kb,
                                                                      tile.col0 + j)
                                            : 0.0;
        }
    };
    auto commit = [&](int buf) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            int i, k;
            if (!g.transA) { i = tid & 63; k = (tid >> 6) + 2 * r; }
            else { k = tid & 15; i = (tid >> 4) + 8 * r; }
            As[buf][k][i] = ra[r];
            int j, kb;
            if (!g.transB) { kb = tid & 15; j = (tid >> 4) + 8 * r; }
            else { j = tid & 63; kb = (tid >> 6) + 2 * r; }
            Bs[buf][kb][j] = rb[r];
        }
    };
    auto advance = [&](int& s, int& kk0) {
        kk0 += BK;
        if (kk0 >= g.segs[s].K) { kk0 = 0; ++s; }
    };

    if (seg < tile.seg_end) {
        stage(seg, k0);
        int buf = 0;
        while (true) {
            commit(buf);
            __syncthreads();
            int ns = seg, nk = k0;
            advance(ns, nk);
            const bool more = ns < tile.seg_end;
            if (more) stage(ns, nk);
            const int g4 = lane >> 2, t4 = lane & 3;
#pragma unroll
            for (int kq = 0; kq < BK; kq += 4) {
                double af[4], bf[4];
#pragma unroll
                for (int mi = 0; mi < 4; ++mi) af[mi] = As[buf][kq + t4][wm + mi * 8 + g4];
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) bf[ni] = Bs[buf][kq + t4][wn + ni * 8 + g4];
#pragma unroll
                for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                    for (int ni = 0; ni < 4; ++ni) dmma(acc[mi][ni][0], acc[mi][ni][1], af[mi], bf[ni]);
            }
            if (!more) break;
            seg = ns; k0 = nk;
            buf ^= 1;
        }
    }
    {
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
}

// ===========================================================================
// BF16x3 split-precision grouped GEMM, 128x128 tile, 256 threads (2x4 warps of
// 64x32), BK = 32, mma.sync m16n8k16 bf16 -> f32
// ===========================================================================
namespace spk {
constexpr int BM = 128, BN = 128, BK = 32, NT = 256;
constexpr int LDS = BK + 8;   // 80-byte rows: ldmatrix reads are conflict-free
constexpr int TILE_ELEMS = BM * LDS;
constexpr int SMEM_BYTES = 2 /*stages*/ * 4 /*Ahi,Alo,Bhi,Blo*/ * TILE_ELEMS * 2 /*bytes*/;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
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
// split two fp32 values into packed bf16x2 hi and lo words
__device__ __forceinline__ void split2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
    __nv_bfloat16 l0 = __float2bfloat16_rn(x0 - __bfloat162float(h0));
    __nv_bfloat16 l1 = __float2bfloat16_rn(x1 - __bfloat162float(h1));
    hi = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
    lo = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
}

template <typename TA, typename TB, typename TC>
__global__ void __launch_bounds__(spk::NT) gg_split_kernel(GGArgs g) {
    using namespace spk;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __nv_bfloat16* sm = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    // stage s: [Ahi | Alo | Bhi | Blo], each BM x LDS (A rows = m, B rows = n, k contiguous)
    auto tileptr = [&](int stage, int which) { return sm + (stage * 4 + which) * TILE_ELEMS; };

    const GTile tile = g.tiles[blockIdx.x];
    const TA* __restrict__ A = (const TA*)g.A;
    const TB* __restrict__ B = (const TB*)g.B;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 2) * 64, wn = (warp & 3) * 32;
    const int mrem = min(BM, tile.m - tile.row0), nrem = min(BN, tile.n - tile.col0);

    float acc[4][4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;

    // staging registers: 8 pairs for A, 8 pairs for B (fp32)
    float ra[8][2], rb[8][2];
    auto stage = [&](int s, int kk0) {
        const GSeg sg = g.segs[s];
        const int krem = sg.K - kk0;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            int i, kp;
            if (!g.transA) { i = tid & 127; kp = ((tid >> 7) + 2 * r) * 2; }
            else { kp = (tid & 15) * 2; i = (tid >> 4) + 16 * r; }
#pragma unroll
            for (int h = 0; h < 2; ++h)
                ra[r][h] = (i < mrem && kp + h < krem)
                               ? load_A<TA, float>(A, g.terms, sg.term_begin, sg.term_count, sg.lda, g.transA,
                                                   tile.row0 + i, kk0 + kp + h)
                               : 0.f;
            int j, kq;
            if (!g.transB) { kq = (tid & 15) * 2; j = (tid >> 4) + 16 * r; }
            else { j = tid & 127; kq = ((tid >> 7) + 2 * r) * 2; }
#pragma unroll
            for (int h = 0; h < 2; ++h)
                rb[r][h] = (j < nrem && kq + h < krem)
                               ? load_B<TB, float>(B, sg.b_off, sg.ldb, g.transB, kk0 + kq + h, tile.col0 + j)
                               : 0.f;
        }
    };
    auto commit = [&](int st) {
        __nv_bfloat16 *Ah = tileptr(st, 0), *Al = tileptr(st, 1), *Bh = tileptr(st, 2), *Bl = tileptr(st, 3);
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            int i, kp;
            if (!g.transA) { i = tid & 127; kp = ((tid >> 7) + 2 * r) * 2; }
            else { kp = (tid & 15) * 2; i = (tid >> 4) + 16 * r; }
            uint32_t hi, lo;
            split2(ra[r][0], ra[r][1], hi, lo);
            *reinterpret_cast<uint32_t*>(Ah + i * LDS + kp) = hi;
            *reinterpret_cast<uint32_t*>(Al + i * LDS + kp) = lo;
            int j, kq;
            if (!g.transB) { kq = (tid & 15) * 2; j = (tid >> 4) + 16 * r; }
            else { j = tid & 127; kq = ((tid >> 7) + 2 * r) * 2; }
            split2(rb[r][0], rb[r][1], hi, lo);
            *reinterpret_cast<uint32_t*>(Bh + j * LDS + kq) = hi;
            *reinterpret_cast<uint32_t*>(Bl + j * LDS + kq) = lo;
        }
    };

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
            const __nv_bfloat16 *Ah = tileptr(st, 0), *Al = tileptr(st, 1), *Bh = tileptr(st, 2),
                                *Bl = tileptr(st, 3);
#pragma unroll
            for (int kk = 0; kk < BK; kk += 16) {
                uint32_t ah[4][4], al[4][4], bh[4][2], bl[4][2];
#pragma unroll
                for (int mi = 0; mi < 4; ++mi) {
                    const int row = wm + mi * 16 + (lane & 15);
                    const int col = kk + (lane >> 4) * 8;
                    ldsm_x4(ah[mi][0], ah[mi][1], ah[mi][2], ah[mi][3], smem_u32(Ah + row * LDS + col));
                    ldsm_x4(al[mi][0], al[mi][1], al[mi][2], al[mi][3], smem_u32(Al + row * LDS + col));
                }
#pragma unroll
                for (int np = 0; np < 2; ++np) {
                    const int row = wn + np * 16 + (lane & 7) + ((lane >> 4) << 3);
                    const int col = kk + ((lane >> 3) & 1) * 8;
                    ldsm_x4(bh[2 * np][0], bh[2 * np][1], bh[2 * np + 1][0], bh[2 * np + 1][1],
                            smem_u32(Bh + row * LDS + col));
                    ldsm_x4(bl[2 * np][0], bl[2 * np][1], bl[2 * np + 1][0], bl[2 * np + 1][1],
                            smem_u32(Bl + row * LDS + col));
                }
#pragma unroll
                for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                    for (int ni = 0; ni < 4; ++ni) {
                        mma_bf16(acc[mi][ni], al[mi], bh[ni][0], bh[ni][1]);
                        mma_bf16(acc[mi][ni], ah[mi], bl[ni][0], bl[ni][1]);
                        mma_bf16(acc[mi][ni], ah[mi], bh[ni][0], bh[ni][1]);
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
    for (int mi = 0; mi < 4; ++mi)
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
    cudaError_t e = cudaSuccess;
    auto set = [&](const void* f) {
        cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, spk::SMEM_BYTES);
        if (r != cudaSuccess) e = r;
    };
    set((const void*)gg_split_kernel<double, double, double>);
    set((const void*)gg_split_kernel<double, double, float>);
    set((const void*)gg_split_kernel<double, float, double>);
    set((const void*)gg_split_kernel<double, float, float>);
    set((const void*)gg_split_kernel<float, double, double>);
    set((const void*)gg_split_kernel<float, double, float>);
    set((const void*)gg_split_kernel<float, float, double>);
    set((const void*)gg_split_kernel<float, float, float>);
    return e;
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
        case 0: gg_split_kernel<double, double, double><<<a.ntiles, spk::NT, spk::SMEM_BYTES, st>>>(a); break;
        case 1: gg_split_kernel<double, double, float><<<a.ntiles, spk::NT, spk::SMEM_BYTES, st>>>(a); break;
        case 2: gg_split_kernel<double, float, double><<<a.ntiles, spk::NT, spk::SMEM_BYTES, st>>>(a); break;
        case 3: gg_split_kernel<double, float, float><<<a.ntiles, spk::NT, spk::SMEM_BYTES, st>>>(a); break;
        case 4: gg_split_kernel<float, double, double><<<a.ntiles, spk::NT, spk::SMEM_BYTES, st>>>(a); break;
        case 5: gg_split_kernel<float, double, float><<<a.ntiles, spk::NT, spk::SMEM_BYTES, st>>>(a); break;
        case 6: gg_split_kernel<float, float, double><<<a.ntiles, spk::NT, spk::SMEM_BYTES, st>>>(a); break;
        case 7: gg_split_kernel<float, float, float><<<a.ntiles, spk::NT, spk::SMEM_BYTES, st>>>(a); break;
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
