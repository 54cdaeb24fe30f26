// Device-resident Lanczos step.
//
// One Lanczos iteration after the HxV w = H K_j is a fixed sequence of four
// launches that keep every scalar on the device:
//
//   lz_local : c_{j-1} = <K_{j-1}, w>, c_j = <K_j, w>
//   lz_proj  : w <- w - c_{j-1} K_{j-1} - c_j K_j  (the three-term recurrence),
//              then d_i = <K_i, w> for all i <= j
//   lz_orth  : w <- w - sum_i d_i K_i               (one full Gram-Schmidt pass),
//              alpha_j = c_j + d_j, beta_j = |w|, j <- j + 1
//   lz_next  : K_{j+1} = q = w / beta_j
//
// The local step removes the large components of w first, so the full pass
// works on a vector that is already nearly orthogonal to the basis and one
// pass keeps the basis orthogonal to working precision (the local step plus
// one pass cost 2(j+1)+5 FP64 FMAs per element against 4(j+1) for two full
// passes; on GB300 the FP64 rate, not HBM, bounds these loops).
//
// The Krylov vectors are FP64, or FP32 for the split-precision phase (whose
// operator carries 4e-6 relative rounding noise, far above FP32's): FP32 halves
// the bytes and moves the FMAs off GB300's slow FP64 pipe.  Chunk partial sums,
// alpha, beta and the coefficients are FP64 either way.
//
// The iteration index lives in device memory, so the HxV plan and these
// kernels form one CUDA graph that the host replays per iteration.  Reductions
// are deterministic: each block writes the partial sums of its element chunk,
// and the last block to finish (a device-scope counter incremented after a
// fence) adds the partials in chunk order.  No block waits on another.
#include <algorithm>

#include "convert.hpp"
#include "kernels.hpp"

namespace vmps {

namespace {
constexpr int kLzThreads = 256, kLzWarps = kLzThreads / 32;
constexpr int kLzCoefBlocks = 152;   // rows of d summed in parallel (one per block, strided)

__device__ __forceinline__ double lz_warp_sum(double s) {
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// true in the block that finishes last; its reads of the other blocks'
// partials go through L2 (__ldcg)
__device__ __forceinline__ bool lz_last_block(unsigned* counter) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// sum of part[row][0..nchunk) by one warp (lane 0 holds the result)
__device__ __forceinline__ double lz_row_sum(const double* part, int row, int nchunk, int lane) {
    double s = 0;
    for (int c = lane; c < nchunk; c += 32) s += __ldcg(part + (int64_t)row * nchunk + c);
    return lz_warp_sum(s);
}

// the same sum by the whole block (every thread returns it): a few independent
// loads per thread instead of nchunk / 32 dependent rounds of one warp, which
// left a single block reducing long after the others had finished
__device__ __forceinline__ double lz_block_row_sum(const double* part, int row, int nchunk) {
    __shared__ double red[kLzWarps];
    const double* p = part + (int64_t)row * nchunk;
    double s = 0;
#pragma unroll 8
    for (int c = threadIdx.x; c < nchunk; c += kLzThreads) s += __ldcg(p + c);
    s = lz_warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    double t = 0;
#pragma unroll
    for (int q = 0; q < kLzWarps; ++q) t += red[q];
    __syncthreads();   // red is reused by the next call
    return t;
}

// 16-byte groups of vector elements (float4 / double2): the step kernels issue
// one load per group, not per element (per element and basis row the work is a
// load, a shared load and an FMA, so instruction issue, not HBM, bounded the
// scalar form)
template <typename V>
struct LzPack {
    static constexpr int W = 16 / (int)sizeof(V);
    V v[W];
};
template <typename V>
__device__ __forceinline__ LzPack<V> lz_ld16(const V* p) {
    LzPack<V> r;
    *reinterpret_cast<uint4*>(&r) = *reinterpret_cast<const uint4*>(p);
    return r;
}
template <typename V>
__device__ __forceinline__ void lz_st16(V* p, const LzPack<V>& r) {
    *reinterpret_cast<uint4*>(p) = *reinterpret_cast<const uint4*>(&r);
}
// whole 16-byte groups per thread in a chunk of E * 256 elements
template <typename V, int E>
struct LzVecOk {
    static constexpr bool value = E % LzPack<V>::W == 0;
};

// partial dot of basis row `ki` (chunk-relative) with the chunk of w staged in
// shared memory: one warp, len valid elements, four independent accumulators
// in the vector type, FP64 from the warp sum on.  Full chunks go by 16-byte
// groups; the partial last chunk element by element.
template <typename V, int E>
__device__ __forceinline__ double lz_chunk_dot(const V* __restrict__ ki, const V* wsh, int len, int lane) {
    V s[4] = {0, 0, 0, 0};
    constexpr int W = LzPack<V>::W;
    bool done = false;
    if constexpr (LzVecOk<V, E>::value) {
        if (len == E * 256) {
#pragma unroll
            for (int t = 0; t < E * 8 / W; ++t) {
                const int x = (lane + 32 * t) * W;
                const LzPack<V> a = lz_ld16(ki + x), b = lz_ld16(wsh + x);
#pragma unroll
                for (int q = 0; q < W; ++q) s[t & 3] = fma(a.v[q], b.v[q], s[t & 3]);
            }
            done = true;
        }
    }
    if (!done) {
#pragma unroll
        for (int t = 0; t < E * 8; ++t) {
            const int x = lane + 32 * t;
            if (x < len) s[t & 3] = fma(ki[x], wsh[x], s[t & 3]);
        }
    }
    return lz_warp_sum((double)((s[0] + s[1]) + (s[2] + s[3])));
}

template <typename V, int E>
__global__ void __launch_bounds__(kLzThreads) lz_local_kernel(LzArgs a) {
    const int j = (int)a.ctl[0];
    if (j >= a.kmax) return;
    __shared__ double red[2][kLzWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t e0 = (int64_t)blockIdx.x * (E * kLzThreads) + threadIdx.x;
    const V* K = (const V*)a.K;
    const V* w = (const V*)a.w;
    const V* kj = K + (int64_t)j * a.ld;
    const V* km = j > 0 ? K + (int64_t)(j - 1) * a.ld : nullptr;
    V s0 = 0, s1 = 0;
#pragma unroll
    for (int u = 0; u < E; ++u) {
        const int64_t e = e0 + u * kLzThreads;
        if (e < a.n) {
            const V x = w[e];
            s1 = fma(kj[e], x, s1);
            if (km) s0 = fma(km[e], x, s0);
        }
    }
    const double d0 = lz_warp_sum((double)s0), d1 = lz_warp_sum((double)s1);
    if (lane == 0) { red[0][warp] = d0; red[1][warp] = d1; }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0;
        for (int q = 0; q < kLzWarps; ++q) t += red[threadIdx.x][q];
        a.part[(int64_t)threadIdx.x * a.nchunk + blockIdx.x] = t;
    }
    if (!lz_last_block(a.ctl + 1)) return;
    const double t0 = lz_block_row_sum(a.part, 0, a.nchunk), t1 = lz_block_row_sum(a.part, 1, a.nchunk);
    if (threadIdx.x == 0) {
        a.cl[0] = t0;
        a.cl[1] = t1;
        a.ctl[1] = 0;
    }
}

template <typename V, int E>
__global__ void __launch_bounds__(kLzThreads) lz_proj_kernel(LzArgs a) {
    __shared__ __align__(16) V wsh[E * kLzThreads];   // this block's chunk of w after the local step
    const int j = (int)a.ctl[0];
    if (j >= a.kmax) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t cb = (int64_t)blockIdx.x * (E * kLzThreads);
    const int len = (int)(a.n - cb < E * kLzThreads ? a.n - cb : E * kLzThreads);
    const V c0 = (V)a.cl[0], c1 = (V)a.cl[1];
    const V* K = (const V*)a.K;
    V* w = (V*)a.w;
    const V* kj = K + (int64_t)j * a.ld + cb;
    const V* km = j > 0 ? K + (int64_t)(j - 1) * a.ld + cb : nullptr;
    bool done = false;
    if constexpr (LzVecOk<V, E>::value) {
        constexpr int W = LzPack<V>::W;
        if (len == E * kLzThreads) {
#pragma unroll
            for (int u = 0; u < E / W; ++u) {
                const int x = (threadIdx.x + u * kLzThreads) * W;
                LzPack<V> v = lz_ld16(w + cb + x);
                const LzPack<V> b = lz_ld16(kj + x);
#pragma unroll
                for (int q = 0; q < W; ++q) v.v[q] = fma(-c1, b.v[q], v.v[q]);
                if (km) {
                    const LzPack<V> m = lz_ld16(km + x);
#pragma unroll
                    for (int q = 0; q < W; ++q) v.v[q] = fma(-c0, m.v[q], v.v[q]);
                }
                lz_st16(w + cb + x, v);
                lz_st16(wsh + x, v);
            }
            done = true;
        }
    }
    if (!done) {
#pragma unroll
        for (int u = 0; u < E; ++u) {
            const int x = threadIdx.x + u * kLzThreads;
            V v = 0;
            if (x < len) {
                v = fma(-c1, kj[x], w[cb + x]);
                if (km) v = fma(-c0, km[x], v);
                w[cb + x] = v;
            }
            wsh[x] = v;
        }
    }
    __syncthreads();
    // one warp per basis row: d_i partial over this chunk (summed by lz_coef)
    for (int i = warp; i <= j; i += kLzWarps) {
        const double t = lz_chunk_dot<V, E>(K + (int64_t)i * a.ld + cb, wsh, len, lane);
        if (lane == 0) a.part[(int64_t)i * a.nchunk + blockIdx.x] = t;
    }
}

// d_i = sum over chunks of lz_proj's partials, one block per basis row
__global__ void __launch_bounds__(kLzThreads) lz_coef_kernel(LzArgs a) {
    const int j = (int)a.ctl[0];
    if (j >= a.kmax) return;
    for (int i = blockIdx.x; i <= j; i += gridDim.x) {
        const double t = lz_block_row_sum(a.part, i, a.nchunk);
        if (threadIdx.x == 0) a.coef[i] = t;
    }
}

template <typename V, int E>
__global__ void __launch_bounds__(kLzThreads) lz_orth_kernel(LzArgs a) {
    const int j = (int)a.ctl[0];
    if (j >= a.kmax) return;
    __shared__ double red[kLzWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t e0 = (int64_t)blockIdx.x * (E * kLzThreads) + threadIdx.x;
    const V* K = (const V*)a.K;
    V* w = (V*)a.w;
    V s = 0;
    const int64_t cb = (int64_t)blockIdx.x * (E * kLzThreads);
    bool done = false;
    if constexpr (LzVecOk<V, E>::value) {
      constexpr int W = LzPack<V>::W;
      if (cb + E * kLzThreads <= a.n) {
        // full chunk: each thread owns E / W 16-byte groups
        LzPack<V> wr[E / W];
#pragma unroll
        for (int u = 0; u < E / W; ++u) wr[u] = lz_ld16(w + cb + (threadIdx.x + u * kLzThreads) * W);
#pragma unroll 2
        for (int i = 0; i <= j; ++i) {
            const V* ki = K + (int64_t)i * a.ld + cb;
            const V d = (V)a.coef[i];
#pragma unroll
            for (int u = 0; u < E / W; ++u) {
                const LzPack<V> kv = lz_ld16(ki + (threadIdx.x + u * kLzThreads) * W);
#pragma unroll
                for (int q = 0; q < W; ++q) wr[u].v[q] = fma(-d, kv.v[q], wr[u].v[q]);
            }
        }
#pragma unroll
        for (int u = 0; u < E / W; ++u) {
            lz_st16(w + cb + (threadIdx.x + u * kLzThreads) * W, wr[u]);
#pragma unroll
            for (int q = 0; q < W; ++q) s = fma(wr[u].v[q], wr[u].v[q], s);
        }
        done = true;
      }
    }
    if (!done) {
        V wr[E];
#pragma unroll
        for (int u = 0; u < E; ++u) {
            const int64_t e = e0 + u * kLzThreads;
            wr[u] = e < a.n ? w[e] : V(0);
        }
#pragma unroll 4
        for (int i = 0; i <= j; ++i) {
            const V* ki = K + (int64_t)i * a.ld;
            const V d = (V)a.coef[i];
#pragma unroll
            for (int u = 0; u < E; ++u) {
                const int64_t e = e0 + u * kLzThreads;
                if (e < a.n) wr[u] = fma(-d, ki[e], wr[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < E; ++u) {
            const int64_t e = e0 + u * kLzThreads;
            if (e < a.n) {
                w[e] = wr[u];
                s = fma(wr[u], wr[u], s);
            }
        }
    }
    const double ds = lz_warp_sum((double)s);
    if (lane == 0) red[warp] = ds;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int q = 0; q < kLzWarps; ++q) t += red[q];
        a.part[blockIdx.x] = t;
    }
    if (!lz_last_block(a.ctl + 3)) return;
    const double ww = lz_block_row_sum(a.part, 0, a.nchunk);
    if (threadIdx.x == 0) {
        const double alpha = a.cl[1] + a.coef[j];
        const double beta = sqrt(ww);
        a.ab[j] = alpha;
        a.ab[a.kmax + j] = beta;
        a.ab[2 * a.kmax + j] = beta > 1e-300 ? 1.0 / beta : 0.0;
        if (a.host_ab) {
            volatile double* h = a.host_ab;
            h[j] = alpha;
            h[a.kmax + j] = beta;
        }
        a.ctl[3] = 0;
        a.ctl[0] = (unsigned)(j + 1);
    }
}

template <typename V>
__global__ void lz_next_kernel(LzArgs a) {
    const int jn = (int)a.ctl[0];
    if (jn < 1 || jn > a.kmax) return;
    const V s = (V)a.ab[2 * a.kmax + jn - 1];
    V* k = (V*)a.K + (int64_t)jn * a.ld;
    const V* w = (const V*)a.w;
    V* q = (V*)a.q;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        const V v = w[i] * s;
        k[i] = v;
        q[i] = v;
    }
}

__device__ __forceinline__ double lz_f64(double x) { return x; }
__device__ __forceinline__ double lz_f64(float x) { return f32_to_f64(x); }   // exact, integer pipe

// y[e] = sum_{i < m} c[i] K_i[e] in FP64 (Ritz vectors and corrections)
template <typename V>
__global__ void lz_combine_kernel(const V* __restrict__ K, int64_t ld, int m, int64_t n,
                                  const double* __restrict__ c, double* __restrict__ y) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        double s = 0;
        for (int i = 0; i < m; ++i) s = fma(c[i], lz_f64(K[(int64_t)i * ld + e]), s);
        y[e] = s;
    }
}

// out[i] = <K_i, r> for i < m, deterministic: per-chunk partials here (r is
// FP64, rounded to the basis type when staged), summed by lz_rowsum_kernel
template <typename V, int E>
__global__ void __launch_bounds__(kLzThreads) lz_mdot_kernel(const V* __restrict__ K, int64_t ld, int m, int64_t n,
                                                              const double* __restrict__ r,
                                                              double* __restrict__ part, int nchunk) {
    __shared__ __align__(16) V rsh[E * kLzThreads];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t cb = (int64_t)blockIdx.x * (E * kLzThreads);
    const int len = (int)(n - cb < E * kLzThreads ? n - cb : E * kLzThreads);
#pragma unroll
    for (int u = 0; u < E; ++u) {
        const int x = threadIdx.x + u * kLzThreads;
        rsh[x] = (V)(x < len ? r[cb + x] : 0.0);
    }
    __syncthreads();
    for (int i = warp; i < m; i += kLzWarps) {
        const double t = lz_chunk_dot<V, E>(K + (int64_t)i * ld + cb, rsh, len, lane);
        if (lane == 0) part[(int64_t)i * nchunk + blockIdx.x] = t;
    }
}

// out[i] = sum over chunks of part[i], i < rows, one block per row
__global__ void __launch_bounds__(kLzThreads) lz_rowsum_kernel(const double* part, int nchunk, int rows,
                                                                double* out) {
    for (int i = blockIdx.x; i < rows; i += gridDim.x) {
        const double t = lz_block_row_sum(part, i, nchunk);
        if (threadIdx.x == 0) out[i] = t;
    }
}

__global__ void lz_to_f32_kernel(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        y[e] = f64_to_f32_rn(x[e]);
}

// One step of the Chebyshev recursion for nrhs vectors at once (grid: chunks x
// right-hand sides x parts).  Step n makes t_{n+1} = c_a (H t_n - b t_n) - c_p t_{n-1}
// with (c_a, c_p) = (1/a, 0) for n = 0 and (2/a, 1) after, and accumulates in
// FP64 the two inner products of the moment doubling relations
//   mu_{2n} = 2 <t_n, t_n> - mu_0,  mu_{2n+1} = 2 <t_{n+1}, t_n> - mu_1
// (mu_0 = <t_0, t_0>, mu_1 = <t_1, t_0> at n = 0), per part of the vector (the
// element ranges of different start vectors sharing one layout).  The last block
// to finish writes the moments and advances n.
template <int E>
__global__ void __launch_bounds__(kLzThreads) cheb_step_kernel(ChebArgs a) {
    const int step = (int)a.ctl[0];
    const double ca = step == 0 ? a.inv_a : 2.0 * a.inv_a, cp = step == 0 ? 0.0 : 1.0;
    const int k = blockIdx.y, pj = blockIdx.z, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)k * a.vs;
    const int64_t pe = a.pbeg[pj + 1];
    const int64_t e0 = a.pbeg[pj] + (int64_t)blockIdx.x * (E * kLzThreads) + threadIdx.x;
    __shared__ double red[2][kLzWarps];
    double s0 = 0, s1 = 0;
#pragma unroll
    for (int u = 0; u < E; ++u) {
        const int64_t e = e0 + u * kLzThreads;
        if (e < pe) {
            const double x = a.tn[base + e];
            const double v = fma(ca, fma(-a.b, x, a.w[base + e]), -cp * a.tprev[base + e]);
            a.tnext[base + e] = v;
            s0 = fma(x, x, s0);
            s1 = fma(v, x, s1);
        }
    }
    s0 = lz_warp_sum(s0);
    s1 = lz_warp_sum(s1);
    if (lane == 0) { red[0][warp] = s0; red[1][warp] = s1; }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0;
        for (int q = 0; q < kLzWarps; ++q) t += red[threadIdx.x][q];
        a.part[(((int64_t)k * a.nparts + pj) * 2 + threadIdx.x) * a.nchunk + blockIdx.x] = t;
    }
    // last block of the whole grid
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(a.ctl + 1, 1u) == gridDim.x * gridDim.y * gridDim.z - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int r = warp; r < a.nrhs * a.nparts; r += kLzWarps) {
        const double d0 = lz_row_sum(a.part, 2 * r, a.nchunk, lane);
        const double d1 = lz_row_sum(a.part, 2 * r + 1, a.nchunk, lane);
        if (lane == 0) {
            double* mu = a.mu + (int64_t)r * a.nmom;
            if (step == 0) {
                mu[0] = d0;
                if (a.nmom > 1) mu[1] = d1;
            } else {
                const int i = 2 * step;
                if (i < a.nmom) mu[i] = 2.0 * d0 - mu[0];
                if (i + 1 < a.nmom) mu[i + 1] = 2.0 * d1 - mu[1];
            }
        }
    }
    if (threadIdx.x == 0) {
        a.ctl[1] = 0;
        a.ctl[0] = (unsigned)(step + 1);
    }
}
}  // namespace

// elements per thread (E) and chunk count for a vector length: the smallest
// E in {1, 2, 4, 8, 16} that keeps the grid within 8 blocks per SM
LzShape lz_shape(int64_t n, int num_sms) {
    LzShape s;
    const int64_t cap = (int64_t)8 * (num_sms > 0 ? num_sms : 152);
    s.per_thread = 1;
    while (s.per_thread < kLzMaxPerThread && (n + (int64_t)s.per_thread * kLzThreads - 1) /
                                                     ((int64_t)s.per_thread * kLzThreads) > cap)
        s.per_thread *= 2;
    s.chunk = s.per_thread * kLzThreads;
    s.nchunk = (int)std::max<int64_t>(1, (n + s.chunk - 1) / s.chunk);
    return s;
}

cudaError_t lz_init() { return cudaSuccess; }

#define LZ_DISPATCH(PER, CALL)                 \
    switch (PER) {                             \
        case 1: CALL(1); break;                \
        case 2: CALL(2); break;                \
        case 4: CALL(4); break;                \
        case 8: CALL(8); break;                \
        case 16: CALL(16); break;              \
        default: return cudaErrorInvalidValue; \
    }

template <typename V>
static cudaError_t lz_step(const LzArgs& a, int per_thread, cudaStream_t st) {
#define LZ_CALL(EE)                                                   \
    lz_local_kernel<V, EE><<<a.nchunk, kLzThreads, 0, st>>>(a);       \
    lz_proj_kernel<V, EE><<<a.nchunk, kLzThreads, 0, st>>>(a);        \
    lz_coef_kernel<<<kLzCoefBlocks, kLzThreads, 0, st>>>(a);           \
    lz_orth_kernel<V, EE><<<a.nchunk, kLzThreads, 0, st>>>(a);
    LZ_DISPATCH(per_thread, LZ_CALL)
#undef LZ_CALL
    const int g = (int)std::min<int64_t>((a.n + 255) / 256, 152 * 8);
    lz_next_kernel<V><<<g, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_lz_step(const LzArgs& a, int per_thread, cudaStream_t st) {
    if (a.kmax < 1 || a.kmax > kLzMaxIter || a.n <= 0 || a.nchunk < 1 || !a.K || !a.w || !a.q || !a.part ||
        !a.coef || !a.cl || !a.ab || !a.ctl)
        return cudaErrorInvalidValue;
    if ((int64_t)a.nchunk * per_thread * kLzThreads < a.n) return cudaErrorInvalidValue;
    return a.fp32 ? lz_step<float>(a, per_thread, st) : lz_step<double>(a, per_thread, st);
}

cudaError_t launch_lz_combine(const void* K, int fp32, int64_t ld, int m, int64_t n, const double* c, double* y,
                              cudaStream_t st) {
    if (m < 1 || n <= 0 || !K || !c || !y) return cudaErrorInvalidValue;
    const int g = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
    if (fp32) lz_combine_kernel<float><<<g, 256, 0, st>>>((const float*)K, ld, m, n, c, y);
    else lz_combine_kernel<double><<<g, 256, 0, st>>>((const double*)K, ld, m, n, c, y);
    return cudaGetLastError();
}

cudaError_t launch_lz_mdot(const void* K, int fp32, int64_t ld, int m, int64_t n, const double* r, double* part,
                           const LzShape& sh, double* out, cudaStream_t st) {
    if (m < 1 || m > kLzMaxIter || n <= 0 || !K || !r || !part || !out) return cudaErrorInvalidValue;
    if ((int64_t)sh.nchunk * sh.chunk < n) return cudaErrorInvalidValue;
#define LZ_CALL(EE)                                                                                        \
    if (fp32) lz_mdot_kernel<float, EE><<<sh.nchunk, kLzThreads, 0, st>>>((const float*)K, ld, m, n, r, part, \
                                                                          sh.nchunk);                       \
    else lz_mdot_kernel<double, EE><<<sh.nchunk, kLzThreads, 0, st>>>((const double*)K, ld, m, n, r, part,   \
                                                                        sh.nchunk);
    LZ_DISPATCH(sh.per_thread, LZ_CALL)
#undef LZ_CALL
    lz_rowsum_kernel<<<m < kLzCoefBlocks ? m : kLzCoefBlocks, kLzThreads, 0, st>>>(part, sh.nchunk, m, out);
    return cudaGetLastError();
}
#undef LZ_DISPATCH

cudaError_t launch_lz_to_f32(const double* x, float* y, int64_t n, cudaStream_t st) {
    if (n <= 0 || !x || !y) return cudaErrorInvalidValue;
    const int g = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
    lz_to_f32_kernel<<<g, 256, 0, st>>>(x, y, n);
    return cudaGetLastError();
}

cudaError_t launch_cheb_step(const ChebArgs& a, int per_thread, cudaStream_t st) {
    if (a.nrhs < 1 || a.nrhs > 65535 || a.n <= 0 || a.nchunk < 1 || a.nmom < 1 || !a.w || !a.tn || !a.tprev ||
        !a.tnext || !a.part || !a.mu || !a.ctl || a.nparts < 1 || a.nparts > kChebMaxParts)
        return cudaErrorInvalidValue;
    if (a.vs < a.n || a.pbeg[0] != 0 || a.pbeg[a.nparts] != a.n) return cudaErrorInvalidValue;
    for (int j = 0; j < a.nparts; ++j)
        if (a.pbeg[j + 1] <= a.pbeg[j] || (int64_t)a.nchunk * per_thread * kLzThreads < a.pbeg[j + 1] - a.pbeg[j])
            return cudaErrorInvalidValue;
    const dim3 grid(a.nchunk, a.nrhs, a.nparts);
#define LZ_CALL(EE) cheb_step_kernel<EE><<<grid, kLzThreads, 0, st>>>(a);
    switch (per_thread) {
        case 1: LZ_CALL(1); break;
        case 2: LZ_CALL(2); break;
        case 4: LZ_CALL(4); break;
        case 8: LZ_CALL(8); break;
        case 16: LZ_CALL(16); break;
        default: return cudaErrorInvalidValue;
    }
#undef LZ_CALL
    return cudaGetLastError();
}

}  // namespace vmps
