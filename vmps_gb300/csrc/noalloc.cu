// Allocation-free FP64 chain product: out = alpha * op(X) * Y * op(Z).
//
// Some callers of this library cannot allocate device memory at the point where
// they need one block product: a host framework that has handed all of the
// GPU's memory to its own pool leaves nothing for cudaMalloc, and a solver loop
// that must not stall cannot afford the device-wide synchronisation that
// cudaMalloc / cudaFree imply.  This entry point serves them: the caller passes
// device pointers for the inputs and the output, and the intermediate product
// op(X) * Y lives in a fixed array that is part of the library image on every
// GPU that loads it (kScratchDoubles doubles = 8 MiB, held until the process
// exits).  No allocation of any kind happens here.
//
// Rules for callers:
// * the intermediate must fit: m * n <= kScratchDoubles (m = rows of op(X),
//   n = columns of Y); larger problems are rejected with VMPS_E_ARG;
// * all calls on a device share the one scratch array: two calls whose work
//   overlaps on the GPU (different streams, or different host threads on the
//   same device) race on it and corrupt each other's result;
// * the scratch keeps whatever the last call left there; nothing in it needs to
//   start at zero because every element of the intermediate is written before
//   it is read;
// * every call looks up the array's device address in the current context (a
//   runtime query, no allocation), so the address stays valid across
//   cudaDeviceReset; the first call on a device may also load the library's
//   device code into the context, so make that first call outside any stream
//   capture.
#include <cuda_runtime.h>

#include <string>

#include "../../include/vmps_gb300.h"

namespace {

constexpr long long kScratchDoubles = 1LL << 20;   // 8 MiB

// The array lives in device memory.  In host code its name is only a handle
// for the runtime: never pass &g_chain_scratch to a kernel; look the device
// address up with cudaGetSymbolAddress instead (chain_scratch_ptr below).
static __device__ __align__(256) double g_chain_scratch[kScratchDoubles];

// Device address of the scratch array in the current context.  Looked up on
// every call (a runtime query; it allocates nothing): an address cached across
// calls would dangle once the context it came from is gone (cudaDeviceReset, or
// a primary context released and created again), and the next call would then
// write through it.
cudaError_t chain_scratch_ptr(double** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_chain_scratch);
    if (e != cudaSuccess) return e;
    *out = static_cast<double*>(p);
    return cudaSuccess;
}

// C (m x n, ld = ldc) = alpha * op(A) * op(B); column-major operands with any
// leading dimension, 64 x 64 tiles, 128 threads, DMMA m8n8k4, scalar guarded loads
constexpr int BM = 64, BN = 64, BK = 16, NT = 128;
constexpr int SA = BM + 4;

__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(NT) chain_gemm_kernel(const double* __restrict__ A, long long lda, int transA,
                                                        const double* __restrict__ B, long long ldb, int transB,
                                                        double* __restrict__ C, long long ldc, int m, int n, int k,
                                                        double alpha) {
    __shared__ double As[BK][SA];
    __shared__ double Bs[BK][SA];
    const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    double acc[4][4][2];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = 0.0;
    for (int k0 = 0; k0 < k; k0 += BK) {
        for (int e = tid; e < BM * BK; e += NT) {
            const int i = e % BM, kk = e / BM;
            const int gi = row0 + i, gk = k0 + kk;
            double v = 0.0;
            if (gi < m && gk < k) v = transA ? A[gk + (long long)gi * lda] : A[gi + (long long)gk * lda];
            As[kk][i] = v;
            const int j = e % BN;
            const int gj = col0 + j;
            double w = 0.0;
            if (gj < n && gk < k) w = transB ? B[gj + (long long)gk * ldb] : B[gk + (long long)gj * ldb];
            Bs[kk][j] = w;
        }
        __syncthreads();
        const int g4 = lane >> 2, t4 = lane & 3;
#pragma unroll
        for (int kq = 0; kq < BK; kq += 4) {
            double af[4], bf[4];
#pragma unroll
            for (int mi = 0; mi < 4; ++mi) af[mi] = As[kq + t4][wm + mi * 8 + g4];
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) bf[ni] = Bs[kq + t4][wn + ni * 8 + g4];
#pragma unroll
            for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) dmma(acc[mi][ni][0], acc[mi][ni][1], af[mi], bf[ni]);
        }
        __syncthreads();
    }
    const int g4 = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = row0 + wm + mi * 8 + g4, c = col0 + wn + ni * 8 + t4 * 2 + h;
                if (r < m && c < n) C[r + (long long)c * ldc] = alpha * acc[mi][ni][h];
            }
}

}  // namespace

namespace vmps {
void set_last_error_message(const std::string& msg);   // runtime.cpp: read back by vmps_last_error()
}

namespace {
int fail(int code, const std::string& msg) {
    vmps::set_last_error_message(msg);
    return code;
}
}  // namespace

extern "C" int vmps_chain_fp64_noalloc(const double* X, int64_t x_rows, int64_t x_cols, int32_t transX,
                                       const double* Y, int64_t y_rows, int64_t y_cols, const double* Z,
                                       int64_t z_rows, int64_t z_cols, int32_t transZ, double alpha, double* out,
                                       void* stream) {
    if (!X || !Y || !Z || !out) return fail(VMPS_E_ARG, "vmps_chain_fp64_noalloc: null pointer");
    if (x_rows <= 0 || x_cols <= 0 || y_rows <= 0 || y_cols <= 0 || z_rows <= 0 || z_cols <= 0)
        return fail(VMPS_E_ARG, "vmps_chain_fp64_noalloc: non-positive dimension");
    const int64_t m = transX ? x_cols : x_rows, k = transX ? x_rows : x_cols;
    const int64_t n = y_cols, zn = transZ ? z_cols : z_rows, p = transZ ? z_rows : z_cols;
    if (k != y_rows || zn != n)
        return fail(VMPS_E_SHAPE, "vmps_chain_fp64_noalloc: op(X) * Y * op(Z) shapes do not chain");
    if (m > (1 << 30) || n > (1 << 30) || p > (1 << 30) || k > (1 << 30))
        return fail(VMPS_E_ARG, "vmps_chain_fp64_noalloc: dimension too large");
    if (m * n > kScratchDoubles)
        return fail(VMPS_E_ARG, "vmps_chain_fp64_noalloc: intermediate op(X)*Y has " + std::to_string(m * n) +
                                    " elements, the fixed scratch holds " + std::to_string(kScratchDoubles));
    double* T = nullptr;
    cudaError_t e = chain_scratch_ptr(&T);
    if (e != cudaSuccess) return fail(VMPS_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // T (m x n, ld = m) = op(X) * Y
    dim3 g1((unsigned)((n + BN - 1) / BN), (unsigned)((m + BM - 1) / BM));
    chain_gemm_kernel<<<g1, NT, 0, st>>>(X, x_rows, transX, Y, y_rows, 0, T, m, (int)m, (int)n, (int)k, 1.0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(VMPS_E_CUDA, std::string("chain_gemm_kernel: ") + cudaGetErrorString(e));
    // out (m x p, ld = m) = alpha * T * op(Z)
    dim3 g2((unsigned)((p + BN - 1) / BN), (unsigned)((m + BM - 1) / BM));
    chain_gemm_kernel<<<g2, NT, 0, st>>>(T, m, 0, Z, z_rows, transZ, out, m, (int)m, (int)p, (int)n, alpha);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(VMPS_E_CUDA, std::string("chain_gemm_kernel: ") + cudaGetErrorString(e));
    return VMPS_OK;
}
