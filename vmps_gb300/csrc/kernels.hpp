// Host-callable launchers of kernels.cu
#pragma once
#include <cuda_runtime.h>

#include "engine.hpp"

namespace vmps {

struct GGArgs {
    const void* A;
    const void* B;
    void* C;
    const void* A2;   // split precision: lo halves of A, B (hi in A, B)
    const void* B2;
    void* C2;         // split precision with a split output: lo half of C
    int* err;         // device error word: bit 0 = a bounded wait ran out (tcgen05 engine)
    // tcgen05 engine: TMA descriptors (128 bytes each) of the prepared A / B blocks,
    // the K steps and the per-CTA tile ranges of the schedule (ncta CTAs)
    const void* amaps;
    const void* bmaps;
    const TStep* steps;
    const int32_t* cta_tiles;
    int ncta;
    const GTile* tiles;
    const GSeg* segs;
    const GTerm* terms;
    int ntiles;
    int transA, transB, transC;
};

struct PackBlock { int64_t coff, doff, rows, cols, ld; double scale; };

cudaError_t kernels_init();
// FP64 grouped GEMM (DMMA)
cudaError_t launch_gg64(const GGArgs& a, cudaStream_t st);
// split-precision grouped GEMM on pre-split K-contiguous operands;
// out_split = 1: C/C2 are bf16 hi/lo, 0: C is double
cudaError_t launch_gg_split(int out_split, const GGArgs& a, cudaStream_t st);
// tcgen05 engine (umma.cu): persistent, TMA-fed; tiles up to 128 x 64
cudaError_t umma_init();
cudaError_t launch_gg_umma(int out_split, const GGArgs& a, cudaStream_t st);
cudaError_t launch_prep(const PrepBlock* pb, int nb, const double* src, void* hi, void* lo, cudaStream_t st);
cudaError_t launch_split(const double* src, void* hi, void* lo, int64_t n, cudaStream_t st);
// compact (scaled per block) -> padded bf16 hi / lo, the values launch_pack + launch_split give
cudaError_t launch_pack_split(const PackBlock* blocks, int nb, const double* src, void* hi, void* lo, cudaStream_t st);
cudaError_t launch_pack(const PackBlock* blocks, int nb, const double* src, double* dst, int to_padded,
                        cudaStream_t st);
int64_t dot_chunk(int64_t n);
int dot_nchunk(int64_t n);
cudaError_t launch_dot(const double* x, const double* y, int64_t n, double* part, double* out, cudaStream_t st);
cudaError_t launch_mdot(const double* V, int nv, int64_t n, const double* w, double* part, double* out,
                        cudaStream_t st);
cudaError_t launch_mgs(const double* V, int nv, int64_t n, const double* coef, double* w, cudaStream_t st);
cudaError_t launch_axpy(double a, const double* x, double* y, int64_t n, cudaStream_t st);
cudaError_t launch_scale(double a, double* x, int64_t n, cudaStream_t st);
cudaError_t launch_combine(const double* V, int nv, int64_t n, const double* c, double* y, cudaStream_t st);
cudaError_t launch_finite(const double* x, int64_t n, int* bad, cudaStream_t st);

}  // namespace vmps
