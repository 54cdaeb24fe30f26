// Host-callable launchers of kernels.cu
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "engine.hpp"

namespace vmps {

struct GGArgs {
    const void* A;
    const void* B;
    void* C;
    int* err;         // device error word: bit 0 = a bounded wait ran out (tcgen05 engine)
    // tcgen05 engine: the K steps and the per-CTA tile ranges of the schedule (ncta CTAs)
    const TStep* steps;
    const int32_t* cta_tiles;
    int ncta;
    const GTile* tiles;
    const GSeg* segs;
    const GTerm* terms;
    int ntiles;
    int transA, transB, transC;
    int64_t vstride;   // multi-RHS phase 2: element stride between the output vectors
    long long wait_budget;   // tcgen05 engine: clock cycles a main-loop barrier wait may take (0: ~2 s)
};

// tcgen05 engine: TMA descriptors of a phase, passed by value as a grid-constant
// kernel parameter (parameter-space descriptors need no tensor-map proxy fence)
struct TmaMaps {
    CUtensorMap a[kMaxMapsA];
    CUtensorMap b[kMaxMapsB];
};

// one column piece of a column-major FP64 block written into its panel rows:
// column c -> panel row c (dst_off + c*dst_pitch), element r -> K index r
struct PanelPiece { int64_t src_off, dst_off; int32_t rows, cols, src_ld, dst_pitch; double scale; };

struct PackBlock { int64_t coff, doff, rows, cols, ld; double scale; };

cudaError_t kernels_init();
// FP64 grouped GEMM (DMMA)
cudaError_t launch_gg64(const GGArgs& a, cudaStream_t st);
// split-precision (BF16x3) grouped GEMM, tcgen05 engine (umma.cu): persistent,
// TMA-fed, tiles up to 128 x 256; out_split = 1: C is a bf16 [hi|lo] panel arena,
// 0: C is double
cudaError_t umma_init();
// out_mode: 0 FP64 output, 1 bf16 [hi|lo] panel rows (split intermediates), 2 FP32 output
// multi: tiles of a multi-RHS plan (interleaved right-hand sides)
// tf32: the operands are 3xTF32 panels (kind::tf32 MMAs, K steps of 16); single right-hand side
cudaError_t launch_gg_umma(int out_mode, bool multi, const GGArgs& a, const TmaMaps& maps, cudaStream_t st,
                           bool tf32 = false);
// split operands: FP64 blocks -> bf16 [hi|lo] panels
cudaError_t launch_prep(const PrepBlock* pb, int nb, const double* src, void* dst, cudaStream_t st);
cudaError_t launch_panel_split(const PanelPiece* pieces, int np, const double* src, void* dst, cudaStream_t st);
cudaError_t launch_panel_split_f32(const PanelPiece* pieces, int np, const float* src, void* dst, cudaStream_t st);
// 3xTF32 operands: FP64 blocks (or FP64 / FP32 vector pieces) -> FP32 [16 hi | 16 lo] panels
cudaError_t launch_prep_tf32(const PrepBlock* pb, int nb, const double* src, void* dst, cudaStream_t st);
cudaError_t launch_panel_split_tf32(const PanelPiece* pieces, int np, const double* src, const float* srcf, void* dst,
                                    cudaStream_t st);
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
cudaError_t launch_hadamard(const double* a, const double* b, double* out, int64_t n, cudaStream_t st);   // out = a * b
cudaError_t launch_combine(const double* V, int nv, int64_t n, const double* c, double* y, cudaStream_t st);
cudaError_t launch_finite(const double* x, int64_t n, int* bad, cudaStream_t st);
// split-K partials of a grouped GEMM summed in order: out[e] = sum_j part[j * n + e] (double or float)
cudaError_t launch_splitk_reduce(const void* part, int nparts, int64_t n, void* out, int f32, cudaStream_t st);
// excited-state projector after an HxV: out_r += sum_p E <dvec_p, y_r> avec_p (r < nrhs, vectors
// at stride n; y and out double or float, the other pointer null); deterministic
struct PenaltyArgs {
    const double* dvec;   // [npen][n]: projector vectors for the overlap
    const double* avec;   // [npen][n]: projector vectors added to the output
    double* part;         // [npen * nrhs][nchunk] chunk partials
    double* coef;         // [npen * nrhs]: E * overlap
    int64_t n, chunk;
    int npen, nrhs, nchunk;
    double E;
};
cudaError_t launch_penalty(const PenaltyArgs& a, const double* y, const float* yf, double* o, float* of,
                           cudaStream_t st);
// VUMPS transfer operator: out = sum_b w_b tr(V_b LR_b) (deterministic); out[V block] = V - T + s * 1
struct TracePair { int64_t v_off, lr_off; int32_t rows, cols, v_ld, lr_ld; double weight; };
struct CombineBlock { int64_t v_off, t_off; int32_t rows, cols, v_ld, t_ld; };
cudaError_t launch_trace_pairs(const TracePair* tp, int n, const double* V, const double* LR, double* part, double* out,
                               cudaStream_t st);
cudaError_t launch_transfer_combine(const CombineBlock* cb, int n, const double* V, const double* T, double* out,
                                    const double* s, cudaStream_t st);

// ---- device-resident Lanczos step (lanczos.cu) ----------------------------------
constexpr int kLzMaxIter = 1024;       // Krylov dimension limit of the device step
constexpr int kLzMaxPerThread = 16;    // vector elements per thread of one block chunk
struct LzArgs {
    void* K;            // basis (double or float), row i at K + i * ld; kmax + 1 rows
    int64_t ld;
    void* w;            // HxV output, orthogonalised in place
    void* q;            // HxV input: copy of the newest basis vector
    double* part;       // per-chunk partial sums [max(kmax, 2)][nchunk]
    double* cl;         // [2]: <K_{j-1}, w>, <K_j, w>
    double* coef;       // [kmax]: full-pass coefficients
    double* ab;         // [3][kmax]: alpha, beta, 1/beta
    double* host_ab;    // host-mapped mirror of alpha and beta [2][kmax], or null
    unsigned* ctl;      // [0] iteration index j, [1..3] block counters (zero on entry)
    int64_t n;          // vector length (padded layout)
    int kmax;           // iterations the buffers hold
    int nchunk;         // blocks per launch (chunks of per_thread * 256 elements)
    int fp32;           // vectors are float (split-precision phase), else double
};
struct LzShape { int per_thread = 1, chunk = 256, nchunk = 1; };
LzShape lz_shape(int64_t n, int num_sms);
cudaError_t lz_init();
cudaError_t launch_lz_step(const LzArgs& a, int per_thread, cudaStream_t st);
cudaError_t launch_lz_combine(const void* K, int fp32, int64_t ld, int m, int64_t n, const double* c, double* y,
                              cudaStream_t st);
// out[i] = <K_i, r>, i < m (deterministic; part holds m * sh.nchunk doubles)
cudaError_t launch_lz_mdot(const void* K, int fp32, int64_t ld, int m, int64_t n, const double* r, double* part,
                           const LzShape& sh, double* out, cudaStream_t st);
cudaError_t launch_lz_to_f32(const double* x, float* y, int64_t n, cudaStream_t st);

// ---- Chebyshev recursion over many right-hand sides (lanczos.cu) -------------------
constexpr int kChebMaxParts = 8;
struct ChebArgs {
    const double* w;      // H t_n, nrhs vectors at stride vs
    const double* tn;     // t_n
    const double* tprev;  // t_{n-1} (read from step 1 on; zero before)
    double* tnext;        // t_{n+1}
    double* part;         // per-chunk partial sums [nrhs][nparts][2][nchunk]
    double* mu;           // moments [nrhs][nparts][nmom]
    unsigned* ctl;        // [0] step n, [1] block counter (zero on entry)
    int64_t n, vs;        // vector length (padded layout), stride between vectors
    int nrhs, nmom, nchunk;
    double inv_a, b;      // the recursion runs on (H - b) / a
    // moments per part: part j of every vector is elements [pbeg[j], pbeg[j+1]) (nparts 1:
    // the whole vector); nchunk covers the longest part
    int nparts;
    int64_t pbeg[kChebMaxParts + 1];
};
cudaError_t launch_cheb_step(const ChebArgs& a, int per_thread, cudaStream_t st);

}  // namespace vmps
