/*
 * vmps_gb300.h -- C ABI of the GB300 effective-Hamiltonian engine.
 *
 * The engine replaces the block-sparse tensor contractions that VMPS runs inside
 * its Lanczos / GMRES loops:
 *
 *   HxV(PivotMatrix1, PivotVector, PivotVector)   pivot/DmrgPivotMatrix1.h:123-332
 *   HxV(PivotMatrix2, PivotVector, PivotVector)   pivot/DmrgPivotMatrix2.h:78-273
 *   HxV(PivotMatrix0, PivotVector, PivotVector)   pivot/DmrgPivotMatrix0.h:31-96
 *   contract_L(Tripod, A, W, A, qloc, qOp, Tripod) tensors/DmrgContractions.h:34-158
 *   contract_R(Tripod, A, W, A, qloc, qOp, Tripod) tensors/DmrgContractions.h:179-311
 *   precalc_blockStructure(...)                    tensors/DmrgIndexGymnastics.h:487-590,699-856
 *   PivotVector dot / norm / addScale              pivot/DmrgPivotVector.h:121-358
 *
 * Everything crosses this boundary as plain pointers and sizes.  Block-sparse
 * tensors are described by `vmps_blocks` tables (one row per dense block, data
 * column-major with leading dimension = rows, exactly the storage of an Eigen
 * MatrixXd) and the MPO site tensor W by a COO table `vmps_mpo_site`.
 *
 * Error convention: every entry point returns 0 on success or a negative
 * VMPS_E_* code; the library never aborts.  vmps_last_error() returns a
 * thread-local message for the last failure.  The reference itself has no
 * error channel (asserts only, pivot/DmrgPivotVector.h:307-318).
 *
 * Threading: a context owns one CUDA stream.  Different contexts may be used
 * concurrently from different host threads (VUMPS runs HAC/HC solves for
 * several sites from OpenMP threads, VUMPS/VumpsSolver.h:1168-1171).
 */
#ifndef VMPS_GB300_H
#define VMPS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ---------------------------------------------------------- */
#define VMPS_OK              0
#define VMPS_E_ARG          -1   /* invalid argument / inconsistent tables      */
#define VMPS_E_CUDA         -2   /* CUDA runtime error                         */
#define VMPS_E_NOMEM        -3   /* device or host allocation failed           */
#define VMPS_E_SHAPE        -4   /* block shapes do not chain                  */
#define VMPS_E_TIMEOUT      -5   /* a bounded device wait gave up              */
#define VMPS_E_NONFINITE    -6   /* NaN/Inf detected in an input vector        */
#define VMPS_E_UNSUPPORTED  -7

/* ---- arithmetic of the block products --------------------------------------*/
#define VMPS_PREC_FP64       0   /* plain FP64 (DMMA), parity with the Eigen path */
#define VMPS_PREC_BF16X3     1   /* hi*hi + hi*lo + lo*hi bf16 products, FP32 accumulate */
#define VMPS_PREC_TF32X3     2   /* the same three products with TF32 hi/lo operands (3xTF32): about
                                    2^-21 relative per product against 2^-16, at half the bf16 tensor
                                    rate; pivot HxVs and Lanczos solves (not the multi-RHS, Chebyshev,
                                    environment and transfer-operator entry points)         */

/* ---- symmetry descriptor ----------------------------------------------------
 * A quantum number is nq int32 values.  kind[i] says how component i fuses:
 *   VMPS_SYM_U1  : additive (symmetry/U1.h:170-176), vacuum 0
 *   VMPS_SYM_SU2 : q = 2S+1, |q1-q2|+1 .. q1+q2-1 step 2 (symmetry/SU2.h:174-183), vacuum 1
 * Products of components follow symmetry/S1xS2.h:192-208.                     */
#define VMPS_SYM_U1  0
#define VMPS_SYM_SU2 1
typedef struct {
    int32_t nq;
    int32_t kind[4];
} vmps_symmetry;

/* ---- block table -------------------------------------------------------------
 * One row per dense block.  For a site tensor / PivotVector, `leg` is the
 * physical index s (block = A[s].block[q]); for a Tripod, `leg` is the MPO
 * auxiliary index a (block = T.block[q][a][0]) and qmid holds the middle QN.
 * Blocks of size 0 are simply omitted.  offset is in elements of the
 * accompanying data array; storage is column-major with ld = rows.           */
typedef struct {
    int64_t        nblocks;
    const int32_t* qin;     /* [nblocks*nq] */
    const int32_t* qout;    /* [nblocks*nq] */
    const int32_t* qmid;    /* [nblocks*nq] for Tripods, NULL otherwise */
    const int32_t* leg;     /* [nblocks] */
    const int64_t* rows;    /* [nblocks] */
    const int64_t* cols;    /* [nblocks] */
    const int64_t* offset;  /* [nblocks] */
} vmps_blocks;

/* ---- MPO site tensor W[s1][s2][k].block[qW](row,col) as COO ------------------
 * Mirrors Biped<Symmetry,SparseMatrix> W[s1][s2][k] of MpoTerms.h:1175-1232:
 * s1 = bra (row of the local operator), s2 = ket, k indexes qop, (qin,qout)
 * the auxiliary QNs of the block, (row,col) the position inside the block.   */
typedef struct {
    int64_t        nnz;
    const int32_t* s1;
    const int32_t* s2;
    const int32_t* k;
    const int32_t* qin;     /* [nnz*nq] */
    const int32_t* qout;    /* [nnz*nq] */
    const int32_t* row;
    const int32_t* col;
    const double*  val;
    int32_t        nloc;
    const int32_t* qloc;    /* [nloc*nq] local basis QNs */
    int32_t        nop;
    const int32_t* qop;     /* [nop*nq] operator QNs */
} vmps_mpo_site;

/* ---- cost / structure report of a prepared contraction ----------------------*/
typedef struct {
    int64_t n_tasks;          /* reference task count: sum_q qrhs[q].size()             */
    int64_t n_chains;         /* (out, X, Y, Z) triple products after merging duplicates */
    int64_t n_chains_raw;     /* triple products the reference loop evaluates            */
    int64_t n_intermediates;  /* shared first-stage products                             */
    int64_t n_out_blocks;
    int64_t n_tiles_phase1;
    int64_t n_tiles_phase2;
    double  flops_reference;  /* sum over raw chains of 2*min(mkn+mnp, knp+mkp)          */
    double  flops_merged;     /* same rule on the merged chain list (algorithmic count)  */
    double  flops_executed;   /* flops the two grouped-GEMM phases perform                */
    double  flops_phase1;
    double  flops_phase2;
    double  bytes_algorithmic;/* 8*(distinct X,Z blocks used + |Y| + |out|)              */
    double  bytes_intermediate;/* device bytes of the shared first-stage products          */
    int64_t n_segments_phase2;/* (out, B-operand) groups of the second stage              */
    int64_t n_terms_phase2;   /* first-stage products summed into them                    */
    double  flops_phase2_unsummed; /* second stage without summing first-stage products    */
    int32_t association;      /* 0: (X*Y)*Z first, 1: X*(Y*Z) first                      */
    int32_t reserved;
    /* split precision: bf16 tensor-core flops the MMAs issue per phase, tile
     * padding included (3 products x 2 x 128 x round16(tile width) x 32 per K step) */
    double  tensor_flops_phase1;
    double  tensor_flops_phase2;
} vmps_plan_stats;

typedef struct vmps_ctx_s   vmps_ctx;
typedef struct vmps_pivot_s vmps_pivot;
typedef struct vmps_env_s   vmps_env;
typedef struct vmps_dvec_s  vmps_dvec;

/* ---- context ----------------------------------------------------------------*/
int         vmps_ctx_create(int device, vmps_ctx** out);
int         vmps_ctx_destroy(vmps_ctx* ctx);
/* Clock-cycle budget of every main-loop barrier wait in the split-precision
 * (tcgen05) engine of this context; 0 restores the default (about 2 s).  When a
 * wait runs out the kernel stops issuing work, lets the copies and tensor-core
 * operations already in flight finish (those drain waits keep the full budget),
 * releases its tensor memory and returns; the call then fails with
 * VMPS_E_TIMEOUT and the context stays usable.  A budget shorter than the
 * engine's normal wait times makes that path run on purpose (failure tests).
 * The reference has no device waits; this has no counterpart there.           */
int         vmps_ctx_set_wait_budget(vmps_ctx* ctx, int64_t cycles);
const char* vmps_last_error(void);
const char* vmps_version(void);

/* ---- effective Hamiltonians (PivotMatrix1 / PivotMatrix2 / PivotMatrix0) -------
 * Builds the task list once on the host (restating precalc_blockStructure,
 * tensors/DmrgIndexGymnastics.h:487-590 and :699-856), folds every W value and
 * SU(2) prefactor into one scalar per (out, L_a, V, R_b) chain, merges
 * duplicates, plans the grouped GEMMs and uploads L and R to the device.
 * V describes the PivotVector layout (Vin and Vout share it, as the reference's
 * `Vout = Vin; OxV(...)` does, pivot/DmrgPivotMatrix1.h:127).
 * For pivot2, V.leg is the combined index s1s3 of Qbasis::combine
 * (tensors/Qbasis.h:685-798) of qloc12 x qloc34.                               */
int vmps_pivot1_create(vmps_ctx* ctx, const vmps_symmetry* sym,
                       const vmps_blocks* L, const double* Ldata,
                       const vmps_blocks* R, const double* Rdata,
                       const vmps_mpo_site* W, const vmps_blocks* V,
                       vmps_pivot** out);
int vmps_pivot2_create(vmps_ctx* ctx, const vmps_symmetry* sym,
                       const vmps_blocks* L, const double* Ldata,
                       const vmps_blocks* R, const double* Rdata,
                       const vmps_mpo_site* W12, const vmps_mpo_site* W34,
                       const vmps_blocks* V, vmps_pivot** out);
int vmps_pivot0_create(vmps_ctx* ctx, const vmps_symmetry* sym,
                       const vmps_blocks* L, const double* Ldata,
                       const vmps_blocks* R, const double* Rdata,
                       const vmps_blocks* V, vmps_pivot** out);
/* Pivots with several terms: PivotMatrix1::Terms / PivotMatrix2::Terms
 * (pivot/DmrgPivotMatrix1.h:56, the sum over terms at :273-287; the same in
 * pivot/DmrgPivotMatrix2.h).  Term t has its own environments L[t], R[t] and MPO
 * tensors W[t] (two-site: W12[t], W34[t]); all terms share the PivotVector layout
 * V.  HxV returns the sum over terms, computed as one grouped HxV.  nterms = 1 is
 * the same as vmps_pivot1_create / vmps_pivot2_create.                         */
int vmps_pivot1_create_terms(vmps_ctx* ctx, const vmps_symmetry* sym, int nterms,
                             const vmps_blocks* const* L, const double* const* Ldata,
                             const vmps_blocks* const* R, const double* const* Rdata,
                             const vmps_mpo_site* const* W, const vmps_blocks* V,
                             vmps_pivot** out);
int vmps_pivot2_create_terms(vmps_ctx* ctx, const vmps_symmetry* sym, int nterms,
                             const vmps_blocks* const* L, const double* const* Ldata,
                             const vmps_blocks* const* R, const double* const* Rdata,
                             const vmps_mpo_site* const* W12, const vmps_mpo_site* const* W34,
                             const vmps_blocks* V, vmps_pivot** out);
/* Excited-state projector of PivotMatrix1/2 (A0proj, Epenalty;
 * pivot/DmrgPivotMatrix1.h:64-68, applied at :304-331): after every HxV of the
 * pivot, for n < nproj, Vout += Epenalty * <A0_n|Vin> * A0_n, the overlap being the
 * plain sum over blocks of tr(A0_n^dagger Vin) as the reference takes it (no SU(2)
 * weight).  A0 holds nproj vectors in the compact layout of V (vector n at
 * n * dim); blocks of A0proj that V's layout lacks drop out, as they do in the
 * reference.  Applies to vmps_hxv, vmps_hxv_device, vmps_hxv_multi (at most 64
 * right-hand sides), the Lanczos solves and the Chebyshev moments.  nproj = 0
 * removes the projector.                                                       */
int vmps_pivot_set_penalty(vmps_pivot* p, int nproj, const double* A0, double Epenalty);
int vmps_pivot_destroy(vmps_pivot* p);
int vmps_pivot_stats(const vmps_pivot* p, int precision, vmps_plan_stats* out);
/* number of doubles of a PivotVector in the compact layout of V */
int vmps_pivot_dim(const vmps_pivot* p, int64_t* out);
/* The task list of a pivot as chains out += c * L[x] * V[y] * R[z] (block indices of
 * the tables the pivot was made from), in the builder's order, and the reference's
 * task count: the precalc_blockStructure result of the pivot
 * (tensors/DmrgIndexGymnastics.h:487-590, 699-856).  cap = 0 returns the count only;
 * otherwise idx holds 4 entries (out, x, y, z) and coef one per chain.               */
int vmps_pivot_chains(const vmps_pivot* p, int64_t cap, int64_t* n, int64_t* idx, double* coef, int64_t* n_tasks);

/* Autotuner of the split-precision grouped GEMM (the reference picks a product
 * order per chain, DmrgExternal.h:141-215; here the tile shape of the whole
 * grouped launch is chosen).  Candidates: tile N caps of 256 or 128 columns for
 * each of the two phases and a split-K of 1, 2 or 4 for the second phase (more
 * than 1 only when that phase has fewer tiles than twice the SM count; the parts
 * are summed in a fixed order, so results stay deterministic).  Each candidate is
 * timed on this pivot (the median of `trials` HxVs, CUDA events, after a warm-up)
 * and the fastest kept if it beats the default (256, 256, 1) by 2 %.  The choice is cached for the process under the
 * pivot's sector-layout key (the histogram of its chains' block sizes); a pivot
 * whose key is cached takes the cached choice without timing, and with the
 * environment variable VMPS_AUTOTUNE=1 every new layout is tuned (3 trials) when
 * its first split plan is built.  The FP64 plan is not affected.               */
typedef struct {
    int32_t ncap1, ncap2, splitk;  /* the chosen tiling                               */
    int32_t candidates;            /* plans timed (0 when the choice came from the cache) */
    int32_t from_cache;
    int32_t reserved;
    double  ms_default, ms_best;   /* ms per HxV of the default and the chosen plan    */
    uint64_t layout_key;
} vmps_tune_info;
int vmps_pivot_autotune(vmps_pivot* p, int trials, vmps_tune_info* out);
int vmps_tune_cache_clear(void);
/* Set the split-precision tiling of a pivot directly (N caps multiples of 32 up to
 * 256, split-K 1..8), bypassing the tuner; the plan is rebuilt on next use.    */
int vmps_pivot_set_tiling(vmps_pivot* p, int ncap1, int ncap2, int splitk);

/* HxV with host buffers in the compact layout of V: Vout = H * Vin.
 * Host->device copy, the product and the device->host copy all happen here
 * (split-precision plans of large vectors overlap the copies of some chunks with
 * the compute of others).
 * Replaces HxV(PivotMatrixN, Vin, Vout), pivot/DmrgPivotMatrix1.h:124-129.  */
int vmps_hxv(vmps_pivot* p, const double* vin, double* vout, int precision);

/* ---- device-resident PivotVectors (Lanczos vectors) ---------------------------*/
int vmps_dvec_create(vmps_pivot* p, vmps_dvec** out);
int vmps_dvec_destroy(vmps_dvec* v);
int vmps_dvec_upload(vmps_dvec* v, const double* host);     /* compact layout */
int vmps_dvec_download(const vmps_dvec* v, double* host);
/* Vout = H * Vin, both on the device (no host copies). */
int vmps_hxv_device(vmps_pivot* p, const vmps_dvec* vin, vmps_dvec* vout, int precision);
/* dot with the SU(2) weight coeff_dot(qout) of pivot/DmrgPivotVector.h:296-339 */
int vmps_dvec_dot(const vmps_dvec* a, const vmps_dvec* b, double* out);
/* y += alpha*x (addScale, pivot/DmrgPivotVector.h:289-293) */
int vmps_dvec_axpy(double alpha, const vmps_dvec* x, vmps_dvec* y);
int vmps_dvec_scale(vmps_dvec* x, double alpha);
int vmps_dvec_copy(const vmps_dvec* src, vmps_dvec* dst);
/* synchronise the pivot's stream and time n device HxVs with CUDA events */
int vmps_hxv_time(vmps_pivot* p, const vmps_dvec* vin, vmps_dvec* vout, int precision,
                  int n_iter, int use_graph, double* ms_per_hxv, double* ms_phase2);

/* ---- Lanczos ground state on the device ----------------------------------------
 * Full-reorthogonalisation Lanczos (the reference calls the external
 * LanczosSolver<PivotMatrix,PivotVector>::edgeState, solvers/DmrgSolver.h:1306-1313)
 * run on the device: one iteration (HxV, the three-term recurrence, one full
 * Gram-Schmidt pass, alpha, beta, the next Krylov vector) is a CUDA graph the host
 * replays while it solves the tridiagonal problem one iteration behind.
 * precision VMPS_PREC_BF16X3 first applies FP64 HxV once to the start vector: if its
 * residual is below 1e-5 of its energy (a converged neighbourhood the split
 * operator cannot resolve) the solve continues as FP64 Lanczos.  Otherwise it runs
 * the Krylov phase with split-precision HxV and refines its Ritz vector x in
 * rounds: one FP64 HxV gives x's Rayleigh quotient E and residual r = Hx - Ex;
 * a split-precision Lanczos run from the pair (x, r/|r|), whose first tridiagonal
 * row (E, |r|) is FP64-exact, solves the correction equation and gives the next x.
 * It stops when |r| <= tol_state and |r|^2 / gap <= tol_eigval |E| (gap from the
 * last run's Ritz values); a round that does not halve |r| hands the rest of the
 * budget to FP64 Lanczos steps.  Where an FP64 HxV costs fewer than ten split
 * Lanczos steps (a cost model of the two plans, so the choice is the same in every
 * run) the residual instead drives a Jacobi-Davidson correction inside the split
 * Krylov space, followed by FP64 Lanczos steps; the environment variable
 * VMPS_LANCZOS_REFINE = rounds | polish | auto overrides the choice, and
 * VMPS_LANCZOS_PROBE = off skips the FP64 probe (the split phase always runs).  refine_iters
 * counts the FP64 HxVs after the Krylov phase (the probe is one more).
 * Krylov vectors, dots and the tridiagonal solve are FP64 throughout.  v (compact
 * layout) is the start vector on entry and the ground state on exit.
 * max_iter and refine_iters are below 1024.                                     */
typedef struct {
    int32_t iterations;        /* Krylov steps in the first phase            */
    int32_t refine_iterations; /* refinement rounds (+ closing FP64 steps)    */
    int32_t hxv_fp64;
    int32_t hxv_split;
    double  energy_first;      /* eigenvalue after the first phase            */
    double  residual;          /* ||H v - E v|| of the returned vector: the
                                  FP64 residual when refined, else |beta_m y_m|
                                  of the Lanczos run for its operator           */
    double  ms_total;
    double  ms_wait;           /* host time blocked on the device's iterations */
    double  ms_host;           /* host time in the tridiagonal solves          */
} vmps_lanczos_stats;
int vmps_lanczos_ground(vmps_pivot* p, double* v, int precision, int max_iter,
                        double tol_eigval, double tol_state, int refine_iters,
                        double* energy, vmps_lanczos_stats* stats);

/* ---- two-site tensor ---------------------------------------------------------------
 * contract_AA2 (tensors/DmrgContractions.h:1870-1927, abelian QNs): V[k] = sum over the
 * given (k, i, j) triples of A1[i] * A2[j] (block products), as one FP64 grouped GEMM on
 * the device; prods holds nprod triples, V's blocks without a product are zero.   */
int vmps_two_site_contract(vmps_ctx* ctx, const vmps_symmetry* sym, const vmps_blocks* A1, const double* a1,
                           const vmps_blocks* A2, const double* a2, const vmps_blocks* V, double* v,
                           int64_t nprod, const int64_t* prods);
/* General grouped block products: C[k] = sum over the given (k, i, j) triples of
 * coef[q] * A[i] * B[j] (coef NULL: all 1), one FP64 grouped GEMM on the device;
 * C's blocks without a product are zero.  Used for the subspace-expansion term of
 * RICH_SVD (Mps::enrich_left / enrich_right, Mps.h:3181-3600): alpha * w * L_a * A
 * and alpha * w * A * R_b, each into its column (row) range of the expansion block. */
/* 6j symbols {j1 j2 j3; j4 j5 j6} for n argument sets, each given as the multiplet
 * dimensions q = 2j + 1 (q[6*i .. 6*i+5]); zero where a triangle rule fails.  The Racah
 * formula the task builder folds into its SU(2) prefactors (the reference takes
 * coupling_6j for SU2::coeff_6j, symmetry/SU2.h:378-386); callers use it for host-side
 * recoupling, e.g. the SU(2) two-site contraction and split (contract_AA2 /
 * split_AA2, tensors/DmrgContractions.h:1870-1927, 2461-2631).  Host only.     */
int vmps_su2_coupling_6j(int64_t n, const int32_t* q, double* out);
int vmps_block_products(vmps_ctx* ctx, const vmps_symmetry* sym, const vmps_blocks* A, const double* a,
                        const vmps_blocks* B, const double* b, const vmps_blocks* C, double* c,
                        int64_t nprod, const int64_t* prods, const double* coef);
/* The same with the products found here: for every A1 block (s1, qin, qmid) and A2
 * block (s3, qmid, qout), the V block (s13_of_pair[s1 * n3 + s3], qin, qout) if V has
 * it (abelian QNs: each pair of local states is one combined state).            */
int vmps_two_site_contract_pairs(vmps_ctx* ctx, const vmps_symmetry* sym, const vmps_blocks* A1, const double* a1,
                                 const vmps_blocks* A2, const double* a2, const vmps_blocks* V, double* v,
                                 int n1, int n3, const int32_t* s13_of_pair);

/* ---- two-site split on the host cores ----------------------------------------------
 * split_AA2 with Biped::truncateSVD (tensors/DmrgContractions.h:2461-2631,
 * tensors/Biped.h:744-932), abelian QNs.  For every middle QN qmid the blocks of the
 * two-site tensor V (leg = combined index s13 = (pair1[s13], pair3[s13])) form the
 * sector matrix Psi[(s1, qin), (s3, qout)], qin + qloc1[s1] = qmid = qout - qloc3[s3],
 * rows in (s1, sorted qin) order and columns in (s3, sorted qout) order.  Its singular
 * values and the orthonormal factor of the sweep direction come from the eigensystem
 * of the Gram matrix (Psi Psi^T for move_right, Psi^T Psi otherwise; LAPACK dsyevd).
 * The dmax largest values over all sectors are kept (none at or below eps_svd times
 * the largest; ties at the threshold in sector order), renormalised; move_right: A1 = U,
 * A2 = S V^T, else A1 = U S, A2 = V^T.  A1 and A2 come in site-layout block order
 * (for s, for qin in sorted order, qout = qin + qloc[s] when present), compact
 * column-major data.  Sectors run on `threads` host threads (one LAPACK call each:
 * the caller keeps that LAPACK single-threaded meanwhile).
 * vmps_hostla_load binds the ILP64 LAPACK / BLAS (dsyevd, dsyrk, dgemm, optionally
 * with a scipy_ prefix) of the shared library at `path` (numpy's bundled OpenBLAS).
 * Results: vmps_split_info gives the counts, vmps_split_get copies out
 * (qmid: nmid * nq, dmid: nmid; then A1's and A2's tables and data).              */
typedef struct {
    int32_t nq;
    int32_t n1, n3, n13;                        /* local dims; combined dim        */
    const int32_t* qloc1;                       /* [n1 * nq]                       */
    const int32_t* qloc3;                       /* [n3 * nq]                       */
    const int32_t* pair1;                       /* [n13]: s1 of combined index     */
    const int32_t* pair3;                       /* [n13]: s3 of combined index     */
    int32_t nin;  const int32_t* qin;  const int64_t* din;    /* left bond basis  */
    int32_t nout; const int32_t* qout; const int64_t* dout;   /* right bond basis */
    int64_t dmax;
    double  eps_svd;
    int32_t move_right;
    int32_t threads;
} vmps_split_args;
typedef struct vmps_split_s vmps_split;
/* Gauge step of a single-site sweep (Mps::sweepStep with QR, Mps.h; Biped::QR,
 * tensors/Biped.h): move_right: for every outgoing QN the blocks of A (stacked by
 * rows in table order) are replaced by Q of their reduced QR, and the blocks of the
 * right neighbour N with that incoming QN are multiplied by R from the left; otherwise
 * the LQ form for every incoming QN (blocks side by side, scaled by w[i] when w is not
 * NULL, the SU(2) weights sqrt(q_out / q_in)), and N's blocks with that outgoing QN
 * are multiplied by L from the right.  A and N are updated in place; sectors run on
 * `threads` host threads.  Needs vmps_hostla_load.                                  */
int  vmps_gauge_step(int nq, int move_right, const vmps_blocks* A, double* a, const double* w,
                     const vmps_blocks* N, double* n, int threads);
int  vmps_hostla_load(const char* path);
int  vmps_two_site_split(const vmps_split_args* args, const vmps_blocks* V, const double* v, vmps_split** out);
/* The same split with the largest sectors on the GPU in FP64: a sector whose Gram
 * matrix has order >= VMPS_SPLIT_GPU_MIN (environment variable, 512 by default)
 * may form it with cuBLAS dsyrk, take its full eigensystem with cuSOLVER dsyevd and
 * the non-orthonormal factor with cuBLAS dgemm, on the context's stream and a host
 * thread of their own, while the host threads factor the other sectors as above.
 * Largest first, a sector goes to the device when the estimated end of the split
 * (the later of the device queue and the host threads' makespan) comes earlier;
 * VMPS_SPLIT_DEVICE=all sends every sector of order >= VMPS_SPLIT_GPU_MIN.  The
 * truncation rule and the output layout are the host routine's.  Still needs
 * vmps_hostla_load for the host sectors.                                       */
int  vmps_two_site_split_device(vmps_ctx* ctx, const vmps_split_args* args, const vmps_blocks* V, const double* v,
                                vmps_split** out);
int  vmps_split_info(const vmps_split* s, int* nmid, double* disc, int64_t* nblocks1, int64_t* size1,
                     int64_t* nblocks2, int64_t* size2);
int  vmps_split_get(const vmps_split* s, int32_t* qmid, int64_t* dmid,
                    int32_t* leg1, int32_t* qin1, int32_t* qout1, int64_t* rows1, int64_t* cols1, double* a1,
                    int32_t* leg2, int32_t* qin2, int32_t* qout2, int64_t* rows2, int64_t* cols2, double* a2);
void vmps_split_destroy(vmps_split* s);

/* ---- many right-hand sides --------------------------------------------------------
 * Vout_k = H Vin_k for k < nrhs (compact layouts, vector k at element k * dim).
 * Split precision runs all right-hand sides in one grouped HxV (one vector split,
 * phase 1 with the vectors side by side, phase 2 with every vector's segments);
 * FP64 applies the plain HxV per vector.  Each right-hand side's result equals the
 * single-vector HxV bit for bit.                                                  */
int vmps_hxv_multi(vmps_pivot* p, const double* vin, double* vout, int nrhs, int precision);
/* extreme Ritz values of H after `iters` FP64 Lanczos steps from v (compact): inner
 * bounds of the spectrum for the rescaling of a polynomial expansion             */
int vmps_spectral_bounds(vmps_pivot* p, const double* v, int iters, double* emin, double* emax);
/* Chebyshev moments mu_k[n] = <v0_k| T_n((H - b)/a) |v0_k>, n < nmom, of nrhs start
 * vectors v0 (compact, vector k at k * dim) advanced together: the recursion
 * t_{n+1} = 2 H~ t_n - t_{n-1} of polyIter / MpsCompressor::polyCompress
 * (DmrgLinearAlgebra.h:550-566, solvers/MpsCompressor.h:1372-1564) on the pivot,
 * with FP64 vectors and FP64 moments; the HxVs in `precision` (split: one grouped
 * launch for all right-hand sides).  ceil(nmom/2) HxVs per vector through
 * mu_{2n} = 2<t_n,t_n> - mu_0, mu_{2n+1} = 2<t_{n+1},t_n> - mu_1.  mu: nrhs x nmom. */
typedef struct {
    int32_t steps;        /* recursion steps (HxV applications per vector)     */
    int32_t hxv;          /* steps * nrhs                                       */
    double  ms_device;    /* CUDA-event time of the steps                        */
    double  ms_per_step;
    double  ms_total;     /* the whole call, plans and copies included           */
} vmps_cheb_stats;
int vmps_chebyshev_moments(vmps_pivot* p, const double* v0, int nrhs, int nmom, double a, double b,
                           int precision, double* mu, vmps_cheb_stats* stats);
/* The same with moments per part: the layout of V is cut at block boundaries
 * part_blocks[0] = 0 < part_blocks[1] < ... < part_blocks[nparts] = number of V blocks
 * (nparts <= 8) and mu (nrhs x nparts x nmom) holds the moments of each part of each
 * vector.  On a union pivot whose parts are sectors of different quantum numbers
 * (each part closed under H; see vmps_gb300/union.py), part j of vector k is a start
 * vector of its own: one grouped launch per step advances nrhs x nparts vectors with
 * different block layouts (C5: c_k|0> for both spin projections at once).  The
 * reference runs one polyIter chain per start vector (DmrgLinearAlgebra.h:550-566). */
int vmps_chebyshev_moments_parts(vmps_pivot* p, const double* v0, int nrhs, int nmom, double a, double b,
                                 int precision, int nparts, const int64_t* part_blocks, double* mu,
                                 vmps_cheb_stats* stats);

/* ---- environment updates (contract_L / contract_R, FULL mode) -----------------
 * Step 1 builds the task list and the output Tripod layout; the caller reads the
 * layout, allocates the output data, and step 2 runs the contraction.
 * Replaces contract_L / contract_R of tensors/DmrgContractions.h:34-311.        */
#define VMPS_ENV_LEFT  0
#define VMPS_ENV_RIGHT 1
int vmps_env_create(vmps_ctx* ctx, const vmps_symmetry* sym, int side,
                    const vmps_blocks* Eold, const vmps_blocks* Abra,
                    const vmps_mpo_site* W, const vmps_blocks* Aket,
                    vmps_env** out);
/* CONTRACT_LR_MODE (tensors/DmrgContractions.h:13): restrict the W nonzeros by
 * the position of an auxiliary index in the full MPO basis, as the VUMPS
 * transfer operator does (VUMPS/VumpsMpoTransferMatrix.h:99-155):
 *   TRIANGULAR : left: order(Lold.mid, a) > fixed_ab;  right: fixed_ab > order(Rold.mid, b)
 *   FIXED_ROWS : left: order(Lold.mid, a) == fixed_ab; right: order(Lnew.mid, a) == fixed_ab
 *   FIXED_COLS : left: order(Lnew.mid, b) == fixed_ab; right: order(Rold.mid, b) == fixed_ab
 * The order map (basis_order_map) has n_order entries: QN order_qn[i*nq..],
 * index inside that QN sector order_index[i], position order_value[i].       */
#define VMPS_ENV_FULL       0
#define VMPS_ENV_TRIANGULAR 1
#define VMPS_ENV_FIXED_ROWS 2
#define VMPS_ENV_FIXED_COLS 3
int vmps_env_create_mode(vmps_ctx* ctx, const vmps_symmetry* sym, int side, int mode, int64_t fixed_ab,
                         int64_t n_order, const int32_t* order_qn, const int32_t* order_index,
                         const int64_t* order_value,
                         const vmps_blocks* Eold, const vmps_blocks* Abra,
                         const vmps_mpo_site* W, const vmps_blocks* Aket,
                         vmps_env** out);
/* output layout; arrays must hold nblocks (and nblocks*nq for QNs) entries     */
int vmps_env_layout(const vmps_env* e, int64_t* nblocks, int64_t* total_elems);
int vmps_env_layout_get(const vmps_env* e, int32_t* qin, int32_t* qout, int32_t* qmid,
                        int32_t* leg, int64_t* rows, int64_t* cols, int64_t* offset);
int vmps_env_stats(const vmps_env* e, int precision, vmps_plan_stats* out);
int vmps_env_run(vmps_env* e, const double* Eold, const double* Abra,
                 const double* Aket, double* Enew, int precision);
int vmps_env_destroy(vmps_env* e);

/* ---- VUMPS MpoTransferMatrix -----------------------------------------------
 * The linear operator (1 - T_L + |R)(1|) (dir LEFT) or (1 - T_R + |1)(L|) (dir
 * RIGHT) of the VUMPS environment equations, HxV(MpoTransferMatrix, Vin, Vout)
 * of VUMPS/VumpsMpoTransferMatrix.h:99-212:
 *   T V  = the chain of contract_L over the cell sites 0..ncell-1 (FIXED_ROWS on
 *          site 0, FIXED_COLS on site ncell-1) or of contract_R over
 *          ncell-1..0 (FIXED_COLS on site ncell-1, FIXED_ROWS on site 0);
 *   Vout = Vin - T Vin + contract_LR(ab, Vin, LReigen) * 1 on the blocks of the
 *          auxiliary slot ab (basis_order[ab], which must lie in the vacuum
 *          sector) that T Vin and Vin share; zero elsewhere.
 * Abra/Aket/W are arrays of ncell site tensors (indexed by cell site); LReigen
 * is a Biped (qin, qout, rows, cols, offset); V is the Tripod layout of the
 * transfer vector (Vin and Vout share it).  The site tensors are uploaded
 * once; vmps_transfer_hxv takes host buffers in the layout of V.              */
typedef struct vmps_transfer_s vmps_transfer;
int vmps_transfer_create(vmps_ctx* ctx, const vmps_symmetry* sym, int dir, int ncell,
                         const vmps_blocks* const* Abra, const double* const* Abra_data,
                         const vmps_blocks* const* Aket, const double* const* Aket_data,
                         const vmps_mpo_site* const* W,
                         const vmps_blocks* LReigen, const double* LReigen_data,
                         int64_t ab, int64_t n_order, const int32_t* order_qn,
                         const int32_t* order_index, const int64_t* order_value,
                         const vmps_blocks* V, vmps_transfer** out);
int vmps_transfer_hxv(vmps_transfer* t, const double* vin, double* vout, int precision);
/* Solves (1 - T + |R)(1|) x = b (the operator of vmps_transfer_hxv) on the transfer-vector
 * space (the slot-ab blocks, dot weighted by coeff_dot) by restarted GMRES on the device:
 * VumpsSolver's solve_linear (VUMPS/VumpsSolver.h:1907-1940) with the ALGS GMResSolver
 * restated.  Krylov vectors stay on the device; one iteration = the operator, two
 * classical Gram-Schmidt passes and a norm (deterministic reductions); the host keeps the
 * Hessenberg matrix and its Givens rotations and reads one column per iteration.
 * precision FP64: GMRES with the FP64 operator to tol (relative residual).  BF16X3:
 * mixed-precision refinement -- the residual r = b - A x with the FP64 operator, the
 * correction A d = r by GMRES with the split operator to inner_tol, x += d -- until the
 * FP64 residual is below tol; when a round does not halve the residual (or after
 * max_outer rounds) FP64 GMRES finishes from the best x.  b, x: compact host vectors (x
 * is overwritten; no initial guess).  Device memory: dimK + 8 vectors of the padded
 * layout, kept by the transfer operator for later solves.                              */
typedef struct {
    int32_t iterations;       /* GMRES iterations (operator applications in the Krylov loops) */
    int32_t fp64_iterations;  /* those with the FP64 operator                                 */
    int32_t outer;            /* split-precision refinement rounds (BF16X3)                   */
    int32_t fp64_hxv;         /* FP64 operator applications outside the Krylov loops          */
    int32_t restarts;
    int32_t reserved;
    double  residual;         /* final relative residual |b - A x| / |b| (FP64 operator)      */
    double  ms_total;
} vmps_gmres_stats;
int vmps_transfer_solve(vmps_transfer* t, const double* b, double* x, double tol, int dimK, int max_restarts,
                        int precision, double inner_tol, int max_outer, vmps_gmres_stats* stats);
int vmps_transfer_destroy(vmps_transfer* t);

/* ---- allocation-free chain product -------------------------------------------
 * No counterpart in the reference: an extra entry point of this library.
 * out (m x p) = alpha * op(X) * Y * op(Z) in FP64 for single dense blocks
 * (op = transpose when trans* != 0), all column-major with leading dimension =
 * rows, all pointers device pointers on the calling thread's current device.
 * It allocates nothing: the intermediate op(X) * Y sits in a fixed 8 MiB array
 * inside the library (2^20 doubles, present on every GPU that loads the library
 * until the process exits), for callers that cannot call cudaMalloc at that
 * point -- a framework that has given all device memory to its own pool, or a
 * loop that cannot afford the device synchronisation of cudaMalloc/cudaFree.
 * m * n above 2^20 returns VMPS_E_ARG.  All calls on a device share that array:
 * calls that overlap on the GPU race.  Every call looks the array's device
 * address up in the current context (no allocation), so it stays valid across
 * cudaDeviceReset; the first call on a device may load the library's device
 * code, so make that first call outside any stream capture.  `stream` is a
 * cudaStream_t (NULL = default stream); the work is asynchronous on it. */
int vmps_chain_fp64_noalloc(const double* X, int64_t x_rows, int64_t x_cols, int32_t transX,
                            const double* Y, int64_t y_rows, int64_t y_cols,
                            const double* Z, int64_t z_rows, int64_t z_cols, int32_t transZ,
                            double alpha, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VMPS_GB300_H */
