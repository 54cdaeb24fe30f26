// Internal interfaces shared by the host task-list builder (tasks.cpp), the
// device runtime / C ABI (runtime.cpp) and the kernels (kernels.cu).
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include <stdexcept>

#include "qn.hpp"
#include "../../include/vmps_gb300.h"

struct CUstream_st;   // cudaStream_t is CUstream_st*

namespace vmps {

// ---------------------------------------------------------------------------
// Host views of the C-ABI tables
// ---------------------------------------------------------------------------
struct BlockTable {
    int64_t n = 0;
    std::vector<QN> qin, qout, qmid;
    std::vector<int32_t> leg;
    std::vector<int64_t> rows, cols, off;   // compact (host) layout
    bool has_mid = false;
    int64_t total = 0;                      // elements in the compact data array
};
BlockTable parse_blocks(const Symmetry& sym, const vmps_blocks* b, bool need_mid);

// Tripod = Multipede<3>: blocks keyed by {qin,qout,qmid}, each an array over
// the auxiliary index a (tensors/Multipede.h:77-95, access T.block[q][a][0]).
struct TripodView {
    std::vector<QN3> keys;
    std::unordered_map<QN3, int, QNTupleHash<3>> dict;
    std::vector<std::vector<int64_t>> aux;    // aux[q][a] -> block row, -1 = empty
    int64_t at(int q, int a) const {
        const auto& v = aux[q];
        return (a >= 0 && a < (int)v.size()) ? v[a] : -1;
    }
};
TripodView make_tripod_view(const BlockTable& t);

// vector<Biped> (site tensor A[s] or PivotVector::data[s]); dict[s] maps {qin,qout}
struct BipedsView {
    std::vector<std::unordered_map<QN2, int64_t, QNTupleHash<2>>> dict;
    int64_t find(int s, const QN& a, const QN& b) const {
        if (s < 0 || s >= (int)dict.size()) return -1;
        auto it = dict[s].find(QN2{{a, b}});
        return it == dict[s].end() ? -1 : it->second;
    }
};
BipedsView make_bipeds_view(const BlockTable& t, int nlegs);

struct MpoNz { int32_t row, col; double val; };
struct MpoView {
    int nloc = 0, nop = 0;
    std::vector<QN> qloc, qop;
    // blocks[(s1*nloc+s2)*nop+k] : {qin,qout} -> nonzeros of W[s1][s2][k].block[qW]
    std::vector<std::unordered_map<QN2, std::vector<MpoNz>, QNTupleHash<2>>> blocks;
    const std::vector<MpoNz>* find(int s1, int s2, int k, const QN& a, const QN& b) const {
        const auto& m = blocks[((size_t)s1 * nloc + s2) * nop + k];
        auto it = m.find(QN2{{a, b}});
        return it == m.end() ? nullptr : &it->second;
    }
};
MpoView parse_mpo(const Symmetry& sym, const vmps_mpo_site* W);

// ---------------------------------------------------------------------------
// Chains: out[o] += c * op(X[x]) * Y[y] * op(Z[z])
//   HxV (1-,2-,0-site): X = L_a, Y = V, Z = R_b          (no transposes)
//   contract_L        : X = Abra^dagger, Y = Lold_a, Z = Aket
//   contract_R        : X = Aket, Y = Rold_b, Z = Abra^dagger
// ---------------------------------------------------------------------------
struct Chain { int64_t out, x, y, z; double c; };

struct ChainSet {
    std::vector<Chain> chains;
    int64_t n_tasks = 0;        // sum_q qrhs[q].size() of the reference task list
    int64_t n_chains_raw = 0;   // (task, W-nonzero) products the reference evaluates
    double flops_reference = 0; // 2*min(...) summed over those raw products
};

// builders (tasks.cpp)
ChainSet build_pivot1(const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                      const MpoView& W, const BlockTable& V);
ChainSet build_pivot2(const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                      const MpoView& W12, const MpoView& W34, const BlockTable& V);
ChainSet build_pivot0(const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                      const BlockTable& V);
// the same chain lists as build_pivot2 / build_pivot1, matched on the GPU (abelian
// symmetries; builder.cu)
ChainSet build_pivot2_device(CUstream_st* st, const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                             const MpoView& W12, const MpoView& W34, const BlockTable& V);
ChainSet build_pivot1_device(CUstream_st* st, const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                             const MpoView& W, const BlockTable& V);
// the reference's chain cost (DmrgExternal.h:147-159), for the builders' flop counts
double chain_flops_ref(double m, double k, double n, double p);
// contract_L / contract_R modes (tensors/DmrgContractions.h:13, :100-104, :245-249):
// basis_order_map (MPO auxiliary QN, index inside its sector) -> position in the full auxiliary basis
struct AuxKey {
    QN q; int32_t idx;
    bool operator==(const AuxKey& o) const { return q == o.q && idx == o.idx; }
};
struct AuxKeyHash {
    size_t operator()(const AuxKey& k) const { return QNHash()(k.q) * 1000003u ^ (size_t)(uint32_t)k.idx; }
};
struct EnvMode {
    int mode = VMPS_ENV_FULL;
    int64_t fixed_ab = 0;
    std::unordered_map<AuxKey, int64_t, AuxKeyHash> order;
    int64_t at(const QN& q, int32_t idx) const {
        auto it = order.find(AuxKey{q, idx});
        if (it == order.end()) throw std::invalid_argument("basis_order_map has no entry for an auxiliary index in use");
        return it->second;
    }
};
// contract_L / contract_R: also derives the output Tripod layout
ChainSet build_env(const Symmetry& sym, int side, const BlockTable& Eold, const BlockTable& Abra,
                   const MpoView& W, const BlockTable& Aket, BlockTable* Enew, const EnvMode& mode = EnvMode());

// combined two-site index s1s3 of Qbasis::combine (tensors/Qbasis.h:685-798)
struct CombinedBasis {
    int n = 0;
    // index[(s1*n34+s3)] -> vector of (qmerge, s1s3)
    std::vector<std::vector<std::pair<QN, int>>> index;
    std::vector<QN> q_of;   // QN of combined state
};
CombinedBasis combine_bases(const Symmetry& sym, const std::vector<QN>& q12, const std::vector<QN>& q34);

// ---------------------------------------------------------------------------
// Grouped-GEMM plan (device work lists)
// ---------------------------------------------------------------------------
// Device block layout: column-major, ld = rows rounded up to 8, block starts
// aligned to 32 elements; padding stays zero.
inline int64_t pad_ld(int64_t rows) { return (rows + 7) / 8 * 8; }
inline int64_t pad_off(int64_t x) { return (x + 31) / 32 * 32; }

struct DevLayout {             // one arena (L, R, V, T ...)
    std::vector<int64_t> off, rows, cols, ld;
    int64_t total = 0;         // elements incl. padding
};
DevLayout make_dev_layout(const std::vector<int64_t>& rows, const std::vector<int64_t>& cols);

// GPU work items (POD, copied verbatim to the device)
struct GTerm { int64_t off; double coef; };
// (split plans: akoff = K offset of the A operand inside its panel rows, a multiple of
// 32; nonzero for the right-hand sides after the first of a multi-RHS plan)
struct GSeg  { int64_t b_off; int32_t term_begin, term_count; int32_t lda, ldb, K, akoff; };
// one output tile: rows [row0, row0+tm) x cols [col0, col0+tn) of a block
// (split plans: step0 / nsteps index its K steps in PhasePlan::steps)
// (multi-RHS split plans: rstride = the per-right-hand-side column stride ycolsP of a
// phase-1 tile, nrhs = R on every tile of the plan; the intermediates' panel rows and
// the phase-2 tile rows are interleaved, row R*i + k = row i of right-hand side k)
struct GTile { int64_t c_off; int32_t ldc, row0, col0, tm, tn, seg_begin, seg_end, step0, nsteps, rstride, nrhs; };
// at most this many A terms per segment (the FP64 kernel stages them in shared memory)
constexpr int kMaxTerms = 16;
// FP64 engine tiles are at most 64 x 64 (rows split on multiples of 16, columns
// on multiples of 8); tcgen05 engine tiles at most 128 x 256
constexpr int kTileMax = 64;
constexpr int kUmmaTileM = 128, kUmmaTileN = 256;
constexpr int kUmmaBK = 32;   // K extent of one tcgen05 engine step

// ---------------------------------------------------------------------------
// Split-precision operand panels
// ---------------------------------------------------------------------------
// Every split operand lives in one bf16 arena made of "class panels".  Blocks
// with the same padded contraction length kpad (panel_kpad(K)) are stacked as
// consecutive rows of one row-major matrix whose rows are kpad/32 chunks of
// [32 hi | 32 lo] elements, so row pitch = 2*kpad elements:
//     element (row i, k) of a block:  hi at off + i*pitch + (k/32)*64 + k%32,
//                                     lo at the same position + 32.
// One 128-byte row segment holds the hi and lo halves of one 32-wide K step,
// which is exactly one TMA request per row and one 128-byte-swizzled row of the
// tensor-core operand.  Padding (k >= K) is zero.
int32_t panel_kpad(int64_t K);
struct PanelClass { int32_t kpad; int64_t base, rows; };   // base: element offset; rows: stacked rows
struct PanelArena {
    std::vector<PanelClass> cls;
    int64_t total = 0;                                      // elements (hi and lo together)
};
// a block of a panel arena: `outer` rows of contraction length K, at row `row`
// of class `cls`; off = element offset of its row 0, pitch = 2*kpad of the class
struct OpBlock { int64_t off; int32_t outer, K, cls, row, pitch, pad; };

// one K step of the tcgen05 engine: TMA descriptors (indices into the phase's
// descriptor lists) of A and B, x = 2*k0 (column of the B operand's [hi|lo]
// panel; bit 0 set when only the step's first 16 K columns lie inside the
// segment), the panel rows the A and B boxes start at, the box heights, and
// xa = 2*(akoff + k0), the column of the A operand's panel
struct TStep { int32_t amap, bmap, x, ay, by, arows, brows, xa; };
// a TMA descriptor of a phase: box of `rows` rows over the panel matrix of class `cls`
struct MapKey { int32_t cls, rows; };
constexpr int kMaxMapsA = 64, kMaxMapsB = 128;

struct PhasePlan {
    std::vector<GTerm> terms;
    std::vector<GSeg>  segs;
    std::vector<GTile> tiles;
    // split plans: per segment, the A and B operand block (OpBlock index)
    std::vector<int32_t> seg_amap, seg_bmap;
    // tcgen05 engine schedule (schedule_tma): K steps, descriptors, and the tiles
    // of CTA b are tiles[cta_tiles[b] .. cta_tiles[b+1])
    std::vector<TStep> steps;
    std::vector<MapKey> amaps, bmaps;
    std::vector<int32_t> cta_tiles;
    int ncta = 0;
    bool transA = false, transB = false, transC = false;
    int  slotA = 0, slotB = 0, slotC = 0;   // arena ids
    double flops = 0;
};

enum Slot { SLOT_X = 0, SLOT_Y = 1, SLOT_Z = 2, SLOT_OUT = 3, SLOT_T = 4 };

// Split-precision operand preparation: one block of a column-major FP64 source
// (rows x cols, leading dimension src_ld) written into its panel (dst_off,
// dst_ld = panel pitch).  trans = 0: panel row j holds source column j (K runs
// down the column); trans = 1: panel row i holds source row i.
struct PrepBlock { int64_t src_off, dst_off; int32_t src_ld, dst_ld, rows, cols, trans, pad; double scale; };

struct Plan {
    PhasePlan p1, p2;
    DevLayout T;               // FP64 plans: intermediate arena layout
    int association = 0;       // 0: T = op(X)*Y first; 1: U = Y*op(Z) first
    int64_t n_chains = 0, n_intermediates = 0, n_out_blocks = 0;
    double flops_merged = 0, bytes_alg = 0;
    double flops_p2_unsummed = 0;
    // split-precision plans only
    bool split = false;
    PanelArena ax, ay, at, az;                    // panels of op(X), Y, T = op(X)Y, c*op(Z)
    std::vector<PrepBlock> prepX, prepZ;          // X blocks, and c*op(Z) copies
    std::vector<OpBlock> opX, opY, opZ, opT;      // blocks of each panel arena
    // multi-RHS split plans: nrhs vectors Y_k (and outputs O_k) at element stride
    // Y.total (O.total = vstride); V block y's panel holds rhs k's columns from
    // panel row k * ycolsP[y] on (ycolsP = cols rounded up to 32 when nrhs > 1);
    // phase 1 writes the intermediate of rhs k to the interleaved panel rows R*i + k,
    // so one phase-2 tile (R*m rows) serves every right-hand side of its rows
    int nrhs = 1;
    int64_t vstride = 0;
    std::vector<int32_t> ycolsP;
    // split-K of phase 2 (single right-hand side): part j of every output block's
    // K concatenation writes the whole block at element offset j * vstride of a
    // partial buffer; a reduction sums the parts in order into the output
    int splitk = 1;
    // panel element: bf16 (elt 2; a 128-byte row segment is [32 hi | 32 lo], one K
    // step of 32) or tf32 in FP32 storage (elt 4; [16 hi | 16 lo], one K step of 16).
    // Offsets, pitches and TMA x coordinates are in elements either way (x = 2 * k0).
    int elt = 2;
    int kstep = kUmmaBK;
};
// Tile options of a split-precision plan (chosen by the autotuner): the N caps of
// the phase-1 and phase-2 tiles (multiples of 32, at most kUmmaTileN) and the
// split-K factor of phase 2.
struct SplitTiling {
    int ncap1 = 256, ncap2 = 256, splitk = 1;
    bool operator==(const SplitTiling& o) const { return ncap1 == o.ncap1 && ncap2 == o.ncap2 && splitk == o.splitk; }
};
// FP64 plan: two phases, the second sums first-stage products on the fly
Plan make_plan(const ChainSet& cs, const DevLayout& X, const DevLayout& Y, const DevLayout& Z,
               const DevLayout& O, bool transX, bool transZ, int tile_m, int tile_n);
// Split-precision plan for the tcgen05 engine: op(X), Y and the chain-scaled
// copies c*op(Z) in panels; phase 1 computes the intermediates T = op(X)Y into
// panels, phase 2 the outputs as K-concatenations over chains.
// nrhs > 1: the same contraction applied to nrhs vectors at once (phase 1 one
// GEMM per V block with the right-hand sides side by side in N; phase 2 the
// single-vector segments once per right-hand side, reading its K range of T).
Plan make_split_plan(const ChainSet& cs, const DevLayout& X, const DevLayout& Y, const DevLayout& Z,
                     const DevLayout& O, bool transX, bool transZ, int nrhs = 1,
                     const SplitTiling& tiling = SplitTiling(), bool tf32 = false);
// One FP64 grouped-GEMM phase of plain block products C[k] = sum A[i] * B[j] over
// the (k, i, j) triples (contract_AA2's two-site tensor): one tile range per
// output block, one segment per product; output blocks without a product are
// written with zeros.
PhasePlan make_product_plan(const DevLayout& A, const DevLayout& B, const DevLayout& C,
                            const std::vector<std::array<int64_t, 3>>& prods, const double* coef = nullptr);
// Static schedule of a split phase for the persistent tcgen05 engine on ncta
// CTAs: K steps of kUmmaBK per segment with their TMA boxes, tiles assigned
// longest-first to the least-loaded CTA and stored CTA by CTA.
void schedule_tma(PhasePlan& ph, int ncta, const std::vector<OpBlock>& A, const std::vector<OpBlock>& B,
                  int kstep = kUmmaBK);
// TMA box heights, the smallest that covers the tile: fine = the tile's rows
// (columns) rounded up to 16; coarse (fewer descriptors) = A boxes of 16/32/64/128
// rows, B boxes a multiple of 32 up to 256 (16 for the narrowest)
int32_t box_rows_a(int32_t tm, bool fine = true);
int32_t box_rows_b(int32_t tn, bool fine = true);

}  // namespace vmps
