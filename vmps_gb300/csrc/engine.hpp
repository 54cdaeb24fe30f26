// Internal interfaces shared by the host task-list builder (tasks.cpp), the
// device runtime / C ABI (runtime.cpp) and the kernels (kernels.cu).
#pragma once
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include <stdexcept>

#include "qn.hpp"
#include "../../include/vmps_gb300.h"

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
struct GSeg  { int64_t b_off; int32_t term_begin, term_count; int32_t lda, ldb, K, pad; };
// one output tile: rows [row0, row0+tm) x cols [col0, col0+tn) of a block
// (tcgen05 engine: step0 / nsteps index its K steps in PhasePlan::steps)
struct GTile { int64_t c_off; int32_t ldc, row0, col0, tm, tn, seg_begin, seg_end, step0, nsteps; };
// one K step of the tcgen05 engine: TMA descriptors of A and B, the K offset in
// the segment and the tile origin; flags bit 0 / bit 1: first use of the A / B
// descriptor by this CTA (acquire it for the tensor-map proxy); brows: rows of
// the B box (the tile's MMA N, a multiple of 16, is at most this)
struct TStep { int32_t amap, bmap, k0, row0, col0, flags, brows, pad; };
constexpr int kUmmaBK = 32;   // K extent of one tcgen05 engine step
// at most this many A terms per segment (the kernels stage them in shared memory)
constexpr int kMaxTerms = 16;
// tile edges (rows split on multiples of 16, columns on multiples of 8):
// mma.sync engines at most 64 x 64, the tcgen05 engine at most 128 x 64
constexpr int kTileMax = 64;
constexpr int kUmmaTileM = 128, kUmmaTileN = 256;

struct PhasePlan {
    std::vector<GTerm> terms;
    std::vector<GSeg>  segs;
    std::vector<GTile> tiles;
    // split plans: per segment, the prepared-operand block of A and of B (TMA descriptor index)
    std::vector<int32_t> seg_amap, seg_bmap;
    // tcgen05 engine schedule (schedule_tma): K steps, and the tiles of CTA b are
    // tiles[cta_tiles[b] .. cta_tiles[b+1])
    std::vector<TStep> steps;
    std::vector<int32_t> cta_tiles;
    int ncta = 0;
    bool transA = false, transB = false, transC = false;
    int  slotA = 0, slotB = 0, slotC = 0;   // arena ids
    double flops = 0;
};

enum Slot { SLOT_X = 0, SLOT_Y = 1, SLOT_Z = 2, SLOT_OUT = 3, SLOT_T = 4 };

// A prepared split-precision operand block: `outer` rows (rows of A / columns of
// B) of K contiguous elements, row stride ld, at element offset off of its
// [hi | lo] arena (lo half at +total); box: rows of its TMA box (tcgen05 engine)
struct OpBlock { int64_t off; int32_t outer, K, ld, box; };

// Split-precision operand preparation: one block of a column-major FP64 source
// (rows x cols, leading dimension src_ld) written as bf16 hi/lo pairs in the
// K-contiguous layout the tensor-core kernels read.  trans = 0: destination row
// j holds source column j; trans = 1: destination row i holds source row i.
struct PrepBlock { int64_t src_off, dst_off; int32_t src_ld, dst_ld, rows, cols, trans, pad; double scale; };

struct Plan {
    PhasePlan p1, p2;
    DevLayout T;               // intermediate arena layout
    int association = 0;       // 0: T = op(X)*Y first; 1: U = Y*op(Z) first
    int64_t n_chains = 0, n_intermediates = 0, n_out_blocks = 0;
    double flops_merged = 0, bytes_alg = 0;
    double flops_p2_unsummed = 0;
    // split-precision plans only
    bool split = false;
    int split_kernel = 0;                         // 0: mma.sync engine, 1: tcgen05 engine
    int64_t Xp_total = 0, Zp_total = 0;           // prepared-operand arena sizes (elements)
    std::vector<PrepBlock> prepX, prepZ;          // X blocks, and c*op(Z) copies
    std::vector<OpBlock> opX, opY, opZ, opT;      // prepared blocks of each arena
};
// FP64 plan: two phases, the second sums first-stage products on the fly
Plan make_plan(const ChainSet& cs, const DevLayout& X, const DevLayout& Y, const DevLayout& Z,
               const DevLayout& O, bool transX, bool transZ, int tile_m, int tile_n);
// split-precision plan: every operand pre-split into K-contiguous bf16 hi/lo
// copies; the chain coefficient rides on a scaled copy of op(Z); the second
// phase is a K-concatenation over chains
// Static schedule of a split phase for the persistent tcgen05 engine on ncta
// CTAs: K steps of kUmmaBK per segment, tiles assigned longest-first to the
// least-loaded CTA and stored CTA by CTA.
void schedule_tma(PhasePlan& ph, int ncta, const std::vector<OpBlock>& B);
// rows of the TMA box of a B operand block with `outer` rows, tiled by
// split_extent(outer, 8, tile_n): the largest tile extent rounded up to 16
int32_t b_box_rows(int64_t outer, int tile_n);
Plan make_split_plan(const ChainSet& cs, const DevLayout& X, const DevLayout& Y, const DevLayout& Z,
                     const DevLayout& O, bool transX, bool transZ, int tile_m, int tile_n);

}  // namespace vmps
