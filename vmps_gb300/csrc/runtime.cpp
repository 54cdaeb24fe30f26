// Device runtime and C ABI (include/vmps_gb300.h).
//
// One vmps_ctx = one CUDA stream on one device.  A vmps_pivot owns the device
// copies of L and R for one site (the reference's PivotMatrix owns value copies
// of L, R, W and its task list, pivot/DmrgPivotMatrix1.h:12-20,56-61), the
// grouped-GEMM work lists for each precision, and scratch for the intermediate
// products.  PivotVectors live on the device in a padded block layout
// (engine.hpp: ld multiple of 8, 32-element aligned starts, zero padding) and
// are scaled per block by sqrt(coeff_dot(qout)) so that the SU(2)-weighted
// inner product of pivot/DmrgPivotVector.h:323 becomes a plain dot product.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <cstdlib>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.hpp"
#include "kernels.hpp"

using namespace vmps;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;
static int set_err(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
namespace vmps {
void set_last_error_message(const std::string& msg) { g_last_error = msg; }
}
struct CudaFail : std::runtime_error {
    using std::runtime_error::runtime_error;
};
// a bounded device wait gave up (the device error word was set)
struct WaitTimeout : std::runtime_error {
    using std::runtime_error::runtime_error;
};
#define CK(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            throw CudaFail(std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + ":" + \
                           std::to_string(__LINE__) + ")");                                              \
    } while (0)

#define API_BEGIN try {
#define API_END                                                                 \
    }                                                                           \
    catch (const WaitTimeout& e) { return set_err(VMPS_E_TIMEOUT, e.what()); }  \
    catch (const CudaFail& e) { return set_err(VMPS_E_CUDA, e.what()); }        \
    catch (const std::bad_alloc& e) { return set_err(VMPS_E_NOMEM, e.what()); } \
    catch (const std::domain_error& e) { return set_err(VMPS_E_SHAPE, e.what()); } \
    catch (const std::invalid_argument& e) { return set_err(VMPS_E_ARG, e.what()); } \
    catch (const std::exception& e) { return set_err(VMPS_E_ARG, e.what()); }   \
    return VMPS_OK;

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            if (p) cudaFree(p);
            p = o.p; bytes = o.bytes;
            o.p = nullptr; o.bytes = 0;
        }
        return *this;
    }
    ~DBuf() { if (p) cudaFree(p); }
    void alloc(size_t b, cudaStream_t st = 0, bool zero = true) {
        if (p && bytes >= b) { if (zero) CK(cudaMemsetAsync(p, 0, b, st)); return; }
        if (p) { cudaFree(p); p = nullptr; }
        bytes = std::max<size_t>(b, 256);
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) { p = nullptr; throw std::bad_alloc(); }
        if (zero) CK(cudaMemsetAsync(p, 0, bytes, st));
    }
    template <typename T> T* as() const { return (T*)p; }
};

template <typename T> static void upload_vec(DBuf& d, const std::vector<T>& v, cudaStream_t st) {
    d.alloc(std::max<size_t>(1, v.size()) * sizeof(T), st, false);
    if (!v.empty()) CK(cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

// Krylov workspace of a context: basis, work vectors, reduction scratch and a
// host-mapped mirror of the recurrence coefficients; grown on demand and kept
// for later Lanczos runs (a DMRG sweep runs one per site).
struct LzWork {
    DBuf K, w, q, x, u, part, small;
    DBuf K32, w32, q32;           // FP32 basis and vectors of split-precision runs (allocated on first use)
    double* host = nullptr;       // pinned, mapped: alpha [cap] | beta [cap]
    double* host_dev = nullptr;   // its device address
    int cap = 0;                  // iterations the buffers hold (cap + 1 basis rows)
    int host_cap = 0;             // cap the host mirror was allocated for
    int64_t n = 0, ld = 0;        // vector length and basis row stride
    LzShape sh;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    LzWork() = default;
    LzWork(const LzWork&) = delete;
    LzWork& operator=(const LzWork&) = delete;
    ~LzWork() {
        if (host) cudaFreeHost(host);
        for (auto& e : ev) if (e) cudaEventDestroy(e);
    }
    // `small` (doubles): cl[2] | coef[cap] | ab[3 cap] | g[cap] | ctl (8 unsigned)
    double* cl() const { return small.as<double>(); }
    double* coef() const { return cl() + 2; }
    double* ab() const { return coef() + cap; }
    double* g() const { return ab() + 3 * cap; }
    unsigned* ctl() const { return (unsigned*)(g() + cap); }
};

struct TwoSiteScratch;   // device buffers of vmps_two_site_contract*

struct vmps_ctx_s {
    std::unique_ptr<LzWork> lz;   // Lanczos workspace (vmps_lanczos_ground)
    std::unique_ptr<TwoSiteScratch> two_site;
    std::mutex lz_mu;             // one Lanczos run at a time per context
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;   // host<->device transfers overlapped with compute
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    int* err = nullptr;   // device error word written by the tcgen05 engine
    bool pageable_access = false;   // the device reads pageable host memory in place
    int num_sms = 152;              // CTAs of the persistent tcgen05 engine (host-only: GB300's count)
    long long wait_budget = 0;      // main-loop wait budget of the tcgen05 engine in cycles (0: ~2 s)
    std::shared_ptr<void> la;       // device state of the two-site split (hostla.cpp)
};

// read and clear the device error word (after the stream has been synchronised)
static void check_device_error(vmps_ctx* c) {
    if (!c || !c->err) return;
    int h = 0;
    CK(cudaMemcpyAsync(&h, c->err, 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (h) {
        CK(cudaMemsetAsync(c->err, 0, 4, c->stream));
        throw WaitTimeout("a bounded device wait in the tcgen05 engine ran out (error word " + std::to_string(h) + ")");
    }
}

namespace vmps {
cudaStream_t ctx_stream(vmps_ctx* c) { return c->stream; }
int ctx_device(const vmps_ctx* c) { return c->device; }
std::shared_ptr<void>& ctx_la_slot(vmps_ctx* c) { return c->la; }
}  // namespace vmps

// device copy of one phase's work lists
struct DevPhase {
    DBuf tiles, segs, terms;
    DBuf steps, cta_tiles;   // tcgen05 engine schedule
    std::unique_ptr<TmaMaps> maps;   // tcgen05 engine: the phase's TMA descriptors (kernel parameter)
    int ntiles = 0, ncta = 0;
    const PhasePlan* host = nullptr;
    void upload(const PhasePlan& ph, cudaStream_t st) {
        host = &ph;
        ntiles = (int)ph.tiles.size();
        upload_vec(tiles, ph.tiles, st);
        upload_vec(segs, ph.segs, st);
        upload_vec(terms, ph.terms, st);
        ncta = ph.ncta;
        if (ph.ncta > 0) {
            upload_vec(steps, ph.steps, st);
            upload_vec(cta_tiles, ph.cta_tiles, st);
        }
    }
};

struct TwoSiteScratch {
    DBuf a1, a2, v, stage, pack;
    DevPhase phase;
};

// Host-buffer HxV pipeline: the vector's blocks in contiguous chunks, and each
// phase of the split plan cut into one launch per chunk -- phase 1 by the input
// chunk of its V block, phase 2 by the output chunk of its output block -- so
// that transfers of one chunk overlap the compute of another.  The output side
// uses fewer, larger chunks: a phase-2 launch must hold enough tiles per CTA to
// stay balanced.
struct VecChunk {
    int64_t coff, clen;    // compact (host) element range
    int64_t doff, dlen;    // padded (device) element range
    int piece0, piece1;    // pack pieces
};
struct DevChunked {
    std::vector<VecChunk> in, out;    // input chunks (phase 1 cut), output chunks (phase 2 cut)
    bool compact_out = false;         // phase 2 writes the compact (host-layout) vector directly
    DBuf ypieces;                     // PanelPiece list: the compact vector (scaled per block) -> Y2
    std::deque<PhasePlan> p1h, p2h;   // host sub-plans (DevPhase::host points here)
    std::deque<DevPhase> p1, p2;
    std::vector<cudaEvent_t> ev_in, ev_out;
    cudaEvent_t ev_start = nullptr;
    ~DevChunked() {
        for (auto e : ev_in) cudaEventDestroy(e);
        for (auto e : ev_out) cudaEventDestroy(e);
        if (ev_start) cudaEventDestroy(ev_start);
    }
};

// Split plans keep each bf16 operand in a panel arena (engine.hpp): op(X) in
// X2, the vector Y in Y2 (split per call), the intermediates in T, the scaled
// copies c*op(Z) in Z2.
struct DevPlan {
    Plan plan;
    DevPhase p1, p2;
    DBuf T;                        // FP64: T (double); split: T panels (bf16)
    DBuf X2, Z2, Y2;               // split: operand panels (bf16)
    DBuf prepX, prepZ;             // PrepBlock lists
    DBuf ypieces;                  // PanelPiece list: the FP64 Y arena -> Y2
    int nprepX = 0, nprepZ = 0, nypieces = 0;
    std::unique_ptr<DevChunked> chunks;   // host-buffer pipeline (split plans of pivots)
    // split-K partial outputs (plan.splitk parts of vstride elements), one buffer per
    // output type so that the zero padding of each stays zero
    DBuf part_d, part_f;
    bool ready = false;
};

// ---------------------------------------------------------------------------
// TMA descriptors of the tcgen05 engine
// ---------------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !f)
            throw CudaFail("cuTensorMapEncodeTiled is not available from the driver");
        return reinterpret_cast<EncodeTiledFn>(f);
    }();
    return fn;
}

// The TMA descriptors of one split phase: for each (panel class, box height) key
// a 2-d tensor over the class matrix (2*kpad bf16 columns, its stacked rows) with
// boxes of 64 columns (one 32-wide K step, hi and lo) x the key's rows, 128-byte
// swizzle and zero fill below the last row.
// (elt 2: bf16 panels, boxes of 64 elements; elt 4: 3xTF32 panels in FP32 storage, boxes of
// 32 elements -- 128 bytes either way)
static void encode_panel_map(CUtensorMap* m, const PanelArena& ar, const DBuf& arena, const MapKey& k, int elt) {
    if (k.cls < 0 || k.cls >= (int)ar.cls.size()) throw std::logic_error("TMA descriptor of an unknown panel class");
    if (elt != 2 && elt != 4) throw std::logic_error("panel element must be 2 or 4 bytes");
    const PanelClass& c = ar.cls[k.cls];
    if (k.rows < 16 || k.rows > 256 || k.rows % 16 != 0) throw std::logic_error("TMA box rows out of range");
    if (c.base % 64 != 0 || c.kpad % 32 != 0) throw std::logic_error("panel class not 128-byte aligned");
    const cuuint64_t dims[2] = {(cuuint64_t)2 * c.kpad, (cuuint64_t)std::max<int64_t>(c.rows, 1)};
    const cuuint64_t strides[1] = {(cuuint64_t)2 * c.kpad * elt};
    const cuuint32_t box[2] = {(cuuint32_t)(128 / elt), (cuuint32_t)k.rows};
    const cuuint32_t estr[2] = {1, 1};
    void* base = static_cast<unsigned char*>(arena.p) + (size_t)c.base * elt;
    CUresult res = encode_tiled()(m, elt == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                  base, dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (res != CUDA_SUCCESS)
        throw CudaFail("cuTensorMapEncodeTiled failed (" + std::to_string((int)res) + ") for a panel class of " +
                       std::to_string(c.rows) + " rows x " + std::to_string(c.kpad));
}

static std::unique_ptr<TmaMaps> build_phase_maps(const PhasePlan& ph, const PanelArena& A, const DBuf& Aarena,
                                                 const PanelArena& B, const DBuf& Barena, int elt) {
    if ((int)ph.amaps.size() > kMaxMapsA || (int)ph.bmaps.size() > kMaxMapsB)
        throw std::logic_error("tcgen05 plan: too many TMA descriptors in one phase");
    auto m = std::make_unique<TmaMaps>();
    std::memset(m.get(), 0, sizeof(TmaMaps));
    for (size_t i = 0; i < ph.amaps.size(); ++i) encode_panel_map(&m->a[i], A, Aarena, ph.amaps[i], elt);
    for (size_t i = 0; i < ph.bmaps.size(); ++i) encode_panel_map(&m->b[i], B, Barena, ph.bmaps[i], elt);
    return m;
}

// column pieces (at most kPackPiece elements) of the blocks of a column-major
// FP64 layout into the panels of opY: column c of block y -> panel row c
static std::vector<PanelPiece> panel_pieces(const std::vector<int64_t>& off, const std::vector<int64_t>& rows,
                                            const std::vector<int64_t>& cols, const std::vector<int64_t>& ld,
                                            const std::vector<OpBlock>& op, const std::vector<double>* scale);

// compact <-> padded copy descriptors of one block table.  Blocks are cut into
// pieces of whole columns holding at most kPackPiece elements (one pass of a
// 256-thread block with four loads in flight per thread), so that large blocks
// spread over many thread blocks of the copy kernels.
constexpr int64_t kPackPiece = 1024;
static std::vector<PackBlock> pack_blocks(const BlockTable& t, const DevLayout& d, const std::vector<double>* scale) {
    std::vector<PackBlock> v;
    v.reserve((size_t)t.n);
    for (int64_t i = 0; i < t.n; ++i) {
        const int64_t rows = t.rows[i], cols = t.cols[i];
        if (rows <= 0 || cols <= 0) continue;
        const int64_t per = std::max<int64_t>(1, kPackPiece / rows);   // columns per piece
        for (int64_t c0 = 0; c0 < cols; c0 += per) {
            const int64_t nc = std::min(per, cols - c0);
            v.push_back(PackBlock{t.off[i] + c0 * rows, d.off[i] + c0 * d.ld[i], rows, nc, d.ld[i],
                                  scale ? (*scale)[i] : 1.0});
        }
    }
    return v;
}

// index of the first pack piece of every block (and the total at the end), with
// the same cut as pack_blocks
static std::vector<int> pack_piece_starts(const BlockTable& t) {
    std::vector<int> s((size_t)t.n + 1, 0);
    for (int64_t i = 0; i < t.n; ++i) {
        const int64_t rows = t.rows[i], cols = t.cols[i];
        int64_t np = 0;
        if (rows > 0 && cols > 0) {
            const int64_t per = std::max<int64_t>(1, kPackPiece / rows);
            np = (cols + per - 1) / per;
        }
        s[i + 1] = s[i] + (int)np;
    }
    return s;
}

static std::vector<PanelPiece> panel_pieces(const std::vector<int64_t>& off, const std::vector<int64_t>& rows,
                                            const std::vector<int64_t>& cols, const std::vector<int64_t>& ld,
                                            const std::vector<OpBlock>& op, const std::vector<double>* scale) {
    std::vector<PanelPiece> v;
    for (size_t i = 0; i < rows.size(); ++i) {
        if (rows[i] <= 0 || cols[i] <= 0) continue;
        if (op[i].K != rows[i] || op[i].outer != cols[i]) throw std::logic_error("vector panel does not match its block");
        const int64_t per = std::max<int64_t>(1, kPackPiece / rows[i]);   // the cut of pack_blocks
        for (int64_t c0 = 0; c0 < cols[i]; c0 += per) {
            const int64_t nc = std::min(per, cols[i] - c0);
            v.push_back(PanelPiece{off[i] + c0 * ld[i], op[i].off + c0 * op[i].pitch, (int32_t)rows[i], (int32_t)nc,
                                   (int32_t)ld[i], op[i].pitch, scale ? (*scale)[i] : 1.0});
        }
    }
    return v;
}

// pieces of the vector split of a split plan: right-hand side k's block y (at
// k * Y.total + Y.off[y]) into panel rows from k * ycolsP[y] of the block's panel;
// with one right-hand side exactly the pieces of panel_pieces
static std::vector<PanelPiece> vector_panel_pieces(const DevLayout& Y, const Plan& plan) {
    std::vector<PanelPiece> v;
    for (int k = 0; k < plan.nrhs; ++k)
        for (size_t i = 0; i < Y.rows.size(); ++i) {
            const int64_t rows = Y.rows[i], cols = Y.cols[i];
            if (rows <= 0 || cols <= 0) continue;
            const OpBlock& op = plan.opY[i];
            if (op.K != rows || op.outer != (int64_t)plan.nrhs * plan.ycolsP[i] || plan.ycolsP[i] < cols)
                throw std::logic_error("vector panel does not match its block");
            const int64_t per = std::max<int64_t>(1, kPackPiece / rows);
            for (int64_t c0 = 0; c0 < cols; c0 += per) {
                const int64_t nc = std::min(per, cols - c0);
                v.push_back(PanelPiece{(int64_t)k * Y.total + Y.off[i] + c0 * Y.ld[i],
                                       op.off + ((int64_t)k * plan.ycolsP[i] + c0) * op.pitch, (int32_t)rows,
                                       (int32_t)nc, (int32_t)Y.ld[i], op.pitch, 1.0});
            }
        }
    return v;
}

// A pointer the device may dereference for a caller's host buffer, or null when
// the buffer must be staged with a copy: page-locked (registered) memory has a
// device mapping; pageable memory is read in place when the device walks the
// host page tables (coherent CPU-GPU systems such as Grace with NVLink-C2C).
static const void* device_view(const vmps_ctx* c, const void* host) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    switch (a.type) {
        case cudaMemoryTypeHost: return a.devicePointer;
        case cudaMemoryTypeDevice:
        case cudaMemoryTypeManaged: return a.device == c->device ? host : nullptr;
        default: return c->pageable_access ? host : nullptr;
    }
}

// compact host vector -> padded device arena (scaled per block), no staging
// copy when the device can read the host buffer
static void pack_in(const vmps_ctx* c, const DBuf& pk, int npk, const double* host, int64_t total, DBuf& stage,
                    double* dst, cudaStream_t st) {
    if (npk == 0) return;
    const double* src = static_cast<const double*>(device_view(c, host));
    if (!src) {
        stage.alloc((size_t)std::max<int64_t>(total, 1) * 8, st, false);
        CK(cudaMemcpyAsync(stage.p, host, (size_t)total * 8, cudaMemcpyHostToDevice, st));
        src = stage.as<double>();
    }
    CK(launch_pack(pk.as<PackBlock>(), npk, src, dst, 1, st));
}

// padded device arena -> compact host vector
static void pack_out(const vmps_ctx* c, const DBuf& pk, int npk, const double* src, int64_t total, DBuf& stage,
                     double* host, cudaStream_t st) {
    if (npk == 0) return;
    double* dst = static_cast<double*>(const_cast<void*>(device_view(c, host)));
    if (dst) {
        CK(launch_pack(pk.as<PackBlock>(), npk, src, dst, 0, st));
        return;
    }
    stage.alloc((size_t)std::max<int64_t>(total, 1) * 8, st, false);
    CK(launch_pack(pk.as<PackBlock>(), npk, src, stage.as<double>(), 0, st));
    CK(cudaMemcpyAsync(host, stage.p, (size_t)total * 8, cudaMemcpyDeviceToHost, st));
}

// FP64 device arenas of one grouped-GEMM problem
struct Operands {
    const double* X = nullptr;
    const double* Y = nullptr;
    const double* Z = nullptr;
    double* O = nullptr;
    int* err = nullptr;
    // split plans only: FP32 vectors in place of Y and O (same padded layout)
    const float* Yf = nullptr;
    float* Of = nullptr;
    // pivots with an excited-state projector: applied after the second phase
    const PenaltyArgs* pen = nullptr;
    long long wait_budget = 0;   // tcgen05 engine main-loop wait budget (cycles, 0: default)
};

// Invariants the tcgen05 engine relies on, checked on the host once per plan:
// every segment names operand blocks that exist and share its K; every tile lies
// inside its blocks, fits the 128 x 256 accumulator and its TMA boxes; split
// outputs (T panels) are tiled on whole panel K steps.
static void validate_tma_plan(const PhasePlan& ph, const std::vector<OpBlock>& A, const std::vector<OpBlock>& B,
                              bool split_out) {
    if (ph.seg_amap.size() != ph.segs.size() || ph.seg_bmap.size() != ph.segs.size())
        throw std::logic_error("tcgen05 plan: segment operand maps missing");
    for (size_t s = 0; s < ph.segs.size(); ++s) {
        const int32_t a = ph.seg_amap[s], b = ph.seg_bmap[s];
        if (a < 0 || a >= (int32_t)A.size() || b < 0 || b >= (int32_t)B.size())
            throw std::logic_error("tcgen05 plan: operand block index out of range");
        const int32_t ko = ph.segs[s].akoff;
        // the A operand may be a K range of wider panel rows (multi-RHS intermediates)
        if (B[b].K != ph.segs[s].K || ph.segs[s].K <= 0 || ko < 0 || ko % 32 != 0 || ko + ph.segs[s].K > A[a].K)
            throw std::logic_error("tcgen05 plan: contraction length mismatch");
    }
    for (const GTile& t : ph.tiles) {
        if (t.tm <= 0 || t.tn <= 0 || t.tm > kUmmaTileM || t.tn > kUmmaTileN || t.row0 < 0 || t.col0 < 0)
            throw std::logic_error("tcgen05 plan: tile shape out of range");
        if (t.seg_begin < 0 || t.seg_end < t.seg_begin || t.seg_end > (int32_t)ph.segs.size())
            throw std::logic_error("tcgen05 plan: tile segment range out of range");
        for (int32_t s = t.seg_begin; s < t.seg_end; ++s)
            if (t.row0 + t.tm > A[ph.seg_amap[s]].outer || t.col0 + t.tn > B[ph.seg_bmap[s]].outer)
                throw std::logic_error("tcgen05 plan: tile outside its operand blocks");
        if (split_out && (!ph.transC || t.col0 % 32 != 0 || t.ldc % 64 != 0 || t.c_off % 64 != 0))
            throw std::logic_error("tcgen05 plan: split-output tile not on whole panel K steps");
        if (t.nrhs > 1 && ((split_out && (t.rstride <= 0 || t.rstride % 32 != 0 || t.col0 + t.tn > t.nrhs * t.rstride)) ||
                           (!split_out && ph.transC)))
            throw std::logic_error("tcgen05 plan: multi-RHS tile with a bad right-hand-side stride");
    }
}

// the schedule: CTA tile ranges partition the tiles, every tile's steps lie in
// the step list, TMA coordinates are 128-byte aligned and inside their panel
// classes' columns, boxes cover the tiles, descriptors exist
static void validate_tma_schedule(const PhasePlan& ph, const PanelArena& A, const PanelArena& B, int elt = 2) {
    const int32_t box = 128 / elt;   // elements of one 128-byte TMA box row
    if (ph.tiles.empty()) return;
    if (ph.ncta <= 0 || (int)ph.cta_tiles.size() != ph.ncta + 1 || ph.cta_tiles.front() != 0 ||
        ph.cta_tiles.back() != (int32_t)ph.tiles.size())
        throw std::logic_error("tcgen05 plan: CTA ranges do not cover the tiles");
    for (int b = 0; b < ph.ncta; ++b)
        if (ph.cta_tiles[b + 1] < ph.cta_tiles[b]) throw std::logic_error("tcgen05 plan: CTA ranges out of order");
    if ((int)ph.amaps.size() > kMaxMapsA || (int)ph.bmaps.size() > kMaxMapsB)
        throw std::logic_error("tcgen05 plan: too many TMA descriptors in one phase");
    int64_t next = 0;
    for (const GTile& t : ph.tiles) {
        if (t.step0 != next || t.nsteps < 0) throw std::logic_error("tcgen05 plan: tile steps not contiguous");
        next += t.nsteps;
        for (int j = t.step0; j < t.step0 + t.nsteps && j < (int)ph.steps.size(); ++j) {
            const TStep& s = ph.steps[j];
            if (s.amap < 0 || s.amap >= (int)ph.amaps.size() || s.bmap < 0 || s.bmap >= (int)ph.bmaps.size())
                throw std::logic_error("tcgen05 plan: step descriptor out of range");
            const MapKey& ka = ph.amaps[s.amap];
            const MapKey& kb = ph.bmaps[s.bmap];
            if (ka.rows != s.arows || kb.rows != s.brows || s.arows < t.tm || s.brows < ((t.tn + 15) / 16) * 16 ||
                s.arows > kUmmaTileM || s.brows > kUmmaTileN)
                throw std::logic_error("tcgen05 plan: TMA box does not cover its tile");
            const int32_t xb = s.x & ~1;   // bit 0 flags a padding second K16 slice
            if (xb % box != 0 || xb < 0 || s.xa % box != 0 || s.xa < 0 || s.xa >= 2 * A.cls[ka.cls].kpad ||
                xb >= 2 * B.cls[kb.cls].kpad || s.ay < 0 || s.by < 0 || s.ay >= A.cls[ka.cls].rows ||
                s.by >= B.cls[kb.cls].rows)
                throw std::logic_error("tcgen05 plan: TMA coordinate outside its panel");
        }
    }
    if (next != (int64_t)ph.steps.size()) throw std::logic_error("tcgen05 plan: step count mismatch");
}

static void schedule_and_validate(Plan& p, int ncta) {
    validate_tma_plan(p.p1, p.opX, p.opY, true);
    validate_tma_plan(p.p2, p.opT, p.opZ, false);
    schedule_tma(p.p1, ncta, p.opX, p.opY, p.kstep);
    schedule_tma(p.p2, ncta, p.opT, p.opZ, p.kstep);
    validate_tma_schedule(p.p1, p.ax, p.ay, p.elt);
    validate_tma_schedule(p.p2, p.at, p.az, p.elt);
}

// device buffers and work lists of a freshly made plan; Y is the FP64 layout
// the per-call vector split reads
static void plan_to_device(DevPlan& dp, const DevLayout& Y, cudaStream_t st) {
    dp.p1.upload(dp.plan.p1, st);
    dp.p2.upload(dp.plan.p2, st);
    if (!dp.plan.split) {
        dp.T.alloc((size_t)dp.plan.T.total * 8, st, true);
        return;
    }
    // zero-filled: panel padding stays zero
    const size_t elt = (size_t)dp.plan.elt;
    dp.T.alloc((size_t)dp.plan.at.total * elt, st, true);
    dp.X2.alloc((size_t)dp.plan.ax.total * elt, st, true);
    dp.Z2.alloc((size_t)dp.plan.az.total * elt, st, true);
    dp.Y2.alloc((size_t)dp.plan.ay.total * elt, st, true);
    upload_vec(dp.prepX, dp.plan.prepX, st);
    upload_vec(dp.prepZ, dp.plan.prepZ, st);
    dp.nprepX = (int)dp.plan.prepX.size();
    dp.nprepZ = (int)dp.plan.prepZ.size();
    const auto yp = vector_panel_pieces(Y, dp.plan);
    upload_vec(dp.ypieces, yp, st);
    dp.nypieces = (int)yp.size();
    dp.p1.maps = build_phase_maps(dp.plan.p1, dp.plan.ax, dp.X2, dp.plan.ay, dp.Y2, dp.plan.elt);
    dp.p2.maps = build_phase_maps(dp.plan.p2, dp.plan.at, dp.T, dp.plan.az, dp.Z2, dp.plan.elt);
    if (dp.plan.splitk > 1) {
        const size_t n = (size_t)dp.plan.splitk * (size_t)dp.plan.vstride;
        dp.part_d.alloc(n * 8, st, true);
        dp.part_f.alloc(n * 4, st, true);
    }
}

// split plans: the bf16 panels of the X and scaled Z operands
static void split_prepare(DevPlan& dp, const double* X, const double* Z, cudaStream_t st) {
    if (!dp.plan.split) return;
    if (dp.plan.elt == 4) {
        CK(launch_prep_tf32(dp.prepX.as<PrepBlock>(), dp.nprepX, X, dp.X2.p, st));
        CK(launch_prep_tf32(dp.prepZ.as<PrepBlock>(), dp.nprepZ, Z, dp.Z2.p, st));
        return;
    }
    CK(launch_prep(dp.prepX.as<PrepBlock>(), dp.nprepX, X, dp.X2.p, st));
    CK(launch_prep(dp.prepZ.as<PrepBlock>(), dp.nprepZ, Z, dp.Z2.p, st));
}

static void run_phase_on(const DevPlan& dp, int ph, const DevPhase& d, const PhasePlan& h, const Operands& ops,
                         cudaStream_t st) {
    GGArgs a{};
    a.tiles = d.tiles.as<GTile>();
    a.segs = d.segs.as<GSeg>();
    a.terms = d.terms.as<GTerm>();
    a.ntiles = d.ntiles;
    a.transA = h.transA; a.transB = h.transB; a.transC = h.transC;
    a.err = ops.err;
    a.wait_budget = ops.wait_budget;
    if (!dp.plan.split) {
        auto slot = [&](int s) -> const void* {
            switch (s) {
                case SLOT_X: return ops.X;
                case SLOT_Y: return ops.Y;
                case SLOT_Z: return ops.Z;
                case SLOT_OUT: return ops.O;
                case SLOT_T: return dp.T.p;
            }
            return nullptr;
        };
        a.A = slot(h.slotA);
        a.B = slot(h.slotB);
        a.C = const_cast<void*>(slot(h.slotC));
        // every operand of a non-empty phase must be a live device buffer
        if (d.ntiles > 0 && (!a.C || !a.tiles || !a.segs || !a.terms || (!h.segs.empty() && (!a.A || !a.B))))
            throw std::invalid_argument("grouped GEMM launched with an unallocated operand");
        CK(launch_gg64(a, st));
        return;
    }
    a.A = ph == 1 ? dp.X2.p : dp.T.p;
    a.B = ph == 1 ? dp.Y2.p : dp.Z2.p;
    a.C = ph == 1 ? dp.T.p : (ops.Of ? (void*)ops.Of : (void*)ops.O);
    if (ph == 2 && dp.plan.splitk > 1) {
        // split-K: the parts go to a partial buffer (zeroed once: padding stays zero)
        const DBuf& pb = ops.Of ? dp.part_f : dp.part_d;
        const size_t bytes = (size_t)dp.plan.splitk * (size_t)dp.plan.vstride * (ops.Of ? 4 : 8);
        if (!pb.p || pb.bytes < bytes) throw std::invalid_argument("split-K plan without its partial buffer");
        a.C = pb.p;
    }
    a.steps = d.steps.as<TStep>();
    a.cta_tiles = d.cta_tiles.as<int32_t>();
    a.ncta = d.ncta;
    a.vstride = dp.plan.vstride;
    if (d.ntiles > 0 && (!a.A || !a.B || !a.C || !a.tiles || !a.steps || !a.cta_tiles || !d.maps))
        throw std::invalid_argument("grouped GEMM launched with an unallocated operand");
    if (d.ntiles > 0)
        CK(launch_gg_umma(ph == 1 ? 1 : (ops.Of ? 2 : 0), dp.plan.nrhs > 1, a, *d.maps, st, dp.plan.elt == 4));
}

static void run_phase(const DevPlan& dp, int ph, const Operands& ops, cudaStream_t st) {
    if (ph == 1) run_phase_on(dp, 1, dp.p1, dp.plan.p1, ops, st);
    else run_phase_on(dp, 2, dp.p2, dp.plan.p2, ops, st);
}

// one application of a planned contraction: (split plans) split Y, phase 1, phase 2
static void run_plan(const DevPlan& dp, const Operands& ops, cudaStream_t st) {
    if ((ops.Yf || ops.Of) && !dp.plan.split) throw std::invalid_argument("FP32 vectors need a split plan");
    if (dp.plan.split && dp.plan.elt == 4) {
        CK(launch_panel_split_tf32(dp.ypieces.as<PanelPiece>(), dp.nypieces, ops.Yf ? nullptr : ops.Y, ops.Yf, dp.Y2.p,
                                   st));
    } else if (dp.plan.split) {
        if (ops.Yf) CK(launch_panel_split_f32(dp.ypieces.as<PanelPiece>(), dp.nypieces, ops.Yf, dp.Y2.p, st));
        else CK(launch_panel_split(dp.ypieces.as<PanelPiece>(), dp.nypieces, ops.Y, dp.Y2.p, st));
    }
    run_phase(dp, 1, ops, st);
    run_phase(dp, 2, ops, st);
    if (dp.plan.split && dp.plan.splitk > 1)
        CK(launch_splitk_reduce(ops.Of ? dp.part_f.p : dp.part_d.p, dp.plan.splitk, dp.plan.vstride,
                                ops.Of ? (void*)ops.Of : (void*)ops.O, ops.Of ? 1 : 0, st));
    if (ops.pen && ops.pen->npen > 0) {
        PenaltyArgs a = *ops.pen;
        a.nrhs = dp.plan.nrhs;
        CK(launch_penalty(a, ops.Y, ops.Yf, ops.O, ops.Of, st));
    }
}

// tensor work a split phase issues: 3 products of M=128 x N=round16(tn) x K per
// step, K = kstep/2 for steps whose second K slice is padding (skipped), else kstep
static double phase_tensor_flops(const PhasePlan& ph, int kstep = kUmmaBK) {
    double f = 0;
    for (const GTile& t : ph.tiles) {
        double k = 0;
        for (int j = t.step0; j < t.step0 + t.nsteps && j < (int)ph.steps.size(); ++j)
            k += (ph.steps[j].x & 1) ? kstep / 2 : kstep;
        if (ph.steps.empty()) k = (double)t.nsteps * kstep;
        f += k * 3.0 * 2.0 * kUmmaTileM * ((t.tn + 15) / 16 * 16);
    }
    return f;
}

static void fill_stats(const ChainSet& cs, const Plan& p, int prec, vmps_plan_stats* s) {
    std::memset(s, 0, sizeof(*s));
    s->n_tasks = cs.n_tasks;
    s->n_chains = p.n_chains;
    s->n_chains_raw = cs.n_chains_raw;
    s->n_intermediates = p.n_intermediates;
    s->n_out_blocks = p.n_out_blocks;
    s->n_tiles_phase1 = (int64_t)p.p1.tiles.size();
    s->n_tiles_phase2 = (int64_t)p.p2.tiles.size();
    s->flops_reference = cs.flops_reference;
    s->flops_merged = p.flops_merged;
    s->flops_phase1 = p.p1.flops;
    s->flops_phase2 = p.p2.flops;
    s->flops_executed = p.p1.flops + p.p2.flops;
    s->bytes_algorithmic = p.bytes_alg;
    s->bytes_intermediate = p.split ? (double)p.elt * (double)p.at.total : 8.0 * (double)p.T.total;
    (void)prec;
    s->n_segments_phase2 = (int64_t)p.p2.segs.size();
    s->n_terms_phase2 = (int64_t)p.p2.terms.size();
    s->flops_phase2_unsummed = p.flops_p2_unsummed;
    s->association = p.association;
    if (p.split) {
        s->tensor_flops_phase1 = phase_tensor_flops(p.p1, p.kstep);
        s->tensor_flops_phase2 = phase_tensor_flops(p.p2, p.kstep);
    }
}


// ---------------------------------------------------------------------------
// pivot (PivotMatrix0/1/2)
// ---------------------------------------------------------------------------
struct vmps_pivot_s {
    vmps_ctx* ctx = nullptr;
    Symmetry sym;
    BlockTable Lt, Rt, Vt;
    DevLayout Ld, Rd, Vd;
    ChainSet cs;
    DevPlan plans[3];   // by precision: FP64, BF16x3, 3xTF32
    DBuf dL, dR;
    DBuf dPack;                 // PackBlock[] of the vector layout
    int npack = 0;
    std::vector<double> vscale; // sqrt(coeff_dot(qout)) per V block
    DBuf stage_in, stage_out;   // compact vectors for host-buffer HxV
    DBuf vin, vout;             // padded vectors for host-buffer HxV
    DBuf part, scal;            // reduction scratch
    DBuf flag;
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
    const void* graph_in[3] = {nullptr, nullptr, nullptr};
    const void* graph_out[3] = {nullptr, nullptr, nullptr};
    std::map<int, std::unique_ptr<DevPlan>> multi;   // split plans for nrhs > 1 vectors, by nrhs
    DBuf mvin, mvout;                                // nrhs padded vectors for host-buffer multi-RHS HxV
    // excited-state projector (A0proj, Epenalty): projector vectors in the padded layout
    // with the SU(2) dot weights folded in, chunk partials and coefficients
    DBuf pen_d, pen_a, pen_part, pen_coef;
    PenaltyArgs pen{};
    // tiling of the split-precision plan (autotuner or its cache), and the key of
    // the pivot's block-size histogram in that cache (0 = not computed yet)
    SplitTiling tiling;
    bool tiling_set = false;
    uint64_t layout_key = 0;
    ~vmps_pivot_s() {
        for (auto& g : graph) if (g) cudaGraphExecDestroy(g);
    }
    cudaStream_t st() const { return ctx->stream; }
};

struct vmps_dvec_s {
    vmps_pivot* p = nullptr;
    DBuf d;
    int64_t n = 0;   // padded length
};

// compact staging vectors (host layout) and padded I/O vectors of a pivot,
// each allocated on first use and independently of the other
static void ensure_staging(vmps_pivot* p) {
    const size_t cb = (size_t)std::max<int64_t>(p->Vt.total, 1) * 8;
    if (!p->stage_in.p) p->stage_in.alloc(cb, p->st(), false);
    if (!p->stage_out.p) p->stage_out.alloc(cb, p->st(), false);
}
static void ensure_io(vmps_pivot* p) {
    if (!p->vin.p) p->vin.alloc((size_t)p->Vd.total * 8, p->st(), true);
    if (!p->vout.p) p->vout.alloc((size_t)p->Vd.total * 8, p->st(), true);
}

static void make_chunks(vmps_pivot* p, DevPlan& dp);
static SplitTiling pivot_tiling(vmps_pivot* p);

static DevPlan& get_plan(vmps_pivot* p, int prec) {
    if (prec != VMPS_PREC_FP64 && prec != VMPS_PREC_BF16X3 && prec != VMPS_PREC_TF32X3)
        throw std::invalid_argument("unknown precision");
    DevPlan& dp = p->plans[prec];
    if (dp.ready) return dp;
    if (prec == VMPS_PREC_FP64) dp.plan = make_plan(p->cs, p->Ld, p->Vd, p->Rd, p->Vd, false, false, 64, 64);
    else if (prec == VMPS_PREC_TF32X3) {
        dp.plan = make_split_plan(p->cs, p->Ld, p->Vd, p->Rd, p->Vd, false, false, 1, SplitTiling(), true);
        schedule_and_validate(dp.plan, p->ctx->num_sms);
    } else {
        dp.plan = make_split_plan(p->cs, p->Ld, p->Vd, p->Rd, p->Vd, false, false, 1, pivot_tiling(p));
        schedule_and_validate(dp.plan, p->ctx->num_sms);
    }
    if (p->ctx->device < 0) { dp.ready = true; return dp; }   // host-only: plan without device copies
    plan_to_device(dp, p->Vd, p->st());
    split_prepare(dp, p->dL.as<double>(), p->dR.as<double>(), p->st());
    if (prec == VMPS_PREC_BF16X3 && dp.plan.splitk == 1) make_chunks(p, dp);
    CK(cudaStreamSynchronize(p->st()));
    dp.ready = true;
    return dp;
}

// the split plan of a pivot for nrhs vectors at once (built on first use)
static DevPlan& get_multi_plan(vmps_pivot* p, int nrhs) {
    if (nrhs == 1) return get_plan(p, VMPS_PREC_BF16X3);
    auto& slot = p->multi[nrhs];
    if (slot && slot->ready) return *slot;
    slot.reset(new DevPlan());
    DevPlan& dp = *slot;
    dp.plan = make_split_plan(p->cs, p->Ld, p->Vd, p->Rd, p->Vd, false, false, nrhs);
    schedule_and_validate(dp.plan, p->ctx->num_sms);
    if (p->ctx->device < 0) { dp.ready = true; return dp; }
    plan_to_device(dp, p->Vd, p->st());
    split_prepare(dp, p->dL.as<double>(), p->dR.as<double>(), p->st());
    CK(cudaStreamSynchronize(p->st()));
    dp.ready = true;
    return dp;
}

// Cut a pivot's split plan into the host-buffer pipeline (see DevChunked).  Only
// for vectors of at least kChunkBytes per chunk and a compact layout whose
// blocks are stored in order without gaps.
constexpr int64_t kChunkBytes = 4 << 20;
constexpr int kMaxChunksIn = 4, kMaxChunksOut = 3;
static void make_chunks(vmps_pivot* p, DevPlan& dp) {
    const BlockTable& t = p->Vt;
    const int64_t nb = t.n;
    if (!dp.plan.split || nb < 2) return;
    const int64_t kmax = std::min<int64_t>(nb, t.total * 8 / kChunkBytes);
    if (kmax < 2) return;
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t next = b + 1 < nb ? t.off[b + 1] : t.total;
        if (t.off[b] + t.rows[b] * t.cols[b] != next) return;   // not in order / gaps: no pipeline
    }
    if (t.off[0] != 0) return;
    auto ch = std::make_unique<DevChunked>();
    const std::vector<int> ps = pack_piece_starts(t);
    // k chunks of about equal compact size; chunk_of[block]
    auto partition = [&](int k, std::vector<VecChunk>& io, std::vector<int>& chunk_of) {
        chunk_of.assign((size_t)nb, 0);
        int64_t b0 = 0;
        for (int c = 0; c < k && b0 < nb; ++c) {
            const int64_t target = (t.total * (c + 1)) / k;
            int64_t b1 = b0 + 1;
            while (b1 < nb && (c == k - 1 || t.off[b1] < target)) ++b1;
            VecChunk v{};
            v.coff = t.off[b0];
            v.clen = (b1 < nb ? t.off[b1] : t.total) - v.coff;
            v.doff = p->Vd.off[b0];
            v.dlen = (b1 < nb ? p->Vd.off[b1] : p->Vd.total) - v.doff;
            v.piece0 = ps[b0];
            v.piece1 = ps[b1];
            for (int64_t b = b0; b < b1; ++b) chunk_of[b] = (int)io.size();
            io.push_back(v);
            b0 = b1;
        }
    };
    std::vector<int> in_of, out_of;
    partition((int)std::min<int64_t>(kMaxChunksIn, kmax), ch->in, in_of);
    partition((int)std::min<int64_t>(kMaxChunksOut, kmax), ch->out, out_of);
    if (ch->in.size() < 2 || ch->out.size() < 2) return;
    std::unordered_map<int64_t, int64_t> block_of_off;
    for (int64_t b = 0; b < nb; ++b) block_of_off[p->Vd.off[b]] = b;
    // with unit block scales the output needs no unscaling: phase 2 stores into
    // the compact layout (column-major blocks, ld = rows) and the unpack pass goes
    ch->compact_out = std::all_of(p->vscale.begin(), p->vscale.end(), [](double s) { return s == 1.0; });
    auto cut = [&](const PhasePlan& full, int ph, std::deque<PhasePlan>& hs, std::deque<DevPhase>& ds) {
        const std::vector<int>& chunk_of = ph == 1 ? in_of : out_of;
        const int kk = (int)(ph == 1 ? ch->in.size() : ch->out.size());
        std::vector<std::vector<GTile>> per(kk);
        for (const GTile& tl : full.tiles) {
            int64_t blk;
            if (ph == 1) {
                if (tl.seg_end <= tl.seg_begin) throw std::logic_error("phase-1 tile without a segment");
                blk = full.seg_bmap[tl.seg_begin];   // the V block this intermediate multiplies
            } else {
                auto it = block_of_off.find(tl.c_off);
                if (it == block_of_off.end()) throw std::logic_error("phase-2 tile outside the vector layout");
                blk = it->second;
                if (ch->compact_out) {
                    GTile c = tl;
                    c.c_off = t.off[blk];
                    c.ldc = (int32_t)t.rows[blk];
                    per[chunk_of[blk]].push_back(c);
                    continue;
                }
            }
            per[chunk_of[blk]].push_back(tl);
        }
        for (int c = 0; c < kk; ++c) {
            hs.emplace_back();
            PhasePlan& sp = hs.back();
            sp.terms = full.terms;
            sp.segs = full.segs;
            sp.seg_amap = full.seg_amap;
            sp.seg_bmap = full.seg_bmap;
            sp.transA = full.transA; sp.transB = full.transB; sp.transC = full.transC;
            sp.slotA = full.slotA; sp.slotB = full.slotB; sp.slotC = full.slotC;
            sp.tiles = std::move(per[c]);
            if (ph == 1) {
                schedule_tma(sp, p->ctx->num_sms, dp.plan.opX, dp.plan.opY, dp.plan.kstep);
                validate_tma_schedule(sp, dp.plan.ax, dp.plan.ay, dp.plan.elt);
            } else {
                schedule_tma(sp, p->ctx->num_sms, dp.plan.opT, dp.plan.opZ, dp.plan.kstep);
                validate_tma_schedule(sp, dp.plan.at, dp.plan.az, dp.plan.elt);
            }
            ds.emplace_back();
            ds.back().upload(sp, p->st());
            ds.back().maps = ph == 1 ? build_phase_maps(sp, dp.plan.ax, dp.X2, dp.plan.ay, dp.Y2, dp.plan.elt)
                                     : build_phase_maps(sp, dp.plan.at, dp.T, dp.plan.az, dp.Z2, dp.plan.elt);
        }
    };
    cut(dp.plan.p1, 1, ch->p1h, ch->p1);
    cut(dp.plan.p2, 2, ch->p2h, ch->p2);
    {
        // the compact vector into Y2's panels, in the piece order of pack_piece_starts
        std::vector<int64_t> ld(t.rows.begin(), t.rows.end());
        const auto yp = panel_pieces(t.off, t.rows, t.cols, ld, dp.plan.opY, &p->vscale);
        if ((int)yp.size() != ps[nb]) throw std::logic_error("vector pieces differ from the pack pieces");
        upload_vec(ch->ypieces, yp, p->st());
    }
    ch->ev_in.resize(ch->in.size(), nullptr);
    ch->ev_out.resize(ch->out.size(), nullptr);
    for (auto& ev : ch->ev_in) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    for (auto& ev : ch->ev_out) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ch->ev_start, cudaEventDisableTiming));
    dp.chunks = std::move(ch);
}

// host-buffer HxV through the chunk pipeline: copies on the copy stream, compute
// on the context stream, ordered by events
static void hxv_host_pipelined(vmps_pivot* p, DevPlan& dp, const double* vin, double* vout) {
    DevChunked& ch = *dp.chunks;
    cudaStream_t cs = p->st(), xs = p->ctx->copy_stream;
    double* din = p->vin.as<double>();
    double* dout = p->vout.as<double>();
    double* sin = p->stage_in.as<double>();
    double* sout = p->stage_out.as<double>();
    const PackBlock* pk = p->dPack.as<PackBlock>();
    Operands ops;
    ops.X = p->dL.as<double>();
    ops.Z = p->dR.as<double>();
    ops.Y = din;
    ops.O = ch.compact_out ? sout : dout;
    ops.err = p->ctx->err;
    ops.wait_budget = p->ctx->wait_budget;
    const int kin = (int)ch.in.size(), kout = (int)ch.out.size();
    // the copy stream starts after everything already queued on the compute stream
    CK(cudaEventRecord(ch.ev_start, cs));
    CK(cudaStreamWaitEvent(xs, ch.ev_start, 0));
    for (int c = 0; c < kin; ++c) {
        const VecChunk& v = ch.in[c];
        CK(cudaMemcpyAsync(sin + v.coff, vin + v.coff, (size_t)v.clen * 8, cudaMemcpyHostToDevice, xs));
        CK(cudaEventRecord(ch.ev_in[c], xs));
        CK(cudaStreamWaitEvent(cs, ch.ev_in[c], 0));
        CK(launch_panel_split(ch.ypieces.as<PanelPiece>() + v.piece0, v.piece1 - v.piece0, sin, dp.Y2.p, cs));
        run_phase_on(dp, 1, ch.p1[c], ch.p1h[c], ops, cs);
    }
    // phase 2 of chunk o is queued before the copy-out of chunk o-1, so that a
    // copy call that blocks the host (pageable memory) does not hold back compute
    for (int o = 0; o <= kout; ++o) {
        if (o < kout) {
            const VecChunk& v = ch.out[o];
            run_phase_on(dp, 2, ch.p2[o], ch.p2h[o], ops, cs);
            if (!ch.compact_out) CK(launch_pack(pk + v.piece0, v.piece1 - v.piece0, dout, sout, 0, cs));
            CK(cudaEventRecord(ch.ev_out[o], cs));
        }
        if (o >= 1) {
            const VecChunk& w = ch.out[o - 1];
            CK(cudaStreamWaitEvent(xs, ch.ev_out[o - 1], 0));
            CK(cudaMemcpyAsync(vout + w.coff, sout + w.coff, (size_t)w.clen * 8, cudaMemcpyDeviceToHost, xs));
        }
    }
    CK(cudaStreamSynchronize(xs));
    CK(cudaStreamSynchronize(cs));
}

static void require_device(const vmps_ctx* c) {
    if (!c || c->device < 0) throw std::invalid_argument("operation needs a device context (this one is host-only)");
}

// the operands every HxV of a pivot shares: L and R arenas, the error word and
// the excited-state projector when one is set
static Operands pivot_ops(const vmps_pivot* p) {
    Operands ops;
    ops.X = p->dL.as<double>();
    ops.Z = p->dR.as<double>();
    ops.err = p->ctx->err;
    ops.wait_budget = p->ctx->wait_budget;
    if (p->pen.npen > 0) ops.pen = &p->pen;
    return ops;
}

static void pivot_hxv_dev(vmps_pivot* p, int prec, const double* vin, double* vout) {
    require_device(p->ctx);
    DevPlan& dp = get_plan(p, prec);
    Operands ops = pivot_ops(p);
    ops.Y = vin;
    ops.O = vout;
    ops.err = p->ctx->err;
    run_plan(dp, ops, p->st());
}

// ---------------------------------------------------------------------------
// Autotuner of the split-precision tiling.  The candidates are the phase-1 and
// phase-2 tile N caps (256 or 128 columns) and the split-K factor of phase 2
// (1, 2, 4; more than 1 only while phase 2 has fewer tiles than twice the SM
// count, where it is the only source of parallelism).  Each candidate plan is
// built and timed on the pivot itself (CUDA events, `trials` HxVs after one
// warm-up); the fastest wins, ties to the default.  The choice is cached per
// sector layout: the key is the block-size histogram of the pivot's chains
// ((m, k, n, p) of op(X) m x k, Y k x n, Z n x p, with counts), so the pivots of
// later sweeps over the same bond bases reuse it without timing.
// ---------------------------------------------------------------------------
static std::mutex g_tune_mu;
static std::unordered_map<uint64_t, SplitTiling> g_tune_cache;

static uint64_t pivot_layout_key(vmps_pivot* p) {
    if (p->layout_key) return p->layout_key;
    std::map<std::array<int64_t, 4>, int64_t> hist;
    for (const Chain& c : p->cs.chains)
        ++hist[{p->Lt.rows[c.x], p->Lt.cols[c.x], p->Vt.cols[c.y], p->Rt.cols[c.z]}];
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        for (int i = 0; i < 8; ++i) { h ^= (v >> (8 * i)) & 0xffu; h *= 1099511628211ull; }
    };
    mix((uint64_t)p->Vt.n);
    mix((uint64_t)p->Vt.total);
    for (const auto& kv : hist) {
        for (int64_t v : kv.first) mix((uint64_t)v);
        mix((uint64_t)kv.second);
    }
    p->layout_key = h ? h : 1;
    return p->layout_key;
}

// VMPS_AUTOTUNE = 1: the first split plan of a pivot whose layout is not in the
// cache is tuned (3 timed HxVs per candidate)
static bool autotune_on_first_plan() {
    const char* v = std::getenv("VMPS_AUTOTUNE");
    return v && !std::strcmp(v, "1");
}

static SplitTiling tune_pivot(vmps_pivot* p, int trials, double* ms_default, double* ms_best, int* ncand);

static SplitTiling pivot_tiling(vmps_pivot* p) {
    if (p->tiling_set) return p->tiling;
    const uint64_t key = pivot_layout_key(p);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            p->tiling = it->second;
            p->tiling_set = true;
            return p->tiling;
        }
    }
    if (p->ctx->device >= 0 && autotune_on_first_plan()) {
        double a = 0, b = 0;
        int n = 0;
        p->tiling = tune_pivot(p, 3, &a, &b, &n);
        p->tiling_set = true;
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = p->tiling;
        return p->tiling;
    }
    return SplitTiling();
}

static double time_split_plan(vmps_pivot* p, const SplitTiling& tl, int trials, int64_t* tiles2) {
    cudaStream_t st = p->st();
    DevPlan dp;
    dp.plan = make_split_plan(p->cs, p->Ld, p->Vd, p->Rd, p->Vd, false, false, 1, tl);
    schedule_and_validate(dp.plan, p->ctx->num_sms);
    if (tiles2) *tiles2 = (int64_t)dp.plan.p2.tiles.size();
    plan_to_device(dp, p->Vd, st);
    split_prepare(dp, p->dL.as<double>(), p->dR.as<double>(), st);
    Operands ops = pivot_ops(p);
    ops.Y = p->vin.as<double>();
    ops.O = p->vout.as<double>();
    run_plan(dp, ops, st);   // warm-up
    CK(cudaStreamSynchronize(st));
    // one event between consecutive HxVs; the median per-HxV time is robust to a
    // slow outlier (a first launch under a profiler, a clock change)
    std::vector<cudaEvent_t> ev((size_t)trials + 1, nullptr);
    std::vector<double> t((size_t)trials);
    try {
        for (auto& e : ev) CK(cudaEventCreate(&e));
        CK(cudaEventRecord(ev[0], st));
        for (int i = 0; i < trials; ++i) {
            run_plan(dp, ops, st);
            CK(cudaEventRecord(ev[(size_t)i + 1], st));
        }
        CK(cudaEventSynchronize(ev[(size_t)trials]));
        for (int i = 0; i < trials; ++i) {
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, ev[(size_t)i], ev[(size_t)i + 1]));
            t[(size_t)i] = ms;
        }
    } catch (...) {
        for (auto e : ev) if (e) cudaEventDestroy(e);
        throw;
    }
    for (auto e : ev) cudaEventDestroy(e);
    check_device_error(p->ctx);
    std::sort(t.begin(), t.end());
    return t[t.size() / 2];
}

static SplitTiling tune_pivot(vmps_pivot* p, int trials, double* ms_default, double* ms_best, int* ncand) {
    require_device(p->ctx);
    ensure_staging(p);
    ensure_io(p);
    // a nonzero input (the timing does not depend on the values)
    std::vector<double> ones((size_t)std::max<int64_t>(p->Vt.total, 1), 1.0);
    pack_in(p->ctx, p->dPack, p->npack, ones.data(), p->Vt.total, p->stage_in, p->vin.as<double>(), p->st());
    CK(cudaStreamSynchronize(p->st()));
    const SplitTiling def;
    int64_t tiles2 = 0;
    time_split_plan(p, def, 1, nullptr);   // module and descriptor warm-up before anything is compared
    double best = time_split_plan(p, def, trials, &tiles2);
    *ms_default = best;
    const double margin = 0.98;   // a candidate must beat the default by 2 % (timing noise)
    SplitTiling pick = def;
    int n = 1;
    std::vector<SplitTiling> cand;
    for (int c1 : {256, 128})
        for (int c2 : {256, 128})
            for (int sk : {1, 2, 4}) {
                SplitTiling t;
                t.ncap1 = c1; t.ncap2 = c2; t.splitk = sk;
                if (t == def) continue;
                if (sk > 1 && tiles2 >= 2LL * p->ctx->num_sms) continue;
                cand.push_back(t);
            }
    for (const SplitTiling& t : cand) {
        const double ms = time_split_plan(p, t, trials, nullptr);
        ++n;
        if (ms < best && ms < margin * *ms_default) { best = ms; pick = t; }
    }
    *ms_best = best;
    *ncand = n;
    return pick;
}

static void upload_blocks_padded(const vmps_ctx* c, const BlockTable& t, const DevLayout& d, const double* host, DBuf& dst,
                                 cudaStream_t st) {
    dst.alloc((size_t)d.total * 8, st, true);
    if (t.n == 0) return;
    DBuf tmp, pk;
    auto pb = pack_blocks(t, d, nullptr);
    upload_vec(pk, pb, st);
    pack_in(c, pk, (int)pb.size(), host, t.total, tmp, dst.as<double>(), st);
    CK(cudaStreamSynchronize(st));   // tmp and pk are released on return
}

static Symmetry make_sym(const vmps_symmetry* s) {
    if (!s || s->nq < 1 || s->nq > kMaxNq) throw std::invalid_argument("symmetry needs 1 <= nq <= 4");
    Symmetry y;
    y.nq = s->nq;
    for (int i = 0; i < s->nq; ++i) {
        if (s->kind[i] != VMPS_SYM_U1 && s->kind[i] != VMPS_SYM_SU2) throw std::invalid_argument("unknown QN kind");
        y.kind[i] = s->kind[i];
    }
    return y;
}

static int pivot_create_common(vmps_ctx* ctx, const Symmetry& sym, const vmps_blocks* L, const double* Ldata,
                               const vmps_blocks* R, const double* Rdata, const vmps_blocks* V,
                               std::unique_ptr<vmps_pivot>& p) {
    if (!ctx) throw std::invalid_argument("null context");
    if (!Ldata || !Rdata) throw std::invalid_argument("null L/R data");
    p.reset(new vmps_pivot_s());
    p->ctx = ctx;
    p->sym = sym;
    p->Lt = parse_blocks(sym, L, true);
    p->Rt = parse_blocks(sym, R, true);
    p->Vt = parse_blocks(sym, V, false);
    p->Ld = make_dev_layout(p->Lt.rows, p->Lt.cols);
    p->Rd = make_dev_layout(p->Rt.rows, p->Rt.cols);
    p->Vd = make_dev_layout(p->Vt.rows, p->Vt.cols);
    return 0;
}

// The two-site task list of an abelian pivot is matched on the GPU of a device
// context (builder.cu: the same chains in the same order as the host builder);
// VMPS_HOST_BUILDER=1 keeps it on the host.
static bool device_builder(const vmps_ctx* c, const Symmetry& sym) {
    if (!c || c->device < 0 || sym.nonabelian()) return false;
    const char* v = std::getenv("VMPS_HOST_BUILDER");
    return !(v && *v && std::strcmp(v, "0") != 0);
}

static void pivot_finish(vmps_pivot* p, const double* Ldata, const double* Rdata) {
    // SU(2): fold sqrt(w_out / w_in) into each chain (weighted dot -> plain dot)
    p->vscale.assign(p->Vt.n, 1.0);
    if (p->sym.nonabelian()) {
        for (int64_t i = 0; i < p->Vt.n; ++i) p->vscale[i] = std::sqrt(p->sym.coeff_dot(p->Vt.qout[i]));
        for (auto& c : p->cs.chains) c.c *= p->vscale[c.out] / p->vscale[c.y];
    }
    if (p->ctx->device < 0) return;
    CK(cudaSetDevice(p->ctx->device));
    upload_blocks_padded(p->ctx, p->Lt, p->Ld, Ldata, p->dL, p->st());
    upload_blocks_padded(p->ctx, p->Rt, p->Rd, Rdata, p->dR, p->st());
    auto pb = pack_blocks(p->Vt, p->Vd, &p->vscale);
    p->npack = (int)pb.size();
    upload_vec(p->dPack, pb, p->st());
    const int nc = dot_nchunk(p->Vd.total);
    p->part.alloc((size_t)std::max(nc, 1) * 8 * 1024, p->st(), true);
    p->scal.alloc(4096 * 8, p->st(), true);
    p->flag.alloc(64, p->st(), true);
    CK(cudaStreamSynchronize(p->st()));
}

extern "C" {

const char* vmps_last_error(void) { return g_last_error.c_str(); }
const char* vmps_version(void) { return "vmps_gb300 0.1 (sm_103a)"; }

int vmps_ctx_create(int device, vmps_ctx** out) {
    API_BEGIN
    if (!out) return set_err(VMPS_E_ARG, "null out");
    if (device == -1) {   // host-only context: task lists and plans, no device work
        auto* c = new vmps_ctx_s();
        c->device = -1;
        *out = c;
        return VMPS_OK;
    }
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return set_err(VMPS_E_ARG, "device index out of range");
    CK(cudaSetDevice(device));
    CK(kernels_init());
    auto* c = new vmps_ctx_s();
    c->device = device;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    CK(cudaEventCreate(&c->ev2));
    CK(cudaMalloc((void**)&c->err, 64));
    CK(cudaMemset(c->err, 0, 64));
    int pma = 0, pmt = 0;
    if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&pmt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess) {
        (void)cudaGetLastError();
        pma = pmt = 0;
    }
    c->pageable_access = pma && pmt;
    CK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
    *out = c;
    API_END
}

int vmps_ctx_set_wait_budget(vmps_ctx* ctx, int64_t cycles) {
    if (!ctx) return set_err(VMPS_E_ARG, "null context");
    if (cycles < 0) return set_err(VMPS_E_ARG, "negative wait budget");
    ctx->wait_budget = (long long)cycles;
    return VMPS_OK;
}

int vmps_ctx_destroy(vmps_ctx* ctx) {
    if (!ctx) return VMPS_OK;
    if (ctx->device < 0) { delete ctx; return VMPS_OK; }
    cudaStreamSynchronize(ctx->stream);
    ctx->la.reset();   // library handles bound to the stream go first
    cudaEventDestroy(ctx->ev0);
    cudaEventDestroy(ctx->ev1);
    cudaEventDestroy(ctx->ev2);
    if (ctx->err) cudaFree(ctx->err);
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return VMPS_OK;
}

int vmps_pivot1_create(vmps_ctx* ctx, const vmps_symmetry* symd, const vmps_blocks* L, const double* Ldata,
                       const vmps_blocks* R, const double* Rdata, const vmps_mpo_site* W, const vmps_blocks* V,
                       vmps_pivot** out) {
    API_BEGIN
    if (!out) return set_err(VMPS_E_ARG, "null out");
    Symmetry sym = make_sym(symd);
    std::unique_ptr<vmps_pivot> p;
    pivot_create_common(ctx, sym, L, Ldata, R, Rdata, V, p);
    MpoView Wv = parse_mpo(sym, W);
    p->cs = device_builder(ctx, sym) ? build_pivot1_device(ctx->stream, sym, p->Lt, p->Rt, Wv, p->Vt)
                                     : build_pivot1(sym, p->Lt, p->Rt, Wv, p->Vt);
    pivot_finish(p.get(), Ldata, Rdata);
    *out = p.release();
    API_END
}

int vmps_pivot2_create(vmps_ctx* ctx, const vmps_symmetry* symd, const vmps_blocks* L, const double* Ldata,
                       const vmps_blocks* R, const double* Rdata, const vmps_mpo_site* W12,
                       const vmps_mpo_site* W34, const vmps_blocks* V, vmps_pivot** out) {
    API_BEGIN
    if (!out) return set_err(VMPS_E_ARG, "null out");
    Symmetry sym = make_sym(symd);
    std::unique_ptr<vmps_pivot> p;
    pivot_create_common(ctx, sym, L, Ldata, R, Rdata, V, p);
    MpoView W1 = parse_mpo(sym, W12), W2 = parse_mpo(sym, W34);
    p->cs = device_builder(ctx, sym) ? build_pivot2_device(ctx->stream, sym, p->Lt, p->Rt, W1, W2, p->Vt)
                                     : build_pivot2(sym, p->Lt, p->Rt, W1, W2, p->Vt);
    pivot_finish(p.get(), Ldata, Rdata);
    *out = p.release();
    API_END
}

int vmps_pivot0_create(vmps_ctx* ctx, const vmps_symmetry* symd, const vmps_blocks* L, const double* Ldata,
                       const vmps_blocks* R, const double* Rdata, const vmps_blocks* V, vmps_pivot** out) {
    API_BEGIN
    if (!out) return set_err(VMPS_E_ARG, "null out");
    Symmetry sym = make_sym(symd);
    std::unique_ptr<vmps_pivot> p;
    pivot_create_common(ctx, sym, L, Ldata, R, Rdata, V, p);
    p->cs = build_pivot0(sym, p->Lt, p->Rt, p->Vt);
    pivot_finish(p.get(), Ldata, Rdata);
    *out = p.release();
    API_END
}

// ---- pivots with several terms (PivotMatrix1/2::Terms) ------------------------
// The reference sums the HxV of every term (pivot/DmrgPivotMatrix1.h:273-287,
// pivot/DmrgPivotMatrix2.h the same).  Here the terms' L and R tables are laid
// end to end in one arena each, every term's chains are built against its own
// tables and shifted to its blocks' place in the arenas, and all chains go into
// one plan: one grouped HxV for the sum, output tiles owned as before.
static void append_table(BlockTable& all, const BlockTable& t, int64_t data_base) {
    for (int64_t i = 0; i < t.n; ++i) {
        all.qin.push_back(t.qin[i]);
        all.qout.push_back(t.qout[i]);
        all.qmid.push_back(t.qmid[i]);
        all.leg.push_back(t.leg[i]);
        all.rows.push_back(t.rows[i]);
        all.cols.push_back(t.cols[i]);
        all.off.push_back(data_base + t.off[i]);
    }
    all.n += t.n;
    all.has_mid = true;
    all.total = data_base + t.total;
}

static int pivot_create_terms(vmps_ctx* ctx, const vmps_symmetry* symd, int kind, int nterms,
                              const vmps_blocks* const* L, const double* const* Ldata, const vmps_blocks* const* R,
                              const double* const* Rdata, const vmps_mpo_site* const* W,
                              const vmps_mpo_site* const* W34, const vmps_blocks* V, vmps_pivot** out) {
    if (!out) return set_err(VMPS_E_ARG, "null out");
    if (!ctx) return set_err(VMPS_E_ARG, "null context");
    if (nterms < 1 || !L || !Ldata || !R || !Rdata || !W || (kind == 2 && !W34))
        return set_err(VMPS_E_ARG, "a pivot needs at least one term and non-null term arrays");
    Symmetry sym = make_sym(symd);
    std::unique_ptr<vmps_pivot> p(new vmps_pivot_s());
    p->ctx = ctx;
    p->sym = sym;
    p->Vt = parse_blocks(sym, V, false);
    std::vector<double> lcat, rcat;
    for (int t = 0; t < nterms; ++t) {
        if (!Ldata[t] || !Rdata[t] || !W[t] || (kind == 2 && !W34[t]))
            throw std::invalid_argument("term " + std::to_string(t) + ": null data or MPO");
        BlockTable Lt = parse_blocks(sym, L[t], true), Rt = parse_blocks(sym, R[t], true);
        ChainSet cs;
        if (kind == 1) cs = build_pivot1(sym, Lt, Rt, parse_mpo(sym, W[t]), p->Vt);
        else cs = build_pivot2(sym, Lt, Rt, parse_mpo(sym, W[t]), parse_mpo(sym, W34[t]), p->Vt);
        const int64_t xb = p->Lt.n, zb = p->Rt.n;
        for (auto& c : cs.chains) {
            c.x += xb;
            c.z += zb;
            p->cs.chains.push_back(c);
        }
        p->cs.n_tasks += cs.n_tasks;
        p->cs.n_chains_raw += cs.n_chains_raw;
        p->cs.flops_reference += cs.flops_reference;
        const int64_t lb = (int64_t)lcat.size(), rb = (int64_t)rcat.size();
        append_table(p->Lt, Lt, lb);
        append_table(p->Rt, Rt, rb);
        lcat.insert(lcat.end(), Ldata[t], Ldata[t] + Lt.total);
        rcat.insert(rcat.end(), Rdata[t], Rdata[t] + Rt.total);
    }
    p->Ld = make_dev_layout(p->Lt.rows, p->Lt.cols);
    p->Rd = make_dev_layout(p->Rt.rows, p->Rt.cols);
    p->Vd = make_dev_layout(p->Vt.rows, p->Vt.cols);
    pivot_finish(p.get(), lcat.data(), rcat.data());
    *out = p.release();
    return VMPS_OK;
}

int vmps_pivot1_create_terms(vmps_ctx* ctx, const vmps_symmetry* sym, int nterms, const vmps_blocks* const* L,
                             const double* const* Ldata, const vmps_blocks* const* R, const double* const* Rdata,
                             const vmps_mpo_site* const* W, const vmps_blocks* V, vmps_pivot** out) {
    API_BEGIN
    return pivot_create_terms(ctx, sym, 1, nterms, L, Ldata, R, Rdata, W, nullptr, V, out);
    API_END
}

int vmps_pivot2_create_terms(vmps_ctx* ctx, const vmps_symmetry* sym, int nterms, const vmps_blocks* const* L,
                             const double* const* Ldata, const vmps_blocks* const* R, const double* const* Rdata,
                             const vmps_mpo_site* const* W12, const vmps_mpo_site* const* W34,
                             const vmps_blocks* V, vmps_pivot** out) {
    API_BEGIN
    return pivot_create_terms(ctx, sym, 2, nterms, L, Ldata, R, Rdata, W12, W34, V, out);
    API_END
}

// ---- autotuner entry points -------------------------------------------------------
int vmps_pivot_autotune(vmps_pivot* p, int trials, vmps_tune_info* out) {
    API_BEGIN
    if (!p || trials < 1 || trials > 1000) return set_err(VMPS_E_ARG, "bad argument");
    require_device(p->ctx);
    vmps_tune_info info{};
    const uint64_t key = pivot_layout_key(p);
    bool cached = false;
    SplitTiling t;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) { t = it->second; cached = true; }
    }
    if (!cached) {
        double a = 0, b = 0;
        int n = 0;
        t = tune_pivot(p, trials, &a, &b, &n);
        info.ms_default = a;
        info.ms_best = b;
        info.candidates = n;
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = t;
    }
    if (!p->tiling_set || !(p->tiling == t)) {
        // the split plan is rebuilt with the chosen tiling on next use
        p->tiling = t;
        p->tiling_set = true;
        DevPlan& dp = p->plans[VMPS_PREC_BF16X3];
        dp.~DevPlan();
        new (&dp) DevPlan();
        if (p->graph[VMPS_PREC_BF16X3]) {
            cudaGraphExecDestroy(p->graph[VMPS_PREC_BF16X3]);
            p->graph[VMPS_PREC_BF16X3] = nullptr;
        }
        p->graph_in[VMPS_PREC_BF16X3] = p->graph_out[VMPS_PREC_BF16X3] = nullptr;
    }
    info.ncap1 = t.ncap1;
    info.ncap2 = t.ncap2;
    info.splitk = t.splitk;
    info.from_cache = cached ? 1 : 0;
    info.layout_key = key;
    if (out) *out = info;
    API_END
}

int vmps_pivot_set_tiling(vmps_pivot* p, int ncap1, int ncap2, int splitk) {
    API_BEGIN
    if (!p) return set_err(VMPS_E_ARG, "null pivot");
    for (int cap : {ncap1, ncap2})
        if (cap < 32 || cap > kUmmaTileN || cap % 32 != 0)
            return set_err(VMPS_E_ARG, "tile N caps must be multiples of 32 up to 256");
    if (splitk < 1 || splitk > 8) return set_err(VMPS_E_ARG, "split-K must be 1..8");
    SplitTiling t;
    t.ncap1 = ncap1; t.ncap2 = ncap2; t.splitk = splitk;
    p->tiling = t;
    p->tiling_set = true;
    DevPlan& dp = p->plans[VMPS_PREC_BF16X3];
    dp.~DevPlan();
    new (&dp) DevPlan();
    if (p->graph[VMPS_PREC_BF16X3]) {
        cudaGraphExecDestroy(p->graph[VMPS_PREC_BF16X3]);
        p->graph[VMPS_PREC_BF16X3] = nullptr;
    }
    p->graph_in[VMPS_PREC_BF16X3] = p->graph_out[VMPS_PREC_BF16X3] = nullptr;
    API_END
}

int vmps_tune_cache_clear(void) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache.clear();
    return VMPS_OK;
}

// ---- excited-state projector (A0proj, Epenalty) ---------------------------------
// pivot/DmrgPivotMatrix1.h:64-68 and :304-331: after the HxV, for every projector
// vector A0_n: overlap = sum over blocks of tr(A0_n^dagger Vin) (no SU(2) weight),
// Vout += Epenalty * overlap * A0_n.  The device vectors carry sqrt(coeff_dot) per
// block (v_dev = s v), so the overlap uses A0 / s and the update adds s A0.
constexpr int kPenMaxRhs = 64;   // right-hand sides one projected HxV may carry

int vmps_pivot_set_penalty(vmps_pivot* p, int nproj, const double* A0, double Epenalty) {
    API_BEGIN
    if (!p) return set_err(VMPS_E_ARG, "null pivot");
    if (nproj < 0 || (nproj > 0 && !A0)) return set_err(VMPS_E_ARG, "bad projector arguments");
    if (!std::isfinite(Epenalty)) return set_err(VMPS_E_NONFINITE, "Epenalty is not finite");
    const int64_t dim = p->Vt.total;
    for (int64_t i = 0; i < (int64_t)nproj * dim; ++i)
        if (!std::isfinite(A0[i])) return set_err(VMPS_E_NONFINITE, "projector vector has NaN/Inf");
    // cached HxV graphs were captured without (or with another) projector
    for (auto& g : p->graph) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    for (int i = 0; i < 3; ++i) p->graph_in[i] = p->graph_out[i] = nullptr;
    p->pen = PenaltyArgs{};
    if (nproj == 0) return VMPS_OK;
    require_device(p->ctx);
    cudaStream_t st = p->st();
    const int64_t n = p->Vd.total;
    std::vector<double> dh((size_t)nproj * dim), ah((size_t)nproj * dim);
    for (int k = 0; k < nproj; ++k)
        for (int64_t b = 0; b < p->Vt.n; ++b) {
            const double sc = p->vscale[b];
            const int64_t o = (int64_t)k * dim + p->Vt.off[b], e = p->Vt.rows[b] * p->Vt.cols[b];
            for (int64_t i = 0; i < e; ++i) {
                dh[o + i] = A0[o + i] / sc;
                ah[o + i] = A0[o + i] * sc;
            }
        }
    auto pb = pack_blocks(p->Vt, p->Vd, nullptr);
    DBuf pk, tmp;
    upload_vec(pk, pb, st);
    p->pen_d.alloc((size_t)nproj * n * 8, st, true);
    p->pen_a.alloc((size_t)nproj * n * 8, st, true);
    for (int k = 0; k < nproj; ++k) {
        pack_in(p->ctx, pk, (int)pb.size(), dh.data() + (int64_t)k * dim, dim, tmp, p->pen_d.as<double>() + k * n, st);
        pack_in(p->ctx, pk, (int)pb.size(), ah.data() + (int64_t)k * dim, dim, tmp, p->pen_a.as<double>() + k * n, st);
        CK(cudaStreamSynchronize(st));   // the staging buffer is reused by the next vector
    }
    PenaltyArgs a{};
    a.n = n;
    a.chunk = dot_chunk(n);
    a.nchunk = dot_nchunk(n);
    a.npen = nproj;
    a.nrhs = 1;
    a.E = Epenalty;
    p->pen_part.alloc((size_t)nproj * kPenMaxRhs * a.nchunk * 8, st, true);
    p->pen_coef.alloc((size_t)nproj * kPenMaxRhs * 8, st, true);
    a.dvec = p->pen_d.as<double>();
    a.avec = p->pen_a.as<double>();
    a.part = p->pen_part.as<double>();
    a.coef = p->pen_coef.as<double>();
    CK(cudaStreamSynchronize(st));
    p->pen = a;
    API_END
}

// Destroy functions never touch the owning context or pivot: callers (and
// garbage collectors) may release objects in any order.  cudaFree waits for
// the device work that still uses the memory.
int vmps_pivot_destroy(vmps_pivot* p) {
    delete p;
    return VMPS_OK;
}

int vmps_pivot_stats(const vmps_pivot* pc, int prec, vmps_plan_stats* out) {
    API_BEGIN
    if (!pc || !out) return set_err(VMPS_E_ARG, "null argument");
    auto* p = const_cast<vmps_pivot*>(pc);
    DevPlan& dp = get_plan(p, prec);
    fill_stats(p->cs, dp.plan, prec, out);
    API_END
}

int vmps_pivot_chains(const vmps_pivot* p, int64_t cap, int64_t* n, int64_t* idx, double* coef, int64_t* n_tasks) {
    if (!p || !n) return set_err(VMPS_E_ARG, "null argument");
    const auto& ch = p->cs.chains;
    *n = (int64_t)ch.size();
    if (n_tasks) *n_tasks = p->cs.n_tasks;
    if (cap <= 0) return VMPS_OK;
    if (cap < *n || !idx || !coef) return set_err(VMPS_E_ARG, "chain buffers smaller than the chain list");
    for (size_t i = 0; i < ch.size(); ++i) {
        idx[4 * i] = ch[i].out;
        idx[4 * i + 1] = ch[i].x;
        idx[4 * i + 2] = ch[i].y;
        idx[4 * i + 3] = ch[i].z;
        coef[i] = ch[i].c;
    }
    return VMPS_OK;
}

int vmps_pivot_dim(const vmps_pivot* p, int64_t* out) {
    if (!p || !out) return set_err(VMPS_E_ARG, "null argument");
    *out = p->Vt.total;
    return VMPS_OK;
}

int vmps_hxv(vmps_pivot* p, const double* vin, double* vout, int prec) {
    API_BEGIN
    if (!p || !vin || !vout) return set_err(VMPS_E_ARG, "null argument");
    require_device(p->ctx);
    cudaStream_t st = p->st();
    ensure_staging(p);
    ensure_io(p);
    DevPlan& dp = get_plan(p, prec);
    if (dp.chunks && p->pen.npen == 0) {   // the projector needs the whole output: no pipeline
        hxv_host_pipelined(p, dp, vin, vout);
        check_device_error(p->ctx);
        return VMPS_OK;
    }
    pack_in(p->ctx, p->dPack, p->npack, vin, p->Vt.total, p->stage_in, p->vin.as<double>(), st);
    pivot_hxv_dev(p, prec, p->vin.as<double>(), p->vout.as<double>());
    pack_out(p->ctx, p->dPack, p->npack, p->vout.as<double>(), p->Vt.total, p->stage_out, vout, st);
    CK(cudaStreamSynchronize(st));
    check_device_error(p->ctx);
    API_END
}

int vmps_hxv_multi(vmps_pivot* p, const double* vin, double* vout, int nrhs, int prec) {
    API_BEGIN
    if (!p || !vin || !vout || nrhs < 1) return set_err(VMPS_E_ARG, "bad argument");
    if (prec == VMPS_PREC_TF32X3) return set_err(VMPS_E_UNSUPPORTED, "3xTF32 runs single-vector HxVs");
    if (prec != VMPS_PREC_FP64 && prec != VMPS_PREC_BF16X3) return set_err(VMPS_E_ARG, "unknown precision");
    if (p->pen.npen > 0 && nrhs > kPenMaxRhs)
        return set_err(VMPS_E_UNSUPPORTED, "a pivot with a projector takes at most 64 right-hand sides");
    require_device(p->ctx);
    cudaStream_t st = p->st();
    ensure_staging(p);
    const int64_t dim = p->Vt.total, n = p->Vd.total;
    p->mvin.alloc((size_t)nrhs * n * 8, st, true);
    p->mvout.alloc((size_t)nrhs * n * 8, st, true);
    double* din = p->mvin.as<double>();
    double* dout = p->mvout.as<double>();
    for (int k = 0; k < nrhs; ++k)
        pack_in(p->ctx, p->dPack, p->npack, vin + (int64_t)k * dim, dim, p->stage_in, din + (int64_t)k * n, st);
    if (prec == VMPS_PREC_BF16X3) {
        DevPlan& dp = get_multi_plan(p, nrhs);
        Operands ops = pivot_ops(p);
        ops.Y = din;
        ops.O = dout;
        run_plan(dp, ops, st);
    } else {
        for (int k = 0; k < nrhs; ++k) pivot_hxv_dev(p, prec, din + (int64_t)k * n, dout + (int64_t)k * n);
    }
    for (int k = 0; k < nrhs; ++k)
        pack_out(p->ctx, p->dPack, p->npack, dout + (int64_t)k * n, dim, p->stage_out, vout + (int64_t)k * dim, st);
    CK(cudaStreamSynchronize(st));
    check_device_error(p->ctx);
    API_END
}

// ---- device vectors ---------------------------------------------------------
int vmps_dvec_create(vmps_pivot* p, vmps_dvec** out) {
    API_BEGIN
    if (!p || !out) return set_err(VMPS_E_ARG, "null argument");
    require_device(p->ctx);
    auto* v = new vmps_dvec_s();
    v->p = p;
    v->n = p->Vd.total;
    try { v->d.alloc((size_t)v->n * 8, p->st(), true); } catch (...) { delete v; throw; }
    *out = v;
    API_END
}
int vmps_dvec_destroy(vmps_dvec* v) {
    delete v;
    return VMPS_OK;
}
int vmps_dvec_upload(vmps_dvec* v, const double* host) {
    API_BEGIN
    if (!v || !host) return set_err(VMPS_E_ARG, "null argument");
    vmps_pivot* p = v->p;
    cudaStream_t st = p->st();
    ensure_staging(p);
    pack_in(p->ctx, p->dPack, p->npack, host, p->Vt.total, p->stage_in, v->d.as<double>(), st);
    CK(cudaMemsetAsync(p->flag.p, 0, 4, st));
    CK(launch_finite(v->d.as<double>(), v->n, p->flag.as<int>(), st));
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, p->flag.p, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (bad) return set_err(VMPS_E_NONFINITE, "input vector holds NaN or Inf");
    API_END
}
int vmps_dvec_download(const vmps_dvec* v, double* host) {
    API_BEGIN
    if (!v || !host) return set_err(VMPS_E_ARG, "null argument");
    vmps_pivot* p = v->p;
    cudaStream_t st = p->st();
    ensure_staging(p);
    pack_out(p->ctx, p->dPack, p->npack, v->d.as<double>(), p->Vt.total, p->stage_out, host, st);
    CK(cudaStreamSynchronize(st));
    API_END
}
int vmps_hxv_device(vmps_pivot* p, const vmps_dvec* vin, vmps_dvec* vout, int prec) {
    API_BEGIN
    if (!p || !vin || !vout || vin->p != p || vout->p != p) return set_err(VMPS_E_ARG, "vectors of another pivot");
    if (vin == vout) return set_err(VMPS_E_ARG, "HxV needs distinct input and output vectors");
    pivot_hxv_dev(p, prec, vin->d.as<double>(), vout->d.as<double>());
    API_END
}
int vmps_dvec_dot(const vmps_dvec* a, const vmps_dvec* b, double* out) {
    API_BEGIN
    if (!a || !b || !out || a->p != b->p) return set_err(VMPS_E_ARG, "bad vectors");
    vmps_pivot* p = a->p;
    CK(launch_dot(a->d.as<double>(), b->d.as<double>(), a->n, p->part.as<double>(), p->scal.as<double>(), p->st()));
    CK(cudaMemcpyAsync(out, p->scal.p, 8, cudaMemcpyDeviceToHost, p->st()));
    CK(cudaStreamSynchronize(p->st()));
    API_END
}
int vmps_dvec_axpy(double alpha, const vmps_dvec* x, vmps_dvec* y) {
    API_BEGIN
    if (!x || !y || x->p != y->p) return set_err(VMPS_E_ARG, "bad vectors");
    CK(launch_axpy(alpha, x->d.as<double>(), y->d.as<double>(), x->n, x->p->st()));
    API_END
}
int vmps_dvec_scale(vmps_dvec* x, double alpha) {
    API_BEGIN
    if (!x) return set_err(VMPS_E_ARG, "bad vector");
    CK(launch_scale(alpha, x->d.as<double>(), x->n, x->p->st()));
    API_END
}
int vmps_dvec_copy(const vmps_dvec* s, vmps_dvec* d) {
    API_BEGIN
    if (!s || !d || s->p != d->p) return set_err(VMPS_E_ARG, "bad vectors");
    CK(cudaMemcpyAsync(d->d.p, s->d.p, (size_t)s->n * 8, cudaMemcpyDeviceToDevice, s->p->st()));
    API_END
}

int vmps_hxv_time(vmps_pivot* p, const vmps_dvec* vin, vmps_dvec* vout, int prec, int n_iter, int use_graph,
                  double* ms_per_hxv, double* ms_phase2) {
    API_BEGIN
    if (!p || !vin || !vout || n_iter <= 0) return set_err(VMPS_E_ARG, "bad argument");
    cudaStream_t st = p->st();
    DevPlan& dp = get_plan(p, prec);
    const double* vi = vin->d.as<double>();
    double* vo = vout->d.as<double>();
    Operands ops = pivot_ops(p);
    ops.Y = vi;
    ops.O = vo;
    if (use_graph) {
        if (!p->graph[prec] || p->graph_in[prec] != vi || p->graph_out[prec] != vo) {
            if (p->graph[prec]) { cudaGraphExecDestroy(p->graph[prec]); p->graph[prec] = nullptr; }
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            run_plan(dp, ops, st);
            CK(cudaStreamEndCapture(st, &g));
            cudaGraphExec_t ge;
            CK(cudaGraphInstantiate(&ge, g, 0));
            cudaGraphDestroy(g);
            p->graph[prec] = ge;
            p->graph_in[prec] = vi;
            p->graph_out[prec] = vo;
        }
    }
    auto one = [&]() {
        if (use_graph) CK(cudaGraphLaunch(p->graph[prec], st));
        else run_plan(dp, ops, st);
    };
    one();
    CK(cudaStreamSynchronize(st));
    CK(cudaEventRecord(p->ctx->ev0, st));
    for (int i = 0; i < n_iter; ++i) one();
    CK(cudaEventRecord(p->ctx->ev1, st));
    CK(cudaEventSynchronize(p->ctx->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, p->ctx->ev0, p->ctx->ev1));
    check_device_error(p->ctx);
    if (ms_per_hxv) *ms_per_hxv = ms / n_iter;
    if (ms_phase2) {
        // second grouped-GEMM phase alone (its inputs are in place from the runs above)
        CK(cudaEventRecord(p->ctx->ev0, st));
        for (int i = 0; i < n_iter; ++i) run_phase(dp, 2, ops, st);
        CK(cudaEventRecord(p->ctx->ev2, st));
        CK(cudaEventSynchronize(p->ctx->ev2));
        float ms2 = 0;
        CK(cudaEventElapsedTime(&ms2, p->ctx->ev0, p->ctx->ev2));
        *ms_phase2 = ms2 / n_iter;
    }
    API_END
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Lanczos (FP64 Krylov vectors, host tridiagonal solve)
// ---------------------------------------------------------------------------
namespace {
// lowest eigenpair of the symmetric tridiagonal matrix (a: diagonal, b: off-diagonal)
// Sturm-sequence bisection for the eigenvalue, inverse iteration for the vector.
double sturm_count_below(const std::vector<double>& a, const std::vector<double>& b, double x) {
    int cnt = 0;
    double d = 1.0;
    const size_t n = a.size();
    for (size_t i = 0; i < n; ++i) {
        double bb = i ? b[i - 1] * b[i - 1] : 0.0;
        d = (a[i] - x) - (i ? bb / d : 0.0);
        if (d == 0.0) d = -1e-300;
        if (d < 0) ++cnt;
    }
    return cnt;
}
void tridiag_lowest(const std::vector<double>& a, const std::vector<double>& b, double& theta, std::vector<double>& y) {
    const size_t n = a.size();
    double lo = a[0], hi = a[0];
    for (size_t i = 0; i < n; ++i) {
        double r = (i ? std::abs(b[i - 1]) : 0.0) + (i + 1 < n ? std::abs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    const double scale = std::max(std::abs(lo), std::abs(hi)) + 1e-300;
    // bisection to 1e-9 of the spectral scale; inverse iteration then converges
    // at the ratio (shift distance) / (gap) per step and the Rayleigh quotient of
    // its vector carries the eigenvalue to working precision
    for (int it = 0; it < 80 && hi - lo > 1e-9 * scale; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm_count_below(a, b, mid) >= 1) hi = mid; else lo = mid;
    }
    theta = 0.5 * (lo + hi);
    // inverse iteration on (T - shift): tridiagonal LU with partial pivoting
    // (the elimination of LAPACK dgttrf/dgtts2, restated)
    y.assign(n, 1.0 / std::sqrt((double)n));
    const double shift = lo - 1e-9 * scale;
    std::vector<double> d(n), du(n, 0.0), du2(n, 0.0), dl(n, 0.0);
    std::vector<char> swp(n, 0);
    for (size_t i = 0; i < n; ++i) d[i] = a[i] - shift;
    for (size_t i = 0; i + 1 < n; ++i) { du[i] = b[i]; dl[i] = b[i]; }
    for (size_t i = 0; i + 1 < n; ++i) {
        if (std::abs(d[i]) >= std::abs(dl[i])) {
            const double f = d[i] != 0.0 ? dl[i] / d[i] : 0.0;
            dl[i] = f;
            d[i + 1] -= f * du[i];
        } else {
            const double f = d[i] / dl[i];
            d[i] = dl[i];
            dl[i] = f;
            const double t = du[i];
            du[i] = d[i + 1];
            d[i + 1] = t - f * d[i + 1];
            if (i + 2 < n) { du2[i] = du[i + 1]; du[i + 1] = -f * du[i + 1]; }
            swp[i] = 1;
        }
    }
    for (size_t i = 0; i < n; ++i) if (d[i] == 0.0) d[i] = 1e-300;
    std::vector<double> x(n);
    for (int it = 0; it < 3; ++it) {
        x = y;
        for (size_t i = 0; i + 1 < n; ++i) {
            if (!swp[i]) x[i + 1] -= dl[i] * x[i];
            else { const double t = x[i]; x[i] = x[i + 1]; x[i + 1] = t - dl[i] * x[i]; }
        }
        for (size_t ii = n; ii-- > 0;) {
            double s = x[ii];
            if (ii + 1 < n) s -= du[ii] * x[ii + 1];
            if (ii + 2 < n) s -= du2[ii] * x[ii + 2];
            x[ii] = s / d[ii];
        }
        double nrm = 0;
        for (double v : x) nrm += v * v;
        nrm = std::sqrt(nrm);
        for (size_t i = 0; i < n; ++i) y[i] = x[i] / nrm;
    }
    // fix sign convention: largest component positive
    size_t im = 0;
    for (size_t i = 1; i < n; ++i) if (std::abs(y[i]) > std::abs(y[im])) im = i;
    if (y[im] < 0) for (double& v : y) v = -v;
    // Rayleigh quotient y^T T y (y has unit norm)
    double rq = 0;
    for (size_t i = 0; i < n; ++i) {
        double t = a[i] * y[i];
        if (i > 0) t += b[i - 1] * y[i - 1];
        if (i + 1 < n) t += b[i] * y[i + 1];
        rq += y[i] * t;
    }
    if (rq >= lo - 1e-9 * scale && rq <= hi + 1e-9 * scale) theta = rq;
}

// second-lowest eigenvalue of the tridiagonal (Sturm bisection to 1e-9 of the
// spectral scale); +inf for a 1 x 1 matrix
double tridiag_second(const std::vector<double>& a, const std::vector<double>& b) {
    const size_t n = a.size();
    if (n < 2) return HUGE_VAL;
    double lo = a[0], hi = a[0];
    for (size_t i = 0; i < n; ++i) {
        const double r = (i ? std::abs(b[i - 1]) : 0.0) + (i + 1 < n ? std::abs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    const double scale = std::max(std::abs(lo), std::abs(hi)) + 1e-300;
    for (int it = 0; it < 80 && hi - lo > 1e-9 * scale; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm_count_below(a, b, mid) >= 2) hi = mid; else lo = mid;
    }
    return 0.5 * (lo + hi);
}

double dev_dot(vmps_pivot* p, const double* x, const double* y, int64_t n) {
    CK(launch_dot(x, y, n, p->part.as<double>(), p->scal.as<double>(), p->st()));
    double r;
    CK(cudaMemcpyAsync(&r, p->scal.p, 8, cudaMemcpyDeviceToHost, p->st()));
    CK(cudaStreamSynchronize(p->st()));
    return r;
}

// The Krylov workspace of a context (LzWork, declared with the context) for
// vectors of length n and `cap` iterations.
LzWork& lz_work(vmps_ctx* c, int64_t n, int cap) {
    if (!c->lz) c->lz.reset(new LzWork());
    LzWork& W = *c->lz;
    cudaStream_t st = c->stream;
    if (W.n != n || W.cap < cap) {
        W.n = n;
        W.ld = (n + 31) / 32 * 32;
        W.cap = std::max(W.cap, (cap + 31) / 32 * 32);
        W.sh = lz_shape(n, c->num_sms);
        W.K.alloc((size_t)(W.cap + 1) * W.ld * 8, st, false);
        for (DBuf* b : {&W.w, &W.q, &W.x, &W.u}) b->alloc((size_t)W.ld * 8, st, false);
        W.part.alloc((size_t)std::max(W.cap, 2) * W.sh.nchunk * 8, st, false);
        W.small.alloc(((size_t)6 * W.cap + 8) * 8, st, true);
        if (W.host_cap < W.cap) {
            if (W.host) cudaFreeHost(W.host);
            W.host = nullptr;
            W.host_cap = 0;
            CK(cudaHostAlloc((void**)&W.host, (size_t)2 * W.cap * 8, cudaHostAllocMapped));
            CK(cudaHostGetDevicePointer((void**)&W.host_dev, W.host, 0));
            W.host_cap = W.cap;
        }
    }
    for (auto& e : W.ev)
        if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return W;
}

// Start-vector residual (relative to its energy) below which a split-precision
// solve runs as FP64 Lanczos: about twice the residual that the BF16x3
// operator's rounding noise (4e-6 relative) leaves on an exact eigenvector.
constexpr double kSplitProbeRel = 1e-5;
// Model residual (relative to the energy) at which a refined split-precision
// phase stops: a tenth of the FP64 residual the operator's noise leaves on its
// Ritz vector; iterations past it only resolve that noise, and the refinement
// rounds start from the FP64 residual in any case.
constexpr double kSplitStateRel = 5e-7;

// FP32 start of a split-precision run: K32_0 = q32 = (float) K_0, padding zero
void lz_start_f32(LzWork& W, cudaStream_t st) {
    // (DBuf::alloc keeps a buffer that is already large enough)
    W.K32.alloc((size_t)(W.cap + 1) * W.ld * 4, st, false);
    W.w32.alloc((size_t)W.ld * 4, st, false);
    W.q32.alloc((size_t)W.ld * 4, st, false);
    CK(cudaMemsetAsync(W.w32.p, 0, (size_t)W.ld * 4, st));
    CK(launch_lz_to_f32(W.K.as<double>(), W.K32.as<float>(), W.ld, st));
    CK(cudaMemcpyAsync(W.q32.p, W.K32.p, (size_t)W.ld * 4, cudaMemcpyDeviceToDevice, st));
}

// one Lanczos run from K_0 (= q, normalised), at most kmax iterations
struct LzResult {
    int m = 0;          // basis vectors of the Ritz space
    int launched = 0;   // HxV iterations the device ran (the last may run past convergence)
    double theta = 0, res = 0;
    double ms_wait = 0, ms_host = 0;   // host time blocked on the device / in the tridiagonal solves
    bool aborted = false;              // stopped by the probe after iteration 0
    std::vector<double> alpha, beta, y;
};

// probe_rel > 0: iteration 0 runs alone first, and the run stops after it
// (aborted = true) when beta_0 > probe_rel * max(1, |alpha_0|), i.e. when the
// start vector's residual is above that fraction of its energy.
// first_row = {alpha_0, beta_0}: the caller has set K_0, K_1 (and q = K_1) and
// knows the first row of the tridiagonal exactly; the run starts at iteration 1.
// state_rel > 0: the residual test is |r| <= max(tol_state, state_rel * max(1, |theta|)).
LzResult lz_run(vmps_pivot* p, LzWork& W, int prec, int kmax, double tol_eigval, double tol_state,
                double probe_rel = 0, const double* first_row = nullptr, double state_rel = 0) {
    cudaStream_t st = p->st();
    DevPlan& dp = get_plan(p, prec);
    const bool f32 = prec != VMPS_PREC_FP64;   // split-precision runs keep FP32 Krylov vectors
    LzArgs a{};
    a.fp32 = f32;
    a.K = f32 ? W.K32.p : W.K.p;
    a.ld = W.ld;
    a.w = f32 ? W.w32.p : W.w.p;
    a.q = f32 ? W.q32.p : W.q.p;
    a.part = W.part.as<double>();
    a.cl = W.cl();
    a.coef = W.coef();
    a.ab = W.ab();
    a.host_ab = W.host_dev;
    a.ctl = W.ctl();
    a.n = W.n;
    a.kmax = W.cap;
    a.nchunk = W.sh.nchunk;
    const int j0 = first_row ? 1 : 0;
    CK(cudaMemsetAsync(W.ctl(), 0, 8 * sizeof(unsigned), st));
    if (j0) {
        static const unsigned kStartOne = 1;
        CK(cudaMemcpyAsync(W.ctl(), &kStartOne, sizeof(unsigned), cudaMemcpyHostToDevice, st));
    }
    Operands ops = pivot_ops(p);
    if (f32) {
        ops.Yf = W.q32.as<float>();
        ops.Of = W.w32.as<float>();
    } else {
        ops.Y = W.q.as<double>();
        ops.O = W.w.as<double>();
    }
    // one iteration = the HxV plan + the four step kernels, captured once
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
        run_plan(dp, ops, st);
        CK(launch_lz_step(a, W.sh.per_thread, st));
    } catch (...) {
        if (cudaStreamEndCapture(st, &g) == cudaSuccess && g) cudaGraphDestroy(g);
        throw;
    }
    CK(cudaStreamEndCapture(st, &g));
    cudaGraphExec_t ge = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    CK(ie);
    struct ExecGuard {
        cudaGraphExec_t e;
        ~ExecGuard() { cudaGraphExecDestroy(e); }
    } guard{ge};

    // The host trails the device by one iteration: iteration j+1 is queued
    // before the host waits for alpha_j, beta_j and solves the tridiagonal
    // problem, so the device never idles on the host.
    LzResult r;
    volatile const double* hab = W.host;
    double theta = 0, theta_prev = 1e300, res = 0;
    std::vector<double> y;
    if (j0) {
        r.alpha.push_back(first_row[0]);
        r.beta.push_back(first_row[1]);
    }
    auto launch = [&]() {
        CK(cudaGraphLaunch(ge, st));
        CK(cudaEventRecord(W.ev[r.launched & 1], st));
        ++r.launched;
    };
    launch();
    int j = j0;
    for (j = j0; j < kmax; ++j) {
        if (r.launched < kmax - j0 && !(probe_rel > 0 && j == 0)) launch();
        const auto tw = std::chrono::steady_clock::now();
        CK(cudaEventSynchronize(W.ev[(j - j0) & 1]));
        const auto th = std::chrono::steady_clock::now();
        r.ms_wait += std::chrono::duration<double, std::milli>(th - tw).count();
        struct HostTimer {
            std::chrono::steady_clock::time_point t;
            double* acc;
            ~HostTimer() { *acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count(); }
        } host_timer{th, &r.ms_host};
        const double a_j = hab[j], b_j = hab[W.cap + j];
        if (probe_rel > 0 && j == 0) {
            if (b_j > probe_rel * std::max(1.0, std::abs(a_j))) {
                r.aborted = true;
                r.theta = a_j;
                r.res = b_j;
                return r;
            }
            if (r.launched < kmax) launch();
        }
        r.alpha.push_back(a_j);
        tridiag_lowest(r.alpha, r.beta, theta, y);
        res = std::abs(b_j * y.back());
        const bool conv_e = std::abs(theta - theta_prev) <= tol_eigval * std::max(1.0, std::abs(theta));
        theta_prev = theta;
        const double tol_res = std::max(tol_state, state_rel * std::max(1.0, std::abs(theta)));
        if ((conv_e && res <= tol_res) || b_j <= 1e-14 * std::max(1.0, std::abs(theta)) || j + 1 == kmax) {
            ++j;
            break;
        }
        r.beta.push_back(b_j);
    }
    r.m = j;
    r.theta = theta;
    r.res = res;
    r.y = y;
    return r;
}

// x = K y / |K y| for the Ritz coefficients of a run
void lz_ritz(vmps_pivot* p, LzWork& W, const std::vector<double>& y, double* x, bool f32) {
    cudaStream_t st = p->st();
    CK(cudaMemcpyAsync(W.g(), y.data(), y.size() * 8, cudaMemcpyHostToDevice, st));
    CK(launch_lz_combine(f32 ? W.K32.p : W.K.p, f32, W.ld, (int)y.size(), W.n, W.g(), x, st));
    const double nx = std::sqrt(dev_dot(p, x, x, W.n));
    if (!(nx > 0) || !std::isfinite(nx)) throw CudaFail("Ritz vector is zero or not finite");
    CK(launch_scale(1.0 / nx, x, W.n, st));
}

// Correction of a Ritz vector y (unit norm, lowest eigenvector of the
// tridiagonal T = tridiag(beta, alpha, beta)) inside the Krylov space: the
// Jacobi-Davidson correction equation restricted to span(K),
//     P (T - th) P z = -P g,   P = 1 - y y^T,   z orthogonal to y,
// with g = K^T r the projection of the residual r = H x - th x.  Solved by
// conjugate gradients on the m-dimensional system (positive definite on y's
// complement while th lies below the second Ritz value; the iteration stops
// at the first direction of non-positive curvature).  `model` returns the
// second-order energy change 2 g.z + z.(T - th) z of the step.
std::vector<double> krylov_correction(const std::vector<double>& a, const std::vector<double>& b, double th,
                                      const std::vector<double>& y, const std::vector<double>& g, double* model) {
    const size_t m = a.size();
    auto Tv = [&](const std::vector<double>& v, std::vector<double>& out) {
        for (size_t i = 0; i < m; ++i) {
            double s = (a[i] - th) * v[i];
            if (i > 0) s += b[i - 1] * v[i - 1];
            if (i + 1 < m) s += b[i] * v[i + 1];
            out[i] = s;
        }
    };
    auto proj = [&](std::vector<double>& v) {
        double d = 0;
        for (size_t i = 0; i < m; ++i) d += y[i] * v[i];
        for (size_t i = 0; i < m; ++i) v[i] -= d * y[i];
    };
    auto dot = [&](const std::vector<double>& u, const std::vector<double>& v) {
        double s = 0;
        for (size_t i = 0; i < m; ++i) s += u[i] * v[i];
        return s;
    };
    std::vector<double> z(m, 0.0), r(g), p, Ap(m);
    for (double& v : r) v = -v;
    proj(r);
    p = r;
    double rr = dot(r, r);
    const double r0 = std::sqrt(rr);
    for (size_t it = 0; it < 2 * m + 10 && rr > 0 && std::sqrt(rr) > 1e-14 * r0; ++it) {
        Tv(p, Ap);
        proj(Ap);
        const double pAp = dot(p, Ap);
        if (!(pAp > 0)) break;
        const double al = rr / pAp;
        for (size_t i = 0; i < m; ++i) {
            z[i] += al * p[i];
            r[i] -= al * Ap[i];
        }
        proj(r);
        const double rr2 = dot(r, r);
        for (size_t i = 0; i < m; ++i) p[i] = r[i] + (rr2 / rr) * p[i];
        rr = rr2;
    }
    proj(z);
    std::vector<double> Tz(m);
    Tv(z, Tz);
    *model = 2 * dot(g, z) + dot(z, Tz);
    return z;
}
// Ritz vector of a run started from first_row: out = y_0 x0 + sum_{i>=1} y_i K_i,
// normalised.  K_0 of that run is the FP32 copy of x0; the FP64 x0 itself enters
// here so that the result keeps FP64 accuracy along it.
void lz_ritz_mixed(vmps_pivot* p, LzWork& W, const std::vector<double>& y, const double* x0, double* out) {
    cudaStream_t st = p->st();
    const int m = (int)y.size();
    if (m < 1) throw std::logic_error("empty Ritz coefficients");
    if (m > 1) {
        CK(cudaMemcpyAsync(W.g(), y.data() + 1, (size_t)(m - 1) * 8, cudaMemcpyHostToDevice, st));
        CK(launch_lz_combine(W.K32.as<float>() + W.ld, 1, W.ld, m - 1, W.n, W.g(), out, st));
    } else {
        CK(cudaMemsetAsync(out, 0, (size_t)W.n * 8, st));
    }
    CK(launch_axpy(y[0], x0, out, W.n, st));
    const double nx = std::sqrt(dev_dot(p, out, out, W.n));
    if (!(nx > 0) || !std::isfinite(nx)) throw CudaFail("Ritz vector is zero or not finite");
    CK(launch_scale(1.0 / nx, out, W.n, st));
}

// Model residual, relative to the residual a refinement round starts from, at
// which its split-precision run stops: below the reduction the split operator's
// noise allows in one round.
constexpr double kRoundReduce = 1e-3;
// Refinement rounds replace closing FP64 Lanczos steps when an FP64 HxV costs at
// least this many split-precision Lanczos steps: a round spends a few tens of
// split steps and one FP64 HxV where the FP64 steps need several FP64 HxVs.
constexpr double kRoundMinRatio = 10;

// The ratio comes from a cost model of the plans (not from timings, so that the
// choice, and with it every result bit, does not depend on the run): GEMM work at
// the rates the engines reach on GB300 (FP64 DMMA 0.87 TFLOP/s, bf16 tensor work
// as issued 530 TFLOP/s), the Lanczos step's vector reads and writes at 5 TB/s,
// and 3 us per launch.
constexpr double kFp64FlopsPerMs = 0.87e9, kTensorFlopsPerMs = 5.3e11, kStepBytesPerMs = 5.0e9,
                 kLaunchMs = 0.003;
double est_ms_fp64_hxv(const Plan& p) { return (p.p1.flops + p.p2.flops) / kFp64FlopsPerMs + 2 * kLaunchMs; }
// one split Lanczos iteration with a basis of j rows (FP32 vectors): HxV + step kernels
double est_ms_split_step(const Plan& p, int64_t n, int j) {
    // TF32 MMAs run at half the bf16 rate
    const double tensor = (phase_tensor_flops(p.p1, p.kstep) + phase_tensor_flops(p.p2, p.kstep)) * (p.elt == 4 ? 2 : 1);
    const double bytes = 4.0 * (double)n * (2.0 * (j + 1) + 8.0);
    return tensor / kTensorFlopsPerMs + bytes / kStepBytesPerMs + 8 * kLaunchMs;
}

// VMPS_LANCZOS_REFINE = rounds | polish pins the refinement; unset or auto
// chooses by the modelled cost ratio
int refine_mode() {
    const char* v = std::getenv("VMPS_LANCZOS_REFINE");
    if (!v || !*v || !std::strcmp(v, "auto")) return 0;
    if (!std::strcmp(v, "rounds")) return 1;
    if (!std::strcmp(v, "polish")) return 2;
    throw std::invalid_argument("VMPS_LANCZOS_REFINE must be auto, rounds or polish");
}
// VMPS_LANCZOS_PROBE = off: split-precision solves skip the FP64 probe, so the
// split phase runs even from a start vector that is already an eigenvector to
// the split operator's noise level; unset or on keeps the probe
bool probe_enabled() {
    const char* v = std::getenv("VMPS_LANCZOS_PROBE");
    if (!v || !*v || !std::strcmp(v, "on")) return true;
    if (!std::strcmp(v, "off")) return false;
    throw std::invalid_argument("VMPS_LANCZOS_PROBE must be on or off");
}
}  // namespace

extern "C" int vmps_lanczos_ground(vmps_pivot* p, double* v, int prec, int max_iter, double tol_eigval,
                                   double tol_state, int refine_iters, double* energy, vmps_lanczos_stats* stats) {
    API_BEGIN
    if (!p || !v || !energy || max_iter <= 0 || refine_iters < 0) return set_err(VMPS_E_ARG, "bad argument");
    if (max_iter >= kLzMaxIter || refine_iters >= kLzMaxIter)
        return set_err(VMPS_E_ARG, "max_iter and refine_iters must be below " + std::to_string(kLzMaxIter));
    if (prec != VMPS_PREC_FP64 && prec != VMPS_PREC_BF16X3 && prec != VMPS_PREC_TF32X3)
        return set_err(VMPS_E_ARG, "unknown precision");
    require_device(p->ctx);
    std::lock_guard<std::mutex> lock(p->ctx->lz_mu);
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = p->st();
    const bool refine = prec != VMPS_PREC_FP64 && refine_iters > 0;
    const int mode = refine_mode();
    // a refined solve may end in the FP64 probe: the split plan is built when
    // the split phase starts
    get_plan(p, refine ? VMPS_PREC_FP64 : prec);
    const int64_t n = p->Vd.total;
    LzWork& W = lz_work(p->ctx, n, std::max(max_iter, refine_iters));
    // padding positions of the layout stay zero in every vector
    for (double* b : {W.K.as<double>(), W.w.as<double>(), W.q.as<double>(), W.x.as<double>(), W.u.as<double>()})
        CK(cudaMemsetAsync(b, 0, (size_t)W.ld * 8, st));
    double* K0 = W.K.as<double>();
    ensure_staging(p);
    pack_in(p->ctx, p->dPack, p->npack, v, p->Vt.total, p->stage_in, K0, st);
    const double n0 = std::sqrt(dev_dot(p, K0, K0, n));
    if (!(n0 > 0) || !std::isfinite(n0)) return set_err(VMPS_E_NONFINITE, "start vector is zero or not finite");
    CK(launch_scale(1.0 / n0, K0, n, st));
    CK(cudaMemcpyAsync(W.q.p, K0, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));

    vmps_lanczos_stats s{};
    double* x = W.x.as<double>();
    double e = 0, res = 0;
    auto account = [&](const LzResult& r, int run_prec) {
        (run_prec == VMPS_PREC_FP64 ? s.hxv_fp64 : s.hxv_split) += r.launched;
        s.ms_wait += r.ms_wait;
        s.ms_host += r.ms_host;
    };
    bool split_phase = true;
    if (refine && probe_enabled()) {
        // Probe: FP64 Lanczos whose first iteration gives the start vector's
        // FP64 residual.  A start vector already within a few times the split
        // operator's noise of an eigenvector (late sweeps) gains nothing from
        // split HxVs, which cannot resolve it further; the FP64 run goes on and
        // its first HxV is not wasted.  Otherwise the split path starts over.
        LzResult r0 = lz_run(p, W, VMPS_PREC_FP64, max_iter, tol_eigval, tol_state, kSplitProbeRel);
        account(r0, VMPS_PREC_FP64);
        if (!r0.aborted) {
            split_phase = false;
            s.iterations = r0.m;
            s.energy_first = r0.theta;
            lz_ritz(p, W, r0.y, x, false);
            e = r0.theta;
            res = r0.res;
        } else {
            CK(cudaMemcpyAsync(W.q.p, K0, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
        }
    }
    if (split_phase) {
        const bool f32 = prec != VMPS_PREC_FP64;
        if (f32) lz_start_f32(W, st);
        LzResult r1 = lz_run(p, W, prec, max_iter, tol_eigval, tol_state, 0, nullptr, refine ? kSplitStateRel : 0);
        account(r1, prec);
        s.iterations = r1.m;
        s.energy_first = r1.theta;
        e = r1.theta;
        res = r1.res;
        lz_ritz(p, W, r1.y, x, f32);
        if (refine) {
            // FP64 residual of the split-precision Ritz vector x, then one of two
            // refinements, whichever the modelled cost ratio favours:
            //
            // * Rounds (an FP64 HxV costs many split steps).  A round holds x
            //   (FP64, unit norm), its Rayleigh quotient th and residual
            //   r = H x - th x.  A split-precision Lanczos run starts from the pair
            //   K_0 = x, K_1 = r / |r|: the first row of its tridiagonal (th, |r|) is
            //   FP64-exact, the later rows come from split HxVs.  Its Ritz vector
            //   solves the correction equation for x; the split operator's noise
            //   enters only through the correction (second order).  One FP64 HxV
            //   gives the new x's th and r.  A round that does not halve |r| hands
            //   the rest of the budget to FP64 Lanczos steps.
            // * Correction and polish (FP64 HxVs are cheap).  The residual,
            //   projected on the split Krylov space, drives the Jacobi-Davidson
            //   correction equation solved in that space; closing FP64 Lanczos
            //   steps start from the corrected vector.
            double* u = W.u.as<double>();
            double* xn = W.w.as<double>();   // a round's candidate (the FP64 w buffer is idle in split runs)
            int budget = refine_iters;        // FP64 HxVs of the refinement
            auto residual = [&](const double* xv, double& th, double& rn) {
                pivot_hxv_dev(p, VMPS_PREC_FP64, xv, u);
                s.hxv_fp64++;
                --budget;
                th = dev_dot(p, xv, u, n);
                CK(launch_axpy(-th, xv, u, n, st));
                rn = std::sqrt(dev_dot(p, u, u, n));
            };
            // converged: residual within tol_state, and the energy error bound
            // |r|^2 / gap (gap = second Ritz value - first, of the last run's
            // tridiagonal) within tol_eigval
            auto converged = [&](double th, double rn, double gap) {
                return rn <= tol_state && rn * rn <= tol_eigval * std::max(1.0, std::abs(th)) * gap;
            };
            double th = 0, rn = 0;
            residual(x, th, rn);
            const double ms_fp64 = est_ms_fp64_hxv(get_plan(p, VMPS_PREC_FP64).plan);
            const double ms_split_step = est_ms_split_step(get_plan(p, prec).plan, n, std::max(1, r1.m / 2));
            double gap = std::max(0.0, tridiag_second(r1.alpha, r1.beta) - r1.theta);
            bool polish = false;
            e = th;
            res = rn;
            if (converged(th, rn, gap) || budget <= 0) {
            } else if (mode == 1 || (mode == 0 && ms_fp64 >= kRoundMinRatio * ms_split_step)) {
                float* K32 = W.K32.as<float>();
                while (!converged(th, rn, gap) && budget > 0 && rn > 0) {
                    CK(launch_scale(1.0 / rn, u, n, st));
                    CK(launch_lz_to_f32(x, K32, W.ld, st));
                    CK(launch_lz_to_f32(u, K32 + W.ld, W.ld, st));
                    CK(cudaMemcpyAsync(W.q32.p, K32 + W.ld, (size_t)W.ld * 4, cudaMemcpyDeviceToDevice, st));
                    const double row0[2] = {th, rn};
                    LzResult ri = lz_run(p, W, prec, std::max(2, max_iter), HUGE_VAL,
                                         std::max(0.1 * tol_state, kRoundReduce * rn), 0, row0);
                    account(ri, prec);
                    lz_ritz_mixed(p, W, ri.y, x, xn);
                    double th2 = 0, rn2 = 0;
                    residual(xn, th2, rn2);
                    s.refine_iterations++;
                    if (!(rn2 < rn)) {
                        polish = true;
                        break;
                    }
                    CK(cudaMemcpyAsync(x, xn, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
                    polish = rn2 > 0.5 * rn;
                    th = th2;
                    rn = rn2;
                    gap = std::max(0.0, tridiag_second(ri.alpha, ri.beta) - ri.theta);
                    if (polish) break;
                }
                e = th;
                res = rn;
            } else {
                CK(launch_lz_mdot(W.K32.p, 1, W.ld, r1.m, n, u, W.part.as<double>(), W.sh, W.g(), st));
                std::vector<double> g(r1.m);
                CK(cudaMemcpyAsync(g.data(), W.g(), (size_t)r1.m * 8, cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                double model = 0;
                std::vector<double> z = krylov_correction(r1.alpha, r1.beta, th, r1.y, g, &model);
                double zn = 0;
                for (double t : z) zn += t * t;
                if (model < 0 && std::sqrt(zn) < 0.5) {
                    std::vector<double> yz(r1.y);
                    for (size_t i = 0; i < yz.size(); ++i) yz[i] += z[i];
                    lz_ritz(p, W, yz, x, true);
                }
                polish = true;
            }
            if (polish && budget > 0) {
                CK(cudaMemcpyAsync(K0, x, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
                CK(cudaMemcpyAsync(W.q.p, x, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
                LzResult r2 = lz_run(p, W, VMPS_PREC_FP64, std::max(1, budget), tol_eigval, tol_state);
                account(r2, VMPS_PREC_FP64);
                s.refine_iterations += r2.m;
                lz_ritz(p, W, r2.y, x, false);
                e = r2.theta;
                res = r2.res;
            }
        }
    }
    s.residual = res;
    pack_out(p->ctx, p->dPack, p->npack, x, p->Vt.total, p->stage_out, v, st);
    CK(cudaStreamSynchronize(st));
    check_device_error(p->ctx);
    *energy = e;
    s.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = s;
    API_END
}

extern "C" int vmps_spectral_bounds(vmps_pivot* p, const double* v, int iters, double* emin, double* emax) {
    API_BEGIN
    if (!p || !v || !emin || !emax || iters < 1 || iters >= kLzMaxIter) return set_err(VMPS_E_ARG, "bad argument");
    require_device(p->ctx);
    std::lock_guard<std::mutex> lock(p->ctx->lz_mu);
    cudaStream_t st = p->st();
    get_plan(p, VMPS_PREC_FP64);
    const int64_t n = p->Vd.total;
    LzWork& W = lz_work(p->ctx, n, iters);
    for (double* b : {W.K.as<double>(), W.w.as<double>(), W.q.as<double>()})
        CK(cudaMemsetAsync(b, 0, (size_t)W.ld * 8, st));
    double* K0 = W.K.as<double>();
    ensure_staging(p);
    pack_in(p->ctx, p->dPack, p->npack, v, p->Vt.total, p->stage_in, K0, st);
    const double n0 = std::sqrt(dev_dot(p, K0, K0, n));
    if (!(n0 > 0) || !std::isfinite(n0)) return set_err(VMPS_E_NONFINITE, "start vector is zero or not finite");
    CK(launch_scale(1.0 / n0, K0, n, st));
    CK(cudaMemcpyAsync(W.q.p, K0, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    // no convergence test: `iters` steps (or fewer at an invariant subspace)
    LzResult r = lz_run(p, W, VMPS_PREC_FP64, iters, 0.0, -1.0);
    CK(cudaStreamSynchronize(st));
    check_device_error(p->ctx);
    std::vector<double> a(r.alpha), b(r.beta), y;
    b.resize(a.size() > 0 ? a.size() - 1 : 0);
    double lo = 0, hi = 0;
    tridiag_lowest(a, b, lo, y);
    for (double& x : a) x = -x;
    tridiag_lowest(a, b, hi, y);
    *emin = lo;
    *emax = -hi;
    API_END
}

// Chebyshev moments of nrhs start vectors advanced together: the recursion
// t_{n+1} = 2 H~ t_n - t_{n-1} of the reference's polyIter / polyCompress
// (DmrgLinearAlgebra.h:550-566, solvers/MpsCompressor.h:1372-1564) on the
// pivot, with H~ = (H - b)/a.  One step is one CUDA graph: the HxV of all
// right-hand sides (split precision: one grouped multi-RHS launch pair; FP64:
// the plain HxV per vector) and cheb_step_kernel (update and FP64 moments).
// The three vector buffers rotate, so three graphs cover every step.
// the moments of nrhs start vectors, per part (block ranges [part_blocks[j], part_blocks[j+1])
// of the vector layout; nparts 1 with part_blocks null: the whole vector)
static int chebyshev_moments(vmps_pivot* p, const double* v0, int nrhs, int nmom, double a, double b, int prec,
                             int nparts, const int64_t* part_blocks, double* mu, vmps_cheb_stats* stats) {
    API_BEGIN
    if (!p || !v0 || !mu || nrhs < 1 || nrhs > 65535 || nmom < 1) return set_err(VMPS_E_ARG, "bad argument");
    if (nparts < 1 || nparts > kChebMaxParts || (nparts > 1 && !part_blocks))
        return set_err(VMPS_E_ARG, "parts: 1 to 8 block ranges");
    int64_t pbeg[kChebMaxParts + 1];
    {
        const int64_t nb = p->Vt.n;
        for (int j = 0; j <= nparts; ++j) {
            const int64_t bj = part_blocks ? part_blocks[j] : (j == 0 ? 0 : nb);
            if (bj < 0 || bj > nb || (j == 0 && bj != 0) || (j == nparts && bj != nb) ||
                (j > 0 && bj <= (part_blocks ? part_blocks[j - 1] : 0)))
                return set_err(VMPS_E_ARG, "part boundaries must rise from block 0 to the last block");
            pbeg[j] = j == nparts ? p->Vd.total : p->Vd.off[bj];
        }
    }
    if (!(a > 0) || !std::isfinite(a) || !std::isfinite(b)) return set_err(VMPS_E_ARG, "scale a must be > 0");
    if (prec != VMPS_PREC_FP64 && prec != VMPS_PREC_BF16X3 && prec != VMPS_PREC_TF32X3)
        return set_err(VMPS_E_ARG, "unknown precision");
    if (p->pen.npen > 0 && nrhs > kPenMaxRhs)
        return set_err(VMPS_E_UNSUPPORTED, "a pivot with a projector takes at most 64 right-hand sides");
    require_device(p->ctx);
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = p->st();
    // BF16x3: one grouped launch pair for all right-hand sides; FP64 and 3xTF32: the
    // single-vector plan once per right-hand side
    DevPlan& dp = prec == VMPS_PREC_BF16X3 ? get_multi_plan(p, nrhs) : get_plan(p, prec);
    const int64_t dim = p->Vt.total, n = p->Vd.total;
    const size_t vbytes = (size_t)nrhs * n * 8;
    DBuf B[3], Wb, part, mud, ctl;
    for (DBuf& x : B) x.alloc(vbytes, st, true);
    Wb.alloc(vbytes, st, true);
    int64_t longest = 0;
    for (int j = 0; j < nparts; ++j) longest = std::max(longest, pbeg[j + 1] - pbeg[j]);
    const LzShape sh = lz_shape(longest, p->ctx->num_sms);
    part.alloc((size_t)nrhs * nparts * 2 * sh.nchunk * 8, st, false);
    mud.alloc((size_t)nrhs * nparts * nmom * 8, st, true);
    ctl.alloc(64, st, true);
    ensure_staging(p);
    for (int k = 0; k < nrhs; ++k)
        pack_in(p->ctx, p->dPack, p->npack, v0 + (int64_t)k * dim, dim, p->stage_in, B[0].as<double>() + (int64_t)k * n,
                st);
    cudaGraphExec_t g[3] = {nullptr, nullptr, nullptr};
    struct Guard {
        cudaGraphExec_t* g;
        ~Guard() { for (int i = 0; i < 3; ++i) if (g[i]) cudaGraphExecDestroy(g[i]); }
    } guard{g};
    for (int r = 0; r < 3; ++r) {
        ChebArgs c{};
        c.w = Wb.as<double>();
        c.tn = B[r].as<double>();
        c.tprev = B[(r + 2) % 3].as<double>();
        c.tnext = B[(r + 1) % 3].as<double>();
        c.part = part.as<double>();
        c.mu = mud.as<double>();
        c.ctl = ctl.as<unsigned>();
        c.n = n;
        c.vs = n;
        c.nrhs = nrhs;
        c.nmom = nmom;
        c.nchunk = sh.nchunk;
        c.inv_a = 1.0 / a;
        c.b = b;
        c.nparts = nparts;
        for (int j = 0; j <= nparts; ++j) c.pbeg[j] = pbeg[j];
        Operands ops = pivot_ops(p);
        cudaGraph_t gr = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            if (prec == VMPS_PREC_BF16X3) {
                ops.Y = c.tn;
                ops.O = Wb.as<double>();
                run_plan(dp, ops, st);
            } else {
                for (int k = 0; k < nrhs; ++k) {
                    ops.Y = c.tn + (int64_t)k * n;
                    ops.O = Wb.as<double>() + (int64_t)k * n;
                    run_plan(dp, ops, st);
                }
            }
            CK(launch_cheb_step(c, sh.per_thread, st));
        } catch (...) {
            if (cudaStreamEndCapture(st, &gr) == cudaSuccess && gr) cudaGraphDestroy(gr);
            throw;
        }
        CK(cudaStreamEndCapture(st, &gr));
        const cudaError_t ie = cudaGraphInstantiate(&g[r], gr, 0);
        cudaGraphDestroy(gr);
        CK(ie);
    }
    const int steps = (nmom + 1) / 2;
    CK(cudaEventRecord(p->ctx->ev0, st));
    for (int i = 0; i < steps; ++i) CK(cudaGraphLaunch(g[i % 3], st));
    CK(cudaEventRecord(p->ctx->ev1, st));
    CK(cudaMemcpyAsync(mu, mud.p, (size_t)nrhs * nparts * nmom * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    check_device_error(p->ctx);
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, p->ctx->ev0, p->ctx->ev1));
    if (stats) {
        stats->steps = steps;
        stats->hxv = steps * nrhs;
        stats->ms_device = ms;
        stats->ms_per_step = ms / steps;
        stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    API_END
}

extern "C" int vmps_chebyshev_moments(vmps_pivot* p, const double* v0, int nrhs, int nmom, double a, double b,
                                      int prec, double* mu, vmps_cheb_stats* stats) {
    return chebyshev_moments(p, v0, nrhs, nmom, a, b, prec, 1, nullptr, mu, stats);
}

extern "C" int vmps_chebyshev_moments_parts(vmps_pivot* p, const double* v0, int nrhs, int nmom, double a, double b,
                                            int prec, int nparts, const int64_t* part_blocks, double* mu,
                                            vmps_cheb_stats* stats) {
    return chebyshev_moments(p, v0, nrhs, nmom, a, b, prec, nparts, part_blocks, mu, stats);
}

// contract_AA2 (tensors/DmrgContractions.h:1870-1927, abelian): the two-site
// tensor V[k] = sum A1[i] * A2[j] over the (k, i, j) products, as one FP64
// grouped-GEMM launch on padded device copies of the three block tables
// V[k] = sum of A1[i] A2[j] over the (k, i, j) products, one FP64 grouped GEMM
static void two_site_contract(vmps_ctx* ctx, const BlockTable& t1, const double* a1, const BlockTable& t2,
                              const double* a2, const BlockTable& tv, double* v,
                              const std::vector<std::array<int64_t, 3>>& pr, const double* coef = nullptr) {
    const DevLayout d1 = make_dev_layout(t1.rows, t1.cols), d2 = make_dev_layout(t2.rows, t2.cols),
                    dv = make_dev_layout(tv.rows, tv.cols);
    for (const auto& t : pr)
        if (t[0] < 0 || t[0] >= tv.n || t[1] < 0 || t[1] >= t1.n || t[2] < 0 || t[2] >= t2.n)
            throw std::invalid_argument("product index outside its block table");
    PhasePlan ph = make_product_plan(d1, d2, dv, pr, coef);
    cudaStream_t st = ctx->stream;
    // device buffers kept in the context between calls (a sweep makes one call per bond)
    if (!ctx->two_site) ctx->two_site.reset(new TwoSiteScratch());
    TwoSiteScratch& S = *ctx->two_site;
    DBuf &g1 = S.a1, &g2 = S.a2, &gv = S.v, &stage = S.stage;
    upload_blocks_padded(ctx, t1, d1, a1, g1, st);
    upload_blocks_padded(ctx, t2, d2, a2, g2, st);
    gv.alloc((size_t)std::max<int64_t>(dv.total, 1) * 8, st, true);
    DevPhase& dph = S.phase;
    dph.upload(ph, st);
    GGArgs g{};
    g.A = g1.p;
    g.B = g2.p;
    g.C = gv.p;
    g.err = ctx->err;
    g.tiles = dph.tiles.as<GTile>();
    g.segs = dph.segs.as<GSeg>();
    g.terms = dph.terms.as<GTerm>();
    g.ntiles = dph.ntiles;
    CK(launch_gg64(g, st));
    if (tv.n > 0) {
        const auto pb = pack_blocks(tv, dv, nullptr);
        upload_vec(S.pack, pb, st);
        pack_out(ctx, S.pack, (int)pb.size(), gv.as<double>(), tv.total, stage, v, st);
    }
    CK(cudaStreamSynchronize(st));
    dph.host = nullptr;
    check_device_error(ctx);
}

extern "C" int vmps_two_site_contract(vmps_ctx* ctx, const vmps_symmetry* symd, const vmps_blocks* A1,
                                      const double* a1, const vmps_blocks* A2, const double* a2,
                                      const vmps_blocks* V, double* v, int64_t nprod, const int64_t* prods) {
    API_BEGIN
    if (!ctx || !a1 || !a2 || !v || nprod < 0 || (nprod > 0 && !prods)) return set_err(VMPS_E_ARG, "bad argument");
    require_device(ctx);
    const Symmetry sym = make_sym(symd);
    const BlockTable t1 = parse_blocks(sym, A1, false), t2 = parse_blocks(sym, A2, false),
                     tv = parse_blocks(sym, V, false);
    std::vector<std::array<int64_t, 3>> pr((size_t)nprod);
    for (int64_t q = 0; q < nprod; ++q) pr[q] = {prods[3 * q], prods[3 * q + 1], prods[3 * q + 2]};
    two_site_contract(ctx, t1, a1, t2, a2, tv, v, pr);
    API_END
}

// C[k] = sum over the products q = (k, i, j) of coef[q] * A[i] * B[j] (coef NULL: 1),
// one FP64 grouped-GEMM launch; C blocks without a product come back zero
// 6j symbols for host-side SU(2) recoupling, arguments as multiplet dimensions q = 2j + 1
extern "C" int vmps_su2_coupling_6j(int64_t n, const int32_t* q, double* out) {
    API_BEGIN
    if (n < 0 || (n > 0 && (!q || !out))) return set_err(VMPS_E_ARG, "bad argument");
    for (int64_t i = 0; i < n; ++i) {
        const int32_t* a = q + 6 * i;
        for (int j = 0; j < 6; ++j)
            if (a[j] < 1) return set_err(VMPS_E_ARG, "multiplet dimensions must be >= 1");
        out[i] = coupling_6j(a[0] - 1, a[1] - 1, a[2] - 1, a[3] - 1, a[4] - 1, a[5] - 1);
    }
    API_END
}

extern "C" int vmps_block_products(vmps_ctx* ctx, const vmps_symmetry* symd, const vmps_blocks* A, const double* a,
                                   const vmps_blocks* B, const double* b, const vmps_blocks* Ct, double* c,
                                   int64_t nprod, const int64_t* prods, const double* coef) {
    API_BEGIN
    if (!ctx || !a || !b || !c || nprod < 0 || (nprod > 0 && !prods)) return set_err(VMPS_E_ARG, "bad argument");
    require_device(ctx);
    const Symmetry sym = make_sym(symd);
    const BlockTable t1 = parse_blocks(sym, A, false), t2 = parse_blocks(sym, B, false),
                     tc = parse_blocks(sym, Ct, false);
    std::vector<std::array<int64_t, 3>> pr((size_t)nprod);
    for (int64_t q = 0; q < nprod; ++q) {
        pr[q] = {prods[3 * q], prods[3 * q + 1], prods[3 * q + 2]};
        if (coef && !std::isfinite(coef[q])) return set_err(VMPS_E_NONFINITE, "product coefficient is not finite");
    }
    two_site_contract(ctx, t1, a, t2, b, tc, c, pr, coef);
    API_END
}

extern "C" int vmps_two_site_contract_pairs(vmps_ctx* ctx, const vmps_symmetry* symd, const vmps_blocks* A1,
                                            const double* a1, const vmps_blocks* A2, const double* a2,
                                            const vmps_blocks* V, double* v, int n1, int n3,
                                            const int32_t* s13_of_pair) {
    API_BEGIN
    if (!ctx || !a1 || !a2 || !v || n1 < 1 || n3 < 1 || !s13_of_pair) return set_err(VMPS_E_ARG, "bad argument");
    require_device(ctx);
    const Symmetry sym = make_sym(symd);
    if (sym.nonabelian()) return set_err(VMPS_E_ARG, "the pair form needs abelian quantum numbers");
    const BlockTable t1 = parse_blocks(sym, A1, false), t2 = parse_blocks(sym, A2, false),
                     tv = parse_blocks(sym, V, false);
    // V blocks by (s13, qin, qout); A2 blocks by (s3, qin) in table order
    std::unordered_map<QN3, int64_t, QNTupleHash<3>> vfind;
    for (int64_t k = 0; k < tv.n; ++k) {
        QN leg{};
        leg.v[0] = tv.leg[k];
        vfind.emplace(QN3{{leg, tv.qin[k], tv.qout[k]}}, k);
    }
    std::unordered_map<QN2, std::vector<int64_t>, QNTupleHash<2>> a2by;
    for (int64_t j = 0; j < t2.n; ++j) {
        if (t2.leg[j] >= n3) throw std::invalid_argument("A2 block leg outside the local basis");
        QN leg{};
        leg.v[0] = t2.leg[j];
        a2by[QN2{{leg, t2.qin[j]}}].push_back(j);
    }
    std::vector<std::array<int64_t, 3>> pr;
    for (int64_t i = 0; i < t1.n; ++i) {
        const int s1 = t1.leg[i];
        if (s1 >= n1) throw std::invalid_argument("A1 block leg outside the local basis");
        for (int s3 = 0; s3 < n3; ++s3) {
            QN leg{};
            leg.v[0] = s3;
            auto it = a2by.find(QN2{{leg, t1.qout[i]}});
            if (it == a2by.end()) continue;
            QN l13{};
            l13.v[0] = s13_of_pair[s1 * n3 + s3];
            for (int64_t j : it->second) {
                auto kv = vfind.find(QN3{{l13, t1.qin[i], t2.qout[j]}});
                if (kv != vfind.end()) pr.push_back({kv->second, i, j});
            }
        }
    }
    two_site_contract(ctx, t1, a1, t2, a2, tv, v, pr);
    API_END
}

// ---------------------------------------------------------------------------
// environment updates
// ---------------------------------------------------------------------------
struct vmps_env_s {
    vmps_ctx* ctx = nullptr;
    Symmetry sym;
    int side = 0;
    BlockTable Et, Bt, Kt, Nt;   // old env, bra, ket, new env
    DevLayout Ed, Bd, Kd, Nd;
    ChainSet cs;
    DevPlan plans[2];
    DBuf dE, dB, dK, dN, stage, pkN;
    int npkN = 0;
    cudaStream_t st() const { return ctx->stream; }
};

static DevPlan& env_plan(vmps_env* e, int prec) {
    if (prec == VMPS_PREC_TF32X3) throw std::invalid_argument("3xTF32 runs pivot HxVs only");
    if (prec != VMPS_PREC_FP64 && prec != VMPS_PREC_BF16X3) throw std::invalid_argument("unknown precision");
    DevPlan& dp = e->plans[prec];
    if (dp.ready) return dp;
    const bool L = e->side == VMPS_ENV_LEFT;
    // left: X = Abra^dagger, Y = Eold, Z = Aket;  right: X = Aket, Y = Eold, Z = Abra^dagger
    const DevLayout& X = L ? e->Bd : e->Kd;
    const DevLayout& Z = L ? e->Kd : e->Bd;
    if (prec == VMPS_PREC_FP64) dp.plan = make_plan(e->cs, X, e->Ed, Z, e->Nd, L, !L, 64, 64);
    else {
        dp.plan = make_split_plan(e->cs, X, e->Ed, Z, e->Nd, L, !L);
        schedule_and_validate(dp.plan, e->ctx->num_sms);
    }
    if (e->ctx->device < 0) { dp.ready = true; return dp; }
    plan_to_device(dp, e->Ed, e->st());
    CK(cudaStreamSynchronize(e->st()));
    dp.ready = true;
    return dp;
}

extern "C" {

int vmps_env_create(vmps_ctx* ctx, const vmps_symmetry* symd, int side, const vmps_blocks* Eold,
                    const vmps_blocks* Abra, const vmps_mpo_site* W, const vmps_blocks* Aket, vmps_env** out) {
    return vmps_env_create_mode(ctx, symd, side, VMPS_ENV_FULL, 0, 0, nullptr, nullptr, nullptr, Eold, Abra, W, Aket,
                                out);
}

int vmps_env_create_mode(vmps_ctx* ctx, const vmps_symmetry* symd, int side, int mode, int64_t fixed_ab,
                         int64_t n_order, const int32_t* order_qn, const int32_t* order_index,
                         const int64_t* order_value, const vmps_blocks* Eold, const vmps_blocks* Abra,
                         const vmps_mpo_site* W, const vmps_blocks* Aket, vmps_env** out) {
    API_BEGIN
    if (!ctx || !out) return set_err(VMPS_E_ARG, "null argument");
    if (side != VMPS_ENV_LEFT && side != VMPS_ENV_RIGHT) return set_err(VMPS_E_ARG, "side must be LEFT or RIGHT");
    if (mode < VMPS_ENV_FULL || mode > VMPS_ENV_FIXED_COLS) return set_err(VMPS_E_ARG, "unknown contraction mode");
    Symmetry sym = make_sym(symd);
    EnvMode md;
    md.mode = mode;
    md.fixed_ab = fixed_ab;
    if (mode != VMPS_ENV_FULL) {
        if (n_order <= 0 || !order_qn || !order_index || !order_value)
            return set_err(VMPS_E_ARG, "modes other than FULL need the basis order map");
        for (int64_t i = 0; i < n_order; ++i) {
            QN q;
            for (int c = 0; c < sym.nq; ++c) q.v[c] = order_qn[i * sym.nq + c];
            md.order[AuxKey{q, order_index[i]}] = order_value[i];
        }
    }
    std::unique_ptr<vmps_env> e(new vmps_env_s());
    e->ctx = ctx;
    e->sym = sym;
    e->side = side;
    e->Et = parse_blocks(sym, Eold, true);
    e->Bt = parse_blocks(sym, Abra, false);
    e->Kt = parse_blocks(sym, Aket, false);
    MpoView Wv = parse_mpo(sym, W);
    e->cs = build_env(sym, side, e->Et, e->Bt, Wv, e->Kt, &e->Nt, md);
    e->Ed = make_dev_layout(e->Et.rows, e->Et.cols);
    e->Bd = make_dev_layout(e->Bt.rows, e->Bt.cols);
    e->Kd = make_dev_layout(e->Kt.rows, e->Kt.cols);
    e->Nd = make_dev_layout(e->Nt.rows, e->Nt.cols);
    *out = e.release();
    API_END
}

int vmps_env_layout(const vmps_env* e, int64_t* nblocks, int64_t* total) {
    if (!e || !nblocks || !total) return set_err(VMPS_E_ARG, "null argument");
    *nblocks = e->Nt.n;
    *total = e->Nt.total;
    return VMPS_OK;
}

int vmps_env_layout_get(const vmps_env* e, int32_t* qin, int32_t* qout, int32_t* qmid, int32_t* leg, int64_t* rows,
                        int64_t* cols, int64_t* offset) {
    if (!e) return set_err(VMPS_E_ARG, "null argument");
    const int nq = e->sym.nq;
    for (int64_t i = 0; i < e->Nt.n; ++i) {
        for (int c = 0; c < nq; ++c) {
            if (qin) qin[i * nq + c] = e->Nt.qin[i].v[c];
            if (qout) qout[i * nq + c] = e->Nt.qout[i].v[c];
            if (qmid) qmid[i * nq + c] = e->Nt.qmid[i].v[c];
        }
        if (leg) leg[i] = e->Nt.leg[i];
        if (rows) rows[i] = e->Nt.rows[i];
        if (cols) cols[i] = e->Nt.cols[i];
        if (offset) offset[i] = e->Nt.off[i];
    }
    return VMPS_OK;
}

int vmps_env_stats(const vmps_env* ec, int prec, vmps_plan_stats* out) {
    API_BEGIN
    if (!ec || !out) return set_err(VMPS_E_ARG, "null argument");
    auto* e = const_cast<vmps_env*>(ec);
    DevPlan& dp = env_plan(e, prec);
    fill_stats(e->cs, dp.plan, prec, out);
    API_END
}

int vmps_env_run(vmps_env* e, const double* Eold, const double* Abra, const double* Aket, double* Enew, int prec) {
    API_BEGIN
    if (!e || !Eold || !Abra || !Aket || !Enew) return set_err(VMPS_E_ARG, "null argument");
    require_device(e->ctx);
    CK(cudaSetDevice(e->ctx->device));
    cudaStream_t st = e->st();
    DevPlan& dp = env_plan(e, prec);
    upload_blocks_padded(e->ctx, e->Et, e->Ed, Eold, e->dE, st);
    upload_blocks_padded(e->ctx, e->Bt, e->Bd, Abra, e->dB, st);
    upload_blocks_padded(e->ctx, e->Kt, e->Kd, Aket, e->dK, st);
    e->dN.alloc((size_t)e->Nd.total * 8, st, true);
    Operands ops;
    if (e->side == VMPS_ENV_LEFT) { ops.X = e->dB.as<double>(); ops.Z = e->dK.as<double>(); }
    else { ops.X = e->dK.as<double>(); ops.Z = e->dB.as<double>(); }
    ops.Y = e->dE.as<double>();
    ops.O = e->dN.as<double>();
    ops.err = e->ctx->err;
    split_prepare(dp, ops.X, ops.Z, st);
    run_plan(dp, ops, st);
    if (!e->pkN.p) {
        auto pb = pack_blocks(e->Nt, e->Nd, nullptr);
        e->npkN = (int)pb.size();
        upload_vec(e->pkN, pb, st);
    }
    pack_out(e->ctx, e->pkN, e->npkN, e->dN.as<double>(), e->Nt.total, e->stage, Enew, st);
    CK(cudaStreamSynchronize(st));
    check_device_error(e->ctx);
    API_END
}

int vmps_env_destroy(vmps_env* e) {
    delete e;
    return VMPS_OK;
}

// ---------------------------------------------------------------------------
// VUMPS MpoTransferMatrix (VUMPS/VumpsMpoTransferMatrix.h:99-212)
// ---------------------------------------------------------------------------
}  // extern "C"

// a vmps_blocks view of a block table (the table owns the storage it points into)
struct BlocksView {
    std::vector<int32_t> qin, qout, qmid, leg;
    std::vector<int64_t> rows, cols, off;
    vmps_blocks b{};
    BlocksView(const BlockTable& t, int nq) {
        for (int64_t i = 0; i < t.n; ++i)
            for (int c = 0; c < nq; ++c) {
                qin.push_back(t.qin[i].v[c]);
                qout.push_back(t.qout[i].v[c]);
                qmid.push_back(t.has_mid ? t.qmid[i].v[c] : 0);
            }
        leg.assign(t.leg.begin(), t.leg.end());
        rows = t.rows; cols = t.cols; off = t.off;
        b.nblocks = t.n;
        b.qin = qin.data(); b.qout = qout.data(); b.qmid = qmid.data(); b.leg = leg.data();
        b.rows = rows.data(); b.cols = cols.data(); b.offset = off.data();
    }
};

struct vmps_transfer_s {
    vmps_ctx* ctx = nullptr;
    Symmetry sym;
    std::vector<vmps_env*> chain;   // owned; chain[k+1] reads the output of chain[k]
    BlockTable Vt;                  // transfer vector layout
    DevLayout Vd;
    BlockTable LRt;
    DevLayout LRd;
    DBuf dLR, dVout, stage_in, stage_out, pk, dTrace, dCombine, part, scal;
    int npk = 0, ntrace = 0, ncombine = 0;
    std::vector<char> prepped[2];
    QN abq;                         // (QN, index) of the slot ab
    int32_t abi = -1;
    // device GMRES: Krylov basis (dimK + 1 vectors of the padded layout), work vectors,
    // the slot mask and the masked dot weights, reduction scratch
    DBuf gQ, gw, gr, gx, gb, gt, gd, gwm, gm, gpart, gh;
    int gdim = -1;
    ~vmps_transfer_s() {
        for (vmps_env* e : chain) delete e;
    }
    cudaStream_t st() const { return ctx->stream; }
};

// T's operator (VumpsMpoTransferMatrix.h:99-212) on padded device vectors: the cell's
// contract_L/R chain from din, then Vout = Vin - T Vin + LdotR * 1 on the slot-ab blocks
static void transfer_apply(vmps_transfer* t, const double* din, double* dout, int prec) {
    cudaStream_t st = t->st();
    vmps_env* first = t->chain.front();
    if (din != first->dE.as<double>() && first->Ed.total > 0)
        CK(cudaMemcpyAsync(first->dE.p, din, (size_t)first->Ed.total * 8, cudaMemcpyDeviceToDevice, st));
    for (size_t k = 0; k < t->chain.size(); ++k) {
        vmps_env* e = t->chain[k];
        DevPlan& dp = env_plan(e, prec);
        Operands ops;
        if (e->side == VMPS_ENV_LEFT) { ops.X = e->dB.as<double>(); ops.Z = e->dK.as<double>(); }
        else { ops.X = e->dK.as<double>(); ops.Z = e->dB.as<double>(); }
        ops.Y = e->dE.as<double>();
        ops.O = e->dN.as<double>();
        ops.err = t->ctx->err;
        if (!t->prepped[prec][k]) {   // the site tensors are fixed: their split panels are made once
            split_prepare(dp, ops.X, ops.Z, st);
            t->prepped[prec][k] = 1;
        }
        run_plan(dp, ops, st);
        if (k + 1 < t->chain.size() && e->Nd.total > 0)
            CK(cudaMemcpyAsync(t->chain[k + 1]->dE.p, e->dN.p, (size_t)e->Nd.total * 8, cudaMemcpyDeviceToDevice, st));
    }
    CK(launch_trace_pairs(t->dTrace.as<TracePair>(), t->ntrace, first->dE.as<double>(), t->dLR.as<double>(),
                          t->part.as<double>(), t->scal.as<double>(), st));
    CK(cudaMemsetAsync(dout, 0, (size_t)std::max<int64_t>(t->Vd.total, 1) * 8, st));
    CK(launch_transfer_combine(t->dCombine.as<CombineBlock>(), t->ncombine, first->dE.as<double>(),
                               t->chain.back()->dN.as<double>(), dout, t->scal.as<double>(), st));
}

// ---- device GMRES of the transfer operator --------------------------------------
struct GmresNonFinite : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// buffers for a Krylov dimension dimK; the slot mask and its dot weights (coeff_dot(out),
// VumpsMpoTransferMatrix.h:258-275) in the padded layout, padding zero
static void transfer_gmres_setup(vmps_transfer* t, int dimK) {
    cudaStream_t st = t->st();
    const int64_t n = std::max<int64_t>(t->Vd.total, 1);
    if (t->gdim < 0) {
        std::vector<double> wm((size_t)n, 0.0), m((size_t)n, 0.0);
        for (int64_t b = 0; b < t->Vt.n; ++b) {
            if (!(t->Vt.qmid[b] == t->abq) || t->Vt.leg[b] != t->abi) continue;
            const double w = t->sym.coeff_dot(t->Vt.qout[b]);
            for (int64_t c = 0; c < t->Vt.cols[b]; ++c)
                for (int64_t r = 0; r < t->Vt.rows[b]; ++r) {
                    const int64_t e = t->Vd.off[b] + c * t->Vd.ld[b] + r;
                    wm[(size_t)e] = w;
                    m[(size_t)e] = 1.0;
                }
        }
        upload_vec(t->gwm, wm, st);
        upload_vec(t->gm, m, st);
        for (DBuf* d : {&t->gw, &t->gr, &t->gx, &t->gb, &t->gt, &t->gd}) d->alloc((size_t)n * 8, st, true);
        t->gdim = 0;
    }
    if (t->gdim < dimK) {
        t->gQ.alloc((size_t)(dimK + 1) * (size_t)n * 8, st, true);
        t->gpart.alloc((size_t)(dimK + 1) * (size_t)std::max(dot_nchunk(n), 1) * 8, st, true);
        t->gh.alloc((size_t)(3 * (dimK + 1) + 8) * 8, st, true);
        t->gdim = dimK;
    }
}

// <x, y> on the slot-ab blocks with the coeff_dot weights (device reduction, value to the host)
static double transfer_wdot(vmps_transfer* t, const double* x, const double* y) {
    cudaStream_t st = t->st();
    const int64_t n = t->Vd.total;
    double* r = t->gr.as<double>();
    double* h = t->gh.as<double>();
    CK(launch_hadamard(t->gwm.as<double>(), y, r, n, st));
    CK(launch_dot(x, r, n, t->gpart.as<double>(), h, st));
    double v = 0;
    CK(cudaMemcpyAsync(&v, h, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return v;
}

// r = mask * (b - A x) with the FP64 operator (r = mask * b when x is zero)
static void transfer_residual(vmps_transfer* t, const double* b, const double* x, double* r, bool x_zero) {
    cudaStream_t st = t->st();
    const int64_t n = t->Vd.total;
    CK(cudaMemcpyAsync(r, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    if (!x_zero) {
        double* ax = t->dVout.as<double>();
        transfer_apply(t, x, ax, VMPS_PREC_FP64);
        CK(launch_axpy(-1.0, ax, r, n, st));
    }
    CK(launch_hadamard(t->gm.as<double>(), r, r, n, st));
}

// Restarted GMRES for A d = rhs (rhs masked), then x += d: cycles of at most dimK
// iterations until |rhs - A d| <= abs_tol or max_restarts cycles; returns the iterations.
// Arnoldi with two classical Gram-Schmidt passes under the weighted dot; the Hessenberg
// matrix and its Givens rotations on the host, one column read back per iteration.
static int transfer_gmres(vmps_transfer* t, const double* rhs, double* x, double abs_tol, int dimK,
                          int max_restarts, int prec, int32_t* restarts) {
    cudaStream_t st = t->st();
    const int64_t n = t->Vd.total;
    double* Q = t->gQ.as<double>();
    double* w = t->gw.as<double>();
    double* r = t->gr.as<double>();
    double* d = t->gd.as<double>();                  // this call's solution
    double* ax = t->dVout.as<double>();
    const double* m = t->gm.as<double>();
    const double* wm = t->gwm.as<double>();
    const int ld = dimK + 1;
    double* hd = t->gh.as<double>();                 // [h pass 1 (ld) | h pass 2 (ld) | norm (8) | y (ld)]
    double* h2d = hd + ld;
    double* nrm = hd + 2 * ld;
    double* yd = nrm + 8;
    std::vector<double> H((size_t)ld * dimK, 0.0), cs((size_t)dimK), sn((size_t)dimK), g((size_t)ld);
    std::vector<double> col((size_t)(2 * ld + 1));
    CK(cudaMemsetAsync(d, 0, (size_t)n * 8, st));
    int its = 0;
    for (int cycle = 0; cycle < max_restarts; ++cycle) {
        // w = mask * (rhs - A d)
        CK(cudaMemcpyAsync(w, rhs, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
        if (cycle > 0) {
            transfer_apply(t, d, ax, prec);
            CK(launch_axpy(-1.0, ax, w, n, st));
            CK(launch_hadamard(m, w, w, n, st));
        }
        const double beta = std::sqrt(std::max(0.0, transfer_wdot(t, w, w)));
        if (!std::isfinite(beta)) throw GmresNonFinite("GMRES: non-finite residual");
        if (beta <= abs_tol) break;
        if (cycle > 0 && restarts) ++*restarts;
        CK(cudaMemcpyAsync(Q, w, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
        CK(launch_scale(1.0 / beta, Q, n, st));
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int kk = 0;
        for (int k = 0; k < dimK; ++k) {
            transfer_apply(t, Q + (int64_t)k * n, ax, prec);
            ++its;
            CK(launch_hadamard(m, ax, w, n, st));
            for (int pass = 0; pass < 2; ++pass) {
                CK(launch_hadamard(wm, w, r, n, st));
                CK(launch_mdot(Q, k + 1, n, r, t->gpart.as<double>(), pass ? h2d : hd, st));
                CK(launch_mgs(Q, k + 1, n, pass ? h2d : hd, w, st));
            }
            CK(launch_hadamard(wm, w, r, n, st));
            CK(launch_dot(w, r, n, t->gpart.as<double>(), nrm, st));
            CK(cudaMemcpyAsync(col.data(), hd, sizeof(double) * (size_t)(k + 1), cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(col.data() + ld, h2d, sizeof(double) * (size_t)(k + 1), cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(col.data() + 2 * ld, nrm, sizeof(double), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            double* hk = H.data() + (size_t)k * ld;
            for (int j = 0; j <= k; ++j) hk[j] = col[(size_t)j] + col[(size_t)(ld + j)];
            const double hn = std::sqrt(std::max(0.0, col[(size_t)(2 * ld)]));
            hk[k + 1] = hn;
            for (int j = 0; j <= k + 1; ++j)
                if (!std::isfinite(hk[j])) throw GmresNonFinite("GMRES: the operator produced non-finite values");
            // the earlier rotations, then the one that zeroes hk[k+1]
            for (int j = 0; j < k; ++j) {
                const double a = cs[(size_t)j] * hk[j] + sn[(size_t)j] * hk[j + 1];
                hk[j + 1] = -sn[(size_t)j] * hk[j] + cs[(size_t)j] * hk[j + 1];
                hk[j] = a;
            }
            const double den = std::hypot(hk[k], hk[k + 1]);
            cs[(size_t)k] = den > 0 ? hk[k] / den : 1.0;
            sn[(size_t)k] = den > 0 ? hk[k + 1] / den : 0.0;
            hk[k] = den;
            hk[k + 1] = 0.0;
            g[(size_t)k + 1] = -sn[(size_t)k] * g[(size_t)k];
            g[(size_t)k] = cs[(size_t)k] * g[(size_t)k];
            kk = k + 1;
            if (hn <= 1e-14 * beta || std::abs(g[(size_t)k + 1]) <= abs_tol || k + 1 == dimK) break;
            CK(cudaMemcpyAsync(Q + (int64_t)(k + 1) * n, w, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
            CK(launch_scale(1.0 / hn, Q + (int64_t)(k + 1) * n, n, st));
        }
        // y = R^-1 g (upper triangular, kk x kk), d += Q y
        std::vector<double> y((size_t)kk, 0.0);
        for (int i = kk - 1; i >= 0; --i) {
            double sum = g[(size_t)i];
            for (int j = i + 1; j < kk; ++j) sum -= H[(size_t)j * ld + i] * y[(size_t)j];
            const double rii = H[(size_t)i * ld + i];
            y[(size_t)i] = rii != 0 ? sum / rii : 0.0;
        }
        CK(cudaMemcpyAsync(yd, y.data(), sizeof(double) * (size_t)kk, cudaMemcpyHostToDevice, st));
        CK(launch_combine(Q, kk, n, yd, ax, st));
        CK(launch_axpy(1.0, ax, d, n, st));
        CK(cudaStreamSynchronize(st));   // y is a host vector: keep it until its copy has run
    }
    CK(launch_axpy(1.0, d, x, n, st));
    return its;
}

static std::vector<int32_t> block_key(const BlockTable& t, int64_t i, int nq, bool with_leg) {
    std::vector<int32_t> k;
    for (int c = 0; c < nq; ++c) k.push_back(t.qin[i].v[c]);
    for (int c = 0; c < nq; ++c) k.push_back(t.qout[i].v[c]);
    if (t.has_mid)
        for (int c = 0; c < nq; ++c) k.push_back(t.qmid[i].v[c]);
    if (with_leg) k.push_back(t.leg[i]);
    return k;
}

extern "C" {

int vmps_transfer_create(vmps_ctx* ctx, const vmps_symmetry* symd, int dir, int ncell, const vmps_blocks* const* Abra,
                         const double* const* Abra_data, const vmps_blocks* const* Aket,
                         const double* const* Aket_data, const vmps_mpo_site* const* W, const vmps_blocks* LReigen,
                         const double* LReigen_data, int64_t ab, int64_t n_order, const int32_t* order_qn,
                         const int32_t* order_index, const int64_t* order_value, const vmps_blocks* V,
                         vmps_transfer** out) {
    API_BEGIN
    if (!ctx || !symd || !out || !Abra || !Abra_data || !Aket || !Aket_data || !W || !LReigen || !LReigen_data || !V)
        return set_err(VMPS_E_ARG, "null argument");
    if (dir != VMPS_ENV_LEFT && dir != VMPS_ENV_RIGHT) return set_err(VMPS_E_ARG, "direction must be LEFT or RIGHT");
    if (ncell < 1) return set_err(VMPS_E_ARG, "the unit cell needs at least one site");
    if (n_order <= 0 || !order_qn || !order_index || !order_value)
        return set_err(VMPS_E_ARG, "the transfer operator needs the basis order map");
    require_device(ctx);
    Symmetry sym = make_sym(symd);
    const int nq = sym.nq;
    // (QN, index) of auxiliary position ab (basis_order[ab]); contract_LR requires the vacuum sector
    QN abq;
    int32_t abi = -1;
    for (int64_t i = 0; i < n_order; ++i)
        if (order_value[i] == ab) {
            for (int c = 0; c < nq; ++c) abq.v[c] = order_qn[i * nq + c];
            abi = order_index[i];
        }
    if (abi < 0) return set_err(VMPS_E_ARG, "ab is not a position of the basis order map");
    if (!(abq == sym.vacuum())) return set_err(VMPS_E_ARG, "contract_LR needs ab in the vacuum sector");
    std::unique_ptr<vmps_transfer> t(new vmps_transfer_s());
    t->ctx = ctx;
    t->sym = sym;
    t->abq = abq;
    t->abi = abi;
    t->Vt = parse_blocks(sym, V, true);
    t->Vd = make_dev_layout(t->Vt.rows, t->Vt.cols);
    t->LRt = parse_blocks(sym, LReigen, false);
    t->LRd = make_dev_layout(t->LRt.rows, t->LRt.cols);
    cudaStream_t st = ctx->stream;
    CK(cudaSetDevice(ctx->device));
    // the chain (VumpsMpoTransferMatrix.h:115-152): left: sites 0..n-1, FIXED_ROWS on the first and FIXED_COLS
    // on the last (the last rule wins for one site); right: sites n-1..0, FIXED_ROWS on site 0 and FIXED_COLS
    // on site n-1 (the site-0 rule wins for one site)
    std::unique_ptr<BlocksView> cur(new BlocksView(t->Vt, nq));
    for (int k = 0; k < ncell; ++k) {
        const int l = dir == VMPS_ENV_LEFT ? k : ncell - 1 - k;
        int mode = VMPS_ENV_FULL;
        if (dir == VMPS_ENV_LEFT) mode = l == ncell - 1 ? VMPS_ENV_FIXED_COLS : (l == 0 ? VMPS_ENV_FIXED_ROWS : VMPS_ENV_FULL);
        else mode = l == 0 ? VMPS_ENV_FIXED_ROWS : (l == ncell - 1 ? VMPS_ENV_FIXED_COLS : VMPS_ENV_FULL);
        vmps_env* e = nullptr;
        const int rc = vmps_env_create_mode(ctx, symd, dir, mode, ab, n_order, order_qn, order_index, order_value,
                                            &cur->b, Abra[l], W[l], Aket[l], &e);
        if (rc != VMPS_OK) return rc;
        t->chain.push_back(e);
        if (k > 0) {
            const vmps_env* p = t->chain[k - 1];
            if (p->Nd.total != e->Ed.total || p->Nd.rows != e->Ed.rows || p->Nd.cols != e->Ed.cols)
                throw std::logic_error("transfer chain: layouts of consecutive environments differ");
        }
        upload_blocks_padded(ctx, e->Bt, e->Bd, Abra_data[l], e->dB, st);
        upload_blocks_padded(ctx, e->Kt, e->Kd, Aket_data[l], e->dK, st);
        e->dE.alloc((size_t)std::max<int64_t>(e->Ed.total, 1) * 8, st, true);
        e->dN.alloc((size_t)std::max<int64_t>(e->Nd.total, 1) * 8, st, true);
        cur.reset(new BlocksView(e->Nt, nq));
    }
    t->prepped[0].assign(ncell, 0);
    t->prepped[1].assign(ncell, 0);
    upload_blocks_padded(ctx, t->LRt, t->LRd, LReigen_data, t->dLR, st);
    // contract_LR(ab, V, LReigen) (DmrgContractions.h:995-1053): vacuum-mid blocks of V at slot ab with
    // in == out, against the LReigen block (out, in); weight coeff_dot(out)
    std::map<std::vector<int32_t>, int64_t> lr_of;
    for (int64_t i = 0; i < t->LRt.n; ++i) lr_of[block_key(t->LRt, i, nq, false)] = i;
    std::vector<TracePair> tps;
    const QN vac = sym.vacuum();
    for (int64_t b = 0; b < t->Vt.n; ++b) {
        if (!(t->Vt.qmid[b] == vac) || t->Vt.leg[b] != abi || !(t->Vt.qin[b] == t->Vt.qout[b])) continue;
        std::vector<int32_t> key;
        for (int c = 0; c < nq; ++c) key.push_back(t->Vt.qout[b].v[c]);
        for (int c = 0; c < nq; ++c) key.push_back(t->Vt.qin[b].v[c]);
        auto it = lr_of.find(key);
        if (it == lr_of.end()) continue;
        const int64_t j = it->second;
        if (t->LRt.rows[j] != t->Vt.cols[b] || t->LRt.cols[j] != t->Vt.rows[b])
            return set_err(VMPS_E_SHAPE, "LReigen block does not match the transfer vector");
        tps.push_back(TracePair{t->Vd.off[b], t->LRd.off[j], (int32_t)t->Vt.rows[b], (int32_t)t->Vt.cols[b],
                                (int32_t)t->Vd.ld[b], (int32_t)t->LRd.ld[j], sym.coeff_dot(t->Vt.qout[b])});
    }
    // Vout = Vin - T Vin + LdotR * 1 on the slot-ab blocks the chain's output shares with Vin
    std::map<std::vector<int32_t>, int64_t> v_of;
    for (int64_t i = 0; i < t->Vt.n; ++i) v_of[block_key(t->Vt, i, nq, true)] = i;
    const vmps_env* last = t->chain.back();
    std::vector<CombineBlock> cbs;
    for (int64_t k = 0; k < last->Nt.n; ++k) {
        if (!(last->Nt.qmid[k] == abq) || last->Nt.leg[k] != abi) continue;
        auto it = v_of.find(block_key(last->Nt, k, nq, true));
        if (it == v_of.end()) continue;
        const int64_t b = it->second;
        if (t->Vt.rows[b] != last->Nt.rows[k] || t->Vt.cols[b] != last->Nt.cols[k])
            return set_err(VMPS_E_SHAPE, "transfer output block does not match the vector");
        cbs.push_back(CombineBlock{t->Vd.off[b], last->Nd.off[k], (int32_t)t->Vt.rows[b], (int32_t)t->Vt.cols[b],
                                   (int32_t)t->Vd.ld[b], (int32_t)last->Nd.ld[k]});
    }
    t->ntrace = (int)tps.size();
    t->ncombine = (int)cbs.size();
    upload_vec(t->dTrace, tps, st);
    upload_vec(t->dCombine, cbs, st);
    t->part.alloc((size_t)std::max(1, t->ntrace) * 8, st, true);
    t->scal.alloc(64, st, true);
    t->dVout.alloc((size_t)std::max<int64_t>(t->Vd.total, 1) * 8, st, true);
    auto pb = pack_blocks(t->Vt, t->Vd, nullptr);
    t->npk = (int)pb.size();
    upload_vec(t->pk, pb, st);
    CK(cudaStreamSynchronize(st));
    *out = t.release();
    API_END
}

int vmps_transfer_hxv(vmps_transfer* t, const double* vin, double* vout, int prec) {
    API_BEGIN
    if (!t || !vin || !vout) return set_err(VMPS_E_ARG, "null argument");
    if (prec == VMPS_PREC_TF32X3) return set_err(VMPS_E_UNSUPPORTED, "3xTF32 runs pivot HxVs only");
    if (prec != VMPS_PREC_FP64 && prec != VMPS_PREC_BF16X3) return set_err(VMPS_E_ARG, "unknown precision");
    CK(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->st();
    vmps_env* first = t->chain.front();
    pack_in(t->ctx, t->pk, t->npk, vin, t->Vt.total, t->stage_in, first->dE.as<double>(), st);
    transfer_apply(t, first->dE.as<double>(), t->dVout.as<double>(), prec);
    pack_out(t->ctx, t->pk, t->npk, t->dVout.as<double>(), t->Vt.total, t->stage_out, vout, st);
    CK(cudaStreamSynchronize(st));
    check_device_error(t->ctx);
    API_END
}

int vmps_transfer_solve(vmps_transfer* t, const double* b, double* x, double tol, int dimK, int max_restarts,
                        int prec, double inner_tol, int max_outer, vmps_gmres_stats* stats) {
    API_BEGIN
    if (!t || !b || !x) return set_err(VMPS_E_ARG, "null argument");
    if (prec != VMPS_PREC_FP64 && prec != VMPS_PREC_BF16X3) return set_err(VMPS_E_ARG, "FP64 or BF16X3");
    if (!(tol > 0) || dimK < 1 || dimK > 1000 || max_restarts < 1 || max_outer < 1 || !(inner_tol > 0))
        return set_err(VMPS_E_ARG, "GMRES needs tol > 0, 1 <= dimK <= 1000, max_restarts >= 1, max_outer >= 1");
    CK(cudaSetDevice(t->ctx->device));
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = t->st();
    transfer_gmres_setup(t, dimK);
    const int64_t n = t->Vd.total;
    double* db = t->gb.as<double>();
    double* dx = t->gx.as<double>();
    pack_in(t->ctx, t->pk, t->npk, b, t->Vt.total, t->stage_in, db, st);
    CK(launch_hadamard(t->gm.as<double>(), db, db, n, st));   // the slot-ab part of b
    CK(cudaMemsetAsync(dx, 0, (size_t)n * 8, st));
    vmps_gmres_stats S{};
    const double nb = std::sqrt(std::max(0.0, transfer_wdot(t, db, db)));
    if (!std::isfinite(nb)) return set_err(VMPS_E_NONFINITE, "GMRES: non-finite right-hand side");
    if (nb > 0) try {
        if (prec == VMPS_PREC_FP64) {
            S.iterations = transfer_gmres(t, db, dx, tol * nb, dimK, max_restarts, VMPS_PREC_FP64, &S.restarts);
            S.fp64_iterations = S.iterations;
        } else {
            // refinement: FP64 residuals, split-precision corrections.  When a round does not
            // halve the residual (the split operator's error times the condition number is no
            // longer small), a round that made it worse is undone and FP64 GMRES finishes
            double* dr = t->gt.as<double>();
            bool zero = true;
            double prev = std::numeric_limits<double>::infinity();
            for (int outer = 0; outer <= max_outer; ++outer) {
                transfer_residual(t, db, dx, dr, zero);
                if (!zero) ++S.fp64_hxv;
                double res = std::sqrt(std::max(0.0, transfer_wdot(t, dr, dr))) / nb;
                if (res <= tol) break;
                if (res > 0.5 * prev || outer == max_outer) {
                    if (res > prev) {   // the last correction (still in gd) made it worse
                        CK(launch_axpy(-1.0, t->gd.as<double>(), dx, t->Vd.total, st));
                        transfer_residual(t, db, dx, dr, false);
                        ++S.fp64_hxv;
                    }
                    const int its = transfer_gmres(t, dr, dx, tol * nb, dimK, max_restarts, VMPS_PREC_FP64,
                                                   &S.restarts);
                    S.iterations += its;
                    S.fp64_iterations += its;
                    break;
                }
                prev = res;
                // d solves A d = r; x += d (the correction is accumulated straight into x)
                S.iterations += transfer_gmres(t, dr, dx, inner_tol * res * nb, dimK, 2, VMPS_PREC_BF16X3,
                                               &S.restarts);
                S.outer = outer + 1;
                zero = false;
            }
        }
        double* dr = t->gt.as<double>();
        transfer_residual(t, db, dx, dr, false);
        ++S.fp64_hxv;
        S.residual = std::sqrt(std::max(0.0, transfer_wdot(t, dr, dr))) / nb;
    } catch (const GmresNonFinite& e) {
        CK(cudaStreamSynchronize(st));
        return set_err(VMPS_E_NONFINITE, e.what());
    }
    pack_out(t->ctx, t->pk, t->npk, dx, t->Vt.total, t->stage_out, x, st);
    CK(cudaStreamSynchronize(st));
    check_device_error(t->ctx);
    S.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = S;
    API_END
}

int vmps_transfer_destroy(vmps_transfer* t) {
    delete t;
    return VMPS_OK;
}

}  // extern "C"
