// Device task-list builder of the one- and two-site effective Hamiltonians
// (abelian symmetries): the matching of precalc_blockStructure for PivotMatrix1 and
// PivotMatrix2 (tensors/DmrgIndexGymnastics.h:487-590 with LAWA :32-77, and :699-856
// with its AAWWAA core :198-262) on the GPU.
//
// It produces exactly the chain list of the host builders build_pivot1 / build_pivot2
// (tasks.cpp), in the same order.  The two-site loop nest is
//     for (s1, s2, k12) with q(s2) + q(k12) = q(s1), for (s3, s4, k34) likewise,
//       for the combined indices s1s3 of (s1, s3) and s2s4 of (s2, s4),
//         for the L keys qL (in key order) with a two-site block (s1s3, Lin, Lin + q(s1s3)),
//           q24 = the block (s2s4, Lout, Lout + q(s2s4)); the MPO nonzeros of W12 between
//           Lmid and Lmid + q(k12), of W34 on to Rmid; the R key (qRin, qRout, Rmid);
//           for the W12 x W34 nonzero pairs joined on the inner auxiliary index:
//             chain {out q13, L block (qL, row12), in q24, R block (qR, col34), val12 * val34};
// the one-site nest is the same with one MPO site: for (s1, s2, k), for qL, the blocks
// (s1, Lin, Lin + q(s1)) and (s2, Lout, Lout + q(s2)), the nonzeros of W between Lmid
// and Lmid + q(k), the R key, a task when one nonzero has both its L and R blocks.
// The host enumerates the combinations of the local and operator indices (a few
// hundred); one device thread takes one (combination, qL) candidate, so the candidate
// index is the position in the host order.  A counting pass sums each thread block's
// chains, one thread scans the block sums, and the emitting pass repeats the matching,
// scans its block and writes every chain at its place.  The lookups (blocks of the
// vector, MPO nonzeros, R keys) are open-addressing hash tables built on the host with
// the same hash the kernels probe with; every probe sequence is bounded by its table
// size.  The tables travel in one upload into one device arena.
#include "engine.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace vmps {
namespace {

struct DQN { int32_t v[kMaxNq]; };
static_assert(sizeof(DQN) == sizeof(QN), "QN layout");

__host__ __device__ inline uint64_t mix(uint64_t h, uint64_t x) {
    h ^= x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    h ^= h >> 31;
    h *= 0x7fb5d329728ea185ull;
    h ^= h >> 27;
    return h;
}
__host__ __device__ inline uint64_t mix_qn(uint64_t h, const int32_t* v) {
    for (int i = 0; i < kMaxNq; ++i) h = mix(h, (uint32_t)v[i]);
    return h;
}
__host__ __device__ inline bool qeq(const DQN& a, const DQN& b) {
    for (int i = 0; i < kMaxNq; ++i)
        if (a.v[i] != b.v[i]) return false;
    return true;
}
__host__ __device__ inline DQN qsum(const DQN& a, const DQN& b) {
    DQN r;
    for (int i = 0; i < kMaxNq; ++i) r.v[i] = a.v[i] + b.v[i];
    return r;
}

// hash keys
__host__ __device__ inline uint64_t hash_v(int leg, const DQN& a, const DQN& b) {
    return mix_qn(mix_qn(mix(1, (uint32_t)leg), a.v), b.v);
}
__host__ __device__ inline uint64_t hash_r(const DQN& a, const DQN& b, const DQN& c) {
    return mix_qn(mix_qn(mix_qn(2, a.v), b.v), c.v);
}
__host__ __device__ inline uint64_t hash_w(int s1, int s2, int k, const DQN& a, const DQN& b) {
    return mix_qn(mix_qn(mix(mix(mix(3, (uint32_t)s1), (uint32_t)s2), (uint32_t)k), a.v), b.v);
}

// MPO nonzeros of one (s1, s2, k, qin, qout): [start, start + count) of the nonzero arrays
struct WKey { int32_t s1, s2, k, start, count, pad; DQN qin, qout; };
struct Tables {
    // two-site blocks: leg, qin, qout per block; hash slots -> block index
    const int32_t* v_leg; const DQN* v_qin; const DQN* v_qout; const int32_t* v_slot; uint32_t v_mask;
    // L keys: (Lin, Lout, Lmid), aux index -> L block
    const DQN* l_in; const DQN* l_out; const DQN* l_mid; const int32_t* l_aux_off; const int64_t* l_aux; int nkeys;
    // R keys and their hash slots -> key index, aux index -> R block
    const DQN* r_in; const DQN* r_out; const DQN* r_mid; const int32_t* r_slot; uint32_t r_mask;
    const int32_t* r_aux_off; const int64_t* r_aux;
    // MPO sites: keys, hash slots -> key index, nonzeros
    const WKey* w_key[2]; const int32_t* w_slot[2]; uint32_t w_mask[2];
    const int32_t* nz_row[2]; const int32_t* nz_col[2]; const double* nz_val[2];
    const DQN* qop[2]; const DQN* qloc[2];
    // combined basis (two-site): QN of every combined index
    const DQN* q_of; int ncomb;
};
// (s1, s2, k12, s3, s4, k34, s1s3, s2s4) of the host enumeration
struct Combo { int32_t s1, s2, k12, s3, s4, k34, s13, s24; };

__device__ inline int64_t find_v(const Tables& t, int leg, const DQN& a, const DQN& b) {
    const uint32_t n = t.v_mask + 1;
    uint32_t h = (uint32_t)hash_v(leg, a, b) & t.v_mask;
    for (uint32_t p = 0; p < n; ++p, h = (h + 1) & t.v_mask) {
        const int32_t i = t.v_slot[h];
        if (i < 0) return -1;
        if (t.v_leg[i] == leg && qeq(t.v_qin[i], a) && qeq(t.v_qout[i], b)) return i;
    }
    return -1;
}
__device__ inline int find_r(const Tables& t, const DQN& a, const DQN& b, const DQN& c) {
    const uint32_t n = t.r_mask + 1;
    uint32_t h = (uint32_t)hash_r(a, b, c) & t.r_mask;
    for (uint32_t p = 0; p < n; ++p, h = (h + 1) & t.r_mask) {
        const int32_t i = t.r_slot[h];
        if (i < 0) return -1;
        if (qeq(t.r_in[i], a) && qeq(t.r_out[i], b) && qeq(t.r_mid[i], c)) return i;
    }
    return -1;
}
__device__ inline const WKey* find_w(const Tables& t, int w, int s1, int s2, int k, const DQN& a, const DQN& b) {
    const uint32_t n = t.w_mask[w] + 1;
    uint32_t h = (uint32_t)hash_w(s1, s2, k, a, b) & t.w_mask[w];
    for (uint32_t p = 0; p < n; ++p, h = (h + 1) & t.w_mask[w]) {
        const int32_t i = t.w_slot[w][h];
        if (i < 0) return nullptr;
        const WKey& e = t.w_key[w][i];
        if (e.s1 == s1 && e.s2 == s2 && e.k == k && qeq(e.qin, a) && qeq(e.qout, b)) return &e;
    }
    return nullptr;
}
__device__ inline int64_t aux_at(const int32_t* off, const int64_t* aux, int key, int a) {
    const int32_t b = off[key], e = off[key + 1];
    return (a >= 0 && a < e - b) ? aux[b + a] : -1;
}

// in13[c][qL]: the two-site block (c, Lin, Lin + q(c)); at24[c][qL]: (c, Lout, Lout + q(c))
__global__ void match_blocks_kernel(Tables t, int64_t* in13, int64_t* at24) {
    const int64_t n = (int64_t)t.ncomb * t.nkeys;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i / t.nkeys), q = (int)(i % t.nkeys);
        in13[i] = find_v(t, c, t.l_in[q], qsum(t.l_in[q], t.q_of[c]));
        at24[i] = find_v(t, c, t.l_out[q], qsum(t.l_out[q], t.q_of[c]));
    }
}

constexpr int kBuildThreads = 256;

// one two-site candidate (combination, qL): its chains counted (EMIT false) or written from `at`
template <bool EMIT>
__device__ inline int candidate2(const Tables& t, const Combo* combos, const int64_t* in13, const int64_t* at24,
                                 int64_t idx, int64_t at, Chain* out, int* task) {
    const Combo cb = combos[idx / t.nkeys];
    const int qL = (int)(idx % t.nkeys);
    const int64_t q13 = in13[(int64_t)cb.s13 * t.nkeys + qL];
    if (q13 < 0) return 0;
    const int64_t q24 = at24[(int64_t)cb.s24 * t.nkeys + qL];
    if (q24 < 0) return 0;
    const DQN lmid = t.l_mid[qL];
    const DQN qw = qsum(lmid, t.qop[0][cb.k12]);
    const WKey* e12 = find_w(t, 0, cb.s1, cb.s2, cb.k12, lmid, qw);
    if (!e12) return 0;
    const DQN qrmid = qsum(qw, t.qop[1][cb.k34]);
    const WKey* e34 = find_w(t, 1, cb.s3, cb.s4, cb.k34, qw, qrmid);
    if (!e34) return 0;
    const DQN qrout = t.v_qout[q13], qrin = t.v_qout[q24];
    if (!qeq(qsum(qrin, qrmid), qrout)) return 0;   // abelian triangle(qRin, qRmid, qRout)
    const int qR = find_r(t, qrin, qrout, qrmid);
    if (qR < 0) return 0;
    *task = 1;
    int n = 0;
    for (int a = e12->start; a < e12->start + e12->count; ++a)
        for (int b = e34->start; b < e34->start + e34->count; ++b) {
            if (t.nz_col[0][a] != t.nz_row[1][b]) continue;
            const int64_t la = aux_at(t.l_aux_off, t.l_aux, qL, t.nz_row[0][a]);
            const int64_t rb = aux_at(t.r_aux_off, t.r_aux, qR, t.nz_col[1][b]);
            if (la < 0 || rb < 0) continue;
            if (EMIT) out[at + n] = Chain{q13, la, q24, rb, t.nz_val[0][a] * t.nz_val[1][b]};
            ++n;
        }
    return n;
}

// one one-site candidate ((s1, s2, k), qL)
template <bool EMIT>
__device__ inline int candidate1(const Tables& t, const Combo* combos, int64_t idx, int64_t at, Chain* out,
                                 int* task) {
    const Combo cb = combos[idx / t.nkeys];
    const int qL = (int)(idx % t.nkeys);
    const DQN lin = t.l_in[qL], lout = t.l_out[qL], lmid = t.l_mid[qL];
    const DQN rout = qsum(lin, t.qloc[0][cb.s1]);
    const int64_t qbra = find_v(t, cb.s1, lin, rout);
    if (qbra < 0) return 0;
    const DQN rin = qsum(lout, t.qloc[0][cb.s2]);
    const int64_t qket = find_v(t, cb.s2, lout, rin);
    if (qket < 0) return 0;
    const DQN rmid = qsum(lmid, t.qop[0][cb.k12]);
    const WKey* e = find_w(t, 0, cb.s1, cb.s2, cb.k12, lmid, rmid);
    if (!e) return 0;
    if (!qeq(qsum(rin, rmid), rout)) return 0;      // abelian triangle(Rin, Rmid, Rout)
    const int qR = find_r(t, rin, rout, rmid);
    if (qR < 0) return 0;
    int n = 0;
    for (int a = e->start; a < e->start + e->count; ++a) {
        const int64_t la = aux_at(t.l_aux_off, t.l_aux, qL, t.nz_row[0][a]);
        const int64_t rb = aux_at(t.r_aux_off, t.r_aux, qR, t.nz_col[0][a]);
        if (la < 0 || rb < 0) continue;
        if (EMIT) out[at + n] = Chain{qbra, la, qket, rb, t.nz_val[0][a]};
        ++n;
    }
    if (n > 0) *task = 1;   // a task when one nonzero has both blocks
    return n;
}

template <int SITES, bool EMIT>
__device__ inline int candidate(const Tables& t, const Combo* combos, const int64_t* in13, const int64_t* at24,
                                int64_t idx, int64_t at, Chain* out, int* task) {
    if (SITES == 2) return candidate2<EMIT>(t, combos, in13, at24, idx, at, out, task);
    return candidate1<EMIT>(t, combos, idx, at, out, task);
}

// exclusive scan of one value per thread over the block (kBuildThreads threads)
__device__ inline int block_scan(int v, int* sh, int* total) {
    const int tid = threadIdx.x;
    sh[tid] = v;
    __syncthreads();
    for (int d = 1; d < kBuildThreads; d <<= 1) {
        const int x = tid >= d ? sh[tid - d] : 0;
        __syncthreads();
        sh[tid] += x;
        __syncthreads();
    }
    *total = sh[kBuildThreads - 1];
    const int incl = sh[tid];
    __syncthreads();
    return incl - v;
}

template <int SITES>
__global__ void __launch_bounds__(kBuildThreads) count_kernel(Tables t, const Combo* combos, int64_t ncand,
                                                              const int64_t* in13, const int64_t* at24,
                                                              int64_t* block_sum, unsigned long long* tasks) {
    __shared__ int sh[kBuildThreads];
    const int64_t idx = blockIdx.x * (int64_t)kBuildThreads + threadIdx.x;
    int task = 0, n = 0;
    if (idx < ncand) n = candidate<SITES, false>(t, combos, in13, at24, idx, 0, nullptr, &task);
    int total = 0;
    block_scan(n, sh, &total);
    if (threadIdx.x == 0) block_sum[blockIdx.x] = total;
    // tasks: an order-free integer sum
    const unsigned mask = __ballot_sync(0xffffffffu, task != 0);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(tasks, (unsigned long long)__popc(mask));
}

__global__ void scan_sums_kernel(int64_t* block_sum, int64_t nb, int64_t* total) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int64_t acc = 0;
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t v = block_sum[b];
        block_sum[b] = acc;
        acc += v;
    }
    *total = acc;
}

template <int SITES>
__global__ void __launch_bounds__(kBuildThreads) emit_kernel(Tables t, const Combo* combos, int64_t ncand,
                                                             const int64_t* in13, const int64_t* at24,
                                                             const int64_t* block_off, int64_t cap, Chain* out,
                                                             int* overflow) {
    __shared__ int sh[kBuildThreads];
    const int64_t idx = blockIdx.x * (int64_t)kBuildThreads + threadIdx.x;
    int task = 0, n = 0;
    if (idx < ncand) n = candidate<SITES, false>(t, combos, in13, at24, idx, 0, nullptr, &task);
    int total = 0;
    const int pre = block_scan(n, sh, &total);
    const int64_t at = block_off[blockIdx.x] + pre;
    if (n == 0) return;
    if (at + n > cap) {   // the counting pass and this one disagree: report, write nothing
        atomicExch(overflow, 1);
        return;
    }
    candidate<SITES, true>(t, combos, in13, at24, idx, at, out, &task);
}

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("device builder: ") + what + ": " + cudaGetErrorString(e));
}

// The tables of one build in one device allocation: host arrays packed into a staging
// buffer at 256-byte aligned offsets (one upload), scratch placed after them.
struct Arena {
    std::vector<char> host;
    size_t scratch = 0;    // bytes of device-only scratch after the uploaded part
    char* dev = nullptr;
    struct Fix { size_t off; bool scratch; std::function<void(char*)> set; };
    std::vector<Fix> fixes;
    ~Arena() {
        if (dev) cudaFree(dev);
    }
    static size_t align(size_t x) { return (x + 255) / 256 * 256; }
    template <typename T>
    void put(const std::vector<T>& v, const T*& slot) {
        const size_t off = align(host.size());
        host.resize(off + std::max<size_t>(v.size(), 1) * sizeof(T), 0);
        if (!v.empty()) std::memcpy(host.data() + off, v.data(), v.size() * sizeof(T));
        fixes.push_back(Fix{off, false, [&slot](char* p) { slot = reinterpret_cast<const T*>(p); }});
    }
    template <typename T>
    void reserve(size_t n, T*& slot) {
        scratch = align(scratch);
        fixes.push_back(Fix{scratch, true, [&slot](char* p) { slot = reinterpret_cast<T*>(p); }});
        scratch += std::max<size_t>(n, 1) * sizeof(T);
    }
    void upload(cudaStream_t st) {
        const size_t up = align(host.size());
        ck(cudaMalloc((void**)&dev, up + scratch + 256), "cudaMalloc");
        ck(cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, st), "upload");
        for (const Fix& f : fixes) f.set(dev + (f.scratch ? up + f.off : f.off));
    }
};

// open-addressing slots for n entries with hashes h[i]: power of two >= 2n, linear probing
std::vector<int32_t> make_slots(const std::vector<uint64_t>& h, uint32_t& mask) {
    uint32_t size = 16;
    while (size < 2 * h.size()) size <<= 1;
    mask = size - 1;
    std::vector<int32_t> slot(size, -1);
    for (size_t i = 0; i < h.size(); ++i) {
        uint32_t s = (uint32_t)h[i] & mask;
        while (slot[s] >= 0) s = (s + 1) & mask;
        slot[s] = (int32_t)i;
    }
    return slot;
}

DQN dq(const QN& q) {
    DQN d;
    std::memcpy(d.v, q.v.data(), sizeof(d.v));
    return d;
}

// the matching of `nsites` MPO sites (W[0..nsites)) against L, R and the vector V
ChainSet build_device(cudaStream_t st, const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                      const MpoView* const* W, int nsites, const BlockTable& V) {
    if (sym.nonabelian()) throw std::invalid_argument("the device builder takes abelian symmetries");
    ChainSet cs;
    const TripodView Lv = make_tripod_view(L), Rv = make_tripod_view(R);
    CombinedBasis cb;
    if (nsites == 2) cb = combine_bases(sym, W[0]->qloc, W[1]->qloc);
    const int nkeys = (int)Lv.keys.size();
    make_bipeds_view(V, nsites == 2 ? cb.n : W[0]->nloc);   // throws on a duplicate block
    if (nkeys == 0 || V.n == 0 || Rv.keys.empty()) return cs;
    Arena A;
    Tables t{};
    // blocks of the vector
    std::vector<int32_t> v_leg((size_t)V.n);
    std::vector<DQN> v_qin((size_t)V.n), v_qout((size_t)V.n);
    std::vector<uint64_t> hv((size_t)V.n);
    for (int64_t i = 0; i < V.n; ++i) {
        v_leg[i] = V.leg[i];
        v_qin[i] = dq(V.qin[i]);
        v_qout[i] = dq(V.qout[i]);
        hv[i] = hash_v(v_leg[i], v_qin[i], v_qout[i]);
    }
    const auto v_slot = make_slots(hv, t.v_mask);
    A.put(v_leg, t.v_leg); A.put(v_qin, t.v_qin); A.put(v_qout, t.v_qout); A.put(v_slot, t.v_slot);
    // L and R keys with their auxiliary indices
    auto keys = [&](const TripodView& tv, std::vector<DQN>& qi, std::vector<DQN>& qo, std::vector<DQN>& qm,
                    std::vector<int32_t>& off, std::vector<int64_t>& aux) {
        off.push_back(0);
        for (size_t k = 0; k < tv.keys.size(); ++k) {
            qi.push_back(dq(tv.keys[k].q[0]));
            qo.push_back(dq(tv.keys[k].q[1]));
            qm.push_back(dq(tv.keys[k].q[2]));
            aux.insert(aux.end(), tv.aux[k].begin(), tv.aux[k].end());
            off.push_back((int32_t)aux.size());
        }
    };
    std::vector<DQN> li, lo, lm, ri, ro, rm;
    std::vector<int32_t> loff, roff;
    std::vector<int64_t> laux, raux;
    keys(Lv, li, lo, lm, loff, laux);
    keys(Rv, ri, ro, rm, roff, raux);
    std::vector<uint64_t> hr(ri.size());
    for (size_t i = 0; i < ri.size(); ++i) hr[i] = hash_r(ri[i], ro[i], rm[i]);
    const auto r_slot = make_slots(hr, t.r_mask);
    A.put(li, t.l_in); A.put(lo, t.l_out); A.put(lm, t.l_mid); A.put(loff, t.l_aux_off); A.put(laux, t.l_aux);
    t.nkeys = nkeys;
    A.put(ri, t.r_in); A.put(ro, t.r_out); A.put(rm, t.r_mid); A.put(r_slot, t.r_slot);
    A.put(roff, t.r_aux_off); A.put(raux, t.r_aux);
    // MPO nonzeros by (s1, s2, k, qin, qout), each list in the host's order
    std::vector<WKey> wk[2];
    std::vector<int32_t> wrow[2], wcol[2], wslot[2];
    std::vector<double> wval[2];
    std::vector<DQN> wqop[2], wqloc[2];
    for (int w = 0; w < nsites; ++w) {
        std::vector<uint64_t> hw;
        const MpoView& m = *W[w];
        for (int s1 = 0; s1 < m.nloc; ++s1)
            for (int s2 = 0; s2 < m.nloc; ++s2)
                for (int k = 0; k < m.nop; ++k)
                    for (const auto& kv : m.blocks[((size_t)s1 * m.nloc + s2) * m.nop + k]) {
                        WKey e{};
                        e.s1 = s1; e.s2 = s2; e.k = k;
                        e.qin = dq(kv.first.q[0]);
                        e.qout = dq(kv.first.q[1]);
                        e.start = (int32_t)wrow[w].size();
                        e.count = (int32_t)kv.second.size();
                        for (const MpoNz& z : kv.second) {
                            wrow[w].push_back(z.row);
                            wcol[w].push_back(z.col);
                            wval[w].push_back(z.val);
                        }
                        hw.push_back(hash_w(s1, s2, k, e.qin, e.qout));
                        wk[w].push_back(e);
                    }
        wslot[w] = make_slots(hw, t.w_mask[w]);
        for (const QN& q : m.qop) wqop[w].push_back(dq(q));
        for (const QN& q : m.qloc) wqloc[w].push_back(dq(q));
        A.put(wk[w], t.w_key[w]); A.put(wslot[w], t.w_slot[w]);
        A.put(wrow[w], t.nz_row[w]); A.put(wcol[w], t.nz_col[w]); A.put(wval[w], t.nz_val[w]);
        A.put(wqop[w], t.qop[w]); A.put(wqloc[w], t.qloc[w]);
    }
    std::vector<DQN> qof;
    for (const QN& q : cb.q_of) qof.push_back(dq(q));
    A.put(qof, t.q_of);
    t.ncomb = cb.n;
    // the combinations of the host loop nest, in its order
    std::vector<Combo> combos;
    const MpoView& W1 = *W[0];
    for (int s1 = 0; s1 < W1.nloc; ++s1)
    for (int s2 = 0; s2 < W1.nloc; ++s2)
    for (int k12 = 0; k12 < W1.nop; ++k12) {
        if (!sym.triangle(W1.qloc[s2], W1.qop[k12], W1.qloc[s1])) continue;
        if (nsites == 1) {
            combos.push_back(Combo{s1, s2, k12, 0, 0, 0, 0, 0});
            continue;
        }
        const MpoView& W2 = *W[1];
        const int n34 = W2.nloc;
        for (int s3 = 0; s3 < n34; ++s3)
        for (int s4 = 0; s4 < n34; ++s4)
        for (int k34 = 0; k34 < W2.nop; ++k34) {
            if (!sym.triangle(W2.qloc[s4], W2.qop[k34], W2.qloc[s3])) continue;
            for (const auto& m13 : cb.index[s1 * n34 + s3])
                for (const auto& m24 : cb.index[s2 * n34 + s4])
                    combos.push_back(Combo{s1, s2, k12, s3, s4, k34, m13.second, m24.second});
        }
    }
    if (combos.empty()) return cs;
    const Combo* d_combos = nullptr;
    A.put(combos, d_combos);
    const int64_t nmatch = nsites == 2 ? (int64_t)cb.n * nkeys : 0;
    const int64_t ncand = (int64_t)combos.size() * nkeys;
    const int64_t nblk = (ncand + kBuildThreads - 1) / kBuildThreads;
    if (nblk > 0x7fffffff) throw std::invalid_argument("device builder: too many candidates");
    int64_t *in13 = nullptr, *at24 = nullptr, *bsum = nullptr, *total = nullptr;
    unsigned long long* tasks = nullptr;
    int* overflow = nullptr;
    A.reserve((size_t)nmatch, in13);
    A.reserve((size_t)nmatch, at24);
    A.reserve((size_t)nblk, bsum);
    A.reserve(1, total);
    A.reserve(1, tasks);
    A.reserve(1, overflow);
    A.upload(st);
    ck(cudaMemsetAsync(tasks, 0, sizeof(unsigned long long), st), "memset");
    ck(cudaMemsetAsync(overflow, 0, sizeof(int), st), "memset");
    if (nsites == 2) {
        match_blocks_kernel<<<(unsigned)std::min<int64_t>((nmatch + 255) / 256, 4096), 256, 0, st>>>(t, in13, at24);
        ck(cudaGetLastError(), "match_blocks_kernel");
        count_kernel<2><<<(unsigned)nblk, kBuildThreads, 0, st>>>(t, d_combos, ncand, in13, at24, bsum, tasks);
    } else {
        count_kernel<1><<<(unsigned)nblk, kBuildThreads, 0, st>>>(t, d_combos, ncand, in13, at24, bsum, tasks);
    }
    ck(cudaGetLastError(), "count_kernel");
    scan_sums_kernel<<<1, 1, 0, st>>>(bsum, nblk, total);
    ck(cudaGetLastError(), "scan_sums_kernel");
    int64_t nchains = 0;
    unsigned long long ntasks = 0;
    ck(cudaMemcpyAsync(&nchains, total, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "download");
    ck(cudaMemcpyAsync(&ntasks, tasks, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st), "download");
    ck(cudaStreamSynchronize(st), "count");
    cs.n_tasks = (int64_t)ntasks;
    if (nchains == 0) return cs;
    Chain* out = nullptr;
    ck(cudaMalloc((void**)&out, sizeof(Chain) * (size_t)nchains), "cudaMalloc");
    std::unique_ptr<Chain, decltype(&cudaFree)> out_guard(out, &cudaFree);
    if (nsites == 2)
        emit_kernel<2><<<(unsigned)nblk, kBuildThreads, 0, st>>>(t, d_combos, ncand, in13, at24, bsum, nchains, out,
                                                                   overflow);
    else
        emit_kernel<1><<<(unsigned)nblk, kBuildThreads, 0, st>>>(t, d_combos, ncand, in13, at24, bsum, nchains, out,
                                                                   overflow);
    ck(cudaGetLastError(), "emit_kernel");
    cs.chains.resize((size_t)nchains);
    int ovf = 0;
    ck(cudaMemcpyAsync(cs.chains.data(), out, sizeof(Chain) * (size_t)nchains, cudaMemcpyDeviceToHost, st), "download");
    ck(cudaMemcpyAsync(&ovf, overflow, sizeof(int), cudaMemcpyDeviceToHost, st), "download");
    ck(cudaStreamSynchronize(st), "emit");
    if (ovf) throw std::logic_error("device builder: the emitting pass found more chains than the counting pass");
    cs.n_chains_raw = nchains;
    for (const Chain& c : cs.chains)
        cs.flops_reference += chain_flops_ref((double)L.rows[c.x], (double)L.cols[c.x], (double)V.cols[c.y],
                                              (double)R.cols[c.z]);
    return cs;
}

}  // namespace

ChainSet build_pivot2_device(CUstream_st* st, const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                             const MpoView& W12, const MpoView& W34, const BlockTable& V) {
    const MpoView* W[2] = {&W12, &W34};
    return build_device(st, sym, L, R, W, 2, V);
}

ChainSet build_pivot1_device(CUstream_st* st, const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                             const MpoView& W, const BlockTable& V) {
    const MpoView* Ws[1] = {&W};
    return build_device(st, sym, L, R, Ws, 1, V);
}

}  // namespace vmps
