// Host-side task-list builder and grouped-GEMM planner.
//
// The builders restate the quantum-number matching of VMPS:
//   LAWA    tensors/DmrgIndexGymnastics.h:32-77
//   AWAR    tensors/DmrgIndexGymnastics.h:79-124
//   AAWWAA  tensors/DmrgIndexGymnastics.h:198-262
//   precalc_blockStructure (1-site) :487-590, (2-site) :699-856
//   OxV loops pivot/DmrgPivotMatrix1.h:222-266, pivot/DmrgPivotMatrix2.h:182-230
//   HxV(PivotMatrix0) pivot/DmrgPivotMatrix0.h:37-95
//   contract_L tensors/DmrgContractions.h:35-158, contract_R :180-311
// and emit one Chain per (task, W nonzero) product with the SU(2) prefactor and
// the W value folded into a single scalar.  The planner then merges duplicate
// chains, shares first-stage products and lays the work out as tile lists.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <numeric>
#include <queue>
#include <unordered_set>
#include <stdexcept>
#include <tuple>

#include "engine.hpp"

namespace vmps {

// ===========================================================================
// SU(2) recoupling symbols: Racah formula for 6j, 9j as a sum of 6j products
// ===========================================================================
namespace {
struct Factorials {
    std::vector<long double> lf;   // log factorials
    Factorials() {
        lf.resize(512);
        lf[0] = 0;
        for (int i = 1; i < 512; ++i) lf[i] = lf[i - 1] + std::log((long double)i);
    }
};
const Factorials& facts() { static Factorials f; return f; }

bool tri2(int a, int b, int c) {   // arguments are 2j
    if (a < 0 || b < 0 || c < 0) return false;
    if ((a + b + c) & 1) return false;
    return c >= std::abs(a - b) && c <= a + b;
}
long double log_delta(int a, int b, int c) {   // 2j arguments, triangle already checked
    const auto& f = facts().lf;
    return 0.5L * (f[(a + b - c) / 2] + f[(a - b + c) / 2] + f[(-a + b + c) / 2] - f[(a + b + c) / 2 + 1]);
}
}  // namespace

// Memoised per thread: the builders ask for the same few symbols once per task
// (thousands of times per pivot), and each evaluation is an exp/log-factorial sum
// (three 6j per term of a 9j).  Arguments (2j) up to 127 pack into one key.
namespace {
template <int N>
bool pack_key(const int (&a)[N], uint64_t& key) {
    key = 0;
    for (int i = 0; i < N; ++i) {
        if (a[i] < 0 || a[i] > 127) return false;
        key = (key << 7) | (uint64_t)a[i];
    }
    return true;
}
double coupling_6j_eval(int j1, int j2, int j3, int j4, int j5, int j6);
double coupling_9j_eval(int j1, int j2, int j3, int j4, int j5, int j6, int j7, int j8, int j9);
}  // namespace

double coupling_6j(int j1, int j2, int j3, int j4, int j5, int j6) {
    thread_local std::unordered_map<uint64_t, double> memo;
    const int a[6] = {j1, j2, j3, j4, j5, j6};
    uint64_t key;
    if (!pack_key(a, key)) return coupling_6j_eval(j1, j2, j3, j4, j5, j6);
    auto it = memo.find(key);
    if (it != memo.end()) return it->second;
    const double v = coupling_6j_eval(j1, j2, j3, j4, j5, j6);
    memo.emplace(key, v);
    return v;
}

double coupling_9j(int j1, int j2, int j3, int j4, int j5, int j6, int j7, int j8, int j9) {
    thread_local std::unordered_map<uint64_t, double> memo;
    const int a[9] = {j1, j2, j3, j4, j5, j6, j7, j8, j9};
    uint64_t key;
    if (!pack_key(a, key)) return coupling_9j_eval(j1, j2, j3, j4, j5, j6, j7, j8, j9);
    auto it = memo.find(key);
    if (it != memo.end()) return it->second;
    const double v = coupling_9j_eval(j1, j2, j3, j4, j5, j6, j7, j8, j9);
    memo.emplace(key, v);
    return v;
}

namespace {
double coupling_6j_eval(int j1, int j2, int j3, int j4, int j5, int j6) {
    if (!tri2(j1, j2, j3) || !tri2(j1, j5, j6) || !tri2(j4, j2, j6) || !tri2(j4, j5, j3)) return 0.0;
    const auto& f = facts().lf;
    const int a1 = (j1 + j2 + j3) / 2, a2 = (j1 + j5 + j6) / 2, a3 = (j4 + j2 + j6) / 2, a4 = (j4 + j5 + j3) / 2;
    const int b1 = (j1 + j2 + j4 + j5) / 2, b2 = (j2 + j3 + j5 + j6) / 2, b3 = (j3 + j1 + j6 + j4) / 2;
    const int tmin = std::max(std::max(a1, a2), std::max(a3, a4));
    const int tmax = std::min(b1, std::min(b2, b3));
    const long double pre = log_delta(j1, j2, j3) + log_delta(j1, j5, j6) + log_delta(j4, j2, j6) + log_delta(j4, j5, j3);
    long double sum = 0;
    for (int t = tmin; t <= tmax; ++t) {
        long double lt = f[t + 1] - f[t - a1] - f[t - a2] - f[t - a3] - f[t - a4] - f[b1 - t] - f[b2 - t] - f[b3 - t];
        long double term = std::exp(lt + pre);
        sum += (t & 1) ? -term : term;
    }
    return (double)sum;
}

double coupling_9j_eval(int j1, int j2, int j3, int j4, int j5, int j6, int j7, int j8, int j9) {
    // {j1 j2 j3; j4 j5 j6; j7 j8 j9} = sum_x (-1)^{2x} (2x+1) {j1 j4 j7; j8 j9 x}{j2 j5 j8; j4 x j6}{j3 j6 j9; x j1 j2}
    if (!tri2(j1, j2, j3) || !tri2(j4, j5, j6) || !tri2(j7, j8, j9) || !tri2(j1, j4, j7) || !tri2(j2, j5, j8) ||
        !tri2(j3, j6, j9))
        return 0.0;
    int xmin = std::max(std::abs(j1 - j9), std::max(std::abs(j4 - j8), std::abs(j2 - j6)));
    int xmax = std::min(j1 + j9, std::min(j4 + j8, j2 + j6));
    long double sum = 0;
    for (int x = xmin; x <= xmax; x += 2) {
        long double t = (long double)(x + 1) * coupling_6j(j1, j4, j7, j8, j9, x) * coupling_6j(j2, j5, j8, j4, x, j6) *
                        coupling_6j(j3, j6, j9, x, j1, j2);
        sum += (x & 1) ? -t : t;   // (-1)^{2x} with 2x = x here
    }
    return (double)sum;
}
}  // namespace

// ===========================================================================
// parsing
// ===========================================================================
static QN read_qn(const Symmetry& sym, const int32_t* p, int64_t i) {
    QN q;
    for (int c = 0; c < sym.nq; ++c) q.v[c] = p[i * sym.nq + c];
    return q;
}

BlockTable parse_blocks(const Symmetry& sym, const vmps_blocks* b, bool need_mid) {
    BlockTable t;
    if (!b) throw std::invalid_argument("null block table");
    t.n = b->nblocks;
    if (t.n < 0) throw std::invalid_argument("negative block count");
    if (t.n > 0 && (!b->qin || !b->qout || !b->leg || !b->rows || !b->cols || !b->offset))
        throw std::invalid_argument("block table with null arrays");
    if (need_mid && t.n > 0 && !b->qmid) throw std::invalid_argument("Tripod table needs qmid");
    t.has_mid = b->qmid != nullptr;
    t.qin.resize(t.n); t.qout.resize(t.n); t.leg.resize(t.n);
    t.rows.resize(t.n); t.cols.resize(t.n); t.off.resize(t.n);
    if (t.has_mid) t.qmid.resize(t.n);
    for (int64_t i = 0; i < t.n; ++i) {
        t.qin[i] = read_qn(sym, b->qin, i);
        t.qout[i] = read_qn(sym, b->qout, i);
        if (t.has_mid) t.qmid[i] = read_qn(sym, b->qmid, i);
        t.leg[i] = b->leg[i];
        t.rows[i] = b->rows[i];
        t.cols[i] = b->cols[i];
        t.off[i] = b->offset[i];
        if (t.rows[i] <= 0 || t.cols[i] <= 0 || t.off[i] < 0 || t.leg[i] < 0)
            throw std::invalid_argument("block " + std::to_string(i) + " has non-positive shape or negative offset/leg");
        t.total = std::max(t.total, t.off[i] + t.rows[i] * t.cols[i]);
    }
    return t;
}

TripodView make_tripod_view(const BlockTable& t) {
    TripodView v;
    for (int64_t i = 0; i < t.n; ++i) {
        QN3 key{{t.qin[i], t.qout[i], t.qmid[i]}};
        auto it = v.dict.find(key);
        int q;
        if (it == v.dict.end()) {
            q = (int)v.keys.size();
            v.dict.emplace(key, q);
            v.keys.push_back(key);
            v.aux.emplace_back();
        } else {
            q = it->second;
        }
        auto& a = v.aux[q];
        if ((int)a.size() <= t.leg[i]) a.resize(t.leg[i] + 1, -1);
        if (a[t.leg[i]] != -1) throw std::invalid_argument("duplicate Tripod block");
        a[t.leg[i]] = i;
    }
    return v;
}

BipedsView make_bipeds_view(const BlockTable& t, int nlegs) {
    BipedsView v;
    int maxleg = nlegs;
    for (int64_t i = 0; i < t.n; ++i) maxleg = std::max(maxleg, t.leg[i] + 1);
    v.dict.resize(maxleg);
    for (int64_t i = 0; i < t.n; ++i) {
        auto r = v.dict[t.leg[i]].emplace(QN2{{t.qin[i], t.qout[i]}}, i);
        if (!r.second) throw std::invalid_argument("duplicate Biped block");
    }
    return v;
}

MpoView parse_mpo(const Symmetry& sym, const vmps_mpo_site* W) {
    if (!W) throw std::invalid_argument("null MPO site");
    MpoView m;
    m.nloc = W->nloc;
    m.nop = W->nop;
    if (m.nloc <= 0 || m.nop <= 0) throw std::invalid_argument("MPO site needs nloc>0 and nop>0");
    for (int i = 0; i < m.nloc; ++i) m.qloc.push_back(read_qn(sym, W->qloc, i));
    for (int i = 0; i < m.nop; ++i) m.qop.push_back(read_qn(sym, W->qop, i));
    m.blocks.resize((size_t)m.nloc * m.nloc * m.nop);
    for (int64_t i = 0; i < W->nnz; ++i) {
        int s1 = W->s1[i], s2 = W->s2[i], k = W->k[i];
        if (s1 < 0 || s1 >= m.nloc || s2 < 0 || s2 >= m.nloc || k < 0 || k >= m.nop || W->row[i] < 0 || W->col[i] < 0)
            throw std::invalid_argument("MPO entry out of range");
        QN2 key{{read_qn(sym, W->qin, i), read_qn(sym, W->qout, i)}};
        m.blocks[((size_t)s1 * m.nloc + s2) * m.nop + k][key].push_back(MpoNz{W->row[i], W->col[i], W->val[i]});
    }
    return m;
}

// ===========================================================================
// chain cost (DmrgExternal.h:147-159): (AB)C = mkn + mnp, A(BC) = knp + mkp
// ===========================================================================
static inline double chain_flops(double m, double k, double n, double p) {
    return 2.0 * std::min(m * k * n + m * n * p, k * n * p + m * k * p);
}
double chain_flops_ref(double m, double k, double n, double p) { return chain_flops(m, k, n, p); }

// ===========================================================================
// 1-site effective Hamiltonian (PivotMatrix1)
// ===========================================================================
ChainSet build_pivot1(const Symmetry& sym, const BlockTable& L, const BlockTable& R, const MpoView& W,
                      const BlockTable& V) {
    ChainSet cs;
    TripodView Lv = make_tripod_view(L), Rv = make_tripod_view(R);
    BipedsView Vv = make_bipeds_view(V, W.nloc);
    const double eps = 2.220446049250313e-16;
    for (int s1 = 0; s1 < W.nloc; ++s1)
    for (int s2 = 0; s2 < W.nloc; ++s2)
    for (int k = 0; k < W.nop; ++k) {
        if (!sym.triangle(W.qloc[s2], W.qop[k], W.qloc[s1])) continue;
        for (int qL = 0; qL < (int)Lv.keys.size(); ++qL) {
            const QN& Lin = Lv.keys[qL].q[0];
            const QN& Lout = Lv.keys[qL].q[1];
            const QN& Lmid = Lv.keys[qL].q[2];
            // LAWA (tensors/DmrgIndexGymnastics.h:32-77) with Abra = Aket = Vin
            for (const QN& Rout : sym.reduce(Lin, W.qloc[s1])) {
                int64_t qAbra = Vv.find(s1, Lin, Rout);
                if (qAbra < 0) continue;
                for (const QN& Rin : sym.reduce(Lout, W.qloc[s2])) {
                    int64_t qAket = Vv.find(s2, Lout, Rin);
                    if (qAket < 0) continue;
                    for (const QN& Rmid : sym.reduce(Lmid, W.qop[k])) {
                        const auto* nz = W.find(s1, s2, k, Lmid, Rmid);
                        if (!nz) continue;
                        if (!sym.triangle(Rin, Rmid, Rout)) continue;
                        auto itR = Rv.dict.find(QN3{{Rin, Rout, Rmid}});
                        if (itR == Rv.dict.end()) continue;
                        const int qR = itR->second;
                        bool any = false;
                        for (const auto& e : *nz)
                            if (Lv.at(qL, e.row) >= 0 && Rv.at(qR, e.col) >= 0) { any = true; break; }
                        if (!any) continue;
                        double cgc = 1.0;
                        if (sym.nonabelian()) {
                            QN q9[9] = {V.qin[qAket], W.qloc[s2], V.qout[qAket], Lmid, W.qop[k], Rmid,
                                        V.qin[qAbra], W.qloc[s1], V.qout[qAbra]};
                            cgc = sym.coeff_HPsi(q9);
                        }
                        if (std::abs(cgc) < eps) continue;
                        cs.n_tasks++;
                        for (const auto& e : *nz) {
                            int64_t la = Lv.at(qL, e.row), rb = Rv.at(qR, e.col);
                            if (la < 0 || rb < 0) continue;
                            cs.n_chains_raw++;
                            cs.flops_reference += chain_flops((double)L.rows[la], (double)L.cols[la],
                                                              (double)V.cols[qAket], (double)R.cols[rb]);
                            cs.chains.push_back(Chain{qAbra, la, qAket, rb, cgc * e.val});
                        }
                    }
                }
            }
        }
    }
    return cs;
}

// ===========================================================================
// Qbasis::combine of two local bases and the combined index s1s3
// (tensors/Qbasis.h:685-798, leftOffset :438-463, tensors/Basis.h:79-124)
// ===========================================================================
CombinedBasis combine_bases(const Symmetry& sym, const std::vector<QN>& q12, const std::vector<QN>& q34) {
    // Qbasis::pullData(qs): one entry per distinct QN in order of first appearance,
    // repeated QNs enlarge that entry's plain basis (inner index = order of appearance)
    auto pull = [](const std::vector<QN>& qs, std::vector<QN>& distinct, std::vector<int>& dim,
                   std::vector<int>& inner, std::vector<int>& which) {
        inner.resize(qs.size());
        which.resize(qs.size());
        for (size_t s = 0; s < qs.size(); ++s) {
            auto it = std::find(distinct.begin(), distinct.end(), qs[s]);
            int d;
            if (it == distinct.end()) { d = (int)distinct.size(); distinct.push_back(qs[s]); dim.push_back(0); }
            else d = (int)(it - distinct.begin());
            inner[s] = dim[d]++;
            which[s] = d;
        }
    };
    std::vector<QN> d1, d2;
    std::vector<int> dim1, dim2, in1, in2, w1, w2;
    pull(q12, d1, dim1, in1, w1);
    pull(q34, d2, dim2, in2, w2);
    struct Src { QN a, b; int da, db; };
    std::map<QN, std::vector<Src>> hist;   // keyed by merged QN
    for (size_t i = 0; i < d1.size(); ++i)
        for (size_t j = 0; j < d2.size(); ++j)
            for (const QN& q : sym.reduce(d1[i], d2[j])) {
                auto& h = hist[q];
                bool dup = false;
                for (auto& e : h) if (e.a == d1[i] && e.b == d2[j]) dup = true;
                if (!dup) h.push_back(Src{d1[i], d2[j], dim1[i], dim2[j]});
            }
    // sort sources lexicographically (Symmetry::compare on std::array{q1,q2})
    for (auto& kv : hist)
        std::sort(kv.second.begin(), kv.second.end(), [](const Src& x, const Src& y) {
            if (x.a != y.a) return x.a < y.a;
            return x.b < y.b;
        });
    CombinedBasis cb;
    std::map<QN, int> start;
    int cur = 0;
    for (auto& kv : hist) {   // std::map iterates QNs in ascending order (Qbasis::sort)
        start[kv.first] = cur;
        int tot = 0;
        for (auto& e : kv.second) tot += e.da * e.db;
        for (int t = 0; t < tot; ++t) cb.q_of.push_back(kv.first);
        cur += tot;
    }
    cb.n = cur;
    cb.index.resize(q12.size() * q34.size());
    for (size_t s1 = 0; s1 < q12.size(); ++s1)
        for (size_t s3 = 0; s3 < q34.size(); ++s3)
            for (const QN& q : sym.reduce(q12[s1], q34[s3])) {
                int off = 0;
                for (auto& e : hist[q]) {
                    if (e.a == q12[s1] && e.b == q34[s3]) {
                        off += in1[s1] + e.da * in2[s3];   // Basis::fuseData::source: j = i1 + dim1*i2
                        break;
                    }
                    off += e.da * e.db;
                }
                cb.index[s1 * q34.size() + s3].push_back({q, start[q] + off});
            }
    return cb;
}

// ===========================================================================
// 2-site effective Hamiltonian (PivotMatrix2)
// ===========================================================================
// Abelian symmetries: every reduction has exactly one result and all coupling
// coefficients are 1.  The loop nest of build_pivot2 below then visits, for the
// combined index s1s3, only the L keys whose incoming QN has a two-site block
// (s1s3, Lin, Lin + q(s1s3)) -- an ordered list made once -- so it produces the
// same chains in the same order while skipping the keys that produce none.
static ChainSet build_pivot2_abelian(const Symmetry& sym, const BlockTable& L, const BlockTable& R,
                                     const MpoView& W12, const MpoView& W34, const BlockTable& V,
                                     const TripodView& Lv, const TripodView& Rv, const CombinedBasis& cb,
                                     const BipedsView& Vv) {
    ChainSet cs;
    auto add = [&](const QN& a, const QN& b) {
        QN r = a;
        for (int i = 0; i < sym.nq; ++i) r.v[i] += b.v[i];
        return r;
    };
    const int nkeys = (int)Lv.keys.size();
    // per combined index c: (qL, q13) for the keys with a block (c, Lin, Lin + q(c)),
    // and q24 of (c, Lout, Lout + q(c)) for every key
    std::vector<std::vector<std::pair<int, int64_t>>> in13((size_t)cb.n);
    std::vector<std::vector<int64_t>> at24((size_t)cb.n, std::vector<int64_t>((size_t)nkeys, -1));
    for (int c = 0; c < cb.n; ++c)
        for (int qL = 0; qL < nkeys; ++qL) {
            const QN& Lin = Lv.keys[qL].q[0];
            const QN& Lout = Lv.keys[qL].q[1];
            const int64_t q13 = Vv.find(c, Lin, add(Lin, cb.q_of[c]));
            if (q13 >= 0) in13[(size_t)c].push_back({qL, q13});
            at24[(size_t)c][(size_t)qL] = Vv.find(c, Lout, add(Lout, cb.q_of[c]));
        }
    const int n12 = W12.nloc, n34 = W34.nloc;
    for (int s1 = 0; s1 < n12; ++s1)
    for (int s2 = 0; s2 < n12; ++s2)
    for (int k12 = 0; k12 < W12.nop; ++k12) {
        if (!sym.triangle(W12.qloc[s2], W12.qop[k12], W12.qloc[s1])) continue;
        for (int s3 = 0; s3 < n34; ++s3)
        for (int s4 = 0; s4 < n34; ++s4)
        for (int k34 = 0; k34 < W34.nop; ++k34) {
            if (!sym.triangle(W34.qloc[s4], W34.qop[k34], W34.qloc[s3])) continue;
            for (const auto& m13 : cb.index[s1 * n34 + s3])
            for (const auto& m24 : cb.index[s2 * n34 + s4]) {
                const int s1s3 = m13.second, s2s4 = m24.second;
                const auto& t24 = at24[(size_t)s2s4];
                for (const auto& e13 : in13[(size_t)s1s3]) {
                    const int qL = e13.first;
                    const int64_t q13 = e13.second, q24 = t24[(size_t)qL];
                    if (q24 < 0) continue;
                    const QN& Lmid = Lv.keys[qL].q[2];
                    const QN qRout = V.qout[q13], qRin = V.qout[q24];
                    const QN qW = add(Lmid, W12.qop[k12]);
                    const auto* nz12 = W12.find(s1, s2, k12, Lmid, qW);
                    if (!nz12) continue;
                    const QN qRmid = add(qW, W34.qop[k34]);
                    const auto* nz34 = W34.find(s3, s4, k34, qW, qRmid);
                    if (!nz34) continue;
                    if (!sym.triangle(qRin, qRmid, qRout)) continue;
                    auto itR = Rv.dict.find(QN3{{qRin, qRout, qRmid}});
                    if (itR == Rv.dict.end()) continue;
                    const int qR = itR->second;
                    cs.n_tasks++;
                    for (const auto& e12 : *nz12)
                        for (const auto& e34 : *nz34) {
                            if (e12.col != e34.row) continue;
                            const int64_t la = Lv.at(qL, e12.row), rb = Rv.at(qR, e34.col);
                            if (la < 0 || rb < 0) continue;
                            cs.n_chains_raw++;
                            cs.flops_reference += chain_flops((double)L.rows[la], (double)L.cols[la],
                                                              (double)V.cols[q24], (double)R.cols[rb]);
                            cs.chains.push_back(Chain{q13, la, q24, rb, e12.val * e34.val});
                        }
                }
            }
        }
    }
    return cs;
}

ChainSet build_pivot2(const Symmetry& sym, const BlockTable& L, const BlockTable& R, const MpoView& W12,
                      const MpoView& W34, const BlockTable& V) {
    ChainSet cs;
    TripodView Lv = make_tripod_view(L), Rv = make_tripod_view(R);
    CombinedBasis cb = combine_bases(sym, W12.qloc, W34.qloc);
    BipedsView Vv = make_bipeds_view(V, cb.n);
    if (!sym.nonabelian()) return build_pivot2_abelian(sym, L, R, W12, W34, V, Lv, Rv, cb, Vv);
    const double eps = 2.220446049250313e-16;
    const int n12 = W12.nloc, n34 = W34.nloc;
    for (int s1 = 0; s1 < n12; ++s1)
    for (int s2 = 0; s2 < n12; ++s2)
    for (int k12 = 0; k12 < W12.nop; ++k12) {
        if (!sym.triangle(W12.qloc[s2], W12.qop[k12], W12.qloc[s1])) continue;
        for (int s3 = 0; s3 < n34; ++s3)
        for (int s4 = 0; s4 < n34; ++s4)
        for (int k34 = 0; k34 < W34.nop; ++k34) {
            if (!sym.triangle(W34.qloc[s4], W34.qop[k34], W34.qloc[s3])) continue;
            for (const QN& qOp : sym.reduce(W12.qop[k12], W34.qop[k34])) {
                for (const auto& m13 : cb.index[s1 * n34 + s3])
                for (const auto& m24 : cb.index[s2 * n34 + s4]) {
                    const QN& qmerge13 = m13.first;
                    const QN& qmerge24 = m24.first;
                    const int s1s3 = m13.second, s2s4 = m24.second;
                    double cgc9 = 1.0;
                    if (sym.nonabelian()) {
                        QN q9[9] = {W12.qloc[s2], W34.qloc[s4], qmerge24, W12.qop[k12], W34.qop[k34], qOp,
                                    W12.qloc[s1], W34.qloc[s3], qmerge13};
                        cgc9 = sym.coeff_tensorProd(q9);
                    }
                    if (std::abs(cgc9) < eps) continue;
                    for (int qL = 0; qL < (int)Lv.keys.size(); ++qL) {
                        const QN& Lin = Lv.keys[qL].q[0];
                        const QN& Lout = Lv.keys[qL].q[1];
                        const QN& Lmid = Lv.keys[qL].q[2];
                        // AAWWAA (tensors/DmrgIndexGymnastics.h:198-262)
                        for (const QN& qRout : sym.reduce(Lin, qmerge13)) {
                            int64_t q13 = Vv.find(s1s3, Lin, qRout);
                            if (q13 < 0) continue;
                            for (const QN& qRin : sym.reduce(Lout, qmerge24)) {
                                int64_t q24 = Vv.find(s2s4, Lout, qRin);
                                if (q24 < 0) continue;
                                for (const QN& qW : sym.reduce(Lmid, W12.qop[k12])) {
                                    const auto* nz12 = W12.find(s1, s2, k12, Lmid, qW);
                                    if (!nz12) continue;
                                    for (const QN& qRmid : sym.reduce(qW, W34.qop[k34])) {
                                        const auto* nz34 = W34.find(s3, s4, k34, qW, qRmid);
                                        if (!nz34) continue;
                                        if (!sym.triangle(qRin, qRmid, qRout)) continue;
                                        double cgc6 = 1.0;
                                        if (sym.nonabelian()) {
                                            QN q6[6] = {Lmid, W12.qop[k12], qW, W34.qop[k34], qRmid, qOp};
                                            cgc6 = sym.coeff_Apair(q6);
                                        }
                                        if (std::abs(cgc6) < eps) continue;
                                        auto itR = Rv.dict.find(QN3{{qRin, qRout, qRmid}});
                                        if (itR == Rv.dict.end()) continue;
                                        const int qR = itR->second;
                                        double cgcH = 1.0;
                                        if (sym.nonabelian()) {
                                            QN q9[9] = {V.qin[q24], qmerge24, V.qout[q24], Lmid, qOp, qRmid,
                                                        V.qin[q13], qmerge13, V.qout[q13]};
                                            cgcH = sym.coeff_HPsi(q9);
                                        }
                                        const double cgc = cgc6 * cgc9 * cgcH;
                                        cs.n_tasks++;
                                        // OxV(PivotMatrix2) inner loop, pivot/DmrgPivotMatrix2.h:202-228
                                        for (const auto& e12 : *nz12)
                                            for (const auto& e34 : *nz34) {
                                                if (e12.col != e34.row) continue;
                                                int64_t la = Lv.at(qL, e12.row), rb = Rv.at(qR, e34.col);
                                                if (la < 0 || rb < 0) continue;
                                                cs.n_chains_raw++;
                                                cs.flops_reference +=
                                                    chain_flops((double)L.rows[la], (double)L.cols[la],
                                                                (double)V.cols[q24], (double)R.cols[rb]);
                                                cs.chains.push_back(Chain{q13, la, q24, rb, cgc * e12.val * e34.val});
                                            }
                                    }
                                }
                            }
                        }
                    }
                }
            }
        }
    }
    return cs;
}

// ===========================================================================
// 0-site effective Hamiltonian (PivotMatrix0), pivot/DmrgPivotMatrix0.h:37-95
// ===========================================================================
ChainSet build_pivot0(const Symmetry& sym, const BlockTable& L, const BlockTable& R, const BlockTable& V) {
    (void)sym;
    ChainSet cs;
    TripodView Lv = make_tripod_view(L), Rv = make_tripod_view(R);
    BipedsView Vv = make_bipeds_view(V, 1);
    for (int qL = 0; qL < (int)Lv.keys.size(); ++qL) {
        const QN& Lin = Lv.keys[qL].q[0];
        const QN& Lout = Lv.keys[qL].q[1];
        const QN& Lmid = Lv.keys[qL].q[2];
        auto itR = Rv.dict.find(QN3{{Lout, Lin, Lmid}});
        if (itR == Rv.dict.end()) continue;
        const int qR = itR->second;
        int64_t qAin = Vv.find(0, Lout, Lout);
        if (qAin < 0) continue;
        const QN& Rout = Rv.keys[qR].q[1];
        int64_t qAout = Vv.find(0, Rout, Rout);
        if (qAout < 0) continue;
        cs.n_tasks++;
        const int na = (int)std::max(Lv.aux[qL].size(), Rv.aux[qR].size());
        for (int a = 0; a < na; ++a) {
            int64_t la = Lv.at(qL, a), ra = Rv.at(qR, a);
            if (la < 0 || ra < 0) continue;
            cs.n_chains_raw++;
            cs.flops_reference += chain_flops((double)L.rows[la], (double)L.cols[la], (double)V.cols[qAin],
                                              (double)R.cols[ra]);
            cs.chains.push_back(Chain{qAout, la, qAin, ra, 1.0});
        }
    }
    return cs;
}

// ===========================================================================
// contract_L / contract_R (FULL mode), tensors/DmrgContractions.h:35-311
// ===========================================================================
ChainSet build_env(const Symmetry& sym, int side, const BlockTable& E, const BlockTable& Abra, const MpoView& W,
                   const BlockTable& Aket, BlockTable* Enew, const EnvMode& md) {
    ChainSet cs;
    TripodView Ev = make_tripod_view(E);
    BipedsView Bv = make_bipeds_view(Abra, W.nloc), Kv = make_bipeds_view(Aket, W.nloc);
    const double eps = 2.220446049250313e-16;
    // output blocks keyed by (quple, aux index)
    std::unordered_map<QN3, int, QNTupleHash<3>> odict;
    std::vector<QN3> okeys;
    std::vector<std::vector<int64_t>> oaux;   // -> output block id
    std::vector<int64_t> orows, ocols;
    std::vector<QN> oin, oout, omid;
    std::vector<int32_t> oleg;
    auto out_block = [&](const QN3& quple, int a, int64_t rows, int64_t cols) -> int64_t {
        auto it = odict.find(quple);
        int q;
        if (it == odict.end()) {
            q = (int)okeys.size();
            odict.emplace(quple, q);
            okeys.push_back(quple);
            oaux.emplace_back();
        } else q = it->second;
        auto& v = oaux[q];
        if ((int)v.size() <= a) v.resize(a + 1, -1);
        if (v[a] < 0) {
            v[a] = (int64_t)orows.size();
            orows.push_back(rows); ocols.push_back(cols);
            oin.push_back(quple.q[0]); oout.push_back(quple.q[1]); omid.push_back(quple.q[2]);
            oleg.push_back(a);
        } else if (orows[v[a]] != rows || ocols[v[a]] != cols) {
            throw std::invalid_argument("inconsistent output block shapes in environment update");
        }
        return v[a];
    };
    // Abelian symmetries: every reduction has one result, so for each s1 only the
    // E keys with a bra block (s1, ...) can produce chains; they are listed once, in
    // key order, and the loop below visits those alone (same chains, same order)
    const bool abelian = !sym.nonabelian();
    const int nkeys = (int)Ev.keys.size();
    std::vector<std::vector<int>> bra_keys;   // per s1: E keys with a bra block
    std::vector<std::vector<int64_t>> ket_at; // per s2 and E key: the ket block or -1
    if (abelian) {
        auto add = [&](const QN& a, const QN& b, int sign) {
            QN r = a;
            for (int i = 0; i < sym.nq; ++i) r.v[i] += sign * b.v[i];
            return r;
        };
        bra_keys.resize(W.nloc);
        ket_at.assign(W.nloc, std::vector<int64_t>((size_t)nkeys, -1));
        for (int s = 0; s < W.nloc; ++s)
            for (int qE = 0; qE < nkeys; ++qE) {
                const QN& Ein = Ev.keys[qE].q[0];
                const QN& Eout = Ev.keys[qE].q[1];
                const int64_t b = side == VMPS_ENV_LEFT ? Bv.find(s, Ein, add(Ein, W.qloc[s], 1))
                                                        : Bv.find(s, add(Eout, W.qloc[s], -1), Eout);
                if (b >= 0) bra_keys[s].push_back(qE);
                ket_at[s][qE] = side == VMPS_ENV_LEFT ? Kv.find(s, Eout, add(Eout, W.qloc[s], 1))
                                                      : Kv.find(s, add(Ein, W.qloc[s], -1), Ein);
            }
    }
    std::vector<int> all_keys((size_t)nkeys);
    for (int q = 0; q < nkeys; ++q) all_keys[(size_t)q] = q;
    for (int s1 = 0; s1 < W.nloc; ++s1)
    for (int s2 = 0; s2 < W.nloc; ++s2)
    for (int k = 0; k < W.nop; ++k) {
        if (!sym.triangle(W.qloc[s2], W.qop[k], W.qloc[s1])) continue;
        for (int qE : abelian ? bra_keys[s1] : all_keys) {
            if (abelian && ket_at[s2][qE] < 0) continue;
            const QN& Ein = Ev.keys[qE].q[0];
            const QN& Eout = Ev.keys[qE].q[1];
            const QN& Emid = Ev.keys[qE].q[2];
            if (side == VMPS_ENV_LEFT) {
                // LAWA -> quple {Rout, Rin, Rmid}
                for (const QN& Rout : sym.reduce(Ein, W.qloc[s1])) {
                    int64_t qAbra = Bv.find(s1, Ein, Rout);
                    if (qAbra < 0) continue;
                    for (const QN& Rin : sym.reduce(Eout, W.qloc[s2])) {
                        int64_t qAket = Kv.find(s2, Eout, Rin);
                        if (qAket < 0) continue;
                        for (const QN& Rmid : sym.reduce(Emid, W.qop[k])) {
                            const auto* nz = W.find(s1, s2, k, Emid, Rmid);
                            if (!nz) continue;
                            if (!sym.triangle(Rin, Rmid, Rout)) continue;
                            double cgc = 1.0;
                            if (sym.nonabelian()) {
                                QN q9[9] = {Aket.qin[qAket], W.qloc[s2], Aket.qout[qAket], Emid, W.qop[k], Rmid,
                                            Abra.qin[qAbra], W.qloc[s1], Abra.qout[qAbra]};
                                cgc = sym.coeff_buildL(q9);
                            }
                            if (std::abs(cgc) < eps) continue;
                            cs.n_tasks++;
                            QN3 quple{{Rout, Rin, Rmid}};
                            for (const auto& e : *nz) {
                                // mode filter of contract_L (tensors/DmrgContractions.h:100-104)
                                if (md.mode == VMPS_ENV_TRIANGULAR && !(md.at(Emid, e.row) > md.fixed_ab)) continue;
                                if (md.mode == VMPS_ENV_FIXED_COLS && md.at(Rmid, e.col) != md.fixed_ab) continue;
                                if (md.mode == VMPS_ENV_FIXED_ROWS && md.at(Emid, e.row) != md.fixed_ab) continue;
                                int64_t la = Ev.at(qE, e.row);
                                if (la < 0) continue;
                                // Abra^dagger (cols_bra x rows_bra) * L (rows_bra x rows_ket) * Aket
                                int64_t o = out_block(quple, e.col, Abra.cols[qAbra], Aket.cols[qAket]);
                                cs.n_chains_raw++;
                                cs.flops_reference += chain_flops((double)Abra.cols[qAbra], (double)Abra.rows[qAbra],
                                                                  (double)E.cols[la], (double)Aket.cols[qAket]);
                                cs.chains.push_back(Chain{o, qAbra, la, qAket, cgc * e.val});
                            }
                        }
                    }
                }
            } else {
                // AWAR (tensors/DmrgIndexGymnastics.h:79-124) -> quple {Lout, Lin, Lmid}
                const QN& Rin = Ein;
                const QN& Rout = Eout;
                const QN& Rmid = Emid;
                for (const QN& Lin : sym.reduce(Rout, sym.flip(W.qloc[s1]))) {
                    int64_t qAbra = Bv.find(s1, Lin, Rout);
                    if (qAbra < 0) continue;
                    for (const QN& Lout : sym.reduce(Rin, sym.flip(W.qloc[s2]))) {
                        int64_t qAket = Kv.find(s2, Lout, Rin);
                        if (qAket < 0) continue;
                        for (const QN& Lmid : sym.reduce(Rmid, sym.flip(W.qop[k]))) {
                            const auto* nz = W.find(s1, s2, k, Lmid, Rmid);
                            if (!nz) continue;
                            if (!sym.triangle(Lout, Lmid, Lin)) continue;
                            double cgc = 1.0;
                            if (sym.nonabelian()) {
                                QN q9[9] = {Aket.qin[qAket], W.qloc[s2], Aket.qout[qAket], Lmid, W.qop[k], Rmid,
                                            Abra.qin[qAbra], W.qloc[s1], Abra.qout[qAbra]};
                                cgc = sym.coeff_buildR(q9);
                            }
                            if (std::abs(cgc) < eps) continue;
                            cs.n_tasks++;
                            QN3 quple{{Lout, Lin, Lmid}};
                            for (const auto& e : *nz) {
                                // mode filter of contract_R (tensors/DmrgContractions.h:245-249)
                                if (md.mode == VMPS_ENV_TRIANGULAR && !(md.fixed_ab > md.at(Rmid, e.col))) continue;
                                if (md.mode == VMPS_ENV_FIXED_ROWS && md.at(Lmid, e.row) != md.fixed_ab) continue;
                                if (md.mode == VMPS_ENV_FIXED_COLS && md.at(Rmid, e.col) != md.fixed_ab) continue;
                                int64_t rb = Ev.at(qE, e.col);
                                if (rb < 0) continue;
                                // Aket (rows_ket x cols_ket) * R (cols_ket x cols_bra) * Abra^dagger
                                int64_t o = out_block(quple, e.row, Aket.rows[qAket], Abra.rows[qAbra]);
                                cs.n_chains_raw++;
                                cs.flops_reference += chain_flops((double)Aket.rows[qAket], (double)Aket.cols[qAket],
                                                                  (double)E.cols[rb], (double)Abra.rows[qAbra]);
                                cs.chains.push_back(Chain{o, qAket, rb, qAbra, cgc * e.val});
                            }
                        }
                    }
                }
            }
        }
    }
    // compact output layout, blocks in creation order
    BlockTable& t = *Enew;
    t = BlockTable();
    t.n = (int64_t)orows.size();
    t.has_mid = true;
    t.qin = oin; t.qout = oout; t.qmid = omid; t.leg = oleg; t.rows = orows; t.cols = ocols;
    t.off.resize(t.n);
    int64_t cur = 0;
    for (int64_t i = 0; i < t.n; ++i) { t.off[i] = cur; cur += orows[i] * ocols[i]; }
    t.total = cur;
    return cs;
}

// ===========================================================================
// planner
// ===========================================================================
DevLayout make_dev_layout(const std::vector<int64_t>& rows, const std::vector<int64_t>& cols) {
    DevLayout d;
    const size_t n = rows.size();
    d.off.resize(n); d.rows = rows; d.cols = cols; d.ld.resize(n);
    int64_t cur = 0;
    for (size_t i = 0; i < n; ++i) {
        d.ld[i] = pad_ld(rows[i]);
        d.off[i] = cur;
        cur = pad_off(cur + d.ld[i] * cols[i]);
    }
    d.total = std::max<int64_t>(cur, 32);
    return d;
}

namespace {
struct Key4 {
    int64_t a, b, c, d;
    bool operator==(const Key4& o) const { return a == o.a && b == o.b && c == o.c && d == o.d; }
};
struct Key4Hash {
    size_t operator()(const Key4& k) const {
        uint64_t h = (uint64_t)k.a * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)k.b + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
        h ^= (uint64_t)k.c + 0x94D049BB133111EBull + (h << 6) + (h >> 2);
        h ^= (uint64_t)k.d + 0xBF58476D1CE4E5B9ull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};

// split an extent into balanced pieces of at most tmax, each a multiple of
// `gran` except the last: 193 -> 48,48,48,49 rather than 64,64,64,1
static std::vector<std::pair<int64_t, int64_t>> split_extent(int64_t m, int64_t gran, int64_t tmax) {
    std::vector<std::pair<int64_t, int64_t>> out;
    const int64_t nt = (m + tmax - 1) / tmax;
    int64_t base = gran * (m / (nt * gran));
    if (base < gran || m - base * (nt - 1) > tmax) base = gran * ((m + nt * gran - 1) / (nt * gran));
    int64_t r = 0;
    for (int64_t i = 0; i < nt && r < m; ++i) {
        const int64_t len = (i + 1 == nt) ? m - r : std::min(base, m - r);
        out.push_back({r, len});
        r += len;
    }
    return out;
}

// append tiles of an m x n output block whose segments are [sb, se)
void add_tiles(PhasePlan& ph, int64_t c_off, int64_t ldc, int64_t m, int64_t n, int32_t sb, int32_t se, int tile_m,
               int tile_n, int col_gran = 8) {
    for (const auto& rs : split_extent(m, 16, tile_m))
        for (const auto& cs : split_extent(n, col_gran, tile_n)) {
            GTile t{};
            t.c_off = c_off;
            t.ldc = (int32_t)ldc;
            t.row0 = (int32_t)rs.first;
            t.tm = (int32_t)rs.second;
            t.col0 = (int32_t)cs.first;
            t.tn = (int32_t)cs.second;
            t.seg_begin = sb;
            t.seg_end = se;
            ph.tiles.push_back(t);
        }
}

// order tiles by descending work so that the hardware block scheduler runs the
// largest first (longest-processing-time list scheduling)
void sort_tiles(PhasePlan& ph) {
    std::vector<double> cost(ph.tiles.size());
    for (size_t i = 0; i < ph.tiles.size(); ++i) {
        const GTile& t = ph.tiles[i];
        double k = 0;
        for (int s = t.seg_begin; s < t.seg_end; ++s) k += ph.segs[s].K * (double)ph.segs[s].term_count;
        cost[i] = k * t.tm * t.tn + 1.0;
    }
    std::vector<size_t> idx(ph.tiles.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<GTile> t2(ph.tiles.size());
    for (size_t i = 0; i < idx.size(); ++i) t2[i] = ph.tiles[idx[i]];
    ph.tiles.swap(t2);
}
}  // namespace

int32_t panel_kpad(int64_t K) {
    K = std::max<int64_t>(K, 1);
    int64_t q = K <= 256 ? 32 : K <= 1024 ? 128 : K <= 4096 ? 512 : 2048;
    return (int32_t)((K + q - 1) / q * q);
}

int32_t box_rows_a(int32_t tm, bool fine) {
    if (fine) return std::min<int32_t>(128, std::max<int32_t>(16, (tm + 15) / 16 * 16));
    for (int32_t h : {16, 32, 64, 128})
        if (tm <= h) return h;
    return 128;
}

int32_t box_rows_b(int32_t tn, bool fine) {
    if (tn <= 16) return 16;
    return std::min<int32_t>(256, fine ? (tn + 15) / 16 * 16 : (tn + 31) / 32 * 32);
}

void schedule_tma(PhasePlan& ph, int ncta, const std::vector<OpBlock>& A, const std::vector<OpBlock>& B,
                  int kstep) {
    if (kstep != 32 && kstep != 16) throw std::invalid_argument("K step of a split plan must be 32 or 16");
    const size_t nt = ph.tiles.size();
    ph.steps.clear();
    ph.amaps.clear();
    ph.bmaps.clear();
    ph.cta_tiles.assign(1, 0);
    ph.ncta = 0;
    if (nt == 0 || ncta <= 0) return;
    ncta = (int)std::min<size_t>((size_t)ncta, nt);
    // cost of a tile: its K steps plus the epilogue (about one step's time)
    std::vector<int32_t> nsteps(nt, 0);
    std::vector<double> cost(nt);
    for (size_t i = 0; i < nt; ++i) {
        const GTile& t = ph.tiles[i];
        int32_t n = 0;
        for (int s = t.seg_begin; s < t.seg_end; ++s) n += (ph.segs[s].K + kstep - 1) / kstep;
        nsteps[i] = n;
        cost[i] = n + 1.0;
    }
    std::vector<size_t> order(nt);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    // least-loaded CTA first; ties to the lower index (deterministic)
    using Load = std::pair<double, int>;
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
    for (int b = 0; b < ncta; ++b) heap.push({0.0, b});
    std::vector<std::vector<size_t>> per(ncta);
    for (size_t i : order) {
        Load l = heap.top();
        heap.pop();
        per[l.second].push_back(i);
        heap.push({l.first + cost[i], l.second});
    }
    // descriptors: one per (panel class, box height) used, for each side
    std::map<std::pair<int32_t, int32_t>, int32_t> aidx, bidx;
    auto map_of = [](std::map<std::pair<int32_t, int32_t>, int32_t>& idx, std::vector<MapKey>& keys, int32_t cls,
                     int32_t rows) {
        auto it = idx.find({cls, rows});
        if (it != idx.end()) return it->second;
        const int32_t i = (int32_t)keys.size();
        keys.push_back(MapKey{cls, rows});
        idx.emplace(std::make_pair(cls, rows), i);
        return i;
    };
    // box heights: the tile's extent rounded to 16 rows (fewer bytes through TMA) unless
    // that needs more descriptors than a launch takes
    bool fine = true;
    {
        std::set<std::pair<int32_t, int32_t>> ka, kb;
        for (size_t i = 0; i < nt; ++i) {
            const GTile& t = ph.tiles[i];
            for (int s = t.seg_begin; s < t.seg_end; ++s) {
                ka.insert({A[ph.seg_amap[s]].cls, box_rows_a(t.tm)});
                kb.insert({B[ph.seg_bmap[s]].cls, box_rows_b(t.tn)});
            }
        }
        fine = (int)ka.size() <= kMaxMapsA && (int)kb.size() <= kMaxMapsB;
    }
    std::vector<GTile> tiles;
    tiles.reserve(nt);
    ph.cta_tiles.assign(ncta + 1, 0);
    for (int b = 0; b < ncta; ++b) {
        for (size_t i : per[b]) {
            GTile t = ph.tiles[i];
            t.step0 = (int32_t)ph.steps.size();
            t.nsteps = nsteps[i];
            const int32_t ha = box_rows_a(t.tm, fine), hb = box_rows_b(t.tn, fine);
            for (int s = t.seg_begin; s < t.seg_end; ++s) {
                const OpBlock& oa = A[ph.seg_amap[s]];
                const OpBlock& ob = B[ph.seg_bmap[s]];
                const int32_t am = map_of(aidx, ph.amaps, oa.cls, ha), bm = map_of(bidx, ph.bmaps, ob.cls, hb);
                for (int32_t k0 = 0; k0 < ph.segs[s].K; k0 += kstep) {
                    TStep st{};
                    st.amap = am;
                    st.bmap = bm;
                    // bit 0 of x: only the first half of the step's K columns lies inside the segment
                    st.x = 2 * k0 | (ph.segs[s].K - k0 <= kstep / 2 ? 1 : 0);
                    st.xa = 2 * (ph.segs[s].akoff + k0);
                    st.ay = oa.row + t.row0;
                    st.by = ob.row + t.col0;
                    st.arows = ha;
                    st.brows = hb;
                    ph.steps.push_back(st);
                }
            }
            tiles.push_back(t);
        }
        ph.cta_tiles[b + 1] = (int32_t)tiles.size();
    }
    ph.tiles.swap(tiles);
    ph.ncta = ncta;
}

PhasePlan make_product_plan(const DevLayout& A, const DevLayout& B, const DevLayout& C,
                            const std::vector<std::array<int64_t, 3>>& prods, const double* coef) {
    PhasePlan ph;
    ph.transA = false; ph.transB = false; ph.transC = false;
    std::vector<std::vector<size_t>> by_out(C.rows.size());
    for (size_t q = 0; q < prods.size(); ++q) {
        const int64_t k = prods[q][0], i = prods[q][1], j = prods[q][2];
        if (k < 0 || k >= (int64_t)C.rows.size() || i < 0 || i >= (int64_t)A.rows.size() || j < 0 ||
            j >= (int64_t)B.rows.size())
            throw std::invalid_argument("product references a block outside its table");
        if (A.cols[i] != B.rows[j] || C.rows[k] != A.rows[i] || C.cols[k] != B.cols[j])
            throw std::domain_error("block shapes do not chain in product " + std::to_string(q));
        by_out[k].push_back(q);
    }
    for (size_t k = 0; k < C.rows.size(); ++k) {
        const int32_t sb = (int32_t)ph.segs.size();
        for (size_t q : by_out[k]) {
            const int64_t i = prods[q][1], j = prods[q][2];
            GSeg s{};
            s.b_off = B.off[j];
            s.term_begin = (int32_t)ph.terms.size();
            s.term_count = 1;
            ph.terms.push_back(GTerm{A.off[i], coef ? coef[q] : 1.0});
            s.lda = (int32_t)A.ld[i];
            s.ldb = (int32_t)B.ld[j];
            s.K = (int32_t)A.cols[i];
            ph.segs.push_back(s);
            ph.flops += 2.0 * A.rows[i] * A.cols[i] * B.cols[j];
        }
        add_tiles(ph, C.off[k], C.ld[k], C.rows[k], C.cols[k], sb, (int32_t)ph.segs.size(), kTileMax, kTileMax);
    }
    sort_tiles(ph);
    return ph;
}

Plan make_plan(const ChainSet& cs, const DevLayout& X, const DevLayout& Y, const DevLayout& Z, const DevLayout& O,
               bool transX, bool transZ, int tile_m, int tile_n) {
    Plan P;
    // shapes: op(X) m x k, Y k x n, op(Z) n x p, out m x p
    auto xm = [&](int64_t x) { return transX ? X.cols[x] : X.rows[x]; };
    auto xk = [&](int64_t x) { return transX ? X.rows[x] : X.cols[x]; };
    auto zn = [&](int64_t z) { return transZ ? Z.cols[z] : Z.rows[z]; };
    auto zp = [&](int64_t z) { return transZ ? Z.rows[z] : Z.cols[z]; };

    // ---- merge duplicate chains (same out, X, Y, Z): coefficients add
    std::unordered_map<Key4, size_t, Key4Hash> mdict;
    std::vector<Chain> ch;
    ch.reserve(cs.chains.size());
    for (const Chain& c : cs.chains) {
        if (c.out < 0 || c.out >= (int64_t)O.rows.size() || c.x < 0 || c.x >= (int64_t)X.rows.size() || c.y < 0 ||
            c.y >= (int64_t)Y.rows.size() || c.z < 0 || c.z >= (int64_t)Z.rows.size())
            throw std::invalid_argument("chain references a block outside its table");
        if (xk(c.x) != Y.rows[c.y] || Y.cols[c.y] != zn(c.z) || O.rows[c.out] != xm(c.x) || O.cols[c.out] != zp(c.z))
            throw std::domain_error("block shapes do not chain: out " + std::to_string(c.out));
        Key4 k{c.out, c.x, c.y, c.z};
        auto it = mdict.find(k);
        if (it == mdict.end()) { mdict.emplace(k, ch.size()); ch.push_back(c); }
        else ch[it->second].c += c.c;
    }
    P.n_chains = (int64_t)ch.size();

    // algorithmic counts on the merged list
    {
        std::vector<char> ux(X.rows.size(), 0), uz(Z.rows.size(), 0), uo(O.rows.size(), 0);
        double bytes = 0;
        for (const Chain& c : ch) {
            P.flops_merged += chain_flops((double)xm(c.x), (double)xk(c.x), (double)Y.cols[c.y], (double)zp(c.z));
            if (!ux[c.x]) { ux[c.x] = 1; bytes += 8.0 * X.rows[c.x] * X.cols[c.x]; }
            if (!uz[c.z]) { uz[c.z] = 1; bytes += 8.0 * Z.rows[c.z] * Z.cols[c.z]; }
            if (!uo[c.out]) { uo[c.out] = 1; }
        }
        for (size_t i = 0; i < Y.rows.size(); ++i) bytes += 8.0 * Y.rows[i] * Y.cols[i];
        for (size_t i = 0; i < O.rows.size(); ++i) if (uo[i]) bytes += 8.0 * O.rows[i] * O.cols[i];
        P.bytes_alg = bytes;
        int64_t no = 0;
        for (char u : uo) no += u;
        P.n_out_blocks = no;
    }

    // ---- choose the association with fewer executed flops (shared intermediates counted once)
    double f_xy = 0, f_yz = 0;
    {
        std::unordered_map<Key4, char, Key4Hash> sxy, syz;
        for (const Chain& c : ch) {
            const double m = (double)xm(c.x), k = (double)xk(c.x), n = (double)Y.cols[c.y], p = (double)zp(c.z);
            if (sxy.emplace(Key4{c.x, c.y, 0, 0}, 1).second) f_xy += 2 * m * k * n;
            if (syz.emplace(Key4{c.y, c.z, 0, 0}, 1).second) f_yz += 2 * k * n * p;
        }
        // second stage after summing all first-stage products that share (out, Z) resp. (out, X)
        std::unordered_map<Key4, char, Key4Hash> oz, ox;
        for (const Chain& c : ch) {
            const double m = (double)xm(c.x), k = (double)xk(c.x), n = (double)Y.cols[c.y], p = (double)zp(c.z);
            if (oz.emplace(Key4{c.out, c.z, 0, 0}, 1).second) f_xy += 2 * m * n * p;
            if (ox.emplace(Key4{c.out, c.x, 0, 0}, 1).second) f_yz += 2 * m * k * p;
        }
    }
    P.association = (f_yz < f_xy) ? 1 : 0;

    // ---- intermediates
    std::unordered_map<Key4, int64_t, Key4Hash> idict;
    std::vector<std::pair<int64_t, int64_t>> ipairs;   // (x,y) or (y,z)
    std::vector<int64_t> trows, tcols;
    std::vector<int64_t> chain_t(ch.size());
    for (size_t i = 0; i < ch.size(); ++i) {
        const Chain& c = ch[i];
        Key4 k = P.association == 0 ? Key4{c.x, c.y, 0, 0} : Key4{c.y, c.z, 0, 0};
        auto it = idict.find(k);
        if (it == idict.end()) {
            int64_t id = (int64_t)ipairs.size();
            idict.emplace(k, id);
            if (P.association == 0) {
                ipairs.push_back({c.x, c.y});
                trows.push_back(xm(c.x));
                tcols.push_back(Y.cols[c.y]);
            } else {
                ipairs.push_back({c.y, c.z});
                trows.push_back(Y.rows[c.y]);
                tcols.push_back(zp(c.z));
            }
            chain_t[i] = id;
        } else chain_t[i] = it->second;
    }
    P.n_intermediates = (int64_t)ipairs.size();
    P.T = make_dev_layout(trows, tcols);

    // ---- phase 1: T = op(X)*Y  (association 0)  or  U = Y*op(Z)  (association 1)
    PhasePlan& p1 = P.p1;
    if (P.association == 0) {
        p1.slotA = SLOT_X; p1.transA = transX; p1.slotB = SLOT_Y; p1.transB = false;
    } else {
        p1.slotA = SLOT_Y; p1.transA = false; p1.slotB = SLOT_Z; p1.transB = transZ;
    }
    p1.slotC = SLOT_T;
    p1.transC = false;
    for (size_t j = 0; j < ipairs.size(); ++j) {
        int64_t a = ipairs[j].first, b = ipairs[j].second;
        const DevLayout& LA = P.association == 0 ? X : Y;
        const DevLayout& LB = P.association == 0 ? Y : Z;
        int64_t K = P.association == 0 ? xk(a) : Y.cols[a];
        GSeg s{};
        s.b_off = LB.off[b];
        s.ldb = (int32_t)LB.ld[b];
        s.lda = (int32_t)LA.ld[a];
        s.K = (int32_t)K;
        s.term_begin = (int32_t)p1.terms.size();
        s.term_count = 1;
        p1.terms.push_back(GTerm{LA.off[a], 1.0});
        int32_t sb = (int32_t)p1.segs.size();
        p1.segs.push_back(s);
        p1.flops += 2.0 * trows[j] * tcols[j] * K;
        add_tiles(p1, P.T.off[j], P.T.ld[j], trows[j], tcols[j], sb, sb + 1, tile_m, tile_n);
    }
    sort_tiles(p1);

    // ---- phase 2
    PhasePlan& p2 = P.p2;
    p2.slotC = SLOT_OUT;
    // group chains by output block, then by the operand that is not an intermediate
    std::vector<size_t> order(ch.size());
    std::iota(order.begin(), order.end(), 0);
    if (P.association == 0) {
        // out = sum_z (sum_t c_t T_t) * op(Z_z) ;  A = T (multi-term), B = op(Z)
        std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            if (ch[a].out != ch[b].out) return ch[a].out < ch[b].out;
            if (ch[a].z != ch[b].z) return ch[a].z < ch[b].z;
            return chain_t[a] < chain_t[b];
        });
        p2.slotA = SLOT_T; p2.transA = false; p2.slotB = SLOT_Z; p2.transB = transZ; p2.transC = false;
    } else {
        // out^T = sum_x (sum_t c_t U_t)^T * op(X_x)^T ;  A = U^T (multi-term), B = op(X)^T, C stored transposed
        std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            if (ch[a].out != ch[b].out) return ch[a].out < ch[b].out;
            if (ch[a].x != ch[b].x) return ch[a].x < ch[b].x;
            return chain_t[a] < chain_t[b];
        });
        p2.slotA = SLOT_T; p2.transA = true; p2.slotB = SLOT_X; p2.transB = !transX; p2.transC = true;
    }
    size_t i = 0;
    while (i < order.size()) {
        const int64_t o = ch[order[i]].out;
        int32_t sb = (int32_t)p2.segs.size();
        size_t j = i;
        while (j < order.size() && ch[order[j]].out == o) {
            const int64_t other = P.association == 0 ? ch[order[j]].z : ch[order[j]].x;
            GSeg s{};
            s.term_begin = (int32_t)p2.terms.size();
            size_t jj = j;
            while (jj < order.size() && ch[order[jj]].out == o &&
                   (P.association == 0 ? ch[order[jj]].z : ch[order[jj]].x) == other) {
                const int64_t t = chain_t[order[jj]];
                if (!p2.terms.empty() && (int32_t)p2.terms.size() > s.term_begin && p2.terms.back().off == P.T.off[t])
                    p2.terms.back().coef += ch[order[jj]].c;
                else
                    p2.terms.push_back(GTerm{P.T.off[t], ch[order[jj]].c});
                s.lda = (int32_t)P.T.ld[t];
                ++jj;
            }
            const int32_t tend = (int32_t)p2.terms.size();
            if (P.association == 0) {
                s.b_off = Z.off[other];
                s.ldb = (int32_t)Z.ld[other];
                s.K = (int32_t)zn(other);
            } else {
                s.b_off = X.off[other];
                s.ldb = (int32_t)X.ld[other];
                s.K = (int32_t)xk(other);
            }
            // a segment carries at most kMaxTerms terms: longer sums become several
            // segments with the same B operand
            for (int32_t tb = s.term_begin; tb < tend; tb += kMaxTerms) {
                GSeg part = s;
                part.term_begin = tb;
                part.term_count = std::min<int32_t>(kMaxTerms, tend - tb);
                p2.segs.push_back(part);
            }
            j = jj;
        }
        int32_t se = (int32_t)p2.segs.size();
        // tile space: association 0 -> (m x p) of out; association 1 -> (p x m) (transposed store)
        const int64_t m = O.rows[o], p = O.cols[o];
        double kk = 0, kt = 0;
        for (int32_t s = sb; s < se; ++s) { kk += p2.segs[s].K; kt += (double)p2.segs[s].K * p2.segs[s].term_count; }
        p2.flops += 2.0 * m * p * kk;
        P.flops_p2_unsummed += 2.0 * m * p * kt;
        if (P.association == 0) add_tiles(p2, O.off[o], O.ld[o], m, p, sb, se, tile_m, tile_n);
        else add_tiles(p2, O.off[o], O.ld[o], p, m, sb, se, tile_m, tile_n);
        i = j;
    }
    // output blocks that receive no product are still written (with zeros), as the
    // reference's OxV starts from a zeroed copy of Vin (pivot/DmrgPivotMatrix1.h:127,134)
    {
        std::vector<char> seen(O.rows.size(), 0);
        for (const Chain& c : ch) seen[c.out] = 1;
        const int32_t sb = (int32_t)p2.segs.size();
        for (size_t o = 0; o < O.rows.size(); ++o)
            if (!seen[o]) {
                if (P.association == 0) add_tiles(p2, O.off[o], O.ld[o], O.rows[o], O.cols[o], sb, sb, tile_m, tile_n);
                else add_tiles(p2, O.off[o], O.ld[o], O.cols[o], O.rows[o], sb, sb, tile_m, tile_n);
            }
    }
    sort_tiles(p2);
    return P;
}

// ===========================================================================
// split-precision planner
// ===========================================================================
Plan make_split_plan(const ChainSet& cs, const DevLayout& X, const DevLayout& Y, const DevLayout& Z,
                     const DevLayout& O, bool transX, bool transZ, int nrhs, const SplitTiling& tiling, bool tf32) {
    if (nrhs < 1) throw std::invalid_argument("nrhs must be at least 1");
    for (int cap : {tiling.ncap1, tiling.ncap2})
        if (cap < 32 || cap > kUmmaTileN || cap % 32 != 0)
            throw std::invalid_argument("tile N caps must be multiples of 32 up to 256");
    if (tiling.splitk < 1 || tiling.splitk > 8 || (tiling.splitk > 1 && nrhs > 1))
        throw std::invalid_argument("split-K of 1..8, single right-hand side only");
    if (tf32 && nrhs > 1) throw std::invalid_argument("3xTF32 plans take one right-hand side");
    Plan P;
    P.splitk = tiling.splitk;
    P.elt = tf32 ? 4 : 2;
    P.kstep = tf32 ? 16 : kUmmaBK;
    P.split = true;
    P.association = 0;
    P.nrhs = nrhs;
    P.vstride = O.total;
    P.ycolsP.resize(Y.rows.size());
    for (size_t y = 0; y < Y.rows.size(); ++y)
        P.ycolsP[y] = (int32_t)(nrhs > 1 ? (Y.cols[y] + 31) / 32 * 32 : Y.cols[y]);
    auto ywide = [&](size_t y) { return (int64_t)nrhs * P.ycolsP[y]; };   // N of phase 1, K extent of T
    auto xm = [&](int64_t x) { return transX ? X.cols[x] : X.rows[x]; };
    auto xk = [&](int64_t x) { return transX ? X.rows[x] : X.cols[x]; };
    auto zn = [&](int64_t z) { return transZ ? Z.cols[z] : Z.rows[z]; };
    auto zp = [&](int64_t z) { return transZ ? Z.rows[z] : Z.cols[z]; };

    // merge duplicate chains
    std::unordered_map<Key4, size_t, Key4Hash> mdict;
    std::vector<Chain> ch;
    ch.reserve(cs.chains.size());
    for (const Chain& c : cs.chains) {
        if (c.out < 0 || c.out >= (int64_t)O.rows.size() || c.x < 0 || c.x >= (int64_t)X.rows.size() || c.y < 0 ||
            c.y >= (int64_t)Y.rows.size() || c.z < 0 || c.z >= (int64_t)Z.rows.size())
            throw std::invalid_argument("chain references a block outside its table");
        if (xk(c.x) != Y.rows[c.y] || Y.cols[c.y] != zn(c.z) || O.rows[c.out] != xm(c.x) || O.cols[c.out] != zp(c.z))
            throw std::domain_error("block shapes do not chain: out " + std::to_string(c.out));
        Key4 k{c.out, c.x, c.y, c.z};
        auto it = mdict.find(k);
        if (it == mdict.end()) { mdict.emplace(k, ch.size()); ch.push_back(c); }
        else ch[it->second].c += c.c;
    }
    P.n_chains = (int64_t)ch.size();
    {
        std::vector<char> ux(X.rows.size(), 0), uz(Z.rows.size(), 0), uo(O.rows.size(), 0);
        double bytes = 0;
        for (const Chain& c : ch) {
            P.flops_merged += chain_flops((double)xm(c.x), (double)xk(c.x), (double)Y.cols[c.y], (double)zp(c.z));
            if (!ux[c.x]) { ux[c.x] = 1; bytes += 8.0 * X.rows[c.x] * X.cols[c.x]; }
            if (!uz[c.z]) { uz[c.z] = 1; bytes += 8.0 * Z.rows[c.z] * Z.cols[c.z]; }
            uo[c.out] = 1;
        }
        for (size_t i = 0; i < Y.rows.size(); ++i) bytes += 8.0 * nrhs * Y.rows[i] * Y.cols[i];
        int64_t no = 0;
        for (size_t i = 0; i < O.rows.size(); ++i) if (uo[i]) { bytes += 8.0 * nrhs * O.rows[i] * O.cols[i]; ++no; }
        P.bytes_alg = bytes;
        P.n_out_blocks = no;
        P.flops_merged *= nrhs;
    }

    // panel arenas: blocks are added first (class and row), the class matrices
    // are laid out afterwards, then every block gets its element offset
    struct PanelBuilder {
        PanelArena a;
        std::map<int32_t, int32_t> cls_of_kpad;
        std::vector<OpBlock>* ops;
        int32_t add(int64_t outer, int64_t K) {
            const int32_t kp = panel_kpad(K);
            auto it = cls_of_kpad.find(kp);
            int32_t c;
            if (it == cls_of_kpad.end()) {
                c = (int32_t)a.cls.size();
                a.cls.push_back(PanelClass{kp, 0, 0});
                cls_of_kpad.emplace(kp, c);
            } else {
                c = it->second;
            }
            OpBlock b{};
            b.outer = (int32_t)outer;
            b.K = (int32_t)K;
            b.cls = c;
            b.row = (int32_t)a.cls[c].rows;
            b.pitch = 2 * kp;
            a.cls[c].rows += outer;
            ops->push_back(b);
            return (int32_t)ops->size() - 1;
        }
        void finish() {
            int64_t cur = 0;
            for (PanelClass& c : a.cls) {
                c.base = cur;
                // whole 128-byte rows; each class starts on a 1 KiB boundary
                cur = (cur + 2 * (int64_t)c.kpad * std::max<int64_t>(c.rows, 1) + 511) / 512 * 512;
            }
            a.total = std::max<int64_t>(cur, 512);
            for (OpBlock& b : *ops) b.off = a.cls[b.cls].base + (int64_t)b.row * b.pitch;
        }
    };

    // scaled copies c * op(Z) (n x p): panel rows are the p columns of op(Z)
    struct CZ { uint64_t cbits; int64_t z; bool operator==(const CZ& o) const { return cbits == o.cbits && z == o.z; } };
    struct CZH { size_t operator()(const CZ& a) const { return std::hash<uint64_t>()(a.cbits * 0x9E3779B97F4A7C15ull ^ (uint64_t)a.z); } };
    std::unordered_map<CZ, int32_t, CZH> zdict;
    PanelBuilder pz{{}, {}, &P.opZ};
    std::vector<int32_t> chain_zp(ch.size());
    std::vector<std::pair<int64_t, double>> zsrc;   // (z, c) of each prepared copy
    for (size_t i = 0; i < ch.size(); ++i) {
        uint64_t bits;
        std::memcpy(&bits, &ch[i].c, 8);
        CZ key{bits, ch[i].z};
        auto it = zdict.find(key);
        if (it != zdict.end()) { chain_zp[i] = it->second; continue; }
        const int32_t id = pz.add(zp(ch[i].z), zn(ch[i].z));
        zdict.emplace(key, id);
        zsrc.push_back({ch[i].z, ch[i].c});
        chain_zp[i] = id;
    }
    pz.finish();
    P.az = pz.a;
    for (size_t q = 0; q < zsrc.size(); ++q) {
        const int64_t z = zsrc[q].first;
        const OpBlock& ob = P.opZ[q];
        PrepBlock pb{};
        pb.src_off = Z.off[z]; pb.src_ld = (int32_t)Z.ld[z];
        pb.rows = (int32_t)Z.rows[z]; pb.cols = (int32_t)Z.cols[z];
        pb.dst_off = ob.off; pb.dst_ld = ob.pitch;
        pb.trans = transZ ? 1 : 0;   // op(Z) = Z: columns of Z become panel rows; op(Z) = Z^T: rows of Z
        pb.scale = zsrc[q].second;
        P.prepZ.push_back(pb);
    }

    // intermediates T_j = op(X_x) * Y_y (m x n), one per distinct (x, y).  All intermediates
    // of one V block y share B = Y_y and K: phase 1 computes them as one stacked GEMM
    // [op(X_x1); op(X_x2); ...] * Y_y = [T_j1; T_j2; ...], so op(X) is prepared once per
    // (x, y) in a per-y stack of the X panels, and the T_j of one y are consecutive panel rows.
    std::unordered_map<Key4, int64_t, Key4Hash> idict;
    std::vector<std::pair<int64_t, int64_t>> ipairs;
    std::vector<int64_t> chain_t(ch.size());
    for (size_t i = 0; i < ch.size(); ++i) {
        Key4 k{ch[i].x, ch[i].y, 0, 0};
        auto it = idict.find(k);
        if (it != idict.end()) { chain_t[i] = it->second; continue; }
        const int64_t id = (int64_t)ipairs.size();
        idict.emplace(k, id);
        ipairs.push_back({ch[i].x, ch[i].y});
        chain_t[i] = id;
    }
    P.n_intermediates = (int64_t)ipairs.size();
    std::vector<std::vector<int64_t>> by_y(Y.rows.size());
    for (size_t j = 0; j < ipairs.size(); ++j) by_y[ipairs[j].second].push_back((int64_t)j);
    std::vector<int64_t> stack_rows(Y.rows.size(), 0), row_in_stack(ipairs.size(), 0);
    for (size_t y = 0; y < Y.rows.size(); ++y)
        for (int64_t j : by_y[y]) {
            row_in_stack[j] = stack_rows[y];
            stack_rows[y] += xm(ipairs[j].first);
        }

    // X panels: one stack per V block with intermediates
    PanelBuilder px{{}, {}, &P.opX};
    std::vector<int32_t> xstack(Y.rows.size(), -1);
    for (size_t y = 0; y < Y.rows.size(); ++y)
        if (!by_y[y].empty()) xstack[y] = px.add(stack_rows[y], Y.rows[y]);
    px.finish();
    P.ax = px.a;
    for (size_t y = 0; y < Y.rows.size(); ++y)
        for (int64_t j : by_y[y]) {
            const int64_t x = ipairs[j].first;
            const OpBlock& ob = P.opX[xstack[y]];
            PrepBlock pb{};
            pb.src_off = X.off[x]; pb.src_ld = (int32_t)X.ld[x];
            pb.rows = (int32_t)X.rows[x]; pb.cols = (int32_t)X.cols[x];
            pb.dst_off = ob.off + row_in_stack[j] * ob.pitch; pb.dst_ld = ob.pitch;
            pb.trans = transX ? 0 : 1;   // op(X) = X: rows of X become panel rows; op(X) = X^T: columns of X
            pb.scale = 1.0;
            P.prepX.push_back(pb);
        }

    // T panels: the same stacks; T_j is rows [row_in_stack, +m) of its y's stack
    std::vector<OpBlock> tstacks;
    PanelBuilder pt{{}, {}, &tstacks};
    std::vector<int32_t> tstack(Y.rows.size(), -1);
    // (multi-RHS: R*stack rows of K = ycolsP, the rows of rhs k interleaved at R*i + k)
    for (size_t y = 0; y < Y.rows.size(); ++y)
        if (!by_y[y].empty()) tstack[y] = pt.add((int64_t)nrhs * stack_rows[y], P.ycolsP[y]);
    pt.finish();
    P.at = pt.a;
    P.opT.resize(ipairs.size());
    for (size_t j = 0; j < ipairs.size(); ++j) {
        const OpBlock& sk = tstacks[tstack[ipairs[j].second]];
        OpBlock b = sk;
        b.outer = (int32_t)(nrhs * xm(ipairs[j].first));
        b.row = sk.row + (int32_t)(nrhs * row_in_stack[j]);
        b.off = sk.off + (int64_t)nrhs * row_in_stack[j] * sk.pitch;
        P.opT[j] = b;
    }

    // the vector Y in panels: panel rows are its columns, K = its rows
    PanelBuilder py{{}, {}, &P.opY};
    for (size_t y = 0; y < Y.rows.size(); ++y) py.add(ywide(y), Y.rows[y]);
    py.finish();
    P.ay = py.a;

    // phase 1: per V block y, [T_j1; T_j2; ...] = [op(X_x1); ...] * Y_y  (A rows = sum m, B rows = n,
    // K = k), written into T's panel stack
    PhasePlan& p1 = P.p1;
    p1.slotA = SLOT_X; p1.slotB = SLOT_Y; p1.slotC = SLOT_T;
    p1.transA = false; p1.transB = false; p1.transC = true;
    for (size_t y = 0; y < Y.rows.size(); ++y) {
        if (by_y[y].empty()) continue;
        const OpBlock& sx = P.opX[xstack[y]];
        const OpBlock& st = tstacks[tstack[y]];
        GSeg s{};
        s.term_begin = (int32_t)p1.terms.size();
        s.term_count = 1;
        p1.terms.push_back(GTerm{sx.off, 1.0});
        s.K = (int32_t)Y.rows[y];
        const int32_t sb = (int32_t)p1.segs.size();
        p1.segs.push_back(s);
        p1.seg_amap.push_back(xstack[y]);
        p1.seg_bmap.push_back((int32_t)y);
        p1.flops += 2.0 * stack_rows[y] * nrhs * Y.cols[y] * s.K;
        // column tiles start on panel K steps (multiples of 32): the epilogue writes whole row segments
        const size_t t0 = p1.tiles.size();
        add_tiles(p1, st.off, st.pitch, stack_rows[y], ywide(y), sb, sb + 1, kUmmaTileM, tiling.ncap1, 32);
        for (size_t t = t0; t < p1.tiles.size(); ++t) {
            p1.tiles[t].rstride = P.ycolsP[y];
            p1.tiles[t].nrhs = nrhs;
        }
    }
    sort_tiles(p1);

    // phase 2: out_o = sum over chains T_t * (c op(Z_z))  (K-concatenation, one segment per chain)
    PhasePlan& p2 = P.p2;
    p2.slotA = SLOT_T; p2.slotB = SLOT_Z; p2.slotC = SLOT_OUT;
    p2.transA = false; p2.transB = false; p2.transC = false;
    std::vector<size_t> order(ch.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        if (ch[a].out != ch[b].out) return ch[a].out < ch[b].out;
        if (ch[a].z != ch[b].z) return ch[a].z < ch[b].z;
        return chain_t[a] < chain_t[b];
    });
    // (multi-RHS: the tiles span R*m interleaved rows, row R*i + k of output block o
    // being row i of vector k's block o; one tile serves every right-hand side)
    std::vector<char> seen(O.rows.size(), 0);
    auto mark = [&](size_t t0) {
        for (size_t t = t0; t < p2.tiles.size(); ++t) p2.tiles[t].nrhs = nrhs;
    };
    const int nsk = tiling.splitk;
    // tiles of output block o for segments [sb, se): split-K cuts the segment list
    // into nsk parts of about equal K (part j -> element offset j * vstride of the
    // partial buffer); parts without segments write zeros
    auto block_tiles = [&](int64_t o, int32_t sb, int32_t se) {
        const size_t t0 = p2.tiles.size();
        if (nsk == 1) {
            add_tiles(p2, O.off[o], O.ld[o], (int64_t)nrhs * O.rows[o], O.cols[o], sb, se, kUmmaTileM, tiling.ncap2);
        } else {
            double ktot = 0;
            for (int32_t q = sb; q < se; ++q) ktot += p2.segs[q].K;
            int32_t a = sb;
            double acc = 0;
            for (int j = 0; j < nsk; ++j) {
                int32_t b = a;
                const double goal = ktot * (j + 1) / nsk;
                while (b < se && (j == nsk - 1 || acc + 0.5 * p2.segs[b].K <= goal)) acc += p2.segs[b++].K;
                add_tiles(p2, O.off[o] + (int64_t)j * P.vstride, O.ld[o], O.rows[o], O.cols[o], a, b, kUmmaTileM,
                          tiling.ncap2);
                a = b;
            }
        }
        mark(t0);
    };
    size_t i = 0;
    while (i < order.size()) {
        const int64_t o = ch[order[i]].out;
        seen[o] = 1;
        const int32_t sb = (int32_t)p2.segs.size();
        double kk = 0;
        while (i < order.size() && ch[order[i]].out == o) {
            const size_t c = order[i];
            const int64_t t = chain_t[c], zq = chain_zp[c];
            const int64_t y = ipairs[t].second;
            GSeg s{};
            s.term_begin = (int32_t)p2.terms.size();
            s.term_count = 1;
            p2.terms.push_back(GTerm{P.opT[t].off, 1.0});
            s.K = (int32_t)Y.cols[y];
            kk += s.K;
            p2.segs.push_back(s);
            p2.seg_amap.push_back((int32_t)t);
            p2.seg_bmap.push_back((int32_t)zq);
            ++i;
        }
        p2.flops += 2.0 * nrhs * O.rows[o] * O.cols[o] * kk;
        block_tiles(o, sb, (int32_t)p2.segs.size());
    }
    P.flops_p2_unsummed = p2.flops;
    const int32_t sb = (int32_t)p2.segs.size();
    for (size_t o = 0; o < O.rows.size(); ++o)
        if (!seen[o]) block_tiles((int64_t)o, sb, sb);
    sort_tiles(p2);
    return P;
}

}  // namespace vmps
