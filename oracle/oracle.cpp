// ORACLE -- test infrastructure only.
//
// CPU restatement (FP64) of the VMPS effective-Hamiltonian path, used as the
// checker for the GPU engine and as the timed CPU baseline.  It follows the
// reference loops literally (no merging, no sharing of intermediate products):
//
//   precalc_blockStructure 1-site   tensors/DmrgIndexGymnastics.h:487-590 (LAWA :32-77)
//   precalc_blockStructure 2-site   tensors/DmrgIndexGymnastics.h:699-856 (AAWWAA :198-262)
//   OxV(PivotMatrix1)               pivot/DmrgPivotMatrix1.h:131-287
//   OxV(PivotMatrix2)               pivot/DmrgPivotMatrix2.h:85-247
//   HxV(PivotMatrix0)               pivot/DmrgPivotMatrix0.h:31-96
//   contract_L / contract_R (FULL)  tensors/DmrgContractions.h:34-311 (AWAR :79-124)
//   optimal_multiply / mult_cost    DmrgExternal.h:141-215
//   Qbasis::combine / leftOffset    tensors/Qbasis.h:438-463, :685-798
//
// Products inside OxV are evaluated as Eigen evaluates `L * V * R`, i.e.
// (L*V)*R; PivotMatrix0 and contract_L/R use the optimal_multiply rule.
// Parallelism: OpenMP over output blocks, as DMRG_PIVOT1_PARALLELIZE /
// DMRG_PIVOT2_PARALLELIZE do (pivot/DmrgPivotMatrix1.h:219-222).
//
// GEMM: the OpenBLAS library bundled with numpy when its path is handed in
// (oracle_set_blas), else a plain cache-blocked triple loop.
//
// Symmetries: products of U(1) and SU(2) components (oracle_set_symmetry), as
// Sym::S1xS2 composes them (symmetry/S1xS2.h).  SU(2) quantum numbers are
// q = 2S+1; fusion |q1-q2|+1 .. q1+q2-1 step 2 (SU2::reduceSilent,
// symmetry/SU2.h:174-183); the prefactors are the reference's coefficient
// families (symmetry/SU2.h:388-519) evaluated per SU(2) component and
// multiplied (U(1) components contribute 1):
//   coeff_HPsi / coeff_buildL / coeff_tensorProd = 9j * sqrt(q7 q8 q3 q6)
//   coeff_buildR = 9j * sqrt(q7 q8 q3 q6) * q9 / q7
//   coeff_Apair  = 6j * sqrt(q3 q6) * (-1)^((q1+q2+q4+q5-4)/2)
// with the 6j / 9j symbols of SU2Wrappers.h:72-120 (GSL's arguments are 2j = q-1).
#include <dlfcn.h>
#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

namespace {

typedef std::array<int, 4> Q;

struct Tab {   // parsed block table
    int64_t n = 0;
    std::vector<Q> qin, qout, qmid;
    std::vector<int> leg;
    std::vector<int64_t> rows, cols, off;
};

Tab read_tab(int nq, int64_t n, const int32_t* qin, const int32_t* qout, const int32_t* qmid, const int32_t* leg,
             const int64_t* rows, const int64_t* cols, const int64_t* off) {
    Tab t;
    t.n = n;
    for (int64_t i = 0; i < n; ++i) {
        Q a{0, 0, 0, 0}, b{0, 0, 0, 0}, c{0, 0, 0, 0};
        for (int k = 0; k < nq; ++k) {
            a[k] = qin[i * nq + k];
            b[k] = qout[i * nq + k];
            if (qmid) c[k] = qmid[i * nq + k];
        }
        t.qin.push_back(a);
        t.qout.push_back(b);
        t.qmid.push_back(c);
        t.leg.push_back(leg[i]);
        t.rows.push_back(rows[i]);
        t.cols.push_back(cols[i]);
        t.off.push_back(off[i]);
    }
    return t;
}

// unused QN components are zero everywhere

// ---- symmetry: component kinds (0 = U(1), 1 = SU(2)) ----------------------------
int g_nq = 1;
int g_kind[4] = {0, 0, 0, 0};
bool g_nonabelian = false;

// Symmetry::reduceSilent(a, b): all fusion outcomes, components varied from the
// first (outermost) to the last
std::vector<Q> fuse(const Q& a, const Q& b) {
    std::vector<Q> out{Q{0, 0, 0, 0}};
    for (int k = 0; k < g_nq; ++k) {
        std::vector<Q> nxt;
        for (const Q& p : out) {
            if (g_kind[k] == 0) {
                Q r = p; r[k] = a[k] + b[k]; nxt.push_back(r);
            } else {
                for (int q = std::abs(a[k] - b[k]) + 1; q <= a[k] + b[k] - 1; q += 2) { Q r = p; r[k] = q; nxt.push_back(r); }
            }
        }
        out.swap(nxt);
    }
    return out;
}
// Symmetry::flip: U(1) -q, SU(2) q
Q flipq(const Q& a) { Q r = a; for (int k = 0; k < g_nq; ++k) if (g_kind[k] == 0) r[k] = -a[k]; return r; }
// Symmetry::validate({a, b, c}): c is among the fusion outcomes of a and b
bool tri(const Q& a, const Q& b, const Q& c) {
    for (int k = 0; k < g_nq; ++k) {
        if (g_kind[k] == 0) { if (a[k] + b[k] != c[k]) return false; }
        else if (c[k] < std::abs(a[k] - b[k]) + 1 || c[k] > a[k] + b[k] - 1 || ((a[k] + b[k] + c[k]) % 2) == 0) return false;
    }
    for (int k = g_nq; k < 4; ++k) if (a[k] + b[k] != c[k]) return false;
    return true;
}

// ---- 6j and 9j symbols (arguments 2j) ---------------------------------------------
// Racah's single-sum formula with the factorials themselves in long double (the
// arguments stay small: a sum of four 2j values below ~60), 9j as the sum over x of
// (2x+1) times three 6j (the standard reduction).
long double fact(int n) {
    static std::vector<long double> f;
    if (f.empty()) { f.resize(171); f[0] = 1; for (int i = 1; i < 171; ++i) f[i] = f[i - 1] * i; }
    return f[n];
}
bool tri2(int a, int b, int c) {
    return a >= 0 && b >= 0 && c >= 0 && ((a + b + c) % 2 == 0) && c >= std::abs(a - b) && c <= a + b;
}
long double delta2(int a, int b, int c) {
    return std::sqrt(fact((a + b - c) / 2) * fact((a - b + c) / 2) * fact((-a + b + c) / 2) / fact((a + b + c) / 2 + 1));
}
double sixj(int a, int b, int c, int d, int e, int f) {   // {a/2 b/2 c/2; d/2 e/2 f/2}
    if (!tri2(a, b, c) || !tri2(a, e, f) || !tri2(d, b, f) || !tri2(d, e, c)) return 0.0;
    const int t1 = (a + b + c) / 2, t2 = (a + e + f) / 2, t3 = (d + b + f) / 2, t4 = (d + e + c) / 2;
    const int u1 = (a + b + d + e) / 2, u2 = (b + c + e + f) / 2, u3 = (c + a + f + d) / 2;
    const int zmin = std::max(std::max(t1, t2), std::max(t3, t4)), zmax = std::min(u1, std::min(u2, u3));
    long double sum = 0;
    for (int z = zmin; z <= zmax; ++z) {
        long double term = fact(z + 1) / (fact(z - t1) * fact(z - t2) * fact(z - t3) * fact(z - t4) * fact(u1 - z) *
                                          fact(u2 - z) * fact(u3 - z));
        sum += (z % 2) ? -term : term;
    }
    return (double)(sum * delta2(a, b, c) * delta2(a, e, f) * delta2(d, b, f) * delta2(d, e, c));
}
double ninej(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
    if (!tri2(a, b, c) || !tri2(d, e, f) || !tri2(g, h, i) || !tri2(a, d, g) || !tri2(b, e, h) || !tri2(c, f, i))
        return 0.0;
    const int xmin = std::max(std::abs(a - i), std::max(std::abs(d - h), std::abs(b - f)));
    const int xmax = std::min(a + i, std::min(d + h, b + f));
    long double sum = 0;
    for (int x = xmin; x <= xmax; x += 2) {
        long double t = (long double)(x + 1) * sixj(a, d, g, h, i, x) * sixj(b, e, h, d, x, f) * sixj(c, f, i, x, a, b);
        sum += (x % 2) ? -t : t;
    }
    return (double)sum;
}
// the coefficient families, product over the SU(2) components (q = 2S+1)
double c9(const Q* q, int form) {   // form 0: HPsi / buildL / tensorProd, 1: buildR
    double out = 1.0;
    for (int k = 0; k < g_nq; ++k) {
        if (g_kind[k] != 1) continue;
        double v = ninej(q[0][k] - 1, q[1][k] - 1, q[2][k] - 1, q[3][k] - 1, q[4][k] - 1, q[5][k] - 1, q[6][k] - 1,
                         q[7][k] - 1, q[8][k] - 1) *
                   std::sqrt((double)q[6][k] * q[7][k] * q[2][k] * q[5][k]);
        if (form == 1) v *= (double)q[8][k] / (double)q[6][k];
        out *= v;
    }
    return out;
}
double c9(const Q& q1, const Q& q2, const Q& q3, const Q& q4, const Q& q5, const Q& q6, const Q& q7, const Q& q8,
          const Q& q9, int form = 0) {
    const Q q[9] = {q1, q2, q3, q4, q5, q6, q7, q8, q9};
    return c9(q, form);
}
double capair(const Q& q1, const Q& q2, const Q& q3, const Q& q4, const Q& q5, const Q& q6) {
    double out = 1.0;
    for (int k = 0; k < g_nq; ++k) {
        if (g_kind[k] != 1) continue;
        const int ph = (q1[k] + q2[k] + q4[k] + q5[k] - 4) / 2;
        out *= sixj(q1[k] - 1, q2[k] - 1, q3[k] - 1, q4[k] - 1, q5[k] - 1, q6[k] - 1) * std::sqrt((double)q3[k] * q6[k]) *
               ((ph % 2) ? -1.0 : 1.0);
    }
    return out;
}
constexpr double kCgcEps = 2.220446049250313e-16;   // mynumeric_limits<double>::epsilon()

// ---- GEMM ------------------------------------------------------------------
typedef void (*dgemm_t)(const char*, const char*, const int64_t*, const int64_t*, const int64_t*, const double*,
                        const double*, const int64_t*, const double*, const int64_t*, const double*, double*,
                        const int64_t*, size_t, size_t);
dgemm_t g_dgemm = nullptr;

// C (m x n) = alpha * op(A) * op(B) + beta * C, column-major
void gemm(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
          const double* B, int64_t ldb, double beta, double* Cm, int64_t ldc) {
    if (m == 0 || n == 0) return;
    if (g_dgemm) {
        const char TA = ta ? 'T' : 'N', TB = tb ? 'T' : 'N';
        g_dgemm(&TA, &TB, &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, Cm, &ldc, 1, 1);
        return;
    }
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) Cm[i + j * ldc] = beta == 0.0 ? 0.0 : beta * Cm[i + j * ldc];
    const int64_t KB = 128, IB = 64;
    std::vector<double> at(IB * KB);
    for (int64_t k0 = 0; k0 < k; k0 += KB) {
        const int64_t kb = std::min(KB, k - k0);
        for (int64_t i0 = 0; i0 < m; i0 += IB) {
            const int64_t ib = std::min(IB, m - i0);
            for (int64_t kk = 0; kk < kb; ++kk)
                for (int64_t ii = 0; ii < ib; ++ii)
                    at[kk * IB + ii] = ta ? A[(k0 + kk) + (i0 + ii) * lda] : A[(i0 + ii) + (k0 + kk) * lda];
            for (int64_t j = 0; j < n; ++j) {
                double* c = Cm + i0 + j * ldc;
                for (int64_t kk = 0; kk < kb; ++kk) {
                    const double bv = alpha * (tb ? B[j + (k0 + kk) * ldb] : B[(k0 + kk) + j * ldb]);
                    const double* a = &at[kk * IB];
                    for (int64_t ii = 0; ii < ib; ++ii) c[ii] += a[ii] * bv;
                }
            }
        }
    }
}

struct Mat {   // owned dense column-major matrix
    int64_t r = 0, c = 0;
    std::vector<double> d;
    void resize(int64_t rr, int64_t cc) { r = rr; c = cc; d.assign(rr * cc, 0.0); }
};
struct View { const double* p; int64_t r, c; bool t; };   // op(M): t = adjoint (real: transpose)
inline int64_t vr(const View& v) { return v.t ? v.c : v.r; }
inline int64_t vc(const View& v) { return v.t ? v.r : v.c; }

// out += alpha * A * B * C with the chain order of optimal_multiply (DmrgExternal.h:190-215)
// mode 0: optimal rule, mode 1: (A*B)*C always (Eigen's evaluation of A*B*C)
void triple(int mode, double alpha, const View& A, const View& B, const View& Cv, double* out, int64_t ldo) {
    const int64_t m = vr(A), k = vc(A), n = vc(B), p = vc(Cv);
    const uint64_t c0 = (uint64_t)m * k * n + (uint64_t)m * Cv.r * Cv.c;   // (AB)C
    const uint64_t c1 = (uint64_t)k * n * p + (uint64_t)m * k * p;          // A(BC)
    Mat t;
    if (mode == 1 || c0 <= c1) {
        t.resize(m, n);
        gemm(A.t, B.t, m, n, k, 1.0, A.p, A.r, B.p, B.r, 0.0, t.d.data(), m);
        gemm(false, Cv.t, m, p, n, alpha, t.d.data(), m, Cv.p, Cv.r, 1.0, out, ldo);
    } else {
        t.resize(k, p);
        gemm(B.t, Cv.t, k, p, n, 1.0, B.p, B.r, Cv.p, Cv.r, 0.0, t.d.data(), k);
        gemm(A.t, false, m, p, k, alpha, A.p, A.r, t.d.data(), k, 1.0, out, ldo);
    }
}

// ---- reference containers ---------------------------------------------------
typedef std::array<Q, 2> Q2;
typedef std::array<Q, 3> Q3;
struct Tripod {   // Multipede<3>: dict {in,out,mid} -> block index; block[q][a] -> table row
    std::vector<Q3> keys;
    std::map<Q3, int> dict;
    std::vector<std::map<int, int64_t>> aux;
};
Tripod tripod(const Tab& t) {
    Tripod T;
    for (int64_t i = 0; i < t.n; ++i) {
        Q3 k{t.qin[i], t.qout[i], t.qmid[i]};
        auto it = T.dict.find(k);
        int q;
        if (it == T.dict.end()) { q = (int)T.keys.size(); T.dict[k] = q; T.keys.push_back(k); T.aux.emplace_back(); }
        else q = it->second;
        T.aux[q][t.leg[i]] = i;
    }
    return T;
}
int64_t aux_at(const Tripod& T, int q, int a) {
    auto it = T.aux[q].find(a);
    return it == T.aux[q].end() ? -1 : it->second;
}
struct BipedVec { std::vector<std::map<Q2, int64_t>> dict; };
BipedVec bipeds(const Tab& t, int nleg) {
    BipedVec b;
    int m = nleg;
    for (int64_t i = 0; i < t.n; ++i) m = std::max(m, t.leg[i] + 1);
    b.dict.resize(m);
    for (int64_t i = 0; i < t.n; ++i) b.dict[t.leg[i]][Q2{t.qin[i], t.qout[i]}] = i;
    return b;
}
int64_t bfind(const BipedVec& b, int s, const Q& x, const Q& y) {
    if (s < 0 || s >= (int)b.dict.size()) return -1;
    auto it = b.dict[s].find(Q2{x, y});
    return it == b.dict[s].end() ? -1 : it->second;
}
struct Nz { int row, col; double val; };
struct Mpo {
    int nloc, nop;
    std::vector<Q> qloc, qop;
    // W[s1][s2][k] : Biped {qin,qout} -> sparse block
    std::vector<std::map<Q2, std::vector<Nz>>> W;
    const std::vector<Nz>* find(int s1, int s2, int k, const Q& a, const Q& b) const {
        const auto& m = W[((size_t)s1 * nloc + s2) * nop + k];
        auto it = m.find(Q2{a, b});
        return it == m.end() ? nullptr : &it->second;
    }
};
Mpo read_mpo(int nq, int64_t nnz, const int32_t* s1, const int32_t* s2, const int32_t* k, const int32_t* qin,
             const int32_t* qout, const int32_t* row, const int32_t* col, const double* val, int nloc,
             const int32_t* qloc, int nop, const int32_t* qop) {
    Mpo m;
    m.nloc = nloc;
    m.nop = nop;
    auto rd = [&](const int32_t* p, int64_t i) { Q q{0, 0, 0, 0}; for (int c = 0; c < nq; ++c) q[c] = p[i * nq + c]; return q; };
    for (int i = 0; i < nloc; ++i) m.qloc.push_back(rd(qloc, i));
    for (int i = 0; i < nop; ++i) m.qop.push_back(rd(qop, i));
    m.W.resize((size_t)nloc * nloc * nop);
    for (int64_t i = 0; i < nnz; ++i)
        m.W[((size_t)s1[i] * nloc + s2[i]) * nop + k[i]][Q2{rd(qin, i), rd(qout, i)}].push_back(Nz{row[i], col[i], val[i]});
    return m;
}

// ---- precalc results (the reference's qlhs / qrhs / factor_cgcs) ---------------
struct Task1 { int s2; int64_t q2; int qL, qR, k; Q2 qW; double cgc; };
struct Task2 { int64_t q24; int qL, qR; int s1, s2, k12; Q2 qW12; int s3, s4, k34; Q2 qW34; double cgc; };

struct Pivot {
    int kind = 1;
    Tab L, R, V;
    Tripod Lt, Rt;
    Mpo W12, W34;
    std::vector<int64_t> qlhs;   // output block (table row of V)
    std::vector<std::vector<Task1>> qrhs1;
    std::vector<std::vector<Task2>> qrhs2;
    const double* Ld = nullptr;
    const double* Rd = nullptr;
    std::vector<double> Lcopy, Rcopy;
    int64_t n_tasks = 0;
};

// precalc_blockStructure, 1-site (tensors/DmrgIndexGymnastics.h:487-590) with LAWA (:32-77)
void precalc1(Pivot& P) {
    const Mpo& W = P.W12;
    BipedVec Vb = bipeds(P.V, W.nloc);
    std::map<int64_t, std::vector<Task1>> lookup;
    for (int s1 = 0; s1 < W.nloc; ++s1)
    for (int s2 = 0; s2 < W.nloc; ++s2)
    for (int k = 0; k < W.nop; ++k) {
        if (!tri(W.qloc[s2], W.qop[k], W.qloc[s1])) continue;
        for (int qL = 0; qL < (int)P.Lt.keys.size(); ++qL) {
            const Q Lin = P.Lt.keys[qL][0], Lout = P.Lt.keys[qL][1], Lmid = P.Lt.keys[qL][2];
            for (const Q& Rout : fuse(Lin, W.qloc[s1])) {
                int64_t qAbra = bfind(Vb, s1, Lin, Rout);
                if (qAbra < 0) continue;
                for (const Q& Rin : fuse(Lout, W.qloc[s2])) {
                    int64_t qAket = bfind(Vb, s2, Lout, Rin);
                    if (qAket < 0) continue;
                    for (const Q& Rmid : fuse(Lmid, W.qop[k])) {
                        const auto* nz = W.find(s1, s2, k, Lmid, Rmid);
                        if (!nz || !tri(Rin, Rmid, Rout)) continue;
                        auto itR = P.Rt.dict.find(Q3{Rin, Rout, Rmid});
                        if (itR == P.Rt.dict.end()) continue;
                        bool empty = true;
                        for (const auto& e : *nz)
                            if (aux_at(P.Lt, qL, e.row) >= 0 && aux_at(P.Rt, itR->second, e.col) >= 0) empty = false;
                        if (empty) continue;
                        const double cgc = g_nonabelian ? c9(Lout, W.qloc[s2], Rin, Lmid, W.qop[k], Rmid, Lin,
                                                             W.qloc[s1], Rout)
                                                        : 1.0;
                        if (std::abs(cgc) < kCgcEps) continue;
                        lookup[qAbra].push_back(Task1{s2, qAket, qL, itR->second, k, Q2{Lmid, Rmid}, cgc});
                    }
                }
            }
        }
    }
    for (auto& kv : lookup) {
        P.qlhs.push_back(kv.first);
        P.n_tasks += (int64_t)kv.second.size();
        P.qrhs1.push_back(std::move(kv.second));
    }
}

// combined two-site index of Qbasis::combine + outer_num + leftOffset
// (tensors/Qbasis.h:438-463, :685-798): key (s1, s3, merged QN) -> combined index
std::map<std::tuple<int, int, Q>, int> combine_index(const std::vector<Q>& q12, const std::vector<Q>& q34) {
    // distinct QNs and inner indices in order of appearance (Qbasis::pullData)
    auto pull = [](const std::vector<Q>& qs, std::vector<Q>& dq, std::vector<int>& dd, std::vector<int>& inner) {
        for (const Q& q : qs) {
            auto it = std::find(dq.begin(), dq.end(), q);
            size_t d = it - dq.begin();
            if (it == dq.end()) { dq.push_back(q); dd.push_back(0); }
            inner.push_back(dd[d]++);
        }
    };
    std::vector<Q> d1, d2;
    std::vector<int> n1, n2, i1, i2;
    pull(q12, d1, n1, i1);
    pull(q34, d2, n2, i2);
    // history per merged QN: the source pairs (q1, q2), sorted; merged QNs in sorted order
    std::map<Q, std::vector<std::tuple<Q, Q, int, int>>> hist;
    for (size_t a = 0; a < d1.size(); ++a)
        for (size_t b = 0; b < d2.size(); ++b)
            for (const Q& qm : fuse(d1[a], d2[b])) hist[qm].push_back({d1[a], d2[b], n1[a], n2[b]});
    for (auto& kv : hist) std::sort(kv.second.begin(), kv.second.end());
    std::map<Q, int> start;
    int cur = 0;
    for (auto& kv : hist) {
        start[kv.first] = cur;
        for (auto& e : kv.second) cur += std::get<2>(e) * std::get<3>(e);
    }
    std::map<std::tuple<int, int, Q>, int> idx;
    for (size_t s1 = 0; s1 < q12.size(); ++s1)
        for (size_t s3 = 0; s3 < q34.size(); ++s3)
            for (const Q& qm : fuse(q12[s1], q34[s3])) {
                int off = 0;
                for (auto& e : hist[qm]) {
                    if (std::get<0>(e) == q12[s1] && std::get<1>(e) == q34[s3]) { off += i1[s1] + std::get<2>(e) * i2[s3]; break; }
                    off += std::get<2>(e) * std::get<3>(e);
                }
                idx[{(int)s1, (int)s3, qm}] = start[qm] + off;
            }
    return idx;
}

// precalc_blockStructure, 2-site (tensors/DmrgIndexGymnastics.h:699-856) with AAWWAA (:198-262)
void precalc2(Pivot& P) {
    const Mpo &W12 = P.W12, &W34 = P.W34;
    auto cidx = combine_index(W12.qloc, W34.qloc);
    int ncomb = 0;
    for (auto& kv : cidx) ncomb = std::max(ncomb, kv.second + 1);
    BipedVec Vb = bipeds(P.V, ncomb);
    std::map<int64_t, std::vector<Task2>> lookup;
    for (int s1 = 0; s1 < W12.nloc; ++s1)
    for (int s2 = 0; s2 < W12.nloc; ++s2)
    for (int k12 = 0; k12 < W12.nop; ++k12) {
        if (!tri(W12.qloc[s2], W12.qop[k12], W12.qloc[s1])) continue;
        for (int s3 = 0; s3 < W34.nloc; ++s3)
        for (int s4 = 0; s4 < W34.nloc; ++s4)
        for (int k34 = 0; k34 < W34.nop; ++k34) {
            if (!tri(W34.qloc[s4], W34.qop[k34], W34.qloc[s3])) continue;
            for (const Q& qOp : fuse(W12.qop[k12], W34.qop[k34]))
            for (const Q& qm13 : fuse(W12.qloc[s1], W34.qloc[s3]))
            for (const Q& qm24 : fuse(W12.qloc[s2], W34.qloc[s4])) {
                const int s1s3 = cidx[{s1, s3, qm13}], s2s4 = cidx[{s2, s4, qm24}];
                const double cgc9 = g_nonabelian ? c9(W12.qloc[s2], W34.qloc[s4], qm24, W12.qop[k12], W34.qop[k34], qOp,
                                                      W12.qloc[s1], W34.qloc[s3], qm13)
                                                 : 1.0;
                if (std::abs(cgc9) < kCgcEps) continue;
                for (int qL = 0; qL < (int)P.Lt.keys.size(); ++qL) {
                    const Q Lin = P.Lt.keys[qL][0], Lout = P.Lt.keys[qL][1], Lmid = P.Lt.keys[qL][2];
                    for (const Q& qRout : fuse(Lin, qm13)) {
                        int64_t q13 = bfind(Vb, s1s3, Lin, qRout);
                        if (q13 < 0) continue;
                        for (const Q& qRin : fuse(Lout, qm24)) {
                            int64_t q24 = bfind(Vb, s2s4, Lout, qRin);
                            if (q24 < 0) continue;
                            for (const Q& qW : fuse(Lmid, W12.qop[k12])) {
                                if (!W12.find(s1, s2, k12, Lmid, qW)) continue;
                                for (const Q& qRmid : fuse(qW, W34.qop[k34])) {
                                    if (!W34.find(s3, s4, k34, qW, qRmid)) continue;
                                    if (!tri(qRin, qRmid, qRout)) continue;
                                    const double cgc6 =
                                        g_nonabelian ? capair(Lmid, W12.qop[k12], qW, W34.qop[k34], qRmid, qOp) : 1.0;
                                    if (std::abs(cgc6) < kCgcEps) continue;
                                    auto itR = P.Rt.dict.find(Q3{qRin, qRout, qRmid});
                                    if (itR == P.Rt.dict.end()) continue;
                                    const double cgcH =
                                        g_nonabelian ? c9(Lout, qm24, qRin, Lmid, qOp, qRmid, Lin, qm13, qRout) : 1.0;
                                    lookup[q13].push_back(Task2{q24, qL, itR->second, s1, s2, k12, Q2{Lmid, qW}, s3, s4,
                                                                k34, Q2{qW, qRmid}, cgc6 * cgc9 * cgcH});
                                }
                            }
                        }
                    }
                }
            }
        }
    }
    for (auto& kv : lookup) {
        P.qlhs.push_back(kv.first);
        P.n_tasks += (int64_t)kv.second.size();
        P.qrhs2.push_back(std::move(kv.second));
    }
}

View blk(const Tab& t, const double* d, int64_t i, bool trans = false) {
    return View{d + t.off[i], t.rows[i], t.cols[i], trans};
}

// OxV(PivotMatrix1 / PivotMatrix2): Vout zeroed, then per output block sum over tasks
void oxv(const Pivot& P, const double* vin, double* vout) {
    int64_t tot = 0;
    for (int64_t i = 0; i < P.V.n; ++i) tot = std::max(tot, P.V.off[i] + P.V.rows[i] * P.V.cols[i]);
    std::fill(vout, vout + tot, 0.0);
#pragma omp parallel for schedule(dynamic)
    for (int64_t q = 0; q < (int64_t)P.qlhs.size(); ++q) {
        const int64_t o = P.qlhs[q];
        double* out = vout + P.V.off[o];
        const int64_t ldo = P.V.rows[o];
        if (P.kind == 1) {
            for (const Task1& t : P.qrhs1[q]) {
                // Vin[s2].block[q2] : needs the row s1 of W[s1][s2][k] -> recover s1 from the output leg
                const int s1 = P.V.leg[o];
                const auto* nz = P.W12.find(s1, t.s2, t.k, t.qW[0], t.qW[1]);
                if (!nz) continue;
                for (const auto& e : *nz) {
                    int64_t la = aux_at(P.Lt, t.qL, e.row), rb = aux_at(P.Rt, t.qR, e.col);
                    if (la < 0 || rb < 0) continue;
                    triple(1, t.cgc * e.val, blk(P.L, P.Ld, la), blk(P.V, vin, t.q2), blk(P.R, P.Rd, rb), out, ldo);
                }
            }
        } else {
            for (const Task2& t : P.qrhs2[q]) {
                const auto* nz12 = P.W12.find(t.s1, t.s2, t.k12, t.qW12[0], t.qW12[1]);
                const auto* nz34 = P.W34.find(t.s3, t.s4, t.k34, t.qW34[0], t.qW34[1]);
                if (!nz12 || !nz34) continue;
                for (const auto& e12 : *nz12)
                    for (const auto& e34 : *nz34) {
                        if (e12.col != e34.row) continue;
                        int64_t la = aux_at(P.Lt, t.qL, e12.row), rb = aux_at(P.Rt, t.qR, e34.col);
                        if (la < 0 || rb < 0) continue;
                        triple(1, t.cgc * e12.val * e34.val, blk(P.L, P.Ld, la), blk(P.V, vin, t.q24),
                               blk(P.R, P.Rd, rb), out, ldo);
                    }
            }
        }
    }
}

// HxV(PivotMatrix0)
void hxv0(const Pivot& P, const double* vin, double* vout) {
    int64_t tot = 0;
    for (int64_t i = 0; i < P.V.n; ++i) tot = std::max(tot, P.V.off[i] + P.V.rows[i] * P.V.cols[i]);
    std::fill(vout, vout + tot, 0.0);
    BipedVec Vb = bipeds(P.V, 1);
    for (int qL = 0; qL < (int)P.Lt.keys.size(); ++qL) {
        const Q Lin = P.Lt.keys[qL][0], Lout = P.Lt.keys[qL][1], Lmid = P.Lt.keys[qL][2];
        auto itR = P.Rt.dict.find(Q3{Lout, Lin, Lmid});
        if (itR == P.Rt.dict.end()) continue;
        int64_t qin = bfind(Vb, 0, Lout, Lout);
        if (qin < 0) continue;
        const Q Rout = P.Rt.keys[itR->second][1];
        int64_t qout = bfind(Vb, 0, Rout, Rout);
        if (qout < 0) continue;
        for (const auto& kv : P.Lt.aux[qL]) {
            int64_t ra = aux_at(P.Rt, itR->second, kv.first);
            if (ra < 0) continue;
            triple(0, 1.0, blk(P.L, P.Ld, kv.second), blk(P.V, vin, qin), blk(P.R, P.Rd, ra), vout + P.V.off[qout],
                   P.V.rows[qout]);
        }
    }
}

// contract_L / contract_R, FULL mode
struct Env {
    int side = 0, nq = 1;
    int mode = 0;              // CONTRACT_LR_MODE: 0 FULL, 1 TRIANGULAR, 2 FIXED_ROWS, 3 FIXED_COLS
    int64_t fixed_ab = 0;
    std::map<std::pair<Q, int>, int64_t> order;   // basis_order_map
    int64_t at(const Q& q, int i) const { return order.at(std::make_pair(q, i)); }
    Tab E, B, K;
    Mpo W;
    Tab out;   // output layout (creation order)
    struct Item { int64_t o; int64_t x, y, z; double c; };
    std::vector<std::vector<Item>> per_out;
};

void env_plan(Env& V) {
    Tripod Et = tripod(V.E);
    BipedVec Bb = bipeds(V.B, V.W.nloc), Kb = bipeds(V.K, V.W.nloc);
    std::map<std::pair<Q3, int>, int64_t> odict;
    std::vector<Env::Item> items;
    auto oblock = [&](const Q3& qu, int a, int64_t r, int64_t c) {
        auto key = std::make_pair(qu, a);
        auto it = odict.find(key);
        if (it != odict.end()) return it->second;
        int64_t id = V.out.n++;
        odict[key] = id;
        V.out.qin.push_back(qu[0]); V.out.qout.push_back(qu[1]); V.out.qmid.push_back(qu[2]);
        V.out.leg.push_back(a); V.out.rows.push_back(r); V.out.cols.push_back(c);
        V.out.off.push_back(id == 0 ? 0 : V.out.off[id - 1] + V.out.rows[id - 1] * V.out.cols[id - 1]);
        return id;
    };
    const Mpo& W = V.W;
    for (int s1 = 0; s1 < W.nloc; ++s1)
    for (int s2 = 0; s2 < W.nloc; ++s2)
    for (int k = 0; k < W.nop; ++k) {
        if (!tri(W.qloc[s2], W.qop[k], W.qloc[s1])) continue;
        for (int qE = 0; qE < (int)Et.keys.size(); ++qE) {
            const Q Ein = Et.keys[qE][0], Eout = Et.keys[qE][1], Emid = Et.keys[qE][2];
            if (V.side == 0) {
                // contract_L (tensors/DmrgContractions.h:34-158): LAWA, then the key {Rout, Rin, Rmid}
                for (const Q& Rout : fuse(Ein, W.qloc[s1])) {
                    int64_t qb = bfind(Bb, s1, Ein, Rout);
                    if (qb < 0) continue;
                    for (const Q& Rin : fuse(Eout, W.qloc[s2])) {
                        int64_t qk = bfind(Kb, s2, Eout, Rin);
                        if (qk < 0) continue;
                        for (const Q& Rmid : fuse(Emid, W.qop[k])) {
                            const auto* nz = W.find(s1, s2, k, Emid, Rmid);
                            if (!nz || !tri(Rin, Rmid, Rout)) continue;
                            const double cgc = g_nonabelian ? c9(Eout, W.qloc[s2], Rin, Emid, W.qop[k], Rmid, Ein,
                                                                 W.qloc[s1], Rout)
                                                            : 1.0;
                            if (std::abs(cgc) < kCgcEps) continue;
                            for (const auto& e : *nz) {
                                if (V.mode == 1 && !(V.at(Emid, e.row) > V.fixed_ab)) continue;
                                if (V.mode == 3 && V.at(Rmid, e.col) != V.fixed_ab) continue;
                                if (V.mode == 2 && V.at(Emid, e.row) != V.fixed_ab) continue;
                                int64_t la = aux_at(Et, qE, e.row);
                                if (la < 0) continue;
                                int64_t o = oblock(Q3{Rout, Rin, Rmid}, e.col, V.B.cols[qb], V.K.cols[qk]);
                                items.push_back(Env::Item{o, qb, la, qk, cgc * e.val});
                            }
                        }
                    }
                }
            } else {
                // contract_R (tensors/DmrgContractions.h:179-311): AWAR (DmrgIndexGymnastics.h:79-124),
                // then the key {Lout, Lin, Lmid}
                const Q Rin = Ein, Rout = Eout, Rmid = Emid;
                for (const Q& Lin : fuse(Rout, flipq(W.qloc[s1]))) {
                    int64_t qb = bfind(Bb, s1, Lin, Rout);
                    if (qb < 0) continue;
                    for (const Q& Lout : fuse(Rin, flipq(W.qloc[s2]))) {
                        int64_t qk = bfind(Kb, s2, Lout, Rin);
                        if (qk < 0) continue;
                        for (const Q& Lmid : fuse(Rmid, flipq(W.qop[k]))) {
                            const auto* nz = W.find(s1, s2, k, Lmid, Rmid);
                            if (!nz || !tri(Lout, Lmid, Lin)) continue;
                            const double cgc = g_nonabelian ? c9(Lout, W.qloc[s2], Rin, Lmid, W.qop[k], Rmid, Lin,
                                                                 W.qloc[s1], Rout, 1)
                                                            : 1.0;
                            if (std::abs(cgc) < kCgcEps) continue;
                            for (const auto& e : *nz) {
                                if (V.mode == 1 && !(V.fixed_ab > V.at(Rmid, e.col))) continue;
                                if (V.mode == 2 && V.at(Lmid, e.row) != V.fixed_ab) continue;
                                if (V.mode == 3 && V.at(Rmid, e.col) != V.fixed_ab) continue;
                                int64_t rb = aux_at(Et, qE, e.col);
                                if (rb < 0) continue;
                                int64_t o = oblock(Q3{Lout, Lin, Lmid}, e.row, V.K.rows[qk], V.B.rows[qb]);
                                items.push_back(Env::Item{o, qk, rb, qb, cgc * e.val});
                            }
                        }
                    }
                }
            }
        }
    }
    V.per_out.assign(V.out.n, {});
    for (const auto& it : items) V.per_out[it.o].push_back(it);
}

void env_run(const Env& V, const double* Ed, const double* Bd, const double* Kd, double* out) {
    int64_t tot = V.out.n ? V.out.off.back() + V.out.rows.back() * V.out.cols.back() : 0;
    std::fill(out, out + tot, 0.0);
#pragma omp parallel for schedule(dynamic)
    for (int64_t o = 0; o < V.out.n; ++o)
        for (const auto& it : V.per_out[o]) {
            if (V.side == 0)
                triple(0, it.c, blk(V.B, Bd, it.x, true), blk(V.E, Ed, it.y), blk(V.K, Kd, it.z), out + V.out.off[o],
                       V.out.rows[o]);
            else
                triple(0, it.c, blk(V.K, Kd, it.x), blk(V.E, Ed, it.y), blk(V.B, Bd, it.z, true), out + V.out.off[o],
                       V.out.rows[o]);
        }
}

}  // namespace

// ============================================================================
// C interface for ctypes (tests and the CPU baseline only)
// ============================================================================
extern "C" {

int oracle_set_blas(const char* path) {
    if (!path || !*path) { g_dgemm = nullptr; return 0; }
    void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    const char* names[] = {"scipy_dgemm_64_", "dgemm_64_", "dgemm_"};
    for (const char* n : names) {
        void* f = dlsym(h, n);
        if (f) {
            g_dgemm = (dgemm_t)f;
            typedef void (*setnt_t)(int);
            const char* tn[] = {"scipy_openblas_set_num_threads64_", "openblas_set_num_threads64_", "openblas_set_num_threads"};
            for (const char* t : tn) {
                void* g = dlsym(h, t);
                if (g) { ((setnt_t)g)(1); break; }
            }
            return std::string(n) == "dgemm_" ? 2 : 1;
        }
    }
    return -2;
}

// QN component kinds of the objects created next: 0 = U(1), 1 = SU(2)
void oracle_set_symmetry(int nq, const int32_t* kinds) {
    g_nq = std::max(1, std::min(nq, 4));
    g_nonabelian = false;
    for (int k = 0; k < 4; ++k) {
        g_kind[k] = (k < g_nq && kinds) ? kinds[k] : 0;
        if (g_kind[k] == 1) g_nonabelian = true;
    }
}
double oracle_coupling_6j(int a, int b, int c, int d, int e, int f) { return sixj(a, b, c, d, e, f); }
double oracle_coupling_9j(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
    return ninej(a, b, c, d, e, f, g, h, i);
}

void oracle_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
int oracle_max_threads(void) { return omp_get_max_threads(); }

void* oracle_pivot_create(int kind, int nq, int64_t nL, const int32_t* Lqin, const int32_t* Lqout, const int32_t* Lqmid,
                          const int32_t* Lleg, const int64_t* Lrows, const int64_t* Lcols, const int64_t* Loff,
                          const double* Ldata, int64_t nR, const int32_t* Rqin, const int32_t* Rqout,
                          const int32_t* Rqmid, const int32_t* Rleg, const int64_t* Rrows, const int64_t* Rcols,
                          const int64_t* Roff, const double* Rdata, int64_t nV, const int32_t* Vqin,
                          const int32_t* Vqout, const int32_t* Vleg, const int64_t* Vrows, const int64_t* Vcols,
                          const int64_t* Voff,
                          // W12 (or W) and W34 (kind 2)
                          int64_t nnz1, const int32_t* a_s1, const int32_t* a_s2, const int32_t* a_k,
                          const int32_t* a_qin, const int32_t* a_qout, const int32_t* a_row, const int32_t* a_col,
                          const double* a_val, int a_nloc, const int32_t* a_qloc, int a_nop, const int32_t* a_qop,
                          int64_t nnz2, const int32_t* b_s1, const int32_t* b_s2, const int32_t* b_k,
                          const int32_t* b_qin, const int32_t* b_qout, const int32_t* b_row, const int32_t* b_col,
                          const double* b_val, int b_nloc, const int32_t* b_qloc, int b_nop, const int32_t* b_qop) {
    Pivot* P = new Pivot();
    P->kind = kind;
    P->L = read_tab(nq, nL, Lqin, Lqout, Lqmid, Lleg, Lrows, Lcols, Loff);
    P->R = read_tab(nq, nR, Rqin, Rqout, Rqmid, Rleg, Rrows, Rcols, Roff);
    P->V = read_tab(nq, nV, Vqin, Vqout, nullptr, Vleg, Vrows, Vcols, Voff);
    P->Lt = tripod(P->L);
    P->Rt = tripod(P->R);
    int64_t lt = 0, rt = 0;
    for (int64_t i = 0; i < nL; ++i) lt = std::max(lt, Loff[i] + Lrows[i] * Lcols[i]);
    for (int64_t i = 0; i < nR; ++i) rt = std::max(rt, Roff[i] + Rrows[i] * Rcols[i]);
    P->Lcopy.assign(Ldata, Ldata + lt);
    P->Rcopy.assign(Rdata, Rdata + rt);
    P->Ld = P->Lcopy.data();
    P->Rd = P->Rcopy.data();
    if (kind != 0)
        P->W12 = read_mpo(nq, nnz1, a_s1, a_s2, a_k, a_qin, a_qout, a_row, a_col, a_val, a_nloc, a_qloc, a_nop, a_qop);
    if (kind == 2)
        P->W34 = read_mpo(nq, nnz2, b_s1, b_s2, b_k, b_qin, b_qout, b_row, b_col, b_val, b_nloc, b_qloc, b_nop, b_qop);
    if (kind == 1) precalc1(*P);
    else if (kind == 2) precalc2(*P);
    return P;
}

int64_t oracle_pivot_tasks(void* h) { return ((Pivot*)h)->n_tasks; }

void oracle_hxv(void* h, const double* vin, double* vout) {
    Pivot* P = (Pivot*)h;
    if (P->kind == 0) hxv0(*P, vin, vout);
    else oxv(*P, vin, vout);
}

void oracle_pivot_destroy(void* h) { delete (Pivot*)h; }

void* oracle_env_create(int side, int nq, int64_t nE, const int32_t* Eqin, const int32_t* Eqout, const int32_t* Eqmid,
                        const int32_t* Eleg, const int64_t* Erows, const int64_t* Ecols, const int64_t* Eoff,
                        int64_t nB, const int32_t* Bqin, const int32_t* Bqout, const int32_t* Bleg,
                        const int64_t* Brows, const int64_t* Bcols, const int64_t* Boff, int64_t nK,
                        const int32_t* Kqin, const int32_t* Kqout, const int32_t* Kleg, const int64_t* Krows,
                        const int64_t* Kcols, const int64_t* Koff, int64_t nnz, const int32_t* s1, const int32_t* s2,
                        const int32_t* k, const int32_t* qin, const int32_t* qout, const int32_t* row,
                        const int32_t* col, const double* val, int nloc, const int32_t* qloc, int nop,
                        const int32_t* qop, int mode, int64_t fixed_ab, int64_t n_order, const int32_t* order_qn,
                        const int32_t* order_index, const int64_t* order_value) {
    Env* V = new Env();
    V->side = side;
    V->nq = nq;
    V->mode = mode;
    V->fixed_ab = fixed_ab;
    for (int64_t i = 0; i < n_order; ++i) {
        Q q{0, 0, 0, 0};
        for (int c = 0; c < nq; ++c) q[c] = order_qn[i * nq + c];
        V->order[std::make_pair(q, order_index[i])] = order_value[i];
    }
    V->E = read_tab(nq, nE, Eqin, Eqout, Eqmid, Eleg, Erows, Ecols, Eoff);
    V->B = read_tab(nq, nB, Bqin, Bqout, nullptr, Bleg, Brows, Bcols, Boff);
    V->K = read_tab(nq, nK, Kqin, Kqout, nullptr, Kleg, Krows, Kcols, Koff);
    V->W = read_mpo(nq, nnz, s1, s2, k, qin, qout, row, col, val, nloc, qloc, nop, qop);
    env_plan(*V);
    return V;
}

int64_t oracle_env_nblocks(void* h) { return ((Env*)h)->out.n; }

void oracle_env_layout(void* h, int32_t* qin, int32_t* qout, int32_t* qmid, int32_t* leg, int64_t* rows, int64_t* cols,
                       int64_t* off) {
    Env* V = (Env*)h;
    const int nq = V->nq;
    for (int64_t i = 0; i < V->out.n; ++i) {
        for (int c = 0; c < nq; ++c) {
            qin[i * nq + c] = V->out.qin[i][c];
            qout[i * nq + c] = V->out.qout[i][c];
            qmid[i * nq + c] = V->out.qmid[i][c];
        }
        leg[i] = V->out.leg[i];
        rows[i] = V->out.rows[i];
        cols[i] = V->out.cols[i];
        off[i] = V->out.off[i];
    }
}

void oracle_env_run(void* h, const double* E, const double* B, const double* K, double* out) {
    env_run(*(Env*)h, E, B, K, out);
}

void oracle_env_destroy(void* h) { delete (Env*)h; }

}  // extern "C"
