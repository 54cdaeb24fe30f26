// Quantum-number algebra for the host-side task-list builder.
//
// A QN is up to four int components; each component fuses either additively
// (U(1), symmetry/U1.h:170-176, triangle :476-482) or as an SU(2) irrep label
// q = 2S+1 (symmetry/SU2.h:174-183, triangle :548-554).  Products of components
// behave like S1xS2 (symmetry/S1xS2.h:192-208, :729-743): fusion is the
// cartesian product of the component fusions and every SU(2)-type coefficient is
// the product of the per-component coefficients (U(1) components contribute 1).
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <functional>
#include <stdexcept>
#include <vector>

namespace vmps {

constexpr int kMaxNq = 4;

struct QN {
    std::array<int32_t, kMaxNq> v{0, 0, 0, 0};
    bool operator==(const QN& o) const { return v == o.v; }
    bool operator!=(const QN& o) const { return v != o.v; }
    bool operator<(const QN& o) const { return v < o.v; }   // lexicographic, as qarray::operator<
};

struct QNHash {
    size_t operator()(const QN& q) const {
        uint64_t h = 1469598103934665603ull;
        for (int i = 0; i < kMaxNq; ++i) { h ^= (uint32_t)q.v[i] + 0x9e3779b9u; h *= 1099511628211ull; }
        return (size_t)h;
    }
};
template <int N> struct QNTuple {
    std::array<QN, N> q;
    bool operator==(const QNTuple& o) const { return q == o.q; }
};
template <int N> struct QNTupleHash {
    size_t operator()(const QNTuple<N>& t) const {
        size_t h = 0;
        for (int i = 0; i < N; ++i) h = h * 1000003u ^ QNHash()(t.q[i]);
        return h;
    }
};
using QN2 = QNTuple<2>;
using QN3 = QNTuple<3>;

// ---- SU(2) recoupling symbols (Racah formula), arguments are 2j ------------
// Published closed forms (Racah 1942; Edmonds, "Angular Momentum in Quantum
// Mechanics", eqs. 6.3.7 and 6.4.3).  The reference takes them from GSL
// gsl_sf_coupling_{6,9}j or wigxjpf (symmetry/SU2Wrappers.h:71-119), called with
// q-1 = 2S; the same convention is used here.
double coupling_6j(int two_j1, int two_j2, int two_j3, int two_j4, int two_j5, int two_j6);
double coupling_9j(int two_j1, int two_j2, int two_j3, int two_j4, int two_j5, int two_j6,
                   int two_j7, int two_j8, int two_j9);

struct Symmetry {
    int nq = 1;
    std::array<int, kMaxNq> kind{0, 0, 0, 0};   // 0 = U1, 1 = SU2

    bool nonabelian() const {
        for (int i = 0; i < nq; ++i) if (kind[i] == 1) return true;
        return false;
    }
    QN vacuum() const {
        QN q;
        for (int i = 0; i < nq; ++i) q.v[i] = kind[i] == 1 ? 1 : 0;
        return q;
    }
    QN flip(const QN& a) const {   // U1: -q, SU2: q (symmetry/U1.h:63, SU2.h:70)
        QN q = a;
        for (int i = 0; i < nq; ++i) if (kind[i] == 0) q.v[i] = -a.v[i];
        return q;
    }
    // all irreps of a (x) b, in the order of S1xS2::reduceSilent (first component outermost)
    std::vector<QN> reduce(const QN& a, const QN& b) const {
        std::vector<QN> out(1, QN{});
        for (int i = 0; i < nq; ++i) {
            std::vector<int> vals;
            if (kind[i] == 0) vals.push_back(a.v[i] + b.v[i]);
            else for (int x = std::abs(a.v[i] - b.v[i]) + 1; x <= std::abs(a.v[i] + b.v[i]) - 1; x += 2) vals.push_back(x);
            std::vector<QN> nxt;
            nxt.reserve(out.size() * vals.size());
            for (const auto& q : out) for (int x : vals) { QN r = q; r.v[i] = x; nxt.push_back(r); }
            out.swap(nxt);
        }
        return out;
    }
    // validate({a,b,c}): c in a (x) b
    bool triangle(const QN& a, const QN& b, const QN& c) const {
        for (int i = 0; i < nq; ++i) {
            if (kind[i] == 0) { if (a.v[i] + b.v[i] != c.v[i]) return false; }
            else if (!(c.v[i] - 1 >= std::abs(a.v[i] - b.v[i]) && c.v[i] - 1 <= a.v[i] + b.v[i] - 2)) return false;
        }
        return true;
    }
    // coeff_dot (symmetry/SU2.h:284-290): multiplet dimension of the SU(2) components
    double coeff_dot(const QN& q) const {
        double r = 1.0;
        for (int i = 0; i < nq; ++i) if (kind[i] == 1) r *= (double)q.v[i];
        return r;
    }
    // 9j-type prefactor: coupling_9j * sqrt(q7 q8 q3 q6) [* q9/q7 for buildR]
    // coeff_HPsi  symmetry/SU2.h:508-519, coeff_buildL :481-492, coeff_buildR :494-506,
    // coeff_tensorProd :455-466
    double coeff_9j_family(const QN* q, bool buildR) const {
        double r = 1.0;
        for (int i = 0; i < nq; ++i) {
            if (kind[i] != 1) continue;
            int a[9];
            for (int j = 0; j < 9; ++j) a[j] = q[j].v[i];
            double c = coupling_9j(a[0] - 1, a[1] - 1, a[2] - 1, a[3] - 1, a[4] - 1, a[5] - 1,
                                   a[6] - 1, a[7] - 1, a[8] - 1) *
                       std::sqrt((double)a[6] * a[7] * a[2] * a[5]);
            if (buildR) c *= (double)a[8] / (double)a[6];
            r *= c;
        }
        return r;
    }
    double coeff_HPsi(const QN* q9) const { return coeff_9j_family(q9, false); }
    double coeff_buildL(const QN* q9) const { return coeff_9j_family(q9, false); }
    double coeff_buildR(const QN* q9) const { return coeff_9j_family(q9, true); }
    double coeff_tensorProd(const QN* q9) const { return coeff_9j_family(q9, false); }
    // coeff_Apair symmetry/SU2.h:388-397
    double coeff_Apair(const QN* q) const {
        double r = 1.0;
        for (int i = 0; i < nq; ++i) {
            if (kind[i] != 1) continue;
            int a[6];
            for (int j = 0; j < 6; ++j) a[j] = q[j].v[i];
            double c = coupling_6j(a[0] - 1, a[1] - 1, a[2] - 1, a[3] - 1, a[4] - 1, a[5] - 1) *
                       std::sqrt((double)a[2] * a[5]);
            int ph = (a[0] + a[1] + a[3] + a[4] - 4) / 2;
            if (ph & 1) c = -c;
            r *= c;
        }
        return r;
    }
};

}  // namespace vmps

namespace std {
template <> struct hash<vmps::QN> { size_t operator()(const vmps::QN& q) const { return vmps::QNHash()(q); } };
}
