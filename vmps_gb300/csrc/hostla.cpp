// Host dense linear algebra of the two-site sweep: the truncated SVD of
// split_AA2 (tensors/DmrgContractions.h:2461-2631, with Biped::truncateSVD,
// tensors/Biped.h:744-932), abelian quantum numbers.
//
// For every middle QN qmid the two-site tensor's blocks form one sector matrix
//     Psi[(s1, qin), (s3, qout)] = V[s13(s1, s3)](qin, qout),  qin + q(s1) = qmid;
// its singular values and the orthonormal factor the sweep direction keeps come
// from the eigendecomposition of the Gram matrix (Psi Psi^T for a move to the
// right, Psi^T Psi to the left).  The Dmax largest singular values over all
// sectors are kept (none below eps_svd times the largest), renormalised, and the
// two site tensors are assembled in the block order of a site layout
// (for s, for qin in sorted order, qout = qin + q(s) if present).
//
// Small sectors (tens to a few hundred rows) are cheaper on the Grace cores than
// on the GPU at GB300's FP64 rate: LAPACK / BLAS, the ILP64 routines of the
// OpenBLAS that numpy bundles (bound at run time from the path the caller
// passes), one sector per host thread, largest first.  With a device context
// (vmps_two_site_split_device) the sectors whose Gram matrix has order >=
// VMPS_SPLIT_GPU_MIN (512 by default) may run on the GPU in FP64 instead -- the
// Gram matrix (cuBLAS dsyrk, DMMA), its eigensystem (cuSOLVER dsyevd) and the
// non-orthonormal factor (cuBLAS dgemm) -- on a thread of their own while the
// host threads factor the rest; which of them do is decided by estimated costs
// (assign_device_sectors), or VMPS_SPLIT_DEVICE=all sends every one of them.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <limits>
#include <map>
#include <array>
#include <unordered_map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "vmps_gb300.h"

namespace vmps {
void set_last_error_message(const std::string& msg);   // runtime.cpp
cudaStream_t ctx_stream(vmps_ctx* c);                 // runtime.cpp: the context's compute stream
int ctx_device(const vmps_ctx* c);
std::shared_ptr<void>& ctx_la_slot(vmps_ctx* c);      // per-context state of this file
}

namespace {

int set_err(int code, const std::string& msg) {
    vmps::set_last_error_message(msg);
    return code;
}

// a block table the host routines may read: arrays present, shapes positive, offsets non-negative
bool table_ok(const vmps_blocks* t) {
    if (t->nblocks < 0) return false;
    if (t->nblocks == 0) return true;
    if (!t->qin || !t->qout || !t->leg || !t->rows || !t->cols || !t->offset) return false;
    for (int64_t i = 0; i < t->nblocks; ++i)
        if (t->rows[i] <= 0 || t->cols[i] <= 0 || t->offset[i] < 0 || t->leg[i] < 0) return false;
    return true;
}

using lint = int64_t;   // ILP64 LAPACK integers
typedef void (*dsyevd_fn)(const char*, const char*, const lint*, double*, const lint*, double*, double*, const lint*,
                          lint*, const lint*, lint*, size_t, size_t);
typedef void (*dsyev_fn)(const char*, const char*, const lint*, double*, const lint*, double*, double*, const lint*,
                         lint*, size_t, size_t);
typedef void (*dsytrd_fn)(const char*, const lint*, double*, const lint*, double*, double*, double*, double*,
                          const lint*, lint*, size_t);
typedef void (*dsterf_fn)(const lint*, double*, double*, lint*);
typedef void (*dstemr_fn)(const char*, const char*, const lint*, double*, double*, const double*, const double*,
                          const lint*, const lint*, lint*, double*, double*, const lint*, const lint*, lint*, lint*,
                          double*, const lint*, lint*, const lint*, lint*, size_t, size_t);
typedef void (*dormtr_fn)(const char*, const char*, const char*, const lint*, const lint*, const double*, const lint*,
                          const double*, double*, const lint*, double*, const lint*, lint*, size_t, size_t, size_t);
typedef void (*dgeqrf_fn)(const lint*, const lint*, double*, const lint*, double*, double*, const lint*, lint*);
typedef void (*dorgqr_fn)(const lint*, const lint*, const lint*, double*, const lint*, const double*, double*,
                          const lint*, lint*);
typedef void (*dsyrk_fn)(const char*, const char*, const lint*, const lint*, const double*, const double*, const lint*,
                         const double*, double*, const lint*, size_t, size_t);
typedef void (*dgemm_fn)(const char*, const char*, const lint*, const lint*, const lint*, const double*, const double*,
                         const lint*, const double*, const lint*, const double*, double*, const lint*, size_t, size_t);

struct Lapack {
    dsyevd_fn syevd = nullptr;
    dsyev_fn syev = nullptr;
    dsytrd_fn sytrd = nullptr;
    dsterf_fn sterf = nullptr;
    dstemr_fn stemr = nullptr;
    dormtr_fn ormtr = nullptr;
    dsyrk_fn syrk = nullptr;
    dgemm_fn gemm = nullptr;
    dgeqrf_fn geqrf = nullptr;   // the QR gauge step
    dorgqr_fn orgqr = nullptr;
    bool ok() const { return syevd && syev && sytrd && sterf && stemr && ormtr && syrk && gemm && geqrf && orgqr; }
};

// Gram matrices below order kSelectMin get their full eigensystem at once: QR
// iteration (dsyev) below kSyevdMin, divide and conquer (dsyevd) above.  Larger
// ones are reduced to tridiagonal form first; after the truncation only the kept
// eigenvectors are computed (dstemr) and back-transformed (dormtr).  In the
// two-site split about a quarter of each large sector is kept (rank of the middle
// bond), and on the 16 Grace cores concurrent dsyevd calls contend inside
// OpenBLAS's level-3 kernels: an order-64 dsyevd took 0.28 ms alone and 2.1 ms
// with 16 threads busy, where dsyev went from 0.40 to 1.0 ms.  Measured per
// D=1024 bond (sectors up to order 178): 7.8 ms with full eigensystems against
// 9.0 ms selected; per D=4096 bond (up to 772): 0.114 s against 0.106 s.
constexpr int64_t kSyevdMin = 128, kSelectMin = 256;
Lapack g_lapack;
std::mutex g_lapack_mu;

void* find_symbol(void* h, const char* base) {
    for (const char* pre : {"scipy_", ""}) {
        for (const char* suf : {"_64_", "64_"}) {
            const std::string name = std::string(pre) + base + suf;
            if (void* p = dlsym(h, name.c_str())) return p;
        }
    }
    return nullptr;
}

// quantum numbers (at most 4 components) packed into one key whose integer order
// is the lexicographic order of the components (first component most significant)
using QN = std::array<int32_t, 4>;
using QKey = uint64_t;
QKey qkey(const QN& q, int nq) {
    QKey k = 0;
    for (int i = 0; i < nq; ++i) {
        if (q[(size_t)i] <= -32768 || q[(size_t)i] >= 32768) throw std::invalid_argument("quantum number out of range");
        k = (k << 16) | (QKey)(uint16_t)(q[(size_t)i] + 32768);
    }
    return k;
}
QN qload(const int32_t* p, int nq) {
    QN q{0, 0, 0, 0};
    for (int i = 0; i < nq; ++i) q[(size_t)i] = p[i];
    return q;
}

struct Sector {
    QN q;
    uint64_t key = 0;
    int64_t rows = 0, cols = 0;
    std::vector<double> M;        // rows x cols, column-major
    int64_t n = 0;                // Gram matrix order
    std::vector<double> G;        // Householder reflectors of the tridiagonal reduction (n x n)
    std::vector<double> tau, d, e;
    std::vector<double> S;        // singular values, descending (min(rows, cols))
    std::vector<double> Q;        // eigenvectors of the Gram matrix, descending (n x n, then n x kept)
    bool full = false;            // Q holds the full eigensystem (small sectors)
    bool gpu = false;             // factorised on the device
    int64_t kept = 0;
    std::string err;
};

// ---- device path of the large sectors ------------------------------------------
// One per context: cuBLAS and cuSOLVER handles on the context's stream and device
// buffers grown to the largest sector seen.  Used by one thread at a time (the
// split's device thread).
struct GpuLa {
    int device = -1;
    cudaStream_t st = nullptr;
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t sol = nullptr;
    double *M = nullptr, *G = nullptr, *W = nullptr, *Q = nullptr, *F = nullptr, *work = nullptr;
    int* info = nullptr;
    size_t cM = 0, cG = 0, cW = 0, cQ = 0, cF = 0, cwork = 0;
    std::mutex mu;
    ~GpuLa() {
        for (double* p : {M, G, W, Q, F, work}) if (p) cudaFree(p);
        if (info) cudaFree(info);
        if (sol) cusolverDnDestroy(sol);
        if (blas) cublasDestroy(blas);
    }
};
void cu_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
void blas_check(cublasStatus_t e, const char* what) {
    if (e != CUBLAS_STATUS_SUCCESS) throw std::runtime_error(std::string(what) + ": cuBLAS status " + std::to_string((int)e));
}
void sol_check(cusolverStatus_t e, const char* what) {
    if (e != CUSOLVER_STATUS_SUCCESS)
        throw std::runtime_error(std::string(what) + ": cuSOLVER status " + std::to_string((int)e));
}
// grow a device buffer to n doubles (contents are not kept)
void dgrow(double*& p, size_t& cap, size_t n) {
    if (cap >= n && p) return;
    if (p) { cudaFree(p); p = nullptr; cap = 0; }
    cu_check(cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(double)), "cudaMalloc (split)");
    cap = std::max<size_t>(n, 1);
}

GpuLa& gpu_la(vmps_ctx* ctx) {
    std::shared_ptr<void>& slot = vmps::ctx_la_slot(ctx);
    if (!slot) {
        auto g = std::make_shared<GpuLa>();
        g->device = vmps::ctx_device(ctx);
        g->st = vmps::ctx_stream(ctx);
        cu_check(cudaSetDevice(g->device), "cudaSetDevice");
        blas_check(cublasCreate(&g->blas), "cublasCreate");
        blas_check(cublasSetStream(g->blas, g->st), "cublasSetStream");
        sol_check(cusolverDnCreate(&g->sol), "cusolverDnCreate");
        sol_check(cusolverDnSetStream(g->sol, g->st), "cusolverDnSetStream");
        cu_check(cudaMalloc((void**)&g->info, sizeof(int)), "cudaMalloc (split)");
        slot = g;
    }
    return *static_cast<GpuLa*>(slot.get());
}

// values pass of a sector on the device: Gram matrix (dsyrk), full eigensystem
// (dsyevd, ascending), copied back as S (descending square roots) and Q (all
// eigenvectors, descending)
void gpu_factor_values(GpuLa& g, Sector& s, bool right) {
    const int64_t r = s.rows, c = s.cols, n = right ? r : c, k = right ? c : r;
    s.n = n;
    dgrow(g.M, g.cM, (size_t)(r * c));
    dgrow(g.G, g.cG, (size_t)(n * n));
    dgrow(g.W, g.cW, (size_t)n);
    cu_check(cudaMemcpyAsync(g.M, s.M.data(), sizeof(double) * (size_t)(r * c), cudaMemcpyHostToDevice, g.st),
             "upload sector");
    const double one = 1.0, zero = 0.0;
    blas_check(cublasDsyrk(g.blas, CUBLAS_FILL_MODE_LOWER, right ? CUBLAS_OP_N : CUBLAS_OP_T, (int)n, (int)k, &one,
                           g.M, (int)r, &zero, g.G, (int)n),
               "cublasDsyrk");
    int lwork = 0;
    sol_check(cusolverDnDsyevd_bufferSize(g.sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)n, g.G, (int)n,
                                          g.W, &lwork),
              "cusolverDnDsyevd_bufferSize");
    dgrow(g.work, g.cwork, (size_t)lwork);
    sol_check(cusolverDnDsyevd(g.sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)n, g.G, (int)n, g.W,
                               g.work, lwork, g.info),
              "cusolverDnDsyevd");
    std::vector<double> w((size_t)n), Z((size_t)(n * n));
    int info = 0;
    cu_check(cudaMemcpyAsync(w.data(), g.W, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, g.st), "download");
    cu_check(cudaMemcpyAsync(Z.data(), g.G, sizeof(double) * (size_t)(n * n), cudaMemcpyDeviceToHost, g.st),
             "download");
    cu_check(cudaMemcpyAsync(&info, g.info, sizeof(int), cudaMemcpyDeviceToHost, g.st), "download");
    cu_check(cudaStreamSynchronize(g.st), "split stream");
    if (info != 0) {
        s.err = "device eigensolver failed (info " + std::to_string(info) + ")";
        return;
    }
    const int64_t m = std::min(r, c);
    s.S.resize((size_t)m);
    s.Q.resize((size_t)(n * n));
    for (int64_t j = 0; j < n; ++j) {
        const int64_t src = n - 1 - j;
        std::memcpy(s.Q.data() + (size_t)(j * n), Z.data() + (size_t)(src * n), sizeof(double) * (size_t)n);
        if (j < m) s.S[(size_t)j] = std::sqrt(std::max(w[(size_t)src], 0.0));
    }
    s.full = true;
    s.gpu = true;
}

// the non-orthonormal factor of a device sector: scale U_k^T Psi (right, k x c) or
// scale Psi V_k (left, r x k) by dgemm on the device
void gpu_factor_product(GpuLa& g, Sector& s, bool right, double scale, std::vector<double>& F) {
    const int64_t r = s.rows, c = s.cols, n = s.n, k = s.kept;
    dgrow(g.M, g.cM, (size_t)(r * c));
    dgrow(g.Q, g.cQ, (size_t)(n * k));
    const size_t fsz = (size_t)(right ? k * c : r * k);
    dgrow(g.F, g.cF, fsz);
    cu_check(cudaMemcpyAsync(g.M, s.M.data(), sizeof(double) * (size_t)(r * c), cudaMemcpyHostToDevice, g.st),
             "upload sector");
    cu_check(cudaMemcpyAsync(g.Q, s.Q.data(), sizeof(double) * (size_t)(n * k), cudaMemcpyHostToDevice, g.st),
             "upload eigenvectors");
    const double zero = 0.0;
    if (right)
        blas_check(cublasDgemm(g.blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)k, (int)c, (int)r, &scale, g.Q, (int)n, g.M,
                               (int)r, &zero, g.F, (int)k),
                   "cublasDgemm");
    else
        blas_check(cublasDgemm(g.blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)r, (int)k, (int)c, &scale, g.M, (int)r, g.Q,
                               (int)n, &zero, g.F, (int)r),
                   "cublasDgemm");
    F.assign(fsz, 0.0);
    cu_check(cudaMemcpyAsync(F.data(), g.F, sizeof(double) * fsz, cudaMemcpyDeviceToHost, g.st), "download");
    cu_check(cudaStreamSynchronize(g.st), "split stream");
}

// Gram matrix of a sector (move right: M M^T, rows x rows; else M^T M), lower triangle
void gram(Sector& s, bool right, std::vector<double>& G) {
    const lint r = s.rows, n = s.n, k = right ? s.cols : s.rows;
    const double one = 1.0, zero = 0.0;
    G.assign((size_t)(n * n), 0.0);
    g_lapack.syrk("L", right ? "N" : "T", &n, &k, &one, s.M.data(), &r, &zero, G.data(), &n, 1, 1);
}

// values pass: tridiagonal reduction of the Gram matrix (kept for the vectors
// pass) and all its eigenvalues; S = their square roots, descending
void factor_values(Sector& s, bool right) {
    const Lapack& L = g_lapack;
    const lint n = right ? s.rows : s.cols;
    s.n = n;
    gram(s, right, s.G);
    if (n < kSelectMin) {   // the full eigensystem now
        std::vector<double> w((size_t)n);
        lint info = 0;
        if (n >= kSyevdMin) {
            const lint lwork = 1 + 6 * n + 2 * n * n, liwork = 3 + 5 * n;
            std::vector<double> work((size_t)lwork);
            std::vector<lint> iwork((size_t)liwork);
            L.syevd("V", "L", &n, s.G.data(), &n, w.data(), work.data(), &lwork, iwork.data(), &liwork, &info, 1, 1);
        } else {
            const lint lwork = std::max<lint>(1, 66 * n);   // (block size + 2) n
            std::vector<double> work((size_t)lwork);
            L.syev("V", "L", &n, s.G.data(), &n, w.data(), work.data(), &lwork, &info, 1, 1);
        }
        if (info != 0) {
            s.err = "symmetric eigensolver failed (info " + std::to_string(info) + ")";
            return;
        }
        const int64_t m = std::min(s.rows, s.cols);
        s.S.resize((size_t)m);
        s.Q.resize((size_t)(n * n));
        for (int64_t j = 0; j < n; ++j) {
            const int64_t src = n - 1 - j;
            std::memcpy(s.Q.data() + (size_t)(j * n), s.G.data() + (size_t)(src * n), sizeof(double) * (size_t)n);
            if (j < m) s.S[(size_t)j] = std::sqrt(std::max(w[(size_t)src], 0.0));
        }
        std::vector<double>().swap(s.G);
        s.full = true;
        return;
    }
    s.d.resize((size_t)n);
    s.e.resize((size_t)std::max<lint>(n, 1));
    s.tau.resize((size_t)std::max<lint>(n, 1));
    const lint lwork = 64 * std::max<lint>(n, 1);
    std::vector<double> work((size_t)lwork);
    lint info = 0;
    L.sytrd("L", &n, s.G.data(), &n, s.d.data(), s.e.data(), s.tau.data(), work.data(), &lwork, &info, 1);
    if (info != 0) {
        s.err = "dsytrd failed (info " + std::to_string(info) + ")";
        return;
    }
    std::vector<double> w(s.d), e2(s.e);
    L.sterf(&n, w.data(), e2.data(), &info);
    if (info != 0) {
        s.err = "dsterf failed (info " + std::to_string(info) + ")";
        return;
    }
    const int64_t m = std::min(s.rows, s.cols);
    s.S.resize((size_t)m);
    for (int64_t j = 0; j < m; ++j) s.S[(size_t)j] = std::sqrt(std::max(w[(size_t)(n - 1 - j)], 0.0));
}

// vectors pass: eigenvectors of the kept (largest) eigenvalues only, from the
// tridiagonal form (dstemr) and back-transformed with the stored reflectors
// (dormtr); a dstemr failure falls back to the full eigensystem (dsyevd)
void factor_vectors(Sector& s, bool right) {
    const Lapack& L = g_lapack;
    const lint n = s.n, k = s.kept;
    if (k <= 0) return;
    if (s.full) {   // the leading k columns of the full eigensystem
        s.Q.resize((size_t)(n * k));
        return;
    }
    std::vector<double> d(s.d), e(s.e), w((size_t)n), Z((size_t)(n * k));
    std::vector<lint> isuppz((size_t)(2 * k));
    const lint il = n - k + 1, iu = n, lwork = 18 * n, liwork = 10 * n;
    std::vector<double> work((size_t)lwork);
    std::vector<lint> iwork((size_t)liwork);
    lint m = 0, info = 0, tryrac = 1;
    const double vl = 0, vu = 0;
    L.stemr("V", "I", &n, d.data(), e.data(), &vl, &vu, &il, &iu, &m, w.data(), Z.data(), &n, &k, isuppz.data(),
            &tryrac, work.data(), &lwork, iwork.data(), &liwork, &info, 1, 1);
    if (info == 0 && m == k) {
        const lint lw2 = 64 * std::max<lint>(k, 1) + 4096;
        std::vector<double> work2((size_t)lw2);
        L.ormtr("L", "L", "N", &n, &k, s.G.data(), &n, s.tau.data(), Z.data(), &n, work2.data(), &lw2, &info, 1, 1, 1);
        if (info != 0) {
            s.err = "dormtr failed (info " + std::to_string(info) + ")";
            return;
        }
        s.Q.resize((size_t)(n * k));
        for (lint j = 0; j < k; ++j)   // ascending -> descending
            std::memcpy(s.Q.data() + (size_t)(j * n), Z.data() + (size_t)((k - 1 - j) * n), sizeof(double) * (size_t)n);
        return;
    }
    std::vector<double> G;
    gram(s, right, G);
    const lint lw = 1 + 6 * n + 2 * n * n, liw = 3 + 5 * n;
    std::vector<double> wk((size_t)lw), wv((size_t)n);
    std::vector<lint> iwk((size_t)liw);
    L.syevd("V", "L", &n, G.data(), &n, wv.data(), wk.data(), &lw, iwk.data(), &liw, &info, 1, 1);
    if (info != 0) {
        s.err = "dsyevd failed (info " + std::to_string(info) + ")";
        return;
    }
    s.Q.resize((size_t)(n * k));
    for (lint j = 0; j < k; ++j)
        std::memcpy(s.Q.data() + (size_t)(j * n), G.data() + (size_t)((n - 1 - j) * n), sizeof(double) * (size_t)n);
}

}  // namespace

struct vmps_split_s {
    int nq = 1;
    std::vector<QN> qmid;
    std::vector<int64_t> dmid;
    double disc = 0;
    // site tensors in site-layout block order
    std::vector<int32_t> leg1, qin1, qout1, leg2, qin2, qout2;
    std::vector<int64_t> rows1, cols1, rows2, cols2;
    std::vector<double> data1, data2;
};

namespace {

// Below this many floating-point operations a call runs on the calling thread:
// starting host threads costs more than such small sectors (a D=64 sweep).
constexpr double kParallelMinFlops = 4e6;

// fn(0 .. count-1) on up to `threads` host threads (dynamic: the next index to
// the next free thread)
// An exception in fn (an allocation failure, a malformed table) stops the
// remaining work and is rethrown on the calling thread after all threads joined.
template <typename F>
void parallel_for(size_t count, int threads, F fn) {
    const int nt = std::max(1, std::min<int>(threads, (int)count));
    std::atomic<size_t> next{0};
    std::exception_ptr first;
    std::mutex mu;
    auto worker = [&]() {
        try {
            for (size_t i = next++; i < count; i = next++) fn(i);
        } catch (...) {
            std::lock_guard<std::mutex> lock(mu);
            if (!first) first = std::current_exception();
            next = count;
        }
    };
    if (nt == 1) {
        worker();
    } else {
        std::vector<std::thread> th;
        try {
            for (int t = 0; t < nt; ++t) th.emplace_back(worker);
        } catch (...) {   // no thread could be started: stop the ones that run, report
            next = count;
            for (auto& t : th) t.join();
            throw;
        }
        for (auto& t : th) t.join();
    }
    if (first) std::rethrow_exception(first);
}

QN qadd(const QN& a, const int32_t* b, int nq, int sign) {
    QN r = a;
    for (int i = 0; i < nq; ++i) r[(size_t)i] += sign * b[i];
    return r;
}

// order of the Gram matrices that go to the device (VMPS_SPLIT_GPU_MIN overrides)
int64_t split_gpu_min() {
    const char* v = std::getenv("VMPS_SPLIT_GPU_MIN");
    if (!v || !*v) return 512;
    const long long x = std::atoll(v);
    if (x < 1) throw std::invalid_argument("VMPS_SPLIT_GPU_MIN must be a positive integer");
    return (int64_t)x;
}

// Which sectors go to the device.  The device thread factors its sectors one after
// another while `threads` host threads share the rest, so the split ends with the
// later of the two.  Largest first, a sector (of Gram order >= gmin) goes to the
// device when that makes the estimated end earlier; the estimates are fitted to
// GB300 + Grace measurements of the split at a D=4096 bond (Gram orders up to 772:
// 0.115 s on 16 host threads; every sector of order >= 512 on the device: 0.183 s;
// the largest one only: 0.095 s): a host sector of order n and k columns takes
// about 1.3e-10 s * n^2 (n + k), a device sector about 8 ms + 2.5e-11 s * n^2 (n + k)
// (the device's FP64 eigensolver runs its tridiagonal stage at a low rate, and each
// sector pays for its transfers and its own sequence of launches).
void assign_device_sectors(const std::vector<Sector*>& work, bool right, int64_t gmin, int threads,
                           std::vector<Sector*>& gwork, std::vector<Sector*>& hwork) {
    const int nt = std::max(1, threads);
    const char* pol = std::getenv("VMPS_SPLIT_DEVICE");   // "all": every sector of order >= gmin
    if (pol && !std::strcmp(pol, "all")) {
        for (Sector* s : work) ((right ? s->rows : s->cols) >= gmin ? gwork : hwork).push_back(s);
        return;
    }
    std::vector<double> bins((size_t)nt, 0.0);   // host threads' estimated loads (largest-first list scheduling)
    double tdev = 0;
    auto host_cost = [](double n, double k) { return 1.3e-10 * n * n * (n + k); };
    auto dev_cost = [](double n, double k) { return 8e-3 + 2.5e-11 * n * n * (n + k); };
    for (Sector* s : work) {   // work is sorted largest first
        const double n = (double)(right ? s->rows : s->cols), k = (double)(right ? s->cols : s->rows);
        auto lo = std::min_element(bins.begin(), bins.end());
        const double host_end = std::max(*std::max_element(bins.begin(), bins.end()), *lo + host_cost(n, k));
        const double dev_end = std::max(tdev + dev_cost(n, k), *std::max_element(bins.begin(), bins.end()));
        if (n >= (double)gmin && std::max(dev_end, tdev + dev_cost(n, k)) < std::max(host_end, tdev)) {
            tdev += dev_cost(n, k);
            gwork.push_back(s);
        } else {
            *lo += host_cost(n, k);
            hwork.push_back(s);
        }
    }
}

// gpu: device state of a context, or null (host only)
void run_split(const vmps_split_args* a, const vmps_blocks* V, const double* Vd, vmps_split_s& out, GpuLa* gpu) {
    const int nq = a->nq;
    out.nq = nq;
    const bool right = a->move_right != 0;
    // bond bases in sorted QN order
    struct Basis { QKey k; QN q; int64_t d; };
    auto load_basis = [nq](int m, const int32_t* qs, const int64_t* ds) {
        std::vector<Basis> b((size_t)m);
        for (int i = 0; i < m; ++i) {
            b[(size_t)i].q = qload(qs + (size_t)i * nq, nq);
            b[(size_t)i].k = qkey(b[(size_t)i].q, nq);
            b[(size_t)i].d = ds[i];
        }
        std::sort(b.begin(), b.end(), [](const Basis& x, const Basis& y) { return x.k < y.k; });
        return b;
    };
    const std::vector<Basis> bin = load_basis(a->nin, a->qin, a->din);
    const std::vector<Basis> bout = load_basis(a->nout, a->qout, a->dout);
    std::unordered_map<QKey, int64_t> dout;
    for (const Basis& b : bout) dout[b.k] = b.d;
    // sector rows: (s1, qin) in (s1, sorted qin) order; columns: (s3, qout)
    struct Pos { QKey qm; int64_t off; };
    std::unordered_map<QKey, int64_t> nrows, ncols;
    std::unordered_map<QKey, QN> qn_of;
    std::vector<std::unordered_map<QKey, Pos>> roff((size_t)a->n1), coff((size_t)a->n3);
    for (int s1 = 0; s1 < a->n1; ++s1)
        for (const Basis& b : bin) {
            const QN qm = qadd(b.q, a->qloc1 + (size_t)s1 * nq, nq, +1);
            const QKey km = qkey(qm, nq);
            qn_of[km] = qm;
            int64_t& nr = nrows[km];
            roff[(size_t)s1][b.k] = Pos{km, nr};
            nr += b.d;
        }
    for (int s3 = 0; s3 < a->n3; ++s3)
        for (const Basis& b : bout) {
            const QN qm = qadd(b.q, a->qloc3 + (size_t)s3 * nq, nq, -1);
            const QKey km = qkey(qm, nq);
            int64_t& nc = ncols[km];
            coff[(size_t)s3][b.k] = Pos{km, nc};
            nc += b.d;
        }
    // scatter the two-site blocks into their sectors (sectors without blocks are dropped)
    std::unordered_map<QKey, size_t> sidx;
    std::vector<std::unique_ptr<Sector>> sec;
    for (int64_t k = 0; k < V->nblocks; ++k) {
        const int s13 = V->leg[k];
        if (s13 < 0 || s13 >= a->n13) throw std::invalid_argument("two-site block leg outside the combined basis");
        const int s1 = a->pair1[s13], s3 = a->pair3[s13];
        const QKey ki = qkey(qload(V->qin + (size_t)k * nq, nq), nq), ko = qkey(qload(V->qout + (size_t)k * nq, nq), nq);
        auto ri = roff[(size_t)s1].find(ki);
        auto ci = coff[(size_t)s3].find(ko);
        if (ri == roff[(size_t)s1].end() || ci == coff[(size_t)s3].end() || ri->second.qm != ci->second.qm) continue;
        const QKey km = ri->second.qm;
        auto it = sidx.find(km);
        if (it == sidx.end()) {
            std::unique_ptr<Sector> S(new Sector());
            S->q = qn_of[km];
            S->key = km;
            S->rows = nrows[km];
            S->cols = ncols[km];
            S->M.assign((size_t)(S->rows * S->cols), 0.0);
            it = sidx.emplace(km, sec.size()).first;
            sec.push_back(std::move(S));
        }
        Sector& S = *sec[it->second];
        const int64_t r = V->rows[k], c = V->cols[k];
        if (ri->second.off + r > S.rows || ci->second.off + c > S.cols)
            throw std::invalid_argument("two-site block does not fit its sector");
        const double* src = Vd + V->offset[k];
        for (int64_t j = 0; j < c; ++j)
            std::memcpy(S.M.data() + (size_t)((ci->second.off + j) * S.rows + ri->second.off), src + (size_t)(j * r),
                        sizeof(double) * (size_t)r);
    }
    std::vector<Sector*> order;   // sorted by middle QN
    for (auto& p : sec) order.push_back(p.get());
    std::sort(order.begin(), order.end(), [](const Sector* x, const Sector* y) { return x->key < y->key; });
    // factorisations on the host threads, largest first
    std::vector<Sector*> work(order);
    std::sort(work.begin(), work.end(), [right](const Sector* x, const Sector* y) {
        const int64_t nx = right ? x->rows : x->cols, ny = right ? y->rows : y->cols;
        return nx * nx * (right ? x->cols : x->rows) > ny * ny * (right ? y->cols : y->rows);
    });
    double work_flops = 0;
    for (const Sector* s : work) {
        const double n = (double)(right ? s->rows : s->cols);
        work_flops += 10.0 * n * n * n;
    }
    const int threads = work_flops < kParallelMinFlops ? 1 : a->threads;
    // the large sectors (Gram order >= the device threshold) on the device thread,
    // the others on the host threads meanwhile
    std::vector<Sector*> gwork, hwork;
    if (gpu) assign_device_sectors(work, right, split_gpu_min(), threads, gwork, hwork);
    else hwork = work;
    auto on_device = [&](const std::vector<Sector*>& list, auto fn) {
        if (list.empty()) return std::thread();
        return std::thread([&, fn]() {
            std::lock_guard<std::mutex> lock(gpu->mu);
            try {
                cu_check(cudaSetDevice(gpu->device), "cudaSetDevice");
            } catch (const std::exception& e) {
                for (Sector* s : list) s->err = e.what();
                return;
            }
            for (Sector* s : list) {
                try {
                    fn(*s);
                } catch (const std::exception& e) {
                    s->err = e.what();
                    return;
                }
            }
        });
    };
    {
        std::thread gt = on_device(gwork, [&](Sector& s) { gpu_factor_values(*gpu, s, right); });
        try {
            parallel_for(hwork.size(), threads, [&](size_t i) { factor_values(*hwork[i], right); });
        } catch (...) {
            if (gt.joinable()) gt.join();
            throw;
        }
        if (gt.joinable()) gt.join();
    }
    for (Sector* s : order)
        if (!s->err.empty()) throw std::runtime_error(s->err);
    // global truncation: the Dmax largest values above eps_svd * max; ties at the
    // threshold are kept in sector order until Dmax is reached
    std::vector<double> all;
    for (Sector* s : order) all.insert(all.end(), s->S.begin(), s->S.end());
    double smax = 0, tot2 = 0;
    for (double v : all) {
        smax = std::max(smax, v);
        tot2 += v * v;
    }
    std::vector<double> keep;
    for (double v : all)
        if (v > a->eps_svd * smax) keep.push_back(v);
    std::sort(keep.begin(), keep.end(), [](double x, double y) { return x > y; });
    if ((int64_t)keep.size() > a->dmax) keep.resize((size_t)std::max<int64_t>(a->dmax, 0));
    const double thresh = keep.empty() ? std::numeric_limits<double>::infinity() : keep.back();
    int64_t budget = (int64_t)keep.size();
    for (Sector* s : order) {
        s->kept = 0;
        for (double v : s->S) s->kept += v > thresh;
        budget -= s->kept;
    }
    for (Sector* s : order) {
        if (budget <= 0) break;
        int64_t extra = 0;
        for (double v : s->S) extra += v == thresh;
        const int64_t take = std::min(extra, budget);
        s->kept += take;
        budget -= take;
    }
    double norm2 = 0;
    for (Sector* s : order)
        for (int64_t i = 0; i < s->kept; ++i) norm2 += s->S[(size_t)i] * s->S[(size_t)i];
    out.disc = tot2 > 0 ? std::max(0.0, tot2 - norm2) / tot2 : 0.0;
    const double scale = norm2 > 0 ? 1.0 / std::sqrt(norm2) : 1.0;
    std::vector<Sector*> ks;   // kept sectors, in QN order
    std::unordered_map<QKey, size_t> kidx;
    for (Sector* s : order)
        if (s->kept == 0) {   // nothing of this sector is kept
            std::vector<double>().swap(s->G);
            std::vector<double>().swap(s->Q);
            std::vector<double>().swap(s->M);
        }
    for (Sector* s : order)
        if (s->kept > 0) {
            kidx[s->key] = ks.size();
            ks.push_back(s);
            out.qmid.push_back(s->q);
            out.dmid.push_back(s->kept);
        }
    // the kept eigenvectors, then the non-orthonormal factor: A2 = scale U_k^T Psi
    // (right) or A1 = scale Psi V_k (left), largest sectors first
    const Lapack& L = g_lapack;
    std::vector<size_t> vorder(ks.size());
    for (size_t i = 0; i < ks.size(); ++i) vorder[i] = i;
    std::sort(vorder.begin(), vorder.end(), [&](size_t x, size_t y) {
        return ks[x]->n * ks[x]->n * ks[x]->kept > ks[y]->n * ks[y]->n * ks[y]->kept;
    });
    std::vector<std::vector<double>> Fk(ks.size());
    std::vector<size_t> gvec, hvec;
    for (size_t t = 0; t < vorder.size(); ++t) (ks[vorder[t]]->gpu ? gvec : hvec).push_back(vorder[t]);
    std::vector<Sector*> gks;
    for (size_t i : gvec) gks.push_back(ks[i]);
    std::unordered_map<const Sector*, size_t> kpos;
    for (size_t i = 0; i < ks.size(); ++i) kpos[ks[i]] = i;
    std::thread gt = on_device(gks, [&](Sector& s) {
        s.Q.resize((size_t)(s.n * s.kept));   // the leading kept eigenvectors (descending)
        gpu_factor_product(*gpu, s, right, scale, Fk[kpos[&s]]);
    });
    try {
    parallel_for(hvec.size(), threads, [&](size_t t) {
        const size_t i = hvec[t];
        Sector& s = *ks[i];
        factor_vectors(s, right);
        if (!s.err.empty()) return;
        const lint r = s.rows, c = s.cols, k = s.kept, n = s.n;
        const double zero = 0.0;
        if (right) {
            Fk[i].assign((size_t)(k * c), 0.0);   // k x c
            L.gemm("T", "N", &k, &c, &r, &scale, s.Q.data(), &n, s.M.data(), &r, &zero, Fk[i].data(), &k, 1, 1);
        } else {
            Fk[i].assign((size_t)(r * k), 0.0);   // r x k
            L.gemm("N", "N", &r, &k, &c, &scale, s.M.data(), &r, s.Q.data(), &n, &zero, Fk[i].data(), &r, 1, 1);
        }
    });
    } catch (...) {
        if (gt.joinable()) gt.join();
        throw;
    }
    if (gt.joinable()) gt.join();
    for (Sector* s : ks)
        if (!s->err.empty()) throw std::runtime_error(s->err);
    // output sizes first (one allocation per table)
    {
        size_t nb1 = 0, sz1 = 0, nb2 = 0, sz2 = 0;
        for (int s1 = 0; s1 < a->n1; ++s1)
            for (const Basis& b : bin) {
                auto it = kidx.find(qkey(qadd(b.q, a->qloc1 + (size_t)s1 * nq, nq, +1), nq));
                if (it == kidx.end()) continue;
                ++nb1;
                sz1 += (size_t)(b.d * ks[it->second]->kept);
            }
        for (int s3 = 0; s3 < a->n3; ++s3)
            for (const Sector* s : ks) {
                auto di = dout.find(qkey(qadd(s->q, a->qloc3 + (size_t)s3 * nq, nq, +1), nq));
                if (di == dout.end()) continue;
                ++nb2;
                sz2 += (size_t)(s->kept * di->second);
            }
        out.leg1.reserve(nb1); out.rows1.reserve(nb1); out.cols1.reserve(nb1);
        out.qin1.reserve(nb1 * (size_t)nq); out.qout1.reserve(nb1 * (size_t)nq);
        out.leg2.reserve(nb2); out.rows2.reserve(nb2); out.cols2.reserve(nb2);
        out.qin2.reserve(nb2 * (size_t)nq); out.qout2.reserve(nb2 * (size_t)nq);
        out.data1.reserve(sz1);
        out.data2.reserve(sz2);
    }
    // A1 = site layout (qloc1, din, dmid): rows of the sector at (s1, qin)
    for (int s1 = 0; s1 < a->n1; ++s1)
        for (const Basis& b : bin) {
            const QN qm = qadd(b.q, a->qloc1 + (size_t)s1 * nq, nq, +1);
            auto it = kidx.find(qkey(qm, nq));
            if (it == kidx.end()) continue;
            const Sector& s = *ks[it->second];
            const int64_t r = b.d, c = s.kept, ra = roff[(size_t)s1][b.k].off;
            out.leg1.push_back(s1);
            out.qin1.insert(out.qin1.end(), b.q.begin(), b.q.begin() + nq);
            out.qout1.insert(out.qout1.end(), qm.begin(), qm.begin() + nq);
            out.rows1.push_back(r);
            out.cols1.push_back(c);
            const size_t base = out.data1.size();
            out.data1.resize(base + (size_t)(r * c));
            double* dst = out.data1.data() + base;
            if (right) {   // U_k rows ra.. of the eigenvectors
                for (int64_t j = 0; j < c; ++j)
                    std::memcpy(dst + (size_t)(j * r), s.Q.data() + (size_t)(j * s.n + ra), sizeof(double) * (size_t)r);
            } else {       // scale Psi V_k, rows ra..
                const std::vector<double>& f = Fk[it->second];
                for (int64_t j = 0; j < c; ++j)
                    std::memcpy(dst + (size_t)(j * r), f.data() + (size_t)(j * s.rows + ra), sizeof(double) * (size_t)r);
            }
        }
    // A2 = site layout (qloc3, dmid, dout): columns of the sector at (s3, qout)
    for (int s3 = 0; s3 < a->n3; ++s3)
        for (size_t i = 0; i < ks.size(); ++i) {
            const Sector& s = *ks[i];
            const QN qo = qadd(s.q, a->qloc3 + (size_t)s3 * nq, nq, +1);
            const QKey ko = qkey(qo, nq);
            auto di = dout.find(ko);
            if (di == dout.end()) continue;
            const int64_t r = s.kept, c = di->second, ca = coff[(size_t)s3][ko].off;
            out.leg2.push_back(s3);
            out.qin2.insert(out.qin2.end(), s.q.begin(), s.q.begin() + nq);
            out.qout2.insert(out.qout2.end(), qo.begin(), qo.begin() + nq);
            out.rows2.push_back(r);
            out.cols2.push_back(c);
            const size_t base = out.data2.size();
            out.data2.resize(base + (size_t)(r * c));
            double* dst = out.data2.data() + base;
            if (right) {   // scale U_k^T Psi, columns ca..
                std::memcpy(dst, Fk[i].data() + (size_t)(ca * r), sizeof(double) * (size_t)(r * c));
            } else {       // V_k^T: row i = eigenvector i at entries ca..
                for (int64_t j = 0; j < c; ++j)
                    for (int64_t q = 0; q < r; ++q) dst[j * r + q] = s.Q[(size_t)(q * s.n + ca + j)];
            }
        }
}

}  // namespace

namespace {

// Q R of an m x n column-major matrix (m >= n), reduced: a <- Q (m x n), R (n x n, upper)
void qr_reduced(double* a, lint m, lint n, double* R) {
    const Lapack& L = g_lapack;
    std::vector<double> tau((size_t)std::max<lint>(n, 1));
    lint info = 0, lwork = -1;
    double wq = 0;
    L.geqrf(&m, &n, a, &m, tau.data(), &wq, &lwork, &info);   // workspace query
    lwork = std::max<lint>((lint)wq, std::max<lint>(n, 1));
    std::vector<double> work((size_t)lwork);
    L.geqrf(&m, &n, a, &m, tau.data(), work.data(), &lwork, &info);
    if (info != 0) throw std::runtime_error("dgeqrf failed (info " + std::to_string(info) + ")");
    for (lint j = 0; j < n; ++j)
        for (lint i = 0; i < n; ++i) R[j * n + i] = i <= j ? a[j * m + i] : 0.0;
    lwork = -1;
    L.orgqr(&m, &n, &n, a, &m, tau.data(), &wq, &lwork, &info);
    lwork = std::max<lint>((lint)wq, std::max<lint>(n, 1));
    work.assign((size_t)lwork, 0.0);
    L.orgqr(&m, &n, &n, a, &m, tau.data(), work.data(), &lwork, &info);
    if (info != 0) throw std::runtime_error("dorgqr failed (info " + std::to_string(info) + ")");
}

void run_gauge(int nq, bool right, const vmps_blocks* A, double* a, const double* w, const vmps_blocks* Nb,
               double* nb, int threads) {
    const Lapack& L = g_lapack;
    // sectors of A: blocks sharing qout (right) or qin (left), in order of first appearance
    std::unordered_map<QKey, size_t> sidx;
    std::vector<std::vector<int64_t>> members;
    std::vector<QKey> skey;
    for (int64_t i = 0; i < A->nblocks; ++i) {
        const QKey k = qkey(qload((right ? A->qout : A->qin) + (size_t)i * nq, nq), nq);
        auto it = sidx.find(k);
        if (it == sidx.end()) {
            it = sidx.emplace(k, members.size()).first;
            members.emplace_back();
            skey.push_back(k);
        }
        members[it->second].push_back(i);
    }
    const size_t ns = members.size();
    double work_flops = 0;
    for (const auto& mb : members) {
        double m = 0;
        for (int64_t i : mb) m += (double)(right ? A->rows[i] : A->cols[i]);
        const double n = (double)(right ? A->cols[mb[0]] : A->rows[mb[0]]);
        work_flops += 4.0 * m * n * n;
    }
    if (work_flops < kParallelMinFlops) threads = 1;
    std::vector<std::vector<double>> Rf(ns);
    std::vector<int64_t> rdim(ns, 0);
    std::vector<std::string> err(ns);
    parallel_for(ns, threads, [&](size_t q) {
        const auto& mb = members[q];
        // right: M = vstack(A_i), m x n with n = the common column count
        // left:  M^T = vstack((w_i A_i)^T), the LQ of hstack(w_i A_i)
        int64_t m = 0, n = right ? A->cols[mb[0]] : A->rows[mb[0]];
        for (int64_t i : mb) {
            if ((right ? A->cols[i] : A->rows[i]) != n) { err[q] = "blocks of one sector differ in their shared extent"; return; }
            m += right ? A->rows[i] : A->cols[i];
        }
        if (m < n) { err[q] = "sector has fewer rows than columns (no reduced QR of this shape)"; return; }
        std::vector<double> M((size_t)(m * n));
        int64_t r0 = 0;
        for (int64_t i : mb) {
            const double* src = a + A->offset[i];
            const int64_t br = A->rows[i], bc = A->cols[i];
            if (right) {
                for (int64_t j = 0; j < bc; ++j)
                    std::memcpy(M.data() + (size_t)(j * m + r0), src + (size_t)(j * br), sizeof(double) * (size_t)br);
                r0 += br;
            } else {
                const double wi = w ? w[i] : 1.0;
                for (int64_t j = 0; j < bc; ++j)          // row r0 + j of M^T = column j of the block
                    for (int64_t t = 0; t < br; ++t) M[(size_t)(t * m + r0 + j)] = wi * src[(size_t)(j * br + t)];
                r0 += bc;
            }
        }
        Rf[q].assign((size_t)(n * n), 0.0);
        try {
            qr_reduced(M.data(), m, n, Rf[q].data());
        } catch (const std::exception& e) {
            err[q] = e.what();
            return;
        }
        rdim[q] = n;
        r0 = 0;
        for (int64_t i : mb) {
            double* dst = a + A->offset[i];
            const int64_t br = A->rows[i], bc = A->cols[i];
            if (right) {
                for (int64_t j = 0; j < bc; ++j)
                    std::memcpy(dst + (size_t)(j * br), M.data() + (size_t)(j * m + r0), sizeof(double) * (size_t)br);
                r0 += br;
            } else {   // A_i = (Q^T)[:, r0:r0+bc] / w_i
                const double wi = w ? w[i] : 1.0;
                for (int64_t j = 0; j < bc; ++j)
                    for (int64_t t = 0; t < br; ++t) dst[(size_t)(j * br + t)] = M[(size_t)(t * m + r0 + j)] / wi;
                r0 += bc;
            }
        }
    });
    for (const auto& e : err)
        if (!e.empty()) throw std::invalid_argument(e);
    // the neighbour: right: N_i <- R[qin] N_i;  left: N_i <- N_i L[qout], L = R^T
    std::vector<int64_t> nwork;
    std::vector<size_t> nsec;
    for (int64_t i = 0; i < Nb->nblocks; ++i) {
        const QKey k = qkey(qload((right ? Nb->qin : Nb->qout) + (size_t)i * nq, nq), nq);
        auto it = sidx.find(k);
        if (it == sidx.end()) continue;
        if ((right ? Nb->rows[i] : Nb->cols[i]) != rdim[it->second])
            throw std::invalid_argument("neighbour block does not match the gauge factor");
        nwork.push_back(i);
        nsec.push_back(it->second);
    }
    parallel_for(nwork.size(), threads, [&](size_t t) {
        const int64_t i = nwork[t];
        const std::vector<double>& R = Rf[nsec[t]];
        double* blk = nb + Nb->offset[i];
        const lint br = Nb->rows[i], bc = Nb->cols[i];
        std::vector<double> in(blk, blk + (size_t)(br * bc));
        const double one = 1.0, zero = 0.0;
        if (right)
            L.gemm("N", "N", &br, &bc, &br, &one, R.data(), &br, in.data(), &br, &zero, blk, &br, 1, 1);
        else   // N L with L = R^T
            L.gemm("N", "T", &br, &bc, &bc, &one, in.data(), &br, R.data(), &bc, &zero, blk, &br, 1, 1);
    });
}

}  // namespace

extern "C" int vmps_gauge_step(int nq, int move_right, const vmps_blocks* A, double* a, const double* w,
                               const vmps_blocks* N, double* n, int threads) {
    if (nq < 1 || nq > 4 || !A || !N || (A->nblocks > 0 && !a) || (N->nblocks > 0 && !n))
        return set_err(VMPS_E_ARG, "bad argument");
    if (!table_ok(A) || !table_ok(N)) return set_err(VMPS_E_ARG, "block table with null arrays or non-positive shapes");
    if (!g_lapack.ok()) return set_err(VMPS_E_ARG, "host LAPACK not bound (vmps_hostla_load)");
    try {
        run_gauge(nq, move_right != 0, A, a, w, N, n, threads);
    } catch (const std::bad_alloc& e) {
        return set_err(VMPS_E_NOMEM, e.what());
    } catch (const std::exception& e) {
        return set_err(VMPS_E_ARG, e.what());
    }
    return VMPS_OK;
}

extern "C" int vmps_hostla_load(const char* path) {
    std::lock_guard<std::mutex> lock(g_lapack_mu);
    if (g_lapack.ok()) return VMPS_OK;
    if (!path) return set_err(VMPS_E_ARG, "no library path");
    void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return set_err(VMPS_E_ARG, std::string("cannot open ") + path);
    Lapack L;
    L.syevd = (dsyevd_fn)find_symbol(h, "dsyevd");
    L.syev = (dsyev_fn)find_symbol(h, "dsyev");
    L.sytrd = (dsytrd_fn)find_symbol(h, "dsytrd");
    L.sterf = (dsterf_fn)find_symbol(h, "dsterf");
    L.stemr = (dstemr_fn)find_symbol(h, "dstemr");
    L.ormtr = (dormtr_fn)find_symbol(h, "dormtr");
    L.geqrf = (dgeqrf_fn)find_symbol(h, "dgeqrf");
    L.orgqr = (dorgqr_fn)find_symbol(h, "dorgqr");
    L.syrk = (dsyrk_fn)find_symbol(h, "dsyrk");
    L.gemm = (dgemm_fn)find_symbol(h, "dgemm");
    if (!L.ok()) return set_err(VMPS_E_ARG, std::string("no ILP64 dsyevd/dsyev/dsytrd/dsterf/dstemr/dormtr/dsyrk/dgemm/dgeqrf/dorgqr in ") + path);
    g_lapack = L;
    return VMPS_OK;
}

namespace {
int split_entry(vmps_ctx* ctx, const vmps_split_args* a, const vmps_blocks* V, const double* Vdata,
                vmps_split** out) {
    if (!a || !V || !out || (V->nblocks > 0 && !Vdata)) return set_err(VMPS_E_ARG, "bad argument");
    if (a->nq < 1 || a->nq > 4 || a->n1 < 1 || a->n3 < 1 || a->n13 < 1 || !a->pair1 || !a->pair3 ||
        !a->qloc1 || !a->qloc3 || a->nin < 0 || a->nout < 0 || a->dmax < 0 ||
        (a->nin > 0 && (!a->qin || !a->din)) || (a->nout > 0 && (!a->qout || !a->dout)))
        return set_err(VMPS_E_ARG, "bad split arguments");
    if (!table_ok(V)) return set_err(VMPS_E_ARG, "two-site table with null arrays or non-positive shapes");
    for (int i = 0; i < a->nin; ++i)
        if (a->din[i] < 0) return set_err(VMPS_E_ARG, "negative bond dimension");
    for (int i = 0; i < a->nout; ++i)
        if (a->dout[i] < 0) return set_err(VMPS_E_ARG, "negative bond dimension");
    for (int i = 0; i < a->n13; ++i)
        if (a->pair1[i] < 0 || a->pair1[i] >= a->n1 || a->pair3[i] < 0 || a->pair3[i] >= a->n3)
            return set_err(VMPS_E_ARG, "combined index outside the local bases");
    if (!g_lapack.ok()) return set_err(VMPS_E_ARG, "host LAPACK not bound (vmps_hostla_load)");
    try {
        GpuLa* g = nullptr;
        if (ctx) {
            if (vmps::ctx_device(ctx) < 0) return set_err(VMPS_E_ARG, "device split needs a device context");
            g = &gpu_la(ctx);
        }
        std::unique_ptr<vmps_split_s> s(new vmps_split_s());
        run_split(a, V, Vdata, *s, g);
        *out = s.release();
    } catch (const std::bad_alloc& e) {
        return set_err(VMPS_E_NOMEM, e.what());
    } catch (const std::exception& e) {
        return set_err(VMPS_E_ARG, e.what());
    }
    return VMPS_OK;
}
}  // namespace

extern "C" int vmps_two_site_split(const vmps_split_args* a, const vmps_blocks* V, const double* Vdata,
                                   vmps_split** out) {
    return split_entry(nullptr, a, V, Vdata, out);
}

extern "C" int vmps_two_site_split_device(vmps_ctx* ctx, const vmps_split_args* a, const vmps_blocks* V,
                                          const double* Vdata, vmps_split** out) {
    if (!ctx) return set_err(VMPS_E_ARG, "null context");
    return split_entry(ctx, a, V, Vdata, out);
}

extern "C" int vmps_split_info(const vmps_split* s, int* nmid, double* disc, int64_t* nblocks1, int64_t* size1,
                               int64_t* nblocks2, int64_t* size2) {
    if (!s || !nmid || !disc || !nblocks1 || !size1 || !nblocks2 || !size2)
        return set_err(VMPS_E_ARG, "bad argument");
    *nmid = (int)s->qmid.size();
    *disc = s->disc;
    *nblocks1 = (int64_t)s->leg1.size();
    *size1 = (int64_t)s->data1.size();
    *nblocks2 = (int64_t)s->leg2.size();
    *size2 = (int64_t)s->data2.size();
    return VMPS_OK;
}

extern "C" int vmps_split_get(const vmps_split* s, int32_t* qmid, int64_t* dmid, int32_t* leg1, int32_t* qin1,
                              int32_t* qout1, int64_t* rows1, int64_t* cols1, double* data1, int32_t* leg2,
                              int32_t* qin2, int32_t* qout2, int64_t* rows2, int64_t* cols2, double* data2) {
    if (!s) return set_err(VMPS_E_ARG, "bad argument");
    auto put = [](auto* dst, const auto& v) {
        if (!v.empty()) std::memcpy(dst, v.data(), sizeof(v[0]) * v.size());
    };
    if (!qmid || !dmid || !leg1 || !qin1 || !qout1 || !rows1 || !cols1 || !data1 || !leg2 || !qin2 || !qout2 ||
        !rows2 || !cols2 || !data2)
        return set_err(VMPS_E_ARG, "bad argument");
    for (size_t i = 0; i < s->qmid.size(); ++i)
        for (int c = 0; c < s->nq; ++c) qmid[i * (size_t)s->nq + (size_t)c] = s->qmid[i][(size_t)c];
    put(dmid, s->dmid);
    put(leg1, s->leg1); put(qin1, s->qin1); put(qout1, s->qout1); put(rows1, s->rows1); put(cols1, s->cols1);
    put(data1, s->data1);
    put(leg2, s->leg2); put(qin2, s->qin2); put(qout2, s->qout2); put(rows2, s->rows2); put(cols2, s->cols2);
    put(data2, s->data2);
    return VMPS_OK;
}

extern "C" void vmps_split_destroy(vmps_split* s) { delete s; }
