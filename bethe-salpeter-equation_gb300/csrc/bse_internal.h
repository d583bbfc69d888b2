// Internal declarations of the GB300 BSE library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <cuComplex.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bse_gpu.h"

namespace bse {

constexpr double kMinval = 1.0e-5;                               // bse.version13.cpp:28
constexpr double kPi = 3.1415926535897932384626433832;           // bse.version13.cpp:29
constexpr double kConv = (1.602176634 * 1000) / (8.8541878176);  // bse.version13.cpp:32
constexpr int kMaxNw = 16;        // orbitals per spin channel handled by the band kernel
constexpr int kStages = 15;  // bands, tables, build, eig, refine, oscillators, eps, whole solve,
                              // own solver: tridiagonal, eigenvalues, inverse iteration, back-transform, clusters,
                              // two-stage reduction: dense -> band, bulge chase

// Geometry derived once from the lattice (Crystal_Lattice, bse.version13.cpp:85-124).
struct Geometry {
    double vol, area, lz;
    double normal[3];
};

// Interaction parameters the device needs (Coulomb_Potential::pull + model W).
struct Interaction {
    int coulomb_kind, w_kind;
    double radius, min_k2, inv_eps, rk_r0, rk_eps;
    double nx, ny, nz, lz;   // plane normal and cell height for the 2-D kinds
    double cell_avg;         // W at Delta k = 0, G = G0
};

// k-list structure: a lattice in crystal coordinates lets Delta k be tabulated by integer offset.
struct DeltaMap {
    bool on_grid = false;
    int m[3] = {1, 1, 1};          // distinct values per crystal axis
    double step[3] = {0, 0, 0};    // spacing per axis (crystal units)
    int64_t n_delta = 0;           // (2m0-1)(2m1-1)(2m2-1) or nk*nk
    std::vector<int32_t> idx;      // per k: packed integer grid coordinates (on_grid)
    bool periodic = false;         // on_grid, every grid point present once, step * m = 1 on each axis
    std::vector<int32_t> inv;      // periodic: k index of grid coordinates (i0 * m1 + i1) * m2 + i2
};

}  // namespace bse

struct bse_ctx {
    // sizes
    int nw, ns, nb, nk, ng, nv, nc, S, nr;
    int64_t N, n_h, n_rho, n_exc, n_opt;
    bool coupled = false;        // full BSE with the coupling block (tamm_dancoff = 0, not IPA; FP64)
    bse_params p;
    bse::Geometry geo;
    bse::Interaction itx;
    bse::DeltaMap dmap;
    double bmat_h[9] = {};       // reciprocal vectors b1 b2 b3 as columns (host copy of d_bmat)
    int device;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;           // concurrent work of the own solver (joined before use)
    cudaStream_t side2 = nullptr;          // the refinement's FP64 build, concurrent with the same phase
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_h64 = nullptr;
    bool h64_pending = false;              // FP64 copy for the refinement still to be built
    bool h64_side = false;                 // built on the side stream: wait for ev_h64 first
    cublasHandle_t cublas = nullptr;
    cusolverDnHandle_t cusolver = nullptr;
    cudaEvent_t ev[2 * bse::kStages] = {};
    double stage_ms[bse::kStages] = {};
    int stage_mute = 0;          // >0: stage timers untouched (nested solves)
    int64_t launches = 0;
    std::string err;

    // model on the device
    double* d_rcart = nullptr;   // 3 x nr
    double* d_weights = nullptr;
    double2* d_hr = nullptr;     // nw x nw x nr x ns
    double* d_centres = nullptr; // 3 x nw x ns
    double* d_k = nullptr;       // 3 x nk
    double* d_bmat = nullptr;    // reciprocal vectors b1 b2 b3 as columns
    int32_t* d_kidx = nullptr;   // packed grid index per k (on_grid)
    double* d_g = nullptr;       // 3 x ng
    int* d_status = nullptr;     // device-side status word

    // band subset (conduction at k, valence at k-q)
    double* d_ec = nullptr;      // [2][nk][nc]
    double* d_ev = nullptr;      // [2][nk][nv]
    double2* d_cc = nullptr;     // [nk][nc][nb]
    double2* d_cv = nullptr;     // [nk][nv][nb]
    bool bands_valid = false;

    // kernel tables
    double2* d_phi = nullptr;    // [n_delta][nblk][nw][nw] direct-kernel lattice sums (FP64)
    double2* d_phi_c = nullptr;  // RPA + full BSE: the coupling block's sums, with conj(W) (FP64)
    float2* d_phi32 = nullptr;   // the same in FP32 for the mixed build
    double2* d_X = nullptr;      // [ns][ns][nw][nw] exchange lattice sums
    double2* d_qx = nullptr;     // [ns][ns][nw][n_rho/ns] exchange row factors  Qx[s1][s2][beta][r]
    float2* d_qx32 = nullptr;
    double2* d_rho = nullptr;    // n_rho x ng pair densities (column-major)
    bool tables_valid = false;

    // BSE matrix and its spectrum
    void* d_H = nullptr;         // n_h x n_h, complex64 (MIXED) or complex128 (FP64)
    size_t h_elem = 0;
    double2* d_H64 = nullptr;    // MIXED refinement: FP64 lower triangle of the solved block(s)
    void* d_blk = nullptr;       // collinear: the two 2N x 2N diagonal blocks (H0, H1); coupled: L^H J L
    double2* d_aux = nullptr;    // coupled: L^{-1} rho(G0) (2N)
    bool h_valid = false;
    double* d_E = nullptr;       // n_exc eigenvalues
    void* d_A = nullptr;         // eigenvectors of the optically active block (n_opt x n_opt)
    bool eig_valid = false;
    double2* d_f = nullptr;      // n_opt oscillator strengths
    bool osc_valid = false;
    int64_t n_vec_valid = 0;     // leading eigenvector columns of d_A that are formed
    bool f_from_eig = false;     // the own solver produced f for every exciton
    int64_t n_refined = 0;       // leading columns replaced by the FP64 refinement
    int last_clusters = 0;       // clusters the own eigensolver resolved in FP64 in its last call
    double max_residual = 0;     // max ||H x - theta x||_2 (FP64) over the refined eigenpairs
    // workspaces
    void* d_work = nullptr;
    size_t work_bytes = 0;
    // per-launch CUDA-event timing of the tensor-core products of the last two-stage reduction
    // (BSE_KERNEL_TIMING set at bse_create): kind 0 = hemm, 1 = update; events are reused
    struct KernelTime {
        cudaEvent_t ev[2] = {nullptr, nullptr};   // around the launch
        int kind = 0;
        double bytes = 0, flops = 0;
    };
    int build_k_lo = 0, build_k_hi = 0;   // k tile of the next build (rows k1 in [lo, hi)); hi = 0: all
    // test overrides read at bse_create: the polling limit of the solver's bounded waits
    // (BSE_TEST_SPIN_LIMIT, 0 = the built-in limit) and the H(k) Jacobi sweep cap
    // (BSE_TEST_JACOBI_SWEEPS, default 60)
    unsigned spin_limit = 0;
    int jacobi_sweeps = 60;
    bool ktime = false;
    std::vector<KernelTime> kt;
    size_t kt_used = 0;
};

namespace bse {

// --- helpers (host) ---
int fail(bse_ctx* c, int code, const std::string& msg);
int cuda_check(bse_ctx* c, cudaError_t e, const char* what);
int ensure_work(bse_ctx* c, size_t bytes);
void stage_begin(bse_ctx* c, int s);
void stage_end(bse_ctx* c, int s);

// --- stages (each returns a bse_status) ---
int run_bands(bse_ctx* c);
// band subset with conduction states at k and valence states at k - q into the given buffers
// (layouts of d_ec, d_ev, d_cc, d_cv); errors land in d_status as for run_bands (bands.cu)
int band_states_shifted(bse_ctx* c, const double* q, double* ec, double* ev, double2* cc, double2* cv);
// RPA screened interaction: the direct-kernel tables Phi (and Phi32) from W = eps^-1 v (kernel_build.cu)
int run_rpa_tables(bse_ctx* c);
int run_tables(bse_ctx* c);
int run_build(bse_ctx* c, bool full, double* h_out, double* rho_out);
int run_build_rows(bse_ctx* c, int k_lo, int k_hi, double* h_rows);
int run_set_kernel(bse_ctx* c, const double* h);
int run_eig(bse_ctx* c, bool want_vectors);
int run_refine(bse_ctx* c);
// C = op(A) B for FP64 operands in compensated FP32 arithmetic (eigensolve.cu); C packed (ldc = M)
// when the product is split over K (small products), P: scratch of pcap elements for the splits
int df_gemm(bse_ctx* c, bool conj_a, int M, int N, int K, const double2* A, int64_t lda, const double2* B, int64_t ldb,
            double2* C, int64_t ldc, double2* P, int64_t pcap);
// FP64 copy of the solved block(s) for the refinement, launched on c->stream (kernel_build.cu)
int build_h64(bse_ctx* c);
// launch a pending FP64 build on the side stream (after the work already on c->stream)
int fork_h64(bse_ctx* c);
int run_oscillators(bse_ctx* c);
// full BSE: structure-preserving solve of H = J M through M = L L^H (eigensolve.cu)
int run_eig_coupled(bse_ctx* c, bool want_vectors);
int run_eps(bse_ctx* c, const double* omega, int n_omega, double gamma, double* eps2, double* eps1);

// own dense eigensolver (tridiag.cu)
// Eigenvalues of the Hermitian n x n matrix dA (full storage) into dW; the first n_vec
// eigenvectors overwrite dA's first columns; with rho0 given, f_out[l] = rho0^H x_l for all l.
// nested: a small solve inside another stage (the refinement's projected matrix): its own
// stream-ordered workspace instead of the context arena, no stage timers, no diagnostics.
int own_heevd(bse_ctx* c, int n, void* dA, int lda, bool fp64, double* dW, int n_vec, const double2* rho0,
              double2* f_out, bool nested = false);

// two-stage reduction (band.cu): dense -> band -> real tridiagonal (d, e), y <- Q^H y; with keep_q the
// reflectors stay in ws for band_backtransform (X = Q Z, Z real n x n_vec).  bar/err: barrier words.
size_t band_workspace(int n, bool fp64, bool keep_q, int n_vec, int nsm);
int band_tridiag(bse_ctx* c, int n, void* A, int64_t lda, bool fp64, void* d, void* e, void* y, bool keep_q, char* ws,
                 unsigned* bar, int* err, int n_vec);
int band_backtransform(bse_ctx* c, int n, bool fp64, const void* z, int n_vec, void* X, char* ws, unsigned* bar,
                       int* err);

// tensor-core (tcgen05 + TMA, split TF32) products of the complex64 two-stage reduction's
// trailing update (tc_update.cu), on the full-storage m x m trailing matrix A22 (lda even):
// Y = A22 V and A22 -= V W^H + W V^H.  ws: tc_workspace(n, nsm) bytes for every m <= n.
// Return 0, or nonzero when a tensor map or a launch failed; *err is the device error word.
size_t tc_workspace(int n, int nsm);
bool tc_supported(int64_t lda);
// ev (nullable): two events recorded around the tensor-core kernel itself.
int tc_hemm(cudaStream_t st, int nsm, int m, int kk, const float2* A22, int64_t lda, const float2* V, float2* Y, char* ws,
            int* err, int* launches, cudaEvent_t* ev = nullptr);
int tc_rank2k(cudaStream_t st, int nsm, int m, int kk, float2* A22, int64_t lda, const float2* V, const float2* W, char* ws,
              int* err, int* launches, cudaEvent_t* ev = nullptr);
// next event pair of the kernel timing (null when timing is off); bytes / flops are the launch's
// algorithmic traffic and arithmetic
cudaEvent_t* kernel_timer(bse_ctx* c, int kind, double bytes, double flops);

}  // namespace bse
