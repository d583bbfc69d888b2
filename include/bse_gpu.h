/*
 * bse_gpu.h -- C ABI of the GB300 Bethe-Salpeter solver (q->0; Tamm-Dancoff, or the full
 * BSE with the coupling block).
 *
 * The entry points replace the kernel-build-and-diagonalize path of
 * bse.version13.cpp (marcomarino123/Bethe-Salpeter-equation):
 *
 *   bse_compute_bands   Hamiltonian_TB::FFT / pull_ks_states / pull_ks_states_subset
 *                       (bse.version13.cpp:647-705, 706-777, 778-821), batched over k
 *   bse_build_kernel    Excitonic_Hamiltonian::extract_hbse_and_rcv (3041-3047):
 *                       pull_coulomb_potentials (2547-2766, model-W modes),
 *                       pull_resonant_part_and_rcv (2767-2928), spin_transformation (3048-3117),
 *                       add_coupling_part (2929-3040) when tamm_dancoff = 0
 *   bse_diagonalize     Excitonic_Hamiltonian::common_diagonalization (3120-3368)
 *   bse_oscillators     Excitonic_Hamiltonian::pull_excitonic_oscillator_force (3486-3502)
 *   bse_eps             the omega loop of pull_macroscopic_bse_dielectric_function (3525-3657)
 *   bse_solve           all of the above in one call (pull_macroscopic_bse_dielectric_function)
 *
 * Conventions
 *   - every complex array is interleaved double (re, im) == std::complex<double> ==
 *     arma::cx_double; matrices are column-major (== arma::cx_mat::memptr()).
 *   - lengths in Angstrom, momenta in 1/Angstrom (cartesian), energies in eV.
 *   - exciton index (spinless): r = c*nv*nk + v*nk + k  (k fastest), as the reference
 *     (bse.version13.cpp:2022, 2868).  Collinear spin: block b in 0..3 holds
 *     (v-spin, c-spin) = (0,0),(0,1),(1,0),(1,1) (bse.version13.cpp:2522-2526).
 *   - valence bands are counted top-down from the Fermi level, conduction bands
 *     bottom-up; conduction states live at k, valence states at k - q.
 *   - return value: 0 on success, a negative bse_status otherwise.  No entry point
 *     aborts, traps or prints; bse_last_error() gives a one-line reason.
 *   - one context per host thread; calls on one context are serialised on the
 *     context's own CUDA stream.  The caller owns every host buffer it passes.
 */
#ifndef BSE_GPU_H
#define BSE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bse_status {
    BSE_OK = 0,
    BSE_ERR_BAD_INPUT = -1,     /* sizes, NaN, non-Hermitian H(R) pairs, nv+nc > bands ... */
    BSE_ERR_NO_DEVICE = -2,
    BSE_ERR_OOM = -3,
    BSE_ERR_NOT_CONVERGED = -4, /* an iteration-capped device loop ran out of sweeps */
    BSE_ERR_CUDA = -5,
    BSE_ERR_STATE = -6          /* entry point called before the stage it needs */
} bse_status;

/* Bare Coulomb kind used for the exchange kernel v(q+G) (Coulomb_Potential::pull,
 * bse.version13.cpp:1273-1309).  BSE_V_BARE_2D has no counterpart in the reference
 * (its 2-D formula is not reproduced): v(q) = conv * Lz / (2 |q_par|). */
enum { BSE_V_BARE_3D = 0, BSE_V_BARE_2D = 1 };

/* Screened direct kernel W (pull_coulomb_potentials, bse.version13.cpp:2547-2766).
 *   BSE_W_EMPIRICAL: insulator, constant inverse dielectric constant, diagonal in G
 *                    (2697-2728), Delta k = 0 handled by the cell average of v.
 *   BSE_W_RYTOVA_KELDYSH: 2-D screened W = conv*Lz / (2 |q| (eps + r0 |q|)); no
 *                    counterpart in the reference; Delta k = 0 uses the disk average.
 *   BSE_W_BARE:      metal branch without screening, W = v(Delta k + G) (2584-2591).
 *   BSE_W_RPA:       insulator branch with adding_screening = 1 (2597-2690): W_GG'(dk) =
 *                    eps^-1_GG'(dk) v(dk + G') with the static RPA eps^-1 of the kept bands
 *                    (Dielectric_Function::pull_values 2214-2315; rpa_order 0 first order, 1 Dyson),
 *                    dk = 0 from rpa_points seeded points of the mini-BZ sphere.  Needs a complete
 *                    periodic k grid. */
enum { BSE_W_EMPIRICAL = 0, BSE_W_RYTOVA_KELDYSH = 1, BSE_W_BARE = 2, BSE_W_RPA = 3 };

/* Arithmetic of the build and of the dense solve. */
enum { BSE_FP64 = 0,   /* complex128 H, FP64 eigensolve */
       BSE_MIXED = 1   /* complex64 H, FP32 eigensolve, FP64 Rayleigh-Ritz of the lowest n_refine */ };

/* Dense eigensolver. */
enum { BSE_EIG_OWN = 0,       /* this library's tridiagonal reduction + bisection + inverse iteration */
       BSE_EIG_CUSOLVER = 1   /* cuSOLVER heevd, the plain library path */ };

typedef struct bse_model {
    int32_t nw;            /* Wannier functions per spin channel */
    int32_t n_spin;        /* 1: spinless / spin-orbital basis; 2: collinear (two hr.dat blocks) */
    int32_t n_r;           /* number of lattice vectors R */
    const double* r_cart;  /* 3 x n_r, cartesian R (Hamiltonian_TB ctor converts crystal->cartesian, 590-600) */
    const double* weights; /* n_r degeneracy weights; multiplied in, as Hamiltonian_TB::FFT does (676-677) */
    const double* h_r;     /* complex128 nw x nw x n_r per spin channel, spin slowest (arma::cx_cube layout) */
    const double* centres; /* 3 x nw per spin channel, spin slowest (Wannier centres, 617-619) */
    const double* lattice; /* 3 x 3 column-major, columns a1 a2 a3 (Crystal_Lattice, 85-124) */
    int32_t n_k;
    const double* k_cart;  /* 3 x n_k cartesian k-points (K_points, 183-242) */
    int32_t n_g;
    const double* g_cart;  /* 3 x n_g cartesian G vectors, G = 0 at index n_g/2 (G_points, 319-385) */
} bse_model;

typedef struct bse_params {
    int32_t nv, nc;              /* valence / conduction bands kept (3778-3781) */
    double fermi_energy;         /* valence = E <= E_F in every spin row (790-799) */
    double scissor;              /* added to conduction energies (815-816) */
    double q[3];                 /* excitonic momentum, q -> 0 (minval * x, 3590-3601) */
    int32_t tamm_dancoff;        /* 1: resonant block only; 0: full BSE with the coupling block B
                                    (add_coupling_part 2929-3040); BSE_MIXED uses the own solver;
                                    no effect with ipa = 1 */
    int32_t ipa;                 /* 1: no kernel, H = diag(E_c - E_v) (3346-3365) */
    int32_t small_momentum;      /* 1: G=0 pair density is the dipole i q.<c|r|v> (1535-1650) */
    int32_t coulomb_kind;        /* BSE_V_* */
    double coulomb_radius;       /* 3-D: v = conv / (|k|^2 + radius) (1283-1285) */
    double coulomb_min_k2;       /* v = 0 for |k|^2 below this (1281-1282) */
    int32_t w_kind;              /* BSE_W_* */
    double inv_eps;              /* empirical inverse dielectric constant (2697) */
    double rk_r0, rk_eps;        /* Rytova-Keldysh screening length (A) and environment eps */
    double spin_factor;          /* exchange prefactor (2 - spinorial) (2801); set < 0 for the default */
    int32_t precision;           /* BSE_FP64 / BSE_MIXED */
    int32_t eig_solver;          /* BSE_EIG_OWN / BSE_EIG_CUSOLVER */
    int32_t n_refine;            /* MIXED: lowest excitons refined in FP64 */
    double rpa_eta;              /* BSE_W_RPA: broadening of chi0 (eV), 0 for an insulator */
    int32_t rpa_order;           /* BSE_W_RPA: 0 eps^-1 = 1 + v chi0; 1 the Dyson equation */
    int32_t rpa_points;          /* BSE_W_RPA: sphere points for dk = 0 (even: +-q pairs) */
    uint64_t rpa_seed;           /* BSE_W_RPA: seed of those points (std::mt19937_64) */
} bse_params;

typedef struct bse_ctx bse_ctx;

/* Library */
const char* bse_status_string(int status);
const char* bse_last_error(const bse_ctx* ctx);
int bse_version(void);

/* Sizes derived from model+params: n_exc = (3*spin+1)*N eigenvalues, n_rho = (spin+1)*N
 * pair-density rows, n_h = dimension of the (full, before the spin split) BSE matrix.
 * Full BSE (tamm_dancoff = 0): each doubles (resonant rows, then anti-resonant). */
int bse_sizes(const bse_model* model, const bse_params* params,
              int64_t* n_bse, int64_t* n_exc, int64_t* n_rho, int64_t* n_h);

/* Context: validates and uploads the model to the device (cuda:0 unless changed with
 * bse_set_device before).  Replaces the constructors of Hamiltonian_TB, K_points,
 * G_points, Dipole_Elements and Excitonic_Hamiltonian (2485-2544). */
int bse_set_device(int device);
int bse_create(const bse_model* model, const bse_params* params, bse_ctx** out);
void bse_destroy(bse_ctx* ctx);

/* Stage a: batched H(k) assembly and per-k Hermitian eigensolves, subset selection.
 * Replaces Hamiltonian_TB::FFT / pull_ks_states / pull_ks_states_subset for every k. */
int bse_compute_bands(bse_ctx* ctx);

/* Copy the band subset out / in.  Layouts (doubles):
 *   e_c [n_spin_rows=2][nk][nc], e_v [2][nk][nv]           (spin-row 1 == row 0 when spinless)
 *   c_c [nk][nc][nb] complex, c_v [nk][nv][nb] complex       nb = nw * n_spin
 * Conduction states are at k, valence states at k - q.  bse_set_bands lets a caller
 * (or a test) inject states, e.g. to pin the gauge. */
int bse_get_bands(bse_ctx* ctx, double* e_c, double* e_v, double* c_c, double* c_v);
int bse_set_bands(bse_ctx* ctx, const double* e_c, const double* e_v,
                  const double* c_c, const double* c_v);

/* Stage b: kernel build == extract_hbse_and_rcv (3041-3047).  H stays on the device;
 * h_out (nullable) receives the full n_h x n_h complex128 matrix (spin-transformed when
 * n_spin == 2, 3048-3117), rho_out (nullable) the n_rho x n_g complex128 pair densities.
 * Full BSE: h_out = [[A, B], [-B^H, -conj(A)]] (2917-2923, 3035-3038), rho rows N..2N-1 hold
 * rho_vc (2937, 2950). */
int bse_build_kernel(bse_ctx* ctx, double* h_out, double* rho_out);

/* Stage b split over devices (the build's row tiles, one per GPU; no device collective).
 * bse_build_kernel_rows builds only the rows r = g * n_k + k with k in [k_lo, k_hi) (g over the
 * n_h / n_k groups of spin block, c and v) and writes them, ascending, to h_rows as a column-major
 * ((n_h / n_k) (k_hi - k_lo)) x n_h complex128 block; the context's own matrix is left incomplete
 * (a diagonalize before the next build or bse_set_kernel is BSE_ERR_STATE).  bse_set_kernel takes
 * the whole n_h x n_h complex128 matrix (column-major), e.g. gathered from those tiles on the
 * host, as if this context had built it; the pair densities and, in mixed precision, the FP64
 * matrix of the refinement come from the context's own bands and tables.  Tamm-Dancoff only
 * (BSE_ERR_BAD_INPUT for the full BSE).  Same path as bse_build_kernel: the rows of
 * Excitonic_Hamiltonian::pull_resonant_part_and_rcv (bse.version13.cpp:2767-2928) by k of the row. */
int bse_build_kernel_rows(bse_ctx* ctx, int32_t k_lo, int32_t k_hi, double* h_rows);
int bse_set_kernel(bse_ctx* ctx, const double* h);

/* Stage c: dense Hermitian eigensolve == common_diagonalization (3120-3368).
 * e_out (nullable): n_exc eigenvalues ascending (collinear: H0 block then H1 block).
 * a_out (nullable): eigenvectors (spinless n_bse x n_bse; collinear: the
 * spin-conserving block H1, 2N x 2N), complex128 column-major.
 * Full BSE (eig_gen of the 2N x 2N matrix, 3326): a structure-preserving solve through the
 * Cholesky factor of [[A, B], [B^H, conj(A)]], which must be positive definite (a stable
 * ground state; otherwise BSE_ERR_BAD_INPUT).  e_out: all 2N eigenvalues ascending, -E then +E;
 * a_out: 2N x 2N eigenvectors of H in that order, J-normalised: x^H diag(1,-1) x = sign(E).
 * Collinear full BSE: the two 4N spin blocks (H0 = {1,2}, H1 = {0,3} of every quadrant) each solved
 * that way; e_out holds H0's 4N values then H1's, a_out H1's 4N x 4N eigenvectors. */
int bse_diagonalize(bse_ctx* ctx, double* e_out, double* a_out);

/* Stage d: oscillator strengths f_l = sum_i conj(rho_i(G0)) A_il (3486-3502),
 * complex128, one per optically active exciton (spinless N, collinear 2N; full BSE 2N / 4N, from the
 * J-normalised vectors and rho = (rho_cv; rho_vc)). */
int bse_oscillators(bse_ctx* ctx, double* f_out);

/* Stage d: eps(w) = 1 - F sum_l |f_l|^2 / (w - E_l + i gamma), F = conv / (V nk)
 * (3531-3532, 3621-3634).  eps2 = Im eps, eps1 = Re eps (either nullable).  Full BSE
 * (3607-3620): eps(w) = 1 - F rho^H (w - H + i gamma)^{-1} J rho
 *                     = 1 - F sum_l sign(E_l) |f_l|^2 / (w - E_l + i gamma) over all 2N pairs. */
int bse_eps(bse_ctx* ctx, const double* omega, int32_t n_omega, double gamma,
            double* eps2, double* eps1);

/* All stages: bands -> build -> diagonalize -> oscillators -> eps. */
int bse_solve(bse_ctx* ctx, const double* omega, int32_t n_omega, double gamma,
              double* e_out, double* eps2, double* eps1);

/* Batched solves: runs bse_solve on n_ctx existing contexts (each on its own stream) from
 * n_workers host threads, so one model's host-side steps overlap the others' device work.
 * eps2 / eps1 (nullable) are n_ctx x n_omega row-major (model slowest).  Returns the first
 * failing status (every context is still attempted).  No counterpart in the reference. */
int bse_solve_many(bse_ctx** ctxs, int32_t n_ctx, const double* omega, int32_t n_omega, double gamma,
                   double* eps2, double* eps1, int32_t n_workers);

/* Device time (ms, CUDA events on the context stream) of the stages of the last calls:
 * [0] bands, [1] tables, [2] build, [3] eigensolve, [4] refinement, [5] oscillators, [6] eps,
 * [7] the whole of the last bse_solve; with BSE_EIG_OWN, the eigensolve's parts: [8] tridiagonal
 * reduction, [9] eigenvalues, [10] inverse iteration, [11] back-transformation, [12] clusters
 * (runs of eigenvalues FP32 bisection cannot separate, solved together); for the two-stage
 * reduction (N > 8192) the parts of [8]: [13] dense -> band, [14] bulge chase.  A stage keeps the
 * time of the last call that ran it. */
int bse_stage_times(const bse_ctx* ctx, double* ms, int32_t n);

/* Allocation-free dielectric function (no counterpart in the reference).  For callers that
 * cannot call cudaMalloc -- code inside a framework that has reserved the device memory for its
 * own pool gets nothing from the CUDA allocator -- this computes
 * eps(w) = 1 - prefactor * sum_l |f_l|^2 / (w - e_l + i gamma) from HOST arrays e[n_exc],
 * f[n_exc] (complex128) and omega[n_omega] into eps2/eps1 (host, either nullable), staging them
 * in one fixed 3.4 MiB file-scope device array that every GPU loading the library keeps until
 * exit.  Limits below; larger sizes return BSE_ERR_BAD_INPUT.  The first call on a device
 * resolves the array's address and keeps it for the process (not valid across a
 * cudaDeviceReset): make that first call before any stream capture.  Each call returns once its
 * outputs are on the host (it waits for `stream`).  Calls share the array: calls that overlap on
 * the GPU race.  stream: a cudaStream_t, or NULL for the default stream.
 * prefactor is F = conv / (V nk) of bse_eps.  The Tamm-Dancoff form: a full-BSE spectrum (signed
 * anti-resonant pairs) goes through bse_eps. */
#define BSE_EPS_NOALLOC_MAX_EXCITONS 131072
#define BSE_EPS_NOALLOC_MAX_OMEGA 16384
int bse_eps_noalloc(int64_t n_exc, const double* e, const double* f, double prefactor,
                    const double* omega, int32_t n_omega, double gamma,
                    double* eps2, double* eps1, void* stream);

/* Real-space Wannier matrix elements (Real_space_wannier + Dipole_Elements, bse.version13.cpp:
 * 1081-1212, 1441-1456, 1503-1650): M_ab(q + G) = sum_R exp(i q.(o + R)) A_ab(q + G; R),
 * A = Nsc V / Npts sum over the supercell grid of exp(i (q + G).r) w_a(r - R) w_b(r), for the
 * functions f [n_spin][nw][grid[0]][grid[1]][grid[2]] (last index fastest; normalised here on the
 * grid) on r = origin + sum_p (X_p / grid[p]) axes[p] (axes: 3 rows, the supercell's spanning
 * vectors; cells[p] unit cells per direction), R over n_int[p] cells centred on 0 in units of
 * lattice (3 rows), o = the supercell cell nearest to zero as cell indices (quirk kept from the
 * reference).  small_q != 0: the reference's q -> 0 form, i qhat.r in place of the phase, the same
 * for every G (g_list may be null).  m_out: [n_g][n_spin nw][n_spin nw] complex128, zero between
 * spin channels.  Allocates and frees its own device memory; synchronous.  The kernel build uses
 * point-like M; this gives the real-space M for callers that need it. */
int bse_wannier_m(int32_t n_spin, int32_t nw, const int32_t* grid, const int32_t* cells, const double* f,
                  double cell_volume, const double* origin, const double* axes, const double* lattice,
                  const int32_t* n_int, const double* q, int32_t n_g, const double* g_list, int32_t small_q,
                  double* m_out);

/* Diagnostics of the last solve: [0] max FP64 residual ||H x - theta x||_2 (eV) over the refined
 * eigenpairs (an eigenvalue error bound), [1] eigenvalue clusters the own solver solved together,
 * [2] refined eigenpairs, [3] eigenvector columns formed. */
int bse_diagnostics(const bse_ctx* ctx, double* out, int32_t n);

/* Launch/kernel statistics of the context: number of this library's kernel launches since
 * creation or the last reset. */
int64_t bse_kernel_launches(const bse_ctx* ctx);
void bse_reset_kernel_launches(bse_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* BSE_GPU_H */
