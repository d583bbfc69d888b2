// Stage d: oscillator strengths and the Lorentzian-broadened dielectric function.
//
// Replaces Excitonic_Hamiltonian::pull_excitonic_oscillator_force (TDA branch,
// bse.version13.cpp:3490-3493) and the omega loop of pull_macroscopic_bse_dielectric_function
// (3621-3634):
//   f_l   = sum_i conj(rho_i(G0)) A_il
//   eps(w) = 1 - F sum_l |f_l|^2 / (w - E_l + i gamma),  F = conv / (V nk)  (small q, 3531-3532)
// and, for the full BSE (3607-3620), eps(w) = 1 - F rho^H (w - H + i gamma)^{-1} J rho over all 2N
// J-normalised pairs: 1 - F sum_l sign(E_l) |f_l|^2 / (w - E_l + i gamma), rho = (rho_cv; rho_vc).
// The oscillator pass reads the eigenvector matrix once (HBM-bound, one warp per column,
// lanes stride down the column so every load is coalesced; FP32 partial sums per lane for
// complex64 vectors, combined in FP64 with warp shuffles).  The spectrum is one warp per
// frequency, lanes over excitons, FP64 sums reduced with warp shuffles.
#include "bse_internal.h"

namespace bse {
namespace {

template <typename T2, typename ACC>
__global__ void __launch_bounds__(256) oscillator_kernel(int64_t n, int64_t lda, int64_t ncols,
                                                         const double2* __restrict__ rho0,
                                                         const T2* __restrict__ A, double2* __restrict__ f) {
    const int lane = threadIdx.x & 31;
    const int64_t col = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (col >= ncols) return;
    const T2* a = A + col * lda;
    ACC r0 = 0, i0 = 0, r1 = 0, i1 = 0;
    int64_t i = lane;
    for (; i + 32 < n; i += 64) {
        const double2 p = rho0[i], q = rho0[i + 32];
        const T2 x = a[i], y = a[i + 32];
        // conj(rho) * a
        r0 += (ACC)p.x * (ACC)x.x + (ACC)p.y * (ACC)x.y;
        i0 += (ACC)p.x * (ACC)x.y - (ACC)p.y * (ACC)x.x;
        r1 += (ACC)q.x * (ACC)y.x + (ACC)q.y * (ACC)y.y;
        i1 += (ACC)q.x * (ACC)y.y - (ACC)q.y * (ACC)y.x;
    }
    for (; i < n; i += 32) {
        const double2 p = rho0[i];
        const T2 x = a[i];
        r0 += (ACC)p.x * (ACC)x.x + (ACC)p.y * (ACC)x.y;
        i0 += (ACC)p.x * (ACC)x.y - (ACC)p.y * (ACC)x.x;
    }
    double re = (double)r0 + (double)r1, im = (double)i0 + (double)i1;
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) f[col] = make_double2(re, im);
}

// signed_w (full BSE): every pair enters with the sign of its J-norm x^H J x = sign(E_l), so the
// anti-resonant pairs (E_l < 0) give -|f_l|^2 / (w - E_l + i gamma)
__global__ void __launch_bounds__(256) eps_kernel(int64_t n, const double* __restrict__ E,
                                                  const double2* __restrict__ f, const double* __restrict__ omega,
                                                  int n_omega, double gamma, double F, int signed_w,
                                                  double* __restrict__ eps2, double* __restrict__ eps1) {
    const int lane = threadIdx.x & 31;
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (s >= n_omega) return;
    const double w = omega[s], g2 = gamma * gamma;
    double a2 = 0, a1 = 0;
    for (int64_t l = lane; l < n; l += 32) {
        const double2 fl = f[l];
        const double el = E[l];
        double s2 = fl.x * fl.x + fl.y * fl.y;           // conj(f_l) f_l
        if (signed_w && el < 0.0) s2 = -s2;
        const double d = w - el;
        const double inv = s2 / (d * d + g2);
        a2 += inv * gamma;                               // -Im 1/(w - E + i gamma) = gamma / (d^2 + gamma^2)
        a1 += inv * d;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    }
    if (lane == 0) {
        eps2[s] = F * a2;                                // Im(1 - F sum |f|^2 / (w - E + i g))
        eps1[s] = 1.0 - F * a1;
    }
}

}  // namespace

int run_oscillators(bse_ctx* c) {
    int st;
    if (!c->eig_valid) return fail(c, BSE_ERR_STATE, "eigenvectors not available");
    stage_begin(c, 5);
    const int64_t n = c->n_opt;
    const double2* rho0 = c->d_rho + (size_t)c->n_rho * (c->ng / 2);
    // the own solver already produced f = y^H z for every exciton; only refined vectors need a new dot
    // (the full BSE's solves write f for every pair, refined ones included)
    const int64_t ncols = c->f_from_eig ? (c->coupled ? 0 : c->n_refined) : n;
    if (ncols > 0) {
        const unsigned blocks = (unsigned)((ncols * 32 + 255) / 256);
        if (c->p.precision == BSE_MIXED)
            oscillator_kernel<float2, float><<<blocks, 256, 0, c->stream>>>(n, n, ncols, rho0, (const float2*)c->d_A, c->d_f);
        else
            oscillator_kernel<double2, double><<<blocks, 256, 0, c->stream>>>(n, n, ncols, rho0, (const double2*)c->d_A, c->d_f);
        c->launches++;
    }
    stage_end(c, 5);
    if ((st = cuda_check(c, cudaGetLastError(), "oscillator kernel"))) return st;
    c->osc_valid = true;
    return BSE_OK;
}

// Launch of eps_kernel on caller-provided device buffers (used by the allocation-free entry point).
cudaError_t launch_eps_raw(int64_t n, const double* E, const double2* f, const double* omega, int n_omega,
                           double gamma, double F, double* eps2, double* eps1, cudaStream_t stream) {
    eps_kernel<<<(unsigned)(((int64_t)n_omega * 32 + 255) / 256), 256, 0, stream>>>(n, E, f, omega, n_omega, gamma, F, 0,
                                                                                eps2, eps1);
    return cudaGetLastError();
}

double eps_prefactor(const bse_ctx* c) {
    if (c->p.small_momentum) return kConv / (c->geo.vol * c->nk);
    return kConv / (kMinval * kMinval * c->geo.vol * c->nk);
}

int run_eps(bse_ctx* c, const double* omega, int n_omega, double gamma, double* eps2, double* eps1) {
    int st;
    if (!c->osc_valid) return fail(c, BSE_ERR_STATE, "oscillator strengths not available");
    if (n_omega <= 0) return BSE_OK;
    const size_t b = (size_t)n_omega * sizeof(double);
    if ((st = ensure_work(c, 3 * b + 512))) return st;
    double* d_om = (double*)c->d_work;
    double* d_e2 = d_om + n_omega;
    double* d_e1 = d_e2 + n_omega;
    if ((st = cuda_check(c, cudaMemcpyAsync(d_om, omega, b, cudaMemcpyHostToDevice, c->stream), "omega upload"))) return st;
    stage_begin(c, 6);
    const double* E = c->d_E + (c->n_exc - c->n_opt);   // collinear: the optically active block's values
    eps_kernel<<<(unsigned)(((int64_t)n_omega * 32 + 255) / 256), 256, 0, c->stream>>>(
        c->n_opt, E, c->d_f, d_om, n_omega, gamma, eps_prefactor(c), c->coupled ? 1 : 0, d_e2, d_e1);
    c->launches++;
    stage_end(c, 6);
    if ((st = cuda_check(c, cudaGetLastError(), "eps kernel"))) return st;
    if (eps2 && (st = cuda_check(c, cudaMemcpyAsync(eps2, d_e2, b, cudaMemcpyDeviceToHost, c->stream), "eps2 copy"))) return st;
    if (eps1 && (st = cuda_check(c, cudaMemcpyAsync(eps1, d_e1, b, cudaMemcpyDeviceToHost, c->stream), "eps1 copy"))) return st;
    return cuda_check(c, cudaStreamSynchronize(c->stream), "eps sync");
}

}  // namespace bse
