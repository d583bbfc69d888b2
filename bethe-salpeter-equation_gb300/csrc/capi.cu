// C ABI of include/bse_gpu.h: context lifetime, validation, uploads and stage sequencing.
//
// The context plays the role of the reference's object graph (Crystal_Lattice, K_points,
// G_points, Hamiltonian_TB, Dipole_Elements, Excitonic_Hamiltonian, built in main(),
// bse.version13.cpp:3686-3848) with the model resident on the device.  Every entry point
// returns a status code and never aborts (the reference prints and continues, 499-501).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <new>
#include <thread>

#include "bse_internal.h"

namespace {
int g_device = 0;
thread_local std::string g_create_err;
}

namespace bse {

int fail(bse_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    else g_create_err = msg;
    return code;
}

int cuda_check(bse_ctx* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return BSE_OK;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(c, BSE_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
    }
    return fail(c, BSE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int ensure_work(bse_ctx* c, size_t bytes) {
    if (bytes <= c->work_bytes) return BSE_OK;
    if (c->d_work) {
        cudaStreamSynchronize(c->stream);
        cudaFree(c->d_work);
        c->d_work = nullptr;
        c->work_bytes = 0;
    }
    int st = cuda_check(c, cudaMalloc(&c->d_work, bytes), "workspace");
    if (st) return st;
    c->work_bytes = bytes;
    return BSE_OK;
}

void stage_begin(bse_ctx* c, int s) {
    if (!c->stage_mute) cudaEventRecord(c->ev[2 * s], c->stream);
}
void stage_end(bse_ctx* c, int s) {
    if (c->stage_mute) return;
    cudaEventRecord(c->ev[2 * s + 1], c->stream);
    c->stage_ms[s] = -1.0;   // resolved lazily in bse_stage_times
}

cudaEvent_t* kernel_timer(bse_ctx* c, int kind, double bytes, double flops) {
    if (!c->ktime) return nullptr;
    if (c->kt_used == c->kt.size()) {
        bse_ctx::KernelTime r;
        if (cudaEventCreate(&r.ev[0]) != cudaSuccess || cudaEventCreate(&r.ev[1]) != cudaSuccess) {
            cudaGetLastError();
            if (r.ev[0]) cudaEventDestroy(r.ev[0]);
            return nullptr;
        }
        c->kt.push_back(r);
    }
    auto& r = c->kt[c->kt_used++];
    r.kind = kind;
    r.bytes = bytes;
    r.flops = flops;
    return r.ev;
}

}  // namespace bse

using namespace bse;

namespace {

bool finite_all(const double* p, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (!std::isfinite(p[i])) return false;
    return true;
}

template <typename T>
int dmalloc(bse_ctx* c, T** p, size_t bytes, const char* what) {
    return cuda_check(c, cudaMalloc((void**)p, std::max<size_t>(bytes, 16)), what);
}

int upload(bse_ctx* c, void* dst, const void* src, size_t bytes, const char* what) {
    return cuda_check(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream), what);
}

// Crystal coordinates of the k list on a lattice?  (k_cryst_i = a_i . k / 2 pi)
void analyse_k(bse_ctx* c, const bse_model* m) {
    DeltaMap& d = c->dmap;
    const int nk = m->n_k;
    std::vector<double> kc((size_t)3 * nk);
    for (int k = 0; k < nk; k++)
        for (int i = 0; i < 3; i++) {
            double s = 0;
            for (int x = 0; x < 3; x++) s += m->lattice[3 * i + x] * m->k_cart[3 * k + x];
            kc[3 * k + i] = s / (2.0 * kPi);
        }
    bool ok = true;
    double vmin[3];
    for (int i = 0; i < 3 && ok; i++) {
        std::vector<double> v(nk);
        for (int k = 0; k < nk; k++) v[k] = kc[3 * k + i];
        std::sort(v.begin(), v.end());
        std::vector<double> u;
        for (double x : v)
            if (u.empty() || x - u.back() > 1e-9) u.push_back(x);
        vmin[i] = u[0];
        d.m[i] = (int)u.size();
        d.step[i] = 0;
        if (u.size() > 1) {
            d.step[i] = u[1] - u[0];
            for (size_t j = 1; j < u.size(); j++)
                if (std::fabs((u[j] - u[j - 1]) - d.step[i]) > 1e-9) ok = false;
        }
        if (d.m[i] > 1023) ok = false;
    }
    if (ok) {
        d.idx.resize(nk);
        for (int k = 0; k < nk; k++) {
            int32_t packed = 0;
            for (int i = 0; i < 3; i++) {
                int ii = d.m[i] > 1 ? (int)std::lround((kc[3 * k + i] - vmin[i]) / d.step[i]) : 0;
                packed |= (ii & 1023) << (10 * i);
            }
            d.idx[k] = packed;
        }
        d.on_grid = true;
        // a complete periodic grid: k - dk and k + dk are grid points for every grid offset dk
        const int64_t ncell = (int64_t)d.m[0] * d.m[1] * d.m[2];
        bool per = ncell == nk;
        for (int i = 0; i < 3 && per; i++)
            if (d.m[i] > 1 && std::fabs(d.step[i] * d.m[i] - 1.0) > 1e-9) per = false;
        if (per) {
            d.inv.assign(ncell, -1);
            for (int k = 0; k < nk && per; k++) {
                const int32_t x = d.idx[k];
                const int64_t cell = ((int64_t)(x & 1023) * d.m[1] + ((x >> 10) & 1023)) * d.m[2] + ((x >> 20) & 1023);
                if (d.inv[cell] >= 0) per = false;
                else d.inv[cell] = k;
            }
        }
        d.periodic = per;
        if (!per) d.inv.clear();
        d.n_delta = (int64_t)(2 * d.m[0] - 1) * (2 * d.m[1] - 1) * (2 * d.m[2] - 1);
    } else {
        d.on_grid = false;
        d.n_delta = (int64_t)nk * nk;
        for (int i = 0; i < 3; i++) { d.m[i] = 1; d.step[i] = 0; }
    }
}

double cell_average(const bse_ctx* c) {
    const bse_params& p = c->p;
    const Geometry& g = c->geo;
    const int nk = c->nk;
    if (p.w_kind == BSE_W_RYTOVA_KELDYSH || p.coulomb_kind == BSE_V_BARE_2D) {
        double abz = (2.0 * kPi) * (2.0 * kPi) / g.area;
        double qc = std::sqrt(abz / (kPi * nk));
        if (p.w_kind == BSE_W_RYTOVA_KELDYSH) {
            if (p.rk_r0 > 0) return kConv * g.lz * std::log(1.0 + p.rk_r0 * qc / p.rk_eps) / (p.rk_r0 * qc * qc);
            return kConv * g.lz / (p.rk_eps * qc);
        }
        return kConv * g.lz / qc;
    }
    // sphere of the k-point's volume share, intended radius (Q7), bse.version13.cpp:2599, 2628
    double rs = 2.0 * kPi * std::pow(3.0 / (4.0 * kPi * nk * g.vol), 1.0 / 3.0);
    return kConv * 4.0 * kPi * rs * nk * g.vol / std::pow(2.0 * kPi, 3);
}

int validate(const bse_model* m, const bse_params* p) {
    if (!m || !p) return fail(nullptr, BSE_ERR_BAD_INPUT, "null model or params");
    if (m->nw < 1 || m->nw > kMaxNw) return fail(nullptr, BSE_ERR_BAD_INPUT, "nw must be in [1, 16]");
    if (m->n_spin != 1 && m->n_spin != 2) return fail(nullptr, BSE_ERR_BAD_INPUT, "n_spin must be 1 or 2");
    if (m->n_r < 1 || m->n_k < 1 || m->n_g < 1) return fail(nullptr, BSE_ERR_BAD_INPUT, "empty R, k or G list");
    if (!m->r_cart || !m->weights || !m->h_r || !m->centres || !m->lattice || !m->k_cart || !m->g_cart)
        return fail(nullptr, BSE_ERR_BAD_INPUT, "null model array");
    if (p->nv < 1 || p->nc < 1 || p->nv + p->nc > m->nw)
        return fail(nullptr, BSE_ERR_BAD_INPUT, "need 1 <= nv, nc and nv + nc <= nw");
    if (p->nv > 8 || p->nc > 8) return fail(nullptr, BSE_ERR_BAD_INPUT, "nv, nc above 8 are not supported");
    if (p->tamm_dancoff != 0 && p->tamm_dancoff != 1) return fail(nullptr, BSE_ERR_BAD_INPUT, "tamm_dancoff must be 0 or 1");
    if (p->precision != BSE_FP64 && p->precision != BSE_MIXED) return fail(nullptr, BSE_ERR_BAD_INPUT, "precision");
    if (p->tamm_dancoff == 0 && !p->ipa && p->precision == BSE_MIXED) {
        if (p->eig_solver != BSE_EIG_OWN)
            return fail(nullptr, BSE_ERR_BAD_INPUT, "the mixed full BSE (tamm_dancoff = 0) uses the own eigensolver");
    }
    if (p->eig_solver != BSE_EIG_OWN && p->eig_solver != BSE_EIG_CUSOLVER) return fail(nullptr, BSE_ERR_BAD_INPUT, "eig_solver");
    if (p->coulomb_kind != BSE_V_BARE_3D && p->coulomb_kind != BSE_V_BARE_2D) return fail(nullptr, BSE_ERR_BAD_INPUT, "coulomb_kind");
    if (p->w_kind < BSE_W_EMPIRICAL || p->w_kind > BSE_W_RPA) return fail(nullptr, BSE_ERR_BAD_INPUT, "w_kind");
    if (p->w_kind == BSE_W_RPA && !p->ipa) {
        if (p->rpa_order != 0 && p->rpa_order != 1) return fail(nullptr, BSE_ERR_BAD_INPUT, "rpa_order must be 0 or 1");
        if (p->rpa_points < 2 || p->rpa_points % 2) return fail(nullptr, BSE_ERR_BAD_INPUT, "rpa_points must be even and >= 2");
        if (!(p->rpa_eta >= 0.0) || !std::isfinite(p->rpa_eta)) return fail(nullptr, BSE_ERR_BAD_INPUT, "rpa_eta must be >= 0");
    }
    const size_t nw = m->nw, nr = m->n_r, ns = m->n_spin;
    if (!finite_all(m->r_cart, 3 * nr) || !finite_all(m->weights, nr) || !finite_all(m->h_r, 2 * nw * nw * nr * ns) ||
        !finite_all(m->centres, 3 * nw * ns) || !finite_all(m->lattice, 9) || !finite_all(m->k_cart, 3 * (size_t)m->n_k) ||
        !finite_all(m->g_cart, 3 * (size_t)m->n_g))
        return fail(nullptr, BSE_ERR_BAD_INPUT, "NaN or Inf in the model");
    const double pv[] = {p->fermi_energy, p->scissor, p->q[0], p->q[1], p->q[2], p->coulomb_radius, p->coulomb_min_k2,
                         p->inv_eps, p->rk_r0, p->rk_eps, p->spin_factor};
    if (!finite_all(pv, sizeof(pv) / sizeof(double))) return fail(nullptr, BSE_ERR_BAD_INPUT, "NaN or Inf in the parameters");
    if (p->small_momentum && p->q[0] * p->q[0] + p->q[1] * p->q[1] + p->q[2] * p->q[2] == 0.0)
        return fail(nullptr, BSE_ERR_BAD_INPUT, "q must be non-zero");
    // H(R) = H(-R)^dagger for every R whose partner is present, so every H(k) is Hermitian
    double hmax = 0;
    for (size_t i = 0; i < 2 * nw * nw * nr * ns; i++) hmax = std::max(hmax, std::fabs(m->h_r[i]));
    for (size_t s = 0; s < ns; s++)
        for (size_t r = 0; r < nr; r++) {
            const double* R = m->r_cart + 3 * r;
            size_t rm = nr;
            for (size_t j = 0; j < nr; j++) {
                const double* Q = m->r_cart + 3 * j;
                if (std::fabs(R[0] + Q[0]) + std::fabs(R[1] + Q[1]) + std::fabs(R[2] + Q[2]) < 1e-8) { rm = j; break; }
            }
            if (rm == nr) return fail(nullptr, BSE_ERR_BAD_INPUT, "lattice vector -R missing from the R list");
            const double wr = m->weights[r], wm = m->weights[rm];
            for (size_t l = 0; l < nw; l++)
                for (size_t mm = 0; mm < nw; mm++) {
                    const double* a = m->h_r + 2 * (((s * nr + r) * nw + mm) * nw + l);    // H_lm(R)
                    const double* b = m->h_r + 2 * (((s * nr + rm) * nw + l) * nw + mm);   // H_ml(-R)
                    if (std::fabs(wr * a[0] - wm * b[0]) + std::fabs(wr * a[1] + wm * b[1]) > 1e-10 * (1.0 + hmax))
                        return fail(nullptr, BSE_ERR_BAD_INPUT, "non-Hermitian H(R) pair: H(R) != H(-R)^dagger");
                }
        }
    return BSE_OK;
}

void destroy_ctx(bse_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    if (c->side2) cudaStreamSynchronize(c->side2);
    void* ptrs[] = {c->d_rcart, c->d_weights, c->d_hr, c->d_centres, c->d_k, c->d_bmat, c->d_kidx, c->d_g, c->d_status,
                    c->d_ec, c->d_ev, c->d_cc, c->d_cv, c->d_phi, c->d_phi_c, c->d_phi32, c->d_X, c->d_qx, c->d_qx32, c->d_rho,
                    c->d_H, c->d_H64, c->d_blk, c->d_aux, c->d_E, c->d_f, c->d_work};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->cublas) cublasDestroy(c->cublas);
    if (c->cusolver) cusolverDnDestroy(c->cusolver);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_h64) cudaEventDestroy(c->ev_h64);
    for (auto& r : c->kt)
        for (cudaEvent_t e : r.ev)
            if (e) cudaEventDestroy(e);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->side2) cudaStreamDestroy(c->side2);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

}  // namespace

extern "C" {

const char* bse_status_string(int s) {
    switch (s) {
        case BSE_OK: return "BSE_OK";
        case BSE_ERR_BAD_INPUT: return "BSE_ERR_BAD_INPUT";
        case BSE_ERR_NO_DEVICE: return "BSE_ERR_NO_DEVICE";
        case BSE_ERR_OOM: return "BSE_ERR_OOM";
        case BSE_ERR_NOT_CONVERGED: return "BSE_ERR_NOT_CONVERGED";
        case BSE_ERR_CUDA: return "BSE_ERR_CUDA";
        case BSE_ERR_STATE: return "BSE_ERR_STATE";
        default: return "BSE_ERR_UNKNOWN";
    }
}

const char* bse_last_error(const bse_ctx* c) { return c ? c->err.c_str() : g_create_err.c_str(); }

int bse_version(void) { return 10000; }

int bse_sizes(const bse_model* m, const bse_params* p, int64_t* n_bse, int64_t* n_exc, int64_t* n_rho, int64_t* n_h) {
    if (!m || !p) return BSE_ERR_BAD_INPUT;
    const int64_t N = (int64_t)m->n_k * p->nc * p->nv;
    const int S = m->n_spin - 1;
    const int64_t x = (p->tamm_dancoff == 0 && !p->ipa) ? 2 : 1;   // full BSE: every size doubles
    if (n_bse) *n_bse = N;
    if (n_exc) *n_exc = x * (3 * S + 1) * N;
    if (n_rho) *n_rho = x * (S + 1) * N;
    if (n_h) *n_h = x * (3 * S + 1) * N;
    return BSE_OK;
}

int bse_set_device(int device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(nullptr, BSE_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= n) return fail(nullptr, BSE_ERR_BAD_INPUT, "device index out of range");
    g_device = device;
    return BSE_OK;
}

int bse_create(const bse_model* m, const bse_params* p, bse_ctx** out) {
    if (!out) return fail(nullptr, BSE_ERR_BAD_INPUT, "null output pointer");
    *out = nullptr;
    int st = validate(m, p);
    if (st) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(nullptr, BSE_ERR_NO_DEVICE, "no CUDA device");
    }
    bse_ctx* c = new (std::nothrow) bse_ctx();
    if (!c) return fail(nullptr, BSE_ERR_OOM, "host allocation");
    c->device = g_device;
    c->p = *p;
    c->nw = m->nw; c->ns = m->n_spin; c->nb = c->nw * c->ns; c->nk = m->n_k; c->ng = m->n_g;
    c->nv = p->nv; c->nc = p->nc; c->S = c->ns - 1; c->nr = m->n_r;
    c->N = (int64_t)c->nk * c->nc * c->nv;
    c->n_h = (3 * c->S + 1) * c->N;
    c->n_rho = (c->S + 1) * c->N;
    c->n_exc = (3 * c->S + 1) * c->N;
    c->n_opt = (c->S + 1) * c->N;
    c->coupled = p->tamm_dancoff == 0 && !p->ipa;
    if (c->coupled) {   // resonant + anti-resonant rows: every size doubles (collinear: two 4N blocks)
        c->n_h *= 2;
        c->n_rho *= 2;
        c->n_exc *= 2;
        c->n_opt *= 2;
    }
    // geometry (Crystal_Lattice, bse.version13.cpp:85-124)
    {
        const double* a = m->lattice;
        double c12[3] = {a[1] * a[5] - a[2] * a[4], a[2] * a[3] - a[0] * a[5], a[0] * a[4] - a[1] * a[3]};
        double det = c12[0] * a[6] + c12[1] * a[7] + c12[2] * a[8];
        c->geo.vol = std::fabs(det);
        c->geo.area = std::sqrt(c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2]);
        for (int i = 0; i < 3; i++) c->geo.normal[i] = c12[i] / c->geo.area;
        c->geo.lz = c->geo.vol / c->geo.area;
    }
    Interaction& it = c->itx;
    it.coulomb_kind = p->coulomb_kind; it.w_kind = p->w_kind;
    it.radius = p->coulomb_radius; it.min_k2 = p->coulomb_min_k2; it.inv_eps = p->inv_eps;
    it.rk_r0 = p->rk_r0; it.rk_eps = p->rk_eps;
    it.nx = c->geo.normal[0]; it.ny = c->geo.normal[1]; it.nz = c->geo.normal[2]; it.lz = c->geo.lz;
    it.cell_avg = cell_average(c);
    analyse_k(c, m);
    if (p->w_kind == BSE_W_RPA && !p->ipa && !c->dmap.periodic) {
        destroy_ctx(c);
        return fail(nullptr, BSE_ERR_BAD_INPUT, "RPA screening needs a complete periodic k grid (k - dk on the grid)");
    }
    const int NWs = c->nw <= 2 ? 2 : c->nw <= 4 ? 4 : c->nw <= 8 ? 8 : 16;
    const int nblk = 3 * c->S + 1;
    if (!c->dmap.on_grid && (double)c->dmap.n_delta * nblk * NWs * NWs * 24.0 > 16e9) {
        destroy_ctx(c);
        return fail(nullptr, BSE_ERR_BAD_INPUT, "k list is not a lattice and nk^2 Delta-k tables would exceed 16 GB");
    }
    if ((st = cuda_check(c, cudaSetDevice(c->device), "set device"))) { g_create_err = c->err; destroy_ctx(c); return st; }
#define CK(x)                                   \
    do {                                        \
        if ((st = (x))) {                       \
            g_create_err = c->err;              \
            destroy_ctx(c);                     \
            return st;                          \
        }                                       \
    } while (0)
    CK(cuda_check(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream"));
    CK(cuda_check(c, cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking), "side stream"));
    CK(cuda_check(c, cudaStreamCreateWithFlags(&c->side2, cudaStreamNonBlocking), "side stream"));
    CK(cuda_check(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "event"));
    CK(cuda_check(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "event"));
    CK(cuda_check(c, cudaEventCreateWithFlags(&c->ev_h64, cudaEventDisableTiming), "event"));
    for (auto& e : c->ev) CK(cuda_check(c, cudaEventCreate(&e), "event"));
    c->ktime = std::getenv("BSE_KERNEL_TIMING") != nullptr;
    if (const char* v = std::getenv("BSE_TEST_SPIN_LIMIT")) c->spin_limit = (unsigned)std::max(1L, std::atol(v));
    if (const char* v = std::getenv("BSE_TEST_JACOBI_SWEEPS")) c->jacobi_sweeps = std::max(0, std::atoi(v));
    if (cublasCreate(&c->cublas) != CUBLAS_STATUS_SUCCESS) CK(fail(c, BSE_ERR_CUDA, "cublasCreate"));
    if (cusolverDnCreate(&c->cusolver) != CUSOLVER_STATUS_SUCCESS) CK(fail(c, BSE_ERR_CUDA, "cusolverDnCreate"));
    cublasSetStream(c->cublas, c->stream);
    cusolverDnSetStream(c->cusolver, c->stream);
    const size_t nw = c->nw, nr = c->nr, ns = c->ns, nk = c->nk, ng = c->ng, nb = c->nb;
    CK(dmalloc(c, &c->d_rcart, 3 * nr * 8, "R"));
    CK(dmalloc(c, &c->d_weights, nr * 8, "weights"));
    CK(dmalloc(c, &c->d_hr, nw * nw * nr * ns * 16, "H(R)"));
    CK(dmalloc(c, &c->d_centres, 3 * nw * ns * 8, "centres"));
    CK(dmalloc(c, &c->d_k, 3 * nk * 8, "k"));
    CK(dmalloc(c, &c->d_bmat, 9 * 8, "b"));
    CK(dmalloc(c, &c->d_kidx, nk * 4, "k index"));
    CK(dmalloc(c, &c->d_g, 3 * ng * 8, "G"));
    CK(dmalloc(c, &c->d_status, 16, "status"));
    CK(cuda_check(c, cudaMemset(c->d_status, 0, 16), "status clear"));
    CK(dmalloc(c, &c->d_ec, 2 * nk * c->nc * 8, "e_c"));
    CK(dmalloc(c, &c->d_ev, 2 * nk * c->nv * 8, "e_v"));
    CK(dmalloc(c, &c->d_cc, nk * c->nc * nb * 16, "c_c"));
    CK(dmalloc(c, &c->d_cv, nk * c->nv * nb * 16, "c_v"));
    CK(dmalloc(c, &c->d_rho, (size_t)c->n_rho * ng * 16, "rho"));
    CK(dmalloc(c, &c->d_X, ns * ns * nw * nw * 16, "X"));
    CK(dmalloc(c, &c->d_qx, (size_t)c->N * nw * ns * ns * 16, "Qx"));
    const size_t nphi = (size_t)c->dmap.n_delta * nblk * NWs * NWs;
    CK(dmalloc(c, &c->d_phi, nphi * 16, "Phi"));
    if (c->coupled && p->w_kind == BSE_W_RPA) CK(dmalloc(c, &c->d_phi_c, nphi * 16, "Phi (coupling)"));
    const bool mixed = p->precision == BSE_MIXED;
    if (mixed) {
        CK(dmalloc(c, &c->d_phi32, nphi * 8, "Phi32"));
        CK(dmalloc(c, &c->d_qx32, (size_t)c->N * nw * ns * ns * 8, "Qx32"));
    }
    c->h_elem = mixed && !c->coupled ? 8 : 16;   // the full BSE is built in FP64 in both precisions
    CK(dmalloc(c, &c->d_H, (size_t)c->n_h * c->n_h * c->h_elem, "H"));
    if (c->coupled) {
        // spinless: L^H J L (2N); collinear: the two 4N blocks M0, M1 and L^H J L (4N)
        const size_t nb = c->S ? (size_t)c->n_opt : (size_t)c->n_h;
        CK(dmalloc(c, &c->d_blk, (c->S ? 3 : 1) * nb * nb * sizeof(double2), "full-BSE blocks"));
        CK(dmalloc(c, &c->d_aux, nb * sizeof(double2), "L^-1 rho"));
    } else if (c->S) {
        CK(dmalloc(c, &c->d_blk, 2 * (size_t)(2 * c->N) * (2 * c->N) * c->h_elem, "spin blocks"));
    }
    if (mixed && !c->coupled && !p->ipa && p->n_refine > 0) {
        const size_t n64 = c->S ? 4 * c->N : c->N;
        CK(dmalloc(c, &c->d_H64, n64 * n64 * 16, "H64"));
    }
    CK(dmalloc(c, &c->d_E, (size_t)c->n_exc * 8, "E"));
    CK(dmalloc(c, &c->d_f, (size_t)c->n_opt * 16, "f"));
    // uploads
    std::vector<double2> hr(nw * nw * nr * ns);
    std::memcpy(hr.data(), m->h_r, hr.size() * 16);
    CK(upload(c, c->d_rcart, m->r_cart, 3 * nr * 8, "R"));
    CK(upload(c, c->d_weights, m->weights, nr * 8, "weights"));
    CK(upload(c, c->d_hr, m->h_r, hr.size() * 16, "H(R)"));
    CK(upload(c, c->d_centres, m->centres, 3 * nw * ns * 8, "centres"));
    CK(upload(c, c->d_k, m->k_cart, 3 * nk * 8, "k"));
    CK(upload(c, c->d_g, m->g_cart, 3 * ng * 8, "G"));
    {
        // reciprocal vectors b_i = 2 pi (a_j x a_k) / V as columns
        const double* a = m->lattice;
        double b[9];
        const double* a0 = a; const double* a1 = a + 3; const double* a2 = a + 6;
        double x[3][3] = {{a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]},
                          {a2[1] * a0[2] - a2[2] * a0[1], a2[2] * a0[0] - a2[0] * a0[2], a2[0] * a0[1] - a2[1] * a0[0]},
                          {a0[1] * a1[2] - a0[2] * a1[1], a0[2] * a1[0] - a0[0] * a1[2], a0[0] * a1[1] - a0[1] * a1[0]}};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) b[3 * i + j] = x[i][j] * 2.0 * kPi / c->geo.vol;
        CK(upload(c, c->d_bmat, b, 72, "b"));
        std::memcpy(c->bmat_h, b, sizeof(b));
    }
    if (c->dmap.on_grid) CK(upload(c, c->d_kidx, c->dmap.idx.data(), nk * 4, "k index"));
    CK(cuda_check(c, cudaStreamSynchronize(c->stream), "uploads"));
#undef CK
    *out = c;
    return BSE_OK;
}

void bse_destroy(bse_ctx* c) { destroy_ctx(c); }

int bse_compute_bands(bse_ctx* c) {
    if (!c) return BSE_ERR_BAD_INPUT;
    cudaSetDevice(c->device);
    return run_bands(c);
}

int bse_get_bands(bse_ctx* c, double* e_c, double* e_v, double* c_c, double* c_v) {
    if (!c) return BSE_ERR_BAD_INPUT;
    if (!c->bands_valid) return fail(c, BSE_ERR_STATE, "bands not computed");
    int st;
    const size_t nk = c->nk, nb = c->nb;
    if (e_c && (st = cuda_check(c, cudaMemcpyAsync(e_c, c->d_ec, 2 * nk * c->nc * 8, cudaMemcpyDeviceToHost, c->stream), "e_c"))) return st;
    if (e_v && (st = cuda_check(c, cudaMemcpyAsync(e_v, c->d_ev, 2 * nk * c->nv * 8, cudaMemcpyDeviceToHost, c->stream), "e_v"))) return st;
    if (c_c && (st = cuda_check(c, cudaMemcpyAsync(c_c, c->d_cc, nk * c->nc * nb * 16, cudaMemcpyDeviceToHost, c->stream), "c_c"))) return st;
    if (c_v && (st = cuda_check(c, cudaMemcpyAsync(c_v, c->d_cv, nk * c->nv * nb * 16, cudaMemcpyDeviceToHost, c->stream), "c_v"))) return st;
    return cuda_check(c, cudaStreamSynchronize(c->stream), "get bands");
}

int bse_set_bands(bse_ctx* c, const double* e_c, const double* e_v, const double* c_c, const double* c_v) {
    if (!c || !e_c || !e_v || !c_c || !c_v) return BSE_ERR_BAD_INPUT;
    const size_t nk = c->nk, nb = c->nb;
    if (!finite_all(e_c, 2 * nk * c->nc) || !finite_all(e_v, 2 * nk * c->nv) || !finite_all(c_c, 2 * nk * c->nc * nb) ||
        !finite_all(c_v, 2 * nk * c->nv * nb))
        return fail(c, BSE_ERR_BAD_INPUT, "NaN or Inf in the band states");
    int st;
    if ((st = upload(c, c->d_ec, e_c, 2 * nk * c->nc * 8, "e_c"))) return st;
    if ((st = upload(c, c->d_ev, e_v, 2 * nk * c->nv * 8, "e_v"))) return st;
    if ((st = upload(c, c->d_cc, c_c, nk * c->nc * nb * 16, "c_c"))) return st;
    if ((st = upload(c, c->d_cv, c_v, nk * c->nv * nb * 16, "c_v"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "set bands"))) return st;
    c->bands_valid = true;
    c->tables_valid = c->h_valid = c->eig_valid = c->osc_valid = false;
    return BSE_OK;
}

int bse_build_kernel(bse_ctx* c, double* h_out, double* rho_out) {
    if (!c) return BSE_ERR_BAD_INPUT;
    cudaSetDevice(c->device);
    int st;
    if (!c->bands_valid && (st = run_bands(c))) return st;
    return run_build(c, h_out != nullptr, h_out, rho_out);
}

int bse_build_kernel_rows(bse_ctx* c, int32_t k_lo, int32_t k_hi, double* h_rows) {
    if (!c) return BSE_ERR_BAD_INPUT;
    cudaSetDevice(c->device);
    int st;
    if (!c->bands_valid && (st = run_bands(c))) return st;
    return run_build_rows(c, k_lo, k_hi, h_rows);
}

int bse_set_kernel(bse_ctx* c, const double* h) {
    if (!c) return BSE_ERR_BAD_INPUT;
    cudaSetDevice(c->device);
    return run_set_kernel(c, h);
}

int bse_diagonalize(bse_ctx* c, double* e_out, double* a_out) {
    if (!c) return BSE_ERR_BAD_INPUT;
    cudaSetDevice(c->device);
    int st;
    if (!c->eig_valid || c->h_valid) {
        if ((st = run_eig(c, a_out != nullptr))) return st;
    }
    if (a_out && c->n_vec_valid < c->n_opt)
        return fail(c, BSE_ERR_STATE, "eigenvectors were not formed: rebuild, then call bse_diagonalize with a_out");
    if (e_out && (st = cuda_check(c, cudaMemcpyAsync(e_out, c->d_E, c->n_exc * 8, cudaMemcpyDeviceToHost, c->stream), "E copy"))) return st;
    if (a_out) {
        const size_t n = (size_t)c->n_opt * c->n_opt;
        if (c->p.precision == BSE_MIXED) {
            std::vector<float2> tmp(n);
            if ((st = cuda_check(c, cudaMemcpyAsync(tmp.data(), c->d_A, n * 8, cudaMemcpyDeviceToHost, c->stream), "A copy"))) return st;
            if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "A sync"))) return st;
            for (size_t i = 0; i < n; i++) { a_out[2 * i] = tmp[i].x; a_out[2 * i + 1] = tmp[i].y; }
        } else if ((st = cuda_check(c, cudaMemcpyAsync(a_out, c->d_A, n * 16, cudaMemcpyDeviceToHost, c->stream), "A copy"))) {
            return st;
        }
    }
    return cuda_check(c, cudaStreamSynchronize(c->stream), "diagonalize");
}

int bse_oscillators(bse_ctx* c, double* f_out) {
    if (!c) return BSE_ERR_BAD_INPUT;
    cudaSetDevice(c->device);
    int st;
    if (!c->osc_valid && (st = run_oscillators(c))) return st;
    if (f_out && (st = cuda_check(c, cudaMemcpyAsync(f_out, c->d_f, c->n_opt * 16, cudaMemcpyDeviceToHost, c->stream), "f copy"))) return st;
    return cuda_check(c, cudaStreamSynchronize(c->stream), "oscillators");
}

int bse_eps(bse_ctx* c, const double* omega, int32_t n_omega, double gamma, double* eps2, double* eps1) {
    if (!c) return BSE_ERR_BAD_INPUT;
    if (n_omega < 0 || (n_omega > 0 && !omega) || !std::isfinite(gamma)) return fail(c, BSE_ERR_BAD_INPUT, "omega grid");
    cudaSetDevice(c->device);
    return run_eps(c, omega, n_omega, gamma, eps2, eps1);
}

int bse_solve(bse_ctx* c, const double* omega, int32_t n_omega, double gamma, double* e_out, double* eps2, double* eps1) {
    if (!c) return BSE_ERR_BAD_INPUT;
    cudaSetDevice(c->device);
    int st;
    stage_begin(c, 7);
    if ((st = run_bands(c))) return st;
    if ((st = run_build(c, false, nullptr, nullptr))) return st;
    if ((st = run_eig(c, false))) return st;
    if ((st = run_oscillators(c))) return st;
    if ((st = run_eps(c, omega, n_omega, gamma, eps2, eps1))) return st;
    stage_end(c, 7);
    if (e_out && (st = cuda_check(c, cudaMemcpyAsync(e_out, c->d_E, c->n_exc * 8, cudaMemcpyDeviceToHost, c->stream), "E copy"))) return st;
    return cuda_check(c, cudaStreamSynchronize(c->stream), "solve");
}

int bse_solve_many(bse_ctx** ctxs, int32_t n_ctx, const double* omega, int32_t n_omega, double gamma, double* eps2,
                   double* eps1, int32_t n_workers) {
    if (!ctxs || n_ctx < 0 || (n_omega > 0 && !omega)) return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_solve_many: arguments");
    for (int i = 0; i < n_ctx; i++)
        if (!ctxs[i]) return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_solve_many: null context");
    const int nw = std::max(1, std::min<int>(n_workers > 0 ? n_workers : 4, n_ctx));
    std::atomic<int> next(0), first_err(0), first_idx(-1);
    auto work = [&]() {
        for (int i = next.fetch_add(1); i < n_ctx; i = next.fetch_add(1)) {
            int st = bse_solve(ctxs[i], omega, n_omega, gamma, nullptr, eps2 ? eps2 + (size_t)i * n_omega : nullptr,
                               eps1 ? eps1 + (size_t)i * n_omega : nullptr);
            if (st) {
                int expected = 0;
                if (first_err.compare_exchange_strong(expected, st)) first_idx.store(i);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nw; t++) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    if (first_err.load())
        g_create_err = "context " + std::to_string(first_idx.load()) + ": " + ctxs[first_idx.load()]->err;
    return first_err.load();
}

int bse_stage_times(const bse_ctx* cc, double* ms, int32_t n) {
    if (!cc || !ms) return BSE_ERR_BAD_INPUT;
    bse_ctx* c = const_cast<bse_ctx*>(cc);
    cudaStreamSynchronize(c->stream);
    for (int s = 0; s < kStages && s < n; s++) {
        float t = 0;
        if (c->stage_ms[s] < 0 && cudaEventElapsedTime(&t, c->ev[2 * s], c->ev[2 * s + 1]) == cudaSuccess) c->stage_ms[s] = t;
        else if (c->stage_ms[s] < 0) { cudaGetLastError(); c->stage_ms[s] = 0; }
        ms[s] = c->stage_ms[s];
    }
    return BSE_OK;
}

int bse_diagnostics(const bse_ctx* cc, double* out, int32_t n) {
    if (!cc || !out) return BSE_ERR_BAD_INPUT;
    bse_ctx* c = const_cast<bse_ctx*>(cc);
    double v[12] = {c->max_residual, (double)c->last_clusters, (double)c->n_refined, (double)c->n_vec_valid};
    // [4 + 4 kind ..]: milliseconds, launches, algorithmic bytes and flops of the tensor-core
    // products (kind 0 hemm, 1 update) in the last two-stage reduction (BSE_KERNEL_TIMING)
    if (c->kt_used && n > 4) {
        cudaStreamSynchronize(c->stream);
        for (size_t i = 0; i < c->kt_used; i++) {
            const auto& r = c->kt[i];
            float t = 0;
            if (cudaEventElapsedTime(&t, r.ev[0], r.ev[1]) != cudaSuccess) { cudaGetLastError(); t = 0; }
            double* o = v + 4 + 4 * r.kind;
            o[0] += t;
            o[1] += 1;
            o[2] += r.bytes;
            o[3] += r.flops;
        }
    }
    for (int i = 0; i < n && i < 12; i++) out[i] = v[i];
    return BSE_OK;
}

int64_t bse_kernel_launches(const bse_ctx* c) { return c ? c->launches : 0; }
void bse_reset_kernel_launches(bse_ctx* c) {
    if (c) c->launches = 0;
}

}  // extern "C"
