// Stage a: batched H(k) assembly, per-k Hermitian eigensolves and band-subset selection.
//
// Replaces Hamiltonian_TB::FFT (bse.version13.cpp:647-705), pull_ks_states (706-777) and
// pull_ks_states_subset (778-821), which the reference re-runs for every k on every
// pair-density call.  Here every (k, {conduction at k | valence at k-q}) pair is one
// thread: it sums H(k) = sum_R w_R H(R) e^{i k.R} in FP64, diagonalizes it with an
// iteration-capped cyclic complex Jacobi method, sorts ascending, fixes the gauge (the
// first component within 1e-6 of the largest modulus is made real positive) and writes
// only the selected bands.  nw <= 16 keeps the matrices in thread-local storage; the
// stage is latency-bound (a few microseconds of arithmetic per k).
#include "bse_internal.h"

namespace bse {
namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }

// Cyclic Jacobi on the n x n Hermitian matrix A (column-major, destroyed), eigenvectors in V.
// Returns the number of sweeps used, or -1 when the cap of max_sweeps (60) is hit.
template <int NW>
__device__ int jacobi_herm(int n, double2* A, double2* V, int max_sweeps) {
    for (int i = 0; i < n * n; i++) V[i] = make_double2(0, 0);
    for (int i = 0; i < n; i++) V[i + i * n] = make_double2(1, 0);
    double fro = 0;
    for (int i = 0; i < n * n; i++) fro += cabs2(A[i]);
    for (int sweep = 0; sweep < max_sweeps; sweep++) {
        double off = 0;
        for (int q = 0; q < n; q++)
            for (int p = 0; p < q; p++) off += cabs2(A[p + q * n]);
        if (off <= 1e-30 * fro || off == 0.0) return sweep;
        for (int q = 1; q < n; q++)
            for (int p = 0; p < q; p++) {
                double2 apq = A[p + q * n];
                double a = sqrt(cabs2(apq));
                if (a == 0.0) continue;
                double2 ceph = make_double2(apq.x / a, -apq.y / a);   // e^{-i phi}
                double app = A[p + p * n].x, aqq = A[q + q * n].x;
                double tau = (aqq - app) / (2.0 * a);
                double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
                double2 uqp = make_double2(-s * ceph.x, -s * ceph.y);
                double2 uqq = make_double2(c * ceph.x, c * ceph.y);
                for (int k = 0; k < n; k++) {
                    double2 akp = A[k + p * n], akq = A[k + q * n];
                    double2 t1 = cmul(uqp, akq), t2 = cmul(uqq, akq);
                    A[k + p * n] = make_double2(c * akp.x + t1.x, c * akp.y + t1.y);
                    A[k + q * n] = make_double2(s * akp.x + t2.x, s * akp.y + t2.y);
                    double2 vkp = V[k + p * n], vkq = V[k + q * n];
                    double2 t3 = cmul(uqp, vkq), t4 = cmul(uqq, vkq);
                    V[k + p * n] = make_double2(c * vkp.x + t3.x, c * vkp.y + t3.y);
                    V[k + q * n] = make_double2(s * vkp.x + t4.x, s * vkp.y + t4.y);
                }
                double2 cuqp = cconj(uqp), cuqq = cconj(uqq);
                for (int k = 0; k < n; k++) {
                    double2 apk = A[p + k * n], aqk = A[q + k * n];
                    double2 t1 = cmul(cuqp, aqk), t2 = cmul(cuqq, aqk);
                    A[p + k * n] = make_double2(c * apk.x + t1.x, c * apk.y + t1.y);
                    A[q + k * n] = make_double2(s * apk.x + t2.x, s * apk.y + t2.y);
                }
                A[p + q * n] = make_double2(0, 0);
                A[q + p * n] = make_double2(0, 0);
                A[p + p * n].y = 0;
                A[q + q * n].y = 0;
            }
    }
    return -1;
}

template <int NW>
__global__ void __launch_bounds__(64) band_subset_kernel(
    int nk, int nw, int ns, int nr, int nv, int nc,
    const double* __restrict__ rcart, const double* __restrict__ weights,
    const double2* __restrict__ hr, const double* __restrict__ kcart,
    double q0, double q1, double q2, double ef, double scissor,
    double* __restrict__ ec, double* __restrict__ ev,
    double2* __restrict__ cc, double2* __restrict__ cv, int* __restrict__ status, int max_sweeps) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * nk) return;
    const int k = t >> 1, which = t & 1;     // 0: conduction bands at k; 1: valence at k - q
    const double kx = kcart[3 * k] - (which ? q0 : 0.0);
    const double ky = kcart[3 * k + 1] - (which ? q1 : 0.0);
    const double kz = kcart[3 * k + 2] - (which ? q2 : 0.0);
    const int nb = nw * ns;

    double2 A[NW * NW], V[NW * NW];
    double2 vec[2][NW * NW];
    double w[2][NW];
    for (int s = 0; s < ns; s++) {
        // Hamiltonian_TB::FFT: real part  sum w(Re h cos - Im h sin), imaginary sum w(Im h cos + Re h sin)
        for (int i = 0; i < nw * nw; i++) A[i] = make_double2(0, 0);
        for (int r = 0; r < nr; r++) {
            double ph = kx * rcart[3 * r] + ky * rcart[3 * r + 1] + kz * rcart[3 * r + 2];
            double sn, cs;
            sincos(ph, &sn, &cs);
            const double wr = weights[r];
            const double2* h = hr + ((size_t)s * nr + r) * nw * nw;
            for (int i = 0; i < nw * nw; i++) {
                double2 hv = h[i];
                A[i].x += wr * (hv.x * cs - hv.y * sn);
                A[i].y += wr * (hv.y * cs + hv.x * sn);
            }
        }
        int sw = jacobi_herm<NW>(nw, A, V, max_sweeps);
        if (sw < 0) { atomicMin(status, (int)BSE_ERR_NOT_CONVERGED); return; }
        // ascending order (stable), unit columns, gauge
        int ord[NW];
        for (int i = 0; i < nw; i++) ord[i] = i;
        for (int i = 1; i < nw; i++) {
            int x = ord[i], j = i - 1;
            while (j >= 0 && A[ord[j] * (nw + 1)].x > A[x * (nw + 1)].x) { ord[j + 1] = ord[j]; j--; }
            ord[j + 1] = x;
        }
        for (int j = 0; j < nw; j++) {
            const int o = ord[j];
            w[s][j] = A[o * (nw + 1)].x;
            double nrm = 0, mx = 0;
            for (int i = 0; i < nw; i++) { double a2 = cabs2(V[i + o * nw]); nrm += a2; mx = fmax(mx, sqrt(a2)); }
            nrm = sqrt(nrm);
            int piv = 0;
            for (int i = 0; i < nw; i++)
                if (sqrt(cabs2(V[i + o * nw])) >= mx * (1.0 - 1e-6)) { piv = i; break; }
            double2 vp = V[piv + o * nw];
            double ap = sqrt(cabs2(vp));
            double2 ph = make_double2(vp.x / (ap * nrm), -vp.y / (ap * nrm));
            for (int i = 0; i < nw; i++) vec[s][i + j * nw] = cmul(V[i + o * nw], ph);
        }
    }
    if (ns == 1)
        for (int j = 0; j < nw; j++) w[1][j] = w[0][j];
    int nval = 0;
    for (int i = 0; i < nw; i++)
        if (w[0][i] <= ef && w[1][i] <= ef) nval++;
    const int nvs = which ? nv : 0, ncs = which ? 0 : nc, nsel = nvs + ncs;
    if (nval - nvs < 0 || nval + ncs > nw) { atomicMin(status, (int)BSE_ERR_BAD_INPUT); return; }
    double* e_out = which ? ev : ec;
    double2* c_out = which ? cv : cc;
    for (int i = 0; i < nsel; i++) {
        const int src = i < nvs ? (nval - 1) - i : nval + (i - nvs);
        const double sc = i < nvs ? 0.0 : scissor;
        e_out[((size_t)0 * nk + k) * nsel + i] = w[0][src] + sc;
        e_out[((size_t)1 * nk + k) * nsel + i] = w[1][src] + sc;
        for (int s = 0; s < ns; s++)
            for (int j = 0; j < nw; j++)
                c_out[((size_t)k * nsel + i) * nb + s * nw + j] = vec[s][j + src * nw];
    }
}

template <int NW>
void launch_bands(bse_ctx* c, const double* q, double* ec, double* ev, double2* cc, double2* cv) {
    const int threads = 64, blocks = (2 * c->nk + threads - 1) / threads;
    band_subset_kernel<NW><<<blocks, threads, 0, c->stream>>>(
        c->nk, c->nw, c->ns, c->nr, c->nv, c->nc, c->d_rcart, c->d_weights, c->d_hr, c->d_k,
        q[0], q[1], q[2], c->p.fermi_energy, c->p.scissor, ec, ev, cc, cv, c->d_status, c->jacobi_sweeps);
    c->launches++;
}

void launch_bands_any(bse_ctx* c, const double* q, double* ec, double* ev, double2* cc, double2* cv) {
    if (c->nw <= 4) launch_bands<4>(c, q, ec, ev, cc, cv);
    else if (c->nw <= 8) launch_bands<8>(c, q, ec, ev, cc, cv);
    else launch_bands<16>(c, q, ec, ev, cc, cv);
}

}  // namespace

int band_states_shifted(bse_ctx* c, const double* q, double* ec, double* ev, double2* cc, double2* cv) {
    launch_bands_any(c, q, ec, ev, cc, cv);
    return cuda_check(c, cudaGetLastError(), "band kernel launch");
}

int run_bands(bse_ctx* c) {
    stage_begin(c, 0);
    int st;
    if ((st = cuda_check(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream), "status reset"))) return st;
    launch_bands_any(c, c->p.q, c->d_ec, c->d_ev, c->d_cc, c->d_cv);
    if ((st = cuda_check(c, cudaGetLastError(), "band kernel launch"))) return st;
    stage_end(c, 0);
    int h_status = 0;
    if ((st = cuda_check(c, cudaMemcpyAsync(&h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "status read"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "band kernel"))) return st;
    if (h_status == BSE_ERR_NOT_CONVERGED) return fail(c, h_status, "H(k) Jacobi eigensolver hit its sweep cap");
    if (h_status == BSE_ERR_BAD_INPUT)
        return fail(c, h_status, "band subset: fewer valence bands than nv or fewer conduction bands than nc at some k");
    if (h_status) return fail(c, h_status, "band kernel status");
    c->bands_valid = true;
    c->tables_valid = false;
    c->h_valid = c->eig_valid = c->osc_valid = false;
    return BSE_OK;
}

}  // namespace bse
