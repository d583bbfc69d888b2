// Stage b: pair densities and the excitonic kernel build.
//
// Replaces Excitonic_Hamiltonian::pull_coulomb_potentials (model-W modes,
// bse.version13.cpp:2547-2766), Dipole_Elements::pull_values with the point-like M
// (1459-1501, 1922-2158) and pull_resonant_part_and_rcv (2767-2928).
//
// With point-like Wannier centres tau the pair densities of the reference factor:
//   rho_cv(k,G)          = sum_a P[r,(aa)] e^{i(G+q).tau_a},     P[r,(ab)] = conj(c_ca(k)) c_vb(k-q)
//   rho_cc(k2,k1,G)*     = sum_a c_c2a(k2) conj(c_c1a(k1)) e^{-i(G+dk).tau_a}   (dk = k2 - k1)
// so the direct and exchange kernels become small lattice sums per Delta k:
//   H_d[r1,r2] = -1/(V nk) sum_ab P[r1,(ab)] Phi_ab(dk) conj(P[r2,(ab)]),
//                Phi_ab(dk) = sum_G W_G(dk) e^{-i(G+dk).(tau_a - tau_b)}
//   H_x[r1,r2] = sf/(V nk) sum_ab P[r1,(aa)] X_ab conj(P[r2,(bb)]),
//                X_ab = sum_{G != G0} v(q+G) e^{i(G+q).(tau_a - tau_b)}
// (same values as the reference's G-sums over stored all-pairs densities -- the oracle
// keeps those loops).  The coupling block of the full BSE (add_coupling_part, 2929-3040)
// reuses both tables with the other pairing of the band coefficients:
//   B_d[r1,r2] = -1/(V nk) sum_ab P[r1,(ba)] conj(Phi_ab(dk)) P[r2,(ab)],
//   B_x[r1,r2] = sf/(V nk) sum_ab P[r1,(aa)] X_ab P[r2,(bb)].
// Phi is tabulated once per distinct Delta k (on a k-grid there are
// (2n-1)^d of them); the build kernel then writes each element of H exactly once, k1
// fastest so that a warp stores 32 consecutive elements of one column: the kernel is
// bound by the N^2 store of H, not by arithmetic (inner dimension nw <= 16).
#include <cmath>
#include <mutex>
#include <random>
#include <vector>

#include "bse_internal.h"

namespace bse {
namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// Coulomb_Potential::pull (bse.version13.cpp:1273-1309) and the 2-D kinds.
__device__ double dev_coulomb(const Interaction& it, double x, double y, double z) {
    if (it.coulomb_kind == BSE_V_BARE_3D) {
        double k2 = x * x + y * y + z * z;
        if (k2 < it.min_k2) return 0.0;
        return kConv / (k2 + it.radius);
    }
    double qn = x * it.nx + y * it.ny + z * it.nz;
    double px = x - qn * it.nx, py = y - qn * it.ny, pz = z - qn * it.nz;
    double k2 = px * px + py * py + pz * pz;
    if (k2 < it.min_k2 || k2 == 0.0) return 0.0;
    return kConv * it.lz / (2.0 * sqrt(k2));
}

__device__ double dev_rk(const Interaction& it, double x, double y, double z) {
    double qn = x * it.nx + y * it.ny + z * it.nz;
    double px = x - qn * it.nx, py = y - qn * it.ny, pz = z - qn * it.nz;
    double k2 = px * px + py * py + pz * pz;
    if (k2 < it.min_k2 || k2 == 0.0) return 0.0;
    double a = sqrt(k2);
    return kConv * it.lz / (2.0 * a * (it.rk_eps + it.rk_r0 * a));
}

// W_GG(dk) of the model-W modes, diagonal in G (bse.version13.cpp:2573-2728, Q7/Q8).
__device__ double dev_w(const Interaction& it, double dx, double dy, double dz,
                        const double* G, bool is_g0) {
    const double x = dx + G[0], y = dy + G[1], z = dz + G[2];
    if (it.w_kind == BSE_W_BARE) return dev_coulomb(it, x, y, z);
    const double ndk = sqrt(dx * dx + dy * dy + dz * dz);
    if (!(ndk > kMinval) && is_g0)
        return it.w_kind == BSE_W_EMPIRICAL ? it.inv_eps * it.cell_avg : it.cell_avg;
    if (it.w_kind == BSE_W_EMPIRICAL) {
        double s = sqrt(dev_coulomb(it, x, y, z));
        return it.inv_eps * s * s;
    }
    return dev_rk(it, x, y, z);
}

struct ExcSpin { int v, c; };
__constant__ ExcSpin c_exc_spin[4] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};   // bse.version13.cpp:2522-2526

// Delta-k of table entry d (grid offsets or explicit k pair), cartesian.
__device__ void delta_k(int64_t d, bool on_grid, int m0, int m1, int m2, const double* step,
                        const double* bmat, const double* kcart, int nk, double* dk) {
    if (on_grid) {
        const int w0 = 2 * m0 - 1, w1 = 2 * m1 - 1;
        const int d0 = (int)(d % w0) - (m0 - 1);
        const int d1 = (int)((d / w0) % w1) - (m1 - 1);
        const int d2 = (int)(d / ((int64_t)w0 * w1)) - (m2 - 1);
        const double c0 = d0 * step[0], c1 = d1 * step[1], c2 = d2 * step[2];
        for (int x = 0; x < 3; x++) dk[x] = bmat[x] * c0 + bmat[3 + x] * c1 + bmat[6 + x] * c2;
    } else {
        const int k2 = (int)(d / nk), k1 = (int)(d % nk);
        for (int x = 0; x < 3; x++) dk[x] = kcart[3 * k2 + x] - kcart[3 * k1 + x];
    }
}

// Phi[d][blk][a][b] = sum_G W_G(dk) e^{-i (G + dk).(tau^{sc}_a - tau^{sv}_b)}
__global__ void phi_table_kernel(int64_t n_delta, int nblk, int nw, int stride, int ng, Interaction it,
                                 bool on_grid, int m0, int m1, int m2, double s0, double s1, double s2,
                                 const double* __restrict__ bmat, const double* __restrict__ kcart, int nk,
                                 const double* __restrict__ gcart, const double* __restrict__ centres,
                                 double2* __restrict__ phi, float2* __restrict__ phi32) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t total = n_delta * nblk * nw * nw;
    if (t >= total) return;
    const int b = (int)(t % nw), a = (int)((t / nw) % nw);
    const int blk = (int)((t / ((int64_t)nw * nw)) % nblk);
    const int64_t d = t / ((int64_t)nw * nw * nblk);
    const double step[3] = {s0, s1, s2};
    double dk[3];
    delta_k(d, on_grid, m0, m1, m2, step, bmat, kcart, nk, dk);
    const double* ta = centres + 3 * ((size_t)c_exc_spin[blk].c * nw + a);
    const double* tb = centres + 3 * ((size_t)c_exc_spin[blk].v * nw + b);
    const double dx = ta[0] - tb[0], dy = ta[1] - tb[1], dz = ta[2] - tb[2];
    const int g0 = ng / 2;
    double re = 0, im = 0;
    for (int g = 0; g < ng; g++) {
        const double* G = gcart + 3 * g;
        double w = dev_w(it, dk[0], dk[1], dk[2], G, g == g0);
        double ph = -((G[0] + dk[0]) * dx + (G[1] + dk[1]) * dy + (G[2] + dk[2]) * dz);
        double sn, cs;
        sincos(ph, &sn, &cs);
        re += w * cs;
        im += w * sn;
    }
    const size_t o = (((size_t)d * nblk + blk) * stride + a) * stride + b;
    phi[o] = make_double2(re, im);
    if (phi32) phi32[o] = make_float2((float)re, (float)im);
}

// X[s1][s2][a][b] = sum_{G != G0} v(q+G) e^{i (G+q).(tau^{s1}_a - tau^{s2}_b)}
__global__ void exchange_table_kernel(int ns, int nw, int ng, Interaction it, double q0, double q1, double q2,
                                      const double* __restrict__ gcart, const double* __restrict__ centres,
                                      double2* __restrict__ X) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns * ns * nw * nw) return;
    const int b = t % nw, a = (t / nw) % nw, s2 = (t / (nw * nw)) % ns, s1 = t / (nw * nw * ns);
    const double* ta = centres + 3 * ((size_t)s1 * nw + a);
    const double* tb = centres + 3 * ((size_t)s2 * nw + b);
    const double dx = ta[0] - tb[0], dy = ta[1] - tb[1], dz = ta[2] - tb[2];
    const int g0 = ng / 2;
    double re = 0, im = 0;
    for (int g = 0; g < ng; g++) {
        if (g == g0) continue;                                        // bse.version13.cpp:2811-2816
        const double* G = gcart + 3 * g;
        double v = dev_coulomb(it, q0 + G[0], q1 + G[1], q2 + G[2]);   // bse.version13.cpp:2566-2567
        double ph = (G[0] + q0) * dx + (G[1] + q1) * dy + (G[2] + q2) * dz;
        double sn, cs;
        sincos(ph, &sn, &cs);
        re += v * cs;
        im += v * sn;
    }
    X[t] = make_double2(re, im);
}

// rho_cv[s*N + r, g] (Dipole_Elements::pull_values, k-diagonal branch, 1951-2066; Q12/Q13).
// coupled: rows ns*N + s*N + r hold rho_vc[r, g] = sum_a conj(c_va) M_a c_ca of add_coupling_part
// (2937, 2950), with the valence states of rho_cv and the dipole column (Q25).
__global__ void rho_cv_kernel(int nk, int nc, int nv, int nw, int ns, int ng, int small_q, int coupled,
                              double q0, double q1, double q2,
                              const double* __restrict__ gcart, const double* __restrict__ centres,
                              const double2* __restrict__ cc, const double2* __restrict__ cv,
                              double2* __restrict__ rho) {
    const int64_t N = (int64_t)nk * nc * nv, NR = N * ns, nrho = NR * (coupled ? 2 : 1);
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nrho * ng) return;
    const int64_t i = t % nrho;
    const int g = (int)(t / nrho);
    const bool vc = coupled && i >= NR;
    const int64_t ii = vc ? i - NR : i;
    const int s = (int)(ii / N);
    const int64_t r = ii % N;
    const int k = (int)(r % nk), v = (int)((r / nk) % nv), c = (int)(r / ((int64_t)nk * nv));
    const int nb = nw * ns;
    const double qn = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
    const double* G = gcart + 3 * g;
    const bool dip = (g == ng / 2) && small_q;
    double2 acc = make_double2(0, 0);
    for (int a = 0; a < nw; a++) {
        const double* ta = centres + 3 * ((size_t)s * nw + a);
        double2 mel;
        if (dip) {
            mel = make_double2(0.0, (q0 * ta[0] + q1 * ta[1] + q2 * ta[2]) / qn);
        } else {
            double ph = ta[0] * (G[0] + q0) + ta[1] * (G[1] + q1) + ta[2] * (G[2] + q2);
            double sn, cs;
            sincos(ph, &sn, &cs);
            mel = make_double2(cs, sn);
        }
        const double2 ca = cc[((size_t)k * nc + c) * nb + s * nw + a], va = cv[((size_t)k * nv + v) * nb + s * nw + a];
        const double2 x = vc ? cmul(cmul(cconj(va), mel), ca) : cmul(cmul(cconj(ca), mel), va);
        acc.x += x.x;
        acc.y += x.y;
    }
    rho[i + nrho * g] = acc;
}

// Qx[s1][s2][b][r] = fx sum_a P[r,(aa)] X[s1][s2][a][b]  (exchange row factors)
__global__ void exchange_rows_kernel(int nk, int nc, int nv, int nw, int ns, double fx,
                                     const double2* __restrict__ cc, const double2* __restrict__ cv,
                                     const double2* __restrict__ X, double2* __restrict__ qx,
                                     float2* __restrict__ qx32) {
    const int64_t N = (int64_t)nk * nc * nv;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= N * nw * ns * ns) return;
    const int64_t r = t % N;
    const int b = (int)((t / N) % nw);
    const int s2 = (int)((t / (N * nw)) % ns), s1 = (int)(t / (N * nw * ns));
    const int k = (int)(r % nk), v = (int)((r / nk) % nv), c = (int)(r / ((int64_t)nk * nv));
    const int nb = nw * ns;
    double2 acc = make_double2(0, 0);
    for (int a = 0; a < nw; a++) {
        double2 pr = cmul(cconj(cc[((size_t)k * nc + c) * nb + s1 * nw + a]), cv[((size_t)k * nv + v) * nb + s1 * nw + a]);
        double2 x = cmul(pr, X[((s1 * ns + s2) * nw + a) * nw + b]);
        acc.x += x.x;
        acc.y += x.y;
    }
    acc.x *= fx;
    acc.y *= fx;
    qx[t] = acc;
    if (qx32) qx32[t] = make_float2((float)acc.x, (float)acc.y);
}

template <typename T> struct cplx;
template <> struct cplx<float> { typedef float2 t; };
template <> struct cplx<double> { typedef double2 t; };

template <typename T2> __device__ __forceinline__ T2 mk(double x, double y);
template <> __device__ __forceinline__ float2 mk<float2>(double x, double y) { return make_float2((float)x, (float)y); }
template <> __device__ __forceinline__ double2 mk<double2>(double x, double y) { return make_double2(x, y); }

template <typename T2>
__device__ __forceinline__ void cfma(T2& acc, T2 a, T2 b) {   // acc += a * b
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
template <typename T2>
__device__ __forceinline__ void cfma_conjb(T2& acc, T2 a, T2 b) {   // acc += a * conj(b)
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.y, b.x, acc.y);
    acc.y = fma(-a.x, b.y, acc.y);
}
template <typename T2>
__device__ __forceinline__ T2 tmul(T2 a, T2 b) {
    T2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

struct BuildArgs {
    int nk, nc, nv, nw, ns;
    int64_t N, ld;
    int br, bc;                 // row / column spin block of this launch
    int do_direct, do_exch, do_diag, lower;
    float fw_f;
    double fw;
    bool on_grid;
    int m0, m1, m2;
    int nblk;
    int k1_lo, k1_hi;           // rows built: k1 in [k1_lo, k1_hi) (a k tile; the whole list by default)
    const int32_t* kidx;
    const double* ec;
    const double* ev;
    const double2* cc;
    const double2* cv;
};

// One thread per (k1, k2): lane = k1 (consecutive rows of one column), warp = k2.
template <int NW, typename T>
__global__ void __launch_bounds__(256) build_kernel(BuildArgs a, const typename cplx<T>::t* __restrict__ phi,
                                                    const typename cplx<T>::t* __restrict__ qx,
                                                    typename cplx<T>::t* __restrict__ H) {
    typedef typename cplx<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x, warp = threadIdx.y, KW = blockDim.y;
    const int nb = a.nw * a.ns;
    T2* sC = reinterpret_cast<T2*>(smem_raw) + (size_t)warp * (a.nc + a.nv) * nb;   // [nc+nv][nb] of k2
    const int k1 = a.k1_lo + blockIdx.x * 32 + lane;
    const int k2 = blockIdx.y * KW + warp;
    if (k2 < a.nk) {
        for (int i = lane; i < a.nc * nb; i += 32) {
            double2 x = a.cc[(size_t)k2 * a.nc * nb + i];
            sC[i] = mk<T2>(x.x, x.y);
        }
        for (int i = lane; i < a.nv * nb; i += 32) {
            double2 x = a.cv[(size_t)k2 * a.nv * nb + i];
            sC[a.nc * nb + i] = mk<T2>(x.x, x.y);
        }
    }
    __syncwarp();
    if (k1 >= a.k1_hi || k2 >= a.nk) return;

    const int sc = c_exc_spin[a.br].c, sv = c_exc_spin[a.br].v;   // direct: diagonal spin block br
    const int s1 = a.br / 3, s2 = a.bc / 3;                        // exchange: blocks 0 / 3
    int64_t d;
    if (a.on_grid) {
        const int x1 = a.kidx[k1], x2 = a.kidx[k2];
        const int i0 = (x2 & 1023) - (x1 & 1023), i1 = ((x2 >> 10) & 1023) - ((x1 >> 10) & 1023);
        const int i2 = ((x2 >> 20) & 1023) - ((x1 >> 20) & 1023);
        d = (int64_t)(i0 + a.m0 - 1) + (int64_t)(2 * a.m0 - 1) * ((i1 + a.m1 - 1) + (int64_t)(2 * a.m1 - 1) * (i2 + a.m2 - 1));
    } else {
        d = (int64_t)k2 * a.nk + k1;
    }
    const T2* ph = phi ? phi + ((size_t)d * a.nblk + a.br) * NW * NW : nullptr;
    const T2* sCc2 = sC;
    const T2* sCv2 = sC + (size_t)a.nc * nb;
    const T fw = (T)a.fw;

    for (int c1 = 0; c1 < a.nc; c1++) {
        T2 ca[NW];
        for (int al = 0; al < NW; al++) {
            double2 x = al < a.nw ? a.cc[((size_t)k1 * a.nc + c1) * nb + sc * a.nw + al] : make_double2(0, 0);
            ca[al] = mk<T2>(x.x, -x.y);                              // conj(c_c1(k1))
        }
        for (int c2 = 0; c2 < a.nc; c2++) {
            T2 S[NW];
            for (int b = 0; b < NW; b++) S[b] = mk<T2>(0, 0);
            if (a.do_direct) {
                for (int al = 0; al < a.nw; al++) {
                    const T2 coef = tmul(ca[al], sCc2[c2 * nb + sc * a.nw + al]);
                    const T2* prow = ph + al * NW;
#pragma unroll
                    for (int b = 0; b < NW; b++)
                        if (b < a.nw) cfma(S[b], coef, prow[b]);
                }
            }
            for (int v1 = 0; v1 < a.nv; v1++) {
                const int64_t r1 = (int64_t)c1 * a.nv * a.nk + (int64_t)v1 * a.nk + k1;
                T2 tt[NW], qq[NW];
#pragma unroll
                for (int b = 0; b < NW; b++) {
                    tt[b] = mk<T2>(0, 0);
                    qq[b] = mk<T2>(0, 0);
                }
                if (a.do_direct) {
#pragma unroll
                    for (int b = 0; b < NW; b++)
                        if (b < a.nw) {
                            double2 x = a.cv[((size_t)k1 * a.nv + v1) * nb + sv * a.nw + b];
                            tt[b] = tmul(S[b], mk<T2>(x.x, x.y));
                        }
                }
                if (a.do_exch) {
#pragma unroll
                    for (int b = 0; b < NW; b++)
                        if (b < a.nw) qq[b] = qx[((size_t)(s1 * a.ns + s2) * a.nw + b) * a.N + r1];
                }
                for (int v2 = 0; v2 < a.nv; v2++) {
                    const int cv1 = c1 * a.nv + v1, cv2 = c2 * a.nv + v2;
                    if (a.lower && (cv1 < cv2 || (cv1 == cv2 && k1 < k2))) continue;
                    const int64_t r2 = (int64_t)c2 * a.nv * a.nk + (int64_t)v2 * a.nk + k2;
                    T2 acc = mk<T2>(0, 0), accx = mk<T2>(0, 0);
                    if (a.do_direct) {
#pragma unroll
                        for (int b = 0; b < NW; b++)
                            if (b < a.nw) cfma_conjb(acc, tt[b], sCv2[v2 * nb + sv * a.nw + b]);
                    }
                    if (a.do_exch) {
#pragma unroll
                        for (int b = 0; b < NW; b++)
                            if (b < a.nw) {
                                // D2 = conj(c_c2b(k2)) c_v2b(k2-q);  H_x += qx * conj(D2)
                                const T2 d2 = tmul(mk<T2>(sCc2[c2 * nb + s2 * a.nw + b].x, -sCc2[c2 * nb + s2 * a.nw + b].y),
                                                   sCv2[v2 * nb + s2 * a.nw + b]);
                                cfma_conjb(accx, qq[b], d2);
                            }
                    }
                    T2 out;
                    out.x = fw * acc.x + accx.x;
                    out.y = fw * acc.y + accx.y;
                    if (a.do_diag && k1 == k2 && c1 == c2 && v1 == v2) {
                        const int cs = c_exc_spin[a.br].c, vs = c_exc_spin[a.br].v;
                        out.x += (T)(a.ec[((size_t)cs * a.nk + k1) * a.nc + c1] - a.ev[((size_t)vs * a.nk + k1) * a.nv + v1]);
                    }
                    H[(a.br * a.N + r1) + a.ld * (a.bc * a.N + r2)] = out;
                }
            }
        }
    }
}

// One block (row spin block br, column spin block bc) of the coupling part B = H[0:NA, NA:2NA] of the
// full BSE, FP64 (add_coupling_part, bse.version13.cpp:2929-3040).  Same launch shape as
// build_kernel (lane = k1, warp = k2):
//   direct   (rho_kk_cv W conj(rho_kk_vc), 2975-3033; Q26; only bc = the partner block of br): the
//            valence state of exciton r1 (spin sv1) pairs with the conduction state of r2, the
//            valence state of r2 with the conduction state of r1 (spin sc1), through
//            conj(Phi^{bc}_ab(k2 - k1)) -- the table of block bc has c-spin sv1 and v-spin sc1;
//   exchange (rho_cv(r1) conj(rho_vc(r2)), 2940-2967; blocks 0|3 x 0|3): Qx[s1][s2] times P[r2,(bb)].
// Every element of the block is written once.
template <int NW>
__global__ void __launch_bounds__(256) coupling_kernel(BuildArgs a, const double2* __restrict__ phi,
                                                       const double2* __restrict__ qx, double2* __restrict__ H) {
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x, warp = threadIdx.y, KW = blockDim.y;
    const int nb = a.nw * a.ns;
    double2* sC = reinterpret_cast<double2*>(smem_raw) + (size_t)warp * (a.nc + a.nv) * nb;   // [nc+nv][nb] of k2
    const int k1 = blockIdx.x * 32 + lane;
    const int k2 = blockIdx.y * KW + warp;
    if (k2 < a.nk) {
        for (int i = lane; i < a.nc * nb; i += 32) sC[i] = a.cc[(size_t)k2 * a.nc * nb + i];
        for (int i = lane; i < a.nv * nb; i += 32) sC[a.nc * nb + i] = a.cv[(size_t)k2 * a.nv * nb + i];
    }
    __syncwarp();
    if (k1 >= a.nk || k2 >= a.nk) return;
    int64_t d;
    if (a.on_grid) {
        const int x1 = a.kidx[k1], x2 = a.kidx[k2];
        const int i0 = (x2 & 1023) - (x1 & 1023), i1 = ((x2 >> 10) & 1023) - ((x1 >> 10) & 1023);
        const int i2 = ((x2 >> 20) & 1023) - ((x1 >> 20) & 1023);
        d = (int64_t)(i0 + a.m0 - 1) + (int64_t)(2 * a.m0 - 1) * ((i1 + a.m1 - 1) + (int64_t)(2 * a.m1 - 1) * (i2 + a.m2 - 1));
    } else {
        d = (int64_t)k2 * a.nk + k1;
    }
    const double2* ph = phi + ((size_t)d * a.nblk + a.bc) * NW * NW;          // table of the column block
    const double2* sCc2 = sC;
    const double2* sCv2 = sC + (size_t)a.nc * nb;
    const int sv1 = c_exc_spin[a.br].v, sc1 = c_exc_spin[a.br].c;            // direct: spins of row block br
    const int s1 = a.br / 3, s2 = a.bc / 3;                                    // exchange: blocks 0 / 3
    const int64_t NA = (int64_t)a.nblk * a.N;                                  // resonant block size
    for (int v1 = 0; v1 < a.nv; v1++) {
        double2 va[NW];
#pragma unroll
        for (int al = 0; al < NW; al++)
            va[al] = al < a.nw ? a.cv[((size_t)k1 * a.nv + v1) * nb + sv1 * a.nw + al] : make_double2(0, 0);   // c_v1(k1)
        for (int c2 = 0; c2 < a.nc; c2++) {
            double2 S[NW];   // S[b] = sum_a c_v1a(k1) conj(c_c2a(k2)) conj(Phi_ab)
#pragma unroll
            for (int b = 0; b < NW; b++) S[b] = make_double2(0, 0);
            if (a.do_direct) {
                for (int al = 0; al < a.nw; al++) {
                    const double2 coef = tmul(va[al], cconj(sCc2[c2 * nb + sv1 * a.nw + al]));
                    const double2* prow = ph + al * NW;
#pragma unroll
                    for (int b = 0; b < NW; b++)
                        if (b < a.nw) cfma_conjb(S[b], coef, prow[b]);
                }
            }
            for (int c1 = 0; c1 < a.nc; c1++) {
                const int64_t r1 = (int64_t)c1 * a.nv * a.nk + (int64_t)v1 * a.nk + k1;
                double2 tt[NW], qq[NW];
#pragma unroll
                for (int b = 0; b < NW; b++) {
                    tt[b] = make_double2(0, 0);
                    qq[b] = make_double2(0, 0);
                    if (b < a.nw) {
                        if (a.do_direct) tt[b] = tmul(S[b], cconj(a.cc[((size_t)k1 * a.nc + c1) * nb + sc1 * a.nw + b]));   // conj(c_c1b(k1))
                        if (a.do_exch) qq[b] = qx[((size_t)(s1 * a.ns + s2) * a.nw + b) * a.N + r1];
                    }
                }
                for (int v2 = 0; v2 < a.nv; v2++) {
                    const int64_t r2 = (int64_t)c2 * a.nv * a.nk + (int64_t)v2 * a.nk + k2;
                    double2 acc = make_double2(0, 0), accx = make_double2(0, 0);
#pragma unroll
                    for (int b = 0; b < NW; b++)
                        if (b < a.nw) {
                            if (a.do_direct) cfma(acc, tt[b], sCv2[v2 * nb + sc1 * a.nw + b]);   // ... c_v2b(k2)
                            if (a.do_exch)                                                      // Qx P[r2,(bb)]
                                cfma(accx, qq[b], tmul(cconj(sCc2[c2 * nb + s2 * a.nw + b]), sCv2[v2 * nb + s2 * a.nw + b]));
                        }
                    H[(a.br * a.N + r1) + a.ld * (NA + a.bc * a.N + r2)] = make_double2(a.fw * acc.x + accx.x, a.fw * acc.y + accx.y);
                }
            }
        }
    }
}

// M = [[A, B], [B^H, conj(A)]] from the top blocks (NA = resonant size, ld = 2 NA): the Hermitian
// matrix whose J-scaled form J M is the full BSE matrix [[A, B], [-B^H, -conj(A)]] of 2917-2923 and
// 3035-3038 (3107-3114 after the collinear rotation).
__global__ void coupled_lower_blocks_kernel(int64_t NA, double2* __restrict__ M) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= NA * NA) return;
    const int64_t i = t % NA, j = t / NA, ld = 2 * NA;
    M[(NA + i) + ld * (NA + j)] = cconj(M[i + ld * j]);
    M[(NA + i) + ld * j] = cconj(M[j + ld * (NA + i)]);
}

// Collinear full BSE: the two 4N x 4N Hermitian blocks of M, M0 = spin blocks {1,2} and M1 = {0,3}
// of every quadrant (common_diagonalization 3151-3172), from M (8N x 8N).
__global__ void gather_coupled_blocks_kernel(int64_t N, const double2* __restrict__ M, double2* __restrict__ M0,
                                             double2* __restrict__ M1) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t n4 = 4 * N, ld = 8 * N;
    if (t >= n4 * n4) return;
    const int64_t i = t % n4, j = t / n4;
    // index within the 4N block: quadrant (i / 2N) and position p within the 2N half
    auto map0 = [&](int64_t x) { const int64_t q = x / (2 * N), p = x % (2 * N); return q * 4 * N + N + p; };
    auto map1 = [&](int64_t x) { const int64_t q = x / (2 * N), p = x % (2 * N); return q * 4 * N + (p < N ? p : p + 2 * N); };
    M0[t] = M[map0(i) + ld * map0(j)];
    M1[t] = M[map1(i) + ld * map1(j)];
}

// ---- RPA screened interaction (pull_coulomb_potentials 2597-2690, Dielectric_Function::pull_values
// 2214-2315).  Per momentum q (a grid Delta k, or a point of the dk = 0 sphere):
//   rho1_r(G) = sum_a conj(c_ca(k)) e^{i(G+q).tau_a} c_va(k - q),   E1 = E_c(k) - E_v(k - q)
//   rho2_r(G) = sum_a conj(c_ca(k)) e^{-i(G+q).tau_a} c_va(k + q),  E2 = E_c(k) - E_v(k + q)
//   chi0 = 1/(V nk) [rho1^H diag(m1) rho1 + conj(rho2^H diag(conj m2) rho2)],
//   m1 = 1/(-E1 + i eta), m2 = -1/(E2 - i eta)  (omega = 0; the -q densities of the anti-resonant term)
//   eps^-1 = 1 + diag(v) chi0 (order 0) or 1 + diag(v) (1 - chi0 diag(v))^-1 chi0, v_G = v(q + G)
//   W_GG' = eps^-1_GG' v(q + G'),  Phi_ab = sum_GG' e^{-i(G+q).tau^c_a} W_GG' e^{i(G'+q).tau^v_b}
// r = ((s nc + c) nv + v) nk + k; the rho arrays are column-major R x ng per momentum.
__global__ void rpa_rho_kernel(int D, int64_t R, int ng, int nk, int nc, int nv, int nw, int ns,
                               const double* __restrict__ qs, const int* __restrict__ map_m,
                               const int* __restrict__ map_p, const double* __restrict__ gcart,
                               const double* __restrict__ centres, const double2* __restrict__ cc,
                               const double* __restrict__ ec, const double2* __restrict__ cvm,
                               const double* __restrict__ evm, const double2* __restrict__ cvp,
                               const double* __restrict__ evp, double eta, double2* __restrict__ rho1,
                               double2* __restrict__ q1, double2* __restrict__ rho2, double2* __restrict__ q2) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t per = R * ng;
    if (t >= per * D) return;
    const int d = (int)(t / per);
    const int64_t rem = t % per;
    const int g = (int)(rem / R);
    const int64_t r = rem % R;
    const int k = (int)(r % nk), v = (int)((r / nk) % nv);
    const int c = (int)((r / ((int64_t)nk * nv)) % nc), s = (int)(r / ((int64_t)nk * nv * nc));
    const int km = map_m ? map_m[(size_t)d * nk + k] : k, kp = map_p ? map_p[(size_t)d * nk + k] : k;
    const int nb = nw * ns;
    const double* q = qs + 3 * d;
    const double* G = gcart + 3 * g;
    double2 a1 = make_double2(0, 0), a2 = make_double2(0, 0);
    for (int a = 0; a < nw; a++) {
        const double* ta = centres + 3 * ((size_t)s * nw + a);
        const double ph = ta[0] * (G[0] + q[0]) + ta[1] * (G[1] + q[1]) + ta[2] * (G[2] + q[2]);
        double sn, cs;
        sincos(ph, &sn, &cs);
        const double2 cca = cconj(cc[((size_t)k * nc + c) * nb + s * nw + a]);
        const double2 x1 = cmul(cmul(cca, make_double2(cs, sn)), cvm[((size_t)km * nv + v) * nb + s * nw + a]);
        const double2 x2 = cmul(cmul(cca, make_double2(cs, -sn)), cvp[((size_t)kp * nv + v) * nb + s * nw + a]);
        a1.x += x1.x; a1.y += x1.y;
        a2.x += x2.x; a2.y += x2.y;
    }
    const double E1 = ec[((size_t)s * nk + k) * nc + c] - evm[((size_t)s * nk + km) * nv + v];
    const double E2 = ec[((size_t)s * nk + k) * nc + c] - evp[((size_t)s * nk + kp) * nv + v];
    const double d1 = E1 * E1 + eta * eta, d2 = E2 * E2 + eta * eta;
    const double2 m1 = make_double2(-E1 / d1, -eta / d1);    // 1/(-E1 + i eta)
    const double2 m2c = make_double2(-E2 / d2, eta / d2);    // conj(-1/(E2 - i eta))
    const int64_t o = (int64_t)d * per + (int64_t)g * R + r;
    rho1[o] = a1;
    q1[o] = cmul(m1, a1);
    rho2[o] = a2;
    q2[o] = cmul(m2c, a2);
}

// chi0 = fchi (C1 + conj(C2)) into chi0; order 0: einv = 1 + diag(v) chi0; order 1: A = 1 - chi0 diag(v)
__global__ void rpa_chi0_kernel(int D, int ng, double fchi, const double* __restrict__ qs, const double* __restrict__ gcart,
                                Interaction it, int order, const double2* __restrict__ C1, const double2* __restrict__ C2,
                                double2* __restrict__ chi0, double2* __restrict__ A, double2* __restrict__ einv) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t gg = (int64_t)ng * ng;
    if (t >= gg * D) return;
    const int d = (int)(t / gg);
    const int i = (int)((t % gg) % ng), j = (int)((t % gg) / ng);
    const double* q = qs + 3 * d;
    const double2 chi = make_double2(fchi * (C1[t].x + C2[t].x), fchi * (C1[t].y - C2[t].y));
    chi0[t] = chi;
    const double* Gi = gcart + 3 * i;
    const double* Gj = gcart + 3 * j;
    if (order == 0) {
        const double vi = dev_coulomb(it, q[0] + Gi[0], q[1] + Gi[1], q[2] + Gi[2]);
        einv[t] = make_double2((i == j ? 1.0 : 0.0) + vi * chi.x, vi * chi.y);
    } else {
        const double vj = dev_coulomb(it, q[0] + Gj[0], q[1] + Gj[1], q[2] + Gj[2]);
        A[t] = make_double2((i == j ? 1.0 : 0.0) - chi.x * vj, -chi.y * vj);
    }
}

// order 1: einv = 1 + diag(v) X with X = A^-1 chi0 from the batched solve
__global__ void rpa_einv_kernel(int D, int ng, const double* __restrict__ qs, const double* __restrict__ gcart, Interaction it,
                                const double2* __restrict__ X, double2* __restrict__ einv) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t gg = (int64_t)ng * ng;
    if (t >= gg * D) return;
    const int d = (int)(t / gg);
    const int i = (int)((t % gg) % ng), j = (int)((t % gg) / ng);
    const double* q = qs + 3 * d;
    const double* Gi = gcart + 3 * i;
    const double vi = dev_coulomb(it, q[0] + Gi[0], q[1] + Gi[1], q[2] + Gi[2]);
    einv[t] = make_double2((i == j ? 1.0 : 0.0) + vi * X[t].x, vi * X[t].y);
}

// W = einv v(q + G_col) for grid momenta; sphere points accumulate <W> with the head keeping <eps^-1_00>
__global__ void rpa_w_kernel(int D, int ng, const double* __restrict__ qs, const double* __restrict__ gcart, Interaction it,
                             const double2* __restrict__ einv, double2* __restrict__ W, int accumulate) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t gg = (int64_t)ng * ng;
    if (t >= gg * D) return;
    const int d = (int)(t / gg);
    const int i = (int)((t % gg) % ng), j = (int)((t % gg) / ng);
    const double* q = qs + 3 * d;
    const double* Gj = gcart + 3 * j;
    const int g0 = ng / 2;
    const double vj = (accumulate && i == g0 && j == g0) ? 1.0 : dev_coulomb(it, q[0] + Gj[0], q[1] + Gj[1], q[2] + Gj[2]);
    const double2 w = make_double2(einv[t].x * vj, einv[t].y * vj);
    if (accumulate) {
        const int64_t u = t % gg;
        W[u].x += w.x;
        W[u].y += w.y;
    } else {
        W[t] = w;
    }
}

// Phi[dd][blk][a][b] = sum_GG' e^{-i(G+q).tau^{sc}_a} W_GG' e^{i(G'+q).tau^{sv}_b} for D table entries;
// conj_w: the same sums with conj(W_GG'), the coupling block's table (for a real diagonal W the two agree)
__global__ void rpa_phi_kernel(int D, const int64_t* __restrict__ didx, const double* __restrict__ qs, int nblk, int nw,
                               int stride, int ng, const double* __restrict__ gcart, const double* __restrict__ centres,
                               const double2* __restrict__ W, double2* __restrict__ phi, float2* __restrict__ phi32,
                               int conj_w) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)D * nblk * nw * nw) return;
    const int b = (int)(t % nw), a = (int)((t / nw) % nw);
    const int blk = (int)((t / ((int64_t)nw * nw)) % nblk);
    const int d = (int)(t / ((int64_t)nw * nw * nblk));
    const double* q = qs + 3 * d;
    const double* ta = centres + 3 * ((size_t)c_exc_spin[blk].c * nw + a);
    const double* tb = centres + 3 * ((size_t)c_exc_spin[blk].v * nw + b);
    const double2* w = W + (int64_t)d * ng * ng;
    double re = 0, im = 0;
    for (int j = 0; j < ng; j++) {
        const double* Gj = gcart + 3 * j;
        const double pj = (Gj[0] + q[0]) * tb[0] + (Gj[1] + q[1]) * tb[1] + (Gj[2] + q[2]) * tb[2];
        double sj, cj;
        sincos(pj, &sj, &cj);
        double sr = 0, si = 0;   // sum_i e^{-i(G_i+q).tau_a} W_ij
        for (int i = 0; i < ng; i++) {
            const double* Gi = gcart + 3 * i;
            const double pi_ = -((Gi[0] + q[0]) * ta[0] + (Gi[1] + q[1]) * ta[1] + (Gi[2] + q[2]) * ta[2]);
            double si_, ci_;
            sincos(pi_, &si_, &ci_);
            double2 x = w[i + (int64_t)ng * j];
            if (conj_w) x.y = -x.y;
            sr += ci_ * x.x - si_ * x.y;
            si += ci_ * x.y + si_ * x.x;
        }
        re += sr * cj - si * sj;
        im += sr * sj + si * cj;
    }
    const size_t o = (((size_t)didx[d] * nblk + blk) * stride + a) * stride + b;
    phi[o] = make_double2(re, im);
    if (phi32) phi32[o] = make_float2((float)re, (float)im);
}

// Collinear spin rotation U H U (spin_transformation, bse.version13.cpp:3048-3117), in place per
// (row, col) position across the 4x4 spin blocks, so no block reads an already rotated one (Q24).
template <typename T2>
__global__ void spin_rotate_kernel(int64_t N, T2* __restrict__ H, int64_t ld) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= N * N) return;
    const int64_t rr = t % N, cc = t / N;
    const double h = 0.70710678118654752440;
    const double U[4][4] = {{1, 0, 0, 0}, {0, h, h, 0}, {0, h, -h, 0}, {0, 0, 0, 1}};
    double xr[4][4], xi[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            T2 v = H[(i * N + rr) + ld * (j * N + cc)];
            xr[i][j] = v.x;
            xi[i][j] = v.y;
        }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double sr = 0, si = 0;
            for (int l = 0; l < 4; l++)
                for (int k = 0; k < 4; k++) {
                    double w = U[i][l] * U[k][j];
                    sr += w * xr[l][k];
                    si += w * xi[l][k];
                }
            T2 o;
            o.x = sr;
            o.y = si;
            H[(i * N + rr) + ld * (j * N + cc)] = o;
        }
}

// Gather the collinear diagonal blocks: H0 = rotated blocks {1,2}, H1 = blocks {0,3}
// (common_diagonalization, bse.version13.cpp:3143-3149).
template <typename T2>
__global__ void gather_blocks_kernel(int64_t N, const T2* __restrict__ H, T2* __restrict__ H0, T2* __restrict__ H1) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t n2 = 2 * N;
    if (t >= n2 * n2) return;
    const int64_t i = t % n2, j = t / n2, ld = 4 * N;
    const int64_t i0 = i + N, j0 = j + N;                       // blocks 1,2
    const int64_t i1 = i < N ? i : i + 2 * N, j1 = j < N ? j : j + 2 * N;   // blocks 0,3
    H0[t] = H[i0 + ld * j0];
    H1[t] = H[i1 + ld * j1];
}

template <int NW, typename T>
int launch_build_nw(bse_ctx* c, void* H, int64_t ld, bool lower, const void* phi, const void* qx,
                    int br, int bc, int do_direct, int do_exch, int do_diag) {
    BuildArgs a;
    a.nk = c->nk; a.nc = c->nc; a.nv = c->nv; a.nw = c->nw; a.ns = c->ns;
    a.N = c->N; a.ld = ld; a.br = br; a.bc = bc;
    a.do_direct = do_direct; a.do_exch = do_exch; a.do_diag = do_diag; a.lower = lower ? 1 : 0;
    a.fw = -1.0 / (c->geo.vol * c->nk);   // bse.version13.cpp:2845
    a.fw_f = (float)a.fw;
    a.on_grid = c->dmap.on_grid;
    a.m0 = c->dmap.m[0]; a.m1 = c->dmap.m[1]; a.m2 = c->dmap.m[2];
    a.nblk = 3 * c->S + 1;
    a.k1_lo = c->build_k_lo;
    a.k1_hi = c->build_k_hi > 0 ? c->build_k_hi : c->nk;
    a.kidx = c->d_kidx;
    a.ec = c->d_ec; a.ev = c->d_ev; a.cc = c->d_cc; a.cv = c->d_cv;
    const int KW = 8;
    dim3 block(32, KW), grid((a.k1_hi - a.k1_lo + 31) / 32, (c->nk + KW - 1) / KW, 1);
    size_t smem = (size_t)KW * (c->nc + c->nv) * c->nb * sizeof(typename cplx<T>::t);
    // process-wide attribute: set once to the largest size (nc, nv <= 8, nb <= 32)
    static std::once_flag smem_once;
    static cudaError_t smem_err = cudaSuccess;
    std::call_once(smem_once, [] {
        const int smax = 8 * (8 + 8) * 32 * (int)sizeof(typename cplx<T>::t);
        smem_err = cudaFuncSetAttribute(build_kernel<NW, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    });
    if (smem_err != cudaSuccess) return cuda_check(c, smem_err, "build smem attribute");
    build_kernel<NW, T><<<grid, block, smem, c->stream>>>(
        a, (const typename cplx<T>::t*)phi, (const typename cplx<T>::t*)qx, (typename cplx<T>::t*)H);
    c->launches++;
    return cuda_check(c, cudaGetLastError(), "build kernel launch");
}

template <int NW>
int launch_coupling_nw(bse_ctx* c, int br, int bc, int direct, int exch) {
    BuildArgs a = {};
    a.nk = c->nk; a.nc = c->nc; a.nv = c->nv; a.nw = c->nw; a.ns = c->ns;
    a.N = c->N; a.ld = c->n_h;
    a.br = br; a.bc = bc; a.do_direct = direct; a.do_exch = exch;
    a.fw = -1.0 / (c->geo.vol * c->nk);   // bse.version13.cpp:2960
    a.k1_lo = 0;
    a.k1_hi = c->nk;
    a.on_grid = c->dmap.on_grid;
    a.m0 = c->dmap.m[0]; a.m1 = c->dmap.m[1]; a.m2 = c->dmap.m[2];
    a.nblk = 3 * c->S + 1;
    a.kidx = c->d_kidx;
    a.cc = c->d_cc; a.cv = c->d_cv;
    const int KW = 8;
    dim3 block(32, KW), grid((c->nk + 31) / 32, (c->nk + KW - 1) / KW, 1);
    const size_t smem = (size_t)KW * (c->nc + c->nv) * c->nb * sizeof(double2);   // <= 8 * 16 * 32 * 16 = 64 KB
    static std::once_flag smem_once;
    static cudaError_t smem_err = cudaSuccess;
    std::call_once(smem_once, [] {
        smem_err = cudaFuncSetAttribute(coupling_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 * 16 * 32 * 16);
    });
    if (smem_err != cudaSuccess) return cuda_check(c, smem_err, "coupling smem attribute");
    // with an RPA W the coupling block pairs the states through conj(W) (its own table)
    coupling_kernel<NW><<<grid, block, smem, c->stream>>>(a, c->d_phi_c ? c->d_phi_c : c->d_phi, c->d_qx, (double2*)c->d_H);
    c->launches++;
    return cuda_check(c, cudaGetLastError(), "coupling kernel launch");
}

int launch_coupling(bse_ctx* c, int br, int bc, int direct, int exch) {
    if (c->nw <= 2) return launch_coupling_nw<2>(c, br, bc, direct, exch);
    if (c->nw <= 4) return launch_coupling_nw<4>(c, br, bc, direct, exch);
    if (c->nw <= 8) return launch_coupling_nw<8>(c, br, bc, direct, exch);
    return launch_coupling_nw<16>(c, br, bc, direct, exch);
}

template <typename T>
int launch_build(bse_ctx* c, void* H, int64_t ld, bool lower, const void* phi, const void* qx,
                 int br, int bc, int dd, int de, int dg) {
    // phi rows are padded to NW entries: the table is laid out with stride NW == the template
    if (c->nw <= 2) return launch_build_nw<2, T>(c, H, ld, lower, phi, qx, br, bc, dd, de, dg);
    if (c->nw <= 4) return launch_build_nw<4, T>(c, H, ld, lower, phi, qx, br, bc, dd, de, dg);
    if (c->nw <= 8) return launch_build_nw<8, T>(c, H, ld, lower, phi, qx, br, bc, dd, de, dg);
    return launch_build_nw<16, T>(c, H, ld, lower, phi, qx, br, bc, dd, de, dg);
}

}  // namespace

int table_stride(int nw) { return nw <= 2 ? 2 : nw <= 4 ? 4 : nw <= 8 ? 8 : 16; }

int run_tables(bse_ctx* c) {
    int st;
    stage_begin(c, 1);
    const int ns = c->ns, nw = c->nw, ng = c->ng;
    // rho_cv
    {
        const int64_t total = c->n_rho * ng;
        const int thr = 256;
        rho_cv_kernel<<<(unsigned)((total + thr - 1) / thr), thr, 0, c->stream>>>(
            c->nk, c->nc, c->nv, nw, ns, ng, c->p.small_momentum, c->coupled ? 1 : 0, c->p.q[0], c->p.q[1], c->p.q[2],
            c->d_g, c->d_centres, c->d_cc, c->d_cv, c->d_rho);
        c->launches++;
        if ((st = cuda_check(c, cudaGetLastError(), "rho kernel"))) return st;
    }
    if (!c->p.ipa) {
        const int NWs = table_stride(nw);
        // exchange lattice sums and row factors
        exchange_table_kernel<<<(ns * ns * nw * nw + 127) / 128, 128, 0, c->stream>>>(
            ns, nw, ng, c->itx, c->p.q[0], c->p.q[1], c->p.q[2], c->d_g, c->d_centres, c->d_X);
        c->launches++;
        const double sf = c->p.spin_factor >= 0 ? c->p.spin_factor : (double)(2 - c->S);
        const double fx = sf / (c->nk * c->geo.vol);                     // bse.version13.cpp:2801
        const int64_t nq = c->N * nw * ns * ns;
        exchange_rows_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, c->stream>>>(
            c->nk, c->nc, c->nv, nw, ns, fx, c->d_cc, c->d_cv, c->d_X, c->d_qx,
            c->p.precision == BSE_MIXED ? c->d_qx32 : nullptr);
        c->launches++;
        // direct lattice sums, one per distinct Delta k, rows padded to the kernel's stride
        const int nblk = 3 * c->S + 1;
        const int64_t total = c->dmap.n_delta * nblk * NWs * NWs;
        if ((st = cuda_check(c, cudaMemsetAsync(c->d_phi, 0, total * sizeof(double2), c->stream), "phi clear"))) return st;
        if (c->d_phi32 && (st = cuda_check(c, cudaMemsetAsync(c->d_phi32, 0, total * sizeof(float2), c->stream), "phi32 clear"))) return st;
        if (c->d_phi_c && (st = cuda_check(c, cudaMemsetAsync(c->d_phi_c, 0, total * sizeof(double2), c->stream), "phi clear"))) return st;
        if (c->p.w_kind == BSE_W_RPA) {
            if ((st = run_rpa_tables(c))) return st;
        } else {
            const int64_t tk = c->dmap.n_delta * nblk * nw * nw;
            phi_table_kernel<<<(unsigned)((tk + 255) / 256), 256, 0, c->stream>>>(
                c->dmap.n_delta, nblk, nw, NWs, ng, c->itx, c->dmap.on_grid, c->dmap.m[0], c->dmap.m[1], c->dmap.m[2],
                c->dmap.step[0], c->dmap.step[1], c->dmap.step[2], c->d_bmat, c->d_k, c->nk,
                c->d_g, c->d_centres, c->d_phi, c->p.precision == BSE_MIXED ? c->d_phi32 : nullptr);
            c->launches++;
            if ((st = cuda_check(c, cudaGetLastError(), "phi kernel"))) return st;
        }
    }
    stage_end(c, 1);
    if ((st = cuda_check(c, cudaGetLastError(), "tables"))) return st;
    c->tables_valid = true;
    return BSE_OK;
}

// RPA direct-kernel tables: W per grid Delta k (chunks of momenta: densities, two batched ZGEMMs for
// chi0, batched LU for the Dyson form), the dk = 0 entry from the seeded sphere points.
int run_rpa_tables(bse_ctx* c) {
    int st;
    const int nk = c->nk, ng = c->ng, nw = c->nw, ns = c->ns, nc = c->nc, nv = c->nv, nb = c->nb;
    const int64_t R = (int64_t)ns * nk * nc * nv, gg = (int64_t)ng * ng;
    const int nblk = 3 * c->S + 1, NWs = table_stride(nw), order = c->p.rpa_order;
    const double eta = c->p.rpa_eta, fchi = 1.0 / (c->geo.vol * nk);
    const DeltaMap& dm = c->dmap;
    const int m0 = dm.m[0], m1 = dm.m[1], m2 = dm.m[2];
    const int64_t nd = dm.n_delta;
    const int64_t dcenter = (int64_t)(m0 - 1) + (int64_t)(2 * m0 - 1) * ((m1 - 1) + (int64_t)(2 * m1 - 1) * (m2 - 1));
    // momenta per chunk: the densities dominate, 4 R ng complex per momentum
    const int64_t per_d = 4 * R * ng * 16 + 6 * gg * 16 + 2 * (int64_t)nk * 4 + 64;
    const int64_t D = std::max<int64_t>(1, std::min<int64_t>(nd, (int64_t)(2e9 / (double)per_d)));
    // the band kernels below report into the status word: start it at zero (bands may have been
    // set from the host, in which case no band kernel has reset it)
    if ((st = cuda_check(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream), "status reset"))) return st;
    // scratch: valence states at the grid k (and the sphere's k -+ q), conduction dummies, chunk arrays
    char* buf = nullptr;
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t oE = carve(2 * (size_t)nk * nc * 8), oC = carve((size_t)nk * nc * nb * 16);
    const size_t oEv0 = carve(2 * (size_t)nk * nv * 8), oCv0 = carve((size_t)nk * nv * nb * 16);
    const size_t oEvm = carve(2 * (size_t)nk * nv * 8), oCvm = carve((size_t)nk * nv * nb * 16);
    const size_t oEvp = carve(2 * (size_t)nk * nv * 8), oCvp = carve((size_t)nk * nv * nb * 16);
    const size_t oR1 = carve(D * R * ng * 16), oQ1 = carve(D * R * ng * 16), oR2 = carve(D * R * ng * 16), oQ2 = carve(D * R * ng * 16);
    const size_t oC1 = carve(D * gg * 16), oC2 = carve(D * gg * 16), oChi = carve(D * gg * 16), oA = carve(D * gg * 16);
    const size_t oEi = carve(D * gg * 16), oW = carve(D * gg * 16), oAvg = carve(gg * 16);
    const size_t oQs = carve(D * 3 * 8), oDi = carve(D * 8), oMm = carve(D * nk * 4), oMp = carve(D * nk * 4);
    const size_t oPiv = carve(D * ng * 4), oInfo = carve(D * 4), oPa = carve(D * 8), oPb = carve(D * 8);
    if ((st = cuda_check(c, cudaMallocAsync((void**)&buf, off, c->stream), "RPA workspace"))) return st;
    double* ecs = (double*)(buf + oE);
    double2* ccs = (double2*)(buf + oC);
    double* ev0 = (double*)(buf + oEv0);
    double2* cv0 = (double2*)(buf + oCv0);
    double* evm = (double*)(buf + oEvm);
    double2* cvm = (double2*)(buf + oCvm);
    double* evp = (double*)(buf + oEvp);
    double2* cvp = (double2*)(buf + oCvp);
    double2 *r1 = (double2*)(buf + oR1), *q1 = (double2*)(buf + oQ1), *r2 = (double2*)(buf + oR2), *q2 = (double2*)(buf + oQ2);
    double2 *C1 = (double2*)(buf + oC1), *C2 = (double2*)(buf + oC2), *chi = (double2*)(buf + oChi), *A = (double2*)(buf + oA);
    double2 *einv = (double2*)(buf + oEi), *W = (double2*)(buf + oW), *avg = (double2*)(buf + oAvg);
    double* dqs = (double*)(buf + oQs);
    int64_t* ddi = (int64_t*)(buf + oDi);
    int* dmm = (int*)(buf + oMm);
    int* dmp = (int*)(buf + oMp);
    int* piv = (int*)(buf + oPiv);
    int* info = (int*)(buf + oInfo);
    cuDoubleComplex** pa = (cuDoubleComplex**)(buf + oPa);
    cuDoubleComplex** pb = (cuDoubleComplex**)(buf + oPb);
    cublasSetStream(c->cublas, c->stream);
    const cuDoubleComplex one = make_cuDoubleComplex(1, 0), zero = make_cuDoubleComplex(0, 0);
    // chi0 -> eps^-1 for the first Dn momenta of the chunk arrays (qs, rho already set)
    auto eps_inv = [&](int64_t Dn) -> int {
        if (cublasZgemmStridedBatched(c->cublas, CUBLAS_OP_C, CUBLAS_OP_N, ng, ng, (int)R, &one, (const cuDoubleComplex*)r1, (int)R,
                                      R * ng, (const cuDoubleComplex*)q1, (int)R, R * ng, &zero, (cuDoubleComplex*)C1, ng, gg,
                                      (int)Dn) != CUBLAS_STATUS_SUCCESS ||
            cublasZgemmStridedBatched(c->cublas, CUBLAS_OP_C, CUBLAS_OP_N, ng, ng, (int)R, &one, (const cuDoubleComplex*)r2, (int)R,
                                      R * ng, (const cuDoubleComplex*)q2, (int)R, R * ng, &zero, (cuDoubleComplex*)C2, ng, gg,
                                      (int)Dn) != CUBLAS_STATUS_SUCCESS)
            return fail(c, BSE_ERR_CUDA, "cuBLAS failed in chi0");
        const unsigned gb = (unsigned)((Dn * gg + 255) / 256);
        rpa_chi0_kernel<<<gb, 256, 0, c->stream>>>((int)Dn, ng, fchi, dqs, c->d_g, c->itx, order, C1, C2, chi, A, einv);
        c->launches++;
        if (order == 1) {
            std::vector<cuDoubleComplex*> ha(Dn), hb(Dn);
            for (int64_t d = 0; d < Dn; d++) {
                ha[d] = (cuDoubleComplex*)(A + d * gg);
                hb[d] = (cuDoubleComplex*)(chi + d * gg);
            }
            int sst;
            if ((sst = cuda_check(c, cudaMemcpyAsync(pa, ha.data(), Dn * 8, cudaMemcpyHostToDevice, c->stream), "LU pointers"))) return sst;
            if ((sst = cuda_check(c, cudaMemcpyAsync(pb, hb.data(), Dn * 8, cudaMemcpyHostToDevice, c->stream), "LU pointers"))) return sst;
            int hinfo = 0;
            if (cublasZgetrfBatched(c->cublas, ng, pa, ng, piv, info, (int)Dn) != CUBLAS_STATUS_SUCCESS ||
                cublasZgetrsBatched(c->cublas, CUBLAS_OP_N, ng, ng, (const cuDoubleComplex* const*)pa, ng, piv, pb, ng, &hinfo,
                                    (int)Dn) != CUBLAS_STATUS_SUCCESS || hinfo != 0)
                return fail(c, BSE_ERR_CUDA, "cuBLAS failed in the Dyson solve");
            // the host vectors must outlive the copies: wait for them
            if ((sst = cuda_check(c, cudaStreamSynchronize(c->stream), "Dyson solve"))) return sst;
            rpa_einv_kernel<<<gb, 256, 0, c->stream>>>((int)Dn, ng, dqs, c->d_g, c->itx, chi, einv);
            c->launches++;
        }
        return cuda_check(c, cudaGetLastError(), "RPA eps^-1");
    };
    const double zq[3] = {0, 0, 0};
    st = band_states_shifted(c, zq, ecs, ev0, ccs, cv0);                    // valence at the grid k
    // grid coordinates of every k
    std::vector<int> ci(nk), cj(nk), ck(nk);
    for (int k = 0; k < nk; k++) {
        const int32_t x = dm.idx[k];
        ci[k] = x & 1023; cj[k] = (x >> 10) & 1023; ck[k] = (x >> 20) & 1023;
    }
    auto wrap = [](int a, int m) { return ((a % m) + m) % m; };
    const int64_t gtot = (int64_t)D * R * ng;
    for (int64_t d0 = 0; d0 < nd && !st; d0 += D) {
        const int64_t Dn = std::min<int64_t>(D, nd - d0);
        std::vector<double> hq(3 * Dn);
        std::vector<int64_t> hdi(Dn);
        std::vector<int> hmm(Dn * nk), hmp(Dn * nk);
        for (int64_t d = 0; d < Dn; d++) {
            const int64_t dd = d0 + d;
            const int o0 = (int)(dd % (2 * m0 - 1)) - (m0 - 1);
            const int o1 = (int)((dd / (2 * m0 - 1)) % (2 * m1 - 1)) - (m1 - 1);
            const int o2 = (int)(dd / ((int64_t)(2 * m0 - 1) * (2 * m1 - 1))) - (m2 - 1);
            const double cr[3] = {o0 * dm.step[0], o1 * dm.step[1], o2 * dm.step[2]};
            for (int x = 0; x < 3; x++)
                hq[3 * d + x] = c->bmat_h[x] * cr[0] + c->bmat_h[3 + x] * cr[1] + c->bmat_h[6 + x] * cr[2];
            hdi[d] = dd;
            for (int k = 0; k < nk; k++) {
                hmm[d * nk + k] = dm.inv[((int64_t)wrap(ci[k] - o0, m0) * m1 + wrap(cj[k] - o1, m1)) * m2 + wrap(ck[k] - o2, m2)];
                hmp[d * nk + k] = dm.inv[((int64_t)wrap(ci[k] + o0, m0) * m1 + wrap(cj[k] + o1, m1)) * m2 + wrap(ck[k] + o2, m2)];
            }
        }
        if ((st = cuda_check(c, cudaMemcpyAsync(dqs, hq.data(), 3 * Dn * 8, cudaMemcpyHostToDevice, c->stream), "RPA q"))) break;
        if ((st = cuda_check(c, cudaMemcpyAsync(ddi, hdi.data(), Dn * 8, cudaMemcpyHostToDevice, c->stream), "RPA index"))) break;
        if ((st = cuda_check(c, cudaMemcpyAsync(dmm, hmm.data(), Dn * nk * 4, cudaMemcpyHostToDevice, c->stream), "RPA map"))) break;
        if ((st = cuda_check(c, cudaMemcpyAsync(dmp, hmp.data(), Dn * nk * 4, cudaMemcpyHostToDevice, c->stream), "RPA map"))) break;
        rpa_rho_kernel<<<(unsigned)((Dn * R * ng + 255) / 256), 256, 0, c->stream>>>(
            (int)Dn, R, ng, nk, nc, nv, nw, ns, dqs, dmm, dmp, c->d_g, c->d_centres, c->d_cc, c->d_ec, cv0, ev0, cv0, ev0, eta,
            r1, q1, r2, q2);
        c->launches++;
        if ((st = eps_inv(Dn))) break;
        rpa_w_kernel<<<(unsigned)((Dn * gg + 255) / 256), 256, 0, c->stream>>>((int)Dn, ng, dqs, c->d_g, c->itx, einv, W, 0);
        const int64_t tp = Dn * nblk * nw * nw;
        rpa_phi_kernel<<<(unsigned)((tp + 255) / 256), 256, 0, c->stream>>>(
            (int)Dn, ddi, dqs, nblk, nw, NWs, ng, c->d_g, c->d_centres, W, c->d_phi,
            c->p.precision == BSE_MIXED && !c->coupled ? c->d_phi32 : nullptr, 0);
        c->launches += 2;
        if (c->d_phi_c) {
            rpa_phi_kernel<<<(unsigned)((tp + 255) / 256), 256, 0, c->stream>>>(
                (int)Dn, ddi, dqs, nblk, nw, NWs, ng, c->d_g, c->d_centres, W, c->d_phi_c, nullptr, 1);
            c->launches++;
        }
        // the host arrays of this chunk must outlive its copies
        if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "RPA chunk"))) break;
    }
    (void)gtot;
    // dk = 0: <W(q)> over the seeded sphere points, in +-q pairs (the points of the CPU restatement)
    if (!st) st = cuda_check(c, cudaMemsetAsync(avg, 0, gg * 16, c->stream), "RPA average");
    if (!st) {
        const double radius = 2.0 * kPi * std::pow(3.0 / (4.0 * kPi * nk * c->geo.vol), 1.0 / 3.0);
        std::mt19937_64 gen(c->p.rpa_seed);
        auto uni = [&gen]() { return (double)(gen() >> 11) * 0x1.0p-53; };
        double x[3] = {0, 0, 0};
        for (int n = 0; n < c->p.rpa_points && !st;) {
            double y[3];
            for (int i = 0; i < 3; i++) y[i] = uni() > 0.5 ? -uni() * radius : uni() * radius;
            const double ny = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
            if (!(ny <= radius && ny > kMinval * kMinval)) continue;
            for (int i = 0; i < 3; i++) x[i] = y[i];
            // valence at k - x and at k + x; the partner -x swaps them
            const double mx[3] = {-x[0], -x[1], -x[2]};
            if ((st = band_states_shifted(c, x, ecs, evm, ccs, cvm))) break;
            if ((st = band_states_shifted(c, mx, ecs, evp, ccs, cvp))) break;
            for (int sgn = 0; sgn < 2 && !st; sgn++) {
                const double hq[3] = {sgn ? -x[0] : x[0], sgn ? -x[1] : x[1], sgn ? -x[2] : x[2]};
                if ((st = cuda_check(c, cudaMemcpyAsync(dqs, hq, 24, cudaMemcpyHostToDevice, c->stream), "RPA q"))) break;
                rpa_rho_kernel<<<(unsigned)((R * ng + 255) / 256), 256, 0, c->stream>>>(
                    1, R, ng, nk, nc, nv, nw, ns, dqs, nullptr, nullptr, c->d_g, c->d_centres, c->d_cc, c->d_ec,
                    sgn ? cvp : cvm, sgn ? evp : evm, sgn ? cvm : cvp, sgn ? evm : evp, eta, r1, q1, r2, q2);
                c->launches++;
                if ((st = eps_inv(1))) break;
                rpa_w_kernel<<<(unsigned)((gg + 255) / 256), 256, 0, c->stream>>>(1, ng, dqs, c->d_g, c->itx, einv, avg, 1);
                c->launches++;
                if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "RPA sphere point"))) break;
            }
            n += 2;
        }
    }
    if (!st) {
        // <W> / n_points, the head times the cell average of v; then the dk = 0 table entry
        std::vector<double2> h(gg);
        st = cuda_check(c, cudaMemcpyAsync(h.data(), avg, gg * 16, cudaMemcpyDeviceToHost, c->stream), "RPA average");
        if (!st) st = cuda_check(c, cudaStreamSynchronize(c->stream), "RPA average");
        if (!st) {
            const double inv_n = 1.0 / c->p.rpa_points;
            for (auto& v : h) { v.x *= inv_n; v.y *= inv_n; }
            const int g0 = ng / 2;
            h[g0 + (int64_t)ng * g0].x *= c->itx.cell_avg;
            h[g0 + (int64_t)ng * g0].y *= c->itx.cell_avg;
            const double hz[3] = {0, 0, 0};
            const int64_t hd = dcenter;
            st = cuda_check(c, cudaMemcpyAsync(W, h.data(), gg * 16, cudaMemcpyHostToDevice, c->stream), "RPA W0");
            if (!st) st = cuda_check(c, cudaMemcpyAsync(dqs, hz, 24, cudaMemcpyHostToDevice, c->stream), "RPA q0");
            if (!st) st = cuda_check(c, cudaMemcpyAsync(ddi, &hd, 8, cudaMemcpyHostToDevice, c->stream), "RPA index");
            if (!st) {
                rpa_phi_kernel<<<(unsigned)((nblk * nw * nw + 255) / 256), 256, 0, c->stream>>>(
                    1, ddi, dqs, nblk, nw, NWs, ng, c->d_g, c->d_centres, W, c->d_phi,
                    c->p.precision == BSE_MIXED && !c->coupled ? c->d_phi32 : nullptr, 0);
                c->launches++;
                if (c->d_phi_c) {
                    rpa_phi_kernel<<<(unsigned)((nblk * nw * nw + 255) / 256), 256, 0, c->stream>>>(
                        1, ddi, dqs, nblk, nw, NWs, ng, c->d_g, c->d_centres, W, c->d_phi_c, nullptr, 1);
                    c->launches++;
                }
                st = cuda_check(c, cudaStreamSynchronize(c->stream), "RPA dk = 0");
            }
        }
    }
    cudaFreeAsync(buf, c->stream);
    int h_status = 0;
    if (!st) st = cuda_check(c, cudaMemcpyAsync(&h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "status");
    if (!st) st = cuda_check(c, cudaStreamSynchronize(c->stream), "RPA tables");
    if (!st && h_status) st = fail(c, h_status, "band states of the RPA screening");
    return st;
}

int build_h64(bse_ctx* c) {
    int st;
    const bool coll = c->S != 0;
    const int64_t n64 = coll ? 4 * c->N : c->N;
    const int dd = c->p.ipa ? 0 : 1, de = c->p.ipa ? 0 : 1;
    int pairs[6][2] = {{0, 0}, {1, 1}, {2, 2}, {3, 3}, {0, 3}, {3, 0}};
    const int npairs = coll ? 6 : 1;
    if ((st = cuda_check(c, cudaMemsetAsync(c->d_H64, 0, (size_t)n64 * n64 * sizeof(double2), c->stream), "H64 clear"))) return st;
    for (int pi = 0; pi < npairs; pi++) {
        const int br = pairs[pi][0], bc = pairs[pi][1];
        const int direct = (br == bc) ? dd : 0;
        const int exch = ((br == 0 || br == 3) && (bc == 0 || bc == 3)) ? de : 0;
        if ((st = launch_build<double>(c, c->d_H64, n64, !coll, c->d_phi, c->d_qx, br, bc, direct, exch, br == bc))) return st;
    }
    if (coll) {
        const int64_t nn = c->N * c->N;
        spin_rotate_kernel<double2><<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(c->N, c->d_H64, n64);
        c->launches++;
    }
    c->h64_pending = false;
    return cuda_check(c, cudaGetLastError(), "FP64 build");
}

int fork_h64(bse_ctx* c) {
    if (!c->h64_pending || !c->side2) return BSE_OK;
    int st;
    if ((st = cuda_check(c, cudaEventRecord(c->ev_h64, c->stream), "fork"))) return st;
    if ((st = cuda_check(c, cudaStreamWaitEvent(c->side2, c->ev_h64, 0), "fork"))) return st;
    cudaStream_t main_stream = c->stream;
    c->stream = c->side2;            // the build's launches go to the second side stream
    st = build_h64(c);
    c->stream = main_stream;
    if (st) return st;
    if ((st = cuda_check(c, cudaEventRecord(c->ev_h64, c->side2), "FP64 build done"))) return st;
    c->h64_side = true;
    return BSE_OK;
}

int run_build(bse_ctx* c, bool full, double* h_out, double* rho_out) {
    int st;
    if (!c->bands_valid) return fail(c, BSE_ERR_STATE, "bands not computed");
    if (!c->tables_valid && (st = run_tables(c))) return st;
    stage_begin(c, 2);
    const bool mixed = c->p.precision == BSE_MIXED && !c->coupled;   // the full BSE is built in FP64
    const bool coll = c->S == 1;
    // the own eigensolver reads full Hermitian storage; cuSOLVER reads the lower triangle
    const bool tile = c->build_k_hi > 0;   // rows of one k tile (bse_build_kernel_rows)
    const bool lower = !full && !tile && !coll && !c->coupled && h_out == nullptr && c->p.eig_solver != BSE_EIG_OWN;
    const int64_t ld = c->n_h;
    // every element the solver reads is written by the build (lower triangle, or all of it);
    // only the collinear layout has blocks the build never touches
    if ((coll || tile) && (st = cuda_check(c, cudaMemsetAsync(c->d_H, 0, (size_t)ld * ld * c->h_elem, c->stream), "H clear")))
        return st;
    const int dd = c->p.ipa ? 0 : 1, de = c->p.ipa ? 0 : 1;
    const void* phi = mixed ? (const void*)c->d_phi32 : (const void*)c->d_phi;
    const void* qx = mixed ? (const void*)c->d_qx32 : (const void*)c->d_qx;
    // spin-block pairs: direct + diagonal on (b,b), exchange on (0|3, 0|3)
    int pairs[6][2] = {{0, 0}, {1, 1}, {2, 2}, {3, 3}, {0, 3}, {3, 0}};
    const int npairs = coll ? 6 : 1;
    for (int pi = 0; pi < npairs; pi++) {
        const int br = pairs[pi][0], bc = pairs[pi][1];
        const int direct = (br == bc) ? dd : 0;
        const int exch = ((br == 0 || br == 3) && (bc == 0 || bc == 3)) ? de : 0;
        const int diag = br == bc;
        st = mixed ? launch_build<float>(c, c->d_H, ld, lower, phi, qx, br, bc, direct, exch, diag)
                   : launch_build<double>(c, c->d_H, ld, lower, phi, qx, br, bc, direct, exch, diag);
        if (st) return st;
    }
    if (c->coupled) {
        // coupling part, spin-block pairs: exchange on (0|3, 0|3), direct on (b, partner of b) (2986-2989)
        const int cpairs[6][2] = {{0, 0}, {3, 3}, {0, 3}, {3, 0}, {1, 2}, {2, 1}};
        for (int pi = 0; pi < (coll ? 6 : 1); pi++) {
            const int br = cpairs[pi][0], bc = cpairs[pi][1];
            const int partner = (br == 0 || br == 3) ? br : 3 - br;
            const int exch = (br == 0 || br == 3) && (bc == 0 || bc == 3);
            if ((st = launch_coupling(c, br, bc, bc == partner ? 1 : 0, exch ? 1 : 0))) return st;
        }
    }
    if (coll) {
        const int64_t nn = c->N * c->N;
        if (mixed) {
            spin_rotate_kernel<float2><<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(c->N, (float2*)c->d_H, ld);
        } else {
            spin_rotate_kernel<double2><<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(c->N, (double2*)c->d_H, ld);
            if (c->coupled)   // the coupling part is rotated the same way (3096-3105)
                spin_rotate_kernel<double2><<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(
                    c->N, (double2*)c->d_H + ld * (ld / 2), ld);
        }
        c->launches += c->coupled ? 2 : 1;
    }
    if (c->coupled) {
        const int64_t NA = ld / 2;
        coupled_lower_blocks_kernel<<<(unsigned)((NA * NA + 255) / 256), 256, 0, c->stream>>>(NA, (double2*)c->d_H);
        c->launches++;
    }
    stage_end(c, 2);
    if ((st = cuda_check(c, cudaGetLastError(), "build"))) return st;
    // the FP64 copy of the optically active block for the refinement is built later (on the side
    // stream while the FP32 eigensolve runs, or by the refinement itself)
    c->h64_pending = mixed && !c->p.ipa && c->p.n_refine > 0;
    c->h64_side = false;
    if (coll && c->coupled) {
        const int64_t n4 = 4 * c->N;
        gather_coupled_blocks_kernel<<<(unsigned)((n4 * n4 + 255) / 256), 256, 0, c->stream>>>(
            c->N, (const double2*)c->d_H, (double2*)c->d_blk, (double2*)c->d_blk + n4 * n4);
        c->launches++;
    } else if (coll) {
        const int64_t n2 = 2 * c->N;
        const size_t bb = (size_t)n2 * n2 * c->h_elem;
        if (mixed)
            gather_blocks_kernel<float2><<<(unsigned)((n2 * n2 + 255) / 256), 256, 0, c->stream>>>(
                c->N, (const float2*)c->d_H, (float2*)c->d_blk, (float2*)((char*)c->d_blk + bb));
        else
            gather_blocks_kernel<double2><<<(unsigned)((n2 * n2 + 255) / 256), 256, 0, c->stream>>>(
                c->N, (const double2*)c->d_H, (double2*)c->d_blk, (double2*)((char*)c->d_blk + bb));
        c->launches++;
    }
    if ((st = cuda_check(c, cudaGetLastError(), "build post"))) return st;
    if (h_out) {
        const size_t n = (size_t)ld * ld;
        if (mixed) {
            std::vector<float2> tmp(n);
            if ((st = cuda_check(c, cudaMemcpyAsync(tmp.data(), c->d_H, n * sizeof(float2), cudaMemcpyDeviceToHost, c->stream), "H copy"))) return st;
            if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "H copy sync"))) return st;
            for (size_t i = 0; i < n; i++) { h_out[2 * i] = tmp[i].x; h_out[2 * i + 1] = tmp[i].y; }
        } else {
            if ((st = cuda_check(c, cudaMemcpyAsync(h_out, c->d_H, n * sizeof(double2), cudaMemcpyDeviceToHost, c->stream), "H copy"))) return st;
            if (c->coupled) {
                // the device holds M; the caller gets the reference's matrix H = J M (rows NA..2NA-1 negated)
                if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "H copy sync"))) return st;
                for (int64_t j = 0; j < ld; j++)
                    for (int64_t i = ld / 2; i < ld; i++) {
                        h_out[2 * (i + ld * j)] = -h_out[2 * (i + ld * j)];
                        h_out[2 * (i + ld * j) + 1] = -h_out[2 * (i + ld * j) + 1];
                    }
            }
        }
    }
    if (rho_out) {
        if ((st = cuda_check(c, cudaMemcpyAsync(rho_out, c->d_rho, (size_t)c->n_rho * c->ng * sizeof(double2), cudaMemcpyDeviceToHost, c->stream), "rho copy"))) return st;
    }
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "build sync"))) return st;
    c->h_valid = true;
    c->eig_valid = c->osc_valid = false;
    return BSE_OK;
}


// rows r = g * nk + k (g over the n_h / nk groups (spin block, c, v), k in [k_lo, k_hi)) of H into
// a compact column-major (nrows x n_h) complex128 block
template <typename T2>
__global__ void gather_rows_kernel(int64_t n_h, int nk, int k_lo, int nt, const T2* __restrict__ H, double2* __restrict__ out) {
    const int64_t nrows = (n_h / nk) * nt;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nrows * n_h) return;
    const int64_t i = t % nrows, j = t / nrows;
    const int64_t r = (i / nt) * nk + k_lo + (i % nt);
    const T2 v = H[r + n_h * j];
    out[t] = make_double2((double)v.x, (double)v.y);
}

__global__ void narrow_h_kernel(int64_t n, const double2* __restrict__ in, float2* __restrict__ out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) out[t] = make_float2((float)in[t].x, (float)in[t].y);
}

// The rows of H whose k index lies in [k_lo, k_hi) (bse_build_kernel_rows): the build restricted to
// that k tile, the rows copied out in ascending order.  The context's matrix is left incomplete.
int run_build_rows(bse_ctx* c, int k_lo, int k_hi, double* h_rows) {
    int st;
    if (c->coupled) return fail(c, BSE_ERR_BAD_INPUT, "row tiles of the build are for the Tamm-Dancoff matrix");
    if (k_lo < 0 || k_hi > c->nk || k_lo >= k_hi) return fail(c, BSE_ERR_BAD_INPUT, "k tile outside [0, n_k)");
    if (!h_rows) return fail(c, BSE_ERR_BAD_INPUT, "null row buffer");
    c->build_k_lo = k_lo;
    c->build_k_hi = k_hi;
    st = run_build(c, true, nullptr, nullptr);
    c->build_k_lo = c->build_k_hi = 0;
    c->h_valid = false;
    c->h64_pending = false;
    if (st) return st;
    const int64_t n_h = c->n_h, nt = k_hi - k_lo, nrows = (n_h / c->nk) * nt, tot = nrows * n_h;
    double2* buf = nullptr;
    if ((st = cuda_check(c, cudaMallocAsync((void**)&buf, (size_t)tot * sizeof(double2), c->stream), "row buffer"))) return st;
    const unsigned g = (unsigned)((tot + 255) / 256);
    if (c->p.precision == BSE_MIXED)
        gather_rows_kernel<float2><<<g, 256, 0, c->stream>>>(n_h, c->nk, k_lo, (int)nt, (const float2*)c->d_H, buf);
    else
        gather_rows_kernel<double2><<<g, 256, 0, c->stream>>>(n_h, c->nk, k_lo, (int)nt, (const double2*)c->d_H, buf);
    c->launches++;
    st = cuda_check(c, cudaGetLastError(), "row gather");
    if (!st) st = cuda_check(c, cudaMemcpyAsync(h_rows, buf, (size_t)tot * sizeof(double2), cudaMemcpyDeviceToHost, c->stream), "rows copy");
    cudaFreeAsync(buf, c->stream);
    if (!st) st = cuda_check(c, cudaStreamSynchronize(c->stream), "rows sync");
    return st;
}

// H from the host (bse_set_kernel): the matrix a build would have left, e.g. gathered from row
// tiles built on other devices; the pair densities (oscillators) and, for the mixed path, the
// tables of the FP64 refinement come from this context's own bands and tables.
int run_set_kernel(bse_ctx* c, const double* h) {
    int st;
    if (c->coupled) return fail(c, BSE_ERR_BAD_INPUT, "bse_set_kernel takes the Tamm-Dancoff matrix");
    if (!h) return fail(c, BSE_ERR_BAD_INPUT, "null H");
    if (!c->bands_valid && (st = run_bands(c))) return st;
    if (!c->tables_valid && (st = run_tables(c))) return st;
    const int64_t n_h = c->n_h, nn = n_h * n_h;
    const bool mixed = c->p.precision == BSE_MIXED;
    if (mixed) {
        double2* buf = nullptr;
        if ((st = cuda_check(c, cudaMallocAsync((void**)&buf, (size_t)nn * sizeof(double2), c->stream), "H staging"))) return st;
        st = cuda_check(c, cudaMemcpyAsync(buf, h, (size_t)nn * sizeof(double2), cudaMemcpyHostToDevice, c->stream), "H upload");
        if (!st) {
            narrow_h_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(nn, buf, (float2*)c->d_H);
            c->launches++;
            st = cuda_check(c, cudaGetLastError(), "H narrow");
        }
        cudaFreeAsync(buf, c->stream);
        if (st) return st;
    } else if ((st = cuda_check(c, cudaMemcpyAsync(c->d_H, h, (size_t)nn * sizeof(double2), cudaMemcpyHostToDevice, c->stream),
                                "H upload"))) {
        return st;
    }
    if (c->S == 1) {
        const int64_t n2 = 2 * c->N;
        const size_t bb = (size_t)n2 * n2 * c->h_elem;
        if (mixed)
            gather_blocks_kernel<float2><<<(unsigned)((n2 * n2 + 255) / 256), 256, 0, c->stream>>>(
                c->N, (const float2*)c->d_H, (float2*)c->d_blk, (float2*)((char*)c->d_blk + bb));
        else
            gather_blocks_kernel<double2><<<(unsigned)((n2 * n2 + 255) / 256), 256, 0, c->stream>>>(
                c->N, (const double2*)c->d_H, (double2*)c->d_blk, (double2*)((char*)c->d_blk + bb));
        c->launches++;
    }
    if ((st = cuda_check(c, cudaGetLastError(), "set kernel"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "set kernel sync"))) return st;
    c->h64_pending = mixed && !c->p.ipa && c->p.n_refine > 0;
    c->h64_side = false;
    c->h_valid = true;
    c->eig_valid = c->osc_valid = false;
    return BSE_OK;
}

}  // namespace bse
