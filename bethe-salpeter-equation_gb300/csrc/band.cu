// Two-stage Householder tridiagonalization for the own eigensolver at large n.
//
// Same result as the one-stage reduction of tridiag.cu -- Q^H A Q = T real symmetric
// tridiagonal, y = Q^H rho, and X = Q Z for the eigenvectors that are asked for -- with a
// fraction of its memory traffic (the one-stage reduction reads and rewrites the whole trailing
// matrix for every column, 2 * 8 B * n^3 / 3 in total):
//
//  1. dense -> band, bandwidth NB.  For every panel of NB columns, a blocked Householder QR of the
//     part below the band (panel_qr_kernel: cooperative, the panel held in shared memory, two
//     grid barriers per column, the compact-WY factor T and y <- Q_j^H y in the same launch),
//     then the two-sided trailing update A22 <- Q_j^H A22 Q_j as one Hermitian rank-2NB update
//       X = A22 V T,  W = X - 1/2 V (T^H V^H X),  A22 -= V W^H + W V^H
//     through cuBLAS hemm / her2k (plain library BLAS-3), so the trailing matrix is touched once
//     per NB columns instead of once per column;
//  2. band -> tridiagonal by bulge chasing (chase_kernel, persistent).  Sweep s annihilates
//     column s of the band with a length-NB reflector and chases the resulting bulge down the
//     band one NB block per step; the band (with room for the bulge, 2 NB sub-diagonals) stays
//     in L2.  Sweeps run concurrently, sweep s on CTA s mod G; step t of sweep s waits until
//     sweep s-1 has finished step t+2 (the last of its steps whose footprint overlaps), so every
//     element sees the updates in the sequential order;
//  3. X = Q1 Q2 Z: the bulge reflectors, sweep by sweep in reverse order (the reflectors of one
//     sweep act on disjoint rows and commute; apply_q2_kernel), then the panel reflectors in
//     compact-WY form through cuBLAS gemm / trmm.
//
// The reference diagonalizes with LAPACK zheevd (bse.version13.cpp:3195, 3330), whose zhetrd is
// the one-stage blocked reduction; eigenvalues agree to the precision of the arithmetic.
// Every wait on another block is bounded and reports through the error word.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <utility>
#include <string>
#include <type_traits>

#include "blas_ops.h"
#include "bse_internal.h"
#include "dev_util.h"

namespace bse {
namespace {

using namespace dev;

constexpr int NB = 32;          // band width = panel width = reflector length of the chase
constexpr int LDB = 2 * NB;     // sub-diagonals kept per band column (band + bulge)
constexpr int kPanelThreads = 256;
constexpr int kChaseThreads = 128;
constexpr int kQ2Threads = 256;

template <typename T2> __device__ __forceinline__ T2 ld(const T2* p) { return __ldcg(p); }
template <typename T2> inline T2 C2h(double x, double y) {
    T2 r;
    r.x = x;
    r.y = y;
    return r;
}
template <typename T2> __device__ __forceinline__ T2 conj2(T2 a) { return C2<T2>(a.x, -a.y); }
template <typename T2> __device__ __forceinline__ T2 shfl2(T2 v, int src) {
    return C2<T2>(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// zlarfg: H = I - tau v v^H, v_0 = 1, H^H (alpha; x) = (beta; 0) with beta real.
template <typename T2>
__device__ __forceinline__ void householder(T2 alpha, typename Real<T2>::t xnorm2, T2& tau,
                                            typename Real<T2>::t& beta, T2& scal) {
    typedef typename Real<T2>::t R;
    if (xnorm2 == R(0) && alpha.y == R(0)) {
        tau = C2<T2>(0, 0);
        beta = alpha.x;
        scal = C2<T2>(0, 0);
    } else {
        beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2), alpha.x);
        tau = C2<T2>((beta - alpha.x) / beta, -alpha.y / beta);
        scal = cinv(csub(alpha, C2<T2>(beta, 0)));
    }
}

// ------------------------------------------------------------------------------------------
// Stage 1: Householder QR of one m x NB panel (the columns c0..c0+NB-1 below the band).
// ------------------------------------------------------------------------------------------
template <typename T2>
struct PanelArgs {
    int m, kk, S, SP;           // rows, reflectors (min(NB, m)), rows per block, smem column stride
    T2* P;                      // panel (column-major, leading dimension lda); R is written back
    int64_t lda;
    T2* V;                      // explicit reflectors, m x kk (ld m): unit diagonal, zeros above
    T2* T;                      // NB x NB upper triangular compact-WY factor
    T2* tau;                    // NB
    T2* y;                      // rows of the vector Q^H is applied to (length m), or null
    T2* pnorm;                  // [G] partial column norms (.x)
    T2* pw;                     // [G][NB] partial v^H P
    T2* pgram;                  // [G][NB*NB + NB] partial V^H V and V^H y
    T2* bc;                     // [NB + 1] broadcast: T^H V^H y, alpha
    unsigned* flags;            // flag barrier, epochs from `epoch0` up (monotonic over the panels)
    unsigned epoch0;
    int* err;
};

template <typename T2>
__global__ void __launch_bounds__(kPanelThreads, 1) panel_qr_kernel(PanelArgs<T2> a) {
    typedef typename Real<T2>::t R;
    extern __shared__ unsigned char smraw[];
    const int S = a.S, SP = a.SP;
    T2* Ps = reinterpret_cast<T2*>(smraw);              // [NB][SP] the block's rows of the panel
    T2* ys = Ps + (size_t)NB * SP;                      // [S] the block's rows of y
    T2* sw = ys + S;                                    // [NB]
    T2* stau = sw + NB;                                 // [NB]
    T2* Gs = stau + NB;                                 // [NB][NB + 1]
    T2* Ts = Gs + NB * (NB + 1);                        // [NB][NB + 1]
    R* red = reinterpret_cast<R*>(Ts + NB * (NB + 1));  // 32 R
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    const int g = blockIdx.x, G = gridDim.x;
    const int row0 = g * S, nr = max(0, min(S, a.m - row0));
    __shared__ int s_fail;
    if (tid == 0) s_fail = 0;
    unsigned epoch = a.epoch0;
    auto barrier = [&]() { return flag_barrier<false>(a.flags, ++epoch, a.err, &s_fail); };
    const int kk = a.kk;
    const int64_t lda = a.lda;
    const T2 zero = C2<T2>(0, 0), one = C2<T2>(1, 0);
    for (int idx = tid; idx < nr * NB; idx += nthr) {
        const int r = idx % nr, cc = idx / nr;
        Ps[cc * SP + r] = a.P[(row0 + r) + cc * lda];
    }
    if (a.y)
        for (int r = tid; r < nr; r += nthr) ys[r] = a.y[row0 + r];
    __syncthreads();
    // element (global row gr, column cc) of the explicit V from the slab
    auto vexp = [&](int cc, int r) -> T2 {
        const int gr = row0 + r;
        return gr < cc ? zero : (gr == cc ? one : Ps[cc * SP + r]);
    };

    for (int i = 0; i < kk; i++) {
        T2* col = Ps + i * SP;
        R loc[1] = {0};
        for (int r = tid; r < nr; r += nthr)
            if (row0 + r > i) {
                const T2 x = col[r];
                loc[0] += x.x * x.x + x.y * x.y;
            }
        block_sums<R, 1>(loc, red);
        if (tid == 0) {
            a.pnorm[g] = C2<T2>(loc[0], 0);
            if (g == 0) a.bc[NB] = col[i];   // alpha: row i < NB <= S lies in block 0
        }
        if (!barrier()) return;
        R tot[1] = {0};
        for (int q = tid; q < G; q += nthr) tot[0] += ld(a.pnorm + q).x;
        block_sums<R, 1>(tot, red);
        const T2 alpha = ld(a.bc + NB);
        T2 tau, scal;
        R beta;
        householder<T2>(alpha, tot[0], tau, beta, scal);
        for (int r = tid; r < nr; r += nthr)
            if (row0 + r > i) col[r] = cmul(col[r], scal);
        if (tid == 0) stau[i] = tau;
        __syncthreads();
        // partial w_c = sum_{rows >= i} conj(v_r) P[r][c] for the columns right of i (all NB of
        // them: with m < NB the reflectors stop at kk = m but R = Q^H P spans every column)
        for (int cc = i + 1 + warp; cc < NB; cc += nwarp) {
            R ax = 0, ay = 0;
            for (int r = lane; r < nr; r += 32) {
                const int gr = row0 + r;
                if (gr < i) continue;
                const T2 v = gr == i ? one : col[r];
                const T2 q = cconjmul(v, Ps[cc * SP + r]);
                ax += q.x;
                ay += q.y;
            }
            ax = warp_sum(ax);
            ay = warp_sum(ay);
            if (lane == 0) a.pw[(size_t)g * NB + cc] = C2<T2>(ax, ay);
        }
        if (!barrier()) return;
        {
            // 8 threads per column sum the block partials
            const int cc = tid >> 3, sub = tid & 7;
            R sx = 0, sy = 0;
            if (cc > i)
                for (int q = sub; q < G; q += 8) {
                    const T2 u = ld(a.pw + (size_t)q * NB + cc);
                    sx += u.x;
                    sy += u.y;
                }
            for (int o = 4; o > 0; o >>= 1) {
                sx += __shfl_xor_sync(0xffffffffu, sx, o);
                sy += __shfl_xor_sync(0xffffffffu, sy, o);
            }
            if (sub == 0 && cc < NB) sw[cc] = C2<T2>(sx, sy);
        }
        __syncthreads();
        // P <- H^H P = P - conj(tau) v (v^H P) on the columns right of i
        const T2 ctau = conj2(tau);
        for (int idx = tid; idx < nr * (NB - i - 1); idx += nthr) {
            const int r = idx % nr, cc = i + 1 + idx / nr;
            const int gr = row0 + r;
            if (gr < i) continue;
            const T2 v = gr == i ? one : col[r];
            Ps[cc * SP + r] = csub(Ps[cc * SP + r], cmul(ctau, cmul(v, sw[cc])));
        }
        __syncthreads();
        if (g == 0 && tid == 0) {
            col[i] = C2<T2>(beta, 0);
            a.tau[i] = tau;
        }
        __syncthreads();
    }
    // explicit V, partial Gram matrix V^H V (strict upper part) and V^H y
    for (int idx = tid; idx < nr * kk; idx += nthr) {
        const int r = idx % nr, cc = idx / nr;
        a.V[(size_t)(row0 + r) + (size_t)cc * a.m] = vexp(cc, r);
    }
    for (int e = tid; e < NB * NB + NB; e += nthr) {
        R sx = 0, sy = 0;
        if (e < NB * NB) {
            const int p = e % NB, q = e / NB;
            if (p < q && q < kk)
                for (int r = 0; r < nr; r++) {
                    const T2 t = cconjmul(vexp(p, r), vexp(q, r));
                    sx += t.x;
                    sy += t.y;
                }
        } else if (a.y) {
            const int p = e - NB * NB;
            if (p < kk)
                for (int r = 0; r < nr; r++) {
                    const T2 t = cconjmul(vexp(p, r), ys[r]);
                    sx += t.x;
                    sy += t.y;
                }
        }
        a.pgram[(size_t)g * (NB * NB + NB) + e] = C2<T2>(sx, sy);
    }
    if (!barrier()) return;
    if (g == 0) {
        for (int e = tid; e < NB * NB + NB; e += nthr) {
            R sx = 0, sy = 0;
            for (int q = 0; q < G; q++) {
                const T2 u = ld(a.pgram + (size_t)q * (NB * NB + NB) + e);
                sx += u.x;
                sy += u.y;
            }
            if (e < NB * NB) Gs[(e % NB) * (NB + 1) + e / NB] = C2<T2>(sx, sy);
            else sw[e - NB * NB] = C2<T2>(sx, sy);
        }
        for (int e = tid; e < NB * (NB + 1); e += nthr) Ts[e] = zero;
        __syncthreads();
        // T (zlarft, forward, columnwise): T[0:i, i] = -tau_i T[0:i, 0:i] G[0:i, i], T[i][i] = tau_i
        for (int i = 0; i < kk; i++) {
            T2 acc = zero;
            if (tid < i)
                for (int l = tid; l < i; l++) acc = cadd(acc, cmul(Ts[tid * (NB + 1) + l], Gs[l * (NB + 1) + i]));
            __syncthreads();
            if (tid < i) Ts[tid * (NB + 1) + i] = cmul(C2<T2>(-stau[i].x, -stau[i].y), acc);
            if (tid == i) Ts[i * (NB + 1) + i] = stau[i];
            __syncthreads();
        }
        for (int e = tid; e < NB * NB; e += nthr) a.T[e] = Ts[(e % NB) * (NB + 1) + e / NB];
        // T^H (V^H y)
        if (tid < NB) {
            T2 s = zero;
            if (tid < kk)
                for (int l = 0; l <= tid; l++) s = cadd(s, cconjmul(Ts[l * (NB + 1) + tid], sw[l]));
            a.bc[tid] = s;
        }
        // R: the upper trapezoid of the top kk x NB block, the band part of these columns
        for (int idx = tid; idx < kk * NB; idx += nthr) {
            const int r = idx % kk, cc = idx / kk;
            if (r <= cc) a.P[r + cc * lda] = Ps[cc * SP + r];
        }
    }
    if (!a.y) return;
    if (!barrier()) return;
    // y <- y - V (T^H V^H y)
    for (int r = tid; r < nr; r += nthr) {
        T2 s = ys[r];
        for (int p = 0; p < kk; p++) s = csub(s, cmul(vexp(p, r), ld(a.bc + p)));
        a.y[row0 + r] = s;
    }
}

// Copy the band (NB sub-diagonals) of the reduced matrix into band storage with room for the bulge.
template <typename T2>
__global__ void band_extract_kernel(int n, const T2* __restrict__ A, int64_t lda, T2* __restrict__ AB) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)LDB * n) return;
    const int d = (int)(t % LDB), c = (int)(t / LDB);
    AB[t] = (d <= NB && c + d < n) ? A[(c + d) + (int64_t)c * lda] : C2<T2>(0, 0);
}

// ------------------------------------------------------------------------------------------
// Stage 2: bulge chasing on the band.
// ------------------------------------------------------------------------------------------
template <typename T2>
struct ChaseArgs {
    int n;
    T2* AB;          // AB[d + c * LDB] = A[c + d][c], 0 <= d < LDB
    T2* y;           // Q2^H applied in place, or null
    T2* V2;          // reflectors packed by sweep (slot of v_0 = 1 holds tau), or null
    int* prog;       // steps finished per sweep
    int* err;
};

__host__ __device__ __forceinline__ int chase_steps(int n, int s) { return (n - 1 - s + NB - 1) / NB; }
__host__ __device__ __forceinline__ int64_t v2_offset(int n, int64_t s) { return s * (n - 1) - s * (s - 1) / 2; }

// Thread (lane i, warp w) holds elements (i, w + 4 k), k < 8, of the 32 x 32 blocks of one step:
// L = rows I_t x cols I_{t-1} (carried in registers from the previous step), D = I_t x I_t and
// Rb = I_{t+1} x I_t, with I_t = [s+1+t NB, s+(t+1) NB].
template <typename T2>
__global__ void __launch_bounds__(kChaseThreads) chase_kernel(ChaseArgs<T2> a) {
    typedef typename Real<T2>::t R;
    __shared__ T2 sx[NB];
    __shared__ T2 sred[4][NB];
    __shared__ T2 sred2[4][NB];
    const int tid = threadIdx.x, lane = tid & 31, wy = tid >> 5;
    const int n = a.n;
    const T2 zero = C2<T2>(0, 0);
    T2* AB = a.AB;
    for (int s = blockIdx.x; s <= n - 2; s += gridDim.x) {
        const int Tn = chase_steps(n, s);
        const int Tp = s > 0 ? chase_steps(n, s - 1) : 0;
        T2 L[8];
#pragma unroll
        for (int k = 0; k < 8; k++) L[k] = zero;
        for (int t = 0; t < Tn; t++) {
            if (s > 0) {
                if (tid == 0) {
                    const int need = min(t + 3, Tp);
                    volatile int* vp = a.prog + (s - 1);
                    volatile int* verr = a.err;
                    unsigned it = 0;
                    while (*vp < need) {
                        if (*verr != 0) break;
                        if (++it > spin_limit(a.err)) {
                            atomicExch(a.err, 2);
                            break;
                        }
                        __nanosleep(64);
                    }
                    __threadfence();
                }
                __syncthreads();
                if (*(volatile int*)a.err != 0) return;
            }
            const int lo = s + 1 + t * NB, len = min(NB, n - lo), hi = lo + len;
            const int len2 = max(0, min(NB, n - hi));
            // loads of D (Hermitian, from the lower band) and of the block below
            T2 D[8], Rb[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int i = lane, j = wy + 4 * k;
                D[k] = zero;
                Rb[k] = zero;
                if (i < len && j < len)
                    D[k] = i >= j ? ld(AB + (i - j) + (int64_t)(lo + j) * LDB)
                                  : conj2(ld(AB + (j - i) + (int64_t)(lo + i) * LDB));
                if (i < len2 && j < len) Rb[k] = ld(AB + (NB + i - j) + (int64_t)(lo + j) * LDB);
            }
            // the column whose entries below its first one are annihilated, staged in shared memory:
            // warp 0 overwrites it below, so no warp may read it from global memory after the barrier
            if (wy == 0) sx[lane] = t == 0 ? (lane < len ? ld(AB + (1 + lane) + (int64_t)s * LDB) : zero) : L[0];
            __syncthreads();
            const T2 xi = sx[lane];
            const T2 alpha = shfl2(xi, 0);
            const R xn2 = warp_sum(lane >= 1 && lane < len ? xi.x * xi.x + xi.y * xi.y : R(0));
            T2 tau, scal;
            R beta;
            householder<T2>(alpha, xn2, tau, beta, scal);
            const T2 v = lane == 0 ? C2<T2>(1, 0) : (lane < len ? cmul(xi, scal) : zero);
            const T2 ctau = conj2(tau);
            if (t >= 1) {
                // L <- H^H L; its first column becomes (beta, 0, ..., 0)
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const T2 q = cconjmul(v, L[k]);
                    const T2 w = C2<T2>(warp_sum(q.x), warp_sum(q.y));
                    L[k] = csub(L[k], cmul(ctau, cmul(v, w)));
                }
                if (wy == 0) L[0] = lane == 0 ? C2<T2>(beta, 0) : zero;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const int i = lane, j = wy + 4 * k;
                    if (i < len) __stcg(AB + (NB + i - j) + (int64_t)(lo - NB + j) * LDB, L[k]);
                }
            } else if (lane < len && wy == 0) {
                __stcg(AB + (1 + lane) + (int64_t)s * LDB, lane == 0 ? C2<T2>(beta, 0) : zero);
            }
            // D <- H^H D H:  x = tau D v,  w = x - 1/2 conj(tau) (v^H x) v,  D -= v w^H + w v^H
            {
                T2 px = zero;
#pragma unroll
                for (int k = 0; k < 8; k++) px = cadd(px, cmul(D[k], shfl2(v, wy + 4 * k)));
                sred[wy][lane] = px;
            }
            {
                T2 pz = zero;
#pragma unroll
                for (int k = 0; k < 8; k++) pz = cadd(pz, cmul(Rb[k], shfl2(v, wy + 4 * k)));
                sred2[wy][lane] = pz;
            }
            __syncthreads();
            const T2 xr = cmul(tau, cadd(cadd(sred[0][lane], sred[1][lane]), cadd(sred[2][lane], sred[3][lane])));
            const T2 vx = cconjmul(v, xr);
            const T2 sdot = C2<T2>(warp_sum(vx.x), warp_sum(vx.y));
            const T2 wv = csub(xr, cmul(C2<T2>(R(0.5) * ctau.x, R(0.5) * ctau.y), cmul(sdot, v)));
            const T2 zr = cadd(cadd(sred2[0][lane], sred2[1][lane]), cadd(sred2[2][lane], sred2[3][lane]));
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int i = lane, j = wy + 4 * k;
                const T2 vj = shfl2(v, j), wj = shfl2(wv, j);
                D[k] = csub(D[k], cadd(cmulc(v, wj), cmulc(wv, vj)));
                if (i < len && j < len && i >= j) __stcg(AB + (i - j) + (int64_t)(lo + j) * LDB, D[k]);
                // Rb <- Rb H = Rb - tau (Rb v) v^H
                Rb[k] = csub(Rb[k], cmulc(cmul(tau, zr), vj));
            }
            if (wy == 0) {
                if (a.y) {
                    const T2 yi = lane < len ? ld(a.y + lo + lane) : zero;
                    const T2 q = cconjmul(v, yi);
                    const T2 sy = C2<T2>(warp_sum(q.x), warp_sum(q.y));
                    if (lane < len) __stcg(a.y + lo + lane, csub(yi, cmul(ctau, cmul(sy, v))));
                }
                if (a.V2 && lane < len) a.V2[v2_offset(n, s) + (int64_t)t * NB + lane] = lane == 0 ? tau : v;
            }
#pragma unroll
            for (int k = 0; k < 8; k++) L[k] = Rb[k];
            __threadfence();
            __syncthreads();
            if (tid == 0) atomicExch(a.prog + s, t + 1);
        }
    }
}

template <typename T2, typename R>
__global__ void band_diag_kernel(int n, const T2* __restrict__ AB, R* __restrict__ d, R* __restrict__ e) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = AB[(int64_t)i * LDB].x;
    if (i < n - 1) e[i] = AB[1 + (int64_t)i * LDB].x;
}

// ------------------------------------------------------------------------------------------
// Back-transformation.
// ------------------------------------------------------------------------------------------
// Z (row-major, nvec columns per row) <- Q2 Z, sweeps from last to first, one grid barrier each.
// A warp applies one reflector to 32 columns: lane = column, the reflector's rows in registers.
template <typename T2>
__global__ void __launch_bounds__(kQ2Threads, 1) apply_q2_kernel(int n, const T2* __restrict__ V2, T2* __restrict__ Z,
                                                                 int nvec, unsigned* flags, int* err) {
    __shared__ int s_fail;
    if (threadIdx.x == 0) s_fail = 0;
    unsigned epoch = 0;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    const int nch = (nvec + 31) / 32;
    const T2 zero = C2<T2>(0, 0);
    for (int s = n - 2; s >= 0; s--) {
        const int Tn = chase_steps(n, s);
        const int64_t off = v2_offset(n, s);
        for (int item = gw; item < Tn * nch; item += nwarps) {
            const int t = item / nch, col = (item % nch) * 32 + lane;
            const int lo = s + 1 + t * NB, len = min(NB, n - lo);
            const T2 vl = lane < len ? ld(V2 + off + (int64_t)t * NB + lane) : zero;
            const T2 tau = shfl2(vl, 0);
            const bool ok = col < nvec;
            T2 zr[NB];
            T2 w = zero;
#pragma unroll
            for (int i = 0; i < NB; i++) {
                zr[i] = (i < len && ok) ? ld(Z + (int64_t)(lo + i) * nvec + col) : zero;
                const T2 vi = i == 0 ? C2<T2>(1, 0) : shfl2(vl, i);
                w = cadd(w, cconjmul(vi, zr[i]));
            }
            const T2 tw = cmul(tau, w);
#pragma unroll
            for (int i = 0; i < NB; i++) {
                const T2 vi = i == 0 ? C2<T2>(1, 0) : shfl2(vl, i);
                if (i < len && ok) __stcg(Z + (int64_t)(lo + i) * nvec + col, csub(zr[i], cmul(vi, tw)));
            }
        }
        if (!flag_barrier<true>(flags, ++epoch, err, &s_fail)) return;
    }
}

// out (cols x rows, ld_out) = transpose of in (rows x cols, ld_in), real or complex input.
template <typename Tin, typename T2>
__global__ void transpose_kernel(int rows, int cols, const Tin* __restrict__ in, int64_t ld_in, T2* __restrict__ out,
                                 int64_t ld_out) {
    __shared__ T2 tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = bx + threadIdx.x, c = by + j;
        T2 v = C2<T2>(0, 0);
        if (r < rows && c < cols) {
            const Tin x = in[r + (int64_t)c * ld_in];
            if constexpr (std::is_same<Tin, T2>::value) v = x;
            else v = C2<T2>(x, 0);
        }
        tile[j][threadIdx.x] = v;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = by + threadIdx.x, r = bx + j;
        if (r < rows && c < cols) out[c + (int64_t)r * ld_out] = tile[threadIdx.x][j];
    }
}

int blas_check(bse_ctx* c, cublasStatus_t s, const char* what) {
    if (s == CUBLAS_STATUS_SUCCESS) return BSE_OK;
    return fail(c, BSE_ERR_CUDA, std::string("cuBLAS failed in the two-stage reduction: ") + what);
}

// Workspace of the two-stage path; the same layout is used by the reduction and the back-transform.
struct Layout {
    size_t vall, tall, tau, ybuf, xbuf, lr, small, pnorm, pw, pgram, bc, ab, prog, flags, v2, zrm, tcws, total;
    int npanel, gmax;
    int64_t vsize;
};

size_t al256(size_t x) { return (x + 255) / 256 * 256; }

Layout layout(int n, size_t e, bool keep_q, int gmax, int n_vec) {
    Layout L{};
    L.npanel = 0;
    int64_t vs = 0;
    for (int j = 0; (int64_t)(j + 1) * NB < n; j++) {
        const int m = n - (j + 1) * NB;
        vs += (int64_t)m * std::min(NB, m);
        L.npanel++;
    }
    L.vsize = vs;
    L.gmax = gmax;
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += al256(bytes); return o; };
    L.vall = carve((keep_q ? (size_t)vs : (size_t)n * NB) * e);
    L.tall = carve((size_t)std::max(L.npanel, 1) * NB * NB * e);
    L.tau = carve((size_t)std::max(L.npanel, 1) * NB * e);
    L.ybuf = carve((size_t)n * NB * e);
    L.xbuf = carve((size_t)n * NB * e);
    L.lr = carve(4 * (size_t)n * NB * e);   // [V W] and [W V] for the full-storage update
    L.small = carve(4 * (size_t)NB * NB * e + (size_t)NB * std::max(n_vec, 1) * e * 2);
    L.pnorm = carve((size_t)gmax * e);
    L.pw = carve((size_t)gmax * NB * e);
    L.pgram = carve((size_t)gmax * (NB * NB + NB) * e);
    L.bc = carve((NB + 8) * e);
    L.ab = carve((size_t)LDB * n * e);
    L.prog = carve((size_t)n * sizeof(int));
    L.flags = carve((size_t)gmax * 128);   // one barrier flag per block, 128 bytes apart
    L.v2 = carve(keep_q ? (size_t)v2_offset(n, n - 1) * e : 0);
    L.zrm = carve(keep_q ? (size_t)n * std::max(n_vec, 1) * e : 0);
    L.tcws = carve(e == sizeof(float2) ? tc_workspace(n, gmax) : 0);   // tensor-core update operands
    L.total = off;
    return L;
}

int device_sms(bse_ctx* c) {
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    return std::max(1, nsm);
}

template <typename T2>
size_t panel_smem(int S) {
    typedef typename Real<T2>::t R;
    return ((size_t)NB * (S + 1) + S + 2 * NB + 2 * NB * (NB + 1)) * sizeof(T2) + 32 * sizeof(R);
}

template <typename T2> int max_panel_rows() { return sizeof(T2) == 8 ? 640 : 320; }

template <typename T2>
int band_tridiag_t(bse_ctx* c, int n, T2* A, int64_t lda, typename Real<T2>::t* d, typename Real<T2>::t* e, T2* y,
                   bool keep_q, char* ws, unsigned* bar, int* err, int n_vec) {
    typedef typename Real<T2>::t R;
    int st;
    const int nsm = device_sms(c);
    const Layout Ly = layout(n, sizeof(T2), keep_q, nsm, n_vec);
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(panel_qr_kernel<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)panel_smem<T2>(max_panel_rows<T2>()));
    });
    if ((st = cuda_check(c, attr_err, "panel kernel attribute"))) return st;
    if ((st = blas_check(c, cublasSetStream(c->cublas, c->stream), "stream"))) return st;
    cublasMath_t math_prev = CUBLAS_DEFAULT_MATH;
    cublasGetMathMode(c->cublas, &math_prev);
    if (const char* v = std::getenv("BSE_BLAS_MATH")) {
        const std::string mv(v);
        cublasSetMathMode(c->cublas, mv == "pedantic" ? CUBLAS_PEDANTIC_MATH
                                     : mv == "bf16x9" ? CUBLAS_FP32_EMULATED_BF16X9_MATH : CUBLAS_DEFAULT_MATH);
    }
    T2* Vall = (T2*)(ws + Ly.vall);
    T2* Tall = (T2*)(ws + Ly.tall);
    T2* taus = (T2*)(ws + Ly.tau);
    T2* Ybuf = (T2*)(ws + Ly.ybuf);
    T2* Xbuf = (T2*)(ws + Ly.xbuf);
    T2* Msm = (T2*)(ws + Ly.small);
    T2* Nsm = Msm + NB * NB;
    const T2 one = C2h<T2>(1, 0), zero = C2h<T2>(0, 0), mone = C2h<T2>(-1, 0), mhalf = C2h<T2>(-0.5, 0);
    const R rone = 1;
    // trailing update: Hermitian BLAS-3 on the lower triangle (hemm / her2k), or, for complex64,
    // full-storage GEMMs (BSE_BAND_UPDATE=gemm, or =emul for the BF16x9 tensor-core emulation of
    // FP32 GEMM; the own solver's matrix is built in full storage)
    bool full_update = false;
    cublasComputeType_t ctype = CUBLAS_COMPUTE_32F;
    cublasEmulationStrategy_t emu_prev = CUBLAS_EMULATION_STRATEGY_DEFAULT;
    cublasGetEmulationStrategy(c->cublas, &emu_prev);
    if (const char* v = std::getenv("BSE_BAND_UPDATE")) {
        const std::string mv(v);
        if (sizeof(T2) == sizeof(float2) && (mv == "gemm" || mv == "emul")) {
            full_update = true;
            if (mv == "emul") {
                ctype = CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
                cublasSetEmulationStrategy(c->cublas, CUBLAS_EMULATION_STRATEGY_EAGER);
            }
        }
    }
    // complex64: both products of the trailing update on the tensor cores (tc_update.cu) by default;
    // BSE_BAND_UPDATE=cublas keeps cuBLAS hemm / her2k, "gemm" / "emul" the full-storage GEMMs
    bool use_tc = false, tc_h = false, tc_u = false;
    if constexpr (sizeof(T2) == sizeof(float2)) {
        const char* v = std::getenv("BSE_BAND_UPDATE");
        // every trailing order m = n - 32 (j + 1) is even when n is (the TMA tiles need 2m reals
        // in whole 16-byte granules)
        use_tc = !full_update && (!v || std::string(v) == "tc") && n % 2 == 0 && tc_supported(lda);
        // BSE_TC (sweeps): "hemm" or "update" keeps only that product on the tensor cores
        const char* w = std::getenv("BSE_TC");
        const std::string tw = w ? w : "both";
        tc_h = use_tc && (tw == "both" || tw == "hemm");
        tc_u = use_tc && (tw == "both" || tw == "update");
        if (tc_h && !tc_u) full_update = true;   // the tensor-core hemm reads full storage
    }
    char* tcws = ws + Ly.tcws;
    c->kt_used = 0;   // the kernel timing describes the last reduction
    int64_t voff = 0;
    unsigned* flags = (unsigned*)(ws + Ly.flags);
    if ((st = cuda_check(c, cudaMemsetAsync(flags, 0, (size_t)Ly.gmax * 128, c->stream), "barrier flags"))) return st;
    stage_begin(c, 13);
    for (int j = 0; j < Ly.npanel; j++) {
        const int c0 = j * NB, r0 = c0 + NB, m = n - r0, kk = std::min(NB, m);
        T2* Vj = keep_q ? Vall + voff : Vall;
        T2* Tj = Tall + (size_t)j * NB * NB;
        voff += (int64_t)m * kk;
        // rows per block: spread the panel over the SMs, at least NB rows (row i < NB in block 0)
        int S = std::max(64, (int)(((int64_t)m + nsm - 1) / nsm + 31) / 32 * 32);
        if (const char* v = std::getenv("BSE_PANEL_ROWS")) S = std::max(S, (std::atoi(v) + 31) / 32 * 32);
        if (S > max_panel_rows<T2>()) return fail(c, BSE_ERR_BAD_INPUT, "matrix too large for the two-stage panel kernel");
        const int G = (m + S - 1) / S;
        PanelArgs<T2> pa;
        pa.m = m; pa.kk = kk; pa.S = S; pa.SP = S + 1;
        pa.P = A + r0 + (int64_t)c0 * lda; pa.lda = lda;
        pa.V = Vj; pa.T = Tj; pa.tau = taus + (size_t)j * NB;
        pa.y = y ? y + r0 : nullptr;
        pa.pnorm = (T2*)(ws + Ly.pnorm); pa.pw = (T2*)(ws + Ly.pw); pa.pgram = (T2*)(ws + Ly.pgram);
        pa.bc = (T2*)(ws + Ly.bc); pa.flags = flags; pa.err = err;
        pa.epoch0 = (unsigned)j * (2 * NB + 4);   // at most 2 NB + 2 barriers per panel
        void* kargs[] = {&pa};
        if ((st = cuda_check(c, cudaLaunchCooperativeKernel((void*)panel_qr_kernel<T2>, dim3(G), dim3(kPanelThreads), kargs,
                                                            panel_smem<T2>(S), c->stream), "panel QR launch"))) return st;
        c->launches++;
        // A22 <- Q^H A22 Q
        T2* A22 = A + r0 + (int64_t)r0 * lda;
        cublasHandle_t h = c->cublas;
        if constexpr (sizeof(T2) == sizeof(float2)) {
            if (tc_h) {
                int nl = 0;
                cudaEvent_t* ev = kernel_timer(c, 0, 8.0 * m * m, 8.0 * m * m * kk);
                if (tc_hemm(c->stream, nsm, m, kk, A22, lda, Vj, Ybuf, tcws, err, &nl, ev))
                    return fail(c, BSE_ERR_CUDA, "tensor-core hemm of the two-stage reduction failed to launch");
                c->launches += nl;
            }
        }
        if (tc_h) {
        } else if (full_update) {
            if ((st = blas_check(c, cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m, kk, m, &one, A22, CUDA_C_32F, (int)lda, Vj, CUDA_C_32F, m,
                                                 &zero, Ybuf, CUDA_C_32F, m, ctype, CUBLAS_GEMM_DEFAULT), "gemm AV"))) return st;
        } else {
            if ((st = blas_check(c, xhemm(h, m, kk, &one, A22, (int)lda, Vj, m, &zero, Ybuf, m), "hemm"))) return st;
        }
        if ((st = blas_check(c, xtrmm(h, CUBLAS_SIDE_RIGHT, CUBLAS_OP_N, m, kk, &one, Tj, NB, Ybuf, m, Xbuf, m), "trmm"))) return st;
        if ((st = blas_check(c, xgemm(h, CUBLAS_OP_C, CUBLAS_OP_N, kk, kk, m, &one, Vj, m, Xbuf, m, &zero, Msm, NB), "gemm VX"))) return st;
        if ((st = blas_check(c, xtrmm(h, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, kk, kk, &one, Tj, NB, Msm, NB, Nsm, NB), "trmm T^H"))) return st;
        if ((st = blas_check(c, xgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, kk, kk, &mhalf, Vj, m, Nsm, NB, &one, Xbuf, m), "gemm W"))) return st;
        if constexpr (sizeof(T2) == sizeof(float2)) {
            if (tc_u) {
                int nl = 0;
                cudaEvent_t* ev = kernel_timer(c, 1, 16.0 * m * m, 16.0 * m * m * kk);
                if (tc_rank2k(c->stream, nsm, m, kk, A22, lda, Vj, Xbuf, tcws, err, &nl, ev))
                    return fail(c, BSE_ERR_CUDA, "tensor-core update of the two-stage reduction failed to launch");
                c->launches += nl;
            }
        }
        if (tc_u) {
        } else if (full_update) {
            // A22 -= [V W] [W V]^H on full storage, one GEMM with k = 2 kk
            T2* Lm = (T2*)(ws + Ly.lr);
            T2* Rm = Lm + (size_t)2 * NB * n;
            const size_t blk = (size_t)m * kk * sizeof(T2);
            for (auto cp : {std::make_pair(Lm, (const T2*)Vj), std::make_pair(Lm + (size_t)m * kk, (const T2*)Xbuf),
                            std::make_pair(Rm, (const T2*)Xbuf), std::make_pair(Rm + (size_t)m * kk, (const T2*)Vj)})
                if ((st = cuda_check(c, cudaMemcpyAsync(cp.first, cp.second, blk, cudaMemcpyDeviceToDevice, c->stream), "update operands"))) return st;
            if ((st = blas_check(c, cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_C, m, m, 2 * kk, &mone, Lm, CUDA_C_32F, m, Rm, CUDA_C_32F, m,
                                                 &one, A22, CUDA_C_32F, (int)lda, ctype, CUBLAS_GEMM_DEFAULT), "update gemm"))) return st;
        } else {
            if ((st = blas_check(c, xher2k(h, m, kk, &mone, Vj, m, Xbuf, m, &rone, A22, (int)lda), "her2k"))) return st;
        }
    }
    cublasSetMathMode(c->cublas, math_prev);
    cublasSetEmulationStrategy(c->cublas, emu_prev);
    stage_end(c, 13);
    // band -> tridiagonal
    stage_begin(c, 14);
    T2* AB = (T2*)(ws + Ly.ab);
    int* prog = (int*)(ws + Ly.prog);
    band_extract_kernel<T2><<<(unsigned)(((int64_t)LDB * n + 255) / 256), 256, 0, c->stream>>>(n, A, lda, AB);
    c->launches++;
    if ((st = cuda_check(c, cudaMemsetAsync(prog, 0, (size_t)n * sizeof(int), c->stream), "chase progress"))) return st;
    if (n >= 2) {
        ChaseArgs<T2> ca;
        ca.n = n; ca.AB = AB; ca.y = y; ca.V2 = keep_q ? (T2*)(ws + Ly.v2) : nullptr; ca.prog = prog; ca.err = err;
        int per_sm = 0;
        if ((st = cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chase_kernel<T2>, kChaseThreads, 0), "chase occupancy"))) return st;
        int G = std::max(1, std::min(n - 1, nsm * std::min(per_sm, 2)));
        if (const char* v = std::getenv("BSE_CHASE_BLOCKS")) G = std::max(1, std::min(G, std::atoi(v)));
        void* kargs[] = {&ca};
        if ((st = cuda_check(c, cudaLaunchCooperativeKernel((void*)chase_kernel<T2>, dim3(G), dim3(kChaseThreads), kargs, 0,
                                                            c->stream), "bulge chase launch"))) return st;
        c->launches++;
    }
    band_diag_kernel<T2, R><<<(n + 255) / 256, 256, 0, c->stream>>>(n, AB, d, e);
    c->launches++;
    stage_end(c, 14);
    return cuda_check(c, cudaGetLastError(), "two-stage reduction");
}

template <typename T2>
int band_backtransform_t(bse_ctx* c, int n, const typename Real<T2>::t* z, int n_vec, T2* X, char* ws, unsigned* bar,
                         int* err) {
    int st;
    const int nsm = device_sms(c);
    const Layout Ly = layout(n, sizeof(T2), true, nsm, n_vec);
    T2* Zrm = (T2*)(ws + Ly.zrm);
    // Z (real, n x n_vec column-major) -> row-major complex
    {
        dim3 blk(32, 8), grd((n + 31) / 32, (n_vec + 31) / 32);
        transpose_kernel<typename Real<T2>::t, T2><<<grd, blk, 0, c->stream>>>(n, n_vec, z, n, Zrm, n_vec);
        c->launches++;
    }
    if (n >= 2) {
        int per_sm = 0;
        if ((st = cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, apply_q2_kernel<T2>, kQ2Threads, 0), "q2 occupancy"))) return st;
        const int G = nsm * std::max(1, std::min(per_sm, 1));
        const T2* V2 = (const T2*)(ws + Ly.v2);
        unsigned* flags = (unsigned*)(ws + Ly.flags);
        if ((st = cuda_check(c, cudaMemsetAsync(flags, 0, (size_t)Ly.gmax * 128, c->stream), "barrier flags"))) return st;
        void* kargs[] = {(void*)&n, (void*)&V2, (void*)&Zrm, (void*)&n_vec, (void*)&flags, (void*)&err};
        if ((st = cuda_check(c, cudaLaunchCooperativeKernel((void*)apply_q2_kernel<T2>, dim3(G), dim3(kQ2Threads), kargs, 0,
                                                            c->stream), "Q2 launch"))) return st;
        c->launches++;
    }
    {
        dim3 blk(32, 8), grd((n_vec + 31) / 32, (n + 31) / 32);
        transpose_kernel<T2, T2><<<grd, blk, 0, c->stream>>>(n_vec, n, Zrm, n_vec, X, n);
        c->launches++;
    }
    // X <- Q1 X, panels from last to first: X[r0:] -= V (T (V^H X[r0:]))
    if ((st = blas_check(c, cublasSetStream(c->cublas, c->stream), "stream"))) return st;
    const T2* Vall = (const T2*)(ws + Ly.vall);
    const T2* Tall = (const T2*)(ws + Ly.tall);
    T2* W1 = (T2*)(ws + Ly.small) + 2 * NB * NB;
    T2* W2 = W1 + (size_t)NB * n_vec;
    const T2 one = C2h<T2>(1, 0), zero = C2h<T2>(0, 0), mone = C2h<T2>(-1, 0);
    int64_t voff = Ly.vsize;
    for (int j = Ly.npanel - 1; j >= 0; j--) {
        const int r0 = (j + 1) * NB, m = n - r0, kk = std::min(NB, m);
        voff -= (int64_t)m * kk;
        const T2* Vj = Vall + voff;
        const T2* Tj = Tall + (size_t)j * NB * NB;
        cublasHandle_t h = c->cublas;
        if ((st = blas_check(c, xgemm(h, CUBLAS_OP_C, CUBLAS_OP_N, kk, n_vec, m, &one, Vj, m, X + r0, n, &zero, W1, NB), "gemm V^H X"))) return st;
        if ((st = blas_check(c, xtrmm(h, CUBLAS_SIDE_LEFT, CUBLAS_OP_N, kk, n_vec, &one, Tj, NB, W1, NB, W2, NB), "trmm T"))) return st;
        if ((st = blas_check(c, xgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n_vec, kk, &mone, Vj, m, W2, NB, &one, X + r0, n), "gemm X"))) return st;
    }
    return cuda_check(c, cudaGetLastError(), "two-stage back-transformation");
}

}  // namespace

size_t band_workspace(int n, bool fp64, bool keep_q, int n_vec, int nsm) {
    return layout(n, fp64 ? sizeof(double2) : sizeof(float2), keep_q, nsm, n_vec).total;
}

int band_tridiag(bse_ctx* c, int n, void* A, int64_t lda, bool fp64, void* d, void* e, void* y, bool keep_q, char* ws,
                 unsigned* bar, int* err, int n_vec) {
    if (fp64) return band_tridiag_t<double2>(c, n, (double2*)A, lda, (double*)d, (double*)e, (double2*)y, keep_q, ws, bar, err, n_vec);
    return band_tridiag_t<float2>(c, n, (float2*)A, lda, (float*)d, (float*)e, (float2*)y, keep_q, ws, bar, err, n_vec);
}

int band_backtransform(bse_ctx* c, int n, bool fp64, const void* z, int n_vec, void* X, char* ws, unsigned* bar, int* err) {
    if (fp64) return band_backtransform_t<double2>(c, n, (const double*)z, n_vec, (double2*)X, ws, bar, err);
    return band_backtransform_t<float2>(c, n, (const float*)z, n_vec, (float2*)X, ws, bar, err);
}

}  // namespace bse
