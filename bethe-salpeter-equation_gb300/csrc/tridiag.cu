// This library's dense Hermitian eigensolver (BSE_EIG_OWN).
//
// Replaces the eig_sym (LAPACK zheevd) call of common_diagonalization
// (bse.version13.cpp:3195, 3330) with a solver shaped for what the BSE path needs:
//
//  1. tridiag_kernel: Householder reduction Q^H A Q = T (T real symmetric tridiagonal, the
//     zhetd2 algorithm, lower reflectors).  One cooperative persistent kernel: for every
//     reflector k, each block recomputes column k with the pending rank-2 update and the
//     reflector (redundantly, no barrier), then one fused pass over the trailing matrix
//     applies the pending update A -= v w^H + w v^H and accumulates p = tau A v for the new
//     reflector; two grid barriers per reflector finish p and the scalar of w.  The same
//     pass applies Q^H to the optical pair-density vector (y = Q^H rho), so oscillator
//     strengths never need the eigenvectors of A: f_l = y^H z_l with z_l real.
//  2. bisect_kernel: eigenvalues of T by Sturm-count bisection, one thread per eigenvalue;
//     an FP32 bracket first, then FP64 bisection to full precision.
//  3. invit_kernel: eigenvectors z_l of T by inverse iteration (FP64 LU with partial
//     pivoting, dlagtf/dlagts style), one thread per eigenvalue, giving f_l on the fly.
//  4. apply_q_kernel: X = Q Z only for the eigenvectors that are asked for (the FP64
//     refinement subspace, or all of them when the caller wants A).
// Every wait on another block is bounded: a barrier that times out sets an error word and
// the kernel returns; the host reports BSE_ERR_NOT_CONVERGED.
#include <cooperative_groups.h>

#include "bse_internal.h"

namespace bse {
namespace {

template <typename T2> struct Real;
template <> struct Real<float2> { typedef float t; };
template <> struct Real<double2> { typedef double t; };

template <typename T2> __device__ __forceinline__ T2 C2(typename Real<T2>::t x, typename Real<T2>::t y) {
    T2 r; r.x = x; r.y = y; return r;
}
template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { return C2<T2>(a.x + b.x, a.y + b.y); }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { return C2<T2>(a.x - b.x, a.y - b.y); }
template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
    return C2<T2>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T2> __device__ __forceinline__ T2 cmulc(T2 a, T2 b) {
    return C2<T2>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// conj(a) * b
template <typename T2> __device__ __forceinline__ T2 cconjmul(T2 a, T2 b) {
    return C2<T2>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename T2> __device__ __forceinline__ T2 cinv(T2 a) {
    typedef typename Real<T2>::t R;
    R s = a.x * a.x + a.y * a.y;
    return C2<T2>(a.x / s, -a.y / s);
}

constexpr unsigned kSpinLimit = 1u << 26;   // ~seconds of polling before a barrier gives up

// Grid-wide barrier for a cooperative launch.  bar[0] arrivals, bar[1] generation.
// Returns false (after setting *err) if a block did not arrive in time or another block failed.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        volatile int* verr = err;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned it = 0;
            while (*vgen == gen) {
                if (*verr != 0) break;
                if (++it > kSpinLimit) { atomicExch(err, 1); break; }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)err == 0;
}

template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of a real value; every thread gets the result.  `red` holds >= 32 R.
template <typename R>
__device__ __forceinline__ R block_sum(R v, R* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    R t = lane < nw ? red[lane] : R(0);
    t = warp_sum(t);
    return t;
}

template <typename T2>
struct TriArgs {
    int n;
    T2* A;
    int64_t lda;
    typename Real<T2>::t* d;   // n
    typename Real<T2>::t* e;   // n-1
    T2* tau;                   // n-1
    T2* vbuf;                  // [2][n] reflectors (v[k+1] = 1)
    T2* pbuf;                  // [2][n] p = tau A v
    T2* ppart;                 // [nt][n] column partial sums of the fused pass
    T2* dpart;                 // [2][gridDim] block partial dots
    T2* y;                     // n: Q^H applied in place (may be null)
    unsigned* bar;
    int* err;
    int TR;                    // rows per tile
};

// Householder tridiagonalization (lower), full Hermitian storage.  See the file comment.
template <typename T2>
__global__ void __launch_bounds__(512, 1) tridiag_kernel(TriArgs<T2> a) {
    typedef typename Real<T2>::t R;
    extern __shared__ unsigned char smraw[];
    T2* sv = reinterpret_cast<T2*>(smraw);          // pending v (tile rows)
    T2* sw = sv + a.TR;                             // pending w (tile rows)
    T2* sv1 = sw + a.TR;                            // new reflector (tile rows)
    R* red = reinterpret_cast<R*>(sv1 + a.TR);      // 64 R for reductions
    const int n = a.n, tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int nwarp = nthr >> 5, B = gridDim.x, b = blockIdx.x;
    const int64_t lda = a.lda;
    T2* A = a.A;
    T2 alpha_prev = C2<T2>(0, 0);
    bool have_prev = false;
    const T2 zero = C2<T2>(0, 0);

    for (int k = 0; k <= n - 2; k++) {
        const T2* vp = a.vbuf + (size_t)((k + 1) & 1) * n;   // v_{k-1}
        const T2* pp = a.pbuf + (size_t)((k + 1) & 1) * n;   // p_{k-1}
        T2* vk = a.vbuf + (size_t)(k & 1) * n;
        T2* pk = a.pbuf + (size_t)(k & 1) * n;
        auto wprev = [&](int r) -> T2 { return cadd(pp[r], cmul(alpha_prev, vp[r])); };
        // pending update of an element of column k (row r): a - v_r conj(w_k) - w_r conj(v_k)
        T2 vkk = have_prev ? vp[k] : zero, wkk = have_prev ? wprev(k) : zero;
        auto upd_colk = [&](int r) -> T2 {
            T2 x = A[r + (int64_t)k * lda];
            if (have_prev) x = csub(csub(x, cmulc(vp[r], wkk)), cmulc(wprev(r), vkk));
            return x;
        };
        // ---- phase A: reflector of column k (every block, redundantly) ----
        R loc = 0;
        for (int r = k + 2 + tid; r < n; r += nthr) {
            T2 x = upd_colk(r);
            loc += x.x * x.x + x.y * x.y;
        }
        const R xnorm2 = block_sum(loc, red);
        const T2 alpha = upd_colk(k + 1);
        const R dk = upd_colk(k).x;
        T2 tauk;
        R beta;
        T2 scal;
        if (xnorm2 == R(0) && alpha.y == R(0)) {
            tauk = zero;
            beta = alpha.x;
            scal = zero;
        } else {
            beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2), alpha.x);
            tauk = C2<T2>((beta - alpha.x) / beta, -alpha.y / beta);
            scal = cinv(csub(alpha, C2<T2>(beta, 0)));
        }
        if (b == 0) {
            for (int r = k + 1 + tid; r < n; r += nthr) vk[r] = (r == k + 1) ? C2<T2>(1, 0) : cmul(upd_colk(r), scal);
            if (tid == 0) {
                a.d[k] = dk;
                a.e[k] = beta;
                a.tau[k] = tauk;
            }
        }
        // ---- phase B: pending rank-2 update of A[k+1:, k+1:] and column sums of A_new^H v_k ----
        const int m = n - (k + 1);
        const int nt = (m + a.TR - 1) / a.TR;
        const int64_t items = (int64_t)nt * m;
        const int64_t lo = items * b / B, hi = items * (b + 1) / B;
        for (int t = (int)(lo / m); t < nt && (int64_t)t * m < hi; t++) {
            const int r0 = k + 1 + t * a.TR, r1 = min(n, r0 + a.TR);
            __syncthreads();
            for (int r = r0 + tid; r < r1; r += nthr) {
                sv[r - r0] = have_prev ? vp[r] : zero;
                sw[r - r0] = have_prev ? wprev(r) : zero;
                sv1[r - r0] = (r == k + 1) ? C2<T2>(1, 0) : cmul(upd_colk(r), scal);
            }
            __syncthreads();
            const int64_t i0 = max(lo, (int64_t)t * m), i1 = min(hi, (int64_t)(t + 1) * m);
            for (int64_t it = i0 + warp; it < i1; it += nwarp) {
                const int c = k + 1 + (int)(it - (int64_t)t * m);
                const T2 vc = have_prev ? vp[c] : zero;
                const T2 wc = have_prev ? wprev(c) : zero;
                T2* col = A + (int64_t)c * lda;
                R accx = 0, accy = 0;
                for (int r = r0 + lane; r < r1; r += 32) {
                    T2 x = col[r];
                    if (have_prev) {
                        x = csub(csub(x, cmulc(sv[r - r0], wc)), cmulc(sw[r - r0], vc));
                        col[r] = x;
                    }
                    const T2 q = cconjmul(x, sv1[r - r0]);
                    accx += q.x;
                    accy += q.y;
                }
                accx = warp_sum(accx);
                accy = warp_sum(accy);
                if (lane == 0) a.ppart[(size_t)t * n + c] = C2<T2>(accx, accy);
            }
        }
        if (!grid_barrier(a.bar, a.err)) return;
        // ---- phase C1: p_c = tau * sum_t ppart, partial p^H v and v^H y per block ----
        {
            R dx = 0, dy = 0, yx = 0, yy = 0;
            for (int c = k + 1 + b * nthr + tid; c < n; c += B * nthr) {
                T2 s = zero;
                for (int t = 0; t < nt; t++) s = cadd(s, a.ppart[(size_t)t * n + c]);
                const T2 p = cmul(tauk, s);
                pk[c] = p;
                const T2 v = vk[c];
                const T2 q = cconjmul(p, v);
                dx += q.x;
                dy += q.y;
                if (a.y) {
                    const T2 u = cconjmul(v, a.y[c]);
                    yx += u.x;
                    yy += u.y;
                }
            }
            dx = block_sum(dx, red);
            dy = block_sum(dy, red);
            if (a.y) {
                yx = block_sum(yx, red);
                yy = block_sum(yy, red);
            }
            if (tid == 0) {
                a.dpart[b] = C2<T2>(dx, dy);
                a.dpart[B + b] = C2<T2>(yx, yy);
            }
        }
        if (!grid_barrier(a.bar, a.err)) return;
        // ---- phase C2: alpha_k, y <- H_k^H y on this block's slice, reflector storage ----
        {
            T2 s = zero, sy = zero;
            for (int i = 0; i < B; i++) {
                s = cadd(s, a.dpart[i]);
                sy = cadd(sy, a.dpart[B + i]);
            }
            alpha_prev = cmul(C2<T2>(-0.5 * tauk.x, -0.5 * tauk.y), s);
            have_prev = true;
            if (a.y) {
                // y -= conj(tau) (v^H y) v  on the same column slice as C1 (next C1 reads it after a barrier)
                const T2 coef = cmulc(sy, tauk);   // conj(tau) * (v^H y)
                for (int c = k + 1 + b * nthr + tid; c < n; c += B * nthr) a.y[c] = csub(a.y[c], cmul(coef, vk[c]));
            }
            if (b == 0)
                for (int r = k + 2 + tid; r < n; r += nthr) A[r + (int64_t)k * lda] = vk[r];
        }
    }
    if (b == 0 && tid == 0) {
        if (n >= 2) {
            const T2* vp = a.vbuf + (size_t)((n - 2) & 1) * n;
            const T2* pp = a.pbuf + (size_t)((n - 2) & 1) * n;
            const T2 v = vp[n - 1], w = cadd(pp[n - 1], cmul(alpha_prev, vp[n - 1]));
            T2 x = A[(n - 1) + (int64_t)(n - 1) * lda];
            x = csub(csub(x, cmulc(v, w)), cmulc(w, v));
            a.d[n - 1] = x.x;
        } else {
            a.d[0] = A[0].x;
        }
    }
}

// Sturm count: number of eigenvalues of T (diag d, squared off-diagonal e2) that are <= x.
template <typename R>
__device__ __forceinline__ int sturm(int n, const R* __restrict__ d, const R* __restrict__ e2, R x, R pivmin) {
    R q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    int c = q <= R(0);
    for (int j = 1; j < n; j++) {
        q = d[j] - e2[j - 1] / q - x;
        if (fabs(q) < pivmin) q = -pivmin;
        c += q <= R(0);
    }
    return c;
}

// i-th smallest eigenvalue of T: FP32 bisection to a bracket, verified and finished in FP64.
__global__ void __launch_bounds__(128) bisect_kernel(int n, const double* __restrict__ d, const double* __restrict__ e2,
                                                     const float* __restrict__ df, const float* __restrict__ e2f,
                                                     double glo, double ghi, double pivmin, float pivminf,
                                                     double* __restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double tnorm = fmax(fabs(glo), fabs(ghi));
    float a = (float)glo, b = (float)ghi;
    for (int it = 0; it < 22; it++) {
        const float mid = 0.5f * (a + b);
        if (sturm<float>(n, df, e2f, mid, pivminf) > i) b = mid;
        else a = mid;
    }
    const double margin = 64.0 * 1.1920929e-7 * (tnorm + fabs((double)a) + fabs((double)b));
    double lo = (double)a - margin, hi = (double)b + margin;
    if (!(sturm<double>(n, d, e2, lo, pivmin) <= i && sturm<double>(n, d, e2, hi, pivmin) > i)) {
        lo = glo;
        hi = ghi;
    }
    for (int it = 0; it < 100; it++) {
        const double mid = 0.5 * (lo + hi);
        if (hi - lo <= 4.0 * 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)) + 2.0 * pivmin || mid <= lo || mid >= hi) break;
        if (sturm<double>(n, d, e2, mid, pivmin) > i) hi = mid;
        else lo = mid;
    }
    w[i] = 0.5 * (lo + hi);
}

__device__ __forceinline__ double start_value(unsigned i, unsigned k) {
    unsigned h = i * 0x9E3779B9u ^ (k + 0x7F4A7C15u) * 0x85EBCA6Bu;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return 0.5 + (double)(h & 0xFFFFFF) / (double)0x1000000;   // (0.5, 1.5)
}

// Eigenvector of T for eigenvalue w[i] by inverse iteration; f_i = sum_k conj(y_k) z_k.
// Scratch is interleaved ([k][count]) so the threads of a warp touch consecutive words.
template <typename TZ>
__global__ void __launch_bounds__(128) invit_kernel(int n, const double* __restrict__ d, const double* __restrict__ e,
                                                    const double* __restrict__ w, int i0, int count, double tnorm,
                                                    const double2* __restrict__ y, double2* __restrict__ f,
                                                    TZ* __restrict__ z, int64_t ldz, int n_store,
                                                    double* __restrict__ scr, signed char* __restrict__ piv) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int i = i0 + t;
    const double lam = w[i];
    const size_t S = (size_t)count;
    double* Ua = scr;                  // pivots (diagonal of U)
    double* Ub = scr + (size_t)n * S;  // first superdiagonal of U
    double* Ud = scr + 2 * (size_t)n * S;   // second superdiagonal of U (fill-in)
    double* Lc = scr + 3 * (size_t)n * S;   // multipliers
    double* Y = scr + 4 * (size_t)n * S;    // iterate
    const double pert = 2.220446049250313e-16 * fmax(tnorm, 1e-300);
    // LU of T - lam I with partial pivoting (dlagtf)
    double ak = d[0] - lam;
    double bk = n > 1 ? e[0] : 0.0;      // super of the current pivot row
    for (int k = 0; k < n - 1; k++) {
        const double ck = e[k];            // sub-diagonal entry below the pivot
        const double anext = d[k + 1] - lam;
        const double bnext = (k + 1 < n - 1) ? e[k + 1] : 0.0;
        if (fabs(ck) <= fabs(ak)) {
            const double mult = ak != 0.0 ? ck / ak : 0.0;
            Ua[k * S + t] = ak;
            Ub[k * S + t] = bk;
            Ud[k * S + t] = 0.0;
            Lc[k * S + t] = mult;
            piv[k * S + t] = 0;
            ak = anext - mult * bk;
            bk = bnext;
        } else {
            const double mult = ak / ck;
            Ua[k * S + t] = ck;
            Ub[k * S + t] = anext;
            Ud[k * S + t] = bnext;
            Lc[k * S + t] = mult;
            piv[k * S + t] = 1;
            ak = bk - mult * anext;
            bk = -mult * bnext;
        }
    }
    Ua[(size_t)(n - 1) * S + t] = ak;
    for (int k = 0; k < n; k++) Y[k * S + t] = start_value(i, k);
    for (int iter = 0; iter < 3; iter++) {
        // forward: apply L (with interchanges)
        for (int k = 0; k < n - 1; k++) {
            const double mult = Lc[k * S + t];
            const double y0 = Y[k * S + t], y1 = Y[(k + 1) * S + t];
            if (piv[k * S + t] == 0) {
                Y[(k + 1) * S + t] = y1 - mult * y0;
            } else {
                Y[k * S + t] = y1;
                Y[(k + 1) * S + t] = y0 - mult * y1;
            }
        }
        // back substitution with U (zero pivots perturbed)
        double x1 = 0.0, x2 = 0.0, mx = 0.0;
        for (int k = n - 1; k >= 0; k--) {
            double u = Ua[k * S + t];
            if (fabs(u) < pert) u = u < 0 ? -pert : pert;
            const double x = (Y[k * S + t] - Ub[k * S + t] * x1 - Ud[k * S + t] * x2) / u;
            Y[k * S + t] = x;
            x2 = x1;
            x1 = x;
            mx = fmax(mx, fabs(x));
        }
        const double sc = mx > 0 ? 1.0 / mx : 1.0;
        for (int k = 0; k < n; k++) Y[k * S + t] *= sc;
    }
    double nrm = 0.0, fx = 0.0, fy = 0.0;
    for (int k = 0; k < n; k++) {
        const double v = Y[k * S + t];
        nrm += v * v;
        if (y) {
            const double2 yy = y[k];
            fx += yy.x * v;
            fy -= yy.y * v;
        }
    }
    const double inv = 1.0 / sqrt(nrm);
    if (f) f[i] = make_double2(fx * inv, fy * inv);
    if (i < n_store)
        for (int k = 0; k < n; k++) z[(size_t)k + (size_t)i * ldz] = (TZ)(Y[k * S + t] * inv);
}

// X[:, c] <- Q X[:, c] (adjoint = false: H_{n-2} first ... H_0 last) or Q^H X (adjoint = true).
// One block per group of CB columns; reflector k has v[k+1] = 1, v[r] = A[r, k] for r >= k+2.
template <typename T2, int CB>
__global__ void __launch_bounds__(256) apply_q_kernel(int n, const T2* __restrict__ A, int64_t lda,
                                                      const T2* __restrict__ tau, T2* __restrict__ X, int64_t ldx,
                                                      int ncols, bool adjoint) {
    typedef typename Real<T2>::t R;
    __shared__ R red[2 * CB][32];
    __shared__ T2 coef[CB];
    const int c0 = blockIdx.x * CB, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    for (int s = 0; s < n - 1; s++) {
        const int k = adjoint ? s : (n - 2 - s);
        const T2 tk = tau[k];
        if (tk.x == R(0) && tk.y == R(0)) continue;
        R px[CB], py[CB];
#pragma unroll
        for (int j = 0; j < CB; j++) px[j] = py[j] = 0;
        for (int r = k + 1 + tid; r < n; r += blockDim.x) {
            const T2 v = (r == k + 1) ? C2<T2>(1, 0) : A[r + (int64_t)k * lda];
#pragma unroll
            for (int j = 0; j < CB; j++)
                if (c0 + j < ncols) {
                    const T2 q = cconjmul(v, X[r + (int64_t)(c0 + j) * ldx]);
                    px[j] += q.x;
                    py[j] += q.y;
                }
        }
#pragma unroll
        for (int j = 0; j < CB; j++) {
            px[j] = warp_sum(px[j]);
            py[j] = warp_sum(py[j]);
        }
        if (lane == 0)
            for (int j = 0; j < CB; j++) {
                red[2 * j][warp] = px[j];
                red[2 * j + 1][warp] = py[j];
            }
        __syncthreads();
        if (tid < CB) {
            R sx = 0, sy = 0;
            for (int w = 0; w < nwarp; w++) {
                sx += red[2 * tid][w];
                sy += red[2 * tid + 1][w];
            }
            const T2 tt = adjoint ? C2<T2>(tk.x, -tk.y) : tk;
            coef[tid] = cmul(tt, C2<T2>(sx, sy));
        }
        __syncthreads();
        for (int r = k + 1 + tid; r < n; r += blockDim.x) {
            const T2 v = (r == k + 1) ? C2<T2>(1, 0) : A[r + (int64_t)k * lda];
#pragma unroll
            for (int j = 0; j < CB; j++)
                if (c0 + j < ncols) {
                    T2* xp = X + r + (int64_t)(c0 + j) * ldx;
                    *xp = csub(*xp, cmul(coef[j], v));
                }
        }
        __syncthreads();
    }
}

template <typename T2>
__global__ void real_to_complex_kernel(int64_t n, const typename Real<T2>::t* __restrict__ in, T2* __restrict__ out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) out[t] = C2<T2>(in[t], 0);
}

template <typename R>
__global__ void tri_prepare_kernel(int n, const R* __restrict__ d, const R* __restrict__ e, double* __restrict__ dd,
                                   double* __restrict__ ee, double* __restrict__ e2, float* __restrict__ df,
                                   float* __restrict__ e2f) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        dd[t] = (double)d[t];
        df[t] = (float)d[t];
    }
    if (t < n - 1) {
        const double x = (double)e[t];
        ee[t] = x;
        e2[t] = x * x;
        e2f[t] = (float)(x * x);
    }
}

template <typename T2>
__global__ void rho_to_y_kernel(int n, const double2* __restrict__ rho, T2* __restrict__ y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) y[t] = C2<T2>((typename Real<T2>::t)rho[t].x, (typename Real<T2>::t)rho[t].y);
}
template <typename T2>
__global__ void y_to_double_kernel(int n, const T2* __restrict__ y, double2* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = make_double2((double)y[t].x, (double)y[t].y);
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

template <typename T2>
int own_heevd_t(bse_ctx* c, int n, T2* A, int64_t lda, double* dW, int n_vec, const double2* rho0, double2* f_out) {
    typedef typename Real<T2>::t R;
    int st;
    int dev = c->device, nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 512;
    const int TR = 1024;
    const size_t smem = 3 * (size_t)TR * sizeof(T2) + 64 * sizeof(R);
    int per_sm = 0;
    if ((st = cuda_check(c, cudaFuncSetAttribute(tridiag_kernel<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "tridiag smem"))) return st;
    if ((st = cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tridiag_kernel<T2>, threads, smem), "occupancy"))) return st;
    if (per_sm < 1) return fail(c, BSE_ERR_CUDA, "tridiagonal kernel does not fit on an SM");
    const int B = nsm;   // one block per SM: cheapest barrier, 16 warps of loads in flight per SM
    const int nt_max = (n + TR - 1) / TR;
    const int count_max = std::min(n, 8192);
    // workspace
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    const size_t o_d = carve(n * sizeof(R)), o_e = carve(n * sizeof(R)), o_tau = carve(n * sizeof(T2));
    const size_t o_v = carve(2 * (size_t)n * sizeof(T2)), o_p = carve(2 * (size_t)n * sizeof(T2));
    const size_t o_pp = carve((size_t)nt_max * n * sizeof(T2)), o_dp = carve(2 * (size_t)B * sizeof(T2));
    const size_t o_y = carve(n * sizeof(T2)), o_bar = carve(64);
    const size_t o_dd = carve(n * 8), o_ee = carve(n * 8), o_e2 = carve(n * 8), o_df = carve(n * 4), o_e2f = carve(n * 4);
    const size_t o_y64 = carve(n * sizeof(double2));
    const size_t o_scr = carve(5 * (size_t)n * count_max * 8), o_piv = carve((size_t)n * count_max);
    const size_t o_z = carve((size_t)n * std::max(n_vec, 1) * sizeof(R));
    if ((st = ensure_work(c, off))) return st;
    char* w = (char*)c->d_work;
    R* d = (R*)(w + o_d);
    R* e = (R*)(w + o_e);
    T2* tau = (T2*)(w + o_tau);
    T2* y = rho0 ? (T2*)(w + o_y) : nullptr;
    unsigned* bar = (unsigned*)(w + o_bar);
    int* err = (int*)(w + o_bar + 16);
    if ((st = cuda_check(c, cudaMemsetAsync(bar, 0, 64, c->stream), "barrier reset"))) return st;
    if ((st = cuda_check(c, cudaMemsetAsync(w + o_v, 0, 2 * (size_t)n * sizeof(T2), c->stream), "v reset"))) return st;
    if ((st = cuda_check(c, cudaMemsetAsync(w + o_p, 0, 2 * (size_t)n * sizeof(T2), c->stream), "p reset"))) return st;
    if ((st = cuda_check(c, cudaMemsetAsync(tau, 0, n * sizeof(T2), c->stream), "tau reset"))) return st;
    if (y) {
        rho_to_y_kernel<T2><<<(n + 255) / 256, 256, 0, c->stream>>>(n, rho0, y);
        c->launches++;
    }
    TriArgs<T2> ta;
    ta.n = n; ta.A = A; ta.lda = lda; ta.d = d; ta.e = e; ta.tau = tau;
    ta.vbuf = (T2*)(w + o_v); ta.pbuf = (T2*)(w + o_p); ta.ppart = (T2*)(w + o_pp); ta.dpart = (T2*)(w + o_dp);
    ta.y = y; ta.bar = bar; ta.err = err; ta.TR = TR;
    void* kargs[] = {&ta};
    if ((st = cuda_check(c, cudaLaunchCooperativeKernel((void*)tridiag_kernel<T2>, dim3(B), dim3(threads), kargs, smem, c->stream),
                         "tridiagonal kernel launch"))) return st;
    c->launches++;
    // T in FP64 / FP32 copies for the bisection and inverse iteration
    double* dd = (double*)(w + o_dd);
    double* ee = (double*)(w + o_ee);
    double* e2 = (double*)(w + o_e2);
    float* df = (float*)(w + o_df);
    float* e2f = (float*)(w + o_e2f);
    tri_prepare_kernel<R><<<(n + 255) / 256, 256, 0, c->stream>>>(n, d, e, dd, ee, e2, df, e2f);
    c->launches++;
    int herr = 0;
    std::vector<double> hd(n), he(n > 1 ? n - 1 : 1);
    if ((st = cuda_check(c, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "barrier status"))) return st;
    if ((st = cuda_check(c, cudaMemcpyAsync(hd.data(), dd, n * 8, cudaMemcpyDeviceToHost, c->stream), "d"))) return st;
    if (n > 1 && (st = cuda_check(c, cudaMemcpyAsync(he.data(), ee, (n - 1) * 8, cudaMemcpyDeviceToHost, c->stream), "e"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "tridiagonal reduction"))) return st;
    if (herr) return fail(c, BSE_ERR_NOT_CONVERGED, "tridiagonal reduction: a grid barrier timed out");
    // Gershgorin interval and pivmin (host: O(n))
    double glo = 1e300, ghi = -1e300, emax2 = 0;
    for (int i = 0; i < n; i++) {
        const double r = (i > 0 ? std::fabs(he[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(he[i]) : 0.0);
        glo = std::min(glo, hd[i] - r);
        ghi = std::max(ghi, hd[i] + r);
        if (i < n - 1) emax2 = std::max(emax2, he[i] * he[i]);
    }
    if (!std::isfinite(glo) || !std::isfinite(ghi)) return fail(c, BSE_ERR_NOT_CONVERGED, "tridiagonal reduction produced non-finite values");
    const double tnorm = std::max(std::fabs(glo), std::fabs(ghi));
    glo -= 2.220446049250313e-16 * tnorm * n + 1e-300;
    ghi += 2.220446049250313e-16 * tnorm * n + 1e-300;
    const double pivmin = 2.2250738585072014e-308 * std::max(1.0, emax2);
    const float pivminf = 1.17549435e-38f * (float)std::max(1.0, emax2);
    bisect_kernel<<<(n + 127) / 128, 128, 0, c->stream>>>(n, dd, e2, df, e2f, glo, ghi, pivmin, pivminf, dW);
    c->launches++;
    double2* y64 = nullptr;
    if (y) {
        y64 = (double2*)(w + o_y64);
        y_to_double_kernel<T2><<<(n + 255) / 256, 256, 0, c->stream>>>(n, y, y64);
        c->launches++;
    }
    R* z = (R*)(w + o_z);
    for (int i0 = 0; i0 < n; i0 += count_max) {
        const int cnt = std::min(count_max, n - i0);
        if (i0 >= n_vec && !f_out) break;
        invit_kernel<R><<<(cnt + 127) / 128, 128, 0, c->stream>>>(n, dd, ee, dW, i0, cnt, tnorm, y64, f_out, z, n, n_vec,
                                                                   (double*)(w + o_scr), (signed char*)(w + o_piv));
        c->launches++;
    }
    if ((st = cuda_check(c, cudaGetLastError(), "bisection / inverse iteration"))) return st;
    if (n_vec > 0) {
        // X = Q Z for the first n_vec eigenvectors; X is built in a separate buffer because A holds Q
        T2* X = nullptr;
        if ((st = cuda_check(c, cudaMallocAsync((void**)&X, (size_t)n * n_vec * sizeof(T2), c->stream), "eigenvector buffer"))) return st;
        const int64_t nz = (int64_t)n * n_vec;
        real_to_complex_kernel<T2><<<(unsigned)((nz + 255) / 256), 256, 0, c->stream>>>(nz, z, X);
        c->launches++;
        constexpr int CB = 8;
        apply_q_kernel<T2, CB><<<(n_vec + CB - 1) / CB, 256, 0, c->stream>>>(n, A, lda, tau, X, n, n_vec, false);
        c->launches++;
        st = cuda_check(c, cudaMemcpy2DAsync(A, lda * sizeof(T2), X, n * sizeof(T2), n * sizeof(T2), n_vec,
                                             cudaMemcpyDeviceToDevice, c->stream), "eigenvectors");
        cudaFreeAsync(X, c->stream);
        if (st) return st;
    }
    return cuda_check(c, cudaGetLastError(), "own eigensolver");
}

}  // namespace

int own_heevd(bse_ctx* c, int n, void* dA, int lda, bool fp64, double* dW, int n_vec, const double2* rho0, double2* f_out) {
    if (fp64) return own_heevd_t<double2>(c, n, (double2*)dA, lda, dW, n_vec, rho0, f_out);
    return own_heevd_t<float2>(c, n, (float2*)dA, lda, dW, n_vec, rho0, f_out);
}

}  // namespace bse
