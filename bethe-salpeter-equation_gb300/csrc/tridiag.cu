// This library's dense Hermitian eigensolver (BSE_EIG_OWN).
//
// Replaces the eig_sym (LAPACK zheevd) call of common_diagonalization
// (bse.version13.cpp:3195, 3330) with a solver shaped for what the BSE path needs:
//
//  1. tridiag_fused_kernel (tridiag_kernel where its vectors do not fit in shared memory):
//     Householder reduction Q^H A Q = T (T real symmetric tridiagonal, the zhetd2 algorithm,
//     lower reflectors).  One cooperative persistent kernel: for every reflector k, each block
//     recomputes column k with the pending rank-2 update and the reflector (redundantly, no
//     barrier), then one fused pass over the trailing matrix applies the pending update
//     A -= v w^H + w v^H and accumulates p = tau A v for the new reflector; one barrier per
//     reflector.  The same steps apply Q^H to the optical pair-density vector (y = Q^H rho), so
//     oscillator strengths never need the eigenvectors of A: f_l = y^H z_l with z_l real.
//  2. bisect32_kernel: eigenvalues of T by FP32 Sturm-count multisection (several lanes per
//     eigenvalue when the problem is small); runs of eigenvalues FP32 cannot separate form
//     clusters (FP64 division is slow on this part, so no FP64 bisection).
//  3. invit_kernel: eigenvectors z_l of T by inverse iteration (LU with partial pivoting,
//     dlagtf/dlagts style): three FP32 iterations (operands staged through shared memory), then
//     in the FP64 path two FP64 Rayleigh-quotient iterations; one lane per eigenvalue, f_l on the
//     fly.  cluster_kernel / cluster64_kernel: clusters by block inverse iteration + Rayleigh-Ritz.
//  4. build_vpanels_kernel + ut_diag_kernel + cuBLAS herk / gemm / trsm: X = Q Z in panels of 256
//     reflectors (compact WY in its triangular-solve form), only for the eigenvectors that are
//     asked for (the FP64 refinement subspace, or all of them when the caller wants A).
// Every wait on another block is bounded: a barrier that times out sets an error word and
// the kernel returns; the host reports BSE_ERR_NOT_CONVERGED.
#include <cooperative_groups.h>

#include <cmath>
#include <cstdlib>
#include <mutex>
#include <string>
#include <type_traits>

#include "blas_ops.h"
#include "bse_internal.h"
#include "dev_util.h"

namespace bse {
namespace {

using namespace dev;

template <typename T2>
struct TriArgs {
    int n;
    T2* A;
    int64_t lda;
    typename Real<T2>::t* d;   // n
    typename Real<T2>::t* e;   // n-1
    T2* tau;                   // n-1
    T2* vbuf;                  // reflectors: [2][n] shared, or [B][n] per block (redundant mode)
    T2* pbuf;                  // p = tau A v: [2][n] shared, or [B][n] per block
    T2* ppart;                 // [2][nt][n] column partial sums of the fused pass (by reflector parity)
    int64_t ppstride;          // elements between the two parities
    T2* dpart;                 // [2][gridDim] block partial dots (shared mode)
    T2* y;                     // Q^H applied in place: [n] shared, or [B][n] per block (may be null)
    unsigned* bar;
    unsigned* flags;           // fused kernel: one barrier flag per block, 128 bytes apart
    int* err;
    int TR;                    // rows per tile
    int redundant;             // 1: one barrier per reflector, every block finishes p itself
};

// Householder tridiagonalization (lower), full Hermitian storage.  See the file comment.
// Shared mode: v/p/y live once in global memory, two grid barriers per reflector.
// Redundant mode: every block keeps its own v/p/y (identical arithmetic in every block) and
// reduces the column partial sums of all columns itself, so one barrier per reflector suffices.
template <typename T2>
__global__ void __launch_bounds__(512, 1) tridiag_kernel(TriArgs<T2> a) {
    typedef typename Real<T2>::t R;
    extern __shared__ unsigned char smraw[];
    T2* sv = reinterpret_cast<T2*>(smraw);          // pending v (tile rows)
    T2* sw = sv + a.TR;                             // pending w (tile rows)
    T2* sv1 = sw + a.TR;                            // new reflector (tile rows)
    R* red = reinterpret_cast<R*>(sv1 + a.TR);      // 4 x 32 R for reductions
    const int n = a.n, tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int nwarp = nthr >> 5, B = gridDim.x, b = blockIdx.x;
    const bool rd = a.redundant != 0;
    const int64_t lda = a.lda;
    T2* A = a.A;
    T2 alpha_prev = C2<T2>(0, 0);
    bool have_prev = false;
    const T2 zero = C2<T2>(0, 0);
    T2* yb = a.y ? (rd ? a.y + (size_t)b * n : a.y) : nullptr;

    for (int k = 0; k <= n - 2; k++) {
        const T2* vp = rd ? a.vbuf + (size_t)b * n : a.vbuf + (size_t)((k + 1) & 1) * n;   // v_{k-1}
        const T2* pp = rd ? a.pbuf + (size_t)b * n : a.pbuf + (size_t)((k + 1) & 1) * n;   // p_{k-1}
        T2* vk = rd ? a.vbuf + (size_t)b * n : a.vbuf + (size_t)(k & 1) * n;
        T2* pk = rd ? a.pbuf + (size_t)b * n : a.pbuf + (size_t)(k & 1) * n;
        auto wprev = [&](int r) -> T2 { return cadd(pp[r], cmul(alpha_prev, vp[r])); };
        // pending update of an element of column k (row r): a - v_r conj(w_k) - w_r conj(v_k)
        const T2 vkk = have_prev ? vp[k] : zero, wkk = have_prev ? wprev(k) : zero;
        auto upd_colk = [&](int r) -> T2 {
            T2 x = A[r + (int64_t)k * lda];
            if (have_prev) x = csub(csub(x, cmulc(vp[r], wkk)), cmulc(wprev(r), vkk));
            return x;
        };
        // ---- phase A: reflector of column k (every block, redundantly) ----
        R loc[1] = {0};
        for (int r = k + 2 + tid; r < n; r += nthr) {
            T2 x = upd_colk(r);
            loc[0] += x.x * x.x + x.y * x.y;
        }
        block_sums<R, 1>(loc, red);
        const R xnorm2 = loc[0];
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
        if (b == 0 && tid == 0) {
            a.d[k] = dk;
            a.e[k] = beta;
            a.tau[k] = tauk;
        }
        // ---- phase B: pending rank-2 update of A[k+1:, k+1:] and column sums of A_new^H v_k ----
        const int m = n - (k + 1);
        const int nt = (m + a.TR - 1) / a.TR;
        // partial sums alternate between two buffers: in redundant mode a block may start the
        // next reflector's pass while another still reads this one's sums
        T2* ppk = a.ppart + (size_t)(k & 1) * a.ppstride;
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
                int r = r0 + lane;
                for (; r + 224 < r1; r += 256) {         // eight independent loads in flight per lane
                    T2 x[8];
#pragma unroll
                    for (int u = 0; u < 8; u++) x[u] = col[r + 32 * u];
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        const int i = r + 32 * u - r0;
                        if (have_prev) {
                            x[u] = csub(csub(x[u], cmulc(sv[i], wc)), cmulc(sw[i], vc));
                            col[r + 32 * u] = x[u];
                        }
                        const T2 q = cconjmul(x[u], sv1[i]);
                        accx += q.x;
                        accy += q.y;
                    }
                }
                for (; r < r1; r += 32) {
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
                if (lane == 0) ppk[(size_t)t * n + c] = C2<T2>(accx, accy);
            }
        }
        if (!grid_barrier(a.bar, a.err)) return;
        if (rd) {
            // ---- every block: v_k, p_k = tau sum_t ppart, alpha_k and y <- H_k^H y over all columns ----
            // Column k is still read below by every block, so block 0 stores reflector k-1 (held in
            // its v buffer until the loop below overwrites it) into column k-1, which nobody reads now.
            if (b == 0 && k >= 1) {
                for (int r = k + 1 + tid; r < n; r += nthr) A[r + (int64_t)(k - 1) * lda] = vk[r];
                __syncthreads();
            }
            R acc[4] = {0, 0, 0, 0};
            for (int c = k + 1 + tid; c < n; c += nthr) {
                T2 s = zero;
                for (int t = 0; t < nt; t++) s = cadd(s, ppk[(size_t)t * n + c]);
                const T2 p = cmul(tauk, s);
                const T2 v = (c == k + 1) ? C2<T2>(1, 0) : cmul(upd_colk(c), scal);
                pk[c] = p;
                vk[c] = v;
                const T2 q = cconjmul(p, v);
                acc[0] += q.x;
                acc[1] += q.y;
                if (yb) {
                    const T2 u = cconjmul(v, yb[c]);
                    acc[2] += u.x;
                    acc[3] += u.y;
                }
            }
            block_sums<R, 4>(acc, red);
            alpha_prev = cmul(C2<T2>(-0.5 * tauk.x, -0.5 * tauk.y), C2<T2>(acc[0], acc[1]));
            if (yb) {
                const T2 coef = cmulc(C2<T2>(acc[2], acc[3]), tauk);   // conj(tau) (v^H y)
                for (int c = k + 1 + tid; c < n; c += nthr) yb[c] = csub(yb[c], cmul(coef, vk[c]));
            }
            __syncthreads();
        } else {
            if (b == 0)
                for (int r = k + 1 + tid; r < n; r += nthr) vk[r] = (r == k + 1) ? C2<T2>(1, 0) : cmul(upd_colk(r), scal);
            // ---- C1: p_c = tau * sum_t ppart on this block's column slice, partial dots ----
            R acc[4] = {0, 0, 0, 0};
            for (int c = k + 1 + b * nthr + tid; c < n; c += B * nthr) {
                T2 s = zero;
                for (int t = 0; t < nt; t++) s = cadd(s, ppk[(size_t)t * n + c]);
                const T2 p = cmul(tauk, s);
                const T2 v = (c == k + 1) ? C2<T2>(1, 0) : cmul(upd_colk(c), scal);
                pk[c] = p;
                const T2 q = cconjmul(p, v);
                acc[0] += q.x;
                acc[1] += q.y;
                if (yb) {
                    const T2 u = cconjmul(v, yb[c]);
                    acc[2] += u.x;
                    acc[3] += u.y;
                }
            }
            block_sums<R, 4>(acc, red);
            if (tid == 0) {
                a.dpart[b] = C2<T2>(acc[0], acc[1]);
                a.dpart[B + b] = C2<T2>(acc[2], acc[3]);
            }
            if (!grid_barrier(a.bar, a.err)) return;
            // ---- C2: alpha_k, y <- H_k^H y on this block's slice, reflector storage ----
            R s4[4] = {0, 0, 0, 0};
            for (int i = tid; i < B; i += nthr) {
                const T2 u = a.dpart[i], q = a.dpart[B + i];
                s4[0] += u.x;
                s4[1] += u.y;
                s4[2] += q.x;
                s4[3] += q.y;
            }
            block_sums<R, 4>(s4, red);
            alpha_prev = cmul(C2<T2>(-0.5 * tauk.x, -0.5 * tauk.y), C2<T2>(s4[0], s4[1]));
            if (yb) {
                // v_k from the buffer block 0 published before the first barrier (column k is being
                // overwritten by block 0 below)
                const T2 coef = cmulc(C2<T2>(s4[2], s4[3]), tauk);
                for (int c = k + 1 + b * nthr + tid; c < n; c += B * nthr) yb[c] = csub(yb[c], cmul(coef, vk[c]));
            }
            __syncthreads();
            if (b == 0)
                for (int r = k + 2 + tid; r < n; r += nthr) A[r + (int64_t)k * lda] = vk[r];
        }
        have_prev = true;
    }
    if (b == 0 && tid == 0) {
        if (n >= 2) {
            const T2* vp = rd ? a.vbuf : a.vbuf + (size_t)((n - 2) & 1) * n;
            const T2* pp = rd ? a.pbuf : a.pbuf + (size_t)((n - 2) & 1) * n;
            const T2 v = vp[n - 1], w = cadd(pp[n - 1], cmul(alpha_prev, vp[n - 1]));
            T2 x = A[(n - 1) + (int64_t)(n - 1) * lda];
            x = csub(csub(x, cmulc(v, w)), cmulc(w, v));
            a.d[n - 1] = x.x;
        } else {
            a.d[0] = A[0].x;
        }
    }
}

// Segments per trailing column in the fused pass, and loads in flight per lane.
constexpr int kSegMax = 8;
constexpr int kPassUnroll = 16;

// Shared-memory footprint of tridiag_fused_kernel: reduction scratch, the alpha slot, the
// pending reflector v, the pending w = p + alpha v, the new column / reflector, y, and the
// per-segment column sums of the block's columns.
template <typename T2>
size_t fused_smem(int n, bool with_y, int blocks) {
    return 1056 + (size_t)(with_y ? 4 : 3) * n * sizeof(T2) + (size_t)kSegMax * ((n + blocks - 1) / blocks) * sizeof(T2);
}

// One-stage reduction with the working vectors in shared memory (one grid barrier per
// reflector).  Same algorithm and storage as tridiag_kernel's redundant mode; what changes is
// where the vectors live and how the latency of each step is hidden.  Iteration k:
//  1. after the barrier, one round of loads per thread (no dependent loads): the column sums
//     p_{k-1} = tau A^H v_{k-1} of reflector k-1 and the raw column k.  Every block then forms
//     alpha_{k-1}, w_{k-1} = p + alpha v and y <- H_{k-1}^H y, applies the pending rank-2
//     update of reflector k-1 to column k and builds reflector k, all in shared memory;
//  2. the block's share of the trailing columns is split into (column, row segment) items so
//     that every warp has work, and each lane keeps 16 loads of its column in flight; the
//     segment sums of a column are added in a fixed order in shared memory and published as
//     one value per column (double-buffered by reflector parity);
//  3. grid barrier.
// Block 0 stores reflector k-1 into column k-1 in iteration k, when no block reads it any more.
template <typename T2>
__global__ void __launch_bounds__(512, 1) tridiag_fused_kernel(TriArgs<T2> a) {
    typedef typename Real<T2>::t R;
    constexpr int JB = 8;   // columns per thread and load round after the barrier
    extern __shared__ unsigned char smraw[];
    R* red = reinterpret_cast<R*>(smraw);                                // 4 x 32 R (1024 bytes reserved)
    T2* s_alpha = reinterpret_cast<T2*>(smraw + 1024);
    const int n = a.n, tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int nwarp = nthr >> 5, B = gridDim.x, b = blockIdx.x;
    const int64_t lda = a.lda;
    T2* A = a.A;
    T2* sV = reinterpret_cast<T2*>(smraw + 1056);
    T2* sW = sV + n;
    T2* sX = sW + n;
    T2* sY = a.y ? sX + n : nullptr;
    T2* sSeg = sX + (a.y ? 2 : 1) * (size_t)n;                           // [kSegMax][ceil(n / B)]
    const int cstride = (n + B - 1) / B;
    const T2 zero = C2<T2>(0, 0), one = C2<T2>(1, 0);
    __shared__ int s_fail;
    if (tid == 0) s_fail = 0;
    for (int r = tid; r < n; r += nthr) {
        sV[r] = zero;
        sW[r] = zero;
        sX[r] = zero;
        if (sY) sY[r] = a.y[r];
    }
    __syncthreads();
    T2 tau_prev = zero;
    for (int k = 0; k < n; k++) {
        const bool has_c = k >= 1, has_a = k <= n - 2;
        const T2* pin = a.ppart + (size_t)((k + 1) & 1) * n;             // column sums of reflector k-1
        // ---- 1a. loads: p_{k-1} (pre-tau column sums) and the raw column k, rows/columns i >= k ----
        R acc[4] = {0, 0, 0, 0};
        const T2 pk_raw = has_c ? pin[k] : zero;
        for (int i0 = k + tid; i0 < n; i0 += JB * nthr) {
            T2 raw[JB], ps[JB];
#pragma unroll
            for (int u = 0; u < JB; u++) {
                const int i = i0 + u * nthr;
                raw[u] = i < n ? A[i + (int64_t)k * lda] : zero;
                ps[u] = (has_c && i < n) ? pin[i] : zero;
            }
#pragma unroll
            for (int u = 0; u < JB; u++) {
                const int i = i0 + u * nthr;
                if (i < n) {
                    sV[i] = raw[u];                                        // v_{k-2} is no longer needed
                    if (has_c) {
                        const T2 p = cmul(tau_prev, ps[u]);
                        const T2 v = sX[i];
                        sW[i] = p;                                         // w_{k-2} is no longer needed
                        const T2 q = cconjmul(p, v);
                        acc[0] += q.x;
                        acc[1] += q.y;
                        if (sY) {
                            const T2 t = cconjmul(v, sY[i]);
                            acc[2] += t.x;
                            acc[3] += t.y;
                        }
                    }
                }
            }
        }
        // ---- 1b. alpha_{k-1}, w_{k-1}, y <- H_{k-1}^H y, pending update of column k ----
        T2 alpha_c = zero, coef = zero, wkk = zero;
        const T2 vkk = sX[k];
        if (has_c) {
            block_sums<R, 4>(acc, red);
            alpha_c = cmul(C2<T2>(-0.5 * tau_prev.x, -0.5 * tau_prev.y), C2<T2>(acc[0], acc[1]));
            coef = cmulc(C2<T2>(acc[2], acc[3]), tau_prev);                // conj(tau) (v^H y)
            wkk = cadd(cmul(tau_prev, pk_raw), cmul(alpha_c, vkk));
        }
        R loc[1] = {0};
        for (int i = k + tid; i < n; i += nthr) {
            const T2 v = sX[i];
            T2 w = zero;
            if (has_c) {
                w = cadd(sW[i], cmul(alpha_c, v));
                sW[i] = w;
                if (sY) sY[i] = csub(sY[i], cmul(coef, v));
                if (b == 0 && i >= k + 1) A[i + (int64_t)(k - 1) * lda] = v;
            }
            const T2 xv = csub(csub(sV[i], cmulc(v, wkk)), cmulc(w, vkk));
            sV[i] = xv;
            if (i == k) {
                if (b == 0) a.d[k] = xv.x;
            } else if (i == k + 1) {
                *s_alpha = xv;
            } else {
                loc[0] += xv.x * xv.x + xv.y * xv.y;
            }
        }
        if (!has_a) break;
        // ---- 1c. reflector k ----
        block_sums<R, 1>(loc, red);
        const R xnorm2 = loc[0];
        T2 tauk, scal;
        R beta;
        // FP64 square roots and divisions are slow on this part: one thread forms the scalars
        // and the block reads them back; FP32 blocks form them in every thread
        const bool one_thread = sizeof(R) == 8;
        if (!one_thread || tid == 0) {
            const T2 alpha = *s_alpha;
            if (xnorm2 == R(0) && alpha.y == R(0)) {
                tauk = zero;
                beta = alpha.x;
                scal = zero;
            } else {
                beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2), alpha.x);
                tauk = C2<T2>((beta - alpha.x) / beta, -alpha.y / beta);
                scal = cinv(csub(alpha, C2<T2>(beta, 0)));
            }
            if (one_thread) {
                s_alpha[0] = tauk;   // every thread has read alpha (block_sums synchronised after it was set)
                s_alpha[1] = scal;
                red[127] = beta;
            }
        }
        if (one_thread) {
            __syncthreads();
            tauk = s_alpha[0];
            scal = s_alpha[1];
            beta = red[127];
        }
        if (b == 0 && tid == 0) {
            a.e[k] = beta;
            a.tau[k] = tauk;
        }
        for (int i = k + 1 + ((tid + nthr - 1) % nthr); i < n; i += nthr) sV[i] = i == k + 1 ? one : cmul(sV[i], scal);
        __syncthreads();
        {
            T2* t = sV;   // sV <- v_{k-1}, sX <- v_k
            sV = sX;
            sX = t;
        }
        tau_prev = tauk;
        // ---- 2. pending update of this block's trailing columns, column sums of A^H v_k ----
        const int m = n - (k + 1);
        const bool have_prev = k > 0;
        const int c_lo = k + 1 + (int)((int64_t)m * b / B), c_hi = k + 1 + (int)((int64_t)m * (b + 1) / B);
        const int ncols = c_hi - c_lo;
        const int cmax = (m + B - 1) / B;
        // segments per column: fewest sequential rounds of kPassUnroll loads per warp
        int nseg = 1, best = 1 << 30;
        for (int g = 1; g <= kSegMax && (g == 1 || (m + g - 1) / g >= 32); g++) {
            const int rounds = ((cmax * g + nwarp - 1) / nwarp) * (((m + g - 1) / g + 32 * kPassUnroll - 1) / (32 * kPassUnroll));
            if (rounds < best) { best = rounds; nseg = g; }
        }
        const int L = (m + nseg - 1) / nseg;
        for (int it = warp; it < ncols * nseg; it += nwarp) {
            const int cl = it % ncols, g = it / ncols, c = c_lo + cl;
            const int r0 = k + 1 + g * L, r1 = min(n, r0 + L);
            const T2 vc = sV[c], wc = sW[c];
            T2* col = A + (int64_t)c * lda;
            R ax = 0, ay = 0;
            for (int r = r0 + lane; r < r1; r += 32 * kPassUnroll) {
                T2 x[kPassUnroll];
#pragma unroll
                for (int u = 0; u < kPassUnroll; u++) x[u] = r + 32 * u < r1 ? col[r + 32 * u] : zero;
#pragma unroll
                for (int u = 0; u < kPassUnroll; u++) {
                    const int i = r + 32 * u;
                    if (i < r1) {
                        T2 xv = x[u];
                        if (have_prev) {
                            xv = csub(csub(xv, cmulc(sV[i], wc)), cmulc(sW[i], vc));
                            col[i] = xv;
                        }
                        const T2 q = cconjmul(xv, sX[i]);
                        ax += q.x;
                        ay += q.y;
                    }
                }
            }
            ax = warp_sum(ax);
            ay = warp_sum(ay);
            if (lane == 0) sSeg[(size_t)g * cstride + cl] = C2<T2>(ax, ay);
        }
        __syncthreads();
        T2* pout = a.ppart + (size_t)(k & 1) * n;
        for (int cl = tid; cl < ncols; cl += nthr) {
            T2 sum = zero;
            for (int g = 0; g < nseg; g++) sum = cadd(sum, sSeg[(size_t)g * cstride + cl]);
            pout[c_lo + cl] = sum;
        }
        // ---- 3. ----
        if (!flag_barrier<true>(a.flags, (unsigned)(k + 1), a.err, &s_fail)) return;
    }
    __syncthreads();   // the last update of y was made by other threads
    if (b == 0 && sY)
        for (int r = tid; r < n; r += nthr) a.y[r] = sY[r];
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

// The same count with the fast FP32 division (2 ulp; |q| >= pivmin keeps it in range) for the
// mixed path, where the eigenvalues are refined afterwards (FP64 Rayleigh quotients, the FP64
// refinement): the dependent division is the latency of every step of the recurrence.
__device__ __forceinline__ int sturm_fast(int n, const float* __restrict__ d, const float* __restrict__ e2, float x,
                                          float pivmin) {
    float q = d[0] - x;
    if (fabsf(q) < pivmin) q = -pivmin;
    int c = q <= 0.0f;
#pragma unroll 4
    for (int j = 1; j < n; j++) {
        q = d[j] - __fdividef(e2[j - 1], q) - x;
        if (fabsf(q) < pivmin) q = -pivmin;
        c += q <= 0.0f;
    }
    return c;
}

// i-th smallest eigenvalue of T by FP32 bisection to FP32 resolution.  cl[i] = 1 marks an
// eigenvalue whose FP32 estimate lies within `ctol` of a neighbour's (a cluster at FP32
// resolution); those get FP64 bisection in cluster_bisect_kernel.  FP64 division is slow on
// this part, so the FP64 work is spent only where FP32 cannot separate eigenvalues.
template <bool FAST>
__global__ void __launch_bounds__(256) bisect32_kernel(int n, int lp, int rounds, const float* __restrict__ df,
                                                       const float* __restrict__ e2f, float glo, float ghi, float pivminf,
                                                       double* __restrict__ w) {
    // P = 2^lp lanes per eigenvalue evaluate the Sturm count at P interior points of the current
    // interval ((P+1)-section): small problems spread each eigenvalue over a whole warp to fill
    // the GPU, large ones keep plain bisection (P = 1), where more points would only add work
    const int P = 1 << lp, lane = threadIdx.x & 31, grp = lane >> lp, gl = lane & (P - 1);
    const int i = (((blockIdx.x * blockDim.x + threadIdx.x) >> 5) << (5 - lp)) + grp;
    const bool valid = i < n;
    const int ii = valid ? i : n - 1;
    float a = glo, b = ghi;
    bool done = false;
    for (int it = 0; it < rounds; it++) {
        const float h = (b - a) / (float)(P + 1);
        // P = 1: plain bisection at the midpoint (the FP64 path keeps this arithmetic exactly)
        const float x = P == 1 ? 0.5f * (a + b) : a + h * (float)(gl + 1);
        if (P == 1 ? !(x > a && x < b) : !(a + h > a && a + h < b)) done = true;
        if (__all_sync(0xffffffffu, done)) break;
        const int cnt = done ? 0 : (FAST ? sturm_fast(n, df, e2f, x, pivminf) : sturm<float>(n, df, e2f, x, pivminf));
        const unsigned ball = __ballot_sync(0xffffffffu, cnt > ii);
        const unsigned mine = P == 32 ? ball : (ball >> (grp * P)) & ((1u << P) - 1u);
        if (!done) {
            if (P == 1) {
                if (mine) b = x;
                else a = x;
            } else if (mine == 0) {
                a = a + h * (float)P;
            } else {
                const int l0 = __ffs(mine) - 1;   // first point at or above eigenvalue ii
                b = a + h * (float)(l0 + 1);
                a = a + h * (float)l0;
            }
        }
    }
    if (valid && gl == 0) w[i] = 0.5 * ((double)a + (double)b);
}

__device__ __forceinline__ double start_value(unsigned i, unsigned k) {
    unsigned h = i * 0x9E3779B9u ^ (k + 0x7F4A7C15u) * 0x85EBCA6Bu;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return 0.5 + (double)(h & 0xFFFFFF) * (1.0 / 16777216.0);   // (0.5, 1.5)
}
// The same value rounded to FP32 (one rounding of the exact sum, as (float)start_value), without
// FP64 arithmetic: FP64 is slow on this part and the sweeps run one warp per SM.
__device__ __forceinline__ float start_value32(unsigned i, unsigned k) {
    unsigned h = i * 0x9E3779B9u ^ (k + 0x7F4A7C15u) * 0x85EBCA6Bu;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return 0.5f + (float)(h & 0xFFFFFF) * (1.0f / 16777216.0f);
}

// Sequential sweeps over per-thread vectors are latency-bound (one warp per SM on the GPU):
// element k of a thread's vector lives at p[k * RS], and the loops prefetch the line PD rows
// ahead into L1 so the dependent recurrences do not wait on L2.
__device__ __forceinline__ void pf_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// LU with partial pivoting of the tridiagonal T - s I (dlagtf); pivots stored as reciprocals so
// the solves need no division.
template <typename F, int RS, int PD>
__device__ __forceinline__ void tri_factor(int n, const F* __restrict__ d, const F* __restrict__ e, F s, F pert,
                                           F* __restrict__ Ur, F* __restrict__ Ub, F* __restrict__ Ud,
                                           F* __restrict__ Lc, signed char* __restrict__ piv) {
    F ak = d[0] - s;
    F bk = n > 1 ? e[0] : F(0);
    for (int k = 0; k < n - 1; k++) {
        if (k + PD < n) {
            pf_l1(d + k + PD);
            pf_l1(e + k + PD);
        }
        const F ck = e[k];
        const F anext = d[k + 1] - s;
        const F bnext = (k + 1 < n - 1) ? e[k + 1] : F(0);
        if (fabs(ck) <= fabs(ak)) {
            const F u = fabs(ak) < pert ? (ak < 0 ? -pert : pert) : ak;
            const F r = F(1) / u;
            const F mult = ck * r;
            Ur[(size_t)k * RS] = r;
            Ub[(size_t)k * RS] = bk;
            Ud[(size_t)k * RS] = F(0);
            Lc[(size_t)k * RS] = mult;
            piv[(size_t)k * RS] = 0;
            ak = anext - mult * bk;
            bk = bnext;
        } else {
            const F r = F(1) / ck;
            const F mult = ak * r;
            Ur[(size_t)k * RS] = r;
            Ub[(size_t)k * RS] = anext;
            Ud[(size_t)k * RS] = bnext;
            Lc[(size_t)k * RS] = mult;
            piv[(size_t)k * RS] = 1;
            ak = bk - mult * anext;
            bk = -mult * bnext;
        }
    }
    const F u = fabs(ak) < pert ? (ak < 0 ? -pert : pert) : ak;
    Ur[(size_t)(n - 1) * RS] = F(1) / u;
}

// One solve (T - s I) x = y in place on Y, the input scaled by `sin` on the fly; returns the
// max-norm of the solution (the caller folds 1/max into the next sweep).
template <typename F, int RS, int PD>
__device__ __forceinline__ F tri_solve(int n, const F* __restrict__ Ur, const F* __restrict__ Ub,
                                       const F* __restrict__ Ud, const F* __restrict__ Lc,
                                       const signed char* __restrict__ piv, F* __restrict__ Y, F sin) {
    F ycur = Y[0] * sin;
    for (int k = 0; k < n - 1; k++) {
        if (k + PD < n - 1) {
            pf_l1(Lc + (size_t)(k + PD) * RS);
            pf_l1(piv + (size_t)(k + PD) * RS);
            pf_l1(Y + (size_t)(k + 1 + PD) * RS);
        }
        const F mult = Lc[(size_t)k * RS];
        const F ynext = Y[(size_t)(k + 1) * RS] * sin;
        F out;
        if (piv[(size_t)k * RS] == 0) {
            out = ycur;
            ycur = ynext - mult * ycur;
        } else {
            out = ynext;
            ycur = ycur - mult * ynext;
        }
        Y[(size_t)k * RS] = out;
    }
    F x1 = 0, x2 = 0, mx = 0;
    {
        const F x = ycur * Ur[(size_t)(n - 1) * RS];
        Y[(size_t)(n - 1) * RS] = x;
        x1 = x;
        mx = fabs(x);
    }
    for (int k = n - 2; k >= 0; k--) {
        if (k - PD >= 0) {
            pf_l1(Ur + (size_t)(k - PD) * RS);
            pf_l1(Ub + (size_t)(k - PD) * RS);
            pf_l1(Ud + (size_t)(k - PD) * RS);
            pf_l1(Y + (size_t)(k - PD) * RS);
        }
        const F x = (Y[(size_t)k * RS] - Ub[(size_t)k * RS] * x1 - Ud[(size_t)k * RS] * x2) * Ur[(size_t)k * RS];
        Y[(size_t)k * RS] = x;
        x2 = x1;
        x1 = x;
        mx = fmax(mx, fabs(x));
    }
    return mx;
}


// Staged FP32 sweeps for the inverse iterations.  The dependent row recurrences of the LU factor
// and the two triangular solves run one warp per SM (one lane per eigenvalue); with operands read
// from global memory row by row each step waits for a load (long-scoreboard stalls dominated).  Here
// the warp copies chunks of SCH rows of its interleaved [k][32] arrays into shared memory with
// cp.async, SNS chunks ahead, so every step reads shared memory.  All 32 lanes must call these.
constexpr int SCH = 16;                                  // rows per staged chunk
constexpr int SNS = 4;                                   // chunks in flight
constexpr int SRW = SCH * 32;                            // elements of one array in one chunk
constexpr size_t kStageSmem = (size_t)SNS * 4 * SRW * sizeof(float) + (size_t)SNS * SRW;   // 34 KB: several warps per SM

__device__ __forceinline__ void cp16(void* sdst, const void* gsrc) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// rows [r0, r1) of an interleaved array (32 elements of esz bytes per row) -> dst
__device__ __forceinline__ void stage_rows(void* dst, const void* base, int r0, int r1, int esz) {
    const int lane = threadIdx.x & 31;
    const int bytes = (r1 - r0) * 32 * esz;
    const char* src = (const char*)base + (size_t)r0 * 32 * esz;
    for (int q = lane * 16; q < bytes; q += 32 * 16) cp16((char*)dst + q, src + q);
}
// rows [r0, r1) of a plain array of floats (one value per row, shared by the lanes) -> dst
__device__ __forceinline__ void stage_vec(float* dst, const float* base, int r0, int r1) {
    const int lane = threadIdx.x & 31;
    // 16-byte pieces covering [r0, r1) rounded out to multiples of 4 floats (the arrays are
    // allocated with 8 floats of padding)
    const int a0 = r0 & ~3, a1 = (r1 + 3) & ~3;
    for (int q = a0 + lane * 4; q < a1; q += 32 * 4) cp16(dst + (q - a0), base + q);
}

// LU of T - s I (as tri_factor), d/e staged; U/L written to the warp's interleaved arrays
// (warp base pointers: element k of lane l at p[k * 32 + l]).
__device__ void tri_factor_staged(int n, const float* __restrict__ d, const float* __restrict__ e, float s, float pert,
                                  float* __restrict__ Urw, float* __restrict__ Ubw, float* __restrict__ Udw,
                                  float* __restrict__ Lcw, signed char* __restrict__ pvw, float* sm) {
    const int lane = threadIdx.x & 31;
    // stage ch: d and e rows [ch*SCH, ch*SCH + SCH] (one row of lookahead), 16-byte pieces
    constexpr int VW = SCH + 8;
    const int nch = (n + SCH - 1) / SCH;
    auto issue = [&](int ch) {
        if (ch < nch) {
            // rows k in [r0, rk1) read d[k + 1], e[k] and e[k + 1]
            const int st = ch % SNS, r0 = ch * SCH, rk1 = min(n - 1, r0 + SCH);
            stage_vec(sm + (st * 2) * VW, d, r0, min(n, rk1 + 1));
            stage_vec(sm + (st * 2 + 1) * VW, e, r0, min(n - 1, rk1 + 1));
        }
        cp_commit();
    };
    for (int ch = 0; ch < SNS - 1; ch++) issue(ch);
    float ak = 0, bk = 0;
    for (int ch = 0; ch < nch; ch++) {
        issue(ch + SNS - 1);
        cp_wait<SNS - 1>();
        __syncwarp();
        const int st = ch % SNS, r0 = ch * SCH, r1 = min(n - 1, r0 + SCH);
        const float* sd = sm + (st * 2) * VW;
        const float* se = sm + (st * 2 + 1) * VW;
        const int off = r0 & 3;                  // stage_vec starts at r0 rounded down to 4
        if (ch == 0) {
            ak = sd[off] - s;
            bk = n > 1 ? se[off] : 0.0f;
        }
#pragma unroll 4
        for (int k = r0; k < r1; k++) {
            const int q = k - r0 + off;
            const float ck = se[q];
            const float anext = sd[q + 1] - s;
            const float bnext = (k + 1 < n - 1) ? se[q + 1] : 0.0f;
            // pivots are at least `pert` in magnitude: the fast reciprocal (2 ulp) is safe, and the
            // factor and the solves use the same stored values.  Both pivot choices are formed and
            // selected (the lanes of a warp pivot differently; a branch would run both paths).
            const bool sw = fabsf(ck) > fabsf(ak);
            const float ua = fabsf(ak) < pert ? (ak < 0 ? -pert : pert) : ak;
            const float r = __fdividef(1.0f, sw ? ck : ua);
            const float mult = (sw ? ak : ck) * r;
            Urw[(size_t)k * 32 + lane] = r;
            Ubw[(size_t)k * 32 + lane] = sw ? anext : bk;
            Udw[(size_t)k * 32 + lane] = sw ? bnext : 0.0f;
            Lcw[(size_t)k * 32 + lane] = mult;
            pvw[(size_t)k * 32 + lane] = sw ? 1 : 0;
            const float ak_n = sw ? fmaf(-mult, anext, bk) : fmaf(-mult, bk, anext);
            bk = sw ? -mult * bnext : bnext;
            ak = ak_n;
        }
        __syncwarp();
    }
    cp_wait<0>();
    const float u = fabsf(ak) < pert ? (ak < 0 ? -pert : pert) : ak;
    Urw[(size_t)(n - 1) * 32 + lane] = 1.0f / u;
    __threadfence();
    __syncwarp();
}

// (T - s I) x = y in place on the warp's Y (input scaled by sin); returns max |x| of this lane.
__device__ float tri_solve_staged(int n, const float* __restrict__ Urw, const float* __restrict__ Ubw,
                                  const float* __restrict__ Udw, const float* __restrict__ Lcw,
                                  const signed char* __restrict__ pvw, float* __restrict__ Yw, float sin, float* sm) {
    const int lane = threadIdx.x & 31;
    signed char* smp = reinterpret_cast<signed char*>(sm + SNS * 4 * SRW);
    float ycur = Yw[lane] * sin;
    // forward elimination, rows k = 0 .. n-2: Lc[k], piv[k], Y[k+1]
    const int nf = n - 1, nchf = (nf + SCH - 1) / SCH;
    auto issue_f = [&](int ch) {
        if (ch < nchf) {
            const int st = ch % SNS, r0 = ch * SCH, r1 = min(nf, r0 + SCH);
            stage_rows(sm + (st * 4 + 0) * SRW, Lcw, r0, r1, 4);
            stage_rows(sm + (st * 4 + 1) * SRW, Yw + 32, r0, r1, 4);
            stage_rows(smp + st * SRW, pvw, r0, r1, 1);
        }
        cp_commit();
    };
    for (int ch = 0; ch < SNS - 1; ch++) issue_f(ch);
    for (int ch = 0; ch < nchf; ch++) {
        issue_f(ch + SNS - 1);
        cp_wait<SNS - 1>();
        __syncwarp();
        const int st = ch % SNS, r0 = ch * SCH, r1 = min(nf, r0 + SCH);
        const float* sL = sm + (st * 4 + 0) * SRW;
        const float* sY = sm + (st * 4 + 1) * SRW;
        const signed char* sP = smp + st * SRW;
#pragma unroll 8
        for (int k = r0; k < r1; k++) {
            const int q = (k - r0) * 32 + lane;
            const float mult = sL[q];
            const float ynext = sY[q] * sin;
            const bool sw = sP[q] != 0;   // selects, not a branch: the lanes pivot differently
            const float out = sw ? ynext : ycur;
            ycur = sw ? fmaf(-mult, ynext, ycur) : fmaf(-mult, ycur, ynext);
            Yw[(size_t)k * 32 + lane] = out;
        }
        __syncwarp();
    }
    cp_wait<0>();
    __threadfence();
    __syncwarp();
    // back substitution: x_{n-1} = ycur Ur[n-1]; rows k = n-2 .. 0: Y[k], Ub[k], Ud[k], Ur[k]
    float x1 = ycur * Urw[(size_t)(n - 1) * 32 + lane], x2 = 0.0f, mx = fabsf(x1);
    Yw[(size_t)(n - 1) * 32 + lane] = x1;
    const int nb = n - 1, nchb = (nb + SCH - 1) / SCH;
    auto issue_b = [&](int ch) {
        if (ch < nchb) {
            const int st = ch % SNS, r1 = nb - ch * SCH, r0 = max(0, r1 - SCH);
            stage_rows(sm + (st * 4 + 0) * SRW, Urw, r0, r1, 4);
            stage_rows(sm + (st * 4 + 1) * SRW, Ubw, r0, r1, 4);
            stage_rows(sm + (st * 4 + 2) * SRW, Udw, r0, r1, 4);
            stage_rows(sm + (st * 4 + 3) * SRW, Yw, r0, r1, 4);
        }
        cp_commit();
    };
    for (int ch = 0; ch < SNS - 1; ch++) issue_b(ch);
    for (int ch = 0; ch < nchb; ch++) {
        issue_b(ch + SNS - 1);
        cp_wait<SNS - 1>();
        __syncwarp();
        const int st = ch % SNS, r1 = nb - ch * SCH, r0 = max(0, r1 - SCH);
        const float* sR = sm + (st * 4 + 0) * SRW;
        const float* sB = sm + (st * 4 + 1) * SRW;
        const float* sD = sm + (st * 4 + 2) * SRW;
        const float* sY = sm + (st * 4 + 3) * SRW;
#pragma unroll 8
        for (int k = r1 - 1; k >= r0; k--) {
            const int q = (k - r0) * 32 + lane;
            const float x = (sY[q] - sB[q] * x1 - sD[q] * x2) * sR[q];
            Yw[(size_t)k * 32 + lane] = x;
            x2 = x1;
            x1 = x;
            mx = fmaxf(mx, fabsf(x));
        }
        __syncwarp();
    }
    cp_wait<0>();
    __threadfence();
    __syncwarp();
    return mx;
}

// FP64 Rayleigh quotient z^T T z / z^T z of X (FP32 or FP64 elements, scaled by sx), with the
// squared norm.
template <int RS, int PD, typename V>
__device__ __forceinline__ double tri_rq(int n, const double* __restrict__ d, const double* __restrict__ e,
                                         const V* __restrict__ X, double sx, double* den_out) {
    double num = 0, den = 0, xprev = 0, x = (double)X[0] * sx;
    for (int k = 0; k < n; k++) {
        if (k + PD < n) {
            pf_l1(X + (size_t)(k + PD) * RS);
            pf_l1(d + k + PD);
        }
        const double xn = (k + 1 < n) ? (double)X[(size_t)(k + 1) * RS] * sx : 0.0;
        num += x * (d[k] * x + (k > 0 ? e[k - 1] * xprev : 0.0) + (k + 1 < n ? e[k] * xn : 0.0));
        den += x * x;
        xprev = x;
        x = xn;
    }
    *den_out = den;
    return num / den;
}

// Eigenpair (w_i, z_i) of T for an eigenvalue FP32 bisection separates from its neighbours:
// three FP32 inverse iterations from the FP32 estimate; with `fp64` two FP64 Rayleigh-quotient
// iterations follow (the FP64 path), otherwise the eigenvalue is the FP64 Rayleigh quotient of
// the FP32 vector (T itself carries FP32 rounding in the mixed path, so FP64 iterations on it
// would not make the pair more accurate).  Writes w[i], f_i = sum_k conj(y_k) z_k, and z_i for
// i < n_store.  Cluster members (cl[i] != 0) are left to the cluster kernels.
template <typename TZ>
__global__ void __launch_bounds__(32) invit_kernel(int n, const double* __restrict__ d, const double* __restrict__ e,
                                                   const float* __restrict__ df, const float* __restrict__ ef,
                                                   double* __restrict__ w, const signed char* __restrict__ cl,
                                                   int i0, int count, double tnorm, const double2* __restrict__ y,
                                                   double2* __restrict__ f, TZ* __restrict__ z, int64_t ldz,
                                                   int n_store, double* __restrict__ scr, float* __restrict__ scr32,
                                                   signed char* __restrict__ piv, float* __restrict__ scs, int fp64) {
    extern __shared__ float stage_sm[];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = i0 + t;
    // lanes past the batch or on cluster members run the sweeps on a dummy right-hand side (the
    // staged sweeps need the whole warp) and write nothing
    const bool act = t < count && !cl[i];
    // a warp whose eigenvalues all belong to clusters (most of them, where the spectrum is dense)
    // has nothing to do: the block is this one warp
    if (!__any_sync(0xffffffffu, act)) return;
    // this warp's scratch: [array][k][32 lanes], one 128-byte line per row in FP32
    const size_t W32 = (size_t)n * 32;
    const size_t lane = threadIdx.x & 31;
    const double lam0 = act ? w[i] : 0.0;
    float* Urw = scr32 + (size_t)blockIdx.x * 5 * W32;
    float* Ubw = Urw + W32;
    float* Udw = Ubw + W32;
    float* Lcw = Udw + W32;
    float* Yw = Lcw + W32;
    signed char* pvw = piv + (size_t)blockIdx.x * W32;
    float* Y = Yw + lane;
    signed char* pv = pvw + lane;
    tri_factor_staged(n, df, ef, (float)lam0, 1.1920929e-7f * (float)fmax(tnorm, 1e-30), Urw, Ubw, Udw, Lcw, pvw, stage_sm);
#pragma unroll 4
    for (int k = 0; k < n; k++) Y[(size_t)k * 32] = act ? start_value32(i, k) : 0.0f;
    __threadfence();
    __syncwarp();
    float sc = 1.0f;
    for (int it = 0; it < 3; it++) {
        const float mx = tri_solve_staged(n, Urw, Ubw, Udw, Lcw, pvw, Yw, sc, stage_sm);
        sc = mx > 0 ? 1.0f / mx : 1.0f;
    }
    if (!act) return;
    const bool keep = i < n_store;
    if (!fp64) {
        // mixed path: invit_finish_kernel forms the Rayleigh quotient, f_i and z_i from Y and the
        // scale of the last sweep, a warp per eigenvalue
        scs[t] = sc;
        return;
    }
    double* Vr = scr + (size_t)blockIdx.x * 5 * W32 + lane;
    double* Vb = Vr + W32;
    double* Vd = Vb + W32;
    double* Vc = Vd + W32;
    double* X = Vc + W32;
    for (int k = 0; k < n; k++) X[(size_t)k * 32] = (double)Y[(size_t)k * 32] * (double)sc;
    const double pert = 2.220446049250313e-16 * fmax(tnorm, 1e-300);
    double den = 1, sx = 1.0;
    for (int it = 0; it < 2; it++) {
        const double shift = tri_rq<32, 16>(n, d, e, X, sx, &den);
        tri_factor<double, 32, 16>(n, d, e, shift, pert, Vr, Vb, Vd, Vc, pv);
        const double mx = tri_solve<double, 32, 16>(n, Vr, Vb, Vd, Vc, pv, X, sx);
        sx = mx > 0 ? 1.0 / mx : 1.0;
    }
    const double lam = tri_rq<32, 16>(n, d, e, X, sx, &den);
    const double inv = sx / sqrt(den);
    w[i] = lam;
    double fx = 0, fy = 0;
    for (int k = 0; k < n; k++) {
        if (k + 16 < n) pf_l1(X + (size_t)(k + 16) * 32);
        const double x = X[(size_t)k * 32] * inv;
        if (f) {
            const double2 yy = y[k];
            fx += yy.x * x;
            fy -= yy.y * x;
        }
        if (keep) z[(size_t)k + (size_t)i * ldz] = (TZ)x;
    }
    if (f) f[i] = make_double2(fx, fy);
}

// FP64 path: eigenpairs of a cluster (dstein-style), one warp
// per cluster.  Member j gets FP64 inverse iteration with its own shift (lane 0 runs the
// tridiagonal factor and solves) and Gram-Schmidt against the cluster's earlier members (all
// lanes); then a Rayleigh-Ritz step inside the cluster (Jacobi on the c x c projected matrix)
// gives FP64 eigenpairs.  Member vectors stay in Zc (column-major n x c per cluster).  Members
// outside [cout[2t], cout[2t+1]) are guards: solved with the cluster, not written.
__device__ __forceinline__ double warp_dsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Mixed path, after invit_kernel: one warp per eigenvalue (lanes over rows) reads the FP32
// vector Y from the sweep scratch and forms, in FP64, the Rayleigh quotient z^T T z / z^T z (FP32
// bisection leaves an error of a few eps32 |T|; the quotient's is the squared residual), the norm,
// f_i = sum_k conj(y_k) z_k from FP32 products, and stores z_i (i < n_store) with coalesced writes.
// FP64 arithmetic is slow on this part: spread over all SMs it costs little, in the sweeps'
// one-warp-per-SM layout it cost more than the sweeps.
template <typename TZ>
__global__ void __launch_bounds__(256) invit_finish_kernel(int n, const double* __restrict__ d, const double* __restrict__ e,
                                                           const signed char* __restrict__ cl, int i0, int count,
                                                           const float2* __restrict__ y32, const float* __restrict__ scr32,
                                                           const float* __restrict__ scs, double* __restrict__ w,
                                                           double2* __restrict__ f, TZ* __restrict__ z, int64_t ldz, int n_store) {
    const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (t >= count) return;
    const int i = i0 + t;
    if (cl[i]) return;
    const size_t W32 = (size_t)n * 32;
    const float* Y = scr32 + (size_t)(t >> 5) * 5 * W32 + 4 * W32 + (t & 31);   // row k at Y[k * 32]
    const float sc = scs[t];
    double num = 0, den = 0, fx = 0, fy = 0;
    for (int k = lane; k < n; k += 32) {
        const float xf = Y[(size_t)k * 32] * sc;
        const double x = xf;
        double tk = d[k] * x;
        if (k > 0) tk += e[k - 1] * (double)(Y[(size_t)(k - 1) * 32] * sc);
        if (k + 1 < n) tk += e[k] * (double)(Y[(size_t)(k + 1) * 32] * sc);
        num += x * tk;
        den += (double)(xf * xf);
        if (y32) {
            const float2 yy = y32[k];
            fx += (double)(yy.x * xf);
            fy -= (double)(yy.y * xf);
        }
    }
    num = warp_sum(num);
    den = warp_sum(den);
    fx = warp_sum(fx);
    fy = warp_sum(fy);
    const double inv = 1.0 / sqrt(den);
    if (lane == 0) {
        w[i] = num / den;
        if (f) f[i] = make_double2(fx * inv, fy * inv);
    }
    if (i < n_store) {
        const float invf = (float)inv;
        for (int k = lane; k < n; k += 32) z[(size_t)k + (size_t)i * ldz] = (TZ)(Y[(size_t)k * 32] * sc * invf);
    }
}

template <typename TZ>
__global__ void __launch_bounds__(32) cluster64_kernel(int n, const double* __restrict__ d, const double* __restrict__ e,
                                                       const double* __restrict__ w0, double* __restrict__ w,
                                                       const int* __restrict__ cstart, const int* __restrict__ csize,
                                                       const int* __restrict__ cout, const int64_t* __restrict__ coff,
                                                       int ncl, double tnorm, const double2* __restrict__ y,
                                                     double2* __restrict__ f, TZ* __restrict__ z, int64_t ldz, int n_store,
                                                     double* __restrict__ scr, signed char* __restrict__ piv,
                                                     double* __restrict__ Zall) {
    const int t = blockIdx.x, lane = threadIdx.x;
    if (t >= ncl) return;
    const int s0 = cstart[t], c = csize[t];
    // this cluster's scratch: 5 contiguous arrays of n doubles (lane 0 only) and n pivots
    double* Vr = scr + (size_t)t * 5 * n;
    double* Vb = Vr + n;
    double* Vd = Vb + n;
    double* Vc = Vd + n;
    double* X = Vc + n;
    signed char* pv = piv + (size_t)t * n;
    double* Zc = Zall + coff[t];                       // n x c
    const double pert = 2.220446049250313e-16 * fmax(tnorm, 1e-300);
    double sprev = -1e300;
    for (int j = 0; j < c; j++) {
        const double shift = fmax(w0[s0 + j], sprev + 10.0 * pert);
        sprev = shift;
        if (lane == 0) tri_factor<double, 1, 64>(n, d, e, shift, pert, Vr, Vb, Vd, Vc, pv);
        for (int k = lane; k < n; k += 32) X[k] = start_value(s0 + j, k) - 1.0;
        __syncwarp();
        for (int it = 0; it < 5; it++) {
            if (lane == 0) tri_solve<double, 1, 64>(n, Vr, Vb, Vd, Vc, pv, X, 1.0);
            __syncwarp();
            for (int q = 0; q < j; q++) {               // Gram-Schmidt against earlier members
                const double* zq = Zc + (size_t)q * n;
                double dot = 0;
                for (int k = lane; k < n; k += 32) dot += zq[k] * X[k];
                dot = warp_dsum(dot);
                for (int k = lane; k < n; k += 32) X[k] -= dot * zq[k];
                __syncwarp();
            }
            double nrm = 0;
            for (int k = lane; k < n; k += 32) nrm += X[k] * X[k];
            nrm = warp_dsum(nrm);
            const double inv = nrm > 0 ? 1.0 / sqrt(nrm) : 0.0;
            for (int k = lane; k < n; k += 32) X[k] *= inv;
            __syncwarp();
        }
        for (int k = lane; k < n; k += 32) Zc[k + (size_t)j * n] = X[k];
        __syncwarp();
    }
    // Rayleigh-Ritz inside the cluster: M = Zc^T T Zc (lanes over k), Jacobi on lane 0
    constexpr int CMAX = 32;
    __shared__ double M[CMAX * CMAX], Q[CMAX * CMAX];
    for (int a = 0; a < c; a++)
        for (int b = 0; b <= a; b++) {
            const double* za = Zc + (size_t)a * n;
            const double* zb = Zc + (size_t)b * n;
            double acc = 0;
            for (int k = lane; k < n; k += 32) {
                const double tz = d[k] * zb[k] + (k > 0 ? e[k - 1] * zb[k - 1] : 0.0) + (k + 1 < n ? e[k] * zb[k + 1] : 0.0);
                acc += za[k] * tz;
            }
            acc = warp_dsum(acc);
            if (lane == 0) M[a + b * CMAX] = M[b + a * CMAX] = acc;
        }
    __syncwarp();
    if (lane == 0) {
        for (int a = 0; a < c; a++)
            for (int b = 0; b < c; b++) Q[a + b * CMAX] = a == b ? 1.0 : 0.0;
        for (int sweep = 0; sweep < 30; sweep++) {
            double off = 0;
            for (int a = 0; a < c; a++)
                for (int b = a + 1; b < c; b++) off += M[a + b * CMAX] * M[a + b * CMAX];
            if (off < 1e-60) break;
            for (int p = 0; p < c; p++)
                for (int q = p + 1; q < c; q++) {
                    const double apq = M[p + q * CMAX];
                    if (apq == 0.0) continue;
                    const double tau = (M[q + q * CMAX] - M[p + p * CMAX]) / (2.0 * apq);
                    const double tt = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                    const double cs = 1.0 / sqrt(1.0 + tt * tt), sn = tt * cs;
                    for (int k = 0; k < c; k++) {
                        const double mkp = M[k + p * CMAX], mkq = M[k + q * CMAX];
                        M[k + p * CMAX] = cs * mkp - sn * mkq;
                        M[k + q * CMAX] = sn * mkp + cs * mkq;
                    }
                    for (int k = 0; k < c; k++) {
                        const double mpk = M[p + k * CMAX], mqk = M[q + k * CMAX];
                        M[p + k * CMAX] = cs * mpk - sn * mqk;
                        M[q + k * CMAX] = sn * mpk + cs * mqk;
                    }
                    for (int k = 0; k < c; k++) {
                        const double qkp = Q[k + p * CMAX], qkq = Q[k + q * CMAX];
                        Q[k + p * CMAX] = cs * qkp - sn * qkq;
                        Q[k + q * CMAX] = sn * qkp + cs * qkq;
                    }
                }
        }
    }
    __syncwarp();
    __shared__ int ord[CMAX];
    if (lane == 0) {
        for (int a = 0; a < c; a++) ord[a] = a;
        for (int a = 1; a < c; a++) {
            const int x = ord[a];
            int b = a - 1;
            while (b >= 0 && M[ord[b] * (CMAX + 1)] > M[x * (CMAX + 1)]) { ord[b + 1] = ord[b]; b--; }
            ord[b + 1] = x;
        }
    }
    __syncwarp();
    for (int a = 0; a < c; a++) {
        const int i = s0 + a, col = ord[a];
        if (i < cout[2 * t] || i >= cout[2 * t + 1]) continue;   // guard member
        double fx = 0, fy = 0;
        for (int k = lane; k < n; k += 32) {
            double v = 0;
            for (int b = 0; b < c; b++) v += Zc[k + (size_t)b * n] * Q[b + col * CMAX];
            if (y) {
                fx += y[k].x * v;
                fy -= y[k].y * v;
            }
            if (i < n_store) z[(size_t)k + (size_t)i * ldz] = (TZ)v;
        }
        fx = warp_dsum(fx);
        fy = warp_dsum(fy);
        if (lane == 0) {
            w[i] = M[col * (CMAX + 1)];
            if (f) f[i] = make_double2(fx, fy);
        }
    }
}

// Mixed path: eigenpairs of runs of eigenvalues FP32 bisection cannot separate.  Several
// clusters sit side by side on the lanes of one warp (a warp holds clusters of total size <= 32,
// most runs are pairs); lane j of a cluster's segment runs inverse iteration for member j with its
// own shift, the segment orthonormalises its member vectors after every iteration (Cholesky QR,
// Gram matrix accumulated in FP64) so they cannot collapse onto the member nearest to a shift, and
// a generalised Rayleigh-Ritz step inside the cluster (Jacobi on the c x c projected matrix, FP64)
// gives the eigenpairs.  The iterations run in FP32, as the tridiagonal of the mixed path carries
// FP32 rounding itself.  Members outside [cout[2t], cout[2t+1]) are guards, solved but not written.
// Scratch: interleaved [k][32] arrays per lane group.  A block of kClusterWarps warps serves one
// lane group: warp 0 runs the (sequential) triangular solves, and the warps split the rows of the
// Gram, orthonormalisation and output passes, which are row-parallel.  One warp per block: the
// sequential sweeps set the pace, and with one warp per lane group an SM runs several groups'
// sweeps at once instead of one group's sweep while the other warps wait at a barrier.
constexpr int CMAX = 32;
constexpr int kClusterWarps = 1;

// (hi, lo) += v: Knuth's TwoSum keeps the rounding error of each addition in lo (FP32 adds; FP64
// adds run at a small fraction of the FP32 rate on this part).  hi + lo carries ~48 bits.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float v) {
    const float s = __fadd_rn(hi, v);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp));
    hi = s;
    lo = __fadd_rn(lo, err);
}

// this warp's share of rows [kb, ke) of the block's row-parallel passes (multiples of 16 rows)
__device__ __forceinline__ void warp_rows(int n, int& kb, int& ke) {
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int per = ((n + nw - 1) / nw + 15) / 16 * 16;
    kb = min(n, wid * per);
    ke = min(n, kb + per);
}

// out[b][a] = sum_k u_b(k) z_a(k) over the columns z_a = X[k * 32 + a] of lane b's segment
// [slo, slo + sc); lane b accumulates row b; u = z (Gram matrix) or u = T z (projected T).
// The row-parallel passes read every row of the lane group's 32 columns in every lane: the rows of a
// chunk of 16 are staged in a per-warp shared tile (row q at tile[32 q ..]) and read back as
// float4 broadcasts, 8 loads per row where a shuffle per column took 32.
__device__ __forceinline__ void stage_tile(float* tile, const float (&v)[16]) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 16; q++) tile[q * 32 + lane] = v[q];
    __syncwarp();
}

// FP32 partial sums over 16 rows go into compensated FP32 (hi, lo) pairs, added into out in FP64.
// The block's warps split the rows and add their partial sums into out one warp after the other;
// every thread of the block calls this.
template <typename F, bool APPLY_T>
__device__ void cluster_gram(int n, int slo, int sc, const F* __restrict__ X, const F* __restrict__ d,
                             const F* __restrict__ e, double* __restrict__ out, float* tile) {
    static_assert(sizeof(F) == sizeof(float), "FP32 lane groups");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int kb, ke;
    warp_rows(n, kb, ke);
    float acc[CMAX], accl[CMAX];
#pragma unroll
    for (int a = 0; a < CMAX; a++) acc[a] = accl[a] = 0.0f;
    F zprev = (APPLY_T && kb > 0 && kb < n) ? X[(size_t)(kb - 1) * 32] : F(0);
    for (int k0 = kb; k0 < ke; k0 += 16) {
        // the chunk's rows (and one row ahead for T z) are loaded before any is used, so the
        // loads are in flight together instead of one dependent load per row
        F zb[17], db[16], eb[17];
#pragma unroll
        for (int q = 0; q < 17; q++) {
            const int k = k0 + q;
            zb[q] = k < n ? X[(size_t)k * 32] : F(0);
            if (APPLY_T) {
                if (q < 16) db[q] = k < n ? d[k] : F(0);
                eb[q] = k < n - 1 ? e[k] : F(0);
            }
        }
        const F eprev = (APPLY_T && k0 > 0) ? e[k0 - 1] : F(0);
        F part[CMAX];
#pragma unroll
        for (int a = 0; a < CMAX; a++) part[a] = 0;
        {
            float zt[16];
#pragma unroll
            for (int q = 0; q < 16; q++) zt[q] = zb[q];
            stage_tile(tile, zt);
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
            if (k0 + q < ke) {
                const F zc = zb[q];
                F u = zc;
                if (APPLY_T) u = db[q] * zc + (q > 0 ? eb[q - 1] : eprev) * zprev + eb[q] * zb[q + 1];
                const float4* row = reinterpret_cast<const float4*>(tile + q * 32);
#pragma unroll
                for (int a4 = 0; a4 < CMAX / 4; a4++) {
                    const float4 v = row[a4];
                    part[4 * a4] += u * v.x;
                    part[4 * a4 + 1] += u * v.y;
                    part[4 * a4 + 2] += u * v.z;
                    part[4 * a4 + 3] += u * v.w;
                }
                zprev = zc;
            }
        }
#pragma unroll
        for (int a = 0; a < CMAX; a++) two_sum_acc(acc[a], accl[a], (float)part[a]);
    }
    for (int wq = 0; wq < nw; wq++) {
        if (wid == wq)
#pragma unroll
            for (int a = 0; a < CMAX; a++)
                if (sc > 0 && a >= slo && a < slo + sc)
                    out[lane * CMAX + a] = (wq == 0 ? 0.0 : out[lane * CMAX + a]) + ((double)acc[a] + (double)accl[a]);
        __syncthreads();
    }
}

// Cholesky G = R^T R in place (R upper, row-major, row stride CMAX); a pivot below 1e-10 of its
// diagonal entry (a column numerically inside the span of the earlier ones) is raised to that
// level, so the column comes out short instead of blowing up and the next iteration refills it.
__device__ void chol_upper(int c, double* G) {
    for (int j = 0; j < c; j++) {
        const double g0 = G[j * CMAX + j];
        double djj = g0;
        for (int q = 0; q < j; q++) djj -= G[q * CMAX + j] * G[q * CMAX + j];
        djj = sqrt(fmax(djj, 1e-10 * fmax(g0, 1e-300)));
        G[j * CMAX + j] = djj;
        for (int b = j + 1; b < c; b++) {
            double v = G[j * CMAX + b];
            for (int q = 0; q < j; q++) v -= G[q * CMAX + j] * G[q * CMAX + b];
            G[j * CMAX + b] = v / djj;
        }
    }
}

// Rinv = R^{-1} (upper), row-major.
__device__ void inv_upper(int c, const double* R, double* Rinv) {
    for (int jc = 0; jc < c; jc++) {
        for (int r = jc; r >= 0; r--) {
            double v = r == jc ? 1.0 : 0.0;
            for (int q = r + 1; q <= jc; q++) v -= R[r * CMAX + q] * Rinv[q * CMAX + jc];
            Rinv[r * CMAX + jc] = v / R[r * CMAX + r];
        }
        for (int r = jc + 1; r < c; r++) Rinv[r * CMAX + jc] = 0;
    }
}

// Orthonormalise each segment's columns X[k * 32 + lane]: X <- X R^{-1} with G = R^T R, the
// segment's first lane in warp 0 factoring its diagonal block; rows split over the block's warps.
template <typename F>
__device__ void cluster_cholqr(int n, int slo, int sc, F* __restrict__ X, double* __restrict__ Gs,
                               double* __restrict__ Rinv, float* tile) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    cluster_gram<F, false>(n, slo, sc, X, (const F*)nullptr, (const F*)nullptr, Gs, tile);
    if (wid == 0 && sc > 0 && lane == slo) {
        chol_upper(sc, Gs + slo * (CMAX + 1));
        inv_upper(sc, Gs + slo * (CMAX + 1), Rinv + slo * (CMAX + 1));
    }
    __syncthreads();
    F rcol[CMAX];
#pragma unroll
    for (int a = 0; a < CMAX; a++) rcol[a] = (sc > 0 && a >= slo && a <= lane) ? (F)Rinv[a * CMAX + lane] : F(0);
    int kb, ke;
    warp_rows(n, kb, ke);
    for (int k0 = kb; k0 < ke; k0 += 16) {
        float xb[16];
#pragma unroll
        for (int q = 0; q < 16; q++) xb[q] = k0 + q < ke ? X[(size_t)(k0 + q) * 32] : F(0);
        stage_tile(tile, xb);
#pragma unroll
        for (int q = 0; q < 16; q++) {
            if (k0 + q < ke) {
                const float4* row = reinterpret_cast<const float4*>(tile + q * 32);
                F v = 0;
#pragma unroll
                for (int a4 = 0; a4 < CMAX / 4; a4++) {
                    const float4 x = row[a4];
                    v += x.x * rcol[4 * a4] + x.y * rcol[4 * a4 + 1] + x.z * rcol[4 * a4 + 2] + x.w * rcol[4 * a4 + 3];
                }
                if (sc > 0) X[(size_t)(k0 + q) * 32] = v;
            }
        }
    }
    __threadfence();
    __syncthreads();
}

// FP32 counterparts of chol_upper / inv_upper (same layout and pivot floor)
__device__ void chol_upper_f(int c, float* G) {
    for (int j = 0; j < c; j++) {
        const float g0 = G[j * CMAX + j];
        float djj = g0;
        for (int q = 0; q < j; q++) djj -= G[q * CMAX + j] * G[q * CMAX + j];
        djj = sqrtf(fmaxf(djj, 1e-10f * fmaxf(g0, 1e-30f)));
        G[j * CMAX + j] = djj;
        for (int b = j + 1; b < c; b++) {
            float v = G[j * CMAX + b];
            for (int q = 0; q < j; q++) v -= G[q * CMAX + j] * G[q * CMAX + b];
            G[j * CMAX + b] = v / djj;
        }
    }
}
__device__ void inv_upper_f(int c, const float* R, float* Rinv) {
    for (int jc = 0; jc < c; jc++) {
        for (int r = jc; r >= 0; r--) {
            float v = r == jc ? 1.0f : 0.0f;
            for (int q = r + 1; q <= jc; q++) v -= R[r * CMAX + q] * Rinv[q * CMAX + jc];
            Rinv[r * CMAX + jc] = v / R[r * CMAX + r];
        }
        for (int r = jc + 1; r < c; r++) Rinv[r * CMAX + jc] = 0;
    }
}

// Rayleigh-Ritz inside a cluster of the mixed path (one lane), in FP32: M q = theta S q with
// S = Gs = Z^T Z = R^T R, cyclic Jacobi on R^{-T} M R^{-1} until the off-diagonal part is below
// FP32 resolution.  Z is FP32 and T is the FP32 tridiagonal, so the entries of M carry errors of a
// few eps32 |T| already; FP32 arithmetic adds errors of the same size, where FP64 (a small
// fraction of the FP32 rate on this part) made this step the most expensive of the cluster solve.
// Inputs Gs, M: this segment's block, row stride CMAX (FP64, as the Gram passes write them).
// Scratch Sf, Rf; outputs Mf (column-major, diagonal = theta), Qf (column-major, the coefficient
// vectors R^{-1} q'), ord (ascending theta).  All float arrays at the segment's block offset.
__device__ void cluster_rr32(int c, const double* Gs, const double* M, float* Sf, float* Rf, float* Mf, float* Qf,
                             int* ord) {
    for (int a = 0; a < c; a++)
        for (int b = 0; b < c; b++) {
            Sf[a * CMAX + b] = (float)Gs[a * CMAX + b];
            Mf[a * CMAX + b] = (float)(0.5 * (M[a * CMAX + b] + M[b * CMAX + a]));
        }
    chol_upper_f(c, Sf);
    inv_upper_f(c, Sf, Rf);
    for (int a = 0; a < c; a++)            // Qf = Mf Rf (row-major scratch)
        for (int b = 0; b < c; b++) {
            float v = 0;
            for (int q = 0; q <= b; q++) v += Mf[a * CMAX + q] * Rf[q * CMAX + b];
            Qf[a * CMAX + b] = v;
        }
    for (int a = 0; a < c; a++)            // Sf = Rf^T Qf (column-major)
        for (int b = 0; b < c; b++) {
            float v = 0;
            for (int q = 0; q <= a; q++) v += Rf[q * CMAX + a] * Qf[q * CMAX + b];
            Sf[a + b * CMAX] = v;
        }
    for (int a = 0; a < c; a++)
        for (int b = 0; b < c; b++) {
            Mf[a + b * CMAX] = a == b ? Sf[a + a * CMAX] : 0.5f * (Sf[a + b * CMAX] + Sf[b + a * CMAX]);
            Qf[a + b * CMAX] = a == b ? 1.0f : 0.0f;
        }
    for (int sweep = 0; sweep < 30; sweep++) {
        float off = 0, dg = 0;
        for (int a = 0; a < c; a++) {
            dg += Mf[a + a * CMAX] * Mf[a + a * CMAX];
            for (int b = a + 1; b < c; b++) off += Mf[a + b * CMAX] * Mf[a + b * CMAX];
        }
        if (off == 0.0f || off <= 1e-16f * dg) break;
        for (int p = 0; p < c; p++)
            for (int q = p + 1; q < c; q++) {
                const float apq = Mf[p + q * CMAX];
                // below FP32 resolution of the diagonal: zero, no rotation (so the sweeps end)
                if (fabsf(apq) <= 5.9604645e-8f * (fabsf(Mf[p + p * CMAX]) + fabsf(Mf[q + q * CMAX]))) {
                    Mf[p + q * CMAX] = Mf[q + p * CMAX] = 0.0f;
                    continue;
                }
                const float tau = (Mf[q + q * CMAX] - Mf[p + p * CMAX]) / (2.0f * apq);
                const float tt = (tau >= 0 ? 1.0f : -1.0f) / (fabsf(tau) + sqrtf(1.0f + tau * tau));
                const float cs = 1.0f / sqrtf(1.0f + tt * tt), sn = tt * cs;
                for (int k = 0; k < c; k++) {
                    const float mkp = Mf[k + p * CMAX], mkq = Mf[k + q * CMAX];
                    Mf[k + p * CMAX] = cs * mkp - sn * mkq;
                    Mf[k + q * CMAX] = sn * mkp + cs * mkq;
                }
                for (int k = 0; k < c; k++) {
                    const float mpk = Mf[p + k * CMAX], mqk = Mf[q + k * CMAX];
                    Mf[p + k * CMAX] = cs * mpk - sn * mqk;
                    Mf[q + k * CMAX] = sn * mpk + cs * mqk;
                }
                for (int k = 0; k < c; k++) {
                    const float qkp = Qf[k + p * CMAX], qkq = Qf[k + q * CMAX];
                    Qf[k + p * CMAX] = cs * qkp - sn * qkq;
                    Qf[k + q * CMAX] = sn * qkp + cs * qkq;
                }
            }
    }
    for (int a = 0; a < c; a++)            // Qf <- Rf Qf (through Sf)
        for (int b = 0; b < c; b++) {
            float v = 0;
            for (int q = a; q < c; q++) v += Rf[a * CMAX + q] * Qf[q + b * CMAX];
            Sf[a + b * CMAX] = v;
        }
    for (int a = 0; a < c; a++)
        for (int b = 0; b < c; b++) Qf[a + b * CMAX] = Sf[a + b * CMAX];
    for (int a = 0; a < c; a++) ord[a] = a;
    for (int a = 1; a < c; a++) {
        const int x = ord[a];
        int b = a - 1;
        while (b >= 0 && Mf[ord[b] * (CMAX + 1)] > Mf[x * (CMAX + 1)]) { ord[b + 1] = ord[b]; b--; }
        ord[b + 1] = x;
    }
}

template <typename TZ>
__global__ void __launch_bounds__(32 * kClusterWarps) cluster_kernel(int n, const float* __restrict__ df, const float* __restrict__ ef,
                                                     const double* __restrict__ w0, double* __restrict__ w,
                                                     const int* __restrict__ cstart, const int* __restrict__ csize,
                                                     const int* __restrict__ cout, const int* __restrict__ wfirst,
                                                     int wbase, double tnorm, const float2* __restrict__ y,
                                                     double2* __restrict__ f, TZ* __restrict__ z, int64_t ldz,
                                                     int n_store, float* __restrict__ scr32, signed char* __restrict__ piv) {
    __shared__ double Gs[CMAX * CMAX], Rinv[CMAX * CMAX], M[CMAX * CMAX], Q[CMAX * CMAX];
    __shared__ double fred[kClusterWarps][32][2];
    __shared__ int ord[CMAX];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // this block's clusters sit side by side on the lanes; find this lane's cluster and segment
    const int t_end = wfirst[wbase + blockIdx.x + 1];
    int t = -1, slo = 0, sc = 0;
    for (int q = wfirst[wbase + blockIdx.x], off = 0; q < t_end; q++) {
        const int cq = csize[q];
        if (lane >= off && lane < off + cq) {
            t = q;
            slo = off;
            sc = cq;
        }
        off += cq;
    }
    const bool act = t >= 0;
    const int s0 = act ? cstart[t] : 0, m = lane - slo;
    const size_t W32 = (size_t)n * 32;
    extern __shared__ float stage_sm[];
    float* Urw = scr32 + (size_t)blockIdx.x * 5 * W32;
    float* Ubw = Urw + W32;
    float* Udw = Ubw + W32;
    float* Lcw = Udw + W32;
    float* Yw = Lcw + W32;
    signed char* pvw = piv + (size_t)blockIdx.x * W32;
    float* Y = Yw + lane;
    // the passes' row tiles (16 rows x 32 floats per warp) live in the staging area between sweeps
    float* tile = stage_sm + wid * 16 * 32;
    const float pert32 = 1.1920929e-7f * (float)fmax(tnorm, 1e-30);
    const double pert = 2.220446049250313e-16 * fmax(tnorm, 1e-300);
    // shifts: the FP32 estimates in increasing order within each cluster (distinct start vectors
    // and the orthonormalisation keep the members apart, so the shifts may coincide)
    double sh = act ? w0[s0 + m] : 0.0;
    for (int j = 1; j < 32; j++) {
        const double prev = __shfl_sync(0xffffffffu, sh, j - 1);
        if (lane == j && act && m > 0) sh = fmax(sh, prev + 10.0 * pert);
    }
    // warp 0 runs the factor and the solves (lanes without a member factor T itself and solve
    // with a zero right-hand side); the other warps help with the row-parallel passes
    if (wid == 0) tri_factor_staged(n, df, ef, (float)sh, pert32, Urw, Ubw, Udw, Lcw, pvw, stage_sm);
    int kb, ke;
    warp_rows(n, kb, ke);
    for (int k = kb; k < ke; k++) Y[(size_t)k * 32] = act ? start_value32(s0 + m, k) - 1.0f : 0.0f;
    __threadfence();
    __syncthreads();
    for (int it = 0; it < 3; it++) {
        if (wid == 0) tri_solve_staged(n, Urw, Ubw, Udw, Lcw, pvw, Yw, 1.0f, stage_sm);
        __syncthreads();
        cluster_cholqr<float>(n, slo, sc, Y, Gs, Rinv, tile);
    }
    cluster_gram<float, false>(n, slo, sc, Y, df, ef, Gs, tile);
    cluster_gram<float, true>(n, slo, sc, Y, df, ef, M, tile);
    const int blk = slo * (CMAX + 1);
    // FP32 scratch of the Rayleigh-Ritz step in the FP64 arrays Rinv and Q, which no segment reads
    // after the orthonormalisation (every segment keeps to its own block of each array)
    float* Sf = reinterpret_cast<float*>(Rinv);
    float* Rf = Sf + CMAX * CMAX;
    float* Mf = reinterpret_cast<float*>(Q);
    float* Qf = Mf + CMAX * CMAX;
    if (wid == 0 && act && lane == slo)
        cluster_rr32(sc, Gs + blk, M + blk, Sf + blk, Rf + blk, Mf + blk, Qf + blk, ord + slo);
    __syncthreads();
    // member m (lane slo + m) = Z Q[:, ord[m]] of its segment, in FP32 (Z is FP32; FP64 arithmetic
    // is slow on this part); f = y^H z with FP64 sums of FP32 products
    float qcol[CMAX];
    const int col = act ? slo + ord[slo + m] : 0;
#pragma unroll
    for (int b = 0; b < CMAX; b++) qcol[b] = (act && b >= slo && b < slo + sc) ? Qf[b + col * CMAX] : 0.0f;
    const int i = s0 + m;
    const bool outp = act && i >= cout[2 * t] && i < cout[2 * t + 1];
    const bool keep = outp && i < n_store;
    float fx = 0, fxl = 0, fy = 0, fyl = 0;   // compensated sums of the FP32 products
    for (int k0 = kb; k0 < ke; k0 += 16) {
        float yb[16];
#pragma unroll
        for (int q = 0; q < 16; q++) yb[q] = k0 + q < ke ? Y[(size_t)(k0 + q) * 32] : 0.0f;
        stage_tile(tile, yb);
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int k = k0 + q;
            if (k < ke) {
                const float4* row = reinterpret_cast<const float4*>(tile + q * 32);
                float v = 0;
#pragma unroll
                for (int b4 = 0; b4 < CMAX / 4; b4++) {
                    const float4 x = row[b4];
                    v += x.x * qcol[4 * b4] + x.y * qcol[4 * b4 + 1] + x.z * qcol[4 * b4 + 2] + x.w * qcol[4 * b4 + 3];
                }
                if (y && outp) {
                    const float2 yy = y[k];
                    two_sum_acc(fx, fxl, yy.x * v);
                    two_sum_acc(fy, fyl, -(yy.y * v));
                }
                if (keep) z[(size_t)k + (size_t)i * ldz] = (TZ)v;
            }
        }
    }
    fred[wid][lane][0] = (double)fx + (double)fxl;
    fred[wid][lane][1] = (double)fy + (double)fyl;
    __syncthreads();
    if (wid == 0 && outp) {
        double sx = 0, sy = 0;
        for (int q = 0; q < kClusterWarps; q++) {
            sx += fred[q][lane][0];
            sy += fred[q][lane][1];
        }
        w[i] = (double)Mf[col * (CMAX + 1)];
        if (f) f[i] = make_double2(sx, sy);
    }
}

// Back-transformation X <- Q X, Q = H_0 H_1 ... H_{n-2}, in panels of kWY reflectors.  Panel p
// holds reflectors k0 = kWY p .. k0+nb-1 and acts on rows k0+1 .. n-1 (m_p = n-1-k0 of them);
// V[r][i] = 0 above row k0+i+1, 1 at row k0+i+1, A[r, k0+i] below.  With U = diag(1/tau_i) +
// striu(V^H V) (the "UT transform" form of compact WY: U^{-1} is zlarft's T),
//     Q_p = H_k0 ... H_{k0+nb-1} = I - V U^{-1} V^H,
// so X[k0+1:] -= V (U^{-1} (V^H X[k0+1:])) costs two GEMMs and a triangular solve per panel.
// A reflector with tau = 0 is the identity: its column of V is set to zero and U_ii = 1.
constexpr int kWY = 256;

template <typename T2>
__device__ __forceinline__ T2 vpanel(const T2* __restrict__ A, int64_t lda, int k0, int i, int r) {
    const int top = k0 + i + 1;
    if (r < top) return C2<T2>(0, 0);
    if (r == top) return C2<T2>(1, 0);
    return A[r + (int64_t)(k0 + i) * lda];
}

// Offset of panel p in the explicit panel array: kWY * sum_{q<p} m_q with m_q = n - 1 - kWY q.
__host__ __device__ __forceinline__ int64_t vpanel_offset(int n, int p) {
    return kWY * ((int64_t)p * (n - 1) - kWY * (int64_t)p * (p - 1) / 2);
}

// Explicit panels, column-major with leading dimension m_p; reflectors past nb are zero.
// Grid (row blocks, kWY / 8 column groups, panels).
template <typename T2>
__global__ void __launch_bounds__(256) build_vpanels_kernel(int n, const T2* __restrict__ A, int64_t lda, const T2* __restrict__ tau,
                                                            T2* __restrict__ V) {
    const int p = blockIdx.z, k0 = kWY * p, m = n - 1 - k0, nb = min(kWY, m);
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    T2* Vp = V + vpanel_offset(n, p);
    for (int i = 8 * blockIdx.y; i < 8 * blockIdx.y + 8; i++) {
        const bool live = i < nb && (tau[k0 + i].x != 0 || tau[k0 + i].y != 0);
        Vp[r + (int64_t)i * m] = live ? vpanel(A, lda, k0, i, k0 + 1 + r) : C2<T2>(0, 0);
    }
}

// U of every panel from its Gram matrix (strict upper triangle from herk): diagonal 1/tau_i
// (1 for tau_i = 0 and for the padding past nb), strict upper triangle kept, lower part zero.
template <typename T2>
__global__ void ut_diag_kernel(int n, int npanel, const T2* __restrict__ tau, T2* __restrict__ U) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)npanel * kWY * kWY) return;
    const int p = (int)(t / ((int64_t)kWY * kWY)), e = (int)(t % ((int64_t)kWY * kWY));
    const int j = e % kWY, i = e / kWY;   // row j, column i (column-major)
    const int k = kWY * p + i, nb = min(kWY, n - 1 - kWY * p);
    if (j > i) {
        U[t] = C2<T2>(0, 0);
    } else if (j == i) {
        const bool live = i < nb && (tau[k].x != 0 || tau[k].y != 0);
        U[t] = live ? cinv(tau[k]) : C2<T2>(1, 0);
    }
}

// X[r + j ldx] -= D[r + j m] for the m x ncol block (FP64 back-transformation)
__global__ void sub_block_kernel(int m, int ncol, const double2* __restrict__ D, double2* __restrict__ X, int64_t ldx) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * ncol) return;
    const int r = (int)(t % m), j = (int)(t / m);
    double2 x = X[r + (int64_t)j * ldx];
    x.x -= D[t].x;
    x.y -= D[t].y;
    X[r + (int64_t)j * ldx] = x;
}

template <typename T2>
__global__ void real_to_complex_kernel(int64_t n, const typename Real<T2>::t* __restrict__ in, T2* __restrict__ out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) out[t] = C2<T2>(in[t], 0);
}

template <typename R>
__global__ void tri_prepare_kernel(int n, const R* __restrict__ d, const R* __restrict__ e, double* __restrict__ dd,
                                   double* __restrict__ ee, double* __restrict__ e2, float* __restrict__ df,
                                   float* __restrict__ e2f, float* __restrict__ ef) {
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
        ef[t] = (float)x;
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

// above this order the two-stage reduction (band.cu) replaces the one-stage tridiag_kernel
constexpr int kTwoStageMin = 8192;

template <typename T2>
int own_heevd_t(bse_ctx* c, int n, T2* A, int64_t lda, double* dW, int n_vec, const double2* rho0, double2* f_out,
                bool nested) {
    typedef typename Real<T2>::t R;
    int st;
    int dev = c->device, nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // nested FP64 solves are small and bound by FP64 instruction throughput: 4 warps per block keep
    // the per-block work (every block forms the reflector) low
    const int threads = nested ? 128 : 512;
    // tuning overrides (sweeps): BSE_TRIDIAG_BLOCKS (grid size) and BSE_TRIDIAG_TR (tile rows)
    int TR = std::min(4096, std::max(256, (n + 255) / 256 * 256));   // one tile for n <= 4096
    if (const char* v = std::getenv("BSE_TRIDIAG_TR")) TR = std::max(64, std::min(4096, std::atoi(v)));
    const size_t smem = 3 * (size_t)TR * sizeof(T2) + 4 * 32 * sizeof(R);
    int per_sm = 0;
    // the attribute is process-wide: set it once, to the largest tile any call uses (TR <= 4096),
    // so concurrent contexts with different sizes never shrink it under each other
    static std::once_flag smem_once;
    static cudaError_t smem_err = cudaSuccess;
    std::call_once(smem_once, [] {
        const int smax = 3 * 4096 * (int)sizeof(T2) + 4 * 32 * (int)sizeof(R);
        smem_err = cudaFuncSetAttribute(tridiag_kernel<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    });
    if ((st = cuda_check(c, smem_err, "tridiag smem"))) return st;
    static std::once_flag stage_once;
    static cudaError_t stage_err = cudaSuccess;
    std::call_once(stage_once, [] {
        stage_err = cudaFuncSetAttribute(invit_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageSmem);
        if (stage_err == cudaSuccess)
            stage_err = cudaFuncSetAttribute(cluster_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageSmem);
    });
    if ((st = cuda_check(c, stage_err, "inverse-iteration smem"))) return st;
    if ((st = cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tridiag_kernel<T2>, threads, smem), "occupancy"))) return st;
    if (per_sm < 1) return fail(c, BSE_ERR_CUDA, "tridiagonal kernel does not fit on an SM");
    // one block per SM (16 warps of loads in flight each) once the matrix is large enough; small
    // matrices (batched runs) use ~n/15 blocks so several models' reductions can share the GPU;
    // a nested FP64 solve runs alone and is bound by FP64 arithmetic (slow on this part), so it
    // spreads the trailing columns over up to one block per SM
    int B = std::max(4, std::min(nsm, (n + 14) / 15));
    if (nested) B = std::max(4, std::min(nsm, n / 2));
    if (const char* v = std::getenv("BSE_TRIDIAG_BLOCKS")) B = std::max(1, std::min(nsm * per_sm, std::atoi(v)));
    const int nt_max = (n + TR - 1) / TR;
    // inverse-iteration batch: per (eigenvalue, row) 21 bytes of FP32 scratch, plus 40 bytes of FP64
    // scratch in the FP64 path; the mixed path takes batches of up to 32768 eigenvalues (24 GB), so
    // at large n every SM holds several warps of the latency-bound sweeps
    const bool fp64 = sizeof(T2) == sizeof(double2);
    const int count_max = fp64 ? std::min(n, std::max(32 * nsm, (int)std::min<int64_t>(8192, (int64_t)(12e9 / (61.0 * n)))))
                               : std::min(n, std::max(32 * nsm, (int)std::min<int64_t>(32768, (int64_t)(24e9 / (21.0 * n)))));
    // workspace
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    const size_t o_d = carve(n * sizeof(R)), o_e = carve(n * sizeof(R)), o_tau = carve(n * sizeof(T2));
    // one barrier per reflector while every block can afford to finish all column sums itself;
    // BSE_TRIDIAG_MODE=shared|redundant overrides (tests run the large-n path at small n)
    // BSE_TRIDIAG_MODE=shared|redundant|twostage overrides (tests run every path at small n)
    // BSE_TRIDIAG_MODE=fused|shared|redundant|twostage overrides (tests run every path at small n)
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t fused_max = optin > 2048 ? (size_t)optin - 1024 : 0;   // room for the barrier's static word
    bool redundant = n <= 8192;
    bool two_stage = n > kTwoStageMin;
    bool fused = !two_stage && fused_smem<T2>(n, rho0 != nullptr, B) <= fused_max;
    if (const char* mode = std::getenv("BSE_TRIDIAG_MODE")) {
        const std::string md(mode);
        if (md == "shared") redundant = two_stage = fused = false;
        else if (md == "redundant") { redundant = true; two_stage = fused = false; }
        else if (md == "twostage") { redundant = fused = false; two_stage = n >= 3; }
        else if (md == "fused" && fused_smem<T2>(n, rho0 != nullptr, B) <= fused_max) { fused = true; two_stage = false; }
    }
    if (two_stage || fused) redundant = false;
    const size_t nbuf = (two_stage || fused) ? 0 : (redundant ? (size_t)B : 2);
    const size_t o_v = carve(nbuf * n * sizeof(T2)), o_p = carve(nbuf * n * sizeof(T2));
    const int64_t ppstride = (int64_t)(fused ? 1 : nt_max) * n;
    const size_t o_pp = carve(two_stage ? 0 : 2 * (size_t)ppstride * sizeof(T2)), o_dp = carve(2 * (size_t)B * sizeof(T2));
    const size_t o_y = carve((redundant ? (size_t)B : 1) * n * sizeof(T2)), o_bar = carve(64);
    const size_t o_flags = carve((size_t)B * 128);
    const size_t o_band = carve(two_stage ? band_workspace(n, fp64, n_vec > 0, n_vec, nsm) : 0);
    // FP32 copies padded by 8 floats: the staged sweeps copy them in 16-byte pieces
    const size_t o_dd = carve(n * 8), o_ee = carve(n * 8), o_e2 = carve(n * 8), o_df = carve((n + 8) * 4),
                 o_e2f = carve(n * 4);
    const size_t o_ef = carve((n + 8) * 4), o_cl = carve(n);
    const size_t o_y64 = carve(n * sizeof(double2));
    const size_t cpad = (size_t)(count_max + 31) / 32 * 32;   // whole warps of scratch
    const size_t o_scr = carve(fp64 ? 5 * (size_t)n * cpad * 8 : 0), o_scr32 = carve(5 * (size_t)n * cpad * 4);
    const size_t o_piv = carve((size_t)n * cpad), o_scs = carve((size_t)cpad * sizeof(float));
    const size_t o_z = carve((size_t)n * std::max(n_vec, 1) * sizeof(R));
    // nested solves keep the context arena (it holds the caller's buffers) and use their own
    // stream-ordered workspace, released on every return path
    struct StreamBuf {
        void* p;
        cudaStream_t s;
        ~StreamBuf() { if (p) cudaFreeAsync(p, s); }
    } priv{nullptr, c->stream};
    if (nested) {
        if ((st = cuda_check(c, cudaMallocAsync(&priv.p, off, c->stream), "nested eigensolver workspace"))) return st;
    } else if ((st = ensure_work(c, off))) {
        return st;
    }
    char* w = nested ? (char*)priv.p : (char*)c->d_work;
    R* d = (R*)(w + o_d);
    R* e = (R*)(w + o_e);
    T2* tau = (T2*)(w + o_tau);
    T2* y = rho0 ? (T2*)(w + o_y) : nullptr;
    unsigned* bar = (unsigned*)(w + o_bar);
    unsigned* flags = (unsigned*)(w + o_flags);
    int* err = (int*)(w + o_bar + 16);
    if ((st = cuda_check(c, cudaMemsetAsync(bar, 0, 64, c->stream), "barrier reset"))) return st;
    if (c->spin_limit &&
        (st = cuda_check(c, cudaMemcpyAsync(err + 1, &c->spin_limit, sizeof(unsigned), cudaMemcpyHostToDevice, c->stream),
                         "polling limit")))
        return st;
    if ((st = cuda_check(c, cudaMemsetAsync(flags, 0, (size_t)B * 128, c->stream), "barrier flags reset"))) return st;
    if ((st = cuda_check(c, cudaMemsetAsync(w + o_v, 0, nbuf * n * sizeof(T2), c->stream), "v reset"))) return st;
    if ((st = cuda_check(c, cudaMemsetAsync(w + o_p, 0, nbuf * n * sizeof(T2), c->stream), "p reset"))) return st;
    if ((st = cuda_check(c, cudaMemsetAsync(tau, 0, n * sizeof(T2), c->stream), "tau reset"))) return st;
    if (y) {
        // redundant mode: one copy per block (identical updates), block 0's copy is read back
        for (int bb = 0; bb < (redundant ? B : 1); bb++)
            rho_to_y_kernel<T2><<<(n + 255) / 256, 256, 0, c->stream>>>(n, rho0, y + (size_t)bb * n);
        c->launches += redundant ? B : 1;
    }
    TriArgs<T2> ta;
    ta.n = n; ta.A = A; ta.lda = lda; ta.d = d; ta.e = e; ta.tau = tau;
    ta.vbuf = (T2*)(w + o_v); ta.pbuf = (T2*)(w + o_p); ta.ppart = (T2*)(w + o_pp); ta.dpart = (T2*)(w + o_dp);
    ta.y = y; ta.bar = bar; ta.flags = flags; ta.err = err; ta.TR = TR; ta.redundant = redundant ? 1 : 0; ta.ppstride = ppstride;
    void* kargs[] = {&ta};
    stage_begin(c, 8);
    if (two_stage) {
        if ((st = band_tridiag(c, n, A, lda, fp64, d, e, y, n_vec > 0, w + o_band, bar, err, n_vec))) return st;
    } else if (fused) {
        static std::once_flag fused_once;
        static cudaError_t fused_err = cudaSuccess;
        std::call_once(fused_once, [fused_max] {
            fused_err = cudaFuncSetAttribute(tridiag_fused_kernel<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_max);
        });
        if ((st = cuda_check(c, fused_err, "fused tridiagonal smem"))) return st;
        const size_t fsm = fused_smem<T2>(n, y != nullptr, B);
        int fper = 0;
        if ((st = cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fper, tridiag_fused_kernel<T2>, threads, fsm), "occupancy"))) return st;
        if (fper < 1 || B > nsm * fper) return fail(c, BSE_ERR_CUDA, "fused tridiagonal kernel does not fit on the GPU");
        const int FB = B;
        if ((st = cuda_check(c, cudaLaunchCooperativeKernel((void*)tridiag_fused_kernel<T2>, dim3(FB), dim3(threads), kargs, fsm,
                                                            c->stream), "tridiagonal kernel launch"))) return st;
        c->launches++;
    } else {
        if ((st = cuda_check(c, cudaLaunchCooperativeKernel((void*)tridiag_kernel<T2>, dim3(B), dim3(threads), kargs, smem,
                                                            c->stream), "tridiagonal kernel launch"))) return st;
        c->launches++;
    }
    stage_end(c, 8);
    // T in FP64 / FP32 copies for the bisection and inverse iteration
    double* dd = (double*)(w + o_dd);
    double* ee = (double*)(w + o_ee);
    double* e2 = (double*)(w + o_e2);
    float* df = (float*)(w + o_df);
    float* e2f = (float*)(w + o_e2f);
    float* ef = (float*)(w + o_ef);
    tri_prepare_kernel<R><<<(n + 255) / 256, 256, 0, c->stream>>>(n, d, e, dd, ee, e2, df, e2f, ef);
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
    signed char* cl = (signed char*)(w + o_cl);
    stage_begin(c, 9);
    {
        // lanes per eigenvalue: enough threads to hold ~16 warps per SM, at most a warp
        int lp = 0;
        while (!fp64 && lp < 5 && (int64_t)n * (2 << lp) <= (int64_t)nsm * 512) lp++;
        const int P = 1 << lp;
        const int rounds = (int)std::ceil(40.0 / std::log2((double)P + 1.0)) + 2;
        const int64_t threads = ((int64_t)n * P + 255) / 256 * 256;
        if (fp64)
            bisect32_kernel<false><<<(unsigned)(threads / 256), 256, 0, c->stream>>>(n, lp, rounds, df, e2f, (float)glo, (float)ghi, pivminf, dW);
        else
            bisect32_kernel<true><<<(unsigned)(threads / 256), 256, 0, c->stream>>>(n, lp, rounds, df, e2f, (float)glo, (float)ghi, pivminf, dW);
    }
    c->launches++;
    // clusters: runs of eigenvalues closer than FP32 bisection can resolve
    std::vector<double> hw(n);
    if ((st = cuda_check(c, cudaMemcpyAsync(hw.data(), dW, n * 8, cudaMemcpyDeviceToHost, c->stream), "w32"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "bisection"))) return st;
    stage_end(c, 9);
    const double ctol = 16.0 * 1.1920929e-7 * tnorm;
    std::vector<signed char> hcl(n, 0);
    std::vector<int> cs, cz, co;
    // runs of eigenvalues closer than ctol, cut into chunks of at most kChunk outputs at the widest
    // gap (never inside a degenerate group); each chunk is solved together with up to kGuardMembers
    // neighbours per side (within 10 ctol), so that a cut through a run, or a close neighbour
    // outside it, cannot pull a member's Ritz pair over
    constexpr int kChunk = 24, kGuardMembers = 4;
    for (int i = 0; i < n;) {
        int g1 = i;
        while (g1 + 1 < n && hw[g1 + 1] - hw[g1] <= ctol) g1++;
        if (g1 == i) {
            i++;
            continue;
        }
        for (int a = i, b = i; a <= g1; a = b + 1) {
            b = g1;
            if (g1 - a + 1 > kChunk) {
                b = a + kChunk / 2 - 1;
                for (int q = b + 1; q <= a + kChunk - 1; q++)
                    if (hw[q + 1] - hw[q] > hw[b + 1] - hw[b]) b = q;
            }
            int lo = a, hi = b;
            while (lo > 0 && a - lo < kGuardMembers && hw[a] - hw[lo - 1] <= 10.0 * ctol) lo--;
            while (hi + 1 < n && hi - b < kGuardMembers && hw[hi + 1] - hw[b] <= 10.0 * ctol) hi++;
            cs.push_back(lo);
            cz.push_back(hi - lo + 1);
            co.push_back(a);
            co.push_back(b + 1);
            for (int q = a; q <= b; q++) hcl[q] = 1;
        }
        i = g1 + 1;
    }
    const int ncl = (int)cs.size();
    if (!nested) c->last_clusters = ncl;
    if ((st = cuda_check(c, cudaMemcpyAsync(cl, hcl.data(), n, cudaMemcpyHostToDevice, c->stream), "cluster flags"))) return st;
    // mixed path: the cluster kernel runs on the side stream while inverse iteration runs on this
    // one (disjoint eigenvalues and outputs, its own scratch, shifts from the bisection values),
    // when that scratch is small; otherwise it follows inverse iteration on this stream
    bool side_clusters = false;
    int *sdcs = nullptr, *sdcz = nullptr, *sdco = nullptr, *sdwf = nullptr;
    double* sw0 = nullptr;
    float* sscr = nullptr;
    signed char* spiv = nullptr;
    if (!fp64 && ncl > 0 && c->side) {
        std::vector<int> wfirst(1, 0);
        for (int q = 0, used = 0; q < ncl; q++) {
            if (used + cz[q] > 32) {
                wfirst.push_back(q);
                used = 0;
            }
            used += cz[q];
        }
        wfirst.push_back(ncl);
        const int nwarps = (int)wfirst.size() - 1;
        const size_t W32 = (size_t)n * 32;
        if ((size_t)nwarps * (21 * W32) <= ((size_t)256 << 20)) {
            side_clusters = true;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&sdcs, ncl * sizeof(int), c->stream), "clusters"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&sdcz, ncl * sizeof(int), c->stream), "clusters"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&sdco, 2 * ncl * sizeof(int), c->stream), "clusters"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&sdwf, wfirst.size() * sizeof(int), c->stream), "clusters"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&sw0, n * sizeof(double), c->stream), "cluster shifts"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&sscr, (size_t)nwarps * 5 * W32 * sizeof(float), c->stream), "cluster scratch"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&spiv, (size_t)nwarps * W32, c->stream), "cluster pivots"))) return st;
            cudaMemcpyAsync(sdcs, cs.data(), ncl * sizeof(int), cudaMemcpyHostToDevice, c->stream);
            cudaMemcpyAsync(sdcz, cz.data(), ncl * sizeof(int), cudaMemcpyHostToDevice, c->stream);
            cudaMemcpyAsync(sdco, co.data(), 2 * ncl * sizeof(int), cudaMemcpyHostToDevice, c->stream);
            cudaMemcpyAsync(sdwf, wfirst.data(), wfirst.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream);
            cudaMemcpyAsync(sw0, dW, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
            if ((st = cuda_check(c, cudaEventRecord(c->ev_fork, c->stream), "fork"))) return st;
            if ((st = cuda_check(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0), "fork"))) return st;
            if (!c->stage_mute) cudaEventRecord(c->ev[2 * 12], c->side);
            cluster_kernel<R><<<nwarps, 32 * kClusterWarps, kStageSmem, c->side>>>(n, df, ef, sw0, dW, sdcs, sdcz, sdco, sdwf, 0, tnorm,
                                                                                 y ? (const float2*)y : nullptr, f_out, (R*)(w + o_z), n,
                                                                                 n_vec, sscr, spiv);
            c->launches++;
            if (!c->stage_mute) {
                cudaEventRecord(c->ev[2 * 12 + 1], c->side);
                c->stage_ms[12] = -1.0;
            }
            if ((st = cuda_check(c, cudaEventRecord(c->ev_join, c->side), "join"))) return st;
        }
    }
    // the refinement's FP64 matrix builds on a second side stream during inverse iteration and the
    // clusters, which leave most SMs idle
    if (!nested && (st = fork_h64(c))) return st;
    stage_begin(c, 10);
    double2* y64 = nullptr;
    if (y) {
        y64 = (double2*)(w + o_y64);
        y_to_double_kernel<T2><<<(n + 255) / 256, 256, 0, c->stream>>>(n, y, y64);
        c->launches++;
    }
    R* z = (R*)(w + o_z);
    for (int i0 = 0; i0 < n; i0 += count_max) {
        const int cnt = std::min(count_max, n - i0);
        invit_kernel<R><<<(cnt + 31) / 32, 32, kStageSmem, c->stream>>>(n, dd, ee, df, ef, dW, cl, i0, cnt, tnorm, y64, f_out, z, n,
                                                                 n_vec, (double*)(w + o_scr), (float*)(w + o_scr32),
                                                                 (signed char*)(w + o_piv), (float*)(w + o_scs), fp64 ? 1 : 0);
        c->launches++;
        if (!fp64) {
            invit_finish_kernel<R><<<(cnt + 7) / 8, 256, 0, c->stream>>>(n, dd, ee, cl, i0, cnt, y ? (const float2*)y : nullptr,
                                                                        (const float*)(w + o_scr32), (const float*)(w + o_scs), dW,
                                                                        f_out, z, n, n_vec);
            c->launches++;
        }
    }
    stage_end(c, 10);
    if (side_clusters) {
        if ((st = cuda_check(c, cudaStreamWaitEvent(c->stream, c->ev_join, 0), "join"))) return st;
        for (void* p : {(void*)sdcs, (void*)sdcz, (void*)sdco, (void*)sdwf, (void*)sw0, (void*)sscr, (void*)spiv})
            cudaFreeAsync(p, c->stream);
    } else if (ncl > 0) {
        // the inverse-iteration scratch is free again (same stream)
        int* dcs = nullptr;
        int* dcz = nullptr;
        int* dco = nullptr;
        double* w0 = nullptr;
        if ((st = cuda_check(c, cudaMallocAsync((void**)&dcs, ncl * sizeof(int), c->stream), "clusters"))) return st;
        if ((st = cuda_check(c, cudaMallocAsync((void**)&dcz, ncl * sizeof(int), c->stream), "clusters"))) return st;
        if ((st = cuda_check(c, cudaMallocAsync((void**)&dco, 2 * ncl * sizeof(int), c->stream), "clusters"))) return st;
        if ((st = cuda_check(c, cudaMallocAsync((void**)&w0, n * sizeof(double), c->stream), "cluster shifts"))) return st;
        cudaMemcpyAsync(dcs, cs.data(), ncl * sizeof(int), cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(dcz, cz.data(), ncl * sizeof(int), cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(dco, co.data(), 2 * ncl * sizeof(int), cudaMemcpyHostToDevice, c->stream);
        // shifts come from a snapshot: clusters overwrite the eigenvalues of their outputs, which
        // other clusters read as guards
        cudaMemcpyAsync(w0, dW, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
        stage_begin(c, 12);
        if (fp64) {
            // FP64 path: per-member FP64 inverse iteration with Gram-Schmidt, then Rayleigh-Ritz;
            // member vectors in Zc (n x c per cluster)
            std::vector<int64_t> hco(ncl);
            int64_t ctot = 0;
            for (int q = 0; q < ncl; q++) {
                hco[q] = ctot;
                ctot += (int64_t)cz[q] * n;
            }
            int64_t* dcoff = nullptr;
            double* Zall = nullptr;
            double* cscr = nullptr;
            signed char* cpiv = nullptr;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&dcoff, ncl * sizeof(int64_t), c->stream), "clusters"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&Zall, (size_t)ctot * 8, c->stream), "cluster vectors"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&cscr, 5 * (size_t)n * ncl * 8, c->stream), "cluster scratch"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&cpiv, (size_t)n * ncl, c->stream), "cluster pivots"))) return st;
            cudaMemcpyAsync(dcoff, hco.data(), ncl * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream);
            cluster64_kernel<R><<<ncl, 32, 0, c->stream>>>(n, dd, ee, w0, dW, dcs, dcz, dco, dcoff, ncl, tnorm, y64, f_out, z, n,
                                                             n_vec, cscr, cpiv, Zall);
            c->launches++;
            for (void* p : {(void*)dcoff, (void*)Zall, (void*)cscr, (void*)cpiv}) cudaFreeAsync(p, c->stream);
        } else {
            // mixed path: clusters packed side by side into warps of 32 lanes, in batches of as
            // many warps as the interleaved scratch holds
            std::vector<int> wfirst(1, 0);
            for (int q = 0, used = 0; q < ncl; q++) {
                if (used + cz[q] > 32) {
                    wfirst.push_back(q);
                    used = 0;
                }
                used += cz[q];
            }
            wfirst.push_back(ncl);
            const int nwarps = (int)wfirst.size() - 1;
            const int wmax = (int)(cpad / 32);
            int* dwf = nullptr;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&dwf, wfirst.size() * sizeof(int), c->stream), "cluster warps"))) return st;
            cudaMemcpyAsync(dwf, wfirst.data(), wfirst.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream);
            for (int wb = 0; wb < nwarps; wb += wmax) {
                const int nb = std::min(wmax, nwarps - wb);
                cluster_kernel<R><<<nb, 32 * kClusterWarps, kStageSmem, c->stream>>>(n, df, ef, w0, dW, dcs, dcz, dco, dwf, wb, tnorm,
                                                            y ? (const float2*)y : nullptr, f_out, z, n,
                                                            n_vec, (float*)(w + o_scr32), (signed char*)(w + o_piv));
                c->launches++;
            }
            cudaFreeAsync(dwf, c->stream);
        }
        stage_end(c, 12);
        for (void* p : {(void*)dcs, (void*)dcz, (void*)dco, (void*)w0}) cudaFreeAsync(p, c->stream);
    }
    stage_begin(c, 11);
    if ((st = cuda_check(c, cudaGetLastError(), "bisection / inverse iteration"))) return st;
    if (n_vec > 0) {
        // X = Q Z for the first n_vec eigenvectors; X is built in a separate buffer because A holds Q
        T2* X = nullptr;
        if ((st = cuda_check(c, cudaMallocAsync((void**)&X, (size_t)n * n_vec * sizeof(T2), c->stream), "eigenvector buffer"))) return st;
        const int64_t nz = (int64_t)n * n_vec;
        if (two_stage) {
            if ((st = band_backtransform(c, n, fp64, z, n_vec, X, w + o_band, bar, err))) {
                cudaFreeAsync(X, c->stream);
                return st;
            }
        } else {
            real_to_complex_kernel<T2><<<(unsigned)((nz + 255) / 256), 256, 0, c->stream>>>(nz, z, X);
            c->launches++;
        }
        if (n > 1 && !two_stage) {
            // X <- Q X, panels of kWY reflectors from the last to the first
            const int npanel = (n - 1 + kWY - 1) / kWY;
            const int64_t vsize = vpanel_offset(n, npanel);
            T2 *Tf = nullptr, *Vall = nullptr, *W1 = nullptr;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&Tf, (size_t)npanel * kWY * kWY * sizeof(T2), c->stream), "WY factors"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&Vall, (size_t)vsize * sizeof(T2), c->stream), "WY panels"))) return st;
            if ((st = cuda_check(c, cudaMallocAsync((void**)&W1, (size_t)kWY * n_vec * sizeof(T2), c->stream), "WY work"))) return st;
            build_vpanels_kernel<T2><<<dim3((n - 1 + 255) / 256, kWY / 8, npanel), 256, 0, c->stream>>>(n, A, lda, tau, Vall);
            c->launches++;
            cublasSetStream(c->cublas, c->stream);
            for (int p = 0; p < npanel && !st; p++) {
                const int m = n - 1 - kWY * p;
                if (xherk(c->cublas, kWY, m, Vall + vpanel_offset(n, p), m, Tf + (size_t)p * kWY * kWY, kWY) != CUBLAS_STATUS_SUCCESS)
                    st = fail(c, BSE_ERR_CUDA, "cuBLAS failed in the back-transformation (Gram)");
            }
            if (!st) {
                const int64_t nu = (int64_t)npanel * kWY * kWY;
                ut_diag_kernel<T2><<<(unsigned)((nu + 255) / 256), 256, 0, c->stream>>>(n, npanel, tau, Tf);
                c->launches++;
            }
            T2 one, zero, mone;
            one.x = 1; one.y = 0; zero.x = 0; zero.y = 0; mone.x = -1; mone.y = 0;
            if constexpr (std::is_same<T2, double2>::value) {
                // FP64: the two products in compensated FP32 (FP64 GEMMs are slow on this part),
                // the triangular solve in cuBLAS
                const int64_t pcap = (int64_t)1 << 22;
                double2 *D = nullptr, *P = nullptr;
                if ((st = cuda_check(c, cudaMallocAsync((void**)&D, (size_t)(n - 1) * n_vec * sizeof(double2), c->stream), "WY work"))) return st;
                if ((st = cuda_check(c, cudaMallocAsync((void**)&P, (size_t)pcap * sizeof(double2), c->stream), "WY work"))) return st;
                for (int p = npanel - 1; p >= 0 && !st; p--) {
                    const int k0 = kWY * p, m = n - 1 - k0, nb = std::min(kWY, m);
                    const double2* Vp = Vall + vpanel_offset(n, p);
                    const double2* Up = Tf + (size_t)p * kWY * kWY;
                    if ((st = df_gemm(c, true, nb, n_vec, m, Vp, m, X + k0 + 1, n, W1, nb, P, pcap))) break;      // V^H X
                    if (xtrsm_lu(c->cublas, nb, n_vec, Up, kWY, W1, nb) != CUBLAS_STATUS_SUCCESS) {
                        st = fail(c, BSE_ERR_CUDA, "cuBLAS failed in the back-transformation");
                        break;
                    }
                    if ((st = df_gemm(c, false, m, n_vec, nb, Vp, m, W1, nb, D, m, P, pcap))) break;            // V W
                    sub_block_kernel<<<(unsigned)(((int64_t)m * n_vec + 255) / 256), 256, 0, c->stream>>>(m, n_vec, D, X + k0 + 1, n);
                    c->launches++;
                }
                cudaFreeAsync(D, c->stream);
                cudaFreeAsync(P, c->stream);
            } else {
                for (int p = npanel - 1; p >= 0 && !st; p--) {
                    const int k0 = kWY * p, m = n - 1 - k0, nb = std::min(kWY, m);
                    const T2* Vp = Vall + vpanel_offset(n, p);
                    const T2* Up = Tf + (size_t)p * kWY * kWY;
                    cublasStatus_t bs = xgemm(c->cublas, CUBLAS_OP_C, CUBLAS_OP_N, nb, n_vec, m, &one, Vp, m, X + k0 + 1, n, &zero, W1, kWY);
                    if (bs == CUBLAS_STATUS_SUCCESS) bs = xtrsm_lu(c->cublas, nb, n_vec, Up, kWY, W1, kWY);
                    if (bs == CUBLAS_STATUS_SUCCESS)
                        bs = xgemm(c->cublas, CUBLAS_OP_N, CUBLAS_OP_N, m, n_vec, nb, &mone, Vp, m, W1, kWY, &one, X + k0 + 1, n);
                    if (bs != CUBLAS_STATUS_SUCCESS) st = fail(c, BSE_ERR_CUDA, "cuBLAS failed in the back-transformation");
                }
            }
            if (!st) st = cuda_check(c, cudaGetLastError(), "back-transformation");
            for (void* q : {(void*)Tf, (void*)Vall, (void*)W1}) cudaFreeAsync(q, c->stream);
            if (st) {
                cudaFreeAsync(X, c->stream);
                return st;
            }
        }
        st = cuda_check(c, cudaMemcpy2DAsync(A, lda * sizeof(T2), X, n * sizeof(T2), n * sizeof(T2), n_vec,
                                             cudaMemcpyDeviceToDevice, c->stream), "eigenvectors");
        cudaFreeAsync(X, c->stream);
        if (st) return st;
        if (two_stage) {
            if ((st = cuda_check(c, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "barrier status"))) return st;
            if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "back-transformation"))) return st;
            if (herr) return fail(c, BSE_ERR_NOT_CONVERGED, "back-transformation: a grid barrier timed out");
        }
    }
    stage_end(c, 11);
    return cuda_check(c, cudaGetLastError(), "own eigensolver");
}

}  // namespace

int own_heevd(bse_ctx* c, int n, void* dA, int lda, bool fp64, double* dW, int n_vec, const double2* rho0, double2* f_out,
              bool nested) {
    if (nested) c->stage_mute++;
    const int st = fp64 ? own_heevd_t<double2>(c, n, (double2*)dA, lda, dW, n_vec, rho0, f_out, nested)
                        : own_heevd_t<float2>(c, n, (float2*)dA, lda, dW, n_vec, rho0, f_out, nested);
    if (nested) c->stage_mute--;
    return st;
}

}  // namespace bse
