// Stage c: dense Hermitian eigensolve of the BSE matrix and the FP64 refinement.
//
// Replaces Excitonic_Hamiltonian::common_diagonalization (bse.version13.cpp:3120-3368):
// eig_sym (LAPACK zheevd) on the TDA matrix, ascending order, unit eigenvectors; for
// collinear spin the rotated spin-flip block H0 and the spin-conserving block H1 are
// solved separately (3143-3149, 3195-3204).
//
// Solvers: BSE_EIG_OWN runs this library's tridiagonal reduction + bisection + inverse
// iteration (tridiag.cu); BSE_EIG_CUSOLVER calls cuSOLVER's heevd (the plain library path,
// used as the FP64 GPU baseline).  In BSE_MIXED the solve runs on the complex64 matrix
// and the lowest n_refine eigenpairs are then refined in FP64 by one Rayleigh-Ritz step
// on the FP64 matrix: the pencil (X^H H X, X^H X) of the FP32 Ritz vectors X, its products in
// compensated FP32, solved by Ogita-Aishima iterative refinement (a dense FP64 solve of the
// Cholesky-transformed pencil as the fallback).
#include <cstdlib>
#include <string>

#include <algorithm>
#include <numeric>
#include <vector>

#include "bse_internal.h"
#include "dev_util.h"

namespace bse {
namespace {

using namespace dev;

const int kGuard = 32;   // extra Ritz vectors above n_refine so the last refined ones converge

__global__ void widen_kernel(int64_t n, const float2* __restrict__ a, double2* __restrict__ b) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) b[t] = make_double2(a[t].x, a[t].y);
}
__global__ void narrow_kernel(int64_t n, const double2* __restrict__ a, float2* __restrict__ b) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) b[t] = make_float2((float)a[t].x, (float)a[t].y);
}
// Full Hermitian storage of an m x m matrix from its lower triangle (the projected matrix of the
// refinement is formed as X^H (H X), Hermitian only up to rounding).
__global__ void hermitize_lower_kernel(int m, double2* __restrict__ G) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * m) return;
    const int i = (int)(t % m), j = (int)(t / m);   // row i, column j
    if (i < j) {
        const double2 l = G[j + (int64_t)i * m];
        G[t] = make_double2(l.x, -l.y);
    } else if (i == j) {
        G[t].y = 0;
    }
}
__global__ void f2d_kernel(int64_t n, const float* __restrict__ a, double* __restrict__ b) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) b[t] = a[t];
}

// ||HX_j - theta_j X_j||_2 for column j (one block per column)
__global__ void residual_kernel(int64_t n, const double2* __restrict__ HX, const double2* __restrict__ X,
                                const double* __restrict__ theta, double* __restrict__ out) {
    const int64_t j = blockIdx.x;
    const double t = theta[j];
    double s = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 h = HX[i + j * n], x = X[i + j * n];
        const double rx = h.x - t * x.x, ry = h.y - t * x.y;
        s += rx * rx + ry * ry;
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) out[j] = sqrt(s);
    }
}

// Y = H X for Hermitian H (n x n FP64, lower triangle, leading dimension n) and X (n x m FP64),
// in compensated FP32 ("double-float") arithmetic instead of FP64 (whose rate on this part is
// ~1/64 of FP32): H and X are split into FP32 hi + lo parts as tiles are loaded, every hi*hi
// product is formed exactly (TwoProd with an FMA) and added with TwoSum into an (s, t) pair, the
// hi*lo cross terms go into t, lo*lo is dropped.  Relative error ~1e-12, FP64-class for the
// Rayleigh-Ritz step.  Block tile 64 rows x 32 columns of Y; thread (lane c, warp w) owns rows
// 8w .. 8w+7 of column c.
constexpr int HM_TM = 64, HM_TN = 32, HM_TK = 16;

__device__ __forceinline__ float4 split2(double2 v) {
    const float rh = (float)v.x, ih = (float)v.y;
    return make_float4(rh, ih, (float)(v.x - (double)rh), (float)(v.y - (double)ih));
}
// (s, t) += a * b with the product and the sum's rounding errors kept in t
__device__ __forceinline__ void twoacc(float& s, float& t, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    const float ns = __fadd_rn(s, p);
    const float bv = __fsub_rn(ns, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(ns, bv)), __fsub_rn(p, bv));
    s = ns;
    t = __fadd_rn(t, __fadd_rn(e, pe));
}

// (sr + tr, si + ti) += h * x for split operands h, x = (re hi, im hi, re lo, im lo)
__device__ __forceinline__ void cmac_df(float& sr, float& tr, float& si, float& ti, float4 h, float4 x) {
    // real: hr xr - hi xi;  imag: hr xi + hi xr
    twoacc(sr, tr, h.x, x.x);
    twoacc(sr, tr, -h.y, x.y);
    tr = __fmaf_rn(h.x, x.z, __fmaf_rn(h.z, x.x, __fmaf_rn(-h.y, x.w, __fmaf_rn(-h.w, x.y, tr))));
    twoacc(si, ti, h.x, x.y);
    twoacc(si, ti, h.y, x.x);
    ti = __fmaf_rn(h.x, x.w, __fmaf_rn(h.z, x.y, __fmaf_rn(h.y, x.z, __fmaf_rn(h.w, x.x, ti))));
}

// In-place / out-of-place split of FP64 complex values into (re hi, im hi, re lo, im lo) FP32
// pairs, once per operand: the products then stage tiles without FP64 arithmetic (slow on this
// part; every element of H used to be split by each of the m / HM_TN column blocks).
__global__ void split_df_kernel(int64_t len, const double2* in, float4* out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < len) {
        const double2 v = in[t];
        out[t] = split2(v);
    }
}
__device__ __forceinline__ float4 conj_split(float4 h) { return make_float4(h.x, -h.y, h.z, -h.w); }

__global__ void __launch_bounds__(256) hemm_df_kernel(int n, int m, const float4* __restrict__ H,
                                                      const float4* __restrict__ X, double2* __restrict__ Y) {
    __shared__ float4 Hs[HM_TK][HM_TM + 1];   // (re hi, im hi, re lo, im lo), [k][row]
    __shared__ float4 Xs[HM_TK][HM_TN + 1];   // [k][column]
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int i0 = blockIdx.x * HM_TM, c0 = blockIdx.y * HM_TN;
    float sr[8], tr[8], si[8], ti[8];
#pragma unroll
    for (int r = 0; r < 8; r++) sr[r] = tr[r] = si[r] = ti[r] = 0.0f;
    for (int j0 = 0; j0 < n; j0 += HM_TK) {
        if (i0 + HM_TM - 1 < j0) {
            // tile strictly above the diagonal: conj of the stored lower tile, read along its columns
            for (int e = tid; e < HM_TM * HM_TK; e += 256) {
                const int jj = e % HM_TK, ii = e / HM_TK, i = i0 + ii, j = j0 + jj;
                Hs[jj][ii] = (i < n && j < n) ? conj_split(H[j + (size_t)i * n]) : make_float4(0, 0, 0, 0);
            }
        } else {
            for (int e = tid; e < HM_TM * HM_TK; e += 256) {
                const int ii = e % HM_TM, jj = e / HM_TM, i = i0 + ii, j = j0 + jj;
                float4 h = make_float4(0, 0, 0, 0);
                if (i < n && j < n) h = i >= j ? H[i + (size_t)j * n] : conj_split(H[j + (size_t)i * n]);
                Hs[jj][ii] = h;
            }
        }
        for (int e = tid; e < HM_TK * HM_TN; e += 256) {
            const int jj = e % HM_TK, cc = e / HM_TK, j = j0 + jj, col = c0 + cc;
            Xs[jj][cc] = (j < n && col < m) ? X[j + (size_t)col * n] : make_float4(0, 0, 0, 0);
        }
        __syncthreads();
#pragma unroll 4
        for (int jj = 0; jj < HM_TK; jj++) {
            const float4 x = Xs[jj][tx];
#pragma unroll
            for (int r = 0; r < 8; r++) cmac_df(sr[r], tr[r], si[r], ti[r], Hs[jj][ty * 8 + r], x);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int row = i0 + ty * 8 + r, col = c0 + tx;
        if (row < n && col < m)
            Y[row + (size_t)col * n] = make_double2((double)sr[r] + (double)tr[r], (double)si[r] + (double)ti[r]);
    }
}

// C = op(A) B (op = identity or conjugate transpose; A, B FP64, column-major) in the same
// compensated FP32 arithmetic, split over K: block z writes the partial product over its K range
// to C + z * split_stride, and sum_splits_kernel adds the partials in FP64.
// operands are FP64 (split per tile) or already split into FP32 pairs (split_df_kernel)
__device__ __forceinline__ float4 ld_split(const double2* p) { return split2(*p); }
__device__ __forceinline__ float4 ld_split(const float4* p) { return *p; }
__device__ __forceinline__ float4 ld_split_conj(const double2* p) {
    double2 v = *p;
    v.y = -v.y;
    return split2(v);
}
__device__ __forceinline__ float4 ld_split_conj(const float4* p) { return conj_split(*p); }

template <bool CONJ_A, typename TA, typename TB>
__global__ void __launch_bounds__(256) gemm_df_kernel(int M, int N, int K, int kchunk, const TA* __restrict__ A,
                                                      int64_t lda, const TB* __restrict__ B, int64_t ldb,
                                                      double2* __restrict__ C, int64_t ldc, int64_t split_stride) {
    __shared__ float4 As[HM_TK][HM_TM + 1];
    __shared__ float4 Bs[HM_TK][HM_TN + 1];
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int i0 = blockIdx.x * HM_TM, c0 = blockIdx.y * HM_TN;
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    float sr[8], tr[8], si[8], ti[8];
#pragma unroll
    for (int r = 0; r < 8; r++) sr[r] = tr[r] = si[r] = ti[r] = 0.0f;
    for (int j0 = kb; j0 < ke; j0 += HM_TK) {
        if (CONJ_A) {   // op(A)(i, k) = conj(A[k + i lda]): read along k
            for (int e = tid; e < HM_TM * HM_TK; e += 256) {
                const int jj = e % HM_TK, ii = e / HM_TK, i = i0 + ii, k = j0 + jj;
                As[jj][ii] = (i < M && k < ke) ? ld_split_conj(A + k + (size_t)i * lda) : make_float4(0, 0, 0, 0);
            }
        } else {
            for (int e = tid; e < HM_TM * HM_TK; e += 256) {
                const int ii = e % HM_TM, jj = e / HM_TM, i = i0 + ii, k = j0 + jj;
                As[jj][ii] = (i < M && k < ke) ? ld_split(A + i + (size_t)k * lda) : make_float4(0, 0, 0, 0);
            }
        }
        for (int e = tid; e < HM_TK * HM_TN; e += 256) {
            const int jj = e % HM_TK, cc = e / HM_TK, k = j0 + jj, col = c0 + cc;
            Bs[jj][cc] = (k < ke && col < N) ? ld_split(B + k + (size_t)col * ldb) : make_float4(0, 0, 0, 0);
        }
        __syncthreads();
#pragma unroll 4
        for (int jj = 0; jj < HM_TK; jj++) {
            const float4 x = Bs[jj][tx];
#pragma unroll
            for (int r = 0; r < 8; r++) cmac_df(sr[r], tr[r], si[r], ti[r], As[jj][ty * 8 + r], x);
        }
        __syncthreads();
    }
    double2* Cz = C + blockIdx.z * split_stride;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int row = i0 + ty * 8 + r, col = c0 + tx;
        if (row < M && col < N)
            Cz[row + (size_t)col * ldc] = make_double2((double)sr[r] + (double)tr[r], (double)si[r] + (double)ti[r]);
    }
}

__global__ void sum_splits_kernel(int64_t len, int splits, const double2* __restrict__ P, double2* __restrict__ C) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= len) return;
    double x = 0, y = 0;
    for (int z = 0; z < splits; z++) {
        x += P[t + z * len].x;
        y += P[t + z * len].y;
    }
    C[t] = make_double2(x, y);
}

constexpr int kMaxSplits = 16;

// C (M x N, leading dimension M when split) = op(A) B; P: scratch of pcap elements for the
// split-K partials (used when the output tiles alone would not fill the GPU).
template <typename TA, typename TB>
int gemm_df(bse_ctx* c, bool conj_a, int M, int N, int K, const TA* A, int64_t lda, const TB* B, int64_t ldb,
            double2* C, int64_t ldc, double2* P, int64_t pcap) {
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    const int tiles = ((M + HM_TM - 1) / HM_TM) * ((N + HM_TN - 1) / HM_TN);
    int splits = std::max(1, std::min(kMaxSplits, (2 * nsm + tiles - 1) / tiles));
    splits = (int)std::max<int64_t>(1, std::min<int64_t>(splits, pcap / ((int64_t)M * N)));
    int kchunk = ((K + splits - 1) / splits + HM_TK - 1) / HM_TK * HM_TK;
    splits = (K + kchunk - 1) / kchunk;
    const dim3 grid((M + HM_TM - 1) / HM_TM, (N + HM_TN - 1) / HM_TN, splits);
    double2* out = splits > 1 ? P : C;
    const int64_t ldo = splits > 1 ? M : ldc;
    if (conj_a) gemm_df_kernel<true, TA, TB><<<grid, 256, 0, c->stream>>>(M, N, K, kchunk, A, lda, B, ldb, out, ldo, (int64_t)M * N);
    else gemm_df_kernel<false, TA, TB><<<grid, 256, 0, c->stream>>>(M, N, K, kchunk, A, lda, B, ldb, out, ldo, (int64_t)M * N);
    c->launches++;
    if (splits > 1) {
        if (ldc != M) return fail(c, BSE_ERR_CUDA, "split product needs a packed output");
        const int64_t len = (int64_t)M * N;
        sum_splits_kernel<<<(unsigned)((len + 255) / 256), 256, 0, c->stream>>>(len, splits, P, C);
        c->launches++;
    }
    return cuda_check(c, cudaGetLastError(), "compensated product");
}

// ---- eigenpairs of the projected pencil (S, M) by iterative refinement ----
// S = X^H H X and M = X^H X for the FP32 Ritz vectors X: S is nearly diagonal and M nearly the
// identity, so instead of a dense eigensolve the eigenvectors Z (Z^H M Z = I, Z^H S Z = diag)
// are refined from Z = I by the Ogita-Aishima iteration (Ogita & Aishima, "Iterative refinement
// for symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35, 2018):
//     R = I - Z^H M Z,  T = Z^H S Z,  lambda_i = T_ii / (1 - R_ii),
//     E_ij = (T_ij + lambda_j R_ij) / (lambda_j - lambda_i)  (different clusters),
//     E_ij = R_ij / 2  (same cluster),  Z <- Z + Z E,
// which converges quadratically; products in compensated FP32.  Eigenvalues closer than
// max_ij |S_ij - d_j M_ij| / kOaEta (d = diag S / diag M) form clusters, whose blocks of T are
// diagonalised exactly at the end (complex Jacobi, one block per cluster).  Clusters wider than
// kOaMaxCluster, or a last correction above kOaTol, hand the pencil to the dense solver.
constexpr int kOaMaxCluster = 8;
constexpr double kOaEta = 0.05;
constexpr double kOaTol = 1e-4;
constexpr int kOaIters = 3;
constexpr int kOaParts = 128;

__device__ __forceinline__ double block_max(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

// d_i = Re S_ii / Re M_ii; part[block] = max_{i != j} |S_ij - M_ij d_j|^2
__global__ void oa_coupling_kernel(int m, const double2* __restrict__ S, const double2* __restrict__ Mg, double* __restrict__ d,
                                   double* __restrict__ part) {
    __shared__ double red[32];
    const int64_t len = (int64_t)m * m;
    double mx = 0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < len; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % m), j = (int)(t / m);
        const int64_t jj = j + (int64_t)j * m;
        const double dj = S[jj].x / Mg[jj].x;
        if (i == j) {
            d[i] = dj;
            continue;
        }
        const double rx = S[t].x - Mg[t].x * dj, ry = S[t].y - Mg[t].y * dj;
        mx = fmax(mx, rx * rx + ry * ry);
    }
    mx = block_max(mx, red);
    if (threadIdx.x == 0) part[blockIdx.x] = mx;
}

// E from T and Q = Z^H M Z (R = I - Q); part[block] = max |E_ij|^2 over pairs in different clusters
__global__ void oa_e_kernel(int m, const double2* __restrict__ T, const double2* __restrict__ Q, const int* __restrict__ cid,
                            double2* __restrict__ E, double* __restrict__ part) {
    __shared__ double red[32];
    const int64_t len = (int64_t)m * m;
    double mx = 0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < len; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % m), j = (int)(t / m);
        const int64_t ii = i + (int64_t)i * m, jj = j + (int64_t)j * m;
        const double rx = (i == j ? 1.0 : 0.0) - Q[t].x, ry = -Q[t].y;
        if (cid[i] == cid[j]) {
            E[t] = make_double2(0.5 * rx, 0.5 * ry);
        } else {
            const double li = T[ii].x / Q[ii].x, lj = T[jj].x / Q[jj].x;
            const double inv = 1.0 / (lj - li);
            const double ex = (T[t].x + lj * rx) * inv, ey = (T[t].y + lj * ry) * inv;
            E[t] = make_double2(ex, ey);
            mx = fmax(mx, ex * ex + ey * ey);
        }
    }
    mx = block_max(mx, red);
    if (threadIdx.x == 0) part[blockIdx.x] = mx;
}

// Z <- Z + W, or Z <- I + W when `identity`
__global__ void oa_add_kernel(int m, double2* __restrict__ Z, const double2* __restrict__ W, int identity) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * m) return;
    double2 z = identity ? make_double2((t % m) == (t / m) ? 1.0 : 0.0, 0.0) : Z[t];
    z.x += W[t].x;
    z.y += W[t].y;
    Z[t] = z;
}

__global__ void oa_theta_kernel(int m, const double2* __restrict__ T, const double2* __restrict__ Q, double* __restrict__ theta) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) theta[i] = T[i + (int64_t)i * m].x / Q[i + (int64_t)i * m].x;
}

// Cyclic complex Jacobi on a small Hermitian matrix (one thread): A <- U^H A U diagonal, V <- V U.
// Each rotation first turns A_pq real with a phase on column q, then applies the real rotation.
__device__ void jacobi_herm(int c, double2 (*A)[kOaMaxCluster], double2 (*V)[kOaMaxCluster]) {
    for (int sweep = 0; sweep < 40; sweep++) {
        double off = 0, dia = 0;
        for (int p = 0; p < c; p++) {
            dia += A[p][p].x * A[p][p].x;
            for (int q = p + 1; q < c; q++) off += A[p][q].x * A[p][q].x + A[p][q].y * A[p][q].y;
        }
        if (off <= 1e-32 * dia || off == 0.0) break;
        for (int p = 0; p < c; p++)
            for (int q = p + 1; q < c; q++) {
                const double2 b = A[p][q];
                const double ab = sqrt(b.x * b.x + b.y * b.y);
                if (ab == 0.0) continue;
                const double phx = b.x / ab, phy = b.y / ab;
                const double tau = (A[q][q].x - A[p][p].x) / (2.0 * ab);
                const double tt = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                const double cs = 1.0 / sqrt(1.0 + tt * tt), sn = tt * cs;
                // U_pp = cs, U_qp = -sn conj(ph), U_pq = sn, U_qq = cs conj(ph)
                const double2 upp = make_double2(cs, 0), uqp = make_double2(-sn * phx, sn * phy);
                const double2 upq = make_double2(sn, 0), uqq = make_double2(cs * phx, -cs * phy);
                for (int k = 0; k < c; k++) {
                    const double2 x = A[k][p], y = A[k][q];
                    A[k][p] = cadd(cmul(x, upp), cmul(y, uqp));
                    A[k][q] = cadd(cmul(x, upq), cmul(y, uqq));
                }
                for (int k = 0; k < c; k++) {
                    const double2 x = A[p][k], y = A[q][k];
                    A[p][k] = cadd(cconjmul(upp, x), cconjmul(uqp, y));
                    A[q][k] = cadd(cconjmul(upq, x), cconjmul(uqq, y));
                }
                for (int k = 0; k < c; k++) {
                    const double2 x = V[k][p], y = V[k][q];
                    V[k][p] = cadd(cmul(x, upp), cmul(y, uqp));
                    V[k][q] = cadd(cmul(x, upq), cmul(y, uqq));
                }
            }
    }
}

// One block per cluster: diagonalise the cluster's block of T, rotate its columns of Z.
__global__ void __launch_bounds__(256) oa_cluster_kernel(int m, const int* __restrict__ off, const int* __restrict__ idx,
                                                         const double2* __restrict__ T, double2* __restrict__ Z,
                                                         double* __restrict__ theta) {
    __shared__ double2 A[kOaMaxCluster][kOaMaxCluster], V[kOaMaxCluster][kOaMaxCluster];
    __shared__ int ix[kOaMaxCluster];
    const int o = off[blockIdx.x], c = off[blockIdx.x + 1] - o, tid = threadIdx.x;
    if (tid < c) ix[tid] = idx[o + tid];
    __syncthreads();
    for (int e = tid; e < c * c; e += blockDim.x) {
        const int a = e % c, b = e / c;
        const double2 u = T[ix[a] + (int64_t)ix[b] * m], w = T[ix[b] + (int64_t)ix[a] * m];
        A[a][b] = make_double2(0.5 * (u.x + w.x), 0.5 * (u.y - w.y));
        V[a][b] = make_double2(a == b ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    if (tid == 0) jacobi_herm(c, A, V);
    __syncthreads();
    if (tid < c) theta[ix[tid]] = A[tid][tid].x;
    for (int r = tid; r < m; r += blockDim.x) {
        double2 zr[kOaMaxCluster];
#pragma unroll
        for (int a = 0; a < kOaMaxCluster; a++) zr[a] = a < c ? Z[r + (int64_t)ix[a] * m] : make_double2(0, 0);
#pragma unroll
        for (int b = 0; b < kOaMaxCluster; b++) {
            if (b < c) {
                double2 acc = make_double2(0, 0);
#pragma unroll
                for (int a = 0; a < kOaMaxCluster; a++)
                    if (a < c) acc = cadd(acc, cmul(zr[a], V[a][b]));
                Z[r + (int64_t)ix[b] * m] = acc;
            }
        }
    }
}

// Zo[:, j] = Z[:, perm[j]], tho[j] = th[perm[j]]
__global__ void oa_permute_kernel(int m, const int* __restrict__ perm, const double2* __restrict__ Z, const double* __restrict__ th,
                                  double2* __restrict__ Zo, double* __restrict__ tho) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * m) return;
    const int r = (int)(t % m), j = (int)(t / m);
    Zo[t] = Z[r + (int64_t)perm[j] * m];
    if (r == 0) tho[j] = th[perm[j]];
}

// Host side of the refinement of the pencil (S, M) (kernels above).  ws: oa_workspace(m) bytes.
// On return *ok tells whether Z / theta hold the eigenpairs (ascending); otherwise the caller
// solves the pencil densely.
size_t oa_workspace(int64_t m) { return 9 * (size_t)m * m * sizeof(double2) + (size_t)m * 64 + kOaParts * 8 + 4096; }

int oa_refine(bse_ctx* c, int m, const double2* S, const double2* Mg, double2* Zout, double* theta, double2* Pw, int64_t pcap,
              char* ws, bool* ok) {
    int st;
    *ok = false;
    const size_t mm = (size_t)m * m;
    double2* Z = (double2*)ws;
    double2* E = Z + mm;
    double2* Q = E + mm;
    double2* T = Q + mm;
    double2* W1 = T + mm;
    double2* W2 = W1 + mm;
    float4* S4 = (float4*)(W2 + mm);   // S, M and the current Z split into FP32 pairs
    float4* M4 = S4 + mm;
    float4* Z4 = M4 + mm;
    double* d = (double*)(Z4 + mm);
    double* th = d + m;
    double* part = th + m;
    int* cid = (int*)(part + kOaParts);
    int* perm = cid + m;
    int* coff = perm + m;              // cluster offsets (<= m / 2 + 1) and members (<= m)
    int* cidx = coff + (m / 2 + 2);
    const unsigned gm = (unsigned)((mm + 255) / 256);
    // clusters from the diagonal and the largest coupling
    oa_coupling_kernel<<<kOaParts, 256, 0, c->stream>>>(m, S, Mg, d, part);
    c->launches++;
    std::vector<double> hd(m), hp(kOaParts);
    if ((st = cuda_check(c, cudaMemcpyAsync(hd.data(), d, m * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "pencil diagonal"))) return st;
    if ((st = cuda_check(c, cudaMemcpyAsync(hp.data(), part, kOaParts * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "coupling"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "pencil diagonal"))) return st;
    const double coup = std::sqrt(*std::max_element(hp.begin(), hp.end()));
    for (double v : hd)
        if (!std::isfinite(v)) return BSE_OK;
    const double tau = coup / kOaEta;
    std::vector<int> order(m), hcid(m), hoff, hidx;
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return hd[a] < hd[b]; });
    int ncl = 0;
    for (int a = 0; a < m;) {
        int b = a + 1;
        while (b < m && hd[order[b]] - hd[order[b - 1]] <= tau) b++;
        if (b - a > kOaMaxCluster) return BSE_OK;   // too wide: dense solve
        if (b - a >= 2) {
            hoff.push_back((int)hidx.size());
            for (int q = a; q < b; q++) hidx.push_back(order[q]);
        }
        for (int q = a; q < b; q++) hcid[order[q]] = ncl;
        ncl++;
        a = b;
    }
    const int nbig = (int)hoff.size();
    hoff.push_back((int)hidx.size());
    if ((st = cuda_check(c, cudaMemcpyAsync(cid, hcid.data(), m * sizeof(int), cudaMemcpyHostToDevice, c->stream), "clusters"))) return st;
    if (nbig && (st = cuda_check(c, cudaMemcpyAsync(coff, hoff.data(), hoff.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream), "clusters"))) return st;
    if (nbig && (st = cuda_check(c, cudaMemcpyAsync(cidx, hidx.data(), hidx.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream), "clusters"))) return st;
    split_df_kernel<<<gm, 256, 0, c->stream>>>((int64_t)mm, S, S4);
    split_df_kernel<<<gm, 256, 0, c->stream>>>((int64_t)mm, Mg, M4);
    c->launches += 2;
    const float4* cZ4 = Z4;
    // iterations: the first from Z = I needs no product (T = S, Q = M)
    for (int it = 0; it < kOaIters; it++) {
        const double2* Tk = S;
        const double2* Qk = Mg;
        if (it > 0) {
            split_df_kernel<<<gm, 256, 0, c->stream>>>((int64_t)mm, Z, Z4);
            c->launches++;
            if ((st = gemm_df(c, false, m, m, m, (const float4*)M4, m, cZ4, m, W1, m, Pw, pcap))) return st;   // M Z
            if ((st = gemm_df(c, true, m, m, m, cZ4, m, (const double2*)W1, m, Q, m, Pw, pcap))) return st;     // Z^H M Z
            if ((st = gemm_df(c, false, m, m, m, (const float4*)S4, m, cZ4, m, W2, m, Pw, pcap))) return st;    // S Z
            if ((st = gemm_df(c, true, m, m, m, cZ4, m, (const double2*)W2, m, T, m, Pw, pcap))) return st;     // Z^H S Z
            Tk = T;
            Qk = Q;
        }
        oa_e_kernel<<<kOaParts, 256, 0, c->stream>>>(m, Tk, Qk, cid, E, part);
        c->launches++;
        if (it == 0) {
            oa_add_kernel<<<gm, 256, 0, c->stream>>>(m, Z, E, 1);
        } else {
            if ((st = gemm_df(c, false, m, m, m, cZ4, m, (const double2*)E, m, W1, m, Pw, pcap))) return st;    // Z E
            oa_add_kernel<<<gm, 256, 0, c->stream>>>(m, Z, W1, 0);
        }
        c->launches++;
    }
    // Rayleigh quotients at the final Z, cluster blocks diagonalised
    split_df_kernel<<<gm, 256, 0, c->stream>>>((int64_t)mm, Z, Z4);
    c->launches++;
    if ((st = gemm_df(c, false, m, m, m, (const float4*)M4, m, cZ4, m, W1, m, Pw, pcap))) return st;
    if ((st = gemm_df(c, true, m, m, m, cZ4, m, (const double2*)W1, m, Q, m, Pw, pcap))) return st;
    if ((st = gemm_df(c, false, m, m, m, (const float4*)S4, m, cZ4, m, W2, m, Pw, pcap))) return st;
    if ((st = gemm_df(c, true, m, m, m, cZ4, m, (const double2*)W2, m, T, m, Pw, pcap))) return st;
    oa_theta_kernel<<<(m + 255) / 256, 256, 0, c->stream>>>(m, T, Q, th);
    c->launches++;
    if (nbig) {
        oa_cluster_kernel<<<nbig, 256, 0, c->stream>>>(m, coff, cidx, T, Z, th);
        c->launches++;
    }
    // the last correction (converged?) and the order of the eigenvalues
    std::vector<double> hth(m);
    if ((st = cuda_check(c, cudaMemcpyAsync(hp.data(), part, kOaParts * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "correction"))) return st;
    if ((st = cuda_check(c, cudaMemcpyAsync(hth.data(), th, m * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "eigenvalues"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "pencil refinement"))) return st;
    const double last = std::sqrt(*std::max_element(hp.begin(), hp.end()));
    if (!(last <= kOaTol)) return BSE_OK;
    for (double v : hth)
        if (!std::isfinite(v)) return BSE_OK;
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return hth[a] < hth[b]; });
    if ((st = cuda_check(c, cudaMemcpyAsync(perm, order.data(), m * sizeof(int), cudaMemcpyHostToDevice, c->stream), "order"))) return st;
    oa_permute_kernel<<<gm, 256, 0, c->stream>>>(m, perm, Z, th, Zout, theta);
    c->launches++;
    if ((st = cuda_check(c, cudaGetLastError(), "pencil refinement"))) return st;
    *ok = true;
    return BSE_OK;
}

int cusolver_check(bse_ctx* c, cusolverStatus_t s, const char* what) {
    if (s == CUSOLVER_STATUS_SUCCESS) return BSE_OK;
    if (s == CUSOLVER_STATUS_ALLOC_FAILED) return fail(c, BSE_ERR_OOM, std::string(what) + ": cuSOLVER allocation failed");
    return fail(c, BSE_ERR_CUDA, std::string(what) + ": cuSOLVER status " + std::to_string((int)s));
}
int cublas_check(bse_ctx* c, cublasStatus_t s, const char* what) {
    if (s == CUBLAS_STATUS_SUCCESS) return BSE_OK;
    return fail(c, BSE_ERR_CUDA, std::string(what) + ": cuBLAS status " + std::to_string((int)s));
}

// cuSOLVER heevd on one matrix; eigenvalues always returned as double in dW.
int library_heevd(bse_ctx* c, int64_t n, void* A, int64_t lda, bool fp64, double* dW, bool vectors) {
    int st;
    cusolverDnParams_t prm;
    if ((st = cusolver_check(c, cusolverDnCreateParams(&prm), "params"))) return st;
    const cudaDataType ta = fp64 ? CUDA_C_64F : CUDA_C_32F, tw = fp64 ? CUDA_R_64F : CUDA_R_32F;
    const cusolverEigMode_t jobz = vectors ? CUSOLVER_EIG_MODE_VECTOR : CUSOLVER_EIG_MODE_NOVECTOR;
    void* W = dW;
    size_t wbytes = fp64 ? 0 : (size_t)n * sizeof(float);
    size_t dws = 0, hws = 0;
    st = cusolver_check(c, cusolverDnXsyevd_bufferSize(c->cusolver, prm, jobz, CUBLAS_FILL_MODE_LOWER, n, ta, A, lda,
                                                       tw, W, ta, &dws, &hws), "heevd buffer size");
    if (st) { cusolverDnDestroyParams(prm); return st; }
    size_t need = dws + wbytes + sizeof(int) + 256;
    if ((st = ensure_work(c, need))) { cusolverDnDestroyParams(prm); return st; }
    char* w = (char*)c->d_work;
    int* dinfo = (int*)w;
    float* W32 = (float*)(w + 256);
    void* dbuf = w + 256 + ((wbytes + 255) / 256) * 256;
    if (!fp64) W = W32;
    std::vector<char> hbuf(hws > 0 ? hws : 1);
    st = cusolver_check(c, cusolverDnXsyevd(c->cusolver, prm, jobz, CUBLAS_FILL_MODE_LOWER, n, ta, A, lda, tw, W, ta,
                                            dbuf, dws, hbuf.data(), hws, dinfo), "heevd");
    cusolverDnDestroyParams(prm);
    if (st) return st;
    if (!fp64) {
        f2d_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, W32, dW);
        c->launches++;
    }
    int info = 0;
    if ((st = cuda_check(c, cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "heevd info"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "heevd sync"))) return st;
    if (info > 0) return fail(c, BSE_ERR_NOT_CONVERGED, "heevd did not converge");
    if (info < 0) return fail(c, BSE_ERR_BAD_INPUT, "heevd: invalid argument " + std::to_string(-info));
    return BSE_OK;
}

// n_vec: eigenvectors the caller needs (leading columns); rho0/f: optical vector and oscillators.
int solve_one(bse_ctx* c, int64_t n, void* A, int64_t lda, bool fp64, double* dW, int64_t n_vec,
              const double2* rho0, double2* f) {
    if (c->p.eig_solver == BSE_EIG_OWN) {
        int st = own_heevd(c, (int)n, A, (int)lda, fp64, dW, (int)n_vec, rho0, f);
        if (!st && rho0) {
            c->n_vec_valid = n_vec;
            c->f_from_eig = f != nullptr;
        }
        return st;
    }
    // the library path forms oscillators from eigenvectors: the optical block always needs them
    int st = library_heevd(c, n, A, lda, fp64, dW, n_vec > 0 || rho0 != nullptr);
    if (!st && rho0) {
        c->n_vec_valid = n;
        c->f_from_eig = false;
    }
    return st;
}

}  // namespace

int df_gemm(bse_ctx* c, bool conj_a, int M, int N, int K, const double2* A, int64_t lda, const double2* B, int64_t ldb,
            double2* C, int64_t ldc, double2* P, int64_t pcap) {
    return gemm_df(c, conj_a, M, N, K, A, lda, B, ldb, C, ldc, P, pcap);
}

namespace {

// L (lower, from potrf) in place with its strict upper triangle cleared, and W = J L
// (rows N..2N-1 negated), n = 2N.
__global__ void jl_kernel(int64_t n, int64_t N, double2* __restrict__ L, double2* __restrict__ W) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const int64_t i = t % n, j = t / n;
    double2 l = L[t];
    if (i < j) {
        l = make_double2(0, 0);
        L[t] = l;
    }
    W[t] = i >= N ? make_double2(-l.x, -l.y) : l;
}

// W <- (W + W^H) / 2 (the product L^H (J L) is Hermitian up to rounding)
__global__ void hermitian_part_kernel(int64_t n, double2* __restrict__ W) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const int64_t i = t % n, j = t / n;
    if (i < j) return;
    if (i == j) {
        W[t].y = 0.0;
        return;
    }
    const double2 a = W[t], b = W[j + n * i];
    const double2 m = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
    W[t] = m;
    W[j + n * i] = make_double2(m.x, -m.y);
}

// x_l *= |E_l|^(1/2) for the leading ncols columns of X (ld n), and f_l *= |E_l|^(1/2)
__global__ void jnorm_scale_kernel(int64_t n, int64_t ncols, const double* __restrict__ E, double2* __restrict__ X,
                                   double2* __restrict__ f) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f && t < n) {
        const double s = sqrt(fabs(E[t]));
        f[t] = make_double2(f[t].x * s, f[t].y * s);
    }
    if (t >= n * ncols) return;
    const double s = sqrt(fabs(E[t / n]));
    X[t] = make_double2(X[t].x * s, X[t].y * s);
}

}  // namespace

// Full BSE (tamm_dancoff = 0, FP64): common_diagonalization's eig_gen of the 2N x 2N
// matrix (bse.version13.cpp:3326) replaced by a structure-preserving Hermitian solve.  The build
// left M = [[A, B], [B^H, conj(A)]] (H = J M) in d_H.  With M = L L^H (potrf; M must be positive
// definite, the stable-ground-state case), H = J L L^H is similar to the Hermitian W = L^H J L,
// so W y = E y gives H x = E x for x = |E|^{1/2} L^{-H} y, normalised x^H J x = sign(E), and the
// oscillator f = rho^H x = |E|^{1/2} (L^{-1} rho)^H y needs no eigenvector when the own solver
// forms (L^{-1} rho)^H y itself.  Eigenvalues ascending: -E_max .. -E_min, E_min .. E_max.
// One n x n block (n = 2N spinless; 4N for each collinear spin block): M consumed, W the workspace
// (left holding the eigenvectors), rho0 / f null for a values-only block.
int solve_coupled_block(bse_ctx* c, int64_t n, double2* M, double2* W, const double2* rho0, double* E, double2* f,
                        bool want_vectors) {
    int st;
    const int64_t N = n / 2;
    cublasSetStream(c->cublas, c->stream);
    cusolverDnSetStream(c->cusolver, c->stream);
    {
        cusolverDnParams_t prm;
        if ((st = cusolver_check(c, cusolverDnCreateParams(&prm), "params"))) return st;
        size_t dws = 0, hws = 0;
        st = cusolver_check(c, cusolverDnXpotrf_bufferSize(c->cusolver, prm, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_64F, M, n,
                                                           CUDA_C_64F, &dws, &hws), "potrf size");
        if (!st) st = ensure_work(c, dws + 256);
        if (st) { cusolverDnDestroyParams(prm); return st; }
        int* dinfo = (int*)c->d_work;
        std::vector<char> hbuf(std::max<size_t>(hws, 1));
        st = cusolver_check(c, cusolverDnXpotrf(c->cusolver, prm, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_64F, M, n, CUDA_C_64F,
                                                (char*)c->d_work + 256, dws, hbuf.data(), hws, dinfo), "potrf");
        cusolverDnDestroyParams(prm);
        if (st) return st;
        int info = 0;
        if ((st = cuda_check(c, cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "potrf info"))) return st;
        if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "potrf sync"))) return st;
        if (info != 0) {
            c->h_valid = false;
            return fail(c, BSE_ERR_BAD_INPUT, "full BSE: [[A, B], [B*, A*]] is not positive definite (leading minor " +
                                                  std::to_string(info) + "); the structure-preserving solve needs a stable ground state");
        }
    }
    const unsigned gb = (unsigned)((n * n + 255) / 256);
    jl_kernel<<<gb, 256, 0, c->stream>>>(n, N, M, W);
    c->launches++;
    const cuDoubleComplex one = make_cuDoubleComplex(1, 0);
    if ((st = cublas_check(c, cublasZtrmm(c->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_C, CUBLAS_DIAG_NON_UNIT,
                                          n, n, &one, (const cuDoubleComplex*)M, n, (const cuDoubleComplex*)W, n,
                                          (cuDoubleComplex*)W, n), "L^H J L"))) return st;
    hermitian_part_kernel<<<gb, 256, 0, c->stream>>>(n, W);
    c->launches++;
    // L^{-1} rho(G0)
    if (rho0) {
        if ((st = cuda_check(c, cudaMemcpyAsync(c->d_aux, rho0, n * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream), "rho copy"))) return st;
        if ((st = cublas_check(c, cublasZtrsv(c->cublas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n,
                                              (const cuDoubleComplex*)M, n, (cuDoubleComplex*)c->d_aux, 1), "L^-1 rho"))) return st;
    }
    if ((st = cuda_check(c, cudaGetLastError(), "coupled setup"))) return st;
    if ((st = solve_one(c, n, W, n, true, E, want_vectors ? n : 0, rho0 ? c->d_aux : nullptr, rho0 ? f : nullptr))) return st;
    if (!rho0) return BSE_OK;
    // eigenvectors of H: X = L^{-H} Y, then the J-normalisation of X and of the oscillators
    const int64_t nvec = c->n_vec_valid;
    if (nvec > 0 &&
        (st = cublas_check(c, cublasZtrsm(c->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_C, CUBLAS_DIAG_NON_UNIT,
                                          n, nvec, &one, (const cuDoubleComplex*)M, n, (cuDoubleComplex*)W, n), "L^-H Y")))
        return st;
    jnorm_scale_kernel<<<(unsigned)((n * std::max<int64_t>(nvec, 1) + 255) / 256), 256, 0, c->stream>>>(
        n, nvec, E, W, c->f_from_eig ? f : nullptr);
    c->launches++;
    return cuda_check(c, cudaGetLastError(), "coupled eigenvectors");
}

namespace {

// T = -L^{-1} J (Li = L^{-1} lower, FP32): strict upper triangle cleared, columns j < N negated
__global__ void neg_jl32_kernel(int64_t n, int64_t N, const float2* __restrict__ Li, float2* __restrict__ T) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const int64_t i = t % n, j = t / n;
    float2 l = i >= j ? Li[t] : make_float2(0.f, 0.f);
    if (j < N) l = make_float2(-l.x, -l.y);
    T[t] = l;
}

__global__ void hermitian_part32_kernel(int64_t n, float2* __restrict__ W) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const int64_t i = t % n, j = t / n;
    if (i < j) return;
    if (i == j) {
        W[t].y = 0.f;
        return;
    }
    const float2 a = W[t], b = W[j + n * i];
    const float2 m = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
    W[t] = m;
    W[j + n * i] = make_float2(m.x, -m.y);
}

// y = Li x (Li lower triangular, FP32; x, y FP64): one warp per row
__global__ void trmv_lower32_kernel(int64_t n, const float2* __restrict__ Li, const double2* __restrict__ x,
                                    double2* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (i >= n) return;
    double re = 0, im = 0;
    for (int64_t j = lane; j <= i; j += 32) {
        const float2 l = Li[i + n * j];
        const double2 v = x[j];
        re += (double)l.x * v.x - (double)l.y * v.y;
        im += (double)l.x * v.y + (double)l.y * v.x;
    }
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) y[i] = make_double2(re, im);
}

// mu ascending (eigenvalues of -L^{-1} J L^{-H}, mu = -1/lambda) -> lambda ascending with the
// J-normalised oscillators: negative mu (the first npos) are the positive lambda, in ascending order
__global__ void mu_to_lambda_kernel(int64_t n, int64_t npos, const double* __restrict__ mu, const double2* __restrict__ fmu,
                                    double* __restrict__ E, double2* __restrict__ f) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double lam = -1.0 / mu[t];
    const int64_t o = t < npos ? (n - npos) + t : t - npos;
    E[o] = lam;
    if (f) {
        const double s = sqrt(fabs(lam));
        f[o] = make_double2(fmu[t].x * s, fmu[t].y * s);
    }
}

// S = Pbot - Ptop = -X^H J X (m x m)
__global__ void sub_m_kernel(int64_t mm, const double2* __restrict__ Pt, const double2* __restrict__ Pb, double2* __restrict__ S) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < mm) S[t] = make_double2(Pb[t].x - Pt[t].x, Pb[t].y - Pt[t].y);
}

// refined pair j: E_j = -1/theta_j, x_j = E_j^{1/2} XZ_j (J-normalised), f_j = rho^H x_j,
// residual ||M x - E J x|| / E^{1/2} = ||MXZ_j - E_j J XZ_j||; one block per column
__global__ void coupled_refined_kernel(int64_t n, int64_t N, const double* __restrict__ theta, const double2* __restrict__ XZ,
                                       const double2* __restrict__ MXZ, const double2* __restrict__ rho,
                                       double* __restrict__ E, double2* __restrict__ f, double* __restrict__ res) {
    __shared__ double red[3][32];
    const int j = blockIdx.x;
    const double lam = -1.0 / theta[j];
    const double2* x = XZ + (int64_t)j * n;
    const double2* mx = MXZ + (int64_t)j * n;
    double r2 = 0, fr = 0, fi = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double sg = i < N ? lam : -lam;
        const double dx = mx[i].x - sg * x[i].x, dy = mx[i].y - sg * x[i].y;
        r2 += dx * dx + dy * dy;
        fr += rho[i].x * x[i].x + rho[i].y * x[i].y;     // conj(rho) x
        fi += rho[i].x * x[i].y - rho[i].y * x[i].x;
    }
    for (int o = 16; o > 0; o >>= 1) {
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        fr += __shfl_xor_sync(0xffffffffu, fr, o);
        fi += __shfl_xor_sync(0xffffffffu, fi, o);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[0][w] = r2; red[1][w] = fr; red[2][w] = fi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) { r2 += red[0][k]; fr += red[1][k]; fi += red[2][k]; }
        const double s = sqrt(fabs(lam));
        E[j] = lam;
        f[j] = make_double2(fr * s, fi * s);
        res[j] = sqrt(r2);
    }
}

}  // namespace

// Mixed full BSE (spinless, tamm_dancoff = 0, BSE_MIXED): the FP64 M of the build, its FP32 Cholesky
// factor L and inverse, the Hermitian K = -L^{-1} J L^{-H} whose eigenvalues are mu = -1/lambda (the
// smallest positive excitation energies are the lowest mu), the own FP32 eigensolver on K (all values,
// f from (L^{-1} rho)^H y, the lowest n_refine + guard vectors), then an FP64 Rayleigh-Ritz step on the
// definite pencil J x = (1/E) M x in the span of x = L^{-H} y: (S, G) = (-X^H J X, X^H M X), products
// in compensated FP32, eigenpairs by the Ogita-Aishima refinement (dense fallback).
// One n x n block: M64 the FP64 M (consumed), L / K two n x n FP32 workspaces, E the n eigenvalues,
// rho0 / f the optical vector and oscillators (null for a values-only block, which is not refined).
int mixed_coupled_block(bse_ctx* c, int64_t n, double2* M64, float2* L, float2* K, const double2* rho0, double* E,
                        double2* f) {
    int st;
    const int64_t N = n / 2;
    cublasSetStream(c->cublas, c->stream);
    cusolverDnSetStream(c->cusolver, c->stream);
    narrow_kernel<<<(unsigned)((n * n + 255) / 256), 256, 0, c->stream>>>(n * n, M64, L);
    c->launches++;
    {
        cusolverDnParams_t prm;
        if ((st = cusolver_check(c, cusolverDnCreateParams(&prm), "params"))) return st;
        size_t dws1 = 0, hws1 = 0, dws2 = 0, hws2 = 0;
        st = cusolver_check(c, cusolverDnXpotrf_bufferSize(c->cusolver, prm, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_32F, L, n,
                                                           CUDA_C_32F, &dws1, &hws1), "potrf size");
        if (!st) st = cusolver_check(c, cusolverDnXtrtri_bufferSize(c->cusolver, CUBLAS_FILL_MODE_LOWER, CUBLAS_DIAG_NON_UNIT, n,
                                                                    CUDA_C_32F, L, n, &dws2, &hws2), "trtri size");
        if (!st) st = ensure_work(c, std::max(dws1, dws2) + 256);
        if (st) { cusolverDnDestroyParams(prm); return st; }
        int* dinfo = (int*)c->d_work;
        std::vector<char> hbuf(std::max<size_t>(std::max(hws1, hws2), 1));
        st = cusolver_check(c, cusolverDnXpotrf(c->cusolver, prm, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_32F, L, n, CUDA_C_32F,
                                                (char*)c->d_work + 256, dws1, hbuf.data(), hws1, dinfo), "potrf");
        cusolverDnDestroyParams(prm);
        if (st) return st;
        int info = 0;
        if ((st = cuda_check(c, cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "potrf info"))) return st;
        if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "potrf sync"))) return st;
        if (info != 0)
            return fail(c, BSE_ERR_BAD_INPUT, "full BSE: [[A, B], [B*, A*]] is not positive definite (FP32 leading minor " +
                                                  std::to_string(info) + "); the structure-preserving solve needs a stable ground state");
        if ((st = cusolver_check(c, cusolverDnXtrtri(c->cusolver, CUBLAS_FILL_MODE_LOWER, CUBLAS_DIAG_NON_UNIT, n, CUDA_C_32F, L, n,
                                                     (char*)c->d_work + 256, dws2, hbuf.data(), hws2, dinfo), "trtri"))) return st;
    }
    const unsigned gb = (unsigned)((n * n + 255) / 256);
    neg_jl32_kernel<<<gb, 256, 0, c->stream>>>(n, N, L, K);   // K = -Li J (L now holds Li, lower)
    c->launches++;
    const cuComplex one = make_cuComplex(1.f, 0.f);
    if ((st = cublas_check(c, cublasCtrmm(c->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_C, CUBLAS_DIAG_NON_UNIT,
                                          n, n, &one, (const cuComplex*)L, n, (const cuComplex*)K, n, (cuComplex*)K, n),
                           "-Li J Li^H"))) return st;
    hermitian_part32_kernel<<<gb, 256, 0, c->stream>>>(n, K);
    c->launches++;
    if (rho0) {
        trmv_lower32_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, c->stream>>>(n, L, rho0, c->d_aux);   // L^{-1} rho
        c->launches++;
    }
    if ((st = cuda_check(c, cudaGetLastError(), "mixed coupled setup"))) return st;
    const int64_t m = (rho0 && c->p.n_refine > 0) ? std::min<int64_t>(N, (int64_t)c->p.n_refine + kGuard) : 0;
    const int64_t nref = std::min<int64_t>(N, std::max(c->p.n_refine, 0));
    // mu into the upper half of d_E's storage is not possible (n doubles needed): use the arena top
    double* mu = nullptr;
    double2* fmu = nullptr;
    if ((st = cuda_check(c, cudaMallocAsync((void**)&mu, n * sizeof(double), c->stream), "mu"))) return st;
    if (rho0 && (st = cuda_check(c, cudaMallocAsync((void**)&fmu, n * sizeof(double2), c->stream), "f(mu)"))) return st;
    st = own_heevd(c, (int)n, K, (int)n, false, mu, (int)m, rho0 ? c->d_aux : nullptr, fmu);
    if (!st) {
        // count the negative mu (= positive lambda) on the host
        std::vector<double> hmu(n);
        st = cuda_check(c, cudaMemcpyAsync(hmu.data(), mu, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "mu copy");
        if (!st) st = cuda_check(c, cudaStreamSynchronize(c->stream), "mu sync");
        int64_t npos = 0;
        for (double v : hmu) npos += v < 0.0;
        if (!st && npos < m) st = fail(c, BSE_ERR_NOT_CONVERGED, "full BSE: fewer positive excitations than refined pairs");
        if (!st) {
            mu_to_lambda_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, npos, mu, fmu, E, f);
            c->launches++;
            st = cuda_check(c, cudaGetLastError(), "mu -> lambda");
        }
    }
    cudaFreeAsync(mu, c->stream);
    if (fmu) cudaFreeAsync(fmu, c->stream);
    if (st) return st;
    if (m == 0) return BSE_OK;
    // X = L^{-H} Y for the m lowest mu (the m smallest positive excitation energies)
    if ((st = cublas_check(c, cublasCtrmm(c->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_C, CUBLAS_DIAG_NON_UNIT,
                                          n, m, &one, (const cuComplex*)L, n, (const cuComplex*)K, n, (cuComplex*)K, n),
                           "Li^H Y"))) return st;
    // FP64 Rayleigh-Ritz on the pencil (-J, M) in span(X)
    stage_begin(c, 4);
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t oX = carve(n * m * sizeof(double2)), oY = carve(n * m * sizeof(double2));
    const size_t oXs = carve(n * m * sizeof(float4)), oYs = carve(n * m * sizeof(float4));
    const size_t oS = carve(m * m * sizeof(double2)), oG = carve(m * m * sizeof(double2));
    const size_t oPt = carve(m * m * sizeof(double2)), oPb = carve(m * m * sizeof(double2));
    const size_t oZb = carve(m * m * sizeof(double2)), oT = carve(m * sizeof(double)), oR = carve(m * sizeof(double));
    const size_t oOA = carve(oa_workspace(m)), oP = carve((size_t)kMaxSplits * m * m * sizeof(double2));
    if ((st = ensure_work(c, off))) return st;
    char* base = (char*)c->d_work;
    double2* X = (double2*)(base + oX);
    double2* Y = (double2*)(base + oY);
    float4* X4 = (float4*)(base + oXs);
    float4* Y4 = (float4*)(base + oYs);
    double2* S = (double2*)(base + oS);
    double2* G = (double2*)(base + oG);
    double2* Pt = (double2*)(base + oPt);
    double2* Pb = (double2*)(base + oPb);
    double2* Zb = (double2*)(base + oZb);
    double* theta = (double*)(base + oT);
    double* rn = (double*)(base + oR);
    double2* Pw = (double2*)(base + oP);
    const int64_t pcap = (int64_t)kMaxSplits * m * m;
    widen_kernel<<<(unsigned)((n * m + 255) / 256), 256, 0, c->stream>>>(n * m, K, X);
    float4* M4 = reinterpret_cast<float4*>(M64);   // the FP64 M is split in place (the solve consumes it)
    split_df_kernel<<<(unsigned)((n * n + 255) / 256), 256, 0, c->stream>>>(n * n, M64, M4);
    split_df_kernel<<<(unsigned)((n * m + 255) / 256), 256, 0, c->stream>>>(n * m, X, X4);
    c->launches += 3;
    hemm_df_kernel<<<dim3((unsigned)((n + HM_TM - 1) / HM_TM), (unsigned)((m + HM_TN - 1) / HM_TN)), 256, 0, c->stream>>>(
        (int)n, (int)m, M4, X4, Y);                                                                            // M X
    split_df_kernel<<<(unsigned)((n * m + 255) / 256), 256, 0, c->stream>>>(n * m, Y, Y4);
    c->launches += 2;
    if ((st = gemm_df(c, true, (int)m, (int)m, (int)n, (const float4*)X4, n, (const float4*)Y4, n, G, m, Pw, pcap))) return st;    // X^H M X
    if ((st = gemm_df(c, true, (int)m, (int)m, (int)N, (const float4*)X4, n, (const float4*)X4, n, Pt, m, Pw, pcap))) return st;   // top rows
    if ((st = gemm_df(c, true, (int)m, (int)m, (int)N, (const float4*)(X4 + N), n, (const float4*)(X4 + N), n, Pb, m, Pw, pcap))) return st;
    sub_m_kernel<<<(unsigned)((m * m + 255) / 256), 256, 0, c->stream>>>(m * m, Pt, Pb, S);                    // -X^H J X
    c->launches++;
    bool refined = false;
    if ((st = oa_refine(c, (int)m, S, G, Zb, theta, Pw, pcap, base + oOA, &refined))) return st;
    if (!refined) return fail(c, BSE_ERR_NOT_CONVERGED, "full BSE: the pencil refinement did not converge");
    // refined vectors XZ (M-normalised) and M XZ; then E, J-normalised f and residuals of the lowest nref
    if ((st = gemm_df(c, false, (int)n, (int)m, (int)m, (const float4*)X4, n, (const double2*)Zb, m, X, n, Pw, pcap))) return st;  // X Z
    if ((st = gemm_df(c, false, (int)n, (int)m, (int)m, (const float4*)Y4, n, (const double2*)Zb, m, Y, n, Pw, pcap))) return st;  // M X Z
    coupled_refined_kernel<<<(unsigned)nref, 256, 0, c->stream>>>(n, N, theta, X, Y, rho0, E + N, f + N, rn);
    c->launches++;
    std::vector<double> hrn(nref);
    if ((st = cuda_check(c, cudaMemcpyAsync(hrn.data(), rn, nref * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "residuals"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "residuals"))) return st;
    c->max_residual = 0;
    for (double v : hrn) c->max_residual = std::max(c->max_residual, v);
    c->n_refined = nref;
    stage_end(c, 4);
    return cuda_check(c, cudaGetLastError(), "mixed coupled refinement");
}

// collinear full BSE: the two 4N x 4N blocks are solved in turn and each must be positive
// definite; an error names the block (rows of the 8N matrix in the reference's layout)
constexpr const char* kBlockM0 = "collinear full BSE, spin-flip block M0 (exciton spin blocks 1, 2: rows N..3N-1 and 5N..7N-1): ";
constexpr const char* kBlockM1 = "collinear full BSE, optically active block M1 (exciton spin blocks 0, 3: rows 0..N-1, 3N..5N-1, 7N..8N-1): ";

int run_eig_coupled_mixed(bse_ctx* c) {
    int st;
    const double2* rho0 = c->d_rho + (size_t)c->n_rho * (c->ng / 2);
    c->f_from_eig = true;
    c->n_vec_valid = 0;
    c->n_refined = 0;
    if (c->S == 0) {
        const int64_t n = c->n_h;
        float2* L = (float2*)c->d_blk;
        return mixed_coupled_block(c, n, (double2*)c->d_H, L, L + n * n, rho0, c->d_E, c->d_f);
    }
    // collinear: M0 (values only) and the optically active M1, each 4N; L and K in the third slot
    const int64_t n4 = c->n_opt;
    double2* M0 = (double2*)c->d_blk;
    double2* M1 = M0 + n4 * n4;
    float2* L = (float2*)(M1 + n4 * n4);
    if ((st = mixed_coupled_block(c, n4, M0, L, L + n4 * n4, nullptr, c->d_E, nullptr))) {
        c->err = std::string(kBlockM0) + c->err;
        return st;
    }
    if ((st = mixed_coupled_block(c, n4, M1, L, L + n4 * n4, rho0, c->d_E + n4, c->d_f))) c->err = std::string(kBlockM1) + c->err;
    return st;
}

int run_eig_coupled(bse_ctx* c, bool want_vectors) {
    int st;
    if (c->p.precision == BSE_MIXED) {
        if (want_vectors)
            return fail(c, BSE_ERR_STATE, "the mixed full BSE forms no eigenvectors: use precision = BSE_FP64 for a_out");
        return run_eig_coupled_mixed(c);
    }
    const double2* rho0 = c->d_rho + (size_t)c->n_rho * (c->ng / 2);
    if (c->S == 0) {
        double2* W = (double2*)c->d_blk;
        if ((st = solve_coupled_block(c, c->n_h, (double2*)c->d_H, W, rho0, c->d_E, c->d_f, want_vectors))) return st;
        c->d_A = W;
        return BSE_OK;
    }
    // collinear: M0 = spin blocks {1,2} (values only, 3195, 3317) and M1 = {0,3}, the optically
    // active block (Q17), each 4N x 4N with its coupling part
    const int64_t n4 = c->n_opt;
    double2* M0 = (double2*)c->d_blk;
    double2* M1 = M0 + n4 * n4;
    double2* W = M1 + n4 * n4;
    if ((st = solve_coupled_block(c, n4, M0, W, nullptr, c->d_E, nullptr, false))) {
        c->err = std::string(kBlockM0) + c->err;
        return st;
    }
    if ((st = solve_coupled_block(c, n4, M1, W, rho0, c->d_E + n4, c->d_f, want_vectors))) {
        c->err = std::string(kBlockM1) + c->err;
        return st;
    }
    c->d_A = W;
    return BSE_OK;
}

int run_eig(bse_ctx* c, bool want_vectors) {
    int st;
    if (!c->h_valid) return fail(c, BSE_ERR_STATE, "BSE matrix not built (diagonalize consumes it; rebuild first)");
    stage_begin(c, 3);
    if (c->coupled) {
        c->n_refined = 0;
        st = run_eig_coupled(c, want_vectors);
        c->h_valid = false;
        if (st) return st;
        stage_end(c, 3);
        c->eig_valid = true;
        c->osc_valid = false;
        return BSE_OK;
    }
    const bool fp64 = c->p.precision == BSE_FP64;
    const bool refine = !fp64 && !c->p.ipa && c->p.n_refine > 0;
    const int64_t n_opt = c->n_opt;
    const int64_t n_vec = want_vectors ? n_opt : (refine ? std::min<int64_t>(n_opt, (int64_t)c->p.n_refine + kGuard) : 0);
    const double2* rho0 = c->d_rho + (size_t)c->n_rho * (c->ng / 2);
    c->n_refined = 0;
    if (c->S == 0) {
        st = solve_one(c, c->N, c->d_H, c->N, fp64, c->d_E, n_vec, rho0, c->d_f);
        if (st) return st;
        c->d_A = c->d_H;
    } else {
        const int64_t n2 = 2 * c->N;
        char* b0 = (char*)c->d_blk;
        char* b1 = b0 + (size_t)n2 * n2 * c->h_elem;
        if ((st = solve_one(c, n2, b0, n2, fp64, c->d_E, 0, nullptr, nullptr))) return st;      // H0: values only (3317)
        if ((st = solve_one(c, n2, b1, n2, fp64, c->d_E + n2, n_vec, rho0, c->d_f))) return st;  // H1: optically active
        c->d_A = b1;
    }
    stage_end(c, 3);
    c->h_valid = false;
    if (refine) {
        if ((st = run_refine(c))) return st;
    }
    c->eig_valid = true;
    c->osc_valid = false;
    return BSE_OK;
}

// One FP64 Rayleigh-Ritz step on the lowest m FP32 Ritz vectors of the optically active block.
int run_refine(bse_ctx* c) {
    int st;
    stage_begin(c, 4);
    const int64_t n = c->n_opt;
    const int64_t m = std::min<int64_t>(n, (int64_t)c->p.n_refine + kGuard);
    const int64_t nref = std::min<int64_t>(n, c->p.n_refine);
    // FP64 matrix of the solved block, lower triangle: built here, or waited for on the side stream
    if (c->h64_pending) {
        if ((st = build_h64(c))) return st;
    } else if (c->h64_side) {
        if ((st = cuda_check(c, cudaStreamWaitEvent(c->stream, c->ev_h64, 0), "FP64 build wait"))) return st;
        c->h64_side = false;
    }
    double2* H64 = c->d_H64;
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t oX = carve(n * m * sizeof(double2)), oY = carve(n * m * sizeof(double2));
    const size_t oZ = carve(n * m * sizeof(double2)), oN = carve(m * sizeof(double));
    const size_t oG = carve(m * m * sizeof(double2)), oT = carve(m * sizeof(double));
    const size_t oGm = carve(m * m * sizeof(double2)), oZb = carve(m * m * sizeof(double2)), oOA = carve(oa_workspace(m));
    const size_t oXs = carve(n * m * sizeof(float4)), oYs = carve(n * m * sizeof(float4));
    const size_t oP = carve((size_t)kMaxSplits * m * m * sizeof(double2));
    const size_t oB = c->S ? carve((size_t)n * n * sizeof(double2)) : 0;
    // potrf / heevd workspaces on top
    cusolverDnParams_t prm;
    if ((st = cusolver_check(c, cusolverDnCreateParams(&prm), "params"))) return st;
    size_t dws1 = 0, hws1 = 0, dws2 = 0, hws2 = 0;
    if ((st = cusolver_check(c, cusolverDnXpotrf_bufferSize(c->cusolver, prm, CUBLAS_FILL_MODE_LOWER, m, CUDA_C_64F, nullptr, m,
                                                            CUDA_C_64F, &dws1, &hws1), "potrf size"))) return st;
    if ((st = cusolver_check(c, cusolverDnXsyevd_bufferSize(c->cusolver, prm, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m,
                                                            CUDA_C_64F, nullptr, m, CUDA_R_64F, nullptr, CUDA_C_64F, &dws2, &hws2),
                             "heevd size"))) return st;
    const size_t oW = carve(std::max(dws1, dws2) + 256);
    if ((st = ensure_work(c, off))) return st;
    char* base = (char*)c->d_work;
    double2* X = (double2*)(base + oX);
    double2* Y = (double2*)(base + oY);
    double2* G = (double2*)(base + oG);
    double2* Pw = (double2*)(base + oP);
    const int64_t pcap = (int64_t)kMaxSplits * m * m;
    double* theta = (double*)(base + oT);
    int* dinfo = (int*)(base + oW);
    void* dws = base + oW + 256;
    std::vector<char> hws(std::max<size_t>(std::max(hws1, hws2), 1));
    if (c->S) {
        // collinear: FP64 H1 = blocks {0,3} of the rotated FP64 matrix
        double2* B = (double2*)(base + oB);
        const int64_t N = c->N, ld = 4 * N;
        for (int bj = 0; bj < 2; bj++)
            for (int bi = 0; bi < 2; bi++) {
                const double2* src = H64 + (bi * 3 * N) + ld * (bj * 3 * N);
                double2* dst = B + bi * N + n * (bj * N);
                if ((st = cuda_check(c, cudaMemcpy2DAsync(dst, n * sizeof(double2), src, ld * sizeof(double2), N * sizeof(double2), N,
                                                          cudaMemcpyDeviceToDevice, c->stream), "H1 gather"))) return st;
            }
        H64 = B;
    }
    // X = widen(A[:, :m])
    widen_kernel<<<(unsigned)((n * m + 255) / 256), 256, 0, c->stream>>>(n * m, (const float2*)c->d_A, X);
    c->launches++;
    const cuDoubleComplex one = make_cuDoubleComplex(1, 0), zero = make_cuDoubleComplex(0, 0);
    cublasSetStream(c->cublas, c->stream);
    cusolverDnSetStream(c->cusolver, c->stream);
    // M = X^H X, Y = H X (Hermitian, lower triangle), S = X^H Y: products in compensated FP32
    double2* Gm = (double2*)(base + oGm);
    double2* Zb = (double2*)(base + oZb);
    // split H (in place: the FP64 copy is rebuilt by every build) and X into FP32 pairs once
    float4* H4 = reinterpret_cast<float4*>(H64);
    float4* X4 = (float4*)(base + oXs);
    split_df_kernel<<<(unsigned)((n * n + 255) / 256), 256, 0, c->stream>>>(n * n, H64, H4);
    split_df_kernel<<<(unsigned)((n * m + 255) / 256), 256, 0, c->stream>>>(n * m, X, X4);
    c->launches += 2;
    if ((st = gemm_df(c, true, (int)m, (int)m, (int)n, (const float4*)X4, n, (const float4*)X4, n, Gm, m, Pw, pcap))) return st;   // X^H X
    hemm_df_kernel<<<dim3((unsigned)((n + HM_TM - 1) / HM_TM), (unsigned)((m + HM_TN - 1) / HM_TN)), 256, 0, c->stream>>>(
        (int)n, (int)m, H4, X4, Y);
    c->launches++;
    if ((st = cuda_check(c, cudaGetLastError(), "refinement product"))) return st;
    float4* Y4 = (float4*)(base + oYs);
    split_df_kernel<<<(unsigned)((n * m + 255) / 256), 256, 0, c->stream>>>(n * m, Y, Y4);
    c->launches++;
    if ((st = gemm_df(c, true, (int)m, (int)m, (int)n, (const float4*)X4, n, (const float4*)Y4, n, G, m, Pw, pcap))) return st;   // X^H Y
    // eigenpairs of the pencil (S, M): iterative refinement from Z = I (the FP32 Ritz vectors nearly
    // diagonalise it), or, for wide clusters / BSE_REFINE_EIG=cusolver|dense, a dense solve of
    // L^{-1} S L^{-H} (M = L L^H) by this library's FP64 solver or cuSOLVER heevd
    const int refine_mode = [] {
        const char* v = std::getenv("BSE_REFINE_EIG");
        if (!v) return 0;
        const std::string md(v);
        return md == "cusolver" ? 2 : (md == "dense" ? 1 : 0);
    }();
    bool refined = false;
    if (refine_mode == 0) {
        if ((st = oa_refine(c, (int)m, G, Gm, Zb, theta, Pw, pcap, base + oOA, &refined))) return st;
    }
    if (!refined) {
        if ((st = cusolver_check(c, cusolverDnXpotrf(c->cusolver, prm, CUBLAS_FILL_MODE_LOWER, m, CUDA_C_64F, Gm, m, CUDA_C_64F,
                                                     dws, dws1, hws.data(), hws1, dinfo), "potrf"))) return st;
        cuDoubleComplex* L = (cuDoubleComplex*)Gm;
        cuDoubleComplex* Gc = (cuDoubleComplex*)G;
        if ((st = cublas_check(c, cublasZtrsm(c->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT,
                                              m, m, &one, L, m, Gc, m), "trsm"))) return st;
        if ((st = cublas_check(c, cublasZtrsm(c->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_C, CUBLAS_DIAG_NON_UNIT,
                                              m, m, &one, L, m, Gc, m), "trsm"))) return st;
        if (refine_mode == 2) {
            if ((st = cusolver_check(c, cusolverDnXsyevd(c->cusolver, prm, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, CUDA_C_64F,
                                                         G, m, CUDA_R_64F, theta, CUDA_C_64F, dws, dws2, hws.data(), hws2, dinfo),
                                     "heevd m"))) return st;
        } else {
            hermitize_lower_kernel<<<(unsigned)((m * m + 255) / 256), 256, 0, c->stream>>>((int)m, G);
            c->launches++;
            if ((st = own_heevd(c, (int)m, G, (int)m, true, theta, (int)m, nullptr, nullptr, true))) return st;
        }
        if ((st = cublas_check(c, cublasZtrsm(c->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_C, CUBLAS_DIAG_NON_UNIT,
                                              m, m, &one, L, m, Gc, m), "trsm"))) return st;
        if ((st = cuda_check(c, cudaMemcpyAsync(Zb, G, m * m * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream), "Z"))) return st;
    }
    cusolverDnDestroyParams(prm);
    // XZ = X Z (refined Ritz vectors) and HXZ = (H X) Z; residuals r_j = HXZ_j - theta_j XZ_j
    double2* XZ = (double2*)(base + oZ);
    if ((st = gemm_df(c, false, (int)n, (int)m, (int)m, (const float4*)X4, n, (const double2*)Zb, m, XZ, n, Pw, pcap))) return st;   // X Z
    if ((st = gemm_df(c, false, (int)n, (int)m, (int)m, (const float4*)Y4, n, (const double2*)Zb, m, X, n, Pw, pcap))) return st;    // (H X) Z
    double* rn = (double*)(base + oN);
    residual_kernel<<<(unsigned)nref, 256, 0, c->stream>>>(n, X, XZ, theta, rn);
    c->launches++;
    Y = XZ;
    // write back the lowest nref pairs
    double* E = c->S ? c->d_E + 2 * c->N : c->d_E;
    if ((st = cuda_check(c, cudaMemcpyAsync(E, theta, nref * sizeof(double), cudaMemcpyDeviceToDevice, c->stream), "theta"))) return st;
    narrow_kernel<<<(unsigned)((n * nref + 255) / 256), 256, 0, c->stream>>>(n * nref, Y, (float2*)c->d_A);
    c->launches++;
    c->n_refined = nref;
    std::vector<double> hrn(nref);
    if ((st = cuda_check(c, cudaMemcpyAsync(hrn.data(), rn, nref * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "residuals"))) return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "residuals"))) return st;
    c->max_residual = 0;
    for (double v : hrn) c->max_residual = std::max(c->max_residual, v);
    stage_end(c, 4);
    return cuda_check(c, cudaGetLastError(), "refine");
}

}  // namespace bse
