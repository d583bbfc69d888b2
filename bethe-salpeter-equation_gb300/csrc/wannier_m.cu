// Real-space Wannier matrix elements M_ab(q + G) from Wannier functions sampled on a supercell
// grid (the reference's Real_space_wannier + Dipole_Elements, bse.version13.cpp:1081-1212,
// 1441-1456, 1503-1650).  The reference evaluates, for every Wannier pair and G, loops over the
// integration cells and every point of the supercell grid (its OpenMP-parallel hot spot); here a
// block per (spin, w1, w2, G) sums over the grid points, every thread a strided share of them,
// in FP64 with a fixed-order block reduction.
//
//   normalisation (1141-1150): every function scaled so that sum w^2 * Nsc V / Npts = 1;
//   A[spin, R1] (1503-1533) = Nsc V / Npts * sum over points X of the grid with X - d n_pc inside it
//       exp(i (q + G).r(X)) w1(X - d n_pc) w2(X),   d = R1 - n_int / 2 (cells), r(X) = origin +
//       sum_p (X_p / n_pc,p) a_p (a_p = the cell axes: the supercell spanning vectors / cells);
//   small q (1535-1570, 1611-1636): the phase is replaced by i qhat.r(X) and G does not enter;
//   M[G][spin nw + w1, spin nw + w2] (1580-1650) = sum_R1 exp(i q.(o + R)) A[spin, R1], with
//       R = d_0 b_0 + d_1 b_1 + d_2 b_2 (b = the Bravais lattice) and o = origin_unitcell, the
//       cell indices of the supercell cell nearest to zero, added to the cartesian R as the
//       reference does (quirk Q32).
// Blocks of different spin channels stay zero (the reference's M is block-diagonal in spin).
#include "bse_internal.h"

namespace bse {
namespace {

constexpr int kWmThreads = 256;

struct WmArgs {
    int n_spin, nw, n_g, small_q;
    int grid[3], per_cell[3], n_int[3];
    double factor;
    double origin[3], axes[9];   // cell axes a_p as rows
    double lat[9];               // Bravais vectors b_p as rows
    double q[3], qhat[3], o[3];
    const double* f;             // [n_spin][nw][NX][NY][NZ], Z fastest
    const double* inv;           // [n_spin][nw] 1 / sqrt(norm)
    const double* g;             // [n_g][3]
    double2* m;                  // [n_g][nb][nb]
};

__device__ __forceinline__ double block_sum_d(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];   // fixed order
    return t;
}

// 1 / sqrt(sum w^2 * factor), a block per function
__global__ void __launch_bounds__(kWmThreads) wannier_norm_kernel(int64_t npts, double factor, const double* __restrict__ f,
                                                                   double* __restrict__ inv) {
    __shared__ double red[32];
    const double* fw = f + (int64_t)blockIdx.x * npts;
    double s = 0;
    for (int64_t p = threadIdx.x; p < npts; p += blockDim.x) s += fw[p] * fw[p];
    s = block_sum_d(s, red);
    if (threadIdx.x == 0) inv[blockIdx.x] = 1.0 / sqrt(s * factor);
}

__global__ void __launch_bounds__(kWmThreads) wannier_m_kernel(WmArgs a) {
    __shared__ double red[32];
    const int blk = blockIdx.x;
    const int gi = blk % a.n_g, w2 = (blk / a.n_g) % a.nw, w1 = (blk / (a.n_g * a.nw)) % a.nw,
              spin = blk / (a.n_g * a.nw * a.nw);
    const int NX = a.grid[0], NY = a.grid[1], NZ = a.grid[2];
    const int64_t npts = (int64_t)NX * NY * NZ;
    const double* f1 = a.f + ((int64_t)spin * a.nw + w1) * npts;
    const double* f2 = a.f + ((int64_t)spin * a.nw + w2) * npts;
    const double scale = a.factor * a.inv[spin * a.nw + w1] * a.inv[spin * a.nw + w2];
    double k[3];
    for (int c = 0; c < 3; c++) k[c] = a.q[c] + (a.small_q ? 0.0 : a.g[3 * gi + c]);
    double mre = 0, mim = 0;
    for (int i1 = 0; i1 < a.n_int[0]; i1++)
        for (int j1 = 0; j1 < a.n_int[1]; j1++)
            for (int k1 = 0; k1 < a.n_int[2]; k1++) {
                const int d0 = i1 - a.n_int[0] / 2, d1 = j1 - a.n_int[1] / 2, d2 = k1 - a.n_int[2] / 2;
                const int s0 = d0 * a.per_cell[0], s1 = d1 * a.per_cell[1], s2 = d2 * a.per_cell[2];
                double sre = 0, sim = 0;
                for (int64_t p = threadIdx.x; p < npts; p += blockDim.x) {
                    const int Z = (int)(p % NZ), Y = (int)((p / NZ) % NY), X = (int)(p / ((int64_t)NY * NZ));
                    const int Xs = X - s0, Ys = Y - s1, Zs = Z - s2;
                    if (Xs < 0 || Xs >= NX || Ys < 0 || Ys >= NY || Zs < 0 || Zs >= NZ) continue;
                    const double v = f1[((int64_t)Xs * NY + Ys) * NZ + Zs] * f2[p];
                    const double fx = (double)X / a.per_cell[0], fy = (double)Y / a.per_cell[1],
                                 fz = (double)Z / a.per_cell[2];
                    double r[3];
                    for (int c = 0; c < 3; c++) r[c] = a.origin[c] + fx * a.axes[c] + fy * a.axes[3 + c] + fz * a.axes[6 + c];
                    if (a.small_q) {
                        // i qhat.r: imaginary only
                        sim += v * (a.qhat[0] * r[0] + a.qhat[1] * r[1] + a.qhat[2] * r[2]);
                    } else {
                        double sn, cs;
                        sincos(k[0] * r[0] + k[1] * r[1] + k[2] * r[2], &sn, &cs);
                        sre += v * cs;
                        sim += v * sn;
                    }
                }
                sre = block_sum_d(sre, red);
                sim = block_sum_d(sim, red);
                if (threadIdx.x == 0) {
                    sre *= scale;
                    sim *= scale;
                    double ph = 0;
                    for (int c = 0; c < 3; c++)
                        ph += a.q[c] * (a.o[c] + d0 * a.lat[c] + d1 * a.lat[3 + c] + d2 * a.lat[6 + c]);
                    double sn, cs;
                    sincos(ph, &sn, &cs);
                    mre += cs * sre - sn * sim;
                    mim += sn * sre + cs * sim;
                }
            }
    if (threadIdx.x == 0) {
        const int nb = a.n_spin * a.nw;
        a.m[((int64_t)gi * nb + spin * a.nw + w1) * nb + spin * a.nw + w2] = make_double2(mre, mim);
    }
}

}  // namespace
}  // namespace bse

extern "C" int bse_wannier_m(int32_t n_spin, int32_t nw, const int32_t* grid, const int32_t* cells,
                             const double* f, double cell_volume, const double* origin, const double* axes,
                             const double* lattice, const int32_t* n_int, const double* q, int32_t n_g,
                             const double* g_list, int32_t small_q, double* m_out) {
    using bse::fail;
    if (n_spin < 1 || n_spin > 2 || nw < 1 || n_g < 1 || !grid || !cells || !f || !origin || !axes || !lattice ||
        !n_int || !q || !m_out || (!small_q && !g_list))
        return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_wannier_m: bad sizes or null pointer");
    bse::WmArgs a{};
    a.n_spin = n_spin;
    a.nw = nw;
    a.n_g = n_g;
    a.small_q = small_q ? 1 : 0;
    int64_t npts = 1;
    int64_t ncells = 1;
    for (int p = 0; p < 3; p++) {
        if (grid[p] < 1 || cells[p] < 1 || grid[p] % cells[p] || n_int[p] < 1)
            return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_wannier_m: grid points per direction must be a positive multiple of the cells");
        a.grid[p] = grid[p];
        a.per_cell[p] = grid[p] / cells[p];
        a.n_int[p] = n_int[p];
        npts *= grid[p];
        ncells *= cells[p];
    }
    a.factor = (double)ncells * cell_volume / (double)npts;
    for (int c = 0; c < 3; c++) {
        a.origin[c] = origin[c];
        a.q[c] = q[c];
        for (int p = 0; p < 3; p++) {
            a.axes[3 * p + c] = axes[3 * p + c] / cells[p];
            a.lat[3 * p + c] = lattice[3 * p + c];
        }
    }
    const double qn = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    if (a.small_q && qn == 0) return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_wannier_m: the small-q branch needs q != 0");
    for (int c = 0; c < 3; c++) a.qhat[c] = qn > 0 ? q[c] / qn : 0.0;
    // origin_unitcell: the supercell cell whose corner is nearest to zero, strict "<" from (0, 0, 0)
    double best = sqrt(origin[0] * origin[0] + origin[1] * origin[1] + origin[2] * origin[2]);
    a.o[0] = a.o[1] = a.o[2] = 0;
    for (int i = 0; i < cells[0]; i++)
        for (int j = 0; j < cells[1]; j++)
            for (int k = 0; k < cells[2]; k++) {
                double c2 = 0;
                for (int c = 0; c < 3; c++) {
                    const double x = origin[c] + i * a.axes[c] + j * a.axes[3 + c] + k * a.axes[6 + c];
                    c2 += x * x;
                }
                if (sqrt(c2) < best) {
                    best = sqrt(c2);
                    a.o[0] = i;
                    a.o[1] = j;
                    a.o[2] = k;
                }
            }
    const int nb = n_spin * nw;
    const size_t fbytes = (size_t)n_spin * nw * npts * sizeof(double);
    const size_t mbytes = (size_t)n_g * nb * nb * sizeof(double2);
    double *df = nullptr, *dinv = nullptr, *dg = nullptr;
    double2* dm = nullptr;
    int st = BSE_OK;
    auto release = [&]() {
        for (void* p : {(void*)df, (void*)dinv, (void*)dg, (void*)dm})
            if (p) cudaFree(p);
    };
    if ((st = bse::cuda_check(nullptr, cudaMalloc(&df, fbytes), "bse_wannier_m: grid")) ||
        (st = bse::cuda_check(nullptr, cudaMalloc(&dinv, (size_t)n_spin * nw * sizeof(double)), "bse_wannier_m: norms")) ||
        (st = bse::cuda_check(nullptr, cudaMalloc(&dg, (size_t)n_g * 3 * sizeof(double)), "bse_wannier_m: G")) ||
        (st = bse::cuda_check(nullptr, cudaMalloc(&dm, mbytes), "bse_wannier_m: M"))) {
        release();
        return st;
    }
    if ((st = bse::cuda_check(nullptr, cudaMemcpy(df, f, fbytes, cudaMemcpyHostToDevice), "bse_wannier_m: grid upload")) ||
        (st = bse::cuda_check(nullptr, g_list ? cudaMemcpy(dg, g_list, (size_t)n_g * 3 * sizeof(double), cudaMemcpyHostToDevice)
                                              : cudaMemset(dg, 0, (size_t)n_g * 3 * sizeof(double)), "bse_wannier_m: G upload")) ||
        (st = bse::cuda_check(nullptr, cudaMemset(dm, 0, mbytes), "bse_wannier_m: M clear"))) {
        release();
        return st;
    }
    a.f = df;
    a.inv = dinv;
    a.g = dg;
    a.m = dm;
    bse::wannier_norm_kernel<<<n_spin * nw, bse::kWmThreads>>>(npts, a.factor, df, dinv);
    bse::wannier_m_kernel<<<(unsigned)(n_spin * nw * nw * n_g), bse::kWmThreads>>>(a);
    st = bse::cuda_check(nullptr, cudaGetLastError(), "bse_wannier_m: launch");
    if (!st) st = bse::cuda_check(nullptr, cudaMemcpy(m_out, dm, mbytes, cudaMemcpyDeviceToHost), "bse_wannier_m: copy back");
    release();
    return st;
}
