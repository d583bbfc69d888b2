// Allocation-free evaluation of the dielectric function from eigenvalues and oscillator
// strengths (no counterpart in the reference).
//
// Some callers cannot call cudaMalloc: code embedded in a framework that has already reserved
// the device memory for its own pool (a JAX/XLA preallocation, a PyTorch caching allocator at its
// limit) gets no memory from the CUDA allocator, however small the request.  bse_eps_noalloc
// serves them: it stages its inputs and outputs in one file-scope device array of fixed size
// instead of allocating.
//
//   - Limits: n_exc <= BSE_EPS_NOALLOC_MAX_EXCITONS (131072) and
//     n_omega <= BSE_EPS_NOALLOC_MAX_OMEGA (16384); larger requests return
//     BSE_ERR_BAD_INPUT.  The array is 3.4 MiB, and every GPU that loads this library
//     holds it until the process exits.
//   - Set-up: the first call on a device, with that device current, resolves the array's
//     device address (cudaGetSymbolAddress) and keeps it for the rest of the process; make that
//     first call before any stream capture.  A cudaDeviceReset reloads the module and leaves
//     the kept address stale: do not call this entry point again after resetting the device.
//   - Each call copies its inputs to the array, runs the kernel and copies the outputs back on
//     `stream`, and returns once the outputs are on the host (it waits for the stream).
//   - Sharing: every call uses the same array, which keeps the last call's contents.
//     Every output element is written by the kernel, so nothing has to start at zero.
//     Calls that overlap on the GPU (other streams, other host threads) race on the
//     array: serialise them.
#include <mutex>

#include "bse_internal.h"

namespace bse {
cudaError_t launch_eps_raw(int64_t n, const double* E, const double2* f, const double* omega, int n_omega,
                           double gamma, double F, double* eps2, double* eps1, cudaStream_t stream);
}

namespace {

constexpr int64_t kMaxExc = BSE_EPS_NOALLOC_MAX_EXCITONS;
constexpr int64_t kMaxOmega = BSE_EPS_NOALLOC_MAX_OMEGA;
// [E: kMaxExc doubles][f: kMaxExc double2][omega | eps2 | eps1: kMaxOmega doubles each]
constexpr size_t kOffF = kMaxExc * sizeof(double);
constexpr size_t kOffOmega = kOffF + kMaxExc * sizeof(double2);
constexpr size_t kOffEps2 = kOffOmega + kMaxOmega * sizeof(double);
constexpr size_t kOffEps1 = kOffEps2 + kMaxOmega * sizeof(double);
constexpr size_t kScratchBytes = kOffEps1 + kMaxOmega * sizeof(double);

static __device__ __align__(256) unsigned char g_eps_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of the scratch array for the current device (host code may not use the
// symbol itself: on the host it names a stand-in, not device memory).
int scratch_address(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_eps_scratch);
        if (e != cudaSuccess) return bse::cuda_check(nullptr, e, "bse_eps_noalloc: cudaGetSymbolAddress");
        g_addr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_addr[dev]);
    return BSE_OK;
}

}  // namespace

extern "C" int bse_eps_noalloc(int64_t n_exc, const double* e, const double* f, double prefactor,
                               const double* omega, int32_t n_omega, double gamma,
                               double* eps2, double* eps1, void* stream) {
    using bse::fail;
    if (n_exc < 1 || n_exc > kMaxExc)
        return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_eps_noalloc: n_exc must be in [1, 131072]");
    if (n_omega < 1 || n_omega > kMaxOmega)
        return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_eps_noalloc: n_omega must be in [1, 16384]");
    if (!e || !f || !omega || (!eps2 && !eps1))
        return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_eps_noalloc: null input or no output");
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return bse::cuda_check(nullptr, ce, "bse_eps_noalloc: no current device");
    if (dev < 0 || dev >= kMaxDevices) return fail(nullptr, BSE_ERR_BAD_INPUT, "bse_eps_noalloc: device index");
    unsigned char* base = nullptr;
    int st = scratch_address(dev, &base);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* dE = reinterpret_cast<double*>(base);
    double2* dF = reinterpret_cast<double2*>(base + kOffF);
    double* dOm = reinterpret_cast<double*>(base + kOffOmega);
    double* dE2 = reinterpret_cast<double*>(base + kOffEps2);
    double* dE1 = reinterpret_cast<double*>(base + kOffEps1);
    if ((st = bse::cuda_check(nullptr, cudaMemcpyAsync(dE, e, n_exc * sizeof(double), cudaMemcpyHostToDevice, s), "E upload"))) return st;
    if ((st = bse::cuda_check(nullptr, cudaMemcpyAsync(dF, f, n_exc * sizeof(double2), cudaMemcpyHostToDevice, s), "f upload"))) return st;
    if ((st = bse::cuda_check(nullptr, cudaMemcpyAsync(dOm, omega, n_omega * sizeof(double), cudaMemcpyHostToDevice, s), "omega upload"))) return st;
    if ((st = bse::cuda_check(nullptr, bse::launch_eps_raw(n_exc, dE, dF, dOm, n_omega, gamma, prefactor, dE2, dE1, s), "eps kernel"))) return st;
    if (eps2 && (st = bse::cuda_check(nullptr, cudaMemcpyAsync(eps2, dE2, n_omega * sizeof(double), cudaMemcpyDeviceToHost, s), "eps2 copy"))) return st;
    if (eps1 && (st = bse::cuda_check(nullptr, cudaMemcpyAsync(eps1, dE1, n_omega * sizeof(double), cudaMemcpyDeviceToHost, s), "eps1 copy"))) return st;
    return bse::cuda_check(nullptr, cudaStreamSynchronize(s), "bse_eps_noalloc");
}
