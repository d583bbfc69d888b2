// Device helpers shared by the eigensolver kernels: complex arithmetic on float2 / double2,
// warp and block reductions, and the bounded grid-wide barrier of the cooperative kernels.
#pragma once

#include <cuda_runtime.h>

namespace bse {
namespace dev {

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

// The polling limit of the waits that report through the error word err[0]: err[1] when it is
// nonzero (a test override, BSE_TEST_SPIN_LIMIT at bse_create), else kSpinLimit.  The solver's
// error word always has the second int beside it.  The waits check the error word every few
// hundred polls, and at once when a poll count passes the limit.
__device__ __forceinline__ unsigned spin_limit(const int* err) {
    const unsigned v = reinterpret_cast<const volatile unsigned*>(err)[1];
    return v ? v : kSpinLimit;
}

// Grid-wide barrier for a cooperative launch.  bar[0] holds the arrivals of the current
// barrier in its low 16 bits and a generation number in its high 16 bits: each block adds 1
// (acquire-release, so its writes are published and the earlier arrivals' are seen); the last
// arrival adds 2^16 - gridDim.x (release), which clears the count and starts the next
// generation; the others poll with acquire loads until the generation changes.  One atomic
// round trip for the last block and one poll for the rest, and the word is back to a zero count
// after every completed barrier, so kernels with different grid sizes can share it.
// Returns false (after setting *err on a timeout) if a block did not arrive in time or another
// block failed.
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void red_add_release(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned lim = spin_limit(err);
        const unsigned old = atom_add_acq_rel(bar, 1u);
        const unsigned gen = old >> 16;
        if ((old & 0xffffu) == gridDim.x - 1) {
            red_add_release(bar, 0x10000u - gridDim.x);
        } else {
            unsigned it = 0;
            while ((ld_acquire(bar) >> 16) == gen) {
                if ((++it & 255u) == 0 || it > lim) {
                    if (*(volatile int*)err != 0) { ok = 0; break; }
                    if (it > lim) { atomicExch(err, 1); ok = 0; break; }
                    __nanosleep(64);
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// All-to-all flag barrier for a cooperative launch: block b publishes `epoch` in flags[32 b]
// (release; one flag per 128-byte line) and the block waits until every block's flag has reached
// it (acquire).  No atomic round trip: a block passes one flag store and one poll after the last
// block arrives.  WIDE: thread t polls block t (fastest when the blocks arrive together); narrow:
// warp 0 polls (lane l watches blocks l, l + 32, ... not yet seen) with a short sleep between
// rounds, so waiting blocks do not crowd the L2 that a late block is still working in.  Epochs
// increase within a launch (or across the launches that share the flags) and the flags are zeroed
// before the first.  *s_fail (shared, zero at kernel start) records a timeout or another block's
// failure; returns false then.
template <bool WIDE>
__device__ __forceinline__ bool flag_barrier(unsigned* flags, unsigned epoch, int* err, int* s_fail) {
    __syncthreads();
    if (threadIdx.x == 0) st_release(flags + 32 * blockIdx.x, epoch);
    const unsigned lim = spin_limit(err);
    if (WIDE) {
        for (unsigned t = threadIdx.x; t < gridDim.x; t += blockDim.x) {
            const unsigned* f = flags + 32 * t;
            unsigned it = 0;
            while ((int)(ld_acquire(f) - epoch) < 0) {
                if ((++it & 255u) == 0 || it > lim) {
                    if (*(volatile int*)err != 0) { *s_fail = 1; break; }
                    if (it > lim) { atomicExch(err, 1); *s_fail = 1; break; }
                    __nanosleep(64);
                }
            }
        }
    } else if (threadIdx.x < 32) {
        const unsigned G = gridDim.x, lane = threadIdx.x;
        unsigned pending = 0;   // bit q: block lane + 32 q not seen yet
        for (unsigned q = 0; lane + 32 * q < G && q < 32; q++) pending |= 1u << q;
        unsigned it = 0;
        while (true) {
            unsigned still = 0;
            for (unsigned q = 0; q < 32 && (pending >> q); q++)
                if ((pending >> q) & 1u)
                    if ((int)(ld_acquire(flags + 32 * (lane + 32 * q)) - epoch) < 0) still |= 1u << q;
            pending = still;
            if (__all_sync(0xffffffffu, pending == 0)) break;
            if ((++it & 63u) == 0 || it > lim) {
                int bad = *(volatile int*)err != 0;
                if (it > lim) {
                    if (lane == 0) atomicExch(err, 1);
                    bad = 1;
                }
                if (__any_sync(0xffffffffu, bad)) {
                    if (lane == 0) *s_fail = 1;
                    break;
                }
            }
            __nanosleep(20);
        }
    }
    __syncthreads();
    return *s_fail == 0;
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

// Block-wide sums of NV real values at once (one reduction round); every thread gets them.
template <typename R, int NV>
__device__ __forceinline__ void block_sums(R (&v)[NV], R* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; j++) v[j] = warp_sum(v[j]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < NV; j++) red[j * 32 + wid] = v[j];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NV; j++) v[j] = warp_sum(lane < nw ? red[j * 32 + lane] : R(0));
}

}  // namespace dev
}  // namespace bse
