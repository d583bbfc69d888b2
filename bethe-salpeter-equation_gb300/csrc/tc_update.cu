// Tensor-core (tcgen05 + TMA) kernels of the two-stage reduction's trailing update, complex64.
//
// For every panel of the dense -> band stage (band.cu) the trailing Hermitian matrix A22 (m x m,
// complex64, full storage, column-major, leading dimension lda) takes part in two products:
//
//   hemm:    Y = A22 V                         (V: the panel's m x kk reflectors, kk <= 32)
//   update:  A22 -= V W^H + W V^H = L R^H      (L = [V W], R = [W V]: m x 2kk)
//
// Both run here as real GEMMs on the 5th-generation tensor cores (tcgen05.mma kind::f16, BF16
// operands, FP32 accumulation in tensor memory) with every FP32 operand split into three BF16
// parts, x = x0 + x1 + x2 (x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1): 24 significant
// bits, the FP32 significand), and the six products x0 y0 + x0 y1 + x1 y0 + x0 y2 + x2 y0 + x1 y1
// accumulated (the dropped terms are below 2^-24 |x y|), so the products keep the FP32 accuracy of
// the rest of the reduction.  BF16 runs at twice the TF32 rate, so the six BF16 products cost what
// three split-TF32 products (22 significant bits) would.  The complex arithmetic is folded into
// the real K dimension, so neither big operand is expanded:
//
//   hemm   (A22 Hermitian: row i of A22 = conj(column i), and column i is contiguous):
//          Re Y[i,p] = col_i . V_p,   Im Y[i,p] = col_i . V'_p     (K = 2m reals, (re, im) of each j)
//          with V_p the p-th column of V as 2m reals and V'_p = (Im V, -Re V) per element.
//          MMA: M = 128 columns i of A22 (TMA-loaded straight from the matrix, split in shared
//          memory), N = 64 = [V_0..V_31 | V'_0..V'_31] (prepared and split in global memory),
//          K in 32-real blocks;
//          the K range is split over CTAs when there are few column tiles, with partial sums
//          added in a fixed order (bit-reproducible).
//   update: Re (L R^H)[i,j] = Lrow_i . Rrow_j,   Im = Lrow_i . (i R)row_j   (K = 2 * 2kk = 128 reals)
//          MMA: M = 128 rows i (L row-major), N = 128 = [64 rows of R | the same 64 rows of iR],
//          so one accumulator holds the real parts (columns 0..63) and the imaginary parts
//          (64..127) of a 128 x 64 complex tile; L and R are TMA-loaded in FP32 and split in
//          shared memory, iR formed there from R.  The tile of A22 is loaded by TMA into shared
//          memory while the operands stream in, the accumulator is subtracted in place and the
//          tile goes back by a TMA store.
//
// Roles (192 threads): warp 0 issues the TMA loads (one elected thread), warp 1 allocates the
// tensor memory and issues the MMAs (one elected thread), warps 2-5 split the FP32 operands in
// shared memory and run the epilogue (tensor memory -> registers; warp w reads lanes 32 (w % 4)).
// Stages are handed over through mbarriers; every wait is bounded: after kWaitPolls failed polls
// the waiting thread raises the error word and the CTA drains and returns (no hang).
//
// The reference computes the whole eigendecomposition with LAPACK zheevd (bse.version13.cpp:3195,
// 3204, 3330); these products are the BLAS-3 part of its Householder reduction, restated as a
// two-stage reduction (band.cu).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "bse_internal.h"

namespace bse {
namespace tc {

constexpr int kThreads = 192;
constexpr int kRows = 128;                 // MMA M: accumulator lanes
constexpr int kKb = 32;                    // K elements per block: 128 bytes of FP32, 64 of BF16
constexpr uint32_t kWaitPolls = 1u << 22;  // try_wait polls before a wait gives up

// Shared-memory blocks: FP32 as TMA writes it (rows of 128 bytes, 128-byte swizzle), BF16 parts
// as the MMA reads them (rows of 64 bytes, 64-byte swizzle).
// hemm stage: [A fp32 16 KB | A parts 3 x 8 KB | B parts 3 x 4 KB], 4 stages
constexpr int kHemmStages = 4;
constexpr int kHemmChunk = 4;   // K blocks per tensor-memory accumulation chain (K = 128)
constexpr uint32_t kHemmRaw = kRows * kKb * 4, kHemmA = kRows * kKb * 2, kHemmB = 64 * kKb * 2;
constexpr uint32_t kHemmStage = kHemmRaw + 3 * kHemmA + 3 * kHemmB;
constexpr size_t kHemmSmem = (size_t)kHemmStages * kHemmStage + 1024 + 256;
// update: C tile 64 KB + 2 stages of [L fp32 16 KB | R fp32 8 KB | L parts 3 x 8 KB | B parts 3 x 8 KB]
// (a B part: the 64 rows of R, then the 64 rows of iR)
constexpr int kUpdStages = 2;
constexpr int kUpdCols = 64;                               // complex columns per tile
constexpr uint32_t kUpdC = kRows * 2 * kUpdCols * 4;       // 128 rows (256 reals) x 64 columns
constexpr uint32_t kUpdRawL = kRows * kKb * 4, kUpdRawR = kUpdCols * kKb * 4;
constexpr uint32_t kUpdPart = kRows * kKb * 2;             // one 128-row BF16 block
constexpr uint32_t kUpdStage = kUpdRawL + kUpdRawR + 6 * kUpdPart;
constexpr size_t kUpdSmem = (size_t)kUpdC + (size_t)kUpdStages * kUpdStage + 1024 + 256;
static_assert(kHemmSmem <= 232448 && kUpdSmem <= 232448, "shared memory per CTA");
static_assert(kHemmStage % 1024 == 0 && kUpdStage % 1024 == 0 && kUpdC % 1024 == 0, "1024-byte aligned blocks");

// ---------------------------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t saddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* b, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    return done != 0;
}
// Bounded wait for the phase of parity `parity`; false after a timeout or when another role of
// the CTA has given up (s_abort).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* s_abort, int* err) {
    for (uint32_t it = 1;; ++it) {
        if (mbar_test(b, parity)) return true;
        if ((it & 63u) == 0) {
            if (*s_abort) return false;
            if (it > kWaitPolls) {
                *s_abort = 1;
                atomicExch(err, 1);
                return false;
            }
        }
    }
}

// Before the CTA may exit, every TMA load it issued must have landed: wait (bounded, whatever the
// other roles did) for the phase of the last load issued into each barrier.
__device__ __forceinline__ void mbar_drain(uint64_t* b, int last_round) {
    if (last_round < 0) return;
    for (uint32_t it = 0; it < kWaitPolls && !mbar_test(b, (uint32_t)last_round & 1u); ++it) {
    }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            saddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(saddr(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(saddr(src))
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void tma_store_drain() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void prefetch_map(const CUtensorMap* m) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D (tensor memory) (+)= A (shared, M x K) * B (shared, N x K)^T, BF16 in, FP32 accumulate
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accum)
        : "memory");
}
// arrives on `bar` once every MMA issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar)) : "memory");
}
// 16 consecutive 32-bit columns of this thread's tensor-memory lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor of a K-major BF16 block in the 64-byte swizzled layout (rows of
// 64 bytes = 32 K elements, groups of 8 rows 512 bytes apart; the block is 512-byte aligned).
__device__ __forceinline__ uint64_t desc_sw64(const void* p) {
    const uint32_t a = saddr(p);
    uint64_t d = (uint64_t)((a & 0x3FFFFu) >> 4);   // start address
    d |= (uint64_t)1 << 16;                          // leading-dimension offset (unused: K fits one row)
    d |= (uint64_t)(512 >> 4) << 32;                 // stride between 8-row groups
    d |= (uint64_t)1 << 46;                          // descriptor version of tcgen05
    d |= (uint64_t)4 << 61;                          // 64-byte swizzle
    return d;
}
// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// The six BF16 products of one 32-element K block (two MMAs of K = 16 each): parts (0,0), (0,1),
// (1,0), (0,2), (2,0), (1,1) of A = a0 + a1 + a2 and B = b0 + b1 + b2.
__device__ __forceinline__ void mma_block6(uint32_t tmem, const unsigned char* a0, uint32_t a_stride,
                                           const unsigned char* b0, uint32_t b_stride, uint32_t idesc, bool first) {
    constexpr int pa[6] = {0, 0, 1, 0, 2, 1}, pb[6] = {0, 1, 0, 2, 0, 1};
#pragma unroll
    for (int k = 0; k < 2; k++) {
#pragma unroll
        for (int q = 0; q < 6; q++) {
            const uint64_t ad = desc_sw64(a0 + pa[q] * a_stride) + (uint64_t)(k * 2);   // +32 bytes per K step
            const uint64_t bd = desc_sw64(b0 + pb[q] * b_stride) + (uint64_t)(k * 2);
            mma_bf16(tmem, ad, bd, idesc, (first && k == 0 && q == 0) ? 0u : 1u);
        }
    }
}

// x = x0 + x1 + x2, each part the BF16 rounding of what the previous ones leave (exact remainders)
__device__ __forceinline__ void split3(float x, __nv_bfloat16& x0, __nv_bfloat16& x1, __nv_bfloat16& x2) {
    x0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(x0);
    x1 = __float2bfloat16_rn(r1);
    x2 = __float2bfloat16_rn(r1 - __bfloat162float(x1));
}
__device__ __forceinline__ void split3x4(float4 v, uint2 (&o)[3]) {
    __nv_bfloat16 p[3][4];
    split3(v.x, p[0][0], p[1][0], p[2][0]);
    split3(v.y, p[0][1], p[1][1], p[2][1]);
    split3(v.z, p[0][2], p[1][2], p[2][2]);
    split3(v.w, p[0][3], p[1][3], p[2][3]);
#pragma unroll
    for (int q = 0; q < 3; q++) {
        o[q].x = (uint32_t)__bfloat16_as_ushort(p[q][0]) | ((uint32_t)__bfloat16_as_ushort(p[q][1]) << 16);
        o[q].y = (uint32_t)__bfloat16_as_ushort(p[q][2]) | ((uint32_t)__bfloat16_as_ushort(p[q][3]) << 16);
    }
}
// float4 q of an FP32 block as TMA writes it (row r = q / 8; its stored 16-byte chunk q % 8 holds
// elements 4c..4c+3 with c = (q % 8) ^ (r % 8)) -> byte offset of those four elements in the BF16
// block (row r at 64 r, 16-byte chunk (c / 2) ^ ((r / 2) % 4), 8-byte half c % 2)
__host__ __device__ constexpr uint32_t sw128_to_sw64(uint32_t q) {
    const uint32_t r = q >> 3, c = (q & 7u) ^ (r & 7u);
    return r * 64u + (((c >> 1) ^ ((r >> 1) & 3u)) << 4) + ((c & 1u) << 3);
}
// FP32 block of `rows` rows (128-byte swizzle) -> three BF16 part blocks (64-byte swizzle) at
// parts + q * part_stride; with rot, also the parts of i x (per complex pair (re, im) -> (-im, re))
// at rot_parts + q * part_stride
__device__ __forceinline__ void convert_block(const float* raw, int rows, unsigned char* parts, uint32_t part_stride,
                                              unsigned char* rot_parts, int t, int nt) {
    const float4* r4 = reinterpret_cast<const float4*>(raw);
    for (int q = t; q < rows * 8; q += nt) {
        const float4 v = r4[q];
        const uint32_t off = sw128_to_sw64((uint32_t)q);
        uint2 o[3];
        split3x4(v, o);
#pragma unroll
        for (int p = 0; p < 3; p++) *reinterpret_cast<uint2*>(parts + p * part_stride + off) = o[p];
        if (rot_parts) {
            split3x4(make_float4(-v.y, v.x, -v.w, v.z), o);
#pragma unroll
            for (int p = 0; p < 3; p++) *reinterpret_cast<uint2*>(rot_parts + p * part_stride + off) = o[p];
        }
    }
}

__device__ __forceinline__ unsigned char* align1024(unsigned char* p) {
    const uint32_t a = saddr(p);
    return p + ((1024u - (a & 1023u)) & 1023u);
}

// ---------------------------------------------------------------------------------------------
// hemm: partial sums P[split][i][0..63] = (Re, Im) of sum over this split's K range
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1)
    tc_hemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int m, int kb_total,
                   float* __restrict__ P, int64_t ldp, int* err) {
    extern __shared__ unsigned char smraw[];
    unsigned char* sm = align1024(smraw);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + kHemmStages * kHemmStage);
    uint64_t* conv = full + kHemmStages;
    uint64_t* empty = conv + kHemmStages;
    uint64_t* tfull = empty + kHemmStages;   // [2] accumulator buffer b holds a finished chunk
    uint64_t* tempty = tfull + 2;            // [2] accumulator buffer b drained
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tempty + 2);
    __shared__ int s_abort;
    auto raw = [&](int s) { return sm + s * kHemmStage; };                            // FP32 A block
    auto apart = [&](int s) { return sm + s * kHemmStage + kHemmRaw; };               // 3 parts, kHemmA apart
    auto bpart = [&](int s) { return sm + s * kHemmStage + kHemmRaw + 3 * kHemmA; };  // 3 parts, kHemmB apart

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = blockIdx.x * kRows;
    const int split = blockIdx.y, nsplit = gridDim.y;
    const int kb0 = (int)((int64_t)kb_total * split / nsplit);
    const int nkb = (int)((int64_t)kb_total * (split + 1) / nsplit) - kb0;
    const int nchunk = (nkb + kHemmChunk - 1) / kHemmChunk;
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < kHemmStages; s++) {
            mbar_init(full + s, 1);
            mbar_init(conv + s, 128);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(tfull + b, 1);
            mbar_init(tempty + b, 128);
        }
        fence_mbar_init();
    }
    if (warp == 1) tmem_alloc(tslot, 128);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        if (lane == 0) {
            prefetch_map(&tmA);
            prefetch_map(&tmB);
            int issued = 0;
            for (int kb = 0; kb < nkb; kb++) {
                const int s = kb % kHemmStages;
                const uint32_t ph = (uint32_t)(kb / kHemmStages) & 1u;
                if (!mbar_wait(empty + s, ph ^ 1u, &s_abort, err)) break;
                mbar_arrive_tx(full + s, kHemmRaw + 3 * kHemmB);
                const int x = (kb0 + kb) * kKb;
                tma_load_2d(raw(s), &tmA, x, i0, full + s);
                for (int p = 0; p < 3; p++) tma_load_2d(bpart(s) + p * kHemmB, &tmB, x, 64 * p, full + s);
                issued = kb + 1;
            }
            for (int s = 0; s < kHemmStages; s++)
                mbar_drain(full + s, s < issued ? (issued - 1 - s) / kHemmStages : -1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // chains of kHemmChunk K blocks: the tensor pipe's FP32 accumulation truncates, so
            // each chain starts from zero in one of two accumulator buffers and the epilogue adds
            // the finished chains in FP32 registers
            constexpr uint32_t idesc = idesc_bf16(kRows, 64);
            for (int kb = 0; kb < nkb; kb++) {
                const int s = kb % kHemmStages;
                const uint32_t ph = (uint32_t)(kb / kHemmStages) & 1u;
                const int c = kb / kHemmChunk, b = c & 1;
                const bool first = kb % kHemmChunk == 0;
                if (first && c >= 2) {
                    if (!mbar_wait(tempty + b, (uint32_t)(c / 2 - 1) & 1u, &s_abort, err)) break;
                    tc_fence_after();
                }
                if (!mbar_wait(conv + s, ph, &s_abort, err)) break;
                tc_fence_after();
                mma_block6(tmem + (uint32_t)(64 * b), apart(s), kHemmA, bpart(s), kHemmB, idesc, first);
                mma_commit(empty + s);
                if (kb % kHemmChunk == kHemmChunk - 1 || kb == nkb - 1) mma_commit(tfull + b);
            }
        }
    } else {
        const int ct = threadIdx.x - 64;
        const int q = warp & 3;
        const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16);
        float acc[64];
#pragma unroll
        for (int u = 0; u < 64; u++) acc[u] = 0.f;
        bool ok = true;
        auto drain = [&](int c) {
            const int b = c & 1;
            if (!mbar_wait(tfull + b, (uint32_t)(c / 2) & 1u, &s_abort, err)) ok = false;
            __syncwarp();
            tc_fence_after();
#pragma unroll
            for (int cc = 0; cc < 64; cc += 16) {
                float v[16];
                tmem_ld16(tq + (uint32_t)(64 * b + cc), v);
#pragma unroll
                for (int u = 0; u < 16; u++) acc[cc + u] += v[u];
            }
            tc_fence_before();
            mbar_arrive(tempty + b);
        };
        int drained = 0;
        for (int kb = 0; kb < nkb; kb++) {
            const int s = kb % kHemmStages;
            const uint32_t ph = (uint32_t)(kb / kHemmStages) & 1u;
            if (!mbar_wait(full + s, ph, &s_abort, err)) {
                ok = false;
                break;
            }
            convert_block(reinterpret_cast<const float*>(raw(s)), kRows, apart(s), kHemmA, nullptr, ct, 128);
            fence_async_smem();
            mbar_arrive(conv + s);
            // chain c - 1 is finished by the time chain c has been converted
            if (kb % kHemmChunk == kHemmChunk - 1 && kb / kHemmChunk >= 1 && ok) drain(drained++);
        }
        while (ok && drained < nchunk) drain(drained++);
        const int i = i0 + q * 32 + lane;
        if (ok && !s_abort && i < m) {
            float* out = P + ((int64_t)split * ldp + i) * 64;
#pragma unroll
            for (int u = 0; u < 64; u += 4) *reinterpret_cast<float4*>(out + u) = make_float4(acc[u], acc[u + 1], acc[u + 2], acc[u + 3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 128);
    }
}

// Y (m x kk complex, column-major, ld m) = sum over splits, in split order
__global__ void tc_hemm_reduce_kernel(int m, int kk, int nsplit, const float* __restrict__ P, int64_t ldp,
                                      float2* __restrict__ Y) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * kk) return;
    const int i = (int)(t % m), p = (int)(t / m);
    float re = 0.f, im = 0.f;
    for (int s = 0; s < nsplit; s++) {
        const float* r = P + ((int64_t)s * ldp + i) * 64;
        re += r[p];
        im += r[32 + p];
    }
    Y[t] = make_float2(re, im);
}

// B1 parts [3][64][kpad] (BF16): row p < 32 is column p of V as (re, im) pairs, row 32 + p is
// (Im, -Re) of the same column; zero for p >= kk and beyond 2m
__global__ void tc_prep_hemm_kernel(int m, int kk, const float2* __restrict__ V, int kpad, __nv_bfloat16* __restrict__ B) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nb = (int64_t)64 * kpad;
    if (t >= nb) return;
    const int n = (int)(t / kpad), x = (int)(t % kpad);
    const int j = x >> 1, b = x & 1, p = n & 31;
    float val = 0.f;
    if (p < kk && j < m) {
        const float2 v = V[j + (int64_t)p * m];
        val = n < 32 ? (b ? v.y : v.x) : (b ? -v.x : v.y);
    }
    split3(val, B[t], B[nb + t], B[2 * nb + t]);
}

// ---------------------------------------------------------------------------------------------
// update: A22 -= L R^H, one 128 x 64 complex tile per CTA
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1)
    tc_update_kernel(const __grid_constant__ CUtensorMap tmC, const __grid_constant__ CUtensorMap tmL,
                     const __grid_constant__ CUtensorMap tmR, int* err) {
    extern __shared__ unsigned char smraw[];
    unsigned char* sm = align1024(smraw);
    float* Cs = reinterpret_cast<float*>(sm);   // [64 columns][256 reals]
    unsigned char* stg = sm + kUpdC;
    uint64_t* full = reinterpret_cast<uint64_t*>(stg + kUpdStages * kUpdStage);
    uint64_t* conv = full + kUpdStages;
    uint64_t* empty = conv + kUpdStages;
    uint64_t* done = empty + kUpdStages;
    uint64_t* cfull = done + 1;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(cfull + 1);
    __shared__ int s_abort;
    auto rawL = [&](int s) { return stg + s * kUpdStage; };
    auto rawR = [&](int s) { return stg + s * kUpdStage + kUpdRawL; };
    auto lpart = [&](int s) { return stg + s * kUpdStage + kUpdRawL + kUpdRawR; };                  // 3 parts
    auto bpart = [&](int s) { return stg + s * kUpdStage + kUpdRawL + kUpdRawR + 3 * kUpdPart; };   // 3 parts: R | iR
    constexpr int nkb = 128 / kKb;   // K = 128 reals: 2 kk complex pairs

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = blockIdx.x * kRows, j0 = blockIdx.y * kUpdCols;
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < kUpdStages; s++) {
            mbar_init(full + s, 1);
            mbar_init(conv + s, 128);
            mbar_init(empty + s, 1);
        }
        mbar_init(done, 1);
        mbar_init(cfull, 1);
        fence_mbar_init();
    }
    if (warp == 1) tmem_alloc(tslot, 128);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        if (lane == 0) {
            prefetch_map(&tmC);
            prefetch_map(&tmL);
            prefetch_map(&tmR);
            mbar_arrive_tx(cfull, kUpdC);
            tma_load_2d(Cs, &tmC, 2 * i0, j0, cfull);
            int issued = 0;
            for (int kb = 0; kb < nkb; kb++) {
                const int s = kb % kUpdStages;
                const uint32_t ph = (uint32_t)(kb / kUpdStages) & 1u;
                if (!mbar_wait(empty + s, ph ^ 1u, &s_abort, err)) break;
                mbar_arrive_tx(full + s, kUpdRawL + kUpdRawR);
                tma_load_2d(rawL(s), &tmL, kb * kKb, i0, full + s);
                tma_load_2d(rawR(s), &tmR, kb * kKb, j0, full + s);
                issued = kb + 1;
            }
            mbar_drain(cfull, 0);
            for (int s = 0; s < kUpdStages; s++)
                mbar_drain(full + s, s < issued ? (issued - 1 - s) / kUpdStages : -1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16(kRows, 2 * kUpdCols);
            for (int kb = 0; kb < nkb; kb++) {
                const int s = kb % kUpdStages;
                const uint32_t ph = (uint32_t)(kb / kUpdStages) & 1u;
                if (!mbar_wait(conv + s, ph, &s_abort, err)) break;
                tc_fence_after();
                mma_block6(tmem, lpart(s), kUpdPart, bpart(s), kUpdPart, idesc, kb == 0);
                mma_commit(empty + s);
            }
            mma_commit(done);
        }
    } else {
        const int ct = threadIdx.x - 64;
        for (int kb = 0; kb < nkb; kb++) {
            const int s = kb % kUpdStages;
            const uint32_t ph = (uint32_t)(kb / kUpdStages) & 1u;
            if (!mbar_wait(full + s, ph, &s_abort, err)) break;
            convert_block(reinterpret_cast<const float*>(rawL(s)), kRows, lpart(s), kUpdPart, nullptr, ct, 128);
            // rows 0..63 of each B part: R; rows 64..127: iR (64 rows of 64 bytes further on)
            convert_block(reinterpret_cast<const float*>(rawR(s)), kUpdCols, bpart(s), kUpdPart, bpart(s) + kUpdCols * 64, ct, 128);
            fence_async_smem();
            mbar_arrive(conv + s);
        }
        const bool ok = mbar_wait(done, 0, &s_abort, err) && mbar_wait(cfull, 0, &s_abort, err);
        __syncwarp();
        tc_fence_after();
        const int q = warp & 3;
        const int r = q * 32 + lane;   // row of the tile
#pragma unroll 1
        for (int c = 0; c < kUpdCols; c += 16) {
            float re[16], im[16];
            tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, re);
            tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(kUpdCols + c), im);
            if (ok) {
#pragma unroll
                for (int u = 0; u < 16; u++) {
                    float2* cp = reinterpret_cast<float2*>(Cs + (c + u) * 2 * kRows) + r;
                    const float2 x = *cp;
                    *cp = make_float2(x.x - re[u], x.y - im[u]);
                }
            }
        }
        fence_async_smem();
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (ct == 0 && ok && !s_abort) {
            tma_store_2d(&tmC, 2 * i0, j0, Cs);
            tma_store_drain();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 128);
    }
}

// L, R row-major (m rows x 64 complex, FP32): L = [V W], R = [W V], zero beyond kk
__global__ void tc_prep_update_kernel(int m, int kk, const float2* __restrict__ V, const float2* __restrict__ W,
                                      float2* __restrict__ L, float2* __restrict__ R) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * 64) return;
    const int i = (int)(t >> 6), p = (int)(t & 63), pp = p & 31;
    float2 l = make_float2(0.f, 0.f), rr = l;
    if (pp < kk) {
        const float2 v = V[i + (int64_t)pp * m], w = W[i + (int64_t)pp * m];
        l = p < 32 ? v : w;
        rr = p < 32 ? w : v;
    }
    L[t] = l;
    R[t] = rr;
}

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// 2-D tensor map (FP32 with 128-byte swizzle, BF16 with 64-byte swizzle, or FP32 unswizzled):
// inner extent `inner` elements, `outer` rows `stride_bytes` apart, box box0 x box1
enum class MapKind { f32_sw128, bf16_sw64, f32_plain };
bool make_map(CUtensorMap* map, const void* base, uint64_t inner, uint64_t outer, uint64_t stride_bytes, uint32_t box0,
              uint32_t box1, MapKind kind) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {inner, outer};
    const cuuint64_t strides[1] = {stride_bytes};
    const cuuint32_t box[2] = {box0, box1};
    const cuuint32_t estr[2] = {1, 1};
    const CUtensorMapDataType dt = kind == MapKind::bf16_sw64 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const CUtensorMapSwizzle sw = kind == MapKind::f32_sw128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                  : kind == MapKind::bf16_sw64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                               : CU_TENSOR_MAP_SWIZZLE_NONE;
    return fn(map, dt, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t set_attributes() {
    static cudaError_t e = cudaSuccess;
    static std::once_flag once;
    std::call_once(once, [] {
        e = cudaFuncSetAttribute(tc_hemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kHemmSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tc_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kUpdSmem);
    });
    return e;
}

size_t al256(size_t x) { return (x + 255) / 256 * 256; }
int kpad_of(int m) { return (2 * m + kKb - 1) / kKb * kKb; }
int hemm_splits(int m, int nsm) {
    const int tiles = (m + kRows - 1) / kRows, kbt = kpad_of(m) / kKb;
    return std::max(1, std::min(kbt, (nsm + tiles - 1) / tiles));
}

}  // namespace tc

size_t tc_workspace(int n, int nsm) {
    using namespace tc;
    // the hemm (B1 parts, split partials) and the update (L, R) use the same region in turn;
    // nsplit * tiles <= nsm + tiles for every panel
    const size_t tiles = (size_t)(n + kRows - 1) / kRows;
    const size_t hemm = al256((size_t)3 * 64 * kpad_of(n) * sizeof(__nv_bfloat16)) +
                        al256((nsm + tiles) * kRows * 64 * sizeof(float));
    const size_t upd = 2 * al256((size_t)n * 64 * sizeof(float2));
    return std::max(hemm, upd) + 1024;
}

bool tc_supported(int64_t lda) { return (lda % 2) == 0 && tc::encode_fn() != nullptr; }

// Y = A22 V (A22 Hermitian, full storage) with the tensor cores.
int tc_hemm(cudaStream_t st, int nsm, int m, int kk, const float2* A22, int64_t lda, const float2* V, float2* Y, char* ws,
            int* err, int* launches, cudaEvent_t* ev) {
    using namespace tc;
    if (set_attributes() != cudaSuccess) return 1;
    const int kpad = kpad_of(m), tiles = (m + kRows - 1) / kRows, nsplit = hemm_splits(m, nsm);
    __nv_bfloat16* B = reinterpret_cast<__nv_bfloat16*>(ws);
    float* P = reinterpret_cast<float*>(ws + al256((size_t)3 * 64 * kpad * sizeof(__nv_bfloat16)));
    const int64_t ldp = (int64_t)tiles * kRows;
    CUtensorMap mA, mB;
    if (!make_map(&mA, A22, 2 * (uint64_t)m, (uint64_t)m, 2 * (uint64_t)lda * sizeof(float), kKb, kRows, MapKind::f32_sw128) ||
        !make_map(&mB, B, (uint64_t)kpad, 3 * 64, (uint64_t)kpad * sizeof(__nv_bfloat16), kKb, 64, MapKind::bf16_sw64))
        return 2;
    const int64_t nb = (int64_t)64 * kpad;
    tc_prep_hemm_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(m, kk, V, kpad, B);
    if (ev) cudaEventRecord(ev[0], st);
    tc_hemm_kernel<<<dim3((unsigned)tiles, (unsigned)nsplit), kThreads, kHemmSmem, st>>>(mA, mB, m, kpad / kKb, P, ldp, err);
    if (ev) cudaEventRecord(ev[1], st);
    tc_hemm_reduce_kernel<<<(unsigned)(((int64_t)m * kk + 255) / 256), 256, 0, st>>>(m, kk, nsplit, P, ldp, Y);
    *launches += 3;
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

// A22 -= V W^H + W V^H (full storage) with the tensor cores.
int tc_rank2k(cudaStream_t st, int m, int kk, float2* A22, int64_t lda, const float2* V, const float2* W, char* ws, int* err,
              int* launches, cudaEvent_t* ev) {
    using namespace tc;
    if (set_attributes() != cudaSuccess) return 1;
    const size_t blk = al256((size_t)m * 64 * sizeof(float2));
    float2* L = reinterpret_cast<float2*>(ws);
    float2* R = reinterpret_cast<float2*>(ws + blk);
    CUtensorMap mC, mL, mR;
    if (!make_map(&mC, A22, 2 * (uint64_t)m, (uint64_t)m, 2 * (uint64_t)lda * sizeof(float), 2 * kRows, kUpdCols,
                  MapKind::f32_plain) ||
        !make_map(&mL, L, 128, (uint64_t)m, 128 * sizeof(float), kKb, kRows, MapKind::f32_sw128) ||
        !make_map(&mR, R, 128, (uint64_t)m, 128 * sizeof(float), kKb, kUpdCols, MapKind::f32_sw128))
        return 2;
    tc_prep_update_kernel<<<(unsigned)(((int64_t)m * 64 + 255) / 256), 256, 0, st>>>(m, kk, V, W, L, R);
    const dim3 grid((unsigned)((m + kRows - 1) / kRows), (unsigned)((m + kUpdCols - 1) / kUpdCols));
    if (ev) cudaEventRecord(ev[0], st);
    tc_update_kernel<<<grid, kThreads, kUpdSmem, st>>>(mC, mL, mR, err);
    if (ev) cudaEventRecord(ev[1], st);
    *launches += 2;
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

}  // namespace bse

// ---------------------------------------------------------------------------------------------
// Test hooks (not part of the drop-in ABI): one product on host data, for the parity tests.
// ---------------------------------------------------------------------------------------------
namespace {
int run_test(int op, int m, int kk, void* A, long long lda, const void* V, const void* W, void* Y) {
    if (m < 1 || kk < 1 || kk > 32 || lda < m || (lda % 2) != 0 || !bse::tc_supported(lda)) return BSE_ERR_BAD_INPUT;
    int nsm = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return BSE_ERR_NO_DEVICE;
    const size_t a_bytes = (size_t)lda * m * sizeof(float2), v_bytes = (size_t)m * kk * sizeof(float2);
    const size_t ws_bytes = bse::tc_workspace(m, nsm);
    char* buf = nullptr;
    const size_t total = a_bytes + 3 * v_bytes + ws_bytes + 4096;
    if (cudaMalloc(&buf, total) != cudaSuccess) return BSE_ERR_OOM;
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    float2* dA = reinterpret_cast<float2*>(buf);
    float2* dV = reinterpret_cast<float2*>(buf + al(a_bytes));
    float2* dW = reinterpret_cast<float2*>(buf + al(a_bytes) + al(v_bytes));
    float2* dY = reinterpret_cast<float2*>(buf + al(a_bytes) + 2 * al(v_bytes));
    char* ws = buf + al(a_bytes) + 3 * al(v_bytes);
    int* derr = reinterpret_cast<int*>(ws + al(ws_bytes));
    int st = BSE_OK, launches = 0, herr = 0;
    cudaMemcpy(dA, A, a_bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dV, V, v_bytes, cudaMemcpyHostToDevice);
    if (W) cudaMemcpy(dW, W, v_bytes, cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, sizeof(int));
    const int r = op == 0 ? bse::tc_hemm(0, nsm, m, kk, dA, lda, dV, dY, ws, derr, &launches)
                          : bse::tc_rank2k(0, m, kk, dA, lda, dV, dW, ws, derr, &launches);
    if (r != 0) st = BSE_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) st = BSE_ERR_CUDA;
    cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
    if (!st && herr) st = BSE_ERR_NOT_CONVERGED;
    if (!st) {
        if (op == 0) cudaMemcpy(Y, dY, v_bytes, cudaMemcpyDeviceToHost);
        else cudaMemcpy(A, dA, a_bytes, cudaMemcpyDeviceToHost);
    }
    cudaFree(buf);
    return st;
}
}  // namespace

extern "C" {
// Y (m x kk) = A^H V with A m x m (ld lda, even), complex64, column-major host arrays.
int bse_test_tc_hemm(int m, int kk, const void* A, long long lda, const void* V, void* Y) {
    return run_test(0, m, kk, const_cast<void*>(A), lda, V, nullptr, Y);
}
// A (m x m, ld lda, even) -= V W^H + W V^H in place, complex64, column-major host arrays.
int bse_test_tc_rank2k(int m, int kk, void* A, long long lda, const void* V, const void* W) {
    return run_test(1, m, kk, A, lda, V, W, nullptr);
}
}
