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
//          MMA: M = 128 columns i of A22 (TMA-loaded in FP32 straight from the matrix, split in
//          shared memory), N = 64 = [V_0..V_31 | V'_0..V'_31] (prepared and split in global
//          memory), K in 32-real blocks.  Persistent stream-K: the (column tile, K block) units
//          are dealt evenly to one CTA per SM; partial sums end at tile boundaries and are added
//          per tile in CTA order (bit-reproducible).
//   update: Re (L R^H)[i,j] = Lrow_i . Rrow_j,   Im = Lrow_i . (i R)row_j   (K = 2 * 2kk = 128 reals)
//          MMA: M = 128 rows i (L), N = 64 = [32 rows of R | the same 32 rows of iR], so one
//          accumulator holds the real parts (columns 0..31) and the imaginary parts (32..63) of a
//          128 x 32 complex tile.  L, R and iR are split into BF16 parts in global memory by a
//          small kernel.  Persistent: one CTA per SM walks its share of the tiles in row-strip
//          order with the strip's L resident; the A22 tiles come in by TMA, double-buffered
//          together with the accumulators, so the load of one tile overlaps the MMAs of the next,
//          and the workers store the updated tiles straight to A22.
//
// MMAs: the three B parts lie back to back in shared memory, so the six products of a K = 16 step
// take three MMAs, a0 [b0 b1 b2] (N = 192), a1 [b0 b1] (N = 128) and a2 b0 (N = 64), into three
// column groups of the accumulator: a0 b0 | a0 b1 + a1 b0 + a2 b0 | a0 b2 + a1 b1.  Accumulation:
// the tensor pipe's FP32 accumulation truncates; with the smaller products apart from a0 b0 their
// truncation is relative to their own size, the epilogue adds the groups in FP32, and the hemm
// restarts its accumulators every 128 K and adds the finished chains in FP32 registers, so the
// error stays that of an FP32 product (no drift with K).
//
// Roles: warp 0 issues the TMA loads (one elected thread), warp 1 allocates the tensor memory (512
// columns) and issues the MMAs (one elected thread), the worker warps run the rest (warp w reads
// tensor-memory lanes 32 (w % 4)).  hemm: 576 threads, 16 worker warps (four per lane quarter)
// split the streamed FP32 blocks into BF16 parts and drain the accumulators.  update: 352
// threads, 8 worker warps (two per lane quarter, half of the tile's columns each) and warp 10,
// which loads the A22 tiles.  Every role walks its units or tiles with an incrementally advanced
// cursor (no 64-bit division per unit).  Stages are handed over through mbarriers (one arrival
// per warp where a warp signals); every wait is bounded: after kWaitPolls failed polls the waiting
// thread raises the error word and the CTA drains and returns (no hang).
//
// TMA works in 16-byte granules of the 2m-real columns, so the order m must be even (every
// trailing order of the reduction is, for even n).
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

// warp 0 issues the TMA loads, warp 1 the MMAs; the workers follow.  hemm: 16 worker warps (four
// per tensor-memory lane quarter) convert the streamed A22 blocks and drain the accumulators;
// update: 8 worker warps (warps 2-9) and warp 10, which loads the A22 tiles
constexpr int kHemmWorkers = 512;
constexpr int kHemmThreads = 64 + kHemmWorkers;
constexpr int kWorkers = 256;
constexpr int kUpdThreads = 64 + kWorkers + 32;
constexpr int kRows = 128;                 // MMA M: accumulator lanes
constexpr int kKb = 32;                    // K elements per block: 128 bytes of FP32, 64 of BF16
constexpr uint32_t kWaitPolls = 1u << 22;  // try_wait polls before a wait gives up

// Shared-memory blocks: FP32 as TMA writes it (rows of 128 bytes, 128-byte swizzle), BF16 parts
// as the MMA reads them (rows of 64 bytes, 64-byte swizzle).
// hemm (persistent, stream-K): a ring of kHemmRing [FP32 A block 16 KB | B parts 3 x 4 KB] slots
// filled by TMA, and kHemmParts slots of converted A parts (3 x 8 KB)
constexpr int kHemmRing = 6, kHemmParts = 2;
constexpr int kHemmChunk = 4;   // K blocks per tensor-memory accumulation chain (K = 128)
constexpr uint32_t kHemmRaw = kRows * kKb * 4, kHemmA = kRows * kKb * 2, kHemmB = 64 * kKb * 2;
constexpr uint32_t kHemmSlot = kHemmRaw + 3 * kHemmB, kHemmPartSlot = 3 * kHemmA;
constexpr size_t kHemmSmem = (size_t)kHemmRing * kHemmSlot + (size_t)kHemmParts * kHemmPartSlot + 1024 + 512;
// update (persistent, row strips): the strip's L parts resident (4 K blocks x 3 parts x 8 KB),
// kUpdCbuf C tiles of 128 rows x kUpdCols complex columns in flight, a ring of B slots per K block
// (3 parts x [kUpdCols rows of R | kUpdCols rows of iR] x 64 bytes), kUpdAcc accumulator pairs
constexpr int kUpdCols = 32;                               // complex columns per tile
constexpr int kUpdCbuf = 2;
constexpr int kUpdAcc = 2;
constexpr int kUpdRing = 4;
constexpr uint32_t kUpdL = 4 * 3 * kRows * kKb * 2;        // 96 KB
constexpr uint32_t kUpdC = kRows * 2 * kUpdCols * 4;       // 128 rows (256 reals) x kUpdCols columns
constexpr uint32_t kUpdBpart = 2 * kUpdCols * kKb * 2;     // R rows then iR rows, one part
constexpr uint32_t kUpdBslot = 3 * kUpdBpart;
constexpr uint32_t kUpdAccCols = 256;                      // per accumulator: 3 groups x (Re | Im) x kUpdCols
constexpr size_t kUpdSmem = (size_t)kUpdL + (size_t)kUpdCbuf * kUpdC + (size_t)kUpdRing * kUpdBslot + 1024 + 512;
constexpr uint32_t kTmemCols = 512;                        // two accumulators of 3 x 64 columns, 256 apart
static_assert(kUpdAcc * kUpdAccCols <= kTmemCols && 6 * kUpdCols <= (int)kUpdAccCols, "update accumulators");
static_assert(kUpdBpart == 2 * kUpdCols * 64 && kHemmB == 64 * 64, "B parts back to back (NB rows of 64 bytes)");
static_assert(kHemmSmem <= 232448 && kUpdSmem <= 232448, "shared memory per CTA");
static_assert(kHemmSlot % 1024 == 0 && kHemmPartSlot % 1024 == 0 && kUpdC % 1024 == 0 && kUpdBslot % 1024 == 0 &&
                  kUpdL % 1024 == 0 && kUpdBpart % 512 == 0,
              "block alignment");

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
// one arrival per warp, after every lane's preceding work (the barrier counts warps)
__device__ __forceinline__ void mbar_arrive_warp(uint64_t* b) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(b);
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
// 16 consecutive 32-bit columns of this thread's tensor-memory lane at each of 3 addresses,
// one wait for all the loads
__device__ __forceinline__ void tmem_ld3x16(uint32_t a0, uint32_t a1, uint32_t a2, float (&v)[48]) {
    uint32_t r[48];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%48];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%49];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47}, [%50];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47])
        : "r"(a0), "r"(a1), "r"(a2)
        : "memory");
#pragma unroll
    for (int i = 0; i < 48; i++) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive 32-bit columns of this thread's tensor-memory lane at each of 6 addresses,
// one wait for all the loads
__device__ __forceinline__ void tmem_ld6x16(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t a4, uint32_t a5, float (&v)[96]) {
    uint32_t r[96];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%96];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%97];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47}, [%98];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%99];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%64, %65, %66, %67, %68, %69, %70, %71, %72, %73, %74, %75, %76, %77, %78, %79}, [%100];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%80, %81, %82, %83, %84, %85, %86, %87, %88, %89, %90, %91, %92, %93, %94, %95}, [%101];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63]), "=r"(r[64]), "=r"(r[65]), "=r"(r[66]), "=r"(r[67]), "=r"(r[68]), "=r"(r[69]), "=r"(r[70]), "=r"(r[71]), "=r"(r[72]), "=r"(r[73]), "=r"(r[74]), "=r"(r[75]), "=r"(r[76]), "=r"(r[77]), "=r"(r[78]), "=r"(r[79]), "=r"(r[80]), "=r"(r[81]), "=r"(r[82]), "=r"(r[83]), "=r"(r[84]), "=r"(r[85]), "=r"(r[86]), "=r"(r[87]), "=r"(r[88]), "=r"(r[89]), "=r"(r[90]), "=r"(r[91]), "=r"(r[92]), "=r"(r[93]), "=r"(r[94]), "=r"(r[95])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(a4), "r"(a5)
        : "memory");
#pragma unroll
    for (int i = 0; i < 96; i++) v[i] = __uint_as_float(r[i]);
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

// The six BF16 products of one 32-element K block (two K = 16 steps) of A = a0 + a1 + a2 and
// B = b0 + b1 + b2, in three MMAs per step: the B parts lie one after the other (NB rows each, the
// same 64-byte swizzled layout), so a0 [b0 b1 b2] writes columns [0, 3 NB) of t, a1 [b0 b1] adds to
// [NB, 3 NB) and a2 b0 to [NB, 2 NB).  Columns [0, NB) hold a0 b0 ("big"), [NB, 2 NB) a0 b1 + a1 b0
// + a2 b0, [2 NB, 3 NB) a0 b2 + a1 b1.  The tensor pipe's FP32 accumulation truncates: with the
// smaller terms kept apart from a0 b0 their truncation is relative to their own size; the epilogue
// adds the three groups in FP32.  Reading each A part once per step (instead of once per product)
// cuts the shared-memory operand traffic from 36 KB to 24 KB per step at NB = 64.
template <int NB>
__device__ __forceinline__ void mma_block_cat(uint32_t t, const unsigned char* a0, uint32_t a_stride,
                                              const unsigned char* b0, bool first) {
    constexpr uint32_t i3 = idesc_bf16(kRows, 3 * NB), i2 = idesc_bf16(kRows, 2 * NB), i1 = idesc_bf16(kRows, NB);
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const uint64_t bd = desc_sw64(b0) + (uint64_t)(k * 2);   // +32 bytes per K step
        mma_bf16(t, desc_sw64(a0) + (uint64_t)(k * 2), bd, i3, (first && k == 0) ? 0u : 1u);
        mma_bf16(t + NB, desc_sw64(a0 + a_stride) + (uint64_t)(k * 2), bd, i2, 1u);
        mma_bf16(t + NB, desc_sw64(a0 + 2 * a_stride) + (uint64_t)(k * 2), bd, i1, 1u);
    }
}

// x = x0 + x1 + x2, each part the BF16 rounding of what the previous ones leave (exact remainders)
__device__ __forceinline__ void split3(float x, __nv_bfloat16& x0, __nv_bfloat16& x1, __nv_bfloat16& x2) {
    x0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(x0);
    x1 = __float2bfloat16_rn(r1);
    x2 = __float2bfloat16_rn(r1 - __bfloat162float(x1));
}
// two floats -> packed BF16 pair (round to nearest even), a in the low half, b in the high half
__device__ __forceinline__ uint32_t cvt_bf16x2(float a, float b) {
    uint32_t d;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
    return d;
}
// split3 of a pair at once, packed: parts o[0..2] (low half a, high half b)
__device__ __forceinline__ void split3x2(float a, float b, uint32_t (&o)[3]) {
    o[0] = cvt_bf16x2(a, b);
    const float ra = a - __uint_as_float(o[0] << 16), rb = b - __uint_as_float(o[0] & 0xffff0000u);
    o[1] = cvt_bf16x2(ra, rb);
    o[2] = cvt_bf16x2(ra - __uint_as_float(o[1] << 16), rb - __uint_as_float(o[1] & 0xffff0000u));
}
__device__ __forceinline__ void split3x4(float4 v, uint2 (&o)[3]) {
    uint32_t lo[3], hi[3];
    split3x2(v.x, v.y, lo);
    split3x2(v.z, v.w, hi);
#pragma unroll
    for (int q = 0; q < 3; q++) o[q] = make_uint2(lo[q], hi[q]);
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
#pragma unroll 4
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
// hemm, persistent stream-K: the work units are (column tile t of A22, K block kb), t-major, and
// CTA g takes units [lo(g), lo(g + 1)), lo(g) = g W / G, so every SM gets the same number of K
// blocks whatever the tile count.  A CTA ends its tiles' partial sums at tile boundaries:
// P[g][t - first tile of g][row][0..63] = (Re | Im) over its K blocks of tile t.
// ---------------------------------------------------------------------------------------------
struct HemmArgs {
    int m, kb_per_tile, ntiles, slots;
    int64_t units;        // ntiles * kb_per_tile
    float* P;
    int* err;
};

__global__ void __launch_bounds__(kHemmThreads, 1)
    tc_hemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, HemmArgs h) {
    extern __shared__ unsigned char smraw[];
    unsigned char* sm = align1024(smraw);
    unsigned char* parts = sm + kHemmRing * kHemmSlot;
    uint64_t* bars = reinterpret_cast<uint64_t*>(parts + kHemmParts * kHemmPartSlot);
    uint64_t* rfull = bars;                      // [ring] A block and B parts landed (TMA)
    uint64_t* rconv = rfull + kHemmRing;         // [ring] A block converted (converters)
    uint64_t* rmma = rconv + kHemmRing;          // [ring] B parts consumed (MMA)
    uint64_t* pfull = rmma + kHemmRing;          // [parts] A parts written (converters)
    uint64_t* pempty = pfull + kHemmParts;       // [parts] A parts consumed (MMA)
    uint64_t* tfull = pempty + kHemmParts;       // [2] accumulator pair b holds a finished chain
    uint64_t* tempty = tfull + 2;                // [2] accumulator pair b drained
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tempty + 2);
    __shared__ int s_abort;
    auto raw = [&](int s) { return sm + s * kHemmSlot; };
    auto bpart = [&](int s) { return sm + s * kHemmSlot + kHemmRaw; };     // 3 parts, kHemmB apart
    auto apart = [&](int s) { return parts + s * kHemmPartSlot; };           // 3 parts, kHemmA apart

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t G = gridDim.x, g = blockIdx.x;
    const int64_t u0 = g * h.units / G, u1 = (g + 1) * h.units / G;
    const int nu = (int)(u1 - u0);
    const int KB = h.kb_per_tile;
    const int t_first = (int)(u0 / KB);
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < kHemmRing; s++) {
            mbar_init(rfull + s, 1);
            mbar_init(rconv + s, kHemmWorkers / 32);
            mbar_init(rmma + s, 1);
        }
        for (int s = 0; s < kHemmParts; s++) {
            mbar_init(pfull + s, kHemmWorkers / 32);
            mbar_init(pempty + s, 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(tfull + b, 1);
            mbar_init(tempty + b, kHemmWorkers / 32);
        }
        fence_mbar_init();
    }
    if (warp == 1) tmem_alloc(tslot, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    // Every role walks the units u0 + j in order with a (tile, K block) cursor advanced one unit at
    // a time: a 64-bit division per unit and thread cost more issue slots than the conversion.
    // A chain starts at the range start or a multiple of kHemmChunk K blocks and ends at the
    // block before the next multiple, at a tile's last K block, or at the range end.
    const int tile0 = (int)(u0 / KB), kb0 = (int)(u0 % KB);
    auto chain_start = [&](int j, int kb) { return j == 0 || kb % kHemmChunk == 0; };
    auto chain_end = [&](int j, int kb) { return kb % kHemmChunk == kHemmChunk - 1 || kb == KB - 1 || j == nu - 1; };

    if (warp == 0) {
        if (lane == 0) {
            prefetch_map(&tmA);
            prefetch_map(&tmB);
            int issued = 0, tile = tile0, kb = kb0;
            for (int j = 0; j < nu; j++) {
                const int s = j % kHemmRing;
                const uint32_t ph = (uint32_t)(j / kHemmRing) & 1u;
                // the slot is free once its A block is converted and its B parts are consumed
                if (!mbar_wait(rconv + s, ph ^ 1u, &s_abort, h.err) || !mbar_wait(rmma + s, ph ^ 1u, &s_abort, h.err)) break;
                mbar_arrive_tx(rfull + s, kHemmRaw + 3 * kHemmB);
                const int x = kb * kKb, i0 = tile * kRows;
                tma_load_2d(raw(s), &tmA, x, i0, rfull + s);
                for (int p = 0; p < 3; p++) tma_load_2d(bpart(s) + p * kHemmB, &tmB, x, 64 * p, rfull + s);
                issued = j + 1;
                if (++kb == KB) { kb = 0; ++tile; }
            }
            for (int s = 0; s < kHemmRing; s++)
                mbar_drain(rfull + s, s < issued ? (issued - 1 - s) / kHemmRing : -1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int c = -1, kb = kb0;
            for (int j = 0; j < nu; j++, kb = kb + 1 == KB ? 0 : kb + 1) {
                const int s = j % kHemmRing, ps = j % kHemmParts;
                const uint32_t ph = (uint32_t)(j / kHemmRing) & 1u, pph = (uint32_t)(j / kHemmParts) & 1u;
                const bool first = chain_start(j, kb);
                if (first) {
                    c++;
                    if (c >= 2) {
                        if (!mbar_wait(tempty + (c & 1), (uint32_t)(c / 2 - 1) & 1u, &s_abort, h.err)) break;
                        tc_fence_after();
                    }
                }
                if (!mbar_wait(rfull + s, ph, &s_abort, h.err) || !mbar_wait(pfull + ps, pph, &s_abort, h.err)) break;
                tc_fence_after();
                const uint32_t tb = tmem + (uint32_t)(256 * (c & 1));
                mma_block_cat<64>(tb, apart(ps), kHemmA, bpart(s), first);
                mma_commit(rmma + s);
                mma_commit(pempty + ps);
                if (chain_end(j, kb)) mma_commit(tfull + (c & 1));
            }
        }
    } else {
        // workers: warp w reads tensor-memory lanes 32 (w % 4) ..; warps 2-5, 6-9, 10-13, 14-17
        // own accumulator columns 0..15, 16..31 (Re), 32..47, 48..63 (Im)
        const int ct = threadIdx.x - 64;
        const int q = warp & 3, cg = (warp - 2) >> 2;
        const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(16 * cg);
        const int r = q * 32 + lane;
        float acc[16];
#pragma unroll
        for (int e = 0; e < 16; e++) acc[e] = 0.f;
        bool ok = true;
        // chains are drained in order, one behind the conversion; a chain that ends a tile (or
        // the range) writes the tile's partial sums and clears the accumulator
        int drained = 0, nchain = 0;
        int chain_tile[2] = {0, 0}, chain_last[2] = {0, 0};
        auto drain = [&]() {
            const int cc = drained, b = cc & 1;
            const bool got = mbar_wait(tfull + b, (uint32_t)(cc / 2) & 1u, &s_abort, h.err);
            ok = __all_sync(0xffffffffu, got) && ok;   // warp-uniform: the tensor-memory loads need all lanes
            tc_fence_after();
            float v[48];   // the three column groups of this warp's 16 columns
            const uint32_t tb = tq + (uint32_t)(256 * b);
            tmem_ld3x16(tb, tb + 64, tb + 128, v);
#pragma unroll
            for (int x = 0; x < 16; x++) acc[x] += v[x] + (v[16 + x] + v[32 + x]);
            tc_fence_before();
            mbar_arrive_warp(tempty + b);
            if (chain_last[b]) {
                const int t = chain_tile[b], i = t * kRows + r;
                if (ok && !s_abort && i < h.m) {
                    float* out = h.P + (((int64_t)g * h.slots + (t - t_first)) * kRows + r) * 64 + 16 * cg;
#pragma unroll
                    for (int e = 0; e < 16; e += 4)
                        *reinterpret_cast<float4*>(out + e) = make_float4(acc[e], acc[e + 1], acc[e + 2], acc[e + 3]);
                }
#pragma unroll
                for (int e = 0; e < 16; e++) acc[e] = 0.f;
            }
            drained++;
        };
        int tile = tile0, kb = kb0;
        for (int j = 0; j < nu && ok; j++) {
            const int s = j % kHemmRing, ps = j % kHemmParts;
            const uint32_t ph = (uint32_t)(j / kHemmRing) & 1u, pph = (uint32_t)(j / kHemmParts) & 1u;
            const bool got = mbar_wait(rfull + s, ph, &s_abort, h.err) && mbar_wait(pempty + ps, pph ^ 1u, &s_abort, h.err);
            if (!__all_sync(0xffffffffu, got)) {
                ok = false;
                break;
            }
            convert_block(reinterpret_cast<const float*>(raw(s)), kRows, apart(ps), kHemmA, nullptr, ct, kHemmWorkers);
            fence_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(rconv + s);
                mbar_arrive(pfull + ps);
            }
            if (chain_start(j, kb)) {
                chain_tile[nchain & 1] = tile;
                nchain++;
            }
            if (chain_end(j, kb)) {
                chain_last[(nchain - 1) & 1] = (kb == KB - 1 || j == nu - 1) ? 1 : 0;
                // the chain before this one has finished by now
                if (nchain >= 2 && drained < nchain - 1) drain();
            }
            if (++kb == KB) { kb = 0; ++tile; }
        }
        while (ok && drained < nchain) drain();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// Y (m x kk complex, column-major, ld m): for each row, the partial sums of the CTAs whose range
// covers its tile, in CTA order (bit-reproducible)
__global__ void tc_hemm_reduce_kernel(int m, int kk, HemmArgs h, int64_t G, float2* __restrict__ Y) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * kk) return;
    const int i = (int)(t % m), p = (int)(t / m);
    const int tile = i / kRows, r = i % kRows;
    const int64_t KB = h.kb_per_tile, W = h.units;
    const int64_t ua = (int64_t)tile * KB, ub = ua + KB - 1;
    const int64_t ga = ((ua + 1) * G - 1) / W, gb = ((ub + 1) * G - 1) / W;   // CTAs holding units ua, ub
    float re = 0.f, im = 0.f;
    for (int64_t g = ga; g <= gb; g++) {
        const int64_t lo = g * W / G, hi = (g + 1) * W / G;
        if (hi <= ua || lo > ub) continue;   // an empty range
        const int64_t slot = tile - lo / KB;
        const float* v = h.P + ((g * h.slots + slot) * kRows + r) * 64;
        re += v[p];
        im += v[32 + p];
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
// update, persistent: tiles of 128 rows x kUpdCols complex columns in row-strip-major order, CTA g
// taking tiles [g T / G, (g + 1) T / G).  The strip's L parts stay resident while its column
// tiles stream; the C tiles (TMA loads) and the accumulator pairs are double-buffered, so the
// load of one tile overlaps the MMAs of the next.  The workers read their part of a C tile into
// registers, release its buffer at once and store the updated values straight to A22 (coalesced,
// 256 bytes per warp and column): no shared-memory write-back, no TMA store to wait for.
// ---------------------------------------------------------------------------------------------
struct UpdArgs {
    int m, nstrips, ncols;
    int64_t ntiles;
    float2* A;      // A22 (the workers store the updated tiles directly)
    int64_t lda;
    int* err;
};

__global__ void __launch_bounds__(kUpdThreads, 1)
    tc_update_kernel(const __grid_constant__ CUtensorMap tmC, const __grid_constant__ CUtensorMap tmL,
                     const __grid_constant__ CUtensorMap tmR, const __grid_constant__ CUtensorMap tmRi, UpdArgs a) {
    extern __shared__ unsigned char smraw[];
    unsigned char* sm = align1024(smraw);
    unsigned char* Ls = sm;                                   // [kb][part] 128 rows x 64 B
    float* Cs0 = reinterpret_cast<float*>(sm + kUpdL);        // kUpdCbuf x [kUpdCols columns][256 reals]
    unsigned char* ring = sm + kUpdL + kUpdCbuf * kUpdC;
    uint64_t* bars = reinterpret_cast<uint64_t*>(ring + kUpdRing * kUpdBslot);
    uint64_t* bfull = bars;                     // [ring] B parts landed
    uint64_t* bempty = bfull + kUpdRing;        // [ring] B parts consumed
    uint64_t* cfull = bempty + kUpdRing;        // [kUpdCbuf] C tile landed
    uint64_t* cempty = cfull + kUpdCbuf;        // [kUpdCbuf] C tile read out by the workers
    uint64_t* tfull = cempty + kUpdCbuf;        // [kUpdAcc] accumulator pair holds a finished tile
    uint64_t* tempty = tfull + kUpdAcc;         // [kUpdAcc] accumulator pair drained
    uint64_t* lfull = tempty + kUpdAcc;         // L parts of a strip landed
    uint64_t* lfree = lfull + 1;                // MMAs of the previous strip done
    uint32_t* tslot = reinterpret_cast<uint32_t*>(lfree + 1);
    __shared__ int s_abort;
    auto lpart = [&](int kb) { return Ls + kb * 3 * (kRows * kKb * 2); };   // 3 parts, kRows*64 apart
    auto bslot = [&](int s) { return ring + s * kUpdBslot; };             // 3 parts, kUpdBpart apart
    auto Cs = [&](int b) { return Cs0 + b * (kUpdC / 4); };

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t G = gridDim.x, g = blockIdx.x;
    const int64_t t0 = g * a.ntiles / G, t1 = (g + 1) * a.ntiles / G;
    const int nt = (int)(t1 - t0);
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < kUpdRing; s++) {
            mbar_init(bfull + s, 1);
            mbar_init(bempty + s, 1);
        }
        for (int b = 0; b < kUpdCbuf; b++) {
            mbar_init(cfull + b, 1);
            mbar_init(cempty + b, kWorkers / 32);
        }
        for (int b = 0; b < kUpdAcc; b++) {
            mbar_init(tfull + b, 1);
            mbar_init(tempty + b, kWorkers / 32);
        }
        mbar_init(lfull, 1);
        mbar_init(lfree, 1);
        fence_mbar_init();
    }
    if (warp == 1) tmem_alloc(tslot, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    // every role walks its tiles in order with a (strip, column tile) cursor (no 64-bit division
    // per tile); a strip starts at j = 0 or where the column tile wraps to 0
    const int strip0 = (int)(t0 / a.ncols), col0 = (int)(t0 % a.ncols);
    auto advance = [&](int& strip, int& col) {
        if (++col == a.ncols) {
            col = 0;
            ++strip;
        }
    };

    if (warp == 0) {
        if (lane == 0) {
            prefetch_map(&tmL);
            prefetch_map(&tmR);
            prefetch_map(&tmRi);
            // L parts and B operands; the A22 tiles are loaded by warp 10, independently
            int nstrip = 0, issued = 0, lissued = 0, strip = strip0, col = col0;
            for (int j = 0; j < nt; j++, advance(strip, col)) {
                if (j == 0 || col == 0) {
                    if (nstrip > 0 && !mbar_wait(lfree, (uint32_t)(nstrip - 1) & 1u, &s_abort, a.err)) break;
                    mbar_arrive_tx(lfull, kUpdL);
                    for (int kb = 0; kb < 4; kb++)
                        for (int p = 0; p < 3; p++)
                            tma_load_2d(lpart(kb) + p * (kRows * kKb * 2), &tmL, kb * kKb, p * a.m + strip * kRows, lfull);
                    nstrip++;
                    lissued = nstrip;
                }
                bool okb = true;
                for (int kb = 0; kb < 4; kb++) {
                    const int n = 4 * j + kb, s = n % kUpdRing;
                    const uint32_t ph = (uint32_t)(n / kUpdRing) & 1u;
                    if (!mbar_wait(bempty + s, ph ^ 1u, &s_abort, a.err)) { okb = false; break; }
                    mbar_arrive_tx(bfull + s, kUpdBslot);
                    for (int p = 0; p < 3; p++) {
                        tma_load_2d(bslot(s) + p * kUpdBpart, &tmR, kb * kKb, p * a.m + col * kUpdCols, bfull + s);
                        tma_load_2d(bslot(s) + p * kUpdBpart + kUpdCols * 64, &tmRi, kb * kKb, p * a.m + col * kUpdCols,
                                    bfull + s);
                    }
                    issued = n + 1;
                }
                if (!okb) break;
            }
            for (int s = 0; s < kUpdRing; s++) mbar_drain(bfull + s, s < issued ? (issued - 1 - s) / kUpdRing : -1);
            mbar_drain(lfull, lissued - 1);
        }
    } else if (warp == 10) {
        if (lane == 0) {
            // the A22 tiles: tile j into buffer j % kUpdCbuf once tile j - kUpdCbuf has been stored
            prefetch_map(&tmC);
            int issued = 0, strip = strip0, col = col0;
            for (int j = 0; j < nt; j++, advance(strip, col)) {
                const int cb = j % kUpdCbuf;
                if (j >= kUpdCbuf && !mbar_wait(cempty + cb, (uint32_t)(j / kUpdCbuf - 1) & 1u, &s_abort, a.err)) break;
                mbar_arrive_tx(cfull + cb, kUpdC);
                tma_load_2d(Cs(cb), &tmC, 2 * strip * kRows, col * kUpdCols, cfull + cb);
                issued = j + 1;
            }
            for (int b = 0; b < kUpdCbuf; b++) mbar_drain(cfull + b, b < issued ? (issued - 1 - b) / kUpdCbuf : -1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int nstrip = 0, strip = strip0, col = col0;
            for (int j = 0; j < nt; j++, advance(strip, col)) {
                if (j == 0 || col == 0) {
                    if (!mbar_wait(lfull, (uint32_t)nstrip & 1u, &s_abort, a.err)) break;
                    nstrip++;
                }
                const int b = j % kUpdAcc;
                if (j >= kUpdAcc && !mbar_wait(tempty + b, (uint32_t)(j / kUpdAcc - 1) & 1u, &s_abort, a.err)) break;
                tc_fence_after();
                const uint32_t tb = tmem + (uint32_t)(kUpdAccCols * b);
                bool okb = true;
                for (int kb = 0; kb < 4; kb++) {
                    const int n = 4 * j + kb, s = n % kUpdRing;
                    const uint32_t ph = (uint32_t)(n / kUpdRing) & 1u;
                    if (!mbar_wait(bfull + s, ph, &s_abort, a.err)) { okb = false; break; }
                    tc_fence_after();
                    mma_block_cat<2 * kUpdCols>(tb, lpart(kb), kRows * kKb * 2, bslot(s), kb == 0);
                    mma_commit(bempty + s);
                }
                if (!okb) break;
                mma_commit(tfull + b);
                if (j == nt - 1 || col == a.ncols - 1) mma_commit(lfree);
            }
        }
    } else if (warp >= 2 && warp < 10) {
        // workers: warp w reads tensor-memory lanes 32 (w % 4) ..; warps 2-5 take complex columns
        // 0 .. kUpdCols / 2 - 1 of the tile, warps 6-9 the rest
        constexpr int kHalf = kUpdCols / 2;
        const int q = warp & 3, half = (warp - 2) >> 2;
        const int r = q * 32 + lane;   // row of the tile
        const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(kHalf * half);
        int strip = strip0, col = col0;
        for (int j = 0; j < nt; j++, advance(strip, col)) {
            const int b = j % kUpdAcc, cb = j % kUpdCbuf;
            static_assert(kHalf == 16, "two column halves of 16 per tile");
            // this warp's part of the A22 tile into registers; then the buffer may be refilled
            bool ok = __all_sync(0xffffffffu, mbar_wait(cfull + cb, (uint32_t)(j / kUpdCbuf) & 1u, &s_abort, a.err));
            float2 x[kHalf];
            if (ok) {
                const float* C = Cs(cb);
#pragma unroll
                for (int u = 0; u < kHalf; u++) x[u] = reinterpret_cast<const float2*>(C + (kHalf * half + u) * 2 * kRows)[r];
            }
            mbar_arrive_warp(cempty + cb);
            ok = __all_sync(0xffffffffu, ok && mbar_wait(tfull + b, (uint32_t)(j / kUpdAcc) & 1u, &s_abort, a.err));
            tc_fence_after();
            float v[6 * kHalf];   // Re, Im of each column group, this warp's columns
            const uint32_t tb = tq + (uint32_t)(kUpdAccCols * b);
            tmem_ld6x16(tb, tb + kUpdCols, tb + 2 * kUpdCols, tb + 3 * kUpdCols, tb + 4 * kUpdCols, tb + 5 * kUpdCols, v);
            tc_fence_before();
            mbar_arrive_warp(tempty + b);
            if (!ok) break;
            // the updated tile straight to A22 (each column: 32 lanes, 256 contiguous bytes)
            const int row = strip * kRows + r, c0 = col * kUpdCols + kHalf * half;
            if (row < a.m) {
                float2* out = a.A + (int64_t)c0 * a.lda + row;
#pragma unroll
                for (int u = 0; u < kHalf; u++)
                    if (c0 + u < a.m)
                        out[(int64_t)u * a.lda] = make_float2(x[u].x - (v[u] + (v[2 * kHalf + u] + v[4 * kHalf + u])),
                                                              x[u].y - (v[kHalf + u] + (v[3 * kHalf + u] + v[5 * kHalf + u])));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// L, R, iR parts [3][m][128] (BF16, row-major: 64 complex per row): L = [V W], R = [W V], zero
// beyond kk
__global__ void tc_prep_update_kernel(int m, int kk, const float2* __restrict__ V, const float2* __restrict__ W,
                                      __nv_bfloat16* __restrict__ L, __nv_bfloat16* __restrict__ R,
                                      __nv_bfloat16* __restrict__ Ri) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)m * 64;
    if (t >= n) return;
    const int i = (int)(t >> 6), p = (int)(t & 63), pp = p & 31;
    float2 l = make_float2(0.f, 0.f), rr = l;
    if (pp < kk) {
        const float2 v = V[i + (int64_t)pp * m], w = W[i + (int64_t)pp * m];
        l = p < 32 ? v : w;
        rr = p < 32 ? w : v;
    }
    const int64_t e = 2 * t, np = 2 * n;   // real index of the pair, part stride
    split3(l.x, L[e], L[np + e], L[2 * np + e]);
    split3(l.y, L[e + 1], L[np + e + 1], L[2 * np + e + 1]);
    split3(rr.x, R[e], R[np + e], R[2 * np + e]);
    split3(rr.y, R[e + 1], R[np + e + 1], R[2 * np + e + 1]);
    split3(-rr.y, Ri[e], Ri[np + e], Ri[2 * np + e]);
    split3(rr.x, Ri[e + 1], Ri[np + e + 1], Ri[2 * np + e + 1]);
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

}  // namespace tc

size_t tc_workspace(int n, int nsm) {
    using namespace tc;
    // the hemm (B1 parts, stream-K partial sums) and the update (L, R, iR parts) use the same
    // region in turn; a CTA's partial sums cover at most ceil(tiles / G) + 2 tiles
    const size_t tiles = (size_t)(n + kRows - 1) / kRows;
    const size_t hemm = al256((size_t)3 * 64 * kpad_of(n) * sizeof(__nv_bfloat16)) +
                        al256((tiles + 3 * (size_t)nsm) * kRows * 64 * sizeof(float));
    const size_t upd = 3 * al256((size_t)3 * n * 128 * sizeof(__nv_bfloat16));
    return std::max(hemm, upd) + 1024;
}

bool tc_supported(int64_t lda) { return (lda % 2) == 0 && tc::encode_fn() != nullptr; }

// Y = A22 V (A22 Hermitian, full storage) with the tensor cores.
int tc_hemm(cudaStream_t st, int nsm, int m, int kk, const float2* A22, int64_t lda, const float2* V, float2* Y, char* ws,
            int* err, int* launches, cudaEvent_t* ev) {
    using namespace tc;
    if (m % 2) return 4;   // TMA clips the 2m-real columns at 16-byte granules: m even
    if (set_attributes() != cudaSuccess) return 1;
    const int kpad = kpad_of(m), tiles = (m + kRows - 1) / kRows, KB = kpad / kKb;
    HemmArgs h;
    h.m = m;
    h.kb_per_tile = KB;
    h.ntiles = tiles;
    h.units = (int64_t)tiles * KB;
    const int64_t G = std::min<int64_t>(nsm, h.units);
    const int64_t per = (h.units + G - 1) / G;
    h.slots = (int)((per + KB - 1) / KB + 1);
    h.err = err;
    __nv_bfloat16* B = reinterpret_cast<__nv_bfloat16*>(ws);
    h.P = reinterpret_cast<float*>(ws + al256((size_t)3 * 64 * kpad * sizeof(__nv_bfloat16)));
    CUtensorMap mA, mB;
    if (!make_map(&mA, A22, 2 * (uint64_t)m, (uint64_t)m, 2 * (uint64_t)lda * sizeof(float), kKb, kRows, MapKind::f32_sw128) ||
        !make_map(&mB, B, (uint64_t)kpad, 3 * 64, (uint64_t)kpad * sizeof(__nv_bfloat16), kKb, 64, MapKind::bf16_sw64))
        return 2;
    const int64_t nb = (int64_t)64 * kpad;
    tc_prep_hemm_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(m, kk, V, kpad, B);
    if (ev) cudaEventRecord(ev[0], st);
    tc_hemm_kernel<<<(unsigned)G, kHemmThreads, kHemmSmem, st>>>(mA, mB, h);
    if (ev) cudaEventRecord(ev[1], st);
    tc_hemm_reduce_kernel<<<(unsigned)(((int64_t)m * kk + 255) / 256), 256, 0, st>>>(m, kk, h, G, Y);
    *launches += 3;
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

// A22 -= V W^H + W V^H (full storage) with the tensor cores.
int tc_rank2k(cudaStream_t st, int nsm, int m, int kk, float2* A22, int64_t lda, const float2* V, const float2* W, char* ws,
              int* err, int* launches, cudaEvent_t* ev) {
    using namespace tc;
    if (m % 2) return 4;   // the TMA store of a C tile clips at 16-byte granules: 2m reals, m even
    if (set_attributes() != cudaSuccess) return 1;
    const size_t blk = al256((size_t)3 * m * 128 * sizeof(__nv_bfloat16));
    __nv_bfloat16* L = reinterpret_cast<__nv_bfloat16*>(ws);
    __nv_bfloat16* R = reinterpret_cast<__nv_bfloat16*>(ws + blk);
    __nv_bfloat16* Ri = reinterpret_cast<__nv_bfloat16*>(ws + 2 * blk);
    CUtensorMap mC, mL, mR, mRi;
    if (!make_map(&mC, A22, 2 * (uint64_t)m, (uint64_t)m, 2 * (uint64_t)lda * sizeof(float), 2 * kRows, kUpdCols,
                  MapKind::f32_plain) ||
        !make_map(&mL, L, 128, 3 * (uint64_t)m, 128 * sizeof(__nv_bfloat16), kKb, kRows, MapKind::bf16_sw64) ||
        !make_map(&mR, R, 128, 3 * (uint64_t)m, 128 * sizeof(__nv_bfloat16), kKb, kUpdCols, MapKind::bf16_sw64) ||
        !make_map(&mRi, Ri, 128, 3 * (uint64_t)m, 128 * sizeof(__nv_bfloat16), kKb, kUpdCols, MapKind::bf16_sw64))
        return 2;
    tc_prep_update_kernel<<<(unsigned)(((int64_t)m * 64 + 255) / 256), 256, 0, st>>>(m, kk, V, W, L, R, Ri);
    UpdArgs a;
    a.m = m;
    a.nstrips = (m + kRows - 1) / kRows;
    a.ncols = (m + kUpdCols - 1) / kUpdCols;
    a.ntiles = (int64_t)a.nstrips * a.ncols;
    a.A = A22;
    a.lda = lda;
    a.err = err;
    const int64_t G = std::min<int64_t>(nsm, a.ntiles);
    if (ev) cudaEventRecord(ev[0], st);
    tc_update_kernel<<<(unsigned)G, kUpdThreads, kUpdSmem, st>>>(mC, mL, mR, mRi, a);
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
    if (m < 2 || (m % 2) != 0 || kk < 1 || kk > 32 || lda < m || (lda % 2) != 0 || !bse::tc_supported(lda))
        return BSE_ERR_BAD_INPUT;
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
                          : bse::tc_rank2k(0, nsm, m, kk, dA, lda, dV, dW, ws, derr, &launches);
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
