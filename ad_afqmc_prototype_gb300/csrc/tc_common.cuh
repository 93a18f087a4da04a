// Blackwell building blocks shared by the tensor-core kernels: bounded
// mbarrier waits, TMA tile loads, tcgen05 descriptors, MMA issue and tensor
// memory loads, and the host-side tensor-map encoder.
//
// Every wait is bounded (1 s of %globaltimer) and reports a timeout to the
// caller, which raises the kernel's error flag and unwinds.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

#include "afq_internal.cuh"

namespace afq {
namespace tc {

constexpr unsigned long long WAIT_NS = 1000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase with `parity`; false on timeout (limit_ns of
// the global timer) or abort.  The abort flag and the timer are read every
// 16th poll: a poll that has just failed costs no timer read on the way to
// the next one.
__device__ __forceinline__ bool mbar_wait_inl(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                              unsigned long long limit_ns = WAIT_NS) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    for (unsigned it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 15u) == 0u) {
            if (abort_flag && *abort_flag) return false;
            if (now_ns() - t0 > limit_ns) return false;
        }
    }
}
static __device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                              unsigned long long limit_ns = WAIT_NS) {
    return mbar_wait_inl(bar, parity, abort_flag, limit_ns);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(dst),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand tile with 128-byte swizzle: 128-byte rows, 8-row atoms
// 1024 bytes apart (stride byte offset), descriptor version 1 (bit 46),
// swizzle mode 2 (bits 61-63).  The leading byte offset is unused for this
// layout.  Advancing K by 16 bf16 (32 bytes) inside the 128-byte row moves the
// start address; the tile base is 1024-byte aligned so the swizzle phase is 0.
__device__ __forceinline__ uint64_t desc_k128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ void umma_bf16_i(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

#define AFQ_R8(i)                                                                                              \
    "=r"(r[i]), "=r"(r[i + 1]), "=r"(r[i + 2]), "=r"(r[i + 3]), "=r"(r[i + 4]), "=r"(r[i + 5]), "=r"(r[i + 6]), \
        "=r"(r[i + 7])
// 64 consecutive fp32 columns of this warp's 32 lanes; returns after the load completed.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&r)[64]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, "
        "%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, "
        "%48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : AFQ_R8(0), AFQ_R8(8), AFQ_R8(16), AFQ_R8(24), AFQ_R8(32), AFQ_R8(40), AFQ_R8(48), AFQ_R8(56)
        : "r"(taddr)
        : "memory");
}
#undef AFQ_R8

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}


// ------------------------------------------------------------------- host --
// The driver's tensor-map encoder (the same for every device), looked up on
// first use; the function-local static makes the lookup thread-safe.
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;  // per translation unit

static PFN_cuTensorMapEncodeTiled_v12000 lookup_encode() {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess) return nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)fn;
}

static int get_encode() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = lookup_encode();
    if (!fn) return fail(AFQ_E_CUDA, "cuTensorMapEncodeTiled is unavailable");
    g_encode = fn;
    return AFQ_OK;
}

// rows x cols bf16 matrix, row stride ld elements, box = box_rows x box_cols
// (box_cols x 2 bytes <= 128: one 128-byte swizzle row); out-of-range
// elements read as zero.
static int make_map(CUtensorMap* m, const void* base, long long rows, long long cols, long long ld, int box_rows,
                    int box_cols = 64) {
    if (((uintptr_t)base) & 15) return fail(AFQ_E_INVALID_ARGUMENT, "tensor base not 16-byte aligned");
    if ((ld * 2) % 16) return fail(AFQ_E_INVALID_ARGUMENT, "tensor row stride not a multiple of 16 bytes");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
    cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(AFQ_E_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return AFQ_OK;
}

// planes x rows x cols bf16 array (row stride ld elements, plane stride
// rows x ld), box = box_rows x box_cols of one plane; rows past the end of a
// plane read as zero instead of the next plane's rows.
static int make_map3(CUtensorMap* m, const void* base, long long planes, long long rows, long long cols, long long ld,
                     int box_rows, int box_cols = 64) {
    if (((uintptr_t)base) & 15) return fail(AFQ_E_INVALID_ARGUMENT, "tensor base not 16-byte aligned");
    if ((ld * 2) % 16) return fail(AFQ_E_INVALID_ARGUMENT, "tensor row stride not a multiple of 16 bytes");
    cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)(ld * 2), (cuuint64_t)(rows * ld * 2)};
    cuuint32_t box[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)base, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(AFQ_E_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return AFQ_OK;
}

}  // namespace tc
}  // namespace afq
