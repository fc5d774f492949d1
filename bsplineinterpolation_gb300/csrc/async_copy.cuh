// Asynchronous global <-> shared copies used by the tiled line solves:
// TMA bulk copies (cp.async.bulk) completing on an mbarrier, and per-thread
// cp.async element copies. Every wait is bounded: a wait that runs out sets
// the device error flag (read back by intp_stream_synchronize) and returns.
#pragma once

#include <cstdint>

namespace intp_gb300 {

// Set by a kernel whose bounded wait ran out; read and cleared by the host
// (one copy per translation unit that includes this header).
static __device__ int g_device_error;
constexpr int kErrWaitTimeout = 1;

// Diagnostics (intp_debug_set_wait_limit): when nonzero, the binned
// evaluation's wait for each staged tile gives up after this many
// non-blocking probes of its barrier instead of its normal bounded wait.
static __device__ uint32_t g_tile_wait_probes;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Waits for phase `parity` of the barrier; gives up after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = (1u << 26)) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    atomicExch(&g_device_error, kErrWaitTimeout);
    return false;
}

// At most `probes` non-blocking tests of phase `parity` (mbarrier.test_wait);
// on giving up sets the device error flag like mbar_wait.
__device__ __forceinline__ bool mbar_probe(uint64_t* bar, uint32_t parity, uint32_t probes) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t i = 0; i < probes; ++i) {
        uint32_t done;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    atomicExch(&g_device_error, kErrWaitTimeout);
    return false;
}

// TMA bulk copy global -> shared (size a multiple of 16, both 16-byte aligned)
__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// TMA tiled tensor loads global -> shared of one box (the map's box sizes),
// completing on `bar`. Coordinates are in elements, innermost first; the
// innermost coordinate times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst_smem, const void* tmap, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst_smem)),
        "l"(tmap), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst_smem, const void* tmap, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst_smem)),
        "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// TMA bulk copy shared -> global, tracked by the bulk async-group
__device__ __forceinline__ void bulk_store(void* dst, const void* src_smem, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src_smem)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// waits until the shared-memory sources of committed bulk stores were read
__device__ __forceinline__ void bulk_store_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// waits until committed bulk stores have completed
__device__ __forceinline__ void bulk_store_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// orders generic-proxy shared-memory writes before async-proxy reads
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// per-thread asynchronous copy of 4 or 8 bytes global -> shared
template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst_smem, const void* src) {
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async size");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst_smem)), "l"(src), "n"(BYTES)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Defines `int NAME(cudaStream_t)`: reads and clears this translation unit's
// copy of g_device_error (each unit that waits on a barrier has its own).
#define INTP_DEFINE_DEVICE_ERROR_READER(NAME)                                                                 \
    int NAME(cudaStream_t s) {                                                                                \
        int v = 0, zero = 0;                                                                                  \
        if (cudaMemcpyFromSymbolAsync(&v, g_device_error, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess) \
            return 0;                                                                                         \
        cudaMemcpyToSymbolAsync(g_device_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s);            \
        cudaStreamSynchronize(s);                                                                             \
        return v;                                                                                             \
    }

// Defines `cudaError_t NAME(uint32_t)`: sets this translation unit's copy of
// g_tile_wait_probes (0 = the normal wait).
#define INTP_DEFINE_WAIT_PROBE_SETTER(NAME)                                                    \
    cudaError_t NAME(uint32_t probes) {                                                        \
        return cudaMemcpyToSymbol(g_tile_wait_probes, &probes, sizeof(uint32_t), 0,            \
                                  cudaMemcpyHostToDevice);                                     \
    }

}  // namespace intp_gb300
