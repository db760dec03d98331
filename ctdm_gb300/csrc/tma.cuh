// Tensor-memory-accelerator (TMA) staging: tensor maps built on the host, bulk
// tensor loads into shared memory completed on an mbarrier, inline PTX only.
//
// A kernel that stages a tile:
//   thread 0: mbar_init(bar, 1); fence; __syncthreads();
//   thread 0: mbar_expect_tx(bar, bytes); tma_load_3d(...) for each box;
//   ... independent work ...
//   every thread: mbar_wait(bar, 0, err)   (bounded: gives up and flags after a
//                                          fixed number of polls, never spins forever)
//
// Rules kept by the callers: the innermost box extent times the element size is a
// multiple of 16 bytes, the innermost start coordinate times the element size is a
// multiple of 16 bytes, the global base is 16-byte aligned and every global stride
// a multiple of 16 bytes; the shared destination is 128-byte aligned.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace tma {

// ---------------------------------------------------------------- device side
__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes the initialised barrier visible to the asynchronous (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// 3-D tiled bulk tensor load global -> shared, completing `bytes` on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for phase `parity` of `bar`.  Returns false (and records `code` in
// *err when err is given) if the phase has not completed after `polls` polls
// (kMaxPolls unless a diagnostic asks for fewer).  Each poll is a hardware try_wait
// that suspends the thread for a while when the phase is still open: measured on a
// GB300, 3.8 us per poll, so kMaxPolls gives up after about one second, far above
// any real tile copy (microseconds).
constexpr int kMaxPolls = 1 << 18;
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, int code, int polls = kMaxPolls)
{
    for (int i = 0; i < polls; i++)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicExch(err, code);
    return false;
}

// Contiguous bulk copy global -> shared of `bytes` (multiple of 16, both addresses
// 16-byte aligned), completing on `bar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(static_cast<uint64_t>(__cvta_generic_to_global(src))), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Contiguous bulk copy shared -> global in the calling thread's bulk group.  The
// writers of the shared source run fence_async_smem() and a barrier first.
__device__ __forceinline__ void bulk_store(void *dst, const void *src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(
                     static_cast<uint64_t>(__cvta_generic_to_global(dst))),
                 "r"(smem_addr(src)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Waits until every committed bulk store has finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Makes this thread's generic-proxy shared-memory writes visible to bulk copies.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Distributed shared memory: the shared::cluster address of `p` (an address in this
// CTA's shared memory) in the CTA of cluster rank `rank`, and 64-bit accesses to it.
__device__ __forceinline__ uint32_t cluster_addr(uint32_t local_smem_addr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_smem_addr), "r"(rank));
    return r;
}
__device__ __forceinline__ float2 ld_cluster(uint32_t addr)
{
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ void st_cluster(uint32_t addr, float2 v)
{
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}

// Prefetch a tensor map descriptor (a kernel parameter) into the descriptor cache.
__device__ __forceinline__ void prefetch_map(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ---------------------------------------------------------------- host side
// Tiled 3-D map over a dense array of `elem_bytes`-sized elements (1 or 8) with
// extents dims[0] (fastest) .. dims[2] and box extents box[0..2].  The element
// type only fixes the size; the bits are copied unchanged.
cudaError_t make_map_3d(CUtensorMap *map, const void *base, int elem_bytes, const uint64_t dims[3],
                        const uint32_t box[3]);

}  // namespace tma
