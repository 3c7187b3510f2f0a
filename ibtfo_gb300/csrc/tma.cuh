// Tensor-memory-accelerator (TMA) staging of a sweep tile.
//
// The state buffers are 3-D tensors (x = column, y = row, z = conserved
// variable plane) with a row pitch; a tile and its two-cell halo is one box
// of (TX + 4) x (TY + 4) x 4 elements, the shape of the tile's shared-memory
// array, so one bulk tensor copy per CTA stages all four planes.  Elements
// outside the grid arrive as zeros, as the element-wise staging stores them.
// The copy completes on a shared-memory mbarrier; the wait is bounded.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace ibtfo {

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// one 3-D box at (x, y, z) of the tensor described by *map into dst
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
                 : "memory");
}

// true once the barrier's phase `parity` has completed
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return done != 0;
}

// releases the barrier once its phase has completed and no copy is in
// flight, so that the next tile of a persistent CTA can initialise it again
__device__ __forceinline__ void mbar_inval(uint64_t *bar)
{
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// a tensor map that the host wrote into global memory (a batch's case
// table) becomes visible to the tensor-copy unit: acquire fence of the
// tensormap proxy on its 128 bytes, before the first copy that uses it
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *map)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
                 : "memory");
}

// the bounded wait: each try_wait suspends for a hardware-chosen interval,
// so this gives up after far longer than any copy takes
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    for (int it = 0; it < (1 << 20); it++)
        if (mbar_try_wait(bar, parity))
            return true;
    return false;
}

} // namespace ibtfo
