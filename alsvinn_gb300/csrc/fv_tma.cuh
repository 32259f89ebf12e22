// Tile + halo staging by the Tensor Memory Accelerator (sm_90+ bulk tensor
// copies, cp.async.bulk.tensor): one elected thread issues one copy per state
// array for the whole (tile + halo) box of a CTA, completion is tracked by a
// shared-memory mbarrier's transaction count, and every thread waits on the
// barrier's phase with a time limit.
//
// A state array of a grid is described to the TMA unit as a tensor of rank
// dim + 1: (x, [y, [z,]] variable), x fastest, with the padded extents and the
// byte strides of the SoA layout. The box is the tile plus its ghost-cell halo
// in every active dimension, times all variables, so one copy lands the halo
// in shared memory in exactly the order the reconstruction phase reads it
// (variable-major, then z, y, x). Elements of the box outside the padded
// array (tiles at the upper edge of the grid) are filled with zeros; they only
// feed faces outside the grid's interior, which are neither stored nor counted
// in the wave-speed maximum.
//
// TMA rules the host checks before it encodes a map (cuTensorMapEncodeTiled):
// a 16-byte aligned base, byte strides that are multiples of 16 (the padded
// row t_x * sizeof(element)), a box row HX * sizeof(element) that is a
// multiple of 16, box extents <= 256. The x coordinate of every copy is the
// tile origin, a multiple of the tile width, and tile widths times the
// element size are multiples of 16 bytes. Arrays that break a rule run the
// plain load path. Only plain per-CTA copies from this GPU's memory are used
// (no cluster multicast).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "fv_types.h"

namespace gbfv {

// Status a kernel leaves in StepState::status when a halo copy did not
// complete within the time limit.
constexpr int kStatusTmaTimeout = 2;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async proxy
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// One arrival that also announces `bytes` of transactions for this phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

// Waits for the completion of `phase`; false after about one second (or 2^24
// polls, whichever comes first) without completion.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned phase) {
    if (mbar_try_wait(bar, phase)) return true;
    const unsigned long long t0 = global_ns();
    for (int i = 0; i < (1 << 24); ++i) {
        if (mbar_try_wait(bar, phase)) return true;
        if ((i & 255) == 255 && global_ns() - t0 > 1000000000ull) return false;
    }
    return false;
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later async-proxy (TMA) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// A tensor map that the host wrote to global memory (cudaMemcpy) is fetched
// by the tensor-map proxy; this acquire orders the host's write before the
// copies that use it.
__device__ __forceinline__ void fence_tensormap_acquire(const CUtensorMap* map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;\n" ::"l"(map) : "memory");
}

// One box copy global -> shared of a rank DIM + 1 state tensor, box origin
// (x, y, z) in padded coordinates, variable 0. Signals `bar` with the box's
// byte count on completion.
template <int DIM>
__device__ __forceinline__ void tma_load_halo(void* dst, const CUtensorMap* map, unsigned long long* bar, int x, int y,
                                              int z) {
    const unsigned long long m = reinterpret_cast<unsigned long long>(map);
    if constexpr (DIM == 1) {
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
                "r"(smem_addr(dst)),
            "l"(m), "r"(x), "r"(0), "r"(smem_addr(bar))
            : "memory");
    } else if constexpr (DIM == 2) {
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];\n" ::"r"(smem_addr(dst)),
            "l"(m), "r"(x), "r"(y), "r"(0), "r"(smem_addr(bar))
            : "memory");
    } else {
        asm volatile(
            "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
            "[%6];\n" ::"r"(smem_addr(dst)),
            "l"(m), "r"(x), "r"(y), "r"(z), "r"(0), "r"(smem_addr(bar))
            : "memory");
    }
}

}  // namespace gbfv

// Host side: encodes the tensor map of one padded SoA state array for a halo
// box of (hx, hy, hz) cells (the extents of inactive dimensions are ignored).
// Returns false, leaving *map untouched, when the array or the box breaks a
// TMA rule or the driver entry point is unavailable; the caller then uses the
// plain load path.
bool gbfv_encode_state_map(CUtensorMap* map, const void* base, const gbfv::Grid& G, int nvar, int elem, int hx,
                           int hy, int hz);
