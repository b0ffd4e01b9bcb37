// Tensor-memory-accelerator (TMA) staging of state tiles: 2-D tiled bulk
// copies global -> shared that complete on an mbarrier (sm_90+ PTX, used
// here for sm_103a).  Only the types of <cuda.h> are used; the tensor maps
// are encoded through the driver entry point the runtime hands out, so the
// library does not link libcuda.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace goc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// The calling thread arrives on the barrier and announces `bytes` of copies.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the phase of parity `parity` to complete, for at most `limit_ns`
// nanoseconds of the global timer (and at most 2^26 polls, whatever the
// timer does).  Returns false when the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < (1u << 26) && global_ns() - t0 < limit_ns; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Order this thread's earlier generic-proxy accesses of shared memory (made
// visible to it by a preceding barrier) before later async-proxy writes.
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Tiled 2-D copy of the box at (x, y) (elements; x * 4 bytes must be a
// multiple of 16) of `map` into shared memory at `dst`, completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Time after which a staging wait gives up (far longer than any copy takes).
constexpr uint64_t kTmaWaitLimitNs = 200000000ull;  // 0.2 s

// Per-CTA state of the staging of one tile's inputs by TMA: Q^n (eta, hu,
// hv) and, when `aux` is set, the cell-mean depth and the per-cell Coriolis
// f.  Each field comes as a main box of the tile's width starting two
// columns west of the tile (x on a 16-byte boundary) and a 4-column box east
// of it for the last two columns.
struct TileTma {
    const CUtensorMap* in_maps;    // eta, hu, hv main boxes of the input set (null: no staging)
    const CUtensorMap* edge_maps;  // eta, hu, hv east boxes of the input set
    const CUtensorMap* aux_maps;   // cell-mean depth main + east, Coriolis main + east (null: none)
    bool aux_coriolis;             // aux_maps has the Coriolis boxes
    float* edge;                   // shared [5][rows][4]: east boxes of eta, hu, hv, depth, Coriolis
    uint64_t* bar;                 // completes when a staged tile has landed
    uint32_t phase;                // parity of the barrier phase to wait for next
    bool staged;                   // this tile's Q^n is (being) staged
    bool aux;                      // ... and its depth / Coriolis boxes too
    bool next_aux;                 // stage the next tile's depth / Coriolis boxes as well
    int next_tile_y;               // tile row to stage during this tile's last phase (-1: none)
    int* off;                      // shared flag: a wait ran out, the CTA stops staging
    int* err;                      // global flag the host reads
};

}  // namespace goc
