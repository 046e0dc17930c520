// Tensor-memory-accelerator (TMA) staging of a stage kernel's input tile.
//
// One thread of a block issues a single cp.async.bulk.tensor copy of the
// tile plus its halo, all S conserved variables at once, from the SoA state
// [S][rows][pitch] into shared memory; an mbarrier counts the bytes in.  The
// tensor map describes one state register as a 3-D FP64 tensor (x, y,
// variable); it is encoded on the host per launch (a host-only call that
// writes 128 bytes) and passed as a __grid_constant__ kernel parameter.
//
// Alignment: the copy's innermost coordinate x times 8 bytes must be a
// multiple of 16, so x starts on an even cell (kTmaLead cells before the
// tile, one more than the halo when the halo depth is odd) and the box is an
// even number of cells wide.  The state's row pitch and variable stride are
// multiples of 16 bytes and its base 16-byte aligned, or no map is encoded.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mfc_gpu.h"

namespace mfc {

struct TileMap {
  CUtensorMap map;
  int on;  // 0: no map (the kernel loads every tile with plain loads)
};

// x extent of a TMA tile box: H ghost cells each side of TX, started on an
// even cell and rounded up to an even width.
template <int TX, int H>
struct TmaBox {
  static constexpr int kLead = H + (H & 1);                 // cells before the tile's first cell
  static constexpr int kWidth = (kLead + TX + H + 1) / 2 * 2;  // even
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  // make the initialised barrier visible to the copy engine
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later copy-engine (async-proxy) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Acquire of a tensor map held in global memory (written by a copy from the
// host), before the copy engine reads it.
__device__ __forceinline__ void tensormap_acquire(const void* map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// One poll of phase `parity` of `bar`; a thread whose phase is incomplete
// may be suspended for at most about 0.1 ms before the poll returns false.
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity), "r"(100000u)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// 3-D tiled copy global -> shared, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// 4-D tiled copy global -> shared, completing on `bar`.
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, int w,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
      : "memory");
}

// Bounded wait of one thread for phase `parity` of `bar`: false once
// `limit_ns` nanoseconds of the global timer have passed, so a copy that
// never lands ends the wait instead of hanging the block.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// Host: encodes the map of one FP64 state register [S][ny][sy] (x fastest,
// variable stride sv elements) with a box of box_w x box_h x S cells.
// Returns false (map.on = 0) when the layout does not meet the TMA rules or
// the driver entry point is unavailable.
bool encode_tile_map(TileMap& t, const double* base, int nx, int ny, int S, int64_t sy, int64_t sv, int box_w,
                     int box_h);

// The same for a 3-D array [S][nz][ny][sy] (plane stride sz) of FP64
// (elem_bytes 8) or FP32 (4) values as a 4-D tensor (x, y, z, variable) with
// a box of bx x by x bz x S cells.
bool encode_tile_map_3d(TileMap& t, const void* base, int elem_bytes, int nx, int ny, int nz, int S, int64_t sy,
                        int64_t sz, int64_t sv, int bx, int by, int bz);

}  // namespace mfc
