// tma.cuh -- tensor-memory-accelerator (TMA) tile copies and the mbarrier
// they complete on, as inline PTX (sm_90 and later; used here on sm_103a).
//
// A tile copy is issued by one thread of the CTA:
//   load:  cp.async.bulk.tensor global -> shared, completion counted in bytes
//          on an mbarrier (expect_tx by the issuing thread, try_wait by all);
//   store: cp.async.bulk.tensor shared -> global in a bulk group, after every
//          writer has fenced its shared-memory writes to the async proxy.
// Tensor maps are encoded on the host (encode_tiled_map, operator.cu) and
// passed as __grid_constant__ kernel parameters.
//
// Alignment rules the callers keep (checked where they are built):
//   - the global base address is 16-byte aligned and every global stride is a
//     multiple of 16 bytes (cuTensorMapEncodeTiled rejects anything else);
//   - the innermost box extent is a multiple of 16 bytes;
//   - the innermost coordinate x of every copy times the element size is a
//     multiple of 16 bytes (nothing checks this before the copy runs);
//   - each shared-memory destination is 128-byte aligned;
//   - no store starts at a negative coordinate.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace bri17gb {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for phase `parity` of the barrier; gives up after `limit_ns`
// nanoseconds of global time and returns false.  A limit of 0 gives up at
// once, without looking at the barrier (a diagnostic setting that makes the
// failure path run).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  if (limit_ns == 0) return false;
  const uint32_t a = smem_addr(bar);
  uint64_t t0 = 0;
  for (uint32_t it = 0;; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (it == 0) t0 = global_timer_ns();
    else if (global_timer_ns() - t0 > limit_ns) return false;
  }
}

// Default limit of a bounded wait on tile copies: one second of global time.
constexpr uint64_t kWaitLimitNs = 1000000000ull;

// A kernel's report of a failed bounded wait: status[0] is set when a wait
// on tile copies ran out, status[1] when a tile was skipped because its
// shared-memory window was misplaced.  `status` points at page-locked host
// memory mapped into the device (the handle's status words; may be null),
// so the host reads it without a copy; kernels only ever store 1.
__device__ __forceinline__ void report_status(int* status, int which) {
  if (status) {
    *reinterpret_cast<volatile int*>(status + which) = 1;
    __threadfence_system();
  }
}

// 3-D tile load into shared memory; completes `bytes` of transactions on bar.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y,
                                            int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// 3-D tile store from shared memory (bulk group of the issuing thread).
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, int x, int y, int z,
                                             const void* src) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group"
      " [%0, {%1, %2, %3}], [%4];" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(x), "r"(y), "r"(z), "r"(smem_addr(src))
      : "memory");
}

__device__ __forceinline__ void tma_store_commit_and_wait() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Makes this thread's generic-proxy shared-memory writes visible to the
// async proxy (before a barrier and a TMA store that reads them).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Host: encodes a 3-D tiled map over `base` (element type FP32 or FP64 by
// elem_bytes): dims[0] contiguous, byte strides for dims 1 and 2, box
// {box0, box1, 1}, zero fill out of bounds.  Returns false when the driver
// entry point is missing or rejects the map.
bool encode_tiled_map_3d(CUtensorMap* map, const void* base, int elem_bytes, uint64_t dim0,
                         uint64_t dim1, uint64_t dim2, uint64_t stride1_bytes,
                         uint64_t stride2_bytes, uint32_t box0, uint32_t box1);

// Bounded waits that ran out in the FP32 / float-pair TMA kernels since the last call
// (read and cleared on the current device).
cudaError_t tma_wait_timeouts_f32(int* count);
cudaError_t tma_wait_timeouts_df(int* count);
// Limit of the first bounded wait on tile copies in those kernels, on the
// current device (diagnostics; kWaitLimitNs by default).  The wait that
// follows a run-out one, for the CTA's own copies in flight, keeps
// kWaitLimitNs.
cudaError_t tma_set_wait_limit_f32(uint64_t ns);
cudaError_t tma_set_wait_limit_df(uint64_t ns);

}  // namespace bri17gb
