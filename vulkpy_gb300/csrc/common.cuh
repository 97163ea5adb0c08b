// Internal definitions shared by the runtime and the kernel files.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cstdio>
#include <cstdarg>
#include <atomic>
#include <mutex>
#include <string>
#include <utility>
#include <unordered_map>
#include <vector>

#include "../../include/vulkpy_gb300.h"

#define VKC_EXPORT extern "C" __attribute__((visibility("default")))

struct vkc_device {
  int index = 0;
  int sm_count = 0;
  int cc_major = 0, cc_minor = 0;
  cudaStream_t own_stream = nullptr;   // compute stream created at open
  cudaStream_t stream = nullptr;       // current compute stream (own or user's)
  cudaStream_t copy_stream = nullptr;  // uploads into fresh buffers
  cudaMemPool_t upload_pool = nullptr; // their buffers (reused only by later uploads)
  // Upload buffers the caller freed, each with an event on the compute stream
  // after its last use: the next upload of the same size takes one (waiting
  // on that event if needed) instead of allocating (vkc_free / vkc_upload*).
  struct UploadBlock {
    void* ptr;
    size_t bytes;
    cudaEvent_t freed;
  };
  std::vector<UploadBlock> upload_free;
  std::unordered_map<void*, size_t> upload_live;  // upload buffers in use, by size
  cudaEvent_t copy_done = nullptr;     // reused marker for uploads
  cudaStream_t d2h_stream = nullptr;   // asynchronous read-backs (vkc_d2h_async)
  cudaEvent_t d2h_after = nullptr;     // reused marker: compute work a read-back follows
  cudaStream_t side_stream = nullptr;  // independent work forked from `stream` inside one call
  cudaStream_t bias_stream = nullptr;  // a second such branch (the Dense backward's bias sums)
  cudaEvent_t side_fork = nullptr, side_join = nullptr, bias_join = nullptr;
  int side_defer = 0;    // vkc_side_defer: leave the branches open until vkc_side_defer(dev, 0)
  int side_pending = 0;  // branches forked and not yet joined back
  uint32_t* err_word = nullptr;        // device error flags (bit0: gather index)
  uint32_t* done_ctr = nullptr;        // arrival counter of last-block reductions (zero between kernels)
  uint32_t* xo_jump_pows = nullptr;    // xoshiro jump-map powers (lazy)
  uint32_t* xo_next_pows = nullptr;    // xoshiro next-map powers (lazy)
  std::mutex mu;
  char name[256] = {0};
};

struct vkc_job {
  cudaEvent_t ev = nullptr;
  int device = 0;
};

namespace vkc {

// Record an error message for vkc_last_error() and return `code`.
int set_error(int code, const char* fmt, ...);
void clear_error();

// Make `dev` current on this thread; returns VKC_OK or an error code.
int bind(vkc_device_t dev);

extern std::atomic<uint64_t> g_launches;  // kernels launched (all devices)

// Counts an allocation request and reports whether an injected failure
// (vkc_inject_alloc_failure) falls on it.
bool alloc_should_fail();

inline int check_launch(const char* what) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(VKC_ERR_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
  return VKC_OK;
}

// Grid for a grid-stride streaming kernel with `threads` per block.
inline unsigned stream_grid(const vkc_device* dev, size_t work_items, int threads, int blocks_per_sm = 8) {
  size_t want = (work_items + threads - 1) / threads;
  size_t cap = (size_t)dev->sm_count * blocks_per_sm;
  if (want < 1) want = 1;
  return (unsigned)(want < cap ? want : cap);
}

// Blocks of `kernel` resident per SM at `threads` threads and `smem` bytes of
// dynamic shared memory (cudaOccupancyMaxActiveBlocksPerMultiprocessor,
// cached per kernel; at least 1).
int resident_blocks(const void* kernel, int threads, size_t smem = 0);

// Grid for a grid-stride kernel: at most one full wave of resident blocks.
// A grid sized for more blocks than fit (e.g. 8 per SM for a kernel whose
// registers allow 5) runs a partial second wave that leaves SMs idle at the
// end of the launch.
template <class K>
inline unsigned wave_grid(const vkc_device* dev, K* kernel, size_t work_items, int threads, size_t smem = 0) {
  size_t want = (work_items + threads - 1) / threads;
  if (want < 1) want = 1;
  const size_t cap = (size_t)dev->sm_count * (size_t)resident_blocks((const void*)kernel, threads, smem);
  return (unsigned)(want < cap ? want : cap);
}

// Stream-ordered scratch allocation on the device's current stream.
int scratch_alloc(vkc_device_t dev, size_t bytes, void** p);
void scratch_free(vkc_device_t dev, void* p);

// ---- programmatic dependent launch (PDL)
// A kernel launched with launch_pdl may be scheduled while the kernel before
// it on the stream is still running: its blocks become resident as that
// kernel's blocks trigger (pdl_trigger) or exit, then wait in pdl_wait()
// until it has completed and its memory is visible.  So the launch gap and
// the block scheduling of consecutive short kernels overlap.  Every kernel
// launched this way calls pdl_wait() before it touches global memory (after
// it, everything the previous kernel wrote is visible, as after an ordinary
// launch); without the launch attribute both calls are no-ops.
extern std::atomic<int> g_pdl;             // 1: launch_pdl adds the attribute (vkc_set_pdl)
extern std::atomic<int> g_cluster_splitk;  // 1: split-K reduced inside the GEMM (vkc_set_cluster_splitk)

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_pdl.load(std::memory_order_relaxed) ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// launch_pdl with the blocks grouped into 1-D thread-block clusters of
// `cluster` CTAs (grid.x a multiple of it).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl_cluster(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                                      unsigned cluster, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_pdl.load(std::memory_order_relaxed) ? 2 : 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace vkc

#define VKC_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e__ = (call);                                                            \
    if (e__ != cudaSuccess)                                                              \
      return vkc::set_error(VKC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e__));     \
  } while (0)

#define VKC_REQUIRE(cond, ...)                                                           \
  do {                                                                                   \
    if (!(cond)) return vkc::set_error(VKC_ERR_INVALID, __VA_ARGS__);                    \
  } while (0)

#define VKC_BIND(dev)                                                                    \
  do {                                                                                   \
    int r__ = vkc::bind(dev);                                                            \
    if (r__ != VKC_OK) return r__;                                                       \
  } while (0)
