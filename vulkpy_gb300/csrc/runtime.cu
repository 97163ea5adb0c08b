// Device, stream, memory and job management: the CUDA replacement for the
// Vulkan runtime of vulkpy/_vkarray.cc (class GPU 460-574, Buffer<T> 38-130,
// Job 392-457).  One compute stream per opened device; all kernels and
// copies that touch existing buffers are ordered on it, so dependent ops need
// no host waits (the reference waits on fences, _vkarray.cc:430-432).
#include "common.cuh"

#include <chrono>
#include <thread>
#include <cstring>
#include <unordered_map>

namespace vkc {

std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_pdl{1};
std::atomic<int> g_cluster_splitk{0};
std::atomic<uint64_t> g_allocs{0};          // device + pinned host allocations requested
std::atomic<int64_t> g_fail_alloc_in{-1};   // injected failure: fail when this reaches 0
static thread_local std::string g_last_error;

// Host-side fault injection (vkc_inject_alloc_failure): true when the
// allocation being made now is the one chosen to fail.  Counts every
// allocation request, injected or not.
bool alloc_should_fail() {
  g_allocs.fetch_add(1, std::memory_order_relaxed);
  int64_t v = g_fail_alloc_in.load(std::memory_order_relaxed);
  while (v >= 0) {
    if (g_fail_alloc_in.compare_exchange_weak(v, v - 1, std::memory_order_relaxed)) return v == 0;
  }
  return false;
}

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

void clear_error() { g_last_error.clear(); }

int bind(vkc_device_t dev) {
  if (!dev) return set_error(VKC_ERR_INVALID, "device handle is NULL");
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return set_error(VKC_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (cur != dev->index) {
    e = cudaSetDevice(dev->index);
    if (e != cudaSuccess) return set_error(VKC_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  }
  return VKC_OK;
}

int scratch_alloc(vkc_device_t dev, size_t bytes, void** p) {
  *p = nullptr;
  if (bytes == 0) return VKC_OK;
  if (alloc_should_fail())
    return set_error(VKC_ERR_OOM, "cudaMallocAsync(%zu bytes): injected allocation failure", bytes);
  cudaError_t e = cudaMallocAsync(p, bytes, dev->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(VKC_ERR_OOM, "cudaMallocAsync(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  return VKC_OK;
}

void scratch_free(vkc_device_t dev, void* p) {
  if (p) cudaFreeAsync(p, dev->stream);
}

namespace {
struct OccKey {
  const void* kernel;
  int threads;
  size_t smem;
  bool operator==(const OccKey& o) const { return kernel == o.kernel && threads == o.threads && smem == o.smem; }
};
struct OccHash {
  size_t operator()(const OccKey& k) const {
    return std::hash<const void*>()(k.kernel) ^ (std::hash<size_t>()(k.smem) * 31u) ^ ((size_t)k.threads << 20);
  }
};
std::mutex g_occ_mu;
std::unordered_map<OccKey, int, OccHash> g_occ;
}  // namespace

int resident_blocks(const void* kernel, int threads, size_t smem) {
  const OccKey key{kernel, threads, smem};
  {
    std::lock_guard<std::mutex> lk(g_occ_mu);
    auto it = g_occ.find(key);
    if (it != g_occ.end()) return it->second;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n < 1) {
    cudaGetLastError();
    n = 1;
  }
  std::lock_guard<std::mutex> lk(g_occ_mu);
  g_occ[key] = n;
  return n;
}

}  // namespace vkc

using namespace vkc;

VKC_EXPORT const char* vkc_last_error(void) { return g_last_error.c_str(); }

VKC_EXPORT const char* vkc_version(void) { return "vulkpy_gb300 0.1.0 (sm_103a)"; }

VKC_EXPORT int vkc_device_count(int* count) {
  VKC_REQUIRE(count, "count is NULL");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *count = 0;
    return set_error(VKC_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
  }
  *count = n;
  return VKC_OK;
}

VKC_EXPORT int vkc_device_open(int index, float priority, vkc_device_t* out) {
  VKC_REQUIRE(out, "out is NULL");
  *out = nullptr;
  int n = 0;
  int r = vkc_device_count(&n);
  if (r != VKC_OK) return r;
  VKC_REQUIRE(index >= 0 && index < n, "GPU index %d out of range (%d devices)", index, n);
  VKC_CUDA(cudaSetDevice(index));

  auto* dev = new vkc_device();
  dev->index = index;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, index);
  if (e != cudaSuccess) {
    delete dev;
    return set_error(VKC_ERR_CUDA, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
  }
  dev->sm_count = prop.multiProcessorCount;
  dev->cc_major = prop.major;
  dev->cc_minor = prop.minor;
  std::snprintf(dev->name, sizeof(dev->name), "%s", prop.name);

  // Map priority in [0,1] onto the device's stream priority range
  // (greatest priority is the numerically lowest value).
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  float p = priority < 0.f ? 0.f : (priority > 1.f ? 1.f : priority);
  int prio = lo + (int)((hi - lo) * p);
  e = cudaStreamCreateWithPriority(&dev->own_stream, cudaStreamNonBlocking, prio);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&dev->copy_stream, cudaStreamNonBlocking, prio);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&dev->copy_done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&dev->d2h_stream, cudaStreamNonBlocking, prio);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&dev->d2h_after, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&dev->side_stream, cudaStreamNonBlocking, prio);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&dev->side_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&dev->side_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&dev->bias_stream, cudaStreamNonBlocking, prio);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&dev->bias_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&dev->err_word, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(dev->err_word, 0, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&dev->done_ctr, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(dev->done_ctr, 0, sizeof(uint32_t));
  if (e != cudaSuccess) {
    delete dev;
    return set_error(VKC_ERR_CUDA, "device setup: %s", cudaGetErrorString(e));
  }
  dev->stream = dev->own_stream;

  // Keep freed blocks cached in the pool instead of returning them to the OS:
  // arrays are short-lived and large (up to GiBs), re-mapping is expensive.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, index) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  // Uploads get their own pool.  Their buffers are allocated on the copy
  // stream and freed on the compute stream; in the shared pool the compute
  // stream's own allocations took the freed blocks first, so an upload
  // issued while compute runs often found no finished free block and the
  // pool grew (milliseconds of host time) or the copy waited on compute.
  // Here an upload reuses an earlier upload's block once its free has
  // completed, and never waits on the compute stream for one.
  {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = index;
    if (cudaMemPoolCreate(&dev->upload_pool, &props) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      int no = 0;
      cudaMemPoolSetAttribute(dev->upload_pool, cudaMemPoolAttrReleaseThreshold, &thr);
      cudaMemPoolSetAttribute(dev->upload_pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    } else {
      dev->upload_pool = nullptr;
    }
  }
  cudaGetLastError();
  *out = dev;
  return VKC_OK;
}

VKC_EXPORT int vkc_device_close(vkc_device_t dev) {
  if (!dev) return VKC_OK;
  VKC_BIND(dev);
  cudaStreamSynchronize(dev->own_stream);
  if (dev->stream != dev->own_stream) cudaStreamSynchronize(dev->stream);
  cudaStreamSynchronize(dev->copy_stream);
  cudaStreamSynchronize(dev->d2h_stream);
  for (auto& b : dev->upload_free) {
    cudaFreeAsync(b.ptr, dev->own_stream);
    cudaEventDestroy(b.freed);
  }
  dev->upload_free.clear();
  cudaStreamSynchronize(dev->own_stream);
  if (dev->err_word) cudaFree(dev->err_word);
  if (dev->done_ctr) cudaFree(dev->done_ctr);
  if (dev->xo_jump_pows) cudaFree(dev->xo_jump_pows);
  if (dev->xo_next_pows) cudaFree(dev->xo_next_pows);
  cudaStreamSynchronize(dev->side_stream);
  cudaStreamSynchronize(dev->bias_stream);
  cudaEventDestroy(dev->copy_done);
  cudaEventDestroy(dev->d2h_after);
  cudaStreamDestroy(dev->d2h_stream);
  cudaEventDestroy(dev->side_fork);
  cudaEventDestroy(dev->side_join);
  cudaEventDestroy(dev->bias_join);
  cudaStreamDestroy(dev->own_stream);
  cudaStreamDestroy(dev->copy_stream);
  cudaStreamDestroy(dev->side_stream);
  cudaStreamDestroy(dev->bias_stream);
  // released once its last buffer is freed
  if (dev->upload_pool) cudaMemPoolDestroy(dev->upload_pool);
  delete dev;
  return VKC_OK;
}

VKC_EXPORT int vkc_device_synchronize(vkc_device_t dev) {
  VKC_BIND(dev);
  VKC_CUDA(cudaStreamSynchronize(dev->side_stream));
  VKC_CUDA(cudaStreamSynchronize(dev->bias_stream));
  VKC_CUDA(cudaStreamSynchronize(dev->copy_stream));
  VKC_CUDA(cudaStreamSynchronize(dev->d2h_stream));
  VKC_CUDA(cudaStreamSynchronize(dev->stream));
  return VKC_OK;
}

VKC_EXPORT int vkc_device_stream(vkc_device_t dev, void** stream) {
  VKC_REQUIRE(dev && stream, "NULL argument");
  *stream = (void*)dev->stream;
  return VKC_OK;
}

VKC_EXPORT int vkc_device_set_stream(vkc_device_t dev, void* stream) {
  VKC_REQUIRE(dev, "device handle is NULL");
  dev->stream = stream ? (cudaStream_t)stream : dev->own_stream;
  return VKC_OK;
}

VKC_EXPORT int vkc_device_info(vkc_device_t dev, int* sm_count, char* name, size_t name_len) {
  VKC_REQUIRE(dev, "device handle is NULL");
  if (sm_count) *sm_count = dev->sm_count;
  if (name && name_len) std::snprintf(name, name_len, "%s", dev->name);
  return VKC_OK;
}

VKC_EXPORT int vkc_device_check_errors(vkc_device_t dev, uint32_t* flags) {
  VKC_BIND(dev);
  VKC_REQUIRE(flags, "flags is NULL");
  uint32_t h = 0;
  VKC_CUDA(cudaMemcpyAsync(&h, dev->err_word, sizeof(h), cudaMemcpyDeviceToHost, dev->stream));
  VKC_CUDA(cudaMemsetAsync(dev->err_word, 0, sizeof(uint32_t), dev->stream));
  VKC_CUDA(cudaStreamSynchronize(dev->stream));
  *flags = h;
  return VKC_OK;
}

// ---- memory ---------------------------------------------------------------

VKC_EXPORT int vkc_alloc(vkc_device_t dev, size_t bytes, void** ptr) {
  VKC_BIND(dev);
  VKC_REQUIRE(ptr, "ptr is NULL");
  return scratch_alloc(dev, bytes, ptr);
}

namespace {
constexpr size_t kUploadCacheBlocks = 8;          // cached upload buffers per device at most
constexpr size_t kUploadCacheMin = size_t(1) << 20;  // smaller uploads allocate every time

// A device buffer of `bytes` for an upload on the copy stream (dev->mu
// held): a cached buffer of that size whose last use has finished, else a
// new allocation from the upload pool.  A cached buffer whose last use is
// still queued is not waited for: its free event is recorded when the
// caller drops the array, after everything then queued on the compute
// stream, so waiting would hold the copy behind the current compute (in a
// pipelined loop, the buffer freed two steps back is the finished one).
int upload_take(vkc_device_t dev, size_t bytes, void** p) {
  const bool cached = bytes >= kUploadCacheMin;
  for (size_t i = 0; cached && i < dev->upload_free.size(); ++i) {
    if (dev->upload_free[i].bytes != bytes) continue;
    if (cudaEventQuery(dev->upload_free[i].freed) != cudaSuccess) continue;
    vkc_device::UploadBlock b = dev->upload_free[i];
    dev->upload_free.erase(dev->upload_free.begin() + (long)i);
    cudaEventDestroy(b.freed);
    *p = b.ptr;
    dev->upload_live[b.ptr] = bytes;
    return VKC_OK;
  }
  cudaGetLastError();  // a not-ready query is not an error
  if (vkc::alloc_should_fail())
    return set_error(VKC_ERR_OOM, "cudaMallocAsync(%zu bytes): injected allocation failure", bytes);
  cudaError_t e = dev->upload_pool ? cudaMallocFromPoolAsync(p, bytes, dev->upload_pool, dev->copy_stream)
                                   : cudaMallocAsync(p, bytes, dev->copy_stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return set_error(VKC_ERR_OOM, "cudaMallocAsync(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  if (cached) dev->upload_live[*p] = bytes;
  return VKC_OK;
}
}  // namespace

VKC_EXPORT int vkc_free(vkc_device_t dev, void* ptr) {
  if (!ptr) return VKC_OK;
  VKC_BIND(dev);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(dev->stream, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;
  }
  {
    // a large upload buffer goes to the device's upload cache with an event
    // after its last use on the compute stream (see upload_take); not while
    // the stream is captured (the event would be a graph node, recorded only
    // when the graph runs), then it is freed like any buffer
    std::lock_guard<std::mutex> lk(dev->mu);
    auto it = dev->upload_live.find(ptr);
    if (it != dev->upload_live.end() && cap != cudaStreamCaptureStatusNone) {
      dev->upload_live.erase(it);
      it = dev->upload_live.end();
    }
    if (it != dev->upload_live.end()) {
      const size_t bytes = it->second;
      dev->upload_live.erase(it);
      cudaEvent_t ev = nullptr;
      if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess &&
          cudaEventRecord(ev, dev->stream) == cudaSuccess) {
        if (dev->upload_free.size() >= kUploadCacheBlocks) {
          // the oldest cached buffer goes back to its pool, after its last use
          VKC_CUDA(cudaStreamWaitEvent(dev->stream, dev->upload_free.front().freed, 0));
          VKC_CUDA(cudaFreeAsync(dev->upload_free.front().ptr, dev->stream));
          cudaEventDestroy(dev->upload_free.front().freed);
          dev->upload_free.erase(dev->upload_free.begin());
        }
        dev->upload_free.push_back({ptr, bytes, ev});
        return VKC_OK;
      }
      if (ev) cudaEventDestroy(ev);
      cudaGetLastError();
    }
  }
  VKC_CUDA(cudaFreeAsync(ptr, dev->stream));
  return VKC_OK;
}

VKC_EXPORT int vkc_host_alloc(size_t bytes, void** ptr) {
  VKC_REQUIRE(ptr, "ptr is NULL");
  *ptr = nullptr;
  if (bytes == 0) return VKC_OK;
  if (vkc::alloc_should_fail())
    return set_error(VKC_ERR_OOM, "cudaHostAlloc(%zu bytes): injected allocation failure", bytes);
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocPortable);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return set_error(VKC_ERR_OOM, "cudaHostAlloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  return VKC_OK;
}

VKC_EXPORT int vkc_host_free(void* ptr) {
  if (!ptr) return VKC_OK;
  VKC_CUDA(cudaFreeHost(ptr));
  return VKC_OK;
}


VKC_EXPORT int vkc_upload(vkc_device_t dev, const void* src, size_t bytes, void** dptr) {
  VKC_BIND(dev);
  VKC_REQUIRE(dptr && (src || bytes == 0), "NULL argument");
  *dptr = nullptr;
  if (bytes == 0) return VKC_OK;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  VKC_CUDA(cudaStreamIsCapturing(dev->stream, &cap));
  VKC_REQUIRE(cap == cudaStreamCaptureStatusNone, "host uploads are not allowed while the stream is captured");
  std::lock_guard<std::mutex> lk(dev->mu);
  // Allocate and copy on the copy stream so that the upload does not queue
  // behind compute work; the compute stream then waits for the copy.
  const int r = upload_take(dev, bytes, dptr);
  if (r != VKC_OK) return r;
  VKC_CUDA(cudaMemcpyAsync(*dptr, src, bytes, cudaMemcpyHostToDevice, dev->copy_stream));
  VKC_CUDA(cudaEventRecord(dev->copy_done, dev->copy_stream));
  VKC_CUDA(cudaStreamWaitEvent(dev->stream, dev->copy_done, 0));
  VKC_CUDA(cudaEventSynchronize(dev->copy_done));
  return VKC_OK;
}

namespace {
// A job marking everything issued so far on `stream`.
int record_on(vkc_device_t dev, cudaStream_t stream, vkc_job_t* job) {
  auto* j = new vkc_job();
  j->device = dev->index;
  cudaError_t e = cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(j->ev, stream);
  if (e != cudaSuccess) {
    if (j->ev) cudaEventDestroy(j->ev);
    delete j;
    *job = nullptr;
    return set_error(VKC_ERR_CUDA, "job record: %s", cudaGetErrorString(e));
  }
  *job = j;
  return VKC_OK;
}
}  // namespace

VKC_EXPORT int vkc_upload_async(vkc_device_t dev, const void* src, size_t bytes, void** dptr, vkc_job_t* job) {
  VKC_BIND(dev);
  VKC_REQUIRE(dptr && job && (src || bytes == 0), "NULL argument");
  *dptr = nullptr;
  *job = nullptr;
  if (bytes == 0) return VKC_OK;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  VKC_CUDA(cudaStreamIsCapturing(dev->stream, &cap));
  VKC_REQUIRE(cap == cudaStreamCaptureStatusNone, "host uploads are not allowed while the stream is captured");
  std::lock_guard<std::mutex> lk(dev->mu);
  const int r = upload_take(dev, bytes, dptr);
  if (r != VKC_OK) return r;
  VKC_CUDA(cudaMemcpyAsync(*dptr, src, bytes, cudaMemcpyHostToDevice, dev->copy_stream));
  VKC_CUDA(cudaEventRecord(dev->copy_done, dev->copy_stream));
  VKC_CUDA(cudaStreamWaitEvent(dev->stream, dev->copy_done, 0));
  return record_on(dev, dev->copy_stream, job);
}

VKC_EXPORT int vkc_d2h_async(vkc_device_t dev, void* dst, const void* src, size_t bytes, vkc_job_t* job) {
  VKC_BIND(dev);
  VKC_REQUIRE(job, "job is NULL");
  *job = nullptr;
  VKC_REQUIRE(dst && (src || bytes == 0), "NULL argument");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  VKC_CUDA(cudaStreamIsCapturing(dev->stream, &cap));
  VKC_REQUIRE(cap == cudaStreamCaptureStatusNone, "host read-backs are not allowed while the stream is captured");
  std::lock_guard<std::mutex> lk(dev->mu);
  // after everything issued on the compute stream so far, not after what
  // is issued later
  VKC_CUDA(cudaEventRecord(dev->d2h_after, dev->stream));
  VKC_CUDA(cudaStreamWaitEvent(dev->d2h_stream, dev->d2h_after, 0));
  if (bytes) VKC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, dev->d2h_stream));
  return record_on(dev, dev->d2h_stream, job);
}

VKC_EXPORT int vkc_stream_wait_job(vkc_device_t dev, vkc_job_t job) {
  VKC_BIND(dev);
  VKC_REQUIRE(job, "job is NULL");
  VKC_CUDA(cudaStreamWaitEvent(dev->stream, job->ev, 0));
  return VKC_OK;
}

VKC_EXPORT int vkc_h2d(vkc_device_t dev, void* dst, const void* src, size_t bytes, vkc_job_t* job) {
  VKC_BIND(dev);
  if (job) *job = nullptr;
  if (bytes == 0) return VKC_OK;
  VKC_REQUIRE(dst && src, "NULL argument");
  // A pageable source is staged before cudaMemcpyAsync returns; a pinned
  // one is read when the stream reaches the copy, which `job` marks.
  VKC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, dev->stream));
  if (job) return vkc_job_record(dev, job);
  return VKC_OK;
}

VKC_EXPORT int vkc_d2h(vkc_device_t dev, void* dst, const void* src, size_t bytes) {
  VKC_BIND(dev);
  if (bytes == 0) return VKC_OK;
  VKC_REQUIRE(dst && src, "NULL argument");
  VKC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, dev->stream));
  VKC_CUDA(cudaStreamSynchronize(dev->stream));
  return VKC_OK;
}

VKC_EXPORT int vkc_copy(vkc_device_t dev, void* dst, const void* src, size_t bytes) {
  VKC_BIND(dev);
  if (bytes == 0) return VKC_OK;
  VKC_REQUIRE(dst && src, "NULL argument");
  VKC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, dev->stream));
  return VKC_OK;
}

// ---- jobs -------------------------------------------------------------------

VKC_EXPORT int vkc_job_record(vkc_device_t dev, vkc_job_t* job) {
  VKC_BIND(dev);
  VKC_REQUIRE(job, "job is NULL");
  auto* j = new vkc_job();
  j->device = dev->index;
  cudaError_t e = cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(j->ev, dev->stream);
  if (e != cudaSuccess) {
    if (j->ev) cudaEventDestroy(j->ev);
    delete j;
    *job = nullptr;
    return set_error(VKC_ERR_CUDA, "job record: %s", cudaGetErrorString(e));
  }
  *job = j;
  return VKC_OK;
}

VKC_EXPORT int vkc_job_wait(vkc_job_t job, int64_t timeout_ns) {
  if (!job) return VKC_OK;
  if (timeout_ns < 0) {
    cudaError_t e = cudaEventSynchronize(job->ev);
    if (e != cudaSuccess) return set_error(VKC_ERR_CUDA, "Error at Command Wait: %s", cudaGetErrorString(e));
    return VKC_OK;
  }
  // Poll against a host deadline; the GPU keeps running, nothing is aborted.
  auto deadline = std::chrono::steady_clock::now() + std::chrono::nanoseconds(timeout_ns);
  for (;;) {
    cudaError_t e = cudaEventQuery(job->ev);
    if (e == cudaSuccess) return VKC_OK;
    if (e != cudaErrorNotReady) return set_error(VKC_ERR_CUDA, "Error at Command Wait: %s", cudaGetErrorString(e));
    if (std::chrono::steady_clock::now() >= deadline) {
      cudaGetLastError();
      return set_error(VKC_ERR_TIMEOUT, "Timeout at Command Wait");
    }
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

VKC_EXPORT int vkc_job_query(vkc_job_t job, int* done) {
  VKC_REQUIRE(done, "done is NULL");
  if (!job) { *done = 1; return VKC_OK; }
  cudaError_t e = cudaEventQuery(job->ev);
  if (e == cudaSuccess) { *done = 1; return VKC_OK; }
  if (e == cudaErrorNotReady) { cudaGetLastError(); *done = 0; return VKC_OK; }
  return set_error(VKC_ERR_CUDA, "Error at Command Wait: %s", cudaGetErrorString(e));
}

VKC_EXPORT int vkc_timer_record(vkc_device_t dev, vkc_job_t* job) {
  VKC_BIND(dev);
  VKC_REQUIRE(job, "job is NULL");
  auto* j = new vkc_job();
  j->device = dev->index;
  cudaError_t e = cudaEventCreate(&j->ev);
  if (e == cudaSuccess) e = cudaEventRecord(j->ev, dev->stream);
  if (e != cudaSuccess) {
    if (j->ev) cudaEventDestroy(j->ev);
    delete j;
    *job = nullptr;
    return set_error(VKC_ERR_CUDA, "timer record: %s", cudaGetErrorString(e));
  }
  *job = j;
  return VKC_OK;
}

VKC_EXPORT int vkc_job_elapsed_ms(vkc_job_t start, vkc_job_t end, float* ms) {
  VKC_REQUIRE(start && end && ms, "NULL argument");
  VKC_CUDA(cudaEventSynchronize(end->ev));
  VKC_CUDA(cudaEventElapsedTime(ms, start->ev, end->ev));
  return VKC_OK;
}

VKC_EXPORT int vkc_launch_count(uint64_t* count) {
  VKC_REQUIRE(count, "count is NULL");
  *count = vkc::g_launches.load(std::memory_order_relaxed);
  return VKC_OK;
}

VKC_EXPORT int vkc_set_pdl(int enable) {
  vkc::g_pdl.store(enable ? 1 : 0, std::memory_order_relaxed);
  return VKC_OK;
}

VKC_EXPORT int vkc_side_defer(vkc_device_t dev, int defer) {
  VKC_BIND(dev);
  if (defer) {
    dev->side_defer = 1;
    return VKC_OK;
  }
  dev->side_defer = 0;
  if (!dev->side_pending) return VKC_OK;
  dev->side_pending = 0;
  VKC_CUDA(cudaEventRecord(dev->side_join, dev->side_stream));
  VKC_CUDA(cudaEventRecord(dev->bias_join, dev->bias_stream));
  VKC_CUDA(cudaStreamWaitEvent(dev->stream, dev->side_join, 0));
  VKC_CUDA(cudaStreamWaitEvent(dev->stream, dev->bias_join, 0));
  return VKC_OK;
}

VKC_EXPORT int vkc_side_begin(vkc_device_t dev) {
  VKC_BIND(dev);
  VKC_REQUIRE(dev->stream == dev->own_stream, "branch: not on the device's own stream");
  VKC_CUDA(cudaEventRecord(dev->side_fork, dev->stream));
  VKC_CUDA(cudaStreamWaitEvent(dev->side_stream, dev->side_fork, 0));
  VKC_CUDA(cudaEventRecord(dev->bias_join, dev->bias_stream));
  VKC_CUDA(cudaStreamWaitEvent(dev->side_stream, dev->bias_join, 0));
  dev->stream = dev->side_stream;
  dev->side_pending = 1;
  return VKC_OK;
}

VKC_EXPORT int vkc_side_end(vkc_device_t dev) {
  VKC_BIND(dev);
  VKC_REQUIRE(dev->stream == dev->side_stream, "branch: vkc_side_end without vkc_side_begin");
  dev->stream = dev->own_stream;
  if (!dev->side_defer) return vkc_side_defer(dev, 0);
  return VKC_OK;
}

VKC_EXPORT int vkc_set_cluster_splitk(int enable) {
  vkc::g_cluster_splitk.store(enable ? 1 : 0, std::memory_order_relaxed);
  return VKC_OK;
}

VKC_EXPORT int vkc_pool_reserved(vkc_device_t dev, uint64_t* compute_bytes, uint64_t* upload_bytes) {
  VKC_BIND(dev);
  VKC_REQUIRE(compute_bytes && upload_bytes, "NULL argument");
  *compute_bytes = 0;
  *upload_bytes = 0;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev->index) == cudaSuccess)
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, compute_bytes);
  if (dev->upload_pool) cudaMemPoolGetAttribute(dev->upload_pool, cudaMemPoolAttrReservedMemCurrent, upload_bytes);
  cudaGetLastError();
  return VKC_OK;
}

VKC_EXPORT int vkc_alloc_count(uint64_t* count) {
  VKC_REQUIRE(count, "count is NULL");
  *count = vkc::g_allocs.load(std::memory_order_relaxed);
  return VKC_OK;
}

VKC_EXPORT int vkc_inject_alloc_failure(int64_t after) {
  vkc::g_fail_alloc_in.store(after < 0 ? -1 : after, std::memory_order_relaxed);
  return VKC_OK;
}

VKC_EXPORT int vkc_job_destroy(vkc_job_t job) {
  if (!job) return VKC_OK;
  cudaEventDestroy(job->ev);
  delete job;
  return VKC_OK;
}

// ---- CUDA graphs --------------------------------------------------------------

struct vkc_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  vkc_device_t dev = nullptr;
};

VKC_EXPORT int vkc_stream_create(vkc_device_t dev, void** stream) {
  VKC_BIND(dev);
  VKC_REQUIRE(stream, "stream is NULL");
  cudaStream_t s = nullptr;
  VKC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *stream = (void*)s;
  return VKC_OK;
}

VKC_EXPORT int vkc_stream_destroy(vkc_device_t dev, void* stream) {
  if (!stream) return VKC_OK;
  VKC_BIND(dev);
  VKC_CUDA(cudaStreamDestroy((cudaStream_t)stream));
  return VKC_OK;
}

VKC_EXPORT int vkc_stream_wait(vkc_device_t dev, void* waiter, void* signaler) {
  VKC_BIND(dev);
  cudaStream_t w = waiter ? (cudaStream_t)waiter : dev->own_stream;
  cudaStream_t s = signaler ? (cudaStream_t)signaler : dev->own_stream;
  cudaEvent_t ev;
  VKC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(w, ev, 0);
  cudaEventDestroy(ev);  // released once the wait has been recorded
  if (e != cudaSuccess) return set_error(VKC_ERR_CUDA, "stream wait: %s", cudaGetErrorString(e));
  return VKC_OK;
}

VKC_EXPORT int vkc_graph_begin(vkc_device_t dev) {
  VKC_BIND(dev);
  VKC_CUDA(cudaStreamBeginCapture(dev->stream, cudaStreamCaptureModeThreadLocal));
  return VKC_OK;
}

VKC_EXPORT int vkc_graph_end(vkc_device_t dev, vkc_graph_t* out) {
  VKC_BIND(dev);
  VKC_REQUIRE(out, "graph is NULL");
  *out = nullptr;
  cudaGraph_t g = nullptr;
  VKC_CUDA(cudaStreamEndCapture(dev->stream, &g));
  cudaGraphExec_t exec = nullptr;
  // Allocations left live by the captured work are freed and re-made (same
  // virtual address) at the next launch instead of blocking relaunch.
  cudaError_t e = cudaGraphInstantiateWithFlags(&exec, g, cudaGraphInstantiateFlagAutoFreeOnLaunch);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return set_error(VKC_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  }
  auto* gr = new vkc_graph();
  gr->graph = g;
  gr->exec = exec;
  gr->dev = dev;
  *out = gr;
  return VKC_OK;
}

VKC_EXPORT int vkc_graph_launch(vkc_graph_t g) {
  VKC_REQUIRE(g, "graph is NULL");
  VKC_BIND(g->dev);
  VKC_CUDA(cudaGraphLaunch(g->exec, g->dev->stream));
  return VKC_OK;
}

VKC_EXPORT int vkc_graph_destroy(vkc_graph_t g) {
  if (!g) return VKC_OK;
  VKC_BIND(g->dev);
  // The synchronisation below would invalidate a capture in progress on the
  // stream; refuse instead (the caller destroys the graph after the capture).
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  VKC_CUDA(cudaStreamIsCapturing(g->dev->stream, &cs));
  VKC_REQUIRE(cs == cudaStreamCaptureStatusNone, "cannot destroy a graph while a capture is active on its stream");
  cudaStreamSynchronize(g->dev->stream);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return VKC_OK;
}
