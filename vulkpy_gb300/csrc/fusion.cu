// Run-time compiled elementwise kernels (chains of array ops fused into one
// pass over memory).  The host generates CUDA C for a traced chain; this
// file compiles it with NVRTC for sm_103a, loads the cubin as a CUDA library
// and launches it.  NVRTC is loaded with dlopen on first use, so the library
// has no link-time dependency on it.  Compiled kernels are cached by source.
#include "common.cuh"

#include <dlfcn.h>

#include <string>
#include <unordered_map>
#include <vector>

namespace {

// NVRTC entry points (C API, resolved at run time).
typedef int (*nvrtcCreateProgram_t)(void**, const char*, const char*, int, const char* const*, const char* const*);
typedef int (*nvrtcCompileProgram_t)(void*, int, const char* const*);
typedef int (*nvrtcGetSize_t)(void*, size_t*);
typedef int (*nvrtcGetBuf_t)(void*, char*);
typedef int (*nvrtcDestroyProgram_t)(void**);

struct Nvrtc {
  void* handle = nullptr;
  nvrtcCreateProgram_t create = nullptr;
  nvrtcCompileProgram_t compile = nullptr;
  nvrtcGetSize_t cubin_size = nullptr, log_size = nullptr;
  nvrtcGetBuf_t cubin = nullptr, log = nullptr;
  nvrtcDestroyProgram_t destroy = nullptr;
  bool ok = false;
};

Nvrtc& nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* names[] = {"libnvrtc.so.13", "libnvrtc.so.12", "libnvrtc.so",
                           "/usr/local/cuda/lib64/libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so"};
    for (const char* nm : names) {
      n.handle = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
      if (n.handle) break;
    }
    if (!n.handle) return;
    n.create = (nvrtcCreateProgram_t)dlsym(n.handle, "nvrtcCreateProgram");
    n.compile = (nvrtcCompileProgram_t)dlsym(n.handle, "nvrtcCompileProgram");
    n.cubin_size = (nvrtcGetSize_t)dlsym(n.handle, "nvrtcGetCUBINSize");
    n.cubin = (nvrtcGetBuf_t)dlsym(n.handle, "nvrtcGetCUBIN");
    n.log_size = (nvrtcGetSize_t)dlsym(n.handle, "nvrtcGetProgramLogSize");
    n.log = (nvrtcGetBuf_t)dlsym(n.handle, "nvrtcGetProgramLog");
    n.destroy = (nvrtcDestroyProgram_t)dlsym(n.handle, "nvrtcDestroyProgram");
    n.ok = n.create && n.compile && n.cubin_size && n.cubin && n.log_size && n.log && n.destroy;
  });
  return n;
}

struct JitKernel {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
};

std::mutex g_jit_mu;
std::unordered_map<std::string, JitKernel*> g_jit_cache;  // key: device + source

constexpr int kMaxIn = 8, kMaxOut = 4;
struct JitParams {
  const float* in[kMaxIn];
  float* out[kMaxOut];
  unsigned long long n;
};

}  // namespace

typedef struct vkc_kernel* vkc_kernel_t;

VKC_EXPORT int vkc_jit_compile(vkc_device_t dev, const char* source, const char* name, vkc_kernel_t* out) {
  VKC_BIND(dev);
  VKC_REQUIRE(source && name && out, "NULL argument");
  *out = nullptr;
  std::string key = std::to_string(dev->index) + "\n" + name + "\n" + source;
  {
    std::lock_guard<std::mutex> lk(g_jit_mu);
    auto it = g_jit_cache.find(key);
    if (it != g_jit_cache.end()) {
      *out = reinterpret_cast<vkc_kernel_t>(it->second);
      return VKC_OK;
    }
  }
  Nvrtc& nv = nvrtc();
  VKC_REQUIRE(nv.ok, "NVRTC (libnvrtc) is not available: fused kernels cannot be compiled");
  void* prog = nullptr;
  if (nv.create(&prog, source, "vkc_fused.cu", 0, nullptr, nullptr) != 0)
    return vkc::set_error(VKC_ERR_CUDA, "nvrtcCreateProgram failed");
  char arch[64];
  std::snprintf(arch, sizeof(arch), "-arch=sm_%d%da", dev->cc_major, dev->cc_minor);
  // -fmad=false: each traced op rounds on its own, as in the one-op kernels.
  const char* opts[] = {arch, "-fmad=false", "-std=c++17", "-default-device"};
  int rc = nv.compile(prog, 4, opts);
  if (rc != 0) {
    size_t n = 0;
    nv.log_size(prog, &n);
    std::string log(n, '\0');
    if (n) nv.log(prog, &log[0]);
    nv.destroy(&prog);
    return vkc::set_error(VKC_ERR_INVALID, "fused kernel compilation failed: %s", log.c_str());
  }
  size_t sz = 0;
  nv.cubin_size(prog, &sz);
  std::vector<char> cubin(sz);
  nv.cubin(prog, cubin.data());
  nv.destroy(&prog);
  auto* k = new JitKernel();
  cudaError_t e = cudaLibraryLoadData(&k->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&k->kernel, k->lib, name);
  if (e != cudaSuccess) {
    if (k->lib) cudaLibraryUnload(k->lib);
    delete k;
    return vkc::set_error(VKC_ERR_CUDA, "loading fused kernel: %s", cudaGetErrorString(e));
  }
  std::lock_guard<std::mutex> lk(g_jit_mu);
  auto ins = g_jit_cache.emplace(key, k);
  if (!ins.second) {  // another thread won the race
    cudaLibraryUnload(k->lib);
    delete k;
  }
  *out = reinterpret_cast<vkc_kernel_t>(ins.first->second);
  return VKC_OK;
}

VKC_EXPORT int vkc_jit_launch(vkc_device_t dev, vkc_kernel_t kernel, const float* const* in, int n_in,
                              float* const* out, int n_out, size_t n) {
  VKC_BIND(dev);
  VKC_REQUIRE(kernel, "kernel is NULL");
  VKC_REQUIRE(n_in >= 0 && n_in <= kMaxIn && n_out >= 1 && n_out <= kMaxOut, "too many fused operands");
  if (n == 0) return VKC_OK;
  JitParams p{};
  for (int i = 0; i < n_in; ++i) {
    VKC_REQUIRE(in[i] && ((uintptr_t)in[i] & 15u) == 0, "fused input %d must be a 16-byte aligned device pointer", i);
    p.in[i] = in[i];
  }
  for (int i = 0; i < n_out; ++i) {
    VKC_REQUIRE(out[i] && ((uintptr_t)out[i] & 15u) == 0, "fused output %d must be 16-byte aligned", i);
    p.out[i] = out[i];
  }
  p.n = n;
  auto* k = reinterpret_cast<JitKernel*>(kernel);
  unsigned grid = vkc::stream_grid(dev, (n >> 2) + 1, 256);
  void* args[] = {&p};
  cudaError_t e = cudaLaunchKernel((const void*)k->kernel, dim3(grid), dim3(256), args, 0, dev->stream);
  if (e != cudaSuccess) return vkc::set_error(VKC_ERR_CUDA, "fused kernel launch: %s", cudaGetErrorString(e));
  return vkc::check_launch("fused");
}
