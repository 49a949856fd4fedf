// util.cu -- error state, device / stream management, small host helpers.
#include <atomic>
#include <chrono>
#include <cstdarg>
#include <mutex>

#include "common.cuh"

namespace dg {

namespace {
thread_local char g_err[1024] = {0};
std::atomic<long> g_launches{0};
}

void count_launch(long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

const char *last_error() { return g_err; }

void require_device() {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    set_error("no CUDA device available (%s)", e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
    throw Error{DG_ERR_NODEVICE};
  }
}

cudaStream_t stream() {
  thread_local cudaStream_t s = nullptr;
  thread_local int dev = -1;
  int cur = 0;
  DG_CUDA(cudaGetDevice(&cur));
  if (!s || dev != cur) {
    DG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    dev = cur;
  }
  return s;
}

// ---- device memory pool ---------------------------------------------------------------
namespace {
constexpr int kMaxPoolDevices = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[kMaxPoolDevices] = {nullptr};

uint64_t pool_keep_bytes() {
  const char *s = getenv("DG_POOL_KEEP_MB");
  if (s && *s) return (uint64_t)strtoull(s, nullptr, 10) << 20;
  return 8ull << 30;
}
}  // namespace

cudaMemPool_t device_pool() {
  int dev = 0;
  DG_CUDA(cudaGetDevice(&dev));
  DG_REQUIRE(dev >= 0 && dev < kMaxPoolDevices, DG_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  if (!g_pools[dev]) {
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    DG_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = pool_keep_bytes();
    DG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pools[dev] = pool;
  }
  return g_pools[dev];
}

// Pool holds: while any is active on a device, its pool keeps all the memory it has mapped
// across synchronisations (release threshold unbounded), so that allocations of a batch or an
// engine whose working set exceeds the default keep do not unmap and map physical memory each
// time another thread synchronises.  The last hold restores the keep and trims to it.
namespace {
int g_pool_holds[kMaxPoolDevices] = {0};
}
void pool_hold(int device, bool acquire) {
  if (device < 0 || device >= kMaxPoolDevices) return;
  int prev = 0;
  DG_CUDA(cudaGetDevice(&prev));
  DG_CUDA(cudaSetDevice(device));
  cudaMemPool_t pool = device_pool();
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  int &h = g_pool_holds[device];
  if (acquire) {
    if (h++ == 0) {
      uint64_t all = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &all);
    }
  } else if (h > 0 && --h == 0) {
    uint64_t keep = pool_keep_bytes();
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    cudaMemPoolTrimTo(pool, keep);
  }
  cudaSetDevice(prev);
}

void *pool_alloc(size_t bytes, cudaStream_t st) {
  void *p = nullptr;
  DG_CUDA(cudaMallocFromPoolAsync(&p, bytes ? bytes : 1, device_pool(), st));
  return p;
}

void pool_free(void *p, cudaStream_t st) {
  if (p) cudaFreeAsync(p, st);
}

// ---- mapped host blocks ------------------------------------------------------------------
namespace {
struct MappedBlock {
  void *h;
  size_t bytes;
};
struct MappedCache {
  std::vector<MappedBlock> free_blocks;
  ~MappedCache() {
    for (auto &b : free_blocks) cudaFreeHost(b.h);
  }
};
thread_local MappedCache g_mapped_cache;
}  // namespace

void *mapped_acquire(size_t bytes, size_t *got) {
  size_t want = 4096;
  while (want < bytes) want <<= 1;
  auto &fb = g_mapped_cache.free_blocks;
  for (size_t i = 0; i < fb.size(); ++i) {
    if (fb[i].bytes >= want) {
      MappedBlock b = fb[i];
      fb.erase(fb.begin() + (long)i);
      *got = b.bytes;
      return b.h;
    }
  }
  void *h = nullptr;
  DG_CUDA(cudaHostAlloc(&h, want, cudaHostAllocMapped));
  *got = want;
  return h;
}

void mapped_return(void *h, size_t bytes) {
  if (!h) return;
  auto &fb = g_mapped_cache.free_blocks;
  if (fb.size() >= 16) {
    cudaFreeHost(h);
    return;
  }
  fb.push_back(MappedBlock{h, bytes});
}

int sm_count() {
  thread_local int cached = -1, dev = -1;
  int cur = 0;
  DG_CUDA(cudaGetDevice(&cur));
  if (cached < 0 || dev != cur) {
    DG_CUDA(cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, cur));
    dev = cur;
  }
  return cached;
}

int vector_grid(long n) {
  long need = (n + kThreads - 1) / kThreads;
  long cap = (long)sm_count() * 4;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool is_device_only_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice;
}

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

}  // namespace dg

extern "C" {

const char *dg_last_error(void) { return dg::last_error(); }

int dg_device_count(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return count;
}

const char *dg_version(void) { return "dmrg_gb300 0.1 (sm_103a)"; }

long dg_kernel_launches(void) { return dg::g_launches.load(); }

int dg_release_pool(void) {
  return dg::guarded([&] {
    dg::require_device();
    DG_CUDA(cudaStreamSynchronize(dg::stream()));
    DG_CUDA(cudaMemPoolTrimTo(dg::device_pool(), 0));
  });
}

}  // extern "C"
