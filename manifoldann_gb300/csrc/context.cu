// context.cu -- error reporting and per-device contexts.
#include <atomic>
#include <memory>

#include "context.cuh"

namespace mann {

namespace {
thread_local std::string g_last_error;
thread_local int64_t g_launches = 0;
std::mutex g_ctx_mu;
std::unique_ptr<Context> g_ctx[64];
// host-side fault injection (mann_debug_inject): pending failures per kind
std::atomic<int> g_inject_alloc{0};
std::atomic<int> g_inject_launch{0};
std::atomic<int> g_inject_queue{0};

// true once for each pending injected failure of `counter`
bool take_injected(std::atomic<int>& counter) {
  int c = counter.load();
  while (c > 0)
    if (counter.compare_exchange_weak(c, c - 1)) return true;
  return false;
}
}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
void note_launch() { ++g_launches; }
bool injected_launch_error() { return take_injected(g_inject_launch); }
bool injected_dropped_publish() { return take_injected(g_inject_queue); }
int64_t launch_count() { return g_launches; }
const char* last_error_cstr() { return g_last_error.c_str(); }

mann_status Context::scratch(int slot, size_t bytes, void** out) {
  if (bytes == 0) bytes = 256;
  if (take_injected(g_inject_alloc))
    return fail(MANN_ENOMEM, "cudaMalloc of " + std::to_string(bytes) +
                                 " bytes of scratch failed (out of memory, injected by mann_debug_inject)");
  if (slot_bytes[slot] < bytes) {
    if (slot_ptr[slot]) {
      MANN_CUDA_TRY(cudaFree(slot_ptr[slot]));
      slot_ptr[slot] = nullptr;
      slot_bytes[slot] = 0;
    }
    // round up to 2 MiB to limit regrowth
    const size_t want = (bytes + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(MANN_ENOMEM, "cudaMalloc of " + std::to_string(want) + " bytes failed (" +
                                   cudaGetErrorString(e) + ")");
    }
    slot_ptr[slot] = p;
    slot_bytes[slot] = want;
  }
  *out = slot_ptr[slot];
  return MANN_OK;
}

void Context::release_points(const void* owner) {
  auto it = points_cache.find(owner);
  if (it == points_cache.end()) return;
  if (it->second.rows) (void)cudaFree(it->second.rows);
  if (it->second.misc) (void)cudaFree(it->second.misc);
  points_cache.erase(it);
}

mann_status get_context(Context** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(MANN_ENODEV, std::string("no CUDA device: ") + cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= 64) return fail(MANN_ENODEV, "device ordinal out of range");
  std::lock_guard<std::mutex> g(g_ctx_mu);
  if (!g_ctx[dev]) {
    std::unique_ptr<Context> c(new Context());
    c->device = dev;
    cudaDeviceProp prop;
    MANN_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    c->num_sms = prop.multiProcessorCount;
    c->cc_major = prop.major;
    c->cc_minor = prop.minor;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    if (c->cc_major != 10)
      return fail(MANN_ENODEV, "libmanngpu is built for sm_103a (GB300); device " +
                                   std::to_string(dev) + " is sm_" + std::to_string(prop.major) +
                                   std::to_string(prop.minor));
    MANN_CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    MANN_CUDA_TRY(cudaEventCreateWithFlags(&c->last_use, cudaEventDisableTiming));
    MANN_CUDA_TRY(cudaEventCreate(&c->time_a));
    MANN_CUDA_TRY(cudaEventCreate(&c->time_b));
    g_ctx[dev] = std::move(c);
  }
  *out = g_ctx[dev].get();
  return MANN_OK;
}

void Context::time_begin(cudaStream_t s) {
  if (timing && !timed) cudaEventRecord(time_a, s);
}

void Context::time_end(cudaStream_t s) {
  if (timing && !timed) {
    cudaEventRecord(time_b, s);
    timed = true;
  }
}

CallScope::CallScope(Context* ctx, cudaStream_t s) : ctx_(ctx), s_(s), lock_(ctx->mu) {
  // scratch written by the previous call (possibly on another stream) must be
  // free before this call's kernels touch it
  cudaStreamWaitEvent(s_, ctx_->last_use, 0);
}

CallScope::~CallScope() { cudaEventRecord(ctx_->last_use, s_); }

}  // namespace mann

extern "C" mann_status mann_debug_inject(int32_t kind, int32_t count) {
  mann::clear_error();
  if (count < 0) return mann::fail(MANN_EINVAL_ARG, "count must be >= 0");
  if (kind == MANN_INJECT_ALLOC) {
    mann::g_inject_alloc.store(count);
  } else if (kind == MANN_INJECT_LAUNCH) {
    mann::g_inject_launch.store(count);
  } else if (kind == MANN_INJECT_QUEUE) {
    mann::g_inject_queue.store(count);
  } else {
    return mann::fail(MANN_EINVAL_ARG, "unknown injection kind");
  }
  return MANN_OK;
}
