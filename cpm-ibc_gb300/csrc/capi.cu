// Library-wide state of the C-ABI: per-thread error strings, the library
// stream, device queries.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>

#include "cpm_internal.h"

namespace cpm {

static thread_local std::string g_error;

void set_error(const std::string &msg) { g_error = msg; }

int fail(int code, const std::string &msg) {
    g_error = msg;
    return code;
}

// One non-blocking stream per process: the library's work is ordered on it and
// never synchronises the legacy default stream.
cudaStream_t library_stream() {
    static std::once_flag once;
    static cudaStream_t s = nullptr;
    std::call_once(once, [] { cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking); });
    return s;
}

// the stream of the calling thread's current StreamScope, if any
static thread_local cudaStream_t g_scope = nullptr;

cudaStream_t stream() { return g_scope ? g_scope : library_stream(); }

StreamScope::StreamScope(cudaStream_t s) : prev(g_scope) { g_scope = s; }
StreamScope::~StreamScope() { g_scope = prev; }

}  // namespace cpm

extern "C" const char *cpm_last_error(void) { return cpm::g_error.c_str(); }

extern "C" int cpm_set_device(int32_t device) {
    CPM_CUDA_TRY(cudaSetDevice(device));
    return 0;
}

extern "C" int cpm_device_info(char *name, int64_t name_len, int64_t *free_bytes, int64_t *total_bytes, int32_t *sm_count) {
    int dev = 0;
    CPM_CUDA_TRY(cudaGetDevice(&dev));
    cudaDeviceProp p;
    CPM_CUDA_TRY(cudaGetDeviceProperties(&p, dev));
    if (name && name_len > 0) {
        strncpy(name, p.name, (size_t)name_len - 1);
        name[name_len - 1] = 0;
    }
    size_t fr = 0, to = 0;
    CPM_CUDA_TRY(cudaMemGetInfo(&fr, &to));
    if (free_bytes) *free_bytes = (int64_t)fr;
    if (total_bytes) *total_bytes = (int64_t)to;
    if (sm_count) *sm_count = p.multiProcessorCount;
    return 0;
}

extern "C" int cpm_sync(void) {
    CPM_CUDA_TRY(cudaStreamSynchronize(cpm::stream()));
    return 0;
}

extern "C" void *cpm_get_stream(void) { return (void *)cpm::stream(); }

extern "C" int cpm_set_thread_stream(void *s) {
    cpm::g_scope = (cudaStream_t)s;
    return 0;
}

namespace cpm {
static std::atomic<long long> g_launches{0};
void count_launches(long long n) { g_launches += n; }
}  // namespace cpm

extern "C" int64_t cpm_launch_count(void) { return (int64_t)cpm::g_launches.load(); }
