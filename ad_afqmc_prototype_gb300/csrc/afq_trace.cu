// Tracing: a launch counter and optional per-phase device timing.
//
// Timing is a process-wide profiling switch, off by default and not meant
// for concurrent callers: when on, every AFQ_PHASE scope records a CUDA event
// pair on its stream; afq_timing_report() waits for the recorded events and
// accumulates (calls, total ms) per phase name.  Events come from a pool, so
// a report in every iteration does not grow host memory.
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "afq_internal.cuh"

namespace afq {

namespace {
std::atomic<long long> g_launches{0};
bool g_timing = false;
std::mutex g_mu;
struct Rec {
    const char* name;
    cudaEvent_t a, b;
};
std::vector<Rec> g_pending;
std::vector<cudaEvent_t> g_pool;
std::map<std::string, std::pair<long long, double>> g_acc;

cudaEvent_t take_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}
}  // namespace

bool timing_enabled() { return g_timing; }

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ------------------------------------------------ per-device launch facts --
namespace {
std::recursive_mutex g_dev_mu;
int g_dev_sms[kMaxDevices] = {};
}  // namespace

int current_device(int* dev) {
    int d = -1;
    AFQ_CUDA(cudaGetDevice(&d));
    if (d < 0 || d >= kMaxDevices) return fail(AFQ_E_UNSUPPORTED, "device ordinal %d out of range", d);
    *dev = d;
    return AFQ_OK;
}

int device_sms(int* sms) {
    int dev = 0;
    AFQ_TRY(current_device(&dev));
    std::lock_guard<std::recursive_mutex> lk(g_dev_mu);
    if (!g_dev_sms[dev]) {
        int v = 0;
        AFQ_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
        if (v < 1) return fail(AFQ_E_CUDA, "device %d reports %d SMs", dev, v);
        g_dev_sms[dev] = v;
    }
    *sms = g_dev_sms[dev];
    return AFQ_OK;
}

int device_once_run(DeviceOnce& once, int (*fn)(void*), void* arg) {
    int dev = 0;
    AFQ_TRY(current_device(&dev));
    std::lock_guard<std::recursive_mutex> lk(g_dev_mu);
    if (once.done[dev]) return AFQ_OK;
    AFQ_TRY(fn(arg));
    once.done[dev] = true;
    return AFQ_OK;
}

Phase::Phase(const char* n, cudaStream_t s) : name(n), stream(s), start(nullptr) {
    if (!g_timing) return;
    std::lock_guard<std::mutex> lk(g_mu);
    start = take_event();
    if (start) cudaEventRecord(start, stream);
}

Phase::~Phase() {
    if (!start) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t end = take_event();
    if (!end) return;
    cudaEventRecord(end, stream);
    g_pending.push_back({name, start, end});
}

// Eight independent FMA chains per thread: the issue-rate ceiling of the
// SIMT FMA pipe for T (the roofline of the binary64 kernels).
template <class T>
__global__ void k_fma_probe(T* out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <class T>
static int probe(int iters, double* tflops) {
    int dev = 0, sms = 0;
    AFQ_CUDA(cudaGetDevice(&dev));
    AFQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    AFQ_CUDA(cudaMalloc(&out, sizeof(T) * (size_t)blocks * threads));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_fma_probe<T><<<blocks, threads>>>(out, 16, (T)0.999, (T)0.001);
    cudaEventRecord(a);
    k_fma_probe<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(b);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    AFQ_CUDA(e);
    *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
    return AFQ_OK;
}

}  // namespace afq

using namespace afq;

extern "C" {

int afq_probe_fma_peak(int fp64, double* tflops) {
    if (!tflops) return fail(AFQ_E_INVALID_ARGUMENT, "tflops is NULL");
    return fp64 ? probe<double>(20000, tflops) : probe<float>(200000, tflops);
}

long long afq_launch_count(void) { return g_launches.load(); }

int afq_timing_enable(int on) {
    g_timing = on != 0;
    return AFQ_OK;
}

int afq_timing_reset(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& r : g_pending) {
        cudaEventSynchronize(r.b);
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_pending.clear();
    g_acc.clear();
    return AFQ_OK;
}

int afq_timing_report(char* buf, size_t len) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& r : g_pending) {
        AFQ_CUDA(cudaEventSynchronize(r.b));
        float ms = 0.f;
        AFQ_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        auto& a = g_acc[r.name];
        a.first += 1;
        a.second += ms;
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_pending.clear();
    if (!buf || len == 0) return AFQ_OK;
    size_t used = 0;
    buf[0] = '\0';
    for (auto& kv : g_acc) {
        int k = snprintf(buf + used, len - used, "%s %lld %.6f\n", kv.first.c_str(), kv.second.first,
                         kv.second.second);
        if (k < 0 || (size_t)k >= len - used) return fail(AFQ_E_INVALID_ARGUMENT, "timing report buffer too small");
        used += (size_t)k;
    }
    return AFQ_OK;
}

}  // extern "C"
