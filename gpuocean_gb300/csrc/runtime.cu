// Runtime plumbing of the C ABI: errors, device memory, streams, events,
// CUDA graphs and the launch counter.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "common.cuh"
#include "tma.cuh"

namespace goc {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

int set_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return GOC_OK;
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static int cuda_result(cudaError_t e, const char* what) {
    if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return GOC_OK;
}

}  // namespace goc

using namespace goc;

extern "C" {

int goc_version(void) { return 1; }

int goc_last_error(char* buf, int len) {
    if (!buf || len <= 0) return GOC_ERR_ARG;
    std::strncpy(buf, g_last_error.c_str(), (size_t)len - 1);
    buf[len - 1] = '\0';
    return GOC_OK;
}

int goc_device_count(int* count) {
    if (!count) return set_error(GOC_ERR_ARG, "goc_device_count: null count");
    return cuda_result(cudaGetDeviceCount(count), "cudaGetDeviceCount");
}

int goc_set_device(int device) { return cuda_result(cudaSetDevice(device), "cudaSetDevice"); }

int goc_device_synchronize(void) { return cuda_result(cudaDeviceSynchronize(), "cudaDeviceSynchronize"); }

int goc_malloc(void** ptr, size_t bytes) {
    if (!ptr) return set_error(GOC_ERR_ARG, "goc_malloc: null out pointer");
    *ptr = nullptr;
    if (bytes == 0) return GOC_OK;
    return cuda_result(cudaMalloc(ptr, bytes), "cudaMalloc");
}

int goc_free(void* ptr) {
    if (!ptr) return GOC_OK;
    return cuda_result(cudaFree(ptr), "cudaFree");
}

int goc_host_alloc(void** ptr, size_t bytes) {
    if (!ptr) return set_error(GOC_ERR_ARG, "goc_host_alloc: null out pointer");
    *ptr = nullptr;
    if (bytes == 0) return GOC_OK;
    return cuda_result(cudaMallocHost(ptr, bytes), "cudaMallocHost");
}

int goc_host_free(void* ptr) {
    if (!ptr) return GOC_OK;
    return cuda_result(cudaFreeHost(ptr), "cudaFreeHost");
}

int goc_memset_async(void* dst, int value, size_t bytes, void* stream) {
    if (bytes == 0) return GOC_OK;
    if (!dst) return set_error(GOC_ERR_ARG, "goc_memset_async: null destination");
    return cuda_result(cudaMemsetAsync(dst, value, bytes, as_stream(stream)), "cudaMemsetAsync");
}

static int copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, void* stream,
                const char* what) {
    if (bytes == 0) return GOC_OK;
    if (!dst || !src) return set_error(GOC_ERR_ARG, "%s: null pointer", what);
    return cuda_result(cudaMemcpyAsync(dst, src, bytes, kind, as_stream(stream)), what);
}

int goc_memcpy_h2d_async(void* dst, const void* src, size_t bytes, void* stream) {
    return copy(dst, src, bytes, cudaMemcpyHostToDevice, stream, "goc_memcpy_h2d_async");
}

int goc_memcpy_d2h_async(void* dst, const void* src, size_t bytes, void* stream) {
    return copy(dst, src, bytes, cudaMemcpyDeviceToHost, stream, "goc_memcpy_d2h_async");
}

int goc_memcpy_d2d_async(void* dst, const void* src, size_t bytes, void* stream) {
    return copy(dst, src, bytes, cudaMemcpyDeviceToDevice, stream, "goc_memcpy_d2d_async");
}

int goc_stream_create(void** stream) {
    if (!stream) return set_error(GOC_ERR_ARG, "goc_stream_create: null out pointer");
    cudaStream_t s = nullptr;
    int rc = cuda_result(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    *stream = s;
    return rc;
}

int goc_stream_destroy(void* stream) {
    if (!stream) return GOC_OK;
    return cuda_result(cudaStreamDestroy(as_stream(stream)), "cudaStreamDestroy");
}

int goc_stream_synchronize(void* stream) {
    return cuda_result(cudaStreamSynchronize(as_stream(stream)), "cudaStreamSynchronize");
}

// Device-side ordering between one stream and many (no host wait).  Each
// signalling stream gets a timing-free event recorded on it; the event is
// released right after the waits are queued (the waits keep the recorded
// state).
static int wait_on(cudaStream_t waiter, cudaStream_t signaller) {
    if (waiter == signaller) return GOC_OK;
    cudaEvent_t e = nullptr;
    cudaError_t err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaEventRecord(e, signaller);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(waiter, e, 0);
    if (e) cudaEventDestroy(e);
    return cuda_result(err, "stream ordering");
}

int goc_stream_fan_out(void* signaller, void* const* waiters, int n_waiters) {
    if (n_waiters < 0 || (n_waiters > 0 && !waiters)) return set_error(GOC_ERR_ARG, "goc_stream_fan_out: bad list");
    if (n_waiters == 0) return GOC_OK;
    cudaEvent_t e = nullptr;
    cudaError_t err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaEventRecord(e, as_stream(signaller));
    for (int i = 0; err == cudaSuccess && i < n_waiters; ++i)
        if (waiters[i] != signaller) err = cudaStreamWaitEvent(as_stream(waiters[i]), e, 0);
    if (e) cudaEventDestroy(e);
    return cuda_result(err, "goc_stream_fan_out");
}

int goc_stream_fan_in(void* waiter, void* const* signallers, int n_signallers) {
    if (n_signallers < 0 || (n_signallers > 0 && !signallers))
        return set_error(GOC_ERR_ARG, "goc_stream_fan_in: bad list");
    for (int i = 0; i < n_signallers; ++i) {
        int rc = wait_on(as_stream(waiter), as_stream(signallers[i]));
        if (rc) return rc;
    }
    return GOC_OK;
}

int goc_event_create(void** event) {
    if (!event) return set_error(GOC_ERR_ARG, "goc_event_create: null out pointer");
    cudaEvent_t e = nullptr;
    int rc = cuda_result(cudaEventCreate(&e), "cudaEventCreate");
    *event = e;
    return rc;
}

int goc_event_destroy(void* event) {
    if (!event) return GOC_OK;
    return cuda_result(cudaEventDestroy(reinterpret_cast<cudaEvent_t>(event)), "cudaEventDestroy");
}

int goc_event_record(void* event, void* stream) {
    return cuda_result(cudaEventRecord(reinterpret_cast<cudaEvent_t>(event), as_stream(stream)),
                       "cudaEventRecord");
}

int goc_event_elapsed_ms(void* start, void* stop, float* ms) {
    if (!ms) return set_error(GOC_ERR_ARG, "goc_event_elapsed_ms: null out pointer");
    return cuda_result(cudaEventElapsedTime(ms, reinterpret_cast<cudaEvent_t>(start),
                                            reinterpret_cast<cudaEvent_t>(stop)),
                       "cudaEventElapsedTime");
}

int goc_graph_begin_capture(void* stream) {
    if (!stream) return set_error(GOC_ERR_ARG, "goc_graph_begin_capture: capture needs a non-default stream");
    return cuda_result(cudaStreamBeginCapture(as_stream(stream), cudaStreamCaptureModeThreadLocal),
                       "cudaStreamBeginCapture");
}

int goc_graph_end_capture(void* stream, void** graph_exec) {
    if (!graph_exec) return set_error(GOC_ERR_ARG, "goc_graph_end_capture: null out pointer");
    cudaGraph_t graph = nullptr;
    int rc = cuda_result(cudaStreamEndCapture(as_stream(stream), &graph), "cudaStreamEndCapture");
    if (rc) return rc;
    cudaGraphExec_t exec = nullptr;
    rc = cuda_result(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
    cudaGraphDestroy(graph);
    *graph_exec = exec;
    return rc;
}

int goc_graph_launch(void* graph_exec, void* stream) {
    if (!graph_exec) return set_error(GOC_ERR_ARG, "goc_graph_launch: null graph");
    return cuda_result(cudaGraphLaunch(reinterpret_cast<cudaGraphExec_t>(graph_exec), as_stream(stream)),
                       "cudaGraphLaunch");
}

int goc_graph_destroy(void* graph_exec) {
    if (!graph_exec) return GOC_OK;
    return cuda_result(cudaGraphExecDestroy(reinterpret_cast<cudaGraphExec_t>(graph_exec)),
                       "cudaGraphExecDestroy");
}

int64_t goc_kernel_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

}  // extern "C"

// ---------------------------------------------------------------------------
// self-test of the bounded mbarrier wait that guards TMA staging
// ---------------------------------------------------------------------------

namespace goc {
// Waits on a barrier phase that nothing completes; the wait must give up
// after limit_ns and report it.
__global__ void wait_timeout_selftest_kernel(int* timed_out, unsigned long long* waited_ns, uint64_t limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const uint64_t t0 = global_ns();
    const bool done = mbar_wait_bounded(&bar, 0, limit_ns);
    const uint64_t t1 = global_ns();
    __syncthreads();
    if (threadIdx.x == 0) {
        *timed_out = done ? 0 : 1;
        *waited_ns = t1 - t0;
    }
}
}  // namespace goc

extern "C" int goc_selftest_wait_timeout(double limit_ms, int* timed_out, double* waited_ms) {
    if (!timed_out || !waited_ms || !(limit_ms > 0.0) || limit_ms > 1000.0)
        return goc::set_error(GOC_ERR_ARG, "goc_selftest_wait_timeout: limit in (0, 1000] ms and outputs required");
    int* d_flag = nullptr;
    unsigned long long* d_ns = nullptr;
    cudaError_t err = cudaMalloc(&d_flag, sizeof(int));
    if (err == cudaSuccess) err = cudaMalloc(&d_ns, sizeof(unsigned long long));
    if (err == cudaSuccess) {
        goc::wait_timeout_selftest_kernel<<<1, 64>>>(d_flag, d_ns, (uint64_t)(limit_ms * 1e6));
        err = cudaGetLastError();
    }
    int flag = 0;
    unsigned long long ns = 0;
    if (err == cudaSuccess) err = cudaMemcpy(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(&ns, d_ns, sizeof(ns), cudaMemcpyDeviceToHost);
    cudaFree(d_flag);
    cudaFree(d_ns);
    if (err != cudaSuccess) return goc::set_error(GOC_ERR_CUDA, "goc_selftest_wait_timeout: %s", cudaGetErrorString(err));
    *timed_out = flag;
    *waited_ms = ns / 1e6;
    return GOC_OK;
}
