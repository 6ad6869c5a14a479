/*
 * mock_rt.cpp -- TEST INFRASTRUCTURE ONLY: a stand-in for the CUDA runtime
 * calls the library's host code (capi.cu) makes, so that its set-up, pool
 * layout, copies and launch parameters can be checked on a machine without
 * a GPU.  Device memory is host memory, every copy is a memcpy done at once,
 * streams, events and graphs are placeholders, and a device allocation is
 * filled with 0xAB so that reads of never-written bytes stand out.
 */
#include <cuda_runtime_api.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <vector>

struct MockAlloc { size_t n; bool dev; };
struct MockGraph { std::vector<std::function<void()>> ops; };
static MockGraph *g_capture = nullptr;
static int g_graph_launches = 0;
/* a launch made while a capture is open is recorded, not run */
bool mock_capture_push(std::function<void()> f) {
    if (!g_capture) return false;
    g_capture->ops.push_back(std::move(f));
    return true;
}
static std::map<uintptr_t, MockAlloc> g_allocs;

/* the allocation holding p: its base and size */
bool mock_alloc_of(const void *p, const char **base, size_t *n) {
    const uintptr_t a = (uintptr_t)p;
    auto it = g_allocs.upper_bound(a);
    if (it == g_allocs.begin()) return false;
    --it;
    if (a < it->first || a >= it->first + it->second.n) return false;
    *base = (const char *)it->first;
    *n = it->second.n;
    return true;
}
static void *take(size_t n, bool dev) {
    const size_t sz = ((n ? n : 1) + 511) & ~(size_t)511;
    char *p = (char *)aligned_alloc(512, sz);
    if (p && dev) std::memset(p, 0xAB, sz);
    if (p) g_allocs[(uintptr_t)p] = MockAlloc{n ? n : 1, dev};
    return p;
}
static void give(void *p) {
    if (!p) return;
    g_allocs.erase((uintptr_t)p);
    free(p);
}

extern "C" {
size_t mock_live_allocations(void) { return g_allocs.size(); }
cudaError_t cudaMalloc(void **p, size_t n) { *p = take(n, true); return *p ? cudaSuccess : cudaErrorMemoryAllocation; }
cudaError_t cudaMallocAsync(void **p, size_t n, cudaStream_t) { return cudaMalloc(p, n); }
cudaError_t cudaFree(void *p) { give(p); return cudaSuccess; }
cudaError_t cudaFreeAsync(void *p, cudaStream_t) { give(p); return cudaSuccess; }
cudaError_t cudaMallocHost(void **p, size_t n) { *p = take(n, false); return *p ? cudaSuccess : cudaErrorMemoryAllocation; }
cudaError_t cudaFreeHost(void *p) { give(p); return cudaSuccess; }
/* failure injection: the k-th device-to-host copy from now fails (0: none) */
static int g_fail_d2h = 0;
void mock_fail_d2h(int k) { g_fail_d2h = k; }
cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind k) {
    if (k == cudaMemcpyDeviceToHost && g_fail_d2h > 0 && --g_fail_d2h == 0) return cudaErrorUnknown;
    std::memmove(d, s, n);
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, cudaMemcpyKind k, cudaStream_t) { return cudaMemcpy(d, s, n, k); }
cudaError_t cudaMemsetAsync(void *d, int v, size_t n, cudaStream_t) { std::memset(d, v, n); return cudaSuccess; }
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned int) { *s = (cudaStream_t)take(8, false); return cudaSuccess; }
cudaError_t cudaStreamDestroy(cudaStream_t s) { give(s); return cudaSuccess; }
cudaError_t cudaEventCreate(cudaEvent_t *e) { *e = (cudaEvent_t)take(8, false); return cudaSuccess; }
cudaError_t cudaEventDestroy(cudaEvent_t e) { give(e); return cudaSuccess; }
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) { *ms = 1.0f; return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t) { return "mock runtime error"; }
cudaError_t cudaGetDevice(int *d) { *d = 0; return cudaSuccess; }
/* a GB300: compute capability 10.3, 152 SMs */
cudaError_t cudaDeviceGetAttribute(int *v, cudaDeviceAttr a, int) {
    *v = a == cudaDevAttrComputeCapabilityMajor ? 10 : a == cudaDevAttrComputeCapabilityMinor ? 3
       : a == cudaDevAttrMultiProcessorCount ? 152 : 0;
    return cudaSuccess;
}
cudaError_t cudaMemGetInfo(size_t *f, size_t *t) { *f = (size_t)100 << 30; *t = (size_t)200 << 30; return cudaSuccess; }
cudaError_t cudaGetSymbolAddress(void **, const void *) { return cudaErrorInvalidSymbol; }
/* graphs: a capture records the launches made on the stream (the stand-in
 * launches push themselves through mock_capture_push) and a graph launch
 * runs them in order */
cudaError_t cudaStreamIsCapturing(cudaStream_t, cudaStreamCaptureStatus *s) {
    *s = g_capture ? cudaStreamCaptureStatusActive : cudaStreamCaptureStatusNone;
    return cudaSuccess;
}
cudaError_t cudaStreamBeginCapture(cudaStream_t, cudaStreamCaptureMode) {
    if (g_capture) return cudaErrorIllegalState;
    g_capture = new MockGraph;
    return cudaSuccess;
}
cudaError_t cudaStreamEndCapture(cudaStream_t, cudaGraph_t *g) {
    if (!g_capture) return cudaErrorIllegalState;
    *g = (cudaGraph_t)g_capture;
    g_capture = nullptr;
    return cudaSuccess;
}
cudaError_t cudaGraphInstantiate(cudaGraphExec_t *e, cudaGraph_t g, unsigned long long) {
    *e = (cudaGraphExec_t) new MockGraph(*(MockGraph *)g);
    return cudaSuccess;
}
cudaError_t cudaGraphLaunch(cudaGraphExec_t e, cudaStream_t) {
    ++g_graph_launches;
    for (auto &f : ((MockGraph *)e)->ops) f();
    return cudaSuccess;
}
cudaError_t cudaGraphDestroy(cudaGraph_t g) { delete (MockGraph *)g; return cudaSuccess; }
cudaError_t cudaGraphExecDestroy(cudaGraphExec_t e) { delete (MockGraph *)e; return cudaSuccess; }
int mock_graph_launches(void) { return g_graph_launches; }
void **__cudaRegisterFatBinary(void *) { static void *h = nullptr; return &h; }
void __cudaRegisterFatBinaryEnd(void **) {}
void __cudaUnregisterFatBinary(void **) {}
}
