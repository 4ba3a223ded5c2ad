// Per-device context: stream, cuBLAS/cuSOLVER handles, Boys-function grid.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "boys.cuh"
#include "internal.h"

namespace hfgpu {

static thread_local std::string g_last_error;
void set_last_error(const std::string& m) { g_last_error = m; }

static std::atomic<int64_t> g_launches{0};
void count_launch(int n) { g_launches += n; }
int64_t launches_counted() { return g_launches.load(); }

static std::mutex g_ctx_mutex;
static std::vector<Context*> g_ctx;

static Context* make_context(int dev);

Context& context()
{
    int dev = 0;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) throw Error(HFGPU_ERR_NO_DEVICE, "no CUDA device");
    HF_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_ctx_mutex);
    if ((int)g_ctx.size() < ndev) g_ctx.resize(ndev, nullptr);
    if (!g_ctx[dev]) g_ctx[dev] = make_context(dev);
    return *g_ctx[dev];
}

// Extra contexts for concurrent molecules (hfgpu_rhf_batch workers): each has
// its own streams and library handles; released contexts are kept for reuse.
static std::vector<std::vector<Context*>> g_pool;

Context* context_acquire()
{
    int dev = 0, ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) throw Error(HFGPU_ERR_NO_DEVICE, "no CUDA device");
    HF_CUDA(cudaGetDevice(&dev));
    {
        std::lock_guard<std::mutex> lk(g_ctx_mutex);
        if ((int)g_pool.size() < ndev) g_pool.resize(ndev);
        if (!g_pool[dev].empty()) {
            Context* c = g_pool[dev].back();
            g_pool[dev].pop_back();
            return c;
        }
    }
    return make_context(dev);
}

void context_release(Context* c)
{
    if (!c) return;
    std::lock_guard<std::mutex> lk(g_ctx_mutex);
    if ((int)g_pool.size() <= c->device) g_pool.resize(c->device + 1);
    g_pool[c->device].push_back(c);
}

static Context* make_context(int dev)
{
    auto* c = new Context();
    c->device = dev;
    // the main stream outranks the side streams: its chains of small dependent
    // kernels (the SCF set-up under the ERI pass, the symmetrisation after a
    // Fock build) take SMs first as blocks of the side streams' classes drain
    {
        int least = 0, greatest = 0;
        HF_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        HF_CUDA(cudaStreamCreateWithPriority(&c->own_stream, cudaStreamNonBlocking, greatest));
    }
    c->stream = c->own_stream;
    HF_CUBLAS(cublasCreate(&c->blas));
    HF_CUBLAS(cublasSetStream(c->blas, c->stream));
    HF_CUSOLVER(cusolverDnCreate(&c->solver));
    HF_CUSOLVER(cusolverDnSetStream(c->solver, c->stream));
    HF_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev));
    // Stream-ordered allocations (cudaMallocAsync) come from the device's default
    // pool, which by default returns its memory to the driver at every
    // synchronisation; each molecule's GB-sized buffers would then be mapped
    // again.  Keep up to 64 GB cached in the pool (process-local setting).
    {
        cudaMemPool_t pool;
        HF_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
        uint64_t keep = 64ull << 30;
        HF_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    for (int i = 0; i < Context::NAUX; ++i) {
        HF_CUDA(cudaStreamCreateWithFlags(&c->aux[i], cudaStreamNonBlocking));
        HF_CUDA(cudaEventCreateWithFlags(&c->join_ev[i], cudaEventDisableTiming));
    }
    HF_CUDA(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
    std::vector<double> tab((size_t)BOYS_NROW * BOYS_STRIDE);
    boys_make_table(tab.data());
    HF_CUDA(cudaMalloc((void**)&c->boys, tab.size() * sizeof(double)));
    HF_CUDA(cudaMemcpy(c->boys, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
    noalloc_prepare(dev);
    return c;
}

void Context::fork()
{
    HF_CUDA(cudaEventRecord(fork_ev, stream));
    for (int i = 0; i < NAUX; ++i) HF_CUDA(cudaStreamWaitEvent(aux[i], fork_ev, 0));
}

void Context::settle_timers()
{
    for (auto& e : fock_events) {
        HF_CUDA(cudaEventSynchronize(e.b));
        float ms = 0;
        HF_CUDA(cudaEventElapsedTime(&ms, e.a, e.b));
        stat_fock_ms += ms;
        if (e.full) {
            stat_fock_full_ms += ms;
            stat_fock_full_n += 1;
        }
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    fock_events.clear();
}

static double host_now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void Context::trace_begin()
{
    const char* e = std::getenv("HFGPU_TRACE");
    trace_on = e && e[0] && e[0] != '0';
    for (auto& m : trace) cudaEventDestroy(m.ev);
    trace.clear();
    trace_mark("begin");
}

void Context::trace_mark(const char* name)
{
    if (!trace_on) return;
    TraceMark m{name, nullptr, host_now_ms()};
    HF_CUDA(cudaEventCreate(&m.ev));
    HF_CUDA(cudaEventRecord(m.ev, stream));
    trace.push_back(m);
}

void Context::trace_report()
{
    if (!trace_on || trace.size() < 2) return;
    HF_CUDA(cudaEventSynchronize(trace.back().ev));
    struct Row {
        const char* name;
        double dev, host;
        int count;
    };
    std::vector<Row> rows;
    for (size_t i = 1; i < trace.size(); ++i) {
        float ms = 0;
        HF_CUDA(cudaEventElapsedTime(&ms, trace[i - 1].ev, trace[i].ev));
        const double host = trace[i].host_ms - trace[i - 1].host_ms;
        auto it = std::find_if(rows.begin(), rows.end(),
                               [&](const Row& r) { return std::strcmp(r.name, trace[i].name) == 0; });
        if (it == rows.end()) rows.push_back({trace[i].name, ms, host, 1});
        else { it->dev += ms; it->host += host; it->count += 1; }
    }
    double tot = 0;
    for (auto& r : rows) tot += r.dev;
    std::fprintf(stderr, "hfgpu trace: %-14s %10s %10s %6s\n", "phase", "device ms", "host ms", "count");
    for (auto& r : rows) std::fprintf(stderr, "hfgpu trace: %-14s %10.3f %10.3f %6d\n", r.name, r.dev, r.host, r.count);
    std::fprintf(stderr, "hfgpu trace: %-14s %10.3f\n", "total", tot);
    for (auto& m : trace) cudaEventDestroy(m.ev);
    trace.clear();
}

void Context::join()
{
    for (int i = 0; i < NAUX; ++i) {
        HF_CUDA(cudaEventRecord(join_ev[i], aux[i]));
        HF_CUDA(cudaStreamWaitEvent(stream, join_ev[i], 0));
    }
}

}  // namespace hfgpu

extern "C" const char* hfgpu_last_error(void) { return hfgpu::g_last_error.c_str(); }
extern "C" int hfgpu_version(void) { return 1; }
extern "C" int64_t hfgpu_kernel_launches(void) { return hfgpu::g_launches.load(); }
