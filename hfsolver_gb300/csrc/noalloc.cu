// G = J - K/2 from packed integrals without any device allocation.
//
// Who needs this: callers that own every byte of device memory themselves and
// cannot let a library call cudaMalloc, for example an SCF loop embedded in a
// framework whose caching allocator has already reserved the GPU's memory, a
// process running under a fixed device-memory quota, or a caller inside a
// latency-critical loop where a cudaMalloc would synchronise the device.  They
// pass device pointers for the inputs and the output; the only extra memory is
// the scratch array below, a fixed 2 MiB per device, taken when this module is
// loaded on the device (see noalloc_setup) and held until the process exits.
//
// The computation is the Fock two-electron term of hfgpu_formG (same
// arithmetic as jk.cu: each unique packed integral is read once and scattered
// into a half matrix Gh, then G = Gh + Gh^T), with the (k, l) pair of a packed
// row position decoded arithmetically instead of from an allocated table.
#include <mutex>

#include "internal.h"

namespace hfgpu {

constexpr int NOALLOC_MAX_N = 512;  // largest basis: scratch = 512 x 512 doubles = 2 MiB

// Shared by every call on a device: concurrent calls on the GPU would race on it.
static __device__ __align__(256) double g_formG_scratch[NOALLOC_MAX_N * NOALLOC_MAX_N];

// pair index kl = k(k+1)/2 + l  ->  (k, l), exact for kl < 2^24
__device__ __forceinline__ int2 decode_pair(int64_t kl)
{
    int k = (int)((sqrtf(8.0f * (float)kl + 1.0f) - 1.0f) * 0.5f);
    while ((int64_t)k * (k + 1) / 2 > kl) --k;
    while ((int64_t)(k + 1) * (k + 2) / 2 <= kl) ++k;
    return make_int2(k, (int)(kl - (int64_t)k * (k + 1) / 2));
}

__global__ void noalloc_zero_kernel(double* __restrict__ Gh, int64_t nn)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x)
        Gh[i] = 0.0;
}

__global__ void noalloc_jk_kernel(int n, int64_t m, const double* __restrict__ ints, const double* __restrict__ P,
                                  double* __restrict__ Gh)
{
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t ij = warp; ij < m; ij += nwarps) {
        const int2 pij = decode_pair(ij);
        const int i = pij.x, j = pij.y;
        const double fij = (i == j) ? 0.5 : 1.0;
        const double Pij = P[i + (int64_t)j * n];
        const double* row = ints + ij * (ij + 1) / 2;
        double gij = 0.0;
        for (int64_t kl = lane; kl <= ij; kl += 32) {
            const double v = row[kl];
            if (v == 0.0) continue;  // screened-out quartets contribute nothing
            const int2 pkl = decode_pair(kl);
            const int k = pkl.x, l = pkl.y;
            double w = v * fij;
            if (k == l) w *= 0.5;
            if (kl == ij) w *= 0.5;
            gij = fma(2.0 * w, P[k + (int64_t)l * n], gij);
            atomicAdd(&Gh[k + (int64_t)l * n], 2.0 * w * Pij);
            const double hw = -0.5 * w;
            atomicAdd(&Gh[i + (int64_t)k * n], hw * P[j + (int64_t)l * n]);
            atomicAdd(&Gh[j + (int64_t)k * n], hw * P[i + (int64_t)l * n]);
            atomicAdd(&Gh[i + (int64_t)l * n], hw * P[j + (int64_t)k * n]);
            atomicAdd(&Gh[j + (int64_t)l * n], hw * P[i + (int64_t)k * n]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) gij += __shfl_xor_sync(0xffffffffu, gij, o);
        if (lane == 0) atomicAdd(&Gh[i + (int64_t)j * n], gij);
    }
}

__global__ void noalloc_symmetrize_kernel(int n, const double* __restrict__ Gh, double* __restrict__ G)
{
    const int64_t nn = (int64_t)n * n;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nn;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx % n), j = (int)(idx / n);
        G[idx] = Gh[idx] + Gh[j + (int64_t)i * n];
    }
}

// Device address of the scratch array, looked up once per device with that
// device current (the host-side name g_formG_scratch is only a stand-in).  The
// lookup loads this file's module on the device, which is when the 2 MiB array
// is allocated (CUDA loads modules lazily by default).  Every libhfgpu entry
// point that creates the library's device context does this, and so does the
// first allocation-free call on a device that has no context yet.  The cached
// address belongs to the device's current primary context: calls must not cross
// a cudaDeviceReset.
static std::mutex g_noalloc_mutex;
static double* g_noalloc_ptr[64] = {nullptr};
static int g_noalloc_sms[64] = {0};

static void noalloc_setup(int dev, double** ptr, int* sms)
{
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    HF_CHECK(dev >= 0 && dev < 64, HFGPU_ERR_INVALID, "device ordinal out of range");
    if (!g_noalloc_ptr[dev]) {
        double* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_formG_scratch);
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            throw Error(HFGPU_ERR_NOMEM,
                        "hfgpu_formG_device_noalloc: no device memory left for its fixed 2 MiB scratch array "
                        "(taken when the library's module is first loaded on the device; make the first "
                        "libhfgpu call before reserving the device's memory)");
        }
        HF_CUDA(e);
        HF_CHECK(p != nullptr, HFGPU_ERR_CUDA, "cudaGetSymbolAddress returned no address");
        int s = 0;
        HF_CUDA(cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev));
        g_noalloc_sms[dev] = s;
        g_noalloc_ptr[dev] = p;
    }
    if (ptr) *ptr = g_noalloc_ptr[dev];
    if (sms) *sms = g_noalloc_sms[dev];
}

void noalloc_prepare(int dev) { noalloc_setup(dev, nullptr, nullptr); }

}  // namespace hfgpu

extern "C" int hfgpu_formG_device_noalloc(int n, const double* d_int2, const double* d_P, double* d_G,
                                          void* cuda_stream)
{
    using namespace hfgpu;
    try {
        HF_CHECK(n >= 1, HFGPU_ERR_INVALID, "n must be >= 1");
        HF_CHECK(n <= NOALLOC_MAX_N, HFGPU_ERR_INVALID,
                 "hfgpu_formG_device_noalloc: n = " + std::to_string(n) + " exceeds its fixed scratch limit of " +
                     std::to_string(NOALLOC_MAX_N) + " basis functions");
        HF_CHECK(d_int2 && d_P && d_G, HFGPU_ERR_INVALID, "device pointers must not be NULL");
        // an error left by the caller's own earlier asynchronous work is reported as
        // such and left pending, not taken for a failure of this call
        const cudaError_t pending = cudaPeekAtLastError();
        if (pending != cudaSuccess)
            throw Error(HFGPU_ERR_CUDA, std::string("hfgpu_formG_device_noalloc: a CUDA error was already pending "
                                                    "before this call: ") + cudaGetErrorString(pending));
        int dev = 0;
        HF_CUDA(cudaGetDevice(&dev));
        double* Gh = nullptr;
        int sms = 0;
        noalloc_setup(dev, &Gh, &sms);
        cudaStream_t st = (cudaStream_t)cuda_stream;
        const int64_t nn = (int64_t)n * n, m = (int64_t)n * (n + 1) / 2;
        const unsigned gz = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nn + 255) / 256, (int64_t)sms * 8));
        noalloc_zero_kernel<<<gz, 256, 0, st>>>(Gh, nn);
        count_launch();
        HF_CUDA(cudaGetLastError());
        const unsigned gj = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m + 7) / 8, (int64_t)sms * 16));
        noalloc_jk_kernel<<<gj, 256, 0, st>>>(n, m, d_int2, d_P, Gh);
        count_launch();
        HF_CUDA(cudaGetLastError());
        noalloc_symmetrize_kernel<<<gz, 256, 0, st>>>(n, Gh, d_G);
        count_launch();
        HF_CUDA(cudaGetLastError());
        return HFGPU_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return HFGPU_ERR_CUDA;
    }
}
