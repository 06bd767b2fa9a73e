// Library-level entry points: version, error strings, shared host helpers.
#include <math.h>
#include <stdio.h>

#include <atomic>
#include <map>
#include <mutex>
#include <utility>

#include "hgb_common.cuh"

namespace {

__global__ void k_sqrt(double *x, long n) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = sqrt(x[i]);
}

}  // namespace

namespace hgb {

static thread_local char g_last_cuda_error[256] = "";

void set_cuda_error(cudaError_t err) {
    snprintf(g_last_cuda_error, sizeof(g_last_cuda_error), "%s: %s", cudaGetErrorName(err),
             cudaGetErrorString(err));
}

int check_launch() {
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    return HGB_OK;
}

int sm_count() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

int ensure_dyn_smem(const void *func, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> raised;   // (function, device) -> cap set
    if (bytes <= 48 * 1024) return HGB_OK;   // within the default cap
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) {
        set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(mu);
    size_t &cap = raised[std::make_pair(func, dev)];
    if (bytes <= cap) return HGB_OK;
    err = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) {
        set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    cap = bytes;
    return HGB_OK;
}

CyConst cy_const() {
    CyConst c;
    c.c_dadt = -64.0 * pow(HGB_CY_NWTG, 3) / 5.0 / pow(HGB_CY_SPLC, 5);
    c.kfreq = (1.0 / (2.0 * M_PI)) * sqrt(HGB_CY_NWTG);
    c.ksepa = pow(HGB_CY_NWTG, 1.0 / 3.0) / pow(2.0 * M_PI, 2.0 / 3.0);
    c.fourpi = 4 * M_PI * HGB_CY_SPLC / HGB_CY_MPC;
    return c;
}

}  // namespace hgb

extern "C" {

int hgb_version(void) { return 1; }

const char *hgb_error_string(int code) {
    switch (code) {
        case HGB_OK: return "success";
        case HGB_ERR_INVALID_ARGUMENT: return "invalid argument";
        case HGB_ERR_CUDA: return "CUDA error";
        case HGB_ERR_WORKSPACE: return "workspace too small";
        case HGB_ERR_CAPACITY: return "input exceeds the static scratch capacity";
        case HGB_ERR_DEVICE_LIMIT: return "a bounded device wait gave up; outputs not valid";
        default: return "unknown error";
    }
}

const char *hgb_last_cuda_error(void) { return hgb::g_last_cuda_error; }

int hgb_sqrt_inplace(double *x, long n, void *stream) {
    if (!x || n < 0) return HGB_ERR_INVALID_ARGUMENT;
    if (n == 0) return HGB_OK;
    k_sqrt<<<(unsigned)hgb::ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(x, n);
    return hgb::check_launch();
}

}  // extern "C"
