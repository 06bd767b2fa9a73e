// Allocation-free variant of hgb_argsort_f0_desc: the same loudest-first order at the first
// frequency (holodeck/single_sources.py:89), with its scratch in a file-scope device array instead
// of a caller workspace.
//
// Scratch layout (one array per device, HGB_SORT_STATIC_BYTES):
//   keys_a [HGB_SORT_STATIC_MAX_BINS] double   gathered keys
//   keys_b [HGB_SORT_STATIC_MAX_BINS] double   the radix sort's alternate key buffer
//   idx_a  [HGB_SORT_STATIC_MAX_BINS] int32    bin indices (the alternate index buffer is `order`)
//   cub    SORT_CUB_BYTES                      CUB's temporary storage
// Nothing in it has to start at zero: the gather writes every key and index the sort reads, and CUB
// initialises its own counters inside its temporary storage on every call.
#include <cub/device/device_radix_sort.cuh>

#include <mutex>

#include "hgb_common.cuh"

namespace {

constexpr long MAX_BINS = HGB_SORT_STATIC_MAX_BINS;
constexpr size_t KEYS_BYTES = sizeof(double) * MAX_BINS;
constexpr size_t IDX_BYTES = sizeof(int32_t) * MAX_BINS;
constexpr size_t SORT_CUB_BYTES = HGB_SORT_STATIC_BYTES - 2 * KEYS_BYTES - IDX_BYTES;
static_assert(HGB_SORT_STATIC_BYTES > 2 * KEYS_BYTES + IDX_BYTES, "scratch too small for the key buffers");
static_assert(KEYS_BYTES % 256 == 0 && IDX_BYTES % 256 == 0, "scratch regions keep 256-byte alignment");

__device__ __align__(256) unsigned char g_sort_scratch[HGB_SORT_STATIC_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_scratch_mutex;
void *g_scratch_ptr[MAX_DEVICES];   // device address of g_sort_scratch, per device ordinal

// Address of the current device's copy of g_sort_scratch, looked up once per device.
int scratch_of_current_device(unsigned char **out) {
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) {
        hgb::set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    if (dev < 0 || dev >= MAX_DEVICES) return HGB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (err != cudaSuccess) {
            hgb::set_cuda_error(err);
            return HGB_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = (unsigned char *)g_scratch_ptr[dev];
    return HGB_OK;
}

__global__ void k_gather_f0_static(const double *__restrict__ h2fdf, long nb, int nf, double *__restrict__ keys,
                                   int32_t *__restrict__ idx) {
    long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    keys[b] = h2fdf[b * nf];
    idx[b] = (int32_t)b;
}

}  // namespace

extern "C" {

int hgb_argsort_f0_desc_static(const double *h2fdf, long n_bins, int n_freq, int32_t *order, void *stream) {
    HGB_CHECK_ARG(h2fdf && order && n_bins >= 0 && n_freq >= 1);
    if (n_bins > MAX_BINS) return HGB_ERR_CAPACITY;
    if (n_bins == 0) return HGB_OK;
    unsigned char *base = nullptr;
    int rc = scratch_of_current_device(&base);
    if (rc) return rc;
    double *keys_a = (double *)base;
    double *keys_b = (double *)(base + KEYS_BYTES);
    int32_t *idx_a = (int32_t *)(base + 2 * KEYS_BYTES);
    void *cub_tmp = base + 2 * KEYS_BYTES + IDX_BYTES;
    cub::DoubleBuffer<double> keys(keys_a, keys_b);
    cub::DoubleBuffer<int32_t> vals(idx_a, order);
    size_t tb = 0;
    cudaError_t err = cub::DeviceRadixSort::SortPairsDescending(nullptr, tb, keys, vals, (int)n_bins, 0, 64);
    if (err != cudaSuccess) {
        hgb::set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    if (tb > SORT_CUB_BYTES) return HGB_ERR_CAPACITY;
    cudaStream_t st = (cudaStream_t)stream;
    k_gather_f0_static<<<(unsigned)hgb::ceil_div(n_bins, 256), 256, 0, st>>>(h2fdf, n_bins, n_freq, keys_a, idx_a);
    if ((rc = hgb::check_launch())) return rc;
    err = cub::DeviceRadixSort::SortPairsDescending(cub_tmp, tb, keys, vals, (int)n_bins, 0, 64, st);
    if (err != cudaSuccess) {
        hgb::set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    // the sorted indices end in whichever index buffer the last pass wrote
    if (vals.Current() != order) {
        err = cudaMemcpyAsync(order, vals.Current(), sizeof(int32_t) * n_bins, cudaMemcpyDeviceToDevice, st);
        if (err != cudaSuccess) {
            hgb::set_cuda_error(err);
            return HGB_ERR_CUDA;
        }
    }
    return hgb::check_launch();
}

}  // extern "C"
