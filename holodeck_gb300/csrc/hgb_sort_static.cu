// Allocation-free variant of hgb_argsort_f0_desc: the same loudest-first order at the first
// frequency (holodeck/single_sources.py:89), computed by the same radix sort (hgb_sort.cu), with its
// scratch in a file-scope device array instead of a caller workspace.
//
// The array holds the radix sort's scratch for up to HGB_SORT_STATIC_MAX_BINS bins: two key buffers,
// one index buffer (the other is `order`), the per-block digit counts and the digit totals.  Nothing
// in it has to start at zero: every pass writes each count, total, key and index before reading it.
// Calls on different streams of one device share the array, so they must not overlap.
#include <mutex>

#include "hgb_common.cuh"

namespace {

constexpr long MAX_BINS = HGB_SORT_STATIC_MAX_BINS;

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

}  // namespace

extern "C" {

int hgb_argsort_f0_desc_static(const double *h2fdf, long n_bins, int n_freq, int32_t *order, void *stream) {
    HGB_CHECK_ARG(h2fdf && order && n_bins >= 0 && n_freq >= 1);
    if (n_bins > MAX_BINS || hgb::argsort_f0_scratch_bytes(n_bins) > HGB_SORT_STATIC_BYTES) return HGB_ERR_CAPACITY;
    if (n_bins == 0) return HGB_OK;
    unsigned char *base = nullptr;
    int rc = scratch_of_current_device(&base);
    if (rc) return rc;
    return hgb::argsort_f0_desc_into(h2fdf, n_bins, n_freq, order, base, (cudaStream_t)stream);
}

}  // extern "C"
