// Loudest-first bin order at the first frequency (holodeck/single_sources.py:89:
// argsort(-h2fdf[..., 0])): gather the keys, then a radix sort of (key, bin) pairs.
#include <cub/device/device_radix_sort.cuh>

#include "hgb_common.cuh"

namespace {

__global__ void k_gather_f0(const double *__restrict__ h2fdf, long nb, int nf, double *__restrict__ keys,
                            int32_t *__restrict__ idx) {
    long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    keys[b] = h2fdf[b * nf];
    idx[b] = (int32_t)b;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t cub_bytes(long nb) {
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairsDescending((void *)nullptr, tb, (const double *)nullptr, (double *)nullptr,
                                              (const int32_t *)nullptr, (int32_t *)nullptr, (int)nb);
    return tb;
}

}  // namespace

extern "C" {

size_t hgb_sort_workspace_bytes(long n_bins) {
    if (n_bins <= 0) return 0;
    return align256(sizeof(double) * n_bins) * 2 + align256(sizeof(int32_t) * n_bins) + align256(cub_bytes(n_bins));
}

int hgb_argsort_f0_desc(const double *h2fdf, long n_bins, int n_freq, int32_t *order, void *workspace,
                        size_t workspace_bytes, void *stream) {
    HGB_CHECK_ARG(h2fdf && order && n_bins >= 0 && n_bins < (1L << 31) && n_freq >= 1);
    if (n_bins == 0) return HGB_OK;
    size_t need = hgb_sort_workspace_bytes(n_bins);
    if (!workspace || workspace_bytes < need) return HGB_ERR_WORKSPACE;
    char *w = (char *)workspace;
    double *keys_in = (double *)w;
    w += align256(sizeof(double) * n_bins);
    double *keys_out = (double *)w;
    w += align256(sizeof(double) * n_bins);
    int32_t *idx_in = (int32_t *)w;
    w += align256(sizeof(int32_t) * n_bins);
    size_t tb = cub_bytes(n_bins);
    cudaStream_t st = (cudaStream_t)stream;
    k_gather_f0<<<(unsigned)hgb::ceil_div(n_bins, 256), 256, 0, st>>>(h2fdf, n_bins, n_freq, keys_in, idx_in);
    int rc = hgb::check_launch();
    if (rc) return rc;
    cudaError_t err = cub::DeviceRadixSort::SortPairsDescending((void *)w, tb, keys_in, keys_out, idx_in, order,
                                                                (int)n_bins, 0, 64, st);
    if (err != cudaSuccess) {
        hgb::set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    return hgb::check_launch();
}

}  // extern "C"
