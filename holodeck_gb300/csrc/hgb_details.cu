// Model details of a library run: holodeck/librarian/lib_tools.py:845-943 (_calc_model_details).
//
// With w = h2fdf * number on the (M-1, Q-1, Z-1, F) bins and zf the final redshift at bin centres
// (the midpoints of redz_final along mtot, mrat, redz):
//   gwb_m[m, z, f] = sum_q w / denom[f]        num_m[m, z, f] = sum_q number
//   gwb_q[q, z, f] = sum_m w / denom[f]        num_q[q, z, f] = sum_m number
//   gwb_z[z, f]    = sum_mq w / denom[f]       num_z[z, f]    = sum_mq number
//   gwb_rz[k, f]   = sum over bins whose zf falls in redshift bin k of w / denom[f]   (num_rz alike)
//   gwb_mrz[m, k, f], num_mrz[m, k, f]: the same per total-mass bin
//   denom[f] = sum over all bins of w
// The redshift bins are the grid's redz edges with scipy.stats.binned_statistic's rule: [e_k, e_k+1)
// except the last, which is closed; values outside (including the -1 sentinels and NaN) are dropped.
//
// One thread owns one output row (an (m, f) or a (q, f) pair) and accumulates it in the
// reference's flat visiting order, so results are deterministic; consecutive threads take
// consecutive frequencies, so loads and stores are coalesced along the F axis.  FP64, built with
// -fmad=false (products and sums round separately, as numpy's do).
#include <math.h>

#include "hgb_common.cuh"

namespace {

struct DetGeom {
    int nm, nq, nz, nf;   // bin counts along mtot, mrat, redz; frequencies
};

__device__ __forceinline__ long bin_idx(const DetGeom &g, int m, int q, int z, int f) {
    return (((long)m * g.nq + q) * g.nz + z) * g.nf + f;
}

// redz_final is on the (M, Q, Z, F) edges
__device__ __forceinline__ double zf_center(const DetGeom &g, const double *rzf, int m, int q, int z, int f) {
    const int Q = g.nq + 1, Z = g.nz + 1;
    auto at = [&](int i, int j, int k) { return rzf[(((long)(m + i) * Q + (q + j)) * Z + (z + k)) * g.nf + f]; };
    const double a00 = 0.5 * (at(1, 0, 0) + at(0, 0, 0));
    const double a01 = 0.5 * (at(1, 0, 1) + at(0, 0, 1));
    const double a10 = 0.5 * (at(1, 1, 0) + at(0, 1, 0));
    const double a11 = 0.5 * (at(1, 1, 1) + at(0, 1, 1));
    const double b0 = 0.5 * (a10 + a00);
    const double b1 = 0.5 * (a11 + a01);
    return 0.5 * (b1 + b0);
}

// binned_statistic's bin of x among nz + 1 ascending edges, or -1
__device__ __forceinline__ int redz_bin(const double *edges, int nz, double x) {
    if (!(x >= edges[0] && x <= edges[nz])) return -1;
    if (x == edges[nz]) return nz - 1;
    int lo = 0, hi = nz;   // edges[lo] <= x < edges[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (edges[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

// thread per (m, f): sum over q (per z) and the final-redshift histogram of the m slice, visiting
// (q, z) in flat order
__global__ void k_details_m(DetGeom g, const double *__restrict__ number, const double *__restrict__ h2fdf,
                            const double *__restrict__ redz_final, const double *__restrict__ redz_edges,
                            double *__restrict__ gwb_m, double *__restrict__ num_m, double *__restrict__ gwb_mrz,
                            double *__restrict__ num_mrz) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)g.nm * g.nf) return;
    const int m = (int)(idx / g.nf), f = (int)(idx % g.nf);
    for (int z = 0; z < g.nz; z++) {
        const long o = ((long)m * g.nz + z) * g.nf + f;
        gwb_m[o] = 0.0;
        num_m[o] = 0.0;
        gwb_mrz[o] = 0.0;
        num_mrz[o] = 0.0;
    }
    for (int q = 0; q < g.nq; q++) {
        for (int z = 0; z < g.nz; z++) {
            const long b = bin_idx(g, m, q, z, f);
            const double n = number[b];
            const double w = h2fdf[b] * n;
            const long o = ((long)m * g.nz + z) * g.nf + f;
            gwb_m[o] += w;
            num_m[o] += n;
            const int k = redz_bin(redz_edges, g.nz, zf_center(g, redz_final, m, q, z, f));
            if (k >= 0) {
                const long ok = ((long)m * g.nz + k) * g.nf + f;
                gwb_mrz[ok] += w;
                num_mrz[ok] += n;
            }
        }
    }
}

// thread per (q, f): sum over m (per z)
__global__ void k_details_q(DetGeom g, const double *__restrict__ number, const double *__restrict__ h2fdf,
                            double *__restrict__ gwb_q, double *__restrict__ num_q) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)g.nq * g.nf) return;
    const int q = (int)(idx / g.nf), f = (int)(idx % g.nf);
    for (int z = 0; z < g.nz; z++) {
        const long o = ((long)q * g.nz + z) * g.nf + f;
        gwb_q[o] = 0.0;
        num_q[o] = 0.0;
    }
    for (int m = 0; m < g.nm; m++) {
        for (int z = 0; z < g.nz; z++) {
            const long b = bin_idx(g, m, q, z, f);
            const double n = number[b];
            const long o = ((long)q * g.nz + z) * g.nf + f;
            gwb_q[o] += h2fdf[b] * n;
            num_q[o] += n;
        }
    }
}

// thread per (z, f): the redshift marginals from the per-m rows, then (thread per f) the
// denominators, then every gwb_* row divided by its frequency's denominator
__global__ void k_details_z(DetGeom g, const double *__restrict__ gwb_m, const double *__restrict__ num_m,
                            const double *__restrict__ gwb_mrz, const double *__restrict__ num_mrz,
                            double *__restrict__ gwb_z, double *__restrict__ num_z, double *__restrict__ gwb_rz,
                            double *__restrict__ num_rz) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)g.nz * g.nf) return;
    const int z = (int)(idx / g.nf), f = (int)(idx % g.nf);
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
    for (int m = 0; m < g.nm; m++) {
        const long o = ((long)m * g.nz + z) * g.nf + f;
        a += gwb_m[o];
        b += num_m[o];
        c += gwb_mrz[o];
        d += num_mrz[o];
    }
    gwb_z[idx] = a;
    num_z[idx] = b;
    gwb_rz[idx] = c;
    num_rz[idx] = d;
}

__global__ void k_details_denom(DetGeom g, const double *__restrict__ gwb_z, double *__restrict__ denom) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= g.nf) return;
    double s = 0.0;
    for (int z = 0; z < g.nz; z++) s += gwb_z[(long)z * g.nf + f];
    denom[f] = s;
}

__global__ void k_details_normalise(long n, int nf, const double *__restrict__ denom, double *__restrict__ a) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n) a[idx] = a[idx] / denom[idx % nf];
}

}  // namespace

extern "C" {

int hgb_model_details(const double *number, const double *h2fdf, const double *redz_final, const double *redz_edges,
                      int n_mtot, int n_mrat, int n_redz, int n_freq, double *gwb_m, double *gwb_q, double *gwb_z,
                      double *gwb_rz, double *num_m, double *num_q, double *num_z, double *num_rz, double *gwb_mrz,
                      double *num_mrz, double *denom, void *stream) {
    HGB_CHECK_ARG(number && h2fdf && redz_final && redz_edges && denom);
    HGB_CHECK_ARG(gwb_m && gwb_q && gwb_z && gwb_rz && num_m && num_q && num_z && num_rz && gwb_mrz && num_mrz);
    HGB_CHECK_ARG(n_mtot >= 2 && n_mrat >= 2 && n_redz >= 2 && n_freq >= 1);
    DetGeom g{n_mtot - 1, n_mrat - 1, n_redz - 1, n_freq};
    cudaStream_t st = (cudaStream_t)stream;
    const long nmf = (long)g.nm * g.nf, nqf = (long)g.nq * g.nf, nzf = (long)g.nz * g.nf;
    k_details_m<<<(unsigned)hgb::ceil_div(nmf, 64), 64, 0, st>>>(g, number, h2fdf, redz_final, redz_edges, gwb_m,
                                                                 num_m, gwb_mrz, num_mrz);
    int rc = hgb::check_launch();
    if (rc) return rc;
    k_details_q<<<(unsigned)hgb::ceil_div(nqf, 64), 64, 0, st>>>(g, number, h2fdf, gwb_q, num_q);
    if ((rc = hgb::check_launch())) return rc;
    k_details_z<<<(unsigned)hgb::ceil_div(nzf, 128), 128, 0, st>>>(g, gwb_m, num_m, gwb_mrz, num_mrz, gwb_z, num_z,
                                                                   gwb_rz, num_rz);
    if ((rc = hgb::check_launch())) return rc;
    k_details_denom<<<(unsigned)hgb::ceil_div(n_freq, 64), 64, 0, st>>>(g, gwb_z, denom);
    if ((rc = hgb::check_launch())) return rc;
    double *rows[5] = {gwb_m, gwb_q, gwb_z, gwb_rz, gwb_mrz};
    const long sizes[5] = {(long)g.nm * nzf, (long)g.nq * nzf, nzf, nzf, (long)g.nm * nzf};
    for (int k = 0; k < 5; k++) {
        k_details_normalise<<<(unsigned)hgb::ceil_div(sizes[k], 256), 256, 0, st>>>(sizes[k], n_freq, denom, rows[k]);
        if ((rc = hgb::check_launch())) return rc;
    }
    return HGB_OK;
}

}  // extern "C"
