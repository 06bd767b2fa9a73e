// Cell integration and per-bin strain on the (M-1, Q-1, Z-1, F) bin grid (kernel k_cells):
//  * NUMBER: integrate_differential_number_3dx1d (holodeck/sams/sam_cyutils.pyx:115-216)
//  * STRAIN: char_strain_sq_from_bin_edges_redz (holodeck/gravwaves.py:694-724)
//  * both in one pass for gwb() (sam.py:930-935): each vertex of dnum and redz_final is read from
//    L1/L2 by the eight bins that share it, and number / h2fdf are written once.
// One block per (mtot, mrat) cell; its threads walk the (redz, frequency) elements with the
// frequency fastest, so the eight vertex loads of a warp are contiguous runs along the frequency
// axis.  Built with -fmad=false: the eight-vertex sum and the midpoints round like the Cython/numpy
// code; the strain product is regrouped (see cell_strain), which moves it by a few ulp.
#include <math.h>

#include "hgb_common.cuh"

namespace {

struct BinGeom {
    int nm, nq, nz, nf;   // edge counts of mtot, mrat, redz; number of frequencies
};

__device__ __forceinline__ long vtx(const BinGeom &g, int m, int q, int z, int f) {
    return (((long)m * g.nq + q) * g.nz + z) * g.nf + f;
}

// sam_cyutils.pyx:199-214
__device__ __forceinline__ double cell_number(const BinGeom &g, const double *dnum, int m, int q, int z, int f,
                                              const double *log10_mtot, const double *mrat, const double *redz,
                                              const double *dln_freq) {
    double dm = log10_mtot[m + 1] - log10_mtot[m];
    double dmdq = dm * (mrat[q + 1] - mrat[q]);
    double dmdqdz = dmdq * (redz[z + 1] - redz[z]);
    double temp = 0.0;
#pragma unroll
    for (int ii = 0; ii < 2; ii++)
#pragma unroll
        for (int jj = 0; jj < 2; jj++)
#pragma unroll
            for (int kk = 0; kk < 2; kk++) temp += dnum[vtx(g, m + ii, q + jj, z + kk, f)];
    return temp * dmdqdz * dln_freq[f] / 8.0;
}

struct StrainArgs {
    double gw_src_const;
    const double *dc_val, *dc_der;
    int dc_n;
    double dc_h;   // 1 / dc_n
};

// gravwaves.py:694-724 rearranged: hs = K mc (2 mc fr)^(2/3) / dc with fr = fc (1 + zbar) is evaluated
// as [K mc (2 mc)^(2/3)] [fc^(2/3)] [(1 + zbar)^(2/3)] / dc, the first factor once per (mtot, mrat)
// cell and the second once per frequency, so each (bin, frequency) costs one inverse cube root (an
// FP32 estimate and one FP64 Newton step) and the comoving-distance lookup.  The redshift midpoints are taken along mtot, then mrat, then redz.
__device__ __forceinline__ double cell_strain(const BinGeom &g, const double *rz, int m, int q, int z, int f,
                                              double amp_mq, double amp_f, double fc_df, const StrainArgs &s,
                                              int *d_status) {
    double r[2][2][2];
#pragma unroll
    for (int ii = 0; ii < 2; ii++)
#pragma unroll
        for (int jj = 0; jj < 2; jj++)
#pragma unroll
            for (int kk = 0; kk < 2; kk++) {
                double v = rz[vtx(g, m + ii, q + jj, z + kk, f)];
                if (v < 0.0 && v != -1.0) hgb::flag(d_status, HGB_STATUS_INVALID_REDSHIFT);
                r[ii][jj][kk] = v;
            }
    double a00 = 0.5 * (r[1][0][0] + r[0][0][0]);
    double a01 = 0.5 * (r[1][0][1] + r[0][0][1]);
    double a10 = 0.5 * (r[1][1][0] + r[0][1][0]);
    double a11 = 0.5 * (r[1][1][1] + r[0][1][1]);
    double b0 = 0.5 * (a10 + a00);
    double b1 = 0.5 * (a11 + a01);
    double zb = 0.5 * (b1 + b0);
    if (!(zb > 0.0)) return 0.0;   // +inf comoving distance: zero strain
    double dc = hgb::comoving_distance_fast(s.dc_val, s.dc_der, s.dc_n, s.dc_h, zb);
    double zp1 = 1.0 + zb;
    // (1 + z)^(2/3) = (1 + z) r with r = (1 + z)^(-1/3): FP32 start, one Newton step for the inverse
    // cube root, r (4 - y r^3) / 3, in FP64 (relative error about 1e-14; 1 + z lies in (1, 12));
    // 1 / dc likewise, q (2 - dc q) from an FP32 reciprocal
    const double r0 = (double)rcbrtf((float)zp1);
    const double r1 = r0 * (4.0 - zp1 * (r0 * r0 * r0)) * (1.0 / 3.0);
    const double q0 = (double)__frcp_rn((float)dc);
    const double q1 = q0 * (2.0 - dc * q0);
    double hs = amp_mq * amp_f * (zp1 * r1) * q1;
    return (hs * hs) * fc_df;
}

// One block per (mtot, mrat) bin cell; threads stride over its (redz, frequency) elements.
template <bool NUMBER, bool STRAIN>
__global__ void k_cells(BinGeom g, StrainArgs s, const double *__restrict__ mtot, const double *__restrict__ log10_mtot,
                        const double *__restrict__ mrat, const double *__restrict__ redz,
                        const double *__restrict__ fedges, const double *__restrict__ dln_freq,
                        const double *__restrict__ dnum, const double *__restrict__ redz_final,
                        double *__restrict__ number, double *__restrict__ h2fdf, int *d_status) {
    extern __shared__ double sm[];
    double *amp_f = sm;              // [nf] fc^(2/3)
    double *fc_df = sm + g.nf;       // [nf] fc / df
    __shared__ double amp_mq;
    const int cell = blockIdx.x;
    const int m = cell / (g.nq - 1), q = cell % (g.nq - 1);
    if (STRAIN) {
        for (int f = threadIdx.x; f < g.nf; f += blockDim.x) {
            double fc = 0.5 * (fedges[f + 1] + fedges[f]);
            double df = fedges[f + 1] - fedges[f];
            amp_f[f] = pow(fc, 2.0 / 3.0);
            fc_df[f] = fc / df;
        }
        if (threadIdx.x == 0) {
            double mt = 0.5 * (mtot[m + 1] + mtot[m]);
            double mr = 0.5 * (mrat[q + 1] + mrat[q]);
            double mc = mt * pow(mr, 3.0 / 5.0) / pow(1.0 + mr, 6.0 / 5.0);
            amp_mq = s.gw_src_const * mc * pow(2.0 * mc, 2.0 / 3.0);
        }
        __syncthreads();
    }
    const int nzf = (g.nz - 1) * g.nf;
    const long out0 = (long)cell * nzf;
    for (int e = threadIdx.x; e < nzf; e += blockDim.x) {
        int z = e / g.nf, f = e % g.nf;
        if (NUMBER) number[out0 + e] = cell_number(g, dnum, m, q, z, f, log10_mtot, mrat, redz, dln_freq);
        if (STRAIN) h2fdf[out0 + e] = cell_strain(g, redz_final, m, q, z, f, amp_mq, amp_f[f], fc_df[f], s, d_status);
    }
}

// ---- FP32 production mode of k_cells<true, true>
//
// The same quantities from the same FP64 arrays, with FP32 arithmetic (explicit fmaf only; the file
// is built without contraction).  Values enter and leave FP32 through the integer conversions of
// hgb_common.cuh.  Scaling keeps every intermediate a normal float:
//   hs = A_mq A_f (1 + zb)^(2/3) / d_C with A_mq = K mc (2 mc)^(2/3) / D_H per cell and A_f = fc^(2/3),
//   each stored as a mantissa in [1, 2) and a power-of-two exponent (ka, kf); d_C / D_H = (1 - u) g(u)
//   from the FP32 table of hgb_cosmo; h2fdf = (hs_s^2 fc/df) 2^(2 (ka + kf)), hs_s the product of the
//   mantissas.
struct StrainArgs32 {
    const float *g_val, *g_der;
    int n;
    float h;   // 1 / n
};

// d_C / D_H at z > 0: u = (1 + z)^(-1/2), 1 - u = z / (s (s + 1)) with s = sqrt(1 + z) (no cancellation
// as z -> 0), g(u) by cubic Hermite interpolation.
__device__ __forceinline__ float dc_over_dh_f32(const StrainArgs32 &s, float z) {
    const float sq = sqrtf(1.0f + z);
    const float u = __fdividef(1.0f, sq);
    const float w = __fdividef(z, sq * (sq + 1.0f));
    const float x = u * (float)s.n;
    int k = (int)x;
    if (k >= s.n) k = s.n - 1;
    if (k < 0) k = 0;
    const float t = x - (float)k;
    const float t2 = t * t, t3 = t2 * t;
    const float h00 = fmaf(2.0f, t3, fmaf(-3.0f, t2, 1.0f));
    const float h10 = fmaf(-2.0f, t2, t3) + t;
    const float h01 = fmaf(-2.0f, t3, 3.0f * t2);
    const float h11 = t3 - t2;
    const float gk = s.g_val[k], gk1 = s.g_val[k + 1];
    const float dk = s.g_der[k] * s.h, dk1 = s.g_der[k + 1] * s.h;
    const float g = fmaf(h00, gk, fmaf(h10, dk, fmaf(h01, gk1, h11 * dk1)));
    return w * g;
}

constexpr int F32_MAX_FREQ = 256;   // per-frequency terms staged in shared memory

__global__ void k_cells_f32(BinGeom g, StrainArgs32 s, double amp_scale, const double *__restrict__ mtot,
                            const double *__restrict__ log10_mtot, const double *__restrict__ mrat,
                            const double *__restrict__ redz, const double *__restrict__ fedges,
                            const double *__restrict__ dln_freq, const double *__restrict__ dnum,
                            const double *__restrict__ redz_final, double *__restrict__ number,
                            double *__restrict__ h2fdf, int *d_status) {
    __shared__ float s_amp_f[F32_MAX_FREQ], s_fcdf[F32_MAX_FREQ], s_dlnf[F32_MAX_FREQ];
    __shared__ int s_kf[F32_MAX_FREQ];
    extern __shared__ float s_vol[];   // [nz - 1] dlog10M dq dz / 8 of the cell's bins
    __shared__ float s_amp_mq;
    __shared__ int s_ka;
    const int cell = blockIdx.x;
    const int m = cell / (g.nq - 1), q = cell % (g.nq - 1);
    for (int f = threadIdx.x; f < g.nf; f += blockDim.x) {
        const double fc = 0.5 * (fedges[f + 1] + fedges[f]);
        const double df = fedges[f + 1] - fedges[f];
        const float af = powf(hgb::f64_to_f32_rz(fc), 2.0f / 3.0f);   // 1e-10 .. 1e-4 Hz: a normal float
        int kf;
        const float mant = 2.0f * frexpf(af, &kf);                // af = mant 2^(kf - 1), mant in [1, 2)
        s_amp_f[f] = mant;
        s_kf[f] = kf - 1;
        s_fcdf[f] = hgb::f64_to_f32_rz(fc) / hgb::f64_to_f32_rz(df);
        s_dlnf[f] = hgb::f64_to_f32_rz(dln_freq[f]);
    }
    const double dm = log10_mtot[m + 1] - log10_mtot[m];
    const double dmdq = dm * (mrat[q + 1] - mrat[q]);
    for (int z = threadIdx.x; z < g.nz - 1; z += blockDim.x)
        s_vol[z] = hgb::f64_to_f32_rz(dmdq * (redz[z + 1] - redz[z])) * 0.125f;
    if (threadIdx.x == 0) {
        // K mc (2 mc)^(2/3) = K 2^(2/3) mc^(5/3) with mc^(5/3) = mt^(5/3) mr / (1 + mr)^2 for the chirp
        // mass mc = mt mr^(3/5) / (1 + mr)^(6/5): one cube root instead of three powers on the one
        // thread the block waits for
        const double mt = 0.5 * (mtot[m + 1] + mtot[m]);
        const double mr = 0.5 * (mrat[q + 1] + mrat[q]);
        const double c = cbrt(mt), opq = 1.0 + mr;
        const double mc53 = mt * (c * c) * mr / (opq * opq);
        int ka;
        const double mant = 2.0 * frexp(amp_scale * 1.5874010519681994 * mc53, &ka);   // 2^(2/3)
        s_amp_mq = (float)mant;
        s_ka = ka - 1;
    }
    __syncthreads();
    const float amp_mq = s_amp_mq;
    const int ka = s_ka;
    const int nzf = (g.nz - 1) * g.nf;
    const long out0 = (long)cell * nzf;
    for (int e = threadIdx.x; e < nzf; e += blockDim.x) {
        const int z = e / g.nf, f = e % g.nf;
        // number: Kahan sum of the eight vertices (sam_cyutils.pyx:199-214)
        hgb::Kahan32 acc;
        long long rb[2][2][2];
#pragma unroll
        for (int ii = 0; ii < 2; ii++)
#pragma unroll
            for (int jj = 0; jj < 2; jj++)
#pragma unroll
                for (int kk = 0; kk < 2; kk++) {
                    const long v = vtx(g, m + ii, q + jj, z + kk, f);
                    acc.add(hgb::f64_to_f32_rz(dnum[v]));
                    rb[ii][jj][kk] = __double_as_longlong(redz_final[v]);
                }
        number[out0 + e] = hgb::f32_to_f64_scaled(acc.s * s_vol[z] * s_dlnf[f], 0);
        // strain (gravwaves.py:694-724)
        int n_sent = 0;
        bool bad = false;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const long long b = (&rb[0][0][0])[c];
            const bool sent = (b == hgb::F64_MINUS_ONE_BITS);
            n_sent += sent;
            const bool nan = ((b >> 52) & 0x7FF) == 0x7FF && (b & 0xFFFFFFFFFFFFFll);
            bad |= (b < 0) && !sent && !nan && (b != (long long)0x8000000000000000ull);   // < 0, not -1, -0, NaN
        }
        if (bad) hgb::flag(d_status, HGB_STATUS_INVALID_REDSHIFT);
        float zb = 0.0f;
        if (n_sent == 0) {   // all corners >= 0: the midpoints cannot cancel
            float r[2][2][2];
#pragma unroll
            for (int c = 0; c < 8; c++) (&r[0][0][0])[c] = hgb::f64_to_f32_rz(__longlong_as_double((&rb[0][0][0])[c]));
            const float b0 = (r[1][0][0] + r[0][0][0]) + (r[1][1][0] + r[0][1][0]);
            const float b1 = (r[1][0][1] + r[0][0][1]) + (r[1][1][1] + r[0][1][1]);
            zb = 0.125f * (b1 + b0);
        } else if (n_sent < 8) {   // the sentinel enters the mean: the reference's FP64 midpoints
            double r[2][2][2];
#pragma unroll
            for (int c = 0; c < 8; c++) (&r[0][0][0])[c] = __longlong_as_double((&rb[0][0][0])[c]);
            const double a00 = 0.5 * (r[1][0][0] + r[0][0][0]);
            const double a01 = 0.5 * (r[1][0][1] + r[0][0][1]);
            const double a10 = 0.5 * (r[1][1][0] + r[0][1][0]);
            const double a11 = 0.5 * (r[1][1][1] + r[0][1][1]);
            const double zd = 0.5 * (0.5 * (a11 + a01) + 0.5 * (a10 + a00));
            zb = (zd > 0.0) ? hgb::f64_to_f32_rz(zd) : 0.0f;
        }
        double out = 0.0;
        if (zb > 0.0f) {
            const float dc = dc_over_dh_f32(s, zb);
            const float zp1 = 1.0f + zb;
            const float zp23 = zp1 * rcbrtf(zp1);
            const float hs = __fdividef(amp_mq * s_amp_f[f] * zp23, dc);
            out = hgb::f32_to_f64_scaled(hs * hs * s_fcdf[f], 2 * (ka + s_kf[f]));
        }
        h2fdf[out0 + e] = out;
    }
}

// single_sources.py:117-143 on one (bin, frequency): the redshift midpoints (same order as
// cell_strain), -1 where not positive; comoving distance (+inf there); Kepler separation at the
// rest-frame orbital frequency; angular separation.  IEEE semantics give the reference's inf / NaN
// for the -1 bins.  Also records the largest finite magnitude of each grid (as a frexp exponent)
// over the bins with nonzero strain.
__global__ void k_param_grids(BinGeom g, const double *__restrict__ mt_cent, const double *__restrict__ fobs_cent,
                              const double *__restrict__ redz_final, double nwtg, StrainArgs s,
                              const double *__restrict__ h2fdf, double *__restrict__ rz_mid,
                              double *__restrict__ dcom, double *__restrict__ sepa, double *__restrict__ angs,
                              int *scale_log2) {
    const long nb = (long)(g.nm - 1) * (g.nq - 1) * (g.nz - 1);
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nb * g.nf) return;
    const int f = (int)(idx % g.nf);
    const long b = idx / g.nf;
    const int z = (int)(b % (g.nz - 1));
    const int q = (int)((b / (g.nz - 1)) % (g.nq - 1));
    const int m = (int)(b / ((long)(g.nz - 1) * (g.nq - 1)));
    double r[2][2][2];
#pragma unroll
    for (int ii = 0; ii < 2; ii++)
#pragma unroll
        for (int jj = 0; jj < 2; jj++)
#pragma unroll
            for (int kk = 0; kk < 2; kk++) r[ii][jj][kk] = redz_final[vtx(g, m + ii, q + jj, z + kk, f)];
    const double a00 = 0.5 * (r[1][0][0] + r[0][0][0]);
    const double a01 = 0.5 * (r[1][0][1] + r[0][0][1]);
    const double a10 = 0.5 * (r[1][1][0] + r[0][1][0]);
    const double a11 = 0.5 * (r[1][1][1] + r[0][1][1]);
    const double b0 = 0.5 * (a10 + a00);
    const double b1 = 0.5 * (a11 + a01);
    double zb = 0.5 * (b1 + b0);
    double dc = INFINITY;
    if (zb > 0.0) dc = hgb::comoving_distance(s.dc_val, s.dc_der, s.dc_n, zb);
    else zb = -1.0;
    const double frst = fobs_cent[f] * (1.0 + zb);
    const double w = 2.0 * HGB_PI * frst;
    const double sp = pow(nwtg * mt_cent[m] / (w * w), 1.0 / 3.0);
    const double an = sp / (dc / (1.0 + zb));
    rz_mid[idx] = zb;
    dcom[idx] = dc;
    sepa[idx] = sp;
    angs[idx] = an;
    if (scale_log2 && (!h2fdf || h2fdf[idx] != 0.0)) {
        const double v[4] = {zb, dc, sp, an};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (isfinite(v[k]) && v[k] != 0.0) {
                int e;
                frexp(v[k], &e);
                atomicMax(scale_log2 + k, e);
            }
        }
    }
}

}  // namespace

extern "C" {

int hgb_param_grids(const double *mt_cent, int n_mtot, int n_mrat, int n_redz, const double *fobs_orb_cent,
                    int n_freq, const double *redz_final, double nwtg, const hgb_cosmo *cosmo,
                    const double *h2fdf, double *redz_mid, double *dcom, double *sepa, double *angs,
                    int *scale_log2, void *stream) {
    HGB_CHECK_ARG(mt_cent && fobs_orb_cent && redz_final && cosmo && redz_mid && dcom && sepa && angs);
    HGB_CHECK_ARG(n_mtot >= 2 && n_mrat >= 2 && n_redz >= 2 && n_freq >= 1);
    HGB_CHECK_ARG(cosmo->dc_val && cosmo->dc_der && cosmo->dc_n >= 2);
    BinGeom g{n_mtot, n_mrat, n_redz, n_freq};
    StrainArgs s{0.0, cosmo->dc_val, cosmo->dc_der, cosmo->dc_n, 1.0 / cosmo->dc_n};
    cudaStream_t st = (cudaStream_t)stream;
    if (scale_log2) {
        cudaError_t err = cudaMemsetAsync(scale_log2, 0x80, 4 * sizeof(int), st);   // very negative
        if (err != cudaSuccess) {
            hgb::set_cuda_error(err);
            return HGB_ERR_CUDA;
        }
    }
    const long n = (long)(n_mtot - 1) * (n_mrat - 1) * (n_redz - 1) * n_freq;
    k_param_grids<<<(unsigned)hgb::ceil_div(n, 256), 256, 0, st>>>(g, mt_cent, fobs_orb_cent, redz_final, nwtg, s,
                                                                   h2fdf, redz_mid, dcom, sepa, angs, scale_log2);
    return hgb::check_launch();
}

int hgb_integrate_3dx1d(const double *log10_mtot, int n_mtot, const double *mrat, int n_mrat, const double *redz,
                        int n_redz, const double *dln_freq, int n_freq, const double *dnum, double *number,
                        void *stream) {
    HGB_CHECK_ARG(log10_mtot && mrat && redz && dln_freq && dnum && number);
    HGB_CHECK_ARG(n_mtot >= 2 && n_mrat >= 2 && n_redz >= 2 && n_freq >= 1);
    BinGeom g{n_mtot, n_mrat, n_redz, n_freq};
    StrainArgs s{0.0, nullptr, nullptr, 0, 0.0};
    unsigned cells = (unsigned)((n_mtot - 1) * (n_mrat - 1));
    k_cells<true, false><<<cells, 256, 0, (cudaStream_t)stream>>>(g, s, nullptr, log10_mtot, mrat, redz, nullptr,
                                                                  dln_freq, dnum, nullptr, number, nullptr, nullptr);
    return hgb::check_launch();
}

int hgb_char_strain_sq(const double *mtot, int n_mtot, const double *mrat, int n_mrat, int n_redz,
                       const double *fobs_orb_edges, int n_freq, const double *redz_final, double gw_src_const,
                       const hgb_cosmo *cosmo, double *h2fdf, int *d_status, void *stream) {
    HGB_CHECK_ARG(mtot && mrat && fobs_orb_edges && redz_final && cosmo && h2fdf);
    HGB_CHECK_ARG(n_mtot >= 2 && n_mrat >= 2 && n_redz >= 2 && n_freq >= 1);
    HGB_CHECK_ARG(cosmo->dc_val && cosmo->dc_der && cosmo->dc_n >= 2);
    BinGeom g{n_mtot, n_mrat, n_redz, n_freq};
    StrainArgs s{gw_src_const, cosmo->dc_val, cosmo->dc_der, cosmo->dc_n, 1.0 / cosmo->dc_n};
    unsigned cells = (unsigned)((n_mtot - 1) * (n_mrat - 1));
    size_t smem = sizeof(double) * 2 * n_freq;
    HGB_CHECK_ARG(smem <= 48 * 1024);
    k_cells<false, true><<<cells, 256, smem, (cudaStream_t)stream>>>(g, s, mtot, nullptr, mrat, nullptr, fobs_orb_edges,
                                                                     nullptr, nullptr, redz_final, nullptr, h2fdf,
                                                                     d_status);
    return hgb::check_launch();
}

int hgb_number_and_strain_f32(const double *mtot, const double *log10_mtot, int n_mtot, const double *mrat,
                              int n_mrat, const double *redz, int n_redz, const double *fobs_orb_edges,
                              const double *dln_freq, int n_freq, const double *dnum, const double *redz_final,
                              double gw_src_const, const hgb_cosmo *cosmo, double *number, double *h2fdf,
                              int *d_status, void *stream) {
    HGB_CHECK_ARG(mtot && log10_mtot && mrat && redz && fobs_orb_edges && dln_freq && dnum && redz_final);
    HGB_CHECK_ARG(cosmo && number && h2fdf);
    HGB_CHECK_ARG(n_mtot >= 2 && n_mrat >= 2 && n_redz >= 2 && n_freq >= 1 && n_freq <= F32_MAX_FREQ);
    HGB_CHECK_ARG(cosmo->dcg_val && cosmo->dcg_der && cosmo->dc_n >= 2 && cosmo->hubble_distance > 0.0);
    HGB_CHECK_ARG(gw_src_const > 0.0);
    BinGeom g{n_mtot, n_mrat, n_redz, n_freq};
    StrainArgs32 s{cosmo->dcg_val, cosmo->dcg_der, cosmo->dc_n, 1.0f / (float)cosmo->dc_n};
    unsigned cells = (unsigned)((n_mtot - 1) * (n_mrat - 1));
    size_t smem = sizeof(float) * (size_t)(n_redz - 1);
    HGB_CHECK_ARG(smem <= 32 * 1024);
    k_cells_f32<<<cells, 256, smem, (cudaStream_t)stream>>>(g, s, gw_src_const / cosmo->hubble_distance, mtot,
                                                             log10_mtot, mrat, redz, fobs_orb_edges, dln_freq, dnum,
                                                             redz_final, number, h2fdf, d_status);
    return hgb::check_launch();
}

int hgb_number_and_strain(const double *mtot, const double *log10_mtot, int n_mtot, const double *mrat, int n_mrat,
                          const double *redz, int n_redz, const double *fobs_orb_edges, const double *dln_freq,
                          int n_freq, const double *dnum, const double *redz_final, double gw_src_const,
                          const hgb_cosmo *cosmo, double *number, double *h2fdf, int *d_status, void *stream) {
    HGB_CHECK_ARG(mtot && log10_mtot && mrat && redz && fobs_orb_edges && dln_freq && dnum && redz_final);
    HGB_CHECK_ARG(cosmo && number && h2fdf);
    HGB_CHECK_ARG(n_mtot >= 2 && n_mrat >= 2 && n_redz >= 2 && n_freq >= 1);
    HGB_CHECK_ARG(cosmo->dc_val && cosmo->dc_der && cosmo->dc_n >= 2);
    BinGeom g{n_mtot, n_mrat, n_redz, n_freq};
    StrainArgs s{gw_src_const, cosmo->dc_val, cosmo->dc_der, cosmo->dc_n, 1.0 / cosmo->dc_n};
    unsigned cells = (unsigned)((n_mtot - 1) * (n_mrat - 1));
    size_t smem = sizeof(double) * 2 * n_freq;
    HGB_CHECK_ARG(smem <= 48 * 1024);
    k_cells<true, true><<<cells, 256, smem, (cudaStream_t)stream>>>(g, s, mtot, log10_mtot, mrat, redz, fobs_orb_edges,
                                                                    dln_freq, dnum, redz_final, number, h2fdf, d_status);
    return hgb::check_launch();
}

}  // extern "C"
