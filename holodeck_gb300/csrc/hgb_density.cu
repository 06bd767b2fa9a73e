// Static binary density on the (mtot, mrat, redz) grid edges: one thread per grid point.
//
// Follows Semi_Analytic_Model.static_binary_density (holodeck/sams/sam.py:280-398) with
// mass_stellar (sam.py:250-278), the GSMF / GPF / GMT / GMR components
// (holodeck/sams/components.py) and the M-Mbulge relation (holodeck/host_relations.py),
// keeping numpy's operation order.  Built with -fmad=false so that no multiply-add is fused.
#include "hgb_common.cuh"

#define HGB_MSOL 1.988409870698051e+33
#define HGB_LN10 2.302585092994046

namespace {

using hgb::flag;

struct CosmoScalars {
    double H0, Om0, Ode0, age_pref, age_c1, tz_c2, age_limit;
};

// host_relations.py:768-771 -> _log10_relation_reverse (:1137-1178) -> BF_Constant (:190-192)
__device__ __forceinline__ double mstar_from_mbh(const hgb_sam_model &m, double mbh) {
    double xx = log10(mbh / m.mmb[0]);
    xx = (1.0 / m.mmb[1]) * xx;
    double mbulge = m.mmb[2] * pow(10.0, xx);
    return mbulge / m.mmb[3];
}

// host_relations.py:483-512 with MMBulge_Standard.dmbulge_dmbh (:718-741)
__device__ __forceinline__ double dmstar_dmbh(const hgb_sam_model &m, double mstar) {
    double mbulge = mstar * m.mmb[3];
    double dmstar_dmbulge = 1.0 / m.mmb[3];
    double yy = log10(mbulge / m.mmb[2]) * m.mmb[1];
    double mbh = m.mmb[0] * pow(10.0, yy);
    double deriv = mbulge / (m.mmb[1] * mbh);
    return dmstar_dmbulge * deriv;
}

// components.py:132-172 (single) and :229-330 (double Schechter)
__device__ __forceinline__ double gsmf(const hgb_sam_model &m, double mstar, double z) {
    const double *g = m.gsmf;
    if (m.gsmf_kind == HGB_GSMF_SCHECHTER) {
        double phi = pow(10.0, g[0] + g[1] * z);
        double mchar = g[2] + g[3] * z;
        double alpha = g[4] + g[5] * z;
        double xx = mstar / mchar;
        return HGB_LN10 * phi * pow(xx, 1.0 + alpha) * exp(-xx);
    }
    double z2 = z * z;
    double mchar = HGB_MSOL * pow(10.0, g[6] + g[7] * z + g[8] * z2);
    double xx = mstar / mchar;
    double phi1 = pow(10.0, g[0] + g[1] * z + g[2] * z2);
    double phi2 = pow(10.0, g[3] + g[4] * z + g[5] * z2);
    double v1 = HGB_LN10 * phi1 * pow(xx, 1.0 + g[9]) * exp(-xx);
    double v2 = HGB_LN10 * phi2 * pow(xx, 1.0 + g[10]) * exp(-xx);
    return v1 + v2;
}

// components.py:443-483
__device__ __forceinline__ double gmr(const hgb_sam_model &m, double mtot, double mrat, double z) {
    const double *p = m.gmr;
    double zp1 = 1.0 + z;
    double norm = p[0] * pow(zp1, p[1]);
    double malpha = p[2] * pow(zp1, p[3]);
    double mdelta = p[4] * pow(zp1, p[5]);
    double qgamma = p[6] * pow(zp1, p[7]);
    qgamma = qgamma + p[8] * log10(mtot / p[10]);
    double xx = mtot / p[10];
    double mt = pow(xx, malpha);
    double yy = mtot / p[9];
    double mp1t = pow(1.0 + yy, mdelta);
    double qt = pow(mrat, qgamma);
    return norm * mt * mp1t * qt;
}

// One block per (mtot, run of up to DQ mrat) cell group.  The terms that depend only on (mtot, mrat)
// -- the stellar masses, the mass parts of the GPF and GMT power laws, the final mass factor -- and
// those that depend only on redz -- phi, M_char and alpha of the GSMF, the redshift parts of the
// power laws, the age and dt/dz -- are evaluated once per block with one lane per value (on this
// GPU an FP64 warp instruction costs the same with one lane as with 32), then every (mrat, redz)
// point of the group combines them.  Each term and each product keeps numpy's operation order, so
// the results equal the point-by-point evaluation bit for bit.
constexpr int DQ = 16;   // mrat values per block
constexpr int NMQ = 8;   // per-(mtot, mrat) terms
constexpr int NZT = 8;   // per-redz terms

__global__ void k_static_density(hgb_sam_model model, CosmoScalars cs, const double *__restrict__ mtot, int nm,
                                 const double *__restrict__ mrat, int nq, const double *__restrict__ redz, int nz,
                                 double *__restrict__ dens_out, double *__restrict__ gmt_out,
                                 double *__restrict__ zprime_out) {
    extern __shared__ double sm[];
    double *mq = sm;               // [NMQ][DQ]
    double *zt = sm + NMQ * DQ;    // [NZT][nz]
    const int ii = blockIdx.y, q0 = blockIdx.x * DQ;
    const int nqb = min(DQ, nq - q0);
    const int t = threadIdx.x;
    const double mt = mtot[ii];
    // per (mtot, mrat): sam.py:250-278 and sam.py:355-365
    if (t < nqb) {
        const double mr = mrat[q0 + t];
        double m1 = mt / (1.0 + mr);
        double m2 = mt - m1;
        double mstar_pri = mstar_from_mbh(model, m1);
        double mstar_sec = mstar_from_mbh(model, m2);
        double mstar_rat = mstar_sec / mstar_pri;
        double mstar_tot = mstar_pri + mstar_sec;
        double mplaw = model.mmb[1];
        double dqbh_dqgal = mplaw * pow(mstar_rat, mplaw - 1.0);
        double dmstar_dmbh_pri = dmstar_dmbh(model, mstar_pri);
        double qterm = (1.0 + mstar_rat) / (1.0 + mr);
        mq[0 * DQ + t] = mstar_pri;
        mq[1 * DQ + t] = mstar_tot;
        mq[2 * DQ + t] = mstar_rat;
        mq[3 * DQ + t] = (mt / mstar_tot) * (dmstar_dmbh_pri * qterm / dqbh_dqgal);
        if (model.use_gmt) {   // components.py:646-675: p0 (mass/p1)^p2 and q^p4 of p0 A B C
            const double *p = model.gmt;
            double mass_gmt = model.gmt_uses_mtot ? mstar_tot : mstar_pri;
            mq[4 * DQ + t] = p[0] * pow(mass_gmt / p[1], p[2]);
            mq[5 * DQ + t] = pow(mstar_rat, p[4]);
        }
        if (model.rate_kind == HGB_RATE_GPF_GMT) {   // components.py:556-586, the same form
            const double *p = model.gpf;
            double mass_gpf = model.gpf_uses_mtot ? mstar_tot : mstar_pri;
            mq[6 * DQ + t] = p[0] * pow(mass_gpf / p[1], p[2]);
            mq[7 * DQ + t] = pow(mstar_rat, p[4]);
        }
    }
    // per redz
    for (int k = t; k < nz; k += blockDim.x) {
        const double z = redz[k];
        const double zp1 = 1.0 + z;
        zt[0 * nz + k] = 1.0 / (cs.H0 * zp1 * sqrt(cs.Om0 * pow(zp1, 3.0) + cs.Ode0));   // dt/dz
        if (model.use_gmt) {
            zt[1 * nz + k] = pow(1.0 + z, model.gmt[3]);
            zt[2 * nz + k] = cs.age_pref * asinh(cs.age_c1 * pow(1.0 + z, -1.5));   // age
        }
        if (model.rate_kind == HGB_RATE_GPF_GMT) zt[3 * nz + k] = pow(1.0 + z, model.gpf[3]);
        if (model.gsmf_kind == HGB_GSMF_SCHECHTER) {   // components.py:132-172
            const double *g = model.gsmf;
            zt[4 * nz + k] = HGB_LN10 * pow(10.0, g[0] + g[1] * z);   // ln10 phi
            zt[5 * nz + k] = g[2] + g[3] * z;                          // M_char
            zt[6 * nz + k] = 1.0 + (g[4] + g[5] * z);                  // 1 + alpha
        }
    }
    __syncthreads();
    const int np = nqb * nz;
    for (int e = t; e < np; e += blockDim.x) {
        const int jq = e / nz, kk = e % nz;
        const long idx = ((long)ii * nq + (q0 + jq)) * nz + kk;
        const double z = redz[kk];
        const double mstar_pri = mq[0 * DQ + jq], mstar_tot = mq[1 * DQ + jq], mstar_rat = mq[2 * DQ + jq];
        double mass_gsmf = model.gsmf_uses_mtot ? mstar_tot : mstar_pri;
        double gmt_time = 0.0;
        if (model.use_gmt) {
            gmt_time = mq[4 * DQ + jq] * zt[1 * nz + kk] * mq[5 * DQ + jq];
            // utils.py:1772-1808 with the closed-form age / inverse age of the cosmology
            double new_age = zt[2 * nz + kk] + gmt_time;
            double zp = -1.0;
            if (new_age < cs.age_limit) zp = pow(cs.age_c1 / sinh(cs.tz_c2 * new_age), 2.0 / 3.0) - 1.0;
            gmt_out[idx] = gmt_time;
            zprime_out[idx] = zp;
        }
        double rate;
        if (model.rate_kind == HGB_RATE_GPF_GMT) {
            double rv = mq[6 * DQ + jq] * zt[3 * nz + kk] * mq[7 * DQ + jq];
            rv = (rv > model.gpf[5]) ? model.gpf[5] : rv;
            rate = rv / gmt_time;
        } else {
            rate = gmr(model, mstar_tot, mstar_rat, z);
        }
        double g;
        if (model.gsmf_kind == HGB_GSMF_SCHECHTER) {
            double xx = mass_gsmf / zt[5 * nz + kk];
            g = zt[4 * nz + kk] * pow(xx, zt[6 * nz + kk]) * exp(-xx);
        } else {
            g = gsmf(model, mass_gsmf, z);
        }
        double dens = g * rate * zt[0 * nz + kk];
        dens_out[idx] = dens * mq[3 * DQ + jq];
    }
}

__global__ void k_zero_stalled(double *__restrict__ dens, const double *__restrict__ zprime, long n) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n && zprime[idx] < 0.0) dens[idx] = 0.0;
}

}  // namespace

extern "C" {

int hgb_static_density(const hgb_sam_model *model, const hgb_cosmo *cosmo, const double *mtot, int n_mtot,
                       const double *mrat, int n_mrat, const double *redz, int n_redz, double *density,
                       double *gmt_time, double *redz_prime, int *d_status, void *stream) {
    (void)d_status;
    HGB_CHECK_ARG(model && cosmo && mtot && mrat && redz && density);
    HGB_CHECK_ARG(n_mtot > 0 && n_mrat > 0 && n_redz > 0);
    HGB_CHECK_ARG(model->gsmf_kind == HGB_GSMF_SCHECHTER || model->gsmf_kind == HGB_GSMF_DOUBLE_SCHECHTER);
    HGB_CHECK_ARG(model->rate_kind == HGB_RATE_GPF_GMT || model->rate_kind == HGB_RATE_GMR);
    HGB_CHECK_ARG(model->rate_kind == HGB_RATE_GMR || model->use_gmt);
    HGB_CHECK_ARG(!model->use_gmt || (gmt_time && redz_prime));
    CosmoScalars cs{cosmo->H0, cosmo->Om0, cosmo->Ode0, cosmo->age_pref, cosmo->age_c1, cosmo->tz_c2,
                    cosmo->age_limit};
    const size_t smem = sizeof(double) * ((size_t)NMQ * DQ + (size_t)NZT * n_redz);
    HGB_CHECK_ARG(smem <= 48 * 1024);
    dim3 grid((unsigned)hgb::ceil_div(n_mrat, DQ), (unsigned)n_mtot);
    k_static_density<<<grid, 256, smem, (cudaStream_t)stream>>>(*model, cs, mtot, n_mtot, mrat, n_mrat, redz, n_redz,
                                                                density, gmt_time, redz_prime);
    return hgb::check_launch();
}

int hgb_zero_stalled(double *density, const double *redz_prime, long n, void *stream) {
    HGB_CHECK_ARG(density && redz_prime && n >= 0);
    if (n == 0) return HGB_OK;
    int threads = 256;
    k_zero_stalled<<<(unsigned)hgb::ceil_div(n, threads), threads, 0, (cudaStream_t)stream>>>(density, redz_prime,
                                                                                               n);
    return hgb::check_launch();
}

}  // extern "C"
