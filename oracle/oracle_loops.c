/*
 * CPU oracle for the SAM gravitational-wave-background path: the loop-heavy
 * stages restated in plain C.  TEST INFRASTRUCTURE ONLY: used by tests/,
 * __graft_entry__.smoke() and the CPU-baseline legs of bench.py as the
 * checker; never by the holodeck_gb300 product path.
 *
 * Each function follows the named holodeck file:line and keeps its loop order
 * and floating-point operation order.  Build with -ffp-contract=off so that
 * no multiply-add is fused (the reference wheels for x86-64 do not fuse).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

/* constants hard-coded in holodeck/sams/sam_cyutils.pyx:30-42 */
static const double MY_NWTG = 6.6742999e-08;
static const double MY_SPLC = 29979245800.0;
static const double MY_MPC = 3.08567758e+24;
static const double MY_SCHW = 1.4852320538237328e-28;

static double gw_dadt_sep_const(void) { return -64.0 * pow(MY_NWTG, 3) / 5.0 / pow(MY_SPLC, 5); }
static double kepler_const_freq(void) { return (1.0 / (2.0 * M_PI)) * sqrt(MY_NWTG); }
static double kepler_const_sepa(void) { return pow(MY_NWTG, 1.0 / 3.0) / pow(2.0 * M_PI, 2.0 / 3.0); }
static double four_pi_splc_over_mpc(void) { return 4 * M_PI * MY_SPLC / MY_MPC; }

/* sam_cyutils.pyx:46-49 */
static double hard_gw(double mtot, double mrat, double sepa) {
    return gw_dadt_sep_const() * pow(mtot, 3) * mrat / pow(sepa, 3) / pow(1 + mrat, 2);
}

/* sam_cyutils.pyx:52-61 */
static double kepler_freq_from_sepa(double mtot, double sepa) {
    return kepler_const_freq() * sqrt(mtot) / pow(sepa, 1.5);
}
static double kepler_sepa_from_freq(double mtot, double freq) {
    return kepler_const_sepa() * pow(mtot, 1.0 / 3.0) / pow(freq, 2.0 / 3.0);
}

/* sam_cyutils.pyx:66-107: bracket walkers for monotone tables */
static int while_while_increasing(int start, int size, double val, const double *edges) {
    int index = start;
    while ((index < size - 2) && (edges[index + 1] < val)) index += 1;
    while ((index > 0) && (edges[index] > val)) index -= 1;
    return index;
}
static int while_while_decreasing(int start, int size, double val, const double *edges) {
    int index = start;
    while ((index < size - 1) && (edges[index + 1] > val)) index += 1;
    while ((index > 0) && (edges[index - 1] < val)) index -= 1;
    return index;
}

/* holodeck/cyutils.pyx:326-358 */
static double interp_between(double xnew, double xl, double xr, double yl, double yr) {
    return yl + (yr - yl) * (xnew - xl) / (xr - xl);
}
static double interp_at_index(int idx, double xnew, const double *xold, const double *yold) {
    return interp_between(xnew, xold[idx], xold[idx + 1], yold[idx], yold[idx + 1]);
}

/* sam_cyutils.pyx:240-253 */
static double hard_func_2pwl(double norm, double xx, double gi, double go) {
    return -norm * pow(1.0 + xx, -go + gi) / pow(xx, gi - 1);
}
static double hard_func_2pwl_gw(double mt, double mr, double sepa, double norm, double rchar, double gi, double go) {
    double dadt = hard_func_2pwl(norm, sepa / rchar, gi, go);
    dadt += hard_gw(mt, mr, sepa);
    return dadt;
}

/* sam_cyutils.pyx:360-398: trapezoid lifetime minus the target time */
double orc_lifetime_2pwl(double norm_log10, double target_time, double mt, double mr, double sepa_init,
                         double rchar, double gi, double go, int nsteps) {
    double risco_log10 = log10(3.0 * MY_SCHW * mt);
    double sepa_log10 = log10(sepa_init);
    double norm = pow(10.0, norm_log10);
    double dx = (sepa_log10 - risco_log10) / nsteps;
    double time = 0.0;
    double sepa_left = pow(10.0, sepa_log10);
    double dadt_left = hard_func_2pwl_gw(mt, mr, sepa_left, norm, rchar, gi, go);
    for (int ii = 0; ii < nsteps; ii++) {
        sepa_log10 -= dx;
        double sepa_right = pow(10.0, sepa_log10);
        double dadt_right = hard_func_2pwl_gw(mt, mr, sepa_right, norm, rchar, gi, go);
        double dt = 2.0 * (sepa_right - sepa_left) / (dadt_left + dadt_right);
        time += dt;
        sepa_left = sepa_right;
        dadt_left = dadt_right;
    }
    return time - target_time;
}

/* hard_func_2pwl_gw on flat arrays (sam_cyutils.pyx:256-286) */
void orc_hard_func_2pwl_gw(int n, const double *mt, const double *mr, const double *sepa, const double *norm,
                           double rchar, double gi, double go, double *out) {
    for (int i = 0; i < n; i++) out[i] = hard_func_2pwl_gw(mt[i], mr[i], sepa[i], norm[i], rchar, gi, go);
}

/* sam_cyutils.pyx:170-216 */
void orc_integrate_3dx1d(const double *log10_mtot, int n_mtot, const double *mrat, int n_mrat,
                         const double *redz, int n_redz, const double *dln_freq, int n_freq,
                         const double *dnum, double *numb) {
    const long sM = (long)n_mrat * n_redz * n_freq, sQ = (long)n_redz * n_freq, sZ = n_freq;
    const long oM = (long)(n_mrat - 1) * (n_redz - 1) * n_freq, oQ = (long)(n_redz - 1) * n_freq, oZ = n_freq;
    for (int mm = 0; mm < n_mtot - 1; mm++) {
        double dm = log10_mtot[mm + 1] - log10_mtot[mm];
        for (int qq = 0; qq < n_mrat - 1; qq++) {
            double dmdq = dm * (mrat[qq + 1] - mrat[qq]);
            for (int zz = 0; zz < n_redz - 1; zz++) {
                double dmdqdz = dmdq * (redz[zz + 1] - redz[zz]);
                for (int ff = 0; ff < n_freq; ff++) {
                    double temp = 0.0;
                    for (int ii = 0; ii < 2; ii++)
                        for (int jj = 0; jj < 2; jj++)
                            for (int kk = 0; kk < 2; kk++)
                                temp += dnum[(mm + ii) * sM + (qq + jj) * sQ + (zz + kk) * sZ + ff];
                    numb[mm * oM + qq * oQ + zz * oZ + ff] = temp * dmdqdz * dln_freq[ff] / 8.0;
                }
            }
        }
    }
}

/* sam_cyutils.pyx:510-781: differential number with the two-power-law hardening model.
 * redz_final must be pre-filled with -1 and diff_num with 0 (sam_cyutils.pyx:459-460). */
int orc_dbn_2pwl(const double *target_fobs_orb, int n_freq, double sepa_init, int num_steps,
                 const double *hard_norm, double hard_rchar, double gi, double go,
                 const double *nden, const double *mtot, int n_mtot, const double *mrat, int n_mrat,
                 const double *redz, int n_redz, const double *gmt_time,
                 const double *zgrid, const double *dcgrid, const double *agegrid, int n_interp,
                 double *redz_final, double *diff_num) {
    double age_universe = agegrid[n_interp - 1];
    double sepa_init_log10 = log10(sepa_init);
    double *redz_age = (double *)malloc(sizeof(double) * n_redz);
    if (!redz_age) return -1;
    int ii = 0;
    for (int kk = 0; kk < n_redz; kk++) {
        int rev = n_redz - 1 - kk;
        while ((zgrid[ii + 1] > redz[rev]) && (ii < n_interp - 1)) ii += 1;
        redz_age[rev] = interp_at_index(ii, redz[rev], zgrid, agegrid);
    }
    const long sQ = (long)n_redz * n_freq;
    const long sM = (long)n_mrat * sQ;
    for (ii = 0; ii < n_mtot; ii++) {
        double mt = mtot[ii];
        double risco = 3.0 * MY_SCHW * mt;
        double dx = (sepa_init_log10 - log10(risco)) / num_steps;
        for (int jj = 0; jj < n_mrat; jj++) {
            double mr = mrat[jj];
            double sepa_log10 = sepa_init_log10;
            double norm = hard_norm[ii * n_mrat + jj];
            double sepa_left = pow(10.0, sepa_log10);
            double dadt_left = hard_func_2pwl_gw(mt, mr, sepa_left, norm, hard_rchar, gi, go);
            double frst_orb_left = kepler_freq_from_sepa(mt, sepa_left);
            double time_evo = 0.0;
            int interp_left_idx = 0;
            for (int step = 0; step < num_steps; step++) {
                sepa_log10 -= dx;
                double sepa_right = pow(10.0, sepa_log10);
                double frst_orb_right = kepler_freq_from_sepa(mt, sepa_right);
                double dadt_right = hard_func_2pwl_gw(mt, mr, sepa_right, norm, hard_rchar, gi, go);
                double dt = 2.0 * (sepa_right - sepa_left) / (dadt_left + dadt_right);
                time_evo += dt;
                for (int kk = n_redz - 1; kk > -1; kk--) {
                    long base = ii * sM + jj * sQ + (long)kk * n_freq;
                    double gmt = gmt_time[(ii * n_mrat + jj) * (long)n_redz + kk];
                    double time_right = time_evo + gmt + redz_age[kk];
                    double time_left = time_right - dt;
                    if (time_left > age_universe) continue;
                    interp_left_idx = while_while_increasing(interp_left_idx, n_interp, time_left, agegrid);
                    double redz_left = interp_at_index(interp_left_idx, time_left, agegrid, zgrid);
                    if (redz_left < 0.0) continue;
                    int interp_right_idx = while_while_increasing(interp_left_idx, n_interp, time_right, agegrid);
                    double redz_right = interp_at_index(interp_right_idx, time_right, agegrid, zgrid);
                    if (redz_right < 0.0) redz_right = 0.0;
                    double fobs_orb_left = frst_orb_left / (1.0 + redz_left);
                    double fobs_orb_right = frst_orb_right / (1.0 + redz_right);
                    for (int ff = 0; ff < n_freq; ff++) {
                        double ftarget = target_fobs_orb[ff];
                        if ((ftarget < fobs_orb_left) || (fobs_orb_right < ftarget)) continue;
                        double new_time = interp_between(ftarget, fobs_orb_left, fobs_orb_right, time_left, time_right);
                        if (new_time > agegrid[n_interp - 1]) break;
                        int new_idx = while_while_increasing(interp_left_idx, n_interp, new_time, agegrid);
                        double new_redz = interp_at_index(new_idx, new_time, agegrid, zgrid);
                        double dcom = interp_at_index(new_idx, new_time, agegrid, dcgrid);
                        redz_final[base + ff] = new_redz;
                        double target_frst_orb = ftarget * (1.0 + new_redz);
                        double sepa = kepler_sepa_from_freq(mt, target_frst_orb);
                        double dadt = hard_func_2pwl_gw(mt, mr, sepa, norm, hard_rchar, gi, go);
                        double tres = -(2.0 / 3.0) * sepa / dadt;
                        double cosmo_fact = four_pi_splc_over_mpc() * (1.0 + new_redz) * pow(dcom / MY_MPC, 2);
                        diff_num[base + ff] = nden[(ii * n_mrat + jj) * (long)n_redz + kk] * tres * cosmo_fact;
                    }
                }
                dadt_left = dadt_right;
                sepa_left = sepa_right;
                frst_orb_left = frst_orb_right;
            }
        }
    }
    free(redz_age);
    return 0;
}

/* sam_cyutils.pyx:788-899: differential number under GW-only hardening.
 * redz_final must be pre-filled with -1 and diff_num with 0. */
int orc_dbn_gw(const double *target_fobs_orb, int n_freq, const double *nden, const double *mtot, int n_mtot,
               const double *mrat, int n_mrat, int n_redz, const double *redz_prime,
               const double *zgrid, const double *dcgrid, int n_interp,
               double *redz_final, double *diff_num) {
    const long sQ = (long)n_redz * n_freq;
    const long sM = (long)n_mrat * sQ;
    for (int ii = 0; ii < n_mtot; ii++) {
        double mt = mtot[ii];
        double rad_isco = 3.0 * MY_SCHW * mt;
        double frst_orb_isco = kepler_freq_from_sepa(mt, rad_isco);
        for (int jj = 0; jj < n_mrat; jj++) {
            double mr = mrat[jj];
            int interp_idx = 0;
            for (int _kk = 0; _kk < n_redz; _kk++) {
                int kk = n_redz - 1 - _kk;
                double rzp = redz_prime[(ii * n_mrat + jj) * (long)n_redz + kk];
                if (rzp <= 0.0) continue;
                long base = ii * sM + jj * sQ + (long)kk * n_freq;
                for (int ff = 0; ff < n_freq; ff++) {
                    redz_final[base + ff] = rzp;
                    double ftarget = target_fobs_orb[ff];
                    double target_frst_orb = ftarget * (1.0 + rzp);
                    if (target_frst_orb > frst_orb_isco) {
                        for (int fp = ff + 1; fp < n_freq; fp++) redz_final[base + fp] = rzp;
                        break;
                    }
                    interp_idx = while_while_decreasing(interp_idx, n_interp, rzp, zgrid);
                    double dcom = interp_at_index(interp_idx, rzp, zgrid, dcgrid);
                    double sepa = kepler_sepa_from_freq(mt, target_frst_orb);
                    double dadt = hard_gw(mt, mr, sepa);
                    double tres = -(2.0 / 3.0) * sepa / dadt;
                    double cosmo_fact = four_pi_splc_over_mpc() * (1.0 + rzp) * pow(dcom / MY_MPC, 2);
                    diff_num[base + ff] = nden[(ii * n_mrat + jj) * (long)n_redz + kk] * tres * cosmo_fact;
                }
            }
        }
    }
    return 0;
}

/* holodeck/cyutils.pyx:1328-1344, one (realization, frequency) pass: `num` holds the
 * drawn counts of the bins in loudest-first order, `h2fdf` their strain terms. */
void orc_fill_loudest(int nbins, const double *h2fdf_sorted, const double *num_sorted, int nloud,
                      double *hc2ss, double *hc2bg) {
    int ll = 0;
    double sum = 0;
    for (int bb = 0; bb < nbins; bb++) {
        double num = num_sorted[bb];
        if (num < 1) continue;
        double cur = h2fdf_sorted[bb];
        while ((ll < nloud) && (num > 0)) {
            hc2ss[ll] = cur;
            num -= 1;
            ll += 1;
        }
        sum += num * cur;
    }
    *hc2bg = sum;
}

/* holodeck/cyutils.pyx:875-895: accumulate one bin of the second-pass GWB, `num` holding
 * its R draws; gwb is (F, R) */
void orc_poisson_gwb_bin(int nreals, int ff, const double *num, double bin_hc2, double *gwb) {
    for (int rr = 0; rr < nreals; rr++) gwb[(long)ff * nreals + rr] += num[rr] * bin_hc2;
}

/* holodeck/cyutils.pyx:1700-1770 (_loudest_hc_and_par_from_sorted_redz), one (realization,
 * frequency): bins in loudest-first order, `num_sorted` the draws, `par_sorted` the bin's
 * parameters [7][nbins] (mt, mr, rz, redz_final, dcom_final, sepa, angs).  Writes hc2ss[nloud],
 * sspar[4][nloud] (stride ss_stride between parameters), hc2bg and bgpar[7] (stride bg_stride). */
void orc_fill_loudest_par(int nbins, const double *h2fdf_sorted, const double *num_sorted, const double *par_sorted,
                          int nloud, double *hc2ss, double *sspar, long ss_stride, double *hc2bg, double *bgpar,
                          long bg_stride) {
    int ll = 0;
    double sum_bg = 0, wsum[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int bb = 0; bb < nbins; bb++) {
        double num = num_sorted[bb];
        double cur = h2fdf_sorted[bb];
        if ((num < 1) || (cur == 0)) continue;
        while ((ll < nloud) && (num > 0)) {
            hc2ss[ll] = cur;
            for (int k = 0; k < 4; k++) sspar[k * ss_stride + ll] = par_sorted[(long)k * nbins + bb];
            num -= 1;
            ll += 1;
        }
        sum_bg += num * cur;
        for (int k = 0; k < 7; k++) wsum[k] += num * cur * par_sorted[(long)k * nbins + bb];
    }
    *hc2bg = sum_bg;
    for (int k = 0; k < 7; k++) bgpar[k * bg_stride] = wsum[k] / sum_bg;
}
