// Binary hardening on the GPU:
//  * hgb_find_2pwl_hardening_norm: Brent root of the two-power-law lifetime per (mtot, mrat) cell
//    (holodeck/sams/sam_cyutils.pyx:289-398); one warp per cell.
//  * hgb_dbn_2pwl: differential binary number for Fixed_Time_2PL_SAM (sam_cyutils.pyx:510-781) in
//    two phases: k_dbn_2pwl walks the separation steps (one block per (mtot, mrat) cell, one thread
//    per starting redshift, step tables in shared memory) and records, per target frequency, the
//    interpolated time of the bracketing step; k_dbn_2pwl_eval then evaluates redshift, distance,
//    residence time and number for every bracketed (redz, frequency) element in parallel, with the
//    model's (half-)integer exponents taken as products and square roots instead of pow().  The
//    age -> redshift / distance interpolations use per-interval slopes computed once per block
//    (a multiply instead of a divide per lookup; results differ from the reference's divide by an ulp).
//  * hgb_dbn_gw: differential binary number for Hard_GW (sam_cyutils.pyx:788-899); one thread per
//    grid point.
// FP64 throughout (the hardening integral and the lookback-time -> redshift inversion are the
// FP64 islands of the path).  Built with -fmad=false so operation order and rounding follow the
// reference loops; the remaining differences are the last-ulp behaviour of pow/log10.
#include <math.h>

#include <algorithm>

#include "hgb_common.cuh"

namespace {

using hgb::CyConst;

constexpr double NORM_LOG10_LO = -20.0;
constexpr double NORM_LOG10_HI = +20.0;
constexpr double BRENT_XTOL = 1e-3;
constexpr double BRENT_RTOL = 1e-5;
constexpr int BRENT_MAXITER = 100;

// ------------------------------------------------------------------------------------------------
// hardening normalisation
// ------------------------------------------------------------------------------------------------

struct PowPlan {
    int kind;   // 0: pow(), 1: integer, 2: half-integer
    int n;      // |y| rounded down
    int neg;    // y < 0
};

struct NormArgs {
    double target_time, sepa_init_log10, rchar, gi, go;
    int nsteps;
    PowPlan p_outer, p_inner;   // exponents -go + gi and gi - 1 of the hardening rate
};

// Lifetime minus target for one cell, evaluated by the whole warp (sam_cyutils.pyx:360-398).
// sepa/aa/bb/gw hold, per separation node, the norm-independent pieces of the hardening rate;
// the trapezoid terms are formed in parallel and summed in step order by lane 0 so the sum
// rounds like the reference loop.
__device__ double warp_lifetime(double norm_log10, const NormArgs &a, const double *sepa, const double *aa,
                                const double *bb, const double *gw, double *dt, int lane) {
    double norm = pow(10.0, norm_log10);
    for (int s = lane; s < a.nsteps; s += 32) {
        double dl = -norm * aa[s] / bb[s];
        dl += gw[s];
        double dr = -norm * aa[s + 1] / bb[s + 1];
        dr += gw[s + 1];
        dt[s] = 2.0 * (sepa[s + 1] - sepa[s]) / (dl + dr);
    }
    __syncwarp();
    double time = 0.0;
    if (lane == 0) {
        for (int s = 0; s < a.nsteps; s++) time += dt[s];
    }
    time = __shfl_sync(0xffffffffu, time, 0);
    __syncwarp();
    return time - a.target_time;
}

// Brent's method (Brent 1973, "Algorithms for Minimization without Derivatives", ch. 4) with the
// tolerance delta = (xtol + rtol |b|) / 2; returns 0 when the interval does not bracket a root
// and the last iterate when the iteration budget runs out.  All lanes run it in lock step.
__device__ double warp_brent(const NormArgs &a, const double *sepa, const double *aa, const double *bb,
                             const double *gw, double *dt, int lane, int *n_iter_out) {
    double xa = NORM_LOG10_LO, xb = NORM_LOG10_HI;
    double fa = warp_lifetime(xa, a, sepa, aa, bb, gw, dt, lane);
    double fb = warp_lifetime(xb, a, sepa, aa, bb, gw, dt, lane);
    *n_iter_out = 0;
    if (fa * fb > 0.0) return 0.0;
    if (fa == 0.0) return xa;
    if (fb == 0.0) return xb;
    double xc = xa, fc = fa;
    double d = xb - xa, e = d;
    for (int it = 0; it < BRENT_MAXITER; it++) {
        *n_iter_out = it + 1;
        if (fb * fc > 0.0) {
            xc = xa;
            fc = fa;
            d = xb - xa;
            e = d;
        }
        if (fabs(fc) < fabs(fb)) {
            xa = xb; xb = xc; xc = xa;
            fa = fb; fb = fc; fc = fa;
        }
        double tol = 0.5 * (BRENT_XTOL + BRENT_RTOL * fabs(xb));
        double m = 0.5 * (xc - xb);
        if (fb == 0.0 || fabs(m) < tol) return xb;
        if (fabs(e) > tol && fabs(fb) < fabs(fa)) {
            double s;
            if (xa == xc) {
                s = -fb * (xb - xa) / (fb - fa);                               // secant
            } else {
                double da = (fa - fb) / (xa - xb);
                double dc = (fc - fb) / (xc - xb);
                s = -fb * (fc * dc - fa * da) / (dc * da * (fc - fa));         // inverse quadratic
            }
            if (2.0 * fabs(s) < fmin(fabs(e), 3.0 * fabs(m) - tol)) {
                e = d;
                d = s;
            } else {
                d = m;
                e = m;
            }
        } else {
            d = m;
            e = m;
        }
        xa = xb;
        fa = fb;
        xb = xb + ((fabs(d) > tol) ? d : ((m > 0.0) ? tol : -tol));
        fb = warp_lifetime(xb, a, sepa, aa, bb, gw, dt, lane);
    }
    *n_iter_out = BRENT_MAXITER + 1;
    return xb;
}

__global__ void k_hardening_norm(CyConst cc, NormArgs a, const double *__restrict__ mtot,
                                 const double *__restrict__ mrat, int n, double *__restrict__ norm_log10,
                                 double *__restrict__ norm, int *d_status) {
    extern __shared__ double smem[];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int nwarps = blockDim.x >> 5;
    int cell = blockIdx.x * nwarps + warp;
    if (cell >= n) return;   // whole warp exits together
    int S = a.nsteps;
    double *sepa = smem + (size_t)warp * 5 * (S + 1);
    double *aa = sepa + (S + 1);
    double *bb = aa + (S + 1);
    double *gw = bb + (S + 1);
    double *dt = gw + (S + 1);
    double mt = mtot[cell], mr = mrat[cell];

    // separation nodes: log10 separation stepped down by repeated subtraction (sam_cyutils.pyx:367-383)
    double risco_log10 = log10(3.0 * HGB_CY_SCHW * mt);
    double dx = (a.sepa_init_log10 - risco_log10) / S;
    if (lane == 0) {
        double sl = a.sepa_init_log10;
        sepa[0] = sl;
        for (int s = 1; s <= S; s++) {
            sl -= dx;
            sepa[s] = sl;
        }
    }
    __syncwarp();
    for (int s = lane; s <= S; s += 32) {
        double sp = pow(10.0, sepa[s]);
        double xx = sp / a.rchar;
        aa[s] = pow(1.0 + xx, -a.go + a.gi);
        bb[s] = pow(xx, a.gi - 1.0);
        gw[s] = hgb::hard_gw(cc.c_dadt, mt, mr, sp);
        sepa[s] = sp;
    }
    __syncwarp();
    int nit;
    double root = warp_brent(a, sepa, aa, bb, gw, dt, lane, &nit);
    if (lane == 0) {
        norm_log10[cell] = root;
        if (norm) norm[cell] = pow(10.0, root);
        if (nit > BRENT_MAXITER) hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
    }
}

// ------------------------------------------------------------------------------------------------
// differential binary number, Fixed_Time_2PL_SAM
// ------------------------------------------------------------------------------------------------

// x^y for an exponent fixed per call.  Integer and half-integer exponents up to |y| = 8.5 (the
// hardening model's defaults give -3.5 and -2) are evaluated as products and one square root,
// within a few ulp of pow(); any other exponent goes to pow().
PowPlan pow_plan(double y) {
    PowPlan p{0, 0, y < 0.0};
    const double ay = fabs(y), twice = 2.0 * ay;
    if (ay <= 8.5 && twice == floor(twice)) {
        p.n = (int)floor(ay);
        p.kind = (ay == floor(ay)) ? 1 : 2;
    }
    return p;
}

__device__ __forceinline__ double pow_planned(double x, double y, PowPlan p) {
    if (p.kind == 0) return pow(x, y);
    double r = (p.kind == 2) ? sqrt(x) : 1.0;
    for (int i = 0; i < p.n; i++) r *= x;
    return p.neg ? 1.0 / r : r;
}

// x1^y1 / x2^y2 with both exponents planned: the two magnitudes as products and square roots and
// at most one division (within a few ulp of the quotient of the pow() forms)
__device__ __forceinline__ double pow_ratio_planned(double x1, double y1, PowPlan p1, double x2, double y2,
                                                   PowPlan p2) {
    if (p1.kind == 0 || p2.kind == 0) return pow_planned(x1, y1, p1) / pow_planned(x2, y2, p2);
    double r1 = (p1.kind == 2) ? sqrt(x1) : 1.0, r2 = (p2.kind == 2) ? sqrt(x2) : 1.0;
    for (int i = 0; i < p1.n; i++) r1 *= x1;
    for (int i = 0; i < p2.n; i++) r2 *= x2;
    if (p1.neg) return p2.neg ? r2 / r1 : 1.0 / (r1 * r2);
    return p2.neg ? r1 * r2 : r1 / r2;
}

struct Dbn2plArgs {
    double sepa_init_log10, rchar, gi, go;
    int num_steps, n_freq, fobs_sorted;
    int n_mtot, n_mrat, n_redz, n_interp;
    PowPlan p_outer, p_inner;   // exponents -go + gi and gi - 1 of the hardening rate
};

// Several (mtot, mrat) cells per block (`cpb`, chosen by the host so that cpb x n_redz rows nearly
// fill the block): a cell's redshift rows alone would leave most of a warp idle (101 rows are three
// warps and five lanes), and GB300 charges an FP64 warp instruction in full however few lanes are
// active.  Row r of the block is redshift r / nc of its cell r % nc (nc cells in the block); each cell's step
// tables live in its own slice of shared memory, built by the whole block.  Each row's arithmetic is
// the single-cell kernel's.
constexpr int WALK_MAX_CELLS = 16;

__global__ void __launch_bounds__(512) k_dbn_2pwl(CyConst cc, Dbn2plArgs a, int cpb, const double *__restrict__ fobs,
                           const double *__restrict__ hard_norm, const double *__restrict__ nden,
                           const double *__restrict__ mtot, const double *__restrict__ mrat,
                           const double *__restrict__ redz, const double *__restrict__ gmt_time,
                           const double *__restrict__ zgrid_g, const double *__restrict__ agrid_g,
                           const double *__restrict__ dgrid_g, double *__restrict__ redz_final,
                           double *__restrict__ diff_num) {
    extern __shared__ double smem[];
    const int S = a.num_steps, NI = a.n_interp, NF = a.n_freq;
    const int ncell = a.n_mtot * a.n_mrat;
    const int cell0 = blockIdx.x * cpb;
    const int nc = min(cpb, ncell - cell0);   // cells of this block
    double *zg = smem;
    double *ag = zg + NI;
    double *dg = ag + NI;
    double *sz = dg + NI;            // [NI] dz/dt of each age-table interval
    double *ft = sz + NI;
    double *cells = ft + NF;         // per cell: sepa [S+1], frst [S+1], dadt [S+1], dts [S], tevo [S]
    const int per_cell = 3 * (S + 1) + 2 * S;
    __shared__ double s_fmax;
    __shared__ int s_first[WALK_MAX_CELLS];
    __shared__ double s_sqrt_mt[WALK_MAX_CELLS], s_mt3[WALK_MAX_CELLS], s_mr12[WALK_MAX_CELLS];

    for (int i = threadIdx.x; i < NI; i += blockDim.x) {
        zg[i] = zgrid_g[i];
        ag[i] = agrid_g[i];
        dg[i] = dgrid_g[i];
    }
    for (int i = threadIdx.x; i < NF; i += blockDim.x) ft[i] = fobs[i];
    __syncthreads();
    for (int i = threadIdx.x; i < NI - 1; i += blockDim.x) sz[i] = (zg[i + 1] - zg[i]) / (ag[i + 1] - ag[i]);
    if (threadIdx.x < nc) {   // log10 separation nodes by repeated subtraction, one thread per cell
        const int cell = cell0 + threadIdx.x;
        const double mt = mtot[cell / a.n_mrat];
        double *sepa = cells + (size_t)threadIdx.x * per_cell;
        const double risco = 3.0 * HGB_CY_SCHW * mt;
        const double dx = (a.sepa_init_log10 - log10(risco)) / S;
        double sl = a.sepa_init_log10;
        sepa[0] = sl;
        for (int s = 1; s <= S; s++) {
            sl -= dx;
            sepa[s] = sl;
        }
        const double mr = mrat[cell % a.n_mrat];
        s_sqrt_mt[threadIdx.x] = sqrt(mt);
        s_mt3[threadIdx.x] = pow(mt, 3.0);
        s_mr12[threadIdx.x] = pow(1.0 + mr, 2.0);
    }
    __syncthreads();
    // per node: sp^1.5 as sp sqrt(sp), the hardening model's (half-)integer powers as products
    // (pow_planned), and the GW rate with the cell's mt^3 and (1 + mr)^2 taken once: each within a
    // few ulp of the pow() forms of sam_cyutils.pyx:240-253 and holodeck/cyutils.pyx
    for (int i = threadIdx.x; i < nc * (S + 1); i += blockDim.x) {
        const int c = i / (S + 1), s = i % (S + 1), cell = cell0 + c;
        const double mr = mrat[cell % a.n_mrat], norm = hard_norm[cell];
        const double sqrt_mt = s_sqrt_mt[c], mt3 = s_mt3[c], mr12 = s_mr12[c];
        double *sepa = cells + (size_t)c * per_cell;
        double *frst = sepa + (S + 1), *dadt = frst + (S + 1);
        const double sp = pow(10.0, sepa[s]);
        sepa[s] = sp;
        frst[s] = cc.kfreq * sqrt_mt / (sp * sqrt(sp));
        const double xx = sp / a.rchar;
        double dd = -norm * pow_ratio_planned(1.0 + xx, -a.go + a.gi, a.p_outer, xx, a.gi - 1.0, a.p_inner);
        dd += cc.c_dadt * mt3 * mr / (sp * sp * sp) / mr12;
        dadt[s] = dd;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nc * S; i += blockDim.x) {
        const int c = i / S, s = i % S;
        double *sepa = cells + (size_t)c * per_cell;
        const double *dadt = sepa + 2 * (S + 1);
        double *dts = sepa + 3 * (S + 1);
        dts[s] = 2.0 * (sepa[s + 1] - sepa[s]) / (dadt[s] + dadt[s + 1]);
    }
    __syncthreads();
    // Steps that cannot bracket any target are skipped without changing a result: the observed
    // frequency of a step is at most its rest-frame frequency (z >= 0 after clamping) and at least
    // frst / (1 + z_start), because the redshift only decreases from the starting redshift.
    double fmin_all = ft[0], fmax_all = ft[0];
    for (int f = 1; f < NF; f++) {
        fmin_all = fmin_all < ft[f] ? fmin_all : ft[f];
        fmax_all = fmax_all > ft[f] ? fmax_all : ft[f];
    }
    if (threadIdx.x < nc) {   // running time and first useful step, one thread per cell
        double *sepa = cells + (size_t)threadIdx.x * per_cell;
        const double *frst = sepa + (S + 1), *dts = sepa + 3 * (S + 1);
        double *tevo = sepa + 3 * (S + 1) + S;
        double te = 0.0;
        for (int s = 0; s < S; s++) {
            te += dts[s];
            tevo[s] = te;
        }
        int first = 0;   // first step whose right edge reaches fmin
        while (first < S && frst[first + 1] < fmin_all) first++;
        s_first[threadIdx.x] = first;
        if (threadIdx.x == 0) s_fmax = fmax_all;
    }
    __syncthreads();
    const double fmax = s_fmax;

    const double age_universe = ag[NI - 1];
    for (int r = threadIdx.x; r < nc * a.n_redz; r += blockDim.x) {
        // redshift-major: a warp's lanes hold a few neighbouring redshifts of every cell of the block
        // (mostly one mtot, so one rest-frequency table), whose walks have similar lengths
        const int c = r % nc, kk = r / nc;
        const int cell = cell0 + c;
        const double *frst = cells + (size_t)c * per_cell + (S + 1);
        const double *dts = cells + (size_t)c * per_cell + 3 * (S + 1);
        const double *tevo = dts + S;
        const int s_begin = s_first[c];
        long row = ((long)cell * a.n_redz + kk);
        double *rf = redz_final + row * NF;
        double *dn = diff_num + row * NF;
        for (int f = 0; f < NF; f++) {
            rf[f] = -1.0;
            dn[f] = 0.0;
        }
        // age at the starting redshift (sam_cyutils.pyx:563-573)
        double zk = redz[kk];
        int zi = hgb::bracket_decreasing_from0(NI, zk, zg);
        if (zi > NI - 2) zi = NI - 2;
        double rage = hgb::interp_between(zk, zg[zi], zg[zi + 1], ag[zi], ag[zi + 1]);
        double gmt = gmt_time[row];
        const double fstop = fmax * (1.0 + zk) * (1.0 + 1e-12);
        int il = 0;
        int fp = 0;                 // first target >= the left frequency (targets ascending)
        bool have_prev = false;     // right edge of the previous step, reused as this step's left edge
        double prev_tr = 0.0, prev_zr = 0.0, prev_fr = 0.0;
        for (int s = s_begin; s < S; s++) {
            if (frst[s] > fstop) break;
            double time_right = tevo[s] + gmt + rage;
            double time_left, redz_left, fl;
            bool reuse = have_prev;
            have_prev = false;
            if (reuse) {
                time_left = prev_tr;
            } else {
                time_left = time_right - dts[s];
            }
            if (time_left > age_universe) continue;
            if (reuse) {
                redz_left = prev_zr;
            } else {
                il = hgb::while_while_increasing(il, NI, time_left, ag);
                redz_left = zg[il] + (time_left - ag[il]) * sz[il];
            }
            if (redz_left < 0.0) continue;
            fl = reuse ? prev_fr : frst[s] / (1.0 + redz_left);
            int ir = hgb::while_while_increasing(il, NI, time_right, ag);
            double redz_right = zg[ir] + (time_right - ag[ir]) * sz[ir];
            double zr_raw = redz_right;
            if (redz_right < 0.0) redz_right = 0.0;
            double fr = frst[s + 1] / (1.0 + redz_right);
            if (zr_raw >= 0.0) {
                have_prev = true;
                prev_tr = time_right;
                prev_zr = zr_raw;
                prev_fr = fr;
            }
            int il_step = il;
            il = ir;
            int f0;
            if (a.fobs_sorted) {
                while (fp > 0 && ft[fp - 1] >= fl) fp--;
                while (fp < NF && ft[fp] < fl) fp++;
                f0 = fp;
                if (f0 >= NF || ft[f0] > fr) continue;
            } else {
                f0 = 0;
            }
            for (int f = f0; f < NF; f++) {
                double ftarget = ft[f];
                if (ftarget < fl || fr < ftarget) {
                    if (a.fobs_sorted) break;   // ascending targets: nothing further lies inside
                    continue;
                }
                double new_time = hgb::interp_between(ftarget, fl, fr, time_left, time_right);
                if (new_time > ag[NI - 1]) break;
                // phase 1 records the bracket; k_dbn_2pwl_eval turns it into redz_final / diff_num
                rf[f] = (double)il_step;
                dn[f] = new_time;
            }
        }
    }
}

// Phase 2 of the Fixed_Time_2PL_SAM number: every (redz, frequency) element of a (mtot, mrat) cell
// whose target was bracketed (sam_cyutils.pyx:731-768).  One block per cell, so the cell's
// constant powers are taken once and the elements run without divergence.
__global__ void k_dbn_2pwl_eval(CyConst cc, Dbn2plArgs a, const double *__restrict__ fobs,
                                const double *__restrict__ hard_norm, const double *__restrict__ nden,
                                const double *__restrict__ mtot, const double *__restrict__ mrat,
                                const double *__restrict__ zgrid_g, const double *__restrict__ agrid_g,
                                const double *__restrict__ dgrid_g, double *__restrict__ redz_final,
                                double *__restrict__ diff_num) {
    extern __shared__ double smem[];
    const int NI = a.n_interp, NF = a.n_freq;
    double *zg = smem;
    double *ag = zg + NI;
    double *dg = ag + NI;
    double *ft = dg + NI;
    double *sz = ft + NF;            // [NI] dz/dt and d(d_C)/dt of each age-table interval
    double *sd = sz + NI;
    const int cell = blockIdx.x;
    const int ii = cell / a.n_mrat, jj = cell % a.n_mrat;
    for (int i = threadIdx.x; i < NI; i += blockDim.x) {
        zg[i] = zgrid_g[i];
        ag[i] = agrid_g[i];
        dg[i] = dgrid_g[i];
    }
    for (int i = threadIdx.x; i < NF; i += blockDim.x) ft[i] = fobs[i];
    __syncthreads();
    for (int i = threadIdx.x; i < NI - 1; i += blockDim.x) {
        const double dt = ag[i + 1] - ag[i];
        sz[i] = (zg[i + 1] - zg[i]) / dt;
        sd[i] = (dg[i + 1] - dg[i]) / dt;
    }
    __shared__ double s_mt3, s_mr12, s_mt13;
    const double mt = mtot[ii], mr = mrat[jj], norm = hard_norm[cell];
    if (threadIdx.x == 0) {
        s_mt3 = pow(mt, 3.0);
        s_mr12 = pow(1.0 + mr, 2.0);
        s_mt13 = pow(mt, 1.0 / 3.0);
    }
    __syncthreads();
    const double mt13 = s_mt13;
    const double gw_k = cc.c_dadt * s_mt3 * mr / s_mr12;   // GW rate = gw_k / sepa^3
    const double inv_rchar = 1.0 / a.rchar;
    const long nzf = (long)a.n_redz * NF;
    const long base = (long)cell * nzf;
    for (long e = threadIdx.x; e < nzf; e += blockDim.x) {
        double hint = redz_final[base + e];
        if (hint < 0.0) continue;   // no bracket: stays -1 / 0
        const int f = (int)(e % NF);
        const int kk = (int)(e / NF);
        const double new_time = diff_num[base + e];
        int ni = hgb::while_while_increasing((int)hint, NI, new_time, ag);
        double new_redz = zg[ni] + (new_time - ag[ni]) * sz[ni];
        double dcom = dg[ni] + (new_time - ag[ni]) * sd[ni];
        double target_frst_orb = ft[f] * (1.0 + new_redz);
        // target^(-2/3) = r^2 with r = target^(-1/3): FP32 start and one FP64 Newton step,
        // r (4 - y r^3) / 3 (relative error about 1e-14)
        const double r0 = (double)rcbrtf((float)target_frst_orb);
        const double r1 = r0 * (4.0 - target_frst_orb * (r0 * r0 * r0)) * (1.0 / 3.0);
        double sp = cc.ksepa * mt13 * (r1 * r1);
        double xx = sp * inv_rchar;
        double dadt = -norm * pow_ratio_planned(1.0 + xx, -a.go + a.gi, a.p_outer, xx, a.gi - 1.0, a.p_inner);
        dadt += gw_k / (sp * sp * sp);
        double tres = -(2.0 / 3.0) * sp / dadt;
        double dcm = dcom * (1.0 / HGB_CY_MPC);
        double cosmo_fact = cc.fourpi * (1.0 + new_redz) * (dcm * dcm);
        redz_final[base + e] = new_redz;
        diff_num[base + e] = nden[(long)cell * a.n_redz + kk] * tres * cosmo_fact;
    }
}

// ---- FP32 production mode of k_dbn_2pwl_eval
//
// The age -> redshift inversion (bracket, interpolated redshift and comoving distance) stays FP64, as
// in the reference; the residence time and the cosmological factor are FP32.  FP64 work per element:
// the bracket offset, two interpolations and the two products with the density.  The age bracket
// compares the positive FP64 ages as integers (IEEE order of positive doubles), off the FP64 pipe.
// Ranges: the hardening rate is -(A P(x) + G / x^3) with x = sepa / rchar, A = norm and
// G = |GW_DADT_SEP_CONST| mt^3 mr / (1 + mr)^2 / rchar^3 per cell; both constants are scaled by the
// same power of two 2^-e0 (e0 the larger exponent), so the sum is a normal float wherever either term
// matters, and the residence time comes out as t_s 2^-e0.

// x^y for the planned exponents in FP32 (as pow_planned / pow_ratio_planned)
__device__ __forceinline__ float pow_planned_f32(float x, float y, PowPlan p) {
    if (p.kind == 0) return powf(x, y);
    float r = (p.kind == 2) ? sqrtf(x) : 1.0f;
    for (int i = 0; i < p.n; i++) r *= x;
    return p.neg ? __fdividef(1.0f, r) : r;
}

__device__ __forceinline__ int while_while_increasing_bits(int start, int size, double val, const double *edges) {
    const long long v = __double_as_longlong(val);   // val and edges are positive: integer order is IEEE order
    int index = start;
    while ((index < size - 2) && (__double_as_longlong(edges[index + 1]) < v)) index += 1;
    while ((index > 0) && (__double_as_longlong(edges[index]) > v)) index -= 1;
    return index;
}

__global__ void k_dbn_2pwl_eval_f32(CyConst cc, Dbn2plArgs a, const double *__restrict__ fobs,
                                    const double *__restrict__ hard_norm, const double *__restrict__ nden,
                                    const double *__restrict__ mtot, const double *__restrict__ mrat,
                                    const double *__restrict__ zgrid_g, const double *__restrict__ agrid_g,
                                    const double *__restrict__ dgrid_g, double *__restrict__ redz_final,
                                    double *__restrict__ diff_num) {
    extern __shared__ double smem[];
    const int NI = a.n_interp, NF = a.n_freq;
    double *zg = smem;
    double *ag = zg + NI;
    double *dg = ag + NI;
    double *sz = dg + NI;            // [NI] dz/dt and d(d_C)/dt of each age-table interval
    double *sd = sz + NI;
    float *ft = (float *)(sd + NI);  // [NF]
    const int cell = blockIdx.x;
    const int ii = cell / a.n_mrat, jj = cell % a.n_mrat;
    for (int i = threadIdx.x; i < NI; i += blockDim.x) {
        zg[i] = zgrid_g[i];
        ag[i] = agrid_g[i];
        dg[i] = dgrid_g[i];
    }
    for (int i = threadIdx.x; i < NF; i += blockDim.x) ft[i] = hgb::f64_to_f32_rz(fobs[i]);
    __syncthreads();
    for (int i = threadIdx.x; i < NI - 1; i += blockDim.x) {
        const double dt = ag[i + 1] - ag[i];
        sz[i] = (zg[i + 1] - zg[i]) / dt;
        sd[i] = (dg[i + 1] - dg[i]) / dt;
    }
    __shared__ float s_k13, s_as, s_gs, s_rchar_inv;
    __shared__ int s_e0;
    if (threadIdx.x == 0) {
        const double mt = mtot[ii], mr = mrat[jj], norm = hard_norm[cell];
        const double opq = 1.0 + mr, rc = a.rchar;   // products in place of powers: one thread, the block waits
        const double gc = fabs(cc.c_dadt) * (mt * mt * mt) * mr / (opq * opq) / (rc * rc * rc);
        int ea = -100000, eg = -100000;
        if (norm > 0.0) frexp(norm, &ea);
        if (gc > 0.0) frexp(gc, &eg);
        const int e0 = ea > eg ? ea : eg;
        s_e0 = e0;
        s_as = (float)ldexp(norm, -e0);   // in [0.5, 1) or flushed to 0 when negligible
        s_gs = (float)ldexp(gc, -e0);
        s_k13 = (float)(cc.ksepa * cbrt(mt));
        s_rchar_inv = (float)(1.0 / a.rchar);
    }
    __syncthreads();
    const float k13 = s_k13, as = s_as, gs = s_gs, rchar_inv = s_rchar_inv;
    const int e0 = s_e0;
    const float fourpi = (float)cc.fourpi, inv_mpc = (float)(1.0 / HGB_CY_MPC);
    const long nzf = (long)a.n_redz * NF;
    const long base = (long)cell * nzf;
    for (long e = threadIdx.x; e < nzf; e += blockDim.x) {
        const double hint = redz_final[base + e];
        if (__double_as_longlong(hint) < 0) continue;   // no bracket (-1): stays -1 / 0
        const int f = (int)(e % NF);
        const int kk = (int)(e / NF);
        const double new_time = diff_num[base + e];
        const int ni = while_while_increasing_bits((int)hint, NI, new_time, ag);
        const double dt = new_time - ag[ni];
        const double new_redz = zg[ni] + dt * sz[ni];
        const double dcom = dg[ni] + dt * sd[ni];
        const float zp1 = 1.0f + hgb::f64_to_f32_rz(new_redz);
        const float frst = ft[f] * zp1;
        const float r = rcbrtf(frst);
        const float sp = k13 * (r * r);
        const float xx = sp * rchar_inv;
        const float pw = (a.p_outer.kind && a.p_inner.kind)
                             ? pow_planned_f32(1.0f + xx, (float)(-a.go + a.gi), a.p_outer) *
                                   pow_planned_f32(xx, (float)(1.0 - a.gi), PowPlan{a.p_inner.kind, a.p_inner.n,
                                                                                   !a.p_inner.neg})
                             : __fdividef(powf(1.0f + xx, (float)(-a.go + a.gi)), powf(xx, (float)(a.gi - 1.0)));
        const float rate = fmaf(as, pw, __fdividef(gs, xx * xx * xx));
        const float tres = __fdividef((2.0f / 3.0f) * sp, rate);        // residence time 2^e0
        const float dcm = hgb::f64_to_f32_rz(dcom) * inv_mpc;
        const float cosmo_fact = fourpi * zp1 * (dcm * dcm);
        redz_final[base + e] = new_redz;
        diff_num[base + e] = nden[(long)cell * a.n_redz + kk] * hgb::f32_to_f64_scaled(tres, -e0) *
                             hgb::f32_to_f64_scaled(cosmo_fact, 0);
    }
}

// ------------------------------------------------------------------------------------------------
// differential binary number, Hard_GW
// ------------------------------------------------------------------------------------------------

__global__ void k_dbn_gw(CyConst cc, const double *__restrict__ fobs, int NF, const double *__restrict__ nden,
                         const double *__restrict__ mtot, int nm, const double *__restrict__ mrat, int nq, int nz,
                         const double *__restrict__ redz_prime, const double *__restrict__ zgrid,
                         const double *__restrict__ dgrid, int NI, double *__restrict__ redz_final,
                         double *__restrict__ diff_num) {
    long row = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (long)nm * nq * nz) return;
    int jj = (int)((row / nz) % nq);
    int ii = (int)(row / ((long)nz * nq));
    double *rf = redz_final + row * NF;
    double *dn = diff_num + row * NF;
    for (int f = 0; f < NF; f++) {
        rf[f] = -1.0;
        dn[f] = 0.0;
    }
    double rzp = redz_prime[row];
    if (rzp <= 0.0) return;
    double mt = mtot[ii], mr = mrat[jj];
    double rad_isco = 3.0 * HGB_CY_SCHW * mt;
    double frst_orb_isco = cc.kfreq * sqrt(mt) / pow(rad_isco, 1.5);
    int zi = hgb::bracket_decreasing_from0(NI, rzp, zgrid);
    if (zi > NI - 2) zi = NI - 2;
    double dcom = hgb::interp_between(rzp, zgrid[zi], zgrid[zi + 1], dgrid[zi], dgrid[zi + 1]);
    double nd = nden[row];
    for (int f = 0; f < NF; f++) {
        rf[f] = rzp;
        double target_frst_orb = fobs[f] * (1.0 + rzp);
        if (target_frst_orb > frst_orb_isco) {
            for (int fp = f + 1; fp < NF; fp++) rf[fp] = rzp;
            break;
        }
        double sp = cc.ksepa * pow(mt, 1.0 / 3.0) / pow(target_frst_orb, 2.0 / 3.0);
        double dadt = hgb::hard_gw(cc.c_dadt, mt, mr, sp);
        double tres = -(2.0 / 3.0) * sp / dadt;
        double dcm = dcom / HGB_CY_MPC;
        double cosmo_fact = cc.fourpi * (1.0 + rzp) * (dcm * dcm);
        dn[f] = nd * tres * cosmo_fact;
    }
}

// The same root, one warp per cell and eight cells per block.  A lane holds the constants of nodes
// s = lane + 32 k in registers: the hardening shape, the GW rate and the trapezoid coefficient
// c[s] = 2 (sepa[s+1] - sepa[s]).  Each Brent round sums the lifetime c[s] / (v[s] + v[s+1]) with
// one partial per lane and an xor-butterfly reduction.  Every lane ends with the same total
// (addition is commutative), so the warp's Brent state stays uniform and the warps never wait for
// one another.  The evaluation sequence is that of warp_brent; only the grouping of the step sum
// differs from the reference's step order (a relative change of the lifetime near 1e-16, far
// below the 1e-3 root tolerance, which the root follows unless a Brent comparison falls within
// that margin: the normalisation is checked against the reference at 1e-10 in log10).
constexpr int NB_CELLS = 8;    // 256 threads: half an SM's registers, so other stages' blocks fit beside
constexpr int NB_NODES = 10;   // nodes per lane: nsteps + 1 <= 320

__global__ void __launch_bounds__(NB_CELLS * 32, 2) k_hardening_norm_blk(CyConst cc, NormArgs a,
                                                                       const double *__restrict__ mtot,
                                                                       const double *__restrict__ mrat, int n,
                                                                       double *__restrict__ norm_log10,
                                                                       double *__restrict__ norm, int *d_status) {
    extern __shared__ double smem[];   // [NB_CELLS][S + 1]: each warp's log10 separations
    const int S = a.nsteps;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cell = blockIdx.x * NB_CELLS + warp;
    if (cell >= n) return;   // the whole warp: no block-wide barrier follows
    double *row = smem + (size_t)warp * (S + 1);
    const double mt = mtot[cell], mr = mrat[cell];
    const double mt3 = pow(mt, 3.0), mr12 = pow(1.0 + mr, 2.0);
    // log10 separation nodes by repeated subtraction (sam_cyutils.pyx:367-383)
    if (lane == 0) {
        const double risco_log10 = log10(3.0 * HGB_CY_SCHW * mt);
        const double dx = (a.sepa_init_log10 - risco_log10) / S;
        double sl = a.sepa_init_log10;
        row[0] = sl;
        for (int s = 1; s <= S; s++) {
            sl -= dx;
            row[s] = sl;
        }
    }
    __syncwarp();
    // per node: the hardening shape (1 + x)^(gi - go) / x^(gi - 1) and the GW rate, which do not
    // depend on the normalisation, so each Brent round costs one product and one sum per node
    double rr[NB_NODES], gw[NB_NODES], sp[NB_NODES], cf[NB_NODES];
#pragma unroll
    for (int k = 0; k < NB_NODES; k++) {
        const int s = lane + 32 * k;
        rr[k] = 1.0;
        gw[k] = sp[k] = 0.0;
        if (s <= S) {
            const double x = pow(10.0, row[s]);
            const double xx = x / a.rchar;
            rr[k] = pow_ratio_planned(1.0 + xx, -a.go + a.gi, a.p_outer, xx, a.gi - 1.0, a.p_inner);
            gw[k] = cc.c_dadt * mt3 * mr / (x * x * x) / mr12;
            sp[k] = x;
        }
    }
    // c[s] = 2 (sepa[s+1] - sepa[s]) for s < S, 0 beyond
#pragma unroll
    for (int k = 0; k < NB_NODES; k++) {
        double nxt = __shfl_down_sync(0xffffffffu, sp[k], 1);
        const double wrap = __shfl_sync(0xffffffffu, (k + 1 < NB_NODES) ? sp[k + 1] : 0.0, 0);
        if (lane == 31) nxt = wrap;
        const int s = lane + 32 * k;
        cf[k] = (s < S) ? 2.0 * (nxt - sp[k]) : 0.0;
    }

    // Brent's method as in warp_brent, one evaluation per round
    double xa = NORM_LOG10_LO, xb = NORM_LOG10_HI, xc = 0.0, fa = 0.0, fb = 0.0, fc = 0.0, d = 0.0, e = 0.0;
    int stage = 0, it = 0, nit = 0;
    double root = 0.0;
    for (int round = 0; round < BRENT_MAXITER + 2; round++) {
        const double xe = (stage == 0) ? xa : xb;
        const double nrm = pow(10.0, xe);
        double v[NB_NODES];
#pragma unroll
        for (int k = 0; k < NB_NODES; k++) {
            double dl = -nrm * rr[k];
            dl += gw[k];
            v[k] = dl;
        }
        double part = 0.0;
#pragma unroll
        for (int k = 0; k < NB_NODES; k++) {
            double vn = __shfl_down_sync(0xffffffffu, v[k], 1);
            const double wrap = __shfl_sync(0xffffffffu, (k + 1 < NB_NODES) ? v[k + 1] : 0.0, 0);
            if (lane == 31) vn = wrap;
            const int s = lane + 32 * k;
            if (s < S) part += cf[k] / (v[k] + vn);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        const double fv = part - a.target_time;
        if (stage == 0) {
            fa = fv;
            stage = 1;
            continue;
        }
        fb = fv;
        if (stage == 1) {
            stage = 2;
            if (fa * fb > 0.0) {
                root = 0.0;
                break;
            }
            if (fa == 0.0) {
                root = xa;
                break;
            }
            if (fb == 0.0) {
                root = xb;
                break;
            }
            xc = xa;
            fc = fa;
            d = xb - xa;
            e = d;
            it = 0;
        } else {
            it++;
            if (it >= BRENT_MAXITER) {
                root = xb;
                nit = BRENT_MAXITER + 1;
                break;
            }
        }
        nit = it + 1;
        if (fb * fc > 0.0) {
            xc = xa;
            fc = fa;
            d = xb - xa;
            e = d;
        }
        if (fabs(fc) < fabs(fb)) {
            xa = xb; xb = xc; xc = xa;
            fa = fb; fb = fc; fc = fa;
        }
        const double tol = 0.5 * (BRENT_XTOL + BRENT_RTOL * fabs(xb));
        const double m = 0.5 * (xc - xb);
        if (fb == 0.0 || fabs(m) < tol) {
            root = xb;
            break;
        }
        if (fabs(e) > tol && fabs(fb) < fabs(fa)) {
            double sst;
            if (xa == xc) {
                sst = -fb * (xb - xa) / (fb - fa);
            } else {
                const double da = (fa - fb) / (xa - xb);
                const double dc = (fc - fb) / (xc - xb);
                sst = -fb * (fc * dc - fa * da) / (dc * da * (fc - fa));
            }
            if (2.0 * fabs(sst) < fmin(fabs(e), 3.0 * fabs(m) - tol)) {
                e = d;
                d = sst;
            } else {
                d = m;
                e = m;
            }
        } else {
            d = m;
            e = m;
        }
        xa = xb;
        fa = fb;
        xb = xb + ((fabs(d) > tol) ? d : ((m > 0.0) ? tol : -tol));
    }
    if (lane == 0) {
        norm_log10[cell] = root;
        if (norm) norm[cell] = pow(10.0, root);
        if (nit > BRENT_MAXITER) hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
    }
}

size_t norm_blk_smem(int nsteps) { return sizeof(double) * (size_t)NB_CELLS * ((size_t)nsteps + 1); }

size_t norm_smem_per_warp(int nsteps) { return (size_t)5 * (nsteps + 1) * sizeof(double); }

}  // namespace

extern "C" {

int hgb_find_2pwl_hardening_norm(double target_time, const double *mtot, const double *mrat, int n,
                                 double sepa_init, double rchar, double gamma_inner, double gamma_outer,
                                 int nsteps, double *norm_log10, double *norm, int *d_status, void *stream) {
    HGB_CHECK_ARG(mtot && mrat && norm_log10 && n >= 0);
    HGB_CHECK_ARG(nsteps > 0 && sepa_init > 0.0 && rchar > 0.0);
    size_t per_warp = norm_smem_per_warp(nsteps);
    HGB_CHECK_ARG(per_warp <= 200 * 1024);
    if (n == 0) return HGB_OK;
    int wpb = (int)(48 * 1024 / per_warp);
    if (wpb > 4) wpb = 4;
    if (wpb < 1) wpb = 1;
    size_t smem = per_warp * wpb;
    int rc = hgb::ensure_dyn_smem((const void *)k_hardening_norm, smem);
    if (rc) return rc;
    NormArgs a{target_time, log10(sepa_init), rchar, gamma_inner, gamma_outer, nsteps,
               pow_plan(-gamma_outer + gamma_inner), pow_plan(gamma_inner - 1.0)};
    if (nsteps + 1 <= 32 * NB_NODES) {
        const size_t bsmem = norm_blk_smem(nsteps);
        if ((rc = hgb::ensure_dyn_smem((const void *)k_hardening_norm_blk, bsmem))) return rc;
        k_hardening_norm_blk<<<(unsigned)hgb::ceil_div(n, NB_CELLS), NB_CELLS * 32, bsmem, (cudaStream_t)stream>>>(
            hgb::cy_const(), a, mtot, mrat, n, norm_log10, norm, d_status);
        return hgb::check_launch();
    }
    unsigned blocks = (unsigned)hgb::ceil_div(n, wpb);
    k_hardening_norm<<<blocks, 32 * wpb, smem, (cudaStream_t)stream>>>(hgb::cy_const(), a, mtot, mrat, n,
                                                                       norm_log10, norm, d_status);
    return hgb::check_launch();
}

int hgb_dbn_2pwl_phase(const double *fobs_orb, int n_freq, int fobs_sorted, double sepa_init, int num_steps,
                       const double *hard_norm, double rchar, double gamma_inner, double gamma_outer,
                       const double *nden, const double *mtot, int n_mtot, const double *mrat, int n_mrat,
                       const double *redz, int n_redz, const double *gmt_time, const hgb_cosmo *cosmo,
                       double *redz_final, double *diff_num, int phase, void *stream) {
    HGB_CHECK_ARG(phase >= 1 && phase <= 3);
    HGB_CHECK_ARG(fobs_orb && hard_norm && mtot && mrat && cosmo && redz_final && diff_num);
    HGB_CHECK_ARG(!(phase & 1) || (redz && gmt_time));
    HGB_CHECK_ARG(!(phase & 2) || nden);
    HGB_CHECK_ARG(n_freq > 0 && num_steps > 0 && n_mtot > 0 && n_mrat > 0 && n_redz > 0);
    HGB_CHECK_ARG(cosmo->grid_size >= 2 && cosmo->grid_z && cosmo->grid_age && cosmo->grid_dcom);
    HGB_CHECK_ARG(sepa_init > 0.0 && rchar > 0.0);
    Dbn2plArgs a{log10(sepa_init), rchar, gamma_inner, gamma_outer, num_steps, n_freq, fobs_sorted ? 1 : 0,
                 n_mtot, n_mrat, n_redz, cosmo->grid_size, pow_plan(-gamma_outer + gamma_inner),
                 pow_plan(gamma_inner - 1.0)};
    unsigned blocks = (unsigned)((long)n_mtot * n_mrat);
    if (phase & 1) {
        // cells per block: fill up to 512 rows (cpb x n_redz), within a shared-memory budget
        const size_t base = sizeof(double) * ((size_t)4 * cosmo->grid_size + n_freq);
        const size_t per_cell = sizeof(double) * (3 * (size_t)(num_steps + 1) + 2 * (size_t)num_steps);
        HGB_CHECK_ARG(base + per_cell <= 200 * 1024);
        int cpb = 512 / n_redz;
        cpb = std::min<long>(cpb, (long)((160 * 1024 - std::min<size_t>(base, 160 * 1024)) / per_cell));
        cpb = std::max(1, std::min(cpb, WALK_MAX_CELLS));
        const size_t smem = base + per_cell * cpb;
        int src = hgb::ensure_dyn_smem((const void *)k_dbn_2pwl, smem);
        if (src) return src;
        int threads = (int)hgb::ceil_div((long)cpb * n_redz, 32) * 32;
        if (threads > 512) threads = 512;
        const unsigned wblocks = (unsigned)hgb::ceil_div((long)n_mtot * n_mrat, cpb);
        k_dbn_2pwl<<<wblocks, threads, smem, (cudaStream_t)stream>>>(hgb::cy_const(), a, cpb, fobs_orb, hard_norm, nden,
                                                                    mtot, mrat, redz, gmt_time, cosmo->grid_z,
                                                                    cosmo->grid_age, cosmo->grid_dcom, redz_final,
                                                                    diff_num);
        int rc = hgb::check_launch();
        if (rc) return rc;
    }
    if (phase & 2) {
        size_t smem2 = sizeof(double) * ((size_t)5 * cosmo->grid_size + n_freq);
        k_dbn_2pwl_eval<<<blocks, 256, smem2, (cudaStream_t)stream>>>(hgb::cy_const(), a, fobs_orb, hard_norm, nden,
                                                                      mtot, mrat, cosmo->grid_z, cosmo->grid_age,
                                                                      cosmo->grid_dcom, redz_final, diff_num);
        return hgb::check_launch();
    }
    return HGB_OK;
}

int hgb_dbn_2pwl_phase_f32(const double *fobs_orb, int n_freq, int fobs_sorted, double sepa_init, int num_steps,
                           const double *hard_norm, double rchar, double gamma_inner, double gamma_outer,
                           const double *nden, const double *mtot, int n_mtot, const double *mrat, int n_mrat,
                           const double *redz, int n_redz, const double *gmt_time, const hgb_cosmo *cosmo,
                           double *redz_final, double *diff_num, int phase, void *stream) {
    HGB_CHECK_ARG(phase >= 1 && phase <= 3);
    HGB_CHECK_ARG(fobs_orb && hard_norm && mtot && mrat && cosmo && redz_final && diff_num);
    HGB_CHECK_ARG(!(phase & 2) || nden);
    HGB_CHECK_ARG(n_freq > 0 && num_steps > 0 && n_mtot > 0 && n_mrat > 0 && n_redz > 0);
    HGB_CHECK_ARG(cosmo->grid_size >= 2 && cosmo->grid_z && cosmo->grid_age && cosmo->grid_dcom);
    HGB_CHECK_ARG(sepa_init > 0.0 && rchar > 0.0);
    if (phase & 1) {   // the separation-step walk is the hardening integral: FP64 in both modes
        int rc = hgb_dbn_2pwl_phase(fobs_orb, n_freq, fobs_sorted, sepa_init, num_steps, hard_norm, rchar,
                                    gamma_inner, gamma_outer, nden, mtot, n_mtot, mrat, n_mrat, redz, n_redz,
                                    gmt_time, cosmo, redz_final, diff_num, 1, stream);
        if (rc) return rc;
    }
    if (!(phase & 2)) return HGB_OK;
    Dbn2plArgs a{log10(sepa_init), rchar, gamma_inner, gamma_outer, num_steps, n_freq, fobs_sorted ? 1 : 0,
                 n_mtot, n_mrat, n_redz, cosmo->grid_size, pow_plan(-gamma_outer + gamma_inner),
                 pow_plan(gamma_inner - 1.0)};
    unsigned blocks = (unsigned)((long)n_mtot * n_mrat);
    size_t smem = sizeof(double) * (size_t)5 * cosmo->grid_size + sizeof(float) * (size_t)n_freq;
    HGB_CHECK_ARG(smem <= 48 * 1024);
    k_dbn_2pwl_eval_f32<<<blocks, 256, smem, (cudaStream_t)stream>>>(hgb::cy_const(), a, fobs_orb, hard_norm, nden,
                                                                     mtot, mrat, cosmo->grid_z, cosmo->grid_age,
                                                                     cosmo->grid_dcom, redz_final, diff_num);
    return hgb::check_launch();
}

int hgb_dbn_2pwl(const double *fobs_orb, int n_freq, int fobs_sorted, double sepa_init, int num_steps,
                 const double *hard_norm, double rchar, double gamma_inner, double gamma_outer,
                 const double *nden, const double *mtot, int n_mtot, const double *mrat, int n_mrat,
                 const double *redz, int n_redz, const double *gmt_time, const hgb_cosmo *cosmo,
                 double *redz_final, double *diff_num, void *stream) {
    return hgb_dbn_2pwl_phase(fobs_orb, n_freq, fobs_sorted, sepa_init, num_steps, hard_norm, rchar, gamma_inner,
                              gamma_outer, nden, mtot, n_mtot, mrat, n_mrat, redz, n_redz, gmt_time, cosmo,
                              redz_final, diff_num, 3, stream);
}

int hgb_dbn_gw(const double *fobs_orb, int n_freq, const double *nden, const double *mtot, int n_mtot,
               const double *mrat, int n_mrat, int n_redz, const double *redz_prime, const hgb_cosmo *cosmo,
               double *redz_final, double *diff_num, void *stream) {
    HGB_CHECK_ARG(fobs_orb && nden && mtot && mrat && redz_prime && cosmo && redz_final && diff_num);
    HGB_CHECK_ARG(n_freq > 0 && n_mtot > 0 && n_mrat > 0 && n_redz > 0);
    HGB_CHECK_ARG(cosmo->grid_size >= 2 && cosmo->grid_z && cosmo->grid_dcom);
    long n = (long)n_mtot * n_mrat * n_redz;
    int threads = 128;
    k_dbn_gw<<<(unsigned)hgb::ceil_div(n, threads), threads, 0, (cudaStream_t)stream>>>(
        hgb::cy_const(), fobs_orb, n_freq, nden, mtot, n_mtot, mrat, n_mrat, n_redz, redz_prime, cosmo->grid_z,
        cosmo->grid_dcom, cosmo->grid_size, redz_final, diff_num);
    return hgb::check_launch();
}

}  // extern "C"
