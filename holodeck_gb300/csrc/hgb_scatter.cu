// M-Mbulge scatter of the binary density (holodeck/sams/sam.py:1291-1394, add_scatter_to_masses),
// one redshift slice per batch entry, on the geometry prepared by hgb_scatter_plan_build:
//   1. k_gradients: per-point gradients of the slice's density by the minimum-norm-network method
//      (Nielson 1983; the gradient estimate behind scipy's CloughTocher2DInterpolator): Gauss-Seidel
//      sweeps in point order, each point's 2x2 normal system solved with its precomputed inverse,
//      until the largest relative change of a sweep falls below `grad_tol`.  One block per slice;
//      the points of one wavefront level update concurrently and read exactly the neighbour values a
//      sequential sweep would read, so the iterates equal the sequential ones.  k_gradients_lv keeps
//      the slice in shared memory when it fits (grids up to ~9000 points).
//   2. k_clough_tocher: the C1 piecewise-cubic Clough-Tocher interpolant (centroid split) at every
//      node of the regular (log m1, log m2) grid; NaN outside the hull; NaN or negative values are
//      replaced by the value of the nearest point.
//   3. k_back_dot: the Gaussian redistribution W^T (W^T G) as the reference computes it (see
//      hgb_add_scatter_to_masses) followed by the bilinear interpolation back to the points, fused
//      into one dot product per (point, slice) with the plan's per-point row of (W W).
// FP64 throughout; built with -fmad=false (k_gradients_lv fuses its multiply-adds explicitly).
#include <math.h>

#include "hgb_common.cuh"

namespace {

// ---- 1. gradients
__global__ void k_gradients(hgb_scatter_plan P, const double *__restrict__ dens, int nz, double *__restrict__ vals,
                            double *__restrict__ grads, int *d_status) {
    const int z = blockIdx.x;
    const int n = P.n_mtot * P.n_mrat;
    double *f = vals + (long)z * n;
    double *g = grads + 2L * z * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        f[i] = dens[(long)i * nz + z];
        g[2 * i] = 0.0;
        g[2 * i + 1] = 0.0;
    }
    __shared__ double s_err[32];
    __syncthreads();
    bool converged = false;
    for (int it = 0; it < P.grad_maxiter; it++) {
        double err = 0.0;
        for (int lev = 0; lev < P.n_levels; lev++) {
            const int e0 = P.level_ptr[lev], e1 = P.level_ptr[lev + 1];
            for (int idx = e0 + threadIdx.x; idx < e1; idx += blockDim.x) {
                const int i = P.level_vtx[idx];
                const double fi = f[i];
                double sx = 0.0, sy = 0.0;
                for (int p = P.nbr_ptr[i]; p < P.nbr_ptr[i + 1]; p++) {
                    const int j = P.nbr_idx[p];
                    const double ex = P.nbr_w[4 * p], ey = P.nbr_w[4 * p + 1];
                    const double c = 6.0 * (f[j] - fi) - 2.0 * (g[2 * j] * ex + g[2 * j + 1] * ey);
                    sx += c * P.nbr_w[4 * p + 2];
                    sy += c * P.nbr_w[4 * p + 3];
                }
                const double *qi = P.vtx_qinv + 4 * i;
                const double nx = qi[0] * sx + qi[1] * sy;
                const double ny = qi[2] * sx + qi[3] * sy;
                double change = fmax(fabs(nx - g[2 * i]), fabs(ny - g[2 * i + 1]));
                change /= fmax(1.0, fmax(fabs(nx), fabs(ny)));
                err = fmax(err, change);
                g[2 * i] = nx;
                g[2 * i + 1] = ny;
            }
            __syncthreads();
        }
        // block-wide maximum of the sweep's relative change
        for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_xor_sync(0xffffffffu, err, o));
        if ((threadIdx.x & 31) == 0) s_err[threadIdx.x >> 5] = err;
        __syncthreads();
        if (threadIdx.x < 32) {
            double e = (threadIdx.x < (blockDim.x >> 5)) ? s_err[threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) e = fmax(e, __shfl_xor_sync(0xffffffffu, e, o));
            if (threadIdx.x == 0) s_err[0] = e;
        }
        __syncthreads();
        converged = s_err[0] < P.grad_tol;
        __syncthreads();
        if (converged) break;
    }
    if (!converged && threadIdx.x == 0) hgb::flag(d_status, HGB_STATUS_GRADIENT_NOT_CONVERGED);
}

// The same solve with the slice's values and gradients in shared memory, indexed by level-order
// position (a level's points are contiguous), for grids whose state fits on one SM.  GB300's FP64
// units belong to the four SM sub-partitions and charge each warp instruction in full however few
// lanes are active, so the block has four warps, one per sub-partition, and the per-level work is
// spread so that no sub-partition carries much more than a quarter of it:
//   * a level's points (about 20 at 91x81) share the lanes of every warp; warp w sums the terms of
//     edges o, o+4, o+8, ... of its point with o = (w + 2) mod 4, so an interior point's six edges
//     put two terms on warps 2 and 3 and one on warps 0 and 1;
//   * warps 0 and 1 add the four partial sums and solve the x and the y component of the point's
//     2x2 system respectively;
//   * warp 2 evaluates the convergence test of the previous 32 points (their changes and magnitudes,
//     double-buffered in shared memory) while warps 0 and 1 update the current ones.
// The static data of the next level (each warp's first LV_REG edges of its point, the rows of the
// inverse normal matrix that warps 0 and 1 use) is loaded into registers while the current level
// computes.  Per point the terms and the test are those of k_gradients, with two differences of
// rounding: the neighbour sum is grouped as four interleaved partial sums, and the multiply-adds are
// fused (explicit __fma_rn, the file being built with -fmad=false).  An edge term
//   c = 6 (f_j - f_i) - 2 (g_jx w0 + g_jy w1),  sx += c w2,  sy += c w3
// takes 6 FP64 instructions instead of 11: the plan stores -2 w0 and -2 w1 (an exact scaling), so
//   t = fma(g_jy, -2 w1, g_jx (-2 w0)),  c = fma(6, f_j - f_i, t),  sx = fma(c, w2, sx),  sy = fma(c, w3, sy),
// and the 2x2 solve takes 2 instead of 3.  The FP64 pipe bounds this kernel, so the instruction
// count is its time; each fused operation skips one rounding (an ulp of the term).
constexpr int LV_WARPS = 4;
constexpr int LV_REG = 3;   // edges o, o+4, o+8 per warp: interior points have 6 neighbours

__device__ __forceinline__ int lv_edge_offset(int warp) { return (warp + 2) & (LV_WARPS - 1); }

struct LvPre {
    int e0, e1;
    int idx[LV_REG];
    double2 w01[LV_REG], w23[LV_REG];
    double2 q;   // warps 0 / 1: row 0 / 1 of the point's inverse normal matrix
};

__device__ __forceinline__ void lv_load(const hgb_scatter_plan &P, const int *eptr, int p, bool active, int warp,
                                        LvPre &x) {
    x.e0 = active ? eptr[p] : 0;
    x.e1 = active ? eptr[p + 1] : 0;
#pragma unroll
    for (int k = 0; k < LV_REG; k++) {
        const int e = x.e0 + lv_edge_offset(warp) + LV_WARPS * k;
        if (e < x.e1) {
            x.idx[k] = __ldg(P.lv_nbr + e);
            x.w01[k] = __ldg((const double2 *)(P.lv_nbr_w + 4 * (long)e));
            x.w23[k] = __ldg((const double2 *)(P.lv_nbr_w + 4 * (long)e + 2));
        }
    }
    if (active && warp < 2) x.q = __ldg((const double2 *)(P.lv_qinv + 4 * (long)p + 2 * warp));   // row `warp`
}

__global__ void __launch_bounds__(32 * LV_WARPS, 1) k_gradients_lv(hgb_scatter_plan P, const double *__restrict__ dens,
                                                                  int nz, double *__restrict__ vals,
                                                                  double *__restrict__ grads, int *d_status) {
    extern __shared__ double sm[];
    __shared__ double psx[LV_WARPS][32], psy[LV_WARPS][32];
    __shared__ double chg[2][2][32], mag[2][2][32];   // [chunk parity][component][lane]: |change|, |new value|
    __shared__ int s_over;
    const int z = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int n = P.n_mtot * P.n_mrat;
    double *f = sm;                                  // [n]
    double *g = f + n;                               // [n][2]
    int *eptr = (int *)(g + 2 * n);                  // [n + 1]
    int *lptr = eptr + n + 1;                        // [n_levels + 1]
    for (int p = t; p < n; p += blockDim.x) {
        const int i = P.level_vtx[p];
        const double v = dens[(long)i * nz + z];
        f[p] = v;
        vals[(long)z * n + i] = v;
        g[2 * p] = 0.0;
        g[2 * p + 1] = 0.0;
        eptr[p] = P.lv_nbr_ptr[p];
    }
    if (t == 0) eptr[n] = P.lv_nbr_ptr[n];
    for (int l = t; l <= P.n_levels; l += blockDim.x) lptr[l] = P.level_ptr[l];
    __syncthreads();
    const int nlev = P.n_levels;
    const double tol_lo = P.grad_tol * (1.0 - 1e-12);   // below this multiple of the scale: surely < tol
    bool converged = false;
    LvPre nxt;
    lv_load(P, eptr, lptr[0] + lane, lane < lptr[1] - lptr[0], warp, nxt);
    // exact test of one chunk's points from the buffered changes and magnitudes (warp 2)
    auto test_chunk = [&](int b, bool over) {
        const double change = fmax(chg[b][0][lane], chg[b][1][lane]);
        const double scale = fmax(1.0, fmax(mag[b][0][lane], mag[b][1][lane]));
        // relative change, divided out only where the comparison with the tolerance is close (the
        // decision is that of change / scale < tol)
        if (change >= tol_lo * scale) over = over || (change / scale >= P.grad_tol);
        return over;
    };
    for (int it = 0; it < P.grad_maxiter; it++) {
        bool over = false;   // (warp 2) some point changed by >= grad_tol (relative) in this sweep
        int kc = 0;          // chunks updated so far in this sweep
        for (int lev = 0; lev < nlev; lev++) {
            const int p0 = lptr[lev], p1 = lptr[lev + 1];
            const LvPre cur = nxt;
            {   // the next level (the first level again after the last), loaded ahead
                const int nl = (lev + 1 < nlev) ? lev + 1 : 0;
                const int q0 = lptr[nl], q1 = lptr[nl + 1];
                lv_load(P, eptr, q0 + lane, lane < q1 - q0, warp, nxt);
            }
            for (int c0 = p0; c0 < p1; c0 += 32) {   // 32 points at a time (one pass at 91x81)
                const int p = c0 + lane;
                const bool act = p < p1;
                const bool pre = (c0 == p0);         // the prefetched chunk; wider levels load directly
                double sx = 0.0, sy = 0.0;
                if (act) {
                    const double fi = f[p];
                    const int e0 = pre ? cur.e0 : eptr[p], e1 = pre ? cur.e1 : eptr[p + 1];
                    int e = e0 + lv_edge_offset(warp);
                    if (pre) {
#pragma unroll
                        for (int k = 0; k < LV_REG; k++) {
                            if (e < e1) {
                                const int j = cur.idx[k];
                                const double tt = __fma_rn(g[2 * j + 1], cur.w01[k].y, g[2 * j] * cur.w01[k].x);
                                const double cc = __fma_rn(6.0, f[j] - fi, tt);
                                sx = __fma_rn(cc, cur.w23[k].x, sx);
                                sy = __fma_rn(cc, cur.w23[k].y, sy);
                            }
                            e += LV_WARPS;
                        }
                    }
                    for (; e < e1; e += LV_WARPS) {
                        const int j = __ldg(P.lv_nbr + e);
                        const double2 w01 = __ldg((const double2 *)(P.lv_nbr_w + 4 * (long)e));
                        const double2 w23 = __ldg((const double2 *)(P.lv_nbr_w + 4 * (long)e + 2));
                        const double tt = __fma_rn(g[2 * j + 1], w01.y, g[2 * j] * w01.x);
                        const double cc = __fma_rn(6.0, f[j] - fi, tt);
                        sx = __fma_rn(cc, w23.x, sx);
                        sy = __fma_rn(cc, w23.y, sy);
                    }
                }
                psx[warp][lane] = sx;
                psy[warp][lane] = sy;
                __syncthreads();
                const int b = kc & 1;
                if (warp < 2) {   // warp 0 solves the x component, warp 1 the y component
                    double dv = 0.0, av = 0.0;
                    if (act) {
                        const double tx = ((psx[0][lane] + psx[1][lane]) + psx[2][lane]) + psx[3][lane];
                        const double ty = ((psy[0][lane] + psy[1][lane]) + psy[2][lane]) + psy[3][lane];
                        const double2 q = pre ? cur.q : __ldg((const double2 *)(P.lv_qinv + 4 * (long)p + 2 * warp));
                        const double nv = __fma_rn(q.y, ty, q.x * tx);
                        dv = fabs(nv - g[2 * p + warp]);
                        av = fabs(nv);
                        g[2 * p + warp] = nv;
                    }
                    chg[b][warp][lane] = dv;
                    mag[b][warp][lane] = av;
                } else if (warp == 2 && kc > 0) {
                    over = test_chunk(b ^ 1, over);   // the previous chunk, while this one updates
                }
                __syncthreads();
                kc++;
            }
        }
        if (warp == 2) {
            if (kc > 0) over = test_chunk((kc - 1) & 1, over);   // the sweep's last chunk
            const bool any = __any_sync(0xffffffffu, over);
            if (lane == 0) s_over = any ? 1 : 0;
        }
        __syncthreads();
        converged = (s_over == 0);
        __syncthreads();
        if (converged) break;
    }
    if (!converged && t == 0) hgb::flag(d_status, HGB_STATUS_GRADIENT_NOT_CONVERGED);
    for (int p = t; p < n; p += blockDim.x) {
        const int i = P.level_vtx[p];
        grads[2L * z * n + 2 * i] = g[2 * p];
        grads[2L * z * n + 2 * i + 1] = g[2 * p + 1];
    }
}

size_t gradients_lv_smem(const hgb_scatter_plan &P) {
    const size_t n = (size_t)P.n_mtot * P.n_mrat;
    return sizeof(double) * 3 * n + sizeof(int) * (n + 1) + sizeof(int) * (P.n_levels + 1);
}

// ---- 2. Clough-Tocher value at barycentric (l0, l1, l2) of triangle r
__device__ double clough_tocher(const hgb_scatter_plan &P, int r, const double *lam, const double *f,
                                const double *g) {
    int v[3];
    double px[3], py[3], fv[3], gx[3], gy[3], kap[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        v[k] = P.tri[3 * r + k];
        px[k] = P.pts[2 * v[k]];
        py[k] = P.pts[2 * v[k] + 1];
        fv[k] = f[v[k]];
        gx[k] = g[2 * v[k]];
        gy[k] = g[2 * v[k] + 1];
        kap[k] = P.tri_kappa[3 * r + k];
    }
    const double cx = (px[0] + px[1] + px[2]) / 3.0, cy = (py[0] + py[1] + py[2]) / 3.0;
    double al[3], beta[3], ee[3][3];   // ee[i][j]: ordinate on edge i -> j next to vertex i
#pragma unroll
    for (int i = 0; i < 3; i++) {
        al[i] = fv[i] + (gx[i] * (cx - px[i]) + gy[i] * (cy - py[i])) / 3.0;
#pragma unroll
        for (int j = 0; j < 3; j++)
            ee[i][j] = (i == j) ? 0.0 : fv[i] + (gx[i] * (px[j] - px[i]) + gy[i] * (py[j] - py[i])) / 3.0;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int i = (k + 1) % 3, j = (k + 2) % 3;
        const double b210 = ee[i][j], b120 = ee[j][i];
        const double q20 = 3.0 * (al[i] - 0.5 * fv[i] - 0.5 * b210);
        const double q02 = 3.0 * (al[j] - 0.5 * b120 - 0.5 * fv[j]);
        const double t20 = 3.0 * (b210 - fv[i]), t11 = 3.0 * (b120 - b210), t02 = 3.0 * (fv[j] - b120);
        const double q11 = 0.5 * (q20 + q02) + kap[k] * (t11 - 0.5 * (t20 + t02));
        beta[k] = 0.5 * (b210 + b120) + q11 / 3.0;
    }
    double gam[3];
#pragma unroll
    for (int i = 0; i < 3; i++) gam[i] = (al[i] + beta[(i + 1) % 3] + beta[(i + 2) % 3]) / 3.0;
    const double cen = (gam[0] + gam[1] + gam[2]) / 3.0;
    // micro-triangle (P_i, P_j, centroid) opposite the smallest barycentric coordinate
    int k = 0;
    if (lam[1] < lam[k]) k = 1;
    if (lam[2] < lam[k]) k = 2;
    const int i = (k + 1) % 3, j = (k + 2) % 3;
    const double a = lam[i] - lam[k], b = lam[j] - lam[k], c = 3.0 * lam[k];
    const double a2 = a * a, b2 = b * b, c2 = c * c;
    return fv[i] * a2 * a + fv[j] * b2 * b + cen * c2 * c + 3.0 * (ee[i][j] * a2 * b + ee[j][i] * a * b2) +
           3.0 * (al[i] * a2 * c + al[j] * b2 * c) + 3.0 * (gam[i] * a * c2 + gam[j] * b * c2) +
           6.0 * beta[k] * a * b * c;
}

__global__ void k_clough_tocher(hgb_scatter_plan P, const double *__restrict__ vals, const double *__restrict__ grads,
                                double *__restrict__ grid) {
    const int z = blockIdx.y;
    const long NN = (long)P.n_grid * P.n_grid;
    const long node = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= NN) return;
    const int n = P.n_mtot * P.n_mrat;
    const double *f = vals + (long)z * n;
    const double *g = grads + 2L * z * n;
    const int r = P.grid_tri[node];
    double val = NAN;
    if (r >= 0) {
        double lam[3] = {P.grid_bary[3 * node], P.grid_bary[3 * node + 1], P.grid_bary[3 * node + 2]};
        val = clough_tocher(P, r, lam, f, g);
    }
    if (isnan(val) || val < 0.0) val = f[P.grid_near[node]];   // sam.py:1367-1376
    // stored transposed, [z][b][a], so that a point's two m2-columns are contiguous rows
    const long a = node / P.n_grid, b = node % P.n_grid;
    grid[z * NN + b * P.n_grid + a] = val;
}

// ---- 3+4. redistribution and bilinear interpolation back to the points, as one dot product per
// (point, slice): out = sum_j bw_i[j] ((1 - ty) G[j][b] + ty G[j][b + 1]), with the two weight rows
// (1 - ty) bw_i and ty bw_i precomputed, two fused multiply-adds per element; one warp per output.
__global__ void k_back_dot(hgb_scatter_plan P, const double *__restrict__ gridT, int nz, double *__restrict__ dens) {
    const int n = P.n_mtot * P.n_mrat;
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= (long)n * nz) return;
    const int i = (int)(warp / nz), z = (int)(warp % nz);
    const long N = P.n_grid;
    const int b = P.back_idx[2 * i + 1];
    const double *row0 = gridT + (long)z * N * N + (long)b * N;
    const double *row1 = row0 + N;
    const double *w0 = P.back_w + 2L * i * N;   // (1 - ty) bw_i
    const double *w1 = w0 + N;                 // ty bw_i
    double acc = 0.0;
    for (int j = lane; j < N; j += 32) acc = __fma_rn(w0[j], row0[j], __fma_rn(w1[j], row1[j], acc));
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) dens[(long)i * nz + z] = acc;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

size_t hgb_scatter_workspace_bytes(int n_mtot, int n_mrat, int n_redz, int n_grid) {
    if (n_mtot < 2 || n_mrat < 2 || n_redz < 1 || n_grid < 2) return 0;
    size_t n = (size_t)n_mtot * n_mrat, NN = (size_t)n_grid * n_grid;
    return align256(sizeof(double) * n * n_redz) + align256(sizeof(double) * 2 * n * n_redz) +
           align256(sizeof(double) * NN * n_redz);
}

int hgb_add_scatter_to_masses(const hgb_scatter_plan *plan, double *dens, int n_redz, void *workspace,
                              size_t workspace_bytes, int *d_status, void *stream) {
    HGB_CHECK_ARG(plan && dens && n_redz >= 1);
    const hgb_scatter_plan &P = *plan;
    HGB_CHECK_ARG(P.n_mtot >= 2 && P.n_mrat >= 2 && P.n_grid >= 2 && P.n_levels >= 1);
    HGB_CHECK_ARG(P.pts && P.tri && P.tri_kappa && P.vtx_qinv && P.nbr_ptr && P.nbr_idx && P.nbr_w);
    HGB_CHECK_ARG(P.level_ptr && P.level_vtx && P.grid_tri && P.grid_bary && P.grid_near);
    HGB_CHECK_ARG(P.back_idx && P.back_t && P.back_w && P.grad_maxiter >= 1);
    size_t need = hgb_scatter_workspace_bytes(P.n_mtot, P.n_mrat, n_redz, P.n_grid);
    if (!workspace || workspace_bytes < need) return HGB_ERR_WORKSPACE;
    const size_t n = (size_t)P.n_mtot * P.n_mrat, NN = (size_t)P.n_grid * P.n_grid;
    char *w = (char *)workspace;
    double *vals = (double *)w;
    w += align256(sizeof(double) * n * n_redz);
    double *grads = (double *)w;
    w += align256(sizeof(double) * 2 * n * n_redz);
    double *gridA = (double *)w;
    cudaStream_t st = (cudaStream_t)stream;

    const size_t lv_smem = gradients_lv_smem(P);
    int dev = 0, smem_optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (P.lv_nbr_ptr && P.lv_nbr && P.lv_nbr_w && P.lv_qinv && lv_smem + 8192 <= (size_t)smem_optin) {
        const int rc = hgb::ensure_dyn_smem((const void *)k_gradients_lv, lv_smem);
        if (rc) return rc;
        k_gradients_lv<<<n_redz, 32 * LV_WARPS, lv_smem, st>>>(P, dens, n_redz, vals, grads, d_status);
    } else {
        k_gradients<<<n_redz, 256, 0, st>>>(P, dens, n_redz, vals, grads, d_status);
    }
    int rc = hgb::check_launch();
    if (rc) return rc;
    dim3 gct((unsigned)hgb::ceil_div((long)NN, 256), (unsigned)n_redz);
    k_clough_tocher<<<gct, 256, 0, st>>>(P, vals, grads, gridA);
    if ((rc = hgb::check_launch())) return rc;
    const long nwarps = (long)n * n_redz;
    k_back_dot<<<(unsigned)hgb::ceil_div(nwarps * 32, 256), 256, 0, st>>>(P, gridA, n_redz, dens);
    return hgb::check_launch();
}

}  // extern "C"
