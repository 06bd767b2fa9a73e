// M-Mbulge scatter of the binary density (holodeck/sams/sam.py:1291-1394, add_scatter_to_masses),
// one redshift slice per batch entry, on the geometry prepared by hgb_scatter_plan_build:
//   1. k_gradients: per-point gradients of the slice's density by the minimum-norm-network method
//      (Nielson 1983; the gradient estimate behind scipy's CloughTocher2DInterpolator): Gauss-Seidel
//      sweeps in point order, each point's 2x2 normal system solved with its precomputed inverse,
//      until the largest relative change of a sweep falls below `grad_tol`.  One block per slice;
//      the points of one wavefront level update concurrently and read exactly the neighbour values a
//      sequential sweep would read, so the iterates equal the sequential ones.
//   2. k_clough_tocher: the C1 piecewise-cubic Clough-Tocher interpolant (centroid split) at every
//      node of the regular (log m1, log m2) grid; NaN outside the hull; NaN or negative values are
//      replaced by the value of the nearest point.
//   3. k_gemm_f64 twice: out = W^T G W, the Gaussian redistribution along both mass axes.
//   4. k_back: bilinear interpolation of the redistributed grid back to the points.
// FP64 throughout; built with -fmad=false.
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
    grid[z * NN + node] = val;
}

// ---- 3. batched FP64 GEMM  C[b] = op(X) Y   (N x N), tiles 64 x 64 x 16, 4 x 4 outputs per thread
// X_T: X element (row, k) = X[k * N + row] (transposed access); X / Y batch strides may be 0 (shared).
template <bool X_T>
__global__ void __launch_bounds__(256) k_gemm_f64(int N, const double *__restrict__ X, long sx,
                                                  const double *__restrict__ Y, long sy, double *__restrict__ C, long sc) {
    __shared__ double Xs[16][64 + 1];
    __shared__ double Ys[16][64 + 1];
    const int b = blockIdx.z;
    const double *Xb = X + (long)b * sx;
    const double *Yb = Y + (long)b * sy;
    double *Cb = C + (long)b * sc;
    const int row0 = blockIdx.y * 64, col0 = blockIdx.x * 64;
    const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
    for (int k0 = 0; k0 < N; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            int kk = e / 64, rr = e % 64;
            int row = row0 + rr, k = k0 + kk;
            double xv = 0.0;
            if (row < N && k < N) xv = X_T ? Xb[(long)k * N + row] : Xb[(long)row * N + k];
            Xs[kk][rr] = xv;
            int col = col0 + rr;
            Ys[kk][rr] = (col < N && k < N) ? Yb[(long)k * N + col] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            double xr[4], yc[4];
#pragma unroll
            for (int i = 0; i < 4; i++) xr[i] = Xs[kk][tr * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) yc[j] = Ys[kk][tc * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] += xr[i] * yc[j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int row = row0 + tr * 4 + i;
        if (row >= N) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int col = col0 + tc * 4 + j;
            if (col < N) Cb[(long)row * N + col] = acc[i][j];
        }
    }
}

// ---- 4. bilinear interpolation back to the points
__global__ void k_back(hgb_scatter_plan P, const double *__restrict__ grid, int nz, double *__restrict__ dens) {
    const int n = P.n_mtot * P.n_mrat;
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)n * nz) return;
    const int i = (int)(idx / nz), z = (int)(idx % nz);
    const long NN = (long)P.n_grid * P.n_grid;
    const double *G = grid + z * NN;
    const int a = P.back_idx[2 * i], b = P.back_idx[2 * i + 1];
    const double tx = P.back_t[2 * i], ty = P.back_t[2 * i + 1];
    const long N = P.n_grid;
    const double v00 = G[a * N + b], v01 = G[a * N + b + 1], v10 = G[(a + 1) * N + b], v11 = G[(a + 1) * N + b + 1];
    dens[idx] = v00 * (1.0 - tx) * (1.0 - ty) + v01 * (1.0 - tx) * ty + v10 * tx * (1.0 - ty) + v11 * tx * ty;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

size_t hgb_scatter_workspace_bytes(int n_mtot, int n_mrat, int n_redz, int n_grid) {
    if (n_mtot < 2 || n_mrat < 2 || n_redz < 1 || n_grid < 2) return 0;
    size_t n = (size_t)n_mtot * n_mrat, NN = (size_t)n_grid * n_grid;
    return align256(sizeof(double) * n * n_redz) + align256(sizeof(double) * 2 * n * n_redz) +
           2 * align256(sizeof(double) * NN * n_redz);
}

int hgb_add_scatter_to_masses(const hgb_scatter_plan *plan, double *dens, int n_redz, void *workspace,
                              size_t workspace_bytes, int *d_status, void *stream) {
    HGB_CHECK_ARG(plan && dens && n_redz >= 1);
    const hgb_scatter_plan &P = *plan;
    HGB_CHECK_ARG(P.n_mtot >= 2 && P.n_mrat >= 2 && P.n_grid >= 2 && P.n_levels >= 1);
    HGB_CHECK_ARG(P.pts && P.tri && P.tri_kappa && P.vtx_qinv && P.nbr_ptr && P.nbr_idx && P.nbr_w);
    HGB_CHECK_ARG(P.level_ptr && P.level_vtx && P.grid_tri && P.grid_bary && P.grid_near && P.weights);
    HGB_CHECK_ARG(P.back_idx && P.back_t && P.grad_maxiter >= 1);
    size_t need = hgb_scatter_workspace_bytes(P.n_mtot, P.n_mrat, n_redz, P.n_grid);
    if (!workspace || workspace_bytes < need) return HGB_ERR_WORKSPACE;
    const size_t n = (size_t)P.n_mtot * P.n_mrat, NN = (size_t)P.n_grid * P.n_grid;
    char *w = (char *)workspace;
    double *vals = (double *)w;
    w += align256(sizeof(double) * n * n_redz);
    double *grads = (double *)w;
    w += align256(sizeof(double) * 2 * n * n_redz);
    double *gridA = (double *)w;
    w += align256(sizeof(double) * NN * n_redz);
    double *gridB = (double *)w;
    cudaStream_t st = (cudaStream_t)stream;

    k_gradients<<<n_redz, 256, 0, st>>>(P, dens, n_redz, vals, grads, d_status);
    int rc = hgb::check_launch();
    if (rc) return rc;
    dim3 gct((unsigned)hgb::ceil_div((long)NN, 256), (unsigned)n_redz);
    k_clough_tocher<<<gct, 256, 0, st>>>(P, vals, grads, gridA);
    if ((rc = hgb::check_launch())) return rc;
    const int N = P.n_grid;
    dim3 gg((unsigned)hgb::ceil_div(N, 64), (unsigned)hgb::ceil_div(N, 64), (unsigned)n_redz);
    // along the primary-mass axis: B = W^T A  (utils.py:454-461, einsum "j...,jk...")
    k_gemm_f64<true><<<gg, 256, 0, st>>>(N, P.weights, 0, gridA, (long)NN, gridB, (long)NN);
    if ((rc = hgb::check_launch())) return rc;
    // along the secondary-mass axis: A = B W
    k_gemm_f64<false><<<gg, 256, 0, st>>>(N, gridB, (long)NN, P.weights, 0, gridA, (long)NN);
    if ((rc = hgb::check_launch())) return rc;
    k_back<<<(unsigned)hgb::ceil_div((long)n * n_redz, 256), 256, 0, st>>>(P, gridA, n_redz, dens);
    return hgb::check_launch();
}

}  // extern "C"
