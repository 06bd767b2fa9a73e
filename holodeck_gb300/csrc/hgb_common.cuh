// Shared device helpers for the holodeck_gb300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "holodeck_gb300.h"

// ---- constants hard-coded in holodeck/sams/sam_cyutils.pyx:30-42 (the Cython kernels' set)
#define HGB_CY_NWTG 6.6742999e-08
#define HGB_CY_SPLC 29979245800.0
#define HGB_CY_MPC 3.08567758e+24
#define HGB_CY_SCHW 1.4852320538237328e-28
#define HGB_PI 3.14159265358979323846

// ---- astropy CODATA-2018 values used by the Python stages (holodeck/constants.py:23-55)
#define HGB_NWTG 6.6743e-08
#define HGB_SPLC 29979245800.0

namespace hgb {

void set_cuda_error(cudaError_t err);
int check_launch();

// Loudest-first argsort at the first frequency (hgb_sort.cu): scratch bytes for n_bins, and the sort
// itself with the caller's scratch (at least argsort_f0_scratch_bytes(n_bins), 256-byte aligned).
size_t argsort_f0_scratch_bytes(long n_bins);
int argsort_f0_desc_into(const double *h2fdf, long n_bins, int n_freq, int32_t *order, void *scratch,
                         cudaStream_t st);

__device__ __forceinline__ void flag(int *d_status, int bits) {
    if (d_status) atomicOr(d_status, bits);
}

// Compile-time-switchable bounds checks: in a library built with -DHGB_BOUNDS_CHECK,
// HGB_IN_BOUNDS(cond, status) flags HGB_STATUS_BOUNDS when cond is false and yields cond, so the
// caller skips (or clamps) the access; otherwise it is the constant true and costs nothing.
__device__ __forceinline__ bool in_bounds(bool ok, int *d_status) {
    if (!ok) flag(d_status, HGB_STATUS_BOUNDS);
    return ok;
}
#ifdef HGB_BOUNDS_CHECK
#define HGB_IN_BOUNDS(cond, status) (hgb::in_bounds((cond), (status)))
#else
#define HGB_IN_BOUNDS(cond, status) (true)
#endif

// Derived constants of the Cython kernels (sam_cyutils.pyx:38-42), evaluated once on the host
// with the host C library in the same operation order as the Cython module initialisation.
struct CyConst {
    double c_dadt;   // GW_DADT_SEP_CONST = -64 G^3 / 5 / c^5
    double kfreq;    // KEPLER_CONST_FREQ = (1/(2 pi)) sqrt(G)
    double ksepa;    // KEPLER_CONST_SEPA = G^(1/3) / (2 pi)^(2/3)
    double fourpi;   // FOUR_PI_SPLC_OVER_MPC = 4 pi c / Mpc
};
CyConst cy_const();

// sam_cyutils.pyx:46-49
__device__ __forceinline__ double hard_gw(double c_dadt, double mtot, double mrat, double sepa) {
    return c_dadt * pow(mtot, 3.0) * mrat / pow(sepa, 3.0) / pow(1.0 + mrat, 2.0);
}

// sam_cyutils.pyx:240-253: (-norm * (1+x)^(gi-go)) / x^(gi-1) + GW term
__device__ __forceinline__ double hard_func_2pwl_gw(double c_dadt, double mt, double mr, double sepa, double norm,
                                                     double rchar, double gi, double go) {
    double xx = sepa / rchar;
    double dadt = -norm * pow(1.0 + xx, -go + gi) / pow(xx, gi - 1.0);
    dadt += hard_gw(c_dadt, mt, mr, sepa);
    return dadt;
}

// holodeck/cyutils.pyx:326-358
__device__ __forceinline__ double interp_between(double xnew, double xl, double xr, double yl, double yr) {
    return yl + (yr - yl) * (xnew - xl) / (xr - xl);
}

// sam_cyutils.pyx:66-85, the bracket index of `val` in an increasing table, walking from `start`
__device__ __forceinline__ int while_while_increasing(int start, int size, double val, const double *edges) {
    int index = start;
    while ((index < size - 2) && (edges[index + 1] < val)) index += 1;
    while ((index > 0) && (edges[index] > val)) index -= 1;
    return index;
}

// The index sam_cyutils.pyx:88-107 reaches when walking forward from 0 through a decreasing table:
// the first i with edges[i+1] <= val, capped at size-1.
__device__ __forceinline__ int bracket_decreasing_from0(int size, double val, const double *edges) {
    int lo = 0, hi = size - 1;   // answer in [0, size-1]
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (edges[mid + 1] > val) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Comoving distance [cm] from the Hermite table in u = sqrt(1/(1+z)).
__device__ __forceinline__ double comoving_distance(const double *dval, const double *dder, int n, double z) {
    double u = sqrt(1.0 / (1.0 + z));
    double x = u * (double)n;
    int k = (int)x;
    if (k >= n) k = n - 1;
    if (k < 0) k = 0;
    double t = x - (double)k;
    double h = 1.0 / (double)n;
    double t2 = t * t, t3 = t2 * t;
    double h00 = 2.0 * t3 - 3.0 * t2 + 1.0;
    double h10 = t3 - 2.0 * t2 + t;
    double h01 = -2.0 * t3 + 3.0 * t2;
    double h11 = t3 - t2;
    return h00 * dval[k] + h10 * h * dder[k] + h01 * dval[k + 1] + h11 * h * dder[k + 1];
}

// The same lookup for z >= 0 with u = (1 + z)^(-1/2) from an FP32 estimate and one FP64 Newton
// step, u (3 - y u^2) / 2 (relative error about 1e-14, far below the table's own), and h = 1 / n
// supplied by the caller: about a third of the FP64 work of comoving_distance.
__device__ __forceinline__ double comoving_distance_fast(const double *dval, const double *dder, int n, double h,
                                                         double z) {
    const double y = 1.0 + z;
    const double u0 = (double)rsqrtf((float)y);
    const double u = u0 * (3.0 - y * (u0 * u0)) * 0.5;
    double x = u * (double)n;
    int k = (int)x;
    if (k >= n) k = n - 1;
    if (k < 0) k = 0;
    double t = x - (double)k;
    double t2 = t * t, t3 = t2 * t;
    double h00 = 2.0 * t3 - 3.0 * t2 + 1.0;
    double h10 = t3 - 2.0 * t2 + t;
    double h01 = -2.0 * t3 + 3.0 * t2;
    double h11 = t3 - t2;
    return h00 * dval[k] + h10 * h * dder[k] + h01 * dval[k + 1] + h11 * h * dder[k + 1];
}

// ---- FP32-mode helpers.  On this GPU an FP64 instruction costs a warp about as much issue time as
// 32 FP32 ones, so the FP32 kernels move values between the FP64 arrays of the API and FP32
// registers with integer operations instead of FP64 conversions.

// x rounded toward zero to float; |x| below FLT_MIN gives a signed zero, beyond FLT_MAX +-inf
// (NaN stays NaN).  Relative error below 2^-23.
__device__ __forceinline__ float f64_to_f32_rz(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const int ex = (int)((hi >> 20) & 0x7FFu);
    const int e = ex - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (ex == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (((hi & 0xFFFFFu) | lo) ? 0x400000u : 0u));
    if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((unsigned)e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
}

// v * 2^k as a double, exactly, for a float v that is zero, normal, inf or NaN (a subnormal v gives
// a signed zero); |k| must keep the result inside the double range.
__device__ __forceinline__ double f32_to_f64_scaled(float v, int k) {
    const unsigned u = __float_as_uint(v);
    const unsigned sign = u & 0x80000000u;
    const int ef = (int)((u >> 23) & 0xFFu);
    if (ef == 0) return __longlong_as_double((long long)((unsigned long long)sign << 32));
    unsigned hi;
    if (ef == 0xFF) hi = sign | 0x7FF00000u | ((u & 0x7FFFFFu) ? 0x80000u : 0u);
    else hi = sign | ((unsigned)(ef - 127 + 1023 + k) << 20) | ((u & 0x7FFFFFu) >> 3);
    const unsigned lo = (u & 0x7u) << 29;
    return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}

// the bit pattern of -1.0, the "no target reached" sentinel of redz_final
constexpr long long F64_MINUS_ONE_BITS = (long long)0xBFF0000000000000ull;

// Kahan-compensated FP32 accumulator
struct Kahan32 {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

__host__ __device__ __forceinline__ long ceil_div(long a, long b) { return (a + b - 1) / b; }

// Multiprocessor count of the current device (queried once per device, 152 on a GB300).
int sm_count();

// Make `func` launchable with `bytes` of dynamic shared memory on the current device.  The cap
// (cudaFuncAttributeMaxDynamicSharedMemorySize) is per function and shared by every host thread, so
// it is only ever raised, under a lock: a thread that sets a smaller cap between another thread's
// set and launch would make that launch fail with cudaErrorLaunchOutOfResources.
int ensure_dyn_smem(const void *func, size_t bytes);

}  // namespace hgb

#define HGB_CHECK_ARG(cond)                        \
    do {                                           \
        if (!(cond)) return HGB_ERR_INVALID_ARGUMENT; \
    } while (0)
