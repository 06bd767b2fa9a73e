// Poisson realizations of the binary population with the loudest-source split.
//
// Replaces cyutils.loudest_hc_from_sorted (holodeck/cyutils.pyx:1220-1344) and
// cyutils.sam_poisson_gwb (holodeck/cyutils.pyx:854-897).
//
// Layout: the (B, F) number and h2fdf grids are gathered once into loudest-first order and
// transposed to (F, B), so one frequency's sorted bins are contiguous.  A block owns one
// frequency, up to RB*RPT realizations (RPT per thread, kept in shared memory) and one chunk of
// bins; a chunk is every nchunk-th tile of RB sorted bins, so chunks carry the same mix of cheap
// and expensive bins and finish together.  The block stages a tile in shared memory with its
// per-bin sampler constants -- computed once per bin per block, i.e. amortised over all
// realizations -- and each thread walks the tile in sorted order for its realizations.  All
// threads of a warp see the same bin, so the choice of sampler is warp-uniform and bins with zero
// expectation (most of the grid) cost one shared-memory load per thread.
//
// Draws (HGB_RNG_PHILOX): counter-based Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) keyed by
// the 64-bit seed; counters are built from (sorted bin, realization, frequency, stream word), so
// results do not depend on chunking.  Samplers by expectation lambda:
//   lambda <= 0 or NaN        n = 0, no draw
//   lambda < TINY             geometric skipping over a thread's realizations: the gap to the next
//                             realization with n >= 1 is floor(-ln u / lambda) (P(n = 0) = e^-lambda),
//                             so one 64-bit uniform usually settles all RPT realizations; a hit
//                             draws n from the zero-truncated Poisson
//   TINY <= lambda < 10       inversion of a 64-bit uniform against a per-bin table of
//                             floor(CDF(n) 2^64) (n = 0) and floor(CDF(n) 2^32) (n >= 1); two
//                             realizations per Philox call
//   10 <= lambda < 2^22       PTRS, transformed rejection with squeeze (Hormann 1993, Insurance:
//                             Mathematics and Economics 12, 39-45) in FP32, acceptance test in the
//                             log-pmf form of Loader's saddle-point expansion (bd0 + Stirling
//                             remainder), so nothing cancels in FP32; two realizations' first
//                             attempts per Philox call
//   2^22 <= lambda <= 1e10    PTRS in FP64
//   lambda > 1e10             Normal(lambda, sqrt(lambda)) by Box-Muller, as the reference does
// Counts are integers; background sums accumulate n * h2fdf * 2^100 in FP32 with Kahan
// compensation (relative error ~1e-7 of hc^2); the loudest slots hold the exact float64 h2fdf.
// Every rejection / inversion loop is bounded and flags HGB_STATUS_ITERATION_LIMIT when it runs out.
//
// Replay (HGB_RNG_REPLAY): the caller supplies the draws in the reference's order (numpy's PCG64
// stream); one thread per (frequency, realization) walks all bins sequentially and accumulates in
// float64 with round-to-nearest multiply and add, which reproduces the reference bit for bit.
#include <math.h>
#include <stdint.h>

#include "hgb_common.cuh"

namespace {

constexpr int RB = 128;                  // threads per block == bins per staged tile
constexpr int RPT = 8;                   // realizations per thread
constexpr int NT = 24;                   // CDF thresholds per small-lambda bin
constexpr double TINY = 0.02;            // geometric skipping below this expectation
constexpr double NORMAL_THRESH = 1e10;   // long(1e10) in cyutils.pyx:1223
constexpr double PTRS_MIN = 10.0;
constexpr double PTRS32_MAX = 4194304.0; // 2^22: k stays exact in FP32
constexpr int MAX_ATTEMPTS = 64;
constexpr int MAX_INVERSION = 4096;
// stream words (counter .w) of the different draw families
constexpr uint32_t W_PAIR = 0u;             // first draw / first PTRS attempt of a realization pair
constexpr uint32_t W_RETRY = 0x10000000u;   // | attempt: further PTRS attempts of one realization
constexpr uint32_t W_SKIP = 0x20000000u;    // | step: geometric skipping of a thread's realizations
constexpr uint32_t W_WIDE = 0x30000000u;    // | attempt: PTRS64 / Normal draws
constexpr uint32_t DOMAIN_GWB = 0x80000000u;
constexpr float HSCALE = 0x1.0p100f;     // keeps h2fdf (1e-30 .. 1e-20) far from FP32 subnormals
constexpr double HSCALE_INV = 0x1.0p-100;

enum BinKind : int {
    KIND_NONE = 0, KIND_TINY = 1, KIND_SMALL = 2, KIND_PTRS32 = 3, KIND_PTRS64 = 4, KIND_NORMAL = 5
};

// ---- Philox4x32-10
constexpr uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u, PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;

__device__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
    for (int i = 0; i < 10; i++) {
        uint32_t hi0 = __umulhi(PH_M0, c.x), lo0 = PH_M0 * c.x;
        uint32_t hi1 = __umulhi(PH_M1, c.z), lo1 = PH_M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += PH_W0;
        k.y += PH_W1;
    }
    return c;
}

__device__ __forceinline__ double u53(uint32_t hi, uint32_t lo) {   // [0, 1)
    return (double)(((uint64_t)hi << 21) ^ (uint64_t)(lo >> 11)) * 0x1.0p-53;
}
__device__ __forceinline__ float u24(uint32_t w) { return (float)(w >> 8) * 0x1.0p-24f; }   // [0, 1)
__device__ __forceinline__ unsigned long long w64(uint32_t hi, uint32_t lo) {
    return ((unsigned long long)hi << 32) | lo;
}

// log(k!) for k < 16, used by the PTRS acceptance test in the far lower tail
__constant__ double c_lgam[16] = {
    0.0, 0.0, 0.69314718055994531, 1.791759469228055, 3.1780538303479458, 4.7874917427820458,
    6.5792512120101012, 8.5251613610654147, 10.604602902745251, 12.801827480081469, 15.104412573075516,
    17.502307845873887, 19.987214495661885, 22.552163853123425, 25.19122118273868, 27.89927138384089};
// 1/n for the CDF recursion p(n) = p(n-1) lambda / n
__constant__ double c_inv[NT] = {
    0.0, 1.0, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 1.0 / 7, 1.0 / 8, 1.0 / 9, 1.0 / 10, 1.0 / 11,
    1.0 / 12, 1.0 / 13, 1.0 / 14, 1.0 / 15, 1.0 / 16, 1.0 / 17, 1.0 / 18, 1.0 / 19, 1.0 / 20, 1.0 / 21, 1.0 / 22,
    1.0 / 23};

// Per-bin sampler constants of one staged tile, shared by every realization of the block.
struct Tile {
    unsigned long long t0[RB];        // floor(e^-lambda 2^64): u < t0 <=> n = 0
    unsigned long long tskip[RB];     // tiny lambda: floor(e^(-RPT lambda) 2^64): no hit in RPT draws
    unsigned int thr[NT][RB];         // small lambda: floor(CDF(n) 2^32), n >= 1 (row 0 unused)
    double lam[RB];
    double h[RB];                     // exact h2fdf (for the loudest slots)
    float hs[RB];                     // h2fdf * 2^100 (for the background sums)
    float b[RB], a[RB], vr[RB], log_inva[RB], frac43[RB], lamf[RB];
    int lam_int[RB];
    int kind[RB];
};

__device__ __forceinline__ unsigned long long sat64(double p) {
    return (p >= 1.0) ? 0xFFFFFFFFFFFFFFFFull : (unsigned long long)(p * 0x1.0p64);
}

__device__ void bin_setup(Tile &s, int j, double lam, double h) {
    s.lam[j] = lam;
    s.h[j] = h;
    s.hs[j] = (float)(h * (double)HSCALE);
    int kind;
    if (!(lam > 0.0)) kind = KIND_NONE;
    else if (lam > NORMAL_THRESH) kind = KIND_NORMAL;
    else if (lam < TINY) kind = KIND_TINY;
    else if (lam < PTRS_MIN) kind = KIND_SMALL;
    else if (lam < PTRS32_MAX) kind = KIND_PTRS32;
    else kind = KIND_PTRS64;
    s.kind[j] = kind;
    if (kind == KIND_TINY) {
        s.t0[j] = sat64(exp(-lam));
        s.tskip[j] = sat64(exp(-(double)RPT * lam));
    } else if (kind == KIND_SMALL) {
        double p = exp(-lam);
        double cdf = p;
        s.t0[j] = sat64(cdf);
        int n = 1;
        for (; n < NT && cdf < 1.0; n++) {
            p = p * lam * c_inv[n];
            cdf += p;
            s.thr[n][j] = (unsigned int)(sat64(cdf) >> 32);
        }
        for (; n < NT; n++) s.thr[n][j] = 0xFFFFFFFFu;
    } else if (kind == KIND_PTRS32) {
        double slam = sqrt(lam);
        double b = 0.931 + 2.53 * slam;
        double a = -0.059 + 0.02483 * b;
        double inva = 1.1239 + 1.1328 / (b - 3.4);
        double vr = 0.9277 - 3.6224 / (b - 2.0);
        double li = floor(lam);
        s.b[j] = (float)b;
        s.a[j] = (float)a;
        s.vr[j] = (float)vr;
        s.log_inva[j] = (float)log(inva);
        s.lam_int[j] = (int)li;
        s.frac43[j] = (float)((lam - li) + 0.43);
        s.lamf[j] = (float)lam;
    }
}

// log P(k; lambda) for k >= 16 in FP32: -bd0(k, lambda) - log(2 pi k)/2 - stirlerr(k)
// (Loader 2000, "Fast and accurate computation of binomial probabilities").
__device__ __forceinline__ float log_pmf32(int k, float d, float lamf) {
    float kf = (float)k;
    float bd0;
    float sum = kf + lamf;
    if (fabsf(d) < 0.1f * sum) {
        float v = d / sum;
        float s = d * v;
        float ej = 2.0f * kf * v;
        float v2 = v * v;
#pragma unroll 1
        for (int j = 1; j < 24; j++) {
            ej *= v2;
            float s1 = s + ej / (float)(2 * j + 1);
            if (s1 == s) break;
            s = s1;
        }
        bd0 = s;
    } else {
        bd0 = kf * logf(kf / lamf) + lamf - kf;
    }
    float ik2 = 1.0f / (kf * kf);
    float stirl = (0.083333333333f - (0.0027777777778f - 0.00079365079365f * ik2) * ik2) / kf;
    return -bd0 - 0.5f * logf(6.283185307179586f * kf) - stirl;
}

// One PTRS attempt from the uniforms (U word, V word); returns k >= 0 on acceptance, -1 otherwise.
__device__ __forceinline__ int ptrs32_attempt(const Tile &s, int j, uint32_t wu, uint32_t wv) {
    const float b = s.b[j], a = s.a[j], frac43 = s.frac43[j];
    float U = u24(wu) - 0.5f;
    float V = u24(wv);
    float us = 0.5f - fabsf(U);
    if (us < 0.013f && V > us) return -1;
    float kf = floorf((2.0f * a * __frcp_rn(us) + b) * U + frac43);
    if (!(kf > -1.0e7f && kf < 1.0e7f)) return -1;
    int k = s.lam_int[j] + (int)kf;
    if (k < 0) return -1;
    if (us >= 0.07f && V <= s.vr[j]) return k;
    float lhs = logf(V) + s.log_inva[j] - logf(a / (us * us) + b);
    float rhs;
    if (k < 16) {
        double lam = s.lam[j];
        rhs = (float)(-lam + (double)k * log(lam) - c_lgam[k]);
    } else {
        float d = (float)(k - s.lam_int[j]) - (frac43 - 0.43f);
        rhs = log_pmf32(k, d, s.lamf[j]);
    }
    return (lhs <= rhs) ? k : -1;
}

// Further PTRS attempts of realization r after a rejected first attempt.
__device__ int ptrs32_retry(const Tile &s, int j, uint32_t kb, uint32_t r, uint32_t f, uint32_t dom, uint2 key,
                            int *d_status) {
    for (int att = 1; att < MAX_ATTEMPTS; att++) {
        uint4 w = philox(make_uint4(kb, r, f, dom | W_RETRY | (uint32_t)att), key);
        int k = ptrs32_attempt(s, j, w.x, w.y);
        if (k >= 0) return k;
        k = ptrs32_attempt(s, j, w.z, w.w);
        if (k >= 0) return k;
    }
    hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
    return (int)floor(s.lam[j] + 0.5);
}

// PTRS in FP64 for 2^22 <= lambda <= 1e10
__device__ double ptrs64(uint4 ctr, uint2 key, double lam, int *d_status) {
    double slam = sqrt(lam), loglam = log(lam);
    double b = 0.931 + 2.53 * slam;
    double a = -0.059 + 0.02483 * b;
    double inva = 1.1239 + 1.1328 / (b - 3.4);
    double vr = 0.9277 - 3.6224 / (b - 2.0);
    for (int att = 0; att < MAX_ATTEMPTS; att++) {
        ctr.w = (ctr.w & 0xF0000000u) | (uint32_t)att;
        uint4 w = philox(ctr, key);
        double U = u53(w.x, w.y) - 0.5;
        double V = u53(w.z, w.w);
        double us = 0.5 - fabs(U);
        double k = floor((2.0 * a / us + b) * U + lam + 0.43);
        if (us >= 0.07 && V <= vr) return k;
        if (k < 0.0 || (us < 0.013 && V > us)) continue;
        if (log(V) + log(inva) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0)) return k;
    }
    hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
    return floor(lam + 0.5);
}

// Count of a small-lambda bin from a 64-bit uniform (u >= t0 already known to mean n >= 1).
__device__ __forceinline__ int small_count(const Tile &s, int j, unsigned long long u, int *d_status) {
    int n = 1;
    const uint32_t hi = (uint32_t)(u >> 32);
    while (n < NT && hi >= s.thr[n][j]) n++;
    if (n < NT) return n;
    // beyond the table: continue the CDF in FP64
    double lam = s.lam[j];
    double uu = (double)(u >> 11) * 0x1.0p-53;
    double p = exp(-lam);
    double cdf = p;
    int m = 0;
    while (uu >= cdf && m < MAX_INVERSION) {
        m++;
        p *= lam / m;
        cdf += p;
    }
    if (m >= MAX_INVERSION) hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
    return m < NT ? NT : m;
}

// Zero-truncated Poisson count for a tiny-lambda hit, by inversion in FP64 from a 53-bit uniform.
__device__ int truncated_count(double lam, double v, int *d_status) {
    double e = exp(-lam);
    double p = lam * e / (1.0 - e);   // P(n = 1 | n >= 1)
    double cdf = p;
    int n = 1;
    while (v >= cdf && n < MAX_INVERSION) {
        n++;
        p *= lam / n;
        cdf += p;
    }
    if (n >= MAX_INVERSION) hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
    return n;
}

// Real-valued draw for the PTRS64 / Normal kinds.
__device__ double draw_wide(const Tile &s, int j, int kind, uint4 ctr, uint2 key, int *d_status) {
    double lam = s.lam[j];
    if (kind == KIND_PTRS64) return ptrs64(ctr, key, lam, d_status);
    // Normal branch (cyutils.pyx:1328-1330)
    uint4 w = philox(ctr, key);
    double u1 = 1.0 - u53(w.x, w.y);   // (0, 1]
    double u2 = u53(w.z, w.w);
    double z = sqrt(-2.0 * log(u1)) * cos(2.0 * HGB_PI * u2);
    return lam + sqrt(lam) * z;
}

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x) {
    float y = x - comp;
    float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

// ---- gather into loudest-first (F, B) order
__global__ void k_gather_sorted(const double *__restrict__ number, const double *__restrict__ h2fdf,
                                const int32_t *__restrict__ order, long nb, int nf, double *__restrict__ lam_s,
                                double *__restrict__ h_s) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nb * nf) return;
    int f = (int)(idx % nf);
    long k = idx / nf;
    long src = (long)order[k] * nf + f;
    lam_s[(long)f * nb + k] = number[src];
    h_s[(long)f * nb + k] = h2fdf[src];
}

struct LoudArgs {
    long nb;          // bins
    int nf, nr, nl;   // frequencies, realizations, loudest slots
    int nchunk;       // chunk c holds tiles c, c + nchunk, c + 2 nchunk, ...
    uint2 key;
};

// Per-realization state of a block, indexed [slot][thread].
struct RealState {
    float acc[RPT][RB];
    float comp[RPT][RB];
    int nfill[RPT][RB];
};

// Output rows of one chunk: loudest values (and their sorted positions when chunks are merged),
// the number of filled slots and the background sum.
struct LoudOut {
    double *ss;     // [(c * nf + f) * nr + r][nl]
    int *pos;       // same shape, or NULL when there is one chunk
    double *bg;     // [(c * nf + f) * nr + r]
    int *cnt;       // same, or NULL
};

template <bool LOUD>
__device__ __forceinline__ void take(RealState &st, int i, int n, double h, float hs, int nl, int kpos, double *ss,
                                     int *pos) {
    const int t = threadIdx.x;
    if (LOUD) {
        int nfill = st.nfill[i][t];
        while (nfill < nl && n > 0) {
            ss[nfill] = h;
            if (pos) pos[nfill] = kpos;
            n--;
            nfill++;
        }
        st.nfill[i][t] = nfill;
    }
    if (n > 0) {
        float acc = st.acc[i][t], comp = st.comp[i][t];
        kahan_add(acc, comp, (float)n * hs);
        st.acc[i][t] = acc;
        st.comp[i][t] = comp;
    }
}

// Real-valued counts (PTRS64 / Normal) follow cyutils.pyx:1333-1342 literally.
template <bool LOUD>
__device__ __forceinline__ void take_real(RealState &st, int i, double num, double h, float hs, int nl, int kpos,
                                          double *ss, int *pos) {
    const int t = threadIdx.x;
    if (LOUD) {
        if (num < 1.0) return;
        int nfill = st.nfill[i][t];
        while (nfill < nl && num > 0.0) {
            ss[nfill] = h;
            if (pos) pos[nfill] = kpos;
            num -= 1.0;
            nfill++;
        }
        st.nfill[i][t] = nfill;
    }
    if (num != 0.0) {
        float acc = st.acc[i][t], comp = st.comp[i][t];
        kahan_add(acc, comp, (float)(num * (double)hs));
        st.acc[i][t] = acc;
        st.comp[i][t] = comp;
    }
}

// The realization kernel.  LOUD: loudest split over sorted bins (lam / h are the gathered (F, B)
// arrays); otherwise the second-pass GWB over bins in grid order (lam / h are the (B, F) grids).
// grid (chunk, frequency, realization group), RB threads.
template <bool LOUD>
__global__ void __launch_bounds__(RB, 6) k_realize(LoudArgs a, const double *__restrict__ lam_in,
                                                const double *__restrict__ h_in, LoudOut out, int *d_status) {
    __shared__ Tile s;
    __shared__ RealState st;
    const int c = blockIdx.x, f = blockIdx.y, t = threadIdx.x;
    const int r0 = blockIdx.z * RB * RPT + t;
    const uint32_t dom = LOUD ? 0u : DOMAIN_GWB;
    int rpt = 0;   // realizations of this thread: r0 + i * RB, i < rpt
    while (rpt < RPT && r0 + rpt * RB < a.nr) rpt++;
    const long row0 = ((long)c * a.nf + f) * a.nr + r0;   // output row of slot 0; slot i adds i * RB
    for (int i = 0; i < RPT; i++) {
        st.acc[i][t] = 0.0f;
        st.comp[i][t] = 0.0f;
        st.nfill[i][t] = 0;
    }
    const long ntiles = (a.nb + RB - 1) / RB;
    for (long tile = c; tile < ntiles; tile += a.nchunk) {
        const long base = tile * RB;
        const int nt = (int)((a.nb - base) < RB ? (a.nb - base) : RB);
        __syncthreads();
        if (t < nt) {
            const long b = base + t;
            if (LOUD) bin_setup(s, t, lam_in[(long)f * a.nb + b], h_in[(long)f * a.nb + b]);
            else bin_setup(s, t, lam_in[b * a.nf + f], h_in[b * a.nf + f]);
        }
        __syncthreads();
        if (rpt == 0) continue;
        for (int j = 0; j < nt; j++) {
            const int kind = s.kind[j];
            if (kind == KIND_NONE) continue;
            const uint32_t kb = (uint32_t)(base + j);
            const int kpos = (int)(base + j);
            const double h = s.h[j];
            const float hs = s.hs[j];
            if (kind == KIND_TINY) {
                // geometric skipping over the thread's realizations
                uint4 w = philox(make_uint4(kb, (uint32_t)r0, (uint32_t)f, dom | W_SKIP), a.key);
                unsigned long long u = w64(w.x, w.y);
                if (rpt == RPT && u < s.tskip[j]) continue;
                const double lam = s.lam[j];
                int i = 0;
                for (int step = 0; step < 2 * RPT + 2; step++) {
                    if (step > 0) {
                        w = philox(make_uint4(kb, (uint32_t)r0, (uint32_t)f, dom | W_SKIP | (uint32_t)step), a.key);
                        u = w64(w.x, w.y);
                    }
                    double uu = ((double)(u >> 11) + 1.0) * 0x1.0p-53;   // (0, 1]
                    double gap = floor(-log(uu) / lam);
                    if (gap >= (double)(rpt - i)) break;
                    i += (int)gap;
                    int n = truncated_count(lam, u53(w.z, w.w), d_status);
                    take<LOUD>(st, i, n, h, hs, a.nl, kpos, out.ss + (row0 + (long)i * RB) * a.nl,
                               out.pos ? out.pos + (row0 + (long)i * RB) * a.nl : nullptr);
                    i++;
                    if (i >= rpt) break;
                }
            } else if (kind == KIND_SMALL) {
                const unsigned long long t0 = s.t0[j];
#pragma unroll 1
                for (int i = 0; i < rpt; i += 2) {
                    uint4 w = philox(make_uint4(kb, (uint32_t)(r0 + i * RB), (uint32_t)f, dom | W_PAIR), a.key);
                    unsigned long long u = w64(w.x, w.y);
                    if (u >= t0) {
                        int n = small_count(s, j, u, d_status);
                        take<LOUD>(st, i, n, h, hs, a.nl, kpos, out.ss + (row0 + (long)i * RB) * a.nl,
                                   out.pos ? out.pos + (row0 + (long)i * RB) * a.nl : nullptr);
                    }
                    u = w64(w.z, w.w);
                    if (i + 1 < rpt && u >= t0) {
                        int n = small_count(s, j, u, d_status);
                        take<LOUD>(st, i + 1, n, h, hs, a.nl, kpos, out.ss + (row0 + (long)(i + 1) * RB) * a.nl,
                                   out.pos ? out.pos + (row0 + (long)(i + 1) * RB) * a.nl : nullptr);
                    }
                }
            } else if (kind == KIND_PTRS32) {
#pragma unroll 1
                for (int i = 0; i < rpt; i += 2) {
                    const uint32_t ra = (uint32_t)(r0 + i * RB);
                    uint4 w = philox(make_uint4(kb, ra, (uint32_t)f, dom | W_PAIR), a.key);
                    int n = ptrs32_attempt(s, j, w.x, w.y);
                    if (n < 0) n = ptrs32_retry(s, j, kb, ra, (uint32_t)f, dom, a.key, d_status);
                    take<LOUD>(st, i, n, h, hs, a.nl, kpos, out.ss + (row0 + (long)i * RB) * a.nl,
                               out.pos ? out.pos + (row0 + (long)i * RB) * a.nl : nullptr);
                    if (i + 1 < rpt) {
                        n = ptrs32_attempt(s, j, w.z, w.w);
                        if (n < 0) n = ptrs32_retry(s, j, kb, ra + RB, (uint32_t)f, dom, a.key, d_status);
                        take<LOUD>(st, i + 1, n, h, hs, a.nl, kpos, out.ss + (row0 + (long)(i + 1) * RB) * a.nl,
                                   out.pos ? out.pos + (row0 + (long)(i + 1) * RB) * a.nl : nullptr);
                    }
                }
            } else {
#pragma unroll 1
                for (int i = 0; i < rpt; i++) {
                    const uint32_t r = (uint32_t)(r0 + i * RB);
                    double num = draw_wide(s, j, kind, make_uint4(kb, r, (uint32_t)f, dom | W_WIDE), a.key, d_status);
                    take_real<LOUD>(st, i, num, h, hs, a.nl, kpos, out.ss + (row0 + (long)i * RB) * a.nl,
                                    out.pos ? out.pos + (row0 + (long)i * RB) * a.nl : nullptr);
                }
            }
        }
    }
    for (int i = 0; i < rpt; i++) {
        const long row = row0 + (long)i * RB;
        if (LOUD) {
            const int nfill = st.nfill[i][t];
            double *ss = out.ss + row * a.nl;
            for (int l = nfill; l < a.nl; l++) ss[l] = 0.0;
            if (out.cnt) out.cnt[row] = nfill;
        }
        out.bg[row] = ((double)st.acc[i][t] - (double)st.comp[i][t]) * HSCALE_INV;
    }
}

// Merge per-chunk partials: the global loudest slots are the smallest sorted positions among the
// chunks' own loudest lists (each list is in position order); every other listed source and every
// chunk background goes to the background.
__global__ void k_loudest_merge(LoudArgs a, LoudOut part, double *__restrict__ hc2ss, double *__restrict__ hc2bg) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)a.nf * a.nr) return;
    const long stride = (long)a.nf * a.nr;
    double *out = hc2ss + idx * a.nl;
    // heads[c]: next unread entry of chunk c's list (chunks <= 255, lists <= nl <= 255)
    unsigned char heads[256];
    for (int c = 0; c < a.nchunk; c++) heads[c] = 0;
    for (int l = 0; l < a.nl; l++) {
        int best = -1, bpos = 0x7FFFFFFF;
        for (int c = 0; c < a.nchunk; c++) {
            long row = (long)c * stride + idx;
            if (heads[c] < part.cnt[row]) {
                int p = part.pos[row * a.nl + heads[c]];
                if (p < bpos) {
                    bpos = p;
                    best = c;
                }
            }
        }
        if (best < 0) {
            out[l] = 0.0;
            continue;
        }
        long row = (long)best * stride + idx;
        out[l] = part.ss[row * a.nl + heads[best]];
        heads[best]++;
    }
    double bg = 0.0;
    for (int c = 0; c < a.nchunk; c++) {
        long row = (long)c * stride + idx;
        for (int e = heads[c]; e < part.cnt[row]; e++) bg += part.ss[row * a.nl + e];
        bg += part.bg[row];
    }
    hc2bg[idx] = bg;
}

// Replay: thread per (frequency, realization), sequential over the sorted bins (cyutils.pyx:1312-1344).
__global__ void k_loudest_replay(long nb, int nf, int nr, int nl, const double *__restrict__ h_s,
                                 const double *__restrict__ replay, double *__restrict__ hc2ss,
                                 double *__restrict__ hc2bg) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)nf * nr) return;
    int f = (int)(idx / nr), r = (int)(idx % nr);
    const double *hf = h_s + (long)f * nb;
    const double *cnt = replay + ((long)r * nf + f) * nb;
    double *ss = hc2ss + idx * nl;
    for (int l = 0; l < nl; l++) ss[l] = 0.0;
    int ll = 0;
    double sum = 0.0;
    for (long k = 0; k < nb; k++) {
        double num = cnt[k];
        if (num < 1.0) continue;
        double cur = hf[k];
        while (ll < nl && num > 0.0) {
            ss[ll] = cur;
            num = __dsub_rn(num, 1.0);
            ll++;
        }
        sum = __dadd_rn(sum, __dmul_rn(num, cur));
    }
    hc2bg[idx] = sum;
}

__global__ void k_gwb_reduce(int nchunk, long nfr, const double *__restrict__ part, double *__restrict__ gwb) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nfr) return;
    double acc = 0.0;
    for (int c = 0; c < nchunk; c++) acc += part[(long)c * nfr + idx];
    gwb[idx] = acc;
}

__global__ void k_gwb_replay(long nb, int nf, int nr, const double *__restrict__ hc2, const double *__restrict__ replay,
                             double *__restrict__ gwb) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)nf * nr) return;
    int f = (int)(idx / nr), r = (int)(idx % nr);
    double acc = 0.0;
    for (long b = 0; b < nb; b++) {
        double num = replay[(b * nf + f) * (long)nr + r];
        acc = __dadd_rn(acc, __dmul_rn(num, hc2[b * nf + f]));
    }
    gwb[idx] = acc;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int n_rgroups(int nr) { return (int)hgb::ceil_div(nr, (long)RB * RPT); }

int choose_nchunk(long nb, int nf, int nr) {
    long blocks = (long)n_rgroups(nr) * nf;
    long target = 152L * 7 * 2;   // two waves of resident blocks on 152 SMs
    long nchunk = hgb::ceil_div(target, blocks);
    long maxc = hgb::ceil_div(nb, 8L * RB);
    if (nchunk > maxc) nchunk = maxc;
    if (nchunk < 1) nchunk = 1;
    if (nchunk > 255) nchunk = 255;
    return (int)nchunk;
}

struct LoudLayout {
    size_t off_lam, off_h, off_ss, off_pos, off_bg, off_cnt, total;
    int nchunk;
};

LoudLayout loud_layout(long nb, int nf, int nr, int nl, int mode) {
    LoudLayout L{};
    L.nchunk = (mode == HGB_RNG_PHILOX) ? choose_nchunk(nb, nf, nr) : 1;
    size_t o = 0;
    L.off_lam = o;
    o += align256(sizeof(double) * nb * nf);
    L.off_h = o;
    o += align256(sizeof(double) * nb * nf);
    if (L.nchunk > 1) {
        long n = (long)L.nchunk * nf * nr;
        long m = n * (nl > 0 ? nl : 1);
        L.off_ss = o;
        o += align256(sizeof(double) * m);
        L.off_pos = o;
        o += align256(sizeof(int) * m);
        L.off_bg = o;
        o += align256(sizeof(double) * n);
        L.off_cnt = o;
        o += align256(sizeof(int) * n);
    }
    L.total = o;
    return L;
}

LoudArgs make_args(long nb, int nf, int nr, int nl, int nchunk, uint64_t seed) {
    LoudArgs a;
    a.nb = nb;
    a.nf = nf;
    a.nr = nr;
    a.nl = nl;
    a.nchunk = nchunk;
    a.key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    return a;
}

}  // namespace

extern "C" {

size_t hgb_loudest_workspace_bytes(long n_bins, int n_freq, int nreals, int nloud, int mode) {
    if (n_bins <= 0 || n_freq <= 0 || nreals <= 0) return 0;
    return loud_layout(n_bins, n_freq, nreals, nloud, mode).total;
}

int hgb_loudest_hc_from_sorted(const double *number, const double *h2fdf, long n_bins, int n_freq, int nreals,
                               int nloud, const int32_t *order, int mode, uint64_t seed, const double *replay,
                               double *hc2ss, double *hc2bg, void *workspace, size_t workspace_bytes,
                               int *d_status, void *stream) {
    HGB_CHECK_ARG(number && h2fdf && order && hc2bg && n_bins >= 0 && n_freq >= 1 && nreals >= 0 && nloud >= 0);
    HGB_CHECK_ARG(nloud == 0 || hc2ss);
    HGB_CHECK_ARG(nloud <= 255);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || mode == HGB_RNG_REPLAY);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || replay);
    HGB_CHECK_ARG(n_bins < (1L << 31) && n_freq <= 65535 && nreals < (1 << 30));
    if (nreals == 0) return HGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (n_bins == 0) {
        if (nloud) cudaMemsetAsync(hc2ss, 0, sizeof(double) * (size_t)n_freq * nreals * nloud, st);
        cudaMemsetAsync(hc2bg, 0, sizeof(double) * (size_t)n_freq * nreals, st);
        return hgb::check_launch();
    }
    LoudLayout L = loud_layout(n_bins, n_freq, nreals, nloud, mode);
    if (!workspace || workspace_bytes < L.total) return HGB_ERR_WORKSPACE;
    char *w = (char *)workspace;
    double *lam_s = (double *)(w + L.off_lam);
    double *h_s = (double *)(w + L.off_h);
    long n = n_bins * n_freq;
    k_gather_sorted<<<(unsigned)hgb::ceil_div(n, 256), 256, 0, st>>>(number, h2fdf, order, n_bins, n_freq, lam_s, h_s);
    int rc = hgb::check_launch();
    if (rc) return rc;
    if (mode == HGB_RNG_REPLAY) {
        long nt = (long)n_freq * nreals;
        k_loudest_replay<<<(unsigned)hgb::ceil_div(nt, 128), 128, 0, st>>>(n_bins, n_freq, nreals, nloud, h_s, replay,
                                                                             hc2ss, hc2bg);
        return hgb::check_launch();
    }
    LoudArgs a = make_args(n_bins, n_freq, nreals, nloud, L.nchunk, seed);
    dim3 grid((unsigned)a.nchunk, (unsigned)n_freq, (unsigned)n_rgroups(nreals));
    if (a.nchunk == 1) {
        LoudOut o{hc2ss, nullptr, hc2bg, nullptr};
        k_realize<true><<<grid, RB, 0, st>>>(a, lam_s, h_s, o, d_status);
        return hgb::check_launch();
    }
    LoudOut part{(double *)(w + L.off_ss), (int *)(w + L.off_pos), (double *)(w + L.off_bg), (int *)(w + L.off_cnt)};
    k_realize<true><<<grid, RB, 0, st>>>(a, lam_s, h_s, part, d_status);
    rc = hgb::check_launch();
    if (rc) return rc;
    long nt = (long)n_freq * nreals;
    k_loudest_merge<<<(unsigned)hgb::ceil_div(nt, 128), 128, 0, st>>>(a, part, hc2ss, hc2bg);
    return hgb::check_launch();
}

size_t hgb_sam_poisson_gwb_workspace_bytes(long n_bins, int n_freq, int nreals) {
    if (n_bins <= 0 || n_freq <= 0 || nreals <= 0) return 0;
    long nchunk = choose_nchunk(n_bins, n_freq, nreals);
    return align256(sizeof(double) * (size_t)nchunk * n_freq * nreals);
}

int hgb_sam_poisson_gwb(const double *number, const double *hc2, long n_bins, int n_freq, int nreals, int mode,
                        uint64_t seed, const double *replay, double *gwb, void *workspace, size_t workspace_bytes,
                        int *d_status, void *stream) {
    HGB_CHECK_ARG(number && hc2 && gwb && n_bins >= 0 && n_freq >= 1 && nreals >= 0);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || mode == HGB_RNG_REPLAY);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || replay);
    HGB_CHECK_ARG(n_bins < (1L << 31) && n_freq <= 65535 && nreals < (1 << 30));
    if (nreals == 0) return HGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (n_bins == 0) {
        cudaMemsetAsync(gwb, 0, sizeof(double) * (size_t)n_freq * nreals, st);
        return hgb::check_launch();
    }
    if (mode == HGB_RNG_REPLAY) {
        long nt = (long)n_freq * nreals;
        k_gwb_replay<<<(unsigned)hgb::ceil_div(nt, 128), 128, 0, st>>>(n_bins, n_freq, nreals, hc2, replay, gwb);
        return hgb::check_launch();
    }
    if (!workspace || workspace_bytes < hgb_sam_poisson_gwb_workspace_bytes(n_bins, n_freq, nreals))
        return HGB_ERR_WORKSPACE;
    LoudArgs a = make_args(n_bins, n_freq, nreals, 0, choose_nchunk(n_bins, n_freq, nreals), seed);
    dim3 grid((unsigned)a.nchunk, (unsigned)n_freq, (unsigned)n_rgroups(nreals));
    LoudOut o{nullptr, nullptr, (double *)workspace, nullptr};
    k_realize<false><<<grid, RB, 0, st>>>(a, number, hc2, o, d_status);
    int rc = hgb::check_launch();
    if (rc) return rc;
    long nfr = (long)n_freq * nreals;
    k_gwb_reduce<<<(unsigned)hgb::ceil_div(nfr, 256), 256, 0, st>>>(a.nchunk, nfr, (double *)workspace, gwb);
    return hgb::check_launch();
}

}  // extern "C"
