// Poisson realizations of the binary population with the loudest-source split.
//
// Replaces cyutils.loudest_hc_from_sorted (holodeck/cyutils.pyx:1220-1344) and
// cyutils.sam_poisson_gwb (holodeck/cyutils.pyx:854-897).
//
// The reference visits, for every realization r and frequency f, all bins in loudest-first order,
// draws n ~ Poisson(number), hands the first L sources to the loudest slots and adds the rest,
// n * h2fdf, to the background.  Only the first L sources depend on the visiting order; the
// background is an order-free sum.  The GPU path splits the walk accordingly:
//
//   1. k_gather_sorted   number / h2fdf gathered into loudest-first (F, B) order.
//   2. k_cum_sum/write   per frequency, the cumulative expectation C[k] = sum_{k' < k} number[k']
//                        along that order (FP64), in segments.
//   3. k_loud_prefix     one thread per (f, r) fills the L slots exactly in order, jumping from one
//                        occupied bin to the next: with i the first unvisited bin and E ~ Exp(1),
//                        the next bin with n >= 1 is the smallest j >= i with C[j+1] - C[i] > E
//                        (P(no source in bins i..j-1) = exp(-(C[j] - C[i]))), and its count is
//                        zero-truncated Poisson.  So the loudest slots cost ~L events instead of a
//                        walk over the tens of thousands of bins that precede them.  The bin that
//                        fills the last slot adds its remaining sources to the background, and
//                        Q[f, r], the first bin not yet visited, is recorded.
//   4. k_bulk            the background of every bin at sorted position >= Q[f, r]: a block owns
//                        one frequency, RB * RPT realizations and one chunk of bins (every
//                        nchunk-th tile of RB bins, so chunks carry the same mix and finish
//                        together), stages a tile's per-bin sampler constants in shared memory --
//                        computed once per bin, amortised over all realizations -- sorts the tile's
//                        bins into one list per sampler kind, and runs each list as a tight loop in
//                        which every lane draws for its own realizations.
//   5. k_bg_reduce       per (f, r): prefix remainder + the chunks' partial sums, in fixed order.
// sam_poisson_gwb is step 4 with Q = 0 over the bins in grid order, then step 5.
//
// Draws (HGB_RNG_PHILOX): counter-based Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) keyed by
// the 64-bit seed; counters are built from (sorted bin or event index, realization, frequency,
// draw family), so results do not depend on the chunking.  Bulk samplers by expectation lambda:
//   lambda <= 0 or NaN        n = 0, no draw
//   lambda < SPARSE_MAX       geometric skipping over realizations: the gap to the next realization
//                             with n >= 1 is floor(-ln u / lambda), and a hit draws n from the
//                             zero-truncated Poisson.  The block's realizations are cut into runs of
//                             2^lg (about one expected event each) and one thread walks a run, so a
//                             bin costs about one draw per event instead of one per lane
//   SPARSE_MAX <= lambda < 10 a 32-column alias row per bin (n < 31 and the rest at 31): one
//                             lookup and one comparison per draw; four realizations per Philox call
//   10 <= lambda <= 65536     inversion against a per-bin table over lambda +- 7 sqrt(lambda) in
//                             shared memory, with a guide table whose "pure" cells answer most draws
//                             with one lookup; four realizations per Philox call
//   65536 < lambda < 2^22     PTRS, transformed rejection with squeeze (Hormann 1993, Insurance:
//                             Mathematics and Economics 12, 39-45) in FP32: the acceptance test uses
//                             the log-pmf in Loader's saddle-point form (bd0 + Stirling remainder,
//                             Loader 2000), so nothing cancels in FP32.  Each lane runs one loop
//                             over its realizations that consumes two attempts per Philox call and
//                             moves to the next realization on acceptance, so a rejection delays
//                             only its own lane by one attempt
//   2^22 <= lambda <= 1e10    PTRS in FP64 (k_bulk_wide, after k_bulk)
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

#include <type_traits>

#include <atomic>

#include <algorithm>
#include <vector>

#include "hgb_common.cuh"

namespace {

constexpr int RB = 128;                  // threads per block == bins per staged tile
constexpr int NWARP = RB / 32;
constexpr int RPT = 8;                   // realizations per thread
static_assert(RPT == 8, "the table passes draw four realizations per Philox call, two calls per bin");
constexpr int NT = 32;                   // CDF thresholds per small-lambda bin
constexpr double SPARSE_MAX = 0.1;       // geometric skipping over realizations below this expectation
constexpr double NORMAL_THRESH = 1e10;   // long(1e10) in cyutils.pyx:1223
constexpr double PTRS_MIN = 10.0;
constexpr double PTRS32_MAX = 4194304.0; // 2^22: k stays exact in FP32
constexpr int MAX_ATTEMPTS = 64;
constexpr int MAX_PTRS_ITERS = 2 * RPT + 64;   // attempts of one lane over its RPT realizations
constexpr int MAX_INVERSION = 4096;
constexpr int MAX_PREFIX_EXTRA = 1024;   // prefix events beyond L (Normal draws below 1)
constexpr double TABLE_MAX = 47000.0;    // table inversion up to here: k_lo..k_hi spans <= 14 sqrt(lambda) + 10
constexpr int TMAX = 3072;               // table entries (>= 14 sqrt(TABLE_MAX) + 10 = 3046)
constexpr int HALF_WORDS = 2048 + 512;   // tables up to 2048 entries (2^10 u16 guide cells) fit a half
constexpr int ARENA_WORDS = 2 * HALF_WORDS;   // the halves alternate between build and draw
static_assert(TMAX + 2048 <= ARENA_WORDS, "the largest table (2^12 guide cells) fits the whole arena");
constexpr int BATCH_MAX = 32;            // table-kind bins built per batch
constexpr int BULK_BLOCKS_PER_SM = 6;    // k_bulk residency (seven was measured slower: 30.7 against 29.2 ms)
constexpr unsigned GUIDE_PURE = 0x8000u, GUIDE_ONE = 0x4000u, GUIDE_M = 0x0FFFu;   // guide cell fields
static_assert(TMAX - 1 <= (int)GUIDE_M, "table entries fit the guide's index field");
static_assert(ARENA_WORDS >= RB * (NT + 1), "the small-lambda rows share the arena");
constexpr int ANCHOR = 16;               // Loader-form pmf every ANCHOR-th entry, the recursion between
constexpr float TABLE_SIGMAS = 7.0f;     // the table covers lambda +- 7 sqrt(lambda) (tails < 1e-11)
// draw families (counter .w high bits)
constexpr uint32_t W_SMALL = 0x00000000u;   // | call: 4 realizations per call
constexpr uint32_t W_PTRS = 0x10000000u;    // | iteration / 2
constexpr uint32_t W_TABLE = 0x50000000u;   // | call: 4 realizations per call
constexpr uint32_t W_SKIP = 0x20000000u;    // | step: geometric skipping of a lane's realizations
constexpr uint32_t W_SPARSE = 0x60000000u;  // | event: geometric skipping along a run of realizations
constexpr uint32_t W_WIDE = 0x30000000u;    // | slot << 8 | attempt: PTRS64 / Normal draws
constexpr uint32_t W_PREFIX = 0x40000000u;  // | attempt: prefix events (counter .z = event index)
constexpr uint32_t DOMAIN_GWB = 0x80000000u;
constexpr float HSCALE = 0x1.0p100f;     // keeps h2fdf (1e-30 .. 1e-20) far from FP32 subnormals
constexpr double HSCALE_INV = 0x1.0p-100;

enum BinKind : int {
    KIND_NONE = 0, KIND_SPARSE = 1, KIND_SMALL = 2, KIND_TABLE = 3, KIND_PTRS32 = 4, KIND_WIDE = 5, NKIND = 6
};

// ---- Philox4x32-10 with the ten round keys precomputed (they live in the kernel's parameter space)
constexpr uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u, PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;

struct PhiloxKey {
    uint32_t k0[10], k1[10];
};

PhiloxKey make_key(uint64_t seed) {
    PhiloxKey K;
    uint32_t a = (uint32_t)seed, b = (uint32_t)(seed >> 32);
    for (int i = 0; i < 10; i++) {
        K.k0[i] = a;
        K.k1[i] = b;
        a += PH_W0;
        b += PH_W1;
    }
    return K;
}

__device__ __forceinline__ uint4 philox(uint4 c, const PhiloxKey &K) {
#pragma unroll
    for (int i = 0; i < 10; i++) {
        const uint64_t p0 = (uint64_t)PH_M0 * c.x;
        const uint64_t p1 = (uint64_t)PH_M1 * c.z;
        c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ K.k0[i], (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ K.k1[i],
                       (uint32_t)p0);
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
__constant__ float c_lgam[16] = {
    0.0f, 0.0f, 0.69314718055994531f, 1.791759469228055f, 3.1780538303479458f, 4.7874917427820458f,
    6.5792512120101012f, 8.5251613610654147f, 10.604602902745251f, 12.801827480081469f, 15.104412573075516f,
    17.502307845873887f, 19.987214495661885f, 22.552163853123425f, 25.19122118273868f, 27.89927138384089f};

// Stirling-series remainder stirlerr(n) = log(n!) - (n + 1/2) log n + n - log(2 pi)/2, n < 16
// (evaluated from the definition in float64); larger n use the asymptotic series.
__constant__ float c_stirl[16] = {
    0.000000000e+00f, 8.106146680e-02f, 4.134069596e-02f, 2.767792568e-02f, 2.079067210e-02f, 1.664469119e-02f,
    1.387612882e-02f, 1.189670995e-02f, 1.041126526e-02f, 9.255462183e-03f, 8.330563433e-03f, 7.573675488e-03f,
    6.942840107e-03f, 6.408994188e-03f, 5.951370113e-03f, 5.554733552e-03f};
// 1/n for the small-lambda CDF recursion p(n) = p(n-1) lambda / n
__constant__ float c_invf[NT] = {
    0.0f, 1.0f, 1.0f / 2, 1.0f / 3, 1.0f / 4, 1.0f / 5, 1.0f / 6, 1.0f / 7, 1.0f / 8, 1.0f / 9, 1.0f / 10,
    1.0f / 11, 1.0f / 12, 1.0f / 13, 1.0f / 14, 1.0f / 15, 1.0f / 16, 1.0f / 17, 1.0f / 18, 1.0f / 19, 1.0f / 20,
    1.0f / 21, 1.0f / 22, 1.0f / 23, 1.0f / 24, 1.0f / 25, 1.0f / 26, 1.0f / 27, 1.0f / 28, 1.0f / 29, 1.0f / 30,
    1.0f / 31};

// Per-bin sampler constants of one staged tile, shared by every realization of the block.  The
// small-lambda thresholds and the table of the current table-kind bin share one region: the
// small-lambda pass finishes before the first table is built.
struct Tile {
    union {
        // small lambda: one padded 32-column alias row per bin (threshold << 5 | alias); the lanes of
        // a warp read one bin's row at different columns, which the padding puts in different banks
        unsigned int thr[RB][NT + 1];
        unsigned int arena[ARENA_WORDS];          // table kind: packed cdf (u32) + guide (u16) tables
    } u;
    unsigned char sp_lg[RB];          // sparse: log2 of the realization run length of the bin
    int sp_start[RB];                 // sparse: first run of each sparse-list entry
    unsigned long long scan[NWARP];
    double lam[RB];
    float hs[RB];                     // h2fdf * 2^100 (for the background sums)
    float frac[RB], lamf[RB];
    int lam_int[RB];
    int tb_klo[RB], tb_S[RB], tb_gb[RB];   // table kind: first count, entries, log2 guide cells
    int pos[RB];                      // sorted position (loudest) or grid index (gwb) of the bin
    unsigned char list[NKIND][RB];    // tile-local bin indices per kind, in bin order
    int wcount[NWARP][NKIND];
    float lgam[16];
};

__device__ __forceinline__ int kind_count(const Tile &s, int k) {
    int n = 0;
#pragma unroll
    for (int w = 0; w < NWARP; w++) n += s.wcount[w][k];
    return n;
}

// Per-realization sums of a block for the passes whose realization slot is data dependent (table
// tail cells, PTRS, and with the parameter sums every per-lane pass), indexed [slot][thread]:
// plain FP32 where the terms are few (a few percent of the table draws and the PTRS bins), Kahan
// pairs for the parameter path.
struct SlotsPlain {
    float acc[RPT][RB];
};
struct SlotsKahan {
    float acc[RPT][RB];
    float comp[RPT][RB];
};

__device__ __forceinline__ int bin_kind(double lam) {
    if (!(lam > 0.0)) return KIND_NONE;
    if (lam < SPARSE_MAX) return KIND_SPARSE;
    if (lam < PTRS_MIN) return KIND_SMALL;
    if (lam <= TABLE_MAX) return KIND_TABLE;
    if (lam < PTRS32_MAX) return KIND_PTRS32;
    return KIND_WIDE;
}

__device__ void bin_setup(Tile &s, int j, int kind, double lam, double h) {
    s.lam[j] = lam;
    s.hs[j] = (float)(h * (double)HSCALE);
    if (kind == KIND_SPARSE) {
        // runs of 2^lg realizations, lambda 2^lg in [0.5, 1) unless clamped to [8, 1024]
        const float lf = (float)lam;
        s.lamf[j] = lf;
        s.sp_lg[j] = (unsigned char)(lf > 0.0f ? max(3, min(10, -ilogbf(lf) - 1)) : 10);
    } else if (kind == KIND_SMALL) {
        // q(n) = P(n) in FP32 by the recursion P(n) = P(n-1) lambda / n, rounded to 32.32 fixed point,
        // for n < 31; n = 31 carries the rest (P(n >= 31) < 2e-9 for lambda < 10; a rounding excess
        // comes off the mode instead), so sum q = 2^32.  Then a 32-column alias row (Walker 1977,
        // each column 2^27 of the 2^32 units) by the sweep over lights and heavies in index order:
        // word = threshold (27 bits) << 5 | alias (5 bits).
        unsigned *row = s.u.thr[j];
        const float lf = (float)lam;
        float p = expf(-lf);
        unsigned long long cum = 0;
        unsigned qmax = 0;
        int mode = 0;
        for (int n = 0; n < NT - 1; n++) {
            if (n > 0) p = p * lf * c_invf[n];
            const unsigned q = __float2uint_rn(p * 0x1.0p32f);
            row[n] = q;
            cum += q;
            if (q > qmax) {
                qmax = q;
                mode = n;
            }
        }
        if (cum <= 0x100000000ull) {
            row[NT - 1] = (unsigned)(0x100000000ull - cum);   // cum > 0: q(0) > 0
        } else {
            row[mode] -= (unsigned)(cum - 0x100000000ull);
            row[NT - 1] = 0u;
        }
        constexpr unsigned C = 1u << 27;
        unsigned heavy = 0;
        for (int n = 0; n < NT; n++)
            if (row[n] >= C) heavy |= 1u << n;
        int jh = __ffs(heavy) - 1;   // a heavy exists: the 32 entries sum to 32 C
        unsigned rest = heavy & (heavy - 1);
        unsigned r = row[jh];
        for (int n = 0; n < NT; n++) {
            if (heavy >> n & 1) continue;
            const unsigned qn = row[n];
            row[n] = (qn << 5) | (unsigned)jh;
            r -= C - qn;
            while (r < C && rest) {   // heavy jh is used up: its own column, aliased to the next
                const int jn = __ffs(rest) - 1;
                rest &= rest - 1;
                const unsigned qj = row[jn];
                row[jh] = (r << 5) | (unsigned)jn;
                r = qj - (C - r);
                jh = jn;
            }
        }
        row[jh] = ((C - 1) << 5) | (unsigned)jh;   // the last heavy keeps its whole column
    } else if (kind == KIND_TABLE || kind == KIND_PTRS32) {
        const float lf = (float)lam;
        const double li = floor(lam);
        s.lam_int[j] = (int)li;
        s.frac[j] = (float)(lam - li);
        s.lamf[j] = lf;
        if (kind == KIND_TABLE) {
            const float sd = sqrtf(lf);
            const int k_lo = max(0, (int)floorf(lf - TABLE_SIGMAS * sd - 2.0f));
            const int S = min((int)ceilf(lf + TABLE_SIGMAS * sd + 6.0f) - k_lo + 1, TMAX);
            s.tb_klo[j] = k_lo;
            s.tb_S[j] = S;
            s.tb_gb[j] = max(1, 31 - __clz(S - 1));   // ceil(log2 S) - 1: 2^gb >= S / 2 guide cells
        }
    }
}

// bd0(k, lambda) = k log(k / lambda) + lambda - k (Loader 2000) in FP32 from d = k - lambda, which
// the caller forms exactly as (k - floor(lambda)) - frac(lambda).  The quotients use __fdividef
// (2 ulp): bd0 then carries a relative error of a few 1e-7, which moves exp(-bd0) by at most about
// 5e-6 relative in the far tails (bd0 ~ 25, P ~ 1e-11) and about 1e-7 near the mode.
__device__ __forceinline__ float bd0_f32(float kk, float d, float lamf) {
    const float v = __fdividef(d, kk + lamf);
    if (fabsf(v) < 0.1f) {
        const float v2 = v * v;
        return d * v + 2.0f * kk * v * v2 * (0.33333333f + v2 * (0.2f + v2 * (0.14285714f + v2 * 0.11111111f)));
    }
    return kk * log1pf(__fdividef(d, lamf)) - d;
}

__device__ __forceinline__ float stirlerr_f32(int k) {
    if (k < 16) return c_stirl[k];
    const float kk = (float)k;
    const float ik2 = __fdividef(1.0f, kk * kk);
    return __fdividef(0.083333333333f - (0.0027777777778f - 0.00079365079365f * ik2) * ik2, kk);
}

// P(k; lambda) in FP32, relative error ~1e-7 across the table range:
// exp(-bd0 - stirlerr(k)) / sqrt(2 pi k), and exp(-lambda) at k = 0.
__device__ __forceinline__ float pmf_f32(int k, int lam_int, float frac, float lamf) {
    if (k == 0) return expf(-lamf);
    const float kk = (float)k;
    const float d = (float)(k - lam_int) - frac;
    return expf(-bd0_f32(kk, d, lamf) - stirlerr_f32(k)) * rsqrtf(6.283185307179586f * kk);
}

// PTRS constants of one bin (Hormann 1993), formed in registers by every thread that draws it
struct Ptrs32C {
    float b, a, vr, log_inva, loglam, frac, lamf;
    int lam_int;
};

__device__ __forceinline__ Ptrs32C ptrs32_consts(const Tile &s, int j) {
    Ptrs32C p;
    p.lamf = s.lamf[j];
    p.frac = s.frac[j];
    p.lam_int = s.lam_int[j];
    const float slam = sqrtf(p.lamf);
    p.b = 0.931f + 2.53f * slam;
    p.a = -0.059f + 0.02483f * p.b;
    p.vr = 0.9277f - 3.6224f / (p.b - 2.0f);
    p.log_inva = logf(1.1239f + 1.1328f / (p.b - 3.4f));
    p.loglam = logf(p.lamf);
    return p;
}

// One PTRS attempt from the uniforms (U word, V word); returns k >= 0 on acceptance, -1 otherwise.
// __logf's absolute error (< 2^-21 near 1, 3 ulp elsewhere) is far below the FP32 resolution of
// the log-densities compared.
__device__ __forceinline__ int ptrs32_attempt(const Ptrs32C &p, const float *lgam, uint32_t wu, uint32_t wv) {
    const float U = u24(wu) - 0.5f;
    const float V = u24(wv);
    const float us = 0.5f - fabsf(U);
    const float kf = floorf((2.0f * p.a / us + p.b) * U + (p.frac + 0.43f));
    const bool in_range = (kf > -1.0e7f) && (kf < 1.0e7f) && !(us < 0.013f && V > us);
    const int k = in_range ? p.lam_int + (int)kf : -1;
    if (k < 0) return -1;
    if (us >= 0.07f && V <= p.vr) return k;
    const float lhs = __logf(V) + p.log_inva - __logf(p.a / (us * us) + p.b);
    float rhs;
    if (k < 16) {
        rhs = -p.lamf + (float)k * p.loglam - lgam[k];
    } else {
        // log P(k; lambda) = -bd0(k, lambda) - log(2 pi k) / 2 - stirlerr(k)
        const float kk = (float)k;
        const float d = (float)(k - p.lam_int) - p.frac;
        rhs = -bd0_f32(kk, d, p.lamf) - 0.5f * __logf(6.283185307179586f * kk) - stirlerr_f32(k);
    }
    return (lhs <= rhs) ? k : -1;
}

// PTRS in FP64 for 2^22 <= lambda <= 1e10 (and for prefix events with lambda >= 10);
// attempt `att` uses counter ctr with .w = (ctr.w | att).
__device__ double ptrs64(uint4 ctr, const PhiloxKey &key, double lam, int *d_status) {
    double slam = sqrt(lam), loglam = log(lam);
    double b = 0.931 + 2.53 * slam;
    double a = -0.059 + 0.02483 * b;
    double inva = 1.1239 + 1.1328 / (b - 3.4);
    double vr = 0.9277 - 3.6224 / (b - 2.0);
    const uint32_t w0 = ctr.w;
    for (int att = 0; att < MAX_ATTEMPTS; att++) {
        ctr.w = w0 | (uint32_t)att;
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

// Normal(lambda, sqrt(lambda)) by Box-Muller (cyutils.pyx:1328-1330)
__device__ double normal_draw(uint4 ctr, const PhiloxKey &key, double lam) {
    uint4 w = philox(ctr, key);
    double u1 = 1.0 - u53(w.x, w.y);   // (0, 1]
    double u2 = u53(w.z, w.w);
    double z = sqrt(-2.0 * log(u1)) * cos(2.0 * HGB_PI * u2);
    return lam + sqrt(lam) * z;
}

// Zero-truncated Poisson for lambda < 10, by inversion in FP64 from a 53-bit uniform.
__device__ int truncated_count(double lam, double v, int *d_status) {
    double p = lam / expm1(lam);      // P(n = 1 | n >= 1)
    double cdf = p;
    int n = 1;
    while (v >= cdf) {   // stops where the rounded CDF stops growing (v within an ulp of 1)
        if (n >= MAX_INVERSION) {
            hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
            break;
        }
        n++;
        p *= lam / n;
        const double next = cdf + p;
        if (next == cdf) break;
        cdf = next;
    }
    return n;
}

// Zero-truncated Poisson for lambda < SPARSE_MAX in FP32 (P(n >= 2) ~ lambda / 2).
__device__ int truncated_count_f32(float lam, float v, int *d_status) {
    float p = lam / expm1f(lam);      // P(n = 1 | n >= 1)
    float cdf = p;
    int n = 1;
    while (v >= cdf) {   // stops where the rounded CDF stops growing (v within an ulp of 1)
        if (n >= 64) {
            hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
            break;
        }
        n++;
        p *= lam / (float)n;
        const float next = cdf + p;
        if (next == cdf) break;
        cdf = next;
    }
    return n;
}


__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x) {
    float y = x - comp;
    float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

__device__ __forceinline__ void add_bg(SlotsPlain &st, int sl, int t, float x) { st.acc[sl][t] += x; }
__device__ __forceinline__ void slot_zero(SlotsPlain &st, int sl, int t) { st.acc[sl][t] = 0.0f; }
__device__ __forceinline__ double slot_value(const SlotsPlain &st, int sl, int t) { return (double)st.acc[sl][t]; }
__device__ __forceinline__ void slot_zero(SlotsKahan &st, int sl, int t) {
    st.acc[sl][t] = 0.0f;
    st.comp[sl][t] = 0.0f;
}
__device__ __forceinline__ double slot_value(const SlotsKahan &st, int sl, int t) {
    return (double)st.acc[sl][t] - (double)st.comp[sl][t];
}
__device__ __forceinline__ void add_bg(SlotsKahan &st, int sl, int t, float x) {
    float acc = st.acc[sl][t], comp = st.comp[sl][t];
    kahan_add(acc, comp, x);
    st.acc[sl][t] = acc;
    st.comp[sl][t] = comp;
}

// ---- 1. gather into loudest-first (F, B) order
// A 32 x 32 tile of (sorted bin, frequency) per block, transposed through shared memory: the reads
// take 32 consecutive frequencies of one bin's row, the writes 32 consecutive sorted bins of one
// frequency's row, so both sides are contiguous 256-byte runs.
constexpr int GT = 32;   // tile edge
constexpr int GR = 8;    // thread rows (GT x GR threads, GT / GR rows each)

__global__ void __launch_bounds__(GT * GR) k_gather_sorted(const double *__restrict__ number,
                                                           const double *__restrict__ h2fdf,
                                                           const int32_t *__restrict__ order, long nb, int nf,
                                                           double *__restrict__ lam_s, double *__restrict__ h_s,
                                                           int *d_status) {
    __shared__ double tl[GT][GT + 1], th[GT][GT + 1];
    const long k0 = (long)blockIdx.x * GT;
    const int f0 = blockIdx.y * GT;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int j = ty; j < GT; j += GR) {   // row j of the tile: bin k0 + j, frequencies f0 + tx
        const long k = k0 + j;
        const int f = f0 + tx;
        if (k < nb && f < nf) {
            const long o = order[k];
            const long src = o * nf + f;
            const bool ok = HGB_IN_BOUNDS(o >= 0 && o < nb, d_status);   // a caller's order
            tl[j][tx] = ok ? number[src] : 0.0;
            th[j][tx] = ok ? h2fdf[src] : 0.0;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = ty; j < GT; j += GR) {   // frequency f0 + j, bins k0 + tx
        const int f = f0 + j;
        const long k = k0 + tx;
        if (k < nb && f < nf) {
            lam_s[(long)f * nb + k] = tl[tx][j];
            h_s[(long)f * nb + k] = th[tx][j];
        }
    }
}

void launch_gather_sorted(const double *number, const double *h2fdf, const int32_t *order, long nb, int nf,
                          double *lam_s, double *h_s, cudaStream_t st, int *d_status) {
    dim3 grid((unsigned)hgb::ceil_div(nb, GT), (unsigned)hgb::ceil_div(nf, GT));
    k_gather_sorted<<<grid, dim3(GT, GR), 0, st>>>(number, h2fdf, order, nb, nf, lam_s, h_s, d_status);
}

// ---- 2. cumulative expectation along the sorted bins: C[0] = 0, C[k + 1] = C[k] + max(lambda_k, 0)
// (NaN counts as 0; with h_mask, bins whose h2fdf is zero count as 0 -- the parameter path skips
// them).  Each frequency's bins are cut into CUM_SEG segments: k_cum_sum totals the segments,
// k_cum_write scans each segment from the sum of the segments before it.
constexpr int CUM_THREADS = 1024;
constexpr int CUM_PER_THREAD = 4;
constexpr int CUM_SEG = 64;   // segments per frequency: about 8 waves of scan blocks on 152 SMs at 40 frequencies

__device__ __forceinline__ double cum_term(const double *lam, const double *mask, long k) {
    double x = lam[k];
    x = (x > 0.0) ? x : 0.0;
    if (mask && mask[k] == 0.0) x = 0.0;
    return x;
}

__global__ void __launch_bounds__(256) k_cum_sum(long nb, const double *__restrict__ lam_s,
                                                 const double *__restrict__ h_mask, double *__restrict__ seg_tot) {
    __shared__ double red[256];
    const int f = blockIdx.y, sg = blockIdx.x, t = threadIdx.x;
    const long seg = (nb + CUM_SEG - 1) / CUM_SEG;
    const long k0 = (long)sg * seg, k1 = min(k0 + seg, nb);
    const double *lam = lam_s + (long)f * nb;
    const double *mask = h_mask ? h_mask + (long)f * nb : nullptr;
    double local = 0.0;
    for (long k = k0 + t; k < k1; k += 256) local += cum_term(lam, mask, k);
    red[t] = local;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) red[t] += red[t + o];
        __syncthreads();
    }
    if (t == 0) seg_tot[(long)f * CUM_SEG + sg] = red[0];
}

__global__ void __launch_bounds__(CUM_THREADS) k_cum_write(long nb, const double *__restrict__ lam_s,
                                                           const double *__restrict__ h_mask,
                                                           const double *__restrict__ seg_tot,
                                                           double *__restrict__ cum) {
    __shared__ double wsum[CUM_THREADS / 32];
    __shared__ double carry_s;
    const int f = blockIdx.y, sg = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const long seg = (nb + CUM_SEG - 1) / CUM_SEG;
    const long k0 = (long)sg * seg, k1 = min(k0 + seg, nb);
    const double *lam = lam_s + (long)f * nb;
    const double *mask = h_mask ? h_mask + (long)f * nb : nullptr;
    double *C = cum + (long)f * (nb + 1);
    if (t == 0) {
        double c = 0.0;
        for (int j = 0; j < sg; j++) c += seg_tot[(long)f * CUM_SEG + j];
        carry_s = c;
        if (sg == 0) C[0] = 0.0;
    }
    __syncthreads();
    const long span = (long)CUM_THREADS * CUM_PER_THREAD;
    for (long base = k0; base < k1; base += span) {
        double v[CUM_PER_THREAD];
        double local = 0.0;
        const long kk = base + (long)t * CUM_PER_THREAD;
#pragma unroll
        for (int e = 0; e < CUM_PER_THREAD; e++) {
            const long k = kk + e;
            const double x = (k < k1) ? cum_term(lam, mask, k) : 0.0;
            v[e] = x;
            local += x;
        }
        double incl = local;   // inclusive warp scan of the thread totals
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            double y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            double ws = wsum[lane];
            double wi = ws;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                double y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += y;
            }
            wsum[lane] = wi - ws;   // exclusive warp offsets
        }
        __syncthreads();
        double run = carry_s + wsum[warp] + (incl - local);
#pragma unroll
        for (int e = 0; e < CUM_PER_THREAD; e++) {
            const long k = kk + e;
            run += v[e];
            if (k < k1) C[k + 1] = run;
        }
        __syncthreads();
        if (t == CUM_THREADS - 1) carry_s = run;
        __syncthreads();
    }
}

// C for every frequency into cum ((F, B + 1)); seg_tot is (F, CUM_SEG) scratch
int cumulate(long nb, int nf, const double *lam_s, const double *h_mask, double *seg_tot, double *cum,
             cudaStream_t st) {
    dim3 grid(CUM_SEG, (unsigned)nf);
    k_cum_sum<<<grid, 256, 0, st>>>(nb, lam_s, h_mask, seg_tot);
    int rc = hgb::check_launch();
    if (rc) return rc;
    k_cum_write<<<grid, CUM_THREADS, 0, st>>>(nb, lam_s, h_mask, seg_tot, cum);
    return hgb::check_launch();
}

// ---- 3. the loudest slots, thread per (f, r)
struct PrefixArgs {
    long nb;
    int nf, nr, nl;
    int f_offset;     // global index of the first frequency (counters use global frequencies)
    PhiloxKey key;
};

// Source parameters of the params path (cyutils.pyx:1541-1770): bin centres of the three axes,
// the four (B, F) grids of hgb_param_grids, and the loudest-first order to map positions to bins.
struct ParArgs {
    const int32_t *order;
    const double *mt, *mr, *rz;          // (M-1), (Q-1), (Z-1)
    const double *grid[4];               // redz_mid, dcom, sepa, angs, (B, F)
    const int *scale_log2;               // [7]
    int nq, nz;                          // bins along mrat, redz
    double *sspar;                       // (4, F, R, L)
    double *bgp_par;                     // (7, F, R): the prefix remainder's weighted sums
    double *part_par;                    // (C, 7, F, R): the chunks' weighted sums
};

__device__ __forceinline__ double bin_param(const ParArgs &p, long b, int nf, int f, int k) {
    if (k == 0) return p.mt[b / ((long)p.nq * p.nz)];
    if (k == 1) return p.mr[(b / p.nz) % p.nq];
    if (k == 2) return p.rz[b % p.nz];
    return p.grid[k - 3][b * nf + f];
}

template <bool PARAMS>
__global__ void k_loud_prefix(PrefixArgs a, ParArgs pa, const double *__restrict__ lam_s,
                              const double *__restrict__ h_s, const double *__restrict__ cum,
                              double *__restrict__ hc2ss, double *__restrict__ bgp, int *__restrict__ qpos,
                              int *d_status) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)a.nf * a.nr) return;
    const int f = (int)(idx / a.nr), r = (int)(idx % a.nr);
    const long nb = a.nb;
    const double *lam = lam_s + (long)f * nb;
    const double *h = h_s + (long)f * nb;
    const double *C = cum + (long)f * (nb + 1);
    double *ss = hc2ss + idx * a.nl;
    const double total = C[nb];
    int nfill = 0;
    double bg = 0.0;
    double wbg[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    long i = 0;
    const uint32_t max_events = (uint32_t)a.nl + MAX_PREFIX_EXTRA;
    for (uint32_t e = 0; nfill < a.nl && i < nb; e++) {
        if (e >= max_events) {
            hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
            break;
        }
        const uint32_t fg = (uint32_t)(f + a.f_offset);
        const uint4 ctr = make_uint4((uint32_t)r, fg, e, W_PREFIX);
        const uint4 w = philox(ctr, a.key);
        const double target = C[i] - log1p(-u53(w.x, w.y));   // C[i] + Exp(1)
        if (!(total > target)) {   // no further source in this realization
            i = nb;
            break;
        }
        long lo = i, hi = nb - 1;   // smallest j >= i with C[j + 1] > target (C[nb] > target)
        while (lo < hi) {
            const long mid = lo + ((hi - lo) >> 1);
            if (C[mid + 1] > target) hi = mid;
            else lo = mid + 1;
        }
        const long j = lo;
        if (!HGB_IN_BOUNDS(j >= i && j < nb, d_status)) break;
        const double lj = lam[j];
        double num;
        if (lj > NORMAL_THRESH) {
            num = normal_draw(make_uint4((uint32_t)r, fg, e, W_PREFIX | 0x8000u), a.key, lj);
        } else if (lj < PTRS_MIN) {
            num = (double)truncated_count(lj, u53(w.z, w.w), d_status);
        } else {
            num = 0.0;
            for (int rep = 0; rep < 64 && num < 1.0; rep++)
                num = ptrs64(make_uint4((uint32_t)r, fg, e, W_PREFIX | ((uint32_t)(rep + 1) << 8)), a.key,
                             lj, d_status);
            if (num < 1.0) {
                hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
                num = 1.0;
            }
        }
        i = j + 1;
        if (num < 1.0) continue;   // cyutils.pyx:1331-1332
        const double cur = h[j];
        if (PARAMS && cur == 0.0) continue;   // cyutils.pyx:1710 (not reached: such bins are masked in C)
        long bin = PARAMS ? (long)pa.order[j] : 0;
        if (!HGB_IN_BOUNDS(bin >= 0 && bin < nb, d_status)) bin = 0;
        while (nfill < a.nl && num > 0.0) {   // cyutils.pyx:1336-1340, 1711-1723
            ss[nfill] = cur;
            if (PARAMS) {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    pa.sspar[(((long)k * a.nf + f) * a.nr + r) * a.nl + nfill] = bin_param(pa, bin, a.nf, f, k);
            }
            num -= 1.0;
            nfill++;
        }
        bg += num * cur;
        if (PARAMS) {
#pragma unroll
            for (int k = 0; k < 7; k++) wbg[k] += num * cur * bin_param(pa, bin, a.nf, f, k);
        }
    }
    for (int l = nfill; l < a.nl; l++) {
        ss[l] = 0.0;
        if (PARAMS) {
#pragma unroll
            for (int k = 0; k < 4; k++) pa.sspar[(((long)k * a.nf + f) * a.nr + r) * a.nl + l] = 0.0;
        }
    }
    bgp[idx] = bg;
    if (PARAMS) {
#pragma unroll
        for (int k = 0; k < 7; k++) pa.bgp_par[(long)k * a.nf * a.nr + idx] = wbg[k];
    }
    qpos[idx] = (int)i;
}

// ---- 4. bulk background
struct BulkArgs {
    long nb;
    int nf, nr;
    int f_offset;      // global index of the first frequency (counters use global frequencies)
    int nchunk;        // chunk c holds tiles c, c + nchunk, c + 2 nchunk, ...
    uint32_t domain;
    PhiloxKey key;
    int *wide_flag;    // set by k_bulk when it leaves bins to k_bulk_wide (zeroed before the launch)
};

// Inversion table of one table-kind bin (lambda in [10, TABLE_MAX]), built by a warp or a block:
//   cdf[m]   = min(sum of q(k_lo) .. q(k_lo + m), 2^32 - 1), with q(k) = P(k) in 32.32 fixed point
//              (rounded to nearest); cdf[S - 1] = 2^32 - 1, so the mass outside the range (< 1e-11)
//              goes to the end entries;
//   guide[c] = m | flags, m (bits 0-11) the smallest entry with cdf[m] > c 2^(32 - gb), for the
//              2^gb >= S / 2 cells: about one cell per two entries.  Against 2^gb >= S cells the
//              draws cost more (more cells hold several boundaries), but the guide builds faster,
//              tables up to 2048 entries fit half the arena (one warp builds them, not the block) and
//              more tables share a batch barrier: on the bench workload k_bulk takes 27.5 ms against
//              28.9 ms (2^gb >= S / 4: 28.3 ms).  GUIDE_PURE when cdf[m] >= (c + 1) 2^(32 - gb), so
//              every u in the cell
//              maps to m; GUIDE_ONE when instead cdf[m + 1] >= (c + 1) 2^(32 - gb), so u maps to m or
//              m + 1 by one comparison; neither: two or more entries end inside the cell (a "tail"
//              cell of the distribution), resolved by a binary search between guide[c] and
//              guide[c + 1].
// P(k) is FP32: the Loader form at every ANCHOR-th entry and the recursion P(k) = P(k-1) lambda / k
// in between (__fdividef: at most 2 ulp per step, so under 32 ulp of drift before the next anchor).
// Each thread takes E consecutive entries; the guide is the merge of the cdf values with the cell
// starts, split evenly over the threads (merge path), so no thread waits on another's long run of
// cells or entries.

// q of the entries m0 .. m1 - 1 into cdf[m]; returns their sum, which stays below 2^31 (a thread's
// entries span at most 1/32 of the table, well under half the probability)
__device__ __forceinline__ unsigned table_pmf(const Tile &s, int j, unsigned int *cdf, int m0, int m1) {
    const int k_lo = s.tb_klo[j], lam_int = s.lam_int[j];
    const float frac = s.frac[j], lamf = s.lamf[j];
    unsigned local = 0;
    for (int a = m0; a < m1; a += ANCHOR) {
        float kf = (float)(k_lo + a);   // exact: k < 2^24
        float p = pmf_f32(k_lo + a, lam_int, frac, lamf);
        unsigned q = __float2uint_rn(p * 0x1.0p32f);
        cdf[a] = q;
        local += q;
        const int n = min(ANCHOR, m1 - a);
#pragma unroll
        for (int i = 1; i < ANCHOR; i++) {
            if (i < n) {
                kf += 1.0f;
                p *= __fdividef(lamf, kf);
                q = __float2uint_rn(p * 0x1.0p32f);
                cdf[a + i] = q;
                local += q;
            }
        }
    }
    return local;
}

// running sums of the thread's entries on top of base (the 64-bit sum of every earlier entry),
// saturated at 2^32 - 1 with 32-bit arithmetic
__device__ __forceinline__ void table_prefix(unsigned int *cdf, int m0, int m1, unsigned long long base) {
    const bool full = base >= 0xFFFFFFFFull;
    const unsigned b32 = full ? 0xFFFFFFFFu : (unsigned)base;
    const unsigned room = full ? 0u : (unsigned)(0xFFFFFFFFull - base);
    unsigned run = 0;
    for (int m = m0; m < m1; m++) {
        run += cdf[m];
        cdf[m] = b32 + min(run, room);
    }
}

// the guide cells from the finished cdf: thread t of nthr walks diagonals [d0, d1) of the merge of
// cdf[0 .. S-1] with the cell starts c 2^shift (a cdf value goes first on ties)
__device__ __forceinline__ void table_guide(const unsigned int *cdf, unsigned short *guide, int S, int gb, int t,
                                            int nthr) {
    const int shift = 32 - gb, nc = 1 << gb;
    const int total = S + nc;
    const int D = (total + nthr - 1) / nthr;
    const int d0 = min(t * D, total), d1 = min(d0 + D, total);
    int lo = max(0, d0 - nc), hi = min(d0, S);   // cdf values among the first d0 merged elements
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid] <= ((unsigned)(d0 - 1 - mid) << shift)) lo = mid + 1;
        else hi = mid;
    }
    int m = lo, c = d0 - lo;
    unsigned am = cdf[min(m, S - 1)], an = cdf[min(m + 1, S - 1)];   // cdf[m] and cdf[m + 1]
    for (int d = d0; d < d1 && c < nc; d++) {
        if (am <= ((unsigned)c << shift)) {   // m < S - 1: cdf[S - 1] = 2^32 - 1 exceeds every cell start
            m++;
            am = an;
            an = cdf[min(m + 1, S - 1)];
        } else {
            unsigned code = (unsigned)m;
            if ((am >> shift) > (unsigned)c) code |= GUIDE_PURE;
            else if (m + 1 < S && (an >> shift) > (unsigned)c) code |= GUIDE_ONE;
            guide[c] = (unsigned short)code;
            c++;
        }
    }
}

// one warp builds the table of bin j (tables of at most HALF_WORDS words)
__device__ void build_table_warp(const Tile &s, int j, unsigned int *cdf, unsigned short *guide, int lane) {
    const int S = s.tb_S[j];
    const int E = (S + 31) >> 5;
    const int m0 = min(lane * E, S), m1 = min(m0 + E, S);
    const unsigned local = table_pmf(s, j, cdf, m0, m1);
    unsigned long long incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    table_prefix(cdf, m0, m1, incl - local);
    if (m0 < S && m1 == S) cdf[S - 1] = 0xFFFFFFFFu;
    __syncwarp();
    table_guide(cdf, guide, S, s.tb_gb[j], lane, 32);
    __syncwarp();
}

// the whole block builds the table of bin j (large tables); starts and ends with a barrier-protected
// table
__device__ void build_table_block(Tile &s, int j, unsigned int *cdf, unsigned short *guide) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int S = s.tb_S[j];
    const int E = (S + RB - 1) / RB;
    const int m0 = min(t * E, S), m1 = min(m0 + E, S);
    const unsigned local = table_pmf(s, j, cdf, m0, m1);
    unsigned long long incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s.scan[warp] = incl;
    __syncthreads();
    unsigned long long base = incl - local;
    for (int w = 0; w < warp; w++) base += s.scan[w];
    table_prefix(cdf, m0, m1, base);
    if (m0 < S && m1 == S) cdf[S - 1] = 0xFFFFFFFFu;
    __syncthreads();
    table_guide(cdf, guide, S, s.tb_gb[j], t, RB);
    __syncthreads();
}

// arena words of a table-kind bin: S cdf entries and 2^gb u16 guide cells
__device__ __forceinline__ int table_words(const Tile &s, int j) { return s.tb_S[j] + (1 << (s.tb_gb[j] - 1)); }

// SORTED: lam / h are the gathered (F, B) arrays and qpos gives each realization's first bulk
// position; otherwise lam / h are the (B, F) grids and every bin belongs to the bulk.
// Parameter path: the seven weighted background sums per realization, FP32 Kahan in dynamic
// shared memory [k][slot][thread], each term n * h2fdf * 2^100 * p_k * 2^-e_k (e_k the frexp exponent
// of max |p_k|, so every scaled parameter is at most 1).
constexpr int NPAR = 7;
constexpr size_t PAR_SMEM = sizeof(float) * (NPAR * RB + 2 * NPAR * RPT * RB);

__device__ __forceinline__ void add_par(float *psm, int sl, int t, int j, float n) {
    const float *pw = psm;
    float *pacc = psm + NPAR * RB;
    float *pcomp = pacc + NPAR * RPT * RB;
#pragma unroll
    for (int k = 0; k < NPAR; k++) {
        const int o = (k * RPT + sl) * RB + t;
        float acc = pacc[o], comp = pcomp[o];
        kahan_add(acc, comp, n * pw[k * RB + j]);
        pacc[o] = acc;
        pcomp[o] = comp;
    }
}

// Shared state of one k_bulk block (static shared memory of the kernels that run bulk_block).
template <bool PARAMS>
struct BulkShared {
    Tile s;
    typename std::conditional<PARAMS, SlotsKahan, SlotsPlain>::type st;
    int q_min_s, q_max_s;
};

// One k_bulk block's work: chunk c (tiles c, c + nchunk, ...) of frequency f for the realizations of
// group rg (rg * RB * RPT + thread + i * RB, i < RPT), written to part[c][f][r].  Every shared word it
// reads it first writes, so a block may run it for several (c, f, rg) in turn.
template <bool SORTED, bool PARAMS>
__device__ __forceinline__ void bulk_block(const BulkArgs &a, const ParArgs &pa, const double *__restrict__ lam_in,
                                           const double *__restrict__ h_in, const int *__restrict__ qpos,
                                           double *__restrict__ part, int *d_status, const int c, const int f,
                                           const int rg, BulkShared<PARAMS> &sh, float *psm) {
    Tile &s = sh.s;
    auto &st = sh.st;
    int &q_min_s = sh.q_min_s;
    int &q_max_s = sh.q_max_s;
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    const int r0 = rg * RB * RPT + t;
    int rpt = 0;   // realizations of this thread: r0 + i * RB, i < rpt
    while (rpt < RPT && r0 + rpt * RB < a.nr) rpt++;
    // register accumulators for the passes with a fixed realization slot
    float acc_r[RPT], comp_r[RPT];
    int qmin = 0x7FFFFFFF, qmax = 0;
#pragma unroll
    for (int i = 0; i < RPT; i++) {
        acc_r[i] = 0.0f;
        comp_r[i] = 0.0f;
        slot_zero(st, i, t);
        int q = 0x7FFFFFFF;
        if (i < rpt) q = SORTED ? qpos[(long)f * a.nr + r0 + i * RB] : 0;
        if (i < rpt) {
            qmin = min(qmin, q);
            qmax = max(qmax, q);
        }
    }
    if (PARAMS) {
        for (int o = t; o < 2 * NPAR * RPT * RB; o += RB) psm[NPAR * RB + o] = 0.0f;
    }
    if (t < 16) s.lgam[t] = c_lgam[t];
    if (t == 0) {
        q_min_s = 0x7FFFFFFF;
        q_max_s = 0;
    }
    __syncthreads();
    if (SORTED) {
        atomicMin(&q_min_s, qmin);
        atomicMax(&q_max_s, qmax);
    }
    __syncthreads();
    const int block_qmin = SORTED ? q_min_s : 0;
    const int block_qmax = SORTED ? q_max_s : 0;
    const uint4 ctr0 = make_uint4(0u, (uint32_t)r0, (uint32_t)(f + a.f_offset), a.domain);
    // first bulk position of slot sl, for the passes whose slot is data dependent
    const int *q_row = SORTED ? qpos + (long)f * a.nr + r0 : nullptr;
    const long ntiles = (a.nb + RB - 1) / RB;
    for (long tile = c; tile < ntiles; tile += a.nchunk) {
        const long base = tile * RB;
        const int nt = (int)((a.nb - base) < RB ? (a.nb - base) : RB);
        if (base + nt <= (long)block_qmin) continue;   // every bin precedes every realization's bulk
        const bool check = SORTED && base < (long)block_qmax;
        __syncthreads();
        int kind = KIND_NONE;
        if (t < nt) {
            const long b = base + t;
            const double lam = SORTED ? lam_in[(long)f * a.nb + b] : lam_in[b * a.nf + f];
            kind = bin_kind(lam);
            if (kind != KIND_NONE) {
                const double h = SORTED ? h_in[(long)f * a.nb + b] : h_in[b * a.nf + f];
                if (PARAMS && h == 0.0) {
                    kind = KIND_NONE;   // cyutils.pyx:1710: skipped
                } else {
                    bin_setup(s, t, kind, lam, h);
                    s.pos[t] = (int)b;
                    if (PARAMS) {
                        const long bin = SORTED ? (long)pa.order[b] : b;
#pragma unroll
                        for (int k = 0; k < NPAR; k++)
                            psm[k * RB + t] =
                                (float)ldexp(h * (double)HSCALE * bin_param(pa, bin, a.nf, f, k), -pa.scale_log2[k]);
                    }
                }
            }
        }
        // per-kind lists in bin order: warp ballots, then the warps' offsets
        unsigned rank_mask = 0;
#pragma unroll
        for (int k = 1; k < NKIND; k++) {
            const unsigned m = __ballot_sync(0xffffffffu, kind == k);
            if (kind == k) rank_mask = m;
            if (lane == 0) s.wcount[warp][k] = __popc(m);
        }
        __syncthreads();
        if (kind != KIND_NONE) {
            int off = 0;
            for (int w = 0; w < warp; w++) off += s.wcount[w][kind];
            off += __popc(rank_mask & ((1u << lane) - 1u));
            s.list[kind][off] = (unsigned char)t;
        }
        __syncthreads();

        // ---- small lambda: per-bin 32-entry table, four realizations per Philox call
        const int n_small = kind_count(s, KIND_SMALL);
#pragma unroll 1
        for (int li = 0; li < n_small; li++) {
            const int j = s.list[KIND_SMALL][li];
            const int pos = s.pos[j];
            const float hs = s.hs[j];
            const unsigned int *row = s.u.thr[j];
            uint4 wv[RPT / 4];   // every call issued first: independent round chains interleave
#pragma unroll
            for (int call = 0; call < RPT / 4; call++) {
                uint4 ctr = ctr0;
                ctr.x = (uint32_t)pos;
                ctr.w |= W_SMALL | (uint32_t)call;
                wv[call] = philox(ctr, a.key);
            }
#pragma unroll
            for (int call = 0; call < RPT / 4; call++) {
                if (4 * call >= rpt) break;
                const uint4 w = wv[call];
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    const int sl = 4 * call + m;
                    const uint32_t u = (m == 0) ? w.x : (m == 1) ? w.y : (m == 2) ? w.z : w.w;
                    if (sl >= rpt) continue;
                    // column u >> 27, fraction the low 27 bits: P(n) = q(n) / 2^32 exactly
                    const unsigned wd = row[u >> 27];
                    const int n = ((u & 0x07FFFFFFu) < (wd >> 5)) ? (int)(u >> 27) : (int)(wd & 31u);
                    if (n != 0 && (!check || pos >= __ldg(q_row + sl * RB))) {
                        kahan_add(acc_r[sl], comp_r[sl], (float)n * hs);
                        if (PARAMS) add_par(psm, sl, t, j, (float)n);
                    }
                }
            }
        }

        // ---- table kind: inversion tables of up to BATCH_MAX bins at a time.  Tables that fit half the
        // arena are built one per warp into the half the draws are not reading: batch k + 1 is built
        // while batch k is drawn, one barrier per batch.  Larger tables use the whole arena and the
        // whole block.  Four realizations per Philox call.
        const int n_table = kind_count(s, KIND_TABLE);
        if (n_table > 0) {
            // largest tables first: big tables come in batches of their own and the many small ones
            // share later batches, where the warps' builds balance (rank sort of the tile's list;
            // the draws are keyed by bin, so only the summation order of the background changes)
            int jt = 0, rank = 0;
            if (t < n_table) {
                jt = s.list[KIND_TABLE][t];
                const int St = s.tb_S[jt];
                for (int u = 0; u < n_table; u++) {
                    const int Su = s.tb_S[s.list[KIND_TABLE][u]];
                    rank += (Su > St || (Su == St && u < t)) ? 1 : 0;
                }
            }
            __syncthreads();   // every entry is read before any is moved
            if (t < n_table) s.list[KIND_TABLE][rank] = (unsigned char)jt;
            __syncthreads();   // the sorted list is complete before any batch is formed
            int li = 0;
            int cur_li = 0, cur_K = 0, cur_half = 0;
            bool cur_big = false;
            // the batch starting at list entry li (same on every thread)
            auto form = [&](int at, int &K, bool &big) {
                big = table_words(s, s.list[KIND_TABLE][at]) > HALF_WORDS;
                K = 1;
                if (big) return;
                int used = table_words(s, s.list[KIND_TABLE][at]);
                while (at + K < n_table && K < BATCH_MAX) {
                    const int words = table_words(s, s.list[KIND_TABLE][at + K]);
                    if (words > HALF_WORDS || used + words > HALF_WORDS) break;
                    used += words;
                    K++;
                }
            };
            // build a small batch into a half, each table by the least-loaded warp (by entries)
            auto build_small = [&](int at, int K, int half) {
                int load[NWARP] = {};
                int off = half * HALF_WORDS;
                for (int i = 0; i < K; i++) {
                    const int j = s.list[KIND_TABLE][at + i];
                    int wmin = 0;
#pragma unroll
                    for (int w = 1; w < NWARP; w++)
                        if (load[w] < load[wmin]) wmin = w;
                    load[wmin] += s.tb_S[j];
                    if (wmin == warp)
                        build_table_warp(s, j, s.u.arena + off, (unsigned short *)(s.u.arena + off + s.tb_S[j]), lane);
                    off += table_words(s, j);
                }
            };
            form(li, cur_K, cur_big);
            cur_li = li;
            li += cur_K;
            __syncthreads();   // the arena is free (the small-lambda pass is done)
            if (cur_big) {
                const int j = s.list[KIND_TABLE][cur_li];
                build_table_block(s, j, s.u.arena, (unsigned short *)(s.u.arena + s.tb_S[j]));
            } else {
                build_small(cur_li, cur_K, 0);
                __syncthreads();
            }
#pragma unroll 1
            while (true) {
                // prebuild the next batch when both it and the current one are small
                int nxt_li = li, nxt_K = 0;
                bool nxt_big = false;
                if (!cur_big && li < n_table) {
                    form(li, nxt_K, nxt_big);
                    if (nxt_big) nxt_K = 0;
                    else {
                        li += nxt_K;
                        build_small(nxt_li, nxt_K, cur_half ^ 1);
                    }
                }
                // draw the current batch
                int off = cur_big ? 0 : cur_half * HALF_WORDS;
#pragma unroll 1
                for (int i = 0; i < cur_K; i++) {
                    const int j = s.list[KIND_TABLE][cur_li + i];
                    const int pos = s.pos[j];
                    const float hs = s.hs[j];
                    const int k_lo = s.tb_klo[j], S = s.tb_S[j], gb = s.tb_gb[j], shift = 32 - gb;
                    const unsigned int *cdf = s.u.arena + off;
                    const unsigned short *guide = (const unsigned short *)(s.u.arena + off + S);
                    off += table_words(s, j);
                    uint4 wv[RPT / 4];   // every call issued first: independent round chains interleave
#pragma unroll
                    for (int call = 0; call < RPT / 4; call++) {
                        uint4 ctr = ctr0;
                        ctr.x = (uint32_t)pos;
                        ctr.w |= W_TABLE | (uint32_t)call;
                        wv[call] = philox(ctr, a.key);
                    }
                    // Straight-line lookups (no data-dependent branch, so the eight draws
                    // interleave): a pure cell answers from the guide, a one-boundary cell with one
                    // comparison.  Draws in tail cells (a few percent) are marked and finished after
                    // the bin's other draws by a binary search inside the cell.
                    unsigned pend = 0;
#pragma unroll
                    for (int call = 0; call < RPT / 4; call++) {
                        if (4 * call >= rpt) break;
                        const uint4 w = wv[call];
#pragma unroll
                        for (int m = 0; m < 4; m++) {
                            const int sl = 4 * call + m;
                            const uint32_t u = (m == 0) ? w.x : (m == 1) ? w.y : (m == 2) ? w.z : w.w;
                            if (sl >= rpt) continue;
                            const uint32_t uc = min(u, 0xFFFFFFFEu);   // below cdf[S - 1]
                            const unsigned g = guide[uc >> shift];
                            int e = (int)(g & GUIDE_M);
                            if (!HGB_IN_BOUNDS(e < S - 1 || !(g & GUIDE_ONE), d_status)) e = 0;
                            if (g & GUIDE_ONE) e += (uc >= cdf[e]) ? 1 : 0;
                            if (!HGB_IN_BOUNDS(e < S, d_status)) e = S - 1;
                            const bool tail = !(g & (GUIDE_PURE | GUIDE_ONE));
                            pend |= tail ? (1u << sl) : 0u;
                            if (!tail && (!check || pos >= __ldg(q_row + sl * RB))) {
                                kahan_add(acc_r[sl], comp_r[sl], (float)(k_lo + e) * hs);
                                if (PARAMS) add_par(psm, sl, t, j, (float)(k_lo + e));
                            }
                        }
                    }
                    if (__any_sync(0xffffffffu, pend != 0)) {
                        // the lane's tail draws in turn; their slot is data dependent, so the sums
                        // go to the shared-memory Kahan accumulators
#pragma unroll 1
                        while (pend) {
                            const int sl = __ffs(pend) - 1;
                            pend &= pend - 1;
                            const uint4 w = (sl < 4) ? wv[0] : wv[RPT / 4 - 1];
                            const int q4 = sl & 3;
                            const uint32_t u = (q4 == 0) ? w.x : (q4 == 1) ? w.y : (q4 == 2) ? w.z : w.w;
                            const uint32_t uc = min(u, 0xFFFFFFFEu);
                            const unsigned cell = uc >> shift;
                            int lo = (int)(guide[cell] & GUIDE_M);
                            int hi = (cell + 1 < (1u << gb)) ? (int)(guide[cell + 1] & GUIDE_M) : S - 1;
                            if (!HGB_IN_BOUNDS(lo <= hi && hi < S, d_status)) lo = hi = S - 1;
                            while (lo < hi) {   // cdf[hi] > uc throughout
                                const int mid = (lo + hi) >> 1;
                                if (uc >= cdf[mid]) lo = mid + 1;
                                else hi = mid;
                            }
                            if (!check || pos >= __ldg(q_row + sl * RB)) {
                                add_bg(st, sl, t, (float)(k_lo + lo) * hs);
                                if (PARAMS) add_par(psm, sl, t, j, (float)(k_lo + lo));
                            }
                        }
                    }
                }
                __syncthreads();   // the current batch is drawn and the next one built
                if (nxt_K > 0) {
                    cur_li = nxt_li;
                    cur_K = nxt_K;
                    cur_big = false;
                    cur_half ^= 1;
                    continue;
                }
                if (li >= n_table) break;
                form(li, cur_K, cur_big);
                cur_li = li;
                li += cur_K;
                if (cur_big) {
                    const int j = s.list[KIND_TABLE][cur_li];
                    build_table_block(s, j, s.u.arena, (unsigned short *)(s.u.arena + s.tb_S[j]));
                } else {
                    cur_half = 0;
                    build_small(cur_li, cur_K, 0);
                    __syncthreads();
                }
            }
        }

        // ---- PTRS32: one loop per lane over its realizations, two attempts per Philox call
        const int n_ptrs = kind_count(s, KIND_PTRS32);
#pragma unroll 1
        for (int li = 0; li < n_ptrs; li++) {
            if (rpt == 0) break;
            const int j = s.list[KIND_PTRS32][li];
            const int pos = s.pos[j];
            const float hs = s.hs[j];
            const Ptrs32C pc = ptrs32_consts(s, j);
            uint4 ctr = ctr0;
            ctr.x = (uint32_t)pos;
            ctr.w |= W_PTRS;
            int sl = 0, it = 0;
            uint4 w = make_uint4(0, 0, 0, 0);
#pragma unroll 1
            while (sl < rpt) {
                if ((it & 1) == 0) {
                    uint4 cc = ctr;
                    cc.w |= (uint32_t)(it >> 1);
                    w = philox(cc, a.key);
                }
                const int k = (it & 1) ? ptrs32_attempt(pc, s.lgam, w.z, w.w) : ptrs32_attempt(pc, s.lgam, w.x, w.y);
                it++;
                if (k >= 0) {
                    if (!check || pos >= __ldg(q_row + sl * RB)) {
                        add_bg(st, sl, t, (float)k * hs);
                        if (PARAMS) add_par(psm, sl, t, j, (float)k);
                    }
                    sl++;
                } else if (it >= MAX_PTRS_ITERS) {
                    hgb::flag(d_status, HGB_STATUS_ITERATION_LIMIT);
                    const float kfix = floorf(pc.lamf + 0.5f);
                    for (; sl < rpt; sl++)
                        if (!check || pos >= __ldg(q_row + sl * RB)) {
                            add_bg(st, sl, t, kfix * hs);
                            if (PARAMS) add_par(psm, sl, t, j, kfix);
                        }
                }
            }
        }

        // ---- sparse (lambda < SPARSE_MAX): geometric skipping, the gap to the next realization with
        // n >= 1 being floor(-ln u / lambda) and n zero-truncated Poisson
        const int n_sparse = kind_count(s, KIND_SPARSE);
        if (PARAMS) {
            // the lane's own realizations, so the parameter sums stay thread-private
#pragma unroll 1
            for (int li = 0; li < n_sparse; li++) {
                if (rpt == 0) break;
                const int j = s.list[KIND_SPARSE][li];
                const int pos = s.pos[j];
                const float lf = s.lamf[j];
                const float hs = s.hs[j];
                uint4 ctr = ctr0;
                ctr.x = (uint32_t)pos;
                ctr.w |= W_SKIP;
                int i = 0;
                for (int step = 0; step < 2 * RPT + 2; step++) {
                    uint4 cc = ctr;
                    cc.w |= (uint32_t)step;
                    const uint4 w = philox(cc, a.key);
                    // U = (u + 1) 2^-64 in (0, 1]: -ln U = -log1p(-x) with x = (2^64 - 1 - u) 2^-64
                    const float x = fminf(__ull2float_rn(~w64(w.x, w.y)) * 0x1.0p-64f, 0.99999994f);
                    const float gap = floorf(-log1pf(-x) / lf);
                    if (gap >= (float)(rpt - i)) break;
                    i += (int)gap;
                    const int n = truncated_count_f32(lf, u24(w.z), d_status);
                    if (!check || pos >= __ldg(q_row + i * RB)) {
                        add_bg(st, i, t, (float)n * hs);
                        add_par(psm, i, t, j, (float)n);
                    }
                    i++;
                    if (i >= rpt) break;
                }
            }
        } else if (n_sparse > 0) {
            // The block's realizations cut into runs of 2^lg per bin (about one expected event per
            // run); the runs of the tile's sparse bins are numbered in list order and shared out
            // over the threads, each walking its run by geometric gaps.  Events go to per-tile sums
            // by realization in the arena, in 64-bit fixed point with unit 2^(e - 50) for e the
            // largest exponent of the tile's sparse strains: integer atomics, so the sums do not
            // depend on the order the threads reach them (4096 times the largest term of headroom;
            // a realization sees a few events per tile).  Each thread then folds its slots into its
            // Kahan sums.
            unsigned long long *sub = reinterpret_cast<unsigned long long *>(s.u.arena);   // [RPT * RB]
            const int nr_blk = min(RB * RPT, a.nr - rg * RB * RPT);
            int runs = 0, e_hs = -1000;
            if (t < n_sparse) {
                const int js = s.list[KIND_SPARSE][t];
                const int lg = s.sp_lg[js];
                runs = (nr_blk + (1 << lg) - 1) >> lg;
                frexpf(s.hs[js], &e_hs);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) e_hs = max(e_hs, __shfl_xor_sync(0xffffffffu, e_hs, o));
            int incl = runs;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            __syncthreads();   // the arena and the scan words are free
            if (lane == 31) s.scan[warp] = ((unsigned long long)(unsigned)(e_hs + 2048) << 32) | (unsigned)incl;
#pragma unroll
            for (int i = 0; i < RPT; i++) sub[i * RB + t] = 0ull;
            __syncthreads();
            int before = 0, total = 0, e_max = -1000;
#pragma unroll
            for (int w = 0; w < NWARP; w++) {
                const unsigned long long x = s.scan[w];
                const int v = (int)(unsigned)x;
                before += (w < warp) ? v : 0;
                total += v;
                e_max = max(e_max, (int)(x >> 32) - 2048);
            }
            const int fx_shift = 50 - e_max;   // term x -> round(x 2^fx_shift)
            if (t < n_sparse) s.sp_start[t] = before + incl - runs;
            __syncthreads();
            const int *q_blk = SORTED ? q_row - t : nullptr;   // first bulk positions of the block's realizations
#pragma unroll 1
            for (int k = t; k < total; k += RB) {
                int lo = 0, hi = n_sparse - 1;   // the last list entry whose runs start at or before k
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s.sp_start[mid] <= k) lo = mid;
                    else hi = mid - 1;
                }
                const int j = s.list[KIND_SPARSE][lo];
                const int lg = s.sp_lg[j];
                const int run = k - s.sp_start[lo];   // < 128: runs hold at least 8 realizations
                const int re = min((run + 1) << lg, nr_blk);
                const float lf = s.lamf[j], hs = s.hs[j];
                const int pos = s.pos[j];
                const uint4 ctr = make_uint4((uint32_t)pos, ((uint32_t)rg << 7) | (uint32_t)run,
                                             (uint32_t)(f + a.f_offset), a.domain | W_SPARSE);
                int r = run << lg;   // the next gap counts from here
                // every event advances r, so a run takes at most 2^lg + 1 steps
                for (int ev = 0; ev <= (1 << lg); ev++) {
                    uint4 cc = ctr;
                    cc.w |= (uint32_t)ev;
                    const uint4 w = philox(cc, a.key);
                    const float x = fminf(__ull2float_rn(~w64(w.x, w.y)) * 0x1.0p-64f, 0.99999994f);
                    const float gap = floorf(-log1pf(-x) / lf);
                    if (gap >= (float)(re - r)) break;
                    r += (int)gap;
                    const int n = truncated_count_f32(lf, u24(w.z), d_status);
                    if (!check || pos >= __ldg(q_blk + r))
                        atomicAdd(&sub[r], __float2ull_rn(ldexpf((float)n * hs, fx_shift)));
                    if (++r >= re) break;
                }
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < RPT; i++)
                if (i < rpt) kahan_add(acc_r[i], comp_r[i], (float)ldexp((double)sub[i * RB + t], -fx_shift));
        }

        // ---- PTRS64 / Normal (real-valued counts, cyutils.pyx:1327-1330 / :887-891); without the
        // parameter sums these bins go to k_bulk_wide, which keeps their FP64 code out of this kernel
        if (!PARAMS && t == 0 && kind_count(s, KIND_WIDE) > 0) atomicOr(a.wide_flag, 1);
        const int n_wide = PARAMS ? kind_count(s, KIND_WIDE) : 0;
#pragma unroll 1
        for (int li = 0; li < n_wide; li++) {
            const int j = s.list[KIND_WIDE][li];
            const int pos = s.pos[j];
            const double lam = s.lam[j];
            const float hs = s.hs[j];
            for (int sl = 0; sl < rpt; sl++) {
                uint4 ctr = ctr0;
                ctr.x = (uint32_t)pos;
                ctr.w |= W_WIDE | ((uint32_t)sl << 8);
                const double num = (lam > NORMAL_THRESH) ? normal_draw(ctr, a.key, lam) : ptrs64(ctr, a.key, lam, d_status);
                if (!check || pos >= __ldg(q_row + sl * RB)) {
                    add_bg(st, sl, t, (float)(num * (double)hs));
                    if (PARAMS) add_par(psm, sl, t, j, (float)num);
                }
            }
        }
    }
    const bool part_ok = HGB_IN_BOUNDS(c < a.nchunk && f < a.nf, d_status);
#pragma unroll
    for (int i = 0; i < RPT; i++)
        if (i < rpt && part_ok)
            part[((long)c * a.nf + f) * a.nr + r0 + (long)i * RB] =
                (((double)acc_r[i] - (double)comp_r[i]) + slot_value(st, i, t)) * HSCALE_INV;
    if (PARAMS) {
        const float *pacc = psm + NPAR * RB;
        const float *pcomp = pacc + NPAR * RPT * RB;
        for (int k = 0; k < NPAR; k++)
            for (int i = 0; i < rpt; i++) {
                const int o = (k * RPT + i) * RB + t;
                pa.part_par[(((long)c * NPAR + k) * a.nf + f) * a.nr + r0 + (long)i * RB] =
                    ldexp(((double)pacc[o] - (double)pcomp[o]) * HSCALE_INV, pa.scale_log2[k]);
            }
    }
}

// grid (nchunk, nf, realization groups): block (c, f, rg) runs bulk_block for itself
template <bool SORTED, bool PARAMS>
__global__ void __launch_bounds__(RB, PARAMS ? 2 : BULK_BLOCKS_PER_SM) k_bulk(BulkArgs a, ParArgs pa, const double *__restrict__ lam_in,
                                                          const double *__restrict__ h_in,
                                                          const int *__restrict__ qpos, double *__restrict__ part,
                                                          int *d_status) {
    __shared__ BulkShared<PARAMS> sh;
    extern __shared__ float psm[];   // PARAMS only: PAR_SMEM bytes
    bulk_block<SORTED, PARAMS>(a, pa, lam_in, h_in, qpos, part, d_status, blockIdx.x, blockIdx.y, blockIdx.z, sh, psm);
}

// ---- 4c. many samples in one launch.  A sample's realization stage is the (chunk, frequency,
// realization group) blocks of its own k_bulk grid; the work list names them as items
// (sample, c, f, rg), and k_bulk_multi runs bulk_block for each item.  With `next` a block takes
// items from the counter until the list is exhausted (a persistent grid of a few blocks per SM);
// without it block i runs item i.  Each item computes exactly what block (c, f, rg) of the sample's
// own k_bulk launch computes, so a sample's partials do not depend on the batch around it.
struct BulkJob {
    BulkArgs a;
    const double *lam, *h;
    const int *q;
    double *part;
    int *status;
};

__global__ void __launch_bounds__(RB, BULK_BLOCKS_PER_SM) k_bulk_multi(const BulkJob *__restrict__ jobs,
                                                                       const int4 *__restrict__ items, int n_items,
                                                                       int *next) {
    __shared__ BulkShared<false> sh;
    __shared__ int s_item;
    int it = next ? -1 : (int)blockIdx.x;
    while (true) {
        if (next) {
            __syncthreads();   // the previous item is finished with the shared state
            if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
            __syncthreads();
            it = s_item;
        }
        if (it >= n_items) break;
        const int4 w = items[it];
        const BulkJob &J = jobs[w.x];   // read where used (L1), not held in registers
        bulk_block<true, false>(J.a, ParArgs{}, J.lam, J.h, J.q, J.part, J.status, w.y, w.z, w.w, sh, nullptr);
        if (!next) break;
    }
}

// ---- 4b. bins above PTRS32_MAX (PTRS64 / Normal in FP64) when k_bulk leaves them out: the same
// grid, chunks and realizations as k_bulk, run after it on the same stream; each block adds its
// wide bins' sums (FP64, bin order) to the partials k_bulk wrote, and blocks without wide bins
// write nothing.
struct WideShared {
    double w_lam[RB], w_h[RB];
    int w_pos[RB];
    int w_count[NWARP];
};

template <bool SORTED>
__device__ __forceinline__ void wide_block(const BulkArgs &a, const double *__restrict__ lam_in,
                                           const double *__restrict__ h_in, const int *__restrict__ qpos,
                                           double *__restrict__ part, int *d_status, const int c, const int f,
                                           const int rg, WideShared &sh) {
    double *w_lam = sh.w_lam, *w_h = sh.w_h;
    int *w_pos = sh.w_pos, *w_count = sh.w_count;
    if (*(volatile int *)a.wide_flag == 0) return;   // k_bulk met no such bin (uniform over the grid)
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    const int r0 = rg * RB * RPT + t;
    int rpt = 0;
    while (rpt < RPT && r0 + rpt * RB < a.nr) rpt++;
    const int *q_row = SORTED ? qpos + (long)f * a.nr + r0 : nullptr;
    const uint4 ctr0 = make_uint4(0u, (uint32_t)r0, (uint32_t)(f + a.f_offset), a.domain);
    double acc[RPT];
#pragma unroll
    for (int i = 0; i < RPT; i++) acc[i] = 0.0;
    bool any = false;   // block-uniform
    const long ntiles = (a.nb + RB - 1) / RB;
    for (long tile = c; tile < ntiles; tile += a.nchunk) {
        const long base = tile * RB;
        const int nt = (int)((a.nb - base) < RB ? (a.nb - base) : RB);
        bool wide = false;
        double lam = 0.0;
        if (t < nt) {
            lam = SORTED ? lam_in[(long)f * a.nb + base + t] : lam_in[(base + t) * a.nf + f];
            wide = bin_kind(lam) == KIND_WIDE;
        }
        const unsigned m = __ballot_sync(0xffffffffu, wide);
        __syncthreads();   // the previous tile's list is drawn
        if (lane == 0) w_count[warp] = __popc(m);
        __syncthreads();
        int off = 0, n = 0;
#pragma unroll
        for (int w = 0; w < NWARP; w++) {
            off += (w < warp) ? w_count[w] : 0;
            n += w_count[w];
        }
        if (wide) {
            const int k = off + __popc(m & ((1u << lane) - 1u));
            w_lam[k] = lam;
            w_h[k] = SORTED ? h_in[(long)f * a.nb + base + t] : h_in[(base + t) * a.nf + f];
            w_pos[k] = (int)(base + t);
        }
        if (n == 0) continue;
        any = true;
        __syncthreads();
#pragma unroll 1
        for (int li = 0; li < n; li++) {
            const double lj = w_lam[li], hj = w_h[li];
            const int pos = w_pos[li];
#pragma unroll
            for (int sl = 0; sl < RPT; sl++) {
                if (sl >= rpt) break;
                uint4 ctr = ctr0;
                ctr.x = (uint32_t)pos;
                ctr.w |= W_WIDE | ((uint32_t)sl << 8);
                const double num = (lj > NORMAL_THRESH) ? normal_draw(ctr, a.key, lj) : ptrs64(ctr, a.key, lj, d_status);
                if (!SORTED || pos >= __ldg(q_row + sl * RB)) acc[sl] += num * hj;
            }
        }
    }
    if (!any) return;
#pragma unroll
    for (int i = 0; i < RPT; i++)
        if (i < rpt) part[((long)c * a.nf + f) * a.nr + r0 + (long)i * RB] += acc[i];
}

template <bool SORTED>
__global__ void __launch_bounds__(RB) k_bulk_wide(BulkArgs a, const double *__restrict__ lam_in,
                                                   const double *__restrict__ h_in, const int *__restrict__ qpos,
                                                   double *__restrict__ part, int *d_status) {
    __shared__ WideShared sh;
    wide_block<SORTED>(a, lam_in, h_in, qpos, part, d_status, blockIdx.x, blockIdx.y, blockIdx.z, sh);
}

// the wide pass of the items of a work list, grid-stride over the items
__global__ void __launch_bounds__(RB) k_bulk_wide_multi(const BulkJob *__restrict__ jobs,
                                                        const int4 *__restrict__ items, int n_items) {
    __shared__ WideShared sh;
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const int4 w = items[it];
        const BulkJob &J = jobs[w.x];
        wide_block<true>(J.a, J.lam, J.h, J.q, J.part, J.status, w.y, w.z, w.w, sh);
        __syncthreads();   // the shared lists are rewritten by the next item
    }
}

// ---- 5. background = prefix remainder + chunk partials (fixed order)
__global__ void k_bg_reduce(int nchunk, long nfr, const double *__restrict__ bgp, const double *__restrict__ part,
                            double *__restrict__ out) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nfr) return;
    double acc = bgp ? bgp[idx] : 0.0;
    for (int c = 0; c < nchunk; c++) acc += part[(long)c * nfr + idx];
    out[idx] = acc;
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

// Replay with parameters: thread per (frequency, realization), the reference's loop and operation
// order (cyutils.pyx:1686-1770), round-to-nearest multiply / add / divide.
__global__ void k_loudest_par_replay(long nb, int nf, int nr, int nl, const double *__restrict__ h_s, ParArgs pa,
                                     const double *__restrict__ replay, double *__restrict__ hc2ss,
                                     double *__restrict__ hc2bg, double *__restrict__ bgpar) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)nf * nr) return;
    int f = (int)(idx / nr), r = (int)(idx % nr);
    const double *hf = h_s + (long)f * nb;
    const double *cnt = replay + ((long)r * nf + f) * nb;
    double *ss = hc2ss + idx * nl;
    for (int l = 0; l < nl; l++) {
        ss[l] = 0.0;
        for (int k = 0; k < 4; k++) pa.sspar[(((long)k * nf + f) * nr + r) * nl + l] = 0.0;
    }
    int ll = 0;
    double sum = 0.0;
    double w[NPAR] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (long k = 0; k < nb; k++) {
        double num = cnt[k];
        const double cur = hf[k];
        if (num < 1.0 || cur == 0.0) continue;
        const long bin = pa.order[k];
        while (ll < nl && num > 0.0) {
            ss[ll] = cur;
            for (int q = 0; q < 4; q++) pa.sspar[(((long)q * nf + f) * nr + r) * nl + ll] = bin_param(pa, bin, nf, f, q);
            num = __dsub_rn(num, 1.0);
            ll++;
        }
        const double nc = __dmul_rn(num, cur);
        sum = __dadd_rn(sum, nc);
        for (int q = 0; q < NPAR; q++) w[q] = __dadd_rn(w[q], __dmul_rn(nc, bin_param(pa, bin, nf, f, q)));
    }
    hc2bg[idx] = sum;
    for (int q = 0; q < NPAR; q++) bgpar[(long)q * nf * nr + idx] = __ddiv_rn(w[q], sum);
}

// hc2bg and bgpar of the parameter path: prefix remainder + chunk partials, then the weighted means.
__global__ void k_bg_reduce_par(int nchunk, long nfr, const double *__restrict__ bgp, const double *__restrict__ part,
                                ParArgs pa, double *__restrict__ hc2bg, double *__restrict__ bgpar) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nfr) return;
    double bg = bgp[idx];
    for (int c = 0; c < nchunk; c++) bg += part[(long)c * nfr + idx];
    hc2bg[idx] = bg;
    for (int k = 0; k < NPAR; k++) {
        double w = pa.bgp_par[(long)k * nfr + idx];
        for (int c = 0; c < nchunk; c++) w += pa.part_par[((long)c * NPAR + k) * nfr + idx];
        bgpar[(long)k * nfr + idx] = w / bg;
    }
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

// Waves of resident k_bulk blocks (BULK_BLOCKS_PER_SM per SM) that the chunk count aims for; set by
// hgb_set_bulk_waves.
// A block's cost depends strongly on its frequency (the lowest frequencies hold most of the
// occupied bins), so many short blocks balance the SMs better than a few long ones: on the
// 91x81x101 grid with 40 frequencies and 1000 realizations the kernel takes 33.9 / 31.3 / 29.9 /
// 29.7 / 29.2 / 29.2 ms at 2 / 4 / 6 / 8 / 12 / 16 waves on a GB300.
// Workspace sizes are always computed for HGB_BULK_WAVES_MAX, so a change between a workspace query
// and a launch only leaves part of the workspace unused.
std::atomic<int> g_bulk_waves{12};

int bulk_waves() { return g_bulk_waves.load(std::memory_order_relaxed); }

int choose_nchunk(long nb, int nf, int nr, int waves) {
    long blocks = (long)n_rgroups(nr) * nf;
    long target = (long)hgb::sm_count() * BULK_BLOCKS_PER_SM * waves;
    long nchunk = hgb::ceil_div(target, blocks);
    long maxc = hgb::ceil_div(nb, 8L * RB);
    if (nchunk > maxc) nchunk = maxc;
    if (nchunk < 1) nchunk = 1;
    if (nchunk > 65535) nchunk = 65535;
    return (int)nchunk;
}

struct LoudLayout {
    size_t off_lam, off_h, off_cum, off_seg, off_q, off_bgp, off_part, off_flag, total;
    int nchunk;
};

LoudLayout loud_layout(long nb, int nf, int nr, int mode, int waves) {
    LoudLayout L{};
    L.nchunk = choose_nchunk(nb, nf, nr, waves);
    const long nfr = (long)nf * nr;
    size_t o = 0;
    L.off_lam = o;
    o += align256(sizeof(double) * nb * nf);
    L.off_h = o;
    o += align256(sizeof(double) * nb * nf);
    if (mode == HGB_RNG_PHILOX) {
        L.off_cum = o;
        o += align256(sizeof(double) * (nb + 1) * nf);
        L.off_seg = o;
        o += align256(sizeof(double) * CUM_SEG * nf);
        L.off_q = o;
        o += align256(sizeof(int) * nfr);
        L.off_bgp = o;
        o += align256(sizeof(double) * nfr);
        L.off_part = o;
        o += align256(sizeof(double) * (size_t)L.nchunk * nfr);
        L.off_flag = o;
        o += 256;
    }
    L.total = o;
    return L;
}

BulkArgs bulk_args(long nb, int nf, int nr, int nchunk, uint64_t seed, uint32_t domain, int f_offset = 0) {
    BulkArgs a;
    a.nb = nb;
    a.nf = nf;
    a.nr = nr;
    a.f_offset = f_offset;
    a.nchunk = nchunk;
    a.domain = domain;
    a.key = make_key(seed);
    a.wide_flag = nullptr;
    return a;
}

// Measurement hook: events recorded around the bulk kernel when enabled (per host thread).
thread_local bool g_bulk_timing = false;
thread_local cudaEvent_t g_bulk_ev[2] = {nullptr, nullptr};
thread_local bool g_bulk_recorded = false;

int bulk_event(int k, cudaStream_t st) {
    if (!g_bulk_timing) return HGB_OK;
    cudaError_t err = cudaEventRecord(g_bulk_ev[k], st);
    if (err != cudaSuccess) {
        hgb::set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    if (k == 1) g_bulk_recorded = true;
    return HGB_OK;
}

}  // namespace

extern "C" {

int hgb_bulk_timing(int enable) {
    if (enable && !g_bulk_ev[0]) {
        for (int k = 0; k < 2; k++) {
            cudaError_t err = cudaEventCreate(&g_bulk_ev[k]);
            if (err != cudaSuccess) {
                hgb::set_cuda_error(err);
                return HGB_ERR_CUDA;
            }
        }
    }
    g_bulk_timing = enable != 0;
    g_bulk_recorded = false;
    return HGB_OK;
}

float hgb_bulk_last_ms(void) {
    if (!g_bulk_recorded) return -1.0f;
    float ms = -1.0f;
    if (cudaEventElapsedTime(&ms, g_bulk_ev[0], g_bulk_ev[1]) != cudaSuccess) return -1.0f;
    return ms;
}

size_t hgb_loudest_workspace_bytes(long n_bins, int n_freq, int nreals, int nloud, int mode) {
    (void)nloud;
    if (n_bins <= 0 || n_freq <= 0 || nreals <= 0) return 0;
    return loud_layout(n_bins, n_freq, nreals, mode, HGB_BULK_WAVES_MAX).total;
}

int hgb_loudest_hc_from_sorted(const double *number, const double *h2fdf, long n_bins, int n_freq, int nreals,
                               int nloud, const int32_t *order, int mode, uint64_t seed, const double *replay,
                               double *hc2ss, double *hc2bg, void *workspace, size_t workspace_bytes,
                               int *d_status, void *stream) {
    return hgb_loudest_hc_from_sorted_ex(number, h2fdf, n_bins, n_freq, nreals, nloud, order, mode, seed, replay,
                                         hc2ss, hc2bg, workspace, workspace_bytes, d_status, stream, 0);
}

int hgb_loudest_hc_from_sorted_ex(const double *number, const double *h2fdf, long n_bins, int n_freq, int nreals,
                                  int nloud, const int32_t *order, int mode, uint64_t seed, const double *replay,
                                  double *hc2ss, double *hc2bg, void *workspace, size_t workspace_bytes,
                                  int *d_status, void *stream, int freq_offset) {
    HGB_CHECK_ARG(freq_offset >= 0 && (long)freq_offset + n_freq <= 65535);
    HGB_CHECK_ARG(number && h2fdf && order && hc2bg && n_bins >= 0 && n_freq >= 1 && nreals >= 0 && nloud >= 0);
    HGB_CHECK_ARG(nloud == 0 || hc2ss);
    HGB_CHECK_ARG(nloud <= 255);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || mode == HGB_RNG_REPLAY);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || replay);
    HGB_CHECK_ARG(n_bins < (1L << 31) - 1 && n_freq <= 65535 && nreals <= HGB_MAX_NREALS);
    if (nreals == 0) return HGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (n_bins == 0) {
        if (nloud) cudaMemsetAsync(hc2ss, 0, sizeof(double) * (size_t)n_freq * nreals * nloud, st);
        cudaMemsetAsync(hc2bg, 0, sizeof(double) * (size_t)n_freq * nreals, st);
        return hgb::check_launch();
    }
    if (!workspace || workspace_bytes < hgb_loudest_workspace_bytes(n_bins, n_freq, nreals, nloud, mode))
        return HGB_ERR_WORKSPACE;
    LoudLayout L = loud_layout(n_bins, n_freq, nreals, mode, bulk_waves());
    char *w = (char *)workspace;
    double *lam_s = (double *)(w + L.off_lam);
    double *h_s = (double *)(w + L.off_h);
    const long nfr = (long)n_freq * nreals;
    launch_gather_sorted(number, h2fdf, order, n_bins, n_freq, lam_s, h_s, st, d_status);
    int rc = hgb::check_launch();
    if (rc) return rc;
    if (mode == HGB_RNG_REPLAY) {
        k_loudest_replay<<<(unsigned)hgb::ceil_div(nfr, 128), 128, 0, st>>>(n_bins, n_freq, nreals, nloud, h_s, replay,
                                                                             hc2ss, hc2bg);
        return hgb::check_launch();
    }
    double *cum = (double *)(w + L.off_cum);
    int *q = (int *)(w + L.off_q);
    double *bgp = (double *)(w + L.off_bgp);
    double *part = (double *)(w + L.off_part);
    if ((rc = cumulate(n_bins, n_freq, lam_s, nullptr, (double *)(w + L.off_seg), cum, st))) return rc;
    PrefixArgs pa;
    pa.nb = n_bins;
    pa.nf = n_freq;
    pa.nr = nreals;
    pa.nl = nloud;
    pa.f_offset = freq_offset;
    pa.key = make_key(seed);
    k_loud_prefix<false><<<(unsigned)hgb::ceil_div(nfr, 128), 128, 0, st>>>(pa, ParArgs{}, lam_s, h_s, cum, hc2ss, bgp,
                                                                            q, d_status);
    if ((rc = hgb::check_launch())) return rc;
    BulkArgs a = bulk_args(n_bins, n_freq, nreals, L.nchunk, seed, 0u, freq_offset);
    a.wide_flag = (int *)(w + L.off_flag);
    cudaMemsetAsync(a.wide_flag, 0, sizeof(int), st);
    dim3 grid((unsigned)a.nchunk, (unsigned)n_freq, (unsigned)n_rgroups(nreals));
    if ((rc = bulk_event(0, st))) return rc;
    k_bulk<true, false><<<grid, RB, 0, st>>>(a, ParArgs{}, lam_s, h_s, q, part, d_status);
    if ((rc = hgb::check_launch())) return rc;
    if ((rc = bulk_event(1, st))) return rc;
    k_bulk_wide<true><<<grid, RB, 0, st>>>(a, lam_s, h_s, q, part, d_status);
    if ((rc = hgb::check_launch())) return rc;
    k_bg_reduce<<<(unsigned)hgb::ceil_div(nfr, 256), 256, 0, st>>>(a.nchunk, nfr, bgp, part, hc2bg);
    return hgb::check_launch();
}

size_t hgb_loudest_batch_workspace_bytes(const hgb_loudest_sample *samples, int n_samples, int n_freq) {
    if (!samples || n_samples <= 0 || n_freq <= 0) return 0;
    size_t items = 0;
    for (int i = 0; i < n_samples; i++) {
        const hgb_loudest_sample &S = samples[i];
        if (S.n_bins <= 0 || S.nreals <= 0) continue;
        items += (size_t)choose_nchunk(S.n_bins, n_freq, S.nreals, HGB_BULK_WAVES_MAX) * n_freq * n_rgroups(S.nreals);
    }
    return align256(sizeof(BulkJob) * n_samples) + align256(sizeof(int) * n_samples) + align256(sizeof(int4) * items) +
           256;
}

int hgb_loudest_hc_batch(const hgb_loudest_sample *samples, int n_samples, int n_freq, int nloud, int blocks_per_sm,
                         void *workspace, size_t workspace_bytes, void *stream) {
    HGB_CHECK_ARG(samples && n_samples >= 0 && n_freq >= 1 && n_freq <= 65535 && nloud >= 0 && nloud <= 255);
    HGB_CHECK_ARG(blocks_per_sm >= 0 && blocks_per_sm <= BULK_BLOCKS_PER_SM);
    for (int i = 0; i < n_samples; i++) {
        const hgb_loudest_sample &S = samples[i];
        HGB_CHECK_ARG(S.number && S.h2fdf && S.order && S.hc2bg && (nloud == 0 || S.hc2ss));
        HGB_CHECK_ARG(S.n_bins >= 0 && S.n_bins < (1L << 31) - 1 && S.nreals >= 0 && S.nreals <= HGB_MAX_NREALS);
        if (S.n_bins > 0 && S.nreals > 0 &&
            (!S.workspace ||
             S.workspace_bytes < hgb_loudest_workspace_bytes(S.n_bins, n_freq, S.nreals, nloud, HGB_RNG_PHILOX)))
            return HGB_ERR_WORKSPACE;
    }
    if (n_samples == 0) return HGB_OK;
    if (!workspace || workspace_bytes < hgb_loudest_batch_workspace_bytes(samples, n_samples, n_freq))
        return HGB_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    const int waves = bulk_waves();
    char *w = (char *)workspace;
    BulkJob *d_jobs = (BulkJob *)w;
    w += align256(sizeof(BulkJob) * n_samples);
    int *d_flags = (int *)w;
    w += align256(sizeof(int) * n_samples);
    int4 *d_items = (int4 *)w;
    std::vector<BulkJob> jobs;
    std::vector<int> job_sample;
    std::vector<int> nchunk;
    int rc;
    // per sample: the gather into loudest-first order, the exact scan and the loudest slots, as
    // hgb_loudest_hc_from_sorted does
    for (int i = 0; i < n_samples; i++) {
        const hgb_loudest_sample &S = samples[i];
        if (S.nreals == 0) continue;
        if (S.n_bins == 0) {
            if (nloud) cudaMemsetAsync(S.hc2ss, 0, sizeof(double) * (size_t)n_freq * S.nreals * nloud, st);
            cudaMemsetAsync(S.hc2bg, 0, sizeof(double) * (size_t)n_freq * S.nreals, st);
            if ((rc = hgb::check_launch())) return rc;
            continue;
        }
        const LoudLayout L = loud_layout(S.n_bins, n_freq, S.nreals, HGB_RNG_PHILOX, waves);
        char *sw = (char *)S.workspace;
        double *lam_s = (double *)(sw + L.off_lam);
        double *h_s = (double *)(sw + L.off_h);
        launch_gather_sorted(S.number, S.h2fdf, S.order, S.n_bins, n_freq, lam_s, h_s, st, S.d_status);
        if ((rc = hgb::check_launch())) return rc;
        double *cum = (double *)(sw + L.off_cum);
        int *q = (int *)(sw + L.off_q);
        double *bgp = (double *)(sw + L.off_bgp);
        if ((rc = cumulate(S.n_bins, n_freq, lam_s, nullptr, (double *)(sw + L.off_seg), cum, st))) return rc;
        PrefixArgs pa;
        pa.nb = S.n_bins;
        pa.nf = n_freq;
        pa.nr = S.nreals;
        pa.nl = nloud;
        pa.f_offset = 0;
        pa.key = make_key(S.seed);
        const long nfr = (long)n_freq * S.nreals;
        k_loud_prefix<false><<<(unsigned)hgb::ceil_div(nfr, 128), 128, 0, st>>>(pa, ParArgs{}, lam_s, h_s, cum,
                                                                                S.hc2ss, bgp, q, S.d_status);
        if ((rc = hgb::check_launch())) return rc;
        BulkJob J;
        J.a = bulk_args(S.n_bins, n_freq, S.nreals, L.nchunk, S.seed, 0u, 0);
        J.a.wide_flag = d_flags + jobs.size();
        J.lam = lam_s;
        J.h = h_s;
        J.q = q;
        J.part = (double *)(sw + L.off_part);
        J.status = S.d_status;
        jobs.push_back(J);
        job_sample.push_back(i);
        nchunk.push_back(L.nchunk);
    }
    const int nj = (int)jobs.size();
    if (nj == 0) return HGB_OK;
    // the work list: frequency by frequency (the low frequencies hold most occupied bins, so the
    // costly items come first), within a frequency the samples with the most bins per chunk first
    std::vector<int> by_size(nj);
    for (int j = 0; j < nj; j++) by_size[j] = j;
    std::sort(by_size.begin(), by_size.end(), [&](int x, int y) {
        const long bx = jobs[x].a.nb / nchunk[x], byy = jobs[y].a.nb / nchunk[y];
        return bx != byy ? bx > byy : x < y;
    });
    std::vector<int4> items;
    for (int f = 0; f < n_freq; f++)
        for (int j : by_size)
            for (int rg = 0; rg < n_rgroups(jobs[j].a.nr); rg++)
                for (int c = 0; c < nchunk[j]; c++) items.push_back(make_int4(j, c, f, rg));
    const int n_items = (int)items.size();
    int *d_next = (int *)(w + align256(sizeof(int4) * items.size()));
    // pageable host sources: each copy is staged before the call returns, so the vectors may go
    cudaError_t err = cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(BulkJob) * nj, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaMemsetAsync(d_flags, 0, sizeof(int) * nj, st);
    if (err == cudaSuccess) err = cudaMemsetAsync(d_next, 0, sizeof(int), st);
    if (err != cudaSuccess) {
        hgb::set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    if ((rc = bulk_event(0, st))) return rc;
    if (blocks_per_sm > 0) {
        const long grid = std::min((long)n_items, (long)hgb::sm_count() * blocks_per_sm);
        k_bulk_multi<<<(unsigned)grid, RB, 0, st>>>(d_jobs, d_items, n_items, d_next);
    } else {
        k_bulk_multi<<<(unsigned)n_items, RB, 0, st>>>(d_jobs, d_items, n_items, nullptr);
    }
    if ((rc = hgb::check_launch())) return rc;
    if ((rc = bulk_event(1, st))) return rc;
    const long wgrid = std::min((long)n_items, (long)hgb::sm_count() * 8);
    k_bulk_wide_multi<<<(unsigned)wgrid, RB, 0, st>>>(d_jobs, d_items, n_items);
    if ((rc = hgb::check_launch())) return rc;
    for (int j = 0; j < nj; j++) {
        const hgb_loudest_sample &S = samples[job_sample[j]];
        const LoudLayout L = loud_layout(S.n_bins, n_freq, S.nreals, HGB_RNG_PHILOX, waves);
        const long nfr = (long)n_freq * S.nreals;
        char *sw = (char *)S.workspace;
        k_bg_reduce<<<(unsigned)hgb::ceil_div(nfr, 256), 256, 0, st>>>(L.nchunk, nfr, (double *)(sw + L.off_bgp),
                                                                       (double *)(sw + L.off_part), S.hc2bg);
        if ((rc = hgb::check_launch())) return rc;
    }
    return HGB_OK;
}

size_t hgb_loudest_par_workspace_bytes(long n_bins, int n_freq, int nreals, int nloud, int mode) {
    (void)nloud;
    if (n_bins <= 0 || n_freq <= 0 || nreals <= 0) return 0;
    LoudLayout L = loud_layout(n_bins, n_freq, nreals, mode, HGB_BULK_WAVES_MAX);
    size_t o = L.total;
    if (mode == HGB_RNG_PHILOX) {
        const size_t nfr = (size_t)n_freq * nreals;
        o += align256(sizeof(double) * NPAR * nfr);                    // prefix weighted sums
        o += align256(sizeof(double) * NPAR * (size_t)L.nchunk * nfr);  // chunk weighted sums
    }
    return o;
}

int hgb_loudest_hc_and_par_from_sorted(const double *number, const double *h2fdf, int n_m, int n_q, int n_z,
                                       int n_freq, int nreals, int nloud, const int32_t *order, int mode,
                                       uint64_t seed, const double *replay, const double *mt_cent,
                                       const double *mr_cent, const double *rz_cent, const double *redz_mid,
                                       const double *dcom, const double *sepa, const double *angs,
                                       const int *scale_log2, double *hc2ss, double *hc2bg, double *sspar,
                                       double *bgpar, void *workspace, size_t workspace_bytes, int *d_status,
                                       void *stream) {
    HGB_CHECK_ARG(number && h2fdf && order && hc2bg && bgpar && n_m >= 1 && n_q >= 1 && n_z >= 1);
    HGB_CHECK_ARG(n_freq >= 1 && nreals >= 0 && nloud >= 0 && nloud <= 255);
    HGB_CHECK_ARG(nloud == 0 || (hc2ss && sspar));
    HGB_CHECK_ARG(mt_cent && mr_cent && rz_cent && redz_mid && dcom && sepa && angs);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || mode == HGB_RNG_REPLAY);
    HGB_CHECK_ARG(mode == HGB_RNG_REPLAY ? replay != nullptr : scale_log2 != nullptr);
    const long n_bins = (long)n_m * n_q * n_z;
    HGB_CHECK_ARG(n_bins < (1L << 31) - 1 && n_freq <= 65535 && nreals <= HGB_MAX_NREALS);
    if (nreals == 0) return HGB_OK;
    const size_t need = hgb_loudest_par_workspace_bytes(n_bins, n_freq, nreals, nloud, mode);
    if (!workspace || workspace_bytes < need) return HGB_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    LoudLayout L = loud_layout(n_bins, n_freq, nreals, mode, bulk_waves());
    char *w = (char *)workspace;
    double *lam_s = (double *)(w + L.off_lam);
    double *h_s = (double *)(w + L.off_h);
    const long nfr = (long)n_freq * nreals;
    ParArgs pa{};
    pa.order = order;
    pa.mt = mt_cent;
    pa.mr = mr_cent;
    pa.rz = rz_cent;
    pa.grid[0] = redz_mid;
    pa.grid[1] = dcom;
    pa.grid[2] = sepa;
    pa.grid[3] = angs;
    pa.scale_log2 = scale_log2;
    pa.nq = n_q;
    pa.nz = n_z;
    pa.sspar = sspar;
    launch_gather_sorted(number, h2fdf, order, n_bins, n_freq, lam_s, h_s, st, d_status);
    int rc = hgb::check_launch();
    if (rc) return rc;
    if (mode == HGB_RNG_REPLAY) {
        k_loudest_par_replay<<<(unsigned)hgb::ceil_div(nfr, 128), 128, 0, st>>>(n_bins, n_freq, nreals, nloud, h_s, pa,
                                                                                 replay, hc2ss, hc2bg, bgpar);
        return hgb::check_launch();
    }
    double *cum = (double *)(w + L.off_cum);
    int *q = (int *)(w + L.off_q);
    double *bgp = (double *)(w + L.off_bgp);
    double *part = (double *)(w + L.off_part);
    pa.bgp_par = (double *)(w + L.total);
    pa.part_par = (double *)(w + L.total + align256(sizeof(double) * NPAR * nfr));
    if ((rc = cumulate(n_bins, n_freq, lam_s, h_s, (double *)(w + L.off_seg), cum, st))) return rc;
    PrefixArgs pf;
    pf.nb = n_bins;
    pf.nf = n_freq;
    pf.nr = nreals;
    pf.nl = nloud;
    pf.f_offset = 0;
    pf.key = make_key(seed);
    k_loud_prefix<true><<<(unsigned)hgb::ceil_div(nfr, 128), 128, 0, st>>>(pf, pa, lam_s, h_s, cum, hc2ss, bgp, q,
                                                                           d_status);
    if ((rc = hgb::check_launch())) return rc;
    BulkArgs a = bulk_args(n_bins, n_freq, nreals, L.nchunk, seed, 0u);
    a.wide_flag = (int *)(w + L.off_flag);   // unused: the parameter kernel draws its wide bins itself
    dim3 grid((unsigned)a.nchunk, (unsigned)n_freq, (unsigned)n_rgroups(nreals));
    cudaError_t err = cudaFuncSetAttribute(k_bulk<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)PAR_SMEM);
    if (err != cudaSuccess) {
        hgb::set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    k_bulk<true, true><<<grid, RB, PAR_SMEM, st>>>(a, pa, lam_s, h_s, q, part, d_status);
    if ((rc = hgb::check_launch())) return rc;
    k_bg_reduce_par<<<(unsigned)hgb::ceil_div(nfr, 256), 256, 0, st>>>(a.nchunk, nfr, bgp, part, pa, hc2bg, bgpar);
    return hgb::check_launch();
}

int hgb_set_bulk_waves(int waves) {
    HGB_CHECK_ARG(waves >= 1 && waves <= HGB_BULK_WAVES_MAX);
    g_bulk_waves.store(waves, std::memory_order_relaxed);
    return HGB_OK;
}

int hgb_get_bulk_waves(void) { return bulk_waves(); }

size_t hgb_sam_poisson_gwb_workspace_bytes(long n_bins, int n_freq, int nreals) {
    if (n_bins <= 0 || n_freq <= 0 || nreals <= 0) return 0;
    long nchunk = choose_nchunk(n_bins, n_freq, nreals, HGB_BULK_WAVES_MAX);
    return align256(sizeof(double) * (size_t)nchunk * n_freq * nreals) + 256;   // partials, wide-bin flag
}

int hgb_sam_poisson_gwb(const double *number, const double *hc2, long n_bins, int n_freq, int nreals, int mode,
                        uint64_t seed, const double *replay, double *gwb, void *workspace, size_t workspace_bytes,
                        int *d_status, void *stream) {
    HGB_CHECK_ARG(number && hc2 && gwb && n_bins >= 0 && n_freq >= 1 && nreals >= 0);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || mode == HGB_RNG_REPLAY);
    HGB_CHECK_ARG(mode == HGB_RNG_PHILOX || replay);
    HGB_CHECK_ARG(n_bins < (1L << 31) - 1 && n_freq <= 65535 && nreals <= HGB_MAX_NREALS);
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
    BulkArgs a = bulk_args(n_bins, n_freq, nreals, choose_nchunk(n_bins, n_freq, nreals, bulk_waves()), seed,
                          DOMAIN_GWB);
    a.wide_flag = (int *)((char *)workspace + align256(sizeof(double) * (size_t)a.nchunk * n_freq * nreals));
    cudaMemsetAsync(a.wide_flag, 0, sizeof(int), st);
    dim3 grid((unsigned)a.nchunk, (unsigned)n_freq, (unsigned)n_rgroups(nreals));
    k_bulk<false, false><<<grid, RB, 0, st>>>(a, ParArgs{}, number, hc2, nullptr, (double *)workspace, d_status);
    int rc = hgb::check_launch();
    if (rc) return rc;
    k_bulk_wide<false><<<grid, RB, 0, st>>>(a, number, hc2, nullptr, (double *)workspace, d_status);
    if ((rc = hgb::check_launch())) return rc;
    long nfr = (long)n_freq * nreals;
    k_bg_reduce<<<(unsigned)hgb::ceil_div(nfr, 256), 256, 0, st>>>(a.nchunk, nfr, nullptr, (double *)workspace, gwb);
    return hgb::check_launch();
}

}  // extern "C"
