// Loudest-first bin order at the first frequency (holodeck/single_sources.py:89:
// argsort(-h2fdf[..., 0])): a stable least-significant-digit radix sort of (key, bin) pairs.
//
// Keys: the IEEE bits of h2fdf[b, 0] mapped to unsigned 64-bit integers whose ascending order is the
// descending order of the doubles.  -0.0 is taken as +0.0 and every NaN as the largest key, so zeros
// of either sign tie and NaNs come last, as they do in numpy's argsort of the negated values.
// Eight passes of 8 bits, least significant first; every pass is
//   k_sort_count    per-block counts of the 256 digits over a tile of SORT_TILE keys, [digit][block],
//   k_sort_scan     one block per digit: exclusive scan of its per-block counts, and the digit total,
//   k_sort_scatter  the tile's keys moved to their digit's next free slots in input order: each round
//                   of 256 keys is ranked with warp match counts and per-warp digit totals in shared
//                   memory, so equal digits keep their input order (the sort is stable).
// Stability and ascending bin indices in the input make equal keys come out in ascending bin order.
// Buffers ping-pong so that the eighth pass writes the indices into `order`: the key gather writes
// the initial indices there, even passes move (K0, order) -> (K1, idx), odd passes back.
#include "hgb_common.cuh"

namespace {

constexpr int SORT_THREADS = 256;   // one thread per digit value in the scatter's bookkeeping
constexpr int SORT_ITEMS = 8;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;   // keys per block
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int SORT_PASSES = 8;
constexpr int SCAN_THREADS = 1024;

__device__ __forceinline__ unsigned long long desc_key(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned long long mag = b & 0x7fffffffffffffffull;
    if (mag > 0x7ff0000000000000ull) return ~0ull;   // NaN
    if (mag == 0ull) b = 0ull;                        // -0.0
    const unsigned long long asc = (b >> 63) ? ~b : (b | 0x8000000000000000ull);
    return ~asc;
}

__device__ __forceinline__ unsigned digit_of(unsigned long long k, int shift) {
    return (unsigned)(k >> shift) & 255u;
}

__global__ void k_sort_keys(const double *__restrict__ h2fdf, long nb, int nf, unsigned long long *__restrict__ keys,
                            int32_t *__restrict__ idx) {
    const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    keys[b] = desc_key(h2fdf[b * nf]);
    idx[b] = (int32_t)b;
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_count(const unsigned long long *__restrict__ keys, long n,
                                                            int shift, unsigned int *__restrict__ counts) {
    __shared__ unsigned int hist[256];
    const int t = threadIdx.x, lane = t & 31;
    hist[t] = 0u;
    __syncthreads();
    const long base = (long)blockIdx.x * SORT_TILE;
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; j++) {
        const long p = base + (long)j * SORT_THREADS + t;
        const bool valid = p < n;
        const int d = valid ? (int)digit_of(keys[p], shift) : 256 + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);   // one shared add per digit and warp
        if (valid && (peers & lt) == 0u) atomicAdd(&hist[d], (unsigned)__popc(peers));
    }
    __syncthreads();
    counts[(long)t * gridDim.x + blockIdx.x] = hist[t];
}

// Inclusive scan of one value per thread over a block of SCAN_THREADS; `warp_sums` holds 32 entries.
__device__ __forceinline__ unsigned block_inclusive_scan(unsigned v, unsigned *warp_sums, unsigned *total) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned s = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += u;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    if (warp > 0) v += warp_sums[warp - 1];
    *total = warp_sums[31];
    __syncthreads();   // warp_sums is rewritten by the next call
    return v;
}

// Block d: exclusive scan of counts[d][0 .. nblk) in place, and totals[d] = the digit's key count.
__global__ void __launch_bounds__(SCAN_THREADS) k_sort_scan(unsigned int *__restrict__ counts, long nblk,
                                                            unsigned int *__restrict__ totals) {
    __shared__ unsigned warp_sums[32];
    unsigned int *row = counts + (long)blockIdx.x * nblk;
    unsigned carry = 0u;
    for (long b0 = 0; b0 < nblk; b0 += SCAN_THREADS) {
        const long b = b0 + threadIdx.x;
        const unsigned v = (b < nblk) ? row[b] : 0u;
        unsigned tot;
        const unsigned inc = block_inclusive_scan(v, warp_sums, &tot);
        if (b < nblk) row[b] = carry + inc - v;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_scatter(const unsigned long long *__restrict__ kin,
                                                              const int32_t *__restrict__ iin,
                                                              unsigned long long *__restrict__ kout,
                                                              int32_t *__restrict__ iout, long n, int shift,
                                                              const unsigned int *__restrict__ offsets,
                                                              const unsigned int *__restrict__ totals) {
    __shared__ unsigned int base[256];              // next free slot of each digit
    __shared__ unsigned int cnt[SORT_WARPS][256];   // this round's keys per (warp, digit)
    __shared__ unsigned int off[SORT_WARPS][256];   // this round's first slot per (warp, digit)
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    {   // base = keys of smaller digits (exclusive scan of the totals) + this block's offset in digit t
        const unsigned tot = totals[t];
        base[t] = tot;
        __syncthreads();
        unsigned s = tot;
        for (int o = 1; o < 256; o <<= 1) {
            const unsigned u = (t >= o) ? base[t - o] : 0u;
            __syncthreads();
            s += u;
            base[t] = s;
            __syncthreads();
        }
        base[t] = s - tot + offsets[(long)t * gridDim.x + blockIdx.x];
    }
#pragma unroll
    for (int w = 0; w < SORT_WARPS; w++) cnt[w][t] = 0u;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    const long tile = (long)blockIdx.x * SORT_TILE;
    for (int j = 0; j < SORT_ITEMS; j++) {
        const long p = tile + (long)j * SORT_THREADS + t;   // rounds, warps and lanes in input order
        const bool valid = p < n;
        unsigned long long k = 0ull;
        int32_t v = 0;
        int d = 256 + lane;   // out-of-range lanes form groups of their own
        if (valid) {
            k = kin[p];
            v = iin[p];
            d = (int)digit_of(k, shift);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned rank = (unsigned)__popc(peers & lt);
        if (valid && rank == 0u) cnt[warp][d] = (unsigned)__popc(peers);
        __syncthreads();
        {   // thread t: digit t over the warps, in warp order
            unsigned int run = base[t];
#pragma unroll
            for (int w = 0; w < SORT_WARPS; w++) {
                off[w][t] = run;
                run += cnt[w][t];
                cnt[w][t] = 0u;
            }
            base[t] = run;
        }
        __syncthreads();
        if (valid) {
            const unsigned int dst = off[warp][d] + rank;
            kout[dst] = k;
            iout[dst] = v;
        }
        // off is next written after the next round's first barrier, which every reader here passes first
    }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

long sort_blocks(long n) { return hgb::ceil_div(n, SORT_TILE); }

}  // namespace

namespace hgb {

size_t argsort_f0_scratch_bytes(long n_bins) {
    if (n_bins <= 0) return 0;
    return 2 * align256(sizeof(unsigned long long) * n_bins) + align256(sizeof(int32_t) * n_bins) +
           align256(sizeof(unsigned int) * 256 * (size_t)sort_blocks(n_bins)) + align256(sizeof(unsigned int) * 256);
}

int argsort_f0_desc_into(const double *h2fdf, long n_bins, int n_freq, int32_t *order, void *scratch,
                         cudaStream_t st) {
    char *w = (char *)scratch;
    unsigned long long *k0 = (unsigned long long *)w;
    w += align256(sizeof(unsigned long long) * n_bins);
    unsigned long long *k1 = (unsigned long long *)w;
    w += align256(sizeof(unsigned long long) * n_bins);
    int32_t *idx = (int32_t *)w;
    w += align256(sizeof(int32_t) * n_bins);
    const long nblk = sort_blocks(n_bins);
    unsigned int *counts = (unsigned int *)w;
    w += align256(sizeof(unsigned int) * 256 * (size_t)nblk);
    unsigned int *totals = (unsigned int *)w;
    k_sort_keys<<<(unsigned)ceil_div(n_bins, 256), 256, 0, st>>>(h2fdf, n_bins, n_freq, k0, order);
    int rc = check_launch();
    if (rc) return rc;
    for (int pass = 0; pass < SORT_PASSES; pass++) {
        const int shift = 8 * pass;
        const bool even = (pass & 1) == 0;
        const unsigned long long *kin = even ? k0 : k1;
        unsigned long long *kout = even ? k1 : k0;
        const int32_t *iin = even ? order : idx;
        int32_t *iout = even ? idx : order;
        k_sort_count<<<(unsigned)nblk, SORT_THREADS, 0, st>>>(kin, n_bins, shift, counts);
        k_sort_scan<<<256, SCAN_THREADS, 0, st>>>(counts, nblk, totals);
        k_sort_scatter<<<(unsigned)nblk, SORT_THREADS, 0, st>>>(kin, iin, kout, iout, n_bins, shift, counts, totals);
        if ((rc = check_launch())) return rc;
    }
    return HGB_OK;
}

}  // namespace hgb

extern "C" {

size_t hgb_sort_workspace_bytes(long n_bins) { return hgb::argsort_f0_scratch_bytes(n_bins); }

int hgb_argsort_f0_desc(const double *h2fdf, long n_bins, int n_freq, int32_t *order, void *workspace,
                        size_t workspace_bytes, void *stream) {
    HGB_CHECK_ARG(h2fdf && order && n_bins >= 0 && n_bins < (1L << 31) && n_freq >= 1);
    if (n_bins == 0) return HGB_OK;
    if (!workspace || workspace_bytes < hgb_sort_workspace_bytes(n_bins)) return HGB_ERR_WORKSPACE;
    return hgb::argsort_f0_desc_into(h2fdf, n_bins, n_freq, order, workspace, (cudaStream_t)stream);
}

}  // extern "C"
