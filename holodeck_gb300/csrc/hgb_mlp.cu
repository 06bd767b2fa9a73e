// Emulator MLP: forward, backward and AdamW for an ensemble of small multilayer perceptrons that map
// library parameters to per-frequency strain statistics.  No reference counterpart (the reference's
// emulators are Gaussian processes, holodeck/gps/); the training data are libraries the GPU SAM
// itself writes.
//
// Network: E members, each K_0 (inputs, padded to 16) -> N_0 -> ... -> N_{L-1} (outputs), SiLU after
// every layer but the last.  Weights bf16, row-major [N_l][K_l]; biases and master weights fp32.
// Activations between layers are bf16, pre-activations and outputs fp32, and every product is
// accumulated in fp32.
//
// All three contractions (forward Y = X W^T, input gradient dX = dZ W, weight gradient
// dW = dZ^T X) run on the tensor cores the same way: a CTA of 128 threads owns a 128-row output tile
// of NT columns in tensor memory (tcgen05.alloc, fp32 accumulators), stages the operands in shared
// memory in the canonical no-swizzle K-major layout (8 x 16-byte core matrices), one elected thread
// issues tcgen05.mma (kind::f16, bf16 x bf16 -> fp32, M = 128, K = 16 per instruction) and commits
// them to an mbarrier, and the epilogue reads the accumulator back with tcgen05.ld (one TMEM lane per
// output row) and fuses bias, activation or the activation's derivative.
//   * Forward (k_mlp_fwd_tma): both operands are row-major tiles, staged by the tensor memory
//     accelerator (cp.async.bulk.tensor, one box of 8 columns per K-group) against an mbarrier;
//     the whole reduction axis (<= 256) at once, output columns split 64 per CTA, so a layer is one
//     copy / MMA / read-back round trip on (row tiles x column tiles x members) CTAs.
//   * Input and weight gradients (k_mlp_gemm<DxOp / DwOp>): one operand is read transposed (a column
//     gather of a row-major buffer), so the threads stage both operands through registers; the input
//     gradient stages the whole reduction axis with columns split 64 per CTA, the weight gradient
//     keeps all columns in one CTA and reduces one 128-row batch split per CTA.
// Every wait is bounded: on expiry the kernel flags HGB_STATUS_ITERATION_LIMIT, frees its tensor
// memory and returns.
//
// Dynamic shared memory per CTA is 100 KB, so at most two CTAs share an SM and their allocations
// (at most 256 columns each) always fit the SM's 512 TMEM columns (an allocation never waits).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cooperative_groups.h>

#include <atomic>
#include <mutex>

#include "hgb_common.cuh"

namespace cg = cooperative_groups;

namespace {

typedef __nv_bfloat16 bf16;

constexpr int TM = 128;            // output rows per CTA (tcgen05 M)
constexpr int NMAX = 256;          // widest layer (tcgen05 N limit for M = 128)
constexpr int THREADS = 128;
constexpr int SMEM_DYN = 100 * 1024;       // holds both staged slices; caps residency at two CTAs per SM
constexpr uint64_t WAIT_NS = 1000000000ull;   // a wait for the tensor core gives up after 1 s
constexpr int WIDTH = 256;                 // row stride (elements) of the hidden activation buffers

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of a staged slice (k < KC) in the canonical layout
template <int KC>
__device__ __forceinline__ int slice_off(int r, int k) {
    return (((r >> 3) * (KC / 8) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

// shared-memory matrix descriptor: start address, leading byte offset `lbo` (next core matrix along
// K), stride byte offset `sbo` (next 8-row group), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// non-blocking test of the phase with the given parity
__device__ __forceinline__ bool mbar_test(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for the phase with the given parity to complete, for at most WAIT_NS
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    if (mbar_test(mbar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_test(mbar, parity))
        if (global_ns() - t0 > WAIT_NS) return false;
    return true;
}

// 16 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigmoidf_(z); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = sigmoidf_(z);
    return s * (1.0f + z * (1.0f - s));
}

union Pack8 {
    uint4 u;
    bf16 h[8];
};

// ---- epilogues of the three contractions and the gradients' operand loaders -------------------------
// A loader: 8 consecutive reduction entries of output row r; B loader: the same for output column n.
// Both return zeros outside the operands.

struct FwdOp {   // epilogue of the forward: Y[b][n] = act(acc + bias[n]) (operands staged by TMA)
    const bf16 *x;
    long x_es;
    int ldx;
    const bf16 *w;
    long w_es;
    const float *bias;
    long b_es;
    int K, N, batch, act;
    float *pre;        // fp32 pre-activations [b][ldp] (hidden layers; may be null)
    long pre_es;
    bf16 *y;           // bf16 activations [b][ldy] (hidden layers)
    long y_es;
    float *out;        // fp32 outputs [b][N] (last layer)
    long out_es;
    int ldp, ldy;

    __device__ void store(int e, int row, int n0, const float (&v)[16]) const {
        if (row >= batch || n0 >= N) return;
        const float *bb = bias + e * b_es + n0;
        if (act) {
            Pack8 p0, p1;
            float z[16];
#pragma unroll
            for (int i = 0; i < 16; i++) z[i] = v[i] + bb[i];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                p0.h[i] = __float2bfloat16_rn(silu(z[i]));
                p1.h[i] = __float2bfloat16_rn(silu(z[i + 8]));
            }
            uint4 *yd = (uint4 *)(y + e * y_es + (long)row * ldy + n0);
            yd[0] = p0.u;
            yd[1] = p1.u;
            if (pre) {
                float4 *pd = (float4 *)(pre + e * pre_es + (long)row * ldp + n0);
#pragma unroll
                for (int i = 0; i < 4; i++) pd[i] = make_float4(z[4 * i], z[4 * i + 1], z[4 * i + 2], z[4 * i + 3]);
            }
        } else {
            float4 *od = (float4 *)(out + e * out_es + (long)row * N + n0);
#pragma unroll
            for (int i = 0; i < 4; i++)
                od[i] = make_float4(v[4 * i] + bb[4 * i], v[4 * i + 1] + bb[4 * i + 1], v[4 * i + 2] + bb[4 * i + 2],
                                    v[4 * i + 3] + bb[4 * i + 3]);
        }
    }
};

struct DxOp {   // dZprev[b][k] = (sum_n dZ[b][n] W[n][k]) * silu'(Zprev[b][k])
    static constexpr int KC = 256, NT = 64;
    static constexpr bool COL_TILED = true;
    const bf16 *dz;    // [b][WIDTH], reduction over its first N columns
    long dz_es;
    const bf16 *w;     // [N][K]
    long w_es;
    const float *pre;  // Zprev [b][WIDTH]
    long pre_es;
    bf16 *dzp;         // dZprev [b][WIDTH]
    long dzp_es;
    int K, N, batch;

    __device__ int red() const { return N; }
    __host__ __device__ int ncols() const { return K; }
    __device__ uint4 load_a(int e, int row, int n) const {
        if (row >= batch || n >= N) return make_uint4(0, 0, 0, 0);
        return *(const uint4 *)(dz + e * dz_es + (long)row * WIDTH + n);
    }
    __device__ uint4 load_b(int e, int k, int n) const {
        Pack8 p;
        const bf16 *wp = w + e * w_es + k;
#pragma unroll
        for (int j = 0; j < 8; j++)
            p.h[j] = (k < K && n + j < N) ? wp[(long)(n + j) * K] : __float2bfloat16_rn(0.0f);
        return p.u;
    }
    __device__ void store(int e, int row, int k0, const float (&v)[16]) const {
        if (row >= batch || k0 >= K) return;
        const float *zp = pre + e * pre_es + (long)row * WIDTH + k0;
        Pack8 p0, p1;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            p0.h[i] = __float2bfloat16_rn(v[i] * silu_grad(zp[i]));
            p1.h[i] = __float2bfloat16_rn(v[i + 8] * silu_grad(zp[i + 8]));
        }
        uint4 *d = (uint4 *)(dzp + e * dzp_es + (long)row * WIDTH + k0);
        d[0] = p0.u;
        d[1] = p1.u;
    }
};

struct DwOp {   // part[s][n][k] = sum over this split's rows b of dZ[b][n] X[b][k]
    static constexpr int KC = HGB_MLP_SPLIT_ROWS, NT = NMAX;
    static constexpr bool COL_TILED = false;   // blockIdx.y is the batch split
    const bf16 *dz;    // [b][WIDTH]
    long dz_es;
    const bf16 *x;     // layer input [b][ldx]
    long x_es;
    int ldx;
    float *part;       // [E][S][N][K]
    int K, N, batch, rows_per_split, nsplit;

    __device__ int red() const { return rows_per_split; }
    __host__ __device__ int ncols() const { return K; }
    __device__ uint4 load_a(int e, int n, int r) const {   // r: row offset inside the split
        Pack8 p;
        const int b0 = blockIdx.y * rows_per_split + r;
        const bf16 *d = dz + e * dz_es + n;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int b = b0 + j;
            p.h[j] = (n < N && r + j < rows_per_split && b < batch) ? d[(long)b * WIDTH] : __float2bfloat16_rn(0.0f);
        }
        return p.u;
    }
    __device__ uint4 load_b(int e, int k, int r) const {
        Pack8 p;
        const int b0 = blockIdx.y * rows_per_split + r;
        const bf16 *xp = x + e * x_es + k;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int b = b0 + j;
            p.h[j] = (k < K && r + j < rows_per_split && b < batch) ? xp[(long)b * ldx] : __float2bfloat16_rn(0.0f);
        }
        return p.u;
    }
    __device__ void store(int e, int n, int k0, const float (&v)[16]) const {
        if (n >= N || k0 >= K) return;
        float4 *d = (float4 *)(part + (((long)e * nsplit + blockIdx.y) * N + n) * K + k0);
#pragma unroll
        for (int i = 0; i < 4; i++) d[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    }
};

template <int N>
__host__ __device__ constexpr int tmem_cols() { return N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256; }

// One 128 x NT output tile (blockIdx.x: row tile, blockIdx.y: column tile or batch split,
// blockIdx.z: ensemble member).
template <class Op>
__global__ void __launch_bounds__(THREADS) k_mlp_gemm(Op op, int *status) {
    constexpr int KC = Op::KC, NT = Op::NT, COLS = tmem_cols<NT>();
    constexpr int SMEM_A = TM * KC * 2;
    static_assert(SMEM_A + NT * KC * 2 <= SMEM_DYN, "staged slices must fit the dynamic shared memory");
    static_assert(KC % 16 == 0 && NT % 16 == 0 && NT <= NMAX, "tile shape");
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    uint8_t *sa = smem;
    uint8_t *sb = smem + SMEM_A;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int e = blockIdx.z;
    const int row0 = blockIdx.x * TM;
    const int col0 = Op::COL_TILED ? (int)blockIdx.y * NT : 0;
    const int ncols = min(NT, op.ncols() - col0), red = op.red();
    const int npad = (ncols + 15) & ~15;
    const uint32_t mb = smem_u32(&mbar);

    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), COLS);
    if (threadIdx.x == 0) mbar_init(mb, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = idesc_bf16(TM, npad);

    bool ok = true;
    uint32_t parity = 0;
    const int nslices = (red + KC - 1) / KC;
    for (int c = 0; c < nslices; c++) {
        const int k0 = c * KC;
        const int kact = min(KC, ((red - k0) + 15) & ~15);   // staged (and multiplied) part of the slice
        for (int v = threadIdx.x; v < TM * (kact / 8); v += THREADS) {
            const int r = v % TM, kg = v / TM;
            *(uint4 *)(sa + slice_off<KC>(r, kg * 8)) = op.load_a(e, row0 + r, k0 + kg * 8);
        }
        for (int v = threadIdx.x; v < npad * (kact / 8); v += THREADS) {
            const int n = v % npad, kg = v / npad;
            *(uint4 *)(sb + slice_off<KC>(n, kg * 8)) = op.load_b(e, col0 + n, k0 + kg * 8);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
            for (int s = 0; s < kact / 16; s++)
                mma_bf16(tmem, smem_desc(smem_u32(sa) + 256 * s, 128, 16 * KC),
                         smem_desc(smem_u32(sb) + 256 * s, 128, 16 * KC), idesc, (c > 0 || s > 0) ? 1u : 0u);
            mma_commit(mb);
        }
        // every thread waits: the next slice overwrites shared memory, the epilogue reads TMEM
        const bool done = mbar_wait(mb, parity);
        parity ^= 1u;
        if (!__syncthreads_and(done)) {
            ok = false;
            break;
        }
    }
    tc_fence_after();
    if (ok) {
        const int m = warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        for (int n0 = 0; n0 < npad; n0 += 16) {
            float v[16];
            tmem_ld16(lane_addr + (uint32_t)n0, v);
            op.store(e, row0 + m, col0 + n0, v);
        }
    } else {
        if (threadIdx.x == 0) hgb::flag(status, HGB_STATUS_ITERATION_LIMIT);
        mbar_wait(mb, parity ^ 1u);   // give the tensor core a last bounded chance to finish
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, COLS);
}

// ---- forward with TMA operand staging ----------------------------------------------------------------
// The forward's operands are plain row-major tiles (activations [b][k], weights [n][k]), so the tensor
// memory accelerator stages them: a box of 8 columns x R rows lands in shared memory as R rows of
// 16 bytes, which is one K-group of core matrices for all R rows (8-row groups 128 B apart).  Stacking
// the K-groups gives the canonical K-major layout with leading byte offset 16 R and stride byte
// offset 128.  One thread issues every copy against one mbarrier (expect_tx of the boxes' bytes;
// out-of-range rows and columns arrive as zeros), then the MMAs against the same barrier's next phase.

constexpr int FWD_NT = 64;   // output columns per CTA
constexpr int FWD_KMAX = 256;

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(mbar)
        : "memory");
}

// blockIdx.x: 128-row tile, blockIdx.y: 64-column tile, blockIdx.z: member.  xmap: [members or 1][rows][K]
// activations (x_member != 0 when each member has its own), wmap: [members][N][K] weights.
__global__ void __launch_bounds__(THREADS) k_mlp_fwd_tma(const __grid_constant__ CUtensorMap xmap,
                                                         const __grid_constant__ CUtensorMap wmap, FwdOp op,
                                                         int x_member, int *status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    constexpr int COLS = tmem_cols<FWD_NT>();
    uint8_t *sa = smem;                          // K/8 groups of 128 rows x 16 B
    uint8_t *sb = smem + TM * FWD_KMAX * 2;      // K/8 groups of 64 rows x 16 B
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int e = blockIdx.z, row0 = blockIdx.x * TM, col0 = blockIdx.y * FWD_NT;
    const int ncols = min(FWD_NT, op.N - col0);
    const int groups = op.K / 8;
    const uint32_t mb = smem_u32(&mbar);

    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), COLS);
    if (threadIdx.x == 0) mbar_init(mb, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (threadIdx.x == 0) {
        mbar_expect_tx(mb, (uint32_t)groups * (TM + FWD_NT) * 16);
        for (int g = 0; g < groups; g++) {
            tma_load_3d(smem_u32(sa + g * TM * 16), &xmap, g * 8, row0, x_member ? e : 0, mb);
            tma_load_3d(smem_u32(sb + g * FWD_NT * 16), &wmap, g * 8, col0, e, mb);
        }
    }
    bool ok = __syncthreads_and(mbar_wait(mb, 0));
    uint32_t pending = 0;   // parity of a phase still to complete when a wait gives up
    if (ok) {
        if (threadIdx.x == 0) {
            tc_fence_after();
            const uint32_t idesc = idesc_bf16(TM, ncols);
            for (int s = 0; s < op.K / 16; s++)
                mma_bf16(tmem, smem_desc(smem_u32(sa) + 2 * TM * 16 * s, TM * 16, 128),
                         smem_desc(smem_u32(sb) + 2 * FWD_NT * 16 * s, FWD_NT * 16, 128), idesc, s > 0 ? 1u : 0u);
            mma_commit(mb);
        }
        ok = __syncthreads_and(mbar_wait(mb, 1));
        pending = 1;
    }
    tc_fence_after();
    if (ok) {
        const int m = warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        for (int n0 = 0; n0 < ncols; n0 += 16) {
            float v[16];
            tmem_ld16(lane_addr + (uint32_t)n0, v);
            op.store(e, row0 + m, col0 + n0, v);
        }
    } else {
        if (threadIdx.x == 0) hgb::flag(status, HGB_STATUS_ITERATION_LIMIT);
        mbar_wait(mb, pending);   // a last bounded wait for the copies or MMAs in flight
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, COLS);
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// bf16 tensor [d2][d1][d0] (d0 contiguous), strides in bytes, boxes of b0 x b1 x 1, zero fill outside
int encode_bf16_3d(CUtensorMap *map, const void *base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t s1,
                   uint64_t s2, uint32_t b0, uint32_t b1) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = tensor_map_encoder();
    if (!fn) {
        hgb::set_cuda_error(cudaErrorNotSupported);
        return HGB_ERR_CUDA;
    }
    cuuint64_t dims[3] = {d0, d1, d2};
    cuuint64_t strides[2] = {s1, s2};
    cuuint32_t box[3] = {b0, b1, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        hgb::set_cuda_error(cudaErrorInvalidValue);
        return HGB_ERR_INVALID_ARGUMENT;
    }
    return HGB_OK;
}

int launch_fwd_tma(const FwdOp &op, long x_member_stride_elems, int members, int *status, cudaStream_t st) {
    static std::atomic<bool> attr_set{false};
    if (!attr_set.load(std::memory_order_acquire)) {
        cudaError_t err = cudaFuncSetAttribute(k_mlp_fwd_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_DYN);
        if (err != cudaSuccess) {
            hgb::set_cuda_error(err);
            return HGB_ERR_CUDA;
        }
        attr_set.store(true, std::memory_order_release);
    }
    CUtensorMap xmap, wmap;
    const uint64_t xrow = (uint64_t)op.ldx * 2;
    const int x_member = x_member_stride_elems != 0;
    int rc = encode_bf16_3d(&xmap, op.x, (uint64_t)op.K, (uint64_t)op.batch, x_member ? (uint64_t)members : 1, xrow,
                            x_member ? (uint64_t)x_member_stride_elems * 2 : xrow * (uint64_t)op.batch, 8, TM);
    if (rc) return rc;
    rc = encode_bf16_3d(&wmap, op.w, (uint64_t)op.K, (uint64_t)op.N, (uint64_t)members, (uint64_t)op.K * 2,
                        (uint64_t)op.w_es * 2, 8, FWD_NT);
    if (rc) return rc;
    dim3 grid((unsigned)hgb::ceil_div(op.batch, TM), (unsigned)hgb::ceil_div(op.N, FWD_NT), (unsigned)members);
    k_mlp_fwd_tma<<<grid, THREADS, SMEM_DYN, st>>>(xmap, wmap, op, x_member, status);
    return hgb::check_launch();
}

// ---- loss, gradient reduction, optimiser ----------------------------------------------------------

struct NetView {
    int L, E;
    int K[HGB_MLP_MAX_LAYERS], N[HGB_MLP_MAX_LAYERS];
    long w_off[HGB_MLP_MAX_LAYERS], p_off[HGB_MLP_MAX_LAYERS], b_off[HGB_MLP_MAX_LAYERS];
    long n_w, n_p;   // bf16 weights and fp32 parameters per member
};

NetView view_of(const hgb_mlp *net) {
    NetView v{};
    v.L = net->n_layers;
    v.E = net->n_members;
    long ow = 0, op = 0;
    for (int l = 0; l < v.L; l++) {
        v.K[l] = net->dims[l];
        v.N[l] = net->dims[l + 1];
        v.w_off[l] = ow;
        v.p_off[l] = op;
        v.b_off[l] = op + (long)v.N[l] * v.K[l];
        ow += (long)v.N[l] * v.K[l];
        op += (long)v.N[l] * v.K[l] + v.N[l];
    }
    v.n_w = ow;
    v.n_p = op;
    return v;
}

// loss[e] = mean (out - target)^2; dZ of the last layer = d loss / d out (bf16), one block per member
__global__ void k_mse(int batch, int nout, const float *__restrict__ out, const float *__restrict__ target,
                      long t_es, bf16 *__restrict__ dz, long dz_es, float *__restrict__ loss) {
    const int e = blockIdx.x;
    const float scale = 2.0f / ((float)batch * (float)nout);
    float acc = 0.0f;
    for (long i = threadIdx.x; i < (long)batch * nout; i += blockDim.x) {
        const long b = i / nout, n = i % nout;
        const float d = out[e * (long)batch * nout + i] - target[e * t_es + i];
        acc += d * d;
        dz[e * dz_es + b * WIDTH + n] = __float2bfloat16_rn(scale * d);
    }
    __shared__ float red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0 && loss) loss[e] = red[0] / ((float)batch * (float)nout);
}

struct GradArgs {
    NetView v;
    int batch, nsplit;
    const float *part[HGB_MLP_MAX_LAYERS];   // [E][S][N][K]
    const bf16 *dz[HGB_MLP_MAX_LAYERS];      // [E][B][WIDTH]
    long dz_es;
    float *grad;                             // [E][n_p]
};

// weight gradients: the split partials summed in split order; bias gradients: dZ summed over the batch
__global__ void k_grad_reduce(GradArgs a) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)a.v.E * a.v.n_p) return;
    const int e = (int)(idx / a.v.n_p);
    const long p = idx % a.v.n_p;
    int l = 0;
    while (l + 1 < a.v.L && p >= a.v.p_off[l + 1]) l++;
    const int K = a.v.K[l], N = a.v.N[l];
    float g = 0.0f;
    if (p < a.v.b_off[l]) {
        const long wi = p - a.v.p_off[l];
        const float *pp = a.part[l] + (long)e * a.nsplit * N * K + wi;
        for (int s = 0; s < a.nsplit; s++) g += pp[(long)s * N * K];
    } else {
        const int n = (int)(p - a.v.b_off[l]);
        const bf16 *d = a.dz[l] + e * a.dz_es + n;
        for (int b = 0; b < a.batch; b++) g += __bfloat162float(d[(long)b * WIDTH]);
    }
    a.grad[idx] = g;
}

// decoupled AdamW on the fp32 master parameters; weights (not biases) decay; bf16 weight copies written
__global__ void k_adamw(NetView v, float *__restrict__ params, const float *__restrict__ grad, float *__restrict__ m1,
                        float *__restrict__ m2, bf16 *__restrict__ w, float lr, float b1, float b2, float eps, float wd,
                        float bc1, float bc2) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)v.E * v.n_p) return;
    const int e = (int)(idx / v.n_p);
    const long p = idx % v.n_p;
    int l = 0;
    while (l + 1 < v.L && p >= v.p_off[l + 1]) l++;
    const bool is_w = p < v.b_off[l];
    const float g = grad[idx];
    const float a = b1 * m1[idx] + (1.0f - b1) * g;
    const float b = b2 * m2[idx] + (1.0f - b2) * g * g;
    m1[idx] = a;
    m2[idx] = b;
    float x = params[idx];
    if (is_w) x -= lr * wd * x;
    x -= lr * (a / bc1) / (sqrtf(b / bc2) + eps);
    params[idx] = x;
    if (is_w) w[(long)e * v.n_w + v.w_off[l] + (p - v.p_off[l])] = __float2bfloat16_rn(x);
}

__global__ void k_pack_weights(NetView v, const float *__restrict__ params, bf16 *__restrict__ w) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)v.E * v.n_p) return;
    const int e = (int)(idx / v.n_p);
    const long p = idx % v.n_p;
    int l = 0;
    while (l + 1 < v.L && p >= v.p_off[l + 1]) l++;
    if (p < v.b_off[l]) w[(long)e * v.n_w + v.w_off[l] + (p - v.p_off[l])] = __float2bfloat16_rn(params[idx]);
}

int check_net(const hgb_mlp *net) {
    if (!net || net->n_layers < 1 || net->n_layers > HGB_MLP_MAX_LAYERS || net->n_members < 1) return 0;
    if (net->n_members > 65535) return 0;
    for (int l = 0; l <= net->n_layers; l++) {
        const int d = net->dims[l];
        if (d < 16 || d > NMAX || (d & 15)) return 0;
    }
    return 1;
}

template <class Op>
int launch_gemm(const Op &op, int row_tiles, int members, int *status, cudaStream_t st, int splits = 1) {
    static std::atomic<bool> attr_set{false};   // idempotent; set before the first launch of each instantiation
    if (!attr_set.load(std::memory_order_acquire)) {
        cudaError_t err = cudaFuncSetAttribute(k_mlp_gemm<Op>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_DYN);
        if (err != cudaSuccess) {
            hgb::set_cuda_error(err);
            return HGB_ERR_CUDA;
        }
        attr_set.store(true, std::memory_order_release);
    }
    const int ytiles = Op::COL_TILED ? (int)hgb::ceil_div(op.ncols(), Op::NT) : splits;
    dim3 grid((unsigned)row_tiles, (unsigned)ytiles, (unsigned)members);
    k_mlp_gemm<Op><<<grid, THREADS, SMEM_DYN, st>>>(op, status);
    return hgb::check_launch();
}

const float *param_bias(const hgb_mlp *net, const NetView &v, int l) { return net->params + v.b_off[l]; }

// ---- fused forward for small query batches --------------------------------------------------------
// One cluster of FUSED_CL CTAs per member; CTA r of the cluster owns output columns
// [r N_l / FUSED_CL, (r + 1) N_l / FUSED_CL) of every layer l.  At the start it bulk-copies its
// column slice of every layer's weights (cp.async.bulk, one mbarrier per layer, so the later layers'
// copies overlap the first layers' arithmetic) into shared memory.  A layer is a matrix-vector
// product per query on the CUDA cores (a batch of at most FUSED_QMAX rows would leave a 128-row
// tensor-core tile almost empty): each warp takes every fourth column, its lanes split the
// reduction axis in runs of 8, fp32 products, and the warp's columns are summed together by one
// transposing shuffle reduction.  The hidden activations
// (bias, SiLU, rounded to bf16 as in the layered forward) are stored into the next activation
// buffer of every CTA of the cluster (distributed shared memory), and one cluster barrier per layer
// publishes them; the buffers alternate, so a CTA writing layer l + 1's inputs never meets a peer
// still reading layer l's.  The last layer writes fp32 outputs.  The copies' waits are bounded: on
// expiry the CTA flags HGB_STATUS_ITERATION_LIMIT and keeps taking part in every cluster barrier
// (its outputs are not valid), and waits once more, bounded, for its copies before it returns.
// The biases of all of the CTA's columns are loaded into shared memory at the start (one round trip
// instead of one per column).  Inputs, outputs and the status word are read and written with plain
// accesses, so they may be pinned host memory (device-accessible under unified addressing): a
// graphed query then needs no copy nodes.  The status bit is set with a plain read-modify-write.
constexpr int FUSED_CL = 8;
constexpr int FUSED_QMAX = HGB_MLP_FUSED_MAX_BATCH;
constexpr int FUSED_THREADS = 128;
constexpr int FUSED_ACT_BYTES = FUSED_QMAX * WIDTH * 2;   // one bf16 activation buffer
constexpr int FUSED_NCMAX = NMAX / FUSED_CL;              // columns per CTA and layer, at most

struct FusedArgs {
    int L, batch;
    int K[HGB_MLP_MAX_LAYERS], N[HGB_MLP_MAX_LAYERS];
    int w_smem[HGB_MLP_MAX_LAYERS];     // byte offset of layer l's weight slice in shared memory
    long w_off[HGB_MLP_MAX_LAYERS], b_off[HGB_MLP_MAX_LAYERS];
    long n_w, n_p;
    const bf16 *weights;
    const float *params;
    const bf16 *x;
    long x_es;
    float *out;
    int *status;
};

// global -> this CTA's shared memory, completion counted on mbar (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ float dot8_bf16(uint4 a, uint4 b, float acc) {
    const __nv_bfloat162 *pa = reinterpret_cast<const __nv_bfloat162 *>(&a);
    const __nv_bfloat162 *pb = reinterpret_cast<const __nv_bfloat162 *>(&b);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float2 fa = __bfloat1622float2(pa[i]), fb = __bfloat1622float2(pb[i]);
        acc = fmaf(fa.x, fb.x, acc);
        acc = fmaf(fa.y, fb.y, acc);
    }
    return acc;
}

__global__ void __cluster_dims__(FUSED_CL, 1, 1) __launch_bounds__(FUSED_THREADS)
    k_mlp_fwd_fused(const __grid_constant__ FusedArgs a) {
    extern __shared__ __align__(128) unsigned char fsm[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int e = blockIdx.y;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    bf16 *act0 = (bf16 *)fsm;
    bf16 *act1 = (bf16 *)(fsm + FUSED_ACT_BYTES);
    uint64_t *mbar = (uint64_t *)(fsm + 2 * FUSED_ACT_BYTES);
    float *sbias = (float *)(fsm + 2 * FUSED_ACT_BYTES + 128);   // [layer][FUSED_NCMAX]
    if (t == 0) {
        for (int l = 0; l < a.L; l++) mbar_init(smem_u32(&mbar[l]), 1);
    }
    for (int i = t; i < a.L * FUSED_NCMAX; i += FUSED_THREADS) {
        const int l = i / FUSED_NCMAX, n = i % FUSED_NCMAX, nc = a.N[l] / FUSED_CL;
        if (n < nc) sbias[i] = __ldg(a.params + e * a.n_p + a.b_off[l] + rank * nc + n);
    }
    __syncthreads();
    if (t == 0) {
        for (int l = 0; l < a.L; l++) {
            const int nc = a.N[l] / FUSED_CL;
            const uint32_t bytes = (uint32_t)nc * (uint32_t)a.K[l] * 2u;
            mbar_expect_tx(smem_u32(&mbar[l]), bytes);
            bulk_g2s(smem_u32(fsm + a.w_smem[l]), a.weights + e * a.n_w + a.w_off[l] + (long)rank * nc * a.K[l], bytes,
                     smem_u32(&mbar[l]));
        }
    }
    const int Q = a.batch;
    for (int i = t; i < Q * a.K[0]; i += FUSED_THREADS) {
        const int q = i / a.K[0], k = i % a.K[0];
        act0[q * WIDTH + k] = a.x[e * a.x_es + (long)q * a.K[0] + k];
    }
    cluster.sync();   // every CTA of the cluster runs before any stores into its shared memory
    bool ok = true;
    for (int l = 0; l < a.L; l++) {
        const int K = a.K[l], N = a.N[l], nc = N / FUSED_CL, c0 = rank * nc;
        if (ok && !mbar_wait(smem_u32(&mbar[l]), 0)) ok = false;
        const bf16 *W = (const bf16 *)(fsm + a.w_smem[l]);   // [nc][K]
        const bf16 *X = (l & 1) ? act1 : act0;
        bf16 *Y = (l & 1) ? act0 : act1;
        const float *bias = sbias + l * FUSED_NCMAX;
        const bool last = l == a.L - 1;
        // warp w: columns n = w + 4 j, j < ncw (at most 8); lane k: reduction entries 8k .. 8k + 7
        // (K <= 256, so one run per lane).  The eight column sums are reduced together: three
        // exchange levels halve the set a lane carries (4 + 2 + 1 shuffles), two more finish the
        // sum, and lane 4 j ends with column j's total, so the eight epilogues run side by side.
        const int ncw = (nc - warp + 3) / 4;
        const bool has_run = lane < K / 8;
        const int jl = 4 * ((lane >> 4) & 1) + 2 * ((lane >> 3) & 1) + ((lane >> 2) & 1);
        for (int q = 0; q < Q; q++) {
            float v[8];
            const uint4 xv = has_run ? *(const uint4 *)(X + q * WIDTH + lane * 8) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
            for (int j = 0; j < 8; j++)
                v[j] = (has_run && j < ncw) ? dot8_bf16(*(const uint4 *)(W + (long)(warp + 4 * j) * K + lane * 8), xv, 0.0f)
                                            : 0.0f;
            const bool h1 = (lane >> 4) & 1, h2 = (lane >> 3) & 1, h3 = (lane >> 2) & 1;
            float w4[4], w2[2];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float keep = h1 ? v[i + 4] : v[i], give = h1 ? v[i] : v[i + 4];
                w4[i] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
            }
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const float keep = h2 ? w4[i + 2] : w4[i], give = h2 ? w4[i] : w4[i + 2];
                w2[i] = keep + __shfl_xor_sync(0xffffffffu, give, 8);
            }
            float acc = (h3 ? w2[1] : w2[0]) + __shfl_xor_sync(0xffffffffu, h3 ? w2[0] : w2[1], 4);
            acc += __shfl_xor_sync(0xffffffffu, acc, 2);
            acc += __shfl_xor_sync(0xffffffffu, acc, 1);
            if ((lane & 3) == 0 && jl < ncw) {
                const int n = warp + 4 * jl;
                const float z = acc + bias[n];
                if (last) {
                    a.out[((long)e * Q + q) * N + c0 + n] = z;
                } else {
                    const bf16 y = __float2bfloat16_rn(silu(z));
#pragma unroll
                    for (int r = 0; r < FUSED_CL; r++) cluster.map_shared_rank(Y, r)[q * WIDTH + c0 + n] = y;
                }
            }
        }
        cluster.sync();   // layer l + 1's inputs are in every CTA; layer l's are no longer read
    }
    if (!ok) {
        if (t == 0) {
            if (a.status) *(volatile int *)a.status |= HGB_STATUS_ITERATION_LIMIT;
            for (int l = 0; l < a.L; l++) mbar_wait(smem_u32(&mbar[l]), 0);   // bounded: copies in flight
        }
        __syncthreads();
    }
}

size_t fused_smem_bytes(const NetView &v, FusedArgs *fa) {
    // two activation buffers, the mbarriers, the biases, then the weight slices
    size_t off = 2 * (size_t)FUSED_ACT_BYTES + 128 + (((size_t)v.L * FUSED_NCMAX * 4 + 127) & ~(size_t)127);
    for (int l = 0; l < v.L; l++) {
        if (fa) fa->w_smem[l] = (int)off;
        off += ((size_t)(v.N[l] / FUSED_CL) * v.K[l] * 2 + 127) & ~(size_t)127;
    }
    return off;
}

}  // namespace

extern "C" {

long hgb_mlp_param_count(const hgb_mlp *net) { return check_net(net) ? view_of(net).n_p : -1; }

long hgb_mlp_weight_count(const hgb_mlp *net) { return check_net(net) ? view_of(net).n_w : -1; }

int hgb_mlp_forward(const hgb_mlp *net, const uint16_t *x, long x_member_stride, int batch, uint16_t *act,
                    float *pre, float *out, int *d_status, void *stream) {
    HGB_CHECK_ARG(check_net(net) && net->params && net->weights && x && act && out && batch >= 0);
    HGB_CHECK_ARG(x_member_stride >= 0);
    if (batch == 0) return HGB_OK;
    const NetView v = view_of(net);
    cudaStream_t st = (cudaStream_t)stream;
    const long hid_es = (long)batch * WIDTH;            // member stride of one layer's hidden buffer
    const long hid_ls = (long)v.E * hid_es;             // layer stride
    for (int l = 0; l < v.L; l++) {
        FwdOp op{};
        const bool first = l == 0, last = l == v.L - 1;
        op.x = first ? (const bf16 *)x : (const bf16 *)act + (l - 1) * hid_ls;
        op.x_es = first ? x_member_stride : hid_es;
        op.ldx = first ? v.K[0] : WIDTH;
        op.w = (const bf16 *)net->weights + v.w_off[l];
        op.w_es = v.n_w;
        op.bias = param_bias(net, v, l);
        op.b_es = v.n_p;
        op.K = v.K[l];
        op.N = v.N[l];
        op.batch = batch;
        op.act = last ? 0 : 1;
        op.pre = (last || !pre) ? nullptr : pre + l * hid_ls;
        op.pre_es = hid_es;
        op.ldp = WIDTH;
        op.y = last ? nullptr : (bf16 *)act + l * hid_ls;
        op.y_es = hid_es;
        op.ldy = WIDTH;
        op.out = last ? out : nullptr;
        op.out_es = (long)batch * v.N[l];
        int rc = launch_fwd_tma(op, op.x_es, v.E, d_status, st);
        if (rc) return rc;
    }
    return HGB_OK;
}

int hgb_mlp_forward_fused(const hgb_mlp *net, const uint16_t *x, long x_member_stride, int batch, float *out,
                          int *d_status, void *stream) {
    HGB_CHECK_ARG(check_net(net) && net->params && net->weights && x && out && batch >= 0);
    HGB_CHECK_ARG(x_member_stride >= 0 && batch <= HGB_MLP_FUSED_MAX_BATCH && net->n_members <= 65535);
    HGB_CHECK_ARG(((uintptr_t)net->weights & 15) == 0);   // bulk-copy source alignment
    if (batch == 0) return HGB_OK;
    const NetView v = view_of(net);
    FusedArgs fa{};
    fa.L = v.L;
    fa.batch = batch;
    for (int l = 0; l < v.L; l++) {
        fa.K[l] = v.K[l];
        fa.N[l] = v.N[l];
        fa.w_off[l] = v.w_off[l];
        fa.b_off[l] = v.b_off[l];
    }
    fa.n_w = v.n_w;
    fa.n_p = v.n_p;
    fa.weights = (const bf16 *)net->weights;
    fa.params = net->params;
    fa.x = (const bf16 *)x;
    fa.x_es = x_member_stride;
    fa.out = out;
    fa.status = d_status;
    const size_t smem = fused_smem_bytes(v, &fa);
    int rc = hgb::ensure_dyn_smem((const void *)k_mlp_fwd_fused, smem);
    if (rc) return rc;
    dim3 grid(FUSED_CL, (unsigned)v.E);
    k_mlp_fwd_fused<<<grid, FUSED_THREADS, smem, (cudaStream_t)stream>>>(fa);
    return hgb::check_launch();
}

int hgb_emulator_query(const hgb_mlp *net, const double *params, int n_queries, int n_params, const double *lo,
                       const double *hi, const double *mu, const double *sd, int n_out, uint16_t *x_host,
                       float *out_host, int *status_host, double *result, void *stream) {
    HGB_CHECK_ARG(check_net(net) && params && lo && hi && mu && sd && x_host && out_host && status_host && result);
    HGB_CHECK_ARG(n_queries >= 1 && n_queries <= HGB_MLP_FUSED_MAX_BATCH && n_params >= 1);
    HGB_CHECK_ARG(n_params <= net->dims[0] && n_out >= 1 && n_out <= net->dims[net->n_layers]);
    const int K0 = net->dims[0], NL = net->dims[net->n_layers], E = net->n_members;
    // inputs: 2 (p - lo) / (hi - lo) - 1 rounded to float, then to bf16 (nearest, ties to even)
    for (int q = 0; q < n_queries; q++)
        for (int k = 0; k < K0; k++) {
            uint16_t bits = 0;
            if (k < n_params) {
                const double u = (params[(long)q * n_params + k] - lo[k]) / (hi[k] - lo[k]);
                const float f = (float)(2.0 * u - 1.0);
                uint32_t w;
                memcpy(&w, &f, sizeof(w));
                bits = (uint16_t)((w + 0x7FFFu + ((w >> 16) & 1u)) >> 16);
            }
            x_host[(long)q * K0 + k] = bits;
        }
    *(volatile int *)status_host = 0;
    int rc = hgb_mlp_forward_fused(net, x_host, 0, n_queries, out_host, status_host, stream);
    if (rc) return rc;
    cudaError_t err = cudaStreamSynchronize((cudaStream_t)stream);
    if (err != cudaSuccess) {
        hgb::set_cuda_error(err);
        return HGB_ERR_CUDA;
    }
    if (*(volatile int *)status_host) return HGB_ERR_DEVICE_LIMIT;
    // the ensemble mean in the statistics' units: mean over members, then * sd + mu
    for (int q = 0; q < n_queries; q++)
        for (int k = 0; k < n_out; k++) {
            double acc = 0.0;
            for (int e = 0; e < E; e++) acc += (double)out_host[((long)e * n_queries + q) * NL + k];
            result[(long)q * n_out + k] = acc / E * sd[k] + mu[k];
        }
    return HGB_OK;
}

size_t hgb_mlp_backward_workspace_bytes(const hgb_mlp *net, int batch) {
    if (!check_net(net) || batch <= 0) return 0;
    const NetView v = view_of(net);
    const int nsplit = (int)hgb::ceil_div(batch, HGB_MLP_SPLIT_ROWS);
    size_t bytes = sizeof(uint16_t) * (size_t)v.L * v.E * batch * WIDTH;   // dZ per layer
    for (int l = 0; l < v.L; l++) bytes += sizeof(float) * (size_t)v.E * nsplit * v.N[l] * v.K[l];
    return bytes;
}

int hgb_mlp_backward(const hgb_mlp *net, const uint16_t *x, long x_member_stride, int batch, const uint16_t *act,
                     const float *pre, const float *out, const float *target, long target_member_stride, float *grad,
                     float *loss, void *workspace, size_t workspace_bytes, int *d_status, void *stream) {
    HGB_CHECK_ARG(check_net(net) && net->params && net->weights && x && act && pre && out && target && grad);
    HGB_CHECK_ARG(batch >= 1 && x_member_stride >= 0 && target_member_stride >= 0);
    HGB_CHECK_ARG(workspace && workspace_bytes >= hgb_mlp_backward_workspace_bytes(net, batch));
    const NetView v = view_of(net);
    cudaStream_t st = (cudaStream_t)stream;
    const long hid_es = (long)batch * WIDTH, hid_ls = (long)v.E * hid_es;
    const int nsplit = (int)hgb::ceil_div(batch, HGB_MLP_SPLIT_ROWS);
    bf16 *dz = (bf16 *)workspace;
    float *part = (float *)((char *)workspace + sizeof(uint16_t) * (size_t)v.L * hid_ls);
    GradArgs ga{};
    ga.v = v;
    ga.batch = batch;
    ga.nsplit = nsplit;
    ga.dz_es = hid_es;
    ga.grad = grad;
    {
        float *pp = part;
        for (int l = 0; l < v.L; l++) {
            ga.part[l] = pp;
            ga.dz[l] = dz + l * hid_ls;
            pp += (size_t)v.E * nsplit * v.N[l] * v.K[l];
        }
    }
    const int last = v.L - 1;
    k_mse<<<v.E, 256, 0, st>>>(batch, v.N[last], out, target, target_member_stride, dz + last * hid_ls, hid_es, loss);
    int rc = hgb::check_launch();
    if (rc) return rc;
    for (int l = last; l >= 0; l--) {
        DwOp dw{};
        dw.dz = dz + l * hid_ls;
        dw.dz_es = hid_es;
        dw.x = l == 0 ? (const bf16 *)x : (const bf16 *)act + (l - 1) * hid_ls;
        dw.x_es = l == 0 ? x_member_stride : hid_es;
        dw.ldx = l == 0 ? v.K[0] : WIDTH;
        dw.part = const_cast<float *>(ga.part[l]);
        dw.K = v.K[l];
        dw.N = v.N[l];
        dw.batch = batch;
        dw.rows_per_split = HGB_MLP_SPLIT_ROWS;
        dw.nsplit = nsplit;
        if ((rc = launch_gemm(dw, (int)hgb::ceil_div(v.N[l], TM), v.E, d_status, st, nsplit))) return rc;
        if (l == 0) break;
        DxOp dx{};
        dx.dz = dz + l * hid_ls;
        dx.dz_es = hid_es;
        dx.w = (const bf16 *)net->weights + v.w_off[l];
        dx.w_es = v.n_w;
        dx.pre = pre + (l - 1) * hid_ls;
        dx.pre_es = hid_es;
        dx.dzp = dz + (l - 1) * hid_ls;
        dx.dzp_es = hid_es;
        dx.K = v.K[l];
        dx.N = v.N[l];
        dx.batch = batch;
        if ((rc = launch_gemm(dx, (int)hgb::ceil_div(batch, TM), v.E, d_status, st))) return rc;
    }
    const long np = (long)v.E * v.n_p;
    k_grad_reduce<<<(unsigned)hgb::ceil_div(np, 256), 256, 0, st>>>(ga);
    return hgb::check_launch();
}

int hgb_mlp_adamw(const hgb_mlp *net, float *params, const float *grad, float *m1, float *m2, uint16_t *weights,
                  int step, float lr, float beta1, float beta2, float eps, float weight_decay, void *stream) {
    HGB_CHECK_ARG(check_net(net) && params && grad && m1 && m2 && weights && step >= 1);
    const NetView v = view_of(net);
    const long np = (long)v.E * v.n_p;
    const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
    k_adamw<<<(unsigned)hgb::ceil_div(np, 256), 256, 0, (cudaStream_t)stream>>>(
        v, params, grad, m1, m2, (bf16 *)weights, lr, beta1, beta2, eps, weight_decay, bc1, bc2);
    return hgb::check_launch();
}

int hgb_mlp_pack_weights(const hgb_mlp *net, const float *params, uint16_t *weights, void *stream) {
    HGB_CHECK_ARG(check_net(net) && params && weights);
    const NetView v = view_of(net);
    const long np = (long)v.E * v.n_p;
    k_pack_weights<<<(unsigned)hgb::ceil_div(np, 256), 256, 0, (cudaStream_t)stream>>>(v, params, (bf16 *)weights);
    return hgb::check_launch();
}

}  // extern "C"
