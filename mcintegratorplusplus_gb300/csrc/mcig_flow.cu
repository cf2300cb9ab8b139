// mcig_flow.cu -- affine-coupling normalizing flow on BF16 tensor cores, used as an
// independence Metropolis-Hastings proposal (the learned form of the sampler).
//
// The flow (RealNVP couplings) and its parameter layout are defined in
// oracle/flow_oracle.py, which restates them in numpy as the checker:
//   layer l: a = y[perm_l[:d]], b = y[perm_l[d:]],
//            h1 = relu(a W1 + b1), h2 = relu(h1 W2 + b2), o = h2 W3 + b3,
//            s = S tanh(o[:d]/S), t = o[d:],
//            generative  b <- b exp(s) + t,   density  b <- (b - t) exp(-s);
//   base affine x = mu + exp(logsig) y;  log q = log N(z) - sum s - sum logsig.
// Sizes: D <= 32 even, d = D/2 <= 16, hidden H = 128, L <= 16 layers.
//
// Kernels (one CTA = 112 samples in the pass kernel, warps w and w + 7 owning rows
// 16w..16w+15; 128 samples in the backward kernel, warp w alone owning rows 16w..16w+15):
//   flow_pass_kernel     the L layers in one launch, generative or density
//                        direction; GEMMs with mma.sync.m16n8k16 bf16 -> f32,
//                        activations and weights staged in shared memory with
//                        padded rows (conflict-free fragment loads); the density
//                        direction can save a per-layer tape (a, b, s, t).
//   flow_backward_kernel gradient of -mean log q through the density direction:
//                        MLP recomputed from the tape, data gradients and weight
//                        gradients as bf16 mma GEMMs, weight gradients reduced
//                        across CTAs with float atomics.
//   flow_adam_kernel     Adam on the float master parameters; flow_cast_kernel
//                        rebuilds the bf16 weight copies.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mcig.h"
#include "mcig_common.cuh"

int mcig_set_last_error(int code, const char *msg); // mcig_capi.cu

#define FLOW_H 128
#define FLOW_MAXD 32
#define FLOW_MAXL 16
#define FLOW_ROWS 128   // samples per CTA
#define FLOW_THREADS 256
// pass kernel: 112 samples per CTA (147 CTAs cover 16,384 samples on the 152 SMs in one
// wave, where 128-sample CTAs left 24 SMs idle), two warps per 16 rows, each forming half of
// every GEMM's columns
#define FLOW_PASS_ROWS 112
#define FLOW_PASS_PAIRS (FLOW_PASS_ROWS / 16)
#define FLOW_PASS_THREADS (64 * FLOW_PASS_PAIRS)
#define FLOW_SMAX 3.0f

// shared-memory strides (in bf16 elements), padded so that a fragment load of
// 8 rows x 4 words hits 32 different banks
#define LDA_S 24   // a-half tile [128][16 (+8)]
#define LDH_S 136  // hidden tiles [128][128 (+8)]
#define LDO_S 40   // output-gradient tile [128][32 (+8)]

struct FlowLayerPtrs {
    const __nv_bfloat16 *W1n; // [H][16]   B operand of a*W1 (n-major, k contiguous)
    const __nv_bfloat16 *W2n; // [H][H]    B operand of h1*W2
    const __nv_bfloat16 *W3n; // [32][H]   B operand of h2*W3 (rows >= 2d zero)
    const __nv_bfloat16 *W3t; // [H][32]   B operand of g_o*W3^T
    const __nv_bfloat16 *W2t; // [H][H]    B operand of g_h2*W2^T
    const __nv_bfloat16 *W1t; // [16][H]   B operand of g_h1*W1^T (rows >= d zero)
    const float *b1, *b2, *b3;
};

struct FlowArgs {
    int D, d, L, n;           // dimension, half, layers, samples
    int dir;                  // 0 generative (z -> x), 1 density (x -> z)
    const float *in;          // [n][D]
    float *out;               // [n][D]
    float *logq;              // [n]
    const float *mu, *logsig; // base affine
    const int *perm;          // [L][D]
    float *tape;              // density direction: [L][n][4d] (a, b, s, t) or null
    const __nv_bfloat16 *wb;  // bf16 weight copies
    const float *theta;       // float master parameters
    int64_t wstride;          // bf16 elements per layer in wb
    int64_t pstride;          // floats per layer in theta
    // chain-minor alternatives: input in_cm[c * cm_stride + row] (double, replaces in) and
    // output out_cm[c * cm_stride + row] (float, besides or instead of out)
    const double *in_cm;
    float *out_cm;
    int64_t cm_stride;
    const float *in_cmf;      // chain-minor float input in_cmf[c * cm_stride + row] (replaces in)
    // a second set of nb rows after the n rows above (register-fused pass, density direction,
    // no out / tape): row n + r reads in_cmf_b[c * cm_stride + r], its log q goes to logq_b[r]
    int nb;
    const float *in_cmf_b;
    float *logq_b;
    // generative direction: z drawn in the kernel (replaces in): coordinate i of row r is
    // Box-Muller normal i % 4 of Philox block (zcycle lo, zcycle hi, r, FLOW_TAG_Z << 12 | i / 4)
    // with key (zk0, zk1)
    int zgen;
    uint32_t zk0, zk1;
    uint64_t zcycle;
};

#define FLOW_TAG_Z 3

// the standard normal z of row (chain) `row`, coordinate i, of flow proposal cycle `cycle`
__device__ __forceinline__ float flow_z_value(const FlowArgs &f, int row, int i)
{
    const P4 q = philox4x32_10((uint32_t)f.zcycle, (uint32_t)(f.zcycle >> 32), (uint32_t)row,
                               (FLOW_TAG_Z << 12) | (uint32_t)(i >> 2), f.zk0, f.zk1);
    float z0, z1;
    const int k = i & 3;
    box_muller_f(k < 2 ? q.a : q.c, k < 2 ? q.b : q.d, z0, z1);
    return (k & 1) ? z1 : z0;
}

// input value of row r (in the whole set), coordinate c, from whichever source the pass reads
__device__ __forceinline__ float flow_input(const FlowArgs &f, int r, int c)
{
    if (r >= f.n) { return f.in_cmf_b[(int64_t)c * f.cm_stride + (r - f.n)]; }
    if (f.zgen) { return flow_z_value(f, r, c); }
    if (f.in_cm) { return (float)f.in_cm[(int64_t)c * f.cm_stride + r]; }
    if (f.in_cmf) { return f.in_cmf[(int64_t)c * f.cm_stride + r]; }
    return f.in[(int64_t)r * f.D + c];
}

// ------------------------------------------------------------------------
// bf16 tensor-core helpers
// ------------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16 *p) { return *(const uint32_t *)p; }

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// four 8x8 bf16 matrices from shared memory in mma fragment order: thread t gives the
// address of row t % 8 of matrix t / 8 (16-byte aligned rows)
__device__ __forceinline__ void ldmatrix_x4(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const __nv_bfloat16 *p)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

// C[16 x 8 NT] += A[rows r0.., K] * B[K, 8 NT]; A row-major (k contiguous, stride lda),
// B "n-major" (element (k, n) at Bn[n*ldb + k]).  Fragments come from ldmatrix: one x4
// for the A tile of a k-step, one x4 for the B tiles of two n-tiles.  NT is even.
template <int KSTEPS, int NT>
__device__ __forceinline__ void warp_gemm(const __nv_bfloat16 *A, int lda, int r0, const __nv_bfloat16 *Bn, int ldb,
                                          float (&acc)[NT][4])
{
    const int lane = threadIdx.x & 31, mi = lane >> 3, rr = lane & 7;
#pragma unroll
    for (int ks = 0; ks < KSTEPS; ++ks) {
        const int kb = ks * 16;
        uint32_t a0, a1, a2, a3; // matrices: rows 0-7 / 8-15 x k 0-7, then x k 8-15
        ldmatrix_x4(a0, a1, a2, a3, A + (r0 + (mi & 1) * 8 + rr) * lda + kb + (mi >> 1) * 8);
#pragma unroll
        for (int nt = 0; nt < NT; nt += 2) {
            uint32_t b0, b1, b2, b3; // matrices: n-tile nt x k 0-7 / 8-15, then n-tile nt + 1
            ldmatrix_x4(b0, b1, b2, b3, Bn + ((nt + (mi >> 1)) * 8 + rr) * ldb + kb + (mi & 1) * 8);
            mma_bf16(acc[nt], a0, a1, a2, a3, b0, b1);
            mma_bf16(acc[nt + 1], a0, a1, a2, a3, b2, b3);
        }
    }
}

__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3,
                                                  const __nv_bfloat16 *p)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

// C[16 rows (feature r0..) x 8 NT cols] += X^T G over the 128 samples of the tile:
// A(row = feature i, k = sample) = X[sample][i], B(k = sample, n = j) = G[sample][j];
// both row-major by sample, so their fragments are transposed ldmatrix loads.  NT is even.
template <int NT>
__device__ __forceinline__ void warp_gemm_tn(const __nv_bfloat16 *X, int ldx, int r0, const __nv_bfloat16 *Gm, int ldg,
                                             float (&acc)[NT][4])
{
    const int lane = threadIdx.x & 31, mi = lane >> 3, rr = lane & 7;
#pragma unroll 2
    for (int ks = 0; ks < FLOW_ROWS / 16; ++ks) {
        const int s0 = ks * 16;
        uint32_t a0, a1, a2, a3; // (features 0-7 / 8-15) x (samples 0-7), then samples 8-15
        ldmatrix_x4_trans(a0, a1, a2, a3, X + (s0 + (mi >> 1) * 8 + rr) * ldx + r0 + (mi & 1) * 8);
#pragma unroll
        for (int nt = 0; nt < NT; nt += 2) {
            uint32_t b0, b1, b2, b3; // n-tile nt x samples 0-7 / 8-15, then n-tile nt + 1
            ldmatrix_x4_trans(b0, b1, b2, b3, Gm + (s0 + (mi & 1) * 8 + rr) * ldg + (nt + (mi >> 1)) * 8);
            mma_bf16(acc[nt], a0, a1, a2, a3, b0, b1);
            mma_bf16(acc[nt + 1], a0, a1, a2, a3, b2, b3);
        }
    }
}

template <int NT>
__device__ __forceinline__ void zero_acc(float (&acc)[NT][4])
{
#pragma unroll
    for (int i = 0; i < NT; ++i) { acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f; }
}

// epilogue: bias (+ relu) -> bf16 row-major tile
template <int NT>
__device__ __forceinline__ void store_act(const float (&acc)[NT][4], const float *bias, bool relu, __nv_bfloat16 *H, int ldh,
                                          int r0)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const int c = nt * 8 + 2 * t;
        float v0 = acc[nt][0] + bias[c], v1 = acc[nt][1] + bias[c + 1];
        float v2 = acc[nt][2] + bias[c], v3 = acc[nt][3] + bias[c + 1];
        if (relu) {
            v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); v2 = fmaxf(v2, 0.f); v3 = fmaxf(v3, 0.f);
        }
        *(uint32_t *)(H + (r0 + g) * ldh + c) = pack2(__float2bfloat16_rn(v0), __float2bfloat16_rn(v1));
        *(uint32_t *)(H + (r0 + g + 8) * ldh + c) = pack2(__float2bfloat16_rn(v2), __float2bfloat16_rn(v3));
    }
}

// ------------------------------------------------------------------------
// shared-memory plan of one CTA
// ------------------------------------------------------------------------
struct FlowSmem {
    float Y[FLOW_ROWS][FLOW_MAXD + 1];
    float O[FLOW_ROWS][FLOW_MAXD + 1];
    __nv_bfloat16 A[FLOW_ROWS * LDA_S];
    __nv_bfloat16 H1[FLOW_ROWS * LDH_S];
    __nv_bfloat16 H2[FLOW_ROWS * LDH_S];
    __nv_bfloat16 W1n[2][FLOW_H * LDA_S]; // two buffers: layer l computes while layer l+1 arrives
    __nv_bfloat16 W2n[2][FLOW_H * LDH_S];
    __nv_bfloat16 W3n[2][32 * LDH_S];
    float bias[2][2 * FLOW_H + 32];       // b1, b2, b3 of the layer in weight buffer of the same index
    float logdet[FLOW_ROWS];
    int perm[FLOW_MAXL * FLOW_MAXD];      // coordinate permutations of all layers
};

// bf16 weight copies per layer (flow_cast_kernel): offsets in elements
#define WB_W1N 0
#define WB_W2N (WB_W1N + FLOW_H * 16)
#define WB_W3N (WB_W2N + FLOW_H * FLOW_H)
#define WB_W3T (WB_W3N + 32 * FLOW_H)
#define WB_W2T (WB_W3T + FLOW_H * 32)
#define WB_W1T (WB_W2T + FLOW_H * FLOW_H)
#define WB_LAYER (WB_W1T + 16 * FLOW_H)

// float master layout per layer (oracle/flow_oracle.py): W1[d][H] b1[H] W2[H][H] b2[H] W3[H][2d] b3[2d]
__host__ __device__ __forceinline__ int64_t pl_W1(int) { return 0; }
__host__ __device__ __forceinline__ int64_t pl_b1(int d) { return (int64_t)d * FLOW_H; }
__host__ __device__ __forceinline__ int64_t pl_W2(int d) { return pl_b1(d) + FLOW_H; }
__host__ __device__ __forceinline__ int64_t pl_b2(int d) { return pl_W2(d) + FLOW_H * FLOW_H; }
__host__ __device__ __forceinline__ int64_t pl_W3(int d) { return pl_b2(d) + FLOW_H; }
__host__ __device__ __forceinline__ int64_t pl_b3(int d) { return pl_W3(d) + (int64_t)FLOW_H * 2 * d; }
__host__ __device__ __forceinline__ int64_t pl_size(int d) { return pl_b3(d) + 2 * d; }

__global__ void flow_cast_kernel(const float *theta, __nv_bfloat16 *wb, int d, int L)
{
    const int64_t per = WB_LAYER;
    const int64_t total = per * L;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int l = (int)(i / per);
        const int64_t e = i % per;
        const float *P = theta + (int64_t)l * pl_size(d);
        float v = 0.f;
        if (e < WB_W2N) { // W1n[n][k] = W1[k][n]
            const int n = (int)(e / 16), k = (int)(e % 16);
            v = (k < d) ? P[pl_W1(d) + (int64_t)k * FLOW_H + n] : 0.f;
        } else if (e < WB_W3N) { // W2n[n][k] = W2[k][n]
            const int64_t q = e - WB_W2N;
            const int n = (int)(q / FLOW_H), k = (int)(q % FLOW_H);
            v = P[pl_W2(d) + (int64_t)k * FLOW_H + n];
        } else if (e < WB_W3T) { // W3n[n][k] = W3[k][n], n < 2d
            const int64_t q = e - WB_W3N;
            const int n = (int)(q / FLOW_H), k = (int)(q % FLOW_H);
            v = (n < 2 * d) ? P[pl_W3(d) + (int64_t)k * 2 * d + n] : 0.f;
        } else if (e < WB_W2T) { // W3t[n=h][k=o] = W3[h][o]
            const int64_t q = e - WB_W3T;
            const int n = (int)(q / 32), k = (int)(q % 32);
            v = (k < 2 * d) ? P[pl_W3(d) + (int64_t)n * 2 * d + k] : 0.f;
        } else if (e < WB_W1T) { // W2t[n=h1][k=h2] = W2[h1][h2]
            const int64_t q = e - WB_W2T;
            v = P[pl_W2(d) + q];
        } else { // W1t[n=a][k=h1] = W1[a][h1]
            const int64_t q = e - WB_W1T;
            const int n = (int)(q / FLOW_H), k = (int)(q % FLOW_H);
            v = (n < d) ? P[pl_W1(d) + (int64_t)n * FLOW_H + k] : 0.f;
        }
        wb[i] = __float2bfloat16_rn(v);
    }
}

// cooperative copy of a bf16 matrix [rows][cols] (global, dense) into a padded smem tile
// rows x COLS bf16 from global (row-major, contiguous) into shared memory with row
// stride ld, 16 bytes per copy (source offsets, ld and the tiles are multiples of 8 elements)
template <int COLS>
__device__ __forceinline__ void load_tile(__nv_bfloat16 *dst, int ld, const __nv_bfloat16 *src, int rows)
{
    constexpr int VPR = COLS / 8; // 16-byte vectors per row
    const int nv = rows * VPR;
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        const int r = i / VPR, c = (i % VPR) * 8;
        *(uint4 *)(dst + r * ld + c) = *(const uint4 *)(src + (size_t)i * 8);
    }
}

// sum of v over the 8 lanes that share lane & 3 (the accumulator rows of an mma fragment)
__device__ __forceinline__ float sum_over_g(float v)
{
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

// paired float atomic add (address 8-byte aligned)
__device__ __forceinline__ void atomic_add2(float *a, float x, float y) { atomicAdd((float2 *)a, make_float2(x, y)); }

// barrier of the two warps that share 16 rows in the pass kernel (named barrier 1 + pair)
__device__ __forceinline__ void pair_sync(int pair)
{
    asm volatile("bar.sync %0, 64;\n" ::"r"(1 + pair) : "memory");
}

// The MLP of one layer for the 16 rows r0.. shared by the warps of pair `pair`: warp
// `half` forms the columns [64 half, 64 half + 64) of h1 and h2 and [16 half, 16 half + 16)
// of o.  Each GEMM reads the whole row of its input, so the pair meets after each stage;
// every (row, column) is one warp's dot product over the whole row, k ascending.
__device__ __forceinline__ void pair_layer_mlp(FlowSmem &s, int r0, int pair, int half, int buf)
{
    const float *bias = s.bias[buf];
    {
        float acc[8][4];
        zero_acc(acc);
        warp_gemm<1, 8>(s.A, LDA_S, r0, s.W1n[buf] + half * 64 * LDA_S, LDA_S, acc);
        store_act(acc, bias + half * 64, true, s.H1 + half * 64, LDH_S, r0);
    }
    pair_sync(pair);
    {
        float acc[8][4];
        zero_acc(acc);
        warp_gemm<FLOW_H / 16, 8>(s.H1, LDH_S, r0, s.W2n[buf] + half * 64 * LDH_S, LDH_S, acc);
        store_act(acc, bias + FLOW_H + half * 64, true, s.H2 + half * 64, LDH_S, r0);
    }
    pair_sync(pair);
    {
        float acc[2][4];
        zero_acc(acc);
        warp_gemm<FLOW_H / 16, 2>(s.H2, LDH_S, r0, s.W3n[buf] + half * 16 * LDH_S, LDH_S, acc);
        const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
            const int c = half * 16 + nt * 8 + 2 * t;
            s.O[r0 + g][c] = acc[nt][0] + bias[2 * FLOW_H + c];
            s.O[r0 + g][c + 1] = acc[nt][1] + bias[2 * FLOW_H + c + 1];
            s.O[r0 + g + 8][c] = acc[nt][2] + bias[2 * FLOW_H + c];
            s.O[r0 + g + 8][c + 1] = acc[nt][3] + bias[2 * FLOW_H + c + 1];
        }
    }
    pair_sync(pair);
}

// 16-byte asynchronous global -> shared copies (cp.async, completion per thread)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int COLS>
__device__ __forceinline__ void load_tile_async(__nv_bfloat16 *dst, int ld, const __nv_bfloat16 *src, int rows)
{
    constexpr int VPR = COLS / 8;
    const int nv = rows * VPR;
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        const int r = i / VPR, c = (i % VPR) * 8;
        cp_async16(dst + r * ld + c, src + (size_t)i * 8);
    }
}

// the generative-direction weights of one layer and its biases b1, b2 (float, 16-byte
// aligned in the parameter vector) into buffer buf, as one copy group; b3 (2d floats)
// is copied with plain loads
template <class S>
__device__ __forceinline__ void load_layer_weights_async(S &s, const __nv_bfloat16 *wl, const float *P, int d, int buf)
{
    load_tile_async<16>(s.W1n[buf], LDA_S, wl + WB_W1N, FLOW_H);
    load_tile_async<FLOW_H>(s.W2n[buf], LDH_S, wl + WB_W2N, FLOW_H);
    load_tile_async<FLOW_H>(s.W3n[buf], LDH_S, wl + WB_W3N, 32);
    // a layer's floats start on a 16-byte boundary when d is even (odd d: plain loads)
    const bool aligned = ((reinterpret_cast<uintptr_t>(P + pl_b1(d)) | reinterpret_cast<uintptr_t>(P + pl_b2(d))) & 15) == 0;
    if (aligned) {
        for (int i = threadIdx.x; i < FLOW_H / 4; i += blockDim.x) {
            cp_async16(s.bias[buf] + 4 * i, P + pl_b1(d) + 4 * i);
            cp_async16(s.bias[buf] + FLOW_H + 4 * i, P + pl_b2(d) + 4 * i);
        }
    } else {
        for (int i = threadIdx.x; i < FLOW_H; i += blockDim.x) {
            s.bias[buf][i] = P[pl_b1(d) + i];
            s.bias[buf][FLOW_H + i] = P[pl_b2(d) + i];
        }
    }
    cp_async_commit();
    for (int i = threadIdx.x; i < 32; i += blockDim.x) { s.bias[buf][2 * FLOW_H + i] = (i < 2 * d) ? P[pl_b3(d) + i] : 0.f; }
}

// S tanh(o / S) with one exponential: tanh|u| = 1 - 2 / (e^{2|u|} + 1), sign restored
__device__ __forceinline__ float soft_clamp(float o)
{
    const float u = fabsf(o) * (2.f / FLOW_SMAX);
    const float th = 1.f - __fdividef(2.f, __expf(u) + 1.f);
    return copysignf(FLOW_SMAX * th, o);
}

// sum over the 32 lanes of a warp
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) { v += __shfl_xor_sync(0xffffffffu, v, m); }
    return v;
}

// Each pair of warps (w, w + 7) owns 16 rows of the tile through all layers (load, MLP,
// coupling, output): the two warps form half of each GEMM's columns and split the
// element-wise work, so within a layer a pair synchronises only with itself (named
// barriers); one block barrier per layer publishes the layer's weights (prefetched with
// cp.async during the previous layer) and frees the other weight buffer for the next
// prefetch.  Two warps per 16 rows (14 per SM) hide the latency of the dependent GEMM
// chain that one warp per 16 rows left exposed.
__global__ void __launch_bounds__(FLOW_PASS_THREADS, 1) flow_pass_kernel(FlowArgs f)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FlowSmem &s = *(FlowSmem *)smem_raw;
    const int base = blockIdx.x * FLOW_PASS_ROWS;
    const int D = f.D, d = f.d;
    const int rows = min(FLOW_PASS_ROWS, f.n - base);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, pair = warp % FLOW_PASS_PAIRS, half = warp / FLOW_PASS_PAIRS, r0 = pair * 16;
    const float invd = 1.f / (float)d;
    if (f.in_cm || f.in_cmf || f.zgen) { // chain-minor walkers (coalesced over the rows) or drawn z
        for (int i = threadIdx.x; i < D * FLOW_PASS_ROWS; i += blockDim.x) {
            const int c = i / FLOW_PASS_ROWS, r = i % FLOW_PASS_ROWS;
            float v = (r < rows) ? flow_input(f, base + r, c) : 0.f;
            if (f.dir == 1) { v = (v - f.mu[c]) * __expf(-f.logsig[c]); }
            s.Y[r][c] = v;
        }
        __syncthreads();
    } else { // the pair's rows of the tile (rows beyond n are zero), eight per warp
        for (int r = r0 + 8 * half; r < r0 + 8 * half + 8; ++r) {
            if (lane < D) {
                float v = (r < rows) ? f.in[(int64_t)(base + r) * D + lane] : 0.f;
                if (f.dir == 1) { v = (v - f.mu[lane]) * __expf(-f.logsig[lane]); } // density: undo the base affine first
                s.Y[r][lane] = v;
            }
        }
    }
    if (half == 0 && lane < 16) { s.logdet[r0 + lane] = 0.f; }
    for (int i = threadIdx.x; i < f.L * D; i += blockDim.x) { s.perm[i] = f.perm[i]; }
    auto layer_of = [&](int step) { return (f.dir == 0) ? step : f.L - 1 - step; };
    auto params_of = [&](int step) { return f.theta + (int64_t)layer_of(step) * f.pstride; };
    load_layer_weights_async(s, f.wb + (int64_t)layer_of(0) * f.wstride, params_of(0), d, 0);
    for (int step = 0; step < f.L; ++step) {
        const int l = layer_of(step);
        const int buf = step & 1;
        const int *perm = s.perm + l * D;
        cp_async_wait<0>(); // this layer's weights and biases (issued during the previous layer) have arrived
        __syncthreads();    // ... for every thread; and every warp has left the previous layer
        if (step + 1 < f.L) {
            load_layer_weights_async(s, f.wb + (int64_t)layer_of(step + 1) * f.wstride, params_of(step + 1), d, buf ^ 1);
        }
        // a-half of the pair's rows as bf16 (columns d..15 zero), eight rows per warp
        {
            const int pa = (lane & 15) < d ? perm[lane & 15] : 0;
            for (int r = r0 + 8 * half + (lane >> 4); r < r0 + 8 * half + 8; r += 2) {
                const int c = lane & 15;
                s.A[r * LDA_S + c] = __float2bfloat16_rn(c < d ? s.Y[r][pa] : 0.f);
            }
        }
        pair_sync(pair);
        pair_layer_mlp(s, r0, pair, half, buf);
        // coupling of the pair's 16 rows x d columns, (row, column) pairs spread over its 64 lanes
        for (int i = lane + 32 * half; i < 16 * d; i += 64) {
            const int q = (int)(((float)i + 0.5f) * invd);
            const int r = r0 + q, j = i - q * d;
            const float sj = soft_clamp(s.O[r][j]);
            const float tj = s.O[r][d + j];
            const int pb = perm[d + j];
            const float bin = s.Y[r][pb];
            const float bout = (f.dir == 0) ? fmaf(bin, __expf(sj), tj) : (bin - tj) * __expf(-sj);
            if (f.tape && r < rows) {
                float *tp = f.tape + ((int64_t)l * f.n + base + r) * 4 * d;
                tp[j] = s.Y[r][perm[j]];  // a
                tp[d + j] = bout;         // b (density direction: the layer's output half)
                tp[2 * d + j] = sj;
                tp[3 * d + j] = tj;
            }
            s.Y[r][pb] = bout;
            s.O[r][j] = sj; // kept for the row's log-determinant below
        }
        pair_sync(pair);
        if (half == 0 && lane < 16) {
            float ld = 0.f;
            for (int j = 0; j < d; ++j) { ld += s.O[r0 + lane][j]; }
            s.logdet[r0 + lane] += ld;
        }
    }
    pair_sync(pair); // the pair's log-determinants are complete
    // output and log q of the warp's rows
    float ls = 0.f;
    for (int c = 0; c < D; ++c) { ls += f.logsig[c]; }
    for (int r = r0 + half; r < min(r0 + 16, rows); r += 2) {
        float zz = 0.f;
        if (lane < D) {
            float z, o;
            if (f.dir == 0) { // z was the input
                z = flow_input(f, base + r, lane);
                o = f.mu[lane] + __expf(f.logsig[lane]) * s.Y[r][lane];
            } else {
                z = s.Y[r][lane];
                o = z;
            }
            zz = z * z;
            if (f.out) { f.out[(int64_t)(base + r) * D + lane] = o; }
            if (f.out_cm) { s.Y[r][lane] = o; } // stored chain-minor below
        }
        zz = warp_sum(zz);
        if (lane == 0) { f.logq[base + r] = -0.5f * zz - 0.91893853320467274f * D - s.logdet[r] - ls; }
    }
    if (f.out_cm) { // coalesced over the rows, one coordinate at a time
        __syncthreads();
        for (int i = threadIdx.x; i < D * FLOW_PASS_ROWS; i += blockDim.x) {
            const int c = i / FLOW_PASS_ROWS, r = i % FLOW_PASS_ROWS;
            if (r < rows) { f.out_cm[(int64_t)c * f.cm_stride + base + r] = s.Y[r][c]; }
        }
    }
}

// ------------------------------------------------------------------------
// register-fused pass: one warp carries 16 rows through every layer, activations in registers
// ------------------------------------------------------------------------
// The m16n8k16 accumulator fragment of two adjacent 8-column tiles (thread: rows g, g + 8,
// columns 2t, 2t + 1 of each) is, converted to bf16, the A fragment of one 16-wide k slice of
// the next product (rows g, g + 8, k 2t, 2t + 1 and 8 + 2t, 9 + 2t).  So a warp forms
// h1 = relu(a W1 + b1) for its 16 rows in all 128 columns, turns it into the A fragments of
// the second product without a shared-memory round trip, does the same with h2 for the
// third, and only the layer output o = (s, t) (16 x 32 floats) passes through shared memory
// for the coupling.  Warps never wait on one another inside a layer: the block meets once per
// layer to switch the double-buffered weights (prefetched with cp.async, as in
// flow_pass_kernel).  Without the hidden tiles in shared memory a CTA holds up to 16 warps
// (256 rows), so two row sets (the density of the walkers and of the proposals) run in one
// launch with the SMs' warps doubled.  The products and their roundings are those of
// flow_pass_kernel (same bf16 operands, same k order per output), element for element.
#define FLOW_FUSED_MAXW 16
struct FlowFusedSmem {
    __nv_bfloat16 W1n[2][FLOW_H * LDA_S];
    __nv_bfloat16 W2n[2][FLOW_H * LDH_S];
    __nv_bfloat16 W3n[2][32 * LDH_S];
    float bias[2][2 * FLOW_H + 32];
    int perm[FLOW_MAXL * FLOW_MAXD];
    float Y[FLOW_FUSED_MAXW * 16][FLOW_MAXD + 1]; // the rows' coordinates
    float O[FLOW_FUSED_MAXW][16][FLOW_MAXD + 1];  // each warp's layer output, then s
    float logdet[FLOW_FUSED_MAXW * 16];
};

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi)
{
    return pack2(__float2bfloat16_rn(lo), __float2bfloat16_rn(hi));
}

// C[16 x 8 NT] += A[16 x 16 KS] B: A as register fragments (one x4 per k slice), B "n-major"
// in shared memory (element (k, n) at Bn[n * ldb + k]) through ldmatrix, as warp_gemm
template <int KS, int NT>
__device__ __forceinline__ void frag_gemm(const uint32_t (&a)[KS][4], const __nv_bfloat16 *Bn, int ldb, float (&acc)[NT][4])
{
    const int lane = threadIdx.x & 31, mi = lane >> 3, rr = lane & 7;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
#pragma unroll
        for (int nt = 0; nt < NT; nt += 2) {
            uint32_t b0, b1, b2, b3;
            ldmatrix_x4(b0, b1, b2, b3, Bn + ((nt + (mi >> 1)) * 8 + rr) * ldb + ks * 16 + (mi & 1) * 8);
            mma_bf16(acc[nt], a[ks][0], a[ks][1], a[ks][2], a[ks][3], b0, b1);
            mma_bf16(acc[nt + 1], a[ks][0], a[ks][1], a[ks][2], a[ks][3], b2, b3);
        }
    }
}

// relu(acc + bias) of the 128 columns as bf16 A fragments of the next product (8 k slices)
__device__ __forceinline__ void frag_relu_to_a(const float (&acc)[16][4], const float *bias, uint32_t (&h)[8][4])
{
    const int t = threadIdx.x & 3;
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        const int c0 = 16 * kk + 2 * t, c1 = c0 + 8;
        const float *x0 = acc[2 * kk], *x1 = acc[2 * kk + 1];
        h[kk][0] = pack_bf2(fmaxf(x0[0] + bias[c0], 0.f), fmaxf(x0[1] + bias[c0 + 1], 0.f));
        h[kk][1] = pack_bf2(fmaxf(x0[2] + bias[c0], 0.f), fmaxf(x0[3] + bias[c0 + 1], 0.f));
        h[kk][2] = pack_bf2(fmaxf(x1[0] + bias[c1], 0.f), fmaxf(x1[1] + bias[c1 + 1], 0.f));
        h[kk][3] = pack_bf2(fmaxf(x1[2] + bias[c1], 0.f), fmaxf(x1[3] + bias[c1 + 1], 0.f));
    }
}

__global__ void __launch_bounds__(FLOW_FUSED_MAXW * 32, 1) flow_pass_fused_kernel(FlowArgs f)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FlowFusedSmem &s = *(FlowFusedSmem *)smem_raw;
    const int rows_cta = 16 * (int)(blockDim.x >> 5);
    const int base = blockIdx.x * rows_cta;
    const int ntot = f.n + f.nb;
    const int D = f.D, d = f.d;
    const int rows = min(rows_cta, ntot - base);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t4 = lane & 3, r0 = warp * 16;
    const float invd = 1.f / (float)d;
    for (int i = threadIdx.x; i < D * rows_cta; i += blockDim.x) { // coordinate-major: coalesced over the rows
        const int c = i / rows_cta, r = i % rows_cta;
        float v = 0.f;
        if (r < rows) {
            if (f.in_cm || f.in_cmf || f.zgen || base + r >= f.n) { v = flow_input(f, base + r, c); }
            else { v = f.in[(int64_t)(base + r) * D + c]; }
        }
        if (f.dir == 1) { v = (v - f.mu[c]) * __expf(-f.logsig[c]); } // density: undo the base affine first
        s.Y[r][c] = v;
    }
    for (int i = threadIdx.x; i < rows_cta; i += blockDim.x) { s.logdet[i] = 0.f; }
    for (int i = threadIdx.x; i < f.L * D; i += blockDim.x) { s.perm[i] = f.perm[i]; }
    auto layer_of = [&](int step) { return (f.dir == 0) ? step : f.L - 1 - step; };
    auto params_of = [&](int step) { return f.theta + (int64_t)layer_of(step) * f.pstride; };
    load_layer_weights_async(s, f.wb + (int64_t)layer_of(0) * f.wstride, params_of(0), d, 0);
    float (*O)[FLOW_MAXD + 1] = s.O[warp];
    for (int step = 0; step < f.L; ++step) {
        const int l = layer_of(step);
        const int buf = step & 1;
        const int *perm = s.perm + l * D;
        cp_async_wait<0>(); // this layer's weights and biases (issued during the previous layer) have arrived
        __syncthreads();    // ... for every thread; and every warp has left the previous layer
        if (step + 1 < f.L) {
            load_layer_weights_async(s, f.wb + (int64_t)layer_of(step + 1) * f.wstride, params_of(step + 1), d, buf ^ 1);
        }
        const float *bias = s.bias[buf];
        uint32_t h[8][4];
        { // h1: the a-half (columns d..15 zero) as the A fragment of one k slice
            uint32_t a[1][4];
            const int ca = 2 * t4, cb = 8 + 2 * t4;
            const float *ya = s.Y[r0 + g], *yb = s.Y[r0 + g + 8];
            auto av = [&](const float *y, int c) { return c < d ? y[perm[c]] : 0.f; };
            a[0][0] = pack_bf2(av(ya, ca), av(ya, ca + 1));
            a[0][1] = pack_bf2(av(yb, ca), av(yb, ca + 1));
            a[0][2] = pack_bf2(av(ya, cb), av(ya, cb + 1));
            a[0][3] = pack_bf2(av(yb, cb), av(yb, cb + 1));
            float acc[16][4];
            zero_acc(acc);
            frag_gemm<1, 16>(a, s.W1n[buf], LDA_S, acc);
            frag_relu_to_a(acc, bias, h);
        }
        { // h2
            float acc[16][4];
            zero_acc(acc);
            frag_gemm<8, 16>(h, s.W2n[buf], LDH_S, acc);
            frag_relu_to_a(acc, bias + FLOW_H, h);
        }
        { // o = h2 W3 + b3 (32 columns; 2d used)
            float acc[4][4];
            zero_acc(acc);
            frag_gemm<8, 4>(h, s.W3n[buf], LDH_S, acc);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int c = nt * 8 + 2 * t4;
                O[g][c] = acc[nt][0] + bias[2 * FLOW_H + c];
                O[g][c + 1] = acc[nt][1] + bias[2 * FLOW_H + c + 1];
                O[g + 8][c] = acc[nt][2] + bias[2 * FLOW_H + c];
                O[g + 8][c + 1] = acc[nt][3] + bias[2 * FLOW_H + c + 1];
            }
        }
        __syncwarp();
        // coupling of the warp's 16 rows x d columns, (row, column) pairs spread over its lanes
        for (int i = lane; i < 16 * d; i += 32) {
            const int q = (int)(((float)i + 0.5f) * invd);
            const int r = r0 + q, j = i - q * d;
            const float sj = soft_clamp(O[q][j]);
            const float tj = O[q][d + j];
            const int pb = perm[d + j];
            const float bin = s.Y[r][pb];
            const float bout = (f.dir == 0) ? fmaf(bin, __expf(sj), tj) : (bin - tj) * __expf(-sj);
            if (f.tape && r < rows) {
                float *tp = f.tape + ((int64_t)l * f.n + base + r) * 4 * d;
                tp[j] = s.Y[r][perm[j]];  // a
                tp[d + j] = bout;         // b (density direction: the layer's output half)
                tp[2 * d + j] = sj;
                tp[3 * d + j] = tj;
            }
            s.Y[r][pb] = bout;
            O[q][j] = sj; // kept for the row's log-determinant below
        }
        __syncwarp();
        if (lane < 16) {
            float ld = 0.f;
            for (int j = 0; j < d; ++j) { ld += O[lane][j]; }
            s.logdet[r0 + lane] += ld;
        }
        __syncwarp();
    }
    // output and log q of the warp's rows
    float ls = 0.f;
    for (int c = 0; c < D; ++c) { ls += f.logsig[c]; }
    for (int r = r0; r < min(r0 + 16, rows); ++r) {
        float zz = 0.f;
        const int row = base + r;
        if (lane < D) {
            float z, o;
            if (f.dir == 0) { // z was the input
                z = (f.in_cm || f.in_cmf || f.zgen || row >= f.n) ? flow_input(f, row, lane) : f.in[(int64_t)row * D + lane];
                o = f.mu[lane] + __expf(f.logsig[lane]) * s.Y[r][lane];
            } else {
                z = s.Y[r][lane];
                o = z;
            }
            zz = z * z;
            if (f.out && row < f.n) { f.out[(int64_t)row * D + lane] = o; }
            if (f.out_cm) { s.Y[r][lane] = o; } // stored chain-minor below
        }
        zz = warp_sum(zz);
        if (lane == 0) {
            const float lq = -0.5f * zz - 0.91893853320467274f * D - s.logdet[r] - ls;
            if (row < f.n) { f.logq[row] = lq; } else { f.logq_b[row - f.n] = lq; }
        }
    }
    if (f.out_cm) { // coalesced over the rows, one coordinate at a time (first set only)
        __syncthreads();
        for (int i = threadIdx.x; i < D * rows_cta; i += blockDim.x) {
            const int c = i / rows_cta, r = i % rows_cta;
            if (r < rows && base + r < f.n) { f.out_cm[(int64_t)c * f.cm_stride + base + r] = s.Y[r][c]; }
        }
    }
}

// ------------------------------------------------------------------------
// 5th-generation tensor cores (tcgen05): MMA issued by one thread from shared-memory
// operand descriptors, accumulator in tensor memory (TMEM), read back with tcgen05.ld
// ------------------------------------------------------------------------
// Operands are bf16, K-major (k contiguous), in the no-swizzle canonical layout: 8 x 8
// "core matrices" (8 rows of 16 bytes, 128 contiguous bytes), element (r, k) of an R x K
// operand at core matrix (r / 8) * (K / 8) + k / 8, byte (r % 8) * 16 + (k % 8) * 2 within it.
// So the descriptor's leading-dimension offset (next core matrix along K) is 128 bytes and
// its stride-dimension offset (next 8 rows) K * 16 bytes; an MMA of K = 16 covers two core
// matrices along K, and the next one starts 256 bytes further.

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of an R x K canonical operand
__host__ __device__ __forceinline__ uint32_t canon_off(int r, int k, int K)
{
    return (uint32_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading / stride byte offsets (16-byte
// units), descriptor version 1 (bits 46-47), no swizzle (layout type 0)
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor of kind::f16: f32 accumulator (bits 4-5 = 1), A and B bf16
// (bits 7-9 and 10-12 = 1), both K-major, N / 8 at bit 17, M / 16 at bit 24
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B^T for one K = 16 slice (issued by one thread)
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
                 : "memory");
}
// the issuing thread's MMAs so far arrive on the mbarrier when they complete
__device__ __forceinline__ void umma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// wait for the completion of the mbarrier phase with parity `parity`: 4,096 polls back to
// back (an MMA round trip completes within them), then polls 64 ns apart, at most `limit` in
// all (about 2^24 x 64 ns = 1 s); false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint32_t limit = 1u << 24)
{
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(mbar), "r"(parity)
                     : "memory");
        if (done) { return true; }
        if (i >= 4096) { __nanosleep(64); }
    }
    return false;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// shared-memory writes of the generic proxy (st.shared, cp.async) visible to the tensor core
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// TMEM allocation by one whole warp: the address is written to shared memory at dst
__device__ __forceinline__ void tmem_alloc(uint32_t dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(dst), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
// 16 consecutive f32 columns of the warp's 32 TMEM lanes (lane = the thread's row)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                 "%14, %15}, [%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) { v[i] = __uint_as_float(r[i]); }
}

// 32 consecutive f32 columns of the warp's 32 TMEM lanes, without the wait (tmem_ld_wait)
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t (&r)[32])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                 "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                   "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                   "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// Self-test of the path: D[128][N] = A[128][K] B[N][K]^T, one CTA of 128 threads (thread t
// reads row t of D from TMEM lane t).  N a multiple of 16 in [16, 256], K a multiple of 16 in
// [16, 256]; status bit 0 set when the MMA's completion was not seen within the wait limit.
__global__ void __launch_bounds__(128, 1) flow_tc_selftest_kernel(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D,
                                                                   int N, int K, int *status)
{
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char *As = sm, *Bs = sm + 128 * K * 2;
    uint64_t *mbar = (uint64_t *)(Bs + N * K * 2);
    uint32_t *tslot = (uint32_t *)(mbar + 1);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int kc = K / 8;
    for (int i = t; i < 128 * kc; i += 128) {
        const int r = i / kc, c = i % kc;
        *(uint4 *)(As + canon_off(r, 8 * c, K)) = *(const uint4 *)(A + (size_t)r * K + 8 * c);
    }
    for (int i = t; i < N * kc; i += 128) {
        const int r = i / kc, c = i % kc;
        *(uint4 *)(Bs + canon_off(r, 8 * c, K)) = *(const uint4 *)(B + (size_t)r * K + 8 * c);
    }
    uint32_t ncols = 32;
    while (ncols < (uint32_t)N) { ncols <<= 1; }
    if (t == 0) { mbar_init(smem_addr(mbar), 1); }
    if (warp == 0) { tmem_alloc(smem_addr(tslot), ncols); }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tslot;
    if (t == 0) {
        const uint32_t idesc = umma_idesc_bf16(128, N);
        for (int ks = 0; ks < K / 16; ++ks) {
            const uint64_t ad = umma_desc(smem_addr(As) + 256 * ks, 128, 16 * K);
            const uint64_t bd = umma_desc(smem_addr(Bs) + 256 * ks, 128, 16 * K);
            umma_bf16(taddr, ad, bd, idesc, ks > 0 ? 1u : 0u);
        }
        umma_commit(smem_addr(mbar));
    }
    const bool ok = mbar_wait(smem_addr(mbar), 0);
    tc_fence_after();
    if (ok) {
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) { D[(size_t)t * N + c0 + j] = v[j]; }
        }
    } else if (lane == 0) {
        atomicOr(status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) { tmem_dealloc(taddr, ncols); }
}

// ------------------------------------------------------------------------
// the pass on tcgen05: one CTA = 128 samples (the MMA tile's M), 8 warps
// ------------------------------------------------------------------------
// Per layer (the flow definition above), in tensor memory columns [0, 256):
//   MMA1  D[0,128)   = A1 [128 x 16]  * W1n^T   (one K = 16 slice)
//   epilogue: h1 = relu(D + b1) -> bf16 -> A2 (canonical layout)
//   MMA2  D[128,256) = A2 [128 x 128] * W2n^T   (eight slices)
//   epilogue: h2 = relu(D + b2) -> bf16 -> A2 (MMA2 has completed)
//   MMA3  D[0,32)    = A2 [128 x 128] * W3n^T   (N = 32: rows 2d.. of W3n are zero)
//   epilogue: o = D + b3, the coupling of each row in shared memory.
// Warp w reads TMEM lanes 32 (w % 4) .. + 31, i.e. the rows of its quarter, and in the hidden
// epilogues the column half w / 4 of them (two 32-column loads, one wait); the row's
// coupling and output belong to the thread of warp w < 4.  One thread issues the MMAs and
// commits them to an mbarrier that every thread waits on (bounded).  The next layer's
// weights arrive by cp.async into the second of two buffers while the layer computes.  The
// dot products run in the tensor core's order rather than the mma.sync kernel's, so the two
// kernels agree to f32 accumulation rounding (both against the oracle at bf16 tolerance).
#define FTC_ROWS 128
#define FTC_THREADS 256
#define FTC_LDY (FLOW_MAXD + 1)
struct FlowTcSmem {
    __nv_bfloat16 W2[2][FLOW_H * FLOW_H]; // canonical [128][128]
    __nv_bfloat16 A2[FTC_ROWS * FLOW_H];  // canonical [128][128]: h1, then h2
    __nv_bfloat16 W3[2][32 * FLOW_H];     // canonical [32][128]
    __nv_bfloat16 W1[2][FLOW_H * 16];     // canonical [128][16]
    __nv_bfloat16 A1[FTC_ROWS * 16];      // canonical [128][16]
    float Y[FTC_ROWS * FTC_LDY];          // the rows' coordinates
    float O[FTC_ROWS * FTC_LDY];          // the rows' MLP outputs o = (s, t) of the layer
    float bias[2][2 * FLOW_H + 32];
    int perm[FLOW_MAXL * FLOW_MAXD];
    uint64_t mbar;
    uint32_t tslot;
};

// one layer's weights (canonical layouts) and biases into buffer buf, as one cp.async group
__device__ __forceinline__ void tc_load_layer(FlowTcSmem &s, const __nv_bfloat16 *wl, const float *P, int d, int buf)
{
    for (int i = threadIdx.x; i < FLOW_H * 2; i += blockDim.x) { // W1n [128][16]: 2 chunks per row
        const int r = i >> 1, c = i & 1;
        cp_async16((unsigned char *)s.W1[buf] + canon_off(r, 8 * c, 16), wl + WB_W1N + r * 16 + 8 * c);
    }
    for (int i = threadIdx.x; i < FLOW_H * 16; i += blockDim.x) { // W2n [128][128]: 16 chunks per row
        const int r = i >> 4, c = i & 15;
        cp_async16((unsigned char *)s.W2[buf] + canon_off(r, 8 * c, FLOW_H), wl + WB_W2N + r * FLOW_H + 8 * c);
    }
    for (int i = threadIdx.x; i < 32 * 16; i += blockDim.x) { // W3n [32][128]
        const int r = i >> 4, c = i & 15;
        cp_async16((unsigned char *)s.W3[buf] + canon_off(r, 8 * c, FLOW_H), wl + WB_W3N + r * FLOW_H + 8 * c);
    }
    const bool aligned = ((reinterpret_cast<uintptr_t>(P + pl_b1(d)) | reinterpret_cast<uintptr_t>(P + pl_b2(d))) & 15) == 0;
    if (aligned) {
        for (int i = threadIdx.x; i < FLOW_H / 4; i += blockDim.x) {
            cp_async16(s.bias[buf] + 4 * i, P + pl_b1(d) + 4 * i);
            cp_async16(s.bias[buf] + FLOW_H + 4 * i, P + pl_b2(d) + 4 * i);
        }
    } else {
        for (int i = threadIdx.x; i < FLOW_H; i += blockDim.x) {
            s.bias[buf][i] = P[pl_b1(d) + i];
            s.bias[buf][FLOW_H + i] = P[pl_b2(d) + i];
        }
    }
    cp_async_commit();
    for (int i = threadIdx.x; i < 32; i += blockDim.x) { s.bias[buf][2 * FLOW_H + i] = (i < 2 * d) ? P[pl_b3(d) + i] : 0.f; }
}

// relu(D + bias) of 64 columns [c0, c0 + 64) of the thread's row (TMEM lane) into A2 as bf16
__device__ __forceinline__ void tc_hidden_epilogue(FlowTcSmem &s, uint32_t tlane, uint32_t tcol, int c0, const float *bias,
                                                   int row)
{
    unsigned char *dst = (unsigned char *)s.A2;
    uint32_t r0[32], r1[32];
    tmem_ld32_nowait(tlane + tcol + (uint32_t)c0, r0);
    tmem_ld32_nowait(tlane + tcol + (uint32_t)c0 + 32, r1);
    tmem_ld_wait();
#pragma unroll
    for (int q = 0; q < 8; ++q) { // 8 columns (16 bytes of bf16) per store
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = 8 * q + 2 * j; // column c0 + k within the 64
            const float v0 = __uint_as_float(k < 32 ? r0[k] : r1[k - 32]);
            const float v1 = __uint_as_float(k + 1 < 32 ? r0[k + 1] : r1[k + 1 - 32]);
            const float lo = fmaxf(v0 + bias[c0 + k], 0.f), hi = fmaxf(v1 + bias[c0 + k + 1], 0.f);
            w[j] = pack2(__float2bfloat16_rn(lo), __float2bfloat16_rn(hi));
        }
        *(uint4 *)(dst + canon_off(row, c0 + 8 * q, FLOW_H)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// every thread's shared-memory writes done and visible to the tensor core, and the previous
// tensor-memory reads finished, before thread 0 issues the next MMAs
__device__ __forceinline__ void tc_handoff()
{
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

__global__ void __launch_bounds__(FTC_THREADS, 1) flow_pass_tc_kernel(FlowArgs f, int *status)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FlowTcSmem &s = *(FlowTcSmem *)smem_raw;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int quad = warp & 3, half = warp >> 2;
    const int rl = 32 * quad + lane; // the thread's row in the tile = its TMEM lane
    const int base = blockIdx.x * FTC_ROWS, row = base + rl;
    const bool live = row < f.n;
    const bool owner = half == 0; // the row's coupling and output
    const int D = f.D, d = f.d;
    for (int i = t; i < D * FTC_ROWS; i += blockDim.x) { // coordinate-major: coalesced chain-minor reads
        const int c = i / FTC_ROWS, r = i % FTC_ROWS;
        float v = (base + r < f.n) ? flow_input(f, base + r, c) : 0.f;
        if (f.dir == 1) { v = (v - f.mu[c]) * __expf(-f.logsig[c]); } // density: undo the base affine first
        s.Y[r * FTC_LDY + c] = v;
    }
    float *Y = s.Y + rl * FTC_LDY;
    for (int i = t; i < f.L * D; i += blockDim.x) { s.perm[i] = f.perm[i]; }
    const uint32_t mbar = smem_addr(&s.mbar);
    if (t == 0) { mbar_init(mbar, 1); }
    if (warp == 0) { tmem_alloc(smem_addr(&s.tslot), 256); }
    auto layer_of = [&](int step) { return (f.dir == 0) ? step : f.L - 1 - step; };
    auto params_of = [&](int step) { return f.theta + (int64_t)layer_of(step) * f.pstride; };
    tc_load_layer(s, f.wb + (int64_t)layer_of(0) * f.wstride, params_of(0), d, 0);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = s.tslot;
    const uint32_t tlane = taddr + ((uint32_t)(32 * quad) << 16); // this warp's 32 TMEM lanes
    const uint32_t id_h = umma_idesc_bf16(128, FLOW_H), id_o = umma_idesc_bf16(128, 32);
    uint32_t phase = 0;
    bool ok = true;
    float logdet = 0.f;
    for (int step = 0; step < f.L && ok; ++step) {
        const int l = layer_of(step);
        const int buf = step & 1;
        const int *perm = s.perm + l * D;
        const float *bias = s.bias[buf];
        cp_async_wait<0>(); // this layer's weights (issued during the previous layer) have arrived
        __syncthreads();    // and the previous layer's coupling (the row owners' Y) is complete
        { // the a-half of the row as bf16 (columns d..15 zero): columns 8 half .. 8 half + 7
            uint32_t w[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = 8 * half + 2 * j;
                const float lo = (k < d) ? Y[perm[k]] : 0.f, hi = (k + 1 < d) ? Y[perm[k + 1]] : 0.f;
                w[j] = pack2(__float2bfloat16_rn(lo), __float2bfloat16_rn(hi));
            }
            *(uint4 *)((unsigned char *)s.A1 + canon_off(rl, 8 * half, 16)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
        tc_handoff();
        if (step + 1 < f.L) { // the other buffer was last read by the previous layer's MMAs, which have completed
            tc_load_layer(s, f.wb + (int64_t)layer_of(step + 1) * f.wstride, params_of(step + 1), d, buf ^ 1);
        }
        // h1
        if (t == 0) {
            umma_bf16(taddr, umma_desc(smem_addr(s.A1), 128, 16 * 16), umma_desc(smem_addr(s.W1[buf]), 128, 16 * 16), id_h, 0u);
            umma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase));
        phase ^= 1;
        if (!ok) { break; }
        tc_fence_after();
        tc_hidden_epilogue(s, tlane, 0, 64 * half, bias, rl);
        tc_handoff();
        // h2
        if (t == 0) {
            for (int ks = 0; ks < FLOW_H / 16; ++ks) {
                umma_bf16(taddr + 128, umma_desc(smem_addr(s.A2) + 256 * ks, 128, 16 * FLOW_H),
                          umma_desc(smem_addr(s.W2[buf]) + 256 * ks, 128, 16 * FLOW_H), id_h, ks > 0 ? 1u : 0u);
            }
            umma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase));
        phase ^= 1;
        if (!ok) { break; }
        tc_fence_after();
        tc_hidden_epilogue(s, tlane, 128, 64 * half, bias + FLOW_H, rl);
        tc_handoff();
        // o
        if (t == 0) {
            for (int ks = 0; ks < FLOW_H / 16; ++ks) {
                umma_bf16(taddr, umma_desc(smem_addr(s.A2) + 256 * ks, 128, 16 * FLOW_H),
                          umma_desc(smem_addr(s.W3[buf]) + 256 * ks, 128, 16 * FLOW_H), id_o, ks > 0 ? 1u : 0u);
            }
            umma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase));
        phase ^= 1;
        if (!ok) { break; }
        tc_fence_after();
        if (owner) {
            float *O = s.O + rl * FTC_LDY; // o of the row (indexed by the runtime half width d)
            {
                uint32_t r[32];
                tmem_ld32_nowait(tlane, r);
                tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 32; ++j) { O[j] = __uint_as_float(r[j]) + bias[2 * FLOW_H + j]; }
            }
            // coupling of the row
            float *tp = (f.tape && live) ? f.tape + ((int64_t)l * f.n + row) * 4 * d : nullptr;
            for (int j = 0; j < d; ++j) {
                const float sj = soft_clamp(O[j]);
                const float tv = O[d + j];
                const int pb = perm[d + j];
                const float bin = Y[pb];
                const float bout = (f.dir == 0) ? fmaf(bin, __expf(sj), tv) : (bin - tv) * __expf(-sj);
                if (tp) {
                    tp[j] = Y[perm[j]];
                    tp[d + j] = bout;
                    tp[2 * d + j] = sj;
                    tp[3 * d + j] = tv;
                }
                Y[pb] = bout;
                logdet += sj;
            }
        }
    }
    if (!ok && t == 0) { atomicOr(status, 1); }
    cp_async_wait<0>(); // a prefetch issued before a failed wait
    tc_fence_before();
    __syncthreads();
    if (warp == 0) { tmem_dealloc(taddr, 256); }
    if (!ok || !live || !owner) { return; }
    // output and log q of the row
    float ls = 0.f;
    for (int c = 0; c < D; ++c) { ls += f.logsig[c]; }
    float zz = 0.f;
    for (int c = 0; c < D; ++c) {
        float z, o;
        if (f.dir == 0) { // z was the input
            z = flow_input(f, row, c);
            o = f.mu[c] + __expf(f.logsig[c]) * Y[c];
        } else {
            z = Y[c];
            o = z;
        }
        zz = fmaf(z, z, zz);
        if (f.out) { f.out[(int64_t)row * D + c] = o; }
        if (f.out_cm) { f.out_cm[(int64_t)c * f.cm_stride + row] = o; }
    }
    f.logq[row] = -0.5f * zz - 0.91893853320467274f * D - logdet - ls;
}

// ------------------------------------------------------------------------
// backward: gradient of -mean log q through the density direction
// ------------------------------------------------------------------------
struct FlowBwdSmem {
    float G[FLOW_ROWS][FLOW_MAXD + 1];     // d loss / d y of the current level
    __nv_bfloat16 A[FLOW_ROWS * LDA_S];
    __nv_bfloat16 H1[FLOW_ROWS * LDH_S];
    __nv_bfloat16 H2[FLOW_ROWS * LDH_S];
    __nv_bfloat16 GO[FLOW_ROWS * LDO_S];  // d loss / d o (bf16)
    __nv_bfloat16 GH2[FLOW_ROWS * LDH_S]; // d loss / d h2 (pre-activation)
    __nv_bfloat16 GH1[FLOW_ROWS * LDH_S]; // d loss / d h1 (pre-activation)
    __nv_bfloat16 W1n[FLOW_H * LDA_S];
    __nv_bfloat16 W2n[FLOW_H * LDH_S];
    __nv_bfloat16 W3n[FLOW_H * LDO_S];    // W3n [32][LDH_S], later W3t [H][32] with stride LDO_S
    float bias[2 * FLOW_H + 32];
    float red[2 * FLOW_H + 32];           // bias-gradient sums of the tile
};

struct FlowBwdArgs {
    int D, d, L, n;
    float inv_batch;
    const float *z;        // [n][D] output of the density pass
    const float *tape;     // [L][n][4d]
    const int *perm;
    const __nv_bfloat16 *wb;
    const float *theta;
    float *grad;           // float gradient, same layout as theta (zeroed by the caller)
    const float *x;        // [n][D] data (for mu / logsig)
    const float *mu, *logsig;
    int64_t wstride, pstride, base_off; // base_off: offset of mu in theta
};

__global__ void __launch_bounds__(FLOW_THREADS) flow_backward_kernel(FlowBwdArgs f)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FlowBwdSmem &s = *(FlowBwdSmem *)smem_raw;
    const int base = blockIdx.x * FLOW_ROWS;
    const int D = f.D, d = f.d;
    const int rows = min(FLOW_ROWS, f.n - base);
    const int warp = threadIdx.x >> 5, r0 = warp * 16;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int NW = FLOW_THREADS / 32;
    static_assert(FLOW_H == 16 * NW, "dW1 gives each warp 16 of the hidden columns");
    for (int r = warp; r < FLOW_ROWS; r += NW) { // d(0.5|z|^2)/dz / B
        if (lane < D) { s.G[r][lane] = (r < rows) ? f.z[(int64_t)(base + r) * D + lane] * f.inv_batch : 0.f; }
    }
    // weight tiles arrive by cp.async into whichever buffer has just been freed, one copy
    // group each, in the order they are needed: W1n/W2n of the next layer, W3t -> W3n
    // buffer, W2t -> W2n buffer, W1t -> W3n buffer
    load_tile_async<16>(s.W1n, LDA_S, f.wb + WB_W1N, FLOW_H);
    load_tile_async<FLOW_H>(s.W2n, LDH_S, f.wb + WB_W2N, FLOW_H);
    cp_async_commit();
    __syncthreads();
    for (int l = 0; l < f.L; ++l) { // reverse of the density direction
        const int *perm = f.perm + l * D;
        const float *P = f.theta + (int64_t)l * f.pstride;
        float *GP = f.grad + (int64_t)l * f.pstride;
        const __nv_bfloat16 *wl = f.wb + (int64_t)l * f.wstride;
        const __nv_bfloat16 *wnext = (l + 1 < f.L) ? wl + f.wstride : nullptr;
        load_tile_async<32>(s.W3n, LDO_S, wl + WB_W3T, FLOW_H); // W3t [H][32]
        cp_async_commit();
        for (int i = threadIdx.x; i < FLOW_ROWS * 16; i += blockDim.x) {
            const int r = i / 16, c = i % 16;
            const float v = (r < rows && c < d) ? f.tape[((int64_t)l * f.n + base + r) * 4 * d + c] : 0.f;
            s.A[r * LDA_S + c] = __float2bfloat16_rn(v);
        }
        for (int i = threadIdx.x; i < 2 * FLOW_H + 32; i += blockDim.x) { s.red[i] = 0.f; }
        cp_async_wait<1>(); // W1n and W2n of this layer (W3t may still be in flight)
        __syncthreads();
        // recompute h1, h2 (same bf16 GEMMs as the pass kernel)
        for (int i = threadIdx.x; i < FLOW_H; i += blockDim.x) {
            s.bias[i] = P[pl_b1(d) + i];
            s.bias[FLOW_H + i] = P[pl_b2(d) + i];
        }
        __syncthreads();
        {
            float acc[16][4];
            zero_acc(acc);
            warp_gemm<1, 16>(s.A, LDA_S, r0, s.W1n, LDA_S, acc);
            store_act(acc, s.bias, true, s.H1, LDH_S, r0);
        }
        __syncthreads();
        if (wnext) { load_tile_async<16>(s.W1n, LDA_S, wnext + WB_W1N, FLOW_H); } // W1n is free
        cp_async_commit();
        {
            float acc[16][4];
            zero_acc(acc);
            warp_gemm<FLOW_H / 16, 16>(s.H1, LDH_S, r0, s.W2n, LDH_S, acc);
            store_act(acc, s.bias + FLOW_H, true, s.H2, LDH_S, r0);
        }
        __syncthreads();
        load_tile_async<FLOW_H>(s.W2n, LDH_S, wl + WB_W2T, FLOW_H); // W2t [H][H] into the free W2n buffer
        cp_async_commit();
        // coupling backward: g_o = [g_sraw, g_t] for the b half.  Warp w takes rows w, w+8, ...;
        // lane j is output column j, so the tape reads of a row are contiguous and the b3
        // gradient of column j accumulates in lane j's register.
        {
            float gsum = 0.f;
            const int j = lane;
            for (int r = warp; r < FLOW_ROWS; r += FLOW_THREADS / 32) {
                float go = 0.f;
                if (r < rows && j < 2 * d) {
                    const float *tp = f.tape + ((int64_t)l * f.n + base + r) * 4 * d;
                    const int jj = j < d ? j : j - d;
                    const float gb = s.G[r][perm[d + jj]];
                    const float sj = tp[2 * d + jj];
                    if (j < d) {
                        const float gs = -gb * tp[d + jj] + f.inv_batch; // d/ds of (b' - t) e^-s, plus the sum(s) term
                        go = gs * (1.f - (sj / FLOW_SMAX) * (sj / FLOW_SMAX));
                    } else {
                        go = -gb * __expf(-sj);
                    }
                }
                s.GO[r * LDO_S + j] = __float2bfloat16_rn(go);
                gsum += go;
            }
            atomicAdd(&s.red[2 * FLOW_H + j], gsum);
        }
        __syncthreads();
        // b-half gradient passes through: g_b' = g_b e^{-s} (warp per row, lane j)
        for (int r = warp; r < rows; r += NW) {
            if (lane < d) {
                const int bj = perm[d + lane];
                s.G[r][bj] = s.G[r][bj] * __expf(-f.tape[((int64_t)l * f.n + base + r) * 4 * d + 2 * d + lane]);
            }
        }
        // g_h2 = (g_o W3^T) * relu'(h2): W3t [H][32] in the W3n buffer with stride LDO_S
        cp_async_wait<2>(); // W3t (the next layer's W1n and this layer's W2t may still be in flight)
        __syncthreads();
        {
            float acc[16][4];
            zero_acc(acc);
            warp_gemm<2, 16>(s.GO, LDO_S, r0, s.W3n, LDO_S, acc);
#pragma unroll
            for (int nt = 0; nt < 16; ++nt) {
                const int c = nt * 8 + 2 * t;
                float v[4];
                v[0] = __bfloat162float(s.H2[(r0 + g) * LDH_S + c]) > 0.f ? acc[nt][0] : 0.f;
                v[1] = __bfloat162float(s.H2[(r0 + g) * LDH_S + c + 1]) > 0.f ? acc[nt][1] : 0.f;
                v[2] = __bfloat162float(s.H2[(r0 + g + 8) * LDH_S + c]) > 0.f ? acc[nt][2] : 0.f;
                v[3] = __bfloat162float(s.H2[(r0 + g + 8) * LDH_S + c + 1]) > 0.f ? acc[nt][3] : 0.f;
                *(uint32_t *)(s.GH2 + (r0 + g) * LDH_S + c) = pack2(__float2bfloat16_rn(v[0]), __float2bfloat16_rn(v[1]));
                *(uint32_t *)(s.GH2 + (r0 + g + 8) * LDH_S + c) = pack2(__float2bfloat16_rn(v[2]), __float2bfloat16_rn(v[3]));
                const float b0 = sum_over_g(v[0] + v[2]), b1 = sum_over_g(v[1] + v[3]);
                if (g == 0) {
                    atomicAdd(&s.red[FLOW_H + c], b0);
                    atomicAdd(&s.red[FLOW_H + c + 1], b1);
                }
            }
        }
        __syncthreads();
        load_tile_async<FLOW_H>(s.W3n, LDH_S, wl + WB_W1T, 16); // W1t [16][H] into the free W3n buffer
        cp_async_commit();
        // dW3 = h2^T g_o: rows h (16 per warp), 4 n-tiles over the 32 outputs
        {
            float acc[4][4];
            zero_acc(acc);
            warp_gemm_tn<4>(s.H2, LDH_S, r0, s.GO, LDO_S, acc);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int c = nt * 8 + 2 * t;
                if (c < 2 * d) { // 2d is even, so c + 1 < 2d too
                    atomic_add2(&GP[pl_W3(d) + (int64_t)(r0 + g) * 2 * d + c], acc[nt][0], acc[nt][1]);
                    atomic_add2(&GP[pl_W3(d) + (int64_t)(r0 + g + 8) * 2 * d + c], acc[nt][2], acc[nt][3]);
                }
            }
        }
        // g_h1 = (g_h2 W2^T) * relu'(h1): W2t [H][H] in the W2n buffer
        cp_async_wait<1>(); // W2t (W1t may still be in flight)
        __syncthreads();
        {
            float acc[16][4];
            zero_acc(acc);
            warp_gemm<FLOW_H / 16, 16>(s.GH2, LDH_S, r0, s.W2n, LDH_S, acc);
#pragma unroll
            for (int nt = 0; nt < 16; ++nt) {
                const int c = nt * 8 + 2 * t;
                float v[4];
                v[0] = __bfloat162float(s.H1[(r0 + g) * LDH_S + c]) > 0.f ? acc[nt][0] : 0.f;
                v[1] = __bfloat162float(s.H1[(r0 + g) * LDH_S + c + 1]) > 0.f ? acc[nt][1] : 0.f;
                v[2] = __bfloat162float(s.H1[(r0 + g + 8) * LDH_S + c]) > 0.f ? acc[nt][2] : 0.f;
                v[3] = __bfloat162float(s.H1[(r0 + g + 8) * LDH_S + c + 1]) > 0.f ? acc[nt][3] : 0.f;
                *(uint32_t *)(s.GH1 + (r0 + g) * LDH_S + c) = pack2(__float2bfloat16_rn(v[0]), __float2bfloat16_rn(v[1]));
                *(uint32_t *)(s.GH1 + (r0 + g + 8) * LDH_S + c) = pack2(__float2bfloat16_rn(v[2]), __float2bfloat16_rn(v[3]));
                const float b0 = sum_over_g(v[0] + v[2]), b1 = sum_over_g(v[1] + v[3]);
                if (g == 0) {
                    atomicAdd(&s.red[c], b0);
                    atomicAdd(&s.red[c + 1], b1);
                }
            }
        }
        // dW2 = h1^T g_h2: rows h1 (16 per warp) x 128 outputs
        {
            float acc[16][4];
            zero_acc(acc);
            warp_gemm_tn<16>(s.H1, LDH_S, r0, s.GH2, LDH_S, acc);
#pragma unroll
            for (int nt = 0; nt < 16; ++nt) {
                const int c = nt * 8 + 2 * t;
                atomic_add2(&GP[pl_W2(d) + (int64_t)(r0 + g) * FLOW_H + c], acc[nt][0], acc[nt][1]);
                atomic_add2(&GP[pl_W2(d) + (int64_t)(r0 + g + 8) * FLOW_H + c], acc[nt][2], acc[nt][3]);
            }
        }
        __syncthreads();
        // g_a = g_h1 W1^T: W1t [16][H] in the W3n buffer with stride LDH_S
        if (wnext) { load_tile_async<FLOW_H>(s.W2n, LDH_S, wnext + WB_W2N, FLOW_H); } // W2t done: next W2n
        cp_async_commit();
        cp_async_wait<1>(); // W1t (the next layer's W2n may still be in flight)
        __syncthreads();
        {
            float acc[2][4];
            zero_acc(acc);
            warp_gemm<FLOW_H / 16, 2>(s.GH1, LDH_S, r0, s.W3n, LDH_S, acc);
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                const int c = nt * 8 + 2 * t;
                // accumulate into G on the a-half (direct term already there)
                if (c < d) {
                    if (r0 + g < rows) { s.G[r0 + g][perm[c]] += acc[nt][0]; }
                    if (r0 + g + 8 < rows) { s.G[r0 + g + 8][perm[c]] += acc[nt][2]; }
                }
                if (c + 1 < d) {
                    if (r0 + g < rows) { s.G[r0 + g][perm[c + 1]] += acc[nt][1]; }
                    if (r0 + g + 8 < rows) { s.G[r0 + g + 8][perm[c + 1]] += acc[nt][3]; }
                }
            }
        }
        // dW1 = a^T g_h1: the 16 rows of the padded a-half, the 128 outputs split over the
        // warps (16 each), so no warp forms the whole 16 x 128 product while the others wait
        {
            float acc[2][4];
            zero_acc(acc);
            warp_gemm_tn<2>(s.A, LDA_S, 0, s.GH1 + 16 * warp, LDH_S, acc);
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                const int c = 16 * warp + nt * 8 + 2 * t;
                if (g < d) { atomic_add2(&GP[pl_W1(d) + (int64_t)g * FLOW_H + c], acc[nt][0], acc[nt][1]); }
                if (g + 8 < d) { atomic_add2(&GP[pl_W1(d) + (int64_t)(g + 8) * FLOW_H + c], acc[nt][2], acc[nt][3]); }
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < FLOW_H; i += blockDim.x) {
            atomicAdd(&GP[pl_b1(d) + i], s.red[i]);
            atomicAdd(&GP[pl_b2(d) + i], s.red[FLOW_H + i]);
        }
        for (int i = threadIdx.x; i < 2 * d; i += blockDim.x) { atomicAdd(&GP[pl_b3(d) + i], s.red[2 * FLOW_H + i]); }
        __syncthreads();
    }
    // base affine: y_L = (x - mu) exp(-logsig); warp per row, lane c, sums in registers
    float *gmu = f.grad + f.base_off, *gls = f.grad + f.base_off + D;
    float a = 0.f, b = 0.f;
    if (lane < D) {
        const float e = __expf(-f.logsig[lane]);
        for (int r = warp; r < rows; r += NW) {
            const float yl = (f.x[(int64_t)(base + r) * D + lane] - f.mu[lane]) * e;
            a += -s.G[r][lane] * e;
            b += -s.G[r][lane] * yl;
        }
    }
    __syncthreads();
    if (threadIdx.x < 2 * FLOW_MAXD) { s.red[threadIdx.x] = 0.f; }
    __syncthreads();
    if (lane < D) {
        atomicAdd(&s.red[lane], a);
        atomicAdd(&s.red[FLOW_MAXD + lane], b);
    }
    __syncthreads();
    if (threadIdx.x < D) {
        atomicAdd(&gmu[threadIdx.x], s.red[threadIdx.x]);
        atomicAdd(&gls[threadIdx.x], s.red[FLOW_MAXD + threadIdx.x] + (blockIdx.x == 0 ? 1.f : 0.f));
    }
}

__global__ void flow_adam_kernel(float *theta, const float *grad, float *m, float *v, int64_t n, float lr, float b1,
                                 float b2, float eps, float c1, float c2)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * g;
        const float vi = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        theta[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// training minibatch gather: rows idx of src [nsrc][D] into dst [B][D]
__global__ void flow_gather_kernel(const float *src, int64_t nsrc, int D, uint32_t seed, uint32_t step, float *dst, int B)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) { return; }
    const P4 q = philox4x32_10((uint32_t)i, step, 0x5EEDu, 0x7AAu, seed, 0xF10Au);
    const int64_t r = (int64_t)(((uint64_t)q.a * (uint64_t)nsrc) >> 32);
    for (int c = 0; c < D; ++c) { dst[(int64_t)i * D + c] = src[r * D + c]; }
}

// ------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------
struct mcig_flow {
    int D, d, L, device;
    uint64_t seed;
    int64_t np, pstride, base_off;
    float *theta = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wb = nullptr;
    int *perm = nullptr;
    int64_t adam_t = 0;
    cudaStream_t st = nullptr;
    // work buffers
    float *buf_in = nullptr, *buf_out = nullptr, *buf_logq = nullptr, *buf_tape = nullptr, *buf_batch = nullptr;
    int64_t cap = 0, tape_cap = 0, batch_cap = 0;
    // passes on tcgen05 (flow_pass_tc_kernel) or on mma.sync (flow_pass_kernel); status bit 0:
    // a tcgen05 pass did not see an MMA completion within its bounded wait
    int tc = 0;      // pass kernel: 0 register-fused mma.sync, 1 tcgen05, 2 shared-memory mma.sync
    int nsm = 152;   // SMs of the device
    int *status = nullptr;
};

static int flow_err(int code, const std::string &m) { return mcig_set_last_error(code, m.c_str()); }
#define FCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) { return flow_err(MCIG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); } \
    } while (0)

static std::vector<int> flow_perms(int D, int L, uint64_t seed)
{ // splitmix64 Fisher-Yates, as oracle/flow_oracle.py permutations()
    std::vector<int> out;
    for (int l = 0; l < L; ++l) {
        uint64_t s = seed * 0x9E3779B97F4A7C15ULL + (uint64_t)l + 1;
        std::vector<int> p(D);
        for (int i = 0; i < D; ++i) { p[i] = i; }
        for (int i = D - 1; i > 0; --i) {
            s += 0x9E3779B97F4A7C15ULL;
            uint64_t z = s;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
            z = z ^ (z >> 31);
            const int j = (int)(z % (uint64_t)(i + 1));
            std::swap(p[i], p[j]);
        }
        out.insert(out.end(), p.begin(), p.end());
    }
    return out;
}

static int flow_ensure(mcig_flow *f, int64_t n, bool tape)
{
    if (n > f->cap) {
        cudaFree(f->buf_in); cudaFree(f->buf_out); cudaFree(f->buf_logq);
        FCK(cudaMalloc(&f->buf_in, n * f->D * sizeof(float)));
        FCK(cudaMalloc(&f->buf_out, n * f->D * sizeof(float)));
        FCK(cudaMalloc(&f->buf_logq, n * sizeof(float)));
        f->cap = n;
    }
    if (tape && n > f->tape_cap) {
        cudaFree(f->buf_tape);
        FCK(cudaMalloc(&f->buf_tape, (int64_t)f->L * n * 4 * f->d * sizeof(float)));
        f->tape_cap = n;
    }
    return MCIG_OK;
}

static int flow_cast(mcig_flow *f, cudaStream_t st)
{
    flow_cast_kernel<<<256, 256, 0, st>>>(f->theta, f->wb, f->d, f->L);
    FCK(cudaGetLastError());
    return MCIG_OK;
}

extern "C" int64_t mcig_flow_nparams(int ndim, int nlayers)
{
    const int d = ndim / 2;
    return (int64_t)nlayers * pl_size(d) + 2 * (int64_t)ndim;
}

extern "C" int mcig_flow_create(int ndim, int nlayers, int hidden, uint64_t seed, int device, mcig_flow **out)
{
    if (!out) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "out is NULL"); }
    *out = nullptr;
    if (ndim < 2 || ndim > FLOW_MAXD || ndim % 2) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "flow: ndim must be even and in [2, 32]"); }
    if (nlayers < 1 || nlayers > FLOW_MAXL) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "flow: nlayers must be in [1, 16]"); }
    if (hidden != FLOW_H) { return flow_err(MCIG_ERR_UNSUPPORTED, "flow: hidden width must be 128"); }
    FCK(cudaSetDevice(device));
    mcig_flow *f = new mcig_flow();
    f->D = ndim;
    f->d = ndim / 2;
    f->L = nlayers;
    f->device = device;
    f->seed = seed;
    f->pstride = pl_size(f->d);
    f->base_off = (int64_t)nlayers * f->pstride;
    f->np = mcig_flow_nparams(ndim, nlayers);
    cudaStreamCreateWithFlags(&f->st, cudaStreamNonBlocking);
    FCK(cudaMalloc(&f->theta, f->np * sizeof(float)));
    FCK(cudaMalloc(&f->grad, f->np * sizeof(float)));
    FCK(cudaMalloc(&f->m, f->np * sizeof(float)));
    FCK(cudaMalloc(&f->v, f->np * sizeof(float)));
    FCK(cudaMalloc(&f->wb, (int64_t)nlayers * WB_LAYER * sizeof(__nv_bfloat16)));
    FCK(cudaMalloc(&f->perm, (int64_t)nlayers * ndim * sizeof(int)));
    std::vector<int> p = flow_perms(ndim, nlayers, seed);
    FCK(cudaMemcpy(f->perm, p.data(), p.size() * sizeof(int), cudaMemcpyHostToDevice));
    // He-normal hidden weights (Box-Muller on splitmix64), zero output layer: the flow starts as the identity
    std::vector<float> th((size_t)f->np, 0.f);
    uint64_t s = seed ^ 0xA5A5A5A5DEADBEEFULL;
    auto nrm = [&s]() {
        auto nxt = [&s]() {
            s += 0x9E3779B97F4A7C15ULL;
            uint64_t z = s;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
            return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
        };
        const double u1 = 1.0 - nxt(), u2 = nxt();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    };
    for (int l = 0; l < nlayers; ++l) {
        float *P = th.data() + (int64_t)l * f->pstride;
        for (int64_t i = 0; i < (int64_t)f->d * FLOW_H; ++i) { P[pl_W1(f->d) + i] = (float)(nrm() * std::sqrt(2.0 / f->d)); }
        for (int64_t i = 0; i < (int64_t)FLOW_H * FLOW_H; ++i) { P[pl_W2(f->d) + i] = (float)(nrm() * std::sqrt(2.0 / FLOW_H)); }
    }
    FCK(cudaMemcpy(f->theta, th.data(), th.size() * sizeof(float), cudaMemcpyHostToDevice));
    FCK(cudaMemset(f->m, 0, f->np * sizeof(float)));
    FCK(cudaMemset(f->v, 0, f->np * sizeof(float)));
    int rc = flow_cast(f, f->st);
    if (rc) { return rc; }
    FCK(cudaFuncSetAttribute(flow_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FlowSmem)));
    FCK(cudaFuncSetAttribute(flow_pass_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FlowFusedSmem)));
    FCK(cudaDeviceGetAttribute(&f->nsm, cudaDevAttrMultiProcessorCount, device));
    FCK(cudaFuncSetAttribute(flow_pass_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FlowTcSmem)));
    FCK(cudaMalloc(&f->status, sizeof(int)));
    FCK(cudaMemset(f->status, 0, sizeof(int)));
    FCK(cudaFuncSetAttribute(flow_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FlowBwdSmem)));
    FCK(cudaStreamSynchronize(f->st));
    *out = f;
    return MCIG_OK;
}

extern "C" int mcig_flow_destroy(mcig_flow *f)
{
    if (!f) { return MCIG_OK; }
    cudaSetDevice(f->device);
    cudaStreamSynchronize(f->st);
    cudaFree(f->theta); cudaFree(f->grad); cudaFree(f->m); cudaFree(f->v); cudaFree(f->wb); cudaFree(f->perm);
    cudaFree(f->status);
    cudaFree(f->buf_in); cudaFree(f->buf_out); cudaFree(f->buf_logq); cudaFree(f->buf_tape); cudaFree(f->buf_batch);
    cudaStreamDestroy(f->st);
    delete f;
    return MCIG_OK;
}

extern "C" int mcig_flow_tc_selftest(int device, const uint16_t *a, const uint16_t *b, int n, int k, float *d)
{
    if (!a || !b || !d) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "tc self-test: NULL pointer"); }
    if (n < 16 || n > 256 || n % 16 || k < 16 || k > 256 || k % 16) {
        return flow_err(MCIG_ERR_INVALID_ARGUMENT, "tc self-test: N and K must be multiples of 16 in [16, 256]");
    }
    FCK(cudaSetDevice(device));
    __nv_bfloat16 *dA = nullptr, *dB = nullptr;
    float *dD = nullptr;
    int *dst = nullptr;
    FCK(cudaMalloc(&dA, 128 * (size_t)k * 2));
    FCK(cudaMalloc(&dB, (size_t)n * k * 2));
    FCK(cudaMalloc(&dD, 128 * (size_t)n * 4));
    FCK(cudaMalloc(&dst, sizeof(int)));
    FCK(cudaMemcpy(dA, a, 128 * (size_t)k * 2, cudaMemcpyHostToDevice));
    FCK(cudaMemcpy(dB, b, (size_t)n * k * 2, cudaMemcpyHostToDevice));
    FCK(cudaMemset(dst, 0, sizeof(int)));
    const size_t smem = (128 + (size_t)n) * k * 2 + 16;
    FCK(cudaFuncSetAttribute(flow_tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    flow_tc_selftest_kernel<<<1, 128, smem>>>(dA, dB, dD, n, k, dst);
    FCK(cudaGetLastError());
    FCK(cudaDeviceSynchronize());
    int st = 0;
    FCK(cudaMemcpy(&st, dst, sizeof(int), cudaMemcpyDeviceToHost));
    FCK(cudaMemcpy(d, dD, 128 * (size_t)n * 4, cudaMemcpyDeviceToHost));
    cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(dst);
    if (st) { return flow_err(MCIG_ERR_TIMEOUT, "tc self-test: the MMA completion was not seen within the wait limit"); }
    return MCIG_OK;
}

extern "C" int mcig_flow_get_params(const mcig_flow *f, float *theta, int64_t *n)
{
    *n = f->np;
    if (theta) {
        cudaSetDevice(f->device);
        FCK(cudaMemcpy(theta, f->theta, f->np * sizeof(float), cudaMemcpyDeviceToHost));
    }
    return MCIG_OK;
}

extern "C" int mcig_flow_set_params(mcig_flow *f, const float *theta, int64_t n)
{
    if (n != f->np) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "flow: parameter count mismatch"); }
    cudaSetDevice(f->device);
    FCK(cudaMemcpy(f->theta, theta, n * sizeof(float), cudaMemcpyHostToDevice));
    f->adam_t = 0;
    FCK(cudaMemset(f->m, 0, f->np * sizeof(float)));
    FCK(cudaMemset(f->v, 0, f->np * sizeof(float)));
    int rc = flow_cast(f, f->st);
    if (rc) { return rc; }
    FCK(cudaStreamSynchronize(f->st));
    return MCIG_OK;
}

// one pass over device arrays (in [n][D] float -> out, logq); tape optional.  The
// register-fused kernel takes as many warps per CTA (16 rows each, at most 16) as spread the
// rows of both sets over every SM once.
static int flow_pass_launch(mcig_flow *f, FlowArgs &a, int64_t n, cudaStream_t st)
{
    const int64_t total = n + a.nb;
    if (f->tc == 1) {
        const int grid = (int)((n + FTC_ROWS - 1) / FTC_ROWS);
        flow_pass_tc_kernel<<<grid, FTC_THREADS, sizeof(FlowTcSmem), st>>>(a, f->status);
    } else if (f->tc == 2) {
        const int grid = (int)((n + FLOW_PASS_ROWS - 1) / FLOW_PASS_ROWS);
        flow_pass_kernel<<<grid, FLOW_PASS_THREADS, sizeof(FlowSmem), st>>>(a);
    } else {
        const int64_t per_sm = (total + 16 * (int64_t)f->nsm - 1) / (16 * (int64_t)f->nsm);
        const int w = (int)std::min<int64_t>(FLOW_FUSED_MAXW, std::max<int64_t>(1, per_sm));
        const int grid = (int)((total + 16 * w - 1) / (16 * w));
        flow_pass_fused_kernel<<<grid, 32 * w, sizeof(FlowFusedSmem), st>>>(a);
    }
    FCK(cudaGetLastError());
    return MCIG_OK;
}

// the status of the tcgen05 passes since the last check (then cleared)
int mcig_flow_check_status(mcig_flow *f, cudaStream_t st)
{
    int h = 0;
    FCK(cudaMemcpyAsync(&h, f->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    FCK(cudaStreamSynchronize(st));
    if (h) {
        FCK(cudaMemsetAsync(f->status, 0, sizeof(int), st));
        return flow_err(MCIG_ERR_TIMEOUT, "flow: a tensor-core pass did not see its MMA complete within the bounded wait");
    }
    return MCIG_OK;
}

extern "C" int mcig_flow_set_tensor_path(mcig_flow *f, int tc)
{
    if (!f) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "flow is NULL"); }
    if (tc < 0 || tc > 2) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "pass kernel must be 0 (register-fused mma.sync), 1 (tcgen05) or 2 (shared-memory mma.sync)"); }
    f->tc = tc;
    return MCIG_OK;
}

// the density passes (log q) of two chain-minor walker sets in one launch of the register-fused
// kernel: in_cm (double) -> logq_a and in_cmf_b (float) -> logq_b, n walkers each (stride
// nstride); with another pass kernel selected, two launches
int mcig_flow_density2_device(mcig_flow *f, const double *in_cm, const float *in_cmf_b, int64_t nstride, int64_t n,
                              float *logq_a, float *logq_b, cudaStream_t st)
{
    FlowArgs a;
    memset(&a, 0, sizeof(a));
    a.D = f->D; a.d = f->d; a.L = f->L; a.n = (int)n; a.dir = 1;
    a.logq = logq_a;
    a.mu = f->theta + f->base_off; a.logsig = f->theta + f->base_off + f->D;
    a.perm = f->perm; a.wb = f->wb; a.theta = f->theta;
    a.wstride = WB_LAYER; a.pstride = f->pstride;
    a.in_cm = in_cm; a.cm_stride = nstride;
    if (f->tc == 0) {
        a.nb = (int)n; a.in_cmf_b = in_cmf_b; a.logq_b = logq_b;
        return flow_pass_launch(f, a, n, st);
    }
    int rc = flow_pass_launch(f, a, n, st);
    if (rc) { return rc; }
    a.in_cm = nullptr; a.in_cmf = in_cmf_b; a.logq = logq_b;
    return flow_pass_launch(f, a, n, st);
}

// one pass with chain-minor walkers: input in_cm (double, NULL: rows d_in) and output
// out_cm (float, NULL: none), both with stride nstride; log q into d_logq
int mcig_flow_pass_device_cm(mcig_flow *f, int dir, const float *d_in, const double *in_cm, int64_t nstride, int64_t n,
                             float *out_cm, float *d_logq, cudaStream_t st)
{
    FlowArgs a;
    memset(&a, 0, sizeof(a));
    a.D = f->D; a.d = f->d; a.L = f->L; a.n = (int)n; a.dir = dir;
    a.in = d_in; a.out = nullptr; a.logq = d_logq;
    a.mu = f->theta + f->base_off; a.logsig = f->theta + f->base_off + f->D;
    a.perm = f->perm; a.tape = nullptr; a.wb = f->wb; a.theta = f->theta;
    a.wstride = WB_LAYER; a.pstride = f->pstride;
    a.in_cm = in_cm; a.out_cm = out_cm; a.cm_stride = nstride;
    return flow_pass_launch(f, a, n, st);
}

// the flow proposal x' = f(z) of one cycle for n chains: z drawn in the pass from Philox
// (key, cycle), x' written chain-minor (stride nstride), log q of the generative pass to d_logq
int mcig_flow_propose_device(mcig_flow *f, uint64_t cycle, uint32_t key0, uint32_t key1, int64_t nstride, int64_t n,
                             float *out_cm, float *d_logq, cudaStream_t st)
{
    FlowArgs a;
    memset(&a, 0, sizeof(a));
    a.D = f->D; a.d = f->d; a.L = f->L; a.n = (int)n; a.dir = 0;
    a.logq = d_logq;
    a.mu = f->theta + f->base_off; a.logsig = f->theta + f->base_off + f->D;
    a.perm = f->perm; a.wb = f->wb; a.theta = f->theta;
    a.wstride = WB_LAYER; a.pstride = f->pstride;
    a.out_cm = out_cm; a.cm_stride = nstride;
    a.zgen = 1; a.zk0 = key0; a.zk1 = key1; a.zcycle = cycle;
    return flow_pass_launch(f, a, n, st);
}

// the density pass (log q) of n chain-minor float walkers (stride nstride)
int mcig_flow_density_cmf_device(mcig_flow *f, const float *in_cmf, int64_t nstride, int64_t n, float *d_logq,
                                 cudaStream_t st)
{
    FlowArgs a;
    memset(&a, 0, sizeof(a));
    a.D = f->D; a.d = f->d; a.L = f->L; a.n = (int)n; a.dir = 1;
    a.logq = d_logq;
    a.mu = f->theta + f->base_off; a.logsig = f->theta + f->base_off + f->D;
    a.perm = f->perm; a.wb = f->wb; a.theta = f->theta;
    a.wstride = WB_LAYER; a.pstride = f->pstride;
    a.in_cmf = in_cmf; a.cm_stride = nstride;
    return flow_pass_launch(f, a, n, st);
}

int mcig_flow_pass_device(mcig_flow *f, int dir, const float *d_in, int64_t n, float *d_out, float *d_logq, float *d_tape,
                          cudaStream_t st)
{
    FlowArgs a;
    memset(&a, 0, sizeof(a));
    a.in_cm = nullptr; a.out_cm = nullptr; a.cm_stride = 0;
    a.D = f->D; a.d = f->d; a.L = f->L; a.n = (int)n; a.dir = dir;
    a.in = d_in; a.out = d_out; a.logq = d_logq;
    a.mu = f->theta + f->base_off; a.logsig = f->theta + f->base_off + f->D;
    a.perm = f->perm; a.tape = d_tape; a.wb = f->wb; a.theta = f->theta;
    a.wstride = WB_LAYER; a.pstride = f->pstride;
    return flow_pass_launch(f, a, n, st);
}

static int flow_host_pass(mcig_flow *f, int dir, const double *in, int64_t n, double *out, double *logq)
{
    if (n < 1) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "flow: n must be >= 1"); }
    cudaSetDevice(f->device);
    int rc = flow_ensure(f, n, false);
    if (rc) { return rc; }
    std::vector<float> h((size_t)n * f->D);
    for (size_t i = 0; i < h.size(); ++i) { h[i] = (float)in[i]; }
    FCK(cudaMemcpyAsync(f->buf_in, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, f->st));
    rc = mcig_flow_pass_device(f, dir, f->buf_in, n, f->buf_out, f->buf_logq, nullptr, f->st);
    if (rc) { return rc; }
    std::vector<float> lq((size_t)n);
    FCK(cudaMemcpyAsync(h.data(), f->buf_out, h.size() * sizeof(float), cudaMemcpyDeviceToHost, f->st));
    FCK(cudaMemcpyAsync(lq.data(), f->buf_logq, n * sizeof(float), cudaMemcpyDeviceToHost, f->st));
    FCK(cudaStreamSynchronize(f->st));
    if ((rc = mcig_flow_check_status(f, f->st))) { return rc; }
    if (out) { for (size_t i = 0; i < h.size(); ++i) { out[i] = h[i]; } }
    if (logq) { for (int64_t i = 0; i < n; ++i) { logq[i] = lq[i]; } }
    return MCIG_OK;
}

extern "C" int mcig_flow_forward(mcig_flow *f, const double *z, int64_t n, double *x, double *logq)
{
    return flow_host_pass(f, 0, z, n, x, logq);
}

extern "C" int mcig_flow_inverse(mcig_flow *f, const double *x, int64_t n, double *z, double *logq)
{
    return flow_host_pass(f, 1, x, n, z, logq);
}

// loss -mean log q(x) and its gradient on device data d_x [n][D]; gradient left in f->grad
static int flow_loss_grad_device(mcig_flow *f, const float *d_x, int64_t n, float *loss_host, cudaStream_t st)
{
    int rc = flow_ensure(f, n, true);
    if (rc) { return rc; }
    rc = mcig_flow_pass_device(f, 1, d_x, n, f->buf_out, f->buf_logq, f->buf_tape, st);
    if (rc) { return rc; }
    FCK(cudaMemsetAsync(f->grad, 0, f->np * sizeof(float), st));
    FlowBwdArgs b;
    b.D = f->D; b.d = f->d; b.L = f->L; b.n = (int)n;
    b.inv_batch = 1.f / (float)n;
    b.z = f->buf_out; b.tape = f->buf_tape; b.perm = f->perm; b.wb = f->wb; b.theta = f->theta;
    b.grad = f->grad; b.x = d_x; b.mu = f->theta + f->base_off; b.logsig = f->theta + f->base_off + f->D;
    b.wstride = WB_LAYER; b.pstride = f->pstride; b.base_off = f->base_off;
    const int grid = (int)((n + FLOW_ROWS - 1) / FLOW_ROWS);
    flow_backward_kernel<<<grid, FLOW_THREADS, sizeof(FlowBwdSmem), st>>>(b);
    FCK(cudaGetLastError());
    if (loss_host) {
        std::vector<float> lq((size_t)n);
        FCK(cudaMemcpyAsync(lq.data(), f->buf_logq, n * sizeof(float), cudaMemcpyDeviceToHost, st));
        FCK(cudaStreamSynchronize(st));
        double s = 0.;
        for (float v : lq) { s += v; }
        *loss_host = (float)(-s / (double)n);
    }
    return MCIG_OK;
}

extern "C" int mcig_flow_loss_grad(mcig_flow *f, const double *x, int64_t n, double *loss, float *grad)
{
    if (n < 1) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "flow: n must be >= 1"); }
    cudaSetDevice(f->device);
    int rc = flow_ensure(f, n, true);
    if (rc) { return rc; }
    float *d_x = nullptr;
    FCK(cudaMalloc(&d_x, n * f->D * sizeof(float)));
    std::vector<float> h((size_t)n * f->D);
    for (size_t i = 0; i < h.size(); ++i) { h[i] = (float)x[i]; }
    cudaMemcpyAsync(d_x, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, f->st);
    float l = 0.f;
    rc = flow_loss_grad_device(f, d_x, n, &l, f->st);
    if (!rc && grad) {
        cudaMemcpyAsync(grad, f->grad, f->np * sizeof(float), cudaMemcpyDeviceToHost, f->st);
        cudaStreamSynchronize(f->st);
    }
    cudaFree(d_x);
    if (loss) { *loss = l; }
    return rc;
}

// Adam steps on minibatches drawn from device data d_x [nsrc][D], queued on stream st;
// with last_loss the call waits for st and returns the loss of the last minibatch
int mcig_flow_train_device(mcig_flow *f, const float *d_x, int64_t nsrc, int steps, int batch, double lr, float *last_loss,
                           cudaStream_t st)
{
    if (batch < 1 || steps < 0 || nsrc < 1) { return flow_err(MCIG_ERR_INVALID_ARGUMENT, "flow: bad training arguments"); }
    if (batch > f->batch_cap) {
        FCK(cudaStreamSynchronize(st));
        cudaFree(f->buf_batch);
        FCK(cudaMalloc(&f->buf_batch, (int64_t)batch * f->D * sizeof(float)));
        f->batch_cap = batch;
    }
    int rc = flow_ensure(f, batch, true);
    if (rc) { return rc; }
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < steps; ++it) {
        flow_gather_kernel<<<(batch + 127) / 128, 128, 0, st>>>(d_x, nsrc, f->D, (uint32_t)f->seed, (uint32_t)f->adam_t,
                                                               f->buf_batch, batch);
        rc = flow_loss_grad_device(f, f->buf_batch, batch, (it == steps - 1) ? last_loss : nullptr, st);
        if (rc) { return rc; }
        ++f->adam_t;
        const float c1 = 1.f / (1.f - powf(b1, (float)f->adam_t)), c2 = 1.f / (1.f - powf(b2, (float)f->adam_t));
        flow_adam_kernel<<<256, 256, 0, st>>>(f->theta, f->grad, f->m, f->v, f->np, (float)lr, b1, b2, eps, c1, c2);
        FCK(cudaGetLastError());
        rc = flow_cast(f, st);
        if (rc) { return rc; }
    }
    if (last_loss) { FCK(cudaStreamSynchronize(st)); }
    return MCIG_OK;
}

extern "C" int mcig_flow_train(mcig_flow *f, const double *x, int64_t n, int steps, int batch, double lr, double *last_loss)
{
    cudaSetDevice(f->device);
    float *d_x = nullptr;
    FCK(cudaMalloc(&d_x, n * f->D * sizeof(float)));
    std::vector<float> h((size_t)n * f->D);
    for (size_t i = 0; i < h.size(); ++i) { h[i] = (float)x[i]; }
    cudaMemcpy(d_x, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
    float l = 0.f;
    const int rc = mcig_flow_train_device(f, d_x, n, steps, batch, lr, &l, f->st);
    cudaFree(d_x);
    if (last_loss) { *last_loss = l; }
    return rc;
}

// accessors for the sampler (mcig_capi.cu)
int mcig_flow_dim(const mcig_flow *f) { return f->D; }
cudaStream_t mcig_flow_stream(const mcig_flow *f) { return f->st; }
