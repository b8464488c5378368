// KS closure network: a 3-layer 1D convolution (1 -> 32 -> 32 -> 1 channels,
// kernel 5, GELU, circular padding per domain) that corrects a coarse KS step.
// Parameters are FP32 masters rounded to BF16 for the forward pass.  The
// 32 -> 32 layer -- 94 % of the work -- runs on the tensor cores
// (mma.sync.m16n8k16, BF16 operands, FP32 accumulation) forward and backward;
// the 1 -> 32 and 32 -> 1 layers run in FP32 on the CUDA cores with the
// BF16-rounded weights.  oracle/closure.py restates the same arithmetic.
//
// Tiles: a block produces TOUT = 128 consecutive outputs of one domain.  In
// tile coordinates (x0 = first output):
//   us[j] = u[x0 - 6 + j],        j < 152
//   a1[r] : position x0 - 4 + r,  r < 148  (z1 = w1 * us[r .. r+4] + b1)
//   z2[p] : position x0 - 2 + p,  p < 144  (needs a1[p .. p+4]; p < 132 used)
//   d[q]  : position x0 + q,      q < 128  (needs a2[q .. q+4])
// The im2col of layer 2 is free: the A fragment of tap t is the a1 rows
// shifted by t.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

#include "ctx.h"
#include "stencils.cuh"
#include "sw_internal.h"

namespace sw {
namespace cl {

constexpr int CH = 32, KW = 5;
static_assert(CH == 32, "layer 1 maps one warp lane to each channel");
constexpr int TOUT = 128;
constexpr int NU = TOUT + 24;   // 152 input cells
constexpr int NA1 = TOUT + 20;  // 148 a1 rows
constexpr int NZ2 = 144;        // 9 m-tiles of 16 rows
constexpr int NA2 = TOUT + 4;   // 132 a2 rows used
constexpr int LDB = 40;         // bf16 row stride (80 B: conflict-free fragment reads)
constexpr int LDF = 33;         // fp32 row stride
constexpr int THREADS = 256;  // (9 warps, one per layer-2 m-tile, measured slower: 106.5 against 102.3 us per step)
// parameter offsets (flat FP32 vector); the last value is the output scale s
// (delta = s * net(u)), fixed by the caller and left alone by training
constexpr int OW1 = 0, OB1 = 160, OW2 = 192, OB2 = 5312, OW3 = 5344, OB3 = 5504, OSCALE = 5505;
constexpr int NTRAIN = 5505, NPARAM = 5506;

// GELU in its tanh form (Hendrycks & Gimpel, "Gaussian Error Linear Units",
// 2016): gelu(x) = x/2 (1 + tanh(c (x + a x^3))), c = sqrt(2/pi), a = 0.044715,
// with tanh from the SFU's tanh.approx.f32 (relative error below 2^-10.7):
// a handful of instructions where the erf form took a long polynomial, and
// the step is bound by instruction issue.  oracle/closure.py restates the same
// function (with an exact tanh).
constexpr float kGeluC = 0.79788456080286536f, kGeluA = 0.044715f;
__device__ __forceinline__ float tanh_sfu(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu(float x) {  // x/2 + (x/2) t, the operations of gelu2 below
    const float t = tanh_sfu((kGeluC * x) * fmaf(kGeluA, x * x, 1.0f));
    const float hx = 0.5f * x;
    return fmaf(hx, t, hx);
}
// Two GELUs with paired FP32 instructions (one f32x2 instruction does the
// arithmetic of two lanes' worth: the forward step is bound by instruction
// issue).  Each component is gelu of that component, operation for operation.
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 gelu2(float2 x) {
    const float2 inner = __ffma2_rn(f2(kGeluA), __fmul2_rn(x, x), f2(1.0f));
    const float2 arg = __fmul2_rn(__fmul2_rn(f2(kGeluC), x), inner);
    const float2 hx = __fmul2_rn(f2(0.5f), x);
    return __ffma2_rn(hx, make_float2(tanh_sfu(arg.x), tanh_sfu(arg.y)), hx);
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float x2 = x * x;
    const float t = tanh_sfu(kGeluC * x * fmaf(kGeluA, x2, 1.0f));
    return fmaf(0.5f * x * (1.0f - t * t), kGeluC * fmaf(3.0f * kGeluA, x2, 1.0f), 0.5f * (1.0f + t));
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
__device__ __forceinline__ uint32_t ld2(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

// D = A * B + D, m16n8k16, A row-major BF16, B column-major BF16, FP32 accumulate
__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Shared memory of a tile.  The forward kernels allocate only the part up to
// z2 (smem_fwd_bytes); the backward kernel also keeps the pre-activations.
struct Smem {
    float us[NU];
    float w1[CH * KW], b1[CH], b2[CH], w3[CH * KW], b3, scale;
    __nv_bfloat16 a1[NA1 * LDB];                   // layer-1 activations, BF16 (the MMA A operand)
    alignas(16) __nv_bfloat16 w2[KW * CH * LDB];   // w2[t][o][i], i contiguous (the MMA B operand)
    float pred[TOUT + 4];                          // k_step: the KS predictor on x0-2 .. x0+TOUT+1
    float p3[KW * NA2];                            // forward: p3[t][r] = sum_i w3[i][t] a2[r][i]
    float a2[NA2 * LDF];                           // layer-2 activations gelu(z2) (backward only)
    float z2[NA2 * LDF];                           // layer-2 pre-activations (backward only)
    float z1[NA1 * LDF];                           // layer-1 pre-activations (backward only)
};
constexpr int W2P_WORDS = KW * CH * LDB * 2 / 16;  // the staged w2 in 16-byte words

// theta's w2 (flat [o][i][t], FP32) -> BF16 in the shared-memory layout [t][o][i]
// (row stride LDB; the padding columns are zero), once per call of the
// forward kernels instead of once per block.
__global__ void k_pack_w2(const float *__restrict__ theta, __nv_bfloat16 *__restrict__ w2p) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= KW * CH * LDB) return;
    const int t = k / (CH * LDB), o = (k / LDB) % CH, i = k % LDB;
    w2p[k] = __float2bfloat16_rn(i < CH ? theta[OW2 + (o * CH + i) * KW + t] : 0.0f);
}

// Load the tile's inputs (periodic within the domain) and, unless `weights`
// is false, the weights; w2 from the staged copy w2p (16-byte words) when
// given, else from theta.
__device__ void load_tile(Smem &s, const float *__restrict__ theta, const float *__restrict__ u, int64_t n,
                          int64_t x0, const uint4 *__restrict__ w2p = nullptr, bool weights = true) {
    for (int j = threadIdx.x; j < NU; j += blockDim.x) {
        int64_t q = x0 - 6 + j;
        q %= n;
        if (q < 0) q += n;
        s.us[j] = u[q];
    }
    if (!weights) return;
    for (int i = threadIdx.x; i < CH * KW; i += blockDim.x) {
        s.w1[i] = bf16r(theta[OW1 + i]);
        s.w3[i] = bf16r(theta[OW3 + i]);
    }
    for (int i = threadIdx.x; i < CH; i += blockDim.x) {
        s.b1[i] = theta[OB1 + i];
        s.b2[i] = theta[OB2 + i];
    }
    if (threadIdx.x == 0) {
        s.b3 = theta[OB3];
        s.scale = theta[OSCALE];
    }
    if (w2p) {
        uint4 *dst = reinterpret_cast<uint4 *>(s.w2);
        for (int k = threadIdx.x; k < W2P_WORDS; k += blockDim.x) dst[k] = w2p[k];
        return;
    }
    // w2 flat is [o][i][t]; smem is [t][o][i]
    for (int k = threadIdx.x; k < CH * CH * KW; k += blockDim.x) {
        const int o = k / (CH * KW), i = (k / KW) % CH, t = k % KW;
        s.w2[(t * CH + o) * LDB + i] = __float2bfloat16_rn(theta[OW2 + k]);
    }
}

// Layers 1 and 2 of the forward pass.  TRAIN: a1 (BF16), a2 = gelu(z2) (FP32)
// and the pre-activations z1, z2 for the backward pass.  Otherwise layer 3's
// per-row tap sums p3[t][r] = sum_i w3[i][t] gelu(z2[r][i]) are formed in the
// MMA epilogue, so a2 is never stored: each lane holds 8 channels of rows r
// and r + 8, dots them with w3 for the five taps, and the four lanes of a row
// add their sums by shuffles (output q is then b3 + sum_t p3[t][q + t]).
// Requires load_tile and a barrier first.
template <bool TRAIN>
__device__ void forward_12(Smem &s) {
    {
        // lane = output channel o; each warp a contiguous run of rows, with o's
        // five weights and a sliding window of five inputs in registers (one
        // shared load per row; the FMA chain is the same, tap 0 first)
        const int o = threadIdx.x & 31, nw = blockDim.x >> 5;
        const int per = (NA1 + nw - 1) / nw, r0 = (threadIdx.x >> 5) * per;
        const int r1 = min(r0 + per, NA1);
        float w[KW], u[KW];
#pragma unroll
        for (int t = 0; t < KW; ++t) w[t] = s.w1[o * KW + t];
        const float b = s.b1[o];
        int r = r0;
        if constexpr (!TRAIN) {
            // two rows per iteration as f32x2 pairs: window v[0..5] = inputs r .. r+5
            float v[KW + 1];
            if (r0 < r1) {
#pragma unroll
                for (int t = 0; t < KW - 1; ++t) v[t + 2] = s.us[r0 + t];
            }
            for (; r + 1 < r1; r += 2) {
#pragma unroll
                for (int t = 0; t < KW - 1; ++t) v[t] = v[t + 2];
                v[KW - 1] = s.us[r + KW - 1];
                v[KW] = s.us[r + KW];
                float2 z = f2(b);
#pragma unroll
                for (int t = 0; t < KW; ++t) z = __ffma2_rn(f2(w[t]), make_float2(v[t], v[t + 1]), z);
                const float2 g = gelu2(z);
                s.a1[r * LDB + o] = __float2bfloat16_rn(g.x);
                s.a1[(r + 1) * LDB + o] = __float2bfloat16_rn(g.y);
            }
        }
        if (r < r1) {
#pragma unroll
            for (int t = 0; t < KW - 1; ++t) u[t + 1] = s.us[r + t];
        }
        for (; r < r1; ++r) {
#pragma unroll
            for (int t = 0; t < KW - 1; ++t) u[t] = u[t + 1];
            u[KW - 1] = s.us[r + KW - 1];
            float z = b;
#pragma unroll
            for (int t = 0; t < KW; ++t) z = fmaf(w[t], u[t], z);
            if (TRAIN) s.z1[r * LDF + o] = z;
            s.a1[r * LDB + o] = __float2bfloat16_rn(gelu(z));
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    for (int m = warp; m < NZ2 / 16; m += blockDim.x >> 5) {
        const int p0 = m * 16;
        float acc[4][4] = {};
#pragma unroll
        for (int t = 0; t < KW; ++t) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                // rows beyond NA1 are only reached for p >= NA2 (discarded rows): clamp the read
                const int ra = min(p0 + g + t, NA1 - 1), rb = min(p0 + g + 8 + t, NA1 - 1);
                const uint32_t a0 = ld2(&s.a1[ra * LDB + 16 * h + 2 * q]);
                const uint32_t a1 = ld2(&s.a1[rb * LDB + 16 * h + 2 * q]);
                const uint32_t a2 = ld2(&s.a1[ra * LDB + 16 * h + 8 + 2 * q]);
                const uint32_t a3 = ld2(&s.a1[rb * LDB + 16 * h + 8 + 2 * q]);
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const __nv_bfloat16 *wb = &s.w2[(t * CH + nt * 8 + g) * LDB + 16 * h];
                    mma_bf16(acc[nt], a0, a1, a2, a3, ld2(wb + 2 * q), ld2(wb + 8 + 2 * q));
                }
            }
        }
        const int r0 = p0 + g, r1 = p0 + g + 8;
        if constexpr (TRAIN) {
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int o = nt * 8 + 2 * q;
                if (r0 < NA2) {
                    const float z0 = acc[nt][0] + s.b2[o], z1 = acc[nt][1] + s.b2[o + 1];
                    s.z2[r0 * LDF + o] = z0;
                    s.z2[r0 * LDF + o + 1] = z1;
                    s.a2[r0 * LDF + o] = gelu(z0);
                    s.a2[r0 * LDF + o + 1] = gelu(z1);
                }
                if (r1 < NA2) {
                    const float z2 = acc[nt][2] + s.b2[o], z3 = acc[nt][3] + s.b2[o + 1];
                    s.z2[r1 * LDF + o] = z2;
                    s.z2[r1 * LDF + o + 1] = z3;
                    s.a2[r1 * LDF + o] = gelu(z2);
                    s.a2[r1 * LDF + o + 1] = gelu(z3);
                }
            }
        } else {
            // GELU on channel pairs (o, o+1) of a row, the tap sums on row pairs (r0, r1)
            float2 pr[KW];
#pragma unroll
            for (int t = 0; t < KW; ++t) pr[t] = f2(0.0f);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int o = nt * 8 + 2 * q;
                const float2 bias = make_float2(s.b2[o], s.b2[o + 1]);
                const float2 g0 = gelu2(__fadd2_rn(make_float2(acc[nt][0], acc[nt][1]), bias));  // row r0
                const float2 g1 = gelu2(__fadd2_rn(make_float2(acc[nt][2], acc[nt][3]), bias));  // row r1
                const float2 c0 = make_float2(g0.x, g1.x), c1 = make_float2(g0.y, g1.y);         // channel o, o+1
#pragma unroll
                for (int t = 0; t < KW; ++t) {
                    pr[t] = __ffma2_rn(f2(s.w3[o * KW + t]), c0, pr[t]);
                    pr[t] = __ffma2_rn(f2(s.w3[(o + 1) * KW + t]), c1, pr[t]);
                }
            }
#pragma unroll
            for (int t = 0; t < KW; ++t) {
                pr[t].x += __shfl_xor_sync(0xffffffffu, pr[t].x, 1);
                pr[t].y += __shfl_xor_sync(0xffffffffu, pr[t].y, 1);
                pr[t].x += __shfl_xor_sync(0xffffffffu, pr[t].x, 2);
                pr[t].y += __shfl_xor_sync(0xffffffffu, pr[t].y, 2);
            }
            if (q == 0) {
#pragma unroll
                for (int t = 0; t < KW; ++t) {
                    if (r0 < NA2) s.p3[t * NA2 + r0] = pr[t].x;
                    if (r1 < NA2) s.p3[t * NA2 + r1] = pr[t].y;
                }
            }
        }
    }
    __syncthreads();
}

// Layer 3 for output q from the epilogue's tap sums: b3 + sum_t p3[t][q + t].
__device__ __forceinline__ float layer3_sums(const Smem &s, int q) {
    float d = 0.0f;
#pragma unroll
    for (int t = 0; t < KW; ++t) d += s.p3[t * NA2 + q + t];
    return d + s.b3;
}

// Layer 3 for output q (backward pass, from the stored a2): b3 + sum_{t,i} w3[i][t] * a2[q + t][i].
__device__ __forceinline__ float layer3(const Smem &s, int q) {
    float d = 0.0f;
#pragma unroll
    for (int t = 0; t < KW; ++t)
#pragma unroll 8
        for (int i = 0; i < CH; ++i) d = fmaf(s.w3[i * KW + t], s.a2[(q + t) * LDF + i], d);
    return d + s.b3;
}

// ---------------------------------------------------------------- kernels
// delta = f(u) for every cell of n_dom domains of n cells (n a multiple of TOUT).
__global__ void __launch_bounds__(THREADS) k_infer(const float *__restrict__ theta, const uint4 *__restrict__ w2p,
                                                   const float *__restrict__ u, float *__restrict__ delta, int64_t n,
                                                   int64_t tiles_per_dom) {
    extern __shared__ __align__(16) unsigned char raw[];
    Smem &s = *reinterpret_cast<Smem *>(raw);
    const int64_t dom = blockIdx.x / tiles_per_dom, x0 = (blockIdx.x % tiles_per_dom) * TOUT;
    const float *ud = u + dom * n;
    load_tile(s, theta, ud, n, x0, w2p);
    __syncthreads();
    forward_12<false>(s);
    for (int q = threadIdx.x; q < TOUT; q += blockDim.x) delta[dom * n + x0 + q] = s.scale * layer3_sums(s, q);
}

// One coarse KS step fused with the closure: u_out = classic KS step(u_in) + f(u_in).
// The KS predictor/corrector reads u_in on [x0-4, x0+TOUT+4) from the same tile.
__global__ void __launch_bounds__(THREADS) k_step(const float *__restrict__ theta, const uint4 *__restrict__ w2p,
                                                  const Params<float> pk, const float *__restrict__ u,
                                                  float *__restrict__ out, int64_t n, int64_t tiles_per_dom,
                                                  int use_closure) {
    extern __shared__ __align__(16) unsigned char raw[];
    Smem &s = *reinterpret_cast<Smem *>(raw);
    const int64_t dom = blockIdx.x / tiles_per_dom, x0 = (blockIdx.x % tiles_per_dom) * TOUT;
    load_tile(s, theta, u + dom * n, n, x0, w2p, use_closure != 0);  // theta may be null without the closure
    __syncthreads();
    if (use_closure) forward_12<false>(s);
    // predictor on positions x0-2 .. x0+TOUT+1 (us index 4 .. TOUT+7)
    for (int j = threadIdx.x; j < TOUT + 4; j += blockDim.x) {
        const int c = j + 4;
        s.pred[j] = ks_predict(pk, s.us[c - 2], s.us[c - 1], s.us[c], s.us[c + 1], s.us[c + 2]);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < TOUT; q += blockDim.x) {
        const int c = q + 6, j = q + 2;  // us index of x0+q; predictor index of x0+q
        float v = ks_correct(pk, s.us[c], s.pred[j - 2], s.pred[j - 1], s.pred[j], s.pred[j + 1], s.pred[j + 2]);
        if (use_closure) v += s.scale * layer3_sums(s, q);
        out[dom * n + x0 + q] = v;
    }
}

// Loss and parameter gradients (forward + backward), summed over the tiles a
// block visits into its row of `partial` ([gridDim.x][NPARAM + 1], last = loss).
// The loss is on the scaled defect: L = wpt * sum (net(u) - target / s)^2,
// wpt = 1 / (points in the batch), s the output scale.
__global__ void __launch_bounds__(THREADS) k_grad(const float *__restrict__ theta, const float *__restrict__ u,
                                                  const float *__restrict__ target, const int64_t *__restrict__ rows,
                                                  float *__restrict__ partial, int64_t n, int64_t tiles_per_dom,
                                                  int64_t n_tiles, float scale) {
    extern __shared__ __align__(16) unsigned char raw[];
    Smem &s = *reinterpret_cast<Smem *>(raw);
    __shared__ float g[NPARAM + 1];                 // this block's sums of the small-layer gradients and the loss
    __shared__ float dd[TOUT];                      // dL/ddelta
    __shared__ __nv_bfloat16 dzT[CH * (NZ2 + 8)];   // dz2 as [o][p] (BF16), p contiguous, for dW2
    __shared__ __nv_bfloat16 dzP[(NZ2 + 8) * LDB];  // dz2 as [4 + p][o] (BF16), 4 zero rows in front, for da1
    for (int i = threadIdx.x; i < NPARAM + 1; i += blockDim.x) g[i] = 0.0f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, q4 = lane & 3;
    const int nwarp = blockDim.x >> 5;
    // dW2 accumulators: warp w owns (m-tile mo, n-tile nn) pairs k = w, w+8, ... of 2 x 20
    float accw[5][4] = {};
    __syncthreads();

    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const int64_t b = tile / tiles_per_dom, x0 = (tile % tiles_per_dom) * TOUT;
        const int64_t dom = rows ? rows[b] : b;  // minibatch row -> sample
        load_tile(s, theta, u + dom * n, n, x0);
        __syncthreads();
        forward_12<true>(s);
        // delta, dL/ddelta, loss, dW3, db3
        for (int q = threadIdx.x; q < TOUT; q += blockDim.x) {
            const float d = layer3(s, q);
            const float e = d - target[dom * n + x0 + q] / s.scale;
            dd[q] = 2.0f * scale * e;
            atomicAdd(&g[NPARAM], scale * e * e);
        }
        __syncthreads();
        for (int k = threadIdx.x; k < CH * KW; k += blockDim.x) {
            const int i = k / KW, t = k % KW;
            float a = 0.0f;
            for (int q = 0; q < TOUT; ++q) a = fmaf(dd[q], s.a2[(q + t) * LDF + i], a);
            g[OW3 + k] += a;
        }
        if (threadIdx.x < 32) {
            float a = 0.0f;
            for (int q = threadIdx.x; q < TOUT; q += 32) a += dd[q];
#pragma unroll
            for (int off = 16; off; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
            if (threadIdx.x == 0) g[OB3] += a;
        }
        // dz2[p][o] = (sum_t w3[o][t] dd[p - t]) * gelu'(z2[p][o]), p < NA2; zero beyond
        for (int k = threadIdx.x; k < (NZ2 + 8) * CH; k += blockDim.x) {
            const int p = k / CH, o = k % CH;
            float v = 0.0f;
            if (p < NA2) {
                float da = 0.0f;
#pragma unroll
                for (int t = 0; t < KW; ++t) {
                    const int qq = p - t;
                    if (qq >= 0 && qq < TOUT) da = fmaf(s.w3[o * KW + t], dd[qq], da);
                }
                v = da * gelu_grad(s.z2[p * LDF + o]);
            }
            const __nv_bfloat16 b = __float2bfloat16_rn(v);
            dzT[o * (NZ2 + 8) + p] = b;
            if (p + 4 < NZ2 + 8) dzP[(p + 4) * LDB + o] = b;
            if (p < 4) dzP[p * LDB + o] = __float2bfloat16_rn(0.0f);
        }
        __syncthreads();
        // db2
        for (int o = threadIdx.x; o < CH; o += blockDim.x) {
            float a = 0.0f;
            for (int p = 0; p < NA2; ++p) a += __bfloat162float(dzT[o * (NZ2 + 8) + p]);
            g[OB2 + o] += a;
        }
        // dW2[o][(t,i)] += sum_p dz2[p][o] a1[p + t][i]: M = o (2 tiles), N = (t, i) (20 tiles), K = p (9 steps)
#pragma unroll
        for (int slot = 0; slot < 5; ++slot) {
            const int k = warp + slot * 8;  // 8 warps x 5 slots = 40 (m-tile, n-tile) pairs
            const int mo = k / 20, nn = k % 20, t = nn / 4, i0 = (nn % 4) * 8;
            for (int ks = 0; ks < NZ2 / 16; ++ks) {
                const int p0 = ks * 16;
                const __nv_bfloat16 *ra = &dzT[(mo * 16 + gq) * (NZ2 + 8) + p0];
                const __nv_bfloat16 *rb = &dzT[(mo * 16 + gq + 8) * (NZ2 + 8) + p0];
                const uint32_t a0 = ld2(ra + 2 * q4), a1 = ld2(rb + 2 * q4);
                const uint32_t a2 = ld2(ra + 8 + 2 * q4), a3 = ld2(rb + 8 + 2 * q4);
                // B[k = p][n = i]: a1[p0 + k + t][i0 + gq]; rows past NA1 meet dz2 = 0
                const int c = i0 + gq;
                const int r0 = min(p0 + 2 * q4 + t, NA1 - 1), r1 = min(p0 + 2 * q4 + 1 + t, NA1 - 1);
                const int r2 = min(p0 + 8 + 2 * q4 + t, NA1 - 1), r3 = min(p0 + 9 + 2 * q4 + t, NA1 - 1);
                const uint32_t b0 = pack2(s.a1[r0 * LDB + c], s.a1[r1 * LDB + c]);
                const uint32_t b1 = pack2(s.a1[r2 * LDB + c], s.a1[r3 * LDB + c]);
                mma_bf16(accw[slot], a0, a1, a2, a3, b0, b1);
            }
        }
        // da1[r][i] = sum_{t,o} w2[o][i][t] dz2[r - t][o]: M = r (10 tiles of 16 over NA1), N = i (4), K = (t, o) (10)
        // then dz1 = da1 * gelu'(z1), db1, dW1
        for (int m = warp; m < (NA1 + 15) / 16; m += nwarp) {
            const int r0 = m * 16;
            float acc[4][4] = {};
#pragma unroll
            for (int t = 0; t < KW; ++t) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    // A[r][o] = dz2[r - t][o] = dzP[(r - t + 4)][o]; rows beyond the buffer are zero-padded
                    const int ra = min(r0 + gq - t + 4, NZ2 + 7), rb = min(r0 + gq + 8 - t + 4, NZ2 + 7);
                    const uint32_t a0 = ld2(&dzP[ra * LDB + 16 * h + 2 * q4]);
                    const uint32_t a1 = ld2(&dzP[rb * LDB + 16 * h + 2 * q4]);
                    const uint32_t a2 = ld2(&dzP[ra * LDB + 16 * h + 8 + 2 * q4]);
                    const uint32_t a3 = ld2(&dzP[rb * LDB + 16 * h + 8 + 2 * q4]);
#pragma unroll
                    for (int nt = 0; nt < 4; ++nt) {
                        // B[k = o][n = i] = w2[o][i][t]: column i contiguous over o is w2[t] transposed;
                        // w2 smem is [t][o][i], so gather the two o values of the pair
                        const int ic = nt * 8 + gq;
                        const int o0 = 16 * h + 2 * q4;
                        const uint32_t b0 = pack2(s.w2[(t * CH + o0) * LDB + ic], s.w2[(t * CH + o0 + 1) * LDB + ic]);
                        const uint32_t b1 =
                            pack2(s.w2[(t * CH + o0 + 8) * LDB + ic], s.w2[(t * CH + o0 + 9) * LDB + ic]);
                        mma_bf16(acc[nt], a0, a1, a2, a3, b0, b1);
                    }
                }
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int r = r0 + gq + (e >= 2 ? 8 : 0), i = nt * 8 + 2 * q4 + (e & 1);
                    if (r < NA1) s.z1[r * LDF + i] = acc[nt][e] * gelu_grad(s.z1[r * LDF + i]);  // dz1 in place
                }
            }
        }
        __syncthreads();
        for (int k = threadIdx.x; k < CH * (KW + 1); k += blockDim.x) {
            const int o = k / (KW + 1), t = k % (KW + 1);
            float a = 0.0f;
            if (t < KW) {
                for (int r = 0; r < NA1; ++r) a = fmaf(s.z1[r * LDF + o], s.us[r + t], a);
                g[OW1 + o * KW + t] += a;
            } else {
                for (int r = 0; r < NA1; ++r) a += s.z1[r * LDF + o];
                g[OB1 + o] += a;
            }
        }
        __syncthreads();
    }
    // dW2 accumulators -> g (flat w2 is [o][i][t])
#pragma unroll
    for (int slot = 0; slot < 5; ++slot) {
        const int k = warp + slot * 8;
        const int mo = k / 20, nn = k % 20, t = nn / 4, i0 = (nn % 4) * 8;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int o = mo * 16 + gq + (e >= 2 ? 8 : 0), i = i0 + 2 * q4 + (e & 1);
            g[OW2 + (o * CH + i) * KW + t] += accw[slot][e];
        }
    }
    __syncthreads();
    float *row = partial + (int64_t)blockIdx.x * (NPARAM + 1);
    for (int i = threadIdx.x; i < NPARAM + 1; i += blockDim.x) row[i] = g[i];
}

// Sum the blocks' rows: out[j] = sum_b partial[b][j], j < NPARAM + 1.
__global__ void k_reduce(const float *__restrict__ partial, int rows, float *__restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= NPARAM + 1) return;
    float a = 0.0f;
    for (int b = 0; b < rows; ++b) a += partial[(int64_t)b * (NPARAM + 1) + j];
    out[j] = a;
}

// Adam on the FP32 master parameters.
__global__ void k_adam(float *__restrict__ theta, const float *__restrict__ grad, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= NTRAIN) return;
    const float gj = grad[j];
    const float mj = b1 * m[j] + (1.0f - b1) * gj;
    const float vj = b2 * v[j] + (1.0f - b2) * gj * gj;
    m[j] = mj;
    v[j] = vj;
    theta[j] -= lr * (mj / c1) / (sqrtf(vj / c2) + eps);
}

// Cell averages of `factor` fine cells: coarse[d][j] = mean(fine[d][factor j .. factor j + factor - 1]).
__global__ void k_coarse_grain(const double *__restrict__ fine, float *__restrict__ coarse, int64_t n_coarse_total,
                               int factor) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_coarse_total) return;
    double a = 0.0;
    for (int k = 0; k < factor; ++k) a += fine[j * factor + k];
    coarse[j] = (float)(a / factor);
}

// Rows idx[0..m) of the (domains x n) array src into the (m x n) array dst.
template <typename T>
__global__ void k_gather_rows(const T *__restrict__ src, const int32_t *__restrict__ idx, int64_t n,
                              T *__restrict__ dst) {
    const T *a = src + (int64_t)idx[blockIdx.x] * n;
    T *b = dst + (int64_t)blockIdx.x * n;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) b[j] = a[j];
}

// out[d] = ||a_d - b_d|| / ||b_d|| (FP64 sums) for the m rows of b; a's row d is
// row rows[d] of a when rows is given, else row d.  One block per row.
__global__ void __launch_bounds__(256) k_rel_l2(const float *__restrict__ a, const int32_t *__restrict__ rows,
                                                const float *__restrict__ b, int64_t n, double *__restrict__ out) {
    const float *x = a + (int64_t)(rows ? rows[blockIdx.x] : (int)blockIdx.x) * n;
    const float *y = b + (int64_t)blockIdx.x * n;
    double s1 = 0.0, s2 = 0.0;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const double d = (double)x[j] - (double)y[j];
        s1 += d * d;
        s2 += (double)y[j] * (double)y[j];
    }
    __shared__ double r1[256], r2[256];
    r1[threadIdx.x] = s1;
    r2[threadIdx.x] = s2;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) {
            r1[threadIdx.x] += r1[threadIdx.x + k];
            r2[threadIdx.x] += r2[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sqrt(r1[0] / r2[0]);
}

constexpr size_t smem_bytes() { return sizeof(Smem); }
constexpr size_t smem_fwd_bytes() { return offsetof(Smem, a2); }

}  // namespace cl
}  // namespace sw

using namespace sw;

namespace {

int closure_check(sw_ctx *ctx, int32_t n_dom, int64_t n) {
    if (!ctx || n_dom < 1 || n < cl::TOUT || n % cl::TOUT) return SW_ERR_SIZE;
    return SW_OK;
}

// The kernels' shared-memory limits, once per device (the attribute belongs to
// the current device): a bit per device 0..63, set again on every call above.
cudaError_t allow_smem() {
    static std::atomic<uint64_t> done{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = (dev >= 0 && dev < 64) ? (uint64_t(1) << dev) : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(cl::k_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cl::smem_fwd_bytes());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(cl::k_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cl::smem_fwd_bytes());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(cl::k_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cl::smem_bytes());
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
    return e;
}

// The closure calls run on the context's stream, a non-blocking one: order
// them after the work already queued on the legacy default stream (where a
// torch caller's default-stream copies of their inputs are).
int after_legacy(sw_ctx *ctx) {
    SW_CUDA(ctx, cudaEventRecord(ctx->e0, cudaStreamLegacy));
    SW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->e0, 0));
    return SW_OK;
}

// Stage theta's layer-2 weights for the forward kernels (stream-ordered before them).
int stage_w2(sw_ctx *ctx, const float *theta, const uint4 **w2p) {
    if (!ctx->d_w2p) SW_CUDA(ctx, cudaMalloc(&ctx->d_w2p, (size_t)cl::W2P_WORDS * 16));
    const int total = cl::KW * cl::CH * cl::LDB;
    cl::k_pack_w2<<<(total + 255) / 256, 256, 0, ctx->stream>>>(theta, static_cast<__nv_bfloat16 *>(ctx->d_w2p));
    SW_CUDA(ctx, cudaGetLastError());
    *w2p = static_cast<const uint4 *>(ctx->d_w2p);
    return SW_OK;
}

}  // namespace

extern "C" {

int sw_closure_infer(sw_ctx *ctx, const float *theta, const float *u, float *delta, int32_t n_dom, int64_t n) {
    int rc = closure_check(ctx, n_dom, n);
    if (rc) return rc;
    if (!theta || !u || !delta) return SW_ERR_ARG;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    if ((rc = after_legacy(ctx)) != SW_OK) return rc;
    SW_CUDA(ctx, allow_smem());
    const int64_t tiles = n / cl::TOUT;
    const uint4 *w2p = nullptr;
    rc = stage_w2(ctx, theta, &w2p);
    if (rc) return rc;
    cl::k_infer<<<(unsigned)(tiles * n_dom), cl::THREADS, cl::smem_fwd_bytes(), ctx->stream>>>(theta, w2p, u, delta, n,
                                                                                                tiles);
    SW_CUDA(ctx, cudaGetLastError());
    SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SW_OK;
}

}  // extern "C"

namespace {
// The coarse steps of sw_closure_step, enqueued on ctx's stream without
// waiting for them (ctx->d_work is their second row buffer).
int closure_enqueue(sw_ctx *ctx, const sw_config *coarse, const float *theta, float *u, int32_t n_dom, int64_t n,
                    int64_t n_steps, int32_t use_closure) {
    int rc = closure_check(ctx, n_dom, n);
    if (rc) return rc;
    if (!coarse || !u || (use_closure && !theta)) return SW_ERR_ARG;
    if (coarse->problem != SW_KS || coarse->precision != 4) return fail(ctx, SW_ERR_UNSUPPORTED, "closure steps KS FP32");
    if (coarse->flags != 0) return fail(ctx, SW_ERR_UNSUPPORTED, "closure steps take no sw_config.flags");
    sw_config c = *coarse;
    c.nx = n;
    sw_constants k;
    sw_constants_of(&c, &k);
    const Params<float> p = make_params<float>(c, k);
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    if ((rc = after_legacy(ctx)) != SW_OK) return rc;
    SW_CUDA(ctx, allow_smem());
    SW_CUDA(ctx, grow_dev(&ctx->d_work, &ctx->n_work, sizeof(float) * (size_t)n * n_dom));
    float *alt = static_cast<float *>(ctx->d_work), *cur = u;
    const int64_t tiles = n / cl::TOUT;
    const uint4 *w2p = nullptr;
    if (use_closure) {
        rc = stage_w2(ctx, theta, &w2p);
        if (rc) return rc;
    }
    for (int64_t i = 0; i < n_steps; ++i) {
        cl::k_step<<<(unsigned)(tiles * n_dom), cl::THREADS, cl::smem_fwd_bytes(), ctx->stream>>>(
            theta, w2p, p, cur, alt, n, tiles, use_closure);
        std::swap(cur, alt);
    }
    SW_CUDA(ctx, cudaGetLastError());
    if (cur != u) SW_CUDA(ctx, cudaMemcpyAsync(u, cur, sizeof(float) * (size_t)n * n_dom, cudaMemcpyDeviceToDevice,
                                               ctx->stream));
    return SW_OK;
}
}  // namespace

extern "C" {

int sw_closure_step(sw_ctx *ctx, const sw_config *coarse, const float *theta, float *u, int32_t n_dom, int64_t n,
                    int64_t n_steps, int32_t use_closure, sw_result *out) {
    if (!ctx) return SW_ERR_ARG;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    SW_CUDA(ctx, cudaEventRecord(ctx->k0, ctx->stream));
    const int rc = closure_enqueue(ctx, coarse, theta, u, n_dom, n, n_steps, use_closure);
    if (rc) return rc;
    SW_CUDA(ctx, cudaEventRecord(ctx->k1, ctx->stream));
    SW_CUDA(ctx, cudaEventSynchronize(ctx->k1));
    if (out) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->k0, ctx->k1);
        std::memset(out, 0, sizeof(*out));
        out->n_steps = n_steps;
        out->t_final = n_steps * coarse->dt;
        out->kernel_ms = out->elapsed_ms = ms;
        out->launches = n_steps;
    }
    return SW_OK;
}

int sw_closure_grad(sw_ctx *ctx, const float *theta, const float *u, const float *target, const int64_t *rows,
                    int32_t n_dom, int64_t n, float *grad_and_loss) {
    int rc = closure_check(ctx, n_dom, n);
    if (rc) return rc;
    if (!theta || !u || !target || !grad_and_loss) return SW_ERR_ARG;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    if ((rc = after_legacy(ctx)) != SW_OK) return rc;
    SW_CUDA(ctx, allow_smem());
    const int64_t tiles_per = n / cl::TOUT, n_tiles = tiles_per * n_dom;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t grid = std::min<int64_t>(n_tiles, (int64_t)sms * 2);
    SW_CUDA(ctx, grow_dev(&ctx->d_io, &ctx->n_io, sizeof(float) * (size_t)grid * (cl::NPARAM + 1)));
    float *partial = static_cast<float *>(ctx->d_io);
    const float scale = 1.0f / (float)((double)n_dom * n);
    cl::k_grad<<<(unsigned)grid, cl::THREADS, cl::smem_bytes(), ctx->stream>>>(theta, u, target, rows, partial, n,
                                                                                tiles_per, n_tiles, scale);
    SW_CUDA(ctx, cudaGetLastError());
    cl::k_reduce<<<(cl::NPARAM + 1 + 255) / 256, 256, 0, ctx->stream>>>(partial, (int)grid, grad_and_loss);
    SW_CUDA(ctx, cudaGetLastError());
    SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SW_OK;
}

int sw_closure_adam(sw_ctx *ctx, float *theta, const float *grad, float *m, float *v, int32_t step, float lr) {
    if (!ctx || !theta || !grad || !m || !v || step < 1) return SW_ERR_ARG;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    const int rc = after_legacy(ctx);
    if (rc) return rc;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
    cl::k_adam<<<(cl::NTRAIN + 255) / 256, 256, 0, ctx->stream>>>(theta, grad, m, v, lr, b1, b2, 1e-8f, c1, c2);
    SW_CUDA(ctx, cudaGetLastError());
    return SW_OK;
}

int sw_closure_train(sw_ctx *ctx, float *theta, const float *inputs, const float *targets, int64_t n_samples,
                     int64_t n, int32_t batch, int32_t steps, float lr, uint64_t seed, float *loss_host) {
    int rc = closure_check(ctx, batch, n);
    if (rc) return rc;
    if (!theta || !inputs || !targets || n_samples < 1 || steps < 0) return SW_ERR_ARG;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    if ((rc = after_legacy(ctx)) != SW_OK) return rc;
    // Adam moments and a gradient row live in one allocation owned by this call
    float *buf = nullptr;
    int64_t *rows = nullptr;
    SW_CUDA(ctx, cudaMalloc(&buf, sizeof(float) * (3 * cl::NPARAM + 2)));
    cudaError_t e = cudaMalloc(&rows, sizeof(int64_t) * (size_t)batch);
    if (e != cudaSuccess) {
        cudaFree(buf);
        return cuda_fail(ctx, e, "cudaMalloc rows");
    }
    float *m = buf, *v = buf + cl::NPARAM, *grad = buf + 2 * cl::NPARAM;
    cudaMemsetAsync(buf, 0, sizeof(float) * 2 * cl::NPARAM, ctx->stream);
    std::vector<int64_t> host_rows((size_t)batch);
    uint64_t st = seed ? seed : 0x9E3779B97F4A7C15ull;
    for (int32_t s = 0; s < steps && rc == SW_OK; ++s) {
        for (auto &r : host_rows) {  // splitmix64 draws of the minibatch rows
            st += 0x9E3779B97F4A7C15ull;
            uint64_t z = st;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            r = (int64_t)((z ^ (z >> 31)) % (uint64_t)n_samples);
        }
        e = cudaMemcpyAsync(rows, host_rows.data(), sizeof(int64_t) * batch, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "rows"); break; }
        rc = sw_closure_grad(ctx, theta, inputs, targets, rows, batch, n, grad);
        if (rc) break;
        if (loss_host) {
            e = cudaMemcpy(&loss_host[s], grad + cl::NPARAM, sizeof(float), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "loss"); break; }
        }
        rc = sw_closure_adam(ctx, theta, grad, m, v, s + 1, lr);
    }
    cudaStreamSynchronize(ctx->stream);
    cudaFree(rows);
    cudaFree(buf);
    return rc;
}

// Closure steps the ensemble runs in the first segment before the judge has
// picked a variant: about the time the judge's first segment takes beside them.
constexpr int64_t kSpeculativeSteps = 8;

int sw_closure_adaptive(sw_ctx *ctx, sw_ctx *judge, const sw_config *coarse, const sw_config *fine,
                        const float *theta, const double *fine0, int32_t n_dom, int64_t n_fine, int32_t factor,
                        int64_t coarse_steps, int64_t segment, double tau, int32_t shadow_every,
                        int32_t shadow_offset, float *u_out, sw_adaptive_info *info, double *log_out,
                        int32_t log_cap) {
    if (!ctx || !judge || judge == ctx || !coarse || !fine || !fine0 || !u_out || !info) return SW_ERR_ARG;
    if (factor < 1 || n_fine % factor || shadow_every < 1 || shadow_offset < 0 || shadow_offset >= shadow_every ||
        segment < 1 || coarse_steps < 0 || !(tau >= 0))
        return SW_ERR_ARG;
    if (judge->device != ctx->device) return fail(ctx, SW_ERR_ARG, "the judge context must be on the run's device");
    const int64_t n = n_fine / factor;
    int rc = closure_check(ctx, n_dom, n);
    if (rc) return rc;
    std::vector<int32_t> idx;
    for (int32_t d = shadow_offset; d < n_dom; d += shadow_every) idx.push_back(d);
    if (idx.empty()) return fail(ctx, SW_ERR_ARG, "the judge's sample is empty");
    const int32_t m = (int32_t)idx.size();
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    // run context scratch: the sample's coarse rows for each variant and the reference (m x n
    // floats each), the ensemble's state kept at the start of the first segment, errors,
    // indices (each at a 256-byte boundary)
    const size_t fb = sizeof(float) * (size_t)m * n, fbr = (fb + 255) & ~(size_t)255;
    const size_t ub = sizeof(float) * (size_t)n_dom * n, ubr = (ub + 255) & ~(size_t)255;
    SW_CUDA(ctx, grow_dev(&ctx->d_judge, &ctx->n_judge,
                          3 * fbr + ubr + 4 * sizeof(double) * m + sizeof(int32_t) * m + 64));
    // the coarse runs' second row buffer, sized for the ensemble before any run is enqueued
    SW_CUDA(ctx, grow_dev(&ctx->d_work, &ctx->n_work, ub));
    char *scratch = static_cast<char *>(ctx->d_judge);
    float *samp = reinterpret_cast<float *>(scratch), *samp2 = reinterpret_cast<float *>(scratch + fbr);
    float *ref = reinterpret_cast<float *>(scratch + 2 * fbr);
    float *u_kept = reinterpret_cast<float *>(scratch + 3 * fbr);
    double *err = reinterpret_cast<double *>(scratch + 3 * fbr + ubr);  // [2][m]
    int32_t *idx_d = reinterpret_cast<int32_t *>(err + 2 * m);
    SW_CUDA(ctx, grow_dev(&judge->d_judge, &judge->n_judge, sizeof(double) * (size_t)m * n_fine));
    double *shadow = static_cast<double *>(judge->d_judge);
    SW_CUDA(ctx, cudaMemcpy(idx_d, idx.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice));
    if ((rc = after_legacy(ctx)) != SW_OK) return rc;
    cudaStream_t s = ctx->stream;
    cl::k_gather_rows<double><<<m, 256, 0, s>>>(fine0, idx_d, n_fine, shadow);
    SW_CUDA(ctx, cudaGetLastError());
    SW_CUDA(ctx, cudaStreamSynchronize(s));
    if ((rc = sw_coarse_grain(ctx, fine0, u_out, (int64_t)n_dom * n, factor))) return rc;
    std::memset(info, 0, sizeof(*info));
    info->n_shadow = m;
    std::vector<int64_t> nx_s((size_t)m, n_fine);
    std::vector<double> h_err(2 * (size_t)m);
    sw_config fc = *fine;
    fc.time_mode = SW_TIME_STEPS;
    auto rel = [&](const float *a, const int32_t *rows, int slot) -> int {
        cl::k_rel_l2<<<m, 256, 0, s>>>(a, rows, ref, n, err + (size_t)slot * m);
        SW_CUDA(ctx, cudaGetLastError());
        return SW_OK;
    };
    auto stats = [&](int slot, double *mean, double *mx) {
        double a = 0.0, b = 0.0;
        for (int32_t d = 0; d < m; ++d) {
            a += h_err[(size_t)slot * m + d];
            b = std::max(b, h_err[(size_t)slot * m + d]);
        }
        *mean = a / m;
        *mx = b;
    };
    int64_t done = 0;
    int pick = -1;  // 0 plain, 1 closure
    double prev = 0.0;
    int32_t nlog = 0;
    while (done < coarse_steps) {
        const int64_t k = std::min(segment, coarse_steps - done);
        // Enqueued first, in this order on the run's stream: the sample's runs (both
        // variants in the first segment, later the variant the ensemble does not run),
        // then the ensemble's run of the pick.  The judge's segment runs meanwhile on its
        // own context, and the segment takes as long as the longer of the two.  The first
        // segment's pick is not known yet: the ensemble starts the closure for the first
        // kSpeculativeSteps steps (about the judge's time), its state at the segment's
        // start kept, then continues it, or runs the plain step from the kept state
        // should the sample pick that.  The results are those of running the pick alone.
        cl::k_gather_rows<float><<<m, 256, 0, s>>>(u_out, idx_d, n, samp);
        SW_CUDA(ctx, cudaGetLastError());
        int64_t started = 0;  // closure steps the ensemble ran ahead of the first pick
        if (pick < 0) {
            SW_CUDA(ctx, cudaMemcpyAsync(samp2, samp, fb, cudaMemcpyDeviceToDevice, s));
            if ((rc = closure_enqueue(ctx, coarse, theta, samp, m, n, k, 0))) return rc;
            if ((rc = closure_enqueue(ctx, coarse, theta, samp2, m, n, k, 1))) return rc;
            SW_CUDA(ctx, cudaMemcpyAsync(u_kept, u_out, ub, cudaMemcpyDeviceToDevice, s));
            started = std::min(k, kSpeculativeSteps);
            if ((rc = closure_enqueue(ctx, coarse, theta, u_out, n_dom, n, started, 1))) return rc;
        } else {
            if ((rc = closure_enqueue(ctx, coarse, theta, samp, m, n, k, 1 - pick))) return rc;
            if ((rc = closure_enqueue(ctx, coarse, theta, u_out, n_dom, n, k, pick))) return rc;
        }
        fc.n_steps = k * factor;
        if ((rc = sw_run_batch_device(judge, &fc, m, nx_s.data(), shadow, nullptr, nullptr))) return rc;
        if ((rc = sw_coarse_grain(judge, shadow, ref, (int64_t)m * n, factor))) return rc;
        int cur_slot, alt_slot;
        if (pick < 0) {  // first segment: the better variant on the sample runs the ensemble
            if ((rc = rel(samp, nullptr, 0))) return rc;
            if ((rc = rel(samp2, nullptr, 1))) return rc;
            SW_CUDA(ctx, cudaMemcpyAsync(h_err.data(), err, sizeof(double) * 2 * m, cudaMemcpyDeviceToHost, s));
            SW_CUDA(ctx, cudaStreamSynchronize(s));
            double m0, m1, x0, x1;
            stats(0, &m0, &x0);
            stats(1, &m1, &x1);
            pick = (m1 < m0) ? 1 : 0;
            if (pick == 0) {  // the plain step, from the kept state
                SW_CUDA(ctx, cudaMemcpyAsync(u_out, u_kept, ub, cudaMemcpyDeviceToDevice, s));
                if ((rc = sw_closure_step(ctx, coarse, theta, u_out, n_dom, n, k, 0, nullptr))) return rc;
            } else if (k > started) {  // the rest of the closure's segment
                if ((rc = sw_closure_step(ctx, coarse, theta, u_out, n_dom, n, k - started, 1, nullptr))) return rc;
            }
            cur_slot = pick;
            alt_slot = 1 - pick;
        } else {  // the ensemble ran the pick, the sample the other variant
            if ((rc = rel(u_out, idx_d, 0))) return rc;
            if ((rc = rel(samp, nullptr, 1))) return rc;
            SW_CUDA(ctx, cudaMemcpyAsync(h_err.data(), err, sizeof(double) * 2 * m, cudaMemcpyDeviceToHost, s));
            SW_CUDA(ctx, cudaStreamSynchronize(s));
            cur_slot = 0;
            alt_slot = 1;
        }
        double e, emax, eo, eomax;
        stats(cur_slot, &e, &emax);  // the certificate: the sample's mean relative L2 error
        stats(alt_slot, &eo, &eomax);
        done += k;
        if (log_out && nlog < log_cap) {
            double *row = log_out + 4 * (size_t)nlog;
            row[0] = (double)done;
            row[1] = pick;
            row[2] = e;
            row[3] = eo;
            ++nlog;
        }
        const double left = (double)(coarse_steps - done) / (double)k;  // segments still to run
        if (e > tau || e + std::max(e - prev, 0.0) * left > tau) {
            info->fallback = 1;
            break;
        }
        if (pick == 1) ++info->closure_segments;
        else ++info->plain_segments;
        info->shadow_mean_rel_l2 = e;
        info->shadow_max_rel_l2 = emax;
        prev = e;
        if (eo < e) pick = 1 - pick;
    }
    info->n_log = nlog;
    if (info->fallback) {  // every domain by the fine solver from fine0: the answer is the fine solution
        const size_t bytes = sizeof(double) * (size_t)n_dom * n_fine;
        SW_CUDA(ctx, grow_dev(&ctx->d_state, &ctx->n_state, bytes));
        SW_CUDA(ctx, cudaMemcpyAsync(ctx->d_state, fine0, bytes, cudaMemcpyDeviceToDevice, s));
        SW_CUDA(ctx, cudaStreamSynchronize(s));
        std::vector<int64_t> nx_all((size_t)n_dom, n_fine);
        fc.n_steps = coarse_steps * factor;
        if ((rc = sw_run_batch_device(ctx, &fc, n_dom, nx_all.data(), ctx->d_state, nullptr, nullptr))) return rc;
        if ((rc = sw_coarse_grain(ctx, static_cast<const double *>(ctx->d_state), u_out, (int64_t)n_dom * n, factor)))
            return rc;
    }
    return SW_OK;
}

int sw_coarse_grain(sw_ctx *ctx, const double *fine, float *coarse, int64_t n_coarse_total, int32_t factor) {
    if (!ctx || !fine || !coarse || n_coarse_total < 1 || factor < 1) return SW_ERR_ARG;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    const int rc = after_legacy(ctx);
    if (rc) return rc;
    cl::k_coarse_grain<<<(unsigned)((n_coarse_total + 255) / 256), 256, 0, ctx->stream>>>(fine, coarse,
                                                                                            n_coarse_total, factor);
    SW_CUDA(ctx, cudaGetLastError());
    SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SW_OK;
}

}  // extern "C"
