// dsmc_mlp.cu -- the learned (sigma_T c_R)max of a cell.
//
// A 3-64-64-1 perceptron with SiLU activations maps a cell's state
// (log number density, log translational temperature, speed ratio) to
// log (sigma_T c_R)max.  Weights and activations are BF16, every sum is
// accumulated in FP32, and the 64x64 layer runs on the tensor cores
// (mma.sync m16n8k16 bf16 -> f32).  The network is trained on the GPU by this
// file's own forward/backward kernel and an Adam kernel, and evaluated per
// cell inside the step (noTimeCounter then draws its candidates against the
// prediction).
//
// No reference counterpart: dsmcFoam+ keeps only the running maximum
// (noTimeCounter.C:243-246), which stays as the fallback.
//
// Arithmetic of one sample (the CPU oracle restates exactly this):
//   xn  = bf16((x - mu) / sd)                       3 inputs
//   z1  = b1 + W1 xn            a1 = bf16(silu(z1))  64
//   z2  = b2 + W2 a1            a2 = bf16(silu(z2))  64   (tensor cores)
//   out = b3 + w3 . a2                               1
// with every weight read as its bf16 rounding.  Training minimises the mean
// of (out - (y - ymu)/ysd)^2 (or, with a quantile level tau in (0, 1), the
// pinball loss whose minimiser is the tau-quantile of the target given the
// inputs); the backward pass keeps dout, dz2 and dz1 in FP32 and feeds
// bf16(dz2) to the two tensor-core products (dW2 and dh1).
//
// Gradients are reduced without atomics: every CTA writes its partial sums
// and the Adam kernel adds them in CTA order, so training is reproducible.

#include <cuda_bf16.h>

#include <cstring>
#include <string>
#include <vector>

#include "dsmc_kernels.h"
#include "hystrath_gb300.h"

namespace dsmc {
namespace mlp {

constexpr int H = 64;
constexpr int IN = 3;
// flat parameter vector
constexpr int OFF_W1 = 0;                 // [H][IN]
constexpr int OFF_B1 = OFF_W1 + H * IN;   // [H]
constexpr int OFF_W2 = OFF_B1 + H;        // [H][H], row = output
constexpr int OFF_B2 = OFF_W2 + H * H;    // [H]
constexpr int OFF_W3 = OFF_B2 + H;        // [H]
constexpr int OFF_B3 = OFF_W3 + H;        // [1]
constexpr int NPARAM = OFF_B3 + 1;        // 4481
static_assert(NPARAM == DSMC_MLP_NPARAM, "parameter count");
// small gradients reduced per CTA by one thread each: dW1, db1, db2, dw3, db3
constexpr int NSMALL = H * IN + H + H + H + 1;   // 385

constexpr int WARPS = 4;
constexpr int ROWS = WARPS * 16;          // samples per chunk (one m16 tile per warp)
constexpr int LDW = H + 8;                // padded row of the bf16 weight tiles (conflict-free fragments)
constexpr uint32_t TAG_MLP = 7;

struct Norm {
    float mu[IN], sd[IN], ymu, ysd;
};

__device__ __forceinline__ float bf(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ void mma16816(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Weights of one CTA in shared memory (bf16 values; the small ones as float).
struct Weights {
    __nv_bfloat16 W2[H][LDW];    // [out][in]
    __nv_bfloat16 W2T[H][LDW];   // [in][out]
    float W1[H][IN], b1[H], b2[H], w3[H], b3;
};

__device__ void load_weights(Weights& w, const __nv_bfloat16* __restrict__ p) {
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) {
        const int o = i / H, j = i % H;
        const __nv_bfloat16 v = p[OFF_W2 + i];
        w.W2[o][j] = v;
        w.W2T[j][o] = v;
    }
    for (int i = threadIdx.x; i < H * IN; i += blockDim.x) w.W1[i / IN][i % IN] = __bfloat162float(p[OFF_W1 + i]);
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        w.b1[i] = __bfloat162float(p[OFF_B1 + i]);
        w.b2[i] = __bfloat162float(p[OFF_B2 + i]);
        w.w3[i] = __bfloat162float(p[OFF_W3 + i]);
    }
    if (threadIdx.x == 0) w.b3 = __bfloat162float(p[OFF_B3]);
}

__device__ __forceinline__ float layer1(const Weights& w, const float* xn, int o) {
    float z = w.b1[o];
    z = fmaf(w.W1[o][0], xn[0], z);
    z = fmaf(w.W1[o][1], xn[1], z);
    z = fmaf(w.W1[o][2], xn[2], z);
    return z;
}

// Forward pass of one m16 tile by one warp.  xr[0..1] are the normalised
// inputs of rows g and g+8 (lane = 4g + t).  Returns z2 (C layout: tile nt,
// c0 c1 at row g, cols 8nt+2t+{0,1}; c2 c3 at row g+8) and out for rows g
// and g+8; stores a1 to a1s (row-major) when given.
__device__ __forceinline__ void forward_tile(const Weights& w, const float (*xr)[IN], float z2[8][4],
                                             float out[2], __nv_bfloat16 (*a1s)[LDW], int rowBase) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // layer 1 straight into the A fragments of layer 2
    uint32_t A[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        const int f0 = 16 * kt + 2 * t, f1 = f0 + 8;
        float v[2][4];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            v[r][0] = bf(silu(layer1(w, xr[r], f0)));
            v[r][1] = bf(silu(layer1(w, xr[r], f0 + 1)));
            v[r][2] = bf(silu(layer1(w, xr[r], f1)));
            v[r][3] = bf(silu(layer1(w, xr[r], f1 + 1)));
        }
        A[kt][0] = pack2(v[0][0], v[0][1]);
        A[kt][1] = pack2(v[1][0], v[1][1]);
        A[kt][2] = pack2(v[0][2], v[0][3]);
        A[kt][3] = pack2(v[1][2], v[1][3]);
        if (a1s) {
            *reinterpret_cast<uint32_t*>(&a1s[rowBase + g][f0]) = A[kt][0];
            *reinterpret_cast<uint32_t*>(&a1s[rowBase + g + 8][f0]) = A[kt][1];
            *reinterpret_cast<uint32_t*>(&a1s[rowBase + g][f1]) = A[kt][2];
            *reinterpret_cast<uint32_t*>(&a1s[rowBase + g + 8][f1]) = A[kt][3];
        }
    }
    // layer 2 on the tensor cores
    float o0 = 0.f, o1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        const int n = 8 * nt + g;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&w.W2[n][16 * kt + 2 * t]);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&w.W2[n][16 * kt + 2 * t + 8]);
            mma16816(c, A[kt][0], A[kt][1], A[kt][2], A[kt][3], b0, b1);
        }
        const int f = 8 * nt + 2 * t;
        z2[nt][0] = c[0] + w.b2[f];
        z2[nt][1] = c[1] + w.b2[f + 1];
        z2[nt][2] = c[2] + w.b2[f];
        z2[nt][3] = c[3] + w.b2[f + 1];
        // layer 3 partial dot products
        o0 = fmaf(bf(silu(z2[nt][0])), w.w3[f], o0);
        o0 = fmaf(bf(silu(z2[nt][1])), w.w3[f + 1], o0);
        o1 = fmaf(bf(silu(z2[nt][2])), w.w3[f], o1);
        o1 = fmaf(bf(silu(z2[nt][3])), w.w3[f + 1], o1);
    }
    o0 += __shfl_xor_sync(0xFFFFFFFFu, o0, 1);
    o0 += __shfl_xor_sync(0xFFFFFFFFu, o0, 2);
    o1 += __shfl_xor_sync(0xFFFFFFFFu, o1, 1);
    o1 += __shfl_xor_sync(0xFFFFFFFFu, o1, 2);
    out[0] = o0 + w.b3;
    out[1] = o1 + w.b3;
}

__device__ __forceinline__ void normalise(const Norm& nm, const float* x, float* xn) {
#pragma unroll
    for (int k = 0; k < IN; ++k) xn[k] = bf((x[k] - nm.mu[k]) / nm.sd[k]);
}

// ------------------------------------------------------------ training
struct TrainSmem {
    Weights w;
    __nv_bfloat16 a1[ROWS][LDW];
    float a2[ROWS][H];
    float dz2[ROWS][H];
    float dz1[ROWS][H];
    float xn[ROWS][IN];
    float dout[ROWS];
    float sqerr[ROWS];
    float small[NSMALL];
    float loss;
};

// One Adam step's gradient (or, with sampleSeed == 0, the gradient over rows
// [0, n) of X in order).  Each CTA loops over chunks of ROWS samples and
// writes its partial sums to partial[blockIdx.x][NPARAM] and its loss sum to
// lossPartial[blockIdx.x].
__global__ void __launch_bounds__(WARPS * 32)
k_mlp_grad(const __nv_bfloat16* __restrict__ wb, Norm nm, const float* __restrict__ X, const float* __restrict__ Y,
           long long nData, int batch, unsigned long long seed, int step, float tau, float* partial,
           float* lossPartial) {
    extern __shared__ __align__(16) unsigned char smraw[];
    TrainSmem& sm = *reinterpret_cast<TrainSmem*>(smraw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    load_weights(sm.w, wb);
    for (int i = threadIdx.x; i < NSMALL; i += blockDim.x) sm.small[i] = 0.f;
    if (threadIdx.x == 0) sm.loss = 0.f;
    __syncthreads();
    float dW2[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) dW2[nt][0] = dW2[nt][1] = dW2[nt][2] = dW2[nt][3] = 0.f;
    const int nChunks = (batch + ROWS - 1) / ROWS;
    const float invB = 1.0f / (float)batch;
    for (int ch = blockIdx.x; ch < nChunks; ch += gridDim.x) {
        // ---- forward + first backward stage, one m16 tile per warp
        const int rowBase = warp * 16;
        float xr[2][IN], yr[2];
        bool valid[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int row = rowBase + g + 8 * r;
            const long long b = (long long)ch * ROWS + row;
            valid[r] = b < batch;
            long long idx = b;
            if (seed && valid[r]) {
                uint32_t o[4];
                philox4x32_10((uint32_t)b, (uint32_t)step, 0u, TAG_MLP, (uint32_t)seed, (uint32_t)(seed >> 32), o);
                idx = (long long)(u01_from(o[0], o[1]) * (double)nData);
                if (idx >= nData) idx = nData - 1;
            }
            float x[IN] = {0.f, 0.f, 0.f};
            yr[r] = 0.f;
            if (valid[r]) {
                x[0] = X[3 * idx]; x[1] = X[3 * idx + 1]; x[2] = X[3 * idx + 2];
                yr[r] = (Y[idx] - nm.ymu) / nm.ysd;
            }
            normalise(nm, x, xr[r]);
            if (t == 0) {
#pragma unroll
                for (int k = 0; k < IN; ++k) sm.xn[row][k] = valid[r] ? xr[r][k] : 0.f;
            }
        }
        float z2[8][4], out[2];
        forward_tile(sm.w, xr, z2, out, sm.a1, rowBase);
        float dout[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const float e = out[r] - yr[r];
            float l, d;
            if (tau > 0.f) {           // pinball: tau (y - out)+ + (1 - tau) (out - y)+
                l = e < 0.f ? -tau * e : (1.f - tau) * e;
                d = e < 0.f ? -tau : (1.f - tau);
            } else {
                l = e * e;
                d = 2.0f * e;
            }
            dout[r] = valid[r] ? d * invB : 0.f;
            if (t == 0) {
                sm.dout[rowBase + g + 8 * r] = dout[r];
                sm.sqerr[rowBase + g + 8 * r] = valid[r] ? l : 0.f;
            }
        }
        // dz2 = dout w3 silu'(z2), kept in FP32; bf16(dz2) is the A operand of dh1
        uint32_t Ad[4][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int f = 8 * nt + 2 * t;
            float d[4];
            d[0] = dout[0] * sm.w.w3[f] * dsilu(z2[nt][0]);
            d[1] = dout[0] * sm.w.w3[f + 1] * dsilu(z2[nt][1]);
            d[2] = dout[1] * sm.w.w3[f] * dsilu(z2[nt][2]);
            d[3] = dout[1] * sm.w.w3[f + 1] * dsilu(z2[nt][3]);
            sm.dz2[rowBase + g][f] = d[0];
            sm.dz2[rowBase + g][f + 1] = d[1];
            sm.dz2[rowBase + g + 8][f] = d[2];
            sm.dz2[rowBase + g + 8][f + 1] = d[3];
            sm.a2[rowBase + g][f] = bf(silu(z2[nt][0]));
            sm.a2[rowBase + g][f + 1] = bf(silu(z2[nt][1]));
            sm.a2[rowBase + g + 8][f] = bf(silu(z2[nt][2]));
            sm.a2[rowBase + g + 8][f + 1] = bf(silu(z2[nt][3]));
            // C layout of n-tiles 2k and 2k+1 is the A layout of k-tile k
            const int kt = nt >> 1;
            if ((nt & 1) == 0) {
                Ad[kt][0] = pack2(d[0], d[1]);
                Ad[kt][1] = pack2(d[2], d[3]);
            } else {
                Ad[kt][2] = pack2(d[0], d[1]);
                Ad[kt][3] = pack2(d[2], d[3]);
            }
        }
        // dh1 = bf16(dz2) W2 (tensor cores), dz1 = dh1 silu'(z1)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            const int n = 8 * nt + g;
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&sm.w.W2T[n][16 * kt + 2 * t]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&sm.w.W2T[n][16 * kt + 2 * t + 8]);
                mma16816(c, Ad[kt][0], Ad[kt][1], Ad[kt][2], Ad[kt][3], b0, b1);
            }
            const int f = 8 * nt + 2 * t;
            sm.dz1[rowBase + g][f] = c[0] * dsilu(layer1(sm.w, xr[0], f));
            sm.dz1[rowBase + g][f + 1] = c[1] * dsilu(layer1(sm.w, xr[0], f + 1));
            sm.dz1[rowBase + g + 8][f] = c[2] * dsilu(layer1(sm.w, xr[1], f));
            sm.dz1[rowBase + g + 8][f + 1] = c[3] * dsilu(layer1(sm.w, xr[1], f + 1));
        }
        __syncthreads();
        // ---- dW2 += bf16(dz2)^T a1: warp w owns output rows [16w, 16w+16)
#pragma unroll
        for (int ks = 0; ks < ROWS / 16; ++ks) {
            const int s0 = 16 * ks + 2 * t;
            const int o0 = 16 * warp + g;
            const uint32_t a0 = pack2(sm.dz2[s0][o0], sm.dz2[s0 + 1][o0]);
            const uint32_t a1 = pack2(sm.dz2[s0][o0 + 8], sm.dz2[s0 + 1][o0 + 8]);
            const uint32_t a2 = pack2(sm.dz2[s0 + 8][o0], sm.dz2[s0 + 9][o0]);
            const uint32_t a3 = pack2(sm.dz2[s0 + 8][o0 + 8], sm.dz2[s0 + 9][o0 + 8]);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int i = 8 * nt + g;
                __nv_bfloat162 v0, v1;
                v0.x = sm.a1[s0][i]; v0.y = sm.a1[s0 + 1][i];
                v1.x = sm.a1[s0 + 8][i]; v1.y = sm.a1[s0 + 9][i];
                mma16816(dW2[nt], a0, a1, a2, a3, *reinterpret_cast<uint32_t*>(&v0),
                         *reinterpret_cast<uint32_t*>(&v1));
            }
        }
        // ---- small gradients, one output per thread
        for (int q = threadIdx.x; q < NSMALL; q += blockDim.x) {
            float acc = 0.f;
            if (q < H * IN) {
                const int o = q / IN, k = q % IN;
                for (int s = 0; s < ROWS; ++s) acc = fmaf(sm.dz1[s][o], sm.xn[s][k], acc);
            } else if (q < H * IN + H) {
                const int o = q - H * IN;
                for (int s = 0; s < ROWS; ++s) acc += sm.dz1[s][o];
            } else if (q < H * IN + 2 * H) {
                const int o = q - H * IN - H;
                for (int s = 0; s < ROWS; ++s) acc += sm.dz2[s][o];
            } else if (q < H * IN + 3 * H) {
                const int o = q - H * IN - 2 * H;
                for (int s = 0; s < ROWS; ++s) acc = fmaf(sm.dout[s], sm.a2[s][o], acc);
            } else {
                for (int s = 0; s < ROWS; ++s) acc += sm.dout[s];
            }
            sm.small[q] += acc;
        }
        if (threadIdx.x == 0) {
            float l = 0.f;
            for (int s = 0; s < ROWS; ++s) l += sm.sqerr[s];
            sm.loss += l;
        }
        __syncthreads();
    }
    // ---- this CTA's partial sums
    float* P = partial + (size_t)blockIdx.x * NPARAM;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int o = 16 * warp + g, i = 8 * nt + 2 * t;
        P[OFF_W2 + o * H + i] = dW2[nt][0];
        P[OFF_W2 + o * H + i + 1] = dW2[nt][1];
        P[OFF_W2 + (o + 8) * H + i] = dW2[nt][2];
        P[OFF_W2 + (o + 8) * H + i + 1] = dW2[nt][3];
    }
    for (int q = threadIdx.x; q < NSMALL; q += blockDim.x) {
        int p;
        if (q < H * IN) p = OFF_W1 + q;
        else if (q < H * IN + H) p = OFF_B1 + (q - H * IN);
        else if (q < H * IN + 2 * H) p = OFF_B2 + (q - H * IN - H);
        else if (q < H * IN + 3 * H) p = OFF_W3 + (q - H * IN - 2 * H);
        else p = OFF_B3;
        P[p] = sm.small[q];
    }
    if (threadIdx.x == 0) lossPartial[blockIdx.x] = sm.loss;
}

// Sum of the CTA partials in CTA order; with lr > 0 also the Adam update
// (beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected) of the FP32 master
// weights and their bf16 copies.
__global__ void k_mlp_adam(const float* __restrict__ partial, const float* __restrict__ lossPartial, int nPart,
                           float* master, __nv_bfloat16* wb, float* m, float* v, float* gradOut, float lr, int step,
                           float invBatch, float* lossOut) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0 && lossOut) {
        float l = 0.f;
        for (int c = 0; c < nPart; ++c) l += lossPartial[c];
        *lossOut = l * invBatch;
    }
    if (p >= NPARAM) return;
    float gsum = 0.f;
    for (int c = 0; c < nPart; ++c) gsum += partial[(size_t)c * NPARAM + p];
    if (gradOut) gradOut[p] = gsum;
    if (!(lr > 0.f)) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float mm = b1 * m[p] + (1.f - b1) * gsum;
    const float vv = b2 * v[p] + (1.f - b2) * gsum * gsum;
    m[p] = mm;
    v[p] = vv;
    const float mh = mm / (1.f - powf(b1, (float)step));
    const float vh = vv / (1.f - powf(b2, (float)step));
    const float w = master[p] - lr * mh / (sqrtf(vh) + eps);
    master[p] = w;
    wb[p] = __float2bfloat16_rn(w);
}

__global__ void k_mlp_round(const float* master, __nv_bfloat16* wb) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NPARAM) wb[p] = __float2bfloat16_rn(master[p]);
}

// ------------------------------------------------------------ inference
// One warp per 16 rows.  X rows are (x0, x1, x2, valid); out[r] =
// exp(ymu + ysd * net(x) + margin) when asExp, else ymu + ysd * net(x); rows
// with valid == 0 get 0.
__global__ void __launch_bounds__(WARPS * 32)
k_mlp_infer(const __nv_bfloat16* __restrict__ wb, Norm nm, const float4* __restrict__ X, long long n, float* out,
            int asExp, float margin, const long long* step, int every) {
    if (step && every > 0 && (*step % every) != 0) return;
    __shared__ Weights w;
    load_weights(w, wb);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long nTiles = (n + 15) / 16;
    for (long long tile = (long long)blockIdx.x * WARPS + (threadIdx.x >> 5); tile < nTiles;
         tile += (long long)gridDim.x * WARPS) {
        float xr[2][IN];
        bool valid[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const long long row = tile * 16 + g + 8 * r;
            float x[IN] = {0.f, 0.f, 0.f};
            valid[r] = false;
            if (row < n) {
                const float4 q = X[row];
                x[0] = q.x; x[1] = q.y; x[2] = q.z;
                valid[r] = q.w != 0.f;
            }
            normalise(nm, x, xr[r]);
        }
        float z2[8][4], o[2];
        forward_tile(w, xr, z2, o, nullptr, 0);
        if (t == 0) {
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const long long row = tile * 16 + g + 8 * r;
                if (row >= n) continue;
                const float y = nm.ymu + nm.ysd * o[r];
                out[row] = !valid[r] ? 0.f : asExp ? expf(y + margin) : y;
            }
        }
    }
}

int sm_count() {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

}  // namespace mlp

// The model as the cloud sees it: device pointers and normalisation.
struct MlpModel {
    float* master = nullptr;         // [NPARAM] FP32
    __nv_bfloat16* wb = nullptr;     // [NPARAM] bf16 copy used by the kernels
    float* m = nullptr;
    float* v = nullptr;
    float* partial = nullptr;        // [grid][NPARAM]
    float* lossPartial = nullptr;    // [grid]
    float* loss = nullptr;           // [1]
    float* grad = nullptr;           // [NPARAM]
    float tau = 0.f;                 // 0: mean squared error; (0, 1): pinball loss at this quantile
    float* X = nullptr;              // training rows [nData][3]
    float* Y = nullptr;              // [nData]
    long long nData = 0;
    long long capData = 0;
    int grid = 0;
    int adamStep = 0;
    mlp::Norm norm{};
    cudaStream_t stream = nullptr;
    std::string err;
};

void mlp_launch_infer(const MlpModel* m, const float4* X, long long n, float* out, float margin,
                      const long long* step, int every, cudaStream_t st) {
    const long long tiles = (n + 15) / 16;
    long long blocks = (tiles + mlp::WARPS - 1) / mlp::WARPS;
    const long long cap = (long long)mlp::sm_count() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    mlp::k_mlp_infer<<<(int)blocks, mlp::WARPS * 32, 0, st>>>(m->wb, m->norm, X, n, out, 1, margin, step, every);
}

}  // namespace dsmc

using dsmc::MlpModel;
namespace mlp = dsmc::mlp;

struct dsmc_mlp : MlpModel {};

namespace {

thread_local std::string g_mlp_err;

int mfail(dsmc_mlp* m, int code, const std::string& msg) {
    if (m) m->err = msg;
    g_mlp_err = msg;
    return code;
}

#define MLP_TRY(m, call)                                                                     \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return mfail(m, DSMC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t train_smem() { return sizeof(mlp::TrainSmem); }

int run_grad(dsmc_mlp* m, const float* X, const float* Y, long long nData, int batch, unsigned long long seed,
             int step) {
    mlp::k_mlp_grad<<<m->grid, mlp::WARPS * 32, train_smem(), m->stream>>>(
        m->wb, m->norm, X, Y, nData, batch, seed, step, m->tau, m->partial, m->lossPartial);
    return DSMC_OK;
}

}  // namespace

extern "C" {

int dsmc_mlp_nparam(void) { return mlp::NPARAM; }

int dsmc_mlp_create(dsmc_mlp** out) {
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return mfail(nullptr, DSMC_ERR_NO_DEVICE, "no CUDA device: the learned selection has no CPU path");
    dsmc_mlp* m = new dsmc_mlp();
    m->grid = 2 * mlp::sm_count();
    MLP_TRY(m, cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    MLP_TRY(m, cudaFuncSetAttribute(mlp::k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
    MLP_TRY(m, cudaMalloc(&m->master, sizeof(float) * mlp::NPARAM));
    MLP_TRY(m, cudaMalloc(&m->wb, sizeof(__nv_bfloat16) * mlp::NPARAM));
    MLP_TRY(m, cudaMalloc(&m->m, sizeof(float) * mlp::NPARAM));
    MLP_TRY(m, cudaMalloc(&m->v, sizeof(float) * mlp::NPARAM));
    MLP_TRY(m, cudaMalloc(&m->grad, sizeof(float) * mlp::NPARAM));
    MLP_TRY(m, cudaMalloc(&m->partial, sizeof(float) * mlp::NPARAM * m->grid));
    MLP_TRY(m, cudaMalloc(&m->lossPartial, sizeof(float) * m->grid));
    MLP_TRY(m, cudaMalloc(&m->loss, sizeof(float)));
    MLP_TRY(m, cudaMemset(m->master, 0, sizeof(float) * mlp::NPARAM));
    MLP_TRY(m, cudaMemset(m->wb, 0, sizeof(__nv_bfloat16) * mlp::NPARAM));
    MLP_TRY(m, cudaMemset(m->m, 0, sizeof(float) * mlp::NPARAM));
    MLP_TRY(m, cudaMemset(m->v, 0, sizeof(float) * mlp::NPARAM));
    for (int k = 0; k < mlp::IN; ++k) { m->norm.mu[k] = 0.f; m->norm.sd[k] = 1.f; }
    m->norm.ymu = 0.f;
    m->norm.ysd = 1.f;
    *out = m;
    return DSMC_OK;
}

void dsmc_mlp_destroy(dsmc_mlp* m) {
    if (!m) return;
    cudaStreamSynchronize(m->stream);
    void* ptrs[] = {m->master, m->wb, m->m, m->v, m->grad, m->partial, m->lossPartial, m->loss, m->X, m->Y};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    cudaStreamDestroy(m->stream);
    delete m;
}

const char* dsmc_mlp_last_error(const dsmc_mlp* m) { return m ? m->err.c_str() : g_mlp_err.c_str(); }

int dsmc_mlp_set_params(dsmc_mlp* m, const float* params, const float* norm8) {
    MLP_TRY(m, cudaStreamSynchronize(m->stream));
    if (params) {
        MLP_TRY(m, cudaMemcpy(m->master, params, sizeof(float) * mlp::NPARAM, cudaMemcpyHostToDevice));
        mlp::k_mlp_round<<<(mlp::NPARAM + 255) / 256, 256, 0, m->stream>>>(m->master, m->wb);
        MLP_TRY(m, cudaMemsetAsync(m->m, 0, sizeof(float) * mlp::NPARAM, m->stream));
        MLP_TRY(m, cudaMemsetAsync(m->v, 0, sizeof(float) * mlp::NPARAM, m->stream));
        m->adamStep = 0;
    }
    if (norm8) {
        for (int k = 0; k < mlp::IN; ++k) {
            if (!(norm8[mlp::IN + k] > 0.f)) return mfail(m, DSMC_ERR_INVALID, "input scale must be positive");
            m->norm.mu[k] = norm8[k];
            m->norm.sd[k] = norm8[mlp::IN + k];
        }
        if (!(norm8[7] > 0.f)) return mfail(m, DSMC_ERR_INVALID, "output scale must be positive");
        m->norm.ymu = norm8[6];
        m->norm.ysd = norm8[7];
    }
    MLP_TRY(m, cudaStreamSynchronize(m->stream));
    return DSMC_OK;
}

int dsmc_mlp_get_params(dsmc_mlp* m, float* params, float* norm8) {
    MLP_TRY(m, cudaStreamSynchronize(m->stream));
    if (params) MLP_TRY(m, cudaMemcpy(params, m->master, sizeof(float) * mlp::NPARAM, cudaMemcpyDeviceToHost));
    if (norm8) {
        for (int k = 0; k < mlp::IN; ++k) {
            norm8[k] = m->norm.mu[k];
            norm8[mlp::IN + k] = m->norm.sd[k];
        }
        norm8[6] = m->norm.ymu;
        norm8[7] = m->norm.ysd;
    }
    return DSMC_OK;
}

int dsmc_mlp_set_loss(dsmc_mlp* m, float tau) {
    if (!(tau >= 0.f && tau < 1.f)) return mfail(m, DSMC_ERR_INVALID, "tau must be 0 (squared error) or in (0, 1)");
    m->tau = tau;
    return DSMC_OK;
}

int dsmc_mlp_set_data(dsmc_mlp* m, const float* X, const float* Y, long long n) {
    if (n <= 0) return mfail(m, DSMC_ERR_INVALID, "no training rows");
    MLP_TRY(m, cudaStreamSynchronize(m->stream));
    if (n > m->capData) {
        if (m->X) cudaFree(m->X);
        if (m->Y) cudaFree(m->Y);
        m->X = m->Y = nullptr;
        MLP_TRY(m, cudaMalloc(&m->X, sizeof(float) * 3 * n));
        MLP_TRY(m, cudaMalloc(&m->Y, sizeof(float) * n));
        m->capData = n;
    }
    MLP_TRY(m, cudaMemcpy(m->X, X, sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
    MLP_TRY(m, cudaMemcpy(m->Y, Y, sizeof(float) * n, cudaMemcpyHostToDevice));
    m->nData = n;
    return DSMC_OK;
}

int dsmc_mlp_train(dsmc_mlp* m, int steps, int batch, float lr, unsigned long long seed, float* loss_out) {
    if (m->nData <= 0) return mfail(m, DSMC_ERR_INVALID, "no training data (dsmc_mlp_set_data)");
    if (steps < 0 || batch <= 0 || !(lr > 0.f)) return mfail(m, DSMC_ERR_INVALID, "bad training arguments");
    if (seed == 0) seed = 1;
    std::vector<float> losses(loss_out ? steps : 0);
    float* dLoss = nullptr;
    if (loss_out && steps > 0) MLP_TRY(m, cudaMalloc(&dLoss, sizeof(float) * steps));
    for (int s = 0; s < steps; ++s) {
        ++m->adamStep;
        run_grad(m, m->X, m->Y, m->nData, batch, seed, m->adamStep);
        mlp::k_mlp_adam<<<(mlp::NPARAM + 255) / 256, 256, 0, m->stream>>>(
            m->partial, m->lossPartial, m->grid, m->master, m->wb, m->m, m->v, nullptr, lr, m->adamStep,
            1.0f / (float)batch, dLoss ? dLoss + s : nullptr);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess && dLoss) e = cudaMemcpy(loss_out, dLoss, sizeof(float) * steps, cudaMemcpyDeviceToHost);
    if (dLoss) cudaFree(dLoss);
    if (e != cudaSuccess) return mfail(m, DSMC_ERR_CUDA, std::string("training: ") + cudaGetErrorString(e));
    return DSMC_OK;
}

int dsmc_mlp_grad(dsmc_mlp* m, const float* X, const float* Y, int n, float* grad_out, float* loss_out) {
    if (n <= 0) return mfail(m, DSMC_ERR_INVALID, "no rows");
    float *dX = nullptr, *dY = nullptr;
    MLP_TRY(m, cudaMalloc(&dX, sizeof(float) * 3 * n));
    MLP_TRY(m, cudaMalloc(&dY, sizeof(float) * n));
    MLP_TRY(m, cudaMemcpy(dX, X, sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
    MLP_TRY(m, cudaMemcpy(dY, Y, sizeof(float) * n, cudaMemcpyHostToDevice));
    run_grad(m, dX, dY, n, n, 0ull, 0);
    mlp::k_mlp_adam<<<(mlp::NPARAM + 255) / 256, 256, 0, m->stream>>>(
        m->partial, m->lossPartial, m->grid, m->master, m->wb, m->m, m->v, m->grad, 0.f, 1, 1.0f / (float)n, m->loss);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess) e = cudaMemcpy(grad_out, m->grad, sizeof(float) * mlp::NPARAM, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && loss_out) e = cudaMemcpy(loss_out, m->loss, sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dX);
    cudaFree(dY);
    if (e != cudaSuccess) return mfail(m, DSMC_ERR_CUDA, std::string("gradient: ") + cudaGetErrorString(e));
    return DSMC_OK;
}

int dsmc_mlp_predict(dsmc_mlp* m, const float* X, long long n, float* out) {
    if (n <= 0) return DSMC_OK;
    std::vector<float> x4(4 * n);
    for (long long i = 0; i < n; ++i) {
        x4[4 * i] = X[3 * i];
        x4[4 * i + 1] = X[3 * i + 1];
        x4[4 * i + 2] = X[3 * i + 2];
        x4[4 * i + 3] = 1.f;
    }
    float4* dX = nullptr;
    float* dO = nullptr;
    MLP_TRY(m, cudaMalloc(&dX, sizeof(float4) * n));
    MLP_TRY(m, cudaMalloc(&dO, sizeof(float) * n));
    MLP_TRY(m, cudaMemcpy(dX, x4.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    const long long tiles = (n + 15) / 16;
    long long blocks = (tiles + mlp::WARPS - 1) / mlp::WARPS;
    if (blocks > (long long)m->grid * 4) blocks = (long long)m->grid * 4;
    mlp::k_mlp_infer<<<(int)blocks, mlp::WARPS * 32, 0, m->stream>>>(m->wb, m->norm, dX, n, dO, 0, 0.f, nullptr, 0);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess) e = cudaMemcpy(out, dO, sizeof(float) * n, cudaMemcpyDeviceToHost);
    cudaFree(dX);
    cudaFree(dO);
    if (e != cudaSuccess) return mfail(m, DSMC_ERR_CUDA, std::string("inference: ") + cudaGetErrorString(e));
    return DSMC_OK;
}

}  // extern "C"
