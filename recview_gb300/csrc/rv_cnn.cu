// Centre-proposal network (no reference counterpart: RecView's centre choice is a person looking at
// an axis-scan sweep, source/gazoDoc.cpp:1994-2024).  A small BF16 CNN that reads four detector
// rows of a sinogram and regresses the rotation-centre offset plus its own uncertainty; it only
// narrows the plain sweep (rv_centre.cu), whose criterion still picks the centre.
//
//   input  X[N, 4, H, W]  bf16 (four detector rows; 256 views x 512 bins at the production size)
//   6 x { conv 3x3 pad 1 + bias -> ReLU (R, bf16) -> 2x2 average pool (P, bf16) }
//        channels 4 -> 32 -> 32 -> 64 -> 64 -> 128 -> 128
//   flatten P6 -> FC 128 + bias -> ReLU -> FC 2 + bias -> (mu, s)
//   loss   mean_n 0.5 exp(-s) (y - mu)^2 + 0.5 s   (Gaussian negative log-likelihood; sigma^2 = e^s)
//
// Activations are stored in bf16 (halving their traffic), every sum runs in FP32, master weights,
// gradients and Adam moments are FP32.  The network is ~1.5 GFLOP per sample forward; the
// convolutions are SIMT register-tiled kernels (2x2 outputs x 8 channels per thread, input tile
// and weights staged in shared memory), which is ample at this size -- a training epoch of 20k
// samples is a few seconds.
//
// Parameter order in the flat FP32 vector (also the order RvCentreNetGetParams uses):
//   w0[32,4,3,3] b0[32] w1[32,32,3,3] b1[32] ... w5[128,128,3,3] b5[128]
//   f0w[128, 128*(H/64)*(W/64)] f0b[128] f1w[2,128] f1b[2]
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "rv_internal.h"

namespace rv {
namespace cnn {

constexpr int kLayers = 6;
constexpr int kChannels[kLayers + 1] = {4, 32, 32, 64, 64, 128, 128};
constexpr int kHidden = 128;

typedef __nv_bfloat16 bf16;

// ---- convolution forward, fused bias + ReLU + 2x2 average pool --------------------------------
// Block: 16 x 8 threads, each 2x2 outputs of COB output channels -> a 16-row x 32-column output
// tile.  Input channels are staged 8 at a time ((16+2) x (32+2) floats each) with their weights.
constexpr int kTX = 16, kTY = 8, kCI = 8, kCOB = 8;
constexpr int kTileW = 2 * kTX, kTileH = 2 * kTY;            // 32 x 16 outputs
constexpr int kInW = kTileW + 2, kInH = kTileH + 2;          // 34 x 18 inputs

template <bool FLIP_FROM_DZ>
__device__ __forceinline__ float conv_in_value(const void* src, const bf16* R, int n, int c, int C, int H, int W,
                                               int y, int x) {
    if (y < 0 || y >= H || x < 0 || x >= W || c >= C) return 0.0f;
    if (!FLIP_FROM_DZ) {
        return __bfloat162float(static_cast<const bf16*>(src)[(((size_t)n * C + c) * H + y) * W + x]);
    } else {
        // gradient wrt the pre-activation of a layer whose pooled output has gradient dP:
        // dZ = (R > 0) * dP[y/2][x/2] / 4
        const size_t ri = (((size_t)n * C + c) * H + y) * W + x;
        if (!(__bfloat162float(R[ri]) > 0.0f)) return 0.0f;
        const float* dP = static_cast<const float*>(src);
        return 0.25f * dP[(((size_t)n * C + c) * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)];
    }
}

// Forward (FLIP = false): out(y,x)[co] = sum_ci sum_dy,dx in(y+dy-1, x+dx-1)[ci] w[co][ci][dy][dx].
// Data gradient (FLIP = true): the same loop over dZ (built from dP and R on the fly) with the
// kernel flipped and the channel roles swapped: dX(y,x)[ci] = sum_co dZ(y+dy-1, x+dx-1)[co]
// w[co][ci][2-dy][2-dx], written in FP32.
template <bool FLIP>
__global__ void __launch_bounds__(kTX * kTY) k_conv3x3(const void* src, const bf16* R, const float* w, const float* bias,
                                                       bf16* outR, bf16* outP, float* outD, int Cs, int Co, int H,
                                                       int W, int n_groups) {
    __shared__ float tin[kCI][kInH][kInW];
    __shared__ float tw[kCOB][kCI][9];
    const int n = blockIdx.z / n_groups, g = blockIdx.z % n_groups;
    const int co0 = g * kCOB;
    const int x0 = blockIdx.x * kTileW, y0 = blockIdx.y * kTileH;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
    float acc[kCOB][4];
#pragma unroll
    for (int o = 0; o < kCOB; o++)
#pragma unroll
        for (int k = 0; k < 4; k++) acc[o][k] = 0.0f;

    for (int c0 = 0; c0 < Cs; c0 += kCI) {
        __syncthreads();
        for (int e = tid; e < kCI * kInH * kInW; e += kTX * kTY) {
            const int c = e / (kInH * kInW), r = (e / kInW) % kInH, q = e % kInW;
            tin[c][r][q] = conv_in_value<FLIP>(src, R, n, c0 + c, Cs, H, W, y0 + r - 1, x0 + q - 1);
        }
        for (int e = tid; e < kCOB * kCI * 9; e += kTX * kTY) {
            const int o = e / (kCI * 9), c = (e / 9) % kCI, k = e % 9;
            float v = 0.0f;
            if (co0 + o < Co && c0 + c < Cs) {
                if (!FLIP) v = w[(((size_t)(co0 + o) * Cs) + c0 + c) * 9 + k];
                else v = w[(((size_t)(c0 + c) * Co) + co0 + o) * 9 + (8 - k)];   // w[co][ci] flipped
            }
            tw[o][c][k] = v;
        }
        __syncthreads();
#pragma unroll 2
        for (int c = 0; c < kCI; c++) {
            float p[4][4];
#pragma unroll
            for (int r = 0; r < 4; r++)
#pragma unroll
                for (int q = 0; q < 4; q++) p[r][q] = tin[c][2 * ty + r][2 * tx + q];
#pragma unroll
            for (int o = 0; o < kCOB; o++) {
                float wk[9];
#pragma unroll
                for (int k = 0; k < 9; k++) wk[k] = tw[o][c][k];
#pragma unroll
                for (int oy = 0; oy < 2; oy++)
#pragma unroll
                    for (int ox = 0; ox < 2; ox++) {
                        float s = acc[o][oy * 2 + ox];
#pragma unroll
                        for (int dy = 0; dy < 3; dy++)
#pragma unroll
                            for (int dx = 0; dx < 3; dx++) s = fmaf(p[oy + dy][ox + dx], wk[dy * 3 + dx], s);
                        acc[o][oy * 2 + ox] = s;
                    }
            }
        }
    }
    const int y = y0 + 2 * ty, x = x0 + 2 * tx;
    if (y >= H || x >= W) return;
#pragma unroll
    for (int o = 0; o < kCOB; o++) {
        const int co = co0 + o;
        if (co >= Co) break;
        if (!FLIP) {
            const float b = bias[co];
            float sum = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int yy = y + (k >> 1), xx = x + (k & 1);
                const bf16 rv = __float2bfloat16_rn(fmaxf(acc[o][k] + b, 0.0f));
                outR[(((size_t)n * Co + co) * H + yy) * W + xx] = rv;
                sum += __bfloat162float(rv);
            }
            outP[(((size_t)n * Co + co) * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)] = __float2bfloat16_rn(sum * 0.25f);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int yy = y + (k >> 1), xx = x + (k & 1);
                outD[(((size_t)n * Co + co) * H + yy) * W + xx] = acc[o][k];
            }
        }
    }
}

// ---- convolution weight / bias gradient ---------------------------------------------------
// dW[co][ci][dy][dx] = sum_n,y,x dZ[n][co][y][x] A[n][ci][y+dy-1][x+dx-1],  db[co] = sum dZ.
// Block: 128 threads = 16 output-channel pairs x 8 input channels, one 8 x 32 pixel tile, looping
// over the batch; partial sums are added to the FP32 gradient with one atomic per weight.
constexpr int kWT_H = 8, kWT_W = 32, kWCO = 32, kWCI = 8;

__global__ void __launch_bounds__(128) k_conv3x3_wgrad(const bf16* A, const float* dP, const bf16* R, float* dW,
                                                        float* db, int N, int Cin, int Cout, int H, int W,
                                                        int ci_groups) {
    __shared__ float dz[kWCO][kWT_H][kWT_W];
    __shared__ float ta[kWCI][kWT_H + 2][kWT_W + 2];
    const int x0 = blockIdx.x * kWT_W, y0 = blockIdx.y * kWT_H;
    const int cog = blockIdx.z / ci_groups, cig = blockIdx.z % ci_groups;
    const int co_base = cog * kWCO, ci_base = cig * kWCI;
    const int tid = threadIdx.x;
    const int cp = tid >> 3, cil = tid & 7;
    float acc0[9], acc1[9], b0 = 0.0f, b1 = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; k++) acc0[k] = acc1[k] = 0.0f;
    for (int n = 0; n < N; n++) {
        __syncthreads();
        for (int e = tid; e < kWCO * kWT_H * kWT_W; e += 128) {
            const int o = e / (kWT_H * kWT_W), r = (e / kWT_W) % kWT_H, q = e % kWT_W;
            dz[o][r][q] = conv_in_value<true>(dP, R, n, co_base + o, Cout, H, W, y0 + r, x0 + q);
        }
        for (int e = tid; e < kWCI * (kWT_H + 2) * (kWT_W + 2); e += 128) {
            const int c = e / ((kWT_H + 2) * (kWT_W + 2)), r = (e / (kWT_W + 2)) % (kWT_H + 2), q = e % (kWT_W + 2);
            ta[c][r][q] = conv_in_value<false>(A, nullptr, n, ci_base + c, Cin, H, W, y0 + r - 1, x0 + q - 1);
        }
        __syncthreads();
        for (int r = 0; r < kWT_H; r++) {
            for (int q = 0; q < kWT_W; q++) {
                const float z0 = dz[2 * cp][r][q], z1 = dz[2 * cp + 1][r][q];
                b0 += z0;
                b1 += z1;
#pragma unroll
                for (int dy = 0; dy < 3; dy++)
#pragma unroll
                    for (int dx = 0; dx < 3; dx++) {
                        const float a = ta[cil][r + dy][q + dx];
                        acc0[dy * 3 + dx] = fmaf(z0, a, acc0[dy * 3 + dx]);
                        acc1[dy * 3 + dx] = fmaf(z1, a, acc1[dy * 3 + dx]);
                    }
            }
        }
    }
    const int ci = ci_base + cil;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int co = co_base + 2 * cp + h;
        if (co >= Cout) continue;
        if (ci < Cin)
#pragma unroll
            for (int k = 0; k < 9; k++) atomicAdd(&dW[((size_t)co * Cin + ci) * 9 + k], h ? acc1[k] : acc0[k]);
        if (cil == 0 && cig == 0) atomicAdd(&db[co], h ? b1 : b0);
    }
}

// ---- fully connected layers ---------------------------------------------------------------
// out[n][j] = act(sum_k in[n][k] W[j][k] + b[j]); one warp per (n, j).
__global__ void k_fc_fwd(const void* in, int in_bf16, const float* Wt, const float* b, float* out, int N, int K, int J,
                         int relu) {
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (wid >= N * J) return;
    const int n = wid / J, j = wid % J;
    float s = 0.0f;
    for (int k = lane; k < K; k += 32) {
        const float v = in_bf16 ? __bfloat162float(static_cast<const bf16*>(in)[(size_t)n * K + k])
                                : static_cast<const float*>(in)[(size_t)n * K + k];
        s = fmaf(v, Wt[(size_t)j * K + k], s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        s += b[j];
        out[(size_t)n * J + j] = relu ? fmaxf(s, 0.0f) : s;
    }
}

// dW[j][k] = sum_n dout[n][j] in[n][k]; db[j] = sum_n dout[n][j] (thread per weight)
__global__ void k_fc_wgrad(const void* in, int in_bf16, const float* dout, float* dW, float* db, int N, int K, int J) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)J * K) return;
    const int j = (int)(i / K), k = (int)(i % K);
    float s = 0.0f, sb = 0.0f;
    for (int n = 0; n < N; n++) {
        const float v = in_bf16 ? __bfloat162float(static_cast<const bf16*>(in)[(size_t)n * K + k])
                                : static_cast<const float*>(in)[(size_t)n * K + k];
        const float d = dout[(size_t)n * J + j];
        s = fmaf(d, v, s);
        sb += d;
    }
    dW[i] += s;
    if (k == 0) db[j] += sb;
}

// din[n][k] = (sum_j dout[n][j] W[j][k]) * (mask ? (mask[n][k] > 0) : 1)
__global__ void k_fc_dgrad(const float* dout, const float* Wt, const float* mask, float* din, int N, int K, int J) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)N * K) return;
    const int n = (int)(i / K), k = (int)(i % K);
    float s = 0.0f;
    for (int j = 0; j < J; j++) s = fmaf(dout[(size_t)n * J + j], Wt[(size_t)j * K + k], s);
    if (mask && !(mask[i] > 0.0f)) s = 0.0f;
    din[i] = s;
}

// Gaussian NLL of o[n] = (mu, s) against y[n]; dout = d(mean loss)/do; loss_out = mean loss
__global__ void k_nll(const float* o, const float* y, float* dout, float* loss_out, int N) {
    __shared__ float red[32];
    float l = 0.0f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const float mu = o[2 * n], s = o[2 * n + 1];
        const float e = expf(-s), d = y[n] - mu;
        l += 0.5f * e * d * d + 0.5f * s;
        dout[2 * n] = -e * d / (float)N;
        dout[2 * n + 1] = (0.5f - 0.5f * e * d * d) / (float)N;
    }
    for (int o2 = 16; o2 > 0; o2 >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o2);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        *loss_out = t / (float)N;
    }
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                       float eps, float bc1, float bc2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}


// ---- tensor-core convolutions (mma.sync m16n8k16, BF16 operands, FP32 accumulation) ---------------
// Implicit GEMMs over the 3x3 taps.  Fragment layouts of m16n8k16 (g = lane / 4, t = lane % 4):
//   A 16x16 row-major:  a0 (g, 2t..2t+1)  a1 (g+8, 2t..)  a2 (g, 2t+8..)  a3 (g+8, 2t+8..)
//   B 16x8 column-major: b0 (k 2t..2t+1, n g)  b1 (k 2t+8.., n g)
//   C 16x8:             c0 (g, 2t)  c1 (g, 2t+1)  c2 (g+8, 2t)  c3 (g+8, 2t+1)
// Two bf16 values of a register are adjacent in shared memory (lower index in the low half).
// FP32 operands (weights, the pre-activation gradients dZ) are split into bf16 hi + lo
// (x = hi + lo to about 2^-16 relative), and their products are summed from two or three MMAs,
// so the convolutions keep the precision of the FP32 SIMT kernels; activations are stored in
// bf16 and enter exactly.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ unsigned ld_pair(const bf16* p) { return *reinterpret_cast<const unsigned*>(p); }
__device__ __forceinline__ void split_bf16(float v, bf16& hi, bf16& lo) {
    hi = __float2bfloat16_rn(v);
    lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// Weights of one layer rearranged for the tensor-core kernels, as bf16 hi / lo:
//   forward  wf[tap][co][ci]  (co padded to cop, ci to csp = multiple of 16): w[co][ci][tap]
//   dgrad    wd[tap][ci][co]  (ci padded to cip, co to cop16): w[co][ci][8 - tap] (flipped)
__global__ void k_prep_weights(const float* w, int Cin, int Cout, int csp, int cop, int cip, int cop16, bf16* wf_hi,
                               bf16* wf_lo, bf16* wd_hi, bf16* wd_lo) {
    const long long nf = 9LL * cop * csp, nd = 9LL * cip * cop16;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nf + nd; i += (long long)gridDim.x * blockDim.x) {
        float v = 0.0f;
        bf16 hi, lo;
        if (i < nf) {
            const int tap = (int)(i / ((long long)cop * csp)), co = (int)((i / csp) % cop), ci = (int)(i % csp);
            if (co < Cout && ci < Cin) v = w[((size_t)co * Cin + ci) * 9 + tap];
            split_bf16(v, hi, lo);
            wf_hi[i] = hi;
            wf_lo[i] = lo;
        } else {
            const long long j = i - nf;
            const int tap = (int)(j / ((long long)cip * cop16)), ci = (int)((j / cop16) % cip), co = (int)(j % cop16);
            if (co < Cout && ci < Cin) v = w[((size_t)co * Cin + ci) * 9 + (8 - tap)];
            split_bf16(v, hi, lo);
            wd_hi[j] = hi;
            wd_lo[j] = lo;
        }
    }
}

// Forward (DGRAD = false): output tile 8 rows x 32 columns of sample n, output channels
// [co0, co0 + 8 NT); GEMM rows = pixels (16 consecutive columns of one row per M-tile), columns =
// output channels, K = (tap, input channel) in chunks of 16 channels per tap.  Warp w owns rows
// 2(w/2), 2(w/2)+1 and columns 16(w%2) .. +15, so the 2x2 pool of the epilogue stays inside the
// warp (the column partner is the lane 4 apart).  Epilogue: R = bf16(relu(acc + bias)),
// P = bf16(0.25 (R00 + R01 + R10 + R11)) with the SIMT kernel's summation order.
// Data gradient (DGRAD = true): the same GEMM on dZ (bf16 hi in src, lo in R, from k_dz) with
// the flipped kernel and the channel roles swapped; dX is written in FP32.  wp_hi / wp_lo: the layer's weights from k_prep_weights (forward or dgrad
// layout), row length csp (a multiple of 16), cop rows per tap.
constexpr int kTcTH = 8, kTcTW = 32, kTcCS = 24;   // tile rows, columns; channel stride (16 + 8)
constexpr int kTcAElems = (kTcTH + 2) * (kTcTW + 2) * kTcCS;
template <int NT, bool DGRAD>
__global__ void __launch_bounds__(256, 2) k_conv3x3_tc(const void* src, const bf16* R, const bf16* wp_hi, const bf16* wp_lo,
                                                    int csp, int cop, const float* bias, bf16* outR, bf16* outP,
                                                    float* outD, int Cs, int Co, int H, int W, int n_groups) {
    constexpr int TH = kTcTH, TW = kTcTW, CS = kTcCS, NG = 8 * NT, NA = DGRAD ? 2 : 1;
    extern __shared__ __align__(16) bf16 tc_smem[];
    bf16* sA = tc_smem;                          // [NA][(TH+2) (TW+2) pixels][CS]
    bf16* sB = tc_smem + NA * kTcAElems;         // [2][9 taps][NG][CS]
    constexpr int BE = 9 * NG * CS;
    const int n = blockIdx.z / n_groups, grp = blockIdx.z % n_groups;
    const int co0 = grp * NG;
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int wr = (warp >> 1) * 2, wx = (warp & 1) * 16;
    float acc[2][NT][4];
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int j = 0; j < NT; j++)
#pragma unroll
            for (int k = 0; k < 4; k++) acc[m][j][k] = 0.0f;
    for (int c0 = 0; c0 < Cs; c0 += 16) {
        __syncthreads();
        // A tile: (TH+2) x (TW+2) pixels x 16 channels, zero outside the image and above Cs
        for (int e = tid; e < 16 * (TH + 2) * (TW + 2); e += 256) {
            const int c = e / ((TH + 2) * (TW + 2)), rem = e % ((TH + 2) * (TW + 2));
            const int r = rem / (TW + 2), q = rem % (TW + 2);
            const int y = y0 + r - 1, x = x0 + q - 1, ch = c0 + c;
            const int at = (r * (TW + 2) + q) * CS + c;
            if (!DGRAD) {
                bf16 v = __float2bfloat16_rn(0.0f);
                if (ch < Cs && y >= 0 && y < H && x >= 0 && x < W)
                    v = static_cast<const bf16*>(src)[(((size_t)n * Cs + ch) * H + y) * W + x];
                sA[at] = v;
            } else {   // dZ as hi (src) and lo (R), from k_dz
                bf16 hi = __float2bfloat16_rn(0.0f), lo = hi;
                if (ch < Cs && y >= 0 && y < H && x >= 0 && x < W) {
                    const size_t ri = (((size_t)n * Cs + ch) * H + y) * W + x;
                    hi = static_cast<const bf16*>(src)[ri];
                    lo = R[ri];
                }
                sA[at] = hi;
                sA[kTcAElems + at] = lo;
            }
        }
        // B: 16 input channels of each (tap, output channel) row, 16-byte copies of hi and lo
        for (int e = tid; e < 9 * NG * 2; e += 256) {
            const int tap = e / (NG * 2), o = (e >> 1) % NG, half = e & 1;
            const size_t gsrc = ((size_t)tap * cop + co0 + o) * csp + c0 + 8 * half;
            const int at = (tap * NG + o) * CS + 8 * half;
            *reinterpret_cast<uint4*>(sB + at) = *reinterpret_cast<const uint4*>(wp_hi + gsrc);
            *reinterpret_cast<uint4*>(sB + BE + at) = *reinterpret_cast<const uint4*>(wp_lo + gsrc);
        }
        __syncthreads();
#pragma unroll 1
        for (int tap = 0; tap < 9; tap++) {
            const int dy = tap / 3, dx = tap % 3;
            unsigned a[NA][2][4];
#pragma unroll
            for (int h = 0; h < NA; h++)
#pragma unroll
                for (int m = 0; m < 2; m++) {
                    const bf16* row = sA + h * kTcAElems + ((wr + m + dy) * (TW + 2) + wx + dx) * CS;
                    a[h][m][0] = ld_pair(row + g * CS + 2 * t);
                    a[h][m][1] = ld_pair(row + (g + 8) * CS + 2 * t);
                    a[h][m][2] = ld_pair(row + g * CS + 2 * t + 8);
                    a[h][m][3] = ld_pair(row + (g + 8) * CS + 2 * t + 8);
                }
#pragma unroll
            for (int j = 0; j < NT; j++) {
                const bf16* bp = sB + (tap * NG + j * 8 + g) * CS + 2 * t;
                const unsigned bh0 = ld_pair(bp), bh1 = ld_pair(bp + 8);
                const unsigned bl0 = ld_pair(bp + BE), bl1 = ld_pair(bp + BE + 8);
#pragma unroll
                for (int m = 0; m < 2; m++) {
                    mma_bf16(acc[m][j], a[0][m], bl0, bl1);
                    if (DGRAD) mma_bf16(acc[m][j], a[NA - 1][m], bh0, bh1);
                    mma_bf16(acc[m][j], a[0][m], bh0, bh1);
                }
            }
        }
    }
    // epilogue: lane holds, per M-tile m and N-tile j, pixels (x0 + wx + g) and (+8) of row
    // y0 + wr + m, channels co0 + 8j + 2t and +1
#pragma unroll
    for (int j = 0; j < NT; j++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {                 // channel 2t + h
            const int co = co0 + j * 8 + 2 * t + h;
#pragma unroll
            for (int px = 0; px < 2; px++) {          // pixel g + 8 px
                const int x = x0 + wx + g + 8 * px;
                if (!DGRAD) {
                    const float b = co < Co ? bias[co] : 0.0f;
                    float r[2];
#pragma unroll
                    for (int m = 0; m < 2; m++) {
                        const bf16 rv = __float2bfloat16_rn(fmaxf(acc[m][j][2 * px + h] + b, 0.0f));
                        r[m] = __bfloat162float(rv);
                        const int y = y0 + wr + m;
                        if (co < Co && y < H && x < W) outR[(((size_t)n * Co + co) * H + y) * W + x] = rv;
                    }
                    // column partner (x + 1) lives in lane + 4; even columns write the pooled value
                    const float r0n = __shfl_down_sync(0xffffffffu, r[0], 4);
                    const float r1n = __shfl_down_sync(0xffffffffu, r[1], 4);
                    if (!(g & 1)) {
                        const int y = y0 + wr;
                        float sum = r[0];
                        sum += r0n;
                        sum += r[1];
                        sum += r1n;
                        if (co < Co && y < H && x < W)
                            outP[(((size_t)n * Co + co) * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)] =
                                __float2bfloat16_rn(sum * 0.25f);
                    }
                } else {
#pragma unroll
                    for (int m = 0; m < 2; m++) {
                        const int y = y0 + wr + m;
                        if (co < Co && y < H && x < W) outD[(((size_t)n * Co + co) * H + y) * W + x] = acc[m][j][2 * px + h];
                    }
                }
            }
        }
    }
}
// Forward of a layer with at most 4 input channels (the network's first layer): K = (tap, input
// channel) packed as k = 4 tap + ci, so 16 consecutive k cover four taps and the nine taps take
// three K steps (k 36..47 carry zero weights) instead of nine steps of 16 mostly-zero channels.
// Same tile, warp layout and epilogue as k_conv3x3_tc<4, false>; weights from k_prep_weights'
// forward layout (row length csp = 16).
constexpr int kC4Elems = (kTcTH + 2) * (kTcTW + 2) * 4;
__global__ void __launch_bounds__(256, 2) k_conv3x3_tc_c4(const bf16* src, const bf16* wp_hi, const bf16* wp_lo, int csp,
                                                          int cop, const float* bias, bf16* outR, bf16* outP, int Cs,
                                                          int Co, int H, int W, int n_groups) {
    constexpr int TH = kTcTH, TW = kTcTW, CS = kTcCS, NT = 4, NG = 32, KS = 3;
    __shared__ __align__(16) bf16 sA[kC4Elems];                  // [pixel][4 channels]
    __shared__ __align__(16) bf16 sB[2][KS * NG * CS];           // [hi/lo][k step][co][16 k]
    const int n = blockIdx.z / n_groups, grp = blockIdx.z % n_groups;
    const int co0 = grp * NG;
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int wr = (warp >> 1) * 2, wx = (warp & 1) * 16;
    for (int e = tid; e < kC4Elems; e += 256) {
        const int c = e & 3, px = e >> 2;
        const int r = px / (TW + 2), q = px % (TW + 2);
        const int y = y0 + r - 1, x = x0 + q - 1;
        bf16 v = __float2bfloat16_rn(0.0f);
        if (c < Cs && y >= 0 && y < H && x >= 0 && x < W) v = src[(((size_t)n * Cs + c) * H + y) * W + x];
        sA[e] = v;
    }
    for (int e = tid; e < KS * NG * 16; e += 256) {
        const int ks = e / (NG * 16), o = (e / 16) % NG, kl = e % 16;
        const int tap = ks * 4 + kl / 4, ci = kl % 4;
        bf16 hi = __float2bfloat16_rn(0.0f), lo = hi;
        if (tap < 9) {
            const size_t gi = ((size_t)tap * cop + co0 + o) * csp + ci;
            hi = wp_hi[gi];
            lo = wp_lo[gi];
        }
        sB[0][(ks * NG + o) * CS + kl] = hi;
        sB[1][(ks * NG + o) * CS + kl] = lo;
    }
    __syncthreads();
    float acc[2][NT][4];
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int j = 0; j < NT; j++)
#pragma unroll
            for (int k = 0; k < 4; k++) acc[m][j][k] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < KS; ks++) {
        // this lane's k pairs: k = 16 ks + 2t (a0/a1) and + 8 (a2/a3) -> taps and channel 0 or 2
        const int tapa = min(ks * 4 + (t >> 1), 8), tapb = min(ks * 4 + 2 + (t >> 1), 8), ci = 2 * (t & 1);
        unsigned a[2][4];
#pragma unroll
        for (int m = 0; m < 2; m++) {
            const bf16* ra = sA + ((wr + m + tapa / 3) * (TW + 2) + wx + tapa % 3) * 4 + ci;
            const bf16* rb = sA + ((wr + m + tapb / 3) * (TW + 2) + wx + tapb % 3) * 4 + ci;
            a[m][0] = ld_pair(ra + g * 4);
            a[m][1] = ld_pair(ra + (g + 8) * 4);
            a[m][2] = ld_pair(rb + g * 4);
            a[m][3] = ld_pair(rb + (g + 8) * 4);
        }
#pragma unroll
        for (int j = 0; j < NT; j++) {
            const int bo = (ks * NG + j * 8 + g) * CS + 2 * t;
            const unsigned bh0 = ld_pair(sB[0] + bo), bh1 = ld_pair(sB[0] + bo + 8);
            const unsigned bl0 = ld_pair(sB[1] + bo), bl1 = ld_pair(sB[1] + bo + 8);
#pragma unroll
            for (int m = 0; m < 2; m++) {
                mma_bf16(acc[m][j], a[m], bl0, bl1);
                mma_bf16(acc[m][j], a[m], bh0, bh1);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NT; j++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int co = co0 + j * 8 + 2 * t + h;
#pragma unroll
            for (int px = 0; px < 2; px++) {
                const int x = x0 + wx + g + 8 * px;
                const float b = co < Co ? bias[co] : 0.0f;
                float r[2];
#pragma unroll
                for (int m = 0; m < 2; m++) {
                    const bf16 rv = __float2bfloat16_rn(fmaxf(acc[m][j][2 * px + h] + b, 0.0f));
                    r[m] = __bfloat162float(rv);
                    const int y = y0 + wr + m;
                    if (co < Co && y < H && x < W) outR[(((size_t)n * Co + co) * H + y) * W + x] = rv;
                }
                const float r0n = __shfl_down_sync(0xffffffffu, r[0], 4);
                const float r1n = __shfl_down_sync(0xffffffffu, r[1], 4);
                if (!(g & 1)) {
                    const int y = y0 + wr;
                    float sum = r[0];
                    sum += r0n;
                    sum += r[1];
                    sum += r1n;
                    if (co < Co && y < H && x < W)
                        outP[(((size_t)n * Co + co) * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)] =
                            __float2bfloat16_rn(sum * 0.25f);
                }
            }
        }
    }
}

template <int NT, bool DGRAD>
constexpr size_t conv_tc_smem() {
    return ((DGRAD ? 2 : 1) * (size_t)kTcAElems + 2 * 9 * 8 * NT * kTcCS) * sizeof(bf16);
}

// Weight gradient: dW[co][ci][tap] += sum over samples and the CTA's 8 x 32 pixel tile of
// dZ[co][p] A[ci][p + tap offset] (dZ as bf16 hi / lo from k_dz).  GEMM rows = output channels (a block of 32: two M-tiles),
// columns = the 9 taps x 8 input channels of the CTA's input group (one N-tile per tap),
// K = pixels in steps of 16 (half a tile row).  Warp w takes M-tile w % 2 and tap group w / 2
// ({0,1,2}, {3,4}, {5,6}, {7,8}).  dZ is staged [channel][pixel] as bf16 hi and lo (two MMAs per
// tile); the input tile is staged twice, as is and shifted by one column, so every pixel pair
// of a B register is a 4-byte aligned load.  The samples are split over n_split CTAs per tile
// so that small layers still fill the GPU; one atomic add per weight and CTA.
constexpr int kWgPix = kTcTH * kTcTW, kWgPS = kWgPix + 8, kWgRow = kTcTW + 2, kWgPlane = 344, kWgCo = 32;
__global__ void __launch_bounds__(256) k_conv3x3_wgrad_tc(const bf16* A, const bf16* dz_hi, const bf16* dz_lo, float* dW,
                                                          int N, int Cin, int Cout, int H, int W, int ci_groups,
                                                          int n_split) {
    constexpr int TH = kTcTH, TW = kTcTW;
    __shared__ __align__(16) bf16 sZ[2][kWgCo * kWgPS];
    __shared__ __align__(16) bf16 sX[2][8 * kWgPlane];
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    // grid z: (output-channel block, input-channel group, sample range)
    const int part = blockIdx.z % n_split, zz = blockIdx.z / n_split;
    const int cob = zz / ci_groups, cig = zz % ci_groups;
    const int n_begin = (int)(((long long)N * part) / n_split), n_end = (int)(((long long)N * (part + 1)) / n_split);
    const int co_base = cob * kWgCo, ci_base = cig * 8;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int mt = warp & 1, tg = warp >> 1;
    const int tap0 = tg == 0 ? 0 : 2 * tg + 1, ntap = tg == 0 ? 3 : 2;
    const bool active = co_base + mt * 16 < Cout;
    float acc[3][4];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 4; k++) acc[i][k] = 0.0f;
    for (int n = n_begin; n < n_end; n++) {
        __syncthreads();
        if ((W & 31) == 0) {
            // whole tile rows inside the image: 16-byte copies (8 pixels) of hi and lo
            for (int e = tid; e < 2 * kWgCo * TH * (TW / 8); e += 256) {
                const int h = e / (kWgCo * TH * (TW / 8)), rem = e % (kWgCo * TH * (TW / 8));
                const int o = rem / (TH * (TW / 8)), r = (rem / (TW / 8)) % TH, c8 = rem % (TW / 8);
                const int co = co_base + o, y = y0 + r;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (co < Cout && y < H)
                    v = *reinterpret_cast<const uint4*>((h ? dz_lo : dz_hi) + (((size_t)n * Cout + co) * H + y) * W + x0 + 8 * c8);
                *reinterpret_cast<uint4*>(&sZ[h][o * kWgPS + r * TW + 8 * c8]) = v;
            }
        } else {
            for (int e = tid; e < kWgCo * kWgPix; e += 256) {
                const int o = e / kWgPix, p = e % kWgPix;
                const int y = y0 + p / TW, x = x0 + p % TW, co = co_base + o;
                bf16 hi = __float2bfloat16_rn(0.0f), lo = hi;
                if (co < Cout && y < H && x < W) {
                    const size_t ri = (((size_t)n * Cout + co) * H + y) * W + x;
                    hi = dz_hi[ri];
                    lo = dz_lo[ri];
                }
                sZ[0][o * kWgPS + p] = hi;
                sZ[1][o * kWgPS + p] = lo;
            }
        }
        for (int e = tid; e < 8 * (TH + 2) * kWgRow; e += 256) {
            const int c = e / ((TH + 2) * kWgRow), rem = e % ((TH + 2) * kWgRow);
            const int r = rem / kWgRow, q = rem % kWgRow;
            const int y = y0 + r - 1, ci = ci_base + c;
            bf16 v0 = __float2bfloat16_rn(0.0f), v1 = v0;
            if (ci < Cin && y >= 0 && y < H) {
                const size_t rb = (((size_t)n * Cin + ci) * H + y) * W;
                const int xa = x0 + q - 1, xb = x0 + q;
                if (xa >= 0 && xa < W) v0 = A[rb + xa];
                if (xb >= 0 && xb < W) v1 = A[rb + xb];
            }
            sX[0][c * kWgPlane + r * kWgRow + q] = v0;   // element q: input column x0 + q - 1
            sX[1][c * kWgPlane + r * kWgRow + q] = v1;   // element q: input column x0 + q
        }
        __syncthreads();
        if (active) {
#pragma unroll 1
            for (int ks = 0; ks < kWgPix / 16; ks++) {
                const int pr = ks >> 1, pc0 = (ks & 1) * 16;   // pixel row, first column of the step
                unsigned a[2][4];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const bf16* zr = sZ[h] + (mt * 16 + g) * kWgPS + pr * TW + pc0 + 2 * t;
                    a[h][0] = ld_pair(zr);
                    a[h][1] = ld_pair(zr + 8 * kWgPS);
                    a[h][2] = ld_pair(zr + 8);
                    a[h][3] = ld_pair(zr + 8 * kWgPS + 8);
                }
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    if (i < ntap) {
                        const int tap = tap0 + i, dy = tap / 3, dx = tap % 3;
                        // pixel pair (pc, pc + 1), pc = pc0 + 2t (+ 8): input columns pc + dx - 1, pc + dx
                        // of tile row pr + dy; dx = 1 reads the shifted copy
                        const int pc = pc0 + 2 * t;
                        const bf16* xr = (dx == 1) ? sX[1] + g * kWgPlane + (pr + dy) * kWgRow + pc
                                                   : sX[0] + g * kWgPlane + (pr + dy) * kWgRow + pc + dx;
                        const unsigned b0 = ld_pair(xr), b1 = ld_pair(xr + 8);
                        mma_bf16(acc[i], a[1], b0, b1);
                        mma_bf16(acc[i], a[0], b0, b1);
                    }
                }
            }
        }
    }
    if (!active) return;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (i >= ntap) break;
        const int tap = tap0 + i;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int co = co_base + mt * 16 + g + 8 * (k >> 1), ci = ci_base + 2 * t + (k & 1);
            if (co < Cout && ci < Cin) atomicAdd(&dW[((size_t)co * Cin + ci) * 9 + tap], acc[i][k]);
        }
    }
}

// The pre-activation gradient of a layer, once: dZ = (R > 0) dP(y/2, x/2) / 4 written as bf16 hi /
// lo at full resolution ([N][Cout][H][W], read by the weight- and data-gradient kernels), and
// db[co] += its sum over the sample (grid: Cout x N).
__global__ void k_dz(const float* dP, const bf16* R, bf16* dz_hi, bf16* dz_lo, float* db, int Cout, int H, int W) {
    __shared__ float red[8];
    const int co = blockIdx.x, n = blockIdx.y;
    const size_t plane = (((size_t)n * Cout + co) * H) * W;
    const float* dp = dP + (((size_t)n * Cout + co) * (H >> 1)) * (W >> 1);
    float s = 0.0f;
    for (int p = threadIdx.x; p < H * W; p += blockDim.x) {
        const int y = p / W, x = p % W;
        const float v = __bfloat162float(R[plane + p]) > 0.0f ? 0.25f * dp[(y >> 1) * (W >> 1) + (x >> 1)] : 0.0f;
        s += v;
        bf16 hi, lo;
        split_bf16(v, hi, lo);
        dz_hi[plane + p] = hi;
        dz_lo[plane + p] = lo;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float tsum = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) tsum += red[i];
        atomicAdd(&db[co], tsum);
    }
}

}  // namespace cnn
}  // namespace rv

using namespace rv;
using rv::cnn::bf16;

struct RvCentreNet {
    int H = 0, W = 0, B = 0, nflat = 0;
    long long nparams = 0;
    long long off_w[cnn::kLayers] = {}, off_b[cnn::kLayers] = {}, off_f0w = 0, off_f0b = 0, off_f1w = 0, off_f1b = 0;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    // per layer: weights rearranged for the tensor-core kernels (bf16 hi / lo; forward and
    // data-gradient layouts), refreshed at every forward pass
    bf16 *wf_hi[6] = {}, *wf_lo[6] = {}, *wd_hi[6] = {}, *wd_lo[6] = {};
    int csp[6] = {}, cop[6] = {}, cip[6] = {}, cop16[6] = {};
    bf16 *dz_hi = nullptr, *dz_lo = nullptr;   // one layer's dZ at a time (sized for the largest)
    bf16* R[cnn::kLayers] = {};
    bf16* P[cnn::kLayers] = {};
    float* dP[cnn::kLayers] = {};
    float *hidden = nullptr, *out = nullptr, *dout = nullptr, *dh = nullptr, *y = nullptr, *loss = nullptr;
    int step = 0;
};

namespace {

void net_free(RvCentreNet* n) {
    void* bufs[] = {n->params, n->grads, n->m, n->v, n->hidden, n->out, n->dout, n->dh, n->y, n->loss};
    for (void* b : bufs)
        if (b) cudaFree(b);
    for (int l = 0; l < cnn::kLayers; l++) {
        if (n->R[l]) cudaFree(n->R[l]);
        if (n->P[l]) cudaFree(n->P[l]);
        if (n->dP[l]) cudaFree(n->dP[l]);
        if (n->wf_hi[l]) cudaFree(n->wf_hi[l]);   // one allocation holds the four arrays
    }
    if (n->dz_hi) cudaFree(n->dz_hi);             // and one the two dZ halves
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

// Convolutions on the tensor cores (mma.sync BF16 with hi/lo-split FP32 operands) unless
// RV_CNN_SIMT=1 selects the FP32 SIMT kernels (kept for comparison).
bool use_simt() {
    static const bool simt = [] {
        const char* e = getenv("RV_CNN_SIMT");
        return e && atoi(e) != 0;
    }();
    return simt;
}

// output-channel group of the tensor-core conv kernels: 32 channels (4 N-tiles) or 64 (8)
inline int tc_group(int Co) { return Co <= 32 ? 32 : 64; }

// conv forward (fused bias, ReLU, pool) or data gradient on the tensor cores: Cs source channels,
// Co output channels, weights prepared by k_prep_weights (row length csp, cop rows per tap)
template <bool DGRAD>
cudaError_t launch_conv_tc(const void* src, const bf16* R, const bf16* whi, const bf16* wlo, int csp, int cop,
                           const float* b, bf16* outR, bf16* outP, float* outD, int Cs, int Co, int H, int W, int n,
                           cudaStream_t s) {
    const int G = tc_group(Co), groups = cdiv(Co, G);
    const dim3 grid(cdiv(W, cnn::kTcTW), cdiv(H, cnn::kTcTH), n * groups);
    if (G == 32) {
        auto k = cnn::k_conv3x3_tc<4, DGRAD>;
        constexpr size_t sm = cnn::conv_tc_smem<4, DGRAD>();
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k<<<grid, 256, sm, s>>>(src, R, whi, wlo, csp, cop, b, outR, outP, outD, Cs, Co, H, W, groups);
    } else {
        auto k = cnn::k_conv3x3_tc<8, DGRAD>;
        constexpr size_t sm = cnn::conv_tc_smem<8, DGRAD>();
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k<<<grid, 256, sm, s>>>(src, R, whi, wlo, csp, cop, b, outR, outP, outD, Cs, Co, H, W, groups);
    }
    return cudaGetLastError();
}

cudaError_t net_forward(RvCentreNet* net, const bf16* x, int n, cudaStream_t s) {
    for (int l = 0; l < cnn::kLayers; l++) {
        const int Cin = cnn::kChannels[l], Cout = cnn::kChannels[l + 1];
        const int H = net->H >> l, W = net->W >> l;
        const void* src = l == 0 ? (const void*)x : (const void*)net->P[l - 1];
        if (!use_simt()) {
            const long long tot = 9LL * net->cop[l] * net->csp[l] + 9LL * net->cip[l] * net->cop16[l];
            cnn::k_prep_weights<<<cdiv(tot, 256), 256, 0, s>>>(net->params + net->off_w[l], Cin, Cout, net->csp[l],
                                                               net->cop[l], net->cip[l], net->cop16[l], net->wf_hi[l],
                                                               net->wf_lo[l], net->wd_hi[l], net->wd_lo[l]);
            if (Cin <= 4 && tc_group(Cout) == 32) {   // the first layer: taps packed four to a K step
                const int groups = cdiv(Cout, 32);
                const dim3 grid(cdiv(W, cnn::kTcTW), cdiv(H, cnn::kTcTH), n * groups);
                cnn::k_conv3x3_tc_c4<<<grid, 256, 0, s>>>(static_cast<const bf16*>(src), net->wf_hi[l], net->wf_lo[l],
                                                          net->csp[l], net->cop[l], net->params + net->off_b[l],
                                                          net->R[l], net->P[l], Cin, Cout, H, W, groups);
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) return e;
                continue;
            }
            cudaError_t e = launch_conv_tc<false>(src, nullptr, net->wf_hi[l], net->wf_lo[l], net->csp[l], net->cop[l],
                                                  net->params + net->off_b[l], net->R[l], net->P[l], nullptr, Cin, Cout,
                                                  H, W, n, s);
            if (e != cudaSuccess) return e;
            continue;
        }
        const int groups = cdiv(Cout, cnn::kCOB);
        const dim3 grid(cdiv(W, cnn::kTileW), cdiv(H, cnn::kTileH), n * groups);
        cnn::k_conv3x3<false><<<grid, dim3(cnn::kTX, cnn::kTY), 0, s>>>(
            src, nullptr, net->params + net->off_w[l], net->params + net->off_b[l], net->R[l], net->P[l], nullptr, Cin,
            Cout, H, W, groups);
    }
    cnn::k_fc_fwd<<<cdiv((long long)n * cnn::kHidden * 32, 256), 256, 0, s>>>(
        net->P[cnn::kLayers - 1], 1, net->params + net->off_f0w, net->params + net->off_f0b, net->hidden, n, net->nflat,
        cnn::kHidden, 1);
    cnn::k_fc_fwd<<<cdiv((long long)n * 2 * 32, 256), 256, 0, s>>>(net->hidden, 0, net->params + net->off_f1w,
                                                                    net->params + net->off_f1b, net->out, n,
                                                                    cnn::kHidden, 2, 0);
    return cudaGetLastError();
}

// loss and gradients of the mean NLL over n samples (targets in net->y); forward must have run
cudaError_t net_backward(RvCentreNet* net, const bf16* x, int n, cudaStream_t s) {
    cnn::k_nll<<<1, 256, 0, s>>>(net->out, net->y, net->dout, net->loss, n);
    cudaMemsetAsync(net->grads, 0, sizeof(float) * net->nparams, s);
    float* g = net->grads;
    cnn::k_fc_wgrad<<<cdiv(2LL * cnn::kHidden, 256), 256, 0, s>>>(net->hidden, 0, net->dout, g + net->off_f1w,
                                                                  g + net->off_f1b, n, cnn::kHidden, 2);
    cnn::k_fc_dgrad<<<cdiv((long long)n * cnn::kHidden, 256), 256, 0, s>>>(net->dout, net->params + net->off_f1w,
                                                                          net->hidden, net->dh, n, cnn::kHidden, 2);
    cnn::k_fc_wgrad<<<cdiv((long long)cnn::kHidden * net->nflat, 256), 256, 0, s>>>(
        net->P[cnn::kLayers - 1], 1, net->dh, g + net->off_f0w, g + net->off_f0b, n, net->nflat, cnn::kHidden);
    cnn::k_fc_dgrad<<<cdiv((long long)n * net->nflat, 256), 256, 0, s>>>(
        net->dh, net->params + net->off_f0w, nullptr, net->dP[cnn::kLayers - 1], n, net->nflat, cnn::kHidden);
    for (int l = cnn::kLayers - 1; l >= 0; l--) {
        const int Cin = cnn::kChannels[l], Cout = cnn::kChannels[l + 1];
        const int H = net->H >> l, W = net->W >> l;
        const bf16* A = l == 0 ? x : net->P[l - 1];
        if (!use_simt()) {
            cnn::k_dz<<<dim3(Cout, n), 256, 0, s>>>(net->dP[l], net->R[l], net->dz_hi, net->dz_lo, g + net->off_b[l],
                                                    Cout, H, W);
            const int cig = cdiv(Cin, 8);
            const int base = cdiv(W, cnn::kTcTW) * cdiv(H, cnn::kTcTH) * cdiv(Cout, cnn::kWgCo) * cig;
            int split = cdiv(2048, base);   // about two waves of CTAs
            split = split < 1 ? 1 : (split > n ? n : split);
            const dim3 gw(cdiv(W, cnn::kTcTW), cdiv(H, cnn::kTcTH), cdiv(Cout, cnn::kWgCo) * cig * split);
            cnn::k_conv3x3_wgrad_tc<<<gw, 256, 0, s>>>(A, net->dz_hi, net->dz_lo, g + net->off_w[l], n, Cin, Cout, H, W,
                                                       cig, split);
            if (l > 0) {
                cudaError_t e = launch_conv_tc<true>(net->dz_hi, net->dz_lo, net->wd_hi[l], net->wd_lo[l], net->cop16[l],
                                                     net->cip[l], nullptr, nullptr, nullptr, net->dP[l - 1], Cout, Cin,
                                                     H, W, n, s);
                if (e != cudaSuccess) return e;
            }
            continue;
        }
        const int cig = cdiv(Cin, cnn::kWCI);
        const dim3 gw(cdiv(W, cnn::kWT_W), cdiv(H, cnn::kWT_H), cdiv(Cout, cnn::kWCO) * cig);
        cnn::k_conv3x3_wgrad<<<gw, 128, 0, s>>>(A, net->dP[l], net->R[l], g + net->off_w[l], g + net->off_b[l], n, Cin,
                                                Cout, H, W, cig);
        if (l > 0) {
            const int groups = cdiv(Cin, cnn::kCOB);
            const dim3 gd(cdiv(W, cnn::kTileW), cdiv(H, cnn::kTileH), n * groups);
            cnn::k_conv3x3<true><<<gd, dim3(cnn::kTX, cnn::kTY), 0, s>>>(
                net->dP[l], net->R[l], net->params + net->off_w[l], nullptr, nullptr, nullptr, net->dP[l - 1], Cout,
                Cin, H, W, groups);
        }
    }
    return cudaGetLastError();
}

}  // namespace

extern "C" int RvCentreNetCreate(int H, int W, int batch, unsigned long long seed, RvCentreNet** out) {
    if (!out || H < 64 || W < 64 || (H % 64) || (W % 64) || batch < 1 || batch > 2048) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvCentreNetCreate: H and W must be multiples of 64, batch 1..2048");
        return RV_ERR_BAD_ARGUMENT;
    }
    RvCentreNet* n = new RvCentreNet();
    n->H = H;
    n->W = W;
    n->B = batch;
    n->nflat = cnn::kChannels[cnn::kLayers] * (H >> cnn::kLayers) * (W >> cnn::kLayers);
    long long o = 0;
    for (int l = 0; l < cnn::kLayers; l++) {
        n->off_w[l] = o;
        o += (long long)cnn::kChannels[l + 1] * cnn::kChannels[l] * 9;
        n->off_b[l] = o;
        o += cnn::kChannels[l + 1];
    }
    n->off_f0w = o;
    o += (long long)cnn::kHidden * n->nflat;
    n->off_f0b = o;
    o += cnn::kHidden;
    n->off_f1w = o;
    o += 2LL * cnn::kHidden;
    n->off_f1b = o;
    o += 2;
    n->nparams = o;
    bool ok = cuda_ok(cudaMalloc(&n->params, sizeof(float) * o), RV_ERR_DEVICE_OOM, "net parameters") &&
              cuda_ok(cudaMalloc(&n->grads, sizeof(float) * o), RV_ERR_DEVICE_OOM, "net gradients") &&
              cuda_ok(cudaMalloc(&n->m, sizeof(float) * o), RV_ERR_DEVICE_OOM, "net moments") &&
              cuda_ok(cudaMalloc(&n->v, sizeof(float) * o), RV_ERR_DEVICE_OOM, "net moments");
    for (int l = 0; ok && l < cnn::kLayers; l++) {
        const long long full = (long long)batch * cnn::kChannels[l + 1] * (H >> l) * (W >> l);
        ok = cuda_ok(cudaMalloc(&n->R[l], sizeof(bf16) * full), RV_ERR_DEVICE_OOM, "net activations") &&
             cuda_ok(cudaMalloc(&n->P[l], sizeof(bf16) * (full / 4)), RV_ERR_DEVICE_OOM, "net activations") &&
             cuda_ok(cudaMalloc(&n->dP[l], sizeof(float) * (full / 4)), RV_ERR_DEVICE_OOM, "net gradients");
    }
    for (int l = 0; ok && l < cnn::kLayers; l++) {
        const int Cin = cnn::kChannels[l], Cout = cnn::kChannels[l + 1];
        n->csp[l] = (Cin + 15) / 16 * 16;
        n->cop[l] = (Cout + tc_group(Cout) - 1) / tc_group(Cout) * tc_group(Cout);
        n->cip[l] = (Cin + tc_group(Cin) - 1) / tc_group(Cin) * tc_group(Cin);
        n->cop16[l] = (Cout + 15) / 16 * 16;
        const size_t nf = 9 * (size_t)n->cop[l] * n->csp[l], nd = 9 * (size_t)n->cip[l] * n->cop16[l];
        bf16* w = nullptr;
        ok = cuda_ok(cudaMalloc(&w, sizeof(bf16) * 2 * (nf + nd)), RV_ERR_DEVICE_OOM, "net weight layouts");
        if (ok) {
            n->wf_hi[l] = w;
            n->wf_lo[l] = w + nf;
            n->wd_hi[l] = w + 2 * nf;
            n->wd_lo[l] = w + 2 * nf + nd;
        }
    }
    size_t dz_max = 0;
    for (int l = 0; l < cnn::kLayers; l++) {
        const size_t e = (size_t)batch * cnn::kChannels[l + 1] * (H >> l) * (W >> l);
        if (e > dz_max) dz_max = e;
    }
    if (ok) ok = cuda_ok(cudaMalloc(&n->dz_hi, sizeof(bf16) * 2 * dz_max), RV_ERR_DEVICE_OOM, "net dZ");
    if (ok) n->dz_lo = n->dz_hi + dz_max;
    ok = ok && cuda_ok(cudaMalloc(&n->hidden, sizeof(float) * batch * cnn::kHidden), RV_ERR_DEVICE_OOM, "net") &&
         cuda_ok(cudaMalloc(&n->dh, sizeof(float) * batch * cnn::kHidden), RV_ERR_DEVICE_OOM, "net") &&
         cuda_ok(cudaMalloc(&n->out, sizeof(float) * batch * 2), RV_ERR_DEVICE_OOM, "net") &&
         cuda_ok(cudaMalloc(&n->dout, sizeof(float) * batch * 2), RV_ERR_DEVICE_OOM, "net") &&
         cuda_ok(cudaMalloc(&n->y, sizeof(float) * batch), RV_ERR_DEVICE_OOM, "net") &&
         cuda_ok(cudaMalloc(&n->loss, sizeof(float)), RV_ERR_DEVICE_OOM, "net");
    if (!ok) {
        net_free(n);
        delete n;
        return RV_ERR_DEVICE_OOM;
    }
    // He-normal convolution and hidden weights, a small output layer, zero biases: (mu, s) ~ (0, 0)
    std::vector<float> h((size_t)o, 0.0f);
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
    auto unif = [&]() {   // splitmix64 -> (0, 1)
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return ((double)(z >> 11) + 0.5) / 9007199254740992.0;
    };
    auto normal = [&]() { return sqrt(-2.0 * log(unif())) * cos(6.283185307179586 * unif()); };
    for (int l = 0; l < cnn::kLayers; l++) {
        const double sd = sqrt(2.0 / (cnn::kChannels[l] * 9.0));
        for (long long i = 0; i < (long long)cnn::kChannels[l + 1] * cnn::kChannels[l] * 9; i++)
            h[(size_t)(n->off_w[l] + i)] = (float)(sd * normal());
    }
    for (long long i = 0; i < (long long)cnn::kHidden * n->nflat; i++)
        h[(size_t)(n->off_f0w + i)] = (float)(sqrt(2.0 / n->nflat) * normal());
    for (long long i = 0; i < 2LL * cnn::kHidden; i++)
        h[(size_t)(n->off_f1w + i)] = (float)(0.1 * sqrt(1.0 / cnn::kHidden) * normal());
    ok = cuda_ok(cudaMemcpy(n->params, h.data(), sizeof(float) * o, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "net") &&
         cuda_ok(cudaMemset(n->m, 0, sizeof(float) * o), RV_ERR_MEMSET, "net") &&
         cuda_ok(cudaMemset(n->v, 0, sizeof(float) * o), RV_ERR_MEMSET, "net");
    if (!ok) {
        net_free(n);
        delete n;
        return RV_ERR_COPY_H2D;
    }
    *out = n;
    return 0;
}

extern "C" void RvCentreNetDestroy(RvCentreNet* n) {
    if (!n) return;
    net_free(n);
    delete n;
}

extern "C" long long RvCentreNetNumParams(const RvCentreNet* n) { return n ? n->nparams : 0; }

extern "C" int RvCentreNetSetParams(RvCentreNet* n, const float* host) {
    if (!n || !host) return RV_ERR_BAD_ARGUMENT;
    n->step = 0;
    if (!cuda_ok(cudaMemcpy(n->params, host, sizeof(float) * n->nparams, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D,
                 "net parameters") ||
        !cuda_ok(cudaMemset(n->m, 0, sizeof(float) * n->nparams), RV_ERR_MEMSET, "net") ||
        !cuda_ok(cudaMemset(n->v, 0, sizeof(float) * n->nparams), RV_ERR_MEMSET, "net"))
        return RV_ERR_COPY_H2D;
    return 0;
}

extern "C" int RvCentreNetGetParams(const RvCentreNet* n, float* host) {
    if (!n || !host) return RV_ERR_BAD_ARGUMENT;
    return cuda_ok(cudaMemcpy(host, n->params, sizeof(float) * n->nparams, cudaMemcpyDeviceToHost), RV_ERR_COPY_D2H,
                   "net parameters") ? 0 : RV_ERR_COPY_D2H;
}

static int check_batch(const RvCentreNet* n, const void* x, int count) {
    if (!n || !x || count < 1 || count > n->B) {
        set_error(RV_ERR_BAD_ARGUMENT, "centre net: null input or batch outside 1..capacity");
        return RV_ERR_BAD_ARGUMENT;
    }
    return 0;
}

extern "C" int RvCentreNetForward(RvCentreNet* n, const void* d_x, int count, float* mu, float* s, void* stream) {
    int rc = check_batch(n, d_x, count);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (!cuda_ok(net_forward(n, static_cast<const bf16*>(d_x), count, st), RV_ERR_LAUNCH, "net forward"))
        return RV_ERR_LAUNCH;
    std::vector<float> o((size_t)count * 2);
    if (!cuda_ok(cudaMemcpyAsync(o.data(), n->out, sizeof(float) * 2 * count, cudaMemcpyDeviceToHost, st),
                 RV_ERR_COPY_D2H, "net output") ||
        !cuda_ok(cudaStreamSynchronize(st), RV_ERR_LAUNCH, "net forward"))
        return RV_ERR_LAUNCH;
    for (int i = 0; i < count; i++) {
        if (mu) mu[i] = o[2 * (size_t)i];
        if (s) s[i] = o[2 * (size_t)i + 1];
    }
    return 0;
}

// Loss and parameter gradients of one batch (no update); y on the host, grads_host may be NULL.
extern "C" int RvCentreNetGradients(RvCentreNet* n, const void* d_x, const float* y, int count, float* loss,
                                    float* grads_host, void* stream) {
    int rc = check_batch(n, d_x, count);
    if (rc) return rc;
    if (!y) return RV_ERR_BAD_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const bf16* x = static_cast<const bf16*>(d_x);
    if (!cuda_ok(cudaMemcpyAsync(n->y, y, sizeof(float) * count, cudaMemcpyHostToDevice, st), RV_ERR_COPY_H2D,
                 "targets") ||
        !cuda_ok(net_forward(n, x, count, st), RV_ERR_LAUNCH, "net forward") ||
        !cuda_ok(net_backward(n, x, count, st), RV_ERR_LAUNCH, "net backward"))
        return RV_ERR_LAUNCH;
    float l = 0.0f;
    if (!cuda_ok(cudaMemcpyAsync(&l, n->loss, sizeof(float), cudaMemcpyDeviceToHost, st), RV_ERR_COPY_D2H, "loss"))
        return RV_ERR_COPY_D2H;
    if (grads_host && !cuda_ok(cudaMemcpyAsync(grads_host, n->grads, sizeof(float) * n->nparams,
                                               cudaMemcpyDeviceToHost, st), RV_ERR_COPY_D2H, "gradients"))
        return RV_ERR_COPY_D2H;
    if (!cuda_ok(cudaStreamSynchronize(st), RV_ERR_LAUNCH, "net backward")) return RV_ERR_LAUNCH;
    if (loss) *loss = l;
    return 0;
}

// One Adam step (beta 0.9 / 0.999, eps 1e-8) on a batch whose targets are already on the device.
extern "C" int RvCentreNetTrainStep(RvCentreNet* n, const void* d_x, const float* d_y, int count, float lr,
                                    float* loss, void* stream) {
    int rc = check_batch(n, d_x, count);
    if (rc) return rc;
    if (!d_y) return RV_ERR_BAD_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const bf16* x = static_cast<const bf16*>(d_x);
    if (!cuda_ok(cudaMemcpyAsync(n->y, d_y, sizeof(float) * count, cudaMemcpyDeviceToDevice, st), RV_ERR_COPY_H2D,
                 "targets") ||
        !cuda_ok(net_forward(n, x, count, st), RV_ERR_LAUNCH, "net forward") ||
        !cuda_ok(net_backward(n, x, count, st), RV_ERR_LAUNCH, "net backward"))
        return RV_ERR_LAUNCH;
    n->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - powf(b1, (float)n->step), bc2 = 1.0f - powf(b2, (float)n->step);
    cnn::k_adam<<<cdiv(n->nparams, 256), 256, 0, st>>>(n->params, n->grads, n->m, n->v, n->nparams, lr, b1, b2, 1e-8f,
                                                      bc1, bc2);
    if (!cuda_ok(cudaGetLastError(), RV_ERR_LAUNCH, "adam")) return RV_ERR_LAUNCH;
    if (loss) {
        if (!cuda_ok(cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, st), RV_ERR_COPY_D2H, "loss") ||
            !cuda_ok(cudaStreamSynchronize(st), RV_ERR_LAUNCH, "train step"))
            return RV_ERR_LAUNCH;
    }
    return 0;
}
