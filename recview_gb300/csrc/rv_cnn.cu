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

}  // namespace cnn
}  // namespace rv

using namespace rv;
using rv::cnn::bf16;

struct RvCentreNet {
    int H = 0, W = 0, B = 0, nflat = 0;
    long long nparams = 0;
    long long off_w[cnn::kLayers] = {}, off_b[cnn::kLayers] = {}, off_f0w = 0, off_f0b = 0, off_f1w = 0, off_f1b = 0;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
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
    }
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

cudaError_t net_forward(RvCentreNet* net, const bf16* x, int n, cudaStream_t s) {
    for (int l = 0; l < cnn::kLayers; l++) {
        const int Cin = cnn::kChannels[l], Cout = cnn::kChannels[l + 1];
        const int H = net->H >> l, W = net->W >> l;
        const int groups = cdiv(Cout, cnn::kCOB);
        const dim3 grid(cdiv(W, cnn::kTileW), cdiv(H, cnn::kTileH), n * groups);
        cnn::k_conv3x3<false><<<grid, dim3(cnn::kTX, cnn::kTY), 0, s>>>(
            l == 0 ? (const void*)x : (const void*)net->P[l - 1], nullptr, net->params + net->off_w[l],
            net->params + net->off_b[l], net->R[l], net->P[l], nullptr, Cin, Cout, H, W, groups);
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
