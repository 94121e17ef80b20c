// Device kernels of the convolution back-projection path (sm_103a).
//
//  k_normalise  R1      flat/dark log normalisation -> int16 rows (CudaSinogramHost)
//  k_filter     R1+R5+R6+R7  one CTA per sinogram row: [normalise] -> pad/zoom -> forward
//                       radix-2 FFT -> filter -> inverse FFT -> 1/16 sub-sample int table
//                       (REF) or FP32/FP16/BF16 (value, slope) pair row (LIN modes)
//  (the back-projection kernels, REF and LIN, are in rv_bp_ref.cu)
//
// Floating-point discipline: every operation that the reference performs in float is done with
// an explicitly rounded intrinsic (__fmul_rn/__fadd_rn/__fsub_rn) so nvcc never contracts it into
// an FMA; the REF outputs are therefore bit-identical to the reference CPU routine.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include <atomic>
#include <vector>

#include "rv_internal.h"

namespace rv {

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// x * w evaluated as (xr*wr - xi*wi, xr*wi + xi*wr): source/cfft.cpp:234-235
__device__ __forceinline__ float2 cmul(float2 x, float2 w) {
    return make_float2(fsub(fmul(x.x, w.x), fmul(x.y, w.y)), fadd(fmul(x.x, w.y), fmul(x.y, w.x)));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(fadd(a.x, b.x), fadd(a.y, b.y)); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(fsub(a.x, b.x), fsub(a.y, b.y)); }

// ---------------------------------------------------------------------------------------------
// R1: one normalised sample (source/general.cpp:2466-2503).  The incident intensity is a float
// expression in the reference (int*float, ushort+float, float-ushort); only the log ratio is in
// double: v = (short)(int)(3000 log(I0 / S) + 0.5).
// Fast path in FP32: L = logf(fl(I0 / S)), and 3000 L + 0.5 held exactly as p + 0.5 + e
// (p = fl(3000 L), e = fma(3000, L, -p) its exact rounding error; p + 0.5 is exact).  Its
// distance from the true value is 3000 |L - ln(I0/S)| <= 3000 (ulp terms of logf + 2^-24 of the
// correctly rounded quotient); the band below allows 4 ulp(L) for logf's documented 1 ulp and
// 2^-12 for the remaining roundings, so every sample outside it is decided on the right side of
// its integer.  Samples inside the band (under 1% for |L| < 4) are recomputed in FP64 exactly as
// the reference does.  FP64 is slow on this GPU and a divergent FP64 branch costs its whole warp,
// so the row kernels take the fast path for every sample first (norm_fast flags what it cannot
// decide) and run the FP64 recheck (norm_exact) afterwards over a compacted list, 32 flagged
// samples per warp.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float norm_incident(int f0, int f1, int dark, float t0) {
    const float prod = fmul((float)(f1 - f0), t0);
    const float s1 = fadd((float)f0, prod);
    return fsub(s1, (float)dark);
}
// the sample, or (when *recheck is set) a placeholder to be replaced by norm_exact
__device__ __forceinline__ short norm_fast(int raw, int f0, int f1, int dark, float t0, int pixmin, bool* recheck) {
    *recheck = false;
    const float dinc = norm_incident(f0, f1, dark, t0);
    if (!(dinc > 0.0f)) return 0;
    const int s = raw - dark;
    if (s < pixmin) return 0;
    const float L = logf(__fdiv_rn(dinc, (float)s));
    const float p = __fmul_rn(L, 3000.0f);
    const float e = __fmaf_rn(L, 3000.0f, -p);           // 3000 L = p + e exactly
    const float wh = __fadd_rn(p, 0.5f);                  // exact: |p| < 2^22
    const float N = rintf(wh);
    const float t = __fadd_rn(__fsub_rn(wh, N), e);       // (3000 L + 0.5) - N, |t| <= 0.51
    const float ulpL = __fmul_rn(__int_as_float(__float_as_int(L) & 0x7f800000), 1.1920929e-7f);   // 2^-23 2^E
    const float band = __fadd_rn(__fmul_rn(ulpL, 12000.0f), 4.3e-4f);   // 3000 (4 ulp + 2^-24) + 2^-12
    if (fabsf(t) > band) {
        // truncation toward zero of N + t
        const int n = __float2int_rn(N);
        return (short)(n > 0 ? (t > 0.0f ? n : n - 1) : (n < 0 ? (t < 0.0f ? n : n + 1) : 0));
    }
    *recheck = true;
    return 0;
}
// Boundaries of the flagged samples: w = 3000 ln(I0 / S) + 0.5 crosses the integer n exactly
// where I0 = S exp((n - 0.5) / 3000).  g_exp_bound[n - kExpMin] holds that exponential as an
// unevaluated float pair (hi + lo, about 2^-48 relative), filled once per device from the host's
// double exp; g_exp_ready says it is filled (the recheck takes FP64 until then).
constexpr int kExpMin = -30000, kExpMax = 34000, kExpReady = 0x45787042;
__device__ float2 g_exp_bound[kExpMax - kExpMin + 1];
__device__ int g_exp_ready;

// a sample that norm_fast flagged (so dinc > 0 and s >= pixmin): the reference's value.
// Its w lies within norm_fast's band of n = rint(fl(3000 L) + 0.5), so it truncates to n or to
// the neighbour towards zero, decided by the sign of D = I0 - S exp((n - 0.5)/3000): S hi is
// split exactly by one FMA, I0 - S hi is exact (the two agree to 1e-4), and the rest of D is off
// by at most ~2e-12 I0.  |D| > 1e-9 I0 (3e-6 in w, far beyond the reference's own double
// rounding) decides; closer samples, and n outside the table, take the FP64 formula.
__device__ __forceinline__ short norm_exact(int raw, int f0, int f1, int dark, float t0) {
    const float dinc = norm_incident(f0, f1, dark, t0);
    const int s = raw - dark;
    if (*(volatile int*)&g_exp_ready == kExpReady) {
        const float L = logf(__fdiv_rn(dinc, (float)s));
        const int n = __float2int_rn(rintf(__fadd_rn(__fmul_rn(L, 3000.0f), 0.5f)));
        if (n == 0) return 0;
        if (n >= kExpMin && n <= kExpMax) {
            const float2 E = g_exp_bound[n - kExpMin];
            const float sf = (float)s;
            const float ph = __fmul_rn(sf, E.x);
            const float pl = __fmaf_rn(sf, E.x, -ph);   // S hi = ph + pl exactly
            const float D = __fsub_rn(__fsub_rn(__fsub_rn(dinc, ph), pl), __fmul_rn(sf, E.y));
            if (fabsf(D) > __fmul_rn(dinc, 1e-9f))     // w > n  <=>  D > 0
                return (short)(n > 0 ? (D > 0.0f ? n : n - 1) : (D > 0.0f ? n + 1 : n));
        }
    }
    const double vd = __dadd_rn(__dmul_rn(log(__ddiv_rn((double)dinc, (double)s)), 3000.0), 0.5);
    return (short)__double2int_rz(vd);
}
// the Zernike-phase form (always FP64 in the reference)
__device__ __forceinline__ short norm_zernike(int raw, int f0, int f1, int dark, float t0, int pixmin) {
    const float dinc = norm_incident(f0, f1, dark, t0);
    if (!(dinc > 0.0f)) return 0;
    const int s = raw - dark;
    if (s < pixmin) return 0;
    const double v = __dadd_rn(__ddiv_rn(__dmul_rn((double)dinc, 1000.0), (double)s), 0.5);
    return (short)__double2int_rz(v);
}

// Normalises row `job` into out[0..W) (out[x] = sample x - sh, zero outside) with the deferred
// FP64 recheck; relist (>= W ints of shared memory) and *count (a shared counter, zero on entry)
// hold the flagged positions.  Ends with a block barrier.
__device__ __forceinline__ void normalise_row(const uint16_t* r, const uint16_t* f0, const uint16_t* f1,
                                              const uint16_t* dk, int W, int sh, bool zero, float t0, int pixmin,
                                              int zernike, short* out, int* relist, int* count) {
    const int tid = threadIdx.x, NT = blockDim.x;
    const bool vec = sh == 0 && !zernike && (W & 3) == 0 &&
                     ((reinterpret_cast<uintptr_t>(r) | reinterpret_cast<uintptr_t>(f0) | reinterpret_cast<uintptr_t>(f1) |
                       reinterpret_cast<uintptr_t>(dk) | reinterpret_cast<uintptr_t>(out)) & 7) == 0;
    if (vec) {
        // four samples per thread and step, all four rows loaded before any arithmetic.  Plain
        // (generic) loads: the rows may be shared memory (an in-place row's copy) or the caller's
        // host memory, where the read-only global path does not apply.
        for (int x4 = tid; x4 < (W >> 2); x4 += NT) {
            const uint2 vr = reinterpret_cast<const uint2*>(r)[x4];
            const uint2 v0 = reinterpret_cast<const uint2*>(f0)[x4];
            const uint2 v1 = reinterpret_cast<const uint2*>(f1)[x4];
            const uint2 vd = reinterpret_cast<const uint2*>(dk)[x4];
            short o[4] = {0, 0, 0, 0};
            if (!zero) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int sft = 16 * (k & 1);
                    const unsigned wr = k < 2 ? vr.x : vr.y, w0 = k < 2 ? v0.x : v0.y;
                    const unsigned w1 = k < 2 ? v1.x : v1.y, wd = k < 2 ? vd.x : vd.y;
                    bool re;
                    o[k] = norm_fast((int)((wr >> sft) & 0xffffu), (int)((w0 >> sft) & 0xffffu),
                                     (int)((w1 >> sft) & 0xffffu), (int)((wd >> sft) & 0xffffu), t0, pixmin, &re);
                    if (re) relist[atomicAdd(count, 1)] = 4 * x4 + k;
                }
            }
            reinterpret_cast<uint2*>(out)[x4] =
                make_uint2((unsigned)(unsigned short)o[0] | ((unsigned)(unsigned short)o[1] << 16),
                           (unsigned)(unsigned short)o[2] | ((unsigned)(unsigned short)o[3] << 16));
        }
    }
    for (int x = vec ? W : tid; x < W; x += NT) {
        short v = 0;
        const int j = x - sh;  // drift shift (source/general.cpp:2505-2517)
        if (!zero && j >= 0 && j < W) {
            if (zernike) {
                v = norm_zernike(r[j], f0[j], f1[j], dk[j], t0, pixmin);
            } else {
                bool re;
                v = norm_fast(r[j], f0[j], f1[j], dk[j], t0, pixmin, &re);
                if (re) relist[atomicAdd(count, 1)] = x;
            }
        }
        out[x] = v;
    }
    __syncthreads();
    const int n = *count;
    for (int i = tid; i < n; i += NT) {
        const int x = relist[i], j = x - sh;
        out[x] = norm_exact(r[j], f0[j], f1[j], dk[j], t0);
    }
    __syncthreads();
}

// R2 strip assembly (source/gazoDoc.cpp:3318-3342): the integer mean, truncated, of the bin x bin
// block of a raw strip that makes sample x of a binned row (row points at the block's first
// detector row, already shifted by the trim).
__device__ __forceinline__ int binned_sample(const uint16_t* row, long long stride, int bin, int x) {
    const uint16_t* q = row + (long long)x * bin;
    int sum = 0;
    for (int iy = 0; iy < bin; iy++)
        for (int ix = 0; ix < bin; ix++) sum += q[iy * stride + ix];
    return sum / (bin * bin);
}

// normalise_row for raw frames that are binned on the fly: each of the four rows is a strip of
// bin detector rows, `stride` samples apart; samples come from binned_sample.  Same decision rule
// and deferred recheck as normalise_row (no drift shift, no Zernike form on this path).
__device__ __forceinline__ void normalise_row_binned(const uint16_t* r, const uint16_t* f0, const uint16_t* f1,
                                                     const uint16_t* dk, long long stride, int bin, int W, bool zero,
                                                     float t0, int pixmin, short* out, int* relist, int* count) {
    const int tid = threadIdx.x, NT = blockDim.x;
    for (int x = tid; x < W; x += NT) {
        short v = 0;
        if (!zero) {
            bool re;
            v = norm_fast(binned_sample(r, stride, bin, x), binned_sample(f0, stride, bin, x),
                          binned_sample(f1, stride, bin, x), binned_sample(dk, stride, bin, x), t0, pixmin, &re);
            if (re) relist[atomicAdd(count, 1)] = x;
        }
        out[x] = v;
    }
    __syncthreads();
    const int n = *count;
    for (int i = tid; i < n; i += NT) {
        const int x = relist[i];
        out[x] = norm_exact(binned_sample(r, stride, bin, x), binned_sample(f0, stride, bin, x),
                            binned_sample(f1, stride, bin, x), binned_sample(dk, stride, bin, x), t0);
    }
    __syncthreads();
}

__global__ void k_normalise(NormLaunch p) {
    extern __shared__ int sm_norm[];   // [0]: recheck count, [1 .. W]: flagged positions, then
                                       // (row-pointer mode) a copy of the sample row
    const RowJob job = p.jobs[blockIdx.x];
    const int W = p.ixdim;
    const uint16_t *r, *f0, *f1, *dk;
    short* out;
    if (p.row_ptr) {
        // the result replaces the sample row in place: read that row into shared memory first
        // (a drift shift reads other positions of it)
        uint16_t* rowcopy = reinterpret_cast<uint16_t*>(sm_norm + ((W + 4) & ~3));   // 16-byte aligned
        const uint16_t* src = p.row_ptr[job.src_row];
        for (int x = threadIdx.x; x < W; x += blockDim.x) rowcopy[x] = src[x];
        r = rowcopy;
        f0 = p.row_ptr[job.flat0_row];
        f1 = p.row_ptr[job.flat1_row];
        dk = p.row_ptr[job.dark_row];
        out = reinterpret_cast<short*>(const_cast<uint16_t*>(p.row_ptr[job.dst]));
    } else {
        r = p.raw + (size_t)job.src_row * W;
        f0 = p.raw + (size_t)job.flat0_row * W;
        f1 = p.raw + (size_t)job.flat1_row * W;
        dk = p.raw + (size_t)job.dark_row * W;
        out = p.out + (size_t)job.dst * W;
    }
    const int sh = p.shift ? p.shift[blockIdx.x] : 0;
    if (threadIdx.x == 0) sm_norm[0] = 0;
    __syncthreads();
    normalise_row(r, f0, f1, dk, W, sh, job.zero != 0, job.t0, p.pixmin, p.zernike, out, sm_norm + 1, sm_norm);
}

// fills g_exp_bound once per device with two synchronous copies (512 KB), outside stream capture
// (a launch inside a capture leaves it for a later call; until then the recheck uses FP64, with
// the same results).  A caller that captures in cudaStreamCaptureModeGlobal on another thread
// should make one normalising call first.
static void ensure_exp_bound(cudaStream_t s) {
    // per device: the context the table was filled in (a device reset makes a new context whose
    // copy of the table is empty again, so it is filled anew there)
    static std::atomic<unsigned long long> done[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    const unsigned long long ctx = current_context_id();
    if (ctx != 0 && done[dev].load() == ctx) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    std::vector<float2> t(kExpMax - kExpMin + 1);
    for (int n = kExpMin; n <= kExpMax; n++) {
        const double e = exp((n - 0.5) / 3000.0);
        const float hi = (float)e;
        t[n - kExpMin] = make_float2(hi, (float)(e - (double)hi));
    }
    const int ready = kExpReady;
    if (cudaMemcpyToSymbol(g_exp_bound, t.data(), t.size() * sizeof(float2)) == cudaSuccess &&
        cudaMemcpyToSymbol(g_exp_ready, &ready, sizeof(int)) == cudaSuccess)
        done[dev].store(current_context_id());
}

cudaError_t launch_normalise(const NormLaunch& p, cudaStream_t s) {
    ensure_exp_bound(s);
    if (p.njobs <= 0) return cudaSuccess;
    const size_t smem = p.row_ptr ? (((size_t)p.ixdim + 4) & ~(size_t)3) * sizeof(int) + (((size_t)p.ixdim * 2 + 15) & ~(size_t)15)
                                  : ((size_t)p.ixdim + 1) * sizeof(int);
    cudaError_t e = cudaFuncSetAttribute(k_normalise, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_normalise<<<p.njobs, 256, smem, s>>>(p);  // one CTA per row
    return cudaGetLastError();
}


// Shared-memory position of transform element a: bits 1-3 of a are flipped by bits 4-6, so the
// strided stores of the early fused passes (a warp writing elements 2^(l+3) apart) and 16-byte
// stores of adjacent pairs spread over all banks, while runs of 16 consecutive elements (every
// load) stay conflict-free.  Elements 2i and 2i+1 stay adjacent.
__device__ __forceinline__ int fsw(int a) { return a ^ ((a >> 3) & 14); }
// stores elements 2i and 2i+1 as one 16-byte word
__device__ __forceinline__ void st_pair(float2* buf, int i, float2 lo, float2 hi) {
    reinterpret_cast<float4*>(buf)[fsw(2 * i) >> 1] = make_float4(lo.x, lo.y, hi.x, hi.y);
}

// The general radix-2 Stockham passes l = 1 .. np-2 (source/cfft.cpp:210-245, 310-345): pass l
// reads x[j], x[j + n/2] for butterfly j = m 2^l + q and writes y[2m 2^l + q] = x[j] + w b,
// y[(2m+1) 2^l + q] = x[j] - w b (b = x[j + n/2], w = pass l's twiddle q).
// Three consecutive general passes l, l+1, l+2 (l + 2 <= np - 2) close over groups of eight: the inputs
// x[g + k n/8] (g < n/8, k = 0..7) of pass l feed butterflies c, c + 2^l, c + n/4, c + n/4 + 2^l
// of pass l+1 (c = 2g - q), whose outputs are the inputs of butterflies B + t 2^l (t = 0..3,
// B = 4m 2^l + q) of pass l+2, which write o + t 2^l and o + 4 2^l + t 2^l (o = 8m 2^l + q).
// One thread runs all three passes of a group in registers -- the same operations in the same
// order -- so two of every three shared-memory round trips and barriers go.  Two passes left
// over run as a pair over groups of four (c and c + n/4 only), one alone.
template <int BPT>
__device__ __forceinline__ void fft_general_passes(float2* buf, const float2* __restrict__ tw, int np, int half,
                                                   int tid, int NT) {
    int l = 1;
    if (BPT >= 4) {   // rows of n >= 8 x threads; smaller rows keep every thread busy with pairs
        constexpr int G = BPT >= 4 ? BPT / 4 : 1;   // groups of eight per thread
        const int eighth = half >> 2;
        for (; l + 2 < np - 1; l += 3) {
            const int al = 1 << l, mask = al - 1;
            float2 t0[G], t1[G], t2[G], t3[G], t4[G], t5[G], t6[G], t7[G];
#pragma unroll
            for (int i = 0; i < G; i++) {
                const int g = tid + i * NT;
                const int q = g & mask;
                const float2 w1 = __ldg(tw + al + q);                                  // pass l
                const float2 w2a = __ldg(tw + 2 * al + q), w2b = __ldg(tw + 3 * al + q);   // pass l+1
                float2 P[4], M[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float2 x = buf[fsw(g + k * eighth)], xb = cmul(buf[fsw(g + k * eighth + half)], w1);
                    P[k] = cadd(x, xb);
                    M[k] = csub(x, xb);
                }
                const float2 b0 = cmul(P[2], w2a), b1 = cmul(M[2], w2b);
                const float2 b2 = cmul(P[3], w2a), b3 = cmul(M[3], w2b);
                const float2 R0 = cadd(P[0], b0), S0 = csub(P[0], b0);
                const float2 R1 = cadd(M[0], b1), S1 = csub(M[0], b1);
                const float2 R2 = cadd(P[1], b2), S2 = csub(P[1], b2);
                const float2 R3 = cadd(M[1], b3), S3 = csub(M[1], b3);
                // pass l+2: butterfly B + t al reads (R0, R2), (R1, R3), (S0, S2), (S1, S3)
                const float2 c0 = cmul(R2, __ldg(tw + 4 * al + q));
                const float2 c1 = cmul(R3, __ldg(tw + 5 * al + q));
                const float2 c2 = cmul(S2, __ldg(tw + 6 * al + q));
                const float2 c3 = cmul(S3, __ldg(tw + 7 * al + q));
                t0[i] = cadd(R0, c0);
                t4[i] = csub(R0, c0);
                t1[i] = cadd(R1, c1);
                t5[i] = csub(R1, c1);
                t2[i] = cadd(S0, c2);
                t6[i] = csub(S0, c2);
                t3[i] = cadd(S1, c3);
                t7[i] = csub(S1, c3);
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < G; i++) {
                const int g = tid + i * NT;
                const int o = 8 * (g >> l) * al + (g & mask);
                buf[fsw(o)] = t0[i];
                buf[fsw(o + al)] = t1[i];
                buf[fsw(o + 2 * al)] = t2[i];
                buf[fsw(o + 3 * al)] = t3[i];
                buf[fsw(o + 4 * al)] = t4[i];
                buf[fsw(o + 5 * al)] = t5[i];
                buf[fsw(o + 6 * al)] = t6[i];
                buf[fsw(o + 7 * al)] = t7[i];
            }
            __syncthreads();
        }
    }
    if (BPT >= 2) {   // pairs of passes over groups of four
        constexpr int G = BPT >= 2 ? BPT / 2 : 1;   // groups of four per thread
        const int quarter = half >> 1;
        // after the triples at most one pair is left (BPT >= 4); smaller rows take all pairs here
        for (int it = 0; l + 1 < np - 1 && (BPT < 4 || it == 0); l += 2, it++) {
            const int al = 1 << l, mask = al - 1;
            float2 u0[G], u1[G], v0[G], v1[G];
#pragma unroll
            for (int i = 0; i < G; i++) {
                const int g = tid + i * NT;
                const int q = g & mask;
                const float2 w = __ldg(tw + al + q);                  // pass l
                const float2 x0 = buf[fsw(g)], x1 = cmul(buf[fsw(g + half)], w);
                const float2 x2 = buf[fsw(g + quarter)], x3 = cmul(buf[fsw(g + quarter + half)], w);
                u0[i] = cadd(x0, x1);
                u1[i] = csub(x0, x1);
                v0[i] = cmul(cadd(x2, x3), __ldg(tw + 2 * al + q));        // pass l+1, butterfly 2m 2^l + q
                v1[i] = cmul(csub(x2, x3), __ldg(tw + 2 * al + al + q));   // ... 2m 2^l + 2^l + q
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < G; i++) {
                const int g = tid + i * NT;
                const int o = 4 * (g >> l) * al + (g & mask);   // y'[2m 2^(l+1) + q]
                buf[fsw(o)] = cadd(u0[i], v0[i]);
                buf[fsw(o + 2 * al)] = csub(u0[i], v0[i]);
                buf[fsw(o + al)] = cadd(u1[i], v1[i]);
                buf[fsw(o + 3 * al)] = csub(u1[i], v1[i]);
            }
            __syncthreads();
        }
    }
    for (; l < np - 1; l++) {
        const int al = 1 << l, mask = al - 1;
        float2 a[BPT], b[BPT];
#pragma unroll
        for (int i = 0; i < BPT; i++) {
            const int j = tid + i * NT;
            a[i] = buf[fsw(j)];
            b[i] = cmul(buf[fsw(j + half)], __ldg(tw + al + (j & mask)));
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < BPT; i++) {
            const int j = tid + i * NT;
            const int o = 2 * j - (j & mask);
            buf[fsw(o)] = cadd(a[i], b[i]);
            buf[fsw(o + al)] = csub(a[i], b[i]);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------------
// R5+R6+R7: filter one row per CTA.  Shared memory: buf[n] complex (in-place radix-2 passes with
// a register hand-off between read and write phases) and strip[ixdim] shorts; the twiddles come
// from a per-pass table in global memory (pass l reads tw[2^l + q], consecutive per warp, so the
// reads neither conflict nor leave L1).
// The pass structure is the reference's Stockham FFT (source/cfft.cpp:193-369): pass l reads
// x[j] and x[j + n/2] for butterfly j and writes y[2j - q], y[2j - q + al], q = j mod al.
// ---------------------------------------------------------------------------------------------
template <int BPT>
__global__ void __launch_bounds__(512, (BPT <= 4 ? 3 : (BPT == 8 ? 2 : 1))) k_filter(FilterLaunch p) {
    extern __shared__ __align__(16) float2 sm[];
    const int n = p.d.ndim, half = n >> 1, np = p.d.ndimp;
    float2* buf = sm;
    const float2* __restrict__ tw = p.tw;   // per-pass table: pass l reads tw[2^l + q]
    short* strip = reinterpret_cast<short*>(sm + n);
    const int tid = threadIdx.x, NT = blockDim.x;
    const RowJob job = p.jobs[blockIdx.x];
    const int W = p.d.ixdim;

    // ---- sinogram row (R1 on the fly for raw frames) -------------------------------------------
    if (p.raw) {
        // the FFT buffer is free until the placement: it holds the recheck list meanwhile
        __shared__ int s_nre;
        if (tid == 0) s_nre = 0;
        __syncthreads();
        const uint16_t* base = static_cast<const uint16_t*>(p.src) + p.raw_x0;
        const long long rs = p.raw_stride > 0 ? p.raw_stride : W;
        if (p.bin > 1) {
            const long long lr = rs * p.bin;   // samples per logical (binned) row
            normalise_row_binned(base + job.src_row * lr, base + job.flat0_row * lr, base + job.flat1_row * lr,
                                 base + job.dark_row * lr, rs, p.bin, W, job.zero != 0, job.t0, p.pixmin, strip,
                                 reinterpret_cast<int*>(buf), &s_nre);
        } else {
            normalise_row(base + (size_t)job.src_row * rs, base + (size_t)job.flat0_row * rs,
                          base + (size_t)job.flat1_row * rs, base + (size_t)job.dark_row * rs, W, 0, job.zero != 0,
                          job.t0, p.pixmin, 0, strip, reinterpret_cast<int*>(buf), &s_nre);
        }
    } else {
        const short* r = p.row_ptr ? p.row_ptr[job.src_row] : static_cast<const short*>(p.src) + (size_t)job.src_row * W;
        for (int x = tid; x < W; x += NT) strip[x] = job.zero ? (short)0 : r[x];
        __syncthreads();
    }
    // ---- R5: placement with edge padding and integer zoom (source/general.cpp:2105-2126), taken
    // straight into the first forward pass (CFft::FFT1Rev, source/cfft.cpp:193-209): butterfly j
    // combines placed samples half-1-j and n-1-j, whose imaginary parts are zero, so the placed
    // row never goes through shared memory.
    const int z = p.d.iIntpDim;
    const int ic = p.ic_per_job ? job.ic : p.ic;
    const int idx0 = (0 - ic) * z + (half - 1);
    const int idx1 = (W - 1 - ic) * z + (half - 1) + 1;
    // z = 2^iZooming: C's truncating division by z as shifts (a negative numerator is biased
    // by z - 1 first)
    const int lz = __ffs(z) - 1;
    auto divz = [&](int x) { return (x + ((x >> 31) & (z - 1))) >> lz; };
    auto placed = [&](int m) -> float {
        if (m < idx0) return strip[0];
        if (m >= idx1) return strip[W - 1];
        const int k = (m - idx0) >> lz, j = (m - idx0) & (z - 1);
        if (j == 0) return strip[k];
        return (float)(divz((int)strip[k] * (z - j)) + divz((int)strip[k + 1] * j));
    };

    float2 a[BPT], b[BPT];
    // ---- forward transform (CFft::FFT1Rev) ----------------------------------------------------
#pragma unroll
    for (int i = 0; i < BPT; i++) {
        const int j = tid + i * NT;
        const float pa = placed(half - 1 - j), pb = placed(n - 1 - j);
        st_pair(buf, j, make_float2(fadd(pa, pb), 0.0f),     // imaginary parts 0 + 0
                make_float2(fsub(pa, pb), 0.0f));            // and 0 - 0
    }
    __syncthreads();
    fft_general_passes<BPT>(buf, tw, np, half, tid, NT);
    // last forward pass writes reversed (source/cfft.cpp:246-265); the filter multiply
    // (source/general.cpp:2128, CCmplx::operator*=(float)) is applied on the way out, and the
    // first inverse pass (CFft::FFT1, source/cfft.cpp:279-296) follows in registers: butterfly j
    // of the last forward pass writes positions n-j and half-j (0 and half for j = 0), which are
    // exactly the two inputs of the first inverse butterfly half-j (0).
#pragma unroll
    for (int i = 0; i < BPT; i++) {
        const int j = tid + i * NT;
        a[i] = buf[fsw(j)];
        b[i] = (j == 0) ? buf[fsw(j + half)] : cmul(buf[fsw(j + half)], __ldg(tw + half + j));
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < BPT; i++) {
        const int j = tid + i * NT;
        const int op = (j == 0) ? 0 : n - j;
        const int om = (j == 0) ? half : half - j;
        const float2 vp = cadd(a[i], b[i]), vm = csub(a[i], b[i]);
        const float fp = __ldg(p.filt + op), fm = __ldg(p.filt + om);
        const float2 yp = make_float2(fmul(vp.x, fp), fmul(vp.y, fp));   // spectrum at op
        const float2 ym = make_float2(fmul(vm.x, fm), fmul(vm.y, fm));   // spectrum at om
        // inverse butterfly k reads x[k] and x[k + half]: k = om (x[k] = ym, x[k + half] = yp), or
        // k = 0 for j = 0 (x[0] = yp, x[half] = ym)
        const int k = (j == 0) ? 0 : om;
        const float2 lo = (j == 0) ? yp : ym, hi = (j == 0) ? ym : yp;
        st_pair(buf, k, cadd(lo, hi), csub(lo, hi));
    }
    __syncthreads();
    fft_general_passes<BPT>(buf, tw, np, half, tid, NT);
    // last inverse pass with the two halves swapped (source/cfft.cpp:355-368).  Only real parts
    // are used from here on, so the pass forms Re(x w) alone and stores floats.
    float* re = reinterpret_cast<float*>(buf);
    float ar[BPT], br[BPT];
#pragma unroll
    for (int i = 0; i < BPT; i++) {
        const int j = tid + i * NT;
        const float2 x = buf[fsw(j + half)], w = __ldg(tw + half + j);
        ar[i] = buf[fsw(j)].x;
        br[i] = fsub(fmul(x.x, w.x), fmul(x.y, w.y));   // Re of cmul(x, w)
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < BPT; i++) {
        const int j = tid + i * NT;
        re[j] = fsub(ar[i], br[i]);
        re[j + half] = fadd(ar[i], br[i]);
    }
    __syncthreads();

    // ---- R7: CFft::FFT1 reversal + 1/n (source/cfft.cpp:418-425), extraction at ihoffset and
    // the 1/16 sub-sample int table (source/general.cpp:2130-2137).
    const float inv_n = 1.0f / (float)n;
    const int ixdimp = p.d.ixdimp;
    const int rbase = n - 1 - p.d.ihoffset;  // q[j] = re[rbase - j] / n
    if (p.table && p.table_fmt == kTabInt16) {
        // dense 16-int table: thread t writes 16-byte group m = t, t + NT, ... (entries 4m .. 4m+3,
        // pixel j = m / 4), so each warp store covers 512 contiguous bytes; the pixel's p0 and
        // slope are formed per group with the same operations as below
        int4* tab4 = reinterpret_cast<int4*>(p.table + (size_t)job.dst * p.table_stride);
        for (int m = tid; m < 4 * ixdimp; m += NT) {
            const int j = m >> 2, k0 = (m & 3) * 4;
            const float qj = fmul(re[rbase - j], inv_n);
            const float p0 = fmul(qj, 100.0f);
            float p1p0 = 0.0f;
            if (j != ixdimp - 1) {
                const float qn = fmul(re[rbase - j - 1], inv_n);
                p1p0 = fmul(fmul(fsub(qn, qj), 0.0625f), 100.0f);  // (q1-q0)/16*100
            }
            tab4[m] = make_int4(__float2int_rz(fadd(p0, fmul(p1p0, (float)k0))),
                                __float2int_rz(fadd(p0, fmul(p1p0, (float)(k0 + 1)))),
                                __float2int_rz(fadd(p0, fmul(p1p0, (float)(k0 + 2)))),
                                __float2int_rz(fadd(p0, fmul(p1p0, (float)(k0 + 3)))));
        }
    } else if (p.table) {   // float pairs or the padded 17-word layout
        int* tab = p.table + (size_t)job.dst * p.table_stride;
        for (int j = tid; j < ixdimp; j += NT) {
            const float qj = fmul(re[rbase - j], inv_n);
            const float p0 = fmul(qj, 100.0f);
            float p1p0 = 0.0f;
            if (j != ixdimp - 1) {
                const float qn = fmul(re[rbase - j - 1], inv_n);
                p1p0 = fmul(fmul(fsub(qn, qj), 0.0625f), 100.0f);  // (q1-q0)/16*100
            }
            if (p.table_fmt == kTabPair) {
                reinterpret_cast<float2*>(tab)[j] = make_float2(p0, p1p0);
                continue;
            }
            // 17 words per detector pixel (the 17th unused): shared-memory bank spreading
            int* dst = tab + 17 * (size_t)j;
#pragma unroll
            for (int k = 0; k < 16; k++) dst[k] = __float2int_rz(fadd(p0, fmul(p1p0, (float)k)));
        }
        // pair tables are copied in 16-byte units: an odd row ends with a zero pair
        if (p.table_fmt == kTabPair && (ixdimp & 1) && tid == 0)
            reinterpret_cast<float2*>(tab)[ixdimp] = make_float2(0.0f, 0.0f);
    }
    if (p.rows16) {
        // LIN forms: pairs (r[j], r[j+1] - r[j]) of r = q * 100 (slope 0 at the last sample, zero
        // pairs up to the padded stride), FP32, FP16 scaled by the launch's power of two (exact;
        // it keeps every row of the filter far from overflow), or BF16 unscaled (it has FP32's
        // exponent range); row_scale holds the scale (1 for BF16)
        const float scale = p.mode == RV_MODE_LIN_F16 ? p.lin16_scale : 1.0f;
        const float rs = 1.0f / scale;   // exact: a power of two
        if (p.mode != RV_MODE_LIN && tid == 0) p.row_scale[job.dst] = scale;
        const int ps = (int)p.row_stride;
        for (int j = tid; j < ps; j += NT) {
            float v0 = 0.0f, dv = 0.0f;
            if (j < ixdimp) {
                v0 = fmul(fmul(re[rbase - j], inv_n), 100.0f);
                if (j + 1 < ixdimp) dv = fsub(fmul(fmul(re[rbase - j - 1], inv_n), 100.0f), v0);
            }
            const size_t at = (size_t)job.dst * p.row_stride + j;
            if (p.mode == RV_MODE_LIN) static_cast<float2*>(p.rows16)[at] = make_float2(v0, dv);
            else if (p.mode == RV_MODE_LIN_F16) static_cast<__half2*>(p.rows16)[at] = __floats2half2_rn(v0 * rs, dv * rs);
            else static_cast<__nv_bfloat162*>(p.rows16)[at] = __floats2bfloat162_rn(v0 * rs, dv * rs);
        }
    }
}

float fp16_row_scale(const float* filt, int ndim) {
    double s2 = 0.0;
    for (int k = 0; k < ndim; k++) {
        const double h = 0.5 * ((double)filt[k] + (double)filt[(ndim - k) % ndim]);
        s2 += h * h;
    }
    const double bound = 100.0 * 32768.0 * sqrt(s2);
    int e = bound > 0.0 ? (int)ceil(log2(bound / 16384.0)) : 0;
    e = e < -20 ? -20 : (e > 40 ? 40 : e);
    return ldexpf(1.0f, e);
}

cudaError_t launch_filter(const FilterLaunch& p, cudaStream_t s) {
    if (p.njobs <= 0) return cudaSuccess;
    if (p.raw) ensure_exp_bound(s);
    const int n = p.d.ndim, half = n / 2;
    // eight butterflies per thread where the row allows (measured best: a 4096-point row 6.10 ms
    // per 64-slice step with 256 threads, 6.55 with 512, 7.95 with 128; an 8192-point row 13.6 ms
    // per 32-slice step with 512 threads, 14.8 with 256); at most 512 threads, at least a warp
    int nt = half / 8;
    if (nt > 512) nt = 512;
    if (nt < 32) nt = half < 32 ? half : 32;
    const int bpt = half / nt;
    const size_t smem = (size_t)n * sizeof(float2) +
                        (((size_t)p.d.ixdim * sizeof(short) + 15) & ~(size_t)15);
    cudaError_t e = cudaSuccess;
    auto go = [&](auto kern) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return;
        kern<<<p.njobs, nt, smem, s>>>(p);
        e = cudaGetLastError();
    };
    switch (bpt) {
    case 1: go(k_filter<1>); break;
    case 2: go(k_filter<2>); break;
    case 4: go(k_filter<4>); break;
    case 8: go(k_filter<8>); break;
    case 16: go(k_filter<16>); break;
    default: return cudaErrorInvalidValue;
    }
    return e;
}

// plain 16-byte copy (grid-stride): writes host memory directly where the device can
__global__ void k_copy16(int4* __restrict__ dst, const int4* __restrict__ src, size_t n16) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

cudaError_t launch_copy16(void* dst, const void* src, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if ((n & 15) || (reinterpret_cast<uintptr_t>(dst) & 15) || (reinterpret_cast<uintptr_t>(src) & 15))
        return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_copy16<<<2 * sms, 512, 0, s>>>(static_cast<int4*>(dst), static_cast<const int4*>(src), n / 16);
    return cudaGetLastError();
}

bool host_direct_access() {
    static int cached[64];   // per device: 0 unknown, 1 yes, 2 no
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (!cached[dev]) {
        int pageable = 0, host_tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
        const char* off = getenv("RV_NO_HOST_DIRECT");
        cached[dev] = (pageable && host_tables && !(off && atoi(off))) ? 1 : 2;
    }
    return cached[dev] == 1;
}

cudaError_t launch_backproject(const BackprojLaunch& p, cudaStream_t s) {
    if (p.nslices <= 0) return cudaSuccess;
    if (p.ixdimp > kMaxIxdimp) return cudaErrorInvalidValue;
    if (p.mode == RV_MODE_REF) return launch_bp_ref(p, s);
    return launch_bp_lin(p, s);
}

int kernel_launches_per_filter() { return 1; }

}  // namespace rv

// ---------------------------------------------------------------------------------------------
// Throughput probes for the roofline denominators of the back-projection (an FP32/conversion-
// issue-bound kernel): FP32 FMA rate and float->int conversion rate of the whole device.
// ---------------------------------------------------------------------------------------------
namespace rv {
__global__ void k_probe_fma(float* sink, int iters) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = threadIdx.x * 1e-3f + k;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = fmaf(a[k], 0.9999f, 1e-3f);
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += a[k];
    if (s == 1234.5f) sink[0] = s;
}
__global__ void k_probe_f2i(int* sink, int iters) {
    float x[8];
    int acc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { x[k] = threadIdx.x + k * 3.7f; acc[k] = 0; }
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            acc[k] += __float2int_rz(x[k]);
            x[k] = __fadd_rn(x[k], 1.25f);
        }
    }
    int s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += acc[k];
    if (s == 123457) sink[0] = s;
}
// Conflict-free 32-bit shared-memory loads: each warp instruction reads 32 consecutive words
// (one 128-byte wavefront); ld.volatile keeps every load inside the loop (plain loads of an
// unchanging address would be hoisted out of it).
__global__ void k_probe_lds(int* sink, int iters) {
    __shared__ int buf[8 * 1024];
    for (int i = threadIdx.x; i < 8 * 1024; i += blockDim.x) buf[i] = i;
    __syncthreads();
    const unsigned base = static_cast<unsigned>(__cvta_generic_to_shared(buf)) + 4u * (threadIdx.x & 1023u);
    int acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < iters; i++) {
        int v[8];
        asm volatile(
            "ld.volatile.shared.s32 %0, [%8];\n ld.volatile.shared.s32 %1, [%8+4096];\n"
            " ld.volatile.shared.s32 %2, [%8+8192];\n ld.volatile.shared.s32 %3, [%8+12288];\n"
            " ld.volatile.shared.s32 %4, [%8+16384];\n ld.volatile.shared.s32 %5, [%8+20480];\n"
            " ld.volatile.shared.s32 %6, [%8+24576];\n ld.volatile.shared.s32 %7, [%8+28672];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
            : "r"(base));
#pragma unroll
        for (int k = 0; k < 8; k++) acc[k] += v[k];
    }
    int s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += acc[k];
    if (s == 123457) sink[0] = s;
}
}  // namespace rv

extern "C" int RvHostDirectAccess(void) { return rv::host_direct_access() ? 1 : 0; }

extern "C" int RvProbeThroughput(double* out, int n) {
    if (!out || n < 2) return RV_ERR_BAD_ARGUMENT;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* sink = nullptr;
    if (cudaMalloc(&sink, 64) != cudaSuccess) return RV_ERR_DEVICE_OOM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 4, threads = 512, iters = 4096;
    double res[3] = {0, 0, 0};
    for (int which = 0; which < (n >= 3 ? 3 : 2); which++) {
        float best = 1e30f;
        for (int rep = 0; rep < 4; rep++) {
            cudaEventRecord(e0);
            if (which == 0) rv::k_probe_fma<<<blocks, threads>>>((float*)sink, iters);
            else if (which == 1) rv::k_probe_f2i<<<blocks, threads>>>((int*)sink, iters);
            else rv::k_probe_lds<<<blocks, threads>>>((int*)sink, iters);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms < best) best = ms;
        }
        const double ops = (double)blocks * threads * iters * 8;
        if (which == 0) res[0] = 2.0 * ops / (best * 1e-3) / 1e12;   // FLOP/s
        else if (which == 1) res[1] = ops / (best * 1e-3) / 1e9;       // conversions/s
        else res[2] = 4.0 * ops / (best * 1e-3) / 1e9;                 // bytes/s of 32-bit loads
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    out[0] = res[0];  // FP32 FMA TFLOP/s
    out[1] = res[1];  // float->int32 conversions, G/s
    if (n >= 3) out[2] = res[2];  // shared-memory load bandwidth, GB/s (conflict-free 32-bit loads)
    return cudaGetLastError() == cudaSuccess ? 0 : RV_ERR_LAUNCH;
}
