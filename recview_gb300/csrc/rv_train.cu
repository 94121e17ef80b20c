// Training of the centre-proposal network on synthetic scans (no reference counterpart).  Every
// sample is made by the plain method itself: seeded raw frames (RvPhantomFrames) with a known
// centre offset, the reference's normalisation (RvNormaliseStack), and the network input
// (RvCentreNetInput); the target is offset / 16.  Samples stay resident in HBM as bf16 (1 MB
// each), batches are gathered on the device, and the network's own kernels take Adam steps on a
// cosine learning-rate schedule (RvCentreNetTrainStep).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "rv_internal.h"

using namespace rv;

namespace {
constexpr size_t kSampleElems = (size_t)4 * 256 * 512;

uint64_t smix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double sunif(uint64_t& s) { return ((double)(smix(s) >> 11) + 0.5) / 9007199254740992.0; }
}  // namespace

// The 256 frames of a scan the network reads: views nearest to r * views / 256 (angle order).
static void chosen_views(int views, std::vector<float>& deg) {
    deg.resize(256);
    for (int r = 0; r < 256; r++) {
        int i = (int)floor((double)r * views / 256.0 + 0.5);
        if (i >= views) i = views - 1;
        deg[r] = (float)((double)i * (180.0 / views));
    }
}

extern "C" int RvCentreNetMakeSamples(const RvCentreTrainDesc* d, int first, int count, void* d_x, float* d_y,
                                      void* stream) {
    if (!d || !d_x || !d_y || count < 1 || first < 0 || d->W < 512 || (d->W % 512) || d->slices < 4 ||
        d->views < 256) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvCentreNetMakeSamples: invalid description");
        return RV_ERR_BAD_ARGUMENT;
    }
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<float> deg;
    chosen_views(d->views, deg);
    const int F = 256 + 2, S = d->slices, W = d->W;
    void *raw = nullptr, *sino = nullptr;
    if (!cuda_ok(cudaMalloc(&raw, (size_t)(F + 1) * S * W * 2), RV_ERR_DEVICE_OOM, "sample frames") ||
        !cuda_ok(cudaMalloc(&sino, (size_t)(F + 1) * S * W * 2), RV_ERR_DEVICE_OOM, "sample rows")) {
        if (raw) cudaFree(raw);
        return RV_ERR_DEVICE_OOM;
    }
    std::vector<char> binc(F);
    std::vector<float> fdeg(F), fexp(F), y(count);
    int f256[256];
    for (int r = 0; r < 256; r++) f256[r] = 1 + r;
    int rc = 0;
    for (int i = 0; i < count && !rc; i++) {
        const unsigned long long seed = d->seed * 1000003ull + (unsigned long long)(first + i);
        uint64_t s = seed ^ 0x6A09E667F3BCC909ull;
        const double off = (2.0 * sunif(s) - 1.0) * d->max_offset;
        rc = RvPhantomFrames(seed, W, S, deg.data(), 256, (W - 1) / 2.0 + off, d->n_ellipsoids, raw, binc.data(),
                             fdeg.data(), fexp.data(), stream);
        if (rc) break;
        RvStackDesc sd{};
        sd.ixdim = W;
        sd.nframes = F;
        sd.nslices = S;
        sd.bInc = binc.data();
        sd.fdeg = fdeg.data();
        sd.fexp = fexp.data();
        rc = RvNormaliseStack(&sd, raw, static_cast<short*>(sino), stream);
        if (!rc) rc = RvCentreNetInput(static_cast<const short*>(sino), S, W, f256, 0,
                                       static_cast<__nv_bfloat16*>(d_x) + (size_t)i * kSampleElems, stream);
        y[i] = (float)(off / 16.0);
    }
    if (!rc && !cuda_ok(cudaMemcpyAsync(d_y, y.data(), sizeof(float) * count, cudaMemcpyHostToDevice, st),
                        RV_ERR_COPY_H2D, "targets"))
        rc = RV_ERR_COPY_H2D;
    if (!cuda_ok(cudaStreamSynchronize(st), RV_ERR_LAUNCH, "samples")) rc = rc ? rc : RV_ERR_LAUNCH;
    cudaFree(raw);
    cudaFree(sino);
    return rc;
}

extern "C" int RvCentreNetFit(RvCentreNet* net, const void* d_x, const float* d_y, int ntrain, int nval, int epochs,
                              int batch, float lr_max, float lr_min, unsigned long long seed, float* stats, void* stream) {
    if (!net || !d_x || !d_y || ntrain < batch || nval < 0 || epochs < 1 || batch < 1) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvCentreNetFit: invalid argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = (cudaStream_t)stream;
    void* bx = nullptr;
    float* by = nullptr;
    if (!cuda_ok(cudaMalloc(&bx, kSampleElems * 2 * batch), RV_ERR_DEVICE_OOM, "batch") ||
        !cuda_ok(cudaMalloc((void**)&by, sizeof(float) * batch), RV_ERR_DEVICE_OOM, "batch")) {
        if (bx) cudaFree(bx);
        return RV_ERR_DEVICE_OOM;
    }
    std::vector<float> hy(ntrain + nval);
    int rc = cuda_ok(cudaMemcpy(hy.data(), d_y, sizeof(float) * hy.size(), cudaMemcpyDeviceToHost), RV_ERR_COPY_D2H,
                     "targets") ? 0 : RV_ERR_COPY_D2H;
    std::vector<int> perm(ntrain);
    for (int i = 0; i < ntrain; i++) perm[i] = i;
    uint64_t s = seed ^ 0xBB67AE8584CAA73Bull;
    const long long steps = (long long)epochs * (ntrain / batch);
    long long step = 0;
    std::vector<float> yb(batch);
    const __nv_bfloat16* X = static_cast<const __nv_bfloat16*>(d_x);
    for (int ep = 0; ep < epochs && !rc; ep++) {
        for (int i = ntrain - 1; i > 0; i--) std::swap(perm[i], perm[(int)(smix(s) % (uint64_t)(i + 1))]);
        for (int b0 = 0; b0 + batch <= ntrain && !rc; b0 += batch, step++) {
            for (int j = 0; j < batch; j++) {
                const int idx = perm[b0 + j];
                if (!cuda_ok(cudaMemcpyAsync(static_cast<__nv_bfloat16*>(bx) + (size_t)j * kSampleElems,
                                             X + (size_t)idx * kSampleElems, kSampleElems * 2, cudaMemcpyDeviceToDevice, st),
                             RV_ERR_COPY_H2D, "batch gather")) { rc = RV_ERR_COPY_H2D; break; }
                yb[j] = hy[idx];
            }
            if (rc) break;
            // pageable targets: the copy completes before the call returns
            if (!cuda_ok(cudaMemcpyAsync(by, yb.data(), sizeof(float) * batch, cudaMemcpyHostToDevice, st),
                         RV_ERR_COPY_H2D, "batch targets")) { rc = RV_ERR_COPY_H2D; break; }
            const float lr = lr_min + 0.5f * (lr_max - lr_min) * (1.0f + cosf(3.14159265f * (float)step / (float)steps));
            rc = RvCentreNetTrainStep(net, bx, by, batch, lr, nullptr, stream);
        }
    }
    // held-out error of the proposal, in pixels (|16 (mu - y)|), and the wall time
    if (!rc && stats) {
        std::vector<double> err;
        std::vector<float> mu(batch);
        for (int v0 = ntrain; v0 < ntrain + nval && !rc; v0 += batch) {
            const int n = std::min(batch, ntrain + nval - v0);
            rc = RvCentreNetForward(net, X + (size_t)v0 * kSampleElems, n, mu.data(), nullptr, stream);
            for (int j = 0; j < n && !rc; j++) err.push_back(fabs(16.0 * ((double)mu[j] - hy[v0 + j])));
        }
        std::sort(err.begin(), err.end());
        auto pct = [&](double p) { return err.empty() ? 0.0 : err[std::min(err.size() - 1, (size_t)(p * err.size()))]; };
        stats[0] = (float)pct(0.5);
        stats[1] = (float)pct(0.9);
        stats[2] = (float)pct(0.99);
        stats[3] = (float)std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    cudaStreamSynchronize(st);
    cudaFree(bx);
    cudaFree(by);
    return rc;
}
