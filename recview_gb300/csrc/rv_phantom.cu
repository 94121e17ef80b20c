// Device-side data for the learned centre search (no reference counterpart):
//
//  RvPhantomFrames   seeded synthetic raw uint16 frames of an ellipsoid phantom -- flats, samples at
//                    given angles, dark -- with Poisson-like noise, in the stack layout
//                    [(frames+1)][S][W].  The same distributions as the tests' numpy phantom
//                    (recview_gb300/phantom.py) but generated on the device, so thousands of
//                    full-size datasets cost seconds.
//  RvNormaliseStack  the reference's flat/dark log normalisation (GenerateSinogramThread,
//                    source/general.cpp:2377-2532) of every sample frame of a device-resident raw
//                    stack into int16 rows, with the same kernel as CudaSinogramHost.
//  RvCentreNetInput  the network input: four detector rows, 256 views chosen in angle order,
//                    detector bins averaged to 512, log values / 3000, bf16, and the view axis
//                    rearranged so that the two halves of the half-turn meet at the middle row:
//                    rows 0..127 = views 90..180 degrees as measured, rows 128..255 = views
//                    0..90 degrees mirrored about the detector centre.  A view at theta mirrored
//                    that way equals the view at theta + 180 shifted by 2 (centre - detector
//                    centre), so the centre offset becomes a local horizontal shift across the
//                    middle row -- something a small convolutional network can measure.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "rv_internal.h"

using namespace rv;

namespace {

struct Ell {
    float x0, z0, a, b, phi, mu;
};

// splitmix64 stream (host)
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0xD1B54A32D192ED03ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((double)(next() >> 11) + 0.5) / 9007199254740992.0; }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    double normal() { return sqrt(-2.0 * log(uniform())) * cos(6.283185307179586 * uniform()); }
};

// counter-based device noise: a standard normal from (seed, index)
__device__ __forceinline__ uint32_t mix32(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k;
}
__device__ __forceinline__ float gauss(uint64_t seed, uint64_t i) {
    const float u1 = ((float)mix32(seed ^ (2 * i)) + 0.5f) * 2.3283064365386963e-10f;
    const float u2 = ((float)mix32(seed ^ (2 * i + 1) ^ 0x5bd1e995ull) + 0.5f) * 2.3283064365386963e-10f;
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

// raw[(F+1)][S][W]: frame f < F is a flat (theta < 0 marks it) or a sample at theta; F = dark.
__global__ void k_phantom_frames(const Ell* ells, const int* nell, int maxell, const float* theta, const float* flat,
                                 const float* dark, int F, int S, int W, double center, uint64_t seed, uint16_t* raw) {
    const long long total = (long long)(F + 1) * S * W;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % W);
        const int s = (int)((i / W) % S);
        const int f = (int)(i / ((long long)W * S));
        const float dk = dark[(size_t)s * W + x];
        float v;
        if (f == F) {
            v = rintf(dk);
        } else {
            float p = 0.0f;
            const float th = theta[f];
            if (th >= 0.0f) {
                const float c = cosf(th), sn = sinf(th);
                const float t = (float)(((double)x - center) / (W / 2.0));
                const Ell* e = ells + (size_t)s * maxell;
                for (int k = 0; k < nell[s]; k++) {
                    const float sc = e[k].x0 * c + e[k].z0 * sn;
                    const float d = th - e[k].phi;
                    const float ca = e[k].a * cosf(d), sb = e[k].b * sinf(d);
                    const float a2 = ca * ca + sb * sb;
                    const float u = t - sc;
                    const float rad = a2 - u * u;
                    if (rad > 0.0f) p += 2.0f * e[k].mu * e[k].a * e[k].b * sqrtf(rad) / a2;
                }
            }
            const float lam = flat[(size_t)s * W + x] * expf(-p);
            v = rintf(lam + sqrtf(fmaxf(lam, 0.0f)) * gauss(seed, (uint64_t)i)) + dk;
        }
        raw[i] = (uint16_t)fminf(fmaxf(v, 0.0f), 65535.0f);
    }
}

// out[c][r][b] for the 256 x 512 input (see the file comment); in = int16 rows [frames][S][W]
__global__ void k_centre_input(const short* sino, const int* frames, int S, int W, int s0, __nv_bfloat16* out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;   // bin
    const int r = blockIdx.y;                              // row
    const int c = blockIdx.z;                              // detector row (slice)
    if (b >= 512) return;
    const int f = W / 512;
    const bool mirrored = r >= 128;
    const int frame = frames[mirrored ? r - 128 : r + 128];
    const short* row = sino + ((size_t)frame * S + s0 + c) * W;
    float acc = 0.0f;
    for (int k = 0; k < f; k++) {
        const int xs = b * f + k;
        acc += (float)row[mirrored ? W - 1 - xs : xs];
    }
    out[((size_t)c * 256 + r) * 512 + b] = __float2bfloat16_rn(acc / ((float)f * 3000.0f));
}

}  // namespace

extern "C" int RvPhantomFrames(unsigned long long seed, int W, int S, const float* view_deg, int nviews, double center,
                               int n_ellipsoids, void* d_raw, char* bInc, float* fdeg, float* fexp, void* stream) {
    if (W < 8 || S < 1 || nviews < 1 || !view_deg || !d_raw || n_ellipsoids < 0 || n_ellipsoids > 4096) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvPhantomFrames: invalid argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    cudaStream_t st = (cudaStream_t)stream;
    Rng rng(seed);
    // ellipsoids (x0, z0, y0, a, b, c, phi, mu): centres uniform in a ball of radius 0.8
    std::vector<double> e3((size_t)n_ellipsoids * 8);
    for (int k = 0; k < n_ellipsoids; k++) {
        double v0 = rng.normal(), v1 = rng.normal(), v2 = rng.normal();
        const double nrm = sqrt(v0 * v0 + v1 * v1 + v2 * v2) + 1e-300;
        const double r = 0.8 * cbrt(rng.uniform());
        double* q = &e3[(size_t)k * 8];
        q[0] = v0 / nrm * r;
        q[1] = v1 / nrm * r;
        q[2] = v2 / nrm * r;
        q[3] = rng.uniform(0.05, 0.4);
        q[4] = rng.uniform(0.05, 0.4);
        q[5] = rng.uniform(0.05, 0.4);
        q[6] = rng.uniform(0.0, 3.141592653589793);
        q[7] = rng.uniform(-0.2, 1.0);
    }
    // per-slice cross-sections at heights spread over [-0.25, 0.25]
    std::vector<Ell> ells((size_t)S * (n_ellipsoids > 0 ? n_ellipsoids : 1));
    std::vector<int> nell(S, 0);
    const int maxell = n_ellipsoids > 0 ? n_ellipsoids : 1;
    for (int s = 0; s < S; s++) {
        const double y = (s - (S - 1) / 2.0) / (S > 2 ? S / 2.0 : 1.0) * 0.5;
        for (int k = 0; k < n_ellipsoids; k++) {
            const double* q = &e3[(size_t)k * 8];
            const double u = (y - q[2]) / q[5];
            if (fabs(u) >= 1.0) continue;
            const double sc = sqrt(1.0 - u * u);
            ells[(size_t)s * maxell + nell[s]++] = {(float)q[0], (float)q[1], (float)(q[3] * sc), (float)(q[4] * sc),
                                                    (float)q[6], (float)q[7]};
        }
    }
    // flat field 20000 (1 + 0.02 smooth) as a few random sinusoids per row; dark ~ N(100, 3)
    std::vector<float> flat((size_t)S * W), dark((size_t)S * W);
    for (int s = 0; s < S; s++) {
        double amp[4], fr[4], ph[4];
        for (int k = 0; k < 4; k++) {
            amp[k] = rng.normal() * 0.5;
            fr[k] = rng.uniform(0.5, 6.0) * 6.283185307179586 / W;
            ph[k] = rng.uniform(0.0, 6.283185307179586);
        }
        for (int x = 0; x < W; x++) {
            double n = 0.0;
            for (int k = 0; k < 4; k++) n += amp[k] * sin(fr[k] * x + ph[k]);
            flat[(size_t)s * W + x] = (float)(20000.0 * (1.0 + 0.02 * n));
            dark[(size_t)s * W + x] = (float)(100.0 + 3.0 * rng.normal());
        }
    }
    // frames: flat, samples, flat (dark appended by the kernel)
    const int F = nviews + 2;
    std::vector<float> theta(F);
    std::vector<char> binc(F);
    std::vector<float> deg(F), exp_t(F);
    for (int f = 0; f < F; f++) {
        const bool sample = f >= 1 && f <= nviews;
        theta[f] = sample ? (float)((double)view_deg[f - 1] * (3.141592653589793 / 180.0)) : -1.0f;
        binc[f] = sample ? RV_BINC_SAMPLE : 0;
        deg[f] = sample ? view_deg[f - 1] : (f == 0 ? 0.0f : view_deg[nviews - 1]);
        exp_t[f] = (float)f;
    }
    if (bInc) memcpy(bInc, binc.data(), F);
    if (fdeg) memcpy(fdeg, deg.data(), sizeof(float) * F);
    if (fexp) memcpy(fexp, exp_t.data(), sizeof(float) * F);
    const size_t ell_b = sizeof(Ell) * ells.size(), n_b = sizeof(int) * S, th_b = sizeof(float) * F,
                 fd_b = sizeof(float) * (size_t)S * W;
    const size_t off_n = ell_b, off_th = off_n + n_b, off_fl = (off_th + th_b + 15) & ~(size_t)15, off_dk = off_fl + fd_b;
    const size_t total_b = off_dk + fd_b;
    std::vector<unsigned char> h(total_b);
    memcpy(h.data(), ells.data(), ell_b);
    memcpy(h.data() + off_n, nell.data(), n_b);
    memcpy(h.data() + off_th, theta.data(), th_b);
    memcpy(h.data() + off_fl, flat.data(), fd_b);
    memcpy(h.data() + off_dk, dark.data(), fd_b);
    unsigned char* d = nullptr;
    if (!cuda_ok(cudaMallocAsync((void**)&d, total_b, st), RV_ERR_DEVICE_OOM, "phantom parameters"))
        return RV_ERR_DEVICE_OOM;
    int rc = 0;
    if (!cuda_ok(cudaMemcpyAsync(d, h.data(), total_b, cudaMemcpyHostToDevice, st), RV_ERR_COPY_H2D, "phantom"))
        rc = RV_ERR_COPY_H2D;
    if (!rc) {
        const long long n = (long long)(F + 1) * S * W;
        const int blocks = (int)((n + 255) / 256 < 152 * 64 ? (n + 255) / 256 : 152 * 64);
        k_phantom_frames<<<blocks, 256, 0, st>>>((const Ell*)d, (const int*)(d + off_n), maxell,
                                                 (const float*)(d + off_th), (const float*)(d + off_fl),
                                                 (const float*)(d + off_dk), F, S, W, center, seed * 0x2545F4914F6CDD1Dull,
                                                 static_cast<uint16_t*>(d_raw));
        if (!cuda_ok(cudaGetLastError(), RV_ERR_LAUNCH, "phantom kernel")) rc = RV_ERR_LAUNCH;
    }
    // the pageable staging buffer must outlive the copy
    if (!cuda_ok(cudaStreamSynchronize(st), RV_ERR_LAUNCH, "phantom")) rc = rc ? rc : RV_ERR_LAUNCH;
    cudaFreeAsync(d, st);
    return rc;
}

extern "C" int RvNormaliseStack(const RvStackDesc* desc, const void* d_raw, short* d_sino, void* stream) {
    // GenerateSinogramThread's flat bracketing (source/general.cpp:2412-2447) for every SAMPLE frame;
    // rows of other frames are zero
    if (!desc || !d_raw || !d_sino || !desc->bInc || !desc->fexp || desc->nframes < 1 || desc->nslices < 1 ||
        desc->ixdim < 1) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvNormaliseStack: invalid description");
        return RV_ERR_BAD_ARGUMENT;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int nf = desc->nframes, S = desc->nslices, W = desc->ixdim;
    const char* bInc = desc->bInc;
    std::vector<RowJob> jobs;
    int i0 = -1, i1 = -1;
    for (int i = 0; i < nf; i++) {
        if (bInc[i] & RV_BINC_NOUSE) continue;
        if (!(bInc[i] & RV_BINC_SAMPLE)) { i0 = i; break; }
    }
    for (int i = 0; i < nf; i++) {
        if ((bInc[i] & RV_BINC_NOUSE) && !(bInc[i] & RV_BINC_SAMPLE)) continue;
        if (!(bInc[i] & RV_BINC_SAMPLE)) { i0 = i; i1 = -1; continue; }
        if (i1 < 0) {
            for (int j = i; j < nf; j++) {
                if (bInc[j] & RV_BINC_SAMPLE) continue;
                i1 = j;
                break;
            }
            if (i1 < 0 && i0 >= 0) i1 = i0;
        }
        if (i0 < 0 || i1 < 0) {
            set_error(RV_ERR_BAD_ARGUMENT, "RvNormaliseStack: a sample frame has no flat frame");
            return RV_ERR_BAD_ARGUMENT;
        }
        float t0 = desc->fexp[i0];
        const float t1 = desc->fexp[i1], ti = desc->fexp[i];
        if (t0 == t1) t0 = 0;
        else t0 = (ti - t0) / (t1 - t0);
        for (int s = 0; s < S; s++) {
            RowJob j{};
            j.src_row = i * S + s;
            j.flat0_row = i0 * S + s;
            j.flat1_row = i1 * S + s;
            j.dark_row = nf * S + s;
            j.t0 = t0;
            j.zero = (bInc[i] & RV_BINC_SKIP) ? 1 : 0;
            j.dst = i * S + s;
            jobs.push_back(j);
        }
    }
    if (!cuda_ok(cudaMemsetAsync(d_sino, 0, sizeof(short) * (size_t)(nf + 1) * S * W, st), RV_ERR_MEMSET, "sinogram"))
        return RV_ERR_MEMSET;
    if (jobs.empty()) return cuda_ok(cudaStreamSynchronize(st), RV_ERR_LAUNCH, "normalise") ? 0 : RV_ERR_LAUNCH;
    RowJob* d_jobs = nullptr;
    if (!cuda_ok(cudaMallocAsync((void**)&d_jobs, sizeof(RowJob) * jobs.size(), st), RV_ERR_DEVICE_OOM, "row jobs"))
        return RV_ERR_DEVICE_OOM;
    int rc = 0;
    if (!cuda_ok(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(RowJob) * jobs.size(), cudaMemcpyHostToDevice, st),
                 RV_ERR_COPY_H2D, "row jobs"))
        rc = RV_ERR_COPY_H2D;
    if (!rc) {
        NormLaunch nl{};
        nl.raw = static_cast<const uint16_t*>(d_raw);
        nl.out = d_sino;
        nl.jobs = d_jobs;
        nl.njobs = (int)jobs.size();
        nl.ixdim = W;
        nl.pixmin = (desc->iFlag & RV_READTIF8bit) ? RV_SINOGRAM_PIXEL_MIN8bit : RV_SINOGRAM_PIXEL_MIN16bit;
        nl.zernike = (desc->dReconFlags & RV_RQFLAGS_ZERNIKE) ? 1 : 0;
        nl.shift = nullptr;
        if (!cuda_ok(launch_normalise(nl, st), RV_ERR_LAUNCH, "normalise kernel")) rc = RV_ERR_LAUNCH;
    }
    if (!cuda_ok(cudaStreamSynchronize(st), RV_ERR_LAUNCH, "normalise")) rc = rc ? rc : RV_ERR_LAUNCH;
    cudaFreeAsync(d_jobs, st);
    return rc;
}

extern "C" int RvCentreNetInput(const short* d_sino, int S, int W, const int* frames256, int s0, void* d_x,
                                void* stream) {
    if (!d_sino || !frames256 || !d_x || W < 512 || (W % 512) || s0 < 0 || s0 + 4 > S) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvCentreNetInput: W must be a multiple of 512 and 4 rows from s0 must exist");
        return RV_ERR_BAD_ARGUMENT;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int* d_fr = nullptr;
    if (!cuda_ok(cudaMallocAsync((void**)&d_fr, sizeof(int) * 256, st), RV_ERR_DEVICE_OOM, "frames")) return RV_ERR_DEVICE_OOM;
    int rc = 0;
    if (!cuda_ok(cudaMemcpyAsync(d_fr, frames256, sizeof(int) * 256, cudaMemcpyHostToDevice, st), RV_ERR_COPY_H2D, "frames"))
        rc = RV_ERR_COPY_H2D;
    if (!rc) {
        k_centre_input<<<dim3(2, 256, 4), 256, 0, st>>>(d_sino, d_fr, S, W, s0, static_cast<__nv_bfloat16*>(d_x));
        if (!cuda_ok(cudaGetLastError(), RV_ERR_LAUNCH, "input kernel")) rc = RV_ERR_LAUNCH;
    }
    if (!cuda_ok(cudaStreamSynchronize(st), RV_ERR_LAUNCH, "input")) rc = rc ? rc : RV_ERR_LAUNCH;
    cudaFreeAsync(d_fr, st);
    return rc;
}
