// R11: the plain rotation-centre methods.
//
//  RvGetAxis      CGazoDoc::GetAxis (source/gazoDoc.cpp:4036-4626): the 0-degree and ~180-degree
//                 frames are log-converted against a flat, each sampled detector row of the
//                 mirrored 180-degree frame is slid over the 0-degree row, and the sum of squared
//                 differences (SSD) per shift gives a per-row centre (parabola refined), an overall
//                 centre, and a least-squares line centre(iy) = b + a iy.  The SSD matrix is computed
//                 on the device in int64 -- exact, so it equals the reference's double sums -- and
//                 the arg-min / parabola / line-fit bookkeeping runs on the host in the reference's
//                 double/float arithmetic.
//  RvCentreSweep  the axis-scan batch (source/gazoDoc.cpp:1994-2024) -- one slice reconstructed at
//                 many trial centres -- plus a score the reference does not have (it writes one TIFF
//                 per centre and leaves the choice to a person): the total variation of each slice,
//                 box-averaged to about 512 x 512 values, inside the reconstruction circle, lowest =
//                 sharpest (project-defined), with a parabola through the best three trials.  Run
//                 with a smoothing filter (e.g. Hann, cutoff 0.25) the criterion is unimodal over
//                 tens of pixels on noisy full-size data.
#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "rv_internal.h"

namespace rv {

// (short)(log(flat / sample) * LOG_SCALE) (source/gazoDoc.cpp:4380-4381): no +0.5 and no dark; the
// double->short conversion of an out-of-range value (a zero pixel gives +-inf or NaN) follows the
// x64 conversion the reference ran on: the integer-indefinite value, whose low 16 bits are 0.
__device__ __forceinline__ int axis_log(int flat, int sample) {
    const double v = __dmul_rn(log(__ddiv_rn((double)flat, (double)sample)), 3000.0);
    if (!(v > -2147483649.0 && v < 2147483648.0)) return 0;
    return (int)(short)__double2int_rz(v);
}

__global__ void k_axis_log(const uint16_t* s0, const uint16_t* s1, const uint16_t* flat, int* o0, int* o1, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        o0[i] = axis_log(flat[i], s0[i]);
        o1[i] = axis_log(flat[i], s1[i]);
    }
}

// SSD of the mirrored row of frame 1 against row k of frame 0 for every shift (non-offset CT,
// source/gazoDoc.cpp:4473-4492) or around the offset axis (offset CT, :4452-4470).  The buffers
// carry a zero tail so the reference's unchecked offset-CT indices stay inside them.
__global__ void k_axis_ssd(const int* S0, const int* S1, int ixdim, int istep, int ixdimh, int offset,
                           long long* ssd, int* nd) {
    const int row = blockIdx.y;
    const int k = row * istep;
    const int js = blockIdx.x * blockDim.x + threadIdx.x - ixdimh;   // shift
    if (js >= ixdimh) return;
    const long long kix = (long long)k * ixdim;
    long long acc = 0;
    int n = 0;
    if (offset) {
        const int scan = (offset < ixdim / 2) ? offset / 2 : (ixdim - offset) / 2;
        if (abs(js) <= scan) {
            const int j = js + offset;
            for (int i = -scan; i <= scan; i++) {
                const long long d = (long long)S1[j - i + kix] - S0[j + i + kix];
                acc += d * d;
                n++;
            }
        }
    } else {
        const int ifrom = js >= 0 ? 0 : -js;
        const int ito = js >= 0 ? ixdim - js : ixdim;
        for (int i = ifrom; i < ito; i++) {
            const long long d = (long long)S1[ixdim - 1 - i + kix] - S0[i + js + kix];
            acc += d * d;
        }
        n = ito > ifrom ? ito - ifrom : 0;
    }
    ssd[(size_t)row * 2 * ixdimh + js + ixdimh] = acc;
    nd[(size_t)row * 2 * ixdimh + js + ixdimh] = n;
}

// Total variation per slice inside the circle r < 0.45 n of the slice averaged over b x b pixel
// boxes, b = max(1, ixdimp / 512) and n = ixdimp / b (about 512 x 512 values whatever the slice
// size, so reconstruction noise does not swamp the edges); deterministic two-level sum.
__device__ __forceinline__ double tv_box(const int* f, int ixdimp, int b, int X, int Y) {
    long long s = 0;
    for (int j = 0; j < b; j++)
        for (int i = 0; i < b; i++) s += f[(size_t)(Y * b + j) * ixdimp + X * b + i];
    return (double)s / (double)(b * b);
}
__global__ void k_tv_partial(const int* slices, int ixdimp, double* partial) {
    const int slice = blockIdx.y;
    const int* f = slices + (size_t)slice * ixdimp * ixdimp;
    const int b = ixdimp / 512 > 1 ? ixdimp / 512 : 1;
    const int nb = ixdimp / b;
    const double h = nb / 2.0, r2 = (0.45 * nb) * (0.45 * nb);
    double acc = 0.0;
    const long long n = (long long)(nb - 1) * (nb - 1);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / (nb - 1)), x = (int)(i % (nb - 1));
        const double dx = x - h, dy = y - h;
        if (dx * dx + dy * dy >= r2) continue;
        const double v = tv_box(f, ixdimp, b, x, y);
        const double gx = tv_box(f, ixdimp, b, x + 1, y) - v;
        const double gy = tv_box(f, ixdimp, b, x, y + 1) - v;
        acc += sqrt(gx * gx + gy * gy);
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        partial[(size_t)slice * gridDim.x + blockIdx.x] = t;
    }
}

// ---- GetAxis host side ---------------------------------------------------------------------
// Twice the rotation centre, in pixels, implied by a relative shift js of the two frames
// (offset-CT frames are shifted by iAxisOffset first).
static int doubled_centre(int js, int iAxisOffset, int ixdim) {
    return iAxisOffset ? (js + iAxisOffset) * 2 : js + ixdim - 1;
}

// Shift (in [-h, h)) of the smallest value among the valid entries of curve[js + h]; the first
// of equal values wins.  The running minimum is held in type R: the reference keeps it in float
// for the per-row curves and in double for the overall one, which can decide between
// near-equal neighbours, so both are kept.
template <typename R>
static int argmin_shift(const std::vector<double>& curve, const std::vector<unsigned char>& valid, int h) {
    R lowest = (R)SHRT_MAX;
    int best = 0;
    for (int idx = 0; idx < 2 * h; idx++) {
        if (!valid[idx] || !(curve[idx] < lowest)) continue;
        lowest = (R)curve[idx];
        best = idx - h;
    }
    return best;
}

// Centre of the parabola through three neighbouring curve values (left, middle, right) around
// doubled centre c2, in the operation order of source/gazoDoc.cpp:4487-4491; a flat pair of
// outer values keeps c2 / 2.
static double parabola_vertex(double left, double mid, double right, int c2) {
    if (right == left) return c2 / 2.;
    const double r = (mid - left) / (right - left);
    return (4 * r * c2 - (c2 * 2 - 1)) / (4 * r - 2) / 2;
}

// The centre of a curve whose arg-min is `best`: refined by the parabola unless the minimum
// sits on the first or last shift.
static double refined_centre(const std::vector<double>& curve, int h, int best, int iAxisOffset, int ixdim) {
    const int c2 = doubled_centre(best, iAxisOffset, ixdim);
    if (best == -h || best == h - 1) return c2 / 2.;
    return parabola_vertex(curve[best - 1 + h], curve[best + h], curve[best + 1 + h], c2);
}

// Least-squares line centre(k) = intercept + slope k over the accepted rows k.  The sums of k and
// k^2 are 32-bit ints in the reference and wrap on tall frames; unsigned arithmetic reproduces
// the wrap without overflow.
struct AxisLineFit {
    int sum_k = 0, sum_kk = 0, n = 0;
    double sum_c = 0, sum_kc = 0;
    void add(int k, double c) {
        sum_k += k;
        sum_kk = (int)((unsigned)sum_kk + (unsigned)k * (unsigned)k);
        sum_c += c;
        sum_kc += k * c;
        n++;
    }
    // false when fewer than min_rows rows were accepted (the caller then takes the overall centre)
    bool solve(int min_rows, double* intercept, double* slope) const {
        const int den = (int)((unsigned)n * (unsigned)sum_kk - (unsigned)sum_k * (unsigned)sum_k);
        *intercept = (sum_kk * sum_c - sum_k * sum_kc) / den;
        *slope = (sum_c - n * *intercept) / sum_k;
        return n >= min_rows;
    }
};

}  // namespace rv

using namespace rv;

extern "C" int RvGetAxis(const unsigned short* sample0, const unsigned short* sample1, const unsigned short* flat,
                         int ixdim, int iydim, int iAxisOffset, double* pCenter, double* pGrad, double* pOverall) {
    if (!sample0 || !sample1 || !flat || !pCenter || !pGrad || ixdim < 2 || iydim < 1 || iAxisOffset < 0 ||
        iAxisOffset >= ixdim) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvGetAxis: invalid argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    const long long n = (long long)ixdim * iydim;
    const int tail = 2 * ixdim + 16;   // zero tail for the offset-CT indices
    const int ixdimh = ixdim / 5 > 100 ? ixdim / 5 : 100;      // source/gazoDoc.cpp:4417
    const int istep = iydim < 40 ? 1 : iydim / 40;
    const int icdim = (int)ceil(iydim / (double)istep);
    void *d_in = nullptr, *d_lg = nullptr, *d_ssd = nullptr, *d_nd = nullptr;
    const size_t in_b = 3 * (size_t)n * 2, lg_b = 2 * ((size_t)n + tail) * 4;
    const size_t ssd_b = (size_t)icdim * 2 * ixdimh * 8, nd_b = (size_t)icdim * 2 * ixdimh * 4;
    int rc = 0;
    if (cudaMalloc(&d_in, in_b) != cudaSuccess || cudaMalloc(&d_lg, lg_b) != cudaSuccess ||
        cudaMalloc(&d_ssd, ssd_b) != cudaSuccess || cudaMalloc(&d_nd, nd_b) != cudaSuccess) {
        set_error(RV_ERR_DEVICE_OOM, "RvGetAxis: device buffers");
        rc = RV_ERR_DEVICE_OOM;
    }
    std::vector<long long> ssd;
    std::vector<int> nd;
    if (!rc) {
        uint16_t* din = static_cast<uint16_t*>(d_in);
        int* S0 = static_cast<int*>(d_lg);
        int* S1 = S0 + n + tail;
        bool ok = cuda_ok(cudaMemcpy(din, sample0, n * 2, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "frame 0") &&
                  cuda_ok(cudaMemcpy(din + n, sample1, n * 2, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "frame 1") &&
                  cuda_ok(cudaMemcpy(din + 2 * n, flat, n * 2, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "flat") &&
                  cuda_ok(cudaMemset(d_lg, 0, lg_b), RV_ERR_MEMSET, "log frames");
        if (ok) {
            k_axis_log<<<1024, 256>>>(din, din + n, din + 2 * n, S0, S1, n);
            dim3 g((2 * ixdimh + 127) / 128, icdim);
            k_axis_ssd<<<g, 128>>>(S0, S1, ixdim, istep, ixdimh, iAxisOffset, static_cast<long long*>(d_ssd),
                                   static_cast<int*>(d_nd));
            ssd.resize((size_t)icdim * 2 * ixdimh);
            nd.resize(ssd.size());
            ok = cuda_ok(cudaGetLastError(), RV_ERR_LAUNCH, "axis kernels") &&
                 cuda_ok(cudaMemcpy(ssd.data(), d_ssd, ssd_b, cudaMemcpyDeviceToHost), RV_ERR_COPY_D2H, "ssd") &&
                 cuda_ok(cudaMemcpy(nd.data(), d_nd, nd_b, cudaMemcpyDeviceToHost), RV_ERR_COPY_D2H, "ssd counts");
        }
        if (!ok) rc = RvGetLastError();
    }
    if (d_in) cudaFree(d_in);
    if (d_lg) cudaFree(d_lg);
    if (d_ssd) cudaFree(d_ssd);
    if (d_nd) cudaFree(d_nd);
    if (rc) return rc;
    // ---- host bookkeeping in the reference's arithmetic (source/gazoDoc.cpp:4443-4586) ----------
    // one SSD curve per sampled row, and the curve of all rows' sums
    const int nshift = 2 * ixdimh;
    std::vector<double> row_curve(nshift), total_sum(nshift, 0.0), center(icdim);
    std::vector<long long> total_cnt(nshift, 0);
    std::vector<unsigned char> row_valid(nshift), total_valid(nshift);
    for (int k = 0; k < iydim; k += istep) {
        const int icidx = k / istep;
        for (int idx = 0; idx < nshift; idx++) {
            const long long s = ssd[(size_t)icidx * nshift + idx];
            const int cnt = nd[(size_t)icidx * nshift + idx];
            total_sum[idx] += (double)s;
            total_cnt[idx] += cnt;
            row_valid[idx] = cnt != 0;
            row_curve[idx] = cnt ? (double)s / cnt : (double)s;
        }
        const int best = argmin_shift<float>(row_curve, row_valid, ixdimh);
        center[icidx] = refined_centre(row_curve, ixdimh, best, iAxisOffset, ixdim) - 0.5;   // HALFPIXEL_OFFSET
    }
    for (int idx = 0; idx < nshift; idx++) {
        total_valid[idx] = total_cnt[idx] != 0;
        if (total_valid[idx]) total_sum[idx] /= (double)total_cnt[idx];
    }
    const int best_total = argmin_shift<double>(total_sum, total_valid, ixdimh);
    const double overall = refined_centre(total_sum, ixdimh, best_total, iAxisOffset, ixdim) - 0.5;
    // a line through the rows whose centre lies within 3 px of the overall one (:4558-4586)
    AxisLineFit fit;
    for (int k = 0; k < iydim; k += istep) {
        const double c = center[k / istep];
        if (!(fabs(overall - c) > 3)) fit.add(k, c);
    }
    double intercept, slope;
    const bool use_line = fit.solve(iydim / istep / 2, &intercept, &slope);
    if (use_line && !(intercept < 0)) {
        *pCenter = intercept;
        *pGrad = slope;
    } else {
        *pCenter = overall;
        *pGrad = 0;
    }
    if (pOverall) *pOverall = overall;
    return 0;
}

extern "C" int RvCentreSweep(const short* sino, int nviews, int ixdim, int iInterpolation, const float* fdeg,
                             float fTiltAngle, const float* fFilter, const double* centres, int ncent, double* scores,
                             double* best_centre) {
    if (!sino || !fdeg || !fFilter || !centres || !scores || nviews < 1 || ixdim < 4 || ncent < 1) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvCentreSweep: invalid argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    const Dims d = make_dims(ixdim, iInterpolation);
    if (d.ndimp > kMaxNdimp || d.ixdimp > kMaxIxdimp) {
        set_error(RV_ERR_UNSUPPORTED, "RvCentreSweep: ixdim*zoom beyond 16384");
        return RV_ERR_UNSUPPORTED;
    }
    const int fmt = ref_table_fmt();
    const long long ts = ref_table_stride(d.ixdimp, fmt);
    const size_t npix = (size_t)d.ixdimp * d.ixdimp;
    // trial centres in batches whose tables fit a budget (RV_TABLE_BUDGET_MB, default 32768)
    size_t budget_mb = 32768;
    if (const char* e = getenv("RV_TABLE_BUDGET_MB")) budget_mb = (size_t)atoll(e);
    const size_t per_centre = (size_t)nviews * ts * 4;
    int batch = (int)((budget_mb << 20) / (per_centre ? per_centre : 1));
    if (batch < 1) batch = 1;
    if (batch > ncent) batch = ncent;
    std::vector<float2> tw;
    fft_twiddles(d.ndimp, tw);
    constexpr int kTvBlocks = 256;
    void *d_rows = nullptr, *d_filt = nullptr, *d_tw = nullptr, *d_jobs = nullptr, *d_geom = nullptr,
         *d_tab = nullptr, *d_out = nullptr, *d_part = nullptr;
    int rc = 0;
    if (cudaMalloc(&d_rows, (size_t)nviews * ixdim * 2) != cudaSuccess ||
        cudaMalloc(&d_filt, (size_t)d.ndim * 4) != cudaSuccess || cudaMalloc(&d_tw, tw.size() * 8) != cudaSuccess ||
        cudaMalloc(&d_jobs, (size_t)batch * nviews * sizeof(RowJob)) != cudaSuccess ||
        cudaMalloc(&d_geom, (size_t)batch * nviews * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&d_tab, per_centre * batch) != cudaSuccess || cudaMalloc(&d_out, npix * 4 * batch) != cudaSuccess ||
        cudaMalloc(&d_part, (size_t)batch * kTvBlocks * 8) != cudaSuccess) {
        set_error(RV_ERR_DEVICE_OOM, "RvCentreSweep: device buffers");
        rc = RV_ERR_DEVICE_OOM;
    }
    if (!rc && !(cuda_ok(cudaMemcpy(d_rows, sino, (size_t)nviews * ixdim * 2, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "sinogram") &&
                 cuda_ok(cudaMemcpy(d_filt, fFilter, (size_t)d.ndim * 4, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "filter") &&
                 cuda_ok(cudaMemcpy(d_tw, tw.data(), tw.size() * 8, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "twiddles")))
        rc = RvGetLastError();
    std::vector<double> part((size_t)batch * kTvBlocks);
    for (int c0 = 0; !rc && c0 < ncent; c0 += batch) {
        const int nb = ncent - c0 < batch ? ncent - c0 : batch;
        std::vector<float4> geom((size_t)nb * nviews);
        std::vector<RowJob> jobs((size_t)nb * nviews);
        for (int b = 0; b < nb; b++)
            for (int v = 0; v < nviews; v++) {
                float fc, fs, fo;
                view_geometry(d, centres[c0 + b], fdeg[v], fTiltAngle, &fc, &fs, &fo);
                geom[(size_t)b * nviews + v] = make_float4(fc, fs, fo, ray_regime_tag(fc, fs));
                RowJob j{};
                j.src_row = v;
                j.dst = b * nviews + v;
                j.ic = (int)centres[c0 + b];
                jobs[(size_t)b * nviews + v] = j;
            }
        if (!cuda_ok(cudaMemcpy(d_geom, geom.data(), geom.size() * sizeof(float4), cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "geometry") ||
            !cuda_ok(cudaMemcpy(d_jobs, jobs.data(), jobs.size() * sizeof(RowJob), cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "jobs")) {
            rc = RvGetLastError();
            break;
        }
        {   // every trial centre's rows in one filter launch (per-row integer centre)
            FilterLaunch fl{};
            fl.src = d_rows;
            fl.raw = 0;
            fl.jobs = static_cast<const RowJob*>(d_jobs);
            fl.njobs = nb * nviews;
            fl.filt = static_cast<const float*>(d_filt);
            fl.tw = static_cast<const float2*>(d_tw);
            fl.table = static_cast<int*>(d_tab);
            fl.mode = RV_MODE_REF;
            fl.d = d;
            fl.ic_per_job = 1;
            fl.table_stride = ts;
            fl.table_fmt = fmt;
            if (!cuda_ok(launch_filter(fl, 0), RV_ERR_LAUNCH, "filter kernel")) { rc = RV_ERR_LAUNCH; break; }
        }
        {   // and every trial slice in one back-projection launch, each with its own geometry
            BackprojLaunch bl{};
            bl.table = static_cast<const int*>(d_tab);
            bl.geom = static_cast<const float4*>(d_geom);
            bl.geom_slice_stride = nviews;
            bl.nviews = nviews;
            bl.nslices = nb;
            bl.ixdimp = d.ixdimp;
            bl.table_stride = ts;
            bl.slice_table_stride = ts * nviews;
            bl.out = d_out;
            bl.out_slice_stride = (long long)npix;
            bl.mode = RV_MODE_REF;
            bl.table_fmt = fmt;
            if (!cuda_ok(launch_backproject(bl, 0), RV_ERR_LAUNCH, "back-projection kernel")) { rc = RV_ERR_LAUNCH; break; }
        }
        dim3 g(kTvBlocks, nb);
        k_tv_partial<<<g, 256>>>(static_cast<const int*>(d_out), d.ixdimp, static_cast<double*>(d_part));
        if (!cuda_ok(cudaGetLastError(), RV_ERR_LAUNCH, "score kernel") ||
            !cuda_ok(cudaMemcpy(part.data(), d_part, (size_t)nb * kTvBlocks * 8, cudaMemcpyDeviceToHost), RV_ERR_COPY_D2H, "scores")) {
            rc = RvGetLastError();
            break;
        }
        for (int b = 0; b < nb; b++) {
            double t = 0.0;
            for (int k = 0; k < kTvBlocks; k++) t += part[(size_t)b * kTvBlocks + k];
            scores[c0 + b] = t;
        }
    }
    if (!rc) {
        if (const unsigned ks = take_kernel_status(0)) {
            set_error(RV_ERR_KERNEL_STATUS, std::string("back-projection: ") + kernel_status_text(ks));
            rc = RV_ERR_KERNEL_STATUS;
        }
    }
    void* bufs[] = {d_rows, d_filt, d_tw, d_jobs, d_geom, d_tab, d_out, d_part};
    for (void* p : bufs)
        if (p) cudaFree(p);
    if (rc) return rc;
    if (best_centre) {
        int m = 0;
        for (int i = 1; i < ncent; i++)
            if (scores[i] < scores[m]) m = i;
        double c = centres[m];
        if (m > 0 && m < ncent - 1) {
            const double s0 = scores[m - 1], s1 = scores[m], s2 = scores[m + 1];
            const double den = s0 - 2 * s1 + s2;
            const double h0 = centres[m] - centres[m - 1], h1 = centres[m + 1] - centres[m];
            if (den > 0 && fabs(h0 - h1) < 1e-9) c = centres[m] + 0.5 * h0 * (s0 - s2) / den;
        }
        *best_centre = c;
    }
    return 0;
}
