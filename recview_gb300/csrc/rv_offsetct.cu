// Offset-CT sinogram stitching (360-degree scan, rotation axis near one edge of the frame).
//
// The reference does this on the host after normalisation, one row at a time, with a value
// carried along each row (the offset-CT tail of CGazoDoc::GenerateSinogram,
// source/gazoDoc.cpp:3535-3665).  Here the host turns each detector row's centre into a small
// plan of index ranges (OctRow) and the kernel evaluates every output sample independently:
//
//   p = k + shift                      output position of frame sample k
//   copy zone   -> own sample s1[k]
//   mirror zone -> (short)(A + (B - A) t) from the partner row s2 at m = mc - k (A, B = s2[m],
//                  s2[m+1], swapped for one of the four reference cases), crossfaded inside the
//                  overlap as (short)(r v + (1 - r) s1[k]), r = sign (k - base) / den
//   where the mirrored sample does not exist the reference repeats the last value it wrote
//   (zero before the first), i.e. the value at the nearest valid k in loop order.
//
// All double operations use explicit round-to-nearest intrinsics so nothing is contracted into
// an FMA; conversions truncate toward zero like the reference's (short) casts (every value is
// between two int16 samples, so none is out of range).
//
// HBM layout: d_sino [iLenSinogr * iMultiplex][ixlen] int16 (the reference's iSinogr order),
// d_out [nof * iMultiplex][width] int16.  One thread per output position, a block row per
// detector row, a loop over a chunk of views: reads 2 B of each row touched, writes 2 B per
// output sample; FP64 only in the mirror zone.
#include <cuda_runtime.h>
#include <limits.h>
#include <string.h>

#include <vector>

#include "rv_internal.h"

using namespace rv;

namespace {

struct OctRow {
    int shift;             // output position = k + shift
    int dir;               // +1: k increases along the reference's loop (axis right), -1: decreases
    int copy_lo, copy_hi;  // own samples copied (inclusive k range, empty when lo > hi)
    int loop_lo, loop_hi;  // mirrored part
    int val_lo, val_hi;    // k where the mirrored pair s2[m], s2[m+1] exists (within the loop)
    int mc;                // m = mc - k
    int swap;              // 1: A = s2[m+1], B = s2[m]
    int fade_lo, fade_hi;  // crossfade range
    int fade_base, fade_sign, fade_den;
    double t;              // interpolation weight
};

struct OctPlan {
    int B = 1, F = 0, T = 0, ixlen = 0, width = 0, nof = -1, M = 0;
    std::vector<int> partner;   // [nof]: partner frame of each SAMPLE view, -1 otherwise
    std::vector<OctRow> rows;   // [M]
};

constexpr int kOctThreads = 256;
constexpr int kOctViewsPerBlock = 8;

__device__ __forceinline__ short oct_trunc(double x) { return (short)__double2int_rz(x); }

__global__ void __launch_bounds__(kOctThreads) k_offset_ct(const short* __restrict__ sino, short* __restrict__ out,
                                                           const OctRow* __restrict__ rows,
                                                           const int* __restrict__ partner, int nof, int M,
                                                           int ixlen, int width) {
    const int j = blockIdx.y;
    const int p = blockIdx.x * kOctThreads + threadIdx.x;
    if (p >= width) return;
    const OctRow R = rows[j];
    // classify this output position once for all views of the chunk
    int kind = 0;           // 0 zero, 1 own sample, 2 mirrored (+ optional crossfade)
    int ks = 0, m = 0;
    bool fade = false;
    double r = 0.0, omr = 0.0;
    const int k = p - R.shift;
    if (k >= R.copy_lo && k <= R.copy_hi) {
        kind = 1;
        ks = k;
    } else if (k >= R.loop_lo && k <= R.loop_hi && R.val_lo <= R.val_hi) {
        int ke = k;
        bool zero = false;
        if (R.dir > 0) {
            if (k < R.val_lo) zero = true;
            else if (k > R.val_hi) ke = R.val_hi;
        } else {
            if (k > R.val_hi) zero = true;
            else if (k < R.val_lo) ke = R.val_lo;
        }
        if (!zero) {
            kind = 2;
            ks = ke;
            m = R.mc - ke;
            if (ke >= R.fade_lo && ke <= R.fade_hi) {
                fade = true;
                r = __ddiv_rn((double)(R.fade_sign * (ke - R.fade_base)), (double)R.fade_den);
                omr = __dsub_rn(1.0, r);
            }
        }
    }
    const int i1 = min(nof, (int)(blockIdx.z + 1) * kOctViewsPerBlock);
    for (int i = blockIdx.z * kOctViewsPerBlock; i < i1; i++) {
        const int q = partner[i];
        short v = 0;
        if (q >= 0 && kind) {
            const short* s1 = sino + ((long long)i * M + j) * ixlen;
            if (kind == 1) {
                v = __ldg(s1 + ks);
            } else {
                const short* s2 = sino + ((long long)q * M + j) * ixlen;
                int a = __ldg(s2 + m), b = __ldg(s2 + m + 1);
                if (R.swap) { const int x = a; a = b; b = x; }
                v = oct_trunc(__dadd_rn((double)a, __dmul_rn((double)(b - a), R.t)));
                if (fade)
                    v = oct_trunc(__dadd_rn(__dmul_rn(r, (double)v), __dmul_rn(omr, (double)__ldg(s1 + ks))));
            }
        }
        out[((long long)i * M + j) * width + p] = v;
    }
}

bool range_in(int lo, int hi, int a, int b) { return lo > hi || (lo >= a && hi <= b); }

// Builds the plan; returns 0, 21051, 21052 or RV_ERR_BAD_ARGUMENT (with the error recorded).
int make_plan(const RvOffsetCtDesc* d, OctPlan& P, bool rows_too) {
    if (!d || !d->bInc || !d->fdeg || d->iRawSinoXdim < 2 || d->iXdim < 2 || d->iLenSinogr < 2 ||
        d->iMultiplex < 1 || d->iTrimWidth < 0) {
        set_error(RV_ERR_BAD_ARGUMENT, "offset-CT: invalid description");
        return RV_ERR_BAD_ARGUMENT;
    }
    P.B = (d->iInterpolation == 0) ? 4 : ((d->iInterpolation == 1) ? 2 : 1);    // source/gazoDoc.cpp:2987
    P.F = d->iRawSinoXdim;
    P.T = d->iTrimWidth;
    P.ixlen = P.F / P.B;                                                       // :3002-3004 (offset CT: no trim)
    P.width = d->iXdim / P.B;                                                  // :3001
    P.M = d->iMultiplex;
    // GetSinogramYdim(TRUE), source/gazoDoc.cpp:2967-2978: the first frame beyond 180 degrees
    P.nof = -1;
    for (int i = 0; i + 1 < d->iLenSinogr; i++)
        if (d->fdeg[i] > 180.) { P.nof = i; break; }
    if (P.nof < 0) {
        set_error(21051, "offset-CT: no frame beyond 180 degrees");
        return 21051;
    }
    if (P.ixlen < 2 || P.width < 1) {
        set_error(RV_ERR_BAD_ARGUMENT, "offset-CT: frame narrower than two samples after binning");
        return RV_ERR_BAD_ARGUMENT;
    }
    if (P.M > 65535 || (P.nof + kOctViewsPerBlock - 1) / kOctViewsPerBlock > 65535) {
        set_error(RV_ERR_UNSUPPORTED, "offset-CT: more than 65535 detector rows or 524280 views");
        return RV_ERR_UNSUPPORTED;
    }
    if (!rows_too) return 0;
    // partner frames (source/gazoDoc.cpp:3566-3572): the search index only moves forward
    P.partner.assign(P.nof, -1);
    int q = P.nof;
    for (int i = 0; i < P.nof; i++) {
        if (!(d->bInc[i] & RV_BINC_SAMPLE)) continue;
        const double th = d->fdeg[i];
        while ((d->fdeg[q] - th < 180) || !(d->bInc[q] & RV_BINC_SAMPLE)) {
            if (++q >= d->iLenSinogr - 1) {
                set_error(21052, "offset-CT: a view has no partner frame 180 degrees on");
                return 21052;
            }
        }
        P.partner[i] = q;
    }
    // per detector row j: the reference's branch, centre split and index ranges
    P.rows.resize(P.M);
    const int B = P.B, F = P.F, T = P.T, ixlen = P.ixlen;
    const double cen = d->center + 0.5;   // HALFPIXEL_OFFSET (source/gazoDoc.cpp:3563)
    for (int j = 0; j < P.M; j++) {
        OctRow R{};
        int ic, g;
        double dc;
        if (cen > F / 2.) {
            const double fc = (cen + d->deltaCent * j * B + T) / B;     // :3578-3580
            ic = (int)fc;
            dc = fc - ic;
            g = F / B - 1 - ic;                                        // :3582
            R.dir = 1;
            R.shift = -(T / B);
            R.copy_lo = T / B;
            R.copy_hi = ic - g;
            R.loop_lo = ic - g + 1;
            R.loop_hi = (2 * F - T) / B - 1;                            // k < (iNativeXdim - iTrim)/iBinning
            if (dc < 0.5) {                                            // :3587-3601
                R.mc = 2 * ic; R.swap = 1; R.t = 1 - 2 * dc;
                R.val_lo = 2 * ic - (ixlen - 2); R.val_hi = 2 * ic;
            } else {                                                   // :3604-3618 (m shifted by one)
                R.mc = 2 * ic - 1; R.swap = 0; R.t = 2 - 2 * dc;
                R.val_lo = 2 * ic - 1 - (ixlen - 2); R.val_hi = 2 * ic - 1;
            }
            R.fade_lo = ic - g + 1; R.fade_hi = ic + g;
            R.fade_base = ic - g; R.fade_sign = 1;
        } else {
            const double fc = (cen + d->deltaCent * j * B) / B;         // :3621-3623
            ic = (int)(fc + 0.5);
            dc = fc - (int)fc;
            g = ic;
            R.dir = -1;
            R.shift = (F - T) / B;
            R.copy_lo = ic + g;
            R.copy_hi = (F - 1 - T) / B;
            R.loop_hi = ic + g - 1;
            R.loop_lo = (dc < 0.5) ? 2 * ic + 1 - F / B : 2 * ic - F / B;
            R.swap = 0;
            if (dc < 0.5) {                                            // :3629-3643
                R.mc = 2 * ic; R.t = 2 * dc;
            } else {                                                   // :3645-3659
                R.mc = 2 * ic - 1; R.t = 2 * dc - 1;
            }
            R.val_lo = R.mc - (ixlen - 2); R.val_hi = R.mc;
            R.fade_lo = ic - g; R.fade_hi = ic + g - 1;
            R.fade_base = ic + g; R.fade_sign = -1;
        }
        R.fade_den = g * 2 + 1;
        R.val_lo = R.val_lo > R.loop_lo ? R.val_lo : R.loop_lo;
        R.val_hi = R.val_hi < R.loop_hi ? R.val_hi : R.loop_hi;
        // every sample the reference would touch must lie inside its row
        const int flo = R.fade_lo > R.val_lo ? R.fade_lo : R.val_lo;
        const int fhi = R.fade_hi < R.val_hi ? R.fade_hi : R.val_hi;
        const bool ok = range_in(R.copy_lo, R.copy_hi, 0, ixlen - 1) &&
                        range_in(R.copy_lo + R.shift, R.copy_hi + R.shift, 0, P.width - 1) &&
                        range_in(R.loop_lo + R.shift, R.loop_hi + R.shift, 0, P.width - 1) &&
                        range_in(flo, fhi, 0, ixlen - 1) && R.fade_den > 0;
        if (!ok) {
            set_error(RV_ERR_BAD_ARGUMENT,
                      "offset-CT: a row would be read or written outside its bounds (centre, trim or width "
                      "inconsistent)");
            return RV_ERR_BAD_ARGUMENT;
        }
        P.rows[j] = R;
    }
    return 0;
}

int stitch_device(const OctPlan& P, const short* d_sino, short* d_out, cudaStream_t s) {
    if (P.nof == 0) return 0;
    void* d_meta = nullptr;
    const size_t rows_b = sizeof(OctRow) * P.rows.size(), part_b = sizeof(int) * P.partner.size();
    if (!cuda_ok(cudaMallocAsync(&d_meta, rows_b + part_b, s), RV_ERR_DEVICE_OOM, "offset-CT: plan buffer"))
        return RV_ERR_DEVICE_OOM;
    std::vector<unsigned char> h(rows_b + part_b);
    memcpy(h.data(), P.rows.data(), rows_b);
    memcpy(h.data() + rows_b, P.partner.data(), part_b);
    int rc = 0;
    // pageable source: the copy is staged by the driver before the call returns
    if (!cuda_ok(cudaMemcpyAsync(d_meta, h.data(), h.size(), cudaMemcpyHostToDevice, s), RV_ERR_COPY_H2D,
                 "offset-CT: plan upload")) {
        rc = RV_ERR_COPY_H2D;
    } else {
        const dim3 grid((P.width + kOctThreads - 1) / kOctThreads, P.M,
                        (P.nof + kOctViewsPerBlock - 1) / kOctViewsPerBlock);
        k_offset_ct<<<grid, kOctThreads, 0, s>>>(d_sino, d_out, (const OctRow*)d_meta,
                                                  (const int*)((unsigned char*)d_meta + rows_b), P.nof, P.M,
                                                  P.ixlen, P.width);
        if (!cuda_ok(cudaGetLastError(), RV_ERR_LAUNCH, "offset-CT: kernel launch")) rc = RV_ERR_LAUNCH;
    }
    cudaFreeAsync(d_meta, s);
    return rc;
}

}  // namespace

extern "C" int RvOffsetCtDims(const RvOffsetCtDesc* desc, int* nof, int* ixlen, int* width) {
    OctPlan P;
    const int rc = make_plan(desc, P, false);
    if (rc) return rc;
    if (nof) *nof = P.nof;
    if (ixlen) *ixlen = P.ixlen;
    if (width) *width = P.width;
    return 0;
}

extern "C" double RvOffsetCtReconCenter(const RvOffsetCtDesc* desc, double layer_center) {
    // CGazoDoc::DeconvBackProj: a centre in the left half moves by the frame width
    // (source/gazoDoc.cpp:3832-3836), then ri->center = (c + HALFPIXEL_OFFSET) / binning (:3935)
    if (!desc) return layer_center;
    const int B = (desc->iInterpolation == 0) ? 4 : ((desc->iInterpolation == 1) ? 2 : 1);
    double c = layer_center;
    if (c <= desc->iRawSinoXdim / 2.) c = desc->iRawSinoXdim + c;
    return (c + 0.5) / B;
}

extern "C" int RvOffsetCtStitchDevice(const RvOffsetCtDesc* desc, const short* d_sino, short* d_out, void* stream) {
    OctPlan P;
    int rc = make_plan(desc, P, true);
    if (rc) return rc;
    if (!d_sino || !d_out) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvOffsetCtStitchDevice: null buffer");
        return RV_ERR_BAD_ARGUMENT;
    }
    return stitch_device(P, d_sino, d_out, (cudaStream_t)stream);
}

extern "C" int RvOffsetCtStitchHost(const RvOffsetCtDesc* desc, short* const* iSinogr, short* const* ofSinogr) {
    OctPlan P;
    int rc = make_plan(desc, P, true);
    if (rc) return rc;
    if (!iSinogr || !ofSinogr) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvOffsetCtStitchHost: null row table");
        return RV_ERR_BAD_ARGUMENT;
    }
    const long long nin = (long long)desc->iLenSinogr * P.M, nout = (long long)P.nof * P.M;
    std::vector<short> hin((size_t)(nin * P.ixlen)), hout((size_t)(nout * P.width));
    for (long long r = 0; r < nin; r++) {
        if (!iSinogr[r]) {   // rows the reference never reads may be absent; they stay zero
            memset(hin.data() + r * P.ixlen, 0, sizeof(short) * P.ixlen);
            continue;
        }
        memcpy(hin.data() + r * P.ixlen, iSinogr[r], sizeof(short) * P.ixlen);
    }
    short *d_in = nullptr, *d_out = nullptr;
    if (!cuda_ok(cudaMalloc(&d_in, hin.size() * sizeof(short)), RV_ERR_DEVICE_OOM, "offset-CT: input") ||
        !cuda_ok(cudaMalloc(&d_out, hout.size() * sizeof(short) + 2), RV_ERR_DEVICE_OOM, "offset-CT: output")) {
        if (d_in) cudaFree(d_in);
        return RV_ERR_DEVICE_OOM;
    }
    rc = 0;
    if (!cuda_ok(cudaMemcpy(d_in, hin.data(), hin.size() * sizeof(short), cudaMemcpyHostToDevice), RV_ERR_COPY_H2D,
                 "offset-CT: input copy"))
        rc = RV_ERR_COPY_H2D;
    if (!rc) rc = stitch_device(P, d_in, d_out, 0);
    if (!rc && !cuda_ok(cudaMemcpy(hout.data(), d_out, hout.size() * sizeof(short), cudaMemcpyDeviceToHost),
                        RV_ERR_COPY_D2H, "offset-CT: output copy"))
        rc = RV_ERR_COPY_D2H;
    cudaFree(d_in);
    cudaFree(d_out);
    if (rc) return rc;
    for (long long r = 0; r < nout; r++)
        if (ofSinogr[r]) memcpy(ofSinogr[r], hout.data() + r * P.width, sizeof(short) * P.width);
    return 0;
}
