/*
 * rv_oracle.c -- CPU restatement of RecView's convolution back-projection path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed CPU baseline.
 * Nothing in the product links this file.  Build with -ffp-contract=off (gcc otherwise fuses
 * a*b+c into an FMA on aarch64 and changes the bits the reference produces).
 *
 * Every function follows one piece of the reference (file:line in its comment) in the same
 * floating-point operation order.  Parity pins: oracle/_ref (the reference sources compiled
 * unmodified by oracle/build_ref.sh) and the golden vectors in tests/golden.
 */
#include "rv_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* source/constants.h:3-5 (double literals of the reference, kept to the digit) */
#define RVO_DEG_TO_RAD 0.0174532925199
#define RVO_PI 3.1415926535897
#define RVO_PI2 6.283185307178

/* ---------------------------------------------------------------- R3: sizes / geometry ---- */
void rvo_dims(int ixdim, int iInterpolation, RvDims* d) {
    /* source/general.cpp:2021-2035 */
    d->ixdim = ixdim;
    d->iZooming = (iInterpolation > RV_ZOOMING_NONE) ? (iInterpolation - RV_ZOOMING_NONE) : 0;
    d->iIntpDim = (int)pow(2.0, d->iZooming);
    d->ndimp = (int)(log((double)ixdim) / 0.69314718055994530941723212145818) + 1 + d->iZooming;
    d->ndim = (int)pow(2.0, d->ndimp);
    d->ixdimp = ixdim * d->iIntpDim;
    d->ixdimh = d->ixdimp / 2;
    d->ihoffset = d->ndim / 2 - 1 - d->ixdimh;
}

float rvo_fcenter(const RvDims* d, double center) {
    /* source/general.cpp:2036-2037: float arithmetic, (int)center truncates the double. */
    const int ic = (int)center;
    if (d->iIntpDim == 1) {
        float a = (float)d->ixdimh + (float)center;
        a = a - (float)ic;
        return a * (float)RV_DBPT_GINTP;
    }
    float fr = (float)center - (float)ic;
    fr = fr * (float)d->iIntpDim;
    fr = (float)d->ixdimh + fr;
    return fr * (float)RV_DBPT_GINTP;
}

void rvo_view_geometry(const RvDims* d, double center, float fdeg, float tilt, float* fcos,
                       float* fsin, float* foffset) {
    /* source/general.cpp:2139-2142: th from a float sum, cos/sin in double, float results. */
    const float deg = fdeg + tilt;
    const double th = (double)deg * RVO_DEG_TO_RAD;
    const float c = (float)(cos(th) * RV_DBPT_GINTP);
    const float s = (float)(-sin(th) * RV_DBPT_GINTP);
    const float sum = c + s;
    const float prod = (float)d->ixdimh * sum;
    *fcos = c;
    *fsin = s;
    *foffset = rvo_fcenter(d, center) - prod;
}

/* ---------------------------------------------------------------- R4: filter table ------- */
int rvo_set_filter(int kind, double cutoff, double order_d, int ndim, float* F) {
    /* source/gazoDoc.cpp:3762-3811 */
    if (!F || ndim <= 0) return RV_ERR_BAD_ARGUMENT;
    const int ndimh = (int)(ndim * cutoff);
    const float order = (float)order_d;
    const float revndim = 1.f / (float)ndim;
    int i;
    switch (kind) {
    case RV_FILT_HAN:
        for (i = 0; i < ndimh; i++) {
            const float frac = (float)i / (float)ndimh;
            const float w = (float)(1 + cos(RVO_PI * (double)frac));
            F[i] = ((0.5f * revndim) * (float)i) * w;
        }
        for (i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    case RV_FILT_HAM:
        for (i = 0; i < ndimh; i++) {
            const float frac = (float)i / (float)ndimh;
            const float w = (float)(0.54 + 0.46 * cos(RVO_PI * (double)frac));
            F[i] = (revndim * (float)i) * w;
        }
        for (i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    case RV_FILT_RAMP:
        for (i = 0; i < ndimh; i++) F[i] = revndim * (float)i;
        for (i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    case RV_FILT_PARZN:
        for (i = 0; i < ndimh / 2; i++) {
            const float frac = (float)i / (float)ndimh;
            float t = 6.0f * frac;
            t = t * frac;
            t = t * (1.0f - frac);
            F[i] = (revndim * (float)i) * (1.0f - t);
        }
        for (i = ndimh / 2; i < ndimh; i++) {
            const float frac = (float)i / (float)ndimh;
            const float om = 1.0f - frac;
            float v = (revndim * (float)i) * 2.0f;
            v = v * om;
            v = v * om;
            F[i] = v * om;
        }
        for (i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    case RV_FILT_BUTER:
        /* the reference calls pow(float, float) and sqrt(float): the C++ float overloads */
        for (i = 0; i < ndim; i++) {
            const float frac = (float)i / (float)ndimh;
            const float den = sqrtf(1.0f + powf(frac, order));
            F[i] = (revndim * (float)i) / den;
        }
        break;
    case RV_FILT_SHEPP:
        /* Project-defined: Shepp-Logan window sinc(pi f / 2) in the same one-sided layout. */
        for (i = 0; i < ndimh; i++) {
            const float frac = (float)i / (float)ndimh;
            const double x = RVO_PI * (double)frac * 0.5;
            const float w = (i == 0) ? 1.0f : (float)(sin(x) / x);
            F[i] = (revndim * (float)i) * w;
        }
        for (i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    default:
        for (i = 0; i < ndim; i++) F[i] = 1;
        break;
    }
    return 0;
}

/* ---------------------------------------------------------------- R6: FFT ---------------- */
void rvo_fft_twiddles(int np, float* wr, float* wi) {
    /* source/cfft.cpp:374-410 with min0 < 0: p0 = -(float)2pi, a = p0 * (i/n) in float, then
     * the float overloads cos(float)/sin(float).  Their value is taken correctly rounded (the
     * double result rounded to float), independent of the platform's cosf/sinf; the reference
     * build pins the same values (oracle/ref_wrap/libm_pin.cpp). */
    const int n = 1 << np;
    float p0 = (float)RVO_PI2;
    p0 = p0 * -1.0f;
    for (int i = 0; i < n / 2; i++) {
        const float a = p0 * ((float)i / (float)n);
        wr[i] = (float)cos((double)a);
        wi[i] = (float)sin((double)a);
    }
}

/* One radix-2 Stockham pass (the inner stages of source/cfft.cpp:224-244 and :300-336):
 *   y[2*m*al + q]      = x[m*al + q] + x[m*al + q + n/2] * w[q*bt]
 *   y[2*m*al + q + al] = x[m*al + q] - x[m*al + q + n/2] * w[q*bt]
 * with the complex product evaluated as (xr*wr - xi*wi, xr*wi + xi*wr), each op rounded. */
static void rvo_pass(int n, int al, const float* wr, const float* wi, const float* xr,
                     const float* xi, float* yr, float* yi) {
    const int half = n / 2, bt = half / al;
    for (int m = 0; m < bt; m++) {
        for (int q = 0; q < al; q++) {
            const int a = m * al + q, b = a + half, t = q * bt, o = 2 * m * al + q;
            const float p1 = xr[b] * wr[t], p2 = xi[b] * wi[t];
            const float p3 = xr[b] * wi[t], p4 = xi[b] * wr[t];
            const float sr = p1 - p2, si = p3 + p4;
            yr[o] = xr[a] + sr;
            yi[o] = xi[a] + si;
            yr[o + al] = xr[a] - sr;
            yi[o + al] = xi[a] - si;
        }
    }
}

void rvo_fft_forward(int np, const float* wr, const float* wi, float* re, float* im,
                     float* work) {
    const int n = 1 << np, half = n / 2;
    float *ar = work, *ai = work + n, *br = work + 2 * n, *bi = work + 3 * n;
    /* first pass reads the input back to front (source/cfft.cpp:197-209) */
    for (int j = 0; j < half; j++) {
        const int u = half - 1 - j, v = n - 1 - j;
        ar[2 * j] = re[u] + re[v];
        ai[2 * j] = im[u] + im[v];
        ar[2 * j + 1] = re[u] - re[v];
        ai[2 * j + 1] = im[u] - im[v];
    }
    int al = 2;
    for (int l = 1; l < np - 1; l++) {
        rvo_pass(n, al, wr, wi, ar, ai, br, bi);
        float* t;
        t = ar; ar = br; br = t;
        t = ai; ai = bi; bi = t;
        al *= 2;
    }
    /* last pass writes front to back reversed (source/cfft.cpp:246-265) */
    re[0] = ar[0] + ar[half];
    im[0] = ai[0] + ai[half];
    re[half] = ar[0] - ar[half];
    im[half] = ai[0] - ai[half];
    for (int k = 1; k < half; k++) {
        const float p1 = ar[half + k] * wr[k], p2 = ai[half + k] * wi[k];
        const float p3 = ar[half + k] * wi[k], p4 = ai[half + k] * wr[k];
        const float sr = p1 - p2, si = p3 + p4;
        re[n - k] = ar[k] + sr;
        im[n - k] = ai[k] + si;
        re[half - k] = ar[k] - sr;
        im[half - k] = ai[k] - si;
    }
}

void rvo_fft_inverse(int np, const float* wr, const float* wi, float* re, float* im,
                     float* work) {
    const int n = 1 << np, half = n / 2;
    float *ar = work, *ai = work + n, *br = work + 2 * n, *bi = work + 3 * n;
    /* source/cfft.cpp:283-295 */
    for (int j = 0; j < half; j++) {
        ar[2 * j] = re[j] + re[j + half];
        ai[2 * j] = im[j] + im[j + half];
        ar[2 * j + 1] = re[j] - re[j + half];
        ai[2 * j + 1] = im[j] - im[j + half];
    }
    int al = 2;
    for (int l = 1; l < np - 1; l++) {
        rvo_pass(n, al, wr, wi, ar, ai, br, bi);
        float* t;
        t = ar; ar = br; br = t;
        t = ai; ai = bi; bi = t;
        al *= 2;
    }
    /* last pass with min < 0 swaps the two halves (source/cfft.cpp:355-368) */
    for (int k = 0; k < half; k++) {
        const float p1 = ar[half + k] * wr[k], p2 = ai[half + k] * wi[k];
        const float p3 = ar[half + k] * wi[k], p4 = ai[half + k] * wr[k];
        const float sr = p1 - p2, si = p3 + p4;
        br[k] = ar[k] - sr;
        bi[k] = ai[k] - si;
        br[k + half] = ar[k] + sr;
        bi[k + half] = ai[k] + si;
    }
    /* CFft::FFT1 epilogue (source/cfft.cpp:418-425): reverse and scale by 1/n (exact). */
    const float a = 1.f / (float)n;
    for (int i = 0; i < n; i++) {
        re[i] = br[n - 1 - i] * a;
        im[i] = bi[n - 1 - i] * a;
    }
}

/* ---------------------------------------------------------------- R5 / R7 --------------- */
void rvo_place_row(const RvDims* d, double center, const short* strip, float* re, float* im) {
    /* source/general.cpp:2105-2126 */
    const int ndim = d->ndim, z = d->iIntpDim, ixdim = d->ixdim, ic = (int)center;
    memset(re, 0, sizeof(float) * ndim);
    memset(im, 0, sizeof(float) * ndim);
    const int idx0 = (0 - ic) * z + (ndim / 2 - 1);
    const int idx1 = (ixdim - 1 - ic) * z + (ndim / 2 - 1) + 1;
    for (int m = 0; m < idx0; m++) re[m] = strip[0];
    for (int m = idx1; m < ndim; m++) re[m] = strip[ixdim - 1];
    for (int k = 0; k < ixdim; k++) {
        const int idx = (k - ic) * z + (ndim / 2 - 1);
        if (idx < 0) continue;
        if (idx >= ndim) break;
        re[idx] = strip[k];
        if (k == ixdim - 1) break;
        for (int j = 1; j < z; j++) {
            if (idx + j >= ndim) break;
            re[idx + j] = (float)(strip[k] * (z - j) / z + strip[k + 1] * j / z);
        }
    }
}

void rvo_filter_row(const RvDims* d, double center, const short* strip, const float* filt,
                    const float* wr, const float* wi, float* q, float* work) {
    const int ndim = d->ndim;
    float* re = work;
    float* im = work + ndim;
    float* scratch = work + 2 * ndim;
    rvo_place_row(d, center, strip, re, im);
    rvo_fft_forward(d->ndimp, wr, wi, re, im, scratch);
    for (int k = 0; k < ndim; k++) { /* CCmplx::operator*=(float), source/ccmplx.cpp:42-44 */
        re[k] = re[k] * filt[k];
        im[k] = im[k] * filt[k];
    }
    rvo_fft_inverse(d->ndimp, wr, wi, re, im, scratch);
    for (int j = 0; j < d->ixdimp; j++) q[j] = re[j + d->ihoffset];
}

void rvo_row_table(int ixdimp, const float* q, int* igp) {
    /* source/general.cpp:2130-2137 */
    for (int j = 0; j < ixdimp; j++) {
        const float p0 = q[j] * (float)RV_BACKPROJ_SCALE;
        float p1p0 = 0.0f;
        if (j != ixdimp - 1) {
            const float diff = q[j + 1] - q[j];
            p1p0 = (diff / (float)RV_DBPT_GINTP) * (float)RV_BACKPROJ_SCALE;
        }
        for (int k = 0; k < RV_DBPT_GINTP; k++) {
            const float step = p1p0 * (float)k;
            igp[j * RV_DBPT_GINTP + k] = (int)(p0 + step);
        }
    }
}

/* ---------------------------------------------------------------- R8 -------------------- */
void rvo_backproject_view(int ixdimp, float fcos, float fsin, float foffset, const int* igp,
                          int* ifp, int iy0, int iy1) {
    /* source/general.cpp:2147-2158 (scalar path, bUseSIMD == false) */
    const int ixdimpg = ixdimp * RV_DBPT_GINTP;
    for (int iy = iy0; iy < iy1; iy++) {
        int ifpidx = iy * ixdimp - 1;
        const float fyoff = (float)iy * fsin + foffset;
        for (int ix = 0; ix < ixdimp; ix++) {
            const float fx = (float)ix * fcos + fyoff;
            const int ix0 = (int)fx;
            ifpidx++;
            if (ix0 < 0) continue;
            if (ix0 >= ixdimpg) continue;
            ifp[ifpidx] += igp[ix0];
        }
    }
}

static int rvo_view_used(const RECONST_INFO* ri, int i, int* sidx_out) {
    /* source/general.cpp:2087-2102 (the `break` on sidx is reported as -1) */
    if (!(ri->bInc[i] & RV_BINC_SAMPLE)) return 0;
    const int sidx = i * ri->iMultiplex + ri->iOffset;
    if (sidx >= ri->maxSinogrLen) return -1;
    if (ri->dReconFlags & (RV_RQFLAGS_USEONLYEVENFRAMES | RV_RQFLAGS_USEONLYODDFRAMES)) {
        if (i & 1) {
            if (ri->dReconFlags & RV_RQFLAGS_USEONLYEVENFRAMES) return 0;
        } else {
            if (ri->dReconFlags & RV_RQFLAGS_USEONLYODDFRAMES) return 0;
        }
    }
    *sidx_out = sidx;
    return 1;
}

int rvo_reconstruct(RECONST_INFO* ri) {
    RvDims d;
    rvo_dims(ri->ixdim, ri->iInterpolation, &d);
    const int ixdimp = d.ixdimp, ndim = d.ndim;
    const double center = ri->center;
    float* work = (float*)malloc(sizeof(float) * (size_t)ndim * 7);
    float* wr = (float*)malloc(sizeof(float) * (size_t)ndim);
    float* q = (float*)malloc(sizeof(float) * (size_t)ixdimp);
    int* igp = (int*)malloc(sizeof(int) * (size_t)ixdimp * RV_DBPT_GINTP);
    if (!work || !wr || !q || !igp) {
        free(work); free(wr); free(q); free(igp);
        ri->iStatus = RECONST_INFO_ERROR;
        return RV_ERR_HOST_ALLOC;
    }
    float* wi = wr + ndim / 2;
    rvo_fft_twiddles(d.ndimp, wr, wi);
    /* source/general.cpp:2063-2066 */
    const int ibatch = ri->iStartSino, ncpu = ri->iStepSino;
    const int iy0 = (ixdimp * ibatch + ncpu - 1) / ncpu;
    const int iy1 = (ixdimp * (ibatch + 1) + ncpu - 1) / ncpu;
    for (int i = 0; i < ri->iLenSinogr - 1; i++) {
        int sidx = 0;
        const int u = rvo_view_used(ri, i, &sidx);
        if (u < 0) break;
        if (u == 0) continue;
        if (ri->iStartSino == 0) (*(ri->nSinogr))++;
        rvo_filter_row(&d, center, ri->iSinogr[sidx], ri->fFilter, wr, wi, q, work);
        rvo_row_table(ixdimp, q, igp);
        float fcos, fsin, foffset;
        rvo_view_geometry(&d, center, ri->fdeg[i], ri->fTiltAngle, &fcos, &fsin, &foffset);
        rvo_backproject_view(ixdimp, fcos, fsin, foffset, igp, ri->iReconst, iy0, iy1);
    }
    free(work); free(wr); free(q); free(igp);
    if (ri->iStatus != RECONST_INFO_ERROR) ri->iStatus = RECONST_INFO_IDLE;  /* :2181-2182 */
    return 0;
}

typedef struct { RECONST_INFO ri; int rc; } rvo_job;
static void* rvo_worker(void* arg) {
    rvo_job* j = (rvo_job*)arg;
    j->rc = rvo_reconstruct(&j->ri);
    return NULL;
}

int rvo_reconstruct_mt(RECONST_INFO* ri, int nthreads) {
    if (nthreads <= 1) {
        RECONST_INFO one = *ri;
        one.iStartSino = 0;
        one.iStepSino = 1;
        int rc = rvo_reconstruct(&one);
        ri->iStatus = one.iStatus;
        return rc;
    }
    rvo_job* jobs = (rvo_job*)calloc((size_t)nthreads, sizeof(rvo_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) { free(jobs); free(th); return RV_ERR_HOST_ALLOC; }
    for (int t = 0; t < nthreads; t++) {
        jobs[t].ri = *ri;
        jobs[t].ri.iStartSino = t;
        jobs[t].ri.iStepSino = nthreads;
        pthread_create(&th[t], NULL, rvo_worker, &jobs[t]);
    }
    int rc = 0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        if (jobs[t].rc) rc = jobs[t].rc;
    }
    free(jobs); free(th);
    return rc;
}

/* ---------------------------------------------------------------- R1 -------------------- */
int rvo_generate_sinogram(RECONST_INFO* ri) {
    /* source/general.cpp:2393-2520 */
    const int isino = ri->maxSinogrLen;
    const int ixlen = ri->ixdim;
    const int mult = ri->iMultiplex;
    const int ibin = (ri->iInterpolation == 0) ? 4 : ((ri->iInterpolation == 1) ? 2 : 1);
    short** rows = ri->iSinogr;
    const char* bInc = ri->bInc;
    const float* fexp = ri->fexp;
    const float* fdeg = ri->fdeg;
    const int pixmin = (ri->iFlag & RV_READTIF8bit) ? RV_SINOGRAM_PIXEL_MIN8bit
                                                    : RV_SINOGRAM_PIXEL_MIN16bit;
    double* dinc = (double*)malloc(sizeof(double) * (size_t)ixlen);
    if (!dinc) { ri->iStatus = RECONST_INFO_ERROR; return 1; }
    int i0 = -1, i1 = -1;
    for (int i = 0; i < isino - 1; i++) {
        if (bInc[i] & RV_BINC_NOUSE) continue;
        if (!(bInc[i] & RV_BINC_SAMPLE)) { i0 = i; break; }
    }
    for (int i = 0; i < isino - 1; i++) {
        if ((bInc[i] & RV_BINC_NOUSE) && !(bInc[i] & RV_BINC_SAMPLE)) continue;
        if (!(bInc[i] & RV_BINC_SAMPLE)) { i0 = i; i1 = -1; continue; }
        if (i1 < 0) {
            for (int j = i; j < isino - 1; j++) {
                if (bInc[j] & RV_BINC_SAMPLE) continue;
                i1 = j;
                break;
            }
            if (i1 < 0) {
                if (i0 >= 0) i1 = i0;
                else { ri->iStatus = RECONST_INFO_ERROR; break; }
            }
        }
        if (i0 < 0 || i1 < 0) { ri->iStatus = RECONST_INFO_ERROR; free(dinc); return 1; }
        if (i % ri->iStepSino != ri->iStartSino) continue;
        float t0 = fexp[i0];
        const float t1 = fexp[i1];
        const float ti = fexp[i];
        if (t0 == t1) t0 = 0;
        else t0 = (ti - t0) / (t1 - t0);
        const double cth = cos(fdeg[i] * RVO_DEG_TO_RAD);
        const double sth = sin(fdeg[i] * RVO_DEG_TO_RAD);
        int idrift = 0;
        if ((ri->drEnd > ri->drStart) && (ri->dReconFlags & RV_RQFLAGS_DRIFTPARAMS)) {
            if ((ri->drStart < i) && (i < ri->drEnd) && ri->drOmit) {
                for (int k = 0; k < mult; k++) memset(rows[mult * i + k], 0, sizeof(short) * ixlen);
                continue;
            }
            const double dd = ri->drX * cth - ri->drY * sth;
            if (i >= ri->drEnd) idrift = (int)dd;
            else if (i > ri->drStart)
                idrift = (int)(dd * (i - ri->drStart) / (ri->drEnd - ri->drStart));
        }
        if (bInc[i] & RV_BINC_SKIP) {
            for (int k = 0; k < mult; k++) memset(rows[mult * i + k], 0, sizeof(short) * ixlen);
            continue;
        }
        if ((ri->dReconFlags & RV_RQFLAGS_DRIFTLIST) && ri->piDrift) idrift -= ri->piDrift[i];
        for (int k = 0; k < mult; k++) {
            const unsigned short* dark = (const unsigned short*)rows[mult * (isino - 1) + k];
            const unsigned short* in0 = (const unsigned short*)rows[mult * i0 + k];
            const unsigned short* in1 = (const unsigned short*)rows[mult * i1 + k];
            for (int j = 0; j < ixlen; j++) {
                /* int*float, ushort+float and float-ushort all evaluate in float (:2475);
                 * only the result is widened to double. */
                const float prod = (float)((int)in1[j] - (int)in0[j]) * t0;
                const float s1 = (float)in0[j] + prod;
                dinc[j] = (double)(s1 - (float)dark[j]);
            }
            short* strip = rows[mult * i + k];
            const unsigned short* ustrip = (const unsigned short*)strip;
            if (ri->dReconFlags & RV_RQFLAGS_ZERNIKE) {
                for (int j = 0; j < ixlen; j++) {
                    if (dinc[j] <= 0) { strip[j] = 0; continue; }
                    const int s = (int)ustrip[j] - dark[j];
                    if (s < pixmin) { strip[j] = 0; continue; }
                    strip[j] = (short)(int)(dinc[j] * 1000 / s + 0.5);
                }
            } else {
                for (int j = 0; j < ixlen; j++) {
                    if (dinc[j] <= 0) { strip[j] = 0; continue; }
                    const int s = (int)ustrip[j] - dark[j];
                    if (s < pixmin) { strip[j] = 0; continue; }
                    strip[j] = (short)(int)(log(dinc[j] / s) * RV_LOG_SCALE + 0.5);
                }
            }
            const int sh = idrift / ibin;
            if (idrift > 0) {
                for (int j = ixlen - 1; j >= 0; j--) {
                    if (j + sh >= ixlen) continue;
                    strip[j + sh] = strip[j];
                }
                for (int j = sh - 1; j >= 0; j--) strip[j] = 0;
            } else if (idrift < 0) {
                for (int j = 0; j < ixlen; j++) {
                    if (j + sh < 0) continue;
                    strip[j + sh] = strip[j];
                }
                for (int j = ixlen + sh; j < ixlen; j++) strip[j] = 0;
            }
        }
    }
    free(dinc);
    if (ri->iStatus == RECONST_INFO_ERROR) return 1;
    ri->iStatus = RECONST_INFO_IDLE;  /* source/general.cpp:2529-2530 */
    return 0;
}

/* ---------------------------------------------------------------- R9 -------------------- */
void rvo_rescale(int* rec, int ixdimp, double center, int ipintp, int ibinning, int* pimin,
                 int* pimax) {
    /* source/gazoDoc.cpp:3993-3997,4007-4021 */
    const int n2 = ixdimp * ixdimp;
    int imax = 0, imin = INT_MAX;
    for (int i = 0; i < n2; i++) {
        imax = rec[i] > imax ? rec[i] : imax;
        imin = rec[i] < imin ? rec[i] : imin;
    }
    if (imin == imax) imax++;
    const double a = ipintp * center / ibinning;
    const double b = ixdimp - ipintp * center / ibinning;
    int irad2 = (a < b) ? (int)a : (int)b;
    irad2 *= irad2;
    const int ixdimh = ixdimp / 2;
    for (int i = 0; i < ixdimp; i++) {
        int i2 = i - ixdimh;
        i2 *= i2;
        for (int j = 0; j < ixdimp; j++) {
            const int j2 = j - ixdimh;
            const int idx = i * ixdimp + j;
            if (i2 + j2 * j2 > irad2) rec[idx] = 0;
            else {
                const float num = (float)(rec[idx] - imin) * (float)(USHRT_MAX - 1);
                rec[idx] = (int)(num / (float)(imax - imin));
            }
        }
    }
    if (pimin) *pimin = imin;
    if (pimax) *pimax = imax;
}

/* ---------------------------------------------------------------- FP64 oracle ----------- */
static void rvo_pass64(int n, int al, const double* wr, const double* wi, const double* xr,
                       const double* xi, double* yr, double* yi) {
    const int half = n / 2, bt = half / al;
    for (int m = 0; m < bt; m++)
        for (int q = 0; q < al; q++) {
            const int a = m * al + q, b = a + half, t = q * bt, o = 2 * m * al + q;
            const double sr = xr[b] * wr[t] - xi[b] * wi[t];
            const double si = xr[b] * wi[t] + xi[b] * wr[t];
            yr[o] = xr[a] + sr; yi[o] = xi[a] + si;
            yr[o + al] = xr[a] - sr; yi[o + al] = xi[a] - si;
        }
}

/* The same linear map as rvo_fft_forward/inverse (identical index conventions), in double
 * with exact twiddles: the transform the float routine approximates. */
static void rvo_fft64(int np, int inverse, const double* wr, const double* wi, double* re,
                      double* im, double* work) {
    const int n = 1 << np, half = n / 2;
    double *ar = work, *ai = work + n, *br = work + 2 * n, *bi = work + 3 * n;
    for (int j = 0; j < half; j++) {
        const int u = inverse ? j : half - 1 - j, v = inverse ? j + half : n - 1 - j;
        ar[2 * j] = re[u] + re[v]; ai[2 * j] = im[u] + im[v];
        ar[2 * j + 1] = re[u] - re[v]; ai[2 * j + 1] = im[u] - im[v];
    }
    int al = 2;
    for (int l = 1; l < np - 1; l++) {
        rvo_pass64(n, al, wr, wi, ar, ai, br, bi);
        double* t;
        t = ar; ar = br; br = t;
        t = ai; ai = bi; bi = t;
        al *= 2;
    }
    for (int k = 0; k < half; k++) {
        const double sr = ar[half + k] * wr[k] - ai[half + k] * wi[k];
        const double si = ar[half + k] * wi[k] + ai[half + k] * wr[k];
        if (!inverse) {
            const int ip = k ? n - k : 0, im_ = k ? half - k : half;
            br[ip] = ar[k] + sr; bi[ip] = ai[k] + si;
            br[im_] = ar[k] - sr; bi[im_] = ai[k] - si;
        } else {
            br[k] = ar[k] - sr; bi[k] = ai[k] - si;
            br[k + half] = ar[k] + sr; bi[k + half] = ai[k] + si;
        }
    }
    if (!inverse) {
        memcpy(re, br, sizeof(double) * n);
        memcpy(im, bi, sizeof(double) * n);
    } else {
        for (int i = 0; i < n; i++) {
            re[i] = br[n - 1 - i] / n;
            im[i] = bi[n - 1 - i] / n;
        }
    }
}

static int rvo_lin64_band(RECONST_INFO* ri, double* out, int iy0, int iy1) {
    RvDims d;
    rvo_dims(ri->ixdim, ri->iInterpolation, &d);
    const int ixdimp = d.ixdimp, ndim = d.ndim;
    const double center = ri->center;
    double* buf = (double*)malloc(sizeof(double) * (size_t)ndim * 8);
    float* fre = (float*)malloc(sizeof(float) * (size_t)ndim * 2);
    if (!buf || !fre) { free(buf); free(fre); return RV_ERR_HOST_ALLOC; }
    double *re = buf, *im = buf + ndim, *wr = buf + 2 * ndim, *wi = wr + ndim / 2;
    double* work = buf + 3 * ndim;
    for (int i = 0; i < ndim / 2; i++) {
        const double a = -2.0 * M_PI * (double)i / (double)ndim;
        wr[i] = cos(a);
        wi[i] = sin(a);
    }
    const double cen = (double)d.ixdimh + (center - (int)center) * d.iIntpDim;
    for (int i = 0; i < ri->iLenSinogr - 1; i++) {
        int sidx = 0;
        const int u = rvo_view_used(ri, i, &sidx);
        if (u < 0) break;
        if (u == 0) continue;
        rvo_place_row(&d, center, ri->iSinogr[sidx], fre, fre + ndim);
        for (int k = 0; k < ndim; k++) { re[k] = fre[k]; im[k] = 0; }
        rvo_fft64(d.ndimp, 0, wr, wi, re, im, work);
        for (int k = 0; k < ndim; k++) { re[k] *= ri->fFilter[k]; im[k] *= ri->fFilter[k]; }
        rvo_fft64(d.ndimp, 1, wr, wi, re, im, work);
        const double* qd = re + d.ihoffset;
        const double th = (double)(ri->fdeg[i] + ri->fTiltAngle) * (M_PI / 180.0);
        const double c = cos(th), s = -sin(th);
        const double off = cen - d.ixdimh * (c + s);
        for (int iy = iy0; iy < iy1; iy++) {
            for (int ix = 0; ix < ixdimp; ix++) {
                const double x = ix * c + iy * s + off;
                if (!(x >= 0.0) || !(x < ixdimp)) continue;
                int j = (int)x;
                if (j > ixdimp - 1) j = ixdimp - 1;
                const double f = x - j;
                const double q1 = (j + 1 < ixdimp) ? qd[j + 1] : qd[j];
                out[(size_t)iy * ixdimp + ix] += (qd[j] + (q1 - qd[j]) * f) * RV_BACKPROJ_SCALE;
            }
        }
    }
    free(buf); free(fre);
    return 0;
}

int rvo_reconstruct_lin64(RECONST_INFO* ri, double* out) {
    RvDims d;
    rvo_dims(ri->ixdim, ri->iInterpolation, &d);
    memset(out, 0, sizeof(double) * (size_t)d.ixdimp * d.ixdimp);
    return rvo_lin64_band(ri, out, 0, d.ixdimp);
}

typedef struct { RECONST_INFO* ri; double* out; int y0, y1, rc; } RvoLinJob;

static void* rvo_lin64_worker(void* arg) {
    RvoLinJob* j = (RvoLinJob*)arg;
    j->rc = rvo_lin64_band(j->ri, j->out, j->y0, j->y1);
    return NULL;
}

int rvo_reconstruct_lin64_mt(RECONST_INFO* ri, double* out, int nthreads) {
    /* the same sums, image rows split into bands (each band refilters every view) */
    RvDims d;
    rvo_dims(ri->ixdim, ri->iInterpolation, &d);
    memset(out, 0, sizeof(double) * (size_t)d.ixdimp * d.ixdimp);
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    RvoLinJob* jobs = (RvoLinJob*)calloc((size_t)nthreads, sizeof(RvoLinJob));
    if (!th || !jobs) { free(th); free(jobs); return RV_ERR_HOST_ALLOC; }
    for (int t = 0; t < nthreads; t++) {
        jobs[t].ri = ri;
        jobs[t].out = out;
        jobs[t].y0 = (int)((long long)d.ixdimp * t / nthreads);
        jobs[t].y1 = (int)((long long)d.ixdimp * (t + 1) / nthreads);
        pthread_create(&th[t], NULL, rvo_lin64_worker, &jobs[t]);
    }
    int rc = 0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        if (jobs[t].rc) rc = jobs[t].rc;
    }
    free(th); free(jobs);
    return rc;
}

/* ---------------------------------------------------------------- R11 ------------------- */
static short rvo_d2s_x64(double v) {
    /* (short)(double) as the reference's x64 build performs it: via a 32-bit conversion whose
     * out-of-range / NaN result is 0x80000000 (low 16 bits 0). */
    if (!(v > -2147483649.0 && v < 2147483648.0)) return 0;
    return (short)(int)v;
}

int rvo_get_axis(const unsigned short* s0in, const unsigned short* s1in, const unsigned short* inc0,
                 int ixdim, int iydim, int iAxisOffset, double* pCenter, double* pGrad, double* pOverall) {
    /* CGazoDoc::GetAxis after the frame reads (source/gazoDoc.cpp:4379-4626) */
    const int ixydim = ixdim * iydim;
    const int tail = 2 * ixdim + 16;
    int* S0 = (int*)calloc((size_t)ixydim + tail, sizeof(int));
    int* S1 = (int*)calloc((size_t)ixydim + tail, sizeof(int));
    const int ixdimh = ixdim / 5 > 100 ? ixdim / 5 : 100;
    const int istep = iydim < 40 ? 1 : iydim / 40;
    const int icdim = (int)ceil(iydim / (double)istep);
    double* sdiff = (double*)calloc((size_t)ixdimh * 2, sizeof(double));
    double* center = (double*)calloc((size_t)icdim, sizeof(double));
    double* sdifftotal = (double*)calloc((size_t)ixdimh * 2, sizeof(double));
    int* ndifftotal = (int*)calloc((size_t)ixdimh * 2, sizeof(int));
    if (!S0 || !S1 || !sdiff || !center || !sdifftotal || !ndifftotal) {
        free(S0); free(S1); free(sdiff); free(center); free(sdifftotal); free(ndifftotal);
        return RV_ERR_HOST_ALLOC;
    }
    for (int j = 0; j < ixydim; j++) {
        S0[j] = rvo_d2s_x64(log((double)inc0[j] / (double)s0in[j]) * RV_LOG_SCALE);
        S1[j] = rvo_d2s_x64(log((double)inc0[j] / (double)s1in[j]) * RV_LOG_SCALE);
    }
    for (int k = 0; k < iydim; k += istep) {
        const int icidx = k / istep;
        float minDiff = SHRT_MAX;
        int minIdx = 0;
        const int kix = k * ixdim;
        int ixCenter2;
        if (iAxisOffset) {
            const int scan = (iAxisOffset < ixdim / 2) ? iAxisOffset / 2 : (ixdim - iAxisOffset) / 2;
            for (int js = -ixdimh; js < ixdimh; js++) {
                const int idx = js + ixdimh, j = js + iAxisOffset;
                sdiff[idx] = 0;
                if (abs(js) > scan) continue;
                int nd = 0;
                for (int i = -scan; i <= scan; i++) {
                    const int d = S1[j - i + kix] - S0[j + i + kix];
                    sdiff[idx] += (double)d * d;
                    nd++;
                    sdifftotal[idx] += (double)d * d;
                    ndifftotal[idx]++;
                }
                if (nd == 0) continue;
                sdiff[idx] /= nd;
                if (sdiff[idx] < minDiff) { minDiff = (float)sdiff[idx]; minIdx = js; }
            }
            ixCenter2 = (minIdx + iAxisOffset) * 2;
        } else {
            for (int j = -ixdimh; j < ixdimh; j++) {
                const int idx = j + ixdimh;
                sdiff[idx] = 0;
                int nd = 0;
                const int ifrom = j >= 0 ? 0 : -j;
                const int ito = j >= 0 ? ixdim - j : ixdim;
                for (int i = ifrom; i < ito; i++) {
                    const int d = S1[ixdim - 1 - i + kix] - S0[i + j + kix];
                    sdiff[idx] += (double)d * d;
                    nd++;
                    sdifftotal[idx] += (double)d * d;
                    ndifftotal[idx]++;
                }
                if (nd == 0) continue;
                sdiff[idx] /= nd;
                if (sdiff[idx] < minDiff) { minDiff = (float)sdiff[idx]; minIdx = j; }
            }
            ixCenter2 = minIdx + ixdim - 1;
        }
        center[icidx] = 0;
        if ((minIdx == -ixdimh) || (minIdx == ixdimh - 1)) {
            center[icidx] = ixCenter2 / 2.;
        } else {
            const double dy1 = sdiff[minIdx + ixdimh];
            double dy0 = sdiff[minIdx - 1 + ixdimh];
            const double dy2 = sdiff[minIdx + 1 + ixdimh];
            if (dy2 == dy0) center[icidx] = (double)(ixCenter2 / 2.);
            else {
                dy0 = (dy1 - dy0) / (dy2 - dy0);
                center[icidx] = (4 * dy0 * ixCenter2 - (ixCenter2 * 2 - 1)) / (4 * dy0 - 2) / 2;
            }
        }
        center[icidx] -= 0.5;
    }
    double minDifftotal = SHRT_MAX;
    int idifftotal = 0;
    for (int j = -ixdimh; j < ixdimh; j++) {
        const int idx = j + ixdimh;
        if (ndifftotal[idx] == 0) continue;
        sdifftotal[idx] /= ndifftotal[idx];
        if (sdifftotal[idx] < minDifftotal) { minDifftotal = sdifftotal[idx]; idifftotal = j; }
    }
    const int ixCenter2total = iAxisOffset ? (idifftotal + iAxisOffset) * 2 : idifftotal + ixdim - 1;
    double dcentertotal = ixCenter2total / 2.;
    if ((idifftotal > -ixdimh) && (idifftotal < ixdimh - 1)) {
        const double dy1 = sdifftotal[idifftotal + ixdimh];
        double dy0 = sdifftotal[idifftotal - 1 + ixdimh];
        const double dy2 = sdifftotal[idifftotal + 1 + ixdimh];
        if (dy2 != dy0) {
            dy0 = (dy1 - dy0) / (dy2 - dy0);
            dcentertotal = (4 * dy0 * ixCenter2total - (ixCenter2total * 2 - 1)) / (4 * dy0 - 2) / 2;
        }
    }
    dcentertotal -= 0.5;
    const double cavg = dcentertotal, csig = 1;
    int isig1 = 0, isig2 = 0, nsig = 0;
    double sigc = 0, sigcx = 0;
    for (int k = 0; k < iydim; k += istep) {
        const int icidx = k / istep;
        if (fabs(cavg - center[icidx]) > csig * 3) continue;
        isig1 += k;
        isig2 = (int)((unsigned)isig2 + (unsigned)k * (unsigned)k);   /* int arithmetic wraps */
        sigc += center[icidx];
        sigcx += k * center[icidx];
        nsig++;
    }
    const int den = (int)((unsigned)nsig * (unsigned)isig2 - (unsigned)isig1 * (unsigned)isig1);
    double coeffb = (isig2 * sigc - isig1 * sigcx) / den;
    double coeffa = (sigc - nsig * coeffb) / isig1;
    if (nsig < iydim / istep / 2) { isig1 = 1; coeffb = dcentertotal; coeffa = 0; }
    else isig1 = 0;
    if ((coeffb < 0) || isig1) { *pCenter = dcentertotal; *pGrad = 0; }
    else { *pCenter = coeffb; *pGrad = coeffa; }
    if (pOverall) *pOverall = dcentertotal;
    free(S0); free(S1); free(sdiff); free(center); free(sdifftotal); free(ndifftotal);
    return 0;
}

static double rvo_box(const int* f, int ixdimp, int b, int X, int Y) {
    long long s = 0;
    for (int j = 0; j < b; j++)
        for (int i = 0; i < b; i++) s += f[(size_t)(Y * b + j) * ixdimp + X * b + i];
    return (double)s / (double)(b * b);
}

double rvo_tv_score(const int* slice, int ixdimp) {
    /* project-defined sharpness score of a centre sweep: total variation inside r < 0.45 n of the
     * slice averaged over b x b boxes, b = max(1, ixdimp / 512), n = ixdimp / b */
    const int b = ixdimp / 512 > 1 ? ixdimp / 512 : 1;
    const int nb = ixdimp / b;
    const double h = nb / 2.0, r2 = (0.45 * nb) * (0.45 * nb);
    double acc = 0.0;
#define RVO_BOX(X, Y) rvo_box(slice, ixdimp, b, (X), (Y))
    for (int y = 0; y < nb - 1; y++)
        for (int x = 0; x < nb - 1; x++) {
            const double dx = x - h, dy = y - h;
            if (dx * dx + dy * dy >= r2) continue;
            const double v = RVO_BOX(x, y);
            const double gx = RVO_BOX(x + 1, y) - v;
            const double gy = RVO_BOX(x, y + 1) - v;
            acc += sqrt(gx * gx + gy * gy);
        }
#undef RVO_BOX
    return acc;
}

/* ------------------------------------------------------------ offset-CT sinogram stitching ---- */
int rvo_offset_ct_views(const float* fdeg, int iLenSinogr) {
    /* CGazoDoc::GetSinogramYdim(TRUE), source/gazoDoc.cpp:2967-2978: index of the first frame
     * whose angle exceeds 180 degrees (the dark frame, last, is not examined); -1 if none */
    if (!fdeg) return -1;
    for (int i = 0; i + 1 < iLenSinogr; i++)
        if (fdeg[i] > 180.) return i;
    return -1;
}

/* (short)(a + (b - a) t): the mirrored-sample interpolation of source/gazoDoc.cpp:3590-3650,
 * int difference promoted to double, one product, one sum, truncation toward zero */
static short oct_mix(int a, int b, double t) {
    const double prod = (double)(b - a) * t;
    return (short)((double)a + prod);
}

/* crossfade of source/gazoDoc.cpp:3597,3614,3635,3652: (short)(r*v + (1-r)*s) */
static short oct_fade(double r, short v, short s) {
    const double x = r * (double)v;
    const double y = (1. - r) * (double)s;
    return (short)(x + y);
}

int rvo_offset_ct_stitch(const short* sino, long long sino_stride, short* of, long long of_stride,
                         const char* bInc, const float* fdeg, int iLenSinogr, int iMultiplex,
                         double center, double deltaCent, int iInterpolation, int iTrimWidth,
                         int iRawSinoXdim, int iXdim) {
    /* The offset-CT tail of CGazoDoc::GenerateSinogram (source/gazoDoc.cpp:3535-3665), on
     * already normalised int16 rows sino[(i*iMultiplex + j) * sino_stride + x], x < ixlen.
     * Output rows of[(i*iMultiplex + j) * of_stride + x], x < width, for i < nof.  Returns 0,
     * the reference's 21051 (no frame beyond 180 degrees) / 21052 (no partner frame), or -1 when
     * a row would read or write outside its bounds (undefined in the reference). */
    const int B = (iInterpolation == 0) ? 4 : ((iInterpolation == 1) ? 2 : 1);   /* :2987 */
    const int F = iRawSinoXdim, T = iTrimWidth;
    const int ixlen = F / B;                                                      /* :3002-3004 */
    const int width = iXdim / B;                                                  /* :3001 */
    const int nof = rvo_offset_ct_views(fdeg, iLenSinogr);
    if (nof < 0) return 21051;
    for (long long r = 0; r < (long long)nof * iMultiplex; r++) memset(of + r * of_stride, 0, sizeof(short) * width);
    const double cen = center + 0.5;   /* HALFPIXEL_OFFSET */
    int partner = nof;
    for (int i = 0; i < nof; i++) {
        if (!(bInc[i] & RV_BINC_SAMPLE)) continue;
        const double th = fdeg[i];
        /* the first later SAMPLE frame at least 180 degrees on; the search index only advances */
        while ((fdeg[partner] - th < 180) || !(bInc[partner] & RV_BINC_SAMPLE))
            if (++partner >= iLenSinogr - 1) return 21052;
        for (int j = 0; j < iMultiplex; j++) {
            const short* s1 = sino + (long long)(i * iMultiplex + j) * sino_stride;
            const short* s2 = sino + (long long)(partner * iMultiplex + j) * sino_stride;
            short* o = of + (long long)(i * iMultiplex + j) * of_stride;
#define OCT_PUT(pos, val) do { const int p_ = (pos); if (p_ < 0 || p_ >= width) return -1; o[p_] = (val); } while (0)
#define OCT_CHK1(k) do { if ((k) < 0 || (k) >= ixlen) return -1; } while (0)
            short held = 0;   /* the value repeated where the mirrored sample is missing */
            if (cen > F / 2.) {
                /* axis in the right half: own samples left of the overlap, mirrored partner right */
                const double fc = (cen + deltaCent * j * B + T) / B;
                const int ic = (int)fc;
                const double dc = fc - ic;
                const int g = F / B - 1 - ic;          /* half width of the crossfade */
                const int o0 = T / B;
                for (int k = o0; k <= ic - g; k++) { OCT_CHK1(k); OCT_PUT(k - o0, s1[k]); }
                const int kend = (2 * F - T) / B;
                for (int k = ic - g + 1; k < kend; k++) {
                    const int m = 2 * ic - k;
                    int ok;
                    if (dc < 0.5) {
                        ok = (m >= 0) && (m < ixlen - 1);
                        if (ok) held = oct_mix(s2[m + 1], s2[m], 1 - 2 * dc);
                    } else {
                        ok = (m >= 1) && (m < ixlen);
                        if (ok) held = oct_mix(s2[m - 1], s2[m], 2 - 2 * dc);
                    }
                    if (ok && k <= ic + g) {
                        OCT_CHK1(k);
                        held = oct_fade((double)(k - (ic - g)) / (g * 2 + 1), held, s1[k]);
                    }
                    OCT_PUT(k - o0, held);
                }
            } else {
                /* axis in the left half: own samples right of the overlap, mirrored partner left */
                const double fc = (cen + deltaCent * j * B) / B;
                const int ic = (int)(fc + 0.5);
                const double dc = fc - (int)fc;
                const int g = ic;
                const int sh = (F - T) / B;
                for (int k = (F - 1 - T) / B; k >= ic + g; k--) { OCT_CHK1(k); OCT_PUT(k + sh, s1[k]); }
                const int kmin = (dc < 0.5) ? 2 * ic + 1 - F / B : 2 * ic - F / B;
                for (int k = ic + g - 1; k >= kmin; k--) {
                    const int m = (dc < 0.5) ? 2 * ic - k : 2 * ic - 1 - k;
                    if ((m >= 0) && (m < ixlen - 1)) {
                        held = oct_mix(s2[m], s2[m + 1], (dc < 0.5) ? 2 * dc : 2 * dc - 1);
                        if (k >= ic - g) {
                            OCT_CHK1(k);
                            held = oct_fade((double)((ic + g) - k) / (g * 2 + 1), held, s1[k]);
                        }
                    }
                    OCT_PUT(k + sh, held);
                }
            }
#undef OCT_PUT
#undef OCT_CHK1
        }
    }
    return 0;
}

/* ---------------------------------------------------------------- R2: strip assembly ------- */
int rvo_bin_width(int ixFrm, int iTrim, int iInterpolation) {
    /* source/gazoDoc.cpp:2987, 3002-3004 (iBinning from iInterpolation; the trim narrows the row
     * only when 0 < iTrim < ixFrm / 2) */
    const int bin = (iInterpolation == 0) ? 4 : ((iInterpolation == 1) ? 2 : 1);
    if (iTrim < 0 || (iTrim > 0 && iTrim >= ixFrm / 2)) return -1;
    int ixlen = ixFrm;
    if (iTrim > 0) ixlen -= 2 * iTrim;
    return ixlen / bin;
}

int rvo_bin_strip(const unsigned short* strip, int ixFrm, int iTrim, int iInterpolation, int iMultiplex,
                  unsigned short* out, long long out_stride) {
    /* source/gazoDoc.cpp:3318-3342: sample k of slice j = (sum over the bin x bin block of rows
     * j*bin + iy, columns k*bin + ix + iTrim) / bin^2 in int arithmetic; bin 1 is a plain copy */
    const int bin = (iInterpolation == 0) ? 4 : ((iInterpolation == 1) ? 2 : 1);
    const int ixlen = rvo_bin_width(ixFrm, iTrim, iInterpolation);
    if (ixlen < 0) return -1;
    for (int j = 0; j < iMultiplex; j++) {
        for (int k = 0; k < ixlen; k++) {
            int isum = 0;
            for (int iy = 0; iy < bin; iy++)
                for (int ix = 0; ix < bin; ix++)
                    isum += strip[(long long)(j * bin + iy) * ixFrm + k * bin + ix + iTrim];
            out[j * out_stride + k] = (unsigned short)(isum / (bin * bin));
        }
    }
    return ixlen;
}
