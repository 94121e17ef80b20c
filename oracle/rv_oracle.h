/*
 * rv_oracle.h -- CPU restatement of RecView's convolution back-projection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA library and the timed CPU
 * baseline; no product code path links or calls it.  Every function restates one piece of the
 * reference, cited by file:line, in the same floating-point operation order (compile with
 * -ffp-contract=off) so that its results are bit-identical to the reference CPU routine.
 * Parity of this restatement is pinned against the reference's own sources compiled unmodified
 * (oracle/build_ref.sh -> oracle/_ref/) and against the committed golden vectors in tests/golden.
 */
#ifndef RV_ORACLE_H_
#define RV_ORACLE_H_

#include "../include/recview_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* R3: derived sizes (source/general.cpp:2022-2035). */
void rvo_dims(int ixdim, int iInterpolation, RvDims* d);

/* R4: filter table (source/gazoDoc.cpp:3747-3812, plus RV_FILT_SHEPP). */
int rvo_set_filter(int kind, double cutoff, double order, int ndim, float* out);

/* R6: CFft::Init1(np, -1) twiddles (source/cfft.cpp:374-410): n/2 entries each. */
void rvo_fft_twiddles(int np, float* wr, float* wi);
/* R6: CFft::FFT1Rev (source/cfft.cpp:431-434 -> FFTrev :193-277), in place on split arrays.
 * work = 4*n floats. */
void rvo_fft_forward(int np, const float* wr, const float* wi, float* re, float* im, float* work);
/* R6: CFft::FFT1 (source/cfft.cpp:412-429 -> FFT :279-369), in place, including the final
 * reversal and 1/n scaling. */
void rvo_fft_inverse(int np, const float* wr, const float* wi, float* re, float* im, float* work);

/* R5: row placement, edge padding and integer zoom interpolation into re[ndim]
 * (source/general.cpp:2105-2126); im is zeroed. */
void rvo_place_row(const RvDims* d, double center, const short* strip, float* re, float* im);
/* R5+R6+R7a: filtered row q[ixdimp] = Re(p[j + ihoffset]) (source/general.cpp:2105-2130).
 * work = 6*ndim floats. */
void rvo_filter_row(const RvDims* d, double center, const short* strip, const float* filt,
                    const float* wr, const float* wi, float* q, float* work);
/* R7b: int table igp[16*ixdimp] from a filtered row (source/general.cpp:2130-2137). */
void rvo_row_table(int ixdimp, const float* q, int* igp);
/* R3: per-view float geometry (source/general.cpp:2036-2037,2139-2142). */
float rvo_fcenter(const RvDims* d, double center);
void rvo_view_geometry(const RvDims* d, double center, float fdeg, float tilt, float* fcos,
                       float* fsin, float* foffset);
/* R8: scalar back-projection of one view over rows [iy0, iy1) (source/general.cpp:2147-2158). */
void rvo_backproject_view(int ixdimp, float fcos, float fsin, float foffset, const int* igp,
                          int* ifp, int iy0, int iy1);

/* Whole CPU routine (DeconvBackProjThread INTEL body, source/general.cpp:2020-2163) for one
 * worker: rows iy0..iy1 from ri->iStartSino/iStepSino, all SAMPLE views, accumulating into
 * ri->iReconst.  Returns 0, or RV_ERR_HOST_ALLOC. */
int rvo_reconstruct(RECONST_INFO* ri);
/* The reference's multi-worker CPU scheme (source/gazoDoc.cpp:3877-3984): nthreads workers
 * each owning a row band and re-filtering every view; writes disjoint rows of ri->iReconst
 * (the reference sums per-thread buffers that are zero outside each band: same result). */
int rvo_reconstruct_mt(RECONST_INFO* ri, int nthreads);

/* R1: GenerateSinogramThread (source/general.cpp:2377-2532), in place on ri->iSinogr, for
 * frames i with i % iStepSino == iStartSino.  Returns 0 or sets ri->iStatus and returns 1. */
int rvo_generate_sinogram(RECONST_INFO* ri);

/* R9: the rescale that follows the back-projection in CGazoDoc::DeconvBackProj
 * (source/gazoDoc.cpp:3993-4021), in place on slice[ixdimp^2]; center_user = the centre
 * before the HALFPIXEL/binning conversion, ipintp = zoom, ibinning = binning.  Returns imin and
 * imax through the pointers. */
void rvo_rescale(int* slice, int ixdimp, double center_user, int ipintp, int ibinning,
                 int* imin, int* imax);

/* FP64 end-to-end oracle for the linear-interpolation modes: the same padding, filter table
 * and geometry convention as the reference, evaluated in double with exact linear
 * interpolation of the filtered row and double accumulation; out[ixdimp^2] is scaled like the
 * int32 reference (x BACKPROJ_SCALE) so the two are directly comparable. */
int rvo_reconstruct_lin64(RECONST_INFO* ri, double* out);
/* The same with image rows split over nthreads threads (identical sums per pixel). */
int rvo_reconstruct_lin64_mt(RECONST_INFO* ri, double* out, int nthreads);

/* R11: CGazoDoc::GetAxis after the frame reads (source/gazoDoc.cpp:4379-4626): 0-degree frame,
 * ~180-degree frame and flat, ixdim x iydim each; returns the applied centre/gradient and the
 * overall SSD centre. */
int rvo_get_axis(const unsigned short* s0, const unsigned short* s1, const unsigned short* flat,
                 int ixdim, int iydim, int iAxisOffset, double* pCenter, double* pGrad, double* pOverall);
/* Project-defined centre-sweep score: total variation inside the circle r < 0.45 n of the slice
 * averaged over b x b boxes, b = max(1, ixdimp / 512), n = ixdimp / b. */
double rvo_tv_score(const int* slice, int ixdimp);

/* Offset-CT (360-degree scan, axis near a detector edge): GetSinogramYdim(TRUE)
 * (source/gazoDoc.cpp:2967-2978) and the stitching tail of CGazoDoc::GenerateSinogram
 * (source/gazoDoc.cpp:3535-3665) on contiguous int16 rows.  Returns 0, 21051, 21052, or -1 for a
 * configuration whose rows would be read or written out of bounds. */
int rvo_offset_ct_views(const float* fdeg, int iLenSinogr);
int rvo_offset_ct_stitch(const short* sino, long long sino_stride, short* of, long long of_stride,
                         const char* bInc, const float* fdeg, int iLenSinogr, int iMultiplex,
                         double center, double deltaCent, int iInterpolation, int iTrimWidth,
                         int iRawSinoXdim, int iXdim);

/* R2: strip assembly of CGazoDoc::GenerateSinogram for one frame (source/gazoDoc.cpp:3000-3004,
 * 3318-3342): strip = iMultiplex * bin detector rows of ixFrm uint16 samples (bin from
 * iInterpolation: 0 -> 4, 1 -> 2, else 1); row j of out (out_stride samples apart) receives the
 * trimmed width, each sample the integer mean (truncated) of its bin x bin block, shifted right by
 * iTrim samples.  Returns the width ixlen, or -1 when iTrim is negative or not below ixFrm / 2
 * (the reference then reads outside the row). */
int rvo_bin_width(int ixFrm, int iTrim, int iInterpolation);
int rvo_bin_strip(const unsigned short* strip, int ixFrm, int iTrim, int iInterpolation, int iMultiplex,
                  unsigned short* out, long long out_stride);

#ifdef __cplusplus
}
#endif
#endif
