/*
 * recview_gb300.h -- C ABI of the GB300-native convolution back-projection library.
 *
 * Two groups of entry points:
 *
 *  1. The drop-in set.  These are exactly the symbols RecView's document/queue code binds from
 *     the CUDA back-end (source/cudaReconst.h:16-28,42-59 and source/cudaReconstDummy.cpp), with
 *     the same RECONST_INFO layout (source/reconstinfo.h:21-101), the same argument meaning, the
 *     same void-return + ri->iStatus error convention and the same numeric error codes.
 *     A RecView build links this library in place of cudaReconst.cu/cudaReconstHost.cpp.
 *
 *  2. New entry points (prefix Rv) that have no counterpart in the reference: the fused
 *     raw-frame stack path (normalise -> filter -> back-project for many slices in one call),
 *     the filter-table helper, geometry/error utilities and the reduced-storage modes.
 *
 * All signatures use plain pointers and sizes; no torch or CUDA C++ types cross the boundary.
 * Device pointers are typed void* / plain element pointers and streams are passed as void*.
 */
#ifndef RECVIEW_GB300_H_
#define RECVIEW_GB300_H_

#include <stddef.h>
#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- constants shared with the reference (values must stay identical) ------------------- */
/* source/constants.h:39-53 */
#define RV_LOG_SCALE 3000
#define RV_BACKPROJ_SCALE 100
#define RV_DBPT_GINTP 16
#define RV_SINOGRAM_PIXEL_MIN8bit 3
#define RV_SINOGRAM_PIXEL_MIN16bit 20
#define RV_ZOOMING_NONE 2
#define RECONST_INFO_IDLE 0
#define RECONST_INFO_BUSY 1
#define RECONST_INFO_ERROR 2
/* source/DlgQueue.h:19-26 */
#define RV_RQFLAGS_ZERNIKE 2
#define RV_RQFLAGS_DRIFTLIST 4
#define RV_RQFLAGS_DRIFTPARAMS 8
#define RV_RQFLAGS_USEONLYEVENFRAMES 16
#define RV_RQFLAGS_USEONLYODDFRAMES 32
#define RV_RQFLAGS_SINOGRAMKEPT 128
/* source/StdAfx.h:28-31 */
#define RV_BINC_WHITE 0
#define RV_BINC_SAMPLE 1
#define RV_BINC_NOUSE 2
#define RV_BINC_SKIP 4
/* source/general.h:35-36 (ri->iFlag bit) */
#define RV_READTIF8bit 2
/* source/DlgReconOpt.h:4-8; RV_FILT_SHEPP is this library's addition (the reference has no
 * Shepp-Logan window; any kind >= 5 gives an all-ones table there). */
#define RV_FILT_HAN 0
#define RV_FILT_HAM 1
#define RV_FILT_RAMP 2
#define RV_FILT_PARZN 3
#define RV_FILT_BUTER 4
#define RV_FILT_SHEPP 5
/* source/cudaReconst.h:8-13 */
#define CUDA_ERROR_DEVICEINFO_MASK 0x0000ffff
#define CUDA_ERROR_INSUFFICIENT_DRIVER 0x00010000
#define CUDA_ERROR_INSUFFICIENT_COMPUTE_CAPABILITY 0x00020000
#define CUDA_ERROR_VIRTUAL_DEVICE_DETECTED 0x00040000
#define CUDA_ERROR_DEVICE_GETPROPERTY 0x00080000
#define CUDA_ERROR_DEVICE_GETCOUNT 0x00100000

/* Error codes logged by the reference host code (source/cudaReconstHost.cpp:666-811), kept. */
#define RV_ERR_DEVICE_OOM 28801     /* device allocation failed */
#define RV_ERR_HOST_ALLOC 28802     /* host allocation failed */
#define RV_ERR_PINNED_ALLOC 28803   /* pinned host allocation failed */
#define RV_ERR_COPY_H2D 28804
#define RV_ERR_COPY_D2H 28805
#define RV_ERR_MEMSET 28806
#define RV_ERR_STREAM 28807
/* Codes added by this library (no reference counterpart). */
#define RV_ERR_BAD_ARGUMENT 28850   /* NULL pointer / inconsistent RECONST_INFO field */
#define RV_ERR_UNSUPPORTED 28851    /* size beyond a documented limit, unimplemented option */
#define RV_ERR_LAUNCH 28852         /* kernel launch / execution error */
#define RV_ERR_SET_DEVICE 28853     /* cudaSetDevice failed */
#define RV_ERR_KERNEL_STATUS 28854  /* a kernel reported a bounded-wait timeout or bad index */
#define RV_ERR_ABORTED 28855        /* the progress callback asked to stop */

/* ---- RECONST_INFO: byte-for-byte layout of source/reconstinfo.h:21-101 (x64) ------------- */
typedef struct RvFloat2 { float x, y; } RvFloat2;

typedef struct RECONST_INFO {
    unsigned char iStatus;
    int ixdim;
    int iInterpolation;
    double center;
    int iSinoCenter;
    int iLenSinogr;
    int* iReconst;
    int iStartSino;
    int iStepSino;
    unsigned int* pDoc;
    int* nSinogr;
    char dataName[61];
    char* bInc;
    float* fdeg;
    float* fexp;
    int iMultiplex;
    int iOffset;
    int maxSinogrLen;
    short** iSinogr;
    float* fFilter;
    unsigned int dReconFlags;
    float fTiltAngle;
    int drStart;
    int drEnd;
    double drX;
    double drY;
    int drOmit;               /* BOOL */
    unsigned int threadID;
    uintptr_t hThread;
    unsigned int max_d_ifp;
    unsigned int max_d_igp;
    int* d_ifp;
    int* d_igp;
    float* d_filt;
    unsigned int max_d_filt;
    short* d_strip;
    unsigned int max_d_strip;
    RvFloat2* d_p;            /* this library keeps its per-RECONST_INFO context here */
    unsigned int max_d_p;     /* == RV_CTX_TAG while d_p holds a context */
    float* d_px;
    unsigned int max_d_px;
    int fftplan;              /* cufftHandle */
    unsigned int ifftdim;
    void* stream1;            /* cudaStream_t */
    void* stream2;
    unsigned long long i64result;
    unsigned long long i64sum;
    short** ppRef;
    short** ppQry;
    unsigned int uiMaxRef;
    unsigned int uiMaxQry;
    void* pcxyz1;             /* CXyz* */
    void* pcxyz2;
    int iLsqBin;
    int iLsqBxref;
    int* piDrift;
    int iFlag;
} RECONST_INFO;

#define RV_CTX_TAG 0x52564742u  /* 'RVGB' */

/* ==== 1. Drop-in entry points (source/cudaReconst.h) ====================================== */

/* Filtered back-projection of one slice (replaces source/cudaReconstHost.cpp:629-813).
 * Reads ri->iSinogr rows i*iMultiplex+iOffset for views i = iStartSino, iStartSino+iStepSino, ...
 * that are SAMPLE frames, filters them with ri->fFilter, back-projects them and OVERWRITES
 * ri->iReconst[ixdimp*ixdimp] (int32, row-major iy*ixdimp+ix).  Increments *ri->nSinogr per
 * used view.  RQFLAGS_SINOGRAMKEPT + cached buffers reuse the previous call's filtered views
 * with an integer centre shift (source/cudaReconstHost.cpp:658,775).  The arithmetic follows
 * the reference CPU routine (source/general.cpp:2020-2163) bit-for-bit.  On failure sets
 * ri->iStatus = RECONST_INFO_ERROR and reports a code through RvSetErrorCallback.
 * bEnStream selects the two cached streams ri->stream1/2 (created on first use). */
void CudaReconstHost(RECONST_INFO* ri, int idev, bool bReport, bool bEnStream);
/* Same computation (source/cudaReconstHost.cpp:220-291 used cuFFT; this library always uses its
 * own on-device FFT, so both entry points share one implementation). */
void CudaReconstHostFFT(RECONST_INFO* ri, int idev, bool bReport);
/* Frees the device buffers cached in ri (source/cudaReconstHost.cpp:142-203). */
void CudaReconstMemFree(RECONST_INFO* ri);
/* Destroys ri->stream1/2 and frees buffers; bCudaDeviceReset additionally synchronises and
 * resets the device (source/cudaReconstHost.cpp:205-214).  The reset ends only this process's
 * context. */
void CudaReconstResourceFree(RECONST_INFO* ri, bool bCudaDeviceReset);
/* Flat/dark log normalisation of the raw uint16 rows in ri->iSinogr, in place, with the
 * semantics of the reference CPU routine GenerateSinogramThread (source/general.cpp:2377-2532),
 * which the reference uses instead of its own CUDA variant (source/cudaReconstHost.cpp:815-901).
 * Frames i with i % iStepSino == iStartSino are processed; ri->maxSinogrLen = frame count. */
void CudaSinogramHost(RECONST_INFO* ri, int idev, bool bReport);

/* Device queries (source/cudaReconst.cu:449-538). */
int GetCudaDeviceCount(int iMinComputeCapability);
int GetCudaMaxThreadsPerBlock(int iDevice);
int GetCudaWarpSize(int iDevice);
int GetCudaDeviceName(int iDevice, char* pcName, int iszcName);
int GetCudaDeviceComputingCapability(int iDevice, int* piMajor, int* piMinor);
int GetCudaNumberOfCores(int iDevice, int* piCores, int* piProcessors);
int GetCudaClockRate(int iDevice, int* piClockRate, int* piMemRate);

/* Pinned host buffers (source/cudaReconstHost.cpp:216-218).  Return a cudaError_t value. */
int CUDA_MALLOC_HOST_INT(int** ptr, size_t size);
int CUDA_FREE_HOST(void* ptr);

/* 3-D stitching (least squares) is outside this library's scope: these stubs keep the symbol
 * set of source/cudaReconstDummy.cpp:27-39, do nothing and report RV_ERR_UNSUPPORTED. */
void CudaLsqfitMemAlloc(short** d_ppRefPixel, short** d_ppQryPixel, int* pMaxRefPixel,
                        int* pMaxQryPixel, short** ppRefPixel, short** ppQryPixel, int nRefFiles,
                        int nQryFiles, int ixref, unsigned long long** d_result);
void CudaLsqfitMemFree(short** d_ppRefPixel, short** d_ppQryPixel, int nRefFiles, int nQryFiles,
                       unsigned long long* d_result);
void CudaLsqfitHost(short* d_ref, short* d_qry, int ixref, int iyref, int ixqry, int iyqry, int ix,
                    int iy, unsigned long long* ilsq, unsigned long long* nlsq,
                    unsigned long long* d_result, unsigned long long* h_result);

/* The progress/abort callback the reference host calls every 20 views
 * (source/general.cpp:2352-2375).  A RecView build defines it; this library calls it when
 * bReport is set, through a weak reference, or through the hook set by
 * RvSetProgressCallback when the application does not define the symbol. */
bool DBProjDlgCtrl(RECONST_INFO* ri, int iProgStep, int iSino, int* pCurrStep);

/* ==== 2. Entry points added by this library =============================================== */

/* Error reporting: the reference logs codes through its CError object; this library calls
 * the registered callback (may be NULL) and also keeps the last code per calling thread. */
typedef void (*RvErrorCallback)(int code, const char* message);
void RvSetErrorCallback(RvErrorCallback cb);
int RvGetLastError(void);                 /* last code on this thread, 0 if none */
const char* RvGetLastErrorMessage(void);  /* message for the last code on this thread */
void RvClearLastError(void);
typedef bool (*RvProgressCallback)(RECONST_INFO* ri, int iProgStep, int iSino, int* pCurrStep);
void RvSetProgressCallback(RvProgressCallback cb);

/* Filter table in the reference layout (mirrors CGazoDoc::SetFilter, source/gazoDoc.cpp:
 * 3747-3812): one-sided float[ndim]; kinds RV_FILT_*.  Returns 0 or RV_ERR_BAD_ARGUMENT. */
int RvSetFilter(int kind, double cutoff, double order, int ndim, float* out);

/* Derived sizes for a detector width and iInterpolation code (source/general.cpp:2022-2028). */
typedef struct RvDims {
    int ixdim, iZooming, iIntpDim, ndimp, ndim, ixdimp, ixdimh, ihoffset;
} RvDims;
int RvGetDims(int ixdim, int iInterpolation, RvDims* out);

/* ---- fused stack path: raw uint16 frames -> normalised -> filtered -> slices -------------- */
/* Reconstruction modes. */
#define RV_MODE_REF 0   /* reference semantics: 1/16 sub-sample int table, int32 slices (bit-exact) */
#define RV_MODE_LIN 1   /* linear interpolation, FP32 filtered rows, FP32 slices */
#define RV_MODE_LIN_F16 2  /* as LIN, filtered rows stored as FP16 under one power-of-two scale per filter
                              (bounded from the filter table), the interpolation as FP32 fma/add on the FP16
                              operands */
#define RV_MODE_LIN_BF16 3 /* as LIN, filtered rows stored as BF16 (unscaled: FP32's exponent range), the
                              interpolation as FP32 fma/add on the BF16 operands */

/* One stack = the frames of a RecView dataset for nslices detector rows, stored like the
 * reference's sinogram buffer: raw[(frame*nslices + slice)*ixdim + x], frames 0..nframes-1 are
 * the flat (WHITE) and SAMPLE frames in acquisition order, frame nframes is the dark. */
typedef struct RvStackDesc {
    int ixdim;              /* detector width (after trim/binning, as ri->ixdim) */
    int iInterpolation;     /* 2 = none; 3/4/5 = x2/x4/x8 zoom (source/gazoDoc.cpp:1864-1870) */
    double center;          /* rotation centre in ri->center convention */
    int nframes;            /* frames excluding the dark */
    int nslices;            /* detector rows per frame (ri->iMultiplex) */
    const char* bInc;       /* [nframes] RV_BINC_* flags (host) */
    const float* fdeg;      /* [nframes] angles in degrees (host) */
    const float* fexp;      /* [nframes] acquisition times used to interpolate flats (host) */
    float fTiltAngle;
    const float* fFilter;   /* [ndim] filter table in the reference layout (host) */
    unsigned int dReconFlags;  /* RV_RQFLAGS_USEONLY{EVEN,ODD}FRAMES honoured */
    int iFlag;              /* RV_READTIF8bit selects the 8-bit sample threshold */
    int mode;               /* RV_MODE_* */
    int input_is_sinogram;  /* 1: raw already holds log-normalised int16 rows (skip R1) */
    /* R2 strip assembly (source/gazoDoc.cpp:3000-3004,3318-3342), raw frames only.  iRawWidth = 0:
     * the frames are already trimmed and binned (nslices rows of ixdim samples per frame).
     * iRawWidth > 0: every frame holds nslices * bin detector rows of iRawWidth samples (bin = 4
     * for iInterpolation 0, 2 for 1, else 1); the library shifts each row by iTrim samples and
     * averages bin x bin blocks (integer mean, truncated) before the normalisation, and ixdim must
     * be the reference's width ((iRawWidth - 2 iTrim) / bin, the trim applied only when
     * 0 < iTrim < iRawWidth / 2).  iTrim outside [0, iRawWidth / 2) is RV_ERR_BAD_ARGUMENT. */
    int iTrim;
    int iRawWidth;
} RvStackDesc;

typedef struct RvStack RvStack;
/* Validates the description, builds per-view geometry and allocates device buffers. */
int RvStackCreate(const RvStackDesc* desc, RvStack** out);
void RvStackDestroy(RvStack* st);
/* Bytes of one output slice (ixdimp^2 * 4) and of the raw input ((nframes+1)*nslices*ixdim*2,
 * or (nframes+1)*nslices*bin*iRawWidth*2 when the library assembles the strips). */
size_t RvStackSliceBytes(const RvStack* st);
size_t RvStackInputBytes(const RvStack* st);
int RvStackNumViews(const RvStack* st);    /* SAMPLE views that are back-projected */
int RvStackOutputDim(const RvStack* st);   /* ixdimp */
/* Device-resident run: d_raw and d_out are device pointers, stream a cudaStream_t (or NULL for
 * the legacy default stream).  Output: nslices slices of ixdimp^2 int32 (REF) or float (LIN*). */
int RvStackRunDevice(RvStack* st, const void* d_raw, void* d_out, void* stream);
/* Host-buffer run: copies h_raw in, runs, copies the slices to h_out, synchronises.  Host
 * buffers may be pageable or pinned (pinned is faster). */
int RvStackRunHost(RvStack* st, const void* h_raw, void* h_out, void* stream);
/* Per-stage device timings (ms) of the last RvStackRunDevice/RunHost call, measured with CUDA
 * events on the launching stream: [0] filter stage, [1] back-projection, [2] whole call. */
int RvStackLastTimings(const RvStack* st, float* ms3);
/* Number of kernels launched by the last run. */
int RvStackLastLaunchCount(const RvStack* st);

/* Allocation-free variant of the one-slice reconstruction (no counterpart in the reference).
 * For callers that cannot allocate device memory -- e.g. a plugin inside a host program that
 * owns the device-memory pool, or code that must not synchronise the device through an
 * allocation -- but can pass device buffers: d_sino holds nviews log-normalised int16 rows of
 * ixdim samples (the SAMPLE views only, in order), fdeg[nviews] and fFilter[ndim] are host
 * arrays, d_slice receives ixdimp^2 int32 values; results equal CudaReconstHost's bit for bit.
 * Scratch (tables, geometry, FFT twiddles) lives in a fixed 64 MiB __device__ array that every
 * GPU loading this library keeps until the process exits; a slice needing more (about
 * nviews * 64 * ixdimp bytes) is rejected with RV_ERR_UNSUPPORTED.  The first call on a device
 * resolves the array's device address on that device, so make it before any stream capture; the
 * address is resolved again after the device's context has changed (a device reset, e.g.
 * CudaReconstResourceFree(ri, true)).  All calls share the array: calls that overlap on the GPU
 * race.  They also share the device's kernel-status word, so an overlapping call may report the
 * other's bounded-wait time-out.  The call is synchronous: it returns 0 or an RV_ERR_* code after
 * the slice is complete on `stream`. */
int RvReconstructSliceNoAlloc(const short* d_sino, int nviews, int ixdim, int iInterpolation,
                              double center, const float* fdeg, float fTiltAngle,
                              const float* fFilter, int* d_slice, void* stream);
/* Diagnostic query for RvReconstructSliceNoAlloc (no counterpart in the reference): *resolved =
 * the scratch address the entry point would use on the current device now, *fresh = a new
 * cudaGetSymbolAddress of the array.  Host-only (no launch, copy or allocation); they are equal
 * unless the address cache is wrong.  Returns 0 or an RV_ERR_* code. */
int RvNoAllocScratchAddress(void** resolved, void** fresh);

/* Validation mode: while enabled, the REF back-projection runs a bounds-checked variant that
 * skips and counts every table index falling outside the window staged in shared memory (the
 * production kernel relies on the window bound instead of per-access checks).  Slower; for tests. */
int RvSetCheckedBackprojection(int enable);
unsigned long long RvGetWindowViolations(void);

/* R9: the rescale CGazoDoc::DeconvBackProj applies to finished slices (source/gazoDoc.cpp:
 * 3993-4021), on the device, in place on d_slices[nslices][ixdimp^2] (int32): per slice imin/imax
 * (imax starts at 0), pixels outside the circle of radius min(ipintp*c/bin, ixdimp - ipintp*c/bin)
 * (c = the user centre before the half-pixel/binning conversion) set to 0, others mapped to
 * (v - imin) * 65534 / (imax - imin) in float.  Optional d_out16 receives the same values as
 * uint16; minmax (host, 2*nslices) receives imin, imax per slice (imax before the +1 of a flat
 * slice).  Synchronises `stream` before returning. */
int RvRescaleSlices(int* d_slices, int nslices, int ixdimp, double center_user, int ipintp, int ibinning,
                    unsigned short* d_out16, int* minmax, void* stream);

/* ---- output files (R9 / next-row TIFF output) -------------------------------------------------
 * RecView's per-slice 16-bit TIFF (WriteTifMonochrome16, source/general.cpp:1313-1470), byte for
 * byte: slice = the rescaled int values (RvRescaleSlices), negatives stored as 0; artist NULL
 * gives the reference's "SP-uCT, gazoView".  RvTiff16Bytes returns the file size and fills out
 * when cap is large enough (negative RV_ERR_* on bad arguments). */
long long RvTiff16Bytes(const int* slice, int height, int width, const char* description, const char* artist,
                        unsigned char* out, long long cap);
int RvWriteTiff16(const char* path, const int* slice, int height, int width, const char* description,
                  const char* artist);
/* The physical scale of the rescaled values (pixelBase/pixelDiv, source/gazoDoc.cpp:3997-4006) and
 * the ImageDescription string BatchReconst writes (source/gazoDoc.cpp:1985-1988). */
int RvPixelScale(int nSinogr, double pixelWidth, int iBinning, int ipintp, int imin, int imax, int zernike,
                 float* pixelBase, float* pixelDiv);
int RvImageDescription(char* out, int cap, int nSinogr, double pixelWidth, float pixelDiv, float pixelBase,
                       double centre, int filterKind);

/* ---- batched queue (no reference counterpart; replaces the sequential queue loop of
 * source/DlgQueue.cpp:363-470 / CGazoDoc::BatchReconst, source/gazoDoc.cpp:1938-1993) --------
 * Datasets of uneven detector width, view count, centre and zoom are added as stack descriptions
 * with device buffers (raw frames in, int32 slices out).  RvQueueRun groups their slices into
 * waves whose tables fit a device-memory pool (RV_TABLE_BUDGET_MB, default 32768), runs each
 * wave as one filter launch per dataset plus one persistent back-projection kernel that takes
 * tiles of every dataset from a device work list, captures the whole sequence in a CUDA graph on
 * the first run and replays the graph afterwards.  REF mode only; results equal RvStackRunDevice's.
 * Each wave runs one persistent launch per back-projection variant in use.  RvQueueAutotune
 * (optional, before the first run) tunes per shape class -- output size (ixdimp <= 1024 / 2048 /
 * 4096 / more), view count (<= 1000 / 2000 / more), slice pairs possible or not: on 2-8 slices of
 * one dataset of each class it times persistent variants that differ in pixel tile, views per
 * staged chunk, slices per CTA and consumer warps, and keeps the fastest in a process-wide cache
 * keyed by the class (datasets added later with a cached class use it).  *chosen_variant receives
 * the first dataset's choice; RvQueueItemVariant gives any dataset's. */
typedef struct RvQueue RvQueue;
int RvQueueCreate(RvQueue** out);
int RvQueueAdd(RvQueue* q, const RvStackDesc* desc, const void* d_raw, void* d_out);
int RvQueueAutotune(RvQueue* q, void* stream, int* chosen_variant);
int RvQueueItemVariant(const RvQueue* q, int item);   /* -1 for a bad index */
/* Pins dataset `item` to a back-projection variant (0-21), overriding the tuned choice. */
int RvQueueSetItemVariant(RvQueue* q, int item, int variant);
int RvQueueRun(RvQueue* q, void* stream);
float RvQueueLastMs(const RvQueue* q);        /* device time of the last run */
double RvQueueUpdates(const RvQueue* q);      /* pixel-view updates of one run */
void RvQueueDestroy(RvQueue* q);

/* R11: the reference's automatic centre estimate, CGazoDoc::GetAxis (source/gazoDoc.cpp:4036-4626),
 * from frames the caller has read: the first sample frame (0 deg), the sample frame nearest
 * 180 deg minus one step, and a flat, each iydim rows of ixdim uint16 (host).  iAxisOffset > 0
 * selects the offset-CT branch.  pCenter/pGrad receive the applied line centre(iy) = c + g*iy
 * (the user-centre convention of the reference: ri->center = (c + 0.5) / binning); pOverall
 * (may be NULL) the overall SSD centre.  Results equal the reference's. */
int RvGetAxis(const unsigned short* sample0, const unsigned short* sample1, const unsigned short* flat,
              int ixdim, int iydim, int iAxisOffset, double* pCenter, double* pGrad, double* pOverall);

/* R11: the axis-scan sweep (source/gazoDoc.cpp:1994-2024) with a score: one slice (nviews
 * log-normalised int16 rows of ixdim, host) reconstructed at ncent trial centres (ri->center
 * convention), scores[i] = total variation of trial i, averaged over b x b pixel boxes
 * (b = max(1, ixdimp / 512)), inside the circle r < 0.45 of its width (this library's criterion:
 * lowest = sharpest; the reference leaves the choice to a person; use a smoothing filter such as
 * Hann with cutoff 0.25 for noisy data), and
 * best_centre = a parabola through the lowest score and its neighbours (equal steps). */
int RvCentreSweep(const short* sino, int nviews, int ixdim, int iInterpolation, const float* fdeg,
                  float fTiltAngle, const float* fFilter, const double* centres, int ncent,
                  double* scores, double* best_centre);

/* Tuning of the REF back-projection (process-wide; affects stacks created and slices reconstructed
 * afterwards).  format: 0 = the reference's 16-int table per detector pixel, 1 = the same padded
 * to 17 words (fewer shared-memory bank conflicts), 2 = the float pair (p0, slope) per
 * detector pixel, expanded by the kernel with the reference's operations (8x smaller tables,
 * conflict-free lookups).  variant 0..21 selects tile shape / threads / views per chunk, and
 * whether the per-view coordinate products are tabulated in shared memory (0-5) or formed in
 * registers (6-21), whether warps synchronise per chunk (0-8) or only wait for their data
 * (9-21), whether a dedicated warp stages the tables (16-21), whether each warp register
 * covers a compact 8x4 pixel block (0-15, 17) or 32 pixels along the view's ray direction,
 * re-laid per angle range (16, 18-21), and how many slices that share the geometry a CTA
 * reconstructs with one index computation per pixel and view (18, 19: two; 21: three, the rest
 * of a stack as pairs; 20: four; 19 and 20 with 16 consumer warps) (default: format 0,
 * variant 21).  All combinations give
 * bit-identical slices.  Returns RV_ERR_BAD_ARGUMENT outside these ranges. */
int RvSetBackprojectionVariant(int variant, int format);
int RvGetBackprojectionVariant(int* variant, int* format);

/* Device throughput probes used as roofline denominators for the back-projection, which is
 * bound by the shared-memory pipe (its table gathers) rather than HBM or tensor cores:
 * out[0] = FP32 FMA TFLOP/s,
 * out[1] = float->int32 conversions in G/s and, when n >= 3, out[2] = shared-memory load bandwidth
 * in GB/s (conflict-free 32-bit loads, one 128-byte wavefront per warp instruction), all measured
 * on the current device. */
int RvProbeThroughput(double* out, int n);

/* 1 when kernels on the current device read and write pageable host memory directly (the GPU
 * shares the host's page tables, as on Grace-based systems) and RV_NO_HOST_DIRECT is not set:
 * CudaReconstHost then takes the caller's sinogram rows and slice buffer without staged copies
 * (no reference counterpart). */
int RvHostDirectAccess(void);

/* Failure-detection self-check (no reference counterpart): one CTA waits, with the kernels'
 * bounded mbarrier wait (2^log2_tries tries of at most ~1 us each, log2_tries 8..16), on a
 * barrier that nothing completes.  Returns RV_ERR_KERNEL_STATUS when the wait ran out and was
 * reported, as it must (the status is cleared; the context stays usable); *elapsed_ms gets the
 * kernel's duration. */
int RvTestBoundedWait(int log2_tries, double* elapsed_ms);

/* ---- Offset-CT (360-degree scan with the rotation axis near one edge of the frame) ----------
 * Replaces the offset-CT tail of CGazoDoc::GenerateSinogram (source/gazoDoc.cpp:3535-3665):
 * every SAMPLE view i below nof = GetSinogramYdim(TRUE) (the first frame beyond 180 degrees,
 * source/gazoDoc.cpp:2967-2978) is joined with the first later SAMPLE frame at least 180 degrees
 * on into one row of width = iXdim / binning samples: the view's own samples on the axis side,
 * the partner mirrored about the axis (linear interpolation for the sub-pixel axis position) on
 * the other, crossfaded over the overlap, exactly as the reference rounds them.  Non-SAMPLE views
 * give zero rows.  The stitched rows are then reconstructed like any sinogram with ixdim =
 * width, iLenSinogr = nof + 1 and ri->center = RvOffsetCtReconCenter(...)
 * (CGazoDoc::DeconvBackProj, source/gazoDoc.cpp:3832-3836,3935). */
typedef struct RvOffsetCtDesc {
    int iRawSinoXdim;      /* frame width before binning (rq->iRawSinoXdim) */
    int iXdim;             /* stitched width before binning (rq->iXdim; RecView sets 2*iRawSinoXdim) */
    int iInterpolation;    /* rq->iInterpolation: binning 4 / 2 / 1 for 0 / 1 / other values */
    int iTrimWidth;        /* rq->iTrimWidth */
    int iLenSinogr;        /* frames including the dark frame (CGazoDoc::iLenSinogr) */
    int iMultiplex;        /* detector rows (slices) per frame */
    double center;         /* rotation centre passed to GenerateSinogram (frame pixels, user convention) */
    double deltaCent;      /* centre change per detector row (GenerateSinogram's deltaCent) */
    const char* bInc;      /* [iLenSinogr] RV_BINC_* flags (host) */
    const float* fdeg;     /* [iLenSinogr] angles in degrees (host) */
} RvOffsetCtDesc;

/* Sizes: nof stitched views, ixlen = iRawSinoXdim / binning samples per input row, width samples
 * per output row.  Returns 0, 21051 (no frame beyond 180 degrees, as the reference) or
 * RV_ERR_BAD_ARGUMENT. */
int RvOffsetCtDims(const RvOffsetCtDesc* desc, int* nof, int* ixlen, int* width);
/* ri->center for the reconstruction of stitched rows of one detector row whose centre (user
 * convention, frame pixels) is layer_center. */
double RvOffsetCtReconCenter(const RvOffsetCtDesc* desc, double layer_center);
/* Device buffers: d_sino = iLenSinogr * iMultiplex rows of ixlen normalised int16 samples (row
 * i*iMultiplex + j = frame i, detector row j, the reference's iSinogr order); d_out = nof *
 * iMultiplex rows of width samples, all written.  Asynchronous on stream (NULL = legacy default
 * stream).  Returns 0, 21051 / 21052 (no frame beyond 180 degrees / a view without a partner,
 * as the reference), RV_ERR_BAD_ARGUMENT (also when a row would be read or written outside its
 * bounds, which the reference leaves undefined), or a CUDA error code. */
int RvOffsetCtStitchDevice(const RvOffsetCtDesc* desc, const short* d_sino, short* d_out, void* stream);
/* The reference's host form: iSinogr[i*iMultiplex + j] rows in, ofSinogr[i*iMultiplex + j] rows
 * (width samples each, i < nof) out; synchronous.  Same return codes. */
int RvOffsetCtStitchHost(const RvOffsetCtDesc* desc, short* const* iSinogr, short* const* ofSinogr);

/* ---- learned centre proposal (no reference counterpart; RecView leaves the centre choice to a
 * person looking at an axis-scan sweep, source/gazoDoc.cpp:1994-2024) ---------------------------
 * A small BF16 CNN (6 x {conv 3x3 + ReLU + 2x2 average pool}, channels 4-32-32-64-64-128-128, then
 * FC 128 + ReLU, FC 2) maps four detector rows of a sinogram, prepared by RvCentreNetInput, to
 * (mu, s): the centre offset estimate and the log-variance of its error.  Trained on the device
 * with its own forward/backward kernels and Adam.  Parameters are one FP32 vector in the order
 * w0 b0 w1 b1 ... w5 b5 f0w f0b f1w f1b (conv weights [cout][cin][3][3], FC weights [out][in]).
 * Inputs are device bf16 tensors [n][4][H][W]; H and W are multiples of 64. */
typedef struct RvCentreNet RvCentreNet;
int RvCentreNetCreate(int H, int W, int batch, unsigned long long seed, RvCentreNet** out);
void RvCentreNetDestroy(RvCentreNet* net);
long long RvCentreNetNumParams(const RvCentreNet* net);
int RvCentreNetSetParams(RvCentreNet* net, const float* host_params);   /* also resets Adam */
int RvCentreNetGetParams(const RvCentreNet* net, float* host_params);
/* (mu, s) of count samples (host arrays of count; either may be NULL); synchronous. */
int RvCentreNetForward(RvCentreNet* net, const void* d_x, int count, float* mu, float* s, void* stream);
/* Mean Gaussian NLL 0.5 e^-s (y - mu)^2 + 0.5 s over the batch and its parameter gradients
 * (host, RvCentreNetNumParams floats; may be NULL); no update.  y on the host. */
int RvCentreNetGradients(RvCentreNet* net, const void* d_x, const float* y, int count, float* loss,
                         float* grads_host, void* stream);
/* One Adam step (0.9, 0.999, 1e-8) at learning rate lr; d_y on the device; *loss (may be NULL)
 * receives the batch loss before the step (synchronising when requested). */
int RvCentreNetTrainStep(RvCentreNet* net, const void* d_x, const float* d_y, int count, float lr, float* loss,
                         void* stream);
/* Synthetic raw frames for training and evaluating the centre search (no reference counterpart):
 * a seeded ellipsoid phantom (n_ellipsoids, centres in a ball of radius 0.8, semi-axes
 * U[0.05, 0.4], attenuation U[-0.2, 1.0]), flat 20000 (1 + 0.02 smooth), dark ~ N(100, 3),
 * Poisson-like noise, rotation centre `center` (ri->center convention).  d_raw (device) receives
 * [(nviews + 3)][S][W] uint16: frame 0 flat, frames 1..nviews samples at view_deg, frame
 * nviews + 1 flat, the dark frame last; bInc/fdeg/fexp (host, nviews + 2 each, may be NULL) the
 * frame table.  Synchronous. */
int RvPhantomFrames(unsigned long long seed, int W, int S, const float* view_deg, int nviews, double center,
                    int n_ellipsoids, void* d_raw, char* bInc, float* fdeg, float* fexp, void* stream);
/* R1 on a device-resident raw stack (the normalisation of CudaSinogramHost, all SAMPLE frames):
 * d_sino [(nframes + 1)][nslices][ixdim] int16, other rows zero.  Uses desc's ixdim, nframes,
 * nslices, bInc, fexp, dReconFlags (Zernike) and iFlag.  Synchronous. */
int RvNormaliseStack(const RvStackDesc* desc, const void* d_raw, short* d_sino, void* stream);
/* The network input [4][256][512] bf16 (device) from normalised rows d_sino [frames][S][W]
 * (W a multiple of 512): detector rows s0..s0+3, the 256 frames listed (in angle order over the
 * half-turn), W/512 samples averaged per bin, values / 3000, rows 0..127 = frames[128..255] as
 * measured, rows 128..255 = frames[0..127] mirrored about the detector centre (so the two ends of
 * the half-turn meet in the middle row, where the centre offset shows as a horizontal shift).
 * Synchronous. */
int RvCentreNetInput(const short* d_sino, int S, int W, const int* frames256, int s0, void* d_x, void* stream);
/* Synthetic training data made by the plain method: scans of a seeded phantom with the centre
 * (W-1)/2 + U[-max_offset, max_offset], the reference's normalisation, then RvCentreNetInput on
 * the 256 views of a `views`-view half-turn the network reads.  Sample i of a description is
 * always the same scan (seeded by seed and i). */
typedef struct RvCentreTrainDesc {
    int W;                   /* detector width, a multiple of 512 */
    int views;               /* views over 180 degrees of the simulated scans (>= 256) */
    int slices;              /* detector rows per scan (>= 4; rows 0..3 feed the network) */
    int n_ellipsoids;
    double max_offset;       /* pixels */
    unsigned long long seed;
} RvCentreTrainDesc;
/* Samples first..first+count-1 into d_x ([count][4][256][512] bf16, device) and their targets
 * offset/16 into d_y (device).  Synchronous. */
int RvCentreNetMakeSamples(const RvCentreTrainDesc* desc, int first, int count, void* d_x, float* d_y,
                           void* stream);
/* Adam on samples [0, ntrain) of d_x/d_y for `epochs` shuffled passes in batches of `batch`
 * (<= the network's batch), learning rate from lr_max to lr_min on a cosine; samples
 * [ntrain, ntrain + nval) are held out.  stats (may be NULL) receives the held-out |error| of the
 * proposal in pixels at the 50th / 90th / 99th percentile and the wall time in seconds. */
int RvCentreNetFit(RvCentreNet* net, const void* d_x, const float* d_y, int ntrain, int nval, int epochs, int batch,
                   float lr_max, float lr_min, unsigned long long seed, float* stats, void* stream);
/* Centre search (row (f2)): the plain sweep on the grid grid_centre + step*k, k = -half_range..
 * half_range (RvCentreSweep's criterion on detector row s_sweep of d_sino [nframes][S][W], the
 * SAMPLE frames of bInc at fdeg), narrowed by the network when net is not NULL: the network reads
 * rows s_net..s_net+3 (RvCentreNetInput, the proposal is (W-1)/2 + 16 mu with uncertainty
 * 16 e^(s/2) pixels) and the search starts with the 2*window+1 grid trials around the proposal,
 * walking towards lower scores until the lowest is confirmed over +-(window+1) grid steps; a
 * proposal more than window steps from grid_centre gets a second walk from grid_centre.  The full
 * sweep runs instead when the uncertainty exceeds sigma_max or the walks exceed 5 (2*window+1)
 * trials.  centre = the sweep criterion's choice (parabola-refined). */
typedef struct RvCentreSearchResult {
    double centre;     /* chosen centre (ri->center convention) */
    double proposal;   /* network proposal (NaN without a network) */
    double sigma;      /* network's uncertainty in pixels (NaN without a network) */
    int trials;        /* trial reconstructions run */
    int fallback;      /* 1: the full sweep ran */
    double ms;         /* wall time of the search */
} RvCentreSearchResult;
int RvCentreSearch(RvCentreNet* net, const short* d_sino, int S, int W, int nframes, const char* bInc,
                   const float* fdeg, int s_net, int s_sweep, const float* fFilter, double grid_centre,
                   int half_range, double step, int window, double sigma_max, RvCentreSearchResult* out,
                   void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RECVIEW_GB300_H_ */
