"""ctypes mirror of include/recview_gb300.h.

The RECONST_INFO layout is RecView's (source/reconstinfo.h:21-101); the field list here and in the
C header must stay identical.  Nothing in this module touches CUDA: it only describes types and
function prototypes, so it is importable on machines without a GPU.
"""
from __future__ import annotations

import ctypes as C

c_int_p = C.POINTER(C.c_int)
c_float_p = C.POINTER(C.c_float)
c_short_p = C.POINTER(C.c_short)
c_short_pp = C.POINTER(c_short_p)


class RvFloat2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class RECONST_INFO(C.Structure):
    """source/reconstinfo.h:21-101 (x64 layout)."""

    _fields_ = [
        ("iStatus", C.c_ubyte),
        ("ixdim", C.c_int),
        ("iInterpolation", C.c_int),
        ("center", C.c_double),
        ("iSinoCenter", C.c_int),
        ("iLenSinogr", C.c_int),
        ("iReconst", c_int_p),
        ("iStartSino", C.c_int),
        ("iStepSino", C.c_int),
        ("pDoc", C.POINTER(C.c_uint)),
        ("nSinogr", c_int_p),
        ("dataName", C.c_char * 61),
        ("bInc", C.POINTER(C.c_char)),
        ("fdeg", c_float_p),
        ("fexp", c_float_p),
        ("iMultiplex", C.c_int),
        ("iOffset", C.c_int),
        ("maxSinogrLen", C.c_int),
        ("iSinogr", c_short_pp),
        ("fFilter", c_float_p),
        ("dReconFlags", C.c_uint),
        ("fTiltAngle", C.c_float),
        ("drStart", C.c_int),
        ("drEnd", C.c_int),
        ("drX", C.c_double),
        ("drY", C.c_double),
        ("drOmit", C.c_int),
        ("threadID", C.c_uint),
        ("hThread", C.c_size_t),
        ("max_d_ifp", C.c_uint),
        ("max_d_igp", C.c_uint),
        ("d_ifp", c_int_p),
        ("d_igp", c_int_p),
        ("d_filt", c_float_p),
        ("max_d_filt", C.c_uint),
        ("d_strip", c_short_p),
        ("max_d_strip", C.c_uint),
        ("d_p", C.POINTER(RvFloat2)),
        ("max_d_p", C.c_uint),
        ("d_px", c_float_p),
        ("max_d_px", C.c_uint),
        ("fftplan", C.c_int),
        ("ifftdim", C.c_uint),
        ("stream1", C.c_void_p),
        ("stream2", C.c_void_p),
        ("i64result", C.c_ulonglong),
        ("i64sum", C.c_ulonglong),
        ("ppRef", c_short_pp),
        ("ppQry", c_short_pp),
        ("uiMaxRef", C.c_uint),
        ("uiMaxQry", C.c_uint),
        ("pcxyz1", C.c_void_p),
        ("pcxyz2", C.c_void_p),
        ("iLsqBin", C.c_int),
        ("iLsqBxref", C.c_int),
        ("piDrift", c_int_p),
        ("iFlag", C.c_int),
    ]


FIELD_ORDER = [f[0] for f in RECONST_INFO._fields_]


class RvDims(C.Structure):
    _fields_ = [(n, C.c_int) for n in
                ("ixdim", "iZooming", "iIntpDim", "ndimp", "ndim", "ixdimp", "ixdimh", "ihoffset")]


class RvStackDesc(C.Structure):
    _fields_ = [
        ("ixdim", C.c_int),
        ("iInterpolation", C.c_int),
        ("center", C.c_double),
        ("nframes", C.c_int),
        ("nslices", C.c_int),
        ("bInc", C.POINTER(C.c_char)),
        ("fdeg", c_float_p),
        ("fexp", c_float_p),
        ("fTiltAngle", C.c_float),
        ("fFilter", c_float_p),
        ("dReconFlags", C.c_uint),
        ("iFlag", C.c_int),
        ("mode", C.c_int),
        ("input_is_sinogram", C.c_int),
        ("iTrim", C.c_int),
        ("iRawWidth", C.c_int),
    ]


class RvOffsetCtDesc(C.Structure):
    _fields_ = [
        ("iRawSinoXdim", C.c_int),
        ("iXdim", C.c_int),
        ("iInterpolation", C.c_int),
        ("iTrimWidth", C.c_int),
        ("iLenSinogr", C.c_int),
        ("iMultiplex", C.c_int),
        ("center", C.c_double),
        ("deltaCent", C.c_double),
        ("bInc", C.POINTER(C.c_char)),
        ("fdeg", c_float_p),
    ]


class RvCentreTrainDesc(C.Structure):
    _fields_ = [
        ("W", C.c_int),
        ("views", C.c_int),
        ("slices", C.c_int),
        ("n_ellipsoids", C.c_int),
        ("max_offset", C.c_double),
        ("seed", C.c_ulonglong),
    ]


class RvCentreSearchResult(C.Structure):
    _fields_ = [
        ("centre", C.c_double),
        ("proposal", C.c_double),
        ("sigma", C.c_double),
        ("trials", C.c_int),
        ("fallback", C.c_int),
        ("ms", C.c_double),
    ]


# constants (include/recview_gb300.h)
LOG_SCALE = 3000
BACKPROJ_SCALE = 100
DBPT_GINTP = 16
ZOOMING_NONE = 2
RECONST_INFO_IDLE, RECONST_INFO_BUSY, RECONST_INFO_ERROR = 0, 1, 2
RQFLAGS_ZERNIKE = 2
RQFLAGS_DRIFTLIST = 4
RQFLAGS_DRIFTPARAMS = 8
RQFLAGS_USEONLYEVENFRAMES = 16
RQFLAGS_USEONLYODDFRAMES = 32
RQFLAGS_SINOGRAMKEPT = 128
BINC_WHITE, BINC_SAMPLE, BINC_NOUSE, BINC_SKIP = 0, 1, 2, 4
READTIF8bit = 2
FILT_HAN, FILT_HAM, FILT_RAMP, FILT_PARZN, FILT_BUTER, FILT_SHEPP = 0, 1, 2, 3, 4, 5
MODE_REF, MODE_LIN, MODE_LIN_F16, MODE_LIN_BF16 = 0, 1, 2, 3

RV_ERR_DEVICE_OOM = 28801
RV_ERR_HOST_ALLOC = 28802
RV_ERR_PINNED_ALLOC = 28803
RV_ERR_COPY_H2D = 28804
RV_ERR_COPY_D2H = 28805
RV_ERR_MEMSET = 28806
RV_ERR_STREAM = 28807
RV_ERR_BAD_ARGUMENT = 28850
RV_ERR_UNSUPPORTED = 28851
RV_ERR_LAUNCH = 28852
RV_ERR_SET_DEVICE = 28853
RV_ERR_KERNEL_STATUS = 28854
RV_ERR_ABORTED = 28855

ErrorCallback = C.CFUNCTYPE(None, C.c_int, C.c_char_p)
ProgressCallback = C.CFUNCTYPE(C.c_bool, C.POINTER(RECONST_INFO), C.c_int, C.c_int, c_int_p)

# name -> (restype, argtypes) for every symbol include/recview_gb300.h declares
PROTOTYPES = {
    "CudaReconstHost": (None, [C.POINTER(RECONST_INFO), C.c_int, C.c_bool, C.c_bool]),
    "CudaReconstHostFFT": (None, [C.POINTER(RECONST_INFO), C.c_int, C.c_bool]),
    "CudaReconstMemFree": (None, [C.POINTER(RECONST_INFO)]),
    "CudaReconstResourceFree": (None, [C.POINTER(RECONST_INFO), C.c_bool]),
    "CudaSinogramHost": (None, [C.POINTER(RECONST_INFO), C.c_int, C.c_bool]),
    "GetCudaDeviceCount": (C.c_int, [C.c_int]),
    "GetCudaMaxThreadsPerBlock": (C.c_int, [C.c_int]),
    "GetCudaWarpSize": (C.c_int, [C.c_int]),
    "GetCudaDeviceName": (C.c_int, [C.c_int, C.c_char_p, C.c_int]),
    "GetCudaDeviceComputingCapability": (C.c_int, [C.c_int, c_int_p, c_int_p]),
    "GetCudaNumberOfCores": (C.c_int, [C.c_int, c_int_p, c_int_p]),
    "GetCudaClockRate": (C.c_int, [C.c_int, c_int_p, c_int_p]),
    "CUDA_MALLOC_HOST_INT": (C.c_int, [C.POINTER(c_int_p), C.c_size_t]),
    "CUDA_FREE_HOST": (C.c_int, [C.c_void_p]),
    "CudaLsqfitMemAlloc": (None, [c_short_pp, c_short_pp, c_int_p, c_int_p, c_short_pp, c_short_pp,
                                  C.c_int, C.c_int, C.c_int, C.POINTER(C.POINTER(C.c_ulonglong))]),
    "CudaLsqfitMemFree": (None, [c_short_pp, c_short_pp, C.c_int, C.c_int, C.POINTER(C.c_ulonglong)]),
    "CudaLsqfitHost": (None, [c_short_p, c_short_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                              C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong),
                              C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]),
    "RvSetErrorCallback": (None, [ErrorCallback]),
    "RvGetLastError": (C.c_int, []),
    "RvGetLastErrorMessage": (C.c_char_p, []),
    "RvClearLastError": (None, []),
    "RvSetProgressCallback": (None, [ProgressCallback]),
    "RvSetFilter": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_int, c_float_p]),
    "RvGetDims": (C.c_int, [C.c_int, C.c_int, C.POINTER(RvDims)]),
    "RvStackCreate": (C.c_int, [C.POINTER(RvStackDesc), C.POINTER(C.c_void_p)]),
    "RvStackDestroy": (None, [C.c_void_p]),
    "RvStackSliceBytes": (C.c_size_t, [C.c_void_p]),
    "RvStackInputBytes": (C.c_size_t, [C.c_void_p]),
    "RvStackNumViews": (C.c_int, [C.c_void_p]),
    "RvStackOutputDim": (C.c_int, [C.c_void_p]),
    "RvStackRunDevice": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "RvStackRunHost": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "RvStackLastTimings": (C.c_int, [C.c_void_p, c_float_p]),
    "RvStackLastLaunchCount": (C.c_int, [C.c_void_p]),
    "RvSetCheckedBackprojection": (C.c_int, [C.c_int]),
    "RvGetWindowViolations": (C.c_ulonglong, []),
    "RvProbeThroughput": (C.c_int, [C.POINTER(C.c_double), C.c_int]),
    "RvTestBoundedWait": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "RvHostDirectAccess": (C.c_int, []),
    "RvRescaleSlices": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_void_p,
                                  c_int_p, C.c_void_p]),
    "RvGetAxis": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                            C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "RvCentreSweep": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, c_float_p, C.c_float, c_float_p,
                                C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "RvTiff16Bytes": (C.c_longlong, [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_char_p, C.c_void_p,
                                     C.c_longlong]),
    "RvWriteTiff16": (C.c_int, [C.c_char_p, C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_char_p]),
    "RvPixelScale": (C.c_int, [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, c_float_p,
                               c_float_p]),
    "RvImageDescription": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_float, C.c_float, C.c_double,
                                     C.c_int]),
    "RvQueueCreate": (C.c_int, [C.POINTER(C.c_void_p)]),
    "RvQueueAdd": (C.c_int, [C.c_void_p, C.POINTER(RvStackDesc), C.c_void_p, C.c_void_p]),
    "RvQueueAutotune": (C.c_int, [C.c_void_p, C.c_void_p, c_int_p]),
    "RvQueueRun": (C.c_int, [C.c_void_p, C.c_void_p]),
    "RvQueueItemVariant": (C.c_int, [C.c_void_p, C.c_int]),
    "RvQueueSetItemVariant": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "RvQueueLastMs": (C.c_float, [C.c_void_p]),
    "RvQueueUpdates": (C.c_double, [C.c_void_p]),
    "RvQueueDestroy": (None, [C.c_void_p]),
    "RvSetBackprojectionVariant": (C.c_int, [C.c_int, C.c_int]),
    "RvGetBackprojectionVariant": (C.c_int, [c_int_p, c_int_p]),
    "RvReconstructSliceNoAlloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, c_float_p,
                                            C.c_float, c_float_p, C.c_void_p, C.c_void_p]),
    "RvNoAllocScratchAddress": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "RvOffsetCtDims": (C.c_int, [C.POINTER(RvOffsetCtDesc), c_int_p, c_int_p, c_int_p]),
    "RvOffsetCtReconCenter": (C.c_double, [C.POINTER(RvOffsetCtDesc), C.c_double]),
    "RvOffsetCtStitchDevice": (C.c_int, [C.POINTER(RvOffsetCtDesc), C.c_void_p, C.c_void_p, C.c_void_p]),
    "RvOffsetCtStitchHost": (C.c_int, [C.POINTER(RvOffsetCtDesc), C.c_void_p, C.c_void_p]),
    "RvCentreNetCreate": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "RvCentreNetDestroy": (None, [C.c_void_p]),
    "RvCentreNetNumParams": (C.c_longlong, [C.c_void_p]),
    "RvCentreNetSetParams": (C.c_int, [C.c_void_p, c_float_p]),
    "RvCentreNetGetParams": (C.c_int, [C.c_void_p, c_float_p]),
    "RvCentreNetForward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, c_float_p, c_float_p, C.c_void_p]),
    "RvCentreNetGradients": (C.c_int, [C.c_void_p, C.c_void_p, c_float_p, C.c_int, c_float_p, c_float_p,
                                       C.c_void_p]),
    "RvCentreNetTrainStep": (C.c_int, [C.c_void_p, C.c_void_p, c_float_p, C.c_int, C.c_float, c_float_p,
                                       C.c_void_p]),
    "RvPhantomFrames": (C.c_int, [C.c_ulonglong, C.c_int, C.c_int, c_float_p, C.c_int, C.c_double, C.c_int,
                                  C.c_void_p, C.c_void_p, c_float_p, c_float_p, C.c_void_p]),
    "RvNormaliseStack": (C.c_int, [C.POINTER(RvStackDesc), C.c_void_p, C.c_void_p, C.c_void_p]),
    "RvCentreNetInput": (C.c_int, [C.c_void_p, C.c_int, C.c_int, c_int_p, C.c_int, C.c_void_p, C.c_void_p]),
    "RvCentreNetMakeSamples": (C.c_int, [C.POINTER(RvCentreTrainDesc), C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_void_p]),
    "RvCentreNetFit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                 C.c_float, C.c_ulonglong, c_float_p, C.c_void_p]),
    "RvCentreSearch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, c_float_p, C.c_int,
                                 C.c_int, c_float_p, C.c_double, C.c_int, C.c_double, C.c_int, C.c_double,
                                 C.POINTER(RvCentreSearchResult), C.c_void_p]),
}


def bind(lib: C.CDLL) -> C.CDLL:
    """Attach restype/argtypes to every exported symbol; raises if one is missing."""
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
