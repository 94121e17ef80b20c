"""Offset-CT (360-degree) stitching on the GPU: RvOffsetCtStitchDevice / RvOffsetCtStitchHost
against the oracle (pinned to the reference build and the golden vectors) bit for bit, the
library's rejections against the oracle's out-of-bounds verdicts, a full-size frame geometry,
and stitched rows reconstructed through the stack path against the oracle's reconstruction.

Reference: the offset-CT tail of CGazoDoc::GenerateSinogram (source/gazoDoc.cpp:3535-3665),
CGazoDoc::DeconvBackProj (source/gazoDoc.cpp:3832-3836,3935,3947)."""
import ctypes as C

import numpy as np
import pytest

import recview_gb300 as rv
from recview_gb300 import abi, phantom
from recview_gb300.reconst import ReconInfo
from tests.rvtest import oct_random_case
from tests.test_offset_ct import OCT_NAMES, _desc, golden_case

pytestmark = pytest.mark.gpu


def _sizes(lib, d):
    nof, ixlen, width = C.c_int(), C.c_int(), C.c_int()
    rc = lib.RvOffsetCtDims(C.byref(d), C.byref(nof), C.byref(ixlen), C.byref(width))
    return rc, nof.value, ixlen.value, width.value


def stitch_device(lib, case):
    import torch
    d, keep = _desc(case)
    rc, nof, _ixlen, width = _sizes(lib, d)
    if rc:
        return rc, None
    rows = torch.from_numpy(np.ascontiguousarray(case["rows"], np.int16)).cuda()
    out = torch.full((max(nof, 1) * case["M"], width), 0x5A5A, dtype=torch.int16, device="cuda")
    rc = lib.RvOffsetCtStitchDevice(C.byref(d), C.c_void_p(rows.data_ptr()), C.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    return rc, out[:nof * case["M"]].cpu().numpy()


def stitch_host(lib, case):
    d, keep = _desc(case)
    rc, nof, _ixlen, width = _sizes(lib, d)
    if rc:
        return rc, None
    rows = np.ascontiguousarray(case["rows"], np.int16)
    out = np.full((nof * case["M"], width), 0x5A5A, np.int16)
    SP = C.POINTER(C.c_short)
    tin = (SP * rows.shape[0])(*[C.cast(C.c_void_p(rows.ctypes.data + r * rows.strides[0]), SP)
                                 for r in range(rows.shape[0])])
    tout = (SP * out.shape[0])(*[C.cast(C.c_void_p(out.ctypes.data + r * out.strides[0]), SP)
                                 for r in range(out.shape[0])])
    rc = lib.RvOffsetCtStitchHost(C.byref(d), tin, tout)
    return rc, out


@pytest.mark.parametrize("name", OCT_NAMES)
@pytest.mark.parametrize("form", ["device", "host"])
def test_golden_bit_exact(gpu, golden, name, form):
    case, rc_ref, out_ref = golden_case(golden, name)
    rc, out = (stitch_device if form == "device" else stitch_host)(gpu, case)
    assert rc == rc_ref, rv.last_error()
    if rc == 0:
        assert np.array_equal(out, out_ref)


def test_random_cases_match_oracle(gpu, oracle):
    rng = np.random.default_rng(77)
    counts = {"equal": 0, "rejected": 0}
    for trial in range(200):
        case = oct_random_case(rng, 500 + trial)
        rc_o, out_o = oracle.offset_ct(**case)
        rc, out = stitch_device(gpu, case)
        if rc_o == -1:          # a row would leave its bounds: undefined in the reference, rejected here
            assert rc == abi.RV_ERR_BAD_ARGUMENT, trial
            counts["rejected"] += 1
            continue
        assert rc == rc_o, (trial, rc, rc_o, rv.last_error())
        if rc == 0:
            assert np.array_equal(out, out_o), trial
            counts["equal"] += 1
    assert counts["equal"] > 150 and counts["rejected"] > 0


def test_full_size_frames(gpu, oracle):
    """2048-sample frames, 3600 views over 360 degrees (+ the closing view), 64 detector rows ->
    1800 (+1) stitched views of 4096 samples; random int16 rows exercise every sample value."""
    F, V, M = 2048, 3600, 64
    rng = np.random.default_rng(3)
    nf = 1 + (V + 1) + 1 + 1          # flat, samples 0..360 degrees, flat, dark
    rows = rng.integers(-4000, 30000, (nf * M, F), dtype=np.int16)
    bInc = np.zeros(nf, np.int8)
    bInc[1:V + 2] = 1
    fdeg = np.zeros(nf, np.float32)
    fdeg[1:V + 2] = (np.arange(V + 1) * (360.0 / V)).astype(np.float32)
    fdeg[V + 2:] = 360.0
    for cen, dcent in ((1998.37, 0.013), (41.81, -0.007)):
        case = dict(rows=rows, ixlen=F, bInc=bInc, fdeg=fdeg, M=M, center=cen, dcent=dcent, interp=2, trim=0, F=F,
                    iXdim=2 * F)
        rc, out = stitch_device(gpu, case)
        rc_o, out_o = oracle.offset_ct(**case)
        assert rc == 0 and rc_o == 0
        assert out.shape == (oracle.offset_ct_views(fdeg) * M, 2 * F)
        assert np.array_equal(out, out_o)


@pytest.mark.parametrize("cen", [120.6, 7.3])
def test_stitched_rows_reconstruct_like_oracle(gpu, oracle, cen):
    """Stitched rows (device) -> stack path in sinogram mode equals the oracle's FBP of the
    oracle's stitched rows, with ri->center from RvOffsetCtReconCenter."""
    import torch
    F, V, M = 128, 180, 2
    sino, bInc, fdeg = phantom.offset_ct_sinogram(9, F, V, M, cen, n_ellipsoids=8)
    nf = sino.shape[0]
    case = dict(rows=sino.reshape(nf * M, F), ixlen=F, bInc=bInc, fdeg=fdeg, M=M, center=cen, dcent=0.0, interp=2,
                trim=0, F=F, iXdim=2 * F)
    d, keep = _desc(case)
    rc, nof, _ixlen, width = _sizes(gpu, d)
    assert rc == 0
    rc_o, st_o = oracle.offset_ct(**case)
    assert rc_o == 0
    # device: stitch straight into a stack input buffer with one extra (dark) frame
    rows = torch.from_numpy(case["rows"]).cuda()
    buf = torch.zeros(((nof + 1) * M, width), dtype=torch.int16, device="cuda")
    assert gpu.RvOffsetCtStitchDevice(C.byref(d), C.c_void_p(rows.data_ptr()), C.c_void_p(buf.data_ptr()), None) == 0
    c_r = gpu.RvOffsetCtReconCenter(C.byref(d), cen)
    Ft = oracle.set_filter(abi.FILT_SHEPP, rv.dims(width).ndim)
    st = rv.Stack(ixdim=width, nframes=nof, nslices=M, center=c_r, bInc=bInc[:nof], fdeg=fdeg[:nof],
                  fexp=np.zeros(nof, np.float32), fFilter=Ft, input_is_sinogram=True)
    out = torch.empty((M, st.ixdimp, st.ixdimp), dtype=torch.int32, device="cuda")
    st.run_device(buf.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    st.close()
    assert np.array_equal(buf[:nof * M].cpu().numpy(), st_o)
    # oracle: the reference's FBP over the stitched rows (ri->iSinogr = ofSinogr, iLenSinogr = nof + 1)
    rows3 = np.concatenate([st_o, np.zeros((M, width), np.int16)]).reshape(nof + 1, M, width)
    for s in range(M):
        ri = ReconInfo(rows3, fdeg[:nof + 1], bInc[:nof + 1], center=c_r, fFilter=Ft, iMultiplex=M, iOffset=s,
                       maxSinogrLen=(nof + 1) * M, nviews=nof)
        assert np.array_equal(got[s], oracle.reconstruct(ri, threads=4)), s
    # and the stitched reconstruction sees the whole object: energy well inside the doubled field
    assert np.abs(got[0]).sum() > 0
