"""Offset-CT (360-degree) sinogram stitching on the CPU: the oracle restatement against the
golden vectors and the reference build, and the library's host-only helpers.

Reference: CGazoDoc::GetSinogramYdim (source/gazoDoc.cpp:2967-2978) and the offset-CT tail of
CGazoDoc::GenerateSinogram (source/gazoDoc.cpp:3535-3665); reconstruction centre
CGazoDoc::DeconvBackProj (source/gazoDoc.cpp:3832-3836,3935)."""
import ctypes as C

import numpy as np
import pytest

from recview_gb300 import abi
from tests.rvtest import oct_call, oct_random_case, ref_lib

OCT_NAMES = ["oct_right_lo", "oct_right_hi", "oct_left_lo", "oct_left_hi", "oct_bin2", "oct_trim", "oct_skip",
             "oct_e21051", "oct_e21052"]


def golden_case(golden, name):
    F, iXdim, interp, T, M, cen, dcent, rc = golden[f"{name}_params"]
    B = 4 if int(interp) == 0 else (2 if int(interp) == 1 else 1)
    return dict(rows=golden[f"{name}_rows"], ixlen=int(F) // B, bInc=golden[f"{name}_binc"],
                fdeg=golden[f"{name}_fdeg"], M=int(M), center=float(cen), dcent=float(dcent), interp=int(interp),
                trim=int(T), F=int(F), iXdim=int(iXdim)), int(rc), golden[f"{name}_out"]


@pytest.mark.parametrize("name", OCT_NAMES)
def test_oracle_matches_golden(golden, oracle, name):
    case, rc_ref, out_ref = golden_case(golden, name)
    rc, out = oracle.offset_ct(**case)
    assert rc == rc_ref
    if rc == 0:
        assert out.shape == out_ref.shape and np.array_equal(out, out_ref)


def test_golden_cases_cover_every_branch(golden):
    # right/left axis x sub-pixel split below/above one half, binning, trim, skipped views, both errors
    seen = set()
    for name in OCT_NAMES:
        case, rc, _ = golden_case(golden, name)
        if rc:
            seen.add(rc)
            continue
        B = 4 if case["interp"] == 0 else (2 if case["interp"] == 1 else 1)
        cen = case["center"] + 0.5
        right = cen > case["F"] / 2.0
        fc = (cen + case["trim"]) / B if right else cen / B
        seen.add(("R" if right else "L", (fc - int(fc)) >= 0.5))
    assert {("R", False), ("R", True), ("L", False), ("L", True), 21051, 21052} <= seen


REF = ref_lib()


@pytest.mark.skipif(REF is None, reason="reference build not present")
def test_oracle_matches_reference_random(oracle):
    rng = np.random.default_rng(2024)
    n_equal = 0
    for trial in range(150):
        case = oct_random_case(rng, trial)
        rc, out = oracle.offset_ct(**case)
        if rc == -1:
            continue            # out-of-bounds configuration: undefined in the reference, not run there
        nof = oracle.offset_ct_views(case["fdeg"])
        rc2, out2 = oct_call(REF.rvref_offset_ct, case["rows"], case["ixlen"], case["bInc"], case["fdeg"], case["M"],
                             case["center"], case["dcent"], case["interp"], case["trim"], case["F"], case["iXdim"],
                             nof)
        assert rc == rc2, (trial, rc, rc2)
        if rc == 0:
            assert np.array_equal(out, out2), trial
            n_equal += 1
    assert n_equal > 100


def _desc(case):
    keep = [np.ascontiguousarray(case["bInc"], np.int8), np.ascontiguousarray(case["fdeg"], np.float32)]
    d = abi.RvOffsetCtDesc()
    d.iRawSinoXdim, d.iXdim, d.iInterpolation = case["F"], case["iXdim"], case["interp"]
    d.iTrimWidth, d.iLenSinogr, d.iMultiplex = case["trim"], len(keep[1]), case["M"]
    d.center, d.deltaCent = case["center"], case["dcent"]
    d.bInc = C.cast(C.c_void_p(keep[0].ctypes.data), C.POINTER(C.c_char))
    d.fdeg = keep[1].ctypes.data_as(C.POINTER(C.c_float))
    return d, keep


@pytest.mark.parametrize("name", OCT_NAMES)
def test_dims_match_oracle(rvlib, oracle, golden, name):
    """RvOffsetCtDims is host logic: number of stitched views, row widths, and error 21051."""
    case, rc_ref, _ = golden_case(golden, name)
    d, _keep = _desc(case)
    nof, ixlen, width = C.c_int(), C.c_int(), C.c_int()
    rc = rvlib.RvOffsetCtDims(C.byref(d), C.byref(nof), C.byref(ixlen), C.byref(width))
    if rc_ref == 21051:
        assert rc == 21051 and rvlib.RvGetLastError() == 21051
        return
    assert rc == 0
    assert nof.value == oracle.offset_ct_views(case["fdeg"])
    B = 4 if case["interp"] == 0 else (2 if case["interp"] == 1 else 1)
    assert (ixlen.value, width.value) == (case["F"] // B, case["iXdim"] // B)


def test_dims_rejects_bad_description(rvlib):
    d = abi.RvOffsetCtDesc()
    assert rvlib.RvOffsetCtDims(C.byref(d), None, None, None) == abi.RV_ERR_BAD_ARGUMENT
    assert rvlib.RvOffsetCtDims(None, None, None, None) == abi.RV_ERR_BAD_ARGUMENT


@pytest.mark.parametrize("F,interp,c", [(2048, 2, 2000.3), (2048, 2, 30.6), (2048, 2, 1024.0), (2048, 2, 1023.7),
                                        (1024, 1, 1000.0), (1024, 0, 12.25)])
def test_recon_center(rvlib, F, interp, c):
    # DeconvBackProj: a centre at or left of the frame middle moves by the frame width, then
    # ri->center = (c + 0.5) / binning
    d = abi.RvOffsetCtDesc()
    d.iRawSinoXdim, d.iInterpolation = F, interp
    B = 4 if interp == 0 else (2 if interp == 1 else 1)
    want = ((F + c if c <= F / 2.0 else c) + 0.5) / B
    assert rvlib.RvOffsetCtReconCenter(C.byref(d), c) == want
