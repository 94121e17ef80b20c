"""The C-ABI library: it loads without a GPU, exports every symbol the public header declares,
and its host-side helpers agree with the oracle.  No kernel is launched here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from recview_gb300 import abi
from recview_gb300.reconst import dims

HEADER = Path(__file__).resolve().parents[1] / "include" / "recview_gb300.h"
# declared in the header because the library calls it, but defined by the application
APP_PROVIDED = {"DBProjDlgCtrl"}


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = set()
    for m in re.finditer(r"^\s*([A-Za-z_][\w \*]*?)\b([A-Za-z_]\w*)\s*\(", text, flags=re.M):
        if m.group(1).strip().startswith("typedef"):
            continue
        name = m.group(2)
        if name in ("if", "while", "for", "return", "sizeof", "typedef"):
            continue
        names.add(name)
    names -= {"RvErrorCallback", "RvProgressCallback"}
    return sorted(names)


def test_header_declares_what_abi_binds():
    assert set(declared_functions()) - APP_PROVIDED == set(abi.PROTOTYPES)


def test_library_exports_every_declared_symbol(rvlib):
    for name in declared_functions():
        if name in APP_PROVIDED:
            continue
        assert hasattr(rvlib, name), name


def test_header_struct_matches_ctypes():
    text = HEADER.read_text()
    body = text[text.index("typedef struct RECONST_INFO {"):text.index("} RECONST_INFO;")]
    fields = re.findall(r"([A-Za-z_]\w*)(?:\[\d+\])?;", body)
    assert fields == abi.FIELD_ORDER


@pytest.mark.parametrize("kind", range(7))
def test_set_filter_matches_oracle(rvlib, oracle, kind):
    for ndim in (256, 4096):
        for cut in (0.5, 0.3):
            a = np.zeros(ndim, np.float32)
            assert rvlib.RvSetFilter(kind, cut, 3.0, ndim, a.ctypes.data_as(C.POINTER(C.c_float))) == 0
            b = oracle.set_filter(kind, ndim, cut, 3.0)
            assert np.array_equal(a.view(np.int32), b.view(np.int32))


@pytest.mark.parametrize("W,interp", [(512, 2), (2048, 2), (37, 2), (1000, 3), (1024, 4), (96, 5), (4096, 2)])
def test_dims(rvlib, W, interp):
    d = abi.RvDims()
    assert rvlib.RvGetDims(W, interp, C.byref(d)) == 0
    ref = dims(W, interp)
    assert (d.ndim, d.ixdimp, d.ihoffset, d.iIntpDim) == (ref.ndim, ref.ixdimp, ref.ihoffset, ref.iIntpDim)


def test_errors_are_reported_not_raised(rvlib):
    rvlib.RvClearLastError()
    rvlib.CudaLsqfitHost(None, None, 0, 0, 0, 0, 0, 0, None, None, None, None)
    assert rvlib.RvGetLastError() == abi.RV_ERR_UNSUPPORTED
    rvlib.CudaReconstHost(None, 0, False, False)
    assert rvlib.RvGetLastError() == abi.RV_ERR_BAD_ARGUMENT
    assert rvlib.RvSetFilter(0, 0.5, 1.0, 0, None) == abi.RV_ERR_BAD_ARGUMENT


def test_error_callback(rvlib):
    seen = []
    cb = abi.ErrorCallback(lambda code, msg: seen.append((code, msg)))
    rvlib.RvSetErrorCallback(cb)
    try:
        rvlib.CudaLsqfitMemFree(None, None, 0, 0, None)
    finally:
        rvlib.RvSetErrorCallback(abi.ErrorCallback())
    assert seen and seen[0][0] == abi.RV_ERR_UNSUPPORTED


@pytest.mark.parametrize("ixdim,interp,trim,raw_width", [(100, 1, 50, 200),    # trim not below half the width
                                                          (100, 1, -2, 200),    # negative trim
                                                          (99, 1, 0, 200),      # width does not match
                                                          (100, 2, 3, 0)])      # trim without the raw width
def test_stack_rejects_inconsistent_strip_assembly(rvlib, ixdim, interp, trim, raw_width):
    """RvStackCreate validates the strip-assembly fields before touching the device."""
    V = 4
    binc = np.ones(V + 1, np.int8)
    binc[0] = 0
    fdeg = np.zeros(V + 1, np.float32)
    fexp = np.arange(V + 1, dtype=np.float32)
    F = np.zeros(dims(max(ixdim, 4)).ndim, np.float32)
    desc = abi.RvStackDesc()
    desc.ixdim, desc.iInterpolation, desc.center, desc.nframes, desc.nslices = ixdim, interp, ixdim / 2, V + 1, 1
    desc.bInc = C.cast(C.c_void_p(binc.ctypes.data), C.POINTER(C.c_char))
    desc.fdeg = fdeg.ctypes.data_as(C.POINTER(C.c_float))
    desc.fexp = fexp.ctypes.data_as(C.POINTER(C.c_float))
    desc.fFilter = F.ctypes.data_as(C.POINTER(C.c_float))
    desc.iTrim, desc.iRawWidth = trim, raw_width
    h = C.c_void_p()
    assert rvlib.RvStackCreate(C.byref(desc), C.byref(h)) == abi.RV_ERR_BAD_ARGUMENT
    assert not h.value
