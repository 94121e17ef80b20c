"""The allocation-free slice entry point against the regular one.

RvReconstructSliceNoAlloc serves callers that are not allowed to allocate device memory (a
plugin inside a program that owns the device-memory pool, for instance): it keeps its scratch
in a fixed device array instead.  This file is collected last on purpose, so a failure here
cannot hide the rest of the suite; it must also pass when run alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import recview_gb300 as rv
from recview_gb300 import abi
from tests.rvtest import fbp_case

pytestmark = pytest.mark.gpu


def _device_copy(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


@pytest.mark.parametrize("W,V,cen,interp", [(512, 900, 255.5, 2), (200, 181, 97.3, 3)])
def test_no_alloc_matches_regular_entry_point_twice(gpu, oracle, W, V, cen, interp):
    torch = pytest.importorskip("torch")
    ri = fbp_case(90, W, V, cen, interp, oracle=oracle, skip_every=19)
    ri.reset_output()
    want = rv.reconstruct_slice(ri).copy()          # the existing entry point (CudaReconstHost)
    used = np.flatnonzero(ri.bInc & 1)
    d_sino = _device_copy(torch, ri.rows[used])      # the SAMPLE rows, as the caller provides them
    fdeg = np.ascontiguousarray(ri.fdeg[used], np.float32)
    F = ri.fFilter
    d = rv.dims(W, interp)
    L = rv.lib()
    for call in range(2):                            # two calls in a row share the scratch array
        d_out = torch.full((d.ixdimp, d.ixdimp), -7, dtype=torch.int32, device="cuda")
        rc = L.RvReconstructSliceNoAlloc(C.c_void_p(d_sino.data_ptr()), len(used), W, interp, cen,
                                         fdeg.ctypes.data_as(C.POINTER(C.c_float)), 0.0,
                                         F.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(d_out.data_ptr()),
                                         None)
        assert rc == 0, rv.last_error()
        got = d_out.cpu().numpy()
        assert np.array_equal(got, want), f"call {call}: {np.count_nonzero(got != want)} pixels differ"


def test_no_alloc_rejects_oversize(gpu):
    L = rv.lib()
    F = np.zeros(8192, np.float32)
    fdeg = np.zeros(3600, np.float32)
    rc = L.RvReconstructSliceNoAlloc(C.c_void_p(16), 3600, 4096, 2, 2047.5, fdeg.ctypes.data_as(C.POINTER(C.c_float)),
                                     0.0, F.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(16), None)
    assert rc == abi.RV_ERR_UNSUPPORTED
    assert "scratch" in rv.last_error()[1]
