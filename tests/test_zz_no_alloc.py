"""The allocation-free slice entry point against the regular one and the oracle.

RvReconstructSliceNoAlloc serves callers that are not allowed to allocate device memory (a
plugin inside a program that owns the device-memory pool, for instance): it keeps its scratch
in a fixed device array instead.  This file is collected last on purpose, so a failure here
cannot hide the rest of the suite; it must also pass when run alone in a fresh process."""
import ctypes as C
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

import recview_gb300 as rv
from recview_gb300 import abi
from tests.rvtest import fbp_case

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _device_copy(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


@pytest.mark.parametrize("on_stream", [False, True], ids=["legacy-stream", "torch-stream"])
@pytest.mark.parametrize("W,V,cen,interp", [(512, 900, 255.5, 2), (200, 181, 97.3, 3)])
def test_no_alloc_matches_regular_entry_point_twice(gpu, oracle, W, V, cen, interp, on_stream):
    torch = pytest.importorskip("torch")
    ri = fbp_case(90, W, V, cen, interp, oracle=oracle, skip_every=19)
    expect = oracle.reconstruct(ri, threads=4).copy()   # the reference CPU routine's result
    ri.reset_output()
    want = rv.reconstruct_slice(ri).copy()          # the existing entry point (CudaReconstHost)
    assert np.array_equal(want, expect)
    used = np.flatnonzero(ri.bInc & 1)
    d_sino = _device_copy(torch, ri.rows[used])      # the SAMPLE rows, as the caller provides them
    fdeg = np.ascontiguousarray(ri.fdeg[used], np.float32)
    F = ri.fFilter
    d = rv.dims(W, interp)
    L = rv.lib()
    stream = torch.cuda.Stream() if on_stream else None
    handle = C.c_void_p(stream.cuda_stream) if stream is not None else None
    for call in range(2):                            # two calls in a row share the scratch array
        d_out = torch.full((d.ixdimp, d.ixdimp), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = L.RvReconstructSliceNoAlloc(C.c_void_p(d_sino.data_ptr()), len(used), W, interp, cen,
                                         fdeg.ctypes.data_as(C.POINTER(C.c_float)), 0.0,
                                         F.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(d_out.data_ptr()),
                                         handle)
        assert rc == 0, rv.last_error()
        got = d_out.cpu().numpy()
        assert np.array_equal(got, want), f"call {call}: {np.count_nonzero(got != want)} pixels differ"


def test_no_alloc_rejects_oversize(gpu):
    torch = pytest.importorskip("torch")
    L = rv.lib()
    F = np.zeros(8192, np.float32)
    fdeg = np.zeros(3600, np.float32)
    # real (small) device buffers: the size check must refuse before anything touches them
    d_sino = torch.zeros(16, dtype=torch.int16, device="cuda")
    d_out = torch.full((16,), -7, dtype=torch.int32, device="cuda")
    rc = L.RvReconstructSliceNoAlloc(C.c_void_p(d_sino.data_ptr()), 3600, 4096, 2, 2047.5,
                                     fdeg.ctypes.data_as(C.POINTER(C.c_float)), 0.0,
                                     F.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(d_out.data_ptr()), None)
    assert rc == abi.RV_ERR_UNSUPPORTED
    assert "scratch" in rv.last_error()[1]
    torch.cuda.synchronize()
    assert torch.all(d_out == -7).item()


# Run in a child process that never imports torch: the device reset below destroys the context,
# which would pull every allocation out from under torch's caching allocator.  Buffers are pinned
# host memory from the library's own CUDA_MALLOC_HOST_INT, which kernels address directly (unified
# addressing).  The entry point is called after the reset only once the host-only query has shown
# that the address it resolves equals a fresh cudaGetSymbolAddress in the new context.
_RESET_CHILD = textwrap.dedent(r"""
    import ctypes as C, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    import recview_gb300 as rv
    from recview_gb300 import abi
    from tests.rvtest import Oracle, fbp_case

    L = rv.lib()
    assert 0 < L.GetCudaDeviceCount(0) < 0x10000
    oracle = Oracle()
    ri = fbp_case(91, 256, 360, 128.7, 2, oracle=oracle, skip_every=17)
    want = oracle.reconstruct(ri, threads=4).copy()
    used = np.flatnonzero(ri.bInc & 1)
    sino = np.ascontiguousarray(ri.rows[used], np.int16)
    fdeg = np.ascontiguousarray(ri.fdeg[used], np.float32)
    F = ri.fFilter
    npix = rv.dims(256, 2).ixdimp ** 2

    def addresses():
        r, f = C.c_void_p(), C.c_void_p()
        rc = L.RvNoAllocScratchAddress(C.byref(r), C.byref(f))
        assert rc == 0, rv.last_error()
        return r.value, f.value

    def one_call():
        p_in, p_out = C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
        assert L.CUDA_MALLOC_HOST_INT(C.byref(p_in), (sino.nbytes + 3) // 4 * 4) == 0
        assert L.CUDA_MALLOC_HOST_INT(C.byref(p_out), npix * 4) == 0
        C.memmove(p_in, sino.ctypes.data, sino.nbytes)
        rc = L.RvReconstructSliceNoAlloc(C.cast(p_in, C.c_void_p), len(used), 256, 2, 128.7,
                                         fdeg.ctypes.data_as(C.POINTER(C.c_float)), 0.0,
                                         F.ctypes.data_as(C.POINTER(C.c_float)), C.cast(p_out, C.c_void_p), None)
        assert rc == 0, rv.last_error()
        got = np.ctypeslib.as_array(p_out, shape=(npix,)).copy()
        L.CUDA_FREE_HOST(p_in)
        L.CUDA_FREE_HOST(p_out)
        return got

    r0, f0 = addresses()
    assert r0 and r0 == f0, (hex(r0 or 0), hex(f0 or 0))
    assert np.array_equal(one_call(), want.ravel())
    empty = abi.RECONST_INFO()
    empty.iStartSino = 0
    L.CudaReconstResourceFree(C.byref(empty), True)      # cudaDeviceReset: a new context follows
    r1, f1 = addresses()
    assert r1 and r1 == f1, (hex(r1 or 0), hex(f1 or 0))   # never an address of the old context
    assert np.array_equal(one_call(), want.ravel())
    print("NOALLOC_RESET_OK", hex(r0), hex(r1))
""")


def test_no_alloc_after_device_reset(gpu):
    env = dict(os.environ)
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, str(ROOT)], capture_output=True, text=True,
                       timeout=300, env=env, cwd=str(ROOT))
    assert r.returncode == 0 and "NOALLOC_RESET_OK" in r.stdout, r.stdout[-2000:] + r.stderr[-4000:]
