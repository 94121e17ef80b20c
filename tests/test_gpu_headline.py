"""Parity at the full-scale stack geometry: a 2048-pixel detector, 1800 views over 180 degrees,
raw uint16 frames (Poisson counts of an ellipsoid phantom on a smooth flat field, a dark field
~N(100, 3)), rotation centre 1023.5 + U[-10, 10] px, Shepp-Logan filter.  This is the path the
throughput figure is measured on: RvStackRunDevice / RvStackRunHost, the fused normalise + filter
kernel, and the default back-projection on groups of three slices (the rest of a stack as slice
pairs).
Every slice must equal the oracle (the reference CPU routine restated) bit for bit."""
import ctypes as C
import os

import numpy as np
import pytest

import recview_gb300 as rv
from recview_gb300 import abi, phantom
from recview_gb300.reconst import ReconInfo, dims

pytestmark = pytest.mark.gpu

W, V = 2048, 1800
THREADS = max(4, os.cpu_count() or 4)


def _case(seed: int, S: int):
    rng = np.random.default_rng(seed)
    cen = (W - 1) / 2.0 + rng.uniform(-10.0, 10.0)
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(seed, W, V, S, cen, n_ellipsoids=40)
    return raw, bInc, fdeg, fexp, cen


def _oracle_slices(oracle, raw, bInc, fdeg, fexp, cen, F, S):
    """GenerateSinogramThread on the raw frames, then the CPU FBP of each detector row."""
    r = raw.copy()
    ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=S, maxSinogrLen=raw.shape[0])
    oracle.generate_sinogram(ri)
    out = []
    for s in range(S):
        rs = ReconInfo(r.view(np.int16), fdeg, bInc, center=cen, fFilter=F, iMultiplex=S, iOffset=s,
                       maxSinogrLen=r.shape[0] * S, nviews=raw.shape[0] - 1)
        out.append(oracle.reconstruct(rs, threads=THREADS).copy())
    return np.stack(out)


@pytest.fixture(scope="module")
def headline(oracle):
    S = 5   # one group of three slices and one slice pair
    raw, bInc, fdeg, fexp, cen = _case(2026, S)
    F = oracle.set_filter(abi.FILT_SHEPP, dims(W).ndim)
    want = _oracle_slices(oracle, raw, bInc, fdeg, fexp, cen, F, S)
    return raw, bInc, fdeg, fexp, cen, F, want


def test_headline_uses_default_variant(gpu):
    v, f = C.c_int(), C.c_int()
    gpu.RvGetBackprojectionVariant(C.byref(v), C.byref(f))
    assert (v.value, f.value) == (21, 0)   # three-slice groups, dense 16-entry tables: what the bench times


def test_headline_stack_host_bit_exact(gpu, headline):
    raw, bInc, fdeg, fexp, cen, F, want = headline
    S = want.shape[0]
    st = rv.Stack(ixdim=W, nframes=raw.shape[0] - 1, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp,
                  fFilter=F)
    assert st.nviews == V and st.ixdimp == W
    got = st.run_host(raw)
    st.close()
    for s in range(S):
        assert np.array_equal(got[s], want[s]), f"slice {s}: {np.count_nonzero(got[s] != want[s])} pixels differ"


def test_headline_stack_device_bit_exact(gpu, headline):
    torch = pytest.importorskip("torch")
    raw, bInc, fdeg, fexp, cen, F, want = headline
    S = want.shape[0]
    st = rv.Stack(ixdim=W, nframes=raw.shape[0] - 1, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp,
                  fFilter=F)
    d_raw = torch.from_numpy(raw.view(np.int16)).cuda()
    d_out = torch.full((S, W, W), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    for _ in range(2):   # the second run reuses the stack's tables and buffers
        st.run_device(d_raw.data_ptr(), d_out.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        got = d_out.cpu().numpy()
        for s in range(S):
            assert np.array_equal(got[s], want[s]), f"slice {s}: {np.count_nonzero(got[s] != want[s])} pixels differ"
    st.close()


def test_headline_window_bound_checked(gpu, headline):
    """The bounds-checked twin of the default back-projection at the full geometry: no table
    index falls outside the staged window, and the slices are still the oracle's."""
    raw, bInc, fdeg, fexp, cen, F, want = headline
    S = 3   # one group of three slices
    raw2 = np.ascontiguousarray(raw[:, :S, :])
    L = rv.lib()
    assert L.RvSetCheckedBackprojection(1) == 0
    try:
        st = rv.Stack(ixdim=W, nframes=raw2.shape[0] - 1, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp,
                      fFilter=F)
        got = st.run_host(raw2)
        st.close()
        assert L.RvGetWindowViolations() == 0
    finally:
        L.RvSetCheckedBackprojection(0)
    # the slices of a 3-row stack are the same detector rows as the first three of the 5-row one
    for s in range(S):
        assert np.array_equal(got[s], want[s])
