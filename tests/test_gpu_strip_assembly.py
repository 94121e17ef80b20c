"""R2 on the device: raw frames at full detector resolution, trimmed and binned bin x bin by the
filter kernel's load phase (CGazoDoc::GenerateSinogram's strip assembly,
source/gazoDoc.cpp:3000-3004,3318-3342), then normalised, filtered and back-projected.  Every
slice must equal the oracle's: strip assembly, GenerateSinogramThread and the CPU FBP."""
import numpy as np
import pytest

import recview_gb300 as rv
from recview_gb300 import abi, phantom
from recview_gb300.reconst import ReconInfo, dims

pytestmark = pytest.mark.gpu


def _oracle(oracle, binned, bInc, fdeg, fexp, cen, F, interp, S):
    r = np.ascontiguousarray(binned).copy()
    ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=S, maxSinogrLen=r.shape[0],
                   iInterpolation=interp)
    oracle.generate_sinogram(ri)
    outs = []
    for s in range(S):
        rs = ReconInfo(r.view(np.int16), fdeg, bInc, center=cen, fFilter=F, iInterpolation=interp, iMultiplex=S,
                       iOffset=s, maxSinogrLen=r.shape[0] * S, nviews=r.shape[0] - 1)
        outs.append(oracle.reconstruct(rs, threads=8).copy())
    return np.stack(outs)


# (raw frame width, trim, iInterpolation, slices, views): bin 2 / bin 4 / trim only / trim + x2 zoom
CASES = [(256, 5, 1, 3, 120), (384, 3, 0, 2, 90), (300, 9, 2, 3, 150), (260, 66, 3, 2, 100), (128, 0, 1, 4, 60)]


@pytest.mark.parametrize("F,T,interp,S,V", CASES, ids=lambda c: str(c))
def test_stack_strip_assembly_bit_exact(gpu, oracle, F, T, interp, S, V):
    B = 4 if interp == 0 else (2 if interp == 1 else 1)
    ixlen = oracle.L.rvo_bin_width(F, T, interp)
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(400 + F + T, F, V, S * B, F / 2.0 + 1.7, n_ellipsoids=12,
                                                 nflat_before=2, nflat_after=1)
    binned = oracle.bin_frames(raw, F, T, interp, S)          # [frames + 1, S, ixlen]
    cen = ixlen / 2.0 + 0.35 * (1 + (F % 5))
    d = dims(ixlen, interp)
    Fl = oracle.set_filter(abi.FILT_SHEPP, d.ndim)
    want = _oracle(oracle, binned, bInc, fdeg, fexp, cen, Fl, interp, S)
    st = rv.Stack(ixdim=ixlen, nframes=raw.shape[0] - 1, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp,
                  fFilter=Fl, iInterpolation=interp, iTrim=T, raw_width=F)
    assert rv.lib().RvStackInputBytes(st.h) == raw.nbytes
    for _ in range(2):
        got = st.run_host(raw)
        assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} pixels differ"
    st.close()


def test_stack_strip_assembly_device_run(gpu, oracle):
    """RvStackRunDevice on device-resident full-resolution frames (bin 2, trim 4)."""
    torch = pytest.importorskip("torch")
    F, T, interp, S, V = 200, 4, 1, 2, 90
    ixlen = oracle.L.rvo_bin_width(F, T, interp)
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(77, F, V, 2 * S, 99.3, n_ellipsoids=10)
    binned = oracle.bin_frames(raw, F, T, interp, S)
    cen = ixlen / 2.0 - 2.6
    Fl = oracle.set_filter(abi.FILT_SHEPP, dims(ixlen, interp).ndim)
    want = _oracle(oracle, binned, bInc, fdeg, fexp, cen, Fl, interp, S)
    st = rv.Stack(ixdim=ixlen, nframes=raw.shape[0] - 1, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp,
                  fFilter=Fl, iInterpolation=interp, iTrim=T, raw_width=F)
    d_raw = torch.from_numpy(raw.view(np.int16)).cuda()
    d_out = torch.zeros((S, st.ixdimp, st.ixdimp), dtype=torch.int32, device="cuda")
    st.run_device(d_raw.data_ptr(), d_out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), want)
    st.close()
