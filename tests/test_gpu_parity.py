"""GPU parity: the CUDA library through its C ABI against the oracle (the reference CPU routine
restated, pinned to the reference sources and golden vectors).  REF results must be
bit-identical; LIN/FP16/BF16 results are judged against the FP64 end-to-end oracle with the
tolerances written below."""
import ctypes as C

import numpy as np
import pytest

import recview_gb300 as rv
from recview_gb300 import abi, phantom
from recview_gb300.reconst import ReconInfo, dims
from tests.rvtest import fbp_case, rel_l2

pytestmark = pytest.mark.gpu

# (seed, W, V, centre, iInterpolation, filter, flags, tilt)
SLICE_CASES = [
    (1, 512, 900, 255.5, 2, abi.FILT_SHEPP, 0, 0.0),        # the single-slice configuration
    (2, 64, 90, 31.5, 2, abi.FILT_RAMP, 0, 0.0),
    (3, 100, 120, 49.7, 3, abi.FILT_HAN, 0, 0.0),            # x2 zoom
    (4, 96, 100, 50.25, 4, abi.FILT_SHEPP, 0, 0.0),          # x4 zoom
    (5, 48, 60, 20.1, 5, abi.FILT_HAM, 0, 0.0),              # x8 zoom
    (6, 37, 45, 17.8, 2, abi.FILT_PARZN, 0, 0.0),            # odd width, partial tile
    (7, 200, 181, 10.4, 2, abi.FILT_SHEPP, 0, 0.0),          # centre far left: negative fx
    (8, 200, 181, 180.6, 2, abi.FILT_SHEPP, 0, 0.0),         # centre far right
    (9, 160, 150, 80.3, 2, abi.FILT_BUTER, abi.RQFLAGS_USEONLYEVENFRAMES, 0.7),
    (10, 160, 150, 79.9, 2, abi.FILT_SHEPP, abi.RQFLAGS_USEONLYODDFRAMES, -1.3),
    (11, 1000, 400, 499.3, 2, abi.FILT_SHEPP, 0, 0.0),       # not a multiple of the 64 tile
    (12, 300, 360, 150.0, 2, abi.FILT_RAMP, 0, 0.0),         # 360 views over 180 deg, integer centre
    (13, 4096, 24, 2050.8, 2, abi.FILT_SHEPP, 0, 0.0),       # 8192-point transform
    (14, 2048, 8, 1018.4, 4, abi.FILT_HAN, 0, 0.0),          # x4 zoom: 16384-point transform
]


def _gpu_slice(ri: ReconInfo, **kw) -> np.ndarray:
    ri.reset_output()
    return rv.reconstruct_slice(ri, **kw).copy()


@pytest.mark.parametrize("case", SLICE_CASES, ids=lambda c: f"W{c[1]}V{c[2]}c{c[3]}z{c[4]}")
def test_slice_bit_exact(gpu, oracle, case):
    seed, W, V, cen, interp, kind, flags, tilt = case
    ri = fbp_case(seed, W, V, cen, interp, kind=kind, flags=flags, tilt=tilt, skip_every=17, oracle=oracle)
    want = oracle.reconstruct(ri, threads=8)
    n_want = int(ri.nsino[0])
    got = _gpu_slice(ri)
    assert int(ri.nsino[0]) == n_want
    assert ri.ri.iStatus != abi.RECONST_INFO_ERROR
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} pixels differ"


def test_slice_full_size_bit_exact(gpu, oracle):
    """2048-pixel detector x 1800 views (the full-scale geometry), one slice, bit-exact."""
    ri = fbp_case(21, 2048, 1800, 1023.5 + 7.3, 2, oracle=oracle)
    want = oracle.reconstruct(ri, threads=16)
    got = _gpu_slice(ri, streams=True)
    assert np.array_equal(got, want)


def test_streams_and_repeat_calls(gpu, oracle):
    ri = fbp_case(30, 128, 100, 63.5, oracle=oracle)
    want = oracle.reconstruct(ri)
    for streams in (False, True, True, False):
        assert np.array_equal(_gpu_slice(ri, streams=streams), want)
    rv.lib().CudaReconstResourceFree(ri.ref, False)
    assert not ri.ri.stream1 and not ri.ri.d_p
    assert np.array_equal(_gpu_slice(ri), want)
    rv.lib().CudaReconstMemFree(ri.ref)


def test_worker_split_sums_to_whole(gpu, oracle):
    """iStartSino/iStepSino interleave views between workers (source/cudaReconstHost.cpp:712);
    the host-side sum of the partial slices equals the single-worker slice.  With one GPU
    every worker uses device 0, so the worker index is passed as idev only when it is 0."""
    ri = fbp_case(31, 96, 120, 47.2, oracle=oracle)
    want = oracle.reconstruct(ri)
    total = np.zeros_like(want)
    for w in range(3):
        rw = fbp_case(31, 96, 120, 47.2, oracle=oracle, iStartSino=w, iStepSino=3)
        rw.reset_output()
        rv.lib().CudaReconstHost(rw.ref, 0, False, False)
        assert rw.ri.iStatus != abi.RECONST_INFO_ERROR
        total += rw.out
    assert np.array_equal(total, want)


def _oracle_kept(oracle, ri: ReconInfo, old_center: float) -> np.ndarray:
    """The reference's SINOGRAMKEPT path: tables filtered at the old integer centre, geometry of
    the new centre with foffset + 16 * (int(new) - int(old)) (source/cudaReconst.cu:222)."""
    L = oracle.L
    d = ri.d
    F32P = C.POINTER(C.c_float)
    rd = abi.RvDims(d.ixdim, d.iZooming, d.iIntpDim, d.ndimp, d.ndim, d.ixdimp, d.ixdimh, d.ihoffset)
    L.rvo_filter_row.argtypes = [C.POINTER(abi.RvDims), C.c_double, C.POINTER(C.c_short), F32P, F32P, F32P, F32P, F32P]
    L.rvo_row_table.argtypes = [C.c_int, F32P, C.POINTER(C.c_int)]
    L.rvo_view_geometry.argtypes = [C.POINTER(abi.RvDims), C.c_double, C.c_float, C.c_float, F32P, F32P, F32P]
    L.rvo_backproject_view.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), C.c_int, C.c_int]
    tw = np.zeros(d.ndim, np.float32)
    L.rvo_fft_twiddles(d.ndimp, tw.ctypes.data_as(F32P), tw[d.ndim // 2:].ctypes.data_as(F32P))
    work = np.zeros(7 * d.ndim, np.float32)
    q = np.zeros(d.ixdimp, np.float32)
    igp = np.zeros(16 * d.ixdimp, np.int32)
    out = np.zeros((d.ixdimp, d.ixdimp), np.int32)
    shift = 16 * (int(ri.ri.center) - int(old_center))
    for i in range(len(ri.fdeg)):
        if not (ri.bInc[i] & 1):
            continue
        L.rvo_filter_row(C.byref(rd), old_center, ri.rowptrs[i], ri.fFilter.ctypes.data_as(F32P),
                         tw.ctypes.data_as(F32P), tw[d.ndim // 2:].ctypes.data_as(F32P), q.ctypes.data_as(F32P),
                         work.ctypes.data_as(F32P))
        L.rvo_row_table(d.ixdimp, q.ctypes.data_as(F32P), igp.ctypes.data_as(C.POINTER(C.c_int)))
        fc, fs, fo = C.c_float(), C.c_float(), C.c_float()
        L.rvo_view_geometry(C.byref(rd), ri.ri.center, float(ri.fdeg[i]), 0.0, C.byref(fc), C.byref(fs), C.byref(fo))
        foff = np.float32(fo.value) + np.float32(shift)
        L.rvo_backproject_view(d.ixdimp, fc.value, fs.value, float(foff), igp.ctypes.data_as(C.POINTER(C.c_int)),
                               out.ctypes.data_as(C.POINTER(C.c_int)), 0, d.ixdimp)
    return out


def test_sinogram_kept_integer_centre_shift(gpu, oracle):
    ri = fbp_case(40, 128, 120, 63.3, oracle=oracle)
    first = _gpu_slice(ri)
    assert np.array_equal(first, oracle.reconstruct(ri))
    assert ri.ri.iSinoCenter == 63
    ri.ri.dReconFlags |= abi.RQFLAGS_SINOGRAMKEPT
    ri.ri.center = 66.3
    got = _gpu_slice(ri)
    assert ri.ri.iSinoCenter == 63  # kept: the filtered views still belong to centre 63
    assert np.array_equal(got, _oracle_kept(oracle, ri, 63.3))


def test_empty_view_set(gpu, oracle):
    ri = fbp_case(41, 64, 30, 31.5, oracle=oracle)
    ri.bInc[:] = 0
    got = _gpu_slice(ri)
    assert not got.any() and int(ri.nsino[0]) == 0


def test_progress_callback_abort(gpu, oracle):
    """bReport: the hook is called every 20 views; returning true stops adding views."""
    calls = []

    def hook(ri_p, step, i, cur):
        calls.append(i)
        return i >= 40

    cb = abi.ProgressCallback(hook)
    rv.lib().RvSetProgressCallback(cb)
    try:
        ri = fbp_case(42, 64, 100, 31.5, oracle=oracle)
        got = _gpu_slice(ri, report=True)
    finally:
        rv.lib().RvSetProgressCallback(abi.ProgressCallback())
    assert calls == [0, 20, 40]
    ri2 = fbp_case(42, 64, 100, 31.5, oracle=oracle)
    ri2.bInc[40:] = 0
    assert np.array_equal(got, oracle.reconstruct(ri2))


@pytest.fixture(params=[(v, f) for f in (0, 1, 2) for v in range(22)], ids=lambda v: f"variant{v[0]}fmt{v[1]}")
def bp_variant(request, gpu):
    """Every back-projection variant and table format; restores the default afterwards."""
    L = rv.lib()
    old_v, old_p = C.c_int(), C.c_int()
    L.RvGetBackprojectionVariant(C.byref(old_v), C.byref(old_p))
    assert L.RvSetBackprojectionVariant(*request.param) == 0
    yield request.param
    L.RvSetBackprojectionVariant(old_v.value, old_p.value)


@pytest.mark.parametrize("W,V,cen,interp", [(512, 900, 255.5, 2), (200, 181, 10.4, 2), (200, 181, 180.6, 2),
                                            (96, 100, 50.25, 4), (1000, 400, 499.3, 2), (60, 64, 5.5, 5)])
def test_window_bound_holds(bp_variant, oracle, W, V, cen, interp):
    """The production kernel reads the staged table window without per-access checks; the
    checked twin counts any index outside the window, and must count none."""
    L = rv.lib()
    assert L.RvSetCheckedBackprojection(1) == 0
    try:
        ri = fbp_case(50, W, V, cen, interp, oracle=oracle, tilt=0.9)
        got = _gpu_slice(ri)
        assert L.RvGetWindowViolations() == 0
    finally:
        L.RvSetCheckedBackprojection(0)
    assert np.array_equal(got, oracle.reconstruct(ri, threads=8))


@pytest.mark.parametrize("case", SLICE_CASES[:8], ids=lambda c: f"W{c[1]}V{c[2]}c{c[3]}z{c[4]}")
def test_variants_bit_exact(bp_variant, oracle, case):
    seed, W, V, cen, interp, kind, flags, tilt = case
    ri = fbp_case(seed, W, V, cen, interp, kind=kind, flags=flags, tilt=tilt, skip_every=13, oracle=oracle)
    want = oracle.reconstruct(ri, threads=8)
    assert np.array_equal(_gpu_slice(ri), want)


# ---- normalisation (R1) ---------------------------------------------------------------------
@pytest.mark.parametrize("flags,drift,iflag", [(0, None, 0), (abi.RQFLAGS_ZERNIKE, None, 0),
                                               (abi.RQFLAGS_DRIFTPARAMS, "params", 0),
                                               (abi.RQFLAGS_DRIFTLIST, "list", 0), (0, None, abi.READTIF8bit)])
def test_sinogram_host_bit_exact(gpu, oracle, flags, drift, iflag):
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(60, 160, 90, 3, 79.4, n_ellipsoids=8, nflat_before=2, nflat_after=2)
    bInc = bInc.copy()
    bInc[10] |= abi.BINC_SKIP
    outs = []
    for who in ("gpu", "oracle"):
        r = raw.copy()
        ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=3, maxSinogrLen=raw.shape[0],
                       dReconFlags=flags, iFlag=iflag,
                       piDrift=(np.arange(raw.shape[0]) % 9 - 4) if drift == "list" else None)
        if drift == "params":
            ri.ri.drStart, ri.ri.drEnd, ri.ri.drX, ri.ri.drY = 8, 60, 9.6, -4.2
        if who == "gpu":
            rv.normalise(ri)
        else:
            oracle.generate_sinogram(ri)
        outs.append(r)
    assert np.array_equal(outs[0], outs[1])


# ---- fused stack path ---------------------------------------------------------------------------
def _stack_oracle(oracle, raw, bInc, fdeg, fexp, center, F, interp=2, flags=0):
    """Oracle of the stack path: GenerateSinogramThread on the raw buffer, then the CPU
    reconstruction of every slice (iOffset = slice)."""
    r = raw.copy()
    S = raw.shape[1]
    ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=S, maxSinogrLen=raw.shape[0])
    oracle.generate_sinogram(ri)
    outs = []
    for s in range(S):
        rs = ReconInfo(r.view(np.int16), fdeg, bInc, center=center, fFilter=F, iInterpolation=interp,
                       iMultiplex=S, iOffset=s, maxSinogrLen=r.shape[0] * S, nviews=raw.shape[0] - 1,
                       dReconFlags=flags)
        outs.append(oracle.reconstruct(rs, threads=8))
    return np.stack(outs)


@pytest.mark.parametrize("W,V,S,cen,interp,budget", [(256, 300, 4, 131.7, 2, None), (128, 150, 5, 60.2, 3, 1),
                                                     (200, 181, 3, 97.9, 2, None)])
def test_stack_ref_bit_exact(gpu, oracle, monkeypatch, W, V, S, cen, interp, budget):
    if budget is not None:
        monkeypatch.setenv("RV_TABLE_BUDGET_MB", str(budget))  # forces several slice batches
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(70, W, V, S, cen, n_ellipsoids=12, nflat_before=2, nflat_after=1)
    d = dims(W, interp)
    F = oracle.set_filter(abi.FILT_SHEPP, d.ndim)
    st = rv.Stack(ixdim=W, nframes=raw.shape[0] - 1, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp,
                  fFilter=F, iInterpolation=interp)
    got = st.run_host(raw)
    want = _stack_oracle(oracle, raw, bInc, fdeg, fexp, cen, F, interp)
    st.close()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("pieces,budget_mb", [(1, None), (3, 5), (4, 5), (5, 5), (64, None)])
def test_stack_host_pipeline_pieces(gpu, oracle, monkeypatch, pieces, budget_mb):
    """RvStackRunHost overlaps copies with kernels piece by piece; any piece size (and table
    batches of 4 slices under a 5 MB budget) must give the same slices as the oracle."""
    monkeypatch.setenv("RV_STACK_PIECES", str(pieces))
    if budget_mb is not None:
        monkeypatch.setenv("RV_TABLE_BUDGET_MB", str(budget_mb))
    W, V, S, cen = 128, 150, 10, 63.3
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(71, W, V, S, cen, n_ellipsoids=10)
    F = oracle.set_filter(abi.FILT_SHEPP, dims(W).ndim)
    st = rv.Stack(ixdim=W, nframes=raw.shape[0] - 1, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp,
                  fFilter=F)
    want = _stack_oracle(oracle, raw, bInc, fdeg, fexp, cen, F, 2)
    for _ in range(2):                       # a second call reuses buffers, streams and events
        got = st.run_host(raw)
        assert np.array_equal(got, want)
    # per piece a filter and one back-projection launch per slice-group form (triples, pairs)
    assert 2 <= st.launches() <= 3 * pieces
    st.close()


@pytest.mark.parametrize("S", [2, 3], ids=lambda s: f"S{s}")
@pytest.mark.parametrize("mode,tol", [(abi.MODE_LIN, 1e-5), (abi.MODE_LIN_F16, 1e-3), (abi.MODE_LIN_BF16, 8e-3)])
def test_stack_lin_modes_vs_fp64(gpu, oracle, mode, tol, S):
    """LIN modes: FP32 interpolation/accumulation with FP32/FP16/BF16 filtered rows; relative L2
    error against the FP64 end-to-end oracle, inside the reconstruction circle.  Two slices run
    as one slice pair; three as a pair plus a single slice (each with its own row scales)."""
    W, V, cen = 256, 300, 127.6
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(80, W, V, S, cen, n_ellipsoids=12, nflat_before=1, nflat_after=1)
    d = dims(W)
    F = oracle.set_filter(abi.FILT_SHEPP, d.ndim)
    st = rv.Stack(ixdim=W, nframes=raw.shape[0] - 1, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp,
                  fFilter=F, mode=mode)
    got = st.run_host(raw)
    st.close()
    r = raw.copy()
    ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=S, maxSinogrLen=raw.shape[0])
    oracle.generate_sinogram(ri)
    yy, xx = np.mgrid[:W, :W]
    circle = (xx - W / 2) ** 2 + (yy - W / 2) ** 2 < (0.45 * W) ** 2
    for s in range(S):
        rs = ReconInfo(r.view(np.int16), fdeg, bInc, center=cen, fFilter=F, iMultiplex=S, iOffset=s,
                       maxSinogrLen=r.shape[0] * S, nviews=raw.shape[0] - 1)
        ref64 = oracle.lin64(rs)
        err = rel_l2(got[s][circle], ref64[circle])
        assert err < tol, (mode, s, err)


# ---- R9 rescale -------------------------------------------------------------------------------
@pytest.mark.parametrize("W,V,cen,interp,binning", [(256, 300, 131.3, 2, 1), (128, 120, 60.4, 3, 1),
                                                    (200, 181, 99.0, 2, 2)])
def test_rescale_bit_exact(gpu, oracle, W, V, cen, interp, binning):
    torch = pytest.importorskip("torch")
    ri = fbp_case(95, W, V, cen, interp, oracle=oracle)
    sl = oracle.reconstruct(ri)
    d = rv.dims(W, interp)
    center_user = cen * binning - 0.5          # ri->center = (c + 0.5) / binning
    want, imin, imax = oracle.rescale(sl, d.ixdimp, center_user, d.iIntpDim, binning)
    dev = torch.from_numpy(np.stack([sl, sl[::-1].copy()])).cuda()
    out16 = torch.zeros(dev.shape, dtype=torch.int16, device="cuda")
    mm = np.zeros(4, np.int32)
    rc = rv.lib().RvRescaleSlices(C.c_void_p(dev.data_ptr()), 2, d.ixdimp, center_user, d.iIntpDim, binning,
                                  C.c_void_p(out16.data_ptr()), mm.ctypes.data_as(C.POINTER(C.c_int)), None)
    assert rc == 0, rv.last_error()
    got = dev.cpu().numpy()
    assert np.array_equal(got[0], want)
    assert (mm[0], mm[1]) == (imin, imax)
    want2, _, _ = oracle.rescale(sl[::-1], d.ixdimp, center_user, d.iIntpDim, binning)
    assert np.array_equal(got[1], want2)
    assert np.array_equal(out16.cpu().numpy().view(np.uint16)[0].astype(np.int32), want)


# ---- R11 centre methods -----------------------------------------------------------------------
@pytest.mark.parametrize("seed,W,S,V,cen,off", [(1, 256, 48, 180, 131.3, 0), (3, 300, 100, 360, 140.25, 0),
                                                (4, 160, 30, 100, 120.2, 120), (6, 2048, 64, 60, 1030.6, 0)])
def test_get_axis_matches_oracle(gpu, oracle, seed, W, S, V, cen, off):
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(seed, W, V, S, cen, n_ellipsoids=12)
    s0, s1, fl = (np.ascontiguousarray(raw[i]) for i in (1, V, 0))
    want = oracle.get_axis(s0, s1, fl, off)
    a, b, o = C.c_double(), C.c_double(), C.c_double()
    rc = rv.lib().RvGetAxis(s0.ctypes.data, s1.ctypes.data, fl.ctypes.data, W, S, off, C.byref(a), C.byref(b), C.byref(o))
    assert rc == 0, rv.last_error()
    assert (a.value, b.value, o.value) == want


@pytest.mark.parametrize("seed,W,V,cen", [(7, 256, 300, 131.3), (8, 512, 600, 247.8)])
def test_centre_sweep(gpu, oracle, seed, W, V, cen):
    sino, fdeg = phantom.sinogram_2d(seed, W, V, cen)
    F = oracle.set_filter(abi.FILT_SHEPP, rv.dims(W).ndim)
    centres = np.round(cen) + np.arange(-4.0, 4.01, 0.5)
    scores = np.zeros(len(centres))
    best = C.c_double()
    rc = rv.lib().RvCentreSweep(sino.ctypes.data, V, W, 2, fdeg.ctypes.data_as(C.POINTER(C.c_float)), 0.0,
                                F.ctypes.data_as(C.POINTER(C.c_float)),
                                centres.ctypes.data_as(C.POINTER(C.c_double)), len(centres),
                                scores.ctypes.data_as(C.POINTER(C.c_double)), C.byref(best))
    assert rc == 0, rv.last_error()
    bInc = np.ones(V, np.int8)
    for i in (0, int(np.argmin(scores)), len(centres) - 1):
        ri = ReconInfo(sino, fdeg, bInc, center=float(centres[i]), fFilter=F)
        want = oracle.tv_score(oracle.reconstruct(ri))
        assert abs(scores[i] - want) <= 1e-9 * want
    assert abs(best.value - cen) <= 0.25, (best.value, cen)


def test_dropin_staged_copies_equal_direct(gpu, oracle, tmp_path):
    """Where the device reads pageable host memory directly, CudaReconstHost takes the sinogram
    rows from the caller's row pointers and writes the slice with a kernel; RV_NO_HOST_DIRECT=1
    forces the staged copies.  Both give the oracle's slice (the staged run in a subprocess,
    since the choice is made once per process)."""
    import subprocess
    import sys
    ri = fbp_case(41, 256, 240, 127.3, 2, oracle=oracle)
    want = oracle.reconstruct(ri, threads=8)
    assert np.array_equal(_gpu_slice(ri), want)
    script = (
        "import numpy as np, sys\n"
        "sys.path.insert(0, '.')\n"
        "import recview_gb300 as rv\n"
        "from tests.rvtest import Oracle, fbp_case\n"
        "o = Oracle()\n"
        "ri = fbp_case(41, 256, 240, 127.3, 2, oracle=o)\n"
        "ri.reset_output()\n"
        f"np.save(r'{tmp_path / 'staged.npy'}', rv.reconstruct_slice(ri).copy())\n"
    )
    import os
    env = dict(os.environ, RV_NO_HOST_DIRECT="1")
    r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert np.array_equal(np.load(tmp_path / "staged.npy"), want)


def test_sinogram_staged_copies_equal_direct(gpu, oracle, tmp_path):
    """CudaSinogramHost normalises the caller's rows in place through their pointers where the
    device reads pageable host memory; RV_NO_HOST_DIRECT=1 stages them.  Both equal the oracle
    (drift list, so the shifted reads of the in-place row are covered)."""
    import os
    import subprocess
    import sys
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(61, 160, 90, 2, 79.4, n_ellipsoids=8, nflat_before=2, nflat_after=2)
    np.save(tmp_path / "raw.npy", raw)
    drift = np.arange(raw.shape[0]) % 9 - 4
    r = raw.copy()
    ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=2, maxSinogrLen=raw.shape[0],
                   dReconFlags=abi.RQFLAGS_DRIFTLIST, piDrift=drift)
    oracle.generate_sinogram(ri)
    want = r
    for off in ("0", "1"):
        script = (
            "import numpy as np, sys\n"
            "sys.path.insert(0, '.')\n"
            "import recview_gb300 as rv\n"
            "from recview_gb300 import abi, phantom\n"
            "from recview_gb300.reconst import ReconInfo\n"
            f"raw = np.load(r'{tmp_path / 'raw.npy'}')\n"
            f"_, bInc, fdeg, fexp, _ = phantom.raw_stack(61, 160, 90, 2, 79.4, n_ellipsoids=8, nflat_before=2, nflat_after=2)\n"
            "r = raw.copy()\n"
            "ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=2, maxSinogrLen=raw.shape[0],\n"
            "               dReconFlags=abi.RQFLAGS_DRIFTLIST, piDrift=np.arange(raw.shape[0]) % 9 - 4)\n"
            "rv.normalise(ri)\n"
            f"np.save(r'{tmp_path}' + '/out{off}.npy', r)\n"
        )
        env = dict(os.environ, RV_NO_HOST_DIRECT=off)
        p = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=600)
        assert p.returncode == 0, p.stderr[-2000:]
        assert np.array_equal(np.load(tmp_path / f"out{off}.npy"), want), off
