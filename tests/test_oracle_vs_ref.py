"""Randomised parity of the oracle restatement against the reference sources built here
(oracle/build_ref.sh).  Skipped where the reference checkout is absent (e.g. on the GPU machine);
the golden fixtures cover those machines."""
import ctypes as C

import numpy as np
import pytest

from recview_gb300 import abi, phantom
from recview_gb300.reconst import ReconInfo
from tests.rvtest import fbp_case, ref_lib

REF = ref_lib()
pytestmark = pytest.mark.skipif(REF is None, reason="reference build not present")


@pytest.mark.parametrize("seed,W,V,cen,interp", [
    (0, 80, 100, 39.5, 2), (1, 77, 91, 41.2, 2), (2, 50, 64, 20.9, 3), (3, 33, 40, 16.1, 4),
    (4, 128, 160, 70.7, 2), (5, 20, 24, 9.99, 5), (6, 64, 90, 10.4, 2), (7, 64, 90, 52.6, 2)])
def test_fbp_random(oracle, seed, W, V, cen, interp):
    ri = fbp_case(seed, W, V, cen, interp, skip_every=9, oracle=oracle)
    a = oracle.reconstruct(ri)
    ri.reset_output()
    REF.rvref_fbp(C.byref(ri.ri))
    assert np.array_equal(a, ri.out)


def test_fbp_all_filters(oracle):
    for kind in range(6):
        ri = fbp_case(11 + kind, 48, 50, 23.4, kind=kind, oracle=oracle)
        a = oracle.reconstruct(ri)
        ri.reset_output()
        REF.rvref_fbp(C.byref(ri.ri))
        assert np.array_equal(a, ri.out), kind


@pytest.mark.parametrize("flags,drift", [(0, None), (abi.RQFLAGS_DRIFTPARAMS, "params"),
                                         (abi.RQFLAGS_DRIFTLIST, "list"), (abi.RQFLAGS_ZERNIKE, None)])
def test_normalisation_random(oracle, flags, drift):
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(3, 64, 40, 3, 31.7, n_ellipsoids=5, nflat_before=2,
                                                 nflat_after=3)
    outs = []
    for fn in ("ora", "ref"):
        r = raw.copy()
        ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=3,
                       maxSinogrLen=raw.shape[0], dReconFlags=flags,
                       piDrift=(np.arange(raw.shape[0]) % 7 - 3) if drift == "list" else None)
        if drift == "params":
            ri.ri.drStart, ri.ri.drEnd, ri.ri.drX, ri.ri.drY = 5, 30, 6.2, -2.5
        if fn == "ora":
            oracle.generate_sinogram(ri)
        else:
            REF.rvref_gen_sinogram(C.byref(ri.ri))
        outs.append(r)
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("seed,W,S,V,cen,off", [(1, 256, 48, 180, 131.3, 0), (2, 200, 40, 90, 97.8, 0),
                                                (3, 300, 100, 360, 140.25, 0), (4, 160, 30, 100, 120.2, 120),
                                                (5, 160, 30, 100, 40.7, 40)])
def test_get_axis_random(oracle, seed, W, S, V, cen, off):
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(seed, W, V, S, cen, n_ellipsoids=12)
    s0, s1, fl = (np.ascontiguousarray(raw[i]) for i in (1, V, 0))
    a, b = C.c_double(), C.c_double()
    U16P = C.POINTER(C.c_ushort)
    REF.rvref_get_axis(s0.ctypes.data_as(U16P), s1.ctypes.data_as(U16P), fl.ctypes.data_as(U16P), W, S, off,
                       C.byref(a), C.byref(b))
    got = oracle.get_axis(s0, s1, fl, off)
    assert (got[0], got[1]) == (a.value, b.value)


@pytest.mark.parametrize("seed", range(6))
def test_strip_assembly_random(oracle, seed):
    from tests.rvtest import ref_bin_frames
    rng = np.random.default_rng(300 + seed)
    interp = int(rng.choice([0, 1, 2, 3]))
    B = 4 if interp == 0 else (2 if interp == 1 else 1)
    F = int(rng.integers(8 * B, 90))
    T = int(rng.choice([0, 0, 1, 2, 5])) if F > 12 else 0
    S = int(rng.integers(1, 4))
    frames = rng.integers(0, 65536, (4, S * B, F)).astype(np.uint16)
    assert np.array_equal(oracle.bin_frames(frames, F, T, interp, S), ref_bin_frames(REF, frames, F, T, interp, S))
