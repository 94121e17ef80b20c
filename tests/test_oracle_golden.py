"""The oracle restatement against golden vectors produced by the reference's own sources
(tests/golden/make_golden.py).  CPU only; runs everywhere, including where the reference
checkout is absent."""
import numpy as np
import pytest

from recview_gb300 import abi
from recview_gb300.reconst import ReconInfo


def test_reconst_info_layout_matches_reference(golden):
    import ctypes as C
    mine = [getattr(abi.RECONST_INFO, n).offset for n in abi.FIELD_ORDER] + [C.sizeof(abi.RECONST_INFO)]
    assert list(golden["layout"]) == mine


@pytest.mark.parametrize("kind", range(5))
def test_filter_tables(golden, oracle, kind):
    for cut in (0.5, 0.35, 1.0):
        for ndim in (64, 1024):
            want = golden[f"filter_{kind}_{cut}_{ndim}"]
            got = oracle.set_filter(kind, ndim, cut, 3.0)
            if kind == abi.FILT_BUTER:
                # powf is the platform's; allow one float ulp
                assert np.all(np.abs(got.view(np.int32) - want.view(np.int32)) <= 1)
            else:
                assert np.array_equal(got.view(np.int32), want.view(np.int32)), (kind, cut, ndim)


@pytest.mark.parametrize("npow", [3, 6, 9, 12])
@pytest.mark.parametrize("inverse", [0, 1])
def test_fft_bit_exact(golden, oracle, npow, inverse):
    re, im = golden[f"fft_in_{npow}"]
    a, b = oracle.fft(npow, inverse, re, im)
    want = golden[f"fft_out_{npow}_{inverse}"]
    assert np.array_equal(a.view(np.int32), want[0].view(np.int32))
    assert np.array_equal(b.view(np.int32), want[1].view(np.int32))


CASES = ["plain64", "ramp64_off", "han48_tilt", "ham40_even", "parz40_odd", "zoom2_40", "zoom4_24",
         "zoom8_12", "odd37"]


@pytest.mark.parametrize("name", CASES)
def test_fbp_bit_exact(golden, oracle, name):
    W, V, cen, interp, kind, cut, flags, tilt, nsino = golden[f"fbp_{name}_params"]
    ri = ReconInfo(golden[f"fbp_{name}_sino"], golden[f"fbp_{name}_fdeg"], golden[f"fbp_{name}_binc"],
                   center=float(cen), fFilter=golden[f"fbp_{name}_filter"], iInterpolation=int(interp),
                   dReconFlags=int(flags), tilt=float(tilt))
    out = oracle.reconstruct(ri)
    assert int(ri.nsino[0]) == int(nsino)
    assert np.array_equal(out, golden[f"fbp_{name}_out"])


@pytest.mark.parametrize("name", ["sino_plain", "sino_zernike", "sino_8bit"])
def test_normalisation_bit_exact(golden, oracle, name):
    flags, iflag = golden[f"{name}_params"]
    raw = golden[f"{name}_raw"].copy()
    ri = ReconInfo(raw.view(np.int16), golden[f"{name}_fdeg"], golden[f"{name}_binc"], center=0,
                   fexp=golden[f"{name}_fexp"], iMultiplex=raw.shape[1], maxSinogrLen=raw.shape[0],
                   dReconFlags=int(flags), iFlag=int(iflag))
    assert oracle.generate_sinogram(ri) == 0
    assert np.array_equal(raw, golden[f"{name}_out"])


def test_oracle_threads_equal_single(oracle):
    from tests.rvtest import fbp_case
    ri = fbp_case(7, 96, 120, 47.3, oracle=oracle)
    one = oracle.reconstruct(ri, threads=1)
    many = oracle.reconstruct(ri, threads=5)
    assert np.array_equal(one, many)


@pytest.mark.parametrize("name", ["axis_a", "axis_b", "axis_off"])
def test_get_axis_bit_exact(golden, oracle, name):
    s0, s1, fl = golden[f"{name}_frames"]
    off, c, g = golden[f"{name}_params"]
    got = oracle.get_axis(s0, s1, fl, int(off))
    assert got[0] == c and got[1] == g


def test_lin64_threads_equal_serial(oracle):
    """The row-band parallel FP64 oracle sums every pixel exactly as the serial one."""
    from tests.rvtest import fbp_case
    ri = fbp_case(3, 96, 70, 47.3, oracle=oracle)
    assert np.array_equal(oracle.lin64(ri), oracle.lin64(ri, threads=3))


@pytest.mark.parametrize("name", ["bin2_trim3", "bin4_trim5", "bin2_notrim", "bin1_trim7", "bin4_odd"])
def test_strip_assembly(golden, oracle, name):
    """Trim and bin x bin averaging of raw frames (CGazoDoc::GenerateSinogram's strip assembly)."""
    F, T, interp, S = (int(v) for v in golden[f"{name}_params"])
    got = oracle.bin_frames(golden[f"{name}_frames"], F, T, interp, S)
    assert np.array_equal(got, golden[f"{name}_out"])


def test_strip_assembly_rejects_bad_trim(oracle):
    assert oracle.L.rvo_bin_width(40, 20, 1) == -1     # trim not below half the frame width
    assert oracle.L.rvo_bin_width(40, -1, 2) == -1
    assert oracle.L.rvo_bin_width(41, 3, 1) == (41 - 6) // 2
