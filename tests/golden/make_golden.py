"""Generates tests/golden/golden.npz from the reference sources compiled by oracle/build_ref.sh.

Run in a checkout that has the reference (the GPU machine does not): the fixtures then pin the
oracle restatement everywhere.  Inputs are stored with the outputs, so the fixtures do not
depend on the phantom generator's floating-point behaviour on another platform.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
import zlib
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from recview_gb300 import abi, phantom  # noqa: E402
from recview_gb300.build import build_oracle, build_ref  # noqa: E402
from recview_gb300.reconst import ReconInfo, dims  # noqa: E402

F32P = C.POINTER(C.c_float)

# (name, ixdim, nviews, center, iInterpolation, filter kind, cutoff, flags, tilt)
FBP_CASES = [
    ("plain64", 64, 90, 31.5, 2, abi.FILT_SHEPP, 0.5, 0, 0.0),
    ("ramp64_off", 64, 75, 29.3, 2, abi.FILT_RAMP, 0.5, 0, 0.0),
    ("han48_tilt", 48, 60, 24.75, 2, abi.FILT_HAN, 0.5, 0, 0.35),
    ("ham40_even", 40, 64, 20.2, 2, abi.FILT_HAM, 0.4, abi.RQFLAGS_USEONLYEVENFRAMES, 0.0),
    ("parz40_odd", 40, 64, 19.9, 2, abi.FILT_PARZN, 0.5, abi.RQFLAGS_USEONLYODDFRAMES, 0.0),
    ("zoom2_40", 40, 50, 21.6, 3, abi.FILT_SHEPP, 0.5, 0, 0.0),
    ("zoom4_24", 24, 40, 11.3, 4, abi.FILT_RAMP, 0.5, 0, 0.0),
    ("zoom8_12", 12, 30, 6.45, 5, abi.FILT_HAN, 0.5, 0, 0.0),
    ("odd37", 37, 45, 17.8, 2, abi.FILT_SHEPP, 0.5, 0, 0.0),
]

# (name, seed, frame width, iInterpolation, trim, slices, views over 360, centre, centre gradient, edit)
OCT_CASES = [
    ("oct_right_lo", 31, 64, 2, 0, 2, 40, 50.8, 0.0, ""),
    ("oct_right_hi", 32, 64, 2, 0, 2, 40, 52.3, 0.15, ""),
    ("oct_left_lo", 33, 64, 2, 0, 2, 40, 9.6, 0.0, ""),
    ("oct_left_hi", 34, 64, 2, 0, 3, 40, 11.2, -0.2, ""),
    ("oct_bin2", 35, 96, 1, 0, 2, 36, 80.1, 0.0, ""),
    ("oct_trim", 36, 64, 2, 2, 2, 40, 49.4, 0.0, ""),
    ("oct_skip", 37, 48, 2, 0, 1, 30, 39.7, 0.0, "skip"),
    ("oct_e21051", 38, 32, 2, 0, 1, 20, 26.0, 0.0, "no180"),
    ("oct_e21052", 39, 32, 2, 0, 1, 20, 26.0, 0.0, "nopartner"),
]


# (name, seed, raw frame width, trim, iInterpolation (0: bin 4, 1: bin 2, 2: none), slices)
BIN_CASES = [
    ("bin2_trim3", 41, 37, 3, 1, 2),
    ("bin4_trim5", 42, 64, 5, 0, 3),
    ("bin2_notrim", 43, 50, 0, 1, 1),
    ("bin1_trim7", 44, 40, 7, 2, 2),
    ("bin4_odd", 45, 45, 2, 0, 1),
]


def main() -> None:
    ref_path = build_ref()
    if ref_path is None:
        raise SystemExit("reference checkout not found; fixtures can only be generated where it exists")
    ref = C.CDLL(str(ref_path))
    ora = C.CDLL(str(build_oracle()))
    for f in (ref.rvref_set_filter, ora.rvo_set_filter):
        f.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, F32P]
    out: dict[str, np.ndarray] = {}
    # layout of RECONST_INFO in the reference header
    offs = (C.c_size_t * 80)()
    n = ref.rvref_reconstinfo_layout(offs, 80)
    out["layout"] = np.array(offs[:n], dtype=np.int64)
    # filter tables
    for kind in range(5):
        for cut in (0.5, 0.35, 1.0):
            for ndim in (64, 1024):
                t = np.zeros(ndim, np.float32)
                ref.rvref_set_filter(kind, cut, 3.0, ndim, t.ctypes.data_as(F32P))
                out[f"filter_{kind}_{cut}_{ndim}"] = t
    # FFTs
    ref.rvref_fft.argtypes = [C.c_int, C.c_int, F32P, F32P]
    for npow in (3, 6, 9, 12):
        n = 1 << npow
        rng = np.random.default_rng(100 + npow)
        re = (rng.normal(size=n) * 100).astype(np.float32)
        im = rng.normal(size=n).astype(np.float32)
        out[f"fft_in_{npow}"] = np.stack([re, im])
        for inv in (0, 1):
            a, b = re.copy(), im.copy()
            ref.rvref_fft(npow, inv, a.ctypes.data_as(F32P), b.ctypes.data_as(F32P))
            out[f"fft_out_{npow}_{inv}"] = np.stack([a, b])
    # full FBP cases
    for name, W, V, cen, interp, kind, cut, flags, tilt in FBP_CASES:
        sino, fdeg = phantom.sinogram_2d(zlib.crc32(name.encode()) % 1000, W, V, cen)
        d = dims(W, interp)
        F = np.zeros(d.ndim, np.float32)
        ref.rvref_set_filter(kind, cut, 2.0, d.ndim, F.ctypes.data_as(F32P))
        bInc = np.ones(V, np.int8)
        bInc[::11] = 0
        res = []
        for lib, fn in ((ref, "rvref_fbp"), (ora, "rvo_reconstruct")):
            ri = ReconInfo(sino, fdeg, bInc, center=cen, fFilter=F, iInterpolation=interp,
                           dReconFlags=flags, tilt=tilt)
            getattr(lib, fn)(ri.ref)
            res.append((ri.out.copy(), int(ri.nsino[0])))
        assert np.array_equal(res[0][0], res[1][0]), f"oracle differs from the reference on {name}"
        out[f"fbp_{name}_sino"] = sino
        out[f"fbp_{name}_fdeg"] = fdeg
        out[f"fbp_{name}_binc"] = bInc
        out[f"fbp_{name}_filter"] = F
        out[f"fbp_{name}_out"] = res[0][0]
        out[f"fbp_{name}_params"] = np.array([W, V, cen, interp, kind, cut, flags, tilt, res[0][1]])
    # normalisation cases (GenerateSinogramThread)
    for name, seed, flags, iflag in (("sino_plain", 1, 0, 0), ("sino_zernike", 2, abi.RQFLAGS_ZERNIKE, 0),
                                     ("sino_8bit", 3, 0, abi.READTIF8bit)):
        raw, bInc, fdeg, fexp, _ = phantom.raw_stack(seed, 48, 30, 2, 23.7, n_ellipsoids=5,
                                                     nflat_before=2, nflat_after=2)
        bInc = bInc.copy()
        bInc[6] |= abi.BINC_SKIP
        r = raw.copy()
        ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=2,
                       maxSinogrLen=raw.shape[0], dReconFlags=flags, iFlag=iflag)
        ref.rvref_gen_sinogram(ri.ref)
        out[f"{name}_raw"] = raw
        out[f"{name}_binc"] = bInc
        out[f"{name}_fdeg"] = fdeg
        out[f"{name}_fexp"] = fexp
        out[f"{name}_out"] = r
        out[f"{name}_params"] = np.array([flags, iflag])
    # GetAxis (centre estimate from the 0 / ~180 degree frames and a flat)
    U16P = C.POINTER(C.c_ushort)
    ref.rvref_get_axis.argtypes = [U16P, U16P, U16P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]
    for name, seed, W, S, V, cen, off in (("axis_a", 11, 160, 48, 120, 81.3, 0), ("axis_b", 12, 128, 40, 90, 58.7, 0),
                                          ("axis_off", 13, 160, 24, 120, 110.4, 110)):
        raw, bInc, fdeg, fexp, _ = phantom.raw_stack(seed, W, V, S, cen, n_ellipsoids=10)
        s0, s1, fl = (np.ascontiguousarray(raw[i]) for i in (1, V, 0))
        a, b = C.c_double(), C.c_double()
        ref.rvref_get_axis(s0.ctypes.data_as(U16P), s1.ctypes.data_as(U16P), fl.ctypes.data_as(U16P), W, S, off,
                           C.byref(a), C.byref(b))
        out[f"{name}_frames"] = np.stack([s0, s1, fl])
        out[f"{name}_params"] = np.array([off, a.value, b.value])
    # 16-bit TIFF files
    ref.rvref_write_tif16.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_char_p, C.c_void_p, C.c_int]
    rng = np.random.default_rng(5)
    for name, h, w, desc, art in (("tif_a", 7, 9, b"1800\t3.250000\t0.1\t0.2\t1023.5\t6\t55.111697\t0.461227 ",
                                   b"SP-uCT, gazoView"), ("tif_b", 4, 5, b"ab", b"")):
        img = rng.integers(-100, 70000, (h, w)).astype(np.int32)
        buf = np.zeros(1 << 16, np.uint8)
        n = ref.rvref_write_tif16(img.ctypes.data, h, w, desc, art, buf.ctypes.data, buf.size)
        out[f"{name}_img"] = img
        out[f"{name}_desc"] = np.frombuffer(desc, np.uint8)
        out[f"{name}_artist"] = np.frombuffer(art, np.uint8)
        out[f"{name}_bytes"] = buf[:n].copy()
    # offset-CT stitching (360-degree frames, axis near an edge)
    SP = C.POINTER(C.c_short)
    ref.rvref_offset_ct.argtypes = [SP, C.c_longlong, SP, C.c_longlong, C.c_char_p, F32P, C.c_int, C.c_int,
                                    C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int]
    for name, seed, F, interp, T, M, V, cen, dcent, knock in OCT_CASES:
        B = 4 if interp == 0 else (2 if interp == 1 else 1)
        ixlen = F // B
        sino, bInc, fdeg = phantom.offset_ct_sinogram(seed, ixlen, V, M, cen / B, n_ellipsoids=6)
        if knock == "skip":
            bInc[[3, 7, V // 2 + 2]] = 0
        elif knock == "no180":
            fdeg[fdeg > 180] = 180.0
        elif knock == "nopartner":
            bInc[V - 1:V + 2] = 0
        nf = sino.shape[0]
        rows = np.ascontiguousarray(sino.reshape(nf * M, ixlen))
        width = (2 * F) // B
        nof = max(1, int(np.argmax(fdeg[:nf - 1] > 180)))
        res = np.zeros((nof * M, width), np.int16)
        rc = ref.rvref_offset_ct(rows.ctypes.data_as(SP), ixlen, res.ctypes.data_as(SP), width, bInc.tobytes(),
                                 fdeg.ctypes.data_as(F32P), nf, M, cen, dcent, interp, T, F, 2 * F)
        out[f"{name}_rows"] = rows
        out[f"{name}_binc"] = bInc
        out[f"{name}_fdeg"] = fdeg
        out[f"{name}_params"] = np.array([F, 2 * F, interp, T, M, cen, dcent, rc])
        out[f"{name}_out"] = res
    # strip assembly: trim and bin x bin averages of raw frames (CGazoDoc::GenerateSinogram)
    from tests.rvtest import ref_bin_frames
    Lr = C.CDLL(str(ref_path))
    Lr.rvref_bin_strip.argtypes = [C.POINTER(C.c_short), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(C.POINTER(C.c_short))]
    for name, seed, F, T, interp, S in BIN_CASES:
        rng = np.random.default_rng(seed)
        B = 4 if interp == 0 else (2 if interp == 1 else 1)
        frames = rng.integers(0, 65536, (3, S * B, F)).astype(np.uint16)
        frames[0, :, :4] = 65535                      # sums near the top of the range
        out[f"{name}_frames"] = frames
        out[f"{name}_params"] = np.array([F, T, interp, S])
        out[f"{name}_out"] = ref_bin_frames(Lr, frames, F, T, interp, S)
    dst = Path(__file__).with_name("golden.npz")
    np.savez_compressed(dst, **out)
    print(f"wrote {dst} ({dst.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
