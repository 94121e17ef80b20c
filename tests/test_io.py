"""Output files: RecView's 16-bit TIFF byte for byte, and the physical-scale fields."""
import ctypes as C

import numpy as np
import pytest

from tests.rvtest import ref_lib

REF = ref_lib()


def tiff_bytes(rvlib, img, desc, artist):
    img = np.ascontiguousarray(img, np.int32)
    n = rvlib.RvTiff16Bytes(img.ctypes.data, img.shape[0], img.shape[1], desc, artist, None, 0)
    buf = np.zeros(n, np.uint8)
    assert rvlib.RvTiff16Bytes(img.ctypes.data, img.shape[0], img.shape[1], desc, artist, buf.ctypes.data, n) == n
    return buf


@pytest.mark.parametrize("name", ["tif_a", "tif_b"])
def test_tiff_matches_golden(rvlib, golden, name):
    img = golden[f"{name}_img"]
    desc = golden[f"{name}_desc"].tobytes()
    art = golden[f"{name}_artist"].tobytes()
    assert np.array_equal(tiff_bytes(rvlib, img, desc, art), golden[f"{name}_bytes"])


@pytest.mark.skipif(REF is None, reason="reference build not present")
@pytest.mark.parametrize("h,w,desc", [(16, 16, b""), (3, 200, b"x" * 300), (33, 17, b"12\t0.5\t1.0\t2.0\t3.0\t1 ")])
def test_tiff_matches_reference_writer(rvlib, h, w, desc):
    img = np.random.default_rng(h * w).integers(-5, 66000, (h, w)).astype(np.int32)
    buf = np.zeros(1 << 20, np.uint8)
    n = REF.rvref_write_tif16(img.ctypes.data, h, w, desc, b"SP-uCT, gazoView", buf.ctypes.data, buf.size)
    assert np.array_equal(tiff_bytes(rvlib, img, desc, None), buf[:n])


def test_tiff_file_roundtrip(rvlib, tmp_path):
    img = (np.arange(12 * 10) % 65535).reshape(12, 10).astype(np.int32)
    path = tmp_path / "slice.tif"
    assert rvlib.RvWriteTiff16(str(path).encode(), img.ctypes.data, 12, 10, b"desc", None) == 0
    data = np.frombuffer(path.read_bytes(), np.uint8)
    assert data[:2].tobytes() == b"II" and int(data[2]) == 42
    px = np.frombuffer(data[8:8 + 12 * 10 * 2].tobytes(), "<u2").reshape(12, 10)
    assert np.array_equal(px, img.astype(np.uint16))


def test_pixel_scale_and_description(rvlib):
    base, div = C.c_float(), C.c_float()
    assert rvlib.RvPixelScale(1800, 3.25, 1, 1, -1200, 98000, 0, C.byref(base), C.byref(div)) == 0
    sf = 6.2831853 * 10000.0 / (3.25 * 1)
    sc = sf / (3000 * 100 * 1800)
    assert base.value == np.float32(sc * 1 * -1200)
    assert div.value == np.float32(65534 / sc / (98000 + 1200) / 1)
    out = C.create_string_buffer(256)
    assert rvlib.RvImageDescription(out, 256, 1800, 3.25, div.value, base.value, 1023.5, 5) == 0
    assert out.value.decode().split("\t")[5] == "6" and out.value.decode().endswith("0.461227 ")
