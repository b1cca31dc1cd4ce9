"""Radiance .hdr codec (CPU): round trips, run-length and flat scanlines, and
the reference's own shipped bake output."""
import os

import numpy as np
import pytest

from althea_gb300 import hdr

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _quantise_bound(a):
    # RGBE keeps 8 mantissa bits of the largest channel: absolute step
    # max(r,g,b) * 2^-7 at worst (truncation), per pixel.
    return np.max(a[..., :3], axis=-1, keepdims=True) * 2.0 ** -7 + 1e-30


@pytest.mark.parametrize("w,h", [(37, 5), (256, 3), (4, 6), (8, 2)])
def test_round_trip(tmp_path, w, h):
    rng = np.random.default_rng(w * h)
    a = np.exp(rng.normal(0, 3, size=(h, w, 4))).astype(np.float32)
    a[0, : min(3, w)] = 0.0  # zeros
    a[-1, -1, :3] = [1e6, 2.5e5, 3.0]  # a sun
    a[..., 3] = 1.0
    p = str(tmp_path / "x.hdr")
    hdr.write_hdr(p, a)
    b = hdr.read_hdr(p)
    assert b.shape == (h, w, 4)
    assert np.all(b[..., 3] == 1.0)
    assert np.all(np.abs(b[..., :3] - a[..., :3]) <= _quantise_bound(a))
    # decoding then re-encoding an RGBE image is exact
    p2 = str(tmp_path / "y.hdr")
    hdr.write_hdr(p2, b)
    assert np.array_equal(hdr.read_hdr(p2), b)


def test_runs_compress_flat_regions(tmp_path):
    a = np.ones((4, 512, 4), np.float32)
    p = str(tmp_path / "flat.hdr")
    hdr.write_hdr(p, a)
    assert os.path.getsize(p) < 512 * 4 * 4 // 10  # run-length scanlines
    assert np.array_equal(hdr.read_hdr(p), a)


def test_reads_reference_bake_output(tmp_path):
    p = os.path.join(GOLD, "ref_LuxuryRoom_Prefiltered5.hdr")
    img = hdr.read_hdr(p)
    assert img.shape == (64, 128, 4)  # 4096 >> 5 by 2048 >> 5
    assert np.isfinite(img).all() and (img[..., :3] >= 0).all() and img[..., :3].max() > 0
    # re-encoding the decoded pixels reproduces them exactly
    q = str(tmp_path / "again.hdr")
    hdr.write_hdr(q, img)
    assert np.array_equal(hdr.read_hdr(q), img)


def test_rejects_non_radiance(tmp_path):
    p = tmp_path / "bad.hdr"
    p.write_bytes(b"P6\n1 1\n255\n\x00\x00\x00")
    from althea_gb300 import ibl
    with pytest.raises(ibl.IBLError):
        hdr.read_hdr(str(p))


def test_reads_crlf_headers(tmp_path):
    """Header lines ending in \\r\\n (text-mode writers on Windows) read the
    same as \\n ones; the pixel data is binary either way."""
    a = np.full((3, 16, 4), 0.75, np.float32)
    a[..., 3] = 1.0
    p = tmp_path / "lf.hdr"
    hdr.write_hdr(str(p), a)
    raw = p.read_bytes()
    cut = raw.index(b"+X 16\n") + len(b"+X 16\n")
    crlf = tmp_path / "crlf.hdr"
    crlf.write_bytes(raw[:cut].replace(b"\n", b"\r\n") + raw[cut:])
    assert np.array_equal(hdr.read_hdr(str(crlf)), hdr.read_hdr(str(p)))


def _rle_file(w, h, body):
    return b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n" % (h, w) + body


@pytest.mark.parametrize("body", [
    bytes([2, 2, 0, 16]) + bytes([128 + 17, 1]),            # a run past the row's end
    bytes([2, 2, 0, 16]) + bytes([20]) + bytes(20),         # literals past the row's end
    bytes([2, 2, 0, 16]) + bytes([0]),                      # a zero-length literal
    bytes([2, 2, 0, 16]) + bytes([128 + 16, 1, 128 + 16]),  # stops inside a run
    b"",                                                    # no pixels at all
    bytes(16 * 4 - 1),                                      # a flat row one byte short
])
def test_corrupt_pixels_are_refused(tmp_path, body):
    from althea_gb300 import ibl
    p = tmp_path / "corrupt.hdr"
    p.write_bytes(_rle_file(16, 1, body))
    with pytest.raises(ibl.IBLError) as e:
        hdr.read_hdr(str(p))
    assert e.value.status == ibl.ERR_INVALID_ARGUMENT


def test_hand_made_rle_row_decodes():
    """One 16-pixel row written by hand: R a run of 16, G 16 literals, B two
    runs of 8, E a run of 16 (exponent 129: mantissa m decodes to m / 128)."""
    import tempfile
    body = bytes([2, 2, 0, 16])
    body += bytes([128 + 16, 64])
    body += bytes([16]) + bytes(range(0, 160, 10))
    body += bytes([128 + 8, 32, 128 + 8, 128])
    body += bytes([128 + 16, 129])
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "row.hdr")
        with open(p, "wb") as f:
            f.write(_rle_file(16, 1, body))
        img = hdr.read_hdr(p)
    assert img.shape == (1, 16, 4)
    assert np.all(img[0, :, 0] == 0.5)
    assert np.array_equal(img[0, :, 1], np.arange(0, 160, 10, dtype=np.float32) / 128)
    assert np.all(img[0, :8, 2] == 0.25) and np.all(img[0, 8:, 2] == 1.0)
    assert np.all(img[0, :, 3] == 1.0)
