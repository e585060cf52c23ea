"""HdrImage writers (graphics/display.rs:359-465) restated in gartus_gb300.raytracing."""
import struct

import numpy as np

from gartus_gb300.raytracing import HdrImage


def test_radiance_hdr_known_answer():  # display.rs:2186-2199
    img = HdrImage(1, 1, np.array([[[1.0, 0.5, 0.25]]], dtype=np.float32))
    b = img.radiance_hdr_bytes()
    assert b.startswith(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 1 +X 1\n")
    assert list(b[-4:]) == [128, 64, 32, 129]


def test_radiance_hdr_black_negative_and_non_finite():  # encode_rgbe, display.rs:443-465
    px = np.array([[[0.0, 0.0, 0.0], [-1.0, np.nan, np.inf], [3.0, 0.0, 0.0]]], dtype=np.float32)
    b = HdrImage(3, 1, px).radiance_hdr_bytes()
    body = list(b[-12:])
    assert body[0:4] == [0, 0, 0, 0] and body[4:8] == [0, 0, 0, 0]
    # 3.0 = 0.75 * 2^2: exponent 2, mantissa 256 * 3 / 4 = 192
    assert body[8:12] == [192, 0, 0, 130]


def test_pfm_layout(tmp_path):  # write_pfm, display.rs:365-387
    px = np.zeros((2, 3, 3), dtype=np.float32)
    px[0, 0] = (1.0, 2.0, 3.0)  # top-left
    px[1, 2] = (4.0, np.nan, 5.0)  # bottom-right, NaN written as 0
    img = HdrImage(3, 2, px)
    b = img.pfm_bytes()
    head = b"PF\n3 2\n-1.0\n"
    assert b.startswith(head)
    vals = struct.unpack("<18f", b[len(head):])
    assert vals[6:9] == (4.0, 0.0, 5.0)  # the bottom row comes first
    assert vals[9:12] == (1.0, 2.0, 3.0)
    p = tmp_path / "x.pfm"
    img.save_extension(str(p))
    assert p.read_bytes() == b
