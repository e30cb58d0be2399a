"""The warp kernels find a source pixel's row as trunc((m + 1/2) * RN(1/w)) in float arithmetic when the view
has at most 2^21 pixels, instead of the integer division m / w. The quotient's rounding error stays below its
distance 1/(2w) from the nearest integer, so the truncation is the integer quotient. That argument (in
device_common.cuh, pixel_of) covers every width; this test checks it exhaustively over every pixel index below
2^21 for a list of chosen widths and 64 seeded random widths, in IEEE single precision (numpy rounds to nearest
like the device's multiply and correctly rounded division)."""
import numpy as np

WIDTHS = list(range(1, 70)) + [127, 128, 129, 255, 256, 257, 511, 512, 513, 640, 720, 1000, 1023, 1024, 1025,
                               1448, 1920, 2047, 2048, 2049, 3000, 4095, 4096, 8191, 65535, 1 << 20, (1 << 21) - 1]


def test_float_row_index_is_integer_quotient():
    m = np.arange(1 << 21, dtype=np.int64)
    mf = m.astype(np.float32) + np.float32(0.5)
    rng = np.random.default_rng(2021)
    for w in WIDTHS + [int(v) for v in rng.integers(2, 1 << 21, 64)]:
        rw = np.float32(1.0) / np.float32(w)
        y = (mf * rw).astype(np.int64)  # truncation toward zero, as the float -> int conversion in the kernels
        assert np.array_equal(y, m // w), w
