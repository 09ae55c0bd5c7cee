"""tests/blur_png.rs:17-73 re-run on the GPU path: write an 8-bit grey PNG with
an impulse, read it back, UnaryFilter(u8 -> f32), GaussianFilter sigma 2,
UnaryFilter(f32 -> u8, round + clamp), write, read, and check the reference's
assertions -- plus the result against the oracle, bit for bit."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_blur_png_roundtrip(gpu, tmp_path):
    from itkg import png
    size, mid = 32, 16
    img = np.zeros((size, size), np.uint8)
    img[mid, mid] = 255
    inp, outp = tmp_path / "blur_input.png", tmp_path / "blur_output.png"
    png.write_gray8(img, inp)
    loaded = png.read_gray8(inp)
    as_f32 = gpu.CastFilter(loaded, gpu.F32)
    blurred = gpu.GaussianFilter(as_f32, 2.0)
    as_u8 = gpu.CastFilter(blurred, gpu.U8)
    result = as_u8.generate_region(as_u8.largest_region())
    png.write_gray8(result, outp)
    output = png.read_gray8(outp)
    assert output.region.size == (size, size)
    peak_after = int(output.data.max())
    assert peak_after < 255
    assert int(output.data[mid, mid]) == peak_after
    assert int(output.data.astype(np.uint32).sum()) >= 255 * 85 // 100
    want = oracle.cast_f32_to_u8(oracle.gaussian_f32(img.astype(np.float32), 2.0))
    assert np.array_equal(output.data, want)
