"""Dirty-image error against the FP64 oracle on dense uv coverage: the GPU path (FP32 with
compensated cross-item sums) stays within 1e-5 of the image peak in the CRDNHALF window,
with and without the compensation; the reference's own FP32 arithmetic is recorded beside
it (at this density it is far from FP64, which is why results are stated against FP64)."""
import pytest

pytestmark = pytest.mark.gpu


def test_dense_cells_stay_within_1e5_of_fp64(gpu_ctx):
    from oracle import precision
    data = precision.dense_case(stride=64)      # ~1.0 M visibilities
    r = precision.study(gpu_ctx, data, imsize=256, cell=8.0)
    assert r["vis_per_cell"]["max"] > 1000
    assert r["compensated"]["window"] < 1e-5
    assert r["plain_fp32"]["window"] < 1e-5
    assert r["compensated"]["window"] <= r["plain_fp32"]["window"] * 1.5 + 1e-8
