"""FP32 cell coordinates (abl_runtime.cu, bin_in_fp32 and k_bin_assign).

Binning may compute floor((x - lo) / w) in FP32 when the bound
(2|lo|/w + 4n) * 2^-24 on its rounding error is below 2.4e-4, where n is the
number of cells along the axis.  Cells are 2^-10 wider than the radius, so
two agents that pass the reference's float-rounded radius test (at most
2^-22 beyond the radius) must land in cells at most one apart.  numpy's
float32 arithmetic rounds like the device's __fsub_rn / __fmul_rn, so the
device computation is emulated here on adversarial positions: values next
to cell boundaries and pairs exactly one radius apart.
"""
import numpy as np
import pytest

U = 2.0 ** -24


def cell_f32(x, lo, inv, n):
    f = np.floor((x.astype(np.float32) - np.float32(lo)) * np.float32(inv))
    return np.clip(f, 0, n - 1).astype(np.int64)


def coord_f32(x, lo, inv):
    return ((x.astype(np.float32) - np.float32(lo)) * np.float32(inv)).astype(np.float64)


def bound(lo, inv, n):
    return (2.0 * abs(lo) * inv + 4.0 * n) * U


# (lo, radius, extent): boids2d 1M (363 cells), a grid offset from the
# origin, and the largest grids the runtime allows in FP32
GRIDS = [(0.0, 0.05, 18.1019), (-3.0, 0.05, 10.0), (0.0, 1.0, 1000.0), (250.0, 0.5, 200.0)]


@pytest.mark.parametrize("lo,r,extent", GRIDS)
def test_error_bound_holds(lo, r, extent):
    w = r * (1.0 + 2.0 ** -10)
    inv = 1.0 / w
    n = int(np.ceil(extent / w))
    b = bound(lo, inv, n)
    if b > 2.4e-4:
        pytest.skip("the runtime bins this grid in FP64")
    rng = np.random.default_rng(0)
    # positions next to every cell boundary and uniform ones
    k = np.arange(n + 1)
    edges = lo + k * w
    near = np.concatenate([edges + d for d in (-1e-6, -1e-9, 0.0, 1e-9, 1e-6)])
    x = np.concatenate([near, lo + rng.random(200000) * n * w])
    x = x[(x >= lo) & (x <= lo + n * w)]
    err = np.abs(coord_f32(x, lo, inv) - (x - lo) * inv)
    assert err.max() <= b


@pytest.mark.parametrize("lo,r,extent", GRIDS)
def test_neighbours_within_one_cell(lo, r, extent):
    w = r * (1.0 + 2.0 ** -10)
    inv = 1.0 / w
    n = int(np.ceil(extent / w))
    if bound(lo, inv, n) > 2.4e-4:
        pytest.skip("the runtime bins this grid in FP64")
    rng = np.random.default_rng(1)
    # pairs a radius (plus the reference test's slack) apart, placed around
    # cell boundaries
    k = rng.integers(0, n, 200000)
    a = lo + k * w + rng.uniform(-1.1 * r, 0.1 * r, k.size)
    bpos = a + r * (1.0 + 2.0 ** -22)
    keep = (a >= lo) & (bpos <= lo + n * w)
    ca, cb = cell_f32(a[keep], lo, inv, n), cell_f32(bpos[keep], lo, inv, n)
    assert np.all(np.abs(cb - ca) <= 1)
    # and in FP64 on one side (a query computing its cell in FP64)
    cd = np.clip(np.floor((bpos[keep] - lo) * inv), 0, n - 1).astype(np.int64)
    assert np.all(np.abs(cd - ca) <= 1)
