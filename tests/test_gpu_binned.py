"""Centrality-binned averaged profiles (smc_average_binned).

method 0 (sources moved and re-splatted, the reference's rotateGrid) is
checked against smc_average's per-event rotated densities, which
tests/test_gpu_average.py pins to the oracle's run of the reference's
per-event sequence; method 1 (bilinear resampling) against a numpy FP64
resampling of the GPU's own per-event densities, and against method 0 (the
error of resampling instead of re-splatting, which is reported).
"""
import numpy as np
import pytest

from systems import SYSTEMS, values

pytestmark = pytest.mark.gpu

EDGES = [2, 60, 160, 300, 395]


def engine(vals, seed):
    from supermc_gb300.engine import Engine
    return Engine(dict(vals), seed=seed)


def _bins(npart, edges):
    b = np.full(len(npart), -1)
    for k in range(len(edges) - 1):
        b[(npart >= edges[k]) & (npart < edges[k + 1])] = k
    return b


@pytest.fixture(scope="module")
def sample():
    vals = values(SYSTEMS["auau200"], ecc_from_order=2, ecc_to_order=3)
    eng = engine(vals, seed=21)
    n = 24
    out = eng.generate(0, n, want=("rho", "npart", "ncoll"))
    return vals, eng, n, out


def test_source_rotation_bins_equal_per_event_rotations(sample):
    vals, eng, n, out = sample
    mean, counts = eng.average_binned(0, n, EDGES, order=2, method=0)
    bins = _bins(out["npart"].sum(axis=1), EDGES)
    np.testing.assert_array_equal(counts, [np.sum(bins == k) for k in range(len(EDGES) - 1)])
    want = np.zeros_like(mean)
    for e in range(n):
        if bins[e] < 0:
            continue
        m, _ = eng.average(e, 1, 2, 2, False)
        want[bins[e]] += m[0]
    for k in range(len(counts)):
        if counts[k]:
            want[k] /= counts[k]
    np.testing.assert_allclose(mean, want, rtol=0, atol=2e-6 * want.max())


def _frame(rho, vals, order):
    """Centre of mass and the rotation the sources receive
    (GlueDensity::calcCMAngle, src/GlueDensity.cpp:87-144), FP64."""
    nx, ny = rho.shape
    x = -vals["maxx"] + np.arange(nx) * vals["dx"]
    y = -vals["maxy"] + np.arange(ny) * vals["dy"]
    X, Y = np.meshgrid(x, y, indexing="ij")
    r = rho.astype(np.float64)
    W = r.sum()
    xc, yc = (X * r).sum() / W, (Y * r).sum() / W
    z = (X - xc) + 1j * (Y - yc)
    s = (z ** order * r).sum()
    ang = -np.arctan2(-s.imag, -s.real) / order
    return xc, yc, np.cos(ang), np.sin(ang), X, Y


def _bilinear(rho, vals, fr):
    xc, yc, c, s, X, Y = fr
    nx, ny = rho.shape
    px = (c * X + s * Y + xc + vals["maxx"]) / vals["dx"]
    py = (-s * X + c * Y + yc + vals["maxy"]) / vals["dy"]
    i0, j0 = np.floor(px).astype(int), np.floor(py).astype(int)
    tx, ty = px - i0, py - j0
    g = np.zeros((nx + 2, ny + 2))
    g[1:-1, 1:-1] = rho
    ok = (i0 >= -1) & (i0 < nx) & (j0 >= -1) & (j0 < ny)
    i0c, j0c = np.clip(i0, -1, nx - 1) + 1, np.clip(j0, -1, ny - 1) + 1
    v = ((1 - tx) * ((1 - ty) * g[i0c, j0c] + ty * g[i0c, j0c + 1]) +
         tx * ((1 - ty) * g[i0c + 1, j0c] + ty * g[i0c + 1, j0c + 1]))
    return np.where(ok, v, 0.0)


def test_bilinear_bins_against_numpy_resampling(sample):
    vals, eng, n, out = sample
    mean, counts = eng.average_binned(0, n, EDGES, order=2, method=1)
    bins = _bins(out["npart"].sum(axis=1), EDGES)
    want = np.zeros_like(mean)
    for e in range(n):
        if bins[e] >= 0:
            want[bins[e]] += _bilinear(out["rho"][e], vals, _frame(out["rho"][e], vals, 2))
    for k in range(len(counts)):
        if counts[k]:
            want[k] /= counts[k]
    want *= vals["finalfactor"]
    np.testing.assert_allclose(mean, want, rtol=0, atol=2e-5 * want.max())


def test_bilinear_against_source_rotation(sample):
    """Resampling instead of re-splatting: per bin, the relative L1 error of
    the bilinear average (reported; bounded by the interpolation error of a
    Gaussian of width w on a dx grid plus the reference's box truncation)."""
    vals, eng, n, out = sample
    m0, c0 = eng.average_binned(0, n, EDGES, order=2, method=0)
    m1, c1 = eng.average_binned(0, n, EDGES, order=2, method=1)
    np.testing.assert_array_equal(c0, c1)
    for k in range(len(c0)):
        if c0[k] == 0:
            continue
        rel = np.abs(m1[k] - m0[k]).sum() / m0[k].sum()
        print(f"bin {k}: {c0[k]} events, relative L1 error {rel:.3e}")
        assert rel < 0.05
