"""FP32-first decisions of the kernels against the exact FP64 rule (CPU,
numpy float32 arithmetic restating the device expressions).

* The per-cell cut (cells with dc <= 25 w^2, or dc <= dsq for disk nucleons,
  src/Particle.cpp:122-132, src/MCnucl.cpp:732-756): the splats decide a cell
  from its FP32 distance outside a relative band around the cut and fall back
  to the FP64 rule inside it.  `cut_band` (grid_common.cuh) sizes the band
  from an error bound; here the FP32 distance error, at cells next to the
  cut, stays below a third of the band (the bound carries a factor 3).
* Window indices (the reference's (int)((x -+ h - mn) / d) truncations,
  src/MCnucl.cpp:432-478, src/MakeDensity.cpp:2356-2358): the sampler takes
  them from FP32 copies when the FP32 value lies 1e-3 away from an integer
  (`edge_index`, k_sample_pair.cu); the FP32 index then equals the FP64 one.
"""
import numpy as np
import pytest

f32 = np.float32


def cut_band(xmin, nx, dx, ymin, ny, dy, rho2):
    """cut_band of grid_common.cuh."""
    rho = np.sqrt(rho2)
    ext = max(abs(xmin), abs(xmin + (nx - 1) * dx), abs(ymin), abs(ymin + (ny - 1) * dy))
    return min(1e-4, 2.2e-6 * (ext + rho) / rho + 7.2e-7)


def fmaf(a, b, c):
    """float32 fma: the exact product (48 bits) plus c, rounded once (to
    FP64 first: the double rounding is far below the tolerances here)."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


GRIDS = [
    # (maxx, dx, w): the bench's 261^2 grid, the 501^2 averaged grid, a fine grid
    (13.0, 0.1, 0.5),
    (25.0, 0.1, 0.5),
    (10.0, 0.05, 0.4),
]


@pytest.mark.parametrize("maxx,dx,w", GRIDS)
@pytest.mark.parametrize("disk", [False, True])
def test_fp32_distance_error_within_a_third_of_the_band(maxx, dx, w, disk):
    rng = np.random.default_rng(11)
    n = int(round(2 * maxx / dx)) + 1
    xmin = -maxx
    rho2 = 0.1 * 64.0 / np.pi if disk else 25.0 * w * w   # dsq of sigma_NN = 64 mb; 25 w^2
    band = cut_band(xmin, n, dx, xmin, n, dx, rho2)
    lim = f32(rho2)
    worst = 0.0
    for _ in range(4000):
        # a source anywhere its window can reach the grid, a cell next to its cut
        sx, sy = rng.uniform(xmin - 2, -xmin + 2, 2)
        drow = rng.uniform(-np.sqrt(rho2), np.sqrt(rho2))
        i = int(np.clip(round((sx + drow - xmin) / dx), 0, n - 1))
        xg64 = xmin + i * dx
        dy_need = np.sqrt(max(rho2 - (xg64 - sx) ** 2, 0.0))
        for sgn in (-1, 1):
            j = int(np.clip(round((sy + sgn * dy_need - xmin) / dx), 0, n - 1))
            yg64 = xmin + j * dx
            exact = (sx - xg64) ** 2 + (sy - yg64) ** 2            # FP64, as the reference
            dxf = f32(f32(xg64) - f32(sx))                          # xg[i] - g.xf
            dyf = f32(f32(yg64) - f32(sy))                          # yg[j] - g.yf
            dcf = fmaf(dyf, dyf, f32(dxf * dxf))                    # fmaf(dy, dy, dx2)
            if abs(exact - rho2) < 0.1 * rho2:                     # cells near the cut
                worst = max(worst, abs(float(dcf) - exact) / float(lim))
    assert worst > 0
    assert worst < band / 3, (worst, band)


def edge_index_fp32(a, b, mn, d):
    """The FP32 path of edge_index: the index, or None when the FP64 rule
    decides."""
    af, bf, mnf = f32(a), f32(b), f32(mn)
    inv_d = f32(1.0 / d)
    t = f32(f32(f32(af + bf) - mnf) * inv_d)
    fl = np.floor(t)
    fr = f32(t - fl)
    if (abs(af) + abs(bf) + abs(mnf)) * inv_d < 2000 and 1e-3 < fr < 1 - 1e-3:
        i = int(fl)
        return i + 1 if t < 0 else i
    return None


@pytest.mark.parametrize("maxx,dx,h", [(13.0, 0.1, 2.0), (25.0, 0.1, 2.5), (10.0, 0.05, 1.2)])
def test_window_index_fp32_equals_fp64(maxx, dx, h):
    rng = np.random.default_rng(5)
    decided = {"random": 0, "edge": 0}
    for kind in ("random", "edge"):
        for _ in range(10000):
            sgn = rng.choice([-1.0, 1.0])
            if kind == "random":
                x = rng.uniform(-maxx - 3, maxx + 3)
            else:   # within 1e-5 of a window edge: the FP64 rule decides
                k = rng.integers(0, int(2 * maxx / dx))
                x = -maxx + k * dx - sgn * h + rng.uniform(-1e-5, 1e-5)
            got = edge_index_fp32(x, sgn * h, -maxx, dx)
            want = int((x + sgn * h - (-maxx)) / dx)   # C++ truncation toward zero, FP64
            if got is not None:
                decided[kind] += 1
                assert got == want, (x, sgn, got, want)
    assert decided["random"] > 9900   # the FP32 path decides nearly every edge
    assert decided["edge"] == 0       # and leaves the ones next to an integer to FP64
