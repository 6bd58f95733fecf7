"""MC-KLN p_T-differential table and per-cell densities through the C ABI
(MCnucl::makeTable(ptmin, dpt, iPtmax), src/MCnucl.cpp:967-1025, and
MCnucl::setDensity(iy, ipt), :626-687).

Bars: the table at sampled nodes within 1e-9 relative of the FP64 oracle's
rule (smco_kln_dndy_pt; the oracle's rule is pinned to the reference's
adaptive Simpson values in tests/test_oracle.py); every cell's p_T bins
within 2e-5 of the bin's maximum of the six-point lookup of the FP64 table
at the oracle's FP64 thickness (the stencil floor(T/dT) decided as for the
p_T-integrated density); zero wherever T_A or T_B is zero; the p_T-
integrated outputs unchanged.
"""
import ctypes

import numpy as np
import pytest

from systems import oracle_params
from test_gpu_kln import _workload
from test_gpu_parity import engine

pytestmark = pytest.mark.gpu

PT_MIN, D_PT, NBINS = 0.1, 0.1, 20   # PT_Min, d_PT and MaxPT of the reference's parameters.dat
GRID_RTOL = 2e-5


def six_point(x, y, v00, v01, v02, v10, v11, v20):
    """sixPoint2dInterp (src/arsenal.cpp:33-54)"""
    axx = 0.5 * (v00 - 2 * v10 + v20)
    axy = v00 - v01 - v10 + v11
    ayy = 0.5 * (v00 - 2 * v01 + v02)
    bx = 0.5 * (-3 * v00 + 4 * v10 - v20)
    by = 0.5 * (-3 * v00 + 4 * v01 - v02)
    return axx * x * x + axy * x * y + ayy * y * y + bx * x + by * y + v00


def test_pt_table_nodes(oracle):
    from oracle.oracle import KLN
    vals = _workload()
    eng = engine(vals)
    tab = eng.kln_pt_table(PT_MIN, D_PT, NBINS)
    tm, dT = eng.info.kln_tmax, eng.info.kln_dT
    assert tab.shape == (tm, tm, NBINS)
    assert (tab[0] == 0).all() and (tab[:, 0] == 0).all()
    k = KLN()
    oracle.lib.smco_kln_init(ctypes.byref(k), vals["ecm"], vals["lambda"])
    rng = np.random.default_rng(3)
    nodes = np.vstack([[1, 1], [tm - 1, tm - 1], [1, tm - 1], rng.integers(1, tm, size=(40, 2))])
    for i, j in nodes:
        for p in range(NBINS):
            want = oracle.lib.smco_kln_dndy_pt(ctypes.byref(k), i * dT, j * dT, PT_MIN + p * D_PT,
                                               int(vals["kln_nkt"]), int(vals["kln_nphi"]))
            assert tab[i, j, p] == pytest.approx(want, rel=1e-9, abs=0), (i, j, p)
    # the spectrum falls with p_T at every node
    assert (np.diff(tab[1:, 1:], axis=2) < 0).all()


def test_pt_cells_vs_oracle_thickness(oracle):
    vals = _workload()
    eng = engine(vals, seed=5)
    tab = eng.kln_pt_table(PT_MIN, D_PT, NBINS)
    dT = eng.info.kln_dT
    n = 12
    out = eng.generate(0, n, want=("npart", "ncoll", "positions", "ta", "tb", "rho", "rho_pt"))
    assert out["rho_pt"].shape == (n, eng.nx, eng.ny, NBINS)
    plain = engine(vals, seed=5).generate(0, n, want=("rho", "ta", "tb"))
    for key in ("rho", "ta", "tb"):
        np.testing.assert_array_equal(out[key], plain[key])
    op = oracle_params(vals)
    op.kln_tmax = eng.info.kln_tmax   # the table bound of the thickness check (no table read)
    op.kln_dT = dT
    ev = oracle.event(op)
    A = out["positions"].shape[1] // 2
    for k in range(n):
        ev.inject(out["positions"][k, :A], out["positions"][k, A:])
        assert ev.pair() == out["ncoll"][k]
        assert ev.thickness() == 0
        ta, tb = ev.grid(0), ev.grid(1)
        di, dj = ta / dT, tb / dT
        ii, jj = np.floor(di).astype(int), np.floor(dj).astype(int)
        fi, fj = di - ii, dj - jj
        live = (ta > 0) & (tb > 0)
        got = out["rho_pt"][k]
        assert (got[~live] == 0).all()
        a, b = ii[live], jj[live]
        want = six_point(fi[live][:, None], fj[live][:, None], tab[a, b], tab[a, b + 1], tab[a, b + 2],
                         tab[a + 1, b], tab[a + 1, b + 1], tab[a + 2, b])
        err = np.abs(got[live] - want)
        assert (err <= GRID_RTOL * want.max(axis=0)).all(), (k, err.max())
