"""The closed-form dL/d rho the adjoint kernel uses (eccentricity and
centre-of-mass terms) against central differences of L, and the frozen
density against the oracle's own density; FP64 on the CPU, oracle events."""
import numpy as np
import pytest

from adjoint_ref import adjoint_grid, eps_n, grid_coords, objective
from systems import PBPB2760, oracle_params, values


@pytest.fixture(scope="module")
def event(oracle):
    vals = values(PBPB2760, maxx=8, maxy=8)
    p = oracle_params(vals)
    ev = oracle.event(p)
    nA, nB = oracle.nucleus(208), oracle.nucleus(208)
    for k in range(20):
        ev.populate_philox(nA, nB, 7.0, 5, k, 0)
        if ev.pair() > 0:
            break
    ev.thickness()
    assert ev.density() == 0
    X, Y = grid_coords(vals, ev.nx, ev.ny)
    return vals, ev, ev.grid(2), ev.hotspot_mask(), X, Y


def test_frozen_density_is_the_density_at_the_base_point(event):
    vals, ev, rho, mask, X, Y = event
    d = ev.density_frozen(vals["gauss_nucl_width"], vals["alpha"])
    np.testing.assert_allclose(d, rho, rtol=1e-14, atol=0)


def test_eccentricities_of_the_reference_layout(event):
    vals, ev, rho, mask, X, Y = event
    ecc = ev.eccentricities(1, 9, 7.0)
    e = eps_n(rho, mask, X, Y)
    np.testing.assert_allclose(e, [np.hypot(ecc[7], ecc[8]), np.hypot(ecc[12], ecc[13])], rtol=1e-12)


@pytest.mark.parametrize("which", ["eps", "rho", "both"])
def test_adjoint_grid_against_directional_differences(event, which):
    vals, ev, rho, mask, X, Y = event
    rng = np.random.default_rng(3)
    g_eps = np.array([0.7, -1.3]) if which != "rho" else None
    g_rho = rng.uniform(-1, 1, rho.shape) if which != "eps" else None
    lam = adjoint_grid(rho, mask, X, Y, g_eps, g_rho)
    for trial in range(3):
        d = rng.standard_normal(rho.shape) * (rho > 0) * rho.max() * 1e-2
        t = 1e-3
        fd = (objective(rho + t * d, mask, X, Y, g_eps, g_rho) -
              objective(rho - t * d, mask, X, Y, g_eps, g_rho)) / (2 * t)
        an = float((lam * d).sum())
        assert abs(an - fd) <= 1e-7 * max(abs(fd), 1e-12), (an, fd)


@pytest.mark.parametrize("u", [1e-6, 0.02, 0.3, 0.5, 0.8, 0.97, 0.9995])
def test_inverse_cdf_radius_and_its_derivatives(oracle, u):
    """r(u) inverts the truncated Woods-Saxon CDF; dr/dR, dr/da (implicit
    differentiation, moving end point included) agree with central
    differences of r(u; R, a)."""
    from scipy.integrate import quad
    R, a = 6.62, 0.546
    r, dR, da = oracle.ws_icdf(R, a, u)
    f = lambda t: t * t / (1 + np.exp((t - R) / a))
    F = quad(f, 0, r, epsabs=0, epsrel=1e-13)[0] / quad(f, 0, R + 2.5, epsabs=0, epsrel=1e-13)[0]
    assert F == pytest.approx(u, rel=1e-10, abs=1e-15)
    h = 1e-5
    fdR = (oracle.ws_icdf(R + h, a, u)[0] - oracle.ws_icdf(R - h, a, u)[0]) / (2 * h)
    fda = (oracle.ws_icdf(R, a + h, u)[0] - oracle.ws_icdf(R, a - h, u)[0]) / (2 * h)
    assert dR == pytest.approx(fdR, rel=1e-7, abs=1e-9)
    assert da == pytest.approx(fda, rel=1e-7, abs=1e-9)


def test_moved_density_is_the_density_without_displacement(event):
    vals, ev, rho, mask, X, Y = event
    zA = np.zeros((208, 2))
    d = ev.density_moved(vals["gauss_nucl_width"], vals["alpha"], zA, zA)
    np.testing.assert_allclose(d, rho, rtol=1e-14, atol=0)


def test_inverse_cdf_tangents_against_displacements(oracle):
    """Nucleon tangents of an inverse-CDF event against central differences
    of its displacements (centre-of-mass shift included)."""
    vals = values(PBPB2760, maxx=8, maxy=8)
    ev = oracle.event(oracle_params(vals))
    nA = oracle.nucleus(208, icdf=1)
    nB = oracle.nucleus(208, icdf=1)
    ev.populate_philox(nA, nB, 5.0, 9, 0, 0)
    tA, tB = ev.icdf_tangents(nA, nB)
    h = 1e-5
    for k, (dR, da) in enumerate(((h, 0.0), (0.0, h))):
        pA, pB = ev.icdf_displacement(nA, nB, dR, da)
        mA, mB = ev.icdf_displacement(nA, nB, -dR, -da)
        fdA, fdB = (pA - mA) / (2 * h), (pB - mB) / (2 * h)
        np.testing.assert_allclose(fdA, tA[:, 2 * k:2 * k + 2], atol=1e-7)
        np.testing.assert_allclose(fdB, tB[:, 2 * k:2 * k + 2], atol=1e-7)
    # the centre-of-mass shift keeps the tangents' mean at zero
    np.testing.assert_allclose(tA.mean(axis=0), 0, atol=1e-12)
