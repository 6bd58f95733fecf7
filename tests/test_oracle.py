"""The oracle (oracle/smc_oracle.c) against the reference's golden vectors.

The fixtures in tests/golden/ were produced by the reference's own code
(tests/golden/make_golden.py); on the same inputs the oracle must reproduce
them bit for bit where the reference's arithmetic is reproducible
(participants, collisions, grids) and to the reference's printed precision
(8 significant digits) for the eccentricity lines.
"""
import json
import os

import numpy as np
import pytest

from systems import SYSTEMS, fmt8, oracle_params, values
from conftest import GOLDEN


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for Philox4x32-10
    kat = [([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
           ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
           ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
            [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1])]
    for ctr, key, want in kat:
        assert oracle.philox(ctr, key) == want


def test_uniforms_open_interval(oracle):
    u = np.array([oracle.uniform2(7, e, s, k) for e in range(20) for s in range(3) for k in range(20)])
    assert (u > 0).all() and (u < 1).all()
    assert abs(u.mean() - 0.5) < 0.02


def test_constants(oracle):
    c = json.load(open(os.path.join(GOLDEN, "constants.json")))
    for e, v in c["sigma_in"].items():
        assert oracle.lib.smco_sigma_in(float(e)) == v
    for row in c["six_point"]:
        assert oracle.lib.smco_six_point(*row[:8]) == row[8]
    for r, v in c["hulthen_cdf"].items():
        assert oracle.lib.smco_hulthen_cdf(float(r)) == pytest.approx(v, rel=1e-14, abs=1e-300)
    for u, v in c["hulthen_inv"].items():
        assert oracle.lib.smco_hulthen_inv(float(u)) == pytest.approx(v, rel=1e-12)


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_sigma_gg_and_dsq(oracle, golden, name):
    g = golden("glauber_inject.npz")
    dsq, width, sgg, sigin = g[name + "_constants"]
    vals = values(SYSTEMS[name])
    p = oracle_params(vals)
    assert p.dsq == dsq and p.width == width and p.sigin == sigin
    assert oracle.lib.smco_sigeff(sigin, width) == pytest.approx(sgg, rel=1e-13)


def _digest_check(grid, g, key, rtol=0.0):
    cells = g[key + "_cells"].astype(int)
    vals = g[key + "_values"]
    got = grid[cells[:, 0], cells[:, 1]]
    if rtol == 0.0:
        np.testing.assert_array_equal(got, vals)
    else:
        np.testing.assert_allclose(got, vals, rtol=rtol, atol=0)
    np.testing.assert_allclose(grid.sum(axis=1), g[key + "_rowsum"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(grid.sum(axis=0), g[key + "_colsum"], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_injected_events_match_reference(oracle, golden, name):
    g = golden("glauber_inject.npz")
    vals = values(SYSTEMS[name])
    ev = oracle.event(oracle_params(vals))
    pa, pb, bs = g[name + "_pos_a"], g[name + "_pos_b"], g[name + "_b"]
    for k in range(len(bs)):
        ev.inject(pa[k], pb[k])
        assert ev.pair() == g[name + "_ncoll"][k]
        assert ev.npart() == (g[name + "_npart1"][k], g[name + "_npart2"][k])
        np.testing.assert_array_equal(ev.participants(0), g[name + f"_ev{k}_partA"])
        np.testing.assert_array_equal(ev.participants(1), g[name + f"_ev{k}_partB"])
        np.testing.assert_array_equal(ev.collisions(), g[name + f"_ev{k}_coll"])
        assert ev.thickness() == 0 and ev.density() == 0
        if k in (1, 3):
            for w, gname in enumerate(("ta", "tb", "rho")):
                _digest_check(ev.grid(w), g, f"{name}_ev{k}_{gname}")
        ecc = ev.eccentricities(1, 9, bs[k])
        np.testing.assert_array_equal(fmt8(ecc), g[name + "_ecc"][k])


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_rotation_resplat_matches_reference(oracle, golden, name):
    g = golden("glauber_inject.npz")
    ev = oracle.event(oracle_params(values(SYSTEMS[name])))
    ev.inject(g[name + "_pos_a"][3], g[name + "_pos_b"][3])
    ev.pair(); ev.thickness(); ev.density()
    for order in (2, 3):
        assert ev.rotate_resplat(order) == 0
        _digest_check(ev.grid(2), g, f"{name}_rot{order}_rho")


def test_drand48_sampler_matches_reference(oracle, golden):
    """Nucleus::populate with libc drand48: same draws, same positions (to
    libm's last-bit agreement between hosts)."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand48.argtypes = [ctypes.c_long]
    g = golden("sampler_drand48.npz")
    vals = values(SYSTEMS["pbpb2760"])
    ev = oracle.event(oracle_params(vals))
    for key in g.files:
        A, d, s = key.split("_")
        A, d, s = int(A[1:]), int(d[1:]), int(s[1:])
        nuc = oracle.nucleus(A, d)
        libc.srand48(s)
        ev.populate_drand48(nuc, nuc, 5.0)
        got = ev.nucleons(0)
        np.testing.assert_allclose(got, g[key], rtol=0, atol=1e-12)


def test_kln_integrand_matches_reference(oracle, golden):
    import ctypes
    from oracle.oracle import KLN, _ptr
    g = golden("kln.npz")
    k = KLN()
    oracle.lib.smco_kln_init(ctypes.byref(k), 2760.0, 0.288)
    for row, want in zip(g["points"], g["integrand"]):
        x = np.ascontiguousarray(row[2:])
        got = oracle.lib.smco_kln_integrand(ctypes.byref(k), row[0], row[1], _ptr(x))
        assert got == pytest.approx(want, rel=1e-14, abs=0)


def test_kln_quadrature_near_bases(oracle, golden):
    """The deterministic rule against the reference's BASES integral (which
    carries Monte-Carlo error of a few per mille)."""
    import ctypes
    from oracle.oracle import KLN
    g = golden("kln.npz")
    k = KLN()
    oracle.lib.smco_kln_init(ctypes.byref(k), 2760.0, 0.288)
    for (ta, tb), want in zip(g["nodes"], g["bases"]):
        got = oracle.lib.smco_kln_dndy(ctypes.byref(k), ta, tb, 48, 64, 32)
        assert got == pytest.approx(want, rel=5e-3)


def test_kln_pt_rule_matches_reference_simpson(oracle, golden):
    """dN/dy d^2p_T at fixed p_T (MCnucl::makeTable(ptmin, dpt, iPtmax)):
    the oracle's Gauss-Legendre rule (64 k_T x 32 phi nodes) against the
    reference's adaptive Simpson integral (relative precision 1e-4)."""
    import ctypes
    from oracle.oracle import KLN
    g = golden("kln_pt.npz")
    k = KLN()
    oracle.lib.smco_kln_init(ctypes.byref(k), 2760.0, 0.288)
    for (ta, tb, pt), want in zip(g["points"], g["values"]):
        got = oracle.lib.smco_kln_dndy_pt(ctypes.byref(k), ta, tb, pt, 64, 32)
        assert got == pytest.approx(want, rel=5e-4), (ta, tb, pt)


def test_kln_lookup_matches_reference(oracle, golden):
    from oracle.oracle import _ptr
    g = golden("kln.npz")
    vals = values(SYSTEMS["pbpb2760"], which_mc_model=1, sub_model=7)
    p = oracle_params(vals)
    dT = float(g["table_dT"])
    tmax = 211
    I, J = np.meshgrid(np.arange(tmax), np.arange(tmax), indexing="ij")
    table = np.ascontiguousarray(np.where((I > 0) & (J > 0), np.sqrt(I * dT * J * dT) * 3.0 + 0.1 * (I * dT) ** 2, 0.0))
    p.kln_table = _ptr(table)
    p.kln_tmax = tmax
    p.kln_dT = dT
    ev = oracle.event(p)
    ev.inject(g["lookup_pos_a"], g["lookup_pos_b"])
    ev.pair()
    assert ev.thickness() == 0 and ev.density() == 0
    _digest_check(ev.grid(2), g, "lookup_rho")


def test_native_loop_statistics_match_reference(oracle, golden):
    """The op-9 loop with drand48 reproduces the reference's own table."""
    import ctypes
    from oracle.oracle import _ptr
    g = golden("ecc_native.npz")
    vals = values(SYSTEMS["pbpb2760"], ecc_from_order=2, ecc_to_order=5)
    p = oracle_params(vals)
    nuc = oracle.nucleus(208)
    n = 60
    out = np.zeros((n, 49))
    oracle.lib.smco_run_ecc_table(ctypes.byref(p), ctypes.byref(nuc), ctypes.byref(nuc), 0.0, 20.0, n, 2, 5,
                                  7, 0, 0, _ptr(out))
    np.testing.assert_array_equal(fmt8(out), g["pbpb2760"][:n])


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_average_sequence_matches_reference(oracle, golden, name):
    """Averaged mode on events from the drand48 sampler: reaction-plane and
    participant-plane means of orders 2, 3 against the reference's own run
    (the rotation resets each participant's box to its construction-time box
    in the nucleus frame, which truncates the re-splatted Gaussians)."""
    import ctypes
    from systems import oracle_average
    libc = ctypes.CDLL(None)
    libc.srand48.argtypes = [ctypes.c_long]
    g = golden("average.npz")
    vals = values(SYSTEMS[name])
    nA, nB = oracle.nucleus(int(vals["aproj"])), oracle.nucleus(int(vals["atarg"]))
    events = g[name + "_events"]

    def fill(ev, k):
        libc.srand48(int(events[k, 0]))
        ev.populate_drand48(nA, nB, float(events[k, 1]))
        return True

    got, used = oracle_average(oracle, vals, fill, len(events))
    assert used == len(events)
    for (mode, o), grid in got.items():
        key = f"{name}_{mode}{o}_"
        cells = g[key + "cells"].astype(int)
        scale = np.abs(g[key + "values"]).max()
        np.testing.assert_allclose(grid[cells[:, 0], cells[:, 1]], g[key + "values"], rtol=0, atol=1e-10 * scale)
        np.testing.assert_allclose(grid.sum(axis=1), g[key + "rowsum"], rtol=0, atol=1e-9 * scale)


@pytest.mark.parametrize("k,theta", [((1 - 0.118) / 2 / 0.75, 2 / (1 - 0.118) * 0.75),   # participant, default
                                     (0.118 / 0.75, 0.75 / 0.118),                      # binary collision
                                     (2.5, 0.4)])
def test_gamma_weights_follow_the_gamma_distribution(oracle, k, theta):
    """The multiplicity weights of cc_fluctuation_model 6 (the reference
    draws them with gsl_ran_gamma, MCnucl.cpp:1285,1298): KS against
    Gamma(k, theta), unit mean."""
    from scipy import stats
    x = np.array([oracle.lib.smco_gamma_philox(11, ev, 0, s, k, theta) for ev in range(4) for s in range(5000)])
    assert stats.kstest(x, "gamma", args=(k, 0, theta)).pvalue > 1e-3
    assert abs(x.mean() - k * theta) < 5 * np.sqrt(k * theta * theta / len(x))


@pytest.mark.parametrize("nb,k", [(0.3, 0.75), (4.0, 0.75), (25.0, 2.0), (60.0, 0.5)])
def test_nbd_counts_follow_the_negative_binomial(oracle, nb, k):
    """The per-cell counts of cc_fluctuation_model 1/2 (NBD::rand(nb/(nb+k), k)
    in MCnucl::fluctuateCurrentDensity, MCnucl.cpp:869-905): mean nb,
    variance nb (1 + nb/k), the negative-binomial pmf (chi-square)."""
    from scipy import stats
    x = np.array([oracle.lib.smco_nbd_draw(5, ev, c, nb, k) for ev in range(4) for c in range(5000)])
    assert np.all(x == np.floor(x)) and x.min() >= 0
    n = len(x)
    assert abs(x.mean() - nb) < 5 * np.sqrt(nb * (1 + nb / k) / n)
    p = k / (k + nb)   # scipy's success probability
    var = nb * (1 + nb / k)
    assert abs(x.var() / var - 1) < 0.1
    hi = int(stats.nbinom.ppf(0.999, k, p))
    obs = np.bincount(np.minimum(x.astype(int), hi), minlength=hi + 1)
    exp_ = stats.nbinom.pmf(np.arange(hi + 1), k, p) * n
    exp_[-1] += stats.nbinom.sf(hi, k, p) * n
    keep = exp_ > 5
    chi2 = (((obs - exp_) ** 2 / exp_)[keep]).sum()
    assert stats.chi2.sf(chi2, keep.sum() - 1) > 1e-4
