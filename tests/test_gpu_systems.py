"""Collision systems beyond Au+Au and Pb+Pb through the C ABI: p+Pb, d+Au
(Hulthen deuteron), Cu+Cu and deformed U+U at the reference's geometry, and
Cu+Cu, U+U and Au+Au (0.4 fm hard core, 42 mb) with Woods-Saxon parameters
from the optional keys.

For every system: the GPU's Philox sampler against the oracle's (nucleons
within 1e-4 fm, orientations exact); the same nucleon positions injected into
both (Npart, Ncoll exact, grid within 2e-5 of its maximum, eps_n within 1e-6),
on both splats; at the reference's geometry, Npart, Ncoll, b, eps_2 and
eps_3 of generated events against the reference's own drand48 sampler
(two-sample KS).
"""
import numpy as np
import pytest

from systems import ALL_SYSTEMS, NATIVE_SYSTEMS, oracle_nuclei, oracle_params, values
from test_gpu_parity import GRID_RTOL, assert_ecc_close, engine

pytestmark = pytest.mark.gpu


def _stream_id(attempt, sid):
    return (attempt << 8) | sid


@pytest.mark.parametrize("name", list(ALL_SYSTEMS))
def test_generated_nuclei_follow_oracle_sampler(oracle, name):
    """Positions, impact parameters and nucleus orientations of generated
    events against the oracle's Philox sampler (the GPU samples in FP32: a
    rejection decision within FP32 rounding may differ, rarely)."""
    vals = values(ALL_SYSTEMS[name])
    eng = engine(vals, seed=3)
    n = 48
    out = eng.generate(0, n, want=("npart", "ncoll", "b", "attempts", "positions", "orientation"))
    ev = oracle.event(oracle_params(vals))
    nA, nB = oracle_nuclei(oracle, vals)
    agree = 0
    for e in range(n):
        att = int(out["attempts"][e]) - 1
        b = oracle.lib.smco_impact_philox(3, e, att, vals["bmin"], vals["bmax"])
        assert b == pytest.approx(out["b"][e], rel=1e-15)
        for w in range(2):
            u = oracle.uniform2(3, e, _stream_id(att, 0), 1 + w)
            assert out["orientation"][e, 2 * w] == 1.0 - 2.0 * u[0]
            assert out["orientation"][e, 2 * w + 1] == 2 * np.pi * u[1]
        ev.populate_philox(nA, nB, b, 3, e, att)
        ref = np.concatenate([ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]])
        if np.abs(ref - out["positions"][e]).max() < 1e-4:
            agree += 1
    assert agree >= n - 2


@pytest.mark.parametrize("name", list(ALL_SYSTEMS))
def test_injected_events_vs_oracle(oracle, name):
    """Nucleons from the oracle's sampler, injected into both: the pairing,
    density and eccentricities of the same nuclei."""
    vals = values(ALL_SYSTEMS[name])
    ev = oracle.event(oracle_params(vals))
    nA, nB = oracle_nuclei(oracle, vals)
    rng = np.random.default_rng(11)
    pa, pb, bs, res = [], [], [], []
    k = 0
    while len(bs) < 24:
        b = float(np.sqrt(rng.uniform(0, 1)) * 12.0)
        ev.populate_philox(nA, nB, b, 11, k, 0)
        k += 1
        if ev.pair() == 0:
            continue
        xa, xb = ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]
        ev.inject(xa, xb)
        nc = ev.pair()
        assert ev.thickness() == 0 and ev.density() == 0
        pa.append(xa); pb.append(xb); bs.append(b)
        res.append((ev.npart(), nc, ev.grid(2), ev.eccentricities(1, 9, b)))
    for tensor_cores in (False, True):
        eng = engine(vals)
        eng.set_grid_path(tensor_cores)
        out = eng.inject(np.array(pa), np.array(pb), np.array(bs), want=("ecc", "npart", "ncoll", "rho"))
        for e, (np_, nc, rho, ecc) in enumerate(res):
            assert tuple(out["npart"][e]) == np_ and out["ncoll"][e] == nc, (tensor_cores, e)
            assert np.abs(out["rho"][e] - rho).max() <= GRID_RTOL * rho.max(), (tensor_cores, e)
            assert_ecc_close(out["ecc"][e], ecc)


def _ks(a, b):
    from scipy.stats import ks_2samp
    return ks_2samp(a, b).pvalue


@pytest.mark.parametrize("name", list(NATIVE_SYSTEMS))
def test_distributions_match_reference_sampler(golden, name):
    """The GPU's Philox sampler against the reference's own drand48 sampler
    (its op-9 eccentricity table, tests/golden/ecc_native_systems.npz) at the
    same nuclear geometry: Npart, Ncoll, b, |eps_2|, |eps_3|."""
    ref = golden("ecc_native_systems.npz")[name]
    vals = values(NATIVE_SYSTEMS[name], ecc_from_order=2, ecc_to_order=5)
    eng = engine(vals, seed=17)
    ecc = eng.generate(0, 4000, want=("ecc",))["ecc"]
    for col in (45, 46, 48):
        assert _ks(ecc[:, col], ref[:, col]) > 1e-3, col
    for n in (2, 3):
        e_gpu = np.hypot(ecc[:, 5 * (n - 1) + 2], ecc[:, 5 * (n - 1) + 3])
        e_ref = np.hypot(ref[:, 5 * (n - 1) + 2], ref[:, 5 * (n - 1) + 3])
        assert _ks(e_gpu, e_ref) > 1e-3, n


def test_deformed_ecc_files_carry_the_orientations(tmp_path):
    """Generated deformed U+U events written in the deformed layout: the four
    appended fields are each event's orientations."""
    from supermc_gb300.output import write_ecc
    vals = values(NATIVE_SYSTEMS["uu200"], ecc_from_order=2, ecc_to_order=3)
    eng = engine(vals, seed=4)
    out = eng.generate(0, 16, want=("ecc", "orientation"))
    write_ecc(out["ecc"], 2, 3, str(tmp_path / "sn_ecc_eccp_%d.dat"), orientation=out["orientation"])
    for order in (2, 3, 10):
        back = np.loadtxt(tmp_path / f"sn_ecc_eccp_{order}.dat", ndmin=2)
        assert back.shape[1] == (13 if order < 10 else 53)
        np.testing.assert_allclose(back[:, -4:], out["orientation"], rtol=1e-7, atol=1e-12)
