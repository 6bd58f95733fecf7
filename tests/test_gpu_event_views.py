"""Per-event binary-collision and spectator densities through the C ABI
(smc_outputs.rho_binary, spectator_a, spectator_b): MCnucl::calculate_rho_binary
and MCnucl::calculate_spectator_density (src/MCnucl.cpp:481-614), the grids
the reference's Jet mode writes per event (src/MakeDensity.cpp:148-498).

Bars: the grids within 2e-5 of their maximum of the FP64 oracle's on the
same nucleon positions; the event's other outputs unchanged.
"""
import numpy as np
import pytest

from systems import SYSTEMS, oracle_params, values
from test_gpu_kln import _workload
from test_gpu_parity import engine

pytestmark = pytest.mark.gpu

GRID_RTOL = 2e-5
WANT = ("npart", "ncoll", "positions", "ecc", "rho", "rho_binary", "spectator_a", "spectator_b")


def _check(oracle, vals, out, n):
    ev = oracle.event(oracle_params(vals))
    A = out["positions"].shape[1] // 2
    for k in range(n):
        ev.inject(out["positions"][k, :A], out["positions"][k, A:])
        assert ev.pair() == out["ncoll"][k]
        assert tuple(out["npart"][k]) == ev.npart()
        rb = ev.rho_binary()
        spa, spb = ev.spectator_density()
        for key, want in (("rho_binary", rb), ("spectator_a", spa), ("spectator_b", spb)):
            got = out[key][k]
            assert np.abs(got - want).max() <= GRID_RTOL * max(want.max(), 1e-30), (k, key)


@pytest.mark.parametrize("tensor_cores", [False, True], ids=["cuda_cores", "tensor_cores"])
def test_glauber_event_views(oracle, tensor_cores):
    vals = values(SYSTEMS["auau200"])
    eng = engine(vals, seed=3)
    eng.set_grid_path(tensor_cores)
    n = 16
    out = eng.generate(0, n, want=WANT)
    _check(oracle, vals, out, n)
    plain = engine(vals, seed=3)
    plain.set_grid_path(tensor_cores)
    ref = plain.generate(0, n, want=("ecc", "rho"))
    np.testing.assert_array_equal(out["rho"], ref["rho"])
    np.testing.assert_array_equal(out["ecc"], ref["ecc"])


def test_kln_event_views(oracle):
    """MC-KLN splats no collisions: the sampler keeps their records for the
    binary-collision density all the same."""
    vals = _workload()
    eng = engine(vals, seed=4)
    n = 8
    out = eng.generate(0, n, want=WANT)
    _check(oracle, vals, out, n)
    assert (out["rho_binary"].sum(axis=(1, 2)) > 0).all()


def test_event_views_plain_path(oracle):
    vals = values(SYSTEMS["pbpb2760"])
    eng = engine(vals, seed=6)
    n = 4
    out = eng.generate_plain(0, n, want=WANT)
    _check(oracle, vals, out, n)


def test_kln_average_binary_and_spectators(oracle):
    """The averaged mode's binary-collision and spectator means for MC-KLN
    (the views splat as they are, whatever the density model)."""
    from test_gpu_average import _oracle_profiles
    vals = _workload()
    eng = engine(vals, seed=8)
    n = 6
    gen = eng.generate(0, n, want=("positions", "b"))
    A = gen["positions"].shape[1] // 2
    pa, pb = gen["positions"][:, :A].copy(), gen["positions"][:, A:].copy()
    keys = ("rho_binary", "rho_binary_rp", "spectator_a", "spectator_b")
    out = eng.average_profiles(0, 0, 2, 2, want=keys, xy_proj=pa, xy_targ=pb, b=gen["b"])
    from oracle.oracle import _ptr
    table = eng.kln_table()
    p = oracle_params(vals)
    p.kln_table = _ptr(table)
    p.kln_tmax = table.shape[0]
    p.kln_dT = eng.info.kln_dT
    want, used = _oracle_profiles(oracle, vals, pa, pb, orders=(2,), params=p)
    assert used == n
    for key in keys:
        ref = want[(key, 2)]
        assert ref.max() > 0
        assert np.abs(out[key][0] - ref).max() <= 1e-4 * ref.max(), key
