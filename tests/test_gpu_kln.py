"""MC-KLN (which_mc_model 1) on the benchmark workload against the FP64 oracle
with the oracle's own dN/dy table, through the C ABI.

The oracle builds the whole table by its FP64 quadrature (the rule the GPU
uses; the reference's BASES Monte Carlo agrees with it within its own error,
tests/test_oracle.py) and evaluates every event from the GPU's nucleon
positions.  Bars: the table at every node within 1e-9 relative; Npart, Ncoll
identical; T_A, T_B and dN/dy grids within 2e-5 of the grid maximum;
eps_2..eps_5 within 1e-6 absolute; <r^n> and the integral within 1e-6
relative.  The six-point stencil of every cell (floor(T/dT)) must be the
oracle's: a cell whose FP32 thickness leaves it undecided is redone from
FP64 sums on the GPU.
"""
import os

import numpy as np
import pytest

from systems import oracle_params
from test_gpu_parity import engine

pytestmark = pytest.mark.gpu

EPS_ATOL = 1e-6
GRID_RTOL = 2e-5
N_EVENTS = 256


def _workload(**over):
    from bench import WORKLOAD
    from supermc_gb300.params import read_parameters
    d = dict(WORKLOAD)
    d.update(over)
    return read_parameters(None, [f"{k}={v}" for k, v in d.items()])


@pytest.fixture(scope="module")
def kln_oracle_table():
    from oracle.oracle import kln_table
    from supermc_gb300.params import derive
    vals = _workload()
    sub = int(vals["tmax_subdivision"])
    tmax = sub * (int(vals["tmax"]) - 1) + 1
    dT = 10.0 / derive(vals).sigin / sub
    rule = (int(vals["kln_npt"]), int(vals["kln_nkt"]), int(vals["kln_nphi"]))
    return kln_table(vals["ecm"], vals["lambda"], dT, tmax, rule, procs=os.cpu_count()), dT


def _oracle_with_table(oracle, vals, table, dT):
    from oracle.oracle import _ptr
    p = oracle_params(vals)
    p.kln_table = _ptr(table)
    p.kln_tmax = table.shape[0]
    p.kln_dT = dT
    return oracle.event(p)


def test_kln_table_every_node(kln_oracle_table):
    table, dT = kln_oracle_table
    eng = engine(_workload())
    assert eng.info.kln_dT == dT
    tab = eng.kln_table()
    assert tab.shape == table.shape == (211, 211)
    assert (tab[0] == 0).all() and (tab[:, 0] == 0).all()
    rel = np.abs(tab[1:, 1:] - table[1:, 1:]) / np.abs(table[1:, 1:])
    assert rel.max() <= 1e-9, rel.max()


def _compare_events(oracle, vals, table, dT, out, n):
    ev = _oracle_with_table(oracle, vals, table, dT)
    A = out["positions"].shape[1] // 2
    worst = 0.0
    eps_cols = [5 * (m - 1) + c for m in range(2, 6) for c in range(4)]
    rn_cols = [5 * (m - 1) + 4 for m in range(1, 10)]
    for k in range(n):
        ev.inject(out["positions"][k, :A], out["positions"][k, A:])
        nc = ev.pair()
        assert out["ncoll"][k] == nc and tuple(out["npart"][k]) == ev.npart(), k
        assert ev.thickness() == 0 and ev.density() == 0
        for plane, key in ((0, "ta"), (1, "tb"), (2, "rho")):
            ref = ev.grid(plane)
            assert np.abs(out[key][k] - ref).max() <= GRID_RTOL * ref.max(), (k, key)
        want = ev.eccentricities(2, 5, out["b"][k])
        got = out["ecc"][k]
        d = np.abs(got[eps_cols] - want[eps_cols]).max()
        worst = max(worst, d)
        assert d <= EPS_ATOL, (k, d)
        np.testing.assert_allclose(got[rn_cols], want[rn_cols], rtol=1e-6, atol=0)
        np.testing.assert_array_equal(got[[45, 46]], want[[45, 46]])
        np.testing.assert_allclose(got[47], want[47], rtol=1e-6)
    return worst


@pytest.mark.parametrize("tensor_cores", [False, True], ids=["cuda_cores", "tensor_cores"])
def test_kln_generated_events_vs_oracle(oracle, kln_oracle_table, tensor_cores):
    """256 generated events of the benchmark workload through each splat."""
    table, dT = kln_oracle_table
    vals = _workload()
    eng = engine(vals, seed=11)
    eng.set_grid_path(tensor_cores)
    out = eng.generate(0, N_EVENTS, want=("ecc", "npart", "ncoll", "b", "rho", "ta", "tb", "positions"))
    worst = _compare_events(oracle, vals, table, dT, out, N_EVENTS)
    print(f"max |d eps_2..5| = {worst:.3g}")


def test_kln_all_cells_decided_in_fp64(oracle, kln_oracle_table):
    """kln_exact_band = 1: every nonzero cell takes the FP64 thickness path
    (the path the error band sends the undecided cells to); the results
    still match the oracle, and match the default band's."""
    table, dT = kln_oracle_table
    vals = _workload(kln_exact_band=1.0)
    n = 24
    for tensor_cores in (False, True):
        eng = engine(vals, seed=13)
        eng.set_grid_path(tensor_cores)
        out = eng.generate(0, n, want=("ecc", "npart", "ncoll", "b", "rho", "ta", "tb", "positions"))
        _compare_events(oracle, vals, table, dT, out, n)
        ref = engine(_workload(), seed=13)
        ref.set_grid_path(tensor_cores)
        dflt = ref.generate(0, n, want=("ecc", "npart", "ncoll"))
        np.testing.assert_array_equal(out["npart"], dflt["npart"])
        np.testing.assert_allclose(out["ecc"], dflt["ecc"], rtol=1e-6, atol=EPS_ATOL)
