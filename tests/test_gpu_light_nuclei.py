"""Light nuclei from configuration tables through the C ABI
(smc_set_configurations / smc_load_configurations): 3He+Au, 12C+Au and O+O
with the seeded synthetic tables of tests/systems.py.

The GPU's Philox sampler against the oracle's (the light nucleus in FP64 on
both sides, so within 1e-12 fm); the distributions of generated events
against the reference's own sampler on the same tables (its op-9 table,
tests/golden/ecc_light_systems.npz; two-sample KS); mixed batches and captured
graphs with a table; the C++ driver reading tables/ as the reference does.
"""
import os
import subprocess

import numpy as np
import pytest

from systems import (LIGHT_FILES, LIGHT_SYSTEMS, light_engine_tables, oracle_nuclei, oracle_params,
                     synthetic_configurations, values, write_configurations)
from test_gpu_parity import engine

pytestmark = pytest.mark.gpu


def _light_engine(vals, seed=3):
    eng = engine(vals, seed=seed)
    for A, tab in light_engine_tables(vals).items():
        eng.set_configurations(A, tab)
    return eng


@pytest.mark.parametrize("name", list(LIGHT_SYSTEMS))
def test_light_nuclei_follow_oracle_sampler(oracle, name):
    vals = values(LIGHT_SYSTEMS[name])
    eng = _light_engine(vals)
    n = 64
    out = eng.generate(0, n, want=("npart", "ncoll", "b", "attempts", "positions", "orientation"))
    tables = light_engine_tables(vals)
    ev = oracle.event(oracle_params(vals))
    nA, nB = oracle_nuclei(oracle, vals, tables)
    A = int(vals["aproj"])
    both_light = int(vals["atarg"]) in LIGHT_FILES
    agree = 0
    for e in range(n):
        att = int(out["attempts"][e]) - 1
        b = oracle.lib.smco_impact_philox(3, e, att, vals["bmin"], vals["bmax"])
        assert b == pytest.approx(out["b"][e], rel=1e-15)
        ev.populate_philox(nA, nB, b, 3, e, att)
        # the light projectile: FP64 on both sides
        np.testing.assert_allclose(out["positions"][e][:A], ev.nucleons(0)[:, :2], rtol=0, atol=1e-12)
        ref = np.concatenate([ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]])
        tol = 1e-12 if both_light else 1e-4   # a Woods-Saxon target is sampled in FP32
        if np.abs(ref - out["positions"][e]).max() < tol:
            agree += 1
            nc = ev.pair()
            assert tuple(out["npart"][e]) == ev.npart() and out["ncoll"][e] == nc, e
    assert agree >= (n if both_light else n - 2)


def _ks(a, b):
    from scipy.stats import ks_2samp
    return ks_2samp(a, b).pvalue


@pytest.mark.parametrize("name", list(LIGHT_SYSTEMS))
def test_light_distributions_match_reference_sampler(golden, tmp_path, name):
    """The tables written in the reference's file layout and read by
    smc_load_configurations; Npart, Ncoll, b, |eps_2|, |eps_3| of generated
    events against the reference's op-9 table on the same tables."""
    ref = golden("ecc_light_systems.npz")[name]
    vals = values(LIGHT_SYSTEMS[name], ecc_from_order=2, ecc_to_order=5)
    eng = engine(vals, seed=17)
    for A in {int(vals["aproj"]), int(vals["atarg"])} & set(LIGHT_FILES):
        path = tmp_path / LIGHT_FILES[A]
        write_configurations(path, A, synthetic_configurations(A))
        eng.load_configurations(A, str(path))
    ecc = eng.generate(0, 4000, want=("ecc",))["ecc"]
    for col in (45, 46, 48):
        assert _ks(ecc[:, col], ref[:, col]) > 1e-3, col
    for n in (2, 3):
        e_gpu = np.hypot(ecc[:, 5 * (n - 1) + 2], ecc[:, 5 * (n - 1) + 3])
        e_ref = np.hypot(ref[:, 5 * (n - 1) + 2], ref[:, 5 * (n - 1) + 3])
        assert _ks(e_gpu, e_ref) > 1e-3, n


def test_table_switch_recaptures_graph_and_reaches_mixed_batches():
    """A new table reaches the next call: the captured graph is captured
    again, and a mixed batch's light system takes the context's table."""
    import torch
    vals = values(LIGHT_SYSTEMS["he3au200"], ecc_from_order=2, ecc_to_order=3)
    eng = _light_engine(vals, seed=5)
    n = 96
    dev = torch.device("cuda", 0)
    g = {"ecc": torch.zeros((n, 49), dtype=torch.float64, device=dev),
         "npart": torch.zeros((n, 2), dtype=torch.int32, device=dev)}
    eng.generate_graph_into(0, n, g)
    first = eng.generate(0, n, want=("ecc", "npart"))
    np.testing.assert_array_equal(g["ecc"].cpu().numpy(), first["ecc"])
    # a table of one fixed, far-stretched configuration: every 3He the same shape
    wide = np.tile(np.array([[[-3.0, 0.0, 0.0], [0.0, 0.0, 0.0], [3.0, 0.0, 0.0]]]), (5, 1, 1))
    eng.set_configurations(3, wide)
    eng.generate_graph_into(0, n, g)
    second = eng.generate(0, n, want=("ecc", "npart", "positions"))
    np.testing.assert_array_equal(g["ecc"].cpu().numpy(), second["ecc"])
    assert not np.array_equal(second["ecc"], first["ecc"])
    p = second["positions"][:, :3]
    span = np.hypot(p[:, 2, 0] - p[:, 0, 0], p[:, 2, 1] - p[:, 0, 1])
    assert (span <= 6.0 + 1e-9).all() and span.max() > 5.0   # projections of the 6 fm rod
    # mixed: He3+Au next to Au+Au, each event as its own system's context gives it
    systems = [dict(Aproj=3, Atarg=197, ecm=200), dict(Aproj=197, Atarg=197, ecm=200)]
    sel = (np.arange(n) % 2).astype(np.int32)
    mixed = eng.generate_mixed(systems, sel, first_event=0, want=("ecc", "npart"))
    idx = np.flatnonzero(sel == 0)
    np.testing.assert_array_equal(mixed["ecc"][idx], second["ecc"][idx])
    np.testing.assert_array_equal(mixed["npart"][idx], second["npart"][idx])
    # removing the table: Woods-Saxon 3He again
    eng.set_configurations(3, None)
    third = eng.generate(0, n, want=("ecc",))
    assert not np.array_equal(third["ecc"], second["ecc"])


def test_set_configurations_rejects_bad_tables():
    from supermc_gb300._lib import SmcError
    eng = engine(values(LIGHT_SYSTEMS["he3au200"]), seed=1)
    bad = synthetic_configurations(3, nconf=4)
    bad[2, 1, 0] = np.nan
    with pytest.raises(SmcError):
        eng.set_configurations(3, bad)
    assert eng.lib.smc_set_configurations(eng.h, 2, None, 0) == 1   # a deuteron takes no table
    with pytest.raises(ValueError):
        eng.set_configurations(3, synthetic_configurations(4, nconf=2))


def test_driver_reads_light_tables(tmp_path):
    """The C++ driver reads tables/he3_plaintext.dat from its working
    directory (src/Nucleus.cpp:383-407) and writes what the library gives
    for the same table; without the file it stops with an error, as the
    reference does."""
    from supermc_gb300 import build
    from supermc_gb300.output import write_ecc
    from test_gpu_host_cpp import PARAMS
    p = dict(PARAMS, Aproj=3, Atarg=197, cc_fluctuation_model=0, operation=9, nev=200)
    (tmp_path / "parameters.dat").write_text("".join(f"{k} = {v}\n" for k, v in p.items()))
    r = subprocess.run([build.EXE], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and "he3_plaintext.dat" in r.stdout + r.stderr
    (tmp_path / "tables").mkdir()
    tab = synthetic_configurations(3, nconf=300)
    write_configurations(tmp_path / "tables" / "he3_plaintext.dat", 3, tab)
    r = subprocess.run([build.EXE], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    from supermc_gb300.engine import Engine
    eng = Engine({k: v for k, v in p.items() if k not in ("randomSeed", "operation", "nev")}, seed=p["randomSeed"])
    eng.set_configurations(3, tab)
    out = eng.generate(0, 200, want=("ecc",))
    ref = tmp_path / "ref"
    ref.mkdir()
    write_ecc(out["ecc"], 2, 5, str(ref / "sn_ecc_eccp_%d.dat"))
    for order in (2, 3, 4, 5, 10):
        name = f"sn_ecc_eccp_{order}.dat"
        assert (tmp_path / "data" / name).read_text() == (ref / name).read_text(), name
    assert os.path.exists(tmp_path / "data" / "sn_ecc_eccp_10.dat")
