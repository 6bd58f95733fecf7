"""The C++ drop-in driver (supermc_gb300/_build/superMC, the reference's
main over the C ABI) writes the same files as the Python host over the same
calls: operations 9, 1 (also p_T-differential), 2 (Jet mode) and 3."""
import io
import os
import subprocess

import numpy as np
import pytest

from systems import SYSTEMS, values

pytestmark = pytest.mark.gpu

PARAMS = {"which_mc_model": 5, "sub_model": 1, "Aproj": 197, "Atarg": 197, "ecm": 200, "shape_of_nucleons": 4,
          "gauss_nucl_width": 0.5, "collision_criterion": 1, "shape_of_entropy": 2, "alpha": 0.118,
          "maxx": 13, "maxy": 13, "dx": 0.1, "dy": 0.1, "cc_fluctuation_model": 6, "randomSeed": 5,
          "ecc_from_order": 2, "ecc_to_order": 5, "use_sd": 1, "use_ed": 0, "use_block": 1, "use_4col": 1,
          "average_from_order": 2, "average_to_order": 2, "generate_reaction_plane_avg_profile": 1}


def _run(tmp_path, **over):
    from supermc_gb300 import build
    p = dict(PARAMS, **over)
    (tmp_path / "parameters.dat").write_text("".join(f"{k} = {v}\n" for k, v in p.items()))
    r = subprocess.run([build.EXE], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return p


def _engine(p):
    from supermc_gb300.engine import Engine
    q = {k: v for k, v in p.items() if k not in ("randomSeed", "operation", "nev")}
    return Engine(q, seed=p["randomSeed"])


def test_operation_9_eccentricity_files(tmp_path):
    from supermc_gb300.output import write_ecc
    p = _run(tmp_path, operation=9, nev=300)
    ref = tmp_path / "ref"
    ref.mkdir()
    out = _engine(p).generate(0, 300, want=("ecc",))
    write_ecc(out["ecc"], 2, 5, str(ref / "sn_ecc_eccp_%d.dat"))
    for order in (2, 3, 4, 5, 10):
        name = f"sn_ecc_eccp_{order}.dat"
        assert (tmp_path / "data" / name).read_text() == (ref / name).read_text(), name


def test_operation_1_profiles(tmp_path):
    from supermc_gb300.output import write_density_block
    p = _run(tmp_path, operation=1, nev=3)
    out = _engine(p).generate(0, 3, want=("rho", "npart", "ncoll", "collisions", "positions", "wounded"))
    # binary.dat: every event's collisions appended, %10.3g columns
    lines = [f"{x:10.3g}{y:10.3g}" for e in range(3) for x, y in out["collisions"][e][:out["ncoll"][e]]]
    assert (tmp_path / "data" / "binary.dat").read_text() == "".join(l + "\n" for l in lines)
    A = 197
    pos, wnd = out["positions"][2], out["wounded"][2].astype(bool)
    want = "".join(f"{x:10.3g}   {y:10.3g}   {1 if k < A else 2}\n" for k, (x, y) in enumerate(pos) if wnd[k])
    assert (tmp_path / "data" / "wounded.data").read_text() == want
    for e in range(3):
        sd = out["rho"][e].astype(np.float64) * 40.0
        write_density_block(sd, str(tmp_path / "ref_block.dat"))
        assert (tmp_path / "data" / f"sd_event_{e + 1}_block.dat").read_text() == \
            (tmp_path / "ref_block.dat").read_text()
        head = (tmp_path / "data" / f"sd_event_{e + 1}_4col.dat").read_text().split("\n", 1)[0]
        assert head == "# <npart>= %g xmax= %d ymax= %d" % (out["npart"][e].sum(), 261, 261)


def test_operation_3_averages(tmp_path):
    p = _run(tmp_path, operation=3, nev=16)
    # the means the reference writes by default (use_sd, output_TATB,
    # output_rho_binary, output_TA, output_spectator_density), requested
    # together as the driver requests them
    prof = _engine(p).average_profiles(0, 16, 2, 2, want=(
        "sd", "sd_rp", "ta_tb", "ta_tb_rp", "ta", "tb", "ta_rp", "tb_rp", "rho_binary", "rho_binary_rp",
        "spectator_a", "spectator_b"))
    for fname, key in (("sdAvg_order_2", "sd"), ("sdAvg_RP_order_2", "sd_rp"),
                       ("TATB_fromSd_order_2", "ta_tb"), ("TATB_fromSd_RP_order_2", "ta_tb_rp"),
                       ("nuclear_thickness_TA_fromSd_order_2", "ta"), ("nuclear_thickness_TB_fromSd_RP_order_2", "tb_rp"),
                       ("rho_binary_fromSd_order_2", "rho_binary"), ("spectator_density_B_fromSd_order_2", "spectator_b")):
        got = np.loadtxt(tmp_path / "data" / f"{fname}_block.dat")
        np.testing.assert_allclose(got, prof[key][0], rtol=1e-11, atol=1e-300, err_msg=fname)


def test_operation_1_cut_on_total_entropy(tmp_path):
    """cutdSdy = 1: only events with lower <= sum getRho dx dy <= upper are
    written and counted; every generated event's collisions still reach
    binary.dat (src/MakeDensity.cpp:598-617)."""
    lo, hi = 60.0, 140.0
    p = _run(tmp_path, operation=1, nev=4, cutdSdy=1, cutdSdy_lowerBound=lo, cutdSdy_upperBound=hi, use_4col=0)
    n = 400
    out = _engine(p).generate(0, n, want=("rho", "ncoll", "collisions"))
    total = out["rho"].astype(np.float64).sum(axis=(1, 2)) * (0.1 * 0.1)
    keep = np.flatnonzero((total >= lo) & (total <= hi))[:4]
    assert len(keep) == 4
    for k, e in enumerate(keep):
        assert (tmp_path / "data" / f"sd_event_{k + 1}_block.dat").exists()
        block = np.loadtxt(tmp_path / "data" / f"sd_event_{k + 1}_block.dat")
        np.testing.assert_allclose(block, out["rho"][e].astype(np.float64) * 40.0, rtol=1e-11)
    assert not (tmp_path / "data" / "sd_event_5_block.dat").exists()
    lines = [f"{x:10.3g}{y:10.3g}" for e in range(keep[-1] + 1) for x, y in out["collisions"][e][:out["ncoll"][e]]]
    assert (tmp_path / "data" / "binary.dat").read_text() == "".join(l + "\n" for l in lines)


def test_operation_2_jet_mode(tmp_path):
    """Operation 2 (MakeDensity::generate_profile_ebe_Jet, src/MakeDensity.cpp:
    148-498): the per-event tables and grids, the reference's file set (its
    quarks.data aside), contents equal to the events the library generates."""
    import json
    from supermc_gb300.output import write_density_block
    p = _run(tmp_path, operation=2, nev=3, use_4col=1, output_rho_binary=1, output_TA=1, output_rhob=1,
             output_spectator_density=1, ecc_to_order=3)
    out = _engine(p).generate(0, 3, want=("rho", "ecc", "npart", "ncoll", "collisions", "positions", "wounded",
                                          "ta", "tb", "rho_binary", "spectator_a", "spectator_b"))
    names = set(os.listdir(tmp_path / "data"))
    with open(os.path.join(os.path.dirname(__file__), "golden", "text_outputs.json")) as f:
        ref_names = set(json.load(f)["jet/files"]) - {"quarks.data"}
    # the reference's files of events 1 and 2 (it ran two); the same kinds for event 3
    assert ref_names <= names
    assert {n.replace("_event_3", "_event_1") for n in names if "_event_3" in n} <= ref_names
    A = 197
    vz = np.sqrt(1.0 - 1.0 / 100.0 ** 2)
    Y = 0.5 * np.log((1 + vz) / (1 - vz + 1e-100))
    for e in range(3):
        n = e + 1
        pos, wnd = out["positions"][e], out["wounded"][e].astype(bool)
        want = "".join(f"{x:10.3g}   {y:10.3g}   {1 if k < A else 2}\n" for k, (x, y) in enumerate(pos) if wnd[k])
        assert (tmp_path / "data" / f"ParticipantTable_event_{n}.dat").read_text() == want
        want = "".join(f"{x:10.4e}  {y:.4e}  {(Y if k < A else -Y):.4e}\n" for k, (x, y) in enumerate(pos)
                       if not wnd[k])
        assert (tmp_path / "data" / f"Spectators_event_{n}.dat").read_text() == want
        lines = [f"{x:10.3g}{y:10.3g}\n" for x, y in out["collisions"][e][:out["ncoll"][e]]]
        assert (tmp_path / "data" / f"BinaryCollisionTable_event_{n}.dat").read_text() == "".join(lines)
        got = np.loadtxt(tmp_path / "data" / f"sn_ecc_eccp_10_event_{n}.dat", ndmin=2)
        np.testing.assert_allclose(got[0], out["ecc"][e], rtol=1e-7, atol=1e-12)
        for stem, grid in (("sd", out["rho"][e] * 40.0), ("rho_binary", out["rho_binary"][e]),
                           ("nuclear_thickness_TA", out["ta"][e]), ("nuclear_thickness_TB", out["tb"][e]),
                           ("rhob", out["ta"][e].astype(np.float64) + out["tb"][e]),
                           ("spectator_density_A", out["spectator_a"][e]),
                           ("spectator_density_B", out["spectator_b"][e])):
            write_density_block(np.asarray(grid, dtype=np.float64) if stem != "sd" else
                                out["rho"][e].astype(np.float64) * 40.0, str(tmp_path / "ref_block.dat"))
            assert (tmp_path / "data" / f"{stem}_event_{n}_block.dat").read_text() == \
                (tmp_path / "ref_block.dat").read_text(), (stem, n)


def test_operation_1_pt_differential(tmp_path):
    """PT_flag < 0 with MC-KLN: the p_T-differential table and per-event
    densities (MCnucl::makeTable(ptmin, dpt, iPtmax), setDensity(iy, ipt));
    use_5col writes sd_event_<n>_5col.dat (dumpDensity5Col: setSd of every
    bin per cell), and no p_T-integrated profile is written."""
    kln = dict(which_mc_model=1, sub_model=7, **{"lambda": 0.288}, cc_fluctuation_model=0, maxx=6, maxy=6, dx=0.2,
               dy=0.2)
    p = _run(tmp_path, operation=1, nev=2, PT_flag=-1, use_5col=1, **kln)
    eng = _engine(p)
    eng.kln_pt_table(0.1, 0.1, 20)
    out = eng.generate(0, 2, want=("rho_pt", "npart"))
    names = sorted(os.listdir(tmp_path / "data"))
    assert not any(n.endswith("_block.dat") for n in names), names
    for e in range(2):
        text = (tmp_path / "data" / f"sd_event_{e + 1}_5col.dat").read_text()
        head, body = text.split("\n", 1)
        assert head == "%% <npart>= %g xmax= 61 ymax= 61 Ptmax= 20" % out["npart"][e].sum()
        got = np.loadtxt(io.StringIO(body), ndmin=2)
        want = out["rho_pt"][e].reshape(61 * 61, 20).astype(np.float64) * 40.0
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)
        assert got.max() > 0
