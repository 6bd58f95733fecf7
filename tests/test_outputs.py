"""Text outputs in the reference's layouts (smc_write_ecc,
smc_write_density_block, smc_write_density_4col): the values read back from
files the stock reference binary wrote (tests/golden/text_outputs.json, made by
tests/golden/make_golden.py --only text) are written again and must give the
same bytes.  Host code only: no GPU."""
import io
import json
import os

import numpy as np
import pytest

from supermc_gb300 import _lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "text_outputs.json")


@pytest.fixture(scope="module")
def texts():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_eccentricity_files(lib, texts, tmp_path):
    ecc = np.ascontiguousarray(np.loadtxt(io.StringIO(texts["sn_ecc_eccp_10.dat"]), ndmin=2))
    assert ecc.shape[1] == 49
    pattern = str(tmp_path / "sn_ecc_eccp_%d.dat").encode()
    # two calls append like the reference's per-event appends
    first, rest = ecc[:1].copy(), ecc[1:].copy()   # kept alive across the calls
    _lib.check(lib.smc_write_ecc(_lib.ptr(first), 1, 2, 5, pattern), "smc_write_ecc")
    _lib.check(lib.smc_write_ecc(_lib.ptr(rest), len(rest), 2, 5, pattern), "smc_write_ecc")
    for order in (2, 3, 4, 5, 10):
        name = f"sn_ecc_eccp_{order}.dat"
        assert (tmp_path / name).read_text() == texts[name], name


@pytest.mark.parametrize("event", [1, 2])
def test_density_block_and_4col(lib, texts, tmp_path, event):
    g = texts["grid"]
    block = np.ascontiguousarray(np.loadtxt(io.StringIO(texts[f"sd_event_{event}_block.dat"]), ndmin=2))
    assert block.shape == (g["nx"], g["ny"])
    out = str(tmp_path / "block.dat").encode()
    _lib.check(lib.smc_write_density_block(_lib.ptr(block), g["nx"], g["ny"], out), "smc_write_density_block")
    assert (tmp_path / "block.dat").read_text() == texts[f"sd_event_{event}_block.dat"]

    four = texts[f"sd_event_{event}_4col.dat"]
    header, body = four.split("\n", 1)
    npart = float(header.split()[2])
    cols = np.loadtxt(io.StringIO(body), ndmin=2)
    grid = np.ascontiguousarray(cols[:, 3].reshape(g["nx"], g["ny"]))
    out = str(tmp_path / "4col.dat").encode()
    _lib.check(lib.smc_write_density_4col(_lib.ptr(grid), g["nx"], g["ny"], g["xmin"], g["ymin"], g["dx"], g["dy"],
                                          0.0, npart, out), "smc_write_density_4col")
    assert (tmp_path / "4col.dat").read_text() == four


def test_writers_reject_bad_arguments(lib, tmp_path):
    e = np.zeros((1, 49))
    assert lib.smc_write_ecc(_lib.ptr(e), 1, 3, 2, str(tmp_path / "x%d").encode()) == 1
    assert lib.smc_write_density_block(None, 3, 3, str(tmp_path / "b").encode()) != 0


@pytest.mark.gpu
def test_generated_events_round_trip_through_the_writers(tmp_path):
    """GPU events written in the reference's layouts read back as the same
    numbers (at the printed precision)."""
    from supermc_gb300.engine import Engine
    from supermc_gb300.output import write_density_block, write_ecc
    eng = Engine({"which_mc_model": 5, "Aproj": 197, "Atarg": 197, "ecm": 200, "ecc_from_order": 2,
                  "ecc_to_order": 5}, seed=3)
    out = eng.generate(0, 8, want=("ecc", "rho"))
    write_ecc(out["ecc"], 2, 5, str(tmp_path / "sn_ecc_eccp_%d.dat"))
    back = np.loadtxt(tmp_path / "sn_ecc_eccp_10.dat", ndmin=2)
    np.testing.assert_allclose(back, out["ecc"], rtol=1e-7, atol=1e-12)
    for order in range(2, 6):
        per = np.loadtxt(tmp_path / f"sn_ecc_eccp_{order}.dat", ndmin=2)
        np.testing.assert_allclose(per[:, :5], out["ecc"][:, 5 * (order - 1):5 * order], rtol=1e-7, atol=1e-12)
    sd = out["rho"][0].astype(np.float64) * eng.values["finalfactor"]
    write_density_block(sd, str(tmp_path / "sd_event_1_block.dat"))
    np.testing.assert_allclose(np.loadtxt(tmp_path / "sd_event_1_block.dat"), sd, rtol=1e-11, atol=0)


def test_deformed_eccentricity_layout(lib, texts, tmp_path):
    """dumpEccentricities with a deformed nucleus appends four fields to every
    line (src/MakeDensity.cpp:2435-2455, 2483-2492).  The reference prints
    MCnucl::lastCx1, lastPh1, lastCx2, lastPh2 there, members its code never
    assigns, so the stock binary's files hold stray memory in those 64
    characters; every other byte must be the reference's, and the four fields
    hold the given orientations (%16.8g)."""
    ref10 = texts["deformed/sn_ecc_eccp_10.dat"]
    vals = np.loadtxt(io.StringIO(ref10), ndmin=2)
    assert vals.shape[1] == 53
    ecc = np.ascontiguousarray(vals[:, :49])
    n = len(ecc)
    ori = np.ascontiguousarray(np.column_stack([np.linspace(-0.9, 0.8, n), np.linspace(0.1, 6.2, n),
                                                np.linspace(0.3, -0.4, n), np.linspace(3.0, 1.0, n)]))
    pattern = str(tmp_path / "sn_ecc_eccp_%d.dat").encode()
    _lib.check(lib.smc_write_ecc_deformed(_lib.ptr(ecc), _lib.ptr(ori), n, 2, 3, pattern), "smc_write_ecc_deformed")
    for order in (2, 3, 10):
        name = f"sn_ecc_eccp_{order}.dat"
        got = (tmp_path / name).read_text().splitlines()
        want = texts["deformed/" + name].splitlines()
        assert len(got) == len(want) == n
        for k in range(n):
            assert len(got[k]) == len(want[k]), (name, k)
            assert got[k][:-64] == want[k][:-64], (name, k)
            assert got[k][-64:] == "".join("%16.8g" % v for v in ori[k]), (name, k)
    with pytest.raises(Exception):
        _lib.check(lib.smc_write_ecc_deformed(_lib.ptr(ecc), None, n, 2, 3, pattern), "smc_write_ecc_deformed")


def test_npy_files_read_by_numpy(lib, tmp_path):
    """smc_write_npy: numpy.load gives the array back; appends grow the
    first dimension; a mismatched append is refused."""
    from supermc_gb300.output import write_npy
    rng = np.random.default_rng(4)
    for dt in (np.float32, np.float64):
        for shape in ((7,), (5, 9), (3, 4, 6)):
            a = rng.normal(size=shape).astype(dt)
            f = str(tmp_path / f"a_{np.dtype(dt).name}_{len(shape)}.npy")
            write_npy(a, f)
            b = np.load(f)
            assert b.dtype == dt and b.shape == a.shape
            np.testing.assert_array_equal(b, a)
    f = str(tmp_path / "grow.npy")
    a, b = rng.normal(size=(4, 3)), rng.normal(size=(2, 3))
    write_npy(a, f, append=True)
    write_npy(b, f, append=True)
    np.testing.assert_array_equal(np.load(f), np.concatenate([a, b]))
    with pytest.raises(_lib.SmcError):   # other trailing shape
        write_npy(rng.normal(size=(2, 4)), f, append=True)
    with pytest.raises(_lib.SmcError):   # other type
        write_npy(rng.normal(size=(2, 3)).astype(np.float32), f, append=True)
    (tmp_path / "text.npy").write_text("not a npy file\n" * 20)
    with pytest.raises(_lib.SmcError):
        write_npy(a, str(tmp_path / "text.npy"), append=True)
    np.testing.assert_array_equal(np.load(f), np.concatenate([a, b]))   # untouched by the refusals


@pytest.mark.parametrize("deformed", [False, True])
def test_ecc_npy_holds_the_text_columns(lib, tmp_path, deformed):
    """sn_ecc_eccp_<order>.npy holds the columns of the text lines; the text
    is those values printed to 8 (Npart, Ncoll: 5) significant digits."""
    from supermc_gb300.output import write_ecc, write_ecc_npy
    rng = np.random.default_rng(9)
    n = 12
    ecc = rng.normal(size=(n, 49))
    ecc[:, 45:47] = rng.integers(2, 400, size=(n, 2))
    ori = np.column_stack([rng.uniform(-1, 1, n), rng.uniform(0, 6.28, n)] * 2) if deformed else None
    for half in (slice(0, 5), slice(5, n)):   # two appends
        write_ecc(ecc[half], 2, 4, str(tmp_path / "e_%d.dat"), orientation=None if ori is None else ori[half])
        write_ecc_npy(ecc[half], 2, 4, str(tmp_path / "e_%d.npy"), orientation=None if ori is None else ori[half])
    for order in (2, 3, 4, 10):
        b = np.load(tmp_path / f"e_{order}.npy")
        t = np.loadtxt(tmp_path / f"e_{order}.dat", ndmin=2)
        cols = (list(range(5 * (order - 1), 5 * order)) if order < 10 else list(range(45))) + [45, 46, 47, 48]
        want = ecc[:, cols] if ori is None else np.column_stack([ecc[:, cols], ori])
        np.testing.assert_array_equal(b, want)
        assert t.shape == b.shape
        np.testing.assert_allclose(t, b, rtol=6e-8, atol=1e-300)


def test_jet_mode_tables(lib, texts, tmp_path):
    """Operation 2's per-event tables (src/MakeDensity.cpp:148-498):
    ParticipantTable_event_<n>.dat (MCnucl::dumpparticipantTable, appended),
    Spectators_event_<n>.dat (MCnucl::dumpSpectatorsTable, beam rapidity of
    sqrt(s) = 200 GeV), BinaryCollisionTable_event_<n>.dat, and the
    per-event eccentricity files, written again from the values the
    reference's own files hold."""
    part = np.loadtxt(io.StringIO(texts["jet/ParticipantTable_event_1.dat"]), ndmin=2)
    ids = part[:, 2].astype(int)
    A, B = int((ids == 1).sum()), int((ids == 2).sum())
    xy = np.ascontiguousarray(part[:, :2])
    wounded = np.ones(A + B, dtype=np.uint8)
    out = str(tmp_path / "part.dat").encode()
    _lib.check(lib.smc_write_participant_table(_lib.ptr(xy), _lib.ptr(wounded), A, B, out),
               "smc_write_participant_table")
    assert (tmp_path / "part.dat").read_text() == texts["jet/ParticipantTable_event_1.dat"]

    spec = np.loadtxt(io.StringIO(texts["jet/Spectators_event_1.dat"]), ndmin=2)
    A, B = int((spec[:, 2] > 0).sum()), int((spec[:, 2] < 0).sum())
    xy = np.ascontiguousarray(spec[:, :2])
    none = np.zeros(A + B, dtype=np.uint8)
    out = str(tmp_path / "spec.dat").encode()
    _lib.check(lib.smc_write_spectator_table(_lib.ptr(xy), _lib.ptr(none), A, B, 200.0, out),
               "smc_write_spectator_table")
    assert (tmp_path / "spec.dat").read_text() == texts["jet/Spectators_event_1.dat"]

    coll = np.ascontiguousarray(np.loadtxt(io.StringIO(texts["jet/BinaryCollisionTable_event_1.dat"]), ndmin=2))
    out = str(tmp_path / "coll.dat").encode()
    _lib.check(lib.smc_write_binary_table(_lib.ptr(coll), len(coll), out), "smc_write_binary_table")
    assert (tmp_path / "coll.dat").read_text() == texts["jet/BinaryCollisionTable_event_1.dat"]

    ecc = np.ascontiguousarray(np.loadtxt(io.StringIO(texts["jet/sn_ecc_eccp_10_event_1.dat"]), ndmin=2))
    pattern = str(tmp_path / "sn_ecc_eccp_%d_event_1.dat").encode()
    _lib.check(lib.smc_write_ecc(_lib.ptr(ecc), 1, 2, 3, pattern), "smc_write_ecc")
    for name in ("sn_ecc_eccp_2_event_1.dat", "sn_ecc_eccp_10_event_1.dat"):
        assert (tmp_path / name).read_text() == texts["jet/" + name], name


def test_pt_differential_layout(lib, tmp_path):
    """MakeDensity::dumpDensity5Col / dumpDesityptCol (src/MakeDensity.cpp:
    2612-2661): a header line, then the p_T bins of one cell per line."""
    data = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4) * 0.5 + 0.25
    out = str(tmp_path / "pt.dat").encode()
    _lib.check(lib.smc_write_density_pt(_lib.ptr(data), 2, 3, 4, 17.0, 40.0, out), "smc_write_density_pt")
    lines = (tmp_path / "pt.dat").read_text().split("\n")
    assert lines[0] == "% <npart>= 17 xmax= 2 ymax= 3 Ptmax= 4"
    assert lines[1] == "".join("%22.12e" % (v * 40.0) for v in data[0, 0])
    assert len(lines) == 2 + 6 and lines[-1] == ""
