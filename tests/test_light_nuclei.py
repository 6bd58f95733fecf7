"""Light nuclei (3He, 4He, 12C, 16O) from configuration tables, without a GPU:
the oracle's sampler against the reference's own Nucleus::populate, and the
configuration-file readers (the oracle's and the library's
smc_read_configurations) on every record layout of the reference."""
import ctypes
import os

import numpy as np
import pytest

from systems import LIGHT_FILES, SYSTEMS, oracle_params, synthetic_configurations, values, write_configurations


def _libc():
    libc = ctypes.CDLL(None)
    libc.srand48.argtypes = [ctypes.c_long]
    libc.srand.argtypes = [ctypes.c_uint]
    return libc


@pytest.mark.parametrize("A", [3, 4, 12])
def test_oracle_light_nuclei_match_reference_sampler(oracle, golden, A):
    """Nucleus::populate of a light nucleus (src/Nucleus.cpp:187-236, 555-574)
    redone by the oracle's drand48 path: configuration rand() % nconf,
    rotated by the drand48 orientation, shifted, not recentred, sorted.  The
    fixture holds the reference's nucleons and the configurations its draws
    used; the other rows of the oracle's table are left empty."""
    g = golden("light_nuclei_drand48.npz")
    nconf = int(g[f"A{A}_nconf"])
    libc = _libc()
    ev = oracle.event(oracle_params(values(SYSTEMS["auau200"])))
    for seed in (3, 11, 19):
        tab = np.zeros((nconf, A, 3))
        tab[int(g[f"A{A}_s{seed}_idx"])] = g[f"A{A}_s{seed}_conf"]
        nuc = oracle.nucleus(A, conf=tab)
        libc.srand48(seed)
        libc.srand(seed)
        ev.populate_drand48(nuc, nuc, 5.0)
        np.testing.assert_allclose(ev.nucleons(0), g[f"A{A}_s{seed}_pos"], rtol=0, atol=1e-12)


def test_light_nucleus_is_not_recentred(oracle):
    """The Philox path keeps the table's positions about the nucleus centre:
    a configuration whose centre of mass is off the origin stays off it
    (the reference does not recentre light nuclei, src/Nucleus.cpp:210-236)."""
    tab = np.tile(np.array([[1.0, 0.0, 0.0], [1.5, 0.5, 0.0], [2.0, -0.5, 0.0]]), (4, 1, 1))
    nuc = oracle.nucleus(3, conf=tab)
    au = oracle.nucleus(197)
    ev = oracle.event(oracle_params(values(SYSTEMS["auau200"])))
    ev.populate_philox(nuc, au, 4.0, 9, 0, 0)
    xyz = ev.nucleons(0)[:, :3]
    u = oracle.uniform2(9, 0, 0, 1)   # the projectile's orientation (event stream, slot 1)
    ct, phi = 1 - 2 * u[0], 2 * np.pi * u[1]
    st = np.sqrt(1 - ct * ct)
    rot = np.array([[ct * np.cos(phi), -np.sin(phi), st * np.cos(phi)],
                    [ct * np.sin(phi), np.cos(phi), st * np.sin(phi)],
                    [-st, 0.0, ct]])
    want = tab[0] @ rot.T + np.array([2.0, 0.0, 0.0])
    want = want[np.argsort(want[:, 0])]
    np.testing.assert_allclose(xyz, want, rtol=0, atol=1e-12)


def _read_lib(path, A, capacity=None):
    from supermc_gb300 import _lib
    lib = _lib.load()
    n = ctypes.c_int(-1)
    st = lib.smc_read_configurations(A, str(path).encode(), None, 0, ctypes.byref(n))
    if capacity is None:
        capacity = max(n.value, 0)
    out = np.full((max(capacity, 1), A, 3), np.nan)
    st2 = lib.smc_read_configurations(A, str(path).encode(), out.ctypes.data if capacity else None, capacity,
                                      ctypes.byref(n))
    return st, st2, n.value, out[:capacity]


@pytest.mark.parametrize("A", sorted(LIGHT_FILES))
def test_configuration_readers_on_reference_layouts(oracle, tmp_path, A):
    from oracle.oracle import read_configurations
    from supermc_gb300.build import build
    build()
    tab = synthetic_configurations(A, nconf=37)
    path = tmp_path / LIGHT_FILES[A]
    write_configurations(path, A, tab)
    np.testing.assert_array_equal(read_configurations(str(path), A), tab)
    st, st2, n, got = _read_lib(path, A)
    assert (st, st2, n) == (6, 0, 37)   # counting alone reports the capacity status
    np.testing.assert_array_equal(got, tab)
    # a smaller capacity: the first records and SMC_ERR_CAPACITY
    _, st2, n, got = _read_lib(path, A, capacity=5)
    assert (st2, n) == (6, 37)
    np.testing.assert_array_equal(got, tab[:5])


def test_configuration_reader_rejects_bad_files(tmp_path):
    from supermc_gb300.build import build
    build()
    tab = synthetic_configurations(4, nconf=3)
    good = tmp_path / "he4.dat"
    write_configurations(good, 4, tab)
    cut = tmp_path / "cut.dat"
    cut.write_text(good.read_text()[:-40])   # the last record ends early
    text = tmp_path / "text.dat"
    text.write_text("1 2 3 x\n")
    empty = tmp_path / "empty.dat"
    empty.write_text("\n")
    for path in (cut, text, empty, tmp_path / "missing.dat"):
        st, _, _, _ = _read_lib(path, 4, capacity=0)
        assert st == 1, path
    from supermc_gb300 import _lib
    lib = _lib.load()
    n = ctypes.c_int()
    assert lib.smc_read_configurations(2, str(good).encode(), None, 0, ctypes.byref(n)) == 1   # A < 3
    assert lib.smc_read_configurations(4, str(good).encode(), None, 0, None) == 1


@pytest.mark.parametrize("A", [3, 4, 12])
def test_reference_tables_read_alike(A):
    """The reference's own files, where its tree is present: both readers
    give the same table (the reference keeps every complete record)."""
    from oracle.oracle import REF_ROOT, read_configurations
    path = os.path.join(REF_ROOT, "tables", LIGHT_FILES[A])
    if not os.path.exists(path):
        pytest.skip("reference tables not present")
    from supermc_gb300.build import build
    build()
    tab = read_configurations(path, A)
    st, st2, n, got = _read_lib(path, A)
    assert st2 == 0 and n == len(tab)
    np.testing.assert_array_equal(got, tab)
