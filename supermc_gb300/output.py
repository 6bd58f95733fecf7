"""Writers of the reference's text files (host side, through the C ABI's
smc_write_* functions): eccentricity tables, density blocks and 4-column
density files, so that the reference's downstream scripts read the results
unchanged."""
from __future__ import annotations

import numpy as np

from . import _lib


def write_ecc(ecc, from_order: int, to_order: int, pattern: str = "data/sn_ecc_eccp_%d.dat",
              orientation=None) -> None:
    """Appends the MakeDensity::dumpEccentricities lines of ecc[n][49]; with
    orientation[n][4] (cos theta, phi of each nucleus) the deformed-nucleus
    layout."""
    e = np.ascontiguousarray(np.atleast_2d(ecc), dtype=np.float64)
    lib = _lib.load()
    if orientation is None:
        _lib.check(lib.smc_write_ecc(_lib.ptr(e), e.shape[0], from_order, to_order, pattern.encode()),
                   "smc_write_ecc")
        return
    o = np.ascontiguousarray(np.atleast_2d(orientation), dtype=np.float64)
    if o.shape != (e.shape[0], 4):
        raise ValueError("orientation must be [n][4]")
    _lib.check(lib.smc_write_ecc_deformed(_lib.ptr(e), _lib.ptr(o), e.shape[0], from_order, to_order,
                                          pattern.encode()), "smc_write_ecc_deformed")


def write_density_block(grid, filename: str) -> None:
    """MakeDensity::dumpDensityBlock of one [nx][ny] grid (pass the entropy
    density getRho * finalFactor, as the reference writes)."""
    g = np.ascontiguousarray(grid, dtype=np.float64)
    lib = _lib.load()
    _lib.check(lib.smc_write_density_block(_lib.ptr(g), g.shape[0], g.shape[1], filename.encode()),
               "smc_write_density_block")


def write_density_4col(grid, xmin: float, ymin: float, dx: float, dy: float, npart: float, filename: str,
                       rapidity: float = 0.0) -> None:
    """MakeDensity::dumpDensity4Col of one [nx][ny] grid."""
    g = np.ascontiguousarray(grid, dtype=np.float64)
    lib = _lib.load()
    _lib.check(lib.smc_write_density_4col(_lib.ptr(g), g.shape[0], g.shape[1], xmin, ymin, dx, dy, rapidity, npart,
                                          filename.encode()), "smc_write_density_4col")


def write_npy(array, filename: str, append: bool = False) -> None:
    """A float32 / float64 array as a NumPy .npy file through smc_write_npy
    (append: grow an appendable file of the same type and trailing shape)."""
    a = np.ascontiguousarray(array)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    shape = np.array(a.shape, dtype=np.int64)
    lib = _lib.load()
    _lib.check(lib.smc_write_npy(filename.encode(), a.ctypes.data, a.itemsize, a.ndim, shape.ctypes.data,
                                 1 if append else 0), "smc_write_npy")


def write_ecc_npy(ecc, from_order: int, to_order: int, pattern: str = "data/sn_ecc_eccp_%d.npy",
                  orientation=None) -> None:
    """write_ecc's tables as .npy files (smc_write_ecc_npy): the same
    columns at full precision, appended."""
    e = np.ascontiguousarray(np.atleast_2d(ecc), dtype=np.float64)
    o = None
    if orientation is not None:
        o = np.ascontiguousarray(np.atleast_2d(orientation), dtype=np.float64)
        if o.shape != (e.shape[0], 4):
            raise ValueError("orientation must be [n][4]")
    lib = _lib.load()
    _lib.check(lib.smc_write_ecc_npy(_lib.ptr(e), None if o is None else _lib.ptr(o), e.shape[0], from_order,
                                     to_order, pattern.encode()), "smc_write_ecc_npy")


def write_participant_table(positions, wounded, A: int, filename: str) -> None:
    """MCnucl::dumpparticipantTable (appended): the event's participants,
    positions [A+B][2] and wounded [A+B] as the generator returns them."""
    xy = np.ascontiguousarray(positions, dtype=np.float64)
    w = np.ascontiguousarray(wounded, dtype=np.uint8)
    lib = _lib.load()
    _lib.check(lib.smc_write_participant_table(_lib.ptr(xy), _lib.ptr(w), A, len(w) - A, filename.encode()),
               "smc_write_participant_table")


def write_spectator_table(positions, wounded, A: int, ecm: float, filename: str) -> None:
    """MCnucl::dumpSpectatorsTable: the non-participants with the beam
    rapidity of sqrt(s) = ecm."""
    xy = np.ascontiguousarray(positions, dtype=np.float64)
    w = np.ascontiguousarray(wounded, dtype=np.uint8)
    lib = _lib.load()
    _lib.check(lib.smc_write_spectator_table(_lib.ptr(xy), _lib.ptr(w), A, len(w) - A, ecm, filename.encode()),
               "smc_write_spectator_table")


def write_density_pt(rho_pt, npart: float, filename: str, scale: float = 1.0) -> None:
    """MakeDensity::dumpDensity5Col / dumpDesityptCol of one event's
    p_T-differential grid [nx][ny][nbins] (times scale: finalFactor for the
    entropy density)."""
    d = np.ascontiguousarray(rho_pt, dtype=np.float32)
    lib = _lib.load()
    _lib.check(lib.smc_write_density_pt(_lib.ptr(d), d.shape[0], d.shape[1], d.shape[2], npart, scale,
                                        filename.encode()), "smc_write_density_pt")
