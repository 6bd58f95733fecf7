"""The MCnucl call surface (supermc_gb300/host/MCnucl.h, the reference's
src/MCnucl.h:85-140 over the C ABI), driven by a C++ program through one
event as the reference's operations drive MCnucl: generateNuclei(b) until the
event has a collision and passes the centrality cut, calculateThickness,
setDensity, then recenterGrid / rotateGrid of order 2, each re-splatted.
Against the oracle on the same nucleons: Npart, Ncoll exact; T_A, T_B and
the density in each frame within 2e-5 of the grid maximum; the nuclei are
the oracle's Philox sampler's at that event and b."""
import os
import subprocess

import numpy as np
import pytest

from systems import SYSTEMS, oracle_params, values

pytestmark = pytest.mark.gpu

GRID_RTOL = 2e-5


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_mcnucl_event_vs_oracle(oracle, tmp_path, name):
    from supermc_gb300 import build
    vals = values(SYSTEMS[name])
    keys = {"which_mc_model": 5, "sub_model": 1, "Aproj": vals["aproj"], "Atarg": vals["atarg"],
            "ecm": vals["ecm"], "shape_of_nucleons": 4, "gauss_nucl_width": 0.5, "collision_criterion": 1,
            "shape_of_entropy": 2, "alpha": 0.118, "maxx": 13, "maxy": 13, "dx": 0.1, "dy": 0.1,
            "cc_fluctuation_model": 0, "quark_width": 0.3, "finalFactor": 40, "Npmin": 2, "Npmax": 500,
            "randomSeed": 9}
    (tmp_path / "parameters.dat").write_text("".join(f"{k} = {v}\n" for k, v in keys.items()))
    (tmp_path / "data").mkdir()
    r = subprocess.run([build.MCNUCL_EXE, "b=7.5"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    meta = (tmp_path / "mcnucl_meta.txt").read_text().split()
    b, np1, np2, ncoll = float(meta[0]), int(meta[1]), int(meta[2]), int(meta[3])
    dndy, tries = float(meta[4]), int(meta[11])
    ori = [float(v) for v in meta[7:11]]
    xy = np.loadtxt(tmp_path / "mcnucl_nuclei.txt")
    A = int(vals["aproj"])
    nx = ny = 261

    def grid(fname):
        return np.fromfile(tmp_path / fname, dtype=np.float32).reshape(nx, ny).astype(np.float64)

    # the nuclei: the oracle's Philox sampler at this event (ids count from 0) and b
    ev = oracle.event(oracle_params(vals))
    nuc = oracle.nucleus(A)
    event = tries - 1
    ev.populate_philox(nuc, nuc, b, 9, event, 0)
    ref_xy = np.concatenate([ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]])
    assert np.abs(ref_xy - xy).max() < 1e-4
    for w in range(2):
        u = oracle.uniform2(9, event, 0, 1 + w)
        assert ori[2 * w] == 1.0 - 2.0 * u[0] and ori[2 * w + 1] == 2 * np.pi * u[1]
    # the same nucleons through the oracle: pairing, thickness, density
    ev.inject(xy[:A], xy[A:])
    assert ev.pair() == ncoll and ev.npart() == (np1, np2)
    assert ev.thickness() == 0 and ev.density() == 0
    for plane, fname in ((0, "ta.f32"), (1, "tb.f32"), (2, "rho.f32")):
        ref = ev.grid(plane)
        assert np.abs(grid(fname) - ref).max() <= GRID_RTOL * ref.max(), fname
    assert dndy == pytest.approx(ev.grid(2).sum() * 0.1 * 0.1, rel=1e-6)
    # the averaged-mode frames of order 2 (src/MakeDensity.cpp:1289-1334)
    ev.recenter_resplat(2)
    ref = ev.grid(2)
    assert np.abs(grid("rho_rp2.f32") - ref).max() <= GRID_RTOL * ref.max()
    ev.rotate_resplat(2)
    ref = ev.grid(2)
    assert np.abs(grid("rho_pp2.f32") - ref).max() <= GRID_RTOL * ref.max()
    assert (tmp_path / "data" / "binary.dat").read_text().count("\n") == ncoll
