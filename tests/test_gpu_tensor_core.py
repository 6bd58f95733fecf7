"""The tensor-core splat (tcgen05 split-TF32 contraction plus exact removal
of the window cells beyond the reference's cut) against the FP32 CUDA-core
splat and the FP64 oracle, through the C ABI.

Bars: Npart / Ncoll identical; grids within 2e-5 of the grid maximum;
eps_n within 1e-6 absolute (MC-KLN included).
"""
import numpy as np
import pytest

from systems import SYSTEMS, oracle_params, values
from test_gpu_parity import GRID_RTOL, _oracle_events, assert_ecc_close, engine

pytestmark = pytest.mark.gpu

VARIANTS = [
    ("pbpb2760", {}),
    ("auau200", {}),
    ("auau200", dict(sub_model=2)),
    ("auau200", dict(which_mc_model=7)),
    ("auau200", dict(alpha=0.0)),
    ("pbpb2760", dict(shape_of_nucleons=2)),
    ("pbpb2760", dict(collision_criterion=2)),
]


def _both_paths(vals, pa, pb, bs, want):
    eng = engine(vals, seed=0)
    eng.set_grid_path(True)
    tc = eng.inject(pa, pb, bs, want=want)
    eng.set_grid_path(False)
    cc = eng.inject(pa, pb, bs, want=want)
    return tc, cc


@pytest.mark.parametrize("name,over", VARIANTS)
def test_tensor_core_equals_cuda_core_splat(oracle, name, over):
    base = values(SYSTEMS[name])
    pa, pb, bs, _ = _oracle_events(oracle, base, 16, 23)
    vals = values(SYSTEMS[name], **over)
    tc, cc = _both_paths(vals, pa, pb, bs, ("ecc", "npart", "ncoll", "rho"))
    np.testing.assert_array_equal(tc["npart"], cc["npart"])
    np.testing.assert_array_equal(tc["ncoll"], cc["ncoll"])
    for k in range(len(bs)):
        scale = np.abs(cc["rho"][k]).max()
        assert np.abs(tc["rho"][k] - cc["rho"][k]).max() <= GRID_RTOL * scale
    assert_ecc_close(tc["ecc"], cc["ecc"])


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_thickness_planes_vs_oracle(oracle, name):
    """Glauber with T_A, T_B requested: three accumulator planes, beyond the
    tensor-core kernel's shared memory, so the batched call takes the
    CUDA-core splat; the injected events still match the oracle."""
    vals = values(SYSTEMS[name])
    pa, pb, bs, res = _oracle_events(oracle, vals, 12, 31)
    eng = engine(vals)
    eng.set_grid_path(True)
    out = eng.inject(pa, pb, bs, want=("ecc", "rho", "ta", "tb"))
    ev = oracle.event(oracle_params(vals))
    for k in range(len(bs)):
        ev.inject(pa[k], pb[k])
        ev.pair()
        assert ev.thickness() == 0 and ev.density() == 0
        for plane, key in ((0, "ta"), (1, "tb"), (2, "rho")):
            ref = ev.grid(plane)
            assert np.abs(out[key][k] - ref).max() <= GRID_RTOL * ref.max(), (k, key)
        assert_ecc_close(out["ecc"][k], res[k][3])


def test_tensor_core_central_events_many_sources(oracle):
    """Head-on Pb+Pb: ~1800 binary collisions, several source windows and
    operand chunks per tile."""
    vals = values(SYSTEMS["pbpb2760"])
    p = oracle_params(vals)
    ev = oracle.event(p)
    nuc = oracle.nucleus(208)
    pa, pb, res = [], [], []
    for k in range(6):
        ev.populate_philox(nuc, nuc, 0.3 * k, 3, k, 0)
        xa, xb = ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]
        ev.inject(xa, xb)
        nc = ev.pair()
        ev.thickness(); ev.density()
        pa.append(xa); pb.append(xb)
        res.append((nc, ev.grid(2), ev.eccentricities(1, 9, 0.3 * k)))
    eng = engine(vals)
    eng.set_grid_path(True)
    out = eng.inject(np.array(pa), np.array(pb), 0.3 * np.arange(6), want=("ecc", "ncoll", "rho"))
    assert max(r[0] for r in res) > 1000
    for k, (nc, rho, ecc) in enumerate(res):
        assert out["ncoll"][k] == nc
        assert np.abs(out["rho"][k] - rho).max() <= GRID_RTOL * rho.max()
        assert_ecc_close(out["ecc"][k], ecc)


def test_tensor_core_generated_kln_vs_cuda_core():
    """MC-KLN generated batch (the benchmark workload's model): the same
    events through both splats."""
    vals = values(SYSTEMS["pbpb2760"], which_mc_model=1, sub_model=7, ecc_from_order=2, ecc_to_order=5,
                  sigininn_override=64.0)
    eng = engine(vals, seed=5)
    eng.set_grid_path(True)
    tc = eng.generate(0, 256, want=("ecc", "npart", "ncoll", "rho"))
    eng.set_grid_path(False)
    cc = eng.generate(0, 256, want=("ecc", "npart", "ncoll", "rho"))
    np.testing.assert_array_equal(tc["npart"], cc["npart"])
    np.testing.assert_array_equal(tc["ncoll"], cc["ncoll"])
    # dN/dy is the reference's piecewise six-point interpolation in the
    # table; both splats take each cell's stencil as the FP64 sums decide it
    scale = np.abs(cc["rho"]).max(axis=(1, 2))
    assert (np.abs(tc["rho"] - cc["rho"]).max(axis=(1, 2)) <= GRID_RTOL * scale).all()
    assert_ecc_close(tc["ecc"], cc["ecc"])


@pytest.mark.parametrize("over", [dict(maxx=15, maxy=15),                            # 301 x 301
                                  dict(maxx=12.5, maxy=12.5, dx=0.05, dy=0.05),      # 501 x 501
                                  dict(maxx=13, maxy=11.3, dx=0.1, dy=0.1)])         # 261 x 227
def test_grid_sizes_vs_oracle(oracle, over):
    """Grid shapes whose shared-memory layouts differ from 261 x 261 (odd
    word counts of the hot-spot mask), both splat paths against the oracle."""
    vals = values(SYSTEMS["auau200"], **over)
    pa, pb, bs, res = _oracle_events(oracle, vals, 4, 41)
    tc, cc = _both_paths(vals, pa, pb, bs, ("ecc", "npart", "ncoll", "rho"))
    for k, (np_, nc, rho, ecc) in enumerate(res):
        for out in (tc, cc):
            assert tuple(out["npart"][k]) == np_ and out["ncoll"][k] == nc
            assert np.abs(out["rho"][k] - rho).max() <= GRID_RTOL * rho.max()
            assert_ecc_close(out["ecc"][k], ecc)
