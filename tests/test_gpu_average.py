"""Averaged-profile mode (smc_average) against the oracle's run of
MakeDensity::generate_profile_average's per-event sequence
(src/MakeDensity.cpp:1264-1340), which is pinned to the reference by
tests/test_oracle.py::test_average_sequence_matches_reference.

Bar: every mean grid within 2e-5 of its maximum (FP32 splat against FP64),
the reaction-plane means included.
"""
import numpy as np
import pytest

from systems import SYSTEMS, oracle_average, oracle_params, values

pytestmark = pytest.mark.gpu

GRID_TOL = 2e-5


def engine(vals, seed=1):
    from supermc_gb300.engine import Engine
    return Engine(dict(vals), seed=seed)


def assert_means_close(gpu_mean, gpu_rp, want, orders=(2, 3), tol=GRID_TOL):
    for q, o in enumerate(orders):
        for got, key in ((gpu_mean[q], ("rot", o)), (gpu_rp[q], ("rp", o))):
            ref = want[key]
            err = np.abs(got - ref).max()
            assert err <= tol * ref.max(), f"{key}: max error {err:.3g} of max {ref.max():.4g}"


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_average_injected_vs_oracle(oracle, golden, name):
    g = golden("glauber_inject.npz")
    vals = values(SYSTEMS[name])
    pa, pb, bs = g[name + "_pos_a"], g[name + "_pos_b"], g[name + "_b"]
    eng = engine(vals)
    mean, mean_rp = eng.average(0, 0, 2, 3, True, xy_proj=pa, xy_targ=pb, b=bs)

    def fill(ev, k):
        ev.inject(pa[k], pb[k])
        return True

    want, used = oracle_average(oracle, vals, fill, len(bs))
    assert used == len(bs)
    assert_means_close(mean, mean_rp, want)
    # the rotation's truncated re-splat loses a visible part of the entropy
    assert mean[0].sum() < mean_rp[0].sum()


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_average_generated_vs_oracle_sampler(oracle, name):
    """Generated events: the GPU sampler (FP32) and the oracle's Philox
    sampler (FP64) draw the same streams; events whose nucleons agree to
    1e-4 fm are averaged one by one.  The rotation restores each Woods-Saxon
    participant's box to its nucleus-frame construction point."""
    vals = values(SYSTEMS[name])
    eng = engine(vals, seed=11)
    n = 12
    out = eng.generate(0, n, want=("b", "attempts", "positions", "ncoll"))
    nA, nB = oracle.nucleus(int(vals["aproj"])), oracle.nucleus(int(vals["atarg"]))
    ev = oracle.event(oracle_params(vals))
    checked = 0
    for e in range(n):
        att = int(out["attempts"][e]) - 1
        b = float(out["b"][e])
        ev.populate_philox(nA, nB, b, 11, e, att)
        ref = np.concatenate([ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]])
        if np.abs(ref - out["positions"][e]).max() >= 1e-4:
            continue
        mean, mean_rp = eng.average(e, 1, 2, 3, True)

        def fill(evo, k, e=e, att=att, b=b):
            evo.populate_philox(nA, nB, b, 11, e, att)
            return True

        want, used = oracle_average(oracle, vals, fill, 1)
        assert used == 1
        assert_means_close(mean, mean_rp, want, tol=5e-5)
        checked += 1
        if checked == 4:
            break
    assert checked >= 3


def test_average_batch_equals_single_events():
    """The mean over a batch equals the mean of one-event means: events do
    not interact, whatever the chunking."""
    vals = values(SYSTEMS["pbpb2760"])
    eng = engine(vals, seed=5)
    n = 6
    mean, mean_rp = eng.average(100, n, 2, 4, True)
    acc = np.zeros_like(mean)
    acc_rp = np.zeros_like(mean_rp)
    for e in range(n):
        m, r = eng.average(100 + e, 1, 2, 4, True)
        acc += m
        acc_rp += r
    np.testing.assert_allclose(mean, acc / n, rtol=0, atol=1e-6 * mean.max())
    np.testing.assert_allclose(mean_rp, acc_rp / n, rtol=0, atol=1e-6 * mean_rp.max())
    m_only, none = eng.average(100, n, 2, 4, False)
    assert none is None
    assert m_only.shape == mean.shape and np.isfinite(m_only).all()


def test_average_kln_vs_oracle(oracle, golden):
    from oracle.oracle import _ptr
    g = golden("glauber_inject.npz")
    vals = values(SYSTEMS["pbpb2760"], which_mc_model=1, sub_model=7, **{"lambda": 0.288})
    eng = engine(vals)
    table = np.ascontiguousarray(eng.kln_table())
    pa, pb, bs = g["pbpb2760_pos_a"][:4], g["pbpb2760_pos_b"][:4], g["pbpb2760_b"][:4]
    mean, mean_rp = eng.average(0, 0, 2, 3, True, xy_proj=pa, xy_targ=pb, b=bs)
    p = oracle_params(vals)
    p.kln_table = _ptr(table)
    p.kln_tmax = eng.info.kln_tmax
    p.kln_dT = eng.info.kln_dT

    def fill(ev, k):
        ev.inject(pa[k], pb[k])
        return True

    want, used = oracle_average(oracle, vals, fill, len(bs), params=p)
    assert used == len(bs)
    assert_means_close(mean, mean_rp, want, tol=1e-4)


def _oracle_profiles(oracle, vals, pa, pb, orders=(2, 3), params=None):
    """The averaged-mode grids of the oracle after each frame's transform:
    sd, T_A, T_B, T_A T_B, rho_binary, spectators A and B."""
    from systems import oracle_params as op
    ev = oracle.event(params if params is not None else op(vals))
    acc, used = {}, 0
    for k in range(len(pa)):
        ev.inject(pa[k], pb[k])
        if ev.pair() == 0:
            continue
        used += 1
        assert ev.thickness() == 0 and ev.density() == 0
        for o in orders:
            for frame, step in (("rp", ev.recenter_resplat), ("rot", ev.rotate_resplat)):
                assert step(o) == 0
                ta, tb = ev.grid(0), ev.grid(1)
                spa, spb = ev.spectator_density()
                grids = {"sd": ev.grid(2) * vals["finalfactor"], "ta": ta, "tb": tb, "ta_tb": ta * tb,
                         "rho_binary": ev.rho_binary(), "spectator_a": spa, "spectator_b": spb}
                for name, gr in grids.items():
                    key = (name + ("_rp" if frame == "rp" else ""), o)
                    acc[key] = acc.get(key, 0.0) + gr
    return {k: v / used for k, v in acc.items()}, used


ALL = ("sd", "sd_rp", "ta_tb", "ta_tb_rp", "ta", "tb", "ta_rp", "tb_rp", "rho_binary", "rho_binary_rp",
       "spectator_a", "spectator_b", "spectator_a_rp", "spectator_b_rp")


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_average_profiles_all_grids_vs_oracle(oracle, golden, name):
    """T_A T_B, T_A, T_B, rho_binary and spectator means of the averaged mode
    (MakeDensity.cpp:1342-1386, both frames) against the oracle."""
    g = golden("glauber_inject.npz")
    vals = values(SYSTEMS[name])
    pa, pb, bs = g[name + "_pos_a"], g[name + "_pos_b"], g[name + "_b"]
    eng = engine(vals)
    out = eng.average_profiles(0, 0, 2, 3, want=ALL, xy_proj=pa, xy_targ=pb, b=bs)
    want, used = _oracle_profiles(oracle, vals, pa, pb)
    assert eng.last_average_events == used
    for key in ALL:
        for q, o in enumerate((2, 3)):
            ref = want[(key, o)]
            err = np.abs(out[key][q] - ref).max()
            assert err <= GRID_TOL * max(ref.max(), 1e-30), f"{key} order {o}: {err:.3g} of {ref.max():.4g}"


def test_average_profiles_sd_equals_smc_average(golden):
    g = golden("glauber_inject.npz")
    vals = values(SYSTEMS["auau200"])
    pa, pb, bs = g["auau200_pos_a"], g["auau200_pos_b"], g["auau200_b"]
    eng = engine(vals)
    mean, mean_rp = eng.average(0, 0, 2, 3, True, xy_proj=pa, xy_targ=pb, b=bs)
    out = eng.average_profiles(0, 0, 2, 3, want=("sd", "sd_rp", "ta_tb"), xy_proj=pa, xy_targ=pb, b=bs)
    np.testing.assert_allclose(out["sd"], mean, rtol=0, atol=1e-6 * mean.max())
    np.testing.assert_allclose(out["sd_rp"], mean_rp, rtol=0, atol=1e-6 * mean_rp.max())
