"""GPU path (through the C ABI) against the reference fixtures and the oracle.

Bars: Npart, Ncoll and participant sets bit-exact; grids within 2e-5 of the
grid maximum (FP32 splat against FP64); eccentricities eps_1..eps_9 within
1e-6 absolute (the reference prints 8 significant digits).
"""
import ctypes

import numpy as np
import pytest

from systems import SYSTEMS, oracle_params, values

pytestmark = pytest.mark.gpu

ECC_ATOL = 1e-6
GRID_RTOL = 2e-5
RN_COLS = [5 * n + 4 for n in range(9)]                    # <r^n>, n = 1..9
EPS_COLS = [5 * n + k for n in range(9) for k in range(4)]  # Re, Im of eps_n


def assert_ecc_close(got, want):
    """eps_n within 1e-6 absolute; <r^n> within 1e-6 relative; Npart, Ncoll,
    b exact and the integral within 1e-6 relative."""
    got, want = np.atleast_2d(got), np.atleast_2d(want)
    np.testing.assert_allclose(got[:, EPS_COLS], want[:, EPS_COLS], rtol=0, atol=ECC_ATOL)
    np.testing.assert_allclose(got[:, RN_COLS], want[:, RN_COLS], rtol=1e-6, atol=0)
    np.testing.assert_array_equal(got[:, [45, 46]], want[:, [45, 46]])
    np.testing.assert_allclose(got[:, 47], want[:, 47], rtol=1e-6)
    np.testing.assert_allclose(got[:, 48], want[:, 48], rtol=1e-7)


def engine(vals, seed=1, **kw):
    from supermc_gb300.engine import Engine
    return Engine({k: v for k, v in vals.items()}, seed=seed, **kw)


def ecc_cols(ecc, orders):
    """(Re,Im) r^2 and r^n weighted columns of the given orders."""
    idx = []
    for n in orders:
        idx += [5 * (n - 1) + k for k in range(4)]
    return ecc[..., idx]


def _digest(grid, g, key):
    cells = g[key + "_cells"].astype(int)
    ref = g[key + "_values"]
    got = grid[cells[:, 0], cells[:, 1]].astype(np.float64)
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= GRID_RTOL * scale
    np.testing.assert_allclose(grid.sum(axis=1), g[key + "_rowsum"], rtol=0, atol=GRID_RTOL * scale * 50)


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_injected_fixture_events(golden, name):
    g = golden("glauber_inject.npz")
    vals = values(SYSTEMS[name])
    eng = engine(vals)
    out = eng.inject(g[name + "_pos_a"], g[name + "_pos_b"], g[name + "_b"],
                     want=("ecc", "npart", "ncoll", "rho", "ta", "tb", "positions", "wounded", "collisions"))
    np.testing.assert_array_equal(out["npart"][:, 0], g[name + "_npart1"])
    np.testing.assert_array_equal(out["npart"][:, 1], g[name + "_npart2"])
    np.testing.assert_array_equal(out["ncoll"], g[name + "_ncoll"])
    A = eng.A
    for k in range(len(g[name + "_b"])):
        pos, wnd = out["positions"][k], out["wounded"][k].astype(bool)
        for w, key in ((0, "partA"), (1, "partB")):
            sl = slice(0, A) if w == 0 else slice(A, None)
            got = pos[sl][wnd[sl]]
            ref = g[name + f"_ev{k}_{key}"]
            np.testing.assert_array_equal(got[np.lexsort(got.T)], ref[np.lexsort(ref.T)])
        # binary-collision positions of the reference's own run, in its order
        ref_coll = g[f"{name}_ev{k}_coll"]
        np.testing.assert_array_equal(out["collisions"][k][:out["ncoll"][k]], ref_coll.reshape(-1, 2))
        if k in (1, 3):
            for gname in ("ta", "tb", "rho"):
                _digest(out[gname][k], g, f"{name}_ev{k}_{gname}")
    assert_ecc_close(out["ecc"], g[name + "_ecc"])


def _oracle_events(oracle, vals, n, seed):
    """Positions from the oracle's Philox sampler plus the oracle's results
    for those positions injected (the injection semantics the GPU's
    smc_inject follows: a sampled nucleon's box is built at its
    nucleus-frame point and moved, an injected one's at its position, so
    the eccentricity hot-spot lattice can differ by a cell between the two)."""
    p = oracle_params(vals)
    ev = oracle.event(p)
    nA = oracle.nucleus(int(vals["aproj"]))
    nB = oracle.nucleus(int(vals["atarg"]))
    rng = np.random.default_rng(seed)
    pa, pb, bs, res = [], [], [], []
    tries = 0
    while len(bs) < n:
        b = float(rng.uniform(0, 16))
        ev.populate_philox(nA, nB, b, seed, len(bs) + 1000 * tries, 0)
        tries += 1
        if ev.pair() == 0:
            continue
        xa, xb = ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]
        ev.inject(xa, xb)
        nc = ev.pair()
        ev.thickness(); ev.density()
        pa.append(xa); pb.append(xb); bs.append(b)
        res.append((ev.npart(), nc, ev.grid(2), ev.eccentricities(1, 9, b)))
    return np.array(pa), np.array(pb), np.array(bs), res


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_injected_random_events_vs_oracle(oracle, name):
    vals = values(SYSTEMS[name])
    pa, pb, bs, res = _oracle_events(oracle, vals, 48, 11)
    eng = engine(vals)
    out = eng.inject(pa, pb, bs, want=("ecc", "npart", "ncoll", "rho"))
    for k, (np_, nc, rho, ecc) in enumerate(res):
        assert tuple(out["npart"][k]) == np_
        assert out["ncoll"][k] == nc
        assert np.abs(out["rho"][k] - rho).max() <= GRID_RTOL * rho.max()
        assert_ecc_close(out["ecc"][k], ecc)


@pytest.mark.parametrize("over", [
    dict(sub_model=2),                                   # Heinz-Qiu-Moreland weights
    dict(which_mc_model=7),                              # sqrt(T_A T_B)
    dict(shape_of_entropy=1),                            # disk entropy
    dict(shape_of_nucleons=2),                           # width from sigma
    dict(shape_of_nucleons=1, shape_of_entropy=1),       # disk nucleons
    dict(collision_criterion=2),                         # Gaussian collision profile
    dict(alpha=0.0),
    dict(cc_fluctuation_model=6),                        # Gamma multiplicity weights
    dict(cc_fluctuation_model=6, sub_model=2),
    dict(cc_fluctuation_model=6, which_mc_model=7),
    dict(cc_fluctuation_model=6, shape_of_entropy=1),
])
def test_model_variants_vs_oracle(oracle, over):
    vals = values(SYSTEMS["auau200"], **over)
    pa, pb, bs, _ = _oracle_events(oracle, values(SYSTEMS["auau200"]), 8, 5)
    ev = oracle.event(oracle_params(vals))
    eng = engine(vals, seed=0)
    out = eng.inject(pa, pb, bs, want=("ecc", "npart", "ncoll", "rho"))
    for k in range(len(bs)):
        # the injected batch draws event k's Philox streams at attempt 0
        oracle.lib.smco_set_pair_stream(0, k, 0, 1)
        ev.inject(pa[k], pb[k])
        nc = ev.pair()
        assert out["ncoll"][k] == nc and tuple(out["npart"][k]) == ev.npart()
        assert ev.thickness() == 0
        if ev.density() != 0:
            continue
        rho = ev.grid(2)
        assert np.abs(out["rho"][k] - rho).max() <= GRID_RTOL * rho.max()
        assert_ecc_close(out["ecc"][k], ev.eccentricities(1, 9, bs[k]))
    oracle.lib.smco_set_pair_stream(0, 0, 0, 0)


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_generated_positions_follow_oracle_sampler(oracle, name):
    """The GPU sampler (FP32 arithmetic) draws the same Philox streams as the
    oracle's sampler (FP64): nucleons agree to 1e-4 fm in (nearly) all events."""
    vals = values(SYSTEMS[name])
    eng = engine(vals, seed=3)
    n = 64
    out = eng.generate(0, n, want=("npart", "ncoll", "b", "attempts", "positions"))
    p = oracle_params(vals)
    ev = oracle.event(p)
    nA = oracle.nucleus(int(vals["aproj"]))
    nB = oracle.nucleus(int(vals["atarg"]))
    agree = 0
    for e in range(n):
        att = out["attempts"][e] - 1
        b = oracle.lib.smco_impact_philox(3, e, att, 0.0, 20.0)
        assert b == pytest.approx(out["b"][e], rel=1e-15)
        ev.populate_philox(nA, nB, b, 3, e, att)
        ref = np.concatenate([ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]])
        if np.abs(ref - out["positions"][e]).max() < 1e-4:
            agree += 1
    assert agree >= n - 2


def _ks(a, b):
    from scipy.stats import ks_2samp
    return ks_2samp(a, b).pvalue


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_generated_distributions_match_reference_sampler(golden, name):
    """Npart, Ncoll, b and eps_2, eps_3 from the GPU's Philox sampler against
    the reference's own drand48 sampler (op-9 table), same nuclear geometry."""
    ref = golden("ecc_native.npz")[name]
    vals = values(SYSTEMS[name], ecc_from_order=2, ecc_to_order=5)
    eng = engine(vals, seed=17)
    out = eng.generate(0, 4000, want=("ecc", "npart", "ncoll", "b"))
    ecc = out["ecc"]
    np_gpu = ecc[:, 45]
    assert _ks(np_gpu, ref[:, 45]) > 1e-3
    assert _ks(ecc[:, 46], ref[:, 46]) > 1e-3
    assert _ks(ecc[:, 48], ref[:, 48]) > 1e-3
    for n in (2, 3):
        e_gpu = np.hypot(ecc[:, 5 * (n - 1) + 2], ecc[:, 5 * (n - 1) + 3])
        e_ref = np.hypot(ref[:, 5 * (n - 1) + 2], ref[:, 5 * (n - 1) + 3])
        assert _ks(e_gpu, e_ref) > 1e-3


def test_plain_path_equals_batched():
    """The plain per-event path and the batched path run the same kernels
    when the batched splat is the CUDA-core one: identical results.  The
    batched tensor-core splat agrees within the grid / eps bars."""
    vals = values(SYSTEMS["pbpb2760"])
    eng = engine(vals, seed=9)
    want = ("ecc", "npart", "ncoll", "b", "rho")
    plain = eng.generate_plain(100, 24, want=want)
    eng.set_grid_path(False)
    cuda_core = eng.generate(100, 24, want=want)
    for k in want:
        np.testing.assert_array_equal(cuda_core[k], plain[k])
    eng.set_grid_path(True)
    tensor = eng.generate(100, 24, want=want)
    for k in ("npart", "ncoll", "b"):
        np.testing.assert_array_equal(tensor[k], plain[k])
    for k in range(24):
        assert np.abs(tensor["rho"][k] - plain["rho"][k]).max() <= GRID_RTOL * plain["rho"][k].max()
    assert_ecc_close(tensor["ecc"], plain["ecc"])


def test_generate_grid_and_ecc_consistent(oracle):
    """Generated events re-injected: identical results (the pipeline after
    sampling is the injected one)."""
    vals = values(SYSTEMS["auau200"])
    eng = engine(vals, seed=5)
    g = eng.generate(0, 16, want=("ecc", "npart", "ncoll", "b", "rho", "positions"))
    A = eng.A
    inj = eng.inject(g["positions"][:, :A], g["positions"][:, A:], g["b"], want=("ecc", "npart", "ncoll", "rho"))
    for k in ("ecc", "npart", "ncoll", "rho"):
        np.testing.assert_array_equal(inj[k], g[k])


def test_retry_cap_and_config_errors():
    """The reference loops forever on an impossible centrality cut
    (src/MakeDensity.cpp:2147-2162) and exits on bad input; here both are
    status codes and the context stays usable."""
    from supermc_gb300._lib import SmcError
    from supermc_gb300.engine import Engine
    eng = engine(values(SYSTEMS["auau200"], Npmin=1000, max_attempts=5))
    with pytest.raises(SmcError) as e:
        eng.generate(0, 4)
    assert e.value.status == 3
    with pytest.raises(SmcError) as e:
        Engine(dict(SYSTEMS["auau200"], which_mc_model=3))
    assert e.value.status == 2
    ok = engine(values(SYSTEMS["auau200"]))
    assert ok.generate(0, 4)["ncoll"].min() > 0


def test_kln_table_vs_oracle(oracle):
    from oracle.oracle import KLN
    vals = values(SYSTEMS["pbpb2760"], which_mc_model=1, sub_model=7, **{"lambda": 0.288})
    eng = engine(vals)
    tab = eng.kln_table()
    assert tab.shape == (211, 211)
    assert (tab[0] == 0).all() and (tab[:, 0] == 0).all()
    k = KLN()
    oracle.lib.smco_kln_init(ctypes.byref(k), 2760.0, 0.288)
    rng = np.random.default_rng(1)
    dT = eng.info.kln_dT
    for i, j in rng.integers(1, 211, size=(12, 2)):
        want = oracle.lib.smco_kln_dndy(ctypes.byref(k), i * dT, j * dT, 48, 64, 32)
        assert tab[i, j] == pytest.approx(want, rel=1e-9)


def test_kln_events_vs_oracle(oracle):
    """Injected MC-KLN events at sigma_in(2.76 TeV), at the Glauber bars (the
    GPU's table equals the oracle's own, tests/test_gpu_kln.py, where the
    benchmark workload runs against the oracle's table)."""
    from oracle.oracle import _ptr
    vals = values(SYSTEMS["pbpb2760"], which_mc_model=1, sub_model=7, **{"lambda": 0.288})
    eng = engine(vals)
    table = np.ascontiguousarray(eng.kln_table())
    pa, pb, bs, _ = _oracle_events(oracle, values(SYSTEMS["pbpb2760"]), 8, 2)
    out = eng.inject(pa, pb, bs, want=("ecc", "npart", "ncoll", "rho", "ta", "tb"))
    p = oracle_params(vals)
    p.kln_table = _ptr(table)
    p.kln_tmax = eng.info.kln_tmax
    p.kln_dT = eng.info.kln_dT
    ev = oracle.event(p)
    for k in range(len(bs)):
        ev.inject(pa[k], pb[k]); ev.pair()
        assert ev.thickness() == 0 and ev.density() == 0
        for w, key in ((0, "ta"), (1, "tb"), (2, "rho")):
            ref = ev.grid(w)
            assert np.abs(out[key][k] - ref).max() <= GRID_RTOL * ref.max()
        assert_ecc_close(out["ecc"][k], ev.eccentricities(1, 9, bs[k]))


@pytest.mark.parametrize("model,over", [
    (1, dict()),                                                         # Glauber, constant k
    (2, dict()),                                                         # Glauber, k from min(T_A, T_B)
    (2, dict(which_mc_model=1, sub_model=7, **{"lambda": 0.288})),       # MC-KLN
])
def test_nbd_fluctuations_vs_oracle(oracle, model, over):
    """Per-cell negative-binomial densities (cc_fluctuation_model 1, 2): the
    GPU draws each cell's count from the same Philox stream as the oracle.
    A cell whose FP32 mean sits within rounding of a count boundary can
    draw the neighbouring count, so nearly all events match everywhere."""
    from oracle.oracle import _ptr
    vals = values(SYSTEMS["auau200"], cc_fluctuation_model=model, cc_fluctuation_k=0.75, **over)
    pa, pb, bs, _ = _oracle_events(oracle, values(SYSTEMS["auau200"]), 8, 5)
    eng = engine(vals, seed=0)
    out = eng.inject(pa, pb, bs, want=("ecc", "npart", "ncoll", "rho"))
    p = oracle_params(vals)
    if int(vals["which_mc_model"]) == 1:
        table = np.ascontiguousarray(eng.kln_table())
        p.kln_table = _ptr(table)
        p.kln_tmax = eng.info.kln_tmax
        p.kln_dT = eng.info.kln_dT
    ev = oracle.event(p)
    area = vals["dx"] * vals["dy"]
    exact = 0
    try:
        for k in range(len(bs)):
            oracle.lib.smco_set_pair_stream(0, k, 0, 1)
            ev.inject(pa[k], pb[k])
            ev.pair()
            assert ev.thickness() == 0
            if ev.density() != 0:
                continue
            rho = ev.grid(2)
            # counts per cell: integers on both sides
            n_gpu, n_ref = out["rho"][k] * area, rho * area
            assert np.abs(n_gpu - np.round(n_gpu)).max() < 1e-3
            bad = np.abs(n_gpu - n_ref) > 0.5
            assert bad.sum() <= max(2, 1e-3 * (n_ref > 0).sum())
            if not bad.any():
                exact += 1
                assert_ecc_close(out["ecc"][k], ev.eccentricities(1, 9, bs[k]))
    finally:
        oracle.lib.smco_set_pair_stream(0, 0, 0, 0)
    assert exact >= len(bs) - 2
