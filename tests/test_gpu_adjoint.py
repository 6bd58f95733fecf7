"""The adjoint kernel (smc_adjoint) against FP64 central differences
(h = 1e-4) of the oracle's frozen-structure density, on Pb+Pb events whose
nucleon positions come from the oracle's Philox sampler and are injected.
Bar: 1e-4 relative per event and parameter (dL/dw, dL/dalpha)."""
import numpy as np
import pytest

from adjoint_ref import fd_gradient, grid_coords
from systems import PBPB2760, oracle_params, values

pytestmark = pytest.mark.gpu

REL = 1e-4


def _events(oracle, vals, n, seed):
    ev = oracle.event(oracle_params(vals))
    nA, nB = oracle.nucleus(int(vals["aproj"])), oracle.nucleus(int(vals["atarg"]))
    rng = np.random.default_rng(seed)
    pa, pb, bs = [], [], []
    k = 0
    while len(bs) < n:
        b = float(rng.uniform(0, 14))
        ev.populate_philox(nA, nB, b, seed, k, 0)
        k += 1
        if ev.pair() == 0:
            continue
        pa.append(ev.nucleons(0)[:, :2]); pb.append(ev.nucleons(1)[:, :2]); bs.append(b)
    return np.array(pa), np.array(pb), np.array(bs)


def _fd(oracle, vals, pa, pb, g_eps, g_rho):
    ev = oracle.event(oracle_params(vals))
    X, Y = grid_coords(vals, ev.nx, ev.ny)
    out = []
    for k in range(len(pa)):
        ev.inject(pa[k], pb[k])
        ev.pair()
        mask = ev.hotspot_mask()
        out.append(fd_gradient(ev, mask, X, Y, vals["gauss_nucl_width"], vals["alpha"],
                               None if g_eps is None else g_eps[k], None if g_rho is None else g_rho[k]))
    return np.array(out)


@pytest.fixture(scope="module")
def setup(oracle):
    vals = values(PBPB2760, ecc_from_order=2, ecc_to_order=3)
    pa, pb, bs = _events(oracle, vals, 6, 7)
    from supermc_gb300.engine import Engine
    eng = Engine({k: v for k, v in vals.items()}, seed=7)
    return vals, eng, pa, pb, bs


@pytest.mark.parametrize("which", ["eps", "rho", "both"])
def test_adjoint_against_finite_differences(oracle, setup, which):
    vals, eng, pa, pb, bs = setup
    n = len(bs)
    rng = np.random.default_rng(11)
    g_eps = rng.uniform(-1, 1, (n, 2)) if which != "rho" else None
    g_rho = rng.uniform(0, 1, (n, eng.nx, eng.ny)).astype(np.float32) if which != "eps" else None
    grad, per = eng.adjoint(0, n, g_eps=g_eps, g_rho=g_rho, xy_proj=pa, xy_targ=pb, b=bs)
    fd = _fd(oracle, vals, pa, pb, g_eps, g_rho)
    err = np.abs(per[:, :2] - fd) / np.abs(fd)
    print(which, "max rel err per parameter", err.max(axis=0))
    assert err.max() <= REL, (per[:, :2], fd)
    np.testing.assert_allclose(grad[:2], per[:, :2].sum(axis=0), rtol=1e-12)
    assert np.all(per[:, 2:] == 0)


def test_event_average_gradient(oracle, setup):
    """d<|eps_2|>/d theta and d<|eps_3|>/d theta over the sample."""
    vals, eng, pa, pb, bs = setup
    n = len(bs)
    for q in (0, 1):
        g_eps = np.zeros((n, 2))
        g_eps[:, q] = 1.0 / n
        grad, _ = eng.adjoint(0, n, g_eps=g_eps, xy_proj=pa, xy_targ=pb, b=bs)
        fd = _fd(oracle, vals, pa, pb, g_eps, None).sum(axis=0)
        np.testing.assert_allclose(grad[:2], fd, rtol=REL)


def test_generated_events_and_autograd(setup):
    """The autograd Function over smc_generate events: gradients equal
    smc_adjoint's, and central differences of the GPU forward (h = 1e-3,
    FP32) agree to their own precision."""
    import torch
    from supermc_gb300.autograd import glauber_events
    vals, _, _, _, _ = setup
    base = {k: v for k, v in vals.items() if k not in ("gauss_nucl_width", "alpha", "shape_of_nucleons")}
    w = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    a = torch.tensor(0.118, dtype=torch.float64, requires_grad=True)
    eps, _ = glauber_events(w, a, base=base, seed=7, n=32)
    loss = eps[:, 0].mean() + 0.5 * eps[:, 1].mean()
    loss.backward()
    assert torch.isfinite(w.grad) and torch.isfinite(a.grad)

    def f(ww, aa):
        e, _ = glauber_events(torch.tensor(ww, dtype=torch.float64), torch.tensor(aa, dtype=torch.float64),
                              base=base, seed=7, n=32)
        return float(e[:, 0].mean() + 0.5 * e[:, 1].mean())
    h = 1e-3
    fw = (f(0.5 + h, 0.118) - f(0.5 - h, 0.118)) / (2 * h)
    fa = (f(0.5, 0.118 + h) - f(0.5, 0.118 - h)) / (2 * h)
    # the GPU forward re-decides cuts at each width, so allow the cut jumps
    np.testing.assert_allclose(float(w.grad), fw, rtol=2e-2)
    np.testing.assert_allclose(float(a.grad), fa, rtol=2e-2)


def _fd_moved(oracle, vals, pa, pb, g_eps, g_rho, moves, h):
    """Central differences of L over nucleon displacements: moves(ev, k, s)
    gives the (dA, dB) displacement of event k for the step s * h."""
    ev = oracle.event(oracle_params(vals))
    X, Y = grid_coords(vals, ev.nx, ev.ny)
    w, al = vals["gauss_nucl_width"], vals["alpha"]
    from adjoint_ref import objective
    out = []
    for k in range(len(pa)):
        ev.inject(pa[k], pb[k])
        ev.pair()
        mask = ev.hotspot_mask()
        Lp = objective(ev.density_moved(w, al, *moves(ev, k, +1)), mask, X, Y,
                       None if g_eps is None else g_eps[k], None if g_rho is None else g_rho[k])
        Lm = objective(ev.density_moved(w, al, *moves(ev, k, -1)), mask, X, Y,
                       None if g_eps is None else g_eps[k], None if g_rho is None else g_rho[k])
        out.append((Lp - Lm) / (2 * h))
    return np.array(out)


def test_injected_position_tangents(oracle, setup):
    """dL/dR and dL/da through given nucleon tangents: each equals the
    directional derivative of L along the tangents (FP64 central
    differences of the oracle's density with displaced sources)."""
    vals, eng, pa, pb, bs = setup
    n = len(bs)
    rng = np.random.default_rng(5)
    tp = rng.normal(0, 0.3, (n, eng.A, 4))
    tt = rng.normal(0, 0.3, (n, eng.B, 4))
    g_eps = rng.uniform(-1, 1, (n, 2))
    g_rho = rng.uniform(0, 1, (n, eng.nx, eng.ny)).astype(np.float32)
    _, per = eng.adjoint(0, n, g_eps=g_eps, g_rho=g_rho, xy_proj=pa, xy_targ=pb, b=bs, tangent_proj=tp,
                         tangent_targ=tt)
    h = 1e-4
    for q, cols in ((2, slice(0, 2)), (3, slice(2, 4))):
        fd = _fd_moved(oracle, vals, pa, pb, g_eps, g_rho,
                       lambda ev, k, s: (s * h * tp[k][:, cols], s * h * tt[k][:, cols]), h)
        err = np.abs(per[:, q] - fd) / np.abs(fd)
        print("tangent", q, "max rel err", err.max())
        assert err.max() <= REL, (per[:, q], fd)


@pytest.fixture(scope="module")
def icdf_events():
    """Events of the inverse-CDF sampler (a negligible hard core, so that the
    FP32 sampler and the FP64 oracle keep the same nucleons)."""
    vals = values(PBPB2760, ecc_from_order=2, ecc_to_order=3, ws_inverse_cdf=1, proj_d_min=1e-6,
                  targ_d_min=1e-6, proj_r=6.62, targ_r=6.62, proj_a=0.546, targ_a=0.546)
    from supermc_gb300.engine import Engine
    eng = Engine({k: v for k, v in vals.items()}, seed=7)
    n = 12
    out = eng.generate(0, n, want=("ecc", "b", "attempts", "positions", "tangents", "npart", "ncoll"))
    return vals, eng, n, out


def _oracle_icdf_event(oracle, vals, out, e):
    p = oracle_params(vals)
    ev = oracle.event(p)
    nA = oracle.nucleus(208, R=6.62, a=0.546, dmin=1e-6, icdf=1)
    nB = oracle.nucleus(208, R=6.62, a=0.546, dmin=1e-6, icdf=1)
    att = int(out["attempts"][e]) - 1
    b = oracle.lib.smco_impact_philox(7, e, att, 0.0, 20.0)
    ev.populate_philox(nA, nB, b, 7, e, att)
    return ev, nA, nB


def test_inverse_cdf_sampler_follows_oracle(oracle, icdf_events):
    """Positions and tangents of the GPU's inverse-CDF sampler against the
    oracle's FP64 one (same Philox uniforms)."""
    vals, eng, n, out = icdf_events
    agree = 0
    for e in range(n):
        ev, nA, nB = _oracle_icdf_event(oracle, vals, out, e)
        pos = np.concatenate([ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]])
        tA, tB = ev.icdf_tangents(nA, nB)
        tan = np.concatenate([tA[ev.nucleon_ids(0)], tB[ev.nucleon_ids(1)]])
        if np.abs(pos - out["positions"][e]).max() < 1e-4:
            agree += 1
            np.testing.assert_allclose(out["tangents"][e], tan, atol=2e-5)
    assert agree >= n - 1


def test_inverse_cdf_adjoint_against_finite_differences(oracle, icdf_events):
    """dL/dR, dL/da of generated inverse-CDF events against FP64 central
    differences of the oracle's events, its radii re-drawn at R +- h,
    a +- h from the same uniforms, structure held."""
    vals, eng, n, out = icdf_events
    rng = np.random.default_rng(8)
    g_eps = rng.uniform(-1, 1, (n, 2))
    _, per = eng.adjoint(0, n, g_eps=g_eps)
    h = 1e-4
    ok = 0
    from adjoint_ref import objective
    for e in range(n):
        ev, nA, nB = _oracle_icdf_event(oracle, vals, out, e)
        pos = np.concatenate([ev.nucleons(0)[:, :2], ev.nucleons(1)[:, :2]])
        if np.abs(pos - out["positions"][e]).max() >= 1e-4:
            continue
        ev.pair()
        mask = ev.hotspot_mask()
        X, Y = grid_coords(vals, ev.nx, ev.ny)
        w, al = vals["gauss_nucl_width"], vals["alpha"]
        fd = []
        for dR, da in ((h, 0.0), (0.0, h)):
            Lp = objective(ev.density_moved(w, al, *ev.icdf_displacement(nA, nB, dR, da)), mask, X, Y, g_eps[e], None)
            Lm = objective(ev.density_moved(w, al, *ev.icdf_displacement(nA, nB, -dR, -da)), mask, X, Y, g_eps[e],
                           None)
            fd.append((Lp - Lm) / (2 * h))
        err = np.abs(per[e, 2:] - fd) / np.abs(fd)
        print("event", e, "R, a rel err", err)
        ok += err.max() <= REL
    # an event whose FP32 and FP64 samples differ in a pairing decision has
    # a different structure; at most one such event is allowed
    assert ok >= n - 1


def test_autograd_wrt_woods_saxon_parameters(icdf_events):
    """The autograd Function's R and a gradients are smc_adjoint's."""
    import torch
    from supermc_gb300.autograd import glauber_events
    vals, eng, n, out = icdf_events
    base = {k: v for k, v in vals.items() if k not in ("gauss_nucl_width", "alpha", "shape_of_nucleons",
                                                      "proj_r", "targ_r", "proj_a", "targ_a", "ws_inverse_cdf")}
    w = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    al = torch.tensor(0.118, dtype=torch.float64, requires_grad=True)
    R = torch.tensor(6.62, dtype=torch.float64, requires_grad=True)
    a = torch.tensor(0.546, dtype=torch.float64, requires_grad=True)
    eps, _ = glauber_events(w, al, R, a, base=base, seed=7, n=n)
    np.testing.assert_allclose(eps.detach().numpy()[:, 0], np.hypot(out["ecc"][:, 7], out["ecc"][:, 8]), rtol=1e-12)
    eps[:, 0].mean().backward()
    g = np.zeros((n, 2))
    g[:, 0] = 1.0 / n
    grad, _ = eng.adjoint(0, n, g_eps=g)
    np.testing.assert_allclose([float(w.grad), float(al.grad), float(R.grad), float(a.grad)], grad, rtol=1e-12)


def test_adjoint_with_multiplicity_fluctuations(oracle):
    """Gamma-weighted sources (cc_fluctuation_model 6, weights held fixed):
    w and alpha gradients against the oracle's frozen density with the same
    weights (its Philox stream of each injected event)."""
    vals = values(PBPB2760, ecc_from_order=2, ecc_to_order=3, cc_fluctuation_model=6)
    pa, pb, bs = _events(oracle, values(PBPB2760), 4, 19)
    from supermc_gb300.engine import Engine
    eng = Engine({k: v for k, v in vals.items()}, seed=7)
    rng = np.random.default_rng(2)
    g_eps = rng.uniform(-1, 1, (4, 2))
    g_rho = rng.uniform(0, 1, (4, eng.nx, eng.ny)).astype(np.float32)
    _, per = eng.adjoint(0, 4, g_eps=g_eps, g_rho=g_rho, xy_proj=pa, xy_targ=pb, b=bs)
    ev = oracle.event(oracle_params(vals))
    X, Y = grid_coords(vals, ev.nx, ev.ny)
    try:
        for k in range(4):
            oracle.lib.smco_set_pair_stream(7, k, 0, 1)
            ev.inject(pa[k], pb[k])
            ev.pair()
            fd = fd_gradient(ev, ev.hotspot_mask(), X, Y, vals["gauss_nucl_width"], vals["alpha"], g_eps[k], g_rho[k])
            np.testing.assert_allclose(per[k, :2], fd, rtol=REL)
    finally:
        oracle.lib.smco_set_pair_stream(0, 0, 0, 0)
