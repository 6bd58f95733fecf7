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
