"""Differentiable MC-Glauber events for PyTorch.

``glauber_events(width, alpha, R, a, ...)`` returns the per-event |eps_2|,
|eps_3| (r^n weighting about the centre of mass over the hot-spot region,
MakeDensity::dumpEccentricities, src/MakeDensity.cpp:2244-2511) and,
optionally, the densities rho (MCnucl::setDensity, src/MCnucl.cpp:688-779) of
a fixed set of events, as a ``torch.autograd.Function``: the forward pass is
smc_generate, the backward pass is smc_adjoint (the hand-written adjoint
kernel, which recomputes the events instead of storing them).  The
participants, collisions, splat windows, per-cell cuts and the hot-spot
region of each event are held fixed, so the gradient is that of the smooth
part of the map (they are piecewise constant in the parameters).
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Engine

_cache: dict = {}


def _engine(base: dict, seed: int, width: float, alpha: float, R: float | None, a: float | None) -> Engine:
    key = (tuple(sorted(base.items())), seed, width, alpha, R, a)
    eng = _cache.get(key)
    if eng is None:
        if len(_cache) >= 2:
            _cache.pop(next(iter(_cache))).close()
        p = dict(base)
        p.update({"shape_of_nucleons": 4, "gauss_nucl_width": width, "alpha": alpha})
        if R is not None:
            # radii by inverse CDF, so that positions move with R and a
            p.update({"ws_inverse_cdf": 1, "proj_R": R, "targ_R": R, "proj_a": a, "targ_a": a})
        eng = Engine(p, seed=seed)
        _cache[key] = eng
    return eng


def eps23(ecc: np.ndarray) -> np.ndarray:
    """|eps_2|, |eps_3| (r^n weighting) from rows of smc_outputs.ecc."""
    e2 = np.hypot(ecc[:, 7], ecc[:, 8])
    e3 = np.hypot(ecc[:, 12], ecc[:, 13])
    return np.stack([e2, e3], axis=1)


class GlauberEvents(torch.autograd.Function):
    @staticmethod
    def forward(ctx, width, alpha, R, a, base, seed, first_event, n, want_rho):
        w, al = float(width), float(alpha)
        RR = None if R.numel() == 0 else float(R)
        aa = None if a.numel() == 0 else float(a)
        eng = _engine(base, seed, w, al, RR, aa)
        out = eng.generate(first_event, n, want=("ecc", "rho") if want_rho else ("ecc",))
        ctx.key = (base, seed, w, al, RR, aa, first_event, n)
        eps = torch.from_numpy(eps23(out["ecc"]))
        rho = torch.from_numpy(out["rho"]) if want_rho else torch.zeros(0, dtype=torch.float32)
        return eps, rho

    @staticmethod
    def backward(ctx, g_eps, g_rho):
        base, seed, w, al, RR, aa, first_event, n = ctx.key
        eng = _engine(base, seed, w, al, RR, aa)
        ge = None if g_eps is None else g_eps.detach().cpu().double().numpy()
        gr = None if g_rho is None or g_rho.numel() == 0 else g_rho.detach().cpu().float().numpy()
        grad, _ = eng.adjoint(first_event, n, g_eps=ge, g_rho=gr)
        t = [torch.tensor(x, dtype=torch.float64) for x in grad]
        gR = t[2] if RR is not None else None
        ga = t[3] if aa is not None else None
        return t[0], t[1], gR, ga, None, None, None, None, None


def glauber_events(width, alpha, R=None, a=None, *, base: dict, seed: int = 7, first_event: int = 0, n: int = 64,
                   want_rho: bool = False):
    """(eps [n,2], rho [n,nx,ny] or empty) as differentiable functions of the
    scalar tensors width, alpha and, when given, the Woods-Saxon R and a of
    both nuclei (then the radii are sampled by inverse CDF from fixed
    uniforms, so that the nucleon positions move with R and a)."""
    if (R is None) != (a is None):
        raise ValueError("give both R and a, or neither")
    R = torch.zeros(0, dtype=torch.float64) if R is None else R
    a = torch.zeros(0, dtype=torch.float64) if a is None else a
    return GlauberEvents.apply(width, alpha, R, a, base, seed, first_event, n, want_rho)
