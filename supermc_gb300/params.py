"""superMC configuration: the ``parameters.dat`` key set and its reader.

The file format and key names are those of the reference's ParameterReader
(src/ParameterReader.cpp:31-198): one ``name = value`` per line, ``#`` starts
a comment, names are case-insensitive, every value is a double, and
``key=value`` command-line arguments override the file.  ``DEFAULTS`` holds
the values of the reference's shipped parameters.dat so that a partial file
still yields a complete configuration; a key the reference does not know is
rejected (the reference would silently store it).

Keys added by this implementation (each defaults to the reference's
hard-coded behaviour, see ``EXTENSION_KEYS``): Woods-Saxon radius,
diffuseness and hard-core distance per nucleus and an inelastic
cross-section override.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

# parameters.dat keys of the reference and the values it ships with
DEFAULTS: dict[str, float] = {
    "which_mc_model": 7, "sub_model": 1, "lambda": 0.138, "et": 0, "lgx": 0,
    "tmax": 71, "tmax_subdivision": 3, "alpha": 0.118, "glb_entropy_width": 0.5,
    "aproj": 208, "atarg": 208, "proj_deformed": 0, "targ_deformed": 0,
    "include_nn_correlation": 0, "shape_of_nucleons": 2, "collision_criterion": 2,
    "shape_of_entropy": 2, "quark_width": 0.3, "gaussian_lambda": 4.14,
    "gauss_nucl_width": 0.812, "ecm": 5020.0, "bmin": 0.0, "bmax": 20.0,
    "npmin": 2, "npmax": 500, "cutdsdy": 0, "cutdsdy_lowerbound": 593.51,
    "cutdsdy_upperbound": 889.53, "nev": 50000, "randomseed": -1,
    "backup_number": 100000, "operation": 9, "finalfactor": 40.0,
    "average_from_order": 2, "average_to_order": 3, "ecc_from_order": 1,
    "ecc_to_order": 9, "use_sd": 1, "use_ed": 1, "use_4col": 0, "use_block": 1,
    "use_5col": 0, "use_ptcol": 0, "pt_flag": 1, "mixedmode": 0, "pt_min": 0.1,
    "pt_max": 2, "pt_order": 2, "d_pt": 0.1, "maxx": 15.0, "maxy": 15.0,
    "dx": 0.1, "dy": 0.1, "ny": 1, "ymax": 0, "cc_fluctuation_model": 6,
    "cc_fluctuation_k": 0.75, "cc_fluctuation_gamma_theta": 0.75,
    "output_tatb": 1, "output_rho_binary": 1, "output_ta": 1, "output_rhob": 1,
    "output_spectator_density": 1, "generate_reaction_plane_avg_profile": 1,
    "gluon_field_fluctuations": 0, "gluon_distance_scaling": 1,
}

# keys this implementation adds; <= 0 keeps the reference's hard-coded value
EXTENSION_KEYS: dict[str, float] = {
    "proj_r": 0.0, "proj_a": 0.0, "targ_r": 0.0, "targ_a": 0.0,
    "proj_d_min": 0.0, "targ_d_min": 0.0, "sigininn_override": 0.0,
    # MC-KLN table quadrature (p_T x k_T x phi Gauss-Legendre nodes)
    "kln_npt": 48, "kln_nkt": 64, "kln_nphi": 32,
    # event retry cap and per-event collision capacity (0: library defaults)
    "max_attempts": 0, "max_collisions": 0,
    # Woods-Saxon radii by inverse CDF (differentiable in R and a)
    "ws_inverse_cdf": 0,
    # MC-KLN: relative band around table-cell boundaries decided from FP64
    # thickness sums (0: the FP32 error bound)
    "kln_exact_band": 0.0,
}


# other spellings accepted for extension keys (lower case)
ALIASES: dict[str, str] = {"siginnn_override": "sigininn_override"}


class ParameterError(ValueError):
    """Raised where the reference calls exit() on a bad parameter file."""


def _parse_line(line: str, out: dict[str, float], strict: bool) -> None:
    body = line.split("#", 1)[0]
    if not body.strip():
        return
    if "=" not in body:
        raise ParameterError(f'"=" symbol not found in equation assignment {line!r}')
    lhs, rhs = body.split("=", 1)
    name = lhs.strip().lower()
    name = ALIASES.get(name, name)
    try:
        value = float(rhs.strip())
    except ValueError as exc:
        raise ParameterError(f"cannot convert {rhs.strip()!r} for {name}") from exc
    if strict and name not in DEFAULTS and name not in EXTENSION_KEYS:
        raise ParameterError(f"unknown parameter {name!r}")
    out[name] = value


def read_parameters(path: str | None = None, args: list[str] | None = None,
                    strict: bool = True) -> dict[str, float]:
    """parameters.dat (optional) then key=value overrides, over DEFAULTS."""
    vals: dict[str, float] = dict(DEFAULTS)
    vals.update(EXTENSION_KEYS)
    if path is not None:
        with open(path) as f:
            for line in f:
                _parse_line(line, vals, strict)
    for a in args or []:
        _parse_line(a, vals, strict)
    return vals


def parameters_text(vals: dict[str, float]) -> str:
    """parameters.dat text of the reference's keys (extensions dropped)."""
    return "\n".join(f"{k} = {vals[k]!r}" for k in DEFAULTS) + "\n"


# ---------------------------------------------------------------------------
# derived constants (the reference computes these at start-up)

def sigma_inelastic(ecm: float) -> float:
    """sigma_in = sigma_tot - sigma_el from the PDG-96 Regge fits for pp
    (src/Regge96.cpp:27-50), in mb."""
    s = ecm * ecm
    sig = 22.0 * s ** 0.079 + 56.1 * s ** -0.46
    bel = 2.0 * 2.3 + 2.0 * 2.3 + 4.0 * s ** 0.0808 - 4.2
    return sig - 0.0511 * sig * sig / bel


def grid_points(xmax: float, dx: float) -> int:
    """Maxx = (int)((Xmax-Xmin)/dx+0.1)+1 (src/MCnucl.cpp:39)."""
    return int((xmax - (-xmax)) / dx + 0.1) + 1


@dataclass
class Derived:
    sigin: float       # sigma_in [mb]
    dsq: float         # 0.1*sigma_in/pi [fm^2] (src/MCnucl.cpp:120)
    width: float       # nucleon Gaussian width (src/GaussianNucleonsCal.cpp:34-54)
    nx: int
    ny: int


def derive(vals: dict[str, float]) -> Derived:
    sig = vals.get("sigininn_override", 0.0)
    sigin = sig if sig > 0 else sigma_inelastic(vals["ecm"])
    shape = int(vals["shape_of_nucleons"])
    if shape == 1:
        width = math.sqrt(0.1 * sigin / math.pi) / 2.0
    elif shape == 2:
        width = math.sqrt(0.1 * sigin / math.pi) / math.sqrt(8)
    elif shape == 4:
        width = vals["gauss_nucl_width"]
    else:
        raise ParameterError(f"shape_of_nucleons={shape} is not supported")
    return Derived(sigin=sigin, dsq=0.1 * sigin / math.pi, width=width,
                   nx=grid_points(vals["maxx"], vals["dx"]), ny=grid_points(vals["maxy"], vals["dy"]))
