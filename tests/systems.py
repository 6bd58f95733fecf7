"""Parameter sets shared by the tests (parameters.dat keys) and helpers to
build the oracle's parameter struct from them."""
import math

from supermc_gb300.params import derive, read_parameters

BASE = dict(which_mc_model=5, sub_model=1, shape_of_nucleons=4, gauss_nucl_width=0.5, collision_criterion=1,
            shape_of_entropy=2, alpha=0.118, maxx=13, maxy=13, dx=0.1, dy=0.1, cc_fluctuation_model=0,
            finalFactor=40, Npmin=2, Npmax=500, bmin=0, bmax=20, ecc_from_order=1, ecc_to_order=9,
            quark_width=0.3)
AUAU200 = dict(BASE, Aproj=197, Atarg=197, ecm=200)
PBPB2760 = dict(BASE, Aproj=208, Atarg=208, ecm=2760)
SYSTEMS = {"auau200": AUAU200, "pbpb2760": PBPB2760}

# Further collision systems, at the reference's own nuclear geometry (its
# hard-coded R, a, deformation and 0.9 fm hard core, src/Nucleus.cpp:65-111)
# so that their distributions can be compared with the reference's sampler:
# p+Pb, d+Au (Hulthen deuteron), Cu+Cu, deformed U+U.
NATIVE_SYSTEMS = {
    "ppb5020": dict(BASE, Aproj=1, Atarg=208, ecm=5020),
    "dau200": dict(BASE, Aproj=2, Atarg=197, ecm=200),
    "cucu200": dict(BASE, Aproj=63, Atarg=63, ecm=200),
    "uu200": dict(BASE, Aproj=238, Atarg=238, ecm=200, proj_deformed=1, targ_deformed=1),
}


def _ws(R, a):
    return dict(proj_r=R, proj_a=a, targ_r=R, targ_a=a)


# The same systems with Woods-Saxon parameters given by the optional keys
# (the reference has no keys for them): Cu+Cu R=4.2 a=0.596, deformed U+U
# R=6.81 a=0.55, and Au+Au R=6.38 a=0.535 with a 0.4 fm hard core at
# sigma_NN = 42 mb.
OVERRIDE_SYSTEMS = {
    "cucu200_R42": dict(NATIVE_SYSTEMS["cucu200"], **_ws(4.2, 0.596)),
    "uu200_R681": dict(NATIVE_SYSTEMS["uu200"], **_ws(6.81, 0.55)),
    "auau_R638_dmin04_sig42": dict(AUAU200, sigininn_override=42.0, proj_d_min=0.4, targ_d_min=0.4,
                                   **_ws(6.38, 0.535)),
}
ALL_SYSTEMS = dict(SYSTEMS, **NATIVE_SYSTEMS, **OVERRIDE_SYSTEMS)

# Light nuclei from configuration tables (src/Nucleus.cpp:150-164, 210-236):
# 3He+Au, 12C+Au and O+O at 200 GeV, with the synthetic tables below.
LIGHT_SYSTEMS = {
    "he3au200": dict(BASE, Aproj=3, Atarg=197, ecm=200),
    "cau200": dict(BASE, Aproj=12, Atarg=197, ecm=200),
    "oo200": dict(BASE, Aproj=16, Atarg=16, ecm=200),
}
# the reference's file for each light mass number (read from tables/)
LIGHT_FILES = {3: "he3_plaintext.dat", 4: "he4_plaintext.dat", 12: "carbon_plaintext.dat",
               16: "oxygen_plaintext.dat"}


def synthetic_configurations(A: int, nconf: int = 1500):
    """A seeded stand-in for a light nucleus's configuration table:
    [nconf][A][3] positions (fm) from an isotropic Gaussian with the
    nucleus's rms charge radius, each configuration's centre of mass at the
    origin (as in the reference's tables)."""
    import numpy as np
    rms = {3: 1.97, 4: 1.68, 12: 2.47, 16: 2.70}.get(A, 1.2 * A ** (1.0 / 3.0))
    rng = np.random.default_rng(7000 + A)
    x = rng.normal(0.0, rms / np.sqrt(3.0), size=(nconf, A, 3))
    return x - x.mean(axis=1, keepdims=True)


def write_configurations(path, A: int, xyz):
    """A configuration table in the reference's file layout for A
    (src/Nucleus.cpp:383-478): he3 records carry 4 further fields after the
    9 coordinates, carbon records 2 fields before the 36, the others none;
    17 significant digits, so the file reads back exactly."""
    lead, trail = (2 if A == 12 else 0), (4 if A == 3 else 0)
    with open(path, "w") as f:
        for k, conf in enumerate(xyz):
            fields = ["0.0"] * lead + ["%.17g" % v for v in conf.reshape(-1)] + ["0.0"] * (trail - 1 if trail else 0)
            if trail:
                fields.append(str(k + 1))
            f.write(" ".join(fields) + "\n")


def light_engine_tables(vals):
    """{A: table} of the light nuclei of a parameter set."""
    return {A: synthetic_configurations(A) for A in {int(vals["aproj"]), int(vals["atarg"])} if A in LIGHT_FILES}


def oracle_nuclei(oracle, vals, tables=None):
    """The oracle's projectile and target nuclei of a parameter set (mass
    number, deformation and the optional Woods-Saxon / hard-core keys);
    tables {A: [nconf][A][3]}: configuration tables of light nuclei."""
    tables = tables or {}
    return tuple(oracle.nucleus(int(vals[f"a{w}"]), int(vals[f"{w}_deformed"]), vals[f"{w}_r"], vals[f"{w}_a"],
                                vals[f"{w}_d_min"], conf=tables.get(int(vals[f"a{w}"])))
                 for w in ("proj", "targ"))


def values(system: dict, **over) -> dict:
    d = dict(system)
    d.update(over)
    return read_parameters(None, [f"{k}={v}" for k, v in d.items()])


def oracle_params(vals: dict, sigma_gg: float | None = None):
    from oracle.oracle import Params
    from oracle.oracle import Oracle
    d = derive(vals)
    if sigma_gg is None:
        sigma_gg = Oracle().lib.smco_sigeff(d.sigin, d.width)
    return Params(nx=d.nx, ny=d.ny, xmax=vals["maxx"], ymax=vals["maxy"], dx=vals["dx"], dy=vals["dy"],
                  width=d.width, quark_width=vals["quark_width"], dsq=d.dsq, sigin=d.sigin, sigma_gg=sigma_gg,
                  alpha=vals["alpha"], which_mc_model=int(vals["which_mc_model"]),
                  sub_model=int(vals["sub_model"]), shape_of_nucleons=int(vals["shape_of_nucleons"]),
                  shape_of_entropy=int(vals["shape_of_entropy"]),
                  collision_criterion=int(vals["collision_criterion"]), final_factor=vals["finalfactor"],
                  npmin=int(vals["npmin"]), npmax=int(vals["npmax"]),
                  cc_fluctuation_model=int(vals["cc_fluctuation_model"]),
                  cc_fluctuation_gamma_theta=vals["cc_fluctuation_gamma_theta"],
                  cc_fluctuation_k=vals["cc_fluctuation_k"])


def fmt8(a):
    """Round like the reference's text output (setprecision(8))."""
    import numpy as np
    return np.vectorize(lambda v: float("%.8g" % v))(a)


def oracle_average(oracle, vals, fill, n, orders=(2, 3), params=None):
    """The oracle through MakeDensity::generate_profile_average's per-event
    sequence (src/MakeDensity.cpp:1264-1340): density, then per order the
    reaction-plane recentre + re-splat and the rotation + re-splat.
    fill(ev, k) populates event k (False skips it); events without a
    collision are skipped.  Returns ({("rp"|"rot", order): mean grid of
    rho * finalFactor}, events used)."""
    ev = oracle.event(params if params is not None else oracle_params(vals))
    acc, used = {}, 0
    for k in range(n):
        if not fill(ev, k) or ev.pair() == 0:
            continue
        used += 1
        if ev.thickness() or ev.density():
            raise RuntimeError("oracle thickness/density failed")
        for o in orders:
            ev.recenter_resplat(o)
            acc[("rp", o)] = acc.get(("rp", o), 0.0) + ev.grid(2)
            ev.rotate_resplat(o)
            acc[("rot", o)] = acc.get(("rot", o), 0.0) + ev.grid(2)
    ff = vals["finalfactor"]
    return {key: g / used * ff for key, g in acc.items()}, used
