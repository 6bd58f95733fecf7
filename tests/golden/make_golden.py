"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a container that holds the reference source tree (--ref, default
the SUPERMC_REFERENCE_ROOT setting of oracle/oracle.py): it builds oracle/_ref/libsmc_ref.so from those sources
(oracle/Makefile.ref) and drives the reference's own code through the
injection harness (oracle/ref_harness.cpp).  The fixtures then pin the
oracle and the GPU path on machines without the reference.

    python tests/golden/make_golden.py [--ref <reference tree>]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle.oracle import REF_ROOT, Reference, build_reference  # noqa: E402
from supermc_gb300.params import parameters_text, read_parameters  # noqa: E402

# parameter sets (parameters.dat keys) of the fixtures
SYSTEMS = {
    "auau200": ["which_mc_model=5", "sub_model=1", "shape_of_nucleons=4", "gauss_nucl_width=0.5",
                "collision_criterion=1", "shape_of_entropy=2", "alpha=0.118", "ecm=200", "maxx=13", "maxy=13",
                "dx=0.1", "dy=0.1", "cc_fluctuation_model=0", "Aproj=197", "Atarg=197", "operation=0",
                "use_ed=0", "finalFactor=40", "Npmin=2", "Npmax=500", "bmin=0", "bmax=20",
                "ecc_from_order=1", "ecc_to_order=9"],
    "pbpb2760": ["which_mc_model=5", "sub_model=1", "shape_of_nucleons=4", "gauss_nucl_width=0.5",
                 "collision_criterion=1", "shape_of_entropy=2", "alpha=0.118", "ecm=2760", "maxx=13",
                 "maxy=13", "dx=0.1", "dy=0.1", "cc_fluctuation_model=0", "Aproj=208", "Atarg=208",
                 "operation=0", "use_ed=0", "finalFactor=40", "Npmin=2", "Npmax=500", "bmin=0", "bmax=20",
                 "ecc_from_order=1", "ecc_to_order=9"],
}


EOS_DIR = os.path.join(REF_ROOT, "EOS")
TABLES_DIR = os.path.join(REF_ROOT, "tables")


def ref_for(args, extra=()):
    vals = read_parameters(None, list(SYSTEMS[args[0]]) + list(extra), strict=False)
    return Reference(parameters_text(vals), eos_dir=EOS_DIR), vals


def grid_digest(g: np.ndarray, rng: np.random.Generator, ncell: int = 1500):
    nz = np.argwhere(g != 0)
    pick = nz[rng.choice(len(nz), size=min(ncell, len(nz)), replace=False)] if len(nz) else np.zeros((0, 2), int)
    return {"cells": pick.astype(np.int16), "values": g[pick[:, 0], pick[:, 1]] if len(pick) else np.zeros(0),
            "rowsum": g.sum(axis=1), "colsum": g.sum(axis=0), "total": np.array(g.sum())}


def sample_positions(ref: Reference, b: float):
    """Both nuclei from the reference's own sampler (Nucleus::populate)."""
    a = ref.populate(0, b / 2.0)[:, :2].copy()
    t = ref.populate(1, -b / 2.0)[:, :2].copy()
    return a, t


def make_inject(out):
    rng = np.random.default_rng(20261203)
    data = {}
    for name in SYSTEMS:
        ref, vals = ref_for([name])
        ev_pos_a, ev_pos_b, ev_b, ecc, np1, np2, nc, partA, partB, colls = [], [], [], [], [], [], [], [], [], []
        digests = {}
        for k, b in enumerate([0.7, 3.1, 5.6, 8.2, 10.9, 13.4]):
            ref.srand(1000 + k)
            xa, xb = sample_positions(ref, b)
            n1, n2, c = ref.inject(xa, xb)
            e = ref.eccentricities(1, 9, n1 + n2, c, b)
            ev_pos_a.append(xa); ev_pos_b.append(xb); ev_b.append(b)
            ecc.append(e); np1.append(n1); np2.append(n2); nc.append(c)
            partA.append(ref.participants(0)); partB.append(ref.participants(1)); colls.append(ref.collisions())
            if k in (1, 3):
                for w, gname in enumerate(("ta", "tb", "rho")):
                    for kk, vv in grid_digest(ref.grid(w), rng).items():
                        digests[f"ev{k}_{gname}_{kk}"] = vv
        pre = f"{name}_"
        data.update({pre + "pos_a": np.array(ev_pos_a), pre + "pos_b": np.array(ev_pos_b),
                     pre + "b": np.array(ev_b), pre + "ecc": np.array(ecc), pre + "npart1": np.array(np1),
                     pre + "npart2": np.array(np2), pre + "ncoll": np.array(nc)})
        for k in range(len(ev_b)):
            data[pre + f"ev{k}_partA"] = partA[k]
            data[pre + f"ev{k}_partB"] = partB[k]
            data[pre + f"ev{k}_coll"] = colls[k]
        data.update({pre + k: v for k, v in digests.items()})
        c = ref.constants()
        data[pre + "constants"] = np.array([c["dsq"], c["width"], c["sigma_gg"], c["sigin"]])
        # averaged-mode rotation of the event with b = 8.2 fm (orders 2, 3)
        xa, xb = ev_pos_a[3], ev_pos_b[3]
        ref.inject(xa, xb)
        for order in (2, 3):
            ref.rotate_resplat(order)
            for kk, vv in grid_digest(ref.grid(2), rng).items():
                data[pre + f"rot{order}_rho_{kk}"] = vv
    np.savez_compressed(os.path.join(out, "glauber_inject.npz"), **data)


AVG_EVENTS = [(3001, 2.4), (3002, 6.5), (3003, 9.8), (3004, 4.1)]   # (drand48 seed, b)


def make_average(out):
    """MakeDensity::generate_profile_average's per-event sequence on events
    from the reference's own sampler: density, then for orders 2 and 3 the
    reaction-plane recentre + re-splat and the rotation + re-splat; the
    event means of getRho * finalFactor are digested."""
    rng = np.random.default_rng(77)
    data = {}
    for name in SYSTEMS:
        ref, vals = ref_for([name])
        ff = float(vals["finalfactor"])
        acc = {(o, m): 0.0 for o in (2, 3) for m in ("rp", "rot")}
        used = []
        for seed, b in AVG_EVENTS:
            ref.srand(seed)
            n1, n2, nc = ref.sample_event(b)
            if nc == 0:
                continue
            used.append((seed, b))
            ref.density()
            for o in (2, 3):
                ref.recenter_resplat(o)
                acc[(o, "rp")] = acc[(o, "rp")] + ref.grid(2)
                ref.rotate_resplat(o)
                acc[(o, "rot")] = acc[(o, "rot")] + ref.grid(2)
        data[name + "_events"] = np.array(used)
        for (o, m), g in acc.items():
            for kk, vv in grid_digest(g / len(used) * ff, rng).items():
                data[f"{name}_{m}{o}_{kk}"] = vv
    np.savez_compressed(os.path.join(out, "average.npz"), **data)


def make_sampler(out):
    data = {}
    for A, deformed in [(208, 0), (197, 0), (238, 1), (63, 0), (2, 0), (1, 0)]:
        ref, _ = ref_for(["pbpb2760"], [f"Aproj={A}", f"Atarg={A}", f"proj_deformed={deformed}",
                                        f"targ_deformed={deformed}"])
        for seed in (3, 11):
            ref.srand(seed)
            data[f"A{A}_d{deformed}_s{seed}"] = ref.populate(0, 2.5)
    np.savez_compressed(os.path.join(out, "sampler_drand48.npz"), **data)


def make_native_tables(out, nev):
    data = {}
    for name in SYSTEMS:
        ref, _ = ref_for([name], ["ecc_from_order=2", "ecc_to_order=5"])
        ref.srand(7)
        tab = ref.generate_ecc_table(nev)
        data[name] = tab
    np.savez_compressed(os.path.join(out, "ecc_native.npz"), **data)


# further systems at the reference's own geometry (tests/systems.py NATIVE_SYSTEMS)
NATIVE_SYSTEM_ARGS = {
    "ppb5020": ["Aproj=1", "Atarg=208", "ecm=5020"],
    "dau200": ["Aproj=2", "Atarg=197", "ecm=200"],
    "cucu200": ["Aproj=63", "Atarg=63", "ecm=200"],
    "uu200": ["Aproj=238", "Atarg=238", "ecm=200", "proj_deformed=1", "targ_deformed=1"],
}


def make_native_systems(out, nev):
    """The reference's op-9 table (its own drand48 sampler) for p+Pb, d+Au,
    Cu+Cu and deformed U+U: the 49 columns of each sn_ecc_eccp_10.dat line
    (a deformed run appends four more, dropped here)."""
    data = {}
    for name, extra in NATIVE_SYSTEM_ARGS.items():
        ref, _ = ref_for(["auau200"], extra + ["ecc_from_order=2", "ecc_to_order=5"])
        ref.srand(7)
        data[name] = ref.generate_ecc_table(nev)[:, :49]
    np.savez_compressed(os.path.join(out, "ecc_native_systems.npz"), **data)


def make_light(out, nev):
    """Light nuclei from configuration tables.
    light_nuclei_drand48.npz: Nucleus::populate of 3He, 4He and 12C from the
    reference's own tables (srand48 / srand seeds 3, 11, 19): the nucleons,
    and the one configuration each draw used (index rand() % nconf, its
    [A][3] positions) -- what the oracle needs to redo the draw.
    ecc_light_systems.npz: the reference's op-9 table (its own sampler) for
    the systems of tests/systems.py LIGHT_SYSTEMS with the seeded synthetic
    tables of synthetic_configurations written in the reference's layout."""
    import ctypes
    import tempfile
    sys.path.insert(0, os.path.dirname(HERE))
    from systems import LIGHT_FILES, LIGHT_SYSTEMS, synthetic_configurations, write_configurations
    from oracle.oracle import read_configurations
    libc = ctypes.CDLL(None)
    libc.srand.argtypes = [ctypes.c_uint]
    pin = {}
    for A in (3, 4, 12):
        tab = read_configurations(os.path.join(TABLES_DIR, LIGHT_FILES[A]), A)
        ref, _ = ref_for(["auau200"], [f"Aproj={A}"])
        pin[f"A{A}_nconf"] = np.array(len(tab))
        for seed in (3, 11, 19):
            ref.srand(seed)
            pin[f"A{A}_s{seed}_pos"] = ref.populate(0, 2.5)
            libc.srand(seed)
            k = libc.rand() % len(tab)
            pin[f"A{A}_s{seed}_idx"] = np.array(k)
            pin[f"A{A}_s{seed}_conf"] = tab[k]
    np.savez_compressed(os.path.join(out, "light_nuclei_drand48.npz"), **pin)
    data = {}
    for name, sysd in LIGHT_SYSTEMS.items():
        tdir = tempfile.mkdtemp(prefix="smc_light_")
        for A in {sysd["Aproj"], sysd["Atarg"]}:
            if A in LIGHT_FILES:
                write_configurations(os.path.join(tdir, LIGHT_FILES[A]), A, synthetic_configurations(A))
        extra = [f"Aproj={sysd['Aproj']}", f"Atarg={sysd['Atarg']}", f"ecm={sysd['ecm']}", "ecc_from_order=2",
                 "ecc_to_order=5"]
        vals = read_parameters(None, list(SYSTEMS["auau200"]) + extra, strict=False)
        ref = Reference(parameters_text(vals), eos_dir=EOS_DIR, tables_dir=tdir)
        ref.srand(7)
        data[name] = ref.generate_ecc_table(nev)[:, :49]
    np.savez_compressed(os.path.join(out, "ecc_light_systems.npz"), **data)


def make_kln(out):
    ref, vals = ref_for(["pbpb2760"], ["which_mc_model=1", "sub_model=7", "lambda=0.288"])
    ref.lib.refh_kln_setup(2760.0, 0.288)
    rng = np.random.default_rng(5)
    pts, vals_out, nodes, bases = [], [], [], []
    for ta, tb in [(0.3, 0.9), (1.7, 2.2), (4.4, 0.5), (9.0, 7.5)]:
        ref.lib.refh_kln_prepare(0.0, ta, tb)
        for _ in range(40):
            x = rng.random(3)
            pts.append([ta, tb, *x])
            vals_out.append(ref.lib.refh_kln_integrand(0.0, ta, tb, *x))
        nodes.append([ta, tb])
        bases.append(ref.lib.refh_kln_dndy(0.0, ta, tb))
    # per-cell lookup: an analytic table installed into the reference's MCnucl
    sig = ref.constants()["sigin"]
    tmax, dT = 211, 10.0 / sig / 3
    I, J = np.meshgrid(np.arange(tmax), np.arange(tmax), indexing="ij")
    table = np.where((I > 0) & (J > 0), np.sqrt(I * dT * J * dT) * 3.0 + 0.1 * (I * dT) ** 2, 0.0)
    ref.set_kln_table(table, dT)
    grng = np.random.default_rng(9)
    ref.srand(21)
    xa, xb = sample_positions(ref, 6.0)
    ref.inject(xa, xb)
    dig = grid_digest(ref.grid(2), grng)
    np.savez_compressed(os.path.join(out, "kln.npz"), points=np.array(pts), integrand=np.array(vals_out),
                        nodes=np.array(nodes), bases=np.array(bases), table_dT=np.array(dT),
                        lookup_pos_a=xa, lookup_pos_b=xb, sigin=np.array(sig),
                        **{"lookup_rho_" + k: v for k, v in dig.items()})


def make_kln_pt(out):
    """KLNModel::getdNdy at fixed p_T (adaptive Simpson, the rows of
    MCnucl::makeTable(ptmin, dpt, iPtmax)) at a few (T_A, T_B, p_T)."""
    ref, vals = ref_for(["pbpb2760"], ["which_mc_model=1", "sub_model=7", "lambda=0.288"])
    ref.lib.refh_kln_setup(2760.0, 0.288)
    pts, vals_out = [], []
    for ta, tb in [(0.3, 0.9), (1.7, 2.2), (4.4, 0.5), (9.0, 7.5)]:
        for pt in (0.1, 0.5, 1.0, 1.5, 2.0):
            pts.append([ta, tb, pt])
            vals_out.append(ref.lib.refh_kln_dndy_pt(0.0, ta, tb, pt))
    np.savez_compressed(os.path.join(out, "kln_pt.npz"), points=np.array(pts), values=np.array(vals_out))


def make_constants(out):
    ref, _ = ref_for(["auau200"])
    c = {"sigma_in": {str(e): ref.lib.refh_sigma_in(e) for e in (62.4, 200.0, 2760.0, 3670.0, 5020.0, 5520.0)},
         "six_point": [[0.3, 0.7, 1, 2, 3, 4, 5, 6, ref.lib.refh_six_point(0.3, 0.7, 1, 2, 3, 4, 5, 6)],
                       [0.9, 0.1, -1, 0.5, 2, 7, 1, 3, ref.lib.refh_six_point(0.9, 0.1, -1, 0.5, 2, 7, 1, 3)]],
         "hulthen_cdf": {str(r): ref.lib.refh_hulthen_cdf(r) for r in (0.5, 1.0, 2.0, 4.0, 7.0, 15.0)},
         "hulthen_inv": {str(u): ref.lib.refh_hulthen_inv(u) for u in (0.05, 0.3, 0.5, 0.77, 0.95)}}
    with open(os.path.join(out, "constants.json"), "w") as f:
        json.dump(c, f, indent=1)


def make_text(out):
    """Raw text files of the stock reference binary: the eccentricity files of
    operation 9 (4 Au+Au events, orders 2..5; 3 deformed U+U events, orders
    2..3, keys "deformed/<name>") and the block / 4-column density files of
    operation 1 (2 events on a 13x13 grid)."""
    import subprocess
    import tempfile
    ref, vals = ref_for(["auau200"])
    exe = os.path.join(REPO, "oracle", "_ref", "superMC.e")
    texts = {}
    runs = ((9, "", ["nev=4", "ecc_from_order=2", "ecc_to_order=5"]),
            (1, "", ["nev=2", "maxx=3", "maxy=3", "dx=0.5", "dy=0.5", "use_block=1", "use_4col=1"]),
            (9, "deformed/", ["nev=3", "ecc_from_order=2", "ecc_to_order=3", "Aproj=238", "Atarg=238",
                              "proj_deformed=1", "targ_deformed=1"]),
            (2, "jet/", ["nev=2", "maxx=3", "maxy=3", "dx=0.5", "dy=0.5", "use_block=1", "use_4col=1", "use_ed=0",
                         "ecc_from_order=2", "ecc_to_order=3", "output_rho_binary=1", "output_TA=1",
                         "output_rhob=1", "output_spectator_density=1"]))
    for op, key, args in runs:
        wd = tempfile.mkdtemp(prefix="smc_text_", dir=ref.workdir)
        os.makedirs(os.path.join(wd, "data"))
        os.symlink(os.path.join(ref.workdir, "tables"), os.path.join(wd, "tables"))
        os.symlink(EOS_DIR, os.path.join(wd, "EOS"))
        with open(os.path.join(wd, "parameters.dat"), "w") as f:
            f.write(parameters_text(vals))
        subprocess.run([exe, f"operation={op}", "randomSeed=7"] + args, cwd=wd, check=True, capture_output=True)
        if op == 2:
            # Jet mode: the file set, and the per-event tables (formats)
            names = ["ParticipantTable_event_1.dat", "Spectators_event_1.dat", "BinaryCollisionTable_event_1.dat",
                     "sn_ecc_eccp_2_event_1.dat", "sn_ecc_eccp_10_event_1.dat"]
            texts[key + "files"] = sorted(os.listdir(os.path.join(wd, "data")))
            for name in names:
                with open(os.path.join(wd, "data", name)) as f:
                    texts[key + name] = f.read()
            continue
        orders = (2, 3, 10) if key else (2, 3, 4, 5, 10)
        names = ([f"sn_ecc_eccp_{k}.dat" for k in orders] if op == 9 else
                 [f"sd_event_{e}_{kind}.dat" for e in (1, 2) for kind in ("block", "4col")])
        for name in names:
            with open(os.path.join(wd, "data", name)) as f:
                texts[key + name] = f.read()
    texts["grid"] = {"xmin": -3.0, "ymin": -3.0, "dx": 0.5, "dy": 0.5, "nx": 13, "ny": 13}
    with open(os.path.join(out, "text_outputs.json"), "w") as f:
        json.dump(texts, f, indent=0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=REF_ROOT)
    ap.add_argument("--nev", type=int, default=1500)
    ap.add_argument("--only", choices=["constants", "sampler", "inject", "average", "kln", "kln_pt", "native",
                                       "native_systems", "light", "text"],
                    help="regenerate one fixture only")
    a = ap.parse_args()
    if build_reference(a.ref) is None:
        sys.exit(f"reference tree not found at {a.ref}")
    global EOS_DIR, TABLES_DIR
    EOS_DIR = os.path.join(a.ref, "EOS")
    TABLES_DIR = os.path.join(a.ref, "tables")
    steps = {"constants": lambda: make_constants(HERE), "sampler": lambda: make_sampler(HERE),
             "inject": lambda: make_inject(HERE), "average": lambda: make_average(HERE),
             "kln": lambda: make_kln(HERE), "kln_pt": lambda: make_kln_pt(HERE), "native": lambda: make_native_tables(HERE, a.nev),
             "native_systems": lambda: make_native_systems(HERE, a.nev),
             "light": lambda: make_light(HERE, a.nev),
             "text": lambda: make_text(HERE)}
    for k, f in steps.items():
        if a.only in (None, k):
            f()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
