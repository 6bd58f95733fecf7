"""ctypes wrappers for the checker libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU legs of bench.py.  Two libraries are wrapped:

* ``Oracle`` -- the FP64 C restatement (oracle/smc_oracle.c), built by
  :func:`build_oracle` into ``oracle/_build/libsmc_oracle.so`` on any machine;
* ``Reference`` -- the reference superMC sources compiled from source with
  the injection harness (oracle/Makefile.ref -> ``oracle/_ref/libsmc_ref.so``),
  available only where the reference tree is present.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libsmc_oracle.so")
# where the reference's source tree lies on the machine that builds the
# reference checker (the only setting that names it; absent elsewhere)
REF_ROOT = os.environ.get("SUPERMC_REFERENCE_ROOT", "/root/reference")
REF_SO = os.path.join(HERE, "_ref", "libsmc_ref.so")

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def build_oracle(force: bool = False) -> str:
    """Compile oracle/smc_oracle.c (FP contraction off so rounding matches
    the reference's x86-64 build on any host)."""
    src = os.path.join(HERE, "smc_oracle.c")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        tmp = ORACLE_SO + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, src, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_reference(ref_root: str | None = None) -> str | None:
    """Build the reference checker when its source tree is present."""
    ref_root = ref_root or REF_ROOT
    if not os.path.isdir(os.path.join(ref_root, "src")):
        return None
    repo = os.path.dirname(HERE)
    subprocess.check_call(["make", "-s", "-f", "oracle/Makefile.ref", f"REF={ref_root}", "-j8"], cwd=repo)
    return REF_SO


def _ptr(a: np.ndarray, kind=_D):
    return a.ctypes.data_as(kind)


class Params(ctypes.Structure):
    """Mirror of smco_params (oracle/smc_oracle.h)."""

    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("xmax", ctypes.c_double), ("ymax", ctypes.c_double),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double),
        ("width", ctypes.c_double), ("quark_width", ctypes.c_double),
        ("dsq", ctypes.c_double), ("sigin", ctypes.c_double), ("sigma_gg", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("which_mc_model", ctypes.c_int), ("sub_model", ctypes.c_int),
        ("shape_of_nucleons", ctypes.c_int), ("shape_of_entropy", ctypes.c_int),
        ("collision_criterion", ctypes.c_int),
        ("final_factor", ctypes.c_double),
        ("npmin", ctypes.c_int), ("npmax", ctypes.c_int),
        ("kln_table", _D), ("kln_tmax", ctypes.c_int), ("kln_dT", ctypes.c_double),
        ("cc_fluctuation_model", ctypes.c_int), ("cc_fluctuation_gamma_theta", ctypes.c_double),
        ("cc_fluctuation_k", ctypes.c_double),
    ]


class Nucleus(ctypes.Structure):
    _fields_ = [
        ("A", ctypes.c_int), ("deformed", ctypes.c_int),
        ("R", ctypes.c_double), ("a", ctypes.c_double),
        ("beta2", ctypes.c_double), ("beta4", ctypes.c_double),
        ("d_min", ctypes.c_double), ("rmax_cut", ctypes.c_double), ("rw_max", ctypes.c_double),
        ("icdf", ctypes.c_int),
        ("conf", _D), ("nconf", ctypes.c_int),
    ]


class KLN(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("ecm", "lambda_", "y", "ptmin", "ptmax", "lambda_qcd",
                                                "alpha_max", "g2hfac")]


class Oracle:
    def __init__(self):
        lib = ctypes.CDLL(build_oracle())
        self.lib = lib
        lib.smco_sigma_in.restype = ctypes.c_double
        lib.smco_sigma_in.argtypes = [ctypes.c_double]
        lib.smco_sigeff.restype = ctypes.c_double
        lib.smco_sigeff.argtypes = [ctypes.c_double, ctypes.c_double]
        lib.smco_hulthen_cdf.restype = ctypes.c_double
        lib.smco_hulthen_cdf.argtypes = [ctypes.c_double]
        lib.smco_hulthen_inv.restype = ctypes.c_double
        lib.smco_hulthen_inv.argtypes = [ctypes.c_double]
        lib.smco_six_point.restype = ctypes.c_double
        lib.smco_six_point.argtypes = [ctypes.c_double] * 8
        lib.smco_uniform2.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, _D]
        lib.smco_philox4x32.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
        lib.smco_nucleus_init.argtypes = [ctypes.POINTER(Nucleus), ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.smco_event_new.restype = ctypes.c_void_p
        lib.smco_event_new.argtypes = [ctypes.POINTER(Params)]
        lib.smco_event_free.argtypes = [ctypes.c_void_p]
        lib.smco_event_inject.argtypes = [ctypes.c_void_p, _D, ctypes.c_int, _D, ctypes.c_int]
        lib.smco_event_populate_drand48.argtypes = [ctypes.c_void_p, ctypes.POINTER(Nucleus),
                                                    ctypes.POINTER(Nucleus), ctypes.c_double]
        lib.smco_event_populate_philox.argtypes = [ctypes.c_void_p, ctypes.POINTER(Nucleus),
                                                   ctypes.POINTER(Nucleus), ctypes.c_double,
                                                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        lib.smco_impact_philox.restype = ctypes.c_double
        lib.smco_impact_philox.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_double]
        for f in ("smco_event_pair", "smco_event_ncoll", "smco_event_thickness", "smco_event_density"):
            getattr(lib, f).argtypes = [ctypes.c_void_p]
        lib.smco_event_npart.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.smco_event_nucleons.argtypes = [ctypes.c_void_p, ctypes.c_int, _D, ctypes.c_int]
        lib.smco_event_participants.argtypes = [ctypes.c_void_p, ctypes.c_int, _D, ctypes.c_int]
        lib.smco_event_participant_index.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, ctypes.c_int]
        lib.smco_event_collisions.argtypes = [ctypes.c_void_p, _D, ctypes.c_int]
        lib.smco_event_grid.argtypes = [ctypes.c_void_p, ctypes.c_int, _D]
        lib.smco_event_rho_binary.argtypes = [ctypes.c_void_p]
        lib.smco_event_eccentricities.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                  ctypes.c_double, _D]
        lib.smco_event_spectator_density.argtypes = [ctypes.c_void_p, _D, _D]
        lib.smco_event_hotspot_mask.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.smco_event_density_frozen.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _D]
        lib.smco_event_density_moved.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                                 ctypes.c_void_p, ctypes.c_void_p, _D]
        lib.smco_ws_icdf.restype = ctypes.c_double
        lib.smco_ws_icdf.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        lib.smco_event_icdf_displacement.argtypes = [ctypes.c_void_p, ctypes.POINTER(Nucleus),
                                                     ctypes.POINTER(Nucleus), ctypes.c_double, ctypes.c_double,
                                                     _D, _D]
        lib.smco_event_icdf_tangents.argtypes = [ctypes.c_void_p, ctypes.POINTER(Nucleus),
                                                 ctypes.POINTER(Nucleus), _D, _D]
        lib.smco_event_nucleon_ids.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, ctypes.c_int]
        lib.smco_event_cm_angle.argtypes = [ctypes.c_void_p, ctypes.c_int, _D, _D, _D]
        lib.smco_event_rotate_resplat.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.smco_event_recenter_resplat.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.smco_kln_init.argtypes = [ctypes.POINTER(KLN), ctypes.c_double, ctypes.c_double]
        lib.smco_kln_integrand.restype = ctypes.c_double
        lib.smco_kln_integrand.argtypes = [ctypes.POINTER(KLN), ctypes.c_double, ctypes.c_double, _D]
        lib.smco_kln_dndy_pt.restype = ctypes.c_double
        lib.smco_kln_dndy_pt.argtypes = [ctypes.POINTER(KLN), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int]
        lib.smco_kln_dndy.restype = ctypes.c_double
        lib.smco_kln_dndy.argtypes = [ctypes.POINTER(KLN), ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.smco_gauss_legendre01.argtypes = [ctypes.c_int, _D, _D]
        lib.smco_nbd_draw.restype = ctypes.c_double
        lib.smco_nbd_draw.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_double,
                                      ctypes.c_double]
        lib.smco_gamma_philox.restype = ctypes.c_double
        lib.smco_gamma_philox.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint32,
                                          ctypes.c_double, ctypes.c_double]
        lib.smco_set_pair_stream.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
        lib.smco_run_ecc_table.restype = ctypes.c_long
        lib.smco_run_ecc_table.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(Nucleus),
                                           ctypes.POINTER(Nucleus), ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_long,
                                           ctypes.c_int, ctypes.c_uint64, _D]

    # ---- helpers ---------------------------------------------------------
    def nucleus(self, A, deformed=0, R=0.0, a=0.0, dmin=0.0, icdf=0, conf=None) -> Nucleus:
        """conf: light-nucleus configurations [nconf][A][3] (kept alive by
        the returned structure)."""
        n = Nucleus()
        self.lib.smco_nucleus_init(ctypes.byref(n), A, deformed, R, a, dmin)
        n.icdf = icdf
        if conf is not None:
            t = np.ascontiguousarray(np.asarray(conf, dtype=np.float64))
            assert t.ndim == 3 and t.shape[1:] == (A, 3), t.shape
            n._conf_keep = t
            n.conf = _ptr(t)
            n.nconf = t.shape[0]
        return n

    def ws_icdf(self, R, a, u):
        """(r, dr/dR, dr/da) of the inverse-CDF Woods-Saxon radius."""
        dR, da = ctypes.c_double(), ctypes.c_double()
        r = self.lib.smco_ws_icdf(R, a, u, ctypes.byref(dR), ctypes.byref(da))
        return r, dR.value, da.value

    def uniform2(self, seed, event, stream, slot):
        u = np.zeros(2)
        self.lib.smco_uniform2(seed, event, stream, slot, _ptr(u))
        return u

    def philox(self, ctr, key):
        c = (ctypes.c_uint32 * 4)(*ctr)
        k = (ctypes.c_uint32 * 2)(*key)
        o = (ctypes.c_uint32 * 4)()
        self.lib.smco_philox4x32(c, k, o)
        return list(o)

    def event(self, params: Params) -> "OracleEvent":
        return OracleEvent(self, params)


class OracleEvent:
    def __init__(self, orc: Oracle, params: Params):
        self.o = orc
        self.lib = orc.lib
        self.params = params
        self.h = self.lib.smco_event_new(ctypes.byref(params))
        self.nx, self.ny = params.nx, params.ny

    def __del__(self):
        try:
            self.lib.smco_event_free(self.h)
        except Exception:
            pass

    def inject(self, xyA, xyB):
        a = np.ascontiguousarray(xyA, dtype=np.float64).reshape(-1, 2)
        b = np.ascontiguousarray(xyB, dtype=np.float64).reshape(-1, 2)
        self.lib.smco_event_inject(self.h, _ptr(a), len(a), _ptr(b), len(b))

    def pair(self):
        return self.lib.smco_event_pair(self.h)

    def npart(self):
        return self.lib.smco_event_npart(self.h, 0), self.lib.smco_event_npart(self.h, 1)

    def nucleons(self, which):
        out = np.zeros((400, 3))
        n = self.lib.smco_event_nucleons(self.h, which, _ptr(out), 400)
        return out[:n].copy()

    def participants(self, which):
        out = np.zeros((400, 2))
        n = self.lib.smco_event_participants(self.h, which, _ptr(out), 400)
        return out[:n].copy()

    def participant_index(self, which):
        out = np.zeros(400, dtype=np.int32)
        n = self.lib.smco_event_participant_index(self.h, which, _ptr(out, _I), 400)
        return out[:n].copy()

    def collisions(self):
        n = self.lib.smco_event_ncoll(self.h)
        out = np.zeros((max(n, 1), 2))
        self.lib.smco_event_collisions(self.h, _ptr(out), n)
        return out[:n].copy()

    def thickness(self):
        return self.lib.smco_event_thickness(self.h)

    def density(self):
        return self.lib.smco_event_density(self.h)

    def grid(self, which):
        g = np.zeros((self.nx, self.ny))
        self.lib.smco_event_grid(self.h, which, _ptr(g))
        return g

    def rho_binary(self):
        self.lib.smco_event_rho_binary(self.h)
        return self.grid(3)

    def eccentricities(self, from_order, to_order, b):
        out = np.zeros(49)
        self.lib.smco_event_eccentricities(self.h, from_order, to_order, b, _ptr(out))
        return out

    def spectator_density(self):
        a, b = np.zeros((self.nx, self.ny)), np.zeros((self.nx, self.ny))
        self.lib.smco_event_spectator_density(self.h, _ptr(a), _ptr(b))
        return a, b

    def hotspot_mask(self):
        m = np.zeros((self.nx, self.ny), dtype=np.uint8)
        self.lib.smco_event_hotspot_mask(self.h, m.ctypes.data)
        return m.astype(bool)

    def density_moved(self, w, alpha, dA=None, dB=None):
        g = np.zeros((self.nx, self.ny))
        a = None if dA is None else np.ascontiguousarray(dA, dtype=np.float64)
        b = None if dB is None else np.ascontiguousarray(dB, dtype=np.float64)
        rc = self.lib.smco_event_density_moved(self.h, w, alpha, None if a is None else a.ctypes.data,
                                               None if b is None else b.ctypes.data, _ptr(g))
        if rc:
            raise RuntimeError(f"smco_event_density_moved: {rc}")
        return g

    def icdf_displacement(self, nA, nB, dR, da):
        """Nucleon displacements by id ([A,2], [B,2]) for (R, a) += (dR, da)."""
        A, B = len(self.nucleons(0)), len(self.nucleons(1))
        dA, dB = np.zeros((A, 2)), np.zeros((B, 2))
        self.lib.smco_event_icdf_displacement(self.h, ctypes.byref(nA), ctypes.byref(nB), dR, da, _ptr(dA),
                                              _ptr(dB))
        return dA, dB

    def icdf_tangents(self, nA, nB):
        """(dx/dR, dy/dR, dx/da, dy/da) per nucleon by id ([A,4], [B,4])."""
        A, B = len(self.nucleons(0)), len(self.nucleons(1))
        tA, tB = np.zeros((A, 4)), np.zeros((B, 4))
        self.lib.smco_event_icdf_tangents(self.h, ctypes.byref(nA), ctypes.byref(nB), _ptr(tA), _ptr(tB))
        return tA, tB

    def nucleon_ids(self, which):
        out = np.zeros(400, dtype=np.int32)
        n = self.lib.smco_event_nucleon_ids(self.h, which, _ptr(out, _I), 400)
        return out[:n].copy()

    def density_frozen(self, w, alpha):
        g = np.zeros((self.nx, self.ny))
        rc = self.lib.smco_event_density_frozen(self.h, w, alpha, _ptr(g))
        if rc:
            raise RuntimeError(f"smco_event_density_frozen: {rc}")
        return g

    def cm_angle(self, n):
        x, y, a = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self.lib.smco_event_cm_angle(self.h, n, ctypes.byref(x), ctypes.byref(y), ctypes.byref(a))
        return x.value, y.value, a.value

    def rotate_resplat(self, order):
        return self.lib.smco_event_rotate_resplat(self.h, order)

    def recenter_resplat(self, order):
        return self.lib.smco_event_recenter_resplat(self.h, order)

    def populate_drand48(self, nA, nB, b):
        self.lib.smco_event_populate_drand48(self.h, ctypes.byref(nA), ctypes.byref(nB), b)

    def populate_philox(self, nA, nB, b, seed, event, attempt):
        self.lib.smco_event_populate_philox(self.h, ctypes.byref(nA), ctypes.byref(nB), b, seed, event, attempt)


def _kln_rows_worker(args):
    """Rows of the MC-KLN table by the oracle's FP64 quadrature (pool worker)."""
    ecm, lam, dT, rows, tmax, rule = args
    orc = Oracle()
    k = KLN()
    orc.lib.smco_kln_init(ctypes.byref(k), ecm, lam)
    out = []
    for i in rows:
        row = [0.0] * tmax
        if i > 0:
            for j in range(1, tmax):
                row[j] = orc.lib.smco_kln_dndy(ctypes.byref(k), dT * i, dT * j, *rule)
        out.append((i, row))
    return out


def read_configurations(path: str, A: int) -> np.ndarray:
    """A light-nucleus configuration file in the reference's layout for A
    (src/Nucleus.cpp:383-478: he3 records hold 9 coordinates and 4 further
    fields, carbon records 2 fields and 36 coordinates, the others 3 A
    coordinates), as [nconf][A][3]."""
    lead, trail = (2 if A == 12 else 0), (4 if A == 3 else 0)
    rec = lead + 3 * A + trail
    with open(path) as f:
        vals = np.array(f.read().split(), dtype=np.float64)
    if len(vals) == 0 or len(vals) % rec:
        raise ValueError(f"{path}: {len(vals)} fields, not whole records of {rec}")
    return vals.reshape(-1, rec)[:, lead:lead + 3 * A].reshape(-1, A, 3).copy()


def kln_table(ecm: float, lam: float, dT: float, tmax: int, rule=(48, 64, 32), procs: int | None = None):
    """The whole MC-KLN dN/dy table [tmax][tmax] (MCnucl::makeTable,
    src/MCnucl.cpp:911-960) by the oracle's FP64 Gauss-Legendre quadrature of
    KLNModel::func, rows spread over a process pool (spawned, so that it is
    safe after a CUDA context exists).  Row and column 0 are zero."""
    import multiprocessing as mp
    procs = procs or max(1, os.cpu_count() or 1)
    rows = list(range(tmax))
    chunks = [rows[k::procs] for k in range(procs)]
    with mp.get_context("spawn").Pool(procs) as pool:
        parts = pool.map(_kln_rows_worker, [(ecm, lam, dT, c, tmax, tuple(rule)) for c in chunks])
    tab = np.zeros((tmax, tmax))
    for part in parts:
        for i, row in part:
            tab[i] = row
    return tab


class Reference:
    """The reference's own code (compiled from source) with injected inputs."""

    LIGHT_TABLES = ("he3_plaintext.dat", "he4_plaintext.dat", "carbon_plaintext.dat", "oxygen_plaintext.dat")

    def __init__(self, params_text: str, eos_dir: str | None = None, workdir: str | None = None,
                 tables_dir: str | None = None):
        """tables_dir: where the reference's light-nucleus configuration files
        are (default: the reference tree's tables/); the Nucleus constructor
        reads them from tables/ of the work directory."""
        eos_dir = eos_dir or os.path.join(REF_ROOT, "EOS")
        tables_dir = tables_dir or os.path.join(REF_ROOT, "tables")
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        lib = ctypes.CDLL(REF_SO)
        self.lib = lib
        lib.refh_init.argtypes = [ctypes.c_char_p] * 3
        lib.refh_inject_event.argtypes = [_D, ctypes.c_int, _D, ctypes.c_int, _I, _I, _I, ctypes.c_int]
        lib.refh_grid_dims.argtypes = [_I, _I]
        lib.refh_get_grid.argtypes = [ctypes.c_int, _D]
        lib.refh_participants.argtypes = [ctypes.c_int, _D, ctypes.c_int]
        lib.refh_nucleons.argtypes = [ctypes.c_int, _D, ctypes.c_int]
        lib.refh_collisions.argtypes = [_D, ctypes.c_int]
        lib.refh_eccentricities.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, _D]
        lib.refh_rotate_and_resplat.argtypes = [ctypes.c_int]
        lib.refh_recenter_and_resplat.argtypes = [ctypes.c_int]
        lib.refh_density.argtypes = []
        lib.refh_generate_ecc_table.argtypes = [ctypes.c_int]
        lib.refh_sample_event.argtypes = [ctypes.c_double, _I, _I, _I]
        lib.refh_populate.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, _D, ctypes.c_int]
        lib.refh_srand.argtypes = [ctypes.c_long]
        lib.refh_set_kln_table.argtypes = [_D, ctypes.c_int, ctypes.c_double]
        for f in ("refh_sigma_in", "refh_hulthen_cdf", "refh_hulthen_inv"):
            getattr(lib, f).restype = ctypes.c_double
            getattr(lib, f).argtypes = [ctypes.c_double]
        lib.refh_constants.argtypes = [_D]
        lib.refh_six_point.restype = ctypes.c_double
        lib.refh_six_point.argtypes = [ctypes.c_double] * 8
        lib.refh_kln_setup.argtypes = [ctypes.c_double, ctypes.c_double]
        lib.refh_kln_prepare.argtypes = [ctypes.c_double] * 3
        lib.refh_kln_integrand.restype = ctypes.c_double
        lib.refh_kln_integrand.argtypes = [ctypes.c_double] * 6
        lib.refh_kln_dndy_pt.restype = ctypes.c_double
        lib.refh_kln_dndy_pt.argtypes = [ctypes.c_double] * 4
        lib.refh_kln_dndy.restype = ctypes.c_double
        lib.refh_kln_dndy.argtypes = [ctypes.c_double] * 3
        self.workdir = workdir or tempfile.mkdtemp(prefix="smc_ref_")
        os.makedirs(os.path.join(self.workdir, "tables"), exist_ok=True)
        for f in self.LIGHT_TABLES:
            src, dst = os.path.join(tables_dir, f), os.path.join(self.workdir, "tables", f)
            if os.path.exists(src) and not os.path.lexists(dst):
                os.symlink(os.path.abspath(src), dst)
        cwd = os.getcwd()
        rc = lib.refh_init(self.workdir.encode(), eos_dir.encode(), params_text.encode())
        os.chdir(cwd)  # the harness chdir()s into its work dir; callers keep theirs
        if rc != 0:
            raise RuntimeError(f"refh_init failed: {rc}")
        nx, ny = ctypes.c_int(), ctypes.c_int()
        lib.refh_grid_dims(ctypes.byref(nx), ctypes.byref(ny))
        self.nx, self.ny = nx.value, ny.value

    def _in_workdir(self, fn, *args):
        cwd = os.getcwd()
        os.chdir(self.workdir)
        try:
            return fn(*args)
        finally:
            os.chdir(cwd)

    def inject(self, xyA, xyB, density=True):
        a = np.ascontiguousarray(xyA, dtype=np.float64).reshape(-1, 2)
        b = np.ascontiguousarray(xyB, dtype=np.float64).reshape(-1, 2)
        n1, n2, nc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.lib.refh_inject_event(_ptr(a), len(a), _ptr(b), len(b), ctypes.byref(n1), ctypes.byref(n2),
                                   ctypes.byref(nc), 1 if density else 0)
        return n1.value, n2.value, nc.value

    def grid(self, which):
        g = np.zeros((self.nx, self.ny))
        self.lib.refh_get_grid(which, _ptr(g))
        return g

    def participants(self, which):
        out = np.zeros((400, 2))
        n = self.lib.refh_participants(which, _ptr(out), 400)
        return out[:n].copy()

    def nucleons(self, which):
        out = np.zeros((400, 3))
        n = self.lib.refh_nucleons(which, _ptr(out), 400)
        return out[:n].copy()

    def collisions(self):
        out = np.zeros((50000, 2))
        n = self.lib.refh_collisions(_ptr(out), 50000)
        return out[:n].copy()

    def eccentricities(self, from_order, to_order, npart, ncoll, b):
        out = np.zeros(49)
        k = self._in_workdir(self.lib.refh_eccentricities, from_order, to_order, float(npart), float(ncoll),
                             float(b), _ptr(out))
        assert k == 49, k
        return out

    def rotate_resplat(self, order):
        self.lib.refh_rotate_and_resplat(order)

    def recenter_resplat(self, order):
        self.lib.refh_recenter_and_resplat(order)

    def srand(self, seed):
        self.lib.refh_srand(seed)

    def populate(self, which, xc, yc=0.0):
        out = np.zeros((400, 3))
        n = self.lib.refh_populate(which, xc, yc, _ptr(out), 400)
        return out[:n].copy()

    def density(self):
        self.lib.refh_density()

    def sample_event(self, b):
        n1, n2, nc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.lib.refh_sample_event(b, ctypes.byref(n1), ctypes.byref(n2), ctypes.byref(nc))
        return n1.value, n2.value, nc.value

    def generate_ecc_table(self, nev):
        self._in_workdir(self.lib.refh_generate_ecc_table, nev)
        path = os.path.join(self.workdir, "data", "sn_ecc_eccp_10.dat")
        return np.loadtxt(path, ndmin=2)

    def constants(self):
        c = np.zeros(4)
        self.lib.refh_constants(_ptr(c))
        return dict(dsq=c[0], width=c[1], sigma_gg=c[2], sigin=c[3])

    def set_kln_table(self, table, dT):
        t = np.ascontiguousarray(table, dtype=np.float64)
        self.lib.refh_set_kln_table(_ptr(t), t.shape[0], dT)
