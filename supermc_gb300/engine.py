"""Python host interface over the C ABI (include/supermc.h).

``Engine`` owns one library context.  It is built from the superMC
``parameters.dat`` key set (see :mod:`supermc_gb300.params`) and exposes the
batched event generator, the injected-positions path and the plain
per-event path.  Results come back as numpy arrays (host buffers) or are
written into caller-provided device tensors.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .params import DEFAULTS, EXTENSION_KEYS, read_parameters


def smc_params_from(vals: dict[str, float], seed: int = 1) -> _lib.SmcParams:
    v = dict(DEFAULTS)
    v.update(EXTENSION_KEYS)
    v.update({k.lower(): x for k, x in vals.items()})
    p = _lib.SmcParams()
    p.which_mc_model = int(v["which_mc_model"])
    p.sub_model = int(v["sub_model"])
    p.shape_of_nucleons = int(v["shape_of_nucleons"])
    p.shape_of_entropy = int(v["shape_of_entropy"])
    p.collision_criterion = int(v["collision_criterion"])
    p.Aproj, p.Atarg = int(v["aproj"]), int(v["atarg"])
    p.proj_deformed, p.targ_deformed = int(v["proj_deformed"]), int(v["targ_deformed"])
    p.ecm, p.alpha = v["ecm"], v["alpha"]
    p.gauss_nucl_width, p.quark_width, p.lambda_ = v["gauss_nucl_width"], v["quark_width"], v["lambda"]
    p.bmin, p.bmax = v["bmin"], v["bmax"]
    p.npmin, p.npmax = int(v["npmin"]), int(v["npmax"])
    p.maxx, p.maxy, p.dx, p.dy = v["maxx"], v["maxy"], v["dx"], v["dy"]
    p.final_factor = v["finalfactor"]
    p.tmax, p.tmax_subdivision = int(v["tmax"]), int(v["tmax_subdivision"])
    p.ecc_from_order, p.ecc_to_order = int(v["ecc_from_order"]), int(v["ecc_to_order"])
    p.proj_R, p.proj_a, p.targ_R, p.targ_a = v["proj_r"], v["proj_a"], v["targ_r"], v["targ_a"]
    p.proj_d_min, p.targ_d_min = v["proj_d_min"], v["targ_d_min"]
    p.sigin_override = v["sigininn_override"]
    p.kln_npt, p.kln_nkt, p.kln_nphi = int(v["kln_npt"]), int(v["kln_nkt"]), int(v["kln_nphi"])
    p.seed = int(seed) & ((1 << 64) - 1)
    p.max_attempts = int(v["max_attempts"])
    p.max_collisions = int(v["max_collisions"])
    p.ws_inverse_cdf = int(v["ws_inverse_cdf"])
    p.cc_fluctuation_model = int(v["cc_fluctuation_model"])
    p.cc_fluctuation_gamma_theta = v["cc_fluctuation_gamma_theta"]
    p.cc_fluctuation_k = v["cc_fluctuation_k"]
    p.kln_exact_band = v["kln_exact_band"]
    return p


OUTPUT_NAMES = ("ecc", "rho", "ta", "tb", "npart", "ncoll", "b", "attempts", "positions", "wounded", "tangents",
                "collisions", "orientation", "rho_pt", "rho_binary", "spectator_a", "spectator_b")
# keys that describe one collision system of a mixed batch
SYSTEM_KEYS = ("aproj", "atarg", "proj_deformed", "targ_deformed", "ecm", "sigininn_override", "proj_r", "proj_a",
               "targ_r", "targ_a", "proj_d_min", "targ_d_min")


class Engine:
    def __init__(self, params: dict[str, float] | None = None, seed: int = 1, **overrides):
        vals = read_parameters(None, [f"{k}={v}" for k, v in (params or {}).items()])
        vals.update({k.lower(): float(x) for k, x in overrides.items()})
        self.values = vals
        self.lib = _lib.load()
        self.params = smc_params_from(vals, seed)
        h = ctypes.c_void_p()
        _lib.check(self.lib.smc_create(ctypes.byref(self.params), ctypes.byref(h)), "smc_create")
        self.h = h
        info = _lib.SmcInfo()
        _lib.check(self.lib.smc_get_info(self.h, ctypes.byref(info)), "smc_get_info")
        self.info = info
        self.nx, self.ny, self.A, self.B = info.nx, info.ny, info.A, info.B
        self.pt_bins = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.smc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------
    def _host_buffers(self, n: int, want) -> dict[str, np.ndarray]:
        g = (n, self.nx, self.ny)
        AB = self.A + self.B
        shapes = {"ecc": ((n, _lib.ECC_LEN), np.float64), "rho": (g, np.float32), "ta": (g, np.float32),
                  "tb": (g, np.float32), "npart": ((n, 2), np.int32), "ncoll": ((n,), np.int32),
                  "b": ((n,), np.float64), "attempts": ((n,), np.int32),
                  "positions": ((n, AB, 2), np.float64), "wounded": ((n, AB), np.uint8),
                  "tangents": ((n, AB, 4), np.float64),
                  "collisions": ((n, self.info.max_collisions, 2), np.float64),
                  "orientation": ((n, 4), np.float64),
                  "rho_pt": ((n, self.nx, self.ny, max(1, self.pt_bins)), np.float32),
                  "rho_binary": (g, np.float32), "spectator_a": (g, np.float32), "spectator_b": (g, np.float32)}
        return {k: np.zeros(*shapes[k]) for k in want}

    @staticmethod
    def _outputs(bufs: dict, device: bool) -> _lib.SmcOutputs:
        o = _lib.SmcOutputs()
        o.device = 1 if device else 0
        for k in OUTPUT_NAMES:
            setattr(o, k, _lib.ptr(bufs.get(k)))
        return o

    def generate(self, first_event: int, n: int, want=("ecc", "npart", "ncoll", "b")) -> dict[str, np.ndarray]:
        """Batched event generation into host arrays."""
        bufs = self._host_buffers(n, want)
        o = self._outputs(bufs, False)
        _lib.check(self.lib.smc_generate(self.h, first_event, n, ctypes.byref(o)), "smc_generate")
        return bufs

    def generate_plain(self, first_event: int, n: int, want=("ecc", "npart", "ncoll", "b")) -> dict[str, np.ndarray]:
        """The unbatched path: one event per launch sequence."""
        bufs = self._host_buffers(n, want)
        o = self._outputs(bufs, False)
        _lib.check(self.lib.smc_generate_plain(self.h, first_event, n, ctypes.byref(o)), "smc_generate_plain")
        return bufs

    def generate_mixed(self, systems: list[dict], system_of_event, first_event: int = 0,
                       want=("ecc", "npart", "ncoll", "b"), device_bufs: dict | None = None, graph: bool = False):
        """Events of several collision systems in one batch.  systems are
        parameters.dat key sets: the nucleus and energy keys (SYSTEM_KEYS)
        start from their defaults, every other key is this engine's unless
        given (only the impact-parameter range and the Npart cut may differ
        besides); system_of_event[e] selects event first_event + e's system.
        graph: the batch as one CUDA graph (smc_generate_mixed_graph; device
        buffers only)."""
        nsys = len(systems)
        arr = (_lib.SmcParams * nsys)()
        for k, sysv in enumerate(systems):
            # the nucleus and energy keys start from their defaults; the
            # model, grid and cut keys are this engine's
            vals = dict(self.values)
            for key in SYSTEM_KEYS:
                vals[key] = DEFAULTS[key] if key in DEFAULTS else EXTENSION_KEYS[key]
            vals.update({key.lower(): float(v) for key, v in sysv.items()})
            arr[k] = smc_params_from(vals, self.params.seed)
        sel = np.ascontiguousarray(system_of_event, dtype=np.int32)
        n = len(sel)
        if device_bufs is not None:
            o = self._outputs(device_bufs, True)
            bufs = device_bufs
        else:
            bufs = self._host_buffers(n, want)
            o = self._outputs(bufs, False)
        if graph:
            if device_bufs is None:
                raise ValueError("a graph-captured mixed batch writes device buffers")
            _lib.check(self.lib.smc_generate_mixed_graph(self.h, arr, nsys, first_event, n, _lib.ptr(sel),
                                                         ctypes.byref(o)), "smc_generate_mixed_graph")
        else:
            _lib.check(self.lib.smc_generate_mixed(self.h, arr, nsys, first_event, n, _lib.ptr(sel),
                                                   ctypes.byref(o)), "smc_generate_mixed")
        return bufs

    def generate_graph_into(self, first_event: int, n: int, device_bufs: dict) -> None:
        """generate_into through smc_generate_graph: the batch's launches
        captured once as a CUDA graph and replayed."""
        o = self._outputs(device_bufs, True)
        _lib.check(self.lib.smc_generate_graph(self.h, first_event, n, ctypes.byref(o)), "smc_generate_graph")

    def generate_into(self, first_event: int, n: int, device_bufs: dict, plain: bool = False) -> None:
        """Writes into caller-owned device tensors (keys of OUTPUT_NAMES)."""
        o = self._outputs(device_bufs, True)
        fn = self.lib.smc_generate_plain if plain else self.lib.smc_generate
        _lib.check(fn(self.h, first_event, n, ctypes.byref(o)), "smc_generate")

    def inject(self, xy_proj, xy_targ, b=None, want=("ecc", "npart", "ncoll", "rho")) -> dict[str, np.ndarray]:
        """Pairing, grids and eccentricities from given nucleon positions
        (xy_proj [n,A,2], xy_targ [n,B,2], b [n])."""
        xp = np.ascontiguousarray(xy_proj, dtype=np.float64)
        xt = np.ascontiguousarray(xy_targ, dtype=np.float64)
        if xp.ndim == 2:
            xp, xt = xp[None], xt[None]
        n = xp.shape[0]
        if xp.shape[1:] != (self.A, 2) or xt.shape[1:] != (self.B, 2) or xt.shape[0] != n:
            raise ValueError("positions must be [n,A,2] and [n,B,2]")
        bb = None if b is None else np.ascontiguousarray(np.broadcast_to(b, (n,)), dtype=np.float64)
        bufs = self._host_buffers(n, want)
        o = self._outputs(bufs, False)
        _lib.check(self.lib.smc_inject(self.h, n, _lib.ptr(xp), _lib.ptr(xt), _lib.ptr(bb), ctypes.byref(o)),
                   "smc_inject")
        return bufs

    def average(self, first_event: int, n: int, from_order: int = 2, to_order: int = 3,
                reaction_plane: bool = True, xy_proj=None, xy_targ=None, b=None):
        """Event-averaged entropy densities (rho * finalFactor) rotated to each
        order's participant plane (and, with reaction_plane, recentred only).
        Returns (mean, mean_rp), each [orders][nx][ny]; the number of events
        with a collision that entered them is left in last_average_events."""
        no = to_order - from_order + 1
        mean = np.zeros((no, self.nx, self.ny))
        mean_rp = np.zeros((no, self.nx, self.ny)) if reaction_plane else None
        xp = xt = bb = None
        if xy_proj is not None:
            xp = np.ascontiguousarray(xy_proj, dtype=np.float64)
            xt = np.ascontiguousarray(xy_targ, dtype=np.float64)
            n = xp.shape[0]
            if b is not None:
                bb = np.ascontiguousarray(np.broadcast_to(b, (n,)), dtype=np.float64)
        used = ctypes.c_int(0)
        _lib.check(self.lib.smc_average(self.h, first_event, n, _lib.ptr(xp), _lib.ptr(xt), _lib.ptr(bb),
                                        from_order, to_order, 1 if reaction_plane else 0, _lib.ptr(mean),
                                        _lib.ptr(mean_rp), ctypes.byref(used)), "smc_average")
        self.last_average_events = used.value
        return mean, mean_rp

    def average_profiles(self, first_event: int, n: int, from_order: int = 2, to_order: int = 3,
                         want=("sd", "sd_rp"), xy_proj=None, xy_targ=None, b=None) -> dict:
        """Averaged-mode means (smc_average_profiles): any of sd, ta_tb, ta,
        tb, rho_binary, spectator_a, spectator_b and their _rp (reaction
        plane) versions, each [orders, nx, ny]; the events used are left in
        last_average_events."""
        no = to_order - from_order + 1
        outs = {k: np.zeros((no, self.nx, self.ny)) for k in want}
        o = _lib.SmcAverageOutputs(*[_lib.ptr(outs.get(k)) for k in _lib.AVERAGE_FIELDS])
        xp = xt = bb = None
        if xy_proj is not None:
            xp = np.ascontiguousarray(xy_proj, dtype=np.float64)
            xt = np.ascontiguousarray(xy_targ, dtype=np.float64)
            n = xp.shape[0]
            if b is not None:
                bb = np.ascontiguousarray(np.broadcast_to(b, (n,)), dtype=np.float64)
        used = ctypes.c_int(0)
        _lib.check(self.lib.smc_average_profiles(self.h, first_event, n, _lib.ptr(xp), _lib.ptr(xt), _lib.ptr(bb),
                                                 from_order, to_order, ctypes.byref(o), ctypes.byref(used)),
                   "smc_average_profiles")
        self.last_average_events = used.value
        return outs

    def average_binned(self, first_event: int, n: int, npart_edges, order: int = 2, method: int = 1):
        """Npart-binned event averages of rho * finalFactor, each event
        recentred and rotated to its order-n participant plane: method 0
        moves and re-splats the sources (the reference's method), method 1
        resamples the density bilinearly.  Returns (mean [nbins,nx,ny],
        counts [nbins])."""
        edges = np.ascontiguousarray(npart_edges, dtype=np.int32)
        nb = len(edges) - 1
        mean = np.zeros((nb, self.nx, self.ny))
        counts = np.zeros(nb, dtype=np.int32)
        _lib.check(self.lib.smc_average_binned(self.h, first_event, n, order, method, nb, _lib.ptr(edges),
                                               _lib.ptr(mean), _lib.ptr(counts)), "smc_average_binned")
        return mean, counts

    def adjoint(self, first_event: int, n: int, g_eps=None, g_rho=None, xy_proj=None, xy_targ=None, b=None,
                tangent_proj=None, tangent_targ=None):
        """Gradients of L = sum_e g_eps[e,0] |eps_2| + g_eps[e,1] |eps_3| +
        sum g_rho[e] * rho_e with respect to (width, alpha, R, a) for the
        events first_event.. (or the injected positions, with optional
        position tangents [n,A,4], [n,B,4]), the structure of each event
        (participants, windows, cuts, hot-spot region) held fixed.  g_eps
        [n,2] and g_rho [n,nx,ny] are host arrays or None.  Returns
        (grad [4], per-event grad [n,4])."""
        ge = None if g_eps is None else np.ascontiguousarray(g_eps, dtype=np.float64).reshape(n, 2)
        gr = None if g_rho is None else np.ascontiguousarray(g_rho, dtype=np.float32).reshape(n, self.nx, self.ny)
        xp = xt = bb = None
        if xy_proj is not None:
            xp = np.ascontiguousarray(xy_proj, dtype=np.float64).reshape(n, self.A, 2)
            xt = np.ascontiguousarray(xy_targ, dtype=np.float64).reshape(n, self.B, 2)
            if b is not None:
                bb = np.ascontiguousarray(np.broadcast_to(b, (n,)), dtype=np.float64)
        tp = tt = None
        if tangent_proj is not None:
            tp = np.ascontiguousarray(tangent_proj, dtype=np.float64).reshape(n, self.A, 4)
            tt = np.ascontiguousarray(tangent_targ, dtype=np.float64).reshape(n, self.B, 4)
        per = np.zeros((n, 4))
        grad = np.zeros(4)
        ct = _lib.SmcAdjointArgs(0, _lib.ptr(ge), _lib.ptr(gr), _lib.ptr(tp), _lib.ptr(tt), _lib.ptr(per))
        _lib.check(self.lib.smc_adjoint(self.h, first_event, n, _lib.ptr(xp), _lib.ptr(xt), _lib.ptr(bb),
                                        ctypes.byref(ct), _lib.ptr(grad)), "smc_adjoint")
        return grad, per

    def kln_pt_table(self, pt_min: float = 0.1, d_pt: float = 0.1, nbins: int = 20) -> np.ndarray:
        """The p_T-differential dN/dy d^2p_T table [tmax][tmax][nbins] at
        p_T = pt_min + k d_pt (smc_kln_pt_table; MCnucl::makeTable(ptmin,
        dpt, iPtmax)); afterwards the "rho_pt" output holds every event's
        per-cell values of these bins."""
        t = self.info.kln_tmax
        out = np.zeros((t, t, nbins))
        _lib.check(self.lib.smc_kln_pt_table(self.h, pt_min, d_pt, nbins, _lib.ptr(out), out.size),
                   "smc_kln_pt_table")
        self.pt_bins = nbins
        return out

    def kln_table(self) -> np.ndarray:
        t = self.info.kln_tmax
        out = np.zeros((t, t))
        _lib.check(self.lib.smc_kln_table(self.h, _lib.ptr(out), t * t), "smc_kln_table")
        return out

    def set_configurations(self, A: int, xyz) -> None:
        """Light nuclei of mass number A from a table of configurations,
        xyz [nconf][A][3] in fm (None or an empty table: Woods-Saxon again);
        smc_set_configurations."""
        if xyz is None or len(xyz) == 0:
            _lib.check(self.lib.smc_set_configurations(self.h, A, None, 0), "smc_set_configurations")
            return
        t = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64))
        if t.ndim != 3 or t.shape[1:] != (A, 3):
            raise ValueError(f"configurations for A={A}: shape [nconf][{A}][3], got {t.shape}")
        _lib.check(self.lib.smc_set_configurations(self.h, A, _lib.ptr(t), t.shape[0]), "smc_set_configurations")

    def load_configurations(self, A: int, path: str) -> None:
        """set_configurations from a file in the reference's layout for A
        (tables/he3_plaintext.dat, he4_plaintext.dat, carbon_plaintext.dat,
        oxygen_plaintext.dat); smc_load_configurations."""
        _lib.check(self.lib.smc_load_configurations(self.h, A, str(path).encode()), "smc_load_configurations")

    def autotune(self, n_events: int = 8192) -> dict:
        """Times the splat paths and events per launch on this context's
        workload and keeps the fastest (smc_autotune)."""
        t = _lib.SmcTuning()
        _lib.check(self.lib.smc_autotune(self.h, n_events, ctypes.byref(t)), "smc_autotune")
        names = [f"{p}_{c}" for p in ("tensor_cores", "cuda_cores") for c in (2048, 4096, 8192, 16384)]
        return {"tensor_cores": bool(t.tensor_cores), "chunk": t.chunk,
                "events_per_s": dict(zip(names, list(t.events_per_s)))}

    def set_grid_path(self, tensor_cores: bool) -> None:
        """Batched splat on the tcgen05 tensor cores (default) or the FP32 CUDA cores."""
        _lib.check(self.lib.smc_set_grid_path(self.h, 1 if tensor_cores else 0), "smc_set_grid_path")

    def set_timing(self, enabled: bool) -> None:
        _lib.check(self.lib.smc_set_timing(self.h, 1 if enabled else 0), "smc_set_timing")

    def stats(self) -> dict:
        st = _lib.SmcStats()
        _lib.check(self.lib.smc_get_stats(self.h, ctypes.byref(st)), "smc_get_stats")
        return {k: getattr(st, k) for k, _ in _lib.SmcStats._fields_}

    def reset_stats(self) -> None:
        _lib.check(self.lib.smc_reset_stats(self.h), "smc_reset_stats")

    def set_stream(self, stream_handle: int | None) -> None:
        _lib.check(self.lib.smc_set_stream(self.h, stream_handle), "smc_set_stream")
