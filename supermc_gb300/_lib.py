"""ctypes binding of the C ABI declared in include/supermc.h.

The library is the in-tree ``supermc_gb300/_build/libsupermc_gb300.so``;
loading fails loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("SUPERMC_GB300_LIB") or os.path.join(HERE, "_build", "libsupermc_gb300.so")

SMC_OK = 0
SMC_ERR_CUDA = 7
STATUS_NAMES = {
    0: "SMC_OK", 1: "SMC_ERR_ARGUMENT", 2: "SMC_ERR_CONFIG", 3: "SMC_ERR_RETRY_CAP",
    4: "SMC_ERR_KLN_TABLE", 5: "SMC_ERR_ZERO_DNDY", 6: "SMC_ERR_CAPACITY", 7: "SMC_ERR_CUDA",
    8: "SMC_ERR_NO_DEVICE", 9: "SMC_ERR_SCRATCH_LIMIT",
}
ECC_LEN = 49

# the entry points include/supermc.h declares (tests/test_capi.py checks the set)
EXPORTS = ["smc_create", "smc_destroy", "smc_get_info", "smc_status_string", "smc_cuda_error_string",
           "smc_set_stream",
           "smc_synchronize", "smc_generate", "smc_inject", "smc_generate_mixed", "smc_generate_plain",
           "smc_set_timing",
           "smc_set_grid_path", "smc_get_stats", "smc_reset_stats", "smc_kln_table", "smc_write_ecc",
           "smc_write_density_block", "smc_write_density_4col", "smc_inject_noalloc", "smc_average",
           "smc_average_binned", "smc_adjoint", "smc_autotune", "smc_generate_graph", "smc_average_profiles",
           "smc_write_binary_table", "smc_write_nucleon_tables", "smc_write_ecc_deformed",
           "smc_generate_mixed_graph", "smc_sample_nuclei", "smc_set_configurations",
           "smc_load_configurations", "smc_read_configurations", "smc_write_npy", "smc_write_ecc_npy",
           "smc_kln_pt_table", "smc_write_participant_table", "smc_write_spectator_table",
           "smc_write_density_pt"]


class SmcError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)}")
        self.status = status


class SmcParams(ctypes.Structure):
    _fields_ = [
        ("which_mc_model", ctypes.c_int), ("sub_model", ctypes.c_int),
        ("shape_of_nucleons", ctypes.c_int), ("shape_of_entropy", ctypes.c_int),
        ("collision_criterion", ctypes.c_int),
        ("Aproj", ctypes.c_int), ("Atarg", ctypes.c_int),
        ("proj_deformed", ctypes.c_int), ("targ_deformed", ctypes.c_int),
        ("ecm", ctypes.c_double), ("alpha", ctypes.c_double), ("gauss_nucl_width", ctypes.c_double),
        ("quark_width", ctypes.c_double), ("lambda_", ctypes.c_double),
        ("bmin", ctypes.c_double), ("bmax", ctypes.c_double),
        ("npmin", ctypes.c_int), ("npmax", ctypes.c_int),
        ("maxx", ctypes.c_double), ("maxy", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
        ("final_factor", ctypes.c_double),
        ("tmax", ctypes.c_int), ("tmax_subdivision", ctypes.c_int),
        ("ecc_from_order", ctypes.c_int), ("ecc_to_order", ctypes.c_int),
        ("proj_R", ctypes.c_double), ("proj_a", ctypes.c_double),
        ("targ_R", ctypes.c_double), ("targ_a", ctypes.c_double),
        ("proj_d_min", ctypes.c_double), ("targ_d_min", ctypes.c_double),
        ("sigin_override", ctypes.c_double),
        ("kln_npt", ctypes.c_int), ("kln_nkt", ctypes.c_int), ("kln_nphi", ctypes.c_int),
        ("seed", ctypes.c_uint64),
        ("max_attempts", ctypes.c_int), ("max_collisions", ctypes.c_int),
        ("ws_inverse_cdf", ctypes.c_int),
        ("cc_fluctuation_model", ctypes.c_int), ("cc_fluctuation_gamma_theta", ctypes.c_double),
        ("cc_fluctuation_k", ctypes.c_double),
        ("kln_exact_band", ctypes.c_double),
    ]


class SmcInfo(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("sigin", ctypes.c_double), ("dsq", ctypes.c_double), ("width", ctypes.c_double),
        ("sigma_gg", ctypes.c_double), ("kln_tmax", ctypes.c_int), ("kln_dT", ctypes.c_double),
        ("A", ctypes.c_int), ("B", ctypes.c_int), ("max_collisions", ctypes.c_int),
    ]


class SmcStats(ctypes.Structure):
    _fields_ = [("events", ctypes.c_uint64), ("attempts", ctypes.c_uint64), ("launches", ctypes.c_uint64),
                ("sample_launches", ctypes.c_uint64), ("grid_launches", ctypes.c_uint64),
                ("sample_ms", ctypes.c_double), ("grid_ms", ctypes.c_double),
                ("post_launches", ctypes.c_uint64), ("post_ms", ctypes.c_double)]


class SmcOutputs(ctypes.Structure):
    _fields_ = [
        ("device", ctypes.c_int),
        ("ecc", ctypes.c_void_p), ("rho", ctypes.c_void_p), ("ta", ctypes.c_void_p), ("tb", ctypes.c_void_p),
        ("npart", ctypes.c_void_p), ("ncoll", ctypes.c_void_p), ("b", ctypes.c_void_p),
        ("attempts", ctypes.c_void_p), ("positions", ctypes.c_void_p), ("wounded", ctypes.c_void_p),
        ("tangents", ctypes.c_void_p), ("collisions", ctypes.c_void_p), ("orientation", ctypes.c_void_p),
        ("rho_pt", ctypes.c_void_p), ("rho_binary", ctypes.c_void_p), ("spectator_a", ctypes.c_void_p),
        ("spectator_b", ctypes.c_void_p),
    ]


AVERAGE_FIELDS = ("sd", "sd_rp", "ta_tb", "ta_tb_rp", "ta", "tb", "ta_rp", "tb_rp", "rho_binary", "rho_binary_rp",
                  "spectator_a", "spectator_b", "spectator_a_rp", "spectator_b_rp")


class SmcAverageOutputs(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in AVERAGE_FIELDS]


class SmcTuning(ctypes.Structure):
    _fields_ = [("tensor_cores", ctypes.c_int), ("chunk", ctypes.c_int), ("events_per_s", ctypes.c_double * 8)]


class SmcAdjointArgs(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("g_eps", ctypes.c_void_p), ("g_rho", ctypes.c_void_p),
                ("tangent_proj", ctypes.c_void_p), ("tangent_targ", ctypes.c_void_p),
                ("grad_events", ctypes.c_void_p)]


_lib = None


def load() -> ctypes.CDLL:
    """Loads the in-tree library (build it with supermc_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is missing: build the CUDA extension first "
                      "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    lib.smc_create.argtypes = [ctypes.POINTER(SmcParams), ctypes.POINTER(vp)]
    lib.smc_destroy.argtypes = [vp]
    lib.smc_destroy.restype = None
    lib.smc_get_info.argtypes = [vp, ctypes.POINTER(SmcInfo)]
    lib.smc_status_string.argtypes = [ctypes.c_int]
    lib.smc_status_string.restype = ctypes.c_char_p
    lib.smc_cuda_error_string.argtypes = []
    lib.smc_cuda_error_string.restype = ctypes.c_char_p
    lib.smc_set_stream.argtypes = [vp, vp]
    lib.smc_synchronize.argtypes = [vp]
    lib.smc_generate.argtypes = [vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(SmcOutputs)]
    lib.smc_generate_plain.argtypes = [vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(SmcOutputs)]
    lib.smc_generate_mixed.argtypes = [vp, ctypes.POINTER(SmcParams), ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                       vp, ctypes.POINTER(SmcOutputs)]
    lib.smc_generate_mixed_graph.argtypes = [vp, ctypes.POINTER(SmcParams), ctypes.c_int, ctypes.c_uint64,
                                             ctypes.c_int, vp, ctypes.POINTER(SmcOutputs)]
    lib.smc_inject.argtypes = [vp, ctypes.c_int, vp, vp, vp, ctypes.POINTER(SmcOutputs)]
    lib.smc_sample_nuclei.argtypes = [vp, ctypes.c_uint64, ctypes.c_double, vp, vp, vp, vp, vp]
    lib.smc_set_configurations.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int]
    lib.smc_load_configurations.argtypes = [vp, ctypes.c_int, ctypes.c_char_p]
    lib.smc_read_configurations.argtypes = [ctypes.c_int, ctypes.c_char_p, vp, ctypes.c_int, vp]
    lib.smc_write_npy.argtypes = [ctypes.c_char_p, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int]
    lib.smc_write_ecc_npy.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
    lib.smc_kln_table.argtypes = [vp, vp, ctypes.c_int]
    lib.smc_kln_pt_table.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int, vp, ctypes.c_size_t]
    lib.smc_set_timing.argtypes = [vp, ctypes.c_int]
    lib.smc_set_grid_path.argtypes = [vp, ctypes.c_int]
    lib.smc_write_ecc.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
    lib.smc_write_ecc_deformed.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
    lib.smc_write_density_block.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
    lib.smc_write_density_4col.argtypes = [vp, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6 + [ctypes.c_char_p]
    lib.smc_get_stats.argtypes = [vp, ctypes.POINTER(SmcStats)]
    lib.smc_write_binary_table.argtypes = [vp, ctypes.c_int, ctypes.c_char_p]
    lib.smc_write_nucleon_tables.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
                                             ctypes.c_char_p]
    lib.smc_reset_stats.argtypes = [vp]
    lib.smc_write_participant_table.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
    lib.smc_write_spectator_table.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_char_p]
    lib.smc_write_density_pt.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_char_p]
    lib.smc_average.argtypes = [vp, ctypes.c_uint64, ctypes.c_int, vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, vp, vp, ctypes.POINTER(ctypes.c_int)]
    lib.smc_inject_noalloc.argtypes = [ctypes.POINTER(SmcParams), ctypes.c_int, vp, vp, vp, vp, vp, vp, vp]
    lib.smc_average_binned.argtypes = [vp, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       vp, vp, vp]
    lib.smc_average_profiles.argtypes = [vp, ctypes.c_uint64, ctypes.c_int, vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(SmcAverageOutputs), ctypes.POINTER(ctypes.c_int)]
    lib.smc_generate_graph.argtypes = [vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(SmcOutputs)]
    lib.smc_autotune.argtypes = [vp, ctypes.c_int, ctypes.POINTER(SmcTuning)]
    lib.smc_adjoint.argtypes = [vp, ctypes.c_uint64, ctypes.c_int, vp, vp, vp, ctypes.POINTER(SmcAdjointArgs), vp]
    _lib = lib
    return lib


def check(status: int, what: str) -> None:
    if status != SMC_OK:
        if status == SMC_ERR_CUDA and _lib is not None:
            what = f"{what} ({_lib.smc_cuda_error_string().decode()})"
        raise SmcError(status, what)


def ptr(a) -> int | None:
    """Address of a numpy array or a torch tensor (None passes NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    return a.data_ptr()
