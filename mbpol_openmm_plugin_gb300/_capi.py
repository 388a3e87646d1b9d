"""ctypes binding to the C ABI in include/mbpol_gb300.h.

The shared library is built in-tree (``python -m mbpol_openmm_plugin_gb300.build``
or ``__graft_entry__.build()``).  There is no CPU fallback: if the library or
a CUDA device is missing, the calls raise."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libmbpol_gb300.so")

MBPOL_OK = 0
STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARGUMENT", 2: "CUDA", 3: "NOT_CONVERGED", 4: "BOX_TOO_SMALL",
    5: "CAPACITY", 6: "STATE", 7: "NO_DEVICE",
}
TERM_ONEBODY, TERM_TWOBODY, TERM_THREEBODY, TERM_ELECTROSTATICS, TERM_DISPERSION = range(5)
NUM_TERMS = 5
ALL_TERMS = 0x1F

EXPORTED = [
    "mbpol_electrostatics_params_default", "mbpol_context_create", "mbpol_context_destroy",
    "mbpol_add_average3_site", "mbpol_add_onebody_force", "mbpol_add_twobody_force",
    "mbpol_add_threebody_force", "mbpol_add_electrostatics_force", "mbpol_add_dispersion_force",
    "mbpol_add_dispersion_ions",
    "mbpol_set_positions", "mbpol_compute", "mbpol_set_masses", "mbpol_set_velocities", "mbpol_md_run",
    "mbpol_get_state", "mbpol_get_induced_dipoles", "mbpol_get_counts", "mbpol_get_electrostatic_potential",
    "mbpol_get_system_multipole_moments",
    "mbpol_profile_enable", "mbpol_profile_read", "mbpol_launch_count", "mbpol_status_string", "mbpol_last_error",
    "mbpol_twobody_dimers_noalloc",
    "mbpol_guess_collect", "mbpol_guess_num_samples", "mbpol_guess_train", "mbpol_guess_get_params",
    "mbpol_guess_set_params", "mbpol_guess_descriptors", "mbpol_guess_loss_grad", "mbpol_guess_fit_predictor",
    "mbpol_set_clusters", "mbpol_get_cluster_results", "mbpol_set_threebody_evaluator",
    "mbpol_probe_thole_inverse_rs", "mbpol_probe_water_charges", "mbpol_set_autotune", "mbpol_set_launch_shape",
    "mbpol_get_launch_shape",
    "mbpol_guess_select_network", "mbpol_update_parameters",
]
GUESS_BLOCK_FLOATS = 9033  # MBPOL_GUESS_BLOCK_FLOATS
GUESS_PREDICTOR_ORDER = 7  # MBPOL_GUESS_PREDICTOR_ORDER
GUESS_HISTORY = 12  # MBPOL_GUESS_HISTORY
GUESS_PARAMS = 8905
GUESS_INPUTS = 64
NOALLOC_MAX_DIMERS = 65536  # MBPOL_NOALLOC_MAX_DIMERS
KERNELS = ["poly2b", "poly3b", "elec_fixed_field", "elec_induced_update", "elec_pme_dipoles", "elec_energy_forces",
           "elec_direct_field"]


class MBPolError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class ElectrostaticsParams(ctypes.Structure):
    _fields_ = [
        ("nonbonded_method", ctypes.c_int),
        ("cutoff", ctypes.c_double),
        ("ewald_alpha", ctypes.c_double),
        ("pme_grid", ctypes.c_int * 3),
        ("ewald_error_tolerance", ctypes.c_double),
        ("max_iterations", ctypes.c_int),
        ("target_epsilon", ctypes.c_double),
        ("thole", ctypes.c_double * 5),
        ("include_charge_redistribution", ctypes.c_int),
        ("guess", ctypes.c_int),
        ("pme_fixed_field", ctypes.c_int),
    ]


_lib = None


def load(path=None):
    """Load (once) and return the library; raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise MBPolError(7, "CUDA library %s is not built (run __graft_entry__.build())" % path)
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    I, D = ctypes.c_int, ctypes.c_double
    sig = {
        "mbpol_electrostatics_params_default": (None, [ctypes.POINTER(ElectrostaticsParams)]),
        "mbpol_context_create": (I, [I, I, ctypes.POINTER(P)]),
        "mbpol_context_destroy": (I, [P]),
        "mbpol_add_average3_site": (I, [P, I, I, I, I, D, D, D]),
        "mbpol_add_onebody_force": (I, [P, I, P, I]),
        "mbpol_add_twobody_force": (I, [P, I, P, I, D]),
        "mbpol_add_threebody_force": (I, [P, I, P, I, D, I]),
        "mbpol_add_electrostatics_force": (I, [P, ctypes.POINTER(ElectrostaticsParams), P, P, P, P, P]),
        "mbpol_add_dispersion_force": (I, [P, I, P, I, D, P, P]),
        "mbpol_add_dispersion_ions": (I, [P, I, P]),
        "mbpol_set_positions": (I, [P, P, P]),
        "mbpol_compute": (I, [P, ctypes.c_uint, P, P]),
        "mbpol_set_masses": (I, [P, P]),
        "mbpol_set_velocities": (I, [P, P]),
        "mbpol_md_run": (I, [P, I, D, D, D, ctypes.c_ulonglong, ctypes.POINTER(D), P, ctypes.POINTER(ctypes.c_long)]),
        "mbpol_get_state": (I, [P, P, P, P]),
        "mbpol_get_induced_dipoles": (I, [P, P, ctypes.POINTER(I), ctypes.POINTER(D)]),
        "mbpol_get_counts": (I, [P, P]),
        "mbpol_get_electrostatic_potential": (I, [P, I, P, P]),
        "mbpol_get_system_multipole_moments": (I, [P, P, P]),
        "mbpol_guess_fit_predictor": (I, [P, P, P, P, I, P, P]),
        "mbpol_profile_enable": (I, [I]),
        "mbpol_launch_count": (ctypes.c_ulonglong, []),
        "mbpol_profile_read": (I, [I, ctypes.POINTER(D), ctypes.POINTER(ctypes.c_long)]),
        "mbpol_status_string": (ctypes.c_char_p, [I]),
        "mbpol_last_error": (ctypes.c_char_p, []),
        "mbpol_twobody_dimers_noalloc": (I, [P, P, P, I, P, P, P, P]),
        "mbpol_guess_collect": (I, [P]),
        "mbpol_guess_num_samples": (I, [P, ctypes.POINTER(ctypes.c_long)]),
        "mbpol_guess_train": (I, [P, I, I, D, ctypes.c_ulonglong, ctypes.POINTER(D)]),
        "mbpol_guess_get_params": (I, [P, P]),
        "mbpol_guess_set_params": (I, [P, P]),
        "mbpol_guess_descriptors": (I, [P, P]),
        "mbpol_guess_loss_grad": (I, [P, P, P, I, ctypes.POINTER(D), P, P]),
        "mbpol_set_clusters": (I, [P, P, I]),
        "mbpol_set_threebody_evaluator": (I, [P, I]),
        "mbpol_probe_thole_inverse_rs": (I, [D, D, D, D, P]),
        "mbpol_probe_water_charges": (I, [P, P, P]),
        "mbpol_set_autotune": (I, [P, I]),
        "mbpol_set_launch_shape": (I, [P, I, I]),
        "mbpol_get_launch_shape": (I, [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]),
        "mbpol_guess_select_network": (I, [P, I]),
        "mbpol_update_parameters": (I, [P, ctypes.c_uint, I, P, P, P, P, P, P]),
        "mbpol_get_cluster_results": (I, [P, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != MBPOL_OK:
        msg = load().mbpol_last_error().decode(errors="replace")
        raise MBPolError(status, msg)


def ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def as_c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)
