"""ctypes mirror of include/mytrim_gpu.h and the loader of libmytrim_gpu.so.

The library is the product: if it is missing or fails to load, importing the
engine raises -- there is no CPU fallback.
"""
import ctypes as C
from pathlib import Path

MAX_ELEMENTS = 4
MAX_LAYERS = 8
SCOEF_ROWS = 92

OK = 0
STATUS_NAMES = {
    0: "MTG_OK", 1: "MTG_ERR_BAD_INPUT", 2: "MTG_ERR_DATA", 3: "MTG_ERR_OOM",
    4: "MTG_ERR_QUEUE_FULL", 5: "MTG_ERR_TIMEOUT", 6: "MTG_ERR_NUMERIC", 7: "MTG_ERR_CUDA",
    8: "MTG_ERR_NO_DEVICE", 9: "MTG_ERR_STATE",
}
ERR_QUEUE_FULL = 4

PREC_FP64, PREC_FP32, PREC_FP32_SURROGATE = 0, 1, 2
BC_PBC, BC_INF, BC_CUT = 0, 1, 2
TALLY_VACCOUNT, TALLY_RANGE, TALLY_PRIMARIES = 0, 1, 2


class ScoefRow(C.Structure):
    _fields_ = [("mm1", C.c_double), ("m1", C.c_double), ("mnat", C.c_double), ("rho", C.c_double),
                ("atrho", C.c_double), ("vfermi", C.c_double), ("heat", C.c_double), ("lfctr", C.c_double),
                ("pcoef", C.c_double * 8)]


class Element(C.Structure):
    _fields_ = [("Z", C.c_int), ("m", C.c_double), ("t", C.c_double), ("Edisp", C.c_double),
                ("Elbind", C.c_double)]


class Material(C.Structure):
    _fields_ = [("rho", C.c_double), ("n_elements", C.c_int), ("elements", Element * MAX_ELEMENTS)]


GEOM_LAYERS, GEOM_CLUSTERS = 0, 1
POT_UNIVERSAL, POT_MOLIERE, POT_CKR = 0, 1, 2


class Sample(C.Structure):
    _fields_ = [("n_layers", C.c_int), ("thickness", C.c_double * MAX_LAYERS),
                ("material", Material * MAX_LAYERS), ("w", C.c_double * 3), ("bc", C.c_int * 3),
                ("geometry", C.c_int), ("cluster_hash", C.c_int * 3), ("n_clusters", C.c_longlong),
                ("clusters", C.POINTER(C.c_double))]


class Ion(C.Structure):
    _fields_ = [("Z", C.c_int), ("m", C.c_double), ("E", C.c_double), ("Ef", C.c_double),
                ("dir", C.c_double * 3), ("pos", C.c_double * 3)]


class Sim(C.Structure):
    _fields_ = [("sample", Sample), ("ion", Ion), ("n_primaries", C.c_longlong),
                ("first_primary", C.c_longlong), ("tally_mode", C.c_int),
                ("primaries_only", C.c_int), ("hist_range_bin", C.c_double), ("hist_range_n", C.c_int),
                ("hist_vac_bin", C.c_double), ("hist_vac_n", C.c_int), ("surface_binding", C.c_double),
                ("voxel_n", C.c_int * 3), ("voxel_origin", C.c_double * 3), ("voxel_size", C.c_double * 3),
                ("hist_lateral_bin", C.c_double), ("hist_lateral_n", C.c_int), ("max_generation", C.c_int),
                ("hist_evac_rows", C.c_int), ("potential", C.c_int), ("md_tag_Z", C.c_int),
                ("md_tag_Emin", C.c_double), ("md_tag_Emax", C.c_double)]


class Config(C.Structure):
    _fields_ = [("tmin", C.c_double), ("tau", C.c_double), ("cw", C.c_double), ("length_scale", C.c_double),
                ("precision", C.c_int), ("seed", C.c_ulonglong), ("max_collisions_per_member", C.c_longlong),
                ("stack_capacity", C.c_int), ("block_threads", C.c_int), ("max_primaries_per_refill", C.c_int),
                ("refill_min_idle", C.c_int)]


class Totals(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("primaries", "members", "collisions", "vacancies", "replacements",
                                             "interstitials", "substitutionals", "lost")] + \
               [(n, C.c_double) for n in ("Eel", "Enuc", "Elost", "Eunfollowed")] + \
               [("range_n", C.c_longlong)] + \
               [(n, C.c_double) for n in ("sx", "sxx", "sy", "syy", "sz", "szz",
                                          "vac_s2", "eel_s2", "enuc_s2", "coll_s2")] + \
               [(n, C.c_longlong) for n in ("newton_iterations", "rejection_passes", "surrogate_fallbacks",
                                            "sputtered", "backscattered")] + \
               [(n, C.c_double) for n in ("Esputtered", "Evoxel")] + \
               [("hist_dropped", C.c_longlong)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}

    @classmethod
    def field_names(cls):
        return [n for n, _ in cls._fields_]


class MemberRecord(C.Structure):
    _fields_ = [("key", C.c_ulonglong), ("sim", C.c_int), ("species", C.c_int), ("gen", C.c_int),
                ("state", C.c_int), ("ncoll", C.c_uint), ("nvac", C.c_uint), ("E", C.c_double),
                ("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("eel", C.c_double)]


class Event(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("x", "y", "z", "E", "aux", "m")] + \
               [("key", C.c_ulonglong), ("primary", C.c_longlong)] + \
               [(n, C.c_int) for n in ("sim", "kind", "Z", "gen", "state", "tag", "md")]


# event kinds (mtg_event_kind)
EV_VACANCY, EV_REPLACEMENT, EV_BRANCH, EV_DISSIPATE, EV_REST, EV_LOST, EV_HISTORY = 1, 2, 3, 4, 5, 6, 7


class SurrogateConfig(C.Structure):
    _fields_ = [("n_train", C.c_longlong), ("batch", C.c_int), ("epochs", C.c_int), ("qat_epochs", C.c_int),
                ("lr", C.c_float), ("seed", C.c_ulonglong), ("w_tau", C.c_float), ("target", C.c_int),
                ("weighting", C.c_int)]


SURROGATE_TARGETS = {"quadrature": 0, "magic": 1}  # MTG_SURROGATE_TARGET_*
SURROGATE_WEIGHTS = {"uniform": 0, "transfer": 1}  # MTG_SURROGATE_WEIGHT_*


class SurrogateReport(C.Structure):
    _fields_ = [("final_loss", C.c_double), ("train_seconds", C.c_double), ("steps", C.c_longlong)]


SURROGATE_NPARAM = 8642


class Stats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("reduce_ms", C.c_double), ("launches", C.c_int),
                ("drains", C.c_int), ("grid", C.c_int), ("block", C.c_int), ("stack_capacity", C.c_int),
                ("overflowed", C.c_longlong), ("collisions", C.c_longlong), ("device_bytes", C.c_size_t),
                ("h2d_bytes", C.c_longlong), ("d2h_bytes", C.c_longlong), ("warp_steps", C.c_longlong),
                ("kernel_level", C.c_int), ("max_take", C.c_int), ("events_overflowed", C.c_int),
                ("overflow_retries", C.c_int)]


class Tuning(C.Structure):
    _fields_ = [("block_threads", C.c_int), ("max_primaries_per_refill", C.c_int), ("stack_capacity", C.c_int),
                ("refill_min_idle", C.c_int), ("heuristic_take", C.c_int), ("default_collisions_per_s", C.c_double),
                ("best_collisions_per_s", C.c_double), ("trials", C.c_int), ("changed", C.c_int)]


# mtg_stats.kernel_level values
KERNEL_LEVELS = ("lean", "mid", "events", "geometry", "full", "clusters", "clusters+events")

# symbol -> (restype, argtypes); must match include/mytrim_gpu.h
_P = C.c_void_p
SIGNATURES = {
    "mtg_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "mtg_destroy": (C.c_int, [_P]),
    "mtg_last_error": (C.c_char_p, [_P]),
    "mtg_set_tables": (C.c_int, [_P, C.POINTER(ScoefRow), C.c_int]),
    "mtg_load_tables": (C.c_int, [_P, C.c_char_p]),
    "mtg_configure": (C.c_int, [_P, C.POINTER(Config)]),
    "mtg_run": (C.c_int, [_P, C.POINTER(Sim), C.c_int, C.POINTER(Totals), C.POINTER(C.c_longlong)]),
    "mtg_prepare": (C.c_int, [_P, C.POINTER(Sim), C.c_int]),
    "mtg_launch_async": (C.c_int, [_P, _P]),
    "mtg_collect": (C.c_int, [_P, C.POINTER(Totals), C.POINTER(C.c_longlong)]),
    "mtg_get_primaries": (C.c_int, [_P, C.c_longlong, C.c_longlong, C.POINTER(C.c_longlong),
                                    C.POINTER(C.c_longlong), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_int)]),
    "mtg_get_voxels": (C.c_int, [_P, C.c_int, C.POINTER(C.c_float), C.c_longlong]),
    "mtg_get_voxels64": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double), C.c_longlong]),
    "mtg_autotune": (C.c_int, [_P, C.c_void_p, C.c_int, C.c_longlong, C.POINTER(Tuning)]),
    "mtg_set_record_capacity": (C.c_int, [_P, C.c_longlong]),
    "mtg_get_records": (C.c_int, [_P, C.POINTER(MemberRecord), C.c_longlong, C.POINTER(C.c_longlong)]),
    "mtg_set_event_log": (C.c_int, [_P, C.c_uint, C.c_longlong]),
    "mtg_get_events": (C.c_int, [_P, C.POINTER(Event), C.c_longlong, C.POINTER(C.c_longlong),
                                 C.POINTER(C.c_longlong)]),
    "mtg_stopping": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(Material), C.POINTER(C.c_double),
                               C.c_longlong, C.c_int, C.POINTER(C.c_double)]),
    "mtg_scatter": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_longlong, C.c_int,
                              C.POINTER(C.c_double)]),
    "mtg_scatter_potential": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_longlong, C.c_int,
                                        C.c_int, C.POINTER(C.c_double)]),
    "mtg_get_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "mtg_surrogate_train": (C.c_int, [_P, C.POINTER(SurrogateConfig), C.POINTER(SurrogateReport)]),
    "mtg_surrogate_get_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_longlong]),
    "mtg_surrogate_set_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_longlong]),
    "mtg_surrogate_gradients": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                          C.c_longlong, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "mtg_surrogate_quadrature": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_longlong,
                                           C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mtg_reduce_primaries_noalloc": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, C.c_longlong, _P, _P,
                                               C.c_char_p, C.c_size_t]),
}

_lib = None


def library_path():
    return Path(__file__).resolve().parent / "_lib" / "libmytrim_gpu.so"


def load(path=None):
    """Load libmytrim_gpu.so (raises if it is missing -- there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else library_path()
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with mytrim_gb300.build.build() "
                           "(the engine has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class EngineError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
