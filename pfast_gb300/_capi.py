"""ctypes binding of libpfast_gb300.so (the C ABI declared in include/pfast_gb300.h).

The library is the only compute path: lib() loads it on first use and raises if
it has not been built; there is no CPU fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpfast_gb300.so")

PFAST_OK = 0
PFAST_ERR_INVALID = 1
PFAST_ERR_CUDA = 2
PFAST_ERR_NOMEM = 3
PFAST_ERR_NO_DEVICE = 4
PFAST_ERR_NO_REFLECTION_POINT = 5
PFAST_ERR_NEGATIVE_TIME = 6
PFAST_ERR_OVER_CORRECTED = 7
PFAST_ERR_LINE_SEARCH = 8

PFAST_PLAIN_FP64 = 0
PFAST_MIXED = 1
PFAST_SCHEDULE_AUTO, PFAST_SCHEDULE_DIAGONAL, PFAST_SCHEDULE_PERSISTENT, PFAST_SCHEDULE_HYBRID = 0, 1, 2, 3
PFAST_TILE_AUTO, PFAST_TILE_4x8x32, PFAST_TILE_8x4x32 = 0, 1, 2
# autotuner candidates, in the order of pfast_survey3d_autotune's stats array
PFAST_TUNE_CANDIDATES = ("diagonal 4x8x32", "diagonal 8x4x32", "persistent 4x8x32", "persistent 8x4x32",
                         "hybrid 4x8x32", "hybrid 8x4x32")


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("maxswp", C.c_int), ("max_batch", C.c_int), ("polish_floor", C.c_double),
                ("schedule", C.c_int), ("near_source_radius", C.c_int), ("tile_shape", C.c_int)]


class Stats(C.Structure):
    _fields_ = [
        ("fwd_node_updates", C.c_longlong), ("adj_node_updates", C.c_longlong),
        ("fwd64_node_updates", C.c_longlong), ("adj64_node_updates", C.c_longlong),
        ("fwd_iters_max", C.c_int), ("adj_iters_max", C.c_int),
        ("fwd32_iters_max", C.c_int), ("adj32_iters_max", C.c_int),
        ("not_converged", C.c_int), ("batches", C.c_int),
        ("launches", C.c_longlong),
        ("ms_fwd32", C.c_double), ("ms_fwd64", C.c_double),
        ("ms_adj32", C.c_double), ("ms_adj64", C.c_double),
        ("ms_other", C.c_double), ("ms_total", C.c_double), ("candidates", C.c_int),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


SWEEP_KINDS = ("fwd64_plain", "fwd32", "fwd64_polish", "adj64_plain", "adj32", "adj64_polish")


def phase_candidates(stats):
    """{sweep kind: (schedule, tile shape) candidate name} of the phases an evaluation ran,
    decoded from pfast_stats.candidates."""
    c = int(stats["candidates"])
    return {k: PFAST_TUNE_CANDIDATES[(c >> 4 * i & 15) - 1] for i, k in enumerate(SWEEP_KINDS) if c >> 4 * i & 15}


PFAST_SCHEME_HS, PFAST_SCHEME_CGDESCENT, PFAST_SCHEME_LBFGS = 1, 2, 3
PFAST_LS_NONE, PFAST_LS_SECANT_EXACT, PFAST_LS_SECANT_WOLFE, PFAST_LS_CUBIC = 0, 1, 2, 3
PFAST_RT_TRANSMISSION, PFAST_RT_REFLECTION, PFAST_RT_JOINT = 1, 2, 3
PFAST_INV_MAX_TRIALS = 16
(PFAST_INV_VP, PFAST_INV_GRAD_RAW, PFAST_INV_GRAD, PFAST_INV_DIRECTION, PFAST_INV_GR_RAW, PFAST_INV_GR,
 PFAST_INV_GT_RAW, PFAST_INV_GT) = range(8)


class InvertOptions(C.Structure):
    _fields_ = [
        ("eval", Options), ("schemetag", C.c_int), ("lsrc", C.c_int), ("LM", C.c_int),
        ("max_linesearch", C.c_int), ("rttag", C.c_int),
        ("nux", C.c_double), ("nuy", C.c_double), ("nuz", C.c_double),
        ("minv", C.c_double), ("maxv", C.c_double), ("conv_tol", C.c_double),
        ("keep_components", C.c_int),
    ]


class InvertReport(C.Structure):
    _fields_ = [
        ("iter", C.c_int), ("E", C.c_double), ("Et", C.c_double), ("Er", C.c_double),
        ("alpha_start", C.c_double), ("ntrials", C.c_int),
        ("trial", (C.c_double * 6) * PFAST_INV_MAX_TRIALS),
        ("count", C.c_int), ("stopped", C.c_int), ("stepsize", C.c_double), ("converged", C.c_int),
        ("evals", C.c_int), ("ms_eval", C.c_double), ("ms_linesearch", C.c_double), ("ms_total", C.c_double),
    ]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_ if name != "trial"}
        d["trials"] = [tuple(self.trial[k]) for k in range(self.ntrials)]
        return d


PFAST_REQ_FORWARD, PFAST_REQ_GRADIENT = 0, 1


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_int), ("hbm_budget_bytes", C.c_double), ("max_bypass", C.c_int)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("model_id", C.c_longlong), ("survey_id", C.c_longlong), ("opt", Options),
                ("out", C.c_void_p), ("out_misfit", C.c_void_p)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("batch", C.c_int), ("queue_ms", C.c_double), ("run_ms", C.c_double),
                ("total_ms", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


SWEEP_KINDS = ("fwd64_plain", "fwd32", "fwd64_polish", "adj64_plain", "adj32", "adj64_polish")


def phase_candidates(stats):
    """{sweep kind: (schedule, tile shape) candidate name} of the phases an evaluation ran,
    decoded from pfast_stats.candidates."""
    c = int(stats["candidates"])
    return {k: PFAST_TUNE_CANDIDATES[(c >> 4 * i & 15) - 1] for i, k in enumerate(SWEEP_KINDS) if c >> 4 * i & 15}


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("failed", C.c_longlong),
                ("running", C.c_int), ("waiting", C.c_int), ("resident_models", C.c_int),
                ("resident_surveys", C.c_int), ("used_bytes", C.c_double), ("peak_bytes", C.c_double),
                ("budget_bytes", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


SWEEP_KINDS = ("fwd64_plain", "fwd32", "fwd64_polish", "adj64_plain", "adj32", "adj64_polish")


def phase_candidates(stats):
    """{sweep kind: (schedule, tile shape) candidate name} of the phases an evaluation ran,
    decoded from pfast_stats.candidates."""
    c = int(stats["candidates"])
    return {k: PFAST_TUNE_CANDIDATES[(c >> 4 * i & 15) - 1] for i, k in enumerate(SWEEP_KINDS) if c >> 4 * i & 15}


# (name, restype, argtypes) of every entry point in include/pfast_gb300.h
_p, _i, _d = C.c_void_p, C.c_int, C.c_double
SIGNATURES = [
    ("pfast_version", C.c_char_p, []),
    ("pfast_status_string", C.c_char_p, [_i]),
    ("pfast_last_error", C.c_char_p, []),
    ("pfast_default_options", None, [_p]),
    ("pfast_ctx_create", _i, [_i, _p]),
    ("pfast_ctx_destroy", _i, [_p]),
    ("pfast_ctx_set_stream", _i, [_p, _p]),
    ("pfast_ctx_set_graphs", _i, [_p, C.c_int]),
    ("pfast_ctx_synchronize", _i, [_p]),
    ("pfast_fsm3d", _i, [_p, _p, _p, _i, _i, _d, _d, _d, _i, _i, _i, _i]),
    ("pfast_adjoint_fsm3d", _i, [_p, _p, _p, _p, _p, _p, _p, _i, _i, _d, _d, _d, _i, _i, _i, _i, _p]),
    ("pfast_RT_fsm2d", _i, [_p, _p, _p, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _i, _i, _i]),
    ("pfast_Tadjoint_fsm2d", _i, [_p, _p, _p, _p, _p, _p, _p, _i, _i, _d, _d, _i, _i, _i, _p]),
    ("pfast_Radjoint_fsm2d", _i, [_p, _p, _p, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _i, _i, _i, _p]),
    ("pfast_survey3d_create", _i, [_p, _i, _i, _i, _d, _d, _d, _i, _p, _p, _p, _p, _p, _p]),
    ("pfast_survey3d_destroy", _i, [_p]),
    ("pfast_survey3d_eval", _i, [_p, _p, _p, _p, _p, _p, _p]),
    ("pfast_survey3d_forward", _i, [_p, _p, _p, _p, _p, _p]),
    ("pfast_survey3d_autotune", _i, [_p, _p, _p, _p, _p]),
    ("pfast_surveys3d_eval", _i, [_p, _i, _p, _p, _p, _p, _p, _p]),
    ("pfast_eval3d", _i, [_p, _p, _i, _i, _i, _d, _d, _d, _i, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    ("pfast_forward3d", _i, [_p, _p, _i, _i, _i, _d, _d, _d, _i, _p, _p, _p, _p, _p, _p]),
    ("pfast_survey2d_create", _i, [_p, _i, _i, _d, _d, _i, _p, _p, _i, _p, _p, _p, _i, _p, _p, _p]),
    ("pfast_survey2d_destroy", _i, [_p]),
    ("pfast_survey2d_forward", _i, [_p, _p, _p, _p, _p, _p]),
    ("pfast_survey2d_eval", _i, [_p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    ("pfast_fsm3d_noalloc", _i, [_p, _p, _i, _i, _i, _i, _d, _d, _d, _i, _i, _i, _p]),
    ("pfast_forward2d", _i, [_p, _p, _i, _i, _d, _d, _i, _p, _p, _i, _p, _i, _p, _p, _p, _p]),
    ("pfast_eval2d", _i, [_p, _p, _p, _i, _i, _d, _d, _i, _p, _p, _i, _p, _p, _p, _i, _p, _p, _p, _p, _p, _p, _p, _p,
                          _p]),
    ("pfast_invert_default_options", None, [_i, _p]),
    ("pfast_inversion2d_create", _i, [_p, _p, _p, _p, _p, _p]),
    ("pfast_inversion3d_create", _i, [_p, _p, _p, _p, _p]),
    ("pfast_inversion_resume", _i, [_p, _i, _p, _p, _p, _i, _d]),
    ("pfast_inversion_step", _i, [_p, _p]),
    ("pfast_inversion_get", _i, [_p, _i, _p]),
    ("pfast_inversion_field", _i, [_p, _i, _p]),
    ("pfast_inversion_destroy", _i, [_p]),
    ("pfast_server_create", _i, [_p, _p]),
    ("pfast_server_destroy", _i, [_p]),
    ("pfast_server_put_model", _i, [_p, C.c_longlong, _i, _i, _i, _i, _d, _d, _d, _p, _p]),
    ("pfast_server_put_survey3d", _i, [_p, C.c_longlong, _i, _i, _i, _d, _d, _d, _i, _p, _p, _p, _p, _p]),
    ("pfast_server_put_survey2d", _i, [_p, C.c_longlong, _i, _i, _d, _d, _i, _p, _p, _i, _p, _p, _p, _i, _p, _p]),
    ("pfast_server_drop", _i, [_p, _i, C.c_longlong]),
    ("pfast_server_submit", _i, [_p, _p, _p]),
    ("pfast_server_wait", _i, [_p, C.c_longlong, _p]),
    ("pfast_server_stats_get", _i, [_p, _p]),
]
PFAST_NOALLOC_MAX_NODES = 1048576

_lib = None


def lib():
    """The loaded library (raises if it was never built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"pfast_gb300 CUDA library missing at {LIB_PATH}: build it with "
                              "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class PfastError(RuntimeError):
    def __init__(self, status, where=""):
        L = lib()
        msg = L.pfast_last_error().decode(errors="replace")
        name = L.pfast_status_string(status).decode(errors="replace")
        super().__init__(f"{where}: {name} (status {status}): {msg}")
        self.status = status


def check(status, where=""):
    if status != PFAST_OK:
        raise PfastError(status, where)
