"""ctypes binding of libnlfem_gpu.so (the C ABI declared in include/nlfem_gpu.h).

There is no CPU fallback: if the shared library is missing or no CUDA device is visible, every
compute call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnlfem_gpu.so")

NLFEM_OK = 0
NLFEM_PREC_FP64 = 0
NLFEM_PREC_MIXED = 1
NLFEM_PREC_FP64_ONESIDED = 2
ERRORS = {1: "invalid input", 2: "CUDA error", 3: "out of memory", 4: "unsupported option",
          5: "degenerate element", 6: "device wait timed out"}

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)
_ip = ctypes.POINTER(ctypes.c_int)


class Problem(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("outdim", ctypes.c_int), ("is_dg", ctypes.c_int),
        ("nE", ctypes.c_long), ("nV", ctypes.c_long),
        ("elements", _lp), ("elementLabels", _lp), ("vertices", _dp), ("vertexLabels", _lp),
        ("Px", _dp), ("nPx", ctypes.c_int), ("dx", _dp),
        ("Py", _dp), ("nPy", ctypes.c_int), ("dy", _dp),
        ("Pg", _dp), ("tensorGaussDegree", ctypes.c_int), ("dg", _dp),
        ("sqdelta", ctypes.c_double), ("fractional_s", ctypes.c_double),
        ("kernel", ctypes.c_char_p), ("forcing", ctypes.c_char_p),
        ("method_remote", ctypes.c_char_p), ("method_close", ctypes.c_char_p),
        ("is_PlacePointOnCap", ctypes.c_int), ("is_fullConnectedComponentSearch", ctypes.c_int),
        ("precision", ctypes.c_int), ("verbose", ctypes.c_int),
        ("zeta_indices", _lp), ("zeta_indptr", _lp), ("nZeta", ctypes.c_long),
    ]


class CSR(ctypes.Structure):
    _fields_ = [("K", ctypes.c_long), ("nnz", ctypes.c_long), ("indptr", _lp),
                ("indices", _lp), ("values", _dp)]


class CSR32(ctypes.Structure):
    _fields_ = [("K", ctypes.c_long), ("nnz", ctypes.c_long), ("indptr", _ip),
                ("indices", _ip), ("values", _dp)]


class Tuning(ctypes.Structure):
    _fields_ = [("bfs_blocks_per_sm", ctypes.c_int), ("pass_blocks_per_sm", ctypes.c_int),
                ("bfs_candidates", ctypes.c_int), ("pass_candidates", ctypes.c_int),
                ("bfs_ms", ctypes.c_double * 8), ("pass_ms", ctypes.c_double * 8)]


class Stats(ctypes.Structure):
    _fields_ = [("n_pairs", ctypes.c_long), ("n_candidates", ctypes.c_long),
                ("n_close", ctypes.c_long), ("nnz_structural", ctypes.c_long),
                ("n_subtri", ctypes.c_long), ("n_ambiguous", ctypes.c_long),
                ("ms_total", ctypes.c_double), ("ms_bfs", ctypes.c_double),
                ("ms_pattern", ctypes.c_double), ("ms_quad", ctypes.c_double),
                ("ms_finish", ctypes.c_double), ("n_launches", ctypes.c_long),
                ("n_items_in", ctypes.c_long), ("n_items_cut", ctypes.c_long),
                ("slot_map", ctypes.c_long), ("dev_bytes", ctypes.c_long)]


class NlfemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nlfem_gpu: {ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


_lib = None


def load():
    """Load (building it if needed) the GPU library; raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) or os.environ.get("NLFEM_GPU_REBUILD"):
        from . import build
        build.build()
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libnlfem_gpu.so missing at {LIB_PATH}; run nlfem_gb300.build.build()")
    l = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER(Problem)
    l.nlfem_last_error.restype = ctypes.c_char_p
    l.nlfem_device_count.restype = ctypes.c_int
    l.nlfem_get_stats.argtypes = [ctypes.POINTER(Stats)]
    l.nlfem_stiffness_matrix.argtypes = [P, ctypes.POINTER(CSR)]
    l.nlfem_load_vector.argtypes = [P, _dp]
    l.nlfem_stiffness_batch.argtypes = [P, ctypes.c_int, ctypes.POINTER(CSR)]
    l.nlfem_csr_free.argtypes = [ctypes.POINTER(CSR)]
    l.nlfem_csr_free.restype = None
    l.nlfem_session_create.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    l.nlfem_session_assemble.argtypes = [ctypes.c_void_p]
    l.nlfem_session_assemble_graph.argtypes = [ctypes.c_void_p]
    l.nlfem_session_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Tuning)]
    l.nlfem_session_download.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(CSR)]
    l.nlfem_session_set_search_epoch.argtypes = [ctypes.c_void_p, ctypes.c_uint]
    l.nlfem_session_destroy.argtypes = [ctypes.c_void_p]
    l.nlfem_session_destroy.restype = None
    l.nlfem_pair_list.argtypes = [P, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(_lp)]
    l.nlfem_pair_blocks.argtypes = [P, ctypes.c_long, _lp, ctypes.c_int, _dp, _ip]
    l.nlfem_method_retriangulate.argtypes = [_dp, _dp, ctypes.c_double, _dp, ctypes.c_int]
    l.nlfem_retriangulate_batch.argtypes = [ctypes.c_long, _dp, _dp, ctypes.c_double, ctypes.c_int, _ip, _dp]
    l.nlfem_retriangulate_certified_batch.argtypes = [ctypes.c_long, _dp, _dp, ctypes.c_double, ctypes.c_int, _ip, _ip, _dp]
    l.nlfem_toRef.argtypes = [_dp, _dp, _dp]
    l.nlfem_toPhys.argtypes = [_dp, _dp, ctypes.c_int, _dp]
    l.nlfem_solve2x2.argtypes = [_dp, _dp, _dp]
    l.nlfem_measure_peaks.argtypes = [_dp, _dp]
    C32 = ctypes.POINTER(CSR32)
    l.nlfem_stiffness_matrix32.argtypes = [P, C32]
    l.nlfem_stiffness_batch32.argtypes = [P, ctypes.c_int, C32]
    l.nlfem_csr32_free.argtypes = [C32]
    l.nlfem_csr32_free.restype = None
    l.nlfem_session_download32.argtypes = [ctypes.c_void_p, ctypes.c_int, C32]
    l.nlfem_cache_release.argtypes = []
    l.nlfem_cache_release.restype = None
    l.nlfem_session_solve.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_int, _dp,
                                      ctypes.POINTER(ctypes.c_int)]
    l.nlfem_evaluate_mass.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_long,
                                      ctypes.c_long, _lp, _lp, _dp, _lp, ctypes.c_int, _dp, _dp, _dp, _dp]
    vp = ctypes.c_void_p   # device pointers and the stream are passed as raw addresses
    l.nlfem_load_vector_noalloc.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_long, vp, vp, vp, vp,
                                            _dp, ctypes.c_int, _dp, ctypes.c_char_p, vp, vp]
    _lib = l
    return l


def check(code):
    if code != NLFEM_OK:
        raise NlfemError(code, load().nlfem_last_error().decode(errors="replace"))


def stats():
    s = Stats()
    load().nlfem_get_stats(ctypes.byref(s))
    return {k: getattr(s, k) for k, _ in Stats._fields_}


# Symbols declared in include/nlfem_gpu.h (checked by the CPU test suite).
EXPORTED = [
    "nlfem_last_error", "nlfem_device_count", "nlfem_get_stats", "nlfem_stiffness_matrix",
    "nlfem_load_vector", "nlfem_stiffness_batch", "nlfem_csr_free", "nlfem_session_create",
    "nlfem_session_assemble", "nlfem_session_assemble_graph", "nlfem_session_autotune", "nlfem_session_download",
    "nlfem_session_destroy", "nlfem_session_set_search_epoch",
    "nlfem_pair_list", "nlfem_pair_blocks", "nlfem_method_retriangulate",
    "nlfem_retriangulate_batch", "nlfem_retriangulate_certified_batch", "nlfem_toRef", "nlfem_toPhys", "nlfem_solve2x2",
    "nlfem_par_assemble", "nlfem_load_vector_noalloc", "nlfem_measure_peaks",
    "nlfem_stiffness_matrix32", "nlfem_stiffness_batch32", "nlfem_csr32_free", "nlfem_session_download32",
    "nlfem_cache_release", "nlfem_evaluate_mass", "nlfem_session_solve",
]
