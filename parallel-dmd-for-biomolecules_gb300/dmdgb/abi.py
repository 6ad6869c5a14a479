"""ctypes mirror of include/dmd.h and loaders for the in-tree shared objects.

The engine library (libdmd_gb300.so, built by build.py from csrc/) is the
product.  ``load_engine`` fails loudly when it is missing; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_DIR = os.path.dirname(PKG_DIR)
# DMD_CHECKED=1 selects the checked build (device index checks, build.py)
ENGINE_SO = os.path.join(PKG_DIR, "_build_checked" if os.environ.get("DMD_CHECKED", "") == "1" else "_build",
                         "libdmd_gb300.so")

DMD_OK = 0
ERRORS = {
    -1: "DMD_E_INPUT", -2: "DMD_E_OVERLAP", -3: "DMD_E_NEG_TIME", -4: "DMD_E_DEVICE_TIMEOUT",
    -5: "DMD_E_OOM", -6: "DMD_E_CUDA", -7: "DMD_E_CAPACITY", -8: "DMD_E_STATE",
}
FLAG_STOP_AT_OUTPUT = 1
FLAG_COUNT_PHYSICAL = 2
FLAG_SERIAL = 4
FLAG_ALLOW_OVERLAP = 8
FLAG_CHECK_OVERLAP = 16
FLAG_TIGHT_LOOP_BOUND = 32
EV_GHOST, EV_INTERVAL, EV_REBUILD, EV_OUTPUT = 100, 101, 102, 103

dbl_p = C.POINTER(C.c_double)
i32_p = C.POINTER(C.c_int32)
i64_p = C.POINTER(C.c_int64)
i8_p = C.POINTER(C.c_int8)


class Tables(C.Structure):
    _fields_ = [
        ("sigma", C.c_double * 4), ("welldia", C.c_double * 4), ("epsilon", C.c_double * 4),
        ("mass", C.c_double * 29),
        ("bds", (C.c_double * 20) * 20), ("wel", (C.c_double * 20) * 20), ("ep", (C.c_double * 20) * 20),
        ("rca", C.c_double * 20), ("rnh", C.c_double * 20), ("rco", C.c_double * 20),
        ("del_rca", C.c_double * 20), ("del_rnh", C.c_double * 20), ("del_rco", C.c_double * 20),
        ("sqz", (C.c_double * 5) * 20),
    ]


class RunCfg(C.Structure):
    _fields_ = [
        ("tstar", C.c_double), ("seed", C.c_uint64), ("canon", C.c_int32), ("hbonds", C.c_int32),
        ("numbin", C.c_int32), ("n_wrap", C.c_int32), ("rl_const", C.c_double), ("t_fact", C.c_double),
        ("n_forced", C.c_double), ("list_cap", C.c_int32), ("flags", C.c_int32),
        ("chaptype", C.c_int32), ("species2_chain", C.c_int32),
    ]


class System(C.Structure):
    """dmd_system; the array fields hold addresses (int32 or float64 data as
    the header declares them) so that filling one is cheap."""
    _fields_ = [
        ("n_beads", C.c_int32), ("n_chains", C.c_int32), ("chain_len", C.c_void_p), ("residues", C.c_void_p),
        ("hp", C.c_void_p), ("boxl", C.c_double),
        ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p), ("vx", C.c_void_p), ("vy", C.c_void_p),
        ("vz", C.c_void_p), ("bptnr", C.c_void_p), ("t0", C.c_double), ("coll0", C.c_int64),
    ]


class Event(C.Structure):
    _fields_ = [("coll", C.c_int64), ("t", C.c_double), ("tfalse", C.c_double), ("i", C.c_int32),
                ("j", C.c_int32), ("type", C.c_int32), ("evcode", C.c_int32)]


EVENT_DTYPE = np.dtype([("coll", "<i8"), ("t", "<f8"), ("tfalse", "<f8"), ("i", "<i4"), ("j", "<i4"),
                        ("type", "<i4"), ("evcode", "<i4")])
assert EVENT_DTYPE.itemsize == C.sizeof(Event)


class EventLog(C.Structure):
    _fields_ = [("events", C.POINTER(Event)), ("capacity", C.c_int64), ("count", C.c_int64)]


class Diag(C.Structure):
    _fields_ = [
        ("e_total", C.c_double), ("temperature", C.c_double), ("rg", C.c_double), ("e2e", C.c_double),
        ("ehh_ii", C.c_double), ("ehh_ij", C.c_double), ("e_kin", C.c_double),
        ("hb_alpha", C.c_int32), ("hb_ii", C.c_int32), ("hb_ij", C.c_int32), ("max_down", C.c_int32),
        ("nevents", C.c_int64 * 32),
        ("coll", C.c_int64), ("n_pair", C.c_int64), ("n_ghost", C.c_int64), ("n_interval", C.c_int64),
        ("n_output", C.c_int64), ("n_updates", C.c_int64), ("n_forced_updates", C.c_int64),
        ("t", C.c_double), ("tfalse", C.c_double), ("nbr_mean", C.c_double),
        ("n_batches", C.c_int64), ("n_rolled_back", C.c_int64), ("n_candidates", C.c_int64),
        ("nc_boundbad", C.c_int64), ("nc_unboundbad", C.c_int64), ("run_cycles", C.c_int64),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("nevents",)}
        d["nevents"] = list(self.nevents)
        return d


class GenSpec(C.Structure):
    _fields_ = [("n_chains", C.c_int32), ("chain_len", i32_p), ("residues", i32_p), ("boxl", C.c_double),
                ("tstar", C.c_double), ("seed", C.c_uint64), ("min_sep", C.c_double)]


# the symbols include/dmd.h declares
ENGINE_SYMBOLS = [
    "dmd_create", "dmd_run", "dmd_predict_all", "dmd_get_state", "dmd_set_state", "dmd_diagnostics", "dmd_get_evcode",
    "dmd_destroy", "dmd_last_error", "dmd_debug_bounds", "dmd_version", "dmd_batch_create", "dmd_batch_run",
    "dmd_batch_get_state", "dmd_batch_diagnostics", "dmd_batch_destroy", "dmd_batch_last_error",
    "dmd_generate", "dmd_static_evcode", "dmd_inspect", "dmd_last_run_ms", "dmd_batch_last_run_ms", "dmd_predict_all_noalloc",
    "dmd_batch_set_cluster", "dmd_set_cluster", "dmd_batch_cluster", "dmd_batch_set_cell_div",
    "dmd_batch_set_compact_limit", "dmd_set_compact_limit",
    "dmd_batch_run_graph", "dmd_batch_run_cycles", "dmd_batch_autotune", "dmd_batch_autotune_cached", "dmd_batch_device_bytes", "dmd_batch_upload_bytes", "dmd_batch_readback_bytes", "dmd_state_bytes", "dmd_save_state", "dmd_load_state",
    "dmd_server_create", "dmd_server_submit", "dmd_server_step", "dmd_server_status", "dmd_server_result",
    "dmd_server_release", "dmd_server_stats", "dmd_server_last_error", "dmd_server_destroy",
    "dmd_sidechain_search", "dmd_sidechain_grid",
    "dmd_phipsi_sample", "dmd_phipsi_histogram", "dmd_batch_phipsi_sample", "dmd_batch_phipsi_histogram",
]

REQ_QUEUED, REQ_ACTIVE, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


def tables_struct(t) -> Tables:
    s = Tables()
    for name, _ in Tables._fields_:
        arr = np.ascontiguousarray(np.asarray(getattr(t, name), dtype=np.float64))
        C.memmove(C.addressof(getattr(s, name)), arr.ctypes.data, arr.nbytes)
    return s


def ptr(a, typ):
    return a.ctypes.data_as(typ) if a is not None else None


def _declare(lib) -> None:
    lib.dmd_create.argtypes = [C.POINTER(RunCfg), C.POINTER(Tables), C.POINTER(System), C.POINTER(C.c_void_p)]
    lib.dmd_create.restype = C.c_int
    lib.dmd_debug_bounds.argtypes = [C.POINTER(C.c_longlong)]
    lib.dmd_debug_bounds.restype = C.c_int
    lib.dmd_run.argtypes = [C.c_void_p, C.c_int64, C.POINTER(EventLog)]
    lib.dmd_run.restype = C.c_int
    lib.dmd_predict_all.argtypes = [C.c_void_p, dbl_p, i32_p, i32_p]
    lib.dmd_predict_all.restype = C.c_int
    lib.dmd_get_state.argtypes = [C.c_void_p] + [C.c_void_p] * 9 + [dbl_p, dbl_p, i64_p]
    lib.dmd_set_state.argtypes = [C.c_void_p] + [C.c_void_p] * 7 + [C.c_double, C.c_int64]
    lib.dmd_set_state.restype = C.c_int
    lib.dmd_sidechain_search.argtypes = [C.c_int32] + [C.c_void_p] * 5 + [C.POINTER(Tables), C.c_double, C.c_double] + \
        [C.c_void_p] * 3 + [C.c_char_p, C.c_int32]
    lib.dmd_sidechain_search.restype = C.c_int
    lib.dmd_sidechain_grid.argtypes = [C.c_double, C.c_double]
    lib.dmd_sidechain_grid.restype = C.c_int64
    lib.dmd_get_state.restype = C.c_int
    lib.dmd_diagnostics.argtypes = [C.c_void_p, C.POINTER(Diag)]
    lib.dmd_diagnostics.restype = C.c_int
    lib.dmd_get_evcode.argtypes = [C.c_void_p, i8_p]
    lib.dmd_get_evcode.restype = C.c_int
    lib.dmd_destroy.argtypes = [C.c_void_p]
    lib.dmd_destroy.restype = None
    lib.dmd_last_error.argtypes = [C.c_void_p]
    lib.dmd_last_error.restype = C.c_char_p
    lib.dmd_version.argtypes = []
    lib.dmd_version.restype = C.c_char_p
    lib.dmd_batch_create.argtypes = [C.c_int32, C.POINTER(RunCfg), C.POINTER(Tables), C.POINTER(System),
                                     C.POINTER(C.c_void_p)]
    lib.dmd_batch_create.restype = C.c_int
    lib.dmd_batch_run.argtypes = [C.c_void_p, C.c_int64, C.POINTER(EventLog)]
    lib.dmd_batch_run.restype = C.c_int
    lib.dmd_batch_get_state.argtypes = [C.c_void_p, C.c_int32] + [C.c_void_p] * 9 + [dbl_p, dbl_p, i64_p]
    lib.dmd_batch_get_state.restype = C.c_int
    lib.dmd_batch_diagnostics.argtypes = [C.c_void_p, C.c_int32, C.POINTER(Diag)]
    lib.dmd_batch_diagnostics.restype = C.c_int
    lib.dmd_batch_destroy.argtypes = [C.c_void_p]
    lib.dmd_batch_destroy.restype = None
    lib.dmd_batch_last_error.argtypes = [C.c_void_p]
    lib.dmd_batch_last_error.restype = C.c_char_p
    lib.dmd_generate.argtypes = [C.POINTER(GenSpec), C.POINTER(Tables), C.c_int32] + [dbl_p] * 6 + [C.c_char_p, C.c_int32]
    lib.dmd_generate.restype = C.c_int
    lib.dmd_last_run_ms.argtypes = [C.c_void_p]
    lib.dmd_last_run_ms.restype = C.c_double
    lib.dmd_batch_last_run_ms.argtypes = [C.c_void_p]
    lib.dmd_batch_last_run_ms.restype = C.c_double
    lib.dmd_batch_set_cluster.argtypes = [C.c_void_p, C.c_int32]
    lib.dmd_batch_set_cluster.restype = C.c_int
    lib.dmd_set_cluster.argtypes = [C.c_void_p, C.c_int32]
    lib.dmd_set_cluster.restype = C.c_int
    lib.dmd_batch_cluster.argtypes = [C.c_void_p]
    lib.dmd_batch_cluster.restype = C.c_int32
    lib.dmd_batch_set_cell_div.argtypes = [C.c_void_p, C.c_int32]
    lib.dmd_batch_set_cell_div.restype = C.c_int
    for fn in ("dmd_batch_set_compact_limit", "dmd_set_compact_limit"):
        getattr(lib, fn).argtypes = [C.c_void_p, C.c_int32]
        getattr(lib, fn).restype = C.c_int
    lib.dmd_batch_device_bytes.argtypes = [C.c_void_p]
    lib.dmd_batch_device_bytes.restype = C.c_int64
    lib.dmd_batch_upload_bytes.argtypes = [C.c_void_p]
    lib.dmd_batch_upload_bytes.restype = C.c_int64
    lib.dmd_batch_readback_bytes.argtypes = [C.c_void_p]
    lib.dmd_batch_readback_bytes.restype = C.c_int64
    lib.dmd_batch_run_graph.argtypes = [C.c_void_p, C.c_int64, C.c_int32]
    lib.dmd_batch_run_graph.restype = C.c_int
    lib.dmd_batch_run_cycles.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_int64)]
    lib.dmd_batch_run_cycles.restype = C.c_int
    lib.dmd_phipsi_sample.argtypes = [C.c_void_p]
    lib.dmd_phipsi_sample.restype = C.c_int
    lib.dmd_phipsi_histogram.argtypes = [C.c_void_p, i64_p, i64_p, C.c_int32]
    lib.dmd_phipsi_histogram.restype = C.c_int
    lib.dmd_batch_phipsi_sample.argtypes = [C.c_void_p, C.c_int32]
    lib.dmd_batch_phipsi_sample.restype = C.c_int
    lib.dmd_batch_phipsi_histogram.argtypes = [C.c_void_p, C.c_int32, i64_p, i64_p, C.c_int32]
    lib.dmd_batch_phipsi_histogram.restype = C.c_int
    lib.dmd_batch_autotune.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dbl_p]
    lib.dmd_batch_autotune.restype = C.c_int
    lib.dmd_batch_autotune_cached.argtypes = [C.c_void_p, C.c_int64, C.c_char_p, C.POINTER(C.c_int32),
                                              C.POINTER(C.c_int32), dbl_p, C.POINTER(C.c_int32)]
    lib.dmd_batch_autotune_cached.restype = C.c_int
    lib.dmd_predict_all_noalloc.argtypes = [C.POINTER(RunCfg), C.POINTER(Tables), C.POINTER(System),
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int32]
    lib.dmd_predict_all_noalloc.restype = C.c_int
    lib.dmd_static_evcode.argtypes = [C.POINTER(RunCfg), C.POINTER(Tables), C.POINTER(System), i8_p, C.c_char_p, C.c_int32]
    lib.dmd_static_evcode.restype = C.c_int
    lib.dmd_inspect.argtypes = [C.POINTER(RunCfg), C.POINTER(Tables), C.POINTER(System), dbl_p, C.c_int32, C.c_char_p, C.c_int32]
    lib.dmd_inspect.restype = C.c_int
    lib.dmd_state_bytes.argtypes = [C.c_void_p]
    lib.dmd_state_bytes.restype = C.c_int64
    lib.dmd_save_state.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    lib.dmd_save_state.restype = C.c_int
    lib.dmd_load_state.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    lib.dmd_load_state.restype = C.c_int
    lib.dmd_server_create.argtypes = [C.c_int32, C.c_int64, C.c_int64, C.POINTER(C.c_void_p)]
    lib.dmd_server_create.restype = C.c_int
    lib.dmd_server_submit.argtypes = [C.c_void_p, C.POINTER(RunCfg), C.POINTER(Tables), C.POINTER(System), C.c_int64,
                                      i64_p]
    lib.dmd_server_submit.restype = C.c_int
    lib.dmd_server_step.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    lib.dmd_server_step.restype = C.c_int
    lib.dmd_server_status.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_int32), i64_p, dbl_p, dbl_p, dbl_p]
    lib.dmd_server_status.restype = C.c_int
    lib.dmd_server_result.argtypes = [C.c_void_p, C.c_int64, C.POINTER(Diag)] + [dbl_p] * 6 + [i32_p] * 2 + [dbl_p, dbl_p, i64_p]
    lib.dmd_server_result.restype = C.c_int
    lib.dmd_server_release.argtypes = [C.c_void_p, C.c_int64]
    lib.dmd_server_release.restype = C.c_int
    lib.dmd_server_stats.argtypes = [C.c_void_p, i64_p, i64_p, dbl_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), i64_p, i64_p]
    lib.dmd_server_stats.restype = C.c_int
    lib.dmd_server_last_error.argtypes = [C.c_void_p]
    lib.dmd_server_last_error.restype = C.c_char_p
    lib.dmd_server_destroy.argtypes = [C.c_void_p]
    lib.dmd_server_destroy.restype = None


_engine = None


def load_engine(path: str = ENGINE_SO):
    """The GB300 engine library.  Raises if it has not been built."""
    global _engine
    if _engine is None:
        if not os.path.exists(path):
            raise RuntimeError(f"GB300 engine library missing: {path} (run __graft_entry__.build())")
        lib = C.CDLL(path)
        _declare(lib)
        _engine = lib
    return _engine
