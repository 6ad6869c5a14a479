"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU restatement of the
reference engine (dmd_oracle.cpp).  It is the oracle the GB300 engine is
tested against and the timed CPU baseline; the product never imports it."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300"))
from dmdgb import abi  # noqa: E402
from dmdgb.params import default_tables  # noqa: E402

LIB_PATH = os.path.join(HERE, "_build", "libdmd_oracle.so")
_lib = None


def build() -> str:
    r = subprocess.run(["make", "-C", HERE], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.ora_create.restype = C.c_void_p
        L.ora_create.argtypes = [C.POINTER(abi.RunCfg), C.POINTER(abi.Tables), C.POINTER(abi.System), C.c_char_p, C.c_int]
        L.ora_run.restype = C.c_int64
        L.ora_run.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
        L.ora_predict_all.argtypes = [C.c_void_p, abi.dbl_p, abi.i32_p, abi.i32_p]
        L.ora_get_state.argtypes = [C.c_void_p] + [abi.dbl_p] * 6 + [abi.i32_p] * 3 + [abi.dbl_p, abi.dbl_p, abi.i64_p]
        L.ora_diagnostics.argtypes = [C.c_void_p, C.POINTER(abi.Diag)]
        L.ora_phipsi_sample.argtypes = [C.c_void_p, C.c_void_p]
        L.ora_get_evcode.argtypes = [C.c_void_p, abi.i8_p]
        L.ora_get_lists.argtypes = [C.c_void_p, abi.i32_p, abi.i32_p, abi.i32_p, abi.i32_p, C.c_int32]
        L.ora_get_scalars.argtypes = [C.c_void_p, abi.dbl_p, C.c_int]
        L.ora_n_outputs.argtypes = [C.c_void_p]
        L.ora_get_output.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.Diag)]
        L.ora_destroy.argtypes = [C.c_void_p]
        L.ora_destroy.restype = None
        L.ora_sidechain_grid.restype = C.c_int64
        L.ora_sidechain_grid.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_int64]
        L.ora_sidechain_search.restype = C.c_int64
        L.ora_sidechain_search.argtypes = [C.c_int32] + [C.c_void_p] * 5 + [C.POINTER(abi.Tables), C.c_double,
                                                                              C.c_double, C.c_int32, C.c_int32] + \
            [C.c_void_p] * 3
        _lib = L
    return _lib


def generate(spec, tables=None, min_sep: float = 5.0):
    """The seeded system generator (dmd_generate) from the oracle library's
    own copy, so that a CPU-only run never loads the engine library."""
    from dmdgb import systems
    L = lib()
    L.dmd_generate.argtypes = [C.POINTER(abi.GenSpec), C.POINTER(abi.Tables), C.c_int32] + [abi.dbl_p] * 6 + \
        [C.c_char_p, C.c_int32]
    L.dmd_generate.restype = C.c_int
    return systems.generate(spec, tables, min_sep, lib=L)


class Oracle:
    def __init__(self, spec, tables=None, flags: int = 0, list_cap: int = 0):
        self.L = lib()
        self.spec = spec
        self.n = spec.n_beads
        self._tables = abi.tables_struct(tables or default_tables())
        self._cfg = spec.run_cfg(flags, list_cap)
        self._sys = spec.c_system()
        err = C.create_string_buffer(512)
        self.h = self.L.ora_create(C.byref(self._cfg), C.byref(self._tables), C.byref(self._sys), err, 512)
        if not self.h:
            raise RuntimeError("oracle create failed: " + err.value.decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def run(self, n_events: int, log_capacity: int = 0):
        if log_capacity > 0:
            buf = np.zeros(log_capacity, abi.EVENT_DTYPE)
            n = self.L.ora_run(self.h, int(n_events), buf.ctypes.data, log_capacity)
            if n < 0:
                raise RuntimeError("oracle run failed")
            return buf[:min(n, log_capacity)]
        n = self.L.ora_run(self.h, int(n_events), None, 1)
        if n < 0:
            raise RuntimeError("oracle run failed")
        return n

    def predictions(self):
        tim = np.zeros(self.n)
        np_ = np.zeros(self.n, np.int32)
        ct = np.zeros(self.n, np.int32)
        self.L.ora_predict_all(self.h, abi.ptr(tim, abi.dbl_p), abi.ptr(np_, abi.i32_p), abi.ptr(ct, abi.i32_p))
        return tim, np_, ct

    def state(self) -> dict:
        n = self.n
        a = {k: np.zeros(n) for k in ("x", "y", "z", "vx", "vy", "vz")}
        bp = np.zeros(n, np.int32)
        ident = np.zeros(n, np.int32)
        er = np.zeros(4 * n, np.int32)
        t = C.c_double()
        tf = C.c_double()
        coll = C.c_int64()
        self.L.ora_get_state(self.h, *[abi.ptr(a[k], abi.dbl_p) for k in ("x", "y", "z", "vx", "vy", "vz")],
                             abi.ptr(bp, abi.i32_p), abi.ptr(ident, abi.i32_p), abi.ptr(er, abi.i32_p),
                             C.byref(t), C.byref(tf), C.byref(coll))
        a.update(bptnr=bp, identity=ident, extra_repuls=er.reshape(n, 4), t=t.value, tfalse=tf.value, coll=coll.value)
        return a

    def diagnostics(self) -> dict:
        d = abi.Diag()
        self.L.ora_diagnostics(self.h, C.byref(d))
        return d.as_dict()

    def phipsi_sample(self, hist: np.ndarray):
        """Adds the current backbone (phi, psi) bins (code/phipsi.f) to hist (361 x 361 int64)."""
        assert hist.dtype == np.int64 and hist.size == 361 * 361 and hist.flags.c_contiguous
        self.L.ora_phipsi_sample(self.h, hist.ctypes.data)

    def evcode(self) -> np.ndarray:
        out = np.zeros((self.n, self.n), np.int8)
        self.L.ora_get_evcode(self.h, out.ctypes.data_as(abi.i8_p))
        return out

    def lists(self, cap: int = 256):
        n = self.n
        uc = np.zeros(n, np.int32)
        dc = np.zeros(n, np.int32)
        up = np.zeros(n * cap, np.int32)
        dn = np.zeros(n * cap, np.int32)
        self.L.ora_get_lists(self.h, abi.ptr(uc, abi.i32_p), abi.ptr(up, abi.i32_p), abi.ptr(dc, abi.i32_p),
                             abi.ptr(dn, abi.i32_p), cap)
        return uc, up.reshape(n, cap), dc, dn.reshape(n, cap)

    def scalars(self) -> dict:
        out = np.zeros(16)
        self.L.ora_get_scalars(self.h, abi.ptr(out, abi.dbl_p), 16)
        keys = ["interval", "interval_max", "sig_max_all", "hdelr", "num_cell", "width", "rlsq1", "rlsq15",
                "rlsq16", "rlsq40", "n_forced", "t_fact", "evp1_15", "tim_ghost", "tim_interval", "tim_output"]
        return dict(zip(keys, out.tolist()))

    def outputs(self):
        out = []
        for k in range(self.L.ora_n_outputs(self.h)):
            d = abi.Diag()
            self.L.ora_get_output(self.h, k, C.byref(d))
            out.append(d.as_dict())
        return out


def sidechain_grid(move: float, step: float) -> np.ndarray:
    """The offsets of one axis of genconfig's search grid (a Fortran DO loop
    over a real variable: repeated addition)."""
    m = lib().ora_sidechain_grid(float(move), float(step), None, 0)
    out = np.zeros(max(m, 0))
    lib().ora_sidechain_grid(float(move), float(step), out.ctypes.data, len(out))
    return out


def sidechain_search(ca, nh, co, side, residues, move: float = 3.5, step: float = 0.005, tables=None, only=None):
    """genconfig's side-chain placement search on the CPU (positions [n, 3]
    in angstrom): (moved side chains, r3 minima, winning grid indices).
    only=(r0, r1) searches residues r0..r1-1 and copies the others."""
    ca, nh, co, side = [np.ascontiguousarray(a, np.float64).reshape(-1, 3) for a in (ca, nh, co, side)]
    res = np.ascontiguousarray(residues, np.int32)
    n = len(res)
    r0, r1 = only if only is not None else (0, n)
    t = abi.tables_struct(tables or default_tables())
    out = np.zeros((n, 3))
    rmin = np.zeros(n)
    idx = np.zeros(n, np.int64)
    m = lib().ora_sidechain_search(n, ca.ctypes.data, nh.ctypes.data, co.ctypes.data, side.ctypes.data, res.ctypes.data,
                                   C.byref(t), float(move), float(step), int(r0), int(r1), out.ctypes.data,
                                   rmin.ctypes.data, idx.ctypes.data)
    if m < 0:
        raise ValueError("bad side-chain search input")
    return out, rmin, idx
