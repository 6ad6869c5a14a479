"""Python host of the GB300 engine: the calls a driver makes in place of the
reference's program dmd main loop (code/main.F90:117-1258), through the C
ABI of include/dmd.h.  There is no CPU path: every method runs the CUDA
engine and raises if the library or the GPU is unavailable.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence

import numpy as np

from . import abi
from .params import Tables, default_tables
from .systems import SystemSpec


class DMDError(RuntimeError):
    def __init__(self, rc: int, msg: str):
        super().__init__(f"{abi.ERRORS.get(rc, rc)}: {msg}")
        self.rc = rc


def _check(rc: int, lib, handle, fn="dmd_last_error"):
    if rc != 0:
        msg = getattr(lib, fn)(handle)
        raise DMDError(rc, msg.decode() if msg else "")


def _state_buffers(n: int):
    """Output arrays of a state read (views of one float64 and one int32
    block) and the get_state arguments that point at them."""
    f = np.empty(6 * n, np.float64)
    i = np.empty(6 * n, np.int32)
    fa, ia = f.ctypes.data, i.ctypes.data
    sc = (C.c_double(), C.c_double(), C.c_int64())
    out = {k: f[q * n:(q + 1) * n] for q, k in enumerate(("x", "y", "z", "vx", "vy", "vz"))}
    out.update(bptnr=i[:n], identity=i[n:2 * n], extra_repuls=i[2 * n:].reshape(n, 4))
    args = [fa + 8 * n * q for q in range(6)] + [ia, ia + 4 * n, ia + 8 * n] + [C.byref(v) for v in sc]

    def fin(o):
        o.update(t=sc[0].value, tfalse=sc[1].value, coll=sc[2].value)
        return o
    return out, args, fin


class Engine:
    """One system on the GPU (the plain one-system-per-launch path)."""

    def __init__(self, spec: SystemSpec, tables: Optional[Tables] = None, flags: int = 0, list_cap: int = 0,
                 cluster: int = 0):
        self.lib = abi.load_engine()
        self.spec = spec
        self.n = spec.n_beads
        self._tables = abi.tables_struct(tables or default_tables())
        self._cfg = spec.run_cfg(flags, list_cap)
        self._sys = spec.c_system()
        h = C.c_void_p()
        rc = self.lib.dmd_create(C.byref(self._cfg), C.byref(self._tables), C.byref(self._sys), C.byref(h))
        self.h = h
        if rc != 0:
            msg = self.lib.dmd_last_error(h)
            self.lib.dmd_destroy(h)
            self.h = None
            raise DMDError(rc, msg.decode() if msg else "")
        if cluster:
            _check(self.lib.dmd_set_cluster(self.h, int(cluster)), self.lib, self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.dmd_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, n_events: int, log_capacity: int = 0) -> Optional[np.ndarray]:
        """Commit n_events events; returns the event log (structured array) if
        log_capacity > 0."""
        log = None
        if log_capacity > 0:
            buf = np.zeros(log_capacity, abi.EVENT_DTYPE)
            log = abi.EventLog(buf.ctypes.data_as(C.POINTER(abi.Event)), log_capacity, 0)
            rc = self.lib.dmd_run(self.h, int(n_events), C.byref(log))
            _check(rc, self.lib, self.h)
            return buf[:min(log.count, log_capacity)]
        rc = self.lib.dmd_run(self.h, int(n_events), None)
        _check(rc, self.lib, self.h)
        return None

    def set_compact_limit(self, max_down: int):
        """Longest down list (0..32) for which the compact event-loop variant
        runs (0: always the full one); results do not depend on it."""
        _check(self.lib.dmd_set_compact_limit(self.h, int(max_down)), self.lib, self.h)

    def save_state(self) -> bytes:
        """The whole engine state (resumes bit-identically with load_state)."""
        n = int(self.lib.dmd_state_bytes(self.h))
        if n < 0:
            _check(n, self.lib, self.h)
        buf = C.create_string_buffer(n)
        _check(self.lib.dmd_save_state(self.h, buf, n), self.lib, self.h)
        return buf.raw

    def load_state(self, blob: bytes):
        """Restore a state saved from an engine created from the same system."""
        buf = C.create_string_buffer(blob, len(blob))
        _check(self.lib.dmd_load_state(self.h, buf, len(blob)), self.lib, self.h)

    def predictions(self):
        tim = np.zeros(self.n)
        np_ = np.zeros(self.n, np.int32)
        ct = np.zeros(self.n, np.int32)
        _check(self.lib.dmd_predict_all(self.h, abi.ptr(tim, abi.dbl_p), abi.ptr(np_, abi.i32_p),
                                        abi.ptr(ct, abi.i32_p)), self.lib, self.h)
        return tim, np_, ct

    def state(self) -> dict:
        out, args, fin = _state_buffers(self.n)
        _check(self.lib.dmd_get_state(self.h, *args), self.lib, self.h)
        return fin(out)

    def set_state(self, x, y, z, vx, vy, vz, bptnr=None, t: float = 0.0, coll: int = 0):
        """Restart this system from the given state (positions in box units
        at time t, velocities, 1-based H-bond partners or None, collision
        count), as dmd_create from that state would; the previous state
        stays if the call fails."""
        cols = [np.ascontiguousarray(a, np.float64) for a in (x, y, z, vx, vy, vz)]
        if any(c.shape != (self.n,) for c in cols):
            raise ValueError(f"positions and velocities need {self.n} entries each")
        bp = None if bptnr is None else np.ascontiguousarray(bptnr, np.int32)
        if bp is not None and bp.shape != (self.n,):
            raise ValueError(f"bptnr needs {self.n} entries")
        _check(self.lib.dmd_set_state(self.h, *[c.ctypes.data for c in cols], None if bp is None else bp.ctypes.data,
                                      float(t), int(coll)), self.lib, self.h)

    def state_now(self) -> dict:
        """The state at the current time, in dmd_set_state's terms: positions
        advanced by vx * tfalse (code/config.f:15-24; dmd_set_state wraps
        them into the box), velocities, bptnr, t and coll."""
        s = self.state()
        out = {k: s[k] + s[v] * s["tfalse"] for k, v in (("x", "vx"), ("y", "vy"), ("z", "vz"))}
        out.update(vx=s["vx"], vy=s["vy"], vz=s["vz"], bptnr=s["bptnr"], t=s["t"], coll=s["coll"])
        return out

    def diagnostics(self) -> dict:
        d = abi.Diag()
        _check(self.lib.dmd_diagnostics(self.h, C.byref(d)), self.lib, self.h)
        return d.as_dict()

    def phipsi_sample(self):
        """Adds the current backbone (phi, psi) bins to the histogram (code/phipsi.f)."""
        _check(self.lib.dmd_phipsi_sample(self.h), self.lib, self.h)

    def phipsi_histogram(self, reset: bool = False):
        """(361 x 361 counts [phi + 180, psi + 180] in whole degrees, samples)."""
        hist = np.zeros((361, 361), np.int64)
        n = C.c_int64()
        _check(self.lib.dmd_phipsi_histogram(self.h, hist.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(n),
                                             int(bool(reset))), self.lib, self.h)
        return hist, n.value

    def evcode(self) -> np.ndarray:
        out = np.zeros((self.n, self.n), np.int8)
        _check(self.lib.dmd_get_evcode(self.h, out.ctypes.data_as(abi.i8_p)), self.lib, self.h)
        return out


class Batch:
    """Many independent systems advanced by one persistent launch."""

    def __init__(self, specs: Sequence[SystemSpec], tables: Optional[Tables] = None, flags: int = 0, list_cap: int = 0,
                 cluster: int = 0):
        self.lib = abi.load_engine()
        self.specs = list(specs)
        n = len(self.specs)
        self._tables = abi.tables_struct(tables or default_tables())
        self._cfgs = (abi.RunCfg * n)(*[s.run_cfg(flags, list_cap) for s in self.specs])
        self._syss = (abi.System * n)(*[s.c_system() for s in self.specs])
        h = C.c_void_p()
        rc = self.lib.dmd_batch_create(n, self._cfgs, C.byref(self._tables), self._syss, C.byref(h))
        self.h = h
        if rc != 0:
            msg = self.lib.dmd_batch_last_error(h)
            self.lib.dmd_batch_destroy(h)
            self.h = None
            raise DMDError(rc, msg.decode() if msg else "")
        if cluster:
            self.set_cluster(cluster)

    def set_cluster(self, ctas: int):
        """CTAs per system (1, 2, 4, 8; 0 = automatic).  Results do not depend on it."""
        _check(self.lib.dmd_batch_set_cluster(self.h, int(ctas)), self.lib, self.h, "dmd_batch_last_error")

    @property
    def cluster(self) -> int:
        """The cluster size the last run used."""
        return int(self.lib.dmd_batch_cluster(self.h))

    def set_cell_div(self, div: int):
        """Coarser rebuild grid (finest cells per side / div); results do not depend on it."""
        _check(self.lib.dmd_batch_set_cell_div(self.h, int(div)), self.lib, self.h, "dmd_batch_last_error")

    def set_compact_limit(self, max_down: int):
        """Longest down list (0..32) for which the compact event-loop variant
        runs (0: always the full one); results do not depend on it."""
        _check(self.lib.dmd_batch_set_compact_limit(self.h, int(max_down)), self.lib, self.h, "dmd_batch_last_error")

    def run_graph(self, n_events: int, n_launches: int):
        """n_launches launches of n_events each, replayed from a captured CUDA graph."""
        _check(self.lib.dmd_batch_run_graph(self.h, int(n_events), int(n_launches)), self.lib, self.h,
               "dmd_batch_last_error")

    def run_cycles(self, n_events: int, launches_per_graph: int = 8) -> int:
        """n_events per system as rebuild cycles (one neighbour-list rebuild
        per launch) replayed from a captured CUDA graph; returns the launches."""
        k = C.c_int64()
        _check(self.lib.dmd_batch_run_cycles(self.h, int(n_events), int(launches_per_graph), C.byref(k)), self.lib,
               self.h, "dmd_batch_last_error")
        return int(k.value)

    def autotune(self, trial_events: int = 5000, cache: str = None) -> dict:
        """Pick the cluster size and rebuild grid by timing trial runs on a copy;
        with cache (a JSON file path) a stored choice for the same shapes and
        device is taken without trials, and a new one is stored."""
        c, d = C.c_int32(), C.c_int32()
        ms = C.c_double()
        if cache is None:
            _check(self.lib.dmd_batch_autotune(self.h, int(trial_events), C.byref(c), C.byref(d), C.byref(ms)),
                   self.lib, self.h, "dmd_batch_last_error")
            return {"cluster": c.value, "cell_div": d.value, "trial_ms": ms.value}
        hit = C.c_int32()
        _check(self.lib.dmd_batch_autotune_cached(self.h, int(trial_events), os.fsencode(cache), C.byref(c),
                                                  C.byref(d), C.byref(ms), C.byref(hit)),
               self.lib, self.h, "dmd_batch_last_error")
        return {"cluster": c.value, "cell_div": d.value, "trial_ms": ms.value, "cached": bool(hit.value)}

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def close(self):
        if getattr(self, "h", None):
            self.lib.dmd_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def run(self, n_events: int, log_capacity: int = 0) -> Optional[List[np.ndarray]]:
        n = len(self.specs)
        if log_capacity > 0:
            bufs = [np.zeros(log_capacity, abi.EVENT_DTYPE) for _ in range(n)]
            logs = (abi.EventLog * n)(*[abi.EventLog(b.ctypes.data_as(C.POINTER(abi.Event)), log_capacity, 0)
                                        for b in bufs])
            rc = self.lib.dmd_batch_run(self.h, int(n_events), logs)
            _check(rc, self.lib, self.h, "dmd_batch_last_error")
            return [b[:min(logs[r].count, log_capacity)] for r, b in enumerate(bufs)]
        rc = self.lib.dmd_batch_run(self.h, int(n_events), None)
        _check(rc, self.lib, self.h, "dmd_batch_last_error")
        return None

    def state(self, r: int) -> dict:
        if not 0 <= r < len(self.specs):
            raise DMDError(-1, "replica index out of range")
        out, args, fin = _state_buffers(self.specs[r].n_beads)
        _check(self.lib.dmd_batch_get_state(self.h, r, *args), self.lib, self.h, "dmd_batch_last_error")
        return fin(out)

    def diagnostics(self, r: int) -> dict:
        d = abi.Diag()
        _check(self.lib.dmd_batch_diagnostics(self.h, r, C.byref(d)), self.lib, self.h, "dmd_batch_last_error")
        return d.as_dict()

    def phipsi_sample(self, r: int = -1):
        """Adds the backbone (phi, psi) bins of system r (-1: every system)."""
        _check(self.lib.dmd_batch_phipsi_sample(self.h, int(r)), self.lib, self.h, "dmd_batch_last_error")

    def phipsi_histogram(self, r: int, reset: bool = False):
        """System r's (361 x 361 counts [phi + 180, psi + 180], samples)."""
        hist = np.zeros((361, 361), np.int64)
        n = C.c_int64()
        _check(self.lib.dmd_batch_phipsi_histogram(self.h, int(r), hist.ctypes.data_as(C.POINTER(C.c_int64)),
                                                   C.byref(n), int(bool(reset))), self.lib, self.h,
               "dmd_batch_last_error")
        return hist, n.value
