"""Serving: continuous batching of independent DMD simulation requests.

The scheduler is native (``dmd_server_*`` in include/dmd.h): requests are
set up on the submitting thread, admitted first in first out while launch
slots and the device-memory budget allow, and every ``step()`` advances all
running requests by up to ``chunk_events`` events in one launch while the
next admitted requests are uploaded on a second stream.  This module wraps
that API and adds the request-trace driver that measures completion
latency (p50/p99) and aggregate events/s.

There is no counterpart in the reference, which runs one system per MPI
job (``parallel-dmd-PRIME20/qfile/script.sh``).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import abi
from .engine import DMDError
from .params import Tables, default_tables
from .systems import SystemSpec


def _check(rc: int, lib, h):
    if rc != 0:
        msg = lib.dmd_server_last_error(h)
        raise DMDError(rc, msg.decode() if msg else "")


class Server:
    """A GPU serving loop: ``submit`` requests, call ``step`` until they are
    done, read ``result``.  Results do not depend on what else is running."""

    def __init__(self, max_slots: int = 152, hbm_budget: int = 0, chunk_events: int = 20000,
                 tables: Optional[Tables] = None):
        self.lib = abi.load_engine()
        self._tables = abi.tables_struct(tables or default_tables())
        h = C.c_void_p()
        rc = self.lib.dmd_server_create(int(max_slots), int(hbm_budget), int(chunk_events), C.byref(h))
        self.h = h
        if rc != 0:
            msg = self.lib.dmd_server_last_error(h)
            self.lib.dmd_server_destroy(h)
            self.h = None
            raise DMDError(rc, msg.decode() if msg else "")
        self._n: Dict[int, int] = {}
        self._keep: Dict[int, tuple] = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.dmd_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, spec: SystemSpec, n_events: int, flags: int = 0) -> int:
        cfg = spec.run_cfg(flags)
        sys_ = spec.c_system()
        rid = C.c_int64()
        _check(self.lib.dmd_server_submit(self.h, C.byref(cfg), C.byref(self._tables), C.byref(sys_),
                                          int(n_events), C.byref(rid)), self.lib, self.h)
        self._n[rid.value] = spec.n_beads
        return rid.value

    def step(self) -> Tuple[int, int]:
        na, nf = C.c_int32(), C.c_int32()
        _check(self.lib.dmd_server_step(self.h, C.byref(na), C.byref(nf)), self.lib, self.h)
        return na.value, nf.value

    def status(self, rid: int) -> dict:
        st, done = C.c_int32(), C.c_int64()
        ts, ta, tf = C.c_double(), C.c_double(), C.c_double()
        rc = self.lib.dmd_server_status(self.h, int(rid), C.byref(st), C.byref(done), C.byref(ts), C.byref(ta),
                                        C.byref(tf))
        if rc != 0 and st.value != abi.REQ_FAILED:
            _check(rc, self.lib, self.h)
        return {"state": st.value, "events_done": done.value, "t_submit": ts.value, "t_admit": ta.value,
                "t_finish": tf.value, "rc": rc}

    def result(self, rid: int) -> dict:
        n = self._n[rid]
        a = {k: np.zeros(n) for k in ("x", "y", "z", "vx", "vy", "vz")}
        bp = np.zeros(n, np.int32)
        ident = np.zeros(n, np.int32)
        d = abi.Diag()
        t, tf, coll = C.c_double(), C.c_double(), C.c_int64()
        _check(self.lib.dmd_server_result(self.h, int(rid), C.byref(d),
                                          *[abi.ptr(a[k], abi.dbl_p) for k in ("x", "y", "z", "vx", "vy", "vz")],
                                          abi.ptr(bp, abi.i32_p), abi.ptr(ident, abi.i32_p), C.byref(t), C.byref(tf),
                                          C.byref(coll)), self.lib, self.h)
        a.update(bptnr=bp, identity=ident, t=t.value, tfalse=tf.value, coll=coll.value, diag=d.as_dict())
        return a

    def release(self, rid: int):
        _check(self.lib.dmd_server_release(self.h, int(rid)), self.lib, self.h)
        self._n.pop(rid, None)

    def stats(self) -> dict:
        steps, ev = C.c_int64(), C.c_int64()
        ms = C.c_double()
        nw, na = C.c_int32(), C.c_int32()
        used, budget = C.c_int64(), C.c_int64()
        _check(self.lib.dmd_server_stats(self.h, C.byref(steps), C.byref(ev), C.byref(ms), C.byref(nw), C.byref(na),
                                         C.byref(used), C.byref(budget)), self.lib, self.h)
        return {"steps": steps.value, "events": ev.value, "kernel_ms": ms.value, "waiting": nw.value,
                "active": na.value, "bytes_used": used.value, "bytes_budget": budget.value}


# ------------------------------------------------------------- request traces
def poisson_arrivals(rate: float, duration: float, seed: int = 1) -> np.ndarray:
    """Arrival times (s) of a Poisson process of the given rate over
    [0, duration)."""
    rng = np.random.default_rng([seed, 77])
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            return np.asarray(out)
        out.append(t)


@dataclass
class TraceResult:
    latencies: List[float] = field(default_factory=list)   # completion - arrival, s
    events: int = 0
    wall: float = 0.0
    kernel_ms: float = 0.0
    steps: int = 0
    failed: int = 0
    max_active: int = 0
    # requests still in the server when a horizon stopped the trace
    unfinished_ages: List[float] = field(default_factory=list)   # horizon - arrival, s
    unfinished_events_done: int = 0
    unfinished_events_left: int = 0
    not_submitted: int = 0

    def summary(self) -> dict:
        lat = np.asarray(self.latencies) if self.latencies else np.zeros(1)
        out = {"requests": len(self.latencies), "failed": self.failed,
               "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
               "events": self.events, "wall_s": self.wall,
               "events_per_s": self.events / self.wall if self.wall > 0 else None,
               "kernel_s": self.kernel_ms / 1000.0, "steps": self.steps, "max_active": self.max_active}
        if self.unfinished_ages or self.not_submitted:
            cens = np.concatenate([np.asarray(self.latencies, float), np.asarray(self.unfinished_ages, float)])
            served = self.events + self.unfinished_events_done
            out.update({"backlog_requests": len(self.unfinished_ages),
                        "backlog_events": self.unfinished_events_left,
                        "events_served": served,
                        "served_events_per_s": served / self.wall if self.wall > 0 else None,
                        "p50_lower_bound_s": float(np.percentile(cens, 50)) if len(cens) else None,
                        "p99_lower_bound_s": float(np.percentile(cens, 99)) if len(cens) else None})
        return out


def serve_trace(server: Server, arrivals: Sequence[float], requests: Sequence[Tuple[SystemSpec, int]],
                horizon_s: Optional[float] = None) -> TraceResult:
    """Replay a trace in real time: request k (a generated system and its
    event count) is submitted when the wall clock passes arrivals[k], the
    server is stepped continuously, and each request's latency is its
    completion time minus its arrival time.  With horizon_s the replay
    stops at that wall-clock time and reports what is left (backlog)."""
    res = TraceResult()
    late: Dict[int, float] = {}     # request id -> submit delay after arrival, s
    live: Dict[int, int] = {}       # request id -> trace index
    t0 = time.monotonic()
    k_next = 0
    while k_next < len(arrivals) or live:
        now = time.monotonic() - t0
        if horizon_s is not None and now >= horizon_s:
            for rid, k in live.items():
                st = server.status(rid)
                res.unfinished_ages.append(now - float(arrivals[k]))
                res.unfinished_events_done += st["events_done"]
                res.unfinished_events_left += requests[k][1] - st["events_done"]
            for k in range(k_next, len(arrivals)):
                if arrivals[k] <= now:
                    res.unfinished_ages.append(now - float(arrivals[k]))
                    res.unfinished_events_left += requests[k][1]
            res.not_submitted = len(arrivals) - k_next
            break
        while k_next < len(arrivals) and arrivals[k_next] <= now:
            spec, nev = requests[k_next]
            rid = server.submit(spec, nev)
            late[rid] = (time.monotonic() - t0) - float(arrivals[k_next])
            live[rid] = k_next
            k_next += 1
        if not live:
            if k_next < len(arrivals):
                time.sleep(max(0.0, min(0.01, float(arrivals[k_next]) - (time.monotonic() - t0))))
            continue
        na, nf = server.step()
        res.max_active = max(res.max_active, na)
        for rid in list(live):
            st = server.status(rid)
            if st["state"] in (abi.REQ_DONE, abi.REQ_FAILED):
                res.latencies.append(st["t_finish"] - st["t_submit"] + late[rid])
                if st["state"] == abi.REQ_FAILED:
                    res.failed += 1
                res.events += st["events_done"]
                server.release(rid)
                del live[rid]
    res.wall = time.monotonic() - t0
    s = server.stats()
    res.kernel_ms = s["kernel_ms"]
    res.steps = s["steps"]
    return res
