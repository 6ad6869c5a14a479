"""The library's host code (capi.cu: set-up, pools, copies, launch
parameters, state read-back and replacement) on the CPU, linked against a
stand-in CUDA runtime (tests/host_mock/): device memory is host memory and
a launch checks what its kernel would be given instead of running it."""
import ctypes as C
import os
import shutil
import subprocess
import types

import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.params import default_tables
from helpers import dense_system

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
MOCK = os.path.join(HERE, "host_mock")
CSRC = os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300", "csrc")
OUT = os.path.join(MOCK, "_build")
LIB = os.path.join(OUT, "libdmd_hostmock.so")


def _build() -> str:
    srcs = [os.path.join(CSRC, "capi.cu"), os.path.join(CSRC, "generate.cpp"), os.path.join(MOCK, "mock_rt.cpp"),
            os.path.join(MOCK, "mock_engine.cu")]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(REPO, "include", "dmd.h")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in deps):
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I" + os.path.join(REPO, "include"), "-I" + CSRC]
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    objs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        if s.endswith(".cu"):
            cmd = [nvcc, "-O1", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off"] + inc + ["-c", s, "-o", o]
        else:
            cmd = ["g++", "-O1", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + cuda_inc] + inc + ["-c", s, "-o", o]
        subprocess.run(cmd, check=True, capture_output=True)
        objs.append(o)
    subprocess.run(["g++", "-shared", "-o", LIB + ".tmp"] + objs + ["-Wl,--no-undefined"], check=True,
                   capture_output=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class _Tolerant:
    """abi's declarations, skipping the entry points this library leaves out."""
    def __init__(self, lib):
        self._lib = lib

    def __getattr__(self, name):
        try:
            return getattr(self._lib, name)
        except AttributeError:
            return types.SimpleNamespace()


@pytest.fixture(scope="module")
def mock():
    lib = C.CDLL(_build())
    abi._declare(_Tolerant(lib))
    lib.mock_report.restype = C.c_char_p
    lib.mock_live_allocations.restype = C.c_size_t
    lib.mock_counts.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_longlong),
                                C.POINTER(C.c_int), C.POINTER(C.c_int)]
    return lib


def counts(lib):
    v = [C.c_int(), C.c_int(), C.c_int(), C.c_longlong(), C.c_int(), C.c_int()]
    lib.mock_counts(*[C.byref(x) for x in v])
    return [x.value for x in v]


def state_of(lib, h, r, n, batch=True):
    f = np.zeros((6, n))
    i = np.zeros((6, n), np.int32)
    t, tf, coll = C.c_double(), C.c_double(), C.c_int64()
    args = [f[k].ctypes.data for k in range(6)] + [i[0].ctypes.data, i[1].ctypes.data, i[2].ctypes.data]
    if batch:
        rc = lib.dmd_batch_get_state(h, r, *args, C.byref(t), C.byref(tf), C.byref(coll))
    else:
        rc = lib.dmd_get_state(h, *args, C.byref(t), C.byref(tf), C.byref(coll))
    assert rc == 0
    return f, i, t.value, coll.value


def test_layout_check_flags_an_overlap(mock):
    assert mock.mock_selftest() == 1


def test_batch_pools_launches_and_state(mock):
    """Five 32-replica-workload systems and three KLVFFAE systems in one
    batch: every launch's pools are laid out as the kernels index them, the
    chain tables are right, and the state read back is the input wrapped
    into the box with no H-bond."""
    specs = sorted(systems.config_c3(32, seed=1), key=lambda s: s.n_beads)[:4] + [systems.config_c3(32, seed=1)[31]]
    specs += [systems.klvffae_system(4, 5.0, 0.2 + 0.05 * r, seed=r + 1) for r in range(3)]
    for s in specs:
        systems.generate(s)
    n = len(specs)
    tabs = abi.tables_struct(default_tables())
    cfgs = (abi.RunCfg * n)(*[s.run_cfg(0, 0) for s in specs])
    syss = (abi.System * n)(*[s.c_system() for s in specs])
    mock.mock_reset()
    base = mock.mock_live_allocations()
    h = C.c_void_p()
    assert mock.dmd_batch_create(n, cfgs, C.byref(tabs), syss, C.byref(h)) == 0, mock.dmd_batch_last_error(h)
    cap = 64
    bufs = [np.zeros(cap, abi.EVENT_DTYPE) for _ in range(n)]
    logs = (abi.EventLog * n)(*[abi.EventLog(b.ctypes.data_as(C.POINTER(abi.Event)), cap, 0) for b in bufs])
    assert mock.dmd_batch_run(h, 1000, logs) == 0, mock.dmd_batch_last_error(h)
    d = abi.Diag()
    assert mock.dmd_batch_diagnostics(h, 2, C.byref(d)) == 0
    init, run, diag, target, C_, compact = counts(mock)
    assert (init, diag) == (1, 1) and run >= 1 and target == 1000
    assert mock.mock_report() == b"", mock.mock_report().decode()
    for r, s in enumerate(specs):
        f, i, t, coll = state_of(mock, h, r, s.n_beads)
        for k, a in enumerate((s.x, s.y, s.z)):
            assert np.array_equal(f[k], a - np.round(a))
        for k, a in enumerate((s.vx, s.vy, s.vz)):
            assert np.array_equal(f[3 + k], a)
        assert (i[0] == 0).all() and (i[2] == 0).all()          # bptnr, extra_repuls: none (1-based 0)
        assert set(np.unique(i[1]).tolist()) <= set([1, 2, 4] + list(range(10, 29)))
        assert t == 0.0 and coll == 1000                          # the stand-in kernel counts its target
    mock.dmd_batch_destroy(h)
    assert mock.mock_live_allocations() <= base + 1          # the pinned stage stays for the next creation


def test_set_state_replaces_in_place_and_keeps_state_on_error(mock):
    spec = systems.generate(dense_system(seed=6))
    n = spec.n_beads
    tabs = abi.tables_struct(default_tables())
    cfg = spec.run_cfg(0, 0)
    sys_ = spec.c_system()
    mock.mock_reset()
    base = mock.mock_live_allocations()
    h = C.c_void_p()
    assert mock.dmd_create(C.byref(cfg), C.byref(tabs), C.byref(sys_), C.byref(h)) == 0
    rng = np.random.default_rng(2)
    new = [np.ascontiguousarray(a) + rng.normal(0, 1e-3, n) for a in (spec.x, spec.y, spec.z)]
    newv = [np.ascontiguousarray(a) * 0.5 for a in (spec.vx, spec.vy, spec.vz)]
    cols = new + newv
    assert mock.dmd_set_state(h, *[c.ctypes.data for c in cols], None, 2.5, 1234) == 0, mock.dmd_last_error(h)
    f, i, t, coll = state_of(mock, h, 0, n, batch=False)
    assert t == 2.5 and coll == 1234
    for k in range(3):
        assert np.array_equal(f[k], cols[k] - np.round(cols[k])) and np.array_equal(f[3 + k], cols[3 + k])
    bad = np.full(n, np.nan)
    assert mock.dmd_set_state(h, *[bad.ctypes.data] * 6, None, 0.0, 0) == -1
    assert b"non-finite" in mock.dmd_last_error(h)
    f2, i2, t2, coll2 = state_of(mock, h, 0, n, batch=False)
    assert np.array_equal(f2, f) and t2 == 2.5 and coll2 == 1234
    short = np.zeros(n, np.int32)
    short[0] = n + 5                                          # a partner beyond the system
    assert mock.dmd_set_state(h, *[c.ctypes.data for c in cols], short.ctypes.data, 0.0, 0) == -1
    assert mock.dmd_run(h, 500, None) == 0
    assert mock.mock_report() == b"", mock.mock_report().decode()
    mock.dmd_destroy(h)
    assert mock.mock_live_allocations() <= base + 1


def test_creation_errors_leave_nothing_behind(mock):
    """A system that fails its set-up returns DMD_E_INPUT with the
    replica's index, and destroying the handle frees everything."""
    good = systems.generate(systems.klvffae_system(2, 5.0, 0.2, seed=1))
    bad = systems.generate(systems.klvffae_system(2, 5.0, 0.2, seed=2))
    bad.vx = bad.vx.copy()
    bad.vx[3] = np.inf
    specs = [good, bad]
    tabs = abi.tables_struct(default_tables())
    cfgs = (abi.RunCfg * 2)(*[s.run_cfg(0, 0) for s in specs])
    syss = (abi.System * 2)(*[s.c_system() for s in specs])
    base = mock.mock_live_allocations()
    h = C.c_void_p()
    assert mock.dmd_batch_create(2, cfgs, C.byref(tabs), syss, C.byref(h)) == -1
    assert b"system 1" in mock.dmd_batch_last_error(h)
    mock.dmd_batch_destroy(h)
    assert mock.mock_live_allocations() <= base + 1


def _server(lib, slots, budget, chunk):
    s = C.c_void_p()
    assert lib.dmd_server_create(slots, budget, chunk, C.byref(s)) == 0
    return s


def _submit(lib, s, spec, n_events):
    tabs = abi.tables_struct(default_tables())
    cfg = spec.run_cfg(0, 0)
    sys_ = spec.c_system()
    rid = C.c_int64()
    rc = lib.dmd_server_submit(s, C.byref(cfg), C.byref(tabs), C.byref(sys_), n_events, C.byref(rid))
    return rc, rid.value


def _status(lib, s, rid):
    st, done = C.c_int32(), C.c_int64()
    ts, ta, tf = C.c_double(), C.c_double(), C.c_double()
    rc = lib.dmd_server_status(s, rid, C.byref(st), C.byref(done), C.byref(ts), C.byref(ta), C.byref(tf))
    return rc, st.value, done.value, ta.value


def _drain(lib, s, ids, limit=200):
    max_active, steps = 0, 0
    while True:
        na, nf = C.c_int32(), C.c_int32()
        assert lib.dmd_server_step(s, C.byref(na), C.byref(nf)) == 0, lib.dmd_server_last_error(s)
        max_active = max(max_active, na.value)
        steps += 1
        if all(_status(lib, s, i)[1] == 2 for i in ids):
            return max_active, steps
        assert steps < limit


def test_server_admits_in_order_within_slots_and_chunks(mock):
    """Requests are admitted first in, first out, never more than the slots
    at once; each step advances a request by at most its chunk-sized target
    until its events are done; the result is its own state."""
    specs = [systems.generate(systems.klvffae_system(2 + r % 3, 5.0, 0.2, seed=r + 1)) for r in range(6)]
    events = [2500, 1000, 3000, 500, 1000, 1500]
    mock.mock_reset()
    s = _server(mock, 2, 0, 1000)
    ids = []
    for spec, ev in zip(specs, events):
        rc, rid = _submit(mock, s, spec, ev)
        assert rc == 0
        ids.append(rid)
    max_active, steps = _drain(mock, s, ids)
    assert max_active <= 2
    admits = [_status(mock, s, i)[3] for i in ids]
    assert admits == sorted(admits)
    for rid, ev, spec in zip(ids, events, specs):
        rc, st, done, _ = _status(mock, s, rid)
        assert (rc, st, done) == (0, 2, ev)
        n = spec.n_beads
        f = np.zeros((6, n))
        i = np.zeros((2, n), np.int32)
        t, tf, coll = C.c_double(), C.c_double(), C.c_int64()
        d = abi.Diag()
        assert mock.dmd_server_result(s, rid, C.byref(d), *[abi.ptr(f[k], abi.dbl_p) for k in range(6)],
                                      abi.ptr(i[0], abi.i32_p), abi.ptr(i[1], abi.i32_p), C.byref(t), C.byref(tf),
                                      C.byref(coll)) == 0
        assert np.array_equal(f[0], spec.x - np.round(spec.x)) and np.array_equal(f[5], spec.vz)
        assert coll.value == ev
        assert mock.dmd_server_release(s, rid) == 0
        assert _status(mock, s, rid)[0] != 0
    assert mock.mock_report() == b"", mock.mock_report().decode()
    mock.dmd_server_destroy(s)


def test_server_respects_the_memory_budget(mock):
    """A budget that holds one request's pool admits one at a time; a request
    larger than the budget is refused at submission."""
    spec = systems.generate(systems.klvffae_system(3, 5.0, 0.2, seed=4))
    s = _server(mock, 8, 0, 1000)
    rc, rid = _submit(mock, s, spec, 1000)
    na, nf = C.c_int32(), C.c_int32()
    assert rc == 0 and mock.dmd_server_step(s, C.byref(na), C.byref(nf)) == 0
    steps, events, wait, act, used, budget = C.c_int64(), C.c_int64(), C.c_int32(), C.c_int32(), C.c_int64(), C.c_int64()
    ms = C.c_double()
    assert mock.dmd_server_stats(s, C.byref(steps), C.byref(events), C.byref(ms), C.byref(wait), C.byref(act),
                                 C.byref(used), C.byref(budget)) == 0
    need = used.value
    assert need > 0
    mock.dmd_server_destroy(s)
    s = _server(mock, 8, int(need * 1.5), 1000)
    ids = []
    for r in range(3):
        rc, rid = _submit(mock, s, systems.generate(systems.klvffae_system(3, 5.0, 0.2, seed=10 + r)), 2000)
        assert rc == 0
        ids.append(rid)
    max_active, _ = _drain(mock, s, ids)
    assert max_active == 1
    big = systems.generate(systems.klvffae_system(12, 5.0, 0.2, seed=20))
    rc, _ = _submit(mock, s, big, 1000)
    assert rc == -7 and b"budget" in mock.dmd_server_last_error(s)
    mock.dmd_server_destroy(s)


def test_compact_variant_hands_over_to_the_full_one(mock):
    """A system whose lists outgrow the compact variant stops with need_full;
    the host runs the full variant for that system's remaining events only
    (the others enter with target 0), and every system ends with its target."""
    mock.mock_set_handoff.argtypes = [C.c_int]
    mock.mock_last_target_of.restype = C.c_longlong
    mock.mock_last_target_of.argtypes = [C.c_int]
    specs = [systems.generate(systems.klvffae_system(3, 5.0, 0.2 + 0.02 * r, seed=30 + r)) for r in range(4)]
    n = len(specs)
    tabs = abi.tables_struct(default_tables())
    cfgs = (abi.RunCfg * n)(*[s.run_cfg(0, 0) for s in specs])
    syss = (abi.System * n)(*[s.c_system() for s in specs])
    mock.mock_reset()
    h = C.c_void_p()
    assert mock.dmd_batch_create(n, cfgs, C.byref(tabs), syss, C.byref(h)) == 0
    mock.mock_set_handoff(2)
    assert mock.dmd_batch_run(h, 3001, None) == 0, mock.dmd_batch_last_error(h)
    init, run, diag, target, C_, compact = counts(mock)
    assert run == 2 and compact == 0 and target == 0           # the follow-up: full variant, per-system targets
    assert [mock.mock_last_target_of(r) for r in range(n)] == [0, 0, 3001 - 1500, 0]
    for r, s in enumerate(specs):
        assert state_of(mock, h, r, s.n_beads)[3] == 3001
    assert mock.mock_report() == b"", mock.mock_report().decode()
    mock.dmd_batch_destroy(h)


def test_rebuild_cycle_graph_replays_until_every_target(mock):
    """dmd_batch_run_cycles captures its launches once and replays the graph
    until every system has run its events; each launch takes the remaining
    counts the previous one wrote back.  In the stand-in, system r runs at
    most 1000 + 500 r events per launch (its rebuild interval), so 5000
    events take 5, 4, 3 and 3 launches; system 2 hands over to the full
    variant halfway through its first launch and makes no progress in the
    second (compact) one: three replays of two launches, the last two on
    the full variant."""
    mock.mock_set_handoff.argtypes = [C.c_int]
    specs = [systems.generate(systems.klvffae_system(3, 5.0, 0.2 + 0.02 * r, seed=40 + r)) for r in range(4)]
    n = len(specs)
    tabs = abi.tables_struct(default_tables())
    cfgs = (abi.RunCfg * n)(*[s.run_cfg(0, 0) for s in specs])
    syss = (abi.System * n)(*[s.c_system() for s in specs])
    mock.mock_reset()
    h = C.c_void_p()
    assert mock.dmd_batch_create(n, cfgs, C.byref(tabs), syss, C.byref(h)) == 0
    g0 = mock.mock_graph_launches()
    mock.mock_set_handoff(2)
    k = C.c_int64()
    assert mock.dmd_batch_run_cycles(h, 5000, 2, C.byref(k)) == 0, mock.dmd_batch_last_error(h)
    init, run, diag, target, C_, compact = counts(mock)
    assert k.value == 6 and run == 6 and mock.mock_graph_launches() - g0 == 3
    assert compact == 0                                         # recaptured on the full variant
    for r, s in enumerate(specs):
        assert state_of(mock, h, r, s.n_beads)[3] == 5000
    # a second call reuses the full-variant graph: every system starts again
    assert mock.dmd_batch_run_cycles(h, 1000, 2, C.byref(k)) == 0
    assert k.value == 2
    for r, s in enumerate(specs):
        assert state_of(mock, h, r, s.n_beads)[3] == 6000
    assert mock.dmd_batch_run_cycles(h, 10, 0, None) == -1     # no launches per graph
    assert mock.mock_report() == b"", mock.mock_report().decode()
    mock.dmd_batch_destroy(h)


def test_autotune_cache_file(mock, tmp_path):
    """The autotuner's choice is kept in a JSON file: the first batch of a
    shape runs the trials and stores its choice, a second batch of the same
    shapes takes it without a launch, another shape adds an entry, and a
    file that is not a cache is refused and left as it was."""
    import json

    def make(k, seed):
        specs = [systems.generate(systems.klvffae_system(k, 5.0, 0.2, seed=seed + r)) for r in range(3)]
        tabs = abi.tables_struct(default_tables())
        cfgs = (abi.RunCfg * 3)(*[s.run_cfg(0, 0) for s in specs])
        syss = (abi.System * 3)(*[s.c_system() for s in specs])
        h = C.c_void_p()
        assert mock.dmd_batch_create(3, cfgs, C.byref(tabs), syss, C.byref(h)) == 0
        return h

    path = str(tmp_path / "tune.json")
    c, d, ms, hit = C.c_int32(), C.c_int32(), C.c_double(), C.c_int32()
    mock.mock_reset()
    h = make(3, 50)
    assert mock.dmd_batch_autotune_cached(h, 2000, path.encode(), C.byref(c), C.byref(d), C.byref(ms), C.byref(hit)) == 0
    runs = counts(mock)[1]
    assert hit.value == 0 and runs > 0
    doc = json.load(open(path))
    assert doc["format"] == "dmd-autotune-1" and len(doc["entries"]) == 1
    (key, e), = doc["entries"].items()
    assert key.startswith("cc10.3/sm152/") and e["cluster"] == c.value and e["cell_div"] == d.value
    assert e["systems"] == 3 and e["trial_events"] == 2000
    mock.dmd_batch_destroy(h)
    h = make(3, 50)
    assert mock.dmd_batch_autotune_cached(h, 2000, path.encode(), C.byref(c), C.byref(d), C.byref(ms), C.byref(hit)) == 0
    assert hit.value == 1 and counts(mock)[1] == runs          # no trial launch
    assert c.value == e["cluster"] and d.value == e["cell_div"]
    assert mock.dmd_batch_run(h, 100, None) == 0 and mock.dmd_batch_cluster(h) == e["cluster"]
    mock.dmd_batch_destroy(h)
    h = make(4, 60)
    assert mock.dmd_batch_autotune_cached(h, 2000, path.encode(), None, None, None, C.byref(hit)) == 0
    assert hit.value == 0 and len(json.load(open(path))["entries"]) == 2
    bad = tmp_path / "other.json"
    bad.write_text('{"format": "something else", "entries": {}}')
    assert mock.dmd_batch_autotune_cached(h, 2000, str(bad).encode(), None, None, None, None) == -1
    assert b"not a dmd-autotune-1 file" in mock.dmd_batch_last_error(h)
    assert bad.read_text() == '{"format": "something else", "entries": {}}'
    mock.dmd_batch_destroy(h)
    assert mock.mock_report() == b"", mock.mock_report().decode()


def test_phipsi_sample_counts_and_reset(mock):
    """The (phi, psi) histogram's host side: samples of every system or of
    one, the count per system, reset, and a replica index out of range."""
    specs = [systems.generate(systems.klvffae_system(3, 5.0, 0.2, seed=70 + r)) for r in range(3)]
    tabs = abi.tables_struct(default_tables())
    cfgs = (abi.RunCfg * 3)(*[s.run_cfg(0, 0) for s in specs])
    syss = (abi.System * 3)(*[s.c_system() for s in specs])
    mock.mock_reset()
    h = C.c_void_p()
    assert mock.dmd_batch_create(3, cfgs, C.byref(tabs), syss, C.byref(h)) == 0
    n = C.c_int64()
    hist = np.ones(361 * 361, np.int64)
    assert mock.dmd_batch_phipsi_histogram(h, 0, hist.ctypes.data_as(abi.i64_p), C.byref(n), 0) == 0
    assert n.value == 0 and hist.sum() == 0                      # nothing sampled yet
    assert mock.dmd_batch_phipsi_sample(h, -1) == 0
    assert mock.dmd_batch_phipsi_sample(h, 2) == 0
    counts = []
    for r in range(3):
        assert mock.dmd_batch_phipsi_histogram(h, r, None, C.byref(n), 0) == 0
        counts.append(n.value)
    assert counts == [1, 1, 2]
    assert mock.dmd_batch_phipsi_histogram(h, 2, None, C.byref(n), 1) == 0 and n.value == 2
    assert mock.dmd_batch_phipsi_histogram(h, 2, None, C.byref(n), 0) == 0 and n.value == 0
    assert mock.dmd_batch_phipsi_sample(h, 3) == -1
    assert mock.dmd_batch_phipsi_histogram(h, -1, None, None, 0) == -1
    assert mock.mock_report() == b"", mock.mock_report().decode()
    mock.dmd_batch_destroy(h)


def test_server_step_books_a_failed_read_back(mock):
    """A result read-back that fails while a finished request is retired
    fails that request alone: its pool is freed and it leaves the active
    set, the step reports the error, and the next steps run the other
    request to completion without touching the freed pool."""
    mock.mock_fail_d2h.argtypes = [C.c_int]
    a = systems.generate(systems.klvffae_system(2, 5.0, 0.2, seed=41))
    b = systems.generate(systems.klvffae_system(3, 5.0, 0.2, seed=42))
    mock.mock_reset()
    base = mock.mock_live_allocations()
    s = _server(mock, 4, 0, 1000)
    rc, ida = _submit(mock, s, a, 800)       # finishes in its first running step
    assert rc == 0
    rc, idb = _submit(mock, s, b, 3000)
    assert rc == 0
    na, nf = C.c_int32(), C.c_int32()
    assert mock.dmd_server_step(s, C.byref(na), C.byref(nf)) == 0   # admits both
    assert na.value == 2
    # next step: copy 1 reads request a's scalars, copy 2 is the first copy of its result
    mock.mock_fail_d2h(2)
    rc = mock.dmd_server_step(s, C.byref(na), C.byref(nf))
    assert rc == -6, rc                                               # DMD_E_CUDA
    assert b"request" in mock.dmd_server_last_error(s)
    assert (na.value, nf.value) == (1, 1)
    rc_a, st_a, _, _ = _status(mock, s, ida)
    assert rc_a == -6 and st_a == 3                                   # DMD_REQ_FAILED, its status
    mock.mock_fail_d2h(0)
    _drain(mock, s, [idb])
    rc_b, st_b, done_b, _ = _status(mock, s, idb)
    assert (rc_b, st_b, done_b) == (0, 2, 3000)
    assert mock.mock_report() == b"", mock.mock_report().decode()
    mock.dmd_server_destroy(s)
    assert mock.mock_live_allocations() <= base + 1


def _noalloc_call(lib, spec, list_cap=0):
    n = spec.n_beads
    cfg = spec.run_cfg(0, list_cap)
    tabs = abi.tables_struct(default_tables())
    sys_ = spec.c_system()
    outs = [np.zeros(n), np.zeros(n, np.int32), np.zeros(n, np.int32)]
    err = C.create_string_buffer(256)
    rc = lib.dmd_predict_all_noalloc(C.byref(cfg), C.byref(tabs), C.byref(sys_), *[o.ctypes.data for o in outs],
                                     None, err, 256)
    return rc, err.value


def test_noalloc_rejects_list_cap_and_grid_beyond_its_array(mock):
    """The allocation-free prediction pass refuses, before any device call,
    neighbour lists longer than 64 entries and a rebuild grid of more than
    48 cells per side, each with DMD_E_CAPACITY and a message."""
    spec = systems.generate(systems.klvffae_system(4, 5.0, 0.2, seed=3))
    rc, msg = _noalloc_call(mock, spec, list_cap=65)
    assert rc == -7 and b"list_cap at most 64" in msg, (rc, msg)
    wide = systems.generate(systems.klvffae_system(4, 0.01, 0.2, seed=3))  # 0.01 mM: a box of ~870 A
    rc, msg = _noalloc_call(mock, wide)
    assert rc == -7 and b"cells per side" in msg, (rc, msg)
