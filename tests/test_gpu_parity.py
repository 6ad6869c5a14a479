"""GPU engine against the CPU restatement of the reference: the committed
event sequence (bead pair, final collision type, pair code, time) and the
final state must be identical bit for bit, on the same seeded inputs."""
import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.engine import Batch, Engine
from helpers import dense_system, describe, first_mismatch
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _compare_run(spec, n_events, flags=0):
    with Engine(spec, flags=flags) as eng:
        glog = eng.run(n_events, log_capacity=n_events + 64)
        gst = eng.state()
    ora = Oracle(spec, flags=flags)
    olog = ora.run(n_events, log_capacity=n_events + 64)
    ost = ora.state()
    k = first_mismatch(glog, olog)
    assert k < 0, f"event logs diverge at {k} of {len(olog)}:\n{describe(glog, olog, k)}"
    for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity", "extra_repuls"):
        assert np.array_equal(gst[key], ost[key]), f"final {key} differs"
    assert gst["t"] == ost["t"] and gst["tfalse"] == ost["tfalse"] and gst["coll"] == ost["coll"]
    return glog


def test_predict_all_initial(built):
    spec = systems.generate(systems.config_c1())
    with Engine(spec) as eng:
        gt, gp, gc = eng.predictions()
    ot, op, oc = Oracle(spec).predictions()
    assert np.array_equal(gp, op)
    assert np.array_equal(gc, oc)
    assert np.array_equal(gt, ot)


@pytest.mark.parametrize("pick", ["smallest", "largest"])
def test_predict_all_initial_c3(built, pick):
    """The first rebuild's predictions of the 32-replica workload's smallest
    and largest systems (626 and 5,576 beads: the full prediction is shared
    by several CTAs per system)."""
    specs = sorted(systems.config_c3(32, seed=1), key=lambda s: s.n_beads)
    spec = systems.generate(specs[0] if pick == "smallest" else specs[-1])
    with Engine(spec) as eng:
        gt, gp, gc = eng.predictions()
    ot, op, oc = Oracle(spec).predictions()
    assert np.array_equal(gp, op)
    assert np.array_equal(gc, oc)
    assert np.array_equal(gt, ot)


def test_set_state_restarts(built):
    """dmd_set_state on a running system equals dmd_create from the same
    state, and both follow the oracle restarted from it (the reference's
    restart from its records, code/main.F90:240-321), H-bonds included."""
    import dataclasses
    spec = dense_system(n_chains=10, L=10, box=38.0, tstar=0.12, seed=21, rng_seed=5)
    with Engine(spec) as eng:
        eng.run(40000)
        now = eng.state_now()
    assert (now["bptnr"] > 0).any(), "the restart should carry H-bonds"
    restart = dataclasses.replace(spec, x=now["x"], y=now["y"], z=now["z"], vx=now["vx"], vy=now["vy"], vz=now["vz"],
                                  bptnr=now["bptnr"], t0=now["t"], coll0=now["coll"])
    n = 8000
    with Engine(spec) as eng:
        eng.run(500)   # another state first
        eng.set_state(now["x"], now["y"], now["z"], now["vx"], now["vy"], now["vz"], now["bptnr"], now["t"], now["coll"])
        slog = eng.run(n, log_capacity=n + 64)
        sst = eng.state()
    with Engine(restart) as eng:
        clog = eng.run(n, log_capacity=n + 64)
    ora = Oracle(restart)
    olog = ora.run(n, log_capacity=n + 64)
    ost = ora.state()
    assert first_mismatch(slog, clog) < 0
    k = first_mismatch(slog, olog)
    assert k < 0, f"restart diverges from the oracle at {k}:\n{describe(slog, olog, k)}"
    for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity", "extra_repuls"):
        assert np.array_equal(sst[key], ost[key]), key
    assert sst["t"] == ost["t"] and sst["coll"] == ost["coll"]


def test_set_state_rejects_bad_input_and_keeps_state(built):
    spec = dense_system(seed=6)
    with Engine(spec) as eng:
        eng.run(1000)
        before = eng.state()
        bad = np.full(eng.n, np.nan)
        with pytest.raises(Exception):
            eng.set_state(bad, bad, bad, bad, bad, bad)
        after = eng.state()
        for key in ("x", "vx", "bptnr"):
            assert np.array_equal(before[key], after[key])
        eng.run(100)


def test_c1_event_sequence(built):
    spec = systems.generate(systems.config_c1())
    log = _compare_run(spec, 20000)
    assert (log["type"] == abi.EV_GHOST).any() and (log["type"] == abi.EV_REBUILD).any()


def test_dense_all_event_kinds(built):
    spec = dense_system()
    log = _compare_run(spec, 40000)
    kinds = set(np.unique(log["type"]).tolist())
    assert {1, 2, 3}.issubset(kinds)


def test_no_thermostat(built):
    spec = dense_system(seed=5)
    spec.canon = False
    _compare_run(spec, 20000)


def test_evcode_after_run(built):
    spec = dense_system(n_chains=4, L=10, box=45.0, seed=9)
    with Engine(spec) as eng:
        eng.run(30000)
        g = eng.evcode()
    ora = Oracle(spec)
    ora.run(30000)
    assert np.array_equal(g, ora.evcode())


def test_batch_equals_single(built):
    specs = [systems.generate(systems.klvffae_system(4, 5.0, 0.2 + 0.05 * r, seed=r + 1)) for r in range(3)]
    b = Batch(specs)
    logs = b.run(5000, log_capacity=5100)
    for r, spec in enumerate(specs):
        olog = Oracle(spec).run(5000, log_capacity=5100)
        assert first_mismatch(logs[r], olog) < 0


def test_diagnostics_match(built):
    spec = dense_system(seed=4)
    with Engine(spec) as eng:
        eng.run(20000)
        gd = eng.diagnostics()
    ora = Oracle(spec)
    ora.run(20000)
    od = ora.diagnostics()
    for k in ("e_total", "temperature", "rg", "e2e", "ehh_ii", "ehh_ij"):
        assert gd[k] == pytest.approx(od[k], rel=1e-12, abs=1e-12), k
    for k in ("hb_alpha", "hb_ii", "hb_ij", "coll", "n_pair", "n_ghost", "n_interval", "n_updates"):
        assert gd[k] == od[k], k


def test_hbond_events(built):
    """A crowded cold system in which H-bonds form and break: captures,
    escapes, bounces and the shoulder events of repuls_add all occur."""
    spec = dense_system(n_chains=10, L=10, box=38.0, tstar=0.12, seed=21, rng_seed=5)
    log = _compare_run(spec, 400000)
    kinds = set(np.unique(log["type"]).tolist())
    assert {14, 16, 20, 21, 22, 26}.issubset(kinds), kinds


def test_c3_replicas_batched(built):
    """Replicas of the 32-replica workload, advanced together in one launch,
    each against its own serial oracle run."""
    specs = systems.config_c3(32, seed=1)
    small = sorted(specs, key=lambda s: s.n_beads)[:4] + [specs[31]]
    for s in small:
        systems.generate(s)
    n = 30000
    b = Batch(small)
    logs = b.run(n, log_capacity=n + 64)
    for r, s in enumerate(small):
        ora = Oracle(s)
        olog = ora.run(n, log_capacity=n + 64)
        k = first_mismatch(logs[r], olog)
        assert k < 0, f"replica {r}: logs diverge at {k}:\n{describe(logs[r], olog, k)}"
        st, ost = b.state(r), ora.state()
        for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity"):
            assert np.array_equal(st[key], ost[key]), (r, key)
    b.close()


@pytest.mark.parametrize("ctas", [1, 2, 4, 8])
def test_cluster_sizes(built, ctas):
    """The same systems advanced with 1, 2, 4 or 8 CTAs per system commit
    the oracle's event sequence."""
    specs = systems.config_c3(32, seed=2)
    pick = [sorted(specs, key=lambda s: s.n_beads)[0], specs[7], specs[30]]
    for s in pick:
        systems.generate(s)
    n = 20000
    b = Batch(pick, cluster=ctas)
    logs = b.run(n, log_capacity=n + 64)
    assert b.cluster == ctas
    for r, s in enumerate(pick):
        ora = Oracle(s)
        olog = ora.run(n, log_capacity=n + 64)
        k = first_mismatch(logs[r], olog)
        assert k < 0, f"C={ctas} replica {r}: logs diverge at {k}:\n{describe(logs[r], olog, k)}"
        st, ost = b.state(r), ora.state()
        for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity"):
            assert np.array_equal(st[key], ost[key]), (ctas, r, key)
    b.close()


def test_cluster_hbond_plain(built):
    """The plain path on a cluster of 4 CTAs, on the H-bond-rich system."""
    spec = dense_system(n_chains=10, L=10, box=38.0, tstar=0.12, seed=21, rng_seed=5)
    with Engine(spec, cluster=4) as eng:
        glog = eng.run(200000, log_capacity=200064)
    ora = Oracle(spec)
    olog = ora.run(200000, log_capacity=200064)
    k = first_mismatch(glog, olog)
    assert k < 0, f"logs diverge at {k}:\n{describe(glog, olog, k)}"


def test_graph_replay_and_grid(built):
    """Launches replayed from a captured CUDA graph, and a coarser rebuild
    grid, commit the same events as one plain run."""
    specs = systems.config_c3(32, seed=3)[:3]
    for s in specs:
        systems.generate(s)
    ref = Batch(specs)
    ref.run(24000)
    want = [ref.state(r) for r in range(3)]
    ref.close()
    g = Batch(specs)
    g.set_cell_div(2)
    g.run_graph(6000, 2)
    g.run_graph(6000, 2)      # the second call replays the same graph
    for r in range(3):
        st = g.state(r)
        for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity"):
            assert np.array_equal(st[key], want[r][key]), (r, key)
        assert st["coll"] == want[r]["coll"]
    g.close()


def test_autotune_cache(built, tmp_path):
    """The autotuner's choice kept in a JSON file is taken by a second batch
    of the same replicas without trials."""
    specs = systems.config_c3(32, seed=4)[:4]
    for s in specs:
        systems.generate(s)
    path = str(tmp_path / "tune.json")
    with Batch(specs) as b:
        first = b.autotune(3000, cache=path)
    with Batch(specs) as b:
        again = b.autotune(3000, cache=path)
        b.run(2000)
        assert b.lib.dmd_batch_cluster(b.h) == first["cluster"]
    assert not first["cached"] and again["cached"]
    assert (again["cluster"], again["cell_div"]) == (first["cluster"], first["cell_div"])


def test_rebuild_cycle_graph(built):
    """Rebuild cycles replayed from a captured CUDA graph (each launch ends
    every system at its next neighbour-list rebuild) commit the same events
    as one plain run, and take at least one launch per rebuild."""
    specs = systems.config_c3(32, seed=3)[:3]
    for s in specs:
        systems.generate(s)
    ref = Batch(specs)
    ref.run(30000)
    want = [ref.state(r) for r in range(3)]
    ref.close()
    g = Batch(specs)
    u0 = [g.diagnostics(r)["n_updates"] for r in range(3)]
    k1 = g.run_cycles(15000, 2)
    u1 = [g.diagnostics(r)["n_updates"] for r in range(3)]
    k2 = g.run_cycles(15000, 2)   # the second call replays the same graph
    u2 = [g.diagnostics(r)["n_updates"] for r in range(3)]
    for r in range(3):
        st = g.state(r)
        for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity"):
            assert np.array_equal(st[key], want[r][key]), (r, key)
        assert st["coll"] == want[r]["coll"]
    assert max(b - a for a, b in zip(u0, u1)) >= 1
    assert k1 >= max(b - a for a, b in zip(u0, u1)) and k1 % 2 == 0
    assert k2 >= max(b - a for a, b in zip(u1, u2)) and k2 % 2 == 0
    g.close()


def test_autotune_keeps_state(built):
    specs = systems.config_c3(32, seed=4)[:4]
    for s in specs:
        systems.generate(s)
    b = Batch(specs)
    before = [b.state(r) for r in range(4)]
    cfg = b.autotune(3000)
    assert cfg["cluster"] in (1, 2, 4) and cfg["cell_div"] in (1, 2) and cfg["trial_ms"] > 0
    for r in range(4):
        st = b.state(r)
        assert np.array_equal(st["x"], before[r]["x"]) and st["coll"] == before[r]["coll"]
    logs = b.run(10000, log_capacity=10064)
    for r, s in enumerate(specs):
        olog = Oracle(s).run(10000, log_capacity=10064)
        assert first_mismatch(logs[r], olog) < 0, r
    b.close()


def test_capacity_error_is_reported(built):
    """Neighbour lists larger than their capacity end in DMD_E_CAPACITY with
    a message (at creation or at the first rebuild), no fault, and the
    library stays usable."""
    from dmdgb.engine import DMDError
    spec = dense_system(seed=6)
    with pytest.raises(DMDError) as ei:
        with Engine(spec, list_cap=2) as eng:
            eng.run(2000)
    assert ei.value.rc == -7, str(ei.value)
    with Engine(spec) as eng:          # a normal engine afterwards, still exact
        glog = eng.run(2000, log_capacity=2064)
    olog = Oracle(spec).run(2000, log_capacity=2064)
    assert first_mismatch(glog, olog) < 0


def test_compact_variant_hands_over(built):
    """The compact event loop (down lists of at most max_down beads) stops a
    system at the rebuild whose lists outgrow it and the full loop finishes
    the run: the events are still the oracle's, and the switch happened."""
    spec = dense_system(seed=8)
    n, chunk = 60000, 6000
    with Engine(spec) as eng:
        limit = eng.diagnostics()["max_down"]
        assert 0 < limit <= 32
        eng.set_compact_limit(limit)
        logs, crossed = [], False
        for _ in range(n // chunk):
            before = eng.diagnostics()["max_down"]
            logs.append(eng.run(chunk, log_capacity=chunk + 64))
            after = eng.diagnostics()["max_down"]
            crossed |= before <= limit < after
        gst = eng.state()
    assert crossed, "the lists never outgrew the compact limit"
    ora = Oracle(spec)
    olog = ora.run(n, log_capacity=n + 64)
    glog = np.concatenate(logs)
    k = first_mismatch(glog, olog)
    assert k < 0, f"event logs diverge at {k}:\n{describe(glog, olog, k)}"
    ost = ora.state()
    for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr"):
        assert np.array_equal(gst[key], ost[key]), key


def test_compact_variant_batch_and_graph(built):
    """Replicas that cross the compact limit at different times, in a batch
    run, in graph replay and in rebuild-cycle replay: the follow-up full
    launches give every replica the events of one plain run."""
    specs = systems.config_c3(32, seed=5)[:4]
    for s in specs:
        systems.generate(s)
    ref = Batch(specs)
    ref.set_compact_limit(0)          # the full variant throughout
    ref.run(16000)
    want = [ref.state(r) for r in range(4)]
    ref.close()
    b0 = Batch(specs)
    limit = min(32, max(b0.diagnostics(r)["max_down"] for r in range(4)))
    b0.close()
    for graph in (False, True, "cycles"):
        b = Batch(specs)
        b.set_compact_limit(limit)
        if graph == "cycles":
            b.run_cycles(16000, 3)
        elif graph:
            b.run_graph(4000, 4)
        else:
            b.run(16000)
        for r in range(4):
            st = b.state(r)
            for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity"):
                assert np.array_equal(st[key], want[r][key]), (graph, r, key)
            assert st["coll"] == want[r]["coll"], (graph, r)
        b.close()


def _compare_states(st, ost, what):
    for key in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity", "extra_repuls"):
        assert np.array_equal(st[key], ost[key]), f"{what}: final {key} differs"
    assert st["t"] == ost["t"] and st["coll"] == ost["coll"], what


@pytest.mark.parametrize("ctas", [1, 2])
def test_c2_event_sequence(built, ctas):
    """48 x KLVFFAE (1,344 beads, 252 A box, T* = 0.18): the single-system
    workload's first 20,000 events on one CTA and on a 2-CTA cluster."""
    spec = systems.generate(systems.config_c2())
    n = 20000
    with Engine(spec, cluster=ctas) as eng:
        glog = eng.run(n, log_capacity=n + 64)
        gst = eng.state()
    ora = Oracle(spec)
    olog = ora.run(n, log_capacity=n + 64)
    k = first_mismatch(glog, olog)
    assert k < 0, f"C2 (C={ctas}) diverges at {k}:\n{describe(glog, olog, k)}"
    _compare_states(gst, ora.state(), f"C2 C={ctas}")


def test_c4_event_sequence(built):
    """1,000 random 10-mers (40,000 beads, 10 mM, T* = 0.22): the large
    single-system workload's first 12,000 events on a 4-CTA cluster (global
    footprint tables, candidates spread over the cluster's shared memory)
    and on one CTA, both against one oracle run."""
    spec = systems.generate(systems.config_c4())
    n = 12000
    runs = {}
    for ctas in (4, 1):
        with Engine(spec, cluster=ctas) as eng:
            runs[ctas] = (eng.run(n, log_capacity=n + 64), eng.state())
    ora = Oracle(spec)
    olog = ora.run(n, log_capacity=n + 64)
    ost = ora.state()
    for ctas, (glog, gst) in runs.items():
        k = first_mismatch(glog, olog)
        assert k < 0, f"C4 (C={ctas}) diverges at {k}:\n{describe(glog, olog, k)}"
        _compare_states(gst, ost, f"C4 C={ctas}")


def test_c3_largest_replica_batched(built):
    """The 32-replica workload's largest system (5,576 beads: footprint
    tables in global memory) advanced in one launch beside the smallest,
    20,000 events each, against the oracle."""
    specs = sorted(systems.config_c3(32, seed=1), key=lambda s: s.n_beads)
    pick = [specs[-1], specs[0]]
    for s in pick:
        systems.generate(s)
    assert pick[0].n_beads > 5000
    n = 20000
    b = Batch(pick)
    logs = b.run(n, log_capacity=n + 64)
    for r, s in enumerate(pick):
        ora = Oracle(s)
        olog = ora.run(n, log_capacity=n + 64)
        k = first_mismatch(logs[r], olog)
        assert k < 0, f"replica of {s.n_beads} beads diverges at {k}:\n{describe(logs[r], olog, k)}"
        _compare_states(b.state(r), ora.state(), f"{s.n_beads} beads")
    b.close()


def test_two_species_event_sequence(built):
    """-Dchaptype=2 (code/make_code.f:489-548): two peptide species whose
    species-2 side chains meet as hard cores across chains; the events of a
    crowded mixed system against the oracle with the same rule."""
    spec = dense_system(n_chains=8, L=10, box=42.0, tstar=0.2, seed=31, rng_seed=9)
    spec.chaptype = 2
    spec.species2_chain = 4
    n = 40000
    with Engine(spec) as eng:
        glog = eng.run(n, log_capacity=n + 64)
        gst = eng.state()
    ora = Oracle(spec)
    olog = ora.run(n, log_capacity=n + 64)
    k = first_mismatch(glog, olog)
    assert k < 0, f"two-species run diverges at {k}:\n{describe(glog, olog, k)}"
    _compare_states(gst, ora.state(), "two species")


def test_c3_replica_long_run(built):
    """Replica 29 of the 32-replica workload (1,260 beads, T* = 0.48) over
    2.2 million events, chunk by chunk against the oracle: past 1.75 million
    events a bonded H-bond pair sits just outside its well, where the
    reference's root is a NaN that nothing selects (nc_sqwel.f:69-93)."""
    s = systems.generate(systems.config_c3(32, seed=1)[29])
    b = Batch([s])
    ora = Oracle(s)
    chunk = 200000
    for c in range(11):
        glog = b.run(chunk, log_capacity=chunk + 64)[0]
        olog = ora.run(chunk, log_capacity=chunk + 64)
        k = first_mismatch(glog, olog)
        assert k < 0, f"chunk {c}: logs diverge at {k}:\n{describe(glog, olog, k)}"
    _compare_states(b.state(0), ora.state(), "replica 29 after 2.2e6 events")
    b.close()
