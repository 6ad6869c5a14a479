"""Physics checks of the CPU restatement itself (it is the oracle, so it is
pinned independently): conservation laws and analytic two-bead answers.
The reference ships no tests or golden trajectories (its only run-time
checks are the energy-drift and overlap tests of code/main.F90:928-942 and
code/checkover.f), so these are the known-answer tests."""
import numpy as np
import pytest

from dmdgb import abi, systems
from helpers import dense_system
from oracle.oracle import Oracle


def _momentum(o, spec):
    st = o.state()
    bm = _masses(spec)
    return np.array([np.sum(bm * st["vx"]), np.sum(bm * st["vy"]), np.sum(bm * st["vz"])])


def _masses(spec):
    from dmdgb.params import default_tables
    t = default_tables()
    mass = t.mass.copy()
    mass[3] = mass[20]
    out, p = [], 0
    for L in spec.chain_len:
        seq = spec.residues[p:p + L]
        out += [mass[2]] * L + [mass[1]] * L + [mass[4]] * L + [mass[r] for r in seq if r != 9]
        p += L
    return np.array(out)


def test_energy_conserved_without_thermostat():
    """code/main.F90:928-942 checks nint(E) per event when built without
    -Dcanon; the restatement holds E to 1e-10 relative over 30,000 events."""
    spec = dense_system(seed=6)
    spec.canon = False
    o = Oracle(spec)
    e0 = o.diagnostics()["e_total"]
    for _ in range(6):
        o.run(5000)
        e = o.diagnostics()["e_total"]
        assert abs(e - e0) <= 1e-10 * abs(e0), (e, e0)


def test_momentum_conserved_by_pair_events():
    spec = dense_system(seed=8)
    spec.canon = False
    o = Oracle(spec)
    p0 = _momentum(o, spec)
    o.run(20000)
    p1 = _momentum(o, spec)
    scale = np.sum(_masses(spec) * np.abs(spec.vx))
    assert np.all(np.abs(p1 - p0) <= 1e-12 * scale)


def test_thermostat_drives_temperature():
    """Andersen ghost collisions pull T = sum m v^2 / 3N toward 12 T*."""
    spec = systems.generate(systems.klvffae_system(4, 5.0, 0.30, seed=3))
    o = Oracle(spec)
    temps = []
    for _ in range(20):
        o.run(20000)
        temps.append(o.diagnostics()["temperature"])
    assert abs(np.mean(temps[5:]) - 12 * 0.30) < 0.25 * 12 * 0.30


def test_event_counters_consistent():
    spec = dense_system(seed=2)
    o = Oracle(spec)
    log = o.run(10000, log_capacity=10000)
    d = o.diagnostics()
    assert d["coll"] == 10000 == len(log)
    assert d["n_pair"] == int(np.sum(log["type"] <= 27))
    assert d["n_ghost"] == int(np.sum(log["type"] == abi.EV_GHOST))
    assert d["n_updates"] == int(np.sum(log["type"] == abi.EV_REBUILD))
    assert sum(d["nevents"]) == d["n_pair"]
    assert np.all(np.diff(log["coll"]) == 1)
    t_abs = log["t"] + log["tfalse"]
    assert np.all(np.diff(t_abs) >= -1e-10)   # strict time order (up to the 1e-10 guard)


def test_bond_windows_hold():
    """After many events every bonded pair is inside its (1 +- del) window
    (code/checkover.f:74-126)."""
    spec = dense_system(seed=10)
    o = Oracle(spec)
    o.run(20000)
    st = o.state()
    ev = o.evcode()
    x = st["x"] + st["vx"] * st["tfalse"]
    y = st["y"] + st["vy"] * st["tfalse"]
    z = st["z"] + st["vz"] * st["tfalse"]
    ii, jj = np.nonzero(np.triu((ev >= 4) & (ev <= 9)))
    d = np.stack([x[ii] - x[jj], y[ii] - y[jj], z[ii] - z[jj]], 1)
    d -= np.round(d)
    r = np.sqrt((d ** 2).sum(1)) * spec.boxl
    bl = np.array([0, 0, 0, 0, 1.46, 1.51, 1.33, 2.41, 2.45, 3.8])[ev[ii, jj]]
    assert np.all(r >= bl * (1 - 0.02375) * (1 - 1e-9)) and np.all(r <= bl * (1 + 0.02375) * (1 + 1e-9))
