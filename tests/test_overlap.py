"""The overlap and bond-window check of code/checkover.f:18-131 on initial
states (the reference runs it at start-up, code/main.F90:347) and at output
events under -Ddebugging (code/main.F90:1193-1205), and the H-bond
consistency counters of code/check_nc_int.f:9-360.

The faults are made on the host: a bead moved onto another chain's bead,
a side chain pulled out of its bond window."""
import dataclasses

import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.engine import DMDError, Engine
from helpers import dense_system, first_mismatch
from oracle.oracle import Oracle


def _base():
    return systems.generate(systems.klvffae_system(4, 5.0, 0.2, seed=3))


def _overlapping(spec):
    """bead 0 of chain 1 (a C-alpha) put 1 A from bead 0 of chain 0"""
    x, y, z = spec.x.copy(), spec.y.copy(), spec.z.copy()
    j = 28
    x[j], y[j], z[j] = x[0] + 1.0 / spec.boxl, y[0], z[0]
    return dataclasses.replace(spec, x=x, y=y, z=z), (1, j + 1)


def _broken_bond(spec):
    """the side chain of residue 2 of chain 0 pulled 0.6 A away from its C-alpha"""
    p = [spec.x.copy(), spec.y.copy(), spec.z.copy()]
    r = 22                                   # R of residue 2 (bonded to C-alpha 2, bead 1)
    d = np.array([q[r] - q[1] for q in p])
    d = d - np.round(d)
    for k in range(3):
        p[k][r] = p[k][r] + 0.6 / spec.boxl * d[k] / np.linalg.norm(d)
    return dataclasses.replace(spec, x=p[0], y=p[1], z=p[2]), (2, r + 1)


def test_oracle_flags_overlap_and_broken_bond(built):
    spec = _base()
    Oracle(spec)                              # a generated state passes
    for make in (_overlapping, _broken_bond):
        bad, pair = make(spec)
        with pytest.raises(RuntimeError, match="overlap|window") as ei:
            Oracle(bad)
        assert f"beads {pair[0]} and {pair[1]}" in str(ei.value)
        # the reference's start-up only reports the overlap and goes on; the
        # prediction of an overlapping pair may then stop at its negative
        # time (code/events.f:59-73), but not at the overlap check
        try:
            Oracle(bad, flags=abi.FLAG_ALLOW_OVERLAP)
        except RuntimeError as e:
            assert "negative predicted time" in str(e), str(e)


def test_oracle_nc_int_counters_on_a_fresh_state(built):
    d = Oracle(dense_system(seed=4)).diagnostics()
    assert d["nc_boundbad"] == 0
    assert d["nc_unboundbad"] >= 0


@pytest.mark.gpu
def test_create_rejects_overlap_and_broken_bond(built):
    spec = _base()
    for make in (_overlapping, _broken_bond):
        bad, pair = make(spec)
        with pytest.raises(DMDError) as ei:
            Engine(bad)
        assert ei.value.rc == -2, str(ei.value)
        named = [int(w) for w in str(ei.value).split("beads ")[1].split(" overlap")[0].split(" and ")]
        assert pair[1] in named, str(ei.value)      # the moved bead (the device reports the pair it met first)
        try:                                  # no overlap check: at most the negative-time stop
            Engine(bad, flags=abi.FLAG_ALLOW_OVERLAP).close()
        except DMDError as e:
            assert e.rc == -3, str(e)
    with Engine(spec) as eng:                 # the library is still usable and exact
        glog = eng.run(3000, log_capacity=3064)
    assert first_mismatch(glog, Oracle(spec).run(3000, log_capacity=3064)) < 0


@pytest.mark.gpu
def test_set_state_rejects_overlap_and_keeps_state(built):
    spec = _base()
    bad, _ = _overlapping(spec)
    with Engine(spec) as eng:
        eng.run(2000)
        before = eng.state()
        with pytest.raises(DMDError) as ei:
            eng.set_state(bad.x, bad.y, bad.z, bad.vx, bad.vy, bad.vz)
        assert ei.value.rc == -2
        after = eng.state()
        for k in ("x", "vx", "bptnr"):
            assert np.array_equal(before[k], after[k])
        assert before["coll"] == after["coll"]


@pytest.mark.gpu
def test_output_event_check_and_nc_counters(built):
    """With the output-event check on, an H-bond-rich run stays clean and
    commits the same events as the oracle with the same check; the
    check_nc_int counters agree with the oracle's."""
    spec = dense_system(n_chains=4, L=10, box=30.0, tstar=0.12, seed=21, rng_seed=5)
    n = 1450000                               # the first output event comes at about 1.42e6
    flags = abi.FLAG_CHECK_OVERLAP
    with Engine(spec, flags=flags) as eng:
        glog = eng.run(n, log_capacity=n + 64)
        gd = eng.diagnostics()
    ora = Oracle(spec, flags=flags)
    olog = ora.run(n, log_capacity=n + 64)
    od = ora.diagnostics()
    assert (glog["type"] == abi.EV_OUTPUT).any(), "no output event in the run"
    assert first_mismatch(glog, olog) < 0
    assert gd["hb_ii"] + gd["hb_ij"] > 0
    for k in ("nc_boundbad", "nc_unboundbad"):
        assert gd[k] == od[k], k
