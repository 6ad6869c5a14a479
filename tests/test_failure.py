"""The bounded-wait failure path of the event loop, exercised without a
GPU fault: with DMD_FLAG_TIGHT_LOOP_BOUND the loop's iteration bound (the
guard that replaces the reference's unbounded wait for a worker,
code/main.F90:627) is 8 batches, so a run of more events stops between two
batches with DMD_E_DEVICE_TIMEOUT.  The handle reports the error on every
later call, and a fresh handle on the same device is still exact."""
import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.engine import Batch, DMDError, Engine
from helpers import first_mismatch
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def test_loop_bound_stops_with_device_timeout(built):
    spec = systems.generate(systems.config_c1())
    with Engine(spec, flags=abi.FLAG_TIGHT_LOOP_BOUND) as eng:
        with pytest.raises(DMDError) as ei:
            eng.run(5000)
        assert ei.value.rc == -4, str(ei.value)
        assert "iteration bound" in str(ei.value)
        st = eng.state()                      # the state reads back: stopped between batches
        assert 0 < st["coll"] < 5000
        with pytest.raises(DMDError) as again:
            eng.run(10)
        assert again.value.rc == -4
    with Engine(spec) as eng:                 # a fresh handle: exact
        glog = eng.run(3000, log_capacity=3064)
    assert first_mismatch(glog, Oracle(spec).run(3000, log_capacity=3064)) < 0


def test_loop_bound_in_a_batch_stops_only_that_replica(built):
    """Replicas of one launch: the one with the tight bound stops, the
    others reach their targets with the oracle's events."""
    specs = [systems.generate(systems.klvffae_system(4, 5.0, 0.2 + 0.05 * r, seed=r + 1)) for r in range(3)]
    flags = [0, abi.FLAG_TIGHT_LOOP_BOUND, 0]
    import ctypes as C
    from dmdgb.params import default_tables
    lib = abi.load_engine()
    tabs = abi.tables_struct(default_tables())
    cfgs = (abi.RunCfg * 3)(*[s.run_cfg(f, 0) for s, f in zip(specs, flags)])
    syss = (abi.System * 3)(*[s.c_system() for s in specs])
    h = C.c_void_p()
    assert lib.dmd_batch_create(3, cfgs, C.byref(tabs), syss, C.byref(h)) == 0
    rc = lib.dmd_batch_run(h, 4000, None)
    assert rc == -4 and b"system 1" in lib.dmd_batch_last_error(h)
    d = abi.Diag()
    for r in (0, 2):
        assert lib.dmd_batch_diagnostics(h, r, C.byref(d)) == 0
        assert d.coll == 4000
    lib.dmd_batch_destroy(h)
