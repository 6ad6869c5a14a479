"""dmd_predict_all_noalloc: the prediction pass for callers that cannot
allocate device memory (their device memory belongs to another runtime or a
fixed pool).  The test owns the output buffers, as such a caller would, and
checks the pass against dmd_create + dmd_predict_all on two calls in a row
(bit-identical, the tolerance of the other parity tests).  It sits in its
own file, collected last."""
import ctypes as C

import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.engine import Engine
from dmdgb.params import default_tables
from helpers import dense_system

pytestmark = pytest.mark.gpu


def _noalloc(spec, torch, list_cap=0):
    lib = abi.load_engine()
    n = spec.n_beads
    tim = torch.full((n,), -7.0, dtype=torch.float64, device="cuda")
    nptnr = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    ct = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    cfg = spec.run_cfg(0, list_cap)
    t = abi.tables_struct(default_tables())
    s = spec.c_system()
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.dmd_predict_all_noalloc(C.byref(cfg), C.byref(t), C.byref(s), tim.data_ptr(), nptnr.data_ptr(),
                                     ct.data_ptr(), C.c_void_p(stream), err, 256)
    assert rc == 0, err.value.decode()
    return tim.cpu().numpy(), nptnr.cpu().numpy(), ct.cpu().numpy()


def test_noalloc_matches_create_predict_twice(built):
    torch = pytest.importorskip("torch")
    specs = [systems.generate(systems.config_c1()), dense_system(seed=12)]
    for spec in specs:   # two calls in a row, different systems: no state carries over
        with Engine(spec) as eng:
            want = eng.predictions()
        got = _noalloc(spec, torch)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)


def test_noalloc_rejects_oversize(built):
    torch = pytest.importorskip("torch")
    lib = abi.load_engine()
    spec = systems.generate(systems.klvffae_system(300, 5.0, 0.2, 1))  # 8,400 beads > 8,192
    n = spec.n_beads
    out = [torch.zeros(n, dtype=d, device="cuda") for d in (torch.float64, torch.int32, torch.int32)]
    cfg = spec.run_cfg()
    t = abi.tables_struct(default_tables())
    s = spec.c_system()
    err = C.create_string_buffer(256)
    rc = lib.dmd_predict_all_noalloc(C.byref(cfg), C.byref(t), C.byref(s), *[o.data_ptr() for o in out], None, err, 256)
    assert rc == -7 and b"8192" in err.value


def test_noalloc_list_cap_at_its_limit(built):
    """Neighbour lists of 64 entries, the most the static array takes, on a
    crowded system: the same predictions as dmd_create with that capacity."""
    torch = pytest.importorskip("torch")
    spec = dense_system(seed=13)
    with Engine(spec, list_cap=64) as eng:
        want = eng.predictions()
    got = _noalloc(spec, torch, list_cap=64)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_noalloc_refuses_while_capturing(built):
    """A call made while the stream is being captured into a CUDA graph
    returns DMD_E_STATE and leaves the capture intact."""
    torch = pytest.importorskip("torch")
    lib = abi.load_engine()
    spec = systems.generate(systems.config_c1())
    n = spec.n_beads
    out = [torch.zeros(n, dtype=d, device="cuda") for d in (torch.float64, torch.int32, torch.int32)]
    x = torch.zeros(4, device="cuda")
    cfg = spec.run_cfg()
    t = abi.tables_struct(default_tables())
    s = spec.c_system()
    err = C.create_string_buffer(256)
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            x.add_(1.0)
            stream = torch.cuda.current_stream().cuda_stream
            rc = lib.dmd_predict_all_noalloc(C.byref(cfg), C.byref(t), C.byref(s), *[o.data_ptr() for o in out],
                                             C.c_void_p(stream), err, 256)
    torch.cuda.current_stream().wait_stream(side)
    assert rc == -8 and b"captured" in err.value, (rc, err.value)
    g.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0
