"""The C-ABI library loads and exports every function include/dmd.h
declares (CPU only: no compute call)."""
import ctypes as C
import os
import re

from dmdgb import abi

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "dmd.h")


def declared():
    text = open(HDR).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dmd_[a-z_0-9]+)\s*\(", text)))


def test_header_lists_entry_points():
    names = declared()
    assert "dmd_create" in names and "dmd_run" in names and "dmd_batch_run" in names
    assert set(abi.ENGINE_SYMBOLS) == set(names)


def test_library_exports_all(built):
    lib = abi.load_engine()
    for n in declared():
        assert hasattr(lib, n), n
    assert lib.dmd_version().decode().startswith("dmd-gb300")


def test_errors_are_status_codes(built):
    """Bad input returns a negative status and a message; nothing exits."""
    lib = abi.load_engine()
    h = C.c_void_p()
    cfg = abi.RunCfg(0.2, 1, 1, 1, 2000, 2, 1.2, 5e-5, 150.0, 0, 0, 1, 0)
    t = abi.Tables()
    s = abi.System()  # empty system
    rc = lib.dmd_create(C.byref(cfg), C.byref(t), C.byref(s), C.byref(h))
    assert rc == -1
    assert b"empty" in lib.dmd_last_error(h)
    lib.dmd_destroy(h)
    assert lib.dmd_set_state(None, None, None, None, None, None, None, None, 0.0, 0) == -1


def test_system_struct_matches_header_layout():
    """abi.System mirrors struct dmd_system: the array fields hold addresses,
    and the field offsets are those of the C declaration."""
    from dmdgb import systems
    spec = systems.klvffae_system(2, 5.0, 0.2, seed=1)
    n = spec.n_beads
    import numpy as np
    spec.x, spec.y, spec.z, spec.vx, spec.vy, spec.vz = [np.full(n, float(k)) for k in range(6)]
    s = spec.c_system()
    assert s.n_beads == n == 2 * (3 * 7 + 7) and s.n_chains == 2   # KLVFFAE: no glycine
    assert s.x == spec._keep[4].ctypes.data and s.hp is None and s.bptnr is None
    # sizeof and offsetof of struct dmd_system as gcc lays out include/dmd.h
    assert C.sizeof(abi.System) == 112
    assert (abi.System.boxl.offset, abi.System.x.offset, abi.System.t0.offset, abi.System.coll0.offset) == (32, 40, 96, 104)


def test_run_cfg_struct_matches_header_layout():
    """abi.RunCfg mirrors struct dmd_run_cfg (gcc layout of include/dmd.h)."""
    assert C.sizeof(abi.RunCfg) == 72
    assert (abi.RunCfg.rl_const.offset, abi.RunCfg.list_cap.offset, abi.RunCfg.flags.offset,
            abi.RunCfg.chaptype.offset, abi.RunCfg.species2_chain.offset) == (32, 56, 60, 64, 68)


def test_bead_count_rule():
    """Three backbone beads per residue and a side chain for every residue
    but glycine (code 9), over the residues the chains use."""
    from dmdgb.systems import beads_of
    rng = __import__("numpy").random.default_rng(5)
    for _ in range(20):
        cl = [int(v) for v in rng.integers(3, 12, size=rng.integers(1, 6))]
        res = [int(v) for v in rng.integers(9, 29, size=sum(cl) + int(rng.integers(0, 3)))]
        want = 0
        p = 0
        for L in cl:
            want += 3 * L + sum(1 for r in res[p:p + L] if r != 9)
            p += L
        assert beads_of(cl, res) == want
        import numpy as np
        assert beads_of(np.array(cl, np.int32), np.array(res, np.int32)) == want


def test_state_buffers_point_at_outputs():
    """The get_state arguments address the returned arrays: six float64
    columns, then bptnr, identity and the 4-wide extra_repuls block."""
    from dmdgb.engine import _state_buffers
    n = 37
    out, args, fin = _state_buffers(n)
    for q, k in enumerate(("x", "y", "z", "vx", "vy", "vz")):
        assert args[q] == out[k].ctypes.data and out[k].shape == (n,)
    assert args[6] == out["bptnr"].ctypes.data and args[7] == out["identity"].ctypes.data
    assert args[8] == out["extra_repuls"].ctypes.data and out["extra_repuls"].shape == (n, 4)
    assert out["extra_repuls"].ctypes.data + 16 * n == out["bptnr"].ctypes.data + 24 * n
    d = fin(out)
    assert d["t"] == 0.0 and d["coll"] == 0
