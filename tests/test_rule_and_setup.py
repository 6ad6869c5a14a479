"""The engine's pair-type rule against the literal dense restatement of
code/make_code.f, and the set-up values (intervals, cutoffs) against the
restatement of code/main.F90:144-156 and code/nbor_setup.f.  CPU only: the
engine exposes both through host-only ABI calls."""
import ctypes as C

import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.params import default_tables
from helpers import dense_system
from oracle.oracle import Oracle


def _engine_static(spec):
    lib = abi.load_engine()
    t = abi.tables_struct(default_tables())
    cfg = spec.run_cfg()
    s = spec.c_system()
    out = np.zeros((spec.n_beads, spec.n_beads), np.int8)
    err = C.create_string_buffer(256)
    rc = lib.dmd_static_evcode(C.byref(cfg), C.byref(t), C.byref(s), out.ctypes.data_as(abi.i8_p), err, 256)
    assert rc == 0, err.value
    return out


def _engine_inspect(spec):
    lib = abi.load_engine()
    t = abi.tables_struct(default_tables())
    cfg = spec.run_cfg()
    s = spec.c_system()
    out = np.zeros(16)
    err = C.create_string_buffer(256)
    m = lib.dmd_inspect(C.byref(cfg), C.byref(t), C.byref(s), abi.ptr(out, abi.dbl_p), 16, err, 256)
    assert m > 0, err.value
    keys = ["interval", "interval_max", "sig_max_all", "hdelr", "ncell", "rl", "rlsq1", "rlsq15", "rlsq16",
            "rlsq40", "n_forced", "t_fact", "evp1_15"]
    return dict(zip(keys, out[:m].tolist()))


def _mixed(seed, n_chains=5, lens=(6, 9, 12, 7, 16), hbonds=True):
    rng = np.random.default_rng(seed)
    L = [lens[k % len(lens)] for k in range(n_chains)]
    res = []
    for ln in L:
        seq = systems.random_sequence(rng, ln)
        seq[rng.integers(0, ln)] = 17   # at least one proline
        seq[rng.integers(0, ln)] = 9    # and one glycine
        res += seq
    spec = systems.SystemSpec(L, res, 90.0, 0.2, seed, hbonds=hbonds)
    return systems.generate(spec, min_sep=4.0)


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_rule_equals_literal_make_code(seed):
    spec = _mixed(seed)
    ora = Oracle(spec)
    assert np.array_equal(_engine_static(spec), ora.evcode())


def test_rule_no_hbonds():
    spec = _mixed(7, hbonds=False)
    assert np.array_equal(_engine_static(spec), Oracle(spec).evcode())


def test_rule_klvffae_two_species_layout():
    """The reference's shipped build: 48 chains of KLVFFAE in two identical
    species blocks; codes 4-12, 15-26 as code/make_code.f lays them out."""
    spec = systems.generate(systems.klvffae_system(6, 5.0, 0.2, 1))
    ev = _engine_static(spec)
    assert np.array_equal(ev, Oracle(spec).evcode())
    L, s = 7, 0
    assert ev[s + 0, s + L + 0] == 4 and ev[s + 0, s + 2 * L + 0] == 5 and ev[s + 0, s + 1] == 9
    assert ev[s + 0, s + 3 * L] == 10 and ev[s + L, s + 3 * L] == 11 and ev[s + 2 * L, s + 3 * L] == 12
    assert ev[s + L + 0, s + 2 * L + 4] == 15 and ev[s + L + 0, s + 2 * L + 3] == 1
    assert ev[s + 3 * L, 28 + 3 * L] == 16            # side chains of two chains
    assert ev[s + L + 0, 28 + 2 * L + 0] == 15        # NH-CO of two chains
    assert np.array_equal(ev, ev.T)


@pytest.mark.parametrize("maker", ["c1", "dense", "mixed"])
def test_setup_values_match(maker):
    spec = {"c1": lambda: systems.generate(systems.config_c1()), "dense": lambda: dense_system(),
            "mixed": lambda: _mixed(5)}[maker]()
    e = _engine_inspect(spec)
    o = Oracle(spec).scalars()
    for k in ("interval", "interval_max", "sig_max_all", "hdelr", "rlsq1", "rlsq15", "rlsq16", "rlsq40", "evp1_15"):
        assert e[k] == o[k], k


def _two_species(seed, split=3):
    """A mixed system run with -Dchaptype=2: chains split.. are species 2."""
    spec = _mixed(seed, n_chains=6, lens=(8, 10, 12))
    spec.chaptype = 2
    spec.species2_chain = split
    return spec


def _chain_of_beads(spec):
    out, p = [], 0
    for c, L in enumerate(spec.chain_len):
        res = spec.residues[p:p + L]
        out += [c] * (3 * L + sum(1 for r in res if r != 9))
        p += L
    return np.asarray(out)


@pytest.mark.parametrize("seed,split", [(11, 3), (12, 0), (13, 6)])
def test_rule_two_species_equals_literal_make_code(seed, split):
    """code/make_code.f:489-548: side chains of two different species-2
    chains meet as hard cores; species 1 and mixed pairs keep the well."""
    import dataclasses
    spec = _two_species(seed, split)
    ev = _engine_static(spec)
    assert np.array_equal(ev, Oracle(spec).evcode())
    ev1 = _engine_static(dataclasses.replace(spec, chaptype=1))
    chain = _chain_of_beads(spec)
    diff = np.argwhere(ev != ev1)
    for a, b in diff:                        # every change: 16 -> 1 between two species-2 chains
        assert (ev1[a, b], ev[a, b]) == (16, 1)
        assert chain[a] != chain[b] and chain[a] >= split and chain[b] >= split
    if split <= 4:
        assert len(diff) > 0


def test_setup_values_two_species():
    spec = _two_species(14, 2)
    e = _engine_inspect(spec)
    o = Oracle(spec).scalars()
    for k in ("interval", "interval_max", "sig_max_all", "hdelr", "rlsq1", "rlsq15", "rlsq16", "rlsq40", "evp1_15"):
        assert e[k] == o[k], k


def test_chaptype_is_checked():
    spec = _two_species(15, 2)
    spec.species2_chain = 99
    lib = abi.load_engine()
    t = abi.tables_struct(default_tables())
    cfg = spec.run_cfg()
    s = spec.c_system()
    out = np.zeros((spec.n_beads, spec.n_beads), np.int8)
    err = C.create_string_buffer(256)
    assert lib.dmd_static_evcode(C.byref(cfg), C.byref(t), C.byref(s), out.ctypes.data_as(abi.i8_p), err, 256) == -1
    assert b"species2_chain" in err.value
