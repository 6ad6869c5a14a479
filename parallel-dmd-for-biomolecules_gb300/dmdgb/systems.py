"""Synthetic PRIME20 systems of the shapes the benchmark configurations name.

Each builder returns a :class:`SystemSpec`: chains, sequences, box, run
settings, and (after :func:`generate`) positions and velocities from the
engine's seeded generator (dmd_generate, a restatement of the reference's
genconfig insertion and velocity steps).  There is no public dataset for
this engine; these seeded systems stand in for the reference's hand-made
genconfig runs.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import abi
from .params import LETTER_TO_ID, Tables, default_tables

AVOGADRO = 6.02214076e23
KLVFFAE = [LETTER_TO_ID[c] for c in "KLVFFAE"]  # 16 23 28 25 25 20 14 (parameters/identity.inp)


def box_for(n_chains: int, conc_mM: float) -> float:
    """Cubic box side (angstrom) holding n_chains at a concentration in mM."""
    per_a3 = conc_mM * 1e-3 * AVOGADRO / 1e27
    return (n_chains / per_a3) ** (1.0 / 3.0)


def beads_of(chain_len: List[int], residues: List[int]) -> int:
    """Beads of a system: three backbone beads per residue plus one side
    chain for every residue that is not glycine (code 9)."""
    total = int(np.sum(np.asarray(chain_len, dtype=np.int64)))
    res = np.asarray(residues[:total] if isinstance(residues, list) else np.asarray(residues)[:total])
    return 3 * total + int(np.count_nonzero(res != 9))


@dataclass
class SystemSpec:
    chain_len: List[int]
    residues: List[int]
    boxl: float
    tstar: float
    seed: int = 1
    canon: bool = True
    hbonds: bool = True
    name: str = ""
    n_events: int = 0
    x: Optional[np.ndarray] = None
    y: Optional[np.ndarray] = None
    z: Optional[np.ndarray] = None
    vx: Optional[np.ndarray] = None
    vy: Optional[np.ndarray] = None
    vz: Optional[np.ndarray] = None
    bptnr: Optional[np.ndarray] = None
    hp: Optional[np.ndarray] = None
    t0: float = 0.0
    coll0: int = 0
    chaptype: int = 1          # 2: two peptide species, chains species2_chain.. of the second
    species2_chain: int = 0
    _keep: list = field(default_factory=list, repr=False)

    @property
    def n_beads(self) -> int:
        return beads_of(self.chain_len, self.residues)

    @property
    def n_chains(self) -> int:
        return len(self.chain_len)

    def run_cfg(self, flags: int = 0, list_cap: int = 0) -> abi.RunCfg:
        return abi.RunCfg(float(self.tstar), int(self.seed), int(bool(self.canon)), int(bool(self.hbonds)),
                          2000, 2, 1.2, 5e-5, 150.0, int(list_cap), int(flags), int(self.chaptype),
                          int(self.species2_chain))

    def c_system(self) -> abi.System:
        """C view of this system; the arrays stay referenced by the spec."""
        if self.x is None:
            raise ValueError("positions missing: call generate() first")
        cl = np.ascontiguousarray(self.chain_len, np.int32)
        res = np.ascontiguousarray(self.residues, np.int32)
        arrs = [np.ascontiguousarray(a, np.float64) for a in (self.x, self.y, self.z, self.vx, self.vy, self.vz)]
        hp = None if self.hp is None else np.ascontiguousarray(self.hp, np.int32)
        bp = None if self.bptnr is None else np.ascontiguousarray(self.bptnr, np.int32)
        self._keep = [cl, res, hp, bp] + arrs
        def addr(a):
            return None if a is None else a.ctypes.data
        return abi.System(beads_of(cl, res), len(cl), addr(cl), addr(res), addr(hp), float(self.boxl),
                          *[addr(a) for a in arrs], addr(bp), float(self.t0), int(self.coll0))


def generate(spec: SystemSpec, tables: Optional[Tables] = None, min_sep: float = 5.0, lib=None) -> SystemSpec:
    """Seeded positions and velocities from dmd_generate: the engine
    library's, or that of another library that exports it (lib, a ctypes
    CDLL with abi's declaration of dmd_generate)."""
    lib = lib or abi.load_engine()
    t = abi.tables_struct(tables or default_tables())
    n = spec.n_beads
    arrs = [np.zeros(n) for _ in range(6)]
    cl = np.ascontiguousarray(spec.chain_len, np.int32)
    res = np.ascontiguousarray(spec.residues, np.int32)
    g = abi.GenSpec(len(cl), abi.ptr(cl, abi.i32_p), abi.ptr(res, abi.i32_p), float(spec.boxl), float(spec.tstar),
                    int(spec.seed), float(min_sep))
    err = C.create_string_buffer(256)
    rc = lib.dmd_generate(C.byref(g), C.byref(t), n, *[abi.ptr(a, abi.dbl_p) for a in arrs], err, 256)
    if rc != 0:
        raise RuntimeError(f"dmd_generate failed: {err.value.decode()}")
    spec.x, spec.y, spec.z, spec.vx, spec.vy, spec.vz = arrs
    return spec


def sidechain_search(ca, nh, co, side, residues, move: float = 3.5, step: float = 0.005,
                     tables: Optional[Tables] = None):
    """The initial-configuration generator's side-chain placement search
    (genconfig/gen_config_random-SQZ.f90:250-348) on the GPU, for the
    consecutive residues of one chain: positions [n, 3] in angstrom
    (C-alpha, NH, CO, side-chain start), identities 9..28.  Returns the moved
    side chains [n, 3], each residue's r3 and its winning grid point (-1:
    none admissible, side chain left at its start)."""
    lib = abi.load_engine()
    ca, nh, co, side = [np.ascontiguousarray(a, np.float64).reshape(-1, 3) for a in (ca, nh, co, side)]
    res = np.ascontiguousarray(residues, np.int32)
    n = len(res)
    if not (len(ca) == len(nh) == len(co) == len(side) == n):
        raise ValueError("one C-alpha, NH, CO and side-chain position per residue")
    t = abi.tables_struct(tables or default_tables())
    out = np.zeros((n, 3))
    rmin = np.zeros(n)
    idx = np.zeros(n, np.int64)
    err = C.create_string_buffer(256)
    rc = lib.dmd_sidechain_search(n, ca.ctypes.data, nh.ctypes.data, co.ctypes.data, side.ctypes.data,
                                  res.ctypes.data, C.byref(t), float(move), float(step), out.ctypes.data,
                                  rmin.ctypes.data, idx.ctypes.data, err, 256)
    if rc != 0:
        raise RuntimeError(f"dmd_sidechain_search failed ({abi.ERRORS.get(rc, rc)}): {err.value.decode()}")
    return out, rmin, idx


def random_sequence(rng: np.random.Generator, length: int) -> List[int]:
    """Residue identities uniform over the 20 PRIME20 types (9..28)."""
    return [int(v) for v in rng.integers(9, 29, size=length)]


# ----------------------------------------------------------- configurations
def klvffae_system(n_chains: int, conc_mM: float, tstar: float, seed: int, n_events: int = 0,
                   name: str = "") -> SystemSpec:
    return SystemSpec([7] * n_chains, KLVFFAE * n_chains, box_for(n_chains, conc_mM), tstar, seed,
                      name=name or f"{n_chains}xKLVFFAE", n_events=n_events)


def config_c1(seed: int = 1) -> SystemSpec:
    """8 x KLVFFAE (224 beads), 5 mM (box 138.5 A), T* = 0.20, Andersen, 1e6 events."""
    return klvffae_system(8, 5.0, 0.20, seed, 10**6, "C1: 8xKLVFFAE 5mM T*=0.20")


def config_c2(seed: int = 1) -> SystemSpec:
    """48 x KLVFFAE (1,344 beads), 5 mM (box 251.7 A), T* = 0.18, 1e8 events."""
    return klvffae_system(48, 5.0, 0.18, seed, 10**8, "C2: 48xKLVFFAE 5mM T*=0.18")


def config_c3(n_replicas: int = 32, seed: int = 1) -> List[SystemSpec]:
    """Replica r: T* = 0.18 + r*0.32/31, a seeded count of 8..96 chains of
    random 16-residue sequences at 5 mM, 1e7 events each."""
    out = []
    for r in range(n_replicas):
        rng = np.random.default_rng([seed, r])
        nch = int(rng.integers(8, 97))
        res = []
        for _ in range(nch):
            res += random_sequence(rng, 16)
        tstar = 0.18 + r * (0.32 / 31.0) if n_replicas > 1 else 0.18
        out.append(SystemSpec([16] * nch, res, box_for(nch, 5.0), tstar, seed * 1000 + r,
                              name=f"C3 replica {r}: {nch}x16 T*={tstar:.3f}", n_events=10**7))
    return out


def config_c4(seed: int = 1, n_chains: int = 1000) -> SystemSpec:
    """1,000 chains of one seeded random 10-mer (about 40,000 beads), 10 mM, T* = 0.22."""
    rng = np.random.default_rng([seed, 4])
    seq = random_sequence(rng, 10)
    return SystemSpec([10] * n_chains, seq * n_chains, box_for(n_chains, 10.0), 0.22, seed,
                      name=f"C4: {n_chains}x10-mer 10mM T*=0.22", n_events=10**8)


def extended_length(L: int) -> float:
    """Largest extent (angstrom) of the generator's extended chain of L residues."""
    return 3.45 * L + 10.0


def serving_request(k: int, seed: int = 1) -> SystemSpec:
    """Request k of the serving trace: 4-200 chains of 6-40 residues, residues
    uniform over the 20 types, 2-10 mM, T* in 0.15-0.30, 1e6-1e7 events.
    The box is widened when the extended chains would not fit (the generator
    places straight chains)."""
    rng = np.random.default_rng([seed, 5, k])
    nch = int(rng.integers(4, 201))
    L = int(rng.integers(6, 41))
    conc = float(rng.uniform(2.0, 10.0))
    tstar = float(rng.uniform(0.15, 0.30))
    nev = int(rng.integers(10**6, 10**7 + 1))
    res = []
    for _ in range(nch):
        res += random_sequence(rng, L)
    box = max(box_for(nch, conc), extended_length(L) + 15.0)
    return SystemSpec([L] * nch, res, box, tstar, seed * 100000 + k, name=f"request {k}: {nch}x{L}",
                      n_events=nev)
