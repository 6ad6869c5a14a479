"""Input surface of the reference PRIME20 DMD program.

Readers (and writers where the reference writes them) for the files the
reference consumes and produces, so that the GB300 engine accepts the same
inputs:

* ``parameters/`` and ``parametersep/`` tables, read with the reference's
  Fortran formats (code/inputinfo.f:103-420);
* the run file ``temp_*`` (T*, ncoll) read from stdin by the reference
  (code/main.F90:126-128);
* Fortran sequential unformatted records ``.config`` / ``.lastvel`` /
  ``.bptnr`` (code/config.f:15-40, code/inputinfo.f:75-101) and the text
  ``.energy`` line (code/main.F90:1210, format 22223).
"""
from __future__ import annotations

import json
import os
import re
import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

# residue identities 9..28 in the reference's order (code/inputinfo.f:196)
RESIDUE_LETTERS = "GRNDQEHKPSTACILMFWYV"
LETTER_TO_ID = {c: 9 + k for k, c in enumerate(RESIDUE_LETTERS)}


def _fixed(line: str, widths: Sequence[int], kinds: str) -> list:
    """Read one record with a Fortran fixed-field format.

    ``kinds``: 'x' skip, 'i' integer, 'f' real with an explicit decimal
    point (the files shipped with the reference always carry one).
    """
    out = []
    pos = 0
    for w, k in zip(widths, kinds):
        f = line[pos:pos + w]
        pos += w
        if k == "x":
            continue
        f = f.strip()
        if k == "i":
            out.append(int(f) if f else 0)
        else:
            out.append(float(f.replace("D", "E").replace("d", "e")) if f else 0.0)
    return out


def _list_directed(path: str) -> List[str]:
    """Tokens of a Fortran list-directed read (whitespace / comma separated)."""
    with open(path) as fh:
        text = fh.read()
    return [t for t in re.split(r"[\s,]+", text) if t]


def _fortran_real(tok: str) -> float:
    return float(tok.replace("D", "E").replace("d", "e"))


@dataclass
class Tables:
    """Raw parameter tables (angstrom), field for field the C struct dmd_tables."""

    sigma: np.ndarray = field(default_factory=lambda: np.zeros(4))
    welldia: np.ndarray = field(default_factory=lambda: np.zeros(4))
    epsilon: np.ndarray = field(default_factory=lambda: np.zeros(4))
    mass: np.ndarray = field(default_factory=lambda: np.zeros(29))
    bds: np.ndarray = field(default_factory=lambda: np.zeros((20, 20)))
    wel: np.ndarray = field(default_factory=lambda: np.zeros((20, 20)))
    ep: np.ndarray = field(default_factory=lambda: np.zeros((20, 20)))
    rca: np.ndarray = field(default_factory=lambda: np.zeros(20))
    rnh: np.ndarray = field(default_factory=lambda: np.zeros(20))
    rco: np.ndarray = field(default_factory=lambda: np.zeros(20))
    del_rca: np.ndarray = field(default_factory=lambda: np.zeros(20))
    del_rnh: np.ndarray = field(default_factory=lambda: np.zeros(20))
    del_rco: np.ndarray = field(default_factory=lambda: np.zeros(20))
    sqz: np.ndarray = field(default_factory=lambda: np.zeros((20, 5)))

    def to_json(self) -> dict:
        return {k: np.asarray(v).tolist() for k, v in self.__dict__.items()}

    @classmethod
    def from_json(cls, d: dict) -> "Tables":
        t = cls()
        for k, v in d.items():
            setattr(t, k, np.asarray(v, dtype=np.float64))
        return t


def read_protein_data(path: str, t: Tables) -> None:
    """code/inputinfo.f:152-178: 12 list-directed reals."""
    v = [_fortran_real(x) for x in _list_directed(path)[:12]]
    if len(v) < 12:
        raise ValueError(f"{path}: expected 12 values")
    t.sigma[:] = v[0:4]
    t.welldia[:] = v[4:8]
    t.epsilon[:] = v[8:12]


def read_mass_data(path: str, t: Tables) -> None:
    """code/inputinfo.f:416-421: 23 records '(4x,i2,2x,f8.3)'."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    n = 0
    for line in lines:
        if not line.strip():
            continue
        ident, m = _fixed(line.ljust(16), (4, 2, 2, 8), "xixf")
        if not 1 <= ident <= 28:
            raise ValueError(f"{path}: identity {ident} out of range")
        t.mass[ident] = m
        n += 1
        if n == 23:
            break
    if n < 23:
        raise ValueError(f"{path}: expected 23 records")


def read_beadwell(path: str, t: Tables) -> None:
    """code/inputinfo.f:389-397: 400 records '(2(2x,i2,2x),2(f6.3,2x))'."""
    with open(path) as fh:
        lines = [l for l in fh.read().splitlines() if l.strip()]
    if len(lines) < 400:
        raise ValueError(f"{path}: expected 400 records")
    for line in lines[:400]:
        a, b, bd, wl = _fixed(line.ljust(28), (2, 2, 2, 2, 2, 2, 6, 2, 6), "xixxixfxf")
        if not (9 <= a <= 28 and 9 <= b <= 28):
            raise ValueError(f"{path}: identity out of 9..28")
        t.bds[a - 9, b - 9] = bd
        t.wel[a - 9, b - 9] = wl


def read_ep_table(path: str, t: Tables) -> None:
    """code/inputinfo.f:280-286: 400 records '(2(2x,i2,2x),f8.3)'."""
    with open(path) as fh:
        lines = [l for l in fh.read().splitlines() if l.strip()]
    if len(lines) < 400:
        raise ValueError(f"{path}: expected 400 records")
    for line in lines[:400]:
        a, b, e = _fixed(line.ljust(20), (2, 2, 2, 2, 2, 2, 8), "xixxixf")
        if not (9 <= a <= 28 and 9 <= b <= 28):
            raise ValueError(f"{path}: identity out of 9..28")
        t.ep[a - 9, b - 9] = e


def read_rcarnrco(path: str, t: Tables) -> None:
    """code/inputinfo.f:290-296: 20 records '(6(f6.3,2x))'."""
    with open(path) as fh:
        lines = [l for l in fh.read().splitlines() if l.strip()]
    for i, line in enumerate(lines[:20]):
        v = _fixed(line.ljust(48), (6, 2) * 6, "fx" * 6)
        t.rca[i], t.rnh[i], t.rco[i], t.del_rca[i], t.del_rnh[i], t.del_rco[i] = v


def read_sqz6to10(path: str, t: Tables) -> None:
    """code/inputinfo.f:404-413: 20 records '(5(f6.3,2x))' = sz8,sz6,sz7,sz9,sz10."""
    with open(path) as fh:
        lines = [l for l in fh.read().splitlines() if l.strip()]
    for i, line in enumerate(lines[:20]):
        t.sqz[i, :] = _fixed(line.ljust(40), (6, 2) * 5, "fx" * 5)


def read_tables(parameters_dir: str, ep_file: str) -> Tables:
    """All tables the engine needs, from a reference-style parameters/ dir and
    one parametersep/ file (the reference hard-codes
    parametersep/ep19p_ha55a_weakhp.data, code/inputinfo.f:282)."""
    t = Tables()
    read_protein_data(os.path.join(parameters_dir, "protein.data"), t)
    read_mass_data(os.path.join(parameters_dir, "mass.data"), t)
    read_beadwell(os.path.join(parameters_dir, "beadwell_ha55a.data"), t)
    read_rcarnrco(os.path.join(parameters_dir, "rcarnrco.data"), t)
    read_sqz6to10(os.path.join(parameters_dir, "sqz6to10.data"), t)
    read_ep_table(ep_file, t)
    return t


_DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data")


_DEFAULT_JSON = None


def default_tables() -> Tables:
    """PRIME20 tables shipped with the package (parsed from the reference's
    parameters/ and parametersep/ep19p_ha55a_weakhp.data by
    data/make_tables.py); the file is read once per process."""
    global _DEFAULT_JSON
    if _DEFAULT_JSON is None:
        with open(os.path.join(_DATA, "prime20_tables.json")) as fh:
            _DEFAULT_JSON = json.load(fh)
    return Tables.from_json(_DEFAULT_JSON)


# ---------------------------------------------------------------- run file
def read_run_file(path: str) -> tuple:
    """temp_* file: line 1 T*, line 2 ncoll (code/main.F90:126-128)."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    tstar = _fortran_real(lines[0].split()[0])
    ncoll = int(lines[1].split()[0])
    return tstar, ncoll


# ------------------------------------------------------ species description
@dataclass
class Species:
    """One species block of the reference: chnln residues, numbeads beads per
    chain, identities per bead (identity.inp), firstside flags, hp flags."""

    chnln: int
    identity: List[int]
    firstside: List[int]
    hp: List[int]

    @property
    def numbeads(self) -> int:
        return len(self.identity)

    def residues(self) -> List[int]:
        """Residue identity per residue (9 = glycine, no side-chain bead)."""
        out, r = [], 0
        for k in range(self.chnln):
            if self.firstside[k]:
                out.append(self.identity[3 * self.chnln + r])
                r += 1
            else:
                out.append(9)
        return out


def read_species(parameters_dir: str, chnln: Sequence[int], numbeads: Sequence[int]) -> List[Species]:
    """identity.inp, firstside{1,2}.data, hp{1,2}.inp (code/inputinfo.f:103-260)."""
    ident = [int(x) for x in _list_directed(os.path.join(parameters_dir, "identity.inp"))]
    out, off = [], 0
    for s, (L, nb) in enumerate(zip(chnln, numbeads), start=1):
        fs = [int(x) for x in _list_directed(os.path.join(parameters_dir, f"firstside{s}.data"))][:L]
        hp = [int(x) for x in _list_directed(os.path.join(parameters_dir, f"hp{s}.inp"))][:nb]
        out.append(Species(L, ident[off:off + nb], fs, hp))
        off += nb
    return out


# ------------------------------------------------- unformatted record files
def read_records(path: str) -> List[bytes]:
    """Fortran sequential unformatted file: 4-byte length markers around each
    record (little endian)."""
    recs = []
    with open(path, "rb") as fh:
        data = fh.read()
    pos = 0
    while pos + 4 <= len(data):
        (n,) = struct.unpack_from("<i", data, pos)
        if n < 0 or pos + 8 + n > len(data):
            raise ValueError(f"{path}: corrupt record framing at byte {pos}")
        body = data[pos + 4:pos + 4 + n]
        (n2,) = struct.unpack_from("<i", data, pos + 4 + n)
        if n2 != n or len(body) != n:
            raise ValueError(f"{path}: corrupt record framing at byte {pos}")
        recs.append(body)
        pos += 8 + n
    if pos != len(data):
        raise ValueError(f"{path}: trailing bytes after the last record")
    return recs


def write_record(fh, payload: bytes) -> None:
    fh.write(struct.pack("<i", len(payload)))
    fh.write(payload)
    fh.write(struct.pack("<i", len(payload)))


def parse_config_record(body: bytes, n: int) -> tuple:
    """(coll, t, x, y, z) of a .config record (code/config.f:15-24)."""
    if len(body) != 16 + 24 * n:
        raise ValueError(f"config record of {len(body)} bytes does not hold {n} beads")
    coll, t = struct.unpack_from("<qd", body, 0)
    a = np.frombuffer(body, dtype="<f8", offset=16).reshape(3, n)
    return coll, t, a[0].copy(), a[1].copy(), a[2].copy()


def parse_lastvel_record(body: bytes, n: int) -> tuple:
    """(coll, vx, vy, vz) of a .lastvel record (code/config.f:31-40)."""
    if len(body) != 8 + 24 * n:
        raise ValueError(f"lastvel record of {len(body)} bytes does not hold {n} beads")
    (coll,) = struct.unpack_from("<q", body, 0)
    a = np.frombuffer(body, dtype="<f8", offset=8).reshape(3, n)
    return coll, a[0].copy(), a[1].copy(), a[2].copy()


def parse_bptnr_record(body: bytes, n: int) -> tuple:
    """(coll, bptnr) of a .bptnr record (code/config.f:25-28)."""
    if len(body) != 8 + 4 * n:
        raise ValueError(f"bptnr record of {len(body)} bytes does not hold {n} beads")
    (coll,) = struct.unpack_from("<q", body, 0)
    return coll, np.frombuffer(body, dtype="<i4", offset=8).copy()


def config_record(coll: int, t: float, x, y, z) -> bytes:
    return struct.pack("<qd", int(coll), float(t)) + np.concatenate(
        [np.asarray(x, "<f8"), np.asarray(y, "<f8"), np.asarray(z, "<f8")]).tobytes()


def lastvel_record(coll: int, vx, vy, vz) -> bytes:
    return struct.pack("<q", int(coll)) + np.concatenate(
        [np.asarray(vx, "<f8"), np.asarray(vy, "<f8"), np.asarray(vz, "<f8")]).tobytes()


def bptnr_record(coll: int, bptnr) -> bytes:
    return struct.pack("<q", int(coll)) + np.asarray(bptnr, "<i4").tobytes()


def energy_line(coll: int, tred: float, e: float, temp: float, hb_alpha: int, hb_ii: int, hb_ij: int,
                ehh_ii: float, ehh_ij: float, rg: float, e2e: float) -> str:
    """One line of the .energy file, format (i15,3f12.4,3i8,4f12.4)
    (code/main.F90:1210,1380)."""
    return "%15d%12.4f%12.4f%12.4f%8d%8d%8d%12.4f%12.4f%12.4f%12.4f" % (
        coll, tred, e, temp, hb_alpha, hb_ii, hb_ij, ehh_ii, ehh_ij, rg, e2e)


def next_run_name(results_dir: str) -> tuple:
    """runNNNN numbering of code/files_opn.f:17-46: the first NNNN whose
    .energy (or .energy.gz) is absent, and the previous one."""
    i = 0
    while True:
        name = "%04d" % i
        if not (os.path.exists(os.path.join(results_dir, f"run{name}.energy")) or
                os.path.exists(os.path.join(results_dir, f"run{name}.energy.gz"))):
            break
        i += 1
        if i > 9999:
            raise RuntimeError("too many output files")
    return "%04d" % i, "%04d" % (i - 1)
