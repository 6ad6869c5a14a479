"""Command-line driver in the place of the reference's ``program dmd``
(code/main.F90:117-1380): read the run file, the parameter tables, the
species description and the starting records; run on the GPU engine,
returning at every output event to append the reference's output records;
write a checkpoint of the whole engine state at the end.

    python -m dmdgb.run --params parameters --ep parametersep/ep19p_ha55a_weakhp.data \\
        --temp temp_020 --species 8:7 --start genconfig/results/run0000 --results results

The species are the compile-time constants of the reference's def.h
(``nop1:chnln1[,nop2:chnln2]``: chain count and residues per chain).  With
``--restart NNNN`` the run continues from the last records of
results/runNNNN.{config,lastvel,bptnr} (the reference's runr path,
code/main.F90:240-321: lists, queue and intervals are rebuilt); with
``--resume FILE`` it continues bit-identically from a checkpoint written by
an earlier run of this driver on the same system.
"""
from __future__ import annotations

import argparse
import os
import sys
from typing import List, Optional, Tuple

import numpy as np

from . import abi, params
from .engine import Engine
from .systems import SystemSpec


def parse_species(text: str) -> List[Tuple[int, int]]:
    out = []
    for part in text.split(","):
        nop, chnln = part.split(":")
        out.append((int(nop), int(chnln)))
    return out


def build_spec(params_dir: str, species: List[Tuple[int, int]], tstar: float, boxl: float) -> SystemSpec:
    """Chains, residues and hydrophobic flags from identity.inp,
    firstside{s}.data and hp{s}.inp (code/inputinfo.f:103-260)."""
    chnln = [L for _, L in species]
    numbeads = []
    fs_all = []
    for s, (_, L) in enumerate(species, start=1):
        fs = [int(x) for x in params._list_directed(os.path.join(params_dir, f"firstside{s}.data"))][:L]
        fs_all.append(fs)
        numbeads.append(3 * L + sum(1 for f in fs if f))
    sp = params.read_species(params_dir, chnln, numbeads)
    chain_len, residues, hp = [], [], []
    for (nop, L), S in zip(species, sp):
        for _ in range(nop):
            chain_len.append(L)
            residues += S.residues()
            hp += S.hp
    return SystemSpec(chain_len, residues, boxl, tstar, hp=np.asarray(hp, np.int32))


def last_records(prefix: str, n: int, need_bptnr: bool) -> tuple:
    """The last .config/.lastvel (and .bptnr) records of a run prefix."""
    cfg = params.read_records(prefix + ".config")
    coll, t, x, y, z = params.parse_config_record(cfg[-1], n)
    _, vx, vy, vz = params.parse_lastvel_record(params.read_records(prefix + ".lastvel")[-1], n)
    bp = None
    if need_bptnr and os.path.exists(prefix + ".bptnr"):
        _, bp = params.parse_bptnr_record(params.read_records(prefix + ".bptnr")[-1], n)
    return coll, t, x, y, z, vx, vy, vz, bp


def append_outputs(prefix: str, eng: Engine, tstar: float, sigma1: float) -> dict:
    """The records code/config.f writes at an output event (positions at the
    current time, x + vx*tfalse, appended to .config and .bptnr; the last
    velocities replace .lastvel) and the .energy line of code/main.F90:1210
    (time in reduced units (t + tfalse) * sqrt(12 T*) / sigma(1))."""
    st = eng.state()
    tf = st["tfalse"]
    x, y, z = st["x"] + st["vx"] * tf, st["y"] + st["vy"] * tf, st["z"] + st["vz"] * tf
    coll = st["coll"]
    with open(prefix + ".config", "ab") as fh:
        params.write_record(fh, params.config_record(coll, st["t"] + tf, x, y, z))
    with open(prefix + ".lastvel", "wb") as fh:
        params.write_record(fh, params.lastvel_record(coll, st["vx"], st["vy"], st["vz"]))
    with open(prefix + ".bptnr", "ab") as fh:
        params.write_record(fh, params.bptnr_record(coll, st["bptnr"]))
    d = eng.diagnostics()
    t_red = (st["t"] + tf) * np.sqrt(12.0 * tstar) / sigma1
    with open(prefix + ".energy", "a") as fh:
        fh.write(params.energy_line(coll, t_red, d["e_total"], d["temperature"], d["hb_alpha"], d["hb_ii"],
                                    d["hb_ij"], d["ehh_ii"], d["ehh_ij"], d["rg"], d["e2e"]) + "\n")
    return d


def main(argv: Optional[List[str]] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--params", help="the reference's parameters/ directory (default: the built-in PRIME20 tables)")
    ap.add_argument("--ep", help="the parametersep/ep*.data table (with --params)")
    ap.add_argument("--temp", required=True, help="run file: T* on line 1, collisions on line 2")
    ap.add_argument("--species", help="nop1:chnln1[,nop2:chnln2] (with --params: identity.inp, firstside, hp)")
    ap.add_argument("--sequence", help="instead of --species: N:id,id,... (N chains of these residue identities 9-28)")
    ap.add_argument("--results", required=True, help="output directory (runNNNN.* files)")
    g = ap.add_mutually_exclusive_group(required=True)
    g.add_argument("--start", help="records prefix of a starting configuration (e.g. genconfig .../run0000)")
    g.add_argument("--restart", help="NNNN: continue from results/runNNNN's last records")
    ap.add_argument("--resume", help="checkpoint file of an earlier run of this driver (bit-identical continuation)")
    ap.add_argument("--boxl", type=float, default=0.0, help="box side in Angstrom (default: from the records' run)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-thermostat", action="store_true")
    ap.add_argument("--checkpoint", help="write the engine state here at the end")
    a = ap.parse_args(argv)

    tstar, ncoll = params.read_run_file(a.temp)
    tables = params.read_tables(a.params, a.ep) if a.params else params.default_tables()
    os.makedirs(a.results, exist_ok=True)
    if a.restart:
        prefix_in = os.path.join(a.results, f"run{a.restart}")
    else:
        prefix_in = a.start
    if a.boxl <= 0:
        raise SystemExit("--boxl is required (the records hold positions in box units)")
    if a.sequence:
        nch, ids = a.sequence.split(":")
        seq = [int(v) for v in ids.split(",")]
        spec = SystemSpec([len(seq)] * int(nch), seq * int(nch), a.boxl, tstar)
    elif a.species and a.params:
        spec = build_spec(a.params, parse_species(a.species), tstar, a.boxl)
    else:
        raise SystemExit("give --sequence, or --species with --params")
    spec.seed = a.seed
    spec.canon = not a.no_thermostat
    coll, t, x, y, z, vx, vy, vz, bp = last_records(prefix_in, spec.n_beads, need_bptnr=bool(a.restart))
    spec.x, spec.y, spec.z, spec.vx, spec.vy, spec.vz = x, y, z, vx, vy, vz
    spec.bptnr = bp
    spec.t0, spec.coll0 = (t, coll) if a.restart else (0.0, 0)
    name, _ = params.next_run_name(a.results)
    prefix = os.path.join(a.results, f"run{name}")
    d = None
    with Engine(spec, tables=tables, flags=abi.FLAG_STOP_AT_OUTPUT) as eng:
        if a.resume:
            with open(a.resume, "rb") as fh:
                eng.load_state(fh.read())
        while True:
            left = ncoll - eng.state()["coll"]
            if left <= 0:
                break
            eng.run(left)                          # returns at every output event
            d = append_outputs(prefix, eng, tstar, float(tables.sigma[0]))
        if a.checkpoint:
            with open(a.checkpoint, "wb") as fh:
                fh.write(eng.save_state())
    if d is not None:
        print(f"run{name}: {ncoll} collisions, E = {d['e_total']:.4f}, T = {d['temperature']:.4f}", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
