"""The command-line driver in the place of program dmd: reference records in,
reference records out, and a checkpoint that resumes bit-identically."""
import os

import numpy as np
import pytest

from dmdgb import params, systems
from dmdgb.run import main


def _start_records(tmp, spec):
    prefix = os.path.join(tmp, "start")
    with open(prefix + ".config", "wb") as fh:
        params.write_record(fh, params.config_record(0, 0.0, spec.x, spec.y, spec.z))
    with open(prefix + ".lastvel", "wb") as fh:
        params.write_record(fh, params.lastvel_record(0, spec.vx, spec.vy, spec.vz))
    return prefix


def _temp(tmp, name, tstar, ncoll):
    p = os.path.join(tmp, name)
    with open(p, "w") as fh:
        fh.write(f"{tstar}\n{ncoll}\n")
    return p


def test_parse_species():
    from dmdgb.run import parse_species
    assert parse_species("8:7") == [(8, 7)]
    assert parse_species("4:16,2:10") == [(4, 16), (2, 10)]


@pytest.mark.gpu
def test_driver_records_and_resume(built, tmp_path):
    spec = systems.generate(systems.config_c1())
    seq = ",".join(str(r) for r in systems.KLVFFAE)
    start = _start_records(str(tmp_path), spec)
    common = ["--sequence", f"8:{seq}", "--boxl", str(spec.boxl), "--start", start]
    # straight: 9,000 collisions
    d1 = tmp_path / "straight"
    assert main(["--temp", _temp(str(tmp_path), "t9000", spec.tstar, 9000), "--results", str(d1)] + common) == 0
    # split: 4,000 with a checkpoint, then resumed to 9,000
    d2 = tmp_path / "split"
    ck = str(tmp_path / "ck.bin")
    assert main(["--temp", _temp(str(tmp_path), "t4000", spec.tstar, 4000), "--results", str(d2),
                 "--checkpoint", ck] + common) == 0
    assert main(["--temp", _temp(str(tmp_path), "t9000b", spec.tstar, 9000), "--results", str(d2),
                 "--resume", ck] + common) == 0
    a = params.read_records(str(d1 / "run0000.config"))
    b = params.read_records(str(d2 / "run0001.config"))
    assert a[-1] == b[-1]                                  # the last configuration, byte for byte
    va = params.read_records(str(d1 / "run0000.lastvel"))
    vb = params.read_records(str(d2 / "run0001.lastvel"))
    assert len(va) == 1 and va[0] == vb[0]
    lines = open(d1 / "run0000.energy").read().splitlines()
    assert len(lines) == len(a) and int(lines[-1][:15]) == 9000
