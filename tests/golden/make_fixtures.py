"""Writes the golden fixtures of tests/golden/ from a reference checkout.

Run here, where the reference is mounted read-only:
    python tests/golden/make_fixtures.py <reference>/parallel-dmd-PRIME20   (or set DMD_REFERENCE_DIR)

* reference_records.json: framing and sampled values of the genconfig
  output records results/run0000.config and run0000.lastvel (the known
  answer of the unformatted record reader), with the first velocity that
  genconfig/checks/velocitycheck.out prints;
* tables_digest.json: a digest of every parsed parameter table.
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300"))
import numpy as np  # noqa: E402

from dmdgb import params  # noqa: E402


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a, dtype="<f8")).tobytes()).hexdigest()


def main(ref: str) -> None:
    recs = params.read_records(os.path.join(ref, "genconfig/results/run0000.config"))
    n = (len(recs[0]) - 16) // 24
    coll, t, x, y, z = params.parse_config_record(recs[0], n)
    vrec = params.read_records(os.path.join(ref, "genconfig/results/run0000.lastvel"))
    vcoll, vx, vy, vz = params.parse_lastvel_record(vrec[0], n)
    with open(os.path.join(ref, "genconfig/checks/velocitycheck.out")) as fh:
        first = fh.readline().split()
    out = {
        "n_beads": n, "config_record_bytes": len(recs[0]), "lastvel_record_bytes": len(vrec[0]),
        "coll": coll, "t": t, "x_head": x[:8].tolist(), "x_tail": x[-8:].tolist(), "z_head": z[:8].tolist(),
        "vx_head": vx[:8].tolist(), "vz_tail": vz[-8:].tolist(),
        "config_sha256": hashlib.sha256(recs[0]).hexdigest(), "lastvel_sha256": hashlib.sha256(vrec[0]).hexdigest(),
        "velocitycheck_first": float(first[2]),
        "x_minmax": [float(x.min()), float(x.max())],
    }
    with open(os.path.join(HERE, "reference_records.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    t = params.read_tables(os.path.join(ref, "parameters"), os.path.join(ref, "parametersep/ep19p_ha55a_weakhp.data"))
    with open(os.path.join(HERE, "tables_digest.json"), "w") as fh:
        json.dump({k: digest(v) for k, v in t.__dict__.items()}, fh, indent=1)
    tstar, ncoll = params.read_run_file(os.path.join(ref, "temp_020"))
    with open(os.path.join(HERE, "run_file.json"), "w") as fh:
        json.dump({"temp_020": [tstar, ncoll]}, fh)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["DMD_REFERENCE_DIR"])
