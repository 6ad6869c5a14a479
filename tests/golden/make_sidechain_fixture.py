"""Writes tests/golden/sidechain_template.json: the known answer of the
side-chain placement search of the reference's initial-configuration
generator (genconfig/gen_config_random-SQZ.f90:250-348).

Run here, where the reference is mounted read-only:
    python tests/golden/make_sidechain_fixture.py <reference>/parallel-dmd-PRIME20   (or set DMD_REFERENCE_DIR)

The inputs are the generator's own: its 31-residue template chain
(genconfig/inputs/peptide{x,y,z}.inp: C-alpha, NH, CO and side-chain beads
in angstrom) and the side-chain identities of genconfig/inputs/identity.inp.
The generator's compile-time chain length is 22 (gen_config_random-SQZ.f90:10),
so residues 1-22 of the template are searched; each side chain starts on the
line from its C-alpha through the template's side chain at the C-alpha
pseudo-bond length (:233-242).  The identities of that run are the last 22
of the 31 that identity.inp lists (the file holds the 31-residue template's
sequence): every side chain of configone1.pdb sits at exactly those
residues' three pseudo-bond lengths (r3 <= 0.004 A), with the glycines at
residues 1, 6, 12 and 16 that make its 84 beads.  The expected result is the generator's own
output genconfig/checks/configone1.pdb (the first species after the search,
glycine side chains dropped, coordinates to 3 decimals).  The oracle's full
search (1,401^3 grid points per residue, one process per residue) is
checked against it here and stored beside it, so that the tests can compare
the GPU search with both without the reference.
"""
import json
import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300"))
import numpy as np  # noqa: E402

CHNLN = 22       # gen_config_random-SQZ.f90:10
CHNLN1P = 31     # :8, the template's length
MOVE, STEP = 3.5, 0.005   # :230, :252


def list_directed(path):
    with open(path) as fh:
        return fh.read().replace(",", " ").split()


def read_template(ref):
    xyz = []
    for a in "xyz":
        v = list_directed(os.path.join(ref, f"genconfig/inputs/peptide{a}.inp"))
        n = int(v[0])
        xyz.append(np.array([float(s.replace("D", "E").replace("d", "e")) for s in v[2:2 + n]]))
    return np.stack(xyz, axis=1)          # [124, 3]


def read_table_rows(path, ncol):
    rows = []
    with open(path) as fh:
        for line in fh:
            f = line.split()
            if len(f) >= ncol:
                rows.append([float(s) for s in f[:ncol]])
    return np.array(rows[:20])


def read_pdb(path):
    out = []
    with open(path) as fh:
        next(fh)
        for line in fh:
            if line.startswith("atom"):
                t = line.rstrip("\n")[-24:]
                out.append([float(t[0:8]), float(t[8:16]), float(t[16:24])])
    return np.array(out)


def generator_tables(rcarn, sqz):
    """The engine's tables with the generator's own copies of rcarnrco.data
    and sqz6to10.data (they differ from the simulation's in a few entries)."""
    from dmdgb.params import default_tables
    t = default_tables()
    t.rca, t.rnh, t.rco = rcarn[:, 0].copy(), rcarn[:, 1].copy(), rcarn[:, 2].copy()
    t.sqz = sqz.copy()
    return t


def search_one(args):
    k, ca, nh, co, side, res, rcarn, sqz = args
    from oracle import oracle as ora
    out, rmin, idx = ora.sidechain_search(ca, nh, co, side, res, MOVE, STEP, tables=generator_tables(rcarn, sqz),
                                          only=(k, k + 1))
    return k, out[k].tolist(), float(rmin[k]), int(idx[k])


def main(ref):
    rcarn = read_table_rows(os.path.join(ref, "genconfig/parameters/rcarnrco.data"), 6)
    sqz = read_table_rows(os.path.join(ref, "genconfig/parameters/sqz6to10.data"), 5)
    tab = generator_tables(rcarn, sqz)
    tpl = read_template(ref)
    ids = [int(s) for s in list_directed(os.path.join(ref, "genconfig/inputs/identity.inp"))]
    seq = ids[4 * CHNLN1P - CHNLN:4 * CHNLN1P]
    ca, nh, co = tpl[0:CHNLN], tpl[CHNLN1P:CHNLN1P + CHNLN], tpl[2 * CHNLN1P:2 * CHNLN1P + CHNLN]
    sc_t = tpl[3 * CHNLN1P:3 * CHNLN1P + CHNLN]
    side = np.zeros((CHNLN, 3))
    for k in range(CHNLN):            # :233-242, in the reference's operation order
        r2 = sc_t[k] - ca[k]
        scale = tab.rca[seq[k] - 9] / np.sqrt(r2[0] ** 2 + r2[1] ** 2 + r2[2] ** 2)
        side[k] = ca[k] + scale * r2
    pdb = read_pdb(os.path.join(ref, "genconfig/checks/configone1.pdb"))
    nongly = [k for k in range(CHNLN) if seq[k] != 9]
    assert len(pdb) == 3 * CHNLN + len(nongly)
    assert np.abs(pdb[:CHNLN] - ca).max() < 6e-4 and np.abs(pdb[2 * CHNLN:3 * CHNLN] - co).max() < 6e-4
    expected = pdb[3 * CHNLN:]
    work = [(k, ca, nh, co, side, seq, rcarn, sqz) for k in range(CHNLN)]
    with mp.get_context("spawn").Pool(min(len(work), os.cpu_count() or 1)) as pool:
        res = sorted(pool.map(search_one, work))
    side_out = np.array([r[1] for r in res])
    rmin = [r[2] for r in res]
    index = [r[3] for r in res]
    dev = np.abs(side_out[nongly] - expected).max()
    print(f"oracle vs configone1.pdb: largest deviation {dev:.6f} A over {len(nongly)} side chains")
    out = {
        "source": "genconfig/inputs/peptide{x,y,z}.inp, identity.inp; genconfig/checks/configone1.pdb",
        "move": MOVE, "step": STEP, "residues": seq,
        "rca": rcarn[:, 0].tolist(), "rnh": rcarn[:, 1].tolist(), "rco": rcarn[:, 2].tolist(), "sqz": sqz.tolist(),
        "ca": ca.tolist(), "nh": nh.tolist(), "co": co.tolist(), "side_start": side.tolist(),
        "configone1_side": expected.tolist(), "configone1_residues": nongly,
        "oracle_side": side_out.tolist(), "oracle_rmin": rmin, "oracle_index": index,
        "oracle_vs_configone1_max_dev": dev,
    }
    with open(os.path.join(HERE, "sidechain_template.json"), "w") as fh:
        json.dump(out, fh, indent=0)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["DMD_REFERENCE_DIR"])
