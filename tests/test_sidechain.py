"""The initial-configuration generator's side-chain placement search
(genconfig/gen_config_random-SQZ.f90:250-348): the CPU restatement against
the reference's own output (tests/golden/sidechain_template.json, made by
make_sidechain_fixture.py from genconfig's template and configone1.pdb) and
a literal restatement, and dmd_sidechain_search on the GPU against both."""
import json
import os

import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.params import default_tables
from oracle import oracle as ora

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sidechain_template.json")


def fixture():
    with open(GOLD) as fh:
        d = json.load(fh)
    t = default_tables()
    t.rca, t.rnh, t.rco = np.array(d["rca"]), np.array(d["rnh"]), np.array(d["rco"])
    t.sqz = np.array(d["sqz"])
    arr = {k: np.array(d[k]) for k in ("ca", "nh", "co", "side_start", "oracle_side", "configone1_side")}
    return d, t, arr


def literal_search(ca, nh, co, side, res, t, move, step):
    """gen_config_random-SQZ.f90:250-319 written out loop by loop (small grids)."""
    m = int((move - (-move) + step) / step)
    D = []
    d = -move
    for _ in range(m):
        D.append(d)
        d = d + step
    n = len(res)
    out, rmins, idxs = side.copy(), [], []
    for k in range(n):
        row = res[k] - 9
        S = side[k]
        rmin, best = 100.0, -1
        for i1, d1 in enumerate(D):
            for i2, d2 in enumerate(D):
                for i3, d3 in enumerate(D):
                    p = (S[0] + d1, S[1] + d2, S[2] + d3)

                    def dist(R):
                        a, b, c = p[0] - R[0], p[1] - R[1], p[2] - R[2]
                        return np.sqrt(a * a + b * b + c * c)
                    r3 = abs(t.rca[row] - dist(ca[k])) + abs(t.rnh[row] - dist(nh[k])) + abs(t.rco[row] - dist(co[k]))
                    isz = False
                    if k >= 1 and (dist(co[k - 1]) < t.sqz[row][1] or dist(ca[k - 1]) < t.sqz[row][0]):
                        isz = True
                    if k + 1 < n and (dist(nh[k + 1]) < t.sqz[row][2] or dist(ca[k + 1]) < t.sqz[row][3]):
                        isz = True
                    if r3 < rmin and not isz:
                        rmin, best = r3, (i1 * m + i2) * m + i3
        if best >= 0:
            out[k] = S + np.array([D[best // (m * m)], D[(best // m) % m], D[best % m]])
        rmins.append(rmin)
        idxs.append(best)
    return out, np.array(rmins), np.array(idxs)


def test_grid_is_the_fortran_loop():
    """Trip count INT((2 move + step) / step), values by repeated addition."""
    g = ora.sidechain_grid(3.5, 0.005)
    assert len(g) == 1401 and g[0] == -3.5
    d = -3.5
    for k in range(1401):
        assert g[k] == d
        d = d + 0.005
    assert len(ora.sidechain_grid(0.5, 0.005)) == 200   # 1.005 / 0.005 rounds just below 201


def test_oracle_matches_literal_restatement():
    d, t, a = fixture()
    res = d["residues"][:4]
    rng = np.random.default_rng(3)
    side = a["side_start"][:4] + rng.normal(0, 0.4, (4, 3))
    for move, step in ((0.03, 0.005), (0.02, 0.0075)):
        want = literal_search(a["ca"][:4], a["nh"][:4], a["co"][:4], side, res, t, move, step)
        got = ora.sidechain_search(a["ca"][:4], a["nh"][:4], a["co"][:4], side, res, move, step, tables=t)
        assert np.array_equal(got[2], want[2]) and np.array_equal(got[1], want[1]) and np.array_equal(got[0], want[0])


def test_fixture_pins_the_reference_output():
    """The oracle's full search (1,401^3 points per residue, run when the
    fixture was made) reproduces configone1.pdb to its 3 decimals, and every
    stored winner gives the stored r3 and is admissible."""
    d, t, a = fixture()
    nongly = d["configone1_residues"]
    assert len(nongly) == 18 and np.abs(a["oracle_side"][nongly] - a["configone1_side"]).max() <= 5e-4
    g = ora.sidechain_grid(d["move"], d["step"])
    m = len(g)
    res = d["residues"]
    for k, (idx, rmin) in enumerate(zip(d["oracle_index"], d["oracle_rmin"])):
        assert idx >= 0 and rmin < 0.01
        off = np.array([g[idx // (m * m)], g[(idx // m) % m], g[idx % m]])
        assert np.array_equal(a["side_start"][k] + off, a["oracle_side"][k])
        p = a["side_start"][k] + off   # the same sums as S + d per axis

        def dist(R):
            x, y, z = p[0] - R[0], p[1] - R[1], p[2] - R[2]
            return np.sqrt(x * x + y * y + z * z)
        row = res[k] - 9
        r3 = abs(t.rca[row] - dist(a["ca"][k])) + abs(t.rnh[row] - dist(a["nh"][k])) + abs(t.rco[row] - dist(a["co"][k]))
        assert r3 == rmin


def test_bad_input_is_rejected_before_the_device(built):
    """Input errors return DMD_E_INPUT with a message and touch no GPU."""
    d, t, a = fixture()
    with pytest.raises(RuntimeError, match="identity"):
        systems.sidechain_search(a["ca"][:2], a["nh"][:2], a["co"][:2], a["side_start"][:2], [5, 28], tables=t)
    with pytest.raises(RuntimeError, match="step"):
        systems.sidechain_search(a["ca"][:2], a["nh"][:2], a["co"][:2], a["side_start"][:2], [9, 28], step=0.0, tables=t)
    with pytest.raises(RuntimeError, match="4096"):
        systems.sidechain_search(a["ca"][:2], a["nh"][:2], a["co"][:2], a["side_start"][:2], [9, 28], move=30.0,
                                 step=0.005, tables=t)
    assert abi.load_engine().dmd_sidechain_grid(3.5, 0.005) == 1401


@pytest.mark.gpu
def test_gpu_search_reproduces_the_reference_template(built):
    """The full search of the generator's 22-residue template on the GPU:
    the oracle's winners bit for bit, configone1.pdb to its 3 decimals."""
    d, t, a = fixture()
    out, rmin, idx = systems.sidechain_search(a["ca"], a["nh"], a["co"], a["side_start"], d["residues"], d["move"],
                                              d["step"], tables=t)
    assert np.array_equal(idx, np.array(d["oracle_index"]))
    assert np.array_equal(rmin, np.array(d["oracle_rmin"]))
    assert np.array_equal(out, a["oracle_side"])
    assert np.abs(out[d["configone1_residues"]] - a["configone1_side"]).max() <= 5e-4


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["perturbed", "squeezed", "coarse"])
def test_gpu_search_matches_oracle(built, case):
    """Reduced grids on perturbed starts: the same winners, r3 and positions
    as the oracle, including starts next to the neighbouring residues'
    backbone (the squeeze limits bind) and grids whose last value falls
    short of +move."""
    d, t, a = fixture()
    rng = np.random.default_rng({"perturbed": 1, "squeezed": 2, "coarse": 3}[case])
    n = 8
    res = list(d["residues"][:n])
    side = a["side_start"][:n].copy()
    move, step = 0.35, 0.005
    if case == "perturbed":
        side += rng.normal(0, 0.5, (n, 3))
    elif case == "squeezed":
        for k in range(1, n - 1):   # halfway towards the previous C-alpha or the next NH
            side[k] = 0.5 * (side[k] + (a["ca"][k - 1] if k % 2 else a["nh"][k + 1]))
        move = 0.6
    else:
        res = [int(v) for v in rng.integers(9, 29, size=n)]
        move, step = 1.3, 0.0173
    want = ora.sidechain_search(a["ca"][:n], a["nh"][:n], a["co"][:n], side, res, move, step, tables=t)
    got = systems.sidechain_search(a["ca"][:n], a["nh"][:n], a["co"][:n], side, res, move, step, tables=t)
    assert np.array_equal(got[2], want[2]), (got[2], want[2])
    assert np.array_equal(got[1], want[1])
    assert np.array_equal(got[0], want[0])
