"""The reference's in-run analysis: the backbone dihedral histogram of
code/phipsi.f (-Dwrite_phipsi), res(phi + 180, psi + 180) in whole degrees
over residues 2..L-1 of every chain, sampled at output events
(code/main.F90:1227-1231,1315-1317).

The restatement in the oracle is checked against the IUPAC dihedrals
phi = C(i-1)-N(i)-Ca(i)-C(i) and psi = N(i)-Ca(i)-C(i)-N(i+1) computed here
by the textbook atan2 formula: phipsi.f's frame (x along N->Ca, y towards
C perpendicular to it, z = x cross y; the angle of C(i-1) from y, negative
when z > 0) gives exactly that dihedral with its sign.  The device histogram
must equal the oracle's."""
import numpy as np
import pytest

from dmdgb import systems
from dmdgb.engine import Batch, Engine
from helpers import dense_system
from oracle.oracle import Oracle


def _wrap(d):
    return d - np.round(d)


def _dihedral(a, b, c, d):
    """IUPAC dihedral a-b-c-d in degrees, (-180, 180]."""
    b1, b2, b3 = _wrap(b - a), _wrap(c - b), _wrap(d - c)
    n1, n2 = np.cross(b1, b2), np.cross(b2, b3)
    return np.degrees(np.arctan2(np.cross(n1, n2) @ (b2 / np.linalg.norm(b2)), n1 @ n2))


def _chain_starts(spec):
    """First bead of each chain: 3L backbone beads plus one side chain per
    residue that is not glycine (code 9)."""
    starts, s, k = [], 0, 0
    res = np.asarray(spec.residues)
    for L in spec.chain_len:
        starts.append(s)
        s += 3 * L + int(np.count_nonzero(res[k:k + L] != 9))
        k += L
    return starts


def _expected_from(spec, st):
    tf = st["tfalse"]
    p = np.stack([st["x"] + st["vx"] * tf, st["y"] + st["vy"] * tf, st["z"] + st["vz"] * tf], axis=1)
    hist = np.zeros((361, 361), np.int64)
    near = 0
    for s, L in zip(_chain_starts(spec), spec.chain_len):
        for r in range(2, L):
            ca, nh, co = s + r - 1, s + L + r - 1, s + 2 * L + r - 1
            phi = _dihedral(p[co - 1], p[nh], p[ca], p[co])
            psi = _dihedral(p[nh], p[ca], p[co], p[nh + 1])
            deg = [phi + 180.0, psi + 180.0]
            near += sum(abs(x - round(x)) < 1e-6 for x in deg)
            hist[int(np.floor(deg[0])), int(np.floor(deg[1]))] += 1
    return hist, near


@pytest.mark.parametrize("make", ["c1", "dense"])
def test_oracle_phipsi_is_the_iupac_dihedral(built, make):
    spec = systems.generate(systems.config_c1()) if make == "c1" else dense_system(seed=4)
    ora = Oracle(spec)
    total = np.zeros((361, 361), np.int64)
    want = np.zeros((361, 361), np.int64)
    for _ in range(5):
        ora.run(3000)
        one = np.zeros((361, 361), np.int64)
        ora.phipsi_sample(one)
        exp, near = _expected_from(spec, ora.state())
        assert near == 0, "an angle within 1e-6 degree of a bin edge: pick another state"
        assert np.array_equal(one, exp)
        total += one
        want += exp
    ora.phipsi_sample(total)   # accumulates
    assert total.sum() == 6 * sum(L - 2 for L in spec.chain_len)


@pytest.mark.gpu
def test_device_phipsi_equals_oracle(built):
    spec = dense_system(seed=4)
    ora = Oracle(spec)
    oh = np.zeros((361, 361), np.int64)
    with Engine(spec) as eng:
        for _ in range(6):
            eng.run(3000)
            ora.run(3000)
            eng.phipsi_sample()
            ora.phipsi_sample(oh)
        gh, n = eng.phipsi_histogram()
        assert n == 6 and np.array_equal(gh, oh)
        gh2, n2 = eng.phipsi_histogram(reset=True)
        assert n2 == 6 and np.array_equal(gh2, oh)
        gh3, n3 = eng.phipsi_histogram()
        assert n3 == 0 and gh3.sum() == 0


@pytest.mark.gpu
def test_batch_phipsi_per_replica(built):
    specs = systems.config_c3(32, seed=3)[:3]
    for s in specs:
        systems.generate(s)
    with Batch(specs) as b:
        b.run(4000)
        b.phipsi_sample()          # every replica
        b.run(4000)
        b.phipsi_sample(1)         # replica 1 only
        for r, s in enumerate(specs):
            ora = Oracle(s)
            oh = np.zeros((361, 361), np.int64)
            ora.run(4000)
            ora.phipsi_sample(oh)
            if r == 1:
                ora.run(4000)
                ora.phipsi_sample(oh)
            gh, n = b.phipsi_histogram(r)
            assert n == (2 if r == 1 else 1) and np.array_equal(gh, oh), r
