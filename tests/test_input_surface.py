"""Input surface: the reference's parameter tables, run files and
unformatted records, read by the package's parsers (CPU only)."""
import hashlib
import io
import json
import os

import numpy as np
import pytest

from conftest import REFERENCE, has_reference
from dmdgb import params

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a, dtype="<f8")).tobytes()).hexdigest()


def test_shipped_tables_match_digest():
    """The package's PRIME20 tables equal the parse of the reference files."""
    t = params.default_tables()
    want = json.load(open(os.path.join(GOLD, "tables_digest.json")))
    for k, h in want.items():
        assert _digest(getattr(t, k)) == h, k


def test_shipped_table_values():
    t = params.default_tables()
    assert list(t.sigma) == [3.3, 3.7, 2.708, 4.0]
    assert list(t.welldia) == [4.5, 0.0, 0.0, 4.5]
    assert list(t.epsilon) == [12.0, 0.0, 1.2, 12.0]
    assert t.mass[2] == 0.866 and t.mass[1] == 0.999 and t.mass[4] == 1.863 and t.mass[20] == 1.0
    assert np.array_equal(t.bds, t.bds.T) and np.array_equal(t.wel, t.wel.T) and np.array_equal(t.ep, t.ep.T)
    assert t.rca[0] == 0.654 and t.rco[19] == 2.959 and t.sqz[0][0] == 4.064


def test_shipped_tables_against_values_typed_from_the_files():
    """Entries typed by hand from the reference's parameter files (row and
    column as the files state them), so that the parse is checked against
    values it did not produce: parameters/beadwell_ha55a.data (pair
    diameter, well diameter), parametersep/ep19p_ha55a_weakhp.data (raw
    value), parameters/rcarnrco.data (CA-R, NH-R, CO-R and the three
    window fractions), parameters/sqz6to10.data (sz8, sz6, sz7, sz9, sz10)
    and parameters/mass.data."""
    t = params.default_tables()
    i = lambda ident: ident - 9        # residue identity 9..28 -> row 0..19
    # beadwell: "G  9  G  9   3.100   3.100", "G  9  R 10   3.200   3.200",
    # "S 18  V 28   2.800   6.158", "V 28  Y 27   3.000   6.521", "V 28  V 28   3.300   6.306"
    for a, b, bd, wl in ((9, 9, 3.1, 3.1), (9, 10, 3.2, 3.2), (18, 28, 2.8, 6.158), (28, 27, 3.0, 6.521),
                         (28, 28, 3.3, 6.306)):
        assert (t.bds[i(a), i(b)], t.wel[i(a), i(b)]) == (bd, wl), (a, b)
    # ep19p_ha55a_weakhp: "G  9  G  9     0.000", "T 19  L 23     0.015", "T 19  M 24    -0.116"
    assert t.ep[i(9), i(9)] == 0.0 and t.ep[i(19), i(23)] == 0.015 and t.ep[i(19), i(24)] == -0.116
    # rcarnrco: G " 0.654   1.908   1.967   0.023   0.023   0.023", R " 4.700   5.100   5.900 ...",
    # V " 2.002   2.775   2.959 ..."
    assert (t.rca[0], t.rnh[0], t.rco[0]) == (0.654, 1.908, 1.967)
    assert (t.rca[1], t.rnh[1], t.rco[1]) == (4.7, 5.1, 5.9)
    assert (t.rca[19], t.rnh[19], t.rco[19]) == (2.002, 2.775, 2.959)
    assert t.del_rca[0] == t.del_rnh[0] == t.del_rco[19] == 0.023
    # sqz6to10: G " 4.064   2.600   2.601   4.013   4.904", R " 5.703   4.827 ...", L (row 15)
    assert list(t.sqz[0]) == [4.064, 2.6, 2.601, 4.013, 4.904]
    assert list(t.sqz[1]) == [5.703, 4.827, 4.651, 5.535, 4.978]
    assert list(t.sqz[i(23)]) == [4.936, 3.918, 3.724, 4.863, 5.001]
    # mass.data: "CA   2     0.866", "NH   1     0.999", "CO   4     1.863", " G   9     0.067", " R  10     6.728"
    assert (t.mass[2], t.mass[1], t.mass[4], t.mass[9], t.mass[10]) == (0.866, 0.999, 1.863, 0.067, 6.728)


@pytest.mark.skipif(not has_reference(), reason="reference checkout not mounted")
def test_parse_reference_tables():
    """The parser on the reference files (when mounted) gives the shipped tables."""
    t = params.read_tables(os.path.join(REFERENCE, "parameters"),
                           os.path.join(REFERENCE, "parametersep", "ep19p_ha55a_weakhp.data"))
    shipped = params.default_tables()
    for k in shipped.__dict__:
        assert np.array_equal(getattr(t, k), getattr(shipped, k)), k


@pytest.mark.skipif(not has_reference(), reason="reference checkout not mounted")
def test_reference_species_files():
    sp = params.read_species(os.path.join(REFERENCE, "parameters"), [7, 7], [28, 28])
    assert sp[0].residues() == [16, 23, 28, 25, 25, 20, 14]  # KLVFFAE
    assert sp[1].residues() == sp[0].residues()
    assert sp[0].hp == [0] * 21 + [1] * 7


def test_run_file(tmp_path):
    p = tmp_path / "temp_020"
    p.write_text("0.200D0 # reduced temperature\n1000000000 #number of collisions\n")
    assert params.read_run_file(str(p)) == (0.2, 1000000000)
    assert json.load(open(os.path.join(GOLD, "run_file.json")))["temp_020"] == [0.2, 1000000000]


def test_record_fixture_roundtrip(tmp_path):
    """Writer and reader agree on the framing of the genconfig records."""
    g = json.load(open(os.path.join(GOLD, "reference_records.json")))
    n = g["n_beads"]
    x = np.linspace(-0.49, 0.49, n)
    body = params.config_record(7, 1.5, x, -x, x * 0.5)
    assert len(body) == g["config_record_bytes"]
    vbody = params.lastvel_record(7, x, x, x)
    assert len(vbody) == g["lastvel_record_bytes"]
    f = tmp_path / "r.config"
    with open(f, "wb") as fh:
        params.write_record(fh, body)
        params.write_record(fh, body)
    recs = params.read_records(str(f))
    assert len(recs) == 2
    coll, t, rx, ry, rz = params.parse_config_record(recs[1], n)
    assert coll == 7 and t == 1.5 and np.array_equal(rx, x) and np.array_equal(rz, x * 0.5)


def test_corrupt_record_rejected(tmp_path):
    f = tmp_path / "bad.config"
    f.write_bytes(b"\x10\x00\x00\x00" + b"\x00" * 12)
    with pytest.raises(ValueError):
        params.read_records(str(f))


@pytest.mark.skipif(not has_reference(), reason="reference checkout not mounted")
def test_reference_records_known_answer():
    """genconfig's results/run0000.{config,lastvel}: 672 beads, 16,144-byte
    config record = 8 + 8 + 3*672*8, first velocity as velocitycheck.out."""
    g = json.load(open(os.path.join(GOLD, "reference_records.json")))
    recs = params.read_records(os.path.join(REFERENCE, "genconfig/results/run0000.config"))
    assert len(recs) == 1 and len(recs[0]) == 16144 == 8 + 8 + 3 * 672 * 8
    assert hashlib.sha256(recs[0]).hexdigest() == g["config_sha256"]
    coll, t, x, y, z = params.parse_config_record(recs[0], 672)
    assert coll == 0 and t == 0.0 and x[:8].tolist() == g["x_head"]
    assert -0.5 <= x.min() and x.max() <= 0.5
    v = params.read_records(os.path.join(REFERENCE, "genconfig/results/run0000.lastvel"))
    coll, vx, vy, vz = params.parse_lastvel_record(v[0], 672)
    # velocitycheck.out prints 15 significant digits of the same value
    assert vx[0] == pytest.approx(g["velocitycheck_first"], rel=1e-14)
    assert g["velocitycheck_first"] == 3.10855611236532


def test_energy_line_format():
    line = params.energy_line(123, 1.5, -20.25, 2.4, 1, 2, 3, 0.5, 0.25, 6.5, 20.0)
    assert len(line) == 15 + 3 * 12 + 3 * 8 + 4 * 12
    assert line[:15].strip() == "123"


def test_run_numbering(tmp_path):
    assert params.next_run_name(str(tmp_path)) == ("0000", "-001")
    (tmp_path / "run0000.energy").write_text("")
    (tmp_path / "run0001.energy.gz").write_text("")
    assert params.next_run_name(str(tmp_path)) == ("0002", "0001")
