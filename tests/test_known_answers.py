"""Two-bead known answers: every predictor branch of code/core.f, bond.f,
sqwel.f, nc_sqwel.f and sqshlder.f and every collision type of
code/eventdyn.f, checked against closed forms from mechanics, with the
contact diameters, well depths and masses taken from the parameter files
as the reference defines them (code/inputinfo.f, code/scale_down.f) and
its constants (code/def.h, code/scale_down.f:32-35, code/make_code.f).

  time   two beads at separation r0 with relative velocity v reach the
         sphere |r| = R first at t = (-(r0.v) - sqrt((r0.v)^2 -
         |v|^2 (|r0|^2 - R^2))) / |v|^2 when approaching from outside,
         at the + root when leaving from inside; a head-on pair at d0
         closing at speed u meets at (d0 - R) / u;
  impulse along r only: momentum kept, tangential relative velocity kept;
         the normal relative velocity reversed at a hard wall; on crossing
         a step of depth eps the kinetic energy changes by -+eps (well
         capture +eps, escape -eps, shoulder entry -eps, exit +eps), and a
         pair without the energy to climb the step bounces.

The CPU test pins the oracle (the CPU restatement the engine is tested against) to
these answers; the GPU test runs the same cases through the engine's own
device predictor and impulse (tests/gpu_src/known_answers.cu), and the
core and bond cases also through the light batches' half-warp collision,
and requires the closed forms and bit equality with the oracle."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.params import default_tables

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300", "csrc")

# code/def.h: bond lengths (angstrom), window half-width, squeeze factors
DNC, DCC, DCN, DTIE, DTIE2, DCACA = 1.46, 1.51, 1.33, 2.41, 2.45, 3.8
DEL = 0.02375
SQZ = {17: 1.1436, 18: 0.88, 19: 0.87829, 20: 0.8, 21: 0.7713}
SHOULDER_NH_CA = 5.00          # code/scale_down.f:32 (shder_dist1: NH-CA)
HB_CORE_BONDED = 1.05 * 2.24   # code/inputinfo.f: ev_param(1,15) times the NH-CO pair diameter
ID_NH, ID_CA, ID_CO = 1, 2, 4
ID_L, ID_V = 23, 28

# two chains of KLVFFAE: bead order per chain CA 1..7, NH 1..7, CO 1..7, R 1..7
CA0, NH3, CA_B, NH_B, CO3_B, R_L0, R_V_B, R_L_B = 0, 9, 30, 35, 44, 22, 51, 50
LOW_E, HIGH_E = 0.5, 12.0       # closing speeds: below / above every step height here


def _system():
    return systems.generate(systems.klvffae_system(2, 5.0, 0.2, seed=1))


def _pair_table(boxl):
    """(name, i, j, ida, idb, evcode, bonded, R_contact, R_wall, eps, kind)
    for each pair type; distances in box units.  kind: core, bond, well
    (core inside a well of depth eps), hbwell, shoulder (core inside a
    shoulder of height eps), hbbond (bonded H-bond pair), hbfar (an NH-CO
    pair that may not bond: a hard wall at the well)."""
    t = default_tables()
    sig = {ID_NH: t.sigma[0], ID_CA: t.sigma[1], ID_CO: t.sigma[3]}
    wdia = {ID_NH: t.welldia[0], ID_CO: t.welldia[3]}
    eps1 = t.epsilon[0]
    B = boxl
    s_ca = sig[ID_CA]
    s_ca_co = 0.5 * (sig[ID_CA] + sig[ID_CO])
    s_nh_co = 0.5 * (sig[ID_NH] + sig[ID_CO])
    s_nh_ca = 0.5 * (sig[ID_NH] + sig[ID_CA])
    w_hb = 0.5 * (wdia[ID_NH] + wdia[ID_CO])
    lv = (ID_L - 9, ID_V - 9)
    return [
        ("core CA-CA (1)", CA0, CA_B, 0, 0, 1, 0, s_ca / B, None, 0.0, "core"),
        ("squeezed core CA-CO (17)", CA0, CO3_B, 0, 0, 17, 0, SQZ[17] * s_ca_co / B, None, 0.0, "core"),
        ("squeezed core CA-R(L) (24)", CA0, R_L_B, 0, 0, 24, 0, t.sqz[ID_L - 9][0] / B, None, 0.0, "core"),
        ("bond CA-NH (4)", CA0, NH_B, 0, 0, 4, 0, DNC * (1 - DEL) / B, DNC * (1 + DEL) / B, 0.0, "bond"),
        ("bond CA-CA (9)", CA0, CA_B, 0, 0, 9, 0, DCACA * (1 - DEL) / B, DCACA * (1 + DEL) / B, 0.0, "bond"),
        ("hydrophobic well L-V (16)", R_L0, R_V_B, 0, 0, 16, 0, t.bds[lv] / B, t.wel[lv] / B,
         eps1 * -t.ep[lv], "well"),
        ("H-bond well NH-CO (15)", NH3, CO3_B, 0, 0, 15, 0, s_nh_co / B, w_hb / B,
         np.sqrt(eps1 * t.epsilon[3]), "hbwell"),
        ("bonded H-bond NH-CO (15)", NH3, CO3_B, ID_NH + 4, ID_CO + 4, 15, 1, HB_CORE_BONDED / B, w_hb / B,
         np.sqrt(eps1 * t.epsilon[3]), "hbbond"),
        ("H-bond well, partner taken (15)", NH3, CO3_B, ID_NH, ID_CO + 4, 15, 0, None, w_hb / B, 0.0, "hbfar"),
        ("shoulder NH-CA (40)", NH3, CA_B, 0, 0, 40, 0, s_nh_ca / B, SHOULDER_NH_CA / B, eps1, "shoulder"),
    ]


def _unit(rng):
    u = rng.normal(size=3)
    return u / np.linalg.norm(u)


def _place(rng, r, v, mi, mj):
    """Positions/velocities of i and j with relative position r = ri - rj and
    relative velocity v = vi - vj, somewhere in the box, with a random
    centre-of-mass velocity."""
    xj = rng.uniform(-0.4, 0.4, 3)
    xi = xj + r
    vc = rng.normal(size=3) * 0.3
    vi = vc + v * mj / (mi + mj)
    vj = vc - v * mi / (mi + mj)
    return np.concatenate([xi, vi, xj, vj])


def _cases(boxl, masses):
    """Cases: (label, pair row, state, ct_in, expected type, expected time
    or None, expected step of kinetic energy or None).  Prediction cases
    have ct_in 0; impulse cases put the pair on the wall it meets."""
    rng = np.random.default_rng(2024)
    out = []
    for row in _pair_table(boxl):
        name, i, j, ida, idb, ev, bonded, Rc, Rw, eps, kind = row
        mi, mj = masses[(i, j)]

        def add(label, r, v, ty, t_exp, ct_in=0, dke=None):
            out.append((f"{name}: {label}", row, _place(rng, r, v, mi, mj), ct_in, ty, t_exp, dke))

        def approach(d0, R, u, b=0.0):
            """relative position d0 along n with offset b, closing at u along -n"""
            n = _unit(rng)
            p = _unit(rng)
            p = p - p.dot(n) * n
            p /= np.linalg.norm(p)
            r = d0 * n + b * p
            v = -u * n
            return r, v, (d0 - np.sqrt(R * R - b * b)) / u if b < R else None

        def leave(d0, R, u):
            n = _unit(rng)
            return d0 * n, u * n, (R - d0) / u

        def wall(R, u, sign):
            """on the sphere |r| = R, moving with normal speed u (sign -1: in)"""
            n = _unit(rng)
            p = _unit(rng)
            p = p - p.dot(n) * n
            return R * n, sign * u * n + 0.3 * u * p

        if kind == "core":
            r, v, t = approach(1.5 * Rc, Rc, 0.8)
            add("head-on approach", r, v, 1, t)
            r, v, t = approach(1.7 * Rc, Rc, 1.1, b=0.6 * Rc)
            add("oblique approach", r, v, 1, t)
            r, v, _ = approach(1.5 * Rc, Rc, 0.8, b=1.2 * Rc)
            add("miss", r, v, 0, None)
            r, v, _ = leave(1.5 * Rc, Rc, 0.8)
            add("separating", r, v, 0, None)
            r, v = wall(Rc, 0.9, -1.0)
            add("impulse", r, v, None, None, ct_in=1, dke=0.0)
        elif kind == "bond":
            mid = 0.5 * (Rc + Rw)
            r, v, t = approach(mid, Rc, 0.7)
            add("inner wall", r, v, 2, t)
            r, v, t = leave(mid, Rw, 0.7)
            add("outer wall", r, v, 3, t)
            r, v = wall(Rc, 0.9, -1.0)
            add("inner impulse", r, v, None, None, ct_in=2, dke=0.0)
            r, v = wall(Rw, 0.9, 1.0)
            add("outer impulse", r, v, None, None, ct_in=3, dke=0.0)
        elif kind in ("well", "hbwell", "shoulder"):
            enter, exit_, k_in, k_out = {"well": (4, 8, 20, 21), "hbwell": (7, 16, None, None),
                                         "shoulder": (12, 10, 25, 24)}[kind]
            r, v, t = approach(1.4 * Rw, Rw, 0.9)
            add("entry from outside", r, v, enter, t)
            r, v, _ = approach(1.4 * Rw, Rw, 0.9, b=1.1 * Rw)
            add("miss", r, v, 0, None)
            mid = 0.5 * (Rc + Rw)
            r, v, t = approach(mid, Rc, 0.6)
            add("core inside", r, v, 1, t)
            r, v, t = leave(mid, Rw, 0.6)
            add("exit from inside", r, v, exit_, t)
            r, v, _ = leave(1.4 * Rw, Rw, 0.6)
            add("separating outside", r, v, 0, None)
            if kind == "well":
                r, v = wall(Rw, LOW_E, -1.0)
                add("capture", r, v, None, None, ct_in=4, dke=eps)
                r, v = wall(Rw, HIGH_E, 1.0)
                add("escape", r, v, None, None, ct_in=8, dke=-eps)
                r, v = wall(Rw, LOW_E, 1.0)
                add("bounce inside", r, v, None, None, ct_in=8, dke=0.0)
                r, v = wall(Rc, 0.9, -1.0)
                add("core impulse", r, v, None, None, ct_in=1, dke=0.0)
            elif kind == "shoulder":
                r, v = wall(Rw, HIGH_E, -1.0)
                add("climb onto the shoulder", r, v, None, None, ct_in=6, dke=-eps)
                r, v = wall(Rw, LOW_E, -1.0)
                add("bounce off the shoulder", r, v, None, None, ct_in=6, dke=0.0)
                r, v = wall(Rw, 0.9, 1.0)
                add("step off the shoulder", r, v, None, None, ct_in=5, dke=eps)
                r, v = wall(Rw, 0.9, -1.0)
                add("shoulder closed (a hard wall)", r, v, None, None, ct_in=13, dke=0.0)
                r, v = wall(Rc, 0.9, -1.0)
                add("core under the shoulder", r, v, None, None, ct_in=1, dke=0.0)
            elif kind == "hbwell":
                r, v = wall(Rc, 0.9, -1.0)
                add("core inside the well", r, v, None, None, ct_in=1, dke=0.0)
        elif kind == "hbbond":
            mid = 0.5 * (Rc + Rw)
            r, v, t = approach(mid, Rc, 0.6)
            add("core", r, v, 1, t)
            # rounding can leave a bonded pair just outside its well; moving
            # mostly sideways, its discriminant is negative and the
            # reference's root (nc_sqwel.f:69-93) is a NaN that nothing
            # selects: no event
            n = _unit(rng)
            tvec = _unit(rng)
            tvec = tvec - tvec.dot(n) * n
            tvec /= np.linalg.norm(tvec)
            add("just outside, moving sideways", 1.02 * Rw * n, 0.1 * n + 1.0 * tvec, 0, None)
            r, v, t = leave(mid, Rw, 0.6)
            add("exit", r, v, 8, t)
            r, v = wall(Rw, HIGH_E, 1.0)
            add("dissociation", r, v, None, None, ct_in=8, dke=-eps)
            r, v = wall(Rw, LOW_E, 1.0)
            add("held", r, v, None, None, ct_in=8, dke=0.0)
        elif kind == "hbfar":
            r, v, t = approach(1.4 * Rw, Rw, 0.9)
            add("wall at the well", r, v, 9, t)
            r, v = wall(Rw, 0.9, -1.0)
            add("impulse", r, v, None, None, ct_in=9, dke=0.0)
    return out


FINAL_CT = {1: {1}, 2: {2}, 3: {3}, 4: {20}, 8: {21, 22}, 9: {23}, 5: {24}, 6: {25, 26}, 13: {27}}


def _check_case(case, tij, ty, valid, st_out, ct_out, masses):
    label, row, st, ct_in, ty_exp, t_exp, dke = case
    name, i, j, ida, idb, ev, bonded, Rc, Rw, eps, kind = row
    assert valid, label
    if ct_in == 0:
        if np.isnan(tij):                     # the reference's NaN root: never selected, no event
            assert ty_exp == 0 and t_exp is None, label
            return
        assert ty == ty_exp, f"{label}: type {ty}, expected {ty_exp}"
        if t_exp is None:
            assert tij == 1e9 or np.isnan(tij), f"{label}: time {tij} for no event"
        else:
            assert tij == pytest.approx(t_exp, rel=1e-12), label
        return
    mi, mj = masses[(i, j)]
    assert ct_out in FINAL_CT[ct_in], f"{label}: final type {ct_out}"
    vi0, vj0, vi1, vj1 = st[3:6], st[9:12], st_out[3:6], st_out[9:12]
    p0 = mi * vi0 + mj * vj0
    p1 = mi * vi1 + mj * vj1
    scale = mi * np.abs(vi0).max() + mj * np.abs(vj0).max()
    assert np.allclose(p1, p0, rtol=0, atol=1e-13 * scale), f"{label}: momentum"
    n = st[0:3] - st[6:9]
    n = n / np.linalg.norm(n)
    w0, w1 = vi0 - vj0, vi1 - vj1
    tang0, tang1 = w0 - w0.dot(n) * n, w1 - w1.dot(n) * n
    assert np.allclose(tang1, tang0, rtol=0, atol=1e-12 * np.abs(w0).max()), f"{label}: tangential velocity"
    ke0 = 0.5 * (mi * vi0.dot(vi0) + mj * vj0.dot(vj0))
    ke1 = 0.5 * (mi * vi1.dot(vi1) + mj * vj1.dot(vj1))
    assert ke1 - ke0 == pytest.approx(dke, abs=1e-11 * max(ke0, 1.0)), f"{label}: kinetic energy step"
    if dke == 0.0:
        assert w1.dot(n) == pytest.approx(-w0.dot(n), rel=1e-12), f"{label}: normal velocity not reversed"


def _run_oracle(spec, cases):
    from oracle.oracle import Oracle, lib
    L = lib()
    L.ora_pair_case.argtypes = [C.c_void_p] + [C.c_int32] * 6 + [C.c_void_p, C.c_int32] + [C.c_void_p] * 5
    o = Oracle(spec)
    res = []
    for case in cases:
        _, row, st, ct_in, *_ = case
        _, i, j, ida, idb, ev, bonded, *_ = row
        st = np.ascontiguousarray(st, np.float64)
        tij, ty, cto = C.c_double(), C.c_int32(), C.c_int32()
        out = np.zeros(12)
        m = np.zeros(2)
        rc = L.ora_pair_case(o.h, i, j, ida, idb, ev, bonded, st.ctypes.data, ct_in or 0, C.byref(tij), C.byref(ty),
                             out.ctypes.data, C.byref(cto), m.ctypes.data)
        assert rc == 0
        res.append((tij.value, ty.value, True, out, cto.value, m))
    return res


def _masses(spec):
    t = default_tables()
    bmass = t.mass.copy()
    bmass[3] = bmass[20]
    ident = {CA0: ID_CA, CA_B: ID_CA, NH3: ID_NH, NH_B: ID_NH, CO3_B: ID_CO, R_L0: ID_L, R_V_B: ID_V, R_L_B: ID_L}
    return {(row[1], row[2]): (bmass[ident[row[1]]], bmass[ident[row[2]]]) for row in _pair_table(spec.boxl)}


def test_oracle_known_answers(built):
    spec = _system()
    masses = _masses(spec)
    cases = _cases(spec.boxl, masses)
    res = _run_oracle(spec, cases)
    kinds = set()
    for case, (tij, ty, ok, out, cto, m) in zip(cases, res):
        row = case[1]
        assert tuple(m) == masses[(row[1], row[2])], "bead masses"
        _check_case(case, tij, ty, ok, out, cto, masses)
        kinds.add(ty if case[3] == 0 else cto)
    # every predictor outcome and every final collision type of eventdyn.f
    assert {1, 2, 3, 4, 7, 8, 9, 10, 12, 16}.issubset(kinds), kinds
    assert {20, 21, 22, 23, 24, 25, 26, 27}.issubset(kinds), kinds


def _harness():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = os.path.join(HERE, "gpu_src", "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libknown_answers.so")
    src = os.path.join(HERE, "gpu_src", "known_answers.cu")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(p) for p in deps):
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false",
                        "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + CSRC, "-I" + os.path.join(REPO, "include"),
                        "-shared", src, "-o", so + ".tmp"], check=True, capture_output=True, timeout=900)
        os.replace(so + ".tmp", so)
    return C.CDLL(so)


@pytest.mark.gpu
def test_device_known_answers(built):
    spec = _system()
    masses = _masses(spec)
    cases = _cases(spec.boxl, masses)
    n = len(cases)
    L = _harness()
    col = lambda k: np.ascontiguousarray([c[1][k] for c in cases], np.int32)
    i, j, ida, idb, ev, bond = (col(k) for k in (1, 2, 3, 4, 5, 6))
    st = np.ascontiguousarray(np.concatenate([c[2] for c in cases]), np.float64)
    ct = np.ascontiguousarray([c[3] or 0 for c in cases], np.int32)
    tij, ty, valid, cto = np.zeros(n), np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32)
    out = np.zeros(12 * n)
    light = np.zeros(12 * n)
    t = abi.tables_struct(default_tables())
    cfg = spec.run_cfg()
    sys_ = spec.c_system()
    err = C.create_string_buffer(256)
    rc = L.ka_pair_cases(C.byref(cfg), C.byref(t), C.byref(sys_), n, *[a.ctypes.data for a in (i, j, ida, idb, ev, bond)],
                         st.ctypes.data, ct.ctypes.data, tij.ctypes.data, ty.ctypes.data, valid.ctypes.data,
                         out.ctypes.data, cto.ctypes.data, light.ctypes.data, err, 256)
    assert rc == 0, err.value.decode()
    ora = _run_oracle(spec, cases)
    for q, case in enumerate(cases):
        _check_case(case, tij[q], int(ty[q]), bool(valid[q]), out[12 * q:12 * q + 12], int(cto[q]), masses)
        otij, oty, _, oout, octo, _ = ora[q]
        if np.isnan(otij):                    # the reference's NaN root: no event on the device
            otij, oty = 1e9, 0
        assert (tij[q], int(ty[q]), int(cto[q])) == (otij, oty, octo), case[0]
        assert np.array_equal(out[12 * q:12 * q + 12], oout), case[0]
        if case[3] in (1, 2, 3):   # the light batches' half-warp collision gives the same bits
            assert np.array_equal(light[12 * q:12 * q + 12], oout), case[0] + " (half-warp collision)"
