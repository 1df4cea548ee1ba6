"""nsem_euler on the GPU: the driver's time loop, field files and schemes
against the oracle run on the driver's own case arrays (bit for bit for the
FP64 forms, with the correctly rounded pow the GPU uses)."""
import os

import numpy as np
import pytest

import oracle
from conftest import load_golden, rel_l2
from driver_util import dump_case, make_case, node_order, rotate_case_z, run_driver
from nebulasem_gb300.fields import read_field

pytestmark = pytest.mark.gpu

P0, R, GAMMA, T0 = 1e5, 287.0, 1004.5 / 717.5, 300.0


def fields(d, idx, names=("rho", "U", "T", "p")):
    return {f: read_field(os.path.join(d, f"{f}{idx}.bin")).values for f in names}


@pytest.mark.parametrize("visc", [0.0, 1.5])
def test_segregated_run_matches_oracle(tmp_path, visc):
    """100 (30 with viscosity) steps of the reference's scheme, written at
    the end; rho, U, T bit for bit, p the EOS of the last step."""
    steps = 30 if visc else 100
    d = make_case(tmp_path, "c1_2d", dt=0.005, steps=steps, viscosity=visc)
    a = dump_case(d)
    a["viscosity"] = visc
    r = run_driver(d, "--print-every", "7")
    assert "Mass loss" in r.stdout
    out = fields(d, 1)
    m = oracle.OracleMesh(a)
    oracle.set_pow(1)
    try:
        rho1, U1, T1 = m.segregated(a["fld_rho"], a["fld_U"], a["fld_T"], 0.005, steps - 1)
        rho, U, T = m.segregated(rho1, U1, T1, 0.005, 1)
    finally:
        oracle.set_pow(0)
    assert np.array_equal(out["rho"][:, 0], rho)
    assert np.array_equal(out["U"].reshape(-1), np.asarray(U).reshape(-1))
    assert np.array_equal(out["T"][:, 0], T)
    # p' of the last step: rho^{n+1} with theta^n (euler.cpp:210-213)
    Tf = np.asarray(T1) + T0
    want = np.array([P0 * oracle.pow_dd(((r_ * t_) * R) / P0, GAMMA) for r_, t_ in zip(rho, Tf)])
    n = len(rho)
    assert np.array_equal(out["p"][:, 0], want - a["p_ref"][:n])
    g = read_field(os.path.join(d, "gravity1.bin")).values
    assert np.all(g == np.array([0.0, 0.0, -9.81]))


@pytest.mark.parametrize("fixture", ["seg_srtb", "seg_srtb_curved", "seg_hill", "seg_graded"])
def test_srtb_example_run(tmp_path, fixture):
    """The reference's srtb example as shipped (viscosity 1.5, gravity
    -9.80606, the Fluid:: defaults for P0, cp, cv), on its box, on the
    srtb-curved example's arcs and under a cosine hill: the driver's run is the
    oracle's bit for bit (correctly rounded pow) and follows the unmodified
    euler binary's fields; the geometry is the binary's to the bit, and the C
    library's pow, off by an ulp on some arguments, leaves ~1e-15 in rho and
    ~1e-10 in the velocity of this flow from rest after 100 steps.  On the
    curved blocks the precision form's SSP-RK3 run stays within 1e-5 of the
    FP64 form's."""
    g = load_golden(fixture)
    steps = int(g["nsteps"])
    curved = {"curved": str(g["curved"])} if "curved" in g else {}
    if "grading" in g:
        gr = g["grading"]
        curved["grading"] = (tuple(int(v) for v in gr[0]), tuple(float(v) for v in gr[1]))
    d = make_case(tmp_path, "c1_2d", dt=float(g["dt"]), steps=steps, viscosity=1.5,
                  P0=float(g["P0"]), cp=float(g["cp"]), cv=float(g["cv"]), gz=float(g["gravity"][2]),
                  **curved)
    a = dump_case(d)
    a.update({k: g[k] for k in ("P0", "cp", "cv", "R", "gamma", "gravity")})
    a["viscosity"] = 1.5
    run_driver(d, "--print-every", "25")
    out = fields(d, 1, ("rho", "U", "T"))
    m = oracle.OracleMesh(a)
    oracle.set_pow(1)
    try:
        rho, U, T = m.segregated(a["fld_rho"], a["fld_U"], a["fld_T"], float(g["dt"]), steps)
    finally:
        oracle.set_pow(0)
    assert np.array_equal(out["rho"][:, 0], rho)
    assert np.array_equal(out["U"].reshape(-1), np.asarray(U).reshape(-1))
    assert np.array_equal(out["T"][:, 0], T)
    n = int(a["meta"][7])
    kd, kg = node_order(a["cC"], n), node_order(g["cC"], n)
    assert np.array_equal(a["cC"].reshape(-1, 3)[kd], g["cC"].reshape(-1, 3)[:n][kg])
    assert rel_l2(out["rho"][kd, 0], g["fldN_rho"][kg]) < 1e-13
    assert rel_l2(out["T"][kd, 0], g["fldN_T"][kg]) < 1e-10
    assert rel_l2(out["U"][kd], g["fldN_U"].reshape(-1, 3)[kg]) < 2e-9
    if "curved" in g:
        ssprk3_precision_vs_fp64(d)


def ssprk3_precision_vs_fp64(d):
    """SSP-RK3 through the driver on the case: the precision form's fields
    against the FP64 form's, relative L2 <= 1e-5 (rho, U, theta')."""
    run_driver(d, "--scheme", "ssprk3", "--print-every", "50")
    ref = fields(d, 1, ("rho", "U", "T"))
    run_driver(d, "--scheme", "ssprk3", "--prec", "mixed", "--print-every", "50")
    got = fields(d, 1, ("rho", "U", "T"))
    for f in ("rho", "U", "T"):
        assert rel_l2(got[f], ref[f]) <= 1e-5, (f, rel_l2(got[f], ref[f]))


def test_segregated_run_follows_euler_binary(tmp_path):
    """The driver's output files against the unmodified binary's (fixture),
    node by node through the coordinates: the geometry is the binary's to the
    bit; the correctly rounded pow against the C library's leaves round-off."""
    g = load_golden("seg_c1_2d")
    d = make_case(tmp_path, "c1_2d", dt=float(g["dt"]), steps=int(g["nsteps"]))
    a = dump_case(d)
    run_driver(d, "--print-every", "100")
    out = fields(d, 1)
    n = int(a["meta"][7])
    kd, kg = node_order(a["cC"], n), node_order(g["cC"], n)
    assert rel_l2(out["rho"][kd, 0], g["fldN_rho"][kg]) < 1e-13
    assert rel_l2(out["T"][kd, 0], g["fldN_T"][kg]) < 1e-10
    assert rel_l2(out["U"][kd], g["fldN_U"].reshape(-1, 3)[kg]) < 2e-9


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_ssprk3_run(tmp_path, prec):
    """The coupled SSP-RK3 through the driver (3D, 2x2x2 elements, N=4)."""
    steps = 20
    d = make_case(tmp_path, "g3_2", dt=0.01, steps=steps)
    a = dump_case(d)
    run_driver(d, "--scheme", "ssprk3", "--prec", prec, "--print-every", "5")
    out = fields(d, 1, ("rho", "U", "T"))
    m = oracle.OracleMesh(a)
    rho0 = a["fld_rho"]
    U0 = a["fld_U"].reshape(-1, 3)
    u0 = [rho0, U0[:, 0] * rho0, U0[:, 1] * rho0, U0[:, 2] * rho0, rho0 * (a["fld_T"] + T0)]
    oracle.set_pow(1)
    try:
        u = m.ssprk3(u0, 0.01, steps)
    finally:
        oracle.set_pow(0)
    rho = u[0]
    U = np.stack([u[1] / rho, u[2] / rho, u[3] / rho], axis=1)
    T = u[4] / rho - T0
    if prec == "fp64":
        assert np.array_equal(out["rho"][:, 0], rho)
        assert np.array_equal(out["U"], U)
        assert np.array_equal(out["T"][:, 0], T)
    else:
        assert rel_l2(out["rho"][:, 0], rho) < 1e-5
        assert rel_l2(out["U"], U) < 1e-5
        assert rel_l2(out["T"][:, 0], T) < 1e-5


def test_convection_run_matches_oracle(tmp_path):
    """solver convection: the scalar app's loop through the same driver."""
    g = load_golden("conv_c1_2d")
    steps = int(g["nsteps"])
    d = make_case(tmp_path, "c1_2d", dt=float(g["dt"]), steps=steps, solver="convection",
                  wind=(5.0, 0.0, 3.0))
    a = dump_case(d)
    run_driver(d, "--print-every", "10")
    T = read_field(os.path.join(d, "T1.bin")).values[:, 0]
    want = oracle.OracleMesh(a).convection(a["fld_U"].reshape(-1, 3), a["fld_T"], float(g["dt"]), steps)
    assert np.array_equal(T, want)
    n = int(a["meta"][7])
    kd, kg = node_order(a["cC"], n), node_order(g["cC"], n)
    assert rel_l2(T[kd], g["fldN_T"][kg]) < 1e-10


def test_restart_from_written_fields(tmp_path):
    """A run of 100 steps writing every 50, then a second run restarting at
    step 50 from the first run's files: the restart reads rho, U, T, p of
    index 1 and recomputes rho from p and T as euler.cpp:131-147 does at the
    start of every run; its step-100 fields equal the oracle run through the
    same restart bit for bit."""
    import math
    d = make_case(tmp_path, "c1_2d", dt=0.005, steps=100)
    a = dump_case(d)
    ctl = os.path.join(d, "controls")
    with open(ctl) as f:
        s = f.read().replace("write_interval               100", "write_interval               50")
    with open(ctl, "w") as f:
        f.write(s)
    run_driver(d, "--print-every", "50")
    with open(ctl, "w") as f:
        f.write(s.replace("start_step                   0", "start_step                   50"))
    for f_ in ("rho2", "U2", "T2", "p2"):
        os.remove(os.path.join(d, f_ + ".bin"))
    run_driver(d, "--print-every", "25")
    out = fields(d, 2, ("rho", "U", "T"))

    m = oracle.OracleMesh(a)
    n = int(a["meta"][7])
    p_ref = a["p_ref"][:n]
    oracle.set_pow(1)
    try:
        r49, U49, T49 = m.segregated(a["fld_rho"], a["fld_U"], a["fld_T"], 0.005, 49)
        r50, U50, T50 = m.segregated(r49, U49, T49, 0.005, 1)
        pp = np.array([P0 * oracle.pow_dd(((r_ * (t_ + T0)) * R) / P0, GAMMA)
                       for r_, t_ in zip(r50, T49)]) - p_ref
        written = fields(d, 1, ("rho", "U", "T", "p"))
        assert np.array_equal(written["p"][:, 0], pp)
        # the driver's host set-up: C library pow, as the reference's
        gam = 1004.5 / 717.5
        rr = np.array([(P0 / (R * (t_ + T0))) * math.pow((p_ + pr_) / P0, 1 / gam)
                       for t_, p_, pr_ in zip(T50, pp, p_ref)])
        rho, U, T = m.segregated(rr, U50, T50, 0.005, 50)
    finally:
        oracle.set_pow(0)
    assert np.array_equal(out["rho"][:, 0], rho)
    assert np.array_equal(out["U"].reshape(-1), np.asarray(U).reshape(-1))
    assert np.array_equal(out["T"][:, 0], T)


def test_inclined_block_run(tmp_path):
    """A block rotated by 30 degrees (full, non-diagonal metric): the FP64
    forms through the driver are the oracle's bit for bit; the precision form
    (general-geometry kernels, viscous) within 1e-5 of the FP64 form."""
    steps = 20
    d = make_case(tmp_path, "c1_2d", dt=0.005, steps=steps, viscosity=1.5)
    rotate_case_z(d, 30.0)
    a = dump_case(d)
    a["viscosity"] = 1.5
    run_driver(d, "--print-every", "10")
    out = fields(d, 1, ("rho", "U", "T"))
    m = oracle.OracleMesh(a)
    oracle.set_pow(1)
    try:
        rho, U, T = m.segregated(a["fld_rho"], a["fld_U"], a["fld_T"], 0.005, steps)
    finally:
        oracle.set_pow(0)
    assert np.array_equal(out["rho"][:, 0], rho)
    assert np.array_equal(out["U"].reshape(-1), np.asarray(U).reshape(-1))
    assert np.array_equal(out["T"][:, 0], T)
    ssprk3_precision_vs_fp64(d)


def test_text_output_and_high_order(tmp_path):
    """write_format TEXT: the driver writes `.txt` fields with 12 significant
    digits, which read back to the binary run's values within 1e-11; and a
    3D N=7 case through the driver is the oracle's bit for bit."""
    d = make_case(tmp_path / "txt", "c1_2d", dt=0.005, steps=20)
    ctl = os.path.join(d, "controls")
    with open(ctl) as f:
        s = f.read()
    with open(ctl, "w") as f:
        f.write(s.replace("    mesh                         grid",
                          "    mesh                         grid\n    write_format TEXT"))
    run_driver(d, "--print-every", "20")
    txt = {k: read_field(os.path.join(d, f"{k}1.txt")).values for k in ("rho", "U", "T", "p")}
    b = make_case(tmp_path / "bin", "c1_2d", dt=0.005, steps=20)
    run_driver(b, "--print-every", "20")
    bins = fields(b, 1)
    for k in ("rho", "p"):
        assert np.abs(txt[k] - bins[k]).max() <= 1e-11 * np.abs(bins[k]).max(), k
    assert np.abs(txt["U"] - bins["U"]).max() <= 1e-11 * np.abs(bins["U"]).max() + 1e-300
    assert np.abs(txt["T"] - bins["T"]).max() <= 1e-11 * np.abs(bins["T"]).max()

    d7 = make_case(tmp_path / "n7", "g3_2n7", dt=0.005, steps=10)
    a = dump_case(d7)
    run_driver(d7, "--print-every", "5")
    out = fields(d7, 1, ("rho", "U", "T"))
    m = oracle.OracleMesh(a)
    oracle.set_pow(1)
    try:
        rho, U, T = m.segregated(a["fld_rho"], a["fld_U"], a["fld_T"], 0.005, 10)
    finally:
        oracle.set_pow(0)
    assert np.array_equal(out["rho"][:, 0], rho)
    assert np.array_equal(out["U"].reshape(-1), np.asarray(U).reshape(-1))
    assert np.array_equal(out["T"][:, 0], T)


def test_convection_leveque_ab2_run_matches_binary(tmp_path):
    """solver convection with problem_init LEVEQUE and AB2 through the driver
    on the GPU: the written scalar equals the unmodified convection binary's
    bit for bit (nodes matched by coordinates)."""
    from oracle.make_case import write_leveque_case
    g = load_golden("conv_leveque_ab2")
    dt, steps = float(g["dt"]), int(g["nsteps"])
    d = os.path.join(str(tmp_path), "leveque")
    write_leveque_case(d, n=8, order=4, dt=dt, steps=steps)
    a = dump_case(d)
    run_driver(d, "--print-every", "7")
    T = read_field(os.path.join(d, "T1.bin")).values[:, 0]
    n = int(a["meta"][7])
    kd, kg = node_order(a["cC"], n), node_order(g["cC"], n)
    assert np.array_equal(T[kd], g["fldN_T"][kg])
