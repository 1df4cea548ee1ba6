"""nsem_euler, the C++ host driver (control-file-driven time loop): its case
set-up on the CPU.  The mesh it builds from the reference's block description
equals the Python host's box mesh bit for bit; its initial fields are the
reference's euler set-up; the oracle run on its arrays follows the unmodified
`euler` binary's trajectory to round-off; its field files are in the
reference's binary format; unsupported options are refused."""
import os

import numpy as np
import pytest

import oracle
from conftest import load_golden, rel_l2
from driver_util import dump_case, make_case, node_order, rotate_case_z, run_driver
from nebulasem_gb300.fields import read_field
from nebulasem_gb300.mesh import box_mesh, bubble_state
from oracle.make_case import CASES

GEOM_U32 = ["meta", "FO", "FN", "allFaces", "faceIdx0", "faceIdx1", "bcU"]
GEOM_LAST_BITS = ("cC", "cV", "Jinv", "fN")
GEOM_F64 = ["cC", "cV", "Jinv", "fN", "fI", "xgl0", "xgl1", "xgl2", "wgl0", "wgl1", "wgl2",
            "psi0", "psi1", "psi2", "dpsi0", "dpsi1", "dpsi2"]


@pytest.mark.parametrize("case,n", [("c1_2d", (10, 1, 10)), ("g3_2", (2, 2, 2)),
                                    ("g3_4n3", (4, 4, 2))])
def test_mesh_equals_python_box_mesh(tmp_path, case, n):
    """The block `wall 3{4 3 2}` of g3_4n3 has 4 elements in y: the mesh app
    adds one division to an odd wall-graded count (hexMesh.cpp:51-66).

    Connectivity, face slots and LGL tables are identical; the driver forms
    the geometry as the reference's mesh app and LoadMesh do (transfinite
    vertex lattice, calcGeometry volumes and areas, metric from the node
    coordinates), which differs from the Python box mesh's affine formulas in
    the last bits only."""
    c = CASES[case]
    d = dump_case(make_case(tmp_path, case, dt=0.01, steps=10))
    m = box_mesh(n, c["order"], c["length"], dim=c["dim"])
    # the Python host marks every wall SYMMETRY for U, as these cases do
    for k in GEOM_U32 + GEOM_F64:
        a, b = np.asarray(d[k]).reshape(-1), np.asarray(m[k]).reshape(-1)
        if k in GEOM_LAST_BITS:
            assert a.shape == b.shape, k
            assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), k
        else:
            assert np.array_equal(a, b), k
    u, p_ref, rho_ref, _ = bubble_state(m, c["amp"], c["center"], c["radius"])
    # numpy's vectorised pow / cos may differ from the C library in the last bit
    assert rel_l2(d["p_ref"], p_ref) < 1e-15
    assert rel_l2(d["rho_ref"], rho_ref) < 1e-15
    assert rel_l2(d["fld_rho"], u[0]) < 1e-15
    T = u[4] / u[0] - 300.0
    assert np.abs(d["fld_T"] - T).max() < 1e-12
    assert not np.any(d["fld_U"])


FLUID = ("P0", "cp", "cv", "R", "gamma", "gravity")


@pytest.mark.parametrize("fixture,case", [("seg_c1_2d", "c1_2d"), ("seg_g3_2", "g3_2"),
                                          ("seg_c1_2d_visc", "c1_2d"), ("seg_srtb", "c1_2d"),
                                          ("seg_srtb_curved", "c1_2d"), ("seg_hill", "c1_2d"),
                                          ("seg_graded", "c1_2d")])
def test_driver_case_follows_euler_binary(tmp_path, fixture, case):
    """The oracle (C library pow, as the binary) run on the driver's mesh and
    initial fields against the unmodified euler binary's fields after the
    same steps on the reference's own mesh: the driver forms the geometry as
    the reference's mesh app and LoadMesh do, so node coordinates and the
    fields after the steps agree bit for bit."""
    g = load_golden(fixture)
    visc = float(g["viscosity"])
    fluid = {}
    if "P0" in g:   # the srtb example's constants
        fluid = dict(P0=float(g["P0"]), cp=float(g["cp"]), cv=float(g["cv"]),
                     gz=float(g["gravity"][2]))
    if "curved" in g:   # a block with curved edges
        fluid["curved"] = str(g["curved"])
    if "grading" in g:  # wall grading (counts, factors)
        gr = g["grading"]
        fluid["grading"] = (tuple(int(v) for v in gr[0]), tuple(float(v) for v in gr[1]))
    d = dump_case(make_case(tmp_path, case, dt=float(g["dt"]), steps=int(g["nsteps"]),
                            viscosity=visc, **fluid))
    d["viscosity"] = visc
    d.update({k: g[k] for k in FLUID if k in g})
    n = int(d["meta"][7])
    m = oracle.OracleMesh(d)
    oracle.set_pow(0)
    rho, U, T = m.segregated(d["fld_rho"], d["fld_U"], d["fld_T"], float(g["dt"]), int(g["nsteps"]))
    kd, kg = node_order(d["cC"], n), node_order(g["cC"], n)
    assert np.array_equal(d["cC"].reshape(-1, 3)[kd], g["cC"].reshape(-1, 3)[:n][kg])
    assert np.array_equal(rho[kd], g["fldN_rho"][kg])
    assert np.array_equal(np.asarray(T)[kd], g["fldN_T"][kg])
    Ud, Ug = np.asarray(U).reshape(-1, 3)[kd], g["fldN_U"].reshape(-1, 3)[kg]
    assert np.array_equal(Ud, Ug)


def test_initial_fields_in_reference_binary_format(tmp_path):
    d = make_case(tmp_path, "c1_2d", dt=0.01, steps=10)
    dump_case(d)
    bc = lambda t: b"".join(bytes([len(s)]) + s.encode()
                            for s in ["{"] + sum([[p, "{", "type", t, "}"]
                                                  for p in ("top", "bottom", "sides")], []) + ["}"])
    T = read_field(os.path.join(d, "dump", "T0.bin"))
    assert T.values.shape == (2500, 1)
    assert T.boundary == b"\x08boundary" + (3).to_bytes(4, "little") + bc("NEUMANN")
    U = read_field(os.path.join(d, "dump", "U0.bin"))
    assert U.values.shape == (2500, 3)
    assert U.boundary == b"\x08boundary" + (3).to_bytes(4, "little") + bc("SYMMETRY")
    r = read_field(os.path.join(d, "dump", "rho0.bin"))
    dd = oracle.load_dump(os.path.join(d, "dump"))
    assert np.array_equal(r.values[:, 0], dd["fld_rho"])


def _edit(path, old, new):
    with open(path) as f:
        s = f.read()
    assert old in s, old
    with open(path, "w") as f:
        f.write(s.replace(old, new))


@pytest.mark.parametrize("file,old,new,msg", [
    ("U0.txt", "type SYMMETRY", "type DIRICHLET", "DIRICHLET of U"),
    ("T0.txt", "type NEUMANN", "type SYMMETRY", "SYMMETRY of T"),
    ("controls", "TRANSIENT", "STEADY", "TRANSIENT"),
    ("controls", "RUSANOV", "HYBRID", "RUSANOV"),
    ("controls", "time_scheme                  BDF1", "time_scheme BDF2", "BDF2"),
    ("controls", "npy       0", "npy       4", "npy 0"),
    ("grid", "3{10 1 10} 3{1 1 1}",
     "3{10 1 10} 3{1 1 1}\n8{0 1 5 4 3 2 6 7} linear 3{2 1 2}", "more than one block"),
    ("grid", "sides   4{1 5 6 2} 4{0 4 7 3}", "sides   4{1 5 6 2}", "no patch"),
    ("controls", "n_deferred                   0", "n_deferred 0\n    amr_step 1", "amr_step"),
])
def test_refuses_what_the_gpu_path_does_not_model(tmp_path, file, old, new, msg):
    d = make_case(tmp_path, "c1_2d", dt=0.01, steps=10)
    _edit(os.path.join(d, file), old, new)
    r = run_driver(d, "--dump", os.path.join(d, "dump"), check=False)
    assert r.returncode == 1
    assert msg in r.stderr, r.stderr


def test_missing_field_is_an_error(tmp_path):
    d = make_case(tmp_path, "c1_2d", dt=0.01, steps=10)
    os.remove(os.path.join(d, "p0.txt"))
    r = run_driver(d, "--dump", os.path.join(d, "dump"), check=False)
    assert r.returncode == 1 and "p0" in r.stderr


def test_controls_comments_and_unknown_blocks(tmp_path):
    d = make_case(tmp_path, "g3_2", dt=0.01, steps=10)
    with open(os.path.join(d, "controls")) as f:
        s = f.read()
    s = "# a comment line\nrefinement\n{\n    field rho\n    limit 4\n}\n" + \
        s.replace("dt                           0.01", "dt 0.02   # half the step")
    with open(os.path.join(d, "controls"), "w") as f:
        f.write(s)
    dump_case(d)


def test_block_with_permuted_vertices(tmp_path):
    """The 2D description lists its block as 8{0 1 5 4 3 2 6 7}: the local
    axes map to x, y, z through the key points (meshApp.cpp edge order)."""
    d = dump_case(make_case(tmp_path, "c1_2d", dt=0.01, steps=10))
    assert list(d["meta"][:3]) == [5, 1, 5]
    assert int(d["meta"][5]) == 100


def test_gaussian_outside_initialiser(tmp_path):
    """`gaussian-outside value pert centre radius radius2` (field.h:1459-1480):
    pert inside the sphere, pert exp(-R^2) outside with R = (r - radius) /
    radius2, as the reference's ctbs example initialises theta'."""
    d = make_case(tmp_path, "c1_2d", dt=0.01, steps=10)
    with open(os.path.join(d, "T0.txt")) as f:
        s = f.read()
    s = s.replace("internal 1", "internal 2").replace(
        "cosine 0 0.5    500 50 350   250 1000 250",
        "gaussian-outside 150  0.5    500 50 300   150 50\n"
        "    gaussian-outside 150 -0.15   560 50 640     0 50")
    with open(os.path.join(d, "T0.txt"), "w") as f:
        f.write(s)
    a = dump_case(d)
    n = int(a["meta"][7])
    x = a["cC"].reshape(-1, 3)[:n]

    def go(value, pert, c, r1, r2):
        R = np.sqrt(((x - np.asarray(c)) ** 2).sum(axis=1))
        R = (R - r1) / r2
        v = np.exp(-R * R)
        v[np.abs(v) <= 1e-7] = 0.0
        return value + np.where(R <= 0, pert, pert * v)

    want = 0.0 + go(150, 0.5, (500, 50, 300), 150, 50)
    want = want + go(150, -0.15, (560, 50, 640), 0, 50)
    assert np.abs(a["fld_T"] - want).max() <= 1e-12


def test_inclined_block_is_the_rotated_case(tmp_path):
    """A 2D case on a block rotated by 30 degrees about z (gravity along z, so
    the physics is the same in the rotated plane): the driver's geometry is
    the rotated one (pseudo-inverse metric, node weights, area vectors) and
    the oracle's 20 segregated steps on it equal the unrotated case's at the
    corresponding nodes, velocity rotated, to round-off."""
    import math
    kw = dict(dt=0.005, steps=20, viscosity=1.5)
    a0 = dump_case(make_case(tmp_path / "flat", "c1_2d", **kw))
    d = make_case(tmp_path / "rot", "c1_2d", **kw)
    rotate_case_z(d, 30.0)
    a1 = dump_case(d)
    n = int(a0["meta"][7])
    assert np.array_equal(a0["meta"], a1["meta"])
    c, s_ = math.cos(math.radians(30.0)), math.sin(math.radians(30.0))
    R = np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1]])
    x0 = a0["cC"].reshape(-1, 3)[:n]
    x1 = a1["cC"].reshape(-1, 3)[:n]
    assert np.abs(x0 @ R.T - x1).max() < 1e-9
    assert rel_l2(a1["cV"], a0["cV"]) < 1e-14
    # Jinv transforms like dxi/dx: Jinv_rot = R Jinv (rows: x, y, z)
    idx = [[0, 3, 5], [6, 1, 4], [8, 7, 2]]
    J0 = a0["Jinv"].reshape(-1, 9)[:n][:, idx]
    J1 = a1["Jinv"].reshape(-1, 9)[:n][:, idx]
    assert np.abs(np.einsum("ij,njk->nik", R, J0) - J1).max() < 1e-14
    outs = []
    for a in (a0, a1):
        a["viscosity"] = 1.5
        m = oracle.OracleMesh(a)
        oracle.set_pow(0)
        outs.append(m.segregated(a["fld_rho"], a["fld_U"], a["fld_T"], 0.005, 20))
    (r0, U0, T0), (r1, U1, T1) = outs
    assert rel_l2(r1, r0) < 1e-14
    assert rel_l2(T1, T0) < 1e-10
    assert rel_l2(np.asarray(U0).reshape(-1, 3) @ R.T, np.asarray(U1).reshape(-1, 3)) < 1e-8


@pytest.mark.parametrize("shape", ["cosine", "gaussian", "ridge", "schar"])
def test_bump_edges_follow_their_shape(tmp_path, shape):
    """Terrain from the bump edge shapes of the mesh app (hexMesh.cpp:20-45):
    the bottom vertices of the element columns lie on h f(m) with m the
    distance from the key point's foot along the edge over the scale (capped
    at 1/2 except for schar).  The cosine shape is pinned bit for bit against
    the euler binary by the seg_hill fixture."""
    d = make_case(tmp_path, "c1_2d", dt=0.01, steps=10, curved="hill")
    if shape != "cosine":
        grid = os.path.join(d, "grid")
        s = open(grid).read().replace("cosine", shape)
        open(grid, "w").write(s)
    dd = dump_case(d)
    npx, npy, npz = (int(v) for v in dd["meta"][:3])
    NP = npx * npy * npz
    cC = dd["cC"].reshape(-1, 3)
    xs, zs = [], []
    for ix in range(10):
        e = ix * 10                     # the element at iz = 0 of column ix
        for li in (0, npx - 1):
            t = (li * npy + 0) * npz + 0
            xs.append(cC[e * NP + t, 0])
            zs.append(cC[e * NP + t, 2])
    xs, zs = np.array(xs), np.array(zs)
    m = np.abs(xs / 1000.0 - 0.5) / 0.6
    if shape != "schar":
        m = np.minimum(m, 0.5)
    f = {"cosine": np.cos(np.pi * m) ** 2, "gaussian": np.exp(-16 * m ** 2),
         "ridge": 1 - 2 * m, "schar": np.exp(-m ** 2) * np.cos(np.pi * m) ** 2}[shape]
    assert np.abs(zs - 150.0 * f).max() < 1e-9
    # a genuinely curved metric: the elements over the slope are not affine
    J = dd["Jinv"].reshape(-1, 9)[: int(dd["meta"][7])]
    assert np.abs(J[:, 5]).max() > 1e-5 or np.abs(J[:, 8]).max() > 1e-5


def test_driver_leveque_case_follows_convection_binary(tmp_path):
    """The advection-leveque set-up (unit square in x-y, z faces deleted,
    npz 0, problem_init LEVEQUE, AB2) made small: the oracle run on the
    driver's mesh and initial scalar, with the analytic wind on the driver's
    node coordinates, ends in the unmodified convection binary's scalar bit
    for bit (nodes matched by coordinates)."""
    from oracle.make_case import leveque_wind, write_leveque_case
    g = load_golden("conv_leveque_ab2")
    dt, steps = float(g["dt"]), int(g["nsteps"])
    case = os.path.join(str(tmp_path), "leveque")
    write_leveque_case(case, n=8, order=4, dt=dt, steps=steps)
    a = dump_case(case)
    n, n_all = int(a["meta"][7]), int(a["meta"][8])
    A, sc = leveque_wind(np.asarray(a["cC"])[:3 * n_all], steps, dt)
    assert np.array_equal(np.asarray(sc), g["wind_scale"])
    t = oracle.OracleMesh(a).convection_wind(np.asarray(A), sc, 2, a["fld_T"], dt, steps)
    kd, kg = node_order(a["cC"], n), node_order(g["cC"], n)
    assert np.array_equal(a["cC"].reshape(-1, 3)[:n][kd], g["cC"].reshape(-1, 3)[:n][kg])
    assert np.array_equal(t[kd], g["fldN_T"][kg])
