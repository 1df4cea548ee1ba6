"""Write a rising-bubble case directory in the reference's input formats.

Test infrastructure: the case directories feed the reference-built oracle
harness (oracle/_ref/euler_oracle) that generates the golden fixtures, and
the product's own host driver reads the same files.  Formats follow the
reference's examples: controls file with brace blocks (src/util/util.cpp:32-79),
block-mesh description read by the mesh app (apps/mesh/meshApp.cpp), and
field files with an `internal` initialiser plus per-boundary conditions
(src/field/field.h:1409-1519).
"""
import argparse
import os

CONTROLS = """general
{{
    solver                       euler
    mesh                         grid
    P0                           {P0}
    T0                           300
    cp                           {cp}
    cv                           {cv}
    state                        TRANSIENT
    start_step                   0
    end_step                     {end_step}
    write_interval               {end_step}
    dt                           {dt}
    n_deferred                   0
    convection_scheme            RUSANOV
    time_scheme                  BDF1
    print_time                   0
    viscosity                    {viscosity}
    Pr                           {Pr}
    gravity   0 0 {gz}
    npx       {npx}
    npy       {npy}
    npz       {npz}
}}

euler
{{
    diffusion                    {diffusion}
    buoyancy                     YES
}}
"""

GRID_2D = """8
{{
0 0 0
{lx} 0 0
{lx} 0 {lz}
0 0 {lz}
0 {ly} 0
{lx} {ly} 0
{lx} {ly} {lz}
0 {ly} {lz}
}}

8{{0 1 5 4 3 2 6 7}} wall 3{{{nx} 1 {nz}}} 3{{1 1 1}}

top     4{{3 2 6 7}}
bottom  4{{0 1 5 4}}
delete  4{{0 1 2 3}} 4{{4 5 6 7}}
sides   4{{1 5 6 2}} 4{{0 4 7 3}}
"""

GRID_3D = """8
{{
0 0 0
{lx} 0 0
{lx} {ly} 0
0 {ly} 0
0 0 {lz}
{lx} 0 {lz}
{lx} {ly} {lz}
0 {ly} {lz}
}}

8{{0 1 2 3 4 5 6 7}} wall 3{{{nx} {ny} {nz}}} 3{{1 1 1}}

top     4{{4 5 6 7}}
bottom  4{{0 1 2 3}}
sides   4{{0 1 5 4}} 4{{3 2 6 7}} 4{{0 3 7 4}} 4{{1 2 6 5}}
"""

FIELD = """size {size}
internal 1
{{
    {init}
}}
boundary 3
{{
    top {{
        type {bc}
    }}
    bottom {{
        type {bc}
    }}
    sides {{
        type {bc}
    }}
}}
"""


# Curved block edges for the 2D block 8{0 1 5 4 3 2 6 7}: extra key points (in
# units of the block lengths) and `edges` lines of the mesh app
# (apps/mesh/meshApp.cpp:159-185).  "arc_y": the reference's srtb-curved
# example, its x edges bowed out in y through arcs; "hill": a cosine hill
# 0.15 lz high over 60 % of the bottom edges, as the hills examples build
# terrain.
CURVED = {
    "arc_y": ([(0.5, 2.0, 0.0), (0.5, 4.0, 0.0), (0.5, 4.0, 1.0), (0.5, 2.0, 1.0)],
              ["arc 0 8", "arc 1 9", "arc 2 10", "arc 3 11"]),
    "hill": ([(0.5, 0.0, 0.15), (0.5, 1.0, 0.15)],
             ["cosine 0 8 0.6", "cosine 1 9 0.6"]),
}


def curved_grid(grid, curved, lx, ly, lz):
    """Insert a CURVED variant's key points and edges into a 2D grid text."""
    pts, edges = CURVED[curved]
    lines = grid.split("\n")
    nkp = int(lines[0])
    extra = [f"{a * lx!r} {b * ly!r} {c * lz!r}" for a, b, c in pts]
    lines[0] = str(nkp + len(extra))
    close = lines.index("}")
    lines[close:close] = extra
    blk = next(q for q, l in enumerate(lines) if l.startswith("8{"))
    lines[blk + 1:blk + 1] = [f"edges {len(edges)}{{"] + ["    " + e for e in edges] + ["}"]
    return "\n".join(lines)


# adaptive refinement of the initial mesh by the reference's prepare -refine
# (src/field/field.cpp:625-960): cells whose normalised |theta'| indicator
# reaches field_max are split once (2D: in the x-z plane, direction = the
# collapsed axis; 3D: direction 0 0 0), leaving 2:1 non-conforming faces
REFINE = """
refinement
{{
    direction       {direction}
    field           T
    field_min       0.01
    field_max       {field_max}
    max_level       1
    limit           100000
}}

prepare
{{
    fields    4 {{ U T p rho }}
}}
"""


# The reference's advection-leveque example, made small: the unit square in
# x-y (z faces deleted, npz 0), problem_init LEVEQUE (the wind
# (sin^2(pi x) sin(2 pi y), -sin^2(pi y) sin(2 pi x), 0) cos(pi t / T),
# apps/convection/convection.cpp:86-91) and a cosine2 scalar bump
GRID_XY = """8
{{
0 0 0
1 0 0
1 1 0
0 1 0
0 0 0.1
1 0 0.1
1 1 0.1
0 1 0.1
}}

8{{0 1 2 3 4 5 6 7}} wall 3{{{nx} {ny} 1}} 3{{1 1 1}}

top     4{{3 2 6 7}}
bottom  4{{0 1 5 4}}
delete  4{{0 1 2 3}} 4{{4 5 6 7}}
sides   4{{1 2 5 6}} 4{{0 4 7 3}}
"""


def write_leveque_case(out, *, n, order, dt, steps, time_scheme="AB2"):
    """The advection-leveque example's set-up on an n x n block of order `order`
    for `steps` steps (end_step = steps, so the wind reverses once); a
    controls_setup beside it names the euler app for the oracle harness."""
    os.makedirs(out, exist_ok=True)
    ctl = CONTROLS.format(end_step=steps, dt=dt, npx=order, npy=order, npz=0, viscosity=0.0,
                          Pr=0.9, diffusion="NO", P0=100000, cp=1004.5, cv=717.5, gz=0)
    ctl = ctl.replace("time_scheme                  BDF1",
                      f"time_scheme                  {time_scheme}")
    setup = ctl
    ctl = ctl.replace("solver                       euler", "solver                       convection")
    ctl += "\nconvection\n{\n    t_UR            0.8\n    problem_init    LEVEQUE\n}\n"
    with open(os.path.join(out, "controls"), "w") as f:
        f.write(ctl)
    with open(os.path.join(out, "controls_setup"), "w") as f:
        f.write(setup)
    with open(os.path.join(out, "grid"), "w") as f:
        f.write(GRID_XY.format(nx=n, ny=n))
    files = {
        "T0.txt": (1, "cosine2 0 0.5    0.25 0.25 0.05   0.25 0.25 1", "NEUMANN"),
        "U0.txt": (3, "uniform 0 0 0", "SYMMETRY"),
        "p0.txt": (1, "uniform 0", "NEUMANN"),
        "rho0.txt": (1, "uniform 0", "NEUMANN"),
    }
    for name, (size, init, bc) in files.items():
        with open(os.path.join(out, name), "w") as f:
            f.write(FIELD.format(size=size, init=init, bc=bc))


def leveque_wind(cC, steps, dt):
    """The LEVEQUE wind's spatial part on every node and its time factor per
    step, with the C library's sin, cos and pow in the app's operation order
    (u = pow(sin(PI x), 2.0) * sin(2 PI y) * cos(PI t / T), t = i dt for step
    i = 1..steps, T = end_step dt; w = 0)."""
    import math
    PI = 3.14159265358979323846264
    xyz = cC.reshape(-1, 3)
    A = [[math.pow(math.sin(PI * x), 2.0) * math.sin(2 * PI * y),
          -math.pow(math.sin(PI * y), 2.0) * math.sin(2 * PI * x), 0.0] for x, y, _ in xyz]
    period = steps * dt
    scale = [math.cos(PI * (i * dt) / period) for i in range(1, steps + 1)]
    return A, scale


def write_case(out, *, dim, n, order, length, dt, steps, amp, center, radius, viscosity=0.0,
               Pr=0.9, solver="euler", wind=None, time_scheme="BDF1", P0=100000, cp=1004.5,
               cv=717.5, gz=-9.81, curved=None, refine=None, grading=None):
    os.makedirs(out, exist_ok=True)
    lx, ly, lz = length
    nx, ny, nz = n
    npy = 0 if dim == 2 else order
    with open(os.path.join(out, "controls"), "w") as f:
        ctl = CONTROLS.format(end_step=steps, dt=dt, npx=order, npy=npy, npz=order,
                              viscosity=viscosity, Pr=Pr,
                              diffusion="YES" if viscosity else "NO",
                              P0=P0, cp=cp, cv=cv, gz=gz)
        ctl = ctl.replace("time_scheme                  BDF1",
                          f"time_scheme                  {time_scheme}")
        if solver != "euler":
            ctl = ctl.replace("solver                       euler",
                              f"solver                       {solver}")
            ctl += "\n" + solver + "\n{\n    problem_init NONE\n}\n"
        if refine:
            ctl += REFINE.format(direction="0 1 0" if dim == 2 else "0 0 0",
                                 field_max=refine)
        f.write(ctl)
    grid = GRID_2D if dim == 2 else GRID_3D
    grid = grid.format(lx=lx, ly=ly, lz=lz, nx=nx, ny=ny, nz=nz)
    if curved:
        assert dim == 2, "curved variants are for the 2D block"
        grid = curved_grid(grid, curved, lx, ly, lz)
    if grading:
        # wall-graded block: grading = (counts, factors), e.g. odd counts that
        # the mesh app rounds up (hexMesh.cpp:51-66)
        counts, factors = grading
        old = "3{%d %d %d} 3{1 1 1}" % (nx, ny, nz)
        assert old in grid, "grading applies to the wall-spaced block"
        grid = grid.replace(old, "3{%d %d %d} 3{%r %r %r}" % (*counts, *factors))
    with open(os.path.join(out, "grid"), "w") as f:
        f.write(grid)
    cx, cy, cz = center
    rx, ry, rz = radius
    cos_init = f"cosine 0 {amp}    {cx} {cy} {cz}   {rx} {ry} {rz}"
    # the scalar convection case carries a uniform wind with zero-gradient walls
    U_init = "uniform 0 0 0" if wind is None else "uniform {} {} {}".format(*wind)
    U_bc = "SYMMETRY" if wind is None else "NEUMANN"
    files = {
        "T0.txt": (1, cos_init, "NEUMANN"),
        "U0.txt": (3, U_init, U_bc),
        "p0.txt": (1, "uniform 0", "NEUMANN"),
        "rho0.txt": (1, "uniform 0", "NEUMANN"),
    }
    for name, (size, init, bc) in files.items():
        with open(os.path.join(out, name), "w") as f:
            f.write(FIELD.format(size=size, init=init, bc=bc))


# Rising-bubble workloads (2D: one element thick in y, y faces deleted); the
# scalar convection cases reuse the meshes and the cosine bump as the scalar.
# The fluid constants of the reference's srtb example (its controls set
# viscosity 1.5 and gravity -9.80606 and leave P0, cp, cv at the Fluid::
# defaults of apps/utils/properties.cpp): pass as write_case(**SRTB_FLUID).
SRTB_FLUID = dict(P0=101325, cp=1004.67, cv=715.5, gz=-9.80606, viscosity=1.5)
CASES = {
    # 1000 x 1000 m, 10x10 elements, N=4, theta' = 0.25(1+cos(pi r/250))
    "c1_2d": dict(dim=2, n=(10, 1, 10), order=4, length=(1000, 100, 1000),
                  amp=0.5, center=(500, 50, 350), radius=(250, 1000, 250)),
    # 2000^3 m box, amplitude 0.5 K, radius 400 m, centre (1000,1000,600)
    "c2_32": dict(dim=3, n=(32, 32, 32), order=4, length=(2000, 2000, 2000),
                  amp=0.5, center=(1000, 1000, 600), radius=(400, 400, 400)),
    "c3_16n7": dict(dim=3, n=(16, 16, 16), order=7, length=(2000, 2000, 2000),
                    amp=0.5, center=(1000, 1000, 600), radius=(400, 400, 400)),
    "c4_16": dict(dim=3, n=(16, 16, 16), order=4, length=(2000, 2000, 2000),
                  amp=0.5, center=(1000, 1000, 600), radius=(400, 400, 400)),
    # small 3D cases for golden fixtures (same bubble, coarser meshes)
    "g3_2": dict(dim=3, n=(2, 2, 2), order=4, length=(2000, 2000, 2000),
                 amp=0.5, center=(1000, 1000, 600), radius=(400, 400, 400)),
    "g3_4n3": dict(dim=3, n=(4, 3, 2), order=3, length=(2000, 1500, 1000),
                   amp=0.5, center=(1000, 750, 300), radius=(400, 400, 400)),
    "g3_2n7": dict(dim=3, n=(2, 2, 2), order=7, length=(2000, 2000, 2000),
                   amp=0.5, center=(1000, 1000, 600), radius=(400, 400, 400)),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("out")
    ap.add_argument("--dt", type=float, default=0.01)
    ap.add_argument("--steps", type=int, default=10)
    a = ap.parse_args()
    write_case(a.out, dt=a.dt, steps=a.steps, **CASES[a.case])


if __name__ == "__main__":
    main()
