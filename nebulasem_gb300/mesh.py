"""Host-side mesh and initial state for rising-bubble box workloads.

Produces the arrays of the reference's Mesh:: / DG:: layout (the layout the
C ABI takes) for a uniform box of hexahedral elements, with the reference's
conventions:
  - LGL nodes/weights by Newton iteration from Chebyshev guesses and the
    Lagrange basis / derivative tables, as src/field/dg.cpp:32-143;
  - element order z fastest, then y, then x; element face lists in the order
    z-, z+, y-, y+, x-, x+ (src/field/dg.cpp:172 face_map, mesh.cpp
    fixHexCells); one ghost "boundary cell" per boundary face;
  - face slots and weights of DG::init_geom (dg.cpp:323-410): owner node on
    the face, neighbour node opposite, fN = area normal * w_a w_b / 4,
    fI = 0.5 inside and 0 on the boundary, unused slots -> sentinel n_all;
  - node mass weight cV = V * (w_i w_j w_k / 8) (dg.cpp:315-318), metric
    Jinv = diag(2/h) with collapsed directions zeroed (dg.cpp:412-476);
  - 2D ("npy 0"): one element thick in y, y faces deleted.
The node coordinates and metrics are the exact affine values, so they can
differ from the reference's transfinite-interpolation coordinates in the
last bits; the golden fixtures carry the reference's own geometry.
"""
import math

import numpy as np

XX, YY, ZZ, XY, YZ, XZ, YX, ZY, ZX = range(9)
TIDX = ((XX, XY, XZ), (YX, YY, YZ), (ZX, ZY, ZZ))   # tensor component (row, column)


def legendre(p, x):
    """P_p(x) and its first two derivatives by the three-term recurrence."""
    L1 = L1_1 = L1_2 = 0.0
    L0, L0_1, L0_2 = 1.0, 0.0, 0.0
    for i in range(1, p + 1):
        L2, L2_1, L2_2 = L1, L1_1, L1_2
        L1, L1_1, L1_2 = L0, L0_1, L0_2
        a = (2 * i - 1.0) / i
        b = (i - 1.0) / i
        L0 = a * x * L1 - b * L2
        L0_1 = a * (L1 + x * L1_1) - b * L2_1
        L0_2 = a * (2 * L1_1 + x * L1_2) - b * L2_2
    return L0, L0_1, L0_2


def lgl(n):
    """n Legendre-Gauss-Lobatto nodes and weights on [-1, 1]."""
    x = np.zeros(n)
    w = np.zeros(n)
    if n == 1:
        return np.array([0.0]), np.array([2.0])
    p = n - 1
    ph = n // 2
    pi = 3.14159265358979323846264
    for i in range(ph):
        xi = math.cos((2 * i + 1) * pi / (2 * n))
        for _ in range(20):
            L0, L0_1, L0_2 = legendre(p, xi)
            dx = -(1 - xi * xi) * L0_1 / (-2 * xi * L0_1 + (1 - xi * xi) * L0_2)
            xi += dx
            if abs(dx) < 1.0e-20:
                break
        x[p - i] = xi
        w[p - i] = 2 / (p * (p + 1) * L0 * L0)
    if n != 2 * ph:
        L0, _, _ = legendre(p, 0.0)
        x[ph] = 0.0
        w[ph] = 2 / (p * (p + 1) * L0 * L0)
    for i in range(ph):
        x[i] = -x[p - i]
        w[i] = +w[p - i]
    return x, w


def lagrange_tables(xg):
    """psi[j*n+s] = l_j(x_s); dpsi[s*n+i] = l_i'(x_s) (dg.cpp:103-143)."""
    n = len(xg)
    psi = np.zeros(n * n)
    dpsi = np.zeros(n * n)
    for s in range(n):
        x = xg[s]
        for j in range(n):
            prod = 1.0
            for k in range(n):
                if k != j:
                    prod *= (x - xg[k]) / (xg[j] - xg[k])
            psi[j * n + s] = prod
    for s in range(n):
        x = xg[s]
        for i in range(n):
            acc = 0.0
            for j in range(n):
                if i != j:
                    prod = 1.0
                    for k in range(n):
                        if k != i and k != j:
                            prod *= (x - xg[k]) / (xg[i] - xg[k])
                    acc += prod / (xg[i] - xg[j])
            dpsi[s * n + i] = acc
    return psi, dpsi


def rotation_y(deg):
    """Rotation matrix about the y axis by deg degrees (x towards -z)."""
    c, s = np.cos(np.radians(deg)), np.sin(np.radians(deg))
    return np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])


def box_mesh(n, order, length, dim=3, tilt=0.0):
    """Uniform box of n = (nx, ny, nz) elements of order N; dim=2 collapses y.
    tilt: the box rotated by that many degrees about the y axis through its
    centre (inclined elements: full metric Jinv = R diag(2/h), normals R fN)."""
    nx, ny, nz = n
    if dim == 2:
        ny = 1
    NPX = order + 1
    NPY = order + 1 if dim == 3 else 1
    NPZ = order + 1
    NP = NPX * NPY * NPZ
    if NPX <= NPY and NPX <= NPZ:
        NPF = NPY * NPZ
    elif NPY <= NPX and NPY <= NPZ:
        NPF = NPX * NPZ
    else:
        NPF = NPX * NPY
    tabs = [lgl(NPX), lgl(NPY), lgl(NPZ)]
    xg = [t[0] for t in tabs]
    wg = [t[1] for t in tabs]
    lt = [lagrange_tables(x) for x in xg]
    hx, hy, hz = length[0] / nx, length[1] / ny, length[2] / nz
    ne = nx * ny * nz

    # element indices
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ix, iy, iz = ix.reshape(-1), iy.reshape(-1), iz.reshape(-1)

    def eid(a, b, c):
        return (a * ny + b) * nz + c

    # faces: interior z, y, x, then boundary z-, z+, y-, y+, x-, x+
    sides = [(2, -1), (2, +1), (1, -1), (1, +1), (0, -1), (0, +1)]  # (axis, sign) per face id
    area = {0: hy * hz, 1: hx * hz, 2: hx * hy}
    stride = {0: ny * nz, 1: nz, 2: 1}
    eidx = np.arange(ne)
    coord = {0: ix, 1: iy, 2: iz}
    lim = {0: nx, 1: ny, 2: nz}
    elem_faces = np.full((ne, 6), -1, dtype=np.int64)
    groups = []  # (owner elems, neighbour cells, face_o, normal, face ids, interior?)
    nf = 0
    for axis, fo in ((2, 1), (1, 3), (0, 5)):
        if dim == 2 and axis == 1:
            continue
        own = eidx[coord[axis] < lim[axis] - 1]
        nb = own + stride[axis]
        fid = nf + np.arange(len(own))
        nf += len(own)
        elem_faces[own, fo] = fid
        elem_faces[nb, fo - 1] = fid
        nv = [0.0, 0.0, 0.0]
        nv[axis] = area[axis]
        groups.append((own, nb, fo, nv, fid, True))
    n_bf = 0
    bgroups = []
    for fo, (axis, sgn) in enumerate(sides):
        if dim == 2 and axis == 1:
            continue
        own = eidx[coord[axis] == (0 if sgn < 0 else lim[axis] - 1)]
        fid = nf + np.arange(len(own))
        nf += len(own)
        elem_faces[own, fo] = fid
        ghost = ne + n_bf + np.arange(len(own))
        n_bf += len(own)
        nv = [0.0, 0.0, 0.0]
        nv[axis] = sgn * area[axis]
        groups.append((own, ghost, fo, nv, fid, False))
        bgroups.append(fid)
    n_cells = ne + n_bf
    n_int = ne * NP
    n_all = n_cells * NP

    # node coordinates, weights, metric
    li, lj, lk = np.meshgrid(np.arange(NPX), np.arange(NPY), np.arange(NPZ), indexing="ij")
    li, lj, lk = li.reshape(-1), lj.reshape(-1), lk.reshape(-1)
    rx = (xg[0][li] + 1) / 2
    ry = (xg[1][lj] + 1) / 2
    rz = (xg[2][lk] + 1) / 2
    cC = np.zeros((n_all, 3))
    cC[:n_int, 0] = (ix[:, None] * hx + rx[None, :] * hx).reshape(-1)
    cC[:n_int, 1] = (iy[:, None] * hy + ry[None, :] * hy).reshape(-1)
    cC[:n_int, 2] = (iz[:, None] * hz + rz[None, :] * hz).reshape(-1)
    wgt = wg[0][li] * wg[1][lj] * wg[2][lk] / 8
    V = hx * hy * hz
    cV = np.zeros(n_all)
    cV[:n_int] = np.tile(V * wgt, ne)
    J = np.zeros(9)
    J[XX] = 2.0 / hx if NPX > 1 else 0.0
    J[YY] = 2.0 / hy if NPY > 1 else 0.0
    J[ZZ] = 2.0 / hz if NPZ > 1 else 0.0
    Jinv = np.zeros((n_all, 9))
    Jinv[:n_int] = J

    # face slots (dg.cpp:323-410)
    FO = np.full(nf * NPF, n_all, dtype=np.uint32)
    FN = np.full(nf * NPF, n_all, dtype=np.uint32)
    fN = np.zeros((nf * NPF, 3))
    fI = np.zeros(nf * NPF)
    bcU = np.zeros(nf * NPF, dtype=np.uint32)
    face_map = [0, NPZ - 1, 0, NPY - 1, 0, NPX - 1]

    def local(fo, a, b, v):
        if fo in (0, 1):
            return a * NPY * NPZ + b * NPZ + v          # (i, j, v)
        if fo in (2, 3):
            return a * NPY * NPZ + v * NPZ + b          # (i, v, k)
        return v * NPY * NPZ + a * NPZ + b              # (v, j, k)

    for own, nb, fo, nv, fid, interior in groups:
        vo, vn = face_map[fo], face_map[fo ^ 1]
        if fo in (0, 1):
            ra, rb, wa, wb = NPX, NPY, wg[0], wg[1]
        elif fo in (2, 3):
            ra, rb, wa, wb = NPX, NPZ, wg[0], wg[2]
        else:
            ra, rb, wa, wb = NPY, NPZ, wg[1], wg[2]
        A, B = np.meshgrid(np.arange(ra), np.arange(rb), indexing="ij")
        A, B = A.reshape(-1), B.reshape(-1)
        k = (fid[:, None] * NPF + (A * rb + B)[None, :]).reshape(-1)
        o = (own[:, None] * NP + local(fo, A, B, vo)[None, :]).reshape(-1)
        nn = (nb[:, None] * NP + local(fo, A, B, vn)[None, :]).reshape(-1)
        w = np.tile(wa[A] * wb[B] / 4, len(fid))
        FO[k] = o
        FN[k] = nn
        fN[k, 0] = nv[0] * w
        fN[k, 1] = nv[1] * w
        fN[k, 2] = nv[2] * w
        if interior:
            fI[k] = 0.5
        else:
            bcU[k] = 2
            cC[nn] = cC[o]
            cV[nn] = cV[o]

    # cell face lists (interior: z-, z+, y-, y+, x-, x+; ghost: its face)
    order_ids = [0, 1, 2, 3, 4, 5] if dim == 3 else [0, 1, 4, 5]
    nfe = len(order_ids)
    bf = np.concatenate(bgroups) if bgroups else np.zeros(0, dtype=np.int64)
    all_faces = np.concatenate([elem_faces[:, order_ids].reshape(-1), bf]).astype(np.uint32)
    idx0 = np.concatenate([np.arange(ne) * nfe, ne * nfe + np.arange(n_bf)]).astype(np.uint32)
    idx1 = (idx0 + 1).astype(np.uint32)
    idx1[:ne] = idx0[:ne] + nfe

    if tilt:
        R = rotation_y(tilt)
        c0 = np.asarray(length, dtype=np.float64) / 2
        cC = (cC - c0) @ R.T + c0
        Jd = J[[XX, YY, ZZ]]
        for r in range(3):
            for c in range(3):
                Jinv[:n_int, TIDX[r][c]] = R[r, c] * Jd[c]
        fN = fN @ R.T

    meta = np.zeros(16, dtype=np.uint32)
    meta[:11] = [NPX, NPY, NPZ, NP, NPF, ne, n_cells, n_int, n_all, nf, len(all_faces)]
    out = {
        "meta": meta, "cC": cC.reshape(-1), "cV": cV, "Jinv": Jinv.reshape(-1),
        "FO": FO, "FN": FN, "fN": fN.reshape(-1), "fI": fI,
        "allFaces": all_faces, "faceIdx0": idx0,
        "faceIdx1": idx1, "bcU": bcU,
    }
    for d in range(3):
        out[f"xgl{d}"], out[f"wgl{d}"] = xg[d], wg[d]
        out[f"psi{d}"], out[f"dpsi{d}"] = lt[d]
    return out


def bubble_state(mesh, amp, center, radius, P0=1e5, T0=300.0, cp=1004.5, cv=717.5,
                 gravity=(0.0, 0.0, -9.81)):
    """Rising-bubble initial state (euler.cpp:104-149 with the field-file
    initialisers `cosine 0 amp c r` for T and `uniform 0` for U and p).

    Returns (u, p_ref, rho_ref, gh): conserved state on interior nodes and the
    hydrostatic background on all nodes.
    """
    n_int = int(mesh["meta"][7])
    n_all = int(mesh["meta"][8])
    cC = np.asarray(mesh["cC"]).reshape(-1, 3)[:n_all]
    R = cp - cv
    gam = cp / cv
    g = np.asarray(gravity, dtype=np.float64)
    gh = cC[:, 0] * g[0] + (cC[:, 1] * g[1] + (cC[:, 2] * g[2] + 0.0))
    p_ref = P0 * np.power(1.0 + gh / (cp * T0), cp / R)
    rho_ref = (P0 / (R * T0)) * np.power(p_ref / P0, 1 / gam)
    d = (cC - np.asarray(center)) / np.asarray(radius)
    r = np.sqrt(d[:, 0] * d[:, 0] + (d[:, 1] * d[:, 1] + (d[:, 2] * d[:, 2] + 0.0)))
    r = np.minimum(1.0, r)
    theta_p = 0.0 + (amp / 2) * (1.0 + np.cos(r * 3.14159265358979323846264))
    p = 0.0 + p_ref
    rho = (P0 / (R * (theta_p + T0))) * np.power(p / P0, 1 / gam)
    rho = rho[:n_int]
    th = theta_p[:n_int] + T0
    u = [rho.copy(), np.zeros(n_int), np.zeros(n_int), np.zeros(n_int), rho * th]
    return u, p_ref, rho_ref, gh


WORKLOADS = {
    # 2D bubble: 1000 x 1000 m, 10 x 10 elements, N = 4 (one element thick in y)
    "bubble2d_10x10_n4": dict(n=(10, 1, 10), order=4, length=(1000.0, 100.0, 1000.0), dim=2,
                              amp=0.5, center=(500.0, 50.0, 350.0), radius=(250.0, 1000.0, 250.0)),
    # 3D bubble, 2000^3 m box, theta' amplitude 0.5 K, radius 400 m, centre (1000,1000,600)
    "bubble3d_32_n4": dict(n=(32, 32, 32), order=4, length=(2000.0,) * 3, dim=3,
                           amp=0.5, center=(1000.0, 1000.0, 600.0), radius=(400.0,) * 3),
    "bubble3d_16_n7": dict(n=(16, 16, 16), order=7, length=(2000.0,) * 3, dim=3,
                           amp=0.5, center=(1000.0, 1000.0, 600.0), radius=(400.0,) * 3),
    "bubble3d_16_n4": dict(n=(16, 16, 16), order=4, length=(2000.0,) * 3, dim=3,
                           amp=0.5, center=(1000.0, 1000.0, 600.0), radius=(400.0,) * 3),
    "bubble3d_48_n4": dict(n=(48, 48, 48), order=4, length=(2000.0,) * 3, dim=3,
                           amp=0.5, center=(1000.0, 1000.0, 600.0), radius=(400.0,) * 3),
    "bubble3d_8_n4": dict(n=(8, 8, 8), order=4, length=(2000.0,) * 3, dim=3,
                          amp=0.5, center=(1000.0, 1000.0, 600.0), radius=(400.0,) * 3),
    # the 32^3 and 16^3 boxes tilted by 30 degrees about y (inclined elements:
    # the precision form's general-geometry kernels), bubble tilted with them
    "bubble3d_32_n4_tilt30": dict(n=(32, 32, 32), order=4, length=(2000.0,) * 3, dim=3, tilt=30.0,
                                  amp=0.5, center=(1000.0, 1000.0, 600.0), radius=(400.0,) * 3),
    "bubble3d_16_n4_tilt30": dict(n=(16, 16, 16), order=4, length=(2000.0,) * 3, dim=3, tilt=30.0,
                                  amp=0.5, center=(1000.0, 1000.0, 600.0), radius=(400.0,) * 3),
}


def workload(name):
    """Mesh dict (with background fields) and initial state of a named workload."""
    w = WORKLOADS[name]
    tilt = w.get("tilt", 0.0)
    m = box_mesh(w["n"], w["order"], w["length"], dim=w["dim"], tilt=tilt)
    center = np.asarray(w["center"], dtype=np.float64)
    if tilt:
        c0 = np.asarray(w["length"], dtype=np.float64) / 2
        center = rotation_y(tilt) @ (center - c0) + c0
    u, p_ref, rho_ref, gh = bubble_state(m, w["amp"], center, w["radius"])
    m["p_ref"], m["rho_ref"], m["gh"] = p_ref, rho_ref, gh
    return m, u
