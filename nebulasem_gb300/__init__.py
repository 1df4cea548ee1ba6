"""GB300-native dGSEM Euler hot path of NebulaSEM, Python bindings.

The compute path is libnsem_gpu.so (hand-written sm_103a CUDA behind the C ABI
of include/nsem.h); this module only loads it with ctypes and converts numpy
arrays to the ABI's plain pointers.  There is no CPU fallback: if the library
cannot be loaded, every call raises.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libnsem_gpu.so")

FP64 = 0
MIXED = 1
SSPRK3 = 0
REF_SEGREGATED = 1

STATUS = {0: "OK", 1: "BAD_ARG", 2: "CUDA_ERROR", 3: "NONFINITE", 4: "TIMEOUT",
          5: "UNSUPPORTED", 6: "NO_MEMORY", 7: "TOO_LARGE"}
VARS = ("rho", "rhou", "rhov", "rhow", "rhotheta")

_lib = None


class NsemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("npx", ctypes.c_int32), ("npy", ctypes.c_int32), ("npz", ctypes.c_int32),
        ("npf", ctypes.c_int32), ("n_elem", ctypes.c_int32), ("n_cells", ctypes.c_int32),
        ("n_face", ctypes.c_int32),
        ("cC", ctypes.c_void_p), ("cV", ctypes.c_void_p), ("Jinv", ctypes.c_void_p),
        ("FO", ctypes.c_void_p), ("FN", ctypes.c_void_p), ("fN", ctypes.c_void_p),
        ("fI", ctypes.c_void_p), ("all_faces", ctypes.c_void_p),
        ("face_idx0", ctypes.c_void_p), ("face_idx1", ctypes.c_void_p),
        ("psi", ctypes.c_void_p * 3), ("dpsi", ctypes.c_void_p * 3),
        ("bc_U", ctypes.c_void_p),
        ("n_mortar", ctypes.c_int32), ("mortar", ctypes.c_void_p),
        ("psi_ref", ctypes.c_void_p * 6), ("psi_cor", ctypes.c_void_p * 6),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("P0", ctypes.c_double), ("T0", ctypes.c_double), ("cp", ctypes.c_double),
        ("cv", ctypes.c_double), ("gravity", ctypes.c_double * 3), ("dt", ctypes.c_double),
        ("p_ref", ctypes.c_void_p), ("rho_ref", ctypes.c_void_p), ("device", ctypes.c_int32),
        ("viscosity", ctypes.c_double), ("Pr", ctypes.c_double),
    ]


def load(build_if_missing=True):
    """Load libnsem_gpu.so (building it with nvcc first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError(f"{LIB_PATH} is missing; run nebulasem_gb300.build.build()")
        _build.build()
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    vp = ctypes.POINTER(ctypes.c_void_p)
    sigs = {
        "nsem_create": ([ctypes.POINTER(MeshDesc), ctypes.POINTER(Params), vp], ctypes.c_int),
        "nsem_destroy": ([P], None),
        "nsem_last_error": ([P], ctypes.c_char_p),
        "nsem_abi_version": ([], ctypes.c_int),
        "nsem_num_nodes": ([P], ctypes.c_int64),
        "nsem_stream": ([P], ctypes.c_void_p),
        "nsem_set_state": ([P, P, P, P], ctypes.c_int),
        "nsem_get_state": ([P, P, P, P], ctypes.c_int),
        "nsem_set_fields": ([P, P, P, P], ctypes.c_int),
        "nsem_get_fields": ([P, P, P, P], ctypes.c_int),
        "nsem_get_pressure": ([P, P], ctypes.c_int),
        "nsem_tendency": ([P, ctypes.c_int, vp, P], ctypes.c_int),
        "nsem_step": ([P, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "nsem_diagnostics": ([P, P, P, P], ctypes.c_int),
        "nsem_sync": ([P], ctypes.c_int),
        "nsem_profile": ([P, ctypes.c_int, ctypes.c_int, P, P, P], ctypes.c_int),
        "nsem_vjp": ([P, vp, vp], ctypes.c_int),
        "nsem_forward_checkpointed": ([P, ctypes.c_int, ctypes.c_int, P], ctypes.c_int),
        "nsem_adjoint": ([P, vp, vp, P], ctypes.c_int),
        "nsem_forward_checkpointed_prec": ([P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P],
                                           ctypes.c_int),
        "nsem_vjp_prec": ([P, ctypes.c_int, vp, vp], ctypes.c_int),
        "nsem_jvp": ([P, vp, vp], ctypes.c_int),
        "nsem_convection_set": ([P, P, P], ctypes.c_int),
        "nsem_convection_step": ([P, ctypes.c_int], ctypes.c_int),
        "nsem_convection_get": ([P, P], ctypes.c_int),
        "nsem_convection_wind": ([P, P, ctypes.c_int], ctypes.c_int),
        "nsem_convection_step_scaled": ([P, ctypes.c_int, P], ctypes.c_int),
        "nsem_tlm": ([P, ctypes.c_int, vp, vp, P], ctypes.c_int),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))


def _u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32).reshape(-1))


class Solver:
    """One libnsem_gpu context: mesh + state on one GPU.

    ``mesh`` is a dict in the reference's layout (the keys of the golden
    fixtures: meta, cC, cV, Jinv, FO, FN, fN, fI, allFaces, faceIdx0,
    faceIdx1, psi0-2, dpsi0-2, bcU and optionally p_ref, rho_ref).  Fluid
    constants not given as arguments come from the dict's P0, T0, cp, cv,
    gravity, viscosity, Pr when present, else 1e5, 300, 1004.5, 717.5,
    (0, 0, -9.81), 0, 0.9.
    """

    def __init__(self, mesh, dt, P0=None, T0=None, cp=None, cv=None, gravity=None, device=0,
                 use_ref_background=True, viscosity=None, Pr=None):
        def const(name, given, default):
            if given is not None:
                return given
            return mesh[name] if name in mesh else default
        P0 = float(const("P0", P0, 1e5))
        T0 = float(const("T0", T0, 300.0))
        cp = float(const("cp", cp, 1004.5))
        cv = float(const("cv", cv, 717.5))
        gravity = [float(x) for x in np.asarray(const("gravity", gravity, (0.0, 0.0, -9.81)))]
        lib = load()
        meta = np.asarray(mesh["meta"], dtype=np.int64)
        npx, npy, npz, np_, npf = (int(v) for v in meta[:5])
        n_elem, n_cells, n_int, n_all, n_face = (int(v) for v in meta[5:10])
        self.n_int = n_int
        self.n_all = n_all
        keep = {
            "cC": _f64(mesh["cC"]), "cV": _f64(mesh["cV"]), "Jinv": _f64(mesh["Jinv"]),
            "FO": _u32(mesh["FO"]), "FN": _u32(mesh["FN"]), "fN": _f64(mesh["fN"]),
            "fI": _f64(mesh["fI"]), "allFaces": _u32(mesh["allFaces"]),
            "faceIdx0": _u32(mesh["faceIdx0"]), "faceIdx1": _u32(mesh["faceIdx1"]),
            "bcU": _u32(mesh["bcU"]),
        }
        for d in range(3):
            keep[f"psi{d}"] = _f64(mesh[f"psi{d}"])
            keep[f"dpsi{d}"] = _f64(mesh[f"dpsi{d}"])
        md = MeshDesc()
        md.npx, md.npy, md.npz, md.npf = npx, npy, npz, npf
        md.n_elem, md.n_cells, md.n_face = n_elem, n_cells, n_face
        md.cC, md.cV, md.Jinv = _p(keep["cC"]), _p(keep["cV"]), _p(keep["Jinv"])
        md.FO, md.FN, md.fN, md.fI = _p(keep["FO"]), _p(keep["FN"]), _p(keep["fN"]), _p(keep["fI"])
        md.all_faces = _p(keep["allFaces"])
        md.face_idx0 = _p(keep["faceIdx0"])
        md.face_idx1 = _p(keep["faceIdx1"])
        md.bc_U = _p(keep["bcU"])
        for d in range(3):
            md.psi[d] = keep[f"psi{d}"].ctypes.data
            md.dpsi[d] = keep[f"dpsi{d}"].ctypes.data
        # non-conforming faces of an adaptively refined mesh (the harness's
        # `mortar` and psiRef/psiCor dumps)
        if "mortar" in mesh and len(mesh["mortar"]):
            keep["mortar"] = _u32(mesh["mortar"])
            md.n_mortar = len(keep["mortar"]) // 4
            md.mortar = _p(keep["mortar"])
            for d in range(3):
                for h in range(2):
                    for nm, arr in (("psiRef", md.psi_ref), ("psiCor", md.psi_cor)):
                        keep[f"{nm}{d}{h}"] = _f64(mesh[f"{nm}{d}{h}"])
                        arr[d * 2 + h] = keep[f"{nm}{d}{h}"].ctypes.data
        pr = Params()
        pr.P0, pr.T0, pr.cp, pr.cv, pr.dt = P0, T0, cp, cv, dt
        for c in range(3):
            pr.gravity[c] = gravity[c]
        if use_ref_background and "p_ref" in mesh and "rho_ref" in mesh:
            keep["p_ref"] = _f64(mesh["p_ref"])
            keep["rho_ref"] = _f64(mesh["rho_ref"])
            pr.p_ref = _p(keep["p_ref"])
            pr.rho_ref = _p(keep["rho_ref"])
        pr.device = device
        # artificial viscosity of the segregated scheme (diffusion YES)
        pr.viscosity = float(mesh.get("viscosity", 0.0) if viscosity is None else viscosity)
        pr.Pr = float(mesh.get("Pr", 0.9) if Pr is None else Pr)
        ctx = ctypes.c_void_p()
        st = lib.nsem_create(ctypes.byref(md), ctypes.byref(pr), ctypes.byref(ctx))
        self._ctx = ctx
        if st != 0:
            msg = lib.nsem_last_error(ctx).decode() if ctx.value else ""
            if ctx.value:
                lib.nsem_destroy(ctx)
            self._ctx = None
            raise NsemError(st, msg)
        self._lib = lib
        self.dt = dt

    def _check(self, st):
        if st != 0:
            raise NsemError(st, self._lib.nsem_last_error(self._ctx).decode())

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.nsem_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return self._lib.nsem_stream(self._ctx)

    def set_state(self, u):
        """u: list of 5 arrays (rho, rhou, rhov, rhow, rhotheta) on interior nodes."""
        rho = _f64(u[0])
        mom = np.ascontiguousarray(np.stack([_f64(u[1]), _f64(u[2]), _f64(u[3])], axis=1))
        rt = _f64(u[4])
        self._check(self._lib.nsem_set_state(self._ctx, _p(rho), _p(mom), _p(rt)))
        self._check(self._lib.nsem_sync(self._ctx))

    def set_state_raw(self, rho, rho_u_aos, rho_theta):
        """Copy a state from caller-owned (ideally pinned) host arrays; rho_u_aos is (n, 3)."""
        self._check(self._lib.nsem_set_state(self._ctx, _p(rho), _p(rho_u_aos), _p(rho_theta)))

    def get_state_raw(self, rho, rho_u_aos, rho_theta):
        """Copy the state into caller-owned host arrays (synchronises)."""
        self._check(self._lib.nsem_get_state(self._ctx, _p(rho), _p(rho_u_aos), _p(rho_theta)))

    def profile(self, nsteps, prec=FP64):
        """Run nsteps un-graphed with CUDA events around every launch.

        Returns {kernel: (total_ms, launches)} for the kernel classes of the
        step (prim, face, volume for the plain form)."""
        ms = (ctypes.c_double * 8)()
        cnt = (ctypes.c_int * 8)()
        names = ctypes.create_string_buffer(8 * 32)
        self._check(self._lib.nsem_profile(self._ctx, int(nsteps), prec, ms, cnt, names))
        out = {}
        raw = names.raw
        for i in range(8):
            nm = raw[32 * i: 32 * (i + 1)].split(b"\0", 1)[0].decode()
            if nm:
                out[nm] = (ms[i], cnt[i])
        return out

    def vjp(self, w, prec=FP64):
        """g = J_L(u)^T w at the current state (plain or precision form)."""
        n = self.n_int
        ws = [_f64(a) for a in w]
        g = [np.empty(n) for _ in range(5)]
        wa = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in ws])
        ga = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in g])
        self._check(self._lib.nsem_vjp_prec(self._ctx, int(prec), wa, ga))
        return g

    def jvp(self, dv):
        """Ld = J_L(u) dv at the current state (plain form)."""
        n = self.n_int
        ds = [_f64(a) for a in dv]
        out = [np.empty(n) for _ in range(5)]
        da = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in ds])
        oa = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in out])
        self._check(self._lib.nsem_jvp(self._ctx, da, oa))
        return out

    def tlm(self, nsteps, du0):
        """Advance nsteps FP64 steps carrying the perturbation du0 through the
        linearised steps.  Returns (du_final, device ms)."""
        n = self.n_int
        ds = [_f64(a) for a in du0]
        out = [np.empty(n) for _ in range(5)]
        da = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in ds])
        oa = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in out])
        ms = ctypes.c_double()
        self._check(self._lib.nsem_tlm(self._ctx, int(nsteps), da, oa, ctypes.byref(ms)))
        return out, ms.value

    def forward_checkpointed(self, nsteps, ckpt_every, prec=FP64):
        """Advance nsteps steps in the given form keeping checkpoints;
        returns device ms.  adjoint() then differentiates this run."""
        ms = ctypes.c_double()
        self._check(self._lib.nsem_forward_checkpointed_prec(
            self._ctx, int(nsteps), int(ckpt_every), int(prec), ctypes.byref(ms)))
        return ms.value

    def adjoint(self, lam_final):
        """dJ/du0 from dJ/du_final for the last checkpointed forward run.
        Returns (lam0, device ms of the reverse sweep)."""
        n = self.n_int
        ls = [_f64(a) for a in lam_final]
        out = [np.empty(n) for _ in range(5)]
        la = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in ls])
        oa = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in out])
        ms = ctypes.c_double()
        self._check(self._lib.nsem_adjoint(self._ctx, la, oa, ctypes.byref(ms)))
        return out, ms.value

    def set_fields(self, rho, U, T):
        """The euler app's fields: rho, U (n_int x 3), T = theta' (kept as given)."""
        r = _f64(rho)
        u = np.ascontiguousarray(np.asarray(U, dtype=np.float64).reshape(-1, 3))
        t = _f64(T)
        self._check(self._lib.nsem_set_fields(self._ctx, _p(r), _p(u), _p(t)))

    def get_fields(self):
        n = self.n_int
        r, u, t = np.empty(n), np.empty((n, 3)), np.empty(n)
        self._check(self._lib.nsem_get_fields(self._ctx, _p(r), _p(u), _p(t)))
        return r, u, t

    def get_pressure(self):
        """p - p_ref as the euler app holds it (after a segregated step: the p'
        of that step, from rho^{n+1} and theta^n; otherwise of the state)."""
        p = np.empty(self.n_int)
        self._check(self._lib.nsem_get_pressure(self._ctx, _p(p)))
        return p

    def convection_set(self, U, T):
        """Scalar DG convection: the fixed wind U (n_int x 3) and the scalar T."""
        u = np.ascontiguousarray(np.asarray(U, dtype=np.float64).reshape(-1, 3))
        t = _f64(T)
        self._check(self._lib.nsem_convection_set(self._ctx, _p(u), _p(t)))

    def convection_step(self, nsteps):
        self._check(self._lib.nsem_convection_step(self._ctx, int(nsteps)))

    def convection_wind(self, U_all=None, time_scheme=1):
        """Analytic wind (spatial part on all n_all nodes, (n_all, 3)) and the
        time scheme (1: BDF1/AB1, 2: AB2) of the convection app."""
        u = None if U_all is None else _f64(np.asarray(U_all).reshape(-1))
        self._check(self._lib.nsem_convection_wind(self._ctx, _p(u) if u is not None else None,
                                                   int(time_scheme)))

    def convection_step_scaled(self, nsteps, scale=None):
        """nsteps steps with the wind's spatial part times scale[s]."""
        sc = None if scale is None else _f64(scale)
        self._check(self._lib.nsem_convection_step_scaled(
            self._ctx, int(nsteps), _p(sc) if sc is not None else None))

    def convection_get(self):
        t = np.empty(self.n_int)
        self._check(self._lib.nsem_convection_get(self._ctx, _p(t)))
        return t

    def get_state(self):
        n = self.n_int
        rho, mom, rt = np.empty(n), np.empty((n, 3)), np.empty(n)
        self._check(self._lib.nsem_get_state(self._ctx, _p(rho), _p(mom), _p(rt)))
        return [rho, mom[:, 0].copy(), mom[:, 1].copy(), mom[:, 2].copy(), rt]

    def tendency(self, prec=FP64, return_p=False):
        n = self.n_int
        L = [np.empty(n) for _ in range(5)]
        arr = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in L])
        p = np.empty(n)
        self._check(self._lib.nsem_tendency(self._ctx, prec, arr, _p(p)))
        return (L, p) if return_p else L

    def step(self, nsteps, prec=FP64, sync=True, scheme=SSPRK3):
        self._check(self._lib.nsem_step(self._ctx, int(nsteps), scheme, prec))
        if sync:
            self._check(self._lib.nsem_sync(self._ctx))

    def sync(self):
        self._check(self._lib.nsem_sync(self._ctx))

    def diagnostics(self):
        m, e, v = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self._lib.nsem_diagnostics(self._ctx, ctypes.byref(m), ctypes.byref(e),
                                               ctypes.byref(v)))
        return np.array([m.value, e.value, v.value])


# Algorithmic HBM bytes per DOF of one SSP-RK3 stage: the compulsory FP64
# state traffic of the Shu-Osher stages (stage 1 reads u^n, writes u1; stage 2
# reads u1 and u^n, writes u2; stage 3 reads u2 and u^n, writes u^{n+1}), the
# same figure for both forms because both keep the RK state in FP64.
ALG_BYTES_PER_DOF_STAGE = {1: 16.0, 2: 24.0, 3: 24.0}
ALG_BYTES_PER_DOF_STAGE_AVG = 64.0 / 3.0


def mixed_own_bytes_per_node_stage():
    """HBM bytes per node that the precision form's own layout must move, by
    stage: stage 1 reads the FP32 shadow of u'^n and writes the FP32 increment
    (20 + 20 B); stage 2 reads the shadow and the first increment and writes the
    second (60 B); stage 3 reads u'^n (FP64), its shadow and the second
    increment and writes u'^{n+1} and its shadow (40 + 20 + 20 + 40 + 20 B).
    240 B per node and step, 16 B per DOF-stage."""
    return {1: 40.0, 2: 60.0, 3: 140.0}
