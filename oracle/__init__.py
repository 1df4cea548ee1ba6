"""Python access to the oracle (test infrastructure only).

The oracle is a C restatement of the reference's dGSEM Euler operator chain
(oracle/nsem_oracle.c), pinned bit for bit against golden fixtures produced by
the reference library itself (oracle/ref_harness.cpp, tests/golden/).  Only
tests, the smoke check and the benchmark's CPU-baseline leg use it; the
shipped library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libnsem_oracle.so")
_lib = None

VARS = ("rho", "rhou", "rhov", "rhow", "rhotheta")


def build(force=False):
    """Compile the C restatement with make (gcc, OpenMP, no FP contraction)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Mesh(ctypes.Structure):
    _fields_ = [
        ("npx", ctypes.c_int32), ("npy", ctypes.c_int32), ("npz", ctypes.c_int32),
        ("np", ctypes.c_int32), ("npf", ctypes.c_int32),
        ("n_elem", ctypes.c_int32), ("n_cells", ctypes.c_int32),
        ("n_int", ctypes.c_int32), ("n_all", ctypes.c_int32), ("n_face", ctypes.c_int32),
        ("cC", ctypes.c_void_p), ("cV", ctypes.c_void_p), ("Jinv", ctypes.c_void_p),
        ("FO", ctypes.c_void_p), ("FN", ctypes.c_void_p),
        ("fN", ctypes.c_void_p), ("fI", ctypes.c_void_p),
        ("all_faces", ctypes.c_void_p), ("face_idx0", ctypes.c_void_p),
        ("face_idx1", ctypes.c_void_p),
        ("psi", ctypes.c_void_p * 3), ("dpsi", ctypes.c_void_p * 3),
        ("bcU", ctypes.c_void_p), ("p_ref", ctypes.c_void_p), ("rho_ref", ctypes.c_void_p),
        ("gravity", ctypes.c_double * 3),
        ("P0", ctypes.c_double), ("R", ctypes.c_double), ("gamma", ctypes.c_double),
        ("T0", ctypes.c_double), ("nu", ctypes.c_double), ("Pr", ctypes.c_double),
        ("n_mortar", ctypes.c_int32), ("mortar", ctypes.c_void_p),
        ("psi_ref", ctypes.c_void_p * 6), ("psi_cor", ctypes.c_void_p * 6),
    ]


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER(ctypes.c_void_p)
        _lib.nsem_oracle_tendency.argtypes = [ctypes.POINTER(_Mesh), P, P, ctypes.c_void_p]
        _lib.nsem_oracle_ssprk3.argtypes = [ctypes.POINTER(_Mesh), P, ctypes.c_double, ctypes.c_int]
        _lib.nsem_oracle_diagnostics.argtypes = [ctypes.POINTER(_Mesh), P, ctypes.c_void_p,
                                                 ctypes.c_double, ctypes.c_void_p]
        _lib.nsem_oracle_pow_dd.argtypes = [ctypes.c_double, ctypes.c_double]
        _lib.nsem_oracle_pow_dd.restype = ctypes.c_double
        _lib.nsem_oracle_pow_dd_accurate.argtypes = [ctypes.c_double, ctypes.c_double]
        _lib.nsem_oracle_pow_dd_accurate.restype = ctypes.c_double
        D = ctypes.POINTER(ctypes.c_double)
        _lib.nsem_oracle_pow_fast_core.argtypes = [ctypes.c_double, ctypes.c_double, D, D, D,
                                                   ctypes.POINTER(ctypes.c_int)]
        _lib.nsem_oracle_pow_fast_core.restype = ctypes.c_int
        I64 = ctypes.POINTER(ctypes.c_int64)
        _lib.nsem_oracle_pow_fast_sweep.argtypes = [ctypes.c_int64, ctypes.c_uint64, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_double, I64, I64]
        _lib.nsem_oracle_set_pow.argtypes = [ctypes.c_int]
        _lib.nsem_oracle_threads.restype = ctypes.c_int
        _lib.nsem_oracle_jvp.argtypes = [ctypes.POINTER(_Mesh), P, P, P, P]
        _lib.nsem_oracle_tlm_ssprk3.argtypes = [ctypes.POINTER(_Mesh), P, P, ctypes.c_double,
                                                ctypes.c_int]
        _lib.nsem_oracle_tlm_ssprk3_multi.argtypes = [ctypes.POINTER(_Mesh), P, P, ctypes.c_int,
                                                      ctypes.c_double, ctypes.c_int]
        _lib.nsem_oracle_tlm_ssprk3_multi.restype = ctypes.c_int
        _lib.nsem_oracle_segregated.argtypes = [ctypes.POINTER(_Mesh), ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_double, ctypes.c_int]
        _lib.nsem_oracle_convection.argtypes = [ctypes.POINTER(_Mesh), ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        _lib.nsem_oracle_convection_wind.argtypes = [ctypes.POINTER(_Mesh), ctypes.c_void_p,
                                                     ctypes.c_void_p, ctypes.c_int,
                                                     ctypes.c_void_p, ctypes.c_double,
                                                     ctypes.c_int]
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleMesh:
    """Geometry + reference state in the reference's node/slot layout.

    ``g`` is a dict of numpy arrays with the names of the harness dumps
    (meta, cC, cV, Jinv, FO, FN, fN, fI, allFaces, faceIdx0, faceIdx1,
    psi0..2, dpsi0..2, bcU, p_ref, rho_ref) plus scalars P0, R, gamma, gravity.
    """

    def __init__(self, g):
        meta = np.asarray(g["meta"], dtype=np.uint32)
        self.npx, self.npy, self.npz, self.np, self.npf = (int(v) for v in meta[:5])
        self.n_elem, self.n_cells, self.n_int, self.n_all, self.n_face = (
            int(v) for v in meta[5:10])
        pad = self.np

        def f64(name, width=1, padded=False):
            a = np.ascontiguousarray(np.asarray(g[name], dtype=np.float64).reshape(-1))
            if padded:
                a = np.concatenate([a, np.zeros(pad * width)])
            return a

        def u32(name):
            return np.ascontiguousarray(np.asarray(g[name], dtype=np.uint32).reshape(-1))

        self._keep = {
            "cC": f64("cC", 3, True), "cV": f64("cV", 1, True), "Jinv": f64("Jinv", 9, True),
            "FO": u32("FO"), "FN": u32("FN"), "fN": f64("fN"), "fI": f64("fI"),
            "allFaces": u32("allFaces"), "faceIdx0": u32("faceIdx0"),
            "faceIdx1": u32("faceIdx1"), "bcU": u32("bcU"),
            "p_ref": f64("p_ref", 1, True), "rho_ref": f64("rho_ref", 1, True),
        }
        for d in range(3):
            self._keep[f"psi{d}"] = f64(f"psi{d}")
            self._keep[f"dpsi{d}"] = f64(f"dpsi{d}")
        k = self._keep
        s = _Mesh()
        s.npx, s.npy, s.npz, s.np, s.npf = self.npx, self.npy, self.npz, self.np, self.npf
        s.n_elem, s.n_cells, s.n_int, s.n_all, s.n_face = (
            self.n_elem, self.n_cells, self.n_int, self.n_all, self.n_face)
        for name in ("cC", "cV", "Jinv", "FO", "FN", "fN", "fI", "bcU", "p_ref", "rho_ref"):
            setattr(s, name, _ptr(k[name]))
        s.all_faces = _ptr(k["allFaces"])
        s.face_idx0 = _ptr(k["faceIdx0"])
        s.face_idx1 = _ptr(k["faceIdx1"])
        for d in range(3):
            s.psi[d] = _ptr(k[f"psi{d}"]).value
            s.dpsi[d] = _ptr(k[f"dpsi{d}"]).value
        grav = np.asarray(g.get("gravity", (0.0, 0.0, -9.81)), dtype=np.float64)
        s.gravity[0], s.gravity[1], s.gravity[2] = (float(v) for v in grav)
        s.P0 = float(g.get("P0", 1e5))
        cp, cv = float(g.get("cp", 1004.5)), float(g.get("cv", 717.5))
        s.R = float(g.get("R", cp - cv))
        s.gamma = float(g.get("gamma", cp / cv))
        s.T0 = float(g.get("T0", 300.0))
        s.nu = float(g.get("viscosity", 0.0))
        s.Pr = float(g.get("Pr", 0.9))
        # non-conforming faces of a refined mesh (segregated scheme)
        mort = np.asarray(g["mortar"], dtype=np.uint32).reshape(-1) if "mortar" in g else None
        s.n_mortar = 0 if mort is None else len(mort) // 4
        if s.n_mortar:
            self._keep["mortar"] = np.ascontiguousarray(mort)
            s.mortar = _ptr(self._keep["mortar"])
            for d in range(3):
                for h in range(2):
                    for nm, arr in (("psiRef", s.psi_ref), ("psiCor", s.psi_cor)):
                        key = f"{nm}{d}{h}"
                        self._keep[key] = f64(key)
                        arr[d * 2 + h] = _ptr(self._keep[key]).value
        self.cv_heat = cv
        self.struct = s
        self.gh = f64("gh") if "gh" in g else None

    def _vec(self, arrays):
        """Contiguous FP64 copies (where needed) and their pointers; callers
        keep the returned arrays alive until the C call has returned."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in arrays]
        for a in arrs:
            assert a.shape == (self.n_int,)
        ptrs = (ctypes.c_void_p * 5)(*[a.ctypes.data for a in arrs])
        return arrs, ptrs

    def tendency(self, u, return_p=False):
        ua, up = self._vec(u)
        L = [np.empty(self.n_int) for _ in range(5)]
        _, lp = self._vec(L)
        p = np.empty(self.n_all)
        lib().nsem_oracle_tendency(ctypes.byref(self.struct), up, lp, _ptr(p))
        del ua
        return (L, p) if return_p else L

    def ssprk3(self, u, dt, nsteps):
        arrs, up = self._vec([np.array(a, dtype=np.float64, copy=True) for a in u])
        lib().nsem_oracle_ssprk3(ctypes.byref(self.struct), up, float(dt), int(nsteps))
        return arrs

    def jvp(self, u, du):
        """Tendency L(u) and its directional derivative J_L(u) du (dual numbers)."""
        ua, up = self._vec(u)
        da, dp = self._vec(du)
        L = [np.empty(self.n_int) for _ in range(5)]
        Ld = [np.empty(self.n_int) for _ in range(5)]
        _, lp = self._vec(L)
        _, ldp = self._vec(Ld)
        lib().nsem_oracle_jvp(ctypes.byref(self.struct), up, dp, lp, ldp)
        del ua, da
        return L, Ld

    def tlm_ssprk3(self, u, du, dt, nsteps):
        """Tangent-linear SSP-RK3: returns (u_n, du_n) after nsteps."""
        ua, up = self._vec([np.array(a, dtype=np.float64, copy=True) for a in u])
        da, dp = self._vec([np.array(a, dtype=np.float64, copy=True) for a in du])
        lib().nsem_oracle_tlm_ssprk3(ctypes.byref(self.struct), up, dp, float(dt), int(nsteps))
        return ua, da

    def tlm_ssprk3_multi(self, u, dus, dt, nsteps):
        """Tangent-linear SSP-RK3 along len(dus) <= 8 directions in one pass:
        returns (u_n, [du_n per direction])."""
        nd = len(dus)
        ua, up = self._vec([np.array(a, dtype=np.float64, copy=True) for a in u])
        da = [np.array(a, dtype=np.float64, copy=True) for d in dus for a in d]
        for a in da:
            assert a.shape == (self.n_int,)
        dp = (ctypes.c_void_p * (5 * nd))(*[a.ctypes.data for a in da])
        rc = lib().nsem_oracle_tlm_ssprk3_multi(ctypes.byref(self.struct), up, dp, nd,
                                                float(dt), int(nsteps))
        if rc != 0:
            raise ValueError("tlm_ssprk3_multi: 1 <= directions <= 8")
        return ua, [da[5 * d:5 * d + 5] for d in range(nd)]

    def segregated(self, rho, U, T, dt, nsteps):
        """The reference's segregated forward-Euler steps on the primitive
        fields rho, U (n_int x 3), T = theta'; returns the advanced copies."""
        r = np.array(rho, dtype=np.float64, copy=True)
        u = np.ascontiguousarray(np.array(U, dtype=np.float64, copy=True).reshape(-1, 3))
        t = np.array(T, dtype=np.float64, copy=True)
        assert r.shape == (self.n_int,) and u.shape == (self.n_int, 3) and t.shape == (self.n_int,)
        lib().nsem_oracle_segregated(ctypes.byref(self.struct), _ptr(r), _ptr(u), _ptr(t),
                                     float(dt), int(nsteps))
        return r, u, t

    def convection(self, U, T, dt, nsteps):
        """The reference's scalar convection of T in the fixed wind U (n_int x 3)."""
        u = np.ascontiguousarray(np.asarray(U, dtype=np.float64).reshape(-1, 3))
        t = np.array(T, dtype=np.float64, copy=True)
        assert u.shape == (self.n_int, 3) and t.shape == (self.n_int,)
        lib().nsem_oracle_convection(ctypes.byref(self.struct), _ptr(u), _ptr(t), float(dt),
                                     int(nsteps))
        return t

    def convection_wind(self, U_all, scale, order, T, dt, nsteps):
        """The convection app with an analytic wind: spatial part U_all on all
        n_all nodes (n_all x 3) times scale[s] at step s (first two
        components), order 1 (BDF1/AB1) or 2 (AB2)."""
        u = np.ascontiguousarray(np.asarray(U_all, dtype=np.float64).reshape(-1, 3))
        sc = np.ascontiguousarray(np.asarray(scale, dtype=np.float64))
        t = np.array(T, dtype=np.float64, copy=True)
        assert u.shape == (self.n_all, 3) and t.shape == (self.n_int,) and sc.shape == (nsteps,)
        lib().nsem_oracle_convection_wind(ctypes.byref(self.struct), _ptr(u), _ptr(sc), int(order),
                                          _ptr(t), float(dt), int(nsteps))
        return t

    def diagnostics(self, u):
        ua, up = self._vec(u)
        out = np.zeros(3)
        lib().nsem_oracle_diagnostics(ctypes.byref(self.struct), up, _ptr(self.gh),
                                      self.cv_heat, _ptr(out))
        del ua
        return out


def set_pow(which):
    """0: C library pow (as the reference); 1: double-double restatement."""
    lib().nsem_oracle_set_pow(int(which))


def pow_dd(x, y):
    return lib().nsem_oracle_pow_dd(float(x), float(y))


def pow_dd_accurate(x, y):
    """The double-double phase of pow_dd alone (no fast phase)."""
    return lib().nsem_oracle_pow_dd_accurate(float(x), float(y))


def pow_fast_core(x, y):
    """The fast phase's unrounded 2^k (hi + lo) and error bound err (scaled
    by 2^-k like hi), or None outside its domain."""
    hi, lo, err, k = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    if not lib().nsem_oracle_pow_fast_core(float(x), float(y), ctypes.byref(hi), ctypes.byref(lo),
                                           ctypes.byref(err), ctypes.byref(k)):
        return None
    return hi.value, lo.value, err.value, k.value


def pow_fast_sweep(n, seed, xlo, xhi, y):
    """(fallbacks, mismatches) of the fast phase over n log-uniform x."""
    fb, mm = ctypes.c_int64(), ctypes.c_int64()
    lib().nsem_oracle_pow_fast_sweep(int(n), int(seed), float(xlo), float(xhi), float(y),
                                     ctypes.byref(fb), ctypes.byref(mm))
    return fb.value, mm.value


def load_dump(path):
    """Read a harness dump directory (raw .f64/.u32 files) into a dict."""
    out = {}
    for fn in os.listdir(path):
        stem, ext = os.path.splitext(fn)
        if ext == ".f64":
            out[stem] = np.fromfile(os.path.join(path, fn), dtype=np.float64)
        elif ext == ".u32":
            out[stem] = np.fromfile(os.path.join(path, fn), dtype=np.uint32)
    return out


def state(d, tag):
    return [d[f"{tag}_{v}"] for v in VARS]
