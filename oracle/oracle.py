"""ctypes front end of the C restatement of UG's lmgc path (lmgc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the oracle the CUDA path is compared against.
The ug_gb300 product never imports this module.

Also reads the UGFX container written by oracle/ug_export.cc (the UG
reference driven as an oracle) into a dict of numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "liblmgc_oracle.so")

JAC, GS, ILU = 0, 1, 2
SMOOTHERS = {"jac": JAC, "gs": GS, "ilu": ILU}
MAX_S = 8


def read_ugfx(path: str) -> dict:
    """Parse the named-array container written by ug_export."""
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    if data[:6] != b"UGFX1\n":
        raise ValueError(f"{path}: not a UGFX file")
    p = 6
    while p < len(data):
        e = data.index(b"\0", p)
        name = data[p:e].decode()
        t = chr(data[e + 1])
        (n,) = struct.unpack_from("<q", data, e + 2)
        p = e + 10
        if t == "d":
            out[name] = np.frombuffer(data, np.float64, n, p).copy(); p += 8 * n
        elif t == "i":
            out[name] = np.frombuffer(data, np.int32, n, p).copy(); p += 4 * n
        elif t == "s":
            out[name] = data[p:p + n].decode(); p += n
        else:
            raise ValueError(f"bad record type {t!r}")
    return out


def build(quiet: bool = True) -> str:
    """Compile liblmgc_oracle.so (plain C, no dependency on the reference)."""
    cmd = ["make", "-C", HERE, "oracle_lib"]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


class _Level(C.Structure):
    _fields_ = [("n", C.c_int), ("s", C.c_int), ("rowptr", C.c_void_p), ("col", C.c_void_p),
                ("val", C.c_void_p), ("vclass", C.c_void_p), ("vnclass", C.c_void_p),
                ("skip", C.c_void_p), ("prowptr", C.c_void_p), ("pcol", C.c_void_p),
                ("pw", C.c_void_p)]


class _MG(C.Structure):
    _fields_ = [("nlevels", C.c_int), ("lev", C.c_void_p), ("baselevel", C.c_int),
                ("nu1", C.c_int), ("nu2", C.c_int), ("gamma", C.c_int), ("smoother", C.c_int),
                ("damp", C.c_double * MAX_S), ("beta", C.c_double * MAX_S),
                ("cdamp", C.c_double * MAX_S), ("base_abslimit", C.c_double * MAX_S),
                ("imat", C.c_void_p)]


class _Imat(C.Structure):
    _fields_ = [("rowptr", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_matmul_minus.argtypes = [P, P, P]
        L.orc_jac.argtypes = [P, P, P]
        L.orc_lgs.argtypes = [P, P, P]
        L.orc_ilu_decomp.argtypes = [P, P, P]
        L.orc_luiter.argtypes = [P, P, P, P]
        L.orc_nrm2x.argtypes = [P, P, P]
        L.orc_restrict.argtypes = [P, P, P, P, P]
        L.orc_interpolate.argtypes = [P, P, P, P]
        L.orc_interpolate_new.argtypes = [P, P, P, P]
        L.orc_interpolate_new_imat.argtypes = [P, P, P, P, P]
        L.orc_project.argtypes = [P, P, P]
        L.orc_restrict_imat.argtypes = [P, P, P, P, P, P]
        L.orc_interpolate_imat.argtypes = [P, P, P, P, P]
        L.orc_ls_solve.argtypes = [P, P, P, P, P, C.c_int, P, P]
        L.orc_ls_solve_levels.argtypes = [P, P, P, P, P, C.c_int, P, P]
        L.orc_cg_solve_levels.argtypes = [P, P, P, P, P, C.c_int, P, P]
        L.orc_bcgs_solve_levels.argtypes = [P, P, P, P, P, C.c_int, P, P]
        L.orc_cube_create.argtypes = [C.c_int, C.c_ulonglong, C.c_double, C.c_double, C.c_int, C.POINTER(P)]
        L.orc_cube_create.restype = C.c_int
        L.orc_cube_create_rule.argtypes = [C.c_int, C.c_int, C.c_ulonglong, C.c_double, C.c_double, C.c_int,
                                           C.POINTER(P)]
        L.orc_cube_create_rule.restype = C.c_int
        L.orc_cube_level.argtypes = [P, C.c_int, C.POINTER(_Level), C.POINTER(C.POINTER(C.c_double))]
        L.orc_cube_level.restype = C.c_int
        L.orc_cube_rhs.argtypes = [P, C.POINTER(C.c_int)]
        L.orc_cube_rhs.restype = C.POINTER(C.c_double)
        L.orc_cube_destroy.argtypes = [P]
        L.orc_fullrefinelevel.argtypes = [P]
        L.orc_fullrefinelevel.restype = C.c_int
        L.orc_cg_solve.argtypes = [P, P, P, P, P, C.c_int, P, P]
        L.orc_bcgs_solve.argtypes = [P, P, P, P, P, C.c_int, P, P]
        for f in ("orc_jac", "orc_lgs", "orc_ilu_decomp", "orc_luiter", "orc_ls_solve", "orc_cg_solve",
                  "orc_bcgs_solve", "orc_ls_solve_levels", "orc_cg_solve_levels", "orc_bcgs_solve_levels"):
            getattr(L, f).restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def cube_levels(nref: int, seed: int, corr: float = 0.1, var: float = 1.0, threads: int | None = None,
                ug_rules: bool = False):
    """The 3D P1 diffusion workload's hierarchy from the oracle's own
    generator (cube_gen.c): unit cube, six Kuhn tetrahedra refined nref times
    (ug_rules: by UG's red rules with the shortest interior diagonal, UG's
    own mesh; else the Freudenthal triangulation), k = exp(g) per element,
    seeded right-hand side.  Returns (levels, rhs, xyz): level dicts as
    Hierarchy takes them, the finest level's right-hand side and every
    level's node coordinates (n x 3)."""
    L = lib()
    h = C.c_void_p()
    nt = threads if threads else max(1, min(16, os.cpu_count() or 1))
    rc = L.orc_cube_create_rule(int(bool(ug_rules)), nref, seed, corr, var, nt, C.byref(h))
    if rc:
        raise RuntimeError(f"orc_cube_create failed ({rc})")
    try:
        levels, xyzs = [], []
        for l in range(nref + 1):
            lv = _Level()
            xp = C.POINTER(C.c_double)()
            assert L.orc_cube_level(h, l, C.byref(lv), C.byref(xp)) == 0
            n = lv.n
            nnz = np.ctypeslib.as_array(C.cast(lv.rowptr, C.POINTER(C.c_int)), (n + 1,))[-1]

            def arr(ptr, cnt, t):
                return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(t)), (int(cnt),)).copy()

            d = {"n": n, "s": 1, "rowptr": arr(lv.rowptr, n + 1, C.c_int), "col": arr(lv.col, nnz, C.c_int),
                 "val": arr(lv.val, nnz, C.c_double), "vclass": arr(lv.vclass, n, C.c_int),
                 "vnclass": arr(lv.vnclass, n, C.c_int), "skip": arr(lv.skip, n, C.c_int)}
            if l > 0:
                d["prowptr"] = arr(lv.prowptr, n + 1, C.c_int)
                d["pcol"] = arr(lv.pcol, d["prowptr"][-1], C.c_int)
                d["pw"] = arr(lv.pw, d["prowptr"][-1], C.c_double)
            levels.append(d)
            xyzs.append(np.ctypeslib.as_array(xp, (n * 3,)).copy().reshape(n, 3))
        ln = C.c_int()
        rp = L.orc_cube_rhs(h, C.byref(ln))
        rhs = np.ctypeslib.as_array(rp, (ln.value,)).copy()
    finally:
        L.orc_cube_destroy(h)
    return levels, rhs, xyzs


class Hierarchy:
    """Levels of a flattened multigrid hierarchy, as plain numpy arrays.

    ``levels[l]`` is a dict with n, s, rowptr, col, val, vclass, vnclass, skip
    and (l >= 1) prowptr, pcol, pw.  The C structs point into these arrays, so
    the object keeps them alive."""

    def __init__(self, levels: list[dict], imat: list | None = None):
        """imat: per level an interpolation matrix {rowptr, col, val} (UG's
        IMATRIX; None on level 0), used by the transfer's matrix mode."""
        self.imat = None
        if imat is not None:
            self.imat = [None if m is None else {"rowptr": np.ascontiguousarray(m["rowptr"], np.int32),
                                                 "col": np.ascontiguousarray(m["col"], np.int32),
                                                 "val": np.ascontiguousarray(m["val"], np.float64)}
                         for m in imat]
            self._ci = (_Imat * len(self.imat))()
            for i, m in enumerate(self.imat):
                if m is not None:
                    self._ci[i] = _Imat(_p(m["rowptr"]), _p(m["col"]), _p(m["val"]))
        self.levels = []
        for L in levels:
            d = {"n": int(L["n"]), "s": int(L["s"])}
            for k in ("rowptr", "col", "vclass", "vnclass", "skip", "prowptr", "pcol"):
                d[k] = None if L.get(k) is None else np.ascontiguousarray(L[k], np.int32)
            for k in ("val", "pw"):
                d[k] = None if L.get(k) is None else np.ascontiguousarray(L[k], np.float64)
            self.levels.append(d)
        self._c = (_Level * len(self.levels))()
        for i, d in enumerate(self.levels):
            self._c[i] = _Level(d["n"], d["s"], _p(d["rowptr"]), _p(d["col"]), _p(d["val"]),
                                _p(d["vclass"]), _p(d["vnclass"]), _p(d["skip"]), _p(d["prowptr"]),
                                _p(d["pcol"]), _p(d["pw"]))

    @classmethod
    def from_ugfx(cls, fx: dict) -> "Hierarchy":
        s = int(fx["blocksize"][0])
        levels = []
        for l in range(int(fx["nlevels"][0])):
            p = f"L{l}_"
            L = {"n": int(fx[p + "n"][0]), "s": s, "rowptr": fx[p + "rowptr"], "col": fx[p + "col"],
                 "val": fx[p + "val"], "vclass": fx[p + "vclass"], "vnclass": fx[p + "vnclass"],
                 "skip": fx[p + "skip"]}
            if l > 0:
                q = f"P{l}_"
                L.update(prowptr=fx[q + "rowptr"], pcol=fx[q + "col"], pw=fx[q + "w"])
            levels.append(L)
        imat = None
        if int(fx.get("imat", [0])[0]):
            imat = [None] + [{"rowptr": fx[f"M{l}_rowptr"], "col": fx[f"M{l}_col"], "val": fx[f"M{l}_val"]}
                             for l in range(1, len(levels))]
        return cls(levels, imat)

    def lev(self, l):
        return C.byref(self._c[l])

    # ---- kernels
    def matmul_minus(self, l, x, y):
        x = np.array(x, np.float64); y = np.ascontiguousarray(y, np.float64)
        lib().orc_matmul_minus(self.lev(l), _p(x), _p(y)); return x

    def jac(self, l, d):
        v = np.zeros_like(d, dtype=np.float64); d = np.ascontiguousarray(d, np.float64)
        rc = lib().orc_jac(self.lev(l), _p(v), _p(d)); assert rc == 0, rc; return v

    def lgs(self, l, d):
        v = np.zeros_like(d, dtype=np.float64); d = np.ascontiguousarray(d, np.float64)
        rc = lib().orc_lgs(self.lev(l), _p(v), _p(d)); assert rc == 0, rc; return v

    def ilu_decomp(self, l, beta=None):
        L = self.levels[l]
        lu = np.empty_like(L["val"])
        b = None if beta is None else np.ascontiguousarray(np.resize(beta, MAX_S), np.float64)
        rc = lib().orc_ilu_decomp(self.lev(l), _p(lu), _p(b)); assert rc == 0, rc; return lu

    def luiter(self, l, lu, d):
        v = np.zeros_like(d, dtype=np.float64); d = np.ascontiguousarray(d, np.float64)
        lu = np.ascontiguousarray(lu, np.float64)
        rc = lib().orc_luiter(self.lev(l), _p(lu), _p(v), _p(d)); assert rc == 0, rc; return v

    def nrm2x(self, l, x):
        out = np.zeros(MAX_S); x = np.ascontiguousarray(x, np.float64)
        lib().orc_nrm2x(self.lev(l), _p(x), _p(out)); return out[: self.levels[l]["s"]]

    def restrict(self, l, to_coarse, from_fine, damp=None):
        to = np.array(to_coarse, np.float64); fr = np.ascontiguousarray(from_fine, np.float64)
        dm = np.ones(MAX_S) if damp is None else np.resize(np.asarray(damp, np.float64), MAX_S)
        lib().orc_restrict(self.lev(l), self.lev(l - 1), _p(to), _p(fr), _p(dm)); return to

    def interpolate(self, l, from_coarse, damp=None):
        L = self.levels[l]
        to = np.zeros(L["n"] * L["s"]); fr = np.ascontiguousarray(from_coarse, np.float64)
        dm = np.ones(MAX_S) if damp is None else np.resize(np.asarray(damp, np.float64), MAX_S)
        lib().orc_interpolate(self.lev(l), _p(to), _p(fr), _p(dm)); return to

    def restrict_imat(self, l, to_coarse, from_fine, damp=None):
        """RestrictByMatrix with level l's interpolation matrix."""
        to = np.array(to_coarse, np.float64); fr = np.ascontiguousarray(from_fine, np.float64)
        dm = np.ones(MAX_S) if damp is None else np.resize(np.asarray(damp, np.float64), MAX_S)
        lib().orc_restrict_imat(self.lev(l), C.byref(self._ci[l]), self.lev(l - 1), _p(to), _p(fr), _p(dm))
        return to

    def interpolate_imat(self, l, from_coarse, damp=None):
        """InterpolateCorrectionByMatrix with level l's interpolation matrix."""
        L = self.levels[l]
        to = np.zeros(L["n"] * L["s"]); fr = np.ascontiguousarray(from_coarse, np.float64)
        dm = np.ones(MAX_S) if damp is None else np.resize(np.asarray(damp, np.float64), MAX_S)
        lib().orc_interpolate_imat(self.lev(l), C.byref(self._ci[l]), _p(to), _p(fr), _p(dm))
        return to

    def interpolate_new(self, l, vnew, x_fine, x_coarse):
        """StandardIntNewNodeVector: fine vectors with VNEW take P x_coarse;
        with interpolation matrices (the transfer's `$M` mode)
        InterpolateNewVectorsByMatrix instead."""
        xf = np.array(x_fine, np.float64); xc = np.ascontiguousarray(x_coarse, np.float64)
        vn = np.ascontiguousarray(vnew, np.int32)
        if self.imat is not None:
            lib().orc_interpolate_new_imat(self.lev(l), C.byref(self._ci[l]), _p(vn), _p(xf), _p(xc))
        else:
            lib().orc_interpolate_new(self.lev(l), _p(vn), _p(xf), _p(xc))
        return xf

    def project(self, l, x_coarse, x_fine):
        """StandardProject: coarse vectors with a son node take its values."""
        xc = np.array(x_coarse, np.float64); xf = np.ascontiguousarray(x_fine, np.float64)
        lib().orc_project(self.lev(l), _p(xc), _p(xf)); return xc

    def interpolate_new_vectors(self, fl, tl, x_all, vnew):
        """InterpolateNewVectors (transfer.cc:775): levels fl+1..tl in turn,
        on an every-level vector (levels concatenated)."""
        x = np.array(x_all, np.float64)
        offs = np.cumsum([0] + self.level_lengths())
        for l in range(fl + 1, tl + 1):
            x[offs[l]:offs[l + 1]] = self.interpolate_new(l, vnew[l], x[offs[l]:offs[l + 1]], x[offs[l - 1]:offs[l]])
        return x

    def project_solution(self, fl, tl, x_all):
        """ProjectSolution (transfer.cc:794): levels tl-1 down to fl."""
        x = np.array(x_all, np.float64)
        offs = np.cumsum([0] + self.level_lengths())
        for l in range(tl - 1, fl - 1, -1):
            x[offs[l]:offs[l + 1]] = self.project(l + 1, x[offs[l]:offs[l + 1]], x[offs[l + 1]:offs[l + 2]])
        return x

    # ---- solver
    def bcgs_solve(self, rhs, **kw):
        """bcgs (ls.cc:1711-2062) preconditioned by lmgc, configured as ls_solve;
        iterations count half steps, as UG's.  Returns (x, iterations, converged,
        history)."""
        return self.ls_solve(rhs, _solver="bcgs", **kw)

    def cg_solve(self, rhs, **kw):
        """cg (ls.cc:901-1064) preconditioned by lmgc, configured as ls_solve.
        Returns (x, iterations, converged, history)."""
        return self.ls_solve(rhs, _solver="cg", **kw)

    def level_lengths(self):
        return [L["n"] * L["s"] for L in self.levels]

    def fullrefinelevel(self):
        """FULLREFINELEVEL (gm/algebra.cc:2838): the lowest level with a
        FINE_GRID_DOF vector; the top level on a uniformly refined hierarchy."""
        mg = self._mg()
        return lib().orc_fullrefinelevel(C.byref(mg))

    def cg_solve_surface(self, rhs_all, **kw):
        """cg preconditioned by lmgc on every level (see ls_solve_surface)."""
        return self.ls_solve_surface(rhs_all, _solver="cg", **kw)

    def bcgs_solve_surface(self, rhs_all, **kw):
        """bcgs preconditioned by lmgc on every level; iterations count half steps."""
        return self.ls_solve_surface(rhs_all, _solver="bcgs", **kw)

    def ls_solve_surface(self, rhs_all, *, x0_all=None, red=1e-10, abslimit=1e-50, maxit=100, _solver="ls", **kw):
        """ls + lmgc on a locally refined hierarchy: rhs_all and the returned x
        hold every level 0..top, concatenated.  The defect and its norms run over
        UG's surface and the correction is added on every level baselevel..top.
        Returns (x_all, iterations, converged, history)."""
        lens = self.level_lengths()
        offs = np.concatenate([[0], np.cumsum(lens)])
        b = np.array(rhs_all, np.float64)
        x = np.zeros(offs[-1]) if x0_all is None else np.array(x0_all, np.float64)
        assert b.size == offs[-1] and x.size == offs[-1], "arrays must hold every level"
        bp = (C.c_void_p * len(lens))(*[b.ctypes.data + 8 * int(o) for o in offs[:-1]])
        xp = (C.c_void_p * len(lens))(*[x.ctypes.data + 8 * int(o) for o in offs[:-1]])
        mg = self._mg(**kw)
        s = self.levels[-1]["s"]
        redv = np.resize(np.asarray(red, np.float64), MAX_S)
        absv = np.resize(np.asarray(abslimit, np.float64), MAX_S)
        hist = np.zeros((2 * maxit + 1) * s)
        conv = C.c_int(0)
        f = {"cg": lib().orc_cg_solve_levels, "bcgs": lib().orc_bcgs_solve_levels}.get(_solver,
                                                                                        lib().orc_ls_solve_levels)
        it = f(C.byref(mg), xp, bp, _p(redv), _p(absv), maxit, _p(hist), C.byref(conv))
        if it < 0:
            raise RuntimeError(f"oracle {_solver} failed: {it}")
        return x, it, bool(conv.value), hist[: (it + 1) * s].reshape(it + 1, s)

    def _mg(self, *, smoother="jac", baselevel=0, nu1=2, nu2=2, gamma=1, damp=None, beta=None, cdamp=None,
            base_abslimit=1e-10, matrix_transfer=False):
        mg = _MG()
        if matrix_transfer:
            assert self.imat is not None, "no interpolation matrices"
            mg.imat = C.addressof(self._ci)
        mg.nlevels = len(self.levels); mg.lev = C.addressof(self._c)
        mg.baselevel, mg.nu1, mg.nu2, mg.gamma = baselevel, nu1, nu2, gamma
        mg.smoother = SMOOTHERS[smoother] if isinstance(smoother, str) else smoother
        for i in range(MAX_S):
            mg.damp[i] = 1.0 if damp is None else float(np.resize(damp, MAX_S)[i])
            mg.beta[i] = 0.0 if beta is None else float(np.resize(beta, MAX_S)[i])
            mg.cdamp[i] = 1.0 if cdamp is None else float(np.resize(cdamp, MAX_S)[i])
            mg.base_abslimit[i] = float(np.resize(base_abslimit, MAX_S)[i])
        return mg

    def ls_solve(self, rhs, *, smoother="jac", baselevel=0, nu1=2, nu2=2, gamma=1, damp=None,
                 beta=None, cdamp=None, red=1e-10, abslimit=1e-50, maxit=100, x0=None,
                 base_abslimit=1e-10, _solver="ls", matrix_transfer=False):
        """ls + lmgc as configured by `npinit lmgc $n1 $n2 $g $b` and `npinit ls
        $red $abslimit $m` (matrix_transfer: `npinit transfer $M`).  Returns
        (x, iterations, converged, history)."""
        top = len(self.levels) - 1
        s = self.levels[top]["s"]
        mg = _MG()
        if matrix_transfer:
            assert self.imat is not None, "no interpolation matrices"
            mg.imat = C.addressof(self._ci)
        mg.nlevels = len(self.levels); mg.lev = C.addressof(self._c)
        mg.baselevel, mg.nu1, mg.nu2, mg.gamma = baselevel, nu1, nu2, gamma
        mg.smoother = SMOOTHERS[smoother] if isinstance(smoother, str) else smoother
        for i in range(MAX_S):
            mg.damp[i] = 1.0 if damp is None else float(np.resize(damp, MAX_S)[i])
            mg.beta[i] = 0.0 if beta is None else float(np.resize(beta, MAX_S)[i])
            mg.cdamp[i] = 1.0 if cdamp is None else float(np.resize(cdamp, MAX_S)[i])
            mg.base_abslimit[i] = float(np.resize(base_abslimit, MAX_S)[i])
        x = np.zeros(self.levels[top]["n"] * s) if x0 is None else np.array(x0, np.float64)
        b = np.array(rhs, np.float64)
        redv = np.resize(np.asarray(red, np.float64), MAX_S)
        absv = np.resize(np.asarray(abslimit, np.float64), MAX_S)
        hist = np.zeros((2 * maxit + 1) * s)
        conv = C.c_int(0)
        f = {"cg": lib().orc_cg_solve, "bcgs": lib().orc_bcgs_solve}.get(_solver, lib().orc_ls_solve)
        it = f(C.byref(mg), _p(x), _p(b), _p(redv), _p(absv), maxit, _p(hist), C.byref(conv))
        if it < 0:
            raise RuntimeError(f"oracle {_solver} failed: {it}")
        return x, it, bool(conv.value), hist[: (it + 1) * s].reshape(it + 1, s)
