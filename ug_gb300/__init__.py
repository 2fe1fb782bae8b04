"""ug_gb300: UG's linear multigrid hot path (lmgc with jac / gs / ilu, the
standard transfer, ex and ls) as hand-written CUDA for GB300 (sm_103a).

This module is the host-side mirror of UG's numproc interface over the C ABI
in include/ug_gb300.h (libug_gb300.so, built in tree by ug_gb300/build.py):
a ``MultiGrid`` holds the device-resident hierarchy, its vectors ("createvector")
and numproc objects ("npcreate" / "npinit" / "npexecute"), with the same
class roles, argument syntax and error behaviour as UG 3.12.1:

    mg = MultiGrid(levels)                   # flattened hierarchy (grid change)
    mg.createvector("sol", "rhs")
    mg.npcreate("transfer", "transfer.gtransfer"); mg.npinit("transfer", transfer)
    mg.npcreate("smooth", "iter.gjac");     mg.npinit("smooth", "$damp 0.8")
    ...
    mg.npexecute("mgs", "$i $d $r $s $p")

There is no CPU fallback: without the library or a CUDA device every call
that needs the GPU raises GmgError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

__all__ = ["GmgError", "Generator", "MultiGrid", "LResult", "lib", "LIB_PATH",
           "ORDER_LIST", "ORDER_COLOR", "ORDER_DOMAIN", "FP64", "FP32"]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libug_gb300.so")
MAX_S = 8
ORDER_LIST, ORDER_COLOR, ORDER_DOMAIN = 0, 1, 2
FP64, FP32 = 0, 1
NP_NOT_INIT, NP_NOT_ACTIVE, NP_ACTIVE, NP_EXECUTABLE = 0, 1, 2, 3


class GmgError(RuntimeError):
    pass


class LevelDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("s", C.c_int), ("rowptr", C.c_void_p), ("col", C.c_void_p),
                ("val", C.c_void_p), ("vclass", C.c_void_p), ("vnclass", C.c_void_p), ("skip", C.c_void_p),
                ("prowptr", C.c_void_p), ("pcol", C.c_void_p), ("pw", C.c_void_p)]


class MgOpts(C.Structure):
    _fields_ = [("order", C.c_int), ("fp32_copy", C.c_int), ("autotune", C.c_int), ("device", C.c_int),
                ("disable_pdl", C.c_int)]


class LResult(C.Structure):
    """LRESULT (np/procs/ls.h:71-77)."""
    _fields_ = [("error_code", C.c_int), ("converged", C.c_int), ("first_defect", C.c_double * MAX_S),
                ("last_defect", C.c_double * MAX_S), ("number_of_linear_iterations", C.c_int)]

    @property
    def iters(self):
        return self.number_of_linear_iterations


_lib = None


def lib(build_if_missing: bool = True):
    """Load libug_gb300.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise GmgError(f"{LIB_PATH} is missing: run python -m ug_gb300.build")
        from . import build as _b
        _b.build()
    L = C.CDLL(LIB_PATH)
    P, I, D, LL = C.c_void_p, C.c_int, C.c_double, C.c_longlong
    sig = {
        "gmg_last_error": ([], C.c_char_p),
        "gmg_mg_create": ([P, I, P, P], I), "gmg_mg_destroy": ([P], I), "gmg_mg_set_stream": ([P, P], I),
        "gmg_mg_nlevels": ([P], I), "gmg_mg_level_size": ([P, I, P, P, P], I), "gmg_mg_get_order": ([P, I, P], I),
        "gmg_mg_get_matrix": ([P, I, P, P, P], I), "gmg_mg_num_waves": ([P, I], I),
        "gmg_mg_device_bytes": ([P], LL), "gmg_mg_launch_count": ([P, I], LL), "gmg_mg_sync": ([P], I),
        "gmg_vec_create": ([P, C.c_char_p, I, P], I), "gmg_vec_by_name": ([P, C.c_char_p], P),
        "gmg_mat_by_name": ([P, C.c_char_p], P), "gmg_vec_upload": ([P, I, P], I),
        "gmg_vec_download": ([P, I, P], I), "gmg_vec_device_ptr": ([P, I, P], I),
        "gmg_np_create": ([P, C.c_char_p, C.c_char_p], I), "gmg_np_init": ([P, C.c_char_p, C.c_char_p, P], I),
        "gmg_np_execute": ([P, C.c_char_p, C.c_char_p], I), "gmg_np_by_name": ([P, C.c_char_p], P),
        "gmg_np_display": ([P, C.c_char_p, I], I),
        "gmg_iter_preprocess": ([P, I, P, P, P, P, P], I), "gmg_iter_iter": ([P, I, P, P, P, P], I),
        "gmg_iter_postprocess": ([P, I, P, P, P, P], I), "gmg_iter_smooth": ([P, I, P, P, P, P, I, P], I),
        "gmg_transfer_preprocess": ([P, P, I, P, P, P, P], I),
        "gmg_transfer_restrict_defect": ([P, I, P, P, P, P, P], I),
        "gmg_transfer_interpolate_correction": ([P, I, P, P, P, P, P], I),
        "gmg_transfer_postprocess": ([P, P, I, P, P, P, P], I),
        "gmg_transfer_interpolate_new_vectors": ([P, I, I, P, P], I),
        "gmg_transfer_project_solution": ([P, I, I, P, P], I),
        "gmg_transfer_adapt_correction": ([P, I, P, P, P, P], I), "gmg_mg_set_new_vectors": ([P, I, P], I),
        "gmg_mg_update_values": ([P, I, P], I), "gmg_mg_level_variant": ([P, I, P, P, P], I),
    "gmg_mg_level_cta_chain": ([P, I, P], I), "gmg_mg_set_level_cta_chain": ([P, I, I], I),
    "gmg_mg_domain_info": ([P, I, P, P, P], I), "gmg_colour_graph": ([I, P, P, P, P], I),
    "gmg_mg_set_iface_sweep": ([P, I], I), "gmg_mg_set_direct_host": ([P, I], I),
        "gmg_ls_preprocess": ([P, I, P, P, P, P, P], I), "gmg_ls_defect": ([P, I, P, P, P, P], I),
        "gmg_ls_residuum": ([P, I, I, P, P, P, P], I), "gmg_ls_solver": ([P, I, P, P, P, P, P, P], I),
        "gmg_ls_postprocess": ([P, I, P, P, P, P], I),
        "gmg_dset": ([P, I, P, D], I), "gmg_dcopy": ([P, I, P, P], I), "gmg_dadd": ([P, I, P, P], I),
        "gmg_dmatmul_minus": ([P, I, P, P, P], I), "gmg_dnrm2x": ([P, I, P, P], I),
        "gmg_dmatmul": ([P, I, P, P, P], I), "gmg_dmatmul_add": ([P, I, P, P, P], I),
        "gmg_dscalx": ([P, I, P, P], I), "gmg_daxpy": ([P, I, P, P, P], I), "gmg_ddot": ([P, I, P, P, P], I),
        "gmg_l_jac": ([P, I, P, P, P], I), "gmg_l_lgs": ([P, I, P, P, P], I),
        "gmg_l_ilu_decomp": ([P, I, P, P], I), "gmg_l_luiter": ([P, I, P, P, P], I),
        "gmg_l_ilu_factors": ([P, I, P], I), "gmg_mg_set_imatrix": ([P, I, P, P, P], I),
        "gmg_restrict_by_matrix": ([P, I, P, P, P], I), "gmg_interpolate_correction_by_matrix": ([P, I, P, P, P], I),
        "gmg_standard_restrict": ([P, I, P, P, P], I), "gmg_standard_interpolate_correction": ([P, I, P, P, P], I),
        "gmg_solve_host": ([P, C.c_char_p, P, P, P], I),
        "gmg_mg_create_batched": ([P, P, I, P, P], I), "gmg_mg_num_instances": ([P], I),
        "gmg_mg_instance_info": ([P, I, P, P, P], I), "gmg_vec_upload_packed": ([P, P], I),
        "gmg_vec_download_packed": ([P, P], I), "gmg_ls_instance_result": ([P, I, P], I),
        "gmg_pool_create": ([I, I, C.c_char_p, D, I, I, P], I), "gmg_pool_destroy": ([P], I),
        "gmg_pool_multigrid": ([P], P), "gmg_pool_set_stream": ([P, P], I), "gmg_pool_slots": ([P, P, P, P], I),
        "gmg_pool_admit": ([P, I, C.c_ulonglong, D, D], I), "gmg_pool_launch": ([P], I),
        "gmg_pool_poll": ([P, P, P], I), "gmg_pool_fetch": ([P, I, P, P], I),
        "gmg_pool_slot_matrix": ([P, I, I, P], I), "gmg_pool_set_field_precision": ([P, I], I),
        "gmg_pool_create_mixed": ([P, I, C.c_char_p, D, I, I, P], I), "gmg_pool_slot_info": ([P, I, P, P], I),
        "gmg_pool_create_mesh": ([I, P, I, C.c_char_p, D, I, I, P], I),
        "gmg_mg_full_refine_level": ([P], I), "gmg_vec_upload_levels": ([P, P], I),
        "gmg_vec_download_levels": ([P, P], I),
        "gmg_lgen_create": ([I, I, C.c_ulonglong, P], I), "gmg_lgen_levels": ([P, P, P], I),
        "gmg_lgen_rhs": ([P, P, P], I), "gmg_lgen_coords": ([P, I, P], I), "gmg_lgen_destroy": ([P], I),
        "gmg_gen_create": ([I, I, C.c_ulonglong, D, D, P], I), "gmg_gen_levels": ([P, P, P], I),
        "gmg_gen_rhs": ([P, P, P], I), "gmg_gen_coords": ([P, I, P], I), "gmg_gen_destroy": ([P], I),
        "gmg_mg_replace_levels": ([P, I, P, I], I),
        "gmg_order_bw": ([P, P, P], I), "gmg_order_lex": ([P, I, P, I, C.c_char_p, D, P], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _err(what: str):
    msg = lib().gmg_last_error()
    raise GmgError(f"{what}: {msg.decode() if msg else 'failed'}")


def _ptr(a):
    return None if a is None else a.ctypes.data


def _sc(v, default=1.0):
    a = np.full(MAX_S, default, np.float64)
    if v is not None:
        v = np.atleast_1d(np.asarray(v, np.float64))
        a[:] = np.resize(v, MAX_S)
    return a


def colour_graph(rowptr, col):
    """The multicolour order's colouring of a CSR pattern (gmg_colour_graph):
    DSATUR, then tabu search for fewer colours.  Returns (colour, ncolours)."""
    rp = np.ascontiguousarray(rowptr, np.int32)
    cl = np.ascontiguousarray(col, np.int32)
    n = len(rp) - 1
    colour = np.empty(max(n, 1), np.int32)
    nc = C.c_int()
    if lib().gmg_colour_graph(n, _ptr(rp), _ptr(cl), _ptr(colour), C.byref(nc)):
        _err("gmg_colour_graph")
    return colour[:n], nc.value


class Generator:
    """Structured hierarchy of a workload, built on the host (no GPU needed).

    kind 0: 2D Q1 Poisson on the unit square (one quad refined nref times);
    kind 1: 3D P1 diffusion on the unit cube (six Kuhn tets refined nref
    times), k = exp(g) with correlation ``corr`` and variance ``var``;
    kind 2: 2D P1 plane-strain elasticity, 2x2 blocks;
    kind 3: kind 1's problem on the tetrahedra UG's red rules produce (the
    octahedron cut along its shortest interior diagonal, UG's tie-break;
    kind 1 keeps the Freudenthal triangulation instead)."""

    POISSON2D, DIFFUSION3D, ELASTICITY2D, DIFFUSION3D_UG = 0, 1, 2, 3

    def __init__(self, kind: int, nref: int, seed: int = 1, corr: float = 0.1, var: float = 0.0):
        L = lib()
        h = C.c_void_p()
        if L.gmg_gen_create(kind, nref, seed, corr, var, C.byref(h)):
            _err("gmg_gen_create")
        self._h = h
        self.kind, self.nref = kind, nref
        lev = C.POINTER(LevelDesc)()
        nl = C.c_int()
        L.gmg_gen_levels(h, C.byref(lev), C.byref(nl))
        self._desc = lev
        self.nlevels = nl.value
        rp = C.POINTER(C.c_double)()
        ln = C.c_int()
        L.gmg_gen_rhs(h, C.byref(rp), C.byref(ln))
        self.rhs = np.ctypeslib.as_array(rp, (ln.value,)).copy()

    def level(self, l: int) -> dict:
        """Numpy copies of one level's arrays (UG list order)."""
        d = self._desc[l]
        n, s = d.n, d.s

        def arr(p, cnt, ct):
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), (cnt,)).copy() if p and cnt else None

        rowptr = arr(d.rowptr, n + 1, C.c_int)
        nnz = int(rowptr[-1])
        out = {"n": n, "s": s, "rowptr": rowptr, "col": arr(d.col, nnz, C.c_int),
               "val": arr(d.val, nnz * s * s, C.c_double), "vclass": arr(d.vclass, n, C.c_int),
               "vnclass": arr(d.vnclass, n, C.c_int), "skip": arr(d.skip, n, C.c_int)}
        if l > 0:
            prow = arr(d.prowptr, n + 1, C.c_int)
            out.update(prowptr=prow, pcol=arr(d.pcol, int(prow[-1]), C.c_int), pw=arr(d.pw, int(prow[-1]), C.c_double))
        out["xyz"] = np.ctypeslib.as_array(self._coords(l), (n * 3,)).copy().reshape(n, 3)
        return out

    def levels(self):
        return [self.level(l) for l in range(self.nlevels)]

    def _coords(self, l):
        xp = C.POINTER(C.c_double)()
        lib().gmg_gen_coords(self._h, l, C.byref(xp))
        return xp

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.gmg_gen_destroy(self._h)
            self._h = None


class LocalGenerator(Generator):
    """Locally refined hierarchy (gmg_lgen_create): plane-strain P1 elasticity
    on the L-shaped domain, ``nuni`` uniform refinements of the six coarse
    triangles, then ``nloc`` steps toward the re-entrant corner (step k
    refines the leaf elements with a corner within 0.5^k), closed and
    classified by UG's rules.  ``rhs`` holds every level, concatenated."""

    def __init__(self, nuni: int, nloc: int, seed: int = 1):
        L = lib()
        h = C.c_void_p()
        if L.gmg_lgen_create(nuni, nloc, seed, C.byref(h)):
            _err("gmg_lgen_create")
        self._h = h
        self.kind, self.nuni, self.nloc = "lshape", nuni, nloc
        lev = C.POINTER(LevelDesc)()
        nl = C.c_int()
        L.gmg_lgen_levels(h, C.byref(lev), C.byref(nl))
        self._desc = lev
        self.nlevels = nl.value
        self.nref = self.nlevels - 1
        rp = C.POINTER(C.c_double)()
        ln = C.c_longlong()
        L.gmg_lgen_rhs(h, C.byref(rp), C.byref(ln))
        self.rhs = np.ctypeslib.as_array(rp, (ln.value,)).copy()

    def _coords(self, l):
        xp = C.POINTER(C.c_double)()
        lib().gmg_lgen_coords(self._h, l, C.byref(xp))
        return xp

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.gmg_lgen_destroy(self._h)
            self._h = None


def levels_from_ugfx(fx: dict) -> list[dict]:
    """Level dicts from an exported UG hierarchy (golden fixture)."""
    s = int(np.asarray(fx["blocksize"]).ravel()[0])
    out = []
    for l in range(int(np.asarray(fx["nlevels"]).ravel()[0])):
        p = f"L{l}_"
        d = {"n": int(np.asarray(fx[p + "n"]).ravel()[0]), "s": s, "rowptr": fx[p + "rowptr"], "col": fx[p + "col"],
             "val": fx[p + "val"], "vclass": fx[p + "vclass"], "vnclass": fx[p + "vnclass"], "skip": fx[p + "skip"]}
        if l > 0:
            q = f"P{l}_"
            d.update(prowptr=fx[q + "rowptr"], pcol=fx[q + "col"], pw=fx[q + "w"])
        out.append(d)
    return out


def _desc_array(levels, keep: list):
    """gmg_level_desc array of a Generator or a list of level dicts; the numpy
    arrays it points into are appended to ``keep``."""
    if isinstance(levels, Generator):
        keep.append(levels)
        return levels._desc, levels.nlevels
    nl = len(levels)
    desc_arr = (LevelDesc * nl)()
    for i, d in enumerate(levels):
        ints = {k: (None if d.get(k) is None else np.ascontiguousarray(d[k], np.int32))
                for k in ("rowptr", "col", "vclass", "vnclass", "skip", "prowptr", "pcol")}
        dbl = {k: (None if d.get(k) is None else np.ascontiguousarray(d[k], np.float64)) for k in ("val", "pw")}
        keep += list(ints.values()) + list(dbl.values())
        desc_arr[i] = LevelDesc(int(d["n"]), int(d["s"]), _ptr(ints["rowptr"]), _ptr(ints["col"]),
                                _ptr(dbl["val"]), _ptr(ints["vclass"]), _ptr(ints["vnclass"]),
                                _ptr(ints["skip"]), _ptr(ints["prowptr"]), _ptr(ints["pcol"]),
                                _ptr(dbl["pw"]))
    keep.append(desc_arr)
    return desc_arr, nl


def order_bw(level: dict) -> tuple[np.ndarray, int]:
    """UG's order.bw (np/procs/order.cc:343) on one level: (perm, bandwidth),
    perm[i] = the current index of the vector placed at i (gmg_order_bw)."""
    keep = []
    desc, _ = _desc_array([level], keep)
    perm = np.empty(int(level["n"]), np.int32)
    bw = C.c_int(0)
    if lib().gmg_order_bw(C.byref(desc[0]), _ptr(perm), C.byref(bw)):
        _err("order bw")
    return perm, bw.value


def order_lex(level: dict, xyz, config: str, inv_mesh_size: float, dim: int | None = None) -> np.ndarray:
    """UG's order.lex $config <config> (order.cc:287, LexOrderVectorsInGrid
    gm/algebra.cc:4699) on one level; xyz one row of coordinates per vector
    (gmg_order_lex)."""
    keep = []
    desc, _ = _desc_array([level], keep)
    xyz = np.ascontiguousarray(np.asarray(xyz, np.float64).reshape(int(level["n"]), -1))
    dim = len(config) if dim is None else dim
    perm = np.empty(int(level["n"]), np.int32)
    if lib().gmg_order_lex(C.byref(desc[0]), dim, _ptr(xyz), xyz.shape[1], config.encode(), float(inv_mesh_size),
                           _ptr(perm)):
        _err(f"order lex {config}")
    return perm


def lex_inv_mesh_size(level: int, n_level0: int, dim: int, radius: float) -> float:
    """UG's scaling of position differences in LexOrderVectorsInGrid
    (gm/algebra.cc:4721): 2^level * NN(level 0)^(1/dim) / radius."""
    return float(2 ** level) * float(n_level0) ** (1.0 / dim) / radius


def order_levels(levels: list[dict], order: str, xyz=None, radius: float | None = None):
    """UG's `npexecute <order numproc> $a` on a flattened hierarchy: every
    level renumbered by order.bw (``order="bw"``) or order.lex
    (``order="lex:<config>"``, positions ``xyz[l]`` per level; the domain
    radius defaults to half the largest extent of level 0).  Returns
    (levels in the new order, the permutation of every level)."""
    if order == "bw":
        perms = [order_bw(d)[0] for d in levels]
    elif order.startswith("lex:"):
        config = order[4:]
        dim = len(config)
        if xyz is None:
            raise GmgError("order lex needs the vector positions of every level")
        pos = [np.asarray(x, np.float64).reshape(int(d["n"]), -1)[:, :dim] for x, d in zip(xyz, levels)]
        if radius is None:
            radius = 0.5 * float(np.max(pos[0].max(axis=0) - pos[0].min(axis=0)))
        perms = [order_lex(d, pos[l], config, lex_inv_mesh_size(l, int(levels[0]["n"]), dim, radius))
                 for l, d in enumerate(levels)]
    else:
        raise GmgError(f"unknown order {order!r} (bw or lex:<config>)")
    return permute_levels(levels, perms), perms


def permute_vector(v, perm, s: int = 1) -> np.ndarray:
    """A level vector (s components per row) in the order perm."""
    return np.asarray(v).reshape(-1, s)[np.asarray(perm)].ravel()


def permute_levels(levels: list[dict], perms: list) -> list[dict]:
    """Level dicts renumbered by one permutation per level (None = keep):
    rows and columns of A, the per-row classes, P's rows on the level and P's
    columns on the next finer level.  Each row keeps its entries in stored
    order (UG's order numprocs leave the matrix lists alone)."""
    inv = []
    for d, p in zip(levels, perms):
        if p is None:
            inv.append(None)
            continue
        p = np.asarray(p, np.int64)
        q = np.empty_like(p)
        q[p] = np.arange(p.size)
        inv.append(q)

    def rows(rowptr, col, vals, p, cmap, width):
        rowptr = np.asarray(rowptr, np.int64)
        col = np.asarray(col)
        lens = np.diff(rowptr)
        if p is not None:
            lens = lens[p]
        newptr = np.zeros(lens.size + 1, np.int64)
        np.cumsum(lens, out=newptr[1:])
        if p is None:
            idx = np.arange(col.size)
        else:
            starts = rowptr[:-1][p]
            idx = np.repeat(starts - newptr[:-1], lens) + np.arange(int(newptr[-1]))
        newcol = col[idx]
        if cmap is not None:
            newcol = cmap[newcol]
        newval = np.asarray(vals).reshape(col.size, width)[idx].ravel()
        return newptr.astype(np.int32), newcol.astype(np.int32), newval

    out = []
    for l, d in enumerate(levels):
        p, q = perms[l], inv[l]
        s = int(d["s"])
        e = dict(d)
        e["rowptr"], e["col"], e["val"] = rows(d["rowptr"], d["col"], d["val"], p, q, s * s)
        for k in ("vclass", "vnclass", "skip"):
            if d.get(k) is not None and p is not None:
                e[k] = np.asarray(d[k])[np.asarray(p)]
        if d.get("prowptr") is not None:
            e["prowptr"], e["pcol"], e["pw"] = rows(d["prowptr"], d["pcol"], d["pw"], p, inv[l - 1], 1)
        out.append(e)
    return out


class MultiGrid:
    """Device-resident multigrid hierarchy with UG-style user data and numprocs.

    ``levels`` is a Generator or a list of level dicts; a list of several
    such hierarchies (``batched=True``) builds one batched hierarchy of
    independent instances (gmg_mg_create_batched), whose vectors move as
    packed arrays (``upload_packed`` / ``download_packed`` / ``split``)."""

    def __init__(self, levels, order: int = ORDER_LIST, fp32: bool = False, autotune: bool = False, device: int = 0,
                 pdl: bool = True, batched: bool = False):
        L = lib()
        opts = MgOpts(order, int(fp32), int(autotune), device, int(not pdl))
        h = C.c_void_p()
        keep: list = []
        if batched:
            descs = [_desc_array(inst, keep) for inst in levels]
            ninst = len(descs)
            ptrs = (C.c_void_p * ninst)(*[C.cast(d, C.c_void_p).value for d, _ in descs])
            nls = np.array([n for _, n in descs], np.int32)
            if L.gmg_mg_create_batched(C.cast(ptrs, C.c_void_p), _ptr(nls), ninst, C.byref(opts), C.byref(h)):
                _err("gmg_mg_create_batched")
            nl = int(nls.max())
        else:
            desc_arr, nl = _desc_array(levels, keep)
            if L.gmg_mg_create(C.cast(desc_arr, C.c_void_p), nl, C.byref(opts), C.byref(h)):
                _err("gmg_mg_create")
        self._h = h
        self.nlevels = nl
        self.top = nl - 1
        self.ninst = L.gmg_mg_num_instances(h)
        if self.ninst:
            top, nt, po = C.c_int(), C.c_int(), C.c_longlong()
            self.inst_top, self.inst_n, self.pack_off = [], [], []
            for k in range(self.ninst):
                L.gmg_mg_instance_info(h, k, C.byref(top), C.byref(nt), C.byref(po))
                self.inst_top.append(top.value)
                self.inst_n.append(nt.value)
                self.pack_off.append(po.value)
            self.block = self.size(0)[1]
            self.packed_len = (self.pack_off[-1] + self.inst_n[-1]) * self.block
        self._refresh_levels()
        del keep  # the device holds its own copies

    def _refresh_levels(self):
        # locally refined: the surface spans levels frl..top, host vectors hold every level
        self.nlevels = lib().gmg_mg_nlevels(self._h)
        self.top = self.nlevels - 1
        self.frl = lib().gmg_mg_full_refine_level(self._h)
        self.local = self.frl < self.top
        self.level_len = [self.size(l)[0] * self.size(l)[1] for l in range(self.nlevels)]

    def replace_levels(self, from_level: int, levels) -> None:
        """gmg_mg_replace_levels: levels from_level.. replaced by ``levels``
        (level dicts, the new levels from_level, from_level+1, ...) after an
        adaptation changed them; the levels below are kept as they are."""
        keep: list = []
        desc_arr, n = _desc_array(list(levels), keep)
        if lib().gmg_mg_replace_levels(self._h, int(from_level), C.cast(desc_arr, C.c_void_p), n):
            _err("gmg_mg_replace_levels")
        self._refresh_levels()

    # ---- locally refined hierarchies
    def split_levels(self, flat) -> list:
        """Per-level views of an every-level vector (levels concatenated)."""
        offs = np.concatenate([[0], np.cumsum(self.level_len)])
        return [flat[offs[l]:offs[l + 1]] for l in range(self.nlevels)]

    def upload_levels(self, name: str, data):
        a = np.ascontiguousarray(data, np.float64).ravel()
        if a.size != sum(self.level_len):
            raise GmgError(f"upload_levels {name}: {a.size} values for {sum(self.level_len)}")
        if lib().gmg_vec_upload_levels(self.vec(name), _ptr(a)):
            _err(f"upload_levels {name}")

    def download_levels(self, name: str) -> np.ndarray:
        a = np.empty(sum(self.level_len))
        if lib().gmg_vec_download_levels(self.vec(name), _ptr(a)):
            _err(f"download_levels {name}")
        return a

    # ---- batched hierarchies
    def split(self, packed) -> list:
        """Per-instance views of a packed vector."""
        s = self.block
        return [packed[o * s:(o + n) * s] for o, n in zip(self.pack_off, self.inst_n)]

    def pack(self, parts) -> np.ndarray:
        out = np.concatenate([np.ascontiguousarray(p, np.float64).ravel() for p in parts])
        if out.size != self.packed_len:
            raise GmgError(f"pack: {out.size} values for {self.packed_len}")
        return out

    def upload_packed(self, name: str, data):
        a = np.ascontiguousarray(data, np.float64).ravel()
        if a.size != self.packed_len:
            raise GmgError(f"upload_packed {name}: {a.size} values for {self.packed_len}")
        if lib().gmg_vec_upload_packed(self.vec(name), _ptr(a)):
            _err(f"upload_packed {name}")

    def download_packed(self, name: str) -> np.ndarray:
        a = np.empty(self.packed_len)
        if lib().gmg_vec_download_packed(self.vec(name), _ptr(a)):
            _err(f"download_packed {name}")
        return a

    def instance_result(self, ls: str, k: int) -> LResult:
        lr = LResult()
        if lib().gmg_ls_instance_result(self.np(ls), k, C.byref(lr)):
            _err("gmg_ls_instance_result")
        return lr

    # ---- hierarchy
    def size(self, level: int):
        n, s, nnz = C.c_int(), C.c_int(), C.c_longlong()
        if lib().gmg_mg_level_size(self._h, level, C.byref(n), C.byref(s), C.byref(nnz)):
            _err("gmg_mg_level_size")
        return n.value, s.value, nnz.value

    def order(self, level: int) -> np.ndarray:
        n, _, _ = self.size(level)
        p = np.empty(n, np.int32)
        lib().gmg_mg_get_order(self._h, level, _ptr(p))
        return p

    def matrix(self, level: int):
        n, s, nnz = self.size(level)
        rp, col, val = np.empty(n + 1, np.int32), np.empty(nnz, np.int32), np.empty(nnz * s * s)
        lib().gmg_mg_get_matrix(self._h, level, _ptr(rp), _ptr(col), _ptr(val))
        return rp, col, val

    def num_waves(self, level: int) -> int:
        return lib().gmg_mg_num_waves(self._h, level)

    def device_bytes(self) -> int:
        return lib().gmg_mg_device_bytes(self._h)

    def launch_count(self, reset: bool = False) -> int:
        return lib().gmg_mg_launch_count(self._h, int(reset))

    def sync(self):
        if lib().gmg_mg_sync(self._h):
            _err("gmg_mg_sync")

    # ---- user data
    def createvector(self, *names, prec: int = FP64):
        for n in names:
            if lib().gmg_vec_create(self._h, n.encode(), prec, None):
                _err(f"createvector {n}")

    def vec(self, name: str):
        v = lib().gmg_vec_by_name(self._h, name.encode())
        if not v:
            raise GmgError(f"no vector {name}")
        return v

    def mat(self, name: str = "MAT"):
        m = lib().gmg_mat_by_name(self._h, name.encode())
        if not m:
            raise GmgError(f"no matrix {name}")
        return m

    def upload(self, name: str, level: int, data):
        n, s, _ = self.size(level)
        a = np.ascontiguousarray(data, np.float64).ravel()
        if a.size != n * s:
            raise GmgError(f"upload {name}: {a.size} values for {n}x{s}")
        if lib().gmg_vec_upload(self.vec(name), level, _ptr(a)):
            _err(f"upload {name}")

    def download(self, name: str, level: int) -> np.ndarray:
        n, s, _ = self.size(level)
        a = np.empty(n * s)
        if lib().gmg_vec_download(self.vec(name), level, _ptr(a)):
            _err(f"download {name}")
        return a

    def device_ptr(self, name: str, level: int) -> int:
        p = C.c_void_p()
        if lib().gmg_vec_device_ptr(self.vec(name), level, C.byref(p)):
            _err("device_ptr")
        return p.value

    # ---- numprocs
    def npcreate(self, obj: str, cls: str):
        if lib().gmg_np_create(self._h, obj.encode(), cls.encode()):
            _err(f"npcreate {obj} $c {cls}")

    def npinit(self, obj: str, args: str = "") -> int:
        st = C.c_int()
        rc = lib().gmg_np_init(self._h, obj.encode(), args.encode(), C.byref(st))
        if rc and st.value != NP_NOT_ACTIVE:
            _err(f"npinit {obj}")
        return st.value

    def npexecute(self, obj: str, args: str):
        if lib().gmg_np_execute(self._h, obj.encode(), args.encode()):
            _err(f"npexecute {obj} {args}")

    def np(self, obj: str):
        p = lib().gmg_np_by_name(self._h, obj.encode())
        if not p:
            raise GmgError(f"no numproc {obj}")
        return p

    def npdisplay(self, obj: str) -> str:
        buf = C.create_string_buffer(4096)
        lib().gmg_np_display(self.np(obj), buf, 4096)
        return buf.value.decode()

    # NP_ITER
    def iter_preprocess(self, obj, level, x, b, A="MAT"):
        bl, res = C.c_int(), C.c_int()
        if lib().gmg_iter_preprocess(self.np(obj), level, self.vec(x), self.vec(b), self.mat(A), C.byref(bl), C.byref(res)):
            _err(f"{obj} PreProcess")
        return bl.value

    def iter_iter(self, obj, level, c, b, A="MAT"):
        res = C.c_int()
        if lib().gmg_iter_iter(self.np(obj), level, self.vec(c), self.vec(b), self.mat(A), C.byref(res)):
            _err(f"{obj} Iter")

    def iter_smooth(self, obj, level, t, b, c, steps, A="MAT"):
        """lmgc's smoothing loop: `steps` times t = Iter(b), c += t."""
        res = C.c_int()
        if lib().gmg_iter_smooth(self.np(obj), level, self.vec(t), self.vec(b), self.mat(A), self.vec(c), steps,
                                 C.byref(res)):
            _err(f"{obj} smoothing steps")

    def iter_postprocess(self, obj, level, x, b, A="MAT"):
        res = C.c_int()
        if lib().gmg_iter_postprocess(self.np(obj), level, self.vec(x), self.vec(b), self.mat(A), C.byref(res)):
            _err(f"{obj} PostProcess")

    # NP_TRANSFER
    def restrict_defect(self, obj, level, to, frm, damp=None, A="MAT"):
        res = C.c_int()
        d = _sc(damp)
        if lib().gmg_transfer_restrict_defect(self.np(obj), level, self.vec(to), self.vec(frm), self.mat(A), _ptr(d), C.byref(res)):
            _err(f"{obj} RestrictDefect")

    def interpolate_correction(self, obj, level, to, frm, damp=None, A="MAT"):
        res = C.c_int()
        d = _sc(damp)
        if lib().gmg_transfer_interpolate_correction(self.np(obj), level, self.vec(to), self.vec(frm), self.mat(A), _ptr(d), C.byref(res)):
            _err(f"{obj} InterpolateCorrection")

    # NP_LINEAR_SOLVER
    def ls_preprocess(self, obj, level, x, b, A="MAT"):
        bl, res = C.c_int(), C.c_int()
        if lib().gmg_ls_preprocess(self.np(obj), level, self.vec(x), self.vec(b), self.mat(A), C.byref(bl), C.byref(res)):
            _err(f"{obj} PreProcess")
        return bl.value

    def level_variant(self, level: int) -> dict:
        """The kernel variant of a level (autotuner's choice, -1 = by size)."""
        t, p, st = C.c_int(), C.c_int(), C.c_int()
        if lib().gmg_mg_level_variant(self._h, level, C.byref(t), C.byref(p), C.byref(st)):
            _err("level_variant")
        on = C.c_int()
        if lib().gmg_mg_level_cta_chain(self._h, level, C.byref(on)):
            _err("level_cta_chain")
        return {"tpr": t.value, "prefetch": p.value, "stream": st.value, "cta_chain": on.value}

    def domain_info(self, level: int) -> dict:
        """Subdomain order of a level: subdomains, interior rows, interface colours."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        if lib().gmg_mg_domain_info(self._h, level, C.byref(a), C.byref(b), C.byref(c)):
            _err("domain_info")
        return {"subdomains": a.value, "interior_rows": b.value, "interface_colours": c.value}

    def set_direct_host(self, on: bool):
        """Host vectors straight from / to pageable memory (True; needs a
        device that reads host page tables) or through pinned staging."""
        if lib().gmg_mg_set_direct_host(self._h, int(bool(on))):
            _err("set_direct_host")

    def set_iface_sweep(self, mode: int):
        """Interface ILU sweeps of the subdomain order: 0 one launch per
        colour, 1 (default) one cooperative launch per direction for FP64
        sweeps, 2 for FP32 sweeps as well."""
        if lib().gmg_mg_set_iface_sweep(self._h, int(mode)):
            _err("set_iface_sweep")

    def set_cta_chain(self, level: int, blocks):
        """Run the level's chained Gauss-Seidel steps as one launch per colour
        wave (0 / False), in one thread block (1 / True) or in one cluster of
        2, 4, 8 or 16 blocks; before the first graph-captured solve."""
        if lib().gmg_mg_set_level_cta_chain(self._h, level, int(blocks)):
            _err("set_cta_chain")

    def update_values(self, level: int, val):
        """New matrix values of a level (gmg_level_desc layout), structure unchanged."""
        a = np.ascontiguousarray(val, np.float64).ravel()
        n, s, nnz = self.size(level)
        if a.size != nnz * s * s:
            raise GmgError(f"update_values: {a.size} values for {nnz} blocks of {s}x{s}")
        if lib().gmg_mg_update_values(self._h, level, _ptr(a)):
            _err("update_values")

    def set_new_vectors(self, level: int, vnew):
        """VNEW flags of a level's vectors (list order)."""
        a = np.ascontiguousarray(vnew, np.int32)
        if a.size != self.size(level)[0]:
            raise GmgError(f"set_new_vectors: {a.size} flags for {self.size(level)[0]} vectors")
        if lib().gmg_mg_set_new_vectors(self._h, level, _ptr(a)):
            _err("set_new_vectors")

    def transfer_interpolate_new_vectors(self, obj, fl, tl, x):
        res = C.c_int()
        if lib().gmg_transfer_interpolate_new_vectors(self.np(obj), fl, tl, self.vec(x), C.byref(res)):
            _err(f"{obj} InterpolateNewVectors")

    def transfer_project_solution(self, obj, fl, tl, x):
        res = C.c_int()
        if lib().gmg_transfer_project_solution(self.np(obj), fl, tl, self.vec(x), C.byref(res)):
            _err(f"{obj} ProjectSolution")

    def ls_defect(self, obj, level, x, b, A="MAT"):
        res = C.c_int()
        if lib().gmg_ls_defect(self.np(obj), level, self.vec(x), self.vec(b), self.mat(A), C.byref(res)):
            _err(f"{obj} Defect")

    def ls_residuum(self, obj, fl, tl, x, b, lr: LResult, A="MAT"):
        if lib().gmg_ls_residuum(self.np(obj), fl, tl, self.vec(x), self.vec(b), self.mat(A), C.byref(lr)):
            _err(f"{obj} Residuum")
        return lr

    def ls_solver(self, obj, level, x, b, lr: LResult, abslimit=None, reduction=None, A="MAT"):
        a = None if abslimit is None else _sc(abslimit)
        r = None if reduction is None else _sc(reduction)
        if lib().gmg_ls_solver(self.np(obj), level, self.vec(x), self.vec(b), self.mat(A), _ptr(a), _ptr(r), C.byref(lr)):
            _err(f"{obj} Solver")
        return lr

    def ls_postprocess(self, obj, level, x, b, A="MAT"):
        res = C.c_int()
        if lib().gmg_ls_postprocess(self.np(obj), level, self.vec(x), self.vec(b), self.mat(A), C.byref(res)):
            _err(f"{obj} PostProcess")

    # level kernels (ugblas / ugiter / transgrid)
    def dset(self, level, x, a):
        if lib().gmg_dset(self._h, level, self.vec(x), float(a)):
            _err("dset")

    def dcopy(self, level, x, y):
        if lib().gmg_dcopy(self._h, level, self.vec(x), self.vec(y)):
            _err("dcopy")

    def dadd(self, level, x, y):
        if lib().gmg_dadd(self._h, level, self.vec(x), self.vec(y)):
            _err("dadd")

    def dmatmul_minus(self, level, x, y, A="MAT"):
        if lib().gmg_dmatmul_minus(self._h, level, self.vec(x), self.mat(A), self.vec(y)):
            _err("dmatmul_minus")

    def dmatmul(self, level, x, y, A="MAT"):
        if lib().gmg_dmatmul(self._h, level, self.vec(x), self.mat(A), self.vec(y)):
            _err("dmatmul")

    def dmatmul_add(self, level, x, y, A="MAT"):
        if lib().gmg_dmatmul_add(self._h, level, self.vec(x), self.mat(A), self.vec(y)):
            _err("dmatmul_add")

    def dscalx(self, level, x, a):
        f = _sc(a)
        if lib().gmg_dscalx(self._h, level, self.vec(x), _ptr(f)):
            _err("dscalx")

    def daxpy(self, level, x, a, y):
        f = _sc(a)
        if lib().gmg_daxpy(self._h, level, self.vec(x), _ptr(f), self.vec(y)):
            _err("daxpy")

    def ddot(self, level, x, y) -> float:
        r = C.c_double()
        if lib().gmg_ddot(self._h, level, self.vec(x), self.vec(y), C.byref(r)):
            _err("ddot")
        return r.value

    def dnrm2x(self, level, x):
        out = np.zeros(MAX_S)
        if lib().gmg_dnrm2x(self._h, level, self.vec(x), _ptr(out)):
            _err("dnrm2x")
        return out[: self.size(level)[1]]

    def l_jac(self, level, v, d, M="MAT"):
        if lib().gmg_l_jac(self._h, level, self.vec(v), self.mat(M), self.vec(d)):
            _err("l_jac")

    def l_lgs(self, level, v, d, M="MAT"):
        if lib().gmg_l_lgs(self._h, level, self.vec(v), self.mat(M), self.vec(d)):
            _err("l_lgs")

    def set_imatrix(self, level, rowptr, col, val):
        """The level's interpolation matrix (UG's IMATRIX, list order, s x s
        blocks coarse component major) for the transfer's matrix mode ($M)."""
        rp = np.ascontiguousarray(rowptr, np.int32)
        cl = np.ascontiguousarray(col, np.int32)
        vl = np.ascontiguousarray(val, np.float64)
        if lib().gmg_mg_set_imatrix(self._h, level, rp.ctypes.data, cl.ctypes.data, vl.ctypes.data):
            _err("set_imatrix")

    def restrict_by_matrix(self, level, to, frm, damp=None):
        d = _sc(damp)
        if lib().gmg_restrict_by_matrix(self._h, level, self.vec(to), self.vec(frm), _ptr(d)):
            _err("RestrictByMatrix")

    def interpolate_correction_by_matrix(self, level, to, frm, damp=None):
        d = _sc(damp)
        if lib().gmg_interpolate_correction_by_matrix(self._h, level, self.vec(to), self.vec(frm), _ptr(d)):
            _err("InterpolateCorrectionByMatrix")

    def l_ilu_factors(self, level):
        """The ILU(0) factors of a level as l_ilubthdecomp leaves them (the
        device matrix layout of `matrix(level)`, processing order)."""
        n, s, nnz = self.size(level)
        lu = np.empty(nnz * s * s)
        if lib().gmg_l_ilu_factors(self._h, level, lu.ctypes.data):
            _err("l_ilu_factors")
        return lu

    def l_ilu_decomp(self, level, beta=None, M="MAT"):
        b = _sc(beta, 0.0)
        if lib().gmg_l_ilu_decomp(self._h, level, self.mat(M), _ptr(b)):
            _err("l_ilubthdecomp")

    def l_luiter(self, level, v, d, M="MAT"):
        if lib().gmg_l_luiter(self._h, level, self.vec(v), self.mat(M), self.vec(d)):
            _err("l_luiter")

    def standard_restrict(self, level, to, frm, damp=None):
        d = _sc(damp)
        if lib().gmg_standard_restrict(self._h, level, self.vec(to), self.vec(frm), _ptr(d)):
            _err("StandardRestrict")

    def standard_interpolate_correction(self, level, to, frm, damp=None):
        d = _sc(damp)
        if lib().gmg_standard_interpolate_correction(self._h, level, self.vec(to), self.vec(frm), _ptr(d)):
            _err("StandardInterpolateCorrection")

    def solve_host(self, solver: str, b, x=None):
        """gmg_solve_host: b (finest level, list order; packed on a batched
        hierarchy; every level, concatenated, on a locally refined one) ->
        (x, LResult), x in the layout of b."""
        n, s, _ = self.size(self.top)
        length = self.packed_len if self.ninst else (sum(self.level_len) if self.local else n * s)
        bb = np.ascontiguousarray(b, np.float64).ravel()
        if bb.size != length:
            raise GmgError(f"solve {solver}: {bb.size} values for {length}")
        xx = np.empty(length) if x is None else x
        lr = LResult()
        if lib().gmg_solve_host(self._h, solver.encode(), _ptr(bb), _ptr(xx), C.byref(lr)):
            _err(f"solve {solver}")
        return xx, lr

    def close(self):
        if getattr(self, "_h", None):
            lib().gmg_mg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def imatrices_from_ugfx(fx: dict) -> list:
    """The interpolation matrices of a UG export (None on level 0)."""
    n = int(fx["nlevels"][0])
    return [None] + [(fx[f"M{l}_rowptr"], fx[f"M{l}_col"], fx[f"M{l}_val"]) for l in range(1, n)]


def setup_lmgc(mg: MultiGrid, smoother: str = "jac", baselevel: int = 0, nu1: int = 2, nu2: int = 2,
               damp: float | None = None, red: float = 1e-10, abslimit: float = 1e-50, maxit: int = 100,
               mixed: bool = False, x: str = "sol", b: str = "rhs", name: str = "mgs",
               fuse: int | None = None, graph: bool = True, bsmem: int | None = None,
               dloop: bool = True, narrow: bool = True, transfer: str = "", defect: bool = False) -> str:
    """The standard script of the workloads, as UG numproc commands:

        npcreate transfer $c gtransfer; npcreate smooth $c g<smoother>;
        npcreate base $c gex; npcreate basesolver $c gls ($red 1e-14 $m 1 $I base);
        npcreate lmgc $c glmgc ($S smooth smooth basesolver $T transfer $n1 $n2 $b);
        npcreate mgs $c gls ($A MAT $x sol $b rhs $red $abslimit $m $I lmgc)."""
    for v in (x, b):
        try:
            mg.vec(v)
        except GmgError:
            mg.createvector(v)
    mg.npcreate("transfer", "transfer.gtransfer"); mg.npinit("transfer", transfer)
    mg.npcreate("smooth", f"iter.g{smoother}")
    if damp is None:
        damp = 0.8 if smoother == "jac" else 1.0
    mg.npinit("smooth", f"$damp {damp}")
    mg.npcreate("base", "iter.gex"); mg.npinit("base", "")
    mg.npcreate("basesolver", "linear_solver.gls"); mg.npinit("basesolver", "$red 1e-14 $m 1 $I base")
    mg.npcreate("lmgc", "iter.glmgc")
    fz = ("" if fuse is None else f" $fuse {int(fuse)}") + ("" if bsmem is None else f" $bsmem {int(bsmem)}")
    fz += "" if narrow else " $narrow 0"
    fz += " $defect 1" if defect else ""
    mg.npinit("lmgc", f"$S smooth smooth basesolver $T transfer $n1 {nu1} $n2 {nu2} $b {baselevel}{fz}")
    mg.npcreate(name, "linear_solver.gls")
    st = mg.npinit(name, f"$A MAT $x {x} $b {b} $red {red} $abslimit {abslimit} $m {maxit} $I lmgc"
                         f" $mixed {int(mixed)} $graph {int(graph)} $dloop {int(dloop)}")
    if st != NP_EXECUTABLE:
        raise GmgError(f"{name} not executable (status {st})")
    return name
