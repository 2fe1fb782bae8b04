// gpu_numprocs.cc -- UG numproc classes that run on the GB300 library.
//
// This file is the UG side of the drop-in: it is compiled into a UG 3.12.1
// build (against UG's own headers, next to np/procs/) and linked with
// libug_gb300 (include/ug_gb300.h).  InitGpuNumProcs() registers, with
// CreateClass (np/udm/numproc.cc:110), the classes
//
//   iter.gjac  iter.ggs  iter.gilu  iter.gex  iter.glmgc     (NP_ITER, np/procs/iter.h:68-101)
//   transfer.gtransfer                                       (NP_TRANSFER, np/procs/transfer.h:79-166)
//   linear_solver.gls  linear_solver.gcg  linear_solver.gbcgs (NP_LINEAR_SOLVER, np/procs/ls.h:79-132)
//
// whose function pointers forward to the library's gmg_iter_* /
// gmg_transfer_* / gmg_ls_* entry points.  A UG script swaps class names
// only ("npcreate mgs $c gls; npinit mgs $A MAT $x sol $b rhs ...").
//
// How the two sides meet:
//   * the device hierarchy of a MULTIGRID is built on the first PreProcess
//     (and again whenever the grid's shape changed): every level's VECTOR
//     list and MATRIX lists are flattened into gmg_level_desc arrays (list
//     order, diagonal first, VCLASS / VNCLASS / VECSKIP, the standard
//     transfer's weights) and handed to gmg_mg_create; on an unchanged shape
//     the new MATRIX values go to gmg_mg_update_values;
//   * every npcreate / npinit of these classes is recorded and replayed into
//     the device hierarchy in the same order (so "$S smooth smooth base"
//     finds its objects there); the matrix descriptor is the device's "MAT",
//     vectors are device vectors named after UG's VECDATA_DESCs;
//   * vector data crosses at the boundary of each forwarded call: the inputs
//     are uploaded from the VECTORs (levels 0..level, list order), the
//     outputs written back;
//   * errors of the library (no device, bad arguments, a failed
//     decomposition) return through NP_RETURN (np/np.h:89) with the
//     library's message printed by UserWriteF, as UG's own numprocs report.
//
// `$order list|color|domain` on a gls / gcg / gbcgs object chooses the
// device processing order (default list: Gauss-Seidel and ILU sweep UG's
// VECTOR lists); it is taken out of the arguments forwarded to the library.
#include <config.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "gm.h"
#include "iter.h"
#include "ls.h"
#include "np.h"
#include "numproc.h"
#include "shapes.h"
#include "transfer.h"
#include "udm.h"
#include "ugdevices.h"

#include "ug_gb300.h"

USING_UG_NAMESPACES

namespace {

// ------------------------------------------------------------------ flattening
struct FlatLevel {
  int n = 0, s = 1;
  std::vector<int> rowptr, col, vclass, vnclass, skip, prow, pcol;
  std::vector<double> val, pw;
};

// the VECTOR lists of every level as list-order indices
struct Lists {
  std::vector<std::vector<VECTOR *>> vecs;
  std::vector<std::unordered_map<const VECTOR *, int>> idx;
};

Lists index_levels(MULTIGRID *mg) {
  Lists L;
  const int top = TOPLEVEL(mg);
  L.vecs.resize(top + 1);
  L.idx.resize(top + 1);
  for (int l = 0; l <= top; ++l)
    for (VECTOR *v = FIRSTVECTOR(GRID_ON_LEVEL(mg, l)); v; v = SUCCVC(v)) {
      L.idx[l][v] = (int)L.vecs[l].size();
      L.vecs[l].push_back(v);
    }
  return L;
}

// returns 0, or a nonzero code with msg set
int flatten(MULTIGRID *mg, MATDATA_DESC *A, std::vector<FlatLevel> &out, std::string &msg) {
  const Lists L = index_levels(mg);
  const int top = TOPLEVEL(mg);
  out.assign(top + 1, FlatLevel());
  for (int l = 0; l <= top; ++l) {
    FlatLevel &F = out[l];
    F.n = (int)L.vecs[l].size();
    F.rowptr.assign(1, 0);
    for (VECTOR *v : L.vecs[l]) {
      const int tv = VTYPE(v);
      const int s = MD_ROWS_IN_RT_CT(A, tv, tv);
      if (s <= 0 || s > GMG_MAX_S) { msg = "matrix block size out of range"; return 1; }
      if (F.rowptr.size() == 1) F.s = s;
      if (s != F.s) { msg = "VECTOR types with different component counts are not supported"; return 1; }
      F.vclass.push_back(VCLASS(v));
      F.vnclass.push_back(VNCLASS(v));
      F.skip.push_back((int)VECSKIP(v));
      for (MATRIX *m = VSTART(v); m; m = MNEXT(m)) {
        VECTOR *w = MDEST(m);
        auto it = L.idx[l].find(w);
        if (it == L.idx[l].end()) { msg = "MATRIX entry to a VECTOR of another level"; return 1; }
        F.col.push_back(it->second);
        const SHORT *cmp = MD_MCMPPTR_OF_RT_CT(A, tv, VTYPE(w));
        for (int k = 0; k < s * s; ++k) F.val.push_back(MVALUE(m, cmp[k]));
      }
      F.rowptr.push_back((int)F.col.size());
    }
    if (l == 0) continue;
    // standard transfer weights (transgrid.cc:117-347): a corner node copies
    // its father; any other node takes the father element's corners with the
    // shape functions GNs at its local coordinates
    std::vector<std::vector<std::pair<int, double>>> rows(F.n);
    for (NODE *nd = FIRSTNODE(GRID_ON_LEVEL(mg, l)); nd; nd = SUCCN(nd)) {
      auto it = L.idx[l].find(NVECTOR(nd));
      if (it == L.idx[l].end()) continue;
      if (CORNERTYPE(nd)) {
        rows[it->second].push_back({L.idx[l - 1].at(NVECTOR((NODE *)NFATHER(nd))), 1.0});
      } else {
        VERTEX *vx = MYVERTEX(nd);
        ELEMENT *fe = VFATHER(vx);
        const int nc = CORNERS_OF_ELEM(fe);
        DOUBLE c[MAX_CORNERS_OF_ELEM];
        GNs(nc, LCVECT(vx), c);
        for (int i = 0; i < nc; ++i)
          if (c[i] != 0.0) rows[it->second].push_back({L.idx[l - 1].at(NVECTOR(CORNER(fe, i))), c[i]});
      }
    }
    F.prow.assign(1, 0);
    for (auto &r : rows) {
      for (auto &e : r) { F.pcol.push_back(e.first); F.pw.push_back(e.second); }
      F.prow.push_back((int)F.pcol.size());
    }
  }
  return 0;
}

std::vector<gmg_level_desc> descs(std::vector<FlatLevel> &lev) {
  std::vector<gmg_level_desc> d(lev.size());
  for (size_t l = 0; l < lev.size(); ++l) {
    FlatLevel &F = lev[l];
    d[l] = gmg_level_desc{F.n, F.s, F.rowptr.data(), F.col.data(), F.val.data(), F.vclass.data(),
                          F.vnclass.data(), F.skip.data(), l ? F.prow.data() : nullptr,
                          l ? F.pcol.data() : nullptr, l ? F.pw.data() : nullptr};
  }
  return d;
}

// ------------------------------------------------------------------ device side of a MULTIGRID
struct Record {
  std::string name, cls, args;  // object name, class ("iter.glmgc"), npinit arguments
  bool inited = false;
};

struct Device {
  gmg_mg *mg = nullptr;
  std::vector<long long> shape;  // per level: VECTORs, MATRIX entries
  int order = GMG_ORDER_LIST;
  std::vector<Record> nps;       // npcreate / npinit order
};

std::map<MULTIGRID *, Device> g_dev;

std::string object_name(NP_BASE *np) {  // "linear_solver.gls.mgs" -> "mgs"
  const char *full = ENVITEM_NAME(np), *dot = strrchr(full, '.');
  return dot ? std::string(dot + 1) : std::string(full);
}
std::string class_name(NP_BASE *np) {  // -> "linear_solver.gls"
  const char *full = ENVITEM_NAME(np), *dot = strrchr(full, '.');
  return dot ? std::string(full, dot - full) : std::string();
}

Record *record_of(NP_BASE *np) {
  Device &D = g_dev[NP_MG(np)];
  const std::string nm = object_name(np);
  for (Record &r : D.nps)
    if (r.name == nm) return &r;
  D.nps.push_back(Record{nm, class_name(np), "", false});
  return &D.nps.back();
}

// the npinit arguments as one string ("$A MAT $x sol ..."); `$order` and the
// matrix name are the glue's: the first is taken out, the second becomes MAT
std::string join_args(INT argc, char **argv, int *order) {
  std::string out;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    while (!a.empty() && (a.back() == ' ' || a.back() == '\n')) a.pop_back();
    if (a.compare(0, 6, "order ") == 0) {
      if (order) {
        const std::string o = a.substr(6);
        *order = o == "color" ? GMG_ORDER_COLOR : o == "domain" ? GMG_ORDER_DOMAIN : GMG_ORDER_LIST;
      }
      continue;
    }
    if (a.compare(0, 2, "A ") == 0) a = "A MAT";
    out += (out.empty() ? "$" : " $") + a;
  }
  return out;
}

void report(const char *where) {
  const char *e = gmg_last_error();
  UserWriteF("gpu numprocs: %s: %s\n", where, e && *e ? e : "failed");
}

// the device hierarchy of mg, built or refreshed from UG's lists and values;
// every recorded numproc replayed into a new one.  0 or nonzero (reported).
int ensure_device(MULTIGRID *mg, MATDATA_DESC *A) {
  if (!A) { UserWriteF("gpu numprocs: no matrix descriptor\n"); return 1; }
  Device &D = g_dev[mg];
  std::vector<FlatLevel> lev;
  std::string msg;
  if (flatten(mg, A, lev, msg)) { UserWriteF("gpu numprocs: flattening: %s\n", msg.c_str()); return 1; }
  std::vector<long long> shape;
  for (auto &F : lev) { shape.push_back(F.n); shape.push_back(F.rowptr.back()); }
  if (D.mg && shape == D.shape) {
    for (size_t l = 0; l < lev.size(); ++l)
      if (gmg_mg_update_values(D.mg, (int)l, lev[l].val.data())) { report("gmg_mg_update_values"); return 1; }
    return 0;
  }
  if (D.mg) { gmg_mg_destroy(D.mg); D.mg = nullptr; }
  std::vector<gmg_level_desc> d = descs(lev);
  gmg_mg_opts o{};
  o.order = D.order;
  o.fp32_copy = 1;
  int dev = 0;
  o.device = dev;
  if (gmg_mg_create(d.data(), (int)d.size(), &o, &D.mg)) { D.mg = nullptr; report("gmg_mg_create"); return 1; }
  D.shape = shape;
  for (VECDATA_DESC *vd = GetFirstVector(mg); vd; vd = GetNextVector(vd)) {
    gmg_vec *v = nullptr;
    if (!gmg_vec_by_name(D.mg, ENVITEM_NAME(vd)) && gmg_vec_create(D.mg, ENVITEM_NAME(vd), GMG_PREC_FP64, &v)) {
      report("gmg_vec_create");
      return 1;
    }
  }
  for (Record &r : D.nps) {
    if (gmg_np_create(D.mg, r.name.c_str(), r.cls.c_str())) { report("npcreate"); return 1; }
    int st = 0;
    if (r.inited && gmg_np_init(D.mg, r.name.c_str(), r.args.c_str(), &st) && st != NP_NOT_ACTIVE) {
      report("npinit");
      return 1;
    }
  }
  return 0;
}

gmg_np *dev_np(NP_BASE *np) {
  Device &D = g_dev[NP_MG(np)];
  return D.mg ? gmg_np_by_name(D.mg, object_name(np).c_str()) : nullptr;
}
gmg_vec *dev_vec(MULTIGRID *mg, VECDATA_DESC *vd) {
  Device &D = g_dev[mg];
  return (D.mg && vd) ? gmg_vec_by_name(D.mg, ENVITEM_NAME(vd)) : nullptr;
}
gmg_mat *dev_mat(MULTIGRID *mg) {
  Device &D = g_dev[mg];
  return D.mg ? gmg_mat_by_name(D.mg, "MAT") : nullptr;
}

// VECTOR values of levels lo..hi <-> device (list order, s components)
int move(MULTIGRID *mg, VECDATA_DESC *vd, int lo, int hi, bool up) {
  gmg_vec *dv = dev_vec(mg, vd);
  if (!dv) { UserWriteF("gpu numprocs: vector %s has no device copy\n", vd ? ENVITEM_NAME(vd) : "(null)"); return 1; }
  std::vector<double> h;
  for (int l = std::max(lo, 0); l <= hi; ++l) {
    h.clear();
    std::vector<VECTOR *> vs;
    for (VECTOR *v = FIRSTVECTOR(GRID_ON_LEVEL(mg, l)); v; v = SUCCVC(v)) vs.push_back(v);
    for (VECTOR *v : vs)
      for (int c = 0; c < VD_NCMPS_IN_TYPE(vd, VTYPE(v)); ++c) h.push_back(up ? VVALUE(v, VD_CMP_OF_TYPE(vd, VTYPE(v), c)) : 0.0);
    if (up) {
      if (gmg_vec_upload(dv, l, h.data())) { report("gmg_vec_upload"); return 1; }
    } else {
      if (gmg_vec_download(dv, l, h.data())) { report("gmg_vec_download"); return 1; }
      size_t i = 0;
      for (VECTOR *v : vs)
        for (int c = 0; c < VD_NCMPS_IN_TYPE(vd, VTYPE(v)); ++c) VVALUE(v, VD_CMP_OF_TYPE(vd, VTYPE(v), c)) = h[i++];
    }
  }
  return 0;
}
int up(MULTIGRID *mg, VECDATA_DESC *vd, int lo, int hi) { return move(mg, vd, lo, hi, true); }
int down(MULTIGRID *mg, VECDATA_DESC *vd, int lo, int hi) { return move(mg, vd, lo, hi, false); }

void lres_to_ug(const gmg_lresult &g, LRESULT *u) {
  u->error_code = g.error_code;
  u->converged = g.converged;
  for (int i = 0; i < MAX_VEC_COMP && i < GMG_MAX_S; ++i) {
    u->first_defect[i] = g.first_defect[i];
    u->last_defect[i] = g.last_defect[i];
  }
  u->number_of_linear_iterations = g.number_of_linear_iterations;
}

// ------------------------------------------------------------------ NP_ITER
struct NP_GPU_ITER {
  NP_ITER iter;
};

INT GpuIterInit(NP_BASE *base, INT argc, char **argv) {
  Record *r = record_of(base);
  r->args = join_args(argc, argv, nullptr);
  r->inited = true;
  return NPIterInit((NP_ITER *)base, argc, argv);
}

INT GpuIterDisplay(NP_BASE *base) {
  Record *r = record_of(base);
  UserWriteF("class %s (GB300)\nnpinit %s\n", r->cls.c_str(), r->args.c_str());
  return NPIterDisplay((NP_ITER *)base);
}

INT GpuIterPreProcess(NP_ITER *it, INT level, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A, INT *bl,
                      INT *result) {
  MULTIGRID *mg = NP_MG(it);
  if (ensure_device(mg, A)) NP_RETURN(1, result[0]);
  int res = 0, blv = 0;
  if (up(mg, x, 0, level) || up(mg, b, 0, level)) NP_RETURN(1, result[0]);
  if (gmg_iter_preprocess(dev_np(&it->base), level, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), &blv, &res)) {
    report("PreProcess");
    NP_RETURN(1, result[0]);
  }
  *bl = blv;
  return 0;
}

INT GpuIterIter(NP_ITER *it, INT level, VECDATA_DESC *c, VECDATA_DESC *b, MATDATA_DESC *A, INT *result) {
  MULTIGRID *mg = NP_MG(it);
  if (!g_dev[mg].mg && ensure_device(mg, A)) NP_RETURN(1, result[0]);
  int res = 0;
  if (up(mg, c, 0, level) || up(mg, b, 0, level)) NP_RETURN(1, result[0]);
  if (gmg_iter_iter(dev_np(&it->base), level, dev_vec(mg, c), dev_vec(mg, b), dev_mat(mg), &res)) {
    report("Iter");
    NP_RETURN(1, result[0]);
  }
  if (down(mg, c, 0, level) || down(mg, b, 0, level)) NP_RETURN(1, result[0]);
  return 0;
}

INT GpuIterPostProcess(NP_ITER *it, INT level, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A, INT *result) {
  MULTIGRID *mg = NP_MG(it);
  if (!g_dev[mg].mg) return 0;
  int res = 0;
  if (gmg_iter_postprocess(dev_np(&it->base), level, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), &res)) {
    report("PostProcess");
    NP_RETURN(1, result[0]);
  }
  return 0;
}

INT GpuIterConstruct(NP_BASE *base) {
  base->Init = GpuIterInit;
  base->Display = GpuIterDisplay;
  base->Execute = NPIterExecute;
  NP_ITER *it = (NP_ITER *)base;
  it->PreProcess = GpuIterPreProcess;
  it->Iter = GpuIterIter;
  it->PostProcess = GpuIterPostProcess;
  record_of(base);
  return 0;
}

// ------------------------------------------------------------------ NP_TRANSFER
struct NP_GPU_TRANSFER {
  NP_TRANSFER tr;
};

INT GpuTransferInit(NP_BASE *base, INT argc, char **argv) {
  Record *r = record_of(base);
  r->args = join_args(argc, argv, nullptr);
  r->inited = true;
  return NPTransferInit((NP_TRANSFER *)base, argc, argv);
}

INT GpuTransferDisplay(NP_BASE *base) {
  Record *r = record_of(base);
  UserWriteF("class %s (GB300)\nnpinit %s\n", r->cls.c_str(), r->args.c_str());
  return NPTransferDisplay((NP_TRANSFER *)base);
}

INT GpuTransferPreProcess(NP_TRANSFER *t, INT *fl, INT tl, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A,
                          INT *result) {
  MULTIGRID *mg = NP_MG(t);
  if (ensure_device(mg, A)) NP_RETURN(1, result[0]);
  int f = *fl, res = 0;
  if (gmg_transfer_preprocess(dev_np(&t->base), &f, tl, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), &res)) {
    report("transfer PreProcess");
    NP_RETURN(1, result[0]);
  }
  *fl = f;
  return 0;
}

INT GpuRestrictDefect(NP_TRANSFER *t, INT level, VECDATA_DESC *to, VECDATA_DESC *from, MATDATA_DESC *A,
                      VEC_SCALAR damp, INT *result) {
  MULTIGRID *mg = NP_MG(t);
  if (!g_dev[mg].mg && ensure_device(mg, A)) NP_RETURN(1, result[0]);
  double d[GMG_MAX_S];
  for (int i = 0; i < GMG_MAX_S; ++i) d[i] = i < MAX_VEC_COMP ? damp[i] : 1.0;
  int res = 0;
  if (up(mg, to, level - 1, level - 1) || up(mg, from, level, level)) NP_RETURN(1, result[0]);
  if (gmg_transfer_restrict_defect(dev_np(&t->base), level, dev_vec(mg, to), dev_vec(mg, from), dev_mat(mg), d,
                                   &res)) {
    report("RestrictDefect");
    NP_RETURN(1, result[0]);
  }
  if (down(mg, to, level - 1, level - 1)) NP_RETURN(1, result[0]);
  return 0;
}

INT GpuInterpolateCorrection(NP_TRANSFER *t, INT level, VECDATA_DESC *to, VECDATA_DESC *from, MATDATA_DESC *A,
                             VEC_SCALAR damp, INT *result) {
  MULTIGRID *mg = NP_MG(t);
  if (!g_dev[mg].mg && ensure_device(mg, A)) NP_RETURN(1, result[0]);
  double d[GMG_MAX_S];
  for (int i = 0; i < GMG_MAX_S; ++i) d[i] = i < MAX_VEC_COMP ? damp[i] : 1.0;
  int res = 0;
  if (up(mg, from, level - 1, level - 1)) NP_RETURN(1, result[0]);
  if (gmg_transfer_interpolate_correction(dev_np(&t->base), level, dev_vec(mg, to), dev_vec(mg, from), dev_mat(mg),
                                          d, &res)) {
    report("InterpolateCorrection");
    NP_RETURN(1, result[0]);
  }
  if (down(mg, to, level, level)) NP_RETURN(1, result[0]);
  return 0;
}

INT GpuInterpolateNewVectors(NP_TRANSFER *t, INT fl, INT tl, VECDATA_DESC *x, INT *result) {
  MULTIGRID *mg = NP_MG(t);
  if (!g_dev[mg].mg) NP_RETURN(1, result[0]);
  int res = 0;
  if (up(mg, x, fl, tl)) NP_RETURN(1, result[0]);
  if (gmg_transfer_interpolate_new_vectors(dev_np(&t->base), fl, tl, dev_vec(mg, x), &res)) {
    report("InterpolateNewVectors");
    NP_RETURN(1, result[0]);
  }
  if (down(mg, x, fl, tl)) NP_RETURN(1, result[0]);
  return 0;
}

INT GpuProjectSolution(NP_TRANSFER *t, INT fl, INT tl, VECDATA_DESC *x, INT *result) {
  MULTIGRID *mg = NP_MG(t);
  if (!g_dev[mg].mg) NP_RETURN(1, result[0]);
  int res = 0;
  if (up(mg, x, fl, tl)) NP_RETURN(1, result[0]);
  if (gmg_transfer_project_solution(dev_np(&t->base), fl, tl, dev_vec(mg, x), &res)) {
    report("ProjectSolution");
    NP_RETURN(1, result[0]);
  }
  if (down(mg, x, fl, tl)) NP_RETURN(1, result[0]);
  return 0;
}

INT GpuAdaptCorrection(NP_TRANSFER *t, INT level, VECDATA_DESC *c, VECDATA_DESC *b, MATDATA_DESC *A, INT *result) {
  MULTIGRID *mg = NP_MG(t);
  if (!g_dev[mg].mg) return 0;
  int res = 0;
  if (gmg_transfer_adapt_correction(dev_np(&t->base), level, dev_vec(mg, c), dev_vec(mg, b), dev_mat(mg), &res)) {
    report("AdaptCorrection");
    NP_RETURN(1, result[0]);
  }
  return 0;
}

INT GpuTransferPostProcess(NP_TRANSFER *t, INT *fl, INT tl, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A,
                           INT *result) {
  MULTIGRID *mg = NP_MG(t);
  if (!g_dev[mg].mg) return 0;
  int f = *fl, res = 0;
  if (gmg_transfer_postprocess(dev_np(&t->base), &f, tl, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), &res)) {
    report("transfer PostProcess");
    NP_RETURN(1, result[0]);
  }
  *fl = f;
  return 0;
}

INT GpuTransferConstruct(NP_BASE *base) {
  base->Init = GpuTransferInit;
  base->Display = GpuTransferDisplay;
  base->Execute = NPTransferExecute;
  NP_TRANSFER *t = (NP_TRANSFER *)base;
  t->PreProcess = GpuTransferPreProcess;
  t->PreProcessSolution = NULL;
  t->PreProcessProject = NULL;
  t->RestrictDefect = GpuRestrictDefect;
  t->InterpolateCorrection = GpuInterpolateCorrection;
  t->InterpolateNewVectors = GpuInterpolateNewVectors;
  t->ProjectSolution = GpuProjectSolution;
  t->AdaptCorrection = GpuAdaptCorrection;
  t->PostProcess = GpuTransferPostProcess;
  t->PostProcessProject = NULL;
  t->PostProcessSolution = NULL;
  record_of(base);
  return 0;
}

// ------------------------------------------------------------------ NP_LINEAR_SOLVER
struct NP_GPU_LS {
  NP_LINEAR_SOLVER ls;
};

INT GpuLsInit(NP_BASE *base, INT argc, char **argv) {
  Record *r = record_of(base);
  int order = g_dev[NP_MG(base)].order;
  r->args = join_args(argc, argv, &order);
  r->inited = true;
  Device &D = g_dev[NP_MG(base)];
  if (order != D.order && D.mg) {  // a new processing order needs a new device hierarchy
    gmg_mg_destroy(D.mg);
    D.mg = nullptr;
  }
  D.order = order;
  return NPLinearSolverInit((NP_LINEAR_SOLVER *)base, argc, argv);
}

INT GpuLsDisplay(NP_BASE *base) {
  Record *r = record_of(base);
  UserWriteF("class %s (GB300)\nnpinit %s\n", r->cls.c_str(), r->args.c_str());
  return NPLinearSolverDisplay((NP_LINEAR_SOLVER *)base);
}

INT GpuLsPreProcess(NP_LINEAR_SOLVER *ls, INT level, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A, INT *bl,
                    INT *result) {
  MULTIGRID *mg = NP_MG(ls);
  if (ensure_device(mg, A)) NP_RETURN(1, result[0]);
  if (up(mg, x, 0, level) || up(mg, b, 0, level)) NP_RETURN(1, result[0]);
  int blv = 0, res = 0;
  if (gmg_ls_preprocess(dev_np(&ls->base), level, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), &blv, &res)) {
    report("linear solver PreProcess");
    NP_RETURN(1, result[0]);
  }
  *bl = blv;
  return 0;
}

INT GpuLsDefect(NP_LINEAR_SOLVER *ls, INT level, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A, INT *result) {
  MULTIGRID *mg = NP_MG(ls);
  if (!g_dev[mg].mg) NP_RETURN(1, result[0]);
  int res = 0;
  if (up(mg, x, 0, level) || up(mg, b, 0, level)) NP_RETURN(1, result[0]);
  if (gmg_ls_defect(dev_np(&ls->base), level, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), &res)) {
    report("Defect");
    NP_RETURN(1, result[0]);
  }
  if (down(mg, b, 0, level)) NP_RETURN(1, result[0]);
  return 0;
}

INT GpuLsResiduum(NP_LINEAR_SOLVER *ls, INT fl, INT tl, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A,
                  LRESULT *lr) {
  MULTIGRID *mg = NP_MG(ls);
  gmg_lresult g{};
  if (!g_dev[mg].mg || up(mg, b, 0, tl) ||
      gmg_ls_residuum(dev_np(&ls->base), fl, tl, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), &g)) {
    report("Residuum");
    lr->error_code = __LINE__;
    return 1;
  }
  lres_to_ug(g, lr);
  return 0;
}

INT GpuLsSolver(NP_LINEAR_SOLVER *ls, INT level, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A,
                VEC_SCALAR abslimit, VEC_SCALAR reduction, LRESULT *lr) {
  MULTIGRID *mg = NP_MG(ls);
  double al[GMG_MAX_S], red[GMG_MAX_S];
  for (int i = 0; i < GMG_MAX_S; ++i) {
    al[i] = i < MAX_VEC_COMP ? abslimit[i] : abslimit[0];
    red[i] = i < MAX_VEC_COMP ? reduction[i] : reduction[0];
  }
  gmg_lresult g{};
  g.first_defect[0] = lr->first_defect[0];
  if (!g_dev[mg].mg || up(mg, x, 0, level) || up(mg, b, 0, level)) {
    lr->error_code = __LINE__;
    return 1;
  }
  for (int i = 0; i < GMG_MAX_S && i < MAX_VEC_COMP; ++i) g.first_defect[i] = lr->first_defect[i];
  if (gmg_ls_solver(dev_np(&ls->base), level, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), al, red, &g)) {
    report("Solver");
    lr->error_code = __LINE__;
    return 1;
  }
  lres_to_ug(g, lr);
  if (down(mg, x, 0, level) || down(mg, b, 0, level)) {
    lr->error_code = __LINE__;
    return 1;
  }
  return 0;
}

INT GpuLsPostProcess(NP_LINEAR_SOLVER *ls, INT level, VECDATA_DESC *x, VECDATA_DESC *b, MATDATA_DESC *A,
                     INT *result) {
  MULTIGRID *mg = NP_MG(ls);
  if (!g_dev[mg].mg) return 0;
  int res = 0;
  if (gmg_ls_postprocess(dev_np(&ls->base), level, dev_vec(mg, x), dev_vec(mg, b), dev_mat(mg), &res)) {
    report("linear solver PostProcess");
    NP_RETURN(1, result[0]);
  }
  if (down(mg, x, 0, level)) NP_RETURN(1, result[0]);
  return 0;
}

INT GpuLsConstruct(NP_BASE *base) {
  base->Init = GpuLsInit;
  base->Display = GpuLsDisplay;
  base->Execute = NPLinearSolverExecute;
  NP_LINEAR_SOLVER *ls = (NP_LINEAR_SOLVER *)base;
  ls->PreProcess = GpuLsPreProcess;
  ls->Defect = GpuLsDefect;
  ls->Residuum = GpuLsResiduum;
  ls->Solver = GpuLsSolver;
  ls->PostProcess = GpuLsPostProcess;
  record_of(base);
  return 0;
}

}  // namespace

// Registers the GB300 numproc classes (call once, after InitUg, like the
// Init* functions of np/initnp.cc).  0 on success, else the __LINE__ of the
// failing CreateClass.
INT InitGpuNumProcs(void) {
  static const char *iters[] = {".gjac", ".ggs", ".gilu", ".gex", ".glmgc"};
  for (const char *c : iters)
    if (CreateClass((std::string(ITER_CLASS_NAME) + c).c_str(), sizeof(NP_GPU_ITER), GpuIterConstruct))
      return __LINE__;
  if (CreateClass(TRANSFER_CLASS_NAME ".gtransfer", sizeof(NP_GPU_TRANSFER), GpuTransferConstruct)) return __LINE__;
  static const char *lss[] = {".gls", ".gcg", ".gbcgs"};
  for (const char *c : lss)
    if (CreateClass((std::string(LINEAR_SOLVER_CLASS_NAME) + c).c_str(), sizeof(NP_GPU_LS), GpuLsConstruct))
      return __LINE__;
  return 0;
}

// The flattened hierarchy of mg as the device receives it (for checking a
// UG build's flattening without a device): levels, VECTORs and MATRIX
// entries of level `level`, transfer weights of that level.
INT GpuNumProcsFlatten(MULTIGRID *mg, MATDATA_DESC *A, INT level, INT *nlevels, INT *n, INT *nnz, INT *npw) {
  std::vector<FlatLevel> lev;
  std::string msg;
  if (flatten(mg, A, lev, msg)) {
    UserWriteF("gpu numprocs: flattening: %s\n", msg.c_str());
    return 1;
  }
  *nlevels = (INT)lev.size();
  if (level < 0 || level >= (INT)lev.size()) return 1;
  *n = lev[level].n;
  *nnz = lev[level].rowptr.back();
  *npw = level ? (INT)lev[level].pw.size() : 0;
  return 0;
}
