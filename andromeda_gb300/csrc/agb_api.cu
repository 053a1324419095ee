// C ABI of the GB300 BEM hot path: context, mesh/problem state, fused
// assembly, block LSQR solve and the resistance-tensor workflow.
#include "../../include/andromeda_gb300.h"
#include "agb_assembly.cuh"
#include "agb_lsqr.cuh"
#include "agb_general.cuh"
#include "agb_batch.cuh"
#include "agb_lu.cuh"
#include "agb_mlp.cuh"
#include "agb_mfree.cuh"
#include <random>
#include "quad_tables.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

namespace agb {
cudaError_t upload_gauss_tables();
}

using namespace agb;

struct agb_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // mesh (host)
  int nnodes = 0, nelem = 0;
  std::vector<double> xyz;
  std::vector<int> etype, con, bcid;
  bool has_mesh = false;
  // problem
  int kind = 0, neq = 0;
  IntegOpt iopt;  // triangle integration options (agb_set_integration)
  int solver = AGB_SOLVER_LSQR;  // agb_set_solver
  int gmres_restart = 40;        // agb_set_gmres_restart (LIS's default restart length)
  bool resid_fp64 = false;       // agb_set_residual_mode
  MfOp mfop;                   // matrix-free operator (AGB_MATRIX_FREE)
  float* d_self6 = nullptr;
  double* d_lu = nullptr;      // column-major LU factors of the unscaled FP64 system (agb_solve_lu)
  std::vector<int> lu_ipiv;    // its pivots (1-based)
  bool lu_ready = false;
  int lu_info = 0;
  std::vector<int> walls;
  std::vector<double> normMul;
  double diff = 1.0;
  std::vector<int> known;
  int itri = 5, iqud = 4;
  bool has_problem = false;
  // subdomain order
  std::vector<int> elemList, posOfElem, wallIdx;
  int ne = 0;
  bool all_dirichlet = false, all_tri = false;
  // device state
  double* d_xyz = nullptr;
  int *d_etype = nullptr, *d_con = nullptr, *d_wall = nullptr;
  double* d_normMul = nullptr;
  ElemGeom* d_geom = nullptr;
  RuleDev rule;
  // general path (all source rows, any BC mix)
  GeneralLayout gl;
  GeneralDev gd;
  double* d_rhsM = nullptr;   // dense rhs matrix of the general system (nrow x nb)
  bool general = false;       // the assembled system came from the general path
  double* d_b = nullptr;
  size_t cap_b = 0;
  // assembled system
  int prec = -1;
  void* d_A = nullptr;
  int64_t lda = 0;
  int m = 0, n = 0;
  double* d_q = nullptr;
  bool q_ready = false;  // d_q holds lsqr_precon's column scaling of the assembled system
  std::vector<int> node_wall_in;  // agb_set_node_walls: wall id per global node (< 0: the automatic rule)
  bool assembled = false;
  DenseLsqr lsqr;
  // scratch
  void* d_pts = nullptr;
  void* d_src = nullptr;
  void* d_nrm = nullptr;
  void* d_colscale = nullptr;
  double *d_u = nullptr, *d_rhs = nullptr, *d_x = nullptr, *d_ft = nullptr;
  double *d_res = nullptr, *d_dx = nullptr;  // refinement: FP64 residual and correction
  int *d_active = nullptr;
  unsigned char* d_rowact = nullptr;
  size_t cap_u = 0, cap_rhs = 0, cap_x = 0, cap_act = 0, cap_res = 0, cap_dx = 0;
  // live kernel timing (CUDA events on the context stream)
  cudaEvent_t tev[4] = {};
  double t_asm = 0.0, t_rhs = 0.0;
  long n_asm = 0, n_rhs = 0;
  long nlaunch = 0;  // kernels launched outside the solver
  long lsqr_prev_launches = 0;  // launches of solver instances since replaced
};

namespace {
thread_local std::string g_free_err;
}
__attribute__((visibility("hidden"))) void agb_set_free_error(const std::string& msg) { g_free_err = msg; }
namespace {

int fail(agb_context* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_free_err = msg;
  return code;
}

// Host checks of a mesh before anything reaches the device (they need no
// context): every coordinate finite, connectivity inside [0, nnodes), and the
// normal of every element -- the cross product of its nodes 1-3, as
// CalElementNormal (lib_mesh.f90:716) takes it -- finite and of a length above
// 1e-12 of the product of the two edge lengths (nodes 1-3 neither coincident
// nor collinear to rounding), so that no element's normal divides by a zero
// length.  Elements e0..e1-1 index the nodes of xyz.  Returns the first defect,
// empty for a sound mesh.
std::string mesh_defect(int nnodes, const double* xyz, int e0, int e1, const int* etype, const int* con) {
  for (size_t i = 0; i < 3 * (size_t)nnodes; ++i)
    if (!std::isfinite(xyz[i])) return "node " + std::to_string(i / 3) + " has a coordinate that is not finite";
  for (int e = e0; e < e1; ++e) {
    if (etype[e] != AGB_TRI && etype[e] != AGB_QUAD) return "element " + std::to_string(e) + ": type must be 2 or 3";
    const int nno = etype[e] == AGB_TRI ? 3 : 4;
    const int* ce = con + 4 * (size_t)e;
    for (int k = 0; k < nno; ++k)
      if (ce[k] < 0 || ce[k] >= nnodes) return "element " + std::to_string(e) + ": connectivity out of range";
    const double* a = xyz + 3 * (size_t)ce[0];
    const double* b = xyz + 3 * (size_t)ce[1];
    const double* d = xyz + 3 * (size_t)ce[2];
    const double u0 = b[0] - a[0], u1 = b[1] - a[1], u2 = b[2] - a[2];
    const double v0 = d[0] - a[0], v1 = d[1] - a[1], v2 = d[2] - a[2];
    const double n0 = u1 * v2 - u2 * v1, n1 = u2 * v0 - u0 * v2, n2 = u0 * v1 - u1 * v0;
    const double len2 = n0 * n0 + n1 * n1 + n2 * n2;
    const double edges2 = (u0 * u0 + u1 * u1 + u2 * u2) * (v0 * v0 + v1 * v1 + v2 * v2);
    if (!(len2 > 1e-24 * edges2) || !std::isfinite(len2))
      return "element " + std::to_string(e) + " is degenerate: its nodes 1-3 span no normal";
  }
  return std::string();
}
#define CUDA_OR_FAIL(ctx, expr)                                                               \
  do {                                                                                        \
    cudaError_t e_ = (expr);                                                                  \
    if (e_ != cudaSuccess) return fail(ctx, AGB_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename P>
void dfree(P*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}
// device temporary owned by one scope: freed on every return unless released
template <typename P>
struct DevTemp {
  P* p = nullptr;
  DevTemp() = default;
  DevTemp(const DevTemp&) = delete;
  DevTemp& operator=(const DevTemp&) = delete;
  ~DevTemp() { reset(); }
  void reset() { dfree(p); }
  P* release() {
    P* q = p;
    p = nullptr;
    return q;
  }
};

// Wandzura-Xiao orbit expansion into barycentric points on the reference
// equilateral triangle (the construction of WandzuratXiaoBary,
// mod_trikotnik.f90:682-781): every orbit point and its images under the two
// maps of Table 1 of the paper, then barycentric coordinates w.r.t. the
// vertices (-1/2, sqrt3/2), (-1/2, -sqrt3/2), (1, 0).
void expand_rule(int itri, std::vector<double>& l, std::vector<double>& w) {
  const int o0 = agb_tables::kWxOrbitOffset[itri - 1], o1 = agb_tables::kWxOrbitOffset[itri];
  const double pi = 4.0 * std::atan(1.0);
  const double s = std::sin(2.0 / 3.0 * pi), c = std::cos(2.0 / 3.0 * pi);
  const double s4 = std::sin(4.0 / 3.0 * pi), c4 = std::cos(4.0 / 3.0 * pi);
  std::vector<double> X, Y;
  w.clear();
  auto images = [&](double x, double y, double cc, double ss, double wt) {
    const double xb = x * cc - y * ss, yb = -x * ss - y * cc;
    const double xc = xb * cc + yb * ss, yc = -xb * ss + yb * cc;
    X.insert(X.end(), {x, xb, xc});
    Y.insert(Y.end(), {y, yb, yc});
    w.insert(w.end(), {wt, wt, wt});
  };
  for (int j = o0; j < o1; ++j) {
    const auto& ob = agb_tables::kWxOrbits[j];
    if (ob.m == 1) {
      X.push_back(ob.x); Y.push_back(ob.y); w.push_back(ob.w);
    } else {
      images(ob.x, ob.y, c, s, ob.w);
      if (ob.m == 6) images(ob.x, -ob.y, c4, s4, ob.w);
    }
  }
  const int Q = (int)X.size();
  l.assign(3 * Q, 0.0);
  const double x1 = -0.5, y1 = 0.5 * std::sqrt(3.0), x2 = -0.5, y2 = -0.5 * std::sqrt(3.0), x3 = 1.0, y3 = 0.0;
  for (int i = 0; i < Q; ++i) {
    const double v0x = x2 - x1, v0y = y2 - y1, v1x = x3 - x1, v1y = y3 - y1, v2x = X[i] - x1, v2y = Y[i] - y1;
    const double d00 = v0x * v0x + v0y * v0y, d01 = v0x * v1x + v0y * v1y, d11 = v1x * v1x + v1y * v1y;
    const double d20 = v2x * v0x + v2y * v0y, d21 = v2x * v1x + v2y * v1y;
    const double den = d00 * d11 - d01 * d01;
    const double a = (d11 * d20 - d01 * d21) / den, b = (d00 * d21 - d01 * d20) / den;
    l[i] = a;
    l[Q + i] = b;
    l[2 * Q + i] = 1.0 - a - b;
  }
}

template <typename T>
cudaError_t ensure(T*& p, size_t& cap, size_t count) {
  if (count <= cap && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(count, 1) * sizeof(T));
  if (e == cudaSuccess) cap = count;
  return e;
}

void free_system(agb_context* c) {
  c->lsqr.packed = false;
  dfree(c->d_self6);
  c->lsqr.mf = nullptr;
  dfree(c->d_lu);
  c->lu_ready = false;
  dfree(c->d_rhsM);
  c->general = false;
  dfree(c->d_A);
  dfree(c->d_q);
  c->q_ready = false;
  dfree(c->d_pts);
  dfree(c->d_src);
  dfree(c->d_nrm);
  dfree(c->d_colscale);
  c->lsqr.release();
  c->assembled = false;
  c->prec = -1;
}
void free_problem(agb_context* c) {
  free_system(c);
  dfree(c->d_etype);
  dfree(c->d_con);
  dfree(c->d_wall);
  dfree(c->d_normMul);
  dfree(c->d_geom);
  dfree(c->d_rowact);  // sized by the element count of the problem
  dfree(c->rule.l);
  dfree(c->rule.w);
  c->gd.release();
  c->node_wall_in.clear();
  c->has_problem = false;
}

// Numbering of the subdomain (SetUpSubdomains lib_sdBem.f90:319, sdSetUpXandB
// lib_sdBem.f90:4, StokesBigSystemXB lib_Stokes.f90:1180) and the BC routing
// maps of sdSetUpSysMrhsM_CRS (lib_CRS.f90:148) / formUrow / formQrow
// (lib_StokesFull.f90:4,94).
void build_layout(agb_context* c) {
  GeneralLayout& L = c->gl;
  L = GeneralLayout();
  L.kind = c->kind;
  L.neq = c->neq;
  const int nw = (int)c->walls.size();
  // nodes of the subdomain, wall of the last element (in subdomain order) touching them
  std::vector<int> wallOf(c->nnodes, -1);
  for (int p = 0; p < c->ne; ++p) {
    const int e = c->elemList[p];
    const int nno = c->etype[e] == AGB_TRI ? 3 : 4;
    for (int k = 0; k < nno; ++k) wallOf[c->con[4 * e + k]] = c->wallIdx[p];
  }
  // walls the driver placed the nodes on (subdomain%BCidList after the BiC file's
  // EDGE / CORNER directives, agb_set_node_walls); ids checked against the walls there
  if (!c->node_wall_in.empty())
    for (int i = 0; i < c->nnodes; ++i) {
      if (wallOf[i] < 0 || c->node_wall_in[i] < 0) continue;
      for (int k = 0; k < nw; ++k)
        if (c->walls[k] == c->node_wall_in[i]) wallOf[i] = k;
    }
  L.posOfNode.assign(c->nnodes, -1);
  for (int i = 0; i < c->nnodes; ++i)
    if (wallOf[i] >= 0) {
      L.posOfNode[i] = (int)L.nodeList.size();
      L.nodeList.push_back(i);
      L.nodeWall.push_back(wallOf[i]);
    }
  L.nn = (int)L.nodeList.size();
  L.nq = c->ne;
  L.nsp = L.nn + L.nq;
  // node -> (element position, local index), ascending element position
  std::vector<std::vector<std::pair<int, int>>> adj(L.nn);
  for (int p = 0; p < c->ne; ++p) {
    const int e = c->elemList[p];
    const int nno = c->etype[e] == AGB_TRI ? 3 : 4;
    for (int k = 0; k < nno; ++k) adj[L.posOfNode[c->con[4 * e + k]]].push_back({p, k});
  }
  L.adj_ptr.assign(L.nn + 1, 0);
  for (int j = 0; j < L.nn; ++j) {
    L.adj_ptr[j + 1] = L.adj_ptr[j] + (int)adj[j].size();
    for (auto& pk : adj[j]) { L.adj_p.push_back(pk.first); L.adj_k.push_back(pk.second); }
  }
  auto bcOf = [&](int en, int widx) { return c->known[en * nw + widx]; };
  // per-equation numbering (1-based as the reference, -999 = not set)
  const int NS = -999;
  std::vector<std::vector<int>> col(L.neq, std::vector<int>(L.nn, NS)), qcol(L.neq, std::vector<int>(L.nq, NS));
  std::vector<int> nx(L.neq, 0), nb(L.neq, 0), neqn(L.neq, 0);
  for (int en = 0; en < L.neq; ++en) {
    for (int i = 0; i < L.nn; ++i) {
      const int bc = bcOf(en, L.nodeWall[i]);
      if (bc == AGB_BC_FUNCTION_) { nb[en]++; col[en][i] = nb[en]; }
      else if (bc == AGB_BC_FLUX_) { nx[en]++; col[en][i] = nx[en]; neqn[en]++; }
      else if (bc == AGB_BC_CONTACT_) { neqn[en]++; if (col[en][i] == NS) { nx[en]++; col[en][i] = nx[en]; } }
    }
    for (int p = 0; p < L.nq; ++p) {
      const int bc = bcOf(en, c->wallIdx[p]);
      if (bc == AGB_BC_FUNCTION_) { nx[en]++; qcol[en][p] = nx[en]; neqn[en]++; }
      else if (bc == AGB_BC_FLUX_) { nb[en]++; qcol[en][p] = nb[en]; }
      else if (bc == AGB_BC_CONTACT_) { neqn[en]++; if (qcol[en][p] == NS) { nx[en]++; qcol[en][p] = nx[en]; } }
    }
  }
  // offsets of the big system (equation blocks one after another)
  std::vector<int> offx(L.neq, 0), offb(L.neq, 0);
  for (int en = 1; en < L.neq; ++en) { offx[en] = offx[en - 1] + nx[en - 1]; offb[en] = offb[en - 1] + nb[en - 1]; }
  L.nx = L.nb = L.nrow = 0;
  for (int en = 0; en < L.neq; ++en) { L.nx += nx[en]; L.nb += nb[en]; L.nrow += neqn[en]; }
  // rows: u-source points first, then q-source points; equation-minor
  for (int i = 0; i < L.nn; ++i)
    for (int een = 0; een < L.neq; ++een) {
      const int bc = bcOf(een, L.nodeWall[i]);
      if (bc == AGB_BC_FLUX_ || bc == AGB_BC_CONTACT_) { L.row_src.push_back(i); L.row_een.push_back(een); }
    }
  for (int p = 0; p < L.nq; ++p)
    for (int een = 0; een < L.neq; ++een) {
      const int bc = bcOf(een, c->wallIdx[p]);
      if (bc == AGB_BC_FUNCTION_ || bc == AGB_BC_CONTACT_) { L.row_src.push_back(L.nn + p); L.row_een.push_back(een); }
    }
  const bool stk = (c->kind == AGB_STOKES);
  L.tmap_tgt.assign(L.neq * L.nn, 0); L.tmap_col.assign(L.neq * L.nn, 0); L.tmap_val.assign(L.neq * L.nn, 0.0);
  L.gmap_tgt.assign(L.neq * L.nq, 0); L.gmap_col.assign(L.neq * L.nq, 0); L.gmap_val.assign(L.neq * L.nq, 0.0);
  L.node_known.assign(L.neq * L.nn, 0); L.node_xcol.assign(L.neq * L.nn, -1); L.node_bcol.assign(L.neq * L.nn, -1);
  L.elem_known.assign(L.neq * L.nq, 0); L.elem_xcol.assign(L.neq * L.nq, -1); L.elem_bcol.assign(L.neq * L.nq, -1);
  for (int en = 0; en < L.neq; ++en) {
    for (int j = 0; j < L.nn; ++j) {
      const int bc = bcOf(en, L.nodeWall[j]), t = en * L.nn + j;
      if (bc == AGB_BC_FUNCTION_) {
        L.tmap_tgt[t] = 2; L.tmap_col[t] = col[en][j] - 1 + offb[en]; L.tmap_val[t] = 1.0;
        L.node_known[t] = 1; L.node_bcol[t] = L.tmap_col[t];
      } else if (bc == AGB_BC_FLUX_ || bc == AGB_BC_CONTACT_) {
        L.tmap_tgt[t] = 1; L.tmap_col[t] = col[en][j] - 1 + offx[en]; L.tmap_val[t] = stk ? -1.0 : 1.0;
        L.node_xcol[t] = L.tmap_col[t];
      }
    }
    for (int p = 0; p < L.nq; ++p) {
      const int bc = bcOf(en, c->wallIdx[p]), t = en * L.nq + p;
      const double sc = c->normMul[c->wallIdx[p]] / c->diff;
      if (bc == AGB_BC_FUNCTION_ || bc == AGB_BC_CONTACT_) {
        L.gmap_tgt[t] = 1; L.gmap_col[t] = qcol[en][p] - 1 + offx[en]; L.gmap_val[t] = stk ? -sc : sc;
        L.elem_xcol[t] = L.gmap_col[t];
      } else if (bc == AGB_BC_FLUX_) {
        L.gmap_tgt[t] = 2; L.gmap_col[t] = qcol[en][p] - 1 + offb[en]; L.gmap_val[t] = sc;
        L.elem_known[t] = 1; L.elem_bcol[t] = L.gmap_col[t];
      }
    }
  }
}

int check_ctx(agb_context* c, bool need_problem) {
  if (!c) return AGB_ERR_ARG;
  if (!c->has_mesh) return fail(c, AGB_ERR_STATE, "no mesh set (agb_set_mesh)");
  if (need_problem && !c->has_problem) return fail(c, AGB_ERR_STATE, "no problem set (agb_set_problem)");
  return AGB_OK;
}

// Upload u fields [nrhs][neq][nnodes]; mark active elements (any nonzero
// nodal value) and rows whose own element is active.
int stage_u(agb_context* c, int nrhs, const double* u, int* na_out) {
  const size_t cnt = (size_t)nrhs * c->neq * c->nnodes;
  CUDA_OR_FAIL(c, ensure(c->d_u, c->cap_u, cnt));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_u, u, cnt * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  std::vector<char> nz(c->nnodes, 0);
  for (size_t t = 0; t < cnt; ++t)
    if (u[t] != 0.0) nz[t % c->nnodes] = 1;
  std::vector<int> act;
  std::vector<unsigned char> rowact(c->ne, 0);
  for (int p = 0; p < c->ne; ++p) {
    const int e = c->elemList[p];
    const int nno = (c->etype[e] == AGB_TRI) ? 3 : 4;
    bool a = false;
    for (int k = 0; k < nno; ++k) a = a || nz[c->con[4 * e + k]];
    if (a) { act.push_back(p); rowact[p] = 1; }
  }
  CUDA_OR_FAIL(c, ensure(c->d_active, c->cap_act, std::max<size_t>(act.size(), (size_t)c->ne)));
  if (!c->d_rowact) CUDA_OR_FAIL(c, cudaMalloc(&c->d_rowact, std::max(c->ne, 1)));
  if (!act.empty())
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_active, act.data(), act.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_rowact, rowact.data(), c->ne, cudaMemcpyHostToDevice, c->stream));
  // the host vectors above are freed on return: make the copies complete
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  *na_out = (int)act.size();
  return AGB_OK;
}

// rhs on the device for nrhs fields already staged in d_u
int device_rhs(agb_context* c, int nrhs, int na) {
  CUDA_OR_FAIL(c, ensure(c->d_rhs, c->cap_rhs, (size_t)nrhs * c->m));
  if (c->kind == AGB_STOKES) {
    StokesRhsArgs a;
    a.ne = c->ne; a.Q = c->rule.Q; a.ldp = (c->ne + 31) / 32 * 32; a.k = nrhs; a.nnodes = c->nnodes;
    a.pts = c->d_pts;
    a.geom = c->d_geom; a.rule_l = c->rule.l; a.rule_w = c->rule.w; a.u = c->d_u;
    a.active = c->d_active; a.na = na; a.row_active = c->d_rowact; a.rhs = c->d_rhs;
    cudaEventRecord(c->tev[2], c->stream);
    if (c->prec != AGB_FP64) CUDA_OR_FAIL(c, launch_stokes_rhs<float>(a, c->stream));
    else CUDA_OR_FAIL(c, launch_stokes_rhs<double>(a, c->stream));
    cudaEventRecord(c->tev[3], c->stream);
    c->nlaunch += (na > 0) ? 3 : 1;
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->tev[2], c->tev[3]) == cudaSuccess) { c->t_rhs += ms; ++c->n_rhs; }
    (void)cudaGetLastError();
  } else {
    LaplaceArgs a;
    a.ne = c->ne; a.Q = c->rule.Q; a.k = nrhs; a.nnodes = c->nnodes; a.iqud = c->iqud;
    a.geom = c->d_geom; a.rule_l = c->rule.l; a.rule_w = c->rule.w; a.u = c->d_u; a.diff = c->diff;
    a.A = nullptr; a.lda = c->lda; a.rhs = c->d_rhs;
    cudaError_t e = launch_laplace_system(a, c->stream);
    c->nlaunch += 1;
    CUDA_OR_FAIL(c, e);
  }
  return AGB_OK;
}

int assemble_general(agb_context* c, int precision);
// relative LSQR tolerance of each refinement correction solve
constexpr double kRefineEps = 1.0e-2;
// restarts of BiCGSTAB on its true residual
constexpr int kBicgRestarts = 4;
__global__ void k_axpy(int64_t n, const double* __restrict__ d, double* __restrict__ x) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) x[t] += d[t];
}
// lsqr_precon's column scaling q of the assembled system, formed on first use
int ensure_q(agb_context* c) {
  if (c->q_ready) return AGB_OK;
  if (!c->lsqr.precon(c->d_A, c->d_q)) return fail(c, AGB_ERR_CUDA, c->lsqr.err);
  c->nlaunch += 2;
  // complete before any reader outside the context stream (agb_get_system copies on the default stream)
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  c->q_ready = true;
  return AGB_OK;
}
int do_solve(agb_context* c, int nrhs, double* d_x, int maxit, double eps, int refine, int* nit, int* istop,
             bool x0_zero) {
  if ((!c->lsqr.A && !c->lsqr.mf) || c->lsqr.k != nrhs) {
    if (!c->lsqr.setup(c->d_A, c->prec != AGB_FP64, c->m, c->n, c->lda, nrhs, c->stream))
      return fail(c, AGB_ERR_CUDA, "lsqr setup: " + c->lsqr.err);
  }
  c->lsqr.resid_fp64 = c->resid_fp64;
  std::vector<int> nt(nrhs, 0), is(nrhs, 0);
  if (c->solver == AGB_SOLVER_BICGSTAB || c->solver == AGB_SOLVER_HYBRID) {
    if (!c->lsqr.packed)
      return fail(c, AGB_ERR_UNSUPPORTED, "BiCGSTAB needs the packed mixed system (Stokes, velocity known on every "
                                          "wall, triangles, default integration, AGB_MIXED)");
    if (!c->lsqr.bicgstab(c->d_rhs, d_x, eps, maxit, nt.data(), is.data()))
      return fail(c, AGB_ERR_CUDA, "bicgstab: " + c->lsqr.err);
    // The recursive residual of the FP32 products can drift from the true one:
    // form r = b - A x over the stored matrix in float-float (or FP64)
    // arithmetic and, while a right-hand side's true residual is above eps
    // ||b||, solve A d = r by BiCGSTAB (to eps ||b|| / ||r||) and set x += d --
    // iterative refinement in extended precision around the mixed solver.
    {
      const int64_t m = c->m, n = c->n;
      std::vector<double> hb((size_t)nrhs * m), hr((size_t)nrhs * m);
      std::vector<double> bn(nrhs, 0.0);
      CUDA_OR_FAIL(c, cudaMemcpyAsync(hb.data(), c->d_rhs, hb.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                      c->stream));
      CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
      for (int r = 0; r < nrhs; ++r) {
        double ss = 0.0;
        for (int64_t i = 0; i < m; ++i) ss += hb[(size_t)r * m + i] * hb[(size_t)r * m + i];
        bn[r] = std::sqrt(ss);
      }
      CUDA_OR_FAIL(c, ensure(c->d_res, c->cap_res, (size_t)nrhs * m));
      CUDA_OR_FAIL(c, ensure(c->d_dx, c->cap_dx, (size_t)nrhs * n));
      for (int pass = 0; pass <= kBicgRestarts; ++pass) {
        if (!c->lsqr.residual(c->d_rhs, d_x, nullptr, c->d_res)) return fail(c, AGB_ERR_CUDA, "residual: " + c->lsqr.err);
        CUDA_OR_FAIL(c, cudaMemcpyAsync(hr.data(), c->d_res, hr.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                        c->stream));
        CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
        double worst = 0.0;
        bool again = false;
        for (int r = 0; r < nrhs; ++r) {
          double ss = 0.0;
          for (int64_t i = 0; i < m; ++i) ss += hr[(size_t)r * m + i] * hr[(size_t)r * m + i];
          const double rel = bn[r] > 0.0 ? std::sqrt(ss) / bn[r] : 0.0;
          if (rel > eps && (is[r] == 0 || is[r] == 4)) {  // claimed converged, or restarted
            again = true;
            worst = std::max(worst, rel);
            is[r] = 4;  // true residual above eps (until a restart brings it down)
          } else {
            if (is[r] == 4) is[r] = 0;
            // a right-hand side that is done gets no further correction
            CUDA_OR_FAIL(c, cudaMemsetAsync(c->d_res + (size_t)r * m, 0, (size_t)m * sizeof(double), c->stream));
          }
        }
        if (!again || pass == kBicgRestarts) break;
        std::vector<int> n2(nrhs, 0), i2(nrhs, 0);
        CUDA_OR_FAIL(c, cudaMemsetAsync(c->d_dx, 0, (size_t)nrhs * n * sizeof(double), c->stream));
        if (!c->lsqr.bicgstab(c->d_res, c->d_dx, eps / worst, maxit, n2.data(), i2.data()))
          return fail(c, AGB_ERR_CUDA, "bicgstab (restart): " + c->lsqr.err);
        k_axpy<<<(unsigned)(((int64_t)nrhs * n + 255) / 256), 256, 0, c->stream>>>((int64_t)nrhs * n, c->d_dx, d_x);
        CUDA_OR_FAIL(c, cudaGetLastError());
        c->nlaunch += 1;
        for (int r = 0; r < nrhs; ++r) {
          nt[r] += n2[r];
          if (is[r] == 4 && i2[r] >= 2) is[r] = i2[r];  // the restart broke down or diverged
        }
      }
    }
    bool all_converged = true;
    for (int r = 0; r < nrhs; ++r) all_converged = all_converged && is[r] == 0;
    if (c->solver == AGB_SOLVER_HYBRID && !all_converged) {
      // LSQR (the reference's lsqr_solve, default iteration limit) from a zero
      // start on every right-hand side
      std::vector<int> nl(nrhs, 0), il(nrhs, 0);
      if (int rc = ensure_q(c)) return rc;
      CUDA_OR_FAIL(c, cudaMemsetAsync(d_x, 0, (size_t)nrhs * c->n * sizeof(double), c->stream));
      if (!c->lsqr.solve(c->d_rhs, d_x, c->d_q, eps, 0, nl.data(), il.data(), nullptr, 8, true))
        return fail(c, AGB_ERR_CUDA, "lsqr after bicgstab: " + c->lsqr.err);
      for (int r = 0; r < nrhs; ++r) {
        nt[r] += nl[r];
        is[r] = 10 + il[r];
      }
    }
    for (int r = 0; r < nrhs; ++r) {
      if (nit) nit[r] = nt[r];
      if (istop) istop[r] = is[r];
    }
    return AGB_OK;
  }
  if (c->solver == AGB_SOLVER_GMRES) {
    if (!c->lsqr.packed)
      return fail(c, AGB_ERR_UNSUPPORTED, "GMRES needs the packed mixed system (Stokes, velocity known on every "
                                          "wall, triangles, default integration, AGB_MIXED)");
    if (!c->lsqr.gmres(c->d_rhs, d_x, nullptr, eps, maxit, c->gmres_restart, nt.data(), is.data()))
      return fail(c, AGB_ERR_CUDA, "gmres: " + c->lsqr.err);
    for (int r = 0; r < nrhs; ++r) {
      if (nit) nit[r] = nt[r];
      if (istop) istop[r] = is[r];
    }
    return AGB_OK;
  }
  c->lsqr.bj = false;
  if (c->solver == AGB_SOLVER_LSQR_BLOCK) {
    if (!c->lsqr.packed)
      return fail(c, AGB_ERR_UNSUPPORTED, "the block preconditioner needs the packed mixed system (Stokes, velocity "
                                          "known on every wall, triangles, default integration, AGB_MIXED)");
    if (!c->lsqr.block_precon()) return fail(c, AGB_ERR_NUMERIC, "lsqr: " + c->lsqr.err);
    c->lsqr.bj = true;
  }
  if (int rc = ensure_q(c)) return rc;
  if (!c->lsqr.solve(c->d_rhs, d_x, c->d_q, eps, maxit, nt.data(), is.data(), nullptr, 8, x0_zero))
    return fail(c, AGB_ERR_CUDA, "lsqr: " + c->lsqr.err);
  for (int r = 0; r < nrhs; ++r) {
    if (nit) nit[r] = nt[r];
    if (istop) istop[r] = is[r];
  }
  // iterative refinement: r = b - A x with FP64 accumulation over the stored
  // matrix, the correction A d = r by LSQR from zero to the relative tolerance
  // kRefineEps, x += d
  for (int pass = 1; pass <= refine; ++pass) {
    CUDA_OR_FAIL(c, ensure(c->d_res, c->cap_res, (size_t)nrhs * c->m));
    CUDA_OR_FAIL(c, ensure(c->d_dx, c->cap_dx, (size_t)nrhs * c->n));
    if (!c->lsqr.residual(c->d_rhs, d_x, c->d_q, c->d_res)) return fail(c, AGB_ERR_CUDA, "residual: " + c->lsqr.err);
    // the solve from zero adds its start vector to the result: it must be zero
    CUDA_OR_FAIL(c, cudaMemsetAsync(c->d_dx, 0, (size_t)nrhs * c->n * sizeof(double), c->stream));
    if (!c->lsqr.solve(c->d_res, c->d_dx, c->d_q, kRefineEps, maxit, nt.data(), is.data(), nullptr, 8, true))
      return fail(c, AGB_ERR_CUDA, "lsqr (refinement): " + c->lsqr.err);
    k_axpy<<<(unsigned)(((int64_t)nrhs * c->n + 255) / 256), 256, 0, c->stream>>>((int64_t)nrhs * c->n, c->d_dx, d_x);
    CUDA_OR_FAIL(c, cudaGetLastError());
    c->nlaunch += 1;
    for (int r = 0; r < nrhs; ++r) {
      if (nit) nit[r] += nt[r];
    }
  }
  return AGB_OK;
}
// All source rows on the GPU in FP64 (general_integrals), BC routing into a
// dense system (general_form), optional FP32 copy for the mixed solve, then the
// column scaling of lsqr_precon.
int assemble_general(agb_context* c, int precision) {
  const GeneralLayout& L = c->gl;
  if (L.nrow == 0 || L.nx == 0) return fail(c, AGB_ERR_ARG, "the boundary conditions leave no unknown");
  const int ncomp = (c->kind == AGB_STOKES) ? 9 : 1;
  // temporaries freed on every return (an allocation failure on a large body
  // must not leave gigabytes of integrals or system behind)
  DevTemp<double> T, G, err, sys;
  DevTemp<float> a32;
  CUDA_OR_FAIL(c, cudaMalloc(&T.p, (size_t)ncomp * L.nsp * L.nn * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&G.p, (size_t)ncomp * L.nsp * L.nq * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&err.p, (size_t)L.nsp * sizeof(double)));
  cudaError_t e = general_integrals(L, c->gd, c->d_geom, c->d_xyz, c->rule, c->iqud, c->iopt, T.p, G.p, err.p,
                                    c->stream);
  c->nlaunch += 2 * (int)((L.nsp + 65534) / 65535 + 1);
  if (e != cudaSuccess) return fail(c, AGB_ERR_CUDA, std::string("general integrals: ") + cudaGetErrorString(e));
  c->lda = ((int64_t)L.nx + 31) / 32 * 32;
  c->m = L.nrow;
  c->n = L.nx;
  CUDA_OR_FAIL(c, cudaMalloc(&sys.p, (size_t)L.nrow * c->lda * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMemsetAsync(sys.p, 0, (size_t)L.nrow * c->lda * sizeof(double), c->stream));
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_rhsM, (size_t)L.nrow * std::max(L.nb, 1) * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMemsetAsync(c->d_rhsM, 0, (size_t)L.nrow * std::max(L.nb, 1) * sizeof(double), c->stream));
  CUDA_OR_FAIL(c, general_form(L, c->gd, T.p, G.p, sys.p, c->lda, c->d_rhsM, c->stream));
  c->nlaunch += 1;
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  T.reset();
  G.reset();
  err.reset();
  c->prec = precision;
  if (precision == AGB_MIXED) {
    CUDA_OR_FAIL(c, cudaMalloc(&a32.p, (size_t)L.nrow * c->lda * sizeof(float)));
    CUDA_OR_FAIL(c, to_fp32(sys.p, a32.p, (int64_t)L.nrow * c->lda, c->stream));
    c->nlaunch += 1;
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    sys.reset();
    c->d_A = a32.release();
  } else {
    c->d_A = sys.release();
  }
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_q, c->lda * sizeof(double)));
  if (!c->lsqr.setup(c->d_A, precision == AGB_MIXED, c->m, c->n, c->lda, 1, c->stream)) return fail(c, AGB_ERR_CUDA, c->lsqr.err);
  if (!c->lsqr.precon(c->d_A, c->d_q)) return fail(c, AGB_ERR_CUDA, c->lsqr.err);
  c->q_ready = true;
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  c->general = true;
  c->assembled = true;
  return AGB_OK;
}

// Known vector b[r][nb] and warm start x[r][nx] from nodal u [r][neq][nnodes]
// and element q [r][neq][nelem] (global numbering); q may be NULL (zero).
void gather_fields(const agb_context* c, int nrhs, const double* u, const double* q, std::vector<double>& b,
                   std::vector<double>* x) {
  const GeneralLayout& L = c->gl;
  b.assign((size_t)nrhs * std::max(L.nb, 1), 0.0);
  if (x) x->assign((size_t)nrhs * L.nx, 0.0);
  for (int r = 0; r < nrhs; ++r)
    for (int en = 0; en < L.neq; ++en) {
      for (int j = 0; j < L.nn; ++j) {
        const int t = en * L.nn + j;
        const double v = u ? u[((size_t)r * L.neq + en) * c->nnodes + L.nodeList[j]] : 0.0;
        if (L.node_known[t]) b[(size_t)r * L.nb + L.node_bcol[t]] = v;
        else if (x && L.node_xcol[t] >= 0) (*x)[(size_t)r * L.nx + L.node_xcol[t]] = v;
      }
      for (int p = 0; p < L.nq; ++p) {
        const int t = en * L.nq + p;
        const double v = q ? q[((size_t)r * L.neq + en) * c->nelem + c->elemList[p]] : 0.0;
        if (L.elem_known[t]) b[(size_t)r * L.nb + L.elem_bcol[t]] = v;
        else if (x && L.elem_xcol[t] >= 0) (*x)[(size_t)r * L.nx + L.elem_xcol[t]] = v;
      }
    }
}

// rhs (device d_rhs, [r][m]) for the general system: rhsM * b (Stokes) or
// rhsM * (-b) (Laplace)
int general_rhs(agb_context* c, int nrhs, const std::vector<double>& b) {
  const GeneralLayout& L = c->gl;
  CUDA_OR_FAIL(c, ensure(c->d_rhs, c->cap_rhs, (size_t)nrhs * c->m));
  CUDA_OR_FAIL(c, ensure(c->d_b, c->cap_b, b.size()));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_b, b.data(), b.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, dense_rhs(L.nrow, std::max(L.nb, 1), c->d_rhsM, nrhs, c->d_b, c->kind == AGB_LAPLACE ? -1.0 : 1.0,
                            c->d_rhs, c->stream));
  c->nlaunch += 1;
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return AGB_OK;
}

}  // namespace

extern "C" {

const char* agb_version(void) { return "andromeda_gb300 0.1 (sm_103a)"; }

int agb_create(agb_context** out, int device) {
  if (!out) return AGB_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    g_free_err = std::string("no CUDA device: ") + cudaGetErrorString(e);
    return AGB_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) {
    g_free_err = "device index out of range";
    return AGB_ERR_ARG;
  }
  agb_context* c = new agb_context();
  c->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = upload_gauss_tables();
  if (e == cudaSuccess) e = upload_general_tables();
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->tev[i]);
  if (e != cudaSuccess) {
    g_free_err = std::string("agb_create: ") + cudaGetErrorString(e);
    delete c;
    return AGB_ERR_CUDA;
  }
  *out = c;
  return AGB_OK;
}

int agb_destroy(agb_context* c) {
  if (!c) return AGB_OK;
  cudaSetDevice(c->device);
  free_problem(c);
  dfree(c->d_xyz);
  dfree(c->d_u);
  dfree(c->d_rhs);
  dfree(c->d_x);
  dfree(c->d_res);
  dfree(c->d_dx);
  dfree(c->d_ft);
  dfree(c->d_active);
  dfree(c->d_rowact);
  for (int i = 0; i < 4; ++i)
    if (c->tev[i]) cudaEventDestroy(c->tev[i]);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return AGB_OK;
}

const char* agb_last_error(const agb_context* c) { return c ? c->err.c_str() : g_free_err.c_str(); }

int agb_set_mesh(agb_context* c, int nnodes, const double* xyz, int nelem, const int* etype, const int* con,
                 const int* bcid) {
  // the mesh is checked before the context, so that these checks run without a GPU
  if (nnodes <= 0 || nelem <= 0 || !xyz || !etype || !con || !bcid) return fail(c, AGB_ERR_ARG, "empty mesh");
  const std::string defect = mesh_defect(nnodes, xyz, 0, nelem, etype, con);
  if (!defect.empty()) return fail(c, AGB_ERR_ARG, "agb_set_mesh: " + defect);
  if (!c) return fail(c, AGB_ERR_ARG, "agb_set_mesh: no context");
  cudaSetDevice(c->device);
  free_problem(c);
  c->nnodes = nnodes;
  c->nelem = nelem;
  c->xyz.assign(xyz, xyz + 3 * (size_t)nnodes);
  c->etype.assign(etype, etype + nelem);
  c->con.assign(con, con + 4 * (size_t)nelem);
  c->bcid.assign(bcid, bcid + nelem);
  dfree(c->d_xyz);
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_xyz, c->xyz.size() * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_xyz, c->xyz.data(), c->xyz.size() * sizeof(double), cudaMemcpyHostToDevice,
                                  c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  c->has_mesh = true;
  return AGB_OK;
}

int agb_set_problem(agb_context* c, int kind, int nwalls, const int* walls, const double* normMul, double diff,
                    const int* known, int itri, int iqud) {
  int rc = check_ctx(c, false);
  if (rc) return rc;
  if (kind != AGB_LAPLACE && kind != AGB_STOKES) return fail(c, AGB_ERR_ARG, "kind must be AGB_LAPLACE or AGB_STOKES");
  if (nwalls <= 0 || !walls || !known) return fail(c, AGB_ERR_ARG, "no walls");
  if (itri < 1 || itri > 5) return fail(c, AGB_ERR_ARG, "itri must be 1..5");
  if (iqud < 1 || iqud > 8) return fail(c, AGB_ERR_ARG, "iqud must be 1..8");
  if (!(diff != 0.0) || !std::isfinite(diff)) return fail(c, AGB_ERR_ARG, "diff must be finite and nonzero");
  cudaSetDevice(c->device);
  free_problem(c);
  c->kind = kind;
  c->neq = (kind == AGB_STOKES) ? 3 : 1;
  c->walls.assign(walls, walls + nwalls);
  c->normMul.assign(nwalls, 1.0);
  if (normMul) c->normMul.assign(normMul, normMul + nwalls);
  c->diff = diff;
  c->known.assign(known, known + c->neq * nwalls);
  c->itri = itri;
  c->iqud = iqud;
  // subdomain element order: walls in list order, then element index (SetUpSubdomains)
  c->elemList.clear();
  c->wallIdx.clear();
  c->posOfElem.assign(c->nelem, -1);
  for (int k = 0; k < nwalls; ++k)
    for (int e = 0; e < c->nelem; ++e)
      if (c->bcid[e] == walls[k] && c->posOfElem[e] < 0) {
        c->posOfElem[e] = (int)c->elemList.size();
        c->elemList.push_back(e);
        c->wallIdx.push_back(k);
      }
  c->ne = (int)c->elemList.size();
  if (c->ne == 0) return fail(c, AGB_ERR_ARG, "no element belongs to the subdomain walls");
  c->all_dirichlet = true;
  for (int v : c->known)
    if (v != AGB_BC_FUNCTION) c->all_dirichlet = false;
  c->all_tri = true;
  for (int e : c->elemList)
    if (c->etype[e] != AGB_TRI) c->all_tri = false;
  // device copies in subdomain order
  std::vector<int> et(c->ne), cn(4 * (size_t)c->ne);
  for (int p = 0; p < c->ne; ++p) {
    const int e = c->elemList[p];
    et[p] = c->etype[e];
    for (int k = 0; k < 4; ++k) cn[4 * p + k] = c->con[4 * e + k];
  }
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_etype, c->ne * sizeof(int)));
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_con, 4 * (size_t)c->ne * sizeof(int)));
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_wall, c->ne * sizeof(int)));
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_normMul, nwalls * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_geom, c->ne * sizeof(ElemGeom)));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_etype, et.data(), c->ne * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_con, cn.data(), cn.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_wall, c->wallIdx.data(), c->ne * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_normMul, c->normMul.data(), nwalls * sizeof(double), cudaMemcpyHostToDevice,
                                  c->stream));
  CUDA_OR_FAIL(c, launch_geometry(c->ne, c->d_xyz, c->d_etype, c->d_con, c->d_wall, c->d_normMul, c->d_geom, c->stream));
  c->nlaunch += 1;
  std::vector<double> l, w;
  expand_rule(itri, l, w);
  c->rule.Q = (int)w.size();
  CUDA_OR_FAIL(c, cudaMalloc(&c->rule.l, l.size() * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&c->rule.w, w.size() * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->rule.l, l.data(), l.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->rule.w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  build_layout(c);
  CUDA_OR_FAIL(c, c->gd.upload(c->gl));
  c->m = c->gl.nrow;
  c->n = c->gl.nx;
  c->has_problem = true;
  return AGB_OK;
}

int agb_set_node_walls(agb_context* c, int nnodes, const int* node_wall) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (nnodes != c->nnodes) return fail(c, AGB_ERR_ARG, "agb_set_node_walls: nnodes differs from the mesh's");
  if (node_wall)
    for (int i = 0; i < nnodes; ++i) {
      const int w = node_wall[i];
      if (w < 0) continue;
      bool ok = false;
      for (int v : c->walls) ok = ok || v == w;
      if (!ok)
        return fail(c, AGB_ERR_ARG, "agb_set_node_walls: node " + std::to_string(i) + " placed on wall " +
                                        std::to_string(w) + ", which is not a wall of the problem");
    }
  cudaSetDevice(c->device);
  free_system(c);  // the numbering changes: any assembled system is stale
  if (node_wall) c->node_wall_in.assign(node_wall, node_wall + nnodes);
  else c->node_wall_in.clear();
  build_layout(c);
  CUDA_OR_FAIL(c, c->gd.upload(c->gl));
  c->m = c->gl.nrow;
  c->n = c->gl.nx;
  return AGB_OK;
}

int agb_set_integration(agb_context* c, int sing_mode, int rec_depth, double near_eta, int near_depth) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (sing_mode != 0 && sing_mode != 1) return fail(c, AGB_ERR_ARG, "sing_mode must be 0 (analytic) or 1 (recursive)");
  if (rec_depth < 0 || rec_depth > 30) return fail(c, AGB_ERR_ARG, "rec_depth must be 0..30");
  if (!(near_eta >= 0.0) || !std::isfinite(near_eta)) return fail(c, AGB_ERR_ARG, "near_eta must be finite and >= 0");
  if (near_depth < 0 || near_depth > 20) return fail(c, AGB_ERR_ARG, "near_depth must be 0..20");
  c->iopt.sing = sing_mode;
  c->iopt.rdepth = rec_depth;
  c->iopt.near_eta = near_eta;
  c->iopt.near_depth = near_depth;
  c->assembled = false;
  return AGB_OK;
}

int agb_set_solver(agb_context* c, int solver) {
  if (!c) return fail(c, AGB_ERR_ARG, "agb_set_solver: no context");
  if (solver != AGB_SOLVER_LSQR && solver != AGB_SOLVER_BICGSTAB && solver != AGB_SOLVER_HYBRID &&
      solver != AGB_SOLVER_LSQR_BLOCK && solver != AGB_SOLVER_GMRES)
    return fail(c, AGB_ERR_ARG,
                "solver must be AGB_SOLVER_LSQR, AGB_SOLVER_BICGSTAB, AGB_SOLVER_HYBRID, AGB_SOLVER_LSQR_BLOCK or "
                "AGB_SOLVER_GMRES");
  c->solver = solver;
  return AGB_OK;
}

int agb_set_residual_mode(agb_context* c, int mode) {
  if (!c) return fail(c, AGB_ERR_ARG, "agb_set_residual_mode: no context");
  if (mode != 0 && mode != 1) return fail(c, AGB_ERR_ARG, "agb_set_residual_mode: mode must be 0 or 1");
  c->resid_fp64 = mode == 1;
  c->lsqr.resid_fp64 = c->resid_fp64;
  return AGB_OK;
}

int agb_set_gmres_restart(agb_context* c, int restart) {
  if (!c) return fail(c, AGB_ERR_ARG, "agb_set_gmres_restart: no context");
  if (restart < 1 || restart > 512) return fail(c, AGB_ERR_ARG, "agb_set_gmres_restart: restart must be 1..512");
  c->gmres_restart = restart;
  return AGB_OK;
}

int agb_get_geometry(agb_context* c, double* normal, double* area, double* centroid) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  cudaSetDevice(c->device);
  std::vector<ElemGeom> g(c->ne);
  CUDA_OR_FAIL(c, cudaMemcpy(g.data(), c->d_geom, c->ne * sizeof(ElemGeom), cudaMemcpyDeviceToHost));
  if (normal) std::fill(normal, normal + 3 * (size_t)c->nelem, 0.0);
  if (area) std::fill(area, area + c->nelem, 0.0);
  if (centroid) std::fill(centroid, centroid + 3 * (size_t)c->nelem, 0.0);
  for (int p = 0; p < c->ne; ++p) {
    const int e = c->elemList[p];
    for (int i = 0; i < 3; ++i) {
      if (normal) normal[3 * e + i] = g[p].n[i];
      if (centroid) centroid[3 * e + i] = g[p].c[i];
    }
    if (area) area[e] = g[p].area;
  }
  return AGB_OK;
}

int agb_system_size(agb_context* c, int* m, int* n) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (m) *m = c->m;
  if (n) *n = c->n;
  return AGB_OK;
}

int agb_assemble(agb_context* c, int precision) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (precision != AGB_FP64 && precision != AGB_MIXED && precision != AGB_MATRIX_FREE)
    return fail(c, AGB_ERR_ARG, "precision must be AGB_FP64, AGB_MIXED or AGB_MATRIX_FREE");
  const bool fast = c->all_dirichlet && c->iopt.is_default() &&
                    ((c->kind == AGB_LAPLACE && precision == AGB_FP64) || (c->kind == AGB_STOKES && c->all_tri));
  cudaSetDevice(c->device);
  free_system(c);
  if (precision == AGB_MATRIX_FREE) {
    if (!(fast && c->kind == AGB_STOKES))
      return fail(c, AGB_ERR_UNSUPPORTED, "the matrix-free operator needs a Stokes problem with velocity known on "
                                          "every wall, triangles and the default integration");
    c->prec = precision;
    c->lda = ((int64_t)c->n + 31) / 32 * 32;
    const int ldp = (c->ne + 31) / 32 * 32;
    const int Q = c->rule.Q;
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_q, c->lda * sizeof(double)));
    CUDA_OR_FAIL(c, cudaMemsetAsync(c->d_q, 0, c->lda * sizeof(double), c->stream));
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_pts, (size_t)Q * ldp * sizeof(QPt<float>)));
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_src, 3 * (size_t)ldp * sizeof(float)));
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_nrm, 3 * (size_t)ldp * sizeof(float)));
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_colscale, (size_t)ldp * sizeof(float)));
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_self6, (size_t)c->ne * 6 * sizeof(float)));
    std::vector<float> csf(ldp, 0.f);
    for (int p = 0; p < c->ne; ++p) csf[p] = (float)(-c->normMul[c->wallIdx[p]] / c->diff);
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_colscale, csf.data(), ldp * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CUDA_OR_FAIL(c, launch_expand_points<float>(c->ne, ldp, c->d_geom, c->rule, (QPt<float>*)c->d_pts,
                                                (float*)c->d_src, (float*)c->d_nrm, c->stream));
    c->mfop.ne = c->ne; c->mfop.Q = Q; c->mfop.ldp = ldp;
    c->mfop.pts = (const QPt<float>*)c->d_pts; c->mfop.src = (const float*)c->d_src;
    c->mfop.colscale = (const float*)c->d_colscale; c->mfop.self6 = c->d_self6;
    CUDA_OR_FAIL(c, mf_setup_self(c->mfop, c->d_geom, c->diff, c->stream));
    c->nlaunch += 2;
    c->lsqr.mf = &c->mfop;
    if (!c->lsqr.setup(nullptr, true, c->m, c->n, c->lda, 1, c->stream)) return fail(c, AGB_ERR_CUDA, c->lsqr.err);
    cudaEventRecord(c->tev[0], c->stream);
    if (!c->lsqr.precon(nullptr, c->d_q)) return fail(c, AGB_ERR_CUDA, c->lsqr.err);
    c->q_ready = true;
    cudaEventRecord(c->tev[1], c->stream);
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->tev[0], c->tev[1]) == cudaSuccess) { c->t_asm += ms; ++c->n_asm; }
    (void)cudaGetLastError();
    c->assembled = true;
    return AGB_OK;
  }
  if (!fast) return assemble_general(c, precision);
  c->prec = precision;
  const bool f32 = (precision == AGB_MIXED);
  const size_t tsz = f32 ? sizeof(float) : sizeof(double);
  c->lda = ((int64_t)c->n + 31) / 32 * 32;
  const bool packedA = (c->kind == AGB_STOKES && f32);  // mixed Stokes: packed symmetric blocks (allocated below)
  if (!packedA) {
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_A, (size_t)c->m * c->lda * tsz));
    if (c->lda > c->n)
      CUDA_OR_FAIL(c, cudaMemset2DAsync((char*)c->d_A + c->n * tsz, c->lda * tsz, 0, (c->lda - c->n) * tsz, c->m,
                                        c->stream));
  }
  CUDA_OR_FAIL(c, cudaMalloc(&c->d_q, c->lda * sizeof(double)));
  if (c->kind == AGB_STOKES) {
    const int ldp = (c->ne + 31) / 32 * 32;
    const int Q = c->rule.Q;
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_pts, (size_t)Q * ldp * (f32 ? sizeof(QPt<float>) : sizeof(QPt<double>))));
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_src, 3 * (size_t)ldp * tsz));
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_nrm, 3 * (size_t)ldp * tsz));
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_colscale, (size_t)ldp * tsz));
    std::vector<double> cs(ldp, 0.0);
    for (int p = 0; p < c->ne; ++p) cs[p] = -c->normMul[c->wallIdx[p]] / c->diff;
    if (f32) {
      // packed symmetric blocks (pk_idx layout, 2/3 of the bytes of the m x lda matrix)
      const int pldp = (c->ne + 63) / 64 * 64;
      CUDA_OR_FAIL(c, cudaMalloc(&c->d_A, (size_t)c->ne * 6 * pldp * sizeof(float)));
      CUDA_OR_FAIL(c, cudaMemsetAsync(c->d_A, 0, (size_t)c->ne * 6 * pldp * sizeof(float), c->stream));
      std::vector<float> csf(cs.begin(), cs.end());
      CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_colscale, csf.data(), ldp * sizeof(float), cudaMemcpyHostToDevice, c->stream));
      CUDA_OR_FAIL(c, launch_expand_points<float>(c->ne, ldp, c->d_geom, c->rule, (QPt<float>*)c->d_pts,
                                                  (float*)c->d_src, (float*)c->d_nrm, c->stream));
      cudaEventRecord(c->tev[0], c->stream);
      CUDA_OR_FAIL(c, launch_stokes_G_packed(c->ne, Q, ldp, pldp, (const QPt<float>*)c->d_pts,
                                             (const float*)c->d_src, (const float*)c->d_colscale, (float*)c->d_A,
                                             c->stream));
      cudaEventRecord(c->tev[1], c->stream);
      CUDA_OR_FAIL(c, launch_stokes_self_packed(c->ne, pldp, c->d_geom, c->diff, (float*)c->d_A, c->stream));
      c->lsqr.packed = true;
      c->lsqr.pk_ne = c->ne;
      c->lsqr.pk_ldp = pldp;
      c->nlaunch += 3;  // expand, single layer, self blocks
    } else {
      CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_colscale, cs.data(), ldp * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      CUDA_OR_FAIL(c, launch_expand_points<double>(c->ne, ldp, c->d_geom, c->rule, (QPt<double>*)c->d_pts,
                                                   (double*)c->d_src, (double*)c->d_nrm, c->stream));
      cudaEventRecord(c->tev[0], c->stream);
      CUDA_OR_FAIL(c, launch_stokes_G<double>(c->ne, Q, ldp, (const QPt<double>*)c->d_pts, (const double*)c->d_src,
                                              (const double*)c->d_colscale, (double*)c->d_A, c->lda, c->stream));
      cudaEventRecord(c->tev[1], c->stream);
      CUDA_OR_FAIL(c, launch_stokes_self<double>(c->ne, c->d_geom, c->diff, (double*)c->d_A, c->lda, c->stream));
      c->nlaunch += 3;
    }
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->tev[0], c->tev[1]) == cudaSuccess) { c->t_asm += ms; ++c->n_asm; }
    (void)cudaGetLastError();
  } else {
    LaplaceArgs a;
    a.ne = c->ne; a.Q = c->rule.Q; a.k = 0; a.nnodes = c->nnodes; a.iqud = c->iqud;
    a.geom = c->d_geom; a.rule_l = c->rule.l; a.rule_w = c->rule.w; a.u = nullptr; a.diff = c->diff;
    a.A = (double*)c->d_A; a.lda = c->lda; a.rhs = nullptr;
    CUDA_OR_FAIL(c, launch_laplace_system(a, c->stream));
    c->nlaunch += 1;
  }
  // column scaling of lsqr_precon: the packed system keeps its matrix unscaled
  // (the sweeps apply q), so q is formed when a solver first needs it (the
  // LSQR paths; GMRES and BiCGSTAB never use it); any other system is scaled
  // in place here
  if (!c->lsqr.setup(c->d_A, f32, c->m, c->n, c->lda, 1, c->stream)) return fail(c, AGB_ERR_CUDA, c->lsqr.err);
  c->q_ready = false;
  if (!c->lsqr.packed) {
    if (!c->lsqr.precon(c->d_A, c->d_q)) return fail(c, AGB_ERR_CUDA, c->lsqr.err);
    c->q_ready = true;
  }
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  c->assembled = true;
  return AGB_OK;
}

int agb_get_system(agb_context* c, int scaled, double* A, double* q) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (!c->assembled) return fail(c, AGB_ERR_STATE, "system not assembled");
  if (c->prec == AGB_MATRIX_FREE && A) return fail(c, AGB_ERR_UNSUPPORTED, "the matrix-free system is not stored");
  cudaSetDevice(c->device);
  std::vector<double> qh(c->lda);
  if (int rc = ensure_q(c)) return rc;
  CUDA_OR_FAIL(c, cudaMemcpy(qh.data(), c->d_q, c->lda * sizeof(double), cudaMemcpyDeviceToHost));
  if (q) std::copy(qh.begin(), qh.begin() + c->n, q);
  if (A && c->lsqr.packed) {  // expand the symmetric blocks: A[3i+a][b ne + j] = Ap[pk_idx(i, sym(a,b), j)]
    const int ne = c->lsqr.pk_ne, ldp = c->lsqr.pk_ldp;
    static const int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    std::vector<float> row((size_t)6 * ldp);
    for (int i = 0; i < ne; ++i) {
      CUDA_OR_FAIL(c, cudaMemcpy(row.data(), (float*)c->d_A + (size_t)i * 6 * ldp, row.size() * sizeof(float),
                                 cudaMemcpyDeviceToHost));
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          for (int j = 0; j < ne; ++j) {
            const double v = (double)row[pk_idx(0, sym[a][b], j, ldp)];
            const size_t col = (size_t)b * ne + j;
            A[(size_t)(3 * i + a) * c->n + col] = scaled ? v * qh[col] : v;
          }
    }
    return AGB_OK;
  }
  if (A) {
    const bool f32 = c->prec == AGB_MIXED;
    std::vector<char> buf((size_t)c->lda * (f32 ? 4 : 8));
    for (int r = 0; r < c->m; ++r) {
      CUDA_OR_FAIL(c, cudaMemcpy(buf.data(), (char*)c->d_A + (size_t)r * c->lda * (f32 ? 4 : 8), buf.size(),
                                 cudaMemcpyDeviceToHost));
      for (int j = 0; j < c->n; ++j) {
        double v = f32 ? (double)((float*)buf.data())[j] : ((double*)buf.data())[j];
        A[(size_t)r * c->n + j] = scaled ? v : v / qh[j];
      }
    }
  }
  return AGB_OK;
}

int agb_rhs(agb_context* c, int nrhs, const double* u, double* rhs) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (!c->assembled) return fail(c, AGB_ERR_STATE, "system not assembled");
  if (nrhs < 1 || nrhs > AGB_MAX_RHS || !u) return fail(c, AGB_ERR_ARG, "nrhs must be 1..8");
  cudaSetDevice(c->device);
  if (c->general) {
    std::vector<double> b;
    gather_fields(c, nrhs, u, nullptr, b, nullptr);
    if ((rc = general_rhs(c, nrhs, b))) return rc;
  } else {
    int na = 0;
    if ((rc = stage_u(c, nrhs, u, &na))) return rc;
    if ((rc = device_rhs(c, nrhs, na))) return rc;
  }
  if (rhs)
    CUDA_OR_FAIL(c, cudaMemcpyAsync(rhs, c->d_rhs, (size_t)nrhs * c->m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return AGB_OK;
}

int agb_solve(agb_context* c, int nrhs, const double* u, double* x, int maxit, double eps, int refine, int* nit,
              int* istop) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (!c->assembled) return fail(c, AGB_ERR_STATE, "system not assembled");
  if (nrhs < 1 || nrhs > AGB_MAX_RHS || !u || !x) return fail(c, AGB_ERR_ARG, "nrhs must be 1..8");
  if (maxit < 0 || !(eps >= 0.0) || refine < 0) return fail(c, AGB_ERR_ARG, "bad solver parameters");
  cudaSetDevice(c->device);
  if (c->general) {
    std::vector<double> b;
    gather_fields(c, nrhs, u, nullptr, b, nullptr);
    if ((rc = general_rhs(c, nrhs, b))) return rc;
  } else {
    int na = 0;
    if ((rc = stage_u(c, nrhs, u, &na))) return rc;
    if ((rc = device_rhs(c, nrhs, na))) return rc;
  }
  CUDA_OR_FAIL(c, ensure(c->d_x, c->cap_x, (size_t)nrhs * c->n));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_x, x, (size_t)nrhs * c->n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  bool zero = true;
  for (size_t t = 0; t < (size_t)nrhs * c->n && zero; ++t) zero = (x[t] == 0.0);
  if ((rc = do_solve(c, nrhs, c->d_x, maxit, eps, refine, nit, istop, zero))) return rc;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(x, c->d_x, (size_t)nrhs * c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return AGB_OK;
}

int agb_force_torque(agb_context* c, int nrhs, const double* x, int wall, double* ft) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (c->kind != AGB_STOKES) return fail(c, AGB_ERR_UNSUPPORTED, "force/torque needs a Stokes problem");
  if (nrhs < 1 || nrhs > AGB_MAX_RHS || !x || !ft) return fail(c, AGB_ERR_ARG, "bad arguments");
  int widx = -1;
  for (size_t k = 0; k < c->walls.size(); ++k)
    if (c->walls[k] == wall) widx = (int)k;
  if (widx < 0) return fail(c, AGB_ERR_ARG, "wall not in the subdomain");
  cudaSetDevice(c->device);
  CUDA_OR_FAIL(c, ensure(c->d_x, c->cap_x, (size_t)nrhs * c->n));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_x, x, (size_t)nrhs * c->n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (!c->d_ft) CUDA_OR_FAIL(c, cudaMalloc(&c->d_ft, 6 * AGB_MAX_RHS * sizeof(double)));
  CUDA_OR_FAIL(c, launch_force_torque(c->ne, nrhs, c->d_geom, c->d_x, widx, c->d_ft, c->stream));
  c->nlaunch += 1;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(ft, c->d_ft, 6 * (size_t)nrhs * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return AGB_OK;
}

// Right-hand sides of the six rigid motions of the container (e_x, e_y, e_z
// translations, then e_a x r rotations), particle at rest: the outer-wall
// velocities of StokesInlet3sidesForceCRS / ...TorqueOmegaCRS
// (lib_particle.f90:341,176), into c->d_rhs [6][m].
static int resistance_rhs(agb_context* c, int oidx) {
  int rc;
  const int k = 6;
  std::vector<double> u((size_t)k * 3 * c->nnodes, 0.0);
  std::vector<char> onOuter(c->nnodes, 0);
  for (int p = 0; p < c->ne; ++p)
    if (c->wallIdx[p] == oidx) {
      const int e = c->elemList[p];
      const int nno = (c->etype[e] == AGB_TRI) ? 3 : 4;
      for (int kk = 0; kk < nno; ++kk) onOuter[c->con[4 * e + kk]] = 1;
    }
  for (int i = 0; i < c->nnodes; ++i) {
    if (!onOuter[i]) continue;
    const double* x = &c->xyz[3 * i];
    for (int a = 0; a < 3; ++a) u[((size_t)a * 3 + a) * c->nnodes + i] = 1.0;
    // e_a x r
    const double w[3][3] = {{0, -x[2], x[1]}, {x[2], 0, -x[0]}, {-x[1], x[0], 0}};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) u[((size_t)(3 + a) * 3 + b) * c->nnodes + i] = w[a][b];
  }
  if (c->general) {
    std::vector<double> b;
    gather_fields(c, k, u.data(), nullptr, b, nullptr);
    if ((rc = general_rhs(c, k, b))) return rc;
  } else {
    int na = 0;
    if ((rc = stage_u(c, k, u.data(), &na))) return rc;
    if ((rc = device_rhs(c, k, na))) return rc;
  }
  return AGB_OK;
}

int agb_resistance_tensor(agb_context* c, int precision, int particle_wall, int outer_wall, int maxit, double eps,
                          int refine, double* R, int* nit, int* istop, double* times_ms) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (c->kind != AGB_STOKES) return fail(c, AGB_ERR_UNSUPPORTED, "resistance tensor needs a Stokes problem");
  if (!c->all_dirichlet) return fail(c, AGB_ERR_UNSUPPORTED, "resistance tensor needs velocity known on every wall");
  if (!R) return fail(c, AGB_ERR_ARG, "R is NULL");
  int pidx = -1, oidx = -1;
  for (size_t k = 0; k < c->walls.size(); ++k) {
    if (c->walls[k] == particle_wall) pidx = (int)k;
    if (c->walls[k] == outer_wall) oidx = (int)k;
  }
  if (pidx < 0 || oidx < 0) return fail(c, AGB_ERR_ARG, "particle/outer wall not in the subdomain");
  cudaSetDevice(c->device);
  using clk = std::chrono::steady_clock;
  auto ms = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
  cudaEvent_t d0 = nullptr, d1 = nullptr;
  CUDA_OR_FAIL(c, cudaEventCreate(&d0));
  CUDA_OR_FAIL(c, cudaEventCreate(&d1));
  CUDA_OR_FAIL(c, cudaEventRecord(d0, c->stream));
  auto t0 = clk::now();
  if ((rc = agb_assemble(c, precision))) return rc;
  auto t1 = clk::now();
  const int k = 6;
  if ((rc = resistance_rhs(c, oidx))) return rc;
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  auto t2 = clk::now();
  CUDA_OR_FAIL(c, ensure(c->d_x, c->cap_x, (size_t)k * c->n));
  CUDA_OR_FAIL(c, cudaMemsetAsync(c->d_x, 0, (size_t)k * c->n * sizeof(double), c->stream));
  std::vector<int> nt(k), is(k);
  if ((rc = do_solve(c, k, c->d_x, maxit, eps, refine, nt.data(), is.data(), true))) return rc;
  auto t3 = clk::now();
  if (!c->d_ft) CUDA_OR_FAIL(c, cudaMalloc(&c->d_ft, 6 * AGB_MAX_RHS * sizeof(double)));
  CUDA_OR_FAIL(c, launch_force_torque(c->ne, k, c->d_geom, c->d_x, pidx, c->d_ft, c->stream));
  c->nlaunch += 1;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(R, c->d_ft, 36 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaEventRecord(d1, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  auto t4 = clk::now();
  float dev_ms = 0.f;
  CUDA_OR_FAIL(c, cudaEventElapsedTime(&dev_ms, d0, d1));
  cudaEventDestroy(d0);
  cudaEventDestroy(d1);
  for (int r = 0; r < k; ++r) {
    if (nit) nit[r] = nt[r];
    if (istop) istop[r] = is[r];
  }
  if (times_ms) {
    times_ms[0] = ms(t0, t1);
    times_ms[1] = ms(t1, t2);
    times_ms[2] = ms(t2, t3);
    times_ms[3] = ms(t3, t4);
    times_ms[4] = ms(t0, t4);
    times_ms[5] = dev_ms;
  }
  return AGB_OK;
}

// The CRS is checked on the host before it reaches the GPU: 1-based,
// nondecreasing row starts ia(1) = 1, ia(m+1) = nnz+1, 1 <= ja <= n.
static bool crs_valid(int m, int n, int64_t nnz, const int64_t* ia, const int* ja) {
  if (ia[0] != 1 || ia[m] != nnz + 1) return false;
  for (int r = 0; r < m; ++r)
    if (ia[r + 1] < ia[r]) return false;
  for (int64_t t = 0; t < nnz; ++t)
    if (ja[t] < 1 || ja[t] > n) return false;
  return true;
}

int agb_lsqr_precon(int m, int n, int64_t nnz, double* q, const int64_t* ia, const int* ja, double* a) {
  if (m <= 0 || n <= 0 || nnz < 0 || !q || !ia || !ja || !a) return fail(nullptr, AGB_ERR_ARG, "bad CRS arguments");
  if (!crs_valid(m, n, nnz, ia, ja)) return fail(nullptr, AGB_ERR_ARG, "malformed CRS (ia/ja out of range)");
  std::string err;
  if (!crs_lsqr_precon(m, n, nnz, q, ia, ja, a, err)) return fail(nullptr, AGB_ERR_CUDA, err);
  return AGB_OK;
}

int agb_lsqr_solve(int m, int n, int64_t nnz, int* maxit, double eps, int* nit, int* ierr, const double* q,
                   const int64_t* ia, const int* ja, double* a, const double* b, double* x) {
  if (m <= 0 || n <= 0 || nnz < 0 || !maxit || !nit || !ierr || !q || !ia || !ja || !a || !b || !x)
    return fail(nullptr, AGB_ERR_ARG, "bad CRS arguments");
  if (!crs_valid(m, n, nnz, ia, ja)) return fail(nullptr, AGB_ERR_ARG, "malformed CRS (ia/ja out of range)");
  std::string err;
  if (!crs_lsqr_solve(m, n, nnz, *maxit, eps, *nit, *ierr, q, ia, ja, a, b, x, err)) return fail(nullptr, AGB_ERR_CUDA, err);
  return AGB_OK;
}

int agb_kernel_times(agb_context* c, int reset, double* out) {
  if (!c) return AGB_ERR_ARG;
  if (out) {
    out[0] = c->lsqr.t_av;  out[1] = (double)c->lsqr.n_av;
    out[2] = c->lsqr.t_atu; out[3] = (double)c->lsqr.n_atu;
    out[4] = c->t_asm;      out[5] = (double)c->n_asm;
    out[6] = c->t_rhs;      out[7] = (double)c->n_rhs;
    out[8] = (double)(c->nlaunch + c->lsqr.launches + c->lsqr_prev_launches);
    out[9] = 0.0;
  }
  if (reset) {
    c->lsqr.t_av = c->lsqr.t_atu = 0.0;
    c->lsqr.n_av = c->lsqr.n_atu = 0;
    c->t_asm = c->t_rhs = 0.0;
    c->n_asm = c->n_rhs = 0;
    c->nlaunch = 0;
    c->lsqr.launches = 0;
    c->lsqr_prev_launches = 0;
  }
  return AGB_OK;
}

// Post-processing of a solved field: the surface pressure and the values at
// points inside the domain (FP64, the element integrals of the general path).
namespace {
struct PostBufs {
  double *u = nullptr, *q = nullptr, *pts = nullptr, *out = nullptr, *err = nullptr;
  ~PostBufs() { cudaFree(u); cudaFree(q); cudaFree(pts); cudaFree(out); cudaFree(err); }
};
// q[comp][nelem] (mesh order) -> [comp][ne] (subdomain order), uploaded with u
int post_upload(agb_context* c, PostBufs& B, const double* u, const double* q) {
  const int nc = c->neq;
  std::vector<double> qs((size_t)nc * c->ne);
  for (int comp = 0; comp < nc; ++comp)
    for (int pos = 0; pos < c->ne; ++pos) qs[(size_t)comp * c->ne + pos] = q[(size_t)comp * c->nelem + c->elemList[pos]];
  CUDA_OR_FAIL(c, cudaMalloc(&B.u, (size_t)nc * c->nnodes * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&B.q, qs.size() * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMemcpy(B.u, u, (size_t)nc * c->nnodes * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_OR_FAIL(c, cudaMemcpy(B.q, qs.data(), qs.size() * sizeof(double), cudaMemcpyHostToDevice));
  return AGB_OK;
}
double osem_pi() { return (double)std::atan(1.0f) * 4.0 * 8.0; }  // the reference's ATAN(1.0) is single precision
}  // namespace

int agb_surface_pressure(agb_context* c, const double* u, const double* q, double* p) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (!u || !q || !p) return fail(c, AGB_ERR_ARG, "agb_surface_pressure: missing arrays");
  if (c->kind != AGB_STOKES) return fail(c, AGB_ERR_UNSUPPORTED, "agb_surface_pressure: Stokes problems only");
  cudaSetDevice(c->device);
  PostBufs B;
  if ((rc = post_upload(c, B, u, q))) return rc;
  CUDA_OR_FAIL(c, cudaMalloc(&B.out, (size_t)c->ne * sizeof(double)));
  CUDA_OR_FAIL(c, surface_pressure(c->ne, c->d_geom, c->rule, c->iqud, c->iopt, B.u, c->nnodes, B.q, c->diff,
                                   osem_pi(), B.out, c->stream));
  c->nlaunch += 1;
  std::vector<double> ps(c->ne);
  CUDA_OR_FAIL(c, cudaMemcpyAsync(ps.data(), B.out, ps.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  std::fill(p, p + c->nelem, 0.0);
  for (int pos = 0; pos < c->ne; ++pos) p[c->elemList[pos]] = ps[pos];
  return AGB_OK;
}

int agb_domain_values(agb_context* c, int npts, const double* pts, const double* u, const double* q, double* out,
                      double* err) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (npts < 0 || (npts > 0 && (!pts || !u || !q || !out || !err)))
    return fail(c, AGB_ERR_ARG, "agb_domain_values: missing arrays");
  if (npts == 0) return AGB_OK;
  for (int64_t i = 0; i < 3 * (int64_t)npts; ++i)
    if (!std::isfinite(pts[i])) return fail(c, AGB_ERR_ARG, "agb_domain_values: a point coordinate is not finite");
  cudaSetDevice(c->device);
  PostBufs B;
  if ((rc = post_upload(c, B, u, q))) return rc;
  const int nv = (c->kind == AGB_STOKES) ? 4 : 1;
  CUDA_OR_FAIL(c, cudaMalloc(&B.pts, 3 * (size_t)npts * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&B.out, (size_t)nv * npts * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&B.err, (size_t)npts * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMemcpy(B.pts, pts, 3 * (size_t)npts * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_OR_FAIL(c, domain_values(c->kind == AGB_STOKES, c->ne, c->d_geom, c->rule, c->iqud, c->iopt, npts, B.pts, c->d_xyz, B.u,
                                c->nnodes, B.q, c->diff, osem_pi(), B.out, B.err, c->stream));
  c->nlaunch += 1;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(out, B.out, (size_t)nv * npts * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(err, B.err, (size_t)npts * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return AGB_OK;
}

int agb_integral_matrices(agb_context* c, double* T, double* G, double* errs) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  cudaSetDevice(c->device);
  const GeneralLayout& L = c->gl;
  const int ncomp = (c->kind == AGB_STOKES) ? 9 : 1;
  double *dT = nullptr, *dG = nullptr, *derr = nullptr;
  CUDA_OR_FAIL(c, cudaMalloc(&dT, (size_t)ncomp * L.nsp * L.nn * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&dG, (size_t)ncomp * L.nsp * L.nq * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMalloc(&derr, (size_t)L.nsp * sizeof(double)));
  cudaError_t e = general_integrals(L, c->gd, c->d_geom, c->d_xyz, c->rule, c->iqud, c->iopt, dT, dG, derr, c->stream);
  std::vector<double> hT((size_t)ncomp * L.nsp * L.nn), hG((size_t)ncomp * L.nsp * L.nq), herr(L.nsp);
  if (e == cudaSuccess) e = cudaMemcpy(hT.data(), dT, hT.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hG.data(), dG, hG.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(herr.data(), derr, herr.size() * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(dT);
  cudaFree(dG);
  cudaFree(derr);
  if (e != cudaSuccess) return fail(c, AGB_ERR_CUDA, std::string("agb_integral_matrices: ") + cudaGetErrorString(e));
  // column-major per component, as Hmat(nsp, nnodes) of the reference
  for (int cp = 0; cp < ncomp; ++cp)
    for (int r = 0; r < L.nsp; ++r) {
      if (T)
        for (int j = 0; j < L.nn; ++j)
          T[(size_t)cp * L.nsp * L.nn + (size_t)j * L.nsp + r] = hT[((size_t)cp * L.nsp + r) * L.nn + j];
      if (G)
        for (int p = 0; p < L.nq; ++p)
          G[(size_t)cp * L.nsp * L.nq + (size_t)p * L.nsp + r] = hG[((size_t)cp * L.nsp + r) * L.nq + p];
    }
  if (errs) {
    double eu = -1e300, eq = -1e300;
    for (int r = 0; r < L.nsp; ++r) {
      if (r < L.nn) eu = std::max(eu, herr[r]);
      else eq = std::max(eq, herr[r]);
    }
    errs[0] = eu;
    errs[1] = eq;
  }
  return AGB_OK;
}

int agb_layout_sizes(agb_context* c, int* sizes) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (sizes) {
    sizes[0] = c->gl.nsp; sizes[1] = c->gl.nn; sizes[2] = c->gl.nq;
    sizes[3] = c->gl.nrow; sizes[4] = c->gl.nx; sizes[5] = c->gl.nb;
  }
  return AGB_OK;
}

int agb_solve_fields(agb_context* c, int nrhs, const double* u_in, const double* q_in, double* u_out, double* q_out,
                     int maxit, double eps, int refine, int* nit, int* istop) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (!c->assembled) return fail(c, AGB_ERR_STATE, "system not assembled");
  if (nrhs < 1 || nrhs > AGB_MAX_RHS || !u_in || !u_out || !q_out) return fail(c, AGB_ERR_ARG, "nrhs must be 1..8");
  if (maxit < 0 || !(eps >= 0.0) || refine < 0) return fail(c, AGB_ERR_ARG, "bad solver parameters");
  cudaSetDevice(c->device);
  std::vector<double> b, x;
  gather_fields(c, nrhs, u_in, q_in, b, &x);
  if (c->general) {
    if ((rc = general_rhs(c, nrhs, b))) return rc;
  } else {
    int na = 0;
    if ((rc = stage_u(c, nrhs, u_in, &na))) return rc;
    if ((rc = device_rhs(c, nrhs, na))) return rc;
  }
  CUDA_OR_FAIL(c, ensure(c->d_x, c->cap_x, (size_t)nrhs * c->n));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_x, x.data(), x.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  bool zero = true;
  for (double v : x) zero = zero && (v == 0.0);
  if ((rc = do_solve(c, nrhs, c->d_x, maxit, eps, refine, nit, istop, zero))) return rc;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(x.data(), c->d_x, x.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  // StokesDistributeUnknowns / the distribution loop of sdSolveCRS
  const GeneralLayout& L = c->gl;
  const size_t nu = (size_t)nrhs * L.neq * c->nnodes, nqv = (size_t)nrhs * L.neq * c->nelem;
  std::copy(u_in, u_in + nu, u_out);
  if (q_in) std::copy(q_in, q_in + nqv, q_out);
  else std::fill(q_out, q_out + nqv, 0.0);
  for (int r = 0; r < nrhs; ++r)
    for (int en = 0; en < L.neq; ++en) {
      for (int j = 0; j < L.nn; ++j) {
        const int t = en * L.nn + j;
        if (!L.node_known[t] && L.node_xcol[t] >= 0)
          u_out[((size_t)r * L.neq + en) * c->nnodes + L.nodeList[j]] = x[(size_t)r * L.nx + L.node_xcol[t]];
      }
      for (int p = 0; p < L.nq; ++p) {
        const int t = en * L.nq + p;
        if (!L.elem_known[t] && L.elem_xcol[t] >= 0)
          q_out[((size_t)r * L.neq + en) * c->nelem + c->elemList[p]] = x[(size_t)r * L.nx + L.elem_xcol[t]];
      }
    }
  return AGB_OK;
}


// One body of a batch on the device: pieces of the wave's arena.
struct BatchSlot {
  int body = 0, nn = 0, ne = 0, ldp = 0, pldp = 0, m = 0, n = 0, groups = 1, na = 0;
  int64_t lda = 0;
  size_t o_xyz, o_et, o_con, o_wall, o_geom, o_pts, o_src, o_nrm, o_cs, o_A, o_q, o_u, o_act, o_ract, o_rhs, o_x,
      o_ft, o_P;  // device offsets
  size_t h_xyz, h_et, h_con, h_wall, h_cs, h_u, h_act, h_ract;  // offsets in the upload image
};

int agb_batch_resistance(agb_context* c, int nbodies, const int* node_off, const double* xyz, const int* elem_off,
                         const int* etype, const int* con, const int* bcid, int particle_wall, int outer_wall,
                         int itri, int maxit, double eps, double mem_gb, int autotune, double* R, int* nit,
                         int* istop, double* stats) {
  // the bodies are checked before the context, so that these checks run without a GPU
  if (nbodies < 1 || !node_off || !xyz || !elem_off || !etype || !con || !bcid || !R)
    return fail(c, AGB_ERR_ARG, "agb_batch_resistance: missing arrays");
  if (itri < 1 || itri > 5 || maxit < 0 || !(eps >= 0.0) || !(mem_gb >= 0.0))
    return fail(c, AGB_ERR_ARG, "agb_batch_resistance: bad parameters");
  for (int i = 0; i < nbodies; ++i) {
    if (node_off[i + 1] <= node_off[i] || elem_off[i + 1] <= elem_off[i])
      return fail(c, AGB_ERR_ARG, "agb_batch_resistance: empty body " + std::to_string(i));
    const int nn = node_off[i + 1] - node_off[i];
    bool pw = false, ow = false;
    for (int e = elem_off[i]; e < elem_off[i + 1]; ++e) {
      if (etype[e] != AGB_TRI) return fail(c, AGB_ERR_UNSUPPORTED, "batched bodies must be triangle meshes");
      if (bcid[e] != particle_wall && bcid[e] != outer_wall)
        return fail(c, AGB_ERR_ARG, "batched body " + std::to_string(i) + " has a third wall");
      pw = pw || bcid[e] == particle_wall;
      ow = ow || bcid[e] == outer_wall;
      for (int k = 0; k < 3; ++k)
        if (con[4 * (size_t)e + k] < 0 || con[4 * (size_t)e + k] >= nn)
          return fail(c, AGB_ERR_ARG, "connectivity out of range in body " + std::to_string(i));
    }
    if (!pw || !ow) return fail(c, AGB_ERR_ARG, "batched body " + std::to_string(i) + " lacks a wall");
    const std::string defect = mesh_defect(nn, xyz + 3 * (size_t)node_off[i], elem_off[i], elem_off[i + 1], etype, con);
    if (!defect.empty()) return fail(c, AGB_ERR_ARG, "batched body " + std::to_string(i) + ": " + defect);
  }
  if (!c) return fail(c, AGB_ERR_ARG, "agb_batch_resistance: no context");
  cudaSetDevice(c->device);
  using clk = std::chrono::steady_clock;
  auto ms = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
  const auto t_start = clk::now();
  cudaStream_t st = c->stream;
  cudaEvent_t d0 = nullptr, d1 = nullptr;
  CUDA_OR_FAIL(c, cudaEventCreate(&d0));
  CUDA_OR_FAIL(c, cudaEventCreate(&d1));
  CUDA_OR_FAIL(c, cudaEventRecord(d0, st));
  // quadrature rule (shared by all bodies)
  std::vector<double> rl, rw;
  expand_rule(itri, rl, rw);
  const int Q = (int)rw.size();
  RuleDev rule;
  rule.Q = Q;
  CUDA_OR_FAIL(c, cudaMallocAsync(&rule.l, rl.size() * sizeof(double), st));
  CUDA_OR_FAIL(c, cudaMallocAsync(&rule.w, rw.size() * sizeof(double), st));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(rule.l, rl.data(), rl.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(rule.w, rw.data(), rw.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  // slot layout of every body
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  std::vector<BatchSlot> slots(nbodies);
  std::vector<size_t> dev_bytes(nbodies), up_bytes(nbodies);
  for (int i = 0; i < nbodies; ++i) {
    BatchSlot& b = slots[i];
    b.body = i;
    b.nn = node_off[i + 1] - node_off[i];
    b.ne = elem_off[i + 1] - elem_off[i];
    b.ldp = (b.ne + 31) / 32 * 32;
    b.pldp = (b.ne + 63) / 64 * 64;
    b.m = b.n = 3 * b.ne;
    b.lda = ((int64_t)b.n + 31) / 32 * 32;
    b.groups = std::max(1, std::min(32, b.m / 512));
    size_t o = 0;
    auto take = [&](size_t bytes) { const size_t r = o; o += al(bytes); return r; };
    b.o_xyz = take(3 * (size_t)b.nn * 8); b.o_et = take((size_t)b.ne * 4); b.o_con = take(4 * (size_t)b.ne * 4);
    b.o_wall = take((size_t)b.ne * 4); b.o_cs = take((size_t)b.ldp * 4); b.o_u = take(18 * (size_t)b.nn * 8);
    b.o_act = take((size_t)b.ne * 4); b.o_ract = take((size_t)b.ne);
    const size_t upload = o;  // the pieces above are uploaded from one host image
    b.h_xyz = b.o_xyz; b.h_et = b.o_et; b.h_con = b.o_con; b.h_wall = b.o_wall; b.h_cs = b.o_cs; b.h_u = b.o_u;
    b.h_act = b.o_act; b.h_ract = b.o_ract;
    b.o_geom = take((size_t)b.ne * sizeof(ElemGeom));
    b.o_pts = take((size_t)Q * b.ldp * sizeof(QPt<float>));
    b.o_src = take(3 * (size_t)b.ldp * 4); b.o_nrm = take(3 * (size_t)b.ldp * 4);
    b.o_A = take((size_t)b.ne * 6 * b.pldp * 4);  // packed symmetric blocks (pk_idx layout)
    b.o_q = take((size_t)b.lda * 8);
    b.o_rhs = take(6 * (size_t)b.m * 8); b.o_x = take(6 * (size_t)b.n * 8); b.o_ft = take(6 * AGB_MAX_RHS * 8);
    b.o_P = take((size_t)b.groups * b.lda * 8);
    dev_bytes[i] = o;
    up_bytes[i] = upload;
  }
  // solver vectors of the batched LSQR (pool of batch_lsqr_solve) per body
  auto solver_bytes = [&](int i) {
    const BatchSlot& b = slots[i];
    const double mpad = std::ceil(b.m / 256.0) * 256.0;
    const bool bicg_used = c->solver == AGB_SOLVER_BICGSTAB || c->solver == AGB_SOLVER_HYBRID;
    const double bicg = bicg_used ? mpad * 8 * 8 * 7.0 + mpad * 8 : 0.0;
    const double pc9 = (c->solver == AGB_SOLVER_LSQR_BLOCK || c->solver == AGB_SOLVER_GMRES) ? 72.0 * b.ne : 0.0;
    const double mr = c->gmres_restart;
    const double gm = (c->solver == AGB_SOLVER_GMRES)
                          ? 64.0 * (mr * mpad + (mr + 1) * mr + 5 * (mr + 1) + mpad + mpad / 32 * (mr + 1)) +
                                192.0 * b.ne
                          : 0.0;
    return mpad * 8 * 12.0 + (double)b.lda * 8 * (8 * 3 + 4 + 8 * 8) + 65536.0 + bicg + pc9 + gm;
  };
  double budget = mem_gb * 1e9;
  if (budget <= 0.0) {
    size_t fr = 0, tot = 0;
    CUDA_OR_FAIL(c, cudaMemGetInfo(&fr, &tot));
    budget = 0.8 * (double)fr;
  }
  // waves: largest bodies first, packed greedily under the budget
  std::vector<int> order(nbodies);
  for (int i = 0; i < nbodies; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return dev_bytes[a] > dev_bytes[b]; });
  std::vector<std::vector<int>> waves;
  double used = 0.0;
  for (int i : order) {
    const double bb = (double)dev_bytes[i] + solver_bytes(i);
    if (waves.empty() || (used + bb > budget && !waves.back().empty())) {
      waves.emplace_back();
      used = 0.0;
    }
    waves.back().push_back(i);
    used += bb;
  }
  BatchTune tune;
  BatchStats bst;
  bool tuned = false;
  double t_asm = 0.0, t_solve = 0.0, t_ft = 0.0;
  long asm_launches = 0;
  char* arena = nullptr;
  char* h_img = nullptr;
  size_t arena_cap = 0, img_cap = 0;
  auto release = [&]() {
    if (arena) cudaFree(arena);
    if (h_img) cudaFreeHost(h_img);
    cudaFree(rule.l);
    cudaFree(rule.w);
    cudaEventDestroy(d0);
    cudaEventDestroy(d1);
  };
  auto bail = [&](int code, const std::string& msg) {
    cudaStreamSynchronize(st);
    release();
    return fail(c, code, "agb_batch_resistance: " + msg);
  };
  for (const auto& w : waves) {
    const auto ta = clk::now();
    // arena of the wave
    std::vector<size_t> base(w.size()), hbase(w.size());
    size_t total = 0, htotal = 0;
    for (size_t t = 0; t < w.size(); ++t) {
      base[t] = total; total += dev_bytes[w[t]];
      hbase[t] = htotal; htotal += up_bytes[w[t]];
    }
    if (total > arena_cap) {
      if (arena) { cudaStreamSynchronize(st); cudaFree(arena); arena = nullptr; }
      if (cudaMalloc(&arena, total) != cudaSuccess) return bail(AGB_ERR_CUDA, "arena of " + std::to_string(total) + " bytes");
      arena_cap = total;
    }
    if (htotal > img_cap) {
      if (h_img) { cudaStreamSynchronize(st); cudaFreeHost(h_img); h_img = nullptr; }
      if (cudaMallocHost(&h_img, htotal) != cudaSuccess) return bail(AGB_ERR_CUDA, "host staging");
      img_cap = htotal;
    }
    // host image: nodes, elements (particle wall first, then the container), u of
    // the six rigid motions of the container, active elements and rows
    cudaStreamSynchronize(st);  // the previous wave's upload of the image has completed
    for (size_t t = 0; t < w.size(); ++t) {
      BatchSlot& b = slots[w[t]];
      const int i = b.body;
      char* h = h_img + hbase[t];
      double* hx = (double*)(h + b.h_xyz);
      std::memcpy(hx, xyz + 3 * (size_t)node_off[i], 3 * (size_t)b.nn * 8);
      int* het = (int*)(h + b.h_et);
      int* hcon = (int*)(h + b.h_con);
      int* hwall = (int*)(h + b.h_wall);
      float* hcs = (float*)(h + b.h_cs);
      double* hu = (double*)(h + b.h_u);
      int* hact = (int*)(h + b.h_act);
      unsigned char* hract = (unsigned char*)(h + b.h_ract);
      std::vector<char> onOuter(b.nn, 0);
      int p = 0;
      for (int k = 0; k < 2; ++k)
        for (int e = elem_off[i]; e < elem_off[i + 1]; ++e) {
          if (bcid[e] != (k == 0 ? particle_wall : outer_wall)) continue;
          het[p] = AGB_TRI;
          for (int kk = 0; kk < 4; ++kk) hcon[4 * p + kk] = (kk < 3) ? con[4 * (size_t)e + kk] : -1;
          hwall[p] = k;
          hract[p] = (unsigned char)k;
          if (k == 1)
            for (int kk = 0; kk < 3; ++kk) onOuter[hcon[4 * p + kk]] = 1;
          ++p;
        }
      for (int q = 0; q < b.ldp; ++q) hcs[q] = (q < b.ne) ? -1.0f : 0.0f;  // -(normMul/mu), mu = 1
      std::memset(hu, 0, 18 * (size_t)b.nn * 8);
      for (int n = 0; n < b.nn; ++n) {
        if (!onOuter[n]) continue;
        const double* x = hx + 3 * (size_t)n;
        for (int a = 0; a < 3; ++a) hu[((size_t)a * 3 + a) * b.nn + n] = 1.0;
        const double wv[3][3] = {{0, -x[2], x[1]}, {x[2], 0, -x[0]}, {-x[1], x[0], 0}};
        for (int a = 0; a < 3; ++a)
          for (int bb = 0; bb < 3; ++bb) hu[((size_t)(3 + a) * 3 + bb) * b.nn + n] = wv[a][bb];
      }
      b.na = 0;
      for (int q = 0; q < b.ne; ++q)
        if (hract[q]) hact[b.na++] = q;
    }
    // one upload per body (its pieces are contiguous in both images)
    for (size_t t = 0; t < w.size(); ++t)
      if (cudaMemcpyAsync(arena + base[t], h_img + hbase[t], up_bytes[w[t]], cudaMemcpyHostToDevice, st) != cudaSuccess)
        return bail(AGB_ERR_CUDA, "upload");
    static const double kNormMul[2] = {1.0, 1.0};
    double* d_nm = nullptr;
    if (cudaMallocAsync(&d_nm, 2 * sizeof(double), st) != cudaSuccess ||
        cudaMemcpyAsync(d_nm, kNormMul, 2 * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return bail(AGB_ERR_CUDA, "normMul");
    std::vector<BatchBody> bodies(w.size());
    for (size_t t = 0; t < w.size(); ++t) {
      const BatchSlot& b = slots[w[t]];
      char* d = arena + base[t];
      ElemGeom* geom = (ElemGeom*)(d + b.o_geom);
      float* A = (float*)(d + b.o_A);
      cudaError_t e = launch_geometry(b.ne, (const double*)(d + b.o_xyz), (const int*)(d + b.o_et),
                                      (const int*)(d + b.o_con), (const int*)(d + b.o_wall), d_nm, geom, st);
      if (e == cudaSuccess)
        e = launch_expand_points<float>(b.ne, b.ldp, geom, rule, (QPt<float>*)(d + b.o_pts), (float*)(d + b.o_src),
                                        (float*)(d + b.o_nrm), st);
      if (e == cudaSuccess) e = cudaMemsetAsync(A, 0, (size_t)b.ne * 6 * b.pldp * 4, st);  // zero pad columns
      if (e == cudaSuccess)
        e = launch_stokes_G_packed(b.ne, Q, b.ldp, b.pldp, (const QPt<float>*)(d + b.o_pts),
                                   (const float*)(d + b.o_src), (const float*)(d + b.o_cs), A, st);
      if (e == cudaSuccess) e = launch_stokes_self_packed(b.ne, b.pldp, geom, 1.0, A, st);
      // lsqr_precon's column scaling: only the LSQR solvers (and the hybrid's LSQR
      // fallback) read it
      if (e == cudaSuccess && c->solver != AGB_SOLVER_GMRES && c->solver != AGB_SOLVER_BICGSTAB)
        e = packed_colnorms(A, b.ne, b.pldp, b.lda, (double*)(d + b.o_q), (double*)(d + b.o_P), b.groups, st);
      if (e == cudaSuccess) {
        StokesRhsArgs a;
        a.ne = b.ne; a.Q = Q; a.ldp = b.ldp; a.k = 6; a.nnodes = b.nn;
        a.pts = d + b.o_pts;
        a.geom = geom; a.rule_l = rule.l; a.rule_w = rule.w; a.u = (const double*)(d + b.o_u);
        a.active = (const int*)(d + b.o_act); a.na = b.na; a.row_active = (const unsigned char*)(d + b.o_ract);
        a.rhs = (double*)(d + b.o_rhs);
        e = launch_stokes_rhs<float>(a, st);
      }
      if (e != cudaSuccess) return bail(AGB_ERR_CUDA, std::string("assembly: ") + cudaGetErrorString(e));
      asm_launches += 5 + (c->solver != AGB_SOLVER_GMRES && c->solver != AGB_SOLVER_BICGSTAB ? 2 : 0) +
                      (b.na > 0 ? 2 : 0);
      bodies[t].A = A;
      bodies[t].lda = b.lda;
      bodies[t].m = b.m;
      bodies[t].n = b.n;
      bodies[t].pk_ne = b.ne;
      bodies[t].pk_ldp = b.pldp;
      bodies[t].b = (const double*)(d + b.o_rhs);
      bodies[t].q = (const double*)(d + b.o_q);
      bodies[t].x = (double*)(d + b.o_x);
    }
    cudaFreeAsync(d_nm, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return bail(AGB_ERR_CUDA, "assembly of the wave");
    const auto tb = clk::now();
    if (autotune && !tuned && (c->solver == AGB_SOLVER_LSQR || c->solver == AGB_SOLVER_LSQR_BLOCK)) {
      std::string rep, err;
      if (!batch_autotune(bodies, st, tune, rep, err)) return bail(AGB_ERR_CUDA, "autotune: " + err);
      tuned = true;
    }
    std::vector<int> nv, iv;
    std::string err;
    if (c->solver == AGB_SOLVER_GMRES) {
      if (!batch_gmres_solve(bodies, 6, eps, maxit, c->gmres_restart, st, nv, iv, &bst, err))
        return bail(AGB_ERR_CUDA, "solve: " + err);
    } else if (c->solver == AGB_SOLVER_BICGSTAB || c->solver == AGB_SOLVER_HYBRID) {
      if (!batch_bicgstab_solve(bodies, 6, eps, maxit, st, nv, iv, &bst, err)) return bail(AGB_ERR_CUDA, "solve: " + err);
      // FP64 refinement of the bodies whose recursive residual converged but whose
      // true residual did not (istop 4): BiCGSTAB on r = b - A x from zero to
      // eps ||b|| / ||r||, x += d, at most kBicgRestarts times
      for (int pass = 0; pass < kBicgRestarts; ++pass) {
        std::vector<BatchBody> redo;
        std::vector<size_t> where;
        for (size_t t = 0; t < bodies.size(); ++t) {
          bool any4 = false;
          for (int r = 0; r < 6; ++r) any4 = any4 || iv[6 * t + r] == 4;
          if (any4) {
            redo.push_back(bodies[t]);
            where.push_back(t);
          }
        }
        if (redo.empty()) break;
        std::vector<double*> rbuf(redo.size(), nullptr), dbuf(redo.size(), nullptr);
        auto free_bufs = [&]() {
          for (auto p : rbuf) if (p) cudaFreeAsync(p, st);
          for (auto p : dbuf) if (p) cudaFreeAsync(p, st);
        };
        bool okb = true;
        for (size_t u = 0; u < redo.size() && okb; ++u) {
          okb = cudaMallocAsync(&rbuf[u], (size_t)6 * redo[u].m * sizeof(double), st) == cudaSuccess &&
                cudaMallocAsync(&dbuf[u], (size_t)6 * redo[u].n * sizeof(double), st) == cudaSuccess &&
                cudaMemsetAsync(dbuf[u], 0, (size_t)6 * redo[u].n * sizeof(double), st) == cudaSuccess;
        }
        std::vector<double> rel;
        if (!okb || !batch_residual(redo, 6, st, rbuf, rel, err)) {
          free_bufs();
          return bail(AGB_ERR_CUDA, "restart residual: " + (okb ? err : std::string("allocation")));
        }
        // each correction to its own column's tolerance eps ||b|| / ||r||: one
        // tolerance for all would push the columns nearly done below the FP32
        // rounding of the products, where BiCGSTAB stagnates
        double worst = 0.0;
        std::vector<double> tolc(6 * redo.size(), 0.5);
        for (size_t u = 0; u < redo.size(); ++u)
          for (int r = 0; r < 6; ++r) {
            const double v = rel[6 * u + r];
            if (v > eps && iv[6 * where[u] + r] == 4) {
              worst = std::max(worst, v);
              tolc[6 * u + r] = std::min(0.5, eps / v);
            } else if (cudaMemsetAsync(rbuf[u] + (size_t)r * redo[u].m, 0, (size_t)redo[u].m * sizeof(double), st) !=
                     cudaSuccess) okb = false;  // done, or failed otherwise: no correction
          }
        std::vector<BatchBody> corr = redo;
        for (size_t u = 0; u < redo.size(); ++u) {
          corr[u].b = rbuf[u];
          corr[u].x = dbuf[u];
        }
        if (okb && worst <= 0.0) {  // the true residuals are within eps already
          free_bufs();
          for (size_t u = 0; u < redo.size(); ++u)
            for (int r = 0; r < 6; ++r)
              if (iv[6 * where[u] + r] == 4) iv[6 * where[u] + r] = 0;
          break;
        }
        std::vector<int> n2, i2;
        if (!okb ||
            !batch_bicgstab_solve(corr, 6, std::min(0.5, eps / worst), maxit, st, n2, i2, &bst, err, &tolc) ||
            !batch_axpy(redo, 6, dbuf, st, err) || !batch_residual(redo, 6, st, {}, rel, err)) {
          free_bufs();
          return bail(AGB_ERR_CUDA, "restart: " + err);
        }
        free_bufs();
        for (size_t u = 0; u < redo.size(); ++u)
          for (int r = 0; r < 6; ++r) {
            const size_t t = 6 * where[u] + r;
            nv[t] += n2[6 * u + r];
            if (iv[t] == 4) iv[t] = rel[6 * u + r] <= eps ? 0 : (i2[6 * u + r] == 2 || i2[6 * u + r] == 3 ? i2[6 * u + r] : 4);
          }
      }
      if (c->solver == AGB_SOLVER_HYBRID) {
        // bodies with a right-hand side BiCGSTAB did not converge: batched LSQR
        // (default tiles, the reference's iteration limit) from a zero start
        std::vector<BatchBody> redo;
        std::vector<size_t> where;
        for (size_t t = 0; t < bodies.size(); ++t) {
          bool ok = true;
          for (int r = 0; r < 6; ++r) ok = ok && iv[6 * t + r] == 0;
          if (!ok) {
            redo.push_back(bodies[t]);
            where.push_back(t);
          }
        }
        if (!redo.empty()) {
          std::vector<int> nl, il;
          if (!batch_lsqr_solve(redo, 6, eps, 0, tune, st, nl, il, &bst, err))
            return bail(AGB_ERR_CUDA, "solve (LSQR after BiCGSTAB): " + err);
          for (size_t u = 0; u < where.size(); ++u)
            for (int r = 0; r < 6; ++r) {
              nv[6 * where[u] + r] += nl[6 * u + r];
              iv[6 * where[u] + r] = 10 + il[6 * u + r];
            }
        }
      }
    } else if (!batch_lsqr_solve(bodies, 6, eps, maxit, tune, st, nv, iv, &bst, err,
                                 c->solver == AGB_SOLVER_LSQR_BLOCK)) {
      return bail(AGB_ERR_CUDA, "solve: " + err);
    }
    const auto tc = clk::now();
    for (size_t t = 0; t < w.size(); ++t) {
      const BatchSlot& b = slots[w[t]];
      char* d = arena + base[t];
      if (launch_force_torque(b.ne, 6, (const ElemGeom*)(d + b.o_geom), (const double*)(d + b.o_x), 0,
                              (double*)(d + b.o_ft), st) != cudaSuccess ||
          cudaMemcpyAsync(R + 36 * (size_t)b.body, d + b.o_ft, 36 * sizeof(double), cudaMemcpyDeviceToHost, st) !=
              cudaSuccess)
        return bail(AGB_ERR_CUDA, "force/torque");
      for (int r = 0; r < 6; ++r) {
        if (nit) nit[6 * (size_t)b.body + r] = nv[6 * t + r];
        if (istop) istop[6 * (size_t)b.body + r] = iv[6 * t + r];
      }
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return bail(AGB_ERR_CUDA, "force/torque");
    asm_launches += (long)w.size();
    const auto td = clk::now();
    t_asm += ms(ta, tb);
    t_solve += ms(tb, tc);
    t_ft += ms(tc, td);
  }
  CUDA_OR_FAIL(c, cudaEventRecord(d1, st));
  CUDA_OR_FAIL(c, cudaEventSynchronize(d1));
  float dev_ms = 0.f;
  cudaEventElapsedTime(&dev_ms, d0, d1);
  release();
  if (stats) {
    stats[0] = t_asm; stats[1] = t_solve; stats[2] = ms(t_start, clk::now()); stats[3] = (double)waves.size();
    stats[4] = bst.av_ms; stats[5] = bst.atu_ms; stats[6] = (double)bst.av_launches; stats[7] = (double)bst.atu_launches;
    stats[8] = bst.bytes_av; stats[9] = (double)(bst.launches + asm_launches);
    stats[10] = bst.av_rows; stats[11] = bst.atu_rs; stats[12] = bst.atu_rows; stats[13] = (double)bst.iterations;
    stats[14] = dev_ms; stats[15] = t_ft;
  }
  return AGB_OK;
}


// ---------------------------------------------------------------------------
// Direct solver of the FULL path
// ---------------------------------------------------------------------------
__global__ void k_lu_from_system(const double* __restrict__ A, int64_t lda, int m, int n, const double* __restrict__ q,
                                 double* __restrict__ out) {
  // out (column-major, leading dimension m) = A_rowmajor ./ q (undo lsqr_precon's column scaling)
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;  // bx: column j block, by: row i block
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = by + r, j = bx + threadIdx.x;
    if (i < m && j < n) tile[r][threadIdx.x] = A[(int64_t)i * lda + j] / q[j];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int j = bx + r, i = by + threadIdx.x;
    if (i < m && j < n) out[(int64_t)j * m + i] = tile[threadIdx.x][r];
  }
}

int agb_form_pre_fm(int pret, int neq, double* q, double* a, float* cpu, int* ierr) {
  if (neq < 1 || !q || !a) return fail(nullptr, AGB_ERR_ARG, "agb_form_pre_fm: bad arguments");
  auto t0 = std::chrono::steady_clock::now();
  if (ierr) *ierr = 0;
  if (pret == 1) {
    for (int i = 0; i < neq; ++i) q[i] = 1.0 / a[(size_t)i * neq + i];  // frmdiafm(neq, 1, a, q)
  } else if (pret == 2) {
    cudaStream_t s = nullptr;
    double* dA = nullptr;
    int* dpiv = nullptr;
    int info = 0;
    std::string err;
    const size_t bytes = (size_t)neq * neq * sizeof(double);
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
      return fail(nullptr, AGB_ERR_CUDA, "agb_form_pre_fm: stream");
    bool ok = cudaMalloc(&dA, bytes) == cudaSuccess && cudaMalloc(&dpiv, neq * sizeof(int)) == cudaSuccess &&
              cudaMemcpyAsync(dA, a, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
    if (ok) ok = lu_factor_dev(dA, neq, neq, dpiv, &info, s, nullptr, err);
    std::vector<int> hp(neq);
    if (ok) ok = cudaMemcpyAsync(a, dA, bytes, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                 cudaMemcpyAsync(hp.data(), dpiv, neq * sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                 cudaStreamSynchronize(s) == cudaSuccess;
    cudaFree(dA);
    cudaFree(dpiv);
    cudaStreamDestroy(s);
    if (!ok) return fail(nullptr, AGB_ERR_CUDA, "agb_form_pre_fm: " + (err.empty() ? std::string("CUDA error") : err));
    for (int i = 0; i < neq; ++i) q[i] = (double)hp[i];
    if (ierr) *ierr = info;
  } else if (pret != 0) {
    return fail(nullptr, AGB_ERR_ARG, "agb_form_pre_fm: preconditioner type must be 0, 1 or 2");
  }
  if (cpu) *cpu += (float)std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return AGB_OK;
}

int agb_solv_eqn_fm(int slvt, int pret, int prep, int maxit, int stopt, double eps, int neq, double* q, double* a,
                    const double* b, double* x, int* nit, double* cpu, int* ierr) {
  (void)maxit; (void)stopt; (void)eps;  // direct solver: no iteration control
  if (neq < 1 || !q || !a || !b || !x) return fail(nullptr, AGB_ERR_ARG, "agb_solv_eqn_fm: bad arguments");
  if (slvt != 0) return fail(nullptr, AGB_ERR_UNSUPPORTED, "agb_solv_eqn_fm: solver type must be 0 (direct)");
  auto t0 = std::chrono::steady_clock::now();
  double nb = 0.0;
  for (int i = 0; i < neq; ++i) nb += b[i] * b[i];
  if (nb == 0.0) {  // b = 0: x = 0, nit = 0, ierr = 0
    std::fill(x, x + neq, 0.0);
    if (nit) *nit = 0;
    if (ierr) *ierr = 0;
    return AGB_OK;
  }
  if (pret != 0 && prep == 1) {
    float c2 = 0.f;
    int rc = agb_form_pre_fm(pret, neq, q, a, &c2, ierr);
    if (rc) return rc;
  }
  if (pret != 2) return fail(nullptr, AGB_ERR_UNSUPPORTED, "agb_solv_eqn_fm: the direct solver needs the LU (pret 2)");
  std::vector<int> piv(neq);
  for (int i = 0; i < neq; ++i) {
    piv[i] = (int)q[i];
    if (piv[i] < 1 || piv[i] > neq) return fail(nullptr, AGB_ERR_ARG, "agb_solv_eqn_fm: q holds no LU pivots");
  }
  cudaStream_t s = nullptr;
  double *dA = nullptr, *dB = nullptr;
  std::string err;
  const size_t bytes = (size_t)neq * neq * sizeof(double);
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return fail(nullptr, AGB_ERR_CUDA, "agb_solv_eqn_fm: stream");
  bool ok = cudaMalloc(&dA, bytes) == cudaSuccess && cudaMalloc(&dB, neq * sizeof(double)) == cudaSuccess &&
            cudaMemcpyAsync(dA, a, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(dB, b, neq * sizeof(double), cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (ok) ok = lu_solve_dev(dA, neq, neq, piv.data(), 1, dB, s, nullptr, err);
  if (ok) ok = cudaMemcpyAsync(x, dB, neq * sizeof(double), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
               cudaStreamSynchronize(s) == cudaSuccess;
  cudaFree(dA);
  cudaFree(dB);
  cudaStreamDestroy(s);
  if (!ok) return fail(nullptr, AGB_ERR_CUDA, "agb_solv_eqn_fm: " + (err.empty() ? std::string("CUDA error") : err));
  if (ierr) *ierr = 0;
  if (cpu) *cpu += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return AGB_OK;
}

int agb_solve_lu(agb_context* c, int nrhs, const double* u, double* x, int* info) {
  int rc = check_ctx(c, true);
  if (rc) return rc;
  if (!c->assembled) return fail(c, AGB_ERR_STATE, "system not assembled");
  if (c->prec != AGB_FP64) return fail(c, AGB_ERR_UNSUPPORTED, "the direct solver needs the FP64 system");
  if (c->m != c->n) return fail(c, AGB_ERR_UNSUPPORTED, "the direct solver needs a square system");
  if (nrhs < 1 || nrhs > AGB_MAX_RHS || !u || !x) return fail(c, AGB_ERR_ARG, "nrhs must be 1..8");
  cudaSetDevice(c->device);
  const int n = c->n;
  if (!c->lu_ready) {
    int* dpiv = nullptr;
    CUDA_OR_FAIL(c, cudaMalloc(&c->d_lu, (size_t)n * n * sizeof(double)));
    dim3 g((n + 31) / 32, (n + 31) / 32), b(32, 8);
    if (int rc = ensure_q(c)) return rc;
    k_lu_from_system<<<g, b, 0, c->stream>>>((const double*)c->d_A, c->lda, n, n, c->d_q, c->d_lu);
    c->nlaunch += 1;
    CUDA_OR_FAIL(c, cudaGetLastError());
    CUDA_OR_FAIL(c, cudaMalloc(&dpiv, n * sizeof(int)));
    int inf = 0;
    std::string err;
    const bool ok = lu_factor_dev(c->d_lu, n, n, dpiv, &inf, c->stream, &c->nlaunch, err);
    c->lu_ipiv.resize(n);
    const bool ok2 = ok && cudaMemcpy(c->lu_ipiv.data(), dpiv, n * sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(dpiv);
    if (!ok2) return fail(c, AGB_ERR_CUDA, "lu: " + err);
    c->lu_info = inf;
    c->lu_ready = true;
  }
  if (info) *info = c->lu_info;
  if (c->general) {
    std::vector<double> b;
    gather_fields(c, nrhs, u, nullptr, b, nullptr);
    if ((rc = general_rhs(c, nrhs, b))) return rc;
  } else {
    int na = 0;
    if ((rc = stage_u(c, nrhs, u, &na))) return rc;
    if ((rc = device_rhs(c, nrhs, na))) return rc;
  }
  CUDA_OR_FAIL(c, ensure(c->d_x, c->cap_x, (size_t)nrhs * n));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->d_x, c->d_rhs, (size_t)nrhs * n * sizeof(double), cudaMemcpyDeviceToDevice,
                                  c->stream));
  std::string err;
  if (!lu_solve_dev(c->d_lu, n, n, c->lu_ipiv.data(), nrhs, c->d_x, c->stream, &c->nlaunch, err))
    return fail(c, AGB_ERR_CUDA, "lu solve: " + err);
  CUDA_OR_FAIL(c, cudaMemcpyAsync(x, c->d_x, (size_t)nrhs * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return AGB_OK;
}


// ---------------------------------------------------------------------------
// MLP surrogate of the resistance tensor
// ---------------------------------------------------------------------------
struct agb_mlp {
  agb::Mlp net;
  std::string err;
};

static int mlp_fail(agb_mlp* m, int code, const std::string& msg) {
  if (m) m->err = msg;
  return fail(nullptr, code, msg);
}

int agb_mlp_create(agb_mlp** out, int device, int nin, int nhidden, int nout, unsigned long long seed) {
  if (!out || nin < 1 || nhidden < 1 || nout < 1) return fail(nullptr, AGB_ERR_ARG, "agb_mlp_create: bad sizes");
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return fail(nullptr, AGB_ERR_CUDA, "agb_mlp_create: device");
  agb_mlp* m = new agb_mlp();
  m->net.nin = nin;
  m->net.nh = nhidden;
  m->net.nout = nout;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || !m->net.init(device, seed, s)) {
    const std::string e = "agb_mlp_create: " + m->net.err;
    if (s) cudaStreamDestroy(s);
    delete m;
    return fail(nullptr, AGB_ERR_CUDA, e);
  }
  *out = m;
  return AGB_OK;
}

int agb_mlp_destroy(agb_mlp* m) {
  if (!m) return AGB_OK;
  cudaSetDevice(m->net.device);
  cudaStream_t s = m->net.s;
  m->net.release();
  if (s) cudaStreamDestroy(s);
  delete m;
  return AGB_OK;
}

int agb_mlp_num_params(agb_mlp* m, long long* n) {
  if (!m || !n) return AGB_ERR_ARG;
  *n = (long long)m->net.nparams();
  return AGB_OK;
}

int agb_mlp_get_params(agb_mlp* m, float* p) {
  if (!m || !p) return AGB_ERR_ARG;
  cudaSetDevice(m->net.device);
  if (cudaMemcpy(p, m->net.params, m->net.nparams() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return mlp_fail(m, AGB_ERR_CUDA, "agb_mlp_get_params");
  return AGB_OK;
}

int agb_mlp_set_params(agb_mlp* m, const float* p) {
  if (!m || !p) return AGB_ERR_ARG;
  cudaSetDevice(m->net.device);
  if (cudaMemcpy(m->net.params, p, m->net.nparams() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return mlp_fail(m, AGB_ERR_CUDA, "agb_mlp_set_params");
  return AGB_OK;
}

int agb_mlp_set_normalization(agb_mlp* m, const float* x_mean, const float* x_std, const float* y_mean,
                              const float* y_std) {
  if (!m || !x_mean || !x_std || !y_mean || !y_std) return AGB_ERR_ARG;
  const int nin = m->net.nin, nout = m->net.nout;
  std::vector<float> h(2 * (nin + nout));
  for (int i = 0; i < nin; ++i) {
    if (!(x_std[i] > 0.f)) return mlp_fail(m, AGB_ERR_ARG, "x_std must be positive");
    h[i] = x_mean[i]; h[nin + i] = x_std[i];
  }
  for (int i = 0; i < nout; ++i) {
    if (!(y_std[i] > 0.f)) return mlp_fail(m, AGB_ERR_ARG, "y_std must be positive");
    h[2 * nin + i] = y_mean[i]; h[2 * nin + nout + i] = y_std[i];
  }
  cudaSetDevice(m->net.device);
  if (cudaMemcpy(m->net.norm, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return mlp_fail(m, AGB_ERR_CUDA, "agb_mlp_set_normalization");
  return AGB_OK;
}

int agb_mlp_gradient(agb_mlp* m, int n, const float* X, const float* Y, int split, float* grad, double* loss) {
  if (!m || n < 1 || !X || !Y || !grad) return AGB_ERR_ARG;
  agb::Mlp& net = m->net;
  cudaSetDevice(net.device);
  float *dX = nullptr, *dY = nullptr;
  bool ok = net.ensure_ws(n) && cudaMalloc(&dX, (size_t)n * net.nin * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&dY, (size_t)n * net.nout * sizeof(float)) == cudaSuccess &&
            cudaMemcpyAsync(dX, X, (size_t)n * net.nin * sizeof(float), cudaMemcpyHostToDevice, net.s) == cudaSuccess &&
            cudaMemcpyAsync(dY, Y, (size_t)n * net.nout * sizeof(float), cudaMemcpyHostToDevice, net.s) == cudaSuccess;
  if (ok) {
    net.load_inputs(n, dX);
    net.forward(n, true, split != 0);
    net.backward(n, dY, split != 0);
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpyAsync(grad, net.grads, net.nparams() * sizeof(float), cudaMemcpyDeviceToHost, net.s) == cudaSuccess;
    if (ok && loss) *loss = net.loss_sum(n) / ((double)n * net.nout);
    ok = ok && cudaStreamSynchronize(net.s) == cudaSuccess;
  }
  cudaFree(dX);
  cudaFree(dY);
  if (!ok) return mlp_fail(m, AGB_ERR_CUDA, "agb_mlp_gradient: " + net.err);
  return AGB_OK;
}

__global__ void k_mlp_gather_rows(int rows, int width, const int* __restrict__ idx, const float* __restrict__ src,
                                  float* __restrict__ dst) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)rows * width) return;
  const int r = (int)(t / width), j = (int)(t % width);
  dst[t] = src[(int64_t)idx[r] * width + j];
}

int agb_mlp_train(agb_mlp* m, int n, const float* X, const float* Y, int epochs, int batch, float lr,
                  unsigned long long seed, double* loss_hist, double* stats) {
  if (!m || n < 1 || !X || !Y || epochs < 1 || batch < 1 || !(lr > 0.f)) return AGB_ERR_ARG;
  agb::Mlp& net = m->net;
  cudaSetDevice(net.device);
  batch = std::min(batch, n);
  float *dX = nullptr, *dY = nullptr, *bX = nullptr, *bY = nullptr;
  int* didx = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  bool ok = net.ensure_ws(batch) && cudaMalloc(&dX, (size_t)n * net.nin * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&dY, (size_t)n * net.nout * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&bX, (size_t)batch * net.nin * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&bY, (size_t)batch * net.nout * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&didx, (size_t)n * sizeof(int)) == cudaSuccess &&
            cudaMemcpyAsync(dX, X, (size_t)n * net.nin * sizeof(float), cudaMemcpyHostToDevice, net.s) == cudaSuccess &&
            cudaMemcpyAsync(dY, Y, (size_t)n * net.nout * sizeof(float), cudaMemcpyHostToDevice, net.s) == cudaSuccess;
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  std::mt19937_64 rng(seed);
  const long l0 = net.launches;
  cudaEventRecord(e0, net.s);
  for (int ep = 0; ok && ep < epochs; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    ok = cudaMemcpyAsync(didx, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, net.s) == cudaSuccess;
    double se = 0.0;
    for (int b0 = 0; ok && b0 + batch <= n; b0 += batch) {  // full batches only
      k_mlp_gather_rows<<<(unsigned)(((int64_t)batch * net.nin + 255) / 256), 256, 0, net.s>>>(batch, net.nin,
                                                                                                 didx + b0, dX, bX);
      k_mlp_gather_rows<<<(unsigned)(((int64_t)batch * net.nout + 255) / 256), 256, 0, net.s>>>(batch, net.nout,
                                                                                                  didx + b0, dY, bY);
      net.launches += 2;
      net.load_inputs(batch, bX);
      net.forward(batch, true, false);
      net.backward(batch, bY, false);
      net.adam(lr);
      se += net.loss_sum(batch);
      ok = cudaGetLastError() == cudaSuccess;
    }
    if (loss_hist) loss_hist[ep] = se / ((double)(n / batch) * batch * net.nout);
    cudaStreamSynchronize(net.s);  // the host permutation is rewritten next epoch
  }
  cudaEventRecord(e1, net.s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaFree(dX); cudaFree(dY); cudaFree(bX); cudaFree(bY); cudaFree(didx);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok) return mlp_fail(m, AGB_ERR_CUDA, "agb_mlp_train: " + net.err);
  if (stats) {
    stats[0] = ms;
    stats[1] = (double)(net.launches - l0);
    stats[2] = (double)net.step;
  }
  return AGB_OK;
}

int agb_mlp_predict(agb_mlp* m, int n, const float* X, float* Y, int split, double* device_ms) {
  if (!m || n < 0 || (n > 0 && (!X || !Y))) return AGB_ERR_ARG;
  if (n == 0) return AGB_OK;
  agb::Mlp& net = m->net;
  cudaSetDevice(net.device);
  const int chunk = std::min(n, 1 << 17);
  float *dX = nullptr, *dY = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  if (split < 0 || split > 2) return mlp_fail(m, AGB_ERR_ARG, "agb_mlp_predict: split must be 0, 1 or 2");
  bool ok = (split == 1 || net.ensure_ws(chunk)) && cudaMalloc(&dX, (size_t)n * net.nin * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&dY, (size_t)n * net.nout * sizeof(float)) == cudaSuccess &&
            cudaMemcpyAsync(dX, X, (size_t)n * net.nin * sizeof(float), cudaMemcpyHostToDevice, net.s) == cudaSuccess;
  if (ok) {
    cudaEventRecord(e0, net.s);
    if (split == 1) {  // fused split-BF16 inference on tcgen05: one kernel over all n queries
      ok = net.infer(n, dX, dY);
    } else {           // layer-by-layer GEMMs (split 2: split-BF16, 0: plain BF16 products)
      for (int r0 = 0; r0 < n; r0 += chunk) {
        const int rows = std::min(chunk, n - r0);
        net.load_inputs(rows, dX + (size_t)r0 * net.nin);
        net.forward(rows, false, split != 0);
        net.output(rows, dY + (size_t)r0 * net.nout);
      }
    }
    cudaEventRecord(e1, net.s);
    ok = ok && cudaGetLastError() == cudaSuccess &&
         cudaMemcpyAsync(Y, dY, (size_t)n * net.nout * sizeof(float), cudaMemcpyDeviceToHost, net.s) == cudaSuccess &&
         cudaStreamSynchronize(net.s) == cudaSuccess;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (device_ms) *device_ms = ms;
  }
  cudaFree(dX);
  cudaFree(dY);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok) return mlp_fail(m, AGB_ERR_CUDA, "agb_mlp_predict: " + net.err);
  return AGB_OK;
}

long long agb_mlp_launches(agb_mlp* m) { return m ? (long long)m->net.launches : 0; }

}  // extern "C"
