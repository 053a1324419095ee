// General assembly path: every source row (u- and q-source points), triangles
// and quads, any boundary-condition mix of one subdomain.  FP64.
#pragma once
#include "agb_assembly.cuh"
#include <string>
#include <vector>

namespace agb {

// Host-side description of the subdomain numbering (sdSetUpXandB /
// StokesBigSystemXB of the reference) and of the source rows.
struct GeneralLayout {
  int kind = 1, neq = 1;
  int nn = 0, nq = 0, nsp = 0;            // subdomain nodes, elements (q-nodes), source rows
  std::vector<int> nodeList;               // sd node position -> global node
  std::vector<int> nodeWall;               // sd node position -> wall index (BCidList)
  std::vector<int> posOfNode;              // global node -> sd position or -1
  // node -> (element position, local index) adjacency, ascending element position
  std::vector<int> adj_ptr, adj_p, adj_k;
  // system numbering: rows = (source row r, equation een); T/G column maps
  int nrow = 0, nx = 0, nb = 0;
  std::vector<int> row_src, row_een;
  // per (en, sd node): target 0 none / 1 system / 2 rhs, column, sign
  std::vector<int> tmap_tgt, tmap_col;
  std::vector<double> tmap_val;
  // per (en, element position): target, column, scale (+-multi/diff)
  std::vector<int> gmap_tgt, gmap_col;
  std::vector<double> gmap_val;
  // known / unknown bookkeeping for the field solve:
  // per (en, sd node) and (en, element): 0 unknown (column in x), 1 known (column in b)
  std::vector<int> node_known, elem_known, node_xcol, node_bcol, elem_xcol, elem_bcol;
};

struct GeneralDev {
  int* adj_ptr = nullptr;
  int* adj_p = nullptr;
  int* adj_k = nullptr;
  int* nodeList = nullptr;
  int* posOfNode = nullptr;  // global node -> sd position
  int* row_src = nullptr;
  int* row_een = nullptr;
  int* tmap_tgt = nullptr;
  int* tmap_col = nullptr;
  double* tmap_val = nullptr;
  int* gmap_tgt = nullptr;
  int* gmap_col = nullptr;
  double* gmap_val = nullptr;
  void release();
  cudaError_t upload(const GeneralLayout& L);
};

// Integral matrices of all nsp source rows, row-major on the device:
// Laplace: T[1][nsp][nn] (= H), G[1][nsp][nq]; Stokes: T[9][nsp][nn]
// (Txx,Txy,Txz,Tyy,Tyz,Tzz,prTx,prTy,prTz) and G[9][nsp][nq] (Gxx..Gzz,
// prGx..prGz).  err_row[nsp] receives the reference's self-check residual.
cudaError_t general_integrals(const GeneralLayout& L, const GeneralDev& D, const ElemGeom* geom, const double* xyz,
                              const RuleDev& rule, int iqud, const IntegOpt& opt, double* T, double* G,
                              double* err_row, cudaStream_t s);

// Dense system (nrow x lda, row-major) and right-hand-side matrix (nrow x nb)
// from the integral matrices (BC routing of sdSetUpSysMrhsM_CRS / formUrow /
// formQrow).  sys and rhsM must be zeroed by the caller.
cudaError_t general_form(const GeneralLayout& L, const GeneralDev& D, const double* T, const double* G, double* sys,
                         int64_t lda, double* rhsM, cudaStream_t s);

// y[r][row] = sign * sum_col rhsM[row][col] b[r][col]
cudaError_t dense_rhs(int nrow, int nb, const double* rhsM, int k, const double* b, double sign, double* y,
                      cudaStream_t s);

// Gauss-Legendre tables of the general path's module (once per device)
cudaError_t upload_general_tables();

// FP64 -> FP32 copy of the system (for the mixed solve of a general system)
cudaError_t to_fp32(const double* a, float* b, int64_t count, cudaStream_t s);

// Surface pressure at the centroids of the subdomain's elements (pressureStokes,
// lib_Stokes.f90:4): u [3][nnodes], q [3][ne] in subdomain order, p [ne].
cudaError_t surface_pressure(int ne, const ElemGeom* geom, const RuleDev& rule, int iqud, const IntegOpt& opt,
                             const double* u, int nnodes, const double* q, double diff, double osemPi, double* p,
                             cudaStream_t s);
// Values at npts points of the domain (GetStokesDomainValue lib_Stokes.f90:3043 /
// GetSubDomainValue lib_domain.f90:210): Stokes out[4k..4k+3] = velocity,
// pressure (u [3][nnodes], q [3][ne]); Laplace out[k] (u [nnodes], q [ne]);
// err[k] the reference's check of the point.
cudaError_t domain_values(bool stokes, int ne, const ElemGeom* geom, const RuleDev& rule, int iqud, const IntegOpt& opt,
                          int npts, const double* pts, const double* xyz, const double* u, int nnodes,
                          const double* q, double diff, double osemPi, double* out, double* err, cudaStream_t s);

}  // namespace agb
