// Assembly kernels of the BEM influence matrices (launch helpers).
#pragma once
#include "agb_common.cuh"

namespace agb {

// One quadrature point of a triangle: position and weight*area.
template <typename T> struct QPt;
template <> struct __align__(16) QPt<float> { float x, y, z, w; };
template <> struct __align__(32) QPt<double> { double x, y, z, w; };

struct RuleDev {
  int Q = 0;
  double* l = nullptr;  // device [3][Q] barycentric coordinates
  double* w = nullptr;  // device [Q] weights
};

// Geometry of the subdomain's elements, in subdomain order (wall-major).
cudaError_t launch_geometry(int ne, const double* xyz, const int* etype, const int* con, const int* wall_of_elem,
                            const double* normMul, ElemGeom* geom, cudaStream_t s);

// Quadrature points pts[q][ldp] (T) of all triangles (quads get zero weight;
// the fused kernels require triangle meshes).
template <typename T>
cudaError_t launch_expand_points(int ne, int ldp, const ElemGeom* geom, const RuleDev& rule, QPt<T>* pts,
                                 T* src /*[3][ldp] collocation points*/, T* nrm /*[3][ldp] normal*multi*/,
                                 cudaStream_t s);

// Stokes single-layer system for all-Dirichlet walls:
// A[3i+a][b*ne+j] = -(multi_j/mu) * int_{e_j} G_ab(x_i, y) dy  (regular part)
template <typename T>
cudaError_t launch_stokes_G(int ne, int Q, int ldp, const QPt<T>* pts, const T* src, const T* colscale, T* A,
                            int64_t lda, cudaStream_t s);
// The same single layer in the packed layout of the symmetric 3x3 blocks
// (pk_idx, plane length pldp = multiple of 64, row pitch 6 pldp floats), with
// the analytic self blocks; 2/3 of the bytes of the full matrix.  ldp is the
// pitch of the point table.
cudaError_t launch_stokes_G_packed(int ne, int Q, int ldp, int pldp, const QPt<float>* pts, const float* src,
                                   const float* colscale, float* Ap, cudaStream_t s);
cudaError_t launch_stokes_self_packed(int ne, int pldp, const ElemGeom* geom, double diff, float* Ap, cudaStream_t s);
// Self-element 3x3 blocks, analytic FP64 (Ren-Chan), written in T.
template <typename T>
cudaError_t launch_stokes_self(int ne, const ElemGeom* geom, double diff, T* A, int64_t lda, cudaStream_t s);

// Right-hand sides b(3i+a, c) = sum_nodes T_ab(i, node) u_b^c(node) (with the
// rigid-body free term) for k velocity fields given at nodes u[c][3][nnodes].
struct StokesRhsArgs {
  int ne, Q, ldp, k, nnodes;
  const void* pts;           // QPt<T>[Q][ldp] of launch_expand_points (same T as the launch)
  const ElemGeom* geom;
  const double* rule_l;      // [3][Q]
  const double* rule_w;      // [Q]
  const double* u;           // [k][3][nnodes]
  const int* active;         // [na] element positions with nonzero u
  int na;
  const unsigned char* row_active;  // [ne] 1 if the row's own element has nonzero u
  double* rhs;               // [k][3*ne] column-major
};
template <typename T>
cudaError_t launch_stokes_rhs(const StokesRhsArgs& a, cudaStream_t s);

// Laplace all-Dirichlet system: A[i][j] = (multi_j/diff) G_ij, rhs = -H u.
struct LaplaceArgs {
  int ne, Q, k, nnodes, iqud;
  const ElemGeom* geom;
  const double* rule_l;
  const double* rule_w;
  const double* u;   // [k][nnodes]
  double diff;
  double* A;         // row-major, lda
  int64_t lda;
  double* rhs;       // [k][ne]
};
cudaError_t launch_laplace_system(const LaplaceArgs& a, cudaStream_t s);

// Force and torque of tractions x (FP64, [k][3*ne] component-major blocks) on
// the elements of one wall: ft[c][6].
cudaError_t launch_force_torque(int ne, int k, const ElemGeom* geom, const double* x, int wall_index, double* ft,
                                cudaStream_t s);

}  // namespace agb
