// Shared definitions of the GB300 BEM library (device + host).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#define AGB_PI 3.141592653589793238462643383

// Element types of the reference (mod_mesh.f90): 2 = 3-node triangle, 3 = 4-node quad
enum { AGB_TRI = 2, AGB_QUAD = 3 };
// Boundary-condition types (mod_mesh.f90:110)
enum { AGB_BC_FUNCTION_ = 1, AGB_BC_FLUX_ = 2, AGB_BC_CONTACT_ = 3 };

// Maximum right-hand sides carried by one block-LSQR solve.
#define AGB_MAX_RHS 8
// Maximum quadrature points per triangle (ITRI 5).
#define AGB_MAX_Q 126

// Per-element geometry, FP64 (computed on the device from the nodes).
struct ElemGeom {
  double v[4][3];   // vertices (4th unused for triangles)
  double n[3];      // unit normal (nodes 1-3), NOT multiplied by normMul
  double area;      // Heron (tri) / 8x8 Gauss (quad)
  double c[3];      // collocation point: centroid
  double multi;     // normMul of the element's wall
  int type;         // AGB_TRI / AGB_QUAD
  int nno;          // 3 / 4
  int con[4];       // 0-based node ids
  int wall;         // index of the element's wall in the subdomain list
};

static inline const char* agb_cuda_str(cudaError_t e) { return cudaGetErrorString(e); }

// Integration options of the triangle integrals:
//   sing 0: analytic self-element integrals (the reference's assembly);
//   sing 1: recursive midpoint subdivision toward the source, rdepth levels
//           (Triangle_BEMInt lib_sdBem.f90:775-852 / Triangle_StokesInt
//           lib_Stokes.f90:2251-2336 with IntRecDepth = parTriRecur); quads keep
//           the analytic scheme;
//   near_eta > 0: adaptive near-singular rule for non-singular triangles: a
//           (sub-)triangle whose centroid is closer to the source than near_eta x
//           its longest edge is split into its four children, up to near_depth
//           levels (<= 20); leaves take the regular rule.
struct IntegOpt {
  int sing = 0;
  int rdepth = 20;
  double near_eta = 0.0;
  int near_depth = 0;
  bool is_default() const { return sing == 0 && !(near_eta > 0.0 && near_depth > 0); }
};

// Packed symmetric-block layout of the Stokes single layer (mixed path): the
// six components c = xx, xy, xz, yy, yz, zz of block (i, j) are stored as
// Ap[i][j / 64][c][j % 64] -- within a row, every 64 element columns carry all
// six planes contiguously (1.5 KB runs); ldp (columns per plane) is a multiple of 64.
__host__ __device__ __forceinline__ int64_t pk_idx(int i, int c, int j, int ldp) {
  return (int64_t)i * 6 * ldp + (int64_t)(j >> 6) * 384 + c * 64 + (j & 63);
}

