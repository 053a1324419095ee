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
