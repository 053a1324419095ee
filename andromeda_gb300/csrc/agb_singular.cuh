// Analytic self-element integrals of the Laplace and Stokes kernels over flat
// triangles and bilinear quads, FP64, usable on host and device.
//
// Method: Ren & Chan (2015), "Analytical evaluation of the BEM singular
// integrals for 3D Laplace and Stokes flow equations using coordinate
// transformation", EABE 53:1-8, with the tensor terms of Ravnik (2022).  The
// reference implements the same closed forms in src/mod_singInt.f90
// (si_tri_lap :127, si_tri_stk :34, si_qua_lap :172, si_qua_stk :266); the
// closed forms themselves (Eqs. 23-34 of the paper) are mathematics and are
// written here from their published statement:
//
//   the triangle is translated to its centroid, rotated into the xy plane by
//   the orthonormal frame {e1 = (p2-p1)/|.|, e2 = e3 x e1, e3 = unit normal of
//   (p3-p1) x (p2-p1)} and mapped to the reference triangle with the 2x2
//   Jacobian A = [p1-p3, p2-p3] (in-plane coordinates); a = |A_1|^2,
//   b = |A_2|^2, c = 2 A_1.A_2, and for the tensor part d,e,f per component
//   pair (xx, xy, yy).  The source sits at reference coordinate (1,0), (0,1),
//   (0,0) or the centroid (1/3,1/3).
//
// Results carry the reference's scaling: Laplace integral of 1/(4 pi r);
// Stokes integral of delta_ij/r + r_i r_j/r^3 (no 1/(8 pi)).
#pragma once
#include "agb_common.cuh"

#ifdef __CUDACC__
#define AGB_HD __host__ __device__ __forceinline__
#else
#define AGB_HD inline
#endif

namespace agb_sing {

struct RefMap {
  double a, b, c;        // metric of the map to the reference triangle
  double d[3], e[3], f[3];  // tensor coefficients for xx (0), xy (1), yy (2)
  double R[3][3];        // rows: local axes e1, e2, e3 in global coordinates
};

AGB_HD void cross3(const double* u, const double* v, double* w) {
  w[0] = u[1] * v[2] - u[2] * v[1];
  w[1] = u[2] * v[0] - u[0] * v[2];
  w[2] = u[0] * v[1] - u[1] * v[0];
}
AGB_HD void unit3(double* u) {
  double s = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  u[0] /= s; u[1] /= s; u[2] /= s;
}

// Local frame and reference-triangle metric of the triangle (p1,p2,p3).
AGB_HD RefMap ref_map(const double* p1, const double* p2, const double* p3) {
  RefMap M;
  double g[3], q1[3], q2[3], q3[3];
  for (int i = 0; i < 3; ++i) g[i] = (p1[i] + p2[i] + p3[i]) / 3.0;
  for (int i = 0; i < 3; ++i) { q1[i] = p1[i] - g[i]; q2[i] = p2[i] - g[i]; q3[i] = p3[i] - g[i]; }
  double ax1[3], ax2[3], ax3[3], e31[3];
  for (int i = 0; i < 3; ++i) { ax1[i] = q2[i] - q1[i]; e31[i] = q3[i] - q1[i]; }
  cross3(e31, ax1, ax3);   // normal direction (p3-p1) x (p2-p1)
  cross3(ax3, ax1, ax2);   // in-plane, orthogonal to ax1
  unit3(ax1); unit3(ax2); unit3(ax3);
  for (int i = 0; i < 3; ++i) { M.R[0][i] = ax1[i]; M.R[1][i] = ax2[i]; M.R[2][i] = ax3[i]; }
  // in-plane coordinates of the three vertices
  double x1 = ax1[0] * q1[0] + ax1[1] * q1[1] + ax1[2] * q1[2];
  double y1 = ax2[0] * q1[0] + ax2[1] * q1[1] + ax2[2] * q1[2];
  double x2 = ax1[0] * q2[0] + ax1[1] * q2[1] + ax1[2] * q2[2];
  double y2 = ax2[0] * q2[0] + ax2[1] * q2[1] + ax2[2] * q2[2];
  double x3 = ax1[0] * q3[0] + ax1[1] * q3[1] + ax1[2] * q3[2];
  double y3 = ax2[0] * q3[0] + ax2[1] * q3[1] + ax2[2] * q3[2];
  double j11 = x1 - x3, j12 = x2 - x3, j21 = y1 - y3, j22 = y2 - y3;
  M.a = j11 * j11 + j21 * j21;
  M.b = j12 * j12 + j22 * j22;
  M.c = 2.0 * (j11 * j12 + j21 * j22);
  M.d[0] = j11 * j11; M.e[0] = j12 * j12; M.f[0] = 2.0 * j11 * j12;   // xx
  M.d[1] = j11 * j21; M.e[1] = j12 * j22; M.f[1] = j11 * j22 + j21 * j12;  // xy
  M.d[2] = j21 * j21; M.e[2] = j22 * j22; M.f[2] = 2.0 * j21 * j22;   // yy
  return M;
}

AGB_HD double pw15(double v) { return v * sqrt(v); }

// Scalar part: integral of 1/rho over the reference triangle for the source
// at vertex 1 (1,0), vertex 2 (0,1), vertex 3 (0,0) and the centroid.
AGB_HD double scalar_part(int where, double a, double b, double c) {
  const double s = a + b - c;
  switch (where) {
    case 1: return log((2.0 * sqrt(b) * sqrt(s) + 2.0 * b - c) / (2.0 * sqrt(a) * sqrt(b) - c)) / sqrt(b);
    case 2: return log((2.0 * sqrt(a) * sqrt(s) + 2.0 * a - c) / (2.0 * sqrt(a) * sqrt(b) - c)) / sqrt(a);
    case 3: return log((2.0 * sqrt(a) * sqrt(s) + 2.0 * a - c) / (2.0 * sqrt(b) * sqrt(s) - 2.0 * b + c)) / sqrt(s);
    default: {
      const double p = 4.0 * a + b - 2.0 * c, q = a + 4.0 * b - 2.0 * c, t = a + b + c;
      double r1 = log((4.0 * a + 2.0 * b + 2.0 * sqrt(p) * sqrt(s) - 3.0 * c) /
                      (-2.0 * a - 4.0 * b + 2.0 * sqrt(q) * sqrt(s) + 3.0 * c)) / sqrt(s);
      double r2 = log((4.0 * a + 2.0 * sqrt(p) * sqrt(a) - c) / (-2.0 * a - c + 2.0 * sqrt(t) * sqrt(a))) / sqrt(a);
      double r3 = log(((4.0 * b + 2.0 * sqrt(q) * sqrt(b) - c) * (2.0 * b + 2.0 * sqrt(t) * sqrt(b) + c)) /
                      ((b + sqrt(p) * sqrt(b) - c) * (-b + sqrt(p) * sqrt(b) + c))) / sqrt(b);
      return (r1 + r2 + r3) / 3.0;
    }
  }
}

// Tensor part: integral of (rho_i rho_j)/rho^3 in reference coordinates with
// coefficients (d,e,f) of the component pair.
AGB_HD double tensor_part(int where, double a, double b, double c, double d, double e, double f) {
  const double s = a + b - c, q = 4.0 * a * b - c * c;
  const double ra = sqrt(a), rb = sqrt(b), rs = sqrt(s);
  switch (where) {
    case 1: {
      double num = 2.0 * rb * (b * rs * c * d - pw15(a) * (c * e + 2.0 * b * (e - f)) + a * rs * (c * e - 2.0 * b * f) +
                               ra * (2.0 * b * b * d + c * c * e - b * c * (d + f))) -
                   ra * rs * q * e * (log(2.0 * ra * rb - c) - log(2.0 * b + 2.0 * rb * rs - c));
      return num / (ra * pw15(b) * rs * q);
    }
    case 2: {
      double t1 = (2.0 * rb * (-2.0 * b * b * d + (a - c) * c * e + b * (2.0 * a * (e - f) + c * (d + f))) +
                   rs * q * e * (-1.0 + log(-2.0 * b + 2.0 * rb * rs + c))) / rs;
      double inner = 2.0 * pw15(b) * c * (-b + rb * rs + c) * d +
                     a * a * (4.0 * b * rs * e - 2.0 * rb * c * e + 4.0 * pw15(b) * f) +
                     a * (2.0 * b * rs * c * e + 2.0 * rb * c * c * e - rs * c * c * e + 4.0 * b * b * rb * f -
                          4.0 * b * b * rs * f - 2.0 * pw15(b) * c * (d + e + 2.0 * f)) +
                     a * rs * (-q) * e * log(-2.0 * b + 2.0 * rb * rs + c);
      double t2 = (pw15(b) * rs * (-q) * d * log(2.0 * ra * rb - c) +
                   pw15(b) * rs * q * d * log(2.0 * a + 2.0 * ra * rs - c) + ra * inner) /
                  (pw15(a) * rs);
      return (t1 + t2) / (pw15(b) * q);
    }
    case 3: {
      double L1 = log(2.0 * ra * rb + c);
      double num = -4.0 * a * b * e + c * c * e +
                   (2.0 * b * (2.0 * b * b * d + c * (c - a) * e - b * (2.0 * a * (e - f) + c * (d + f)))) / s +
                   (2.0 * ra * rb * (-2.0 * b * b * d + (a - c) * c * e + b * (2.0 * a * (e - f) + c * (d + f)))) / s +
                   (pw15(b) * q * (d + e - f) * log(2.0 * a + 2.0 * ra * rs - c)) / pw15(s) +
                   (-2.0 * pw15(b) * c * d - 2.0 * a * rb * c * e + 4.0 * a * pw15(b) * f + ra * (-q) * e * (-1.0 + L1)) / ra +
                   q * e * L1 -
                   (pw15(b) * q * (d + e - f) * log(-2.0 * b + 2.0 * rb * rs + c)) / pw15(s);
      return num / (pw15(b) * q);
    }
    default: {
      const double p = 4.0 * a + b - 2.0 * c, qq = a + 4.0 * b - 2.0 * c, t = a + b + c;
      const double rp = sqrt(p), rq = sqrt(qq), rt = sqrt(t);
      double G = 2.0 * rb * (b * c * d + a * c * e - 2.0 * a * b * f) * (rt - rp) / (a * q);
      G += 2.0 * rb * (b * (2.0 * b - c) * d - a * (2.0 * b * e + c * e - 2.0 * b * f) + c * (c * e - b * f)) * (rq - rp) /
           (s * q);
      double l1 = log((4.0 * a + 2.0 * b + 2.0 * rp * rs - 3.0 * c) / (-2.0 * a - 4.0 * b + 2.0 * rq * rs + 3.0 * c));
      G += e * rb * l1 / rs + rb * (b * d - a * e + c * e - b * f) * l1 / pw15(s);
      double l2 = log((4.0 * a + 2.0 * ra * rp - c) / (-2.0 * a - c + 2.0 * ra * rt));
      G += e * rb * l2 / ra + rb * (b * d - a * e) * l2 / pw15(a);
      double l3 = log(((4.0 * b + 2.0 * rb * rq - c) * (2.0 * b + 2.0 * rb * rt + c)) /
                      (4.0 * (b + rb * rp - c) * (-b + rb * rp + c)));
      G += e * l3 + e * log(4.0);
      return G / (3.0 * pw15(b));
    }
  }
}

// Laplace self-triangle: integral of 1/(4 pi r); `where` 1..4 as above.
AGB_HD double tri_laplace(const double* p1, const double* p2, const double* p3, double area, int where) {
  RefMap M = ref_map(p1, p2, p3);
  return 0.25 / AGB_PI * (2.0 * area) * scalar_part(where, M.a, M.b, M.c);
}

// Stokes self-triangle: G = {xx,xy,xz,yy,yz,zz}
AGB_HD void tri_stokes(const double* p1, const double* p2, const double* p3, double area, int where, double* G) {
  RefMap M = ref_map(p1, p2, p3);
  const double ff = scalar_part(where, M.a, M.b, M.c);
  const double gxx = tensor_part(where, M.a, M.b, M.c, M.d[0], M.e[0], M.f[0]);
  const double gxy = tensor_part(where, M.a, M.b, M.c, M.d[1], M.e[1], M.f[1]);
  const double gyy = tensor_part(where, M.a, M.b, M.c, M.d[2], M.e[2], M.f[2]);
  const double j = 2.0 * area;
  const double L[3][3] = {{j * (ff + gxx), j * gxy, 0.0}, {j * gxy, j * (ff + gyy), 0.0}, {0.0, 0.0, j * ff}};
  // global = R^T L R
  double o[3][3];
  for (int r = 0; r < 3; ++r)
    for (int s = 0; s < 3; ++s) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) acc += M.R[k][r] * L[k][l] * M.R[l][s];
      o[r][s] = acc;
    }
  G[0] = o[0][0]; G[1] = o[0][1]; G[2] = o[0][2]; G[3] = o[1][1]; G[4] = o[1][2]; G[5] = o[2][2];
}

AGB_HD double heron(const double* p1, const double* p2, const double* p3) {
  double a = sqrt((p1[0] - p2[0]) * (p1[0] - p2[0]) + (p1[1] - p2[1]) * (p1[1] - p2[1]) + (p1[2] - p2[2]) * (p1[2] - p2[2]));
  double b = sqrt((p3[0] - p2[0]) * (p3[0] - p2[0]) + (p3[1] - p2[1]) * (p3[1] - p2[1]) + (p3[2] - p2[2]) * (p3[2] - p2[2]));
  double c = sqrt((p1[0] - p3[0]) * (p1[0] - p3[0]) + (p1[1] - p3[1]) * (p1[1] - p3[1]) + (p1[2] - p3[2]) * (p1[2] - p3[2]));
  double s = 0.5 * (a + b + c);
  return sqrt(s * (s - a) * (s - b) * (s - c));
}

// Quad self-element: fan of triangles with the source as their first vertex
// (corner source: 2 triangles, centre source: 4), as si_qua_lap/si_qua_stk.
// where = 1..4 corner, 5 centre.
AGB_HD double quad_laplace(const double (*v)[3], int where) {
  double tot = 0.0;
  if (where == 5) {
    double m[3];
    for (int i = 0; i < 3; ++i) m[i] = 0.25 * (v[0][i] + v[1][i] + v[2][i] + v[3][i]);
    for (int k = 0; k < 4; ++k) {
      const double* b = v[k];
      const double* c = v[(k + 1) & 3];
      tot += tri_laplace(m, b, c, heron(m, b, c), 1);
    }
    return tot;
  }
  const int s = where - 1;
  const double* a = v[s];
  const double* b = v[(s + 1) & 3];
  const double* c = v[(s + 2) & 3];
  const double* d = v[(s + 3) & 3];
  tot = tri_laplace(a, b, c, heron(a, b, c), 1);
  tot += tri_laplace(a, c, d, heron(a, c, d), 1);
  return tot;
}

AGB_HD void quad_stokes(const double (*v)[3], int where, double* G) {
  double g[6];
  for (int k = 0; k < 6; ++k) G[k] = 0.0;
  if (where == 5) {
    double m[3];
    for (int i = 0; i < 3; ++i) m[i] = 0.25 * (v[0][i] + v[1][i] + v[2][i] + v[3][i]);
    for (int k = 0; k < 4; ++k) {
      const double* b = v[k];
      const double* c = v[(k + 1) & 3];
      tri_stokes(m, b, c, heron(m, b, c), 1, g);
      for (int i = 0; i < 6; ++i) G[i] += g[i];
    }
    return;
  }
  const int s = where - 1;
  const double* a = v[s];
  const double* b = v[(s + 1) & 3];
  const double* c = v[(s + 2) & 3];
  const double* d = v[(s + 3) & 3];
  tri_stokes(a, b, c, heron(a, b, c), 1, g);
  for (int i = 0; i < 6; ++i) G[i] += g[i];
  tri_stokes(a, c, d, heron(a, c, d), 1, g);
  for (int i = 0; i < 6; ++i) G[i] += g[i];
}

}  // namespace agb_sing
