// =============================================================================
// CPU FP64 ORACLE of the Andromeda BEM hot path -- TEST INFRASTRUCTURE ONLY.
//
// This file restates, routine by routine, the reference Fortran algorithms of
// WildSmilodon/Andromeda (src/*.f90, src/lib_lsqr.f) in plain C++ double
// precision.  It is the checker for the CUDA library in andromeda_gb300/ and
// the timed CPU baseline; it is never linked into the product.  Only the tests,
// __graft_entry__.smoke() and bench.py's CPU legs load it (liborc.so).
//
// Parity pin: the reference cannot be compiled here (no Fortran compiler, LIS
// or MPI).  The restatement is pinned against the reference's own known
// answers -- the Triangle_TestIntegration analytic values
// (src/mod_trikotnik.f90:124-154), the built-in rigid-body/free-term
// diagnostics (src/lib_sdBem.f90:566-581,714-718; src/lib_Stokes.f90:1781-1812,
// 2153-2178) and the analytic sphere resistances (src/lib_particle.f90:1961-1976)
// -- see tests/test_oracle_golden.py.
//
// Index conventions: all arrays passed in from outside are 0-based; element
// connectivity is 4 ints per element (unused 4th = -1 for triangles); wall ids
// (bcid) are the user's integers.  Dense matrices of the reference
// (Hmat(nsp,nnodes) etc.) are stored column-major exactly like Fortran.
// =============================================================================
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <string>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../andromeda_gb300/csrc/quad_tables.h"

namespace orc {

static const double PI = 3.141592653589793238462643383;  // mCommon pi (mod_common.f90:7)
enum { iFunction = 1, iFlux = 2, iContact = 3 };        // mod_mesh.f90:110

// -----------------------------------------------------------------------------
// Quadrature
// -----------------------------------------------------------------------------
struct TriRule {
  int n = 0;
  std::vector<double> l1, l2, l3, w;
};

// Triangle_GetBarycentricCoordinates (mod_trikotnik.f90:236-279)
static void bary(double x1, double y1, double z1, double x2, double y2, double z2,
                 double x3, double y3, double z3, double px, double py, double pz,
                 double& l1, double& l2, double& l3) {
  double v0x = x2 - x1, v0y = y2 - y1, v0z = z2 - z1;
  double v1x = x3 - x1, v1y = y3 - y1, v1z = z3 - z1;
  double v2x = px - x1, v2y = py - y1, v2z = pz - z1;
  double d00 = v0x * v0x + v0y * v0y + v0z * v0z;
  double d01 = v0x * v1x + v0y * v1y + v0z * v1z;
  double d11 = v1x * v1x + v1y * v1y + v1z * v1z;
  double d20 = v2x * v0x + v2y * v0y + v2z * v0z;
  double d21 = v2x * v1x + v2y * v1y + v2z * v1z;
  double denom = d00 * d11 - d01 * d01;
  l1 = (d11 * d20 - d01 * d21) / denom;
  l2 = (d00 * d21 - d01 * d20) / denom;
  l3 = 1.0 - l1 - l2;
}

// Triangle_IntegrationInit + WandzuratXiaoBary (mod_trikotnik.f90:282-781)
static TriRule wx_rule(int itri) {
  TriRule r;
  if (itri < 1 || itri > 5) return r;
  const int o0 = agb_tables::kWxOrbitOffset[itri - 1], o1 = agb_tables::kWxOrbitOffset[itri];
  const double x1 = -0.5, y1 = +0.5 * std::sqrt(3.0), x2 = -0.5, y2 = -0.5 * std::sqrt(3.0), x3 = 1.0, y3 = 0.0;
  const double pi = 4.0 * std::atan(1.0);
  const double s = std::sin(2.0 / 3.0 * pi), c = std::cos(2.0 / 3.0 * pi);
  const double s4 = std::sin(4.0 / 3.0 * pi), c4 = std::cos(4.0 / 3.0 * pi);
  std::vector<double> X, Y;
  for (int j = o0; j < o1; ++j) {
    const auto& ob = agb_tables::kWxOrbits[j];
    auto push3 = [&](double x, double y, double cc, double ss) {
      double xa = x, ya = y;
      double xb = xa * cc - ya * ss, yb = -xa * ss - ya * cc;
      double xc = xb * cc + yb * ss, yc = -xb * ss + yb * cc;
      X.push_back(xa); Y.push_back(ya); r.w.push_back(ob.w);
      X.push_back(xb); Y.push_back(yb); r.w.push_back(ob.w);
      X.push_back(xc); Y.push_back(yc); r.w.push_back(ob.w);
    };
    if (ob.m == 1) {
      X.push_back(ob.x); Y.push_back(ob.y); r.w.push_back(ob.w);
    } else if (ob.m == 3) {
      push3(ob.x, ob.y, c, s);
    } else if (ob.m == 6) {
      push3(ob.x, ob.y, c, s);
      push3(ob.x, -ob.y, c4, s4);
    }
  }
  r.n = (int)X.size();
  r.l1.resize(r.n); r.l2.resize(r.n); r.l3.resize(r.n);
  for (int i = 0; i < r.n; ++i)
    bary(x1, y1, 0.0, x2, y2, 0.0, x3, y3, 0.0, X[i], Y[i], 0.0, r.l1[i], r.l2[i], r.l3[i]);
  return r;
}

// Gauss table (mod_gauss.f90:33-393), 1-based ranges.
static inline double GI(int i) { return agb_tables::kGaussGi[i - 1]; }
static inline double OME(int i) { return agb_tables::kGaussOme[i - 1]; }

// Triangle_Area, Heron (mod_trikotnik.f90:786-802) == tri_area (mod_singInt.f90:394-413)
static double tri_area(double x1, double y1, double z1, double x2, double y2, double z2,
                       double x3, double y3, double z3) {
  double a = std::sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2) + (z1 - z2) * (z1 - z2));
  double b = std::sqrt((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2) + (z3 - z2) * (z3 - z2));
  double c = std::sqrt((x1 - x3) * (x1 - x3) + (y1 - y3) * (y1 - y3) + (z1 - z3) * (z1 - z3));
  double p = 0.5 * (a + b + c);
  return std::sqrt(p * (p - a) * (p - b) * (p - c));
}

// -----------------------------------------------------------------------------
// Ren & Chan (2015) / Ravnik (2022) analytic singular integrals
// (mod_singInt.f90:34-1157)
// -----------------------------------------------------------------------------
static double sq(double v) { return std::sqrt(v); }
static double p15(double v) { return std::pow(v, 1.5); }

static double getXi100(double a, double b, double c) {
  double d = 2.0 * sq(b) * sq(a + b - c) + 2.0 * b - c;
  double e = 2.0 * sq(a) * sq(b) - c;
  return std::log(d / e) / sq(b);
}
static double getXi010(double a, double b, double c) {
  double d = 2.0 * sq(a) * sq(a + b - c) + 2.0 * a - c;
  double e = 2.0 * sq(a) * sq(b) - c;
  return std::log(d / e) / sq(a);
}
static double getXi000(double a, double b, double c) {
  double d = 2.0 * sq(a) * sq(a + b - c) + 2.0 * a - c;
  double e = 2.0 * sq(b) * sq(a + b - c) - 2.0 * b + c;
  return std::log(d / e) / sq(a + b - c);
}
static double getXi13130(double a, double b, double c) {
  double d = 4.0 * a + 2.0 * b + 2.0 * sq(4.0 * a + b - 2.0 * c) * sq(a + b - c) - 3.0 * c;
  double e = -2.0 * a - 4.0 * b + 2.0 * sq(a + 4.0 * b - 2.0 * c) * sq(a + b - c) + 3.0 * c;
  double t1 = std::log(d / e) / sq(a + b - c);
  d = 4.0 * a + 2.0 * sq(4.0 * a + b - 2.0 * c) * sq(a) - c;
  e = -2.0 * a - c + 2.0 * sq(a + b + c) * sq(a);
  double t2 = std::log(d / e) / sq(a);
  d = (4.0 * b + 2.0 * sq(a + 4.0 * b - 2.0 * c) * sq(b) - c) * (2.0 * b + 2.0 * sq(a + b + c) * sq(b) + c);
  e = (b + sq(4.0 * a + b - 2.0 * c) * sq(b) - c) * (-b + sq(4.0 * a + b - 2.0 * c) * sq(b) + c);
  double t3 = std::log(d / e) / sq(b);
  return (t1 + t2 + t3) / 3.0;
}
// Eq. (34) of Ren & Chan: tensor part for the centroid source (getXi13130G)
static double getXi13130G(double a, double b, double c, double d, double e, double f) {
  double G = 0.0, st, im;
  st = 2.0 * sq(b) * (b * c * d + a * c * e - 2.0 * a * b * f) * (sq(a + b + c) - sq(4.0 * a + b - 2.0 * c));
  im = a * (4.0 * a * b - c * c);
  G += st / im;
  st = 2.0 * sq(b) * (b * (2.0 * b - c) * d - a * (2.0 * b * e + c * e - 2.0 * b * f) + c * (c * e - b * f)) *
       (sq(a + 4.0 * b - 2.0 * c) - sq(4.0 * a + b - 2.0 * c));
  im = (a + b - c) * (4.0 * a * b - c * c);
  G += st / im;
  st = 4.0 * a + 2.0 * b + 2.0 * sq(4.0 * a + b - 2.0 * c) * sq(a + b - c) - 3.0 * c;
  im = -2.0 * a - 4.0 * b + 2.0 * sq(a + 4.0 * b - 2.0 * c) * sq(a + b - c) + 3.0 * c;
  G += e * sq(b) * std::log(st / im) / sq(a + b - c);
  G += sq(b) * (b * d - a * e + c * e - b * f) * std::log(st / im) / p15(a + b - c);
  st = 4.0 * a + 2.0 * sq(a) * sq(4.0 * a + b - 2.0 * c) - c;
  im = -2.0 * a - c + 2.0 * sq(a) * sq(a + b + c);
  G += e * sq(b) * std::log(st / im) / sq(a);
  G += sq(b) * (b * d - a * e) * std::log(st / im) / p15(a);
  st = (4.0 * b + 2.0 * sq(b) * sq(a + 4.0 * b - 2.0 * c) - c) * (2.0 * b + 2.0 * sq(b) * sq(a + b + c) + c);
  im = 4.0 * (b + sq(b) * sq(4.0 * a + b - 2.0 * c) - c) * (-b + sq(b) * sq(4.0 * a + b - 2.0 * c) + c);
  G += e * std::log(st / im);
  G += e * std::log(4.0);
  G /= (3.0 * p15(b));
  return G;
}
static double getXi000G(double a, double b, double c, double d, double e, double f) {
  double abc = a + b - c, q = 4 * a * b - c * c;
  return (-4 * a * b * e + c * c * e +
          (2 * b * (2 * b * b * d + c * (-a + c) * e - b * (2 * a * (e - f) + c * (d + f)))) / abc +
          (2 * sq(a) * sq(b) * (-2 * b * b * d + (a - c) * c * e + b * (2 * a * (e - f) + c * (d + f)))) / abc +
          (p15(b) * q * (d + e - f) * std::log(2 * a + 2 * sq(a) * sq(abc) - c)) / p15(abc) +
          (-2 * p15(b) * c * d - 2 * a * sq(b) * c * e + 4 * a * p15(b) * f +
           sq(a) * (-4 * a * b + c * c) * e * (-1 + std::log(2 * sq(a) * sq(b) + c))) / sq(a) +
          4 * a * b * e * std::log(2 * sq(a) * sq(b) + c) - c * c * e * std::log(2 * sq(a) * sq(b) + c) -
          (p15(b) * q * (d + e - f) * std::log(-2 * b + 2 * sq(b) * sq(abc) + c)) / p15(abc)) /
         (p15(b) * q);
}
static double getXi100G(double a, double b, double c, double d, double e, double f) {
  double abc = a + b - c, q = 4 * a * b - c * c;
  return (2 * sq(b) * (b * sq(abc) * c * d - p15(a) * (c * e + 2 * b * (e - f)) + a * sq(abc) * (c * e - 2 * b * f) +
                       sq(a) * (2 * b * b * d + c * c * e - b * c * (d + f))) -
          sq(a) * sq(abc) * q * e * (std::log(2 * sq(a) * sq(b) - c) - std::log(2 * b + 2 * sq(b) * sq(abc) - c))) /
         (sq(a) * p15(b) * sq(abc) * q);
}
static double getXi010G(double a, double b, double c, double d, double e, double f) {
  double abc = a + b - c, q = 4 * a * b - c * c;
  double t1 = (2 * sq(b) * (-2 * b * b * d + (a - c) * c * e + b * (2 * a * (e - f) + c * (d + f))) +
               sq(abc) * q * e * (-1 + std::log(-2 * b + 2 * sq(b) * sq(abc) + c))) / sq(abc);
  double t2 =
      (p15(b) * sq(abc) * (-4 * a * b + c * c) * d * std::log(2 * sq(a) * sq(b) - c) +
       p15(b) * sq(abc) * q * d * std::log(2 * a + 2 * sq(a) * sq(abc) - c) +
       sq(a) * (2 * p15(b) * c * (-b + sq(b) * sq(abc) + c) * d +
                a * a * (4 * b * sq(abc) * e - 2 * sq(b) * c * e + 4 * p15(b) * f) +
                a * (2 * b * sq(abc) * c * e + 2 * sq(b) * c * c * e - sq(abc) * c * c * e + 4 * std::pow(b, 2.5) * f -
                     4 * b * b * sq(abc) * f - 2 * p15(b) * c * (d + e + 2 * f)) +
                a * sq(abc) * (-4 * a * b + c * c) * e * std::log(-2 * b + 2 * sq(b) * sq(abc) + c))) /
      (p15(a) * sq(abc));
  return (t1 + t2) / (p15(b) * q);
}

// siCrossProduct a = b x c (mod_singInt.f90:1114-1123)
static void cross(double a[3], const double b[3], const double c[3]) {
  a[0] = b[1] * c[2] - b[2] * c[1];
  a[1] = -b[0] * c[2] + b[2] * c[0];
  a[2] = b[0] * c[1] - b[1] * c[0];
}
// siNormVector (mod_singInt.f90:1141-1155); its uninitialised accumulator is
// taken as zero (the value an optimising gfortran build produces).
static void normv(double a[3]) {
  double n = 0.0;
  for (int i = 0; i < 3; ++i) n += a[i] * a[i];
  n = std::sqrt(n);
  for (int i = 0; i < 3; ++i) a[i] /= n;
}
// getMrot (mod_singInt.f90:905-946): rows of Mrot are the in-plane unit
// vectors ov1, ov2 and the normal ov3.
static void getMrot(const double rr1[3], const double rr2[3], const double rr3[3], double M[3][3]) {
  double ov1[3], ov2[3], ov3[3], ov4[3];
  for (int i = 0; i < 3; ++i) { ov1[i] = rr2[i] - rr1[i]; ov4[i] = rr3[i] - rr1[i]; }
  cross(ov3, ov4, ov1);
  cross(ov2, ov3, ov1);
  normv(ov1); normv(ov2); normv(ov3);
  for (int j = 0; j < 3; ++j) { M[0][j] = ov1[j]; M[1][j] = ov2[j]; M[2][j] = ov3[j]; }
}
// getrcABC / getABCDEF (mod_singInt.f90:1010-1108) + getABC/getDEF (:952-1004)
struct Frame { double a, b, c, dxx, exx, fxx, dxy, exy, fxy, dyy, eyy, fyy; double M[3][3]; };
static Frame getFrame(const double v[9]) {
  Frame F;
  double r1[3] = {v[0], v[1], v[2]}, r2[3] = {v[3], v[4], v[5]}, r3[3] = {v[6], v[7], v[8]};
  double cc[3], rr1[3], rr2[3], rr3[3], q1[3], q2[3], q3[3];
  for (int i = 0; i < 3; ++i) cc[i] = (r1[i] + r2[i] + r3[i]) / 3.0;
  for (int i = 0; i < 3; ++i) { rr1[i] = r1[i] - cc[i]; rr2[i] = r2[i] - cc[i]; rr3[i] = r3[i] - cc[i]; }
  getMrot(rr1, rr2, rr3, F.M);
  for (int i = 0; i < 3; ++i) {
    q1[i] = F.M[i][0] * rr1[0] + F.M[i][1] * rr1[1] + F.M[i][2] * rr1[2];
    q2[i] = F.M[i][0] * rr2[0] + F.M[i][1] * rr2[1] + F.M[i][2] * rr2[2];
    q3[i] = F.M[i][0] * rr3[0] + F.M[i][1] * rr3[1] + F.M[i][2] * rr3[2];
  }
  double A11 = q1[0] - q3[0], A12 = q2[0] - q3[0], A21 = q1[1] - q3[1], A22 = q2[1] - q3[1];
  F.a = A11 * A11 + A21 * A21;
  F.b = A12 * A12 + A22 * A22;
  F.c = 2.0 * (A11 * A12 + A21 * A22);
  F.dxx = A11 * A11; F.exx = A12 * A12; F.fxx = 2.0 * A11 * A12;
  F.dyy = A21 * A21; F.eyy = A22 * A22; F.fyy = 2.0 * A21 * A22;
  F.dxy = A11 * A21; F.exy = A12 * A22; F.fxy = A11 * A22 + A21 * A12;
  return F;
}
// si_tri_lap (mod_singInt.f90:127-167)
static double si_tri_lap(const double v[9], double area, int isrc) {
  Frame F = getFrame(v);
  double f;
  switch (isrc) {
    case 1: f = getXi100(F.a, F.b, F.c); break;
    case 2: f = getXi010(F.a, F.b, F.c); break;
    case 3: f = getXi000(F.a, F.b, F.c); break;
    case 4: f = getXi13130(F.a, F.b, F.c); break;
    default: fprintf(stderr, "Error in si_tri_lap\n"); return NAN;
  }
  double jac = 2.0 * area;
  return 0.25 / PI * jac * f;
}
// si_tri_stk (mod_singInt.f90:34-123): G = {xx,xy,xz,yy,yz,zz}
static void si_tri_stk(const double v[9], double area, int isrc, double G[6]) {
  Frame F = getFrame(v);
  double ff, gxx, gxy, gyy;
  double (*fg)(double, double, double, double, double, double) = nullptr;
  switch (isrc) {
    case 1: ff = getXi100(F.a, F.b, F.c); fg = getXi100G; break;
    case 2: ff = getXi010(F.a, F.b, F.c); fg = getXi010G; break;
    case 3: ff = getXi000(F.a, F.b, F.c); fg = getXi000G; break;
    case 4: ff = getXi13130(F.a, F.b, F.c); fg = getXi13130G; break;
    default: fprintf(stderr, "Error in si_tri_stk\n"); for (int i = 0; i < 6; ++i) G[i] = NAN; return;
  }
  gxx = fg(F.a, F.b, F.c, F.dxx, F.exx, F.fxx);
  gxy = fg(F.a, F.b, F.c, F.dxy, F.exy, F.fxy);
  gyy = fg(F.a, F.b, F.c, F.dyy, F.eyy, F.fyy);
  double mat[3][3] = {{2.0 * area * (ff + gxx), 2.0 * area * gxy, 0.0},
                      {2.0 * area * gxy, 2.0 * area * (ff + gyy), 0.0},
                      {0.0, 0.0, 2.0 * area * ff}};
  // mat = MrotT * mat * Mrot
  double t[3][3], o[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += F.M[k][i] * mat[k][j];
      t[i][j] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += t[i][k] * F.M[k][j];
      o[i][j] = s;
    }
  G[0] = o[0][0]; G[1] = o[0][1]; G[2] = o[0][2]; G[3] = o[1][1]; G[4] = o[1][2]; G[5] = o[2][2];
}
static void tri9(double* v, const double* a, const double* b, const double* c) {
  for (int i = 0; i < 3; ++i) { v[i] = a[i]; v[3 + i] = b[i]; v[6 + i] = c[i]; }
}
// si_qua_lap (mod_singInt.f90:172-260): split at the source vertex/centre
static double si_qua_lap(const double q[12], int isrc) {
  const double* P[5];
  double p5[3];
  for (int k = 0; k < 4; ++k) P[k] = q + 3 * k;
  double v[9];
  auto one = [&](int i, int j, int k) {
    tri9(v, P[i], P[j], P[k]);
    double ar = tri_area(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8]);
    return si_tri_lap(v, ar, 1);
  };
  switch (isrc) {
    case 1: return one(0, 1, 2) + one(0, 2, 3);
    case 2: return one(1, 2, 3) + one(1, 3, 0);
    case 3: return one(2, 3, 0) + one(2, 0, 1);
    case 4: return one(3, 0, 1) + one(3, 1, 2);
    case 5: {
      for (int i = 0; i < 3; ++i) p5[i] = 0.25 * (q[i] + q[3 + i] + q[6 + i] + q[9 + i]);
      P[4] = p5;
      double s1 = one(4, 0, 1), s2 = one(4, 1, 2), s3 = one(4, 2, 3), s4 = one(4, 3, 0);
      return s1 + s2 + s3 + s4;
    }
  }
  fprintf(stderr, "ERROR in si_qua_lap\n");
  return NAN;
}
// si_qua_stk (mod_singInt.f90:266-387)
static void si_qua_stk(const double q[12], int isrc, double G[6]) {
  const double* P[5];
  double p5[3];
  for (int k = 0; k < 4; ++k) P[k] = q + 3 * k;
  double v[9], g1[6], g2[6], g3[6], g4[6];
  auto one = [&](int i, int j, int k, double* g) {
    tri9(v, P[i], P[j], P[k]);
    double ar = tri_area(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8]);
    si_tri_stk(v, ar, 1, g);
  };
  switch (isrc) {
    case 1: one(0, 1, 2, g1); one(0, 2, 3, g2); break;
    case 2: one(1, 2, 3, g1); one(1, 3, 0, g2); break;
    case 3: one(2, 3, 0, g1); one(2, 0, 1, g2); break;
    case 4: one(3, 0, 1, g1); one(3, 1, 2, g2); break;
    case 5:
      for (int i = 0; i < 3; ++i) p5[i] = 0.25 * (q[i] + q[3 + i] + q[6 + i] + q[9 + i]);
      P[4] = p5;
      one(4, 0, 1, g1); one(4, 1, 2, g2); one(4, 2, 3, g3); one(4, 3, 0, g4);
      for (int i = 0; i < 6; ++i) G[i] = g1[i] + g2[i] + g3[i] + g4[i];
      return;
    default: fprintf(stderr, "ERROR in si_qua_stk\n"); for (int i = 0; i < 6; ++i) G[i] = NAN; return;
  }
  for (int i = 0; i < 6; ++i) G[i] = g1[i] + g2[i];
}

// -----------------------------------------------------------------------------
// Kernels and regular integrators
// -----------------------------------------------------------------------------
// BemKernel (lib_sdBem.f90:911-936)
static inline void bem_kernel(double sx, double sy, double sz, double fx, double fy, double fz,
                              double nx, double ny, double nz, double& G, double& H) {
  double RX = -fx + sx, RY = -fy + sy, RZ = -fz + sz;
  double RA = std::sqrt(RX * RX + RY * RY + RZ * RZ);
  double IRA2 = 1.0 / (RA * RA);
  G = 0.25 / (PI * RA);
  H = (RX * nx + RY * ny + RZ * nz) * IRA2 * G;
}
// -----------------------------------------------------------------------------
// Sub-triangles.  A sub-triangle of an element is held as the barycentric
// coordinates (in the element) of its three vertices, B[k][j].  A quadrature
// point with sub-triangle barycentrics l maps to the element barycentrics
// L_j = sum_k l_k B[k][j]; the position is sum_j L_j v_j and the linear shape
// weights are L_j (the element's).  The midpoint split of
// Triangle_BEMInt / Triangle_StokesInt (lib_sdBem.f90:775-852,
// lib_Stokes.f90:2251-2336): with the edge midpoints 4 = (1+2)/2, 5 = (2+3)/2,
// 6 = (1+3)/2, child 0 = (1,4,6), 1 = (4,2,5), 2 = (6,5,3), 3 = (4,5,6).
// Children have a quarter of the parent's area and half its edges.
// -----------------------------------------------------------------------------
struct Bary { double b[3][3]; };
static Bary bary_identity() {
  Bary B;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j) B.b[k][j] = (k == j) ? 1.0 : 0.0;
  return B;
}
static Bary sub_child(const Bary& P, int d) {
  double m4[3], m5[3], m6[3];
  for (int j = 0; j < 3; ++j) {
    m4[j] = 0.5 * (P.b[0][j] + P.b[1][j]);
    m5[j] = 0.5 * (P.b[2][j] + P.b[1][j]);
    m6[j] = 0.5 * (P.b[0][j] + P.b[2][j]);
  }
  Bary C;
  for (int j = 0; j < 3; ++j) {
    switch (d) {
      case 0: C.b[0][j] = P.b[0][j]; C.b[1][j] = m4[j]; C.b[2][j] = m6[j]; break;
      case 1: C.b[0][j] = m4[j]; C.b[1][j] = P.b[1][j]; C.b[2][j] = m5[j]; break;
      case 2: C.b[0][j] = m6[j]; C.b[1][j] = m5[j]; C.b[2][j] = P.b[2][j]; break;
      default: C.b[0][j] = m4[j]; C.b[1][j] = m5[j]; C.b[2][j] = m6[j]; break;
    }
  }
  return C;
}

// Integration options of the triangle integrals.
//   sing 0: analytic self-element integrals (the reference's assembly);
//   sing 1: recursive midpoint subdivision toward the source, rdepth levels
//           (Triangle_BEMInt / Triangle_StokesInt with IntRecDepth = parTriRecur,
//           the alternative left commented out at lib_sdBem.f90:510,668 and
//           lib_Stokes.f90:1697,2030; live in lib_domain.f90:286).  Quads keep
//           the analytic scheme.
//   near_eta > 0: adaptive near-singular rule for non-singular triangles (no
//           reference counterpart): a (sub-)triangle whose centroid lies closer
//           to the source than near_eta x its longest edge is split into its four
//           children, up to near_depth levels; leaves take the regular rule.
struct IntegOpt {
  int sing = 0;
  int rdepth = 20;
  double near_eta = 0.0;
  int near_depth = 0;
};

// Visits the sub-triangles of element v for source s in the order of the
// reference's recursion (children 0..3, depth first) and calls
// rule(B, area_of_sub, skip_centroid).  skip_centroid is set for the last piece
// of a centroid-source recursion: the source is that piece's centroid, and a
// rule with a centroid point (ITRI 1, 2, 4) would divide by r = 0 there (the
// reference's Triangle_BEMInt does); that one point is left out.
template <class F>
static void tri_walk(const IntegOpt& o, const double v[9], const double s[3], double area, int isrc, F&& rule) {
  if (isrc) {
    // Triangle_BEMInt: only the child holding the source (vertex isrc, or the
    // centre child for the centroid) recurses; the final piece is integrated
    // with the regular rule.
    const int ks = isrc - 1;
    Bary B = bary_identity();
    double a = area;
    for (int lev = 0; lev < o.rdepth; ++lev) {
      for (int d = 0; d < ks; ++d) rule(sub_child(B, d), 0.25 * a, false);
      B = sub_child(B, ks);
      a *= 0.25;
    }
    rule(B, a, isrc == 4);
    for (int lev = o.rdepth - 1; lev >= 0; --lev) {
      Bary Bl = bary_identity();
      double al = area;
      for (int t = 0; t < lev; ++t) { Bl = sub_child(Bl, ks); al *= 0.25; }
      for (int d = ks + 1; d < 4; ++d) rule(sub_child(Bl, d), 0.25 * al, false);
    }
    return;
  }
  if (o.near_eta > 0.0 && o.near_depth > 0) {
    auto edge = [&](int p, int q) {
      const double dx = v[3 * p] - v[3 * q], dy = v[3 * p + 1] - v[3 * q + 1], dz = v[3 * p + 2] - v[3 * q + 2];
      return std::sqrt(dx * dx + dy * dy + dz * dz);
    };
    const double diam = std::max(edge(0, 1), std::max(edge(1, 2), edge(2, 0)));
    // depth-first stack of sub-triangles: 2 bits per level (child index) + the level in bits 58..63
    uint64_t stack[64];
    int top = 0;
    stack[top++] = 0;
    while (top > 0) {
      const uint64_t e = stack[--top];
      const int lev = (int)(e >> 58);
      Bary B = bary_identity();
      double a = area, h = diam;
      for (int t = 0; t < lev; ++t) {
        B = sub_child(B, (int)((e >> (2 * t)) & 3u));
        a *= 0.25;
        h *= 0.5;
      }
      double c[3] = {0.0, 0.0, 0.0};
      for (int j = 0; j < 3; ++j) {
        const double Lc = (B.b[0][j] + B.b[1][j] + B.b[2][j]) / 3.0;
        for (int i = 0; i < 3; ++i) c[i] += Lc * v[3 * j + i];
      }
      const double d = std::sqrt((s[0] - c[0]) * (s[0] - c[0]) + (s[1] - c[1]) * (s[1] - c[1]) +
                                 (s[2] - c[2]) * (s[2] - c[2]));
      if (lev < o.near_depth && d < o.near_eta * h) {
        for (int ch = 3; ch >= 0; --ch) stack[top++] = (e & ((1ull << 58) - 1)) | ((uint64_t)ch << (2 * lev)) |
                                                       ((uint64_t)(lev + 1) << 58);
      } else {
        rule(B, a, false);
      }
    }
    return;
  }
  rule(bary_identity(), area, false);
}
// the centroid point of a symmetric rule: l1 = l2 = l3
static inline bool is_centroid_point(double l1, double l2, double l3) {
  return std::fabs(l1 - l2) < 1e-12 && std::fabs(l2 - l3) < 1e-12;
}

// Triangle_3DLapInt (lib_sdBem.f90:859-905) over the sub-triangle B;
// accumulates into out[0..3] (G, H at the three element nodes)
static void tri_lap_sub(const TriRule& R, const double v[9], const Bary& B, const double s[3], const double n[3],
                        double area, double out[4], bool skip_centroid = false) {
  for (int i = 0; i < R.n; ++i) {
    if (skip_centroid && is_centroid_point(R.l1[i], R.l2[i], R.l3[i])) continue;
    double L[3];
    for (int j = 0; j < 3; ++j) L[j] = R.l1[i] * B.b[0][j] + R.l2[i] * B.b[1][j] + R.l3[i] * B.b[2][j];
    double x = L[0] * v[0] + L[1] * v[3] + L[2] * v[6];
    double y = L[0] * v[1] + L[1] * v[4] + L[2] * v[7];
    double z = L[0] * v[2] + L[1] * v[5] + L[2] * v[8];
    double G, H;
    bem_kernel(s[0], s[1], s[2], x, y, z, n[0], n[1], n[2], G, H);
    out[0] += R.w[i] * G * area;
    out[1] += R.w[i] * H * area * L[0];
    out[2] += R.w[i] * H * area * L[1];
    out[3] += R.w[i] * H * area * L[2];
  }
}
static void tri_lap_regular(const TriRule& R, const double v[9], const double s[3], const double n[3],
                            double area, double out[4]) {
  tri_lap_sub(R, v, bary_identity(), s, n, area, out);
}
// Quad_BEMIntNum (lib_intAna.f90:219-344); out[0]=G, out[1..4]=H at nodes.
// ndiv > 0 replaces the edge-length subdivision by ndiv x ndiv cells: 1 is the
// regular branch of Quad_BEMInt (lib_int.f90:329-601, ndivXi = ndivEt = 1).
static void quad_lap_regular(int iqud, const double q[12], const double s[3], double multi, double out[5],
                             int ndiv = 0) {
  const double *P1 = q, *P2 = q + 3, *P3 = q + 6, *P4 = q + 9;
  int ng1 = agb_tables::kGaussNg1[iqud - 1], ng2 = agb_tables::kGaussNg2[iqud - 1];
  for (int k = 0; k < 5; ++k) out[k] = 0.0;
  const double minedge = 1.0;
  auto dist = [](const double* a, const double* b) {
    return std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
  };
  double d1 = dist(P1, P2), d2 = dist(P2, P3), d3 = dist(P3, P4), d4 = dist(P4, P1);
  double d13 = std::max(d1, d3), d24 = std::max(d2, d4);
  int ndx = std::max(2, (int)(d13 / minedge + 0.5));
  int nde = std::max(2, (int)(d24 / minedge + 0.5));
  if (ndiv > 0) ndx = nde = ndiv;
  for (int ix = 1; ix <= ndx; ++ix)
    for (int ie = 1; ie <= nde; ++ie) {
      double a = -1.0 + (ix - 1) * 2.0 / ndx, b = -1.0 + ix * 2.0 / ndx;
      double c = -1.0 + (ie - 1) * 2.0 / nde, d = -1.0 + ie * 2.0 / nde;
      double dex = 0.25 * (b - a) * (d - c);
      for (int i = ng1; i <= ng2; ++i) {
        double gii = a + 0.5 * (GI(i) + 1.0) * (b - a);
        double e1m = 1.0 - gii, e1p = 1.0 + gii;
        for (int j = ng1; j <= ng2; ++j) {
          double gij = c + 0.5 * (GI(j) + 1.0) * (d - c);
          double e2m = 1.0 - gij, e2p = 1.0 + gij;
          double f4[4] = {0.25 * e1m * e2m, 0.25 * e1p * e2m, 0.25 * e1p * e2p, 0.25 * e1m * e2p};
          double X[3], KS[3], ET[3];
          for (int k = 0; k < 3; ++k) {
            X[k] = f4[0] * P1[k] + f4[1] * P2[k] + f4[2] * P3[k] + f4[3] * P4[k];
            KS[k] = 0.25 * (-e2m * P1[k] + e2m * P2[k] + e2p * P3[k] - e2p * P4[k]);
            ET[k] = 0.25 * (-e1m * P1[k] - e1p * P2[k] + e1p * P3[k] + e1m * P4[k]);
          }
          double anx = KS[1] * ET[2] - ET[1] * KS[2];
          double any = ET[0] * KS[2] - KS[0] * ET[2];
          double anz = KS[0] * ET[1] - ET[0] * KS[1];
          double ajac = 1.0 / std::sqrt(anx * anx + any * any + anz * anz);
          double n1 = multi * anx * ajac, n2 = multi * any * ajac, n3 = multi * anz * ajac;
          ajac = dex * OME(i) * OME(j) / ajac;
          double G, H;
          bem_kernel(s[0], s[1], s[2], X[0], X[1], X[2], n1, n2, n3, G, H);
          for (int k = 0; k < 4; ++k) out[1 + k] += H * ajac * f4[k];
          out[0] += G * ajac;
        }
      }
    }
}

// StokesKernel (lib_Stokes.f90:2450-2544).  G,T as 3x3; prG, prT 3-vectors.
static inline void stokes_kernel(const double s[3], const double f[3], const double n[3], double G[3][3],
                                 double T[3][3], double prG[3], double prT[3]) {
  double rx = f[0] - s[0], ry = f[1] - s[1], rz = f[2] - s[2];
  double rxx = rx * rx, rxy = rx * ry, rxz = rx * rz, ryy = ry * ry, ryz = ry * rz, rzz = rz * rz;
  double ir2 = 1.0 / (rxx + ryy + rzz);
  double ir = std::sqrt(ir2);
  double ir3 = ir2 * ir;
  G[0][0] = ir * (1.0 + rxx * ir2); G[0][1] = rxy * ir3; G[0][2] = rxz * ir3;
  G[1][0] = G[0][1]; G[1][1] = ir * (1.0 + ryy * ir2); G[1][2] = ryz * ir3;
  G[2][0] = G[0][2]; G[2][1] = G[1][2]; G[2][2] = ir * (1.0 + rzz * ir2);
  double c = -6.0 * ir2 * ir3 * (rx * n[0] + ry * n[1] + rz * n[2]);
  T[0][0] = c * rxx; T[0][1] = c * rxy; T[0][2] = c * rxz;
  T[1][0] = T[0][1]; T[1][1] = c * ryy; T[1][2] = c * ryz;
  T[2][0] = T[0][2]; T[2][1] = T[1][2]; T[2][2] = c * rzz;
  c = 2.0 * ir3;
  prG[0] = c * rx; prG[1] = c * ry; prG[2] = c * rz;
  c = 4.0 * ir3;
  prT[0] = c * ((-1.0 + 3.0 * rxx * ir2) * n[0] + 3.0 * rxy * ir2 * n[1] + 3.0 * rxz * ir2 * n[2]);
  prT[1] = c * (3.0 * rxy * ir2 * n[0] + (-1.0 + 3.0 * ryy * ir2) * n[1] + 3.0 * ryz * ir2 * n[2]);
  prT[2] = c * (3.0 * rxz * ir2 * n[0] + 3.0 * ryz * ir2 * n[1] + (-1.0 + 3.0 * rzz * ir2) * n[2]);
}

// Per-element Stokes result: G[6] (xx,xy,xz,yy,yz,zz), prG[3],
// T[6][4] (component x local node), prT[3][4].
struct StkElem {
  double G[6], prG[3], T[6][4], prT[3][4];
  void zero() { std::memset(this, 0, sizeof(*this)); }
};
static const int kSym[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};

// Triangle_3DStokesInt (lib_Stokes.f90:2341-2446) over the sub-triangle B
static void tri_stk_sub(const TriRule& R, const double v[9], const Bary& B, const double s[3], const double n[3],
                        double area, StkElem& E, bool skip_centroid = false) {
  double G[3][3], T[3][3], prG[3], prT[3], f[3];
  for (int i = 0; i < R.n; ++i) {
    if (skip_centroid && is_centroid_point(R.l1[i], R.l2[i], R.l3[i])) continue;
    double l[3];
    for (int j = 0; j < 3; ++j) l[j] = R.l1[i] * B.b[0][j] + R.l2[i] * B.b[1][j] + R.l3[i] * B.b[2][j];
    f[0] = l[0] * v[0] + l[1] * v[3] + l[2] * v[6];
    f[1] = l[0] * v[1] + l[1] * v[4] + l[2] * v[7];
    f[2] = l[0] * v[2] + l[1] * v[5] + l[2] * v[8];
    stokes_kernel(s, f, n, G, T, prG, prT);
    double w = R.w[i] * area;
    double wl[3] = {w * l[0], w * l[1], w * l[2]};
    for (int k = 0; k < 6; ++k) E.G[k] += w * G[kSym[k][0]][kSym[k][1]];
    for (int k = 0; k < 3; ++k) E.prG[k] += w * prG[k];
    for (int k = 0; k < 6; ++k)
      for (int j = 0; j < 3; ++j) E.T[k][j] += wl[j] * T[kSym[k][0]][kSym[k][1]];
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j) E.prT[k][j] += wl[j] * prT[k];
  }
}
static void tri_stk_regular(const TriRule& R, const double v[9], const double s[3], const double n[3], double area,
                            StkElem& E) {
  tri_stk_sub(R, v, bary_identity(), s, n, area, E);
}
// Quad_StokesIntNum (lib_Stokes.f90:3754-3940): fixed 3x3 subcells; ndiv = 1 is
// the regular branch of Quad_StokesInt (lib_Stokes.f90:3398-3752, one cell).
static void quad_stk_regular(int iqud, const double q[12], const double s[3], double multi, StkElem& E,
                             int ndiv = 3) {
  const double *P1 = q, *P2 = q + 3, *P3 = q + 6, *P4 = q + 9;
  int ng1 = agb_tables::kGaussNg1[iqud - 1], ng2 = agb_tables::kGaussNg2[iqud - 1];
  E.zero();
  const int ndx = ndiv, nde = ndiv;
  double G[3][3], T[3][3], prG[3], prT[3];
  for (int ix = 1; ix <= ndx; ++ix)
    for (int ie = 1; ie <= nde; ++ie) {
      double a = -1.0 + (ix - 1) * 2.0 / ndx, b = -1.0 + ix * 2.0 / ndx;
      double c = -1.0 + (ie - 1) * 2.0 / nde, d = -1.0 + ie * 2.0 / nde;
      double dex = 0.25 * (b - a) * (d - c);
      for (int i = ng1; i <= ng2; ++i) {
        double gii = a + 0.5 * (GI(i) + 1.0) * (b - a);
        double e1m = 1.0 - gii, e1p = 1.0 + gii;
        for (int j = ng1; j <= ng2; ++j) {
          double gij = c + 0.5 * (GI(j) + 1.0) * (d - c);
          double e2m = 1.0 - gij, e2p = 1.0 + gij;
          double f4[4] = {0.25 * e1m * e2m, 0.25 * e1p * e2m, 0.25 * e1p * e2p, 0.25 * e1m * e2p};
          double X[3], KS[3], ET[3];
          for (int k = 0; k < 3; ++k) {
            X[k] = f4[0] * P1[k] + f4[1] * P2[k] + f4[2] * P3[k] + f4[3] * P4[k];
            KS[k] = 0.25 * (-e2m * P1[k] + e2m * P2[k] + e2p * P3[k] - e2p * P4[k]);
            ET[k] = 0.25 * (-e1m * P1[k] - e1p * P2[k] + e1p * P3[k] + e1m * P4[k]);
          }
          double anx = KS[1] * ET[2] - ET[1] * KS[2];
          double any = ET[0] * KS[2] - KS[0] * ET[2];
          double anz = KS[0] * ET[1] - ET[0] * KS[1];
          double ajac = 1.0 / std::sqrt(anx * anx + any * any + anz * anz);
          double nn[3] = {multi * anx * ajac, multi * any * ajac, multi * anz * ajac};
          ajac = dex * OME(i) * OME(j) / ajac;
          stokes_kernel(s, X, nn, G, T, prG, prT);
          double w = ajac;
          for (int k = 0; k < 6; ++k) E.G[k] += w * G[kSym[k][0]][kSym[k][1]];
          for (int k = 0; k < 3; ++k) E.prG[k] += w * prG[k];
          for (int isip = 0; isip < 4; ++isip) {
            double ww = ajac * f4[isip];
            for (int k = 0; k < 6; ++k) E.T[k][isip] += ww * T[kSym[k][0]][kSym[k][1]];
            for (int k = 0; k < 3; ++k) E.prT[k][isip] += ww * prT[k];
          }
        }
      }
    }
}

// Singular branch of Quad_BEMInt (lib_int.f90:408-524) and Quad_StokesInt
// (lib_Stokes.f90:3494-3654): the source at local node isrc (1..4 corners,
// 5 centre: ksi/eta data at lib_int.f90:362-363) splits the parameter square
// into four triangles, each integrated in polar coordinates about the source
// (theta over [TH0, TH1], rho over [0, ROTH(theta)], ng x ng Gauss points of
// rule iqud); the Jacobian rho cancels the 1/r singularity.  A triangle of zero
// width (source on its edge) is skipped, as the reference's GOTO 1000 does.
// visit(X, nn (unit normal times multi), w, f4) receives every point.
template <class F>
static void quad_polar(int iqud, const double q[12], int isrc, double multi, F&& visit) {
  static const double ksi[5] = {0.0, 1.0, 1.0, 0.0, 0.5}, eta[5] = {0.0, 0.0, 1.0, 1.0, 0.5};
  const double PI = 3.14159265358979323846, PI2 = 2.0 * PI;
  const double *P1 = q, *P2 = q + 3, *P3 = q + 6, *P4 = q + 9;
  const int ng1 = agb_tables::kGaussNg1[iqud - 1], ng2 = agb_tables::kGaussNg2[iqud - 1];
  const double xx1 = ksi[isrc - 1], yy1 = eta[isrc - 1];  // one cell: a = c = -1, b = d = 1
  for (int k = 1; k <= 4; ++k) {
    double al, fii, th0, th1;
    if (k == 1) {
      if (1.0 - xx1 == 0.0) continue;
      al = std::sqrt(yy1 * yy1 + (1.0 - xx1) * (1.0 - xx1));
      fii = std::acos(yy1 / al);
      th0 = 1.5 * PI + std::acos(yy1 / al);
      th1 = PI2 + std::atan((1.0 - yy1) / (1.0 - xx1));
    } else if (k == 2) {
      if (1.0 - yy1 == 0.0) continue;
      al = std::sqrt((1.0 - yy1) * (1.0 - yy1) + (1.0 - xx1) * (1.0 - xx1));
      fii = std::acos((1.0 - xx1) / al);
      th0 = std::asin((1.0 - yy1) / al);
      th1 = 0.5 * PI + std::atan(xx1 / (1.0 - yy1));
    } else if (k == 3) {
      if (xx1 == 0.0) continue;
      al = std::sqrt(xx1 * xx1 + (1.0 - yy1) * (1.0 - yy1));
      fii = std::acos((1.0 - yy1) / al);
      th0 = 0.5 * PI + std::acos((1.0 - yy1) / al);
      th1 = PI + std::atan(yy1 / xx1);
    } else {
      if (yy1 == 0.0) continue;
      al = std::sqrt(yy1 * yy1 + xx1 * xx1);
      fii = std::acos(xx1 / al);
      th0 = PI + std::acos(xx1 / al);
      th1 = 1.5 * PI + std::atan((1.0 - xx1) / yy1);
    }
    for (int i = ng1; i <= ng2; ++i)
      for (int j = ng1; j <= ng2; ++j) {
        const double th = (th1 - th0) * GI(i) / 2.0 + (th1 + th0) / 2.0;
        const double roth = al * std::sin(fii) / std::sin(th - th0 + fii);
        const double ro = roth * GI(j) / 2.0 + roth / 2.0;
        const double eti = 2.0 * (xx1 + ro * std::cos(th)) - 1.0;
        const double etj = 2.0 * (yy1 + ro * std::sin(th)) - 1.0;
        const double e1m = 1.0 - eti, e1p = 1.0 + eti, e2m = 1.0 - etj, e2p = 1.0 + etj;
        const double f4[4] = {0.25 * e1m * e2m, 0.25 * e1p * e2m, 0.25 * e1p * e2p, 0.25 * e1m * e2p};
        double X[3], KS[3], ET[3];
        for (int c = 0; c < 3; ++c) {
          X[c] = f4[0] * P1[c] + f4[1] * P2[c] + f4[2] * P3[c] + f4[3] * P4[c];
          KS[c] = 0.25 * (-e2m * P1[c] + e2m * P2[c] + e2p * P3[c] - e2p * P4[c]);
          ET[c] = 0.25 * (-e1m * P1[c] - e1p * P2[c] + e1p * P3[c] + e1m * P4[c]);
        }
        const double anx = KS[1] * ET[2] - ET[1] * KS[2];
        const double any = ET[0] * KS[2] - KS[0] * ET[2];
        const double anz = KS[0] * ET[1] - ET[0] * KS[1];
        const double ajac = 1.0 / std::sqrt(anx * anx + any * any + anz * anz);
        const double nn[3] = {multi * anx * ajac, multi * any * ajac, multi * anz * ajac};
        const double w = (th1 - th0) * roth * ro * OME(i) * OME(j) / ajac;
        visit(X, nn, w, f4);
      }
  }
}
// Laplace: out[0] = G, out[1..4] = H at the nodes (BemKernel, lib_sdBem.f90:911)
static void quad_lap_polar(int iqud, const double q[12], const double s[3], int isrc, double multi, double out[5]) {
  for (int k = 0; k < 5; ++k) out[k] = 0.0;
  const double fpi = 1.0 / (4.0 * 3.14159265358979323846);
  quad_polar(iqud, q, isrc, multi, [&](const double* X, const double* nn, double w, const double* f4) {
    const double rx = s[0] - X[0], ry = s[1] - X[1], rz = s[2] - X[2];
    const double ra = std::sqrt(rx * rx + ry * ry + rz * rz);
    const double fg = fpi / ra;
    const double fh = (rx * nn[0] + ry * nn[1] + rz * nn[2]) / (ra * ra) * fg;
    for (int k = 0; k < 4; ++k) out[1 + k] += fh * w * f4[k];
    out[0] += fg * w;
  });
}
// Stokes: G and T of the element; its pressure integrals prG (a Cauchy
// principal value) and prT (hypersingular) are left zero, as the analytic
// self-element branch leaves them (lib_intAna.f90:43-82) -- the polar rule
// cannot integrate them, and the reference never calls this branch with its
// source on the element (lib_Stokes.f90:3199 passes isrc = 0).
static void quad_stk_polar(int iqud, const double q[12], const double s[3], int isrc, double multi, StkElem& E) {
  E.zero();
  double G[3][3], T[3][3], prG[3], prT[3];
  quad_polar(iqud, q, isrc, multi, [&](const double* X, const double* nn, double w, const double* f4) {
    stokes_kernel(s, X, nn, G, T, prG, prT);
    for (int k = 0; k < 6; ++k) E.G[k] += w * G[kSym[k][0]][kSym[k][1]];
    for (int isip = 0; isip < 4; ++isip) {
      const double ww = w * f4[isip];
      for (int k = 0; k < 6; ++k) E.T[k][isip] += ww * T[kSym[k][0]][kSym[k][1]];
    }
  });
}

// -----------------------------------------------------------------------------
// Problem state: mesh + single subdomain + boundary conditions
// -----------------------------------------------------------------------------
struct CRS {
  int neq = 0;
  int64_t nnz = 0;
  std::vector<int64_t> i;  // 1-based row starts (neq+1)
  std::vector<int> j;      // 1-based columns
  std::vector<double> v;
};

struct Eqn {
  int nx = 0, nb = 0, neq = 0;
  std::vector<int> col, qcol;  // 1-based numbering, -999 = not set
  std::vector<double> u, q, x, b, pivot;
  CRS sys, rhs;
};

struct Problem {
  int kind = 1;  // 1 Laplace, 2 Stokes
  int neq = 1;
  // mesh (lib_mesh / mod_mesh)
  int nnodes = 0, nelem = 0;
  std::vector<double> x;       // 3*nnodes
  std::vector<int> type, nno;  // type 2 tri, 3 quad
  std::vector<int> con;        // 4*nelem, 0-based
  std::vector<int> bcid;       // wall id per element
  std::vector<double> normal, area, qx;
  // subdomain
  std::vector<int> loWalls;
  std::vector<double> normMul;
  double diff = 1.0;
  std::vector<int> known;  // [neq][nw] BC type per equation and subdomain wall
  std::vector<int> elementList, qnodeList, qbcidList, nodeList, BCidList;
  int sd_nnodes = 0, sd_nqnodes = 0, nsp = 0;
  // quadrature
  TriRule tri;
  int iqud = 4;
  IntegOpt opt;
  // integral matrices
  std::vector<double> H, G;   // Laplace: nsp x sd_nnodes / nsp x sd_nqnodes, column-major
  std::vector<double> M[18];  // Stokes: Txx..Tzz, prTx..prTz (nsp x nn), Gxx..Gzz, prGx..prGz (nsp x nq)
  double fspCerr = 0, qspCerr = 0;
  // equations
  std::vector<Eqn> eqn;
  Eqn stk;  // Stokes big system (col/qcol are 3*nnodes / 3*nqnodes)
  int knownOf(int en, int wall) const {
    for (size_t k = 0; k < loWalls.size(); ++k)
      if (loWalls[k] == wall) return known[en * loWalls.size() + k];
    return 0;
  }
  double multiOf(int wall) const {
    double m = 1.0;
    for (size_t k = 0; k < loWalls.size(); ++k)
      if (loWalls[k] == wall) m = normMul[k];
    return m;
  }
};

// CalElementNormal (lib_mesh.f90:716-769), CalElementArea (lib_int.f90:606-721),
// CalQMesh (lib_mesh.f90:577-629)
static void geometry(Problem& P) {
  P.normal.assign(3 * P.nelem, 0.0);
  P.area.assign(P.nelem, 0.0);
  P.qx.assign(3 * P.nelem, 0.0);
  for (int e = 0; e < P.nelem; ++e) {
    const double* t1 = &P.x[3 * P.con[4 * e + 0]];
    const double* t2 = &P.x[3 * P.con[4 * e + 1]];
    const double* t3 = &P.x[3 * P.con[4 * e + 2]];
    double v1[3] = {t2[0] - t1[0], t2[1] - t1[1], t2[2] - t1[2]};
    double v2[3] = {t3[0] - t1[0], t3[1] - t1[1], t3[2] - t1[2]};
    double n[3] = {v1[1] * v2[2] - v1[2] * v2[1], -v1[0] * v2[2] + v1[2] * v2[0], v1[0] * v2[1] - v1[1] * v2[0]};
    double d = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int i = 0; i < 3; ++i) P.normal[3 * e + i] = n[i] / d;
    if (P.type[e] == 2) {
      P.area[e] = tri_area(t1[0], t1[1], t1[2], t2[0], t2[1], t2[2], t3[0], t3[1], t3[2]);
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += (1.0 / 3.0) * P.x[3 * P.con[4 * e + k] + j];
        P.qx[3 * e + j] = s;
      }
    } else {
      const double* t4 = &P.x[3 * P.con[4 * e + 3]];
      const double* Q[4] = {t1, t2, t3, t4};
      int ng1 = agb_tables::kGaussNg1[3], ng2 = agb_tables::kGaussNg2[3];
      double integral = 0.0, a = -1, b = 1, c = -1, dd = 1, dex = 0.25 * (b - a) * (dd - c);
      for (int i = ng1; i <= ng2; ++i) {
        double gii = a + 0.5 * (GI(i) + 1.0) * (b - a);
        double e1m = 1.0 - gii, e1p = 1.0 + gii;
        for (int j = ng1; j <= ng2; ++j) {
          double gij = c + 0.5 * (GI(j) + 1.0) * (dd - c);
          double e2m = 1.0 - gij, e2p = 1.0 + gij;
          double f4[4] = {0.25 * e1m * e2m, 0.25 * e1p * e2m, 0.25 * e1p * e2p, 0.25 * e1m * e2p};
          double KS[3], ET[3];
          for (int k = 0; k < 3; ++k) {
            KS[k] = 0.25 * (-e2m * Q[0][k] + e2m * Q[1][k] + e2p * Q[2][k] - e2p * Q[3][k]);
            ET[k] = 0.25 * (-e1m * Q[0][k] - e1p * Q[1][k] + e1p * Q[2][k] + e1m * Q[3][k]);
          }
          double anx = KS[1] * ET[2] - ET[1] * KS[2];
          double any = ET[0] * KS[2] - KS[0] * ET[2];
          double anz = KS[0] * ET[1] - ET[0] * KS[1];
          double ajac = dex * OME(i) * OME(j) * std::sqrt(anx * anx + any * any + anz * anz);
          for (int isip = 0; isip < 4; ++isip) integral += ajac * f4[isip];
        }
      }
      P.area[e] = integral;
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int k = 0; k < 4; ++k) s += 0.25 * P.x[3 * P.con[4 * e + k] + j];
        P.qx[3 * e + j] = s;
      }
    }
  }
}

// SetUpSubdomains (lib_sdBem.f90:319-430), single subdomain
static void setup_subdomain(Problem& P) {
  P.elementList.clear();
  for (int w : P.loWalls)
    for (int e = 0; e < P.nelem; ++e)
      if (P.bcid[e] == w) P.elementList.push_back(e);
  P.sd_nqnodes = (int)P.elementList.size();
  P.qnodeList = P.elementList;
  P.qbcidList.resize(P.sd_nqnodes);
  for (int i = 0; i < P.sd_nqnodes; ++i) P.qbcidList[i] = P.bcid[P.elementList[i]];
  std::vector<int> tmp(P.nnodes, 0);
  std::vector<char> has(P.nnodes, 0);
  for (int e : P.elementList)
    for (int j = 0; j < P.nno[e]; ++j) { tmp[P.con[4 * e + j]] = P.bcid[e]; has[P.con[4 * e + j]] = 1; }
  P.nodeList.clear(); P.BCidList.clear();
  for (int i = 0; i < P.nnodes; ++i)
    if (has[i]) { P.nodeList.push_back(i); P.BCidList.push_back(tmp[i]); }
  P.sd_nnodes = (int)P.nodeList.size();
  P.nsp = P.sd_nnodes + P.sd_nqnodes;
}

// Elements of the subdomain in the reference's traversal order: walls of the
// subdomain in list order, then element index (lib_sdBem.f90:471-474).
static void element_vertices(const Problem& P, int e, double* v) {
  for (int k = 0; k < P.nno[e]; ++k)
    for (int i = 0; i < 3; ++i) v[3 * k + i] = P.x[3 * P.con[4 * e + k] + i];
}

// sdIntRowU (lib_sdBem.f90:438-584): source at node irow (global index)
static void lap_row_u(const Problem& P, int irow, double* rowH, double* rowG, double& err) {
  std::fill(rowH, rowH + P.nnodes, 0.0);
  std::fill(rowG, rowG + P.nelem, 0.0);
  const double s[3] = {P.x[3 * irow], P.x[3 * irow + 1], P.x[3 * irow + 2]};
  for (size_t jj = 0; jj < P.loWalls.size(); ++jj) {
    int iWall = P.loWalls[jj];
    double mm = P.normMul[jj];
    for (int ie = 0; ie < P.nelem; ++ie) {
      if (P.bcid[ie] != iWall) continue;
      int isrc = 0;
      for (int j = 0; j < P.nno[ie]; ++j)
        if (irow == P.con[4 * ie + j]) isrc = j + 1;
      double v[12], integ = 0.0, inteH[4] = {0, 0, 0, 0};
      element_vertices(P, ie, v);
      if (P.type[ie] == 2) {
        double n[3] = {mm * P.normal[3 * ie], mm * P.normal[3 * ie + 1], mm * P.normal[3 * ie + 2]};
        if (isrc == 0 || P.opt.sing == 1) {
          double out[4] = {0, 0, 0, 0};
          tri_walk(P.opt, v, s, P.area[ie], isrc,
                   [&](const Bary& B, double a, bool sk) { tri_lap_sub(P.tri, v, B, s, n, a, out, sk); });
          integ = out[0]; inteH[0] = out[1]; inteH[1] = out[2]; inteH[2] = out[3];
        } else {
          integ = si_tri_lap(v, P.area[ie], isrc);
        }
      } else {
        if (isrc == 0) {
          double out[5];
          quad_lap_regular(P.iqud, v, s, mm, out);
          integ = out[0];
          for (int k = 0; k < 4; ++k) inteH[k] = out[1 + k];
        } else if (P.opt.sing == 1) {
          double out[5];
          quad_lap_polar(P.iqud, v, s, isrc, mm, out);
          integ = out[0];
          for (int k = 0; k < 4; ++k) inteH[k] = out[1 + k];
        } else {
          integ = si_qua_lap(v, isrc);
        }
      }
      for (int j = 0; j < P.nno[ie]; ++j) rowH[P.con[4 * ie + j]] += inteH[j];
      rowG[ie] = integ;
    }
  }
  double c = 0.0;
  for (int i = 0; i < P.nnodes; ++i) c -= rowH[i];
  rowH[irow] += c;
  for (int j = 0; j < 3; ++j) {
    c = 0.0;
    for (int i = 0; i < P.nnodes; ++i) c += rowH[i] * P.x[3 * i + j];
    for (int i = 0; i < P.nelem; ++i) c -= rowG[i] * P.normal[3 * i + j] * P.multiOf(P.bcid[i]);
    err = std::max(err, std::fabs(c));
  }
}
// sdIntRowQ (lib_sdBem.f90:589-733): source at centroid of element irow
static void lap_row_q(const Problem& P, int irow, double* rowH, double* rowG, double& err) {
  std::fill(rowH, rowH + P.nnodes, 0.0);
  std::fill(rowG, rowG + P.nelem, 0.0);
  const double s[3] = {P.qx[3 * irow], P.qx[3 * irow + 1], P.qx[3 * irow + 2]};
  for (size_t jj = 0; jj < P.loWalls.size(); ++jj) {
    int iWall = P.loWalls[jj];
    double mm = P.normMul[jj];
    for (int ie = 0; ie < P.nelem; ++ie) {
      if (P.bcid[ie] != iWall) continue;
      int isrc = 0;
      if (ie == irow) isrc = (P.type[ie] == 2) ? 4 : 5;
      double v[12], integ = 0.0, inteH[4] = {0, 0, 0, 0};
      element_vertices(P, ie, v);
      if (P.type[ie] == 2) {
        double n[3] = {mm * P.normal[3 * ie], mm * P.normal[3 * ie + 1], mm * P.normal[3 * ie + 2]};
        if (isrc == 0 || P.opt.sing == 1) {
          double out[4] = {0, 0, 0, 0};
          tri_walk(P.opt, v, s, P.area[ie], isrc,
                   [&](const Bary& B, double a, bool sk) { tri_lap_sub(P.tri, v, B, s, n, a, out, sk); });
          integ = out[0]; inteH[0] = out[1]; inteH[1] = out[2]; inteH[2] = out[3];
        } else {
          integ = si_tri_lap(v, P.area[ie], isrc);
        }
      } else {
        if (isrc == 0) {
          double out[5];
          quad_lap_regular(P.iqud, v, s, mm, out);
          integ = out[0];
          for (int k = 0; k < 4; ++k) inteH[k] = out[1 + k];
        } else if (P.opt.sing == 1) {
          double out[5];
          quad_lap_polar(P.iqud, v, s, isrc, mm, out);
          integ = out[0];
          for (int k = 0; k < 4; ++k) inteH[k] = out[1 + k];
        } else {
          integ = si_qua_lap(v, isrc);
        }
      }
      for (int j = 0; j < P.nno[ie]; ++j) rowH[P.con[4 * ie + j]] += inteH[j];
      rowG[ie] = integ;
    }
  }
  double c = 0.0;
  for (int i = 0; i < P.nnodes; ++i) c -= rowH[i];
  err = std::max(err, std::fabs(0.5 - c));
  double shpf = (P.type[irow] == 2) ? 1.0 / 3.0 : 0.25;
  for (int j = 0; j < P.nno[irow]; ++j) rowH[P.con[4 * irow + j]] += shpf * c;
}

// sdFormIntegralMatrices (lib_int.f90:225-323)
static void lap_form_matrices(Problem& P) {
  P.H.assign((size_t)P.nsp * P.sd_nnodes, 0.0);
  P.G.assign((size_t)P.nsp * P.sd_nqnodes, 0.0);
  double errU = 0.0, errQ = 0.0;
#pragma omp parallel
  {
    std::vector<double> rowH(P.nnodes), rowG(P.nelem);
    double eu = 0.0, eq = 0.0;
#pragma omp for schedule(dynamic, 4)
    for (int r = 0; r < P.nsp; ++r) {
      if (r < P.sd_nnodes) lap_row_u(P, P.nodeList[r], rowH.data(), rowG.data(), eu);
      else lap_row_q(P, P.qnodeList[r - P.sd_nnodes], rowH.data(), rowG.data(), eq);
      for (int j = 0; j < P.sd_nnodes; ++j) P.H[(size_t)j * P.nsp + r] = rowH[P.nodeList[j]];
      for (int j = 0; j < P.sd_nqnodes; ++j) P.G[(size_t)j * P.nsp + r] = rowG[P.qnodeList[j]];
    }
#pragma omp critical
    { errU = std::max(errU, eu); errQ = std::max(errQ, eq); }
  }
  P.fspCerr = errU;
  P.qspCerr = errQ;
}

// Stokes rows. Row arrays laid out [comp][n]: T comps 0..5 (xx,xy,xz,yy,yz,zz),
// prT 6..8 over nnodes; G comps 0..5 and prG 6..8 over nelem.
struct StkRow {
  std::vector<double> T, G;  // 9*nnodes, 9*nelem
  int nn, ne;
  StkRow(int nn_, int ne_) : T(9 * (size_t)nn_), G(9 * (size_t)ne_), nn(nn_), ne(ne_) {}
  double& t(int c, int i) { return T[(size_t)c * nn + i]; }
  double& g(int c, int i) { return G[(size_t)c * ne + i]; }
};

static void stk_element(const Problem& P, int ie, const double s[3], int isrc, double mm, StkElem& E) {
  double v[12];
  element_vertices(P, ie, v);
  E.zero();
  if (P.type[ie] == 2) {
    if (isrc == 0 || P.opt.sing == 1) {
      double n[3] = {mm * P.normal[3 * ie], mm * P.normal[3 * ie + 1], mm * P.normal[3 * ie + 2]};
      tri_walk(P.opt, v, s, P.area[ie], isrc, [&](const Bary& B, double a, bool sk) { tri_stk_sub(P.tri, v, B, s, n, a, E, sk); });
    } else {
      si_tri_stk(v, P.area[ie], isrc, E.G);  // T, prT, prG stay zero (lib_intAna.f90:136-148)
    }
  } else {
    if (isrc == 0) quad_stk_regular(P.iqud, v, s, mm, E);
    else if (P.opt.sing == 1) quad_stk_polar(P.iqud, v, s, isrc, mm, E);
    else si_qua_stk(v, isrc, E.G);  // Quad_StokesIntAna (lib_intAna.f90:43-82)
  }
}

// sdIntRowQStokes (lib_Stokes.f90:1562-1897)
static void stk_row_q(const Problem& P, int irow, StkRow& R, double& err) {
  std::fill(R.T.begin(), R.T.end(), 0.0);
  std::fill(R.G.begin(), R.G.end(), 0.0);
  const double osemPi = (double)std::atan(1.0f) * 4.0 * 8.0;  // single-precision ATAN(1.0)
  const double s[3] = {P.qx[3 * irow], P.qx[3 * irow + 1], P.qx[3 * irow + 2]};
  StkElem E;
  for (size_t jj = 0; jj < P.loWalls.size(); ++jj) {
    int iWall = P.loWalls[jj];
    double mm = P.normMul[jj];
    for (int ie = 0; ie < P.nelem; ++ie) {
      if (P.bcid[ie] != iWall) continue;
      int isrc = 0;
      if (ie == irow) isrc = (P.type[ie] == 2) ? 4 : 5;
      stk_element(P, ie, s, isrc, mm, E);
      for (int j = 0; j < P.nno[ie]; ++j)
        for (int k = 0; k < 6; ++k) R.t(k, P.con[4 * ie + j]) += E.T[k][j];
      for (int k = 0; k < 6; ++k) R.g(k, ie) = E.G[k];
      if (isrc == 0) {
        for (int j = 0; j < P.nno[ie]; ++j)
          for (int k = 0; k < 3; ++k) R.t(6 + k, P.con[4 * ie + j]) += E.prT[k][j];
        for (int k = 0; k < 3; ++k) R.g(6 + k, ie) = E.prG[k];
      }
    }
  }
  err = -9.99;
  double cx = 0, cy = 0, cz = 0;
  for (int i = 0; i < P.nnodes; ++i) { cx -= R.t(1, i); cy -= R.t(4, i); cz -= R.t(2, i); }
  err = std::max(err, std::fabs(cx)); err = std::max(err, std::fabs(cy)); err = std::max(err, std::fabs(cz));
  cx = cy = cz = 0;
  for (int i = 0; i < P.nnodes; ++i) { cx -= R.t(0, i); cy -= R.t(3, i); cz -= R.t(5, i); }
  err = std::max(err, std::fabs(cx - 0.5 * osemPi));
  err = std::max(err, std::fabs(cy - 0.5 * osemPi));
  err = std::max(err, std::fabs(cz - 0.5 * osemPi));
  int ie = irow;
  double shpf = (P.type[ie] == 2) ? 1.0 / 3.0 : 0.25;
  for (int j = 0; j < P.nno[ie]; ++j) {
    int nd = P.con[4 * ie + j];
    R.t(0, nd) += shpf * cx; R.t(3, nd) += shpf * cy; R.t(5, nd) += shpf * cz;
  }
  cx = cy = cz = 0;
  for (int j = 0; j < P.nnodes; ++j) { cx += R.t(6, j); cy += R.t(7, j); cz += R.t(8, j); }
  for (int j = 0; j < P.nno[irow]; ++j) {
    int nd = P.con[4 * irow + j];
    R.t(6, nd) -= cx / P.nno[irow]; R.t(7, nd) -= cy / P.nno[irow]; R.t(8, nd) -= cz / P.nno[irow];
  }
}
// sdIntRowUStokes (lib_Stokes.f90:1904-2245)
static void stk_row_u(const Problem& P, int irow, StkRow& R, double& err) {
  std::fill(R.T.begin(), R.T.end(), 0.0);
  std::fill(R.G.begin(), R.G.end(), 0.0);
  const double s[3] = {P.x[3 * irow], P.x[3 * irow + 1], P.x[3 * irow + 2]};
  StkElem E;
  for (size_t jj = 0; jj < P.loWalls.size(); ++jj) {
    int iWall = P.loWalls[jj];
    double mm = P.normMul[jj];
    for (int ie = 0; ie < P.nelem; ++ie) {
      if (P.bcid[ie] != iWall) continue;
      int isrc = 0;
      for (int j = 0; j < P.nno[ie]; ++j)
        if (irow == P.con[4 * ie + j]) isrc = j + 1;
      stk_element(P, ie, s, isrc, mm, E);
      for (int j = 0; j < P.nno[ie]; ++j) {
        int nd = P.con[4 * ie + j];
        for (int k = 0; k < 6; ++k) R.t(k, nd) += E.T[k][j];
        for (int k = 0; k < 3; ++k) R.t(6 + k, nd) += E.prT[k][j];
      }
      for (int k = 0; k < 6; ++k) R.g(k, ie) = E.G[k];
      for (int k = 0; k < 3; ++k) R.g(6 + k, ie) = E.prG[k];
    }
  }
  err = -9.99;
  double cx = 0, cy = 0, cz = 0;
  for (int i = 0; i < P.nnodes; ++i) { cx -= R.t(0, i); cy -= R.t(3, i); cz -= R.t(5, i); }
  R.t(0, irow) += cx; R.t(3, irow) += cy; R.t(5, irow) += cz;
  cx = cy = cz = 0;
  for (int i = 0; i < P.nelem; ++i) {
    double m = P.multiOf(P.bcid[i]);
    const double* n = &P.normal[3 * i];
    cx = cx - R.g(0, i) * n[0] * m - R.g(1, i) * n[1] * m - R.g(2, i) * n[2] * m;
    cy = cy - R.g(1, i) * n[0] * m - R.g(3, i) * n[1] * m - R.g(4, i) * n[2] * m;
    cz = cz - R.g(2, i) * n[0] * m - R.g(4, i) * n[1] * m - R.g(5, i) * n[2] * m;
  }
  err = std::max(err, std::fabs(cx)); err = std::max(err, std::fabs(cy)); err = std::max(err, std::fabs(cz));
}

// sdFormIntegralMatricesStokes (lib_Stokes.f90:1391-1555).  Matrix order in
// P.M: 0..5 T(xx,xy,xz,yy,yz,zz), 6..8 prT, 9..14 G, 15..17 prG.
static void stk_form_matrices(Problem& P) {
  for (int k = 0; k < 9; ++k) P.M[k].assign((size_t)P.nsp * P.sd_nnodes, 0.0);
  for (int k = 9; k < 18; ++k) P.M[k].assign((size_t)P.nsp * P.sd_nqnodes, 0.0);
  double errU = -1e300, errQ = -1e300;
#pragma omp parallel
  {
    StkRow R(P.nnodes, P.nelem);
    double eu = -1e300, eq = -1e300;
#pragma omp for schedule(dynamic, 4)
    for (int r = 0; r < P.nsp; ++r) {
      double e;
      if (r < P.sd_nnodes) { stk_row_u(P, P.nodeList[r], R, e); eu = std::max(eu, e); }
      else { stk_row_q(P, P.qnodeList[r - P.sd_nnodes], R, e); eq = std::max(eq, e); }
      for (int k = 0; k < 9; ++k)
        for (int j = 0; j < P.sd_nnodes; ++j) P.M[k][(size_t)j * P.nsp + r] = R.t(k, P.nodeList[j]);
      for (int k = 0; k < 9; ++k)
        for (int j = 0; j < P.sd_nqnodes; ++j) P.M[9 + k][(size_t)j * P.nsp + r] = R.g(k, P.qnodeList[j]);
    }
#pragma omp critical
    { errU = std::max(errU, eu); errQ = std::max(errQ, eq); }
  }
  P.fspCerr = errU;
  P.qspCerr = errQ;
}

// sdSetUpXandB (lib_sdBem.f90:4-107)
static void setup_xb(Problem& P) {
  const int notSet = -999;
  P.eqn.assign(P.neq, Eqn());
  for (int en = 0; en < P.neq; ++en) {
    Eqn& E = P.eqn[en];
    E.col.assign(P.nnodes, notSet);
    E.qcol.assign(P.nelem, notSet);
    for (int i = 0; i < P.sd_nnodes; ++i) {
      int isp = P.nodeList[i], bc = P.knownOf(en, P.BCidList[i]);
      if (bc == iFunction) { E.nb++; E.col[isp] = E.nb; }
      else if (bc == iFlux) { E.nx++; E.col[isp] = E.nx; E.neq++; }
      else if (bc == iContact) { E.neq++; if (E.col[isp] == notSet) { E.nx++; E.col[isp] = E.nx; } }
    }
    for (int i = 0; i < P.sd_nqnodes; ++i) {
      int isp = P.qnodeList[i], bc = P.knownOf(en, P.qbcidList[i]);
      if (bc == iFunction) { E.nx++; E.qcol[isp] = E.nx; E.neq++; }
      else if (bc == iFlux) { E.nb++; E.qcol[isp] = E.nb; }
      else if (bc == iContact) { E.neq++; if (E.qcol[isp] == notSet) { E.nx++; E.qcol[isp] = E.nx; } }
    }
    E.x.assign(E.nx, 0.0);
    E.pivot.assign(E.nx, 0.0);
    E.b.assign(E.nb, 0.0);
    E.u.assign(P.nnodes, 0.0);
    E.q.assign(P.nelem, 0.0);
  }
}

// sdSetUpSysMrhsM_CRS (lib_CRS.f90:148-343): Laplace, no zero dropping
static void lap_form_crs(Problem& P, int en) {
  Eqn& E = P.eqn[en];
  CRS &S = E.sys, &Rm = E.rhs;
  S = CRS(); Rm = CRS();
  S.neq = Rm.neq = E.neq;
  S.i.assign(E.neq + 1, 0); Rm.i.assign(E.neq + 1, 0);
  int row = 0, r = 0;
  auto emitH = [&](int rr) {
    for (int j = 0; j < P.sd_nnodes; ++j) {
      int col = E.col[P.nodeList[j]], bc = P.knownOf(en, P.BCidList[j]);
      double val = P.H[(size_t)j * P.nsp + rr];
      if (bc == iFunction) { Rm.v.push_back(val); Rm.j.push_back(col); }
      if (bc == iFlux || bc == iContact) { S.v.push_back(val); S.j.push_back(col); }
    }
    for (int j = 0; j < P.sd_nqnodes; ++j) {
      int col = E.qcol[P.qnodeList[j]], wallC = P.qbcidList[j], bc = P.knownOf(en, wallC);
      double val = P.multiOf(wallC) / P.diff * P.G[(size_t)j * P.nsp + rr];
      if (bc == iFunction || bc == iContact) { S.v.push_back(val); S.j.push_back(col); }
      if (bc == iFlux) { Rm.v.push_back(val); Rm.j.push_back(col); }
    }
  };
  for (int i = 0; i < P.sd_nnodes; ++i, ++r) {
    int bc = P.knownOf(en, P.BCidList[i]);
    if (bc == iFlux || bc == iContact) {
      S.i[row] = (int64_t)S.v.size() + 1; Rm.i[row] = (int64_t)Rm.v.size() + 1; row++;
      emitH(r);
    }
  }
  for (int i = 0; i < P.sd_nqnodes; ++i, ++r) {
    int bc = P.knownOf(en, P.qbcidList[i]);
    if (bc == iFunction || bc == iContact) {
      S.i[row] = (int64_t)S.v.size() + 1; Rm.i[row] = (int64_t)Rm.v.size() + 1; row++;
      emitH(r);
    }
  }
  S.i[row] = (int64_t)S.v.size() + 1;
  Rm.i[row] = (int64_t)Rm.v.size() + 1;
  S.nnz = (int64_t)S.v.size();
  Rm.nnz = (int64_t)Rm.v.size();
}

// StokesBigSystemXB (lib_Stokes.f90:1180-1276)
static void stk_setup_xb(Problem& P) {
  Eqn& S = P.stk;
  S = Eqn();
  S.col.assign(3 * P.nnodes, -999);
  S.qcol.assign(3 * P.nelem, -999);
  for (int i = 0; i < P.sd_nnodes; ++i) {
    int isp = P.nodeList[i], wall = P.BCidList[i];
    S.nx = S.nb = S.neq = 0;
    for (int en = 0; en < 3; ++en) {
      int ispL = isp + en * P.nnodes, bc = P.knownOf(en, wall);
      if (bc == iFunction) S.col[ispL] = P.eqn[en].col[isp] + S.nb;
      else if (bc == iFlux || bc == iContact) S.col[ispL] = P.eqn[en].col[isp] + S.nx;
      S.nx += P.eqn[en].nx; S.nb += P.eqn[en].nb; S.neq += P.eqn[en].neq;
    }
  }
  for (int i = 0; i < P.sd_nqnodes; ++i) {
    int isp = P.qnodeList[i], wall = P.qbcidList[i];
    S.nx = S.nb = S.neq = 0;
    for (int en = 0; en < 3; ++en) {
      int ispL = isp + en * P.nelem, bc = P.knownOf(en, wall);
      if (bc == iFunction || bc == iContact) S.qcol[ispL] = P.eqn[en].qcol[isp] + S.nx;
      else if (bc == iFlux) S.qcol[ispL] = P.eqn[en].qcol[isp] + S.nb;
      S.nx += P.eqn[en].nx; S.nb += P.eqn[en].nb; S.neq += P.eqn[en].neq;
    }
  }
  S.x.assign(S.nx, 0.0);
  S.pivot.assign(S.nx, 0.0);
  S.b.assign(S.nb, 0.0);
}

// Index of the Stokes component matrix for (een, en): T uses 0..5, G uses 9..14
static int symIndex(int a, int b) {
  if (a > b) std::swap(a, b);
  static const int tab[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  return tab[a][b];
}

// formQrow / formUrow (lib_StokesFull.f90:4-167): one row of sysM and rhsM
static void stk_form_row(const Problem& P, int een, int r, std::vector<double>& sysRow, std::vector<double>& rhsRow) {
  const Eqn& S = P.stk;
  std::fill(sysRow.begin(), sysRow.end(), 0.0);
  std::fill(rhsRow.begin(), rhsRow.end(), 0.0);
  for (int j = 0; j < P.sd_nnodes; ++j) {
    int wallC = P.BCidList[j], isp = P.nodeList[j];
    for (int en = 0; en < 3; ++en) {
      int col = S.col[isp + en * P.nnodes], bc = P.knownOf(en, wallC);
      double val = P.M[symIndex(een, en)][(size_t)j * P.nsp + r];
      if (bc == iFunction) rhsRow[col - 1] = val;
      if (bc == iFlux || bc == iContact) sysRow[col - 1] = -val;
    }
  }
  for (int j = 0; j < P.sd_nqnodes; ++j) {
    int wallC = P.qbcidList[j], isp = P.qnodeList[j];
    for (int en = 0; en < 3; ++en) {
      int col = S.qcol[isp + en * P.nelem], bc = P.knownOf(en, wallC);
      double val = P.M[9 + symIndex(een, en)][(size_t)j * P.nsp + r];
      val = P.multiOf(wallC) / P.diff * val;
      if (bc == iFunction || bc == iContact) sysRow[col - 1] = -val;
      if (bc == iFlux) rhsRow[col - 1] = val;
    }
  }
}

// stokesFormCRSsysMrhsM (lib_Stokes.f90:475-637): CRS with exact zeros dropped
static void stk_form_crs(Problem& P) {
  Eqn& S = P.stk;
  S.neq = 0;
  for (int en = 0; en < 3; ++en) S.neq += P.eqn[en].neq;
  CRS &A = S.sys, &B = S.rhs;
  A = CRS(); B = CRS();
  A.neq = B.neq = S.neq;
  A.i.assign(S.neq + 1, 0); B.i.assign(S.neq + 1, 0);
  std::vector<double> sysRow(S.neq > S.nx ? S.neq : S.nx), rhsRow(std::max(S.nb, 1));
  sysRow.assign(std::max(S.neq, S.nx), 0.0);
  int row = 0, r = 0;
  auto emit = [&](int een, int rr) {
    A.i[row] = (int64_t)A.v.size() + 1; B.i[row] = (int64_t)B.v.size() + 1; row++;
    stk_form_row(P, een, rr, sysRow, rhsRow);
    for (int col = 0; col < S.nx; ++col)
      if (sysRow[col] != 0.0) { A.v.push_back(sysRow[col]); A.j.push_back(col + 1); }
    for (int col = 0; col < S.nb; ++col)
      if (rhsRow[col] != 0.0) { B.v.push_back(rhsRow[col]); B.j.push_back(col + 1); }
  };
  for (int i = 0; i < P.sd_nnodes; ++i, ++r)
    for (int een = 0; een < 3; ++een) {
      int bc = P.knownOf(een, P.BCidList[i]);
      if (bc == iFlux || bc == iContact) emit(een, r);
    }
  for (int i = 0; i < P.sd_nqnodes; ++i, ++r)
    for (int een = 0; een < 3; ++een) {
      int bc = P.knownOf(een, P.qbcidList[i]);
      if (bc == iFunction || bc == iContact) emit(een, r);
    }
  A.i[row] = (int64_t)A.v.size() + 1;
  B.i[row] = (int64_t)B.v.size() + 1;
  A.nnz = (int64_t)A.v.size();
  B.nnz = (int64_t)B.v.size();
}

// CRSxV (lib_CRS.f90:764-787)
static void crs_x_v(const CRS& M, const double* vek, double* rez) {
  for (int i = 0; i < M.neq; ++i) {
    double s = 0.0;
    for (int64_t j = M.i[i]; j <= M.i[i + 1] - 1; ++j) s += M.v[j - 1] * vek[M.j[j - 1] - 1];
    rez[i] = s;
  }
}

// -----------------------------------------------------------------------------
// LSQR (lib_lsqr.f) with reference-BLAS level-1 semantics
// -----------------------------------------------------------------------------
// dnrm2: scaled sum of squares (reference BLAS 3.x algorithm)
static double dnrm2(int n, const double* x) {
  if (n < 1) return 0.0;
  if (n == 1) return std::fabs(x[0]);
  double scale = 0.0, ssq = 1.0;
  for (int i = 0; i < n; ++i) {
    if (x[i] != 0.0) {
      double a = std::fabs(x[i]);
      if (scale < a) { ssq = 1.0 + ssq * (scale / a) * (scale / a); scale = a; }
      else ssq += (a / scale) * (a / scale);
    }
  }
  return scale * std::sqrt(ssq);
}
static void dscal(int n, double a, double* x) { for (int i = 0; i < n; ++i) x[i] *= a; }
// lsqr_d2norm (lib_lsqr.f:1236-1263)
static double d2norm(double a, double b) {
  double scale = std::fabs(a) + std::fabs(b);
  if (scale == 0.0) return 0.0;
  return scale * std::sqrt((a / scale) * (a / scale) + (b / scale) * (b / scale));
}
struct CrsView { int m, n; int64_t nnz; const int64_t* ia; const int* ja; double* a; };
// lsqr_matvec1: y = y + A x (lib_lsqr.f:203-233)
static void matvec1(const CrsView& A, const double* x, double* y) {
  for (int i = 0; i < A.m; ++i) {
    double s = 0.0;
    for (int64_t j = A.ia[i]; j <= A.ia[i + 1] - 1; ++j) s += A.a[j - 1] * x[A.ja[j - 1] - 1];
    y[i] += s;
  }
}
// lsqr_tmatvec2: x = x + A^T y (lib_lsqr.f:237-263)
static void tmatvec2(const CrsView& A, const double* y, double* x) {
  for (int j = 0; j < A.m; ++j)
    for (int64_t i = A.ia[j]; i <= A.ia[j + 1] - 1; ++i) x[A.ja[i - 1] - 1] += A.a[i - 1] * y[j];
}

struct LsqrStats { int istop, itn; double anorm, acond, rnorm, arnorm, xnorm; };

// lsqr_LSQR (lib_lsqr.f:470-1231), damp = 0, wantse = false
static LsqrStats lsqr_core(const CrsView& A, double* u, double* x, double* v, double* w, double atol, double btol,
                           double conlim, int itnlim) {
  const int m = A.m, n = A.n;
  LsqrStats S{};
  const double zero = 0.0, one = 1.0, damp = 0.0;
  int itn = 0, istop = 0, nstop = 0;
  double ctol = zero;
  if (conlim > zero) ctol = one / conlim;
  double anorm = 0, acond = 0, dnorm = 0, dxmax = 0, res2 = 0, psi = 0, xnorm = 0, xnorm1 = 0, cs2 = -one, sn2 = 0, z = 0;
  for (int i = 0; i < n; ++i) { v[i] = zero; x[i] = zero; }
  double alpha = zero, beta = dnrm2(m, u);
  if (beta > zero) {
    dscal(m, one / beta, u);
    tmatvec2(A, u, v);
    alpha = dnrm2(n, v);
  }
  if (alpha > zero) {
    dscal(n, one / alpha, v);
    for (int i = 0; i < n; ++i) w[i] = v[i];
  }
  double arnorm = alpha * beta;
  double rnorm = beta, bnorm = beta, rhobar = alpha, phibar = beta;
  if (arnorm == zero) goto done;
  for (;;) {
    itn++;
    dscal(m, -alpha, u);
    matvec1(A, v, u);
    beta = dnrm2(m, u);
    {
      double temp = d2norm(alpha, beta);
      temp = d2norm(temp, damp);
      anorm = d2norm(anorm, temp);
    }
    if (beta > zero) {
      dscal(m, one / beta, u);
      dscal(n, -beta, v);
      tmatvec2(A, u, v);
      alpha = dnrm2(n, v);
      if (alpha > zero) dscal(n, one / alpha, v);
    }
    double rhbar1 = rhobar;
    double rho = d2norm(rhbar1, beta);
    double cs = rhbar1 / rho, sn = beta / rho;
    double theta = sn * alpha;
    rhobar = -cs * alpha;
    double phi = cs * phibar;
    phibar = sn * phibar;
    double tau = sn * phi;
    double t1 = phi / rho, t2 = -theta / rho, t3 = one / rho, dknorm = zero;
    for (int i = 0; i < n; ++i) {
      double t = w[i];
      x[i] = t1 * t + x[i];
      w[i] = t2 * t + v[i];
      dknorm = (t3 * t) * (t3 * t) + dknorm;
    }
    dknorm = std::sqrt(dknorm);
    dnorm = d2norm(dnorm, dknorm);
    double dxk = std::fabs(phi * dknorm);
    if (dxmax < dxk) dxmax = dxk;
    double delta = sn2 * rho, gambar = -cs2 * rho;
    double rhs = phi - delta * z;
    double zbar = rhs / gambar;
    xnorm = d2norm(xnorm1, zbar);
    double gamma = d2norm(gambar, theta);
    cs2 = gambar / gamma;
    sn2 = theta / gamma;
    z = rhs / gamma;
    xnorm1 = d2norm(xnorm1, z);
    acond = anorm * dnorm;
    res2 = d2norm(res2, psi);
    rnorm = d2norm(res2, phibar);
    arnorm = alpha * std::fabs(tau);
    double test1 = rnorm / bnorm;
    double test2 = zero;
    if (rnorm > zero) test2 = arnorm / (anorm * rnorm);
    double test3 = one / acond;
    double tt1 = test1 / (one + anorm * xnorm / bnorm);
    double rtol = btol + atol * anorm * xnorm / bnorm;
    double tt3 = one + test3, tt2 = one + test2;
    tt1 = one + tt1;
    if (itn >= itnlim) istop = 5;
    if (tt3 <= one) istop = 4;
    if (tt2 <= one) istop = 2;
    if (tt1 <= one) istop = 1;
    if (test3 <= ctol) istop = 4;
    if (test2 <= atol) istop = 2;
    if (test1 <= rtol) istop = 1;
    if (istop == 0) nstop = 0;
    else {
      int nconv = 1;
      nstop++;
      if (nstop < nconv && itn < itnlim) istop = 0;
    }
    if (istop != 0) break;
  }
done:
  S.istop = istop; S.itn = itn; S.anorm = anorm; S.acond = acond; S.rnorm = rnorm; S.arnorm = arnorm; S.xnorm = xnorm;
  return S;
}

// lsqr_precon (lib_lsqr.f:131-167): q = 1/||A(:,j)||, A <- A diag(q) in place
static void lsqr_precon(int m, int n, int64_t nnz, double* q, const int64_t* ia, const int* ja, double* a) {
  (void)nnz;
  for (int i = 0; i < n; ++i) q[i] = 0.0;
  for (int j = 0; j < m; ++j)
    for (int64_t i = ia[j]; i <= ia[j + 1] - 1; ++i) q[ja[i - 1] - 1] += a[i - 1] * a[i - 1];
  for (int i = 0; i < n; ++i) q[i] = 1.0 / std::sqrt(q[i]);
  for (int i = 0; i < m; ++i)
    for (int64_t ij = ia[i]; ij <= ia[i + 1] - 1; ++ij) a[ij - 1] *= q[ja[ij - 1] - 1];
}

// lsqr_solve (lib_lsqr.f:33-127)
static LsqrStats lsqr_solve(int m, int n, int64_t nnz, int& maxit, double eps, int& nit, int& ierr, const double* q,
                            const int64_t* ia, const int* ja, double* a, const double* b, double* x) {
  std::vector<double> x0(n), wm(m, 0.0), u(m), v(n), w(n);
  const double conlim = 1.0e8;
  if (maxit == 0) maxit = 10 * (m + n + 50);
  for (int i = 0; i < n; ++i) x0[i] = x[i];
  for (int i = 0; i < n; ++i) x[i] = x[i] / q[i];
  CrsView A{m, n, nnz, ia, ja, a};
  matvec1(A, x, wm.data());
  for (int i = 0; i < m; ++i) u[i] = b[i] - wm[i];
  double nrm_r = dnrm2(m, u.data()), nrm_b = dnrm2(m, b);
  double atol = eps, btol = eps * nrm_b / nrm_r;
  LsqrStats S = lsqr_core(A, u.data(), x, v.data(), w.data(), atol, btol, conlim, maxit);
  nit = S.itn;
  for (int i = 0; i < n; ++i) x[i] = q[i] * x[i];
  for (int i = 0; i < n; ++i) x[i] = x0[i] + x[i];
  ierr = (S.istop > 3) ? S.istop : 0;
  return S;
}

// CalFluxIntegralSingleWall (lib_particle.f90:1880-1904) and
// getTorqueIntegrateFluxes (lib_particle.f90:1793-1831)
static void force_torque(const Problem& P, const double* qx, const double* qy, const double* qz, int wall, double F[3],
                         double T[3]) {
  F[0] = F[1] = F[2] = 0.0;
  T[0] = T[1] = T[2] = 0.0;
  for (int i = 0; i < P.nelem; ++i)
    if (P.bcid[i] == wall) {
      F[0] += P.area[i] * qx[i]; F[1] += P.area[i] * qy[i]; F[2] += P.area[i] * qz[i];
    }
  for (int i = 0; i < P.nelem; ++i) {
    if (P.bcid[i] != wall) continue;
    double q[3] = {qx[i], qy[i], qz[i]}, r[3] = {0, 0, 0}, cp[3];
    for (int in = 0; in < P.nno[i]; ++in)
      for (int j = 0; j < 3; ++j) r[j] += P.x[3 * P.con[4 * i + in] + j];
    for (int j = 0; j < 3; ++j) r[j] /= (double)P.nno[i];
    cp[0] = r[1] * q[2] - r[2] * q[1];
    cp[1] = -r[0] * q[2] + r[2] * q[0];
    cp[2] = r[0] * q[1] - r[1] * q[0];
    for (int j = 0; j < 3; ++j) T[j] += P.area[i] * cp[j];
  }
}

// -----------------------------------------------------------------------------
// The LIS path of the Stokes system (SLET LIS): StokesBigSystemSOLVElis
// (lib_StokesLis.f90:4-56) solves, with the LIS library, the square system whose
// row of every equation is the number of its own unknown (DivideRows,
// lib_StokesLis.f90:66-161: row = stk%col of the node component for a u-source
// equation, stk%qcol of the element component for a q-source one), right-hand
// side rhsM * known values (plis_rhs_matvec, mod_plis.f90:93-107), and the LIS
// options of the and.inp key LISS, default "-i bicgstab -p jacobi -tol 1.0e-8
// -maxiter 1000" (mod_par.f90:288).  LIS (2.1.6 in the reference's container
// build, 2.1.10 in its install notes) is not part of the reference sources;
// restated here is the published preconditioned BiCGSTAB of van der Vorst (1992)
// in the form of Barrett et al., "Templates for the Solution of Linear Systems"
// (SIAM 1994, Fig. 2.10), with the Jacobi preconditioner M = diag(A), a zero
// initial guess (LIS's default) and the stop ||b - A x||_2 <= tol ||b||_2.
// status: 0 converged, 1 iteration limit, 2 breakdown (rho, r~.v, t.t or omega
// zero).
// -----------------------------------------------------------------------------
struct LisSystem {
  int n = 0;
  std::vector<int64_t> ia;  // 0-based CSR in the LIS row order
  std::vector<int> ja;
  std::vector<double> a, diag;
  std::vector<int> row_of_crs;  // CRS-path row -> LIS row
};

// Builds the LIS-ordered system from the CRS-path system of stk_form_crs.
// Returns false if the equations are not one per unknown (contact conditions).
static bool lis_system(const Problem& P, LisSystem& L) {
  const Eqn& S = P.stk;
  const CRS& A = S.sys;
  if (A.neq != S.nx) return false;
  L.n = S.nx;
  L.row_of_crs.assign(A.neq, -1);
  int row = 0;
  for (int i = 0; i < P.sd_nnodes; ++i)
    for (int een = 0; een < 3; ++een) {
      const int bc = P.knownOf(een, P.BCidList[i]);
      if (bc == iFlux || bc == iContact) L.row_of_crs[row++] = S.col[P.nodeList[i] + een * P.nnodes] - 1;
    }
  for (int i = 0; i < P.sd_nqnodes; ++i)
    for (int een = 0; een < 3; ++een) {
      const int bc = P.knownOf(een, P.qbcidList[i]);
      if (bc == iFunction || bc == iContact) L.row_of_crs[row++] = S.qcol[P.qnodeList[i] + een * P.nelem] - 1;
    }
  std::vector<int> crs_of_row(L.n, -1);
  for (int r = 0; r < A.neq; ++r) {
    const int lr = L.row_of_crs[r];
    if (lr < 0 || lr >= L.n || crs_of_row[lr] >= 0) return false;
    crs_of_row[lr] = r;
  }
  L.ia.assign(L.n + 1, 0);
  L.ja.clear();
  L.a.clear();
  L.diag.assign(L.n, 0.0);
  for (int lr = 0; lr < L.n; ++lr) {
    const int r = crs_of_row[lr];
    for (int64_t k = A.i[r] - 1; k < A.i[r + 1] - 1; ++k) {
      L.ja.push_back(A.j[k] - 1);
      L.a.push_back(A.v[k]);
      if (A.j[k] - 1 == lr) L.diag[lr] = A.v[k];
    }
    L.ia[lr + 1] = (int64_t)L.a.size();
  }
  return true;
}

static void lis_matvec(const LisSystem& L, const double* x, double* y) {
  for (int i = 0; i < L.n; ++i) {
    double s = 0.0;
    for (int64_t k = L.ia[i]; k < L.ia[i + 1]; ++k) s += L.a[k] * x[L.ja[k]];
    y[i] = s;
  }
}

static double dot(int n, const double* a, const double* b) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

// Preconditioned BiCGSTAB (Templates Fig. 2.10) with M = diag(A), x0 = 0.
static int bicgstab_jacobi(const LisSystem& L, const double* b, double* x, double tol, int maxiter, int& iters,
                           double& relres) {
  const int n = L.n;
  std::vector<double> r(b, b + n), rt(b, b + n), p(n, 0.0), v(n, 0.0), ph(n), s(n), sh(n), t(n);
  std::fill(x, x + n, 0.0);
  const double bnrm = std::sqrt(dot(n, b, b));
  iters = 0;
  relres = 1.0;
  if (bnrm == 0.0) { relres = 0.0; return 0; }
  for (int i = 0; i < n; ++i)
    if (L.diag[i] == 0.0) return 2;
  double rho_old = 1.0, alpha = 1.0, omega = 1.0;
  for (int it = 1; it <= maxiter; ++it) {
    iters = it;
    const double rho = dot(n, rt.data(), r.data());
    if (rho == 0.0) return 2;
    if (it == 1) p = r;
    else {
      const double beta = (rho / rho_old) * (alpha / omega);
      for (int i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
    }
    for (int i = 0; i < n; ++i) ph[i] = p[i] / L.diag[i];
    lis_matvec(L, ph.data(), v.data());
    const double rtv = dot(n, rt.data(), v.data());
    if (rtv == 0.0) return 2;
    alpha = rho / rtv;
    for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
    const double snrm = std::sqrt(dot(n, s.data(), s.data())) / bnrm;
    if (snrm <= tol) {
      for (int i = 0; i < n; ++i) x[i] += alpha * ph[i];
      relres = snrm;
      return 0;
    }
    for (int i = 0; i < n; ++i) sh[i] = s[i] / L.diag[i];
    lis_matvec(L, sh.data(), t.data());
    const double tt = dot(n, t.data(), t.data());
    if (tt == 0.0) return 2;
    omega = dot(n, t.data(), s.data()) / tt;
    for (int i = 0; i < n; ++i) x[i] += alpha * ph[i] + omega * sh[i];
    for (int i = 0; i < n; ++i) r[i] = s[i] - omega * t[i];
    relres = std::sqrt(dot(n, r.data(), r.data())) / bnrm;
    if (relres <= tol) return 0;
    if (omega == 0.0) return 2;
    rho_old = rho;
  }
  return 1;
}

// LIS with the options "-i gmres -restart m" (the LISS key of and.inp,
// mod_par.f90:418): restarted GMRES(m) of Saad and Schultz (SIAM J. Sci. Stat.
// Comput. 7, 1986; Saad, "Iterative Methods for Sparse Linear Systems", 2nd ed.,
// Alg. 6.9: Arnoldi with Givens rotations), x0 = 0, right preconditioned so that
// it minimises ||b - A x||_2 and stops at ||b - A x|| <= tol ||b||.  The
// preconditioner M is block diagonal: the blocks of the unknowns that belong to
// one node or one element (groups, LIS row numbers), inverted in FP64.  Gram-
// Schmidt twice per step (CGS2).  At the end of every cycle the residual is
// recomputed as b - A x; a cycle that does not lower it by 10 % stops with
// status 3.  status: 0 converged, 1 iteration limit, 3 stagnated.
static void block_inverses(const LisSystem& L, const std::vector<std::vector<int>>& groups,
                           std::vector<std::vector<double>>& inv) {
  inv.assign(groups.size(), {});
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const std::vector<int>& g = groups[gi];
    const int k = (int)g.size();
    std::vector<double> B((size_t)k * k, 0.0), I((size_t)k * k, 0.0);
    for (int a = 0; a < k; ++a) {
      for (int64_t t = L.ia[g[a]]; t < L.ia[g[a] + 1]; ++t)
        for (int b = 0; b < k; ++b)
          if (L.ja[t] == g[b]) B[(size_t)a * k + b] = L.a[t];
      I[(size_t)a * k + a] = 1.0;
    }
    // Gauss-Jordan with partial pivoting on the k x k block (k <= 3)
    for (int col = 0; col < k; ++col) {
      int piv = col;
      for (int r = col + 1; r < k; ++r)
        if (std::fabs(B[(size_t)r * k + col]) > std::fabs(B[(size_t)piv * k + col])) piv = r;
      for (int c2 = 0; c2 < k; ++c2) {
        std::swap(B[(size_t)col * k + c2], B[(size_t)piv * k + c2]);
        std::swap(I[(size_t)col * k + c2], I[(size_t)piv * k + c2]);
      }
      const double d = B[(size_t)col * k + col];
      for (int c2 = 0; c2 < k; ++c2) {
        B[(size_t)col * k + c2] /= d;
        I[(size_t)col * k + c2] /= d;
      }
      for (int r = 0; r < k; ++r) {
        if (r == col) continue;
        const double f = B[(size_t)r * k + col];
        for (int c2 = 0; c2 < k; ++c2) {
          B[(size_t)r * k + c2] -= f * B[(size_t)col * k + c2];
          I[(size_t)r * k + c2] -= f * I[(size_t)col * k + c2];
        }
      }
    }
    inv[gi] = I;
  }
}

static void block_apply(const std::vector<std::vector<int>>& groups, const std::vector<std::vector<double>>& inv,
                        const double* v, double* z) {
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const std::vector<int>& g = groups[gi];
    const int k = (int)g.size();
    for (int a = 0; a < k; ++a) {
      double s = 0.0;
      for (int b = 0; b < k; ++b) s += inv[gi][(size_t)a * k + b] * v[g[b]];
      z[g[a]] = s;
    }
  }
}

static int gmres_block(const LisSystem& L, const std::vector<std::vector<int>>& groups, const double* b, double* x,
                       double tol, int maxiter, int restart, int& iters, double& relres) {
  const int n = L.n, mr = restart;
  std::vector<std::vector<double>> inv;
  block_inverses(L, groups, inv);
  std::fill(x, x + n, 0.0);
  iters = 0;
  const double bnrm = std::sqrt(dot(n, b, b));
  relres = bnrm > 0.0 ? 1.0 : 0.0;
  if (bnrm == 0.0) return 0;
  std::vector<double> r(b, b + n), w(n), z(n), Ax(n);
  std::vector<std::vector<double>> V(mr, std::vector<double>(n));
  std::vector<double> H((size_t)(mr + 1) * mr, 0.0), cs(mr), sn(mr), g(mr + 1), y(mr), h(mr + 1);
  double prev = 1.0;
  bool first = true;
  for (;;) {
    const double beta = std::sqrt(dot(n, r.data(), r.data()));
    relres = beta / bnrm;
    if (relres <= tol) return 0;
    if (iters >= maxiter) return 1;
    if (!first && relres > 0.9 * prev) return 3;
    first = false;
    prev = relres;
    for (int i = 0; i < n; ++i) V[0][i] = r[i] / beta;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int jc = 0;
    for (int j = 0; j < mr; ++j) {
      block_apply(groups, inv, V[j].data(), z.data());
      lis_matvec(L, z.data(), w.data());
      for (int i = 0; i <= j; ++i) H[(size_t)i * mr + j] = 0.0;
      for (int pass = 0; pass < 2; ++pass) {
        for (int i = 0; i <= j; ++i) h[i] = dot(n, V[i].data(), w.data());
        for (int i = 0; i <= j; ++i) {
          H[(size_t)i * mr + j] += h[i];
          for (int t = 0; t < n; ++t) w[t] -= h[i] * V[i][t];
        }
      }
      const double hn = std::sqrt(dot(n, w.data(), w.data()));
      for (int l = 0; l < j; ++l) {
        const double x0 = H[(size_t)l * mr + j], x1 = H[(size_t)(l + 1) * mr + j];
        H[(size_t)l * mr + j] = cs[l] * x0 + sn[l] * x1;
        H[(size_t)(l + 1) * mr + j] = -sn[l] * x0 + cs[l] * x1;
      }
      const double hd = H[(size_t)j * mr + j];
      const double rr = std::hypot(hd, hn);
      cs[j] = rr > 0.0 ? hd / rr : 1.0;
      sn[j] = rr > 0.0 ? hn / rr : 0.0;
      H[(size_t)j * mr + j] = rr;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      ++iters;
      jc = j + 1;
      if (std::fabs(g[j + 1]) / bnrm <= tol || !(hn > 0.0) || iters >= maxiter || j + 1 == mr) break;
      for (int t = 0; t < n; ++t) V[j + 1][t] = w[t] / hn;
    }
    for (int l = jc - 1; l >= 0; --l) {
      double v = g[l];
      for (int q = l + 1; q < jc; ++q) v -= H[(size_t)l * mr + q] * y[q];
      const double d = H[(size_t)l * mr + l];
      y[l] = d != 0.0 ? v / d : 0.0;
    }
    std::fill(w.begin(), w.end(), 0.0);
    for (int l = 0; l < jc; ++l)
      for (int t = 0; t < n; ++t) w[t] += y[l] * V[l][t];
    block_apply(groups, inv, w.data(), z.data());
    for (int t = 0; t < n; ++t) x[t] += z[t];
    lis_matvec(L, x, Ax.data());
    for (int t = 0; t < n; ++t) r[t] = b[t] - Ax[t];
  }
}

// -----------------------------------------------------------------------------
// Post-processing of a solved Stokes / Laplace field: the surface pressure and
// values at points inside the domain.  Not on the solve path; the integrals of
// a domain point are the element integrals of the assembly with no singular
// element (isrc = 0).
// -----------------------------------------------------------------------------

// pressureStokes (lib_Stokes.f90:4-94): pressure at the q-source points
// (element centroids) from the pressure rows of the integral matrices, in the
// differenced form of Ingber (1991) for the stresslet part, times 2 for a
// point on a smooth wall.  u: 3 x nnodes, q: 3 x nelem (component-major).  The
// centroid velocity is InterpolateToQMesh (lib_mesh.f90:635-684): 1/3 per
// node on a triangle, the bilinear shape functions at the centre (1/4) on a
// quad.  As in the reference, row r of the q-source rows takes the centroid
// velocity of element r and writes p[r]; with the subdomain's elements in
// mesh order (walls listed in the order the mesh holds them) row r is element
// r.  The centroid velocity multiplies the row sum of prT, which the pressure
// correction of sdIntRowQStokes (lib_Stokes.f90:1851-1863) sets to zero, so it
// moves p by rounding only.  Needs the Stokes integral matrices
// (orc_form_integrals).
static void pressure_stokes(const Problem& P, const double* u, const double* q, double* p) {
  const double osemPi = (double)std::atan(1.0f) * 4.0 * 8.0;  // single-precision ATAN(1.0)
  const int nn = P.nnodes, ne = P.nelem;
  std::vector<double> vq(3 * (size_t)ne, 0.0);
  for (int e = 0; e < ne; ++e) {
    const double f = (P.type[e] == 2) ? 1.0 / 3.0 : 0.25;
    for (int c = 0; c < 3; ++c) {
      double acc = 0.0;
      for (int k = 0; k < P.nno[e]; ++k) acc += f * u[(size_t)c * nn + P.con[4 * e + k]];
      vq[(size_t)c * ne + e] = acc;
    }
  }
  const size_t nsp = (size_t)P.nsp;
  const std::vector<double>&prTx = P.M[6], &prTy = P.M[7], &prTz = P.M[8];
  const std::vector<double>&prGx = P.M[15], &prGy = P.M[16], &prGz = P.M[17];
  for (int row = 0; row < P.sd_nqnodes; ++row) {
    const size_t i = (size_t)P.sd_nnodes + row;
    double acc = 0.0;
    for (int j = 0; j < P.sd_nnodes; ++j) {
      const int icol = P.nodeList[j];
      const size_t k = (size_t)j * nsp + i;
      acc = acc + P.diff * (prTx[k] * (u[icol] - vq[row]) + prTy[k] * (u[(size_t)nn + icol] - vq[(size_t)ne + row]) +
                            prTz[k] * (u[2 * (size_t)nn + icol] - vq[2 * (size_t)ne + row]));
    }
    for (int j = 0; j < P.sd_nqnodes; ++j) {
      const int icol = P.qnodeList[j];
      const size_t k = (size_t)j * nsp + i;
      acc = acc - (prGx[k] * q[icol] + prGy[k] * q[(size_t)ne + icol] + prGz[k] * q[2 * (size_t)ne + icol]);
    }
    p[row] = -acc / osemPi * 2.0;
  }
}

// GetStokesDomainValue (lib_Stokes.f90:3043-3373): velocity (out[0..2]) and
// pressure (out[3]) at a point s of the domain from the boundary velocity u
// (3 x nnodes) and traction q (3 x nelem).  Triangles: Triangle_StokesInt with
// isrc = 0 (the regular rule; the near-singular options of the problem apply);
// quads: the regular branch of Quad_StokesInt (one cell).  err: the
// reference's check of the point -- the stresslet diagonal sums to 8 pi and
// sum G.n vanishes for a point inside; getStokesDV (lib_Stokes.f90:3020-3035)
// flags err > 1e-2 as outside.
static void stokes_domain_value(const Problem& P, const double s[3], const double* u, const double* q, double out[4],
                                double& err) {
  const double osemPi = (double)std::atan(1.0f) * 4.0 * 8.0;
  const int nn = P.nnodes, ne = P.nelem;
  StkRow R(nn, ne);
  StkElem E;
  for (size_t jj = 0; jj < P.loWalls.size(); ++jj) {
    const int iWall = P.loWalls[jj];
    const double mm = P.normMul[jj];
    for (int ie = 0; ie < ne; ++ie) {
      if (P.bcid[ie] != iWall) continue;
      double v[12];
      element_vertices(P, ie, v);
      E.zero();
      if (P.type[ie] == 2) {
        const double n[3] = {mm * P.normal[3 * ie], mm * P.normal[3 * ie + 1], mm * P.normal[3 * ie + 2]};
        tri_walk(P.opt, v, s, P.area[ie], 0, [&](const Bary& B, double a, bool sk) { tri_stk_sub(P.tri, v, B, s, n, a, E, sk); });
      } else {
        quad_stk_regular(P.iqud, v, s, mm, E, 1);
      }
      for (int j = 0; j < P.nno[ie]; ++j) {
        const int nd = P.con[4 * ie + j];
        for (int k = 0; k < 6; ++k) R.t(k, nd) += E.T[k][j];
        for (int k = 0; k < 3; ++k) R.t(6 + k, nd) += E.prT[k][j];
      }
      for (int k = 0; k < 6; ++k) R.g(k, ie) = E.G[k];
      for (int k = 0; k < 3; ++k) R.g(6 + k, ie) = E.prG[k];
    }
  }
  err = -9.99;
  double cx = 0, cy = 0, cz = 0;
  for (int i = 0; i < nn; ++i) { cx -= R.t(0, i); cy -= R.t(3, i); cz -= R.t(5, i); }
  err = std::max(err, std::fabs(cx / osemPi - 1.0));
  err = std::max(err, std::fabs(cy / osemPi - 1.0));
  err = std::max(err, std::fabs(cz / osemPi - 1.0));
  cx = cy = cz = 0;
  for (int i = 0; i < ne; ++i) {
    const double m = P.multiOf(P.bcid[i]);
    const double* n = &P.normal[3 * i];
    cx = cx - R.g(0, i) * n[0] * m - R.g(1, i) * n[1] * m - R.g(2, i) * n[2] * m;
    cy = cy - R.g(1, i) * n[0] * m - R.g(3, i) * n[1] * m - R.g(4, i) * n[2] * m;
    cz = cz - R.g(2, i) * n[0] * m - R.g(4, i) * n[1] * m - R.g(5, i) * n[2] * m;
  }
  err = std::max(err, std::fabs(cx));
  err = std::max(err, std::fabs(cy));
  err = std::max(err, std::fabs(cz));
  const double *ux = u, *uy = u + nn, *uz = u + 2 * (size_t)nn;
  const double *qx = q, *qy = q + ne, *qz = q + 2 * (size_t)ne;
  double rx = 0, ry = 0, rz = 0, pr = 0;
  for (int i = 0; i < nn; ++i) {
    rx = rx + R.t(0, i) * ux[i]; rx = rx + R.t(1, i) * uy[i]; rx = rx + R.t(2, i) * uz[i];
    ry = ry + R.t(1, i) * ux[i]; ry = ry + R.t(3, i) * uy[i]; ry = ry + R.t(4, i) * uz[i];
    rz = rz + R.t(2, i) * ux[i]; rz = rz + R.t(4, i) * uy[i]; rz = rz + R.t(5, i) * uz[i];
    pr = pr + P.diff * (R.t(6, i) * ux[i] + R.t(7, i) * uy[i] + R.t(8, i) * uz[i]);
  }
  for (int i = 0; i < ne; ++i) {
    rx = rx + R.g(0, i) * qx[i] / P.diff; rx = rx + R.g(1, i) * qy[i] / P.diff; rx = rx + R.g(2, i) * qz[i] / P.diff;
    ry = ry + R.g(1, i) * qx[i] / P.diff; ry = ry + R.g(3, i) * qy[i] / P.diff; ry = ry + R.g(4, i) * qz[i] / P.diff;
    rz = rz + R.g(2, i) * qx[i] / P.diff; rz = rz + R.g(4, i) * qy[i] / P.diff; rz = rz + R.g(5, i) * qz[i] / P.diff;
    pr = pr - (R.g(6, i) * qx[i] + R.g(7, i) * qy[i] + R.g(8, i) * qz[i]);
  }
  out[0] = -rx / osemPi;
  out[1] = -ry / osemPi;
  out[2] = -rz / osemPi;
  out[3] = -pr / osemPi;
}

// GetSubDomainValue (lib_domain.f90:210-344) with VerifyIntegrals
// (lib_domain.f90:354-391): the Laplace field at a point s of the domain from
// the boundary values u (nnodes) and fluxes q (nelem), divided by the point's
// free-term coefficient c = -sum H (1 inside).  Triangles: Triangle_BEMInt with
// isrc = 0; quads: the regular branch of Quad_BEMInt (one cell).  err: the
// linear-field check (u = x_j, q = n_j) of VerifyIntegrals.
static double laplace_domain_value(const Problem& P, const double s[3], const double* u, const double* q, double& err) {
  const int nn = P.nnodes, ne = P.nelem;
  std::vector<double> rowH(nn, 0.0), rowG(ne, 0.0);
  for (size_t jj = 0; jj < P.loWalls.size(); ++jj) {
    const int iWall = P.loWalls[jj];
    const double mm = P.normMul[jj];
    for (int ie = 0; ie < ne; ++ie) {
      if (P.bcid[ie] != iWall) continue;
      double v[12], integ = 0.0, inteH[4] = {0, 0, 0, 0};
      element_vertices(P, ie, v);
      if (P.type[ie] == 2) {
        const double n[3] = {mm * P.normal[3 * ie], mm * P.normal[3 * ie + 1], mm * P.normal[3 * ie + 2]};
        double o[4] = {0, 0, 0, 0};
        tri_walk(P.opt, v, s, P.area[ie], 0, [&](const Bary& B, double a, bool sk) { tri_lap_sub(P.tri, v, B, s, n, a, o, sk); });
        integ = o[0]; inteH[0] = o[1]; inteH[1] = o[2]; inteH[2] = o[3];
      } else {
        double o[5];
        quad_lap_regular(P.iqud, v, s, mm, o, 1);
        integ = o[0];
        for (int k = 0; k < 4; ++k) inteH[k] = o[1 + k];
      }
      for (int j = 0; j < P.nno[ie]; ++j) rowH[P.con[4 * ie + j]] += inteH[j];
      rowG[ie] = integ;
    }
  }
  double c = 0.0;
  for (int i = 0; i < nn; ++i) c = c - rowH[i];
  err = 0.0;
  for (int j = 0; j < 3; ++j) {
    double cc = 0.0;
    for (int i = 0; i < nn; ++i) cc = cc + rowH[i] * P.x[3 * i + j];
    cc = cc + s[j] * c;
    for (int i = 0; i < ne; ++i) cc = cc - rowG[i] * P.normal[3 * i + j] * P.multiOf(P.bcid[i]);
    err = std::max(err, std::fabs(cc));
  }
  double res = 0.0;
  for (int i = 0; i < nn; ++i) res = res - rowH[i] * u[i];
  for (int i = 0; i < ne; ++i) {
    double multi = 0.0;  // GetNormalMulti (lib_domain.f90:188-205): 0 for an element of no subdomain wall
    for (size_t jj = 0; jj < P.loWalls.size(); ++jj)
      if (P.bcid[i] == P.loWalls[jj]) multi = P.normMul[jj];
    res = res - rowG[i] * q[i] * multi / P.diff;
  }
  return res / c;
}

}  // namespace orc

using namespace orc;

// =============================================================================
// C API used by the tests (ctypes)
// =============================================================================
// -----------------------------------------------------------------------------
// LINPACK direct solver of the FULL path (lib_solveFM.f): dgefa :198, dgesl
// :318, with the reference-BLAS idamax (first index of the largest |x|), dscal
// and daxpy.  a is column-major a(lda, n); ipvt holds 1-based pivot rows as
// doubles (the reference declares it REAL(8)).
// -----------------------------------------------------------------------------
static int linpack_dgefa(double* a, int lda, int n, double* ipvt) {
  auto A = [&](int i, int j) -> double& { return a[(size_t)(j - 1) * lda + (i - 1)]; };  // 1-based
  int info = 0;
  const int nm1 = n - 1;
  for (int k = 1; k <= nm1; ++k) {
    const int kp1 = k + 1;
    // l = idamax(n-k+1, a(k,k), 1) + k - 1
    int l = k;
    double dmax = std::fabs(A(k, k));
    for (int i = k + 1; i <= n; ++i)
      if (std::fabs(A(i, k)) > dmax) { dmax = std::fabs(A(i, k)); l = i; }
    ipvt[k - 1] = (double)l;
    if (A(l, k) == 0.0) { info = k; continue; }
    if (l != k) std::swap(A(l, k), A(k, k));
    double t = -1.0 / A(k, k);
    for (int i = k + 1; i <= n; ++i) A(i, k) *= t;  // dscal(n-k, t, a(k+1,k), 1)
    for (int j = kp1; j <= n; ++j) {
      t = A(l, j);
      if (l != k) { A(l, j) = A(k, j); A(k, j) = t; }
      for (int i = k + 1; i <= n; ++i) A(i, j) += t * A(i, k);  // daxpy(n-k, t, a(k+1,k), 1, a(k+1,j), 1)
    }
  }
  ipvt[n - 1] = (double)n;
  if (A(n, n) == 0.0) info = n;
  return info;
}
static void linpack_dgesl(const double* a, int lda, int n, const double* ipvt, double* b, int job) {
  auto A = [&](int i, int j) { return a[(size_t)(j - 1) * lda + (i - 1)]; };
  auto B = [&](int i) -> double& { return b[i - 1]; };
  const int nm1 = n - 1;
  if (job == 0) {
    for (int k = 1; k <= nm1; ++k) {
      const int l = (int)ipvt[k - 1];
      const double t = B(l);
      if (l != k) { B(l) = B(k); B(k) = t; }
      for (int i = k + 1; i <= n; ++i) B(i) += t * A(i, k);
    }
    for (int kb = 1; kb <= n; ++kb) {
      const int k = n + 1 - kb;
      B(k) = B(k) / A(k, k);
      const double t = -B(k);
      for (int i = 1; i <= k - 1; ++i) B(i) += t * A(i, k);
    }
  } else {
    for (int k = 1; k <= n; ++k) {
      double t = 0.0;
      for (int i = 1; i <= k - 1; ++i) t += A(i, k) * B(i);
      B(k) = (B(k) - t) / A(k, k);
    }
    for (int kb = 1; kb <= nm1; ++kb) {
      const int k = n - kb;
      double t = 0.0;
      for (int i = k + 1; i <= n; ++i) t += A(i, k) * B(i);
      B(k) += t;
      const int l = (int)ipvt[k - 1];
      if (l != k) std::swap(B(l), B(k));
    }
  }
}

extern "C" {

int orc_wx_rule(int itri, double* l1, double* l2, double* l3, double* w) {
  TriRule r = wx_rule(itri);
  for (int i = 0; i < r.n; ++i) { l1[i] = r.l1[i]; l2[i] = r.l2[i]; l3[i] = r.l3[i]; w[i] = r.w[i]; }
  return r.n;
}

// Triangle_TestIntegration (mod_trikotnik.f90:108-191): out = integ1..integ4
void orc_triangle_test(int itri, double out[4]) {
  TriRule R = wx_rule(itri);
  double x1 = 0, y1 = 0, z1 = 1, x2 = 2, y2 = 0, z2 = 1, x3 = 2, y3 = 2, z3 = 1, sx = 0, sy = 0, sz = 1;
  double area = tri_area(x1, y1, z1, x2, y2, z2, x3, y3, z3);
  double i1 = 0, i2 = 0, i3 = 0, i4 = 0;
  for (int i = 0; i < R.n; ++i) {
    double x = R.l1[i] * x1 + R.l2[i] * x2 + R.l3[i] * x3;
    double y = R.l1[i] * y1 + R.l2[i] * y2 + R.l3[i] * y3;
    double z = R.l1[i] * z1 + R.l2[i] * z2 + R.l3[i] * z3;
    i1 += R.w[i] * std::pow(x, 10) * std::pow(y, 10);
    i2 += R.w[i] * std::sin(x * y);
    i3 += R.w[i] * std::exp(-x * y);
    i4 += R.w[i] / std::sqrt((x - sx) * (x - sx) + (y - sy) * (y - sy) + (z - sz) * (z - sz));
  }
  out[0] = i1 * area; out[1] = i2 * area; out[2] = i3 * area;
  out[3] = i4 * area / (16.0 * std::atan(1.0));
}

double orc_tri_area(const double v[9]) { return tri_area(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8]); }
double orc_si_tri_lap(const double v[9], int isrc) { return si_tri_lap(v, orc_tri_area(v), isrc); }
void orc_si_tri_stk(const double v[9], int isrc, double G[6]) { si_tri_stk(v, orc_tri_area(v), isrc, G); }
double orc_si_qua_lap(const double q[12], int isrc) { return si_qua_lap(q, isrc); }
// the polar singular quad scheme: out[0] = G, out[1..4] = H (Laplace); G[6] (Stokes)
void orc_quad_lap_polar(int iqud, const double q[12], const double s[3], int isrc, double multi, double out[5]) {
  quad_lap_polar(iqud, q, s, isrc, multi, out);
}
void orc_quad_stk_polar(int iqud, const double q[12], const double s[3], int isrc, double multi, double G[6]) {
  StkElem E;
  quad_stk_polar(iqud, q, s, isrc, multi, E);
  for (int k = 0; k < 6; ++k) G[k] = E.G[k];
}
void orc_si_qua_stk(const double q[12], int isrc, double G[6]) { si_qua_stk(q, isrc, G); }

// Regular (non-singular) element integrals, for kernel-level checks.
// Triangle Laplace: out = {G, H1, H2, H3}; n is the (already multiplied) normal.
void orc_tri_lap_regular(int itri, const double v[9], const double s[3], const double n[3], double out[4]) {
  TriRule R = wx_rule(itri);
  for (int k = 0; k < 4; ++k) out[k] = 0.0;
  tri_lap_regular(R, v, s, n, orc_tri_area(v), out);
}
// Triangle Stokes: out = G[6], prG[3], T[6][3], prT[3][3]
void orc_tri_stk_regular(int itri, const double v[9], const double s[3], const double n[3], double out[36]) {
  TriRule R = wx_rule(itri);
  StkElem E;
  E.zero();
  tri_stk_regular(R, v, s, n, orc_tri_area(v), E);
  int p = 0;
  for (int k = 0; k < 6; ++k) out[p++] = E.G[k];
  for (int k = 0; k < 3; ++k) out[p++] = E.prG[k];
  for (int k = 0; k < 6; ++k) for (int j = 0; j < 3; ++j) out[p++] = E.T[k][j];
  for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) out[p++] = E.prT[k][j];
}

// Triangle element integrals under the integration options (sing, rdepth,
// near_eta, near_depth of IntegOpt): Laplace out = {G, H1, H2, H3}; Stokes out =
// G[6], prG[3], T[6][3], prT[3][3].  isrc 0 (regular), 1..3 (vertex), 4 (centroid).
void orc_tri_lap_opt(int itri, const double v[9], const double s[3], const double n[3], int isrc, int sing, int rdepth,
                     double near_eta, int near_depth, double out[4]) {
  TriRule R = wx_rule(itri);
  IntegOpt o;
  o.sing = sing; o.rdepth = rdepth; o.near_eta = near_eta; o.near_depth = near_depth;
  for (int k = 0; k < 4; ++k) out[k] = 0.0;
  tri_walk(o, v, s, orc_tri_area(v), isrc, [&](const Bary& B, double a, bool sk) { tri_lap_sub(R, v, B, s, n, a, out, sk); });
}
void orc_tri_stk_opt(int itri, const double v[9], const double s[3], const double n[3], int isrc, int sing, int rdepth,
                     double near_eta, int near_depth, double out[36]) {
  TriRule R = wx_rule(itri);
  IntegOpt o;
  o.sing = sing; o.rdepth = rdepth; o.near_eta = near_eta; o.near_depth = near_depth;
  StkElem E;
  E.zero();
  tri_walk(o, v, s, orc_tri_area(v), isrc, [&](const Bary& B, double a, bool sk) { tri_stk_sub(R, v, B, s, n, a, E, sk); });
  int p = 0;
  for (int k = 0; k < 6; ++k) out[p++] = E.G[k];
  for (int k = 0; k < 3; ++k) out[p++] = E.prG[k];
  for (int k = 0; k < 6; ++k) for (int j = 0; j < 3; ++j) out[p++] = E.T[k][j];
  for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) out[p++] = E.prT[k][j];
}

// ---- problem object ----------------------------------------------------------
// kind 1 = Laplace (1 equation), 2 = Stokes (3 equations).  known[en*nwalls+k]
// is the BC type (1 function, 2 flux, 3 contact) of equation en on wall walls[k].
void* orc_problem_create(int kind, int nnodes, const double* xyz, int nelem, const int* etype, const int* con,
                         const int* bcid, int nwalls, const int* walls, const double* normMul, double diff,
                         const int* known, int itri, int iqud) {
  Problem* P = new Problem();
  P->kind = kind;
  P->neq = (kind == 2) ? 3 : 1;
  P->nnodes = nnodes;
  P->nelem = nelem;
  P->x.assign(xyz, xyz + 3 * (size_t)nnodes);
  P->type.assign(etype, etype + nelem);
  P->nno.resize(nelem);
  for (int e = 0; e < nelem; ++e) P->nno[e] = (etype[e] == 2) ? 3 : 4;
  P->con.assign(con, con + 4 * (size_t)nelem);
  P->bcid.assign(bcid, bcid + nelem);
  P->loWalls.assign(walls, walls + nwalls);
  P->normMul.assign(normMul, normMul + nwalls);
  P->diff = diff;
  P->known.assign(known, known + P->neq * nwalls);
  P->tri = wx_rule(itri);
  P->iqud = iqud;
  geometry(*P);
  setup_subdomain(*P);
  setup_xb(*P);
  if (kind == 2) stk_setup_xb(*P);
  return P;
}
void orc_problem_destroy(void* h) { delete (Problem*)h; }

// HandleCornersEdges (lib_sdBem.f90:112-310), the BiC file's EDGE and CORNER
// directives of the (single) subdomain: every node shared by an element of wall
// w1 and an element of wall w2 (EDGE; CORNER: and of wall w3) takes the wall
// target in BCidList, i.e. the boundary condition of that wall.  The reference
// runs its element loops over the subdomain's element list (the CORNER loop's
// bounds use the global element count, which is the same list for a subdomain
// holding every element); the set of nodes found is the intersection of the
// walls' node sets, which is what is computed here.  The numbering of the
// unknowns follows BCidList and is set up again.
static void renumber(Problem& P) {
  setup_xb(P);
  if (P.kind == 2) stk_setup_xb(P);
}
static std::vector<char> wall_nodes(const Problem& P, int w) {
  std::vector<char> on(P.nnodes, 0);
  for (int e : P.elementList)
    if (P.bcid[e] == w)
      for (int j = 0; j < P.nno[e]; ++j) on[P.con[4 * e + j]] = 1;
  return on;
}
void orc_problem_edge_corner(void* h, int w1, int w2, int w3, int target) {
  Problem* P = (Problem*)h;
  const std::vector<char> a = wall_nodes(*P, w1), b = wall_nodes(*P, w2);
  std::vector<char> c(P->nnodes, 1);
  if (w3 >= 0) c = wall_nodes(*P, w3);
  for (int m = 0; m < P->sd_nnodes; ++m) {
    const int i = P->nodeList[m];
    if (a[i] && b[i] && c[i]) P->BCidList[m] = target;
  }
  renumber(*P);
}
// subdomain%BCidList from the driver: node_wall[global node] = wall id, < 0 keeps
// the node's wall
void orc_problem_set_node_walls(void* h, const int* node_wall) {
  Problem* P = (Problem*)h;
  for (int m = 0; m < P->sd_nnodes; ++m)
    if (node_wall[P->nodeList[m]] >= 0) P->BCidList[m] = node_wall[P->nodeList[m]];
  renumber(*P);
}
// BCidList per global node (-1: not a node of the subdomain)
void orc_problem_node_walls(void* h, int* node_wall) {
  Problem* P = (Problem*)h;
  std::fill(node_wall, node_wall + P->nnodes, -1);
  for (int m = 0; m < P->sd_nnodes; ++m) node_wall[P->nodeList[m]] = P->BCidList[m];
}
// Integration options (IntegOpt) for the next orc_form_integrals.
void orc_problem_set_integration(void* h, int sing, int rdepth, double near_eta, int near_depth) {
  Problem* P = (Problem*)h;
  P->opt.sing = sing; P->opt.rdepth = rdepth; P->opt.near_eta = near_eta; P->opt.near_depth = near_depth;
  P->H.clear(); P->G.clear();
  for (auto& m : P->M) m.clear();
}

// sizes: [nsp, sd_nnodes, sd_nqnodes, neq_rows, nx, nb] of the (big) system
void orc_problem_sizes(void* h, int out[6]) {
  Problem* P = (Problem*)h;
  out[0] = P->nsp; out[1] = P->sd_nnodes; out[2] = P->sd_nqnodes;
  if (P->kind == 2) {
    int neq = 0;
    for (int en = 0; en < 3; ++en) neq += P->eqn[en].neq;
    out[3] = neq; out[4] = P->stk.nx; out[5] = P->stk.nb;
  } else {
    out[3] = P->eqn[0].neq; out[4] = P->eqn[0].nx; out[5] = P->eqn[0].nb;
  }
}
void orc_geometry(void* h, double* normal, double* area, double* centroid) {
  Problem* P = (Problem*)h;
  std::copy(P->normal.begin(), P->normal.end(), normal);
  std::copy(P->area.begin(), P->area.end(), area);
  std::copy(P->qx.begin(), P->qx.end(), centroid);
}
void orc_lists(void* h, int* nodeList, int* qnodeList) {
  Problem* P = (Problem*)h;
  std::copy(P->nodeList.begin(), P->nodeList.end(), nodeList);
  std::copy(P->qnodeList.begin(), P->qnodeList.end(), qnodeList);
}

// CoR_Integrals: fills the dense integral matrices; errs = {fspCerr, qspCerr}
void orc_form_integrals(void* h, double errs[2]) {
  Problem* P = (Problem*)h;
  if (P->kind == 2) stk_form_matrices(*P);
  else lap_form_matrices(*P);
  errs[0] = P->fspCerr;
  errs[1] = P->qspCerr;
}
// Copy one integral matrix (column-major nsp x ncols).  Laplace: 0 H, 1 G.
// Stokes: 0..17 in the order Txx,Txy,Txz,Tyy,Tyz,Tzz,prTx,prTy,prTz,Gxx..Gzz,prGx..prGz.
void orc_get_integral_matrix(void* h, int which, double* out) {
  Problem* P = (Problem*)h;
  const std::vector<double>& M = (P->kind == 2) ? P->M[which] : (which == 0 ? P->H : P->G);
  std::copy(M.begin(), M.end(), out);
}
// One row of integrals for a source point (row r of the nsp rows), full-length
// over global nodes / elements.  Laplace: rowH(nnodes), rowG(nelem).
// Stokes: rowT(9*nnodes) rowG(9*nelem) in the component order above.
double orc_integral_row(void* h, int r, double* rowT, double* rowG) {
  Problem* P = (Problem*)h;
  double err = 0.0;
  if (P->kind == 2) {
    StkRow R(P->nnodes, P->nelem);
    if (r < P->sd_nnodes) stk_row_u(*P, P->nodeList[r], R, err);
    else stk_row_q(*P, P->qnodeList[r - P->sd_nnodes], R, err);
    std::copy(R.T.begin(), R.T.end(), rowT);
    std::copy(R.G.begin(), R.G.end(), rowG);
  } else {
    if (r < P->sd_nnodes) lap_row_u(*P, P->nodeList[r], rowT, rowG, err);
    else lap_row_q(*P, P->qnodeList[r - P->sd_nnodes], rowT, rowG, err);
  }
  return err;
}

// System formation (CRS, 1-based) -- Laplace: per equation 0; Stokes: big system
void orc_form_system(void* h) {
  Problem* P = (Problem*)h;
  if (P->kind == 2) stk_form_crs(*P);
  else lap_form_crs(*P, 0);
}
static CRS& pick_crs(Problem* P, int which) {
  Eqn& E = (P->kind == 2) ? P->stk : P->eqn[0];
  return which == 0 ? E.sys : E.rhs;
}
int64_t orc_crs_nnz(void* h, int which) { return pick_crs((Problem*)h, which).nnz; }
void orc_get_crs(void* h, int which, int64_t* ia, int* ja, double* a) {
  CRS& C = pick_crs((Problem*)h, which);
  std::copy(C.i.begin(), C.i.end(), ia);
  std::copy(C.j.begin(), C.j.end(), ja);
  std::copy(C.v.begin(), C.v.end(), a);
}

// Plain lsqr_precon / lsqr_solve with the reference signature (1-based CRS).
void orc_lsqr_precon(int m, int n, int64_t nnz, double* q, const int64_t* ia, const int* ja, double* a) {
  lsqr_precon(m, n, nnz, q, ia, ja, a);
}
void orc_lsqr_solve(int m, int n, int64_t nnz, int* maxit, double eps, int* nit, int* ierr, const double* q,
                    const int64_t* ia, const int* ja, double* a, const double* b, double* x, double stats[7]) {
  LsqrStats S = lsqr_solve(m, n, nnz, *maxit, eps, *nit, *ierr, q, ia, ja, a, b, x);
  if (stats) {
    stats[0] = S.istop; stats[1] = S.itn; stats[2] = S.anorm; stats[3] = S.acond; stats[4] = S.rnorm;
    stats[5] = S.arnorm; stats[6] = S.xnorm;
  }
}

// Laplace solve (laplace.f90:1-52 + sdSolveCRS lib_CRS.f90:4-142) for known
// nodal u (function walls) / element q (flux walls).  u_io(nnodes), q_io(nelem)
// hold the known values and the initial guess; on return the unknowns.
int orc_laplace_solve(void* h, double* u_io, double* q_io, int maxit, double eps, int* nit) {
  Problem* P = (Problem*)h;
  if (P->kind != 1) return -1;
  if (P->H.empty()) { double e[2]; orc_form_integrals(h, e); }
  lap_form_crs(*P, 0);
  Eqn& E = P->eqn[0];
  E.u.assign(u_io, u_io + P->nnodes);
  E.q.assign(q_io, q_io + P->nelem);
  for (int i = 0; i < P->sd_nnodes; ++i) {
    int isp = P->nodeList[i], bc = P->knownOf(0, P->BCidList[i]);
    if (bc == iFunction) E.b[E.col[isp] - 1] = E.u[isp];
    else E.x[E.col[isp] - 1] = E.u[isp];
  }
  for (int i = 0; i < P->sd_nqnodes; ++i) {
    int isp = P->qnodeList[i], bc = P->knownOf(0, P->qbcidList[i]);
    if (bc == iFlux) E.b[E.qcol[isp] - 1] = E.q[isp];
    else E.x[E.qcol[isp] - 1] = E.q[isp];
  }
  std::vector<double> nb(E.nb), b(E.neq);
  for (int i = 0; i < E.nb; ++i) nb[i] = -E.b[i];
  crs_x_v(E.rhs, nb.data(), b.data());
  lsqr_precon(E.sys.neq, E.nx, E.sys.nnz, E.pivot.data(), E.sys.i.data(), E.sys.j.data(), E.sys.v.data());
  int ierr = 0, mi = maxit;
  lsqr_solve(E.sys.neq, E.nx, E.sys.nnz, mi, eps, *nit, ierr, E.pivot.data(), E.sys.i.data(), E.sys.j.data(),
             E.sys.v.data(), b.data(), E.x.data());
  for (int i = 0; i < P->sd_nnodes; ++i) {
    int isp = P->nodeList[i], bc = P->knownOf(0, P->BCidList[i]);
    E.u[isp] = (bc == iFunction) ? E.b[E.col[isp] - 1] : E.x[E.col[isp] - 1];
  }
  for (int i = 0; i < P->sd_nqnodes; ++i) {
    int isp = P->qnodeList[i], bc = P->knownOf(0, P->qbcidList[i]);
    E.q[isp] = (bc == iFlux) ? E.b[E.qcol[isp] - 1] : E.x[E.qcol[isp] - 1];
  }
  std::copy(E.u.begin(), E.u.end(), u_io);
  std::copy(E.q.begin(), E.q.end(), q_io);
  return ierr;
}

// Stokes: form CRS and precondition once (stokes.f90:109-110); then solve for
// a sequence of boundary states like the 3-sides workflows
// (lib_particle.f90:6-476): u_io[nrhs][3][nnodes] known velocities,
// q_io[nrhs][3][nelem] receives tractions.  x is warm-started from the previous
// right-hand side's solution exactly as the reference does through eqn%q.
// Returns F and T on wall `fwall` per rhs: ft[nrhs][6].
int orc_stokes_solve_sequence(void* h, int nrhs, const double* u_in, double* q_out, int maxit, double eps,
                              int fwall, double* ft, int* nits) {
  Problem* P = (Problem*)h;
  if (P->kind != 2) return -1;
  if (P->M[0].empty()) { double e[2]; orc_form_integrals(h, e); }
  stk_form_crs(*P);
  Eqn& S = P->stk;
  lsqr_precon(S.sys.neq, S.nx, S.sys.nnz, S.pivot.data(), S.sys.i.data(), S.sys.j.data(), S.sys.v.data());
  for (int en = 0; en < 3; ++en) { P->eqn[en].q.assign(P->nelem, 0.0); }
  int ierr_all = 0;
  for (int r = 0; r < nrhs; ++r) {
    for (int en = 0; en < 3; ++en)
      P->eqn[en].u.assign(u_in + ((size_t)r * 3 + en) * P->nnodes, u_in + ((size_t)r * 3 + en + 1) * P->nnodes);
    // formStokesLeftRightHandSideVectors (lib_StokesFull.f90:379-438)
    for (int i = 0; i < P->sd_nnodes; ++i) {
      int isp = P->nodeList[i], wall = P->BCidList[i];
      for (int en = 0; en < 3; ++en) {
        int ispL = isp + en * P->nnodes, bc = P->knownOf(en, wall);
        if (bc == iFunction) S.b[S.col[ispL] - 1] = P->eqn[en].u[isp];
        else S.x[S.col[ispL] - 1] = P->eqn[en].u[isp];
      }
    }
    for (int i = 0; i < P->sd_nqnodes; ++i) {
      int isp = P->qnodeList[i], wall = P->qbcidList[i];
      for (int en = 0; en < 3; ++en) {
        int ispL = isp + en * P->nelem, bc = P->knownOf(en, wall);
        if (bc == iFlux) S.b[S.qcol[ispL] - 1] = P->eqn[en].q[isp];
        else S.x[S.qcol[ispL] - 1] = P->eqn[en].q[isp];
      }
    }
    std::vector<double> b(S.sys.neq);
    crs_x_v(S.rhs, S.b.data(), b.data());
    int ierr = 0, nit = 0, mi = maxit;
    lsqr_solve(S.sys.neq, S.nx, S.sys.nnz, mi, eps, nit, ierr, S.pivot.data(), S.sys.i.data(), S.sys.j.data(),
               S.sys.v.data(), b.data(), S.x.data());
    if (nits) nits[r] = nit;
    if (ierr) ierr_all = ierr;
    // StokesDistributeUnknowns (lib_StokesFull.f90:446-501)
    for (int i = 0; i < P->sd_nqnodes; ++i) {
      int isp = P->qnodeList[i], wall = P->qbcidList[i];
      for (int en = 0; en < 3; ++en) {
        int ispL = isp + en * P->nelem, bc = P->knownOf(en, wall);
        P->eqn[en].q[isp] = (bc == iFlux) ? S.b[S.qcol[ispL] - 1] : S.x[S.qcol[ispL] - 1];
      }
    }
    for (int en = 0; en < 3; ++en)
      std::copy(P->eqn[en].q.begin(), P->eqn[en].q.end(), q_out + ((size_t)r * 3 + en) * P->nelem);
    if (ft) force_torque(*P, P->eqn[0].q.data(), P->eqn[1].q.data(), P->eqn[2].q.data(), fwall, ft + 6 * r, ft + 6 * r + 3);
  }
  return ierr_all;
}

// The LIS path (StokesBigSystemSOLVElis, lib_StokesLis.f90:4): for each of the
// nrhs velocity fields u_in[r][3][nnodes] (known values; the unknown u are not
// used), BiCGSTAB with Jacobi on the LIS-ordered system, then
// StokesDistributeUnknowns into q_out[r][3][nelem] and, for wall fwall, force
// and torque ft[r][6].  nits[r] / status[r] per field (status as
// bicgstab_jacobi, 3: the system is not one equation per unknown).  Returns
// the largest status.
int orc_stokes_solve_lis_m(void* h, int nrhs, const double* u_in, double* q_out, double tol, int maxiter,
                           int fwall, double* ft, int* nits, int* status, double* relres, int method, int restart);
int orc_stokes_solve_lis(void* h, int nrhs, const double* u_in, double* q_out, double tol, int maxiter, int fwall,
                         double* ft, int* nits, int* status, double* relres) {
  return orc_stokes_solve_lis_m(h, nrhs, u_in, q_out, tol, maxiter, fwall, ft, nits, status, relres, 0, 0);
}

// As orc_stokes_solve_lis with the LIS solver chosen: method 0 BiCGSTAB with
// Jacobi (the default options), 1 GMRES(restart) with the node/element block
// preconditioner (gmres_block).
int orc_stokes_solve_lis_m(void* h, int nrhs, const double* u_in, double* q_out, double tol, int maxiter,
                           int fwall, double* ft, int* nits, int* status, double* relres, int method, int restart) {
  Problem* P = (Problem*)h;
  if (P->kind != 2) return -1;
  if (P->M[0].empty()) { double e[2]; orc_form_integrals(h, e); }
  stk_form_crs(*P);
  Eqn& S = P->stk;
  LisSystem L;
  const bool ok = lis_system(*P, L);
  // unknowns of one node or one element (LIS rows = unknown numbers): the blocks of gmres_block
  std::vector<std::vector<int>> groups;
  if (ok && method == 1) {
    for (int i = 0; i < P->sd_nnodes; ++i) {
      std::vector<int> g;
      for (int een = 0; een < 3; ++een) {
        const int bc = P->knownOf(een, P->BCidList[i]);
        if (bc == iFlux || bc == iContact) g.push_back(S.col[P->nodeList[i] + een * P->nnodes] - 1);
      }
      if (!g.empty()) groups.push_back(g);
    }
    for (int i = 0; i < P->sd_nqnodes; ++i) {
      std::vector<int> g;
      for (int een = 0; een < 3; ++een) {
        const int bc = P->knownOf(een, P->qbcidList[i]);
        if (bc == iFunction || bc == iContact) g.push_back(S.qcol[P->qnodeList[i] + een * P->nelem] - 1);
      }
      if (!g.empty()) groups.push_back(g);
    }
  }
  int worst = 0;
  for (int r = 0; r < nrhs; ++r) {
    for (int en = 0; en < 3; ++en) {
      P->eqn[en].u.assign(u_in + ((size_t)r * 3 + en) * P->nnodes, u_in + ((size_t)r * 3 + en + 1) * P->nnodes);
      P->eqn[en].q.assign(P->nelem, 0.0);
    }
    if (!ok) { status[r] = 3; nits[r] = 0; worst = 3; continue; }
    for (int i = 0; i < P->sd_nnodes; ++i) {
      int isp = P->nodeList[i], wall = P->BCidList[i];
      for (int en = 0; en < 3; ++en) {
        int ispL = isp + en * P->nnodes;
        if (P->knownOf(en, wall) == iFunction) S.b[S.col[ispL] - 1] = P->eqn[en].u[isp];
      }
    }
    for (int i = 0; i < P->sd_nqnodes; ++i) {
      int isp = P->qnodeList[i], wall = P->qbcidList[i];
      for (int en = 0; en < 3; ++en) {
        int ispL = isp + en * P->nelem;
        if (P->knownOf(en, wall) == iFlux) S.b[S.qcol[ispL] - 1] = P->eqn[en].q[isp];
      }
    }
    std::vector<double> bc(S.sys.neq), b(L.n);
    crs_x_v(S.rhs, S.b.data(), bc.data());
    for (int k = 0; k < S.sys.neq; ++k) b[L.row_of_crs[k]] = bc[k];
    int it = 0;
    double rr = 0.0;
    const int st = method == 1 ? gmres_block(L, groups, b.data(), S.x.data(), tol, maxiter, restart > 0 ? restart : 40,
                                             it, rr)
                               : bicgstab_jacobi(L, b.data(), S.x.data(), tol, maxiter, it, rr);
    nits[r] = it;
    status[r] = st;
    if (relres) relres[r] = rr;
    worst = std::max(worst, st);
    for (int i = 0; i < P->sd_nqnodes; ++i) {
      int isp = P->qnodeList[i], wall = P->qbcidList[i];
      for (int en = 0; en < 3; ++en) {
        int ispL = isp + en * P->nelem, bcq = P->knownOf(en, wall);
        P->eqn[en].q[isp] = (bcq == iFlux) ? S.b[S.qcol[ispL] - 1] : S.x[S.qcol[ispL] - 1];
      }
    }
    for (int en = 0; en < 3; ++en)
      std::copy(P->eqn[en].q.begin(), P->eqn[en].q.end(), q_out + ((size_t)r * 3 + en) * P->nelem);
    if (ft) force_torque(*P, P->eqn[0].q.data(), P->eqn[1].q.data(), P->eqn[2].q.data(), fwall, ft + 6 * r, ft + 6 * r + 3);
  }
  return worst;
}

// Force and torque of a traction field on one wall (lib_particle.f90:1751-1904)
void orc_force_torque(void* h, const double* qx, const double* qy, const double* qz, int wall, double ft[6]) {
  force_torque(*(Problem*)h, qx, qy, qz, wall, ft, ft + 3);
}

// Surface pressure at the q-source points (pressureStokes); u 3 x nnodes, q 3 x
// nelem component-major, p sd_nqnodes.  Returns -1 without Stokes matrices.
int orc_pressure_stokes(void* h, const double* u, const double* q, double* p) {
  Problem* P = (Problem*)h;
  if (P->kind != 2 || P->M[6].empty() || P->M[15].empty()) return -1;
  pressure_stokes(*P, u, q, p);
  return 0;
}
// Values at npts domain points pts[3*k]: Stokes out[4*k] = (ux, uy, uz, p) with
// u 3 x nnodes, q 3 x nelem; Laplace out[k] with u nnodes, q nelem.  err[k] the
// reference's integration check of the point.  OpenMP over the points.
void orc_domain_values(void* h, int npts, const double* pts, const double* u, const double* q, double* out,
                       double* err) {
  Problem* P = (Problem*)h;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < npts; ++k) {
    double e = 0.0;
    if (P->kind == 2) stokes_domain_value(*P, pts + 3 * (size_t)k, u, q, out + 4 * (size_t)k, e);
    else out[k] = laplace_domain_value(*P, pts + 3 * (size_t)k, u, q, e);
    err[k] = e;
  }
}

// CPU baseline sample: integrate rows [r0, r1) of the reference's nsp rows
// (u-source rows first, then q-source rows) with nthreads OpenMP threads and
// return the elapsed seconds; a checksum of the rows keeps the work observable.
double orc_time_rows(void* h, int r0, int r1, int nthreads, double* checksum) {
  Problem* P = (Problem*)h;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  const double t0 = omp_get_wtime();
#else
  (void)nthreads;
#endif
  double cs = 0.0;
#pragma omp parallel reduction(+ : cs)
  {
    StkRow R(P->nnodes, P->nelem);
    std::vector<double> rh(P->nnodes), rg(P->nelem);
#pragma omp for schedule(dynamic, 1)
    for (int r = r0; r < r1; ++r) {
      double e = 0.0;
      if (P->kind == 2) {
        if (r < P->sd_nnodes) stk_row_u(*P, P->nodeList[r], R, e);
        else stk_row_q(*P, P->qnodeList[r - P->sd_nnodes], R, e);
        cs += R.T[r % R.T.size()] + R.G[r % R.G.size()];
      } else {
        if (r < P->sd_nnodes) lap_row_u(*P, P->nodeList[r], rh.data(), rg.data(), e);
        else lap_row_q(*P, P->qnodeList[r - P->sd_nnodes], rh.data(), rg.data(), e);
        cs += rh[r % rh.size()] + rg[r % rg.size()];
      }
    }
  }
  if (checksum) *checksum = cs;
#ifdef _OPENMP
  return omp_get_wtime() - t0;
#else
  return 0.0;
#endif
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}


// dgefa / dgesl (lib_solveFM.f:198,318) for the direct-solver checks.
int orc_dgefa(double* a, int lda, int n, double* ipvt) { return linpack_dgefa(a, lda, n, ipvt); }
void orc_dgesl(const double* a, int lda, int n, const double* ipvt, double* b, int job) {
  linpack_dgesl(a, lda, n, ipvt, b, job);
}
}  // extern "C"
