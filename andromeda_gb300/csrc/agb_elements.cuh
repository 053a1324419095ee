// Element integrals of one (source point, element) pair, FP64, device side.
// Shared by the general (all-rows, all-BC) assembly of agb_general.cu.
//
// Reference behaviour (src/ file:line):
//   triangle Laplace   Triangle_BEMIntAnal lib_sdBem.f90:741 -> Triangle_3DLapInt :859
//                      (BemKernel :911) or si_tri_lap mod_singInt.f90:127
//   quad Laplace       Quad_BEMIntNumAna lib_intAna.f90:156 -> Quad_BEMIntNum :219 or
//                      si_qua_lap mod_singInt.f90:172 (sing_mode 1: the polar
//                      singular branch of Quad_BEMInt lib_int.f90:408)
//   triangle Stokes    Triangle_StokesIntAna lib_intAna.f90:96 -> Triangle_3DStokesInt
//                      lib_Stokes.f90:2341 (StokesKernel :2450) or si_tri_stk
//   quad Stokes        Quad_StokesIntNumAna lib_intAna.f90:5 -> Quad_StokesIntNum
//                      lib_Stokes.f90:3754 (fixed 3x3 subcells) or si_qua_stk
//                      (sing_mode 1: the polar singular branch of Quad_StokesInt
//                      lib_Stokes.f90:3494)
#pragma once
#include "agb_common.cuh"
#include "agb_singular.cuh"

namespace agb {

// The Gauss-Legendre tables gtGi/gtOme/gtNg1/gtNg2 are __constant__ arrays
// defined by the including translation unit (without relocatable device code
// every module holds, and uploads, its own copy).

// Laplace: g, h[4] (nodal, linear shape functions)
struct LapElem {
  double g, h[4];
};
// Stokes: G {xx,xy,xz,yy,yz,zz}, prG[3], T[6][4] (component x local node), prT[3][4]
struct StkElem {
  double G[6], prG[3], T[6][4], prT[3][4];
};

// A sub-triangle as the element barycentrics of its three vertices B[k][j].
// Midpoint split with 4 = (1+2)/2, 5 = (2+3)/2, 6 = (1+3)/2: child 0 = (1,4,6),
// 1 = (4,2,5), 2 = (6,5,3), 3 = (4,5,6); each child has a quarter of the area
// and half the edges of its parent.
struct Bary {
  double b[3][3];
};
__device__ __forceinline__ Bary bary_identity() {
  Bary B;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j) B.b[k][j] = (k == j) ? 1.0 : 0.0;
  return B;
}
__device__ __forceinline__ Bary sub_child(const Bary& P, int d) {
  Bary C;
  for (int j = 0; j < 3; ++j) {
    const double m4 = 0.5 * (P.b[0][j] + P.b[1][j]);
    const double m5 = 0.5 * (P.b[2][j] + P.b[1][j]);
    const double m6 = 0.5 * (P.b[0][j] + P.b[2][j]);
    if (d == 0) { C.b[0][j] = P.b[0][j]; C.b[1][j] = m4; C.b[2][j] = m6; }
    else if (d == 1) { C.b[0][j] = m4; C.b[1][j] = P.b[1][j]; C.b[2][j] = m5; }
    else if (d == 2) { C.b[0][j] = m6; C.b[1][j] = m5; C.b[2][j] = P.b[2][j]; }
    else { C.b[0][j] = m4; C.b[1][j] = m5; C.b[2][j] = m6; }
  }
  return C;
}

// Visits the sub-triangles of triangle E for source s in the order of the
// reference's recursion (children 0..3, depth first): rule(B, area_of_sub,
// skip_centroid).  skip_centroid marks the last piece of a centroid-source
// recursion, whose centroid is the source: a rule with a centroid point
// (ITRI 1, 2, 4) would divide by r = 0 there, so that point is left out.
template <class F>
__device__ inline void tri_walk(const IntegOpt& o, const ElemGeom& E, const double* s, int isrc, F&& rule) {
  if (isrc) {
    // only the child holding the source recurses; the last piece takes the regular rule
    const int ks = isrc - 1;
    Bary B = bary_identity();
    double a = E.area;
    for (int lev = 0; lev < o.rdepth; ++lev) {
      for (int d = 0; d < ks; ++d) rule(sub_child(B, d), 0.25 * a, false);
      B = sub_child(B, ks);
      a *= 0.25;
    }
    rule(B, a, isrc == 4);
    for (int lev = o.rdepth - 1; lev >= 0; --lev) {
      Bary Bl = bary_identity();
      double al = E.area;
      for (int t = 0; t < lev; ++t) {
        Bl = sub_child(Bl, ks);
        al *= 0.25;
      }
      for (int d = ks + 1; d < 4; ++d) rule(sub_child(Bl, d), 0.25 * al, false);
    }
    return;
  }
  if (o.near_eta > 0.0 && o.near_depth > 0) {
    auto edge = [&](int p, int q) {
      const double dx = E.v[p][0] - E.v[q][0], dy = E.v[p][1] - E.v[q][1], dz = E.v[p][2] - E.v[q][2];
      return sqrt(dx * dx + dy * dy + dz * dz);
    };
    const double diam = fmax(edge(0, 1), fmax(edge(1, 2), edge(2, 0)));
    // depth-first stack: 2 bits per level (child index), the level in bits 58..63;
    // at most 3 * near_depth + 1 <= 61 entries
    uint64_t stack[64];
    int top = 0;
    stack[top++] = 0;
    while (top > 0) {
      const uint64_t e = stack[--top];
      const int lev = (int)(e >> 58);
      Bary B = bary_identity();
      double a = E.area, h = diam;
      for (int t = 0; t < lev; ++t) {
        B = sub_child(B, (int)((e >> (2 * t)) & 3u));
        a *= 0.25;
        h *= 0.5;
      }
      double c[3] = {0.0, 0.0, 0.0};
      for (int j = 0; j < 3; ++j) {
        const double Lc = (B.b[0][j] + B.b[1][j] + B.b[2][j]) / 3.0;
        for (int i = 0; i < 3; ++i) c[i] += Lc * E.v[j][i];
      }
      const double d = sqrt((s[0] - c[0]) * (s[0] - c[0]) + (s[1] - c[1]) * (s[1] - c[1]) +
                            (s[2] - c[2]) * (s[2] - c[2]));
      if (lev < o.near_depth && d < o.near_eta * h && top <= 60) {
        for (int ch = 3; ch >= 0; --ch)
          stack[top++] = (e & ((1ull << 58) - 1)) | ((uint64_t)ch << (2 * lev)) | ((uint64_t)(lev + 1) << 58);
      } else {
        rule(B, a, false);
      }
    }
    return;
  }
  rule(bary_identity(), E.area, false);
}
__device__ __forceinline__ bool is_centroid_point(double l1, double l2, double l3) {
  return fabs(l1 - l2) < 1e-12 && fabs(l2 - l3) < 1e-12;
}

__device__ __forceinline__ void quad_map(const double (*P)[3], double gii, double gij, double* X, double* N, double* f4) {
  const double e1m = 1.0 - gii, e1p = 1.0 + gii, e2m = 1.0 - gij, e2p = 1.0 + gij;
  f4[0] = 0.25 * e1m * e2m; f4[1] = 0.25 * e1p * e2m; f4[2] = 0.25 * e1p * e2p; f4[3] = 0.25 * e1m * e2p;
  double KS[3], ET[3];
  for (int k = 0; k < 3; ++k) {
    X[k] = f4[0] * P[0][k] + f4[1] * P[1][k] + f4[2] * P[2][k] + f4[3] * P[3][k];
    KS[k] = 0.25 * (-e2m * P[0][k] + e2m * P[1][k] + e2p * P[2][k] - e2p * P[3][k]);
    ET[k] = 0.25 * (-e1m * P[0][k] - e1p * P[1][k] + e1p * P[2][k] + e1m * P[3][k]);
  }
  N[0] = KS[1] * ET[2] - ET[1] * KS[2];
  N[1] = ET[0] * KS[2] - KS[0] * ET[2];
  N[2] = KS[0] * ET[1] - ET[0] * KS[1];
}

// Singular branch of Quad_BEMInt (lib_int.f90:408-524) / Quad_StokesInt
// (lib_Stokes.f90:3494-3654), selected by sing_mode 1 for a quad's own node or
// centre (isrc 1..5): the parameter square is split at the source into four
// triangles, each integrated in polar coordinates about it (theta over
// [th0, th1], rho over [0, roth(theta)], the quad rule's Gauss points on both);
// the Jacobian rho cancels the 1/r singularity.  A triangle of zero width
// (source on its edge) is skipped.  visit(X, nn (unit normal x multi), w, f4).
template <class F>
__device__ inline void quad_polar(const ElemGeom& E, int isrc, int iqud, F&& visit) {
  const double ksi[5] = {0.0, 1.0, 1.0, 0.0, 0.5}, eta[5] = {0.0, 0.0, 1.0, 1.0, 0.5};
  const double xx1 = ksi[isrc - 1], yy1 = eta[isrc - 1];
  const int ng1 = gtNg1[iqud - 1], ng2 = gtNg2[iqud - 1];
  for (int k = 1; k <= 4; ++k) {
    double al, fii, th0, th1;
    if (k == 1) {
      if (1.0 - xx1 == 0.0) continue;
      al = sqrt(yy1 * yy1 + (1.0 - xx1) * (1.0 - xx1));
      fii = acos(yy1 / al);
      th0 = 1.5 * AGB_PI + acos(yy1 / al);
      th1 = 2.0 * AGB_PI + atan((1.0 - yy1) / (1.0 - xx1));
    } else if (k == 2) {
      if (1.0 - yy1 == 0.0) continue;
      al = sqrt((1.0 - yy1) * (1.0 - yy1) + (1.0 - xx1) * (1.0 - xx1));
      fii = acos((1.0 - xx1) / al);
      th0 = asin((1.0 - yy1) / al);
      th1 = 0.5 * AGB_PI + atan(xx1 / (1.0 - yy1));
    } else if (k == 3) {
      if (xx1 == 0.0) continue;
      al = sqrt(xx1 * xx1 + (1.0 - yy1) * (1.0 - yy1));
      fii = acos((1.0 - yy1) / al);
      th0 = 0.5 * AGB_PI + acos((1.0 - yy1) / al);
      th1 = AGB_PI + atan(yy1 / xx1);
    } else {
      if (yy1 == 0.0) continue;
      al = sqrt(yy1 * yy1 + xx1 * xx1);
      fii = acos(xx1 / al);
      th0 = AGB_PI + acos(xx1 / al);
      th1 = 1.5 * AGB_PI + atan((1.0 - xx1) / yy1);
    }
    for (int i = ng1; i <= ng2; ++i)
      for (int j = ng1; j <= ng2; ++j) {
        const double th = (th1 - th0) * gtGi[i - 1] / 2.0 + (th1 + th0) / 2.0;
        const double roth = al * sin(fii) / sin(th - th0 + fii);
        const double ro = roth * gtGi[j - 1] / 2.0 + roth / 2.0;
        const double eti = 2.0 * (xx1 + ro * cos(th)) - 1.0;
        const double etj = 2.0 * (yy1 + ro * sin(th)) - 1.0;
        double X[3], N[3], f4[4];
        quad_map(E.v, eti, etj, X, N, f4);
        const double aj = 1.0 / sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        const double nn[3] = {E.multi * N[0] * aj, E.multi * N[1] * aj, E.multi * N[2] * aj};
        const double w = (th1 - th0) * roth * ro * gtOme[i - 1] * gtOme[j - 1] / aj;
        visit(X, nn, w, f4);
      }
  }
}

// ---- Laplace ---------------------------------------------------------------
// qdiv > 0: a regular quad is integrated over qdiv x qdiv cells instead of the
// edge-length subdivision (1: the regular branch of Quad_BEMInt, lib_int.f90:329).
__device__ inline LapElem lap_element(const ElemGeom& E, const double* s, int isrc, const double* rl, const double* rw,
                                      int Q, int iqud, const IntegOpt& opt, int qdiv = 0) {
  LapElem o;
  o.g = 0.0;
  o.h[0] = o.h[1] = o.h[2] = o.h[3] = 0.0;
  const double fpi = 0.25 / AGB_PI;
  if (E.type == AGB_TRI) {
    if (isrc && opt.sing == 0) {
      o.g = agb_sing::tri_laplace(E.v[0], E.v[1], E.v[2], E.area, isrc);
      return o;
    }
    const double n[3] = {E.multi * E.n[0], E.multi * E.n[1], E.multi * E.n[2]};
    tri_walk(opt, E, s, isrc, [&](const Bary& B, double area, bool skip_centroid) {
      for (int q = 0; q < Q; ++q) {
        const double l1 = rl[q], l2 = rl[Q + q], l3 = rl[2 * Q + q];
        if (skip_centroid && is_centroid_point(l1, l2, l3)) continue;
        double L[3];
        for (int j = 0; j < 3; ++j) L[j] = l1 * B.b[0][j] + l2 * B.b[1][j] + l3 * B.b[2][j];
        const double x = L[0] * E.v[0][0] + L[1] * E.v[1][0] + L[2] * E.v[2][0];
        const double y = L[0] * E.v[0][1] + L[1] * E.v[1][1] + L[2] * E.v[2][1];
        const double z = L[0] * E.v[0][2] + L[1] * E.v[1][2] + L[2] * E.v[2][2];
        const double RX = s[0] - x, RY = s[1] - y, RZ = s[2] - z;
        const double RA = sqrt(RX * RX + RY * RY + RZ * RZ);
        const double FG = fpi / RA;
        const double FH = (RX * n[0] + RY * n[1] + RZ * n[2]) * (1.0 / (RA * RA)) * FG;
        o.g += rw[q] * FG * area;
        o.h[0] += rw[q] * FH * area * L[0];
        o.h[1] += rw[q] * FH * area * L[1];
        o.h[2] += rw[q] * FH * area * L[2];
      }
    });
    return o;
  }
  if (isrc && opt.sing == 0) {
    o.g = agb_sing::quad_laplace(E.v, isrc);
    return o;
  }
  if (isrc) {
    quad_polar(E, isrc, iqud, [&](const double* X, const double* nn, double w, const double* f4) {
      const double RX = s[0] - X[0], RY = s[1] - X[1], RZ = s[2] - X[2];
      const double RA = sqrt(RX * RX + RY * RY + RZ * RZ);
      const double FG = fpi / RA;
      const double FH = (RX * nn[0] + RY * nn[1] + RZ * nn[2]) * (1.0 / (RA * RA)) * FG;
      for (int k = 0; k < 4; ++k) o.h[k] += FH * w * f4[k];
      o.g += FG * w;
    });
    return o;
  }
  const int ng1 = gtNg1[iqud - 1], ng2 = gtNg2[iqud - 1];
  auto dist = [&](int p, int q) {
    const double dx = E.v[p][0] - E.v[q][0], dy = E.v[p][1] - E.v[q][1], dz = E.v[p][2] - E.v[q][2];
    return sqrt(dx * dx + dy * dy + dz * dz);
  };
  const double d13 = fmax(dist(0, 1), dist(2, 3)), d24 = fmax(dist(1, 2), dist(3, 0));
  const int ndx = qdiv > 0 ? qdiv : max(2, (int)(d13 / 1.0 + 0.5)), nde = qdiv > 0 ? qdiv : max(2, (int)(d24 / 1.0 + 0.5));
  for (int ix = 1; ix <= ndx; ++ix)
    for (int ie = 1; ie <= nde; ++ie) {
      const double a = -1.0 + (ix - 1) * 2.0 / ndx, b = -1.0 + ix * 2.0 / ndx;
      const double c = -1.0 + (ie - 1) * 2.0 / nde, d = -1.0 + ie * 2.0 / nde;
      const double dex = 0.25 * (b - a) * (d - c);
      for (int i = ng1; i <= ng2; ++i)
        for (int j = ng1; j <= ng2; ++j) {
          const double gii = a + 0.5 * (gtGi[i - 1] + 1.0) * (b - a);
          const double gij = c + 0.5 * (gtGi[j - 1] + 1.0) * (d - c);
          double X[3], N[3], f4[4];
          quad_map(E.v, gii, gij, X, N, f4);
          double aj = 1.0 / sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
          const double n1 = E.multi * N[0] * aj, n2 = E.multi * N[1] * aj, n3 = E.multi * N[2] * aj;
          aj = dex * gtOme[i - 1] * gtOme[j - 1] / aj;
          const double RX = s[0] - X[0], RY = s[1] - X[1], RZ = s[2] - X[2];
          const double RA = sqrt(RX * RX + RY * RY + RZ * RZ);
          const double FG = fpi / RA;
          const double FH = (RX * n1 + RY * n2 + RZ * n3) * (1.0 / (RA * RA)) * FG;
          for (int k = 0; k < 4; ++k) o.h[k] += FH * aj * f4[k];
          o.g += FG * aj;
        }
    }
  return o;
}

// ---- Stokes ----------------------------------------------------------------
__device__ __forceinline__ void stk_kernel(const double* s, const double* f, const double* n, double G[6], double T[6],
                                           double prG[3], double prT[3]) {
  const double rx = f[0] - s[0], ry = f[1] - s[1], rz = f[2] - s[2];
  const double rxx = rx * rx, rxy = rx * ry, rxz = rx * rz, ryy = ry * ry, ryz = ry * rz, rzz = rz * rz;
  const double ir2 = 1.0 / (rxx + ryy + rzz);
  const double ir = sqrt(ir2);
  const double ir3 = ir2 * ir;
  G[0] = ir * (1.0 + rxx * ir2); G[1] = rxy * ir3; G[2] = rxz * ir3;
  G[3] = ir * (1.0 + ryy * ir2); G[4] = ryz * ir3; G[5] = ir * (1.0 + rzz * ir2);
  double c = -6.0 * ir2 * ir3 * (rx * n[0] + ry * n[1] + rz * n[2]);
  T[0] = c * rxx; T[1] = c * rxy; T[2] = c * rxz; T[3] = c * ryy; T[4] = c * ryz; T[5] = c * rzz;
  c = 2.0 * ir3;
  prG[0] = c * rx; prG[1] = c * ry; prG[2] = c * rz;
  c = 4.0 * ir3;
  prT[0] = c * ((-1.0 + 3.0 * rxx * ir2) * n[0] + 3.0 * rxy * ir2 * n[1] + 3.0 * rxz * ir2 * n[2]);
  prT[1] = c * (3.0 * rxy * ir2 * n[0] + (-1.0 + 3.0 * ryy * ir2) * n[1] + 3.0 * ryz * ir2 * n[2]);
  prT[2] = c * (3.0 * rxz * ir2 * n[0] + 3.0 * ryz * ir2 * n[1] + (-1.0 + 3.0 * rzz * ir2) * n[2]);
}

// qdiv: cells per direction of a regular quad (3: Quad_StokesIntNum; 1: the regular
// branch of Quad_StokesInt, lib_Stokes.f90:3398, used for points in the domain).
__device__ inline void stk_element(const ElemGeom& E, const double* s, int isrc, const double* rl, const double* rw,
                                   int Q, int iqud, const IntegOpt& opt, StkElem& o, int qdiv = 3) {
  for (int k = 0; k < 6; ++k) {
    o.G[k] = 0.0;
    for (int j = 0; j < 4; ++j) o.T[k][j] = 0.0;
  }
  for (int k = 0; k < 3; ++k) {
    o.prG[k] = 0.0;
    for (int j = 0; j < 4; ++j) o.prT[k][j] = 0.0;
  }
  if (isrc && opt.sing == 0) {
    if (E.type == AGB_TRI) agb_sing::tri_stokes(E.v[0], E.v[1], E.v[2], E.area, isrc, o.G);
    else agb_sing::quad_stokes(E.v, isrc, o.G);
    return;
  }
  double G[6], T[6], prG[3], prT[3];
  if (isrc && E.type != AGB_TRI) {
    // G and T by the polar rule; the pressure integrals of the own element
    // (principal value / hypersingular) stay zero, as the analytic branch leaves them
    quad_polar(E, isrc, iqud, [&](const double* X, const double* nn, double w, const double* f4) {
      stk_kernel(s, X, nn, G, T, prG, prT);
      for (int k = 0; k < 6; ++k) o.G[k] += w * G[k];
      for (int sp = 0; sp < 4; ++sp) {
        const double ww = w * f4[sp];
        for (int k = 0; k < 6; ++k) o.T[k][sp] += ww * T[k];
      }
    });
    return;
  }
  if (E.type == AGB_TRI) {
    const double n[3] = {E.multi * E.n[0], E.multi * E.n[1], E.multi * E.n[2]};
    tri_walk(opt, E, s, isrc, [&](const Bary& B, double area, bool skip_centroid) {
      for (int q = 0; q < Q; ++q) {
        const double l1 = rl[q], l2 = rl[Q + q], l3 = rl[2 * Q + q];
        if (skip_centroid && is_centroid_point(l1, l2, l3)) continue;
        double l[3];
        for (int j = 0; j < 3; ++j) l[j] = l1 * B.b[0][j] + l2 * B.b[1][j] + l3 * B.b[2][j];
        const double f[3] = {l[0] * E.v[0][0] + l[1] * E.v[1][0] + l[2] * E.v[2][0],
                             l[0] * E.v[0][1] + l[1] * E.v[1][1] + l[2] * E.v[2][1],
                             l[0] * E.v[0][2] + l[1] * E.v[1][2] + l[2] * E.v[2][2]};
        stk_kernel(s, f, n, G, T, prG, prT);
        const double w = rw[q] * area;
        for (int k = 0; k < 6; ++k) o.G[k] += w * G[k];
        for (int k = 0; k < 3; ++k) o.prG[k] += w * prG[k];
        for (int j = 0; j < 3; ++j) {
          const double wl = w * l[j];
          for (int k = 0; k < 6; ++k) o.T[k][j] += wl * T[k];
          for (int k = 0; k < 3; ++k) o.prT[k][j] += wl * prT[k];
        }
      }
    });
    return;
  }
  const int ng1 = gtNg1[iqud - 1], ng2 = gtNg2[iqud - 1];
  for (int ix = 1; ix <= qdiv; ++ix)
    for (int ie = 1; ie <= qdiv; ++ie) {
      const double a = -1.0 + (ix - 1) * 2.0 / qdiv, b = -1.0 + ix * 2.0 / qdiv;
      const double c = -1.0 + (ie - 1) * 2.0 / qdiv, d = -1.0 + ie * 2.0 / qdiv;
      const double dex = 0.25 * (b - a) * (d - c);
      for (int i = ng1; i <= ng2; ++i)
        for (int j = ng1; j <= ng2; ++j) {
          const double gii = a + 0.5 * (gtGi[i - 1] + 1.0) * (b - a);
          const double gij = c + 0.5 * (gtGi[j - 1] + 1.0) * (d - c);
          double X[3], N[3], f4[4];
          quad_map(E.v, gii, gij, X, N, f4);
          double aj = 1.0 / sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
          const double nn[3] = {E.multi * N[0] * aj, E.multi * N[1] * aj, E.multi * N[2] * aj};
          aj = dex * gtOme[i - 1] * gtOme[j - 1] / aj;
          stk_kernel(s, X, nn, G, T, prG, prT);
          for (int k = 0; k < 6; ++k) o.G[k] += aj * G[k];
          for (int k = 0; k < 3; ++k) o.prG[k] += aj * prG[k];
          for (int sp = 0; sp < 4; ++sp) {
            const double w = aj * f4[sp];
            for (int k = 0; k < 6; ++k) o.T[k][sp] += w * T[k];
            for (int k = 0; k < 3; ++k) o.prT[k][sp] += w * prT[k];
          }
        }
    }
}

}  // namespace agb
