// Icosahedral-hexagonal grid and metric tables for the FIM horizontal dynamics.
//
// Host-side C++ builder of the tables the dycore routines read from
// module_constants (FIMsrc/cntl/module_constants.F90:45-104):
//   prox, proxs, nprox, cs, sn, sidevec_c, sidevec_e, sideln, rprox_ln,
//   area, corner_xy, hfcoef, lat, lon.
//
// Geometry follows the reference generator chain:
//   * 12 icosahedron vertices at +-90 deg and +-26.5650428671016 deg
//     (FIMsrc/prep/grid/top_gridpoints.F90), rotated 10 deg in longitude
//     (FIMsrc/prep/grid/icos.F90:68-70).
//   * gtype 0 "standard recursive" refinement: every triangle is split in 4 by
//     the normalised great-circle midpoints of its edges
//     (FIMsrc/prep/grid/bisect_triangle.F90:134-191, middle.F90).
//   * 10 rhombi of sl x sl cells plus the two poles, nip = 10*sl^2+2
//     (FIMsrc/prep/grid/icos.F90:91).
//   * neighbours ordered counter-clockwise seen from outside the sphere; the
//     Voronoi corner j is the circumcentre of (cell, prox j, prox j+1)
//     (FIMsrc/prep/grid/GridGen.F90:244-299) and edge j runs from corner j-1 to
//     corner j (the index shift of FIMsrc/prep/grid/getlvl.F90:125-143).
//   * metric tables exactly as FIMsrc/prep/grid/getlvl.F90:145-294, evaluated in
//     double precision; the least-squares pseudo-inverse for hfcoef
//     (FIMsrc/prep/lsfit/LSfitting.F90:73-130, LAPACK sgesvd there) is computed
//     here with Householder QR (Golub & Van Loan, Matrix Computations, 5.2),
//     which gives the same Moore-Penrose inverse for a full-column-rank system.
//
// Cell numbering and neighbour slot order are the reference's (curve = 0, the
// IJ order): the north pole is cell 1, then the rhombi in the order U0, L0, U1,
// L1, ..., U4, L4 (upper rhombus k between the north pole and upper vertices
// k, k+1; lower rhombus k below it), sl*sl cells each in rows of sl, and the
// south pole last (icos.F90:174-239, the rhombus offsets of proc_grid).  The
// neighbours of a cell are found by walking the triangulation and are listed
// counter-clockwise seen from outside the sphere, starting where the
// reference's pattern tables of GridGen.F90:98-217,529-623 start (see
// first_neighbour), so prox, proxs and nprox equal the reference's tables
// entry for entry; the tests check them against a restatement of the
// reference generator.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <array>

#include "../../include/fim_gpu.h"

namespace {

struct V3 { double x, y, z; };
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalize(V3 a) {
  double d = std::sqrt(dot(a, a));
  return {a.x / d, a.y / d, a.z / d};
}
// great-circle midpoint; symmetric in (p, q) bit for bit because p+q == q+p
inline V3 mid(V3 p, V3 q) { return normalize(add(p, q)); }

inline V3 from_ll(double lat, double lon) {
  return {std::cos(lat) * std::cos(lon), std::cos(lat) * std::sin(lon), std::sin(lat)};
}
inline void to_ll(V3 p, double* lat, double* lon) {
  *lat = std::atan2(p.z, std::sqrt(p.x * p.x + p.y * p.y));
  double l = std::atan2(p.y, p.x);
  if (l < 0.0) l += 2.0 * M_PI;
  *lon = l;
}

// general stereographic projection of (lat,lon) about (latc,lonc), in units of
// the earth radius (FIMsrc/prep/grid/getlvl.F90:402-417)
inline void ll2xy(double lonc, double latc, double lon, double lat, double* xm, double* ym) {
  double mf = 2.0 / (1.0 + std::sin(lat) * std::sin(latc) +
                     std::cos(lat) * std::cos(latc) * std::cos(lon - lonc));
  *xm = mf * (std::cos(lat) * std::sin(lon - lonc));
  *ym = mf * (std::sin(lat) * std::cos(latc) - std::cos(lat) * std::sin(latc) * std::cos(lon - lonc));
}

// Triangular lattice T[a][b] (a+b <= n) over the spherical triangle (v0,v1,v2),
// with a counted along v0->v1 and b along v0->v2, refined by recursive
// bisection from n=1 to n=sl.
struct TriLattice {
  int n = 1;
  std::vector<V3> p;  // (n+1)*(n+1) storage, only a+b<=n used
  V3& at(int a, int b) { return p[(size_t)a * (n + 1) + b]; }
  void build(V3 v0, V3 v1, V3 v2, int sl) {
    n = 1;
    p.assign(4, V3{0, 0, 0});
    at(0, 0) = v0; at(1, 0) = v1; at(0, 1) = v2;
    while (n < sl) {
      TriLattice nx;
      nx.n = 2 * n;
      nx.p.assign((size_t)(nx.n + 1) * (nx.n + 1), V3{0, 0, 0});
      for (int a = 0; a <= n; a++)
        for (int b = 0; a + b <= n; b++) {
          nx.at(2 * a, 2 * b) = at(a, b);
          if (a + 1 + b <= n) nx.at(2 * a + 1, 2 * b) = mid(at(a, b), at(a + 1, b));
          if (a + b + 1 <= n) nx.at(2 * a, 2 * b + 1) = mid(at(a, b), at(a, b + 1));
          if (a + b + 1 <= n) nx.at(2 * a + 1, 2 * b + 1) = mid(at(a + 1, b), at(a, b + 1));
        }
      *this = std::move(nx);
    }
  }
};

// Householder QR least squares: pinv (5 x n, row-major pinv[bf*n+j]) of the
// n x 5 matrix A (row-major A[j*5+bf]), n in {5, 6}.
void pseudo_inverse(const double* A_in, int n, double* pinv) {
  const int m = 5;
  double A[6 * 5];
  std::memcpy(A, A_in, sizeof(double) * n * m);
  double Q[6 * 6];  // accumulate Q^T applied to identity
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) Q[i * n + j] = (i == j) ? 1.0 : 0.0;
  for (int c = 0; c < m; c++) {
    double norm = 0.0;
    for (int r = c; r < n; r++) norm += A[r * m + c] * A[r * m + c];
    norm = std::sqrt(norm);
    if (norm == 0.0) continue;
    double alpha = (A[c * m + c] > 0.0) ? -norm : norm;
    double v[6];
    for (int r = 0; r < n; r++) v[r] = 0.0;
    for (int r = c; r < n; r++) v[r] = A[r * m + c];
    v[c] -= alpha;
    double vnorm2 = 0.0;
    for (int r = c; r < n; r++) vnorm2 += v[r] * v[r];
    if (vnorm2 == 0.0) continue;
    // A <- (I - 2 v v^T / v^T v) A
    for (int cc = c; cc < m; cc++) {
      double s = 0.0;
      for (int r = c; r < n; r++) s += v[r] * A[r * m + cc];
      s = 2.0 * s / vnorm2;
      for (int r = c; r < n; r++) A[r * m + cc] -= s * v[r];
    }
    // Q <- H Q   (Q holds Q^T)
    for (int cc = 0; cc < n; cc++) {
      double s = 0.0;
      for (int r = c; r < n; r++) s += v[r] * Q[r * n + cc];
      s = 2.0 * s / vnorm2;
      for (int r = c; r < n; r++) Q[r * n + cc] -= s * v[r];
    }
  }
  // A now holds R in its top m rows; pinv = R^{-1} (Q^T)[0:m, :]
  for (int j = 0; j < n; j++) {
    double x[5];
    for (int r = m - 1; r >= 0; r--) {
      double s = Q[r * n + j];
      for (int cc = r + 1; cc < m; cc++) s -= A[r * m + cc] * x[cc];
      x[r] = s / A[r * m + r];
    }
    for (int r = 0; r < m; r++) pinv[r * n + j] = x[r];
  }
}

struct Builder {
  int glvl, sl, nip;
  std::vector<V3> xyz;
  std::vector<int> nprox;
  std::vector<std::array<int, 6>> ring;

  // 0-based index of the first cell of rhombus d (d = 0..4 upper, 5..9
  // lower): rhombus pairs (upper k, lower k) follow each other
  // (icos.F90:212-237: offsets 2k*sl^2 and (2k+1)*sl^2 after the north pole).
  int base(int d) const { return 1 + (2 * (d % 5) + (d >= 5 ? 1 : 0)) * sl * sl; }

  // 0-based index of the neighbour the reference lists first for the cell
  // (d, i, j), 1 <= i <= sl, 0 <= j < sl (GridGen.F90:98-217 and
  // special_points, :529-623).  Inside a rhombus and along its j-boundaries
  // that is the cell before it in its row (index - 1); along the rhombus's
  // i-boundaries (i = 1 or i = sl) it is the cell of the previous row
  // (index - sl), which for the first row of a lower rhombus is the last row
  // of the upper rhombus above it.  Exceptions: the first row's ends in an
  // upper rhombus (i = 1 next to the north pole starts at the pole, i = sl,
  // a pentagon, at index - 1) and the pentagon at the end of a lower
  // rhombus's first row (index - 1).
  int first_neighbour(int d, int i, int j) const {
    const bool upper = d < 5;
    const int idx = base(d) + j * sl + (i - 1);
    if (upper && i == 1 && j == 0) return 0;  // north pole
    const bool iedge = (i == 1 || i == sl);
    const bool first_row_end = (j == 0) && (upper || i == sl);
    return (iedge && !first_row_end) ? idx - sl : idx - 1;
  }

  // global 0-based index of the closed-rhombus lattice point (d, i, j),
  // 0 <= i, j <= sl; d = 0..4 upper rhombi, 5..9 lower rhombi.
  int owner(int d, int i, int j) const {
    for (;;) {
      bool upper = d < 5;
      int k = d % 5;
      if (upper) {
        if (i == 0 && j == 0) return 0;                     // north pole
        if (i == 0) { d = (k + 1) % 5; i = j; j = 0; continue; }   // edge N-U(k+1)
        if (j == sl) { d = 5 + k; j = 0; continue; }         // edge U(k+1)-L(k)
        return base(d) + j * sl + (i - 1);
      } else {
        if (i == sl && j == sl) return nip - 1;             // south pole
        if (i == 0) { d = (k + 1) % 5; i = sl; continue; }   // edge U(k+1)-L(k+1)
        if (j == sl) { d = 5 + (k + 1) % 5; j = i; i = sl; continue; }  // edge L(k+1)-S
        return base(d) + j * sl + (i - 1);
      }
    }
  }

  int build(int glvl_) {
    glvl = glvl_;
    sl = 1 << glvl;
    nip = 10 * sl * sl + 2;
    const double d2r = M_PI / 180.0;
    const double lat0 = 26.5650428671016 * d2r;  // top_gridpoints.F90 Lat0
    const double rot = 10.0;                     // icos.F90 theta
    V3 NP = from_ll(90.0 * d2r, 0.0), SP = from_ll(-90.0 * d2r, 0.0);
    V3 U[5], L[5];
    for (int k = 0; k < 5; k++) {
      U[k] = from_ll(lat0, (72.0 * k + rot) * d2r);
      L[k] = from_ll(-lat0, (72.0 * k + 36.0 + rot) * d2r);
    }
    xyz.assign(nip, V3{0, 0, 0});
    xyz[0] = NP;
    xyz[nip - 1] = SP;
    // rhombus corners A (apex), B, C (short diagonal), D (opposite apex)
    std::vector<TriLattice> t1(10), t2(10);
    for (int d = 0; d < 10; d++) {
      int k = d % 5;
      V3 A, B, C, D;
      if (d < 5) { A = NP; B = U[k]; C = U[(k + 1) % 5]; D = L[k]; }
      else { A = U[(k + 1) % 5]; B = L[k]; C = L[(k + 1) % 5]; D = SP; }
      t1[d].build(A, B, C, sl);
      t2[d].build(D, C, B, sl);
    }
    auto pos = [&](int d, int i, int j) -> V3 {
      if (i + j <= sl) return t1[d].at(i, j);
      return t2[d].at(sl - i, sl - j);
    };
    for (int d = 0; d < 10; d++)
      for (int j = 0; j < sl; j++)
        for (int i = 1; i <= sl; i++) xyz[base(d) + j * sl + (i - 1)] = pos(d, i, j);

    // successor map around every vertex from consistently oriented triangles
    std::vector<std::array<int, 12>> succ(nip);  // pairs (b, c): c follows b CCW
    std::vector<int> nsucc(nip, 0);
    auto add_tri = [&](int a, int b, int c) {
      if (dot(xyz[a], cross(xyz[b], xyz[c])) < 0.0) std::swap(b, c);
      int tri[3] = {a, b, c};
      for (int r = 0; r < 3; r++) {
        int v0 = tri[r], v1 = tri[(r + 1) % 3], v2 = tri[(r + 2) % 3];
        int& ns = nsucc[v0];
        for (int q = 0; q < ns; q++)
          if (succ[v0][2 * q] == v1) return;  // already recorded (shared triangle)
        if (ns >= 6) return;
        succ[v0][2 * ns] = v1;
        succ[v0][2 * ns + 1] = v2;
        ns++;
      }
    };
    for (int d = 0; d < 10; d++)
      for (int j = 0; j < sl; j++)
        for (int i = 0; i < sl; i++) {
          int p00 = owner(d, i, j), p10 = owner(d, i + 1, j), p01 = owner(d, i, j + 1),
              p11 = owner(d, i + 1, j + 1);
          add_tri(p00, p10, p01);
          add_tri(p10, p11, p01);
        }
    // the neighbour each cell's ring starts with
    std::vector<int> first(nip, -1);
    first[0] = base(0);                // north pole: first cell of U0
    first[nip - 1] = base(9) + sl * sl - 1;  // south pole: last cell of L4
    for (int d = 0; d < 10; d++)
      for (int j = 0; j < sl; j++)
        for (int i = 1; i <= sl; i++) first[base(d) + j * sl + (i - 1)] = first_neighbour(d, i, j);
    nprox.assign(nip, 0);
    ring.assign(nip, std::array<int, 6>{-1, -1, -1, -1, -1, -1});
    for (int v = 0; v < nip; v++) {
      int n = nsucc[v];
      if (n != 5 && n != 6) return -1;
      const int start = first[v];
      bool found = false;
      for (int q = 0; q < n; q++) found = found || (succ[v][2 * q] == start);
      if (!found) return -4;
      int cur = start;
      for (int e = 0; e < n; e++) {
        ring[v][e] = cur;
        int nxt = -1;
        for (int q = 0; q < n; q++)
          if (succ[v][2 * q] == cur) nxt = succ[v][2 * q + 1];
        if (nxt < 0) return -2;
        cur = nxt;
      }
      if (cur != start) return -3;
      nprox[v] = n;
    }
    return 0;
  }
};

}  // namespace

extern "C" int fim_grid_nip(int glvl) {
  if (glvl < 0 || glvl > 11) return -1;
  int sl = 1 << glvl;
  return 10 * sl * sl + 2;
}

extern "C" int fim_grid_build(int glvl, fim_grid_desc* g) {
  if (!g || glvl < 1 || glvl > 11) return FIM_EINVAL;
  Builder b;
  int rc = b.build(glvl);
  if (rc != 0) return FIM_ENUMERIC;
  const int nip = b.nip;
  if (g->nip != nip) return FIM_EINVAL;
  g->glvl = glvl;
  const double ae = 6371220.0;  // getlvl.F90:22

  std::vector<double> lat(nip), lon(nip);
  for (int i = 0; i < nip; i++) to_ll(b.xyz[i], &lat[i], &lon[i]);

  for (int ipn = 0; ipn < nip; ipn++) {
    int np = b.nprox[ipn];
    g->nprox[ipn] = np;
    if (g->lat) g->lat[ipn] = lat[ipn];
    if (g->lon) g->lon[ipn] = lon[ipn];
    for (int e = 0; e < 6; e++) {
      int pe = (e < np) ? e : np - 1;  // pentagon: prox(6)=prox(5) (dyn_init.F90:545-549)
      g->prox[ipn * 6 + e] = b.ring[ipn][pe] + 1;
      g->proxs[ipn * 6 + e] = -99;
    }
  }
  // proxs: neighbour's index of the shared edge (getlvl.F90:145-157)
  for (int ipn = 0; ipn < nip; ipn++)
    for (int e = 0; e < b.nprox[ipn]; e++) {
      int nb = b.ring[ipn][e];
      for (int j = 0; j < b.nprox[nb]; j++)
        if (b.ring[nb][j] == ipn) { g->proxs[ipn * 6 + e] = j + 1; break; }
    }

  std::vector<double> conr_lat(6), conr_lon(6);
  for (int ipn = 0; ipn < nip; ipn++) {
    const int np = b.nprox[ipn];
    const V3 c = b.xyz[ipn];
    // Voronoi corners: corner j between neighbours j and j+1 (GridGen.F90:244-258)
    double clat[6], clon[6];
    for (int j = 0; j < np; j++) {
      V3 v1 = sub(b.xyz[b.ring[ipn][j]], c);
      V3 v2 = sub(b.xyz[b.ring[ipn][(j + 1) % np]], c);
      V3 v = normalize(cross(v1, v2));
      to_ll(v, &clat[j], &clon[j]);
    }
    // edge isn spans corners (isn-1, isn) (getlvl.F90:125-143)
    double e_lat[6][2], e_lon[6][2], lle_lat[6], lle_lon[6];
    for (int isn = 0; isn < np; isn++) {
      int ism = (isn + np - 1) % np;
      e_lat[isn][0] = clat[ism]; e_lon[isn][0] = clon[ism];
      e_lat[isn][1] = clat[isn]; e_lon[isn][1] = clon[isn];
      V3 pm = mid(from_ll(e_lat[isn][0], e_lon[isn][0]), from_ll(e_lat[isn][1], e_lon[isn][1]));
      to_ll(pm, &lle_lat[isn], &lle_lon[isn]);
    }
    const double la = lat[ipn], lo = lon[ipn];
    double conr_xy[6][2][2];
    double area = 0.0;
    for (int e = 0; e < 6; e++) {
      int o = ipn * 6 + e;
      for (int q = 0; q < 4; q++) { g->cs[o * 4 + q] = 0.0; g->sn[o * 4 + q] = 0.0; }
      for (int q = 0; q < 2; q++) { g->sidevec_c[o * 2 + q] = 0.0; g->sidevec_e[o * 2 + q] = 0.0; }
      g->sideln[o] = 0.0;
      g->rprox_ln[o] = 0.0;
      for (int q = 0; q < 6; q++) g->hfcoef[o * 6 + q] = 0.0;
      if (g->corner_xy) { g->corner_xy[(ipn * 2 + 0) * 6 + e] = 0.0; g->corner_xy[(ipn * 2 + 1) * 6 + e] = 0.0; }
    }
    for (int isn = 0; isn < np; isn++) {
      int o = ipn * 6 + isn;
      int nb = b.ring[ipn][isn];
      double px, py;
      ll2xy(lo, la, lon[nb], lat[nb], &px, &py);
      g->rprox_ln[o] = 1.0 / (ae * std::sqrt(px * px + py * py));
      for (int ipt = 0; ipt < 2; ipt++)
        ll2xy(lo, la, e_lon[isn][ipt], e_lat[isn][ipt], &conr_xy[isn][ipt][0], &conr_xy[isn][ipt][1]);
      double map = 2.0 / (1.0 + std::sin(lle_lat[isn]) * std::sin(la) +
                          std::cos(lle_lat[isn]) * std::cos(la) * std::cos(lle_lon[isn] - lo));
      for (int ixy = 0; ixy < 2; ixy++)
        g->sidevec_c[o * 2 + ixy] = ae * (conr_xy[isn][1][ixy] - conr_xy[isn][0][ixy]) * map;
      double xxp, yyp, xxm, yym;
      ll2xy(lle_lon[isn], lle_lat[isn], e_lon[isn][1], e_lat[isn][1], &xxp, &yyp);
      ll2xy(lle_lon[isn], lle_lat[isn], e_lon[isn][0], e_lat[isn][0], &xxm, &yym);
      g->sidevec_e[o * 2 + 0] = ae * (xxp - xxm);
      g->sidevec_e[o * 2 + 1] = ae * (yyp - yym);
      g->sideln[o] = std::sqrt(g->sidevec_e[o * 2] * g->sidevec_e[o * 2] +
                               g->sidevec_e[o * 2 + 1] * g->sidevec_e[o * 2 + 1]);
    }
    for (int isn = 0; isn < np; isn++) {
      int o = ipn * 6 + isn;
      double xx = ae * 0.5 * (conr_xy[isn][1][0] + conr_xy[isn][0][0]);
      double yy = ae * 0.5 * (conr_xy[isn][1][1] + conr_xy[isn][0][1]);
      area += 0.5 * (xx * g->sidevec_c[o * 2 + 1] - yy * g->sidevec_c[o * 2 + 0]);
    }
    g->area[ipn] = area;
    if (g->corner_xy)
      for (int ixy = 0; ixy < 2; ixy++)
        for (int isn = 0; isn < np; isn++)
          g->corner_xy[(ipn * 2 + ixy) * 6 + isn] = ae * conr_xy[isn][0][ixy];

    // basis-function moments for the high-order edge reconstruction
    // (getlvl.F90:219-250)
    double ap[5] = {0, 0, 0, 0, 0};
    for (int isn = 0; isn < np; isn++) {
      int o = ipn * 6 + isn;
      double xim1 = conr_xy[isn][0][0], xi = conr_xy[isn][1][0];
      double yim1 = conr_xy[isn][0][1], yi = conr_xy[isn][1][1];
      double xx = ae * 0.5 * (xim1 + xi), yy = ae * 0.5 * (yim1 + yi);
      double tri = 0.5 * (xx * g->sidevec_c[o * 2 + 1] - yy * g->sidevec_c[o * 2 + 0]) / area;
      ap[0] += tri / 3.0 * (xim1 + xi);
      ap[1] += tri / 3.0 * (yim1 + yi);
      ap[2] += tri / 6.0 * (xim1 * xim1 + xim1 * xi + xi * xi);
      ap[3] += tri / 12.0 * (2.0 * xim1 * yim1 + 2.0 * xi * yi + xim1 * yi + xi * yim1);
      ap[4] += tri / 6.0 * (yim1 * yim1 + yim1 * yi + yi * yi);
    }
    double pxy[6][5];
    for (int isn = 0; isn < np; isn++) {
      double xim1 = conr_xy[isn][0][0], xi = conr_xy[isn][1][0];
      double yim1 = conr_xy[isn][0][1], yi = conr_xy[isn][1][1];
      pxy[isn][0] = 0.5 * (xim1 + xi) - ap[0];
      pxy[isn][1] = 0.5 * (yim1 + yi) - ap[1];
      pxy[isn][2] = 1.0 / 3.0 * (xim1 * xim1 + xi * xi + xim1 * xi) - ap[2];
      pxy[isn][3] = 1.0 / 6.0 * (2.0 * xim1 * yim1 + 2.0 * xi * yi + xim1 * yi + xi * yim1) - ap[3];
      pxy[isn][4] = 1.0 / 3.0 * (yim1 * yim1 + yi * yi + yim1 * yi) - ap[4];
    }
    // observation matrix of the bi-quadratic basis x, y, x^2, xy, y^2
    // (LSfitting.F90:220-268) at the neighbour positions
    double A[6 * 5], pinv[5 * 6];
    for (int isn = 0; isn < np; isn++) {
      int nb = b.ring[ipn][isn];
      double x, y;
      ll2xy(lo, la, lon[nb], lat[nb], &x, &y);
      A[isn * 5 + 0] = x; A[isn * 5 + 1] = y; A[isn * 5 + 2] = x * x;
      A[isn * 5 + 3] = x * y; A[isn * 5 + 4] = y * y;
    }
    pseudo_inverse(A, np, pinv);
    for (int isn = 0; isn < np; isn++)
      for (int ico = 0; ico < np; ico++) {
        double s = 0.0;
        for (int ibf = 0; ibf < 5; ibf++) s += pxy[isn][ibf] * pinv[ibf * np + ico];
        g->hfcoef[(ipn * 6 + isn) * 6 + ico] = s;
      }

    // rotation coefficients at the edge midpoint for the cell, the neighbour
    // across the edge and the neighbours across edges isn-1 and isn+1
    // (getlvl.F90:273-294)
    for (int isn = 0; isn < np; isn++) {
      int o = ipn * 6 + isn;
      int ip1 = (isn + 1) % np, im1 = (isn + np - 1) % np;
      double xltc = lle_lat[isn], xlnc = lle_lon[isn];
      double eltp[4] = {la, lat[b.ring[ipn][isn]], lat[b.ring[ipn][im1]], lat[b.ring[ipn][ip1]]};
      double elnp[4] = {lo, lon[b.ring[ipn][isn]], lon[b.ring[ipn][im1]], lon[b.ring[ipn][ip1]]};
      for (int ipt = 0; ipt < 4; ipt++) {
        double rf = 1.0 / (1.0 + std::sin(xltc) * std::sin(eltp[ipt]) +
                           std::cos(xltc) * std::cos(eltp[ipt]) * std::cos(elnp[ipt] - xlnc));
        g->cs[o * 4 + ipt] = rf * (std::cos(xltc) * std::cos(eltp[ipt]) +
                                   (1.0 + std::sin(xltc) * std::sin(eltp[ipt])) * std::cos(elnp[ipt] - xlnc));
        g->sn[o * 4 + ipt] = -rf * std::sin(elnp[ipt] - xlnc) * (std::sin(xltc) + std::sin(eltp[ipt]));
      }
    }
  }
  return FIM_OK;
}
