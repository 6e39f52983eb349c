// Physics coupling, the dynamics side of phy_run (cpl_run.F90:35-536 with
// dffusn8_lyr, dffusn.F90:110-129): the conversion of the dynamics state
// (level fastest) into the GFS physics state (nip, nvl; cell fastest, FP64 as
// the reference's kind_evod arrays) and back.
//
//   k_cpl_d2p    cpl_dyn_to_phy: layer pressure (Phillips' average of p^kappa),
//                temperature from virtual potential temperature, winds,
//                moisture/ozone/cloud with their floors, and the six copies
//                the tendency method keeps.
//   k_cpl_tend   cpl_phy_to_dyn with addtend: physics tendencies (level fastest)
//   k_cpl_dffusn dffusn8_lyr on the tendencies (smoothtend), out of place
//   k_cpl_p2d    cpl_phy_to_dyn: winds, potential temperature, moisture tracers
//                and the precipitation / evaporation columns globsum reads.
//
// A block covers 32 cells x 32 levels.  The GFS arrays are read and written
// with threadIdx.x = cell (256-byte rows); the level-fastest dynamics fields
// that cpl_phy_to_dyn writes pass through a 32 x 33 shared tile, one field at
// a time, so their stores are 128-byte rows along k.
#include "fim_internal.h"

namespace fim {

constexpr int kCplTile = 32;
constexpr int kCplRows = 8;

// p^kappa layer mean of the FP64 build, cpl_run.F90:236-237 as written
__device__ __forceinline__ double phillips(double pk, double pk1) {
  const double rocp1 = kRd / kCp + 1., rocpr = kCp / kRd;
  return pow((pow(pk, rocp1) - pow(pk1, rocp1)) / ((pk - pk1) * rocp1), rocpr);
}

// The same mean in FP32 without the cancellation of pk^a - pk1^a
// (a = kappa + 1): with x = (pk - pk1) / pk,
//   (pk^a - pk1^a) / ((pk - pk1) a) = pk^kappa * E / (a x),
//   E = 1 - (1 - x)^a = -expm1(a log1p(-x)),
// so p = pk * (E / (a x))^(1/kappa); every factor keeps FP32's relative
// accuracy (the layer-mean ratio E / (a x) lies in (1 - kappa x / 2, 1]).
__device__ __forceinline__ float phillips(float pk, float pk1) {
  const float kap = float(kRd / kCp), a = kap + 1.f;
  const float x = (pk - pk1) / pk;
  const float e = -expm1f(a * log1pf(-x));
  return pk * powf(e / (a * x), 1.f / kap);
}

// Thread values (cell threadIdx.x, levels threadIdx.y + 8 j) to the block's
// 32 x 32 tile of a level-fastest field, and the tile out as rows along k:
// a warp's store is 32 consecutive levels of one cell
template <typename R>
__device__ __forceinline__ void tile_out(R* __restrict__ dst, size_t stride, int nk, int i0, int k0, int N,
                                         R (*tile)[kCplTile + 1], const R (&v)[kCplTile / kCplRows]) {
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int j = 0; j < kCplTile / kCplRows; j++) tile[tx][ty + kCplRows * j] = v[j];
  __syncthreads();
#pragma unroll
  for (int r = ty; r < kCplTile; r += kCplRows) {
    const int i = i0 + r, k = k0 + tx;
    if (i < N && k < nk) dst[(size_t)i * stride + k] = tile[r][tx];
  }
  __syncthreads();
}

constexpr int kCplV = kCplTile / kCplRows;  // levels a thread

// The dynamics fields are read with threadIdx.x = cell: the block's 8 warps
// take the levels of the same 32 column segments of 128 bytes in turn, so
// all but the first find them in L1 (measured faster here than staging the
// nine fields through the shared tile one after another).
template <typename R>
__global__ void __launch_bounds__(kCplTile * kCplRows) k_cpl_d2p(int N, int L, const R* __restrict__ pr3d,
    const R* __restrict__ us3d, const R* __restrict__ vs3d, const R* __restrict__ ws3d,
    const R* __restrict__ tr3d, double* __restrict__ gfs_ps, double* __restrict__ gfs_dp,
    double* __restrict__ gfs_p, double* __restrict__ gfs_u, double* __restrict__ gfs_v,
    double* __restrict__ gfs_dpdt, double* __restrict__ gfs_q, double* __restrict__ gfs_oz,
    double* __restrict__ gfs_cld, double* __restrict__ gfs_t, double* __restrict__ old6) {
  const int i = blockIdx.x * kCplTile + threadIdx.x;
  if (i >= N) return;
  const int L1 = L + 1;
  const size_t NL = (size_t)N * L;
  if (blockIdx.y == 0 && threadIdx.y == 0) gfs_ps[i] = 0.001 * (double)pr3d[(size_t)i * L1];
  const int k1 = (blockIdx.y + 1) * kCplTile < L ? (blockIdx.y + 1) * kCplTile : L;
  for (int k = blockIdx.y * kCplTile + threadIdx.y; k < k1; k += kCplRows) {
    const size_t c = (size_t)i * L + k, g = (size_t)k * N + i;
    const R pk = pr3d[(size_t)i * L1 + k], pk1 = pr3d[(size_t)i * L1 + k + 1];
    const R th = tr3d[c], qv = tr3d[NL + c], cld = tr3d[2 * NL + c], oz = tr3d[3 * NL + c];
    const double u = (double)us3d[c], v = (double)vs3d[c], w = (double)ws3d[c];
    double p, t, q;
    if constexpr (sizeof(R) == 8) {
      p = phillips((double)pk, (double)pk1);
      q = fmax(kQvmin, (double)qv);
      const double theta_nv = (double)th / (1. + 0.6078 * fmax(kQvmin, q));
      t = theta_nv * pow(p / kP1000, kRd / kCp);
    } else {
      const float pf = phillips((float)pk, (float)pk1);
      const float qf = fmaxf(float(kQvmin), (float)qv);
      const float theta_nv = (float)th / (1.f + 0.6078f * qf);
      p = (double)pf;
      q = (double)qf;
      t = (double)(theta_nv * powf(pf / float(kP1000), float(kRd / kCp)));
    }
    gfs_dp[g] = (0.001 * (double)pk) - (0.001 * (double)pk1);
    gfs_p[g] = p;
    gfs_u[g] = u;
    gfs_v[g] = v;
    gfs_dpdt[g] = 0.001 * w;
    gfs_q[g] = q;
    gfs_oz[g] = (double)oz;
    gfs_cld[g] = (double)cld;
    gfs_t[g] = t;
    old6[g] = u;
    old6[NL + g] = v;
    old6[2 * NL + g] = t;
    old6[3 * NL + g] = q;
    old6[4 * NL + g] = (double)oz;
    old6[5 * NL + g] = (double)cld;
  }
}

// physics tendencies of u, v, t, q, cld, oz (cpl_run.F90:414-425), level
// fastest: tend[f][i*L + k]
__global__ void __launch_bounds__(kCplTile * kCplRows) k_cpl_tend(int N, int L, double dtp,
    const double* __restrict__ gfs_u, const double* __restrict__ gfs_v, const double* __restrict__ gfs_t,
    const double* __restrict__ gfs_q, const double* __restrict__ gfs_cld, const double* __restrict__ gfs_oz,
    const double* __restrict__ old6, double* __restrict__ tend) {
  const int i = blockIdx.x * kCplTile + threadIdx.x;
  if (i >= N) return;
  const size_t NL = (size_t)N * L;
  const int k1 = (blockIdx.y + 1) * kCplTile < L ? (blockIdx.y + 1) * kCplTile : L;
  for (int k = blockIdx.y * kCplTile + threadIdx.y; k < k1; k += kCplRows) {
    const size_t c = (size_t)i * L + k, g = (size_t)k * N + i;
    tend[c] = (gfs_u[g] - old6[g]) / dtp;
    tend[NL + c] = (gfs_v[g] - old6[NL + g]) / dtp;
    tend[2 * NL + c] = (gfs_t[g] - old6[2 * NL + g]) / dtp;
    tend[3 * NL + c] = (gfs_q[g] - old6[3 * NL + g]) / dtp;
    tend[4 * NL + c] = (gfs_cld[g] - old6[5 * NL + g]) / dtp;
    tend[5 * NL + c] = (gfs_oz[g] - old6[4 * NL + g]) / dtp;
  }
}

// dffusn8_lyr (dffusn_lyr.exe): thickness-weighted 1-ring diffusion of the
// six tendency fields (blockIdx.y), out of place; thread per (cell, level)
template <typename R>
__global__ void __launch_bounds__(256) k_cpl_dffusn(Grid<R> g, double dfflen, const R* __restrict__ delp,
                                                   const double* __restrict__ in, double* __restrict__ out) {
  const int N = g.N, L = g.L;
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (long long)N * L) return;
  const int i = (int)(gid / L), k = (int)(gid - (long long)i * L);
  const size_t NL = (size_t)N * L;
  in += blockIdx.y * NL;
  out += blockIdx.y * NL;
  const double thshld = 1.e-11;
  const size_t c = (size_t)i * L + k;
  const double f = in[c], a = fmax((double)delp[c], thshld);
  const int np = g.nprox[i];
  double flxdv = 0.;
  for (int e = 0; e < np; e++) {
    const int ipx = g.prox[i * 6 + e];
    const size_t cx = (size_t)ipx * L + k;
    const double b = fmax((double)delp[cx], thshld);
    flxdv = flxdv + (f - in[cx]) * (double)g.sideln[i * 6 + e] * 2. * (a * b / (a + b));
  }
  out[c] = f + flxdv * (-dfflen * (double)g.rarea[i] / a);
}

// cpl_phy_to_dyn (cpl_run.F90:453-480): the new dynamics state; tend is null
// without addtend
template <typename R>
__global__ void __launch_bounds__(kCplTile * kCplRows) k_cpl_p2d(int N, int L, double dt,
    const double* __restrict__ gfs_p, const double* __restrict__ gfs_u, const double* __restrict__ gfs_v,
    const double* __restrict__ gfs_q, const double* __restrict__ gfs_cld, const double* __restrict__ gfs_oz,
    const double* __restrict__ gfs_t, const double* __restrict__ old6, const double* __restrict__ tend,
    const double* __restrict__ geshem, const double* __restrict__ rainc, const double* __restrict__ evap,
    R* __restrict__ us3d, R* __restrict__ vs3d, R* __restrict__ tr3d, R* __restrict__ rn2d,
    R* __restrict__ rc2d, R* __restrict__ qf2d) {
  __shared__ R tile[kCplTile][kCplTile + 1];
  const int i0 = blockIdx.x * kCplTile, k0 = blockIdx.y * kCplTile;
  const int i = i0 + threadIdx.x;
  const size_t NL = (size_t)N * L;
  const bool live = i < N;
  if (live && blockIdx.y == 0 && threadIdx.y == 0) {
    rn2d[i] = R((double)rn2d[i] + fmax(0., geshem[i]) * 1000.);
    rc2d[i] = R((double)rc2d[i] + fmax(0., rainc[i]) * 1000.);
    qf2d[i] = R(-evap[i]);
  }
  R ou[kCplV], ov[kCplV], oth[kCplV], oq[kCplV], oc[kCplV], oo[kCplV];
#pragma unroll
  for (int j = 0; j < kCplV; j++) {
    const int k = k0 + threadIdx.y + kCplRows * j;
    ou[j] = ov[j] = oth[j] = oq[j] = oc[j] = oo[j] = R(0);
    if (!live || k >= L) continue;
    const size_t c = (size_t)i * L + k, g = (size_t)k * N + i;
    double u, v, t, q, cld, oz;
    if (tend) {
      u = old6[g] + tend[c] * dt;
      v = old6[NL + g] + tend[NL + c] * dt;
      t = old6[2 * NL + g] + tend[2 * NL + c] * dt;
      q = old6[3 * NL + g] + tend[3 * NL + c] * dt;
      cld = old6[5 * NL + g] + tend[4 * NL + c] * dt;
      oz = old6[4 * NL + g] + tend[5 * NL + c] * dt;
    } else {
      u = gfs_u[g]; v = gfs_v[g]; t = gfs_t[g]; q = gfs_q[g]; cld = gfs_cld[g]; oz = gfs_oz[g];
    }
    const double p = gfs_p[g];
    if constexpr (sizeof(R) == 8) {
      oth[j] = t * pow(kP1000 / p, kRd / kCp) * (1. + 0.6078 * fmax(kQvmin, q));
    } else {
      const float qf = fmaxf(float(kQvmin), (float)q);
      oth[j] = (float)t * powf(float(kP1000) / (float)p, float(kRd / kCp)) * (1.f + 0.6078f * qf);
    }
    ou[j] = R(u);
    ov[j] = R(v);
    oq[j] = R(fmax(kQvmin, q));
    oc[j] = R(fmax(kQwmin, cld));
    oo[j] = R(fmax(kQvmin, oz));
  }
  tile_out<R>(us3d, L, L, i0, k0, N, tile, ou);
  tile_out<R>(vs3d, L, L, i0, k0, N, tile, ov);
  tile_out<R>(tr3d, L, L, i0, k0, N, tile, oth);
  tile_out<R>(tr3d + NL, L, L, i0, k0, N, tile, oq);
  tile_out<R>(tr3d + 2 * NL, L, L, i0, k0, N, tile, oc);
  tile_out<R>(tr3d + 3 * NL, L, L, i0, k0, N, tile, oo);
}

template <typename R>
void launch_cpl_dyn_to_phy(const Launch& l, const Grid<R>& g, const R* pr3d, const R* us3d, const R* vs3d,
                           const R* ws3d, const R* tr3d, double* const gfs[10], double* old6) {
  const dim3 grid((g.N + kCplTile - 1) / kCplTile, (g.L + kCplTile - 1) / kCplTile);
  FIM_KBEGIN(l, "k_cpl_d2p");
  k_cpl_d2p<R><<<grid, dim3(kCplTile, kCplRows), 0, l.stream>>>(g.N, g.L, pr3d, us3d, vs3d, ws3d, tr3d, gfs[0],
                                                                 gfs[1], gfs[2], gfs[3], gfs[4], gfs[5], gfs[6],
                                                                 gfs[7], gfs[8], gfs[9], old6);
  FIM_KEND(l);
}

// gfs7 = p, u, v, q, cld, oz, t; col3 = geshem, rainc, evap; tend: 6 N L
// doubles of scratch when addtend
template <typename R>
void launch_cpl_phy_to_dyn(const Launch& l, const Grid<R>& g, double dt, double dtp, bool addtend,
                           bool smoothtend, const double* const gfs7[7], const double* old6,
                           const double* const col3[3], const R* dp3d, R* us3d, R* vs3d, R* tr3d, R* rn2d,
                           R* rc2d, R* qf2d, double* tend) {
  const dim3 grid((g.N + kCplTile - 1) / kCplTile, (g.L + kCplTile - 1) / kCplTile);
  const dim3 block(kCplTile, kCplRows);
  const double* td = nullptr;
  if (addtend) {
    FIM_KBEGIN(l, "k_cpl_tend");
    k_cpl_tend<<<grid, block, 0, l.stream>>>(g.N, g.L, dtp, gfs7[1], gfs7[2], gfs7[6], gfs7[3], gfs7[4], gfs7[5],
                                             old6, tend);
    FIM_KEND(l);
    td = tend;
    if (smoothtend) {
      const size_t NL = (size_t)g.N * g.L;
      double* sm = tend + 6 * NL;
      FIM_KBEGIN(l, "k_cpl_dffusn");
      k_cpl_dffusn<R><<<dim3((unsigned)((NL + 255) / 256), 6), 256, 0, l.stream>>>(g, dt * 20., dp3d, tend, sm);
      FIM_KEND(l);
      td = sm;
    }
  }
  FIM_KBEGIN(l, "k_cpl_p2d");
  k_cpl_p2d<R><<<grid, block, 0, l.stream>>>(g.N, g.L, dt, gfs7[0], gfs7[1], gfs7[2], gfs7[3], gfs7[4], gfs7[5],
                                              gfs7[6], old6, td, col3[0], col3[1], col3[2], us3d, vs3d, tr3d,
                                              rn2d, rc2d, qf2d);
  FIM_KEND(l);
}

#define INSTANTIATE(R)                                                                                       \
  template void launch_cpl_dyn_to_phy<R>(const Launch&, const Grid<R>&, const R*, const R*, const R*,       \
                                         const R*, const R*, double* const[10], double*);                    \
  template void launch_cpl_phy_to_dyn<R>(const Launch&, const Grid<R>&, double, double, bool, bool,         \
                                         const double* const[7], const double*, const double* const[3],      \
                                         const R*, R*, R*, R*, R*, R*, R*, double*);
INSTANTIATE(float)
INSTANTIATE(double)

}  // namespace fim
