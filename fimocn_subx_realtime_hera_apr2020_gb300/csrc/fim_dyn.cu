// Horizontal stencil kernels of the FIM dynamics step: edgvar1, edgvar3,
// cnuity1..5, trcadv1..3, del4prep/dissip/momtum1.
//
// Layout is the reference's (level index fastest), so one thread per
// (level, cell) gives fully coalesced loads along k for own and neighbour
// columns alike; a warp covers 32 consecutive levels of one cell and the grid
// tables of that cell are warp-uniform (broadcast loads).  Kernels whose
// result couples levels of one column (the cnuity5 pressure/omega scan and the
// momtum1 Rayleigh damping) run one warp per column and scan with shuffles.
// Ensemble members map to gridDim.y; all members share the grid tables.
//
// Every kernel restates the arithmetic of the reference routine it names,
// in the same order, with the reference's 'real' mapped to the template type R.
#include "fim_internal.h"

namespace fim {

template <typename R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }
template <typename R> __device__ __forceinline__ R rabs(R a) { return a < R(0) ? -a : a; }

constexpr int kBlock = 256;

__device__ __forceinline__ bool cell_level(int N, int L, int& i, int& k) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * L) return false;
  i = gid / L;
  k = gid - i * L;
  return true;
}

inline unsigned blocks_for(long long n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

// --------------------------------------------------------------------------
// edgvar1 (edgvar1.F90:156-511, eqwgt=.true., janjic=0): rotate u,v of the
// cell, the cell across the edge and the cells across the two adjacent edges
// into the edge frame, equal-weight interpolate with magnitude correction;
// mid-layer pressure, Montgomery potential, kinetic energy and tracer 1 (all
// tracers and dp when hi_order == 0) on the cell's own edges.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_edgvar1(Grid<R> g, Strides s, int hi_order,
    const R* __restrict__ u, const R* __restrict__ v, const R* __restrict__ delp,
    const R* __restrict__ pres, const R* __restrict__ montg, const R* __restrict__ tracr,
    R* __restrict__ u_edg, R* __restrict__ v_edg, R* __restrict__ dp_edg, R* __restrict__ lp_edg,
    R* __restrict__ mont_edg, R* __restrict__ uvsq_edg, R* __restrict__ trc_edg, const float2* __restrict__ mpf,
    R* __restrict__ thold) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N, L1 = L + 1;
  const size_t m = blockIdx.y;
  if (mpf) mpf += m * s.cell;
  if (thold) {
    // the potential temperature of this step's edge values, for momtum1
    thold += m * s.cell;
    thold[(size_t)i * L + k] = tracr[m * s.tr + (size_t)i * L + k];
  }
  u += m * s.cell; v += m * s.cell; delp += m * s.cell; pres += m * s.intf;
  montg += m * s.cell; tracr += m * s.tr;
  u_edg += m * s.edge; v_edg += m * s.edge; dp_edg += m * s.edge; lp_edg += m * s.edge;
  mont_edg += m * s.edge; uvsq_edg += m * s.edge; trc_edg += m * s.tredg;
  const R divby6 = R(1) / R(6), eps = R(0.001), two = R(2), half = R(0.5);
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  const R u1 = u[(size_t)i * L + k], v1 = v[(size_t)i * L + k];
  const R p1a = pres[(size_t)i * L1 + k], p1b = pres[(size_t)i * L1 + k + 1];
  const R m1 = montg[(size_t)i * L + k];
  for (int e = 0; e < np; e++) {
    const int i2 = pr[e], i3t = pr[e == 0 ? np - 1 : e - 1], i3l = pr[e == np - 1 ? 0 : e + 1];
    const R* cs = g.cs + (i * 6 + e) * 4;
    const R* sn = g.sn + (i * 6 + e) * 4;
    const R ut = u[(size_t)i3t * L + k], vt = v[(size_t)i3t * L + k];
    const R u2 = u[(size_t)i2 * L + k], v2 = v[(size_t)i2 * L + k];
    const R ul = u[(size_t)i3l * L + k], vl = v[(size_t)i3l * L + k];
    const R u3trl = cs[2] * ut + sn[2] * vt, v3trl = -sn[2] * ut + cs[2] * vt;
    const R u1ldg = cs[0] * u1 + sn[0] * v1, v1ldg = -sn[0] * u1 + cs[0] * v1;
    const R u2ldg = cs[1] * u2 + sn[1] * v2, v2ldg = -sn[1] * u2 + cs[1] * v2;
    const R u3ldg = cs[3] * ul + sn[3] * vl, v3ldg = -sn[3] * ul + cs[3] * vl;
    R ue = (two * (u1ldg + u2ldg) + u3trl + u3ldg) * divby6;
    R ve = (two * (v1ldg + v2ldg) + v3trl + v3ldg) * divby6;
    const R m_1ldg = sqrt(u1ldg * u1ldg + v1ldg * v1ldg);
    const R m_2ldg = sqrt(u2ldg * u2ldg + v2ldg * v2ldg);
    const R m_3trl = sqrt(u3trl * u3trl + v3trl * v3trl);
    const R m_3ldg = sqrt(u3ldg * u3ldg + v3ldg * v3ldg);
    const R m_1 = sqrt(ue * ue + ve * ve);
    const R m_2 = (two * (m_1ldg + m_2ldg) + m_3trl + m_3ldg) * divby6;
    ue = ue * m_2 / rmax(eps, m_1);
    ve = ve * m_2 / rmax(eps, m_1);
    const size_t o = ((size_t)i * 6 + e) * L + k;
    u_edg[o] = ue;
    v_edg[o] = ve;
    if (!hi_order)
      dp_edg[o] = (two * (delp[(size_t)i * L + k] + delp[(size_t)i2 * L + k]) + delp[(size_t)i3t * L + k] +
                   delp[(size_t)i3l * L + k]) * divby6;
    lp_edg[o] = (p1a + p1b + pres[(size_t)i2 * L1 + k] + pres[(size_t)i2 * L1 + k + 1] +
                 half * (pres[(size_t)i3t * L1 + k] + pres[(size_t)i3t * L1 + k + 1] +
                         pres[(size_t)i3l * L1 + k] + pres[(size_t)i3l * L1 + k + 1])) * divby6;
    if (mpf) {
      // edge minus cell value from float-float differences (no cancellation)
      const float2 mc = mpf[(size_t)i * L + k];
      mont_edg[o] = R((2.f * ff_diff(mpf[(size_t)i2 * L + k], mc) + ff_diff(mpf[(size_t)i3t * L + k], mc) +
                       ff_diff(mpf[(size_t)i3l * L + k], mc)) * (1.f / 6.f));
    } else {
      mont_edg[o] = (two * (m1 + montg[(size_t)i2 * L + k]) + montg[(size_t)i3t * L + k] +
                     montg[(size_t)i3l * L + k]) * divby6;
    }
    uvsq_edg[o] = half * (ue * ue + ve * ve);
  }
  const int ntr = hi_order ? 1 : g.T;
  for (int t = 0; t < ntr; t++) {
    const R* tr = tracr + (size_t)t * N * L;
    R* te = trc_edg + (size_t)t * N * 6 * L;
    te[((size_t)i * 6 + 5) * L + k] = R(0);
    for (int e = 0; e < np; e++) {
      const int i2 = pr[e], i3t = pr[e == 0 ? np - 1 : e - 1], i3l = pr[e == np - 1 ? 0 : e + 1];
      te[((size_t)i * 6 + e) * L + k] = (two * (tr[(size_t)i * L + k] + tr[(size_t)i2 * L + k]) +
                                         tr[(size_t)i3t * L + k] + tr[(size_t)i3l * L + k]) * divby6;
    }
  }
}

// --------------------------------------------------------------------------
// edgvar3 loop 1 with edgvalEval (edgvar3.F90:66-94,136-163): least-squares
// (hfcoef) reconstruction of dp (field 0) and tracers 2..ntra (field t) on the
// cell's own edges; pentagons store 0 in the sixth slot.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_edgvar3_own(Grid<R> g, Strides s,
    const R* __restrict__ delp, const R* __restrict__ tracr, R* __restrict__ dp_edg, R* __restrict__ trc_edg) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  const int f = blockIdx.z;
  const R* src = (f == 0) ? delp + m * s.cell : tracr + m * s.tr + (size_t)f * N * L;
  R* dst = (f == 0) ? dp_edg + m * s.edge : trc_edg + m * s.tredg + (size_t)f * N * 6 * L;
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  const R bc = src[(size_t)i * L + k];
  R d[6];
#pragma unroll
  for (int j = 0; j < 6; j++) d[j] = (j < np) ? src[(size_t)pr[j] * L + k] - bc : R(0);
  const R* hf = g.hfcoef + (size_t)i * 36;
#pragma unroll
  for (int ie = 0; ie < 6; ie++) {
    R val = R(0);
    if (ie < np) {
      val = bc;
#pragma unroll
      for (int j = 0; j < 6; j++)
        if (j < np) val = val + d[j] * hf[ie * 6 + j];
    }
    dst[((size_t)i * 6 + ie) * L + k] = val;
  }
}

// edgvar3 loop 2 (edgvar3.F90:110-132): the lower-numbered cell of each pair
// stores the two-sided average in both slots, as the reference does; each slot
// has exactly one writer, which is also its only reader.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_edgvar3_avg(Grid<R> g, Strides s, R* __restrict__ dp_edg,
                                                       R* __restrict__ trc_edg) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  const int f = blockIdx.z;
  R* x = (f == 0) ? dp_edg + m * s.edge : trc_edg + m * s.tredg + (size_t)f * N * 6 * L;
  const int np = g.nprox[i];
  for (int e = 0; e < np; e++) {
    const int nb = g.prox[i * 6 + e];
    if (i < nb) {
      const int os = g.proxs[i * 6 + e];
      const size_t a = ((size_t)i * 6 + e) * L + k, b = ((size_t)nb * 6 + os) * L + k;
      const R w = R(0.5) * (x[a] + x[b]);
      x[a] = w;
      x[b] = w;
    }
  }
}

// --------------------------------------------------------------------------
// cnuity1 + cnuity2 (cnuity_compute.F90:41-146): normal velocity on the cell's
// edge and on the neighbour's copy of it, donor-cell mass flux, antidiffusive
// flux, low-order tendency and low-order thickness; also the Zalesak sums
// P+/P- of cnuity3 (cnuity_compute.F90:186-194), which only need own edges.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_cnuity12(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ u_edg, const R* __restrict__ v_edg, const R* __restrict__ dp_edg,
    const R* __restrict__ delp, R* __restrict__ massfx, R* __restrict__ dplo_tndcy, R* __restrict__ antifx,
    R* __restrict__ delp_lo, R* __restrict__ p_plus, R* __restrict__ p_mnus) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  u_edg += m * s.edge; v_edg += m * s.edge; dp_edg += m * s.edge; delp += m * s.cell;
  massfx += m * s.mf; dplo_tndcy += m * s.ab; antifx += m * s.edge; delp_lo += m * s.cell;
  p_plus += m * s.cell; p_mnus += m * s.cell;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  R* mfn = massfx + (size_t)nf * N * 6 * L;
  const int np = g.nprox[i];
  const R half = R(0.5);
  const R dpi = delp[(size_t)i * L + k];
  R sum = R(0), pp = R(0), pm = R(0);
  if (np < 6) {
    mfn[((size_t)i * 6 + 5) * L + k] = R(0);
    antifx[((size_t)i * 6 + 5) * L + k] = R(0);
  }
  for (int e = 0; e < np; e++) {
    const int ipx = g.prox[i * 6 + e], edx = g.proxs[i * 6 + e];
    const R* sv = g.sve + (i * 6 + e) * 2;
    const R* sx = g.sve + (ipx * 6 + edx) * 2;
    const size_t o = ((size_t)i * 6 + e) * L + k, ox = ((size_t)ipx * 6 + edx) * L + k;
    const R vn = sv[1] * u_edg[o] - sv[0] * v_edg[o];
    const R vx = sx[1] * u_edg[ox] - sx[0] * v_edg[ox];
    const R flxhi = vn * dp_edg[o];
    const R mf = half * ((vn + rabs(vn)) * dpi - (vx + rabs(vx)) * delp[(size_t)ipx * L + k]);
    mfn[o] = mf;
    const R a = flxhi - mf;
    antifx[o] = a;
    sum = sum + mf;
    if (a <= R(0)) pp = pp - a;
    else pm = pm + a;
  }
  const size_t c = (size_t)i * L + k;
  const R tn = -sum * g.rarea[i];
  dplo_tndcy[(size_t)nf * N * L + c] = tn;
  delp_lo[c] = dpi + ab1 * tn + ab2 * dplo_tndcy[(size_t)of * N * L + c] + ab3 * dplo_tndcy[(size_t)vof * N * L + c];
  p_plus[c] = pp;
  p_mnus[c] = pm;
}

// cnuity3 (cnuity_compute.F90:206-252): 1-ring max/min of old and low-order
// thickness, Zalesak Q+/Q- and the limiters R+/R-.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_cnuity3(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ delp_lo, const R* __restrict__ delp, const R* __restrict__ dp_tndcy,
    const R* __restrict__ p_plus, const R* __restrict__ p_mnus, R* __restrict__ r_plus, R* __restrict__ r_mnus) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  delp_lo += m * s.cell; delp += m * s.cell; dp_tndcy += m * s.ab;
  p_plus += m * s.cell; p_mnus += m * s.cell; r_plus += m * s.cell; r_mnus += m * s.cell;
  const int of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11);
  const size_t c = (size_t)i * L + k;
  const int* pr = g.prox + i * 6;
  const R dlo = delp_lo[c];
  R dpmax = rmax(dlo, delp[c]), dpmin = rmin(dlo, delp[c]);
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const R a = delp_lo[(size_t)pr[e] * L + k], b = delp[(size_t)pr[e] * L + k];
    dpmax = rmax(dpmax, rmax(a, b));
    dpmin = rmin(dpmin, rmin(a, b));
  }
  dpmax = rmax(R(0), dpmax);
  dpmin = rmax(R(0), dpmin);
  const R to = dp_tndcy[(size_t)of * N * L + c], tv = dp_tndcy[(size_t)vof * N * L + c];
  const R q_plus = (dpmax - dlo - (ab2 * rmin(R(0), to) + ab3 * rmax(R(0), tv))) / ab1 * g.area[i];
  const R q_mnus = (dlo - dpmin + (ab2 * rmax(R(0), to) + ab3 * rmin(R(0), tv))) / ab1 * g.area[i];
  r_plus[c] = rmax(R(0), rmin(R(1), q_plus / rmax(p_plus[c], thshld)));
  r_mnus[c] = rmax(R(0), rmin(R(1), q_mnus / rmax(p_mnus[c], thshld)));
}

// cnuity4 (cnuity_compute.F90:291-369): clip the antidiffusive flux with the
// own and neighbour limiters, total mass flux, AB3 thickness update.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_cnuity4(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ antifx, const R* __restrict__ r_plus, const R* __restrict__ r_mnus,
    R* __restrict__ massfx, const R* __restrict__ dplo_tndcy, R* __restrict__ dp_tndcy, R* __restrict__ delp,
    int* __restrict__ flags) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  antifx += m * s.edge; r_plus += m * s.cell; r_mnus += m * s.cell; massfx += m * s.mf;
  dplo_tndcy += m * s.ab; dp_tndcy += m * s.ab; delp += m * s.cell;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  R* mfn = massfx + (size_t)nf * N * 6 * L;
  const size_t c = (size_t)i * L + k;
  const R rp = r_plus[c], rm = r_mnus[c];
  const int np = g.nprox[i];
  R at = R(0);
  for (int e = 0; e < np; e++) {
    const int px = g.prox[i * 6 + e];
    const size_t o = ((size_t)i * 6 + e) * L + k;
    R a = antifx[o];
    const R clip = (a >= R(0)) ? rmin(rm, r_plus[(size_t)px * L + k]) : rmin(rp, r_mnus[(size_t)px * L + k]);
    a = a * clip;
    mfn[o] = mfn[o] + a;
    at = at + a;
  }
  at = -at * g.rarea[i];
  const R tn = dplo_tndcy[(size_t)nf * N * L + c] + at;
  dp_tndcy[(size_t)nf * N * L + c] = tn;
  const R dn = delp[c] + ab1 * tn + ab2 * dp_tndcy[(size_t)of * N * L + c] + ab3 * dp_tndcy[(size_t)vof * N * L + c];
  delp[c] = dn;
  if (!(dn > R(0))) atomicOr(flags + m, kFlagBadDp);
}

// cnuity5 (cnuity_compute.F90:408-445): one warp per column; the top-down
// pressure sum and the omega flux-convergence integral are warp scans in FP64
// (FP64 column accumulation in both precisions), then Exner function and the
// v.grad(p) term per level.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_cnuity5(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    R* __restrict__ pres, R* __restrict__ delp, R* __restrict__ exner, const R* __restrict__ dp_tndcy,
    R* __restrict__ omega, const R* __restrict__ lp_edg, const R* __restrict__ u, const R* __restrict__ v,
    int ab3_delp) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int N = g.N, L = g.L, L1 = L + 1;
  if (warp >= N) return;
  const int i = warp;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  pres += m * s.intf; delp += m * s.cell; exner += m * s.intf; dp_tndcy += m * s.ab;
  omega += m * s.cell; lp_edg += m * s.edge; u += m * s.cell; v += m * s.cell;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3), dt = R(sp->dt);
  const R cp = R(kCp), p1000 = R(kP1000), rdcp = R(kRd) / R(kCp);
  const int np = g.nprox[i];
  const R rar = g.rarea[i];
  if constexpr (sizeof(R) == 4) {
    // float-float column sums (FP64-accurate on the FP32 pipes)
    FF2 carry_p{pres[(size_t)i * L1 + L], 0.f}, carry_c{0.f, 0.f};
    for (int base = 0; base < L; base += 32) {
      const int j = base + lane;
      const bool act = j < L;
      const int k = L - 1 - j;
      float d = 0.f, lyr = 0.f;
      if (act) {
        const size_t c = (size_t)i * L + k;
        const R tnf = dp_tndcy[(size_t)nf * N * L + c], tof = dp_tndcy[(size_t)of * N * L + c],
                tvf = dp_tndcy[(size_t)vof * N * L + c];
        if (ab3_delp) {
          // massflux_newdepth's AB3 thickness update (massadv_compute.F90:85-91)
          R dn = delp[c] + ab1 * tnf + ab2 * tof + ab3 * tvf;
          dn = dn > R(0) ? dn : R(0);
          delp[c] = dn;
        }
        d = delp[c];
        lyr = (ab1 * tnf + ab2 * tof + ab3 * tvf) / dt;
      }
      FF2 sd{d, 0.f}, sl{lyr, 0.f};
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const FF2 a = ff_shfl_up(sd, off), b = ff_shfl_up(sl, off);
        if (lane >= off) { sd = ff_add(sd, a); sl = ff_add(sl, b); }
      }
      if (act) {
        const size_t c = (size_t)i * L + k;
        const FF2 p = ff_add(carry_p, sd);
        const R pr = p.hi;
        pres[(size_t)i * L1 + k] = pr;
        exner[(size_t)i * L1 + k] = cp * pow(pr / p1000, rdcp);
        // omega = (integral of layers above) + half of this layer
        const FF2 above = ff_add(carry_c, ff_add(sl, FF2{-lyr, 0.f}));
        R om = R(above.hi + above.lo) + R(0.5) * lyr;
        R dpdx = R(0), dpdy = R(0);
        for (int e = 0; e < np; e++) {
          const R* sv = g.svc + (i * 6 + e) * 2;
          const R lp = lp_edg[((size_t)i * 6 + e) * L + k];
          dpdx = dpdx + lp * sv[1];
          dpdy = dpdy - lp * sv[0];
        }
        om = om + (u[c] * dpdx + v[c] * dpdy) * rar;
        omega[c] = om;
      }
      carry_p = ff_add(carry_p, ff_shfl(sd, 31));
      carry_c = ff_add(carry_c, ff_shfl(sl, 31));
    }
    return;
  }
  double carry_p = (double)pres[(size_t)i * L1 + L];
  double carry_c = 0.0;
  for (int base = 0; base < L; base += 32) {
    const int j = base + lane;
    const bool act = j < L;
    const int k = L - 1 - j;
    double d = 0.0, lt = 0.0;
    R lyr = R(0);
    if (act) {
      const size_t c = (size_t)i * L + k;
      const R tnf = dp_tndcy[(size_t)nf * N * L + c], tof = dp_tndcy[(size_t)of * N * L + c],
              tvf = dp_tndcy[(size_t)vof * N * L + c];
      if (ab3_delp) {
        // massflux_newdepth's AB3 thickness update (massadv_compute.F90:85-91)
        R dn = delp[c] + ab1 * tnf + ab2 * tof + ab3 * tvf;
        dn = dn > R(0) ? dn : R(0);
        delp[c] = dn;
      }
      d = (double)delp[c];
      lyr = (ab1 * tnf + ab2 * tof + ab3 * tvf) / dt;
      lt = (double)lyr;
    }
    double sd = d, sl = lt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const double a = __shfl_up_sync(0xffffffffu, sd, off);
      const double b = __shfl_up_sync(0xffffffffu, sl, off);
      if (lane >= off) { sd += a; sl += b; }
    }
    if (act) {
      const size_t c = (size_t)i * L + k;
      const double p = carry_p + sd;
      const R pr = R(p);
      pres[(size_t)i * L1 + k] = pr;
      exner[(size_t)i * L1 + k] = cp * pow(pr / p1000, rdcp);
      // omega = (integral of layers above) + half of this layer
      R om = R(carry_c + (sl - lt)) + R(0.5) * lyr;
      R dpdx = R(0), dpdy = R(0);
      for (int e = 0; e < np; e++) {
        const R* sv = g.svc + (i * 6 + e) * 2;
        const R lp = lp_edg[((size_t)i * 6 + e) * L + k];
        dpdx = dpdx + lp * sv[1];
        dpdy = dpdy - lp * sv[0];
      }
      om = om + (u[c] * dpdx + v[c] * dpdy) * rar;
      omega[c] = om;
    }
    carry_p += __shfl_sync(0xffffffffu, sd, 31);
    carry_c += __shfl_sync(0xffffffffu, sl, 31);
  }
}

// --------------------------------------------------------------------------
// mass_adv (flux_conserv_schm = 2, the reference default): flux_limiter.F90
// edgeNormVel + limiter (M1 branch).  k_massadv_lim: bounded edge thickness
// q* per edge and the outflow bounds q_min_out/q_max_out per cell
// (flux_limiter.F90:149-233).  k_massadv_flux: limited edge thickness with
// the upwind cell's bounds, mass flux, dp tendency (flux_limiter.F90:247-259,
// massadv_compute.F90:45-83); the AB3 thickness update runs in k_cnuity5.
template <typename R>
__device__ __forceinline__ void ma_edge(const Grid<R>& g, int i, int k, int e, int np, const R* u_edg,
                                        const R* v_edg, const R* dp_edg, const R* delp, R& vn, R& qs, int& ipx) {
  const int L = g.L;
  const int* pr = g.prox + i * 6;
  ipx = pr[e];
  const int nbm1 = pr[e == 0 ? np - 1 : e - 1], nbp1 = pr[e == np - 1 ? 0 : e + 1];
  const R* sv = g.sve + (i * 6 + e) * 2;
  const size_t o = ((size_t)i * 6 + e) * L + k;
  vn = sv[1] * u_edg[o] - sv[0] * v_edg[o];
  const R a = delp[(size_t)i * L + k], b = delp[(size_t)ipx * L + k], c = delp[(size_t)nbm1 * L + k],
          d = delp[(size_t)nbp1 * L + k];
  const R qmn = rmin(rmin(rmin(a, b), c), d), qmx = rmax(rmax(rmax(a, b), c), d);
  qs = rmax(qmn, rmin(qmx, dp_edg[o]));
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_massadv_lim(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ u_edg, const R* __restrict__ v_edg, const R* __restrict__ dp_edg,
    const R* __restrict__ delp, const R* __restrict__ dp_tndcy, R* __restrict__ qmin_out, R* __restrict__ qmax_out) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  u_edg += m * s.edge; v_edg += m * s.edge; dp_edg += m * s.edge; delp += m * s.cell; dp_tndcy += m * s.ab;
  qmin_out += m * s.cell; qmax_out += m * s.cell;
  const int of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3), dt = R(sp->dt);
  const size_t c = (size_t)i * L + k;
  const R gv = delp[c], rar = g.rarea[i];
  const int np = g.nprox[i];
  R qminin = sizeof(R) == 8 ? R(1.79769313486231571e308) : R(3.40282347e38f), qmaxin = R(0);
  R cqmin = R(0), cqmax = R(0), cin = R(0), cout = R(0);
  for (int e = 0; e < np; e++) {
    R vn, qs;
    int ipx;
    ma_edge(g, i, k, e, np, u_edg, v_edg, dp_edg, delp, vn, qs, ipx);
    const R cn = rabs(vn) * dt * rar;
    if (vn > R(0)) {
      cout = cout + cn;
    } else {
      const R gx = delp[(size_t)ipx * L + k];
      const R qmn = rmin(qs, gx), qmx = rmax(qs, gx);
      cin = cin + cn;
      qminin = rmin(qminin, qmn);
      qmaxin = rmax(qmaxin, qmx);
      cqmin = cqmin + cn * qmn;
      cqmax = cqmax + cn * qmx;
    }
  }
  const R qmin_next = rmin(gv, qminin), qmax_next = rmax(gv, qmaxin);
  if (cout != R(0)) {
    const R to = dp_tndcy[(size_t)of * N * L + c], tv = dp_tndcy[(size_t)vof * N * L + c];
    qmin_out[c] = (gv + ab1 / dt * cqmax - qmax_next * (R(1) + cin - cout) + ab2 * to + ab3 * tv) / cout / ab1 * dt;
    qmax_out[c] = (gv + ab1 / dt * cqmin - qmin_next * (R(1) + cin - cout) + ab2 * to + ab3 * tv) / cout / ab1 * dt;
  } else {
    qmin_out[c] = R(-100000.0);
    qmax_out[c] = R(100000.0);
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_massadv_flux(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ u_edg, const R* __restrict__ v_edg, R* __restrict__ dp_edg, const R* __restrict__ delp,
    const R* __restrict__ qmin_out, const R* __restrict__ qmax_out, R* __restrict__ massfx, R* __restrict__ dp_tndcy) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  u_edg += m * s.edge; v_edg += m * s.edge; dp_edg += m * s.edge; delp += m * s.cell; dp_tndcy += m * s.ab;
  qmin_out += m * s.cell; qmax_out += m * s.cell; massfx += m * s.mf;
  const int nf = sp->nf;
  R* mfn = massfx + (size_t)nf * N * 6 * L;
  const int np = g.nprox[i];
  R vnv[6], dpe[6];
#pragma unroll
  for (int e = 0; e < 6; e++) {
    if (e < np) {
      R vn, qs;
      int ipx;
      ma_edge(g, i, k, e, np, u_edg, v_edg, dp_edg, delp, vn, qs, ipx);
      const size_t cs = (size_t)(vn > R(0) ? i : ipx) * L + k;
      vnv[e] = vn;
      dpe[e] = rmax(qmin_out[cs], rmin(qmax_out[cs], qs));
    }
  }
  R t = R(0);
#pragma unroll
  for (int e = 0; e < 6; e++) {
    if (e < np) {
      const size_t o = ((size_t)i * 6 + e) * L + k;
      dp_edg[o] = dpe[e];
      const R mf = vnv[e] * dpe[e];
      mfn[o] = mf;
      t = t + mf;
    }
  }
  dp_tndcy[(size_t)nf * N * L + (size_t)i * L + k] = -t * g.rarea[i];
}

template <typename R>
void launch_massadv(const Launch& l, const Grid<R>& g, const Strides& s, const CnuityScratch<R>& w, const R* u,
                    const R* v, const R* u_edg, const R* v_edg, R* dp_edg, const R* lp_edg, R* delp, R* pres,
                    R* exner, R* dp_tndcy, R* massfx, R* omega) {
  dim3 grid(blocks_for((long long)g.N * g.L), l.members);
  FIM_KBEGIN(l, "k_massadv_lim");
  k_massadv_lim<R><<<grid, kBlock, 0, l.stream>>>(g, s, l.sp, u_edg, v_edg, dp_edg, delp, dp_tndcy, w.r_plus,
                                                   w.r_mnus);
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_massadv_flux");
  k_massadv_flux<R><<<grid, kBlock, 0, l.stream>>>(g, s, l.sp, u_edg, v_edg, dp_edg, delp, w.r_plus, w.r_mnus,
                                                    massfx, dp_tndcy);
  FIM_KEND(l);
  dim3 gw(blocks_for((long long)g.N * 32), l.members);
  FIM_KBEGIN(l, "k_cnuity5");
  k_cnuity5<R><<<gw, kBlock, 0, l.stream>>>(g, s, l.sp, pres, delp, exner, dp_tndcy, omega, lp_edg, u, v, 1);
  FIM_KEND(l);
}

// --------------------------------------------------------------------------
// trcadv1 (trcadv_compute.F90:55-135) for tracers t0..t0+gridDim.z-1.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_trcadv1(Grid<R> g, Strides s, const StepParams* __restrict__ sp, int t0,
    const R* __restrict__ massfx, const R* __restrict__ trc_edg, const R* __restrict__ tracr,
    const R* __restrict__ trcdp, R* __restrict__ trl_tdcy, const R* __restrict__ delp,
    R* __restrict__ antiflx, R* __restrict__ trmin, R* __restrict__ trmax, R* __restrict__ trcr_lo, size_t sc_stride) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const int tz = blockIdx.z, t = t0 + tz;
  const size_t NL = (size_t)N * L;
  massfx += m * s.mf; delp += m * s.cell;
  trc_edg += m * s.tredg + (size_t)t * 6 * NL;
  tracr += m * s.tr + (size_t)t * NL;
  trcdp += m * s.tr + (size_t)t * NL;
  trl_tdcy += m * s.trab + (size_t)t * 3 * NL;
  const size_t so = (m * gridDim.z + tz) * sc_stride;
  antiflx += so * 6; trmin += so; trmax += so; trcr_lo += so;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11), half = R(0.5);
  const R* mfn = massfx + (size_t)nf * N * 6 * L;
  const int np = g.nprox[i];
  const size_t c = (size_t)i * L + k;
  const R tri = tracr[c];
  if (np < 6) antiflx[((size_t)i * 6 + 5) * L + k] = R(0);
  R sumlo = R(0);
  for (int e = 0; e < np; e++) {
    const int ipx = g.prox[i * 6 + e], edx = g.proxs[i * 6 + e];
    const size_t o = ((size_t)i * 6 + e) * L + k;
    const R mf = mfn[o], mx = mfn[((size_t)ipx * 6 + edx) * L + k];
    const R flx_hi = mf * trc_edg[o];
    const R lo = half * ((mf + rabs(mf)) * tri - (mx + rabs(mx)) * tracr[(size_t)ipx * L + k]);
    antiflx[o] = flx_hi - lo;
    sumlo = sumlo + lo;
  }
  const R tn = -sumlo * g.rarea[i];
  trl_tdcy[(size_t)nf * NL + c] = tn;
  const R trcdp_lo = trcdp[c] + ab1 * tn + ab2 * trl_tdcy[(size_t)of * NL + c] + ab3 * trl_tdcy[(size_t)vof * NL + c];
  const int* pr = g.prox + i * 6;
  R mx = tri, mn = tri;
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const R x = tracr[(size_t)pr[e] * L + k];
    mx = rmax(mx, x);
    mn = rmin(mn, x);
  }
  mx = rmax(R(0), mx);
  mn = rmax(R(0), mn);
  trmax[c] = mx;
  trmin[c] = mn;
  trcr_lo[c] = rmax(mn, rmin(mx, trcdp_lo / rmax(thshld, delp[c])));
}

// trcadv2 (trcadv_compute.F90:171-235)
template <typename R>
__global__ void __launch_bounds__(kBlock) k_trcadv2(Grid<R> g, Strides s, const StepParams* __restrict__ sp, int t0,
    const R* __restrict__ trc_tdcy, const R* __restrict__ delp, const R* __restrict__ antiflx,
    R* __restrict__ trmin, R* __restrict__ trmax, const R* __restrict__ trcr_lo, R* __restrict__ r_plus,
    R* __restrict__ r_mnus, size_t sc_stride) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const int tz = blockIdx.z, t = t0 + tz;
  const size_t NL = (size_t)N * L;
  delp += m * s.cell;
  trc_tdcy += m * s.trab + (size_t)t * 3 * NL;
  const size_t so = (m * gridDim.z + tz) * sc_stride;
  antiflx += so * 6; trmin += so; trmax += so; trcr_lo += so; r_plus += so; r_mnus += so;
  const int of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11);
  const int np = g.nprox[i];
  const size_t c = (size_t)i * L + k;
  R s_plus = R(0), s_mnus = R(0);
  for (int e = 0; e < np; e++) {
    const R a = antiflx[((size_t)i * 6 + e) * L + k];
    s_plus = s_plus - rmin(R(0), a);
    s_mnus = s_mnus + rmax(R(0), a);
  }
  const R lo = trcr_lo[c];
  R mx = rmax(trmax[c], lo), mn = rmin(trmin[c], lo);
  const int* pr = g.prox + i * 6;
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const R x = trcr_lo[(size_t)pr[e] * L + k];
    mx = rmax(mx, x);
    mn = rmin(mn, x);
  }
  mx = rmax(R(0), mx);
  mn = rmax(R(0), mn);
  trmax[c] = mx;
  trmin[c] = mn;
  const R dp = delp[c];
  const R to = trc_tdcy[(size_t)of * NL + c], tv = trc_tdcy[(size_t)vof * NL + c];
  const R q_plus = ((mx - lo) * dp - (ab2 * rmin(R(0), to) + ab3 * rmax(R(0), tv))) / ab1 * g.area[i];
  const R q_mnus = ((lo - mn) * dp + (ab2 * rmax(R(0), to) + ab3 * rmin(R(0), tv))) / ab1 * g.area[i];
  r_plus[c] = rmax(R(0), rmin(R(1), q_plus / rmax(s_plus, thshld)));
  r_mnus[c] = rmax(R(0), rmin(R(1), q_mnus / rmax(s_mnus, thshld)));
}

// trcadv3 (trcadv_compute.F90:270-309)
template <typename R>
__global__ void __launch_bounds__(kBlock) k_trcadv3(Grid<R> g, Strides s, const StepParams* __restrict__ sp, int t0,
    R* __restrict__ trc_tdcy, const R* __restrict__ trl_tdcy, R* __restrict__ trcdp, R* __restrict__ tracr,
    const R* __restrict__ delp, const R* __restrict__ antiflx, const R* __restrict__ r_mnus,
    const R* __restrict__ r_plus, const R* __restrict__ trmin, const R* __restrict__ trmax, size_t sc_stride) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const int tz = blockIdx.z, t = t0 + tz;
  const size_t NL = (size_t)N * L;
  delp += m * s.cell;
  trc_tdcy += m * s.trab + (size_t)t * 3 * NL;
  trl_tdcy += m * s.trab + (size_t)t * 3 * NL;
  trcdp += m * s.tr + (size_t)t * NL;
  tracr += m * s.tr + (size_t)t * NL;
  const size_t so = (m * gridDim.z + tz) * sc_stride;
  antiflx += so * 6; trmin += so; trmax += so; r_plus += so; r_mnus += so;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11);
  const int np = g.nprox[i];
  const size_t c = (size_t)i * L + k;
  const R rp = r_plus[c], rm = r_mnus[c];
  R at = R(0);
  for (int e = 0; e < np; e++) {
    const int px = g.prox[i * 6 + e];
    R a = antiflx[((size_t)i * 6 + e) * L + k];
    if (a >= R(0)) a = a * rmin(rm, r_plus[(size_t)px * L + k]);
    else a = a * rmin(rp, r_mnus[(size_t)px * L + k]);
    at = at + a;
  }
  at = -at * g.rarea[i];
  const R tn = trl_tdcy[(size_t)nf * NL + c] + at;
  trc_tdcy[(size_t)nf * NL + c] = tn;
  const R td = trcdp[c] + ab1 * tn + ab2 * trc_tdcy[(size_t)of * NL + c] + ab3 * trc_tdcy[(size_t)vof * NL + c];
  trcdp[c] = td;
  tracr[c] = rmax(trmin[c], rmin(trmax[c], td / rmax(thshld, delp[c])));
}

// --------------------------------------------------------------------------
// del4prep (momtum_compute.F90:16-95) on u+grndspd, v; writes prepared fields.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_del4prep(Grid<R> g, Strides s, const R* __restrict__ u,
    const R* __restrict__ v, R* __restrict__ wu, R* __restrict__ wv) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L;
  const size_t m = blockIdx.y;
  u += m * s.cell; v += m * s.cell; wu += m * s.cell; wv += m * s.cell;
  const int np = g.nprox[i];
  R au = R(0), av = R(0);
  for (int e = 0; e < np; e++) {
    const int ipx = g.prox[i * 6 + e];
    const R* cs = g.cs + (i * 6 + e) * 4;
    const R* sn = g.sn + (i * 6 + e) * 4;
    const R ux = u[(size_t)ipx * L + k] + g.grndspd[ipx], vx = v[(size_t)ipx * L + k];
    const R uxy2 = cs[1] * ux + sn[1] * vx;
    const R vxy2 = -sn[1] * ux + cs[1] * vx;
    au = au + cs[0] * uxy2 - sn[0] * vxy2;
    av = av + sn[0] * uxy2 + cs[0] * vxy2;
  }
  const R factor = g.biharw[k] / R(np);
  const size_t c = (size_t)i * L + k;
  wu[c] = (u[c] + g.grndspd[i]) - au * factor;
  wv[c] = v[c] - av * factor;
}

// dissip (momtum_compute.F90:149-208): thickness-weighted harmonic momentum
// fluxes across the edges, rotated back; increments du, dv. The work fields are
// u+grndspd, v (momtum.F90:99-106) or the del4prep output when wu != nullptr.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_dissip(Grid<R> g, Strides s, const R* __restrict__ u,
    const R* __restrict__ v, const R* __restrict__ wu, const R* __restrict__ wv, const R* __restrict__ delp,
    R* __restrict__ du, R* __restrict__ dv) {
  int i, k;
  if (!cell_level(g.N, g.L, i, k)) return;
  const int L = g.L;
  const size_t m = blockIdx.y;
  u += m * s.cell; v += m * s.cell; delp += m * s.cell; du += m * s.cell; dv += m * s.cell;
  const bool prep = wu != nullptr;
  if (prep) { wu += m * s.cell; wv += m * s.cell; }
  const R thshld = R(1.e-11), two = R(2);
  const size_t c = (size_t)i * L + k;
  const R ui = prep ? wu[c] : u[c] + g.grndspd[i];
  const R vi = prep ? wv[c] : v[c];
  const R dpi = rmax(delp[c], thshld);
  const R factor = g.rarea[i] / dpi;
  const R dfl = g.dfflen[k];
  const int np = g.nprox[i];
  R su = R(0), sv = R(0);
  for (int e = 0; e < np; e++) {
    const int ipx = g.prox[i * 6 + e];
    const R* cs = g.cs + (i * 6 + e) * 4;
    const R* sn = g.sn + (i * 6 + e) * 4;
    const size_t cx = (size_t)ipx * L + k;
    const R ux = prep ? wu[cx] : u[cx] + g.grndspd[ipx];
    const R vx = prep ? wv[cx] : v[cx];
    const R uxy1 = cs[0] * ui + sn[0] * vi, vxy1 = -sn[0] * ui + cs[0] * vi;
    const R uxy2 = cs[1] * ux + sn[1] * vx, vxy2 = -sn[1] * ux + cs[1] * vx;
    const R b = rmax(delp[cx], thshld);
    const R hf = dpi * b / (dpi + b);
    const R sl = g.sideln[i * 6 + e];
    const R ufx = (uxy2 - uxy1) * dfl * sl * two * hf;
    const R vfx = (vxy2 - vxy1) * dfl * sl * two * hf;
    const R uflux = cs[0] * ufx - sn[0] * vfx;
    const R vflux = sn[0] * ufx + cs[0] * vfx;
    su = su + uflux * factor;
    sv = sv + vflux * factor;
  }
  du[c] = su;
  dv[c] = sv;
}

// momtum1 (momtum_compute.F90:278-423, janjic=0) after adding the dissipation
// increments (momtum.F90:130-139); one warp per column so the Rayleigh damping
// of the top layers can read the updated top three levels.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_momtum1(Grid<R> g, Strides s, Knobs kn, const StepParams* __restrict__ sp,
    R* __restrict__ u, R* __restrict__ v, const R* __restrict__ du, const R* __restrict__ dv,
    const R* __restrict__ exner, R* __restrict__ relvor, const R* __restrict__ u_edg, const R* __restrict__ v_edg,
    const R* __restrict__ trc_edg, const R* __restrict__ mont_edg, const R* __restrict__ uvsq_edg,
    R* __restrict__ u_tndcy, R* __restrict__ v_tndcy, const float2* __restrict__ mpf, const R* __restrict__ tr0) {
  __shared__ R top[kBlock / 32][3][2];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int N = g.N, L = g.L, L1 = L + 1;
  if (warp >= N) return;
  const int i = warp;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  u += m * s.cell; v += m * s.cell; exner += m * s.intf; relvor += m * s.cell;
  u_edg += m * s.edge; v_edg += m * s.edge; trc_edg += m * s.tredg; mont_edg += m * s.edge;
  uvsq_edg += m * s.edge; u_tndcy += m * s.ab; v_tndcy += m * s.ab;
  const bool have_d = du != nullptr;
  if (have_d) { du += m * s.cell; dv += m * s.cell; }
  const bool split = mpf != nullptr;
  if (split) { mpf += m * s.cell; tr0 += m * s.cell; }
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const size_t NL = (size_t)N * L;
  const int np = g.nprox[i];
  const R rar = g.rarea[i], cor = g.corio[i];
  constexpr int kCh = kMaxL / 32;
  R un[kCh], vn[kCh];
#pragma unroll
  for (int ch = 0; ch < kCh; ch++) {
    const int k = ch * 32 + lane;
    un[ch] = R(0); vn[ch] = R(0);
    if (k < L) {
      const size_t c = (size_t)i * L + k;
      R uu = u[c], vv = v[c];
      if (have_d) { uu = uu + du[c]; vv = vv + dv[c]; }
      const R exm = R(0.5) * (exner[(size_t)i * L1 + k] + exner[(size_t)i * L1 + k + 1]);
      R pgfx = R(0), pgfy = R(0), rv = R(0);
      if (!split) {
        for (int e = 0; e < np; e++) {
          const R* svc = g.svc + (i * 6 + e) * 2;
          const R* sve = g.sve + (i * 6 + e) * 2;
          const size_t o = ((size_t)i * 6 + e) * L + k;
          const R mu = mont_edg[o] + uvsq_edg[o];
          const R th = trc_edg[o];
          pgfx = pgfx - mu * svc[1] + exm * th * svc[1];
          pgfy = pgfy + mu * svc[0] - exm * th * svc[0];
          rv = rv + (sve[0] * u_edg[o] + sve[1] * v_edg[o]);
        }
      } else {
        // FP32-mixed: the same line integrals with the cell values split off,
        // sum_e (M_e + K_e - exm th_e) s_e
        //   = sum_e (dM_e + K_e - exm dth_e) s_e + (M_c - exm th_c) sum_e s_e,
        // dM_e, dth_e the edge-minus-cell values (edgvar1's weights applied to
        // neighbour differences); the large cell term is formed in FP64.
        const int* pr = g.prox + i * 6;
        const R thc = tr0[(size_t)i * L + k];
        R dth[6];
#pragma unroll
        for (int j = 0; j < 6; j++) dth[j] = (j < np) ? tr0[(size_t)pr[j] * L + k] - thc : R(0);
        const R divby6 = R(1) / R(6);
        for (int e = 0; e < np; e++) {
          const R* svc = g.svc + (i * 6 + e) * 2;
          const R* sve = g.sve + (i * 6 + e) * 2;
          const size_t o = ((size_t)i * 6 + e) * L + k;
          const int et = e == 0 ? np - 1 : e - 1, el = e == np - 1 ? 0 : e + 1;
          R dte = R(0);
#pragma unroll
          for (int j = 0; j < 6; j++) {
            if (j == e) dte = dte + R(2) * dth[j];
            if (j == et || j == el) dte = dte + dth[j];
          }
          dte = dte * divby6;
          const R w = mont_edg[o] + uvsq_edg[o] - exm * dte;
          pgfx = pgfx - w * svc[1];
          pgfy = pgfy + w * svc[0];
          rv = rv + (sve[0] * u_edg[o] + sve[1] * v_edg[o]);
        }
        // Montgomery potential minus exner x theta, cancellation-free
        const float2 mp = mpf[(size_t)i * L + k];
        const FF2 cf = ff_add(FF2{mp.x, mp.y}, ff_neg(two_prod(float(exm), float(thc))));
        const R cell = R(cf.hi + cf.lo);
        pgfx = pgfx - cell * g.svsum[i * 2 + 1];
        pgfy = pgfy + cell * g.svsum[i * 2 + 0];
      }
      pgfx = pgfx * rar;
      pgfy = pgfy * rar;
      rv = rv * rar;
      relvor[c] = rv;
      const R uzeta = (cor + rv) * uu, vzeta = (cor + rv) * vv;
      const R ut = pgfx + vzeta, vt = pgfy - uzeta;
      u_tndcy[(size_t)nf * NL + c] = ut;
      v_tndcy[(size_t)nf * NL + c] = vt;
      uu = uu + ab1 * ut + ab2 * u_tndcy[(size_t)of * NL + c] + ab3 * u_tndcy[(size_t)vof * NL + c];
      vv = vv + ab1 * vt + ab2 * v_tndcy[(size_t)of * NL + c] + ab3 * v_tndcy[(size_t)vof * NL + c];
      un[ch] = uu;
      vn[ch] = vv;
      if (k >= L - 3) { top[wib][L - 1 - k][0] = uu; top[wib][L - 1 - k][1] = vv; }
    }
  }
  __syncwarp();
  const R q1 = top[wib][0][0] * top[wib][0][0] + top[wib][0][1] * top[wib][0][1];
  const R q2 = top[wib][1][0] * top[wib][1][0] + top[wib][1][1] * top[wib][1][1];
  const R q3 = top[wib][2][0] * top[wib][2][0] + top[wib][2][1] * top[wib][2][1];
  const R thr = R(kn.rlthresh);
  R qq = rmax(rmax(q1, q2), q3) / (thr * thr);
  const int ndamp = (int)(0.25 * L);
  const bool damp = qq > R(1);
  if (damp) qq = sqrt((qq - R(1)) * qq);
  const R dtf = R(sp->dt) / R(86400.), rl = R(kn.rleigh), rt = R(kn.rltaper);
#pragma unroll
  for (int ch = 0; ch < kCh; ch++) {
    const int k = ch * 32 + lane;
    if (k < L) {
      R uu = un[ch], vv = vn[ch];
      if (damp && k >= L - 1 - ndamp) {
        const R factor = R(1) - dtf * rl * qq * pow(R(2), rt * R(k + 1 - L));
        uu = uu * factor;
        vv = vv * factor;
      }
      u[(size_t)i * L + k] = uu;
      v[(size_t)i * L + k] = vv;
    }
  }
}

// abstart (abstart.F90:33-65) advanced on the device so a captured step graph
// can be replayed: its += 1, rotate the AB3 slots, set the weights.
__global__ void k_step_begin(StepParams* sp, int members) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= members || !sp[m].active) return;
  sp += m;
  StepParams p = *sp;
  p.its += 1;
  p.nf = (p.nf + 1) % 3;
  p.of = (p.of + 1) % 3;
  p.vof = (p.vof + 1) % 3;
  if (p.its == 1) { p.ab1 = p.dt; p.ab2 = 0.; p.ab3 = 0.; }
  if (p.its == 2) { p.ab1 = p.dt * 1.5; p.ab2 = -p.dt * .5; p.ab3 = 0.; }
  if (p.its == 3) { p.ab1 = p.dt * 23. / 12.; p.ab2 = -p.dt * 16. / 12.; p.ab3 = p.dt * 5. / 12.; }
  *sp = p;
}

// ---------------------------- launchers -----------------------------------

template <typename R>
void launch_edgvar1(const Launch& l, const Grid<R>& g, const Strides& s, int hi_order, const R* u,
                    const R* v, const R* delp, const R* pres, const R* montg, const R* tracr,
                    R* u_edg, R* v_edg, R* dp_edg, R* lp_edg, R* mont_edg, R* uvsq_edg, R* trc_edg,
                    const float2* mpf, R* thold) {
  dim3 grid(blocks_for((long long)g.N * g.L), l.members);
  FIM_KBEGIN(l, "k_edgvar1");
  k_edgvar1<R><<<grid, kBlock, 0, l.stream>>>(g, s, hi_order, u, v, delp, pres, montg, tracr, u_edg, v_edg,
                                               dp_edg, lp_edg, mont_edg, uvsq_edg, trc_edg, mpf, thold);
  FIM_KEND(l);
}

template <typename R>
void launch_edgvar3(const Launch& l, const Grid<R>& g, const Strides& s, const R* delp, const R* tracr,
                    R* dp_edg, R* trc_edg, int nfields) {
  dim3 grid(blocks_for((long long)g.N * g.L), l.members, nfields);
  FIM_KBEGIN(l, "k_edgvar3_own");
  k_edgvar3_own<R><<<grid, kBlock, 0, l.stream>>>(g, s, delp, tracr, dp_edg, trc_edg);
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_edgvar3_avg");
  k_edgvar3_avg<R><<<grid, kBlock, 0, l.stream>>>(g, s, dp_edg, trc_edg);
  FIM_KEND(l);
}

template <typename R>
void launch_cnuity(const Launch& l, const Grid<R>& g, const Strides& s, const CnuityScratch<R>& w, const R* u,
                   const R* v, const R* u_edg, const R* v_edg, const R* dp_edg, const R* lp_edg,
                   R* delp, R* pres, R* exner, R* dp_tndcy, R* dplo_tndcy, R* massfx, R* omega) {
  dim3 grid(blocks_for((long long)g.N * g.L), l.members);
  FIM_KBEGIN(l, "k_cnuity12");
  k_cnuity12<R><<<grid, kBlock, 0, l.stream>>>(g, s, l.sp, u_edg, v_edg, dp_edg, delp, massfx, dplo_tndcy,
                                                w.antifx, w.delp_lo, w.p_plus, w.p_mnus);
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_cnuity3");
  k_cnuity3<R><<<grid, kBlock, 0, l.stream>>>(g, s, l.sp, w.delp_lo, delp, dp_tndcy, w.p_plus, w.p_mnus,
                                               w.r_plus, w.r_mnus);
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_cnuity4");
  k_cnuity4<R><<<grid, kBlock, 0, l.stream>>>(g, s, l.sp, w.antifx, w.r_plus, w.r_mnus, massfx, dplo_tndcy,
                                               dp_tndcy, delp, l.flags);
  FIM_KEND(l);
  dim3 gw(blocks_for((long long)g.N * 32), l.members);
  FIM_KBEGIN(l, "k_cnuity5");
  k_cnuity5<R><<<gw, kBlock, 0, l.stream>>>(g, s, l.sp, pres, delp, exner, dp_tndcy, omega, lp_edg, u, v, 0);
  FIM_KEND(l);
}

template <typename R>
void launch_trcadv(const Launch& l, const Grid<R>& g, const Strides& s, const TrcadvScratch<R>& w,
                   const R* trc_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx,
                   const R* delp) {
  const size_t scs = (size_t)g.N * g.L;
  for (int t0 = 0; t0 < g.T; t0 += w.tchunk) {
    const int nt = (g.T - t0 < w.tchunk) ? g.T - t0 : w.tchunk;
    dim3 grid(blocks_for((long long)g.N * g.L), l.members, nt);
    FIM_KBEGIN(l, "k_trcadv1");
    k_trcadv1<R><<<grid, kBlock, 0, l.stream>>>(g, s, l.sp, t0, massfx, trc_edg, tracr, trcdp, trl_tdcy, delp,
                                                 w.antiflx, w.trmin, w.trmax, w.trcr_lo, scs);
    FIM_KEND(l);
    FIM_KBEGIN(l, "k_trcadv2");
    k_trcadv2<R><<<grid, kBlock, 0, l.stream>>>(g, s, l.sp, t0, trc_tdcy, delp, w.antiflx, w.trmin, w.trmax,
                                                 w.trcr_lo, w.r_plus, w.r_mnus, scs);
    FIM_KEND(l);
    FIM_KBEGIN(l, "k_trcadv3");
    k_trcadv3<R><<<grid, kBlock, 0, l.stream>>>(g, s, l.sp, t0, trc_tdcy, trl_tdcy, trcdp, tracr, delp,
                                                 w.antiflx, w.r_mnus, w.r_plus, w.trmin, w.trmax, scs);
    FIM_KEND(l);
  }
}

template <typename R>
void launch_momtum(const Launch& l, const Grid<R>& g, const Strides& s, const Knobs& kn, const MomtumScratch<R>& w,
                   R* u, R* v, const R* exner, R* relvor, const R* u_edg, const R* v_edg,
                   const R* trc_edg, const R* mont_edg, const R* uvsq_edg, R* u_tndcy, R* v_tndcy,
                   const R* dp3d, const float2* mpf, const R* tr0) {
  dim3 grid(blocks_for((long long)g.N * g.L), l.members);
  const R* du = nullptr;
  const R* dv = nullptr;
  if (kn.dfflen_max > 0.) {
    const R* wu = nullptr;
    const R* wv = nullptr;
    if (kn.biharm) {
      FIM_KBEGIN(l, "k_del4prep");
      k_del4prep<R><<<grid, kBlock, 0, l.stream>>>(g, s, u, v, w.wu, w.wv);
      FIM_KEND(l);
      wu = w.wu;
      wv = w.wv;
    }
    FIM_KBEGIN(l, "k_dissip");
    k_dissip<R><<<grid, kBlock, 0, l.stream>>>(g, s, u, v, wu, wv, dp3d, w.du, w.dv);
    FIM_KEND(l);
    du = w.du;
    dv = w.dv;
  }
  dim3 gw(blocks_for((long long)g.N * 32), l.members);
  FIM_KBEGIN(l, "k_momtum1");
  k_momtum1<R><<<gw, kBlock, 0, l.stream>>>(g, s, kn, l.sp, u, v, du, dv, exner, relvor, u_edg, v_edg, trc_edg,
                                             mont_edg, uvsq_edg, u_tndcy, v_tndcy, mpf, tr0);
  FIM_KEND(l);
}

void launch_step_begin(const Launch& l, StepParams* sp) {
  FIM_KBEGIN(l, "k_step_begin");
  k_step_begin<<<(l.members + 31) / 32, 32, 0, l.stream>>>(sp, l.members);
  FIM_KEND(l);
}

#define INSTANTIATE(R)                                                                                          \
  template void launch_edgvar1<R>(const Launch&, const Grid<R>&, const Strides&, int, const R*, const R*,      \
                                  const R*, const R*, const R*, const R*, R*, R*, R*, R*, R*, R*, R*,          \
                                  const float2*, R*);                                                         \
  template void launch_edgvar3<R>(const Launch&, const Grid<R>&, const Strides&, const R*, const R*, R*, R*,  \
                                  int);                                                                      \
  template void launch_cnuity<R>(const Launch&, const Grid<R>&, const Strides&, const CnuityScratch<R>&,      \
                                 const R*, const R*, const R*, const R*, const R*, const R*, R*, R*, R*, R*,  \
                                 R*, R*, R*);                                                                 \
  template void launch_massadv<R>(const Launch&, const Grid<R>&, const Strides&, const CnuityScratch<R>&,     \
                                  const R*, const R*, const R*, const R*, R*, const R*, R*, R*, R*, R*, R*,   \
                                  R*);                                                                       \
  template void launch_trcadv<R>(const Launch&, const Grid<R>&, const Strides&, const TrcadvScratch<R>&,      \
                                 const R*, R*, R*, R*, R*, const R*, const R*);                               \
  template void launch_momtum<R>(const Launch&, const Grid<R>&, const Strides&, const Knobs&,                 \
                                 const MomtumScratch<R>&, R*, R*, const R*, R*, const R*, const R*, const R*, \
                                 const R*, const R*, R*, R*, const R*, const float2*, const R*);
INSTANTIATE(float)
INSTANTIATE(double)

}  // namespace fim
