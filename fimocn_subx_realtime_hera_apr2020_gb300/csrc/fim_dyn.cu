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

// |(a, b)|: IEEE sqrt in FP64; in the FP32-mixed build x * rsqrt(x), a few
// ulp from the rounded root and about a third of its instructions (edgvar1
// forms 30 magnitudes a level)
template <typename R>
__device__ __forceinline__ R vmag(R a, R b) { return sqrt(a * a + b * b); }
template <>
__device__ __forceinline__ float vmag<float>(float a, float b) {
  const float x = a * a + b * b;
  return x > 0.f ? x * rsqrtf(x) : 0.f;
}

// --------------------------------------------------------------------------
// edgvar1 (edgvar1.F90:156-511, eqwgt=.true., janjic=0): rotate u,v of the
// cell, the cell across the edge and the cells across the two adjacent edges
// into the edge frame, equal-weight interpolate with magnitude correction;
// mid-layer pressure, Montgomery potential, kinetic energy and tracer 1 (all
// tracers and dp when hi_order == 0) on the cell's own edges.
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock) k_edgvar1(Grid<R> g, Strides s, int hi_order,
    const R* __restrict__ u, const R* __restrict__ v, const R* __restrict__ delp,
    const R* __restrict__ pres, const R* __restrict__ montg, const R* __restrict__ tracr,
    R* __restrict__ u_edg, R* __restrict__ v_edg, R* __restrict__ dp_edg, R* __restrict__ lp_edg,
    R* __restrict__ mont_edg, R* __restrict__ uvsq_edg, R* __restrict__ trc_edg, const float2* __restrict__ mpf,
    R* __restrict__ thold) {
  int i, k;
  if (!cell_levels<VK>(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N, L1 = L + 1;
  const size_t m = blockIdx.y;
  if (mpf) mpf += m * s.cell;
  const size_t c = (size_t)i * L + k;
  if (thold) {
    // the potential temperature of this step's edge values, for momtum1
    R th[VK];
    ldv<VK>(tracr + m * s.tr + c, th);
    stv<VK>(thold + m * s.cell + c, th);
  }
  u += m * s.cell; v += m * s.cell; delp += m * s.cell; pres += m * s.intf;
  montg += m * s.cell; tracr += m * s.tr;
  u_edg += m * s.edge; v_edg += m * s.edge; dp_edg += m * s.edge; lp_edg += m * s.edge;
  mont_edg += m * s.edge; uvsq_edg += m * s.edge; trc_edg += m * s.tredg;
  const R divby6 = R(1) / R(6), eps = R(0.001), two = R(2), half = R(0.5);
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  R u1[VK], v1[VK], p1a[VK], p1b[VK], m1[VK];
  ldv<VK>(u + c, u1);
  ldv<VK>(v + c, v1);
  ldv<VK>(montg + c, m1);
  FOR_V { p1a[j] = pres[(size_t)i * L1 + k + j]; p1b[j] = pres[(size_t)i * L1 + k + j + 1]; }
  for (int e = 0; e < np; e++) {
    const int i2 = pr[e], i3t = pr[e == 0 ? np - 1 : e - 1], i3l = pr[e == np - 1 ? 0 : e + 1];
    const R* cs = g.cs + (i * 6 + e) * 4;
    const R* sn = g.sn + (i * 6 + e) * 4;
    R ut[VK], vt[VK], u2[VK], v2[VK], ul[VK], vl[VK];
    ldv<VK>(u + (size_t)i3t * L + k, ut);
    ldv<VK>(v + (size_t)i3t * L + k, vt);
    ldv<VK>(u + (size_t)i2 * L + k, u2);
    ldv<VK>(v + (size_t)i2 * L + k, v2);
    ldv<VK>(u + (size_t)i3l * L + k, ul);
    ldv<VK>(v + (size_t)i3l * L + k, vl);
    R ue[VK], ve[VK], lp[VK], mo[VK], uv[VK];
    FOR_V {
      const R u3trl = cs[2] * ut[j] + sn[2] * vt[j], v3trl = -sn[2] * ut[j] + cs[2] * vt[j];
      const R u1ldg = cs[0] * u1[j] + sn[0] * v1[j], v1ldg = -sn[0] * u1[j] + cs[0] * v1[j];
      const R u2ldg = cs[1] * u2[j] + sn[1] * v2[j], v2ldg = -sn[1] * u2[j] + cs[1] * v2[j];
      const R u3ldg = cs[3] * ul[j] + sn[3] * vl[j], v3ldg = -sn[3] * ul[j] + cs[3] * vl[j];
      R uu = (two * (u1ldg + u2ldg) + u3trl + u3ldg) * divby6;
      R vv = (two * (v1ldg + v2ldg) + v3trl + v3ldg) * divby6;
      const R m_1ldg = vmag(u1ldg, v1ldg);
      const R m_2ldg = vmag(u2ldg, v2ldg);
      const R m_3trl = vmag(u3trl, v3trl);
      const R m_3ldg = vmag(u3ldg, v3ldg);
      const R m_1 = vmag(uu, vv);
      const R m_2 = (two * (m_1ldg + m_2ldg) + m_3trl + m_3ldg) * divby6;
      const R q = fdiv(m_2, rmax(eps, m_1));  // one division for both components
      uu = uu * q;
      vv = vv * q;
      ue[j] = uu;
      ve[j] = vv;
      uv[j] = half * (uu * uu + vv * vv);
      const size_t kk = (size_t)k + j;
      lp[j] = (p1a[j] + p1b[j] + pres[(size_t)i2 * L1 + kk] + pres[(size_t)i2 * L1 + kk + 1] +
               half * (pres[(size_t)i3t * L1 + kk] + pres[(size_t)i3t * L1 + kk + 1] +
                       pres[(size_t)i3l * L1 + kk] + pres[(size_t)i3l * L1 + kk + 1])) * divby6;
    }
    const size_t o = ((size_t)i * 6 + e) * L + k;
    stv<VK>(u_edg + o, ue);
    stv<VK>(v_edg + o, ve);
    stv<VK>(lp_edg + o, lp);
    stv<VK>(uvsq_edg + o, uv);
    if (!hi_order) {
      R d1[VK], d2[VK], dt[VK], dl[VK], de[VK];
      ldv<VK>(delp + c, d1);
      ldv<VK>(delp + (size_t)i2 * L + k, d2);
      ldv<VK>(delp + (size_t)i3t * L + k, dt);
      ldv<VK>(delp + (size_t)i3l * L + k, dl);
      FOR_V de[j] = (two * (d1[j] + d2[j]) + dt[j] + dl[j]) * divby6;
      stv<VK>(dp_edg + o, de);
    }
    if (mpf) {
      // edge minus cell value from float-float differences (no cancellation)
      FOR_V {
        const size_t kk = (size_t)k + j;
        const float2 mc = mpf[(size_t)i * L + kk];
        mo[j] = R((2.f * ff_diff(mpf[(size_t)i2 * L + kk], mc) + ff_diff(mpf[(size_t)i3t * L + kk], mc) +
                   ff_diff(mpf[(size_t)i3l * L + kk], mc)) * (1.f / 6.f));
      }
    } else {
      R m2[VK], mt[VK], ml[VK];
      ldv<VK>(montg + (size_t)i2 * L + k, m2);
      ldv<VK>(montg + (size_t)i3t * L + k, mt);
      ldv<VK>(montg + (size_t)i3l * L + k, ml);
      FOR_V mo[j] = (two * (m1[j] + m2[j]) + mt[j] + ml[j]) * divby6;
    }
    stv<VK>(mont_edg + o, mo);
  }
  const int ntr = hi_order ? 1 : g.T;
  for (int t = 0; t < ntr; t++) {
    const R* tr = tracr + (size_t)t * N * L;
    R* te = trc_edg + (size_t)t * N * 6 * L;
    R z[VK], t1[VK];
    FOR_V z[j] = R(0);
    stv<VK>(te + ((size_t)i * 6 + 5) * L + k, z);
    ldv<VK>(tr + c, t1);
    for (int e = 0; e < np; e++) {
      const int i2 = pr[e], i3t = pr[e == 0 ? np - 1 : e - 1], i3l = pr[e == np - 1 ? 0 : e + 1];
      R t2[VK], tt[VK], tl[VK], out[VK];
      ldv<VK>(tr + (size_t)i2 * L + k, t2);
      ldv<VK>(tr + (size_t)i3t * L + k, tt);
      ldv<VK>(tr + (size_t)i3l * L + k, tl);
      FOR_V out[j] = (two * (t1[j] + t2[j]) + tt[j] + tl[j]) * divby6;
      stv<VK>(te + ((size_t)i * 6 + e) * L + k, out);
    }
  }
}

// --------------------------------------------------------------------------
// edgvar2 (edgvar2.F90:24-319, hiOrderUVComp; the MORE_VARS block is compiled
// out in the reference): the edge wind is rescaled to the mean of the speeds
// at the edge's two corners seen from the three cells around each corner,
// each a cell's speed plus its speed-gradient projected on the corner.
//  k_edgvar2_grad: per cell-level the speed |u| and the gradient of the edge
//                  speeds (gradient(), edgvar2.F90:231-258) -> w[0..2]
//  k_edgvar2:      per cell-level and edge, the corner speeds of the cell, the
//                  neighbour across the edge and the neighbours across the
//                  adjacent edges, the ratio to |u_edg| (1 below 1e-5), and
//                  uvsq_edg of the rescaled wind.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_edgvar2_grad(Grid<R> g, Strides s, const R* __restrict__ u,
    const R* __restrict__ v, const R* __restrict__ u_edg, const R* __restrict__ v_edg, R* __restrict__ w) {
  int i, k;
  if (!cell_levels<1>(g.N, g.L, i, k)) return;
  const int L = g.L;
  const size_t m = blockIdx.y, NL = (size_t)g.N * L;
  u += m * s.cell; v += m * s.cell; u_edg += m * s.edge; v_edg += m * s.edge; w += m * 3 * NL;
  const size_t c = (size_t)i * L + k;
  const int np = g.nprox[i];
  R g1 = R(0), g2 = R(0);
  for (int e = 0; e < np; e++) {
    const size_t o = ((size_t)i * 6 + e) * L + k;
    const R sp = sqrt(u_edg[o] * u_edg[o] + v_edg[o] * v_edg[o]);
    g1 = g1 + sp * g.svc[(i * 6 + e) * 2 + 1];
    g2 = g2 - sp * g.svc[(i * 6 + e) * 2 + 0];
  }
  const R rar = g.rarea[i];
  w[c] = sqrt(u[c] * u[c] + v[c] * v[c]);
  w[NL + c] = g1 * rar;
  w[2 * NL + c] = g2 * rar;
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_edgvar2(Grid<R> g, Strides s, const R* __restrict__ w,
    R* __restrict__ u_edg, R* __restrict__ v_edg, R* __restrict__ uvsq_edg) {
  int i, k;
  if (!cell_levels<1>(g.N, g.L, i, k)) return;
  const int L = g.L;
  const size_t m = blockIdx.y, NL = (size_t)g.N * L;
  u_edg += m * s.edge; v_edg += m * s.edge; uvsq_edg += m * s.edge; w += m * 3 * NL;
  const R divby6 = R(1) / R(6), eps = R(0.00001);
  const int np = g.nprox[i];
  // corner q of cell x: its speed plus 0.5 * (grad . corner_xy(q))
  auto corner = [&](int x, int q) -> R {
    const size_t cx = (size_t)x * L + k;
    const R gc = R(0.5) * (w[NL + cx] * g.cxy[(x * 2 + 0) * 6 + q] + w[2 * NL + cx] * g.cxy[(x * 2 + 1) * 6 + q]);
    return w[cx] + gc;
  };
  for (int e = 0; e < np; e++) {
    const int nba = g.prox[i * 6 + e], nbaedg = g.proxs[i * 6 + e];
    const int em1 = (e - 1 + np) % np, ep1 = (e + 1) % np;
    const int nbm1 = g.prox[i * 6 + em1], nbp1 = g.prox[i * 6 + ep1];
    const R uv1conr1 = corner(i, e);
    const R uv2conr1 = corner(nba, (nbaedg + 1) % g.nprox[nba]);
    const R uv3conr1 = corner(nbm1, g.proxs[i * 6 + em1]);
    const R uv1conr2 = corner(i, ep1);
    const R uv2conr2 = corner(nba, nbaedg);
    const R uv3conr2 = corner(nbp1, (g.proxs[i * 6 + ep1] + 1) % g.nprox[nbp1]);
    const size_t o = ((size_t)i * 6 + e) * L + k;
    R ue = u_edg[o], ve = v_edg[o];
    const R uvm1 = sqrt(ue * ue + ve * ve);
    const R uvm2 = (uv1conr1 + uv2conr1 + uv3conr1 + uv1conr2 + uv2conr2 + uv3conr2) * divby6;
    const R r_m = uvm1 < eps ? R(1) : uvm2 / uvm1;
    ue = ue * r_m;
    ve = ve * r_m;
    u_edg[o] = ue;
    v_edg[o] = ve;
    uvsq_edg[o] = R(.5) * (ue * ue + ve * ve);
  }
}

template <typename R>
void launch_edgvar2(const Launch& l, const Grid<R>& g, const Strides& s, const R* u, const R* v, R* u_edg,
                    R* v_edg, R* uvsq_edg, R* w) {
  dim3 grid(blocks_for((long long)g.N * g.L), l.members);
  FIM_KBEGIN(l, "k_edgvar2_grad");
  k_edgvar2_grad<R><<<grid, kBlock, 0, l.stream>>>(g, s, u, v, u_edg, v_edg, w);
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_edgvar2");
  k_edgvar2<R><<<grid, kBlock, 0, l.stream>>>(g, s, w, u_edg, v_edg, uvsq_edg);
  FIM_KEND(l);
}

// --------------------------------------------------------------------------
// edgvar3 loop 1 with edgvalEval (edgvar3.F90:66-94,136-163): least-squares
// (hfcoef) reconstruction of dp (field 0) and tracers 2..ntra (field t) on the
// cell's own edges; pentagons store 0 in the sixth slot.
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock) k_edgvar3_own(Grid<R> g, Strides s,
    const R* __restrict__ delp, const R* __restrict__ tracr, R* __restrict__ dp_edg, R* __restrict__ trc_edg) {
  int i, k;
  if (!cell_levels<VK>(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  const int f = blockIdx.z;
  const R* src = (f == 0) ? delp + m * s.cell : tracr + m * s.tr + (size_t)f * N * L;
  R* dst = (f == 0) ? dp_edg + m * s.edge : trc_edg + m * s.tredg + (size_t)f * N * 6 * L;
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  R bc[VK];
  ldv<VK>(src + (size_t)i * L + k, bc);
  // branch-free gathers over the six prox slots (all valid cells); a
  // pentagon's slot 5 is dropped by selects
  R d[6][VK];
#pragma unroll
  for (int e = 0; e < 6; e++) {
    ldv<VK>(src + (size_t)pr[e] * L + k, d[e]);
    FOR_V d[e][j] = e < np ? d[e][j] - bc[j] : R(0);
  }
  const R* hf = g.hfcoef + (size_t)i * 36;
#pragma unroll
  for (int ie = 0; ie < 6; ie++) {
    R val[VK];
    FOR_V val[j] = bc[j];
#pragma unroll
    for (int e = 0; e < 6; e++) {
      const R h = hf[ie * 6 + e];
      FOR_V val[j] = e < np ? val[j] + d[e][j] * h : val[j];
    }
    FOR_V val[j] = ie < np ? val[j] : R(0);
    stv<VK>(dst + ((size_t)i * 6 + ie) * L + k, val);
  }
}

// edgvar3 loop 2 (edgvar3.F90:110-132): the lower-numbered cell of each pair
// stores the two-sided average in both slots, as the reference does; each slot
// has exactly one writer, which is also its only reader.
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock) k_edgvar3_avg(Grid<R> g, Strides s, R* __restrict__ dp_edg,
                                                       R* __restrict__ trc_edg) {
  int i, k;
  if (!cell_levels<VK>(g.N, g.L, i, k)) return;
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
      R xa[VK], xb[VK], w[VK];
      ldv<VK>(x + a, xa);
      ldv<VK>(x + b, xb);
      FOR_V w[j] = R(0.5) * (xa[j] + xb[j]);
      stv<VK>(x + a, w);
      stv<VK>(x + b, w);
    }
  }
}

// --------------------------------------------------------------------------
// cnuity1 + cnuity2 (cnuity_compute.F90:41-146): normal velocity on the cell's
// edge and on the neighbour's copy of it, donor-cell mass flux, antidiffusive
// flux, low-order tendency and low-order thickness; also the Zalesak sums
// P+/P- of cnuity3 (cnuity_compute.F90:186-194), which only need own edges.
// The bodies of cnuity12/3/4 take the (virtual) block index, so the persistent
// variant below runs the same code; their pointers carry no __restrict__ (the
// persistent variant reads in one stage what another block wrote in the
// stage before, which read-only loads must not do).
template <typename R, int VK>
__device__ __forceinline__ void cnuity12_body(int bx, int by, const Grid<R>& g, const Strides& s,
    const StepParams* sp, const R* u_edg, const R* v_edg, const R* dp_edg, const R* delp, R* massfx,
    R* dplo_tndcy, R* antifx, R* delp_lo, R* p_plus, R* p_mnus) {
  int i, k;
  if (!cell_levels_at<VK>(g.N, g.L, bx, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = by;
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
  R dpi[VK], sum[VK], pp[VK], pm[VK];
  ldv<VK>(delp + (size_t)i * L + k, dpi);
  FOR_V { sum[j] = R(0); pp[j] = R(0); pm[j] = R(0); }
  if (np < 6) {
    R z[VK];
    FOR_V z[j] = R(0);
    stv<VK>(mfn + ((size_t)i * 6 + 5) * L + k, z);
    stv<VK>(antifx + ((size_t)i * 6 + 5) * L + k, z);
  }
  // branch-free over the six slots: a pentagon's slot 5 reads valid rows
  // (mirror edge 0) and is neither accumulated nor stored
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const bool live = e < np;
    const int ipx = g.prox[i * 6 + e], edx = live ? g.proxs[i * 6 + e] : 0;
    const R* sv = g.sve + (i * 6 + e) * 2;
    const R* sx = g.sve + (ipx * 6 + edx) * 2;
    const size_t o = ((size_t)i * 6 + e) * L + k, ox = ((size_t)ipx * 6 + edx) * L + k;
    R ue[VK], ve[VK], ux[VK], vx_[VK], de[VK], dx[VK], mf[VK], an[VK];
    ldv<VK>(u_edg + o, ue);
    ldv<VK>(v_edg + o, ve);
    ldv<VK>(u_edg + ox, ux);
    ldv<VK>(v_edg + ox, vx_);
    // edgvar3's two-sided average 0.5*(own + neighbour's own), formed here
    // (exact also when dp_edg already holds it: 0.5*(w + w) == w)
    R dm[VK];
    ldv<VK>(dp_edg + o, de);
    ldv<VK>(dp_edg + ox, dm);
    FOR_V de[j] = half * (de[j] + dm[j]);
    ldv<VK>(delp + (size_t)ipx * L + k, dx);
    FOR_V {
      const R vn = sv[1] * ue[j] - sv[0] * ve[j];
      const R vx = sx[1] * ux[j] - sx[0] * vx_[j];
      const R flxhi = vn * de[j];
      mf[j] = half * ((vn + rabs(vn)) * dpi[j] - (vx + rabs(vx)) * dx[j]);
      const R a = flxhi - mf[j];
      an[j] = a;
      sum[j] = live ? sum[j] + mf[j] : sum[j];
      if (live && a <= R(0)) pp[j] = pp[j] - a;
      else if (live) pm[j] = pm[j] + a;
    }
    if (live) {
      stv<VK>(mfn + o, mf);
      stv<VK>(antifx + o, an);
    }
  }
  const size_t c = (size_t)i * L + k;
  const R rar = g.rarea[i];
  R tn[VK], to[VK], tv[VK], lo[VK];
  FOR_V tn[j] = -sum[j] * rar;
  stv<VK>(dplo_tndcy + (size_t)nf * N * L + c, tn);
  ldv<VK>(dplo_tndcy + (size_t)of * N * L + c, to);
  ldv<VK>(dplo_tndcy + (size_t)vof * N * L + c, tv);
  FOR_V lo[j] = dpi[j] + ab1 * tn[j] + ab2 * to[j] + ab3 * tv[j];
  stv<VK>(delp_lo + c, lo);
  stv<VK>(p_plus + c, pp);
  stv<VK>(p_mnus + c, pm);
}
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock) k_cnuity12(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ u_edg, const R* __restrict__ v_edg, const R* __restrict__ dp_edg,
    const R* __restrict__ delp, R* __restrict__ massfx, R* __restrict__ dplo_tndcy, R* __restrict__ antifx,
    R* __restrict__ delp_lo, R* __restrict__ p_plus, R* __restrict__ p_mnus) {
  cnuity12_body<R, VK>(blockIdx.x, blockIdx.y, g, s, sp, u_edg, v_edg, dp_edg, delp, massfx, dplo_tndcy, antifx,
                       delp_lo, p_plus, p_mnus);
}

// cnuity3 (cnuity_compute.F90:206-252): 1-ring max/min of old and low-order
// thickness, Zalesak Q+/Q- and the limiters R+/R-.
template <typename R, int VK>
__device__ __forceinline__ void cnuity3_body(int bx, int by, const Grid<R>& g, const Strides& s,
    const StepParams* sp, const R* delp_lo, const R* delp, const R* dp_tndcy, const R* p_plus, const R* p_mnus,
    R* r_plus, R* r_mnus) {
  int i, k;
  if (!cell_levels_at<VK>(g.N, g.L, bx, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = by;
  sp += m;
  if (!sp->active) return;
  delp_lo += m * s.cell; delp += m * s.cell; dp_tndcy += m * s.ab;
  p_plus += m * s.cell; p_mnus += m * s.cell; r_plus += m * s.cell; r_mnus += m * s.cell;
  const int of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R rab1 = R(1) / ab1;  // Q+/Q- divide by ab1: one reciprocal
  const R thshld = R(1.e-11);
  const size_t c = (size_t)i * L + k;
  const int* pr = g.prox + i * 6;
  R dlo[VK], dc[VK], mx[VK], mn[VK];
  ldv<VK>(delp_lo + c, dlo);
  ldv<VK>(delp + c, dc);
  FOR_V { mx[j] = rmax(dlo[j], dc[j]); mn[j] = rmin(dlo[j], dc[j]); }
#pragma unroll
  for (int e = 0; e < 6; e++) {
    R a[VK], b[VK];
    ldv<VK>(delp_lo + (size_t)pr[e] * L + k, a);
    ldv<VK>(delp + (size_t)pr[e] * L + k, b);
    FOR_V { mx[j] = rmax(mx[j], rmax(a[j], b[j])); mn[j] = rmin(mn[j], rmin(a[j], b[j])); }
  }
  R to[VK], tv[VK], pp[VK], pm[VK], rp[VK], rm[VK];
  ldv<VK>(dp_tndcy + (size_t)of * N * L + c, to);
  ldv<VK>(dp_tndcy + (size_t)vof * N * L + c, tv);
  ldv<VK>(p_plus + c, pp);
  ldv<VK>(p_mnus + c, pm);
  const R ar = g.area[i];
  FOR_V {
    const R dpmax = rmax(R(0), mx[j]), dpmin = rmax(R(0), mn[j]);
    const R q_plus = (dpmax - dlo[j] - (ab2 * rmin(R(0), to[j]) + ab3 * rmax(R(0), tv[j]))) * rab1 * ar;
    const R q_mnus = (dlo[j] - dpmin + (ab2 * rmax(R(0), to[j]) + ab3 * rmin(R(0), tv[j]))) * rab1 * ar;
    rp[j] = rmax(R(0), rmin(R(1), fdiv(q_plus, rmax(pp[j], thshld))));
    rm[j] = rmax(R(0), rmin(R(1), fdiv(q_mnus, rmax(pm[j], thshld))));
  }
  stv<VK>(r_plus + c, rp);
  stv<VK>(r_mnus + c, rm);
}
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock) k_cnuity3(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ delp_lo, const R* __restrict__ delp, const R* __restrict__ dp_tndcy,
    const R* __restrict__ p_plus, const R* __restrict__ p_mnus, R* __restrict__ r_plus, R* __restrict__ r_mnus) {
  cnuity3_body<R, VK>(blockIdx.x, blockIdx.y, g, s, sp, delp_lo, delp, dp_tndcy, p_plus, p_mnus, r_plus, r_mnus);
}

// cnuity4 (cnuity_compute.F90:291-369): clip the antidiffusive flux with the
// own and neighbour limiters, total mass flux, AB3 thickness update.
template <typename R, int VK>
__device__ __forceinline__ void cnuity4_body(int bx, int by, const Grid<R>& g, const Strides& s,
    const StepParams* sp, const R* antifx, const R* r_plus, const R* r_mnus, R* massfx, const R* dplo_tndcy,
    R* dp_tndcy, R* delp, int* flags) {
  int i, k;
  if (!cell_levels_at<VK>(g.N, g.L, bx, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = by;
  sp += m;
  if (!sp->active) return;
  antifx += m * s.edge; r_plus += m * s.cell; r_mnus += m * s.cell; massfx += m * s.mf;
  dplo_tndcy += m * s.ab; dp_tndcy += m * s.ab; delp += m * s.cell;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  R* mfn = massfx + (size_t)nf * N * 6 * L;
  const size_t c = (size_t)i * L + k;
  R rp[VK], rm[VK], at[VK];
  ldv<VK>(r_plus + c, rp);
  ldv<VK>(r_mnus + c, rm);
  FOR_V at[j] = R(0);
  const int np = g.nprox[i];
  for (int e = 0; e < np; e++) {
    const int px = g.prox[i * 6 + e];
    const size_t o = ((size_t)i * 6 + e) * L + k;
    R a[VK], mf[VK], rpx[VK], rmx[VK];
    ldv<VK>(antifx + o, a);
    ldv<VK>(mfn + o, mf);
    ldv<VK>(r_plus + (size_t)px * L + k, rpx);
    ldv<VK>(r_mnus + (size_t)px * L + k, rmx);
    FOR_V {
      const R clip = (a[j] >= R(0)) ? rmin(rm[j], rpx[j]) : rmin(rp[j], rmx[j]);
      const R ac = a[j] * clip;
      mf[j] = mf[j] + ac;
      at[j] = at[j] + ac;
    }
    stv<VK>(mfn + o, mf);
  }
  const R rar = g.rarea[i];
  R tl[VK], tn[VK], to[VK], tv[VK], dn[VK];
  ldv<VK>(dplo_tndcy + (size_t)nf * N * L + c, tl);
  FOR_V tn[j] = tl[j] + (-at[j] * rar);
  stv<VK>(dp_tndcy + (size_t)nf * N * L + c, tn);
  ldv<VK>(dp_tndcy + (size_t)of * N * L + c, to);
  ldv<VK>(dp_tndcy + (size_t)vof * N * L + c, tv);
  ldv<VK>(delp + c, dn);
  bool bad = false;
  FOR_V {
    dn[j] = dn[j] + ab1 * tn[j] + ab2 * to[j] + ab3 * tv[j];
    bad = bad || !(dn[j] > R(0));
  }
  stv<VK>(delp + c, dn);
  if (bad) atomicOr(flags + m, kFlagBadDp);
}
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock) k_cnuity4(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ antifx, const R* __restrict__ r_plus, const R* __restrict__ r_mnus,
    R* __restrict__ massfx, const R* __restrict__ dplo_tndcy, R* __restrict__ dp_tndcy, R* __restrict__ delp,
    int* __restrict__ flags) {
  cnuity4_body<R, VK>(blockIdx.x, blockIdx.y, g, s, sp, antifx, r_plus, r_mnus, massfx, dplo_tndcy, dp_tndcy, delp,
                      flags);
}

// ---- persistent variant of cnuity1..4 ---------------------------------------
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of a cooperative launch.  Every block adds one to *ctr
// and waits until it reaches target; the wait gives up after limit_ns (and
// after 2^22 polls whatever the timer says), sets kFlagTimeout in *flags and
// returns false, so the kernel ends and the host reads FIM_ETIMEDOUT.
__device__ bool coop_barrier(unsigned* ctr, unsigned target, unsigned long long limit_ns, int* flags) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctr, 1u);
    int good = 1;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0;; it++) {
      if (*(volatile unsigned*)ctr >= target) break;
      if (it >= (1u << 22) || global_ns() - t0 > limit_ns) {
        good = 0;
        break;
      }
      __nanosleep(64);
    }
    if (!good) atomicOr(flags, kFlagTimeout);
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// cnuity1..4 of every member in one cooperative launch: the blocks resident
// on the GPU walk the virtual blocks of each stage, with a grid barrier
// between the stages in place of kernel boundaries.  extra arrivals are added
// to each barrier's target (a barrier that can never complete: the test of
// the time limit).
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock) k_cnuity_coop(Grid<R> g, Strides s, const StepParams* sp, int members,
    const R* u_edg, const R* v_edg, const R* dp_edg, R* delp, R* massfx, R* dplo_tndcy, R* dp_tndcy, R* antifx,
    R* delp_lo, R* p_plus, R* p_mnus, R* r_plus, R* r_mnus, int* flags, unsigned* bar, unsigned extra,
    unsigned long long limit_ns) {
  const int nvb = (int)(((long long)g.N * (g.L / VK) + kBlock - 1) / kBlock);
  const int total = nvb * members;
  for (int w = blockIdx.x; w < total; w += gridDim.x)
    cnuity12_body<R, VK>(w % nvb, w / nvb, g, s, sp, u_edg, v_edg, dp_edg, delp, massfx, dplo_tndcy, antifx,
                         delp_lo, p_plus, p_mnus);
  if (!coop_barrier(bar, gridDim.x + extra, limit_ns, flags)) return;
  for (int w = blockIdx.x; w < total; w += gridDim.x)
    cnuity3_body<R, VK>(w % nvb, w / nvb, g, s, sp, delp_lo, delp, dp_tndcy, p_plus, p_mnus, r_plus, r_mnus);
  if (!coop_barrier(bar, 2 * gridDim.x + extra, limit_ns, flags)) return;
  for (int w = blockIdx.x; w < total; w += gridDim.x)
    cnuity4_body<R, VK>(w % nvb, w / nvb, g, s, sp, antifx, r_plus, r_mnus, massfx, dplo_tndcy, dp_tndcy, delp,
                        flags);
}

// cnuity5 (cnuity_compute.F90:408-445) for 32 columns per warp, 32 levels
// (top-down) at a time.  The layer thickness and pressure tendency of each
// level are formed with lane = level, one column at a time (128-byte rows),
// into a shared tile; the top-down pressure sum and the omega flux-convergence
// integral run with lane = column up the tile in the reference's order (FP64,
// or float-float in the FP32-mixed build); the Exner function and the
// v.grad(p) term are formed with lane = level again.
template <typename R>
constexpr int kC5Warps = sizeof(R) == 4 ? 4 : 2;
template <typename R>
__global__ void __launch_bounds__(32 * kC5Warps<R>) k_cnuity5(Grid<R> g, Strides s,
    const StepParams* __restrict__ sp, R* __restrict__ pres, R* __restrict__ delp, R* __restrict__ exner,
    const R* __restrict__ dp_tndcy, R* __restrict__ omega, const R* __restrict__ lp_edg, const R* __restrict__ u,
    const R* __restrict__ v, int ab3_delp) {
  __shared__ R tiles[kC5Warps<R>][2][32][33];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int N = g.N, L = g.L, L1 = L + 1;
  const int i0 = (blockIdx.x * kC5Warps<R> + wib) * 32;
  if (i0 >= N) return;
  const int ncol = N - i0 < 32 ? N - i0 : 32;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  pres += m * s.intf; delp += m * s.cell; exner += m * s.intf; dp_tndcy += m * s.ab;
  omega += m * s.cell; lp_edg += m * s.edge; u += m * s.cell; v += m * s.cell;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3), dt = R(sp->dt);
  const R cp = R(kCp), p1000 = R(kP1000), rdcp = R(kRd) / R(kCp);
  const size_t NL = (size_t)N * L;
  R (*tp)[33] = tiles[wib][0];  // thickness in, pressure out
  R (*tw)[33] = tiles[wib][1];  // layer pressure tendency in, omega's first terms out
  const bool live = lane < ncol;
  // the top-down sums of column i0 + lane
  FF2 pf{0.f, 0.f}, cf{0.f, 0.f};
  double pd = 0.0, cd = 0.0;
  if (live) {
    const R ptop = pres[(size_t)(i0 + lane) * L1 + L];
    pf = FF2{(float)ptop, 0.f};
    pd = (double)ptop;
  }
  for (int base = 0; base < L; base += 32) {
    const int j = base + lane;
    const bool act = j < L;
    const int k = L - 1 - j;
    const int nq = L - base < 32 ? L - base : 32;
#pragma unroll 4
    for (int r = 0; r < 32; r++)
      if (r < ncol && act) {
        const size_t c = (size_t)(i0 + r) * L + k;
        const R tnf = dp_tndcy[(size_t)nf * NL + c], tof = dp_tndcy[(size_t)of * NL + c],
                tvf = dp_tndcy[(size_t)vof * NL + c];
        R d;
        if (ab3_delp) {
          // massflux_newdepth's AB3 thickness update (massadv_compute.F90:85-91)
          R dn = delp[c] + ab1 * tnf + ab2 * tof + ab3 * tvf;
          dn = dn > R(0) ? dn : R(0);
          delp[c] = dn;
          d = dn;
        } else {
          d = delp[c];
        }
        tp[r][lane] = d;
        tw[r][lane] = (ab1 * tnf + ab2 * tof + ab3 * tvf) / dt;
      }
    __syncwarp();
    if (live) {
      for (int q = 0; q < nq; q++) {
        const R d = tp[lane][q], lyr = tw[lane][q];
        if constexpr (sizeof(R) == 4) {
          pf = ff_add(pf, FF2{d, 0.f});
          tp[lane][q] = pf.hi;
          // omega = (integral of the layers above) + half of this layer
          tw[lane][q] = R(cf.hi + cf.lo) + R(0.5) * lyr;
          cf = ff_add(cf, FF2{lyr, 0.f});
        } else {
          pd = pd + (double)d;
          tp[lane][q] = R(pd);
          tw[lane][q] = R(cd + 0.5 * (double)lyr);
          cd = cd + (double)lyr;
        }
      }
    }
    __syncwarp();
#pragma unroll 2
    for (int r = 0; r < 32; r++)
      if (r < ncol && act) {
        const int i = i0 + r;
        const size_t c = (size_t)i * L + k;
        const R pr = tp[r][lane];
        pres[(size_t)i * L1 + k] = pr;
        exner[(size_t)i * L1 + k] = cp * pow(pr / p1000, rdcp);
        // pressure gradient over the cell's edges (all six slots hold valid
        // rows; a pentagon's slot 5 is left out)
        const int np = g.nprox[i];
        R lp[6];
#pragma unroll
        for (int e = 0; e < 6; e++) lp[e] = lp_edg[((size_t)i * 6 + e) * L + k];
        R dpdx = R(0), dpdy = R(0);
#pragma unroll
        for (int e = 0; e < 6; e++)
          if (e < np) {
            const R* sv = g.svc + (i * 6 + e) * 2;
            dpdx = dpdx + lp[e] * sv[1];
            dpdy = dpdy - lp[e] * sv[0];
          }
        omega[c] = tw[r][lane] + (u[c] * dpdx + v[c] * dpdy) * g.rarea[i];
      }
    __syncwarp();
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
  dim3 gw((unsigned)((g.N + 32 * kC5Warps<R> - 1) / (32 * kC5Warps<R>)), l.members);
  FIM_KBEGIN(l, "k_cnuity5");
  k_cnuity5<R><<<gw, 32 * kC5Warps<R>, 0, l.stream>>>(g, s, l.sp, pres, delp, exner, dp_tndcy, omega, lp_edg, u,
                                                      v, 1);
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
  trcr_lo[c] = rmax(mn, rmin(mx, fdiv(trcdp_lo, rmax(thshld, delp[c]))));
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
  const R rab1 = R(1) / ab1;  // one reciprocal, as k_tr_lim
  const R q_plus = ((mx - lo) * dp - (ab2 * rmin(R(0), to) + ab3 * rmax(R(0), tv))) * rab1 * g.area[i];
  const R q_mnus = ((lo - mn) * dp + (ab2 * rmax(R(0), to) + ab3 * rmin(R(0), tv))) * rab1 * g.area[i];
  r_plus[c] = rmax(R(0), rmin(R(1), fdiv(q_plus, rmax(s_plus, thshld))));
  r_mnus[c] = rmax(R(0), rmin(R(1), fdiv(q_mnus, rmax(s_mnus, thshld))));
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
  tracr[c] = rmax(trmin[c], rmin(trmax[c], fdiv(td, rmax(thshld, delp[c]))));
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
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock) k_dissip(Grid<R> g, Strides s, const R* __restrict__ u,
    const R* __restrict__ v, const R* __restrict__ wu, const R* __restrict__ wv, const R* __restrict__ delp,
    R* __restrict__ du, R* __restrict__ dv) {
  int i, k;
  if (!cell_levels<VK>(g.N, g.L, i, k)) return;
  const int L = g.L;
  const size_t m = blockIdx.y;
  u += m * s.cell; v += m * s.cell; delp += m * s.cell; du += m * s.cell; dv += m * s.cell;
  const bool prep = wu != nullptr;
  if (prep) { wu += m * s.cell; wv += m * s.cell; }
  const R thshld = R(1.e-11), two = R(2);
  const size_t c = (size_t)i * L + k;
  R ui[VK], vi[VK], dpi[VK], factor[VK], dfl[VK], su[VK], sv[VK];
  if (prep) {
    ldv<VK>(wu + c, ui);
    ldv<VK>(wv + c, vi);
  } else {
    ldv<VK>(u + c, ui);
    ldv<VK>(v + c, vi);
    const R gs = g.grndspd[i];
    FOR_V ui[j] = ui[j] + gs;
  }
  ldv<VK>(delp + c, dpi);
  const R rar = g.rarea[i];
  FOR_V {
    dpi[j] = rmax(dpi[j], thshld);
    factor[j] = fdiv(rar, dpi[j]);
    dfl[j] = g.dfflen[k + j];
    su[j] = R(0);
    sv[j] = R(0);
  }
  const int np = g.nprox[i];
  // all six prox slots hold valid cells (a pentagon's slot 5 repeats a
  // neighbour), so the gathers carry no branch; slot 5 of a pentagon is
  // dropped by the selects
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const bool live = e < np;
    const int ipx = g.prox[i * 6 + e];
    const R* cs = g.cs + (i * 6 + e) * 4;
    const R* sn = g.sn + (i * 6 + e) * 4;
    const size_t cx = (size_t)ipx * L + k;
    R ux[VK], vx[VK], bx[VK];
    if (prep) {
      ldv<VK>(wu + cx, ux);
      ldv<VK>(wv + cx, vx);
    } else {
      ldv<VK>(u + cx, ux);
      ldv<VK>(v + cx, vx);
      const R gx = g.grndspd[ipx];
      FOR_V ux[j] = ux[j] + gx;
    }
    ldv<VK>(delp + cx, bx);
    const R sl = g.sideln[i * 6 + e];
    FOR_V {
      const R uxy1 = cs[0] * ui[j] + sn[0] * vi[j], vxy1 = -sn[0] * ui[j] + cs[0] * vi[j];
      const R uxy2 = cs[1] * ux[j] + sn[1] * vx[j], vxy2 = -sn[1] * ux[j] + cs[1] * vx[j];
      const R b = rmax(bx[j], thshld);
      const R hf = fdiv(dpi[j] * b, dpi[j] + b);
      const R ufx = (uxy2 - uxy1) * dfl[j] * sl * two * hf;
      const R vfx = (vxy2 - vxy1) * dfl[j] * sl * two * hf;
      const R uflux = cs[0] * ufx - sn[0] * vfx;
      const R vflux = sn[0] * ufx + cs[0] * vfx;
      su[j] = live ? su[j] + uflux * factor[j] : su[j];
      sv[j] = live ? sv[j] + vflux * factor[j] : sv[j];
    }
  }
  stv<VK>(du + c, su);
  stv<VK>(dv + c, sv);
}

// momtum1 (momtum_compute.F90:278-423, janjic=0) after adding the dissipation
// increments (momtum.F90:130-139); one warp per column so the Rayleigh damping
// of the top layers can read the updated top three levels.  Four blocks a
// SM (64 registers, a few spilled) measured 1.77 ms at glvl 8 against 1.96
// at three (80 registers).
template <typename R, int NC>
__global__ void __launch_bounds__(kBlock, 4) k_momtum1(Grid<R> g, Strides s, Knobs kn, const StepParams* __restrict__ sp,
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
  const int* pr = g.prox + i * 6;
  const R rar = g.rarea[i], cor = g.corio[i];
  // Loads use a clamped level and the six edge slots of every cell (a
  // pentagon's slot 5 and its prox entry are valid memory), so they carry no
  // branch and can be issued together; results and stores are masked.
  R un[NC], vn[NC];
#pragma unroll
  for (int ch = 0; ch < NC; ch++) {
    const int k = ch * 32 + lane;
    const int kk = k < L ? k : L - 1;
    const size_t c = (size_t)i * L + kk;
    R uu = u[c], vv = v[c];
    if (have_d) { uu = uu + du[c]; vv = vv + dv[c]; }
    const R exm = R(0.5) * (exner[(size_t)i * L1 + kk] + exner[(size_t)i * L1 + kk + 1]);
    R pgfx = R(0), pgfy = R(0), rv = R(0);
    if (!split) {
#pragma unroll
      for (int e = 0; e < 6; e++) {
        const bool live = e < np;
        const R* svc = g.svc + (i * 6 + e) * 2;
        const R* sve = g.sve + (i * 6 + e) * 2;
        const size_t o = ((size_t)i * 6 + e) * L + kk;
        const R mu = mont_edg[o] + uvsq_edg[o];
        const R th = trc_edg[o];
        const R ue = u_edg[o], ve = v_edg[o];
        if (live) {
          pgfx = pgfx - mu * svc[1] + exm * th * svc[1];
          pgfy = pgfy + mu * svc[0] - exm * th * svc[0];
          rv = rv + (sve[0] * ue + sve[1] * ve);
        }
      }
    } else {
      // FP32-mixed: the same line integrals with the cell values split off,
      // sum_e (M_e + K_e - exm th_e) s_e
      //   = sum_e (dM_e + K_e - exm dth_e) s_e + (M_c - exm th_c) sum_e s_e,
      // dM_e, dth_e the edge-minus-cell values (edgvar1's weights applied to
      // neighbour differences); the large cell term is formed in FP64.
      const R thc = tr0[(size_t)i * L + kk];
      R dth[6];
#pragma unroll
      for (int j = 0; j < 6; j++) {
        const R tn = tr0[(size_t)pr[j] * L + kk];
        dth[j] = (j < np) ? tn - thc : R(0);
      }
      const R divby6 = R(1) / R(6);
#pragma unroll
      for (int e = 0; e < 6; e++) {
        const bool live = e < np;
        const R* svc = g.svc + (i * 6 + e) * 2;
        const R* sve = g.sve + (i * 6 + e) * 2;
        const size_t o = ((size_t)i * 6 + e) * L + kk;
        const int et = e == 0 ? np - 1 : e - 1, el = e == np - 1 ? 0 : e + 1;
        R dte = R(0);
#pragma unroll
        for (int j = 0; j < 6; j++) {
          if (j == e) dte = dte + R(2) * dth[j];
          if (j == et || j == el) dte = dte + dth[j];
        }
        dte = dte * divby6;
        const R mo = mont_edg[o], kv = uvsq_edg[o], ue = u_edg[o], ve = v_edg[o];
        if (live) {
          const R w = mo + kv - exm * dte;
          pgfx = pgfx - w * svc[1];
          pgfy = pgfy + w * svc[0];
          rv = rv + (sve[0] * ue + sve[1] * ve);
        }
      }
      // Montgomery potential minus exner x theta, cancellation-free
      const float2 mp = mpf[(size_t)i * L + kk];
      const FF2 cf = ff_add(FF2{mp.x, mp.y}, ff_neg(two_prod(float(exm), float(thc))));
      const R cell = R(cf.hi + cf.lo);
      pgfx = pgfx - cell * g.svsum[i * 2 + 1];
      pgfy = pgfy + cell * g.svsum[i * 2 + 0];
    }
    pgfx = pgfx * rar;
    pgfy = pgfy * rar;
    rv = rv * rar;
    const R uzeta = (cor + rv) * uu, vzeta = (cor + rv) * vv;
    const R ut = pgfx + vzeta, vt = pgfy - uzeta;
    uu = uu + ab1 * ut + ab2 * u_tndcy[(size_t)of * NL + c] + ab3 * u_tndcy[(size_t)vof * NL + c];
    vv = vv + ab1 * vt + ab2 * v_tndcy[(size_t)of * NL + c] + ab3 * v_tndcy[(size_t)vof * NL + c];
    un[ch] = uu;
    vn[ch] = vv;
    if (k < L) {
      relvor[c] = rv;
      u_tndcy[(size_t)nf * NL + c] = ut;
      v_tndcy[(size_t)nf * NL + c] = vt;
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
  for (int ch = 0; ch < NC; ch++) {
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
  // 8-byte accesses: at 4 levels a thread the kernel holds ~100 registers and
  // runs at half the occupancy, which costs more than the wider accesses gain
  const int vk = pick_vk<R>(g.L, {u, v, delp, montg, tracr, u_edg, v_edg, dp_edg, lp_edg, mont_edg, uvsq_edg,
                                  trc_edg, thold}, 2);
  FIM_KBEGIN(l, "k_edgvar1");
  FIM_VK_DISPATCH(R, vk, (k_edgvar1<R, VK><<<dim3(blocks_for((long long)g.N * (g.L / VK)), l.members), kBlock, 0,
                                             l.stream>>>(g, s, hi_order, u, v, delp, pres, montg, tracr, u_edg,
                                                         v_edg, dp_edg, lp_edg, mont_edg, uvsq_edg, trc_edg, mpf,
                                                         thold)));
  FIM_KEND(l);
}

template <typename R>
void launch_edgvar3(const Launch& l, const Grid<R>& g, const Strides& s, const R* delp, const R* tracr,
                    R* dp_edg, R* trc_edg, int nfields, bool average) {
  const int vk = pick_vk<R>(g.L, {delp, tracr, dp_edg, trc_edg});
  FIM_KBEGIN(l, "k_edgvar3_own");
  FIM_VK_DISPATCH(R, vk, (k_edgvar3_own<R, VK><<<dim3(blocks_for((long long)g.N * (g.L / VK)), l.members, nfields),
                                                 kBlock, 0, l.stream>>>(g, s, delp, tracr, dp_edg, trc_edg)));
  FIM_KEND(l);
  if (!average) return;
  FIM_KBEGIN(l, "k_edgvar3_avg");
  FIM_VK_DISPATCH(R, vk, (k_edgvar3_avg<R, VK><<<dim3(blocks_for((long long)g.N * (g.L / VK)), l.members, nfields),
                                                 kBlock, 0, l.stream>>>(g, s, dp_edg, trc_edg)));
  FIM_KEND(l);
}

template <typename R>
void launch_cnuity(const Launch& l, const Grid<R>& g, const Strides& s, const CnuityScratch<R>& w, const R* u,
                   const R* v, const R* u_edg, const R* v_edg, const R* dp_edg, const R* lp_edg,
                   R* delp, R* pres, R* exner, R* dp_tndcy, R* dplo_tndcy, R* massfx, R* omega) {
  const int vk = pick_vk<R>(g.L, {u_edg, v_edg, dp_edg, delp, massfx, dplo_tndcy, dp_tndcy, w.antifx, w.delp_lo,
                                  w.p_plus, w.p_mnus, w.r_plus, w.r_mnus});
  if (l.coop) {
    // one cooperative launch of as many blocks as the GPU holds at once
    FIM_KBEGIN(l, "k_cnuity_coop");
    cudaMemsetAsync(l.coop->barrier, 0, sizeof(unsigned), l.stream);
    FIM_VK_DISPATCH(R, vk, ({
      int dev = 0, sms = 0, per = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cnuity_coop<R, VK>, kBlock, 0);
      const long long need = (long long)blocks_for((long long)g.N * (g.L / VK)) * l.members;
      const unsigned nb = (unsigned)(need < (long long)sms * per ? need : (long long)sms * per);
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(nb > 0 ? nb : 1);
      cfg.blockDim = dim3(kBlock);
      cfg.stream = l.stream;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      cudaLaunchKernelEx(&cfg, k_cnuity_coop<R, VK>, g, s, l.sp, l.members, u_edg, v_edg, dp_edg, delp, massfx,
                         dplo_tndcy, dp_tndcy, w.antifx, w.delp_lo, w.p_plus, w.p_mnus, w.r_plus, w.r_mnus,
                         l.flags, l.coop->barrier, l.coop->extra, l.coop->limit_ns);
    }));
    FIM_KEND(l);
  } else {
  FIM_KBEGIN(l, "k_cnuity12");
  FIM_VK_DISPATCH(R, vk, (k_cnuity12<R, VK><<<dim3(blocks_for((long long)g.N * (g.L / VK)), l.members), kBlock, 0,
                                              l.stream>>>(g, s, l.sp, u_edg, v_edg, dp_edg, delp, massfx,
                                                          dplo_tndcy, w.antifx, w.delp_lo, w.p_plus, w.p_mnus)));
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_cnuity3");
  FIM_VK_DISPATCH(R, vk, (k_cnuity3<R, VK><<<dim3(blocks_for((long long)g.N * (g.L / VK)), l.members), kBlock, 0,
                                             l.stream>>>(g, s, l.sp, w.delp_lo, delp, dp_tndcy, w.p_plus, w.p_mnus,
                                                         w.r_plus, w.r_mnus)));
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_cnuity4");
  FIM_VK_DISPATCH(R, vk, (k_cnuity4<R, VK><<<dim3(blocks_for((long long)g.N * (g.L / VK)), l.members), kBlock, 0,
                                             l.stream>>>(g, s, l.sp, w.antifx, w.r_plus, w.r_mnus, massfx,
                                                         dplo_tndcy, dp_tndcy, delp, l.flags)));
  FIM_KEND(l);
  }
  dim3 gw((unsigned)((g.N + 32 * kC5Warps<R> - 1) / (32 * kC5Warps<R>)), l.members);
  FIM_KBEGIN(l, "k_cnuity5");
  k_cnuity5<R><<<gw, 32 * kC5Warps<R>, 0, l.stream>>>(g, s, l.sp, pres, delp, exner, dp_tndcy, omega, lp_edg, u,
                                                      v, 0);
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
    const int vk = pick_vk<R>(g.L, {u, v, wu, wv, dp3d, w.du, w.dv});
    FIM_KBEGIN(l, "k_dissip");
    FIM_VK_DISPATCH(R, vk, (k_dissip<R, VK><<<dim3(blocks_for((long long)g.N * (g.L / VK)), l.members), kBlock, 0,
                                              l.stream>>>(g, s, u, v, wu, wv, dp3d, w.du, w.dv)));
    FIM_KEND(l);
    du = w.du;
    dv = w.dv;
  }
  dim3 gw(blocks_for((long long)g.N * 32), l.members);
  FIM_KBEGIN(l, "k_momtum1");
  const int nc = (g.L + 31) / 32;
#define FIM_MOMTUM1(NC)                                                                                        \
  k_momtum1<R, NC><<<gw, kBlock, 0, l.stream>>>(g, s, kn, l.sp, u, v, du, dv, exner, relvor, u_edg, v_edg, trc_edg, \
                                                 mont_edg, uvsq_edg, u_tndcy, v_tndcy, mpf, tr0)
  if (nc == 1) FIM_MOMTUM1(1);
  else if (nc == 2) FIM_MOMTUM1(2);
  else if (nc == 3) FIM_MOMTUM1(3);
  else FIM_MOMTUM1(4);
#undef FIM_MOMTUM1
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
  template void launch_edgvar2<R>(const Launch&, const Grid<R>&, const Strides&, const R*, const R*, R*, R*,  \
                                  R*, R*);                                                                    \
  template void launch_edgvar3<R>(const Launch&, const Grid<R>&, const Strides&, const R*, const R*, R*, R*,  \
                                  int, bool);                                                                \
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
