// Tracer transport of the fused step: edgvar3's tracer reconstruction and
// trcadv1..3 (trcadv_compute.F90:19-315) for all tracers, without
// materialising the averaged tracer edge values or the antidiffusive fluxes.
//
//   k_tr_own   edgvalEval per tracer 2..ntra (edgvar3.F90:66-94): own-side edge
//              values into trc_edg (the two-sided average of edgvar3 loop 2 is
//              formed where it is used, 0.5*(own + neighbour's own), which is the
//              value the reference stores in both slots).
//   k_tr_lo    trcadv1: low-order fluxes, low-order AB3 update, trcr_lo, and the
//              Zalesak sums S+/S- of trcadv2; copies the old tracer.
//   k_tr_lim   trcadv2: bounds relaxed with the 1-ring trcr_lo, Q+/Q-, R+/R-.
//   k_tr_hi    trcadv3: recomputes each antidiffusive flux, clips it with the
//              own/neighbour limiters, AB3 update of tracer x thickness, new tracer.
//
// One thread per (level, cell) loops over the tracers, so the mass fluxes and
// the donor-cell coefficients of its six edges are loaded once for all
// tracers.  Every flux is formed from the same operands in the same order as
// the per-routine kernels, so results are bit-identical to them.
#include "fim_internal.h"

namespace fim {

template <typename R> __device__ __forceinline__ R tmax(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R tmin(R a, R b) { return a < b ? a : b; }
template <typename R> __device__ __forceinline__ R tabs(R a) { return a < R(0) ? -a : a; }

constexpr int kTB = 256;
inline unsigned tblocks(long long n) { return (unsigned)((n + kTB - 1) / kTB); }

__device__ __forceinline__ bool cl(int N, int L, int& i, int& k) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * L) return false;
  i = gid / L;
  k = gid - i * L;
  return true;
}

// own-side least-squares edge values of tracers 1..T-1 (0-based), z = tracer
template <typename R>
__global__ void __launch_bounds__(kTB) k_tr_own(Grid<R> g, Strides s, const R* __restrict__ tracr,
                                                R* __restrict__ trc_edg) {
  int i, k;
  if (!cl(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  const int t = blockIdx.z + 1;
  const R* src = tracr + m * s.tr + (size_t)t * N * L;
  R* dst = trc_edg + m * s.tredg + (size_t)t * N * 6 * L;
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

// Per-edge operands shared by all tracers of a (level, cell).
template <typename R>
struct EdgeOps {
  int np;
  int ipx[6];
  size_t own[6], mir[6];  // offsets of own and neighbour's edge slot
  R mf[6], a[6], b[6];    // massfx(nf), mf+|mf|, mx+|mx|
};

template <typename R>
__device__ __forceinline__ void load_edges(const Grid<R>& g, const R* mfn, int i, int k, EdgeOps<R>& E) {
  const int L = g.L;
  E.np = g.nprox[i];
#pragma unroll
  for (int e = 0; e < 6; e++) {
    if (e < E.np) {
      const int ipx = g.prox[i * 6 + e], edx = g.proxs[i * 6 + e];
      E.ipx[e] = ipx;
      E.own[e] = ((size_t)i * 6 + e) * L + k;
      E.mir[e] = ((size_t)ipx * 6 + edx) * L + k;
      const R m = mfn[E.own[e]], mx = mfn[E.mir[e]];
      E.mf[e] = m;
      E.a[e] = m + tabs(m);
      E.b[e] = mx + tabs(mx);
    }
  }
}

// tracer t's averaged edge value on edge e (t = 0: edgvar1's value)
template <typename R>
__device__ __forceinline__ R edge_value(const R* te, int t, const EdgeOps<R>& E, int e) {
  return (t == 0) ? te[E.own[e]] : R(0.5) * (te[E.own[e]] + te[E.mir[e]]);
}

// trcadv1 for all tracers + the S+/S- sums of trcadv2 + copy of the old tracer
template <typename R>
__global__ void __launch_bounds__(kTB) k_tr_lo(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ massfx, const R* __restrict__ trc_edg, const R* __restrict__ tracr,
    const R* __restrict__ trcdp, R* __restrict__ trl_tdcy, const R* __restrict__ delp,
    R* __restrict__ trcr_lo, R* __restrict__ s_plus, R* __restrict__ s_mnus, R* __restrict__ trold,
    size_t sc) {
  int i, k;
  if (!cl(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const size_t NL = (size_t)N * L;
  massfx += m * s.mf; trc_edg += m * s.tredg; tracr += m * s.tr; trcdp += m * s.tr;
  trl_tdcy += m * s.trab; delp += m * s.cell;
  const size_t so = m * nt * sc;
  trcr_lo += so; s_plus += so; s_mnus += so; trold += so;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11), half = R(0.5);
  EdgeOps<R> E;
  load_edges(g, massfx + (size_t)nf * N * 6 * L, i, k, E);
  const size_t c = (size_t)i * L + k;
  const R rar = g.rarea[i];
  const R dpc = tmax(thshld, delp[c]);
  const int* pr = g.prox + i * 6;
  for (int tz = 0; tz < nt; tz++) {
    const int t = t0 + tz;
    const R* tr = tracr + (size_t)t * NL;
    const R* te = trc_edg + (size_t)t * 6 * NL;
    const R tri = tr[c];
    R sumlo = R(0), sp_ = R(0), sm_ = R(0);
#pragma unroll
    for (int e = 0; e < 6; e++) {
      if (e < E.np) {
        const R hi = E.mf[e] * edge_value(te, t, E, e);
        const R lo = half * (E.a[e] * tri - E.b[e] * tr[(size_t)E.ipx[e] * L + k]);
        const R anti = hi - lo;
        sumlo = sumlo + lo;
        sp_ = sp_ - tmin(R(0), anti);
        sm_ = sm_ + tmax(R(0), anti);
      }
    }
    R* tl = trl_tdcy + (size_t)t * 3 * NL;
    const R tn = -sumlo * rar;
    tl[(size_t)nf * NL + c] = tn;
    const R lo = trcdp[(size_t)t * NL + c] + ab1 * tn + ab2 * tl[(size_t)of * NL + c] + ab3 * tl[(size_t)vof * NL + c];
    R mx = tri, mn = tri;
#pragma unroll
    for (int e = 0; e < 6; e++) {
      const R x = tr[(size_t)pr[e] * L + k];
      mx = tmax(mx, x);
      mn = tmin(mn, x);
    }
    mx = tmax(R(0), mx);
    mn = tmax(R(0), mn);
    const size_t q = (size_t)tz * sc + c;
    trcr_lo[q] = tmax(mn, tmin(mx, lo / dpc));
    s_plus[q] = sp_;
    s_mnus[q] = sm_;
    trold[q] = tri;
  }
}

// trcadv2: Q+/Q- and the limiters R+/R-; the relaxed bounds are
// max/min over the 1-ring of the old tracer and of trcr_lo (exact operations,
// so any association gives the reference's values).
template <typename R>
__global__ void __launch_bounds__(kTB) k_tr_lim(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ trc_tdcy, const R* __restrict__ delp, const R* __restrict__ trold,
    const R* __restrict__ trcr_lo, const R* __restrict__ s_plus, const R* __restrict__ s_mnus,
    R* __restrict__ r_plus, R* __restrict__ r_mnus, size_t sc) {
  int i, k;
  if (!cl(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const size_t NL = (size_t)N * L;
  trc_tdcy += m * s.trab; delp += m * s.cell;
  const size_t so = m * nt * sc;
  trold += so; trcr_lo += so; s_plus += so; s_mnus += so; r_plus += so; r_mnus += so;
  const int of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11);
  const size_t c = (size_t)i * L + k;
  const int* pr = g.prox + i * 6;
  const R dp = delp[c];
  const R ar = g.area[i];
  for (int tz = 0; tz < nt; tz++) {
    const int t = t0 + tz;
    const R* to = trold + (size_t)tz * sc;
    const R* lo = trcr_lo + (size_t)tz * sc;
    const R lc = lo[c];
    R mx = tmax(to[c], lc), mn = tmin(to[c], lc);
#pragma unroll
    for (int e = 0; e < 6; e++) {
      const size_t cx = (size_t)pr[e] * L + k;
      mx = tmax(mx, tmax(to[cx], lo[cx]));
      mn = tmin(mn, tmin(to[cx], lo[cx]));
    }
    mx = tmax(R(0), mx);
    mn = tmax(R(0), mn);
    const R* tc = trc_tdcy + (size_t)t * 3 * NL;
    const R tof = tc[(size_t)of * NL + c], tvf = tc[(size_t)vof * NL + c];
    const R q_plus = ((mx - lc) * dp - (ab2 * tmin(R(0), tof) + ab3 * tmax(R(0), tvf))) / ab1 * ar;
    const R q_mnus = ((lc - mn) * dp + (ab2 * tmax(R(0), tof) + ab3 * tmin(R(0), tvf))) / ab1 * ar;
    const size_t q = (size_t)tz * sc + c;
    r_plus[q] = tmax(R(0), tmin(R(1), q_plus / tmax(s_plus[q], thshld)));
    r_mnus[q] = tmax(R(0), tmin(R(1), q_mnus / tmax(s_mnus[q], thshld)));
  }
}

// trcadv3: clip the recomputed antidiffusive fluxes, AB3 update, new tracer
template <typename R>
__global__ void __launch_bounds__(kTB) k_tr_hi(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ massfx, const R* __restrict__ trc_edg, R* __restrict__ tracr,
    R* __restrict__ trcdp, R* __restrict__ trc_tdcy, const R* __restrict__ trl_tdcy, const R* __restrict__ delp,
    const R* __restrict__ trold, const R* __restrict__ trcr_lo, const R* __restrict__ r_plus,
    const R* __restrict__ r_mnus, size_t sc) {
  int i, k;
  if (!cl(g.N, g.L, i, k)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const size_t NL = (size_t)N * L;
  massfx += m * s.mf; trc_edg += m * s.tredg; tracr += m * s.tr; trcdp += m * s.tr;
  trc_tdcy += m * s.trab; trl_tdcy += m * s.trab; delp += m * s.cell;
  const size_t so = m * nt * sc;
  trold += so; trcr_lo += so; r_plus += so; r_mnus += so;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11), half = R(0.5);
  EdgeOps<R> E;
  load_edges(g, massfx + (size_t)nf * N * 6 * L, i, k, E);
  const size_t c = (size_t)i * L + k;
  const R rar = g.rarea[i];
  const R dpc = tmax(thshld, delp[c]);
  const int* pr = g.prox + i * 6;
  for (int tz = 0; tz < nt; tz++) {
    const int t = t0 + tz;
    const R* to = trold + (size_t)tz * sc;
    const R* te = trc_edg + (size_t)t * 6 * NL;
    const R* rp = r_plus + (size_t)tz * sc;
    const R* rm = r_mnus + (size_t)tz * sc;
    const R tri = to[c];
    const R rpc = rp[c], rmc = rm[c];
    R at = R(0);
#pragma unroll
    for (int e = 0; e < 6; e++) {
      if (e < E.np) {
        const size_t cx = (size_t)E.ipx[e] * L + k;
        const R hi = E.mf[e] * edge_value(te, t, E, e);
        const R lo = half * (E.a[e] * tri - E.b[e] * to[cx]);
        R a = hi - lo;
        if (a >= R(0)) a = a * tmin(rmc, rp[cx]);
        else a = a * tmin(rpc, rm[cx]);
        at = at + a;
      }
    }
    // bounds of trcadv2, recomputed (max/min are exact)
    const R* lo_ = trcr_lo + (size_t)tz * sc;
    R mx = tmax(tri, lo_[c]), mn = tmin(tri, lo_[c]);
#pragma unroll
    for (int e = 0; e < 6; e++) {
      const size_t cx = (size_t)pr[e] * L + k;
      mx = tmax(mx, tmax(to[cx], lo_[cx]));
      mn = tmin(mn, tmin(to[cx], lo_[cx]));
    }
    mx = tmax(R(0), mx);
    mn = tmax(R(0), mn);
    at = -at * rar;
    R* tc = trc_tdcy + (size_t)t * 3 * NL;
    const R tn = trl_tdcy[(size_t)t * 3 * NL + (size_t)nf * NL + c] + at;
    tc[(size_t)nf * NL + c] = tn;
    const R td = trcdp[(size_t)t * NL + c] + ab1 * tn + ab2 * tc[(size_t)of * NL + c] + ab3 * tc[(size_t)vof * NL + c];
    trcdp[(size_t)t * NL + c] = td;
    tracr[(size_t)t * NL + c] = tmax(mn, tmin(mx, td / dpc));
  }
}

template <typename R>
void launch_tracers_fused(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w,
                          R* trc_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx,
                          const R* delp) {
  const size_t sc = (size_t)g.N * g.L;
  dim3 grid(tblocks((long long)g.N * g.L), l.members);
  for (int t0 = 0; t0 < g.T; t0 += w.tchunk) {
    const int nt = (g.T - t0 < w.tchunk) ? g.T - t0 : w.tchunk;
    FIM_KBEGIN(l, "k_tr_lo");
    k_tr_lo<R><<<grid, kTB, 0, l.stream>>>(g, s, l.sp, t0, nt, massfx, trc_edg, tracr, trcdp, trl_tdcy, delp,
                                            w.trcr_lo, w.s_plus, w.s_mnus, w.trold, sc);
    FIM_KEND(l);
    FIM_KBEGIN(l, "k_tr_lim");
    k_tr_lim<R><<<grid, kTB, 0, l.stream>>>(g, s, l.sp, t0, nt, trc_tdcy, delp, w.trold, w.trcr_lo, w.s_plus,
                                             w.s_mnus, w.r_plus, w.r_mnus, sc);
    FIM_KEND(l);
    FIM_KBEGIN(l, "k_tr_hi");
    k_tr_hi<R><<<grid, kTB, 0, l.stream>>>(g, s, l.sp, t0, nt, massfx, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy,
                                            delp, w.trold, w.trcr_lo, w.r_plus, w.r_mnus, sc);
    FIM_KEND(l);
  }
}

template <typename R>
void launch_tracer_own(const Launch& l, const Grid<R>& g, const Strides& s, const R* tracr, R* trc_edg) {
  if (g.T < 2) return;
  dim3 grid(tblocks((long long)g.N * g.L), l.members, g.T - 1);
  FIM_KBEGIN(l, "k_tr_own");
  k_tr_own<R><<<grid, kTB, 0, l.stream>>>(g, s, tracr, trc_edg);
  FIM_KEND(l);
}

#define INSTANTIATE(R)                                                                                        \
  template void launch_tracers_fused<R>(const Launch&, const Grid<R>&, const Strides&,                       \
                                        const TrcFusedScratch<R>&, R*, R*, R*, R*, R*, const R*, const R*);  \
  template void launch_tracer_own<R>(const Launch&, const Grid<R>&, const Strides&, const R*, R*);
INSTANTIATE(float)
INSTANTIATE(double)

}  // namespace fim
