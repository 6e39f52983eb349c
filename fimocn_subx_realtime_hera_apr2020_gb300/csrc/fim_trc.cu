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
// Every flux is formed from the same operands in the same order as the
// per-routine kernels, so results are bit-identical to them.
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

// One thread per (level, cell, tracer).  The tracer is the fastest-varying
// part of the block index, so the blocks of one cell range and all tracers of
// a chunk run back to back and the mass fluxes they share are L2 hits.
__device__ __forceinline__ bool clt(int N, int L, int nt, int& i, int& k, int& tz) {
  tz = blockIdx.x % nt;
  const int cb = blockIdx.x / nt;
  const int gid = cb * blockDim.x + threadIdx.x;
  if (gid >= N * L) return false;
  i = gid / L;
  k = gid - i * L;
  return true;
}

// trcadv1 + the S+/S- sums of trcadv2 + copy of the old tracer
template <typename R>
__global__ void __launch_bounds__(kTB) k_tr_lo(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ massfx, const R* __restrict__ trc_edg, const R* __restrict__ tracr,
    const R* __restrict__ trcdp, R* __restrict__ trl_tdcy, const R* __restrict__ delp,
    R* __restrict__ trcr_lo, R* __restrict__ s_plus, R* __restrict__ s_mnus, R* __restrict__ trold,
    size_t sc) {
  int i, k, tz;
  if (!clt(g.N, g.L, nt, i, k, tz)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const int t = t0 + tz;
  const size_t NL = (size_t)N * L;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R* mfn = massfx + m * s.mf + (size_t)nf * 6 * NL;
  const R* te = trc_edg + m * s.tredg + (size_t)t * 6 * NL;
  const R* tr = tracr + m * s.tr + (size_t)t * NL;
  R* tl = trl_tdcy + m * s.trab + (size_t)t * 3 * NL;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11), half = R(0.5);
  const int c = i * L + k;
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  const int* ps = g.proxs + i * 6;
  const R tri = tr[c];
  R sumlo = R(0), sp_ = R(0), sm_ = R(0), mx = tri, mn = tri;
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const int ipx = pr[e];
    const R trx = tr[ipx * L + k];
    mx = tmax(mx, trx);
    mn = tmin(mn, trx);
    if (e < np) {
      const int own = (i * 6 + e) * L + k, mir = (ipx * 6 + ps[e]) * L + k;
      const R mf = mfn[own], mfx = mfn[mir];
      const R tev = (t == 0) ? te[own] : half * (te[own] + te[mir]);
      const R hi = mf * tev;
      const R lo = half * ((mf + tabs(mf)) * tri - (mfx + tabs(mfx)) * trx);
      const R anti = hi - lo;
      sumlo = sumlo + lo;
      sp_ = sp_ - tmin(R(0), anti);
      sm_ = sm_ + tmax(R(0), anti);
    }
  }
  const R tn = -sumlo * g.rarea[i];
  tl[(size_t)nf * NL + c] = tn;
  const R lo = trcdp[m * s.tr + (size_t)t * NL + c] + ab1 * tn + ab2 * tl[(size_t)of * NL + c] +
               ab3 * tl[(size_t)vof * NL + c];
  mx = tmax(R(0), mx);
  mn = tmax(R(0), mn);
  const size_t q = (m * nt + tz) * sc + c;
  trcr_lo[q] = tmax(mn, tmin(mx, lo / tmax(thshld, delp[m * s.cell + c])));
  s_plus[q] = sp_;
  s_mnus[q] = sm_;
  trold[q] = tri;
}

// trcadv2: Q+/Q- and the limiters R+/R-; the relaxed bounds are
// max/min over the 1-ring of the old tracer and of trcr_lo (exact operations,
// so any association gives the reference's values).
template <typename R>
__global__ void __launch_bounds__(kTB) k_tr_lim(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ trc_tdcy, const R* __restrict__ delp, const R* __restrict__ trold,
    const R* __restrict__ trcr_lo, const R* __restrict__ s_plus, const R* __restrict__ s_mnus,
    R* __restrict__ r_plus, R* __restrict__ r_mnus, size_t sc) {
  int i, k, tz;
  if (!clt(g.N, g.L, nt, i, k, tz)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const int t = t0 + tz;
  const size_t NL = (size_t)N * L;
  const int of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11);
  const int c = i * L + k;
  const size_t so = (m * nt + tz) * sc;
  const R* to = trold + so;
  const R* lo = trcr_lo + so;
  const int* pr = g.prox + i * 6;
  const R lc = lo[c];
  R mx = tmax(to[c], lc), mn = tmin(to[c], lc);
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const int cx = pr[e] * L + k;
    const R a = to[cx], b = lo[cx];
    mx = tmax(mx, tmax(a, b));
    mn = tmin(mn, tmin(a, b));
  }
  mx = tmax(R(0), mx);
  mn = tmax(R(0), mn);
  const R* tc = trc_tdcy + m * s.trab + (size_t)t * 3 * NL;
  const R tof = tc[(size_t)of * NL + c], tvf = tc[(size_t)vof * NL + c];
  const R dp = delp[m * s.cell + c], ar = g.area[i];
  const R q_plus = ((mx - lc) * dp - (ab2 * tmin(R(0), tof) + ab3 * tmax(R(0), tvf))) / ab1 * ar;
  const R q_mnus = ((lc - mn) * dp + (ab2 * tmax(R(0), tof) + ab3 * tmin(R(0), tvf))) / ab1 * ar;
  r_plus[so + c] = tmax(R(0), tmin(R(1), q_plus / tmax(s_plus[so + c], thshld)));
  r_mnus[so + c] = tmax(R(0), tmin(R(1), q_mnus / tmax(s_mnus[so + c], thshld)));
}

// trcadv3: clip the recomputed antidiffusive fluxes, AB3 update, new tracer
template <typename R>
__global__ void __launch_bounds__(kTB) k_tr_hi(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ massfx, const R* __restrict__ trc_edg, R* __restrict__ tracr,
    R* __restrict__ trcdp, R* __restrict__ trc_tdcy, const R* __restrict__ trl_tdcy, const R* __restrict__ delp,
    const R* __restrict__ trold, const R* __restrict__ trcr_lo, const R* __restrict__ r_plus,
    const R* __restrict__ r_mnus, size_t sc) {
  int i, k, tz;
  if (!clt(g.N, g.L, nt, i, k, tz)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const int t = t0 + tz;
  const size_t NL = (size_t)N * L;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11), half = R(0.5);
  const R* mfn = massfx + m * s.mf + (size_t)nf * 6 * NL;
  const R* te = trc_edg + m * s.tredg + (size_t)t * 6 * NL;
  const size_t so = (m * nt + tz) * sc;
  const R* to = trold + so;
  const R* lo = trcr_lo + so;
  const R* rp = r_plus + so;
  const R* rm = r_mnus + so;
  const int c = i * L + k;
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  const int* ps = g.proxs + i * 6;
  const R tri = to[c], rpc = rp[c], rmc = rm[c], lc = lo[c];
  R at = R(0), mx = tmax(tri, lc), mn = tmin(tri, lc);
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const int ipx = pr[e];
    const int cx = ipx * L + k;
    const R trx = to[cx], lox = lo[cx];
    mx = tmax(mx, tmax(trx, lox));
    mn = tmin(mn, tmin(trx, lox));
    if (e < np) {
      const int own = (i * 6 + e) * L + k, mir = (ipx * 6 + ps[e]) * L + k;
      const R mf = mfn[own], mfx = mfn[mir];
      const R tev = (t == 0) ? te[own] : half * (te[own] + te[mir]);
      const R hi = mf * tev;
      const R lo_ = half * ((mf + tabs(mf)) * tri - (mfx + tabs(mfx)) * trx);
      R a = hi - lo_;
      if (a >= R(0)) a = a * tmin(rmc, rp[cx]);
      else a = a * tmin(rpc, rm[cx]);
      at = at + a;
    }
  }
  mx = tmax(R(0), mx);
  mn = tmax(R(0), mn);
  at = -at * g.rarea[i];
  R* tc = trc_tdcy + m * s.trab + (size_t)t * 3 * NL;
  const R tn = trl_tdcy[m * s.trab + (size_t)t * 3 * NL + (size_t)nf * NL + c] + at;
  tc[(size_t)nf * NL + c] = tn;
  R* td = trcdp + m * s.tr + (size_t)t * NL;
  const R tdn = td[c] + ab1 * tn + ab2 * tc[(size_t)of * NL + c] + ab3 * tc[(size_t)vof * NL + c];
  td[c] = tdn;
  tracr[m * s.tr + (size_t)t * NL + c] = tmax(mn, tmin(mx, tdn / tmax(thshld, delp[m * s.cell + c])));
}

template <typename R>
void launch_tracers_fused(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w,
                          R* trc_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx,
                          const R* delp) {
  const size_t sc = (size_t)g.N * g.L;
  for (int t0 = 0; t0 < g.T; t0 += w.tchunk) {
    const int nt = (g.T - t0 < w.tchunk) ? g.T - t0 : w.tchunk;
    dim3 grid(tblocks((long long)g.N * g.L) * nt, l.members);
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
