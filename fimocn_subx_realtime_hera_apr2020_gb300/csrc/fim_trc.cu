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
//              The low-order tendency of this step, which k_tr_lo stored, is
//              recomputed from the same fluxes in the same order rather than
//              read back.
//
// Every flux is formed from the same operands in the same order as the
// per-routine kernels, so results are bit-identical to them.
#include "fim_internal.h"

namespace fim {

template <typename R> __device__ __forceinline__ R tmax(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R tmin(R a, R b) { return a < b ? a : b; }
template <typename R> __device__ __forceinline__ R tabs(R a) { return a < R(0) ? -a : a; }
// max/min of three (exact; FP32 uses the three-input instructions)
template <typename R> __device__ __forceinline__ R tmax3(R a, R b, R c) { return tmax(a, tmax(b, c)); }
template <typename R> __device__ __forceinline__ R tmin3(R a, R b, R c) { return tmin(a, tmin(b, c)); }
template <> __device__ __forceinline__ float tmax3<float>(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
template <> __device__ __forceinline__ float tmin3<float>(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
// product rounded on its own (never contracted into a following add)
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// Blocks of up to kTB threads capped at 64 registers a thread (32 resident
// warps per SM keep enough loads in flight for these gather-heavy,
// latency-bound kernels); the block size actually launched (128 or 256, the
// cell patch) and the levels per thread are picked by tune_tracers.
#ifndef FIM_TRC_MINB
#define FIM_TRC_MINB 4
#endif
constexpr int kTB = 256;
constexpr int kTBMin = FIM_TRC_MINB;
inline unsigned tblocks(long long n, int tb) { return (unsigned)((n + tb - 1) / tb); }

// own-side least-squares edge values of tracers 1..T-1 (0-based), z = tracer
template <typename R, int VK>
__global__ void __launch_bounds__(kTB, kTBMin) k_tr_own(Grid<R> g, Strides s, const R* __restrict__ tracr,
                                                R* __restrict__ trc_edg) {
  const int L = g.L, N = g.N, LV = L / VK;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * LV) return;
  const int i = gid / LV, k = (gid - i * LV) * VK;
  const size_t m = blockIdx.y;
  const int t = blockIdx.z + 1;
  const R* src = tracr + m * s.tr + (size_t)t * N * L;
  R* dst = trc_edg + m * s.tredg + (size_t)t * N * 6 * L;
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  R bc[VK];
  ldv<VK>(src + i * L + k, bc);
  // every prox slot is a valid cell (a pentagon's slot 5 repeats a
  // neighbour), so the gathers carry no branch and can all be in flight;
  // slot 5 of a pentagon is dropped by selects
  R d[6][VK];
#pragma unroll
  for (int e = 0; e < 6; e++) {
    ldv<VK>(src + pr[e] * L + k, d[e]);
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
    stv<VK>(dst + (i * 6 + ie) * L + k, val);
  }
}

// One thread per (VK levels, cell, tracer).  The tracer is the fastest-varying
// part of the block index, so the blocks of one cell range and all tracers of
// a chunk run back to back and the mass fluxes they share are L2 hits.
template <int VK>
__device__ __forceinline__ bool clt(int N, int L, int nt, int& i, int& k, int& tz) {
  tz = blockIdx.x % nt;
  const int cb = blockIdx.x / nt;
  const int LV = L / VK;
  const int gid = cb * blockDim.x + threadIdx.x;
  if (gid >= N * LV) return false;
  i = gid / LV;
  k = (gid - i * LV) * VK;
  return true;
}

// trcadv1 + the S+/S- sums of trcadv2 + copy of the old tracer
template <typename R, int VK>
__global__ void __launch_bounds__(kTB, kTBMin) k_tr_lo(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ massfx, const R* __restrict__ trc_edg, const R* __restrict__ tracr,
    const R* __restrict__ trcdp, R* __restrict__ trl_tdcy, const R* __restrict__ delp,
    R* __restrict__ trcr_lo, R* __restrict__ s_plus, R* __restrict__ s_mnus, R* __restrict__ trold,
    size_t sc) {
  int i, k, tz;
  if (!clt<VK>(g.N, g.L, nt, i, k, tz)) return;
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
  R tri[VK], sumlo[VK], sp_[VK], sm_[VK], mx[VK], mn[VK];
  ldv<VK>(tr + c, tri);
  FOR_V { sumlo[j] = R(0); sp_[j] = R(0); sm_[j] = R(0); mx[j] = tri[j]; mn[j] = tri[j]; }
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const int ipx = pr[e];
    R trx[VK];
    ldv<VK>(tr + ipx * L + k, trx);
    FOR_V { mx[j] = tmax(mx[j], trx[j]); mn[j] = tmin(mn[j], trx[j]); }
    if (e < np) {
      const int own = (i * 6 + e) * L + k, mir = (ipx * 6 + ps[e]) * L + k;
      R mf[VK], mfx[VK], tev[VK];
      ldv<VK>(mfn + own, mf);
      ldv<VK>(mfn + mir, mfx);
      ldv<VK>(te + own, tev);
      if (t != 0) {
        R tem[VK];
        ldv<VK>(te + mir, tem);
        FOR_V tev[j] = half * (tev[j] + tem[j]);
      }
      FOR_V {
        const R hi = mf[j] * tev[j];
        const R lo = half * ((mf[j] + tabs(mf[j])) * tri[j] - (mfx[j] + tabs(mfx[j])) * trx[j]);
        const R anti = hi - lo;
        sumlo[j] = sumlo[j] + lo;
        sp_[j] = sp_[j] - tmin(R(0), anti);
        sm_[j] = sm_[j] + tmax(R(0), anti);
      }
    }
  }
  const R rar = g.rarea[i];
  R tn[VK], tlo[VK], tlv[VK], td[VK], dp[VK], out[VK];
  FOR_V tn[j] = -sumlo[j] * rar;
  stv<VK>(tl + (size_t)nf * NL + c, tn);
  ldv<VK>(tl + (size_t)of * NL + c, tlo);
  ldv<VK>(tl + (size_t)vof * NL + c, tlv);
  ldv<VK>(trcdp + m * s.tr + (size_t)t * NL + c, td);
  ldv<VK>(delp + m * s.cell + c, dp);
  const size_t q = (m * nt + tz) * sc + c;
  FOR_V {
    const R lo = td[j] + ab1 * tn[j] + ab2 * tlo[j] + ab3 * tlv[j];
    const R hx = tmax(R(0), mx[j]), hn = tmax(R(0), mn[j]);
    out[j] = tmax(hn, tmin(hx, fdiv(lo, tmax(thshld, dp[j]))));
  }
  stv<VK>(trcr_lo + q, out);
  stv<VK>(s_plus + q, sp_);
  stv<VK>(s_mnus + q, sm_);
  stv<VK>(trold + q, tri);
}

// trcadv2: Q+/Q- and the limiters R+/R-; the relaxed bounds are
// max/min over the 1-ring of the old tracer and of trcr_lo (exact operations,
// so any association gives the reference's values).
template <typename R, int VK>
__global__ void __launch_bounds__(kTB, kTBMin) k_tr_lim(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ trc_tdcy, const R* __restrict__ delp, const R* __restrict__ trold,
    const R* __restrict__ trcr_lo, const R* __restrict__ s_plus, const R* __restrict__ s_mnus,
    R* __restrict__ r_plus, R* __restrict__ r_mnus, size_t sc) {
  int i, k, tz;
  if (!clt<VK>(g.N, g.L, nt, i, k, tz)) return;
  const int L = g.L, N = g.N;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const int t = t0 + tz;
  const size_t NL = (size_t)N * L;
  const int of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R rab1 = R(1) / ab1;  // Q+/Q- divide by ab1: one reciprocal (as k_trcadv2)
  const R thshld = R(1.e-11);
  const int c = i * L + k;
  const size_t so = (m * nt + tz) * sc;
  const R* to = trold + so;
  const R* lo = trcr_lo + so;
  const int* pr = g.prox + i * 6;
  R lc[VK], tc0[VK], mx[VK], mn[VK];
  ldv<VK>(lo + c, lc);
  ldv<VK>(to + c, tc0);
  FOR_V { mx[j] = tmax(tc0[j], lc[j]); mn[j] = tmin(tc0[j], lc[j]); }
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const int cx = pr[e] * L + k;
    R a[VK], b[VK];
    ldv<VK>(to + cx, a);
    ldv<VK>(lo + cx, b);
    FOR_V { mx[j] = tmax3(mx[j], a[j], b[j]); mn[j] = tmin3(mn[j], a[j], b[j]); }
  }
  const R* tc = trc_tdcy + m * s.trab + (size_t)t * 3 * NL;
  R tof[VK], tvf[VK], dp[VK], spl[VK], smn[VK], rp[VK], rm[VK];
  ldv<VK>(tc + (size_t)of * NL + c, tof);
  ldv<VK>(tc + (size_t)vof * NL + c, tvf);
  ldv<VK>(delp + m * s.cell + c, dp);
  ldv<VK>(s_plus + so + c, spl);
  ldv<VK>(s_mnus + so + c, smn);
  const R ar = g.area[i];
  FOR_V {
    const R hx = tmax(R(0), mx[j]), hn = tmax(R(0), mn[j]);
    const R q_plus = ((hx - lc[j]) * dp[j] - (ab2 * tmin(R(0), tof[j]) + ab3 * tmax(R(0), tvf[j]))) * rab1 * ar;
    const R q_mnus = ((lc[j] - hn) * dp[j] + (ab2 * tmax(R(0), tof[j]) + ab3 * tmin(R(0), tvf[j]))) * rab1 * ar;
    rp[j] = tmax(R(0), tmin(R(1), fdiv(q_plus, tmax(spl[j], thshld))));
    rm[j] = tmax(R(0), tmin(R(1), fdiv(q_mnus, tmax(smn[j], thshld))));
  }
  stv<VK>(r_plus + so + c, rp);
  stv<VK>(r_mnus + so + c, rm);
}

// trcadv3: clip the recomputed antidiffusive fluxes, AB3 update, new tracer
template <typename R, int VK>
__global__ void __launch_bounds__(kTB, kTBMin) k_tr_hi(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int t0, int nt, const R* __restrict__ massfx, const R* __restrict__ trc_edg, R* __restrict__ tracr,
    R* __restrict__ trcdp, R* __restrict__ trc_tdcy, const R* __restrict__ delp,
    const R* __restrict__ trold, const R* __restrict__ trcr_lo, const R* __restrict__ r_plus,
    const R* __restrict__ r_mnus, size_t sc) {
  int i, k, tz;
  if (!clt<VK>(g.N, g.L, nt, i, k, tz)) return;
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
  R tri[VK], rpc[VK], rmc[VK], lc[VK], at[VK], sumlo[VK], mx[VK], mn[VK];
  ldv<VK>(to + c, tri);
  ldv<VK>(rp + c, rpc);
  ldv<VK>(rm + c, rmc);
  ldv<VK>(lo + c, lc);
  FOR_V { at[j] = R(0); sumlo[j] = R(0); mx[j] = tmax(tri[j], lc[j]); mn[j] = tmin(tri[j], lc[j]); }
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const int ipx = pr[e];
    const int cx = ipx * L + k;
    R trx[VK], lox[VK];
    ldv<VK>(to + cx, trx);
    ldv<VK>(lo + cx, lox);
    FOR_V { mx[j] = tmax3(mx[j], trx[j], lox[j]); mn[j] = tmin3(mn[j], trx[j], lox[j]); }
    if (e < np) {
      const int own = (i * 6 + e) * L + k, mir = (ipx * 6 + ps[e]) * L + k;
      R mf[VK], mfx[VK], tev[VK], rpx[VK], rmx[VK];
      ldv<VK>(mfn + own, mf);
      ldv<VK>(mfn + mir, mfx);
      ldv<VK>(te + own, tev);
      if (t != 0) {
        R tem[VK];
        ldv<VK>(te + mir, tem);
        FOR_V tev[j] = half * (tev[j] + tem[j]);
      }
      ldv<VK>(rp + cx, rpx);
      ldv<VK>(rm + cx, rmx);
      FOR_V {
        const R hi = mf[j] * tev[j];
        const R lo_ = half * ((mf[j] + tabs(mf[j])) * tri[j] - (mfx[j] + tabs(mfx[j])) * trx[j]);
        sumlo[j] = sumlo[j] + lo_;
        R a = hi - lo_;
        if (a >= R(0)) a = a * tmin(rmc[j], rpx[j]);
        else a = a * tmin(rpc[j], rmx[j]);
        at[j] = at[j] + a;
      }
    }
  }
  const R rar = g.rarea[i];
  R* tc = trc_tdcy + m * s.trab + (size_t)t * 3 * NL;
  R* td = trcdp + m * s.tr + (size_t)t * NL;
  R tof[VK], tvf[VK], tdv[VK], dp[VK], tn[VK], out[VK];
  // -sumlo * rarea is the low-order tendency k_tr_lo stored, rounded alike
  FOR_V tn[j] = mul_rn(-sumlo[j], rar) + (-at[j] * rar);
  stv<VK>(tc + (size_t)nf * NL + c, tn);
  ldv<VK>(tc + (size_t)of * NL + c, tof);
  ldv<VK>(tc + (size_t)vof * NL + c, tvf);
  ldv<VK>(td + c, tdv);
  ldv<VK>(delp + m * s.cell + c, dp);
  FOR_V {
    tdv[j] = tdv[j] + ab1 * tn[j] + ab2 * tof[j] + ab3 * tvf[j];
    const R hx = tmax(R(0), mx[j]), hn = tmax(R(0), mn[j]);
    out[j] = tmax(hn, tmin(hx, fdiv(tdv[j], tmax(thshld, dp[j]))));
  }
  stv<VK>(td + c, tdv);
  stv<VK>(tracr + m * s.tr + (size_t)t * NL + c, out);
}

template <typename R, int VK>
void tracers_fused_vk(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w,
                      R* trc_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx, const R* delp,
                      int tb, bool probe, const ChunkHook* hook) {
  const size_t sc = (size_t)g.N * g.L;
  for (int t0 = 0; t0 < g.T; t0 += w.tchunk) {
    const int nt = (g.T - t0 < w.tchunk) ? g.T - t0 : w.tchunk;
    if (hook && hook->fn) hook->fn(hook->arg, 0, t0, nt);
    dim3 grid(tblocks((long long)g.N * (g.L / VK), tb) * nt, l.members);
    FIM_KBEGIN(l, "k_tr_lo");
    k_tr_lo<R, VK><<<grid, tb, 0, l.stream>>>(g, s, l.sp, t0, nt, massfx, trc_edg, tracr, trcdp, trl_tdcy, delp,
                                               w.trcr_lo, w.s_plus, w.s_mnus, w.trold, sc);
    FIM_KEND(l);
    FIM_KBEGIN(l, "k_tr_lim");
    k_tr_lim<R, VK><<<grid, tb, 0, l.stream>>>(g, s, l.sp, t0, nt, trc_tdcy, delp, w.trold, w.trcr_lo,
                                                w.s_plus, w.s_mnus, w.r_plus, w.r_mnus, sc);
    FIM_KEND(l);
    if (probe) return;  // the first chunk's k_tr_lo and k_tr_lim only
    FIM_KBEGIN(l, "k_tr_hi");
    k_tr_hi<R, VK><<<grid, tb, 0, l.stream>>>(g, s, l.sp, t0, nt, massfx, trc_edg, tracr, trcdp, trc_tdcy,
                                               delp, w.trold, w.trcr_lo, w.r_plus, w.r_mnus, sc);
    FIM_KEND(l);
    if (hook && hook->fn) hook->fn(hook->arg, 1, t0, nt);
  }
}

// Levels per thread: 16-byte accesses where nvl allows; every array offset
// is then a multiple of VK elements, and every base is a cudaMalloc'd field
// (256-byte aligned), checked here.
template <typename R>
int tracer_vk(const Grid<R>& g, std::initializer_list<const void*> ptrs, int want) {
  return pick_vk<R>(g.L, ptrs, want);
}

inline int tracer_tb(int tb) { return tb == 256 ? 256 : 128; }

template <typename R>
void fused_dispatch(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w, R* trc_edg,
                    R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx, const R* delp, bool probe,
                    const ChunkHook* hook = nullptr) {
  const int vk = tracer_vk(g, {trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, w.trcr_lo, w.s_plus,
                               w.s_mnus, w.trold, w.r_plus, w.r_mnus}, w.vk);
  const int tb = tracer_tb(w.tb);
  if (vk == 4)
    tracers_fused_vk<R, (sizeof(R) == 4 ? 4 : 2)>(l, g, s, w, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx,
                                                  delp, tb, probe, hook);
  else if (vk == 2)
    tracers_fused_vk<R, 2>(l, g, s, w, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, tb, probe, hook);
  else
    tracers_fused_vk<R, 1>(l, g, s, w, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, tb, probe, hook);
}

template <typename R>
void launch_tracers_fused(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w,
                          R* trc_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx,
                          const R* delp, const ChunkHook* hook) {
  fused_dispatch<R>(l, g, s, w, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, false, hook);
}

template <typename R, int VK>
void tracer_own_vk(const Launch& l, const Grid<R>& g, const Strides& s, const R* tracr, R* trc_edg, int tb) {
  dim3 grid(tblocks((long long)g.N * (g.L / VK), tb), l.members, g.T - 1);
  FIM_KBEGIN(l, "k_tr_own");
  k_tr_own<R, VK><<<grid, tb, 0, l.stream>>>(g, s, tracr, trc_edg);
  FIM_KEND(l);
}

template <typename R>
void launch_tracer_own(const Launch& l, const Grid<R>& g, const Strides& s, const R* tracr, R* trc_edg, int want,
                       int tb) {
  if (g.T < 2) return;
  const int vk = tracer_vk(g, {tracr, trc_edg}, want);
  tb = tracer_tb(tb);
  if (vk == 4) tracer_own_vk<R, (sizeof(R) == 4 ? 4 : 2)>(l, g, s, tracr, trc_edg, tb);
  else if (vk == 2) tracer_own_vk<R, 2>(l, g, s, tracr, trc_edg, tb);
  else tracer_own_vk<R, 1>(l, g, s, tracr, trc_edg, tb);
}

// Autotuner: time k_tr_own + k_tr_lo + k_tr_lim (first tracer chunk) for
// every (levels per thread, block size) that the layout admits and keep the
// fastest.  The caller provides step parameters whose nf slot the next step
// overwrites, so the probe leaves no state behind.
template <typename R>
int tune_tracers(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w, R* trc_edg,
                 R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx, const R* delp, int* best_vk,
                 int* best_tb, float* best_ms) {
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return (int)cudaGetLastError();
  if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return (int)cudaGetLastError(); }
  Launch lq = l;
  lq.prof = nullptr;
  lq.counter = nullptr;
  float best = 1e30f;
  int rc = 0;
  const int vmax = (int)(16 / sizeof(R));
  for (int tb : {128, 256}) {
    for (int vk = 1; vk <= vmax; vk *= 2) {
      TrcFusedScratch<R> wv = w;
      wv.vk = vk;
      wv.tb = tb;
      if (tracer_vk(g, {trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, w.trcr_lo}, vk) != vk) continue;
      float ms = 0.f;
      for (int rep = 0; rep < 3; rep++) {  // the first repetition warms up
        cudaEventRecord(a, lq.stream);
        launch_tracer_own<R>(lq, g, s, tracr, trc_edg, vk, tb);
        fused_dispatch<R>(lq, g, s, wv, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, true);
        cudaEventRecord(b, lq.stream);
        if (cudaEventSynchronize(b) != cudaSuccess) { rc = (int)cudaGetLastError(); break; }
        float t = 0.f;
        cudaEventElapsedTime(&t, a, b);
        if (rep > 0) ms += t;
      }
      if (rc) break;
      if (ms < best) { best = ms; *best_vk = vk; *best_tb = tb; }
    }
    if (rc) break;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (!rc) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = (int)e;
  }
  if (best_ms) *best_ms = best / 2;
  return rc;
}

#define INSTANTIATE(R)                                                                                        \
  template void launch_tracers_fused<R>(const Launch&, const Grid<R>&, const Strides&,                       \
                                        const TrcFusedScratch<R>&, R*, R*, R*, R*, R*, const R*, const R*,   \
                                        const ChunkHook*);                                                    \
  template void launch_tracer_own<R>(const Launch&, const Grid<R>&, const Strides&, const R*, R*, int, int); \
  template int tune_tracers<R>(const Launch&, const Grid<R>&, const Strides&, const TrcFusedScratch<R>&, R*, \
                               R*, R*, R*, R*, const R*, const R*, int*, int*, float*);
INSTANTIATE(float)
INSTANTIATE(double)

}  // namespace fim
