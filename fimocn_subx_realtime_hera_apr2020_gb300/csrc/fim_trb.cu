// Class-B tracer transport (module_transp3d, transp3d.F90:21-241, and
// module_fct3d, fct3d.F90:4-482): tracers advected on a long time step from
// the time integral of the mass fluxes.
//
//   k_transp1    every step: cumufx += adbash-weighted massfx (transp1)
//   every dtratio steps (checked on the device per member, so one CUDA graph
//   serves every step):
//   k_transp_w   per column, the time-integrated vertical mass flux that
//                closes the continuity equation between dpinit and dp3d;
//                summed bottom-up in the reference's order, so the sign tests
//                fct3d makes on it see the reference's values
//   k_fct3d_col  per (column, class-B tracer): massless-layer fill, piecewise
//                parabolic fit and the vertical tracer flux over the upstream
//                slab (serial in k)
//   k_fct3d_lo   per (level, cell, tracer): donor-cell horizontal fluxes,
//                local bounds, low-order update, limiter ratios
//   k_fct3d_hi   per (level, cell, tracer): limited antidiffusive fluxes
//                (recomputed from the same operands) and the final update
//   k_transp0    cumufx = 0, dpinit = dp3d
#include "fim_internal.h"

namespace fim {

template <typename R> __device__ __forceinline__ R bmax(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R bmin(R a, R b) { return a < b ? a : b; }
template <typename R> __device__ __forceinline__ R babs(R a) { return a < R(0) ? -a : a; }

constexpr int kTB2 = 128;
inline unsigned bblocks(long long n) { return (unsigned)((n + kTB2 - 1) / kTB2); }

// every > 0: act only at steps its % every == 0 of an active member
__device__ __forceinline__ bool member_runs(const StepParams* sp, int every) {
  return sp->active && (every <= 0 || sp->its % every == 0);
}

// transp1 (transp3d.F90:61-72)
template <typename R>
__global__ void __launch_bounds__(kTB2) k_transp1(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    R* __restrict__ cumufx, const R* __restrict__ massfx) {
  const int N = g.N, L = g.L;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * L) return;
  const int i = gid / L, k = gid - i * L;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  cumufx += m * s.edge;
  massfx += m * s.mf;
  const size_t NE = (size_t)N * 6 * L;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const int np = g.nprox[i];
  for (int e = 0; e < np; e++) {
    const size_t o = ((size_t)i * 6 + e) * L + k;
    cumufx[o] = cumufx[o] + ab1 * massfx[(size_t)sp->nf * NE + o] + ab2 * massfx[(size_t)sp->of * NE + o] +
                ab3 * massfx[(size_t)sp->vof * NE + o];
  }
}

// transp2 (transp3d.F90:131-160): w(k) = sum_{j<=k} (dpinit - dpfinl - hordiv*rarea)(j)
template <typename R>
__global__ void __launch_bounds__(kTB2) k_transp_w(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int every, const R* __restrict__ cumufx, const R* __restrict__ dpinit, const R* __restrict__ dpfinl,
    R* __restrict__ w) {
  const int N = g.N, L = g.L;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const size_t m = blockIdx.y;
  sp += m;
  if (!member_runs(sp, every)) return;
  cumufx += m * s.edge; dpinit += m * s.cell; dpfinl += m * s.cell; w += m * s.cell;
  const int np = g.nprox[i];
  const R rar = g.rarea[i];
  R acc = R(0);
  for (int k = 0; k < L; k++) {
    R hordiv = R(0);
    for (int e = 0; e < np; e++) hordiv = hordiv + cumufx[((size_t)i * 6 + e) * L + k];
    const size_t c = (size_t)i * L + k;
    const R vertdv = (dpinit[c] - dpfinl[c]) - hordiv * rar;
    acc = k == 0 ? vertdv : acc + vertdv;
    w[c] = acc;
  }
}

// PPM coefficients of layer k (fct3d.F90:185-214; constant in the end layers)
template <typename R>
__device__ __forceinline__ void ppm(const R* f, const R* to, int k, int L, R& a, R& b, R& c) {
  const R epsil = R(1.e-11);
  if (k == 0 || k == L - 1) { a = f[k]; b = R(0); c = R(0); return; }
  const R dxlft = bmax(epsil, to[k - 1]), dxmid = bmax(epsil, to[k]), dxrgt = bmax(epsil, to[k + 1]);
  const R yl = (dxlft * f[k] + dxmid * f[k - 1]) / (dxlft + dxmid);
  const R yr = (dxrgt * f[k] + dxmid * f[k + 1]) / (dxrgt + dxmid);
  a = R(1.5) * f[k] - R(.25) * (yl + yr);
  b = yr - yl;
  c = R(6) * (R(.5) * (yl + yr) - f[k]);
  if (babs(yr - yl) < R(6) * babs(R(.5) * (yl + yr) - f[k])) {
    if (babs(yr - yl) > R(2) * babs(R(.5) * (yl + yr) - f[k])) {
      if ((yr - yl) * (R(.5) * (yl + yr) - f[k]) > R(0)) {
        a = R(.25) * (R(3) * f[k] + yl);
        c = R(3) * (f[k] - yl);
        b = c;
      } else {
        a = R(.25) * (R(3) * f[k] + yr);
        c = R(3) * (f[k] - yr);
        b = -c;
      }
    } else {
      a = f[k];
      b = R(0);
      c = R(0);
    }
  }
}

// fct3d.F90:131-262 for one (column, tracer): filled field F and vertical
// tracer flux V (V(nvl) = 0), the column staged in shared memory
constexpr int kColB = 64;  // threads of k_fct3d_col; each stages one column of nvl+1 values
template <typename R>
size_t fct3d_col_smem(int L) { return sizeof(R) * kColB * (L + 1); }

template <typename R>
__global__ void __launch_bounds__(kColB) k_fct3d_col(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int every, int t0, int ntrb, const R* __restrict__ tracr, const R* __restrict__ thko, const R* __restrict__ w,
    R* __restrict__ F, R* __restrict__ V) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int N = g.N, L = g.L;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * ntrb) return;
  const int i = gid / ntrb, t = gid - i * ntrb;
  const size_t m = blockIdx.y;
  sp += m;
  if (!member_runs(sp, every)) return;
  const R athird = R(1) / R(3), onemu = R(1.e-6);
  const R* to = thko + m * s.cell + (size_t)i * L;
  const R* wc = w + m * s.cell + (size_t)i * L;
  const R* src = tracr + m * s.tr + ((size_t)(t0 + t) * N + i) * L;
  const size_t so = ((m * ntrb + t) * N + i) * L;
  R* f = reinterpret_cast<R*>(smraw) + (size_t)threadIdx.x * (L + 1);
  for (int k = 0; k < L; k++) f[k] = src[k];
  for (int k = L - 2; k >= 0; k--) f[k] = (f[k] * to[k] + f[k + 1] * onemu) / (to[k] + onemu);
  for (int k = 1; k < L; k++) f[k] = (f[k] * to[k] + f[k - 1] * onemu) / (to[k] + onemu);
  for (int k = 0; k < L; k++) F[so + k] = f[k];
  for (int k = 0; k < L - 1; k++) {
    const R wk = wc[k];
    R slab = onemu, amount = R(0);
    if (wk < R(0)) {
      amount = slab * f[k + 1];
      int kp = k;
      for (;;) {
        kp++;
        if (slab >= -wk) break;
        if (to[kp] > R(0)) {
          R a, b, c;
          ppm(f, to, kp, L, a, b, c);
          const R dslab = bmin(slab + to[kp], -wk) - bmin(slab, -wk);
          const R dx = dslab / to[kp];
          const R fcdx = a + b * R(.5) * (dx - R(1)) + c * (R(.25) - dx * (R(.5) - dx * athird));
          amount = amount + fcdx * dslab;
          slab = slab + dslab;
        }
        if (!(kp < L - 1)) break;
      }
    } else if (wk > R(0)) {
      amount = slab * f[k];
      int kp = k + 1;
      for (;;) {
        kp--;
        if (slab >= wk) break;
        if (to[kp] > R(0)) {
          R a, b, c;
          ppm(f, to, kp, L, a, b, c);
          const R dslab = bmin(slab + to[kp], wk) - bmin(slab, wk);
          const R dx = dslab / to[kp];
          const R fcdx = a + b * R(.5) * (R(1) - dx) + c * (R(.25) - dx * (R(.5) - dx * athird));
          amount = amount + fcdx * dslab;
          slab = slab + dslab;
        }
        if (!(kp > 1)) break;  // fct3d.F90:253: the downward walk stops above layer 1
      }
    }
    V[so + k] = wk * amount / slab;
  }
  V[so + L - 1] = R(0);  // no flux through the top
}

// fct3d.F90:281-355: low-order fluxes, bounds, low-order update, limiter ratios
template <typename R>
__global__ void __launch_bounds__(kTB2) k_fct3d_lo(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int every, int ntrb, const R* __restrict__ u, const R* __restrict__ w, const R* __restrict__ thko,
    const R* __restrict__ thkn, const R* __restrict__ F, const R* __restrict__ V, R* __restrict__ fmx,
    R* __restrict__ fmn, R* __restrict__ flo, R* __restrict__ flp, R* __restrict__ fln) {
  const int N = g.N, L = g.L;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * L) return;
  const int i = gid / L, k = gid - i * L;
  const int t = blockIdx.z;
  const size_t m = blockIdx.y;
  sp += m;
  if (!member_runs(sp, every)) return;
  const R epsil = R(1.e-11), onemu = R(1.e-6), half = R(0.5);
  u += m * s.edge;
  w += m * s.cell; thko += m * s.cell; thkn += m * s.cell;
  const size_t so = (m * ntrb + t) * (size_t)N * L;
  const R* f = F + so;
  const R* vf = V + so;
  const size_t c = (size_t)i * L + k;
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  const int* ps = g.proxs + i * 6;
  const R fi = f[c];
  R mx = fi, mn = fi, hordiv = R(0), totin = R(0), totou = R(0);
  for (int e = 0; e < np; e++) {
    const int ix = pr[e];
    const R ue = u[((size_t)i * 6 + e) * L + k], ux = u[((size_t)ix * 6 + ps[e]) * L + k];
    const R fx = f[(size_t)ix * L + k];
    const R flx = half * ((ue + babs(ue)) * fi - (ux + babs(ux)) * fx);
    const R uan = half * (fi + fx) * ue - flx;
    hordiv = hordiv + flx;
    totin = totin - bmin(R(0), uan);
    totou = totou + bmax(R(0), uan);
    mx = bmax(mx, fx);
    mn = bmin(mn, fx);
  }
  if (k < L - 1 && w[c] < R(0)) {
    mx = bmax(mx, vf[c] / w[c]);
    mn = bmin(mn, vf[c] / w[c]);
  }
  if (k > 0 && w[c - 1] > R(0)) {
    mx = bmax(mx, vf[c - 1] / w[c - 1]);
    mn = bmin(mn, vf[c - 1] / w[c - 1]);
  }
  const R rar = g.rarea[i];
  hordiv = hordiv * rar;
  const R vertdv = k == 0 ? vf[c] : vf[c] - vf[c - 1];
  const R q = fi * thko[c] - hordiv - vertdv;
  const R tn = thkn[c];
  const R amount = bmax(R(0), bmax(mn * tn, bmin(q, mx * tn)));
  const R lo = (fi * onemu + amount) / (onemu + tn);
  fmx[so + c] = mx;
  fmn[so + c] = mn;
  flo[so + c] = lo;
  flp[so + c] = (mx - lo) * tn / (totin + epsil) * rar;
  fln[so + c] = (lo - mn) * tn / (totou + epsil) * rar;
}

// fct3d.F90:368-389: limited antidiffusive fluxes and the final update
template <typename R>
__global__ void __launch_bounds__(kTB2) k_fct3d_hi(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int every, int t0, int ntrb, const R* __restrict__ u, const R* __restrict__ thkn, const R* __restrict__ F,
    const R* __restrict__ fmx, const R* __restrict__ fmn, const R* __restrict__ flo, const R* __restrict__ flp,
    const R* __restrict__ fln, R* __restrict__ tracr) {
  const int N = g.N, L = g.L;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * L) return;
  const int i = gid / L, k = gid - i * L;
  const int t = blockIdx.z;
  const size_t m = blockIdx.y;
  sp += m;
  if (!member_runs(sp, every)) return;
  const R onemu = R(1.e-6), half = R(0.5);
  u += m * s.edge;
  thkn += m * s.cell;
  const size_t so = (m * ntrb + t) * (size_t)N * L;
  const R* f = F + so;
  const size_t c = (size_t)i * L + k;
  const int np = g.nprox[i];
  const int* pr = g.prox + i * 6;
  const int* ps = g.proxs + i * 6;
  const R fi = f[c], flpc = flp[so + c], flnc = fln[so + c];
  R hordiv = R(0);
  for (int e = 0; e < np; e++) {
    const int ix = pr[e];
    const R ue = u[((size_t)i * 6 + e) * L + k], ux = u[((size_t)ix * 6 + ps[e]) * L + k];
    const R fx = f[(size_t)ix * L + k];
    const R flx = half * ((ue + babs(ue)) * fi - (ux + babs(ux)) * fx);
    const R uan = half * (fi + fx) * ue - flx;
    const size_t cx = so + (size_t)ix * L + k;
    const R clip = uan >= R(0) ? bmin(R(1), bmin(flnc, flp[cx])) : bmin(R(1), bmin(flpc, fln[cx]));
    hordiv = hordiv + uan * clip;
  }
  hordiv = hordiv * g.rarea[i];
  const R tn = thkn[c], lo = flo[so + c];
  const R q = lo * tn - hordiv;
  const R amount = bmax(R(0), bmax(fmn[so + c] * tn, bmin(q, fmx[so + c] * tn)));
  tracr[m * s.tr + ((size_t)(t0 + t) * N + i) * L + k] = (lo * onemu + amount) / (onemu + tn);
}

// transp0 (transp3d.F90:36-37)
template <typename R>
__global__ void __launch_bounds__(kTB2) k_transp0(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int every, R* __restrict__ cumufx, const R* __restrict__ dp3d, R* __restrict__ dpinit) {
  const int N = g.N, L = g.L;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * L) return;
  const int i = gid / L, k = gid - i * L;
  const size_t m = blockIdx.y;
  sp += m;
  if (!member_runs(sp, every)) return;
  cumufx += m * s.edge;
#pragma unroll
  for (int e = 0; e < 6; e++) cumufx[((size_t)i * 6 + e) * L + k] = R(0);
  const size_t c = m * s.cell + (size_t)i * L + k;
  dpinit[c] = dp3d[c];
}

template <typename R>
void launch_transp1(const Launch& l, const Grid<R>& g, const Strides& s, R* cumufx, const R* massfx) {
  dim3 grid(bblocks((long long)g.N * g.L), l.members);
  FIM_KBEGIN(l, "k_transp1");
  k_transp1<R><<<grid, kTB2, 0, l.stream>>>(g, s, l.sp, cumufx, massfx);
  FIM_KEND(l);
}

template <typename R>
void launch_transp0(const Launch& l, const Grid<R>& g, const Strides& s, int every, R* cumufx, const R* dp3d,
                    R* dpinit) {
  dim3 grid(bblocks((long long)g.N * g.L), l.members);
  FIM_KBEGIN(l, "k_transp0");
  k_transp0<R><<<grid, kTB2, 0, l.stream>>>(g, s, l.sp, every, cumufx, dp3d, dpinit);
  FIM_KEND(l);
}

template <typename R>
void launch_transp2(const Launch& l, const Grid<R>& g, const Strides& s, const ClassBScratch<R>& w, int every,
                    int ntrb, R* tracr, const R* cumufx, const R* dpinit, const R* dpfinl) {
  if (ntrb <= 0) return;
  dim3 gc(bblocks(g.N), l.members);
  FIM_KBEGIN(l, "k_transp_w");
  k_transp_w<R><<<gc, kTB2, 0, l.stream>>>(g, s, l.sp, every, cumufx, dpinit, dpfinl, w.w);
  FIM_KEND(l);
  dim3 gf((unsigned)(((long long)g.N * ntrb + kColB - 1) / kColB), l.members);
  FIM_KBEGIN(l, "k_fct3d_col");
  k_fct3d_col<R><<<gf, kColB, fct3d_col_smem<R>(g.L), l.stream>>>(g, s, l.sp, every, g.T, ntrb, tracr, dpinit,
                                                                   w.w, w.F, w.V);
  FIM_KEND(l);
  dim3 gs(bblocks((long long)g.N * g.L), l.members, ntrb);
  FIM_KBEGIN(l, "k_fct3d_lo");
  k_fct3d_lo<R><<<gs, kTB2, 0, l.stream>>>(g, s, l.sp, every, ntrb, cumufx, w.w, dpinit, dpfinl, w.F, w.V,
                                           w.fmx, w.fmn, w.flo, w.flp, w.fln);
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_fct3d_hi");
  k_fct3d_hi<R><<<gs, kTB2, 0, l.stream>>>(g, s, l.sp, every, g.T, ntrb, cumufx, dpfinl, w.F, w.fmx, w.fmn,
                                           w.flo, w.flp, w.fln, tracr);
  FIM_KEND(l);
}

template <typename R>
int prepare_classb(int L) {
  const size_t bytes = fct3d_col_smem<R>(L);
  if (bytes <= 48 * 1024) return 0;
  const cudaError_t e =
      cudaFuncSetAttribute(k_fct3d_col<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return e == cudaSuccess ? 0 : (int)e;
}

#define INSTANTIATE(R)                                                                                        \
  template void launch_transp1<R>(const Launch&, const Grid<R>&, const Strides&, R*, const R*);              \
  template void launch_transp0<R>(const Launch&, const Grid<R>&, const Strides&, int, R*, const R*, R*);    \
  template void launch_transp2<R>(const Launch&, const Grid<R>&, const Strides&, const ClassBScratch<R>&,   \
                                  int, int, R*, const R*, const R*, const R*);                             \
  template int prepare_classb<R>(int);
INSTANTIATE(float)
INSTANTIATE(double)

}  // namespace fim
