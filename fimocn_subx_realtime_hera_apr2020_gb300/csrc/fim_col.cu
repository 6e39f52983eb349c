// Column kernels of the FIM dynamics step: hybgen (regrid_1d, dffusn_lev,
// remap_1d with restp_1d, equilb, inflate, pcwise), hystat, globsum.
//
// hybgen's column logic is serial in k with data-dependent branches, so it
// runs one thread per column over per-thread column arrays; the 1-ring
// interface smoothing between regrid and remap is a (level, cell) stencil.
// hystat's bottom-up Montgomery/geopotential recursion is a warp scan in FP64.
// globsum accumulates per thread (FP64, or float-float compensated sums in the
// FP32 build, whose error is that of an FP64 sum) and reduces per block into a
// deterministic partial buffer.
#include <cstdint>

#include "fim_internal.h"

namespace fim {

template <typename R> __device__ __forceinline__ R cmax(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R cmin(R a, R b) { return a < b ? a : b; }
template <typename R> __device__ __forceinline__ R cabs(R a) { return a < R(0) ? -a : a; }

constexpr int kColBlock = 128;
constexpr int kBlock2 = 256;
inline unsigned nblocks(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// ---------------------------------------------------------------- hybgen --
// restp_1d (hybgen.F90:792-890).  The running minimum oldth is formed in
// place in thold (the caller's column, not read again).  The new theta
// column is targt except its two end layers (hybgen.F90:832-834), so it is
// not stored: th0 and thL are its ends and tn(k) its layer k.
template <typename R, int ML>
__device__ void restp_1d(R* thold, const R* pkold, int kold, R* pknew, const R* targt, int knew, int* bad) {
  R* oldth = thold;
  for (int k = kold; k >= 2; k--) oldth[k - 2] = cmin(oldth[k - 1], oldth[k - 2]);
  const R th0 = cmin(cmin(oldth[0], oldth[kold - 1]), targt[0]);
  const R thL = cmax(cmax(oldth[0], oldth[kold - 1]), targt[knew - 1]);
  auto tn = [&](int k) -> R { return k == 0 ? th0 : k == knew - 1 ? thL : targt[k]; };
  pknew[0] = pkold[0];
  pknew[knew] = pkold[kold];
  R colint = R(0), colscl = R(0), cloutt = R(0);
  for (int k = 0; k < kold; k++) {
    colint = colint + oldth[k] * (pkold[k + 1] - pkold[k]);
    colscl = colscl + cabs(oldth[k] * (pkold[k + 1] - pkold[k]));
  }
  int ko = 0;
  R tk = th0;
  for (int k = 0; k < knew - 1; k++) {
    const R tk1 = tn(k + 1);
    R pinteg = R(0), tha, thb = tk;
    for (;;) {
      tha = thb;
      thb = cmin(tk1, cmax(tk, oldth[ko]));
      pinteg = pinteg + pkold[ko] * (thb - tha);
      if (oldth[ko] < tk1) {
        if (ko < kold - 1) { ko++; continue; }
        tha = thb;
        thb = tk1;
        pinteg = pinteg + pkold[kold] * (thb - tha);
      }
      break;
    }
    pknew[k + 1] = pknew[k];
    if (tk1 > tk) pknew[k + 1] = pinteg / (tk1 - tk);
    cloutt = cloutt + tk * (pknew[k + 1] - pknew[k]);
    tk = tk1;
  }
  cloutt = cloutt + thL * (pknew[knew] - pknew[knew - 1]);
  if (cabs(cloutt - colint) > cmax(R(1.e-33), col_tol<R>(1.e-6) * colscl)) *bad = 1;
}

// equilb scenario 1 (hybgen.F90:1316-1363); in place on pres
template <typename R>
__device__ void equilb(const R* thet, R* pnew, int kk, R slak) {
  const R thin = R(kRd) / R(kP1000);
  for (int k = 3; k <= kk - 2; k++) {
    if (pnew[k - 3] > pnew[0] - thin) continue;
    const R dp1 = pnew[k - 3] - pnew[k - 2];
    const R dp2 = pnew[k - 2] - pnew[k - 1];
    const R dp3 = pnew[k - 1] - pnew[k];
    const R dp4 = pnew[k] - pnew[k + 1];
    const R dp5 = pnew[k + 1] - pnew[k + 2];
    const R th2 = thet[k - 2], th3 = thet[k - 1], th4 = thet[k];
    if (dp2 > dp1 && dp4 > dp5) {
      const R goal = R(.5) * (dp3 + cmin(dp2, dp4));
      if (dp2 > goal && dp4 > goal) {
        R dis3 = cmin(dp2 - goal, goal - dp3) * slak;
        R dis4 = cmin(dp4 - goal, goal - dp3) * slak;
        if (th3 > th2 && th4 > th3) {
          const R ratio = (th4 - th3) / (th3 - th2);
          if (ratio > R(1)) dis4 = dis3 / ratio;
          else dis3 = dis4 * ratio;
        }
        pnew[k - 1] = pnew[k - 1] + dis3;
        pnew[k] = pnew[k] - dis4;
      }
    }
  }
}

template <typename R>
__device__ __forceinline__ R cushn(R a, R b) {
  const R m = cmin(a, R(2) * b);
  return R(.25) * (m * m) / b + cmax(a, R(2) * b) - b;
}

// inflate (hybgen.F90:893-1007)
template <typename R>
__device__ void inflate(const Knobs& kn, const R* dpsig, int L, R psurf, R* exner) {
  const R thin = R(kRd) / R(kP1000);
  const R rd = R(kRd), p1000 = R(kP1000), cp = R(kCp);
  R dpsum = R(0);
  const R extop = cp * pow(R(kn.ptop) / p1000, rd / cp);
  const R top = R(.2);
  const R shrink = cmin(R(1), (psurf / p1000 - top) / (R(1) - top));
  int last = 1;
  for (int k = 1; k <= L - 1; k++) {
    R dp0 = rd * dpsig[k - 1] / p1000 * shrink;
    dpsum = dpsum + dp0;
    const R exold = exner[k];
    if (k <= kn.kbl) {
      last = k + 1;
      exner[k] = exner[k - 1] - dp0;
    } else {
      if (k > last) {
        dp0 = dp0 / cmin(R(10), R(1.25) * ldexp(R(1), k - last));
        dp0 = cmax(dp0, rd * R(100) / p1000);
      }
      const R dp1 = cushn(cmax(R(0), exner[k - 1] - cmin(exold, exner[0] - dpsum)), dp0);
      if (exner[k - 1] - dp1 < exold - thin) {
        if (k == last) last = k + 1;
        exner[k] = cmax(extop, exner[k - 1] - dp1);
      }
    }
  }
  if (kn.thktop > 0.) {
    const R thk = R(kn.thktop);
    for (int k = L; k >= 2; k--) {
      R q = exner[k - 1] / cp;
      q = q * q * sqrt(q);
      const R dk = R(.25) * R(L - k);
      const R dp0 = rd * thk / p1000 * (R(1) / (R(1) + dk * dk)) / q;
      const R exold = exner[k - 1];
      const R dp1 = cushn(cmax(R(0), exold - exner[k]), dp0);
      if (exner[k] + dp1 > exold + thin) exner[k - 1] = exner[k] + dp1;
      if (exner[k - 1] < exner[k - 2] - dp0) break;
    }
  }
}

// regrid_1d (hybgen.F90:207-512, hybrid-isentropic branch) for one column:
// thcol (L) and excol (L+1) are overwritten; excol ends as the new Exner fcn.
template <typename R, int ML>
__device__ void regrid_1d(const Knobs& kn, const R* targt, const R* dpsig, int L, int its, R* thcol, R* excol,
                          R prcol0, int* bad) {
  const R thin = R(kRd) / R(kP1000), tolrnce = R(0.001), dffudt = R(.1);
  const R eqlb_slak = R(.1) * R(its) / (R(10) + R(its));
  // one local work array: the column's own excol serves as exwrk, thcol as
  // restp_1d's oldth, the new theta column is targt but for its ends (which
  // equilb does not read), and the heat fluxes are formed as the update runs
  R exnew[ML + 1];
  for (int k = 0; k < L; k++)
    if (excol[k] < excol[k + 1] - thin) excol[k + 1] = excol[k];
  for (int k = L - 2; k >= 0; k--) thcol[k] = cmin(thcol[k], thcol[k + 1]);
  R* exwrk = excol;
  const R tt = targt[L - 1];
  for (int k = L; k >= 2; k--) {
    if (thcol[k - 1] <= tt + tolrnce) break;
    const R wgt1 = cmax(R(0), exwrk[k - 2] - exwrk[k - 1]);
    const R wgt2 = cmax(thin, exwrk[k - 1] - exwrk[k]);
    const R tr = (thcol[k - 2] * wgt1 + thcol[k - 1] * wgt2) / (wgt1 + wgt2);
    if (tr > tt - tolrnce) {
      exwrk[k - 1] = exwrk[L];
      for (int k1 = k - 1; k1 <= L; k1++) thcol[k1 - 1] = tr;
    } else {
      exwrk[k - 1] = cmin(exwrk[k - 2], cmax(exwrk[k], (exwrk[k - 1] * (thcol[k - 1] - thcol[k - 2]) +
                                                         exwrk[k] * (tt - thcol[k - 1])) /
                                                            (tt - thcol[k - 2])));
      for (int k1 = k; k1 <= L; k1++) thcol[k1 - 1] = tt;
      break;
    }
  }
  restp_1d<R, ML>(thcol, exwrk, L, exnew, targt, L, bad);
  const R grv = R(kGrvity);
  // heatfx(j) of hybgen.F90's heat diffusion, from the work copy only (zero
  // at j = 0 and nvl-1)
  auto heatfx = [&](int j) -> R {
    R h = R(0);
    if (j >= 1 && j <= L - 2 && exwrk[j] < exwrk[0] - R(.01) && exwrk[j + 1] > exwrk[L] + R(.01)) {
      const R cnv = grv / targt[j];
      h = dffudt * cnv * cnv * R(.5) * (targt[j + 1] - targt[j - 1]) / cmax(R(.03) * cnv, exwrk[j] - exwrk[j + 1]);
    }
    return h;
  };
  for (int iter = 1; iter <= 3; iter++) {
    for (int k = 0; k <= L; k++) exwrk[k] = exnew[k];
    R hprev = R(0);  // heatfx(k - 1)
    for (int k = 1; k <= L - 1; k++) {
      const R hcur = heatfx(k);
      if (exwrk[k] < exwrk[0] - R(.01) && exwrk[k] > exwrk[L] + R(.01))
        exnew[k] = cmax(exwrk[k + 1], cmin(exwrk[k - 1], exwrk[k] + (hcur - hprev) / (targt[k] - targt[k - 1])));
      hprev = hcur;
    }
    bool event = false;
    for (int k = 2; k <= L + 1; k++)
      if (exnew[k - 1] > exnew[k - 2] + thin) event = true;
    if (!event) break;
  }
  equilb<R>(targt, exnew, L, eqlb_slak);  // reads layers 1..nvl-2 only
  inflate<R>(kn, dpsig, L, prcol0, exnew);
  for (int k = 0; k <= L; k++) excol[k] = exnew[k];
}

// pcwise (hybgen.F90:1010-1279): 1-D PCM/PLM/PPM remap of yold from cell
// boundaries xold to xnew.  Returns true when the column-integral check fails.
template <typename R, int ML>
__device__ bool pcwise(int kk, const R* xold, const R* yold, const R* xnew, R* ynew, int miglim, int remap_optn) {
  R delz[ML + 1], fco[ML], fcn[ML], vertfx[ML + 1], fldnew[ML], a[ML], b[ML], cc[ML];
  const R athird = R(1) / R(3), small = R(1.e-22);
  const bool flip = !(xold[0] < xold[kk]);
  for (int k = 0; k <= kk; k++) delz[k] = flip ? (-xnew[k]) - (-xold[k]) : xnew[k] - xold[k];
  for (int k = 0; k < kk; k++) {
    fco[k] = flip ? cmax(R(0), (-xold[k + 1]) - (-xold[k])) : cmax(R(0), xold[k + 1] - xold[k]);
    fcn[k] = flip ? cmax(R(0), (-xnew[k + 1]) - (-xnew[k])) : cmax(R(0), xnew[k + 1] - xnew[k]);
  }
  R bfore = R(0), colscl = R(0);
  for (int k = 0; k < kk; k++) {
    bfore = bfore + yold[k] * fco[k];
    colscl = colscl + cabs(yold[k] * fco[k]);
  }
  for (int k = 0; k < kk; k++) fldnew[k] = yold[k];
  for (int k = kk - 2; k >= 0; k--) fldnew[k] = (fldnew[k] * fco[k] + fldnew[k + 1] * small) / (fco[k] + small);
  for (int k = 1; k < kk; k++) fldnew[k] = (fldnew[k] * fco[k] + fldnew[k - 1] * small) / (fco[k] + small);
  a[0] = fldnew[0]; b[0] = R(0); cc[0] = R(0);
  a[kk - 1] = fldnew[kk - 1]; b[kk - 1] = R(0); cc[kk - 1] = R(0);
  for (int k = 1; k < kk - 1; k++) {
    if (remap_optn == 1) {
      a[k] = fldnew[k]; b[k] = R(0); cc[k] = R(0);
    } else if (remap_optn == 2) {
      a[k] = fldnew[k];
      b[k] = R(0);
      if (fldnew[k] <= cmin(fldnew[k - 1], fldnew[k + 1]) || fldnew[k] >= cmax(fldnew[k - 1], fldnew[k + 1])) {
        b[k] = R(0);
      } else if ((fldnew[k + 1] - fldnew[k - 1]) * (fldnew[k - 1] + fldnew[k + 1] - R(2) * fldnew[k]) > R(0)) {
        b[k] = fldnew[k] - fldnew[k - 1];
      } else {
        b[k] = fldnew[k + 1] - fldnew[k];
      }
      cc[k] = R(0);
    } else {
      const R yl = (cmax(small, fco[k - 1]) * fldnew[k] + cmax(small, fco[k]) * fldnew[k - 1]) /
                   (cmax(small, fco[k - 1]) + cmax(small, fco[k]));
      const R yr = (cmax(small, fco[k + 1]) * fldnew[k] + cmax(small, fco[k]) * fldnew[k + 1]) /
                   (cmax(small, fco[k + 1]) + cmax(small, fco[k]));
      a[k] = R(1.5) * fldnew[k] - R(.25) * (yl + yr);
      b[k] = yr - yl;
      cc[k] = R(6) * (R(.5) * (yl + yr) - fldnew[k]);
      if (cabs(yr - yl) < R(6) * cabs(R(.5) * (yl + yr) - fldnew[k])) {
        if (cabs(yr - yl) > R(2) * cabs(R(.5) * (yl + yr) - fldnew[k])) {
          if ((yr - yl) * (R(.5) * (yl + yr) - fldnew[k]) > R(0)) {
            a[k] = R(.25) * (R(3) * fldnew[k] + yl);
            cc[k] = R(3) * (fldnew[k] - yl);
            b[k] = cc[k];
          } else {
            a[k] = R(.25) * (R(3) * fldnew[k] + yr);
            cc[k] = R(3) * (fldnew[k] - yr);
            b[k] = -cc[k];
          }
        } else {
          a[k] = fldnew[k]; b[k] = R(0); cc[k] = R(0);
        }
      }
    }
  }
  for (int k = 1; k < kk; k++) {
    R slab = R(0), amount = R(0);
    vertfx[k] = R(0);
    const R dz = delz[k];
    if (miglim == 1) {
      if (dz > R(0)) {
        const int lyr = k;
        if (fco[lyr] > R(0)) {
          const R dslab = cmin(slab + fco[lyr], dz) - cmin(slab, dz);
          const R dx = dslab / fco[lyr];
          const R fcdx = a[lyr] + b[lyr] * R(.5) * (dx - R(1)) + cc[lyr] * (R(.25) - dx * (R(.5) - dx * athird));
          amount = amount + fcdx * dslab;
          slab = slab + dslab;
        }
      } else if (dz < R(0)) {
        const int lyr = k - 1;
        if (fco[lyr] > R(0)) {
          const R dslab = cmin(slab + fco[lyr], -dz) - cmin(slab, -dz);
          const R dx = dslab / fco[lyr];
          const R fcdx = a[lyr] + b[lyr] * R(.5) * (R(1) - dx) + cc[lyr] * (R(.25) - dx * (R(.5) - dx * athird));
          amount = amount + fcdx * dslab;
          slab = slab + dslab;
        }
      }
    } else {
      if (dz > R(0)) {
        int lyr = k - 1;
        for (;;) {
          lyr = lyr + 1;
          if (slab >= dz) break;
          if (fco[lyr] > R(0)) {
            const R dslab = cmin(slab + fco[lyr], dz) - cmin(slab, dz);
            const R dx = dslab / fco[lyr];
            const R fcdx = a[lyr] + b[lyr] * R(.5) * (dx - R(1)) + cc[lyr] * (R(.25) - dx * (R(.5) - dx * athird));
            amount = amount + fcdx * dslab;
            slab = slab + dslab;
          }
          if (!(lyr < kk - 1)) break;
        }
      } else if (dz < R(0)) {
        int lyr = k;
        for (;;) {
          lyr = lyr - 1;
          if (slab >= -dz) break;
          if (fco[lyr] > R(0)) {
            const R dslab = cmin(slab + fco[lyr], -dz) - cmin(slab, -dz);
            const R dx = dslab / fco[lyr];
            const R fcdx = a[lyr] + b[lyr] * R(.5) * (R(1) - dx) + cc[lyr] * (R(.25) - dx * (R(.5) - dx * athird));
            amount = amount + fcdx * dslab;
            slab = slab + dslab;
          }
          if (!(lyr > 0)) break;
        }
      }
    }
    if (slab != R(0)) vertfx[k] = -dz * amount / slab;
  }
  vertfx[0] = R(0);
  vertfx[kk] = R(0);
  R after = R(0);
  for (int k = 0; k < kk; k++) {
    const R amount = fldnew[k] * fco[k] - (vertfx[k + 1] - vertfx[k]);
    ynew[k] = (amount + fldnew[k] * small) / (fcn[k] + small);
    after = after + amount;
  }
  return cabs(bfore - after) > cmax(R(1.e-33), col_tol<R>(1.e-11) * colscl);
}

// A warp's 32 columns (lane = column) move between global memory and the
// lanes' column arrays through a 32 x 33 shared tile, 32 levels at a time, so
// the global accesses run along k (128-byte rows) rather than one column per
// lane.  n values of column i0 + lane start at src + (i0 + lane) * stride.
template <typename R>
__device__ __forceinline__ void columns_in(const R* __restrict__ src, size_t stride, int n, int ncol, int i0,
                                           int lane, R (*tile)[33], R* col) {
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int kk = c0 + lane;
#pragma unroll 8
    for (int r = 0; r < 32; r++)
      if (r < ncol && kk < n) tile[r][lane] = src[(size_t)(i0 + r) * stride + kk];
    __syncwarp();
    const int m = n - c0 < 32 ? n - c0 : 32;
    if (lane < ncol)
      for (int q = 0; q < m; q++) col[c0 + q] = tile[lane][q];
    __syncwarp();
  }
}
template <typename R>
__device__ __forceinline__ void columns_out(R* __restrict__ dst, size_t stride, int n, int ncol, int i0, int lane,
                                            R (*tile)[33], const R* col) {
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int m = n - c0 < 32 ? n - c0 : 32;
    if (lane < ncol)
      for (int q = 0; q < m; q++) tile[lane][q] = col[c0 + q];
    __syncwarp();
    const int kk = c0 + lane;
#pragma unroll 8
    for (int r = 0; r < 32; r++)
      if (r < ncol && kk < n) dst[(size_t)(i0 + r) * stride + kk] = tile[r][lane];
    __syncwarp();
  }
}

template <typename R, int ML>
__global__ void __launch_bounds__(kColBlock) k_regrid(Grid<R> g, Strides s, Knobs kn,
    const StepParams* __restrict__ sp, const R* __restrict__ targt, const R* __restrict__ tr3d,
    const R* __restrict__ ex3d, const R* __restrict__ pr3d, R* __restrict__ exsmo, int* __restrict__ flags,
    int bnd) {
  __shared__ R tiles[kColBlock / 32][32][33];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int i0 = blockIdx.x * blockDim.x + wib * 32;
  const int N = g.N, L = g.L, L1 = L + 1;
  if (i0 >= N) return;
  const int ncol = N - i0 < 32 ? N - i0 : 32;
  const int i = i0 + lane;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active || (bnd && sp->its <= 1)) return;
  tr3d += m * s.tr; ex3d += m * s.intf; pr3d += m * s.intf; exsmo += m * s.intf;
  R thcol[ML], excol[ML + 1];
  columns_in(tr3d, (size_t)L, L, ncol, i0, lane, tiles[wib], thcol);
  columns_in(ex3d, (size_t)L1, L1, ncol, i0, lane, tiles[wib], excol);
  int bad = 0;
  if (lane < ncol)
    regrid_1d<R, ML>(kn, targt, g.dpsig, L, sp->its - bnd, thcol, excol, pr3d[(size_t)i * L1], &bad);
  columns_out(exsmo, (size_t)L1, L1, ncol, i0, lane, tiles[wib], excol);
  if (bad) atomicOr(flags + m, kFlagColumnIntegral);
}

// dffusn_lev (dffusn.F90:37-58 with dffusn_lev.exe) on interfaces kbl+2..nvl,
// out of place so every cell reads the unsmoothed neighbours.  A thread takes
// kDffK interfaces of one cell, kg + j*ng (ng = ceil((nvl+1)/kDffK)), so each
// load of a warp stays contiguous and the neighbour values of all its
// interfaces are in flight together (all six prox slots hold valid cells; a
// pentagon's slot 5 is left out of the sum).
constexpr int kDffK = 4;
template <typename R>
__global__ void __launch_bounds__(kBlock2) k_dffusn_lev(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int bnd, int k1, int k2, const R* __restrict__ fld, R* __restrict__ out) {
  const int N = g.N, L1 = g.L + 1;
  const int ng = (L1 + kDffK - 1) / kDffK;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * ng) return;
  const int i = gid / ng, kg = gid - i * ng;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active || (bnd && sp->its <= 1)) return;
  fld += m * s.intf; out += m * s.intf;
  const int np = g.nprox[i];
  const R* col = fld + (size_t)i * L1;
  const R* nb[6];
#pragma unroll
  for (int e = 0; e < 6; e++) nb[e] = fld + (size_t)g.prox[i * 6 + e] * L1;
  R val[kDffK], x[kDffK][6];
#pragma unroll
  for (int j = 0; j < kDffK; j++) {
    const int k = kg + j * ng;
    const bool act = k < L1;
    const int kk = act ? k : 0;
    val[j] = col[kk];
#pragma unroll
    for (int e = 0; e < 6; e++) x[j][e] = nb[e][kk];
  }
  const R rar = g.rarea[i];
#pragma unroll
  for (int j = 0; j < kDffK; j++) {
    const int k = kg + j * ng;
    if (k >= L1) continue;
    R v = val[j];
    if (k >= k1 && k <= k2) {
      R flxdv = R(0);
#pragma unroll
      for (int e = 0; e < 6; e++)
        if (e < np) flxdv = flxdv + (v - x[j][e]) * g.sideln[i * 6 + e];
      const R factor = -g.smoo[k] * rar;
      v = v + flxdv * factor;
    }
    out[(size_t)i * L1 + k] = v;
  }
}

// remap_1d (hybgen.F90:515-789) followed by the hybgen bookkeeping
// (hybgen.F90:189-191): new u, v, tracers, Exner, pressure, thickness, sdot.
template <typename R, int ML>
__global__ void __launch_bounds__(kColBlock) k_remap(Grid<R> g, Strides s, Knobs kn,
    const StepParams* __restrict__ sp, const R* __restrict__ targt, const R* __restrict__ exsmo,
    R* __restrict__ us3d, R* __restrict__ vs3d, R* __restrict__ tr3d, R* __restrict__ sdot,
    R* __restrict__ ex3d, R* __restrict__ dp3d, R* __restrict__ pr3d, int* __restrict__ flags, int bnd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int N = g.N, L = g.L, L1 = L + 1;
  if (i >= N) return;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active || (bnd && sp->its <= 1)) return;
  const int T = min(g.T, sp->ntr);
  exsmo += m * s.intf; us3d += m * s.cell; vs3d += m * s.cell; tr3d += m * s.tr; sdot += m * s.intf;
  ex3d += m * s.intf; dp3d += m * s.cell; pr3d += m * s.intf;
  const int its = sp->its - bnd;
  const R cp = R(kCp), rd = R(kRd), p1000 = R(kP1000), small = R(1.e-6);
  R exold[ML + 1], exnew[ML + 1], prcol[ML + 1], prnew[ML + 1], pk1col[ML + 1], pk1new[ML + 1];
  R yold[ML], ynew[ML], dpcol[ML];
  for (int k = 0; k <= L; k++) {
    exold[k] = ex3d[(size_t)i * L1 + k];
    prcol[k] = pr3d[(size_t)i * L1 + k];
    exnew[k] = exsmo[(size_t)i * L1 + k];
  }
  for (int k = 0; k <= L; k++) pk1col[k] = exold[k] * prcol[k] / cp;
  if (kn.intfc_smooth > 0.) inflate<R>(kn, g.dpsig, L, prcol[0], exnew);
  if (its > 0) {
    const R sl = R(kn.slak);
    for (int k = 0; k <= L; k++) exnew[k] = sl * exnew[k] + (R(1) - sl) * exold[k];
  }
  const int mg = kn.miglim;
  if (mg > 0) {
    for (int k = 1 + mg; k <= L + 1 - mg; k++)
      exnew[k - 1] = cmax(R(.0001) * exold[k - 1] + R(.9999) * exold[k - 1 + mg],
                          cmin(R(.0001) * exold[k - 1] + R(.9999) * exold[k - 1 - mg], exnew[k - 1]));
    for (int k = 2; k <= mg; k++) {
      exnew[k - 1] = cmin(exold[0], exnew[k - 1]);
      exnew[L - k] = cmax(exold[L], exnew[L - k]);
    }
  }
  for (int k = L; k >= 0; k--) prnew[k] = p1000 * pow(exnew[k] / cp, cp / rd);
  for (int k = 0; k < L; k++) dpcol[k] = prnew[k] - prnew[k + 1];
  for (int k = 0; k <= L; k++) pk1new[k] = exnew[k] * prnew[k] / cp;
  prnew[L] = prcol[L];
  pk1new[L] = pk1col[L];
  prnew[0] = prcol[0];
  pk1new[0] = pk1col[0];
  bool bad = false;
  // u and v
  for (int f = 0; f < 2; f++) {
    R* col = (f == 0 ? us3d : vs3d) + (size_t)i * L;
    for (int k = 0; k < L; k++) yold[k] = col[k];
    bad |= pcwise<R, ML>(L, prcol, yold, prnew, ynew, mg, kn.remap_optn);
    for (int k = 0; k < L; k++) col[k] = ynew[k];
  }
  // tracers 2..ntra in pressure, with the optional massless-layer fill
  for (int t = 1; t < T; t++) {
    R* col = tr3d + ((size_t)t * N + i) * L;
    for (int k = 0; k < L; k++) yold[k] = col[k];
    bad |= pcwise<R, ML>(L, prcol, yold, prnew, ynew, mg, kn.remap_optn);
    if (kn.thktop == 0.) {
      for (int k = 3; k <= L; k++) {
        const R qq = R(1) / (dpcol[k - 1] + small);
        ynew[k - 1] = (ynew[k - 1] * dpcol[k - 1] + ynew[k - 2] * small) * qq;
      }
    }
    for (int k = 0; k < L; k++) col[k] = ynew[k];
  }
  // potential temperature in p^(kappa+1), then the target redistribution
  {
    R* col = tr3d + (size_t)i * L;
    for (int k = 0; k < L; k++) yold[k] = col[k];
    bad |= pcwise<R, ML>(L, pk1col, yold, pk1new, ynew, mg, kn.remap_optn);
    for (int k = L; k >= 3; k--) {
      const R dplo = cmax(pk1new[k - 2] - pk1new[k - 1], pk1new[0] * small);
      const R dpup = cmax(pk1new[k - 1] - pk1new[k], pk1new[0] * small);
      const R tha = ynew[k - 2], thb = ynew[k - 1];
      const R devilo = (tha - targt[k - 2]) * dplo;
      const R deviup = (thb - targt[k - 1]) * dpup;
      if (deviup > R(0) && devilo < R(0)) {
        ynew[k - 2] = tha + cmin(deviup, -devilo) / dplo;
        ynew[k - 1] = thb - cmin(deviup, -devilo) / dpup;
      } else if (deviup < R(0) && devilo > R(0)) {
        ynew[k - 2] = tha - cmin(devilo, -deviup) / dplo;
        ynew[k - 1] = thb + cmin(devilo, -deviup) / dpup;
      }
    }
    {
      R colin = R(0), clout = R(0), colscl = R(0);
      for (int k = 0; k < L; k++) {
        colin = colin + yold[k] * (pk1col[k] - pk1col[k + 1]);
        clout = clout + ynew[k] * (pk1new[k] - pk1new[k + 1]);
        colscl = colscl + cabs(yold[k] * (pk1col[k] - pk1col[k + 1]));
      }
      if (cabs(clout - colin) > cmax(R(1.e-33), col_tol<R>(2.e-6) * colscl)) bad = true;
    }
    for (int k = 0; k < L; k++) col[k] = ynew[k];
  }
  for (int k = 0; k < L; k++)
    if (exnew[k] < exnew[k + 1]) exnew[k + 1] = exnew[k];
  for (int k = 0; k <= L; k++) {
    sdot[(size_t)i * L1 + k] = exnew[k] - exold[k];
    ex3d[(size_t)i * L1 + k] = exnew[k];
    pr3d[(size_t)i * L1 + k] = prnew[k];
  }
  for (int k = 0; k < L; k++) dp3d[(size_t)i * L + k] = dpcol[k];
  if (bad) atomicOr(flags + m, kFlagColumnIntegral);
}

// ------------------------------------------ remap, warp per column, lane = levels --
// remap_1d (hybgen.F90:515-700) for the default knobs: PLM pcwise with
// one-layer migration (remap_optn = 2, miglim = 1).
//  k_inflate: inflate, the one serial recursion of the column set-up, lane =
//             column over 32 columns per warp staged in shared memory;
//  k_remap_v: each warp runs kColsPerWarp consecutive columns.  Lane l holds
//             levels l*VL .. l*VL+VL-1 of the field in hand (u, v, tracers
//             2..ntra in pressure, theta in p^(kappa+1)), so a field's column
//             is one contiguous read and write.  The three interface arrays
//             and the fields of the warp's columns stream through a ring of
//             shared-memory slots filled by cp.async several items ahead,
//             across column boundaries.
// Given the filled values, pcwise's flux form is level-parallel: PLM slopes
// and interface fluxes take the neighbouring levels from the adjacent lanes.
// The massless-layer fills of pcwise and remap_1d's tracer fill are
// first-order linear recurrences x(k) = a(k) x(k-+1) + b(k): each lane
// composes the maps of its levels, a warp scan of the composed maps gives the
// value entering each lane, and the lane runs the recurrence in the
// reference's form over its own levels.  The pairwise theta redistribution
// toward the target (hybgen.F90:648-667) is a nonlinear sweep over the
// column: it runs after the warp's last column with lane = column.
// With one-layer migration the donor layer, slab width and dx of every
// interface depend on the coordinate only, so they are formed once per column
// and held in registers; divisions by the coordinate thicknesses (fco +
// small, fcn + small) become products with reciprocals.  Results differ from
// the serial pcwise by rounding.
constexpr int kWarpsInflate = 4;
constexpr int kWarpsRemapV = 4;
constexpr int kColsPerWarp = 8;

// pcwise's massless-layer fill moves y(k) by (y(k+-1) - y(k)) * 1e-22 / fco(k):
// below the rounding of either precision unless fco(k) is under ~1e-4.
template <typename R>
__device__ __forceinline__ R fill_thin() { return R(1.2e-4); }

// PLM slope of a layer from its filled value f and its neighbours' fm, fp
template <typename R>
__device__ __forceinline__ R plm_slope(R fm, R f, R fp) {
  const R b = ((fp - fm) * (fm + fp - R(2) * f) > R(0)) ? f - fm : fp - f;
  return (f <= cmin(fm, fp) || f >= cmax(fm, fp)) ? R(0) : b;
}

// asynchronous global -> shared copy of B = 4, 8 or 16 bytes
template <int B>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// sum over a segment of W lanes (the lanes of one column)
template <typename R, int W = 32>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int off = W / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off, W);
  return v;
}


// Value entering each lane of a recurrence x <- a x + b whose per-lane
// composed map is (a, b): from the lanes below (up) or above (down); the
// first lane of the sweep receives 0 (its own map is constant there).
// (lane: the lane within its W-lane segment)
template <typename R, int W = 32>
__device__ __forceinline__ R affine_entry_up(int lane, R a, R b) {
#pragma unroll
  for (int off = 1; off < W; off <<= 1) {
    const R ao = __shfl_up_sync(0xffffffffu, a, off, W), bo = __shfl_up_sync(0xffffffffu, b, off, W);
    if (lane >= off) { b = a * bo + b; a = a * ao; }
  }
  const R e = __shfl_up_sync(0xffffffffu, b, 1, W);
  return lane == 0 ? R(0) : e;
}
template <typename R, int W = 32>
__device__ __forceinline__ R affine_entry_down(int lane, R a, R b) {
#pragma unroll
  for (int off = 1; off < W; off <<= 1) {
    const R ao = __shfl_down_sync(0xffffffffu, a, off, W), bo = __shfl_down_sync(0xffffffffu, b, off, W);
    if (lane + off < W) { b = a * bo + b; a = a * ao; }
  }
  const R e = __shfl_down_sync(0xffffffffu, b, 1, W);
  return lane == W - 1 ? R(0) : e;
}

// shared memory of one warp: the copy ring (an item is, for each of the H
// columns in hand, the three interface arrays or three fields), the column
// arrays of those columns, and theta of the warp's columns awaiting the
// redistribution (values, p^(kappa+1) thicknesses, their floor and, FP64
// build, the input column integrals)
template <typename R, int VL, int H>
struct RemapV {
  static constexpr int S = 32 / H * VL + 4;                        // nvl + 1 <= (32/H) VL + 1
  static constexpr int D = H > 1 ? 2 : (sizeof(R) == 4 ? 4 : 3);   // items in flight
  R ring[D][H][3][S];
  R exold[H][S], prcol[H][S], exnew[H][S], prnew[H][S], pk1col[H][S], pk1new[H][S], dpcol[H][S];
  R tg[S];
  R thb[kColsPerWarp][S], dkb[kColsPerWarp][S];
  R dpb[kColsPerWarp][S];  // new thicknesses, for theta x thickness (trdp) after the redistribution
  R flo[kColsPerWarp], colin[kColsPerWarp], colscl[kColsPerWarp];
};
static_assert(sizeof(RemapV<float, 1, 1>) % 16 == 0 && sizeof(RemapV<double, 1, 1>) % 16 == 0 &&
                  sizeof(RemapV<float, 4, 2>) % 16 == 0,
              "ring slots of consecutive warps stay 16-byte aligned");

// pcwise's coordinate quantities for one lane's levels and interfaces
template <typename R, int VL>
struct LaneGeo {
  R fo[VL], rfo[VL], rfn[VL];  // level kb+v: fco, 1/(fco+small), 1/(fcn+small)
  R nd[VL], hh[VL];            // interface kb+v: -delz (0: no flux), (dx-1 | 1-dx)/2
  unsigned up;                 // bit v: interface kb+v takes layer kb+v as donor
  bool thin;                   // (whole warp) some layer is thin enough for the fill to matter
};

template <typename R>
__device__ __forceinline__ R coord_thick(bool flip, const R* x, int k) {
  return flip ? cmax(R(0), (-x[k + 1]) - (-x[k])) : cmax(R(0), x[k + 1] - x[k]);
}

template <typename R, int VL, int W = 32>
__device__ __forceinline__ void lane_geo(int L, int lane, const R* xo, const R* xn, LaneGeo<R, VL>& G) {
  const R small = R(1.e-22);
  const bool flip = !(xo[0] < xo[L]);
  const int kb = lane * VL;
  bool thin = false;
  unsigned up = 0u;
#pragma unroll
  for (int v = 0; v < VL; v++) {
    const int k = kb + v;
    R fo = R(0), fn = R(0);
    if (k < L) {
      fo = coord_thick(flip, xo, k);
      fn = coord_thick(flip, xn, k);
      thin = thin || fo < fill_thin<R>();
    }
    G.fo[v] = fo;
    G.rfo[v] = fdiv(R(1), fo + small);
    G.rfn[v] = fdiv(R(1), fn + small);
    R nd = R(0), hh = R(0);
    if (k >= 1 && k <= L - 1) {
      const R d = flip ? (-xn[k]) - (-xo[k]) : xn[k] - xo[k];
      if (d != R(0)) {
        const R fl = coord_thick(flip, xo, d > R(0) ? k : k - 1);
        if (fl > R(0)) {
          const R dd = d > R(0) ? d : -d;
          const R dsl = cmin(R(0) + fl, dd) - cmin(R(0), dd);
          const R dx = fdiv(dsl, fl);
          const R hx = d > R(0) ? dx - R(1) : R(1) - dx;
          if (dsl != R(0)) {
            nd = -d;
            hh = R(.5) * hx;
          }
        }
        if (d > R(0)) up |= 1u << v;
      }
    }
    G.nd[v] = nd;
    G.hh[v] = hh;
  }
  G.up = up;
  // decided over the whole warp: pcwise's fill branch holds full-warp
  // shuffles, so both columns of a paired warp must take it together (the
  // fill is the reference's own step, exact for columns without thin layers)
  G.thin = __any_sync(0xffffffffu, thin);
}

// pcwise (PLM, miglim = 1) of NF fields sharing one coordinate, lane =
// levels kb .. kb+VL-1 of each; the fields' chains are independent and
// interleave.  Returns true when pcwise's column-integral check
// (hybgen.F90:1262) fails.  That check compares two sums of the same
// telescoping fluxes; in FP32 it would only measure the rounding of those
// sums and cost 0.49 ms a step at glvl 8 (a tenth of the remap), so it runs
// in the FP64 build, and the FP32-mixed build keeps the two physical column
// checks (restp_1d's, and remap_1d's theta integral).
template <typename R, int VL, int NF, int W = 32>
__device__ __forceinline__ bool pcwise_v(int L, int lane, R (&y)[NF][VL], const LaneGeo<R, VL>& G) {
  const R small = R(1.e-22);
  const int kb = lane * VL;
  R bfore[NF], colscl[NF];
  if (sizeof(R) == 8) {
#pragma unroll
    for (int h = 0; h < NF; h++) {
      bfore[h] = R(0);
      colscl[h] = R(0);
#pragma unroll
      for (int v = 0; v < VL; v++)
        if (kb + v < L) {
          bfore[h] += y[h][v] * G.fo[v];
          colscl[h] += cabs(y[h][v] * G.fo[v]);
        }
    }
  }
  R yf[NF][VL];
  if (G.thin) {
    // backward fill: nb(nvl) = y(nvl), nb(k) = (y(k) fco(k) + nb(k+1) small) / (fco(k) + small)
    R nb[NF][VL];
#pragma unroll
    for (int h = 0; h < NF; h++) {
      R a = R(1), b = R(0);
#pragma unroll
      for (int v = VL - 1; v >= 0; v--) {
        const int k = kb + v;
        if (k == L - 1) {
          a = R(0);
          b = y[h][v];
        } else if (k < L) {
          const R A = small * G.rfo[v];
          b = A * b + y[h][v] * G.fo[v] * G.rfo[v];
          a = A * a;
        }
      }
      R x = affine_entry_down<R, W>(lane, a, b);
#pragma unroll
      for (int v = VL - 1; v >= 0; v--) {
        const int k = kb + v;
        if (k == L - 1) x = y[h][v];
        else if (k < L) x = (y[h][v] * G.fo[v] + x * small) * G.rfo[v];
        nb[h][v] = x;
      }
    }
    // forward fill: yf(1) = nb(1), yf(k) = (nb(k) fco(k) + yf(k-1) small) / (fco(k) + small)
#pragma unroll
    for (int h = 0; h < NF; h++) {
      R a = R(1), b = R(0);
#pragma unroll
      for (int v = 0; v < VL; v++) {
        const int k = kb + v;
        if (k == 0) {
          a = R(0);
          b = nb[h][v];
        } else if (k < L) {
          const R A = small * G.rfo[v];
          b = A * b + nb[h][v] * G.fo[v] * G.rfo[v];
          a = A * a;
        }
      }
      R x = affine_entry_up<R, W>(lane, a, b);
#pragma unroll
      for (int v = 0; v < VL; v++) {
        const int k = kb + v;
        if (k == 0) x = nb[h][v];
        else if (k < L) x = (nb[h][v] * G.fo[v] + x * small) * G.rfo[v];
        yf[h][v] = x;
      }
    }
  } else {
#pragma unroll
    for (int h = 0; h < NF; h++)
#pragma unroll
      for (int v = 0; v < VL; v++) yf[h][v] = y[h][v];
  }
  bool bad = false;
#pragma unroll
  for (int h = 0; h < NF; h++) {
    // PLM slopes (zero in the end layers)
    const R ym = __shfl_up_sync(0xffffffffu, yf[h][VL - 1], 1, W);
    const R yp = __shfl_down_sync(0xffffffffu, yf[h][0], 1, W);
    R bk[VL];
#pragma unroll
    for (int v = 0; v < VL; v++) {
      const int k = kb + v;
      const R fm = v > 0 ? yf[h][v - 1] : ym;
      const R fp = v < VL - 1 ? yf[h][v + 1] : yp;
      bk[v] = (k >= 1 && k <= L - 2) ? plm_slope(fm, yf[h][v], fp) : R(0);
    }
    // interface fluxes; one donor layer: vertfx = -dz * (fcdx * slab) / slab = -dz * fcdx
    const R bm = __shfl_up_sync(0xffffffffu, bk[VL - 1], 1, W);
    R fl[VL];
#pragma unroll
    for (int v = 0; v < VL; v++) {
      const bool up = (G.up >> v) & 1u;
      const R a = up ? yf[h][v] : (v > 0 ? yf[h][v - 1] : ym);
      const R b = up ? bk[v] : (v > 0 ? bk[v - 1] : bm);
      fl[v] = G.nd[v] != R(0) ? G.nd[v] * (a + b * G.hh[v]) : R(0);
    }
    const R fnext = __shfl_down_sync(0xffffffffu, fl[0], 1, W);
    R after = R(0);
#pragma unroll
    for (int v = 0; v < VL; v++) {
      const int k = kb + v;
      if (k < L) {
        const R vn = (k + 1 < L) ? (v < VL - 1 ? fl[v + 1] : fnext) : R(0);
        const R amount = yf[h][v] * G.fo[v] - (vn - fl[v]);
        after += amount;
        y[h][v] = (amount + yf[h][v] * small) * G.rfn[v];
      }
    }
    if (sizeof(R) == 8) {
      const R dif = warp_sum<R, W>(bfore[h] - after), scl = warp_sum<R, W>(colscl[h]);
      bad |= cabs(dif) > cmax(R(1.e-33), col_tol<R>(1.e-11) * scl);
    }
  }
  return bad;
}

// remap_1d's fill of thin layers from above for tracers 2..ntra (thktop = 0):
// y(k) = (y(k) dp(k) + y(k-1) small) / (dp(k) + small), k = 3..nvl
template <typename R, int VL, int NF, int W = 32>
__device__ __forceinline__ void fill_from_above(int L, int lane, R (&y)[NF][VL], const R (&dpv)[VL],
                                                const R (&qqv)[VL]) {
  const R small = R(1.e-6);
  const int kb = lane * VL;
#pragma unroll
  for (int h = 0; h < NF; h++) {
    R a = R(1), b = R(0);
#pragma unroll
    for (int v = 0; v < VL; v++) {
      const int k = kb + v;
      if (k < 2) {
        a = R(0);
        b = y[h][v];
      } else if (k < L) {
        const R A = small * qqv[v];
        b = A * b + y[h][v] * dpv[v] * qqv[v];
        a = A * a;
      }
    }
    R x = affine_entry_up<R, W>(lane, a, b);
#pragma unroll
    for (int v = 0; v < VL; v++) {
      const int k = kb + v;
      if (k < 2) {
        x = y[h][v];
      } else if (k < L) {
        x = (y[h][v] * dpv[v] + x * small) * qqv[v];
        y[h][v] = x;
      }
    }
  }
}

// VL consecutive values at p (VL * sizeof(R) bytes, aligned to min(16, that))
template <typename R, int VL>
__device__ __forceinline__ void st_lane(R* p, const R (&y)[VL]) {
  if constexpr (VL * sizeof(R) <= 16) {
    stv<VL>(p, y);
  } else {
#pragma unroll
    for (int h = 0; h < VL; h += 2) {
      double2 t;
      t.x = y[h];
      t.y = y[h + 1];
      *reinterpret_cast<double2*>(p + h) = t;
    }
  }
}

// one lane's levels of a field column: VL wide when vec, else value by value
template <typename R, int VL>
__device__ __forceinline__ void store_levels(R* dst, int L, int kb, int vec, const R (&y)[VL]) {
  if (vec) {
    if (kb < L) st_lane<R, VL>(dst + kb, y);
  } else {
#pragma unroll
    for (int v = 0; v < VL; v++)
      if (kb + v < L) dst[kb + v] = y[v];
  }
}

// tracer t (0-based, >= 1) of column i leaving the remap when tracer x
// thickness is formed here: hystat's floor for tracers 2 and 3 (applied to y,
// which the caller then stores), then trdp = y * dp (hystat.F90:90-101)
template <typename R, int VL>
__device__ __forceinline__ void tracer_out(int t, R qvmin, R qwmin, const R (&dp)[VL], R (&y)[VL], R* trdp,
                                           size_t NL, int i, int L, int kb, int vec) {
  if (t == 1 || t == 2) {
    const R floor = t == 1 ? qvmin : qwmin;
#pragma unroll
    for (int v = 0; v < VL; v++) y[v] = cmax(floor, y[v]);
  }
  R z[VL];
#pragma unroll
  for (int v = 0; v < VL; v++) z[v] = y[v] * dp[v];
  store_levels<R, VL>(trdp + (size_t)t * NL + (size_t)i * L, L, kb, vec, z);
}

// inflate (hybgen.F90:893-1007) of 32 columns per warp, lane = column
template <typename R, int ML>
__global__ void __launch_bounds__(32 * kWarpsInflate) k_inflate(Grid<R> g, Strides s, Knobs kn,
    const StepParams* __restrict__ sp, const R* __restrict__ pr3d, R* __restrict__ exn, int bnd) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int N = g.N, L = g.L, L1 = L + 1;
  const int i0 = (blockIdx.x * kWarpsInflate + wib) * 32;
  if (i0 >= N) return;
  const int ncol = (N - i0 < 32) ? N - i0 : 32;
  const size_t m = blockIdx.y;
  if (!sp[m].active || (bnd && sp[m].its <= 1)) return;
  pr3d += m * s.intf; exn += m * s.intf;
  R* col = reinterpret_cast<R*>(smraw) + (size_t)wib * (32 * (ML + 1) + 1);
  for (int q = lane; q < ncol * L1; q += 32) col[q] = exn[(size_t)i0 * L1 + q];
  __syncwarp();
  if (lane < ncol) inflate<R>(kn, g.dpsig, L, pr3d[(size_t)(i0 + lane) * L1], col + lane * L1);
  __syncwarp();
  for (int q = lane; q < ncol * L1; q += 32) exn[(size_t)i0 * L1 + q] = col[q];
}

// vec: every field column starts on a min(16, VL*sizeof(R))-byte boundary
// and nvl is a multiple of VL (the copies and stores are then VL wide)
// WL: lanes per column (32, or 16 with two columns per warp in hand)
template <typename R, int VL, int WL>
__global__ void __launch_bounds__(32 * kWarpsRemapV) k_remap_v(Grid<R> g, Strides s, Knobs kn,
    const StepParams* __restrict__ sp, const R* __restrict__ targt, const R* __restrict__ exsmo,
    R* __restrict__ us3d, R* __restrict__ vs3d, R* __restrict__ tr3d, R* __restrict__ sdot,
    R* __restrict__ ex3d, R* __restrict__ dp3d, R* __restrict__ pr3d, int* __restrict__ flags, int bnd,
    int vec, R* __restrict__ trdp) {
  constexpr int H = 32 / WL;  // columns in hand per warp
  using SW = RemapV<R, VL, H>;
  constexpr int D = SW::D;
  constexpr int CB = VL * (int)sizeof(R) < 16 ? VL * (int)sizeof(R) : 16;  // bytes per copy
  constexpr int CE = CB / (int)sizeof(R);                                  // values per copy
  // fields whose pcwise runs interleaved (register budget)
  constexpr int NT = (sizeof(R) == 4 && VL <= 2) ? 3 : 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int N = g.N, L = g.L, L1 = L + 1, T = g.T;
  const int c0 = (blockIdx.x * kWarpsRemapV + wib) * kColsPerWarp;
  if (c0 >= N) return;
  const int ncol = (N - c0 < kColsPerWarp) ? N - c0 : kColsPerWarp;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active || (bnd && sp->its <= 1)) return;
  SW& S = reinterpret_cast<SW*>(smraw)[wib];
  exsmo += m * s.intf; us3d += m * s.cell; vs3d += m * s.cell; tr3d += m * s.tr; sdot += m * s.intf;
  ex3d += m * s.intf; dp3d += m * s.cell; pr3d += m * s.intf;
  if (trdp) trdp += m * s.tr;
  const int its = sp->its - bnd;
  const R cp = R(kCp), rd = R(kRd), p1000 = R(kP1000), small = R(1.e-6);
  // hystat's floors of tracers 2 and 3 (hystat.F90:90-93) when trdp is formed here
  const R qvmin = R(kQvmin), qwmin = R(kQwmin);
  const int hw = lane / WL, ls = lane - hw * WL;  // column in hand, lane within it
  const int kb = ls * VL;
  const int ngroups = (ncol + H - 1) / H;            // columns gc*H + hw, gc < ngroups
  // fields in order o: 0 = theta, 1 = u, 2 = v, 3.. = tracers 2..ntra;
  // items per column: the interface arrays (ex3d, pr3d, exsmo), then the
  // fields three by three
  const int F = min(T, sp->ntr) + 2, I = 1 + (F + 2) / 3;
  auto field = [&](int o, int i) -> R* {
    return o == 1 ? us3d + (size_t)i * L : o == 2 ? vs3d + (size_t)i * L
         : tr3d + ((size_t)(o == 0 ? 0 : o - 2) * N + i) * L;
  };
  // copy item j of the columns gc*H + hw into ring slot q (an empty group past the last)
  auto issue = [&](int gc, int j, int q) {
    if (gc < ngroups && gc * H + hw < ncol) {
      const int i = c0 + gc * H + hw;
      if (j == 0) {
#pragma unroll
        for (int h = 0; h < 3; h++) {
          const R* src = (h == 0 ? ex3d : h == 1 ? pr3d : exsmo) + (size_t)i * L1;
          for (int k = ls; k <= L; k += WL) cp_async<sizeof(R)>(&S.ring[q][hw][h][k], src + k);
        }
      } else {
#pragma unroll
        for (int h = 0; h < 3; h++) {
          const int o = 3 * (j - 1) + h;
          if (o < F) {
            const R* src = field(o, i);
            if (vec) {
              if (kb < L) {
#pragma unroll
                for (int e = 0; e < VL; e += CE) cp_async<CB>(&S.ring[q][hw][h][kb + e], src + kb + e);
              }
            } else {
#pragma unroll
              for (int v = 0; v < VL; v++)
                if (kb + v < L) cp_async<sizeof(R)>(&S.ring[q][hw][h][kb + v], src + kb + v);
            }
          }
        }
      }
    }
    cp_async_commit();
  };
  for (int k = lane; k < L; k += 32) S.tg[k] = targt[k];
  int ic = 0, ij = 0;   // next item to copy
  for (int q = 0; q < D; q++) {
    issue(ic, ij, q);
    if (++ij == I) { ij = 0; ++ic; }
  }
  LaneGeo<R, VL> gp;
  R dpv[VL], qqv[VL];
  bool bad = false;
  int gc = 0, j = 0, qs = 0;   // item in hand: column group, item, ring slot
  while (gc < ngroups) {
    cp_async_wait<D - 1>();
    __syncwarp();
    const int cs = gc * H + hw;            // this lane's column (index within the warp)
    const bool valid = cs < ncol;          // the second column of a last odd group is idle
    const int i = c0 + (valid ? cs : 0);
    R y[3][VL];
    if (j == 0) {
      for (int k = ls; k <= L; k += WL) {
        S.exold[hw][k] = S.ring[qs][hw][0][k];
        S.prcol[hw][k] = S.ring[qs][hw][1][k];
        S.exnew[hw][k] = S.ring[qs][hw][2][k];
      }
    } else {
#pragma unroll
      for (int h = 0; h < 3; h++)
#pragma unroll
        for (int v = 0; v < VL; v++) y[h][v] = kb + v < L ? S.ring[qs][hw][h][kb + v] : R(0);
    }
    __syncwarp();
    issue(ic, ij, qs);   // D items ahead, into the slot just read
    if (++ij == I) { ij = 0; ++ic; }
    if (j == 0) {
      // new interfaces (exsmo -> exnew), pressures and p^(kappa+1) of the column
      for (int k = ls; k <= L; k += WL) {
        const R eo = S.exold[hw][k];
        R en = S.exnew[hw][k];
        if (its > 0) {
          const R sl = R(kn.slak);
          en = sl * en + (R(1) - sl) * eo;
        }
        S.exnew[hw][k] = en;
        S.pk1col[hw][k] = eo * S.prcol[hw][k] / cp;
      }
      __syncwarp();
      // miglim = 1: exnew(2..nvl) between the neighbouring old interfaces
      for (int k = 2 + ls; k <= L; k += WL)
        S.exnew[hw][k - 1] = cmax(R(.0001) * S.exold[hw][k - 1] + R(.9999) * S.exold[hw][k],
                              cmin(R(.0001) * S.exold[hw][k - 1] + R(.9999) * S.exold[hw][k - 2], S.exnew[hw][k - 1]));
      __syncwarp();
      for (int k = ls; k <= L; k += WL) {
        // the reference's own operations: the pressures of unmoved
        // interfaces then reproduce the old ones exactly, so the layer
        // thicknesses keep summing to the unchanged column mass
        const R en = S.exnew[hw][k];
        const R pn = p1000 * pow(en / cp, cp / rd);
        S.prnew[hw][k] = pn;
        S.pk1new[hw][k] = en * pn / cp;
      }
      __syncwarp();
      for (int k = ls; k < L; k += WL) S.dpcol[hw][k] = S.prnew[hw][k] - S.prnew[hw][k + 1];
      __syncwarp();
      if (ls == 0) {
        S.prnew[hw][L] = S.prcol[hw][L];
        S.pk1new[hw][L] = S.pk1col[hw][L];
        S.prnew[hw][0] = S.prcol[hw][0];
        S.pk1new[hw][0] = S.pk1col[hw][0];
        S.flo[cs] = S.pk1col[hw][0] * small;
      }
      __syncwarp();
      for (int k = ls; k < L; k += WL) S.dkb[cs][k] = S.pk1new[hw][k] - S.pk1new[hw][k + 1];
      if (trdp)
        for (int k = ls; k < L; k += WL) S.dpb[cs][k] = S.dpcol[hw][k];
      lane_geo<R, VL, WL>(L, ls, S.prcol[hw], S.prnew[hw], gp);
#pragma unroll
      for (int v = 0; v < VL; v++) {
        dpv[v] = kb + v < L ? S.dpcol[hw][kb + v] : R(0);
        qqv[v] = fdiv(R(1), dpv[v] + small);
      }
      __syncwarp();
    } else if (j == 1) {
      // theta in p^(kappa+1), held for the redistribution after the last column
      {
        LaneGeo<R, VL> gk;
        lane_geo<R, VL, WL>(L, ls, S.pk1col[hw], S.pk1new[hw], gk);
        {
          R colin = R(0), colscl = R(0);
#pragma unroll
          for (int v = 0; v < VL; v++)
            if (kb + v < L) {
              const R w = y[0][v] * (S.pk1col[hw][kb + v] - S.pk1col[hw][kb + v + 1]);
              colin += w;
              colscl += cabs(w);
            }
          colin = warp_sum<R, WL>(colin);
          colscl = warp_sum<R, WL>(colscl);
          if (ls == 0) {
            S.colin[cs] = colin;
            S.colscl[cs] = colscl;
          }
        }
        R t[1][VL];
#pragma unroll
        for (int v = 0; v < VL; v++) t[0][v] = y[0][v];
        const bool bt = pcwise_v<R, VL, 1, WL>(L, ls, t, gk);
        bad |= valid && bt;
#pragma unroll
        for (int v = 0; v < VL; v++)
          if (kb + v < L) S.thb[cs][kb + v] = t[0][v];
      }
      // u, v in pressure
      if constexpr (NT == 3) {
        R uv[2][VL];
#pragma unroll
        for (int v = 0; v < VL; v++) {
          uv[0][v] = y[1][v];
          uv[1][v] = y[2][v];
        }
        const bool bu = pcwise_v<R, VL, 2, WL>(L, ls, uv, gp);
        bad |= valid && bu;
        if (valid) {
          store_levels<R, VL>(us3d + (size_t)i * L, L, kb, vec, uv[0]);
          store_levels<R, VL>(vs3d + (size_t)i * L, L, kb, vec, uv[1]);
        }
      } else {
#pragma unroll
        for (int h = 1; h < 3; h++) {
          R t[1][VL];
#pragma unroll
          for (int v = 0; v < VL; v++) t[0][v] = y[h][v];
          const bool bu = pcwise_v<R, VL, 1, WL>(L, ls, t, gp);
          bad |= valid && bu;
          if (valid) store_levels<R, VL>(field(h, i), L, kb, vec, t[0]);
        }
      }
    } else {
      // tracers 2..ntra in pressure
      const int o0 = 3 * (j - 1);
      if constexpr (NT == 3) {
        const bool bq = pcwise_v<R, VL, 3, WL>(L, ls, y, gp);
        bad |= valid && bq;
        if (kn.thktop == 0.) fill_from_above<R, VL, 3, WL>(L, ls, y, dpv, qqv);
#pragma unroll
        for (int h = 0; h < 3; h++)
          if (valid && o0 + h < F) {
            if (trdp) tracer_out<R, VL>(o0 + h - 2, qvmin, qwmin, dpv, y[h], trdp, (size_t)N * L, i, L, kb, vec);
            store_levels<R, VL>(field(o0 + h, i), L, kb, vec, y[h]);
          }
      } else {
#pragma unroll
        for (int h = 0; h < 3; h++) {
          if (o0 + h < F) {
            R t[1][VL];
#pragma unroll
            for (int v = 0; v < VL; v++) t[0][v] = y[h][v];
            const bool bq = pcwise_v<R, VL, 1, WL>(L, ls, t, gp);
            bad |= valid && bq;
            if (kn.thktop == 0.) fill_from_above<R, VL, 1, WL>(L, ls, t, dpv, qqv);
            if (valid) {
              if (trdp) tracer_out<R, VL>(o0 + h - 2, qvmin, qwmin, dpv, t[0], trdp, (size_t)N * L, i, L, kb, vec);
              store_levels<R, VL>(field(o0 + h, i), L, kb, vec, t[0]);
            }
          }
        }
      }
    }
    if (j == I - 1) {
      // exnew made non-increasing downward: prefix minimum over the
      // interfaces; the column's lane l holds interfaces l*VL .. l*VL+VL-1
      // (running minimum within the lane, one scan of the lane minima over
      // the column's WL lanes), interface nvl (when WL*VL == nvl) takes the
      // minimum over all of them
      const size_t ci = (size_t)i * L1;
      const R top = S.exnew[hw][0];  // fill: no interface lies above the column top
      R pm[VL];
#pragma unroll
      for (int v = 0; v < VL; v++) {
        const int k = kb + v;
        const R x = k <= L ? S.exnew[hw][k] : top;
        pm[v] = v == 0 ? x : cmin(pm[v - 1], x);
      }
      R tot = pm[VL - 1];
#pragma unroll
      for (int off = 1; off < WL; off <<= 1) {
        const R o = __shfl_up_sync(0xffffffffu, tot, off, WL);
        if (ls >= off) tot = cmin(tot, o);
      }
      const R above = __shfl_up_sync(0xffffffffu, tot, 1, WL);
      const R all = __shfl_sync(0xffffffffu, tot, WL - 1, WL);
#pragma unroll
      for (int v = 0; v < VL; v++) {
        const int k = kb + v;
        if (valid && k <= L) {
          const R x = ls > 0 ? cmin(pm[v], above) : pm[v];
          sdot[ci + k] = x - S.exold[hw][k];
          ex3d[ci + k] = x;
          pr3d[ci + k] = S.prnew[hw][k];
          if (k < L) dp3d[(size_t)i * L + k] = S.dpcol[hw][k];
        }
      }
      if (valid && WL * VL == L && ls == 0) {
        const R x = cmin(S.exnew[hw][L], all);
        sdot[ci + L] = x - S.exold[hw][L];
        ex3d[ci + L] = x;
        pr3d[ci + L] = S.prnew[hw][L];
      }
      __syncwarp();
    }
    if (++j == I) { j = 0; ++gc; }
    if (++qs == D) qs = 0;
  }
  cp_async_wait<0>();
  __syncwarp();
  // theta redistribution among neighbouring layers (hybgen.F90:648-667),
  // lane = column: pairs (k-1, k) from the bottom up, each pair seeing the
  // upper layer of the pair below as already adjusted
  if (lane < ncol && L >= 3) {
    R* th = S.thb[lane];
    const R* dk = S.dkb[lane];
    const R fl = S.flo[lane];
    R thb = th[L - 1];
    for (int k = L; k >= 3; k--) {
      const R tha = th[k - 2];
      const R dplo = cmax(dk[k - 2], fl), dpup = cmax(dk[k - 1], fl);
      const R devilo = (tha - S.tg[k - 2]) * dplo;
      const R deviup = (thb - S.tg[k - 1]) * dpup;
      R na = tha, nbv = thb;
      if (deviup > R(0) && devilo < R(0)) {
        const R cc = cmin(deviup, -devilo);
        na = tha + cc / dplo;
        nbv = thb - cc / dpup;
      } else if (deviup < R(0) && devilo > R(0)) {
        const R cc = cmin(devilo, -deviup);
        na = tha - cc / dplo;
        nbv = thb + cc / dpup;
      }
      th[k - 1] = nbv;
      thb = na;
    }
    th[1] = thb;
    {
      R clout = R(0);
      for (int k = 0; k < L; k++) clout = clout + th[k] * dk[k];
      if (cabs(clout - S.colin[lane]) > cmax(R(1.e-33), col_tol<R>(2.e-6) * S.colscl[lane])) bad = true;
    }
  }
  __syncwarp();
  for (int cc = hw; cc < ncol; cc += H) {
    R y[VL];
#pragma unroll
    for (int v = 0; v < VL; v++) y[v] = kb + v < L ? S.thb[cc][kb + v] : R(0);
    store_levels<R, VL>(tr3d + (size_t)(c0 + cc) * L, L, kb, vec, y);
    if (trdp) {
      R z[VL];
#pragma unroll
      for (int v = 0; v < VL; v++) z[v] = kb + v < L ? y[v] * S.dpb[cc][kb + v] : R(0);
      store_levels<R, VL>(trdp + (size_t)(c0 + cc) * L, L, kb, vec, z);
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flags + m, kFlagColumnIntegral);
}

template <typename R, int VL, int WL>
size_t remap_v_smem() { return sizeof(RemapV<R, VL, 32 / WL>) * kWarpsRemapV; }
template <typename R, int ML>
size_t inflate_smem() { return sizeof(R) * (32 * (ML + 1) + 1) * kWarpsInflate; }

// levels per lane of k_remap_v
inline int remap_vl(int L) { return L <= 32 ? 1 : L <= 64 ? 2 : 4; }

// two columns per warp (16 lanes x 4 levels) for FP32 with 32 < nvl <= 64:
// each ring item, scan and shuffle then serves two columns
template <typename R>
inline bool remap_paired(int L) { return sizeof(R) == 4 && L > 32 && L <= 64; }

template <typename R>
int prepare_hybgen(int L) {
  cudaError_t e = cudaSuccess;
  const int vl = remap_vl(L);
  if (remap_paired<R>(L)) {
    if constexpr (sizeof(R) == 4)
      e = cudaFuncSetAttribute(k_remap_v<R, 4, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)remap_v_smem<R, 4, 16>());
  } else if (vl == 1)
    e = cudaFuncSetAttribute(k_remap_v<R, 1, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)remap_v_smem<R, 1, 32>());
  else if (vl == 2)
    e = cudaFuncSetAttribute(k_remap_v<R, 2, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)remap_v_smem<R, 2, 32>());
  else
    e = cudaFuncSetAttribute(k_remap_v<R, 4, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)remap_v_smem<R, 4, 32>());
  if (e == cudaSuccess) {
    if (L <= 64)
      e = cudaFuncSetAttribute(k_inflate<R, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)inflate_smem<R, 64>());
    else
      e = cudaFuncSetAttribute(k_inflate<R, kMaxL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)inflate_smem<R, kMaxL>());
  }
  return e == cudaSuccess ? 0 : (int)e;
}

// ---------------------------------------------------------------- hystat --
// hystat (hystat.F90:53-109): lane = column, 32 columns per warp.  The
// column set-up reads each kHyChunk-level chunk of thickness, theta and
// Exner function of the warp's columns into shared memory, then
// every lane runs the reference's recursions up its own column (surface
// pressure sum, Montgomery potential bottom-up, geopotential at the interface
// above), in FP64 (FP64 build) or float-float (FP32-mixed build, which also
// keeps the (hi, lo) Montgomery potential for the pressure gradient), and the
// results leave through the same tiles.  The humidity floors and tracer x
// thickness are k_hystat_trdp.  A chunk is kHyChunk levels; a load or store
// instruction of the warp covers 32 / kHyChunk rows (columns).
#ifndef FIM_HY_CHUNK
#define FIM_HY_CHUNK 16
#endif
constexpr int kHyChunk = FIM_HY_CHUNK;
constexpr int kHyRows = 32 / kHyChunk;
template <typename R>
constexpr int kHyWarps = sizeof(R) == 4 ? 4 : 2;
template <typename R>
__global__ void __launch_bounds__(32 * kHyWarps<R>) k_hystat(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    R* __restrict__ ph3d, const R* __restrict__ ex3d, R* __restrict__ mp3d, const R* __restrict__ dp3d,
    const R* __restrict__ tr3d, R* __restrict__ psrf, R* __restrict__ ptdcy,
    float2* __restrict__ mpf, int bnd) {
  __shared__ R tiles[kHyWarps<R>][3][32][kHyChunk + 1];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int N = g.N, L = g.L, L1 = L + 1;
  const int i0 = (blockIdx.x * kHyWarps<R> + wib) * 32;
  if (i0 >= N) return;
  const int ncol = N - i0 < 32 ? N - i0 : 32;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active || (bnd && sp->its <= 1)) return;
  ph3d += m * s.intf; ex3d += m * s.intf; mp3d += m * s.cell; dp3d += m * s.cell; tr3d += m * s.tr;
  psrf += m * s.col; ptdcy += m * 2 * s.col;
  if (mpf) mpf += m * s.cell;
  const int its = sp->its - bnd;
  const int i = i0 + lane;
  const bool live = lane < ncol;
  R (*tdp)[kHyChunk + 1] = tiles[wib][0];  // thickness in, Montgomery potential out
  R (*tth)[kHyChunk + 1] = tiles[wib][1];  // theta in, low part of the Montgomery potential out (FP32)
  R (*tex)[kHyChunk + 1] = tiles[wib][2];  // Exner function in, geopotential out
  // the staging lanes: row (column) rr * kHyRows + lrow, level lk of the chunk
  const int lrow = lane / kHyChunk, lk = lane - lrow * kHyChunk;
  const R ph0 = live ? ph3d[(size_t)i * L1] : R(0);
  const R exL = live ? ex3d[(size_t)i * L1 + L] : R(0);
  const R work = live ? psrf[i] : R(0);
  FF2 psf{0.f, 0.f}, mpff{0.f, 0.f};
  double psd = 0.0, mpd = 0.0;
  R thp = R(0);
  for (int c0 = 0; c0 < L; c0 += kHyChunk) {
    const int kk = c0 + lk;
    const int nq = L - c0 < kHyChunk ? L - c0 : kHyChunk;
#pragma unroll 8
    for (int rr = 0; rr < 32 / kHyRows; rr++) {
      const int r = rr * kHyRows + lrow;
      if (r < ncol && kk < L) {
        const size_t ic = (size_t)(i0 + r);
        tdp[r][lk] = dp3d[ic * L + kk];
        tth[r][lk] = tr3d[ic * L + kk];
        tex[r][lk] = ex3d[ic * L1 + kk];
      }
    }
    __syncwarp();
    if (live) {
      for (int q = 0; q < nq; q++) {
        const int k = c0 + q;
        const R d = tdp[lane][q], t = tth[lane][q], e = tex[lane][q];
        if constexpr (sizeof(R) == 4) {
          // float-float recursions (FP64-accurate on the FP32 pipes)
          psf = ff_add(psf, FF2{d, 0.f});
          FF2 term;
          if (k == 0) {
            term = ff_add(two_prod(e, t), FF2{ph0, 0.f});
          } else {
            tex[lane][q] = ff_add(mpff, ff_neg(two_prod(thp, e))).hi;  // geopotential at interface k
            const FF2 dd = two_sum(t, -thp);
            term = ff_add(two_prod(e, dd.hi), FF2{e * dd.lo, 0.f});
          }
          mpff = k == 0 ? term : ff_add(mpff, term);
          tdp[lane][q] = mpff.hi;
          tth[lane][q] = mpff.lo;
        } else {
          psd += (double)d;
          double term;
          if (k == 0) {
            term = (double)e * (double)t + (double)ph0;
          } else {
            tex[lane][q] = R(mpd - (double)thp * (double)e);
            term = (double)e * ((double)t - (double)thp);
          }
          mpd = k == 0 ? term : mpd + term;
          tdp[lane][q] = R(mpd);
        }
        thp = t;
      }
    }
    __syncwarp();
#pragma unroll 8
    for (int rr = 0; rr < 32 / kHyRows; rr++) {
      const int r = rr * kHyRows + lrow;
      if (r < ncol && kk < L) {
        const size_t ic = (size_t)(i0 + r);
        mp3d[ic * L + kk] = tdp[r][lk];
        if (mpf) mpf[ic * L + kk] = make_float2((float)tdp[r][lk], (float)tth[r][lk]);
        if (kk >= 1) ph3d[ic * L1 + kk] = tex[r][lk];
      }
    }
    __syncwarp();
  }
  if (live) {
    R pn;
    if constexpr (sizeof(R) == 4) {
      ph3d[(size_t)i * L1 + L] = ff_add(mpff, ff_neg(two_prod(thp, exL))).hi;
      pn = psf.hi;
    } else {
      ph3d[(size_t)i * L1 + L] = R(mpd - (double)thp * (double)exL);
      pn = R(psd);
    }
    psrf[i] = pn;
    if (its > 0) ptdcy[(size_t)(its % 2) * N + i] = pn - work;
  }
}

// hystat.F90:72-98, the per-level part: humidity floors and tracer x
// thickness, VK levels per thread (a stream over all tracers of a column
// slice; kept apart from the column scans so its loads are not serialised
// behind them)
template <typename R, int VK>
__global__ void __launch_bounds__(kBlock2) k_hystat_trdp(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    const R* __restrict__ dp3d, R* __restrict__ tr3d, R* __restrict__ trdp, int bnd) {
  int i, k;
  if (!cell_levels<VK>(g.N, g.L, i, k)) return;
  const int N = g.N, L = g.L;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active || (bnd && sp->its <= 1)) return;
  const int T = min(g.T, sp->ntr);
  const size_t NL = (size_t)N * L;
  const size_t c = (size_t)i * L + k;
  dp3d += m * s.cell; tr3d += m * s.tr; trdp += m * s.tr;
  const R qvmin = R(kQvmin), qwmin = R(kQwmin);
  R dp[VK];
  ldv<VK>(dp3d + c, dp);
#pragma unroll 4
  for (int t = 0; t < T; t++) {
    R x[VK], y[VK];
    ldv<VK>(tr3d + (size_t)t * NL + c, x);
    if (t == 1 || t == 2) {
      const R floor = t == 1 ? qvmin : qwmin;
      FOR_V x[j] = cmax(floor, x[j]);
      stv<VK>(tr3d + (size_t)t * NL + c, x);
    }
    FOR_V y[j] = x[j] * dp[j];
    stv<VK>(trdp + (size_t)t * NL + c, y);
  }
}

// --------------------------------------------------------------- globsum --
// float-float compensated accumulator (Knuth two-sum), ~48-bit significand
struct FF {
  float hi, lo;
  __device__ void add(float x) {
    const float s = hi + x;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo += err;
  }
  __device__ double value() const { return (double)hi + (double)lo; }
};
template <typename R> struct Acc;
template <> struct Acc<double> {
  double v = 0.0;
  __device__ void add(double x) { v += x; }
  __device__ double value() const { return v; }
};
template <> struct Acc<float> {
  FF f{0.f, 0.f};
  __device__ void add(float x) { f.add(x); }
  __device__ double value() const { return f.value(); }
};

constexpr int kMaxT = 32;

// Slots of one block's partial sums: 0 = sum(area*dp), 1+t = sum(area*dp*tr_t)
// (level sums), kMaxT+1.. = the column sums of globsum.F90:81-85
// (rain, convective rain, non-convective rain, latent energy).
constexpr int kGsCol = kMaxT + 1;
constexpr int kGsSlots = kMaxT + 5;

// Level sums: a block takes one chunk of kGsChunkPer(VK) cell-levels and a
// group of kGsGroup consecutive slots q (0: area x dp, 1..ntr: area x dp x
// tracer q-1): it reads the chunk's thicknesses and cell areas once for the
// group and one tracer array per slot.  The group holding slot 0 also forms
// the column sums of the cells whose first level lies in the chunk.  Every
// slot is summed per thread in level order and per block in a fixed order,
// and the partials are per (chunk, slot): the sums are deterministic and do
// not depend on the grouping.
constexpr int kGsGroup = 7;
constexpr int kGsIter = 16;
template <int VK>
__host__ __device__ constexpr int kGsChunkPer() { return kBlock2 * VK * kGsIter; }

template <typename R, int VK> struct GsVec;
template <typename R> struct GsVec<R, 1> {
  static __device__ __forceinline__ void ld(const R* p, R (&r)[1]) { r[0] = *p; }
};
template <> struct GsVec<float, 4> {
  static __device__ __forceinline__ void ld(const float* p, float (&r)[4]) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    r[0] = t.x; r[1] = t.y; r[2] = t.z; r[3] = t.w;
  }
};
template <> struct GsVec<double, 2> {
  static __device__ __forceinline__ void ld(const double* p, double (&r)[2]) {
    const double2 t = *reinterpret_cast<const double2*>(p);
    r[0] = t.x; r[1] = t.y;
  }
};

template <typename R, int VK>
__global__ void __launch_bounds__(kBlock2) k_globsum_levels(Grid<R> g, Strides s, const StepParams* __restrict__ sp,
    int T, const R* __restrict__ dp3d, const R* __restrict__ tr, const R* __restrict__ rn2d, const R* __restrict__ rc2d,
    const R* __restrict__ pr3d, const R* __restrict__ ex3d, const R* __restrict__ qf2d,
    double* __restrict__ partial, int nchunk) {
  const int N = g.N, L = g.L, L1 = L + 1;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  const int ngrp = (T + kGsGroup) / kGsGroup;  // groups of the T + 1 slots
  const int chunk = blockIdx.x / ngrp, q0 = (blockIdx.x - chunk * ngrp) * kGsGroup;
  const int nq = (T + 1 - q0 < kGsGroup) ? T + 1 - q0 : kGsGroup;
  dp3d += m * s.cell; tr += m * s.tr; pr3d += m * s.intf; ex3d += m * s.intf;
  // N * L < 2^31 (checked on the host): 32-bit cell-level indices
  const unsigned NL = (unsigned)N * (unsigned)L;
  constexpr int CH = kGsChunkPer<VK>();
  const unsigned e0 = (unsigned)chunk * CH;
  Acc<R> acc[kGsGroup];
  // the group's arrays: slot 0 reads the thicknesses again (an L1 hit) and
  // adds area x dp; slots past the last repeat slot T and add nothing, so
  // every load of an iteration is issued before the first sum
  const R* xp[kGsGroup];
  // tracers past the member's own count add nothing (and are not read)
  const int ntm = min(T, sp->ntr);
#pragma unroll
  for (int u = 0; u < kGsGroup; u++) {
    const int q = q0 + u <= T ? q0 + u : T;
    xp[u] = (q == 0 || q > ntm) ? dp3d : tr + (size_t)(q - 1) * NL;
  }
  auto sum_at = [&](unsigned idx) {
    const R ar = g.area[idx / (unsigned)L];
    R dp[VK], ad[VK], x[kGsGroup][VK];
    GsVec<R, VK>::ld(dp3d + idx, dp);
#pragma unroll
    for (int u = 0; u < kGsGroup; u++) GsVec<R, VK>::ld(xp[u] + idx, x[u]);
#pragma unroll
    for (int j = 0; j < VK; j++) ad[j] = ar * dp[j];
#pragma unroll
    for (int u = 0; u < kGsGroup; u++)
      if (u < nq && q0 + u <= ntm) {
#pragma unroll
        for (int j = 0; j < VK; j++) acc[u].add(u == 0 && q0 == 0 ? ad[j] : ad[j] * x[u][j]);
      }
  };
  if (e0 + CH <= NL) {
    for (int it = 0; it < kGsIter; it++) sum_at(e0 + ((unsigned)it * kBlock2 + threadIdx.x) * VK);
  } else {
    for (int it = 0; it < kGsIter; it++) {
      const unsigned idx = e0 + ((unsigned)it * kBlock2 + threadIdx.x) * VK;
      if (idx < NL) sum_at(idx);
    }
  }
  double col[4] = {0., 0., 0., 0.};
  if (q0 == 0) {
    const double dt = sp->dt, rdcp = kRd / kCp;
    const size_t i0 = ((size_t)e0 + L - 1) / L;
    size_t i1 = ((size_t)e0 + CH + L - 1) / L;
    if (i1 > (size_t)N) i1 = N;
    for (size_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const double a = g.area_d[i];
      const double rn = rn2d ? (double)rn2d[m * s.col + i] : 0.0;
      const double rc = rc2d ? (double)rc2d[m * s.col + i] : 0.0;
      const double qf = qf2d ? (double)qf2d[m * s.col + i] : 0.0;
      col[0] += a * rn;
      col[1] += a * rc;
      col[2] += a * (rn - rc);
      const double den = (double)pr3d[i * L1] / (rdcp * (double)ex3d[i * L1] * (double)tr[i * L]);
      col[3] += a * den * qf * dt / (1.25 * 2.5e6);
    }
  }
  __shared__ double red[kBlock2 / 32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* out = partial + (m * nchunk + chunk) * kGsSlots;
  const int nout = nq + (q0 == 0 ? 4 : 0);
#pragma unroll
  for (int u = 0; u < kGsGroup + 4; u++) {
    if (u >= nout) break;  // uniform across the block
    double v = 0.;
#pragma unroll
    for (int w = 0; w < kGsGroup; w++)
      if (w == u) v = acc[w].value();
#pragma unroll
    for (int w = 0; w < 4; w++)
      if (u == nq + w) v = col[w];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) red[wib] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kBlock2 / 32; w++) t += red[w];
      out[u < nq ? q0 + u : kGsCol + (u - nq)] = t;
    }
    __syncthreads();
  }
}

// Final reduction of the block partials; one warp per output slot.
template <typename R>
__global__ void k_globsum_final(const StepParams* __restrict__ sp, int T, const double* __restrict__ partial,
                                int nblk, double* __restrict__ sums) {
  const size_t m = blockIdx.x;
  sp += m;
  if (!sp->active) return;
  const int lane = threadIdx.x & 31;
  double* out = sums + m * (8 + T);
  for (int j = threadIdx.x >> 5; j < T + 5; j += blockDim.x >> 5) {
    const int q = j <= T ? j : kGsCol + (j - T - 1);
    double t = 0.;
    for (int b = lane; b < nblk; b += 32) t += partial[(m * nblk + b) * kGsSlots + q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (lane != 0) continue;
    if (q == 0) {
      out[0] = t / kGrvity;
    } else if (q <= T) {
      out[8 + (q - 1)] = t;
      if (q == 2) out[1] = t / kGrvity;
      if (q == 3) out[2] = t / kGrvity;
      if (q == 4) out[3] = t / kGrvity;
    } else {
      // qmstr (sumr), qmstrc (sumrc), qmstrn (sumrn), qmste (sume)
      const int c = q - kGsCol;
      out[c == 0 ? 5 : c == 1 ? 7 : c == 2 ? 6 : 4] = t;
    }
  }
}

// pressure and thickness from Exner (dyn_init.F90:895-906)
template <typename R>
__global__ void __launch_bounds__(kBlock2) k_prdp_from_ex(Grid<R> g, Strides s, const R* __restrict__ ex3d,
    R* __restrict__ pr3d, R* __restrict__ dp3d) {
  const int N = g.N, L = g.L, L1 = L + 1;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * L1) return;
  const int i = gid / L1, k = gid - i * L1;
  const size_t m = blockIdx.y;
  ex3d += m * s.intf; pr3d += m * s.intf; dp3d += m * s.cell;
  const R cp = R(kCp), rd = R(kRd), p1000 = R(kP1000);
  const R p = p1000 * pow(ex3d[(size_t)i * L1 + k] / cp, cp / rd);
  pr3d[(size_t)i * L1 + k] = p;
  if (k < L) {
    const R pu = p1000 * pow(ex3d[(size_t)i * L1 + k + 1] / cp, cp / rd);
    dp3d[(size_t)i * L + k] = p - pu;
  }
}


template <typename R>
bool launch_hybgen(const Launch& l, const Grid<R>& g, const Strides& s, const Knobs& kn, const HybgenScratch<R>& w,
                   const R* targt, R* us3d, R* vs3d, R* tr3d, R* sdot, R* ex3d, R* dp3d, R* pr3d, R* trdp) {
  bool trdp_done = false;
  dim3 gc(nblocks(g.N, kColBlock), l.members);
  if (g.L <= 64) {
    FIM_KBEGIN(l, "k_regrid");
    k_regrid<R, 64><<<gc, kColBlock, 0, l.stream>>>(g, s, kn, l.sp, targt, tr3d, ex3d, pr3d, w.exsmo, l.flags,
                                                     l.boundary);
  } else {
    FIM_KBEGIN(l, "k_regrid");
    k_regrid<R, kMaxL><<<gc, kColBlock, 0, l.stream>>>(g, s, kn, l.sp, targt, tr3d, ex3d, pr3d, w.exsmo,
                                                        l.flags, l.boundary);
  }
  FIM_KEND(l);
  const R* ex_in = w.exsmo;
  if (kn.intfc_smooth > 0.) {
    dim3 gs(nblocks((long long)g.N * ((g.L + kDffK) / kDffK), kBlock2), l.members);
    // Fortran levels kbl+2..nvl -> 0-based interfaces kbl+1..nvl-1
    FIM_KBEGIN(l, "k_dffusn_lev");
    k_dffusn_lev<R><<<gs, kBlock2, 0, l.stream>>>(g, s, l.sp, l.boundary, kn.kbl + 1, g.L - 1, w.exsmo,
                                                   w.exsmo2);
    FIM_KEND(l);
    ex_in = w.exsmo2;
  }
  if (kn.remap_optn == 2 && kn.miglim == 1) {
    if (kn.intfc_smooth > 0.) {
      // ex_in is the smoothing scratch here: inflate it in place
      dim3 gi(nblocks(g.N, 32 * kWarpsInflate), l.members);
      FIM_KBEGIN(l, "k_inflate");
      if (g.L <= 64)
        k_inflate<R, 64><<<gi, 32 * kWarpsInflate, inflate_smem<R, 64>(), l.stream>>>(g, s, kn, l.sp, pr3d,
                                                                                      w.exsmo2, l.boundary);
      else
        k_inflate<R, kMaxL><<<gi, 32 * kWarpsInflate, inflate_smem<R, kMaxL>(), l.stream>>>(g, s, kn, l.sp, pr3d,
                                                                                            w.exsmo2, l.boundary);
      FIM_KEND(l);
    }
    dim3 gw(nblocks(g.N, kWarpsRemapV * kColsPerWarp), l.members);
    const bool paired = remap_paired<R>(g.L);
    const int vl = paired ? 4 : remap_vl(g.L);
    const int cb = (int)(vl * sizeof(R) < 16 ? vl * sizeof(R) : 16);
    int vec = g.L % vl == 0;
    for (const void* p : {(const void*)us3d, (const void*)vs3d, (const void*)tr3d})
      if ((uintptr_t)p % cb != 0) vec = 0;
    FIM_KBEGIN(l, "k_remap");
#define FIM_REMAP_V(VL, WL)                                                                                  \
  k_remap_v<R, VL, WL><<<gw, 32 * kWarpsRemapV, remap_v_smem<R, VL, WL>(), l.stream>>>(                       \
      g, s, kn, l.sp, targt, ex_in, us3d, vs3d, tr3d, sdot, ex3d, dp3d, pr3d, l.flags, l.boundary, vec, trdp)
    if (paired) {
      if constexpr (sizeof(R) == 4) FIM_REMAP_V(4, 16);
    } else if (vl == 1) FIM_REMAP_V(1, 32);
    else if (vl == 2) FIM_REMAP_V(2, 32);
    else FIM_REMAP_V(4, 32);
#undef FIM_REMAP_V
    trdp_done = trdp != nullptr;
  } else if (g.L <= 64) {
    FIM_KBEGIN(l, "k_remap");
    k_remap<R, 64><<<gc, kColBlock, 0, l.stream>>>(g, s, kn, l.sp, targt, ex_in, us3d, vs3d, tr3d, sdot, ex3d,
                                                    dp3d, pr3d, l.flags, l.boundary);
  } else {
    FIM_KBEGIN(l, "k_remap");
    k_remap<R, kMaxL><<<gc, kColBlock, 0, l.stream>>>(g, s, kn, l.sp, targt, ex_in, us3d, vs3d, tr3d, sdot, ex3d,
                                                       dp3d, pr3d, l.flags, l.boundary);
  }
  FIM_KEND(l);
  return trdp_done;
}

template <typename R>
void launch_hystat(const Launch& l, const Grid<R>& g, const Strides& s, R* ph3d, const R* ex3d, R* mp3d,
                   const R* dp3d, R* tr3d, R* trdp, R* psrf, R* ptdcy, float2* mpf, bool trdp_done) {
  dim3 gw(nblocks(g.N, 32 * kHyWarps<R>), l.members);
  FIM_KBEGIN(l, "k_hystat");
  k_hystat<R><<<gw, 32 * kHyWarps<R>, 0, l.stream>>>(g, s, l.sp, ph3d, ex3d, mp3d, dp3d, tr3d, psrf, ptdcy, mpf,
                                                  l.boundary);
  FIM_KEND(l);
  if (trdp_done) return;  // the remap formed the floors and tracer x thickness
  const int vk = pick_vk<R>(g.L, {dp3d, tr3d, trdp});
  FIM_KBEGIN(l, "k_hystat_trdp");
  FIM_VK_DISPATCH(R, vk, (k_hystat_trdp<R, VK><<<dim3(nblocks((long long)g.N * (g.L / VK), kBlock2), l.members),
                                                 kBlock2, 0, l.stream>>>(g, s, l.sp, dp3d, tr3d, trdp,
                                                                         l.boundary)));
  FIM_KEND(l);
}

// partial buffer: the most chunks any layout uses (1 level a thread)
size_t globsum_partials(int N, int L, int T, int members) {
  (void)T;
  const long long NL = (long long)N * L;
  return (size_t)members * (size_t)((NL + kGsChunkPer<1>() - 1) / kGsChunkPer<1>()) * kGsSlots;
}

template <typename R>
void launch_globsum(const Launch& l, const Grid<R>& g, const Strides& s, int ntr, const R* dp3d, const R* tr,
                    const R* rn2d, const R* rc2d, const R* pr3d, const R* ex3d, const R* qf2d,
                    double* partial, double* sums) {
  FIM_KBEGIN(l, "k_globsum_levels");
  constexpr int VK = sizeof(R) == 4 ? 4 : 2;
  const bool vec = g.L % VK == 0 && (uintptr_t)dp3d % (VK * sizeof(R)) == 0 && (uintptr_t)tr % (VK * sizeof(R)) == 0;
  const long long NL = (long long)g.N * g.L;
  const unsigned ngrp = (unsigned)(ntr + kGsGroup) / kGsGroup;
  int nchunk;
  if (vec) {
    nchunk = (int)((NL + kGsChunkPer<VK>() - 1) / kGsChunkPer<VK>());
    k_globsum_levels<R, VK><<<dim3((unsigned)nchunk * ngrp, l.members), kBlock2, 0, l.stream>>>(
        g, s, l.sp, ntr, dp3d, tr, rn2d, rc2d, pr3d, ex3d, qf2d, partial, nchunk);
  } else {
    nchunk = (int)((NL + kGsChunkPer<1>() - 1) / kGsChunkPer<1>());
    k_globsum_levels<R, 1><<<dim3((unsigned)nchunk * ngrp, l.members), kBlock2, 0, l.stream>>>(
        g, s, l.sp, ntr, dp3d, tr, rn2d, rc2d, pr3d, ex3d, qf2d, partial, nchunk);
  }
  FIM_KEND(l);
  FIM_KBEGIN(l, "k_globsum_final");
  k_globsum_final<R><<<l.members, kBlock2, 0, l.stream>>>(l.sp, ntr, partial, nchunk, sums);
  FIM_KEND(l);
}

template <typename R>
void launch_prdp_from_ex(const Launch& l, const Grid<R>& g, const Strides& s, const R* ex3d, R* pr3d, R* dp3d) {
  dim3 gs(nblocks((long long)g.N * (g.L + 1), kBlock2), l.members);
  FIM_KBEGIN(l, "k_prdp_from_ex");
  k_prdp_from_ex<R><<<gs, kBlock2, 0, l.stream>>>(g, s, ex3d, pr3d, dp3d);
  FIM_KEND(l);
}

#define INSTANTIATE(R)                                                                                       \
  template int prepare_hybgen<R>(int);                                                                       \
  template bool launch_hybgen<R>(const Launch&, const Grid<R>&, const Strides&, const Knobs&,               \
                                 const HybgenScratch<R>&, const R*, R*, R*, R*, R*, R*, R*, R*, R*);            \
  template void launch_hystat<R>(const Launch&, const Grid<R>&, const Strides&, R*, const R*, R*, const R*, \
                                 R*, R*, R*, R*, float2*, bool);                                                  \
  template void launch_globsum<R>(const Launch&, const Grid<R>&, const Strides&, int, const R*, const R*,        \
                                  const R*, const R*, const R*, const R*, const R*, double*, double*);      \
  template void launch_prdp_from_ex<R>(const Launch&, const Grid<R>&, const Strides&, const R*, R*, R*);
INSTANTIATE(float)
INSTANTIATE(double)

}  // namespace fim
