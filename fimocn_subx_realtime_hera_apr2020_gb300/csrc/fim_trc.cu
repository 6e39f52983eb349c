// Tracer transport of the fused step: edgvar3's tracer reconstruction and
// trcadv1..3 (trcadv_compute.F90:19-315) for all tracers, on cell patches
// staged in shared memory.
//
// A patch is a parallelogram of up to 8 x 8 cells of one rhombus (each pole
// is a patch of its own); its frame adds every cell within two neighbour
// steps of the patch.  A block takes one patch, one tile of LK levels and one
// ensemble member, and runs the tracers of a chunk in turn, staging the next
// tracer's operands by cp.async while it works on the current one.
//
//   k_trf_lo  edgvalEval (edgvar3.F90:66-94): the own-side edge values of the
//             patch cells and the ring-1 neighbours' values on the patch's
//             boundary edges, in shared memory only; trcadv1 (:19-141):
//             high- and low-order fluxes, low-order AB3 update, trcr_lo; the
//             antidiffusive fluxes and the Zalesak sums S+/S- of trcadv2
//             (:143-241); a copy of the old tracer.
//   k_trf_hi  trcadv2: R+/R- of the patch cells and of their first ring, the
//             bounds taken over the 1-ring of the old tracer and of trcr_lo;
//             trcadv3 (:243-315): the antidiffusive fluxes clipped with the
//             limiters of their two cells, AB3 update of tracer x thickness,
//             new tracer.
//
// The edge values (six per cell-level and tracer) and R+/R- never reach HBM:
// per cell-level and tracer the pair reads and writes 32 words (10 of them
// the step's own state traffic), where edge values written and read back and
// R+/R- stored cost 46.  The old tracer is copied because k_trf_hi overwrites
// the tracer in place while the blocks of neighbouring patches still read it.
//
// Every value is formed from the same operands in the same order as the
// per-routine kernels (k_edgvar3_own, k_trcadv1..3), so the fused step is
// bit-identical to the routine sequence.  nprox is 5 or 6 (checked when the
// context is created), so only slot 5 of a cell can be missing: the tests
// "e < nprox" are written (e < 5 || e < np) and cost nothing for slots 0..4.
#include "fim_internal.h"

#include <algorithm>
#include <cmath>

namespace fim {

namespace {

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

// asynchronous global -> shared copy of B = 4, 8 or 16 bytes (16: through L2 only)
template <int B>
__device__ __forceinline__ void stage_copy(void* smem, const void* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if constexpr (B == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"(B) : "memory");
}
__device__ __forceinline__ void stage_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Row of slot e of patch cell x in the edge-indexed shared arrays (edge
// values, mass fluxes, antidiffusive fluxes): the slots of odd cells are
// swapped in pairs, so the same slot of two consecutive cells falls in
// different halves of the shared-memory banks (rows of 64 bytes).  The
// patch tables' mirror rows use the same mapping.
__host__ __device__ __forceinline__ int erow(int x, int e) { return x * 6 + (e ^ (x & 1)); }

// frame-local index of prox slot e (one byte each, slots 0..3 in x, 4..5 in y)
__device__ __forceinline__ int nb_at(uint2 nb, int e) {
  return e < 4 ? (int)((nb.x >> (8 * e)) & 255u) : (int)((nb.y >> (8 * (e - 4))) & 255u);
}

// Shared-memory layout of the two kernels (offsets in elements of R, then the
// patch tables after a 16-byte boundary).
//   lo: tracer frame x 2 buffers [S2][LK]; edge values [SE][LK]; mass
//       fluxes [SE][LK] in the rows of the edge values (the patch cells' six
//       slots, then the ring edges' neighbour sides); the patch cells'
//       low-order AB3 slots of and vof and tracer x thickness, x 2 buffers
//       [3][SC][LK]; least-squares coefficients, 36 per patch cell (row
//       stride 36), then 6 per ring edge.
//   hi: old-tracer and trcr_lo frames [S2][LK]; the ring-1 frame's AB3 slots
//       of and vof, S+ and S- [4][S1][LK]; R+, R- [S1][LK]; the patch cells'
//       antidiffusive fluxes [SC][6][LK], low-order tendency and tracer x
//       thickness [SC][LK]; the ring-1 frame's thickness [S1][LK] and cell
//       areas [S1].
struct PatchLayout {
  size_t trs, E, mf, ops, hf;                          // lo
  size_t TO, TL, opq, Rp, Rm, af, tlt, tdb, dpf, arf;  // hi
  size_t r_elems, tab, bytes;
  template <typename R>
  __host__ __device__ static PatchLayout make(const FrameTab& f, int LK, bool hi) {
    PatchLayout p{};
    const size_t S2 = f.S2, S1 = f.S1, SC = f.SC, SE = f.SE, SR = f.SR;
    size_t o = 0;
    if (!hi) {
      p.trs = o; o += 2 * S2 * LK;
      p.E = o; o += SE * LK;
      p.mf = o; o += SE * LK;
      p.ops = o; o += 2 * 3 * SC * LK;
      p.hf = o; o += SC * 36 + SR * 6;
    } else {
      p.TO = o; o += S2 * LK;
      p.TL = o; o += S2 * LK;
      p.opq = o; o += 4 * S1 * LK;
      p.Rp = o; o += S1 * LK;
      p.Rm = o; o += S1 * LK;
      p.af = o; o += 6 * SC * LK;
      p.tlt = o; o += SC * LK;
      p.tdb = o; o += SC * LK;
      p.dpf = o; o += S1 * LK;
      p.arf = o; o += S1;
    }
    p.r_elems = o;
    size_t b = (o * sizeof(R) + 15) & ~(size_t)15;
    p.tab = b;
    b += S2 * 4 + S1 * 8 + SC * 6 * 2 + SR * 2 + S1;
    p.bytes = (b + 15) & ~(size_t)15;
    return p;
  }
};

struct FrameSm {
  int* cells;
  uint2* nbr;
  unsigned short* mir;
  unsigned short* red;
  unsigned char* np;  // nprox of the interior and ring-1 cells
};

// the patch's tables into shared memory; callers synchronise before use
template <typename R>
__device__ __forceinline__ FrameSm load_tables(const Grid<R>& g, const FrameTab& ft, unsigned char* base,
                                               size_t tab, int tile, int C, int n1, int n2, int nre) {
  FrameSm t;
  t.cells = reinterpret_cast<int*>(base + tab);
  t.nbr = reinterpret_cast<uint2*>(t.cells + ft.S2);
  t.mir = reinterpret_cast<unsigned short*>(t.nbr + ft.S1);
  t.red = t.mir + ft.SC * 6;
  t.np = reinterpret_cast<unsigned char*>(t.red + ft.SR);
  const int* gc = ft.cells + (size_t)tile * ft.S2;
  for (int x = threadIdx.x; x < n2; x += blockDim.x) t.cells[x] = gc[x];
  for (int x = threadIdx.x; x < n1; x += blockDim.x) {
    t.nbr[x] = ft.nbr[(size_t)tile * ft.S1 + x];
    t.np[x] = (unsigned char)g.nprox[gc[x]];
  }
  for (int x = threadIdx.x; x < C * 6; x += blockDim.x) t.mir[x] = ft.mir[(size_t)tile * ft.SC * 6 + x];
  for (int x = threadIdx.x; x < nre; x += blockDim.x) t.red[x] = ft.redge[(size_t)tile * ft.SR + x];
  return t;
}

// least-squares coefficients of the patch cells (all 36) and of the ring
// edges (the row of the edge's slot) into hf; needs the tables in place
template <typename R>
__device__ __forceinline__ void load_coefs(const Grid<R>& g, const FrameSm& fs, R* hf, int C, int nre) {
  for (int q = threadIdx.x; q < C * 36; q += blockDim.x) {
    const int x = q / 36;
    hf[q] = g.hfcoef[(size_t)fs.cells[x] * 36 + (q - x * 36)];
  }
  for (int q = threadIdx.x; q < nre * 6; q += blockDim.x) {
    const int r = q / 6, code = fs.red[r];
    hf[C * 36 + q] = g.hfcoef[(size_t)fs.cells[code >> 3] * 36 + (code & 7) * 6 + (q - r * 6)];
  }
}

// rows of lk levels (from src, already offset to the tile's first level) of
// the n cells cells[0..n) into dst[x * LK + level]
template <typename R, int VK, int GC>
__device__ __forceinline__ void stage_rows(R* dst, const R* src, const int* cells, int n, int lk, int L) {
  constexpr int LK = VK * GC;
  for (int it = threadIdx.x; it < n * GC; it += blockDim.x) {
    const int x = it / GC, v = (it - x * GC) * VK;
    if (v < lk) stage_copy<VK * (int)sizeof(R)>(dst + x * LK + v, src + cells[x] * L + v);
  }
}

// The frame rows a thread copies.  The block has SC * GC threads and GC
// threads take one row, so thread (x0, v) takes rows x0, x0 + SC, x0 + 2 SC
// of every frame field (the frame lists interior, ring-1 and ring-2 cells in
// that order, so a field over its first n rows takes the rows below n).  The
// element offsets of those rows' level tiles are formed once per block; a
// copy is then an add and one cp.async.  Frames of more than 3 SC cells (the
// small patches of coarse grids) take the general loop.
template <typename R, int VK, int GC>
struct RowPlan {
  int x0, v, off[3];
  bool fast;
  __device__ __forceinline__ void init(const FrameSm& fs, int SC, int n2, int lk, int L) {
    x0 = threadIdx.x / GC;
    v = (threadIdx.x - x0 * GC) * VK;
    fast = n2 <= 3 * SC;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int x = x0 + j * SC;
      off[j] = (x < n2 && v < lk) ? fs.cells[x] * L + v : -1;
    }
  }
  // rows [0, n) of the field at src (offset to the tile's first level) into
  // dst[x * LK + level]
  __device__ __forceinline__ void copy(R* dst, const R* src, const FrameSm& fs, int SC, int n, int lk,
                                       int L) const {
    constexpr int LK = VK * GC;
    if (fast) {
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const int x = x0 + j * SC;
        if (x < n && off[j] >= 0) stage_copy<VK * (int)sizeof(R)>(dst + x * LK + v, src + off[j]);
      }
    } else {
      stage_rows<R, VK, GC>(dst, src, fs.cells, n, lk, L);
    }
  }
};

// six coefficients hf[0..6) as three pairs (8- or 16-byte shared loads)
template <typename R>
__device__ __forceinline__ void coef6(const R* hf, R (&h)[6]) {
  using P2 = typename VecOf<R, 2>::T;
  const P2* q = reinterpret_cast<const P2*>(hf);
#pragma unroll
  for (int u = 0; u < 3; u++) {
    const P2 w = q[u];
    h[2 * u] = w.x;
    h[2 * u + 1] = w.y;
  }
}

// own-side least-squares edge value of every slot ie of a patch cell
// (k_edgvar3_own's arithmetic): val = bc + sum_e hfcoef(e, ie) (tr_e - bc),
// d[e] = tr_e - bc (0 past nprox); hf = the cell's 36 coefficients
template <typename R, int VK, int LK>
__device__ __forceinline__ void own_values(const R* hf, int x, int v, const R (&bc)[VK], const R (&d)[6][VK],
                                           int np, R* E) {
#pragma unroll
  for (int ie = 0; ie < 6; ie++) {
    R h[6];
    coef6<R>(hf + ie * 6, h);
    R val[VK];
    FOR_V val[j] = bc[j];
#pragma unroll
    for (int e = 0; e < 6; e++) {
      FOR_V val[j] = (e < 5 || e < np) ? val[j] + d[e][j] * h[e] : val[j];
    }
    FOR_V val[j] = (ie < 5 || ie < np) ? val[j] : R(0);
    stv<VK>(E + erow(x, ie) * LK + v, val);
  }
}

// the value on slot p of ring-1 cell y (its side of the edge it shares with a
// patch cell), into edge-value row 6C + r; hf = that slot's 6 coefficients
template <typename R, int VK, int LK>
__device__ __forceinline__ void ring_value(const R* T, const FrameSm& fs, const R* hf, int code, int row, int v,
                                           R* E) {
  const int y = code >> 3;
  const int np = fs.np[y];
  const uint2 nb = fs.nbr[y];
  R bc[VK], val[VK], h[6];
  coef6<R>(hf, h);
  ldv<VK>(T + y * LK + v, bc);
  FOR_V val[j] = bc[j];
#pragma unroll
  for (int e = 0; e < 6; e++) {
    R d[VK];
    ldv<VK>(T + nb_at(nb, e) * LK + v, d);
    FOR_V d[j] = (e < 5 || e < np) ? d[j] - bc[j] : R(0);
    FOR_V val[j] = (e < 5 || e < np) ? val[j] + d[j] * h[e] : val[j];
  }
  stv<VK>(E + row * LK + v, val);
}

// The thread's patch cell and levels (one per thread: the block has SC * GC
// threads), with the layer thickness, which it keeps in registers for the
// whole tracer loop.
template <typename R, int VK>
struct CellItem {
  bool on;
  int i, x, v, k, c, np;
  R rar;
  R dp[VK];
  template <int GC>
  __device__ __forceinline__ void load(const Grid<R>& g, const Strides& s, const FrameSm& fs, size_t m,
                                       const R* delp, int C, int k0, int lk) {
    x = threadIdx.x / GC;
    v = (threadIdx.x - x * GC) * VK;
    on = x < C && v < lk;
    if (!on) return;
    const int L = g.L;
    i = fs.cells[x];
    k = k0 + v;
    c = i * L + k;
    np = fs.np[x];
    rar = g.rarea[i];
    ldv<VK>(delp + m * s.cell + c, dp);
  }
};

// trcadv1 + the S+/S- sums of trcadv2 + copy of the old tracer, per patch
template <typename R, int VK, int GC>
__global__ void __launch_bounds__(64 * GC, 8 / GC) k_trf_lo(Grid<R> g, Strides s, FrameTab ft,
    const StepParams* __restrict__ sp, int t0, int nt, const R* __restrict__ massfx, const R* __restrict__ trc_edg,
    const R* __restrict__ tracr, const R* __restrict__ trcdp, R* __restrict__ trl_tdcy, const R* __restrict__ delp,
    R* __restrict__ trcr_lo, R* __restrict__ s_plus, R* __restrict__ s_mnus, R* __restrict__ trold,
    R* __restrict__ antifx, size_t sc) {
  constexpr int LK = VK * GC;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  // the member's tracers in this chunk (fim_member_set_tracers); the
  // scratch keeps the chunk's layout
  const int ntm = min(nt, sp->ntr - t0);
  if (ntm <= 0) return;
  const int L = g.L, N = g.N;
  const int nlc = (L + LK - 1) / LK;
  const int tile = blockIdx.x / nlc;
  const int k0 = (blockIdx.x - tile * nlc) * LK;
  const int lk = min(LK, L - k0);
  const int4 cn = ft.cnt[tile];
  const int C = cn.x, n1 = cn.y, n2 = cn.z, nre = cn.w;
  extern __shared__ __align__(16) unsigned char fsm[];
  const PatchLayout lay = PatchLayout::make<R>(ft, LK, false);
  R* const sr = reinterpret_cast<R*>(fsm);
  R* const trs = sr + lay.trs;
  R* const E = sr + lay.E;
  R* const MF = sr + lay.mf;
  R* const ops = sr + lay.ops;
  R* const hf = sr + lay.hf;
  const FrameSm fs = load_tables<R>(g, ft, fsm, lay.tab, tile, C, n1, n2, nre);
  __syncthreads();
  load_coefs<R>(g, fs, hf, C, nre);
  const size_t NL = (size_t)N * L;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R thshld = R(1.e-11), half = R(0.5);
  const R* mfn = massfx + m * s.mf + (size_t)nf * 6 * NL;
  const R* te0 = trc_edg + m * s.tredg;  // theta (t = 0): edgvar1's edge values
  // this step's tracer t: its frame, and the patch cells' AB3 slots of/vof
  // and tracer x thickness
  RowPlan<R, VK, GC> rp;
  rp.init(fs, ft.SC, n2, lk, L);
  auto stage = [&](int t, int b) {
    rp.copy(trs + b * ft.S2 * LK, tracr + m * s.tr + (size_t)t * NL + k0, fs, ft.SC, n2, lk, L);
    const R* tl = trl_tdcy + m * s.trab + (size_t)t * 3 * NL + k0;
    R* o = ops + b * 3 * ft.SC * LK;
    rp.copy(o, tl + (size_t)of * NL, fs, ft.SC, C, lk, L);
    rp.copy(o + ft.SC * LK, tl + (size_t)vof * NL, fs, ft.SC, C, lk, L);
    rp.copy(o + 2 * ft.SC * LK, trcdp + m * s.tr + (size_t)t * NL + k0, fs, ft.SC, C, lk, L);
    stage_commit();
  };
  // the mass fluxes of the patch cells' edges and of the ring edges'
  // neighbour sides (tracer independent), with the first tracer's operands
  for (int it = threadIdx.x; it < (6 * C + nre) * GC; it += blockDim.x) {
    const int r = it / GC, v = (it - r * GC) * VK;
    if (v >= lk) continue;
    int cell, slot, row = r;
    if (r < 6 * C) {
      const int x = r / 6;
      cell = fs.cells[x];
      slot = r - x * 6;
      row = erow(x, slot);
    } else {
      const int code = fs.red[r - 6 * C];
      cell = fs.cells[code >> 3];
      slot = code & 7;
    }
    stage_copy<VK * (int)sizeof(R)>(MF + row * LK + v, mfn + (cell * 6 + slot) * L + k0 + v);
  }
  stage(t0, 0);
  CellItem<R, VK> ci;
  ci.template load<GC>(g, s, fs, m, delp, C, k0, lk);
  for (int tz = 0; tz < ntm; tz++) {
    const int t = t0 + tz, b = tz & 1;
    stage_wait();
    __syncthreads();
    if (tz + 1 < ntm) stage(t + 1, b ^ 1);
    const R* T = trs + b * ft.S2 * LK;
    if (t != 0) {
      // edge values: the six of the thread's patch cell, then the ring cells'
      // sides of the patch's boundary edges
      if (ci.on) {
        const uint2 nb = fs.nbr[ci.x];
        R bc[VK], d[6][VK];
        ldv<VK>(T + ci.x * LK + ci.v, bc);
#pragma unroll
        for (int e = 0; e < 6; e++) {
          ldv<VK>(T + nb_at(nb, e) * LK + ci.v, d[e]);
          FOR_V d[e][j] = (e < 5 || e < ci.np) ? d[e][j] - bc[j] : R(0);
        }
        own_values<R, VK, LK>(hf + ci.x * 36, ci.x, ci.v, bc, d, ci.np, E);
      }
      for (int it = threadIdx.x; it < nre * GC; it += blockDim.x) {
        const int r = it / GC, ve = (it - r * GC) * VK;
        if (ve < lk) ring_value<R, VK, LK>(T, fs, hf + C * 36 + r * 6, fs.red[r], 6 * C + r, ve, E);
      }
      __syncthreads();
    }
    if (!ci.on) continue;
    const int x = ci.x, v = ci.v, i = ci.i, c = ci.c;
    const uint2 nb = fs.nbr[x];
    R tri[VK], sumlo[VK], sp_[VK], sm_[VK], mx[VK], mn[VK];
    ldv<VK>(T + x * LK + v, tri);
    FOR_V { sumlo[j] = R(0); sp_[j] = R(0); sm_[j] = R(0); mx[j] = tri[j]; mn[j] = tri[j]; }
#pragma unroll
    for (int e = 0; e < 6; e++) {
      R trx[VK];
      ldv<VK>(T + nb_at(nb, e) * LK + v, trx);
      FOR_V { mx[j] = tmax(mx[j], trx[j]); mn[j] = tmin(mn[j], trx[j]); }
      if (e < 5 || e < ci.np) {
        R tev[VK];
        if (t != 0) {
          R tem[VK];
          ldv<VK>(E + erow(x, e) * LK + v, tev);
          ldv<VK>(E + fs.mir[x * 6 + e] * LK + v, tem);
          FOR_V tev[j] = half * (tev[j] + tem[j]);
        } else {
          ldv<VK>(te0 + (i * 6 + e) * L + ci.k, tev);
        }
        R anti[VK];
        R mfo[VK], mfm[VK];
        ldv<VK>(MF + erow(x, e) * LK + v, mfo);
        ldv<VK>(MF + fs.mir[x * 6 + e] * LK + v, mfm);
        FOR_V {
          const R mf = mfo[j], mfx = mfm[j];
          const R hi = mf * tev[j];
          const R lo = half * ((mf + tabs(mf)) * tri[j] - (mfx + tabs(mfx)) * trx[j]);
          anti[j] = hi - lo;
          sumlo[j] = sumlo[j] + lo;
          sp_[j] = sp_[j] - tmin(R(0), anti[j]);
          sm_[j] = sm_[j] + tmax(R(0), anti[j]);
        }
        stv<VK>(antifx + (m * nt + tz) * 6 * sc + (size_t)(i * 6 + e) * L + ci.k, anti);
      }
    }
    const R* o = ops + b * 3 * ft.SC * LK + x * LK + v;
    R tn[VK], tlo[VK], tlv[VK], td[VK], out[VK];
    FOR_V tn[j] = -sumlo[j] * ci.rar;
    stv<VK>(trl_tdcy + m * s.trab + (size_t)t * 3 * NL + (size_t)nf * NL + c, tn);
    ldv<VK>(o, tlo);
    ldv<VK>(o + ft.SC * LK, tlv);
    ldv<VK>(o + 2 * ft.SC * LK, td);
    const size_t q = (m * nt + tz) * sc + c;
    FOR_V {
      const R lo = td[j] + ab1 * tn[j] + ab2 * tlo[j] + ab3 * tlv[j];
      const R hx = tmax(R(0), mx[j]), hn = tmax(R(0), mn[j]);
      out[j] = tmax(hn, tmin(hx, fdiv(lo, tmax(thshld, ci.dp[j]))));
    }
    stv<VK>(trcr_lo + q, out);
    stv<VK>(s_plus + q, sp_);
    stv<VK>(s_mnus + q, sm_);
    stv<VK>(trold + q, tri);
  }
}

// Where k_trf_hi writes tracer x thickness and the new tracer: the state
// (member stride s.tr, tracer t at t * NL), or, for the shape probe, chunk
// scratch (member stride nt * NL, tracer t at (t - t0) * NL).
template <typename R>
struct TrOut {
  R* trdp;
  R* tr;
  size_t mstride;
  int tbase;
};

// R+/R- of trcadv2 (k_trcadv2's arithmetic) for frame cell xe at levels ve,
// from the staged old tracer and trcr_lo, AB3 slots, S+/S- and thickness; the
// bounds (before the clamp at zero) and the slots of/vof are returned for
// trcadv3
template <typename R, int VK, int LK>
__device__ __forceinline__ void limiters(const FrameSm& fs, const R* TO, const R* TL, const R* opq, const R* dpf,
                                         const R* arf, int S1, int xe, int ve, R ab2, R ab3, R rab1,
                                         R* Rp, R* Rm, R (&mx)[VK], R (&mn)[VK], R (&tof)[VK], R (&tvf)[VK]) {
  const R thshld = R(1.e-11);
  const uint2 nb = fs.nbr[xe];
  const int o = xe * LK + ve;
  R lc[VK], tc0[VK];
  ldv<VK>(TL + o, lc);
  ldv<VK>(TO + o, tc0);
  FOR_V { mx[j] = tmax(tc0[j], lc[j]); mn[j] = tmin(tc0[j], lc[j]); }
#pragma unroll
  for (int e = 0; e < 6; e++) {
    R aa[VK], bb[VK];
    ldv<VK>(TO + nb_at(nb, e) * LK + ve, aa);
    ldv<VK>(TL + nb_at(nb, e) * LK + ve, bb);
    FOR_V { mx[j] = tmax3(mx[j], aa[j], bb[j]); mn[j] = tmin3(mn[j], aa[j], bb[j]); }
  }
  R dp[VK], spl[VK], smn[VK], rp[VK], rm[VK];
  ldv<VK>(opq + o, tof);
  ldv<VK>(opq + S1 * LK + o, tvf);
  ldv<VK>(opq + 2 * S1 * LK + o, spl);
  ldv<VK>(opq + 3 * S1 * LK + o, smn);
  ldv<VK>(dpf + o, dp);
  const R ar = arf[xe];
  FOR_V {
    const R hx = tmax(R(0), mx[j]), hn = tmax(R(0), mn[j]);
    const R q_plus = ((hx - lc[j]) * dp[j] - (ab2 * tmin(R(0), tof[j]) + ab3 * tmax(R(0), tvf[j]))) * rab1 * ar;
    const R q_mnus = ((lc[j] - hn) * dp[j] + (ab2 * tmax(R(0), tof[j]) + ab3 * tmin(R(0), tvf[j]))) * rab1 * ar;
    rp[j] = tmax(R(0), tmin(R(1), fdiv(q_plus, tmax(spl[j], thshld))));
    rm[j] = tmax(R(0), tmin(R(1), fdiv(q_mnus, tmax(smn[j], thshld))));
  }
  stv<VK>(Rp + o, rp);
  stv<VK>(Rm + o, rm);
}

// trcadv2's limiters over the patch and its first ring, then trcadv3: the
// antidiffusive fluxes k_trf_lo stored are clipped with the limiters of
// their two cells and summed; the low-order tendency k_trf_lo stored
// (-sum of the low-order fluxes x rarea, rounded) is added; AB3 update of
// tracer x thickness; new tracer.
//
// Copies: the limiters' operands of tracer t (frames, slots, S+/S-) are
// staged while the block clips tracer t-1; the clip's operands of tracer t
// (fluxes, tendency, tracer x thickness) while it forms tracer t's limiters.
template <typename R, int VK, int GC>
__global__ void __launch_bounds__(64 * GC) k_trf_hi(Grid<R> g, Strides s, FrameTab ft,
    const StepParams* __restrict__ sp, int t0, int nt, const R* __restrict__ trl_tdcy, const R* trcdp,
    R* __restrict__ trc_tdcy, const R* __restrict__ delp, const R* __restrict__ trold,
    const R* __restrict__ trcr_lo, const R* __restrict__ s_plus, const R* __restrict__ s_mnus,
    const R* __restrict__ antifx, TrOut<R> out, size_t sc) {
  // trcdp (read) and out.trdp (written) are the same array in the step
  constexpr int LK = VK * GC;
  const size_t m = blockIdx.y;
  sp += m;
  if (!sp->active) return;
  // the member's tracers in this chunk (fim_member_set_tracers); the
  // scratch keeps the chunk's layout
  const int ntm = min(nt, sp->ntr - t0);
  if (ntm <= 0) return;
  const int L = g.L, N = g.N;
  const int nlc = (L + LK - 1) / LK;
  const int tile = blockIdx.x / nlc;
  const int k0 = (blockIdx.x - tile * nlc) * LK;
  const int lk = min(LK, L - k0);
  const int4 cn = ft.cnt[tile];
  const int C = cn.x, n1 = cn.y, n2 = cn.z, nre = cn.w;
  extern __shared__ __align__(16) unsigned char fsm[];
  const PatchLayout lay = PatchLayout::make<R>(ft, LK, true);
  R* const sr = reinterpret_cast<R*>(fsm);
  R* const TO = sr + lay.TO;
  R* const TL = sr + lay.TL;
  R* const opq = sr + lay.opq;
  R* const Rp = sr + lay.Rp;
  R* const Rm = sr + lay.Rm;
  R* const af = sr + lay.af;
  R* const tlt = sr + lay.tlt;
  R* const tdb = sr + lay.tdb;
  R* const dpf = sr + lay.dpf;
  R* const arf = sr + lay.arf;
  const FrameSm fs = load_tables<R>(g, ft, fsm, lay.tab, tile, C, n1, n2, nre);
  __syncthreads();
  for (int x = threadIdx.x; x < n1; x += blockDim.x) arf[x] = g.area[fs.cells[x]];
  const size_t NL = (size_t)N * L;
  const int nf = sp->nf, of = sp->of, vof = sp->vof;
  const R ab1 = R(sp->ab1), ab2 = R(sp->ab2), ab3 = R(sp->ab3);
  const R rab1 = R(1) / ab1;  // Q+/Q- divide by ab1: one reciprocal (as k_trcadv2)
  const R thshld = R(1.e-11);
  // the limiters' operands of tracer t0 + tz
  RowPlan<R, VK, GC> rp;
  rp.init(fs, ft.SC, n2, lk, L);
  auto stage_lim = [&](int tz) {
    const size_t so = (m * nt + tz) * sc + k0;
    rp.copy(TO, trold + so, fs, ft.SC, n2, lk, L);
    rp.copy(TL, trcr_lo + so, fs, ft.SC, n2, lk, L);
    const R* tc = trc_tdcy + m * s.trab + (size_t)(t0 + tz) * 3 * NL + k0;
    rp.copy(opq, tc + (size_t)of * NL, fs, ft.SC, n1, lk, L);
    rp.copy(opq + ft.S1 * LK, tc + (size_t)vof * NL, fs, ft.SC, n1, lk, L);
    rp.copy(opq + 2 * ft.S1 * LK, s_plus + so, fs, ft.SC, n1, lk, L);
    rp.copy(opq + 3 * ft.S1 * LK, s_mnus + so, fs, ft.SC, n1, lk, L);
    stage_commit();
  };
  // the clip's operands: the patch cells' six fluxes, low-order tendency
  // (slot nf) and tracer x thickness
  // (each thread copies the six flux rows of its own cell)
  const int afo = (rp.x0 < C && rp.v < lk) ? fs.cells[rp.x0] * 6 * L + rp.v : -1;
  auto stage_clip = [&](int tz) {
    const R* a = antifx + (m * nt + tz) * 6 * sc + k0;
    if (afo >= 0) {
#pragma unroll
      for (int e = 0; e < 6; e++)
        stage_copy<VK * (int)sizeof(R)>(af + erow(rp.x0, e) * LK + rp.v, a + afo + e * L);
    }
    const size_t tt = (size_t)(t0 + tz);
    rp.copy(tlt, trl_tdcy + m * s.trab + tt * 3 * NL + (size_t)nf * NL + k0, fs, ft.SC, C, lk, L);
    rp.copy(tdb, trcdp + m * s.tr + tt * NL + k0, fs, ft.SC, C, lk, L);
    stage_commit();
  };
  stage_rows<R, VK, GC>(dpf, delp + m * s.cell + k0, fs.cells, n1, lk, L);
  stage_lim(0);
  const int x = threadIdx.x / GC, v = (threadIdx.x - x * GC) * VK;
  const bool on = x < C && v < lk;
  for (int tz = 0; tz < ntm; tz++) {
    const int t = t0 + tz;
    stage_wait();
    __syncthreads();
    stage_clip(tz);
    // R+/R- of the thread's patch cell (its bounds and slots kept for
    // trcadv3), then of the ring-1 cells
    R mx[VK], mn[VK], tof[VK], tvf[VK];
    if (on) limiters<R, VK, LK>(fs, TO, TL, opq, dpf, arf, ft.S1, x, v, ab2, ab3, rab1, Rp, Rm, mx, mn, tof, tvf);
    for (int it = threadIdx.x; it < (n1 - C) * GC; it += blockDim.x) {
      const int xe = C + it / GC, ve = (it % GC) * VK;
      if (ve >= lk) continue;
      R mx2[VK], mn2[VK], tof2[VK], tvf2[VK];
      limiters<R, VK, LK>(fs, TO, TL, opq, dpf, arf, ft.S1, xe, ve, ab2, ab3, rab1, Rp, Rm, mx2, mn2, tof2, tvf2);
    }
    stage_wait();
    __syncthreads();
    if (tz + 1 < ntm) stage_lim(tz + 1);
    if (!on) continue;
    const int i = fs.cells[x];
    const int c = i * L + k0 + v;
    const int np = fs.np[x];
    const uint2 nb = fs.nbr[x];
    R rpc[VK], rmc[VK], at[VK];
    ldv<VK>(Rp + x * LK + v, rpc);
    ldv<VK>(Rm + x * LK + v, rmc);
    FOR_V at[j] = R(0);
#pragma unroll
    for (int e = 0; e < 6; e++) {
      if (e < 5 || e < np) {
        const int y = nb_at(nb, e);
        R a[VK], rpx[VK], rmx[VK];
        ldv<VK>(af + erow(x, e) * LK + v, a);
        ldv<VK>(Rp + y * LK + v, rpx);
        ldv<VK>(Rm + y * LK + v, rmx);
        FOR_V {
          R aa = a[j];
          if (aa >= R(0)) aa = aa * tmin(rmc[j], rpx[j]);
          else aa = aa * tmin(rpc[j], rmx[j]);
          at[j] = at[j] + aa;
        }
      }
    }
    const R rar = g.rarea[i];
    R tl[VK], tdv[VK], dp[VK], tn[VK], res[VK];
    ldv<VK>(tlt + x * LK + v, tl);
    ldv<VK>(tdb + x * LK + v, tdv);
    ldv<VK>(dpf + x * LK + v, dp);
    // the low-order tendency plus the clipped fluxes' divergence
    FOR_V tn[j] = tl[j] + (-at[j] * rar);
    stv<VK>(trc_tdcy + m * s.trab + (size_t)t * 3 * NL + (size_t)nf * NL + c, tn);
    const size_t ob = m * out.mstride + (size_t)(t - out.tbase) * NL + c;
    FOR_V {
      tdv[j] = tdv[j] + ab1 * tn[j] + ab2 * tof[j] + ab3 * tvf[j];
      const R hx = tmax(R(0), mx[j]), hn = tmax(R(0), mn[j]);
      res[j] = tmax(hn, tmin(hx, fdiv(tdv[j], tmax(thshld, dp[j]))));
    }
    stv<VK>(out.trdp + ob, tdv);
    stv<VK>(out.tr + ob, res);
  }
}

template <typename R, int VK, int GC>
void trf_chunks(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w, R* trc_edg,
                R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx, const R* delp, bool probe,
                const ChunkHook* hook) {
  constexpr int LK = VK * GC;
  const FrameTab& ft = w.ft;
  const size_t sc = (size_t)g.N * g.L;
  const int nlc = (g.L + LK - 1) / LK;
  const size_t sm_lo = PatchLayout::make<R>(ft, LK, false).bytes, sm_hi = PatchLayout::make<R>(ft, LK, true).bytes;
  dim3 grid((unsigned)(ft.ntile * nlc), l.members);
  const int tb = ft.SC * GC;
  for (int t0 = 0; t0 < g.T; t0 += w.tchunk) {
    const int nt = (g.T - t0 < w.tchunk) ? g.T - t0 : w.tchunk;
    if (hook && hook->fn) hook->fn(hook->arg, 0, t0, nt);
    FIM_KBEGIN(l, "k_trf_lo");
    k_trf_lo<R, VK, GC><<<grid, tb, sm_lo, l.stream>>>(g, s, ft, l.sp, t0, nt, massfx, trc_edg, tracr, trcdp,
                                                        trl_tdcy, delp, w.trcr_lo, w.s_plus, w.s_mnus, w.trold,
                                                        w.antifx, sc);
    FIM_KEND(l);
    // the probe sends the new tracer and tracer x thickness to scratch
    const TrOut<R> out = probe ? TrOut<R>{w.r_plus, w.r_mnus, (size_t)nt * sc, t0} : TrOut<R>{trcdp, tracr, s.tr, 0};
    FIM_KBEGIN(l, "k_trf_hi");
    k_trf_hi<R, VK, GC><<<grid, tb, sm_hi, l.stream>>>(g, s, ft, l.sp, t0, nt, trl_tdcy, trcdp, trc_tdcy, delp,
                                                        w.trold, w.trcr_lo, w.s_plus, w.s_mnus, w.antifx, out, sc);
    FIM_KEND(l);
    if (probe) return;  // the first chunk only
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

template <typename R>
void fused_dispatch(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w, R* trc_edg,
                    R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx, const R* delp, bool probe,
                    const ChunkHook* hook) {
  const int vk = tracer_vk(g, {trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, w.trcr_lo, w.s_plus,
                               w.s_mnus, w.trold, w.r_plus, w.r_mnus, w.antifx}, w.vk);
  const bool g4 = w.gc >= 4;
#define FIM_TRF(VKV)                                                                                            \
  do {                                                                                                          \
    if (g4) trf_chunks<R, VKV, 4>(l, g, s, w, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, probe, hook); \
    else trf_chunks<R, VKV, 2>(l, g, s, w, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, probe, hook);    \
  } while (0)
  if (vk == 4) FIM_TRF((sizeof(R) == 4 ? 4 : 2));
  else if (vk == 2) FIM_TRF(2);
  else FIM_TRF(1);
#undef FIM_TRF
}

template <typename R, int VK, int GC>
int prepare_one(const FrameTab& ft) {
  constexpr int LK = VK * GC;
  const size_t lo = PatchLayout::make<R>(ft, LK, false).bytes, hi = PatchLayout::make<R>(ft, LK, true).bytes;
  cudaError_t e = cudaFuncSetAttribute(k_trf_lo<R, VK, GC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lo);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_trf_hi<R, VK, GC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hi);
  return (int)e;
}

}  // namespace

// ---- cell patches ---------------------------------------------------------

int build_frames(int N, const int* prox, const int* proxs, const int* nprox, int side, FrameHost* F) {
  if (side < 1 || side > 8) return 1;
  std::vector<std::vector<int>> tiles;
  // the reference's IJ numbering: north pole, 10 rhombi of sl x sl cells in
  // rows of sl, south pole; a cell strictly inside a rhombus then has the
  // cells +-1 and +-sl among its neighbours
  const long long sl = std::llround(std::sqrt((N - 2) / 10.0));
  bool ij = sl >= 1 && 10 * sl * sl + 2 == N;
  auto has = [&](int c, int n) {
    for (int e = 0; e < nprox[c]; e++)
      if (prox[c * 6 + e] == n) return true;
    return false;
  };
  for (long long r = 0; ij && r < 10; r++)
    for (long long a = 1; ij && a + 1 < sl; a++)
      for (long long b = 1; ij && b + 1 < sl; b++) {
        const int c = (int)(1 + r * sl * sl + a * sl + b);
        if (!has(c, c - 1) || !has(c, c + 1) || !has(c, c - (int)sl) || !has(c, c + (int)sl)) ij = false;
      }
  if (ij) {
    tiles.push_back({0});
    for (long long r = 0; r < 10; r++)
      for (long long ta = 0; ta < sl; ta += side)
        for (long long tb = 0; tb < sl; tb += side) {
          std::vector<int> t;
          for (long long a = ta; a < std::min(ta + side, sl); a++)
            for (long long b = tb; b < std::min(tb + side, sl); b++) t.push_back((int)(1 + r * sl * sl + a * sl + b));
          tiles.push_back(t);
        }
    tiles.push_back({N - 1});
  } else {
    // any other numbering: grow each patch breadth-first from the lowest
    // unassigned cell
    std::vector<char> used(N, 0);
    const size_t cap = (size_t)side * side;
    for (int c0 = 0; c0 < N; c0++) {
      if (used[c0]) continue;
      std::vector<int> t{c0};
      used[c0] = 1;
      for (size_t q = 0; q < t.size() && t.size() < cap; q++)
        for (int e = 0; e < nprox[t[q]] && t.size() < cap; e++) {
          const int n = prox[t[q] * 6 + e];
          if (!used[n]) { used[n] = 1; t.push_back(n); }
        }
      std::sort(t.begin(), t.end());
      tiles.push_back(t);
    }
  }
  // frames
  const int nt = (int)tiles.size();
  std::vector<int> loc(N, -1);
  struct Fr { std::vector<int> cells; int C, n1, n2; std::vector<uint32_t> nbr; std::vector<uint16_t> mir, red; };
  std::vector<Fr> fr(nt);
  int S2 = 0, S1 = 0, SC = 0, SR = 0;
  for (int ti = 0; ti < nt; ti++) {
    Fr& f = fr[ti];
    f.cells = tiles[ti];
    f.C = (int)f.cells.size();
    for (int x = 0; x < f.C; x++) loc[f.cells[x]] = x;
    for (int ring = 0; ring < 2; ring++) {
      const int lo = ring == 0 ? 0 : f.C, hi = (int)f.cells.size();
      std::vector<int> add;
      for (int x = lo; x < hi; x++) {
        const int c = f.cells[x];
        for (int e = 0; e < nprox[c]; e++) {
          const int n = prox[c * 6 + e];
          if (loc[n] == -1) { loc[n] = -2; add.push_back(n); }
        }
      }
      std::sort(add.begin(), add.end());
      for (int n : add) { loc[n] = (int)f.cells.size(); f.cells.push_back(n); }
      if (ring == 0) f.n1 = (int)f.cells.size();
    }
    f.n2 = (int)f.cells.size();
    if (f.n2 > 255) {
      for (int c : f.cells) loc[c] = -1;
      return 2;
    }
    f.nbr.assign((size_t)f.n1 * 2, 0u);
    for (int x = 0; x < f.n1; x++)
      for (int e = 0; e < 6; e++) {
        const int l6 = loc[prox[f.cells[x] * 6 + e]];
        if (l6 < 0) { for (int c : f.cells) loc[c] = -1; return 3; }
        f.nbr[(size_t)x * 2 + e / 4] |= (uint32_t)l6 << (8 * (e % 4));
      }
    f.mir.assign((size_t)f.C * 6, 0);
    for (int x = 0; x < f.C; x++) {
      const int c = f.cells[x];
      for (int e = 0; e < 6; e++) {
        if (e >= nprox[c]) { f.mir[(size_t)x * 6 + e] = (uint16_t)erow(x, e); continue; }
        const int y = loc[prox[c * 6 + e]], p = proxs[c * 6 + e];
        if (y < f.C) {
          f.mir[(size_t)x * 6 + e] = (uint16_t)erow(y, p);
        } else {
          f.mir[(size_t)x * 6 + e] = (uint16_t)(6 * f.C + f.red.size());
          f.red.push_back((uint16_t)((y << 3) | p));
        }
      }
    }
    for (int c : f.cells) loc[c] = -1;
    S2 = std::max(S2, f.n2);
    S1 = std::max(S1, f.n1);
    SC = std::max(SC, f.C);
    SR = std::max(SR, (int)f.red.size());
  }
  S2 = (S2 + 3) & ~3;  // keeps the tables after the cell list 16-byte aligned
  S1 = (S1 + 1) & ~1;
  SR = std::max(2, (SR + 1) & ~1);
  F->ntile = nt; F->S2 = S2; F->S1 = S1; F->SC = SC; F->SR = SR; F->SE = 6 * SC + SR;
  F->cells.assign((size_t)nt * S2, 0);
  F->nbr.assign((size_t)nt * S1 * 2, 0u);
  F->cnt.assign((size_t)nt * 4, 0);
  F->mir.assign((size_t)nt * SC * 6, 0);
  F->red.assign((size_t)nt * SR, 0);
  for (int ti = 0; ti < nt; ti++) {
    const Fr& f = fr[ti];
    std::copy(f.cells.begin(), f.cells.end(), F->cells.begin() + (size_t)ti * S2);
    std::copy(f.nbr.begin(), f.nbr.end(), F->nbr.begin() + (size_t)ti * S1 * 2);
    std::copy(f.mir.begin(), f.mir.end(), F->mir.begin() + (size_t)ti * SC * 6);
    std::copy(f.red.begin(), f.red.end(), F->red.begin() + (size_t)ti * SR);
    F->cnt[(size_t)ti * 4 + 0] = f.C;
    F->cnt[(size_t)ti * 4 + 1] = f.n1;
    F->cnt[(size_t)ti * 4 + 2] = f.n2;
    F->cnt[(size_t)ti * 4 + 3] = (int)f.red.size();
  }
  return 0;
}

int check_frames(int N, const int* prox, const int* proxs, const int* nprox, const FrameHost& F) {
  std::vector<int> seen(N, 0);
  for (int t = 0; t < F.ntile; t++) {
    const int C = F.cnt[(size_t)t * 4], n1 = F.cnt[(size_t)t * 4 + 1], n2 = F.cnt[(size_t)t * 4 + 2],
              nre = F.cnt[(size_t)t * 4 + 3];
    if (C < 1 || C > F.SC || n1 > F.S1 || n2 > F.S2 || nre > F.SR || 6 * C + nre > F.SE) return 1;
    const int* cells = &F.cells[(size_t)t * F.S2];
    for (int x = 0; x < n2; x++)
      if (cells[x] < 0 || cells[x] >= N) return 2;
    for (int x = 0; x < C; x++) seen[cells[x]]++;
    for (int x = 0; x < n1; x++)
      for (int e = 0; e < 6; e++) {
        const int y = (F.nbr[((size_t)t * F.S1 + x) * 2 + e / 4] >> (8 * (e % 4))) & 255;
        if (y >= n2 || cells[y] != prox[cells[x] * 6 + e]) return 3;
      }
    for (int x = 0; x < C; x++) {
      const int c = cells[x];
      for (int e = 0; e < nprox[c]; e++) {
        const int row = F.mir[((size_t)t * F.SC + x) * 6 + e];
        int y, p;
        if (row < 6 * C) {
          y = row / 6;
          p = (row % 6) ^ (y & 1);
        } else {
          const int r = row - 6 * C;
          if (r >= nre) return 4;
          const int code = F.red[(size_t)t * F.SR + r];
          y = code >> 3;
          p = code & 7;
          if (y < C || y >= n1) return 5;
        }
        if (cells[y] != prox[c * 6 + e] || p != proxs[c * 6 + e]) return 6;
      }
    }
  }
  for (int i = 0; i < N; i++)
    if (seen[i] != 1) return 7;
  return 0;
}

template <typename R>
int prepare_tracers(const FrameTab& ft) {
  int e;
  if ((e = prepare_one<R, 1, 2>(ft)) || (e = prepare_one<R, 1, 4>(ft))) return e;
  if ((e = prepare_one<R, 2, 2>(ft)) || (e = prepare_one<R, 2, 4>(ft))) return e;
  if (sizeof(R) == 4) {
    if ((e = prepare_one<R, (sizeof(R) == 4 ? 4 : 2), 2>(ft)) || (e = prepare_one<R, (sizeof(R) == 4 ? 4 : 2), 4>(ft)))
      return e;
  }
  return 0;
}

template <typename R>
void launch_tracers_fused(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w,
                          R* trc_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx,
                          const R* delp, const ChunkHook* hook) {
  fused_dispatch<R>(l, g, s, w, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, false, hook);
}

// Autotuner: time k_trf_lo + k_trf_hi (first tracer chunk, results of
// k_trf_hi sent to scratch) for every (levels per thread, level tile) that
// the layout admits and keep the fastest.  The caller provides step
// parameters whose nf slot the next step overwrites, so the probe leaves no
// state behind.
template <typename R>
int tune_tracers(const Launch& l, const Grid<R>& g, const Strides& s, const TrcFusedScratch<R>& w, R* trc_edg,
                 R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx, const R* delp, int* best_vk,
                 int* best_gc, float* best_ms) {
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return (int)cudaGetLastError();
  if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return (int)cudaGetLastError(); }
  Launch lq = l;
  lq.prof = nullptr;
  lq.counter = nullptr;
  float best = 1e30f;
  int rc = 0;
  const int vmax = (int)(16 / sizeof(R));
  for (int gc : {2, 4}) {
    for (int vk = vmax; vk >= 1 && vk >= vmax / 2; vk /= 2) {
      TrcFusedScratch<R> wv = w;
      wv.vk = vk;
      wv.gc = gc;
      if (tracer_vk(g, {trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, w.trcr_lo}, vk) != vk) continue;
      float ms = 0.f;
      for (int rep = 0; rep < 3; rep++) {  // the first repetition warms up
        cudaEventRecord(a, lq.stream);
        fused_dispatch<R>(lq, g, s, wv, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp, true, nullptr);
        cudaEventRecord(b, lq.stream);
        if (cudaEventSynchronize(b) != cudaSuccess) { rc = (int)cudaGetLastError(); break; }
        float t = 0.f;
        cudaEventElapsedTime(&t, a, b);
        if (rep > 0) ms += t;
      }
      if (rc) break;
      if (ms < best) { best = ms; *best_vk = vk; *best_gc = gc; }
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
  template int prepare_tracers<R>(const FrameTab&);                                                           \
  template int tune_tracers<R>(const Launch&, const Grid<R>&, const Strides&, const TrcFusedScratch<R>&, R*, \
                               R*, R*, R*, R*, const R*, const R*, int*, int*, float*);
INSTANTIATE(float)
INSTANTIATE(double)

}  // namespace fim
