// C-ABI of the GB300 FIM dynamics step (declared in include/fim_gpu.h).
//
// The context owns the device copy of the grid tables, the derived per-cell
// and per-level fields of dyn_init, the AB3 step parameters, the per-member
// status words and the scratch buffers of the routines.  Entry points mirror
// the reference subroutines' argument lists; fields are device pointers, or
// host pointers staged through the device when the context was created with
// host_pointers = 1.  Nothing here aborts: every failure is a status code.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/fim_gpu.h"
#include "fim_internal.h"

using namespace fim;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct fim_state {
  void* f[FIM_NFIELDS] = {};
  size_t count[FIM_NFIELDS] = {};  // elements per member
  int slots[FIM_NFIELDS] = {};     // member slots held: M, or the member group for the step's work fields
  double* sums = nullptr;          // [M][8+T]
  float2* mpf = nullptr;           // FP32-mixed: float-float Montgomery potential [M][nvl*nip]
  void* thold = nullptr;           // FP32-mixed: theta seen by edgvar1 this step [M][nvl*nip]
  // FP32-mixed: FP64 copies of initial fields (fim_state_upload_f64), held
  // until the member's initial adjustment consumes them; [field * M + member]
  std::vector<double*> init64;
  // host buffers of fim_step_io, [field * M + member]
  std::vector<void*> host;
  cudaGraphExec_t graph = nullptr;
  long long graph_kernels = 0;
  int graph_gen = 0;  // the context's graph_gen the graph was captured under
};

struct fim_ctx {
  fim_config cfg{};
  int prec = FIM_PREC_F64;
  int N = 0, L = 0, T = 0, M = 1;
  size_t esz = 8;
  cudaStream_t stream = nullptr;
  // persistent cnuity1..4 (fim_set_persistent); graph_gen counts the changes,
  // so a state's step graph is captured again after one
  bool coop_on = false;
  CoopCfg coop{nullptr, 0u, 1000000000ull};
  int graph_gen = 0;
  // fim_step_io's copy streams (host to device, device to host) and events
  cudaStream_t io_in = nullptr, io_out = nullptr;
  // the branch of a step that forms the budget sums beside momtum (they share
  // no written data), forked from and joined to the step's stream
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int prio = 0;  // priority of the streams above (fim_config.stream_priority, clamped)
  std::vector<cudaEvent_t> io_ev;
  std::vector<void*> owned;          // device allocations freed at destroy
  std::vector<size_t> owned_bytes;   // their sizes, entry for entry
  Grid<double> gd{};
  Grid<float> gf{};
  Strides str{};
  Knobs kn{};
  std::vector<double> thetac, dpsig;
  std::vector<double> lat;           // cell latitudes (radians), for fim_state_synthetic
  double* d_synth = nullptr;         // device: lat [N], dpsig / sum(dpsig) [L]
  void* d_thetac = nullptr;
  std::vector<StepParams> h_sp;  // one per member
  StepParams* d_sp = nullptr;
  int* d_flags = nullptr;
  long long launches = 0;
  // scratch (sized for all members)
  void *antifx = nullptr, *delp_lo = nullptr, *p_plus = nullptr, *p_mnus = nullptr, *r_plus = nullptr,
       *r_mnus = nullptr;
  void *t_antiflx = nullptr, *t_trmin = nullptr, *t_trmax = nullptr, *t_trcr_lo = nullptr, *t_rp = nullptr,
       *t_rm = nullptr;
  int tchunk = 0;
  void *f_trcr_lo = nullptr, *f_sp = nullptr, *f_sm = nullptr, *f_trold = nullptr, *f_rp = nullptr,
       *f_rm = nullptr, *f_af = nullptr;
  int ftchunk = 0;
  int trc_vk = 0;  // levels per thread of the fused tracer kernels (0: widest that nvl allows)
  int trc_gc = 4;   // threads per cell of a patch: level tile of trc_vk * trc_gc levels
  FrameTab ftab{};  // cell patches of the fused tracer kernels (device tables)
  bool autotune = true, tuned = false;
  float tune_ms = 0.f;
  int TB = 0, dtratio = 6;  // class-B tracers and their time-step ratio
  int G = 1;                // members advanced together through the dynamics (member_group)
  void *cb_w = nullptr, *cb_F = nullptr, *cb_V = nullptr, *cb_fmx = nullptr, *cb_fmn = nullptr,
       *cb_flo = nullptr, *cb_flp = nullptr, *cb_fln = nullptr;
  void *du = nullptr, *dv = nullptr, *wu = nullptr, *wv = nullptr;
  void* e2w = nullptr;  // edgvar2 in the step: speed and gradient, 3 nvl nip per member of a group
  void *exsmo = nullptr, *exsmo2 = nullptr;
  double* gs_partial = nullptr;
  double* cpl_old = nullptr;  // physics coupling: the six gfs_*_old copies (6 nvl nip)
  double* gs_sums = nullptr;  // per-routine globsum output [M][8+T]
  Prof prof;
  std::string err;
};

namespace {

int set_err(fim_ctx* c, int code, const char* what, cudaError_t e = cudaSuccess) {
  if (c) {
    char buf[512];
    if (e != cudaSuccess) snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    else snprintf(buf, sizeof buf, "%s", what);
    c->err = buf;
  }
  return code;
}

#define CK(call, what)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) {                             \
      if (e_ == cudaErrorMemoryAllocation) {             \
        cudaGetLastError();                              \
        return set_err(c, FIM_ENOMEM, what, e_);         \
      }                                                  \
      return set_err(c, FIM_ECUDA, what, e_);            \
    }                                                    \
  } while (0)

int dalloc(fim_ctx* c, void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return set_err(c, e == cudaErrorMemoryAllocation ? FIM_ENOMEM : FIM_ECUDA, "cudaMalloc", e);
  }
  c->owned.push_back(*p);
  c->owned_bytes.push_back(bytes);
  return FIM_OK;
}

// frees a buffer dalloc gave out (no-op for null or unknown pointers)
void dfree(fim_ctx* c, void* p) {
  for (size_t k = 0; p && k < c->owned.size(); k++)
    if (c->owned[k] == p) {
      cudaFree(p);
      c->owned.erase(c->owned.begin() + k);
      c->owned_bytes.erase(c->owned_bytes.begin() + k);
      return;
    }
}

// element-wise precision changes between the FP32-mixed state and FP64 work
// arrays
__global__ void k_widen(const float* __restrict__ a, double* __restrict__ b, size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    b[q] = (double)a[q];
}
__global__ void k_narrow(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    b[q] = (float)a[q];
}
// x -> nearest float hi and the float nearest to the remainder: hi + lo
// carries x to ~48 bits (the float-float Montgomery potential)
__global__ void k_split(const double* __restrict__ a, float2* __restrict__ b, size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const double x = a[q];
    const float hi = (float)x;
    b[q] = make_float2(hi, (float)(x - (double)hi));
  }
}
// x -> the FP32 value the state will hold, kept in FP64
__global__ void k_round_f32(double* __restrict__ a, size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    a[q] = (double)(float)a[q];
}
dim3 conv_grid(size_t n) {
  const size_t b = (n + 255) / 256;
  return dim3((unsigned)(b < 152 * 16 ? (b ? b : 1) : 152 * 16));
}

template <typename R>
int upload_conv(fim_ctx* c, const double* src, size_t n, const R** dst) {
  std::vector<R> tmp(n);
  for (size_t q = 0; q < n; q++) tmp[q] = (R)src[q];
  void* p;
  int rc = dalloc(c, &p, n * sizeof(R));
  if (rc) return rc;
  CK(cudaMemcpy(p, tmp.data(), n * sizeof(R), cudaMemcpyHostToDevice), "upload table");
  *dst = (const R*)p;
  return FIM_OK;
}

int upload_int(fim_ctx* c, const std::vector<int>& v, const int** dst) {
  void* p;
  int rc = dalloc(c, &p, v.size() * sizeof(int));
  if (rc) return rc;
  CK(cudaMemcpy(p, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice), "upload int table");
  *dst = (const int*)p;
  return FIM_OK;
}

template <typename R>
Grid<R>& grid_of(fim_ctx* c);
template <>
Grid<double>& grid_of<double>(fim_ctx* c) { return c->gd; }
template <>
Grid<float>& grid_of<float>(fim_ctx* c) { return c->gf; }

// 0-based index tables from the grid's Fortran ones, validated: nprox 5 or
// 6, neighbours in range, and every edge has a mirror, prox(proxs(e),
// prox(e)) == i (edgvar3's two-sided averages and trcadv's mirror mass
// fluxes read the neighbour's side through it).
int index_tables(const fim_grid_desc* g, std::vector<int>& prox, std::vector<int>& proxs, std::vector<int>& nprox) {
  const int N = g->nip;
  if (N < 12 || !g->prox || !g->proxs || !g->nprox) return FIM_EINVAL;
  prox.assign((size_t)N * 6, 0);
  proxs.assign((size_t)N * 6, 0);
  nprox.assign(N, 0);
  for (int i = 0; i < N; i++) {
    nprox[i] = g->nprox[i];
    if (nprox[i] != 5 && nprox[i] != 6) return FIM_EINVAL;
    for (int e = 0; e < 6; e++) {
      const int p = g->prox[i * 6 + e] - 1;
      if (p < 0 || p >= N) return FIM_EINVAL;
      prox[i * 6 + e] = p;
      const int q = g->proxs[i * 6 + e];
      proxs[i * 6 + e] = (e < nprox[i]) ? q - 1 : -1;
      if (e < nprox[i] && (q < 1 || q > 6)) return FIM_EINVAL;
    }
  }
  for (int i = 0; i < N; i++)
    for (int e = 0; e < nprox[i]; e++) {
      const int x = prox[i * 6 + e];
      if (x == i || prox[x * 6 + proxs[i * 6 + e]] != i) return FIM_EINVAL;
    }
  return FIM_OK;
}

// The cell patches of the fused tracer kernels: 8 x 8 cells of a rhombus,
// with the frame tables uploaded once per context.
int build_patches(fim_ctx* c, const std::vector<int>& prox, const std::vector<int>& proxs,
                  const std::vector<int>& nprox) {
  FrameHost h;
  int side = 8;
  while (build_frames(c->N, prox.data(), proxs.data(), nprox.data(), side, &h) != 0) {
    if (--side < 1) return set_err(c, FIM_EINVAL, "tracer patches: a frame exceeds 255 cells");
  }
  FrameTab& f = c->ftab;
  f.ntile = h.ntile; f.S2 = h.S2; f.S1 = h.S1; f.SC = h.SC; f.SE = h.SE; f.SR = h.SR;
  void* p;
  int rc;
  if ((rc = dalloc(c, &p, h.cells.size() * sizeof(int)))) return rc;
  CK(cudaMemcpy(p, h.cells.data(), h.cells.size() * sizeof(int), cudaMemcpyHostToDevice), "patch cells");
  f.cells = (const int*)p;
  if ((rc = dalloc(c, &p, h.nbr.size() * sizeof(uint32_t)))) return rc;
  CK(cudaMemcpy(p, h.nbr.data(), h.nbr.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "patch neighbours");
  f.nbr = (const uint2*)p;
  if ((rc = dalloc(c, &p, h.cnt.size() * sizeof(int)))) return rc;
  CK(cudaMemcpy(p, h.cnt.data(), h.cnt.size() * sizeof(int), cudaMemcpyHostToDevice), "patch counts");
  f.cnt = (const int4*)p;
  if ((rc = dalloc(c, &p, h.mir.size() * sizeof(uint16_t)))) return rc;
  CK(cudaMemcpy(p, h.mir.data(), h.mir.size() * sizeof(uint16_t), cudaMemcpyHostToDevice), "patch mirrors");
  f.mir = (const unsigned short*)p;
  if ((rc = dalloc(c, &p, h.red.size() * sizeof(uint16_t)))) return rc;
  CK(cudaMemcpy(p, h.red.data(), h.red.size() * sizeof(uint16_t), cudaMemcpyHostToDevice), "patch ring edges");
  f.redge = (const unsigned short*)p;
  return FIM_OK;
}

template <typename R>
int build_grid(fim_ctx* c, const fim_grid_desc* g, const std::vector<double>& rarea, const std::vector<double>& corio,
               const std::vector<double>& grnd, const std::vector<double>& dfflen, const std::vector<double>& biharw,
               const std::vector<double>& smoo, const std::vector<int>& prox, const std::vector<int>& proxs,
               const std::vector<int>& nprox) {
  Grid<R>& G = grid_of<R>(c);
  const int N = c->N;
  G.N = N; G.L = c->L; G.T = c->T;
  int rc;
  { const int* t_; if ((rc = upload_int(c, prox, &t_))) return rc; G.prox = t_; }
  { const int* t_; if ((rc = upload_int(c, proxs, &t_))) return rc; G.proxs = t_; }
  { const int* t_; if ((rc = upload_int(c, nprox, &t_))) return rc; G.nprox = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, g->cs, (size_t)N * 24, &t_))) return rc; G.cs = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, g->sn, (size_t)N * 24, &t_))) return rc; G.sn = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, g->sidevec_c, (size_t)N * 12, &t_))) return rc; G.svc = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, g->sidevec_e, (size_t)N * 12, &t_))) return rc; G.sve = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, g->sideln, (size_t)N * 6, &t_))) return rc; G.sideln = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, g->area, (size_t)N, &t_))) return rc; G.area = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, rarea.data(), (size_t)N, &t_))) return rc; G.rarea = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, corio.data(), (size_t)N, &t_))) return rc; G.corio = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, grnd.data(), (size_t)N, &t_))) return rc; G.grndspd = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, g->hfcoef, (size_t)N * 36, &t_))) return rc; G.hfcoef = t_; }
  G.cxy = nullptr;
  if (g->corner_xy) {
    const R* t_;
    if ((rc = upload_conv<R>(c, g->corner_xy, (size_t)N * 12, &t_))) return rc;
    G.cxy = t_;
  }
  { const double* t_; if ((rc = upload_conv<double>(c, g->area, (size_t)N, &t_))) return rc; G.area_d = t_; }
  {
    std::vector<double> sv((size_t)N * 2, 0.0);
    for (int i = 0; i < N; i++)
      for (int e = 0; e < nprox[i]; e++) {
        sv[(size_t)i * 2 + 0] += g->sidevec_c[((size_t)i * 6 + e) * 2 + 0];
        sv[(size_t)i * 2 + 1] += g->sidevec_c[((size_t)i * 6 + e) * 2 + 1];
      }
    const R* t_;
    if ((rc = upload_conv<R>(c, sv.data(), sv.size(), &t_))) return rc;
    G.svsum = t_;
  }
  { const R* t_; if ((rc = upload_conv<R>(c, dfflen.data(), (size_t)c->L, &t_))) return rc; G.dfflen = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, biharw.data(), (size_t)c->L, &t_))) return rc; G.biharw = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, smoo.data(), (size_t)c->L + 1, &t_))) return rc; G.smoo = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, c->thetac.data(), (size_t)c->L, &t_))) return rc; G.thetac = t_; }
  { const R* t_; if ((rc = upload_conv<R>(c, c->dpsig.data(), (size_t)c->L, &t_))) return rc; G.dpsig = t_; }
  return FIM_OK;
}

Launch make_launch(fim_ctx* c, int members) {
  Launch l;
  l.stream = c->stream;
  l.members = members;
  l.sp = c->d_sp;
  l.flags = c->d_flags;
  l.counter = &c->launches;
  l.prof = &c->prof;
  l.coop = c->coop_on ? &c->coop : nullptr;
  return l;
}

int push_sp(fim_ctx* c) {
  // pageable source: the copy is staged before cudaMemcpyAsync returns
  CK(cudaMemcpyAsync(c->d_sp, c->h_sp.data(), sizeof(StepParams) * c->h_sp.size(), cudaMemcpyHostToDevice,
                     c->stream), "push step params");
  return FIM_OK;
}

// the post-dyn_init parameters of one member (dyn_init.F90:1092-1094:
// nf,of,vof = 0,2,1 in Fortran numbering, i.e. one abstart before use)
void reset_member(fim_ctx* c, int m) {
  StepParams& p = c->h_sp[m];
  p.its = 0;
  p.nf = -1;
  p.of = 1;
  p.vof = 0;
  p.ab1 = p.ab2 = p.ab3 = 0.;
  p.dt = c->cfg.dt;
  p.active = 1;
}

int check_launch(fim_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(c, FIM_ECUDA, what, e);
  return FIM_OK;
}

// host abstart mirror (abstart.F90:33-65, 0-based slots)
void host_abstart(StepParams& p, int its) {
  p.its = its;
  p.nf = (p.nf + 1) % 3;
  p.of = (p.of + 1) % 3;
  p.vof = (p.vof + 1) % 3;
  if (its == 1) { p.ab1 = p.dt; p.ab2 = 0.; p.ab3 = 0.; }
  if (its == 2) { p.ab1 = p.dt * 1.5; p.ab2 = -p.dt * .5; p.ab3 = 0.; }
  if (its == 3) { p.ab1 = p.dt * 23. / 12.; p.ab2 = -p.dt * 16. / 12.; p.ab3 = p.dt * 5. / 12.; }
}

// ---- scratch --------------------------------------------------------------
int ensure(fim_ctx* c, void** p, size_t elems) {
  if (*p) return FIM_OK;
  return dalloc(c, p, elems * c->esz);
}

int ensure_cnuity(fim_ctx* c, int members) {
  const size_t NL = (size_t)c->N * c->L * members;
  int rc;
  if ((rc = ensure(c, &c->antifx, NL * 6))) return rc;
  if ((rc = ensure(c, &c->delp_lo, NL))) return rc;
  if ((rc = ensure(c, &c->p_plus, NL))) return rc;
  if ((rc = ensure(c, &c->p_mnus, NL))) return rc;
  if ((rc = ensure(c, &c->r_plus, NL))) return rc;
  if ((rc = ensure(c, &c->r_mnus, NL))) return rc;
  return FIM_OK;
}

int ensure_trcadv(fim_ctx* c, int members) {
  if (c->t_antiflx) return FIM_OK;
  const size_t NL = (size_t)c->N * c->L;
  // bound the tracer chunk so the six scratch fields take at most ~12 GB
  size_t per_tracer = NL * members * 11 * c->esz;
  int tch = c->T;
  while (tch > 1 && per_tracer * tch > (size_t)12 << 30) tch = (tch + 1) / 2;
  c->tchunk = tch;
  const size_t n = NL * members * tch;
  int rc;
  if ((rc = ensure(c, &c->t_antiflx, n * 6))) return rc;
  if ((rc = ensure(c, &c->t_trmin, n))) return rc;
  if ((rc = ensure(c, &c->t_trmax, n))) return rc;
  if ((rc = ensure(c, &c->t_trcr_lo, n))) return rc;
  if ((rc = ensure(c, &c->t_rp, n))) return rc;
  if ((rc = ensure(c, &c->t_rm, n))) return rc;
  return FIM_OK;
}

// The strides of a state's fields in the step: with the fused tracer
// transport trc_edg holds theta's edge values only, 6 nvl nip a member.
Strides step_strides(const fim_ctx* c) {
  Strides s = c->str;
  if (c->kn.hi_order) s.tredg = (size_t)6 * c->L * c->N;
  return s;
}

int ensure_trc_fused(fim_ctx* c, int members) {
  if (c->f_trcr_lo) return FIM_OK;
  {
    const int e = c->prec == FIM_PREC_F64 ? prepare_tracers<double>(c->ftab) : prepare_tracers<float>(c->ftab);
    if (e) return set_err(c, FIM_ECUDA, "tracer kernel attributes", (cudaError_t)e);
  }
  const size_t NL = (size_t)c->N * c->L;
  // per tracer of a chunk: trcr_lo, S+, S-, the old tracer, the probe's two
  // outputs and six antidiffusive fluxes; chunks of at most ~48 GB (glvl 8,
  // nvl 64, 21 tracers: one chunk of 42 GB)
  size_t per_tracer = NL * members * 12 * c->esz;
  int tch = c->cfg.tracer_chunk > 0 ? std::min(c->T, c->cfg.tracer_chunk) : c->T;
  while (tch > 1 && per_tracer * tch > (size_t)48 << 30) tch = (tch + 1) / 2;
  c->ftchunk = tch;
  const size_t n = NL * members * tch;
  int rc;
  if ((rc = ensure(c, &c->f_trcr_lo, n))) return rc;
  if ((rc = ensure(c, &c->f_sp, n))) return rc;
  if ((rc = ensure(c, &c->f_sm, n))) return rc;
  if ((rc = ensure(c, &c->f_trold, n))) return rc;
  if ((rc = ensure(c, &c->f_rp, n))) return rc;
  if ((rc = ensure(c, &c->f_rm, n))) return rc;
  if ((rc = ensure(c, &c->f_af, n * 6))) return rc;
  return FIM_OK;
}

int ensure_momtum(fim_ctx* c, int members) {
  const size_t NL = (size_t)c->N * c->L * members;
  int rc;
  if ((rc = ensure(c, &c->du, NL))) return rc;
  if ((rc = ensure(c, &c->dv, NL))) return rc;
  if (c->cfg.hi_order_uv_comp && (rc = ensure(c, &c->e2w, 3 * NL))) return rc;
  if (c->kn.biharm) {
    if ((rc = ensure(c, &c->wu, NL))) return rc;
    if ((rc = ensure(c, &c->wv, NL))) return rc;
  }
  return FIM_OK;
}

int ensure_hybgen(fim_ctx* c, int members) {
  const size_t NI = (size_t)c->N * (c->L + 1) * members;
  int rc;
  if ((rc = ensure(c, &c->exsmo, NI))) return rc;
  if ((rc = ensure(c, &c->exsmo2, NI))) return rc;
  const int e = c->prec == FIM_PREC_F64 ? prepare_hybgen<double>(c->L) : prepare_hybgen<float>(c->L);
  if (e) return set_err(c, FIM_ECUDA, "hybgen kernel attributes", (cudaError_t)e);
  return FIM_OK;
}

int ensure_globsum(fim_ctx* c, int members) {
  if (c->gs_partial) return FIM_OK;
  int rc;
  if ((rc = dalloc(c, (void**)&c->gs_partial, globsum_partials(c->N, c->L, c->T, members) * sizeof(double)))) return rc;
  if ((rc = dalloc(c, (void**)&c->gs_sums, (size_t)members * (8 + c->T + c->TB) * sizeof(double)))) return rc;
  return FIM_OK;
}

int ensure_classb(fim_ctx* c, int members) {
  if (c->TB <= 0 || c->cb_w) return FIM_OK;
  const size_t NL = (size_t)c->N * c->L * members, NB = NL * c->TB;
  int rc;
  if ((rc = ensure(c, &c->cb_w, NL))) return rc;
  void** f[] = {&c->cb_F, &c->cb_V, &c->cb_fmx, &c->cb_fmn, &c->cb_flo, &c->cb_flp, &c->cb_fln};
  for (void** p : f)
    if ((rc = ensure(c, p, NB))) return rc;
  const int e = c->prec == FIM_PREC_F64 ? prepare_classb<double>(c->L) : prepare_classb<float>(c->L);
  if (e) return set_err(c, FIM_ECUDA, "class-B kernel attributes", (cudaError_t)e);
  return FIM_OK;
}

template <typename R>
ClassBScratch<R> classb_scratch(fim_ctx* c) {
  return ClassBScratch<R>{(R*)c->cb_w, (R*)c->cb_F, (R*)c->cb_V, (R*)c->cb_fmx, (R*)c->cb_fmn, (R*)c->cb_flo,
                          (R*)c->cb_flp, (R*)c->cb_fln};
}

// ---- host-pointer staging -------------------------------------------------
struct Stager {
  fim_ctx* c;
  bool host;
  std::vector<void*> bufs;
  struct Out { void* host; void* dev; size_t bytes; };
  std::vector<Out> outs;
  int rc = FIM_OK;
  explicit Stager(fim_ctx* c_) : c(c_), host(c_->cfg.host_pointers != 0) {}
  ~Stager() {
    for (void* p : bufs) cudaFreeAsync(p, c->stream);
  }
  // intent: 0 in, 1 inout, 2 out
  template <typename R>
  R* map(const R* p, size_t n, int intent) {
    if (!host || p == nullptr) return const_cast<R*>(p);
    void* d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, n * sizeof(R) + 16, c->stream);
    if (e != cudaSuccess) { cudaGetLastError(); rc = set_err(c, FIM_ENOMEM, "stage alloc", e); return nullptr; }
    bufs.push_back(d);
    if (intent != 2) {
      e = cudaMemcpyAsync(d, p, n * sizeof(R), cudaMemcpyHostToDevice, c->stream);
      if (e != cudaSuccess) { rc = set_err(c, FIM_ECUDA, "stage in", e); return nullptr; }
    } else {
      cudaMemsetAsync(d, 0, n * sizeof(R), c->stream);
    }
    if (intent != 0) outs.push_back({(void*)p, d, n * sizeof(R)});
    return (R*)d;
  }
  int finish() {
    if (rc) return rc;
    for (auto& o : outs) {
      cudaError_t e = cudaMemcpyAsync(o.host, o.dev, o.bytes, cudaMemcpyDeviceToHost, c->stream);
      if (e != cudaSuccess) return set_err(c, FIM_ECUDA, "stage out", e);
    }
    if (host) {
      cudaError_t e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) return set_err(c, FIM_ECUDA, "stage sync", e);
    }
    return FIM_OK;
  }
};

template <typename R>
int check_prec(fim_ctx* c) {
  if (!c) return FIM_EINVAL;
  if ((sizeof(R) == 8) != (c->prec == FIM_PREC_F64))
    return set_err(c, FIM_EINVAL, "entry-point family does not match the context precision");
  return FIM_OK;
}

// ---- per-routine implementations -----------------------------------------
template <typename R>
int edgvar_impl(fim_ctx* c, int which, const R* u_vel, const R* v_vel, const R* delp, const R* pres,
                const R* montg, const R* tracr, R* u_edg, R* v_edg, R* dp_edg, R* lp_edg, R* mont_edg,
                R* uvsq_edg, R* trc_edg) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  const size_t NL = (size_t)c->N * c->L, NI = (size_t)c->N * (c->L + 1), NE = NL * 6;
  Stager s(c);
  const R* du = s.map(u_vel, NL, 0);
  const R* dv = s.map(v_vel, NL, 0);
  const R* ddp = s.map(delp, NL, 0);
  const R* dpr = s.map(pres, NI, 0);
  const R* dmo = s.map(montg, NL, 0);
  const R* dtr = s.map(tracr, NL * c->T, 0);
  if (which == 2 && !grid_of<R>(c).cxy)
    return set_err(c, FIM_EINVAL, "edgvar2 needs the grid's corner_xy table");
  const int io = which == 1 ? 2 : 1;
  R* due = s.map(u_edg, NE, io);
  R* dve = s.map(v_edg, NE, io);
  R* dde = s.map(dp_edg, NE, 1);
  R* dle = s.map(lp_edg, NE, io);
  R* dme = s.map(mont_edg, NE, io);
  R* dqe = s.map(uvsq_edg, NE, io);
  R* dte = s.map(trc_edg, NE * c->T, 1);
  if (s.rc) return s.rc;
  Launch l = make_launch(c, 1);
  Grid<R>& g = grid_of<R>(c);
  if (which == 1) {
    launch_edgvar1<R>(l, g, c->str, c->kn.hi_order, du, dv, ddp, dpr, dmo, dtr, due, dve, dde, dle, dme, dqe, dte);
  } else if (which == 2) {
    R* w = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&w, 3 * NL * sizeof(R), c->stream);
    if (e != cudaSuccess) { cudaGetLastError(); return set_err(c, FIM_ENOMEM, "edgvar2 scratch", e); }
    s.bufs.push_back(w);
    launch_edgvar2<R>(l, g, c->str, du, dv, due, dve, dqe, w);
  } else {
    launch_edgvar3<R>(l, g, c->str, ddp, dtr, dde, dte, c->kn.hi_order ? c->T : 1);
  }
  if ((rc = check_launch(c, which == 1 ? "edgvar1" : which == 2 ? "edgvar2" : "edgvar3"))) return rc;
  return s.finish();
}

template <typename R>
int cnuity_impl(fim_ctx* c, const R* u_velo, const R* v_velo, const R* u_edg, const R* v_edg, const R* dp_edg,
                const R* lp_edg, R* delp, R* pres, R* exner, R* dp_tndcy, R* dplo_tndcy, R* massfx, R* omega) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  if ((rc = ensure_cnuity(c, c->G))) return rc;
  const size_t NL = (size_t)c->N * c->L, NI = (size_t)c->N * (c->L + 1), NE = NL * 6;
  Stager s(c);
  const R* a = s.map(u_velo, NL, 0);
  const R* b = s.map(v_velo, NL, 0);
  const R* ue = s.map(u_edg, NE, 0);
  const R* ve = s.map(v_edg, NE, 0);
  const R* de = s.map(dp_edg, NE, 0);
  const R* le = s.map(lp_edg, NE, 0);
  R* dp = s.map(delp, NL, 1);
  R* pr = s.map(pres, NI, 1);
  R* ex = s.map(exner, NI, 1);
  R* dt = s.map(dp_tndcy, NL * 3, 1);
  R* dl = s.map(dplo_tndcy, NL * 3, 1);
  R* mf = s.map(massfx, NE * 3, 1);
  R* om = s.map(omega, NL, 2);
  if (s.rc) return s.rc;
  if ((rc = push_sp(c))) return rc;
  CnuityScratch<R> w{(R*)c->antifx, (R*)c->delp_lo, (R*)c->p_plus, (R*)c->p_mnus, (R*)c->r_plus, (R*)c->r_mnus};
  launch_cnuity<R>(make_launch(c, 1), grid_of<R>(c), c->str, w, a, b, ue, ve, de, le, dp, pr, ex, dt, dl, mf, om);
  if ((rc = check_launch(c, "cnuity"))) return rc;
  return s.finish();
}

template <typename R>
int massadv_impl(fim_ctx* c, const R* u_velo, const R* v_velo, const R* u_edg, const R* v_edg, R* dp_edg,
                 const R* lp_edg, R* delp, R* pres, R* exner, R* dp_tndcy, R* massfx, R* omega) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  if ((rc = ensure_cnuity(c, c->G))) return rc;
  const size_t NL = (size_t)c->N * c->L, NI = (size_t)c->N * (c->L + 1), NE = NL * 6;
  Stager s(c);
  const R* a = s.map(u_velo, NL, 0);
  const R* b = s.map(v_velo, NL, 0);
  const R* ue = s.map(u_edg, NE, 0);
  const R* ve = s.map(v_edg, NE, 0);
  R* de = s.map(dp_edg, NE, 1);
  const R* le = s.map(lp_edg, NE, 0);
  R* dp = s.map(delp, NL, 1);
  R* pr = s.map(pres, NI, 1);
  R* ex = s.map(exner, NI, 1);
  R* dt = s.map(dp_tndcy, NL * 3, 1);
  R* mf = s.map(massfx, NE * 3, 1);
  R* om = s.map(omega, NL, 2);
  if (s.rc) return s.rc;
  if ((rc = push_sp(c))) return rc;
  CnuityScratch<R> w{(R*)c->antifx, (R*)c->delp_lo, (R*)c->p_plus, (R*)c->p_mnus, (R*)c->r_plus, (R*)c->r_mnus};
  launch_massadv<R>(make_launch(c, 1), grid_of<R>(c), c->str, w, a, b, ue, ve, de, le, dp, pr, ex, dt, mf, om);
  if ((rc = check_launch(c, "mass_adv"))) return rc;
  return s.finish();
}

template <typename R>
int trcadv_impl(fim_ctx* c, const R* trcr_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trclo_tdcy, const R* massfx,
                const R* delp) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  if ((rc = ensure_trcadv(c, c->G))) return rc;
  const size_t NL = (size_t)c->N * c->L, NE = NL * 6;
  Stager s(c);
  const R* te = s.map(trcr_edg, NE * c->T, 0);
  R* tr = s.map(tracr, NL * c->T, 1);
  R* td = s.map(trcdp, NL * c->T, 1);
  R* tt = s.map(trc_tdcy, NL * 3 * c->T, 1);
  R* tl = s.map(trclo_tdcy, NL * 3 * c->T, 1);
  const R* mf = s.map(massfx, NE * 3, 0);
  const R* dp = s.map(delp, NL, 0);
  if (s.rc) return s.rc;
  if ((rc = push_sp(c))) return rc;
  TrcadvScratch<R> w{(R*)c->t_antiflx, (R*)c->t_trmin, (R*)c->t_trmax, (R*)c->t_trcr_lo, (R*)c->t_rp, (R*)c->t_rm,
                     c->tchunk};
  launch_trcadv<R>(make_launch(c, 1), grid_of<R>(c), c->str, w, te, tr, td, tt, tl, mf, dp);
  if ((rc = check_launch(c, "trcadv"))) return rc;
  return s.finish();
}

template <typename R>
int momtum_impl(fim_ctx* c, R* u_velo, R* v_velo, const R* exner, R* relvor, const R* u_edg, const R* v_edg,
                const R* trcr_edg, const R* mont_edg, const R* uvsq_edg, R* u_tndcy, R* v_tndcy, const R* dp3d) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  if ((rc = ensure_momtum(c, c->G))) return rc;
  const size_t NL = (size_t)c->N * c->L, NI = (size_t)c->N * (c->L + 1), NE = NL * 6;
  Stager s(c);
  R* u = s.map(u_velo, NL, 1);
  R* v = s.map(v_velo, NL, 1);
  const R* ex = s.map(exner, NI, 0);
  R* rv = s.map(relvor, NL, 2);
  const R* ue = s.map(u_edg, NE, 0);
  const R* ve = s.map(v_edg, NE, 0);
  const R* te = s.map(trcr_edg, NE, 0);  // only tracer 1 (theta) is read
  const R* me = s.map(mont_edg, NE, 0);
  const R* qe = s.map(uvsq_edg, NE, 0);
  R* ut = s.map(u_tndcy, NL * 3, 1);
  R* vt = s.map(v_tndcy, NL * 3, 1);
  const R* dp = s.map(dp3d, NL, 0);
  if (s.rc) return s.rc;
  if ((rc = push_sp(c))) return rc;
  MomtumScratch<R> w{(R*)c->du, (R*)c->dv, (R*)c->wu, (R*)c->wv};
  launch_momtum<R>(make_launch(c, 1), grid_of<R>(c), c->str, c->kn, w, u, v, ex, rv, ue, ve, te, me, qe, ut, vt, dp);
  if ((rc = check_launch(c, "momtum"))) return rc;
  return s.finish();
}

template <typename R>
int hybgen_impl(fim_ctx* c, int its, const R* targt, R* us3d, R* vs3d, R* tr3d, R* sdot, R* ex3d, R* dp3d,
                R* pr3d) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  if (c->L > kMaxL) return set_err(c, FIM_EINVAL, "nvl exceeds the column-kernel limit");
  if ((rc = ensure_hybgen(c, c->M))) return rc;
  const size_t NL = (size_t)c->N * c->L, NI = (size_t)c->N * (c->L + 1);
  Stager s(c);
  const R* tg = targt ? s.map(targt, (size_t)c->L, 0) : grid_of<R>(c).thetac;
  R* u = s.map(us3d, NL, 1);
  R* v = s.map(vs3d, NL, 1);
  R* tr = s.map(tr3d, NL * c->T, 1);
  R* sd = s.map(sdot, NI, 2);
  R* ex = s.map(ex3d, NI, 1);
  R* dp = s.map(dp3d, NL, 1);
  R* pr = s.map(pr3d, NI, 1);
  if (s.rc) return s.rc;
  for (auto& p : c->h_sp) p.its = its;
  if ((rc = push_sp(c))) return rc;
  HybgenScratch<R> w{(R*)c->exsmo, (R*)c->exsmo2};
  launch_hybgen<R>(make_launch(c, 1), grid_of<R>(c), c->str, c->kn, w, tg, u, v, tr, sd, ex, dp, pr);
  if ((rc = check_launch(c, "hybgen"))) return rc;
  return s.finish();
}

template <typename R>
int hystat_impl(fim_ctx* c, int its, R* ph3d, const R* ex3d, R* mp3d, const R* dp3d, R* tr3d, R* trdp, R* psrf,
                R* ptdcy) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  const size_t NL = (size_t)c->N * c->L, NI = (size_t)c->N * (c->L + 1);
  Stager s(c);
  R* ph = s.map(ph3d, NI, 1);
  const R* ex = s.map(ex3d, NI, 0);
  R* mp = s.map(mp3d, NL, 2);
  const R* dp = s.map(dp3d, NL, 0);
  R* tr = s.map(tr3d, NL * c->T, 1);
  R* td = s.map(trdp, NL * c->T, 2);
  R* ps = s.map(psrf, (size_t)c->N, 1);
  R* pt = s.map(ptdcy, (size_t)c->N * 2, 1);
  if (s.rc) return s.rc;
  for (auto& p : c->h_sp) p.its = its;
  if ((rc = push_sp(c))) return rc;
  launch_hystat<R>(make_launch(c, 1), grid_of<R>(c), c->str, ph, ex, mp, dp, tr, td, ps, pt);
  if ((rc = check_launch(c, "hystat"))) return rc;
  return s.finish();
}

// cpl_run.F90:151-263 (callphy branch of cpl_dyn_to_phy)
template <typename R>
int cpl_dyn_to_phy_impl(fim_ctx* c, int its, int callphy, const R* pr3d, const R* us3d, const R* vs3d,
                        const R* ws3d, const R* tr3d, double* const gfs_in[10]) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  (void)its;
  if (!callphy) return FIM_OK;
  for (int q = 0; q < 10; q++)
    if (!gfs_in[q]) return FIM_EINVAL;
  if (!pr3d || !us3d || !vs3d || !ws3d || !tr3d) return FIM_EINVAL;
  const size_t NL = (size_t)c->N * c->L, NI = (size_t)c->N * (c->L + 1);
  if (!c->cpl_old && (rc = dalloc(c, (void**)&c->cpl_old, 6 * NL * sizeof(double)))) return rc;
  Stager s(c);
  const R* pr = s.map(pr3d, NI, 0);
  const R* u = s.map(us3d, NL, 0);
  const R* v = s.map(vs3d, NL, 0);
  const R* w = s.map(ws3d, NL, 0);
  const R* tr = s.map(tr3d, NL * c->T, 0);
  double* gfs[10];
  for (int q = 0; q < 10; q++) gfs[q] = s.map(gfs_in[q], q == 0 ? (size_t)c->N : NL, 2);
  if (s.rc) return s.rc;
  launch_cpl_dyn_to_phy<R>(make_launch(c, 1), grid_of<R>(c), pr, u, v, w, tr, gfs, c->cpl_old);
  if ((rc = check_launch(c, "cpl_dyn_to_phy"))) return rc;
  return s.finish();
}

// cpl_run.F90:266-536 (callphy branch of cpl_phy_to_dyn): the dynamics state
// and the precipitation / evaporation columns
template <typename R>
int cpl_phy_to_dyn_impl(fim_ctx* c, int its, int callphy, int addtend, int smoothtend, double dtp,
                        const double* const gfs_in[7], const double* const col_in[3], const R* dp3d, R* us3d,
                        R* vs3d, R* tr3d, R* rn2d, R* rc2d, R* qf2d) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  (void)its;
  if (!callphy) return FIM_OK;
  for (int q = 0; q < 7; q++)
    if (!gfs_in[q]) return FIM_EINVAL;
  for (int q = 0; q < 3; q++)
    if (!col_in[q]) return FIM_EINVAL;
  if (!us3d || !vs3d || !tr3d || !rn2d || !rc2d || !qf2d || (addtend && smoothtend && !dp3d)) return FIM_EINVAL;
  if (addtend && (!c->cpl_old || !(dtp > 0.)))
    return set_err(c, FIM_EINVAL, "cpl_phy_to_dyn with addtend needs a preceding cpl_dyn_to_phy and dtp > 0");
  const size_t NL = (size_t)c->N * c->L;
  Stager s(c);
  const double* gfs[7];
  for (int q = 0; q < 7; q++) gfs[q] = s.map(gfs_in[q], NL, 0);
  const double* col[3];
  for (int q = 0; q < 3; q++) col[q] = s.map(col_in[q], (size_t)c->N, 0);
  const R* dp = s.map(dp3d, NL, 0);
  R* u = s.map(us3d, NL, 1);
  R* v = s.map(vs3d, NL, 1);
  R* tr = s.map(tr3d, NL * c->T, 1);
  R* rn = s.map(rn2d, (size_t)c->N, 1);
  R* rcp = s.map(rc2d, (size_t)c->N, 1);
  R* qf = s.map(qf2d, (size_t)c->N, 1);
  if (s.rc) return s.rc;
  double* tend = nullptr;
  if (addtend) {
    const size_t bytes = (smoothtend ? 12 : 6) * NL * sizeof(double);
    cudaError_t e = cudaMallocAsync((void**)&tend, bytes, c->stream);
    if (e != cudaSuccess) { cudaGetLastError(); return set_err(c, FIM_ENOMEM, "coupling scratch", e); }
    s.bufs.push_back(tend);
  }
  launch_cpl_phy_to_dyn<R>(make_launch(c, 1), grid_of<R>(c), c->cfg.dt, dtp, addtend != 0, smoothtend != 0, gfs,
                           c->cpl_old, col, dp, u, v, tr, rn, rcp, qf, tend);
  if ((rc = check_launch(c, "cpl_phy_to_dyn"))) return rc;
  return s.finish();
}

template <typename R>
int globsum_impl(fim_ctx* c, const R* dp3d, const R* tr, const R* rn2d, const R* rc2d, const R* pr3d,
                 const R* ex3d, const R* qf2d, double* qtrcr, fim_budget* out) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  const int ntr = c->T + c->TB;
  if ((rc = ensure_globsum(c, c->M))) return rc;
  const size_t NL = (size_t)c->N * c->L, NI = (size_t)c->N * (c->L + 1);
  Stager s(c);
  const R* dp = s.map(dp3d, NL, 0);
  const R* t = s.map(tr, NL * ntr, 0);
  const R* rn = s.map(rn2d, (size_t)c->N, 0);
  const R* rcp = s.map(rc2d, (size_t)c->N, 0);
  const R* pr = s.map(pr3d, NI, 0);
  const R* ex = s.map(ex3d, NI, 0);
  const R* qf = s.map(qf2d, (size_t)c->N, 0);
  if (s.rc) return s.rc;
  if ((rc = push_sp(c))) return rc;
  launch_globsum<R>(make_launch(c, 1), grid_of<R>(c), c->str, ntr, dp, t, rn, rcp, pr, ex, qf, c->gs_partial,
                    c->gs_sums);
  if ((rc = check_launch(c, "globsum"))) return rc;
  if ((rc = s.finish())) return rc;
  std::vector<double> h(8 + ntr);
  CK(cudaMemcpyAsync(h.data(), c->gs_sums, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "globsum out");
  CK(cudaStreamSynchronize(c->stream), "globsum sync");
  if (qtrcr) for (int q = 0; q < ntr; q++) qtrcr[q] = h[8 + q];
  if (out) {
    out->qmass = h[0]; out->qmsqv = h[1]; out->qmsqw = h[2]; out->qmso3 = h[3];
    out->qmste = h[4]; out->qmstr = h[5]; out->qmstrn = h[6]; out->qmstrc = h[7];
  }
  return FIM_OK;
}

template <typename R>
int transp0_impl(fim_ctx* c, R* cumufx, const R* dp3d, R* dpinit) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  const size_t NL = (size_t)c->N * c->L;
  Stager s(c);
  R* cu = s.map(cumufx, NL * 6, 2);
  const R* dp = s.map(dp3d, NL, 0);
  R* di = s.map(dpinit, NL, 2);
  if (s.rc) return s.rc;
  if ((rc = push_sp(c))) return rc;
  launch_transp0<R>(make_launch(c, 1), grid_of<R>(c), c->str, 0, cu, dp, di);
  if ((rc = check_launch(c, "transp0"))) return rc;
  return s.finish();
}

template <typename R>
int transp1_impl(fim_ctx* c, R* cumufx, const R* massfx) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  const size_t NE = (size_t)c->N * c->L * 6;
  Stager s(c);
  R* cu = s.map(cumufx, NE, 1);
  const R* mf = s.map(massfx, NE * 3, 0);
  if (s.rc) return s.rc;
  if ((rc = push_sp(c))) return rc;
  launch_transp1<R>(make_launch(c, 1), grid_of<R>(c), c->str, cu, mf);
  if ((rc = check_launch(c, "transp1"))) return rc;
  return s.finish();
}

template <typename R>
int transp2_impl(fim_ctx* c, R* tracr, const R* cumufx, const R* dpinit, const R* dpfinl) {
  int rc = check_prec<R>(c);
  if (rc) return rc;
  if (c->TB <= 0) return FIM_OK;
  if ((rc = ensure_classb(c, c->G))) return rc;
  const size_t NL = (size_t)c->N * c->L;
  Stager s(c);
  R* tr = s.map(tracr, NL * (c->T + c->TB), 1);
  const R* cu = s.map(cumufx, NL * 6, 0);
  const R* di = s.map(dpinit, NL, 0);
  const R* df = s.map(dpfinl, NL, 0);
  if (s.rc) return s.rc;
  if ((rc = push_sp(c))) return rc;
  launch_transp2<R>(make_launch(c, 1), grid_of<R>(c), c->str, classb_scratch<R>(c), 0, c->TB, tr, cu, di, df);
  if ((rc = check_launch(c, "transp2"))) return rc;
  return s.finish();
}

// ---- fused step over the device-resident state ---------------------------
// The step's edge work fields are rewritten every step before they are read:
// with member groups they hold one group at a time.
bool group_field(int f) {
  return f == FIM_U_EDG || f == FIM_V_EDG || f == FIM_DP_EDG || f == FIM_LP_EDG || f == FIM_MONT_EDG ||
         f == FIM_UVSQ_EDG || f == FIM_GEOP_EDG || f == FIM_TRC_EDG;
}

template <typename R>
R* F(fim_state* st, int f) { return (R*)st->f[f]; }

// ---- the step with host transfers (fim_step_io) ------------------------------
// Each field a caller keeps on the host goes up before the first kernel that
// reads or writes it and comes down once its last writer of the step is done,
// on two copy streams beside the compute stream.  Stages of the step, in
// dyn_run order: A = hybgen + hystat (of the previous step) and the edge
// interpolation; C = cnuity or mass_adv (+ class-B transport); T = the tracer
// transport, chunk by chunk; U = momtum; E = the budget sums.
enum IoStage { kIoNone = 0, kIoA, kIoC, kIoT, kIoU, kIoE };
// names of the stages in the profiler's timeline marks
static const char* const kIoStageName[] = {"-", "A", "C", "T", "U", "E"};
struct IoClass {
  int up;     // stage before which the field must be on the device (kIoNone: output only)
  int down;   // stage after which it is final
  bool ab3;   // AB3 tendency field: slots of, vof up, slot nf down
};

bool io_class(int f, IoClass* k) {
  switch (f) {
    case FIM_US3D: case FIM_VS3D: *k = {kIoA, kIoU, false}; return true;
    case FIM_DP3D: case FIM_PR3D: case FIM_EX3D: case FIM_MASSFX: *k = {kIoA, kIoC, false}; return true;
    // hystat writes one of ptdcy's two time levels a step: the other goes up too
    case FIM_PH3D: case FIM_MP3D: case FIM_PSRF: case FIM_PTDCY: *k = {kIoA, kIoA, false}; return true;
    case FIM_TR3D: case FIM_TRDP: *k = {kIoA, kIoT, false}; return true;
    case FIM_CUMUFX: case FIM_DPINIT: *k = {kIoA, kIoE, false}; return true;
    case FIM_SDOT: *k = {kIoNone, kIoA, false}; return true;
    case FIM_WS3D: *k = {kIoNone, kIoC, false}; return true;
    case FIM_RELVOR: *k = {kIoNone, kIoU, false}; return true;
    case FIM_DP_TDCY: case FIM_DPL_TDCY: *k = {kIoC, kIoC, true}; return true;
    case FIM_TRC_TDCY: case FIM_TRL_TDCY: *k = {kIoT, kIoT, true}; return true;
    case FIM_U_TDCY: case FIM_V_TDCY: *k = {kIoU, kIoU, true}; return true;
    default: return false;  // the edge work fields live on the device only
  }
}

struct StepIo {
  fim_ctx* c = nullptr;
  fim_state* st = nullptr;
  int its = 1;
  std::vector<int> nf, of;  // per member, 0-based slots of the step (after its abstart)
  std::vector<int> vof;
  int tchunk = 1;
  int nev = 0;              // events handed out
  int64_t h2d = 0, d2h = 0;
  cudaEvent_t up_ev[kIoE + 1] = {};
  std::vector<cudaEvent_t> up_chunk;  // per tracer chunk
  int rc = FIM_OK;
  ChunkHook hook;
};

cudaEvent_t io_event(StepIo& io) {
  fim_ctx* c = io.c;
  if (io.nev == (int)c->io_ev.size()) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    c->io_ev.push_back(e);
  }
  return c->io_ev[io.nev++];
}

// copy of one member's field: whole (slot < 0, tracers [t0, t0+nt) for the
// tracer fields) or one AB3 slot of tracers [t0, t0+nt)
int io_copy(StepIo& io, int f, int m, int slot, int t0, int nt, bool up) {
  fim_ctx* c = io.c;
  fim_state* st = io.st;
  char* h = (char*)st->host[(size_t)f * c->M + m];
  if (!h) return FIM_OK;
  char* d = (char*)st->f[f] + (size_t)m * st->count[f] * c->esz;
  const size_t blk = (size_t)c->N * c->L * c->esz;
  cudaStream_t q = up ? c->io_in : c->io_out;
  const cudaMemcpyKind kind = up ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  cudaError_t e;
  size_t bytes;
  if (slot >= 0) {  // nt blocks of nvl x nip values, pitch three blocks
    const size_t off = ((size_t)t0 * 3 + slot) * blk;
    e = up ? cudaMemcpy2DAsync(d + off, 3 * blk, h + off, 3 * blk, blk, nt, kind, q)
           : cudaMemcpy2DAsync(h + off, 3 * blk, d + off, 3 * blk, blk, nt, kind, q);
    bytes = blk * nt;
  } else {
    size_t off = 0, n = st->count[f] * c->esz;
    if (f == FIM_TR3D || f == FIM_TRDP) {
      off = (size_t)t0 * blk;
      n = (size_t)nt * blk;
    }
    e = up ? cudaMemcpyAsync(d + off, h + off, n, kind, q) : cudaMemcpyAsync(h + off, d + off, n, kind, q);
    bytes = n;
  }
  if (e != cudaSuccess) return set_err(c, FIM_ECUDA, up ? "step io upload" : "step io download", e);
  (up ? io.h2d : io.d2h) += (int64_t)bytes;
  return FIM_OK;
}

// uploads needed before stage `stage` (tracers [t0, t0+nt) for kIoT), then an
// event the compute stream waits on
// a timeline mark on stream q when the profiler is on: "<what>.<stage>.<t0>"
void io_mark(StepIo& io, const char* what, int stage, int t0, cudaStream_t q) {
  fim_ctx* c = io.c;
  if (c->prof.on) c->prof.mark(std::string(what) + "." + kIoStageName[stage] + "." + std::to_string(t0), q);
}

int io_upload(StepIo& io, int stage, int t0, int nt, cudaEvent_t* done) {
  fim_ctx* c = io.c;
  int rc;
  io_mark(io, "up_begin", stage, t0, c->io_in);
  for (int f = 0; f < FIM_NFIELDS; f++) {
    IoClass k;
    if (!io_class(f, &k) || k.up != stage) continue;
    // From a member's second step on, the step opens with hybgen and hystat
    // of the step before (dyn_run.F90:119-132), which rewrite the layer
    // thicknesses, the Montgomery potential and tracer x thickness whole
    // before anything reads them (hybgen.F90:189-191, hystat.F90:58-101; the
    // remap forms trdp as it stores each tracer): the host's copies are not
    // needed.  Class-B tracers' trdp is not recomputed, so with ntrb > 0 trdp
    // goes up.
    if (io.its > 1 && (f == FIM_MP3D || f == FIM_DP3D || (f == FIM_TRDP && c->TB == 0))) continue;
    for (int m = 0; m < c->M; m++) {
      if (k.ab3) {
        const int n = (f == FIM_TRC_TDCY || f == FIM_TRL_TDCY) ? nt : 1, a = n == 1 && stage != kIoT ? 0 : t0;
        if ((rc = io_copy(io, f, m, io.of[m], a, n, true))) return rc;
        if ((rc = io_copy(io, f, m, io.vof[m], a, n, true))) return rc;
      } else if ((rc = io_copy(io, f, m, -1, 0, c->T + c->TB, true))) {
        return rc;
      }
    }
  }
  io_mark(io, "up_end", stage, t0, c->io_in);
  *done = io_event(io);
  if (!*done) return set_err(c, FIM_ECUDA, "step io event");
  CK(cudaEventRecord(*done, c->io_in), "step io record");
  return FIM_OK;
}

// downloads of the fields final after stage `stage`, behind the compute
// stream's work so far
int io_download(StepIo& io, int stage, int t0, int nt) {
  fim_ctx* c = io.c;
  io_mark(io, "computed", stage, t0, c->stream);
  cudaEvent_t e = io_event(io);
  if (!e) return set_err(c, FIM_ECUDA, "step io event");
  CK(cudaEventRecord(e, c->stream), "step io record");
  CK(cudaStreamWaitEvent(c->io_out, e, 0), "step io wait");
  io_mark(io, "down_begin", stage, t0, c->io_out);
  int rc;
  for (int f = 0; f < FIM_NFIELDS; f++) {
    IoClass k;
    if (!io_class(f, &k)) continue;
    // class-B tracers (after the class-A ones) come down with the budgets
    const bool trf = f == FIM_TR3D || f == FIM_TRDP;
    const bool here = k.down == stage || (trf && stage == kIoE && c->TB > 0);
    if (!here) continue;
    for (int m = 0; m < c->M; m++) {
      if (k.ab3) {
        const int n = (f == FIM_TRC_TDCY || f == FIM_TRL_TDCY) ? nt : 1, a = n == 1 && stage != kIoT ? 0 : t0;
        if ((rc = io_copy(io, f, m, io.nf[m], a, n, false))) return rc;
      } else if (trf) {
        const int a = stage == kIoE ? c->T : t0, n = stage == kIoE ? c->TB : nt;
        if ((rc = io_copy(io, f, m, -1, a, n, false))) return rc;
      } else if ((rc = io_copy(io, f, m, -1, 0, 0, false))) {
        return rc;
      }
    }
  }
  io_mark(io, "down_end", stage, t0, c->io_out);
  return FIM_OK;
}

int io_wait(StepIo& io, cudaEvent_t e) {
  fim_ctx* c = io.c;
  CK(cudaStreamWaitEvent(c->stream, e, 0), "step io wait");
  return FIM_OK;
}

void io_chunk_hook(void* arg, int phase, int t0, int nt) {
  StepIo& io = *(StepIo*)arg;
  if (io.rc) return;
  const int ci = t0 / io.tchunk;
  if (phase == 0) io.rc = io_wait(io, io.up_chunk[ci]);
  else io.rc = io_download(io, kIoT, t0, nt);
}

template <typename R>
int enqueue_step(fim_ctx* c, fim_state* st, StepIo* io = nullptr) {
  const int M = c->M;
  Launch l = make_launch(c, M);
  Grid<R>& g = grid_of<R>(c);
  const Strides s = step_strides(c);
  int rc;
  if (io && (rc = io_wait(*io, io->up_ev[kIoA]))) return rc;
  launch_step_begin(l, c->d_sp);
  // dyn_run.F90:119-132: the step opens with hybgen and hystat of step its-1
  // (skipped at a member's first step, after dyn_init's own adjustment)
  Launch lb = l;
  lb.boundary = 1;
  HybgenScratch<R> hw{(R*)c->exsmo, (R*)c->exsmo2};
  // the remap also forms hystat's floors and tracer x thickness (one pass
  // over the tracers instead of two)
  const bool trdp_done =
      launch_hybgen<R>(lb, g, s, c->kn, hw, g.thetac, F<R>(st, FIM_US3D), F<R>(st, FIM_VS3D), F<R>(st, FIM_TR3D),
                       F<R>(st, FIM_SDOT), F<R>(st, FIM_EX3D), F<R>(st, FIM_DP3D), F<R>(st, FIM_PR3D),
                       F<R>(st, FIM_TRDP));
  launch_hystat<R>(lb, g, s, F<R>(st, FIM_PH3D), F<R>(st, FIM_EX3D), F<R>(st, FIM_MP3D), F<R>(st, FIM_DP3D),
                   F<R>(st, FIM_TR3D), F<R>(st, FIM_TRDP), F<R>(st, FIM_PSRF), F<R>(st, FIM_PTDCY), st->mpf,
                   trdp_done);
  if (io && (rc = io_download(*io, kIoA, 0, 0))) return rc;
  // one member group and no host transfers: the budget sums run beside momtum
  const bool branch = !io && c->G == c->M && c->aux;
  // the dynamics of the step, one member group at a time; the edge work
  // fields and the scratch hold one group, the prognostic fields all members
  for (int m0 = 0; m0 < M; m0 += c->G) {
    const int gm = M - m0 < c->G ? M - m0 : c->G;
    Launch lg = l;
    lg.members = gm;
    lg.sp = c->d_sp + m0;
    lg.flags = c->d_flags + m0;
    auto P = [&](int f) {
      return (R*)st->f[f] + (st->slots[f] == M ? (size_t)m0 * st->count[f] : (size_t)0);
    };
    float2* mpf = st->mpf ? st->mpf + (size_t)m0 * st->count[FIM_MP3D] : nullptr;
    launch_edgvar1<R>(lg, g, s, c->kn.hi_order, P(FIM_US3D), P(FIM_VS3D), P(FIM_DP3D),
                      P(FIM_PR3D), P(FIM_MP3D), P(FIM_TR3D), P(FIM_U_EDG),
                      P(FIM_V_EDG), P(FIM_DP_EDG), P(FIM_LP_EDG), P(FIM_MONT_EDG),
                      P(FIM_UVSQ_EDG), P(FIM_TRC_EDG), mpf, (R*)st->thold);
    if (c->cfg.hi_order_uv_comp)
      launch_edgvar2<R>(lg, g, s, P(FIM_US3D), P(FIM_VS3D), P(FIM_U_EDG), P(FIM_V_EDG), P(FIM_UVSQ_EDG),
                        (R*)c->e2w);
    if (c->kn.hi_order) {
      // own-side dp edge values; the two-sided average is formed where it is
      // used (k_cnuity12); mass_adv reads the averaged dp edges, so it keeps
      // the pass.  The tracers' edge values are formed on chip by the tracer
      // kernels
      launch_edgvar3<R>(lg, g, s, P(FIM_DP3D), P(FIM_TR3D), P(FIM_DP_EDG), P(FIM_TRC_EDG),
                        1, c->cfg.flux_conserv_schm != 1);
    }
    CnuityScratch<R> cw{(R*)c->antifx, (R*)c->delp_lo, (R*)c->p_plus, (R*)c->p_mnus, (R*)c->r_plus, (R*)c->r_mnus};
    if (io && (rc = io_wait(*io, io->up_ev[kIoC]))) return rc;
    if (c->cfg.flux_conserv_schm == 1)
      launch_cnuity<R>(lg, g, s, cw, P(FIM_US3D), P(FIM_VS3D), P(FIM_U_EDG), P(FIM_V_EDG),
                       P(FIM_DP_EDG), P(FIM_LP_EDG), P(FIM_DP3D), P(FIM_PR3D),
                       P(FIM_EX3D), P(FIM_DP_TDCY), P(FIM_DPL_TDCY), P(FIM_MASSFX),
                       P(FIM_WS3D));
    else
      launch_massadv<R>(lg, g, s, cw, P(FIM_US3D), P(FIM_VS3D), P(FIM_U_EDG), P(FIM_V_EDG),
                        P(FIM_DP_EDG), P(FIM_LP_EDG), P(FIM_DP3D), P(FIM_PR3D),
                        P(FIM_EX3D), P(FIM_DP_TDCY), P(FIM_MASSFX), P(FIM_WS3D));
    if (c->TB > 0) {
      // class-B transport (dyn_run.F90:388-403); transp2/transp0 act at steps
      // with mod(its, dtratio) == 0, decided per member on the device
      launch_transp1<R>(lg, g, s, P(FIM_CUMUFX), P(FIM_MASSFX));
      launch_transp2<R>(lg, g, s, classb_scratch<R>(c), c->dtratio, c->TB, P(FIM_TR3D), P(FIM_CUMUFX),
                        P(FIM_DPINIT), P(FIM_DP3D));
      launch_transp0<R>(lg, g, s, c->dtratio, P(FIM_CUMUFX), P(FIM_DP3D), P(FIM_DPINIT));
    }
    if (io && (rc = io_download(*io, kIoC, 0, 0))) return rc;
    // momtum reads theta's edge values (edgvar1), the edge winds and the new
    // thicknesses, none of which the tracer transport writes, and writes
    // nothing it reads: with host transfers it runs first, so the step ends on
    // the tracer chunks whose results stream out as they finish
    auto momentum = [&]() -> int {
      if (io && (rc = io_wait(*io, io->up_ev[kIoU]))) return rc;
      MomtumScratch<R> mw{(R*)c->du, (R*)c->dv, (R*)c->wu, (R*)c->wv};
      launch_momtum<R>(lg, g, s, c->kn, mw, P(FIM_US3D), P(FIM_VS3D), P(FIM_EX3D),
                       P(FIM_RELVOR), P(FIM_U_EDG), P(FIM_V_EDG), P(FIM_TRC_EDG),
                       P(FIM_MONT_EDG), P(FIM_UVSQ_EDG), P(FIM_U_TDCY), P(FIM_V_TDCY),
                       P(FIM_DP3D), mpf, (const R*)st->thold);
      if (io && (rc = io_download(*io, kIoU, 0, 0))) return rc;
      return FIM_OK;
    };
    if (io && (rc = momentum())) return rc;
    if (c->kn.hi_order) {
      TrcFusedScratch<R> fw{(R*)c->f_trcr_lo, (R*)c->f_sp, (R*)c->f_sm, (R*)c->f_trold, (R*)c->f_rp, (R*)c->f_rm,
                            (R*)c->f_af,
                            io ? io->tchunk : c->ftchunk, c->trc_vk, c->trc_gc, c->ftab};
      launch_tracers_fused<R>(lg, g, s, fw, P(FIM_TRC_EDG), P(FIM_TR3D), P(FIM_TRDP),
                              P(FIM_TRC_TDCY), P(FIM_TRL_TDCY), P(FIM_MASSFX),
                              P(FIM_DP3D), io ? &io->hook : nullptr);
    } else {
      TrcadvScratch<R> tw{(R*)c->t_antiflx, (R*)c->t_trmin, (R*)c->t_trmax, (R*)c->t_trcr_lo, (R*)c->t_rp,
                          (R*)c->t_rm, c->tchunk};
      if (io) io_chunk_hook(io, 0, 0, c->T);
      launch_trcadv<R>(lg, g, s, tw, P(FIM_TRC_EDG), P(FIM_TR3D), P(FIM_TRDP),
                       P(FIM_TRC_TDCY), P(FIM_TRL_TDCY), P(FIM_MASSFX), P(FIM_DP3D));
      if (io) io_chunk_hook(io, 1, 0, c->T);
    }
    if (io && io->rc) return io->rc;
    if (branch) {
      // budgets of the state the step returns, on the branch stream beside
      // momtum: they read the thicknesses and tracers, which momtum does not
      // write, and momtum reads nothing they write
      CK(cudaEventRecord(c->ev_fork, c->stream), "step fork");
      CK(cudaStreamWaitEvent(c->aux, c->ev_fork, 0), "step fork");
      Launch la = l;
      la.stream = c->aux;
      launch_globsum<R>(la, g, s, c->T + c->TB, F<R>(st, FIM_DP3D), F<R>(st, FIM_TR3D), (const R*)nullptr,
                        (const R*)nullptr, F<R>(st, FIM_PR3D), F<R>(st, FIM_EX3D), (const R*)nullptr,
                        c->gs_partial, st->sums);
      CK(cudaEventRecord(c->ev_join, c->aux), "step join");
    }
    if (!io && (rc = momentum())) return rc;
  }
  if (branch) {
    CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "step join");
  } else {
    // budgets of the state the step returns
    launch_globsum<R>(l, g, s, c->T + c->TB, F<R>(st, FIM_DP3D), F<R>(st, FIM_TR3D), (const R*)nullptr,
                      (const R*)nullptr,
                      F<R>(st, FIM_PR3D), F<R>(st, FIM_EX3D), (const R*)nullptr, c->gs_partial, st->sums);
  }
  if (io && (rc = io_download(*io, kIoE, 0, 0))) return rc;
  return FIM_OK;
}

int ensure_all(fim_ctx* c) {
  int rc;
  if (!c->aux) {
    CK(cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, c->prio), "step branch stream");
    CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "step branch event");
    CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "step branch event");
  }
  if ((rc = ensure_cnuity(c, c->G))) return rc;
  if (c->kn.hi_order) {
    if ((rc = ensure_trc_fused(c, c->G))) return rc;
  } else if ((rc = ensure_trcadv(c, c->G))) return rc;
  if ((rc = ensure_momtum(c, c->G))) return rc;
  if ((rc = ensure_hybgen(c, c->M))) return rc;
  if ((rc = ensure_globsum(c, c->M))) return rc;
  if ((rc = ensure_classb(c, c->G))) return rc;
  return FIM_OK;
}

template <typename R>
R* FM(fim_ctx* c, fim_state* st, int f, int m) { return (R*)st->f[f] + (size_t)m * st->count[f]; }

// The initial fields dyn_init's adjustment reads (besides the state it
// recomputes): winds, thicknesses, pressures, Exner function, surface
// geopotential (ph3d's bottom interface) and tracers.
bool init_input(int f) {
  return f == FIM_US3D || f == FIM_VS3D || f == FIM_DP3D || f == FIM_PR3D || f == FIM_EX3D || f == FIM_PH3D ||
         f == FIM_TR3D;
}

// dyn_init.F90:870-906,1037 for member m of an FP32-mixed state, in FP64:
// hybgen, the pressures and thicknesses of the new interfaces and hystat run
// on FP64 copies of the member's fields (the fim_state_upload_f64 copies
// where given, else the FP32 fields widened), and the results are rounded
// into the state once; hystat runs on the rounded tracers and thicknesses,
// and the Montgomery potential keeps its float-float pair.
// Run once per member, so the state a forecast starts from does not carry
// the FP32 rounding of the adjustment's column arithmetic (the Exner
// function in particular, which the pressure gradient sees through the
// Montgomery potential).
int adjust_member_f64(fim_ctx* c, fim_state* st, int m) {
  const int used[] = {FIM_US3D, FIM_VS3D, FIM_DP3D, FIM_PR3D, FIM_EX3D, FIM_PH3D,
                      FIM_MP3D, FIM_TR3D, FIM_TRDP, FIM_SDOT, FIM_PSRF, FIM_PTDCY};
  const size_t NI = (size_t)c->N * (c->L + 1);
  size_t total = 2 * NI;  // hybgen's two smoothed-interface scratch arrays
  for (int f : used) total += st->count[f];
  void* blk = nullptr;
  int rc = dalloc(c, &blk, total * sizeof(double));
  if (rc) return rc;
  double* w[FIM_NFIELDS] = {};
  double* q = (double*)blk;
  for (int f : used) {
    w[f] = q;
    q += st->count[f];
  }
  HybgenScratch<double> hw{q, q + NI};
  cudaStream_t str = c->stream;
  for (int f : used) {
    const size_t n = st->count[f];
    float* src = (float*)st->f[f] + (size_t)m * n;
    double* staged = st->init64[(size_t)f * c->M + m];
    if (staged)
      CK(cudaMemcpyAsync(w[f], staged, n * sizeof(double), cudaMemcpyDeviceToDevice, str), "adjustment input");
    else
      k_widen<<<conv_grid(n), 256, 0, str>>>(src, w[f], n);
  }
  const int e = prepare_hybgen<double>(c->L);
  if (e) { dfree(c, blk); return set_err(c, FIM_ECUDA, "hybgen kernel attributes", (cudaError_t)e); }
  Launch l = make_launch(c, 1);
  l.sp = c->d_sp + m;
  l.flags = c->d_flags + m;
  Grid<double>& g = c->gd;
  launch_hybgen<double>(l, g, c->str, c->kn, hw, g.thetac, w[FIM_US3D], w[FIM_VS3D], w[FIM_TR3D], w[FIM_SDOT],
                        w[FIM_EX3D], w[FIM_DP3D], w[FIM_PR3D]);
  launch_prdp_from_ex<double>(l, g, c->str, w[FIM_EX3D], w[FIM_PR3D], w[FIM_DP3D]);
  // hystat then sees the potential temperature, tracers, thicknesses and
  // surface geopotential the FP32 state will hold: the Montgomery potential
  // is exact for that theta, so the step's pressure gradient -grad(M) +
  // Pi grad(theta) does not pick up theta's rounding (x Pi ~ 1000) as a
  // force.  The Exner function stays FP64 here.
  for (int f : {FIM_TR3D, FIM_DP3D, FIM_PH3D})
    k_round_f32<<<conv_grid(st->count[f]), 256, 0, str>>>(w[f], st->count[f]);
  CK(cudaMemsetAsync(w[FIM_PSRF], 0, st->count[FIM_PSRF] * sizeof(double), str), "zero psrf");
  CK(cudaMemsetAsync(w[FIM_PTDCY], 0, st->count[FIM_PTDCY] * sizeof(double), str), "zero ptdcy");
  launch_hystat<double>(l, g, c->str, w[FIM_PH3D], w[FIM_EX3D], w[FIM_MP3D], w[FIM_DP3D], w[FIM_TR3D],
                        w[FIM_TRDP], w[FIM_PSRF], w[FIM_PTDCY]);
  for (int f : used) {
    const size_t n = st->count[f];
    k_narrow<<<conv_grid(n), 256, 0, str>>>(w[f], (float*)st->f[f] + (size_t)m * n, n);
  }
  const size_t nm = st->count[FIM_MP3D];
  k_split<<<conv_grid(nm), 256, 0, str>>>(w[FIM_MP3D], st->mpf + (size_t)m * nm, nm);
  if ((rc = check_launch(c, "FP64 initial adjustment"))) return rc;
  // the work arrays and the member's FP64 inputs are released once the
  // kernels reading them are done
  CK(cudaStreamSynchronize(str), "FP64 initial adjustment");
  dfree(c, blk);
  for (int f = 0; f < FIM_NFIELDS; f++) {
    double*& p = st->init64[(size_t)f * c->M + m];
    dfree(c, p);
    p = nullptr;
  }
  return FIM_OK;
}

// dyn_init.F90:870-906,1037-1094 for members [m0, m0+nm)
template <typename R>
int state_init_impl(fim_ctx* c, fim_state* st, int m0, int nm) {
  int rc;
  if ((rc = ensure_all(c))) return rc;
  for (int m = m0; m < m0 + nm; m++) {
    c->h_sp[m].its = 0;
    c->h_sp[m].active = 1;
  }
  if ((rc = push_sp(c))) return rc;
  Launch l = make_launch(c, nm);
  l.sp = c->d_sp + m0;
  l.flags = c->d_flags + m0;
  Grid<R>& g = grid_of<R>(c);
  HybgenScratch<R> hw{(R*)c->exsmo, (R*)c->exsmo2};
  auto P = [&](int f) { return FM<R>(c, st, f, m0); };
  if constexpr (sizeof(R) == 4) {
    for (int m = m0; m < m0 + nm; m++)
      if ((rc = adjust_member_f64(c, st, m))) return rc;
  } else {
    launch_hybgen<R>(l, g, c->str, c->kn, hw, g.thetac, P(FIM_US3D), P(FIM_VS3D), P(FIM_TR3D), P(FIM_SDOT),
                     P(FIM_EX3D), P(FIM_DP3D), P(FIM_PR3D));
    launch_prdp_from_ex<R>(l, g, c->str, P(FIM_EX3D), P(FIM_PR3D), P(FIM_DP3D));
    CK(cudaMemsetAsync(P(FIM_PSRF), 0, nm * st->count[FIM_PSRF] * c->esz, c->stream), "zero psrf");
    CK(cudaMemsetAsync(P(FIM_PTDCY), 0, nm * st->count[FIM_PTDCY] * c->esz, c->stream), "zero ptdcy");
    launch_hystat<R>(l, g, c->str, P(FIM_PH3D), P(FIM_EX3D), P(FIM_MP3D), P(FIM_DP3D), P(FIM_TR3D), P(FIM_TRDP),
                     P(FIM_PSRF), P(FIM_PTDCY));
  }
  if (c->TB > 0)  // dyn_init.F90:1096-1097
    launch_transp0<R>(l, g, c->str, 0, P(FIM_CUMUFX), P(FIM_DP3D), P(FIM_DPINIT));
  const int zero[] = {FIM_U_TDCY, FIM_V_TDCY, FIM_DP_TDCY, FIM_DPL_TDCY, FIM_TRC_TDCY, FIM_TRL_TDCY, FIM_MASSFX};
  for (int f : zero) CK(cudaMemsetAsync(P(f), 0, nm * st->count[f] * c->esz, c->stream), "zero tendencies");
  for (int m = m0; m < m0 + nm; m++) reset_member(c, m);
  if ((rc = push_sp(c))) return rc;
  if ((rc = check_launch(c, "state init"))) return rc;
  CK(cudaStreamSynchronize(c->stream), "state init sync");
  return FIM_OK;
}

}  // namespace

namespace {

// Shape autotuning of the fused tracer kernels, once per context before the
// first step is captured: the probe runs with every active member's step
// parameters advanced one slot (as k_step_begin will), so the AB3 tendency
// slot it writes is the one the coming step overwrites.
template <typename R>
int autotune_impl(fim_ctx* c, fim_state* st) {
  std::vector<StepParams> next = c->h_sp;
  for (auto& p : next) {
    p.nf = (p.nf + 1) % 3;
    p.of = (p.of + 1) % 3;
    p.vof = (p.vof + 1) % 3;
  }
  CK(cudaMemcpyAsync(c->d_sp, next.data(), sizeof(StepParams) * next.size(), cudaMemcpyHostToDevice, c->stream),
     "tune params");
  Launch l = make_launch(c, c->G < c->M ? c->G : c->M);
  TrcFusedScratch<R> fw{(R*)c->f_trcr_lo, (R*)c->f_sp, (R*)c->f_sm, (R*)c->f_trold, (R*)c->f_rp, (R*)c->f_rm,
                            (R*)c->f_af,
                        c->ftchunk, c->trc_vk, c->trc_gc, c->ftab};
  int vk = c->trc_vk, gc = c->trc_gc;
  const int e = tune_tracers<R>(l, grid_of<R>(c), step_strides(c), fw, F<R>(st, FIM_TRC_EDG), F<R>(st, FIM_TR3D),
                                F<R>(st, FIM_TRDP), F<R>(st, FIM_TRC_TDCY), F<R>(st, FIM_TRL_TDCY),
                                F<R>(st, FIM_MASSFX), F<R>(st, FIM_DP3D), &vk, &gc, &c->tune_ms);
  if (e) return set_err(c, FIM_ECUDA, "tracer shape autotuning", (cudaError_t)e);
  c->trc_vk = vk;
  c->trc_gc = gc;
  c->tuned = true;
  return push_sp(c);
}

}  // namespace

// Device address of the allocation-free cnuity's static scratch array on the
// current device (defined with fim_cnuity_noalloc below).
int cnuity_static_addr(fim_ctx* c, unsigned char** out);

// ============================== extern "C" ==================================
extern "C" {

int fim_ctx_create(const fim_grid_desc* g, const fim_config* cfg, fim_ctx** out) {
  if (!g || !cfg || !out) return FIM_EINVAL;
  *out = nullptr;
  if (cfg->nvl < 4 || cfg->nvl > kMaxL || cfg->ntra < 4 || cfg->ntra > 32 || g->nip < 12 || cfg->dt <= 0.)
    return FIM_EINVAL;
  // kernels index one member's edge field (nvl x 6 x nip) with 32-bit offsets
  if ((long long)g->nip * 6 * (cfg->nvl + 1) > 2147483647LL) return FIM_EINVAL;
  if (cfg->flux_conserv_schm != 1 && cfg->flux_conserv_schm != 2) return FIM_ENOTSUP;
  if (cfg->pure_sig) return FIM_ENOTSUP;
  if (cfg->remap_optn < 1 || cfg->remap_optn > 3) return FIM_EINVAL;
  if (cfg->precision != FIM_PREC_F64 && cfg->precision != FIM_PREC_F32) return FIM_EINVAL;
  if (cfg->ntrb < 0 || cfg->ntra + cfg->ntrb > 32 || (cfg->ntrb > 0 && cfg->dtratio < 1)) return FIM_EINVAL;
  if (cfg->member_group < 0) return FIM_EINVAL;
  if (cfg->hi_order_uv_comp && !g->corner_xy) return FIM_EINVAL;  // edgvar2 needs corner_xy
  if (!cfg->thetac || !cfg->dpsig || !g->prox || !g->proxs || !g->nprox || !g->area || !g->cs || !g->sn ||
      !g->sidevec_c || !g->sidevec_e || !g->sideln || !g->hfcoef || !g->lat)
    return FIM_EINVAL;
  fim_ctx* c = new (std::nothrow) fim_ctx;
  if (!c) return FIM_ENOMEM;
  c->cfg = *cfg;
  c->prec = cfg->precision;
  c->esz = c->prec == FIM_PREC_F64 ? 8 : 4;
  c->N = g->nip;
  c->L = cfg->nvl;
  c->T = cfg->ntra;
  c->M = cfg->members < 1 ? 1 : cfg->members;
  c->thetac.assign(cfg->thetac, cfg->thetac + c->L);
  c->dpsig.assign(cfg->dpsig, cfg->dpsig + c->L);
  c->lat.assign(g->lat, g->lat + c->N);
  c->TB = cfg->ntrb;
  c->dtratio = cfg->dtratio;
  c->G = (cfg->member_group > 0 && cfg->member_group < c->M) ? cfg->member_group : c->M;
  c->str = make_strides(c->N, c->L, c->T, c->TB);
  // FIM_TRC_VK=1|2|4 and FIM_TRC_GC=2|4 pin the fused tracer kernels'
  // shape (levels per thread, threads per cell); FIM_AUTOTUNE=0 keeps the
  // default shape untimed
  if (const char* v = getenv("FIM_TRC_VK")) c->trc_vk = atoi(v);
  if (const char* v = getenv("FIM_TRC_GC")) c->trc_gc = atoi(v) >= 4 ? 4 : 2;
  if (const char* v = getenv("FIM_AUTOTUNE")) c->autotune = atoi(v) != 0;
  if (getenv("FIM_TRC_VK") || getenv("FIM_TRC_GC")) c->autotune = false;
  const int N = c->N, L = c->L;
  std::vector<int> prox, proxs, nprox;
  if (index_tables(g, prox, proxs, nprox) != FIM_OK) { delete c; return FIM_EINVAL; }
  // derived fields (dyn_init.F90:309-338,752-767)
  std::vector<double> rarea(N), corio(N), grnd(N), dfflen(L), biharw(L), smoo(L + 1, 0.0);
  for (int i = 0; i < N; i++) {
    corio[i] = kOmegx2 * std::sin(g->lat[i]);
    rarea[i] = 1. / g->area[i];
    grnd[i] = kEarthRad * 2. * kPi * std::cos(g->lat[i]) / 86164.;
  }
  const int ndamp = (int)(0.1 * L);
  for (int k = 1; k <= L; k++) {
    double wgt = std::max(0., (double)(k - L + ndamp) / (double)ndamp);
    dfflen[k - 1] = cfg->dt * (cfg->veldff_bkgnd * (1. - wgt) + std::max(cfg->veldff_bkgnd, cfg->veldff_boost) * wgt);
  }
  double dmax = dfflen[0];
  for (int k = 1; k < L; k++) dmax = std::max(dmax, dfflen[k]);
  for (int k = cfg->kbl + 2; k <= L; k++) {
    double d1 = (double)((cfg->kbl + 1) - k), d2 = (double)((L + 1) - k);
    smoo[k - 1] = cfg->dt * cfg->intfc_smooth * (d1 * d1 / (9. + d1 * d1)) * (d2 * d2 / (9. + d2 * d2));
  }
  int biharm = 0;
  for (int k = 1; k <= L; k++) {
    double w = 0.;
    if (k >= cfg->biharm_frst && k <= cfg->biharm_last) w = 1.;
    if (cfg->biharm_frst > 1 && cfg->biharm_frst < L) w = std::max(0., std::min(1., .5 + .2 * (double)(k - cfg->biharm_frst)));
    if (cfg->biharm_last > 1 && cfg->biharm_last < L) w = std::max(0., std::min(1., .5 + .2 * (double)(cfg->biharm_last - k)));
    biharw[k - 1] = w;
    if (w > 0.) biharm = 1;
    dfflen[k - 1] = dfflen[k - 1] * (1. + 4. * w * w);
  }
  c->kn.kbl = cfg->kbl;
  c->kn.miglim = cfg->miglim;
  c->kn.remap_optn = cfg->remap_optn;
  c->kn.hi_order = cfg->hi_order_flux_comp ? 1 : 0;
  c->kn.intfc_smooth = cfg->intfc_smooth;
  c->kn.slak = cfg->slak;
  c->kn.ptop = cfg->ptop;
  c->kn.thktop = cfg->thktop;
  c->kn.rleigh = cfg->rleigh;
  c->kn.rlthresh = cfg->rlthresh;
  c->kn.rltaper = cfg->rltaper;
  c->kn.dfflen_max = dmax;
  c->kn.biharm = biharm;

  int least = 0, greatest = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e == cudaSuccess) {
    c->prio = std::max(greatest, std::min(least, cfg->stream_priority));
    e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, c->prio);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return FIM_ECUDA;
  }
  // FP64 tables in both precisions: the FP32-mixed build runs the one-time
  // initial adjustment (hybgen, pressures, hystat) in FP64
  int rc = build_grid<double>(c, g, rarea, corio, grnd, dfflen, biharw, smoo, prox, proxs, nprox);
  if (!rc && c->prec == FIM_PREC_F32)
    rc = build_grid<float>(c, g, rarea, corio, grnd, dfflen, biharw, smoo, prox, proxs, nprox);
  if (!rc && c->kn.hi_order) rc = build_patches(c, prox, proxs, nprox);
  if (!rc) rc = dalloc(c, (void**)&c->d_sp, sizeof(StepParams) * c->M);
  if (!rc) rc = dalloc(c, (void**)&c->d_flags, sizeof(int) * c->M);
  if (!rc) {
    c->h_sp.assign(c->M, StepParams{});
    for (int m = 0; m < c->M; m++) reset_member(c, m);
    if (cudaMemset(c->d_flags, 0, sizeof(int) * c->M) != cudaSuccess) rc = FIM_ECUDA;
    if (!rc) rc = push_sp(c);
  }
  if (rc) {
    fim_ctx_destroy(c);
    return rc;
  }
  // Look up the static scratch array of fim_cnuity_noalloc now: under lazy
  // module loading that lookup loads the module that holds the array and
  // commits its memory, which is then done while the caller may still
  // allocate.  A failure is not fatal here (contexts that never call
  // fim_cnuity_noalloc do not need the array); that entry point retries the
  // lookup and reports the error.
  unsigned char* stat = nullptr;
  if (cnuity_static_addr(c, &stat) != FIM_OK) {
    cudaGetLastError();
    c->err.clear();
  }
  *out = c;
  return FIM_OK;
}

int fim_ctx_destroy(fim_ctx* c) {
  if (!c) return FIM_EINVAL;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (cudaStream_t q : {c->io_in, c->io_out, c->aux})
    if (q) {
      cudaStreamSynchronize(q);
      cudaStreamDestroy(q);
    }
  for (cudaEvent_t e : c->io_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : {c->ev_fork, c->ev_join})
    if (e) cudaEventDestroy(e);
  for (void* p : c->owned) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return FIM_OK;
}

const char* fim_ctx_last_error(const fim_ctx* c) { return c ? c->err.c_str() : "null context"; }
void* fim_ctx_stream(fim_ctx* c) { return c ? (void*)c->stream : nullptr; }
int64_t fim_launch_count(const fim_ctx* c) { return c ? c->launches : -1; }
int64_t fim_ctx_device_bytes(const fim_ctx* c) {
  if (!c) return -1;
  int64_t b = 0;
  for (size_t q : c->owned_bytes) b += (int64_t)q;
  return b;
}

int fim_get_ab(const fim_ctx* c, int* nf, int* of, int* vof, double* ab1, double* ab2, double* ab3) {
  if (!c) return FIM_EINVAL;
  const StepParams& p = c->h_sp[0];
  if (nf) *nf = p.nf + 1;
  if (of) *of = p.of + 1;
  if (vof) *vof = p.vof + 1;
  if (ab1) *ab1 = p.ab1;
  if (ab2) *ab2 = p.ab2;
  if (ab3) *ab3 = p.ab3;
  return FIM_OK;
}

int fim_set_ab(fim_ctx* c, int nf, int of, int vof, double ab1, double ab2, double ab3) {
  if (!c || nf < 1 || nf > 3 || of < 1 || of > 3 || vof < 1 || vof > 3) return FIM_EINVAL;
  for (auto& p : c->h_sp) {
    p.nf = nf - 1;
    p.of = of - 1;
    p.vof = vof - 1;
    p.ab1 = ab1;
    p.ab2 = ab2;
    p.ab3 = ab3;
  }
  return push_sp(c);
}

int fim_abstart(fim_ctx* c, int its, int its_start, int* nf, int* of, int* vof, double* adbash1, double* adbash2,
                double* adbash3) {
  (void)its_start;
  if (!c || its < 1) return FIM_EINVAL;
  for (auto& p : c->h_sp) host_abstart(p, its);
  int rc = push_sp(c);
  if (rc) return rc;
  return fim_get_ab(c, nf, of, vof, adbash1, adbash2, adbash3);
}

#define EDGVAR_ARGS_R(R)                                                                                      \
  fim_ctx *c, int its, const R *u_vel, const R *v_vel, const R *delp, const R *pres, const R *exner,       \
      const R *geop, const R *montg, const R *tracr, R *u_edg, R *v_edg, R *dp_edg, R *lp_edg, R *geop_edg, \
      R *mont_edg, R *uvsq_edg, R *trc_edg

int fim_edgvar1_r8(EDGVAR_ARGS_R(double)) {
  (void)its; (void)exner; (void)geop; (void)geop_edg;
  return edgvar_impl<double>(c, 1, u_vel, v_vel, delp, pres, montg, tracr, u_edg, v_edg, dp_edg, lp_edg, mont_edg,
                             uvsq_edg, trc_edg);
}
int fim_edgvar1_r4(EDGVAR_ARGS_R(float)) {
  (void)its; (void)exner; (void)geop; (void)geop_edg;
  return edgvar_impl<float>(c, 1, u_vel, v_vel, delp, pres, montg, tracr, u_edg, v_edg, dp_edg, lp_edg, mont_edg,
                            uvsq_edg, trc_edg);
}
int fim_edgvar3_r8(EDGVAR_ARGS_R(double)) {
  (void)its; (void)exner; (void)geop; (void)geop_edg;
  return edgvar_impl<double>(c, 3, u_vel, v_vel, delp, pres, montg, tracr, u_edg, v_edg, dp_edg, lp_edg, mont_edg,
                             uvsq_edg, trc_edg);
}
int fim_edgvar2_r8(EDGVAR_ARGS_R(double)) {
  (void)its; (void)exner; (void)geop; (void)geop_edg;
  return edgvar_impl<double>(c, 2, u_vel, v_vel, delp, pres, montg, tracr, u_edg, v_edg, dp_edg, lp_edg, mont_edg,
                             uvsq_edg, trc_edg);
}
int fim_edgvar2_r4(EDGVAR_ARGS_R(float)) {
  (void)its; (void)exner; (void)geop; (void)geop_edg;
  return edgvar_impl<float>(c, 2, u_vel, v_vel, delp, pres, montg, tracr, u_edg, v_edg, dp_edg, lp_edg, mont_edg,
                            uvsq_edg, trc_edg);
}
int fim_edgvar3_r4(EDGVAR_ARGS_R(float)) {
  (void)its; (void)exner; (void)geop; (void)geop_edg;
  return edgvar_impl<float>(c, 3, u_vel, v_vel, delp, pres, montg, tracr, u_edg, v_edg, dp_edg, lp_edg, mont_edg,
                            uvsq_edg, trc_edg);
}

int fim_cnuity_r8(fim_ctx* c, int its, const double* u_velo, const double* v_velo, const double* u_edg,
                  const double* v_edg, const double* dp_edg, const double* lp_edg, double* delp, double* pres,
                  double* exner, double* dp_tndcy, double* dplo_tndcy, double* massfx, double* omega) {
  (void)its;
  return cnuity_impl<double>(c, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy,
                             dplo_tndcy, massfx, omega);
}
int fim_cnuity_r4(fim_ctx* c, int its, const float* u_velo, const float* v_velo, const float* u_edg,
                  const float* v_edg, const float* dp_edg, const float* lp_edg, float* delp, float* pres,
                  float* exner, float* dp_tndcy, float* dplo_tndcy, float* massfx, float* omega) {
  (void)its;
  return cnuity_impl<float>(c, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy,
                            dplo_tndcy, massfx, omega);
}

int fim_mass_adv_r8(fim_ctx* c, int its, const double* u_velo, const double* v_velo, const double* u_edg,
                    const double* v_edg, double* dp_edg, const double* lp_edg, double* delp, double* pres,
                    double* exner, double* dp_tndcy, double* massfx, double* omega) {
  (void)its;
  return massadv_impl<double>(c, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy, massfx,
                              omega);
}
int fim_mass_adv_r4(fim_ctx* c, int its, const float* u_velo, const float* v_velo, const float* u_edg,
                    const float* v_edg, float* dp_edg, const float* lp_edg, float* delp, float* pres, float* exner,
                    float* dp_tndcy, float* massfx, float* omega) {
  (void)its;
  return massadv_impl<float>(c, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy, massfx,
                             omega);
}

int fim_trcadv_r8(fim_ctx* c, int its, const double* trcr_edg, double* tracr, double* trcdp, double* trc_tdcy,
                  double* trclo_tdcy, const double* massfx, const double* delp) {
  (void)its;
  return trcadv_impl<double>(c, trcr_edg, tracr, trcdp, trc_tdcy, trclo_tdcy, massfx, delp);
}
int fim_trcadv_r4(fim_ctx* c, int its, const float* trcr_edg, float* tracr, float* trcdp, float* trc_tdcy,
                  float* trclo_tdcy, const float* massfx, const float* delp) {
  (void)its;
  return trcadv_impl<float>(c, trcr_edg, tracr, trcdp, trc_tdcy, trclo_tdcy, massfx, delp);
}

int fim_momtum_r8(fim_ctx* c, int its, double* u_velo, double* v_velo, const double* exner, double* relvor,
                  const double* u_edg, const double* v_edg, const double* trcr_edg, const double* geop_edg,
                  const double* mont_edg, const double* uvsq_edg, double* u_tndcy, double* v_tndcy,
                  const double* dp3d) {
  (void)its; (void)geop_edg;
  return momtum_impl<double>(c, u_velo, v_velo, exner, relvor, u_edg, v_edg, trcr_edg, mont_edg, uvsq_edg, u_tndcy,
                             v_tndcy, dp3d);
}
int fim_momtum_r4(fim_ctx* c, int its, float* u_velo, float* v_velo, const float* exner, float* relvor,
                  const float* u_edg, const float* v_edg, const float* trcr_edg, const float* geop_edg,
                  const float* mont_edg, const float* uvsq_edg, float* u_tndcy, float* v_tndcy, const float* dp3d) {
  (void)its; (void)geop_edg;
  return momtum_impl<float>(c, u_velo, v_velo, exner, relvor, u_edg, v_edg, trcr_edg, mont_edg, uvsq_edg, u_tndcy,
                            v_tndcy, dp3d);
}

int fim_hybgen_r8(fim_ctx* c, int its, const double* targt, double* us3d, double* vs3d, double* tr3d, double* sdot,
                  double* ex3d, double* dp3d, double* pr3d) {
  return hybgen_impl<double>(c, its, targt, us3d, vs3d, tr3d, sdot, ex3d, dp3d, pr3d);
}
int fim_hybgen_r4(fim_ctx* c, int its, const float* targt, float* us3d, float* vs3d, float* tr3d, float* sdot,
                  float* ex3d, float* dp3d, float* pr3d) {
  return hybgen_impl<float>(c, its, targt, us3d, vs3d, tr3d, sdot, ex3d, dp3d, pr3d);
}

int fim_hystat_r8(fim_ctx* c, int its, double* ph3d, const double* ex3d, double* mp3d, const double* dp3d,
                  double* tr3d, double* trdp, double* psrf, double* ptdcy) {
  return hystat_impl<double>(c, its, ph3d, ex3d, mp3d, dp3d, tr3d, trdp, psrf, ptdcy);
}
int fim_hystat_r4(fim_ctx* c, int its, float* ph3d, const float* ex3d, float* mp3d, const float* dp3d, float* tr3d,
                  float* trdp, float* psrf, float* ptdcy) {
  return hystat_impl<float>(c, its, ph3d, ex3d, mp3d, dp3d, tr3d, trdp, psrf, ptdcy);
}

#define FIM_GFS10 gfs_ps, gfs_dp, gfs_p, gfs_u, gfs_v, gfs_dpdt, gfs_q, gfs_oz, gfs_cld, gfs_t
int fim_cpl_dyn_to_phy_r8(fim_ctx* c, int its, int callphy, const double* pr3d, const double* us3d,
                          const double* vs3d, const double* ws3d, const double* tr3d, double* gfs_ps,
                          double* gfs_dp, double* gfs_p, double* gfs_u, double* gfs_v, double* gfs_dpdt,
                          double* gfs_q, double* gfs_oz, double* gfs_cld, double* gfs_t) {
  double* const g[10] = {FIM_GFS10};
  return cpl_dyn_to_phy_impl<double>(c, its, callphy, pr3d, us3d, vs3d, ws3d, tr3d, g);
}
int fim_cpl_dyn_to_phy_r4(fim_ctx* c, int its, int callphy, const float* pr3d, const float* us3d,
                          const float* vs3d, const float* ws3d, const float* tr3d, double* gfs_ps,
                          double* gfs_dp, double* gfs_p, double* gfs_u, double* gfs_v, double* gfs_dpdt,
                          double* gfs_q, double* gfs_oz, double* gfs_cld, double* gfs_t) {
  double* const g[10] = {FIM_GFS10};
  return cpl_dyn_to_phy_impl<float>(c, its, callphy, pr3d, us3d, vs3d, ws3d, tr3d, g);
}
#undef FIM_GFS10
int fim_cpl_phy_to_dyn_r8(fim_ctx* c, int its, int callphy, int addtend, int smoothtend, double dtp,
                          const double* gfs_p, const double* gfs_u, const double* gfs_v, const double* gfs_q,
                          const double* gfs_cld, const double* gfs_oz, const double* gfs_t, const double* geshem,
                          const double* rainc, const double* evap, const double* dp3d, double* us3d,
                          double* vs3d, double* tr3d, double* rn2d, double* rc2d, double* qf2d) {
  const double* const g[7] = {gfs_p, gfs_u, gfs_v, gfs_q, gfs_cld, gfs_oz, gfs_t};
  const double* const col[3] = {geshem, rainc, evap};
  return cpl_phy_to_dyn_impl<double>(c, its, callphy, addtend, smoothtend, dtp, g, col, dp3d, us3d, vs3d, tr3d,
                                     rn2d, rc2d, qf2d);
}
int fim_cpl_phy_to_dyn_r4(fim_ctx* c, int its, int callphy, int addtend, int smoothtend, double dtp,
                          const double* gfs_p, const double* gfs_u, const double* gfs_v, const double* gfs_q,
                          const double* gfs_cld, const double* gfs_oz, const double* gfs_t, const double* geshem,
                          const double* rainc, const double* evap, const float* dp3d, float* us3d, float* vs3d,
                          float* tr3d, float* rn2d, float* rc2d, float* qf2d) {
  const double* const g[7] = {gfs_p, gfs_u, gfs_v, gfs_q, gfs_cld, gfs_oz, gfs_t};
  const double* const col[3] = {geshem, rainc, evap};
  return cpl_phy_to_dyn_impl<float>(c, its, callphy, addtend, smoothtend, dtp, g, col, dp3d, us3d, vs3d, tr3d,
                                    rn2d, rc2d, qf2d);
}

int fim_globsum_r8(fim_ctx* c, int its, const double* dp3d, const double* tr, const double* rn2d, const double* rc2d,
                   const double* pr3d, const double* ex3d, const double* qf2d, double* qtrcr, fim_budget* out) {
  (void)its;
  return globsum_impl<double>(c, dp3d, tr, rn2d, rc2d, pr3d, ex3d, qf2d, qtrcr, out);
}
int fim_globsum_r4(fim_ctx* c, int its, const float* dp3d, const float* tr, const float* rn2d, const float* rc2d,
                   const float* pr3d, const float* ex3d, const float* qf2d, double* qtrcr, fim_budget* out) {
  (void)its;
  return globsum_impl<float>(c, dp3d, tr, rn2d, rc2d, pr3d, ex3d, qf2d, qtrcr, out);
}

int fim_transp0_r8(fim_ctx* c, int its, double* cumufx, const double* dp3d, double* dpinit) {
  (void)its;
  return transp0_impl<double>(c, cumufx, dp3d, dpinit);
}
int fim_transp0_r4(fim_ctx* c, int its, float* cumufx, const float* dp3d, float* dpinit) {
  (void)its;
  return transp0_impl<float>(c, cumufx, dp3d, dpinit);
}
int fim_transp1_r8(fim_ctx* c, int its, double* cumufx, const double* massfx) {
  (void)its;
  return transp1_impl<double>(c, cumufx, massfx);
}
int fim_transp1_r4(fim_ctx* c, int its, float* cumufx, const float* massfx) {
  (void)its;
  return transp1_impl<float>(c, cumufx, massfx);
}
int fim_transp2_r8(fim_ctx* c, int its, double* tracr, const double* cumufx, const double* dpinit,
                   const double* dpfinl) {
  (void)its;
  return transp2_impl<double>(c, tracr, cumufx, dpinit, dpfinl);
}
int fim_transp2_r4(fim_ctx* c, int its, float* tracr, const float* cumufx, const float* dpinit,
                   const float* dpfinl) {
  (void)its;
  return transp2_impl<float>(c, tracr, cumufx, dpinit, dpfinl);
}

// ---- state ------------------------------------------------------------------
int fim_state_alloc(fim_ctx* c, fim_state** out) {
  if (!c || !out) return FIM_EINVAL;
  fim_state* st = new (std::nothrow) fim_state;
  if (!st) return FIM_ENOMEM;
  const size_t N = c->N, L = c->L, T = c->T, TB = c->TB, NL = N * L, NI = N * (L + 1);
  const size_t cnt[FIM_NFIELDS] = {
      NL, NL, NL, NI, NI, NI, NL, NL * (T + TB),   // us vs dp pr ex ph mp tr
      NL * (T + TB), NL * 3, NL * 3, NL * 3, NL * 3,  // trdp u_tdcy v_tdcy dp_tdcy dpl_tdcy
      NL * 3 * T, NL * 3 * T, NL * 6 * 3,          // trc_tdcy trl_tdcy massfx
      NL, NI, NL, N, N * 2,                        // ws sdot relvor psrf ptdcy
      NL * 6, NL * 6, NL * 6, NL * 6, NL * 6, NL * 6, NL * 6,  // edge fields
      // trc_edg: theta's edge values only with the fused tracer transport
      // (the tracer kernels form the others on chip)
      NL * 6 * (c->kn.hi_order ? 1 : T), NL * 6, NL};  // trc_edg cumufx dpinit
  for (int f = 0; f < FIM_NFIELDS; f++) {
    st->count[f] = cnt[f];
    st->slots[f] = group_field(f) ? c->G : c->M;
    // the class-B integrals exist only with class-B tracers
    const size_t n = (f == FIM_CUMUFX || f == FIM_DPINIT) && c->TB == 0 ? 0 : cnt[f] * st->slots[f];
    if (n == 0) st->count[f] = 0;
    int rc = dalloc(c, &st->f[f], n * c->esz);
    if (rc) { delete st; return rc; }
    cudaMemsetAsync(st->f[f], 0, n * c->esz + (n == 0 ? 16 : 0), c->stream);
  }
  int rc = dalloc(c, (void**)&st->sums, (size_t)c->M * (8 + c->T + c->TB) * sizeof(double));
  if (rc) { delete st; return rc; }
  st->init64.assign((size_t)FIM_NFIELDS * c->M, nullptr);
  st->host.assign((size_t)FIM_NFIELDS * c->M, nullptr);
  if (c->prec == FIM_PREC_F32) {
    if ((rc = dalloc(c, (void**)&st->mpf, (size_t)c->M * cnt[FIM_MP3D] * sizeof(float2)))) { delete st; return rc; }
    if ((rc = dalloc(c, &st->thold, (size_t)c->G * cnt[FIM_MP3D] * c->esz))) { delete st; return rc; }
    cudaMemsetAsync(st->mpf, 0, (size_t)c->M * cnt[FIM_MP3D] * sizeof(float2), c->stream);
  }
  if ((rc = ensure_all(c))) { delete st; return rc; }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) { delete st; return set_err(c, FIM_ECUDA, "state alloc"); }
  *out = st;
  return FIM_OK;
}

int fim_state_free(fim_ctx* c, fim_state* st) {
  if (!c || !st) return FIM_EINVAL;
  cudaStreamSynchronize(c->stream);
  if (st->graph) cudaGraphExecDestroy(st->graph);
  for (int f = 0; f < FIM_NFIELDS; f++) dfree(c, st->f[f]);
  for (void* extra : {(void*)st->sums, (void*)st->mpf, st->thold}) dfree(c, extra);
  for (double* p : st->init64) dfree(c, p);
  delete st;
  return FIM_OK;
}

int fim_state_field(fim_ctx* c, fim_state* st, int field, int member, void** dptr, int64_t* count) {
  if (!c || !st || field < 0 || field >= FIM_NFIELDS || member < 0 || member >= c->M) return FIM_EINVAL;
  if (member >= st->slots[field])
    return set_err(c, FIM_EINVAL, "the step's edge work fields hold only member_group members");
  if (dptr) *dptr = (char*)st->f[field] + (size_t)member * st->count[field] * c->esz;
  if (count) *count = (int64_t)st->count[field];
  return FIM_OK;
}

int fim_state_upload(fim_ctx* c, fim_state* st, int field, int member, const void* host) {
  void* d;
  int64_t n;
  int rc = fim_state_field(c, st, field, member, &d, &n);
  if (rc) return rc;
  CK(cudaMemcpyAsync(d, host, (size_t)n * c->esz, cudaMemcpyHostToDevice, c->stream), "state upload");
  return FIM_OK;
}

int fim_state_upload_f64(fim_ctx* c, fim_state* st, int field, int member, const double* host) {
  if (!c || !st || !host) return FIM_EINVAL;
  if (c->prec == FIM_PREC_F64) return fim_state_upload(c, st, field, member, host);
  if (!init_input(field))
    return set_err(c, FIM_EINVAL, "fim_state_upload_f64 takes the initial fields us3d vs3d dp3d pr3d ex3d ph3d tr3d");
  void* d;
  int64_t n;
  int rc = fim_state_field(c, st, field, member, &d, &n);
  if (rc) return rc;
  double*& s = st->init64[(size_t)field * c->M + member];
  if (!s && (rc = dalloc(c, (void**)&s, (size_t)n * sizeof(double)))) return rc;
  CK(cudaMemcpyAsync(s, host, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "state upload f64");
  k_narrow<<<conv_grid((size_t)n), 256, 0, c->stream>>>(s, (float*)d, (size_t)n);
  return check_launch(c, "state upload f64");
}

int fim_state_download(fim_ctx* c, fim_state* st, int field, int member, void* host) {
  void* d;
  int64_t n;
  int rc = fim_state_field(c, st, field, member, &d, &n);
  if (rc) return rc;
  CK(cudaMemcpyAsync(host, d, (size_t)n * c->esz, cudaMemcpyDeviceToHost, c->stream), "state download");
  return FIM_OK;
}

// one AB3 slot of a tendency field: nb blocks of nvl x nip values, the slot's
// block every third
static int ab3_slot_copy(fim_ctx* c, fim_state* st, int field, int member, int slot, void* host, bool up) {
  const bool tr = field == FIM_TRC_TDCY || field == FIM_TRL_TDCY;
  if (!tr && field != FIM_U_TDCY && field != FIM_V_TDCY && field != FIM_DP_TDCY && field != FIM_DPL_TDCY)
    return set_err(c, FIM_EINVAL, "not an AB3 tendency field");
  if (slot < 1 || slot > 3 || !host) return FIM_EINVAL;
  void* d;
  int64_t n;
  int rc = fim_state_field(c, st, field, member, &d, &n);
  if (rc) return rc;
  const size_t blk = (size_t)c->N * c->L * c->esz;
  const size_t nb = tr ? (size_t)c->T : 1;
  if ((size_t)n * c->esz != 3 * blk * nb) return set_err(c, FIM_EINVAL, "AB3 field size");
  char* dv = (char*)d + (size_t)(slot - 1) * blk;
  char* hv = (char*)host + (size_t)(slot - 1) * blk;
  if (up)
    CK(cudaMemcpy2DAsync(dv, 3 * blk, hv, 3 * blk, blk, nb, cudaMemcpyHostToDevice, c->stream), "slot upload");
  else
    CK(cudaMemcpy2DAsync(hv, 3 * blk, dv, 3 * blk, blk, nb, cudaMemcpyDeviceToHost, c->stream), "slot download");
  return FIM_OK;
}

int fim_state_upload_slot(fim_ctx* c, fim_state* st, int field, int member, int slot, const void* host) {
  if (!c || !st) return FIM_EINVAL;
  return ab3_slot_copy(c, st, field, member, slot, const_cast<void*>(host), true);
}

int fim_state_download_slot(fim_ctx* c, fim_state* st, int field, int member, int slot, void* host) {
  if (!c || !st) return FIM_EINVAL;
  return ab3_slot_copy(c, st, field, member, slot, host, false);
}

int fim_state_init(fim_ctx* c, fim_state* st) {
  if (!c || !st) return FIM_EINVAL;
  return c->prec == FIM_PREC_F64 ? state_init_impl<double>(c, st, 0, c->M)
                                 : state_init_impl<float>(c, st, 0, c->M);
}

int fim_state_init_member(fim_ctx* c, fim_state* st, int member) {
  if (!c || !st || member < 0 || member >= c->M) return FIM_EINVAL;
  return c->prec == FIM_PREC_F64 ? state_init_impl<double>(c, st, member, 1)
                                 : state_init_impl<float>(c, st, member, 1);
}

int fim_member_set_active(fim_ctx* c, fim_state* st, int member, int active) {
  (void)st;
  if (!c || member < 0 || member >= c->M) return FIM_EINVAL;
  c->h_sp[member].active = active ? 1 : 0;
  return push_sp(c);
}

int fim_state_synthetic(fim_ctx* c, fim_state* st, int member, unsigned long long seed, int ntra, double sigma_ps,
                        double noise) {
  if (!c || !st || member < 0 || member >= c->M || ntra < 1 || ntra > c->T + c->TB || !(sigma_ps >= 0.0) ||
      !(noise >= 0.0))
    return FIM_EINVAL;
  if (!c->d_synth) {
    std::vector<double> h(c->lat);
    double sum = 0.0;
    for (double d : c->dpsig) sum += d;
    for (double d : c->dpsig) h.push_back(d / sum);
    int rc = dalloc(c, (void**)&c->d_synth, h.size() * sizeof(double));
    if (rc) return rc;
    // pageable source: staged before the call returns
    CK(cudaMemcpyAsync(c->d_synth, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream),
       "synthetic state tables");
  }
  void* f[FIM_NFIELDS] = {};
  for (int k : {FIM_US3D, FIM_VS3D, FIM_DP3D, FIM_PR3D, FIM_EX3D, FIM_PH3D, FIM_MP3D, FIM_TR3D}) {
    int rc = fim_state_field(c, st, k, member, &f[k], nullptr);
    if (rc) return rc;
  }
  const double* lat = c->d_synth;
  const double* dps = c->d_synth + c->N;
  const int nslot = c->T + c->TB;
  int e;
  if (c->prec == FIM_PREC_F64)
    e = launch_synthetic<double>(c->stream, c->N, c->L, nslot, ntra, lat, dps, seed, sigma_ps, noise, c->kn.ptop,
                                 (double*)f[FIM_US3D], (double*)f[FIM_VS3D], (double*)f[FIM_DP3D],
                                 (double*)f[FIM_PR3D], (double*)f[FIM_EX3D], (double*)f[FIM_PH3D],
                                 (double*)f[FIM_MP3D], (double*)f[FIM_TR3D]);
  else
    e = launch_synthetic<float>(c->stream, c->N, c->L, nslot, ntra, lat, dps, seed, sigma_ps, noise, c->kn.ptop,
                                (float*)f[FIM_US3D], (float*)f[FIM_VS3D], (float*)f[FIM_DP3D], (float*)f[FIM_PR3D],
                                (float*)f[FIM_EX3D], (float*)f[FIM_PH3D], (float*)f[FIM_MP3D],
                                (float*)f[FIM_TR3D]);
  if (e) return set_err(c, FIM_ECUDA, "synthetic state", (cudaError_t)e);
  return FIM_OK;
}

int fim_member_set_tracers(fim_ctx* c, int member, int ntr) {
  if (!c || member < 0 || member >= c->M || ntr < 1 || ntr > c->T) return FIM_EINVAL;
  if (ntr < c->T && (c->TB > 0 || !c->kn.hi_order))
    return set_err(c, FIM_ENOTSUP, "a member's own tracer count needs the fused tracer transport "
                                   "(hi_order_flux_comp) and no class-B tracers");
  c->h_sp[member].ntr = ntr;
  return push_sp(c);
}

int fim_member_its(const fim_ctx* c, int member) {
  if (!c || member < 0 || member >= c->M) return -1;
  return c->h_sp[member].its;
}

int fim_member_get_step(const fim_ctx* c, int member, int* itsm1, int* nf, int* of, int* vof, double* ab1,
                        double* ab2, double* ab3) {
  if (!c || member < 0 || member >= c->M) return FIM_EINVAL;
  const StepParams& p = c->h_sp[member];
  if (itsm1) *itsm1 = p.its;
  if (nf) *nf = p.nf + 1;
  if (of) *of = p.of + 1;
  if (vof) *vof = p.vof + 1;
  if (ab1) *ab1 = p.ab1;
  if (ab2) *ab2 = p.ab2;
  if (ab3) *ab3 = p.ab3;
  return FIM_OK;
}

int fim_member_set_step(fim_ctx* c, int member, int itsm1, int nf, int of, int vof, double ab1, double ab2,
                        double ab3) {
  if (!c || member < 0 || member >= c->M || itsm1 < 0 || nf < 1 || nf > 3 || of < 1 || of > 3 || vof < 1 ||
      vof > 3)
    return FIM_EINVAL;
  StepParams& p = c->h_sp[member];
  p.its = itsm1;
  p.nf = nf - 1;
  p.of = of - 1;
  p.vof = vof - 1;
  p.ab1 = ab1;
  p.ab2 = ab2;
  p.ab3 = ab3;
  p.active = 1;
  return push_sp(c);
}

static int run_step(fim_ctx* c, fim_state* st, int use_graph) {
  int rc;
  if (c->autotune && !c->tuned && c->kn.hi_order && c->T > 1) {
    rc = c->prec == FIM_PREC_F64 ? autotune_impl<double>(c, st) : autotune_impl<float>(c, st);
    if (rc) return rc;
  }
  if (use_graph) {
    if (st->graph && st->graph_gen != c->graph_gen) {
      cudaGraphExecDestroy(st->graph);
      st->graph = nullptr;
    }
    if (!st->graph) {
      // the step is its-invariant: every step-dependent scalar is read from
      // the per-member device parameter block that k_step_begin advances
      cudaGraph_t graph;
      long long before = c->launches;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      rc = c->prec == FIM_PREC_F64 ? enqueue_step<double>(c, st) : enqueue_step<float>(c, st);
      cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
      if (rc) return rc;
      if (e != cudaSuccess) return set_err(c, FIM_ECUDA, "end capture", e);
      st->graph_kernels = c->launches - before;
      st->graph_gen = c->graph_gen;
      c->launches = before;
      e = cudaGraphInstantiate(&st->graph, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) { st->graph = nullptr; return set_err(c, FIM_ECUDA, "graph instantiate", e); }
    }
    CK(cudaGraphLaunch(st->graph, c->stream), "graph launch");
    c->launches += st->graph_kernels;
  } else {
    rc = c->prec == FIM_PREC_F64 ? enqueue_step<double>(c, st) : enqueue_step<float>(c, st);
    if (rc) return rc;
    if ((rc = check_launch(c, "step"))) return rc;
  }
  for (auto& p : c->h_sp)
    if (p.active) host_abstart(p, p.its + 1);
  return FIM_OK;
}

int fim_step(fim_ctx* c, fim_state* st, int its, int use_graph) {
  if (!c || !st || its < 1) return FIM_EINVAL;
  int rc = ensure_all(c);
  if (rc) return rc;
  bool dirty = false;
  for (auto& p : c->h_sp) {
    if (!p.active) { p.active = 1; dirty = true; }
    if (p.its != its - 1) { p.its = its - 1; dirty = true; }
  }
  if (dirty && (rc = push_sp(c))) return rc;
  return run_step(c, st, use_graph);
}

int fim_set_persistent(fim_ctx* c, int on, double timeout_s) {
  if (!c || !(timeout_s > 0.) || timeout_s > 60.) return FIM_EINVAL;
  if (on && !c->coop.barrier) {
    int rc = dalloc(c, (void**)&c->coop.barrier, sizeof(unsigned));
    if (rc) return rc;
  }
  c->coop_on = on != 0;
  c->coop.limit_ns = (unsigned long long)(timeout_s * 1e9);
  c->graph_gen++;
  return FIM_OK;
}

int fim_set_barrier_test(fim_ctx* c, int phantom_arrivals) {
  if (!c || phantom_arrivals < 0 || phantom_arrivals > 1) return FIM_EINVAL;
  c->coop.extra = (unsigned)phantom_arrivals;
  c->graph_gen++;
  return FIM_OK;
}

int fim_state_set_host(fim_ctx* c, fim_state* st, int field, int member, void* host) {
  if (!c || !st || field < 0 || field >= FIM_NFIELDS || member < 0 || member >= c->M) return FIM_EINVAL;
  IoClass k;
  if (!io_class(field, &k))
    return set_err(c, FIM_EINVAL, "the edge work fields stay on the device (fim_state_set_host)");
  st->host[(size_t)field * c->M + member] = host;
  return FIM_OK;
}

int fim_step_io(fim_ctx* c, fim_state* st, int its, int64_t* h2d_bytes, int64_t* d2h_bytes) {
  if (!c || !st || its < 1) return FIM_EINVAL;
  if (c->G != c->M) return set_err(c, FIM_ENOTSUP, "fim_step_io runs all members in one group");
  int rc = ensure_all(c);
  if (rc) return rc;
  if (c->autotune && !c->tuned && c->kn.hi_order && c->T > 1) {
    rc = c->prec == FIM_PREC_F64 ? autotune_impl<double>(c, st) : autotune_impl<float>(c, st);
    if (rc) return rc;
  }
  for (cudaStream_t* q : {&c->io_in, &c->io_out})
    if (!*q) CK(cudaStreamCreateWithPriority(q, cudaStreamNonBlocking, c->prio), "step io stream");
  for (auto& p : c->h_sp) {
    p.active = 1;
    p.its = its - 1;
  }
  if ((rc = push_sp(c))) return rc;
  StepIo io;
  io.c = c;
  io.st = st;
  io.its = its;
  for (int m = 0; m < c->M; m++) {  // the slots after the step's abstart
    const StepParams& p = c->h_sp[m];
    io.nf.push_back((p.nf + 1) % 3);
    io.of.push_back((p.of + 1) % 3);
    io.vof.push_back((p.vof + 1) % 3);
  }
  // tracer chunks of about a seventh of the tracers: the slots of a chunk go
  // up while the chunk before it is transported, its results come down while
  // the next one is; what is left after the last upload is that chunk's
  // transport and its downloads (at glvl 8, 3 tracers: ~2 GB, ~10 ms)
  io.tchunk = c->kn.hi_order ? std::max(1, std::min(c->ftchunk, (c->T + 6) / 7)) : c->T;
  io.hook.fn = io_chunk_hook;
  io.hook.arg = &io;
  // the copies start behind the work already queued on the compute stream
  cudaEvent_t start = io_event(io);
  if (!start) return set_err(c, FIM_ECUDA, "step io event");
  CK(cudaEventRecord(start, c->stream), "step io record");
  if (c->prof.on) c->prof.mark("start", c->stream);
  CK(cudaStreamWaitEvent(c->io_in, start, 0), "step io wait");
  CK(cudaStreamWaitEvent(c->io_out, start, 0), "step io wait");
  if ((rc = io_upload(io, kIoA, 0, 0, &io.up_ev[kIoA]))) return rc;
  if ((rc = io_upload(io, kIoC, 0, 0, &io.up_ev[kIoC]))) return rc;
  if ((rc = io_upload(io, kIoU, 0, 0, &io.up_ev[kIoU]))) return rc;
  for (int t0 = 0; t0 < c->T; t0 += io.tchunk) {
    cudaEvent_t e;
    if ((rc = io_upload(io, kIoT, t0, std::min(io.tchunk, c->T - t0), &e))) return rc;
    io.up_chunk.push_back(e);
  }
  rc = c->prec == FIM_PREC_F64 ? enqueue_step<double>(c, st, &io) : enqueue_step<float>(c, st, &io);
  if (rc) return rc;
  if ((rc = check_launch(c, "step io"))) return rc;
  // the step ends when its last download has landed
  cudaEvent_t done = io_event(io);
  if (!done) return set_err(c, FIM_ECUDA, "step io event");
  CK(cudaEventRecord(done, c->io_out), "step io record");
  CK(cudaStreamWaitEvent(c->stream, done, 0), "step io wait");
  for (auto& p : c->h_sp)
    if (p.active) host_abstart(p, p.its + 1);
  if (c->prof.on) c->prof.mark("end", c->stream);
  CK(cudaStreamSynchronize(c->stream), "step io");
  if (c->prof.on) c->prof.collect_marks();
  if (h2d_bytes) *h2d_bytes = io.h2d;
  if (d2h_bytes) *d2h_bytes = io.d2h;
  return FIM_OK;
}

int fim_step_active(fim_ctx* c, fim_state* st, int use_graph) {
  if (!c || !st) return FIM_EINVAL;
  int rc = ensure_all(c);
  if (rc) return rc;
  return run_step(c, st, use_graph);
}

int fim_state_budget(fim_ctx* c, fim_state* st, int member, double* qtrcr, fim_budget* out) {
  if (!c || !st || member < 0 || member >= c->M) return FIM_EINVAL;
  const int ntr = c->T + c->TB;
  std::vector<double> h(8 + ntr);
  CK(cudaMemcpyAsync(h.data(), st->sums + (size_t)member * (8 + ntr), h.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, c->stream), "budget");
  CK(cudaStreamSynchronize(c->stream), "budget sync");
  if (qtrcr) for (int q = 0; q < ntr; q++) qtrcr[q] = h[8 + q];
  if (out) {
    out->qmass = h[0]; out->qmsqv = h[1]; out->qmsqw = h[2]; out->qmso3 = h[3];
    out->qmste = h[4]; out->qmstr = h[5]; out->qmstrn = h[6]; out->qmstrc = h[7];
  }
  return FIM_OK;
}

int fim_profile_enable(fim_ctx* c, int on) {
  if (!c) return FIM_EINVAL;
  if (!on) c->prof.collect();
  c->prof.on = on != 0;
  return FIM_OK;
}

int fim_profile_report(fim_ctx* c, char* buf, int len) {
  if (!c || !buf || len <= 0) return FIM_EINVAL;
  c->prof.collect();
  std::string out;
  char line[256];
  for (auto& kv : c->prof.agg) {
    snprintf(line, sizeof line, "%s %lld %.6f\n", kv.first.c_str(), kv.second.first, kv.second.second);
    out += line;
  }
  if ((int)out.size() + 1 > len) return FIM_EINVAL;
  memcpy(buf, out.c_str(), out.size() + 1);
  c->prof.agg.clear();
  return FIM_OK;
}

int fim_grid_patches(const fim_grid_desc* g, int side, int* npatch, int* max_cells, int* max_frame,
                     int* max_ring_edges) {
  if (!g || side < 1 || side > 8) return FIM_EINVAL;
  std::vector<int> prox, proxs, nprox;
  if (index_tables(g, prox, proxs, nprox) != FIM_OK) return FIM_EINVAL;
  FrameHost h;
  if (build_frames(g->nip, prox.data(), proxs.data(), nprox.data(), side, &h) != 0) return FIM_EINVAL;
  if (check_frames(g->nip, prox.data(), proxs.data(), nprox.data(), h) != 0) return FIM_EINVAL;
  int mc = 0, mf = 0, mr = 0;
  for (int t = 0; t < h.ntile; t++) {
    mc = std::max(mc, h.cnt[(size_t)t * 4]);
    mf = std::max(mf, h.cnt[(size_t)t * 4 + 2]);
    mr = std::max(mr, h.cnt[(size_t)t * 4 + 3]);
  }
  if (npatch) *npatch = h.ntile;
  if (max_cells) *max_cells = mc;
  if (max_frame) *max_frame = mf;
  if (max_ring_edges) *max_ring_edges = mr;
  return FIM_OK;
}

int fim_tracer_shape(const fim_ctx* c, int* levels_per_thread, int* threads_per_block, float* probe_ms) {
  if (!c) return FIM_EINVAL;
  if (levels_per_thread) *levels_per_thread = c->trc_vk;
  if (threads_per_block) *threads_per_block = c->ftab.SC * c->trc_gc;
  if (probe_ms) *probe_ms = c->tuned ? c->tune_ms : 0.f;
  return FIM_OK;
}

int fim_check(fim_ctx* c, fim_state* st, int* flags) {
  (void)st;
  if (!c) return FIM_EINVAL;
  std::vector<int> h(c->M);
  CK(cudaMemcpyAsync(h.data(), c->d_flags, sizeof(int) * c->M, cudaMemcpyDeviceToHost, c->stream), "flags");
  CK(cudaMemsetAsync(c->d_flags, 0, sizeof(int) * c->M, c->stream), "flags reset");
  CK(cudaStreamSynchronize(c->stream), "flags sync");
  int f = 0;
  for (int v : h) f |= v;
  if (flags) *flags = f;
  if (f & kFlagTimeout) return FIM_ETIMEDOUT;
  return (f & kFlagBadDp) ? FIM_ENUMERIC : FIM_OK;
}

}  // extern "C"

// ---- cnuity without allocation ---------------------------------------------
// fim_cnuity_r8/_r4 allocate their FCT scratch (the antidiffusive fluxes, the
// low-order thickness and the four limiter fields: 11 values per cell-level)
// on the context's first call.  fim_cnuity_noalloc takes that scratch from one
// array that is part of the loaded library image instead, for callers that may
// not allocate device memory while they run: a host model whose device memory
// is carved up once by its own pool at start-up, a memory-capped process, or a
// time loop that cannot afford the device-wide synchronisation of cudaMalloc.
// Each GPU that loads this library holds the array (kCnuityStaticBytes) until
// the process exits.  Every call on a device shares it and it keeps the
// previous call's contents; the cnuity kernels write every scratch value they
// read before reading it, so nothing is cleared.  Calls whose kernels overlap
// on the GPU (two streams, two contexts, two host threads) race on it.
namespace {

constexpr size_t kCnuityStaticBytes = size_t(64) << 20;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_cnuity_static[kCnuityStaticBytes];

std::mutex g_static_mu;
void* g_static_addr[kStaticMaxDevices] = {};

}  // namespace

// Device address of g_cnuity_static on the current device, looked up once per
// device (the host-side name is only a handle for the runtime, not an address).
int cnuity_static_addr(fim_ctx* c, unsigned char** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_err(c, FIM_ECUDA, "cudaGetDevice", e);
  if (dev < 0 || dev >= kStaticMaxDevices) return set_err(c, FIM_EINVAL, "device ordinal beyond 63");
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_cnuity_static);
    if (e != cudaSuccess) return set_err(c, FIM_ECUDA, "cudaGetSymbolAddress(static cnuity scratch)", e);
    g_static_addr[dev] = p;
  }
  *out = (unsigned char*)g_static_addr[dev];
  return FIM_OK;
}

namespace {

size_t round256(size_t b) { return (b + 255) / 256 * 256; }

template <typename R>
int cnuity_noalloc_impl(fim_ctx* c, const void* u_velo, const void* v_velo, const void* u_edg, const void* v_edg,
                        const void* dp_edg, const void* lp_edg, void* delp, void* pres, void* exner, void* dp_tndcy,
                        void* dplo_tndcy, void* massfx, void* omega) {
  if (c->cfg.host_pointers)
    return set_err(c, FIM_EINVAL, "fim_cnuity_noalloc takes device pointers only (host_pointers context)");
  // like fim_cnuity_r8/_r4 the call advances member 0 only
  const size_t cells = (size_t)c->N * c->L;
  const size_t one = round256(cells * sizeof(R)), six = round256(cells * 6 * sizeof(R));
  const size_t need = six + 5 * one;
  if (need > kCnuityStaticBytes) {
    char msg[200];
    snprintf(msg, sizeof msg,
             "fim_cnuity_noalloc: this grid needs %zu bytes of scratch, the static array holds %zu "
             "(11 x nip x nvl values)", need, kCnuityStaticBytes);
    return set_err(c, FIM_EINVAL, msg);
  }
  const void* ptrs[] = {u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy, dplo_tndcy,
                        massfx, omega};
  for (const void* p : ptrs)
    if (!p) return set_err(c, FIM_EINVAL, "fim_cnuity_noalloc: null field pointer");
  unsigned char* base = nullptr;
  int rc = cnuity_static_addr(c, &base);
  if (rc) return rc;
  if ((rc = push_sp(c))) return rc;
  CnuityScratch<R> w{(R*)base, (R*)(base + six), (R*)(base + six + one), (R*)(base + six + 2 * one),
                     (R*)(base + six + 3 * one), (R*)(base + six + 4 * one)};
  launch_cnuity<R>(make_launch(c, 1), grid_of<R>(c), c->str, w, (const R*)u_velo, (const R*)v_velo,
                   (const R*)u_edg, (const R*)v_edg, (const R*)dp_edg, (const R*)lp_edg, (R*)delp, (R*)pres,
                   (R*)exner, (R*)dp_tndcy, (R*)dplo_tndcy, (R*)massfx, (R*)omega);
  return check_launch(c, "cnuity (static scratch)");
}

}  // namespace

extern "C" int fim_cnuity_noalloc(fim_ctx* c, int its, const void* u_velo, const void* v_velo, const void* u_edg,
                                  const void* v_edg, const void* dp_edg, const void* lp_edg, void* delp, void* pres,
                                  void* exner, void* dp_tndcy, void* dplo_tndcy, void* massfx, void* omega) {
  (void)its;
  if (!c) return FIM_EINVAL;
  if (c->prec == FIM_PREC_F64)
    return cnuity_noalloc_impl<double>(c, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner,
                                       dp_tndcy, dplo_tndcy, massfx, omega);
  return cnuity_noalloc_impl<float>(c, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy,
                                    dplo_tndcy, massfx, omega);
}
