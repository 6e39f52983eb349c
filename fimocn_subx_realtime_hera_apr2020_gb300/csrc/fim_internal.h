// Internal declarations shared by the kernels and the C-ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <map>
#include <string>
#include <vector>

namespace fim {

// Physical constants of FIMsrc/cntl/module_constants.F90:14-27.
constexpr double kPi = 3.14159265;
constexpr double kEarthRad = 6371220.;
constexpr double kOmegx2 = 1.4584e-4;
constexpr double kGrvity = 9.80665;
constexpr double kP1000 = 100000.;
constexpr double kCp = 1004.6855;
constexpr double kRd = 287.0586;
constexpr double kQvmin = 1.e-10;
constexpr double kQwmin = 1.e-10;

// Largest layer count the column kernels accept.
constexpr int kMaxL = 128;

// Step-dependent scalars that the reference keeps in module_variables
// (nf, of, vof, adbash1..3) plus the step number used by hybgen and hystat.
// They live in device memory so a captured step graph can be replayed.
// One block per ensemble member (indexed by the member, blockIdx.y in the
// kernels), so members of one batch can be at different steps.
struct StepParams {
  int its;
  int nf, of, vof;      // 0-based AB3 slots
  double ab1, ab2, ab3; // AB3 weights (s)
  double dt;
  int active;           // 0: the member's slot is idle, kernels skip it
  // tracers the member transports (fim_member_set_tracers): the tracer
  // transport, the remap and the budget sums leave slots ntr.. as they are
  int ntr = 0x7fffffff;
};

// device status bits
enum : int {
  kFlagBadDp = 1,       // non-positive or NaN layer thickness after cnuity
  kFlagColumnIntegral = 2,  // hybgen column-integral conservation check failed
  kFlagNaN = 4,
  kFlagTimeout = 8,     // a grid barrier of a persistent launch gave up waiting
};

// Relative tolerance of hybgen's column-integral checks: the reference's own
// in FP64 (acurcy of restp_1d 1e-6, hybgen.F90:873; of remap_1d 2e-6, :694;
// of the real*8 pcwise 1e-11, :1262); in the FP32-mixed build one bound for
// the checks it runs, ~500 float epsilons, well above the rounding of a
// column sum of nvl <= 128 FP32 terms and well below a lost or doubled layer.
template <typename R>
__host__ __device__ constexpr R col_tol(double ref) {
  return R(sizeof(R) == 8 ? ref : 3.e-5);
}

// Grid tables on the device, metric tables in the compute type R.
template <typename R>
struct Grid {
  int N, L, T;
  const int* __restrict__ prox;   // [N*6] 0-based
  const int* __restrict__ proxs;  // [N*6] 0-based (pentagon slot 5 = -1)
  const int* __restrict__ nprox;  // [N]
  const R* __restrict__ cs;       // [N*6*4]
  const R* __restrict__ sn;
  const R* __restrict__ svc;      // sidevec_c [N*6*2]
  const R* __restrict__ sve;      // sidevec_e [N*6*2]
  const R* __restrict__ sideln;   // [N*6]
  const R* __restrict__ area;     // [N]
  const R* __restrict__ rarea;
  const R* __restrict__ corio;
  const R* __restrict__ grndspd;
  const R* __restrict__ hfcoef;   // [N*6*6]: hfcoef[(i*6+edge)*6+j]
  const R* __restrict__ cxy;      // [N*2*6]: corner_xy(6,2,nip), cxy[(i*2+xy)*6+corner]; null if not given
  const double* __restrict__ area_d;  // [N] double areas for budgets
  const R* __restrict__ svsum;        // [N*2] sum over edges of sidevec_c(1:2), summed in FP64
  // per-level tables
  const R* __restrict__ dfflen;   // [L]
  const R* __restrict__ biharw;   // [L]
  const R* __restrict__ smoo;     // [L+1]
  const R* __restrict__ thetac;   // [L]
  const R* __restrict__ dpsig;    // [L]
};

struct Knobs {
  int kbl, miglim, remap_optn, hi_order;
  double intfc_smooth, slak, ptop, thktop, rleigh, rlthresh, rltaper;
  double dfflen_max;
  int biharm;  // any biharw > 0
};

// Per-member element strides of the state arrays.
struct Strides {
  size_t cell;   // L*N
  size_t intf;   // (L+1)*N
  size_t edge;   // 6*L*N
  size_t ab;     // 3*L*N
  size_t tr;     // (T+TB)*L*N: tr3d and trdp
  size_t trab;   // 3*T*L*N
  size_t tredg;  // 6*T*L*N
  size_t mf;     // 3*6*L*N
  size_t col;    // N
};

// T class-A tracers (edges, tendencies); tr3d/trdp also hold TB class-B ones
inline Strides make_strides(int N, int L, int T, int TB = 0) {
  Strides s;
  s.cell = (size_t)L * N;
  s.intf = (size_t)(L + 1) * N;
  s.edge = (size_t)6 * L * N;
  s.ab = (size_t)3 * L * N;
  s.tr = (size_t)(T + TB) * L * N;
  s.trab = (size_t)3 * T * L * N;
  s.tredg = (size_t)6 * T * L * N;
  s.mf = (size_t)18 * L * N;
  s.col = (size_t)N;
  return s;
}

// Per-kernel timing with CUDA events on the launching stream (bench only).
struct Prof {
  bool on = false;
  struct Rec { const char* name; cudaEvent_t a, b; };
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> pool;
  std::map<std::string, std::pair<long long, double>> agg;  // name -> (launches, ms)
  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  void begin(const char* name, cudaStream_t s) {
    Rec r{name, get(), get()};
    cudaEventRecord(r.a, s);
    pending.push_back(r);
  }
  void end(cudaStream_t s) { cudaEventRecord(pending.back().b, s); }
  void collect() {
    for (auto& r : pending) {
      cudaEventSynchronize(r.b);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.a, r.b);
      auto& a = agg[r.name];
      a.first += 1;
      a.second += ms;
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    pending.clear();
  }
  // fim_step_io's timeline: host time stamps taken by callbacks queued on
  // the compute and copy streams, kept as offsets from the step's first
  // mark; each name accumulates (steps, ms) in agg as "io:<name>"
  struct Mark { std::string name; double ms = 0.0; };
  std::vector<Mark*> marks;
  static void CUDART_CB stamp(void* p) {
    static_cast<Mark*>(p)->ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
  }
  void mark(const std::string& name, cudaStream_t s) {
    Mark* m = new Mark{name};
    if (cudaLaunchHostFunc(s, stamp, m) != cudaSuccess) {
      cudaGetLastError();
      delete m;
      return;
    }
    marks.push_back(m);
  }
  // once the streams holding the marks are idle
  void collect_marks() {
    for (Mark* m : marks) {
      auto& a = agg["io:" + m->name];
      a.first += 1;
      a.second += m->ms - marks[0]->ms;
    }
    for (Mark* m : marks) delete m;
    marks.clear();
  }
  ~Prof() {
    for (auto& r : pending) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : pool) cudaEventDestroy(e);
    for (Mark* m : marks) delete m;
  }
};

// Launch context handed to every launcher.
struct CoopCfg;
struct Launch {
  cudaStream_t stream;
  int members;         // gridDim.y
  const StepParams* sp;  // device
  int* flags;          // device status word per member [members]
  long long* counter;  // host launch counter
  Prof* prof = nullptr;  // per-kernel event timing when enabled
  // 1 for the column adjustment that opens a step (dyn_run's hybgen/hystat
  // of step its-1): the column kernels then act for its-1 and skip a member
  // at its first step, where dyn_init's adjustment stands in
  int boundary = 0;
  // non-null: cnuity1..4 run as one cooperative persistent launch
  const CoopCfg* coop = nullptr;
};

// The persistent cnuity1..4 launch: its grid barrier's counter (device),
// arrivals added to each barrier's target (0; a test sets 1 so that the first
// barrier never completes) and the barrier's time limit.
struct CoopCfg {
  unsigned* barrier;
  unsigned extra;
  unsigned long long limit_ns;
};

#define FIM_KBEGIN(l, name) do { if ((l).prof && (l).prof->on) (l).prof->begin(name, (l).stream); } while (0)
#define FIM_KEND(l)                                                      \
  do {                                                                   \
    if ((l).prof && (l).prof->on) (l).prof->end((l).stream);             \
    if ((l).counter) ++*(l).counter;                                     \
  } while (0)


// ---- level vectors: VK consecutive levels per thread ----------------------
// Cell and edge fields are level-fastest, so VK consecutive levels of one
// column are one 4/8/16-byte access.  pick_vk chooses the widest VK (at most
// 16 bytes) that nvl and the alignment of every pointer admit.
template <typename R, int VK> struct VecOf;
template <typename R> struct VecOf<R, 1> { using T = R; };
template <> struct VecOf<float, 2> { using T = float2; };
template <> struct VecOf<float, 4> { using T = float4; };
template <> struct VecOf<double, 2> { using T = double2; };

template <int VK, typename R>
__device__ __forceinline__ void ldv(const R* p, R (&r)[VK]) {
  if constexpr (VK == 1) {
    r[0] = *p;
  } else if constexpr (VK == 2) {
    const typename VecOf<R, 2>::T t = *reinterpret_cast<const typename VecOf<R, 2>::T*>(p);
    r[0] = t.x; r[1] = t.y;
  } else {
    const float4 t = *reinterpret_cast<const float4*>(p);
    r[0] = t.x; r[1] = t.y; r[2] = t.z; r[3] = t.w;
  }
}

template <int VK, typename R>
__device__ __forceinline__ void stv(R* p, const R (&r)[VK]) {
  if constexpr (VK == 1) {
    *p = r[0];
  } else if constexpr (VK == 2) {
    typename VecOf<R, 2>::T t; t.x = r[0]; t.y = r[1];
    *reinterpret_cast<typename VecOf<R, 2>::T*>(p) = t;
  } else {
    float4 t; t.x = r[0]; t.y = r[1]; t.z = r[2]; t.w = r[3];
    *reinterpret_cast<float4*>(p) = t;
  }
}

#define FOR_V _Pragma("unroll") for (int j = 0; j < VK; j++)

// a / b for the clamped quotients of the FCT limiters: IEEE division in FP64;
// __fdividef in the FP32-mixed build (within 2 ulp while |b| < 2^126; the
// denominators are clamped to >= 1e-11 and are far below that bound).  The
// fused and the per-routine tracer kernels use it alike, so they stay
// bit-identical.
template <typename R>
__device__ __forceinline__ R fdiv(R a, R b) { return a / b; }
template <>
__device__ __forceinline__ float fdiv<float>(float a, float b) { return __fdividef(a, b); }

// (cell, first level) of thread threadIdx.x of (virtual) block bx over
// nip x (nvl/VK)
template <int VK>
__device__ __forceinline__ bool cell_levels_at(int N, int L, int bx, int& i, int& k) {
  const int LV = L / VK;
  const int gid = bx * blockDim.x + threadIdx.x;
  if (gid >= N * LV) return false;
  i = gid / LV;
  k = (gid - i * LV) * VK;
  return true;
}

// (cell, first level) of thread gid over nip x (nvl/VK)
template <int VK>
__device__ __forceinline__ bool cell_levels(int N, int L, int& i, int& k) {
  const int LV = L / VK;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= N * LV) return false;
  i = gid / LV;
  k = (gid - i * LV) * VK;
  return true;
}

template <typename R>
inline int pick_vk(int L, std::initializer_list<const void*> ptrs, int want = 0) {
  int vk = want > 0 ? want : (int)(16 / sizeof(R));
  if ((int)sizeof(R) * vk > 16) vk = (int)(16 / sizeof(R));
  while (vk > 1 && L % vk != 0) vk /= 2;
  for (const void* p : ptrs)
    while (vk > 1 && p && ((uintptr_t)p % (vk * sizeof(R))) != 0) vk /= 2;
  return vk;
}

// run CALL with the compile-time constant VK equal to vk (4 only for float)
#define FIM_VK_DISPATCH(R, vk, CALL)                          \
  do {                                                        \
    if ((vk) >= 4 && sizeof(R) == 4) {                        \
      constexpr int VK = sizeof(R) == 4 ? 4 : 2;              \
      CALL;                                                   \
    } else if ((vk) >= 2) {                                   \
      constexpr int VK = 2;                                   \
      CALL;                                                   \
    } else {                                                  \
      constexpr int VK = 1;                                   \
      CALL;                                                   \
    }                                                         \
  } while (0)

// ---- float-float arithmetic (FP32-mixed build) ----------------------------
// A value hi + lo with |lo| <= ulp(hi)/2 carries ~48 significant bits on the
// FP32 pipes, which GB300 runs at 64x its FP64 rate.  two_sum and two_prod are
// exact (Knuth; Dekker with a fused multiply-add); ff_add is the usual
// double-float sum with one renormalisation.
struct FF2 {
  float hi, lo;
};
__device__ __forceinline__ FF2 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ FF2 two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF2 ff_add(FF2 a, FF2 b) {
  const FF2 s = two_sum(a.hi, b.hi);
  const float e = s.lo + (a.lo + b.lo);
  const float hi = s.hi + e;
  return {hi, e - (hi - s.hi)};
}
__device__ __forceinline__ FF2 ff_neg(FF2 a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ FF2 ff_shfl_up(FF2 a, int off) {
  return {__shfl_up_sync(0xffffffffu, a.hi, off), __shfl_up_sync(0xffffffffu, a.lo, off)};
}
__device__ __forceinline__ FF2 ff_shfl(FF2 a, int src) {
  return {__shfl_sync(0xffffffffu, a.hi, src), __shfl_sync(0xffffffffu, a.lo, src)};
}
__device__ __forceinline__ FF2 ff_shfl_xor(FF2 a, int m) {
  return {__shfl_xor_sync(0xffffffffu, a.hi, m), __shfl_xor_sync(0xffffffffu, a.lo, m)};
}
// (x.hi + x.lo) - (y.hi + y.lo) rounded once to float
__device__ __forceinline__ float ff_diff(float2 x, float2 y) {
  const FF2 d = two_sum(x.x, -y.x);
  return d.hi + (d.lo + (x.y - y.y));
}

// ---- launchers (instantiated for float and double) ----------------------
// mpf (FP32-mixed step only, may be null): float-float copy (hi, lo) of the
// Montgomery potential; mont_edg then holds the edge value minus the cell value.
template <typename R>
void launch_edgvar1(const Launch&, const Grid<R>&, const Strides&, int hi_order, const R* u,
                    const R* v, const R* delp, const R* pres, const R* montg, const R* tracr,
                    R* u_edg, R* v_edg, R* dp_edg, R* lp_edg, R* mont_edg, R* uvsq_edg, R* trc_edg,
                    const float2* mpf = nullptr, R* thold = nullptr);
// nfields: 1 = dp only, T = dp and tracers 2..ntra (edgvar3's full output);
// average = false leaves the own-side values (k_cnuity12 averages the layer
// thickness's itself)
template <typename R>
void launch_edgvar3(const Launch&, const Grid<R>&, const Strides&, const R* delp, const R* tracr,
                    R* dp_edg, R* trc_edg, int nfields, bool average = true);
template <typename R>
struct CnuityScratch { R *antifx, *delp_lo, *p_plus, *p_mnus, *r_plus, *r_mnus; };
template <typename R>
void launch_cnuity(const Launch&, const Grid<R>&, const Strides&, const CnuityScratch<R>&, const R* u,
                   const R* v, const R* u_edg, const R* v_edg, const R* dp_edg, const R* lp_edg,
                   R* delp, R* pres, R* exner, R* dp_tndcy, R* dplo_tndcy, R* massfx, R* omega);
// flux_conserv_schm = 2 (the bounds use the r_plus/r_mnus scratch slots)
template <typename R>
void launch_massadv(const Launch&, const Grid<R>&, const Strides&, const CnuityScratch<R>&, const R* u,
                    const R* v, const R* u_edg, const R* v_edg, R* dp_edg, const R* lp_edg, R* delp, R* pres,
                    R* exner, R* dp_tndcy, R* massfx, R* omega);
template <typename R>
struct TrcadvScratch { R *antiflx, *trmin, *trmax, *trcr_lo, *r_plus, *r_mnus; int tchunk; };
template <typename R>
void launch_trcadv(const Launch&, const Grid<R>&, const Strides&, const TrcadvScratch<R>&,
                   const R* trc_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx,
                   const R* delp);
// Cell patches of the fused tracer kernels (fim_trc.cu).  A patch is a set
// of interior cells; its frame lists them first, then every other cell one
// neighbour step away (ring 1), then two steps away (ring 2), so a block can
// stage the frame in shared memory and find every neighbour it needs there.
struct FrameTab {
  int ntile = 0;
  // capacities: frame cells, interior + ring-1 cells, interior cells,
  // edge-value rows (6 per interior cell + ring edges), ring edges
  int S2 = 0, S1 = 0, SC = 0, SE = 0, SR = 0;
  const int* cells = nullptr;            // [ntile][S2] cell index, frame order
  const uint2* nbr = nullptr;            // [ntile][S1] frame-local index of prox slots 0..5, a byte each
  const int4* cnt = nullptr;             // [ntile] interior cells, + ring 1, + ring 2, ring edges
  const unsigned short* mir = nullptr;   // [ntile][SC][6] edge-value row of the other side of each edge
  const unsigned short* redge = nullptr; // [ntile][SR] ring edges: (frame-local cell << 3) | slot
};
struct FrameHost {
  int ntile = 0, S2 = 0, S1 = 0, SC = 0, SE = 0, SR = 0;
  std::vector<int> cells, cnt;
  std::vector<uint32_t> nbr;
  std::vector<uint16_t> mir, red;
};
// patches of side x side cells of each rhombus (the reference's IJ
// numbering), else grown breadth-first; 0 on success
int build_frames(int N, const int* prox, const int* proxs, const int* nprox, int side, FrameHost* out);
// 0 if every cell is in exactly one patch and every frame neighbour and edge
// mirror of the tables resolves to prox/proxs
int check_frames(int N, const int* prox, const int* proxs, const int* nprox, const FrameHost& f);
// fused tracer path of the step (fim_trc.cu)
template <typename R>
struct TrcFusedScratch {
  R *trcr_lo, *s_plus, *s_mnus, *trold;
  R *r_plus, *r_mnus;  // scratch for the shape probe's outputs
  R* antifx;           // antidiffusive fluxes (6 per cell-level) of the chunk
  int tchunk;
  int vk;  // levels per thread (0: widest the layout admits)
  int gc;  // threads per cell and level tile: the tile is vk * gc levels
  FrameTab ft;
};
// one-time launch attributes (shared-memory size) of the tracer kernels for
// these patches; returns a cudaError_t value
template <typename R>
int prepare_tracers(const FrameTab& ft);
// times the tracer kernel shapes on the given state (see fim_trc.cu); returns a cudaError_t value
template <typename R>
int tune_tracers(const Launch&, const Grid<R>&, const Strides&, const TrcFusedScratch<R>&, R* trc_edg, R* tracr,
                 R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx, const R* delp, int* best_vk, int* best_gc,
                 float* best_ms);
// Called by launch_tracers_fused before (phase 0) and after (phase 1) the
// kernels of each tracer chunk [t0, t0 + nt): the step with host transfers
// (fim_step_io) orders the chunk's AB3 slot uploads and its downloads there.
struct ChunkHook {
  void (*fn)(void* arg, int phase, int t0, int nt) = nullptr;
  void* arg = nullptr;
};
template <typename R>
void launch_tracers_fused(const Launch&, const Grid<R>&, const Strides&, const TrcFusedScratch<R>&,
                          R* trc_edg, R* tracr, R* trcdp, R* trc_tdcy, R* trl_tdcy, const R* massfx,
                          const R* delp, const ChunkHook* hook = nullptr);
template <typename R>
struct MomtumScratch { R *du, *dv, *wu, *wv; };
// With mpf != null (FP32-mixed step) the pressure-gradient line integrals use
// the cell values split off (see k_momtum1): tr0 = the potential temperature
// edgvar1 saw (thold), svsum = per-cell sums of sidevec_c.
template <typename R>
void launch_momtum(const Launch&, const Grid<R>&, const Strides&, const Knobs&, const MomtumScratch<R>&,
                   R* u, R* v, const R* exner, R* relvor, const R* u_edg, const R* v_edg,
                   const R* trc_edg, const R* mont_edg, const R* uvsq_edg, R* u_tndcy, R* v_tndcy,
                   const R* dp3d, const float2* mpf = nullptr, const R* tr0 = nullptr);
template <typename R>
struct HybgenScratch { R *exsmo, *exsmo2; };
// one-time launch attributes of the hybgen kernels (shared-memory size);
// returns a cudaError_t value
template <typename R>
int prepare_hybgen(int L);
// trdp != null: the default-knob remap also applies hystat's humidity floors
// and writes tracer x thickness of the new state (returns true; hystat can
// then skip that stream)
template <typename R>
bool launch_hybgen(const Launch&, const Grid<R>&, const Strides&, const Knobs&, const HybgenScratch<R>&,
                   const R* targt, R* us3d, R* vs3d, R* tr3d, R* sdot, R* ex3d, R* dp3d, R* pr3d,
                   R* trdp = nullptr);
template <typename R>
void launch_hystat(const Launch&, const Grid<R>&, const Strides&, R* ph3d, const R* ex3d, R* mp3d,
                   const R* dp3d, R* tr3d, R* trdp, R* psrf, R* ptdcy, float2* mpf = nullptr,
                   bool trdp_done = false);
// class-B transport (fim_trb.cu); scratch per member: w (nvl x nip), the
// other fields (nvl x nip x ntrb)
template <typename R>
struct ClassBScratch { R *w, *F, *V, *fmx, *fmn, *flo, *flp, *fln; };
template <typename R>
void launch_transp1(const Launch&, const Grid<R>&, const Strides&, R* cumufx, const R* massfx);
// every > 0: only members at a step its with its % every == 0
template <typename R>
void launch_transp0(const Launch&, const Grid<R>&, const Strides&, int every, R* cumufx, const R* dp3d,
                    R* dpinit);
template <typename R>
void launch_transp2(const Launch&, const Grid<R>&, const Strides&, const ClassBScratch<R>&, int every, int ntrb,
                    R* tracr, const R* cumufx, const R* dpinit, const R* dpfinl);
template <typename R>
int prepare_classb(int L);
// sums per member: [member][8 + T] doubles; partial buffer sized by globsum_partials()
// ntr: tracers summed (class A and B); sums per member: [member][8 + ntr]
template <typename R>
void launch_globsum(const Launch&, const Grid<R>&, const Strides&, int ntr, const R* dp3d, const R* tr,
                    const R* rn2d, const R* rc2d, const R* pr3d, const R* ex3d, const R* qf2d,
                    double* partial, double* sums);
size_t globsum_partials(int N, int L, int T, int members);
// edgvar2 (fim_dyn.cu): w = 3 N L values of scratch
template <typename R>
void launch_edgvar2(const Launch&, const Grid<R>&, const Strides&, const R* u, const R* v, R* u_edg, R* v_edg,
                    R* uvsq_edg, R* w);
// physics coupling (fim_cpl.cu); GFS arrays (nip, nvl), cell fastest, FP64
// gfs = ps, dp, p, u, v, dpdt, q, oz, cld, t; old6 = u, v, t, q, oz, cld
template <typename R>
void launch_cpl_dyn_to_phy(const Launch&, const Grid<R>&, const R* pr3d, const R* us3d, const R* vs3d,
                           const R* ws3d, const R* tr3d, double* const gfs[10], double* old6);
// gfs7 = p, u, v, q, cld, oz, t; col3 = geshem, rainc, evap; tend: 12 N L
// doubles of scratch with addtend (6 N L without smoothtend)
template <typename R>
void launch_cpl_phy_to_dyn(const Launch&, const Grid<R>&, double dt, double dtp, bool addtend, bool smoothtend,
                           const double* const gfs7[7], const double* old6, const double* const col3[3],
                           const R* dp3d, R* us3d, R* vs3d, R* tr3d, R* rn2d, R* rc2d, R* qf2d, double* tend);
template <typename R>
void launch_prdp_from_ex(const Launch&, const Grid<R>&, const Strides&, const R* ex3d, R* pr3d, R* dp3d);
void launch_step_begin(const Launch&, StepParams* sp);  // advances every active member

// fim_synth.cu: the seeded balanced state of one member slot
template <typename R>
int launch_synthetic(cudaStream_t stream, int N, int L, int nslot, int ntra, const double* lat,
                     const double* dps, unsigned long long seed, double sigma_ps, double noise, double ptop,
                     R* us3d, R* vs3d, R* dp3d, R* pr3d, R* ex3d, R* ph3d, R* mp3d, R* tr3d);

}  // namespace fim
