/*
 * fim_gpu.h -- C-ABI of the GB300 horizontal dynamics step of FIM
 * (Flow-following finite-volume Icosahedral Model).
 *
 * Every routine of the reference dycore step has one entry point here with the
 * reference's Fortran argument order, so the Fortran driver dyn_run can call it
 * through an iso_c_binding interface.  Arrays keep the reference layout:
 * column-major with the level index fastest, e.g. u(nvl,nip),
 * pres(nvl+1,nip), u_edg(nvl,6,nip), tracr(nvl,nip,ntra),
 * trc_tdcy(nvl,nip,3,ntra), massfx(nvl,6,nip,3).
 *
 * Two families of entry points exist: the *_r8 family takes double fields
 * (a real*8 build of the caller, the FP64 context), the *_r4 family float
 * fields (the reference's default -r4 build, the FP32-mixed context).
 * Field pointers are device pointers when the context was created with
 * host_pointers == 0 (the fast, device-resident mode) and host pointers
 * otherwise (each call then stages its inputs and outputs through the device).
 *
 * All functions return a status code and never abort the process.
 * The AB3 (Adams-Bashforth) time-slot indices and weights that the reference
 * keeps in module_variables live in the context; fim_abstart_* advances them.
 */
#ifndef FIM_GPU_H
#define FIM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FIM_OK 0
#define FIM_EINVAL 1      /* bad argument, size or configuration */
#define FIM_ENOMEM 2      /* device or host allocation failed */
#define FIM_ECUDA 3       /* a CUDA runtime call failed */
#define FIM_ENUMERIC 4    /* NaN or non-positive layer thickness detected */
#define FIM_ETIMEDOUT 5   /* a bounded device-side wait gave up */
#define FIM_ENOTSUP 6     /* option of the reference that this build does not implement */

#define FIM_PREC_F64 0    /* every field and every operation in double */
#define FIM_PREC_F32 1    /* FP32 fields and arithmetic, FP64 column scans and budgets */

/*
 * Grid tables, in the layout of FIMsrc/cntl/module_constants.F90:45-104 with
 * Fortran (1-based) cell and edge numbers.  Filled by fim_grid_build or by the
 * caller from its own glvl.dat (FIMsrc/fim/horizontal/dyn_init.F90:373-549).
 */
typedef struct fim_grid_desc {
  int glvl;
  int nip;                 /* 10*4^glvl+2 */
  int32_t *nprox;          /* nprox(nip): 5 or 6 */
  int32_t *prox;           /* prox(6,nip): neighbour across edge; prox(6)=prox(5) at pentagons */
  int32_t *proxs;          /* proxs(6,nip): the neighbour's number of the shared edge */
  double *lat, *lon;       /* lat(nip), lon(nip) in radians (may be NULL for ctx creation: then corio/grndspd need them) */
  double *area;            /* area(nip) m^2 */
  double *cs, *sn;         /* cs(4,6,nip), sn(4,6,nip) */
  double *sidevec_c;       /* sidevec_c(2,6,nip) */
  double *sidevec_e;       /* sidevec_e(2,6,nip) */
  double *sideln;          /* sideln(6,nip) */
  double *rprox_ln;        /* rprox_ln(6,nip) */
  double *corner_xy;       /* corner_xy(6,2,nip), optional */
  double *hfcoef;          /* hfcoef(6,6,nip) */
} fim_grid_desc;

/* Namelist knobs used on the path (FIMsrc/cntl/fimnamelist.F90:95-119,
 * FIMsrc/cntl/module_control.F90:97-100), reference defaults in brackets. */
typedef struct fim_config {
  int nvl;                 /* layers */
  int ntra;                /* class-A tracers, slot 1 = potential temperature (>= 4) */
  int precision;           /* FIM_PREC_F64 or FIM_PREC_F32 */
  int members;             /* ensemble members sharing the grid (>= 1) */
  int host_pointers;       /* 1: entry points receive host arrays */
  double dt;               /* time step, s */
  int kbl;                 /* [2] fixed-depth layers near the surface */
  int flux_conserv_schm;   /* 1: FCT cnuity; 2: mass_adv flux limiter (the reference default) */
  int hi_order_flux_comp;  /* [1] edgvar3 supplies dp_edg and tracers 2..ntra */
  double intfc_smooth;     /* [30] m/s */
  double slak;             /* [0.5] */
  int miglim;              /* [1] */
  int remap_optn;          /* [2] 1 PCM, 2 PLM, 3 PPM */
  double ptop;             /* [30] Pa */
  double thktop;           /* [30] Pa */
  double veldff_bkgnd;     /* [0.3] */
  double veldff_boost;     /* [3] */
  int biharm_frst, biharm_last; /* [0,0] */
  double rleigh;           /* [2] 1/day */
  double rlthresh;         /* [90] m/s */
  double rltaper;          /* [0.4] */
  int pure_sig;            /* [0]; 1 is not supported (FIM_ENOTSUP) */
  const double *thetac;    /* thetac(nvl): hybgen target potential temperature */
  const double *dpsig;     /* dpsig(nvl): minimum layer thickness, Pa */
  int ntrb;                /* [0] class-B tracers, stored after the ntra class-A ones
                              (tracer slots ntra+1..ntra+ntrb); ntra+ntrb <= 32 */
  int dtratio;             /* [6] class-B / class-A time-step ratio (fimnamelist.F90:87) */
  int member_group;        /* [0] members advanced together through the dynamics of a
                              step; 0 = all.  The step's edge work fields and scratch
                              are held for one group, which bounds their memory */
  int hi_order_uv_comp;    /* [0] hiOrderUVComp: edgvar2 after edgvar1 in fim_step
                              (needs the grid's corner_xy) */
  int stream_priority;     /* [0] CUDA priority of the context's streams (lower runs
                              first; clamped to the device's range): contexts that
                              share a GPU, e.g. serving pools of different grids,
                              can let the short steps through first */
  int tracer_chunk;        /* [0] tracers a launch of the fused tracer kernels takes
                              (their scratch is 12 nvl nip values a tracer and member);
                              0: as many as ~48 GB of scratch allows */
} fim_config;

typedef struct fim_ctx fim_ctx;

/* Global budget sums of FIMsrc/fim/horizontal/globsum.F90:39-130 (real*8). */
typedef struct fim_budget {
  double qmass, qmsqv, qmsqw, qmso3, qmste, qmstr, qmstrn, qmstrc;
} fim_budget;

/* ---- grid ------------------------------------------------------------- */
/* nip of an icosahedral grid level; -1 for an unsupported level */
int fim_grid_nip(int glvl);
/* Build the level-glvl grid into caller buffers sized by g->nip
 * (FIMsrc/prep/grid/icos.F90, GridGen.F90, getlvl.F90). */
int fim_grid_build(int glvl, fim_grid_desc *g);

/* ---- context ---------------------------------------------------------- */
/* Upload the grid tables and derived fields (dyn_init.F90:311-338,545-549,
 * 752-767) and fix the configuration; replaces GPUinit/copytoGPUinit
 * (FIMsrc/fim/horizontal/cuda/GPUinit.cu:12-54, dyn_init.F90:199,1198).
 * FIM_EINVAL when a neighbour number or an edge's mirror slot is out of range,
 * or an edge has no mirror: prox(proxs(e,i), prox(e,i)) must be i. */
int fim_ctx_create(const fim_grid_desc *grid, const fim_config *cfg, fim_ctx **out);
int fim_ctx_destroy(fim_ctx *ctx);
/* last CUDA error text of the context (GetLastError.cu:6-14 replacement) */
const char *fim_ctx_last_error(const fim_ctx *ctx);
/* device stream the context launches on (a cudaStream_t) */
void *fim_ctx_stream(fim_ctx *ctx);
/* bytes of device memory the context (and its states) currently own: grid
 * tables, state fields and every scratch buffer allocated so far (no
 * counterpart in the reference, which allocates host arrays) */
int64_t fim_ctx_device_bytes(const fim_ctx *ctx);
/* AB3 slots (Fortran numbering 1..3) and weights of the context */
int fim_get_ab(const fim_ctx *ctx, int *nf, int *of, int *vof, double *ab1, double *ab2, double *ab3);
int fim_set_ab(fim_ctx *ctx, int nf, int of, int vof, double ab1, double ab2, double ab3);

/* ---- per-routine entry points, reference argument order -------------- */
/* FIMsrc/fim/horizontal/abstart.F90:14-68 */
int fim_abstart(fim_ctx *ctx, int its, int its_start, int *nf, int *of, int *vof,
                double *adbash1, double *adbash2, double *adbash3);

/* FIMsrc/fim/horizontal/edgvar1.F90:27-29 (eqwgt, janjic=0 branches) */
int fim_edgvar1_r8(fim_ctx *ctx, int its, const double *u_vel, const double *v_vel,
                   const double *delp, const double *pres, const double *exner,
                   const double *geop, const double *montg, const double *tracr,
                   double *u_edg, double *v_edg, double *dp_edg, double *lp_edg,
                   double *geop_edg, double *mont_edg, double *uvsq_edg, double *trc_edg);
int fim_edgvar1_r4(fim_ctx *ctx, int its, const float *u_vel, const float *v_vel,
                   const float *delp, const float *pres, const float *exner,
                   const float *geop, const float *montg, const float *tracr,
                   float *u_edg, float *v_edg, float *dp_edg, float *lp_edg,
                   float *geop_edg, float *mont_edg, float *uvsq_edg, float *trc_edg);

/* FIMsrc/fim/horizontal/edgvar2.F90:24-27 (hiOrderUVComp; the MORE_VARS block,
 * compiled out in the reference, is left out): rescales u_edg, v_edg and
 * updates uvsq_edg; the other edge fields pass through.  Needs the grid's
 * corner_xy (FIM_EINVAL without it). */
int fim_edgvar2_r8(fim_ctx *ctx, int its, const double *u_vel, const double *v_vel,
                   const double *delp, const double *pres, const double *exner,
                   const double *geop, const double *montg, const double *tracr,
                   double *u_edg, double *v_edg, double *dp_edg, double *lp_edg,
                   double *geop_edg, double *mont_edg, double *uvsq_edg, double *trc_edg);
int fim_edgvar2_r4(fim_ctx *ctx, int its, const float *u_vel, const float *v_vel,
                   const float *delp, const float *pres, const float *exner,
                   const float *geop, const float *montg, const float *tracr,
                   float *u_edg, float *v_edg, float *dp_edg, float *lp_edg,
                   float *geop_edg, float *mont_edg, float *uvsq_edg, float *trc_edg);

/* FIMsrc/fim/horizontal/edgvar3.F90:25-27 */
int fim_edgvar3_r8(fim_ctx *ctx, int its, const double *u_vel, const double *v_vel,
                   const double *delp, const double *pres, const double *exner,
                   const double *geop, const double *montg, const double *tracr,
                   double *u_edg, double *v_edg, double *dp_edg, double *lp_edg,
                   double *geop_edg, double *mont_edg, double *uvsq_edg, double *trc_edg);
int fim_edgvar3_r4(fim_ctx *ctx, int its, const float *u_vel, const float *v_vel,
                   const float *delp, const float *pres, const float *exner,
                   const float *geop, const float *montg, const float *tracr,
                   float *u_edg, float *v_edg, float *dp_edg, float *lp_edg,
                   float *geop_edg, float *mont_edg, float *uvsq_edg, float *trc_edg);

/* FIMsrc/fim/horizontal/cnuity.F90:23-25 (cnuity1..5) */
int fim_cnuity_r8(fim_ctx *ctx, int its, const double *u_velo, const double *v_velo,
                  const double *u_edg, const double *v_edg, const double *dp_edg,
                  const double *lp_edg, double *delp, double *pres, double *exner,
                  double *dp_tndcy, double *dplo_tndcy, double *massfx, double *omega);
int fim_cnuity_r4(fim_ctx *ctx, int its, const float *u_velo, const float *v_velo,
                  const float *u_edg, const float *v_edg, const float *dp_edg,
                  const float *lp_edg, float *delp, float *pres, float *exner,
                  float *dp_tndcy, float *dplo_tndcy, float *massfx, float *omega);

/* Allocation-free cnuity (no counterpart in the reference).  For callers that
 * may not allocate device memory while they run: fim_cnuity_r8/_r4 allocate
 * their FCT scratch on the first call; this entry point takes it from one
 * static 64 MiB array in the library image instead (every GPU that loads the
 * library holds it until exit).  Same arguments as fim_cnuity_r8 (context in
 * FIM_PREC_F64) or fim_cnuity_r4 (FIM_PREC_F32), passed as untyped device
 * pointers; host_pointers contexts are rejected.  Like those, it advances
 * member 0.  The scratch takes 11 x nip x nvl values: glvl 5 / nvl 64 fits in
 * FP64, glvl 6 / nvl 64 does not fit in either precision and is rejected with
 * FIM_EINVAL.  fim_ctx_create looks up the array's device address
 * (cudaGetSymbolAddress) on its device; under lazy module loading that is
 * when the module holding the array loads and its 64 MiB are committed, so
 * a caller that creates its contexts during start-up allocates nothing
 * later.  If that lookup failed, the first fim_cnuity_noalloc call on the
 * device retries it; that call should then come before any stream capture.
 * All calls on a device share the array: calls whose kernels overlap on the
 * GPU race. */
int fim_cnuity_noalloc(fim_ctx *ctx, int its, const void *u_velo, const void *v_velo,
                       const void *u_edg, const void *v_edg, const void *dp_edg,
                       const void *lp_edg, void *delp, void *pres, void *exner,
                       void *dp_tndcy, void *dplo_tndcy, void *massfx, void *omega);

/* FIMsrc/fim/horizontal/massadv.F90:21-23 (flux_conserv_schm = 2, the
 * reference default: flux limiter of flux_limiter.F90 + update_pres);
 * dp_edg is limited in place */
int fim_mass_adv_r8(fim_ctx *ctx, int its, const double *u_velo, const double *v_velo,
                    const double *u_edg, const double *v_edg, double *dp_edg, const double *lp_edg,
                    double *delp, double *pres, double *exner, double *dp_tndcy, double *massfx,
                    double *omega);
int fim_mass_adv_r4(fim_ctx *ctx, int its, const float *u_velo, const float *v_velo,
                    const float *u_edg, const float *v_edg, float *dp_edg, const float *lp_edg,
                    float *delp, float *pres, float *exner, float *dp_tndcy, float *massfx,
                    float *omega);

/* FIMsrc/fim/horizontal/trcadv.F90:19-20 (trcadv1..3, all tracers) */
int fim_trcadv_r8(fim_ctx *ctx, int its, const double *trcr_edg, double *tracr, double *trcdp,
                  double *trc_tdcy, double *trclo_tdcy, const double *massfx, const double *delp);
int fim_trcadv_r4(fim_ctx *ctx, int its, const float *trcr_edg, float *tracr, float *trcdp,
                  float *trc_tdcy, float *trclo_tdcy, const float *massfx, const float *delp);

/* FIMsrc/fim/horizontal/momtum.F90:16-18 (dissip, del4prep, momtum1) */
int fim_momtum_r8(fim_ctx *ctx, int its, double *u_velo, double *v_velo, const double *exner,
                  double *relvor, const double *u_edg, const double *v_edg,
                  const double *trcr_edg, const double *geop_edg, const double *mont_edg,
                  const double *uvsq_edg, double *u_tndcy, double *v_tndcy, const double *dp3d);
int fim_momtum_r4(fim_ctx *ctx, int its, float *u_velo, float *v_velo, const float *exner,
                  float *relvor, const float *u_edg, const float *v_edg,
                  const float *trcr_edg, const float *geop_edg, const float *mont_edg,
                  const float *uvsq_edg, float *u_tndcy, float *v_tndcy, const float *dp3d);

/* FIMsrc/fim/horizontal/hybgen.F90:20-26 (regrid_1d, dffusn_lev, remap_1d);
 * targt may be NULL to use the context's thetac */
int fim_hybgen_r8(fim_ctx *ctx, int its, const double *targt, double *us3d, double *vs3d,
                  double *tr3d, double *sdot, double *ex3d, double *dp3d, double *pr3d);
int fim_hybgen_r4(fim_ctx *ctx, int its, const float *targt, float *us3d, float *vs3d,
                  float *tr3d, float *sdot, float *ex3d, float *dp3d, float *pr3d);

/* FIMsrc/fim/horizontal/hystat.F90:23-24 */
int fim_hystat_r8(fim_ctx *ctx, int its, double *ph3d, const double *ex3d, double *mp3d,
                  const double *dp3d, double *tr3d, double *trdp, double *psrf, double *ptdcy);
int fim_hystat_r4(fim_ctx *ctx, int its, float *ph3d, const float *ex3d, float *mp3d,
                  const float *dp3d, float *tr3d, float *trdp, float *psrf, float *ptdcy);

/* Physics coupling, the dynamics side of phy_run (FIMsrc/fim/horizontal/cpl_run.F90,
 * cpl_dyn_to_phy :151-263 and cpl_phy_to_dyn :266-536, called from run.F90:325-331).
 * The GFS physics arrays are double (kind_evod) in both families, (nip, nvl)
 * with the cell index fastest; gfs_ps is (nip).  callphy = 0 does nothing, as
 * in the reference.  cpl_dyn_to_phy also keeps, in the context, the six
 * gfs_*_old copies (u, v, t, q, oz, cld) that cpl_phy_to_dyn's tendency
 * method (addtend) uses; addtend without a preceding cpl_dyn_to_phy is
 * FIM_EINVAL.  smoothtend applies dffusn8_lyr (dffusn.F90:110-129) to the
 * tendencies with length dt*20, dt the context's time step; dtp is the
 * physics time step.  Of cpl_phy_to_dyn's surface outputs only the columns
 * globsum reads are formed: rn2d += max(0,geshem)*1000,
 * rc2d += max(0,rainc)*1000, qf2d = -evap; the others are plain copies of
 * physics fields that a host driver makes. */
int fim_cpl_dyn_to_phy_r8(fim_ctx *ctx, int its, int callphy, const double *pr3d, const double *us3d,
                          const double *vs3d, const double *ws3d, const double *tr3d, double *gfs_ps,
                          double *gfs_dp, double *gfs_p, double *gfs_u, double *gfs_v, double *gfs_dpdt,
                          double *gfs_q, double *gfs_oz, double *gfs_cld, double *gfs_t);
int fim_cpl_dyn_to_phy_r4(fim_ctx *ctx, int its, int callphy, const float *pr3d, const float *us3d,
                          const float *vs3d, const float *ws3d, const float *tr3d, double *gfs_ps,
                          double *gfs_dp, double *gfs_p, double *gfs_u, double *gfs_v, double *gfs_dpdt,
                          double *gfs_q, double *gfs_oz, double *gfs_cld, double *gfs_t);
int fim_cpl_phy_to_dyn_r8(fim_ctx *ctx, int its, int callphy, int addtend, int smoothtend, double dtp,
                          const double *gfs_p, const double *gfs_u, const double *gfs_v, const double *gfs_q,
                          const double *gfs_cld, const double *gfs_oz, const double *gfs_t,
                          const double *geshem, const double *rainc, const double *evap, const double *dp3d,
                          double *us3d, double *vs3d, double *tr3d, double *rn2d, double *rc2d, double *qf2d);
int fim_cpl_phy_to_dyn_r4(fim_ctx *ctx, int its, int callphy, int addtend, int smoothtend, double dtp,
                          const double *gfs_p, const double *gfs_u, const double *gfs_v, const double *gfs_q,
                          const double *gfs_cld, const double *gfs_oz, const double *gfs_t,
                          const double *geshem, const double *rainc, const double *evap, const float *dp3d,
                          float *us3d, float *vs3d, float *tr3d, float *rn2d, float *rc2d, float *qf2d);

/* Class-B tracer transport (module_transp3d, FIMsrc/fim/horizontal/transp3d.F90).
 * transp0 (transp3d.F90:21): cumufx = 0, dpinit = dp3d.
 * transp1 (transp3d.F90:43): cumufx += adbash1..3 x massfx(nf,of,vof), with the
 *   AB3 slots and weights of the context (fim_abstart / fim_set_ab).
 * transp2 (transp3d.F90:82, fct3d.F90:4): vertical mass flux from the
 *   time-integrated continuity equation, then 3-D FCT transport of the class-B
 *   tracers, the slots ntra+1..ntra+ntrb of tracr (nvl,nip,ntra+ntrb).
 * fim_step calls transp1 after cnuity/mass_adv every step and transp2 and
 * transp0 at steps its with mod(its,dtratio) == 0 (dyn_run.F90:388-403). */
int fim_transp0_r8(fim_ctx *ctx, int its, double *cumufx, const double *dp3d, double *dpinit);
int fim_transp0_r4(fim_ctx *ctx, int its, float *cumufx, const float *dp3d, float *dpinit);
int fim_transp1_r8(fim_ctx *ctx, int its, double *cumufx, const double *massfx);
int fim_transp1_r4(fim_ctx *ctx, int its, float *cumufx, const float *massfx);
int fim_transp2_r8(fim_ctx *ctx, int its, double *tracr, const double *cumufx, const double *dpinit,
                   const double *dpfinl);
int fim_transp2_r4(fim_ctx *ctx, int its, float *tracr, const float *cumufx, const float *dpinit,
                   const float *dpfinl);

/* FIMsrc/fim/horizontal/globsum.F90:39; rn2d, rc2d, qf2d may be NULL (zero);
 * qtrcr(ntra) and the budget are double in both families */
int fim_globsum_r8(fim_ctx *ctx, int its, const double *dp3d, const double *tr,
                   const double *rn2d, const double *rc2d, const double *pr3d,
                   const double *ex3d, const double *qf2d, double *qtrcr, fim_budget *out);
int fim_globsum_r4(fim_ctx *ctx, int its, const float *dp3d, const float *tr,
                   const float *rn2d, const float *rc2d, const float *pr3d,
                   const float *ex3d, const float *qf2d, double *qtrcr, fim_budget *out);

/* ---- device-resident state and the fused step ------------------------ */
/* Prognostic and work arrays of FIMsrc/cntl/module_variables.F90:23-91 for all
 * members of the context, owned by the library. */
typedef struct fim_state fim_state;

/* field identifiers for fim_state_field */
enum fim_field {
  FIM_US3D = 0, FIM_VS3D, FIM_DP3D, FIM_PR3D, FIM_EX3D, FIM_PH3D, FIM_MP3D, FIM_TR3D,
  FIM_TRDP, FIM_U_TDCY, FIM_V_TDCY, FIM_DP_TDCY, FIM_DPL_TDCY, FIM_TRC_TDCY, FIM_TRL_TDCY,
  FIM_MASSFX, FIM_WS3D, FIM_SDOT, FIM_RELVOR, FIM_PSRF, FIM_PTDCY,
  FIM_U_EDG, FIM_V_EDG, FIM_DP_EDG, FIM_LP_EDG, FIM_MONT_EDG, FIM_UVSQ_EDG, FIM_GEOP_EDG,
  FIM_TRC_EDG, FIM_CUMUFX, FIM_DPINIT, FIM_NFIELDS
};

/* tr3d and trdp of a state hold ntra+ntrb tracers; cumufx (nvl,6,nip) and
 * dpinit (nvl,nip) are the class-B transport's flux integral and initial
 * thickness (module_variables.F90:27,89), empty (count 0) without class-B
 * tracers.  With member_group < members the edge work fields (u_edg ..
 * trc_edg) exist for member_group members only.
 * With hi_order_flux_comp (the fused tracer transport, which forms the
 * tracers' edge values on chip) trc_edg holds theta's edge values only
 * (6 nvl nip values a member).  After a fused step the edge work fields are
 * in the step's internal form: in an FP32 context mont_edg holds
 * edge-minus-cell values. */
int fim_state_alloc(fim_ctx *ctx, fim_state **out);
int fim_state_free(fim_ctx *ctx, fim_state *st);
/* device pointer and element count of one member's field */
int fim_state_field(fim_ctx *ctx, fim_state *st, int field, int member, void **dptr, int64_t *count);
/* host <-> device copy of one member's field (element type per precision) */
int fim_state_upload(fim_ctx *ctx, fim_state *st, int field, int member, const void *host);
int fim_state_download(fim_ctx *ctx, fim_state *st, int field, int member, void *host);
/* FP64 initial field for an FP32-mixed state (no counterpart in the
 * reference, whose -r4 build reads its initial state in real*4): the field's
 * FP32 copy is set as by fim_state_upload, and the FP64 values are kept
 * until fim_state_init / fim_state_init_member, whose initial adjustment
 * (hybgen, pressures from the Exner function, hystat) then starts from them.
 * That adjustment runs in FP64 in both precisions; fields given only in FP32
 * enter it widened.  Only the fields the adjustment reads are taken: us3d,
 * vs3d, dp3d, pr3d, ex3d, ph3d (its bottom interface, the surface
 * geopotential) and tr3d; FIM_EINVAL otherwise.  In an FP64 context this is
 * fim_state_upload. */
int fim_state_upload_f64(fim_ctx *ctx, fim_state *st, int field, int member, const double *host);
/* The same for one AB3 slot (1..3, Fortran numbering) of a tendency field
 * (u_tdcy, v_tdcy, dp_tdcy, dpl_tdcy: one nvl x nip block per slot; trc_tdcy,
 * trl_tdcy: one per tracer).  host holds the whole field as for
 * fim_state_upload; only the slot's blocks move.  No reference counterpart:
 * a driver that keeps the state on the host between steps moves the slots the
 * next step reads (of, vof: fim_member_get_step's slots advanced by one) and
 * the one it writes (nf) instead of the whole history.  FIM_EINVAL for other
 * fields or slots. */
int fim_state_upload_slot(fim_ctx *ctx, fim_state *st, int field, int member, int slot, const void *host);
int fim_state_download_slot(fim_ctx *ctx, fim_state *st, int field, int member, int slot, void *host);

/* dyn_init.F90:870-906,1037-1094 for every member: trdp, hybgen(its=0),
 * pressure/thickness from Exner, hystat(its=0), zero tendencies, AB3 slots.
 * In an FP32-mixed context the adjustment (hybgen to hystat) runs in FP64 on
 * the member's fields (see fim_state_upload_f64) and its results are rounded
 * into the state once, the Montgomery potential into its float-float pair. */
int fim_state_init(fim_ctx *ctx, fim_state *st);

/* One dyn_run iteration of every member (dyn_run.F90:119-425): hybgen and
 * hystat of step its-1 (from a member's second step on; dyn_init's stand in
 * before the first), then abstart, edgvar1, edgvar3, cnuity or mass_adv,
 * trcadv and momtum of step its, then the globsum budgets of the resulting
 * state.  The state between calls is therefore the reference's state between
 * dyn_run calls, which is what its restart files hold.
 * use_graph != 0 captures the step once as a CUDA graph and replays it. */
int fim_step(fim_ctx *ctx, fim_state *st, int its, int use_graph);

/* Continuous batching: every member slot carries its own step counter and
 * AB3 slots, so members of one batch can start at different times.
 * fim_state_init_member initialises one slot (after its fields were
 * uploaded) and activates it; fim_step_active advances every active slot by
 * one step; idle slots are skipped by the kernels. */
int fim_state_init_member(fim_ctx *ctx, fim_state *st, int member);
int fim_member_set_active(fim_ctx *ctx, fim_state *st, int member, int active);
int fim_member_its(const fim_ctx *ctx, int member);
/* A member that carries fewer tracers than the context (ntr of ntra, theta
 * included): the tracer transport, the remap and the budget sums of later
 * steps leave its tracer slots ntr..ntra-1 as they are (zero, for a slot
 * padded with zeros) and do no work for them; its tracers 1..ntr evolve as
 * in a context of ntr tracers.  FIM_ENOTSUP without hi_order_flux_comp or
 * with class-B tracers.  No counterpart in the reference (serving). */
int fim_member_set_tracers(fim_ctx *ctx, int member, int ntr);
/* A seeded balanced initial state made on the device in one member slot
 * (no counterpart in the reference, whose initial state comes from GFS data,
 * dyn_init.F90:826): surface pressure 1000 hPa + N(0, sigma_ps) Pa,
 * thicknesses proportional to dpsig, theta 300 -> 600 K, u = 35 m/s cos(lat)
 * (+ N(0, noise) m/s on u and v), tracers 2..ntra U[0, 1e-2), the slot's
 * tracers past ntra zero, ph3d and mp3d zero.  A counter-based generator:
 * the state depends only on the seed and the grid.  Asynchronous on the
 * context stream; fim_state_init(_member) follows as after an upload. */
int fim_state_synthetic(fim_ctx *ctx, fim_state *st, int member, unsigned long long seed, int ntra,
                        double sigma_ps, double noise);

/* Step state of one member for restart files: the completed step count
 * (itsm1, restart.F90:58), the AB3 slots nf/of/vof in Fortran numbering and
 * the weights adbash1..3 (the first record of restart_dyn.F90:37/114).
 * fim_member_set_step restores them and activates the member; its next step
 * is itsm1+1 (restart.F90:125), with the weights abstart would carry on. */
int fim_member_get_step(const fim_ctx *ctx, int member, int *itsm1, int *nf, int *of, int *vof,
                        double *adbash1, double *adbash2, double *adbash3);
int fim_member_set_step(fim_ctx *ctx, int member, int itsm1, int nf, int of, int vof,
                        double adbash1, double adbash2, double adbash3);
int fim_step_active(fim_ctx *ctx, fim_state *st, int use_graph);

/* The step with the state on the host (no counterpart in the reference,
 * whose state lives in host memory).  fim_state_set_host registers the host
 * copy of one member's field (null unregisters); pinned memory (cudaHostAlloc
 * or cudaHostRegister) lets the copies run beside the kernels.  The edge work
 * fields stay on the device (FIM_EINVAL).  fim_step_io(its) then runs
 * fim_step(its) with the registered fields moved in and out: each goes up
 * before the first kernel that reads or writes it and comes down as soon as
 * the step's last writer of it is done, on two copy streams beside the
 * compute stream.  The step is cut at the stages of dyn_run: hybgen + hystat
 * + edge interpolation, cnuity (its AB3 slots arrive just before it), momtum
 * (which shares no field with the tracer transport, so it runs before it
 * here), the tracer transport in chunks of about a seventh of the tracers
 * (each chunk's AB3 slots arrive while the chunk before it runs; its results
 * leave while the next one runs).  Results equal fim_step's bit for bit.  AB3
 * tendency fields move only the slots the step reads (of, vof) and writes
 * (nf); ws3d, sdot and relvor, which the step rewrites whole, only come down
 * (ptdcy, of whose two time levels a step writes one, goes both ways); from
 * its = 2 on, dp3d, mp3d and trdp (the class-A tracers' part; with ntrb = 0)
 * only come down too, because the step's opening hybgen and hystat rewrite
 * them before any read.
 * Returns when every download has landed; *h2d_bytes and *d2h_bytes (may be
 * null) get the bytes moved.  FIM_ENOTSUP with member_group < members. */
int fim_state_set_host(fim_ctx *ctx, fim_state *st, int field, int member, void *host);

/* Persistent cnuity (no counterpart in the reference).  With on = 1, cnuity1
 * to cnuity4 (cnuity_compute.F90:17-374) of every member run as one
 * cooperative launch of as many blocks as the GPU holds at once, the stages
 * separated by grid barriers instead of kernel boundaries; results are the
 * kernel-per-stage path's bit for bit.  Each barrier gives up after timeout_s
 * seconds (0 < timeout_s <= 60): the launch then ends, and fim_check returns
 * FIM_ETIMEDOUT (that step's results are not valid; the context stays
 * usable).  Applies to fim_step, fim_step_io and the per-routine cnuity from
 * the next call on; a state's step graph is captured again.
 * fim_set_barrier_test(ctx, 1) makes each barrier wait for one block more than
 * the launch has, so that it runs out (the test of the time limit); 0 restores
 * it. */
int fim_set_persistent(fim_ctx *ctx, int on, double timeout_s);
int fim_set_barrier_test(fim_ctx *ctx, int phantom_arrivals);
int fim_step_io(fim_ctx *ctx, fim_state *st, int its, int64_t *h2d_bytes, int64_t *d2h_bytes);

/* Member budgets after the last step (qmass, tracer integrals qtrcr(ntra)). */
int fim_state_budget(fim_ctx *ctx, fim_state *st, int member, double *qtrcr, fim_budget *out);

/* Accumulated device-side status flags (NaN / non-positive thickness); resets them. */
int fim_check(fim_ctx *ctx, fim_state *st, int *flags);

/* Per-kernel CUDA-event timing on the context stream (for measurement;
 * steps must run without graph replay while it is on). */
int fim_profile_enable(fim_ctx *ctx, int on);
/* "kernel launches total_ms" lines accumulated since the last report; with
 * fim_step_io also its timeline, "io:<mark> steps total_ms" with each mark's
 * time from the step's start (up_begin/up_end of each stage's uploads,
 * computed when a stage's last kernel is done, down_begin/down_end of its
 * downloads, end) */
int fim_profile_report(fim_ctx *ctx, char *buf, int len);

/* Kernel launches issued since the context was created (own kernels only). */
int64_t fim_launch_count(const fim_ctx *ctx);

/* Shape of the fused tracer kernels (no counterpart in the reference): levels
 * per thread (1, 2 or 4) and threads per block (the cell patch's cells times
 * 2 or 4 threads a cell; a block covers levels-per-thread x threads-a-cell
 * levels), picked by timing the candidates on the state before the first
 * fused step (0 levels: the widest the layout admits, before tuning);
 * probe_ms is the winner's time for one probe.  FIM_TRC_VK / FIM_TRC_GC pin
 * the shape and FIM_AUTOTUNE=0 skips the timing. */
int fim_tracer_shape(const fim_ctx *ctx, int *levels_per_thread, int *threads_per_block, float *probe_ms);

/* Cell patches of the fused tracer kernels for a grid (no counterpart in the
 * reference), built as fim_ctx_create builds them and checked on the host:
 * every cell in exactly one patch, every frame neighbour equal to prox and
 * every edge's other side equal to prox/proxs.  No device use.  Patches are
 * side x side cells of one rhombus (1 <= side <= 8; each pole is a patch of
 * its own), or grown breadth-first for another cell numbering.  Outputs (each
 * may be null): the number of patches, the largest patch, the largest frame
 * (a patch and its two neighbour rings) and the most ring edges of a patch.
 * FIM_OK, or FIM_EINVAL for malformed tables, a side out of range or a frame
 * over 255 cells. */
int fim_grid_patches(const fim_grid_desc *grid, int side, int *npatch, int *max_cells, int *max_frame,
                     int *max_ring_edges);

#ifdef __cplusplus
}
#endif
#endif /* FIM_GPU_H */
