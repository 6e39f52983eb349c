/*
 * CPU oracle of the FIM horizontal dynamics step -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, double-precision restatement of the reference Fortran routines
 * (the .F90 files of FIMsrc/fim/horizontal), loop for loop, used by the test suite, the
 * smoke check and the CPU-baseline leg of bench.py as the checker.  The
 * product library never links or calls it.
 *
 * Parity status: the floating-point routines are UNPINNED.  The reference
 * ships no golden vectors or unit fixtures for this path and cannot be
 * compiled on either machine (Fortran, no compiler); the restatement is
 * pinned only by the reference's own in-code invariants (column-integral
 * conservation in hybgen, FCT positivity/monotonicity, global mass
 * conservation) which the tests check.  The integer grid tables the oracle
 * and the product read (prox, proxs, nprox) are pinned bit for bit against a
 * restatement of the reference's grid generator (grid_ref.py).
 *
 * Index conventions: 0-based, reference layout with the level index fastest.
 *   cell field (nvl,nip):        f[i*nvl + k]
 *   interface field (nvl+1,nip): f[i*(nvl+1) + k]
 *   edge field (nvl,6,nip):      f[(i*6 + e)*nvl + k]
 *   AB3 field (nvl,nip,3):       f[(s*nip + i)*nvl + k]
 *   tracers (nvl,nip,ntra):      f[(t*nip + i)*nvl + k]
 *   tracer AB3 (nvl,nip,3,ntra): f[((t*3 + s)*nip + i)*nvl + k]
 *   tracer edges (nvl,6,nip,ntra): f[((t*nip + i)*6 + e)*nvl + k]
 *   massfx (nvl,6,nip,3):        f[((s*nip + i)*6 + e)*nvl + k]
 * Grid tables are 0-based: prox[i*6+e], proxs[i*6+e], cs[(i*6+e)*4+q], ...
 */
#ifndef FIM_ORACLE_H
#define FIM_ORACLE_H

typedef struct orc_ctx {
  int nip, nvl, ntra;
  const int *prox, *proxs, *nprox;
  const double *cs, *sn, *sidevec_c, *sidevec_e, *sideln, *area, *rarea, *corio, *grndspd;
  const double *hfcoef;
  double dt;
  int kbl, hi_order, miglim, remap_optn;
  int flux_schm;                        /* 1 FCT cnuity, 2 mass_adv flux limiter */
  double intfc_smooth, slak, ptop, thktop, rleigh, rlthresh, rltaper;
  const double *thetac, *dpsig;         /* [nvl] */
  const double *dfflen, *biharw;        /* [nvl] */
  const double *smoo_coeff;             /* [nvl+1] */
  double dfflen_max;
  int nf, of, vof;                      /* 0-based AB3 slots */
  double ab1, ab2, ab3;
  long diag_flags;                      /* conservation-check failures seen */
  int ntrb;                             /* class-B tracers after the ntra class-A ones */
  const double *corner_xy;              /* [nip][2][6]: corner_xy(6,2,nip), for edgvar2 */
} orc_ctx;

void orc_derived(int nip, int nvl, int kbl, double dt, double intfc_smooth,
                 double veldff_bkgnd, double veldff_boost, int biharm_frst, int biharm_last,
                 const double *lat, const double *area, const double *sideln,
                 double *rarea, double *corio, double *grndspd, double *dfflen,
                 double *biharw, double *smoo_coeff, double *dfflen_max);

void orc_set_threads(int n);
void orc_abstart(orc_ctx *c, int its);
void orc_edgvar1(const orc_ctx *c, const double *u, const double *v, const double *delp,
                 const double *pres, const double *exner, const double *geop,
                 const double *montg, const double *tracr, double *u_edg, double *v_edg,
                 double *dp_edg, double *lp_edg, double *geop_edg, double *mont_edg,
                 double *uvsq_edg, double *trc_edg);
/* edgvar2 (edgvar2.F90:24-319, MORE_VARS off): rescale the edge wind to the
 * corner-gradient speed average; u_edg, v_edg, uvsq_edg in place */
void orc_edgvar2(const orc_ctx *c, const double *u, const double *v, double *u_edg, double *v_edg,
                 double *uvsq_edg);
void orc_edgvar3(const orc_ctx *c, const double *delp, const double *tracr,
                 double *dp_edg, double *trc_edg);
void orc_cnuity(const orc_ctx *c, const double *u, const double *v, const double *u_edg,
                const double *v_edg, const double *dp_edg, const double *lp_edg, double *delp,
                double *pres, double *exner, double *dp_tndcy, double *dplo_tndcy,
                double *massfx, double *omega);
void orc_mass_adv(const orc_ctx *c, const double *u, const double *v, const double *u_edg,
                  const double *v_edg, double *dp_edg, const double *lp_edg, double *delp,
                  double *pres, double *exner, double *dp_tndcy, double *massfx, double *omega);
void orc_trcadv(const orc_ctx *c, const double *trc_edg, double *tracr, double *trcdp,
                double *trc_tdcy, double *trl_tdcy, const double *massfx, const double *delp);
void orc_momtum(const orc_ctx *c, double *u, double *v, const double *exner, double *relvor,
                const double *u_edg, const double *v_edg, const double *trc_edg,
                const double *mont_edg, const double *uvsq_edg, double *u_tndcy,
                double *v_tndcy, const double *dp3d);
void orc_hybgen(orc_ctx *c, int its, const double *targt, double *us3d, double *vs3d,
                double *tr3d, double *sdot, double *ex3d, double *dp3d, double *pr3d);
void orc_hystat(const orc_ctx *c, int its, double *ph3d, const double *ex3d, double *mp3d,
                const double *dp3d, double *tr3d, double *trdp, double *psrf, double *ptdcy);
void orc_globsum(const orc_ctx *c, const double *dp3d, const double *tr, const double *rn2d,
                 const double *rc2d, const double *pr3d, const double *ex3d,
                 const double *qf2d, double *qtrcr, double *sums8);
/* class-B tracer transport (transp3d.F90:21-241, fct3d.F90:4-482); class-B
 * tracers are the slots ntra..ntra+ntrb-1 of tracr; cumufx is an edge field */
void orc_transp0(const orc_ctx *c, double *cumufx, const double *dp3d, double *dpinit);
void orc_transp1(const orc_ctx *c, double *cumufx, const double *massfx);
void orc_transp2(const orc_ctx *c, int ntrb, double *tracr, const double *cumufx, const double *dpinit,
                 const double *dpfinl);
/* physics coupling, the dynamics side (cpl_run.F90:151-263, 266-536; dffusn.F90:110-129):
 * GFS arrays (nip, nvl) with the cell index fastest; old6 = the six fields
 * cpl_dyn_to_phy keeps (u, v, t, q, oz, cld), one nvl*nip block each */
void orc_cpl_dyn_to_phy(const orc_ctx *c, const double *pr3d, const double *us3d, const double *vs3d,
                        const double *ws3d, const double *tr3d, double *gfs_ps, double *gfs_dp,
                        double *gfs_p, double *gfs_u, double *gfs_v, double *gfs_dpdt, double *gfs_q,
                        double *gfs_oz, double *gfs_cld, double *gfs_t, double *old6);
void orc_cpl_phy_to_dyn(const orc_ctx *c, int addtend, int smoothtend, double dtp, const double *gfs_p,
                        const double *gfs_u, const double *gfs_v, const double *gfs_q, const double *gfs_cld,
                        const double *gfs_oz, const double *gfs_t, const double *old6, const double *dp3d,
                        double *us3d, double *vs3d, double *tr3d, const double *geshem, const double *rainc,
                        const double *evap, double *rn2d, double *rc2d, double *qf2d);
/* pressure and thickness from Exner after the start-up hybgen (dyn_init.F90:895-906) */
void orc_prdp_from_ex(const orc_ctx *c, const double *ex3d, double *pr3d, double *dp3d);

#endif
