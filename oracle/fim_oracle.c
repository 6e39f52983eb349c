/*
 * CPU oracle of the FIM horizontal dynamics step -- TEST INFRASTRUCTURE ONLY.
 * See fim_oracle.h for the layout and the parity status (unpinned).
 * Each function names the reference lines it restates.  Compiled with
 * -ffp-contract=off so the result does not depend on the host ISA.
 */
#include "fim_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* thread count of the OpenMP loops (the timed CPU baseline runs 1 and all cores) */
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* FIMsrc/cntl/module_constants.F90:14-27 */
static const double PI = 3.14159265;
static const double EARTHRAD = 6371220.;
static const double OMEGX2 = 1.4584e-4;
static const double GRVITY = 9.80665;
static const double P1000 = 100000.;
static const double CP = 1004.6855;
static const double RD = 287.0586;
static const double QVMIN = 1.e-10;
static const double QWMIN = 1.e-10;

#define C2(k, i) ((size_t)(i) * L + (k))
#define I2(k, i) ((size_t)(i) * (L + 1) + (k))
#define E3(k, e, i) (((size_t)(i) * 6 + (e)) * L + (k))
#define S3(k, i, s) (((size_t)(s) * N + (i)) * L + (k))
#define T3(k, i, t) (((size_t)(t) * N + (i)) * L + (k))
#define TS(k, i, s, t) ((((size_t)(t) * 3 + (s)) * N + (i)) * L + (k))
#define TE(k, e, i, t) ((((size_t)(t) * N + (i)) * 6 + (e)) * L + (k))
#define MF(k, e, i, s) ((((size_t)(s) * N + (i)) * 6 + (e)) * L + (k))

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

/* dyn_init.F90:123-126 (taper), 309-338 (dfflen, smoo_coeff, biharw), 752-767 */
void orc_derived(int nip, int nvl, int kbl, double dt, double intfc_smooth,
                 double veldff_bkgnd, double veldff_boost, int biharm_frst, int biharm_last,
                 const double *lat, const double *area, const double *sideln,
                 double *rarea, double *corio, double *grndspd, double *dfflen,
                 double *biharw, double *smoo_coeff, double *dfflen_max) {
  (void)sideln;
  int ndamp = (int)(0.1 * nvl);
  for (int k = 1; k <= nvl; k++) {
    double wgt = dmax(0., (double)(k - nvl + ndamp) / (double)ndamp);
    dfflen[k - 1] = dt * (veldff_bkgnd * (1. - wgt) + dmax(veldff_bkgnd, veldff_boost) * wgt);
  }
  double mx = dfflen[0];
  for (int k = 1; k < nvl; k++) mx = dmax(mx, dfflen[k]);
  *dfflen_max = mx;
  for (int k = 0; k <= nvl; k++) smoo_coeff[k] = 0.;
  for (int k = kbl + 2; k <= nvl; k++) {
    double d1 = (double)((kbl + 1) - k), d2 = (double)((nvl + 1) - k);
    double t1 = d1 * d1 / (9. + d1 * d1), t2 = d2 * d2 / (9. + d2 * d2);
    smoo_coeff[k - 1] = dt * intfc_smooth * t1 * t2;
  }
  for (int k = 1; k <= nvl; k++) {
    double w = 0.;
    if (k >= biharm_frst && k <= biharm_last) w = 1.;
    if (biharm_frst > 1 && biharm_frst < nvl) w = dmax(0., dmin(1., .5 + .2 * (double)(k - biharm_frst)));
    if (biharm_last > 1 && biharm_last < nvl) w = dmax(0., dmin(1., .5 + .2 * (double)(biharm_last - k)));
    biharw[k - 1] = w;
    dfflen[k - 1] = dfflen[k - 1] * (1. + 4. * w * w);
  }
  for (int i = 0; i < nip; i++) {
    corio[i] = OMEGX2 * sin(lat[i]);
    rarea[i] = 1. / area[i];
    grndspd[i] = EARTHRAD * 2. * PI * cos(lat[i]) / 86164.;
  }
}

/* abstart.F90:33-65 with Fortran slots 1..3 mapped to 0..2 */
void orc_abstart(orc_ctx *c, int its) {
  c->nf = (c->nf + 1) % 3;
  c->of = (c->of + 1) % 3;
  c->vof = (c->vof + 1) % 3;
  if (its == 1) { c->ab1 = c->dt; c->ab2 = 0.; c->ab3 = 0.; }
  if (its == 2) { c->ab1 = c->dt * 1.5; c->ab2 = -c->dt * .5; c->ab3 = 0.; }
  if (its == 3) { c->ab1 = c->dt * 23. / 12.; c->ab2 = -c->dt * 16. / 12.; c->ab3 = c->dt * 5. / 12.; }
}

/* edgvar1.F90:156-511 (eqwgt=.true., janjic=0, simpson=.false.) */
void orc_edgvar1(const orc_ctx *c, const double *u, const double *v, const double *delp,
                 const double *pres, const double *exner, const double *geop,
                 const double *montg, const double *tracr, double *u_edg, double *v_edg,
                 double *dp_edg, double *lp_edg, double *geop_edg, double *mont_edg,
                 double *uvsq_edg, double *trc_edg) {
  (void)exner; (void)geop; (void)geop_edg;
  const int N = c->nip, L = c->nvl;
  const double divby6 = 1. / 6., eps = 0.001;
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    const int np = c->nprox[ipn];
    for (int edg = 0; edg < np; edg++) {
      const int i1 = ipn, i2 = c->prox[ipn * 6 + edg];
      const int i3t = c->prox[ipn * 6 + (edg - 1 + np) % np];
      const int i3l = c->prox[ipn * 6 + (edg + 1) % np];
      const double *cs = c->cs + (ipn * 6 + edg) * 4, *sn = c->sn + (ipn * 6 + edg) * 4;
      for (int k = 0; k < L; k++) {
        double u3trl = cs[2] * u[C2(k, i3t)] + sn[2] * v[C2(k, i3t)];
        double v3trl = -sn[2] * u[C2(k, i3t)] + cs[2] * v[C2(k, i3t)];
        double u1ldg = cs[0] * u[C2(k, i1)] + sn[0] * v[C2(k, i1)];
        double v1ldg = -sn[0] * u[C2(k, i1)] + cs[0] * v[C2(k, i1)];
        double u2ldg = cs[1] * u[C2(k, i2)] + sn[1] * v[C2(k, i2)];
        double v2ldg = -sn[1] * u[C2(k, i2)] + cs[1] * v[C2(k, i2)];
        double u3ldg = cs[3] * u[C2(k, i3l)] + sn[3] * v[C2(k, i3l)];
        double v3ldg = -sn[3] * u[C2(k, i3l)] + cs[3] * v[C2(k, i3l)];
        double ue = (2. * (u1ldg + u2ldg) + u3trl + u3ldg) * divby6;
        double ve = (2. * (v1ldg + v2ldg) + v3trl + v3ldg) * divby6;
        double m_1ldg = sqrt(u1ldg * u1ldg + v1ldg * v1ldg);
        double m_2ldg = sqrt(u2ldg * u2ldg + v2ldg * v2ldg);
        double m_3trl = sqrt(u3trl * u3trl + v3trl * v3trl);
        double m_3ldg = sqrt(u3ldg * u3ldg + v3ldg * v3ldg);
        double m_1 = sqrt(ue * ue + ve * ve);
        double m_2 = (2. * (m_1ldg + m_2ldg) + m_3trl + m_3ldg) * divby6;
        ue = ue * m_2 / dmax(eps, m_1);
        ve = ve * m_2 / dmax(eps, m_1);
        u_edg[E3(k, edg, ipn)] = ue;
        v_edg[E3(k, edg, ipn)] = ve;
        if (!c->hi_order)
          dp_edg[E3(k, edg, ipn)] =
              (2. * (delp[C2(k, i1)] + delp[C2(k, i2)]) + delp[C2(k, i3t)] + delp[C2(k, i3l)]) * divby6;
        lp_edg[E3(k, edg, ipn)] =
            (pres[I2(k, i1)] + pres[I2(k + 1, i1)] + pres[I2(k, i2)] + pres[I2(k + 1, i2)] +
             .5 * (pres[I2(k, i3t)] + pres[I2(k + 1, i3t)] + pres[I2(k, i3l)] + pres[I2(k + 1, i3l)])) *
            divby6;
        mont_edg[E3(k, edg, ipn)] =
            (2. * (montg[C2(k, i1)] + montg[C2(k, i2)]) + montg[C2(k, i3t)] + montg[C2(k, i3l)]) * divby6;
        uvsq_edg[E3(k, edg, ipn)] = .5 * (ue * ue + ve * ve);
      }
    }
  }
  const int ntr = c->hi_order ? 1 : c->ntra;
  for (int nt = 0; nt < ntr; nt++) {
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++) {
      const int np = c->nprox[ipn];
      for (int k = 0; k < L; k++) trc_edg[TE(k, 5, ipn, nt)] = 0.;
      for (int edg = 0; edg < np; edg++) {
        const int i1 = ipn, i2 = c->prox[ipn * 6 + edg];
        const int i3t = c->prox[ipn * 6 + (edg - 1 + np) % np];
        const int i3l = c->prox[ipn * 6 + (edg + 1) % np];
        for (int k = 0; k < L; k++)
          trc_edg[TE(k, edg, ipn, nt)] = (2. * (tracr[T3(k, i1, nt)] + tracr[T3(k, i2, nt)]) +
                                          tracr[T3(k, i3t, nt)] + tracr[T3(k, i3l, nt)]) * divby6;
      }
    }
  }
}

/* edgvar3.F90:136-163 */
static void edgval_eval(const orc_ctx *c, int ipn, const double *b /* [7][L] */, double *edgval,
                        size_t estride /* element stride between edges */) {
  const int L = c->nvl, n = c->nprox[ipn];
  for (int i = n; i < 6; i++)
    for (int k = 0; k < L; k++) edgval[i * estride + k] = 0.;
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < L; k++) edgval[i * estride + k] = b[n * L + k];
    for (int j = 0; j < n; j++) {
      const double h = c->hfcoef[(ipn * 6 + i) * 6 + j];
      for (int k = 0; k < L; k++) edgval[i * estride + k] += (b[j * L + k] - b[n * L + k]) * h;
    }
  }
}

/* edgvar3.F90:64-133; loop 2 keeps the reference's store-once pairing */
/* edgvar2 (edgvar2.F90:24-319): uv_speed_edge, gradient, uv_speed, then the
 * per-edge magnitude correction (the MORE_VARS block is compiled out) */
void orc_edgvar2(const orc_ctx *c, const double *u, const double *v, double *u_edg, double *v_edg,
                 double *uvsq_edg) {
  const int N = c->nip, L = c->nvl;
  const double divby6 = 1. / 6., eps = 0.00001;
  double *spe = malloc(sizeof(double) * (size_t)N * 6 * L); /* uv_spd_edg */
  double *gc = malloc(sizeof(double) * (size_t)N * 6 * L);  /* grad_conr */
  double *spd = malloc(sizeof(double) * (size_t)N * L);     /* uv_spd */
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    for (int e = 0; e < c->nprox[ipn]; e++)
      for (int k = 0; k < L; k++)
        spe[E3(k, e, ipn)] = sqrt(u_edg[E3(k, e, ipn)] * u_edg[E3(k, e, ipn)] +
                                  v_edg[E3(k, e, ipn)] * v_edg[E3(k, e, ipn)]);
    for (int k = 0; k < L; k++)
      spd[C2(k, ipn)] = sqrt(u[C2(k, ipn)] * u[C2(k, ipn)] + v[C2(k, ipn)] * v[C2(k, ipn)]);
  }
  /* gradient (edgvar2.F90:231-258) */
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    for (int k = 0; k < L; k++) {
      double g1 = 0., g2 = 0.;
      for (int e = 0; e < c->nprox[ipn]; e++) {
        g1 = g1 + spe[E3(k, e, ipn)] * c->sidevec_c[(ipn * 6 + e) * 2 + 1];
        g2 = g2 - spe[E3(k, e, ipn)] * c->sidevec_c[(ipn * 6 + e) * 2 + 0];
      }
      g1 = g1 * c->rarea[ipn];
      g2 = g2 * c->rarea[ipn];
      for (int e = 0; e < c->nprox[ipn]; e++)
        gc[E3(k, e, ipn)] = 0.5 * (g1 * c->corner_xy[(ipn * 2 + 0) * 6 + e] + g2 * c->corner_xy[(ipn * 2 + 1) * 6 + e]);
    }
  }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    const int np = c->nprox[ipn];
    for (int edg = 0; edg < np; edg++) {
      const int conr1 = edg, conr2 = (edg + 1) % np;
      const int nba = c->prox[ipn * 6 + edg], nbaedg = c->proxs[ipn * 6 + edg];
      const int nbaconr1 = (nbaedg + 1) % c->nprox[nba], nbaconr2 = nbaedg;
      const int edgm1 = (edg - 1 + np) % np;
      const int nbm1 = c->prox[ipn * 6 + edgm1], nbm1conr = c->proxs[ipn * 6 + edgm1];
      const int edgp1 = (edg + 1) % np;
      const int nbp1 = c->prox[ipn * 6 + edgp1], nbp1conr = (c->proxs[ipn * 6 + edgp1] + 1) % c->nprox[nbp1];
      for (int k = 0; k < L; k++) {
        const double uv1conr1 = spd[C2(k, ipn)] + gc[E3(k, conr1, ipn)];
        const double uv2conr1 = spd[C2(k, nba)] + gc[E3(k, nbaconr1, nba)];
        const double uv3conr1 = spd[C2(k, nbm1)] + gc[E3(k, nbm1conr, nbm1)];
        const double uv1conr2 = spd[C2(k, ipn)] + gc[E3(k, conr2, ipn)];
        const double uv2conr2 = spd[C2(k, nba)] + gc[E3(k, nbaconr2, nba)];
        const double uv3conr2 = spd[C2(k, nbp1)] + gc[E3(k, nbp1conr, nbp1)];
        const size_t o = E3(k, edg, ipn);
        const double uvm1 = sqrt(u_edg[o] * u_edg[o] + v_edg[o] * v_edg[o]);
        const double uvm2 = (uv1conr1 + uv2conr1 + uv3conr1 + uv1conr2 + uv2conr2 + uv3conr2) * divby6;
        const double r_m = uvm1 < eps ? 1.0 : uvm2 / uvm1;
        u_edg[o] = u_edg[o] * r_m;
        v_edg[o] = v_edg[o] * r_m;
        uvsq_edg[o] = .5 * (u_edg[o] * u_edg[o] + v_edg[o] * v_edg[o]);
      }
    }
  }
  free(spe); free(gc); free(spd);
}

void orc_edgvar3(const orc_ctx *c, const double *delp, const double *tracr, double *dp_edg,
                 double *trc_edg) {
  const int N = c->nip, L = c->nvl;
#pragma omp parallel
  {
    double *b = (double *)malloc(sizeof(double) * 7 * L);
#pragma omp for schedule(static)
    for (int ipn = 0; ipn < N; ipn++) {
      const int np = c->nprox[ipn];
      for (int e = 0; e < np; e++)
        for (int k = 0; k < L; k++) b[e * L + k] = delp[C2(k, c->prox[ipn * 6 + e])];
      for (int k = 0; k < L; k++) b[np * L + k] = delp[C2(k, ipn)];
      edgval_eval(c, ipn, b, dp_edg + E3(0, 0, ipn), L);
      for (int nt = 1; nt < c->ntra; nt++) {
        for (int e = 0; e < np; e++)
          for (int k = 0; k < L; k++) b[e * L + k] = tracr[T3(k, c->prox[ipn * 6 + e], nt)];
        for (int k = 0; k < L; k++) b[np * L + k] = tracr[T3(k, ipn, nt)];
        edgval_eval(c, ipn, b, trc_edg + TE(0, 0, ipn, nt), L);
      }
    }
    free(b);
  }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    const int np = c->nprox[ipn];
    for (int edg = 0; edg < np; edg++) {
      const int nb = c->prox[ipn * 6 + edg], os = c->proxs[ipn * 6 + edg];
      if (ipn < nb) {
        for (int k = 0; k < L; k++) {
          double w = 0.5 * (dp_edg[E3(k, edg, ipn)] + dp_edg[E3(k, os, nb)]);
          dp_edg[E3(k, edg, ipn)] = w;
          dp_edg[E3(k, os, nb)] = w;
        }
        for (int nt = 1; nt < c->ntra; nt++)
          for (int k = 0; k < L; k++) {
            double w = 0.5 * (trc_edg[TE(k, edg, ipn, nt)] + trc_edg[TE(k, os, nb, nt)]);
            trc_edg[TE(k, edg, ipn, nt)] = w;
            trc_edg[TE(k, os, nb, nt)] = w;
          }
      }
    }
  }
}

/* cnuity.F90:103-226 driving cnuity_compute.F90 cnuity1..cnuity5 */
void orc_cnuity(const orc_ctx *c, const double *u, const double *v, const double *u_edg,
                const double *v_edg, const double *dp_edg, const double *lp_edg, double *delp,
                double *pres, double *exner, double *dp_tndcy, double *dplo_tndcy,
                double *massfx, double *omega) {
  const int N = c->nip, L = c->nvl;
  const int nf = c->nf, of = c->of, vof = c->vof;
  const double ab1 = c->ab1, ab2 = c->ab2, ab3 = c->ab3;
  const double thshld = 1.e-11;
  const size_t NE = (size_t)N * 6 * L, NC = (size_t)N * L;
  double *vnorm = (double *)malloc(sizeof(double) * NE);
  double *antifx = (double *)malloc(sizeof(double) * NE);
  double *delp_lo = (double *)malloc(sizeof(double) * NC);
  double *r_plus = (double *)malloc(sizeof(double) * NC);
  double *r_mnus = (double *)malloc(sizeof(double) * NC);

  /* cnuity1: cnuity_compute.F90:41-91 */
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++)
    for (int edg = 0; edg < c->nprox[ipn]; edg++) {
      const double *sv = c->sidevec_e + (ipn * 6 + edg) * 2;
      for (int k = 0; k < L; k++)
        vnorm[E3(k, edg, ipn)] = sv[1] * u_edg[E3(k, edg, ipn)] - sv[0] * v_edg[E3(k, edg, ipn)];
    }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    for (int k = 0; k < L; k++) {
      antifx[E3(k, 5, ipn)] = 0.;
      massfx[MF(k, 5, ipn, nf)] = 0.;
    }
    for (int edg = 0; edg < c->nprox[ipn]; edg++) {
      const int ipx = c->prox[ipn * 6 + edg], edx = c->proxs[ipn * 6 + edg];
      for (int k = 0; k < L; k++) {
        double vn = vnorm[E3(k, edg, ipn)], vx = vnorm[E3(k, edx, ipx)];
        double flxhi = vn * dp_edg[E3(k, edg, ipn)];
        double m = 0.5 * ((vn + fabs(vn)) * delp[C2(k, ipn)] - (vx + fabs(vx)) * delp[C2(k, ipx)]);
        massfx[MF(k, edg, ipn, nf)] = m;
        antifx[E3(k, edg, ipn)] = flxhi - m;
      }
    }
  }
  /* cnuity2: cnuity_compute.F90:114-146 */
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    for (int k = 0; k < L; k++) dplo_tndcy[S3(k, ipn, nf)] = 0.;
    for (int edg = 0; edg < c->nprox[ipn]; edg++)
      for (int k = 0; k < L; k++) dplo_tndcy[S3(k, ipn, nf)] += massfx[MF(k, edg, ipn, nf)];
    for (int k = 0; k < L; k++) {
      dplo_tndcy[S3(k, ipn, nf)] = -dplo_tndcy[S3(k, ipn, nf)] * c->rarea[ipn];
      delp_lo[C2(k, ipn)] = delp[C2(k, ipn)] + ab1 * dplo_tndcy[S3(k, ipn, nf)] +
                            ab2 * dplo_tndcy[S3(k, ipn, of)] + ab3 * dplo_tndcy[S3(k, ipn, vof)];
    }
  }
  /* cnuity3: cnuity_compute.F90:178-255 */
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    double pp[512], pm[512];
    double *p_plus = L <= 512 ? pp : (double *)malloc(sizeof(double) * L);
    double *p_mnus = L <= 512 ? pm : (double *)malloc(sizeof(double) * L);
    for (int k = 0; k < L; k++) { p_plus[k] = 0.; p_mnus[k] = 0.; }
    for (int edg = 0; edg < c->nprox[ipn]; edg++)
      for (int k = 0; k < L; k++) {
        double a = antifx[E3(k, edg, ipn)];
        if (a <= 0.) p_plus[k] = p_plus[k] - a;
        else p_mnus[k] = p_mnus[k] + a;
      }
    const int *pr = c->prox + ipn * 6;
    for (int k = 0; k < L; k++) {
      double dpmax = dmax(delp_lo[C2(k, ipn)], delp[C2(k, ipn)]);
      double dpmin = dmin(delp_lo[C2(k, ipn)], delp[C2(k, ipn)]);
      for (int e = 0; e < 6; e++) {
        dpmax = dmax(dpmax, delp_lo[C2(k, pr[e])]);
        dpmin = dmin(dpmin, delp_lo[C2(k, pr[e])]);
      }
      for (int e = 0; e < 6; e++) {
        dpmax = dmax(dpmax, delp[C2(k, pr[e])]);
        dpmin = dmin(dpmin, delp[C2(k, pr[e])]);
      }
      dpmax = dmax(0., dpmax);
      dpmin = dmax(0., dpmin);
      double q_plus = (dpmax - delp_lo[C2(k, ipn)] -
                       (ab2 * dmin(0., dp_tndcy[S3(k, ipn, of)]) + ab3 * dmax(0., dp_tndcy[S3(k, ipn, vof)]))) /
                      ab1 * c->area[ipn];
      double q_mnus = (delp_lo[C2(k, ipn)] - dpmin +
                       (ab2 * dmax(0., dp_tndcy[S3(k, ipn, of)]) + ab3 * dmin(0., dp_tndcy[S3(k, ipn, vof)]))) /
                      ab1 * c->area[ipn];
      r_plus[C2(k, ipn)] = dmax(0., dmin(1., q_plus / dmax(p_plus[k], thshld)));
      r_mnus[C2(k, ipn)] = dmax(0., dmin(1., q_mnus / dmax(p_mnus[k], thshld)));
    }
    if (L > 512) { free(p_plus); free(p_mnus); }
  }
  /* cnuity4: cnuity_compute.F90:291-369 */
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++)
    for (int edg = 0; edg < c->nprox[ipn]; edg++) {
      const int px = c->prox[ipn * 6 + edg];
      for (int k = 0; k < L; k++) {
        double a = antifx[E3(k, edg, ipn)], clip;
        if (a >= 0.) clip = dmin(r_mnus[C2(k, ipn)], r_plus[C2(k, px)]);
        else clip = dmin(r_plus[C2(k, ipn)], r_mnus[C2(k, px)]);
        a = a * clip;
        antifx[E3(k, edg, ipn)] = a;
        massfx[MF(k, edg, ipn, nf)] = massfx[MF(k, edg, ipn, nf)] + a;
      }
    }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++)
    for (int k = 0; k < L; k++) {
      double at = 0.;
      for (int edg = 0; edg < c->nprox[ipn]; edg++) at = at + antifx[E3(k, edg, ipn)];
      at = -at * c->rarea[ipn];
      dp_tndcy[S3(k, ipn, nf)] = dplo_tndcy[S3(k, ipn, nf)] + at;
      delp[C2(k, ipn)] = delp[C2(k, ipn)] + ab1 * dp_tndcy[S3(k, ipn, nf)] +
                         ab2 * dp_tndcy[S3(k, ipn, of)] + ab3 * dp_tndcy[S3(k, ipn, vof)];
    }
  /* cnuity5: cnuity_compute.F90:408-445 */
  const double rdcp = RD / CP;
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    double coltend = 0.;
    for (int k = L - 1; k >= 0; k--) {
      pres[I2(k, ipn)] = pres[I2(k + 1, ipn)] + delp[C2(k, ipn)];
      exner[I2(k, ipn)] = CP * pow(pres[I2(k, ipn)] / P1000, rdcp);
      double lyrtend = (ab1 * dp_tndcy[S3(k, ipn, nf)] + ab2 * dp_tndcy[S3(k, ipn, of)] +
                        ab3 * dp_tndcy[S3(k, ipn, vof)]) / c->dt;
      omega[C2(k, ipn)] = coltend + 0.5 * lyrtend;
      coltend = coltend + lyrtend;
      double dpdx = 0., dpdy = 0.;
      for (int edg = 0; edg < c->nprox[ipn]; edg++) {
        const double *sv = c->sidevec_c + (ipn * 6 + edg) * 2;
        dpdx = dpdx + lp_edg[E3(k, edg, ipn)] * sv[1];
        dpdy = dpdy - lp_edg[E3(k, edg, ipn)] * sv[0];
      }
      omega[C2(k, ipn)] = omega[C2(k, ipn)] + (u[C2(k, ipn)] * dpdx + v[C2(k, ipn)] * dpdy) * c->rarea[ipn];
    }
  }
  free(vnorm); free(antifx); free(delp_lo); free(r_plus); free(r_mnus);
}

/* massadv.F90:58-118 (flux_conserv_schm=2): flux_limiter.F90 edgeNormVel
 * (68-92) and limiter (120-262, M1 branch), massadv_compute.F90
 * massflux_newdepth (22-95) and update_pres (97-170, identical to cnuity5) */
void orc_mass_adv(const orc_ctx *c, const double *u, const double *v, const double *u_edg,
                  const double *v_edg, double *dp_edg, const double *lp_edg, double *delp,
                  double *pres, double *exner, double *dp_tndcy, double *massfx, double *omega) {
  const int N = c->nip, L = c->nvl;
  const int nf = c->nf, of = c->of, vof = c->vof;
  const double ab1 = c->ab1, ab2 = c->ab2, ab3 = c->ab3, dt = c->dt;
  const size_t NE = (size_t)N * 6 * L, NC = (size_t)N * L;
  double *vnorm = (double *)calloc(NE, sizeof(double));
  double *c_num = (double *)calloc(NE, sizeof(double));
  double *q_star = (double *)calloc(NE, sizeof(double));
  double *q_min_out = (double *)malloc(sizeof(double) * NC);
  double *q_max_out = (double *)malloc(sizeof(double) * NC);
  const double max_out_bound = 100000.0;
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++)
    for (int edg = 0; edg < c->nprox[ipn]; edg++) {
      const double *sv = c->sidevec_e + (ipn * 6 + edg) * 2;
      for (int k = 0; k < L; k++) {
        vnorm[E3(k, edg, ipn)] = sv[1] * u_edg[E3(k, edg, ipn)] - sv[0] * v_edg[E3(k, edg, ipn)];
        c_num[E3(k, edg, ipn)] = fabs(vnorm[E3(k, edg, ipn)]) * dt * c->rarea[ipn];
      }
    }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    const int np = c->nprox[ipn];
    for (int edg = 0; edg < np; edg++) {
      const int nbm1 = c->prox[ipn * 6 + (edg - 1 + np) % np], nbp1 = c->prox[ipn * 6 + (edg + 1) % np];
      const int ipx = c->prox[ipn * 6 + edg];
      for (int k = 0; k < L; k++) {
        double qmn = dmin(dmin(dmin(delp[C2(k, ipn)], delp[C2(k, ipx)]), delp[C2(k, nbm1)]), delp[C2(k, nbp1)]);
        double qmx = dmax(dmax(dmax(delp[C2(k, ipn)], delp[C2(k, ipx)]), delp[C2(k, nbm1)]), delp[C2(k, nbp1)]);
        q_star[E3(k, edg, ipn)] = dmax(qmn, dmin(qmx, dp_edg[E3(k, edg, ipn)]));
      }
    }
    for (int k = 0; k < L; k++) {
      double qminin = 1.79769313486231571e308, qmaxin = 0.0, cqmin = 0.0, cqmax = 0.0, cin = 0.0, cout = 0.0;
      const double g = delp[C2(k, ipn)];
      for (int edg = 0; edg < np; edg++) {
        const size_t o = E3(k, edg, ipn);
        const int ipx = c->prox[ipn * 6 + edg];
        double qmn, qmx;
        if (vnorm[o] > 0) {
          qmn = dmin(q_star[o], g);
          qmx = dmax(q_star[o], g);
          cout = cout + c_num[o];
        } else {
          qmn = dmin(q_star[o], delp[C2(k, ipx)]);
          qmx = dmax(q_star[o], delp[C2(k, ipx)]);
          cin = cin + c_num[o];
          qminin = dmin(qminin, qmn);
          qmaxin = dmax(qmaxin, qmx);
          cqmin = cqmin + c_num[o] * qmn;
          cqmax = cqmax + c_num[o] * qmx;
        }
      }
      const double qmin_next = dmin(g, qminin), qmax_next = dmax(g, qmaxin);
      if (cout != 0.0) {
        q_min_out[C2(k, ipn)] = (g + ab1 / dt * cqmax - qmax_next * (1.0 + cin - cout) +
                                 ab2 * dp_tndcy[S3(k, ipn, of)] + ab3 * dp_tndcy[S3(k, ipn, vof)]) / cout / ab1 * dt;
        q_max_out[C2(k, ipn)] = (g + ab1 / dt * cqmin - qmin_next * (1.0 + cin - cout) +
                                 ab2 * dp_tndcy[S3(k, ipn, of)] + ab3 * dp_tndcy[S3(k, ipn, vof)]) / cout / ab1 * dt;
      } else {
        q_min_out[C2(k, ipn)] = -max_out_bound;
        q_max_out[C2(k, ipn)] = max_out_bound;
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++)
    for (int edg = 0; edg < c->nprox[ipn]; edg++) {
      const int ipx = c->prox[ipn * 6 + edg];
      for (int k = 0; k < L; k++) {
        const size_t o = E3(k, edg, ipn);
        const int src = vnorm[o] > 0 ? ipn : ipx;
        dp_edg[o] = dmax(q_min_out[C2(k, src)], dmin(q_max_out[C2(k, src)], q_star[o]));
      }
    }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    for (int edg = 0; edg < c->nprox[ipn]; edg++)
      for (int k = 0; k < L; k++) massfx[MF(k, edg, ipn, nf)] = vnorm[E3(k, edg, ipn)] * dp_edg[E3(k, edg, ipn)];
    for (int k = 0; k < L; k++) {
      double t = 0.;
      for (int edg = 0; edg < c->nprox[ipn]; edg++) t = t + massfx[MF(k, edg, ipn, nf)];
      t = -t * c->rarea[ipn];
      dp_tndcy[S3(k, ipn, nf)] = t;
      double d = delp[C2(k, ipn)] + ab1 * t + ab2 * dp_tndcy[S3(k, ipn, of)] + ab3 * dp_tndcy[S3(k, ipn, vof)];
      delp[C2(k, ipn)] = dmax(d, 0.0);
    }
  }
  free(vnorm); free(c_num); free(q_star); free(q_min_out); free(q_max_out);
  /* update_pres (massadv_compute.F90:131-167) is cnuity5 */
  const double rdcp = RD / CP;
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    double coltend = 0.;
    for (int k = L - 1; k >= 0; k--) {
      pres[I2(k, ipn)] = pres[I2(k + 1, ipn)] + delp[C2(k, ipn)];
      exner[I2(k, ipn)] = CP * pow(pres[I2(k, ipn)] / P1000, rdcp);
      double lyrtend = (ab1 * dp_tndcy[S3(k, ipn, nf)] + ab2 * dp_tndcy[S3(k, ipn, of)] +
                        ab3 * dp_tndcy[S3(k, ipn, vof)]) / dt;
      omega[C2(k, ipn)] = coltend + 0.5 * lyrtend;
      coltend = coltend + lyrtend;
      double dpdx = 0., dpdy = 0.;
      for (int edg = 0; edg < c->nprox[ipn]; edg++) {
        const double *sv = c->sidevec_c + (ipn * 6 + edg) * 2;
        dpdx = dpdx + lp_edg[E3(k, edg, ipn)] * sv[1];
        dpdy = dpdy - lp_edg[E3(k, edg, ipn)] * sv[0];
      }
      omega[C2(k, ipn)] = omega[C2(k, ipn)] + (u[C2(k, ipn)] * dpdx + v[C2(k, ipn)] * dpdy) * c->rarea[ipn];
    }
  }
}

/* trcadv.F90:95-207 driving trcadv_compute.F90 trcadv1..trcadv3 */
void orc_trcadv(const orc_ctx *c, const double *trc_edg, double *tracr, double *trcdp,
                double *trc_tdcy, double *trl_tdcy, const double *massfx, const double *delp) {
  const int N = c->nip, L = c->nvl;
  const int nf = c->nf, of = c->of, vof = c->vof;
  const double ab1 = c->ab1, ab2 = c->ab2, ab3 = c->ab3;
  const double thshld = 1.e-11;
  const size_t NE = (size_t)N * 6 * L, NC = (size_t)N * L;
  double *antiflx = (double *)malloc(sizeof(double) * NE);
  double *flx_lo = (double *)malloc(sizeof(double) * NE);
  double *trmax = (double *)malloc(sizeof(double) * NC);
  double *trmin = (double *)malloc(sizeof(double) * NC);
  double *trcr_lo = (double *)malloc(sizeof(double) * NC);
  double *r_plus = (double *)malloc(sizeof(double) * NC);
  double *r_mnus = (double *)malloc(sizeof(double) * NC);
  for (int t = 0; t < c->ntra; t++) {
    /* trcadv1: trcadv_compute.F90:55-135 */
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++) {
      for (int k = 0; k < L; k++) {
        trl_tdcy[TS(k, ipn, nf, t)] = 0.;
        trc_tdcy[TS(k, ipn, nf, t)] = 0.;
        antiflx[E3(k, 5, ipn)] = 0.;
      }
      for (int edg = 0; edg < c->nprox[ipn]; edg++) {
        const int ipx = c->prox[ipn * 6 + edg], edx = c->proxs[ipn * 6 + edg];
        for (int k = 0; k < L; k++) {
          double m = massfx[MF(k, edg, ipn, nf)], mx = massfx[MF(k, edx, ipx, nf)];
          double flx_hi = m * trc_edg[TE(k, edg, ipn, t)];
          double fl = 0.5 * ((m + fabs(m)) * tracr[T3(k, ipn, t)] - (mx + fabs(mx)) * tracr[T3(k, ipx, t)]);
          flx_lo[E3(k, edg, ipn)] = fl;
          antiflx[E3(k, edg, ipn)] = flx_hi - fl;
        }
      }
      for (int edg = 0; edg < c->nprox[ipn]; edg++)
        for (int k = 0; k < L; k++) trl_tdcy[TS(k, ipn, nf, t)] += flx_lo[E3(k, edg, ipn)];
      const int *pr = c->prox + ipn * 6;
      for (int k = 0; k < L; k++) {
        trl_tdcy[TS(k, ipn, nf, t)] = -trl_tdcy[TS(k, ipn, nf, t)] * c->rarea[ipn];
        double trcdp_lo = trcdp[T3(k, ipn, t)] + ab1 * trl_tdcy[TS(k, ipn, nf, t)] +
                          ab2 * trl_tdcy[TS(k, ipn, of, t)] + ab3 * trl_tdcy[TS(k, ipn, vof, t)];
        double mx = tracr[T3(k, ipn, t)], mn = tracr[T3(k, ipn, t)];
        for (int e = 0; e < 6; e++) {
          mx = dmax(mx, tracr[T3(k, pr[e], t)]);
          mn = dmin(mn, tracr[T3(k, pr[e], t)]);
        }
        mx = dmax(0., mx);
        mn = dmax(0., mn);
        trmax[C2(k, ipn)] = mx;
        trmin[C2(k, ipn)] = mn;
        trcr_lo[C2(k, ipn)] = dmax(mn, dmin(mx, trcdp_lo / dmax(thshld, delp[C2(k, ipn)])));
      }
    }
    /* trcadv2: trcadv_compute.F90:171-235 */
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++) {
      const int *pr = c->prox + ipn * 6;
      for (int k = 0; k < L; k++) {
        double s_plus = 0., s_mnus = 0.;
        for (int edg = 0; edg < c->nprox[ipn]; edg++) {
          double a = antiflx[E3(k, edg, ipn)];
          s_plus = s_plus - dmin(0., a);
          s_mnus = s_mnus + dmax(0., a);
        }
        double mx = dmax(trmax[C2(k, ipn)], trcr_lo[C2(k, ipn)]);
        double mn = dmin(trmin[C2(k, ipn)], trcr_lo[C2(k, ipn)]);
        for (int e = 0; e < 6; e++) {
          mx = dmax(mx, trcr_lo[C2(k, pr[e])]);
          mn = dmin(mn, trcr_lo[C2(k, pr[e])]);
        }
        mx = dmax(0., mx);
        mn = dmax(0., mn);
        trmax[C2(k, ipn)] = mx;
        trmin[C2(k, ipn)] = mn;
        double q_plus = ((mx - trcr_lo[C2(k, ipn)]) * delp[C2(k, ipn)] -
                         (ab2 * dmin(0., trc_tdcy[TS(k, ipn, of, t)]) + ab3 * dmax(0., trc_tdcy[TS(k, ipn, vof, t)]))) /
                        ab1 * c->area[ipn];
        double q_mnus = ((trcr_lo[C2(k, ipn)] - mn) * delp[C2(k, ipn)] +
                         (ab2 * dmax(0., trc_tdcy[TS(k, ipn, of, t)]) + ab3 * dmin(0., trc_tdcy[TS(k, ipn, vof, t)]))) /
                        ab1 * c->area[ipn];
        r_plus[C2(k, ipn)] = dmax(0., dmin(1., q_plus / dmax(s_plus, thshld)));
        r_mnus[C2(k, ipn)] = dmax(0., dmin(1., q_mnus / dmax(s_mnus, thshld)));
      }
    }
    /* trcadv3: trcadv_compute.F90:270-309 */
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++) {
      for (int k = 0; k < L; k++) {
        double at = 0.;
        for (int edg = 0; edg < c->nprox[ipn]; edg++) {
          const int px = c->prox[ipn * 6 + edg];
          double a = antiflx[E3(k, edg, ipn)];
          if (a >= 0.) a = a * dmin(r_mnus[C2(k, ipn)], r_plus[C2(k, px)]);
          else a = a * dmin(r_plus[C2(k, ipn)], r_mnus[C2(k, px)]);
          at = at + a;
        }
        at = -at * c->rarea[ipn];
        trc_tdcy[TS(k, ipn, nf, t)] = trl_tdcy[TS(k, ipn, nf, t)] + at;
        trcdp[T3(k, ipn, t)] = trcdp[T3(k, ipn, t)] + ab1 * trc_tdcy[TS(k, ipn, nf, t)] +
                               ab2 * trc_tdcy[TS(k, ipn, of, t)] + ab3 * trc_tdcy[TS(k, ipn, vof, t)];
        tracr[T3(k, ipn, t)] = dmax(trmin[C2(k, ipn)],
                                    dmin(trmax[C2(k, ipn)], trcdp[T3(k, ipn, t)] / dmax(thshld, delp[C2(k, ipn)])));
      }
    }
  }
  free(antiflx); free(flx_lo); free(trmax); free(trmin); free(trcr_lo); free(r_plus); free(r_mnus);
}

/* momtum.F90:86-152 with momtum_compute.F90 del4prep (16-95), dissip (102-229)
 * and momtum1 (231-450, janjic=0) */
void orc_momtum(const orc_ctx *c, double *u, double *v, const double *exner, double *relvor,
                const double *u_edg, const double *v_edg, const double *trc_edg,
                const double *mont_edg, const double *uvsq_edg, double *u_tndcy,
                double *v_tndcy, const double *dp3d) {
  const int N = c->nip, L = c->nvl;
  const int nf = c->nf, of = c->of, vof = c->vof;
  const double ab1 = c->ab1, ab2 = c->ab2, ab3 = c->ab3;
  const double thshld = 1.e-11;
  const size_t NC = (size_t)N * L;
  if (c->dfflen_max > 0.) {
    double *wu = (double *)malloc(sizeof(double) * NC), *wv = (double *)malloc(sizeof(double) * NC);
    double *ou = (double *)malloc(sizeof(double) * NC), *ov = (double *)malloc(sizeof(double) * NC);
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++)
      for (int k = 0; k < L; k++) {
        wu[C2(k, ipn)] = u[C2(k, ipn)];
        wv[C2(k, ipn)] = v[C2(k, ipn)];
        wu[C2(k, ipn)] = wu[C2(k, ipn)] + c->grndspd[ipn];
      }
    double bmax = 0.;
    for (int k = 0; k < L; k++) bmax = dmax(bmax, c->biharw[k]);
    if (bmax > 0.) {
      /* del4prep */
      memcpy(ou, wu, sizeof(double) * NC);
      memcpy(ov, wv, sizeof(double) * NC);
#pragma omp parallel for schedule(static)
      for (int ipn = 0; ipn < N; ipn++)
        for (int k = 0; k < L; k++) {
          double au = 0., av = 0.;
          for (int edg = 0; edg < c->nprox[ipn]; edg++) {
            const int ipx = c->prox[ipn * 6 + edg];
            const double *cs = c->cs + (ipn * 6 + edg) * 4, *sn = c->sn + (ipn * 6 + edg) * 4;
            double uxy2 = cs[1] * ou[C2(k, ipx)] + sn[1] * ov[C2(k, ipx)];
            double vxy2 = -sn[1] * ou[C2(k, ipx)] + cs[1] * ov[C2(k, ipx)];
            au = au + cs[0] * uxy2 - sn[0] * vxy2;
            av = av + sn[0] * uxy2 + cs[0] * vxy2;
          }
          double factor = c->biharw[k] / c->nprox[ipn];
          wu[C2(k, ipn)] = wu[C2(k, ipn)] - au * factor;
          wv[C2(k, ipn)] = wv[C2(k, ipn)] - av * factor;
        }
    }
    /* dissip: fluxes from the (possibly prepared) work fields, then increments */
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++)
      for (int k = 0; k < L; k++) {
        double su = 0., sv = 0.;
        const double factor = c->rarea[ipn] / dmax(dp3d[C2(k, ipn)], thshld);
        for (int edg = 0; edg < c->nprox[ipn]; edg++) {
          const int ipx = c->prox[ipn * 6 + edg];
          const double *cs = c->cs + (ipn * 6 + edg) * 4, *sn = c->sn + (ipn * 6 + edg) * 4;
          double uxy1 = cs[0] * wu[C2(k, ipn)] + sn[0] * wv[C2(k, ipn)];
          double vxy1 = -sn[0] * wu[C2(k, ipn)] + cs[0] * wv[C2(k, ipn)];
          double uxy2 = cs[1] * wu[C2(k, ipx)] + sn[1] * wv[C2(k, ipx)];
          double vxy2 = -sn[1] * wu[C2(k, ipx)] + cs[1] * wv[C2(k, ipx)];
          double a = dmax(dp3d[C2(k, ipn)], thshld), b = dmax(dp3d[C2(k, ipx)], thshld);
          double hf = a * b / (a + b);
          double ufx = (uxy2 - uxy1) * c->dfflen[k] * c->sideln[ipn * 6 + edg] * 2. * hf;
          double vfx = (vxy2 - vxy1) * c->dfflen[k] * c->sideln[ipn * 6 + edg] * 2. * hf;
          double uflux = cs[0] * ufx - sn[0] * vfx;
          double vflux = sn[0] * ufx + cs[0] * vfx;
          su = su + uflux * factor;
          sv = sv + vflux * factor;
        }
        ou[C2(k, ipn)] = su;
        ov[C2(k, ipn)] = sv;
      }
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++)
      for (int k = 0; k < L; k++) {
        u[C2(k, ipn)] = u[C2(k, ipn)] + ou[C2(k, ipn)];
        v[C2(k, ipn)] = v[C2(k, ipn)] + ov[C2(k, ipn)];
      }
    free(wu); free(wv); free(ou); free(ov);
  }
  /* momtum1 */
  const int ndamp = (int)(0.25 * L);
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    for (int k = 0; k < L; k++) {
      double pgfx = 0., pgfy = 0., rv = 0.;
      const double exm = .5 * (exner[I2(k, ipn)] + exner[I2(k + 1, ipn)]);
      for (int edg = 0; edg < c->nprox[ipn]; edg++) {
        const double *svc = c->sidevec_c + (ipn * 6 + edg) * 2;
        const double *sve = c->sidevec_e + (ipn * 6 + edg) * 2;
        const size_t o = E3(k, edg, ipn);
        pgfx = pgfx - (mont_edg[o] + uvsq_edg[o]) * svc[1] + exm * trc_edg[TE(k, edg, ipn, 0)] * svc[1];
        pgfy = pgfy + (mont_edg[o] + uvsq_edg[o]) * svc[0] - exm * trc_edg[TE(k, edg, ipn, 0)] * svc[0];
        rv = rv + (sve[0] * u_edg[o] + sve[1] * v_edg[o]);
      }
      pgfx = pgfx * c->rarea[ipn];
      pgfy = pgfy * c->rarea[ipn];
      rv = rv * c->rarea[ipn];
      relvor[C2(k, ipn)] = rv;
      double uzeta = (c->corio[ipn] + rv) * u[C2(k, ipn)];
      double vzeta = (c->corio[ipn] + rv) * v[C2(k, ipn)];
      u_tndcy[S3(k, ipn, nf)] = pgfx + vzeta;
      v_tndcy[S3(k, ipn, nf)] = pgfy - uzeta;
      u[C2(k, ipn)] = u[C2(k, ipn)] + ab1 * u_tndcy[S3(k, ipn, nf)] + ab2 * u_tndcy[S3(k, ipn, of)] +
                      ab3 * u_tndcy[S3(k, ipn, vof)];
      v[C2(k, ipn)] = v[C2(k, ipn)] + ab1 * v_tndcy[S3(k, ipn, nf)] + ab2 * v_tndcy[S3(k, ipn, of)] +
                      ab3 * v_tndcy[S3(k, ipn, vof)];
    }
    double q1 = u[C2(L - 1, ipn)] * u[C2(L - 1, ipn)] + v[C2(L - 1, ipn)] * v[C2(L - 1, ipn)];
    double q2 = u[C2(L - 2, ipn)] * u[C2(L - 2, ipn)] + v[C2(L - 2, ipn)] * v[C2(L - 2, ipn)];
    double q3 = u[C2(L - 3, ipn)] * u[C2(L - 3, ipn)] + v[C2(L - 3, ipn)] * v[C2(L - 3, ipn)];
    double qq = dmax(dmax(q1, q2), q3) / (c->rlthresh * c->rlthresh);
    if (qq > 1.) {
      qq = sqrt((qq - 1.) * qq);
      for (int k = L - 1 - ndamp; k < L; k++) {
        double factor = 1. - (c->dt / 86400.) * c->rleigh * qq * pow(2., c->rltaper * (double)(k + 1 - L));
        u[C2(k, ipn)] = u[C2(k, ipn)] * factor;
        v[C2(k, ipn)] = v[C2(k, ipn)] * factor;
      }
    }
  }
}

/* ---------------------------- hybgen ---------------------------------- */

/* hybgen.F90:792-890 */
static void restp_1d(const double *thold, const double *pkold, int kold, double *thnew,
                     double *pknew, const double *targt, int knew, long *flags) {
  double oldth[1024];
  oldth[kold - 1] = thold[kold - 1];
  for (int k = kold; k >= 2; k--) oldth[k - 2] = dmin(oldth[k - 1], thold[k - 2]);
  for (int k = 0; k < knew; k++) thnew[k] = targt[k];
  thnew[0] = dmin(dmin(oldth[0], oldth[kold - 1]), targt[0]);
  thnew[knew - 1] = dmax(dmax(oldth[0], oldth[kold - 1]), targt[knew - 1]);
  pknew[0] = pkold[0];
  pknew[knew] = pkold[kold];
  double colint = 0., colscl = 0., cloutt = 0.;
  for (int k = 0; k < kold; k++) {
    colint = colint + oldth[k] * (pkold[k + 1] - pkold[k]);
    colscl = colscl + fabs(oldth[k] * (pkold[k + 1] - pkold[k]));
  }
  int ko = 0;
  for (int k = 0; k < knew - 1; k++) {
    double pinteg = 0., tha, thb = thnew[k];
    for (;;) {
      tha = thb;
      thb = dmin(thnew[k + 1], dmax(thnew[k], oldth[ko]));
      pinteg = pinteg + pkold[ko] * (thb - tha);
      if (oldth[ko] < thnew[k + 1]) {
        if (ko < kold - 1) { ko++; continue; }
        tha = thb;
        thb = thnew[k + 1];
        pinteg = pinteg + pkold[kold] * (thb - tha);
      }
      break;
    }
    pknew[k + 1] = pknew[k];
    if (thnew[k + 1] > thnew[k]) pknew[k + 1] = pinteg / (thnew[k + 1] - thnew[k]);
    cloutt = cloutt + thnew[k] * (pknew[k + 1] - pknew[k]);
  }
  cloutt = cloutt + thnew[knew - 1] * (pknew[knew] - pknew[knew - 1]);
  if (fabs(cloutt - colint) > dmax(1.e-33, 1.e-6 * colscl)) (*flags)++;
}

/* hybgen.F90:1282-1437 (scenario 1) */
static void equilb(const double *thet, double *pres, int kk, double slak) {
  const double thin = RD / P1000;
  double pnew[1025];
  for (int k = 0; k <= kk; k++) pnew[k] = pres[k];
  for (int k = 3; k <= kk - 2; k++) { /* Fortran k */
    if (pnew[k - 3] > pnew[0] - thin) continue;
    double dp1 = pnew[k - 3] - pnew[k - 2];
    double dp2 = pnew[k - 2] - pnew[k - 1];
    double dp3 = pnew[k - 1] - pnew[k];
    double dp4 = pnew[k] - pnew[k + 1];
    double dp5 = pnew[k + 1] - pnew[k + 2];
    double th2 = thet[k - 2], th3 = thet[k - 1], th4 = thet[k];
    if (dp2 > dp1 && dp4 > dp5) {
      double goal = .5 * (dp3 + dmin(dp2, dp4));
      if (dp2 > goal && dp4 > goal) {
        double dis3 = dmin(dp2 - goal, goal - dp3) * slak;
        double dis4 = dmin(dp4 - goal, goal - dp3) * slak;
        if (th3 > th2 && th4 > th3) {
          double ratio = (th4 - th3) / (th3 - th2);
          if (ratio > 1.) dis4 = dis3 / ratio;
          else dis3 = dis4 * ratio;
        }
        pnew[k - 1] = pnew[k - 1] + dis3;
        pnew[k] = pnew[k] - dis4;
      }
    }
  }
  for (int k = 0; k <= kk; k++) pres[k] = pnew[k];
}

/* hybgen.F90:893-1007 */
static void inflate(const orc_ctx *c, double psurf, double *exner) {
  const int L = c->nvl;
  const double thin = RD / P1000;
  double dpsum = 0.;
  const double extop = CP * pow(c->ptop / P1000, RD / CP);
  const double top = .2;
  const double shrink = dmin(1., (psurf / P1000 - top) / (1. - top));
  int last = 1;
#define DP2DEX(a) (RD * (a) / P1000)
#define CUSHN(a, b) (.25 * (dmin((a), 2. * (b)) * dmin((a), 2. * (b))) / (b) + dmax((a), 2. * (b)) - (b))
  for (int k = 1; k <= L - 1; k++) {
    double dp0 = DP2DEX(c->dpsig[k - 1]) * shrink;
    dpsum = dpsum + dp0;
    double exold = exner[k];
    if (k <= c->kbl) {
      double dp1 = dp0;
      last = k + 1;
      exner[k] = exner[k - 1] - dp1;
    } else {
      if (k > last) {
        dp0 = dp0 / dmin(10., 1.25 * ldexp(1.0, k - last));
        dp0 = dmax(dp0, DP2DEX(100.));
      }
      double dp1 = CUSHN(dmax(0., exner[k - 1] - dmin(exold, exner[0] - dpsum)), dp0);
      if (exner[k - 1] - dp1 < exold - thin) {
        if (k == last) last = k + 1;
        exner[k] = dmax(extop, exner[k - 1] - dp1);
      }
    }
  }
  if (c->thktop > 0.) {
    for (int k = L; k >= 2; k--) {
      double q = exner[k - 1] / CP;
      q = q * q * sqrt(q);
      double dk = .25 * (double)(L - k);
      double dp0 = DP2DEX(c->thktop) * (1. / (1. + dk * dk)) / q;
      double exold = exner[k - 1];
      double dp1 = CUSHN(dmax(0., exold - exner[k]), dp0);
      if (exner[k] + dp1 > exold + thin) exner[k - 1] = exner[k] + dp1;
      if (exner[k - 1] < exner[k - 2] - dp0) break;
    }
  }
#undef DP2DEX
#undef CUSHN
}

/* hybgen.F90:207-512 (hybrid-isentropic branch) */
static void regrid_1d(const orc_ctx *c, int its, const double *targt, double *thcol,
                      double *excol, const double *prcol, long *flags) {
  const int L = c->nvl;
  const double thin = RD / P1000, tolrnce = 0.001, dffudt = .1;
  const double eqlb_slak = .1 * (double)its / (10. + (double)its);
  double exwrk[1025], exnew[1025], thnew[1024], heatfx[1024];
  for (int k = 0; k < L; k++)
    if (excol[k] < excol[k + 1] - thin) excol[k + 1] = excol[k];
  for (int k = L - 2; k >= 0; k--) thcol[k] = dmin(thcol[k], thcol[k + 1]);
  for (int k = 0; k <= L; k++) exwrk[k] = excol[k];
  const double tt = targt[L - 1];
  for (int k = L; k >= 2; k--) { /* Fortran k */
    if (thcol[k - 1] <= tt + tolrnce) break;
    double wgt1 = dmax(0., exwrk[k - 2] - exwrk[k - 1]);
    double wgt2 = dmax(thin, exwrk[k - 1] - exwrk[k]);
    double try_ = (thcol[k - 2] * wgt1 + thcol[k - 1] * wgt2) / (wgt1 + wgt2);
    if (try_ > tt - tolrnce) {
      exwrk[k - 1] = exwrk[L];
      for (int k1 = k - 1; k1 <= L; k1++) thcol[k1 - 1] = try_;
    } else {
      exwrk[k - 1] = dmin(exwrk[k - 2], dmax(exwrk[k], (exwrk[k - 1] * (thcol[k - 1] - thcol[k - 2]) +
                                                         exwrk[k] * (tt - thcol[k - 1])) /
                                                            (tt - thcol[k - 2])));
      for (int k1 = k; k1 <= L; k1++) thcol[k1 - 1] = tt;
      break;
    }
  }
  restp_1d(thcol, exwrk, L, thnew, exnew, targt, L, flags);
  heatfx[L - 1] = 0.;
  heatfx[0] = 0.;
  for (int iter = 1; iter <= 3; iter++) {
    for (int k = 0; k <= L; k++) exwrk[k] = exnew[k];
    for (int k = 2; k <= L - 1; k++) { /* Fortran k */
      heatfx[k - 1] = 0.;
      if (exwrk[k - 1] < exwrk[0] - .01 && exwrk[k] > exwrk[L] + .01) {
        double cnv = GRVITY / targt[k - 1];
        heatfx[k - 1] = dffudt * cnv * cnv * .5 * (targt[k] - targt[k - 2]) / dmax(.03 * cnv, exwrk[k - 1] - exwrk[k]);
      }
    }
    for (int k = 1; k <= L - 1; k++) {
      if (exwrk[k] < exwrk[0] - .01 && exwrk[k] > exwrk[L] + .01)
        exnew[k] = dmax(exwrk[k + 1], dmin(exwrk[k - 1], exwrk[k] + (heatfx[k] - heatfx[k - 1]) / (targt[k] - targt[k - 1])));
    }
    int event = 0;
    for (int k = 2; k <= L + 1; k++)
      if (exnew[k - 1] > exnew[k - 2] + thin) event = 1;
    if (!event) break;
  }
  equilb(thnew, exnew, L, eqlb_slak);
  inflate(c, prcol[0], exnew);
  for (int k = 0; k <= L; k++) excol[k] = exnew[k];
}

/* hybgen.F90:1010-1279; returns 1 when the column-integral check fails */
static int pcwise(int kk, const double *xold, const double *yold, const double *xnew, double *ynew,
                  int miglim, int remap_optn) {
  double zold[1025], znew[1025], delz[1025], fco[1024], fcn[1024], vertfx[1025], vertdv[1024];
  double fldnew[1024], a[1024], b[1024], cc[1024];
  const double athird = 1. / 3., small = 1.e-22, acurcy = 1.e-11;
  if (xold[0] < xold[kk]) {
    for (int k = 0; k <= kk; k++) { zold[k] = xold[k]; znew[k] = xnew[k]; }
  } else {
    for (int k = 0; k <= kk; k++) { zold[k] = -xold[k]; znew[k] = -xnew[k]; }
  }
  for (int k = 0; k <= kk; k++) delz[k] = znew[k] - zold[k];
  for (int k = 0; k < kk; k++) {
    fco[k] = dmax(0., zold[k + 1] - zold[k]);
    fcn[k] = dmax(0., znew[k + 1] - znew[k]);
  }
  double bfore = 0., colscl = 0.;
  for (int k = 0; k < kk; k++) {
    bfore = bfore + yold[k] * fco[k];
    colscl = colscl + fabs(yold[k] * fco[k]);
  }
  for (int k = 0; k < kk; k++) fldnew[k] = yold[k];
  for (int k = kk - 2; k >= 0; k--) fldnew[k] = (fldnew[k] * fco[k] + fldnew[k + 1] * small) / (fco[k] + small);
  for (int k = 1; k < kk; k++) fldnew[k] = (fldnew[k] * fco[k] + fldnew[k - 1] * small) / (fco[k] + small);
  a[0] = fldnew[0]; b[0] = 0.; cc[0] = 0.;
  a[kk - 1] = fldnew[kk - 1]; b[kk - 1] = 0.; cc[kk - 1] = 0.;
  for (int k = 1; k < kk - 1; k++) {
    if (remap_optn == 1) {
      a[k] = fldnew[k]; b[k] = 0.; cc[k] = 0.;
    } else if (remap_optn == 2) {
      a[k] = fldnew[k];
      b[k] = 0.;
      if (fldnew[k] <= dmin(fldnew[k - 1], fldnew[k + 1]) || fldnew[k] >= dmax(fldnew[k - 1], fldnew[k + 1])) {
        b[k] = 0.;
      } else if ((fldnew[k + 1] - fldnew[k - 1]) * (fldnew[k - 1] + fldnew[k + 1] - 2. * fldnew[k]) > 0.) {
        b[k] = fldnew[k] - fldnew[k - 1];
      } else {
        b[k] = fldnew[k + 1] - fldnew[k];
      }
      cc[k] = 0.;
    } else {
      double yl = (dmax(small, fco[k - 1]) * fldnew[k] + dmax(small, fco[k]) * fldnew[k - 1]) /
                  (dmax(small, fco[k - 1]) + dmax(small, fco[k]));
      double yr = (dmax(small, fco[k + 1]) * fldnew[k] + dmax(small, fco[k]) * fldnew[k + 1]) /
                  (dmax(small, fco[k + 1]) + dmax(small, fco[k]));
      a[k] = 1.5 * fldnew[k] - .25 * (yl + yr);
      b[k] = yr - yl;
      cc[k] = 6. * (.5 * (yl + yr) - fldnew[k]);
      if (fabs(yr - yl) < 6. * fabs(.5 * (yl + yr) - fldnew[k])) {
        if (fabs(yr - yl) > 2. * fabs(.5 * (yl + yr) - fldnew[k])) {
          if ((yr - yl) * (.5 * (yl + yr) - fldnew[k]) > 0.) {
            a[k] = .25 * (3. * fldnew[k] + yl);
            cc[k] = 3. * (fldnew[k] - yl);
            b[k] = cc[k];
          } else {
            a[k] = .25 * (3. * fldnew[k] + yr);
            cc[k] = 3. * (fldnew[k] - yr);
            b[k] = -cc[k];
          }
        } else {
          a[k] = fldnew[k]; b[k] = 0.; cc[k] = 0.;
        }
      }
    }
  }
  for (int k = 1; k < kk; k++) { /* interfaces 2..kk (Fortran) */
    double slab = 0., amount = 0.;
    vertfx[k] = 0.;
    if (miglim == 1) {
      if (delz[k] > 0.) {
        int lyr = k;
        if (fco[lyr] > 0.) {
          double dslab = dmin(slab + fco[lyr], delz[k]) - dmin(slab, delz[k]);
          double dx = dslab / fco[lyr];
          double fcdx = a[lyr] + b[lyr] * .5 * (dx - 1.) + cc[lyr] * (.25 - dx * (.5 - dx * athird));
          amount = amount + fcdx * dslab;
          slab = slab + dslab;
        }
      } else if (delz[k] < 0.) {
        int lyr = k - 1;
        if (fco[lyr] > 0.) {
          double dslab = dmin(slab + fco[lyr], -delz[k]) - dmin(slab, -delz[k]);
          double dx = dslab / fco[lyr];
          double fcdx = a[lyr] + b[lyr] * .5 * (1. - dx) + cc[lyr] * (.25 - dx * (.5 - dx * athird));
          amount = amount + fcdx * dslab;
          slab = slab + dslab;
        }
      }
    } else {
      if (delz[k] > 0.) {
        int lyr = k - 1;
        for (;;) {
          lyr = lyr + 1;
          if (slab >= delz[k]) break;
          if (fco[lyr] > 0.) {
            double dslab = dmin(slab + fco[lyr], delz[k]) - dmin(slab, delz[k]);
            double dx = dslab / fco[lyr];
            double fcdx = a[lyr] + b[lyr] * .5 * (dx - 1.) + cc[lyr] * (.25 - dx * (.5 - dx * athird));
            amount = amount + fcdx * dslab;
            slab = slab + dslab;
          }
          if (!(lyr < kk - 1)) break;
        }
      } else if (delz[k] < 0.) {
        int lyr = k;
        for (;;) {
          lyr = lyr - 1;
          if (slab >= -delz[k]) break;
          if (fco[lyr] > 0.) {
            double dslab = dmin(slab + fco[lyr], -delz[k]) - dmin(slab, -delz[k]);
            double dx = dslab / fco[lyr];
            double fcdx = a[lyr] + b[lyr] * .5 * (1. - dx) + cc[lyr] * (.25 - dx * (.5 - dx * athird));
            amount = amount + fcdx * dslab;
            slab = slab + dslab;
          }
          if (!(lyr > 0)) break;
        }
      }
    }
    if (slab != 0.) vertfx[k] = -delz[k] * amount / slab;
  }
  vertfx[0] = 0.;
  vertfx[kk] = 0.;
  for (int k = 0; k < kk; k++) vertdv[k] = vertfx[k + 1] - vertfx[k];
  double after = 0.;
  for (int k = 0; k < kk; k++) {
    double amount = fldnew[k] * fco[k] - vertdv[k];
    fldnew[k] = (amount + fldnew[k] * small) / (fcn[k] + small);
    after = after + amount;
  }
  for (int k = 0; k < kk; k++) ynew[k] = fldnew[k];
  return fabs(bfore - after) > dmax(1.e-33, acurcy * colscl);
}

/* hybgen.F90:515-789 */
static void remap_1d(const orc_ctx *c, int its, const double *targt, int ntra, double *trcol /* [ntra][L] */,
                     double *ucol, double *vcol, const double *exold, double *excol, double *dpcol,
                     double *prcol, long *flags) {
  const int L = c->nvl;
  const double small = 1.e-6, acurcy = 2.e-6;
  double pk1col[1025], pk1new[1025], exnew[1025], prnew[1025], unew[1024], vnew[1024];
  double *trnew = (double *)malloc(sizeof(double) * (size_t)ntra * L);
  for (int k = 0; k <= L; k++) pk1col[k] = exold[k] * prcol[k] / CP;
  for (int k = 0; k <= L; k++) exnew[k] = excol[k];
  if (c->intfc_smooth > 0.) inflate(c, prcol[0], exnew);
  if (its > 0)
    for (int k = 0; k <= L; k++) exnew[k] = c->slak * exnew[k] + (1. - c->slak) * exold[k];
  const int mg = c->miglim;
  if (mg > 0) {
    for (int k = 1 + mg; k <= L + 1 - mg; k++) /* Fortran k */
      exnew[k - 1] = dmax(.0001 * exold[k - 1] + .9999 * exold[k - 1 + mg],
                          dmin(.0001 * exold[k - 1] + .9999 * exold[k - 1 - mg], exnew[k - 1]));
    for (int k = 2; k <= mg; k++) {
      exnew[k - 1] = dmin(exold[0], exnew[k - 1]);
      exnew[L + 1 - k - 1] = dmax(exold[L], exnew[L + 1 - k - 1]);
    }
  }
  for (int k = L; k >= 0; k--) prnew[k] = P1000 * pow(exnew[k] / CP, CP / RD);
  for (int k = 0; k < L; k++) dpcol[k] = prnew[k] - prnew[k + 1];
  for (int k = 0; k <= L; k++) pk1new[k] = exnew[k] * prnew[k] / CP;
  prnew[L] = prcol[L];
  pk1new[L] = pk1col[L];
  prnew[0] = prcol[0];
  pk1new[0] = pk1col[0];
  *flags += pcwise(L, prcol, ucol, prnew, unew, mg, c->remap_optn);
  *flags += pcwise(L, prcol, vcol, prnew, vnew, mg, c->remap_optn);
  for (int n = 1; n < ntra; n++)
    *flags += pcwise(L, prcol, trcol + (size_t)n * L, prnew, trnew + (size_t)n * L, mg, c->remap_optn);
  *flags += pcwise(L, pk1col, trcol, pk1new, trnew, mg, c->remap_optn);
  for (int k = L; k >= 3; k--) { /* Fortran k */
    double dplo = dmax(pk1new[k - 2] - pk1new[k - 1], pk1new[0] * small);
    double dpup = dmax(pk1new[k - 1] - pk1new[k], pk1new[0] * small);
    double tha = trnew[k - 2], thb = trnew[k - 1];
    double devilo = (tha - targt[k - 2]) * dplo;
    double deviup = (thb - targt[k - 1]) * dpup;
    if (deviup > 0. && devilo < 0.) {
      trnew[k - 2] = tha + dmin(deviup, -devilo) / dplo;
      trnew[k - 1] = thb - dmin(deviup, -devilo) / dpup;
    } else if (deviup < 0. && devilo > 0.) {
      trnew[k - 2] = tha - dmin(devilo, -deviup) / dplo;
      trnew[k - 1] = thb + dmin(devilo, -deviup) / dpup;
    }
  }
  if (c->thktop == 0.) {
    for (int k = 3; k <= L; k++) {
      double qq = 1. / (dpcol[k - 1] + small);
      ucol[k - 1] = (ucol[k - 1] * dpcol[k - 1] + ucol[k - 2] * small) * qq;
      vcol[k - 1] = (vcol[k - 1] * dpcol[k - 1] + vcol[k - 2] * small) * qq;
      for (int n = 1; n < ntra; n++)
        trnew[n * L + k - 1] = (trnew[n * L + k - 1] * dpcol[k - 1] + trnew[n * L + k - 2] * small) * qq;
    }
  }
  double colin = 0., clout = 0., colscl = 0.;
  for (int k = 0; k < L; k++) {
    colin = colin + trcol[k] * (pk1col[k] - pk1col[k + 1]);
    clout = clout + trnew[k] * (pk1new[k] - pk1new[k + 1]);
    colscl = colscl + fabs(trcol[k] * (pk1col[k] - pk1col[k + 1]));
  }
  if (fabs(clout - colin) > dmax(1.e-33, acurcy * colscl)) (*flags)++;
  for (int k = 0; k < L; k++) { ucol[k] = unew[k]; vcol[k] = vnew[k]; }
  for (size_t q = 0; q < (size_t)ntra * L; q++) trcol[q] = trnew[q];
  for (int k = 0; k <= L; k++) { excol[k] = exnew[k]; prcol[k] = prnew[k]; }
  for (int k = 0; k < L; k++)
    if (excol[k] < excol[k + 1]) excol[k + 1] = excol[k];
  free(trnew);
}

/* hybgen.F90:20-201 with dffusn_lev (dffusn.F90:37-58, dffusn_lev.exe) */
void orc_hybgen(orc_ctx *c, int its, const double *targt_in, double *us3d, double *vs3d,
                double *tr3d, double *sdot, double *ex3d, double *dp3d, double *pr3d) {
  const int N = c->nip, L = c->nvl, L1 = c->nvl + 1, T = c->ntra;
  const double *targt = targt_in ? targt_in : c->thetac;
  double *exsmo = (double *)malloc(sizeof(double) * (size_t)N * L1);
  long flags = 0;
#pragma omp parallel reduction(+ : flags)
  {
    double thcol[1024];
#pragma omp for schedule(static)
    for (int ipn = 0; ipn < N; ipn++) {
      for (int k = 0; k < L; k++) thcol[k] = tr3d[T3(k, ipn, 0)];
      for (int k = 0; k < L1; k++) exsmo[(size_t)ipn * L1 + k] = ex3d[(size_t)ipn * L1 + k];
      regrid_1d(c, its, targt, thcol, exsmo + (size_t)ipn * L1, pr3d + (size_t)ipn * L1, &flags);
    }
  }
  if (c->intfc_smooth > 0.) {
    const int k1 = c->kbl + 2, k2 = L; /* Fortran levels */
    double *flxdv = (double *)calloc((size_t)N * L1, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++)
      for (int edg = 0; edg < c->nprox[ipn]; edg++) {
        const int ipx = c->prox[ipn * 6 + edg];
        for (int k = k1 - 1; k <= k2 - 1; k++)
          flxdv[(size_t)ipn * L1 + k] = flxdv[(size_t)ipn * L1 + k] +
                                        (exsmo[(size_t)ipn * L1 + k] - exsmo[(size_t)ipx * L1 + k]) * c->sideln[ipn * 6 + edg];
      }
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++)
      for (int k = k1 - 1; k <= k2 - 1; k++) {
        double factor = -c->smoo_coeff[k] * c->rarea[ipn];
        exsmo[(size_t)ipn * L1 + k] = exsmo[(size_t)ipn * L1 + k] + flxdv[(size_t)ipn * L1 + k] * factor;
      }
    free(flxdv);
  }
#pragma omp parallel reduction(+ : flags)
  {
    double *trcol = (double *)malloc(sizeof(double) * (size_t)T * L);
#pragma omp for schedule(static)
    for (int ipn = 0; ipn < N; ipn++) {
      for (int t = 0; t < T; t++)
        for (int k = 0; k < L; k++) trcol[(size_t)t * L + k] = tr3d[T3(k, ipn, t)];
      remap_1d(c, its, targt, T, trcol, us3d + (size_t)ipn * L, vs3d + (size_t)ipn * L,
               ex3d + (size_t)ipn * L1, exsmo + (size_t)ipn * L1, dp3d + (size_t)ipn * L,
               pr3d + (size_t)ipn * L1, &flags);
      for (int t = 0; t < T; t++)
        for (int k = 0; k < L; k++) tr3d[T3(k, ipn, t)] = trcol[(size_t)t * L + k];
      for (int k = 0; k < L1; k++) {
        sdot[(size_t)ipn * L1 + k] = exsmo[(size_t)ipn * L1 + k] - ex3d[(size_t)ipn * L1 + k];
        ex3d[(size_t)ipn * L1 + k] = exsmo[(size_t)ipn * L1 + k];
      }
    }
    free(trcol);
  }
  c->diag_flags += flags;
  free(exsmo);
}

/* hystat.F90:53-109 */
void orc_hystat(const orc_ctx *c, int its, double *ph3d, const double *ex3d, double *mp3d,
                const double *dp3d, double *tr3d, double *trdp, double *psrf, double *ptdcy) {
  const int N = c->nip, L = c->nvl, L1 = c->nvl + 1;
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    double work = psrf[ipn];
    double ps = dp3d[C2(L - 1, ipn)];
    for (int k = L - 2; k >= 0; k--) ps = ps + dp3d[C2(k, ipn)];
    psrf[ipn] = ps;
    int ns = its % 2; /* Fortran mod(its,2)+1, 0-based */
    if (its > 0) ptdcy[(size_t)ns * N + ipn] = ps - work;
    const double *ex = ex3d + (size_t)ipn * L1;
    double *ph = ph3d + (size_t)ipn * L1;
    mp3d[C2(0, ipn)] = ex[0] * tr3d[T3(0, ipn, 0)] + ph[0];
    ph[1] = mp3d[C2(0, ipn)] - tr3d[T3(0, ipn, 0)] * ex[1];
    for (int k = 1; k < L; k++) {
      mp3d[C2(k, ipn)] = mp3d[C2(k - 1, ipn)] + ex[k] * (tr3d[T3(k, ipn, 0)] - tr3d[T3(k - 1, ipn, 0)]);
      ph[k + 1] = mp3d[C2(k, ipn)] - tr3d[T3(k, ipn, 0)] * ex[k + 1];
    }
    for (int k = 0; k < L; k++) {
      tr3d[T3(k, ipn, 1)] = dmax(QVMIN, tr3d[T3(k, ipn, 1)]);
      tr3d[T3(k, ipn, 2)] = dmax(QWMIN, tr3d[T3(k, ipn, 2)]);
    }
    for (int t = 0; t < c->ntra; t++)
      for (int k = 0; k < L; k++) trdp[T3(k, ipn, t)] = tr3d[T3(k, ipn, t)] * dp3d[C2(k, ipn)];
  }
}

/* globsum.F90:58-108; sums8 = qmass, qmsqv, qmsqw, qmso3, qmste, qmstr, qmstrn, qmstrc */
void orc_globsum(const orc_ctx *c, const double *dp3d, const double *tr, const double *rn2d,
                 const double *rc2d, const double *pr3d, const double *ex3d,
                 const double *qf2d, double *qtrcr, double *sums8) {
  /* qtrcr covers the class-A and class-B tracers (dyn_run.F90:80) */
  const int N = c->nip, L = c->nvl, L1 = c->nvl + 1, T = c->ntra + c->ntrb;
  double summ = 0., smqv = 0., smqw = 0., smo3 = 0., sumr = 0., sume = 0., sumrc = 0., sumrn = 0.;
  for (int t = 0; t < T; t++) qtrcr[t] = 0.;
  for (int ipn = 0; ipn < N; ipn++) {
    const double a = c->area[ipn];
    for (int k = 0; k < L; k++) {
      summ = summ + a * dp3d[C2(k, ipn)];
      smqv = smqv + a * dp3d[C2(k, ipn)] * tr[T3(k, ipn, 1)];
      smqw = smqw + a * dp3d[C2(k, ipn)] * tr[T3(k, ipn, 2)];
      smo3 = smo3 + a * dp3d[C2(k, ipn)] * tr[T3(k, ipn, 3)];
    }
    double rn = rn2d ? rn2d[ipn] : 0., rc = rc2d ? rc2d[ipn] : 0., qf = qf2d ? qf2d[ipn] : 0.;
    sumr = sumr + a * rn;
    sumrc = sumrc + a * rc;
    sumrn = sumrn + a * (rn - rc);
    double den = pr3d[(size_t)ipn * L1] / ((RD / CP) * ex3d[(size_t)ipn * L1] * tr[T3(0, ipn, 0)]);
    sume = sume + a * den * qf * c->dt / (1.25 * 2.5e6);
    for (int t = 0; t < T; t++)
      for (int k = 0; k < L; k++) qtrcr[t] = qtrcr[t] + a * dp3d[C2(k, ipn)] * tr[T3(k, ipn, t)];
  }
  sums8[0] = summ / GRVITY;
  sums8[1] = smqv / GRVITY;
  sums8[2] = smqw / GRVITY;
  sums8[3] = smo3 / GRVITY;
  sums8[4] = sume;
  sums8[5] = sumr;
  sums8[6] = sumrn;
  sums8[7] = sumrc;
}

/* dyn_init.F90:895-906 */
void orc_prdp_from_ex(const orc_ctx *c, const double *ex3d, double *pr3d, double *dp3d) {
  const int N = c->nip, L = c->nvl, L1 = c->nvl + 1;
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    pr3d[(size_t)ipn * L1] = P1000 * pow(ex3d[(size_t)ipn * L1] / CP, CP / RD);
    for (int k = 0; k < L; k++) {
      pr3d[(size_t)ipn * L1 + k + 1] = P1000 * pow(ex3d[(size_t)ipn * L1 + k + 1] / CP, CP / RD);
      dp3d[C2(k, ipn)] = pr3d[(size_t)ipn * L1 + k] - pr3d[(size_t)ipn * L1 + k + 1];
    }
  }
}

/* ------------------------------------------------------------------------
 * Class-B tracer transport (module_transp3d, transp3d.F90:21-241, with
 * module_fct3d, fct3d.F90:4-482).  Class-B tracers occupy the tracer slots
 * ntra .. ntra+ntrb-1 (0-based) after the class-A ones; cumufx is an edge
 * field, dpinit a cell field.
 * ------------------------------------------------------------------------ */

/* transp0 (transp3d.F90:21-40) */
void orc_transp0(const orc_ctx *c, double *cumufx, const double *dp3d, double *dpinit) {
  const int N = c->nip, L = c->nvl;
  for (size_t q = 0; q < (size_t)N * 6 * L; q++) cumufx[q] = 0.;
  for (size_t q = 0; q < (size_t)N * L; q++) dpinit[q] = dp3d[q];
}

/* transp1 (transp3d.F90:43-79): time integral of the mass fluxes */
void orc_transp1(const orc_ctx *c, double *cumufx, const double *massfx) {
  const int N = c->nip, L = c->nvl;
#pragma omp parallel for schedule(static)
  for (int ico = 0; ico < N; ico++)
    for (int edg = 0; edg < c->nprox[ico]; edg++)
      for (int k = 0; k < L; k++)
        cumufx[E3(k, edg, ico)] = cumufx[E3(k, edg, ico)] + c->ab1 * massfx[MF(k, edg, ico, c->nf)] +
                                  c->ab2 * massfx[MF(k, edg, ico, c->of)] +
                                  c->ab3 * massfx[MF(k, edg, ico, c->vof)];
}

/* fct3d (fct3d.F90:4-482) for tracer slots frst..last (0-based, inclusive):
 * u = time-integrated edge mass fluxes, w = time-integrated vertical mass
 * flux (w(k) > 0: mass from layer k to k+1), thko/thkn = old/new thickness.
 * diagno and recovr are off, as transp2 calls it. */
static void fct3d(const orc_ctx *c, double *fields, int frst, int last, const double *u, const double *w,
                  const double *thko, const double *thkn) {
  const int N = c->nip, L = c->nvl;
  const double athird = 1. / 3., epsil = 1.e-11, onemu = 1.e-6;
  double *fld = malloc(sizeof(double) * N * L), *vertfx = malloc(sizeof(double) * N * L);
  double *vertdv = malloc(sizeof(double) * N * L), *fmx = malloc(sizeof(double) * N * L);
  double *fmn = malloc(sizeof(double) * N * L), *flp = malloc(sizeof(double) * N * L);
  double *fln = malloc(sizeof(double) * N * L), *flx = malloc(sizeof(double) * N * 6 * L);
  double *uan = malloc(sizeof(double) * N * 6 * L);
  for (int n = frst; n <= last; n++) {
    /* vertical flux by summing fld over the upstream slab of thickness w */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
      double *f = fld + (size_t)i * L;
      const double *to = thko + (size_t)i * L;
      for (int k = 0; k < L; k++) f[k] = fields[T3(k, i, n)];
      /* fill massless cells with data from the layer above or below */
      for (int k = L - 2; k >= 0; k--) f[k] = (f[k] * to[k] + f[k + 1] * onemu) / (to[k] + onemu);
      for (int k = 1; k < L; k++) f[k] = (f[k] * to[k] + f[k - 1] * onemu) / (to[k] + onemu);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
      const double *f = fld + (size_t)i * L, *to = thko + (size_t)i * L, *wc = w + (size_t)i * L;
      double *a = malloc(sizeof(double) * L), *b = malloc(sizeof(double) * L), *cc = malloc(sizeof(double) * L);
      a[0] = f[0]; b[0] = 0.; cc[0] = 0.;
      a[L - 1] = f[L - 1]; b[L - 1] = 0.; cc[L - 1] = 0.;
      /* piecewise parabolic fit (fct3d.F90:185-214) */
      for (int k = 1; k < L - 1; k++) {
        const double dxlft = dmax(epsil, to[k - 1]), dxmid = dmax(epsil, to[k]), dxrgt = dmax(epsil, to[k + 1]);
        const double yl = (dxlft * f[k] + dxmid * f[k - 1]) / (dxlft + dxmid);
        const double yr = (dxrgt * f[k] + dxmid * f[k + 1]) / (dxrgt + dxmid);
        a[k] = 1.5 * f[k] - .25 * (yl + yr);
        b[k] = yr - yl;
        cc[k] = 6. * (.5 * (yl + yr) - f[k]);
        if (fabs(yr - yl) < 6. * fabs(.5 * (yl + yr) - f[k])) {
          if (fabs(yr - yl) > 2. * fabs(.5 * (yl + yr) - f[k])) {
            if ((yr - yl) * (.5 * (yl + yr) - f[k]) > 0.) {
              a[k] = .25 * (3. * f[k] + yl);
              cc[k] = 3. * (f[k] - yl);
              b[k] = cc[k];
            } else {
              a[k] = .25 * (3. * f[k] + yr);
              cc[k] = 3. * (f[k] - yr);
              b[k] = -cc[k];
            }
          } else {
            a[k] = f[k];
            b[k] = 0.;
            cc[k] = 0.;
          }
        }
      }
      double *vf = vertfx + (size_t)i * L;
      for (int k = 0; k < L - 1; k++) {
        double slab = onemu, amount = 0.;
        if (wc[k] < 0.) { /* interface moves up */
          amount = slab * f[k + 1];
          int kp = k;
          for (;;) {
            kp++;
            if (slab >= -wc[k]) break;
            if (to[kp] > 0.) {
              const double dslab = dmin(slab + to[kp], -wc[k]) - dmin(slab, -wc[k]);
              const double dx = dslab / to[kp];
              const double fcdx = a[kp] + b[kp] * .5 * (dx - 1.) + cc[kp] * (.25 - dx * (.5 - dx * athird));
              amount = amount + fcdx * dslab;
              slab = slab + dslab;
            }
            if (!(kp < L - 1)) break;
          }
        } else if (wc[k] > 0.) { /* interface moves down */
          amount = slab * f[k];
          int kp = k + 1;
          for (;;) {
            kp--;
            if (slab >= wc[k]) break;
            if (to[kp] > 0.) {
              const double dslab = dmin(slab + to[kp], wc[k]) - dmin(slab, wc[k]);
              const double dx = dslab / to[kp];
              const double fcdx = a[kp] + b[kp] * .5 * (1. - dx) + cc[kp] * (.25 - dx * (.5 - dx * athird));
              amount = amount + fcdx * dslab;
              slab = slab + dslab;
            }
            if (!(kp > 1)) break; /* fct3d.F90:253: the walk stops above layer 1 */
          }
        }
        vf[k] = wc[k] * amount / slab;
      }
      vf[L - 1] = 0.; /* no flux through the top */
      double *vd = vertdv + (size_t)i * L;
      vd[0] = vf[0];
      for (int k = 1; k < L; k++) vd[k] = vf[k] - vf[k - 1];
      free(a); free(b); free(cc);
    }
    /* low-order and antidiffusive fluxes, local bounds (fct3d.F90:281-320) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
      for (int k = 0; k < L; k++) {
        double mx = fld[C2(k, i)], mn = fld[C2(k, i)];
        for (int edg = 0; edg < c->nprox[i]; edg++) {
          const int ix = c->prox[i * 6 + edg], edx = c->proxs[i * 6 + edg];
          const double ue = u[E3(k, edg, i)], ux = u[E3(k, edx, ix)];
          flx[E3(k, edg, i)] = 0.5 * ((ue + fabs(ue)) * fld[C2(k, i)] - (ux + fabs(ux)) * fld[C2(k, ix)]);
          const double q = .5 * (fld[C2(k, i)] + fld[C2(k, ix)]);
          uan[E3(k, edg, i)] = q * ue - flx[E3(k, edg, i)];
          mx = dmax(mx, fld[C2(k, ix)]);
          mn = dmin(mn, fld[C2(k, ix)]);
        }
        if (k < L - 1 && w[C2(k, i)] < 0.) {
          mx = dmax(mx, vertfx[C2(k, i)] / w[C2(k, i)]);
          mn = dmin(mn, vertfx[C2(k, i)] / w[C2(k, i)]);
        }
        if (k > 0 && w[C2(k - 1, i)] > 0.) {
          mx = dmax(mx, vertfx[C2(k - 1, i)] / w[C2(k - 1, i)]);
          mn = dmin(mn, vertfx[C2(k - 1, i)] / w[C2(k - 1, i)]);
        }
        fmx[C2(k, i)] = mx;
        fmn[C2(k, i)] = mn;
      }
    }
    /* low-order update, then the limiter ratios (fct3d.F90:322-355) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
      for (int k = 0; k < L; k++) {
        double hordiv = 0.;
        for (int edg = 0; edg < c->nprox[i]; edg++) hordiv = hordiv + flx[E3(k, edg, i)];
        hordiv = hordiv * c->rarea[i];
        const size_t ck = C2(k, i);
        const double q = fld[ck] * thko[ck] - hordiv - vertdv[ck];
        const double amount = dmax(0., dmax(fmn[ck] * thkn[ck], dmin(q, fmx[ck] * thkn[ck])));
        fld[ck] = (fld[ck] * onemu + amount) / (onemu + thkn[ck]);
      }
      for (int k = 0; k < L; k++) {
        double totin = 0., totou = 0.;
        for (int edg = 0; edg < c->nprox[i]; edg++) {
          totin = totin - dmin(0., uan[E3(k, edg, i)]);
          totou = totou + dmax(0., uan[E3(k, edg, i)]);
        }
        const size_t ck = C2(k, i);
        flp[ck] = (fmx[ck] - fld[ck]) * thkn[ck] / (totin + epsil) * c->rarea[i];
        fln[ck] = (fld[ck] - fmn[ck]) * thkn[ck] / (totou + epsil) * c->rarea[i];
      }
    }
    /* limit the antidiffusive fluxes (fct3d.F90:368-389) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
      for (int k = 0; k < L; k++) {
        double hordiv = 0.;
        for (int edg = 0; edg < c->nprox[i]; edg++) {
          const int ix = c->prox[i * 6 + edg];
          double clip;
          if (uan[E3(k, edg, i)] >= 0.) clip = dmin(1., dmin(fln[C2(k, i)], flp[C2(k, ix)]));
          else clip = dmin(1., dmin(flp[C2(k, i)], fln[C2(k, ix)]));
          hordiv = hordiv + uan[E3(k, edg, i)] * clip;
        }
        hordiv = hordiv * c->rarea[i];
        const size_t ck = C2(k, i);
        const double q = fld[ck] * thkn[ck] - hordiv;
        const double amount = dmax(0., dmax(fmn[ck] * thkn[ck], dmin(q, fmx[ck] * thkn[ck])));
        fields[T3(k, i, n)] = (fld[ck] * onemu + amount) / (onemu + thkn[ck]);
      }
    }
  }
  free(fld); free(vertfx); free(vertdv); free(fmx); free(fmn); free(flp); free(fln); free(flx); free(uan);
}

/* transp2 (transp3d.F90:82-241): the vertical mass flux that closes the
 * time-integrated continuity equation, then fct3d for the class-B tracers */
void orc_transp2(const orc_ctx *c, int ntrb, double *tracr, const double *cumufx, const double *dpinit,
                 const double *dpfinl) {
  const int N = c->nip, L = c->nvl;
  if (ntrb <= 0) return;
  double *w = malloc(sizeof(double) * N * L);
#pragma omp parallel for schedule(static)
  for (int ico = 0; ico < N; ico++) {
    for (int k = 0; k < L; k++) {
      double hordiv = 0.;
      for (int edg = 0; edg < c->nprox[ico]; edg++) hordiv = hordiv + cumufx[E3(k, edg, ico)];
      const double vertdv = (dpinit[C2(k, ico)] - dpfinl[C2(k, ico)]) - hordiv * c->rarea[ico];
      w[C2(k, ico)] = k == 0 ? vertdv : w[C2(k - 1, ico)] + vertdv;
    }
  }
  fct3d(c, tracr, c->ntra, c->ntra + ntrb - 1, cumufx, w, dpinit, dpfinl);
  free(w);
}

/* ---- physics coupling (cpl_run.F90), the dynamics side of phy_run ------
 * GFS arrays are (nip, nvl) with the cell index fastest: g[k*nip + i].
 * old6 holds the six fields cpl_dyn_to_phy keeps for the tendency method
 * (gfs_u_old, gfs_v_old, gfs_t_old, gfs_q_old, gfs_oz_old, gfs_cld_old) in
 * the same layout, one nvl*nip block each. */
#define G2(i, k) ((size_t)(k) * N + (i))

/* cpl_dyn_to_phy, callphy branch (cpl_run.F90:203-260) */
void orc_cpl_dyn_to_phy(const orc_ctx *c, const double *pr3d, const double *us3d, const double *vs3d,
                        const double *ws3d, const double *tr3d, double *gfs_ps, double *gfs_dp,
                        double *gfs_p, double *gfs_u, double *gfs_v, double *gfs_dpdt, double *gfs_q,
                        double *gfs_oz, double *gfs_cld, double *gfs_t, double *old6) {
  const int N = c->nip, L = c->nvl;
  const size_t NL = (size_t)N * L;
  const double rocp1 = RD / CP + 1., rocpr = CP / RD;
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    gfs_ps[ipn] = 0.001 * pr3d[I2(0, ipn)];
    for (int k = 0; k < L; k++) {
      const double pk = pr3d[I2(k, ipn)], pk1 = pr3d[I2(k + 1, ipn)];
      const double q2 = dmax(QVMIN, tr3d[T3(k, ipn, 1)]);
      const size_t g = G2(ipn, k);
      gfs_dp[g] = (0.001 * pk) - (0.001 * pk1);
      gfs_p[g] = pow((pow(pk, rocp1) - pow(pk1, rocp1)) / ((pk - pk1) * rocp1), rocpr);
      gfs_u[g] = us3d[C2(k, ipn)];
      gfs_v[g] = vs3d[C2(k, ipn)];
      gfs_dpdt[g] = 0.001 * ws3d[C2(k, ipn)];
      gfs_q[g] = q2;
      gfs_oz[g] = tr3d[T3(k, ipn, 3)];
      gfs_cld[g] = tr3d[T3(k, ipn, 2)];
      const double theta_nv = tr3d[T3(k, ipn, 0)] / (1. + 0.6078 * dmax(QVMIN, q2));
      gfs_t[g] = theta_nv * pow(gfs_p[g] / P1000, RD / CP);
      old6[0 * NL + g] = gfs_u[g];
      old6[1 * NL + g] = gfs_v[g];
      old6[2 * NL + g] = gfs_t[g];
      old6[3 * NL + g] = gfs_q[g];
      old6[4 * NL + g] = gfs_oz[g];
      old6[5 * NL + g] = gfs_cld[g];
    }
  }
}

/* dffusn8_lyr (dffusn.F90:110-129 with dffusn_lyr.exe) on a (nvl, nip) field */
static void dffusn8_lyr(const orc_ctx *c, double *fld, const double *delp, double dfflen) {
  const int N = c->nip, L = c->nvl;
  const double thshld = 1.e-11;
  double *flxdv = malloc(sizeof(double) * (size_t)N * L);
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    for (int k = 0; k < L; k++) flxdv[C2(k, ipn)] = 0.;
    for (int edg = 0; edg < c->nprox[ipn]; edg++) {
      const int ipx = c->prox[ipn * 6 + edg];
      for (int k = 0; k < L; k++) {
        const double a = dmax(delp[C2(k, ipn)], thshld), b = dmax(delp[C2(k, ipx)], thshld);
        flxdv[C2(k, ipn)] = flxdv[C2(k, ipn)] + (fld[C2(k, ipn)] - fld[C2(k, ipx)]) *
                                                    c->sideln[ipn * 6 + edg] * 2. * (a * b / (a + b));
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++)
    for (int k = 0; k < L; k++) {
      const double factor = -dfflen * c->rarea[ipn] / dmax(delp[C2(k, ipn)], thshld);
      fld[C2(k, ipn)] = fld[C2(k, ipn)] + flxdv[C2(k, ipn)] * factor;
    }
  free(flxdv);
}

/* cpl_phy_to_dyn, callphy branch (cpl_run.F90:407-490): the 3-D state and
 * the precipitation / evaporation columns that globsum reads */
void orc_cpl_phy_to_dyn(const orc_ctx *c, int addtend, int smoothtend, double dtp, const double *gfs_p,
                        const double *gfs_u, const double *gfs_v, const double *gfs_q, const double *gfs_cld,
                        const double *gfs_oz, const double *gfs_t, const double *old6, const double *dp3d,
                        double *us3d, double *vs3d, double *tr3d, const double *geshem, const double *rainc,
                        const double *evap, double *rn2d, double *rc2d, double *qf2d) {
  const int N = c->nip, L = c->nvl;
  const size_t NL = (size_t)N * L;
  const double dt = c->dt, kap = RD / CP;
  double *tdc = NULL; /* u, v, t, q, cld, oz tendencies, (nvl, nip) each */
  if (addtend) {
    tdc = malloc(sizeof(double) * 6 * NL);
    const double *now[6] = {gfs_u, gfs_v, gfs_t, gfs_q, gfs_cld, gfs_oz};
    const int oi[6] = {0, 1, 2, 3, 5, 4};
#pragma omp parallel for schedule(static)
    for (int ipn = 0; ipn < N; ipn++)
      for (int k = 0; k < L; k++)
        for (int f = 0; f < 6; f++)
          tdc[f * NL + C2(k, ipn)] = (now[f][G2(ipn, k)] - old6[oi[f] * NL + G2(ipn, k)]) / dtp;
    if (smoothtend)
      for (int f = 0; f < 6; f++) dffusn8_lyr(c, tdc + f * NL, dp3d, dt * 20.);
  }
#pragma omp parallel for schedule(static)
  for (int ipn = 0; ipn < N; ipn++) {
    for (int k = 0; k < L; k++) {
      const size_t g = G2(ipn, k), d = C2(k, ipn);
      if (addtend) {
        us3d[d] = old6[0 * NL + g] + tdc[0 * NL + d] * dt;
        vs3d[d] = old6[1 * NL + g] + tdc[1 * NL + d] * dt;
        tr3d[T3(k, ipn, 0)] = (old6[2 * NL + g] + tdc[2 * NL + d] * dt) * pow(P1000 / gfs_p[g], kap) *
                              (1. + 0.6078 * dmax(QVMIN, (old6[3 * NL + g] + tdc[3 * NL + d] * dt)));
        tr3d[T3(k, ipn, 1)] = dmax(QVMIN, (old6[3 * NL + g] + tdc[3 * NL + d] * dt));
        tr3d[T3(k, ipn, 2)] = dmax(QWMIN, (old6[5 * NL + g] + tdc[4 * NL + d] * dt));
        tr3d[T3(k, ipn, 3)] = dmax(QVMIN, (old6[4 * NL + g] + tdc[5 * NL + d] * dt));
      } else {
        us3d[d] = gfs_u[g];
        vs3d[d] = gfs_v[g];
        tr3d[T3(k, ipn, 0)] = gfs_t[g] * pow(P1000 / gfs_p[g], kap) * (1. + 0.6078 * dmax(QVMIN, gfs_q[g]));
        tr3d[T3(k, ipn, 1)] = dmax(QVMIN, gfs_q[g]);
        tr3d[T3(k, ipn, 2)] = dmax(QWMIN, gfs_cld[g]);
        tr3d[T3(k, ipn, 3)] = dmax(QVMIN, gfs_oz[g]);
      }
    }
    rn2d[ipn] = rn2d[ipn] + dmax(0., geshem[ipn]) * 1000.;
    rc2d[ipn] = rc2d[ipn] + dmax(0., rainc[ipn]) * 1000.;
    qf2d[ipn] = -evap[ipn];
  }
  free(tdc);
}
#undef G2
