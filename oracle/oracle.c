/*
 * oracle.c -- CPU restatement of ADSeismic's time-stepping hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs load
 * this library.
 *
 * Each function cites the reference file:line it restates.  Expression order
 * follows the reference so that, compiled with -ffp-contract=off, the acoustic
 * step reproduces the reference's compiled CPU operator bit for bit (pinned by
 * tests/test_oracle.py against oracle/_ref and tests/golden).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define AT(a, i, j) (a)[(int64_t)(i) * (NY + 2) + (j)]

/* ------------------------------------------------------------------ */
/* acoustic one step                                                    */
/* ------------------------------------------------------------------ */

/* deps/CustomOps/AcousticOneStepCpu/AcousticOneStepCpu.h:1-48 (variant 0) and
 * src/Core.jl:528-549 (variant 1, phi/psi from the new u). */
void orc_acoustic_step_fwd(const double* w, const double* wold, const double* phi,
                           const double* psi, const double* sigma, const double* tau,
                           const double* c, double dt, double hx, double hy,
                           int64_t NX, int64_t NY, double* u, double* phiout,
                           double* psiout, int variant) {
  const int64_t S = NY + 2;
  if (variant == 0) {
    for (int64_t i = 0; i < NX + 2; i++) {
      for (int64_t j = 0; j < NY + 2; j++) {
        const int64_t k = i * S + j;
        if (i == 0 || i == NX + 1 || j == 0 || j == NY + 1) {
          u[k] = 0.0;
          phiout[k] = 0.0;
          psiout[k] = 0.0;
          continue;
        }
        const double sg = sigma[k], ta = tau[k], ck = c[k];
        double v = (2 - sg * ta * dt * dt - 2 * dt * dt / hx / hx * ck -
                    2 * dt * dt / hy / hy * ck) * w[k] +
                   ck * (dt / hx) * (dt / hx) * (w[k + S] + w[k - S]) +
                   ck * (dt / hy) * (dt / hy) * (w[k + 1] + w[k - 1]) +
                   (dt * dt / (2.0 * hx)) * (phi[k + S] - phi[k - S]) +
                   (dt * dt / (2.0 * hy)) * (psi[k + 1] - psi[k - 1]) -
                   (1 - (sg + ta) * dt / 2) * wold[k];
        u[k] = v / (1 + (sg + ta) / 2 * dt);
        phiout[k] = (1. - dt * sg) * phi[k] +
                    dt * ck * (ta - sg) / 2.0 / hx * (w[k + S] - w[k - S]);
        psiout[k] = (1. - dt * ta) * psi[k] +
                    dt * ck * (sg - ta) / 2.0 / hy * (w[k + 1] - w[k - 1]);
      }
    }
    return;
  }
  /* variant 1: u first over the whole grid (frame = 0), then phi/psi from u. */
  const double dt2 = dt * dt;
  const double kx = 2 * dt2 / (hx * hx), ky = 2 * dt2 / (hy * hy);
  const double cx = (dt / hx) * (dt / hx), cy = (dt / hy) * (dt / hy);
  const double fx = dt2 / (2 * hx), fy = dt2 / (2 * hy);
  for (int64_t i = 0; i < NX + 2; i++) {
    for (int64_t j = 0; j < NY + 2; j++) {
      const int64_t k = i * S + j;
      if (i == 0 || i == NX + 1 || j == 0 || j == NY + 1) {
        u[k] = 0.0;
        continue;
      }
      const double sg = sigma[k], ta = tau[k], ck = c[k];
      double v = (2 - sg * ta * dt2 - kx * ck - ky * ck) * w[k] +
                 ck * cx * (w[k + S] + w[k - S]) + ck * cy * (w[k + 1] + w[k - 1]) +
                 fx * (phi[k + S] - phi[k - S]) + fy * (psi[k + 1] - psi[k - 1]) -
                 (1 - (sg + ta) * dt / 2) * wold[k];
      u[k] = v / (1 + (sg + ta) / 2 * dt);
    }
  }
  for (int64_t i = 0; i < NX + 2; i++) {
    for (int64_t j = 0; j < NY + 2; j++) {
      const int64_t k = i * S + j;
      if (i == 0 || i == NX + 1 || j == 0 || j == NY + 1) {
        phiout[k] = 0.0;
        psiout[k] = 0.0;
        continue;
      }
      const double sg = sigma[k], ta = tau[k], ck = c[k];
      phiout[k] = (1. - dt * sg) * phi[k] + dt * ck * (ta - sg) / (2 * hx) * (u[k + S] - u[k - S]);
      psiout[k] = (1. - dt * ta) * psi[k] + dt * ck * (sg - ta) / (2 * hy) * (u[k + 1] - u[k - 1]);
    }
  }
}

/* deps/CustomOps/AcousticOneStepCpu/AcousticOneStepCpu.h:51-125 (variant 0);
 * variant 1 is the exact transpose of src/Core.jl:528-549. */
void orc_acoustic_step_bwd(double* grad_w, double* grad_wold, double* grad_phi,
                           double* grad_psi, double* grad_c, const double* grad_u,
                           const double* grad_phiout, const double* grad_psiout,
                           const double* w, const double* wold, const double* phi,
                           const double* psi, const double* sigma, const double* tau,
                           const double* c, double dt, double hx, double hy,
                           int64_t NX, int64_t NY, const double* u,
                           const double* phiout, const double* psiout, int variant) {
  (void)wold; (void)phi; (void)psi; (void)phiout; (void)psiout;
  const int64_t S = NY + 2, N = (NX + 2) * (NY + 2);
  memset(grad_w, 0, sizeof(double) * N);
  memset(grad_wold, 0, sizeof(double) * N);
  memset(grad_phi, 0, sizeof(double) * N);
  memset(grad_psi, 0, sizeof(double) * N);
  memset(grad_c, 0, sizeof(double) * N);
  double* gu_tot = NULL;
  const double* gu = grad_u;
  const double* src_field = w;  /* field the phi/psi updates difference */
  if (variant == 1) {
    /* u feeds phi/psi: total gradient of the (interior) new u first. */
    gu_tot = (double*)calloc((size_t)N, sizeof(double));
    for (int64_t i = 1; i < NX + 1; i++)
      for (int64_t j = 1; j < NY + 1; j++) gu_tot[i * S + j] = grad_u[i * S + j];
    for (int64_t i = 1; i < NX + 1; i++) {
      for (int64_t j = 1; j < NY + 1; j++) {
        const int64_t k = i * S + j;
        const double sg = sigma[k], ta = tau[k], ck = c[k];
        const double gx = dt * ck * (ta - sg) / (2 * hx) * grad_phiout[k];
        const double gy = dt * ck * (sg - ta) / (2 * hy) * grad_psiout[k];
        /* u's frame is a constant zero: no gradient flows there. */
        if (i + 1 <= NX) gu_tot[k + S] += gx;
        if (i - 1 >= 1) gu_tot[k - S] -= gx;
        if (j + 1 <= NY) gu_tot[k + 1] += gy;
        if (j - 1 >= 1) gu_tot[k - 1] -= gy;
      }
    }
    gu = gu_tot;
    src_field = u;
  }
  for (int64_t i = 1; i < NX + 1; i++) {
    for (int64_t j = 1; j < NY + 1; j++) {
      const int64_t k = i * S + j;
      const double sg = sigma[k], ta = tau[k], ck = c[k], g = gu[k];
      const double den = (1 + (sg + ta) / 2 * dt);
      grad_c[k] += ((-2 * dt * dt / hx / hx - 2 * dt * dt / hy / hy) * w[k] +
                    (dt / hx) * (dt / hx) * (w[k + S] + w[k - S]) +
                    (dt / hy) * (dt / hy) * (w[k + 1] + w[k - 1])) * g / den;
      grad_w[k] += (2 - sg * ta * dt * dt - 2 * dt * dt / hx / hx * ck -
                    2 * dt * dt / hy / hy * ck) * g / den;
      grad_w[k + S] += ck * (dt / hx) * (dt / hx) * g / den;
      grad_w[k - S] += ck * (dt / hx) * (dt / hx) * g / den;
      grad_w[k + 1] += ck * (dt / hy) * (dt / hy) * g / den;
      grad_w[k - 1] += ck * (dt / hy) * (dt / hy) * g / den;
      grad_phi[k + S] += (dt * dt / (2.0 * hx)) * g / den;
      grad_phi[k - S] += -(dt * dt / (2.0 * hx)) * g / den;
      grad_psi[k + 1] += (dt * dt / (2.0 * hy)) * g / den;
      grad_psi[k - 1] += -(dt * dt / (2.0 * hy)) * g / den;
      grad_wold[k] += -(1 - (sg + ta) * dt / 2) * g / den;

      const double gp = grad_phiout[k], gs = grad_psiout[k];
      grad_phi[k] += (1. - dt * sg) * gp;
      grad_psi[k] += (1. - dt * ta) * gs;
      if (variant == 0) {
        grad_c[k] += dt * (ta - sg) / 2.0 / hx * (w[k + S] - w[k - S]) * gp;
        grad_w[k + S] += dt * ck * (ta - sg) / 2.0 / hx * gp;
        grad_w[k - S] += -dt * ck * (ta - sg) / 2.0 / hx * gp;
        grad_c[k] += dt * (sg - ta) / 2.0 / hy * (w[k + 1] - w[k - 1]) * gs;
        grad_w[k + 1] += dt * ck * (sg - ta) / 2.0 / hy * gs;
        grad_w[k - 1] += -dt * ck * (sg - ta) / 2.0 / hy * gs;
      } else {
        grad_c[k] += dt * (ta - sg) / (2 * hx) * (src_field[k + S] - src_field[k - S]) * gp;
        grad_c[k] += dt * (sg - ta) / (2 * hy) * (src_field[k + 1] - src_field[k - 1]) * gs;
      }
    }
  }
  free(gu_tot);
}

/* src/Core.jl:738-761 (pml_helper) evaluated over the grid as in Core.jl:622-643. */
void orc_acoustic_pml(int64_t NX, int64_t NY, double hx, double hy, int64_t npml,
                      double vp_ref, double Rcoef, int use_pml, double* sigma,
                      double* tau) {
  const double Lx = npml * hx, Ly = npml * hy;
  const double xi_x = vp_ref / Lx * log(1 / Rcoef);
  const double xi_y = vp_ref / Ly * log(1 / Rcoef);
  const double twopi = 2 * M_PI;
  for (int64_t i = 0; i < NX + 2; i++) {
    const double x = i * hx;
    double ox = 0.0;
    if (x < Lx && (use_pml & 1)) {
      const double d = fabs(Lx - x);
      ox = xi_x * (d / Lx - sin(twopi * d / Lx) / twopi);
    } else if (x > hx * (NX + 1) - Lx && (use_pml & 2)) {
      const double d = fabs(x - (hx * (NX + 1) - Lx));
      ox = xi_x * (d / Lx - sin(twopi * d / Lx) / twopi);
    }
    for (int64_t j = 0; j < NY + 2; j++) {
      const double y = j * hy;
      double oy = 0.0;
      if (y < Ly && (use_pml & 4)) {
        const double d = fabs(Ly - y);
        oy = xi_y * (d / Ly - sin(twopi * d / Ly) / twopi);
      } else if (y > hy * (NY + 1) - Ly && (use_pml & 8)) {
        const double d = fabs(y - (hy * (NY + 1) - Ly));
        oy = xi_y * (d / Ly - sin(twopi * d / Ly) / twopi);
      }
      sigma[i * (NY + 2) + j] = ox;
      tau[i * (NY + 2) + j] = oy;
    }
  }
}

/* src/Core.jl:562-620: slots 0,1 zero; slot k (k>=2) = step(k-1, k-2), then
 * u[src] += srcv[k-1]*dt^2 (ScatterAddOps.h:1-7, Core.jl:600-601).
 * Receivers: rcvv[k, r] = U_k[(rcvi-1)(NY+2) + rcvj-1] (Core.jl:726-730). */
void orc_acoustic_forward(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double hx,
                          double hy, const double* sigma, const double* tau,
                          const double* vp, int64_t nsrc, const int64_t* srci,
                          const int64_t* srcj, const double* srcv, int64_t nrcv,
                          const int64_t* rcvi, const int64_t* rcvj, double* rcvv,
                          double* u_hist, int variant) {
  const int64_t N = (NX + 2) * (NY + 2);
  double* c = (double*)malloc(sizeof(double) * N);
  for (int64_t k = 0; k < N; k++) c[k] = vp[k] * vp[k];
  double* U = (double*)calloc((size_t)(3 * N), sizeof(double));
  double* P = (double*)calloc((size_t)(2 * N), sizeof(double));
  double* Q = (double*)calloc((size_t)(2 * N), sizeof(double));
  double *um2 = U, *um1 = U + N, *un = U + 2 * N;
  double *p0 = P, *p1 = P + N, *q0 = Q, *q1 = Q + N;
  const double dt2 = dt * dt;
  for (int64_t r = 0; r < nrcv; r++) { rcvv[r] = 0.0; rcvv[nrcv + r] = 0.0; }
  if (u_hist) memset(u_hist, 0, sizeof(double) * 2 * N);
  for (int64_t k = 2; k <= NSTEP; k++) {
    orc_acoustic_step_fwd(um1, um2, p0, q0, sigma, tau, c, dt, hx, hy, NX, NY, un, p1,
                          q1, variant);
    const double* row = srcv + (k - 1) * nsrc;
    for (int64_t s = 0; s < nsrc; s++)
      un[(srci[s] - 1) * (NY + 2) + srcj[s] - 1] += row[s] * dt2;
    for (int64_t r = 0; r < nrcv; r++)
      rcvv[k * nrcv + r] = un[(rcvi[r] - 1) * (NY + 2) + rcvj[r] - 1];
    if (u_hist) memcpy(u_hist + k * N, un, sizeof(double) * N);
    double* t = um2; um2 = um1; um1 = un; un = t;
    t = p0; p0 = p1; p1 = t;
    t = q0; q0 = q1; q1 = t;
  }
  free(c); free(U); free(P); free(Q);
}

/* Reverse of orc_acoustic_forward over the full history, the adjoint TF builds
 * for the while_loop of src/Core.jl:614 and the gradients call of
 * src/Utils.jl:312; loss = sum((rcvv - obs)^2) (Utils.jl:308); c = vp^2
 * (Core.jl:564) so grad_vp = (grad_c * 2) * vp. */
static double acoustic_gradient_impl(int64_t NX, int64_t NY, int64_t NSTEP, double dt,
                                     double hx, double hy, const double* sigma,
                                     const double* tau, const double* vp, int64_t nsrc,
                                     const int64_t* srci, const int64_t* srcj,
                                     const double* srcv, int64_t nrcv, const int64_t* rcvi,
                                     const int64_t* rcvj, const double* obs, double* grad_vp,
                                     double* grad_srcv, int variant);

double orc_acoustic_gradient(int64_t NX, int64_t NY, int64_t NSTEP, double dt,
                             double hx, double hy, const double* sigma,
                             const double* tau, const double* vp, int64_t nsrc,
                             const int64_t* srci, const int64_t* srcj,
                             const double* srcv, int64_t nrcv, const int64_t* rcvi,
                             const int64_t* rcvj, const double* obs, double* grad_vp,
                             int variant) {
  return acoustic_gradient_impl(NX, NY, NSTEP, dt, hx, hy, sigma, tau, vp, nsrc, srci, srcj,
                                srcv, nrcv, rcvi, rcvj, obs, grad_vp, NULL, variant);
}

/* The same plus the source-time gradient: the loop adds srcv[t-1] dt^2 to
 * u_t at the source cell (t >= 2), the ScatterAdd of src/Core.jl:600-601, so
 * d loss / d srcv[t-1][s] = dt^2 lambdaU_t[cell s] (ScatterAddOps_backward,
 * ScatterAddOps.h:9-18); row 0 is never injected and stays 0.  grad_srcv:
 * (NSTEP, nsrc). */
double orc_acoustic_gradient_src(int64_t NX, int64_t NY, int64_t NSTEP, double dt,
                                 double hx, double hy, const double* sigma,
                                 const double* tau, const double* vp, int64_t nsrc,
                                 const int64_t* srci, const int64_t* srcj,
                                 const double* srcv, int64_t nrcv, const int64_t* rcvi,
                                 const int64_t* rcvj, const double* obs, double* grad_vp,
                                 double* grad_srcv, int variant) {
  return acoustic_gradient_impl(NX, NY, NSTEP, dt, hx, hy, sigma, tau, vp, nsrc, srci, srcj,
                                srcv, nrcv, rcvi, rcvj, obs, grad_vp, grad_srcv, variant);
}

static double acoustic_gradient_impl(int64_t NX, int64_t NY, int64_t NSTEP, double dt,
                                     double hx, double hy, const double* sigma,
                                     const double* tau, const double* vp, int64_t nsrc,
                                     const int64_t* srci, const int64_t* srcj,
                                     const double* srcv, int64_t nrcv, const int64_t* rcvi,
                                     const int64_t* rcvj, const double* obs, double* grad_vp,
                                     double* grad_srcv, int variant) {
  const int64_t N = (NX + 2) * (NY + 2), T = NSTEP;
  const int64_t S = NY + 2;
  double* c = (double*)malloc(sizeof(double) * N);
  for (int64_t k = 0; k < N; k++) c[k] = vp[k] * vp[k];
  /* full forward history of u, phi, psi */
  double* UH = (double*)calloc((size_t)((T + 1) * N), sizeof(double));
  double* PH = (double*)calloc((size_t)((T + 1) * N), sizeof(double));
  double* QH = (double*)calloc((size_t)((T + 1) * N), sizeof(double));
  double* rcvv = (double*)calloc((size_t)((T + 1) * nrcv), sizeof(double));
  /* variant 1 differences the pre-source u in phi/psi: keep it per slot */
  double* UP = variant == 1 ? (double*)calloc((size_t)((T + 1) * N), sizeof(double)) : NULL;
  const double dt2 = dt * dt;
  for (int64_t k = 2; k <= T; k++) {
    double* un = UH + k * N;
    orc_acoustic_step_fwd(UH + (k - 1) * N, UH + (k - 2) * N, PH + (k - 1) * N,
                          QH + (k - 1) * N, sigma, tau, c, dt, hx, hy, NX, NY, un,
                          PH + k * N, QH + k * N, variant);
    if (UP) memcpy(UP + k * N, un, sizeof(double) * N);
    const double* row = srcv + (k - 1) * nsrc;
    for (int64_t s = 0; s < nsrc; s++) un[(srci[s] - 1) * S + srcj[s] - 1] += row[s] * dt2;
    for (int64_t r = 0; r < nrcv; r++) rcvv[k * nrcv + r] = un[(rcvi[r] - 1) * S + rcvj[r] - 1];
  }
  double loss = 0.0;
  for (int64_t k = 0; k <= T; k++)
    for (int64_t r = 0; r < nrcv; r++) {
      const double d = rcvv[k * nrcv + r] - obs[k * nrcv + r];
      loss += d * d;
    }
  /* adjoint variables for every slot */
  double* LU = (double*)calloc((size_t)((T + 1) * N), sizeof(double));
  double* LP = (double*)calloc((size_t)((T + 1) * N), sizeof(double));
  double* LQ = (double*)calloc((size_t)((T + 1) * N), sizeof(double));
  for (int64_t k = 0; k <= T; k++)
    for (int64_t r = 0; r < nrcv; r++)
      LU[k * N + (rcvi[r] - 1) * S + rcvj[r] - 1] +=
          2 * (rcvv[k * nrcv + r] - obs[k * nrcv + r]);
  double* gw = (double*)malloc(sizeof(double) * N);
  double* gwo = (double*)malloc(sizeof(double) * N);
  double* gp = (double*)malloc(sizeof(double) * N);
  double* gq = (double*)malloc(sizeof(double) * N);
  double* gc = (double*)malloc(sizeof(double) * N);
  double* gcacc = (double*)calloc((size_t)N, sizeof(double));
  for (int64_t k = T; k >= 2; k--) {
    orc_acoustic_step_bwd(gw, gwo, gp, gq, gc, LU + k * N, LP + k * N, LQ + k * N,
                          UH + (k - 1) * N, UH + (k - 2) * N, PH + (k - 1) * N,
                          QH + (k - 1) * N, sigma, tau, c, dt, hx, hy, NX, NY,
                          UP ? UP + k * N : UH + k * N, PH + k * N, QH + k * N, variant);
    for (int64_t x = 0; x < N; x++) {
      LU[(k - 1) * N + x] += gw[x];
      LU[(k - 2) * N + x] += gwo[x];
      LP[(k - 1) * N + x] += gp[x];
      LQ[(k - 1) * N + x] += gq[x];
      gcacc[x] += gc[x];
    }
  }
  for (int64_t x = 0; x < N; x++) grad_vp[x] = gcacc[x] * 2 * vp[x];
  if (grad_srcv) {
    for (int64_t k = 0; k < nsrc; k++) grad_srcv[k] = 0.0;
    for (int64_t t = 2; t <= T; t++)
      for (int64_t s = 0; s < nsrc; s++)
        grad_srcv[(t - 1) * nsrc + s] = dt2 * LU[t * N + (srci[s] - 1) * S + srcj[s] - 1];
  }
  free(c); free(UH); free(PH); free(QH); free(rcvv); free(LU); free(LP); free(LQ);
  free(gw); free(gwo); free(gp); free(gq); free(gc); free(gcacc); free(UP);
  return loss;
}

/* ------------------------------------------------------------------ */
/* elastic                                                              */
/* ------------------------------------------------------------------ */

/* src/Core.jl:231-407 (SEISMIC_CPML profiles). */
void orc_elastic_cpml(int64_t NX, int64_t NY, double dx, double dy, double dt,
                      int64_t npml, double npower, double k_max, double alpha_max,
                      double vp_ref, double Rcoef, int use_pml, double* ax, double* bx,
                      double* kx, double* ay, double* by, double* ky) {
  const double tx = npml * dx, ty = npml * dy;
  const double d0x = -(npower + 1) * vp_ref * log(Rcoef) / (2. * tx);
  const double d0y = -(npower + 1) * vp_ref * log(Rcoef) / (2. * ty);
  for (int pass = 0; pass < 2; pass++) {
    const int64_t n = pass == 0 ? NX : NY;
    const double h = pass == 0 ? dx : dy, th = pass == 0 ? tx : ty;
    const double d0 = pass == 0 ? d0x : d0y;
    const int use_min = pass == 0 ? (use_pml & 1) : (use_pml & 4);
    const int use_max = pass == 0 ? (use_pml & 2) : (use_pml & 8);
    double *A = pass == 0 ? ax : ay, *B = pass == 0 ? bx : by, *K = pass == 0 ? kx : ky;
    const double orig_lo = th, orig_hi = (n - 0.5) * h - th;
    for (int64_t i = 0; i < n; i++) {
      const double val = h * i;
      double d[2] = {0, 0}, kk[2] = {1, 1}, al[2] = {0, 0};
      for (int half = 0; half < 2; half++) {
        const double pos = half ? val + h / 2. : val;
        if (use_min) {
          const double a = orig_lo - pos;
          if (a >= 0.0) {
            const double an = a / th;
            d[half] = d0 * pow(an, npower);
            kk[half] = 1. + (k_max - 1.) * pow(an, npower);
            al[half] = alpha_max * an;
          }
        }
        if (use_max) {
          const double a = pos - orig_hi;
          if (a >= 0) {
            const double an = a / th;
            d[half] = d0 * pow(an, npower);
            kk[half] = 1. + (k_max - 1.) * pow(an, npower);
            al[half] = alpha_max * an;
          }
        }
        if (al[half] < 0) al[half] = 0;
        const double b = exp(-(d[half] / kk[half] + al[half]) * dt);
        double aa = 0.0;
        if (fabs(d[half]) > 1e-6)
          aa = d[half] * (b - 1.) / (kk[half] * (d[half] + kk[half] * al[half]));
        A[half * n + i] = aa;
        B[half * n + i] = b;
        K[half * n + i] = kk[half];
      }
    }
  }
}

/* Fourth-order staggered difference used by every fw* function:
 * (27*a0 - 27*am1 - ap1 + am2) / (24*h), evaluated left to right. */
static inline double d4(double a0, double am1, double ap1, double am2, double h24) {
  return (27 * a0 - 27 * am1 - ap1 + am2) / h24;
}

#define F_VX 0
#define F_VY 1
#define F_SXX 2
#define F_SYY 3
#define F_SXY 4
#define F_M(k) (4 + (k)) /* k = 1..8 */

/* One elastic step: src/Core.jl:215-228 calling fw1 (:96-126), fw2 (:128-155),
 * fw3 (:158-182), fw4 (:186-213) and add_source.  Memory variables are rebuilt
 * with makevector (Core.jl:697-699): zero outside each update box.  The K
 * stretching is dropped, as adbroadcast modes 3/4 return their input
 * (Core.jl:686-693).  Profile indexing (0-based cell I, J):
 *   bx[2,1:end-1] -> half-grid x row at I-1;  bx[1,2:end] -> integer x row at I-1
 *   by[1,2:end]   -> integer y row at J-1;    by[2,1:end-1] -> half-grid y row at J-1 */
void orc_elastic_step_fwd(const double* in, double* out, const double* lambda,
                          const double* mu, const double* rho, const double* ax,
                          const double* bx, const double* ay, const double* by,
                          double dt, double dx, double dy, int64_t NX, int64_t NY,
                          int64_t nsrc, const int64_t* srci, const int64_t* srcj,
                          const int64_t* srctype, const double* srcv) {
  const int64_t N = (NX + 2) * (NY + 2);
  const double* vx = in + F_VX * N; const double* vy = in + F_VY * N;
  const double* sxx = in + F_SXX * N; const double* syy = in + F_SYY * N;
  const double* sxy = in + F_SXY * N;
  double* ovx = out + F_VX * N; double* ovy = out + F_VY * N;
  double* osxx = out + F_SXX * N; double* osyy = out + F_SYY * N;
  double* osxy = out + F_SXY * N;
  /* fields start as copies; memory variables as zeros (makevector) */
  memcpy(out, in, sizeof(double) * 5 * N);
  memset(out + 5 * N, 0, sizeof(double) * 8 * N);
  const double hx24 = 24 * dx, hy24 = 24 * dy;
  const double *axi = ax, *axh = ax + NX, *bxi = bx, *bxh = bx + NX;
  const double *ayi = ay, *ayh = ay + NY, *byi = by, *byh = by + NY;
  /* fw1: I in [1, NX-1], J in [2, NY] */
  for (int64_t I = 1; I <= NX - 1; I++)
    for (int64_t J = 2; J <= NY; J++) {
      const double lam_ = 0.5 * (AT(lambda, I + 1, J) + AT(lambda, I, J));
      const double mu_ = 0.5 * (AT(mu, I + 1, J) + AT(mu, I, J));
      const double lm = lam_ + 2 * mu_;
      double dvx = d4(AT(vx, I + 1, J), AT(vx, I, J), AT(vx, I + 2, J), AT(vx, I - 1, J), hx24);
      double dvy = d4(AT(vy, I, J), AT(vy, I, J - 1), AT(vy, I, J + 1), AT(vy, I, J - 2), hy24);
      const double m1 = bxh[I - 1] * AT(in + F_M(1) * N, I, J) + axh[I - 1] * dvx;
      const double m2 = byi[J - 1] * AT(in + F_M(2) * N, I, J) + ayi[J - 1] * dvy;
      AT(out + F_M(1) * N, I, J) = m1;
      AT(out + F_M(2) * N, I, J) = m2;
      dvx = dvx + m1;
      dvy = dvy + m2;
      AT(osxx, I, J) = AT(sxx, I, J) + (lm * dvx + lam_ * dvy) * dt;
      AT(osyy, I, J) = AT(syy, I, J) + (lm * dvy + lam_ * dvx) * dt;
    }
  /* fw2: I in [2, NX], J in [1, NY-1] */
  for (int64_t I = 2; I <= NX; I++)
    for (int64_t J = 1; J <= NY - 1; J++) {
      const double mu_ = 0.5 * (AT(mu, I, J) + AT(mu, I, J + 1));
      double dvydx = d4(AT(vy, I, J), AT(vy, I - 1, J), AT(vy, I + 1, J), AT(vy, I - 2, J), hx24);
      double dvxdy = d4(AT(vx, I, J + 1), AT(vx, I, J), AT(vx, I, J + 2), AT(vx, I, J - 1), hy24);
      const double m3 = bxi[I - 1] * AT(in + F_M(3) * N, I, J) + axi[I - 1] * dvydx;
      const double m4 = byh[J - 1] * AT(in + F_M(4) * N, I, J) + ayh[J - 1] * dvxdy;
      AT(out + F_M(3) * N, I, J) = m3;
      AT(out + F_M(4) * N, I, J) = m4;
      dvydx = dvydx + m3;
      dvxdy = dvxdy + m4;
      AT(osxy, I, J) = AT(sxy, I, J) + mu_ * (dvydx + dvxdy) * dt;
    }
  /* fw3: I in [2, NX], J in [2, NY]; reads the new sxx, sxy */
  for (int64_t I = 2; I <= NX; I++)
    for (int64_t J = 2; J <= NY; J++) {
      double a = d4(AT(osxx, I, J), AT(osxx, I - 1, J), AT(osxx, I + 1, J), AT(osxx, I - 2, J), hx24);
      double b = d4(AT(osxy, I, J), AT(osxy, I, J - 1), AT(osxy, I, J + 1), AT(osxy, I, J - 2), hy24);
      const double m5 = bxi[I - 1] * AT(in + F_M(5) * N, I, J) + axi[I - 1] * a;
      const double m6 = byi[J - 1] * AT(in + F_M(6) * N, I, J) + ayi[J - 1] * b;
      AT(out + F_M(5) * N, I, J) = m5;
      AT(out + F_M(6) * N, I, J) = m6;
      a = a + m5;
      b = b + m6;
      AT(ovx, I, J) = AT(vx, I, J) + (a + b) * dt / AT(rho, I, J);
    }
  /* fw4: I in [1, NX-1], J in [1, NY-1]; reads the new sxy, syy */
  for (int64_t I = 1; I <= NX - 1; I++)
    for (int64_t J = 1; J <= NY - 1; J++) {
      const double rho_ = 0.25 * (AT(rho, I, J) + AT(rho, I + 1, J) + AT(rho, I + 1, J + 1) +
                                  AT(rho, I, J + 1));
      double a = d4(AT(osxy, I + 1, J), AT(osxy, I, J), AT(osxy, I + 2, J), AT(osxy, I - 1, J), hx24);
      double b = d4(AT(osyy, I, J + 1), AT(osyy, I, J), AT(osyy, I, J + 2), AT(osyy, I, J - 1), hy24);
      const double m7 = bxh[I - 1] * AT(in + F_M(7) * N, I, J) + axh[I - 1] * a;
      const double m8 = byh[J - 1] * AT(in + F_M(8) * N, I, J) + ayh[J - 1] * b;
      AT(out + F_M(7) * N, I, J) = m7;
      AT(out + F_M(8) * N, I, J) = m8;
      a = a + m7;
      b = b + m8;
      AT(ovy, I, J) = AT(vy, I, J) + (a + b) * dt / rho_;
    }
  /* add_source: AddSource.cpp:33-89 (CPU adds) */
  if (nsrc > 0) {
    double* f5[5] = {ovx, ovy, osxx, osyy, osxy};
    for (int64_t s = 0; s < nsrc; s++) {
      const int64_t t = srctype[s];
      if (t < 0 || t > 4) continue;
      AT(f5[t], srci[s] - 1, srcj[s] - 1) += srcv[s];
    }
  }
}

/* Exact transpose of orc_elastic_step_fwd (hand-derived; the reference gets it
 * from TF autodiff of src/Core.jl:96-228).  The forward intermediates (strains,
 * updated memory variables, the new stresses) are recomputed from `in`. */
void orc_elastic_step_bwd(const double* in, const double* gout, double* gin,
                          double* glambda, double* gmu, double* grho,
                          const double* lambda, const double* mu, const double* rho,
                          const double* ax, const double* bx, const double* ay,
                          const double* by, double dt, double dx, double dy,
                          int64_t NX, int64_t NY) {
  const int64_t N = (NX + 2) * (NY + 2);
  /* forward (no source: the source add does not change these intermediates
   * for fw1..fw4; the new stresses fw3/fw4 read are the pre-source values) */
  double* fo = (double*)malloc(sizeof(double) * ORC_EL_NFIELD * N);
  orc_elastic_step_fwd(in, fo, lambda, mu, rho, ax, bx, ay, by, dt, dx, dy, NX, NY, 0,
                       NULL, NULL, NULL, NULL);
  const double* vx = in + F_VX * N; const double* vy = in + F_VY * N;
  const double* nsxx = fo + F_SXX * N; const double* nsyy = fo + F_SYY * N;
  const double* nsxy = fo + F_SXY * N;
  const double hx24 = 24 * dx, hy24 = 24 * dy;
  const double *axi = ax, *axh = ax + NX, *bxi = bx, *bxh = bx + NX;
  const double *ayi = ay, *ayh = ay + NY, *byi = by, *byh = by + NY;
  /* gin starts as the identity part for the 5 fields; memory parts are set
   * inside each box (outside the box the input memory has no effect). */
  memcpy(gin, gout, sizeof(double) * 5 * N);
  memset(gin + 5 * N, 0, sizeof(double) * 8 * N);
  double* gvx = gin + F_VX * N; double* gvy = gin + F_VY * N;
  double* gsxx = gin + F_SXX * N; double* gsyy = gin + F_SYY * N;
  double* gsxy = gin + F_SXY * N;
  /* gradient w.r.t. the intermediate (new, pre-source) stresses: the output
   * gradient plus what fw3/fw4 send back */
  double* gns = (double*)malloc(sizeof(double) * 3 * N);
  double *g_nsxx = gns, *g_nsyy = gns + N, *g_nsxy = gns + 2 * N;
  memcpy(g_nsxx, gout + F_SXX * N, sizeof(double) * N);
  memcpy(g_nsyy, gout + F_SYY * N, sizeof(double) * N);
  memcpy(g_nsxy, gout + F_SXY * N, sizeof(double) * N);
  /* fw4^T */
  for (int64_t I = 1; I <= NX - 1; I++)
    for (int64_t J = 1; J <= NY - 1; J++) {
      const double rho_ = 0.25 * (AT(rho, I, J) + AT(rho, I + 1, J) + AT(rho, I + 1, J + 1) +
                                  AT(rho, I, J + 1));
      const double a = d4(AT(nsxy, I + 1, J), AT(nsxy, I, J), AT(nsxy, I + 2, J), AT(nsxy, I - 1, J), hx24);
      const double b = d4(AT(nsyy, I, J + 1), AT(nsyy, I, J), AT(nsyy, I, J + 2), AT(nsyy, I, J - 1), hy24);
      const double e = (a + AT(fo + F_M(7) * N, I, J)) + (b + AT(fo + F_M(8) * N, I, J));
      const double gv = AT(gout + F_VY * N, I, J);
      const double q = gv * dt / rho_;
      const double gm7 = AT(gout + F_M(7) * N, I, J) + q;
      const double gm8 = AT(gout + F_M(8) * N, I, J) + q;
      const double ga = (q + axh[I - 1] * gm7) / hx24;
      const double gb = (q + ayh[J - 1] * gm8) / hy24;
      AT(gin + F_M(7) * N, I, J) = bxh[I - 1] * gm7;
      AT(gin + F_M(8) * N, I, J) = byh[J - 1] * gm8;
      const double gr = -gv * e * dt / (rho_ * rho_) * 0.25;
      AT(grho, I, J) += gr; AT(grho, I + 1, J) += gr;
      AT(grho, I + 1, J + 1) += gr; AT(grho, I, J + 1) += gr;
      AT(g_nsxy, I + 1, J) += 27 * ga; AT(g_nsxy, I, J) -= 27 * ga;
      AT(g_nsxy, I + 2, J) -= ga; AT(g_nsxy, I - 1, J) += ga;
      AT(g_nsyy, I, J + 1) += 27 * gb; AT(g_nsyy, I, J) -= 27 * gb;
      AT(g_nsyy, I, J + 2) -= gb; AT(g_nsyy, I, J - 1) += gb;
    }
  /* fw3^T */
  for (int64_t I = 2; I <= NX; I++)
    for (int64_t J = 2; J <= NY; J++) {
      const double r = AT(rho, I, J);
      const double a = d4(AT(nsxx, I, J), AT(nsxx, I - 1, J), AT(nsxx, I + 1, J), AT(nsxx, I - 2, J), hx24);
      const double b = d4(AT(nsxy, I, J), AT(nsxy, I, J - 1), AT(nsxy, I, J + 1), AT(nsxy, I, J - 2), hy24);
      const double e = (a + AT(fo + F_M(5) * N, I, J)) + (b + AT(fo + F_M(6) * N, I, J));
      const double gv = AT(gout + F_VX * N, I, J);
      const double q = gv * dt / r;
      const double gm5 = AT(gout + F_M(5) * N, I, J) + q;
      const double gm6 = AT(gout + F_M(6) * N, I, J) + q;
      const double ga = (q + axi[I - 1] * gm5) / hx24;
      const double gb = (q + ayi[J - 1] * gm6) / hy24;
      AT(gin + F_M(5) * N, I, J) = bxi[I - 1] * gm5;
      AT(gin + F_M(6) * N, I, J) = byi[J - 1] * gm6;
      AT(grho, I, J) += -gv * e * dt / (r * r);
      AT(g_nsxx, I, J) += 27 * ga; AT(g_nsxx, I - 1, J) -= 27 * ga;
      AT(g_nsxx, I + 1, J) -= ga; AT(g_nsxx, I - 2, J) += ga;
      AT(g_nsxy, I, J) += 27 * gb; AT(g_nsxy, I, J - 1) -= 27 * gb;
      AT(g_nsxy, I, J + 1) -= gb; AT(g_nsxy, I, J - 2) += gb;
    }
  /* the new stresses equal old + increment inside boxes, old elsewhere:
   * d(new)/d(old) is the identity everywhere */
  memcpy(gsxx, g_nsxx, sizeof(double) * N);
  memcpy(gsyy, g_nsyy, sizeof(double) * N);
  memcpy(gsxy, g_nsxy, sizeof(double) * N);
  /* fw2^T */
  for (int64_t I = 2; I <= NX; I++)
    for (int64_t J = 1; J <= NY - 1; J++) {
      const double mu_ = 0.5 * (AT(mu, I, J) + AT(mu, I, J + 1));
      const double a = d4(AT(vy, I, J), AT(vy, I - 1, J), AT(vy, I + 1, J), AT(vy, I - 2, J), hx24);
      const double b = d4(AT(vx, I, J + 1), AT(vx, I, J), AT(vx, I, J + 2), AT(vx, I, J - 1), hy24);
      const double e = (a + AT(fo + F_M(3) * N, I, J)) + (b + AT(fo + F_M(4) * N, I, J));
      const double gs = AT(g_nsxy, I, J);
      const double q = gs * mu_ * dt;
      const double gm3 = AT(gout + F_M(3) * N, I, J) + q;
      const double gm4 = AT(gout + F_M(4) * N, I, J) + q;
      const double ga = (q + axi[I - 1] * gm3) / hx24;
      const double gb = (q + ayh[J - 1] * gm4) / hy24;
      AT(gin + F_M(3) * N, I, J) = bxi[I - 1] * gm3;
      AT(gin + F_M(4) * N, I, J) = byh[J - 1] * gm4;
      const double gmu_ = gs * e * dt * 0.5;
      AT(gmu, I, J) += gmu_; AT(gmu, I, J + 1) += gmu_;
      AT(gvy, I, J) += 27 * ga; AT(gvy, I - 1, J) -= 27 * ga;
      AT(gvy, I + 1, J) -= ga; AT(gvy, I - 2, J) += ga;
      AT(gvx, I, J + 1) += 27 * gb; AT(gvx, I, J) -= 27 * gb;
      AT(gvx, I, J + 2) -= gb; AT(gvx, I, J - 1) += gb;
    }
  /* fw1^T */
  for (int64_t I = 1; I <= NX - 1; I++)
    for (int64_t J = 2; J <= NY; J++) {
      const double lam_ = 0.5 * (AT(lambda, I + 1, J) + AT(lambda, I, J));
      const double mu_ = 0.5 * (AT(mu, I + 1, J) + AT(mu, I, J));
      const double lm = lam_ + 2 * mu_;
      const double a = d4(AT(vx, I + 1, J), AT(vx, I, J), AT(vx, I + 2, J), AT(vx, I - 1, J), hx24);
      const double b = d4(AT(vy, I, J), AT(vy, I, J - 1), AT(vy, I, J + 1), AT(vy, I, J - 2), hy24);
      const double e1 = a + AT(fo + F_M(1) * N, I, J);
      const double e2 = b + AT(fo + F_M(2) * N, I, J);
      const double gx = AT(g_nsxx, I, J), gy = AT(g_nsyy, I, J);
      const double gE1 = dt * (lm * gx + lam_ * gy);
      const double gE2 = dt * (lam_ * gx + lm * gy);
      const double glm = dt * (e1 * gx + e2 * gy);
      const double glam = dt * (e2 * gx + e1 * gy) + glm;
      const double gmu_ = 2 * glm;
      AT(glambda, I + 1, J) += 0.5 * glam; AT(glambda, I, J) += 0.5 * glam;
      AT(gmu, I + 1, J) += 0.5 * gmu_; AT(gmu, I, J) += 0.5 * gmu_;
      const double gm1 = AT(gout + F_M(1) * N, I, J) + gE1;
      const double gm2 = AT(gout + F_M(2) * N, I, J) + gE2;
      const double ga = (gE1 + axh[I - 1] * gm1) / hx24;
      const double gb = (gE2 + ayi[J - 1] * gm2) / hy24;
      AT(gin + F_M(1) * N, I, J) = bxh[I - 1] * gm1;
      AT(gin + F_M(2) * N, I, J) = byi[J - 1] * gm2;
      AT(gvx, I + 1, J) += 27 * ga; AT(gvx, I, J) -= 27 * ga;
      AT(gvx, I + 2, J) -= ga; AT(gvx, I - 1, J) += ga;
      AT(gvy, I, J) += 27 * gb; AT(gvy, I, J - 1) -= 27 * gb;
      AT(gvy, I, J + 1) -= gb; AT(gvy, I, J - 2) += gb;
    }
  free(fo);
  free(gns);
}

/* src/Core.jl:31-94: slot 0 zeros; slot n = one_step(slot n-1, srcv row n-1),
 * n = 1..NSTEP.  Receivers: GetReceive.cpp:10-50, out[(NSTEP+1)*r + k]. */
void orc_elastic_forward(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double dx,
                         double dy, const double* ax, const double* bx, const double* ay,
                         const double* by, const double* lambda, const double* mu,
                         const double* rho, int64_t nsrc, const int64_t* srci,
                         const int64_t* srcj, const int64_t* srctype, const double* srcv,
                         int64_t nrcv, const int64_t* rcvi, const int64_t* rcvj,
                         const int64_t* rcvtype, double* rcvv, double* hist) {
  const int64_t N = (NX + 2) * (NY + 2), SZ = ORC_EL_NFIELD * N, nt = NSTEP + 1;
  double* a = (double*)calloc((size_t)SZ, sizeof(double));
  double* b = (double*)calloc((size_t)SZ, sizeof(double));
  if (hist) memset(hist, 0, sizeof(double) * SZ);
  for (int64_t r = 0; r < nrcv; r++) rcvv[r * nt] = 0.0;
  for (int64_t n = 1; n <= NSTEP; n++) {
    orc_elastic_step_fwd(a, b, lambda, mu, rho, ax, bx, ay, by, dt, dx, dy, NX, NY, nsrc,
                         srci, srcj, srctype, srcv + (n - 1) * nsrc);
    for (int64_t r = 0; r < nrcv; r++) {
      const int64_t t = rcvtype[r];
      rcvv[r * nt + n] = (t >= 0 && t <= 4)
          ? b[t * N + (rcvi[r] - 1) * (NY + 2) + rcvj[r] - 1] : 0.0;
    }
    if (hist) memcpy(hist + n * SZ, b, sizeof(double) * SZ);
    double* t = a; a = b; b = t;
  }
  free(a); free(b);
}

double orc_elastic_gradient(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double dx,
                            double dy, const double* ax, const double* bx,
                            const double* ay, const double* by, const double* lambda,
                            const double* mu, const double* rho, int64_t nsrc,
                            const int64_t* srci, const int64_t* srcj,
                            const int64_t* srctype, const double* srcv, int64_t nrcv,
                            const int64_t* rcvi, const int64_t* rcvj,
                            const int64_t* rcvtype, const double* obs, double* glambda,
                            double* gmu, double* grho) {
  return orc_elastic_gradient_src(NX, NY, NSTEP, dt, dx, dy, ax, bx, ay, by, lambda, mu, rho,
                                  nsrc, srci, srcj, srctype, srcv, nrcv, rcvi, rcvj, rcvtype,
                                  obs, glambda, gmu, grho, NULL);
}

/* The gradient above plus d loss / d srcv (gsrc: (NSTEP, nsrc), or NULL).
 * srcv row n-1 is added to state n (AddSource.cpp:33-89), so its gradient is
 * the adjoint of state n at the source cell, residual of slot n included
 * (AddSource.cpp:91-155 gathers grad_srcv the same way). */
double orc_elastic_gradient_src(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double dx,
                                double dy, const double* ax, const double* bx,
                                const double* ay, const double* by, const double* lambda,
                                const double* mu, const double* rho, int64_t nsrc,
                                const int64_t* srci, const int64_t* srcj,
                                const int64_t* srctype, const double* srcv, int64_t nrcv,
                                const int64_t* rcvi, const int64_t* rcvj,
                                const int64_t* rcvtype, const double* obs, double* glambda,
                                double* gmu, double* grho, double* gsrc) {
  const int64_t N = (NX + 2) * (NY + 2), SZ = ORC_EL_NFIELD * N, nt = NSTEP + 1;
  double* hist = (double*)malloc(sizeof(double) * (size_t)(nt * SZ));
  double* rcvv = (double*)malloc(sizeof(double) * (size_t)(nrcv * nt));
  orc_elastic_forward(NX, NY, NSTEP, dt, dx, dy, ax, bx, ay, by, lambda, mu, rho, nsrc,
                      srci, srcj, srctype, srcv, nrcv, rcvi, rcvj, rcvtype, rcvv, hist);
  double loss = 0.0;
  for (int64_t r = 0; r < nrcv; r++)
    for (int64_t k = 0; k < nt; k++) {
      const double d = rcvv[r * nt + k] - obs[r * nt + k];
      loss += d * d;
    }
  memset(glambda, 0, sizeof(double) * N);
  memset(gmu, 0, sizeof(double) * N);
  memset(grho, 0, sizeof(double) * N);
  double* g = (double*)calloc((size_t)SZ, sizeof(double));
  double* gp = (double*)malloc(sizeof(double) * SZ);
  for (int64_t n = NSTEP; n >= 1; n--) {
    /* residual of slot n into the gradient of state n (GetReceive.cpp:53-96) */
    for (int64_t r = 0; r < nrcv; r++) {
      const int64_t t = rcvtype[r];
      if (t < 0 || t > 4) continue;
      g[t * N + (rcvi[r] - 1) * (NY + 2) + rcvj[r] - 1] +=
          2 * (rcvv[r * nt + n] - obs[r * nt + n]);
    }
    if (gsrc)
      for (int64_t k = 0; k < nsrc; k++) {
        const int64_t t = srctype[k];
        gsrc[(n - 1) * nsrc + k] =
            (t >= 0 && t <= 4) ? g[t * N + (srci[k] - 1) * (NY + 2) + srcj[k] - 1] : 0.0;
      }
    orc_elastic_step_bwd(hist + (n - 1) * SZ, g, gp, glambda, gmu, grho, lambda, mu, rho,
                         ax, bx, ay, by, dt, dx, dy, NX, NY);
    double* t = g; g = gp; gp = t;
  }
  free(hist); free(rcvv); free(g); free(gp);
  return loss;
}

/* AddSource.cpp:33-89 */
void orc_add_source_fwd(double* out5, const double* in5, int64_t nsrc,
                        const int64_t* srci, const int64_t* srcj, const int64_t* srctype,
                        const double* srcv, int64_t NX, int64_t NY) {
  const int64_t N = (NX + 2) * (NY + 2);
  memcpy(out5, in5, sizeof(double) * 5 * N);
  for (int64_t s = 0; s < nsrc; s++) {
    const int64_t t = srctype[s];
    if (t < 0 || t > 4) continue;
    out5[t * N + (srci[s] - 1) * (NY + 2) + srcj[s] - 1] += srcv[s];
  }
}

/* AddSource.cpp:91-155 */
void orc_add_source_bwd(double* gin5, double* grad_srcv, const double* gout5,
                        int64_t nsrc, const int64_t* srci, const int64_t* srcj,
                        const int64_t* srctype, int64_t NX, int64_t NY) {
  const int64_t N = (NX + 2) * (NY + 2);
  memcpy(gin5, gout5, sizeof(double) * 5 * N);
  for (int64_t s = 0; s < nsrc; s++) {
    const int64_t t = srctype[s];
    if (t < 0 || t > 4) continue; /* reference leaves grad_srcv[s] unwritten */
    grad_srcv[s] = gout5[t * N + (srci[s] - 1) * (NY + 2) + srcj[s] - 1];
  }
}

/* GetReceive.cpp:10-50 */
void orc_get_receive_fwd(double* out, const double* const* fields5, int64_t nt,
                         int64_t nrcv, const int64_t* rcvi, const int64_t* rcvj,
                         const int64_t* rcvtype, int64_t NX, int64_t NY) {
  const int64_t N = (NX + 2) * (NY + 2);
  for (int64_t r = 0; r < nrcv; r++) {
    const int64_t t = rcvtype[r];
    if (t < 0 || t > 4) continue;
    const int64_t idx = (rcvi[r] - 1) * (NY + 2) + rcvj[r] - 1;
    for (int64_t k = 0; k < nt; k++) out[nt * r + k] = fields5[t][k * N + idx];
  }
}

/* GetReceive.cpp:52-96 */
void orc_get_receive_bwd(double* const* gfields5, const double* gout, int64_t nt,
                         int64_t nrcv, const int64_t* rcvi, const int64_t* rcvj,
                         const int64_t* rcvtype, int64_t NX, int64_t NY) {
  const int64_t N = (NX + 2) * (NY + 2);
  for (int f = 0; f < 5; f++) memset(gfields5[f], 0, sizeof(double) * nt * N);
  for (int64_t r = 0; r < nrcv; r++) {
    const int64_t t = rcvtype[r];
    if (t < 0 || t > 4) continue;
    const int64_t idx = (rcvi[r] - 1) * (NY + 2) + rcvj[r] - 1;
    for (int64_t k = 0; k < nt; k++) gfields5[t][k * N + idx] += gout[nt * r + k];
  }
}
