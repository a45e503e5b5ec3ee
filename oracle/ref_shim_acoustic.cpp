/*
 * ref_shim_acoustic.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference's own acoustic CPU operator and index ops (included
 * by include path from the reference checkout; nothing is copied into this
 * repository) and exposes them with C linkage for the oracle tests and the CPU
 * baseline:
 *   deps/CustomOps/AcousticOneStepCpu/AcousticOneStepCpu.h  (step fwd/bwd)
 *   deps/CustomOps/ScatterAddOps/ScatterAddOps.h             (source injection)
 *   deps/CustomOps/GatherOps/GatherOps.h                     (receiver gather)
 * plus a restated time loop (src/Core.jl:562-620) that drives them.
 */
#include <cstdint>
#include <cstring>
#include <vector>
typedef long long int64;
#include "AcousticOneStepCpu.h"
#include "ScatterAddOps.h"
#include "GatherOps.h"

extern "C" {

void ref_acoustic_step_fwd(const double* w, const double* wold, const double* phi,
                           const double* psi, const double* sigma, const double* tau,
                           const double* c, double dt, double hx, double hy, int64_t NX,
                           int64_t NY, double* u, double* phiout, double* psiout) {
  AcousticOneStepCpuForward(w, wold, phi, psi, sigma, tau, c, dt, hx, hy, NX, NY, u,
                            phiout, psiout);
}

/* TF zeroes the gradient outputs before the op accumulates
 * (AcousticOneStepCpu.cpp:363-367). */
void ref_acoustic_step_bwd(double* grad_w, double* grad_wold, double* grad_phi,
                           double* grad_psi, double* grad_c, const double* grad_u,
                           const double* grad_phiout, const double* grad_psiout,
                           const double* w, const double* wold, const double* phi,
                           const double* psi, const double* sigma, const double* tau,
                           const double* c, double dt, double hx, double hy, int64_t NX,
                           int64_t NY, const double* u, const double* phiout,
                           const double* psiout) {
  const size_t n = (size_t)((NX + 2) * (NY + 2));
  std::memset(grad_w, 0, n * sizeof(double));
  std::memset(grad_wold, 0, n * sizeof(double));
  std::memset(grad_phi, 0, n * sizeof(double));
  std::memset(grad_psi, 0, n * sizeof(double));
  std::memset(grad_c, 0, n * sizeof(double));
  AcousticOneStepCpuBackward(grad_w, grad_wold, grad_phi, grad_psi, grad_c, grad_u,
                             grad_phiout, grad_psiout, w, wold, phi, psi, sigma, tau, c,
                             dt, hx, hy, NX, NY, u, phiout, psiout);
}

void ref_scatter_add_fwd(double* out, const double* ipt, const int64_t* ii,
                         const double* update, int64_t d, int64_t n) {
  ScatterAddOps_forward(out, ipt, (const int64*)ii, update, (int)d, (int)n);
}

void ref_gather_fwd(double* out, const double* v, const int64_t* ii, int64_t n) {
  GatherOps_forward(out, v, (const int64*)ii, (int)n);
}

/* Restated loop of src/Core.jl:562-620 driving the reference operators:
 * slot k = AcousticOneStepCpuForward(slot k-1, slot k-2), then
 * ScatterAddOps_forward(u, (srci-1)(NY+2)+srcj, srcv[k-1]*dt^2); receivers
 * gathered per slot (Core.jl:726-730).  rcvv: (NSTEP+1, nrcv). */
void ref_acoustic_forward(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double hx,
                          double hy, const double* sigma, const double* tau,
                          const double* vp, int64_t nsrc, const int64_t* srci,
                          const int64_t* srcj, const double* srcv, int64_t nrcv,
                          const int64_t* rcvi, const int64_t* rcvj, double* rcvv) {
  const int64_t N = (NX + 2) * (NY + 2);
  std::vector<double> c(N), U0(N, 0.0), U1(N, 0.0), U2(N), P0(N, 0.0), P1(N),
      Q0(N, 0.0), Q1(N), tmp(N), upd(nsrc);
  for (int64_t k = 0; k < N; k++) c[k] = vp[k] * vp[k];
  std::vector<int64_t> sidx(nsrc), ridx(nrcv);
  for (int64_t s = 0; s < nsrc; s++) sidx[s] = (srci[s] - 1) * (NY + 2) + srcj[s];
  for (int64_t r = 0; r < nrcv; r++) ridx[r] = (rcvi[r] - 1) * (NY + 2) + rcvj[r];
  for (int64_t r = 0; r < 2 * nrcv; r++) rcvv[r] = 0.0;
  const double dt2 = dt * dt;
  double *um2 = U0.data(), *um1 = U1.data(), *un = U2.data();
  double *p0 = P0.data(), *p1 = P1.data(), *q0 = Q0.data(), *q1 = Q1.data();
  for (int64_t k = 2; k <= NSTEP; k++) {
    AcousticOneStepCpuForward(um1, um2, p0, q0, sigma, tau, c.data(), dt, hx, hy, NX, NY,
                              tmp.data(), p1, q1);
    for (int64_t s = 0; s < nsrc; s++) upd[s] = srcv[(k - 1) * nsrc + s] * dt2;
    ScatterAddOps_forward(un, tmp.data(), (const int64*)sidx.data(), upd.data(), (int)N,
                          (int)nsrc);
    GatherOps_forward(rcvv + k * nrcv, un, (const int64*)ridx.data(), (int)nrcv);
    double* t = um2; um2 = um1; um1 = un; un = t;
    t = p0; p0 = p1; p1 = t;
    t = q0; q0 = q1; q1 = t;
  }
}

/* Full-history adjoint driving AcousticOneStepCpuBackward per reversed step,
 * as TF's gradient of the while_loop does (src/Utils.jl:312).  Returns the
 * loss sum((rcvv-obs)^2); grad_vp = (grad_c*2)*vp. */
double ref_acoustic_gradient(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double hx,
                             double hy, const double* sigma, const double* tau,
                             const double* vp, int64_t nsrc, const int64_t* srci,
                             const int64_t* srcj, const double* srcv, int64_t nrcv,
                             const int64_t* rcvi, const int64_t* rcvj, const double* obs,
                             double* grad_vp) {
  const int64_t N = (NX + 2) * (NY + 2), T = NSTEP, S = NY + 2;
  std::vector<double> c(N), UH((T + 1) * N, 0.0), PH((T + 1) * N, 0.0),
      QH((T + 1) * N, 0.0), tmp(N), upd(nsrc), rcvv((T + 1) * nrcv, 0.0);
  for (int64_t k = 0; k < N; k++) c[k] = vp[k] * vp[k];
  std::vector<int64_t> sidx(nsrc), ridx(nrcv);
  for (int64_t s = 0; s < nsrc; s++) sidx[s] = (srci[s] - 1) * S + srcj[s];
  for (int64_t r = 0; r < nrcv; r++) ridx[r] = (rcvi[r] - 1) * S + rcvj[r];
  const double dt2 = dt * dt;
  for (int64_t k = 2; k <= T; k++) {
    AcousticOneStepCpuForward(&UH[(k - 1) * N], &UH[(k - 2) * N], &PH[(k - 1) * N],
                              &QH[(k - 1) * N], sigma, tau, c.data(), dt, hx, hy, NX, NY,
                              tmp.data(), &PH[k * N], &QH[k * N]);
    for (int64_t s = 0; s < nsrc; s++) upd[s] = srcv[(k - 1) * nsrc + s] * dt2;
    ScatterAddOps_forward(&UH[k * N], tmp.data(), (const int64*)sidx.data(), upd.data(),
                          (int)N, (int)nsrc);
    GatherOps_forward(&rcvv[k * nrcv], &UH[k * N], (const int64*)ridx.data(), (int)nrcv);
  }
  double loss = 0.0;
  for (int64_t i = 0; i < (T + 1) * nrcv; i++) {
    const double d = rcvv[i] - obs[i];
    loss += d * d;
  }
  std::vector<double> LU((T + 1) * N, 0.0), LP((T + 1) * N, 0.0), LQ((T + 1) * N, 0.0);
  for (int64_t k = 0; k <= T; k++)
    for (int64_t r = 0; r < nrcv; r++)
      LU[k * N + ridx[r] - 1] += 2 * (rcvv[k * nrcv + r] - obs[k * nrcv + r]);
  std::vector<double> gw(N), gwo(N), gp(N), gq(N), gc(N, 0.0), gacc(N, 0.0);
  for (int64_t k = T; k >= 2; k--) {
    std::fill(gw.begin(), gw.end(), 0.0);
    std::fill(gwo.begin(), gwo.end(), 0.0);
    std::fill(gp.begin(), gp.end(), 0.0);
    std::fill(gq.begin(), gq.end(), 0.0);
    std::fill(gc.begin(), gc.end(), 0.0);
    AcousticOneStepCpuBackward(gw.data(), gwo.data(), gp.data(), gq.data(), gc.data(),
                               &LU[k * N], &LP[k * N], &LQ[k * N], &UH[(k - 1) * N],
                               &UH[(k - 2) * N], &PH[(k - 1) * N], &QH[(k - 1) * N], sigma,
                               tau, c.data(), dt, hx, hy, NX, NY, &UH[k * N], &PH[k * N],
                               &QH[k * N]);
    for (int64_t x = 0; x < N; x++) {
      LU[(k - 1) * N + x] += gw[x];
      LU[(k - 2) * N + x] += gwo[x];
      LP[(k - 1) * N + x] += gp[x];
      LQ[(k - 1) * N + x] += gq[x];
      gacc[x] += gc[x];
    }
  }
  for (int64_t x = 0; x < N; x++) grad_vp[x] = gacc[x] * 2 * vp[x];
  return loss;
}

}  // extern "C"
