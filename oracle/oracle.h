/*
 * oracle.h -- CPU restatement of ADSeismic's time-stepping hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it.
 * The product library (libadseismic_gb300.so) never links or calls it.
 *
 * Everything is FP64, single-threaded, compiled with -ffp-contract=off so that
 * the per-operation rounding follows the reference's C++ / TensorFlow order.
 * Layout: flat row-major (NX+2)x(NY+2), idx = i*(NY+2)+j, j (depth) contiguous.
 * Source/receiver indices are 1-based into the padded grid, as in the reference.
 */
#ifndef ADS_ORACLE_H
#define ADS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- acoustic ---------------- */

/* One acoustic step, variant 0 ("w": PML auxiliaries from the old field,
 * deps/CustomOps/AcousticOneStepCpu/AcousticOneStepCpu.h:1-48) or variant 1
 * ("u": auxiliaries from the new field, src/Core.jl:528-549). */
void orc_acoustic_step_fwd(const double* w, const double* wold, const double* phi,
                           const double* psi, const double* sigma, const double* tau,
                           const double* c, double dt, double hx, double hy,
                           int64_t NX, int64_t NY, double* u, double* phiout,
                           double* psiout, int variant);

/* Transpose of orc_acoustic_step_fwd.  Outputs are overwritten (zeroed, then
 * accumulated) as TF's setZero + AcousticOneStepCpuBackward do
 * (AcousticOneStepCpu.cpp:363-367, AcousticOneStepCpu.h:51-125). */
void orc_acoustic_step_bwd(double* grad_w, double* grad_wold, double* grad_phi,
                           double* grad_psi, double* grad_c, const double* grad_u,
                           const double* grad_phiout, const double* grad_psiout,
                           const double* w, const double* wold, const double* phi,
                           const double* psi, const double* sigma, const double* tau,
                           const double* c, double dt, double hx, double hy,
                           int64_t NX, int64_t NY, const double* u,
                           const double* phiout, const double* psiout, int variant);

/* PML damping profiles as 2D (NX+2)(NY+2) arrays (src/Core.jl:622-655,738-761).
 * use_pml: bit0 XMIN, bit1 XMAX, bit2 YMIN, bit3 YMAX. */
void orc_acoustic_pml(int64_t NX, int64_t NY, double hx, double hy, int64_t npml,
                      double vp_ref, double Rcoef, int use_pml, double* sigma,
                      double* tau);

/* Acoustic time loop (src/Core.jl:562-620) + receiver gather (Core.jl:726-730).
 * vp: (NX+2)(NY+2); srcv: rows of nsrc values, row r used at slot r+1 (0-based),
 * rows 1..NSTEP-1 are read.  rcvv: (NSTEP+1, nrcv).  u_hist: optional
 * (NSTEP+1)*N history (may be NULL). */
void orc_acoustic_forward(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double hx,
                          double hy, const double* sigma, const double* tau,
                          const double* vp, int64_t nsrc, const int64_t* srci,
                          const int64_t* srcj, const double* srcv, int64_t nrcv,
                          const int64_t* rcvi, const int64_t* rcvj, double* rcvv,
                          double* u_hist, int variant);

/* L2 misfit sum((rcvv-obs)^2) (src/Utils.jl:308) and its gradient w.r.t. vp
 * through c = vp^2, by the discrete adjoint over the full stored history
 * (the order TF's reverse while_loop uses).  Returns the loss. */
double orc_acoustic_gradient(int64_t NX, int64_t NY, int64_t NSTEP, double dt,
                             double hx, double hy, const double* sigma,
                             const double* tau, const double* vp, int64_t nsrc,
                             const int64_t* srci, const int64_t* srcj,
                             const double* srcv, int64_t nrcv, const int64_t* rcvi,
                             const int64_t* rcvj, const double* obs, double* grad_vp,
                             int variant);
/* orc_acoustic_gradient plus grad_srcv (NSTEP, nsrc): d loss / d srcv. */
double orc_acoustic_gradient_src(int64_t NX, int64_t NY, int64_t NSTEP, double dt,
                                 double hx, double hy, const double* sigma,
                                 const double* tau, const double* vp, int64_t nsrc,
                                 const int64_t* srci, const int64_t* srcj,
                                 const double* srcv, int64_t nrcv, const int64_t* rcvi,
                                 const int64_t* rcvj, const double* obs, double* grad_vp,
                                 double* grad_srcv, int variant);

/* ---------------- elastic ---------------- */

/* CPML profiles (src/Core.jl:231-407).  ax,bx,kx: 2*NX (row 0 integer grid,
 * row 1 half grid); ay,by,ky: 2*NY. */
void orc_elastic_cpml(int64_t NX, int64_t NY, double dx, double dy, double dt,
                      int64_t npml, double npower, double k_max, double alpha_max,
                      double vp_ref, double Rcoef, int use_pml, double* ax, double* bx,
                      double* kx, double* ay, double* by, double* ky);

/* State: 13 arrays of N = (NX+2)(NY+2): vx, vy, sxx, syy, sxy, m1..m8, stored
 * contiguously in that order (13*N doubles). */
#define ORC_EL_NFIELD 13

/* One elastic step: fw1..fw4 (src/Core.jl:96-213) then add_source
 * (deps/CustomOps/SourceOps/AddSource.cpp:33-89).  in and out must not alias. */
void orc_elastic_step_fwd(const double* in, double* out, const double* lambda,
                          const double* mu, const double* rho, const double* ax,
                          const double* bx, const double* ay, const double* by,
                          double dt, double dx, double dy, int64_t NX, int64_t NY,
                          int64_t nsrc, const int64_t* srci, const int64_t* srcj,
                          const int64_t* srctype, const double* srcv);

/* Transpose of one elastic step about the input state `in`.  gout: gradient
 * w.r.t. the step's output state; gin: gradient w.r.t. its input state
 * (overwritten); glambda/gmu/grho are accumulated (+=). */
void orc_elastic_step_bwd(const double* in, const double* gout, double* gin,
                          double* glambda, double* gmu, double* grho,
                          const double* lambda, const double* mu, const double* rho,
                          const double* ax, const double* bx, const double* ay,
                          const double* by, double dt, double dx, double dy,
                          int64_t NX, int64_t NY);

/* Elastic time loop (src/Core.jl:31-94) + GetReceive (ReceiveOps/GetReceive.cpp:10-50).
 * srcv: (NSTEP, nsrc), row n-1 (0-based) injected at slot n (n=1..NSTEP).
 * rcvv: (nrcv, NSTEP+1). hist: optional (NSTEP+1)*13*N (may be NULL). */
void orc_elastic_forward(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double dx,
                         double dy, const double* ax, const double* bx, const double* ay,
                         const double* by, const double* lambda, const double* mu,
                         const double* rho, int64_t nsrc, const int64_t* srci,
                         const int64_t* srcj, const int64_t* srctype, const double* srcv,
                         int64_t nrcv, const int64_t* rcvi, const int64_t* rcvj,
                         const int64_t* rcvtype, double* rcvv, double* hist);

/* sum((rcvv-obs)^2) and its gradient w.r.t. lambda, mu, rho (overwritten). */
double orc_elastic_gradient(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double dx,
                            double dy, const double* ax, const double* bx,
                            const double* ay, const double* by, const double* lambda,
                            const double* mu, const double* rho, int64_t nsrc,
                            const int64_t* srci, const int64_t* srcj,
                            const int64_t* srctype, const double* srcv, int64_t nrcv,
                            const int64_t* rcvi, const int64_t* rcvj,
                            const int64_t* rcvtype, const double* obs, double* glambda,
                            double* gmu, double* grho);
/* ... and d loss / d srcv into gsrc ((NSTEP, nsrc), or NULL). */
double orc_elastic_gradient_src(int64_t NX, int64_t NY, int64_t NSTEP, double dt, double dx,
                                double dy, const double* ax, const double* bx,
                                const double* ay, const double* by, const double* lambda,
                                const double* mu, const double* rho, int64_t nsrc,
                                const int64_t* srci, const int64_t* srcj,
                                const int64_t* srctype, const double* srcv, int64_t nrcv,
                                const int64_t* rcvi, const int64_t* rcvj,
                                const int64_t* rcvtype, const double* obs, double* glambda,
                                double* gmu, double* grho, double* gsrc);

/* AddSource forward/backward (AddSource.cpp:33-155), GetReceive forward/backward
 * (GetReceive.cpp:10-96), restated. */
void orc_add_source_fwd(double* out5, const double* in5, int64_t nsrc,
                        const int64_t* srci, const int64_t* srcj, const int64_t* srctype,
                        const double* srcv, int64_t NX, int64_t NY);
void orc_add_source_bwd(double* gin5, double* grad_srcv, const double* gout5,
                        int64_t nsrc, const int64_t* srci, const int64_t* srcj,
                        const int64_t* srctype, int64_t NX, int64_t NY);
/* fields5: five (nt, N) histories in the order vx, vy, sxx, syy, sxy. */
void orc_get_receive_fwd(double* out, const double* const* fields5, int64_t nt,
                         int64_t nrcv, const int64_t* rcvi, const int64_t* rcvj,
                         const int64_t* rcvtype, int64_t NX, int64_t NY);
void orc_get_receive_bwd(double* const* gfields5, const double* gout, int64_t nt,
                         int64_t nrcv, const int64_t* rcvi, const int64_t* rcvj,
                         const int64_t* rcvtype, int64_t NX, int64_t NY);

#ifdef __cplusplus
}
#endif
#endif
