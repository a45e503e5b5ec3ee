/*
 * adseismic_gb300.h -- C ABI of the GB300 (sm_103a) implementation of
 * ADSeismic's time-stepping hot path.
 *
 * Conventions (all entry points):
 *  - Arrays are flat, row-major (NX+2) x (NY+2) grids, idx = i*(NY+2) + j,
 *    j (depth) contiguous -- the layout of the reference's custom operators.
 *    A column-major caller (Julia, Fortran) passes the transpose of its
 *    (NX+2, NY+2) array (Julia: permutedims(A, (2, 1))) and reads an (n, m)
 *    row-major result v as permutedims(reshape(v, m, n), (2, 1)).
 *  - Source / receiver indices are 1-based into the padded grid, as in
 *    ADSeismic (the cell of (srci, srcj) is (srci-1)*(NY+2) + srcj-1).
 *  - Device pointers unless a parameter says "host".  Outputs are owned by the
 *    caller and fully overwritten unless a parameter says "accumulated".
 *  - Every call is asynchronous on `stream` (NULL = legacy default stream);
 *    none synchronises the device unless documented.
 *  - Return value: ADS_OK (0) or an ADS_ERR_* code; ads_last_error() gives a
 *    message for the calling thread.  Invalid shapes and indices are rejected
 *    before any launch (the reference only DCHECKs them).
 *  - There is no CPU fallback: without a usable CUDA device every compute call
 *    returns ADS_ERR_CUDA.
 */
#ifndef ADSEISMIC_GB300_H
#define ADSEISMIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* ads_stream_t; /* same object as cudaStream_t */

enum {
  ADS_OK = 0,
  ADS_ERR_INVALID = 1,     /* bad argument, shape or index */
  ADS_ERR_CUDA = 2,        /* CUDA runtime error (launch, device, copy) */
  ADS_ERR_NOMEM = 3,       /* device allocation failed */
  ADS_ERR_UNSUPPORTED = 4, /* valid request outside what this build implements */
  ADS_ERR_TIMEOUT = 5      /* a bounded wait on the device ran out (the tensor-map copies
                              of the FP32 acoustic interior forward); reported by
                              ads_acoustic_plan_device_status, the results of the calls
                              since then are not valid */
};

enum { ADS_F64 = 0, ADS_F32 = 1 };          /* arithmetic / storage type */
enum { ADS_VARIANT_W = 0, ADS_VARIANT_U = 1 }; /* PML auxiliaries from old w / new u */

/* Thread-local description of the last error raised on the calling thread. */
const char* ads_last_error(void);
/* Library version string. */
const char* ads_version(void);
/* Number of this library's kernels launched by the calling process so far
 * (host-side counter; graph replays count every node they contain). */
int64_t ads_launch_count(void);

/* ======================================================================
 * Single-step operators (drop-ins for the reference's custom operators)
 * ====================================================================== */

/* One acoustic step.  Replaces AcousticOneStepForward
 * (deps/CustomOps/AcousticOneStep/AcousticOneStep.h:9-23; CPU twin
 * AcousticOneStepCpuForward, AcousticOneStepCpu/AcousticOneStepCpu.h:1-48):
 * same arguments in the same order, plus `variant` (ADS_VARIANT_W: phi/psi from
 * the old field w as the custom ops do; ADS_VARIANT_U: from the new u as the
 * default TF step src/Core.jl:528-549 does) and `stream`.  Frame cells of u,
 * phiout, psiout are set to 0.  The f64 form reproduces the reference CPU
 * operator bit for bit for ADS_VARIANT_W.  Outputs must not alias inputs. */
int ads_acoustic_step_fwd_f64(const double* w, const double* wold, const double* phi,
                              const double* psi, const double* sigma, const double* tau,
                              const double* c, double dt, double hx, double hy, int64_t NX,
                              int64_t NY, double* u, double* phiout, double* psiout,
                              int variant, ads_stream_t stream);
int ads_acoustic_step_fwd_f32(const float* w, const float* wold, const float* phi,
                              const float* psi, const float* sigma, const float* tau,
                              const float* c, double dt, double hx, double hy, int64_t NX,
                              int64_t NY, float* u, float* phiout, float* psiout,
                              int variant, ads_stream_t stream);

/* Gradient of one acoustic step.  Replaces AcousticOneStepBackward
 * (AcousticOneStep.h:25-47; CPU twin AcousticOneStepCpu.h:51-125 after TF's
 * setZero, AcousticOneStepCpu.cpp:363-367): same arguments and order, plus
 * `variant` and `stream`.  grad_w, grad_wold, grad_phi, grad_psi, grad_c are
 * overwritten.  The reference op also allocates grad_sigma/grad_tau/grad_dt/
 * grad_hx/grad_hy but never writes them (AcousticOneStep.cpp:310-321); they are
 * not produced here.  The gather form is race-free; results agree with the
 * reference's scatter order to rounding. */
int ads_acoustic_step_bwd_f64(double* grad_w, double* grad_wold, double* grad_phi,
                              double* grad_psi, double* grad_c, const double* grad_u,
                              const double* grad_phiout, const double* grad_psiout,
                              const double* w, const double* wold, const double* phi,
                              const double* psi, const double* sigma, const double* tau,
                              const double* c, double dt, double hx, double hy, int64_t NX,
                              int64_t NY, const double* u, const double* phiout,
                              const double* psiout, int variant, ads_stream_t stream);
int ads_acoustic_step_bwd_f32(float* grad_w, float* grad_wold, float* grad_phi,
                              float* grad_psi, float* grad_c, const float* grad_u,
                              const float* grad_phiout, const float* grad_psiout,
                              const float* w, const float* wold, const float* phi,
                              const float* psi, const float* sigma, const float* tau,
                              const float* c, double dt, double hx, double hy, int64_t NX,
                              int64_t NY, const float* u, const float* phiout,
                              const float* psiout, int variant, ads_stream_t stream);

/* ScatterAddOps forward (deps/CustomOps/ScatterAddOps/ScatterAddOps.h:1-7):
 * out = ipt; out[ii[k]-1] += update[k] for k in order.  ii: device, 1-based,
 * n entries; d = length of ipt/out.  out may equal ipt. */
int ads_scatter_add_f64(double* out, const double* ipt, const int64_t* ii,
                        const double* update, int64_t d, int64_t n, ads_stream_t stream);
/* GatherOps forward (deps/CustomOps/GatherOps/GatherOps.h:1-5):
 * out[k] = v[ii[k]-1], ii device 1-based. */
int ads_gather_f64(double* out, const double* v, const int64_t* ii, int64_t n,
                   ads_stream_t stream);

/* AddSource forward (deps/CustomOps/SourceOps/AddSource.cpp:33-89, CPU
 * semantics: the source is ADDED; the reference GPU kernel assigns instead).
 * Fields in the op's order sigmaxx, sigmayy, sigmaxy, vx, vy; out_* may equal
 * in_* (in place).  srci/srcj/srctype: device int64, nsrc entries; srctype 0 vx,
 * 1 vy, 2 sigmaxx, 3 sigmayy, 4 sigmaxy (others ignored); srcv: device, nsrc. */
int ads_add_source_f64(double* out_sxx, double* out_syy, double* out_sxy, double* out_vx,
                       double* out_vy, const double* sxx, const double* syy,
                       const double* sxy, const double* vx, const double* vy,
                       const int64_t* srci, const int64_t* srcj, const int64_t* srctype,
                       int64_t nsrc, int64_t NX, int64_t NY, const double* srcv,
                       ads_stream_t stream);
/* AddSource backward (AddSource.cpp:91-155): gradients of the five fields are
 * copied through and grad_srcv[k] = g_field(srctype[k])[cell k] (written for
 * every source, also when nsrc < 256, unlike AddSource.cu:194). */
int ads_add_source_bwd_f64(double* g_sxx, double* g_syy, double* g_sxy, double* g_vx,
                           double* g_vy, double* grad_srcv, const double* gout_sxx,
                           const double* gout_syy, const double* gout_sxy,
                           const double* gout_vx, const double* gout_vy,
                           const int64_t* srci, const int64_t* srcj,
                           const int64_t* srctype, int64_t nsrc, int64_t NX, int64_t NY,
                           ads_stream_t stream);

/* GetReceive forward (deps/CustomOps/ReceiveOps/GetReceive.cpp:10-50):
 * fields are (nt, N) histories vx, vy, sxx, syy, sxy; out (nrcv, nt):
 * out[nt*r + k] = field(rcvtype[r])[k*N + cell r].  Indices device int64. */
int ads_get_receive_f64(double* out, const double* vx, const double* vy,
                        const double* sxx, const double* syy, const double* sxy,
                        int64_t nt, const int64_t* rcvi, const int64_t* rcvj,
                        const int64_t* rcvtype, int64_t nrcv, int64_t NX, int64_t NY,
                        ads_stream_t stream);
/* GetReceive backward (GetReceive.cpp:52-96): the five (nt, N) gradients are
 * zeroed, then the (nrcv, nt) output gradient is scattered (duplicates add). */
int ads_get_receive_bwd_f64(double* g_vx, double* g_vy, double* g_sxx, double* g_syy,
                            double* g_sxy, const double* gout, int64_t nt,
                            const int64_t* rcvi, const int64_t* rcvj,
                            const int64_t* rcvtype, int64_t nrcv, int64_t NX, int64_t NY,
                            ads_stream_t stream);

/* One elastic step: fw1..fw4 and add_source of src/Core.jl:96-228 fused into
 * two kernels plus a source launch.  State: 13 arrays of N, contiguous, in the
 * order vx, vy, sigmaxx, sigmayy, sigmaxy, mem[1..8] (the Julia one_step's
 * vx, vy, σxx, σyy, σxy, mem).  ax, bx, ay, by: 2*NX and 2*NY CPML rows as
 * compute_PML_Params returns them (row 0 integer grid, row 1 half grid);
 * kx, ky are accepted for signature fidelity and ignored: the reference never
 * applies the K stretching (adbroadcast modes 3/4 return their input,
 * src/Core.jl:686-693).  srci/srcj/srctype/srcv: device, nsrc entries (one
 * time row).  state_out must not alias state_in. */
int ads_elastic_step_fwd_f64(const double* state_in, double* state_out,
                             const double* lambda, const double* mu, const double* rho,
                             const double* ax, const double* bx, const double* kx,
                             const double* ay, const double* by, const double* ky,
                             double dt, double dx, double dy, int64_t NX, int64_t NY,
                             const int64_t* srci, const int64_t* srcj,
                             const int64_t* srctype, const double* srcv, int64_t nsrc,
                             ads_stream_t stream);
/* FP32 form of ads_elastic_step_fwd_f64: one_step of src/Core.jl:215-228
 * with FP32 arrays, profiles and source values.  The reference computes this
 * step in FP64; results agree with it to FP32 rounding. */
int ads_elastic_step_fwd_f32(const float* state_in, float* state_out, const float* lambda,
                             const float* mu, const float* rho, const float* ax,
                             const float* bx, const float* kx, const float* ay,
                             const float* by, const float* ky, double dt, double dx,
                             double dy, int64_t NX, int64_t NY, const int64_t* srci,
                             const int64_t* srcj, const int64_t* srctype, const float* srcv,
                             int64_t nsrc, ads_stream_t stream);
/* Transpose of one elastic step about state_in: grad_in (13*N, overwritten) is
 * the gradient w.r.t. state_in given grad_out w.r.t. the step's output;
 * grad_lambda, grad_mu, grad_rho are ACCUMULATED (+=).  The TF gradient of
 * src/Core.jl:215-228 (fw4 .. fw1 and AddSource reversed). */
int ads_elastic_step_bwd_f64(const double* state_in, const double* grad_out,
                             double* grad_in, double* grad_lambda, double* grad_mu,
                             double* grad_rho, const double* lambda, const double* mu,
                             const double* rho, const double* ax, const double* bx,
                             const double* ay, const double* by, double dt, double dx,
                             double dy, int64_t NX, int64_t NY, ads_stream_t stream);
/* FP32 form of ads_elastic_step_bwd_f64 (FP32 arrays; the parameter gradients
 * are summed in FP64 inside the call and added to the FP32 outputs). */
int ads_elastic_step_bwd_f32(const float* state_in, const float* grad_out, float* grad_in,
                             float* grad_lambda, float* grad_mu, float* grad_rho,
                             const float* lambda, const float* mu, const float* rho,
                             const float* ax, const float* bx, const float* ay,
                             const float* by, double dt, double dx, double dy, int64_t NX,
                             int64_t NY, ads_stream_t stream);

/* Allocation-free form of ads_elastic_step_bwd_f64 (same arguments, same
 * results).  No counterpart in the reference: it exists for callers that cannot
 * allocate device memory when they run the step, such as an operator called
 * from another framework's custom-call hook (that framework owns the device
 * memory, and a cudaMalloc from an extension bypasses its accounting or fails
 * once it has reserved the device) or time-critical loops that must never enter
 * the CUDA allocator.  Its scratch is one fixed array of 34 x 65536 doubles
 * (about 17.8 MB) compiled into the library and resident on every GPU that
 * loads it until the process exits; grids with (NX+2)*(NY+2) > 65536 are
 * rejected with ADS_ERR_INVALID.  The first call on each device looks up the
 * array's device address and caches it (make that first call before any stream
 * capture); the cache assumes the device's primary context lives until the
 * process exits, so do not call it after cudaDeviceReset.  All calls share the
 * one array, which keeps the last call's contents (each call clears what it
 * uses): calls whose executions overlap on the GPU (different streams without
 * ordering, or threads racing on one device) corrupt each other's scratch. */
int ads_elastic_step_bwd_f64_noalloc(const double* state_in, const double* grad_out,
                                     double* grad_in, double* grad_lambda, double* grad_mu,
                                     double* grad_rho, const double* lambda, const double* mu,
                                     const double* rho, const double* ax, const double* bx,
                                     const double* ay, const double* by, double dt, double dx,
                                     double dy, int64_t NX, int64_t NY, ads_stream_t stream);

/* Out-of-range indices given to the index operators above are skipped on the
 * device (never dereferenced) and recorded: bit 0 scatter/gather, bit 1
 * AddSource, bit 2 GetReceive.  Reads the flags into *flags (clearing them when
 * `clear` is non-zero); synchronises the device.  No reference counterpart:
 * the reference performs no index checks. */
int ads_device_index_errors(int clear, int* flags);

/* ======================================================================
 * Setup helpers (host-side, no device work)
 * ====================================================================== */

/* Acoustic PML damping profiles (src/Core.jl:622-655 with pml_helper
 * :738-761).  sigma depends on i only and tau on j only, so they are returned
 * as 1D host arrays sigma_x[NX+2], tau_y[NY+2]; the reference's 2D Σx, Σy are
 * sigma_x[i] and tau_y[j] broadcast.  use_pml: bit0 XMIN, bit1 XMAX, bit2 YMIN,
 * bit3 YMAX (all four = 15). */
int ads_acoustic_pml_profiles(int64_t NX, int64_t NY, double hx, double hy,
                              int64_t npml, double vp_ref, double Rcoef, int use_pml,
                              double* sigma_x, double* tau_y);
/* Elastic CPML profiles (src/Core.jl:231-407) into host arrays ax, bx, kx
 * (2*NX) and ay, by, ky (2*NY). */
int ads_elastic_cpml_profiles(int64_t NX, int64_t NY, double dx, double dy, double dt,
                              int64_t npml, double npower, double k_max, double alpha_max,
                              double vp_ref, double Rcoef, int use_pml, double* ax,
                              double* bx, double* kx, double* ay, double* by, double* ky);

/* ======================================================================
 * Whole-path acoustic plans: forward traces, misfit and velocity gradient
 * for one or many shots (AcousticPropagatorSolver + SimulatedObservation! +
 * compute_loss_and_grads_GPU, src/Core.jl:562-620,726-730, src/Utils.jl:300-332)
 * ====================================================================== */

typedef struct ads_acoustic_config {
  int64_t MX, MY;     /* model interior: vp is (MX+2) x (MY+2) */
  double dx, dy, dt;  /* DELTAX, DELTAY, DELTAT */
  int64_t npml;       /* NPOINTS_PML (inside each shot's window) */
  double Rcoef;       /* PML reflection coefficient (Struct.jl default 0.001) */
  double vp_ref;      /* PML reference velocity (Struct.jl default 1000) */
  int32_t use_pml;    /* bitmask as ads_acoustic_pml_profiles; 15 = all sides */
  int32_t precision;  /* ADS_F64: plain FP64 drop-in; ADS_F32: FP32 stencils and
                         storage, FP64 misfit and gradient accumulation.  FP32 plans
                         step in the increment form (state u_t and d_t = u_t - u_{t-1},
                         the same update in exact arithmetic, whose FP32 rounding
                         does not build up over thousands of steps); with
                         steps_per_block > 1 they keep the three-level form */
  int32_t variant;    /* ADS_VARIANT_W (phi/psi from the old field, the custom
                         operators' form) or ADS_VARIANT_U (from the new field,
                         one_step, the reference's default PropagatorKernel = 0);
                         both with the whole-path adjoint */
  int32_t use_graph;  /* 1: capture the time loops in CUDA graphs (default) */
  int64_t ckpt_every; /* forward checkpoint spacing k in steps; 0 = automatic */
  int32_t rows_per_thread; /* stencil tile height (autotuner); 0 = automatic */
  int32_t steps_per_block; /* time steps per forward launch (FP32: 1, 2, 4, 8;
                              FP64: 1); 0 = automatic (1) */
  int32_t block_rows;      /* tile height of the time-blocked forward; 0 = automatic */
  int32_t autotune;        /* 1: time candidate tile heights of the forward and adjoint
                              kernels at plan creation and keep the fastest; 2: also,
                              for FP32 variant-W plans without resident segments and
                              with steps_per_block 0, time 1, 2 and 4 forward steps
                              per launch and keep the fastest (more than 1 selects
                              the time-blocked three-level form) */
  int32_t resident_segments; /* checkpoint segments (the last ones) whose forward
                                wavefields stay in device memory for the reverse sweep,
                                which then neither restores nor recomputes them:
                                -1 = none, 0 = as many as fit (see resident_mem_pct),
                                N > 0 = at most N.  Results are identical either way. */
  int32_t resident_mem_pct;  /* share of the device memory free at plan creation (after
                                the plan's other buffers) those wavefields may use, in
                                percent (1..95); 0 = 50 */
  int32_t tma;               /* FP32 plans: 1 = the interior forward steps read u, d and
                                c through tensor-map tile copies (TMA) into shared
                                memory, row chunks ahead (where the driver has the
                                tensor-map encoder); 0 = the register-queue kernel
                                (measured faster beside the concurrent PML launch).
                                Results are identical either way. */
  int32_t reserved[1];
} ads_acoustic_config;

typedef struct ads_acoustic_shot {
  int64_t x0;    /* first column of the shot's window in the padded model
                    (0-based); the window's padded grid is (nx+2) x (MY+2) */
  int64_t nx;    /* window interior width NX (PML included) */
  int64_t nstep; /* NSTEP: slots 0..nstep are simulated */
  int64_t nsrc;
  const int64_t* srci; /* host, 1-based, window-local padded grid */
  const int64_t* srcj;
  const double* srcv;  /* host, (srcv_rows, nsrc) row-major, FP64 */
  int64_t srcv_rows;   /* >= nstep; row r is injected after step r+1 (r >= 1) */
  int64_t nrcv;
  const int64_t* rcvi; /* host, 1-based, window-local padded grid */
  const int64_t* rcvj;
} ads_acoustic_shot;

typedef struct ads_acoustic_plan ads_acoustic_plan;

/* Build a plan: validates all geometry, copies sources and receiver maps to
 * the device, allocates every buffer (wavefield rings, checkpoints, segment
 * stores, adjoint state, FP64 accumulators), picks tiles and, with use_graph,
 * captures the forward and reverse time loops as CUDA graphs.  Shots may have
 * different windows, receiver counts and record lengths. */
int ads_acoustic_plan_create(ads_acoustic_plan** plan, const ads_acoustic_config* cfg,
                             const ads_acoustic_shot* shots, int64_t nshots,
                             ads_stream_t stream);
int ads_acoustic_plan_destroy(ads_acoustic_plan* plan);
/* Packed trace layout: shot s occupies elements [offset(s), offset(s) +
 * (nstep_s+1)*nrcv_s) of the trace/observed buffers, row-major (nstep_s+1,
 * nrcv_s) as SimulatedObservation! returns (NSTEP+1, nrcv). */
int64_t ads_acoustic_plan_trace_offset(const ads_acoustic_plan* plan, int64_t shot);
int64_t ads_acoustic_plan_trace_count(const ads_acoustic_plan* plan);
/* Device bytes held by the plan. */
int64_t ads_acoustic_plan_device_bytes(const ads_acoustic_plan* plan);
/* Kernel launches one forward / one gradient call issues. */
int64_t ads_acoustic_plan_launches(const ads_acoustic_plan* plan, int gradient);
/* Checkpoint segments kept resident (see resident_segments); -1 for a null plan. */
int64_t ads_acoustic_plan_resident_segments(const ads_acoustic_plan* plan);
/* Forward steps per launch the plan runs (steps_per_block as configured, or as
 * the autotuner chose it); -1 for a null plan.  No reference counterpart. */
int64_t ads_acoustic_plan_steps_per_block(const ads_acoustic_plan* plan);
/* Rows per warp of the plan's step items, as created or as the autotuner chose
 * them: forward interior (which = 0), adjoint interior (1), forward PML (2),
 * adjoint PML (3); -1 for a null plan or another `which`.  No reference
 * counterpart. */
int64_t ads_acoustic_plan_rows(const ads_acoustic_plan* plan, int which);
/* 1 when the plan's interior forward steps run through tensor-map copies (see
 * ads_acoustic_config.tma), 0 when not, -1 for a null plan.  No reference
 * counterpart. */
int64_t ads_acoustic_plan_tma(const ads_acoustic_plan* plan);
/* The plan's device-side status since its creation: ADS_OK, or ADS_ERR_TIMEOUT
 * when a bounded wait of its kernels ran out (the results of the calls since
 * then are not valid).  Synchronises the stream.  No reference counterpart. */
int ads_acoustic_plan_device_status(ads_acoustic_plan* plan, ads_stream_t stream);
/* Kernel timing: runs one gradient with direct launches (no graphs) and CUDA
 * events recorded around (0) the forward loop (k_ac_fwd launches only), (1)
 * one full checkpoint segment's recompute launches and (2) the same segment's
 * adjoint launches; out9 = {ms, launches, interior cell-steps} for each range.
 * Synchronises `stream`.  Same arguments as ads_acoustic_plan_gradient minus
 * the outputs.  No reference counterpart (instrumentation for the roofline). */
int ads_acoustic_plan_profile(ads_acoustic_plan* plan, const double* vp,
                              const void* observed, double* out9, ads_stream_t stream);
/* Forward: traces (device, plan precision: double for ADS_F64, float for
 * ADS_F32) receive every shot's (nstep+1, nrcv) receiver record. */
int ads_acoustic_plan_forward(ads_acoustic_plan* plan, const double* vp, void* traces,
                              ads_stream_t stream);
/* Gradient: loss (device, 1 double) = sum over shots, slots and receivers of
 * (trace - observed)^2; grad_vp (device, (MX+2)(MY+2) doubles, overwritten) =
 * d loss / d vp summed over shots.  observed: device, plan precision, packed
 * like the traces.  traces_out may be NULL. */
int ads_acoustic_plan_gradient(ads_acoustic_plan* plan, const double* vp,
                               const void* observed, double* loss, double* grad_vp,
                               void* traces_out, ads_stream_t stream);
/* The same plus the source-time gradient grad_srcv = d loss / d srcv: the
 * gradient ScatterAddOps_backward (ScatterAddOps.h:9-18) gives the wavelet of
 * a source injected into u by src/Core.jl:600-601 (variable_source,
 * src/Utils.jl:603-640).  grad_srcv: device doubles, per shot an (nstep, nsrc)
 * row-major block at ads_acoustic_plan_source_offset(plan, shot), in the
 * caller's shot order; row 0 (never injected) is 0.  May be NULL. */
int ads_acoustic_plan_gradient_ex(ads_acoustic_plan* plan, const double* vp,
                                  const void* observed, double* loss, double* grad_vp,
                                  double* grad_srcv, void* traces_out, ads_stream_t stream);
/* Offset (doubles) of a shot's block in grad_srcv; -1 for a bad index. */
int64_t ads_acoustic_plan_source_offset(const ads_acoustic_plan* plan, int64_t shot);
/* Replace shot `shot`'s source wavelets (same cells) in place, with no plan
 * rebuild: srcv is DEVICE memory, (nstep, nsrc) FP64 row-major as srcv was at
 * creation, read on `stream`; later calls on that stream use the new values,
 * stored exactly as plan creation stores them.  This is what assigning the
 * trainable wavelet of variable_source (src/Utils.jl:603-640) does between
 * the reference's session runs, as in its source-location and wavelet
 * inversion.  ADS_ERR_INVALID for a bad shot index or a null srcv. */
int ads_acoustic_plan_set_source_values(ads_acoustic_plan* plan, int64_t shot,
                                        const double* srcv, ads_stream_t stream);

/* One-shot conveniences (plan + run + destroy; they synchronise `stream`). */
int ads_acoustic_forward(const ads_acoustic_config* cfg, const ads_acoustic_shot* shot,
                         const double* vp, void* traces, ads_stream_t stream);
int ads_acoustic_gradient(const ads_acoustic_config* cfg, const ads_acoustic_shot* shot,
                          const double* vp, const void* observed, double* loss,
                          double* grad_vp, ads_stream_t stream);

/* ======================================================================
 * Whole-path elastic plans (ElasticPropagatorSolver + GetReceive + misfit,
 * src/Core.jl:31-94,701-712): all shots share the model grid.
 * ====================================================================== */

typedef struct ads_elastic_config {
  int64_t NX, NY, NSTEP;
  double dx, dy, dt;
  int64_t npml;       /* NPOINTS_PML (Struct.jl default 12) */
  double npower;      /* NPOWER (2) */
  double k_max;       /* K_MAX_PML (1; the reference never applies K) */
  double alpha_max;   /* ALPHA_MAX_PML (2*pi*f0/2) */
  double vp_ref;      /* vp_ref */
  double Rcoef;       /* 0.001 */
  int32_t use_pml;    /* bitmask, 15 = all sides */
  int32_t precision;  /* ADS_F64 or ADS_F32 */
  int32_t use_graph;
  int32_t rows_per_warp; /* rows a warp streams in the step kernels; 0 = automatic */
  int64_t ckpt_every; /* 0 = automatic */
  int32_t resident_segments; /* checkpoint segments (the last ones) whose per-step strains
                                and accelerations the forward loop stores for the
                                reverse sweep, which then neither restores nor
                                recomputes them: -1 = none, 0 = as many as fit
                                (resident_mem_pct), N > 0 = at most N */
  int32_t resident_mem_pct;  /* share of the device memory free at plan creation (after
                                the plan's other buffers) they may use, in percent
                                (1..95); 0 = 50 */
  int32_t source_gradient;   /* 1: the reverse sweep also records d loss / d srcv
                                (ads_elastic_plan_gradient_ex); plan creation then
                                rejects sources of type 0..4 on a cell the stencil
                                of their field does not update (the padded frame:
                                vx rows/columns 3..NX+1 / 3..NY+1 1-based, vy
                                2..NX / 2..NY, sxx and syy 2..NX / 3..NY+1, sxy
                                3..NX+1 / 2..NY are updated); 0: not */
  int32_t autotune;          /* 1: time candidate row heights of the fused step and of the
                                adjoint at plan creation and keep the fastest
                                (ignored when rows_per_warp is set) */
  int32_t adjoint_passes;    /* the reverse sweep's adjoint step: 1 = one fused
                                row-streaming pass (two adjoint state buffers, no
                                intermediate fields in device memory); 3 = three gather passes
                                over intermediate fields, in place; 0 = 1 for FP32
                                plans, 3 for FP64 plans */
  int32_t reserved[3];
} ads_elastic_config;

typedef struct ads_elastic_shot {
  int64_t nsrc;
  const int64_t* srci; /* host, 1-based padded grid */
  const int64_t* srcj;
  const int64_t* srctype; /* 0 vx, 1 vy, 2 sxx, 3 syy, 4 sxy */
  const double* srcv;     /* host, (srcv_rows, nsrc) FP64; row n-1 feeds slot n */
  int64_t srcv_rows;      /* >= NSTEP */
  int64_t nrcv;
  const int64_t* rcvi; /* host, 1-based */
  const int64_t* rcvj;
  const int64_t* rcvtype; /* 0..4 as srctype */
} ads_elastic_shot;

typedef struct ads_elastic_plan ads_elastic_plan;

int ads_elastic_plan_create(ads_elastic_plan** plan, const ads_elastic_config* cfg,
                            const ads_elastic_shot* shots, int64_t nshots,
                            ads_stream_t stream);
int ads_elastic_plan_destroy(ads_elastic_plan* plan);
/* Packed traces: shot s at offset(s), (nrcv_s, NSTEP+1) row-major as
 * GetReceive returns. */
int64_t ads_elastic_plan_trace_offset(const ads_elastic_plan* plan, int64_t shot);
int64_t ads_elastic_plan_trace_count(const ads_elastic_plan* plan);
int64_t ads_elastic_plan_device_bytes(const ads_elastic_plan* plan);
int64_t ads_elastic_plan_launches(const ads_elastic_plan* plan, int gradient);
/* Checkpoint segments kept resident (see resident_segments); -1 for a null plan. */
int64_t ads_elastic_plan_resident_segments(const ads_elastic_plan* plan);
/* The plan's tiling (as configured or as the autotuner chose it): which = 0,
 * rows per adjoint tile (fused adjoint) or strip (three passes); 1, rows per
 * fused-step tile; 2..5, warp items of the fused adjoint per shot whose logic
 * is CPML-free (2), x-CPML / box-edge rows (3), y-CPML / box-edge columns
 * (4) or both (5), 0 for the three passes; -1 for a null plan or another
 * `which`.  No reference counterpart. */
int64_t ads_elastic_plan_rows(const ads_elastic_plan* plan, int which);
/* ads_elastic_plan_gradient plus the source-time gradient grad_srcv = d loss /
 * d srcv, the gradient AddSource's backward (AddSource.cpp:91-155) gathers:
 * device doubles, per shot an (NSTEP, nsrc) row-major block at
 * ads_elastic_plan_source_offset(plan, shot); 0 for sources of a type outside
 * 0..4.  Needs a plan created with source_gradient = 1; may be NULL. */
int ads_elastic_plan_gradient_ex(ads_elastic_plan* plan, const double* lambda,
                                 const double* mu, const double* rho, const void* observed,
                                 double* loss, double* grad_lambda, double* grad_mu,
                                 double* grad_rho, double* grad_srcv, void* traces_out,
                                 ads_stream_t stream);
/* Offset (doubles) of a shot's block in grad_srcv; -1 for a bad index. */
int64_t ads_elastic_plan_source_offset(const ads_elastic_plan* plan, int64_t shot);
/* As ads_acoustic_plan_set_source_values: srcv is DEVICE memory, (NSTEP, nsrc)
 * FP64 row-major. */
int ads_elastic_plan_set_source_values(ads_elastic_plan* plan, int64_t shot,
                                       const double* srcv, ads_stream_t stream);
/* lambda, mu, rho: device, N doubles. */
int ads_elastic_plan_forward(ads_elastic_plan* plan, const double* lambda,
                             const double* mu, const double* rho, void* traces,
                             ads_stream_t stream);
/* grad_lambda, grad_mu, grad_rho: device, N doubles, overwritten. */
int ads_elastic_plan_gradient(ads_elastic_plan* plan, const double* lambda,
                              const double* mu, const double* rho, const void* observed,
                              double* loss, double* grad_lambda, double* grad_mu,
                              double* grad_rho, void* traces_out, ads_stream_t stream);
/* One-shot conveniences (plan + run + destroy; they synchronise `stream`):
 * ElasticPropagatorSolver + SimulatedObservation! for one source
 * (src/Core.jl:31-94,701-712), and with the misfit and its gradients. */
int ads_elastic_forward(const ads_elastic_config* cfg, const ads_elastic_shot* shot,
                        const double* lambda, const double* mu, const double* rho,
                        void* traces, ads_stream_t stream);
int ads_elastic_gradient(const ads_elastic_config* cfg, const ads_elastic_shot* shot,
                         const double* lambda, const double* mu, const double* rho,
                         const void* observed, double* loss, double* grad_lambda,
                         double* grad_mu, double* grad_rho, ads_stream_t stream);
/* Kernel timing (no reference counterpart): every step kernel of the plan is
 * launched 20 times on the plan's buffers between CUDA events.  out: 14
 * doubles, pairs (ms per launch, interior cell-updates per launch) for the
 * forward step, the forward step storing the adjoint's strains, adjoint
 * 1..3 (the fused adjoint step in the first of them, zero time in the other
 * two), the source / receiver and the residual kernels.  Leaves the plan's
 * state zeroed; synchronises the stream. */
int ads_elastic_plan_profile(ads_elastic_plan* plan, const double* lambda,
                             const double* mu, const double* rho, double* out,
                             ads_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
