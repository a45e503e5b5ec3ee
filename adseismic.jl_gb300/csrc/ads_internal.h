// ads_internal.h -- shared host/device helpers of libadseismic_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "adseismic_gb300.h"

namespace ads {

// ----- error state (thread-local message, status codes) -------------------
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
void note_launches(int64_t n);
// Launches issued while a graph is being captured are counted at replay.
void set_launch_counting(bool on);

// Check a CUDA runtime call; on failure record the message and return
// ADS_ERR_CUDA (or ADS_ERR_NOMEM for allocation failures).
#define ADS_CUDA(call)                                                            \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      return ::ads::fail(e_ == cudaErrorMemoryAllocation ? ADS_ERR_NOMEM          \
                                                         : ADS_ERR_CUDA,          \
                         "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                         __FILE__, __LINE__);                                     \
    }                                                                             \
  } while (0)

// Check the launch that was just issued.
#define ADS_LAUNCHED(n)                                                           \
  do {                                                                            \
    cudaError_t e_ = cudaGetLastError();                                          \
    if (e_ != cudaSuccess)                                                        \
      return ::ads::fail(ADS_ERR_CUDA, "kernel launch failed: %s (%s:%d)",        \
                         cudaGetErrorString(e_), __FILE__, __LINE__);             \
    ::ads::note_launches(n);                                                      \
  } while (0)

#define ADS_REQUIRE(cond, ...)                                                    \
  do {                                                                            \
    if (!(cond)) return ::ads::fail(ADS_ERR_INVALID, __VA_ARGS__);                \
  } while (0)

// Fail loudly when no usable device is present (no CPU fallback exists).
int require_device();

// out[e] = (T)(in[e] * scale) for e < n, launched on st (one kernel).
int cast_scaled(float* out, const double* in, int64_t n, double scale, cudaStream_t st);
int cast_scaled(double* out, const double* in, int64_t n, double scale, cudaStream_t st);

inline int64_t div_up(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return div_up(a, b) * b; }

// Host PML helpers (shared by the C API and the plans).
void acoustic_pml_1d(int64_t NX, int64_t NY, double hx, double hy, int64_t npml,
                     double vp_ref, double Rcoef, int use_pml, double* sx, double* ty);
void elastic_cpml(int64_t NX, int64_t NY, double dx, double dy, double dt, int64_t npml,
                  double npower, double k_max, double alpha_max, double vp_ref,
                  double Rcoef, int use_pml, double* ax, double* bx, double* kx,
                  double* ay, double* by, double* ky);

// ---------------------------------------------------------------------------
// Internal grid layout used by the plans: each padded row of ny+2 cells is
// stored with a pitch that is a multiple of 32 elements and an offset of
// JOFF = 31, so that interior column j = 1 starts on a 32-element boundary
// (128 B for FP32, 256 B for FP64) and every warp row load is aligned.  The
// pitch leaves at least 32 spare elements after column ny+1 so that a
// thread's vector load starting at a valid column never leaves its row.
// ---------------------------------------------------------------------------
constexpr int JOFF = 31;
inline int64_t grid_pitch(int64_t ny) { return round_up(ny + 2 + JOFF + 32, 32); }

}  // namespace ads
