// common.cu -- error state, version, launch accounting and host-side PML setup.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "ads_internal.h"

namespace ads {

static thread_local char g_err[1024] = "";
static std::atomic<int64_t> g_launches{0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

static thread_local bool g_counting = true;

void set_launch_counting(bool on) { g_counting = on; }

void note_launches(int64_t n) {
  if (g_counting) g_launches.fetch_add(n, std::memory_order_relaxed);
}

int require_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(ADS_ERR_CUDA, "no CUDA device available (%s); this library has no CPU path",
                e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
  }
  return ADS_OK;
}

// src/Core.jl:738-761 (pml_helper) over x = i*hx and y = j*hy; sigma depends
// on x only and tau on y only (Core.jl:633-638 evaluates it per (i, j)).
void acoustic_pml_1d(int64_t NX, int64_t NY, double hx, double hy, int64_t npml,
                     double vp_ref, double Rcoef, int use_pml, double* sx, double* ty) {
  const double Lx = npml * hx, Ly = npml * hy;
  const double xi_x = vp_ref / Lx * std::log(1 / Rcoef);
  const double xi_y = vp_ref / Ly * std::log(1 / Rcoef);
  const double twopi = 2 * M_PI;
  for (int64_t i = 0; i < NX + 2; i++) {
    const double x = i * hx;
    double o = 0.0;
    if (x < Lx && (use_pml & 1)) {
      const double d = std::fabs(Lx - x);
      o = xi_x * (d / Lx - std::sin(twopi * d / Lx) / twopi);
    } else if (x > hx * (NX + 1) - Lx && (use_pml & 2)) {
      const double d = std::fabs(x - (hx * (NX + 1) - Lx));
      o = xi_x * (d / Lx - std::sin(twopi * d / Lx) / twopi);
    }
    sx[i] = o;
  }
  for (int64_t j = 0; j < NY + 2; j++) {
    const double y = j * hy;
    double o = 0.0;
    if (y < Ly && (use_pml & 4)) {
      const double d = std::fabs(Ly - y);
      o = xi_y * (d / Ly - std::sin(twopi * d / Ly) / twopi);
    } else if (y > hy * (NY + 1) - Ly && (use_pml & 8)) {
      const double d = std::fabs(y - (hy * (NY + 1) - Ly));
      o = xi_y * (d / Ly - std::sin(twopi * d / Ly) / twopi);
    }
    ty[j] = o;
  }
}

// src/Core.jl:231-407: SEISMIC_CPML damping d, stretching K, frequency shift
// alpha on the integer and half grids; b = exp(-(d/K + alpha) dt),
// a = d (b - 1) / (K (d + K alpha)) where |d| > 1e-6.
void elastic_cpml(int64_t NX, int64_t NY, double dx, double dy, double dt, int64_t npml,
                  double npower, double k_max, double alpha_max, double vp_ref,
                  double Rcoef, int use_pml, double* ax, double* bx, double* kx,
                  double* ay, double* by, double* ky) {
  for (int axis = 0; axis < 2; axis++) {
    const int64_t n = axis == 0 ? NX : NY;
    const double h = axis == 0 ? dx : dy;
    const double thick = npml * h;
    const double d0 = -(npower + 1) * vp_ref * std::log(Rcoef) / (2. * thick);
    const bool lo = axis == 0 ? (use_pml & 1) : (use_pml & 4);
    const bool hi = axis == 0 ? (use_pml & 2) : (use_pml & 8);
    double* A = axis == 0 ? ax : ay;
    double* B = axis == 0 ? bx : by;
    double* K = axis == 0 ? kx : ky;
    const double origin_lo = thick, origin_hi = (n - 0.5) * h - thick;
    for (int64_t i = 0; i < n; i++) {
      for (int half = 0; half < 2; half++) {
        const double pos = h * i + (half ? h / 2. : 0.0);
        double d = 0.0, k = 1.0, al = 0.0;
        if (lo) {
          const double a = origin_lo - pos;
          if (a >= 0.0) {
            const double an = a / thick;
            d = d0 * std::pow(an, npower);
            k = 1. + (k_max - 1.) * std::pow(an, npower);
            al = alpha_max * an;
          }
        }
        if (hi) {
          const double a = pos - origin_hi;
          if (a >= 0) {
            const double an = a / thick;
            d = d0 * std::pow(an, npower);
            k = 1. + (k_max - 1.) * std::pow(an, npower);
            al = alpha_max * an;
          }
        }
        if (al < 0) al = 0;
        const double b = std::exp(-(d / k + al) * dt);
        A[half * n + i] = std::fabs(d) > 1e-6 ? d * (b - 1.) / (k * (d + k * al)) : 0.0;
        B[half * n + i] = b;
        K[half * n + i] = k;
      }
    }
  }
}

// out[e] = (T)(in[e] * scale): a plan's source wavelets from a caller's FP64
// device array, rounded as plan creation rounds them on the host.
template <typename T>
__global__ void k_cast_scaled(T* __restrict__ out, const double* __restrict__ in, int64_t n,
                              double scale) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    out[e] = (T)(in[e] * scale);
}

template <typename T>
static int cast_scaled(T* out, const double* in, int64_t n, double scale, cudaStream_t st) {
  if (n <= 0) return ADS_OK;
  const int64_t blocks = std::min<int64_t>(div_up(n, 256), 152 * 16);
  k_cast_scaled<T><<<(unsigned)blocks, 256, 0, st>>>(out, in, n, scale);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

int cast_scaled(float* out, const double* in, int64_t n, double scale, cudaStream_t st) {
  return cast_scaled<float>(out, in, n, scale, st);
}

int cast_scaled(double* out, const double* in, int64_t n, double scale, cudaStream_t st) {
  return cast_scaled<double>(out, in, n, scale, st);
}

}  // namespace ads

extern "C" {

const char* ads_last_error(void) { return ads::g_err; }

const char* ads_version(void) { return "adseismic_gb300 0.1.0 (sm_103a)"; }

int64_t ads_launch_count(void) { return ads::g_launches.load(); }

int ads_acoustic_pml_profiles(int64_t NX, int64_t NY, double hx, double hy, int64_t npml,
                              double vp_ref, double Rcoef, int use_pml, double* sigma_x,
                              double* tau_y) {
  ADS_REQUIRE(NX >= 1 && NY >= 1, "NX, NY must be >= 1 (got %lld, %lld)", (long long)NX,
              (long long)NY);
  ADS_REQUIRE(npml >= 1 && hx > 0 && hy > 0 && Rcoef > 0 && Rcoef < 1,
              "invalid PML parameters");
  ADS_REQUIRE(sigma_x && tau_y, "null output");
  ads::acoustic_pml_1d(NX, NY, hx, hy, npml, vp_ref, Rcoef, use_pml, sigma_x, tau_y);
  return ADS_OK;
}

int ads_elastic_cpml_profiles(int64_t NX, int64_t NY, double dx, double dy, double dt,
                              int64_t npml, double npower, double k_max, double alpha_max,
                              double vp_ref, double Rcoef, int use_pml, double* ax,
                              double* bx, double* kx, double* ay, double* by, double* ky) {
  ADS_REQUIRE(NX >= 1 && NY >= 1, "NX, NY must be >= 1");
  ADS_REQUIRE(npml >= 1 && dx > 0 && dy > 0 && dt > 0 && Rcoef > 0 && Rcoef < 1,
              "invalid CPML parameters");
  ADS_REQUIRE(ax && bx && kx && ay && by && ky, "null output");
  ads::elastic_cpml(NX, NY, dx, dy, dt, npml, npower, k_max, alpha_max, vp_ref, Rcoef,
                    use_pml, ax, bx, kx, ay, by, ky);
  return ADS_OK;
}

}  // extern "C"
