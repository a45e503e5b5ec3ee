// step_ops.cu -- single-step drop-in operators of the reference's custom-op
// library: AcousticOneStep forward/backward, ScatterAddOps, GatherOps,
// AddSource and GetReceive.
//
// This translation unit is compiled with --fmad=false and keeps the
// reference's expression order, so the FP64 acoustic forward reproduces
// AcousticOneStepCpuForward (deps/CustomOps/AcousticOneStepCpu/
// AcousticOneStepCpu.h:1-48) bit for bit.  Threads map x -> j (the contiguous
// depth axis), so every warp access is coalesced (the reference GPU kernel maps
// threadIdx.x to the strided axis, AcousticOneStep.cu:28-34).
#include <algorithm>

#include "ads_internal.h"

namespace ads {

// Device-side record of rejected indices (out-of-range source / receiver /
// scatter indices are skipped, never dereferenced).
__device__ int g_bad_index = 0;

namespace {

constexpr int BJ = 32, BI = 8;

template <typename T>
__global__ void k_acoustic_fwd_w(const T* __restrict__ w, const T* __restrict__ wold,
                                 const T* __restrict__ phi, const T* __restrict__ psi,
                                 const T* __restrict__ sigma, const T* __restrict__ tau,
                                 const T* __restrict__ c, T dt, T hx, T hy, int NX, int NY,
                                 T* __restrict__ u, T* __restrict__ phiout,
                                 T* __restrict__ psiout) {
  const int j = blockIdx.x * BJ + threadIdx.x;
  const int i = blockIdx.y * BI + threadIdx.y;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t S = NY + 2;
  const int64_t k = (int64_t)i * S + j;
  if (i == 0 || i == NX + 1 || j == 0 || j == NY + 1) {
    u[k] = 0;
    phiout[k] = 0;
    psiout[k] = 0;
    return;
  }
  const T sg = sigma[k], ta = tau[k], ck = c[k];
  const T two = 2, one = 1, half = 2;
  T v = (two - sg * ta * dt * dt - two * dt * dt / hx / hx * ck -
         two * dt * dt / hy / hy * ck) * w[k] +
        ck * (dt / hx) * (dt / hx) * (w[k + S] + w[k - S]) +
        ck * (dt / hy) * (dt / hy) * (w[k + 1] + w[k - 1]) +
        (dt * dt / (T(2.0) * hx)) * (phi[k + S] - phi[k - S]) +
        (dt * dt / (T(2.0) * hy)) * (psi[k + 1] - psi[k - 1]) -
        (one - (sg + ta) * dt / half) * wold[k];
  u[k] = v / (one + (sg + ta) / half * dt);
  phiout[k] = (one - dt * sg) * phi[k] + dt * ck * (ta - sg) / T(2.0) / hx * (w[k + S] - w[k - S]);
  psiout[k] = (one - dt * ta) * psi[k] + dt * ck * (sg - ta) / T(2.0) / hy * (w[k + 1] - w[k - 1]);
}

// Variant U (src/Core.jl:528-549): u over the grid first ...
template <typename T>
__global__ void k_acoustic_fwd_u1(const T* __restrict__ w, const T* __restrict__ wold,
                                  const T* __restrict__ phi, const T* __restrict__ psi,
                                  const T* __restrict__ sigma, const T* __restrict__ tau,
                                  const T* __restrict__ c, T dt, T hx, T hy, int NX, int NY,
                                  T* __restrict__ u) {
  const int j = blockIdx.x * BJ + threadIdx.x;
  const int i = blockIdx.y * BI + threadIdx.y;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t S = NY + 2;
  const int64_t k = (int64_t)i * S + j;
  if (i == 0 || i == NX + 1 || j == 0 || j == NY + 1) {
    u[k] = 0;
    return;
  }
  const T sg = sigma[k], ta = tau[k], ck = c[k];
  const T dt2 = dt * dt, one = 1;
  const T kx = T(2) * dt2 / (hx * hx), ky = T(2) * dt2 / (hy * hy);
  const T cx = (dt / hx) * (dt / hx), cy = (dt / hy) * (dt / hy);
  const T fx = dt2 / (T(2) * hx), fy = dt2 / (T(2) * hy);
  T v = (T(2) - sg * ta * dt2 - kx * ck - ky * ck) * w[k] + ck * cx * (w[k + S] + w[k - S]) +
        ck * cy * (w[k + 1] + w[k - 1]) + fx * (phi[k + S] - phi[k - S]) +
        fy * (psi[k + 1] - psi[k - 1]) - (one - (sg + ta) * dt / T(2)) * wold[k];
  u[k] = v / (one + (sg + ta) / T(2) * dt);
}

// ... then phi/psi from the new u.
template <typename T>
__global__ void k_acoustic_fwd_u2(const T* __restrict__ u, const T* __restrict__ phi,
                                  const T* __restrict__ psi, const T* __restrict__ sigma,
                                  const T* __restrict__ tau, const T* __restrict__ c, T dt,
                                  T hx, T hy, int NX, int NY, T* __restrict__ phiout,
                                  T* __restrict__ psiout) {
  const int j = blockIdx.x * BJ + threadIdx.x;
  const int i = blockIdx.y * BI + threadIdx.y;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t S = NY + 2;
  const int64_t k = (int64_t)i * S + j;
  if (i == 0 || i == NX + 1 || j == 0 || j == NY + 1) {
    phiout[k] = 0;
    psiout[k] = 0;
    return;
  }
  const T sg = sigma[k], ta = tau[k], ck = c[k], one = 1;
  phiout[k] = (one - dt * sg) * phi[k] + dt * ck * (ta - sg) / (T(2) * hx) * (u[k + S] - u[k - S]);
  psiout[k] = (one - dt * ta) * psi[k] + dt * ck * (sg - ta) / (T(2) * hy) * (u[k + 1] - u[k - 1]);
}

// Gradient of the new u for variant U: the output gradient plus what phi'/psi'
// send back through their u differences (interior cells only: u's frame is a
// constant zero).
template <typename T>
__device__ __forceinline__ T gu_total(int i, int j, int NX, int NY, int64_t S,
                                      const T* __restrict__ gu, const T* __restrict__ gp,
                                      const T* __restrict__ gq, const T* __restrict__ sigma,
                                      const T* __restrict__ tau, const T* __restrict__ c,
                                      T dt, T hx, T hy) {
  if (i < 1 || i > NX || j < 1 || j > NY) return T(0);
  const int64_t k = (int64_t)i * S + j;
  T g = gu[k];
  // y = x - e_i : x is y's i+1 neighbour
  if (i - 1 >= 1) {
    const int64_t y = k - S;
    g += dt * c[y] * (tau[y] - sigma[y]) / (T(2) * hx) * gp[y];
  }
  if (i + 1 <= NX) {
    const int64_t y = k + S;
    g -= dt * c[y] * (tau[y] - sigma[y]) / (T(2) * hx) * gp[y];
  }
  if (j - 1 >= 1) {
    const int64_t y = k - 1;
    g += dt * c[y] * (sigma[y] - tau[y]) / (T(2) * hy) * gq[y];
  }
  if (j + 1 <= NY) {
    const int64_t y = k + 1;
    g -= dt * c[y] * (sigma[y] - tau[y]) / (T(2) * hy) * gq[y];
  }
  return g;
}

// Gather-form transpose of one step (both variants).  Each output cell sums
// the contributions the reference's scatter loop (AcousticOneStepCpu.h:76-124)
// sends it; frame cells receive them too.
template <typename T, int VARIANT>
__global__ void k_acoustic_bwd(T* __restrict__ grad_w, T* __restrict__ grad_wold,
                               T* __restrict__ grad_phi, T* __restrict__ grad_psi,
                               T* __restrict__ grad_c, const T* __restrict__ grad_u,
                               const T* __restrict__ grad_phiout,
                               const T* __restrict__ grad_psiout, const T* __restrict__ w,
                               const T* __restrict__ sigma, const T* __restrict__ tau,
                               const T* __restrict__ c, T dt, T hx, T hy, int NX, int NY,
                               const T* __restrict__ u) {
  const int j = blockIdx.x * BJ + threadIdx.x;
  const int i = blockIdx.y * BI + threadIdx.y;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t S = NY + 2;
  const int64_t k = (int64_t)i * S + j;
  const T one = 1, two = 2;
  auto interior = [&](int a, int b) { return a >= 1 && a <= NX && b >= 1 && b <= NY; };
  auto G = [&](int a, int b) -> T {
    if (VARIANT == 0) return grad_u[(int64_t)a * S + b];
    return gu_total<T>(a, b, NX, NY, S, grad_u, grad_phiout, grad_psiout, sigma, tau, c,
                       dt, hx, hy);
  };
  auto den = [&](int64_t y) { return one + (sigma[y] + tau[y]) / two * dt; };
  T gw = 0, gwo = 0, gph = 0, gps = 0, gc = 0;
  if (interior(i, j)) {
    const T sg = sigma[k], ta = tau[k], ck = c[k], g = G(i, j), d = den(k);
    gc = ((-two * dt * dt / hx / hx - two * dt * dt / hy / hy) * w[k] +
          (dt / hx) * (dt / hx) * (w[k + S] + w[k - S]) +
          (dt / hy) * (dt / hy) * (w[k + 1] + w[k - 1])) * g / d;
    gw = (two - sg * ta * dt * dt - two * dt * dt / hx / hx * ck -
          two * dt * dt / hy / hy * ck) * g / d;
    gwo = -(one - (sg + ta) * dt / two) * g / d;
    const T gp = grad_phiout[k], gs = grad_psiout[k];
    gph = (one - dt * sg) * gp;
    gps = (one - dt * ta) * gs;
    if (VARIANT == 0) {
      gc += dt * (ta - sg) / T(2.0) / hx * (w[k + S] - w[k - S]) * gp;
      gc += dt * (sg - ta) / T(2.0) / hy * (w[k + 1] - w[k - 1]) * gs;
    } else {
      gc += dt * (ta - sg) / (two * hx) * (u[k + S] - u[k - S]) * gp;
      gc += dt * (sg - ta) / (two * hy) * (u[k + 1] - u[k - 1]) * gs;
    }
  }
  // neighbours y whose stencil reaches x
  const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, -1, 1};
#pragma unroll
  for (int n = 0; n < 4; n++) {
    const int a = i + di[n], b = j + dj[n];
    if (!interior(a, b)) continue;
    const int64_t y = (int64_t)a * S + b;
    const T cy = c[y], g = G(a, b), d = den(y);
    if (n < 2) {
      // x is y's i+1 neighbour when n == 0 (y = x - e_i), i-1 neighbour when n == 1
      const T sgn = n == 0 ? one : -one;
      gw += cy * (dt / hx) * (dt / hx) * g / d;
      gph += sgn * (dt * dt / (T(2.0) * hx)) * g / d;
      if (VARIANT == 0) gw += sgn * dt * cy * (tau[y] - sigma[y]) / T(2.0) / hx * grad_phiout[y];
    } else {
      const T sgn = n == 2 ? one : -one;
      gw += cy * (dt / hy) * (dt / hy) * g / d;
      gps += sgn * (dt * dt / (T(2.0) * hy)) * g / d;
      if (VARIANT == 0) gw += sgn * dt * cy * (sigma[y] - tau[y]) / T(2.0) / hy * grad_psiout[y];
    }
  }
  grad_w[k] = gw;
  grad_wold[k] = gwo;
  grad_phi[k] = gph;
  grad_psi[k] = gps;
  grad_c[k] = gc;
}

template <typename T>
int acoustic_fwd(const T* w, const T* wold, const T* phi, const T* psi, const T* sigma,
                 const T* tau, const T* c, double dt, double hx, double hy, int64_t NX,
                 int64_t NY, T* u, T* phiout, T* psiout, int variant, cudaStream_t st) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 1 && NY >= 1 && NX < (1 << 30) && NY < (1 << 30),
              "NX, NY out of range (%lld, %lld)", (long long)NX, (long long)NY);
  ADS_REQUIRE(w && wold && phi && psi && sigma && tau && c && u && phiout && psiout,
              "null pointer argument");
  ADS_REQUIRE(variant == 0 || variant == 1, "variant must be 0 (w) or 1 (u)");
  dim3 blk(BJ, BI), grd((unsigned)div_up(NY + 2, BJ), (unsigned)div_up(NX + 2, BI));
  if (variant == 0) {
    k_acoustic_fwd_w<T><<<grd, blk, 0, st>>>(w, wold, phi, psi, sigma, tau, c, T(dt), T(hx),
                                              T(hy), (int)NX, (int)NY, u, phiout, psiout);
    ADS_LAUNCHED(1);
  } else {
    k_acoustic_fwd_u1<T><<<grd, blk, 0, st>>>(w, wold, phi, psi, sigma, tau, c, T(dt), T(hx),
                                               T(hy), (int)NX, (int)NY, u);
    ADS_LAUNCHED(1);
    k_acoustic_fwd_u2<T><<<grd, blk, 0, st>>>(u, phi, psi, sigma, tau, c, T(dt), T(hx), T(hy),
                                               (int)NX, (int)NY, phiout, psiout);
    ADS_LAUNCHED(1);
  }
  return ADS_OK;
}

template <typename T>
int acoustic_bwd(T* grad_w, T* grad_wold, T* grad_phi, T* grad_psi, T* grad_c,
                 const T* grad_u, const T* grad_phiout, const T* grad_psiout, const T* w,
                 const T* sigma, const T* tau, const T* c, double dt, double hx, double hy,
                 int64_t NX, int64_t NY, const T* u, int variant, cudaStream_t st) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 1 && NY >= 1 && NX < (1 << 30) && NY < (1 << 30),
              "NX, NY out of range");
  ADS_REQUIRE(grad_w && grad_wold && grad_phi && grad_psi && grad_c && grad_u &&
                  grad_phiout && grad_psiout && w && sigma && tau && c,
              "null pointer argument");
  ADS_REQUIRE(variant == 0 || (variant == 1 && u), "variant must be 0, or 1 with u given");
  dim3 blk(BJ, BI), grd((unsigned)div_up(NY + 2, BJ), (unsigned)div_up(NX + 2, BI));
  if (variant == 0)
    k_acoustic_bwd<T, 0><<<grd, blk, 0, st>>>(grad_w, grad_wold, grad_phi, grad_psi, grad_c,
                                               grad_u, grad_phiout, grad_psiout, w, sigma,
                                               tau, c, T(dt), T(hx), T(hy), (int)NX,
                                               (int)NY, u);
  else
    k_acoustic_bwd<T, 1><<<grd, blk, 0, st>>>(grad_w, grad_wold, grad_phi, grad_psi, grad_c,
                                               grad_u, grad_phiout, grad_psiout, w, sigma,
                                               tau, c, T(dt), T(hx), T(hy), (int)NX,
                                               (int)NY, u);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

// ---------------------------------------------------------------- index ops

__global__ void k_copy(double* __restrict__ out, const double* __restrict__ in, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    out[t] = in[t];
}

__global__ void k_zero(double* __restrict__ out, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    out[t] = 0.0;
}

__global__ void k_scatter_add(double* out, const int64_t* __restrict__ ii,
                              const double* __restrict__ upd, int64_t d, int64_t n) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t x = ii[t] - 1;
  if (x < 0 || x >= d) {
    atomicOr(&g_bad_index, 1);
    return;
  }
  atomicAdd(out + x, upd[t]);
}

__global__ void k_gather(double* __restrict__ out, const double* __restrict__ v,
                         const int64_t* __restrict__ ii, int64_t n, int64_t dlen) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t x = ii[t] - 1;
  if (x < 0 || x >= dlen) {
    atomicOr(&g_bad_index, 1);
    out[t] = 0.0;
    return;
  }
  out[t] = v[x];
}

struct Five {
  double* p[5];
};
struct CFive {
  const double* p[5];
};

// AddSource field order (sxx, syy, sxy, vx, vy); srctype 0 vx, 1 vy, 2 sxx,
// 3 syy, 4 sxy -> positions 3, 4, 0, 1, 2.
__device__ __forceinline__ int type_slot(int64_t t) {
  return t == 0 ? 3 : t == 1 ? 4 : t == 2 ? 0 : t == 3 ? 1 : t == 4 ? 2 : -1;
}

__global__ void k_add_source(Five out, const int64_t* __restrict__ si,
                             const int64_t* __restrict__ sj, const int64_t* __restrict__ st,
                             const double* __restrict__ sv, int64_t nsrc, int64_t NX,
                             int64_t NY) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nsrc) return;
  const int slot = type_slot(st[t]);
  if (slot < 0) return;
  const int64_t a = si[t] - 1, b = sj[t] - 1;
  if (a < 0 || a > NX + 1 || b < 0 || b > NY + 1) {
    atomicOr(&g_bad_index, 2);
    return;
  }
  atomicAdd(out.p[slot] + a * (NY + 2) + b, sv[t]);
}

__global__ void k_add_source_grad(CFive g, double* __restrict__ gs,
                                  const int64_t* __restrict__ si,
                                  const int64_t* __restrict__ sj,
                                  const int64_t* __restrict__ st, int64_t nsrc, int64_t NX,
                                  int64_t NY) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nsrc) return;
  const int slot = type_slot(st[t]);
  const int64_t a = si[t] - 1, b = sj[t] - 1;
  if (slot < 0 || a < 0 || a > NX + 1 || b < 0 || b > NY + 1) {
    if (slot >= 0) atomicOr(&g_bad_index, 2);
    gs[t] = 0.0;
    return;
  }
  gs[t] = g.p[slot][a * (NY + 2) + b];
}

// GetReceive field order (vx, vy, sxx, syy, sxy) = srctype order.
__global__ void k_get_receive(double* __restrict__ out, CFive f, int64_t nt,
                              const int64_t* __restrict__ ri, const int64_t* __restrict__ rj,
                              const int64_t* __restrict__ rt, int64_t nrcv, int64_t NX,
                              int64_t NY) {
  const int64_t r = blockIdx.y;
  const int64_t N = (NX + 2) * (NY + 2);
  if (r >= nrcv) return;
  const int64_t type = rt[r], a = ri[r] - 1, b = rj[r] - 1;
  const bool ok = type >= 0 && type <= 4 && a >= 0 && a <= NX + 1 && b >= 0 && b <= NY + 1;
  if (!ok && threadIdx.x == 0 && blockIdx.x == 0) atomicOr(&g_bad_index, 4);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
       k += (int64_t)gridDim.x * blockDim.x)
    out[nt * r + k] = ok ? f.p[type][k * N + a * (NY + 2) + b] : 0.0;
}

__global__ void k_get_receive_grad(Five g, const double* __restrict__ gout, int64_t nt,
                                   const int64_t* __restrict__ ri,
                                   const int64_t* __restrict__ rj,
                                   const int64_t* __restrict__ rt, int64_t nrcv, int64_t NX,
                                   int64_t NY) {
  const int64_t r = blockIdx.y;
  const int64_t N = (NX + 2) * (NY + 2);
  if (r >= nrcv) return;
  const int64_t type = rt[r], a = ri[r] - 1, b = rj[r] - 1;
  if (!(type >= 0 && type <= 4 && a >= 0 && a <= NX + 1 && b >= 0 && b <= NY + 1)) return;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(g.p[type] + k * N + a * (NY + 2) + b, gout[nt * r + k]);
}

int copy_if_needed(double* out, const double* in, int64_t n, cudaStream_t st) {
  if (out == in || n == 0) return ADS_OK;
  k_copy<<<(unsigned)std::min<int64_t>(div_up(n, 256), 4096), 256, 0, st>>>(out, in, n);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

}  // namespace
}  // namespace ads

using namespace ads;

extern "C" {

int ads_acoustic_step_fwd_f64(const double* w, const double* wold, const double* phi,
                              const double* psi, const double* sigma, const double* tau,
                              const double* c, double dt, double hx, double hy, int64_t NX,
                              int64_t NY, double* u, double* phiout, double* psiout,
                              int variant, ads_stream_t stream) {
  return acoustic_fwd<double>(w, wold, phi, psi, sigma, tau, c, dt, hx, hy, NX, NY, u,
                              phiout, psiout, variant, (cudaStream_t)stream);
}

int ads_acoustic_step_fwd_f32(const float* w, const float* wold, const float* phi,
                              const float* psi, const float* sigma, const float* tau,
                              const float* c, double dt, double hx, double hy, int64_t NX,
                              int64_t NY, float* u, float* phiout, float* psiout,
                              int variant, ads_stream_t stream) {
  return acoustic_fwd<float>(w, wold, phi, psi, sigma, tau, c, dt, hx, hy, NX, NY, u, phiout,
                             psiout, variant, (cudaStream_t)stream);
}

int ads_acoustic_step_bwd_f64(double* grad_w, double* grad_wold, double* grad_phi,
                              double* grad_psi, double* grad_c, const double* grad_u,
                              const double* grad_phiout, const double* grad_psiout,
                              const double* w, const double* wold, const double* phi,
                              const double* psi, const double* sigma, const double* tau,
                              const double* c, double dt, double hx, double hy, int64_t NX,
                              int64_t NY, const double* u, const double* phiout,
                              const double* psiout, int variant, ads_stream_t stream) {
  (void)wold; (void)phi; (void)psi; (void)phiout; (void)psiout;
  return acoustic_bwd<double>(grad_w, grad_wold, grad_phi, grad_psi, grad_c, grad_u,
                              grad_phiout, grad_psiout, w, sigma, tau, c, dt, hx, hy, NX, NY,
                              u, variant, (cudaStream_t)stream);
}

int ads_acoustic_step_bwd_f32(float* grad_w, float* grad_wold, float* grad_phi,
                              float* grad_psi, float* grad_c, const float* grad_u,
                              const float* grad_phiout, const float* grad_psiout,
                              const float* w, const float* wold, const float* phi,
                              const float* psi, const float* sigma, const float* tau,
                              const float* c, double dt, double hx, double hy, int64_t NX,
                              int64_t NY, const float* u, const float* phiout,
                              const float* psiout, int variant, ads_stream_t stream) {
  (void)wold; (void)phi; (void)psi; (void)phiout; (void)psiout;
  return acoustic_bwd<float>(grad_w, grad_wold, grad_phi, grad_psi, grad_c, grad_u,
                             grad_phiout, grad_psiout, w, sigma, tau, c, dt, hx, hy, NX, NY, u,
                             variant, (cudaStream_t)stream);
}

int ads_scatter_add_f64(double* out, const double* ipt, const int64_t* ii,
                        const double* update, int64_t d, int64_t n, ads_stream_t stream) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(d >= 0 && n >= 0, "negative size");
  ADS_REQUIRE(out && ipt && (n == 0 || (ii && update)), "null pointer argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (int e = copy_if_needed(out, ipt, d, st)) return e;
  if (n == 0) return ADS_OK;
  k_scatter_add<<<(unsigned)div_up(n, 256), 256, 0, st>>>(out, ii, update, d, n);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

int ads_gather_f64(double* out, const double* v, const int64_t* ii, int64_t n,
                   ads_stream_t stream) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(n >= 0, "negative size");
  if (n == 0) return ADS_OK;
  ADS_REQUIRE(out && v && ii, "null pointer argument");
  // GatherOps carries no length for v: only indices below 1 can be rejected.
  k_gather<<<(unsigned)div_up(n, 256), 256, 0, (cudaStream_t)stream>>>(out, v, ii, n,
                                                                        INT64_MAX);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

int ads_add_source_f64(double* out_sxx, double* out_syy, double* out_sxy, double* out_vx,
                       double* out_vy, const double* sxx, const double* syy,
                       const double* sxy, const double* vx, const double* vy,
                       const int64_t* srci, const int64_t* srcj, const int64_t* srctype,
                       int64_t nsrc, int64_t NX, int64_t NY, const double* srcv,
                       ads_stream_t stream) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 1 && NY >= 1 && nsrc >= 0, "invalid sizes");
  ADS_REQUIRE(out_sxx && out_syy && out_sxy && out_vx && out_vy && sxx && syy && sxy && vx &&
                  vy && (nsrc == 0 || (srci && srcj && srctype && srcv)),
              "null pointer argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t N = (NX + 2) * (NY + 2);
  double* o[5] = {out_sxx, out_syy, out_sxy, out_vx, out_vy};
  const double* in[5] = {sxx, syy, sxy, vx, vy};
  for (int f = 0; f < 5; f++)
    if (int e = copy_if_needed(o[f], in[f], N, st)) return e;
  if (nsrc == 0) return ADS_OK;
  Five F{{out_sxx, out_syy, out_sxy, out_vx, out_vy}};
  k_add_source<<<(unsigned)div_up(nsrc, 128), 128, 0, st>>>(F, srci, srcj, srctype, srcv,
                                                             nsrc, NX, NY);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

int ads_add_source_bwd_f64(double* g_sxx, double* g_syy, double* g_sxy, double* g_vx,
                           double* g_vy, double* grad_srcv, const double* gout_sxx,
                           const double* gout_syy, const double* gout_sxy,
                           const double* gout_vx, const double* gout_vy,
                           const int64_t* srci, const int64_t* srcj,
                           const int64_t* srctype, int64_t nsrc, int64_t NX, int64_t NY,
                           ads_stream_t stream) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 1 && NY >= 1 && nsrc >= 0, "invalid sizes");
  ADS_REQUIRE(g_sxx && g_syy && g_sxy && g_vx && g_vy && gout_sxx && gout_syy && gout_sxy &&
                  gout_vx && gout_vy && (nsrc == 0 || (srci && srcj && srctype && grad_srcv)),
              "null pointer argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t N = (NX + 2) * (NY + 2);
  double* o[5] = {g_sxx, g_syy, g_sxy, g_vx, g_vy};
  const double* in[5] = {gout_sxx, gout_syy, gout_sxy, gout_vx, gout_vy};
  for (int f = 0; f < 5; f++)
    if (int e = copy_if_needed(o[f], in[f], N, st)) return e;
  if (nsrc == 0) return ADS_OK;
  CFive G{{gout_sxx, gout_syy, gout_sxy, gout_vx, gout_vy}};
  k_add_source_grad<<<(unsigned)div_up(nsrc, 128), 128, 0, st>>>(G, grad_srcv, srci, srcj,
                                                                  srctype, nsrc, NX, NY);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

int ads_get_receive_f64(double* out, const double* vx, const double* vy, const double* sxx,
                        const double* syy, const double* sxy, int64_t nt,
                        const int64_t* rcvi, const int64_t* rcvj, const int64_t* rcvtype,
                        int64_t nrcv, int64_t NX, int64_t NY, ads_stream_t stream) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 1 && NY >= 1 && nt >= 0 && nrcv >= 0 && nrcv < 65536,
              "invalid sizes (nrcv must be < 65536)");
  if (nt == 0 || nrcv == 0) return ADS_OK;
  ADS_REQUIRE(out && vx && vy && sxx && syy && sxy && rcvi && rcvj && rcvtype,
              "null pointer argument");
  CFive F{{vx, vy, sxx, syy, sxy}};
  dim3 grd((unsigned)std::min<int64_t>(div_up(nt, 128), 64), (unsigned)nrcv);
  k_get_receive<<<grd, 128, 0, (cudaStream_t)stream>>>(out, F, nt, rcvi, rcvj, rcvtype, nrcv,
                                                       NX, NY);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

int ads_get_receive_bwd_f64(double* g_vx, double* g_vy, double* g_sxx, double* g_syy,
                            double* g_sxy, const double* gout, int64_t nt,
                            const int64_t* rcvi, const int64_t* rcvj,
                            const int64_t* rcvtype, int64_t nrcv, int64_t NX, int64_t NY,
                            ads_stream_t stream) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 1 && NY >= 1 && nt >= 0 && nrcv >= 0 && nrcv < 65536, "invalid sizes");
  ADS_REQUIRE(g_vx && g_vy && g_sxx && g_syy && g_sxy, "null pointer argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = nt * (NX + 2) * (NY + 2);
  double* g[5] = {g_vx, g_vy, g_sxx, g_syy, g_sxy};
  for (int f = 0; f < 5; f++) {
    if (n == 0) break;
    k_zero<<<(unsigned)std::min<int64_t>(div_up(n, 256), 8192), 256, 0, st>>>(g[f], n);
    ADS_LAUNCHED(1);
  }
  if (nt == 0 || nrcv == 0) return ADS_OK;
  ADS_REQUIRE(gout && rcvi && rcvj && rcvtype, "null pointer argument");
  Five G{{g_vx, g_vy, g_sxx, g_syy, g_sxy}};
  dim3 grd((unsigned)std::min<int64_t>(div_up(nt, 128), 64), (unsigned)nrcv);
  k_get_receive_grad<<<grd, 128, 0, st>>>(G, gout, nt, rcvi, rcvj, rcvtype, nrcv, NX, NY);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

// Reads (and optionally clears) the device-side flags of rejected indices
// (bit 0 scatter, bit 1 source, bit 2 receiver).  Synchronises the device.
int ads_device_index_errors(int clear, int* flags) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(flags, "null output");
  ADS_CUDA(cudaDeviceSynchronize());
  ADS_CUDA(cudaMemcpyFromSymbol(flags, g_bad_index, sizeof(int)));
  if (clear) {
    int z = 0;
    ADS_CUDA(cudaMemcpyToSymbol(g_bad_index, &z, sizeof(int)));
  }
  return ADS_OK;
}

}  // extern "C"
