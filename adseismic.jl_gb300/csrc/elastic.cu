// elastic.cu -- 2D isotropic elastic velocity-stress step with CPML memory
// variables (src/Core.jl:96-228, profiles :231-407), its exact transpose, and
// whole-path multi-shot forward / misfit / gradient w.r.t. lambda, mu, rho.
//
// The reference composes one step from ~50 gather/scatter custom ops per step
// (fw1..fw4 + add_source).  Here the single-step operators are two kernels
// (stresses: fw1+fw2; velocities: fw3+fw4, one thread per cell) and their
// transpose three; the plans step with one fused row-streaming kernel plus a
// tiny source/receiver launch, and run each adjoint step as one fused
// row-streaming kernel (FP32 plans; FP64 plans by default, and any plan on
// request, as three gather-form row-streaming kernels).  In the plans, per-cell
// work on the eight memory
// variables only runs where the 1D CPML profile is active (a != 0 or b != 1);
// elsewhere the forward memory stays exactly zero and its adjoint never
// reaches a gradient (it is multiplied by a = 0), so skipping it changes no
// result.
//
// Cell indexing: (i, j) -> i*P + j + OFF (P = NY+2, OFF = 0 for the
// single-step operators; pitched layout for the plans).
#include <algorithm>
#include <cmath>
#include <memory>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <vector>

#include "ads_internal.h"

namespace ads {
namespace {

enum { VX = 0, VY = 1, SXX = 2, SYY = 3, SXY = 4, M1 = 5 };  // mem k at M1 + k - 1
constexpr int NF = 13;
// temporaries of the adjoint
enum { D1 = 0, D2, D3, D4, D5, D6, D7, D8, R4, GL1, GM1, GM2, NTMP };
// per-step forward store: strains / accelerations the adjoint needs
enum { E1 = 0, E2, E12, A3, A4, NSTORE };

constexpr int BX = 32, BY = 8;

template <typename T>
struct ElModel {
  const T *lam, *mu, *rho;
  const T *axi, *axh, *bxi, *bxh, *ayi, *ayh, *byi, *byh;  // 1D, index I-1 / J-1
  T dt, hx24, hy24;
  T rhx24, rhy24;  // 1 / hx24, 1 / hy24 (FP32 row kernels)
  int NX, NY, OFF, pad;
  int64_t P;
};

template <typename T>
struct ElShot {
  const T* fin[NF];  // single-step operators: step input state
  T* f[NF];          // single-step operators: step output state; plans: state
                     // buffer 0 (buffer 1 follows at f[0] + NF * fs)
  T* g[NF];          // adjoint state (in place)
  T* tmp[NTMP];
  T* store;          // K slots x NSTORE fields
  T* ckpt;           // nseg x NF fields
  double *glam, *gmu, *grho;
  float *gl32, *gm32, *gr32;  // FP32 plans: per-segment partials of glam, gmu, grho
  T *traces, *resid;            // (nrcv, NSTEP+1)
  const T* srcv;                // (NSTEP, nsrc)
  const int64_t* src_cell;      // pitched cell offsets
  const int* src_type;
  const int64_t* rcv_cell;
  T* const* src_ptr;   // per source: its cell in the state (nullptr: type ignored)
  const int* src_dual;  // per source: 1 if no stencil updates its cell
  T* const* rcv_ptr;   // per receiver: its cell in the state (nullptr: records 0)
  T* const* rcv_gptr;  // per receiver: its cell in the adjoint state
  T* const* src_gptr;  // per source: its cell in the adjoint state (source gradients)
  double* gsrc;        // d loss / d srcv, (NSTEP, nsrc) FP64 (source gradients)
  const int* rcv_type;
  int nsrc, nrcv;
  int64_t fs;                   // elements per field
};

template <typename T>
__device__ __forceinline__ T d4(T a0, T am1, T ap1, T am2, T h24) {
  return (T(27) * a0 - T(27) * am1 - ap1 + am2) / h24;
}

#define ELIDX(ii, jj) ((int64_t)(ii) * M.P + (jj) + M.OFF)

// Stress update (fw1: sxx, syy, m1, m2; fw2: sxy, m3, m4) of the single-step
// operator: every cell is written (out of place), the memory variables in full.
template <typename T, bool STORE>
__global__ void __launch_bounds__(BX* BY)
k_el_stress(ElModel<T> M, ElShot<T> one, int store_slot) {
  const ElShot<T>& sh = one;
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  const int NX = M.NX, NY = M.NY;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t x = ELIDX(i, j);
  const bool b1 = i >= 1 && i <= NX - 1 && j >= 2 && j <= NY;
  const bool b2 = i >= 2 && i <= NX && j >= 1 && j <= NY - 1;
  const T* vx = sh.fin[VX];
  const T* vy = sh.fin[VY];
  T* st = STORE ? sh.store + (int64_t)store_slot * NSTORE * sh.fs : nullptr;
  if (b1) {
    const T lam_ = T(0.5) * (M.lam[ELIDX(i + 1, j)] + M.lam[x]);
    const T mu_ = T(0.5) * (M.mu[ELIDX(i + 1, j)] + M.mu[x]);
    const T lm = lam_ + T(2) * mu_;
    const T dvx = d4<T>(vx[ELIDX(i + 1, j)], vx[x], vx[ELIDX(i + 2, j)], vx[ELIDX(i - 1, j)],
                        M.hx24);
    const T dvy = d4<T>(vy[x], vy[ELIDX(i, j - 1)], vy[ELIDX(i, j + 1)], vy[ELIDX(i, j - 2)],
                        M.hy24);
    const T m1 = M.bxh[i - 1] * sh.fin[M1 + 0][x] + M.axh[i - 1] * dvx;
    sh.f[M1 + 0][x] = m1;
    const T m2 = M.byi[j - 1] * sh.fin[M1 + 1][x] + M.ayi[j - 1] * dvy;
    sh.f[M1 + 1][x] = m2;
    const T e1 = dvx + m1, e2 = dvy + m2;
    sh.f[SXX][x] = sh.fin[SXX][x] + (lm * e1 + lam_ * e2) * M.dt;
    sh.f[SYY][x] = sh.fin[SYY][x] + (lm * e2 + lam_ * e1) * M.dt;
    if (STORE) {
      st[E1 * sh.fs + x] = e1;
      st[E2 * sh.fs + x] = e2;
    }
  } else {
    sh.f[SXX][x] = sh.fin[SXX][x];
    sh.f[SYY][x] = sh.fin[SYY][x];
    sh.f[M1 + 0][x] = T(0);
    sh.f[M1 + 1][x] = T(0);
  }
  if (b2) {
    const T mu_ = T(0.5) * (M.mu[x] + M.mu[ELIDX(i, j + 1)]);
    const T dvydx = d4<T>(vy[x], vy[ELIDX(i - 1, j)], vy[ELIDX(i + 1, j)], vy[ELIDX(i - 2, j)],
                          M.hx24);
    const T dvxdy = d4<T>(vx[ELIDX(i, j + 1)], vx[x], vx[ELIDX(i, j + 2)], vx[ELIDX(i, j - 1)],
                          M.hy24);
    const T m3 = M.bxi[i - 1] * sh.fin[M1 + 2][x] + M.axi[i - 1] * dvydx;
    sh.f[M1 + 2][x] = m3;
    const T m4 = M.byh[j - 1] * sh.fin[M1 + 3][x] + M.ayh[j - 1] * dvxdy;
    sh.f[M1 + 3][x] = m4;
    const T e12 = (dvydx + m3) + (dvxdy + m4);
    sh.f[SXY][x] = sh.fin[SXY][x] + mu_ * e12 * M.dt;
    if (STORE) st[E12 * sh.fs + x] = e12;
  } else {
    sh.f[SXY][x] = sh.fin[SXY][x];
    sh.f[M1 + 2][x] = T(0);
    sh.f[M1 + 3][x] = T(0);
  }
}

// Velocity update (fw3: vx, m5, m6 from the new sxx, sxy; fw4: vy, m7, m8
// from the new sxy, syy).
template <typename T, bool STORE>
__global__ void __launch_bounds__(BX* BY)
k_el_velocity(ElModel<T> M, ElShot<T> one, int store_slot) {
  const ElShot<T>& sh = one;
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  const int NX = M.NX, NY = M.NY;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t x = ELIDX(i, j);
  const bool b3 = i >= 2 && i <= NX && j >= 2 && j <= NY;
  const bool b4 = i >= 1 && i <= NX - 1 && j >= 1 && j <= NY - 1;
  const T* sxx = sh.f[SXX];
  const T* syy = sh.f[SYY];
  const T* sxy = sh.f[SXY];
  T* st = STORE ? sh.store + (int64_t)store_slot * NSTORE * sh.fs : nullptr;
  if (b3) {
    const T a = d4<T>(sxx[x], sxx[ELIDX(i - 1, j)], sxx[ELIDX(i + 1, j)], sxx[ELIDX(i - 2, j)],
                      M.hx24);
    const T b = d4<T>(sxy[x], sxy[ELIDX(i, j - 1)], sxy[ELIDX(i, j + 1)], sxy[ELIDX(i, j - 2)],
                      M.hy24);
    const T m5 = M.bxi[i - 1] * sh.fin[M1 + 4][x] + M.axi[i - 1] * a;
    sh.f[M1 + 4][x] = m5;
    const T m6 = M.byi[j - 1] * sh.fin[M1 + 5][x] + M.ayi[j - 1] * b;
    sh.f[M1 + 5][x] = m6;
    const T e3 = (a + m5) + (b + m6);
    sh.f[VX][x] = sh.fin[VX][x] + e3 * M.dt / M.rho[x];
    if (STORE) st[A3 * sh.fs + x] = e3;
  } else {
    sh.f[VX][x] = sh.fin[VX][x];
    sh.f[M1 + 4][x] = T(0);
    sh.f[M1 + 5][x] = T(0);
  }
  if (b4) {
    const T rho_ = T(0.25) * (M.rho[x] + M.rho[ELIDX(i + 1, j)] + M.rho[ELIDX(i + 1, j + 1)] +
                              M.rho[ELIDX(i, j + 1)]);
    const T a = d4<T>(sxy[ELIDX(i + 1, j)], sxy[x], sxy[ELIDX(i + 2, j)], sxy[ELIDX(i - 1, j)],
                      M.hx24);
    const T b = d4<T>(syy[ELIDX(i, j + 1)], syy[x], syy[ELIDX(i, j + 2)], syy[ELIDX(i, j - 1)],
                      M.hy24);
    const T m7 = M.bxh[i - 1] * sh.fin[M1 + 6][x] + M.axh[i - 1] * a;
    sh.f[M1 + 6][x] = m7;
    const T m8 = M.byh[j - 1] * sh.fin[M1 + 7][x] + M.ayh[j - 1] * b;
    sh.f[M1 + 7][x] = m8;
    const T e4 = (a + m7) + (b + m8);
    sh.f[VY][x] = sh.fin[VY][x] + e4 * M.dt / rho_;
    if (STORE) st[A4 * sh.fs + x] = e4;
  } else {
    sh.f[VY][x] = sh.fin[VY][x];
    sh.f[M1 + 6][x] = T(0);
    sh.f[M1 + 7][x] = T(0);
  }
}

// Adjoint 1 (velocity cells): transposes of fw3 and fw4.  Writes D5..D8 and
// R4, updates the memory adjoints m5..m8 and grho (fw3 part) in place.
template <typename T>
__global__ void __launch_bounds__(BX* BY)
k_el_adj1(ElModel<T> M, ElShot<T> one, int store_slot) {
  const ElShot<T>& sh = one;
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  const int NX = M.NX, NY = M.NY;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t x = ELIDX(i, j);
  const bool b3 = i >= 2 && i <= NX && j >= 2 && j <= NY;
  const bool b4 = i >= 1 && i <= NX - 1 && j >= 1 && j <= NY - 1;
  const T* st = sh.store + (int64_t)store_slot * NSTORE * sh.fs;
  if (b3) {
    const T gv = sh.g[VX][x], r = M.rho[x];
    const T q = gv * M.dt / r;
    T gm5 = q, gm6 = q;
    gm5 += sh.g[M1 + 4][x];
    sh.g[M1 + 4][x] = M.bxi[i - 1] * gm5;
    gm6 += sh.g[M1 + 5][x];
    sh.g[M1 + 5][x] = M.byi[j - 1] * gm6;
    sh.tmp[D5][x] = (q + M.axi[i - 1] * gm5) / M.hx24;
    sh.tmp[D6][x] = (q + M.ayi[j - 1] * gm6) / M.hy24;
    sh.grho[x] += (double)(-gv * st[A3 * sh.fs + x] * M.dt / (r * r));
  } else {
    sh.g[M1 + 4][x] = T(0);
    sh.g[M1 + 5][x] = T(0);
  }
  if (b4) {
    const T gv = sh.g[VY][x];
    const T rho_ = T(0.25) * (M.rho[x] + M.rho[ELIDX(i + 1, j)] + M.rho[ELIDX(i + 1, j + 1)] +
                              M.rho[ELIDX(i, j + 1)]);
    const T q = gv * M.dt / rho_;
    T gm7 = q, gm8 = q;
    gm7 += sh.g[M1 + 6][x];
    sh.g[M1 + 6][x] = M.bxh[i - 1] * gm7;
    gm8 += sh.g[M1 + 7][x];
    sh.g[M1 + 7][x] = M.byh[j - 1] * gm8;
    sh.tmp[D7][x] = (q + M.axh[i - 1] * gm7) / M.hx24;
    sh.tmp[D8][x] = (q + M.ayh[j - 1] * gm8) / M.hy24;
    sh.tmp[R4][x] = -gv * st[A4 * sh.fs + x] * M.dt / (rho_ * rho_) * T(0.25);
  } else {
    sh.g[M1 + 6][x] = T(0);
    sh.g[M1 + 7][x] = T(0);
  }
}

template <typename T>
__device__ __forceinline__ T tld(const T* a, const ElModel<T>& M, int i, int j) {
  return (i >= 0 && i <= M.NX + 1 && j >= 0 && j <= M.NY + 1) ? a[ELIDX(i, j)] : T(0);
}

// Adjoint 2 (stress cells): gather D5..D8 into the stress adjoints, then the
// transposes of fw1 and fw2 (D1..D4, memory adjoints m1..m4, lambda/mu parts).
template <typename T>
__global__ void __launch_bounds__(BX* BY)
k_el_adj2(ElModel<T> M, ElShot<T> one, int store_slot) {
  const ElShot<T>& sh = one;
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  const int NX = M.NX, NY = M.NY;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t x = ELIDX(i, j);
  const bool b1 = i >= 1 && i <= NX - 1 && j >= 2 && j <= NY;
  const bool b2 = i >= 2 && i <= NX && j >= 1 && j <= NY - 1;
  const T* const* D = sh.tmp;
  const T gsxx = sh.g[SXX][x] + T(27) * D[D5][x] - T(27) * tld(D[D5], M, i + 1, j) -
                 tld(D[D5], M, i - 1, j) + tld(D[D5], M, i + 2, j);
  const T gsxy = sh.g[SXY][x] + T(27) * D[D6][x] - T(27) * tld(D[D6], M, i, j + 1) -
                 tld(D[D6], M, i, j - 1) + tld(D[D6], M, i, j + 2) +
                 T(27) * tld(D[D7], M, i - 1, j) - T(27) * D[D7][x] -
                 tld(D[D7], M, i - 2, j) + tld(D[D7], M, i + 1, j);
  const T gsyy = sh.g[SYY][x] + T(27) * tld(D[D8], M, i, j - 1) - T(27) * D[D8][x] -
                 tld(D[D8], M, i, j - 2) + tld(D[D8], M, i, j + 1);
  sh.g[SXX][x] = gsxx;
  sh.g[SYY][x] = gsyy;
  sh.g[SXY][x] = gsxy;
  const T* st = sh.store + (int64_t)store_slot * NSTORE * sh.fs;
  if (b1) {
    const T lam_ = T(0.5) * (M.lam[ELIDX(i + 1, j)] + M.lam[x]);
    const T mu_ = T(0.5) * (M.mu[ELIDX(i + 1, j)] + M.mu[x]);
    const T lm = lam_ + T(2) * mu_;
    const T e1 = st[E1 * sh.fs + x], e2 = st[E2 * sh.fs + x];
    const T gE1 = M.dt * (lm * gsxx + lam_ * gsyy);
    const T gE2 = M.dt * (lam_ * gsxx + lm * gsyy);
    const T glm = M.dt * (e1 * gsxx + e2 * gsyy);
    const T glam = M.dt * (e2 * gsxx + e1 * gsyy) + glm;
    sh.tmp[GL1][x] = T(0.5) * glam;
    sh.tmp[GM1][x] = glm;  // 0.5 * (2 glm) to each of mu[i], mu[i+1]
    T gm1 = gE1, gm2 = gE2;
    gm1 += sh.g[M1 + 0][x];
    sh.g[M1 + 0][x] = M.bxh[i - 1] * gm1;
    gm2 += sh.g[M1 + 1][x];
    sh.g[M1 + 1][x] = M.byi[j - 1] * gm2;
    sh.tmp[D1][x] = (gE1 + M.axh[i - 1] * gm1) / M.hx24;
    sh.tmp[D2][x] = (gE2 + M.ayi[j - 1] * gm2) / M.hy24;
  } else {
    sh.g[M1 + 0][x] = T(0);
    sh.g[M1 + 1][x] = T(0);
  }
  if (b2) {
    const T mu_ = T(0.5) * (M.mu[x] + M.mu[ELIDX(i, j + 1)]);
    const T q = gsxy * mu_ * M.dt;
    sh.tmp[GM2][x] = gsxy * st[E12 * sh.fs + x] * M.dt * T(0.5);
    T gm3 = q, gm4 = q;
    gm3 += sh.g[M1 + 2][x];
    sh.g[M1 + 2][x] = M.bxi[i - 1] * gm3;
    gm4 += sh.g[M1 + 3][x];
    sh.g[M1 + 3][x] = M.byh[j - 1] * gm4;
    sh.tmp[D3][x] = (q + M.axi[i - 1] * gm3) / M.hx24;
    sh.tmp[D4][x] = (q + M.ayh[j - 1] * gm4) / M.hy24;
  } else {
    sh.g[M1 + 2][x] = T(0);
    sh.g[M1 + 3][x] = T(0);
  }
}

// Adjoint 3 (velocity cells + parameters): gather D1..D4 into the velocity
// adjoints and the lambda / mu / rho partials into the FP64 accumulators.
template <typename T>
__global__ void __launch_bounds__(BX* BY)
k_el_adj3(ElModel<T> M, ElShot<T> one) {
  const ElShot<T>& sh = one;
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  const int NX = M.NX, NY = M.NY;
  if (i > NX + 1 || j > NY + 1) return;
  const int64_t x = ELIDX(i, j);
  const T* const* D = sh.tmp;
  sh.g[VX][x] += T(27) * tld(D[D1], M, i - 1, j) - T(27) * D[D1][x] -
                 tld(D[D1], M, i - 2, j) + tld(D[D1], M, i + 1, j) +
                 T(27) * tld(D[D4], M, i, j - 1) - T(27) * D[D4][x] -
                 tld(D[D4], M, i, j - 2) + tld(D[D4], M, i, j + 1);
  sh.g[VY][x] += T(27) * D[D2][x] - T(27) * tld(D[D2], M, i, j + 1) -
                 tld(D[D2], M, i, j - 1) + tld(D[D2], M, i, j + 2) + T(27) * D[D3][x] -
                 T(27) * tld(D[D3], M, i + 1, j) - tld(D[D3], M, i - 1, j) +
                 tld(D[D3], M, i + 2, j);
  if (i >= 1 && i <= NX && j >= 1 && j <= NY) {
    sh.glam[x] += (double)(D[GL1][x] + tld(D[GL1], M, i - 1, j));
    sh.gmu[x] += (double)(D[GM1][x] + tld(D[GM1], M, i - 1, j) + D[GM2][x] +
                          tld(D[GM2], M, i, j - 1));
    sh.grho[x] += (double)(D[R4][x] + tld(D[R4], M, i - 1, j) + tld(D[R4], M, i - 1, j - 1) +
                           tld(D[R4], M, i, j - 1));
  }
}

#undef ELIDX

// ---------------------------------------------------------------------------
// Row-streaming kernels for the plans (the fused forward step and the three
// adjoint passes).
//
// A warp owns a strip of rows of one shot, two adjacent columns per lane
// (loaded as one 8/16-byte vector), and walks down its rows: the
// i-neighbours of the 4th-order stencils sit in register windows whose next
// row is loaded one iteration ahead, the j-neighbours (up to two columns
// away) come from the neighbouring lanes.  In the adjoint passes lanes 0 and
// 31 only supply those neighbours: lanes 1..30 update ESTRIP = 60 columns and
// consecutive strips overlap by two columns on each side.  Cells outside the
// update boxes are neither computed nor written.
// ---------------------------------------------------------------------------
constexpr int EC = 2;             // columns per lane
constexpr int ESTRIP = 30 * EC;   // columns an adjoint strip updates
constexpr int EW = 4;             // warps per CTA (independent strips)
constexpr int kTuneMinRows = 6;   // smallest adjoint strip height the autotuner tries
constexpr int kTuneMinRowsF = 12; // smallest fused-step tile height it tries
// Which adjoint passes launch as two concurrent halves (measured: the first
// gains occupancy from it; the gather-heavy second and third do better whole).
#ifndef ADS_EL_SPLIT_ADJ23
#define ADS_EL_SPLIT_ADJ23 0
#endif
constexpr bool kSplitAdj1 = true, kSplitAdj23 = ADS_EL_SPLIT_ADJ23 != 0;
#ifndef ADS_EL_MINB
#define ADS_EL_MINB 6                 // resident CTAs per SM, first adjoint pass (CPML items)
#endif
#ifndef ADS_EL_MINB_ADJ
#define ADS_EL_MINB_ADJ 4             // the same for the two gather-heavy adjoint kernels
#endif
template <typename T>
constexpr int el_minb() { return sizeof(T) == 4 ? ADS_EL_MINB : 2; }
template <typename T>
constexpr int el_minb_adj() { return sizeof(T) == 4 ? ADS_EL_MINB_ADJ : 2; }
#ifndef ADS_EL_MINB_INT
#define ADS_EL_MINB_INT 6             // the same for CPML-free items (no memory variables)
#endif
template <typename T>
constexpr int el_minb_int() { return sizeof(T) == 4 ? ADS_EL_MINB_INT : 2; }

template <typename T>
struct alignas(2 * sizeof(T)) V2 {
  T v[2];
};

// Both cells of a lane as one predicated vector load (zeros where `on` is
// false), so a mask that differs between the lanes of a warp costs no
// branch.  The asm has no memory clobber: the row kernels load each cell at
// most once, and a cell they also write is written later from values that
// depend on the load.
__device__ __forceinline__ V2<float> ld2p(const float* p, int64_t o, bool on) {
  float a = 0.f, b = 0.f;
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %3, 0;\n\t@q ld.global.v2.f32 {%0, %1}, [%2];\n\t}"
      : "+f"(a), "+f"(b)
      : "l"(p + o), "r"((unsigned)on));
  V2<float> x;
  x.v[0] = a;
  x.v[1] = b;
  return x;
}
// 32-bit offsets (within one field of one shot) let the address be formed in
// one wide multiply-add
__device__ __forceinline__ V2<float> ld2p(const float* p, int o, bool on) {
  float a = 0.f, b = 0.f;
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %3, 0;\n\t@q ld.global.v2.f32 {%0, %1}, [%2];\n\t}"
      : "+f"(a), "+f"(b)
      : "l"(p + o), "r"((unsigned)on));
  V2<float> x;
  x.v[0] = a;
  x.v[1] = b;
  return x;
}
__device__ __forceinline__ V2<double> ld2p(const double* p, int o, bool on) {
  double a = 0.0, b = 0.0;
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %3, 0;\n\t@q ld.global.v2.f64 {%0, %1}, [%2];\n\t}"
      : "+d"(a), "+d"(b)
      : "l"(p + o), "r"((unsigned)on));
  V2<double> x;
  x.v[0] = a;
  x.v[1] = b;
  return x;
}
__device__ __forceinline__ V2<double> ld2p(const double* p, int64_t o, bool on) {
  double a = 0.0, b = 0.0;
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %3, 0;\n\t@q ld.global.v2.f64 {%0, %1}, [%2];\n\t}"
      : "+d"(a), "+d"(b)
      : "l"(p + o), "r"((unsigned)on));
  V2<double> x;
  x.v[0] = a;
  x.v[1] = b;
  return x;
}

// Store the two cells of a lane, each only where its flag is set, as three
// independent guarded stores (a vector store when both cells are written,
// else the single cell).
template <typename T, typename I = int64_t>
__device__ __forceinline__ void st2p(T* p, I o, const T (&x)[2], bool k0, bool k1) {
  if (k0 && k1) {
    V2<T> y;
    y.v[0] = x[0];
    y.v[1] = x[1];
    *reinterpret_cast<V2<T>*>(p + o) = y;
  }
  if (k0 && !k1) p[o] = x[0];
  if (k1 && !k0) p[o + 1] = x[1];
}

// Two guarded scalar stores: for store masks that differ between the lanes
// of a warp (columns at a box edge), where the vector form diverges.
template <typename T, typename I = int64_t>
__device__ __forceinline__ void st2s(T* p, I o, const T (&x)[2], bool k0, bool k1) {
  if (k0) p[o] = x[0];
  if (k1) p[o + 1] = x[1];
}

__device__ __forceinline__ float shup(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ double shup(double v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ float shdn(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ double shdn(double v) { return __shfl_down_sync(0xffffffffu, v, 1); }

// Geometry of one warp's strip: columns j, j+1 of this lane, rows [i0, i_end)
// (all inside 1..NX), whether the lane updates its cells, and the guarded
// row loader.
template <typename T>
struct Strip {
  int lane, j, i0, i_end, NX, NY;
  bool out;
  int64_t P;
  __device__ Strip(const ElModel<T>& M, int ncolw, int R, int wi) {
    lane = threadIdx.x & 31;
    NX = M.NX;
    NY = M.NY;
    P = M.P;
    const int strip = wi % ncolw, rt = wi / ncolw;
    j = strip * ESTRIP - 1 + lane * EC;  // odd: 8/16-byte aligned pairs
    out = lane >= 1 && lane <= 30;
    i0 = 1 + rt * R;
    i_end = min(i0 + R, NX + 1);
  }
  __device__ int64_t off(int r) const { return (int64_t)r * P + j + JOFF; }
  // both cells of this lane at row r (zeros outside the padded grid)
  __device__ V2<T> row(const T* p, int r) const {
    return ld2p(p, off(r), j <= NY + 1 && r >= 0 && r <= NX + 1);
  }
};

// FP32 row kernels multiply by 1 / (24 h) and divide by the density with the
// fast reciprocal (within 2 ulp); FP64 keeps the exact divisions.
template <typename T>
__device__ __forceinline__ T d4r(T a0, T am1, T ap1, T am2, T h24, T rh24) {
  if constexpr (sizeof(T) == 4) {
    return (T(27) * a0 - T(27) * am1 - ap1 + am2) * rh24;
  } else {
    return (T(27) * a0 - T(27) * am1 - ap1 + am2) / h24;
  }
}

template <typename T>
__device__ __forceinline__ T divr(T a, T b) {
  if constexpr (sizeof(T) == 4) {
    return __fdividef(a, b);
  } else {
    return a / b;
  }
}

// y-profile coefficients of a lane's two columns (integer and half grid) and
// whether the memory variable they drive is active there.
template <typename T>
struct ColProf {
  T ai[2], bi[2], ah[2], bh[2];
  bool acti[2], acth[2];
  __device__ ColProf(const ElModel<T>& M, int j) {
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const int jc = j + c;
      const bool in = jc >= 1 && jc <= M.NY;
      ai[c] = in ? M.ayi[jc - 1] : T(0);
      bi[c] = in ? M.byi[jc - 1] : T(1);
      ah[c] = in ? M.ayh[jc - 1] : T(0);
      bh[c] = in ? M.byh[jc - 1] : T(1);
      acti[c] = in && (ai[c] != T(0) || bi[c] != T(1));
      acth[c] = in && (ah[c] != T(0) || bh[c] != T(1));
    }
  }
};

// ---------------------------------------------------------------------------
// Fused forward step (fw1..fw4) for the plans: one pass over the fields
// instead of two.  The state alternates between two buffers: step n reads
// slot n-1 from buffer (n-1) & 1 and writes slot n into buffer n & 1, so a
// warp can update the velocities of its rows right after the stresses they
// need while the neighbouring strips and row tiles still read the old fields
// for their own edge stresses.
//
// A warp computes the new stresses of lanes 1..30 on rows i0-2 .. i_end+1
// (one lane and two rows more on each side than it owns) and the new
// velocities of lanes 2..29 on rows i0 .. i_end-1, two rows behind the stress
// row.  It stores what it owns (lanes 2..29, rows i0 .. i_end-1): a strip
// updates FSTRIP = 56 columns.  The arithmetic and its order are those of
// k_el_stress / k_el_velocity.
//
// Cells outside a field's update box are never written: both buffers hold the
// same value there (sources on such cells are added to both buffers and
// checkpoints are restored into both), and that value is what the step
// leaves there.  Out-of-box stresses enter the velocity update with that
// value, as when the step updates the fields in place.
// ---------------------------------------------------------------------------
constexpr int FSTRIP = 28 * EC;
#ifndef ADS_EL_STEP_LAG
#define ADS_EL_STEP_LAG 2             // rows the velocity half of the fused step runs behind
#endif
constexpr int kStepLag = ADS_EL_STEP_LAG;
static_assert(kStepLag == 2 || kStepLag == 3, "the fused step lags its velocities 2 or 3 rows");
#ifndef ADS_EL_MINB_F
#define ADS_EL_MINB_F 3               // resident CTAs per SM, fused kernel of corner items
#endif
#ifndef ADS_EL_MINB_FR
#define ADS_EL_MINB_FR 4              // the same for items with only row or only column logic
#endif
#ifndef ADS_EL_MINB_FI
#define ADS_EL_MINB_FI 5              // the same for CPML-free items
#endif
template <typename T, int KIND>
constexpr int el_minb_step() {
  return sizeof(T) != 4 ? 2 : KIND == 0 ? ADS_EL_MINB_FI : KIND == 3 ? ADS_EL_MINB_F : ADS_EL_MINB_FR;
}

template <typename T, bool STORE, int KIND>
__global__ void __launch_bounds__(EW * 32, el_minb_step<T, KIND>())
k_el_step_rows(ElModel<T> M, const ElShot<T>* __restrict__ shots, const int* __restrict__ wlist,
               int ncolw, int R, int nwt, int store_slot, int pin, int jsh, int ish) {
  // KIND bit 0: rows need the box edge and x-profile logic; bit 1: columns
  // need the box edge and y-profile logic (0: neither, CPML-free interior)
  constexpr bool GR = (KIND & 1) != 0, GC = (KIND & 2) != 0;
  const int wl = blockIdx.x * EW + (threadIdx.x >> 5);
  if (wl >= nwt) return;
  const int wi = wlist[wl];  // the warp's (strip, row tile)
  const ElShot<T>& sh = shots[blockIdx.y];
  const int lane = threadIdx.x & 31, NX = M.NX, NY = M.NY;
  const int strip = wi % ncolw, rt = wi / ncolw;
  // strips and row tiles start jsh columns (even, <= 0) and ish rows (<= 0)
  // before column and row 1
  const int j = strip * FSTRIP - 3 + lane * EC + jsh;  // odd: 8/16-byte aligned pairs
  const bool own = lane >= 2 && lane <= 29;
  const bool colok = j >= -1 && j <= NY + 1;
  const int i0r = 1 + ish + rt * R;
  const int i0 = max(i0r, 1), i_end = min(i0r + R, NX + 1);
  const int64_t fs = sh.fs, P = M.P;
  const int64_t bin = (int64_t)pin * NF * fs, bout = (int64_t)(1 - pin) * NF * fs;
  // offsets within a field fit 32 bits (the plan checks (NX + 2) * P < 2^31)
  const int P32 = (int)P, col = j + JOFF;
  const T* __restrict__ vx = sh.f[VX] + bin;
  const T* __restrict__ vy = sh.f[VY] + bin;
  const T* __restrict__ sxx = sh.f[SXX] + bin;
  const T* __restrict__ syy = sh.f[SYY] + bin;
  const T* __restrict__ sxy = sh.f[SXY] + bin;
  T* __restrict__ vxo = sh.f[VX] + bout;
  T* __restrict__ vyo = sh.f[VY] + bout;
  T* __restrict__ sxxo = sh.f[SXX] + bout;
  T* __restrict__ syyo = sh.f[SYY] + bout;
  T* __restrict__ sxyo = sh.f[SXY] + bout;
  T* __restrict__ st = STORE ? sh.store + (int64_t)store_slot * NSTORE * fs : nullptr;
  // stores of a lane's two cells: lane-dependent masks (column logic) use
  // scalar stores
  auto stw = [&](T* p, int o, const T (&x)[2], bool k0, bool k1) {
    if constexpr (GC) {
      st2s<T>(p, o, x, k0, k1);
    } else {
      st2p(p, o, x, k0, k1);
    }
  };
  auto ld = [&](const T* p, int r) { return ld2p(p, r * P32 + col, colok && r >= 0 && r <= NX + 1); };
  // memory variables 1..8 of the input / output buffer
  const T* __restrict__ m1i = sh.f[M1 + 0] + bin;
  const T* __restrict__ m2i = sh.f[M1 + 1] + bin;
  const T* __restrict__ m3i = sh.f[M1 + 2] + bin;
  const T* __restrict__ m4i = sh.f[M1 + 3] + bin;
  const T* __restrict__ m5i = sh.f[M1 + 4] + bin;
  const T* __restrict__ m6i = sh.f[M1 + 5] + bin;
  const T* __restrict__ m7i = sh.f[M1 + 6] + bin;
  const T* __restrict__ m8i = sh.f[M1 + 7] + bin;
  T* __restrict__ m1o = sh.f[M1 + 0] + bout;
  T* __restrict__ m2o = sh.f[M1 + 1] + bout;
  T* __restrict__ m3o = sh.f[M1 + 2] + bout;
  T* __restrict__ m4o = sh.f[M1 + 3] + bout;
  T* __restrict__ m5o = sh.f[M1 + 4] + bout;
  T* __restrict__ m6o = sh.f[M1 + 5] + bout;
  T* __restrict__ m7o = sh.f[M1 + 6] + bout;
  T* __restrict__ m8o = sh.f[M1 + 7] + bout;
  const ColProf<T> Y(M, j);
  bool cA[2], cB[2];  // columns of the fw1 / fw3 boxes (2..NY) and the fw2 / fw4 boxes (1..NY-1)
#pragma unroll
  for (int c = 0; c < 2; c++) {
    cA[c] = !GC || (j + c >= 2 && j + c <= NY);
    cB[c] = !GC || (j + c >= 1 && j + c <= NY - 1);
  }
  // lanes whose columns carry memory variables (in a box).  The y-profile
  // memory variables are updated in every box cell of a strip with column
  // logic: where the profile is inactive (a = 0, b = 1) the update
  // b * m + a * d gives exactly +0, the value such cells always hold, so no
  // per-lane profile test is needed.
  const bool lA = cA[0] || cA[1], lB = cB[0] || cB[1];
  const bool lAi = GC && lA, lBh = GC && lB;
  // row parts of the boxes: stress rows (fw1: 1..NX-1, fw2: 2..NX) and
  // velocity rows r = s - VL (fw3: 2..NX, fw4: 1..NX-1)
  constexpr int VL = kStepLag;
  auto rs1 = [&](int s) { return !GR || (s >= 1 && s <= NX - 1); };
  auto rs2 = [&](int s) { return !GR || (s >= 2 && s <= NX); };
  auto rv3 = [&](int s) { return !GR || s - VL >= 2; };
  auto rv4 = [&](int s) { return !GR || s - VL <= NX - 1; };
  // memory variables m1..m4 of stress row s (onS) and m5..m8 of velocity row
  // s - VL (onV, where they can be nonzero), loaded one iteration ahead
  auto mload = [&](int s, bool onS, bool onV, V2<T> (&m)[8]) {
    const int o = s * P32 + col, q = o - VL * P32;
    const bool vr = onV && own && s >= i0 + VL;
    if constexpr (GR) {
      m[0] = ld2p(m1i, o, onS && rs1(s) && lA);
      m[2] = ld2p(m3i, o, onS && rs2(s) && lB);
      m[4] = ld2p(m5i, q, vr && rv3(s) && lA);
      m[6] = ld2p(m7i, q, vr && rv4(s) && lB);
    }
    if constexpr (GC) {
      m[1] = ld2p(m2i, o, onS && rs1(s) && lAi);
      m[3] = ld2p(m4i, o, onS && rs2(s) && lBh);
      m[5] = ld2p(m6i, q, vr && rv3(s) && lAi);
      m[7] = ld2p(m8i, q, vr && rv4(s) && lBh);
    }
  };
  const int s0 = i0 - 2;
  // windows at stress row s: old vx rows s-VL..s+2 (X[k] = row s-VL+k), old
  // vy rows s-VL..s+1, lam / mu rows s, s+1, old stresses row s, rho rows
  // s-VL, s-VL+1; new sxx rows s-VL-2..s-1 (NA[k] = row s-VL-2+k), new sxy
  // rows s-VL-1..s-1, new syy rows s-VL..s-1.  With VL = 3 the velocities of
  // row s-3 need no stress of row s, so the two halves of an iteration are
  // independent of each other.
  V2<T> X[VL + 3], Yv[VL + 2], NA[VL + 2], NC[VL + 1], NB[VL];
#pragma unroll
  for (int k = 0; k < VL + 3; k++) X[k] = ld(vx, s0 - VL + k);
#pragma unroll
  for (int k = 0; k < VL + 2; k++) Yv[k] = ld(vy, s0 - VL + k);
#pragma unroll
  for (int k = 0; k < VL + 2; k++) NA[k] = V2<T>{};
#pragma unroll
  for (int k = 0; k < VL + 1; k++) NC[k] = V2<T>{};
#pragma unroll
  for (int k = 0; k < VL; k++) NB[k] = V2<T>{};
  V2<T> L0 = ld(M.lam, s0), L1 = ld(M.lam, s0 + 1), U0 = ld(M.mu, s0), U1 = ld(M.mu, s0 + 1);
  V2<T> A0 = ld(sxx, s0), B0 = ld(syy, s0), C0 = ld(sxy, s0);
  V2<T> R0 = ld(M.rho, s0 - VL), R1 = ld(M.rho, s0 - VL + 1);
  V2<T> mm[8] = {};
  mload(s0, true, true, mm);
  for (int s = s0; s <= i_end + VL - 1; s++) {
    const bool doS = s <= i_end + 1;  // stresses of row s this iteration
    const bool more = s <= i_end;     // stresses of row s + 1 next iteration
    const bool vmore = s + 1 - VL <= i_end - 1;  // velocities of row s + 1 - VL next
    const V2<T> X5 = ld(vx, more ? s + 3 : -1), Y4 = ld(vy, more ? s + 2 : -1),
                L2 = ld(M.lam, more ? s + 2 : -1), U2 = ld(M.mu, more ? s + 2 : -1),
                R2 = ld(M.rho, vmore ? s + 2 - VL : -1);
    const V2<T> An = ld(sxx, more ? s + 1 : -1), Bn = ld(syy, more ? s + 1 : -1),
                Cn = ld(sxy, more ? s + 1 : -1);
    V2<T> mn[8] = {};
    mload(s + 1, more, vmore, mn);
    const int o = s * P32 + col, q = o - VL * P32;
    // x profiles of stress row s and velocity row s - VL
    const int sx = min(max(s, 1), NX) - 1, vx_ = min(max(s - VL, 1), NX) - 1;
    const T axh = GR ? M.axh[sx] : T(0), bxh = GR ? M.bxh[sx] : T(1);
    const T axi = GR ? M.axi[sx] : T(0), bxi = GR ? M.bxi[sx] : T(1);
    const T vaxi = GR ? M.axi[vx_] : T(0), vbxi = GR ? M.bxi[vx_] : T(1);
    const T vaxh = GR ? M.axh[vx_] : T(0), vbxh = GR ? M.bxh[vx_] : T(1);
    const bool r1 = doS && rs1(s), r2 = doS && rs2(s);
    const bool rx1 = GR && r1 && (axh != T(0) || bxh != T(1));
    const bool rx3 = GR && r2 && (axi != T(0) || bxi != T(1));
    const bool vrow = s >= i0 + VL;  // velocities of row s - VL this iteration
    const bool r3 = rv3(s), r4 = rv4(s);
    const bool rx5 = GR && vrow && r3 && (vaxi != T(0) || vbxi != T(1));
    const bool rx7 = GR && vrow && r4 && (vaxh != T(0) || vbxh != T(1));
    // ---- new stresses of row s
    const V2<T>& Xs = X[VL];  // old vx row s
    const V2<T>& Ys = Yv[VL];  // old vy row s
    T xr[5], yr[5], ur[3];
    xr[0] = shup(Xs.v[1]);
    xr[1] = Xs.v[0];
    xr[2] = Xs.v[1];
    xr[3] = shdn(Xs.v[0]);
    xr[4] = shdn(Xs.v[1]);
    yr[0] = shup(Ys.v[0]);
    yr[1] = shup(Ys.v[1]);
    yr[2] = Ys.v[0];
    yr[3] = Ys.v[1];
    yr[4] = shdn(Ys.v[0]);
    ur[0] = U0.v[0];
    ur[1] = U0.v[1];
    ur[2] = shdn(U0.v[0]);
    const bool wrow = own && s >= i0 && s < i_end;  // this lane stores row s
    V2<T> NAs, NBs, NCs;
    T e1s[2], e2s[2], e12s[2], m1v[2], m2v[2], m3v[2], m4v[2];
    bool k1[2], k2[2], u1[2], u2[2], u3[2], u4[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
      k1[c] = r1 && cA[c];
      k2[c] = r2 && cB[c];
      // fw1
      const T lam_ = T(0.5) * (L1.v[c] + L0.v[c]);
      const T mu1 = T(0.5) * (U1.v[c] + U0.v[c]);
      const T lm = lam_ + T(2) * mu1;
      const T dvx = d4r<T>(X[VL + 1].v[c], X[VL].v[c], X[VL + 2].v[c], X[VL - 1].v[c], M.hx24,
                           M.rhx24);
      const T dvy = d4r<T>(yr[2 + c], yr[1 + c], yr[3 + c], yr[c], M.hy24, M.rhy24);
      u1[c] = k1[c] && rx1;
      u2[c] = GC && k1[c];
      m1v[c] = u1[c] ? bxh * mm[0].v[c] + axh * dvx : T(0);
      m2v[c] = u2[c] ? Y.bi[c] * mm[1].v[c] + Y.ai[c] * dvy : T(0);
      const T e1 = dvx + m1v[c], e2 = dvy + m2v[c];
      NAs.v[c] = k1[c] ? A0.v[c] + (lm * e1 + lam_ * e2) * M.dt : A0.v[c];
      NBs.v[c] = k1[c] ? B0.v[c] + (lm * e2 + lam_ * e1) * M.dt : B0.v[c];
      e1s[c] = e1;
      e2s[c] = e2;
      // fw2
      const T mu2 = T(0.5) * (ur[c] + ur[c + 1]);
      const T dvydx = d4r<T>(Yv[VL].v[c], Yv[VL - 1].v[c], Yv[VL + 1].v[c], Yv[VL - 2].v[c],
                             M.hx24, M.rhx24);
      const T dvxdy = d4r<T>(xr[2 + c], xr[1 + c], xr[3 + c], xr[c], M.hy24, M.rhy24);
      u3[c] = k2[c] && rx3;
      u4[c] = GC && k2[c];
      m3v[c] = u3[c] ? bxi * mm[2].v[c] + axi * dvydx : T(0);
      m4v[c] = u4[c] ? Y.bh[c] * mm[3].v[c] + Y.ah[c] * dvxdy : T(0);
      const T e12 = (dvydx + m3v[c]) + (dvxdy + m4v[c]);
      NCs.v[c] = k2[c] ? C0.v[c] + mu2 * e12 * M.dt : C0.v[c];
      e12s[c] = e12;
    }
    if (wrow) {
      stw(sxxo, o, NAs.v, k1[0], k1[1]);
      stw(syyo, o, NBs.v, k1[0], k1[1]);
      stw(sxyo, o, NCs.v, k2[0], k2[1]);
      if (STORE) {
        stw(st + E1 * fs, o, e1s, k1[0], k1[1]);
        stw(st + E2 * fs, o, e2s, k1[0], k1[1]);
        stw(st + E12 * fs, o, e12s, k2[0], k2[1]);
      }
      if constexpr (GR) {
        stw(m1o, o, m1v, u1[0], u1[1]);
        stw(m3o, o, m3v, u3[0], u3[1]);
      }
      if constexpr (GC) {
        stw(m2o, o, m2v, u2[0], u2[1]);
        stw(m4o, o, m4v, u4[0], u4[1]);
      }
    }
    // ---- new velocities of row r = s - VL: new sxx rows r-2..r+1, sxy rows
    // r-1..r+2 (the last of them row s itself when VL = 2), syy row r
    if (vrow) {
      const V2<T>& NC1 = NC[1];
      const V2<T>& NCt = VL == 2 ? NCs : NC[VL];  // new sxy row r + 2
      const V2<T>& NBr = NB[0];
      T qr[5], wr[5], r0[3], r1v[3];
      qr[0] = shup(NC1.v[0]);
      qr[1] = shup(NC1.v[1]);
      qr[2] = NC1.v[0];
      qr[3] = NC1.v[1];
      qr[4] = shdn(NC1.v[0]);
      wr[0] = shup(NBr.v[1]);
      wr[1] = NBr.v[0];
      wr[2] = NBr.v[1];
      wr[3] = shdn(NBr.v[0]);
      wr[4] = shdn(NBr.v[1]);
      r0[0] = R0.v[0];
      r0[1] = R0.v[1];
      r0[2] = shdn(R0.v[0]);
      r1v[0] = R1.v[0];
      r1v[1] = R1.v[1];
      r1v[2] = shdn(R1.v[0]);
      T nvx[2], nvy[2], a3s[2], a4s[2], m5v[2], m6v[2], m7v[2], m8v[2];
      bool k3[2], k4[2], u5[2], u6[2], u7[2], u8[2];
#pragma unroll
      for (int c = 0; c < 2; c++) {
        k3[c] = own && r3 && cA[c];
        k4[c] = own && r4 && cB[c];
        // fw3
        const T a = d4r<T>(NA[2].v[c], NA[1].v[c], NA[3].v[c], NA[0].v[c], M.hx24, M.rhx24);
        const T b = d4r<T>(qr[2 + c], qr[1 + c], qr[3 + c], qr[c], M.hy24, M.rhy24);
        u5[c] = k3[c] && rx5;
        u6[c] = GC && k3[c];
        m5v[c] = u5[c] ? vbxi * mm[4].v[c] + vaxi * a : T(0);
        m6v[c] = u6[c] ? Y.bi[c] * mm[5].v[c] + Y.ai[c] * b : T(0);
        const T e3 = (a + m5v[c]) + (b + m6v[c]);
        nvx[c] = X[0].v[c] + divr<T>(e3 * M.dt, r0[c]);
        a3s[c] = e3;
        // fw4
        const T rho_ = T(0.25) * (r0[c] + r1v[c] + r1v[c + 1] + r0[c + 1]);
        const T a4 = d4r<T>(NC[2].v[c], NC[1].v[c], NCt.v[c], NC[0].v[c], M.hx24, M.rhx24);
        const T b4 = d4r<T>(wr[2 + c], wr[1 + c], wr[3 + c], wr[c], M.hy24, M.rhy24);
        u7[c] = k4[c] && rx7;
        u8[c] = GC && k4[c];
        m7v[c] = u7[c] ? vbxh * mm[6].v[c] + vaxh * a4 : T(0);
        m8v[c] = u8[c] ? Y.bh[c] * mm[7].v[c] + Y.ah[c] * b4 : T(0);
        const T e4 = (a4 + m7v[c]) + (b4 + m8v[c]);
        nvy[c] = Yv[0].v[c] + divr<T>(e4 * M.dt, rho_);
        a4s[c] = e4;
      }
      stw(vxo, q, nvx, k3[0], k3[1]);
      stw(vyo, q, nvy, k4[0], k4[1]);
      if (STORE) {
        stw(st + A3 * fs, q, a3s, k3[0], k3[1]);
        stw(st + A4 * fs, q, a4s, k4[0], k4[1]);
      }
      if constexpr (GR) {
        stw(m5o, q, m5v, u5[0], u5[1]);
        stw(m7o, q, m7v, u7[0], u7[1]);
      }
      if constexpr (GC) {
        stw(m6o, q, m6v, u6[0], u6[1]);
        stw(m8o, q, m8v, u8[0], u8[1]);
      }
    }
#pragma unroll
    for (int k = 0; k < VL + 2; k++) X[k] = X[k + 1];
    X[VL + 2] = X5;
#pragma unroll
    for (int k = 0; k < VL + 1; k++) Yv[k] = Yv[k + 1];
    Yv[VL + 1] = Y4;
    L0 = L1; L1 = L2; U0 = U1; U1 = U2;
    A0 = An; B0 = Bn; C0 = Cn;
    R0 = R1; R1 = R2;
#pragma unroll
    for (int k = 0; k < VL + 1; k++) NA[k] = NA[k + 1];
    NA[VL + 1] = NAs;
#pragma unroll
    for (int k = 0; k < VL; k++) NC[k] = NC[k + 1];
    NC[VL] = NCs;
#pragma unroll
    for (int k = 0; k < VL - 1; k++) NB[k] = NB[k + 1];
    NB[VL - 1] = NBs;
#pragma unroll
    for (int k = 0; k < 8; k++) mm[k] = mn[k];
  }
}

// ---------------------------------------------------------------------------
// Row-streaming forms of the three adjoint kernels for the plans (same strips
// as the forward ones).  FP32 plans add the lambda / mu / rho contributions of
// a step to FP32 per-segment partials (flushed into the FP64 accumulators by
// k_el_flush_acc at the end of each checkpoint segment); FP64 plans add to
// the FP64 accumulators directly.
// ---------------------------------------------------------------------------
template <typename T>
struct ElAcc {
  using type = double;
  static __device__ double* lam(const ElShot<T>& sh) { return sh.glam; }
  static __device__ double* mu(const ElShot<T>& sh) { return sh.gmu; }
  static __device__ double* rho(const ElShot<T>& sh) { return sh.grho; }
};
template <>
struct ElAcc<float> {
  using type = float;
  static __device__ float* lam(const ElShot<float>& sh) { return sh.gl32; }
  static __device__ float* mu(const ElShot<float>& sh) { return sh.gm32; }
  static __device__ float* rho(const ElShot<float>& sh) { return sh.gr32; }
};

// x / (24 h): FP32 multiplies by the reciprocal, FP64 divides.
template <typename T>
__device__ __forceinline__ T hdiv(T x, T h24, T rh24) {
  if constexpr (sizeof(T) == 4) {
    return x * rh24;
  } else {
    return x / h24;
  }
}

// Adjoint 1 (velocity cells) of a strip: transposes of fw3 and fw4.
template <typename T, bool INT, int PART>
__global__ void __launch_bounds__(EW * 32, INT ? el_minb_int<T>() : el_minb<T>())
k_el_adj1_rows(ElModel<T> M, const ElShot<T>* __restrict__ shots, const int* __restrict__ wlist,
               int ncolw, int R, int nwt,
               int store_slot) {
  using A = typename ElAcc<T>::type;
  const int wl = blockIdx.x * EW + (threadIdx.x >> 5);
  if (wl >= nwt) return;
  const int wi = wlist[wl];  // the warp's (strip, row tile)
  const ElShot<T>& sh = shots[blockIdx.y];
  const Strip<T> S(M, ncolw, R, wi);
  const int j = S.j, NX = S.NX, NY = S.NY;
  const int64_t fs = sh.fs;
  const T* __restrict__ gvx = sh.g[VX];
  const T* __restrict__ gvy = sh.g[VY];
  T* __restrict__ g5 = sh.g[M1 + 4];
  T* __restrict__ g6 = sh.g[M1 + 5];
  T* __restrict__ g7 = sh.g[M1 + 6];
  T* __restrict__ g8 = sh.g[M1 + 7];
  T* __restrict__ d5 = sh.tmp[D5];
  T* __restrict__ d6 = sh.tmp[D6];
  T* __restrict__ d7 = sh.tmp[D7];
  T* __restrict__ d8 = sh.tmp[D8];
  T* __restrict__ r4p = sh.tmp[R4];
  const T* __restrict__ st = sh.store + (int64_t)store_slot * NSTORE * fs;
  const T* __restrict__ a3p = st + A3 * fs;
  const T* __restrict__ a4p = st + A4 * fs;
  A* __restrict__ grp = ElAcc<T>::rho(sh);
  const ColProf<T> Y(M, j);
  bool c3[2], c4[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    c3[c] = S.out && (INT || (j + c >= 2 && j + c <= NY));
    c4[c] = S.out && (INT || (j + c >= 1 && j + c <= NY - 1));
  }
  const int i0 = S.i0;
  // CPML items: the memory-variable adjoints g5..g8 of a row, loaded one row
  // ahead where they can be nonzero, with predicated loads
  const bool lx3 = c3[0] || c3[1], lx4 = c4[0] || c4[1];
  const bool ly3 = !INT && ((c3[0] && Y.acti[0]) || (c3[1] && Y.acti[1]));
  const bool ly4 = !INT && ((c4[0] && Y.acth[0]) || (c4[1] && Y.acth[1]));
  auto gload = [&](int r, V2<T> (&g)[4]) {
    if constexpr (!INT) {
      const int rr = min(max(r, 1), NX) - 1;
      const bool on = r < S.i_end;
      const bool q3 = on && PART != 2 && r >= 2, q4 = on && PART != 1 && r <= NX - 1;
      const bool x5 = q3 && (M.axi[rr] != T(0) || M.bxi[rr] != T(1));
      const bool x7 = q4 && (M.axh[rr] != T(0) || M.bxh[rr] != T(1));
      const int64_t o = S.off(r);
      g[0] = ld2p(g5, o, x5 && lx3);
      g[1] = ld2p(g6, o, q3 && ly3);
      g[2] = ld2p(g7, o, x7 && lx4);
      g[3] = ld2p(g8, o, q4 && ly4);
    }
  };
  V2<T> gg[4] = {};
  gload(i0, gg);
  V2<T> R0 = S.row(M.rho, i0), R1 = S.row(M.rho, i0 + 1);
  V2<T> GX = S.row(gvx, i0), GY = S.row(gvy, i0), E3 = S.row(a3p, i0), E4 = S.row(a4p, i0);
  V2<A> GR = S.row(grp, i0);
  for (int i = i0; i < S.i_end; i++) {
    const int64_t o = S.off(i);
    const bool more = i + 1 < S.i_end;
    const int rn = more ? i + 1 : -1;
    const V2<T> R2 = S.row(M.rho, more ? i + 2 : -1);
    const V2<T> GXn = S.row(gvx, rn), GYn = S.row(gvy, rn), E3n = S.row(a3p, rn),
                E4n = S.row(a4p, rn);
    const V2<A> GRn = S.row(grp, rn);
    V2<T> gn[4] = {};
    gload(i + 1, gn);
    T r0[3], r1[3];
    r0[0] = R0.v[0];
    r0[1] = R0.v[1];
    r0[2] = shdn(R0.v[0]);
    r1[0] = R1.v[0];
    r1[1] = R1.v[1];
    r1[2] = shdn(R1.v[0]);
    const T axi = INT ? T(0) : M.axi[i - 1], bxi = INT ? T(1) : M.bxi[i - 1];
    const T axh = INT ? T(0) : M.axh[i - 1], bxh = INT ? T(1) : M.bxh[i - 1];
    const bool r3 = INT || i >= 2, r4 = INT || i <= NX - 1;
    const bool rx5 = !INT && r3 && (axi != T(0) || bxi != T(1));
    const bool rx7 = !INT && r4 && (axh != T(0) || bxh != T(1));
    T o5[2], o6[2], o7[2], o8[2], o4[2], sg5[2], sg6[2], sg7[2], sg8[2];
    A gr[2];
    bool k3[2], k4[2], w5[2], w6[2], w7[2], w8[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
      k3[c] = PART != 2 && r3 && c3[c];
      k4[c] = PART != 1 && r4 && c4[c];
      o5[c] = o6[c] = o7[c] = o8[c] = o4[c] = T(0);
      sg5[c] = sg6[c] = sg7[c] = sg8[c] = T(0);
      w5[c] = w6[c] = w7[c] = w8[c] = false;
      gr[c] = A(0);
      if constexpr (PART != 2) {  // fw3 transpose
      const T gv = GX.v[c], r = r0[c];
      const T q = divr<T>(gv * M.dt, r);
      const bool u5 = k3[c] && rx5, u6 = !INT && k3[c] && Y.acti[c];
      const T gm5 = u5 ? q + gg[0].v[c] : q;
      const T gm6 = u6 ? q + gg[1].v[c] : q;
      sg5[c] = bxi * gm5;
      sg6[c] = Y.bi[c] * gm6;
      w5[c] = u5;
      w6[c] = u6;
      o5[c] = hdiv<T>(q + axi * gm5, M.hx24, M.rhx24);
      o6[c] = hdiv<T>(q + (INT ? T(0) : Y.ai[c]) * gm6, M.hy24, M.rhy24);
      gr[c] = GR.v[c] + (A)divr<T>(-gv * E3.v[c] * M.dt, r * r);
      }
      if constexpr (PART != 1) {  // fw4 transpose
      const T gw = GY.v[c];
      const T rho_ = T(0.25) * (r0[c] + r1[c] + r1[c + 1] + r0[c + 1]);
      const T q4 = divr<T>(gw * M.dt, rho_);
      const bool u7 = k4[c] && rx7, u8 = !INT && k4[c] && Y.acth[c];
      const T gm7 = u7 ? q4 + gg[2].v[c] : q4;
      const T gm8 = u8 ? q4 + gg[3].v[c] : q4;
      sg7[c] = bxh * gm7;
      sg8[c] = Y.bh[c] * gm8;
      w7[c] = u7;
      w8[c] = u8;
      o7[c] = hdiv<T>(q4 + axh * gm7, M.hx24, M.rhx24);
      o8[c] = hdiv<T>(q4 + (INT ? T(0) : Y.ah[c]) * gm8, M.hy24, M.rhy24);
      o4[c] = divr<T>(-gw * E4.v[c] * M.dt, rho_ * rho_) * T(0.25);
      }
    }
    if constexpr (!INT) {
      if constexpr (PART != 2) {
        st2p(g5, o, sg5, w5[0], w5[1]);
        st2p(g6, o, sg6, w6[0], w6[1]);
      }
      if constexpr (PART != 1) {
        st2p(g7, o, sg7, w7[0], w7[1]);
        st2p(g8, o, sg8, w8[0], w8[1]);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) gg[q] = gn[q];
    st2p(d5, o, o5, k3[0], k3[1]);
    st2p(d6, o, o6, k3[0], k3[1]);
    st2p(grp, o, gr, k3[0], k3[1]);
    st2p(d7, o, o7, k4[0], k4[1]);
    st2p(d8, o, o8, k4[0], k4[1]);
    st2p(r4p, o, o4, k4[0], k4[1]);
    R0 = R1; R1 = R2;
    GX = GXn; GY = GYn; E3 = E3n; E4 = E4n; GR = GRn;
  }
}

// Adjoint 2 (stress cells) of a strip: gather D5..D8 into the stress
// adjoints, then the transposes of fw1 and fw2.
template <typename T, bool INT, int PART>
__global__ void __launch_bounds__(EW * 32, el_minb_adj<T>())
k_el_adj2_rows(ElModel<T> M, const ElShot<T>* __restrict__ shots, const int* __restrict__ wlist,
               int ncolw, int R, int nwt,
               int store_slot) {
  const int wl = blockIdx.x * EW + (threadIdx.x >> 5);
  if (wl >= nwt) return;
  const int wi = wlist[wl];  // the warp's (strip, row tile)
  const ElShot<T>& sh = shots[blockIdx.y];
  const Strip<T> S(M, ncolw, R, wi);
  const int j = S.j, NX = S.NX, NY = S.NY;
  const int64_t fs = sh.fs;
  T* __restrict__ gxx = sh.g[SXX];
  T* __restrict__ gyy = sh.g[SYY];
  T* __restrict__ gxy = sh.g[SXY];
  T* __restrict__ g1 = sh.g[M1 + 0];
  T* __restrict__ g2 = sh.g[M1 + 1];
  T* __restrict__ g3 = sh.g[M1 + 2];
  T* __restrict__ g4 = sh.g[M1 + 3];
  const T* __restrict__ d5 = sh.tmp[D5];
  const T* __restrict__ d6 = sh.tmp[D6];
  const T* __restrict__ d7 = sh.tmp[D7];
  const T* __restrict__ d8 = sh.tmp[D8];
  T* __restrict__ d1 = sh.tmp[D1];
  T* __restrict__ d2 = sh.tmp[D2];
  T* __restrict__ d3 = sh.tmp[D3];
  T* __restrict__ d4p = sh.tmp[D4];
  T* __restrict__ gl1 = sh.tmp[GL1];
  T* __restrict__ gm1p = sh.tmp[GM1];
  T* __restrict__ gm2p = sh.tmp[GM2];
  const T* __restrict__ st = sh.store + (int64_t)store_slot * NSTORE * fs;
  const T* __restrict__ e1p = st + E1 * fs;
  const T* __restrict__ e2p = st + E2 * fs;
  const T* __restrict__ e12p = st + E12 * fs;
  const ColProf<T> Y(M, j);
  bool c1[2], c2[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    c1[c] = S.out && (INT || (j + c >= 2 && j + c <= NY));
    c2[c] = S.out && (INT || (j + c >= 1 && j + c <= NY - 1));
  }
  const int i0 = S.i0;
  // CPML items: the memory-variable adjoints g1..g4 of a row, loaded one row
  // ahead where they can be nonzero (x-profile active on the row, y-profile
  // active on the lane's columns) with predicated loads
  const bool lx1 = c1[0] || c1[1], lx2 = c2[0] || c2[1];
  const bool ly1 = !INT && ((c1[0] && Y.acti[0]) || (c1[1] && Y.acti[1]));
  const bool ly2 = !INT && ((c2[0] && Y.acth[0]) || (c2[1] && Y.acth[1]));
  auto gload = [&](int r, V2<T> (&g)[4]) {
    if constexpr (!INT) {
      const int rr = min(max(r, 1), NX) - 1;
      const bool on = r < S.i_end, q1 = on && r <= NX - 1, q2 = on && r >= 2;
      const bool x1 = q1 && (M.axh[rr] != T(0) || M.bxh[rr] != T(1));
      const bool x3 = q2 && (M.axi[rr] != T(0) || M.bxi[rr] != T(1));
      const int64_t o = S.off(r);
      g[0] = ld2p(g1, o, x1 && lx1);
      g[1] = ld2p(g2, o, q1 && ly1);
      g[2] = ld2p(g3, o, x3 && lx2);
      g[3] = ld2p(g4, o, q2 && ly2);
    }
  };
  V2<T> gg[4] = {};
  gload(i0, gg);
  // windows: D5 rows i-1..i+2, D7 rows i-2..i+1, lam / mu rows i, i+1
  V2<T> P0 = S.row(d5, i0 - 1), P1 = S.row(d5, i0), P2 = S.row(d5, i0 + 1), P3 = S.row(d5, i0 + 2);
  V2<T> Q0 = S.row(d7, i0 - 2), Q1 = S.row(d7, i0 - 1), Q2 = S.row(d7, i0), Q3 = S.row(d7, i0 + 1);
  V2<T> L0 = S.row(M.lam, i0), L1 = S.row(M.lam, i0 + 1);
  V2<T> U0 = S.row(M.mu, i0), U1 = S.row(M.mu, i0 + 1);
  V2<T> F6 = S.row(d6, i0), F8 = S.row(d8, i0);
  V2<T> GA = S.row(gxx, i0), GB = S.row(gyy, i0), GC = S.row(gxy, i0);
  V2<T> EA = S.row(e1p, i0), EB = S.row(e2p, i0), EC12 = S.row(e12p, i0);
  for (int i = i0; i < S.i_end; i++) {
    const int64_t o = S.off(i);
    const bool more = i + 1 < S.i_end;
    const int rn = more ? i + 1 : -1;
    const V2<T> P4 = S.row(d5, more ? i + 3 : -1), Q4 = S.row(d7, more ? i + 2 : -1),
                L2 = S.row(M.lam, more ? i + 2 : -1), U2 = S.row(M.mu, more ? i + 2 : -1);
    const V2<T> F6n = S.row(d6, rn), F8n = S.row(d8, rn);
    const V2<T> GAn = S.row(gxx, rn), GBn = S.row(gyy, rn), GCn = S.row(gxy, rn);
    const V2<T> EAn = S.row(e1p, rn), EBn = S.row(e2p, rn), ECn = S.row(e12p, rn);
    V2<T> gn[4] = {};
    gload(i + 1, gn);
    // row i across columns: D6 at j-1..j+3, D8 at j-2..j+2, mu at j..j+2
    T f6[5], f8[5], ur[3];
    f6[0] = shup(F6.v[1]);
    f6[1] = F6.v[0];
    f6[2] = F6.v[1];
    f6[3] = shdn(F6.v[0]);
    f6[4] = shdn(F6.v[1]);
    f8[0] = shup(F8.v[0]);
    f8[1] = shup(F8.v[1]);
    f8[2] = F8.v[0];
    f8[3] = F8.v[1];
    f8[4] = shdn(F8.v[0]);
    ur[0] = U0.v[0];
    ur[1] = U0.v[1];
    ur[2] = shdn(U0.v[0]);
    const T axh = INT ? T(0) : M.axh[i - 1], bxh = INT ? T(1) : M.bxh[i - 1];
    const T axi = INT ? T(0) : M.axi[i - 1], bxi = INT ? T(1) : M.bxi[i - 1];
    const bool r1 = INT || i <= NX - 1, r2 = INT || i >= 2;
    const bool rx1 = !INT && r1 && (axh != T(0) || bxh != T(1));
    const bool rx3 = !INT && r2 && (axi != T(0) || bxi != T(1));
    T oxx[2], oyy[2], oxy[2], ol1[2], om1[2], od1[2], od2[2], om2[2], od3[2], od4[2];
    T sg1[2], sg2[2], sg3[2], sg4[2];
    bool k1[2], k2[2], k12[2], w1[2], w2[2], w3[2], w4[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const bool b1 = r1 && c1[c], b2 = r2 && c2[c];
      k12[c] = b1 || b2;  // the stress adjoints of these cells are updated
      k1[c] = PART != 2 && b1;
      k2[c] = PART != 1 && b2;
      oxx[c] = oyy[c] = oxy[c] = ol1[c] = om1[c] = od1[c] = od2[c] = T(0);
      om2[c] = od3[c] = od4[c] = T(0);
      sg1[c] = sg2[c] = sg3[c] = sg4[c] = T(0);
      w1[c] = w2[c] = w3[c] = w4[c] = false;
      // gathers (zero outside the padded grid: those rows load as zeros and
      // the frame / padding columns of the temporaries are never written)
      if constexpr (PART != 2) {  // sxx / syy adjoints and the fw1 transpose
      const T gsxx = GA.v[c] + T(27) * P1.v[c] - T(27) * P2.v[c] - P0.v[c] + P3.v[c];
      const T gsyy = GB.v[c] + T(27) * f8[1 + c] - T(27) * f8[2 + c] - f8[c] + f8[3 + c];
      oxx[c] = gsxx;
      oyy[c] = gsyy;
      const T lam_ = T(0.5) * (L1.v[c] + L0.v[c]);
      const T mu1 = T(0.5) * (U1.v[c] + U0.v[c]);
      const T lm = lam_ + T(2) * mu1;
      const T e1 = EA.v[c], e2 = EB.v[c];
      const T gE1 = M.dt * (lm * gsxx + lam_ * gsyy);
      const T gE2 = M.dt * (lam_ * gsxx + lm * gsyy);
      const T glm = M.dt * (e1 * gsxx + e2 * gsyy);
      const T glam = M.dt * (e2 * gsxx + e1 * gsyy) + glm;
      ol1[c] = T(0.5) * glam;
      om1[c] = glm;
      const bool u1 = k1[c] && rx1, u2 = !INT && k1[c] && Y.acti[c];
      const T gm1 = u1 ? gE1 + gg[0].v[c] : gE1;
      const T gm2 = u2 ? gE2 + gg[1].v[c] : gE2;
      sg1[c] = bxh * gm1;
      sg2[c] = Y.bi[c] * gm2;
      w1[c] = u1;
      w2[c] = u2;
      od1[c] = hdiv<T>(gE1 + axh * gm1, M.hx24, M.rhx24);
      od2[c] = hdiv<T>(gE2 + (INT ? T(0) : Y.ai[c]) * gm2, M.hy24, M.rhy24);
      }
      if constexpr (PART != 1) {  // sxy adjoint and the fw2 transpose
      const T gsxy = GC.v[c] + T(27) * f6[1 + c] - T(27) * f6[2 + c] - f6[c] + f6[3 + c] +
                     T(27) * Q1.v[c] - T(27) * Q2.v[c] - Q0.v[c] + Q3.v[c];
      oxy[c] = gsxy;
      const T mu2 = T(0.5) * (ur[c] + ur[c + 1]);
      const T q = gsxy * mu2 * M.dt;
      om2[c] = gsxy * EC12.v[c] * M.dt * T(0.5);
      const bool u3 = k2[c] && rx3, u4 = !INT && k2[c] && Y.acth[c];
      const T gm3 = u3 ? q + gg[2].v[c] : q;
      const T gm4 = u4 ? q + gg[3].v[c] : q;
      sg3[c] = bxi * gm3;
      sg4[c] = Y.bh[c] * gm4;
      w3[c] = u3;
      w4[c] = u4;
      od3[c] = hdiv<T>(q + axi * gm3, M.hx24, M.rhx24);
      od4[c] = hdiv<T>(q + (INT ? T(0) : Y.ah[c]) * gm4, M.hy24, M.rhy24);
      }
    }
    if constexpr (!INT) {
      st2p(g1, o, sg1, w1[0], w1[1]);
      st2p(g2, o, sg2, w2[0], w2[1]);
      st2p(g3, o, sg3, w3[0], w3[1]);
      st2p(g4, o, sg4, w4[0], w4[1]);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) gg[q] = gn[q];
    if constexpr (PART != 2) {
      st2p(gxx, o, oxx, k12[0], k12[1]);
      st2p(gyy, o, oyy, k12[0], k12[1]);
    }
    if constexpr (PART != 1) st2p(gxy, o, oxy, k12[0], k12[1]);
    st2p(gl1, o, ol1, k1[0], k1[1]);
    st2p(gm1p, o, om1, k1[0], k1[1]);
    st2p(d1, o, od1, k1[0], k1[1]);
    st2p(d2, o, od2, k1[0], k1[1]);
    st2p(gm2p, o, om2, k2[0], k2[1]);
    st2p(d3, o, od3, k2[0], k2[1]);
    st2p(d4p, o, od4, k2[0], k2[1]);
    P0 = P1; P1 = P2; P2 = P3; P3 = P4;
    Q0 = Q1; Q1 = Q2; Q2 = Q3; Q3 = Q4;
    L0 = L1; L1 = L2; U0 = U1; U1 = U2;
    F6 = F6n; F8 = F8n;
    GA = GAn; GB = GBn; GC = GCn;
    EA = EAn; EB = EBn; EC12 = ECn;
  }
}

// Adjoint 3 (velocity cells + parameters) of a strip: gather D1..D4 into the
// velocity adjoints and the lambda / mu / rho parts into the accumulators.
template <typename T, bool INT, int PART>
__global__ void __launch_bounds__(EW * 32, el_minb_adj<T>())
k_el_adj3_rows(ElModel<T> M, const ElShot<T>* __restrict__ shots, const int* __restrict__ wlist,
               int ncolw, int R, int nwt) {
  using A = typename ElAcc<T>::type;
  const int wl = blockIdx.x * EW + (threadIdx.x >> 5);
  if (wl >= nwt) return;
  const int wi = wlist[wl];  // the warp's (strip, row tile)
  const ElShot<T>& sh = shots[blockIdx.y];
  const Strip<T> S(M, ncolw, R, wi);
  const int j = S.j, NX = S.NX, NY = S.NY;
  T* __restrict__ gvx = sh.g[VX];
  T* __restrict__ gvy = sh.g[VY];
  const T* __restrict__ d1 = sh.tmp[D1];
  const T* __restrict__ d2 = sh.tmp[D2];
  const T* __restrict__ d3 = sh.tmp[D3];
  const T* __restrict__ d4p = sh.tmp[D4];
  const T* __restrict__ gl1 = sh.tmp[GL1];
  const T* __restrict__ gm1p = sh.tmp[GM1];
  const T* __restrict__ gm2p = sh.tmp[GM2];
  const T* __restrict__ r4p = sh.tmp[R4];
  A* __restrict__ al = ElAcc<T>::lam(sh);
  A* __restrict__ am = ElAcc<T>::mu(sh);
  A* __restrict__ ar = ElAcc<T>::rho(sh);
  bool c3[2], c4[2], cp[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    c3[c] = S.out && (INT || (j + c >= 2 && j + c <= NY));
    c4[c] = S.out && (INT || (j + c >= 1 && j + c <= NY - 1));
    cp[c] = S.out && (INT || (j + c >= 1 && j + c <= NY));
  }
  const int i0 = S.i0;
  // windows: D1 rows i-2..i+1, D3 rows i-1..i+2, GL1 / GM1 / R4 rows i-1, i
  V2<T> P0 = S.row(d1, i0 - 2), P1 = S.row(d1, i0 - 1), P2 = S.row(d1, i0), P3 = S.row(d1, i0 + 1);
  V2<T> Q0 = S.row(d3, i0 - 1), Q1 = S.row(d3, i0), Q2 = S.row(d3, i0 + 1), Q3 = S.row(d3, i0 + 2);
  V2<T> GLm = S.row(gl1, i0 - 1), GL0 = S.row(gl1, i0);
  V2<T> GMm = S.row(gm1p, i0 - 1), GM0 = S.row(gm1p, i0);
  V2<T> RRm = S.row(r4p, i0 - 1), RR0 = S.row(r4p, i0);
  V2<T> F2 = S.row(d2, i0), F4 = S.row(d4p, i0), F12 = S.row(gm2p, i0);
  V2<T> VX0 = S.row(gvx, i0), VY0 = S.row(gvy, i0);
  V2<A> AL = S.row(al, i0), AM = S.row(am, i0), AR = S.row(ar, i0);
  for (int i = i0; i < S.i_end; i++) {
    const int64_t o = S.off(i);
    const bool more = i + 1 < S.i_end;
    const int rn = more ? i + 1 : -1;
    const V2<T> P4 = S.row(d1, more ? i + 2 : -1), Q4 = S.row(d3, more ? i + 3 : -1);
    const V2<T> GLn = S.row(gl1, rn), GMn = S.row(gm1p, rn), RRn = S.row(r4p, rn);
    const V2<T> F2n = S.row(d2, rn), F4n = S.row(d4p, rn), F12n = S.row(gm2p, rn);
    const V2<T> VXn = S.row(gvx, rn), VYn = S.row(gvy, rn);
    const V2<A> ALn = S.row(al, rn), AMn = S.row(am, rn), ARn = S.row(ar, rn);
    // row i across columns: D4 at j-2..j+2, D2 at j-1..j+3, GM2 / R4 (rows i-1, i) at j-1..j+1
    T f4[5], f2[5], g12[3], rm[3], r0[3];
    f4[0] = shup(F4.v[0]);
    f4[1] = shup(F4.v[1]);
    f4[2] = F4.v[0];
    f4[3] = F4.v[1];
    f4[4] = shdn(F4.v[0]);
    f2[0] = shup(F2.v[1]);
    f2[1] = F2.v[0];
    f2[2] = F2.v[1];
    f2[3] = shdn(F2.v[0]);
    f2[4] = shdn(F2.v[1]);
    g12[0] = shup(F12.v[1]);
    g12[1] = F12.v[0];
    g12[2] = F12.v[1];
    rm[0] = shup(RRm.v[1]);
    rm[1] = RRm.v[0];
    rm[2] = RRm.v[1];
    r0[0] = shup(RR0.v[1]);
    r0[1] = RR0.v[0];
    r0[2] = RR0.v[1];
    const bool r3 = INT || i >= 2, r4 = INT || i <= NX - 1;
    T ovx[2], ovy[2];
    A ol[2], om[2], orr[2];
    bool k3[2], k4[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
      k3[c] = r3 && c3[c];
      k4[c] = r4 && c4[c];
      ovx[c] = ovy[c] = T(0);
      ol[c] = om[c] = orr[c] = A(0);
      if constexpr (PART != 2) {  // velocity adjoints
      // D1 rows i-2..i+1 = P0..P3; D4 columns jc-2..jc+1 = f4[c..c+3]
      ovx[c] = VX0.v[c] + (T(27) * P1.v[c] - T(27) * P2.v[c] - P0.v[c] + P3.v[c] +
                           T(27) * f4[1 + c] - T(27) * f4[2 + c] - f4[c] + f4[3 + c]);
      // D2 columns jc-1..jc+2 = f2[c..c+3]; D3 rows i-1..i+2 = Q0..Q3
      ovy[c] = VY0.v[c] + (T(27) * f2[1 + c] - T(27) * f2[2 + c] - f2[c] + f2[3 + c] +
                           T(27) * Q1.v[c] - T(27) * Q2.v[c] - Q0.v[c] + Q3.v[c]);
      }
      if constexpr (PART != 1) {  // lambda / mu / rho accumulators
      ol[c] = AL.v[c] + (A)(GL0.v[c] + GLm.v[c]);
      om[c] = AM.v[c] + (A)(GM0.v[c] + GMm.v[c] + g12[1 + c] + g12[c]);
      orr[c] = AR.v[c] + (A)(r0[1 + c] + rm[1 + c] + rm[c] + r0[c]);
      }
    }
    if constexpr (PART != 2) {
      st2p(gvx, o, ovx, k3[0], k3[1]);
      st2p(gvy, o, ovy, k4[0], k4[1]);
    }
    if constexpr (PART != 1) {
      st2p(al, o, ol, cp[0], cp[1]);
      st2p(am, o, om, cp[0], cp[1]);
      st2p(ar, o, orr, cp[0], cp[1]);
    }
    P0 = P1; P1 = P2; P2 = P3; P3 = P4;
    Q0 = Q1; Q1 = Q2; Q2 = Q3; Q3 = Q4;
    GLm = GL0; GL0 = GLn; GMm = GM0; GM0 = GMn; RRm = RR0; RR0 = RRn;
    F2 = F2n; F4 = F4n; F12 = F12n;
    VX0 = VXn; VY0 = VYn;
    AL = ALn; AM = AMn; AR = ARn;
  }
}

// ---------------------------------------------------------------------------
// Fused adjoint step for the plans: the three gather passes above in one
// row-streaming pass over the fused forward step's strips and row tiles.
//
// The adjoint state alternates between two buffers like the forward state:
// the adjoint step of step n reads the adjoint of slot n from buffer pin and
// writes that of slot n-1 into buffer 1-pin.  So a warp can recompute the
// halo values its gathers need from the old adjoint state while the
// neighbouring strips and row tiles write their own cells.
//
// Per iteration a warp runs
//   phase A on row a (lanes 0..31): the transposes of fw3 and fw4 at the
//     velocity cells (D5..D8, R4 of the three-pass form, and the first rho
//     term), and the memory adjoints g5..g8;
//   phase B on row b = a-3 (needed on lanes 1..30): the stress adjoints,
//     gathered from D5..D8 of rows b-2..b+2, and the transposes of fw1 and
//     fw2 (D1..D4, the lambda / mu terms, g1..g4);
//   phase C on row t = b-3 (lanes 2..29 own): the velocity adjoints, gathered
//     from D1..D4 of rows t-2..t+2.
// D1..D8 go through per-warp rings of rows in shared memory instead of device
// memory.  Every ring row a phase reads was written in an earlier iteration,
// so the three phases of an iteration are independent of one another (one
// __syncwarp per iteration orders the ring).  A tile owns R rows: phase A runs
// on R + 8 rows, phase B on R + 4, phase C on R.  The rho accumulator is
// updated in phase A (its fw4 term needs R4 of rows a-1, a) and the lambda /
// mu accumulators in phase B (their terms need rows b-1, b), on the cells the
// warp owns, in the order the three-pass form adds them; values, masks and
// arithmetic are those of k_el_adj1_rows .. k_el_adj3_rows.
// ---------------------------------------------------------------------------
#ifndef ADS_EL_MINB_AI
#define ADS_EL_MINB_AI 4              // resident CTAs per SM, fused adjoint of CPML-free items
#endif
#ifndef ADS_EL_MINB_AC
#define ADS_EL_MINB_AC 3              // the same for items with CPML or box-edge logic
#endif
template <typename T, int KIND>
constexpr int el_minb_fadj() {
  return sizeof(T) != 4 ? 1 : KIND == 0 ? ADS_EL_MINB_AI : ADS_EL_MINB_AC;
}
// Rings of D1..D8 without their 1 / (24 h) factor (the gathers apply it once
// to each 4-term sum): RD rows each (a phase reads up to five rows behind the
// one written), RW elements a row (the warp's 64 columns and two on each
// side).  On CPML-free items D5 = D6, D7 = D8 and D3 = D4 before scaling
// (the memory-variable terms vanish), so those items keep five rings.
template <int KIND>
struct FRing {
  static constexpr bool Q = KIND == 0;
  static constexpr int d5 = 0, d6 = Q ? 0 : 1, d7 = Q ? 1 : 2, d8 = Q ? 1 : 3;
  static constexpr int d1 = Q ? 2 : 4, d2 = Q ? 3 : 5, d3 = Q ? 4 : 6, d4 = Q ? 4 : 7;
  static constexpr int n = Q ? 5 : 8;
};
#ifndef ADS_EL_FADJ_PREFETCH
#define ADS_EL_FADJ_PREFETCH 1        // issue the next iteration's loads before the arithmetic
#endif
constexpr bool kFadjPrefetch = ADS_EL_FADJ_PREFETCH != 0;
constexpr int RD = 6, RW = 68;
template <typename T, int KIND>
constexpr size_t el_fadj_smem() {
  return (size_t)EW * FRing<KIND>::n * RD * RW * sizeof(T);
}

template <typename T, int KIND>
__global__ void __launch_bounds__(EW * 32, el_minb_fadj<T, KIND>())
k_el_adj_rows(ElModel<T> M, const ElShot<T>* __restrict__ shots, const int* __restrict__ wlist,
              int ncolw, int R, int nwt, int store_slot, int pin, int jsh, int ish) {
  // KIND bit 0: rows need the box edge and x-profile logic; bit 1: columns
  // need the box edge and y-profile logic (0: neither)
  constexpr bool GR = (KIND & 1) != 0, GC = (KIND & 2) != 0;
  extern __shared__ __align__(16) unsigned char el_smem[];
  const int wl = blockIdx.x * EW + (threadIdx.x >> 5);
  if (wl >= nwt) return;
  const int wi = wlist[wl];  // the warp's (strip, row tile)
  const ElShot<T>& sh = shots[blockIdx.y];
  const int lane = threadIdx.x & 31, NX = M.NX, NY = M.NY;
  const int strip = wi % ncolw, rt = wi / ncolw;
  const int j = strip * FSTRIP - 3 + lane * EC + jsh;  // odd: 8/16-byte aligned pairs
  const bool own = lane >= 2 && lane <= 29;
  const bool colok = j >= -1 && j <= NY + 1;
  const int i0r = 1 + ish + rt * R;
  const int i0 = max(i0r, 1), i_end = min(i0r + R, NX + 1);
  const int64_t fs = sh.fs, P = M.P;
  const int64_t bin = (int64_t)pin * NF * fs, bout = (int64_t)(1 - pin) * NF * fs;
  const T* __restrict__ gvx = sh.g[VX] + bin;
  const T* __restrict__ gvy = sh.g[VY] + bin;
  const T* __restrict__ gxx = sh.g[SXX] + bin;
  const T* __restrict__ gyy = sh.g[SYY] + bin;
  const T* __restrict__ gxy = sh.g[SXY] + bin;
  T* __restrict__ ovxp = sh.g[VX] + bout;
  T* __restrict__ ovyp = sh.g[VY] + bout;
  T* __restrict__ oxxp = sh.g[SXX] + bout;
  T* __restrict__ oyyp = sh.g[SYY] + bout;
  T* __restrict__ oxyp = sh.g[SXY] + bout;
  const T* __restrict__ st = sh.store + (int64_t)store_slot * NSTORE * fs;
  const T* __restrict__ e1p = st + E1 * fs;
  const T* __restrict__ e2p = st + E2 * fs;
  const T* __restrict__ e12p = st + E12 * fs;
  const T* __restrict__ a3p = st + A3 * fs;
  const T* __restrict__ a4p = st + A4 * fs;
  using A = typename ElAcc<T>::type;
  static_assert(std::is_same<A, T>::value, "the step's partials have the stencil type");
  A* __restrict__ accl = ElAcc<T>::lam(sh);
  A* __restrict__ accm = ElAcc<T>::mu(sh);
  A* __restrict__ accr = ElAcc<T>::rho(sh);
  // memory adjoints 1..8, input / output buffer
  const T* __restrict__ g1i = sh.g[M1 + 0] + bin;
  const T* __restrict__ g2i = sh.g[M1 + 1] + bin;
  const T* __restrict__ g3i = sh.g[M1 + 2] + bin;
  const T* __restrict__ g4i = sh.g[M1 + 3] + bin;
  const T* __restrict__ g5i = sh.g[M1 + 4] + bin;
  const T* __restrict__ g6i = sh.g[M1 + 5] + bin;
  const T* __restrict__ g7i = sh.g[M1 + 6] + bin;
  const T* __restrict__ g8i = sh.g[M1 + 7] + bin;
  T* __restrict__ g1o = sh.g[M1 + 0] + bout;
  T* __restrict__ g2o = sh.g[M1 + 1] + bout;
  T* __restrict__ g3o = sh.g[M1 + 2] + bout;
  T* __restrict__ g4o = sh.g[M1 + 3] + bout;
  T* __restrict__ g5o = sh.g[M1 + 4] + bout;
  T* __restrict__ g6o = sh.g[M1 + 5] + bout;
  T* __restrict__ g7o = sh.g[M1 + 6] + bout;
  T* __restrict__ g8o = sh.g[M1 + 7] + bout;
  // this warp's rings; ring row of row r: (r - rbase) % RD (rbase <= every row read)
  using RG = FRing<KIND>;
  T* const ring = reinterpret_cast<T*>(el_smem) + (threadIdx.x >> 5) * (RG::n * RD * RW) + 2;
  // so[k]: offset of the ring row of row a - k (k < RD; row a - k - RD shares
  // it), rotated at the end of each iteration
  int so[RD];
#pragma unroll
  for (int k = 0; k < RD; k++) so[k] = ((RD + 4 - k) % RD) * RW;
  auto rrow = [&](int g, int k) { return ring + g * (RD * RW) + so[k % RD]; };
  // the pad columns (-2, -1, 64, 65) are read only for lanes whose results
  // are discarded; zero them once so those stay finite
  for (int e = lane; e < RG::n * RD * 4; e += 32) {
    const int row = e >> 2, k = e & 3;
    ring[row * RW + (k < 2 ? k - 2 : 62 + k)] = T(0);
  }
  // a lane's pair, and the pairs around it: columns jc-1..jc+2 (x[0..4] =
  // columns j-1..j+3) and jc-2..jc+1 (x[0..4] = j-2..j+2)
  const int le = lane * EC;
  auto rget = [&](const T* rw) { return *reinterpret_cast<const V2<T>*>(rw + le); };
  auto rput = [&](T* rw, const V2<T>& v) { *reinterpret_cast<V2<T>*>(rw + le) = v; };
  auto rspan_m1 = [&](const T* rw, T (&x)[5]) {
    x[0] = rw[le - 1];
    const V2<T> p = *reinterpret_cast<const V2<T>*>(rw + le);
    const V2<T> q = *reinterpret_cast<const V2<T>*>(rw + le + 2);
    x[1] = p.v[0];
    x[2] = p.v[1];
    x[3] = q.v[0];
    x[4] = q.v[1];
  };
  auto rspan_m2 = [&](const T* rw, T (&x)[5]) {
    const V2<T> p = *reinterpret_cast<const V2<T>*>(rw + le - 2);
    const V2<T> q = *reinterpret_cast<const V2<T>*>(rw + le);
    x[0] = p.v[0];
    x[1] = p.v[1];
    x[2] = q.v[0];
    x[3] = q.v[1];
    x[4] = rw[le + 2];
  };
  auto stw = [&](T* p, int o, const T (&x)[2], bool k0, bool k1) {
    if constexpr (GC) {
      st2s<T>(p, o, x, k0, k1);
    } else {
      st2p(p, o, x, k0, k1);
    }
  };
  // offsets within a field fit 32 bits (the plan checks (NX + 2) * P < 2^31)
  auto off = [&](int r) { return r * (int)P + j + JOFF; };
  auto ld = [&](const T* p, int r) {
    return ld2p(p, off(r), colok && r >= 0 && r <= NX + 1);
  };
  const ColProf<T> Y(M, j);
  // columns of the vx / sxx / syy boxes (2..NY), the vy / sxy boxes (1..NY-1)
  // and of the accumulators (1..NY)
  bool c3[2], c4[2], cp[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const int jc = j + c;
    c3[c] = !GC || (jc >= 2 && jc <= NY);
    c4[c] = !GC || (jc >= 1 && jc <= NY - 1);
    cp[c] = !GC || (jc >= 1 && jc <= NY);
  }
  const bool lc3 = c3[0] || c3[1], lc4 = c4[0] || c4[1];
  const bool ly3 = GC && ((c3[0] && Y.acti[0]) || (c3[1] && Y.acti[1]));
  const bool ly4 = GC && ((c4[0] && Y.acth[0]) || (c4[1] && Y.acth[1]));
  // rows of the vx / sxy boxes (2..NX) and of the vy / sxx / syy boxes (1..NX-1)
  auto rb3 = [&](int r) { return !GR || (r >= 2 && r <= NX); };
  auto rb4 = [&](int r) { return !GR || (r >= 1 && r <= NX - 1); };
  auto xp = [&](const T* p, int r, T dflt) { return GR ? p[min(max(r, 1), NX) - 1] : dflt; };
  // carried: rho rows a, a+1; lam / mu row b; R4 row a-1; GL1 / GM1 row b-1
  V2<T> R0 = ld(M.rho, i0 - 4), R1 = ld(M.rho, i0 - 3);
  V2<T> L0 = ld(M.lam, i0 - 7), U0 = ld(M.mu, i0 - 7);
  V2<T> R4p{}, GL1p{}, GM1p{};
  // the loads of iteration a: phase A row a, phase B row a-3, phase C row a-6
  struct Loads {
    V2<T> GX, GY, EA3, EA4, R2, AR, GA, GB, GCv, EA, EB, EC12, L1, U1, AL, AM, VX0, VY0;
    V2<T> m5, m6, m7, m8, m1, m2, m3, m4;
    T axi, bxi, axh, bxh, baxh, bbxh, baxi, bbxi;
  };
  auto load = [&](int a, Loads& L) {
    const int b = a - 3, t = a - 6;
    const bool doA = a <= i_end + 3, doB = b >= i0 - 2 && b <= i_end + 1, doC = t >= i0;
    const bool ownA = a >= i0 && a < i_end, ownB = b >= i0 && b < i_end;
    const int oa = off(a), ob = off(b), ot = off(t);
    const bool okA = doA && colok && a >= 0 && a <= NX + 1;
    const bool okB = doB && colok && b >= 0 && b <= NX + 1;
    L.GX = ld2p(gvx, oa, okA);
    L.GY = ld2p(gvy, oa, okA);
    L.EA3 = ld2p(a3p, oa, okA);
    L.EA4 = ld2p(a4p, oa, okA);
    L.R2 = ld(M.rho, a + 2);
    L.AR = ld2p(accr, oa, ownA && own && colok);
    L.GA = ld2p(gxx, ob, okB);
    L.GB = ld2p(gyy, ob, okB);
    L.GCv = ld2p(gxy, ob, okB);
    L.EA = ld2p(e1p, ob, okB);
    L.EB = ld2p(e2p, ob, okB);
    L.EC12 = ld2p(e12p, ob, okB);
    L.L1 = ld(M.lam, b + 1);
    L.U1 = ld(M.mu, b + 1);
    L.AL = ld2p(accl, ob, ownB && own && colok);
    L.AM = ld2p(accm, ob, ownB && own && colok);
    L.VX0 = ld2p(gvx, ot, doC && colok);
    L.VY0 = ld2p(gvy, ot, doC && colok);
    L.axi = xp(M.axi, a, T(0));
    L.bxi = xp(M.bxi, a, T(1));
    L.axh = xp(M.axh, a, T(0));
    L.bxh = xp(M.bxh, a, T(1));
    L.baxh = xp(M.axh, b, T(0));
    L.bbxh = xp(M.bxh, b, T(1));
    L.baxi = xp(M.axi, b, T(0));
    L.bbxi = xp(M.bxi, b, T(1));
    const bool r3 = doA && rb3(a), r4 = doA && rb4(a);
    const bool r1b = doB && rb4(b), r2b = doB && rb3(b);
    const bool rx5 = GR && r3 && (L.axi != T(0) || L.bxi != T(1));
    const bool rx7 = GR && r4 && (L.axh != T(0) || L.bxh != T(1));
    const bool rx1 = GR && r1b && (L.baxh != T(0) || L.bbxh != T(1));
    const bool rx3 = GR && r2b && (L.baxi != T(0) || L.bbxi != T(1));
    L.m5 = L.m6 = L.m7 = L.m8 = L.m1 = L.m2 = L.m3 = L.m4 = V2<T>{};
    if constexpr (GR) {
      L.m5 = ld2p(g5i, oa, rx5 && lc3);
      L.m7 = ld2p(g7i, oa, rx7 && lc4);
      L.m1 = ld2p(g1i, ob, rx1 && lc3);
      L.m3 = ld2p(g3i, ob, rx3 && lc4);
    }
    if constexpr (GC) {
      L.m6 = ld2p(g6i, oa, r3 && ly3);
      L.m8 = ld2p(g8i, oa, r4 && ly4);
      L.m2 = ld2p(g2i, ob, r1b && ly3);
      L.m4 = ld2p(g4i, ob, r2b && ly4);
    }
  };
  // (corner items, with both row and column logic, have no registers to spare)
  constexpr bool PF = kFadjPrefetch && KIND != 3;
  Loads cur;
  if (PF) load(i0 - 4, cur);
  __syncwarp();
  for (int a = i0 - 4; a <= i_end + 5; a++) {
    const int b = a - 3, t = a - 6;
    const bool doA = a <= i_end + 3, doB = b >= i0 - 2 && b <= i_end + 1, doC = t >= i0;
    const bool ownA = a >= i0 && a < i_end, ownB = b >= i0 && b < i_end;  // warp-uniform
    const int oa = off(a), ob = off(b), ot = off(t);
    // this iteration's loads were issued one iteration ahead (kFadjPrefetch)
    // or are issued now; the next iteration's go out before the arithmetic
    Loads nxt;
    if (PF) {
      if (a < i_end + 5) load(a + 1, nxt);
    } else {
      load(a, cur);
    }
    const V2<T> GX = cur.GX, GY = cur.GY, EA3 = cur.EA3, EA4 = cur.EA4, R2 = cur.R2, AR = cur.AR;
    const V2<T> GA = cur.GA, GB = cur.GB, GCv = cur.GCv, EA = cur.EA, EB = cur.EB,
                EC12 = cur.EC12, L1 = cur.L1, U1 = cur.U1, AL = cur.AL, AM = cur.AM;
    const V2<T> VX0 = cur.VX0, VY0 = cur.VY0;
    const V2<T> m5 = cur.m5, m6 = cur.m6, m7 = cur.m7, m8 = cur.m8, m1 = cur.m1, m2 = cur.m2,
                m3 = cur.m3, m4 = cur.m4;
    const T axi = cur.axi, bxi = cur.bxi, axh = cur.axh, bxh = cur.bxh;
    const T baxh = cur.baxh, bbxh = cur.bbxh, baxi = cur.baxi, bbxi = cur.bbxi;
    const bool r3 = doA && rb3(a), r4 = doA && rb4(a);
    const bool rx5 = GR && r3 && (axi != T(0) || bxi != T(1));
    const bool rx7 = GR && r4 && (axh != T(0) || bxh != T(1));
    const bool r1b = doB && rb4(b), r2b = doB && rb3(b);
    const bool rx1 = GR && r1b && (baxh != T(0) || bbxh != T(1));
    const bool rx3 = GR && r2b && (baxi != T(0) || bbxi != T(1));
    // ================= phase A: row a
    {
      T r0[3], r1[3];
      r0[0] = R0.v[0];
      r0[1] = R0.v[1];
      r0[2] = shdn(R0.v[0]);
      r1[0] = R1.v[0];
      r1[1] = R1.v[1];
      r1[2] = shdn(R1.v[0]);
      V2<T> D5n, D6n, D7n, D8n, R4n;
      T sg5[2], sg6[2], sg7[2], sg8[2], grt[2];
      bool k3[2], w5[2], w6[2], w7[2], w8[2];
#pragma unroll
      for (int c = 0; c < 2; c++) {
        k3[c] = r3 && c3[c];
        const bool k4 = r4 && c4[c];
        // fw3 transpose
        const T gv = GX.v[c], r = r0[c];
        const T q = divr<T>(gv * M.dt, r);
        const bool u5 = k3[c] && rx5, u6 = GC && k3[c] && Y.acti[c];
        const T gm5 = u5 ? q + m5.v[c] : q;
        const T gm6 = u6 ? q + m6.v[c] : q;
        sg5[c] = bxi * gm5;
        sg6[c] = Y.bi[c] * gm6;
        w5[c] = u5;
        w6[c] = u6;
        D5n.v[c] = k3[c] ? (GR ? q + axi * gm5 : q) : T(0);
        D6n.v[c] = k3[c] ? (GC ? q + Y.ai[c] * gm6 : q) : T(0);
        grt[c] = divr<T>(-gv * EA3.v[c] * M.dt, r * r);
        // fw4 transpose
        const T gw = GY.v[c];
        const T rho_ = T(0.25) * (r0[c] + r1[c] + r1[c + 1] + r0[c + 1]);
        const T q4 = divr<T>(gw * M.dt, rho_);
        const bool u7 = k4 && rx7, u8 = GC && k4 && Y.acth[c];
        const T gm7 = u7 ? q4 + m7.v[c] : q4;
        const T gm8 = u8 ? q4 + m8.v[c] : q4;
        sg7[c] = bxh * gm7;
        sg8[c] = Y.bh[c] * gm8;
        w7[c] = u7;
        w8[c] = u8;
        D7n.v[c] = k4 ? (GR ? q4 + axh * gm7 : q4) : T(0);
        D8n.v[c] = k4 ? (GC ? q4 + Y.ah[c] * gm8 : q4) : T(0);
        R4n.v[c] = k4 ? divr<T>(-gw * EA4.v[c] * M.dt, rho_ * rho_) * T(0.25) : T(0);
      }
      if (doA) {
        rput(rrow(RG::d5, 0), D5n);
        rput(rrow(RG::d7, 0), D7n);
        if constexpr (!RG::Q) {
          rput(rrow(RG::d6, 0), D6n);
          rput(rrow(RG::d8, 0), D8n);
        }
      }
      // R4 of rows a and a-1 at columns jc-1, jc
      T rs[3], rq[3];
      rs[0] = shup(R4n.v[1]);
      rs[1] = R4n.v[0];
      rs[2] = R4n.v[1];
      rq[0] = shup(R4p.v[1]);
      rq[1] = R4p.v[0];
      rq[2] = R4p.v[1];
      if (ownA && own) {
        A orr[2];
#pragma unroll
        for (int c = 0; c < 2; c++)
          orr[c] = (k3[c] ? AR.v[c] + grt[c] : AR.v[c]) + (rs[1 + c] + rq[1 + c] + rq[c] + rs[c]);
        stw(accr, oa, orr, cp[0], cp[1]);
        if constexpr (GR) {
          stw(g5o, oa, sg5, w5[0], w5[1]);
          stw(g7o, oa, sg7, w7[0], w7[1]);
        }
        if constexpr (GC) {
          stw(g6o, oa, sg6, w6[0], w6[1]);
          stw(g8o, oa, sg8, w8[0], w8[1]);
        }
      }
      R4p = R4n;
    }
    // ================= phase B: row b
    if (doB) {
      // D5 rows b-1..b+2, D7 rows b-2..b+1 (this column); row b across
      // columns: D6 at jc-1..jc+2, D8 at jc-2..jc+1, mu at jc..jc+1
      const V2<T> P0 = rget(rrow(RG::d5, 4)), P1 = rget(rrow(RG::d5, 3)),
                  P2 = rget(rrow(RG::d5, 2)), P3 = rget(rrow(RG::d5, 1));
      const V2<T> Q0 = rget(rrow(RG::d7, 5)), Q1 = rget(rrow(RG::d7, 4)),
                  Q2 = rget(rrow(RG::d7, 3)), Q3 = rget(rrow(RG::d7, 2));
      T f6[5], f8[5], ur[3];
      rspan_m1(rrow(RG::d6, 3), f6);
      rspan_m2(rrow(RG::d8, 3), f8);
      ur[0] = U0.v[0];
      ur[1] = U0.v[1];
      ur[2] = shdn(U0.v[0]);
      V2<T> D1n, D2n, D3n, D4n, GL1n, GM1n;
      T oxx[2], oyy[2], oxy[2], sg1[2], sg2[2], sg3[2], sg4[2], gm2v[2];
      bool k12[2], w1[2], w2[2], w3[2], w4[2];
#pragma unroll
      for (int c = 0; c < 2; c++) {
        const bool b1 = r1b && c3[c], b2 = r2b && c4[c];
        k12[c] = b1 || b2;
        const T gsxx =
            GA.v[c] + hdiv<T>(T(27) * P1.v[c] - T(27) * P2.v[c] - P0.v[c] + P3.v[c], M.hx24,
                              M.rhx24);
        const T gsyy =
            GB.v[c] + hdiv<T>(T(27) * f8[1 + c] - T(27) * f8[2 + c] - f8[c] + f8[3 + c], M.hy24,
                              M.rhy24);
        const T gsxy =
            GCv.v[c] +
            hdiv<T>(T(27) * f6[1 + c] - T(27) * f6[2 + c] - f6[c] + f6[3 + c], M.hy24,
                    M.rhy24) +
            hdiv<T>(T(27) * Q1.v[c] - T(27) * Q2.v[c] - Q0.v[c] + Q3.v[c], M.hx24, M.rhx24);
        oxx[c] = gsxx;
        oyy[c] = gsyy;
        oxy[c] = gsxy;
        // fw1 transpose
        const T lam_ = T(0.5) * (L1.v[c] + L0.v[c]);
        const T mu1 = T(0.5) * (U1.v[c] + U0.v[c]);
        const T lm = lam_ + T(2) * mu1;
        const T e1 = EA.v[c], e2 = EB.v[c];
        const T gE1 = M.dt * (lm * gsxx + lam_ * gsyy);
        const T gE2 = M.dt * (lam_ * gsxx + lm * gsyy);
        const T glm = M.dt * (e1 * gsxx + e2 * gsyy);
        const T glam = M.dt * (e2 * gsxx + e1 * gsyy) + glm;
        const bool u1 = b1 && rx1, u2 = GC && b1 && Y.acti[c];
        const T gm1 = u1 ? gE1 + m1.v[c] : gE1;
        const T gm2 = u2 ? gE2 + m2.v[c] : gE2;
        sg1[c] = bbxh * gm1;
        sg2[c] = Y.bi[c] * gm2;
        w1[c] = u1;
        w2[c] = u2;
        GL1n.v[c] = b1 ? T(0.5) * glam : T(0);
        GM1n.v[c] = b1 ? glm : T(0);
        D1n.v[c] = b1 ? (GR ? gE1 + baxh * gm1 : gE1) : T(0);
        D2n.v[c] = b1 ? (GC ? gE2 + Y.ai[c] * gm2 : gE2) : T(0);
        // fw2 transpose
        const T mu2 = T(0.5) * (ur[c] + ur[c + 1]);
        const T q = gsxy * mu2 * M.dt;
        const bool u3 = b2 && rx3, u4 = GC && b2 && Y.acth[c];
        const T gm3 = u3 ? q + m3.v[c] : q;
        const T gm4 = u4 ? q + m4.v[c] : q;
        sg3[c] = bbxi * gm3;
        sg4[c] = Y.bh[c] * gm4;
        w3[c] = u3;
        w4[c] = u4;
        D3n.v[c] = b2 ? (GR ? q + baxi * gm3 : q) : T(0);
        D4n.v[c] = b2 ? (GC ? q + Y.ah[c] * gm4 : q) : T(0);
        gm2v[c] = b2 ? gsxy * EC12.v[c] * M.dt * T(0.5) : T(0);  // GM2, the sxy term of mu
      }
      rput(rrow(RG::d1, 3), D1n);
      rput(rrow(RG::d2, 3), D2n);
      rput(rrow(RG::d3, 3), D3n);
      if constexpr (!RG::Q) rput(rrow(RG::d4, 3), D4n);
      // GM2 of row b at columns jc-1, jc
      T g12[3];
      g12[1] = gm2v[0];
      g12[2] = gm2v[1];
      g12[0] = shup(g12[2]);
      if (ownB && own) {
        A ol[2], om[2];
#pragma unroll
        for (int c = 0; c < 2; c++) {
          ol[c] = AL.v[c] + (GL1n.v[c] + GL1p.v[c]);
          om[c] = AM.v[c] + (GM1n.v[c] + GM1p.v[c] + g12[1 + c] + g12[c]);
        }
        stw(oxxp, ob, oxx, k12[0], k12[1]);
        stw(oyyp, ob, oyy, k12[0], k12[1]);
        stw(oxyp, ob, oxy, k12[0], k12[1]);
        stw(accl, ob, ol, cp[0], cp[1]);
        stw(accm, ob, om, cp[0], cp[1]);
        if constexpr (GR) {
          stw(g1o, ob, sg1, w1[0], w1[1]);
          stw(g3o, ob, sg3, w3[0], w3[1]);
        }
        if constexpr (GC) {
          stw(g2o, ob, sg2, w2[0], w2[1]);
          stw(g4o, ob, sg4, w4[0], w4[1]);
        }
      }
      GL1p = GL1n;
      GM1p = GM1n;
    }
    // ================= phase C: row t
    if (doC) {
      // D1 rows t-2..t+1, D3 rows t-1..t+2 (this column); row t across
      // columns: D4 at jc-2..jc+1, D2 at jc-1..jc+2
      const V2<T> P0 = rget(rrow(RG::d1, 8)), P1 = rget(rrow(RG::d1, 7)),
                  P2 = rget(rrow(RG::d1, 6)), P3 = rget(rrow(RG::d1, 5));
      const V2<T> Q0 = rget(rrow(RG::d3, 7)), Q1 = rget(rrow(RG::d3, 6)),
                  Q2 = rget(rrow(RG::d3, 5)), Q3 = rget(rrow(RG::d3, 4));
      T f4[5], f2[5];
      rspan_m2(rrow(RG::d4, 6), f4);
      rspan_m1(rrow(RG::d2, 6), f2);
      const bool r3t = rb3(t), r4t = rb4(t);
      T ovx[2], ovy[2];
      bool k3t[2], k4t[2];
#pragma unroll
      for (int c = 0; c < 2; c++) {
        k3t[c] = r3t && c3[c];
        k4t[c] = r4t && c4[c];
        ovx[c] = VX0.v[c] +
                 (hdiv<T>(T(27) * P1.v[c] - T(27) * P2.v[c] - P0.v[c] + P3.v[c], M.hx24,
                          M.rhx24) +
                  hdiv<T>(T(27) * f4[1 + c] - T(27) * f4[2 + c] - f4[c] + f4[3 + c], M.hy24,
                          M.rhy24));
        ovy[c] = VY0.v[c] +
                 (hdiv<T>(T(27) * f2[1 + c] - T(27) * f2[2 + c] - f2[c] + f2[3 + c], M.hy24,
                          M.rhy24) +
                  hdiv<T>(T(27) * Q1.v[c] - T(27) * Q2.v[c] - Q0.v[c] + Q3.v[c], M.hx24,
                          M.rhx24));
      }
      if (own) {
        stw(ovxp, ot, ovx, k3t[0], k3t[1]);
        stw(ovyp, ot, ovy, k4t[0], k4t[1]);
      }
    }
    __syncwarp();  // this iteration's ring rows before the next one reads them
    {
      const int s5 = so[RD - 1];
#pragma unroll
      for (int k = RD - 1; k > 0; k--) so[k] = so[k - 1];
      so[0] = s5;
    }
    R0 = R1;
    R1 = R2;
    L0 = L1;
    U0 = U1;
    if (PF) cur = nxt;
  }
}

// End of a checkpoint segment (FP32 plans): accumulators += partials, partials = 0.
__global__ void k_el_flush_acc(const ElShot<float>* __restrict__ shots, int64_t n) {
  const ElShot<float>& sh = shots[blockIdx.y];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    sh.glam[e] += (double)sh.gl32[e];
    sh.gmu[e] += (double)sh.gm32[e];
    sh.grho[e] += (double)sh.gr32[e];
    sh.gl32[e] = 0.0f;
    sh.gm32[e] = 0.0f;
    sh.gr32[e] = 0.0f;
  }
}

// Sources of slot n (added in order by one thread), then receivers of slot n.
// par: the state buffer holding slot n (0 for in-place plans); a source on a
// cell no stencil updates is added to both buffers when dual != 0.
template <typename T>
__global__ void k_el_src_rcv(const ElShot<T>* __restrict__ shots, int n, int nt, int record,
                             int par, int dual) {
  const ElShot<T>& sh = shots[blockIdx.x];
  const int64_t d = (int64_t)NF * sh.fs, mine = par ? d : 0, other = par ? -d : d;
  if (threadIdx.x == 0) {
    const T* row = sh.srcv + (int64_t)(n - 1) * sh.nsrc;
    for (int k = 0; k < sh.nsrc; k++) {
      T* p = sh.src_ptr[k];
      if (!p) continue;
      p[mine] += row[k];
      if (dual && sh.src_dual[k]) p[mine + other] += row[k];
    }
  }
  if (!record) return;
  __syncthreads();
  for (int r = threadIdx.x; r < sh.nrcv; r += blockDim.x) {
    const T* p = sh.rcv_ptr[r];
    sh.traces[(int64_t)r * nt + n] = p ? p[mine] : T(0);
  }
}

// Adjoint state += residual of slot n at the receivers (one thread each).
// par: the adjoint buffer that holds slot n (0 for the in-place form).
template <typename T>
__global__ void k_el_resid(const ElShot<T>* __restrict__ shots, int n, int nt, int par) {
  const ElShot<T>& sh = shots[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= sh.nrcv) return;
  T* p = sh.rcv_gptr[r];
  if (p) atomicAdd(p + (par ? (int64_t)NF * sh.fs : 0), sh.resid[(int64_t)r * nt + n]);
}

// d loss / d srcv row n-1: srcv row n-1 is added to state n, so its gradient
// is the adjoint of state n (residual of slot n included) at the source cell
// (AddSource.cpp:91-155 gathers grad_srcv the same way).  One thread a source.
template <typename T>
__global__ void k_el_src_grad(const ElShot<T>* __restrict__ shots, int n, int par) {
  const ElShot<T>& sh = shots[blockIdx.y];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sh.nsrc) return;
  const T* p = sh.src_gptr[k];
  sh.gsrc[(int64_t)(n - 1) * sh.nsrc + k] =
      p ? (double)p[par ? (int64_t)NF * sh.fs : 0] : 0.0;
}

// State <-> checkpoint copies (13 contiguous fields per shot).  Saving reads
// state buffer par; restoring writes buffer 0 and, for two-buffer plans
// (both != 0), buffer 1 as well.
template <typename T>
__global__ void k_el_ckpt(const ElShot<T>* __restrict__ shots, int slot, int to_ckpt, int par,
                          int both) {
  const ElShot<T>& sh = shots[blockIdx.y];
  const int64_t n = NF * sh.fs;
  T* state = sh.f[0];
  T* ck = sh.ckpt + (int64_t)slot * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (to_ckpt) {
      ck[e] = state[par ? n + e : e];
    } else {
      const T v = ck[e];
      state[e] = v;
      if (both) state[n + e] = v;
    }
  }
}

template <typename T>
__global__ void k_el_cast(T* __restrict__ out, const double* __restrict__ in, int NX, int NY,
                          int64_t P, int off) {
  const int64_t n = (int64_t)(NX + 2) * (NY + 2);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / (NY + 2), j = e % (NY + 2);
    out[i * P + j + off] = (T)in[e];
  }
}

// Sum the shots' FP64 accumulators into the caller's unpitched gradients.
template <typename T>
__global__ void k_el_gather_grads(const ElShot<T>* __restrict__ shots, int nshots, int NX,
                                  int NY, int64_t P, int off, double* __restrict__ gl,
                                  double* __restrict__ gm, double* __restrict__ gr) {
  const int64_t n = (int64_t)(NX + 2) * (NY + 2);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / (NY + 2), j = e % (NY + 2), x = i * P + j + off;
    double a = 0, b = 0, c = 0;
    for (int s = 0; s < nshots; s++) {
      a += shots[s].glam[x];
      b += shots[s].gmu[x];
      c += shots[s].grho[x];
    }
    gl[e] = a;
    gm[e] = b;
    gr[e] = c;
  }
}

// Single-step operator sources: 1-based device indices, CPU AddSource order.
template <typename T>
struct Fields5 {
  T* p[5];
};

template <typename T>
__global__ void k_el_step_src(Fields5<T> f5, const int64_t* __restrict__ si,
                              const int64_t* __restrict__ sj, const int64_t* __restrict__ st,
                              const T* __restrict__ sv, int64_t nsrc, int NX, int NY) {
  if (threadIdx.x != 0) return;
  for (int64_t k = 0; k < nsrc; k++) {
    const int64_t t = st[k], a = si[k] - 1, b = sj[k] - 1;
    if (t < 0 || t > 4) continue;
    if (a < 0 || a > NX + 1 || b < 0 || b > NY + 1) continue;
    f5.p[t][a * (NY + 2) + b] += sv[k];
  }
}

// reduction helpers (deterministic two-pass FP64 misfit)
constexpr unsigned FULLM = 0xffffffffu;
template <typename T>
__global__ void k_el_misfit(const T* __restrict__ tr, const T* __restrict__ obs,
                            T* __restrict__ resid, int64_t n, double* __restrict__ partial) {
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double d = (double)tr[e] - (double)obs[e];
    resid[e] = (T)(2 * d);
    acc += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULLM, acc, o);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULLM, acc, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
  }
}

__global__ void k_el_reduce(const double* __restrict__ partial, int n, double* out) {
  double acc = 0.0;
  for (int e = threadIdx.x; e < n; e += blockDim.x) acc += partial[e];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULLM, acc, o);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULLM, acc, o);
    if (threadIdx.x == 0) *out = acc;
  }
}

template <typename T>
ElModel<T> make_model(int NX, int NY, int64_t P, int off, double dt, double dx, double dy,
                      const T* lam, const T* mu, const T* rho, const T* prof) {
  // prof: axi, axh, bxi, bxh (NX each), ayi, ayh, byi, byh (NY each)
  ElModel<T> M{};
  M.lam = lam;
  M.mu = mu;
  M.rho = rho;
  M.axi = prof;
  M.axh = prof + NX;
  M.bxi = prof + 2 * NX;
  M.bxh = prof + 3 * NX;
  M.ayi = prof + 4 * NX;
  M.ayh = prof + 4 * NX + NY;
  M.byi = prof + 4 * NX + 2 * NY;
  M.byh = prof + 4 * NX + 3 * NY;
  M.dt = (T)dt;
  M.hx24 = (T)(24 * dx);
  M.hy24 = (T)(24 * dy);
  M.rhx24 = (T)(1.0 / (24 * dx));
  M.rhy24 = (T)(1.0 / (24 * dy));
  M.NX = NX;
  M.NY = NY;
  M.OFF = off;
  M.P = P;
  return M;
}

// Host: pack profile rows as the kernels index them (I-1 / J-1).
template <typename T>
std::vector<T> pack_profiles(int64_t NX, int64_t NY, const double* ax, const double* bx,
                             const double* ay, const double* by) {
  std::vector<T> p(4 * NX + 4 * NY);
  for (int64_t i = 0; i < NX; i++) {
    p[i] = (T)ax[i];
    p[NX + i] = (T)ax[NX + i];
    p[2 * NX + i] = (T)bx[i];
    p[3 * NX + i] = (T)bx[NX + i];
  }
  for (int64_t j = 0; j < NY; j++) {
    p[4 * NX + j] = (T)ay[j];
    p[4 * NX + NY + j] = (T)ay[NY + j];
    p[4 * NX + 2 * NY + j] = (T)by[j];
    p[4 * NX + 3 * NY + j] = (T)by[NY + j];
  }
  return p;
}

}  // namespace

// Launchers of the adjoint row kernels: interior / CPML items, part 1 / 2.
#define ADS_EL_SEL(K, ...)                                    \
  do {                                                        \
    if (in) {                                                 \
      if (part == 0) K(__VA_ARGS__, true, 0);                 \
      else if (part == 1) K(__VA_ARGS__, true, 1);            \
      else K(__VA_ARGS__, true, 2);                           \
    } else {                                                  \
      if (part == 0) K(__VA_ARGS__, false, 0);                \
      else if (part == 1) K(__VA_ARGS__, false, 1);           \
      else K(__VA_ARGS__, false, 2);                          \
    }                                                         \
  } while (0)

template <typename T>
void el_adj1(bool in, int part, dim3 g, cudaStream_t s, const ElModel<T>& M, const ElShot<T>* sh,
             const int* wl, int ncolw, int R, int nw, int slot) {
#define ADS_K(IN, PT) \
  k_el_adj1_rows<T, IN, PT><<<g, EW * 32, 0, s>>>(M, sh, wl, ncolw, R, nw, slot)
#define ADS_K1(dummy, IN, PT) ADS_K(IN, PT)
  ADS_EL_SEL(ADS_K1, 0);
#undef ADS_K1
#undef ADS_K
}

template <typename T>
void el_adj2(bool in, int part, dim3 g, cudaStream_t s, const ElModel<T>& M, const ElShot<T>* sh,
             const int* wl, int ncolw, int R, int nw, int slot) {
#define ADS_K1(dummy, IN, PT) \
  k_el_adj2_rows<T, IN, PT><<<g, EW * 32, 0, s>>>(M, sh, wl, ncolw, R, nw, slot)
  ADS_EL_SEL(ADS_K1, 0);
#undef ADS_K1
}

template <typename T>
void el_adj3(bool in, int part, dim3 g, cudaStream_t s, const ElModel<T>& M, const ElShot<T>* sh,
             const int* wl, int ncolw, int R, int nw) {
#define ADS_K1(dummy, IN, PT) \
  k_el_adj3_rows<T, IN, PT><<<g, EW * 32, 0, s>>>(M, sh, wl, ncolw, R, nw)
  ADS_EL_SEL(ADS_K1, 0);
#undef ADS_K1
}
#undef ADS_EL_SEL

template <typename T>
void el_step(bool store, int kind, dim3 g, cudaStream_t s, const ElModel<T>& M,
             const ElShot<T>* sh, const int* wl, int ncolw, int R, int nw, int slot, int pin,
             int jsh, int ish) {
#define ADS_K(ST, KD)                                                                     \
  k_el_step_rows<T, ST, KD><<<g, EW * 32, 0, s>>>(M, sh, wl, ncolw, R, nw, slot, pin, jsh, \
                                                  ish)
#define ADS_KS(ST)                   \
  do {                               \
    switch (kind) {                  \
      case 0: ADS_K(ST, 0); break;   \
      case 1: ADS_K(ST, 1); break;   \
      case 2: ADS_K(ST, 2); break;   \
      default: ADS_K(ST, 3); break;  \
    }                                \
  } while (0)
  if (store) ADS_KS(true);
  else ADS_KS(false);
#undef ADS_KS
#undef ADS_K
}

template <typename T>
void el_fadj(int kind, dim3 g, cudaStream_t s, const ElModel<T>& M, const ElShot<T>* sh,
             const int* wl, int ncolw, int R, int nw, int slot, int pin, int jsh, int ish) {
#define ADS_K(KD)                                                                      \
  k_el_adj_rows<T, KD><<<g, EW * 32, el_fadj_smem<T, KD>(), s>>>(M, sh, wl, ncolw, R, nw, slot, \
                                                            pin, jsh, ish)
  switch (kind) {
    case 0: ADS_K(0); break;
    case 1: ADS_K(1); break;
    case 2: ADS_K(2); break;
    default: ADS_K(3); break;
  }
#undef ADS_K
}

// The fused adjoint's rings take more than the default 48 KB of dynamic
// shared memory a CTA.
template <typename T>
int el_fadj_prepare() {
  ADS_CUDA(cudaFuncSetAttribute(k_el_adj_rows<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)el_fadj_smem<T, 0>()));
  ADS_CUDA(cudaFuncSetAttribute(k_el_adj_rows<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)el_fadj_smem<T, 1>()));
  ADS_CUDA(cudaFuncSetAttribute(k_el_adj_rows<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)el_fadj_smem<T, 2>()));
  ADS_CUDA(cudaFuncSetAttribute(k_el_adj_rows<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)el_fadj_smem<T, 3>()));
  return ADS_OK;
}

// ======================================================================
// whole-path elastic plan
// ======================================================================

// Whether the stencil of field `type` updates 0-based padded cell (i, j)
// (src/Core.jl:96-228): vx rows 2..NX, columns 2..NY; vy 1..NX-1, 1..NY-1;
// sxx, syy 1..NX-1, 2..NY; sxy 2..NX, 1..NY-1.
static bool el_cell_updated(int type, int64_t i, int64_t j, int NX, int NY) {
  switch (type) {
    case VX: return i >= 2 && i <= NX && j >= 2 && j <= NY;
    case VY: return i >= 1 && i <= NX - 1 && j >= 1 && j <= NY - 1;
    case SXX:
    case SYY: return i >= 1 && i <= NX - 1 && j >= 2 && j <= NY;
    case SXY: return i >= 2 && i <= NX && j >= 1 && j <= NY - 1;
    default: return false;
  }
}

struct ElPlanBase {
  virtual ~ElPlanBase() = default;
  virtual int forward(const double* l, const double* m, const double* r, void* traces,
                      cudaStream_t st) = 0;
  virtual int profile(const double* l, const double* m, const double* r, double* out,
                      cudaStream_t st) = 0;
  virtual int gradient(const double* l, const double* m, const double* r, const void* obs,
                       double* loss, double* gl, double* gm, double* gr, void* tr_out,
                       cudaStream_t st, double* grad_srcv) = 0;
  // new wavelets for a shot's sources (device FP64, (NSTEP, nsrc) row-major)
  virtual int set_source_values(int64_t shot, const double* srcv, cudaStream_t st) = 0;
  std::vector<int64_t> trace_off;
  std::vector<int64_t> src_off;  // per shot: offset of its (NSTEP, nsrc) grad_srcv block
  int64_t src_total = 0;
  int64_t trace_total = 0, bytes = 0, launches_fwd = 0, launches_grad = 0;
  int64_t resident = 0;  // checkpoint segments kept resident (no recompute)
  int64_t tiling[2] = {0, 0};  // rows per adjoint tile or strip, rows per fused-step tile
  int64_t adj_items[4] = {0, 0, 0, 0};  // fused adjoint items of each kind
};

namespace {

template <typename T>
struct ElPlan final : ElPlanBase {
  ads_elastic_config cfg{};
  int nshots = 0, K = 0, nseg = 0, NX = 0, NY = 0, NSTEP = 0;
  std::vector<T*> srcv_dev;     // per shot: its wavelets, (NSTEP, nsrc)
  std::vector<int64_t> srcv_n;  // per shot: NSTEP * nsrc
  int set_source_values(int64_t shot, const double* srcv, cudaStream_t st) override {
    ADS_REQUIRE(shot >= 0 && shot < nshots, "shot %lld out of range [0, %d)", (long long)shot,
                nshots);
    ADS_REQUIRE(srcv || srcv_n[shot] == 0, "null srcv");
    return cast_scaled(srcv_dev[shot], srcv, srcv_n[shot], 1.0, st);
  }
  int ncolw = 0, rows_w = 0, nwt = 0;  // warp strips of the row-streaming step kernels
  // Resident segments res_seg .. nseg-1: the forward loop stores their steps'
  // strains / accelerations (store slot K + n - a_res, a_res = 1 + res_seg K)
  // and the reverse sweep neither restores nor recomputes them.  res_seg ==
  // nseg: none.
  int res_seg = 0;
  int a_res() const { return 1 + res_seg * K; }
  // warp items (strip, row tile) of CPML-free tiles and of the rest; the two
  // launches of a step kernel run concurrently (disjoint cells)
  int* d_wl = nullptr;  // interior items, then the CPML items at nw_in
  int nw_in = 0, nw_pm = 0;
  // the fused forward step: its own strips (FSTRIP columns), row tiles and
  // item lists, and the state buffer that holds slot n
  int ncolf = 0, rows_f = 0, nwtf = 0, jsh = 0, ish = 0;
  int nwk[4] = {}, owk[4] = {};  // items of each kind (k_el_step_rows KIND) and their offsets
  int* d_wlf = nullptr;
  // the fused adjoint step (k_el_adj_rows): its own row tiles and item lists
  // (its halo is four rows and two lanes deep), and the adjoint buffer that
  // holds slot n.  fused == false: the three gather passes, in place.
  bool fused = true;
  int ncola = 0, rows_a = 0, nwta = 0, jsha = 0, isha = 0;
  int nwka[4] = {}, owka[4] = {};
  int* d_wla = nullptr;
  // host copies: the packed CPML rows and the item lists of the current tiling
  std::vector<T> hprof;
  std::vector<int> wl_host, wlf_host, wla_host;
  // items for rows_w = rw (three-pass adjoint), rows_f = rf (fused step) and
  // rows_a = ra (fused adjoint)
  void build_lists(int rw, int rf, int ra);
  int upload_lists(cudaStream_t st);
  int autotune(cudaStream_t st, int rw_min, int rf_min);
  static int par(int n) { return n & 1; }
  int apar(int n) const { return fused ? n & 1 : 0; }  // adjoint buffer of slot n
  int adj_launches() const {
    if (fused) return (nwka[0] > 0) + (nwka[1] > 0) + (nwka[2] > 0) + (nwka[3] > 0);
    return group_launches(kSplitAdj1, nw_in, nw_pm) +
           2 * group_launches(kSplitAdj23, nw_in, nw_pm);
  }
  cudaStream_t side[3] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[3] = {};
  // launches of one row-kernel step over the interior and CPML lists, whole
  // (part 0) or as its two halves (parts 1, 2)
  static int group_launches(bool split, int n_in, int n_pm) {
    return (split ? 2 : 1) * ((n_in > 0) + (n_pm > 0));
  }
  int fwd_launches() const {
    return (nwk[0] > 0) + (nwk[1] > 0) + (nwk[2] > 0) + (nwk[3] > 0);
  }
  // fn(stream, kind) for each kind with items (nk[kind] > 0), concurrently
  template <typename F>
  int kinds(cudaStream_t st, const int* nk, F&& fn);
  // fn(stream, interior, part) for each non-empty list (n_in interior items,
  // n_pm CPML items) and part, launched concurrently on the main stream and
  // the side streams (disjoint outputs)
  template <typename F>
  int group(cudaStream_t st, bool split, int n_in, int n_pm, F&& fn);
  int max_rcv = 0;                      // most receivers of a shot
  int64_t P = 0, fs = 0;
  char* pool = nullptr;
  ElShot<T>* d_shots = nullptr;
  ElModel<T> M{};
  T *d_lam = nullptr, *d_mu = nullptr, *d_rho = nullptr, *d_traces = nullptr,
    *d_resid = nullptr;
  double* d_partial = nullptr;
  double* d_gsrc = nullptr;  // every shot's d loss / d srcv block (source gradients)
  static constexpr int kBlocks = 512;
  size_t zero_fwd_off = 0, zero_fwd_len = 0, zero_adj_off = 0, zero_adj_len = 0;
  cudaStream_t cap = nullptr;
  cudaGraphExec_t eF = nullptr, eR = nullptr;
  cudaGraph_t gF = nullptr, gR = nullptr;
  int64_t nF = 0, nR = 0;

  ~ElPlan() override {
    if (eF) cudaGraphExecDestroy(eF);
    if (eR) cudaGraphExecDestroy(eR);
    if (gF) cudaGraphDestroy(gF);
    if (gR) cudaGraphDestroy(gR);
    if (cap) cudaStreamDestroy(cap);
    if (ev_fork) cudaEventDestroy(ev_fork);
    for (auto e : ev_join)
      if (e) cudaEventDestroy(e);
    for (auto q : side)
      if (q) cudaStreamDestroy(q);
    if (pool) cudaFree(pool);
  }

  dim3 grid3() const {
    return dim3((unsigned)div_up(NY + 2, BX), (unsigned)div_up(NX + 2, BY), (unsigned)nshots);
  }
  dim3 grid_rows(int nw) const { return dim3((unsigned)div_up(nw, EW), (unsigned)nshots); }
  // sources / receivers: one CTA per shot, a thread per receiver (up to 1024)
  unsigned rcv_threads() const {
    return (unsigned)std::min<int64_t>(1024, std::max<int64_t>(32, div_up(max_rcv, 32) * 32));
  }
  dim3 grid_resid() const {
    return dim3((unsigned)std::max<int64_t>(1, div_up(max_rcv, 256)), (unsigned)nshots);
  }

  int create(const ads_elastic_config& c, const ads_elastic_shot* shots, int64_t ns,
             cudaStream_t st);
  int step(cudaStream_t st, int n, bool store, int slot, bool record);
  int adjoint_step(cudaStream_t st, int slot, int n);
  int issue_forward(cudaStream_t st, int64_t* count);
  int issue_reverse(cudaStream_t st, int64_t* count);
  int prep(const double* l, const double* m, const double* r, cudaStream_t st);
  int forward(const double* l, const double* m, const double* r, void* traces,
              cudaStream_t st) override;
  int profile(const double* l, const double* m, const double* r, double* out,
              cudaStream_t st) override;
  int gradient(const double* l, const double* m, const double* r, const void* obs,
               double* loss, double* gl, double* gm, double* gr, void* tr_out,
               cudaStream_t st, double* grad_srcv) override;
  int max_src = 0;  // most sources of a shot
  bool src_grad = false;  // the reverse sweep records d loss / d srcv
};

template <typename T>
int ElPlan<T>::create(const ads_elastic_config& c, const ads_elastic_shot* shots, int64_t ns,
                      cudaStream_t st) {
  cfg = c;
  ADS_REQUIRE(ns >= 1 && ns < 65536, "nshots must be in [1, 65535]");
  ADS_REQUIRE(c.NX >= 4 && c.NY >= 4 && c.NX < (1 << 20) && c.NY < (1 << 20),
              "NX, NY must be in [4, 2^20)");
  ADS_REQUIRE(c.NSTEP >= 1 && c.NSTEP < (1 << 24), "NSTEP must be >= 1");
  ADS_REQUIRE(c.dx > 0 && c.dy > 0 && c.dt > 0 && std::isfinite(c.dx) && std::isfinite(c.dy) &&
                  std::isfinite(c.dt) && std::isfinite(c.vp_ref),
              "dx, dy, dt must be positive and finite (and vp_ref finite)");
  ADS_REQUIRE(c.npml >= 1 && c.Rcoef > 0 && c.Rcoef < 1, "invalid CPML parameters");
  ADS_REQUIRE(c.ckpt_every >= 0, "negative ckpt_every");
  ADS_REQUIRE(c.adjoint_passes == 0 || c.adjoint_passes == 1 || c.adjoint_passes == 3,
              "adjoint_passes must be 0, 1 or 3");
  // the fused kernels index a field with 32-bit offsets (a field this size
  // would not leave room for a plan on the device anyway)
  ADS_REQUIRE((int64_t)(c.NX + 2) * grid_pitch(c.NY) < (int64_t(1) << 31),
              "(NX + 2) x pitch must stay below 2^31 elements");
  // automatic (0): the fused adjoint for FP32 plans, the three passes for FP64
  // plans (their fused kernel runs out of registers: measured 1.5x slower)
  fused = c.adjoint_passes == 1 || (c.adjoint_passes == 0 && sizeof(T) == 4);
  if (fused)
    if (int e = el_fadj_prepare<T>()) return e;
  nshots = (int)ns;
  max_rcv = 0;
  for (int64_t s = 0; s < ns; s++) max_rcv = std::max<int>(max_rcv, (int)shots[s].nrcv);
  NX = (int)c.NX;
  NY = (int)c.NY;
  NSTEP = (int)c.NSTEP;
  for (int s = 0; s < ns; s++) {
    const ads_elastic_shot& h = shots[s];
    ADS_REQUIRE(h.nsrc >= 0 && h.nrcv >= 0, "shot %d: negative counts", s);
    ADS_REQUIRE(h.nsrc == 0 || (h.srci && h.srcj && h.srctype && h.srcv && h.srcv_rows >= NSTEP),
                "shot %d: source arrays missing or srcv_rows < NSTEP", s);
    ADS_REQUIRE(h.nrcv == 0 || (h.rcvi && h.rcvj && h.rcvtype), "shot %d: null receivers", s);
    for (int64_t k = 0; k < h.nsrc; k++)
      ADS_REQUIRE(h.srci[k] >= 1 && h.srci[k] <= NX + 2 && h.srcj[k] >= 1 &&
                      h.srcj[k] <= NY + 2,
                  "shot %d source %lld outside the padded grid", s, (long long)k);
    for (int64_t k = 0; k < h.nrcv; k++)
      ADS_REQUIRE(h.rcvi[k] >= 1 && h.rcvi[k] <= NX + 2 && h.rcvj[k] >= 1 &&
                      h.rcvj[k] <= NY + 2,
                  "shot %d receiver %lld outside the padded grid", s, (long long)k);
  }
  K = c.ckpt_every > 0 ? (int)std::min<int64_t>(c.ckpt_every, NSTEP) : std::min(NSTEP, 100);
  nseg = (int)div_up(NSTEP, K);
  src_grad = c.source_gradient != 0;
  // The reverse sweep computes adjoint fields only on cells a stencil updates,
  // so d loss / d srcv exists for sources on those cells alone.
  for (int s = 0; s < ns && src_grad; s++)
    for (int64_t k = 0; k < shots[s].nsrc; k++) {
      const int64_t t = shots[s].srctype[k];
      ADS_REQUIRE(t < 0 || t > 4 ||
                      el_cell_updated((int)t, shots[s].srci[k] - 1, shots[s].srcj[k] - 1, NX, NY),
                  "shot %d source %lld: source_gradient needs a cell the stencil of its field "
                  "updates, not the padded frame",
                  s, (long long)k);
    }
  src_off.resize(ns);
  src_total = 0;
  max_src = 0;
  for (int s = 0; s < ns; s++) {
    src_off[s] = src_total;
    src_total += (int64_t)NSTEP * shots[s].nsrc;
    max_src = std::max<int>(max_src, (int)shots[s].nsrc);
  }
  P = grid_pitch(NY);
  fs = (int64_t)(NX + 2) * P;
  // strips of ESTRIP columns cover 1..NY; rows per warp sized for about one
  // warp per SM slot (at least 8 rows to amortise the 4-row windows) unless given
  ncolw = (int)div_up(NY, ESTRIP);
  {
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess)
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t target = (int64_t)sms * 64;
    const int64_t work = (int64_t)ncolw * NX * ns;
    // (6 to 24 rows measured within 1% of each other on 600 x 300 x 32 shots)
    rows_w = c.rows_per_warp > 0 ? (int)c.rows_per_warp
                                 : (int)std::min<int64_t>(32, std::max<int64_t>(8, div_up(work, target)));
    ADS_REQUIRE(rows_w >= 1 && rows_w <= NX, "rows_per_warp must be in [1, NX]");
    // the fused step recomputes two stress rows on each side of a row tile:
    // 24-row tiles (measured best on 600 x 300 x 32 shots among 16..32),
    // shorter when that leaves less than about one wave of ~20 warps per SM
    const int64_t workf = (int64_t)div_up(NY, FSTRIP) * NX * ns;
    rows_f = c.rows_per_warp > 0
                 ? (int)c.rows_per_warp
                 : (int)std::min<int64_t>(
                       NX, std::min<int64_t>(24, std::max<int64_t>(
                                                     8, div_up(workf, (int64_t)sms * 20))));
    // the fused adjoint recomputes four rows on each side of a row tile: 24-row
    // tiles, shorter when that leaves less than about one wave of ~16 warps per SM
    rows_a = c.rows_per_warp > 0
                 ? (int)c.rows_per_warp
                 : (int)std::min<int64_t>(
                       NX, std::min<int64_t>(24, std::max<int64_t>(
                                                     8, div_up(workf, (int64_t)sms * 16))));
  }
  nwt = ncolw * (int)div_up(NX, rows_w);
  // the autotuner tries rows down to kTuneMinRows (adjoint) and
  // kTuneMinRowsF (fused step): the lists get room for those
  const int rw_min = c.autotune ? std::min(rows_w, kTuneMinRows) : rows_w;
  const int rf_min = c.autotune ? std::min(rows_f, kTuneMinRowsF) : rows_f;
  const int nwt_max = ncolw * (int)div_up(NX, rw_min);
  // upper bound of the fused items for any shift (the shifts are chosen once
  // the CPML profiles are known)
  const int nwtf_max =
      (int)(div_up(NY + FSTRIP - 2, FSTRIP) * div_up(NX + rf_min - 1, rf_min));
  const int ra_min = c.autotune ? std::min(rows_a, kTuneMinRowsF) : rows_a;
  const int nwta_max =
      (int)(div_up(NY + FSTRIP - 2, FSTRIP) * div_up(NX + ra_min - 1, ra_min));
  trace_off.resize(ns);
  trace_total = 0;
  for (int s = 0; s < ns; s++) {
    trace_off[s] = trace_total;
    trace_total += shots[s].nrcv * (int64_t)(NSTEP + 1);
  }
  // ---- layout
  struct Off {
    size_t state, g, tmp, store, ckpt, acc, acc32, srcv, scell, stype, sdual, rcell, rtype, sptr,
        rptr, gptr, sgptr;
  };
  std::vector<Off> o(ns);
  size_t used = 0;
  auto take = [&](size_t b) {
    const size_t r = used;
    used += (b + 255) & ~size_t(255);
    return r;
  };
  const size_t F = sizeof(T) * fs;
  const size_t fwd0 = used;
  for (int s = 0; s < ns; s++) o[s].state = take(2 * NF * F);  // two step buffers
  const size_t traces_o = take(sizeof(T) * std::max<int64_t>(trace_total, 1));
  zero_fwd_off = fwd0;
  zero_fwd_len = used - fwd0;
  const size_t adj0 = used;
  for (int s = 0; s < ns; s++) {
    o[s].g = take((fused ? 2 : 1) * NF * F);  // the fused adjoint alternates two buffers
    o[s].acc = take(3 * sizeof(double) * fs);
    o[s].acc32 = sizeof(T) == 4 ? take(3 * sizeof(float) * fs) : 0;
  }
  zero_adj_off = adj0;
  zero_adj_len = used - adj0;
  for (int s = 0; s < ns; s++) {
    const ads_elastic_shot& h = shots[s];
    o[s].tmp = fused ? 0 : take(NTMP * F);  // D1..D8, R4, GL1, GM1, GM2 of the three passes
    o[s].ckpt = take((size_t)nseg * NF * F);
    o[s].srcv = take(sizeof(T) * std::max<int64_t>(NSTEP * h.nsrc, 1));
    o[s].scell = take(sizeof(int64_t) * std::max<int64_t>(h.nsrc, 1));
    o[s].stype = take(sizeof(int) * std::max<int64_t>(h.nsrc, 1));
    o[s].sdual = take(sizeof(int) * std::max<int64_t>(h.nsrc, 1));
    o[s].rcell = take(sizeof(int64_t) * std::max<int64_t>(h.nrcv, 1));
    o[s].rtype = take(sizeof(int) * std::max<int64_t>(h.nrcv, 1));
    o[s].sptr = take(sizeof(T*) * std::max<int64_t>(h.nsrc, 1));
    o[s].rptr = take(sizeof(T*) * std::max<int64_t>(h.nrcv, 1));
    o[s].gptr = take(sizeof(T*) * std::max<int64_t>(h.nrcv, 1));
    o[s].sgptr = take(sizeof(T*) * std::max<int64_t>(h.nsrc, 1));
  }
  const size_t model_o = take(3 * F);
  const size_t prof_o = take(sizeof(T) * (4 * NX + 4 * NY));
  const size_t resid_o = take(sizeof(T) * std::max<int64_t>(trace_total, 1));
  const size_t part_o = take(sizeof(double) * kBlocks);
  const size_t gsrc_o = take(sizeof(double) * (src_grad ? std::max<int64_t>(src_total, 1) : 1));
  const size_t shots_o = take(sizeof(ElShot<T>) * ns);
  const size_t wl_o = take(sizeof(int) * std::max(nwt_max, 1));
  const size_t wlf_o = take(sizeof(int) * std::max(nwtf_max, 1));
  const size_t wla_o = take(sizeof(int) * std::max(fused ? nwta_max : 1, 1));
  // ---- the shots' stores: K slots for a segment's recompute, then one slot
  // per step of the resident segments (the last ones that fit in the allowed
  // share of the free device memory)
  res_seg = nseg;
  {
    const size_t slot = (size_t)NSTORE * F;
    const size_t base_bytes = used + (size_t)ns * ((size_t)K * slot + 256);
    if (c.resident_segments >= 0) {
      size_t fr = 0, tot = 0, avail = 0;
      if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr > base_bytes) {
        const int pct = c.resident_mem_pct > 0 ? std::min<int>(c.resident_mem_pct, 95) : 50;
        avail = (size_t)((double)(fr - base_bytes) * pct / 100.0);
      } else {
        cudaGetLastError();
      }
      const int lo = c.resident_segments > 0 ? std::max(0, nseg - (int)c.resident_segments) : 0;
      for (int sg = nseg - 1; sg >= lo; sg--) {
        const size_t b = (size_t)ns * ((size_t)(NSTEP - sg * K) * slot + 256);
        if (b > avail) break;
        res_seg = sg;
      }
    }
    const size_t slots = (size_t)K + (res_seg < nseg ? NSTEP - res_seg * K : 0);
    for (int s = 0; s < ns; s++) o[s].store = take(slots * slot);
  }
  bytes = (int64_t)used;
  resident = nseg - res_seg;
  {
    cudaError_t e = cudaMalloc(&pool, used);
    if (e != cudaSuccess) {
      cudaGetLastError();
      pool = nullptr;
      return fail(ADS_ERR_NOMEM, "device allocation of %.3f GB for the plan failed: %s",
                  used / 1e9, cudaGetErrorString(e));
    }
  }
  ADS_CUDA(cudaMemsetAsync(pool, 0, used, st));
  d_lam = (T*)(pool + model_o);
  d_mu = d_lam + fs;
  d_rho = d_mu + fs;
  d_traces = (T*)(pool + traces_o);
  d_resid = (T*)(pool + resid_o);
  d_partial = (double*)(pool + part_o);
  d_gsrc = (double*)(pool + gsrc_o);
  d_shots = (ElShot<T>*)(pool + shots_o);
  // profiles
  std::vector<double> ax(2 * NX), bx(2 * NX), kx(2 * NX), ay(2 * NY), by(2 * NY), ky(2 * NY);
  elastic_cpml(NX, NY, c.dx, c.dy, c.dt, c.npml, c.npower, c.k_max, c.alpha_max, c.vp_ref,
               c.Rcoef, c.use_pml, ax.data(), bx.data(), kx.data(), ay.data(), by.data(),
               ky.data());
  hprof = pack_profiles<T>(NX, NY, ax.data(), bx.data(), ay.data(), by.data());
  const std::vector<T>& prof = hprof;
  build_lists(rows_w, rows_f, rows_a);
  d_wl = (int*)(pool + wl_o);
  d_wlf = (int*)(pool + wlf_o);
  d_wla = (int*)(pool + wla_o);
  if (int e = upload_lists(st)) return e;
  for (auto& q : side) ADS_CUDA(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
  ADS_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
  for (auto& e : ev_join) ADS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  ADS_CUDA(cudaMemcpyAsync(pool + prof_o, prof.data(), sizeof(T) * prof.size(),
                           cudaMemcpyHostToDevice, st));
  M = make_model<T>(NX, NY, P, JOFF, c.dt, c.dx, c.dy, d_lam, d_mu, d_rho,
                    (const T*)(pool + prof_o));
  // shots
  std::vector<ElShot<T>> hs(ns);
  srcv_dev.assign(ns, nullptr);
  srcv_n.assign(ns, 0);
  std::vector<std::vector<char>> stage;
  for (int s = 0; s < ns; s++) {
    const ads_elastic_shot& h = shots[s];
    ElShot<T>& d = hs[s];
    for (int f = 0; f < NF; f++) {
      d.f[f] = (T*)(pool + o[s].state) + f * fs;
      d.fin[f] = d.f[f];
      d.g[f] = (T*)(pool + o[s].g) + f * fs;
    }
    for (int k = 0; k < NTMP; k++) d.tmp[k] = fused ? nullptr : (T*)(pool + o[s].tmp) + k * fs;
    d.store = (T*)(pool + o[s].store);
    d.ckpt = (T*)(pool + o[s].ckpt);
    d.glam = (double*)(pool + o[s].acc);
    d.gmu = d.glam + fs;
    d.grho = d.gmu + fs;
    d.gl32 = sizeof(T) == 4 ? (float*)(pool + o[s].acc32) : nullptr;
    d.gm32 = d.gl32 ? d.gl32 + fs : nullptr;
    d.gr32 = d.gl32 ? d.gm32 + fs : nullptr;
    d.traces = d_traces + trace_off[s];
    d.resid = d_resid + trace_off[s];
    d.srcv = (const T*)(pool + o[s].srcv);
    srcv_dev[s] = (T*)d.srcv;
    srcv_n[s] = (int64_t)NSTEP * h.nsrc;
    d.src_cell = (const int64_t*)(pool + o[s].scell);
    d.src_type = (const int*)(pool + o[s].stype);
    d.src_dual = (const int*)(pool + o[s].sdual);
    d.rcv_cell = (const int64_t*)(pool + o[s].rcell);
    d.rcv_type = (const int*)(pool + o[s].rtype);
    d.src_ptr = (T* const*)(pool + o[s].sptr);
    d.rcv_ptr = (T* const*)(pool + o[s].rptr);
    d.rcv_gptr = (T* const*)(pool + o[s].gptr);
    d.src_gptr = (T* const*)(pool + o[s].sgptr);
    d.gsrc = src_grad ? d_gsrc + src_off[s] : nullptr;
    d.nsrc = (int)h.nsrc;
    d.nrcv = (int)h.nrcv;
    d.fs = fs;
    if (h.nsrc > 0) {
      std::vector<T> sv((size_t)NSTEP * h.nsrc);
      for (int64_t r = 0; r < NSTEP; r++)
        for (int64_t k = 0; k < h.nsrc; k++) sv[r * h.nsrc + k] = (T)h.srcv[r * h.nsrc + k];
      std::vector<int64_t> cell(h.nsrc);
      std::vector<int> type(h.nsrc);
      for (int64_t k = 0; k < h.nsrc; k++) {
        cell[k] = (h.srci[k] - 1) * P + (h.srcj[k] - 1) + JOFF;
        type[k] = (int)h.srctype[k];
      }
      stage.emplace_back((char*)sv.data(), (char*)(sv.data() + sv.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.srcv, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
      stage.emplace_back((char*)cell.data(), (char*)(cell.data() + cell.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.src_cell, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
      stage.emplace_back((char*)type.data(), (char*)(type.data() + type.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.src_type, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
      // sources on cells outside the update box of their field (vx: rows and
      // columns 2..N; vy: 1..N-1; sxx, syy: rows 1..NX-1, columns 2..NY;
      // sxy: rows 2..NX, columns 1..NY-1) are added to both state buffers
      std::vector<int> dual(h.nsrc);
      for (int64_t k = 0; k < h.nsrc; k++) {
        const int64_t i = h.srci[k] - 1, jj = h.srcj[k] - 1;
        dual[k] = el_cell_updated(type[k], i, jj, NX, NY) ? 0 : 1;
      }
      stage.emplace_back((char*)dual.data(), (char*)(dual.data() + dual.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.src_dual, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
      std::vector<T*> ptr(h.nsrc), gptr(h.nsrc);
      for (int64_t k = 0; k < h.nsrc; k++) {
        const bool ok = type[k] >= 0 && type[k] <= 4;
        ptr[k] = ok ? d.f[type[k]] + cell[k] : nullptr;
        gptr[k] = ok ? d.g[type[k]] + cell[k] : nullptr;
      }
      stage.emplace_back((char*)ptr.data(), (char*)(ptr.data() + ptr.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.src_ptr, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
      stage.emplace_back((char*)gptr.data(), (char*)(gptr.data() + gptr.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.src_gptr, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
    }
    if (h.nrcv > 0) {
      std::vector<int64_t> cell(h.nrcv);
      std::vector<int> type(h.nrcv);
      for (int64_t k = 0; k < h.nrcv; k++) {
        cell[k] = (h.rcvi[k] - 1) * P + (h.rcvj[k] - 1) + JOFF;
        type[k] = (int)h.rcvtype[k];
      }
      stage.emplace_back((char*)cell.data(), (char*)(cell.data() + cell.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.rcv_cell, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
      stage.emplace_back((char*)type.data(), (char*)(type.data() + type.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.rcv_type, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
      std::vector<T*> ptr(h.nrcv), gptr(h.nrcv);
      for (int64_t k = 0; k < h.nrcv; k++) {
        const bool ok = type[k] >= 0 && type[k] <= 4;
        ptr[k] = ok ? d.f[type[k]] + cell[k] : nullptr;
        gptr[k] = ok ? d.g[type[k]] + cell[k] : nullptr;
      }
      stage.emplace_back((char*)ptr.data(), (char*)(ptr.data() + ptr.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.rcv_ptr, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
      stage.emplace_back((char*)gptr.data(), (char*)(gptr.data() + gptr.size()));
      ADS_CUDA(cudaMemcpyAsync((void*)d.rcv_gptr, stage.back().data(), stage.back().size(),
                               cudaMemcpyHostToDevice, st));
    }
  }
  ADS_CUDA(cudaMemcpyAsync(d_shots, hs.data(), sizeof(ElShot<T>) * ns, cudaMemcpyHostToDevice,
                           st));
  ADS_CUDA(cudaStreamSynchronize(st));
  if (c.autotune && c.rows_per_warp <= 0)
    if (int e = autotune(st, rw_min, rf_min)) return e;
  tiling[0] = fused ? rows_a : rows_w;
  tiling[1] = rows_f;
  for (int k = 0; k < 4; k++) adj_items[k] = fused ? nwka[k] : 0;
  {
    int64_t n = 0;
    issue_forward(nullptr, &n);
    nF = n;
    issue_reverse(nullptr, &n);
    nR = n;
  }
  launches_fwd = 3 + nF;
  launches_grad = 3 + nF + 2 + nR + 1;
  if (c.use_graph) {
    ADS_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    for (int which = 0; which < 2; which++) {
      ADS_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
      set_launch_counting(false);
      int rc = which == 0 ? issue_forward(cap, nullptr) : issue_reverse(cap, nullptr);
      set_launch_counting(true);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(cap, &g);
      if (rc != ADS_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      ADS_CUDA(e);
      cudaGraphExec_t ex = nullptr;
      ADS_CUDA(cudaGraphInstantiate(&ex, g, 0));
      (which == 0 ? gF : gR) = g;
      (which == 0 ? eF : eR) = ex;
    }
  }
  return ADS_OK;
}

// Warp items of the tiling rows_w = rw (adjoint passes) and rows_f = rf (the
// fused step), from the packed CPML rows hprof.
template <typename T>
void ElPlan<T>::build_lists(int rw, int rf, int ra) {
  rows_w = rw;
  rows_f = rf;
  rows_a = ra;
  nwt = ncolw * (int)div_up(NX, rows_w);
  wl_host.clear();
  wlf_host.clear();
  wla_host.clear();
  // warp items: a (strip, row tile) is interior when every cell it updates lies
  // inside all four update boxes (2 <= i <= NX-1, 2 <= j <= NY-1) with no
  // active CPML profile on its rows and columns (as the kernels see them)
  const T *axi = hprof.data(), *axh = axi + NX, *bxi = axi + 2 * NX, *bxh = axi + 3 * NX;
  const T *ayi = axi + 4 * NX, *ayh = ayi + NY, *byi = ayi + 2 * NY, *byh = ayi + 3 * NY;
  std::vector<char> row_ok(NX + 2, 0), col_ok(NY + 2, 0);
  for (int i = 2; i <= NX - 1; i++)
    row_ok[i] = axh[i - 1] == T(0) && bxh[i - 1] == T(1) && axi[i - 1] == T(0) &&
                bxi[i - 1] == T(1);
  for (int jc = 2; jc <= NY - 1; jc++)
    col_ok[jc] = ayi[jc - 1] == T(0) && byi[jc - 1] == T(1) && ayh[jc - 1] == T(0) &&
                 byh[jc - 1] == T(1);
  std::vector<int> wpm;
  for (int wi = 0; wi < nwt; wi++) {
    const int strip = wi % ncolw, rt = wi / ncolw;
    const int i0 = 1 + rt * rows_w, i1 = std::min(i0 + rows_w, NX + 1);
    bool ok = true;
    for (int i = i0; i < i1 && ok; i++) ok = row_ok[i];
    for (int jc = strip * ESTRIP + 1; jc <= strip * ESTRIP + ESTRIP && ok; jc++)
      ok = jc <= NY - 1 && col_ok[jc];
    (ok ? wl_host : wpm).push_back(wi);
  }
  nw_in = (int)wl_host.size();
  nw_pm = (int)wpm.size();
  wl_host.insert(wl_host.end(), wpm.begin(), wpm.end());
  // Items of a fused kernel (FSTRIP-column strips, R-row tiles) by kind: bit 0
  // when a row it computes (hr rows beyond its own on each side) lies on a box
  // edge or in the x-CPML, bit 1 when a column of its computing lanes (hc
  // columns beyond its own on each side) lies on a box edge or in the y-CPML.
  // The strip and tile origins are shifted (js, is <= 0) to make the most
  // strips and tiles CPML-free (then the fewest).
  auto fused_items = [&](int R, int hr, int hc, int& js, int& is, int& ncol, int& nwtot,
                         int (&nk)[4], int (&ok)[4], std::vector<int>& out) {
    auto tile_ok = [&](int rt, int sh_) {
      const int i0r = 1 + sh_ + rt * R;
      const int i0 = std::max(i0r, 1), i1 = std::min(i0r + R, NX + 1);
      for (int i = i0 - hr; i <= i1 - 1 + hr; i++)
        if (i < 0 || i > NX + 1 || !row_ok[i]) return false;
      return true;
    };
    auto strip_ok = [&](int strip, int sh_) {
      const int a = 1 + sh_ + strip * FSTRIP;
      for (int jc = a - hc; jc <= a + FSTRIP - 1 + hc; jc++)
        if (jc < 0 || jc > NY + 1 || !col_ok[jc]) return false;
      return true;
    };
    int best = -1, bestn = 0;
    for (int sh_ = 0; sh_ > -FSTRIP; sh_ -= 2) {
      const int n = (int)div_up(NY - sh_, FSTRIP);
      int k = 0;
      for (int s = 0; s < n; s++) k += strip_ok(s, sh_);
      if (k > best || (k == best && n < bestn)) {
        best = k;
        bestn = n;
        js = sh_;
      }
    }
    ncol = bestn;
    best = -1;
    int bestt = 0;
    for (int sh_ = 0; sh_ > -R; sh_--) {
      const int n = (int)div_up(NX - sh_, R);
      int k = 0;
      for (int s = 0; s < n; s++) k += tile_ok(s, sh_);
      if (k > best || (k == best && n < bestt)) {
        best = k;
        bestt = n;
        is = sh_;
      }
    }
    nwtot = ncol * bestt;
    std::vector<int> wk[4];
    for (int wi = 0; wi < nwtot; wi++) {
      const int strip = wi % ncol, rt = wi / ncol;
      wk[(tile_ok(rt, is) ? 0 : 1) | (strip_ok(strip, js) ? 0 : 2)].push_back(wi);
    }
    for (int k = 0; k < 4; k++) {
      ok[k] = (int)out.size();
      nk[k] = (int)wk[k].size();
      out.insert(out.end(), wk[k].begin(), wk[k].end());
    }
  };
  // the fused step computes stresses two rows and one lane (two columns)
  // beyond what it owns; the fused adjoint runs phase A four rows and two
  // lanes beyond
  fused_items(rows_f, 2, 2, jsh, ish, ncolf, nwtf, nwk, owk, wlf_host);
  if (fused) fused_items(rows_a, 4, 4, jsha, isha, ncola, nwta, nwka, owka, wla_host);
}

template <typename T>
int ElPlan<T>::upload_lists(cudaStream_t st) {
  ADS_CUDA(cudaMemcpyAsync(d_wl, wl_host.data(), sizeof(int) * wl_host.size(),
                           cudaMemcpyHostToDevice, st));
  if (!wlf_host.empty())
    ADS_CUDA(cudaMemcpyAsync(d_wlf, wlf_host.data(), sizeof(int) * wlf_host.size(),
                             cudaMemcpyHostToDevice, st));
  if (!wla_host.empty())
    ADS_CUDA(cudaMemcpyAsync(d_wla, wla_host.data(), sizeof(int) * wla_host.size(),
                             cudaMemcpyHostToDevice, st));
  ADS_CUDA(cudaStreamSynchronize(st));  // the host lists change between trials
  return ADS_OK;
}

// Autotuner: time the fused step for candidate tile heights rows_f, then the
// three adjoint passes for candidate strip heights rows_w, on the plan's own
// buffers (CUDA events on `st`), and keep the fastest of each.  The state the
// trials touch is reset by every forward / gradient call.
template <typename T>
int ElPlan<T>::autotune(cudaStream_t st, int rw_min, int rf_min) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ADS_CUDA(cudaEventCreate(&e0));
  ADS_CUDA(cudaEventCreate(&e1));
  auto timed = [&](bool adj, float& ms) -> int {
    for (int pass = 0; pass < 2; pass++) {  // pass 0 warms up
      ADS_CUDA(cudaEventRecord(e0, st));
      for (int n = 1; n <= 6; n++)
        if (int e = adj ? adjoint_step(st, 0, n) : step(st, n, false, 0, false)) return e;
      ADS_CUDA(cudaEventRecord(e1, st));
      ADS_CUDA(cudaEventSynchronize(e1));
      ADS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    }
    return ADS_OK;
  };
  int rc = ADS_OK;
  int best_f = rows_f, best_w = rows_w;
  float best = 1e30f;
  for (int rf : {12, 16, 20, 24, 32}) {
    if (rf < rf_min || rf > NX) continue;
    build_lists(best_w, rf, rows_a);
    float ms = 0.f;
    if ((rc = upload_lists(st)) || (rc = timed(false, ms))) break;
    if (ms < best) {
      best = ms;
      best_f = rf;
    }
  }
  best = 1e30f;
  int best_a = rows_a;
  // the fused adjoint: tile heights as the fused step's; the three passes:
  // strip heights
  const std::vector<int> cand =
      fused ? std::vector<int>{12, 16, 20, 24, 32} : std::vector<int>{6, 8, 12, 16, 24, 32};
  for (int rw : cand) {
    if (rc != ADS_OK) break;
    if ((!fused && rw < rw_min) || rw > NX) continue;  // (the lists hold >= 12-row tiles)
    if (fused) {
      build_lists(best_w, best_f, rw);
    } else {
      build_lists(rw, best_f, rows_a);
    }
    float ms = 0.f;
    if ((rc = upload_lists(st)) || (rc = timed(true, ms))) break;
    if (ms < best) {
      best = ms;
      (fused ? best_a : best_w) = rw;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != ADS_OK) return rc;
  build_lists(best_w, best_f, best_a);
  return upload_lists(st);
}

// One forward step n (slot n-1 -> slot n) for every shot.
template <typename T>
template <typename F>
int ElPlan<T>::group(cudaStream_t st, bool split, int n_in, int n_pm, F&& fn) {
  // the CPML items first, as in kinds() (FP64 three-pass gradient, 4 shots
  // on the C4 grid: 1017 against 1059 ms with the CPML-free items first)
  bool in_[4];
  int part_[4], n = 0;
  for (int l = 0; l < 2; l++) {
    const bool in = l == 1;
    if ((in ? n_in : n_pm) == 0) continue;
    for (int part = split ? 1 : 0; part <= (split ? 2 : 0); part++) {
      in_[n] = in;
      part_[n++] = part;
    }
  }
  if (n > 1) {
    ADS_CUDA(cudaEventRecord(ev_fork, st));
    for (int k = 1; k < n; k++) ADS_CUDA(cudaStreamWaitEvent(side[k - 1], ev_fork, 0));
  }
  for (int k = 0; k < n; k++) {
    fn(k == 0 ? st : side[k - 1], in_[k], part_[k]);
    ADS_LAUNCHED(1);
  }
  for (int k = 1; k < n; k++) {
    ADS_CUDA(cudaEventRecord(ev_join[k - 1], side[k - 1]));
    ADS_CUDA(cudaStreamWaitEvent(st, ev_join[k - 1], 0));
  }
  return ADS_OK;
}

template <typename T>
template <typename F>
int ElPlan<T>::kinds(cudaStream_t st, const int* nk, F&& fn) {
  // The CPML kinds first: their few items carry the longest chains, and the
  // launches of a fork start roughly in the order they are issued (measured
  // on the C4 gradient: 20.1 shot-gradients/s against 17.4 with kind 0 first)
  int kd[4], n = 0;
  for (int k = 3; k >= 0; k--)
    if (nk[k] > 0) kd[n++] = k;
  if (n > 1) {
    ADS_CUDA(cudaEventRecord(ev_fork, st));
    for (int k = 1; k < n; k++) ADS_CUDA(cudaStreamWaitEvent(side[k - 1], ev_fork, 0));
  }
  for (int k = 0; k < n; k++) {
    fn(k == 0 ? st : side[k - 1], kd[k]);
    ADS_LAUNCHED(1);
  }
  for (int k = 1; k < n; k++) {
    ADS_CUDA(cudaEventRecord(ev_join[k - 1], side[k - 1]));
    ADS_CUDA(cudaStreamWaitEvent(st, ev_join[k - 1], 0));
  }
  return ADS_OK;
}

// The adjoint of step n (store slot `slot`): the fused kernel's launches over
// the item kinds (adjoint of slot n in buffer apar(n) -> slot n-1 in the
// other), or the three passes in place.
template <typename T>
int ElPlan<T>::adjoint_step(cudaStream_t st, int slot, int n) {
  if (fused)
    return kinds(st, nwka, [&](cudaStream_t s, int k) {
      el_fadj<T>(k, grid_rows(nwka[k]), s, M, d_shots, d_wla + owka[k], ncola, rows_a, nwka[k],
                 slot, apar(n), jsha, isha);
    });
  auto wl = [&](bool in) { return in ? d_wl : d_wl + nw_in; };
  auto nw = [&](bool in) { return in ? nw_in : nw_pm; };
  if (int e = group(st, kSplitAdj1, nw_in, nw_pm, [&](cudaStream_t s, bool in, int part) {
        el_adj1<T>(in, part, grid_rows(nw(in)), s, M, d_shots, wl(in), ncolw, rows_w, nw(in),
                   slot);
      }))
    return e;
  if (int e = group(st, kSplitAdj23, nw_in, nw_pm, [&](cudaStream_t s, bool in, int part) {
        el_adj2<T>(in, part, grid_rows(nw(in)), s, M, d_shots, wl(in), ncolw, rows_w, nw(in),
                   slot);
      }))
    return e;
  return group(st, kSplitAdj23, nw_in, nw_pm, [&](cudaStream_t s, bool in, int part) {
    el_adj3<T>(in, part, grid_rows(nw(in)), s, M, d_shots, wl(in), ncolw, rows_w, nw(in));
  });
}

// One forward step n (slot n-1 in buffer par(n-1) -> slot n in buffer
// par(n)) for every shot.
template <typename T>
int ElPlan<T>::step(cudaStream_t st, int n, bool store, int slot, bool record) {
  const int sl = store ? slot : 0;
  if (int e = kinds(st, nwk, [&](cudaStream_t s, int k) {
        el_step<T>(store, k, grid_rows(nwk[k]), s, M, d_shots, d_wlf + owk[k], ncolf, rows_f,
                   nwk[k], sl, par(n - 1), jsh, ish);
      }))
    return e;
  k_el_src_rcv<T><<<nshots, rcv_threads(), 0, st>>>(d_shots, n, NSTEP + 1, record ? 1 : 0,
                                                    par(n), 1);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

template <typename T>
int ElPlan<T>::issue_forward(cudaStream_t st, int64_t* count) {
  if (count) {
    int64_t c = 0;
    for (int n = 1; n <= NSTEP; n++)
      c += fwd_launches() + 1 + ((n % K == 0 && n / K < res_seg) ? 1 : 0);
    *count = c;
    return ADS_OK;
  }
  ADS_CUDA(cudaMemsetAsync(pool + zero_fwd_off, 0, zero_fwd_len, st));
  for (int n = 1; n <= NSTEP; n++) {
    // steps of resident segments store what their adjoint steps read
    const bool res = n >= a_res();
    if (int e = step(st, n, res, res ? K + n - a_res() : 0, true)) return e;
    // checkpoint s holds slot s*K (state before step sK+1); resident segments need none
    if (n % K == 0 && n / K < res_seg) {
      k_el_ckpt<T><<<dim3(256, nshots), 256, 0, st>>>(d_shots, n / K, 1, par(n), 0);
      ADS_LAUNCHED(1);
    }
  }
  return ADS_OK;
}

template <typename T>
int ElPlan<T>::issue_reverse(cudaStream_t st, int64_t* count) {
  if (count) {
    int64_t c = 1;
    for (int s = nseg - 1; s >= 0; s--) {
      const int a = 1 + s * K, b = std::min(a + K - 1, NSTEP);
      if (s < res_seg) c += 1 + (fwd_launches() + 1) * (b - a + 1);
      c += adj_launches() * (b - a + 1) +
           (b - std::max(a, 2) + 1) + (src_grad ? b - a + 1 : 0) +
           (sizeof(T) == 4 ? 1 : 0);
    }
    *count = c;
    return ADS_OK;
  }
  ADS_CUDA(cudaMemsetAsync(pool + zero_adj_off, 0, zero_adj_len, st));
  k_el_resid<T><<<grid_resid(), 256, 0, st>>>(d_shots, NSTEP, NSTEP + 1, apar(NSTEP));
  ADS_LAUNCHED(1);
  for (int s = nseg - 1; s >= 0; s--) {
    const int a = 1 + s * K, b = std::min(a + K - 1, NSTEP);
    const bool res = s >= res_seg;  // resident: the store already holds the segment
    const int slot0 = res ? K + a - a_res() : 0;  // store slot of step a
    if (!res) {
      k_el_ckpt<T><<<dim3(256, nshots), 256, 0, st>>>(d_shots, s, 0, 0, 1);
      ADS_LAUNCHED(1);
      for (int n = a; n <= b; n++)
        if (int e = step(st, n, true, n - a, false)) return e;
    }
    for (int n = b; n >= a; n--) {
      if (src_grad) {  // the adjoint state refers to slot n, its residual included
        k_el_src_grad<T><<<dim3((unsigned)div_up(std::max(max_src, 1), 128), nshots), 128, 0,
                            st>>>(d_shots, n, apar(n));
        ADS_LAUNCHED(1);
      }
      if (int e = adjoint_step(st, slot0 + n - a, n)) return e;
      // the adjoint state now refers to slot n-1: add its residual (slot 0 is
      // the constant zero state and takes none)
      if (n - 1 >= 1) {
        k_el_resid<T><<<grid_resid(), 256, 0, st>>>(d_shots, n - 1, NSTEP + 1, apar(n - 1));
        ADS_LAUNCHED(1);
      }
    }
    if constexpr (sizeof(T) == 4) {
      k_el_flush_acc<<<dim3(256, nshots), 256, 0, st>>>(d_shots, fs);
      ADS_LAUNCHED(1);
    }
  }
  return ADS_OK;
}

template <typename T>
int ElPlan<T>::prep(const double* l, const double* m, const double* r, cudaStream_t st) {
  ADS_REQUIRE(l && m && r, "null model arrays");
  const unsigned g = (unsigned)std::min<int64_t>(div_up((int64_t)(NX + 2) * (NY + 2), 256), 4096);
  k_el_cast<T><<<g, 256, 0, st>>>(d_lam, l, NX, NY, P, JOFF);
  ADS_LAUNCHED(1);
  k_el_cast<T><<<g, 256, 0, st>>>(d_mu, m, NX, NY, P, JOFF);
  ADS_LAUNCHED(1);
  k_el_cast<T><<<g, 256, 0, st>>>(d_rho, r, NX, NY, P, JOFF);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

template <typename T>
int ElPlan<T>::forward(const double* l, const double* m, const double* r, void* traces,
                       cudaStream_t st) {
  if (int e = prep(l, m, r, st)) return e;
  if (eF) {
    ADS_CUDA(cudaGraphLaunch(eF, st));
    note_launches(nF);
  } else if (int e = issue_forward(st, nullptr)) {
    return e;
  }
  if (traces)
    ADS_CUDA(cudaMemcpyAsync(traces, d_traces, sizeof(T) * trace_total,
                             cudaMemcpyDeviceToDevice, st));
  return ADS_OK;
}

template <typename T>
int ElPlan<T>::gradient(const double* l, const double* m, const double* r, const void* obs,
                        double* loss, double* gl, double* gm, double* gr, void* tr_out,
                        cudaStream_t st, double* grad_srcv) {
  ADS_REQUIRE(obs && loss && gl && gm && gr, "null argument");
  ADS_REQUIRE(!grad_srcv || src_grad,
              "grad_srcv needs a plan created with source_gradient = 1");
  if (int e = forward(l, m, r, nullptr, st)) return e;
  k_el_misfit<T><<<kBlocks, 256, 0, st>>>(d_traces, (const T*)obs, d_resid, trace_total,
                                          d_partial);
  ADS_LAUNCHED(1);
  k_el_reduce<<<1, 1024, 0, st>>>(d_partial, kBlocks, loss);
  ADS_LAUNCHED(1);
  if (eR) {
    ADS_CUDA(cudaGraphLaunch(eR, st));
    note_launches(nR);
  } else if (int e = issue_reverse(st, nullptr)) {
    return e;
  }
  const unsigned g = (unsigned)std::min<int64_t>(div_up((int64_t)(NX + 2) * (NY + 2), 256), 4096);
  k_el_gather_grads<T><<<g, 256, 0, st>>>(d_shots, nshots, NX, NY, P, JOFF, gl, gm, gr);
  ADS_LAUNCHED(1);
  if (tr_out)
    ADS_CUDA(cudaMemcpyAsync(tr_out, d_traces, sizeof(T) * trace_total,
                             cudaMemcpyDeviceToDevice, st));
  if (grad_srcv && src_total > 0)  // the shots' blocks are contiguous, in the caller's order
    ADS_CUDA(cudaMemcpyAsync(grad_srcv, d_gsrc, sizeof(double) * src_total,
                             cudaMemcpyDeviceToDevice, st));
  return ADS_OK;
}

// Per-kernel durations: each step kernel of the plan launched kProfileReps
// times back to back on the plan's buffers between two events (direct
// launches; the state is scratch afterwards and the next forward / gradient
// starts from zero as always).  out[2k] = ms per launch, out[2k+1] = interior
// cell-updates per launch, for k = forward step (the fused kernel's launches
// over the item kinds), forward step storing the adjoint's strains, adjoint
// 1, adjoint 2, adjoint 3, sources / receivers, residual injection.
template <typename T>
int ElPlan<T>::profile(const double* l, const double* m, const double* r, double* out,
                       cudaStream_t st) {
  ADS_REQUIRE(out, "null argument");
  if (int e = prep(l, m, r, st)) return e;
  constexpr int kProfileReps = 20;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ADS_CUDA(cudaEventCreate(&e0));
  ADS_CUDA(cudaEventCreate(&e1));
  const double cells = (double)nshots * NX * NY;
  auto timed = [&](int k, auto&& launch) -> int {
    launch();  // warm-up
    ADS_CUDA(cudaEventRecord(e0, st));
    for (int rep = 0; rep < kProfileReps; rep++) launch();
    ADS_CUDA(cudaEventRecord(e1, st));
    ADS_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    ADS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    out[2 * k] = ms / kProfileReps;
    out[2 * k + 1] = cells;
    return ADS_OK;
  };
  int rc = ADS_OK;
  auto run = [&](int k, auto&& launch) {
    if (rc == ADS_OK) rc = timed(k, launch);
  };
  ADS_CUDA(cudaMemsetAsync(pool + zero_fwd_off, 0, zero_fwd_len, st));
  ADS_CUDA(cudaMemsetAsync(pool + zero_adj_off, 0, zero_adj_len, st));
  auto wl = [&](bool in) { return in ? d_wl : d_wl + nw_in; };
  auto nw = [&](bool in) { return in ? nw_in : nw_pm; };
  for (int k = 0; k < 2; k++)
    run(k, [&] {
      kinds(st, nwk, [&](cudaStream_t s, int kd) {
        el_step<T>(k == 1, kd, grid_rows(nwk[kd]), s, M, d_shots, d_wlf + owk[kd], ncolf,
                   rows_f, nwk[kd], 0, 0, jsh, ish);
      });
    });
  if (fused) {  // the fused adjoint in slot 2; slots 3 and 4 stay empty
    run(2, [&] { adjoint_step(st, 0, 1); });
    out[6] = out[8] = 0.0;
    out[7] = out[9] = cells;
  }
  if (!fused) run(2, [&] {
    group(st, kSplitAdj1, nw_in, nw_pm, [&](cudaStream_t s, bool in, int part) {
      el_adj1<T>(in, part, grid_rows(nw(in)), s, M, d_shots, wl(in), ncolw, rows_w, nw(in), 0);
    });
  });
  if (!fused) run(3, [&] {
    group(st, kSplitAdj23, nw_in, nw_pm, [&](cudaStream_t s, bool in, int part) {
      el_adj2<T>(in, part, grid_rows(nw(in)), s, M, d_shots, wl(in), ncolw, rows_w, nw(in), 0);
    });
  });
  if (!fused) run(4, [&] {
    group(st, kSplitAdj23, nw_in, nw_pm, [&](cudaStream_t s, bool in, int part) {
      el_adj3<T>(in, part, grid_rows(nw(in)), s, M, d_shots, wl(in), ncolw, rows_w, nw(in));
    });
  });
  run(5, [&] {
    k_el_src_rcv<T><<<nshots, rcv_threads(), 0, st>>>(d_shots, 1, NSTEP + 1, 1, 0, 0);
  });
  run(6, [&] { k_el_resid<T><<<grid_resid(), 256, 0, st>>>(d_shots, 1, NSTEP + 1, 0); });
  note_launches(2 * (kProfileReps + 1));  // the pairs count their own launches
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != ADS_OK) return rc;
  ADS_CUDA(cudaGetLastError());
  // leave zeroed state behind
  ADS_CUDA(cudaMemsetAsync(pool + zero_fwd_off, 0, zero_fwd_len, st));
  ADS_CUDA(cudaMemsetAsync(pool + zero_adj_off, 0, zero_adj_len, st));
  return ADS_OK;
}

// ---------------------------------------------------------------------------
// Single-step operators (one_step of src/Core.jl:215-228 and its transpose) in
// the caller's precision: T = double for the f64 entry points, float for f32.
// ---------------------------------------------------------------------------

// Profile rows ax, bx, ay, by (2*NX / 2*NY, row 0 integer grid, row 1 half
// grid) copied into the packed layout the kernels index.
template <typename T>
int el_copy_profiles(T* prof, const T* ax, const T* bx, const T* ay, const T* by, int64_t NX,
                     int64_t NY, cudaStream_t st) {
  ADS_CUDA(cudaMemcpyAsync(prof, ax, sizeof(T) * 2 * NX, cudaMemcpyDeviceToDevice, st));
  ADS_CUDA(cudaMemcpyAsync(prof + 2 * NX, bx, sizeof(T) * 2 * NX, cudaMemcpyDeviceToDevice, st));
  ADS_CUDA(cudaMemcpyAsync(prof + 4 * NX, ay, sizeof(T) * 2 * NY, cudaMemcpyDeviceToDevice, st));
  ADS_CUDA(cudaMemcpyAsync(prof + 4 * NX + 2 * NY, by, sizeof(T) * 2 * NY,
                           cudaMemcpyDeviceToDevice, st));
  return ADS_OK;
}

template <typename T>
int el_step_fwd(const T* state_in, T* state_out, const T* lambda, const T* mu, const T* rho,
                const T* ax, const T* bx, const T* ay, const T* by, double dt, double dx,
                double dy, int64_t NX, int64_t NY, const int64_t* srci, const int64_t* srcj,
                const int64_t* srctype, const T* srcv, int64_t nsrc, ads_stream_t stream) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 4 && NY >= 4 && NX < (1 << 24) && NY < (1 << 24), "NX, NY out of range");
  ADS_REQUIRE(state_in && state_out && lambda && mu && rho && ax && bx && ay && by,
              "null pointer argument");
  ADS_REQUIRE(state_in != state_out, "state_out must not alias state_in");
  ADS_REQUIRE(nsrc >= 0 && (nsrc == 0 || (srci && srcj && srctype && srcv)),
              "invalid source arrays");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t N = (NX + 2) * (NY + 2);
  // profiles, repacked on the device-side scratch
  T* prof = nullptr;
  const size_t prof_n = 4 * NX + 4 * NY;
  ADS_CUDA(cudaMallocAsync((void**)&prof, sizeof(T) * prof_n, st));
  if (int e = el_copy_profiles<T>(prof, ax, bx, ay, by, NX, NY, st)) {
    cudaFreeAsync(prof, st);
    return e;
  }
  ElModel<T> M = make_model<T>((int)NX, (int)NY, NY + 2, 0, dt, dx, dy, lambda, mu, rho, prof);
  ElShot<T> one{};
  for (int f = 0; f < NF; f++) {
    one.fin[f] = state_in + f * N;
    one.f[f] = state_out + f * N;
  }
  one.fs = N;
  dim3 grd((unsigned)div_up(NY + 2, BX), (unsigned)div_up(NX + 2, BY), 1);
  k_el_stress<T, false><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  k_el_velocity<T, false><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  if (nsrc > 0) {
    Fields5<T> f5{{state_out, state_out + N, state_out + 2 * N, state_out + 3 * N,
                   state_out + 4 * N}};
    k_el_step_src<T><<<1, 32, 0, st>>>(f5, srci, srcj, srctype, srcv, nsrc, (int)NX, (int)NY);
    ADS_LAUNCHED(1);
  }
  ADS_CUDA(cudaFreeAsync(prof, st));
  return ADS_OK;
}

// out[e] += (G) acc[e]: the f32 transpose accumulates its parameter gradients in
// FP64 scratch (as the kernels do) and adds them to the caller's FP32 arrays.
template <typename G>
__global__ void k_el_add_grad(G* __restrict__ out, const double* __restrict__ acc, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    out[e] += (G)acc[e];
}

template <typename T, typename G>
int el_step_bwd(const T* state_in, const T* grad_out, T* grad_in, G* grad_lambda, G* grad_mu,
                G* grad_rho, const T* lambda, const T* mu, const T* rho, const T* ax,
                const T* bx, const T* ay, const T* by, double dt, double dx, double dy,
                int64_t NX, int64_t NY, ads_stream_t stream) {
  constexpr bool kDirect = std::is_same<G, double>::value;  // accumulate into the caller's
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 4 && NY >= 4 && NX < (1 << 24) && NY < (1 << 24), "NX, NY out of range");
  ADS_REQUIRE(state_in && grad_out && grad_in && grad_lambda && grad_mu && grad_rho &&
                  lambda && mu && rho && ax && bx && ay && by,
              "null pointer argument");
  ADS_REQUIRE(grad_in != grad_out, "grad_in must not alias grad_out");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t N = (NX + 2) * (NY + 2);
  const size_t prof_n = 4 * NX + 4 * NY;
  // scratch: profiles, forward output state, per-step store, adjoint temps
  // (and, for FP32 outputs, three FP64 accumulators)
  const size_t n_scr = prof_n + (size_t)(NF + NSTORE + NTMP) * N;
  const size_t n_acc = kDirect ? 0 : (size_t)3 * N;
  char* scratch = nullptr;
  const size_t b_scr = sizeof(T) * ((n_scr + 1) & ~size_t(1));
  ADS_CUDA(cudaMallocAsync((void**)&scratch, b_scr + sizeof(double) * n_acc, st));
  ADS_CUDA(cudaMemsetAsync(scratch, 0, b_scr + sizeof(double) * n_acc, st));
  T* prof = (T*)scratch;
  if (int e = el_copy_profiles<T>(prof, ax, bx, ay, by, NX, NY, st)) {
    cudaFreeAsync(scratch, st);
    return e;
  }
  T* fout = prof + prof_n;
  T* store = fout + NF * N;
  T* tmp = store + NSTORE * N;
  double* acc = (double*)(scratch + b_scr);
  ElModel<T> M = make_model<T>((int)NX, (int)NY, NY + 2, 0, dt, dx, dy, lambda, mu, rho, prof);
  ElShot<T> one{};
  for (int f = 0; f < NF; f++) {
    one.fin[f] = state_in + f * N;
    one.f[f] = fout + f * N;
    one.g[f] = grad_in + f * N;
  }
  for (int k = 0; k < NTMP; k++) one.tmp[k] = tmp + k * N;
  one.store = store;
  one.fs = N;
  if constexpr (kDirect) {
    one.glam = grad_lambda;
    one.gmu = grad_mu;
    one.grho = grad_rho;
  } else {
    one.glam = acc;
    one.gmu = acc + N;
    one.grho = acc + 2 * N;
  }
  dim3 grd((unsigned)div_up(NY + 2, BX), (unsigned)div_up(NX + 2, BY), 1);
  k_el_stress<T, true><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  k_el_velocity<T, true><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  ADS_CUDA(cudaMemcpyAsync(grad_in, grad_out, sizeof(T) * NF * N, cudaMemcpyDeviceToDevice, st));
  k_el_adj1<T><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  k_el_adj2<T><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  k_el_adj3<T><<<grd, dim3(BX, BY), 0, st>>>(M, one);
  ADS_LAUNCHED(1);
  if constexpr (!kDirect) {
    const unsigned nb = (unsigned)std::min<int64_t>(div_up(N, 256), 4096);
    k_el_add_grad<G><<<nb, 256, 0, st>>>(grad_lambda, acc, N);
    k_el_add_grad<G><<<nb, 256, 0, st>>>(grad_mu, acc + N, N);
    k_el_add_grad<G><<<nb, 256, 0, st>>>(grad_rho, acc + 2 * N, N);
    ADS_LAUNCHED(3);
  }
  ADS_CUDA(cudaFreeAsync(scratch, st));
  return ADS_OK;
}

}  // namespace
}  // namespace ads

struct ads_elastic_plan {
  std::unique_ptr<ads::ElPlanBase> impl;
};

using namespace ads;

extern "C" {

int ads_elastic_step_fwd_f64(const double* state_in, double* state_out, const double* lambda,
                             const double* mu, const double* rho, const double* ax,
                             const double* bx, const double* kx, const double* ay,
                             const double* by, const double* ky, double dt, double dx,
                             double dy, int64_t NX, int64_t NY, const int64_t* srci,
                             const int64_t* srcj, const int64_t* srctype, const double* srcv,
                             int64_t nsrc, ads_stream_t stream) {
  (void)kx;
  (void)ky;
  return el_step_fwd<double>(state_in, state_out, lambda, mu, rho, ax, bx, ay, by, dt, dx, dy,
                             NX, NY, srci, srcj, srctype, srcv, nsrc, stream);
}

int ads_elastic_step_fwd_f32(const float* state_in, float* state_out, const float* lambda,
                             const float* mu, const float* rho, const float* ax,
                             const float* bx, const float* kx, const float* ay,
                             const float* by, const float* ky, double dt, double dx,
                             double dy, int64_t NX, int64_t NY, const int64_t* srci,
                             const int64_t* srcj, const int64_t* srctype, const float* srcv,
                             int64_t nsrc, ads_stream_t stream) {
  (void)kx;
  (void)ky;
  return el_step_fwd<float>(state_in, state_out, lambda, mu, rho, ax, bx, ay, by, dt, dx, dy,
                            NX, NY, srci, srcj, srctype, srcv, nsrc, stream);
}

int ads_elastic_step_bwd_f64(const double* state_in, const double* grad_out, double* grad_in,
                             double* grad_lambda, double* grad_mu, double* grad_rho,
                             const double* lambda, const double* mu, const double* rho,
                             const double* ax, const double* bx, const double* ay,
                             const double* by, double dt, double dx, double dy, int64_t NX,
                             int64_t NY, ads_stream_t stream) {
  return el_step_bwd<double, double>(state_in, grad_out, grad_in, grad_lambda, grad_mu,
                                     grad_rho, lambda, mu, rho, ax, bx, ay, by, dt, dx, dy, NX,
                                     NY, stream);
}

int ads_elastic_step_bwd_f32(const float* state_in, const float* grad_out, float* grad_in,
                             float* grad_lambda, float* grad_mu, float* grad_rho,
                             const float* lambda, const float* mu, const float* rho,
                             const float* ax, const float* bx, const float* ay,
                             const float* by, double dt, double dx, double dy, int64_t NX,
                             int64_t NY, ads_stream_t stream) {
  return el_step_bwd<float, float>(state_in, grad_out, grad_in, grad_lambda, grad_mu, grad_rho,
                                   lambda, mu, rho, ax, bx, ay, by, dt, dx, dy, NX, NY,
                                   stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free variant of the elastic step transpose.
//
// Some callers cannot allocate device memory at the time they run this step:
// an operator called from another framework's custom-call or kernel hook,
// where that framework owns all device memory and an extension that calls
// cudaMalloc bypasses its memory accounting (and can fail once the framework
// has reserved the device), and time-critical loops that must never enter the
// CUDA allocator, whose calls can synchronise the device and take unbounded
// time.  For them the scratch this step needs (forward output state, per-step
// strains, adjoint temporaries and the packed CPML rows) lives in one fixed
// array in device global memory, compiled into the library.  Every GPU that
// loads the library holds the array (34 x 65536 doubles, about 17.8 MB) until
// the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t kNoAllocMaxCells = 65536;  // (NX+2)*(NY+2) limit
constexpr size_t kNoAllocDoubles = (size_t)(NF + NSTORE + NTMP + 4) * kNoAllocMaxCells;
static __device__ __align__(256) double g_el_bwd_scratch[kNoAllocDoubles];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[128] = {};  // device address of g_el_bwd_scratch, per device

// Device address of the scratch array for the current device, looked up once
// per device (the host-side symbol is only a stand-in, never a device address).
// The cached address belongs to the device's primary context: it assumes that
// context lives for the whole process, so a caller that resets the device
// (cudaDeviceReset) must not call the allocation-free entry point afterwards.
int noalloc_scratch(double** out) {
  int dev = 0;
  ADS_CUDA(cudaGetDevice(&dev));
  ADS_REQUIRE(dev >= 0 && dev < 128, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_el_bwd_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return fail(ADS_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed on device %d: %s", dev,
                  cudaGetErrorString(e));
    }
    g_noalloc_ptr[dev] = (double*)p;
  }
  *out = g_noalloc_ptr[dev];
  return ADS_OK;
}

}  // namespace

extern "C" {

int ads_elastic_step_bwd_f64_noalloc(const double* state_in, const double* grad_out,
                                     double* grad_in, double* grad_lambda, double* grad_mu,
                                     double* grad_rho, const double* lambda, const double* mu,
                                     const double* rho, const double* ax, const double* bx,
                                     const double* ay, const double* by, double dt, double dx,
                                     double dy, int64_t NX, int64_t NY, ads_stream_t stream) {
  if (int e = require_device()) return e;
  ADS_REQUIRE(NX >= 4 && NY >= 4 && NX < (1 << 24) && NY < (1 << 24), "NX, NY out of range");
  const int64_t N = (NX + 2) * (NY + 2);
  ADS_REQUIRE(N <= kNoAllocMaxCells,
              "grid (NX+2)*(NY+2) = %lld exceeds the %lld cells the allocation-free "
              "scratch holds; use ads_elastic_step_bwd_f64",
              (long long)N, (long long)kNoAllocMaxCells);
  ADS_REQUIRE(state_in && grad_out && grad_in && grad_lambda && grad_mu && grad_rho &&
                  lambda && mu && rho && ax && bx && ay && by,
              "null pointer argument");
  ADS_REQUIRE(grad_in != grad_out, "grad_in must not alias grad_out");
  double* scratch = nullptr;
  if (int e = noalloc_scratch(&scratch)) return e;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t prof_n = 4 * NX + 4 * NY;
  const size_t n_scr = prof_n + (size_t)(NF + NSTORE + NTMP) * N;
  // the array keeps the previous call's contents: clear the part used here
  ADS_CUDA(cudaMemsetAsync(scratch, 0, sizeof(double) * n_scr, st));
  double* prof = scratch;
  ADS_CUDA(cudaMemcpyAsync(prof, ax, sizeof(double) * 2 * NX, cudaMemcpyDeviceToDevice, st));
  ADS_CUDA(cudaMemcpyAsync(prof + 2 * NX, bx, sizeof(double) * 2 * NX, cudaMemcpyDeviceToDevice,
                           st));
  ADS_CUDA(cudaMemcpyAsync(prof + 4 * NX, ay, sizeof(double) * 2 * NY, cudaMemcpyDeviceToDevice,
                           st));
  ADS_CUDA(cudaMemcpyAsync(prof + 4 * NX + 2 * NY, by, sizeof(double) * 2 * NY,
                           cudaMemcpyDeviceToDevice, st));
  double* fout = scratch + prof_n;
  double* store = fout + NF * N;
  double* tmp = store + NSTORE * N;
  ElModel<double> M =
      make_model<double>((int)NX, (int)NY, NY + 2, 0, dt, dx, dy, lambda, mu, rho, prof);
  ElShot<double> one{};
  for (int f = 0; f < NF; f++) {
    one.fin[f] = state_in + f * N;
    one.f[f] = fout + f * N;
    one.g[f] = grad_in + f * N;
  }
  for (int k = 0; k < NTMP; k++) one.tmp[k] = tmp + k * N;
  one.store = store;
  one.fs = N;
  one.glam = grad_lambda;
  one.gmu = grad_mu;
  one.grho = grad_rho;
  dim3 grd((unsigned)div_up(NY + 2, BX), (unsigned)div_up(NX + 2, BY), 1);
  k_el_stress<double, true><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  k_el_velocity<double, true><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  ADS_CUDA(cudaMemcpyAsync(grad_in, grad_out, sizeof(double) * NF * N,
                           cudaMemcpyDeviceToDevice, st));
  k_el_adj1<double><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  k_el_adj2<double><<<grd, dim3(BX, BY), 0, st>>>(M, one, 0);
  ADS_LAUNCHED(1);
  k_el_adj3<double><<<grd, dim3(BX, BY), 0, st>>>(M, one);
  ADS_LAUNCHED(1);
  return ADS_OK;
}

int ads_elastic_plan_create(ads_elastic_plan** plan, const ads_elastic_config* cfg,
                            const ads_elastic_shot* shots, int64_t nshots,
                            ads_stream_t stream) {
  ADS_REQUIRE(plan && cfg && shots, "null argument");
  *plan = nullptr;
  if (int e = require_device()) return e;
  ADS_REQUIRE(cfg->precision == ADS_F64 || cfg->precision == ADS_F32,
              "precision must be ADS_F64 or ADS_F32");
  std::unique_ptr<ads_elastic_plan> p(new ads_elastic_plan);
  int rc;
  if (cfg->precision == ADS_F64) {
    auto* q = new ElPlan<double>();
    p->impl.reset(q);
    rc = q->create(*cfg, shots, nshots, (cudaStream_t)stream);
  } else {
    auto* q = new ElPlan<float>();
    p->impl.reset(q);
    rc = q->create(*cfg, shots, nshots, (cudaStream_t)stream);
  }
  if (rc != ADS_OK) return rc;
  *plan = p.release();
  return ADS_OK;
}

int ads_elastic_plan_destroy(ads_elastic_plan* plan) {
  if (!plan) return ADS_OK;
  cudaDeviceSynchronize();
  delete plan;
  return ADS_OK;
}

int64_t ads_elastic_plan_trace_offset(const ads_elastic_plan* plan, int64_t shot) {
  if (!plan || shot < 0 || shot >= (int64_t)plan->impl->trace_off.size()) return -1;
  return plan->impl->trace_off[shot];
}

int64_t ads_elastic_plan_trace_count(const ads_elastic_plan* plan) {
  return plan ? plan->impl->trace_total : -1;
}

int64_t ads_elastic_plan_device_bytes(const ads_elastic_plan* plan) {
  return plan ? plan->impl->bytes : -1;
}

int64_t ads_elastic_plan_resident_segments(const ads_elastic_plan* plan) {
  return plan ? plan->impl->resident : -1;
}

int64_t ads_elastic_plan_rows(const ads_elastic_plan* plan, int which) {
  if (!plan || which < 0 || which > 5) return -1;
  return which < 2 ? plan->impl->tiling[which] : plan->impl->adj_items[which - 2];
}

int64_t ads_elastic_plan_launches(const ads_elastic_plan* plan, int gradient) {
  if (!plan) return -1;
  return gradient ? plan->impl->launches_grad : plan->impl->launches_fwd;
}

int ads_elastic_plan_forward(ads_elastic_plan* plan, const double* lambda, const double* mu,
                             const double* rho, void* traces, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->forward(lambda, mu, rho, traces, (cudaStream_t)stream);
}

int ads_elastic_plan_gradient(ads_elastic_plan* plan, const double* lambda, const double* mu,
                              const double* rho, const void* observed, double* loss,
                              double* grad_lambda, double* grad_mu, double* grad_rho,
                              void* traces_out, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->gradient(lambda, mu, rho, observed, loss, grad_lambda, grad_mu, grad_rho,
                              traces_out, (cudaStream_t)stream, nullptr);
}

int ads_elastic_plan_gradient_ex(ads_elastic_plan* plan, const double* lambda,
                                 const double* mu, const double* rho, const void* observed,
                                 double* loss, double* grad_lambda, double* grad_mu,
                                 double* grad_rho, double* grad_srcv, void* traces_out,
                                 ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->gradient(lambda, mu, rho, observed, loss, grad_lambda, grad_mu, grad_rho,
                              traces_out, (cudaStream_t)stream, grad_srcv);
}

int ads_elastic_plan_set_source_values(ads_elastic_plan* plan, int64_t shot,
                                       const double* srcv, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->set_source_values(shot, srcv, (cudaStream_t)stream);
}

int64_t ads_elastic_plan_source_offset(const ads_elastic_plan* plan, int64_t shot) {
  if (!plan || shot < 0 || shot >= (int64_t)plan->impl->src_off.size()) return -1;
  return plan->impl->src_off[shot];
}

int ads_elastic_plan_profile(ads_elastic_plan* plan, const double* lambda, const double* mu,
                             const double* rho, double* out, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->profile(lambda, mu, rho, out, (cudaStream_t)stream);
}

int ads_elastic_forward(const ads_elastic_config* cfg, const ads_elastic_shot* shot,
                        const double* lambda, const double* mu, const double* rho,
                        void* traces, ads_stream_t stream) {
  ADS_REQUIRE(cfg && shot, "null argument");
  ads_elastic_plan* p = nullptr;
  ads_elastic_config c = *cfg;
  c.use_graph = 0;
  if (int e = ads_elastic_plan_create(&p, &c, shot, 1, stream)) return e;
  int rc = ads_elastic_plan_forward(p, lambda, mu, rho, traces, stream);
  if (rc == ADS_OK && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
    rc = fail(ADS_ERR_CUDA, "stream synchronisation failed");
  ads_elastic_plan_destroy(p);
  return rc;
}

int ads_elastic_gradient(const ads_elastic_config* cfg, const ads_elastic_shot* shot,
                         const double* lambda, const double* mu, const double* rho,
                         const void* observed, double* loss, double* grad_lambda,
                         double* grad_mu, double* grad_rho, ads_stream_t stream) {
  ADS_REQUIRE(cfg && shot, "null argument");
  ads_elastic_plan* p = nullptr;
  ads_elastic_config c = *cfg;
  c.use_graph = 0;
  if (int e = ads_elastic_plan_create(&p, &c, shot, 1, stream)) return e;
  int rc = ads_elastic_plan_gradient(p, lambda, mu, rho, observed, loss, grad_lambda, grad_mu,
                                     grad_rho, nullptr, stream);
  if (rc == ADS_OK && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
    rc = fail(ADS_ERR_CUDA, "stream synchronisation failed");
  ads_elastic_plan_destroy(p);
  return rc;
}

}  // extern "C"
