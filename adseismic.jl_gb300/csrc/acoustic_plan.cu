// acoustic_plan.cu -- whole-path acoustic FWI on one GPU: forward traces,
// L2 misfit, checkpointed discrete adjoint and the velocity gradient for one or
// many shots with uneven windows and record lengths.
//
// Reference semantics (src/Core.jl:562-620, 726-730; src/Utils.jl:300-332):
//   slot 0, 1 = 0;  slot t = step(slot t-1, slot t-2) for t = 2..NSTEP, then
//   u_t[src] += srcv[t-1] * dt^2;  traces[t, r] = u_t[rcv r];
//   loss = sum (traces - observed)^2;  grad_vp = (grad_c * 2) * vp.
//
// Design (one GPU, HBM-resident, no host round trips inside a call):
//  * Every shot keeps its wavefield in a pitched layout (ads_internal.h) so
//    warp rows are 128/256-byte aligned.  A CTA owns a tile of
//    rows_per_thread x 128 cells of one shot; each thread slides down i keeping
//    the i-neighbours in registers and gets j-neighbours by warp shuffles.
//  * One launch advances every active shot by one step; the launch's grid is
//    the prefix of the tile list whose shots are still active (shots are sorted
//    by record length), so uneven NSTEP costs no idle CTAs.
//  * Forward checkpoints (u_t, u_{t-1}, phi_t, psi_t) are written by the step
//    kernel itself every k steps; the reverse sweep restores a checkpoint,
//    recomputes its segment into a (k+1)-slot store and runs the adjoint steps
//    backwards, accumulating grad_c in FP64.
//  * The forward and the reverse time loops are captured once as CUDA graphs
//    and replayed each call.
#include <cuda.h>  // CUtensorMap (the encoder comes through the runtime's driver entry point)

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <vector>

#include "ads_internal.h"

namespace ads {
namespace {

constexpr unsigned FULL = 0xffffffffu;

#ifndef ADS_PF32
#define ADS_PF32 1
#endif
#ifndef ADS_MINB_F32
#define ADS_MINB_F32 8    // 64 registers
#endif
#ifndef ADS_MINB_A32
#define ADS_MINB_A32 5    // 102 -> 96 registers
#endif
#ifndef ADS_MINB_FI32
#define ADS_MINB_FI32 16  // 32 registers: every warp slot of the SM
#endif
#ifndef ADS_MINB_AI32
#define ADS_MINB_AI32 9   // 56 registers
#endif


// Tiles: a warp owns a strip of 32 x CF (forward) or 32 x CA (adjoint)
// columns and rows_per_thread rows of one shot; each thread owns CF / CA
// adjacent columns, loaded as one 8/16-byte vector per row.  J is the column
// width of the per-segment helpers' tiles.
template <typename T>
struct Tile {
  static constexpr int J = sizeof(T) == 4 ? 512 : 256;
  static constexpr int CF = sizeof(T) == 4 ? 2 : 1;
  static constexpr int CA = sizeof(T) == 4 ? 2 : 1;
  // rows of register prefetch in the interior loops (bytes in flight per warp)
  static constexpr int PF = sizeof(T) == 4 ? ADS_PF32 : 1;
  // Step kernels: a CTA of G warps takes one item (a column strip of one
  // shot); its warps take consecutive tiles of rows.  The item is uniform over
  // the CTA, so its fields and everything derived from them stay in uniform
  // registers.
  static constexpr int G = 4;
  static constexpr int TPB = 32 * G;
  static constexpr int WF = 32 * CF;  // columns of a forward strip
  static constexpr int WA = 32 * CA;  // columns of an adjoint strip
  // resident CTAs of TPB threads per SM the register allocation must allow
  // (general / interior-only kernels; 65536 / (TPB x MINB) registers a thread)
  static constexpr int MINB_F = sizeof(T) == 4 ? ADS_MINB_F32 : 3;
  static constexpr int MINB_A = sizeof(T) == 4 ? ADS_MINB_A32 : 3;
  static constexpr int MINB_FI = sizeof(T) == 4 ? ADS_MINB_FI32 : 6;
  static constexpr int MINB_AI = sizeof(T) == 4 ? ADS_MINB_AI32 : 5;
};

template <typename T, int C>
struct alignas(sizeof(T) * C) Vec {
  T v[C];
};

struct CellRef {
  int64_t cell;  // element offset inside the shot's pitched field
  int idx;       // source / receiver index within the shot
  int row;       // its row (1-based padded grid)
};

struct AcItem {
  int shot, i0, j0, pad;
  int src_b, src_e, rcv_b, rcv_e;
};

template <typename T>
struct AcShot {
  int nx, ny, nstep, x0;
  int64_t pitch, fs;  // row pitch and elements per field
  int nsrc, nrcv, nseg, pad_;
  T *u, *p, *q;       // forward rings (2 fields each)
  T* d;               // FP32 increment form: d_t = u_t - u_{t-1}, updated in place
  T* u2;              // time-blocked forward: U_{t-1} of the two state sets
  const int* rcv_next; // next receiver on the same cell, or -1 (time-blocked forward)
  T *seg, *ckpt;      // segment store (k+1 fields), checkpoints (nseg x 4 fields)
  T *lu, *lp, *lq;    // adjoint rings (2 fields each)
  T *c, *sx, *ty;     // c = vp^2 (pitched), PML profiles along i and j
  // damping tables of the PML profiles (KT_N arrays each): along i, nx + 2
  // entries per array, after sx; along j, ny + 2 entries, after ty
  T *sxk, *tyk;
  T* rdt;  // FP64 plans: 1 / (1 + (sigma + tau) dt/2) per cell (pitched), else null
  double* gc;         // FP64 gradient accumulator (pitched)
  float* gc32;        // FP32 per-segment partial of grad_c (FP32 plans)
  const T* srcv;      // (nstep, nsrc), already multiplied by dt^2
  T *traces, *resid;  // (nstep+1, nrcv) packed views
  double* gsrc;       // d loss / d srcv, (nstep, nsrc) FP64
  const CellRef* src_list;  // the shot's sources (pitched cell, index, row)
};

// Damping tables of a PML profile s (sigma along i, tau along j), one array
// each, computed in FP64 on the host and rounded once:
//   r = 1 / (1 + s dt/2), ar = (1 - s dt/2) r, e = 1 - s dt,
//   ex = s dt / (2 hx), ey = s dt / (2 hy).
enum { KT_R, KT_AR, KT_E, KT_EX, KT_EY, KT_N };

// The profile s followed by its KT_N tables.
template <typename T>
std::vector<T> with_tables(const std::vector<double>& s, double dt, double hx, double hy) {
  const size_t n = s.size();
  std::vector<T> o((1 + KT_N) * n);
  for (size_t k = 0; k < n; k++) {
    const double r = 1.0 / std::fma(s[k], 0.5 * dt, 1.0);
    o[k] = (T)s[k];
    o[(1 + KT_R) * n + k] = (T)r;
    o[(1 + KT_AR) * n + k] = (T)(std::fma(-s[k], 0.5 * dt, 1.0) * r);
    o[(1 + KT_E) * n + k] = (T)std::fma(-s[k], dt, 1.0);
    o[(1 + KT_EX) * n + k] = (T)(s[k] * (dt / 2.0 / hx));
    o[(1 + KT_EY) * n + k] = (T)(s[k] * (dt / 2.0 / hy));
  }
  return o;
}

template <typename T>
struct AcConst {
  T dt, hdt, dt2, cx, cy, kxy, fx, fy, ex, ey;
};

// ---------------------------------------------------------------- kernels

// Columns of a warp whose tau profile is zero at j-1..j+1 (for every lane):
// there phi and psi can only be non-zero in rows whose sigma is non-zero.
// In cells with sigma = tau = 0 the forward phi/psi are identically zero
// (phi' = (1 - 0) phi + 0) and their adjoints never reach lambdaU or grad_c
// (they are multiplied by tau - sigma = 0), so those loads and stores are
// skipped; the arithmetic is unchanged (the skipped values enter as exact 0).
template <typename T>
__device__ __forceinline__ bool warp_tau_free(const T* __restrict__ ty, int j, int ny) {
  const bool z = j > ny + 1 ||
                 (ty[j - 1] == T(0) && ty[j] == T(0) && (j + 1 > ny + 1 || ty[j + 1] == T(0)));
  return __all_sync(FULL, z);
}

// Loads of a thread's cells as predicated PTX loads: zeros where `on` is
// false, and no branch, so masks that differ between the lanes of a warp (the
// last columns of a shot, the halo lanes) cost no divergence.  The asm has no
// memory clobber: the step kernels load each cell at most once per launch,
// and a cell they also write is written later, from values computed from the
// load.
__device__ __forceinline__ float ld1p(const float* p, bool on) {
  float a = 0.f;
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q ld.global.f32 %0, [%1];\n\t}"
      : "+f"(a)
      : "l"(p), "r"((unsigned)on));
  return a;
}
__device__ __forceinline__ double ld1p(const double* p, bool on) {
  double a = 0.0;
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q ld.global.f64 %0, [%1];\n\t}"
      : "+d"(a)
      : "l"(p), "r"((unsigned)on));
  return a;
}

// C-wide loads and stores of a thread's columns.  Full-width stores only when
// all C cells are interior; otherwise per cell (the frame must stay zero).
// ldv is a guarded load (the interior loops, whose masks agree across a
// warp); ldvp the predicated form for the PML loops.
template <typename T, int C, typename I = int64_t>
__device__ __forceinline__ Vec<T, C> ldv(const T* base, I off, bool on) {
  Vec<T, C> x;
  if (on) {
    x = *reinterpret_cast<const Vec<T, C>*>(base + off);
  } else {
#pragma unroll
    for (int c = 0; c < C; c++) x.v[c] = T(0);
  }
  return x;
}

template <typename T, int C, typename I = int64_t>
__device__ __forceinline__ Vec<T, C> ldvp(const T* base, I off, bool on) {
  Vec<T, C> x;
  const T* p = base + off;
  if constexpr (C == 2 && sizeof(T) == 4) {
    float a = 0.f, b = 0.f;
    asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %3, 0;\n\t@q ld.global.v2.f32 {%0, %1}, [%2];\n\t}"
        : "+f"(a), "+f"(b)
        : "l"(p), "r"((unsigned)on));
    x.v[0] = a;
    x.v[1] = b;
  } else if constexpr (C == 2) {
    double a = 0.0, b = 0.0;
    asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %3, 0;\n\t@q ld.global.v2.f64 {%0, %1}, [%2];\n\t}"
        : "+d"(a), "+d"(b)
        : "l"(p), "r"((unsigned)on));
    x.v[0] = a;
    x.v[1] = b;
  } else {
#pragma unroll
    for (int c = 0; c < C; c++) x.v[c] = ld1p(p + c, on);
  }
  return x;
}

template <typename T, int C, typename I = int64_t>
__device__ __forceinline__ void stv(T* base, I off, const Vec<T, C>& x, int j, int ny) {
  if constexpr (C == 2) {
    // two guarded stores, predicated rather than branched
    if (j + 1 <= ny) *reinterpret_cast<Vec<T, C>*>(base + off) = x;
    if (j == ny) base[off] = x.v[0];
  } else if (j + C - 1 <= ny) {
    *reinterpret_cast<Vec<T, C>*>(base + off) = x;
  } else {
#pragma unroll
    for (int c = 0; c < C; c++)
      if (j + c <= ny) base[off + c] = x.v[c];
  }
}

// True when tau is zero at every column the warp reads (j-1 .. j+C): there
// phi and psi can only be non-zero in rows whose sigma is non-zero.  In cells
// with sigma = tau = 0 the forward phi/psi are identically zero
// (phi' = (1 - 0) phi + 0) and their adjoints never reach lambdaU or grad_c
// (they are multiplied by tau - sigma = 0), so those loads and stores are
// skipped; the arithmetic is unchanged (the skipped values enter as exact 0).
template <typename T, int C>
__device__ __forceinline__ bool warp_tau_free(const T* __restrict__ ty, int j, int ny) {
  bool z = true;
  if (j <= ny + 1) {
    z = ty[j - 1] == T(0);
#pragma unroll
    for (int c = 0; c <= C; c++)
      if (j + c <= ny + 1) z = z && ty[j + c] == T(0);
  }
  return __all_sync(FULL, z);
}

// The PML damping v / (1 + s dt/2): FP32 plans use the hardware divide
// (within 2 ulp; their error budget against the FP64 oracle is 1e-4) on every
// cell, s = 0 dividing by exactly 1, so lanes with and without damping take
// one path; FP64 plans divide exactly, only where s != 0 (1e-12 parity).
template <typename T, typename K>
__device__ __forceinline__ T pml_damp(T v, T s, const K& k) {
  if constexpr (sizeof(T) == 4) {
    return __fdividef(v, T(1) + s * k.hdt);
  } else {
    return s != T(0) ? v / (T(1) + s * k.hdt) : v;
  }
}

// True when the warp's columns are tau-free and sigma is zero on rows
// i0-1 .. i_end (every row a tile of rows [i0, i_end) reads): phi, psi and
// their adjoints are then zero throughout and the interior update applies.
template <typename T>
__device__ __forceinline__ bool interior_rows(bool tfree, const T* __restrict__ sx, int i0,
                                              int i_end, int lane) {
  bool z = true;
  for (int r = i0 - 1 + lane; r <= i_end; r += 32) z = z && sx[r] == T(0);
  return tfree && __all_sync(FULL, z);
}

// Each warp records the receivers in its own cells (its strip's columns, its
// rows) after a forward step: its lanes wrote them, so a warp barrier suffices.
template <typename T, int C, bool NOREC>
__device__ __forceinline__ void record_traces(const AcItem& it, const AcShot<T>& sh,
                                              const CellRef* __restrict__ rcvs, const T* out,
                                              int t, int lane, int i0, int i_end) {
  if (NOREC || it.rcv_e <= it.rcv_b) return;
  __syncwarp();
  for (int e = it.rcv_b + lane; e < it.rcv_e; e += 32) {
    const CellRef r = rcvs[e];  // r.row: the receiver's row
    if (r.row >= i0 && r.row < i_end) sh.traces[(int64_t)t * sh.nrcv + r.idx] = out[r.cell];
  }
}

// One forward step (variant W: phi/psi from the old field).  MODE 0 (the
// forward loop): rings of two (u_t written over u_{t-2}), receiver traces,
// optional checkpoint write.  MODE 1 (a segment's recompute in the reverse
// sweep): the shot's store addressed by slot t - base, no traces.  MODE 2
// (the forward loop over the resident segments): the store as in MODE 1,
// with traces; those wavefields stay for the reverse sweep, which then needs
// no recompute of those segments.  Every warp takes one item (a
// 32*CF-column strip of rows of one shot); each thread owns CF adjacent
// columns, walks down the rows with the next row's loads issued one iteration
// ahead, and takes the j-neighbours of its edge cells from the neighbouring
// lanes (warp-edge lanes load them).  INT = true: the item is interior
// (sigma = tau = 0 on every row and column it reads, classified on the host)
// and only the plain wave update is compiled, so the kernel needs few
// registers and keeps many warps resident; INT = false: the general PML form.
//
// VU = true (variant U, PML items only): phi_{t-1} and psi_{t-1} were formed
// from u_{t-1} by k_ac_phi_u at the start of this step, so this kernel only
// reads them (as the custom-operator form reads its phi_{t-1}, psi_{t-1}) and
// writes neither; its checkpoints store the phi / psi it read.
//
// CK = true: the kernel may write checkpoint ckpt_slot (MODE 0).  The PML
// kernel takes that code only at checkpoint times, which keeps its other
// steps free of spills; the interior kernel keeps it in every MODE 0 step
// (measured: the form without it spills more at its 32 registers).
//
// INC = true (FP32 plans): the increment form.  The state is u_t and
// d_t = u_t - u_{t-1} (one field, updated in place) instead of u_t and
// u_{t-1}; the step forms d_{t+1} from d_t and the Laplacian written as
// differences of u, then u_{t+1} = u_t + d_{t+1}.  In exact arithmetic this is
// the same update; in FP32 the three-level form's rounding of u_{t+1} (about
// eps |u|) perturbs the difference u_{t+1} - u_t, which the oscillation
// amplifies by 1 / (w dt), while here the rounding of d is relative to |d|.
// Traces and gradients then stay near 1e-6 of the FP64 ones over thousands of
// steps instead of drifting to 1e-4.  The checkpoints hold (u_t, d_t, phi, psi).
template <typename T, int MODE, bool INT, bool VU = false, bool CK = false, bool INC = false>
__global__ void __launch_bounds__(Tile<T>::TPB, INT ? Tile<T>::MINB_FI : Tile<T>::MINB_F)
k_ac_fwd(const AcItem* __restrict__ items, const AcShot<T>* __restrict__ shots,
         const CellRef* __restrict__ srcs, const CellRef* __restrict__ rcvs, AcConst<T> K,
         int t, int base, int ckpt_slot, int ri) {
  constexpr bool SEG = MODE != 0;  // u from the shot's store, not the rings
  constexpr bool NOREC = MODE == 1;  // no receiver traces
  constexpr int C = Tile<T>::CF;
  using V = Vec<T, C>;
  const AcItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int lane = threadIdx.x & 31;
  const int j = it.j0 + lane * C;
  const int nx = sh.nx, ny = sh.ny;
  const int64_t P = sh.pitch, fs = sh.fs;
  const T *w, *wo;
  T* out;
  if (SEG) {
    w = sh.seg + (int64_t)(t - 1 - base) * fs;
    wo = sh.seg + (int64_t)(t - 2 - base) * fs;
    out = sh.seg + (int64_t)(t - base) * fs;
  } else {
    w = sh.u + (int64_t)((t - 1) & 1) * fs;
    out = sh.u + (int64_t)(t & 1) * fs;
    wo = out;  // u_t overwrites u_{t-2}: row r is read one iteration before it is written
  }
  T* dd = sh.d;  // increment form: d_{t-1} in, d_t out (row r read before it is written)
  if (INC) wo = dd;
  const T* pin = sh.p + (int64_t)((t - 1) & 1) * fs;
  T* pout = sh.p + (int64_t)(t & 1) * fs;
  const T* qin = sh.q + (int64_t)((t - 1) & 1) * fs;
  T* qout = sh.q + (int64_t)(t & 1) * fs;
  const T* __restrict__ cc = sh.c;
  const T* __restrict__ sx = sh.sx;
  const T* __restrict__ ty = sh.ty;
  const T* __restrict__ sxk = sh.sxk;
  const T* __restrict__ tyk = sh.tyk;
  const T* __restrict__ rdt = sh.rdt;
  const T* __restrict__ srcv = sh.srcv;
  const bool jld = j <= ny + 1;
  const bool hr = j + C <= ny + 1;  // right halo column exists (last lane of a warp)
  const int64_t col = j + JOFF;
  T tj[C];
#pragma unroll
  for (int c = 0; c < C; c++) tj[c] = (j + c <= ny + 1) ? ty[j + c] : T(0);
  const bool tfree = warp_tau_free<T, C>(ty, j, ny);
  auto nz = [&](int r) { return !(tfree && sx[r] == T(0)); };  // phi/psi may be non-zero
  const int i0 = it.i0 + (threadIdx.x >> 5) * ri, i_end = min(i0 + ri, nx + 1);
  if (i0 > nx) return;  // whole warps only: every later barrier is warp-level
  auto off = [&](int r) { return (int64_t)r * P + col; };
  const bool ck_on = CK && !SEG && ckpt_slot > 0 && ckpt_slot < sh.nseg;
  if (INT || interior_rows<T>(tfree, sx, i0, i_end, lane)) {
    // Interior item: sigma = tau = 0 on every row and column the warp reads,
    // so phi = psi = 0 there and the step reduces to the plain wave update
    // (the dropped terms are exact zeros); it holds no source or receiver.
    // Register queues PF rows deep: w rows i-1 .. i+PF, wo / c / halo rows
    // i .. i+PF-1; each iteration issues the loads of the farthest rows.
    constexpr int PF = Tile<T>::PF;
    // offsets within a field fit 32 bits (the plan checks fs < 2^31), which
    // frees the registers of 64-bit row offsets in the increment form (the
    // three-level form keeps 64-bit offsets: measured fewer spills that way)
    using OffT = std::conditional_t<INC, int, int64_t>;
    const OffT P32 = (OffT)P, col32 = j + JOFF;
    auto off = [&](int r) { return (OffT)r * P32 + col32; };
    V wq[PF + 2], oq[PF], cq[PF];
    T hq[PF];
    auto halo = [&](int r) -> T {
      if (r >= i_end) return T(0);
      if (lane == 0 && jld) return w[off(r) - 1];
      if (lane == 31 && hr) return w[off(r) + C];
      return T(0);
    };
#pragma unroll
    for (int q = 0; q < PF + 2; q++) wq[q] = ldv<T, C>(w, off(i0 - 1 + q), jld && i0 - 1 + q <= i_end);
#pragma unroll
    for (int q = 0; q < PF; q++) {
      const bool on = jld && i0 + q < i_end;
      oq[q] = ldv<T, C>(wo, off(i0 + q), on);
      cq[q] = ldv<T, C>(cc, off(i0 + q), on);
      hq[q] = halo(i0 + q);
    }
    for (int i = i0; i < i_end; i++) {
      const OffT row = off(i);
      const int rn = i + PF;  // farthest row of the wo / c / halo queues
      V wn = ldv<T, C>(w, off(rn + 1), jld && rn + 1 <= i_end);
      V on = ldv<T, C>(wo, off(rn), jld && rn < i_end);
      V cn = ldv<T, C>(cc, off(rn), jld && rn < i_end);
      const T hn = halo(rn);
      const V& wm = wq[0];
      const V& w0 = wq[1];
      const V& wp = wq[2];
      T wL = __shfl_up_sync(FULL, w0.v[C - 1], 1), wR = __shfl_down_sync(FULL, w0.v[0], 1);
      if (lane == 0) wL = hq[0];
      else if (lane == 31) wR = hq[0];
      if (jld) {
        V vo, dv;
#pragma unroll
        for (int c = 0; c < C; c++) {
          const T wS = c == 0 ? wL : w0.v[c - 1];
          const T wN = c == C - 1 ? wR : w0.v[c + 1];
          const T cv = cq[0].v[c];
          T v;
          if constexpr (INC) {
            const T u0 = w0.v[c];
            dv.v[c] = oq[0].v[c] + cv * (K.cx * ((wp.v[c] - u0) + (wm.v[c] - u0)) +
                                         K.cy * ((wN - u0) + (wS - u0)));
            v = u0 + dv.v[c];
          } else if constexpr (sizeof(T) == 8) {
            // FP64 plans (issue-bound): seven operations instead of nine
            v = (T(2) * w0.v[c] - oq[0].v[c]) +
                cv * (K.cx * (wp.v[c] + wm.v[c]) + K.cy * (wN + wS) - K.kxy * w0.v[c]);
          } else {
            v = (T(2) - K.kxy * cv) * w0.v[c] + cv * K.cx * (wp.v[c] + wm.v[c]) +
                cv * K.cy * (wN + wS) - oq[0].v[c];
          }
          if constexpr (!INT) {
            for (int e = it.src_b; e < it.src_e; e++) {
              const CellRef r = srcs[e];
              if (r.cell == row + c) v += srcv[(int64_t)(t - 1) * sh.nsrc + r.idx];
            }
          }
          vo.v[c] = v;
        }
        stv<T, C>(out, row, vo, j, ny);
        if constexpr (INC) stv<T, C>(dd, row, dv, j, ny);
        if (ck_on) {
          T* ck = sh.ckpt + (int64_t)ckpt_slot * 4 * fs;
          stv<T, C>(ck, row, vo, j, ny);
          stv<T, C>(ck + fs, row, INC ? dv : w0, j, ny);
        }
      }
#pragma unroll
      for (int q = 0; q < PF + 1; q++) wq[q] = wq[q + 1];
      wq[PF + 1] = wn;
#pragma unroll
      for (int q = 0; q < PF - 1; q++) {
        oq[q] = oq[q + 1];
        cq[q] = cq[q + 1];
        hq[q] = hq[q + 1];
      }
      oq[PF - 1] = on;
      cq[PF - 1] = cn;
      hq[PF - 1] = hn;
    }
    if constexpr (!INT) record_traces<T, C, NOREC>(it, sh, rcvs, out, t, lane, i0, i_end);
  } else {
  // The general (PML) form.  FP64 plans specialise it by the warp's kind
  // (uniform over the warp): PK = 1 where tau = 0 at every column
  // the warp reads (sigma rows only: the damping factors come per row from the
  // shot's tables), PK = 2 where sigma = 0 on every row it updates (tau columns
  // only: the factors are per-thread constants), PK = 3 elsewhere (the
  // corners: the sigma factors per row, the tau products per cell and
  // 1 / (1 + s dt/2) from the shot's per-cell table).  PK = 0, the general form
  // with its divide, serves FP32 plans.  The specialised forms
  // drop terms that are exact zeros there and multiply by the tabulated
  // reciprocal instead of dividing (within an ulp of the divide; with
  // r = 1 / (1 + s dt/2), (1 - s dt/2) r = 2 r - 1).  FP64 plans are bound by
  // the FP64 issue rate, so the count of FP64 instructions is their cost.
  auto pml_rows = [&](auto kd) {
    constexpr int PK = decltype(kd)::value;
    T rc[C], arc[C], bq[C], ext[C], eyt[C];  // PK 2: per-column constants
#pragma unroll
    for (int c = 0; c < C; c++) {
      rc[c] = arc[c] = bq[c] = T(1);
      ext[c] = eyt[c] = T(0);
      if constexpr (PK == 2) {
        if (j + c <= ny + 1) {
          const int n = ny + 2, q = j + c;
          rc[c] = tyk[KT_R * n + q];
          arc[c] = tyk[KT_AR * n + q];
          bq[c] = tyk[KT_E * n + q];
          ext[c] = tyk[KT_EX * n + q];
          eyt[c] = tyk[KT_EY * n + q];
        }
      }
    }
    bool n0 = nz(i0);
    V wm = ldvp<T, C>(w, off(i0 - 1), jld), w0 = ldvp<T, C>(w, off(i0), jld),
      wp = ldvp<T, C>(w, off(i0 + 1), jld);
    V pm = ldvp<T, C>(pin, off(i0 - 1), jld && nz(i0 - 1)), p0 = ldvp<T, C>(pin, off(i0), jld && n0),
      pp = ldvp<T, C>(pin, off(i0 + 1), jld && nz(i0 + 1));
    V q0 = ldvp<T, C>(qin, off(i0), jld && n0), wo0 = ldvp<T, C>(wo, off(i0), jld),
      c0 = ldvp<T, C>(cc, off(i0), jld);
    // lane 0: column j-1; lane 31: column j+C
    const int64_t hoff = lane == 0 ? -1 : C;
    const bool hon = (lane == 0 && jld) || (lane == 31 && hr);
    T hw = ld1p(w + off(i0) + hoff, hon), hq = ld1p(qin + off(i0) + hoff, hon && n0);
    V rd0{};  // PK 3: 1 / (1 + s dt/2) of the row's cells, one row ahead
    if constexpr (PK == 3) rd0 = ldvp<T, C>(rdt, off(i0), jld);
    for (int i = i0; i < i_end; i++) {
      const int64_t row = off(i);
      const bool more = i + 1 < i_end;
      const bool n1 = more && nz(i + 1);
      V wn = ldvp<T, C>(w, off(i + 2), jld && more);
      V pn_ = ldvp<T, C>(pin, off(i + 2), jld && more && nz(i + 2));
      V qn = ldvp<T, C>(qin, off(i + 1), jld && n1);
      V won = ldvp<T, C>(wo, off(i + 1), jld && more);
      V cn = ldvp<T, C>(cc, off(i + 1), jld && more);
      const T hwn = ld1p(w + row + P + hoff, more && hon),
              hqn = ld1p(qin + row + P + hoff, more && hon && n1);
      V rdn{};
      if constexpr (PK == 3) rdn = ldvp<T, C>(rdt, off(i + 1), jld && more);
      T wL = __shfl_up_sync(FULL, w0.v[C - 1], 1), wR = __shfl_down_sync(FULL, w0.v[0], 1);
      T qL = __shfl_up_sync(FULL, q0.v[C - 1], 1), qR = __shfl_down_sync(FULL, q0.v[0], 1);
      if (lane == 0) {
        wL = hw;
        qL = hq;
      } else if (lane == 31) {
        wR = hw;
        qR = hq;
      }
      if (jld) {
        const T sg = PK == 2 ? T(0) : sx[i];
        // PK 1, 3: the row's factors
        T ar_r = T(1), r_r = T(1), e_r = T(1), exs = T(0), eys = T(0);
        if constexpr (PK == 1 || PK == 3) {
          const int n = nx + 2;
          if constexpr (PK == 1) {
            r_r = sxk[KT_R * n + i];
            ar_r = sxk[KT_AR * n + i];
          }
          e_r = sxk[KT_E * n + i];
          exs = sxk[KT_EX * n + i];
          eys = sxk[KT_EY * n + i];
        }
        V vo, po, qo, dv;
#pragma unroll
        for (int c = 0; c < C; c++) {
          const T wS = c == 0 ? wL : w0.v[c - 1];
          const T wN = c == C - 1 ? wR : w0.v[c + 1];
          const T qS = c == 0 ? qL : q0.v[c - 1];
          const T qN = c == C - 1 ? qR : q0.v[c + 1];
          const T cv = c0.v[c], s = sg + tj[c];
          T v;
          if constexpr (PK == 3) {
            // three-level form, both profiles
            const T rd = rd0.v[c];
            v = ((T(2) - sg * tj[c] * K.dt2 - K.kxy * cv) * w0.v[c] +
                 cv * K.cx * (wp.v[c] + wm.v[c]) + cv * K.cy * (wN + wS) +
                 K.fx * (pp.v[c] - pm.v[c]) + K.fy * (qN - qS)) * rd -
                (T(2) * rd - T(1)) * wo0.v[c];
            for (int e = it.src_b; e < it.src_e; e++) {
              const CellRef r = srcs[e];
              if (r.cell == row + c) v += srcv[(int64_t)(t - 1) * sh.nsrc + r.idx];
            }
            po.v[c] = e_r * p0.v[c] + cv * (K.ex * tj[c] - exs) * (wp.v[c] - wm.v[c]);
            qo.v[c] = (T(1) - K.dt * tj[c]) * q0.v[c] + cv * (eys - K.ey * tj[c]) * (wN - wS);
          } else if constexpr (PK != 0) {
            // three-level form, sigma tau = 0: s = sigma (PK 1) or tau (PK 2)
            v = ((T(2) - K.kxy * cv) * w0.v[c] + cv * K.cx * (wp.v[c] + wm.v[c]) +
                 cv * K.cy * (wN + wS) + K.fx * (pp.v[c] - pm.v[c]) + K.fy * (qN - qS)) *
                    (PK == 1 ? r_r : rc[c]) -
                (PK == 1 ? ar_r : arc[c]) * wo0.v[c];
            for (int e = it.src_b; e < it.src_e; e++) {
              const CellRef r = srcs[e];
              if (r.cell == row + c) v += srcv[(int64_t)(t - 1) * sh.nsrc + r.idx];
            }
            if constexpr (PK == 1) {
              po.v[c] = e_r * p0.v[c] - exs * cv * (wp.v[c] - wm.v[c]);
              qo.v[c] = q0.v[c] + eys * cv * (wN - wS);
            } else {
              po.v[c] = p0.v[c] + ext[c] * cv * (wp.v[c] - wm.v[c]);
              qo.v[c] = bq[c] * q0.v[c] - eyt[c] * cv * (wN - wS);
            }
          } else if constexpr (INC) {
            // d_{t} = [(1 - s dt/2) d_{t-1} + c (cx (u_{i+1} - u) + ...) - sigma tau dt^2 u
            //          + phi / psi terms] / (1 + s dt/2), the three-level update less u_{t-1}
            const T u0 = w0.v[c];
            T dn = (T(1) - s * K.hdt) * wo0.v[c] +
                   cv * (K.cx * ((wp.v[c] - u0) + (wm.v[c] - u0)) +
                         K.cy * ((wN - u0) + (wS - u0))) -
                   sg * tj[c] * K.dt2 * u0 + K.fx * (pp.v[c] - pm.v[c]) + K.fy * (qN - qS);
            dn = pml_damp<T>(dn, s, K);
            for (int e = it.src_b; e < it.src_e; e++) {
              const CellRef r = srcs[e];
              if (r.cell == row + c) dn += srcv[(int64_t)(t - 1) * sh.nsrc + r.idx];
            }
            dv.v[c] = dn;
            v = u0 + dn;
          } else {
            v = (T(2) - sg * tj[c] * K.dt2 - K.kxy * cv) * w0.v[c] +
                cv * K.cx * (wp.v[c] + wm.v[c]) + cv * K.cy * (wN + wS) +
                K.fx * (pp.v[c] - pm.v[c]) + K.fy * (qN - qS) - (T(1) - s * K.hdt) * wo0.v[c];
            v = pml_damp<T>(v, s, K);
            for (int e = it.src_b; e < it.src_e; e++) {
              const CellRef r = srcs[e];
              if (r.cell == row + c) v += srcv[(int64_t)(t - 1) * sh.nsrc + r.idx];
            }
          }
          vo.v[c] = v;
          if constexpr (!VU && PK == 0) {
            po.v[c] = (T(1) - K.dt * sg) * p0.v[c] + K.ex * cv * (tj[c] - sg) * (wp.v[c] - wm.v[c]);
            qo.v[c] = (T(1) - K.dt * tj[c]) * q0.v[c] + K.ey * cv * (sg - tj[c]) * (wN - wS);
          }
        }
        stv<T, C>(out, row, vo, j, ny);
        if constexpr (INC) stv<T, C>(dd, row, dv, j, ny);
        if (!VU && n0) {
          stv<T, C>(pout, row, po, j, ny);
          stv<T, C>(qout, row, qo, j, ny);
        }
        if (ck_on) {
          T* ck = sh.ckpt + (int64_t)ckpt_slot * 4 * fs;
          stv<T, C>(ck, row, vo, j, ny);
          stv<T, C>(ck + fs, row, INC ? dv : w0, j, ny);
          if (n0) {
            stv<T, C>(ck + 2 * fs, row, VU ? p0 : po, j, ny);
            stv<T, C>(ck + 3 * fs, row, VU ? q0 : qo, j, ny);
          }
        }
      }
      wm = w0;
      w0 = wp;
      wp = wn;
      pm = p0;
      p0 = pp;
      pp = pn_;
      q0 = qn;
      wo0 = won;
      c0 = cn;
      hw = hwn;
      hq = hqn;
      n0 = n1;
      if constexpr (PK == 3) rd0 = rdn;
    }
  };
  constexpr bool SPEC = sizeof(T) == 8 && !INC;
  bool sfree = false;
  if constexpr (SPEC) {
    bool z = true;
    for (int r = i0 + lane; r < i_end; r += 32) z = z && sx[r] == T(0);
    sfree = __all_sync(FULL, z);
  }
  if (SPEC && tfree) pml_rows(std::integral_constant<int, SPEC ? 1 : 0>{});
  else if (SPEC && sfree) pml_rows(std::integral_constant<int, SPEC ? 2 : 0>{});
  else pml_rows(std::integral_constant<int, SPEC ? 3 : 0>{});
  record_traces<T, C, NOREC>(it, sh, rcvs, out, t, lane, i0, i_end);
  }
}

// Restore checkpoint `slot` of every active shot: u_{a-1} into segment-store
// slot 1 and, in the three-level form, u_{a-2} into slot 0 (increment form,
// inc = 1: d_{a-1} into the increment field), and phi / psi into set `pset`
// (-1: set (a-1) & 1).
template <typename T>
__global__ void __launch_bounds__(256)
k_ac_restore(const AcShot<T>* __restrict__ shots, int slot, int a, int pset, int inc) {
  const AcShot<T>& sh = shots[blockIdx.y];
  const int64_t P = sh.pitch, fs = sh.fs;
  const T* ck = sh.ckpt + (int64_t)slot * 4 * fs;
  const int ps = pset >= 0 ? pset : ((a - 1) & 1);  // phi/psi set the recompute reads
  T* pr = sh.p + (int64_t)ps * fs;
  T* qr = sh.q + (int64_t)ps * fs;
  T* second = inc ? sh.d : sh.seg;
  for (int i = 1 + blockIdx.x; i <= sh.nx; i += gridDim.x)
    for (int j = 1 + threadIdx.x; j <= sh.ny; j += blockDim.x) {
      const int64_t row = (int64_t)i * P + j + JOFF;
      second[row] = ck[fs + row];
      sh.seg[fs + row] = ck[row];
      pr[row] = ck[2 * fs + row];
      qr[row] = ck[3 * fs + row];
    }
}

// Copy u_{a-2} and u_{a-1} from the rings into the store slots a-2-base and
// a-1-base of every active shot: the start of the resident segments.
template <typename T>
__global__ void __launch_bounds__(256)
k_ac_seed(const AcShot<T>* __restrict__ shots, int a, int base) {
  const AcShot<T>& sh = shots[blockIdx.y];
  const int64_t fs = sh.fs;
  const T* __restrict__ u2 = sh.u + (int64_t)((a - 2) & 1) * fs;
  const T* __restrict__ u1 = sh.u + (int64_t)((a - 1) & 1) * fs;
  T* __restrict__ d2 = sh.seg + (int64_t)(a - 2 - base) * fs;
  T* __restrict__ d1 = sh.seg + (int64_t)(a - 1 - base) * fs;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < fs;
       e += (int64_t)gridDim.x * blockDim.x) {
    d2[e] = u2[e];
    d1[e] = u1[e];
  }
}

// ---------------------------------------------------------------------------
// Interior forward step fed by TMA (FP32 increment form; ads_acoustic_config
// tma = 1).  The register queues of k_ac_fwd keep about three 256-byte rows
// in flight per warp, too few to cover the DRAM latency at full bandwidth;
// here one thread of a CTA
// issues tensor-map tile copies (cp.async.bulk.tensor) of TMA_RB-row chunks
// of u (with a one-column and one-row halo), d and c into shared memory,
// TMA_ST chunks ahead, each chunk completing on its own mbarrier, and the four
// warps compute from shared memory.  The CTA takes a whole interior item (one
// 64-column strip of one shot, rows [i0, i0 + gh)); the arithmetic is that of
// k_ac_fwd's interior loop.  Launched alone it is faster than the register
// kernel (21.3 against 25.9 us on 16 shots of 1000 x 500), but beside the
// concurrent PML-item launch the whole step is not (47.4 against 47.8
// shot-gradients/s at two chunks in flight, 45.1 at four), so it is opt-in.
//
// Every wait is bounded by the SM clock: if a chunk has not arrived after
// about a second the CTA records ADS_ERR_TIMEOUT's flag in *err, waits (again
// bounded) for the copies it has in flight and returns; the plan reports the
// flag on its next call.  The tile origins are multiples of 4 columns by
// construction (strips start at column 1 + 64k of the pitched layout with
// JOFF = 31); the kernel checks that before issuing any copy.
// ---------------------------------------------------------------------------
#ifndef ADS_TMA_RB
#define ADS_TMA_RB 8
#endif
constexpr int TMA_RB = ADS_TMA_RB;                           // rows of a chunk
#ifndef ADS_TMA_ST
#define ADS_TMA_ST 2
#endif
constexpr int TMA_ST = ADS_TMA_ST;                           // chunks in flight
constexpr int TMA_UW = 72;                                   // u box: columns j0-4 .. j0+67
constexpr int TMA_W = 64;                                    // d, c boxes: columns j0 .. j0+63
constexpr int TMA_UBYTES = TMA_UW * (TMA_RB + 2) * 4;        // 2880
constexpr int TMA_DBYTES = TMA_W * TMA_RB * 4;               // 2048
constexpr int TMA_UOFF = 0;
constexpr int TMA_DOFF = (TMA_UBYTES + 127) / 128 * 128;     // 2944
constexpr int TMA_COFF = TMA_DOFF + TMA_DBYTES;
constexpr int TMA_STAGE = TMA_COFF + TMA_DBYTES;             // 7040 bytes a chunk
constexpr int TMA_SMEM = TMA_ST * TMA_STAGE + TMA_ST * 8;    // + the mbarriers
constexpr long long kTmaWaitCycles = 2000000000LL;           // about 1 s at 2 GHz
#ifndef ADS_MINB_FT32
#define ADS_MINB_FT32 12  // resident CTAs per SM of the TMA-fed interior forward (40 registers)
#endif

// Per shot: the tensor maps of u's two-slot ring, the segment store, d and c
// (written once at plan creation; CUtensorMap carries its own alignment).
struct AcTmaMaps {
  CUtensorMap ring, seg, d, c;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t a, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t a, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
// wait for phase `parity` of the mbarrier at a, at most kTmaWaitCycles
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t a, unsigned parity) {
  if (mbar_try_wait(a, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(a, parity))
    if (clock64() - t0 > kTmaWaitCycles) return false;
  return true;
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

template <int MODE, bool CK>
__global__ void __launch_bounds__(Tile<float>::TPB, ADS_MINB_FT32)
k_ac_fwd_tma(const AcItem* __restrict__ items, const AcShot<float>* __restrict__ shots,
             const AcTmaMaps* __restrict__ maps, AcConst<float> K, int t, int base,
             int ckpt_slot, int gh, int* __restrict__ err) {
  constexpr bool SEG = MODE != 0;
  extern __shared__ __align__(128) unsigned char tsm[];
  const AcItem it = items[blockIdx.x];
  const AcShot<float>& sh = shots[it.shot];
  const AcTmaMaps* mp = maps + it.shot;
  const int nx = sh.nx, ny = sh.ny;
  const int i0 = it.i0, i_end = min(i0 + gh, nx + 1);
  if (i0 > nx) return;  // (whole CTA)
  const int nch = (i_end - i0 + TMA_RB - 1) / TMA_RB;
  const int xu = it.j0 + JOFF - 4, xd = it.j0 + JOFF;
  if ((xu & 3) != 0 || (xd & 3) != 0) {  // a tile origin off the 16-byte grid: copy nothing
    if (threadIdx.x == 0) atomicOr(err, 2);
    return;
  }
  const int64_t P = sh.pitch, fs = sh.fs;
  float* out = SEG ? sh.seg + (int64_t)(t - base) * fs : sh.u + (int64_t)(t & 1) * fs;
  float* dd = sh.d;
  const int zu = SEG ? t - 1 - base : (t - 1) & 1;
  const CUtensorMap* mu = SEG ? &mp->seg : &mp->ring;
  const uint32_t sbase = smem_addr(tsm), bar0 = sbase + TMA_ST * TMA_STAGE;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TMA_ST; s++) mbar_init(bar0 + 8 * s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int ch) {  // thread 0
    const int s = ch % TMA_ST;
    const uint32_t st = sbase + s * TMA_STAGE, bar = bar0 + 8 * s;
    const int r0 = i0 + ch * TMA_RB;
    mbar_expect_tx(bar, TMA_UBYTES + 2 * TMA_DBYTES);
    tma_load_3d(st + TMA_UOFF, mu, xu, r0 - 1, zu, bar);
    tma_load_2d(st + TMA_DOFF, &mp->d, xd, r0, bar);
    tma_load_2d(st + TMA_COFF, &mp->c, xd, r0, bar);
  };
  if (threadIdx.x == 0)
    for (int ch = 0; ch < min(TMA_ST, nch); ch++) issue(ch);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = it.j0 + 2 * lane;
  const bool ck_on = CK && !SEG && ckpt_slot > 0 && ckpt_slot < sh.nseg;
  float* ck = ck_on ? sh.ckpt + (int64_t)ckpt_slot * 4 * fs : nullptr;
  for (int ch = 0; ch < nch; ch++) {
    const int s = ch % TMA_ST;
    const bool ok = mbar_wait_bounded(bar0 + 8 * s, (ch / TMA_ST) & 1);
    if (__syncthreads_or(!ok)) {
      // record, let the copies in flight (chunks ch .. ch + TMA_ST - 1) land, stop
      if (threadIdx.x == 0) {
        atomicOr(err, 1);
        for (int c2 = ch; c2 < min(ch + TMA_ST, nch); c2++)
          mbar_wait_bounded(bar0 + 8 * (c2 % TMA_ST), (c2 / TMA_ST) & 1);
      }
      __syncthreads();
      return;
    }
    const float* U = reinterpret_cast<const float*>(tsm + s * TMA_STAGE + TMA_UOFF);
    const float* D = reinterpret_cast<const float*>(tsm + s * TMA_STAGE + TMA_DOFF);
    const float* Cc = reinterpret_cast<const float*>(tsm + s * TMA_STAGE + TMA_COFF);
#pragma unroll
    for (int k = 0; k < TMA_RB / Tile<float>::G; k++) {
      const int q = warp * (TMA_RB / Tile<float>::G) + k;  // row of the chunk
      const int i = i0 + ch * TMA_RB + q;
      if (i >= i_end) break;
      // u rows i-1, i, i+1 are box rows q, q+1, q+2; column j + c is box column 4 + 2 lane + c
      const float* u1 = U + (q + 1) * TMA_UW + 4 + 2 * lane;
      const Vec<float, 2> u0 = *reinterpret_cast<const Vec<float, 2>*>(u1);
      const Vec<float, 2> um = *reinterpret_cast<const Vec<float, 2>*>(u1 - TMA_UW);
      const Vec<float, 2> up = *reinterpret_cast<const Vec<float, 2>*>(u1 + TMA_UW);
      const float uS = u1[-1], uN = u1[2];
      const Vec<float, 2> dv0 = *reinterpret_cast<const Vec<float, 2>*>(D + q * TMA_W + 2 * lane);
      const Vec<float, 2> cv = *reinterpret_cast<const Vec<float, 2>*>(Cc + q * TMA_W + 2 * lane);
      Vec<float, 2> vo, dv;
#pragma unroll
      for (int c = 0; c < 2; c++) {
        const float wS = c == 0 ? uS : u0.v[0];
        const float wN = c == 1 ? uN : u0.v[1];
        const float x0 = u0.v[c];
        dv.v[c] = dv0.v[c] + cv.v[c] * (K.cx * ((up.v[c] - x0) + (um.v[c] - x0)) +
                                        K.cy * ((wN - x0) + (wS - x0)));
        vo.v[c] = x0 + dv.v[c];
      }
      if (j <= ny) {
        const int64_t row = (int64_t)i * P + j + JOFF;
        stv<float, 2>(out, row, vo, j, ny);
        stv<float, 2>(dd, row, dv, j, ny);
        if (ck_on) {
          stv<float, 2>(ck, row, vo, j, ny);
          stv<float, 2>(ck + fs, row, dv, j, ny);
        }
      }
    }
    __syncthreads();  // every warp is done with chunk ch's stage
    if (threadIdx.x == 0 && ch + TMA_ST < nch) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(ch + TMA_ST);
    }
  }
}

// One cell's j-direction adjoint terms: YP (to its j+1 neighbour), YM (to its
// j-1 neighbour), YR (to psi's j+-1 neighbours).
template <typename T>
__device__ __forceinline__ void col_terms(T gui, T gq, T c, T sg, T tj, const AcConst<T>& K,
                                          T& YP, T& YM, T& YR) {
  const T by = c * K.cy * gui, eyg = K.ey * c * (sg - tj) * gq;
  YP = by + eyg;
  YM = by - eyg;
  YR = K.fy * gui;
}

template <typename T>
__device__ __forceinline__ T inv_den(T s, const AcConst<T>& K) {
  return pml_damp<T>(T(1), s, K);
}

// The grad_c accumulator an adjoint step adds to: the FP32 per-segment
// partial in FP32 plans, the FP64 accumulator in FP64 plans.
template <typename T>
struct GradOf {
  using type = double;
};
template <>
struct GradOf<float> {
  using type = float;
};
__device__ __forceinline__ float* grad_base(const AcShot<float>& sh) { return sh.gc32; }
__device__ __forceinline__ double* grad_base(const AcShot<double>& sh) { return sh.gc; }

// grad_c += g for a thread's C cells: the FP32 per-segment partial in FP32
// plans, the FP64 accumulator in FP64 plans; one vector access when all C
// cells are interior.
template <typename T, int C, typename I = int64_t>
__device__ __forceinline__ void add_grad(const AcShot<T>& sh, I row, const T (&g)[C], int j,
                                         int ny) {
  if (sizeof(T) == 4) {
    float* gp = sh.gc32 + row;
    if (j + C - 1 <= ny) {
      Vec<float, C> a = *reinterpret_cast<const Vec<float, C>*>(gp);
#pragma unroll
      for (int c = 0; c < C; c++) a.v[c] += (float)g[c];
      *reinterpret_cast<Vec<float, C>*>(gp) = a;
    } else {
#pragma unroll
      for (int c = 0; c < C; c++)
        if (j + c <= ny) gp[c] += (float)g[c];
    }
  } else {
#pragma unroll
    for (int c = 0; c < C; c++)
      if (j + c <= ny) sh.gc[row + c] += (double)g[c];
  }
}

// Source-time gradient: the forward adds srcv[t-1] dt^2 to u_t at a source
// cell (t >= 2), so d loss / d srcv[t-1] = dt^2 lambdaU_t there.  After the
// adjoint step k (and the residuals of slot k-1) lambdaU_{k-1} is final: the
// warp that wrote a source cell records it.
//
// Variant U: the source value also left phi_{k-1} and psi_{k-1} (the pre-pass
// formed them from u_{k-1} less its source value), so d loss / d srcv is
// lambdaU_{k-1} less the part of it that came back through phi_{k-1},
// psi_{k-1}: Q = sum over the four neighbours of what their lambdaPhi_{k-1},
// lambdaPsi_{k-1} (lp, lq, written by the pre-pass) sent to the cell.
//
// An item's source list may hold sources of neighbouring cells (variant U
// lists also carry those within one cell of the item); only the warp owning a
// source's cell (its rows and the strip's columns) records it.
template <typename T, int C, bool VU>
__device__ __forceinline__ void record_src_grad(const AcItem& it, const AcShot<T>& sh,
                                                const CellRef* __restrict__ srcs, const T* lun,
                                                const T* lp, const T* lq, const AcConst<T>& K,
                                                int k, int lane, int i0, int i_end, double dt2) {
  if (k - 1 < 2 || it.src_e <= it.src_b) return;
  __syncwarp();
  for (int e = it.src_b + lane; e < it.src_e; e += 32) {
    const CellRef r = srcs[e];
    const int jc = (int)(r.cell - (int64_t)r.row * sh.pitch) - JOFF;
    if (r.row < i0 || r.row >= i_end || jc < it.j0 || jc >= it.j0 + 32 * C) continue;
    double g = (double)lun[r.cell];
    if constexpr (VU) {
      const int64_t P = sh.pitch, x = r.cell;
      const T* cc = sh.c;
      const T sm = sh.sx[r.row - 1], s0 = sh.sx[r.row], sp = sh.sx[r.row + 1];
      const T tm = sh.ty[jc - 1], t0 = sh.ty[jc], tp = sh.ty[jc + 1];
      const T q = K.ex * cc[x - P] * (t0 - sm) * lp[x - P] - K.ex * cc[x + P] * (t0 - sp) * lp[x + P] +
                  K.ey * cc[x - 1] * (s0 - tm) * lq[x - 1] - K.ey * cc[x + 1] * (s0 - tp) * lq[x + 1];
      g -= (double)q;
    }
    sh.gsrc[(int64_t)(k - 2) * sh.nsrc + r.idx] = dt2 * g;
  }
}

// The source value added to u_t at pitched cell `cell` (0 where none; t >= 2):
// the sum over the item's listed sources there, as the forward injects them.
template <typename T>
__device__ __forceinline__ T src_at(const AcItem& it, const AcShot<T>& sh,
                                    const CellRef* __restrict__ srcs, int64_t cell, int t) {
  T v = T(0);
  for (int e = it.src_b; e < it.src_e; e++) {
    const CellRef r = srcs[e];
    if (r.cell == cell) v += sh.srcv[(int64_t)(t - 1) * sh.nsrc + r.idx];
  }
  return v;
}

// Residuals of step k-1 go to receiver cells this warp's lanes wrote in the
// adjoint step: a warp barrier suffices.
template <typename T, int C>
__device__ __forceinline__ void inject_residuals(const AcItem& it, const AcShot<T>& sh,
                                                 const CellRef* __restrict__ rcvs, T* lun, int k,
                                                 int lane, int i0, int i_end) {
  if (k - 1 < 2 || it.rcv_e <= it.rcv_b) return;
  __syncwarp();
  for (int e = it.rcv_b + lane; e < it.rcv_e; e += 32) {
    const CellRef r = rcvs[e];
    if (r.row >= i0 && r.row < i_end)
      atomicAdd(lun + r.cell, sh.resid[(int64_t)(k - 1) * sh.nrcv + r.idx]);
  }
}

// One adjoint step k (gather form of the transpose of step k):
//   lambdaU_{k-1} = D lambdaU_{k+1} + sum of what u_k, phi_k, psi_k send to w,
//   lambdaPhi_{k-1}, lambdaPsi_{k-1} likewise, grad_c += d(step k)/dc . lambda_k,
// then lambdaU_{k-1} += residual_{k-1} at the receivers.  What a cell of row
// i+-1 sends to row i (XP/XM: through u's w-stencil and phi's w-difference;
// XR: through u's phi-difference) is formed from that row's lambdaU_k,
// lambdaPhi_k, c and 1/den, carried in registers as the thread walks down.
// FP32 plans add the grad_c contribution to a per-segment FP32 partial
// (flushed into the FP64 accumulator at the end of each segment); FP64 plans
// accumulate in FP64.
// Items, warps and INT as in k_ac_fwd.
//
// VU = true (variant U, PML items only): k_ac_adjphi_u has already formed
// lambdaPhi_{k-1}, lambdaPsi_{k-1} (the adjoints of the phi_{k-1}, psi_{k-1}
// that step k reads); lambdaU_{k-1} takes its phi / psi terms from those
// instead of from lambdaPhi_k, lambdaPsi_k, the grad_c terms of phi_{k-1},
// psi_{k-1} use them too (with u_{k-1} less its source value, as the forward
// pre-pass formed them), and the kernel writes no lambdaPhi / lambdaPsi.
template <typename T, bool INT, bool VU = false>
__global__ void __launch_bounds__(Tile<T>::TPB, INT ? Tile<T>::MINB_AI : Tile<T>::MINB_A)
k_ac_adj(const AcItem* __restrict__ items, const AcShot<T>* __restrict__ shots,
         const CellRef* __restrict__ srcs, const CellRef* __restrict__ rcvs, AcConst<T> K,
         int k, int base, int ri, double dt2) {
  constexpr int C = Tile<T>::CA;
  using V = Vec<T, C>;
  const AcItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int lane = threadIdx.x & 31;
  const int j = it.j0 + lane * C;
  const int nx = sh.nx, ny = sh.ny;
  const int64_t P = sh.pitch, fs = sh.fs;
  const T* w = sh.seg + (int64_t)(k - 1 - base) * fs;   // u_{k-1}
  T* lun = sh.lu + (int64_t)((k + 1) & 1) * fs;         // in: lambdaU_{k+1}; out: _{k-1}
  const T* luc = sh.lu + (int64_t)(k & 1) * fs;         // lambdaU_k
  // lambdaPhi / lambdaPsi read by this step: those of step k (variant W), or
  // those of phi_{k-1}, psi_{k-1} from the pre-pass (variant U)
  const T* lpc = sh.lp + (int64_t)((VU ? k - 1 : k) & 1) * fs;
  T* lpo = sh.lp + (int64_t)((k - 1) & 1) * fs;
  const T* lqc = sh.lq + (int64_t)((VU ? k - 1 : k) & 1) * fs;
  T* lqo = sh.lq + (int64_t)((k - 1) & 1) * fs;
  const T* __restrict__ cc = sh.c;
  const T* __restrict__ sx = sh.sx;
  const T* __restrict__ ty = sh.ty;
  const T* __restrict__ sxk = sh.sxk;
  const T* __restrict__ tyk = sh.tyk;
  const T* __restrict__ rdt = sh.rdt;
  const bool jld = j <= ny + 1;
  const bool hr = j + C <= ny + 1;
  // offsets within a field fit 32 bits (the plan checks fs < 2^31)
  const int col = j + JOFF, P32 = (int)P;
  T tj[C];
#pragma unroll
  for (int c = 0; c < C; c++) tj[c] = (j + c <= ny + 1) ? ty[j + c] : T(0);
  const bool tfree = warp_tau_free<T, C>(ty, j, ny);
  auto nz = [&](int r) { return !(tfree && sx[r] == T(0)); };
  // halo column of a warp-edge lane and its tau
  const int hoff = lane == 0 ? -1 : C;
  const bool hon = (lane == 0 && jld) || (lane == 31 && hr);
  const T th = hon ? ty[j + (int)hoff] : T(0);
  auto off = [&](int r) { return r * P32 + col; };
  const int i0 = it.i0 + (threadIdx.x >> 5) * ri, i_end = min(i0 + ri, nx + 1);
  if (i0 > nx) return;  // whole warps only: every later barrier is warp-level
  if (INT || interior_rows<T>(tfree, sx, i0, i_end, lane)) {
    // Interior tile (1/den = 1, lambdaPhi = lambdaPsi = 0): the transpose of
    // the plain wave update; rows i-1 (m), i (0), i+1 (1) of lambdaU_k and c.
    // Register queues PF rows deep: lambdaU_k, c, u_{k-1} rows i-1 .. i+PF;
    // lambdaU_{k+1}, the grad_c accumulator and the halo cells rows
    // i .. i+PF-1.
    constexpr int PF = Tile<T>::PF;
    using G = typename GradOf<T>::type;
    using VG = Vec<G, C>;
    G* gb = grad_base(sh);
    V uq[PF + 2], cq[PF + 2], wq[PF + 2], lq[PF];
    VG gq[PF];
    T hu[PF], hcq[PF], hwq[PF];
    auto load_halo = [&](int r, T& a, T& b, T& d) {
      a = b = d = T(0);
      if (hon && r < i_end) {
        const int o = off(r) + hoff;
        a = luc[o];
        b = cc[o];
        d = w[o];
      }
    };
#pragma unroll
    for (int q = 0; q < PF + 2; q++) {
      const bool on = jld && i0 - 1 + q <= i_end;
      uq[q] = ldv<T, C>(luc, off(i0 - 1 + q), on);
      cq[q] = ldv<T, C>(cc, off(i0 - 1 + q), on);
      wq[q] = ldv<T, C>(w, off(i0 - 1 + q), on);
    }
#pragma unroll
    for (int q = 0; q < PF; q++) {
      const bool on = jld && i0 + q < i_end;
      lq[q] = ldv<T, C>(lun, off(i0 + q), on);
      gq[q] = ldv<G, C>(gb, off(i0 + q), on);
      load_halo(i0 + q, hu[q], hcq[q], hwq[q]);
    }
    // FP64 plans (issue-bound) carry z = c lambdaU_k of rows i-1, i down the rows:
    // one product per cell instead of three
    constexpr bool ZF = sizeof(T) == 8;
    V zm, z0;
#pragma unroll
    for (int c = 0; c < C; c++) {
      zm.v[c] = ZF ? cq[0].v[c] * uq[0].v[c] : T(0);
      z0.v[c] = ZF ? cq[1].v[c] * uq[1].v[c] : T(0);
    }
    for (int i = i0; i < i_end; i++) {
      const int row = off(i);
      const int rn = i + PF;
      const bool on1 = jld && rn + 1 <= i_end, on0 = jld && rn < i_end;
      V un = ldv<T, C>(luc, off(rn + 1), on1);
      V cn = ldv<T, C>(cc, off(rn + 1), on1);
      V wn = ldv<T, C>(w, off(rn + 1), on1);
      V ln = ldv<T, C>(lun, off(rn), on0);
      VG gn = ldv<G, C>(gb, off(rn), on0);
      T hun, hcn, hwn;
      load_halo(rn, hun, hcn, hwn);
      const V &gum = uq[0], &gu0 = uq[1], &gu1 = uq[2];
      const V &cm = cq[0], &c0 = cq[1], &c1 = cq[2];
      const V &wm = wq[0], &w0 = wq[1], &wp = wq[2];
      // what each cell sends to its j-neighbours: c cy lambdaU (ZF: c lambdaU,
      // the cy applied once to the sum of both neighbours)
      T Y[C];
      V z1;
#pragma unroll
      for (int c = 0; c < C; c++) {
        if constexpr (ZF) {
          z1.v[c] = c1.v[c] * gu1.v[c];
          Y[c] = z0.v[c];
        } else {
          Y[c] = c0.v[c] * K.cy * gu0.v[c];
        }
      }
      T Yl = __shfl_up_sync(FULL, Y[C - 1], 1), Yr = __shfl_down_sync(FULL, Y[0], 1);
      T wL = __shfl_up_sync(FULL, w0.v[C - 1], 1), wR = __shfl_down_sync(FULL, w0.v[0], 1);
      if (lane == 0 || lane == 31) {
        const T h = hon ? (ZF ? hcq[0] * hu[0] : hcq[0] * K.cy * hu[0]) : T(0);
        if (lane == 0) {
          Yl = h;
          wL = hwq[0];
        } else {
          Yr = h;
          wR = hwq[0];
        }
      }
      if (jld) {
        V nu;
        VG ga = gq[0];
#pragma unroll
        for (int c = 0; c < C; c++) {
          const T yl = c == 0 ? Yl : Y[c - 1], yr = c == C - 1 ? Yr : Y[c + 1];
          const T wS = c == 0 ? wL : w0.v[c - 1], wN = c == C - 1 ? wR : w0.v[c + 1];
          const T cv = c0.v[c];
          if constexpr (ZF)
            nu.v[c] = (T(2) * gu0.v[c] - lq[0].v[c]) + K.cx * (zm.v[c] + z1.v[c]) +
                      K.cy * (yl + yr) - K.kxy * z0.v[c];
          else
            nu.v[c] = -lq[0].v[c] + (T(2) - K.kxy * cv) * gu0.v[c] +
                      cm.v[c] * K.cx * gum.v[c] + c1.v[c] * K.cx * gu1.v[c] + yl + yr;
          ga.v[c] += (G)((-K.kxy * w0.v[c] + K.cx * (wp.v[c] + wm.v[c]) + K.cy * (wN + wS)) *
                         gu0.v[c]);
        }
        stv<T, C>(lun, row, nu, j, ny);
        stv<G, C>(gb, row, ga, j, ny);
      }
      if constexpr (ZF) {
        zm = z0;
        z0 = z1;
      }
#pragma unroll
      for (int q = 0; q < PF + 1; q++) {
        uq[q] = uq[q + 1];
        cq[q] = cq[q + 1];
        wq[q] = wq[q + 1];
      }
      uq[PF + 1] = un;
      cq[PF + 1] = cn;
      wq[PF + 1] = wn;
#pragma unroll
      for (int q = 0; q < PF - 1; q++) {
        lq[q] = lq[q + 1];
        gq[q] = gq[q + 1];
        hu[q] = hu[q + 1];
        hcq[q] = hcq[q + 1];
        hwq[q] = hwq[q + 1];
      }
      lq[PF - 1] = ln;
      gq[PF - 1] = gn;
      hu[PF - 1] = hun;
      hcq[PF - 1] = hcn;
      hwq[PF - 1] = hwn;
    }
    if constexpr (!INT) {
      inject_residuals<T, C>(it, sh, rcvs, lun, k, lane, i0, i_end);
      record_src_grad<T, C, VU>(it, sh, srcs, lun, lpc, lqc, K, k, lane, i0, i_end, dt2);
    }
  } else {
  // The general (PML) form.  FP64 plans specialise it by the warp's kind, as
  // k_ac_fwd does: PK = 1 where tau = 0 at every column the
  // warp reads (1/den and the sigma terms per row from the damping tables),
  // PK = 2 where sigma = 0 on rows i0-1 .. i_end (1/den and the tau terms
  // per-thread constants), PK = 3 elsewhere (1/den from the per-cell table,
  // the sigma terms per row); PK = 0 (general, with divides) for FP32 plans.
  // Variant U uses the same forms (its phi / psi terms read the pre-pass's
  // values; it writes no lambdaPhi / lambdaPsi).
  auto pml_rows = [&](auto kd) {
    constexpr int PK = decltype(kd)::value;
    const int nr = nx + 2, ncol = ny + 2;
    // PK 2: the tables at this thread's columns and at its halo column
    T rc[C], arc[C], bq[C], ext[C], eyt[C], hrc = T(1), heyt = T(0);
#pragma unroll
    for (int c = 0; c < C; c++) {
      rc[c] = arc[c] = bq[c] = T(1);
      ext[c] = eyt[c] = T(0);
      if constexpr (PK == 2) {
        if (j + c <= ny + 1) {
          const int q = j + c;
          rc[c] = tyk[KT_R * ncol + q];
          arc[c] = tyk[KT_AR * ncol + q];
          bq[c] = tyk[KT_E * ncol + q];
          ext[c] = tyk[KT_EX * ncol + q];
          eyt[c] = tyk[KT_EY * ncol + q];
        }
      }
    }
    if constexpr (PK == 2) {
      if (hon) {
        hrc = tyk[KT_R * ncol + j + hoff];
        heyt = tyk[KT_EY * ncol + j + hoff];
      }
    }
    // phi / psi may be non-zero in row r (always, where tau != 0)
    auto nzk = [&](int r) { return PK == 2 || nz(r); };
    // 1/den of the cell in row r, column j + c
    auto invd = [&](int r, int c) -> T {
      if constexpr (PK == 1) return sxk[KT_R * nr + r];
      else if constexpr (PK == 2) return rc[c];
      else return inv_den<T>(sx[r] + tj[c], K);
    };
    // rows i-1 (m), i (0), i+1 (p): lambdaU_k, lambdaPhi_k, c and 1/den per cell
    V gum = ldvp<T, C>(luc, off(i0 - 1), jld), gpm = ldvp<T, C>(lpc, off(i0 - 1), jld && nzk(i0 - 1)),
      cm = ldvp<T, C>(cc, off(i0 - 1), jld);
    V gu0 = ldvp<T, C>(luc, off(i0), jld), gp0 = ldvp<T, C>(lpc, off(i0), jld && nzk(i0)),
      c0 = ldvp<T, C>(cc, off(i0), jld);
    V gu1 = ldvp<T, C>(luc, off(i0 + 1), jld), gp1 = ldvp<T, C>(lpc, off(i0 + 1), jld && nzk(i0 + 1)),
      c1 = ldvp<T, C>(cc, off(i0 + 1), jld);
    V invm, inv0, rd1{};  // PK 3: 1/den of rows i-1, i, i+1 from the table
    if constexpr (PK == 3) {
      invm = ldvp<T, C>(rdt, off(i0 - 1), jld);
      inv0 = ldvp<T, C>(rdt, off(i0), jld);
      rd1 = ldvp<T, C>(rdt, off(i0 + 1), jld);
    }
    V gim, gi0;  // lambdaU_k / den of rows i-1, i (carried down the rows)
#pragma unroll
    for (int c = 0; c < C; c++) {
      if constexpr (PK != 3) {
        invm.v[c] = invd(i0 - 1, c);
        inv0.v[c] = invd(i0, c);
      }
      gim.v[c] = gum.v[c] * invm.v[c];
      gi0.v[c] = gu0.v[c] * inv0.v[c];
    }
    V wm = ldvp<T, C>(w, off(i0 - 1), jld), w0 = ldvp<T, C>(w, off(i0), jld),
      wp = ldvp<T, C>(w, off(i0 + 1), jld);
    bool n0 = nzk(i0);
    V gq = ldvp<T, C>(lqc, off(i0), jld && n0), ln = ldvp<T, C>(lun, off(i0), jld);
    T hgu, hgq, hc, hw;
    {
      const int r = off(i0) + hoff;
      hgu = ld1p(luc + r, hon);
      hgq = ld1p(lqc + r, hon && n0);
      hc = ld1p(cc + r, hon);
      hw = ld1p(w + r, hon);
    }
    T hrd = T(1);  // PK 3: 1/den of the halo cell
    if constexpr (PK == 3) hrd = ld1p(rdt + off(i0) + hoff, hon);
    T sgm = PK == 2 ? T(0) : sx[i0 - 1], sg0 = PK == 2 ? T(0) : sx[i0];
    for (int i = i0; i < i_end; i++) {
      const int row = off(i);
      const T sgp = PK == 2 ? T(0) : sx[i + 1];
      V invp, gip, rd2{};
      if constexpr (PK == 3) {
        invp = rd1;
        rd2 = ldvp<T, C>(rdt, off(i + 2), jld && i + 1 < i_end);
      }
#pragma unroll
      for (int c = 0; c < C; c++) {
        if constexpr (PK != 3) invp.v[c] = invd(i + 1, c);
        gip.v[c] = gu1.v[c] * invp.v[c];
      }
      // PK 1, 3: the sigma terms of rows i-1, i, i+1 from the damping tables
      T exm = T(0), ex0 = T(0), exp_ = T(0), eys0 = T(0), ar0 = T(1), e0 = T(1);
      if constexpr (PK == 1 || PK == 3) {
        exm = sxk[KT_EX * nr + i - 1];
        ex0 = sxk[KT_EX * nr + i];
        exp_ = sxk[KT_EX * nr + i + 1];
        eys0 = sxk[KT_EY * nr + i];
        if constexpr (PK == 1) ar0 = sxk[KT_AR * nr + i];
        e0 = sxk[KT_E * nr + i];
      }
      // prefetch: row i+2 (lambdaU_k, lambdaPhi_k, c, u_{k-1}), row i+1 (lambdaPsi_k,
      // lambdaU_{k+1}) and the halo cell of row i+1
      const bool more = i + 1 < i_end;
      const bool n1 = more && nzk(i + 1);
      V gu2 = ldvp<T, C>(luc, off(i + 2), jld && more);
      V gp2 = ldvp<T, C>(lpc, off(i + 2), jld && more && nzk(i + 2));
      V c2 = ldvp<T, C>(cc, off(i + 2), jld && more);
      V w2 = ldvp<T, C>(w, off(i + 2), jld && more);
      V gqn = ldvp<T, C>(lqc, off(i + 1), jld && n1);
      V lnn = ldvp<T, C>(lun, off(i + 1), jld && more);
      const int rh = row + P32 + hoff;
      const T hgun = ld1p(luc + rh, more && hon), hgqn = ld1p(lqc + rh, more && hon && n1),
              hcn = ld1p(cc + rh, more && hon), hwn = ld1p(w + rh, more && hon);
      T hrdn = T(1);
      if constexpr (PK == 3) hrdn = ld1p(rdt + rh, more && hon);
      // j-direction terms of this thread's cells and of the neighbouring columns
      T YP[C], YM[C], YR[C], gui[C];
#pragma unroll
      for (int c = 0; c < C; c++) {
        gui[c] = gi0.v[c];
        if constexpr (PK == 0) {
          col_terms<T>(gui[c], gq.v[c], c0.v[c], sg0, tj[c], K, YP[c], YM[c], YR[c]);
        } else {
          const T by = c0.v[c] * K.cy * gui[c];
          const T ey = PK == 1 ? eys0 : (PK == 2 ? -eyt[c] : eys0 - K.ey * tj[c]);
          const T eyg = ey * c0.v[c] * gq.v[c];
          YP[c] = by + eyg;
          YM[c] = by - eyg;
          YR[c] = K.fy * gui[c];
        }
      }
      T YPl = __shfl_up_sync(FULL, YP[C - 1], 1), YRl = __shfl_up_sync(FULL, YR[C - 1], 1);
      T YMr = __shfl_down_sync(FULL, YM[0], 1), YRr = __shfl_down_sync(FULL, YR[0], 1);
      T wL = __shfl_up_sync(FULL, w0.v[C - 1], 1), wR = __shfl_down_sync(FULL, w0.v[0], 1);
      if (lane == 0 || lane == 31) {
        T a = 0, b = 0, r = 0;
        if (hon) {
          if constexpr (PK == 0) {
            col_terms<T>(hgu * inv_den<T>(sg0 + th, K), hgq, hc, sg0, th, K, a, b, r);
          } else {
            // PK 1: tau = 0 at the halo column too, so its 1/den is the row's
            const T hg = hgu * (PK == 1 ? inv0.v[0] : (PK == 2 ? hrc : hrd));
            const T hey = PK == 1 ? eys0 : (PK == 2 ? -heyt : eys0 - K.ey * th);
            const T by = hc * K.cy * hg, eyg = hey * hc * hgq;
            a = by + eyg;
            b = by - eyg;
            r = K.fy * hg;
          }
        }
        if (lane == 0) {
          YPl = a;
          YRl = r;
          wL = hw;
        } else {
          YMr = b;
          YRr = r;
          wR = hw;
        }
      }
      if (jld) {
        V nu, np, nq;
        T g[C];
#pragma unroll
        for (int c = 0; c < C; c++) {
          const T ypl = c == 0 ? YPl : YP[c - 1], yrl = c == 0 ? YRl : YR[c - 1];
          const T ymr = c == C - 1 ? YMr : YM[c + 1], yrr = c == C - 1 ? YRr : YR[c + 1];
          const T wS = c == 0 ? wL : w0.v[c - 1], wN = c == C - 1 ? wR : w0.v[c + 1];
          const T guim = gim.v[c], guip = gip.v[c];
          const T cv = c0.v[c];
          if constexpr (PK == 0) {
            const T XPm = cm.v[c] * K.cx * guim + K.ex * cm.v[c] * (tj[c] - sgm) * gpm.v[c];
            const T XMp = c1.v[c] * K.cx * guip - K.ex * c1.v[c] * (tj[c] - sgp) * gp1.v[c];
            const T s = sg0 + tj[c];
            nu.v[c] = -(T(1) - s * K.hdt) * inv0.v[c] * ln.v[c] +
                      (T(2) - sg0 * tj[c] * K.dt2 - K.kxy * cv) * gui[c] + XPm + XMp + ypl + ymr;
            if constexpr (!VU) {
              np.v[c] = (T(1) - K.dt * sg0) * gp0.v[c] + K.fx * guim - K.fx * guip;
              nq.v[c] = (T(1) - K.dt * tj[c]) * gq.v[c] + yrl - yrr;
            }
          } else if constexpr (PK == 3) {
            // both profiles: the sigma terms per row, 1/den per cell
            const T ext3 = K.ex * tj[c];
            const T XPm = cm.v[c] * (K.cx * guim + (ext3 - exm) * gpm.v[c]);
            const T XMp = c1.v[c] * (K.cx * guip - (ext3 - exp_) * gp1.v[c]);
            nu.v[c] = -(T(2) * inv0.v[c] - T(1)) * ln.v[c] +
                      (T(2) - sg0 * tj[c] * K.dt2 - K.kxy * cv) * gui[c] + XPm + XMp + ypl + ymr;
            np.v[c] = e0 * gp0.v[c] + K.fx * (guim - guip);
            nq.v[c] = (T(1) - K.dt * tj[c]) * gq.v[c] + yrl - yrr;
          } else {
            // sigma tau = 0; PK 1: tau = 0, PK 2: sigma = 0 (tables / constants)
            const T XPm = cm.v[c] * (K.cx * guim + (PK == 1 ? -exm : ext[c]) * gpm.v[c]);
            const T XMp = c1.v[c] * (K.cx * guip + (PK == 1 ? exp_ : -ext[c]) * gp1.v[c]);
            nu.v[c] = -(PK == 1 ? ar0 : arc[c]) * ln.v[c] + (T(2) - K.kxy * cv) * gui[c] + XPm +
                      XMp + ypl + ymr;
            np.v[c] = (PK == 1 ? e0 * gp0.v[c] : gp0.v[c]) + K.fx * (guim - guip);
            nq.v[c] = (PK == 1 ? gq.v[c] : bq[c] * gq.v[c]) + yrl - yrr;
          }
          T dx_ = wp.v[c] - wm.v[c], dy_ = wN - wS;
          if constexpr (VU) {
            // u_{k-1} without its source value, as the forward pre-pass used it
            if (k - 1 >= 2 && it.src_e > it.src_b) {
              const T sp = src_at(it, sh, srcs, row + P + c, k - 1),
                      sm = src_at(it, sh, srcs, row - P + c, k - 1);
              const T sn = src_at(it, sh, srcs, row + c + 1, k - 1),
                      ss = src_at(it, sh, srcs, row + c - 1, k - 1);
              dx_ = (wp.v[c] - sp) - (wm.v[c] - sm);
              dy_ = (wN - sn) - (wS - ss);
            }
          }
          if constexpr (PK == 0)
            g[c] = (-K.kxy * w0.v[c] + K.cx * (wp.v[c] + wm.v[c]) + K.cy * (wN + wS)) * gui[c] +
                   K.ex * (tj[c] - sg0) * dx_ * gp0.v[c] + K.ey * (sg0 - tj[c]) * dy_ * gq.v[c];
          else if constexpr (PK == 3)
            g[c] = (-K.kxy * w0.v[c] + K.cx * (wp.v[c] + wm.v[c]) + K.cy * (wN + wS)) * gui[c] +
                   (K.ex * tj[c] - ex0) * dx_ * gp0.v[c] + (eys0 - K.ey * tj[c]) * dy_ * gq.v[c];
          else
            g[c] = (-K.kxy * w0.v[c] + K.cx * (wp.v[c] + wm.v[c]) + K.cy * (wN + wS)) * gui[c] +
                   (PK == 1 ? -ex0 : ext[c]) * dx_ * gp0.v[c] +
                   (PK == 1 ? eys0 : -eyt[c]) * dy_ * gq.v[c];
        }
        stv<T, C>(lun, row, nu, j, ny);
        if (!VU && n0) {
          stv<T, C>(lpo, row, np, j, ny);
          stv<T, C>(lqo, row, nq, j, ny);
        }
        add_grad<T, C>(sh, row, g, j, ny);
      }
      gim = gi0; gpm = gp0; cm = c0; sgm = sg0;
      gi0 = gip;
      gu0 = gu1; gp0 = gp1; c0 = c1; inv0 = invp; sg0 = sgp;
      gu1 = gu2; gp1 = gp2; c1 = c2;
      wm = w0; w0 = wp; wp = w2;
      gq = gqn; ln = lnn;
      hgu = hgun; hgq = hgqn; hc = hcn; hw = hwn;
      n0 = n1;
      if constexpr (PK == 3) {
        rd1 = rd2;
        hrd = hrdn;
      }
    }
  };
  constexpr bool SPEC = sizeof(T) == 8;
  bool sfree = false;
  if constexpr (SPEC) {
    bool z = true;
    for (int r = i0 - 1 + lane; r <= i_end; r += 32) z = z && sx[r] == T(0);
    sfree = __all_sync(FULL, z);
  }
  if (SPEC && tfree) pml_rows(std::integral_constant<int, SPEC ? 1 : 0>{});
  else if (SPEC && sfree) pml_rows(std::integral_constant<int, SPEC ? 2 : 0>{});
  else pml_rows(std::integral_constant<int, SPEC ? 3 : 0>{});
  inject_residuals<T, C>(it, sh, rcvs, lun, k, lane, i0, i_end);
  record_src_grad<T, C, VU>(it, sh, srcs, lun, lpc, lqc, K, k, lane, i0, i_end, dt2);
  }
}

// ---------------------------------------------------------------------------
// Variant U (one_step, src/Core.jl:528-549, the reference's default
// PropagatorKernel = 0): phi and psi are updated from the NEW field,
//   u_t = F(u_{t-1}, u_{t-2}, phi_{t-1}, psi_{t-1}) (+ source),
//   phi_t = (1 - dt sigma) phi_{t-1} + dt c (tau - sigma) / (2 hx) (u_t(i+1) - u_t(i-1)),
// with u_t taken before its source value is added (the loop adds the source
// after one_step).  A step kernel cannot form phi_t from u_t at its tile's
// edges (the neighbouring tiles write u_t in the same launch), so the update
// of phi_{t-1}, psi_{t-1} moves to the start of step t, where u_{t-1} is in
// memory: k_ac_phi_u forms them (PML items only; elsewhere they stay 0), then
// the step kernel (k_ac_fwd<..., VU = true>) computes u_t from them exactly as
// the custom-operator form does.  The reverse sweep mirrors it: k_ac_adjphi_u
// forms lambdaPhi_{k-1}, lambdaPsi_{k-1} from lambdaU_k, then
// k_ac_adj<..., VU = true> uses them.  phi_NSTEP is never formed: no trace
// depends on it.
// ---------------------------------------------------------------------------

// phi_{t-1}, psi_{t-1} from phi_{t-2}, psi_{t-2} and u_{t-1} less its source
// value (PML items, forward step t; MODE as k_ac_fwd).  Ring parity: step t
// reads phi from set (t-1) & 1, so phi_{t-2} is in set t & 1.
template <typename T, int MODE>
__global__ void __launch_bounds__(Tile<T>::TPB, Tile<T>::MINB_F)
k_ac_phi_u(const AcItem* __restrict__ items, const AcShot<T>* __restrict__ shots,
           const CellRef* __restrict__ srcs, AcConst<T> K, int t, int base, int ri) {
  constexpr bool SEG = MODE != 0;
  constexpr int C = Tile<T>::CF;
  using V = Vec<T, C>;
  const AcItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int lane = threadIdx.x & 31;
  const int j = it.j0 + lane * C;
  const int nx = sh.nx, ny = sh.ny;
  const int64_t P = sh.pitch, fs = sh.fs;
  const T* w = SEG ? sh.seg + (int64_t)(t - 1 - base) * fs : sh.u + (int64_t)((t - 1) & 1) * fs;
  const T* pin = sh.p + (int64_t)(t & 1) * fs;
  T* pout = sh.p + (int64_t)((t - 1) & 1) * fs;
  const T* qin = sh.q + (int64_t)(t & 1) * fs;
  T* qout = sh.q + (int64_t)((t - 1) & 1) * fs;
  const T* __restrict__ cc = sh.c;
  const T* __restrict__ sx = sh.sx;
  const T* __restrict__ ty = sh.ty;
  const bool jld = j <= ny + 1;
  const bool hr = j + C <= ny + 1;
  const int64_t col = j + JOFF;
  T tj[C];
#pragma unroll
  for (int c = 0; c < C; c++) tj[c] = (j + c <= ny + 1) ? ty[j + c] : T(0);
  const bool tfree = warp_tau_free<T, C>(ty, j, ny);
  auto nz = [&](int r) { return !(tfree && sx[r] == T(0)); };
  const int i0 = it.i0 + (threadIdx.x >> 5) * ri, i_end = min(i0 + ri, nx + 1);
  if (i0 > nx) return;
  auto off = [&](int r) { return (int64_t)r * P + col; };
  const bool srcd = t - 1 >= 2 && it.src_e > it.src_b;  // u_{t-1} received source values
  const int64_t hoff = lane == 0 ? -1 : C;
  const bool hon = (lane == 0 && jld) || (lane == 31 && hr);
  V wm = ldvp<T, C>(w, off(i0 - 1), jld), w0 = ldvp<T, C>(w, off(i0), jld),
    wp = ldvp<T, C>(w, off(i0 + 1), jld);
  bool n0 = nz(i0);
  V p0 = ldvp<T, C>(pin, off(i0), jld && n0), q0 = ldvp<T, C>(qin, off(i0), jld && n0),
    c0 = ldvp<T, C>(cc, off(i0), jld && n0);
  T hw = ld1p(w + off(i0) + hoff, hon && n0);
  for (int i = i0; i < i_end; i++) {
    const int64_t row = off(i);
    const bool more = i + 1 < i_end;
    const bool n1 = more && nz(i + 1);
    V wn = ldvp<T, C>(w, off(i + 2), jld && more);
    V pn = ldvp<T, C>(pin, off(i + 1), jld && n1), qn = ldvp<T, C>(qin, off(i + 1), jld && n1),
      cn = ldvp<T, C>(cc, off(i + 1), jld && n1);
    const T hwn = ld1p(w + row + P + hoff, more && hon && n1);
    T wL = __shfl_up_sync(FULL, w0.v[C - 1], 1), wR = __shfl_down_sync(FULL, w0.v[0], 1);
    if (lane == 0) wL = hw;
    else if (lane == 31) wR = hw;
    if (jld && n0) {
      const T sg = sx[i];
      V po, qo;
#pragma unroll
      for (int c = 0; c < C; c++) {
        const T wS = c == 0 ? wL : w0.v[c - 1];
        const T wN = c == C - 1 ? wR : w0.v[c + 1];
        T dx_ = wp.v[c] - wm.v[c], dy_ = wN - wS;
        if (srcd) {
          const T sp = src_at(it, sh, srcs, row + P + c, t - 1),
                  sm = src_at(it, sh, srcs, row - P + c, t - 1);
          const T sn = src_at(it, sh, srcs, row + c + 1, t - 1),
                  ss = src_at(it, sh, srcs, row + c - 1, t - 1);
          dx_ = (wp.v[c] - sp) - (wm.v[c] - sm);
          dy_ = (wN - sn) - (wS - ss);
        }
        po.v[c] = (T(1) - K.dt * sg) * p0.v[c] + K.ex * c0.v[c] * (tj[c] - sg) * dx_;
        qo.v[c] = (T(1) - K.dt * tj[c]) * q0.v[c] + K.ey * c0.v[c] * (sg - tj[c]) * dy_;
      }
      stv<T, C>(pout, row, po, j, ny);
      stv<T, C>(qout, row, qo, j, ny);
    }
    wm = w0;
    w0 = wp;
    wp = wn;
    p0 = pn;
    q0 = qn;
    c0 = cn;
    hw = hwn;
    n0 = n1;
  }
}

// lambdaPhi_{k-1}, lambdaPsi_{k-1} (the adjoints of the phi_{k-1}, psi_{k-1}
// that forward step k read) from lambdaPhi_k, lambdaPsi_k and lambdaU_k: the
// transpose of phi_{k-1}'s appearance in u_k and in phi_k (PML items of the
// adjoint tiling).  The same expressions as the variant-W kernel's
// lambdaPhi / lambdaPsi.
template <typename T>
__global__ void __launch_bounds__(Tile<T>::TPB, Tile<T>::MINB_F)
k_ac_adjphi_u(const AcItem* __restrict__ items, const AcShot<T>* __restrict__ shots,
              AcConst<T> K, int k, int ri) {
  constexpr int C = Tile<T>::CA;
  using V = Vec<T, C>;
  const AcItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int lane = threadIdx.x & 31;
  const int j = it.j0 + lane * C;
  const int nx = sh.nx, ny = sh.ny;
  const int64_t P = sh.pitch, fs = sh.fs;
  const T* luc = sh.lu + (int64_t)(k & 1) * fs;
  const T* lpc = sh.lp + (int64_t)(k & 1) * fs;
  T* lpo = sh.lp + (int64_t)((k - 1) & 1) * fs;
  const T* lqc = sh.lq + (int64_t)(k & 1) * fs;
  T* lqo = sh.lq + (int64_t)((k - 1) & 1) * fs;
  const T* __restrict__ sx = sh.sx;
  const T* __restrict__ ty = sh.ty;
  const bool jld = j <= ny + 1;
  const bool hr = j + C <= ny + 1;
  const int64_t col = j + JOFF;
  T tj[C];
#pragma unroll
  for (int c = 0; c < C; c++) tj[c] = (j + c <= ny + 1) ? ty[j + c] : T(0);
  const bool tfree = warp_tau_free<T, C>(ty, j, ny);
  auto nz = [&](int r) { return !(tfree && sx[r] == T(0)); };
  const int i0 = it.i0 + (threadIdx.x >> 5) * ri, i_end = min(i0 + ri, nx + 1);
  if (i0 > nx) return;
  auto off = [&](int r) { return (int64_t)r * P + col; };
  const int64_t hoff = lane == 0 ? -1 : C;
  const bool hon = (lane == 0 && jld) || (lane == 31 && hr);
  const T th = hon ? ty[j + (int)hoff] : T(0);
  V gum = ldvp<T, C>(luc, off(i0 - 1), jld), gu0 = ldvp<T, C>(luc, off(i0), jld),
    gup = ldvp<T, C>(luc, off(i0 + 1), jld);
  bool n0 = nz(i0);
  V gp0 = ldvp<T, C>(lpc, off(i0), jld && n0), gq0 = ldvp<T, C>(lqc, off(i0), jld && n0);
  T hgu = ld1p(luc + off(i0) + hoff, hon && n0);
  for (int i = i0; i < i_end; i++) {
    const int64_t row = off(i);
    const bool more = i + 1 < i_end;
    const bool n1 = more && nz(i + 1);
    V gun = ldvp<T, C>(luc, off(i + 2), jld && more);
    V gpn = ldvp<T, C>(lpc, off(i + 1), jld && n1), gqn = ldvp<T, C>(lqc, off(i + 1), jld && n1);
    const T hgun = ld1p(luc + row + P + hoff, more && hon && n1);
    const T sgm = sx[i - 1], sg0 = sx[i], sgp = sx[i + 1];
    // lambdaU / den of this thread's cells (row i), sent to the j-neighbours' psi
    T YR[C];
#pragma unroll
    for (int c = 0; c < C; c++) YR[c] = K.fy * (gu0.v[c] * inv_den<T>(sg0 + tj[c], K));
    T yrl = __shfl_up_sync(FULL, YR[C - 1], 1), yrr = __shfl_down_sync(FULL, YR[0], 1);
    if (lane == 0 || lane == 31) {
      const T h = hon ? K.fy * (hgu * inv_den<T>(sg0 + th, K)) : T(0);
      if (lane == 0) yrl = h;
      else yrr = h;
    }
    if (jld && n0) {
      V np, nq;
#pragma unroll
      for (int c = 0; c < C; c++) {
        const T guim = gum.v[c] * inv_den<T>(sgm + tj[c], K);
        const T guip = gup.v[c] * inv_den<T>(sgp + tj[c], K);
        const T l = c == 0 ? yrl : YR[c - 1], r = c == C - 1 ? yrr : YR[c + 1];
        np.v[c] = (T(1) - K.dt * sg0) * gp0.v[c] + K.fx * guim - K.fx * guip;
        nq.v[c] = (T(1) - K.dt * tj[c]) * gq0.v[c] + l - r;
      }
      stv<T, C>(lpo, row, np, j, ny);
      stv<T, C>(lqo, row, nq, j, ny);
    }
    gum = gu0;
    gu0 = gup;
    gup = gun;
    gp0 = gpn;
    gq0 = gqn;
    hgu = hgun;
    n0 = n1;
  }
}

// ---------------------------------------------------------------------------
// Time-blocked forward (FP32 plans): NS <= KB steps per launch.
//
// A CTA of TB_THREADS threads owns one column each: output columns
// [jo, jo + TB_THREADS - 2 KB) and rows [i0, i0 + RB) of one shot, and reads a
// KB-cell halo around them.  It streams down the rows once; stage s (s = 0..NS-1)
// turns level s (time t0 + s - 1) into level s + 1 one row behind stage s - 1,
// so every level lives in registers (a 3-row window per stage) and only level 0
// is read from and the last level written to HBM.  j-neighbours come from the
// neighbouring lanes (warp edges through shared memory, exchanged once per
// row).  Cells outside the grid act as zeros; the halo's wrong values stay
// outside the output region (one column/row per stage).  FIRST mode reads and
// writes two alternating state sets (U_t, U_{t-1}, phi, psi) and writes
// checkpoints and receiver traces of every level; SEG mode takes U from the
// segment store and writes every level there.
// ---------------------------------------------------------------------------
constexpr int TB_THREADS = 256;
constexpr int TB_WARPS = TB_THREADS / 32;

struct TbItem {
  int shot, i0, jo, pad;
  int src_b, src_e;  // sources in the loaded region
  int rr_b, rr_e;    // receiver rows of the output region
};
struct TbSrc {
  int row, col, idx, pad;
};
struct TbRcvRow {
  int row, map_off;  // receiver index per thread of the tile row (-1: none)
};

template <typename T, bool SEG, int KB>
__global__ void __launch_bounds__(TB_THREADS)
k_ac_fwd_tb(const TbItem* __restrict__ items, const AcShot<T>* __restrict__ shots,
            const TbSrc* __restrict__ tsrc, const TbRcvRow* __restrict__ trow,
            const int* __restrict__ tmap, AcConst<T> K, int t0, int NS, int base, int in_set,
            int ckpt_slot, int RB) {
  __shared__ T edge[2][TB_WARPS][2][KB][2];  // [row parity][warp][lane 0 | 31][stage][u | psi]
  const TbItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nx = sh.nx, ny = sh.ny;
  const int jc = it.jo - KB + tid;
  const bool inside = jc >= 0 && jc <= ny + 1;
  const bool icol = jc >= 1 && jc <= ny;
  const bool outcol = icol && jc >= it.jo && jc < it.jo + TB_THREADS - 2 * KB;
  const int64_t P = sh.pitch, fs = sh.fs;
  const int64_t col = (int64_t)jc + JOFF;
  const int os = 1 - in_set;
  const T *w, *wo;
  if (SEG) {
    w = sh.seg + (int64_t)(t0 - 1 - base) * fs;
    wo = sh.seg + (int64_t)(t0 - 2 - base) * fs;
  } else {
    w = sh.u + (int64_t)in_set * fs;
    wo = sh.u2 + (int64_t)in_set * fs;
  }
  const T* pin = sh.p + (int64_t)in_set * fs;
  const T* qin = sh.q + (int64_t)in_set * fs;
  const T* __restrict__ cc = sh.c;
  const T* __restrict__ sx = sh.sx;
  const T tj = inside ? sh.ty[jc] : T(0);
  const int i1 = min(it.i0 + RB, nx + 1);
  auto ld = [&](const T* a, int r) -> T {
    return (inside && r >= 0 && r <= nx + 1) ? a[(int64_t)r * P + col] : T(0);
  };
  T ua[KB], ub[KB], pa[KB], pb[KB], qb[KB], ou[KB], op[KB], oq[KB], cl[KB + 1];
#pragma unroll
  for (int s = 0; s < KB; s++) {
    ua[s] = ub[s] = pa[s] = pb[s] = qb[s] = ou[s] = op[s] = oq[s] = T(0);
    cl[s] = T(0);
  }
  cl[KB] = T(0);
  const int rA = it.i0 - NS, rB = it.i0 - NS + 1;
  ua[0] = ld(w, rA);
  ub[0] = ld(w, rB);
  pa[0] = ld(pin, rA);
  pb[0] = ld(pin, rB);
  qb[0] = ld(qin, rB);
  cl[0] = ld(cc, rB);
  T uo1 = ld(wo, rB);
  const int r_first = it.i0 - NS + 2, r_last = i1 + NS - 1;
  if (lane == 0 || lane == 31) {
#pragma unroll
    for (int s = 0; s < KB; s++) {
      edge[r_first & 1][warp][lane == 31][s][0] = ub[s];
      edge[r_first & 1][warp][lane == 31][s][1] = qb[s];
    }
  }
  __syncthreads();
  for (int r = r_first; r <= r_last; r++) {
    const int par = r & 1;
    const T nu_in = ld(w, r), np_in = ld(pin, r), nq_in = ld(qin, r), nwo = ld(wo, r);
#pragma unroll
    for (int s = KB; s > 0; s--) cl[s] = cl[s - 1];
    cl[0] = ld(cc, r);
    T prevA = uo1;
#pragma unroll
    for (int s = 0; s < KB; s++) {
      if (s < NS) {
        const int x = r - s - 1;
        const int t = t0 + s;  // time of the level this stage produces
        const T uc = s == 0 ? nu_in : ou[s - 1];
        const T pc = s == 0 ? np_in : op[s - 1];
        T uS = __shfl_up_sync(FULL, ub[s], 1), uN = __shfl_down_sync(FULL, ub[s], 1);
        T qS = __shfl_up_sync(FULL, qb[s], 1), qN = __shfl_down_sync(FULL, qb[s], 1);
        if (lane == 0) {
          uS = warp > 0 ? edge[par][warp - 1][1][s][0] : T(0);
          qS = warp > 0 ? edge[par][warp - 1][1][s][1] : T(0);
        } else if (lane == 31) {
          uN = warp < TB_WARPS - 1 ? edge[par][warp + 1][0][s][0] : T(0);
          qN = warp < TB_WARPS - 1 ? edge[par][warp + 1][0][s][1] : T(0);
        }
        T v = T(0), pn = T(0), qn = T(0);
        if (icol && x >= 1 && x <= nx) {
          const T sg = sx[x], c = cl[s + 1], sm = sg + tj;
          v = (T(2) - sg * tj * K.dt2 - K.kxy * c) * ub[s] + c * K.cx * (uc + ua[s]) +
              c * K.cy * (uN + uS) + K.fx * (pc - pa[s]) + K.fy * (qN - qS) -
              (T(1) - sm * K.hdt) * prevA;
          if (sm != T(0)) v = v / (T(1) + sm * K.hdt);
          if (t <= sh.nstep)
            for (int e = it.src_b; e < it.src_e; e++) {
              const TbSrc q = tsrc[e];
              if (q.row == x && q.col == jc) v += sh.srcv[(int64_t)(t - 1) * sh.nsrc + q.idx];
            }
          pn = (T(1) - K.dt * sg) * pb[s] + K.ex * c * (tj - sg) * (uc - ua[s]);
          qn = (T(1) - K.dt * tj) * qb[s] + K.ey * c * (sg - tj) * (uN - uS);
        }
        if (outcol && x >= it.i0 && x < i1) {
          const int64_t cell = (int64_t)x * P + col;
          if (SEG) sh.seg[(int64_t)(t - base) * fs + cell] = v;
          if (!SEG && t <= sh.nstep) {
            for (int e = it.rr_b; e < it.rr_e; e++) {
              const TbRcvRow rr = trow[e];
              if (rr.row != x) continue;
              for (int idx = tmap[rr.map_off + tid]; idx >= 0; idx = sh.rcv_next[idx])
                sh.traces[(int64_t)t * sh.nrcv + idx] = v;
            }
          }
        }
        const T nextA = ua[s];  // level s at row x-1: the old field of stage s+1
        ua[s] = ub[s];
        ub[s] = uc;
        pa[s] = pb[s];
        pb[s] = pc;
        qb[s] = s == 0 ? nq_in : oq[s - 1];
        ou[s] = v;
        op[s] = pn;
        oq[s] = qn;
        prevA = nextA;
      }
    }
    uo1 = nwo;
    // the last stage finished row r - NS: write the block's final state
    const int xf = r - NS;
    if (outcol && xf >= it.i0 && xf < i1) {
      const int64_t cell = (int64_t)xf * P + col;
      T uf = T(0), ul = T(0), pf = T(0), qf = T(0);
#pragma unroll
      for (int s = 0; s < KB; s++)
        if (s == NS - 1) {
          uf = ou[s];
          ul = ua[s];
          pf = op[s];
          qf = oq[s];
        }
      if (!SEG) {
        sh.u[(int64_t)os * fs + cell] = uf;
        sh.u2[(int64_t)os * fs + cell] = ul;
        if (ckpt_slot > 0 && ckpt_slot < sh.nseg) {
          T* ck = sh.ckpt + (int64_t)ckpt_slot * 4 * fs;
          ck[cell] = uf;
          ck[fs + cell] = ul;
          ck[2 * fs + cell] = pf;
          ck[3 * fs + cell] = qf;
        }
      }
      sh.p[(int64_t)os * fs + cell] = pf;
      sh.q[(int64_t)os * fs + cell] = qf;
    }
    if (lane == 0 || lane == 31) {
#pragma unroll
      for (int s = 0; s < KB; s++) {
        edge[par ^ 1][warp][lane == 31][s][0] = ub[s];
        edge[par ^ 1][warp][lane == 31][s][1] = qb[s];
      }
    }
    __syncthreads();
  }
}

// End of a segment (FP32 plans): grad_c (FP64) += the segment's FP32 partial,
// which is reset to zero.
template <typename T>
__global__ void __launch_bounds__(256)
k_ac_flush_gc(const AcShot<T>* __restrict__ shots) {
  const AcShot<T>& sh = shots[blockIdx.y];
  for (int i = 1 + blockIdx.x; i <= sh.nx; i += gridDim.x)
    for (int j = 1 + threadIdx.x; j <= sh.ny; j += blockDim.x) {
      const int64_t row = (int64_t)i * sh.pitch + j + JOFF;
      sh.gc[row] += (double)sh.gc32[row];
      sh.gc32[row] = 0.f;
    }
}

// c = vp^2 over each shot's padded window (frames included: their c is read,
// multiplied by zero adjoint values).
template <typename T>
__global__ void k_ac_prep(const AcShot<T>* __restrict__ shots, const double* __restrict__ vp,
                          int64_t MYp2) {
  const AcShot<T>& sh = shots[blockIdx.y];
  const int64_t n = (int64_t)(sh.nx + 2) * (sh.ny + 2);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / (sh.ny + 2), j = e % (sh.ny + 2);
    const double v = vp[(sh.x0 + i) * MYp2 + j];
    sh.c[i * sh.pitch + j + JOFF] = (T)(v * v);
  }
}

// 1 / (1 + (sigma_i + tau_j) dt/2) over each shot's padded window: the damping
// of the FP64 PML kernels' corner warps, where both profiles meet.
template <typename T>
__global__ void k_ac_rden(const AcShot<T>* __restrict__ shots, double hdt) {
  const AcShot<T>& sh = shots[blockIdx.y];
  const int64_t n = (int64_t)(sh.nx + 2) * (sh.ny + 2);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / (sh.ny + 2), j = e % (sh.ny + 2);
    sh.rdt[i * sh.pitch + j + JOFF] =
        (T)(1.0 / fma((double)sh.sx[i] + (double)sh.ty[j], hdt, 1.0));
  }
}

// residual = 2 (trace - observed) in T; per-block FP64 partial sums of
// (trace - observed)^2 (deterministic two-pass reduction).
template <typename T>
__global__ void k_misfit(const T* __restrict__ tr, const T* __restrict__ obs,
                         T* __restrict__ resid, int64_t n, double* __restrict__ partial) {
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double d = (double)tr[e] - (double)obs[e];
    if (resid) resid[e] = (T)(2 * d);
    acc += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
  }
}

__global__ void k_reduce_sum(const double* __restrict__ partial, int n, double* out) {
  double acc = 0.0;
  for (int e = threadIdx.x; e < n; e += blockDim.x) acc += partial[e];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o);
    if (threadIdx.x == 0) *out = acc;
  }
}

// lambdaU_T = residual_T at each shot's receivers (rings were zeroed).
template <typename T>
__global__ void k_ac_adj_init(const AcShot<T>* __restrict__ shots,
                              const CellRef* __restrict__ rcvs, const int* __restrict__ rcv_b,
                              const int* __restrict__ rcv_e, double dt2) {
  const int s = blockIdx.x;
  const AcShot<T>& sh = shots[s];
  T* lu = sh.lu + (int64_t)(sh.nstep & 1) * sh.fs;
  for (int e = rcv_b[s] + threadIdx.x; e < rcv_e[s]; e += blockDim.x) {
    const CellRef r = rcvs[e];
    atomicAdd(lu + r.cell, sh.resid[(int64_t)sh.nstep * sh.nrcv + r.idx]);
  }
  // lambdaU_T is final: source-time gradient of the last row, srcv[T-1]
  __syncthreads();
  for (int e = threadIdx.x; e < sh.nsrc; e += blockDim.x) {
    const CellRef r = sh.src_list[e];
    sh.gsrc[(int64_t)(sh.nstep - 1) * sh.nsrc + r.idx] = dt2 * (double)lu[r.cell];
  }
}

// grad_vp = sum over shots covering the cell of (gc * 2) * vp.
template <typename T>
__global__ void k_ac_assemble(const AcShot<T>* __restrict__ shots, int nshots,
                              const double* __restrict__ vp, double* __restrict__ grad,
                              int64_t MXp2, int64_t MYp2) {
  const int64_t n = MXp2 * MYp2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t gi = e / MYp2, j = e % MYp2;
    double acc = 0.0;
    for (int s = 0; s < nshots; s++) {
      const AcShot<T>& sh = shots[s];
      const int64_t li = gi - sh.x0;
      if (li < 0 || li > sh.nx + 1 || j > sh.ny + 1) continue;
      acc += (sh.gc[li * sh.pitch + j + JOFF] * 2) * vp[e];
    }
    grad[e] = acc;
  }
}

// ---------------------------------------------------------------- host plan

struct DevPool {
  char* base = nullptr;
  size_t used = 0, cap = 0;
  size_t take(size_t bytes) {
    const size_t off = used;
    used += (bytes + 255) & ~size_t(255);
    return off;
  }
};

}  // namespace

struct AcPlanBase {
  virtual ~AcPlanBase() = default;
  virtual int forward(const double* vp, void* traces, cudaStream_t st) = 0;
  virtual int gradient(const double* vp, const void* obs, double* loss, double* grad,
                       void* traces_out, cudaStream_t st, double* grad_srcv) = 0;
  virtual int profile(const double* vp, const void* obs, double* out, cudaStream_t st) = 0;
  // new wavelets for a shot's sources (device FP64, (nstep, nsrc) row-major)
  virtual int set_source_values(int64_t shot, const double* srcv, cudaStream_t st) = 0;
  std::vector<int64_t> trace_off;
  int64_t trace_total = 0;
  std::vector<int64_t> src_off;  // per caller shot: offset of its (nstep, nsrc) block
  int64_t src_total = 0;
  int64_t bytes = 0;
  int64_t launches_fwd = 0, launches_grad = 0;
  int64_t resident = 0;  // checkpoint segments kept resident (no recompute)
  int64_t steps_per_block = 1;  // forward steps per launch (configured or tuned)
  int64_t uses_tma = 0;         // interior forward steps through tensor-map copies
  int64_t rows[4] = {0, 0, 0, 0};  // rows per warp: fwd / adj interior, fwd / adj PML
  virtual int device_status(cudaStream_t st) = 0;
};

namespace {

template <typename T>
struct AcPlan final : AcPlanBase {
  ads_acoustic_config cfg{};
  int nshots = 0;
  bool vu = false;    // variant U: phi / psi from the new field (pre-pass kernels)
  bool inc = false;   // FP32 increment form (k_ac_fwd INC); off for time blocking
  // FP32: interior forward steps through k_ac_fwd_tma (tensor maps per shot);
  // d_err collects its status flags (1: a bounded wait ran out, 2: a tile
  // origin off the 16-byte grid, never expected)
  bool tma_ok = false;
  AcTmaMaps* d_maps = nullptr;
  int* d_err = nullptr;
  std::vector<size_t> seg_slots;  // per sorted shot: store slots
  int build_maps(cudaStream_t st);
  int device_status(cudaStream_t st) override {
    int h = 0;
    if (d_err) {
      ADS_CUDA(cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
      ADS_CUDA(cudaStreamSynchronize(st));
    }
    if (h & 1) return fail(ADS_ERR_TIMEOUT, "a bounded wait of the tensor-map pipeline ran out");
    if (h & 2) return fail(ADS_ERR_INVALID, "internal: a tile origin off the 16-byte grid");
    return ADS_OK;
  }
  int K = 0;          // checkpoint spacing
  // Resident segments: segments res_seg .. nseg_max-1 keep the forward
  // wavefields of their steps in the shots' stores (slot t - res_base), so
  // the reverse sweep neither restores nor recomputes them.  res_seg ==
  // nseg_max: none.
  int res_seg = 0, res_base = 0;
  int ri = 8;         // rows per thread
  int nseg_max = 0;
  std::vector<int> order;         // shot order (record length descending)
  std::vector<T*> srcv_dev;        // per caller shot: its wavelets times dt^2
  std::vector<int64_t> srcv_n;     // per caller shot: nstep * nsrc
  std::vector<int> nstep;         // per sorted shot
  std::vector<int> nxs;           // per sorted shot: window width
  int ri_f = 8;                    // rows per thread of the forward tiles
  // per sorted shot, 0-based (i, j, index) of interior sources / receivers
  std::vector<std::vector<int3>> hsrc, hrcv;
  // per sorted shot: the PML profiles the kernels read (host copies)
  std::vector<std::vector<double>> hsx;
  std::vector<double> hty;
  // Warp items of one kernel: interior items (sigma = tau = 0 on every row and
  // column they read) and PML items, each in sorted-shot order, so the items
  // of the first n shots are a prefix of either part.
  struct TileList {
    std::vector<AcItem> in, pm;
    std::vector<int> in_end, pm_end;  // per sorted shot: items of shots [0..s]
    std::vector<CellRef> srcs, rcvs;
  };
  struct DevTiles {
    AcItem* items = nullptr;  // interior items, then the PML items at pm_off
    CellRef *srcs = nullptr, *rcvs = nullptr;
    int pm_off = 0;
    int vu = 0;  // variant U: the PML items get a pre-pass launch too
    std::vector<int> in_end, pm_end;
    int in_upto(int n) const { return n <= 0 ? 0 : in_end[n - 1]; }
    int pm_upto(int n) const { return n <= 0 ? 0 : pm_end[n - 1]; }
    int launches(int n) const { return (in_upto(n) > 0) + (pm_upto(n) > 0) * (1 + vu); }
  };
  DevTiles tf, ta;  // forward / adjoint items
  // pm_rows > 0: PML items are cut into items of pm_rows-row tiles (more warps
  // for the heavier PML kernels); 0 keeps them at `rows`
  void build_tiles(int rows, int width, int64_t pitch, TileList& L, int pm_rows = 0) const;
  int ri_pf = 0, ri_pa = 0;  // row tiles of the PML items (0: same as ri_f / ri)
  int upload_tiles(const TileList& L, DevTiles& D, cudaStream_t st);
  int autotune(cudaStream_t st, int64_t pitch, size_t cap_items);
  // step launches over the first na sorted shots (interior and PML kernels)
  int launch_fwd(cudaStream_t st, int mode, int na, int t, int base, int ck);
  int launch_adj(cudaStream_t st, int na, int k, int base);
  std::vector<int> rcv_b_host, rcv_e_host;
  AcConst<T> kc{};
  double dt2d = 0;  // dt^2 in FP64 (source-time gradient)
  // device
  char* pool = nullptr;
  size_t pool_bytes = 0;
  AcShot<T>* d_shots = nullptr;
  CellRef* d_shot_rcvs = nullptr;
  int *d_rcv_b = nullptr, *d_rcv_e = nullptr;
  T *d_traces = nullptr, *d_resid = nullptr;
  double* d_partial = nullptr;
  static constexpr int kMisfitBlocks = 512;
  static constexpr int kRowBlocks = 128;  // CTAs per shot of the per-segment copy kernels
  size_t zero_fwd_off = 0, zero_fwd_len = 0, zero_adj_off = 0, zero_adj_len = 0;
  std::vector<AcShot<T>> hshots;
  cudaStream_t cap = nullptr;
  // second stream for the PML-item launch of a step, which runs beside the
  // interior-item launch (disjoint cells); fork / join through events
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaGraph_t gF = nullptr, gR = nullptr;
  cudaGraphExec_t eF = nullptr, eR = nullptr;
  int64_t nF = 0, nR = 0;  // kernel launches in each loop
  // Timing events (recorded inside the loops / graphs): [0,1] the forward
  // loop, [2,3] one full segment's recompute launches, [4,5] its adjoint
  // launches; with the launch and interior cell-step counts of each range.
  cudaEvent_t ev[6] = {};
  int seg_timed = -1;
  bool timing_run = false;  // set only for profile(): direct launches, events recorded
  double tcount[6] = {};  // launches, cell-steps for fwd / recompute / adjoint
  // time-blocked forward (FP32): steps per block, tile rows, tile lists
  int KB = 1, RB = 32;
  // time-blocked tiles: items, their sources (halo KB), receiver rows and maps
  struct TbLists {
    std::vector<TbItem> items;
    std::vector<TbSrc> srcs;
    std::vector<TbRcvRow> rows;
    std::vector<int> map, shot_end;
  };
  void build_tb(int kb, int rb, const ads_acoustic_shot* shots, TbLists& L) const;
  int upload_tb(const TbLists& L, cudaStream_t st);
  int tb_rows_for(int kb) const;  // rows of a time-blocked tile for kb steps per launch
  // autotune may pick steps_per_block in {1, 2, 4} (FP32, variant W, no
  // resident segments): the candidate lists and the device capacity they need
  bool tb_auto = false;
  std::vector<std::pair<int, TbLists>> tb_cand;
  int64_t tb_cells = 0;  // interior cells of all shots (tile sizing)
  std::vector<int> tb_shot_end;  // per sorted shot: TB items of shots [0..s]
  TbItem* d_tb_items = nullptr;
  TbSrc* d_tb_srcs = nullptr;
  TbRcvRow* d_tb_rows = nullptr;
  int* d_tb_map = nullptr;
  int tb_items_upto(int n) const { return n <= 0 ? 0 : tb_shot_end[n - 1]; }
  int launch_tb(cudaStream_t st, bool seg, int nit, int t0, int NS, int base, int in_set,
                int ck);

  ~AcPlan() override {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (eF) cudaGraphExecDestroy(eF);
    if (eR) cudaGraphExecDestroy(eR);
    if (gF) cudaGraphDestroy(gF);
    if (gR) cudaGraphDestroy(gR);
    if (cap) cudaStreamDestroy(cap);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    if (pool) cudaFree(pool);
  }

  std::vector<int64_t> cells_prefix;  // interior cells of the first n sorted shots
  int64_t cells_upto(int n) const { return n <= 0 ? 0 : cells_prefix[n - 1]; }
  int profile(const double* vp, const void* obs, double* out, cudaStream_t st) override;
  int set_source_values(int64_t shot, const double* srcv, cudaStream_t st) override {
    ADS_REQUIRE(shot >= 0 && shot < nshots, "shot %lld out of range [0, %d)", (long long)shot,
                nshots);
    ADS_REQUIRE(srcv || srcv_n[shot] == 0, "null srcv");
    return cast_scaled(srcv_dev[shot], srcv, srcv_n[shot], cfg.dt * cfg.dt, st);
  }
  // number of sorted shots with nstep >= t
  int shots_with_nstep_ge(int t) const {
    int n = 0;
    while (n < nshots && nstep[n] >= t) n++;
    return n;
  }

  int create(const ads_acoustic_config& c, const ads_acoustic_shot* shots, int64_t ns,
             cudaStream_t st);
  int issue_forward(cudaStream_t st, int64_t* count);
  int issue_reverse(cudaStream_t st, int64_t* count);
  int run_loop(int which, cudaStream_t st);
  int forward(const double* vp, void* traces, cudaStream_t st) override;
  int gradient(const double* vp, const void* obs, double* loss, double* grad,
               void* traces_out, cudaStream_t st, double* grad_srcv) override;
};

template <typename T>
int AcPlan<T>::create(const ads_acoustic_config& c, const ads_acoustic_shot* shots,
                      int64_t ns, cudaStream_t st) {
  cfg = c;
  nshots = (int)ns;
  const int64_t MY = c.MY;
  // ---- validation
  ADS_REQUIRE(ns >= 1 && ns < (1 << 20), "nshots must be in [1, 2^20)");
  ADS_REQUIRE(c.MX >= 1 && c.MY >= 1 && c.MY < (1 << 24) && c.MX < (1 << 24),
              "model size out of range");
  ADS_REQUIRE(c.dx > 0 && c.dy > 0 && c.dt > 0 && std::isfinite(c.dx) && std::isfinite(c.dy) &&
                  std::isfinite(c.dt) && std::isfinite(c.vp_ref),
              "dx, dy, dt must be positive and finite (and vp_ref finite)");
  ADS_REQUIRE(c.npml >= 1 && c.Rcoef > 0 && c.Rcoef < 1, "invalid PML parameters");
  ADS_REQUIRE(c.variant == ADS_VARIANT_W || c.variant == ADS_VARIANT_U,
              "variant must be ADS_VARIANT_W or ADS_VARIANT_U");
  vu = c.variant == ADS_VARIANT_U;
  ADS_REQUIRE(c.ckpt_every >= 0 && c.rows_per_thread >= 0, "negative tuning parameter");
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[s];
    ADS_REQUIRE(h.nx >= 1 && h.x0 >= 0 && h.x0 + h.nx + 2 <= c.MX + 2,
                "shot %d: window [x0=%lld, x0+nx+2=%lld) outside the model (MX+2=%lld)", s,
                (long long)h.x0, (long long)(h.x0 + h.nx + 2), (long long)(c.MX + 2));
    ADS_REQUIRE(h.nstep >= 2 && h.nstep < (1 << 24), "shot %d: nstep must be >= 2", s);
    // the interior kernels index a field with 32-bit offsets
    ADS_REQUIRE((h.nx + 2) * grid_pitch(c.MY) < (int64_t(1) << 31),
                "shot %d: a field of (nx + 2) x pitch elements must stay below 2^31", s);
    ADS_REQUIRE(h.nsrc >= 0 && h.nrcv >= 0, "shot %d: negative counts", s);
    ADS_REQUIRE(h.nsrc == 0 || (h.srci && h.srcj && h.srcv), "shot %d: null source arrays",
                s);
    ADS_REQUIRE(h.nrcv == 0 || (h.rcvi && h.rcvj), "shot %d: null receiver arrays", s);
    ADS_REQUIRE(h.nsrc == 0 || h.srcv_rows >= h.nstep,
                "shot %d: srcv has %lld rows, need >= nstep = %lld", s,
                (long long)h.srcv_rows, (long long)h.nstep);
    for (int64_t k = 0; k < h.nsrc; k++)
      ADS_REQUIRE(h.srci[k] >= 2 && h.srci[k] <= h.nx + 1 && h.srcj[k] >= 2 &&
                      h.srcj[k] <= MY + 1,
                  "shot %d source %lld at (%lld, %lld) is not an interior cell of the "
                  "padded window (frame sources are not supported)",
                  s, (long long)k, (long long)h.srci[k], (long long)h.srcj[k]);
    for (int64_t k = 0; k < h.nrcv; k++)
      ADS_REQUIRE(h.rcvi[k] >= 1 && h.rcvi[k] <= h.nx + 2 && h.rcvj[k] >= 1 &&
                      h.rcvj[k] <= MY + 2,
                  "shot %d receiver %lld at (%lld, %lld) is outside the padded window", s,
                  (long long)k, (long long)h.rcvi[k], (long long)h.rcvj[k]);
  }
  // ---- constants (double on the host, rounded once to T)
  const double dt = c.dt, hx = c.dx, hy = c.dy;
  kc.dt = (T)dt;
  kc.hdt = (T)(dt / 2);
  kc.dt2 = (T)(dt * dt);
  dt2d = dt * dt;
  kc.cx = (T)((dt / hx) * (dt / hx));
  kc.cy = (T)((dt / hy) * (dt / hy));
  kc.kxy = (T)(2 * dt * dt / hx / hx + 2 * dt * dt / hy / hy);
  kc.fx = (T)(dt * dt / (2.0 * hx));
  kc.fy = (T)(dt * dt / (2.0 * hy));
  kc.ex = (T)(dt / 2.0 / hx);
  kc.ey = (T)(dt / 2.0 / hy);
  // ---- shot order: record length descending (active shots form a prefix)
  order.resize(ns);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return shots[a].nstep > shots[b].nstep; });
  nstep.resize(ns);
  nxs.resize(ns);
  for (int s = 0; s < ns; s++) nxs[s] = (int)shots[order[s]].nx;
  int max_nstep = 0;
  for (int s = 0; s < ns; s++) {
    nstep[s] = (int)shots[order[s]].nstep;
    max_nstep = std::max(max_nstep, nstep[s]);
  }
  // ---- checkpoint spacing
  if (c.ckpt_every > 0) {
    K = (int)std::min<int64_t>(c.ckpt_every, max_nstep);
  } else {
    K = 100;
    if (max_nstep < 400) K = std::max(1, (int)std::ceil(std::sqrt((double)max_nstep) * 2));
  }
  K = std::max(K, 1);
  // ---- tiling (rows per thread): enough CTAs to fill 152 SMs several times
  int64_t cells = 0;
  for (int s = 0; s < ns; s++) cells += shots[s].nx * MY;
  if (c.rows_per_thread > 0) {
    ri = c.rows_per_thread;
  } else {
    ri = 16;
    while (ri > 2 && cells / ((int64_t)ri * Tile<T>::J) < 152 * 8) ri /= 2;
  }
  // ---- time blocking of the forward steps (FP32 plans)
  KB = sizeof(T) == 4 ? (c.steps_per_block > 0 ? c.steps_per_block : 1) : 1;
  ADS_REQUIRE(c.steps_per_block >= 0 && (KB == 1 || KB == 2 || KB == 4 || KB == 8),
              "steps_per_block must be 0 (automatic), 1, 2, 4 or 8");
  ADS_REQUIRE(sizeof(T) == 4 || c.steps_per_block <= 1,
              "time blocking is implemented for FP32 plans (steps_per_block 0 or 1 for FP64)");
  ADS_REQUIRE(!vu || KB == 1,
              "time blocking is implemented for variant W (steps_per_block 0 or 1 for U)");
  tb_cells = cells;
  RB = tb_rows_for(KB);
  // steps per launch are tuned only on request (autotune 2): the time-blocked
  // kernel keeps the three-level form, whose FP32 rounding error is larger
  tb_auto = sizeof(T) == 4 && c.autotune >= 2 && c.steps_per_block == 0 && !vu;
  inc = sizeof(T) == 4 && KB == 1;
  // ---- trace layout (packed in the caller's shot order)
  trace_off.resize(ns);
  trace_total = 0;
  src_off.resize(ns);
  src_total = 0;
  for (int s = 0; s < ns; s++) {
    trace_off[s] = trace_total;
    trace_total += (shots[s].nstep + 1) * shots[s].nrcv;
    src_off[s] = src_total;
    src_total += shots[s].nstep * shots[s].nsrc;
  }
  // ---- memory layout
  const int64_t pitch = grid_pitch(MY);
  size_t off_fwd_begin, off_fwd_end, off_adj_begin, off_adj_end;
  DevPool L;
  struct Offs {
    size_t u, u2, d, p, q, seg, ckpt, lu, lp, lq, c, rdt, sx, ty, gc, gc32, gsrc, srcv, slist;
  };
  std::vector<Offs> offs(ns);
  std::vector<int> nseg(ns);
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[order[s]];
    nseg[s] = (int)div_up(h.nstep - 1, K);
    nseg_max = std::max(nseg_max, nseg[s]);
  }
  off_fwd_begin = L.used;
  for (int s = 0; s < ns; s++) {
    const int64_t fs = (shots[order[s]].nx + 2) * pitch * (int64_t)sizeof(T);
    offs[s].u = L.take(2 * fs);
    offs[s].u2 = L.take(KB > 1 || tb_auto ? 2 * fs : 0);
    offs[s].d = L.take(sizeof(T) == 4 ? fs : 0);
    offs[s].p = L.take(2 * fs);
    offs[s].q = L.take(2 * fs);
  }
  const size_t traces_off = L.take(sizeof(T) * std::max<int64_t>(trace_total, 1));
  off_fwd_end = L.used;
  off_adj_begin = L.used;
  for (int s = 0; s < ns; s++) {
    const int64_t fs = (shots[order[s]].nx + 2) * pitch * (int64_t)sizeof(T);
    offs[s].lu = L.take(2 * fs);
    offs[s].lp = L.take(2 * fs);
    offs[s].lq = L.take(2 * fs);
    offs[s].gc = L.take((shots[order[s]].nx + 2) * pitch * sizeof(double));
    offs[s].gc32 = L.take(sizeof(T) == 4 ? (shots[order[s]].nx + 2) * pitch * sizeof(float) : 0);
    offs[s].gsrc = L.take(sizeof(double) * std::max<int64_t>(shots[order[s]].nstep *
                                                             shots[order[s]].nsrc, 1));
  }
  off_adj_end = L.used;
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[order[s]];
    const int64_t fs = (h.nx + 2) * pitch * (int64_t)sizeof(T);
    offs[s].ckpt = L.take((size_t)nseg[s] * 4 * fs);
    offs[s].c = L.take(fs);
    offs[s].rdt = L.take(sizeof(T) == 8 ? fs : 0);  // FP64 corner warps' 1/den
    offs[s].sx = L.take((1 + KT_N) * sizeof(T) * (h.nx + 2));  // sigma, its tables
    offs[s].ty = L.take((1 + KT_N) * sizeof(T) * (MY + 2));    // tau, its tables
    offs[s].srcv = L.take(sizeof(T) * std::max<int64_t>(h.nstep * h.nsrc, 1));
    offs[s].slist = L.take(sizeof(CellRef) * std::max<int64_t>(h.nsrc, 1));
  }
  const size_t resid_off = L.take(sizeof(T) * std::max<int64_t>(trace_total, 1));
  const size_t partial_off = L.take(sizeof(double) * kMisfitBlocks);
  // interior sources / receivers per sorted shot, and each shot's receiver list
  std::vector<CellRef> shot_rcvs;
  rcv_b_host.resize(ns);
  rcv_e_host.resize(ns);
  hsrc.assign(ns, {});
  hrcv.assign(ns, {});
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[order[s]];
    const int nx = (int)h.nx, ny = (int)MY;
    for (int64_t k = 0; k < h.nsrc; k++)
      hsrc[s].push_back(make_int3((int)h.srci[k] - 1, (int)h.srcj[k] - 1, (int)k));
    rcv_b_host[s] = (int)shot_rcvs.size();
    for (int64_t r = 0; r < h.nrcv; r++) {
      const int i = (int)h.rcvi[r] - 1, j = (int)h.rcvj[r] - 1;
      if (i < 1 || i > nx || j < 1 || j > ny) continue;  // frame: trace stays 0
      hrcv[s].push_back(make_int3(i, j, (int)r));
      shot_rcvs.push_back({(int64_t)i * pitch + j + JOFF, (int)r, i});
    }
    rcv_e_host[s] = (int)shot_rcvs.size();
  }
  // host copies of the PML profiles (the kernels' interior / PML split uses them)
  hsx.assign(ns, {});
  hty.assign(MY + 2, 0.0);
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[order[s]];
    hsx[s].assign(h.nx + 2, 0.0);
    acoustic_pml_1d(h.nx, MY, c.dx, c.dy, c.npml, c.vp_ref, c.Rcoef, c.use_pml,
                    hsx[s].data(), hty.data());
  }
  // forward and adjoint warp items (rows per thread chosen separately; the
  // autotuner may replace both once the plan's buffers exist): enough warps
  // for several resident waves
  if (c.rows_per_thread <= 0) {
    ri_f = 8;
    // FP64 items go down to one row per warp: on small grids a warp's serial
    // chain of FP64 operations, not the item count, sets a step's duration
    const int rmin = sizeof(T) == 8 ? 1 : 2;
    while (ri_f > rmin && cells / ((int64_t)ri_f * Tile<T>::WF) < 152 * 64) ri_f /= 2;
    ri = 16;
    while (ri > rmin && cells / ((int64_t)ri * Tile<T>::WA) < 152 * 32) ri /= 2;
  } else {
    ri_f = ri;
  }
  TileList tiles_a, tiles_f;
  build_tiles(ri, Tile<T>::WA, pitch, tiles_a);
  build_tiles(ri_f, Tile<T>::WF, pitch, tiles_f);
  auto nitems_of = [](const TileList& L) { return L.in.size() + L.pm.size(); };
  // capacity: the autotuner tries rows down to 2 per thread
  size_t cap_items = std::max(nitems_of(tiles_a), nitems_of(tiles_f));
  size_t cap_refs = std::max({tiles_a.srcs.size(), tiles_f.srcs.size(), tiles_a.rcvs.size(),
                              tiles_f.rcvs.size(), (size_t)1});
  if (c.autotune) {
    size_t n2 = 0;
    for (int s = 0; s < ns; s++)
      n2 += (size_t)div_up(shots[order[s]].nx, 2) *
            (size_t)div_up(MY, std::min(Tile<T>::WF, Tile<T>::WA));
    cap_items = std::max(cap_items, n2);
  }
  // time-blocked tiles (build_tb) for the configured steps per launch and, when
  // the autotuner may choose them, for 2 and 4; the device lists get the
  // capacity of the largest
  TbLists tbl;
  std::vector<int> rcv_next_all;
  std::vector<int> rcv_next_off(ns, 0);
  tb_shot_end.assign(ns, 0);
  if (KB > 1) build_tb(KB, RB, shots, tbl);
  if (tb_auto)
    for (int kb : {2, 4}) {
      tb_cand.emplace_back(kb, TbLists{});
      build_tb(kb, tb_rows_for(kb), shots, tb_cand.back().second);
    }
  if (KB > 1 || tb_auto)
    for (int s = 0; s < ns; s++) {  // chain receivers sharing a cell
      const ads_acoustic_shot& h = shots[order[s]];
      rcv_next_off[s] = (int)rcv_next_all.size();
      std::vector<int> next(h.nrcv, -1);
      for (int64_t r = 0; r < h.nrcv; r++)
        for (int64_t q = r + 1; q < h.nrcv; q++)
          if (h.rcvi[q] == h.rcvi[r] && h.rcvj[q] == h.rcvj[r]) {
            next[r] = (int)q;
            break;
          }
      rcv_next_all.insert(rcv_next_all.end(), next.begin(), next.end());
    }
  size_t cap_tbi = tbl.items.size(), cap_tbs = tbl.srcs.size(), cap_tbr = tbl.rows.size(),
         cap_tbm = tbl.map.size();
  for (const auto& cl : tb_cand) {
    cap_tbi = std::max(cap_tbi, cl.second.items.size());
    cap_tbs = std::max(cap_tbs, cl.second.srcs.size());
    cap_tbr = std::max(cap_tbr, cl.second.rows.size());
    cap_tbm = std::max(cap_tbm, cl.second.map.size());
  }
  const size_t tbi_off = L.take(sizeof(TbItem) * std::max<size_t>(cap_tbi, 1));
  const size_t tbs_off = L.take(sizeof(TbSrc) * std::max<size_t>(cap_tbs, 1));
  const size_t tbr_off = L.take(sizeof(TbRcvRow) * std::max<size_t>(cap_tbr, 1));
  const size_t tbm_off = L.take(sizeof(int) * std::max<size_t>(cap_tbm, 1));
  const size_t rnx_off = L.take(sizeof(int) * std::max<size_t>(rcv_next_all.size(), 1));
  const size_t shots_off = L.take(sizeof(AcShot<T>) * ns);
  // (sources / receivers: each is bucketed into exactly one item of a list)
  const size_t items_off = L.take(sizeof(AcItem) * cap_items);
  const size_t srcs_off = L.take(sizeof(CellRef) * cap_refs);
  const size_t rcvs_off = L.take(sizeof(CellRef) * cap_refs);
  const size_t itemsf_off = L.take(sizeof(AcItem) * cap_items);
  const size_t srcsf_off = L.take(sizeof(CellRef) * cap_refs);
  const size_t rcvsf_off = L.take(sizeof(CellRef) * cap_refs);
  const size_t shot_rcvs_off = L.take(sizeof(CellRef) * std::max<size_t>(shot_rcvs.size(), 1));
  const size_t rcvb_off = L.take(sizeof(int) * ns);
  const size_t rcve_off = L.take(sizeof(int) * ns);
  // ---- the shots' stores: K + 2 slots for a segment's recompute, then the
  // slots of the resident segments (the last ones whose wavefields fit in
  // the allowed share of the free device memory)
  res_seg = nseg_max;
  {
    std::vector<size_t> fsb(ns);
    size_t base_bytes = L.used;
    for (int q = 0; q < ns; q++) {
      fsb[q] = (size_t)(shots[order[q]].nx + 2) * pitch * sizeof(T);
      base_bytes += (K + 2) * fsb[q] + 256;
    }
    if (KB == 1 && c.resident_segments >= 0 && nseg_max > 0) {
      size_t fr = 0, tot = 0, avail = 0;
      if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr > base_bytes) {
        const int pct = c.resident_mem_pct > 0 ? std::min<int>(c.resident_mem_pct, 95) : 50;
        avail = (size_t)((double)(fr - base_bytes) * pct / 100.0);
      } else {
        cudaGetLastError();
      }
      const int lo = c.resident_segments > 0 ? std::max(0, nseg_max - c.resident_segments) : 0;
      for (int sg = nseg_max - 1; sg >= lo; sg--) {
        const int a = 2 + sg * K;
        size_t b = 0;
        for (int q = 0; q < ns; q++)
          if (nstep[q] >= a) b += (size_t)(nstep[q] - (a - 2) + 1) * fsb[q] + 256;
        if (b > avail) break;
        res_seg = sg;
      }
    }
    res_base = res_seg * K - (K + 2);  // slot K + 2 holds u_{a-2} of segment res_seg
    for (int q = 0; q < ns; q++) {
      const int a = 2 + res_seg * K;
      const size_t slots =
          (size_t)(K + 2) + (res_seg < nseg_max && nstep[q] >= a ? nstep[q] - (a - 2) + 1 : 0);
      offs[q].seg = L.take(slots * fsb[q]);
      seg_slots.push_back(slots);
    }
  }
  const size_t maps_off = L.take(sizeof(AcTmaMaps) * ns);
  const size_t err_off = L.take(sizeof(int));
  pool_bytes = L.used;
  bytes = (int64_t)pool_bytes;
  resident = nseg_max - res_seg;
  // resident segments skip the recompute, which saves more than time blocking
  // gains; the time-blocked kernel has no resident-store mode, so the
  // autotuner considers it only for plans without them
  if (resident > 0) {
    tb_auto = false;
    tb_cand.clear();
  }
  {
    cudaError_t e = cudaMalloc(&pool, pool_bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      pool = nullptr;
      return fail(ADS_ERR_NOMEM, "device allocation of %.3f GB for the plan failed: %s",
                  pool_bytes / 1e9, cudaGetErrorString(e));
    }
  }
  ADS_CUDA(cudaMemsetAsync(pool, 0, pool_bytes, st));
  zero_fwd_off = off_fwd_begin;
  zero_fwd_len = off_fwd_end - off_fwd_begin;
  zero_adj_off = off_adj_begin;
  zero_adj_len = off_adj_end - off_adj_begin;
  d_traces = (T*)(pool + traces_off);
  d_resid = (T*)(pool + resid_off);
  d_partial = (double*)(pool + partial_off);
  d_shots = (AcShot<T>*)(pool + shots_off);
  ta.items = (AcItem*)(pool + items_off);
  ta.srcs = (CellRef*)(pool + srcs_off);
  ta.rcvs = (CellRef*)(pool + rcvs_off);
  tf.items = (AcItem*)(pool + itemsf_off);
  tf.srcs = (CellRef*)(pool + srcsf_off);
  tf.rcvs = (CellRef*)(pool + rcvsf_off);
  d_shot_rcvs = (CellRef*)(pool + shot_rcvs_off);
  d_rcv_b = (int*)(pool + rcvb_off);
  d_rcv_e = (int*)(pool + rcve_off);
  d_tb_items = (TbItem*)(pool + tbi_off);
  d_tb_srcs = (TbSrc*)(pool + tbs_off);
  d_tb_rows = (TbRcvRow*)(pool + tbr_off);
  d_tb_map = (int*)(pool + tbm_off);
  d_maps = (AcTmaMaps*)(pool + maps_off);
  d_err = (int*)(pool + err_off);
  // per-shot structs and host-side data (profiles, scaled wavelets)
  hshots.resize(ns);
  srcv_dev.assign(ns, nullptr);
  srcv_n.assign(ns, 0);
  std::vector<double> sx, ty;
  std::vector<std::vector<T>> host_bufs;
  // trace offsets in sorted order
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[order[s]];
    AcShot<T>& d = hshots[s];
    d.nx = (int)h.nx;
    d.ny = (int)MY;
    d.nstep = (int)h.nstep;
    d.x0 = (int)h.x0;
    d.pitch = pitch;
    d.fs = (h.nx + 2) * pitch;
    d.nsrc = (int)h.nsrc;
    d.nrcv = (int)h.nrcv;
    d.nseg = nseg[s];
    d.u = (T*)(pool + offs[s].u);
    d.u2 = (T*)(pool + offs[s].u2);
    d.d = sizeof(T) == 4 ? (T*)(pool + offs[s].d) : nullptr;
    d.rcv_next = (const int*)(pool + rnx_off) + rcv_next_off[s];
    d.p = (T*)(pool + offs[s].p);
    d.q = (T*)(pool + offs[s].q);
    d.seg = (T*)(pool + offs[s].seg);
    d.ckpt = (T*)(pool + offs[s].ckpt);
    d.lu = (T*)(pool + offs[s].lu);
    d.lp = (T*)(pool + offs[s].lp);
    d.lq = (T*)(pool + offs[s].lq);
    d.c = (T*)(pool + offs[s].c);
    d.rdt = sizeof(T) == 8 ? (T*)(pool + offs[s].rdt) : nullptr;
    d.sx = (T*)(pool + offs[s].sx);
    d.ty = (T*)(pool + offs[s].ty);
    d.sxk = d.sx + (h.nx + 2);
    d.tyk = d.ty + (MY + 2);
    d.gc = (double*)(pool + offs[s].gc);
    d.gc32 = sizeof(T) == 4 ? (float*)(pool + offs[s].gc32) : nullptr;
    d.gsrc = (double*)(pool + offs[s].gsrc);
    d.src_list = (const CellRef*)(pool + offs[s].slist);
    if (h.nsrc > 0) {
      std::vector<CellRef> sl(h.nsrc);
      for (int64_t k = 0; k < h.nsrc; k++) {
        const int i = (int)h.srci[k] - 1, jj = (int)h.srcj[k] - 1;
        sl[k] = {(int64_t)i * pitch + jj + JOFF, (int)k, i};
      }
      std::vector<T> bytes_((sizeof(CellRef) * sl.size() + sizeof(T) - 1) / sizeof(T));
      std::memcpy(bytes_.data(), sl.data(), sizeof(CellRef) * sl.size());
      host_bufs.emplace_back(std::move(bytes_));
      ADS_CUDA(cudaMemcpyAsync((void*)d.src_list, host_bufs.back().data(),
                               sizeof(CellRef) * sl.size(), cudaMemcpyHostToDevice, st));
    }
    d.srcv = (const T*)(pool + offs[s].srcv);
    srcv_dev[order[s]] = (T*)d.srcv;
    srcv_n[order[s]] = h.nstep * h.nsrc;
    d.traces = d_traces + trace_off[order[s]];
    d.resid = d_resid + trace_off[order[s]];
    sx = hsx[s];
    ty = hty;
    host_bufs.emplace_back(with_tables<T>(sx, c.dt, c.dx, c.dy));
    ADS_CUDA(cudaMemcpyAsync(d.sx, host_bufs.back().data(), sizeof(T) * (1 + KT_N) * sx.size(),
                             cudaMemcpyHostToDevice, st));
    host_bufs.emplace_back(with_tables<T>(ty, c.dt, c.dx, c.dy));
    ADS_CUDA(cudaMemcpyAsync(d.ty, host_bufs.back().data(), sizeof(T) * (1 + KT_N) * ty.size(),
                             cudaMemcpyHostToDevice, st));
    if (h.nsrc > 0) {
      std::vector<T> sv((size_t)(h.nstep * h.nsrc));
      const double dt2 = c.dt * c.dt;
      for (int64_t r = 0; r < h.nstep; r++)
        for (int64_t k = 0; k < h.nsrc; k++)
          sv[r * h.nsrc + k] = (T)(h.srcv[r * h.nsrc + k] * dt2);
      host_bufs.emplace_back(std::move(sv));
      ADS_CUDA(cudaMemcpyAsync((void*)d.srcv, host_bufs.back().data(),
                               sizeof(T) * host_bufs.back().size(), cudaMemcpyHostToDevice,
                               st));
    }
  }
  ADS_CUDA(cudaMemcpyAsync(d_shots, hshots.data(), sizeof(AcShot<T>) * ns,
                           cudaMemcpyHostToDevice, st));
  if constexpr (sizeof(T) == 8) {
    k_ac_rden<T><<<dim3(kRowBlocks, ns), 256, 0, st>>>(d_shots, c.dt / 2);
    ADS_LAUNCHED(1);
  }
  if (int e = upload_tiles(tiles_a, ta, st)) return e;
  if (int e = upload_tiles(tiles_f, tf, st)) return e;
  if (!shot_rcvs.empty())
    ADS_CUDA(cudaMemcpyAsync(d_shot_rcvs, shot_rcvs.data(), sizeof(CellRef) * shot_rcvs.size(),
                             cudaMemcpyHostToDevice, st));
  ADS_CUDA(cudaMemcpyAsync(d_rcv_b, rcv_b_host.data(), sizeof(int) * ns,
                           cudaMemcpyHostToDevice, st));
  ADS_CUDA(cudaMemcpyAsync(d_rcv_e, rcv_e_host.data(), sizeof(int) * ns,
                           cudaMemcpyHostToDevice, st));
  auto up = [&](void* dst, const void* src, size_t n) -> int {
    if (n) ADS_CUDA(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, st));
    return ADS_OK;
  };
  if (KB > 1)
    if (int e = upload_tb(tbl, st)) return e;
  if (int e = up(pool + rnx_off, rcv_next_all.data(), sizeof(int) * rcv_next_all.size()))
    return e;
  ADS_CUDA(cudaStreamSynchronize(st));  // host staging buffers go out of scope
  if (sizeof(T) == 4 && c.tma > 0)
    if (int e = build_maps(st)) return e;
  ADS_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  ADS_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
  ADS_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
  // ---- autotuner: time candidate tilings on the plan's own buffers
  if (c.autotune)
    if (int e = autotune(st, pitch, cap_items)) return e;
  inc = sizeof(T) == 4 && KB == 1;
  // ---- timing ranges: the first full-length segment the reverse sweep meets
  cells_prefix.resize(ns);
  for (int s = 0; s < ns; s++)
    cells_prefix[s] = (s ? cells_prefix[s - 1] : 0) + (int64_t)shots[order[s]].nx * MY;
  // profile() times the recompute and adjoint of the last recomputed segment
  // (or, when every segment is resident, an adjoint-only segment)
  seg_timed = res_seg >= 1 ? res_seg - 1 : (nseg_max >= 2 ? nseg_max - 2 : 0);
  for (auto& e : ev) ADS_CUDA(cudaEventCreate(&e));
  // ---- launch counts
  {
    int64_t n = 0;
    issue_forward(nullptr, &n);
    nF = n;
    n = 0;
    issue_reverse(nullptr, &n);
    nR = n;
  }
  steps_per_block = KB;
  rows[0] = ri_f;
  rows[1] = ri;
  rows[2] = ri_pf > 0 ? ri_pf : ri_f;
  rows[3] = ri_pa > 0 ? ri_pa : ri;
  launches_fwd = 1 + nF;            // prep + loop
  launches_grad = 1 + nF + 2 + nR + 1;  // prep, loop, misfit+reduce, reverse, assemble
  // ---- graphs
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
      if (which == 0) {
        gF = g;
        eF = ex;
      } else {
        gR = g;
        eR = ex;
      }
    }
  }
  return ADS_OK;
}

// Rows of a time-blocked tile: the configured block_rows, else 32 halved
// until the tiles of kb steps per launch fill the SMs about four times over.
template <typename T>
int AcPlan<T>::tb_rows_for(int kb) const {
  if (cfg.block_rows > 0) return (int)cfg.block_rows;
  int rb = 32;
  const int64_t colw = TB_THREADS - 2 * kb;
  while (rb > 4 && tb_cells / ((int64_t)rb * colw) < 152 * 4) rb /= 2;
  return rb;
}

// Time-blocked tiles for kb steps per launch: output columns [jo, jo + W),
// W = TB_THREADS - 2 kb, rows [i0, i0 + rb); the sources of the loaded region
// (halo kb); receiver maps of the output region.
template <typename T>
void AcPlan<T>::build_tb(int kb, int rb, const ads_acoustic_shot* shots, TbLists& L) const {
  L = TbLists{};
  L.shot_end.assign(nshots, 0);
  const int W = TB_THREADS - 2 * kb;
  const int ny = (int)cfg.MY;
  for (int s = 0; s < nshots; s++) {
    const ads_acoustic_shot& h = shots[order[s]];
    const int nx = (int)h.nx;
    for (int i0 = 1; i0 <= nx; i0 += rb) {
      const int i1 = std::min(i0 + rb, nx + 1);
      for (int jo = 1; jo <= ny; jo += W) {
        TbItem it{};
        it.shot = s;
        it.i0 = i0;
        it.jo = jo;
        it.src_b = (int)L.srcs.size();
        for (int64_t k = 0; k < h.nsrc; k++) {
          const int i = (int)h.srci[k] - 1, j = (int)h.srcj[k] - 1;
          if (i >= i0 - kb && i < i1 + kb && j >= jo - kb && j < jo - kb + TB_THREADS)
            L.srcs.push_back({i, j, (int)k, 0});
        }
        it.src_e = (int)L.srcs.size();
        it.rr_b = (int)L.rows.size();
        for (int i = i0; i < i1; i++) {
          int off = -1;
          for (int64_t r = 0; r < h.nrcv; r++) {
            const int ri_ = (int)h.rcvi[r] - 1, rj = (int)h.rcvj[r] - 1;
            if (ri_ != i || rj < jo || rj >= jo + W || rj < 1 || rj > ny) continue;
            bool first = true;  // only the first receiver of a cell enters the map
            for (int64_t q = 0; q < r; q++)
              if (h.rcvi[q] == h.rcvi[r] && h.rcvj[q] == h.rcvj[r]) first = false;
            if (!first) continue;
            if (off < 0) {
              off = (int)L.map.size();
              L.map.insert(L.map.end(), TB_THREADS, -1);
              L.rows.push_back({i, off});
            }
            L.map[off + (rj - jo + kb)] = (int)r;
          }
        }
        it.rr_e = (int)L.rows.size();
        L.items.push_back(it);
      }
    }
    L.shot_end[s] = (int)L.items.size();
  }
}

template <typename T>
int AcPlan<T>::upload_tb(const TbLists& L, cudaStream_t st) {
  auto up = [&](void* dst, const void* src, size_t n) -> int {
    if (n) ADS_CUDA(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, st));
    return ADS_OK;
  };
  if (int e = up(d_tb_items, L.items.data(), sizeof(TbItem) * L.items.size())) return e;
  if (int e = up(d_tb_srcs, L.srcs.data(), sizeof(TbSrc) * L.srcs.size())) return e;
  if (int e = up(d_tb_rows, L.rows.data(), sizeof(TbRcvRow) * L.rows.size())) return e;
  if (int e = up(d_tb_map, L.map.data(), sizeof(int) * L.map.size())) return e;
  tb_shot_end = L.shot_end;
  // the host lists of a candidate stay alive until the copies are done
  ADS_CUDA(cudaStreamSynchronize(st));
  return ADS_OK;
}

// Forward time loop (zero the rings and traces, then one launch per step).
// count != nullptr: only count kernel launches.
// Tiles of `rows` rows x Tile::J columns over every sorted shot, with the
// sources and receivers of each tile (bucketed once per shot).
template <typename T>
void AcPlan<T>::build_tiles(int rows, int width, int64_t pitch, TileList& L,
                            int pm_rows) const {
  L.in.clear();
  L.pm.clear();
  L.srcs.clear();
  L.rcvs.clear();
  L.in_end.assign(nshots, 0);
  L.pm_end.assign(nshots, 0);
  std::vector<int> pm_cost;  // per PML item, for the ordering below
  const int ny = (int)cfg.MY;
  const int gh = Tile<T>::G * rows;  // rows of one item (its G warps' row tiles)
  for (int s = 0; s < nshots; s++) {
    const int nx = nxs[s];
    const int nti = (int)div_up(nx, gh), ntj = (int)div_up(ny, width);
    std::vector<std::vector<int>> bs((size_t)nti * ntj), br((size_t)nti * ntj);
    for (size_t k = 0; k < hsrc[s].size(); k++) {
      const int3 q = hsrc[s][k];
      if (!vu) {
        bs[(size_t)((q.x - 1) / gh) * ntj + (q.y - 1) / width].push_back((int)k);
        continue;
      }
      // variant U: the pre-pass and the adjoint read u less its source value
      // one cell beyond the item, so every item whose rows i0-1 .. i_end and
      // columns j0-1 .. j0+width hold the source lists it
      for (int ti = std::max(0, (q.x - 2) / gh); ti <= std::min(nti - 1, q.x / gh); ti++)
        for (int tj = std::max(0, (q.y - 2) / width); tj <= std::min(ntj - 1, q.y / width);
             tj++) {
          const int i0 = 1 + ti * gh, i_end = std::min(i0 + gh, nx + 1);
          const int j0 = 1 + tj * width;
          if (q.x >= i0 - 1 && q.x <= i_end && q.y >= j0 - 1 && q.y <= j0 + width)
            bs[(size_t)ti * ntj + tj].push_back((int)k);
        }
    }
    for (size_t k = 0; k < hrcv[s].size(); k++) {
      const int3 q = hrcv[s][k];
      br[(size_t)((q.x - 1) / gh) * ntj + (q.y - 1) / width].push_back((int)k);
    }
    // tau-free column strips: tau = 0 at columns j0-1 .. j0+width (inside the frame)
    std::vector<char> col_free(ntj), row_free(nti);
    // relative cost of a PML item: per warp 1 where it is free of both
    // profiles, 3 where it meets one, 6 where it meets both (a corner)
    auto item_cost = [&](const AcItem& it, int r, bool cfree) {
      int c = 0;
      for (int w = 0; w < Tile<T>::G; w++) {
        const int a = it.i0 + w * r, e = std::min(a + r, nx + 1);
        if (a > nx) break;
        bool z = true;
        for (int i = a - 1; i <= e; i++) z = z && hsx[s][i] == 0.0;
        c += z && cfree ? 1 : (z || cfree ? 3 : 6);
      }
      return c;
    };
    for (int tj = 0; tj < ntj; tj++) {
      const int j0 = 1 + tj * width;
      bool z = true;
      for (int j = j0 - 1; j <= std::min(j0 + width, ny + 1); j++) z = z && hty[j] == 0.0;
      col_free[tj] = z;
    }
    for (int ti = 0; ti < nti; ti++) {  // sigma = 0 on rows i0-1 .. i_end
      const int i0 = 1 + ti * gh, i_end = std::min(i0 + gh, nx + 1);
      bool z = true;
      for (int i = i0 - 1; i <= i_end; i++) z = z && hsx[s][i] == 0.0;
      row_free[ti] = z;
    }
    for (int ti = 0; ti < nti; ti++)
      for (int tj = 0; tj < ntj; tj++) {
        AcItem it{};
        it.shot = s;
        it.i0 = 1 + ti * gh;
        it.j0 = 1 + tj * width;
        const size_t b = (size_t)ti * ntj + tj;
        it.src_b = (int)L.srcs.size();
        for (int k : bs[b]) {
          const int3 q = hsrc[s][k];
          L.srcs.push_back({(int64_t)q.x * pitch + q.y + JOFF, q.z, q.x});
        }
        it.src_e = (int)L.srcs.size();
        it.rcv_b = (int)L.rcvs.size();
        for (int k : br[b]) {
          const int3 q = hrcv[s][k];
          L.rcvs.push_back({(int64_t)q.x * pitch + q.y + JOFF, q.z, q.x});
        }
        it.rcv_e = (int)L.rcvs.size();
        // interior items carry no sources or receivers: the interior kernels
        // then need neither (items holding one take the general kernel)
        const bool in = row_free[ti] && col_free[tj] && it.src_e == it.src_b &&
                        it.rcv_e == it.rcv_b;
        if (in) {
          L.in.push_back(it);
        } else if (pm_rows > 0 && pm_rows < rows) {
          // sub-items share the item's source / receiver lists: the kernels
          // match those by cell and row
          for (int i0 = it.i0; i0 < it.i0 + gh && i0 <= nx; i0 += Tile<T>::G * pm_rows) {
            AcItem sub = it;
            sub.i0 = i0;
            L.pm.push_back(sub);
            pm_cost.push_back(item_cost(sub, pm_rows, col_free[tj]));
          }
        } else {
          L.pm.push_back(it);
          pm_cost.push_back(item_cost(it, rows, col_free[tj]));
        }
      }
    L.in_end[s] = (int)L.in.size();
    L.pm_end[s] = (int)L.pm.size();
  }
  // Heaviest PML items first.  Their cost varies several-fold (corner warps
  // take the general form, edge warps a cheaper specialised one, warps past the
  // profile the interior update), and the blocks start roughly in index order,
  // so this order lets the launch end on light items.  Items move only within
  // a group of shots of equal record length: a launch always covers whole
  // groups (the shots with nstep >= t), so the prefix counts at group ends stay
  // valid.
  std::vector<int> idx;
  for (int sa = 0; sa < nshots;) {
    int sb = sa + 1;
    while (sb < nshots && nstep[sb] == nstep[sa]) sb++;
    const int b = sa > 0 ? L.pm_end[sa - 1] : 0, e = L.pm_end[sb - 1];
    idx.resize(e - b);
    std::iota(idx.begin(), idx.end(), b);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int x, int y) { return pm_cost[x] > pm_cost[y]; });
    std::vector<AcItem> sorted(e - b);
    for (int k = 0; k < e - b; k++) sorted[k] = L.pm[idx[k]];
    std::copy(sorted.begin(), sorted.end(), L.pm.begin() + b);
    sa = sb;
  }
}

template <typename T>
int AcPlan<T>::upload_tiles(const TileList& L, DevTiles& D, cudaStream_t st) {
  if (!L.in.empty())
    ADS_CUDA(cudaMemcpyAsync(D.items, L.in.data(), sizeof(AcItem) * L.in.size(),
                             cudaMemcpyHostToDevice, st));
  if (!L.pm.empty())
    ADS_CUDA(cudaMemcpyAsync(D.items + L.in.size(), L.pm.data(), sizeof(AcItem) * L.pm.size(),
                             cudaMemcpyHostToDevice, st));
  if (!L.srcs.empty())
    ADS_CUDA(cudaMemcpyAsync(D.srcs, L.srcs.data(), sizeof(CellRef) * L.srcs.size(),
                             cudaMemcpyHostToDevice, st));
  if (!L.rcvs.empty())
    ADS_CUDA(cudaMemcpyAsync(D.rcvs, L.rcvs.data(), sizeof(CellRef) * L.rcvs.size(),
                             cudaMemcpyHostToDevice, st));
  D.pm_off = (int)L.in.size();
  D.vu = vu ? 1 : 0;
  D.in_end = L.in_end;
  D.pm_end = L.pm_end;
  return ADS_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the library
// does not link the driver API); null when the driver has none.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// The tensor maps of every shot (FP32 plans): u's ring and segment store as
// 3D (pitch x rows x slot) with a 72 x 10 x 1 box, d and c as 2D with a
// 64 x 8 box; zero fill outside the field.  Leaves tma_ok false when the
// driver has no encoder.
template <typename T>
int AcPlan<T>::build_maps(cudaStream_t st) {
  tma_ok = false;
  EncodeTiledFn enc = encode_tiled_fn();
  if (!enc) return ADS_OK;
  std::vector<AcTmaMaps> hm(nshots);
  const cuuint32_t es[3] = {1, 1, 1};
  for (int s = 0; s < nshots; s++) {
    const AcShot<T>& h = hshots[s];
    const cuuint64_t rows = (cuuint64_t)h.nx + 2, P = (cuuint64_t)h.pitch;
    const cuuint64_t rs = P * sizeof(T), ss = (cuuint64_t)h.fs * sizeof(T);
    ADS_REQUIRE(rs % 16 == 0 && ss % 16 == 0 && P >= (cuuint64_t)TMA_UW,
                "internal: field layout unfit for tensor maps");
    auto map3 = [&](CUtensorMap* m, void* base, cuuint64_t slots) {
      const cuuint64_t dim[3] = {P, rows, slots}, str[2] = {rs, ss};
      const cuuint32_t box[3] = {(cuuint32_t)TMA_UW, (cuuint32_t)TMA_RB + 2, 1};
      return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dim, str, box, es,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    };
    auto map2 = [&](CUtensorMap* m, void* base) {
      const cuuint64_t dim[2] = {P, rows}, str[1] = {rs};
      const cuuint32_t box[2] = {(cuuint32_t)TMA_W, (cuuint32_t)TMA_RB};
      return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dim, str, box, es,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    };
    if (map3(&hm[s].ring, (void*)h.u, 2) != CUDA_SUCCESS ||
        map3(&hm[s].seg, (void*)h.seg, (cuuint64_t)seg_slots[s]) != CUDA_SUCCESS ||
        map2(&hm[s].d, (void*)h.d) != CUDA_SUCCESS || map2(&hm[s].c, (void*)h.c) != CUDA_SUCCESS)
      return fail(ADS_ERR_CUDA, "cuTensorMapEncodeTiled rejected a field of shot %d", s);
  }
  ADS_CUDA(cudaMemcpyAsync(d_maps, hm.data(), sizeof(AcTmaMaps) * nshots,
                           cudaMemcpyHostToDevice, st));
  ADS_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st));
  ADS_CUDA(cudaStreamSynchronize(st));
  tma_ok = true;
  uses_tma = 1;
  return ADS_OK;
}

// One forward step of the first na sorted shots: the interior-item kernel and
// the PML-item kernel (each launched only when it has items).
template <typename T>
int AcPlan<T>::launch_fwd(cudaStream_t st, int mode, int na, int t, int base, int ck) {
  constexpr int TPB = Tile<T>::TPB;
  const int ni = tf.in_upto(na), np = tf.pm_upto(na);
  const AcItem* pm = tf.items + tf.pm_off;
  const bool fork = ni > 0 && np > 0;
  cudaStream_t sp = st;  // stream of the PML-item launch
  if (fork) {
    ADS_CUDA(cudaEventRecord(ev_fork, st));
    ADS_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
    sp = side;
  }
#define ADS_FWD_(M, IN, VUF, CKF, INCF, items_, n_, s_, rows_)                              \
  k_ac_fwd<T, M, IN, VUF, CKF, INCF><<<n_, TPB, 0, s_>>>(items_, d_shots, tf.srcs, tf.rcvs, kc, \
                                                         t, base, ck, rows_)
#define ADS_FWD(M, IN, VUF, CKF, items_, n_, s_, rows_)                 \
  do {                                                                  \
    if constexpr (sizeof(T) == 4) {                                     \
      if (inc) ADS_FWD_(M, IN, VUF, CKF, true, items_, n_, s_, rows_);  \
      else ADS_FWD_(M, IN, VUF, CKF, false, items_, n_, s_, rows_);     \
    } else {                                                            \
      ADS_FWD_(M, IN, VUF, CKF, false, items_, n_, s_, rows_);          \
    }                                                                   \
  } while (0)
#define ADS_FWD_MODE(IN, VUF, items_, n_, s_, rows_)                        \
  do {                                                                      \
    if (mode == 1) ADS_FWD(1, IN, VUF, false, items_, n_, s_, rows_);      \
    else if (mode == 2) ADS_FWD(2, IN, VUF, false, items_, n_, s_, rows_); \
    else if (IN || ck > 0) ADS_FWD(0, IN, VUF, true, items_, n_, s_, rows_); \
    else ADS_FWD(0, IN, VUF, false, items_, n_, s_, rows_);                \
  } while (0)
  auto run_in = [&]() -> int {
    if (ni > 0) {
      if constexpr (sizeof(T) == 4) {
        if (tma_ok && inc) {
          const int gh = Tile<T>::G * ri_f;
          if (mode == 1)
            k_ac_fwd_tma<1, false><<<ni, TPB, TMA_SMEM, st>>>(tf.items, d_shots, d_maps, kc, t,
                                                              base, ck, gh, d_err);
          else if (mode == 2)
            k_ac_fwd_tma<2, false><<<ni, TPB, TMA_SMEM, st>>>(tf.items, d_shots, d_maps, kc, t,
                                                              base, ck, gh, d_err);
          else if (ck > 0)
            k_ac_fwd_tma<0, true><<<ni, TPB, TMA_SMEM, st>>>(tf.items, d_shots, d_maps, kc, t,
                                                             base, ck, gh, d_err);
          else
            k_ac_fwd_tma<0, false><<<ni, TPB, TMA_SMEM, st>>>(tf.items, d_shots, d_maps, kc, t,
                                                              base, ck, gh, d_err);
        } else {
          ADS_FWD_MODE(true, false, tf.items, ni, st, ri_f);
        }
      } else {
        ADS_FWD_MODE(true, false, tf.items, ni, st, ri_f);
      }
      ADS_LAUNCHED(1);
    }
    return ADS_OK;
  };
  auto run_pm = [&]() -> int {
    if (np > 0) {
      const int rows = ri_pf > 0 ? ri_pf : ri_f;
      if (vu) {
        // phi_{t-1}, psi_{t-1} from u_{t-1}, then the step reads them
        if (mode == 0)
          k_ac_phi_u<T, 0><<<np, TPB, 0, sp>>>(pm, d_shots, tf.srcs, kc, t, base, rows);
        else
          k_ac_phi_u<T, 1><<<np, TPB, 0, sp>>>(pm, d_shots, tf.srcs, kc, t, base, rows);
        ADS_LAUNCHED(1);
        ADS_FWD_MODE(false, true, pm, np, sp, rows);
      } else {
        ADS_FWD_MODE(false, false, pm, np, sp, rows);
      }
      ADS_LAUNCHED(1);
    }
    return ADS_OK;
  };
  // the PML launch first: the launches of a fork start roughly in the order
  // they are issued, and its items are the heavier (FP64 C2: 36.7 against
  // 35.7 shot-gradients/s; FP32 C3 unchanged)
  if (int e = run_pm()) return e;
  if (int e = run_in()) return e;
#undef ADS_FWD_MODE
#undef ADS_FWD
#undef ADS_FWD_
  if (fork) {
    ADS_CUDA(cudaEventRecord(ev_join, side));
    ADS_CUDA(cudaStreamWaitEvent(st, ev_join, 0));
  }
  return ADS_OK;
}

template <typename T>
int AcPlan<T>::launch_adj(cudaStream_t st, int na, int k, int base) {
  constexpr int TPB = Tile<T>::TPB;
  const int ni = ta.in_upto(na), np = ta.pm_upto(na);
  const bool fork = ni > 0 && np > 0;
  cudaStream_t sp = st;
  if (fork) {
    ADS_CUDA(cudaEventRecord(ev_fork, st));
    ADS_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
    sp = side;
  }
  auto run_in = [&]() -> int {
    if (ni > 0) {
      k_ac_adj<T, true><<<ni, TPB, 0, st>>>(ta.items, d_shots, ta.srcs, ta.rcvs, kc, k, base, ri,
                                            dt2d);
      ADS_LAUNCHED(1);
    }
    return ADS_OK;
  };
  auto run_pm = [&]() -> int {
    if (np > 0) {
      const int rows = ri_pa > 0 ? ri_pa : ri;
      if (vu) {
        // lambdaPhi_{k-1}, lambdaPsi_{k-1} first, then the step's transpose
        k_ac_adjphi_u<T><<<np, TPB, 0, sp>>>(ta.items + ta.pm_off, d_shots, kc, k, rows);
        ADS_LAUNCHED(1);
        k_ac_adj<T, false, true><<<np, TPB, 0, sp>>>(ta.items + ta.pm_off, d_shots, ta.srcs,
                                                     ta.rcvs, kc, k, base, rows, dt2d);
      } else {
        k_ac_adj<T, false><<<np, TPB, 0, sp>>>(ta.items + ta.pm_off, d_shots, ta.srcs, ta.rcvs,
                                               kc, k, base, rows, dt2d);
      }
      ADS_LAUNCHED(1);
    }
    return ADS_OK;
  };
  if (int e = run_pm()) return e;  // the PML launch first, as in launch_fwd
  if (int e = run_in()) return e;
  if (fork) {
    ADS_CUDA(cudaEventRecord(ev_join, side));
    ADS_CUDA(cudaStreamWaitEvent(st, ev_join, 0));
  }
  return ADS_OK;
}

// Autotuner: for each candidate tile height, time a few forward steps and a
// few adjoint steps of the real kernels on the plan's buffers (CUDA events on
// `st`) and keep the fastest height for each kernel.  The buffers the trials
// touch are reset by every forward / gradient call.
template <typename T>
int AcPlan<T>::autotune(cudaStream_t st, int64_t pitch, size_t cap) {
  const int cand[] = {1, 2, 4, 8, 16, 32, 64};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ADS_CUDA(cudaEventCreate(&e0));
  ADS_CUDA(cudaEventCreate(&e1));
  const int tf_end = std::min(7, nstep[0]);
  const int ka_end = std::min(std::min(7, K + 1), nstep[0]);
  float best_f = 1e30f, best_a = 1e30f;
  int bf = ri_f, ba = ri;
  const int ri_f0 = ri_f, ri0 = ri;
  int rc = ADS_OK;
  for (int rows : cand) {
    TileList Lf, La;
    build_tiles(rows, Tile<T>::WF, pitch, Lf);
    build_tiles(rows, Tile<T>::WA, pitch, La);
    if (Lf.in.size() + Lf.pm.size() > cap || La.in.size() + La.pm.size() > cap) continue;
    if ((rc = upload_tiles(Lf, tf, st))) break;
    if ((rc = upload_tiles(La, ta, st))) break;
    ri_f = ri = rows;
    float ms_f = 0.f, ms_a = 0.f;
    int64_t nl = 0;
    for (int pass = 0; pass < 2 && rc == ADS_OK; pass++) {  // pass 0 warms up
      if (cudaEventRecord(e0, st) != cudaSuccess) rc = ADS_ERR_CUDA;
      for (int t = 2; t <= tf_end && rc == ADS_OK; t++) {
        rc = launch_fwd(st, false, shots_with_nstep_ge(t), t, 0, 0);
        nl += tf.launches(shots_with_nstep_ge(t));
      }
      cudaEventRecord(e1, st);
      if (rc != ADS_OK || cudaStreamSynchronize(st) != cudaSuccess ||
          cudaGetLastError() != cudaSuccess) {
        rc = fail(ADS_ERR_CUDA, "autotuner trial failed");
        break;
      }
      cudaEventElapsedTime(&ms_f, e0, e1);
      cudaEventRecord(e0, st);
      for (int k = 2; k <= ka_end && rc == ADS_OK; k++) {
        rc = launch_adj(st, shots_with_nstep_ge(k), k, 0);
        nl += ta.launches(shots_with_nstep_ge(k));
      }
      cudaEventRecord(e1, st);
      if (rc != ADS_OK || cudaStreamSynchronize(st) != cudaSuccess ||
          cudaGetLastError() != cudaSuccess) {
        rc = fail(ADS_ERR_CUDA, "autotuner trial failed");
        break;
      }
      cudaEventElapsedTime(&ms_a, e0, e1);
    }
    if (rc != ADS_OK) break;
    (void)nl;
    if (ms_f < best_f) {
      best_f = ms_f;
      bf = rows;
    }
    if (ms_a < best_a) {
      best_a = ms_a;
      ba = rows;
    }
  }
  if (rc != ADS_OK) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ri_f = ri_f0;
    ri = ri0;
    return rc;
  }
  ri_f = bf;
  ri = ba;
  // second phase: shorter row tiles for the PML items only
  auto time_range = [&](bool fwd, float& ms) -> int {
    for (int pass = 0; pass < 2; pass++) {
      ADS_CUDA(cudaEventRecord(e0, st));
      if (fwd) {
        for (int t = 2; t <= tf_end; t++)
          if (int e = launch_fwd(st, false, shots_with_nstep_ge(t), t, 0, 0)) return e;
      } else {
        for (int k = 2; k <= ka_end; k++)
          if (int e = launch_adj(st, shots_with_nstep_ge(k), k, 0)) return e;
      }
      ADS_CUDA(cudaEventRecord(e1, st));
      ADS_CUDA(cudaEventSynchronize(e1));
      ADS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    }
    return ADS_OK;
  };
  for (int which = 0; which < 2; which++) {
    const bool fwd = which == 0;
    const int rows = fwd ? ri_f : ri;
    const int width = fwd ? Tile<T>::WF : Tile<T>::WA;
    DevTiles& D = fwd ? tf : ta;
    int& pm = fwd ? ri_pf : ri_pa;
    pm = 0;
    TileList L0;
    build_tiles(rows, width, pitch, L0);
    if (int e = upload_tiles(L0, D, st)) return e;
    float best = 0.f;
    if (int e = time_range(fwd, best)) return e;
    int keep = 0;
    for (int d = 2; d <= 4; d *= 2) {
      if (rows % d != 0) continue;
      TileList L;
      build_tiles(rows, width, pitch, L, rows / d);
      if (L.in.size() + L.pm.size() > cap) continue;
      if (int e = upload_tiles(L, D, st)) return e;
      pm = rows / d;
      float ms = 0.f;
      if (int e = time_range(fwd, ms)) return e;
      if (ms < best) {
        best = ms;
        keep = rows / d;
      }
    }
    pm = keep;
    TileList L;
    build_tiles(rows, width, pitch, L, pm);
    if (int e = upload_tiles(L, D, st)) return e;
  }
  // third phase (tb_auto): steps per forward launch, 1 (the tiles chosen
  // above) against the time-blocked kernel at 2 and 4, over the same steps
  if (tb_auto && !tb_cand.empty()) {
    const int t_end = std::min(9, nstep[0]);
    auto time_tb = [&](int kb, float& ms) -> int {
      for (int pass = 0; pass < 2; pass++) {
        ADS_CUDA(cudaEventRecord(e0, st));
        for (int t0 = 2, blk = 0; t0 <= t_end; blk++) {
          const int NS = std::min(kb, t_end - t0 + 1);
          const int na = shots_with_nstep_ge(t0);
          if (kb == 1) {
            if (int e = launch_fwd(st, 0, na, t0, 0, 0)) return e;
          } else if (int e = launch_tb(st, false, tb_items_upto(na), t0, NS, 0, blk & 1, 0)) {
            return e;
          }
          t0 += NS;
        }
        ADS_CUDA(cudaEventRecord(e1, st));
        ADS_CUDA(cudaEventSynchronize(e1));
        ADS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      }
      return ADS_OK;
    };
    float best = 0.f;
    KB = 1;
    if (int e = time_tb(1, best)) return e;
    int best_kb = 1;
    for (const auto& cand : tb_cand) {
      if (int e = upload_tb(cand.second, st)) return e;
      KB = cand.first;
      RB = tb_rows_for(KB);
      float ms = 0.f;
      if (int e = time_tb(KB, ms)) return e;
      if (ms < best) {
        best = ms;
        best_kb = KB;
      }
    }
    KB = best_kb;
    RB = tb_rows_for(KB);
    for (const auto& cand : tb_cand)
      if (cand.first == KB)
        if (int e = upload_tb(cand.second, st)) return e;
    tb_cand.clear();
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ADS_CUDA(cudaStreamSynchronize(st));
  return ADS_OK;
}

template <typename T>
int AcPlan<T>::launch_tb(cudaStream_t st, bool seg, int nit, int t0, int NS, int base,
                         int in_set, int ck) {
  if constexpr (sizeof(T) == 4) {
#define ADS_TB(KBV)                                                                         \
  if (seg)                                                                                  \
    k_ac_fwd_tb<T, true, KBV><<<nit, TB_THREADS, 0, st>>>(d_tb_items, d_shots, d_tb_srcs,   \
                                                          d_tb_rows, d_tb_map, kc, t0, NS,  \
                                                          base, in_set, ck, RB);            \
  else                                                                                      \
    k_ac_fwd_tb<T, false, KBV><<<nit, TB_THREADS, 0, st>>>(d_tb_items, d_shots, d_tb_srcs,  \
                                                           d_tb_rows, d_tb_map, kc, t0, NS, \
                                                           base, in_set, ck, RB);
    switch (KB) {
      case 2: ADS_TB(2) break;
      case 4: ADS_TB(4) break;
      default: ADS_TB(8) break;
    }
#undef ADS_TB
    ADS_LAUNCHED(1);
    return ADS_OK;
  } else {
    (void)st; (void)seg; (void)nit; (void)t0; (void)NS; (void)base; (void)in_set; (void)ck;
    return fail(ADS_ERR_UNSUPPORTED, "time-blocked steps are implemented for FP32 plans");
  }
}

// Forward time loop (zero the state and traces, then the steps 2..NSTEP: one
// launch per step, or per block of up to KB steps that never crosses a
// checkpoint time 1 + sK).  count != nullptr: only count launches and the
// interior cell-steps of the loop.
template <typename T>
int AcPlan<T>::issue_forward(cudaStream_t st, int64_t* count) {
  if (count) {
    *count = 0;
    tcount[0] = tcount[1] = 0;
  } else {
    ADS_CUDA(cudaMemsetAsync(pool + zero_fwd_off, 0, zero_fwd_len, st));
    if (timing_run) ADS_CUDA(cudaEventRecord(ev[0], st));
  }
  const int a_res = res_seg < nseg_max ? 2 + res_seg * K : INT_MAX;  // first resident step
  int t0 = 2, blk = 0;
  while (t0 <= nstep[0]) {
    const int bound = 1 + K * (int)div_up(t0 - 1, K);  // next checkpoint time >= t0
    const int NS = KB > 1 ? std::min({KB, bound - t0 + 1, nstep[0] - t0 + 1}) : 1;
    const int t1 = t0 + NS - 1;
    const int na = shots_with_nstep_ge(t0);
    // checkpoint s >= 1 holds the state before step a_s = 2 + s K, i.e. after
    // t = 1 + s K; resident segments need none
    int ck = ((t1 - 1) % K == 0) ? (t1 - 1) / K : 0;
    if (ck >= res_seg) ck = 0;
    const bool res = t0 >= a_res;
    if (count) {
      const int nl = (KB > 1 ? 1 : tf.launches(na)) + (t0 == a_res ? 1 : 0);
      *count += nl;
      tcount[0] += nl;
      for (int t = t0; t <= t1; t++) tcount[1] += (double)cells_upto(shots_with_nstep_ge(t));
    } else if (KB > 1) {
      if (int e = launch_tb(st, false, tb_items_upto(na), t0, NS, 0, blk & 1, ck)) return e;
    } else {
      if (t0 == a_res) {  // u_{a-2}, u_{a-1} into the resident slots
        k_ac_seed<T><<<dim3(kRowBlocks, na), 256, 0, st>>>(d_shots, a_res, res_base);
        ADS_LAUNCHED(1);
      }
      if (int e = launch_fwd(st, res ? 2 : 0, na, t0, res ? res_base : 0, ck)) return e;
    }
    t0 = t1 + 1;
    blk++;
  }
  if (!count && timing_run) ADS_CUDA(cudaEventRecord(ev[1], st));
  return ADS_OK;
}

// Reverse sweep: zero adjoint state, seed lambdaU_T, then per segment from the
// last: restore, recompute, adjoint steps.
template <typename T>
int AcPlan<T>::issue_reverse(cudaStream_t st, int64_t* count) {
  int64_t n = 0;
  if (!count) {
    ADS_CUDA(cudaMemsetAsync(pool + zero_adj_off, 0, zero_adj_len, st));
    k_ac_adj_init<T><<<nshots, 128, 0, st>>>(d_shots, d_shot_rcvs, d_rcv_b, d_rcv_e, dt2d);
    ADS_LAUNCHED(1);
  }
  n++;
  for (int s = nseg_max - 1; s >= 0; s--) {
    const int a = 2 + s * K;
    // shots whose record reaches step a
    const int na = shots_with_nstep_ge(a);
    if (na == 0) continue;
    const int b_max = std::min(a + K - 1, nstep[0]);
    const bool res = s >= res_seg;  // resident: the store already holds the segment
    const int base = res ? res_base : a - 2;
    if (!res) {
      if (!count) {
        // phi / psi set the recompute's first step reads: variant W's step a
        // reads set (a-1) & 1; variant U's pre-pass of step a reads set a & 1
        k_ac_restore<T><<<dim3(kRowBlocks, na), 256, 0, st>>>(
            d_shots, s, a, KB > 1 ? 0 : (vu ? (a & 1) : -1), inc ? 1 : 0);
        ADS_LAUNCHED(1);
      }
      n++;
    }
    const bool timed = s == seg_timed;
    if (timed && timing_run) ADS_CUDA(cudaEventRecord(ev[2], st));
    if (timed && count) tcount[2] = tcount[3] = tcount[4] = tcount[5] = 0;
    for (int t0 = a, blk = 0; !res && t0 <= b_max - 1; blk++) {
      // active while t < b_shot = min(a+K-1, nstep), i.e. nstep >= t+1
      const int NS = KB > 1 ? std::min(KB, b_max - t0) : 1;
      const int nt = shots_with_nstep_ge(t0 + 1);
      const int nl = KB > 1 ? 1 : tf.launches(nt);
      if (timed && count) {
        tcount[2] += nl;
        for (int t = t0; t < t0 + NS; t++) tcount[3] += (double)cells_upto(shots_with_nstep_ge(t + 1));
      }
      if (!count) {
        if (KB > 1) {
          if (int e = launch_tb(st, true, tb_items_upto(nt), t0, NS, a - 2, blk & 1, 0)) return e;
        } else {
          if (int e = launch_fwd(st, 1, nt, t0, a - 2, 0)) return e;
        }
      }
      n += nl;
      t0 += NS;
    }
    if (timed && timing_run) {
      ADS_CUDA(cudaEventRecord(ev[3], st));
      ADS_CUDA(cudaEventRecord(ev[4], st));
    }
    for (int k = b_max; k >= a; k--) {
      const int nk = shots_with_nstep_ge(k);
      if (timed && count) {
        tcount[4] += ta.launches(nk);
        tcount[5] += (double)cells_upto(nk);
      }
      if (!count) {
        if (int e = launch_adj(st, nk, k, base)) return e;
      }
      n += ta.launches(nk);
    }
    if (timed && timing_run) ADS_CUDA(cudaEventRecord(ev[5], st));
    if (sizeof(T) == 4) {  // fold the segment's FP32 grad_c partial into FP64
      if (!count) {
        k_ac_flush_gc<T><<<dim3(kRowBlocks, na), 256, 0, st>>>(d_shots);
        ADS_LAUNCHED(1);
      }
      n++;
    }
  }
  if (count) *count = n;
  return ADS_OK;
}

template <typename T>
int AcPlan<T>::run_loop(int which, cudaStream_t st) {
  if (eF) {
    ADS_CUDA(cudaGraphLaunch(which == 0 ? eF : eR, st));
    note_launches(which == 0 ? nF : nR);
    return ADS_OK;
  }
  return which == 0 ? issue_forward(st, nullptr) : issue_reverse(st, nullptr);
}

template <typename T>
int AcPlan<T>::forward(const double* vp, void* traces, cudaStream_t st) {
  ADS_REQUIRE(vp, "null vp");
  k_ac_prep<T><<<dim3(256, nshots), 256, 0, st>>>(d_shots, vp, cfg.MY + 2);
  ADS_LAUNCHED(1);
  if (int e = run_loop(0, st)) return e;
  if (traces)
    ADS_CUDA(cudaMemcpyAsync(traces, d_traces, sizeof(T) * trace_total,
                             cudaMemcpyDeviceToDevice, st));
  return ADS_OK;
}

template <typename T>
int AcPlan<T>::gradient(const double* vp, const void* obs, double* loss, double* grad,
                        void* traces_out, cudaStream_t st, double* grad_srcv) {
  ADS_REQUIRE(vp && obs && loss && grad, "null argument");
  k_ac_prep<T><<<dim3(256, nshots), 256, 0, st>>>(d_shots, vp, cfg.MY + 2);
  ADS_LAUNCHED(1);
  if (int e = run_loop(0, st)) return e;
  k_misfit<T><<<kMisfitBlocks, 256, 0, st>>>(d_traces, (const T*)obs, d_resid, trace_total,
                                             d_partial);
  ADS_LAUNCHED(1);
  k_reduce_sum<<<1, 1024, 0, st>>>(d_partial, kMisfitBlocks, loss);
  ADS_LAUNCHED(1);
  if (int e = run_loop(1, st)) return e;
  const int64_t n = (cfg.MX + 2) * (cfg.MY + 2);
  k_ac_assemble<T><<<(unsigned)std::min<int64_t>(div_up(n, 256), 16384), 256, 0, st>>>(
      d_shots, nshots, vp, grad, cfg.MX + 2, cfg.MY + 2);
  ADS_LAUNCHED(1);
  if (traces_out)
    ADS_CUDA(cudaMemcpyAsync(traces_out, d_traces, sizeof(T) * trace_total,
                             cudaMemcpyDeviceToDevice, st));
  if (grad_srcv)  // per shot (nstep, nsrc), packed in the caller's shot order
    for (int s = 0; s < nshots; s++) {
      const AcShot<T>& h = hshots[s];
      const size_t n = (size_t)h.nstep * h.nsrc;
      if (n)
        ADS_CUDA(cudaMemcpyAsync(grad_srcv + src_off[order[s]], h.gsrc, sizeof(double) * n,
                                 cudaMemcpyDeviceToDevice, st));
    }
  return ADS_OK;
}

// One gradient with direct launches (no graphs) and CUDA events around the
// forward loop and around one full segment's recompute and adjoint launches.
template <typename T>
int AcPlan<T>::profile(const double* vp, const void* obs, double* out, cudaStream_t st) {
  ADS_REQUIRE(vp && obs && out, "null argument");
  k_ac_prep<T><<<dim3(256, nshots), 256, 0, st>>>(d_shots, vp, cfg.MY + 2);
  ADS_LAUNCHED(1);
  timing_run = true;
  int rc = issue_forward(st, nullptr);
  if (rc == ADS_OK) {
    k_misfit<T><<<kMisfitBlocks, 256, 0, st>>>(d_traces, (const T*)obs, d_resid, trace_total,
                                               d_partial);
    rc = issue_reverse(st, nullptr);
  }
  timing_run = false;
  if (rc != ADS_OK) return rc;
  ADS_CUDA(cudaStreamSynchronize(st));
  for (int r = 0; r < 3; r++) {
    float ms = 0.f;
    ADS_CUDA(cudaEventElapsedTime(&ms, ev[2 * r], ev[2 * r + 1]));
    out[3 * r] = ms;
    out[3 * r + 1] = tcount[2 * r];
    out[3 * r + 2] = tcount[2 * r + 1];
  }
  return ADS_OK;
}

}  // namespace
}  // namespace ads

struct ads_acoustic_plan {
  std::unique_ptr<ads::AcPlanBase> impl;
  int precision;
};

using namespace ads;

extern "C" {

int ads_acoustic_plan_create(ads_acoustic_plan** plan, const ads_acoustic_config* cfg,
                             const ads_acoustic_shot* shots, int64_t nshots,
                             ads_stream_t stream) {
  ADS_REQUIRE(plan && cfg && shots, "null argument");
  *plan = nullptr;
  if (int e = require_device()) return e;
  ADS_REQUIRE(cfg->precision == ADS_F64 || cfg->precision == ADS_F32,
              "precision must be ADS_F64 or ADS_F32");
  std::unique_ptr<ads_acoustic_plan> p(new ads_acoustic_plan);
  p->precision = cfg->precision;
  int rc;
  if (cfg->precision == ADS_F64) {
    auto* q = new AcPlan<double>();
    p->impl.reset(q);
    rc = q->create(*cfg, shots, nshots, (cudaStream_t)stream);
  } else {
    auto* q = new AcPlan<float>();
    p->impl.reset(q);
    rc = q->create(*cfg, shots, nshots, (cudaStream_t)stream);
  }
  if (rc != ADS_OK) return rc;
  *plan = p.release();
  return ADS_OK;
}

int ads_acoustic_plan_destroy(ads_acoustic_plan* plan) {
  if (!plan) return ADS_OK;
  cudaDeviceSynchronize();
  delete plan;
  return ADS_OK;
}

int64_t ads_acoustic_plan_trace_offset(const ads_acoustic_plan* plan, int64_t shot) {
  if (!plan || shot < 0 || shot >= (int64_t)plan->impl->trace_off.size()) return -1;
  return plan->impl->trace_off[shot];
}

int64_t ads_acoustic_plan_trace_count(const ads_acoustic_plan* plan) {
  return plan ? plan->impl->trace_total : -1;
}

int64_t ads_acoustic_plan_device_bytes(const ads_acoustic_plan* plan) {
  return plan ? plan->impl->bytes : -1;
}

int64_t ads_acoustic_plan_launches(const ads_acoustic_plan* plan, int gradient) {
  if (!plan) return -1;
  return gradient ? plan->impl->launches_grad : plan->impl->launches_fwd;
}

int64_t ads_acoustic_plan_resident_segments(const ads_acoustic_plan* plan) {
  return plan ? plan->impl->resident : -1;
}

int64_t ads_acoustic_plan_steps_per_block(const ads_acoustic_plan* plan) {
  return plan && plan->impl ? plan->impl->steps_per_block : -1;
}

int64_t ads_acoustic_plan_rows(const ads_acoustic_plan* plan, int which) {
  if (!plan || !plan->impl || which < 0 || which > 3) return -1;
  return plan->impl->rows[which];
}

int64_t ads_acoustic_plan_tma(const ads_acoustic_plan* plan) {
  // the interior forward runs through the tensor maps only in the increment form
  return plan && plan->impl ? (plan->impl->uses_tma && plan->impl->steps_per_block == 1) : -1;
}

int ads_acoustic_plan_device_status(ads_acoustic_plan* plan, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->device_status((cudaStream_t)stream);
}

int ads_acoustic_plan_profile(ads_acoustic_plan* plan, const double* vp, const void* observed,
                              double* out9, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->profile(vp, observed, out9, (cudaStream_t)stream);
}

int ads_acoustic_plan_forward(ads_acoustic_plan* plan, const double* vp, void* traces,
                              ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->forward(vp, traces, (cudaStream_t)stream);
}

int ads_acoustic_plan_gradient(ads_acoustic_plan* plan, const double* vp,
                               const void* observed, double* loss, double* grad_vp,
                               void* traces_out, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->gradient(vp, observed, loss, grad_vp, traces_out, (cudaStream_t)stream,
                              nullptr);
}

int ads_acoustic_plan_gradient_ex(ads_acoustic_plan* plan, const double* vp,
                                  const void* observed, double* loss, double* grad_vp,
                                  double* grad_srcv, void* traces_out, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->gradient(vp, observed, loss, grad_vp, traces_out, (cudaStream_t)stream,
                              grad_srcv);
}

int ads_acoustic_plan_set_source_values(ads_acoustic_plan* plan, int64_t shot,
                                        const double* srcv, ads_stream_t stream) {
  ADS_REQUIRE(plan, "null plan");
  return plan->impl->set_source_values(shot, srcv, (cudaStream_t)stream);
}

int64_t ads_acoustic_plan_source_offset(const ads_acoustic_plan* plan, int64_t shot) {
  if (!plan || shot < 0 || shot >= (int64_t)plan->impl->src_off.size()) return -1;
  return plan->impl->src_off[shot];
}

int ads_acoustic_forward(const ads_acoustic_config* cfg, const ads_acoustic_shot* shot,
                         const double* vp, void* traces, ads_stream_t stream) {
  ADS_REQUIRE(cfg && shot, "null argument");
  ads_acoustic_plan* p = nullptr;
  ads_acoustic_config c = *cfg;
  c.use_graph = 0;
  if (int e = ads_acoustic_plan_create(&p, &c, shot, 1, stream)) return e;
  int rc = ads_acoustic_plan_forward(p, vp, traces, stream);
  if (rc == ADS_OK && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
    rc = fail(ADS_ERR_CUDA, "stream synchronisation failed");
  ads_acoustic_plan_destroy(p);
  return rc;
}

int ads_acoustic_gradient(const ads_acoustic_config* cfg, const ads_acoustic_shot* shot,
                          const double* vp, const void* observed, double* loss,
                          double* grad_vp, ads_stream_t stream) {
  ADS_REQUIRE(cfg && shot, "null argument");
  ads_acoustic_plan* p = nullptr;
  ads_acoustic_config c = *cfg;
  c.use_graph = 0;
  if (int e = ads_acoustic_plan_create(&p, &c, shot, 1, stream)) return e;
  int rc = ads_acoustic_plan_gradient(p, vp, observed, loss, grad_vp, nullptr, stream);
  if (rc == ADS_OK && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
    rc = fail(ADS_ERR_CUDA, "stream synchronisation failed");
  ads_acoustic_plan_destroy(p);
  return rc;
}

}  // extern "C"
