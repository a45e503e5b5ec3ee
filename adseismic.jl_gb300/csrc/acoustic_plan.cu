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
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "ads_internal.h"

namespace ads {
namespace {

constexpr int WARPS = 4;
constexpr int TJ = 32 * WARPS;  // tile width along j (one warp per 32 columns)
constexpr unsigned FULL = 0xffffffffu;

struct CellRef {
  int64_t cell;  // element offset inside the shot's pitched field
  int idx;       // source / receiver index within the shot
  int pad;
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
  T *seg, *ckpt;      // segment store (k+1 fields), checkpoints (nseg x 4 fields)
  T *lu, *lp, *lq;    // adjoint rings (2 fields each)
  T *c, *sx, *ty;     // c = vp^2 (pitched), PML profiles along i and j
  double* gc;         // FP64 gradient accumulator (pitched)
  float* gc32;        // FP32 per-segment partial of grad_c (FP32 plans)
  const T* srcv;      // (nstep, nsrc), already multiplied by dt^2
  T *traces, *resid;  // (nstep+1, nrcv) packed views
};

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

// One forward step (variant W: phi/psi from the old field).  SEG=false: rings
// of two (u_t written over u_{t-2}), optional checkpoint write; SEG=true:
// segment store addressed by slot t - base.  Each thread slides down its column
// with the next row's loads issued one iteration ahead.
template <typename T, bool SEG>
__global__ void __launch_bounds__(TJ)
k_ac_fwd(const AcItem* __restrict__ items, const AcShot<T>* __restrict__ shots,
         const CellRef* __restrict__ srcs, const CellRef* __restrict__ rcvs, AcConst<T> K,
         int t, int base, int ckpt_slot, int ri) {
  const AcItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = it.j0 + warp * 32 + lane;
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
    wo = out;  // u_t overwrites u_{t-2}: each cell reads its own old value first
  }
  const T* pin = sh.p + (int64_t)((t - 1) & 1) * fs;
  T* pout = sh.p + (int64_t)(t & 1) * fs;
  const T* qin = sh.q + (int64_t)((t - 1) & 1) * fs;
  T* qout = sh.q + (int64_t)(t & 1) * fs;
  const T* __restrict__ cc = sh.c;
  const T* __restrict__ sx = sh.sx;
  const T* __restrict__ srcv = sh.srcv;
  const bool jin = j <= ny;
  const bool jld = j <= ny + 1;
  const bool jr = j + 1 <= ny + 1;  // lane 31's right neighbour exists
  const int64_t col = j + JOFF;
  const T tj = jld ? sh.ty[j] : T(0);
  const bool tfree = warp_tau_free<T>(sh.ty, j, ny);
  auto nz = [&](int r) { return !(tfree && sx[r] == T(0)); };  // phi/psi may be non-zero
  auto LD = [&](const T* a, int r, bool on) -> T {
    return (jld && on) ? a[(int64_t)r * P + col] : T(0);
  };
  const int i0 = it.i0, i_end = min(i0 + ri, nx + 1);
  bool n0 = nz(i0);
  T wm = LD(w, i0 - 1, true), w0 = LD(w, i0, true), wp = LD(w, i0 + 1, true);
  T pm = LD(pin, i0 - 1, nz(i0 - 1)), p0 = LD(pin, i0, n0), pp = LD(pin, i0 + 1, nz(i0 + 1));
  T q0 = LD(qin, i0, n0), wo0 = LD(wo, i0, true), c0 = LD(cc, i0, true);
  T hw = 0, hq = 0;  // lane 0: (i, j-1); lane 31: (i, j+1)
  {
    const int64_t r = (int64_t)i0 * P + col;
    if (lane == 0 && jld) {
      hw = w[r - 1];
      hq = n0 ? qin[r - 1] : T(0);
    } else if (lane == 31 && jr) {
      hw = w[r + 1];
      hq = n0 ? qin[r + 1] : T(0);
    }
  }
  for (int i = i0; i < i_end; i++) {
    const int64_t row = (int64_t)i * P + col;
    // prefetch: row i+2 of w and phi, row i+1 of psi, w_old, c and the halos
    const bool more = i + 1 < i_end;
    const bool n1 = more && nz(i + 1);
    T wn = 0, pn_ = 0, qn = 0, won = 0, cn = 0, hwn = 0, hqn = 0;
    if (more) {
      wn = LD(w, i + 2, true);
      pn_ = LD(pin, i + 2, nz(i + 2));
      qn = LD(qin, i + 1, n1);
      won = LD(wo, i + 1, true);
      cn = LD(cc, i + 1, true);
      if (lane == 0 && jld) {
        hwn = w[row + P - 1];
        hqn = n1 ? qin[row + P - 1] : T(0);
      } else if (lane == 31 && jr) {
        hwn = w[row + P + 1];
        hqn = n1 ? qin[row + P + 1] : T(0);
      }
    }
    T wS = __shfl_up_sync(FULL, w0, 1), wN = __shfl_down_sync(FULL, w0, 1);
    T qS = __shfl_up_sync(FULL, q0, 1), qN = __shfl_down_sync(FULL, q0, 1);
    if (lane == 0) {
      wS = hw;
      qS = hq;
    } else if (lane == 31) {
      wN = hw;
      qN = hq;
    }
    if (jin) {
      const T c = c0, sg = sx[i], s = sg + tj;
      T v = (T(2) - sg * tj * K.dt2 - K.kxy * c) * w0 + c * K.cx * (wp + wm) +
            c * K.cy * (wN + wS) + K.fx * (pp - pm) + K.fy * (qN - qS) -
            (T(1) - s * K.hdt) * wo0;
      if (s != T(0)) v = v / (T(1) + s * K.hdt);
      for (int e = it.src_b; e < it.src_e; e++) {
        const CellRef r = srcs[e];
        if (r.cell == row) v += srcv[(int64_t)(t - 1) * sh.nsrc + r.idx];
      }
      out[row] = v;
      T pnew = T(0), qnew = T(0);
      if (n0) {
        pnew = (T(1) - K.dt * sg) * p0 + K.ex * c * (tj - sg) * (wp - wm);
        qnew = (T(1) - K.dt * tj) * q0 + K.ey * c * (sg - tj) * (wN - wS);
        pout[row] = pnew;
        qout[row] = qnew;
      }
      if (!SEG && ckpt_slot > 0 && ckpt_slot < sh.nseg) {
        T* ck = sh.ckpt + (int64_t)ckpt_slot * 4 * fs;
        ck[row] = v;
        ck[fs + row] = w0;
        if (n0) {
          ck[2 * fs + row] = pnew;
          ck[3 * fs + row] = qnew;
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
  }
  if (!SEG && it.rcv_e > it.rcv_b) {
    __syncthreads();  // the tile's u_t is in global memory and visible block-wide
    for (int e = it.rcv_b + threadIdx.x; e < it.rcv_e; e += blockDim.x) {
      const CellRef r = rcvs[e];
      sh.traces[(int64_t)t * sh.nrcv + r.idx] = out[r.cell];
    }
  }
}

// Restore checkpoint `slot` of every active shot into the segment store
// (slot 0 <- u_{a-2}, slot 1 <- u_{a-1}) and the phi/psi rings at a-1.
template <typename T>
__global__ void __launch_bounds__(TJ)
k_ac_restore(const AcItem* __restrict__ items, const AcShot<T>* __restrict__ shots,
             int slot, int a, int ri) {
  const AcItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int j = it.j0 + threadIdx.x;
  if (j > sh.ny) return;
  const int64_t P = sh.pitch, fs = sh.fs, col = j + JOFF;
  const T* ck = sh.ckpt + (int64_t)slot * 4 * fs;
  T* pr = sh.p + (int64_t)((a - 1) & 1) * fs;
  T* qr = sh.q + (int64_t)((a - 1) & 1) * fs;
  const int i_end = min(it.i0 + ri, sh.nx + 1);
  for (int i = it.i0; i < i_end; i++) {
    const int64_t row = (int64_t)i * P + col;
    sh.seg[row] = ck[fs + row];
    sh.seg[fs + row] = ck[row];
    pr[row] = ck[2 * fs + row];
    qr[row] = ck[3 * fs + row];
  }
}

// Gradient-side terms of one cell for the i direction (XP: what the cell's
// stencil sends to its i+1 neighbour, XM: to its i-1 neighbour, XR: to
// phi's i+-1 neighbours).
template <typename T>
struct RowTerms {
  T gu, gp, c, inv, XP, XM, XR;
};

template <typename T>
__device__ __forceinline__ RowTerms<T> row_terms(T gu, T gp, T c, T sg, T tj,
                                                 const AcConst<T>& K) {
  RowTerms<T> r;
  const T s = sg + tj;
  r.gu = gu;
  r.gp = gp;
  r.c = c;
  r.inv = s != T(0) ? T(1) / (T(1) + s * K.hdt) : T(1);
  const T gui = gu * r.inv;
  const T bx = c * K.cx * gui, exg = K.ex * c * (tj - sg) * gp;
  r.XP = bx + exg;
  r.XM = bx - exg;
  r.XR = K.fx * gui;
  return r;
}

// j-direction terms of one cell (YP to j+1, YM to j-1, YR to psi's j+-1).
template <typename T>
__device__ __forceinline__ void col_terms(T gui, T gq, T c, T sg, T tj, const AcConst<T>& K,
                                          T& YP, T& YM, T& YR) {
  const T by = c * K.cy * gui, eyg = K.ey * c * (sg - tj) * gq;
  YP = by + eyg;
  YM = by - eyg;
  YR = K.fy * gui;
}

// One adjoint step k (gather form of the transpose of step k):
//   lambdaU_{k-1} = D lambdaU_{k+1} + sum of what u_k, phi_k, psi_k send to w,
//   lambdaPhi_{k-1}, lambdaPsi_{k-1} likewise, grad_c += d(step k)/dc . lambda_k,
// then lambdaU_{k-1} += residual_{k-1} at the receivers.  FP32 plans add the
// grad_c contribution to a per-segment FP32 partial (flushed into the FP64
// accumulator at the end of each segment); FP64 plans accumulate in FP64.
template <typename T>
__global__ void __launch_bounds__(TJ)
k_ac_adj(const AcItem* __restrict__ items, const AcShot<T>* __restrict__ shots,
         const CellRef* __restrict__ rcvs, AcConst<T> K, int k, int base, int ri) {
  const AcItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = it.j0 + warp * 32 + lane;
  const int nx = sh.nx, ny = sh.ny;
  const int64_t P = sh.pitch, fs = sh.fs;
  const T* w = sh.seg + (int64_t)(k - 1 - base) * fs;   // u_{k-1}
  T* lun = sh.lu + (int64_t)((k + 1) & 1) * fs;         // in: lambdaU_{k+1}; out: _{k-1}
  const T* luc = sh.lu + (int64_t)(k & 1) * fs;         // lambdaU_k
  const T* lpc = sh.lp + (int64_t)(k & 1) * fs;
  T* lpo = sh.lp + (int64_t)((k - 1) & 1) * fs;
  const T* lqc = sh.lq + (int64_t)(k & 1) * fs;
  T* lqo = sh.lq + (int64_t)((k - 1) & 1) * fs;
  const T* __restrict__ cc = sh.c;
  const T* __restrict__ sx = sh.sx;
  const T* __restrict__ ty = sh.ty;
  const bool jin = j <= ny;
  const bool jld = j <= ny + 1;
  const bool jr = j + 1 <= ny + 1;
  const int64_t col = j + JOFF;
  const T tj = jld ? ty[j] : T(0);
  const bool tfree = warp_tau_free<T>(ty, j, ny);
  auto nz = [&](int r) { return !(tfree && sx[r] == T(0)); };
  auto LD = [&](const T* a, int r, bool on) -> T {
    return (jld && on) ? a[(int64_t)r * P + col] : T(0);
  };
  // halo cell (i, j -+ 1) terms for lanes 0 / 31
  const T th = lane == 0 ? ty[j - 1] : (jr ? ty[j + 1] : T(0));
  const int64_t hoff = lane == 0 ? -1 : 1;
  const bool hon = (lane == 0 && jld) || (lane == 31 && jr);

  const int i0 = it.i0, i_end = min(i0 + ri, nx + 1);
  RowTerms<T> Rm = row_terms<T>(LD(luc, i0 - 1, true), LD(lpc, i0 - 1, nz(i0 - 1)),
                                LD(cc, i0 - 1, true), sx[i0 - 1], tj, K);
  RowTerms<T> R0 = row_terms<T>(LD(luc, i0, true), LD(lpc, i0, nz(i0)), LD(cc, i0, true),
                                sx[i0], tj, K);
  T gu1 = LD(luc, i0 + 1, true), gp1 = LD(lpc, i0 + 1, nz(i0 + 1)), c1 = LD(cc, i0 + 1, true);
  T wm = LD(w, i0 - 1, true), w0 = LD(w, i0, true), wp = LD(w, i0 + 1, true);
  bool n0 = nz(i0);
  T gq = LD(lqc, i0, n0), lu_next = LD(lun, i0, true);
  T hgu = 0, hgq = 0, hc = 0, hw = 0;
  if (hon) {
    const int64_t r = (int64_t)i0 * P + col + hoff;
    hgu = luc[r];
    hgq = n0 ? lqc[r] : T(0);
    hc = cc[r];
    hw = w[r];
  }
  for (int i = i0; i < i_end; i++) {
    const int64_t row = (int64_t)i * P + col;
    const RowTerms<T> Rp = row_terms<T>(gu1, gp1, c1, sx[i + 1], tj, K);
    // prefetch: row i+2 (lambdaU_k, lambdaPhi_k, c, u_{k-1}), row i+1 (lambdaPsi_k,
    // lambdaU_{k+1}) and the halo cells of row i+1
    const bool more = i + 1 < i_end;
    const bool n1 = more && nz(i + 1);
    T gu2 = 0, gp2 = 0, c2 = 0, w2 = 0, gqn = 0, lun1 = 0, hgun = 0, hgqn = 0, hcn = 0, hwn = 0;
    if (more) {
      gu2 = LD(luc, i + 2, true);
      gp2 = LD(lpc, i + 2, nz(i + 2));
      c2 = LD(cc, i + 2, true);
      w2 = LD(w, i + 2, true);
      gqn = LD(lqc, i + 1, n1);
      lun1 = LD(lun, i + 1, true);
      if (hon) {
        const int64_t r = row + P + hoff;
        hgun = luc[r];
        hgqn = n1 ? lqc[r] : T(0);
        hcn = cc[r];
        hwn = w[r];
      }
    }
    const T sg = sx[i];
    const T gui = R0.gu * R0.inv;
    T YP, YM, YR;
    col_terms<T>(gui, gq, R0.c, sg, tj, K, YP, YM, YR);
    T YPl = __shfl_up_sync(FULL, YP, 1), YRl = __shfl_up_sync(FULL, YR, 1);
    T YMr = __shfl_down_sync(FULL, YM, 1), YRr = __shfl_down_sync(FULL, YR, 1);
    T wS = __shfl_up_sync(FULL, w0, 1), wN = __shfl_down_sync(FULL, w0, 1);
    if (lane == 0 || lane == 31) {
      const T s1 = sg + th;
      const T inv1 = s1 != T(0) ? T(1) / (T(1) + s1 * K.hdt) : T(1);
      T a, b, r;
      col_terms<T>(hgu * inv1, hgq, hc, sg, th, K, a, b, r);
      if (lane == 0) {
        YPl = a;
        YRl = r;
        wS = hw;
      } else {
        YMr = b;
        YRr = r;
        wN = hw;
      }
    }
    if (jin) {
      const T c = R0.c, gp = R0.gp, s = sg + tj;
      const T nu = -(T(1) - s * K.hdt) * R0.inv * lu_next +
                   (T(2) - sg * tj * K.dt2 - K.kxy * c) * gui + Rm.XP + Rp.XM + YPl + YMr;
      const T g = (-K.kxy * w0 + K.cx * (wp + wm) + K.cy * (wN + wS)) * gui +
                  K.ex * (tj - sg) * (wp - wm) * gp + K.ey * (sg - tj) * (wN - wS) * gq;
      lun[row] = nu;
      if (n0) {
        lpo[row] = (T(1) - K.dt * sg) * gp + Rm.XR - Rp.XR;
        lqo[row] = (T(1) - K.dt * tj) * gq + YRl - YRr;
      }
      if (sizeof(T) == 4)
        sh.gc32[row] += (float)g;
      else
        sh.gc[row] += (double)g;
    }
    Rm = R0;
    R0 = Rp;
    gu1 = gu2;
    gp1 = gp2;
    c1 = c2;
    wm = w0;
    w0 = wp;
    wp = w2;
    gq = gqn;
    lu_next = lun1;
    hgu = hgun;
    hgq = hgqn;
    hc = hcn;
    hw = hwn;
    n0 = n1;
  }
  if (k - 1 >= 2 && it.rcv_e > it.rcv_b) {
    __syncthreads();
    for (int e = it.rcv_b + threadIdx.x; e < it.rcv_e; e += blockDim.x) {
      const CellRef r = rcvs[e];
      atomicAdd(lun + r.cell, sh.resid[(int64_t)(k - 1) * sh.nrcv + r.idx]);
    }
  }
}

// End of a segment (FP32 plans): grad_c (FP64) += the segment's FP32 partial,
// which is reset to zero.
template <typename T>
__global__ void __launch_bounds__(TJ)
k_ac_flush_gc(const AcItem* __restrict__ items, const AcShot<T>* __restrict__ shots, int ri) {
  const AcItem it = items[blockIdx.x];
  const AcShot<T>& sh = shots[it.shot];
  const int j = it.j0 + threadIdx.x;
  if (j > sh.ny) return;
  const int i_end = min(it.i0 + ri, sh.nx + 1);
  for (int i = it.i0; i < i_end; i++) {
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
                              const int* __restrict__ rcv_e) {
  const int s = blockIdx.x;
  const AcShot<T>& sh = shots[s];
  T* lu = sh.lu + (int64_t)(sh.nstep & 1) * sh.fs;
  for (int e = rcv_b[s] + threadIdx.x; e < rcv_e[s]; e += blockDim.x) {
    const CellRef r = rcvs[e];
    atomicAdd(lu + r.cell, sh.resid[(int64_t)sh.nstep * sh.nrcv + r.idx]);
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
                       void* traces_out, cudaStream_t st) = 0;
  virtual int profile(const double* vp, const void* obs, double* out, cudaStream_t st) = 0;
  std::vector<int64_t> trace_off;
  int64_t trace_total = 0;
  int64_t bytes = 0;
  int64_t launches_fwd = 0, launches_grad = 0;
};

namespace {

template <typename T>
struct AcPlan final : AcPlanBase {
  ads_acoustic_config cfg{};
  int nshots = 0;
  int K = 0;          // checkpoint spacing
  int ri = 8;         // rows per thread
  int nseg_max = 0;
  std::vector<int> order;         // shot order (record length descending)
  std::vector<int> nstep;         // per sorted shot
  std::vector<int> item_shot_end; // per sorted shot: items of shots [0..s] = [0, end)
  std::vector<int> rcv_b_host, rcv_e_host;
  AcConst<T> kc{};
  // device
  char* pool = nullptr;
  size_t pool_bytes = 0;
  AcShot<T>* d_shots = nullptr;
  AcItem* d_items = nullptr;
  CellRef *d_srcs = nullptr, *d_rcvs = nullptr, *d_shot_rcvs = nullptr;
  int *d_rcv_b = nullptr, *d_rcv_e = nullptr;
  T *d_traces = nullptr, *d_resid = nullptr;
  double* d_partial = nullptr;
  static constexpr int kMisfitBlocks = 512;
  size_t zero_fwd_off = 0, zero_fwd_len = 0, zero_adj_off = 0, zero_adj_len = 0;
  std::vector<AcShot<T>> hshots;
  int nitems = 0;
  cudaStream_t cap = nullptr;
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

  ~AcPlan() override {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (eF) cudaGraphExecDestroy(eF);
    if (eR) cudaGraphExecDestroy(eR);
    if (gF) cudaGraphDestroy(gF);
    if (gR) cudaGraphDestroy(gR);
    if (cap) cudaStreamDestroy(cap);
    if (pool) cudaFree(pool);
  }

  int items_upto(int t_active_count) const {  // items of the first n sorted shots
    return t_active_count <= 0 ? 0 : item_shot_end[t_active_count - 1];
  }
  std::vector<int64_t> cells_prefix;  // interior cells of the first n sorted shots
  int64_t cells_upto(int n) const { return n <= 0 ? 0 : cells_prefix[n - 1]; }
  int profile(const double* vp, const void* obs, double* out, cudaStream_t st) override;
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
               void* traces_out, cudaStream_t st) override;
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
  ADS_REQUIRE(c.dx > 0 && c.dy > 0 && c.dt > 0, "dx, dy, dt must be positive");
  ADS_REQUIRE(c.npml >= 1 && c.Rcoef > 0 && c.Rcoef < 1, "invalid PML parameters");
  ADS_REQUIRE(c.variant == ADS_VARIANT_W,
              "whole-path plans implement variant W (the custom-operator form); use the "
              "single-step operators for variant U");
  ADS_REQUIRE(c.ckpt_every >= 0 && c.rows_per_thread >= 0, "negative tuning parameter");
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[s];
    ADS_REQUIRE(h.nx >= 1 && h.x0 >= 0 && h.x0 + h.nx + 2 <= c.MX + 2,
                "shot %d: window [x0=%lld, x0+nx+2=%lld) outside the model (MX+2=%lld)", s,
                (long long)h.x0, (long long)(h.x0 + h.nx + 2), (long long)(c.MX + 2));
    ADS_REQUIRE(h.nstep >= 2 && h.nstep < (1 << 24), "shot %d: nstep must be >= 2", s);
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
    while (ri > 2 && cells / ((int64_t)ri * TJ) < 152 * 8) ri /= 2;
  }
  // ---- trace layout (packed in the caller's shot order)
  trace_off.resize(ns);
  trace_total = 0;
  for (int s = 0; s < ns; s++) {
    trace_off[s] = trace_total;
    trace_total += (shots[s].nstep + 1) * shots[s].nrcv;
  }
  // ---- memory layout
  const int64_t pitch = grid_pitch(MY);
  size_t off_fwd_begin, off_fwd_end, off_adj_begin, off_adj_end;
  DevPool L;
  struct Offs {
    size_t u, p, q, seg, ckpt, lu, lp, lq, c, sx, ty, gc, gc32, srcv;
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
  }
  off_adj_end = L.used;
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[order[s]];
    const int64_t fs = (h.nx + 2) * pitch * (int64_t)sizeof(T);
    offs[s].seg = L.take((size_t)(K + 1) * fs);
    offs[s].ckpt = L.take((size_t)nseg[s] * 4 * fs);
    offs[s].c = L.take(fs);
    offs[s].sx = L.take(sizeof(T) * (h.nx + 2));
    offs[s].ty = L.take(sizeof(T) * (MY + 2));
    offs[s].srcv = L.take(sizeof(T) * std::max<int64_t>(h.nstep * h.nsrc, 1));
  }
  const size_t resid_off = L.take(sizeof(T) * std::max<int64_t>(trace_total, 1));
  const size_t partial_off = L.take(sizeof(double) * kMisfitBlocks);
  // items, sources, receivers
  std::vector<AcItem> items;
  std::vector<CellRef> srcs, rcvs, shot_rcvs;
  item_shot_end.resize(ns);
  rcv_b_host.resize(ns);
  rcv_e_host.resize(ns);
  for (int s = 0; s < ns; s++) {
    const ads_acoustic_shot& h = shots[order[s]];
    const int nx = (int)h.nx, ny = (int)MY;
    rcv_b_host[s] = (int)shot_rcvs.size();
    for (int64_t r = 0; r < h.nrcv; r++) {
      const int64_t i = h.rcvi[r] - 1, j = h.rcvj[r] - 1;
      if (i < 1 || i > nx || j < 1 || j > ny) continue;  // frame: trace stays 0
      shot_rcvs.push_back({i * pitch + j + JOFF, (int)r, 0});
    }
    rcv_e_host[s] = (int)shot_rcvs.size();
    for (int i0 = 1; i0 <= nx; i0 += ri) {
      for (int j0 = 1; j0 <= ny; j0 += TJ) {
        AcItem it{};
        it.shot = s;
        it.i0 = i0;
        it.j0 = j0;
        it.src_b = (int)srcs.size();
        for (int64_t k = 0; k < h.nsrc; k++) {
          const int64_t i = h.srci[k] - 1, j = h.srcj[k] - 1;
          if (i >= i0 && i < i0 + ri && j >= j0 && j < j0 + TJ)
            srcs.push_back({i * pitch + j + JOFF, (int)k, 0});
        }
        it.src_e = (int)srcs.size();
        it.rcv_b = (int)rcvs.size();
        for (int64_t r = 0; r < h.nrcv; r++) {
          const int64_t i = h.rcvi[r] - 1, j = h.rcvj[r] - 1;
          if (i >= i0 && i < i0 + ri && i <= nx && j >= j0 && j < j0 + TJ && j <= ny && j >= 1)
            rcvs.push_back({i * pitch + j + JOFF, (int)r, 0});
        }
        it.rcv_e = (int)rcvs.size();
        items.push_back(it);
      }
    }
    item_shot_end[s] = (int)items.size();
  }
  nitems = (int)items.size();
  const size_t shots_off = L.take(sizeof(AcShot<T>) * ns);
  const size_t items_off = L.take(sizeof(AcItem) * items.size());
  const size_t srcs_off = L.take(sizeof(CellRef) * std::max<size_t>(srcs.size(), 1));
  const size_t rcvs_off = L.take(sizeof(CellRef) * std::max<size_t>(rcvs.size(), 1));
  const size_t shot_rcvs_off = L.take(sizeof(CellRef) * std::max<size_t>(shot_rcvs.size(), 1));
  const size_t rcvb_off = L.take(sizeof(int) * ns);
  const size_t rcve_off = L.take(sizeof(int) * ns);
  pool_bytes = L.used;
  bytes = (int64_t)pool_bytes;
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
  d_items = (AcItem*)(pool + items_off);
  d_srcs = (CellRef*)(pool + srcs_off);
  d_rcvs = (CellRef*)(pool + rcvs_off);
  d_shot_rcvs = (CellRef*)(pool + shot_rcvs_off);
  d_rcv_b = (int*)(pool + rcvb_off);
  d_rcv_e = (int*)(pool + rcve_off);
  // per-shot structs and host-side data (profiles, scaled wavelets)
  hshots.resize(ns);
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
    d.p = (T*)(pool + offs[s].p);
    d.q = (T*)(pool + offs[s].q);
    d.seg = (T*)(pool + offs[s].seg);
    d.ckpt = (T*)(pool + offs[s].ckpt);
    d.lu = (T*)(pool + offs[s].lu);
    d.lp = (T*)(pool + offs[s].lp);
    d.lq = (T*)(pool + offs[s].lq);
    d.c = (T*)(pool + offs[s].c);
    d.sx = (T*)(pool + offs[s].sx);
    d.ty = (T*)(pool + offs[s].ty);
    d.gc = (double*)(pool + offs[s].gc);
    d.gc32 = sizeof(T) == 4 ? (float*)(pool + offs[s].gc32) : nullptr;
    d.srcv = (const T*)(pool + offs[s].srcv);
    d.traces = d_traces + trace_off[order[s]];
    d.resid = d_resid + trace_off[order[s]];
    sx.assign(h.nx + 2, 0.0);
    ty.assign(MY + 2, 0.0);
    acoustic_pml_1d(h.nx, MY, c.dx, c.dy, c.npml, c.vp_ref, c.Rcoef, c.use_pml, sx.data(),
                    ty.data());
    host_bufs.emplace_back(sx.begin(), sx.end());
    ADS_CUDA(cudaMemcpyAsync(d.sx, host_bufs.back().data(), sizeof(T) * sx.size(),
                             cudaMemcpyHostToDevice, st));
    host_bufs.emplace_back(ty.begin(), ty.end());
    ADS_CUDA(cudaMemcpyAsync(d.ty, host_bufs.back().data(), sizeof(T) * ty.size(),
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
  ADS_CUDA(cudaMemcpyAsync(d_items, items.data(), sizeof(AcItem) * items.size(),
                           cudaMemcpyHostToDevice, st));
  if (!srcs.empty())
    ADS_CUDA(cudaMemcpyAsync(d_srcs, srcs.data(), sizeof(CellRef) * srcs.size(),
                             cudaMemcpyHostToDevice, st));
  if (!rcvs.empty())
    ADS_CUDA(cudaMemcpyAsync(d_rcvs, rcvs.data(), sizeof(CellRef) * rcvs.size(),
                             cudaMemcpyHostToDevice, st));
  if (!shot_rcvs.empty())
    ADS_CUDA(cudaMemcpyAsync(d_shot_rcvs, shot_rcvs.data(), sizeof(CellRef) * shot_rcvs.size(),
                             cudaMemcpyHostToDevice, st));
  ADS_CUDA(cudaMemcpyAsync(d_rcv_b, rcv_b_host.data(), sizeof(int) * ns,
                           cudaMemcpyHostToDevice, st));
  ADS_CUDA(cudaMemcpyAsync(d_rcv_e, rcv_e_host.data(), sizeof(int) * ns,
                           cudaMemcpyHostToDevice, st));
  ADS_CUDA(cudaStreamSynchronize(st));  // host staging buffers go out of scope
  // ---- timing ranges: the first full-length segment the reverse sweep meets
  cells_prefix.resize(ns);
  for (int s = 0; s < ns; s++)
    cells_prefix[s] = (s ? cells_prefix[s - 1] : 0) + (int64_t)shots[order[s]].nx * MY;
  seg_timed = nseg_max >= 2 ? nseg_max - 2 : 0;
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

// Forward time loop (zero the rings and traces, then one launch per step).
// count != nullptr: only count kernel launches.
template <typename T>
int AcPlan<T>::issue_forward(cudaStream_t st, int64_t* count) {
  if (count) {
    *count = 0;
    tcount[0] = tcount[1] = 0;
    for (int t = 2; t <= nstep[0]; t++) {
      *count += 1;
      tcount[0] += 1;
      tcount[1] += (double)cells_upto(shots_with_nstep_ge(t));
    }
    return ADS_OK;
  }
  ADS_CUDA(cudaMemsetAsync(pool + zero_fwd_off, 0, zero_fwd_len, st));
  if (timing_run) ADS_CUDA(cudaEventRecord(ev[0], st));
  for (int t = 2; t <= nstep[0]; t++) {
    const int na = shots_with_nstep_ge(t);
    const int nit = items_upto(na);
    // checkpoint s >= 1 holds the state before step a_s = 2 + s K, i.e. after t = 1 + s K
    const int ck = ((t - 1) % K == 0) ? (t - 1) / K : 0;
    k_ac_fwd<T, false><<<nit, TJ, 0, st>>>(d_items, d_shots, d_srcs, d_rcvs, kc, t, 0, ck, ri);
    ADS_LAUNCHED(1);
  }
  if (timing_run) ADS_CUDA(cudaEventRecord(ev[1], st));
  return ADS_OK;
}

// Reverse sweep: zero adjoint state, seed lambdaU_T, then per segment from the
// last: restore, recompute, adjoint steps.
template <typename T>
int AcPlan<T>::issue_reverse(cudaStream_t st, int64_t* count) {
  int64_t n = 0;
  if (!count) {
    ADS_CUDA(cudaMemsetAsync(pool + zero_adj_off, 0, zero_adj_len, st));
    k_ac_adj_init<T><<<nshots, 128, 0, st>>>(d_shots, d_shot_rcvs, d_rcv_b, d_rcv_e);
    ADS_LAUNCHED(1);
  }
  n++;
  for (int s = nseg_max - 1; s >= 0; s--) {
    const int a = 2 + s * K;
    // shots whose record reaches step a
    const int na = shots_with_nstep_ge(a);
    if (na == 0) continue;
    const int b_max = std::min(a + K - 1, nstep[0]);
    if (!count) {
      k_ac_restore<T><<<items_upto(na), TJ, 0, st>>>(d_items, d_shots, s, a, ri);
      ADS_LAUNCHED(1);
    }
    n++;
    const bool timed = s == seg_timed;
    if (timed && timing_run) ADS_CUDA(cudaEventRecord(ev[2], st));
    if (timed && count) tcount[2] = tcount[3] = tcount[4] = tcount[5] = 0;
    for (int t = a; t <= b_max - 1; t++) {
      // active while t < b_shot = min(a+K-1, nstep), i.e. nstep >= t+1
      const int nt = shots_with_nstep_ge(t + 1);
      if (timed && count) {
        tcount[2] += 1;
        tcount[3] += (double)cells_upto(nt);
      }
      if (!count) {
        k_ac_fwd<T, true><<<items_upto(nt), TJ, 0, st>>>(d_items, d_shots, d_srcs, d_rcvs, kc,
                                                         t, a - 2, 0, ri);
        ADS_LAUNCHED(1);
      }
      n++;
    }
    if (timed && timing_run) {
      ADS_CUDA(cudaEventRecord(ev[3], st));
      ADS_CUDA(cudaEventRecord(ev[4], st));
    }
    for (int k = b_max; k >= a; k--) {
      const int nk = shots_with_nstep_ge(k);
      if (timed && count) {
        tcount[4] += 1;
        tcount[5] += (double)cells_upto(nk);
      }
      if (!count) {
        k_ac_adj<T><<<items_upto(nk), TJ, 0, st>>>(d_items, d_shots, d_rcvs, kc, k, a - 2, ri);
        ADS_LAUNCHED(1);
      }
      n++;
    }
    if (timed && timing_run) ADS_CUDA(cudaEventRecord(ev[5], st));
    if (sizeof(T) == 4) {  // fold the segment's FP32 grad_c partial into FP64
      if (!count) {
        k_ac_flush_gc<T><<<items_upto(na), TJ, 0, st>>>(d_items, d_shots, ri);
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
                        void* traces_out, cudaStream_t st) {
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
  return plan->impl->gradient(vp, observed, loss, grad_vp, traces_out, (cudaStream_t)stream);
}

int ads_acoustic_forward(const ads_acoustic_config* cfg, const ads_acoustic_shot* shot,
                         const double* vp, void* traces, ads_stream_t stream) {
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
