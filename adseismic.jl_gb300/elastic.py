"""Elastic host API mirroring ADSeismic's src/Struct.jl:4-78 and
src/Core.jl:31-412,659-712 on top of the C ABI."""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import ADS_F32, ADS_F64, call, lib
from .acoustic import _ptr, _require_cuda, _stream

NFIELD = 13  # vx, vy, sigmaxx, sigmayy, sigmaxy, mem[1..8]


@dataclass
class ElasticPropagatorParams:
    """src/Struct.jl:4-32 (same fields and defaults)."""
    NX: int = 101
    NY: int = 641
    NSTEP: int = 2000 * 2
    DELTAX: float = 10.0
    DELTAY: float = 10.0
    DELTAT: float = 2.0e-3 / 2
    f0: float = 5.0
    vp_ref: float = 2000.0
    USE_PML_XMIN: bool = True
    USE_PML_XMAX: bool = True
    USE_PML_YMIN: bool = True
    USE_PML_YMAX: bool = True
    NPOINTS_PML: int = 12
    NPOWER: float = 2.0
    K_MAX_PML: float = 1.0
    ALPHA_MAX_PML: float = None  # default 2 pi (f0/2), as Struct.jl:25
    Rcoef: float = 0.001
    IT_DISPLAY: int = 0

    def __post_init__(self):
        if self.ALPHA_MAX_PML is None:
            self.ALPHA_MAX_PML = 2.0 * math.pi * (self.f0 / 2.0)

    @property
    def use_pml(self) -> int:
        return (int(self.USE_PML_XMIN) | int(self.USE_PML_XMAX) << 1 |
                int(self.USE_PML_YMIN) << 2 | int(self.USE_PML_YMAX) << 3)


@dataclass
class ElasticSource:
    """src/Struct.jl:50-55: srctype 0 vx, 1 vy, 2 sxx, 3 syy, 4 sxy; srcv (NSTEP, nsrc)."""
    srci: np.ndarray
    srcj: np.ndarray
    srctype: np.ndarray
    srcv: np.ndarray


@dataclass
class ElasticReceiver:
    """src/Struct.jl:57-62; rcvv (nrcv, NSTEP+1) after SimulatedObservation."""
    rcvi: np.ndarray
    rcvj: np.ndarray
    rcvtype: np.ndarray
    rcvv: object = None


def compute_PML_Params(param: ElasticPropagatorParams):
    """src/Core.jl:231-407: (ax, bx, kx, ay, by, ky) as (2, NX) and (2, NY) arrays."""
    NX, NY = param.NX, param.NY
    a = [np.empty(2 * NX) for _ in range(3)] + [np.empty(2 * NY) for _ in range(3)]
    call("ads_elastic_cpml_profiles", NX, NY, param.DELTAX, param.DELTAY, param.DELTAT,
         param.NPOINTS_PML, param.NPOWER, param.K_MAX_PML, param.ALPHA_MAX_PML, param.vp_ref,
         param.Rcoef, param.use_pml, *[x.ctypes.data_as(C.c_void_p) for x in a])
    return tuple(x.reshape(2, -1) for x in a)


def elastic_one_step(param: ElasticPropagatorParams, rho, lam, mu, state, profiles,
                     srci=None, srcj=None, srcv=None, srctype=None):
    """one_step of src/Core.jl:215-228 on CUDA tensors, float64 (the reference's
    precision) or float32 (the dtype of `state` decides).  state: (13, N)
    (vx, vy, sxx, syy, sxy, mem[1..8]); profiles: (ax, bx, kx, ay, by, ky);
    srcv: this step's (nsrc,) values.  Returns the new (13, N) state."""
    NX, NY = param.NX, param.NY
    ts = [rho, lam, mu, state]
    _require_cuda(*ts)
    dt_ = torch.float32 if state.dtype == torch.float32 else torch.float64
    state = state.contiguous().to(dt_)
    out = torch.empty_like(state)
    ax, bx, kx, ay, by, ky = [torch.as_tensor(p, device=state.device).to(dt_).contiguous()
                              for p in profiles]
    if srci is not None and len(srci):
        dev = state.device
        si = torch.as_tensor(np.asarray(srci), dtype=torch.int64, device=dev)
        sj = torch.as_tensor(np.asarray(srcj), dtype=torch.int64, device=dev)
        stp = torch.as_tensor(np.asarray(srctype), dtype=torch.int64, device=dev)
        sv = torch.as_tensor(srcv, device=dev).to(dt_).contiguous()
        nsrc = len(srci)
    else:
        si = sj = stp = sv = None
        nsrc = 0
    lam, mu, rho = (t.contiguous().to(dt_) for t in (lam, mu, rho))
    name = "ads_elastic_step_fwd_f64" if dt_ == torch.float64 else "ads_elastic_step_fwd_f32"
    call(name, _ptr(state), _ptr(out), _ptr(lam), _ptr(mu), _ptr(rho), _ptr(ax), _ptr(bx),
         _ptr(kx), _ptr(ay), _ptr(by), _ptr(ky), param.DELTAT, param.DELTAX, param.DELTAY, NX,
         NY, _ptr(si), _ptr(sj), _ptr(stp), _ptr(sv), nsrc, _stream())
    return out


def elastic_one_step_grad(param: ElasticPropagatorParams, rho, lam, mu, state, grad_out,
                          profiles):
    """Transpose of elastic_one_step about `state` (float64 or float32, as
    `state`): returns (grad_state, grad_lambda, grad_mu, grad_rho)."""
    dev = state.device
    dt_ = torch.float32 if state.dtype == torch.float32 else torch.float64
    state = state.contiguous().to(dt_)
    gout = grad_out.contiguous().to(dt_)
    gin = torch.empty_like(state)
    N = state.shape[-1]
    gl, gm, gr = (torch.zeros(N, dtype=dt_, device=dev) for _ in range(3))
    ax, bx, kx, ay, by, ky = [torch.as_tensor(p, device=dev).to(dt_).contiguous()
                              for p in profiles]
    lam, mu, rho = (t.contiguous().to(dt_) for t in (lam, mu, rho))
    name = "ads_elastic_step_bwd_f64" if dt_ == torch.float64 else "ads_elastic_step_bwd_f32"
    call(name, _ptr(state), _ptr(gout), _ptr(gin), _ptr(gl), _ptr(gm), _ptr(gr), _ptr(lam),
         _ptr(mu), _ptr(rho), _ptr(ax), _ptr(bx), _ptr(ay), _ptr(by), param.DELTAT,
         param.DELTAX, param.DELTAY, param.NX, param.NY, _stream())
    return gin, gl, gm, gr


class ElasticPlan:
    """Persistent multi-shot elastic plan: forward traces, misfit and the
    gradient w.r.t. lambda, mu, rho.  shots: list of dicts with srci, srcj,
    srctype, srcv (NSTEP, nsrc), rcvi, rcvj, rcvtype.  resident_segments /
    resident_mem_pct: how many of the last checkpoint segments keep their
    per-step adjoint inputs on the device instead of being recomputed (-1
    none, 0 as many as fit in resident_mem_pct percent, default 50, of the
    free device memory).  source_gradient: the reverse sweep also records
    d loss / d srcv (gradient(..., want_source_grad=True)); the plan then
    rejects (AdsError) sources on the padded frame, the cells the stencil of
    their field does not update.  adjoint_passes: 1 runs each adjoint step
    as one fused pass, 3 as the three gather passes, 0 (default) the fused
    pass for FP32 plans and the three passes for FP64 plans."""

    def __init__(self, param: ElasticPropagatorParams, shots, precision="f64",
                 use_graph=True, ckpt_every=0, stream=None, rows_per_warp=0,
                 resident_segments=0, resident_mem_pct=0, source_gradient=False,
                 autotune=False, adjoint_passes=0):
        cfg = _lib.ElasticConfig()
        cfg.NX, cfg.NY, cfg.NSTEP = param.NX, param.NY, param.NSTEP
        cfg.dx, cfg.dy, cfg.dt = param.DELTAX, param.DELTAY, param.DELTAT
        cfg.npml, cfg.npower, cfg.k_max = param.NPOINTS_PML, param.NPOWER, param.K_MAX_PML
        cfg.alpha_max, cfg.vp_ref, cfg.Rcoef = param.ALPHA_MAX_PML, param.vp_ref, param.Rcoef
        cfg.use_pml = param.use_pml
        cfg.precision = ADS_F64 if precision == "f64" else ADS_F32
        cfg.use_graph = int(bool(use_graph))
        cfg.ckpt_every = ckpt_every
        cfg.rows_per_warp = int(rows_per_warp)
        cfg.resident_segments = int(resident_segments)
        cfg.resident_mem_pct = int(resident_mem_pct)
        cfg.source_gradient = int(bool(source_gradient))
        cfg.autotune = int(bool(autotune))
        cfg.adjoint_passes = int(adjoint_passes)
        self.param = param
        self.dtype = torch.float64 if precision == "f64" else torch.float32
        self._keep = []
        arr = (_lib.ElasticShot * len(shots))()
        for k, s in enumerate(shots):
            vals = [np.ascontiguousarray(s[n], dtype=np.int64)
                    for n in ("srci", "srcj", "srctype", "rcvi", "rcvj", "rcvtype")]
            nsrc = len(vals[0])
            srcv = np.ascontiguousarray(s["srcv"], dtype=np.float64)
            srcv = srcv.reshape(-1, nsrc) if nsrc else np.zeros((0, 1))
            self._keep += vals + [srcv]
            a = arr[k]
            a.nsrc = nsrc
            a.srci, a.srcj, a.srctype = (v.ctypes.data for v in vals[:3])
            a.srcv, a.srcv_rows = srcv.ctypes.data, srcv.shape[0] if nsrc else 0
            a.nrcv = len(vals[3])
            a.rcvi, a.rcvj, a.rcvtype = (v.ctypes.data for v in vals[3:])
        self.shots = shots
        h = C.c_void_p()
        call("ads_elastic_plan_create", C.byref(h), C.byref(cfg), arr, len(shots),
             stream if stream is not None else _stream())
        self._h = h
        self._cfg, self._arr = cfg, arr  # what the one-shot entry points take
        L = lib()
        self.trace_count = L.ads_elastic_plan_trace_count(h)
        self.trace_offsets = [L.ads_elastic_plan_trace_offset(h, k) for k in range(len(shots))]
        self.device_bytes = L.ads_elastic_plan_device_bytes(h)
        self.launches_forward = L.ads_elastic_plan_launches(h, 0)
        self.launches_gradient = L.ads_elastic_plan_launches(h, 1)
        self.resident_segments = L.ads_elastic_plan_resident_segments(h)
        self.rows_per_warp = L.ads_elastic_plan_rows(h, 0)
        self.rows_per_tile = L.ads_elastic_plan_rows(h, 1)
        # fused adjoint warp items per shot: CPML-free, rows, columns, both
        self.adjoint_items = [L.ads_elastic_plan_rows(h, k) for k in range(2, 6)]

    def close(self):
        if getattr(self, "_h", None):
            lib().ads_elastic_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def split_traces(self, packed):
        nt = self.param.NSTEP + 1
        out = []
        for k, s in enumerate(self.shots):
            n = len(s["rcvi"]) * nt
            o = self.trace_offsets[k]
            out.append(packed[o:o + n].view(len(s["rcvi"]), nt))
        return out

    def pack(self, per_shot):
        return torch.cat([t.reshape(-1).to(self.dtype) for t in per_shot])

    def forward(self, lam, mu, rho):
        _require_cuda(lam, mu, rho)
        lam, mu, rho = (t.contiguous().to(torch.float64) for t in (lam, mu, rho))
        tr = torch.empty(max(self.trace_count, 1), dtype=self.dtype, device=lam.device)
        call("ads_elastic_plan_forward", self._h, _ptr(lam), _ptr(mu), _ptr(rho), _ptr(tr),
             _stream())
        return tr[:self.trace_count]

    KERNELS = ("step", "step_store", "adj1", "adj2", "adj3", "src_rcv", "resid")

    def profile(self, lam, mu, rho):
        """Per-kernel durations on this plan's buffers (ads_elastic_plan_profile):
        {kernel: (ms per launch, interior cell-updates per launch)}."""
        import numpy as np

        _require_cuda(lam, mu, rho)
        lam, mu, rho = (t.contiguous().to(torch.float64) for t in (lam, mu, rho))
        out = np.zeros(2 * len(self.KERNELS))
        call("ads_elastic_plan_profile", self._h, _ptr(lam), _ptr(mu), _ptr(rho),
             out.ctypes.data_as(C.c_void_p), _stream())
        return {k: (float(out[2 * i]), float(out[2 * i + 1])) for i, k in enumerate(self.KERNELS)}

    def set_source_values(self, shot, srcv):
        """Replace shot `shot`'s source wavelets in place (same cells and types,
        no plan rebuild): srcv is a CUDA tensor of at least (NSTEP, nsrc), as at
        creation.  Ordered on the current stream, like the plan's calls."""
        _require_cuda(srcv)
        v = srcv
        if 0 <= shot < len(self.shots):  # (the library rejects other indices)
            n, m = int(self.param.NSTEP), len(self.shots[shot]["srci"])
            if m:
                v = srcv.to(torch.float64).reshape(-1, m)[:n].contiguous()
                if v.shape[0] < n:
                    raise ValueError(f"srcv has {v.shape[0]} rows, NSTEP = {n}")
        call("ads_elastic_plan_set_source_values", self._h, shot, _ptr(v), _stream())

    def gradient(self, lam, mu, rho, observed, want_traces=False, want_source_grad=False):
        """(loss, grad_lambda, grad_mu, grad_rho[, traces][, grad_srcv]): grad_srcv is
        a list of per-shot (NSTEP, nsrc) FP64 tensors, d loss / d srcv (the gradient
        AddSource's backward gives, AddSource.cpp:91-155); needs source_gradient."""
        _require_cuda(lam, mu, rho, observed)
        lam, mu, rho = (t.contiguous().to(torch.float64) for t in (lam, mu, rho))
        obs = observed.contiguous().to(self.dtype)
        loss = torch.empty(1, dtype=torch.float64, device=lam.device)
        gl, gm, gr = (torch.empty_like(lam) for _ in range(3))
        tr = (torch.empty(max(self.trace_count, 1), dtype=self.dtype, device=lam.device)
              if want_traces else None)
        if want_source_grad:
            T = self.param.NSTEP
            total = sum(T * len(s["srci"]) for s in self.shots)
            gs = torch.zeros(max(total, 1), dtype=torch.float64, device=lam.device)
            call("ads_elastic_plan_gradient_ex", self._h, _ptr(lam), _ptr(mu), _ptr(rho),
                 _ptr(obs), _ptr(loss), _ptr(gl), _ptr(gm), _ptr(gr), _ptr(gs), _ptr(tr),
                 _stream())
            L = lib()
            per_shot = []
            for k, s in enumerate(self.shots):
                o = L.ads_elastic_plan_source_offset(self._h, k)
                m = len(s["srci"])
                per_shot.append(gs[o:o + T * m].view(T, m))
            out = (loss[0], gl, gm, gr) + ((tr[:self.trace_count],) if want_traces else ())
            return out + (per_shot,)
        call("ads_elastic_plan_gradient", self._h, _ptr(lam), _ptr(mu), _ptr(rho), _ptr(obs),
             _ptr(loss), _ptr(gl), _ptr(gm), _ptr(gr), _ptr(tr), _stream())
        if want_traces:
            return loss[0], gl, gm, gr, tr[:self.trace_count]
        return loss[0], gl, gm, gr


class ElasticMisfit(torch.autograd.Function):
    """loss = sum((traces(lambda, mu, rho) - observed)^2) as an autograd node
    whose backward is the elastic plan's checkpointed adjoint (the gradient TF
    builds in src/Utils.jl:312 for elastic sources): apply(lam, mu, rho, plan,
    observed)."""

    @staticmethod
    def forward(ctx, lam, mu, rho, plan: ElasticPlan, observed):
        loss, gl, gm, gr = plan.gradient(lam, mu, rho, observed)
        ctx.save_for_backward(gl, gm, gr)
        ctx.dtypes = (lam.dtype, mu.dtype, rho.dtype)
        return loss

    @staticmethod
    def backward(ctx, g):
        grads = ctx.saved_tensors
        return tuple((g * x).to(d) for x, d in zip(grads, ctx.dtypes)) + (None, None)


class ElasticPropagator:
    """Result handle of ElasticPropagatorSolver (src/Struct.jl:64-73).
    Receiver traces come from SimulatedObservation without any history.  The
    reference's vx, vy, sigmaxx, sigmayy, sigmaxy ((NSTEP+1, NX+2, NY+2)
    histories) and mem ((NSTEP+1, 8, NX+2, NY+2)) are formed on first access
    by the FP64 single-step operator (the loop of src/Core.jl:31-94: slot 0
    zero, slot n = one_step of slot n-1 with source row n-1) and kept on the
    device."""

    def __init__(self, param, src, rho, lam, mu, precision):
        self.param, self.src, self.rho, self.lam, self.mu = param, src, rho, lam, mu
        self.precision = precision
        self._hist = None

    def _history(self):
        if self._hist is None:
            p = self.param
            dev = torch.device("cuda")
            f = lambda a: torch.as_tensor(a, dtype=torch.float64,
                                          device=dev).reshape(-1).contiguous()
            rho, lam, mu = f(self.rho), f(self.lam), f(self.mu)
            prof = [torch.as_tensor(a, dtype=torch.float64, device=dev).contiguous()
                    for a in compute_PML_Params(p)]
            s = self.src
            nsrc = len(s.srci)
            sv = (torch.as_tensor(np.asarray(s.srcv, np.float64).reshape(-1, nsrc),
                                  device=dev) if nsrc else None)
            H = torch.zeros(p.NSTEP + 1, 13, (p.NX + 2) * (p.NY + 2), dtype=torch.float64,
                            device=dev)
            for n in range(1, p.NSTEP + 1):
                H[n] = elastic_one_step(p, rho, lam, mu, H[n - 1], prof, s.srci, s.srcj,
                                        sv[n - 1] if nsrc else None, s.srctype)
            self._hist = H.view(p.NSTEP + 1, 13, p.NX + 2, p.NY + 2)
        return self._hist

    vx = property(lambda self: self._history()[:, 0])
    vy = property(lambda self: self._history()[:, 1])
    sigmaxx = property(lambda self: self._history()[:, 2])
    sigmayy = property(lambda self: self._history()[:, 3])
    sigmaxy = property(lambda self: self._history()[:, 4])
    mem = property(lambda self: self._history()[:, 5:])


def ElasticPropagatorSolver(param: ElasticPropagatorParams, src: ElasticSource, rho, lam, mu,
                            precision="f64"):
    """src/Core.jl:31-94 (argument order rho, lambda, mu as the reference)."""
    return ElasticPropagator(param, src, rho, lam, mu, precision)


def _eshot(src, rcv):
    return dict(srci=src.srci, srcj=src.srcj, srctype=src.srctype, srcv=src.srcv,
                rcvi=rcv.rcvi, rcvj=rcv.rcvj, rcvtype=rcv.rcvtype)


def SimulatedObservation(ep: ElasticPropagator, rcv: ElasticReceiver):
    """src/Core.jl:701-712: rcv.rcvv = (nrcv, NSTEP+1) traces."""
    plan = ElasticPlan(ep.param, [_eshot(ep.src, rcv)], precision=ep.precision,
                       use_graph=False)
    dev = "cuda"
    f = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev).reshape(-1)
    tr = plan.forward(f(ep.lam), f(ep.mu), f(ep.rho))
    torch.cuda.current_stream().synchronize()
    plan.close()
    rcv.rcvv = tr.view(len(rcv.rcvi), ep.param.NSTEP + 1)
    return rcv.rcvv


def _batched_plan(param, srcs, rcvs, precision, ckpt_every=0):
    return ElasticPlan(param, [_eshot(s, r) for s, r in zip(srcs, rcvs)], precision=precision,
                       use_graph=False, ckpt_every=ckpt_every)


def _materials(model):
    """(rho, lambda, mu) in the reference's argument order -> FP64 CUDA vectors."""
    rho, lam, mu = model
    f = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda").reshape(-1)
    return f(lam), f(mu), f(rho)


def compute_forward_GPU(param: ElasticPropagatorParams, srcs, rcvs, model, precision="f64"):
    """src/Utils.jl:574-601 with elastic sources, one GPU: every shot's
    (nrcv, NSTEP+1) traces from one batched plan; model = (rho, lambda, mu)."""
    plan = _batched_plan(param, srcs, rcvs, precision)
    tr = plan.forward(*_materials(model))
    out = [t.clone() for t in plan.split_traces(tr)]
    torch.cuda.current_stream().synchronize()
    plan.close()
    return out


def compute_loss_and_grads_GPU(param: ElasticPropagatorParams, srcs, rcvs, Rs, model,
                               precision="f64", ckpt_every=0, aux_loss=None, as_lists=False):
    """src/Utils.jl:300-332 with elastic sources, one GPU: loss = sum over
    shots of sum((rcvv - Rs)^2) and its gradients with respect to lambda, mu
    and rho, all shots in one batched plan; model = (rho, lambda, mu), Rs per
    shot (nrcv, NSTEP+1).  Returns (loss, grad_lambda, grad_mu, grad_rho), the
    gradients shaped like lambda; compute_properties_grad turns them into
    vp / vs / rho gradients.  aux_loss: an extra term added to the loss (a
    float, or a callable model -> (value, (d/d lambda, d/d mu, d/d rho))), as
    the reference's aux_loss (src/Utils.jl:309-311).  as_lists: the loss and
    the gradient tuple as the one-GPU lists the reference returns."""
    plan = _batched_plan(param, srcs, rcvs, precision, ckpt_every)
    obs = plan.pack([torch.as_tensor(r, device="cuda") for r in Rs])
    loss, *grads = plan.gradient(*_materials(model), obs)
    plan.close()
    shape = tuple(np.shape(model[1]))
    grads = [g.view(shape) for g in grads]
    if aux_loss is not None:
        if callable(aux_loss):
            v, ga = aux_loss(model)
            loss = loss + v
            grads = [g + torch.as_tensor(np.asarray(x), dtype=torch.float64,
                                         device=g.device).view(shape)
                     for g, x in zip(grads, ga)]
        else:
            loss = loss + float(aux_loss)
    torch.cuda.current_stream().synchronize()
    if as_lists:
        return [loss], [tuple(grads)]
    return (loss, *grads)
