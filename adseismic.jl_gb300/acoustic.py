"""Acoustic host API mirroring ADSeismic's src/Struct.jl / src/Core.jl / src/Utils.jl
on top of the C ABI.

Reference names are kept: AcousticPropagatorParams, AcousticSource,
AcousticReceiver, AcousticPropagatorSolver, SimulatedObservation (Julia's
``SimulatedObservation!``) and compute_loss_and_grads_GPU.  Device memory,
streams and autograd come from PyTorch; every computation runs in
libadseismic_gb300.so.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import ADS_F32, ADS_F64, ADS_VARIANT_U, ADS_VARIANT_W, call, lib


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _require_cuda(*ts):
    for t in ts:
        if t is not None and not t.is_cuda:
            raise ValueError("tensors passed to the GPU operators must live on a CUDA device")


@dataclass
class AcousticPropagatorParams:
    """src/Struct.jl:82-121 (same fields and defaults)."""
    NX: int = 101
    NY: int = 641
    NSTEP: int = 2000 * 2
    DELTAX: float = 10.0
    DELTAY: float = 10.0
    DELTAT: float = 2.0e-3 / 2
    USE_PML_XMIN: bool = True
    USE_PML_XMAX: bool = True
    USE_PML_YMIN: bool = True
    USE_PML_YMAX: bool = True
    NPOINTS_PML: int = 12
    NPOWER: int = 2
    damping_x: float = None  # set by compute_PML_Params, as the reference does
    damping_y: float = None
    Rcoef: float = 0.001
    vp_ref: float = 1000.0
    IT_DISPLAY: int = 0
    PropagatorKernel: int = 0

    @property
    def use_pml(self) -> int:
        return (int(self.USE_PML_XMIN) | int(self.USE_PML_XMAX) << 1 |
                int(self.USE_PML_YMIN) << 2 | int(self.USE_PML_YMAX) << 3)


@dataclass
class AcousticSource:
    """src/Struct.jl:123-127; srci/srcj 1-based into the padded grid, srcv (NSTEP, nsrc)."""
    srci: np.ndarray
    srcj: np.ndarray
    srcv: np.ndarray


@dataclass
class AcousticReceiver:
    """src/Struct.jl:129-133; rcvv is filled by SimulatedObservation, (NSTEP+1, nrcv)."""
    rcvi: np.ndarray
    rcvj: np.ndarray
    rcvv: object = None


def compute_PML_Params(param: AcousticPropagatorParams):
    """src/Core.jl:622-655: returns (Sigma_x, Sigma_y) as (NX+2, NY+2) arrays
    and, as the reference does, sets param.damping_x / damping_y to
    vp_ref / L ln(1 / Rcoef) with L the PML thickness along x / y."""
    param.damping_x = param.vp_ref / (param.NPOINTS_PML * param.DELTAX) * np.log(1 / param.Rcoef)
    param.damping_y = param.vp_ref / (param.NPOINTS_PML * param.DELTAY) * np.log(1 / param.Rcoef)
    sx = np.empty(param.NX + 2)
    ty = np.empty(param.NY + 2)
    call("ads_acoustic_pml_profiles", param.NX, param.NY, param.DELTAX, param.DELTAY,
         param.NPOINTS_PML, param.vp_ref, param.Rcoef, param.use_pml,
         sx.ctypes.data_as(C.c_void_p), ty.ctypes.data_as(C.c_void_p))
    Sx = np.repeat(sx[:, None], param.NY + 2, axis=1)
    Sy = np.repeat(ty[None, :], param.NX + 2, axis=0)
    return Sx, Sy


# ------------------------------------------------------------------ single step

def acoustic_one_step(w, wold, phi, psi, sigma, tau, c, dt, hx, hy, NX, NY,
                      variant=ADS_VARIANT_W):
    """AcousticOneStep forward (deps/CustomOps/AcousticOneStep/AcousticOneStep.cpp:14-61)
    on flat CUDA tensors of length (NX+2)(NY+2), float64 or float32."""
    ts = [w, wold, phi, psi, sigma, tau, c]
    _require_cuda(*ts)
    dt_ = w.dtype
    ts = [t.contiguous().to(dt_) for t in ts]
    u, po, qo = (torch.empty_like(ts[0]) for _ in range(3))
    name = "ads_acoustic_step_fwd_f64" if dt_ == torch.float64 else "ads_acoustic_step_fwd_f32"
    call(name, *[_ptr(t) for t in ts], dt, hx, hy, NX, NY, _ptr(u), _ptr(po), _ptr(qo),
         int(variant), _stream())
    return u, po, qo


def acoustic_one_step_grad(gu, gphi, gpsi, w, wold, phi, psi, sigma, tau, c, dt, hx, hy,
                           NX, NY, u, phiout, psiout, variant=ADS_VARIANT_W):
    """AcousticOneStepGrad (AcousticOneStep.cpp:63-93): returns grad_w, grad_wold,
    grad_phi, grad_psi, grad_c (grad_sigma/tau/dt/hx/hy are never produced by the
    reference either)."""
    dt_ = w.dtype
    ins = [t.contiguous().to(dt_) for t in (gu, gphi, gpsi, w, wold, phi, psi, sigma, tau, c)]
    tail = [t.contiguous().to(dt_) for t in (u, phiout, psiout)]
    _require_cuda(*ins, *tail)
    outs = [torch.empty_like(ins[3]) for _ in range(5)]
    name = "ads_acoustic_step_bwd_f64" if dt_ == torch.float64 else "ads_acoustic_step_bwd_f32"
    call(name, *[_ptr(t) for t in outs], *[_ptr(t) for t in ins], dt, hx, hy, NX, NY,
         *[_ptr(t) for t in tail], int(variant), _stream())
    return tuple(outs)


class AcousticOneStep(torch.autograd.Function):
    """The custom operator with its registered gradient (load_op_and_grad in
    src/Core.jl:483-502): forward and backward both run the CUDA kernels."""

    @staticmethod
    def forward(ctx, w, wold, phi, psi, sigma, tau, c, dt, hx, hy, NX, NY, variant=0):
        u, po, qo = acoustic_one_step(w, wold, phi, psi, sigma, tau, c, dt, hx, hy, NX, NY,
                                      variant)
        ctx.save_for_backward(w, wold, phi, psi, sigma, tau, c, u, po, qo)
        ctx.k = (dt, hx, hy, NX, NY, variant)
        return u, po, qo

    @staticmethod
    def backward(ctx, gu, gp, gq):
        w, wold, phi, psi, sigma, tau, c, u, po, qo = ctx.saved_tensors
        dt, hx, hy, NX, NY, variant = ctx.k
        z = torch.zeros_like(w)
        gu = z if gu is None else gu
        gp = z if gp is None else gp
        gq = z if gq is None else gq
        gw, gwo, gph, gps, gc = acoustic_one_step_grad(gu, gp, gq, w, wold, phi, psi, sigma,
                                                       tau, c, dt, hx, hy, NX, NY, u, po, qo,
                                                       variant)
        return gw, gwo, gph, gps, None, None, gc, None, None, None, None, None, None


# ------------------------------------------------------------------ whole path

class AcousticPlan:
    """A persistent multi-shot plan (forward traces, misfit, gradient).

    shots: list of dicts with keys x0, nx, nstep, srci, srcj, srcv, rcvi, rcvj
    (window-local, 1-based indices).  The model vp is (MX+2, MY+2).
    resident_segments / resident_mem_pct: how many of the last checkpoint
    segments keep their forward wavefields on the device instead of being
    recomputed in the reverse sweep (-1 none, 0 as many as fit in
    resident_mem_pct percent, default 50, of the free device memory).
    variant: ADS_VARIANT_W (the custom operators' form, phi / psi from the old
    field; PropagatorKernel 1 and 2) or ADS_VARIANT_U (one_step, phi / psi
    from the new field; PropagatorKernel 0, the reference's default).
    tma (FP32): 1 runs the interior forward steps through tensor-map tile
    copies where the driver supports them, 0 (default) through the
    register-queue kernel; the results are identical."""

    def __init__(self, MX, MY, dx, dy, dt, shots, npml=12, Rcoef=0.001, vp_ref=1000.0,
                 use_pml=15, precision="f64", use_graph=True, ckpt_every=0,
                 rows_per_thread=0, steps_per_block=0, block_rows=0, autotune=False,
                 resident_segments=0, resident_mem_pct=0, stream=None,
                 variant=ADS_VARIANT_W, tma=0):
        cfg = _lib.AcousticConfig()
        cfg.MX, cfg.MY, cfg.dx, cfg.dy, cfg.dt = MX, MY, dx, dy, dt
        cfg.npml, cfg.Rcoef, cfg.vp_ref, cfg.use_pml = npml, Rcoef, vp_ref, use_pml
        cfg.precision = ADS_F64 if precision == "f64" else ADS_F32
        cfg.variant = int(variant)
        cfg.use_graph = int(bool(use_graph))
        cfg.ckpt_every = ckpt_every
        cfg.rows_per_thread = rows_per_thread
        cfg.steps_per_block = steps_per_block
        cfg.block_rows = block_rows
        cfg.autotune = int(autotune)
        cfg.resident_segments = int(resident_segments)
        cfg.resident_mem_pct = int(resident_mem_pct)
        cfg.tma = int(tma)
        self.MX, self.MY = MX, MY
        self.precision = precision
        self.dtype = torch.float64 if precision == "f64" else torch.float32
        self._keep = []
        arr = (_lib.AcousticShot * len(shots))()
        for k, s in enumerate(shots):
            srci = np.ascontiguousarray(s["srci"], dtype=np.int64)
            srcj = np.ascontiguousarray(s["srcj"], dtype=np.int64)
            srcv = np.ascontiguousarray(s["srcv"], dtype=np.float64)
            srcv = srcv.reshape(-1, len(srci)) if len(srci) else np.zeros((0, 1))
            rcvi = np.ascontiguousarray(s["rcvi"], dtype=np.int64)
            rcvj = np.ascontiguousarray(s["rcvj"], dtype=np.int64)
            self._keep += [srci, srcj, srcv, rcvi, rcvj]
            a = arr[k]
            a.x0, a.nx, a.nstep = s.get("x0", 0), s["nx"], s["nstep"]
            a.nsrc = len(srci)
            a.srci, a.srcj = srci.ctypes.data, srcj.ctypes.data
            a.srcv, a.srcv_rows = srcv.ctypes.data, srcv.shape[0] if len(srci) else 0
            a.nrcv = len(rcvi)
            a.rcvi, a.rcvj = rcvi.ctypes.data, rcvj.ctypes.data
        self.nshots = len(shots)
        self.shots = shots
        h = C.c_void_p()
        st = stream if stream is not None else _stream()
        call("ads_acoustic_plan_create", C.byref(h), C.byref(cfg), arr, len(shots), st)
        self._h = h
        self._cfg, self._arr = cfg, arr  # what the one-shot entry points take
        L = lib()
        self.trace_count = L.ads_acoustic_plan_trace_count(h)
        self.trace_offsets = [L.ads_acoustic_plan_trace_offset(h, k) for k in range(len(shots))]
        self.device_bytes = L.ads_acoustic_plan_device_bytes(h)
        self.launches_forward = L.ads_acoustic_plan_launches(h, 0)
        self.launches_gradient = L.ads_acoustic_plan_launches(h, 1)
        self.resident_segments = L.ads_acoustic_plan_resident_segments(h)
        self.steps_per_block = L.ads_acoustic_plan_steps_per_block(h)
        self.uses_tma = bool(L.ads_acoustic_plan_tma(h) == 1)
        # rows per warp of the step items: forward / adjoint interior, forward / adjoint PML
        self.rows = tuple(int(L.ads_acoustic_plan_rows(h, w)) for w in range(4))

    def device_status(self):
        """Raise AdsError (ADS_ERR_TIMEOUT) if a bounded wait of the plan's
        kernels has run out since its creation; synchronises the stream."""
        call("ads_acoustic_plan_device_status", self._h, _stream())

    def close(self):
        if getattr(self, "_h", None):
            lib().ads_acoustic_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def profile(self, vp, observed):
        """One gradient with direct launches and device-timed ranges:
        {'forward'|'recompute'|'adjoint': (ms, launches, interior cell-steps)}."""
        _require_cuda(vp, observed)
        vp = vp.contiguous().to(torch.float64)
        obs = observed.contiguous().to(self.dtype)
        out = np.zeros(9)
        call("ads_acoustic_plan_profile", self._h, _ptr(vp), _ptr(obs),
             out.ctypes.data_as(C.c_void_p), _stream())
        return {k: tuple(out[3 * i:3 * i + 3])
                for i, k in enumerate(("forward", "recompute", "adjoint"))}

    def split_traces(self, packed):
        """Packed trace buffer -> list of (nstep+1, nrcv) views per shot."""
        out = []
        for k, s in enumerate(self.shots):
            n = (s["nstep"] + 1) * len(s["rcvi"])
            o = self.trace_offsets[k]
            out.append(packed[o:o + n].view(s["nstep"] + 1, len(s["rcvi"])))
        return out

    def pack(self, per_shot):
        return torch.cat([t.reshape(-1).to(self.dtype) for t in per_shot])

    def forward(self, vp):
        _require_cuda(vp)
        vp = vp.contiguous().to(torch.float64)
        tr = torch.empty(max(self.trace_count, 1), dtype=self.dtype, device=vp.device)
        call("ads_acoustic_plan_forward", self._h, _ptr(vp), _ptr(tr), _stream())
        return tr[:self.trace_count]

    def set_source_values(self, shot, srcv):
        """Replace shot `shot`'s source wavelets in place (same cells, no plan
        rebuild): srcv is a CUDA tensor of at least (nstep, nsrc), as at
        creation.  Ordered on the current stream, like the plan's calls."""
        _require_cuda(srcv)
        v = srcv
        if 0 <= shot < len(self.shots):  # (the library rejects other indices)
            s = self.shots[shot]
            n, m = int(s["nstep"]), len(s["srci"])
            if m:
                v = srcv.to(torch.float64).reshape(-1, m)[:n].contiguous()
                if v.shape[0] < n:
                    raise ValueError(f"srcv has {v.shape[0]} rows, shot {shot} needs {n}")
        call("ads_acoustic_plan_set_source_values", self._h, shot, _ptr(v), _stream())

    def gradient(self, vp, observed, want_traces=False, want_source_grad=False):
        """(loss, grad_vp[, traces][, grad_srcv]): grad_srcv is a list of per-shot
        (nstep, nsrc) FP64 tensors, d loss / d srcv (the gradient the reference's
        ScatterAdd backward gives a variable source, src/Utils.jl:603-640)."""
        _require_cuda(vp, observed)
        vp = vp.contiguous().to(torch.float64)
        obs = observed.contiguous().to(self.dtype)
        loss = torch.empty(1, dtype=torch.float64, device=vp.device)
        grad = torch.empty_like(vp)
        tr = (torch.empty(max(self.trace_count, 1), dtype=self.dtype, device=vp.device)
              if want_traces else None)
        if want_source_grad:
            total = sum(int(s["nstep"]) * len(s["srci"]) for s in self.shots)
            gs = torch.zeros(max(total, 1), dtype=torch.float64, device=vp.device)
            call("ads_acoustic_plan_gradient_ex", self._h, _ptr(vp), _ptr(obs), _ptr(loss),
                 _ptr(grad), _ptr(gs), _ptr(tr), _stream())
            L = lib()
            per_shot = []
            for k, s in enumerate(self.shots):
                o = L.ads_acoustic_plan_source_offset(self._h, k)
                n, m = int(s["nstep"]), len(s["srci"])
                per_shot.append(gs[o:o + n * m].view(n, m))
            out = (loss[0], grad) + ((tr[:self.trace_count],) if want_traces else ())
            return out + (per_shot,)
        call("ads_acoustic_plan_gradient", self._h, _ptr(vp), _ptr(obs), _ptr(loss), _ptr(grad),
             _ptr(tr), _stream())
        if want_traces:
            return loss[0], grad, tr[:self.trace_count]
        return loss[0], grad


class AcousticPropagator:
    """Result handle of AcousticPropagatorSolver (src/Struct.jl:140-147).
    Receiver traces come from SimulatedObservation without any history (the
    plans keep O(1) steps per shot, in the form PropagatorKernel selects).
    The reference's u, phi and psi fields, the (NSTEP+1, NX+2, NY+2)
    histories, are formed on first access by the FP64 single-step operator
    chain in that form, and kept on the device."""

    def __init__(self, param, src, vp, precision):
        self.param, self.src, self.vp, self.precision = param, src, vp, precision
        self._hist = None

    def _history(self):
        if self._hist is None:
            p = self.param
            none = AcousticReceiver(np.zeros(0, np.int64), np.zeros(0, np.int64))
            U, Ph, Qh = _chain_forward(p, self.src, none, self.vp)[1][:3]
            shape = (p.NSTEP + 1, p.NX + 2, p.NY + 2)
            self._hist = (U.view(shape), Ph.view(shape), Qh.view(shape))
        return self._hist

    @property
    def u(self):
        return self._history()[0]

    @property
    def phi(self):
        return self._history()[1]

    @property
    def psi(self):
        return self._history()[2]


def step_variant(param: AcousticPropagatorParams) -> int:
    """The one-step form param.PropagatorKernel selects (src/Core.jl:580-591):
    0 runs one_step (src/Core.jl:528-549: phi, psi from the new u,
    ADS_VARIANT_U); 1 the custom operator and 2 its TF restatement
    acoustic_one_step_customop_ref (src/Core.jl:504-525), both with phi, psi
    from the old w (ADS_VARIANT_W)."""
    if param.PropagatorKernel not in (0, 1, 2):
        raise ValueError("PropagatorKernel must be 0, 1 or 2")
    return ADS_VARIANT_U if param.PropagatorKernel == 0 else ADS_VARIANT_W


def AcousticPropagatorSolver(param: AcousticPropagatorParams, src: AcousticSource, vp,
                             precision="f64"):
    """src/Core.jl:562-620 (c = vp^2, PML from param, zero initial slots), in
    the form param.PropagatorKernel selects; traces and gradients run on the
    batched plans."""
    step_variant(param)
    return AcousticPropagator(param, src, vp, precision)


def _shot_dict(param, src, rcv):
    return dict(x0=0, nx=param.NX, nstep=param.NSTEP, srci=src.srci, srcj=src.srcj,
                srcv=src.srcv, rcvi=rcv.rcvi, rcvj=rcv.rcvj)


def SimulatedObservation(ap: AcousticPropagator, rcv: AcousticReceiver):
    """src/Core.jl:726-730: fills rcv.rcvv with the (NSTEP+1, nrcv) traces."""
    p = ap.param
    plan = AcousticPlan(p.NX, p.NY, p.DELTAX, p.DELTAY, p.DELTAT, [_shot_dict(p, ap.src, rcv)],
                        npml=p.NPOINTS_PML, Rcoef=p.Rcoef, vp_ref=p.vp_ref,
                        use_pml=p.use_pml, precision=ap.precision, use_graph=False,
                        variant=step_variant(p))
    vp = torch.as_tensor(ap.vp, dtype=torch.float64, device="cuda").reshape(p.NX + 2, p.NY + 2)
    tr = plan.forward(vp)
    torch.cuda.current_stream().synchronize()
    plan.close()
    rcv.rcvv = tr.view(p.NSTEP + 1, len(rcv.rcvi))
    return rcv.rcvv


def compute_forward_GPU(param: AcousticPropagatorParams, srcs, rcvs, vp, precision="f64"):
    """src/Utils.jl:574-601 for one GPU: every shot's (NSTEP+1, nrcv) traces
    from one batched plan.  With ElasticPropagatorParams the model is
    (rho, lambda, mu), as the reference's elastic solver takes it."""
    if not isinstance(param, AcousticPropagatorParams):
        from .elastic import compute_forward_GPU as elastic_forward

        return elastic_forward(param, srcs, rcvs, vp, precision)
    shots = [_shot_dict(param, s, r) for s, r in zip(srcs, rcvs)]
    plan = AcousticPlan(param.NX, param.NY, param.DELTAX, param.DELTAY, param.DELTAT, shots,
                        npml=param.NPOINTS_PML, Rcoef=param.Rcoef, vp_ref=param.vp_ref,
                        use_pml=param.use_pml, precision=precision, use_graph=False,
                        variant=step_variant(param))
    vp = torch.as_tensor(vp, dtype=torch.float64, device="cuda").reshape(param.NX + 2,
                                                                         param.NY + 2)
    out = [t.clone() for t in plan.split_traces(plan.forward(vp))]
    torch.cuda.current_stream().synchronize()
    plan.close()
    return out


def compute_loss_and_grads_GPU(param: AcousticPropagatorParams, srcs, rcvs, Rs, vp,
                               precision="f64", ckpt_every=0, aux_loss=None, as_lists=False):
    """src/Utils.jl:300-332 for one GPU: loss = sum over shots of sum((rcvv - Rs)^2)
    and its gradient w.r.t. vp, all shots in one batched plan, in the form
    param.PropagatorKernel selects.

    aux_loss: an extra term added to the loss before differentiating (the
    reference's aux_loss, src/Utils.jl:309-311): a float, or a callable
    vp -> (value, d value / d vp) when the term depends on the model.
    as_lists: return ([loss], [grad]), the per-GPU lists the reference returns
    (src/Utils.jl:321-331), here for its one GPU.  With ElasticPropagatorParams
    the model is (rho, lambda, mu) and the result (loss, grad_lambda, grad_mu,
    grad_rho)."""
    if not isinstance(param, AcousticPropagatorParams):
        from .elastic import compute_loss_and_grads_GPU as elastic_grads

        return elastic_grads(param, srcs, rcvs, Rs, vp, precision, ckpt_every, aux_loss,
                             as_lists)
    shots = [_shot_dict(param, s, r) for s, r in zip(srcs, rcvs)]
    plan = AcousticPlan(param.NX, param.NY, param.DELTAX, param.DELTAY, param.DELTAT, shots,
                        npml=param.NPOINTS_PML, Rcoef=param.Rcoef, vp_ref=param.vp_ref,
                        use_pml=param.use_pml, precision=precision, use_graph=False,
                        ckpt_every=ckpt_every, variant=step_variant(param))
    vp = torch.as_tensor(vp, dtype=torch.float64, device="cuda").reshape(param.NX + 2,
                                                                         param.NY + 2)
    obs = plan.pack([torch.as_tensor(r, device="cuda") for r in Rs])
    loss, grad = plan.gradient(vp, obs)
    plan.close()
    if aux_loss is not None:
        if callable(aux_loss):
            v, g = aux_loss(vp)
            loss = loss + v
            grad = grad + torch.as_tensor(g, dtype=torch.float64, device=grad.device)
        else:
            loss = loss + float(aux_loss)
    torch.cuda.current_stream().synchronize()
    if as_lists:
        return [loss], [grad]
    return loss, grad


def _chain_forward(param: AcousticPropagatorParams, src: AcousticSource,
                   rcv: AcousticReceiver, vp):
    """The forward half of the operator chain (src/Core.jl:600-614 and
    SimulatedObservation!, src/Core.jl:726-730): AcousticOneStep in the form
    step_variant(param) selects, then ScatterAdd of the dt^2-scaled source
    row, per step; receivers by one Gather over the history.  Returns the
    packed (NSTEP+1, nrcv) traces and what the reverse half needs."""
    variant = step_variant(param)
    dev = torch.device("cuda")
    NX, NY, T = param.NX, param.NY, param.NSTEP
    S, N = NY + 2, (NX + 2) * (NY + 2)
    dt, hx, hy = param.DELTAT, param.DELTAX, param.DELTAY
    f64 = dict(dtype=torch.float64, device=dev)
    Sx, Sy = compute_PML_Params(param)
    sigma = torch.as_tensor(Sx, **f64).reshape(-1).contiguous()
    tau = torch.as_tensor(Sy, **f64).reshape(-1).contiguous()
    vpt = torch.as_tensor(vp, **f64).reshape(-1).contiguous()
    c = vpt * vpt
    srci, srcj = np.asarray(src.srci, np.int64), np.asarray(src.srcj, np.int64)
    rcvi, rcvj = np.asarray(rcv.rcvi, np.int64), np.asarray(rcv.rcvj, np.int64)
    nsrc, nrcv = len(srci), len(rcvi)
    sii = torch.as_tensor((srci - 1) * S + srcj, device=dev)            # 1-based cells
    upd = torch.as_tensor(np.asarray(src.srcv, np.float64).reshape(-1, nsrc), **f64) * (dt * dt)
    rcell = (rcvi - 1) * S + rcvj                                         # 1-based cells
    hist_ii = torch.as_tensor((np.arange(T + 1)[:, None] * N + rcell[None, :]).reshape(-1),
                              device=dev)
    U = torch.zeros(T + 1, N, **f64)
    Ph = torch.zeros(T + 1, N, **f64)
    Qh = torch.zeros(T + 1, N, **f64)
    st = _stream()
    L = lib()
    P = _ptr
    for k in range(2, T + 1):
        _lib.check(L.ads_acoustic_step_fwd_f64(
            P(U[k - 1]), P(U[k - 2]), P(Ph[k - 1]), P(Qh[k - 1]), P(sigma), P(tau), P(c),
            dt, hx, hy, NX, NY, P(U[k]), P(Ph[k]), P(Qh[k]), variant, st))
        if nsrc:
            _lib.check(L.ads_scatter_add_f64(P(U[k]), P(U[k]), P(sii), P(upd[k - 1]), N,
                                             nsrc, st))
    rcvv = torch.empty((T + 1) * nrcv, **f64)
    if nrcv:
        _lib.check(L.ads_gather_f64(P(rcvv), P(U), P(hist_ii), (T + 1) * nrcv, st))
    return rcvv, (U, Ph, Qh, sigma, tau, c, vpt, rcell, variant)


def dropin_loss_and_grad(param: AcousticPropagatorParams, src: AcousticSource,
                         rcv: AcousticReceiver, observed, vp):
    """The plain FP64 operator chain of one shot, as the reference's graph runs
    it: one C-ABI operator call per op and time step, the whole wavefield
    history kept on the device (TensorFlow keeps every while_loop output for
    its gradient).

    Forward: _chain_forward.  Loss = sum((rcvv - obs)^2) (src/Utils.jl:308).
    Reverse (the gradients call of src/Utils.jl:312): the Gather's transpose
    (a ScatterAdd of the residual), then AcousticOneStepGrad per step in the
    same form; ScatterAdd passes its input gradient through.  PropagatorKernel
    1 or 2 gives the custom operators' chain (the plain FP64 drop-in), 0 the
    one_step form.  Returns (loss, grad_vp) as FP64 CUDA tensors.
    """
    rcvv, (U, Ph, Qh, sigma, tau, c, vpt, rcell, variant) = _chain_forward(param, src, rcv, vp)
    dev = U.device
    NX, NY, T = param.NX, param.NY, param.NSTEP
    N = (NX + 2) * (NY + 2)
    dt, hx, hy = param.DELTAT, param.DELTAX, param.DELTAY
    f64 = dict(dtype=torch.float64, device=dev)
    nrcv = len(rcell)
    rii = torch.as_tensor(rcell, device=dev)
    obs = torch.as_tensor(observed, **f64).reshape(-1)
    resid = 2.0 * (rcvv - obs)
    loss = torch.sum((rcvv - obs) ** 2)
    resid = resid.reshape(T + 1, nrcv).contiguous()
    LU = torch.zeros(3, N, **f64)        # lambdaU of slots k, k-1, k-2 (ring of 3)
    LP = torch.zeros(2, N, **f64)
    LQ = torch.zeros(2, N, **f64)
    gw = torch.empty(N, **f64)
    gcs = torch.empty(N, **f64)
    gc = torch.zeros(N, **f64)
    st = _stream()
    L = lib()
    P = _ptr
    for k in range(T, 1, -1):
        lu = LU[k % 3]
        if nrcv:
            _lib.check(L.ads_scatter_add_f64(P(lu), P(lu), P(rii), P(resid[k]), N, nrcv, st))
        # slot k-2 is first reached by this step (grad_wold); slot k-1 already
        # holds grad_wold of step k+1 and gains grad_w of this step
        _lib.check(L.ads_acoustic_step_bwd_f64(
            P(gw), P(LU[(k - 2) % 3]), P(LP[(k - 1) % 2]), P(LQ[(k - 1) % 2]), P(gcs),
            P(lu), P(LP[k % 2]), P(LQ[k % 2]),
            P(U[k - 1]), P(U[k - 2]), P(Ph[k - 1]), P(Qh[k - 1]), P(sigma), P(tau), P(c),
            dt, hx, hy, NX, NY, P(U[k]), P(Ph[k]), P(Qh[k]), variant, st))
        LU[(k - 1) % 3].add_(gw)
        gc.add_(gcs)
    grad_vp = (gc * 2.0) * vpt
    return loss, grad_vp.reshape(NX + 2, NY + 2)


class AcousticMisfit(torch.autograd.Function):
    """loss = sum((traces(vp) - observed)^2) as an autograd node whose backward is
    the plan's checkpointed adjoint (the gradient TF builds in src/Utils.jl:312)."""

    @staticmethod
    def forward(ctx, vp, plan: AcousticPlan, observed):
        loss, grad = plan.gradient(vp, observed)
        ctx.save_for_backward(grad)
        ctx.dtype = vp.dtype
        return loss

    @staticmethod
    def backward(ctx, gl):
        (grad,) = ctx.saved_tensors
        return (gl * grad).to(ctx.dtype), None, None
