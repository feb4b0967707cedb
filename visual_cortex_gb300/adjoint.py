"""Surrogate-gradient adjoint behind torch.autograd.Function (the differentiable form).

``AdjointPatch`` holds a batch of trials of a conductance-based LIF patch (sparse LGN->V1
weights, GABA from the block's I neurons, LGN spike counts per step); ``forward(W, tauE, tauI)``
returns per-window firing rates (Hz) and mean membrane potentials, and differentiates with
respect to the LGN->V1 weights W and the AMPA / GABA decay constants through the hand-written
CUDA adjoint (pv1_adj_forward / pv1_adj_backward: checkpoints every `seg` steps, segment
recompute, fast-sigmoid surrogate).  The kernel constants (Ed, Er, dod) are computed here in
torch from the time constants, so autograd carries the chain rule to tauE/tauI.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N

_PF, _PU = C.c_float, C.c_uint32


class AdjProblem(C.Structure):
    _fields_ = [(n, _PU) for n in ("B", "nblock", "blockSize", "nE", "nLGN", "K", "T", "seg", "win")] + \
               [(n, _PF) for n in ("dt", "vL", "vE", "vI", "vR", "vThres", "gL", "slope")] + \
               [("tRefE", _PU), ("tRefI", _PU)] + \
               [(n, _PF) for n in ("EdE", "ErE", "dodE", "EdI", "ErI", "dodI")] + \
               [("recGrad", _PU), ("ctaSplit", _PU)]


class AdjBuffers(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("ids", "W", "X", "Crec", "I0", "v0", "rates", "vbar", "ck", "gR",
                                          "gV", "gW", "gC", "scratch")]


_SIGS = {
    "pv1_adj_checkpoint_floats": ([C.POINTER(AdjProblem)], C.c_uint64),
    "pv1_adj_scratch_floats": ([C.POINTER(AdjProblem)], C.c_uint64),
    "pv1_adj_forward": ([C.POINTER(AdjProblem), C.POINTER(AdjBuffers), C.c_void_p], C.c_int),
    "pv1_adj_backward": ([C.POINTER(AdjProblem), C.POINTER(AdjBuffers), C.c_void_p], C.c_int),
    "pv1_adj_last_error": ([], C.c_char_p),
}
for _n, (_a, _r) in _SIGS.items():
    getattr(N.lib, _n).argtypes = _a
    getattr(N.lib, _n).restype = _r


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed ({N.ERRORS.get(rc, rc)}): {N.lib.pv1_adj_last_error().decode()}")


def kernel_consts(tau_r: torch.Tensor, tau_d: torch.Tensor, dt: float):
    """(Ed, Er, dod) of src/condShape.h:13-41 for one conductance species, differentiable."""
    return torch.exp(-dt / tau_d), torch.exp(-dt / tau_r), tau_r / (tau_d - tau_r)


@dataclass
class AdjointConfig:
    B: int
    nblock: int
    blockSize: int
    nE: int
    nLGN: int
    K: int
    T: int
    seg: int = 64
    win: int = 160                 # 20 ms at 0.125 ms
    dt: float = 0.125
    vL: float = -65.0
    vE: float = 0.0
    vI: float = -75.0
    vR: float = -60.0
    vThres: float = -50.0
    gL: float = 0.05
    slope: float = 5.0
    # gradient through the recurrent I spikes: exact for the surrogate, but it grows without
    # bound over long windows in a strongly inhibitory network; False holds the recurrent
    # spike input constant in the backward (stop-gradient)
    rec_grad: bool = False
    cta_split: int = 0             # CTAs per (trial, block) in a cluster: 0 automatic, 1 or 2
    tRefE: int = 16                # 2 ms
    tRefI: int = 8                 # 1 ms
    tauRE: float = 1.0             # AMPA rise
    tauRI: float = 1.0             # GABA rise

    @property
    def N(self):
        return self.nblock * self.blockSize


class _AdjFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, W, consts, patch):
        cfg = patch.cfg
        prob = patch._problem(consts)
        dev = W.device
        nWin = cfg.T // cfg.win
        rates = torch.empty(cfg.B, nWin, cfg.N, device=dev, dtype=torch.float32)
        vbar = torch.empty_like(rates)
        ck = torch.empty(int(N.lib.pv1_adj_checkpoint_floats(C.byref(prob))), device=dev, dtype=torch.float32)
        Wc = W.detach().contiguous()
        buf = AdjBuffers(ids=_ptr(patch.ids), W=_ptr(Wc), X=_ptr(patch.X), Crec=_ptr(patch.Crec),
                         I0=_ptr(patch.I0), v0=_ptr(patch.v0), rates=_ptr(rates), vbar=_ptr(vbar), ck=_ptr(ck))
        stream = torch.cuda.current_stream(dev).cuda_stream
        _check(N.lib.pv1_adj_forward(C.byref(prob), C.byref(buf), C.c_void_p(stream)), "pv1_adj_forward")
        ctx.save_for_backward(Wc, ck)
        ctx.patch, ctx.prob = patch, prob
        return rates, vbar

    @staticmethod
    def backward(ctx, gR, gV):
        Wc, ck = ctx.saved_tensors
        patch, prob = ctx.patch, ctx.prob
        dev = Wc.device
        gW = torch.zeros_like(Wc)
        gC = torch.zeros(6, device=dev, dtype=torch.float64)
        scratch = torch.empty(int(N.lib.pv1_adj_scratch_floats(C.byref(prob))), device=dev, dtype=torch.float32)
        gR = None if gR is None else gR.contiguous()
        gV = None if gV is None else gV.contiguous()
        buf = AdjBuffers(ids=_ptr(patch.ids), W=_ptr(Wc), X=_ptr(patch.X), Crec=_ptr(patch.Crec),
                         I0=_ptr(patch.I0), v0=_ptr(patch.v0), ck=_ptr(ck), gR=_ptr(gR), gV=_ptr(gV),
                         gW=_ptr(gW), gC=_ptr(gC), scratch=_ptr(scratch))
        stream = torch.cuda.current_stream(dev).cuda_stream
        _check(N.lib.pv1_adj_backward(C.byref(prob), C.byref(buf), C.c_void_p(stream)), "pv1_adj_backward")
        return gW, gC.to(torch.float32), None


class AdjointPatch:
    """Static inputs of the differentiable patch on one GPU (see module docstring)."""

    def __init__(self, cfg: AdjointConfig, ids, X, Crec, I0, v0, device="cuda"):
        self.cfg = cfg
        self.device = torch.device(device)
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=self.device).contiguous()
        self.ids = t(ids, torch.int32)          # [K][N]
        self.X = t(X, torch.uint8)              # [B][T][nLGN]
        self.Crec = t(Crec, torch.float32)      # [nblock][nI][bs]
        self.I0 = t(I0, torch.float32)          # [N]
        self.v0 = t(v0, torch.float32)          # [B][N]
        assert tuple(self.ids.shape) == (cfg.K, cfg.N)
        assert tuple(self.X.shape) == (cfg.B, cfg.T, cfg.nLGN)
        assert int(self.ids.max()) < cfg.nLGN

    def consts(self, tauE: torch.Tensor, tauI: torch.Tensor) -> torch.Tensor:
        c = self.cfg
        dt = c.dt
        trE = torch.as_tensor(c.tauRE, dtype=tauE.dtype, device=tauE.device)
        trI = torch.as_tensor(c.tauRI, dtype=tauI.dtype, device=tauI.device)
        EdE, ErE, dodE = kernel_consts(trE, tauE, dt)
        EdI, ErI, dodI = kernel_consts(trI, tauI, dt)
        return torch.stack([EdE, ErE, dodE, EdI, ErI, dodI]).to(torch.float32)

    def _problem(self, consts: torch.Tensor) -> AdjProblem:
        c = self.cfg
        v = [float(x) for x in consts.detach().cpu().tolist()]
        return AdjProblem(B=c.B, nblock=c.nblock, blockSize=c.blockSize, nE=c.nE, nLGN=c.nLGN, K=c.K, T=c.T,
                          seg=c.seg, win=c.win, dt=c.dt, vL=c.vL, vE=c.vE, vI=c.vI, vR=c.vR, vThres=c.vThres,
                          gL=c.gL, slope=c.slope, tRefE=c.tRefE, tRefI=c.tRefI, EdE=v[0], ErE=v[1],
                          dodE=v[2], EdI=v[3], ErI=v[4], dodI=v[5], recGrad=int(bool(c.rec_grad)),
                          ctaSplit=int(c.cta_split))

    def forward(self, W: torch.Tensor, tauE: torch.Tensor, tauI: torch.Tensor):
        """(rates [B][nWin][N] in Hz, vbar [B][nWin][N] in mV), differentiable in W, tauE, tauI."""
        return _AdjFn.apply(W, self.consts(tauE, tauI), self)


def make_patch(B: int = 16, nblock: int = 4, T: int = 4000, K: int = 30, seed: int = 0,
               n_lgn: int = 2048, w_lgn: float = 0.35, w_inh: float = 0.25, device: str = "cuda"):
    """The 4096-neuron differentiable patch: the synthetic recipe's LGN cells, LGN->V1 wiring
    (K synapses per neuron), within-block I->all weights and tonic drive; the LGN spike counts
    of each trial come from the GB300 LGN stage driven by a grating at the trial's orientation.
    Returns (patch, W0 [K][N] as a float32 numpy array)."""
    from . import _native as NN
    from . import synth
    from .model import Simulation
    wl = synth.make_workload("adjoint", seed=seed, nblock=nblock, n_lgn=n_lgn, m=K, width=64, height=64,
                             nt=T, far_partners=0, adex_inh=False, patch_deg=2.0, nFrame=120, wFF=w_lgn)
    spec, net = wl.spec, wl.net
    nE, bs = spec.nE, spec.blockSize
    cfg = AdjointConfig(B=B, nblock=nblock, blockSize=bs, nE=nE, nLGN=wl.lgn.nLGN, K=K, T=T)
    X = np.zeros((B, T, cfg.nLGN), np.uint8)
    extent = 2 * (max(float(np.max(np.hypot(wl.lgn.xy[:, 0], wl.lgn.xy[:, 1]))),
                      float(np.max(np.abs(wl.lgn.xy)))) * 1.05 + 0.2)
    for b in range(B):
        frames = synth.grating_frames(120, 64, 64, extent, 4.0, 8.0, 0.5, b * math.pi / B, 120)
        stim = synth.Stimulus(frames=frames, init_LMS=(0.5, 0.5, 0.5))
        seeds = synth.Seeds(lgn=seed + 100 * b + 1, cond=seed + 100 * b + 2, trainDepth=2)
        sim = Simulation(spec, net, wl.lgn, stim, wl.init, seeds)
        try:
            done = 0
            while done < T:
                k = min(1000, T - done)
                sim.set_record(NN.REC_LGN_SP, k + 1) if done == 0 else None
                step0 = sim.step
                sim.run(k)
                _, sp, _ = sim.fetch_records(step0, k, raw=False, lgn_sp=True)
                X[b, done:done + k] = np.clip(np.floor(sp), 0, 255).astype(np.uint8)
                done += k
        finally:
            sim.close()
    ids = net.lgnId[:K].astype(np.int32)
    W0 = net.sLGN[:K].astype(np.float32)
    Crec = np.ascontiguousarray(net.conMat[:, 0, nE:, :] * (w_inh / 0.6)).astype(np.float32)
    I0 = (net.tonicDep * 0.0).astype(np.float32)
    rng = np.random.default_rng(seed + 5)
    v0 = rng.uniform(-65.0, -55.0, size=(B, cfg.N)).astype(np.float32)
    return AdjointPatch(cfg, ids, X, Crec, I0, v0, device=device), W0


def rate_loss(rates: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """MSE between the 20 ms-window firing rates and a teacher's."""
    return torch.mean((rates - target) ** 2)


def main(argv=None):
    """``python -m visual_cortex_gb300.adjoint [--batch B] [--steps T]``: forward + adjoint of the
    synthetic patch, printing device times (used for profiling)."""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--steps", type=int, default=4000)
    a = ap.parse_args(argv)
    patch, W0 = make_patch(B=a.batch, T=a.steps)
    W = torch.tensor(W0, device="cuda", requires_grad=True)
    tE = torch.tensor(5.0, dtype=torch.float64, device="cuda", requires_grad=True)
    tI = torch.tensor(7.0, dtype=torch.float64, device="cuda", requires_grad=True)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    r, _ = patch.forward(W, tE, tI)
    ev[1].record()
    rate_loss(r, torch.zeros_like(r)).backward()
    ev[2].record()
    torch.cuda.synchronize()
    print(f"forward {ev[0].elapsed_time(ev[1]):.2f} ms, backward {ev[1].elapsed_time(ev[2]):.2f} ms")


if __name__ == "__main__":
    main()
