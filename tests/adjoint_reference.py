"""Unrolled PyTorch surrogate model the CUDA adjoint is tested against (test infrastructure).

The same step as visual_cortex_gb300/csrc/pv1_adjoint.cu, written with the same float32
operation order (sums over LGN synapses and over spiking I neurons in ascending order), so
that the forward trajectories agree bit for bit and autograd's gradient can be compared with
the hand-written adjoint.
"""
import torch


class SpikeFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, slope):
        ctx.save_for_backward(x)
        ctx.slope = slope
        return (x > 0).to(x.dtype)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        return g / (1.0 + ctx.slope * x.abs()) ** 2, None


def unrolled(patch, W, consts):
    """rates, vbar of AdjointPatch `patch` computed by autograd-visible torch ops."""
    c = patch.cfg
    dev = W.device
    f = torch.float32
    EdE, ErE, dodE, EdI, ErI, dodI = [consts[i] for i in range(6)]
    B, N, bs, nE = c.B, c.N, c.blockSize, c.nE
    nI = bs - nE
    ids = patch.ids.long()
    X = patch.X
    I0 = patch.I0
    isE = (torch.arange(N, device=dev) % bs) < nE
    tref = torch.where(isE, torch.tensor(c.tRefE, device=dev), torch.tensor(c.tRefI, device=dev))
    v = patch.v0.clone()
    gE = torch.zeros(B, N, device=dev, dtype=f)
    hE, gI, hI = gE.clone(), gE.clone(), gE.clone()
    ref = torch.zeros(B, N, device=dev, dtype=torch.int64)
    dt = torch.tensor(c.dt, dtype=f, device=dev)
    half = dt * torch.tensor(0.5, dtype=f, device=dev)
    scale = torch.tensor(float(c.win), dtype=f, device=dev) * dt * torch.tensor(1e-3, dtype=f, device=dev)
    rates, vbars = [], []
    cnt = torch.zeros(B, N, device=dev, dtype=f)
    vsum = torch.zeros(B, N, device=dev, dtype=f)
    Crec = patch.Crec  # [nblock][nI][bs]

    def fcur(v_, gE_, gI_):
        return -c.gL * (v_ - c.vL) - gE_ * (v_ - c.vE) - gI_ * (v_ - c.vI) + I0

    for t in range(c.T):
        gE1 = gE * EdE + hE * dodE * (EdE - ErE)
        hE1 = hE * ErE
        gI1 = gI * EdI + hI * dodI * (EdI - ErI)
        hI1 = hI * ErI
        refr = ref > 0
        k1 = fcur(v, gE, gI)
        v1 = v + dt * k1
        k2 = fcur(v1, gE1, gI1)
        vn = v + half * (k1 + k2)
        s = SpikeFn.apply(vn - c.vThres, c.slope) * (~refr).to(f)
        sd = s.detach()
        vnext = torch.where(refr, torch.full_like(vn, c.vR), vn * (1 - sd) + c.vR * sd)
        ref = torch.where(refr, ref - 1, torch.where(sd > 0, tref.expand(B, N), torch.zeros_like(ref)))
        # inputs at the end of the step
        x = X[:, t, :].to(f)                               # [B][nLGN]
        for k in range(c.K):
            hE1 = hE1 + W[k] * x[:, ids[k]]
        sI = (s if c.rec_grad else sd).view(B, c.nblock, bs)[:, :, nE:]   # [B][nblock][nI]
        hI1v = hI1.view(B, c.nblock, bs)
        for p in range(nI):
            hI1v = hI1v + sI[:, :, p:p + 1] * Crec[None, :, p, :]
        hI1 = hI1v.reshape(B, N)
        v, gE, hE, gI, hI = vnext, gE1, hE1, gI1, hI1
        cnt = cnt + s
        vsum = vsum + vnext
        if (t + 1) % c.win == 0:
            rates.append(cnt / scale)
            vbars.append(vsum / torch.tensor(float(c.win), dtype=f, device=dev))
            cnt = torch.zeros_like(cnt)
            vsum = torch.zeros_like(vsum)
    return torch.stack(rates, 1), torch.stack(vbars, 1)
