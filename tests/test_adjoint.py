"""The hand-written surrogate-gradient adjoint against an unrolled PyTorch surrogate and
against central finite differences (subthreshold, h = 1e-3).

Tolerances: the forward rates and mean potentials equal the unrolled reference exactly (same
float32 operations in the same order); gradients agree with autograd to 2e-3 relative to the
largest entry (different summation order of the backward); finite differences of the float32
forward agree to 3e-2 relative (h = 1e-3 on a loss of O(1))."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _patch(B=2, nblock=2, bs=128, nE=96, K=8, nLGN=96, T=320, seed=0, vThres=-50.0, w=0.6,
           rate=0.01, rec_grad=True, cta_split=0):
    import torch
    from visual_cortex_gb300.adjoint import AdjointConfig, AdjointPatch
    rng = np.random.default_rng(seed)
    cfg = AdjointConfig(B=B, nblock=nblock, blockSize=bs, nE=nE, nLGN=nLGN, K=K, T=T, seg=64, win=160,
                        vThres=vThres, rec_grad=rec_grad, cta_split=cta_split)
    N = cfg.N
    ids = rng.integers(0, nLGN, size=(K, N)).astype(np.int32)
    X = (rng.random((B, T, nLGN)) < rate).astype(np.uint8)
    Crec = (rng.random((nblock, bs - nE, bs)) < 0.2) * rng.uniform(0.05, 0.3, (nblock, bs - nE, bs))
    I0 = rng.uniform(0.0, 0.6, N).astype(np.float32)
    v0 = rng.uniform(-64.0, -52.0, (B, N)).astype(np.float32)
    patch = AdjointPatch(cfg, ids, X, Crec.astype(np.float32), I0, v0)
    W = torch.tensor(rng.uniform(0.2, 1.0, (K, N)) * w, dtype=torch.float32, device="cuda")
    return patch, W


def _taus(requires_grad=True):
    import torch
    tE = torch.tensor(5.0, dtype=torch.float64, device="cuda", requires_grad=requires_grad)
    tI = torch.tensor(7.0, dtype=torch.float64, device="cuda", requires_grad=requires_grad)
    return tE, tI


def test_forward_matches_unrolled_reference(native):
    import torch
    from adjoint_reference import unrolled
    patch, W = _patch()
    tE, tI = _taus(False)
    r, vb = patch.forward(W, tE, tI)
    r2, vb2 = unrolled(patch, W, patch.consts(tE, tI))
    torch.cuda.synchronize()
    assert float(r.sum()) > 0, "the test patch should spike"
    assert torch.equal(r, r2)
    assert torch.equal(vb, vb2)


@pytest.mark.parametrize("rec_grad", [True, False])
def test_gradients_match_unrolled_autograd(native, rec_grad):
    import torch
    from adjoint_reference import unrolled
    patch, W = _patch(seed=1, rec_grad=rec_grad)
    target = torch.rand(patch.cfg.B, patch.cfg.T // patch.cfg.win, patch.cfg.N, device="cuda") * 40
    vt = torch.full_like(target, -55.0)

    def loss_of(rates, vbar):
        return torch.mean((rates - target) ** 2) + 0.1 * torch.mean((vbar - vt) ** 2)

    W1 = W.clone().requires_grad_(True)
    tE, tI = _taus()
    loss_of(*patch.forward(W1, tE, tI)).backward()
    W2 = W.clone().requires_grad_(True)
    tE2, tI2 = _taus()
    loss_of(*unrolled(patch, W2, patch.consts(tE2, tI2))).backward()
    scale = W2.grad.abs().max()
    assert float(scale) > 0
    assert float((W1.grad - W2.grad).abs().max() / scale) < 2e-3
    for a, b in ((tE, tE2), (tI, tI2)):
        assert abs(float(a.grad) - float(b.grad)) <= 2e-3 * abs(float(b.grad)) + 1e-8, (a.grad, b.grad)


def test_finite_differences_subthreshold(native):
    import torch
    patch, W = _patch(seed=2, vThres=1000.0, T=320)
    vt = torch.full((patch.cfg.B, 2, patch.cfg.N), -58.0, device="cuda")

    def loss(Wx, tE, tI):
        _, vb = patch.forward(Wx, tE, tI)
        return torch.mean((vb.double() - vt.double()) ** 2)

    W1 = W.clone().requires_grad_(True)
    tE, tI = _taus()
    L = loss(W1, tE, tI)
    L.backward()
    assert float(L.detach()) > 0
    h = 1e-3
    rng = np.random.default_rng(3)
    # the largest weight gradients (the ones finite differences resolve) and the two taus
    flat = W1.grad.abs().flatten()
    picks = torch.topk(flat, 6).indices.tolist() + [int(i) for i in rng.integers(0, flat.numel(), 2)]
    with torch.no_grad():
        for idx in picks:
            k, n = divmod(idx, W.shape[1])
            Wp, Wm = W.clone(), W.clone()
            Wp[k, n] += h
            Wm[k, n] -= h
            te, ti = _taus(False)
            fd = (float(loss(Wp, te, ti)) - float(loss(Wm, te, ti))) / (2 * h)
            g = float(W1.grad[k, n])
            assert abs(fd - g) <= 3e-2 * max(abs(g), 1e-3 * float(flat.max())), (k, n, fd, g)
        for which in (0, 1):
            te, ti = _taus(False)
            tp = [te.clone(), ti.clone()]
            tm = [te.clone(), ti.clone()]
            tp[which] += h
            tm[which] -= h
            fd = (float(loss(W, *tp)) - float(loss(W, *tm))) / (2 * h)
            g = float((tE, tI)[which].grad)
            assert abs(fd - g) <= 3e-2 * abs(g) + 1e-6, (which, fd, g)


@pytest.mark.parametrize("rec_grad", [True, False])
def test_cluster_split_matches_single_cta(native, rec_grad):
    """A block held by a 2-CTA cluster (ballots, lambda_hI and the recurrent adjoint exchanged
    through distributed shared memory) computes what one CTA computes: identical forward
    outputs; gradients up to the order of their atomic sums (dL/dW sums the trials of the batch
    with float atomics, dL/d(kernel constants) the CTAs with FP64 atomics)."""
    import torch
    out = []
    for split in (1, 2):
        patch, W = _patch(seed=2, rec_grad=rec_grad, cta_split=split)
        target = torch.rand(patch.cfg.B, patch.cfg.T // patch.cfg.win, patch.cfg.N, device="cuda",
                            generator=torch.Generator(device="cuda").manual_seed(5)) * 40
        W1 = W.clone().requires_grad_(True)
        tE, tI = _taus()
        r, vb = patch.forward(W1, tE, tI)
        (torch.mean((r - target) ** 2) + 0.1 * torch.mean((vb + 55.0) ** 2)).backward()
        out.append((r.detach(), vb.detach(), W1.grad, float(tE.grad), float(tI.grad)))
    (r1, v1, g1, e1, i1), (r2, v2, g2, e2, i2) = out
    assert float(r1.sum()) > 0
    assert torch.equal(r1, r2) and torch.equal(v1, v2)
    assert float((g1 - g2).abs().max() / g1.abs().max()) < 1e-5
    assert e1 == pytest.approx(e2, rel=1e-6, abs=1e-9) and i1 == pytest.approx(i2, rel=1e-6, abs=1e-9)
