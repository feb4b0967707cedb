"""The LGN stage on BF16 tensor cores against its FP64 oracle and the FP32 CUDA-core kernel.

Tolerances: the FP32 spatial stage agrees with FP64 to 1e-5 (absolute, |S| <= 1); FP32 rates
to 1e-4 relative; BF16 rates (8-bit mantissas for S and W, FP32 accumulation) to 2e-2 RMS and
1e-1 max relative — the BF16 error is what the form reports, the bound only guards against a
broken contraction (a wrong operand layout gives errors of order 1)."""
import numpy as np
import pytest


def test_frame_weights_cover_the_kernel():
    from visual_cortex_gb300 import lgn_bf16 as L
    wl = L.make_workload(nCells=64, size=48, nFrame=12, side=15, T=300, seed=1)
    # every step's weights sum to the sum of the temporal samples
    sums = wl.W.sum(axis=2).reshape(-1)[:wl.T]
    np.testing.assert_allclose(sums, wl.tw.sum(), rtol=1e-12, atol=1e-15)
    assert np.all(wl.f0 % 8 == 0)
    F = L.frame_of_samples(wl.sched, wl.T)
    assert F.max() + L.PAD < wl.nFext


@pytest.mark.gpu
def test_bf16_tensor_core_rates_against_fp64(native):
    from visual_cortex_gb300 import lgn_bf16 as L
    wl = L.make_workload(nCells=512, size=64, nFrame=24, side=15, T=640, seed=2)
    tc = L.LgnTensorCore(wl, fr_every=8)
    try:
        tc.run(tensor_cores=False)
        S, sp32, fr32 = tc.fetch(S=True, spikes=True)
        tc.run(tensor_cores=True)
        _, sp16, fr16 = tc.fetch(spikes=True)
        tc.run(tensor_cores=True)   # the pipelined tile loop is deterministic run to run
        _, sp16b, fr16b = tc.fetch(spikes=True)
    finally:
        tc.close()
    np.testing.assert_array_equal(sp16, sp16b)
    np.testing.assert_array_equal(fr16, fr16b)
    cells = np.arange(0, wl.nCells, 7)
    steps = np.arange(0, wl.T, 8)
    from oracle.lgn_fp64 import oracle_rates, rate_errors, spatial64
    S64 = spatial64(wl, cells)
    assert np.abs(S[cells] - S64).max() < 1e-5
    ref = oracle_rates(wl, cells, steps)
    e32 = rate_errors(fr32[:, cells], ref)
    e16 = rate_errors(fr16[:, cells], ref)
    assert e32["max_rel"] < 1e-4, e32
    assert e16["rms_rel"] < 2e-2 and e16["max_rel"] < 1e-1, e16
    assert e16["max_rel"] > 0          # the BF16 path is really a different computation
    # spikes are produced on both paths at similar counts
    n16, n32 = int((sp16 >= 1).sum()), int((sp32 >= 1).sum())
    assert n32 > 0 and abs(n16 - n32) < 0.1 * n32 + 10
