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


@pytest.mark.gpu
def test_external_lgn_source_reproduces_the_plans_own_lgn(native):
    """A plan fed its own LGN spike words from a device array (pv1_set_lgn_source) steps exactly
    as the plan that computed them: the V1 rasters are equal bit for bit over 200 steps (the
    first chunk, full persistent chunks with the overlapped LGN copies, and a partial chunk);
    a run past the source's steps fails."""
    torch = pytest.importorskip("torch")
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation
    wl = synth.make_workload("ext-lgn", seed=12, nblock=4, n_lgn=1024, m=20, width=64, height=64, nt=400,
                             far_partners=100, adex_inh=True, nFrame=60)
    T = 200
    a = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        a.set_record(N.REC_SPIKES | N.REC_LGN_SP, T + 1)
        a.run(T)
        sa = a.fetch_spikes(0, T)
        _, lsp, _ = a.fetch_records(0, T, raw=False, lgn_sp=True, lgn_fr=False)
    finally:
        a.close()
    d = torch.from_numpy(np.ascontiguousarray(lsp, np.float32)).to("cuda:0")
    b = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        b.set_lgn_source(d.data_ptr(), 0, T)
        b.set_record(N.REC_SPIKES, T + 1)
        b.run(T)
        np.testing.assert_array_equal(b.fetch_spikes(0, T), sa)
        assert (sa >= 1).sum() > 100
        with pytest.raises(RuntimeError, match="external LGN source"):
            b.run(8)
    finally:
        b.close()
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_simulation_driven_by_the_bf16_lgn_stage(native):
    """V1 steps driven by the BF16 tensor-core LGN stage through pv1_set_lgn_source, and by the
    FP32 CUDA-core form of the same stage: both runs spike, and their V1 rates agree within 10%
    (the BF16 rates differ from FP32 by a fraction of a percent; the spike draws are the same
    generators)."""
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300 import lgn_bf16 as L
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation
    wl = L.make_workload(nCells=1024, size=64, nFrame=24, side=15, T=640, seed=3)
    v1 = synth.make_workload("bf16-driven", seed=13, nblock=2, n_lgn=1024, m=20, width=64, height=64, nt=640,
                             adex_inh=True, nFrame=40)
    assert v1.lgn.nLGN == wl.nCells
    tc = L.LgnTensorCore(wl, fr_every=64)
    rates, lgn = {}, {}
    try:
        for cores in (True, False):
            tc.run(tensor_cores=cores)
            lgn[cores] = int((tc.fetch(spikes=True, rates=False)[1] >= 1).sum())
            sim = Simulation(v1.spec, v1.net, v1.lgn, v1.stim, v1.init, v1.seeds)
            try:
                sim.set_lgn_source(tc.device_spikes(), 0, wl.T)
                sim.set_record(N.REC_SPIKES, wl.T + 1)
                sim.run(wl.T)
                sp = sim.fetch_spikes(0, wl.T)
            finally:
                sim.close()
            rates[cores] = float(np.floor(np.where(sp >= 1, sp, 0)).sum()) / (v1.spec.nV1 * wl.T * wl.dt * 1e-3)
    finally:
        tc.close()
    assert lgn[True] > 300 and lgn[False] > 300, lgn
    assert rates[True] > 0.5 and rates[False] > 0.5, rates
    assert abs(rates[True] - rates[False]) < 0.1 * rates[False], rates
