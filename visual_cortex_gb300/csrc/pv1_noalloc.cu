// Allocation-free LGN stepping.
//
// Some callers cannot allocate device memory at the point where they need the LGN stage:
// code running inside a host application's real-time loop or a framework that owns every
// device allocation (a pooling allocator, a memory budget fixed at start-up), or code that
// must not call cudaMalloc because it would synchronise the device.  pv1_lgn_spikes_noalloc
// serves them: it runs the LGN rate and spike kernels for a number of steps, writing into
// device buffers the caller provides, and keeps the only scratch it needs (the rates passed
// from the first kernel to the second, and the step counter the kernels read) in a
// file-scope device array of fixed size instead of allocating it.
//
// The array is created when the library is loaded and stays on every GPU that loads the
// library until the process exits (4 MiB + 256 B).  Every call shares it and it keeps the
// last call's contents; nothing in it has to start at zero, because each call writes every
// slot it reads before reading it.  Calls whose work overlaps on the GPU (two streams, or two
// host threads) race on the array.
#include <mutex>
#include <string>

#include "pv1_internal.cuh"

namespace pv1 {
namespace {

constexpr size_t kNoAllocRateFloats = size_t(1) << 20;            // 4 MiB of rates
constexpr size_t kNoAllocHeadBytes = 256;                          // step counter
constexpr size_t kNoAllocBytes = kNoAllocHeadBytes + kNoAllocRateFloats * sizeof(float);
constexpr int kMaxDevices = 64;
// the rate kernel puts the steps of a call on gridDim.y
constexpr uint32_t kNoAllocMaxSteps = 65535;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_mu;
unsigned char *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `device` (looked up once per device, with that
// device current).  Host code must not pass g_noalloc_scratch itself to a kernel: in host
// code that name is a host-side stand-in, not a device address.
cudaError_t scratch_address(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[device]) {
        int cur = -1;
        cudaError_t e = cudaGetDevice(&cur);
        if (e != cudaSuccess) return e;
        if (cur != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (cur != device) cudaSetDevice(cur);
        if (e != cudaSuccess) return e;
        g_scratch_addr[device] = static_cast<unsigned char *>(ptr);
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

__global__ void set_step_kernel(long long *dst, long long v) { *dst = v; }

// Exact-time Poisson spikes for K steps from the rates in `rates` [K][nLGN], one thread per
// magno cell, with the generator state of the plan carried in registers (get_spike,
// src/discrete_input_convol.cu:1589-1619).  Writes row s of the caller's outputs.
__global__ void __launch_bounds__(256) lgn_spike_rows_kernel(LgnParams P, const long long *stepBase,
                                                             int K, const float *__restrict__ rates,
                                                             float *sinfoOut, float *frOut) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= P.nMagno) return;
    int id = P.nParvo_I + cell;
    if (cell >= P.nMagno_I) id += P.nParvo_C;
    float ltr = P.leftTimeRate[id];
    float lnl = P.lastNegLogRand[id];
    curandStateMRG32k3a st = P.state[id];
    const float dt = P.dt;
    (void)stepBase;
    for (int s = 0; s < K; s++) {
        const float fr = rates[(size_t)s * P.nLGN + id];
        const float rate = fr / 1000.0f;
        const float rT = dt * rate;
        float next_rT = lnl - ltr;
        unsigned nsp = 0;
        float tsp = 0.f;
        if (next_rT > rT) {
            ltr += rT;
        } else {
            float old_rT;
            do {
                const float u = curand_uniform(&st);
                lnl = fmaxf(-logf(u), 0.0f * rate);
                old_rT = next_rT;
                next_rT += lnl;
                nsp++;
            } while (next_rT <= rT);
            ltr = rT - old_rT;
            tsp = old_rT / (rate * nsp);
        }
        sinfoOut[(size_t)s * P.nLGN + id] = nsp + tsp / dt;
        if (frOut) frOut[(size_t)s * P.nLGN + id] = fr;
    }
    P.leftTimeRate[id] = ltr;
    P.lastNegLogRand[id] = lnl;
    P.state[id] = st;
}

}  // namespace
}  // namespace pv1

using namespace pv1;

extern "C" int pv1_lgn_spikes_noalloc(pv1_plan *plan, uint32_t nsteps, float *d_sinfo, float *d_fr) {
    if (!plan || !d_sinfo || nsteps == 0) return PV1_E_ARG;
    PlanLgnView view;
    int r = plan_lgn_view(plan, &view);
    if (r) return r;
    if (view.lp.nParvo > 0)
        return plan_fail(plan, PV1_E_UNSUPPORTED, "pv1_lgn_spikes_noalloc: plans with parvo cells are not supported");
    if (view.lp.nFF > 0)
        return plan_fail(plan, PV1_E_UNSUPPORTED,
                         "pv1_lgn_spikes_noalloc: plans with LGN->V1 plasticity are not supported");
    if (view.v1Stepped)
        return plan_fail(plan, PV1_E_STATE,
                         "pv1_lgn_spikes_noalloc: the plan was stepped by pv1_run or a batch; LGN-only stepping "
                         "needs a plan that only this entry point steps");
    if (nsteps > kNoAllocMaxSteps)
        return plan_fail(plan, PV1_E_ARG, "pv1_lgn_spikes_noalloc: at most 65535 steps per call");
    const size_t need = (size_t)nsteps * (size_t)view.lp.nLGN;
    if (need > kNoAllocRateFloats)
        return plan_fail(plan, PV1_E_ARG,
                         "pv1_lgn_spikes_noalloc: nsteps * nLGN exceeds the fixed scratch of 1048576 "
                         "rates (4 MiB); call it with fewer steps at a time");
    unsigned char *base = nullptr;
    cudaError_t e = scratch_address(view.device, &base);
    if (e != cudaSuccess)
        return plan_fail(plan, PV1_E_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
    long long *stepSlot = reinterpret_cast<long long *>(base);
    float *rates = reinterpret_cast<float *>(base + kNoAllocHeadBytes);
    LgnParams lp = view.lp;
    lp.rate = rates;
    lp.outFr = nullptr;
    lp.recU = nullptr;
    lp.recUCount = nullptr;
    set_step_kernel<<<1, 1, 0, view.stream>>>(stepSlot, view.step);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_lgn_rate_only(lp, stepSlot, (int)nsteps, view.stream);
    if (e == cudaSuccess && lp.nMagno > 0) {
        lgn_spike_rows_kernel<<<(lp.nMagno + 255) / 256, 256, 0, view.stream>>>(lp, stepSlot, (int)nsteps, rates,
                                                                                d_sinfo, d_fr);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return plan_fail(plan, PV1_E_CUDA, cudaGetErrorString(e));
    plan_advance_steps(plan, nsteps);
    plan_mark_lgn_only(plan);
    return PV1_OK;
}
