// Host runtime of the patchV1 GB300 hot path: the plan object behind the C ABI of
// include/patchv1_gb300.h.  It owns every device buffer and one CUDA stream, builds the
// device-side tables (far-delivery event lists, temporal-kernel segment table), and issues
// the step loop as CUDA graphs of (one LGN launch + K V1 launches + a step-counter bump).
#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <iterator>
#include <random>
#include <string>
#include <vector>

#include "pv1_internal.cuh"

using namespace pv1;

// One delayed synapse: pre, post, strength, distance (mm), class (1: near block, 0: far).
struct EvSyn {
    int pre, post;
    float str, dist;
    unsigned char near;
};

struct pv1_plan {
    pv1_v1_config cfg{};
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    int nV1 = 0, nE = 0, nI = 0;
    V1Params vp{};
    LgnParams lp{};
    // device allocations (freed in destroy)
    std::vector<void *> allocs;
    int *d_err = nullptr;
    long long *d_stepBase = nullptr;
    bool haveLGNsyn = false, haveNear = false, haveState = false, haveRng = false;
    bool haveFarEng = false;    // far failure: engines seeded (pv1_v1_far_failure_engines)
    // framed output of the physical V1 sheet
    unsigned *d_pixOff = nullptr, *d_pixIds = nullptr;
    float *d_frameAcc = nullptr, *d_frameOut = nullptr;
    int nPixel = 0, nSpikePixel = 0, frameOt = 0, frameOutCap = 0;
    float frameOdt = 0.f;
    long long frameT0 = 0;
    bool lgnReady = false, stimReady = false;
    pv1_lgn_config lcfg{};
    int nMagno = 0, nLGN = 0, mSample = 0;
    float *d_TW = nullptr, *d_SW = nullptr, *d_SC = nullptr, *d_maxConvol = nullptr;
    float *d_S = nullptr;
    int *d_coneType = nullptr;
    // parvocellular cells
    pv1_lgn_parvo_config pcfg{};
    int nParvo = 0, pSample = 0;
    float *d_pTW = nullptr, *d_pSW = nullptr, *d_pSC = nullptr, *d_pS = nullptr;
    int *d_pCone = nullptr;
    // stimulus texture arrays kept between loads of movies of the same size (one layer batch)
    cudaArray_t stimArr[3] = {nullptr, nullptr, nullptr};
    cudaTextureObject_t stimTex[3] = {0, 0, 0};
    uint32_t stimW = 0, stimH = 0, stimL = 0;
    // spatial stage of a movie held in one texture batch is computed on demand: frames
    // [0, framesDone) are in the tables (the initial-luminance row from the load on)
    bool lazyFrames = false;
    int framesDone = 0;
    int nFrame = 0;
    // LGN spike ring
    float *d_lgnRing = nullptr, *d_lgnFr = nullptr;
    int lgnSlots = 0;
    // an external LGN source (pv1_set_lgn_source): rows [extStep0, extStep0 + extSteps)
    const float *extLgn = nullptr;
    long long extStep0 = 0, extSteps = 0;
    int K = 64;  // steps per LGN launch / per persistent V1 launch / per graph
    bool persistent = false;     // V1 steps run as one cooperative launch per chunk
    // the LGN of chunk c+1 runs on its own stream while the persistent V1 kernel runs chunk c
    cudaStream_t lgnStream = nullptr;
    cudaEvent_t evLgn = nullptr, evFree = nullptr;
    long long *d_lgnStep = nullptr;
    // spike rows copied to a host buffer while the run goes on (pv1_run_spikes_to_host)
    cudaStream_t copyStream = nullptr;
    cudaEvent_t evChunk = nullptr, evCopied = nullptr;
    float *sinkHost = nullptr;        // row 0 = step sinkStep0
    long long sinkStep0 = 0;
    bool allowPersistent = true;
    unsigned *d_barrier = nullptr;
    bool modeChosen = false;
    long long graphLaunches = 0;
    // stepping
    long long step = 0;
    bool pending = false;
    // stepped by pv1_lgn_spikes_noalloc: the LGN generators and the step counter moved
    // without the V1 state, so pv1_run, batches and checkpoints refuse the plan
    bool lgnOnly = false;
    // records
    int recFlags = 0;
    int recSlots = 0;
    float *d_rec = nullptr;
    long long recStride = 0;
    // graphs
    cudaGraphExec_t graphExec = nullptr;
    long long launches = 0;
    long long nFarSyn = 0;
    void *flushBuf = nullptr;
    uint64_t flushSize = 0;
    // delayed synapses (host copies, kept while the near and far lists are merged)
    std::vector<EvSyn> farSyn, nearSyn;
};

static void release_stimulus_textures(pv1_plan *p);
static int ensure_frames(pv1_plan *p, long long lastStep);
// every frame of the loaded movie in the spatial-stage tables
static int ensure_all_frames(pv1_plan *p) { return ensure_frames(p, (long long)1 << 40); }

namespace {

int fail(pv1_plan *p, int code, const std::string &msg) {
    if (p) p->err = msg;
    return code;
}

#define PV1_CUDA(p, call)                                                                      \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail((p), PV1_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dev_alloc(pv1_plan *p, T **ptr, size_t n) {
    *ptr = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)ptr, n * sizeof(T));
    if (e != cudaSuccess) return fail(p, PV1_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    p->allocs.push_back((void *)*ptr);
    e = cudaMemsetAsync(*ptr, 0, n * sizeof(T), p->stream);
    if (e != cudaSuccess) return fail(p, PV1_E_CUDA, cudaGetErrorString(e));
    return PV1_OK;
}

template <class T>
int dev_upload(pv1_plan *p, T **ptr, const T *host, size_t n) {
    int r = dev_alloc(p, ptr, n);
    if (r) return r;
    if (host && n) PV1_CUDA(p, cudaMemcpyAsync(*ptr, host, n * sizeof(T), cudaMemcpyHostToDevice, p->stream));
    return PV1_OK;
}

void free_one(pv1_plan *p, void *ptr) {
    auto it = std::find(p->allocs.begin(), p->allocs.end(), ptr);
    if (it != p->allocs.end()) {
        cudaFree(ptr);
        p->allocs.erase(it);
    }
}

int check_device_error(pv1_plan *p) {
    int h = 0;
    PV1_CUDA(p, cudaMemcpyAsync(&h, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    if (h) {
        std::string m = "device error word 0x" + std::to_string(h) + ":";
        if (h & kErrRecordOverflow) m += " draw-record overflow;";
        if (h & kErrNegTsp) m += " negative or NaN spike time;";
        if (h & kErrFarOverflow) m += " far event beyond delay ring;";
        if (h & kErrBounds) m += " bounds check;";
        if (h & kErrBarrier) m += " a barrier wait gave up (pv1_set_wait_limit);";
        return fail(p, PV1_E_DEVICE, m);
    }
    return PV1_OK;
}

void drop_graph(pv1_plan *p) {
    p->modeChosen = false;
    if (p->graphExec) {
        cudaGraphExecDestroy(p->graphExec);
        p->graphExec = nullptr;
    }
}

// With a spike sink set: copies the spike rows of steps [a, a + n) (already issued on the
// plan's stream) to the sink on the copy stream, behind an event on the plan's stream.
int sink_rows(pv1_plan *p, long long a, long long n) {
    if (!p->sinkHost || n <= 0) return PV1_OK;
    PV1_CUDA(p, cudaEventRecord(p->evChunk, p->stream));
    PV1_CUDA(p, cudaStreamWaitEvent(p->copyStream, p->evChunk, 0));
    const size_t nV1 = p->nV1;
    long long done = 0;
    while (done < n) {
        const long long t = a + done;
        const long long slot = t % p->recSlots;
        const long long cnt = std::min<long long>(n - done, p->recSlots - slot);
        PV1_CUDA(p, cudaMemcpyAsync(p->sinkHost + (size_t)(t - p->sinkStep0) * nV1, p->vp.recSpk + (size_t)slot * nV1,
                                    (size_t)cnt * nV1 * sizeof(float), cudaMemcpyDeviceToHost, p->copyStream));
        done += cnt;
    }
    return PV1_OK;
}

// The LGN spike words of steps [t0, t0 + k) into the LGN ring on stream st: the LGN kernels
// (their step counter at d_step), or, with an external source, copies of its rows.  Returns
// the kernel launches through *launches.
int lgn_stage(pv1_plan *p, long long t0, int k, const long long *d_step, cudaStream_t st, long long *launches) {
    if (!p->extLgn) {
        cudaError_t e = launch_lgn_step(p->lp, d_step, k, st);
        if (e != cudaSuccess) return fail(p, PV1_E_CUDA, std::string("lgn_step: ") + cudaGetErrorString(e));
        if (launches) *launches += lgn_step_launches(p->lp, k);
        return PV1_OK;
    }
    if (t0 < p->extStep0 || t0 + k > p->extStep0 + p->extSteps)
        return fail(p, PV1_E_ARG, "the steps run are not all in the external LGN source");
    const size_t row = (size_t)p->nLGN * sizeof(float);
    long long done = 0;
    while (done < k) {
        const long long t = t0 + done;
        const long long slot = t % p->lgnSlots;
        const long long cnt = std::min<long long>(k - done, p->lgnSlots - slot);
        PV1_CUDA(p, cudaMemcpyAsync(p->d_lgnRing + (size_t)slot * p->nLGN, p->extLgn + (size_t)(t - p->extStep0) * p->nLGN,
                                    (size_t)cnt * row, cudaMemcpyDeviceToDevice, st));
        done += cnt;
    }
    return PV1_OK;
}

// Issues k steps (from host step t0) on the plan's stream: the LGN stage for the k steps,
// then either one persistent cooperative V1 launch for all k steps or k per-step V1 launches,
// then the step-counter bump.  Returns the number of kernel launches through *launches.
int issue_chunk(pv1_plan *p, long long t0, int k, int deliverFirst, long long *launches) {
    long long n = 0;
    int r = lgn_stage(p, t0, k, p->d_stepBase, p->stream, &n);
    if (r) return r;
    cudaError_t e = cudaSuccess;
    if (p->persistent) {
        e = launch_v1_persistent(p->vp, p->d_stepBase, k, p->d_lgnRing, p->lgnSlots, deliverFirst, p->d_barrier,
                                 p->stream);
        if (e != cudaSuccess) return fail(p, PV1_E_CUDA, std::string("v1_persistent: ") + cudaGetErrorString(e));
        n += 1;
    } else {
        for (int s = 0; s < k; s++) {
            int deliver = (s == 0) ? deliverFirst : 1;
            e = launch_v1_step(p->vp, p->d_stepBase, s, p->d_lgnRing, p->lgnSlots, deliver, 1, p->stream);
            if (e != cudaSuccess) return fail(p, PV1_E_CUDA, std::string("v1_step: ") + cudaGetErrorString(e));
            if (p->vp.farPullOn) {
                e = launch_far_pull(p->vp, p->d_stepBase, s, p->stream);
                if (e != cudaSuccess) return fail(p, PV1_E_CUDA, std::string("far_pull: ") + cudaGetErrorString(e));
                n += kFarPullLaunches;
            }
        }
        n += k;
    }
    e = launch_advance_step(p->d_stepBase, k, p->stream);
    if (e != cudaSuccess) return fail(p, PV1_E_CUDA, cudaGetErrorString(e));
    if (launches) *launches += n + 1;
    return PV1_OK;
}

// Builds the per-phase segment table of the temporal kernel: for phase p the sample j sits
// (T0 + j*interval)*denorm + p units of dt/denorm after the window tail, i.e. in the frame
// rel = that / ntPerFrame after the tail frame (src/discrete_input_convol.cu:1442-1540).
void build_segments(int nKS, int T0, int interval, int denorm, int ntPerFrame, std::vector<int> &nseg,
                    std::vector<int> &rel, std::vector<int> &j0, int &maxSeg) {
    const int nPhase = ntPerFrame;
    std::vector<std::vector<int>> relv(nPhase), j0v(nPhase);
    maxSeg = 1;
    for (int ph = 0; ph < nPhase; ph++) {
        int last = -1;
        for (int j = 0; j < nKS; j++) {
            long long o = (long long)(T0 + (long long)j * interval) * denorm + ph;
            int r = (int)(o / ntPerFrame);
            if (r != last) {
                relv[ph].push_back(r);
                j0v[ph].push_back(j);
                last = r;
            }
        }
        j0v[ph].push_back(nKS);
        maxSeg = std::max<int>(maxSeg, (int)relv[ph].size());
    }
    nseg.assign(nPhase, 0);
    rel.assign((size_t)nPhase * maxSeg, 0);
    j0.assign((size_t)nPhase * (maxSeg + 1), nKS);
    for (int ph = 0; ph < nPhase; ph++) {
        nseg[ph] = (int)relv[ph].size();
        for (size_t s = 0; s < relv[ph].size(); s++) rel[(size_t)ph * maxSeg + s] = relv[ph][s];
        for (size_t s = 0; s < j0v[ph].size(); s++) j0[(size_t)ph * (maxSeg + 1) + s] = j0v[ph][s];
    }
}

}  // namespace

namespace pv1 {

int plan_lgn_view(pv1_plan *p, PlanLgnView *out) {
    if (!p || !out) return PV1_E_ARG;
    if (!p->lgnReady || !p->stimReady) return fail(p, PV1_E_STATE, "LGN/stimulus not loaded");
    int r = ensure_all_frames(p);
    if (r) return r;
    out->lp = p->lp;
    out->stream = p->stream;
    out->step = p->step;
    out->device = p->device;
    out->v1Stepped = p->pending || (p->step > 0 && !p->lgnOnly);
    return PV1_OK;
}

void plan_advance_steps(pv1_plan *p, long long n) { p->step += n; }

void plan_mark_lgn_only(pv1_plan *p) { p->lgnOnly = true; }

int plan_batch_view(pv1_plan *p, PlanBatchView *out) {
    if (!p || !out) return PV1_E_ARG;
    if (p->lgnOnly) return fail(p, PV1_E_STATE, "the plan was stepped by pv1_lgn_spikes_noalloc (LGN only)");
    if (!p->lgnReady || !p->stimReady) return fail(p, PV1_E_STATE, "LGN/stimulus not loaded");
    int er = ensure_all_frames(p);
    if (er) return er;
    if (!p->haveLGNsyn || !p->haveNear || !p->haveState || !p->haveRng)
        return fail(p, PV1_E_STATE, "V1 synapses/connectivity/state/rng not set");
    if (p->vp.farPullOn || p->vp.nearPullOn)
        return fail(p, PV1_E_UNSUPPORTED, "batched trials with synaptic failure on delayed synapses are not built");
    if (p->vp.ffMode) return fail(p, PV1_E_UNSUPPORTED, "batched trials with LGN->V1 plasticity are not built");
    out->vp = p->vp;
    out->lp = p->lp;
    out->lgnRing = p->d_lgnRing;
    out->lgnSlots = p->lgnSlots;
    out->d_stepBase = p->d_stepBase;
    out->step = p->step;
    out->pending = p->pending;
    out->device = p->device;
    out->stream = p->stream;
    return PV1_OK;
}

void plan_batch_finish(pv1_plan *p, long long step) {
    if (step > p->step) {
        p->step = step;
        p->pending = true;
    }
}

int plan_fail(pv1_plan *p, int code, const char *msg) { return fail(p, code, msg); }

}  // namespace pv1

extern "C" {

int pv1_abi_version(void) { return 1; }

int pv1_set_device(int device) {
    return cudaSetDevice(device) == cudaSuccess ? PV1_OK : PV1_E_CUDA;
}

const char *pv1_last_error(const pv1_plan *plan) { return plan ? plan->err.c_str() : "null plan"; }

int pv1_plan_create(const pv1_v1_config *cfg, pv1_plan **out) {
    if (!cfg || !out) return PV1_E_ARG;
    *out = nullptr;
    const pv1_v1_config &c = *cfg;
    if (c.nType < 1 || c.nType > PV1_MAX_NTYPE || c.nTypeE < 1 || c.nTypeE >= c.nType + 1)
        return PV1_E_ARG;
    if (c.blockSize < 32 || c.blockSize > 1024 || c.nblock < 1) return PV1_E_ARG;
    if (c.typeAcc[c.nType - 1] != c.blockSize) return PV1_E_ARG;
    if (c.ngFF < 1 || c.ngFF > PV1_MAX_NG || c.ngE < 1 || c.ngE > PV1_MAX_NG || c.ngI < 1 ||
        c.ngI > PV1_MAX_NG)
        return PV1_E_ARG;
    if (!(c.dt > 0)) return PV1_E_ARG;
    pv1_plan *p = new pv1_plan();
    p->cfg = c;
    if (cudaGetDevice(&p->device) != cudaSuccess) {
        delete p;
        return PV1_E_CUDA;
    }
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete p;
        return PV1_E_CUDA;
    }
    if (c.noDelay != 0 && c.noDelay != 1) {
        *out = p;
        return fail(p, PV1_E_ARG, "noDelay must be 0 or 1");
    }
    if (c.noDelay == 0 && c.noFarDelay) {
        *out = p;
        return fail(p, PV1_E_ARG, "noFarDelay = 1 requires noDelay = 1");
    }
    p->nV1 = (int)(c.nblock * c.blockSize);
    p->nE = (int)c.typeAcc[c.nTypeE - 1];
    p->nI = (int)c.blockSize - p->nE;
    const int nV1 = p->nV1;
    V1Params &v = p->vp;
    v.nV1 = nV1;
    v.blockSize = (int)c.blockSize;
    v.nblock = (int)c.nblock;
    v.nE = p->nE;
    v.nI = p->nI;
    v.nType = (int)c.nType;
    v.nTypeE = (int)c.nTypeE;
    for (int j = 0; j < kMaxType; j++) v.typeAcc[j] = (int)c.typeAcc[j];
    v.ngFF = (int)c.ngFF;
    v.ngE = (int)c.ngE;
    v.ngI = (int)c.ngI;
    v.dt = c.dt;
    v.condFF = make_cond(c.riseFF, c.decayFF, c.ngFF);
    v.condE = make_cond(c.riseE, c.decayE, c.ngE);
    v.condI = make_cond(c.riseI, c.decayI, c.ngI);
    v.vE = c.vE;
    v.vI = c.vI;
    v.vL = c.vL;
    bool condRng = false, noiseRng = false;
    for (int j = 0; j < kMaxType; j++) {
        v.vR[j] = c.vR[j];
        v.vThres[j] = c.vThres[j];
        v.gL[j] = c.gL[j];
        v.C[j] = c.C[j];
        v.tRef[j] = c.tRef[j];
        v.vT[j] = c.vT[j];
        v.deltaT[j] = c.deltaT[j];
        v.tau_w[j] = c.tau_w[j];
        v.a[j] = c.a[j];
        v.b[j] = c.b[j];
        v.synFailFF[j] = c.synFailFF[j];
        v.synPerConFF[j] = c.synPerConFF[j];
        v.noisyDep[j] = c.noisyDep[j];
        if (j < (int)c.nType && c.synFailFF[j] > 0) condRng = true;
        if (j < (int)c.nType && c.noisyDep[j] > 0) noiseRng = true;
    }
    for (int j = 0; j < kMaxType * kMaxNG; j++) {
        v.pFF[j] = c.pFF[j];
        v.pE[j] = c.pE[j];
        v.pI[j] = c.pI[j];
    }
    for (int j = 0; j < kMaxType * kMaxType; j++) {
        v.synFail[j] = c.synFail[j];
        v.synPerCon[j] = c.synPerCon[j];
        if (j < (int)(c.nType * c.nType) && c.synFail[j] > 0) condRng = true;
    }
    v.condRng = condRng;
    v.noiseRng = noiseRng;
    v.tau_noise = c.tau_noise;
    v.noiseOnTonic = c.noiseOnTonic;
    v.iModel = c.iModel;
    v.noDelay = c.noDelay;
    // dt > the shortest refractory period selects the multi-spike step (src/patch.cu:990-995, 6297)
    {
        float minTRef = c.tRef[0];
        for (int j = 1; j < (int)c.nType; j++) minTRef = std::min(minTRef, c.tRef[j]);
        v.multiSpike = c.dt > minTRef ? 1 : 0;
    }
    v.hWrite = c.hWrite;
    int r = 0;
    r |= dev_alloc(p, &p->d_err, 1);
    r |= dev_alloc(p, &p->d_stepBase, 1);
    r |= dev_alloc(p, &v.v, nV1);
    r |= dev_alloc(p, &v.w, nV1);
    r |= dev_alloc(p, &v.tBack, nV1);
    r |= dev_alloc(p, &v.dep, nV1);
    r |= dev_alloc(p, &v.gFF, (size_t)c.ngFF * nV1);
    r |= dev_alloc(p, &v.hFF, (size_t)c.ngFF * nV1);
    r |= dev_alloc(p, &v.gE, (size_t)c.ngE * nV1);
    r |= dev_alloc(p, &v.hE, (size_t)c.ngE * nV1);
    r |= dev_alloc(p, &v.gI, (size_t)c.ngI * nV1);
    r |= dev_alloc(p, &v.hI, (size_t)c.ngI * nV1);
    r |= dev_alloc(p, &v.tonicDep, nV1);
    r |= dev_alloc(p, &v.lastNoise, nV1);
    r |= dev_alloc(p, &v.sInfo, (size_t)2 * nV1);
    r |= dev_alloc(p, &v.rGenCond, nV1);
    r |= dev_alloc(p, &v.rNoisy, nV1);
    r |= dev_alloc(p, &v.farFlag, 3);
    if (r) {
        *out = p;
        return PV1_E_NOMEM;
    }
    v.err = p->d_err;
    v.recSlots = 1;
    v.waitSpins = kDefaultWaitSpins;
    *out = p;
    PV1_CUDA(p, compute_step_decay(v, p->stream));
    return PV1_OK;
}

void pv1_plan_destroy(pv1_plan *p) {
    if (!p) return;
    cudaStreamSynchronize(p->stream);
    if (p->lgnStream) cudaStreamSynchronize(p->lgnStream);
    drop_graph(p);
    release_stimulus_textures(p);
    if (p->copyStream) cudaStreamSynchronize(p->copyStream);
    if (p->evLgn) cudaEventDestroy(p->evLgn);
    if (p->evFree) cudaEventDestroy(p->evFree);
    if (p->lgnStream) cudaStreamDestroy(p->lgnStream);
    if (p->evChunk) cudaEventDestroy(p->evChunk);
    if (p->evCopied) cudaEventDestroy(p->evCopied);
    if (p->copyStream) cudaStreamDestroy(p->copyStream);
    for (void *ptr : p->allocs) cudaFree(ptr);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

namespace {

// Sample grid of parvo_maxConvol (src/patch.cu:5266-5312): round(mean size ratio of the
// surround-enclosing square to the centre's) * nSpatialSample1D per side, at least 32, at
// most what 48 KB of shared memory holds.  The mean runs over the cells of cone type < 4 --
// the reference's loop also counts L+M magno cells -- and is divided by nParvo.
int parvo_max_sample1d(const pv1_lgn_config &c, const pv1_lgn_params &prm, int nParvo, int n1) {
    const int nLGN = (int)c.nLGN;
    const float nsig = std::fabs(c.nsig);
    auto span = [&](float r) { return (float)((double)(nsig * r) / 1.4142135623730951); };
    float meanRatio = 0.f;
    for (int i = 0; i < nLGN; i++) {
        if (prm.coneType[i] >= 4) continue;
        const float dx = prm.ecc[i] * std::cos(prm.polar[i]) - prm.ecc[nLGN + i] * std::cos(prm.polar[nLGN + i]);
        const float dy = prm.ecc[i] * std::sin(prm.polar[i]) - prm.ecc[nLGN + i] * std::sin(prm.polar[nLGN + i]);
        float r = std::sqrt(dx * dx + dy * dy);
        float wSpan = span(prm.rw[nLGN + i]), hSpan = span(prm.rh[nLGN + i]);
        float R = wSpan > hSpan ? wSpan : hSpan;
        wSpan = span(prm.rw[i]);
        hSpan = span(prm.rh[i]);
        r += wSpan > hSpan ? wSpan : hSpan;
        R = r > R ? r : R;
        meanRatio += std::sqrt(R * R / wSpan / hSpan);
    }
    meanRatio /= nParvo;
    long long m1 = (long long)std::round(meanRatio) * n1;
    if (m1 * m1 < 1024) return 32;
    const size_t avail = 48 * 1024 - 32 * sizeof(float);
    if ((size_t)(m1 * m1) * 2 * sizeof(float) > avail)
        m1 = (long long)std::floor(std::sqrt((double)(avail / sizeof(float) / 2 / (size_t)(n1 * n1)))) * n1;
    return (int)m1;
}

int lgn_setup_impl(pv1_plan *p, const pv1_lgn_config *lc, const pv1_lgn_parvo_config *pc,
                   const pv1_lgn_params *prm, const float *covariant, uint64_t seed) {
    if (!p || !lc || !prm) return PV1_E_ARG;
    const pv1_lgn_config &c = *lc;
    const int nParvo = (int)(c.nParvo_I + c.nParvo_C);
    const int nMagno = (int)(c.nMagno_I + c.nMagno_C);
    if (nParvo > 0 && !pc) return fail(p, PV1_E_UNSUPPORTED, "parvocellular LGN cells need pv1_lgn_setup_parvo");
    if (nParvo > 0 && !covariant) return fail(p, PV1_E_ARG, "parvo cells need the covariant array");
    if (nParvo > 0 && (pc->nSample1D < 1 || pc->nSample1D > 32 || pc->nKernelSample < 1))
        return fail(p, PV1_E_ARG, "parvo nSample1D must be in [1,32] and nKernelSample >= 1");
    if ((int)c.nLGN != nParvo + nMagno) return fail(p, PV1_E_ARG, "nLGN != nParvo + nMagno");
    if (c.mSample1D < 1 || c.mSample1D > 32) return fail(p, PV1_E_ARG, "mSample1D must be in [1,32]");
    if (c.nKernelSample < 1 || c.ntPerFrame < 1 || c.denorm < 1 || c.maxFrame < 1)
        return fail(p, PV1_E_ARG, "bad kernel-sampling bookkeeping");
    if (!(c.nsig > 0)) return fail(p, PV1_E_UNSUPPORTED, "nsig <= 0 (python sampler) is not built");
    p->lcfg = c;
    p->nMagno = nMagno;
    p->nLGN = (int)c.nLGN;
    p->mSample = (int)(c.mSample1D * c.mSample1D);
    const int nLGN = p->nLGN;
    const int nKS = (int)c.nKernelSample;
    LgnParams &L = p->lp;
    L.nMagno = nMagno;
    L.nLGN = nLGN;
    L.nParvo_I = (int)c.nParvo_I;
    L.nMagno_I = (int)c.nMagno_I;
    L.nParvo_C = (int)c.nParvo_C;
    L.nKS = nKS;
    L.dt = c.dt;
    L.convolRatio = c.convolRatio;
    L.frRatio = c.frRatio;
    L.iKernelSampleT0 = (int)c.iKernelSampleT0;
    L.interval = (int)c.kernelSampleInterval;
    L.err = p->d_err;
    // per-cell parameters (2*nLGN arrays)
    float *d_par[12];
    const float *hpar[12] = {prm->polar, prm->ecc, prm->rw, prm->rh, prm->orient, prm->k,
                             prm->ratio, prm->tauR, prm->tauD, prm->nR, prm->nD, prm->delay};
    for (int q = 0; q < 12; q++) {
        if (!hpar[q]) return fail(p, PV1_E_ARG, "missing LGN parameter array");
        int r = dev_upload(p, &d_par[q], hpar[q], (size_t)2 * nLGN);
        if (r) return r;
    }
    // logistic a, b (hStatic_nonlinear, src/LGN_props.h:159-169), float arithmetic
    std::vector<float> la(nLGN), lb(nLGN);
    for (int i = 0; i < nLGN; i++) {
        const float e_kc50 = std::exp(prm->sharpness[i] * prm->c50[i]);
        const float e_kc50_k = std::exp(prm->sharpness[i] * prm->c50[i] - prm->sharpness[i]);
        la[i] = (1 - prm->spont[i]) * (1 + e_kc50) * (1 + e_kc50_k) / (e_kc50 - e_kc50_k);
        lb[i] = 1 - la[i] / (1 + e_kc50_k);
    }
    float *d_c50, *d_sharp, *d_la, *d_lb, *d_absk;
    int r = 0;
    r |= dev_upload(p, &d_c50, prm->c50, nLGN);
    r |= dev_upload(p, &d_sharp, prm->sharpness, nLGN);
    r |= dev_upload(p, &d_la, la.data(), nLGN);
    r |= dev_upload(p, &d_lb, lb.data(), nLGN);
    r |= dev_alloc(p, &p->d_TW, (size_t)nMagno * nKS);
    r |= dev_alloc(p, &p->d_SW, (size_t)nMagno * p->mSample);
    r |= dev_alloc(p, &p->d_SC, (size_t)2 * nMagno * p->mSample);
    r |= dev_alloc(p, &p->d_maxConvol, nLGN);
    r |= dev_alloc(p, &d_absk, nMagno);
    double *d_ctw;
    r |= dev_alloc(p, &d_ctw, (size_t)(nKS + 1) * nMagno);
    float *d_ltr, *d_lnl;
    curandStateMRG32k3a *d_state;
    r |= dev_alloc(p, &d_ltr, nLGN);
    r |= dev_alloc(p, &d_lnl, nLGN);
    r |= dev_alloc(p, &d_state, nLGN);
    if (r) return fail(p, PV1_E_NOMEM, "LGN allocation failed");
    // cone type of each magno center
    std::vector<int> cone(nMagno);
    for (int m = 0; m < nMagno; m++) {
        int id = (int)c.nParvo_I + m;
        if (m >= (int)c.nMagno_I) id += (int)c.nParvo_C;
        cone[m] = (int)prm->coneType[id];
        if (cone[m] > 4) return fail(p, PV1_E_ARG, "cone type > 4");
    }
    r = dev_upload(p, &p->d_coneType, cone.data(), nMagno);
    if (r) return r;
    SetupArgs A{};
    A.nMagno = nMagno;
    A.nLGN = nLGN;
    A.nParvo_I = (int)c.nParvo_I;
    A.nMagno_I = (int)c.nMagno_I;
    A.nParvo_C = (int)c.nParvo_C;
    A.nSample = p->mSample;
    A.nSample1D = (int)c.mSample1D;
    A.nKS = nKS;
    A.kernelSampleDt = c.kernelSampleDt;
    A.kernelSampleT0 = c.kernelSampleT0;
    A.normViewDistance = c.normViewDistance;
    A.L_x0 = c.L_x0;
    A.L_y0 = c.L_y0;
    A.R_x0 = c.R_x0;
    A.R_y0 = c.R_y0;
    A.nsig = c.nsig;
    A.flat = c.flat_retina;
    A.polar = d_par[0];
    A.ecc = d_par[1];
    A.rw = d_par[2];
    A.rh = d_par[3];
    A.orient = d_par[4];
    A.k = d_par[5];
    A.ratio = d_par[6];
    A.tauR = d_par[7];
    A.tauD = d_par[8];
    A.nR = d_par[9];
    A.nD = d_par[10];
    A.delay = d_par[11];
    A.TW = p->d_TW;
    A.SW = p->d_SW;
    A.SC = p->d_SC;
    A.maxConvol = p->d_maxConvol;
    A.absk = d_absk;
    A.ctw = d_ctw;
    A.err = p->d_err;
    int threads = ((p->mSample + 31) / 32) * 32;
    if (nMagno > 0) PV1_CUDA(p, launch_lgn_setup(A, threads, p->stream));
    PV1_CUDA(p, launch_lgn_rng_init(d_state, d_lnl, d_ltr, (unsigned long long)seed, nLGN, p->stream));
    // segment table
    std::vector<int> nseg, rel, j0;
    int maxSeg = 1;
    build_segments(nKS, (int)c.iKernelSampleT0, (int)c.kernelSampleInterval, (int)c.denorm, (int)c.ntPerFrame,
                   nseg, rel, j0, maxSeg);
    if (maxSeg > kMaxSeg) return fail(p, PV1_E_UNSUPPORTED, "temporal window spans more than 255 frames");
    r = dev_alloc(p, &L.rate, (size_t)p->K * nLGN);
    if (r) return r;
    int *d_nseg, *d_rel, *d_j0;
    r = 0;
    r |= dev_upload(p, &d_nseg, nseg.data(), nseg.size());
    r |= dev_upload(p, &d_rel, rel.data(), rel.size());
    r |= dev_upload(p, &d_j0, j0.data(), j0.size());
    if (r) return r;
    L.seg.nPhase = (int)c.ntPerFrame;
    L.seg.maxSeg = maxSeg;
    L.seg.nseg = d_nseg;
    L.seg.rel = d_rel;
    L.seg.j0 = d_j0;
    L.fs.denorm = (int)c.denorm;
    L.fs.ntPerFrame = (int)c.ntPerFrame;
    L.fs.maxFrame = (int)c.maxFrame;
    L.fs.magnoComp = (int)c.magnoComp;
    L.fs.frameOffset = (int)c.frameOffset;
    L.ctw = d_ctw;
    L.absk = d_absk;
    L.maxConvol = p->d_maxConvol;
    L.c50 = d_c50;
    L.sharp = d_sharp;
    L.la = d_la;
    L.lb = d_lb;
    L.leftTimeRate = d_ltr;
    L.lastNegLogRand = d_lnl;
    L.state = d_state;
    // LGN spike ring (rows = step % lgnSlots)
    p->lgnSlots = std::max(2 * p->K, 2);   // two chunks: the one V1 reads, the one the LGN writes
    r = dev_alloc(p, &p->d_lgnRing, (size_t)p->lgnSlots * nLGN);
    if (r) return r;
    L.outSInfo = p->d_lgnRing;
    L.outFr = nullptr;
    L.outSlots = p->lgnSlots;
    p->vp.lgnN = nLGN;
    // parvocellular cells: store_PM(PM=0) and parvo_maxConvol, their own segment table
    p->nParvo = nParvo;
    L.nParvo = nParvo;
    float *d_cov = nullptr;
    if (nParvo > 0) {
        const pv1_lgn_parvo_config &q = *pc;
        p->pcfg = q;
        const int n1 = (int)q.nSample1D, pKS = (int)q.nKernelSample;
        p->pSample = n1 * n1;
        std::vector<int> pcone(2 * (size_t)nParvo);
        for (int cc = 0; cc < nParvo; cc++) {
            const int id = cc < (int)c.nParvo_I ? cc : cc + (int)c.nMagno_I;
            pcone[cc] = (int)prm->coneType[id];
            pcone[nParvo + cc] = (int)prm->coneType[nLGN + id];
            if (pcone[cc] > 4 || pcone[nParvo + cc] > 4) return fail(p, PV1_E_ARG, "cone type > 4");
        }
        float *d_pk;
        double *d_pctw;
        r = 0;
        r |= dev_upload(p, &p->d_pCone, pcone.data(), pcone.size());
        r |= dev_upload(p, &d_cov, covariant, nLGN);
        r |= dev_alloc(p, &p->d_pTW, (size_t)nParvo * 2 * pKS);
        r |= dev_alloc(p, &p->d_pSW, (size_t)p->pSample);
        r |= dev_alloc(p, &p->d_pSC, (size_t)2 * nParvo * 2 * p->pSample);
        r |= dev_alloc(p, &d_pk, (size_t)2 * nParvo);
        r |= dev_alloc(p, &d_pctw, (size_t)2 * (pKS + 1) * nParvo);
        if (r) return fail(p, PV1_E_NOMEM, "parvo LGN allocation failed");
        ParvoSetupArgs PA{};
        PA.nParvo = nParvo;
        PA.flat = c.flat_retina;
        PA.nLGN = nLGN;
        PA.nParvo_I = (int)c.nParvo_I;
        PA.nMagno_I = (int)c.nMagno_I;
        PA.nSample = p->pSample;
        PA.nSample1D = n1;
        PA.nKS = pKS;
        PA.kernelSampleDt = q.kernelSampleDt;
        PA.kernelSampleT0 = q.kernelSampleT0;
        PA.normViewDistance = c.normViewDistance;
        PA.L_x0 = c.L_x0;
        PA.L_y0 = c.L_y0;
        PA.R_x0 = c.R_x0;
        PA.R_y0 = c.R_y0;
        PA.nsig = c.nsig;
        PA.polar = d_par[0];
        PA.ecc = d_par[1];
        PA.rw = d_par[2];
        PA.rh = d_par[3];
        PA.orient = d_par[4];
        PA.k = d_par[5];
        PA.ratio = d_par[6];
        PA.tauR = d_par[7];
        PA.tauD = d_par[8];
        PA.nR = d_par[9];
        PA.nD = d_par[10];
        PA.delay = d_par[11];
        PA.covariant = d_cov;
        PA.maxSample1D = parvo_max_sample1d(c, *prm, nParvo, n1);
        PA.TW = p->d_pTW;
        PA.SW = p->d_pSW;
        PA.SC = p->d_pSC;
        PA.maxConvol = p->d_maxConvol;
        PA.pk = d_pk;
        PA.pctw = d_pctw;
        PA.err = p->d_err;
        PV1_CUDA(p, launch_parvo_setup(PA, p->stream));
        std::vector<int> pnseg, prel, pj0;
        int pMaxSeg = 1;
        build_segments(pKS, (int)q.iKernelSampleT0, (int)q.kernelSampleInterval, (int)c.denorm, (int)c.ntPerFrame,
                       pnseg, prel, pj0, pMaxSeg);
        if (pMaxSeg > kMaxSeg) return fail(p, PV1_E_UNSUPPORTED, "parvo temporal window spans more than 255 frames");
        int *d_pnseg, *d_prel, *d_pj0;
        r = 0;
        r |= dev_upload(p, &d_pnseg, pnseg.data(), pnseg.size());
        r |= dev_upload(p, &d_prel, prel.data(), prel.size());
        r |= dev_upload(p, &d_pj0, pj0.data(), pj0.size());
        if (r) return r;
        L.pseg.nPhase = (int)c.ntPerFrame;
        L.pseg.maxSeg = pMaxSeg;
        L.pseg.nseg = d_pnseg;
        L.pseg.rel = d_prel;
        L.pseg.j0 = d_pj0;
        L.pKS = pKS;
        L.pT0 = (int)q.iKernelSampleT0;
        L.pInterval = (int)q.kernelSampleInterval;
        L.parvoComp = (int)q.parvoComp;
        L.pFrameOffset = (int)q.frameOffset;
        L.pctw = d_pctw;
        L.pk = d_pk;
    }
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    for (int q = 0; q < 12; q++) free_one(p, d_par[q]);
    if (d_cov) free_one(p, d_cov);
    // one temporal-kernel class (every magno cell has bit-identical temporal weights): the
    // fused single-class LGN kernel applies
    L.classCtw = nullptr;
    if (nMagno > 0 && nParvo == 0) {
        std::vector<float> tw((size_t)nMagno * nKS);
        PV1_CUDA(p, cudaMemcpy(tw.data(), p->d_TW, tw.size() * sizeof(float), cudaMemcpyDeviceToHost));
        bool same = true;
        for (int m = 1; m < nMagno && same; m++)
            same = std::memcmp(tw.data(), tw.data() + (size_t)m * nKS, nKS * sizeof(float)) == 0;
        const int shift = (int)((p->K * (long long)c.denorm + c.ntPerFrame - 1) / c.ntPerFrame);
        if (same && maxSeg <= kClassMaxSeg && maxSeg + shift + 1 <= kClassMaxSlots && p->K <= kClassMaxK) {
            double *d_cls;
            r = dev_alloc(p, &d_cls, (size_t)nKS + 1);
            if (r) return r;
            PV1_CUDA(p, cudaMemcpy2D(d_cls, sizeof(double), d_ctw, (size_t)nMagno * sizeof(double), sizeof(double),
                                     (size_t)nKS + 1, cudaMemcpyDeviceToDevice));
            L.classCtw = d_cls;
        }
    }
    int e = check_device_error(p);
    if (e) return e;
    p->lgnReady = true;
    drop_graph(p);
    return PV1_OK;
}

}  // namespace

int pv1_lgn_setup(pv1_plan *p, const pv1_lgn_config *lc, const pv1_lgn_params *prm, uint64_t seed) {
    return lgn_setup_impl(p, lc, nullptr, prm, nullptr, seed);
}

int pv1_lgn_setup_parvo(pv1_plan *p, const pv1_lgn_config *lc, const pv1_lgn_parvo_config *pc,
                        const pv1_lgn_params *prm, const float *covariant, uint64_t seed) {
    if (!pc || !covariant) return p ? fail(p, PV1_E_ARG, "missing parvo config or covariant") : PV1_E_ARG;
    return lgn_setup_impl(p, lc, pc, prm, covariant, seed);
}

int pv1_lgn_get_parvo_tables(pv1_plan *p, float *TW, float *SW, float *SC) {
    if (!p) return PV1_E_ARG;
    if (!p->lgnReady) return fail(p, PV1_E_STATE, "LGN not set up");
    if (p->nParvo == 0) return fail(p, PV1_E_STATE, "no parvo cells");
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    const size_t np = p->nParvo, ns = p->pSample;
    if (TW) PV1_CUDA(p, cudaMemcpy(TW, p->d_pTW, np * 2 * p->pcfg.nKernelSample * sizeof(float), cudaMemcpyDeviceToHost));
    if (SW) PV1_CUDA(p, cudaMemcpy(SW, p->d_pSW, ns * sizeof(float), cudaMemcpyDeviceToHost));
    if (SC) PV1_CUDA(p, cudaMemcpy(SC, p->d_pSC, 4 * np * ns * sizeof(float), cudaMemcpyDeviceToHost));
    return PV1_OK;
}

int pv1_lgn_get_parvo_spatial(pv1_plan *p, float *PS) {
    if (!p || !PS) return PV1_E_ARG;
    if (!p->stimReady) return fail(p, PV1_E_STATE, "no stimulus loaded");
    if (p->nParvo == 0) return fail(p, PV1_E_STATE, "no parvo cells");
    int r = ensure_all_frames(p);
    if (r) return r;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    PV1_CUDA(p, cudaMemcpy(PS, p->d_pS, (size_t)(p->nFrame + 1) * 2 * p->nParvo * sizeof(float), cudaMemcpyDeviceToHost));
    return PV1_OK;
}

int pv1_lgn_get_tables(pv1_plan *p, float *TW, float *SW, float *SC, float *maxConvol) {
    if (!p) return PV1_E_ARG;
    if (!p->lgnReady) return fail(p, PV1_E_STATE, "LGN not set up");
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    const size_t nm = p->nMagno;
    if (TW) PV1_CUDA(p, cudaMemcpy(TW, p->d_TW, nm * p->lcfg.nKernelSample * sizeof(float), cudaMemcpyDeviceToHost));
    if (SW) PV1_CUDA(p, cudaMemcpy(SW, p->d_SW, nm * p->mSample * sizeof(float), cudaMemcpyDeviceToHost));
    if (SC) PV1_CUDA(p, cudaMemcpy(SC, p->d_SC, 2 * nm * p->mSample * sizeof(float), cudaMemcpyDeviceToHost));
    if (maxConvol) PV1_CUDA(p, cudaMemcpy(maxConvol, p->d_maxConvol, p->nLGN * sizeof(float), cudaMemcpyDeviceToHost));
    return PV1_OK;
}

extern "C++" {
static void release_stimulus_textures(pv1_plan *p) {
    for (int ch = 0; ch < 3; ch++) {
        if (p->stimTex[ch]) cudaDestroyTextureObject(p->stimTex[ch]);
        if (p->stimArr[ch]) cudaFreeArray(p->stimArr[ch]);
        p->stimTex[ch] = 0;
        p->stimArr[ch] = nullptr;
    }
    p->stimW = p->stimH = p->stimL = 0;
}

// Computes the spatial stage of the movie frames that steps up to `lastStep` read and that
// are not in the tables yet (frames are computed in order, each once per load).
static int ensure_frames(pv1_plan *p, long long lastStep) {
    if (!p->lazyFrames || p->framesDone >= p->nFrame) return PV1_OK;
    // frames_read_after_step grows with the step; past nFrame frames every frame is needed
    const long long perFrame = std::max<long long>(1, p->lp.fs.ntPerFrame / std::max(p->lp.fs.denorm, 1));
    const long long need64 = lastStep < 0 ? 0
                             : (lastStep >= (long long)(p->nFrame + 1) * (perFrame + 1) ? p->nFrame
                                                                                        : frames_read_after_step(p->lp.fs, lastStep));
    const int need = (int)std::min<long long>(need64, p->nFrame);
    if (need <= p->framesDone) return PV1_OK;
    const int f0 = p->framesDone, n = need - f0;
    if (p->nMagno > 0)
        PV1_CUDA(p, launch_lgn_spatial(p->stimTex[0], p->stimTex[1], p->stimTex[2], p->d_SW, p->d_SC, p->d_coneType,
                                      p->nMagno, p->mSample, f0, n, f0, p->d_S, p->stream));
    if (p->nParvo > 0)
        PV1_CUDA(p, launch_parvo_spatial(p->stimTex[0], p->stimTex[1], p->stimTex[2], p->d_pSW, p->d_pSC, p->d_pCone,
                                        p->nParvo, p->pSample, f0, n, f0, p->d_pS, p->stream));
    p->framesDone = need;
    return PV1_OK;
}
}  // extern "C++"

int pv1_stimulus_load(pv1_plan *p, uint32_t nFrame, uint32_t height, uint32_t width,
                      const float init_LMS[3], const float *frames) {
    if (!p || !init_LMS || (nFrame && !frames)) return PV1_E_ARG;
    if (!p->lgnReady) return fail(p, PV1_E_STATE, "call pv1_lgn_setup first");
    if (nFrame < 1 || width < 1 || height < 1 || width > 16384 || height > 16384)
        return fail(p, PV1_E_ARG, "bad stimulus size");
    const int nMagno = p->nMagno;
    const bool sameSize = p->stimReady && (int)nFrame == p->nFrame;
    int r = 0;
    if (!sameSize) {  // the spatial-stage tables of a movie of another length
        if (p->d_S) free_one(p, p->d_S);
        r = dev_alloc(p, &p->d_S, (size_t)(nFrame + 1) * std::max(nMagno, 1));
        if (r) return r;
        if (p->nParvo > 0) {
            if (p->d_pS) free_one(p, p->d_pS);
            r = dev_alloc(p, &p->d_pS, (size_t)(nFrame + 1) * 2 * p->nParvo);
            if (r) return r;
        }
    }
    const size_t npix = (size_t)width * height;
    // process the movie in batches of <= 2047 layers plus the initial-luminance layer
    const int maxLayers = 2048;
    cudaChannelFormatDesc desc = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
    std::vector<float> initPlanes(3 * npix);
    for (int ch = 0; ch < 3; ch++) std::fill(initPlanes.begin() + ch * npix, initPlanes.begin() + (ch + 1) * npix, init_LMS[ch]);
    for (uint32_t f0 = 0; f0 < nFrame + 1; f0 += maxLayers) {
        const uint32_t nl = std::min<uint32_t>(maxLayers, nFrame + 1 - f0);
        const uint32_t nMovie = f0 < nFrame ? std::min<uint32_t>(nl, nFrame - f0) : 0;
        cudaArray_t arr[3] = {nullptr, nullptr, nullptr};
        cudaTextureObject_t tex[3] = {0, 0, 0};
        // a movie held in one batch keeps its arrays and texture objects for the next load
        const bool single = f0 == 0 && nl == nFrame + 1;
        const bool reuse = single && p->stimArr[0] && p->stimW == width && p->stimH == height && p->stimL == nl;
        if (single && !reuse) release_stimulus_textures(p);
        for (int ch = 0; ch < 3; ch++) {
            if (reuse) arr[ch] = p->stimArr[ch];
            else PV1_CUDA(p, cudaMalloc3DArray(&arr[ch], &desc, make_cudaExtent(width, height, nl), cudaArrayLayered));
            // every movie layer of this channel in one copy: the source slices are the channel's
            // planes, 3 planes apart ([frame][channel][h][w])
            if (nMovie) {
                cudaMemcpy3DParms cp{};
                cp.srcPtr = make_cudaPitchedPtr((void *)(frames + ((size_t)f0 * 3 + ch) * npix), width * sizeof(float),
                                                width, 3 * (size_t)height);
                cp.dstArray = arr[ch];
                cp.dstPos = make_cudaPos(0, 0, 0);
                cp.extent = make_cudaExtent(width, height, nMovie);
                cp.kind = cudaMemcpyHostToDevice;
                PV1_CUDA(p, cudaMemcpy3DAsync(&cp, p->stream));
            }
            if (nMovie < nl) {  // the initial-luminance layer closes the last batch
                cudaMemcpy3DParms cp{};
                cp.srcPtr = make_cudaPitchedPtr((void *)(initPlanes.data() + ch * npix), width * sizeof(float), width,
                                                height);
                cp.dstArray = arr[ch];
                cp.dstPos = make_cudaPos(0, 0, nMovie);
                cp.extent = make_cudaExtent(width, height, 1);
                cp.kind = cudaMemcpyHostToDevice;
                PV1_CUDA(p, cudaMemcpy3DAsync(&cp, p->stream));
            }
            if (reuse) {
                tex[ch] = p->stimTex[ch];
                continue;
            }
            cudaResourceDesc rd{};
            rd.resType = cudaResourceTypeArray;
            rd.res.array.array = arr[ch];
            cudaTextureDesc td{};
            td.addressMode[0] = cudaAddressModeBorder;
            td.addressMode[1] = cudaAddressModeBorder;
            td.filterMode = cudaFilterModeLinear;
            td.readMode = cudaReadModeElementType;
            td.normalizedCoords = 1;
            PV1_CUDA(p, cudaCreateTextureObject(&tex[ch], &rd, &td, nullptr));
        }
        if (single && !reuse) {
            for (int ch = 0; ch < 3; ch++) {
                p->stimArr[ch] = arr[ch];
                p->stimTex[ch] = tex[ch];
            }
            p->stimW = width;
            p->stimH = height;
            p->stimL = nl;
        }
        // a single batch: only the initial-luminance layer now, the movie frames as the steps
        // that read them are run (ensure_frames); several batches: every layer now
        const int first = single ? (int)nMovie : 0;
        if (nMagno > 0)
            PV1_CUDA(p, launch_lgn_spatial(tex[0], tex[1], tex[2], p->d_SW, p->d_SC, p->d_coneType, nMagno,
                                          p->mSample, first, (int)nl - first, (int)f0 + first, p->d_S, p->stream));
        if (p->nParvo > 0)
            PV1_CUDA(p, launch_parvo_spatial(tex[0], tex[1], tex[2], p->d_pSW, p->d_pSC, p->d_pCone, p->nParvo,
                                            p->pSample, first, (int)nl - first, (int)f0 + first, p->d_pS, p->stream));
        p->lazyFrames = single;
        PV1_CUDA(p, cudaStreamSynchronize(p->stream));
        if (!single) {
            for (int ch = 0; ch < 3; ch++) {
                cudaDestroyTextureObject(tex[ch]);
                cudaFreeArray(arr[ch]);
            }
        }
    }
    p->nFrame = (int)nFrame;
    p->framesDone = p->lazyFrames ? 0 : (int)nFrame;
    p->lp.S = p->d_S;
    p->lp.pS = p->d_pS;
    p->lp.fs.nFrame = (int)nFrame;
    p->lp.fs.initRow = (int)nFrame;
    p->stimReady = true;
    // the captured step graph stays valid when the tables kept their place and size
    if (!sameSize) drop_graph(p);
    return PV1_OK;
}

int pv1_host_alloc(uint64_t bytes, void **out) {
    if (!out) return PV1_E_ARG;
    *out = nullptr;
    if (bytes == 0) return PV1_E_ARG;
    return cudaHostAlloc(out, (size_t)bytes, cudaHostAllocDefault) == cudaSuccess ? PV1_OK : PV1_E_NOMEM;
}

void pv1_host_free(void *ptr) {
    if (ptr) cudaFreeHost(ptr);
}

int pv1_lgn_get_spatial(pv1_plan *p, float *S) {
    if (!p || !S) return PV1_E_ARG;
    if (!p->stimReady) return fail(p, PV1_E_STATE, "no stimulus loaded");
    int r = ensure_all_frames(p);
    if (r) return r;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    PV1_CUDA(p, cudaMemcpy(S, p->d_S, (size_t)(p->nFrame + 1) * p->nMagno * sizeof(float), cudaMemcpyDeviceToHost));
    return PV1_OK;
}

int pv1_v1_set_lgn_synapses(pv1_plan *p, uint32_t maxLGN, const uint32_t *nLGNperV1,
                            const uint32_t *lgnId, const float *sLGN) {
    if (!p || !nLGNperV1 || (maxLGN && (!lgnId || !sLGN))) return PV1_E_ARG;
    const int nV1 = p->nV1;
    for (int i = 0; i < nV1; i++)
        if (nLGNperV1[i] > maxLGN) return fail(p, PV1_E_ARG, "nLGNperV1 > maxLGN");
    if (p->lgnReady) {
        for (size_t q = 0; q < (size_t)maxLGN * nV1; q++) {
            const size_t i = q % nV1, j = q / nV1;
            if (j < nLGNperV1[i] && lgnId[q] >= (uint32_t)p->nLGN) return fail(p, PV1_E_ARG, "LGN id out of range");
        }
    }
    if (p->vp.multiSpike && maxLGN > (uint32_t)kMaxLgnMulti)
        return fail(p, PV1_E_UNSUPPORTED, "the multi-spike step (dt > min tRef) takes at most 64 LGN synapses per neuron");
    int *d_n, *d_id;
    float *d_s;
    int r = 0;
    r |= dev_upload(p, &d_n, (const int *)nLGNperV1, nV1);
    r |= dev_upload(p, &d_id, (const int *)lgnId, (size_t)maxLGN * nV1);
    r |= dev_upload(p, &d_s, sLGN, (size_t)maxLGN * nV1);
    if (r) return r;
    p->vp.maxLGN = (int)maxLGN;
    p->vp.nLGNperV1 = d_n;
    p->vp.lgnId = d_id;
    p->vp.sLGN = d_s;
    p->vp.sLGNw = d_s;
    p->haveLGNsyn = true;
    drop_graph(p);
    return PV1_OK;
}

// The LGN stage's trace ring of a plan with learning: one row pair per LGN ring row.
static int ensure_ff_ring(pv1_plan *p) {
    if (!p->vp.ffMode || p->lp.nFF == 0) return PV1_OK;
    if (p->lp.outPre) free_one(p, p->lp.outPre);
    p->lp.outPre = nullptr;
    float *d = nullptr;
    int r = dev_alloc(p, &d, (size_t)p->lgnSlots * p->lp.nFF * 2 * p->nLGN);
    if (r) return r;
    p->lp.outPre = d;
    p->vp.ffPreRing = d;
    return PV1_OK;
}

int pv1_ff_learning_rates(const pv1_ff_learning *l, float dt, float *out) {
    if (!l || !out) return PV1_E_ARG;
    // learnFF_post (src/condShape.h:137-152), Float = float, with its double literals
    const float A_LTP = l->A_LGN * l->sRatioLGN;
    const float tauAvg_in_sec = (float)((double)l->tauAvg / 1000.0);
    float A_ratio = l->r_LTD * A_LTP;
    if (l->targetFR > 0) {
        const float q = l->tauTrip / (l->tauLTD * (tauAvg_in_sec * tauAvg_in_sec));
        A_ratio = (float)((double)A_ratio * ((double)q / 1000.0 / (double)l->targetFR));
    }
    out[0] = A_LTP;
    out[1] = A_ratio;
    out[2] = l->gmaxLGN * l->sRatioLGN;
    out[3] = l->gminLGN * l->sRatioLGN;
    out[4] = expf(-dt / l->decayTimeHomeoFF);
    return PV1_OK;
}

// Floats of learnVar's FF block (src/patch.cu:4365-4377): the post traces of each type, then
// vAvgE [nblock*nE][2] and vAvgI [nblock*nI].
static size_t ff_post_floats(const pv1_plan *p) {
    const size_t nEt = (size_t)p->nE * p->cfg.nblock, nIt = (size_t)p->nI * p->cfg.nblock;
    const V1Params &v = p->vp;
    // learnVar's FF block (src/patch.cu:4367-4392): the FF->E post traces (none with
    // learning 4), the FF->I ones, vAvgE [nEt][2], vAvgI
    return (v.ffMode == 4 ? 0 : 2 * nEt) + 2 * (size_t)v.ffI * nIt + 2 * nEt + nIt;
}

int pv1_set_ff_learning(pv1_plan *p, const pv1_ff_learning *l) {
    if (!p || !l) return PV1_E_ARG;
    const int mode = l->learning;
    if (mode < 1 || mode > 4) return fail(p, PV1_E_ARG, "learning is 1, 2, 3 or 4");
    if (!p->lgnReady || !p->haveLGNsyn) return fail(p, PV1_E_STATE, "set up the LGN and the LGN->V1 synapses first");
    if (p->extLgn)
        return fail(p, PV1_E_UNSUPPORTED, "plasticity needs the plan's own LGN stage (its presynaptic traces)");
    if (p->vp.multiSpike)
        return fail(p, PV1_E_UNSUPPORTED, "plasticity with several spikes per step (dt > min tRef) is not built");
    // learning 1: FF->E (+ cortical variables); 2: FF->E and FF->I; 3: FF->E only; 4: cortical
    // variables only (src/patch.cu:1160-1175)
    const int nE_ = mode == 4 ? 0 : l->nLearnTypeFF_E;
    const int nI_ = mode == 2 ? l->nLearnTypeFF_I : 0;
    if (mode != 4 && nE_ != 1)
        return fail(p, PV1_E_UNSUPPORTED,
                    "learning 1-3 with nLearnTypeFF_E != 1 (0 would clip every LGN->E weight to the zeroed "
                    "struct's [0, 0]; the reference allows at most 1)");
    if (nI_ < 0 || nI_ > 1) return fail(p, PV1_E_UNSUPPORTED, "nLearnTypeFF_I is 0 or 1 (the reference's maximum)");
    if (mode != 4 && !(l->tauLTP > 0 && l->tauLTD > 0 && l->tauTrip > 0 && l->tauAvg > 0))
        return fail(p, PV1_E_ARG, "FF->E learning time constants must be > 0");
    if (nI_ && !(l->tauLTP_I > 0 && l->tauLTD_I > 0 && l->tauTrip_I > 0 && l->tauAvg_I > 0))
        return fail(p, PV1_E_ARG, "FF->I learning time constants must be > 0");
    if (!(l->decayTimeHomeoFF > 0) || l->tauAvgCortical < 0) return fail(p, PV1_E_ARG, "bad time constant");
    if (l->applyHomeo < 0 || l->applyHomeo > 2) return fail(p, PV1_E_ARG, "applyHomeo is 0, 1 or 2");
    const pv1_v1_config &c = p->cfg;
    V1Params &v = p->vp;
    auto type_of = [&](bool inh, FFType &T, float *expHomeo) {
        pv1_ff_learning q = *l;
        if (inh) {
            q.tauLTP = l->tauLTP_I; q.tauLTD = l->tauLTD_I; q.tauTrip = l->tauTrip_I; q.tauAvg = l->tauAvg_I;
            q.targetFR = l->targetFR_I; q.A_LGN = l->A_LGN_I; q.r_LTD = l->r_LTD_I; q.gmaxLGN = l->gmaxLGN_I;
            q.gminLGN = l->gminLGN_I; q.sRatioLGN = l->sRatioLGN_I;
        }
        float r[5];
        pv1_ff_learning_rates(&q, c.dt, r);
        T = FFType{q.tauLTP, q.tauLTD, q.tauTrip, q.tauAvg, q.targetFR, r[0], r[1], r[2], r[3]};
        if (expHomeo) *expHomeo = r[4];
    };
    float expHomeo = 0.f;
    type_of(false, v.ffT[0], &expHomeo);
    type_of(true, v.ffT[1], nullptr);
    const size_t n = p->nV1;
    // the homeostasis totals: each neuron's LGN weights summed in synapse order, and that
    // times FF_InfRatio (src/patch.cu:4335-4352)
    std::vector<float> s((size_t)v.maxLGN * n), tot(2 * n, 0.f);
    std::vector<int> m(n);
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    if (!s.empty()) PV1_CUDA(p, cudaMemcpy(s.data(), v.sLGN, s.size() * sizeof(float), cudaMemcpyDeviceToHost));
    PV1_CUDA(p, cudaMemcpy(m.data(), v.nLGNperV1, n * sizeof(int), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) {
        float t = 0.f;
        for (int j = 0; j < m[i]; j++) t += s[(size_t)j * n + i];
        tot[i] = t;
        tot[n + i] = t * l->FF_InfRatio;
    }
    v.ffMode = mode;
    v.ffLearn = mode <= 3;
    v.ffI = nI_;
    v.ffTypes = nE_ + nI_;
    const size_t nEt = (size_t)p->nE * c.nblock, nIt = (size_t)p->nI * c.nblock;
    v.ffOffI = (int)(mode == 4 ? 0 : 2 * nEt);
    v.ffOffAvgE = v.ffOffI + (int)(2 * (size_t)nI_ * nIt);
    v.ffOffAvgI = v.ffOffAvgE + (int)(2 * nEt);
    float *d_post = nullptr, *d_tot = nullptr, *d_pre = nullptr;
    int r = 0;
    r |= dev_alloc(p, &d_post, ff_post_floats(p));
    r |= dev_upload(p, &d_tot, tot.data(), tot.size());
    r |= dev_alloc(p, &d_pre, (size_t)std::max(v.ffTypes, 1) * p->nLGN);
    if (r) return r;
    v.applyHomeo = l->applyHomeo;
    v.symmetricHomeo = l->symmetricHomeo != 0;
    v.rebound = l->rebound != 0;
    v.expHomeo = expHomeo;
    v.tauAvgCortical = l->tauAvgCortical;
    v.ffPost = d_post;
    v.totalFF = d_tot;
    v.sLGNw = const_cast<float *>(v.sLGN);
    p->lp.nFF = v.ffTypes;
    p->lp.tauLTP[0] = nE_ ? v.ffT[0].tauLTP : v.ffT[1].tauLTP;
    p->lp.tauLTP[1] = v.ffT[1].tauLTP;
    p->lp.ffPre = d_pre;
    r = ensure_ff_ring(p);
    if (r) return r;
    drop_graph(p);
    return PV1_OK;
}

int pv1_v1_set_near(pv1_plan *p, uint32_t nnb, const uint32_t *nNearNB, const uint32_t *nbId,
                    const float *conMat) {
    if (!p || !nNearNB || !nbId || !conMat || nnb < 1) return PV1_E_ARG;
    const int nblock = (int)p->cfg.nblock;
    for (int b = 0; b < nblock; b++) {
        if (nNearNB[b] > nnb) return fail(p, PV1_E_ARG, "nNearNeighborBlock > nearNeighborBlock");
        for (uint32_t q = 0; q < nNearNB[b]; q++)
            if (nbId[(size_t)b * nnb + q] >= (uint32_t)nblock) return fail(p, PV1_E_ARG, "neighbour block id out of range");
    }
    const size_t bs = p->cfg.blockSize;
    // for each pre block, the tiles whose rows its spikers' deliveries read (the kernels send
    // those rows to L2 when the spike happens, a step before the delivery)
    std::vector<int> revOff(nblock + 1, 0), rev;
    for (int pb = 0; pb < nblock; pb++) {
        for (int b = 0; b < nblock; b++)
            for (uint32_t q = 0; q < nNearNB[b]; q++)
                if ((int)nbId[(size_t)b * nnb + q] == pb) rev.push_back(b * (int)nnb + (int)q);
        revOff[pb + 1] = (int)rev.size();
    }
    int *d_n, *d_id, *d_ro, *d_rev = nullptr;
    float *d_c;
    int r = 0;
    r |= dev_upload(p, &d_n, (const int *)nNearNB, nblock);
    r |= dev_upload(p, &d_id, (const int *)nbId, (size_t)nblock * nnb);
    r |= dev_upload(p, &d_c, conMat, (size_t)nblock * nnb * bs * bs);
    r |= dev_upload(p, &d_ro, revOff.data(), revOff.size());
    if (!rev.empty()) r |= dev_upload(p, &d_rev, rev.data(), rev.size());
    if (r) return r;
    p->vp.nnbMax = (int)nnb;
    p->vp.nNearNB = d_n;
    p->vp.nbId = d_id;
    p->vp.conMat = d_c;
    p->vp.nearRevOff = d_ro;
    p->vp.nearRev = d_rev;
    p->haveNear = true;
    drop_graph(p);
    return PV1_OK;
}

}  // extern "C"

namespace {

// Builds the outgoing event lists by pre-neuron from delayed synapses (far ones, and the
// near ones when noDelay = 0) and uploads them: post id, strength, whole-step delay, sub-step
// offset, post type and class (near/far) per synapse.  Within a list the synapses with a
// whole-step delay <= 1 come first, because their events can arrive within the spike's own
// step.  The delay arithmetic is recal_G_vec's / recal_G_mat's (src/coredynamics.cu:282-287,
// 2163-2166), in float.
int build_event_lists(pv1_plan *p, const std::vector<EvSyn> &syn) {
    const int nV1 = p->nV1;
    const pv1_v1_config &c = p->cfg;
    const size_t nnz = syn.size();
    V1Params &v = p->vp;
    if (nnz == 0) {
        v.farOn = 0;
        v.nearOn = 0;
        v.farClass = 0;
        drop_graph(p);
        return PV1_OK;
    }
    std::vector<int> off(nV1 + 1, 0), n1(nV1, 0);
    std::vector<unsigned> it2(nnz);
    std::vector<float> t2p(nnz);
    for (size_t e = 0; e < nnz; e++) {
        off[syn[e].pre + 1]++;
        float time2post = syn[e].dist / c.speedOfThought;
        const unsigned it2post = (unsigned)std::ceil(time2post / c.dt);
        it2[e] = it2post;
        t2p[e] = it2post * c.dt - time2post;
        if (it2post <= 1) n1[syn[e].pre]++;
    }
    for (int i = 0; i < nV1; i++) off[i + 1] += off[i];
    std::vector<int> fillShort(off.begin(), off.end() - 1), fill(nV1);
    for (int i = 0; i < nV1; i++) fill[i] = off[i] + n1[i];
    std::vector<int> post(nnz), steps(nnz);
    std::vector<float> str(nnz), frac(nnz);
    std::vector<unsigned char> isPre(nV1, 0);
    int maxSteps = 0;
    bool anyFar = false, anyNear = false;
    for (size_t e = 0; e < nnz; e++) {
        const int pre = syn[e].pre, i = syn[e].post;
        const unsigned it2post = it2[e];
        const int slot = it2post <= 1 ? fillShort[pre]++ : fill[pre]++;
        post[slot] = i;
        str[slot] = syn[e].str;
        if (it2post > 0xffff) return fail(p, PV1_E_UNSUPPORTED, "synaptic delay longer than 65535 steps");
        // whole-step delay in the low 16 bits, the post neuron's type above, the class at bit 24
        int ptype = (int)c.nType - 1;
        for (int jt = (int)c.nType - 1; jt >= 0; jt--)
            if ((uint32_t)(i % (int)c.blockSize) < c.typeAcc[jt]) ptype = jt;
        steps[slot] = (int)it2post | (ptype << 16) | (syn[e].near ? (1 << 24) : 0);
        frac[slot] = t2p[e];
        if (!syn[e].near) isPre[pre] = 1;
        anyFar |= !syn[e].near;
        anyNear |= syn[e].near != 0;
        maxSteps = std::max(maxSteps, (int)it2post);
    }
    int *d_off, *d_post, *d_steps, *d_n1;
    unsigned long long *d_count;
    float *d_str, *d_frac;
    unsigned char *d_pre;
    unsigned long long *d_acc, *d_nacc = nullptr;
    int4 *d_list;
    const int depth = maxSteps + 2;
    const size_t ringLen = (size_t)depth * (c.ngE + c.ngI) * 2 * nV1;
    int r = 0;
    r |= dev_upload(p, &d_off, off.data(), off.size());
    r |= dev_upload(p, &d_n1, n1.data(), n1.size());
    r |= dev_alloc(p, &d_list, (size_t)3 * nV1);
    r |= dev_alloc(p, &d_count, 3);
    r |= dev_upload(p, &d_post, post.data(), nnz);
    r |= dev_upload(p, &d_steps, steps.data(), nnz);
    r |= dev_upload(p, &d_str, str.data(), nnz);
    r |= dev_upload(p, &d_frac, frac.data(), nnz);
    // the same four values packed per synapse (one 16-byte load in the push)
    std::vector<int4> rec(nnz);
    for (size_t e = 0; e < nnz; e++) {
        float fs = str[e], ff = frac[e];
        int bs_, bf_;
        memcpy(&bs_, &fs, 4);
        memcpy(&bf_, &ff, 4);
        rec[e] = make_int4(post[e], bs_, steps[e], bf_);
    }
    int4 *d_rec;
    r |= dev_upload(p, &d_rec, rec.data(), nnz);
    r |= dev_upload(p, &d_pre, isPre.data(), nV1);
    r |= dev_alloc(p, &d_acc, ringLen);
    if (anyNear) r |= dev_alloc(p, &d_nacc, ringLen);
    if (r) return r;
    v.farOn = 1;
    v.farClass = anyFar ? 1 : 0;
    v.nearOn = anyNear ? 1 : 0;
    v.farOff = d_off;
    v.farPost = d_post;
    v.farSteps = d_steps;
    v.farStr = d_str;
    v.farFrac = d_frac;
    v.farRec = d_rec;
    v.farPre = d_pre;
    v.farAcc = d_acc;
    v.nearAcc = d_nacc;
    v.farDepth = depth;
    v.farN1 = d_n1;
    v.farList = d_list;
    v.farCount = d_count;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    drop_graph(p);
    return PV1_OK;
}

int rebuild_events(pv1_plan *p) {
    std::vector<EvSyn> all;
    all.reserve(p->farSyn.size() + p->nearSyn.size());
    all.insert(all.end(), p->farSyn.begin(), p->farSyn.end());
    all.insert(all.end(), p->nearSyn.begin(), p->nearSyn.end());
    return build_event_lists(p, all);
}

}  // namespace

extern "C" {

// The spike-word ring read by the pulled deliveries: at least D rows, zero-filled (no spikes
// before the first step).
static int ensure_spike_ring(pv1_plan *p, int D) {
    V1Params &v = p->vp;
    if (v.sRing && v.sDepth >= D) return PV1_OK;
    if (v.sRing) free_one(p, v.sRing);
    v.sRing = nullptr;
    float *d = nullptr;
    int r = dev_alloc(p, &d, (size_t)D * p->nV1);
    if (r) return r;
    v.sRing = d;
    v.sDepth = D;
    return PV1_OK;
}

// Far synapses by post in the reference's vec order for the failure path: pre, strength,
// whole-step delay and offset (as build_event_lists computes them), failure rate and its
// normed std per (pre type, post type), the spike-word ring and the per-step scratch.
static int build_far_pull(pv1_plan *p, const uint32_t *nVec, const uint32_t *vecID, const float *conVec,
                          const float *delayVec, size_t nnz) {
    const int nV1 = p->nV1;
    const pv1_v1_config &c = p->cfg;
    V1Params &v = p->vp;
    auto typeOf = [&](int local) {
        int t = (int)c.nType - 1;
        for (int j = (int)c.nType - 1; j >= 0; j--)
            if ((uint32_t)local < c.typeAcc[j]) t = j;
        return t;
    };
    std::vector<int> off(nV1 + 1, 0), pre(nnz), steps(nnz);
    std::vector<float> str(nnz), frac(nnz), pf(nnz), sd(nnz);
    std::vector<unsigned char> isPre(nV1, 0);
    int maxSteps = 0;
    size_t e = 0;
    for (int i = 0; i < nV1; i++) {
        off[i + 1] = off[i] + (int)nVec[i];
        const int itype = typeOf(i % (int)c.blockSize);
        for (uint32_t j = 0; j < nVec[i]; j++, e++) {
            const int q = (int)vecID[e];
            pre[e] = q;
            str[e] = conVec[e];
            float time2post = delayVec[e] / c.speedOfThought;
            const unsigned it2post = (unsigned)std::ceil(time2post / c.dt);
            if (it2post > 0xffff) return fail(p, PV1_E_UNSUPPORTED, "synaptic delay longer than 65535 steps");
            steps[e] = (int)it2post;
            frac[e] = it2post * c.dt - time2post;
            maxSteps = std::max(maxSteps, (int)it2post);
            const int jtype = typeOf(q % (int)c.blockSize);
            const float fp = c.synFail[jtype * c.nType + itype];
            pf[e] = fp;
            sd[e] = fp > 0 ? std::sqrt(fp * (1 - fp) / c.synPerCon[jtype * c.nType + itype]) : 0.f;
            isPre[q] = 1;
        }
    }
    const int D = maxSteps + 2;
    const int ns = (int)(c.ngE + c.ngI);
    int *d_off, *d_pre, *d_steps, *d_cnt, *d_start, *d_prev, *d_flag;
    float *d_str, *d_frac, *d_p, *d_sd, *d_carry, *d_pull;
    unsigned char *d_isPre;
    unsigned *d_eng;
    int r = 0;
    r |= dev_upload(p, &d_off, off.data(), off.size());
    r |= dev_upload(p, &d_pre, pre.data(), nnz);
    r |= dev_upload(p, &d_steps, steps.data(), nnz);
    r |= dev_upload(p, &d_str, str.data(), nnz);
    r |= dev_upload(p, &d_frac, frac.data(), nnz);
    r |= dev_upload(p, &d_p, pf.data(), nnz);
    r |= dev_upload(p, &d_sd, sd.data(), nnz);
    r |= dev_upload(p, &d_isPre, isPre.data(), nV1);
    r |= ensure_spike_ring(p, D);
    r |= dev_alloc(p, &d_eng, nV1);
    r |= dev_alloc(p, &d_cnt, nV1);
    r |= dev_alloc(p, &d_start, nV1);
    r |= dev_alloc(p, &d_prev, nV1);
    r |= dev_alloc(p, &d_carry, nV1);
    r |= dev_alloc(p, &d_pull, (size_t)ns * 2 * nV1);
    r |= dev_alloc(p, &d_flag, 3);
    if (r) return r;
    v.farPullOn = 1;
    v.pullOff = d_off;
    v.pullPre = d_pre;
    v.pullSteps = d_steps;
    v.pullStr = d_str;
    v.pullFrac = d_frac;
    v.pullP = d_p;
    v.pullStd = d_sd;
    v.pullIsPre = d_isPre;
    v.eng = d_eng;
    v.pullCount = d_cnt;
    v.pullStart = d_start;
    v.pullPrev = d_prev;
    v.pullCarry = d_carry;
    v.farPull = d_pull;
    v.pullFlag = d_flag;
    p->haveFarEng = false;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    return PV1_OK;
}

int pv1_v1_far_failure_engines(pv1_plan *p, uint64_t seed, uint32_t nChunk) {
    if (!p || nChunk < 1) return PV1_E_ARG;
    const pv1_v1_config &c = p->cfg;
    V1Params &v = p->vp;
    if (!v.farPullOn) return PV1_OK;
    // chunks of blocks as src/patch.cu:3430-3437 splits them: the first nblock % nChunk chunks
    // one block longer
    const int nb = (int)c.nblock;
    const int nCh = std::min<int>((int)nChunk, nb);
    const int split = nb % nCh, rem = nb / nCh, maxC = rem + (split > 0 ? 1 : 0);
    std::vector<int> cs(nCh + 1, 0);
    for (int q = 0; q < nCh; q++) cs[q + 1] = cs[q] + (q < split ? maxC : rem) * (int)c.blockSize;
    std::vector<unsigned> eng(p->nV1);
    for (int i = 0; i < p->nV1; i++) {
        const uint64_t x = (seed + (uint64_t)i) % 2147483647ull;   // minstd_rand0::seed
        eng[i] = x == 0 ? 1u : (unsigned)x;
    }
    if (v.chunkStart) free_one(p, (void *)v.chunkStart);
    int *d_cs;
    int r = dev_upload(p, &d_cs, cs.data(), cs.size());
    if (r) return r;
    v.chunkStart = d_cs;
    v.nChunk = nCh;
    PV1_CUDA(p, cudaMemcpyAsync(v.eng, eng.data(), eng.size() * sizeof(unsigned), cudaMemcpyHostToDevice, p->stream));
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    p->haveFarEng = true;
    drop_graph(p);
    return PV1_OK;
}

int pv1_v1_set_far(pv1_plan *p, const uint32_t *nVec, const uint32_t *vecID, const float *conVec,
                   const float *delayVec) {
    if (!p || !nVec) return PV1_E_ARG;
    const int nV1 = p->nV1;
    const pv1_v1_config &c = p->cfg;
    size_t nnz = 0;
    for (int i = 0; i < nV1; i++) nnz += nVec[i];
    if (nnz && (!vecID || !conVec || !delayVec)) return PV1_E_ARG;
    p->nFarSyn = (long long)nnz;
    p->farSyn.clear();
    bool failure = false;
    for (int q = 0; q < (int)(c.nType * c.nType); q++) failure = failure || c.synFail[q] > 0;
    p->vp.farPullOn = 0;
    if (nnz && !c.noFarDelay && failure) {
        // far synaptic failure: pulled by post in vec order (pv1_far_pull.cu)
        for (size_t e = 0; e < nnz; e++)
            if (vecID[e] >= (uint32_t)nV1) return fail(p, PV1_E_ARG, "far pre id out of range");
        int r = build_far_pull(p, nVec, vecID, conVec, delayVec, nnz);
        if (r) return r;
    } else if (nnz && !c.noFarDelay) {
        // (noFarDelay = 1 is the reference's path that drops far input)
        p->farSyn.resize(nnz);
        size_t e = 0;
        for (int i = 0; i < nV1; i++)
            for (uint32_t j = 0; j < nVec[i]; j++, e++) {
                if (vecID[e] >= (uint32_t)nV1) return fail(p, PV1_E_ARG, "far pre id out of range");
                p->farSyn[e] = EvSyn{(int)vecID[e], i, conVec[e], delayVec[e], 0};
            }
    }
    int r = rebuild_events(p);
    if (c.noDelay) p->farSyn.clear();   // kept only while near lists may still be merged in
    return r;
}

// Near connectivity with distance delays (noDelay = 0): recal_G_mat
// (src/coredynamics.cu:2063-2309) delivers every non-zero conMat entry of the near blocks at
// the arrival step of its delayMat distance.  Here those entries become delayed events of the
// same event lists as the far synapses (class "near": no far-spike gate on delivery).
// Distance-delayed near synapses with synaptic failure, by post in recal_G_mat's order (near
// blocks as listed, then pre neurons by index, src/coredynamics.cu:2138-2170): pre, strength,
// whole-step delay and offset (ceil(delay/speed/dt) and it2post*dt - delay/speed in float),
// failure rate and normed std of the (pre type, post type) pair -- the pre type from the pre
// neuron's index.
static int build_near_pull(pv1_plan *p, uint32_t nnb, const uint32_t *nNearNB, const uint32_t *nbId,
                           const float *conMat, const float *delayMat) {
    const pv1_v1_config &c = p->cfg;
    const int nV1 = p->nV1, nblock = (int)c.nblock;
    const size_t bs = c.blockSize;
    auto typeOf = [&](int local) {
        int t = (int)c.nType - 1;
        for (int j = (int)c.nType - 1; j >= 0; j--)
            if ((uint32_t)local < c.typeAcc[j]) t = j;
        return t;
    };
    std::vector<int> off(nV1 + 1, 0), pre, steps;
    std::vector<float> str, frac, pf, sd;
    int maxSteps = 0;
    for (int b = 0; b < nblock; b++) {
        if (nNearNB[b] > nnb) return fail(p, PV1_E_ARG, "nNearNeighborBlock > nearNeighborBlock");
        for (size_t j = 0; j < bs; j++) {
            const int post = (int)(b * bs + j);
            const int itype = typeOf((int)j);
            for (uint32_t k = 0; k < nNearNB[b]; k++) {
                const uint32_t nb = nbId[(size_t)b * nnb + k];
                if (nb >= (uint32_t)nblock) return fail(p, PV1_E_ARG, "neighbour block id out of range");
                const size_t base = ((size_t)b * nnb + k) * bs * bs;
                for (size_t i = 0; i < bs; i++) {
                    const float sv = conMat[base + i * bs + j];
                    if (sv == 0) continue;
                    float time2post = delayMat[base + i * bs + j] / c.speedOfThought;
                    const unsigned it2post = (unsigned)std::ceil(time2post / c.dt);
                    if (it2post > 0xffff) return fail(p, PV1_E_UNSUPPORTED, "synaptic delay longer than 65535 steps");
                    const int jtype = typeOf((int)i);
                    const float fp = c.synFail[jtype * c.nType + itype];
                    pre.push_back((int)(nb * bs + i));
                    steps.push_back((int)it2post);
                    str.push_back(sv);
                    frac.push_back(it2post * c.dt - time2post);
                    pf.push_back(fp);
                    sd.push_back(fp > 0 ? std::sqrt(fp * (1 - fp) / c.synPerCon[jtype * c.nType + itype]) : 0.f);
                    maxSteps = std::max(maxSteps, (int)it2post);
                }
            }
            off[post + 1] = (int)pre.size();
        }
    }
    const size_t nnz = pre.size();
    int *d_off, *d_pre, *d_steps;
    float *d_str, *d_frac, *d_p, *d_sd;
    int r = 0;
    r |= dev_upload(p, &d_off, off.data(), off.size());
    r |= dev_upload(p, &d_pre, pre.data(), nnz);
    r |= dev_upload(p, &d_steps, steps.data(), nnz);
    r |= dev_upload(p, &d_str, str.data(), nnz);
    r |= dev_upload(p, &d_frac, frac.data(), nnz);
    r |= dev_upload(p, &d_p, pf.data(), nnz);
    r |= dev_upload(p, &d_sd, sd.data(), nnz);
    if (r) return r;
    r = ensure_spike_ring(p, maxSteps + 2);
    if (r) return r;
    V1Params &v = p->vp;
    v.nearPullOn = 1;
    v.npOff = d_off;
    v.npPre = d_pre;
    v.npSteps = d_steps;
    v.npStr = d_str;
    v.npFrac = d_frac;
    v.npP = d_p;
    v.npStd = d_sd;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    drop_graph(p);
    return PV1_OK;
}

int pv1_v1_set_near_delayed(pv1_plan *p, uint32_t nnb, const uint32_t *nNearNB, const uint32_t *nbId,
                            const float *conMat, const float *delayMat) {
    if (!p || !nNearNB || !nbId || !conMat || !delayMat || nnb < 1) return PV1_E_ARG;
    const pv1_v1_config &c = p->cfg;
    if (c.noDelay) return fail(p, PV1_E_STATE, "pv1_v1_set_near_delayed is for noDelay = 0 plans");
    bool failure = false;
    for (int q = 0; q < (int)(c.nType * c.nType); q++) failure = failure || c.synFail[q] > 0;
    const int nblock = (int)c.nblock;
    const size_t bs = c.blockSize;
    p->nearSyn.clear();
    p->vp.nearPullOn = 0;
    if (failure) {
        int r = build_near_pull(p, nnb, nNearNB, nbId, conMat, delayMat);
        if (r) return r;
        p->haveNear = true;
        return rebuild_events(p);
    }
    for (int b = 0; b < nblock; b++) {
        if (nNearNB[b] > nnb) return fail(p, PV1_E_ARG, "nNearNeighborBlock > nearNeighborBlock");
        for (uint32_t k = 0; k < nNearNB[b]; k++) {
            const uint32_t nb = nbId[(size_t)b * nnb + k];
            if (nb >= (uint32_t)nblock) return fail(p, PV1_E_ARG, "neighbour block id out of range");
            const size_t base = ((size_t)b * nnb + k) * bs * bs;
            for (size_t i = 0; i < bs; i++)
                for (size_t j = 0; j < bs; j++) {
                    const float s = conMat[base + i * bs + j];
                    if (s != 0)
                        p->nearSyn.push_back(EvSyn{(int)(nb * bs + i), (int)(b * bs + j), s, delayMat[base + i * bs + j], 1});
                }
        }
    }
    p->haveNear = true;
    return rebuild_events(p);
}

int pv1_v1_set_state(pv1_plan *p, const float *v, const float *w, const float *gFF,
                     const float *hFF, const float *gE, const float *hE, const float *gI,
                     const float *hI, const float *tonicDep) {
    if (!p || !v || !gFF || !hFF || !gE || !hE || !gI || !hI || !tonicDep) return PV1_E_ARG;
    const size_t n = p->nV1;
    const pv1_v1_config &c = p->cfg;
    V1Params &vp = p->vp;
    auto up = [&](float *dst, const float *src, size_t cnt) {
        return cudaMemcpyAsync(dst, src, cnt * sizeof(float), cudaMemcpyHostToDevice, p->stream);
    };
    PV1_CUDA(p, up(vp.v, v, n));
    if (w) PV1_CUDA(p, up(vp.w, w, n));
    else PV1_CUDA(p, cudaMemsetAsync(vp.w, 0, n * sizeof(float), p->stream));
    PV1_CUDA(p, up(vp.gFF, gFF, c.ngFF * n));
    PV1_CUDA(p, up(vp.hFF, hFF, c.ngFF * n));
    PV1_CUDA(p, up(vp.gE, gE, c.ngE * n));
    PV1_CUDA(p, up(vp.hE, hE, c.ngE * n));
    PV1_CUDA(p, up(vp.gI, gI, c.ngI * n));
    PV1_CUDA(p, up(vp.hI, hI, c.ngI * n));
    PV1_CUDA(p, up(vp.tonicDep, tonicDep, n));
    PV1_CUDA(p, cudaMemsetAsync(vp.tBack, 0, n * sizeof(float), p->stream));
    PV1_CUDA(p, cudaMemsetAsync(vp.lastNoise, 0, n * sizeof(float), p->stream));
    PV1_CUDA(p, cudaMemsetAsync(vp.sInfo, 0, 2 * n * sizeof(float), p->stream));
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    p->haveState = true;
    p->pending = false;
    return PV1_OK;
}

int pv1_v1_init_rng(pv1_plan *p, uint64_t seed, uint32_t trainDepth) {
    if (!p || trainDepth < 1) return PV1_E_ARG;
    PV1_CUDA(p, launch_v1_rng_init(p->vp.rGenCond, p->vp.rNoisy, (unsigned long long)seed, p->nV1,
                                   (int)trainDepth, p->stream));
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    p->haveRng = true;
    return PV1_OK;
}

int pv1_v1_init_spikes(pv1_plan *p, uint64_t seed, uint32_t trainDepth, const float *sp0, uint32_t SCsplit,
                       pv1_init_record *rec) {
    if (!p || trainDepth < 1 || !sp0) return PV1_E_ARG;
    const pv1_v1_config &c = p->cfg;
    if (!p->haveState || !p->haveNear) return fail(p, PV1_E_STATE, "set the state and the connectivity first");
    if (p->step != 0) return fail(p, PV1_E_STATE, "initial spikes are set before the first step");
    if (p->vp.farPullOn && !p->haveFarEng)
        return fail(p, PV1_E_STATE, "far synaptic failure: call pv1_v1_far_failure_engines first");
    if (c.blockSize > 1024) return fail(p, PV1_E_UNSUPPORTED, "initial spikes need blockSize <= 1024");
    Sp0 s0{};
    bool has = false;
    for (uint32_t q = 0; q < 2 * c.nType; q++) {
        if (!(sp0[q] >= 0 && sp0[q] <= 1)) return fail(p, PV1_E_ARG, "sp0 holds per-step chances in [0, 1]");
        s0.c[q] = sp0[q];
        has = has || sp0[q] > 0;
    }
    if (has && p->vp.nearPullOn)
        return fail(p, PV1_E_UNSUPPORTED,
                    "initial spikes with synaptic failure on distance-delayed near synapses are not built");
    const V1Params &vp = p->vp;
    const size_t n = p->nV1;
    const int depth = (int)trainDepth;
    const bool nearNd = has && c.noDelay;
    const size_t ncb = (size_t)p->nE * c.ngE + (size_t)p->nI * c.ngI;
    const uint32_t cap = rec && rec->normals ? rec->normalCap : 0;
    float *dH = nullptr, *dOg = nullptr, *dOh = nullptr, *dU = nullptr, *dZ = nullptr;
    unsigned *dNU = nullptr, *dNZ = nullptr;
    int r = dev_alloc(p, &dH, (size_t)depth * n);
    if (!r && nearNd) r = dev_alloc(p, &dOg, ncb * c.nblock);
    if (!r && nearNd) r = dev_alloc(p, &dOh, ncb * c.nblock);
    if (!r && rec && rec->uniforms) r = dev_alloc(p, &dU, (size_t)2 * depth * n);
    if (!r && rec && rec->nUniform) r = dev_alloc(p, &dNU, n);
    if (!r && cap) r = dev_alloc(p, &dZ, (size_t)cap * n);
    if (!r && rec && rec->nNormal) r = dev_alloc(p, &dNZ, n);
    auto cleanup = [&]() {
        for (void *q : {(void *)dH, (void *)dOg, (void *)dOh, (void *)dU, (void *)dZ, (void *)dNU, (void *)dNZ})
            if (q) free_one(p, q);
    };
    if (r) {
        cleanup();
        return r;
    }
    cudaError_t e = launch_v1_sp_init(vp, (unsigned long long)seed, depth, s0, (int)SCsplit, dH, dOg, dOh, dU, dNU,
                                      p->stream);
    if (e == cudaSuccess && nearNd)
        e = launch_v1_sp_near(vp, dH + (size_t)(depth - 1) * n, dOg, dOh, dZ, dNZ, (int)cap, p->stream);
    if (e == cudaSuccess && has && vp.farOn) {
        e = cudaMemsetAsync(vp.farFlag, 0, 3 * sizeof(int), p->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(vp.farCount, 0, 3 * sizeof(unsigned long long), p->stream);
        if (e == cudaSuccess) e = launch_v1_sp_events(vp, dH, depth, p->stream);
    }
    if (e == cudaSuccess && has && vp.farPullOn) {
        // far failure path: the history slot depth-1 is step -1 of the spike-word ring
        e = cudaMemcpyAsync(vp.sRing + (size_t)(vp.sDepth - 1) * n, dH + (size_t)(depth - 1) * n, n * sizeof(float),
                            cudaMemcpyDeviceToDevice, p->stream);
        if (e == cudaSuccess) e = launch_far_pull(vp, nullptr, -1, p->stream);
        if (e == cudaSuccess) e = launch_far_pull_apply(vp, p->stream);
    }
    auto down = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && dst && src) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, p->stream);
    };
    if (rec) {
        down(rec->uniforms, dU, (size_t)2 * depth * n * sizeof(float));
        down(rec->nUniform, dNU, n * sizeof(unsigned));
        down(rec->normals, dZ, (size_t)cap * n * sizeof(float));
        down(rec->history, dH, (size_t)depth * n * sizeof(float));
        if (rec->nNormal) {
            if (dNZ) down(rec->nNormal, dNZ, n * sizeof(unsigned));
            else memset(rec->nNormal, 0, n * sizeof(uint32_t));
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    cleanup();
    if (e != cudaSuccess) return fail(p, PV1_E_CUDA, cudaGetErrorString(e));
    p->haveRng = true;
    drop_graph(p);
    return check_device_error(p);
}

int pv1_set_record(pv1_plan *p, int flags, uint32_t slots) {
    if (!p) return PV1_E_ARG;
    if (!p->lgnReady) return fail(p, PV1_E_STATE, "call pv1_lgn_setup first");
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    if (flags && slots < 2) return fail(p, PV1_E_ARG, "record ring needs >= 2 slots");
    const pv1_v1_config &c = p->cfg;
    if (p->d_rec) { free_one(p, p->d_rec); p->d_rec = nullptr; }
    if (p->d_lgnFr) { free_one(p, p->d_lgnFr); p->d_lgnFr = nullptr; }
    const long long n = p->nV1;
    p->recStride = pv1_raw_record_floats(p);
    p->recFlags = flags;
    p->recSlots = flags ? (int)slots : 0;
    if (flags & PV1_REC_RAW) {
        int r = dev_alloc(p, &p->d_rec, (size_t)slots * p->recStride);
        if (r) return r;
    }
    if (p->vp.recSpk) { free_one(p, p->vp.recSpk); p->vp.recSpk = nullptr; }
    if (flags & PV1_REC_SPIKES) {
        int r = dev_alloc(p, &p->vp.recSpk, (size_t)slots * n);
        if (r) return r;
    }
    // the LGN ring doubles as the LGN_sp record when it is at least `slots` rows long
    int want = std::max(2 * p->K, 2);
    if (flags & (PV1_REC_LGN_SP | PV1_REC_LGN_FR)) want = std::max<int>(want, (int)slots);
    if (want != p->lgnSlots) {
        free_one(p, p->d_lgnRing);
        p->lgnSlots = want;
        int r = dev_alloc(p, &p->d_lgnRing, (size_t)want * p->nLGN);
        if (r) return r;
    }
    if (flags & PV1_REC_LGN_FR) {
        int r = dev_alloc(p, &p->d_lgnFr, (size_t)want * p->nLGN);
        if (r) return r;
    }
    p->lp.outSInfo = p->d_lgnRing;
    p->lp.outFr = p->d_lgnFr;
    p->lp.outSlots = p->lgnSlots;
    {
        int r = ensure_ff_ring(p);
        if (r) return r;
    }
    p->vp.rec = p->d_rec;
    p->vp.recStride = p->recStride;
    p->vp.recSlots = (flags & (PV1_REC_RAW | PV1_REC_SPIKES)) ? (int)slots : 1;
    (void)n;
    (void)c;
    drop_graph(p);
    return PV1_OK;
}

int64_t pv1_raw_record_floats(const pv1_plan *p) {
    if (!p) return -1;
    const pv1_v1_config &c = p->cfg;
    const long long n = p->nV1;
    const long long mI = (long long)p->nI * c.nblock;
    long long fl = n * (1 + 2 + (c.iModel == 1) + (long long)c.ngFF * (1 + (c.hWrite != 0)) +
                        (long long)(c.ngE + c.ngI) * (1 + (c.hWrite != 0)));
    return fl + mI;
}

// Chooses between the persistent cooperative V1 kernel and per-step launches (once the
// connectivity is known): persistent when every CTA can be resident at once and the LGN
// synapse lists fit in registers.
static int choose_mode(pv1_plan *p) {
    if (p->modeChosen) return PV1_OK;
    bool fits = false;
    int push = 0;
    v1_persistent_ctas(p->vp, p->device, &fits, &push);
    p->persistent = fits && p->allowPersistent && !p->vp.multiSpike && !p->vp.farPullOn && !p->vp.nearPullOn &&
                    !p->vp.ffMode;
    p->vp.pushCta = p->persistent ? push : 0;
    if (p->persistent && !p->d_barrier) {
        int r = dev_alloc(p, &p->d_barrier, 2);
        if (r) return r;
    }
    p->modeChosen = true;
    return PV1_OK;
}

int pv1_set_lgn_source(pv1_plan *p, const float *d_sInfo, int64_t step0, int64_t nsteps) {
    if (!p) return PV1_E_ARG;
    if (!d_sInfo) {
        p->extLgn = nullptr;
        p->extSteps = 0;
        drop_graph(p);
        return PV1_OK;
    }
    if (!p->lgnReady) return fail(p, PV1_E_STATE, "call pv1_lgn_setup first (it gives the LGN cell count)");
    if (step0 < 0 || nsteps <= 0) return fail(p, PV1_E_ARG, "bad step range");
    if (p->vp.ffMode)
        return fail(p, PV1_E_UNSUPPORTED, "an external LGN source has no presynaptic learning traces");
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, d_sInfo) != cudaSuccess || a.type != cudaMemoryTypeDevice || a.device != p->device) {
        cudaGetLastError();
        return fail(p, PV1_E_ARG, "the LGN source must be device memory of the plan's device");
    }
    p->extLgn = d_sInfo;
    p->extStep0 = step0;
    p->extSteps = nsteps;
    drop_graph(p);
    return PV1_OK;
}

int pv1_set_wait_limit(pv1_plan *p, int64_t spins) {
    if (!p) return PV1_E_ARG;
    if (spins < 0) spins = kDefaultWaitSpins;
    p->vp.waitSpins = spins;
    drop_graph(p);   // captured launches hold the old parameters
    return PV1_OK;
}

int pv1_run(pv1_plan *p, uint32_t nsteps, int sync) {
    if (!p) return PV1_E_ARG;
    if (p->lgnOnly) return fail(p, PV1_E_STATE, "the plan was stepped by pv1_lgn_spikes_noalloc (LGN only)");
    if (!p->lgnReady || !p->stimReady) return fail(p, PV1_E_STATE, "LGN/stimulus not loaded");
    if (!p->haveLGNsyn || !p->haveNear || !p->haveState || !p->haveRng)
        return fail(p, PV1_E_STATE, "V1 synapses/connectivity/state/rng not set");
    if (p->vp.farPullOn && !p->haveFarEng)
        return fail(p, PV1_E_STATE, "far synaptic failure: call pv1_v1_far_failure_engines first");
    if (p->recFlags && nsteps > (uint32_t)(p->recSlots - 1))
        return fail(p, PV1_E_ARG, "run longer than the record ring; fetch records in between");
    int r = choose_mode(p);
    if (r) return r;
    r = ensure_frames(p, p->step + (long long)nsteps - 1);
    if (r) return r;
    p->launches = 0;
    PV1_CUDA(p, cudaMemcpyAsync(p->d_stepBase, &p->step, sizeof(long long), cudaMemcpyHostToDevice, p->stream));
    uint32_t done = 0;
    const int K = p->K;
    // the first chunk of a run without a pending delivery differs from the captured one
    if (!p->pending && nsteps > 0) {
        int k = (int)std::min<uint32_t>(nsteps, (uint32_t)K);
        r = issue_chunk(p, p->step, k, 0, &p->launches);
        if (r) return r;
        r = sink_rows(p, p->step + (long long)done, k);
        if (r) return r;
        done += k;
    }
    if (nsteps - done >= (uint32_t)K) {
        if (p->persistent && p->lgnSlots >= 2 * K) {
            // one cooperative V1 launch per chunk on the plan's stream; the LGN of the next chunk
            // of this run (never beyond it) on the LGN stream meanwhile, into the other half of
            // the ring, after the V1 launch that read that half has finished
            if (!p->lgnStream) {
                PV1_CUDA(p, cudaStreamCreateWithFlags(&p->lgnStream, cudaStreamNonBlocking));
                PV1_CUDA(p, cudaEventCreateWithFlags(&p->evLgn, cudaEventDisableTiming));
                PV1_CUDA(p, cudaEventCreateWithFlags(&p->evFree, cudaEventDisableTiming));
                r = dev_alloc(p, &p->d_lgnStep, 1);
                if (r) return r;
            }
            const int nFull = (int)((nsteps - done) / (uint32_t)K);
            const long long t0 = p->step + (long long)done;
            PV1_CUDA(p, cudaMemcpyAsync(p->d_lgnStep, &t0, sizeof(long long), cudaMemcpyHostToDevice, p->stream));
            r = lgn_stage(p, t0, K, p->d_lgnStep, p->stream, &p->launches);
            if (r) return r;
            cudaError_t e = launch_advance_step(p->d_lgnStep, K, p->stream);
            if (e != cudaSuccess) return fail(p, PV1_E_CUDA, std::string("lgn_step: ") + cudaGetErrorString(e));
            p->launches += 1;
            for (int c = 0; c < nFull; c++) {
                if (c > 0) PV1_CUDA(p, cudaStreamWaitEvent(p->stream, p->evLgn, 0));
                PV1_CUDA(p, cudaEventRecord(p->evFree, p->stream));   // chunk c-1's V1 is done
                e = launch_v1_persistent(p->vp, p->d_stepBase, K, p->d_lgnRing, p->lgnSlots, 1, p->d_barrier,
                                         p->stream);
                if (e == cudaSuccess) e = launch_advance_step(p->d_stepBase, K, p->stream);
                if (e != cudaSuccess) return fail(p, PV1_E_CUDA, std::string("v1_persistent: ") + cudaGetErrorString(e));
                p->launches += 2;
                r = sink_rows(p, t0 + (long long)c * K, K);
                if (r) return r;
                if (c + 1 < nFull) {
                    PV1_CUDA(p, cudaStreamWaitEvent(p->lgnStream, p->evFree, 0));
                    r = lgn_stage(p, t0 + (long long)(c + 1) * K, K, p->d_lgnStep, p->lgnStream, &p->launches);
                    if (r) return r;
                    e = launch_advance_step(p->d_lgnStep, K, p->lgnStream);
                    if (e != cudaSuccess) return fail(p, PV1_E_CUDA, std::string("lgn_step: ") + cudaGetErrorString(e));
                    PV1_CUDA(p, cudaEventRecord(p->evLgn, p->lgnStream));
                    p->launches += 1;
                }
                done += K;
            }
        } else if (p->persistent) {
            // a cooperative launch per chunk: issued directly (4 launches per K steps)
            while (nsteps - done >= (uint32_t)K) {
                r = issue_chunk(p, p->step + (long long)done, K, 1, &p->launches);
                if (r) return r;
                r = sink_rows(p, p->step + (long long)done, K);
                if (r) return r;
                done += K;
            }
        } else if (p->extLgn) {
            // the copies of an external source differ chunk by chunk: issued directly
            while (nsteps - done >= (uint32_t)K) {
                r = issue_chunk(p, p->step + (long long)done, K, 1, &p->launches);
                if (r) return r;
                r = sink_rows(p, p->step + (long long)done, K);
                if (r) return r;
                done += K;
            }
        } else {
            long long per = 0;
            if (!p->graphExec) {
                cudaGraph_t g;
                PV1_CUDA(p, cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
                r = issue_chunk(p, p->step + (long long)done, K, 1, &per);
                cudaError_t e2 = cudaStreamEndCapture(p->stream, &g);
                if (r) return r;
                if (e2 != cudaSuccess) return fail(p, PV1_E_CUDA, std::string("capture: ") + cudaGetErrorString(e2));
                PV1_CUDA(p, cudaGraphInstantiate(&p->graphExec, g, 0));
                cudaGraphDestroy(g);
                p->graphLaunches = per;
            }
            while (nsteps - done >= (uint32_t)K) {
                PV1_CUDA(p, cudaGraphLaunch(p->graphExec, p->stream));
                p->launches += p->graphLaunches;
                r = sink_rows(p, p->step + (long long)done, K);
                if (r) return r;
                done += K;
            }
        }
    }
    if (done < nsteps) {
        int k = (int)(nsteps - done);
        r = issue_chunk(p, p->step + (long long)done, k, 1, &p->launches);
        if (r) return r;
        r = sink_rows(p, p->step + (long long)done, k);
        if (r) return r;
        done += k;
    }
    p->step += nsteps;
    if (nsteps > 0) p->pending = true;
    if (sync) return check_device_error(p);
    return PV1_OK;
}

int64_t pv1_last_launch_count(const pv1_plan *p) { return p ? p->launches : -1; }

int pv1_run_spikes_to_host(pv1_plan *p, uint32_t nsteps, float *out) {
    if (!p || (!out && nsteps)) return PV1_E_ARG;
    if (!(p->recFlags & PV1_REC_SPIKES)) return fail(p, PV1_E_STATE, "spike recording is off");
    if (!p->copyStream) {
        PV1_CUDA(p, cudaStreamCreateWithFlags(&p->copyStream, cudaStreamNonBlocking));
        PV1_CUDA(p, cudaEventCreateWithFlags(&p->evChunk, cudaEventDisableTiming));
        PV1_CUDA(p, cudaEventCreateWithFlags(&p->evCopied, cudaEventDisableTiming));
    }
    p->sinkHost = out;
    p->sinkStep0 = p->step;
    int r = pv1_run(p, nsteps, 0);
    p->sinkHost = nullptr;
    if (r) {
        cudaStreamSynchronize(p->copyStream);
        return r;
    }
    // the plan's stream continues after the copies (later runs overwrite the ring)
    PV1_CUDA(p, cudaEventRecord(p->evCopied, p->copyStream));
    PV1_CUDA(p, cudaStreamWaitEvent(p->stream, p->evCopied, 0));
    PV1_CUDA(p, cudaStreamSynchronize(p->copyStream));
    return check_device_error(p);
}

int pv1_fetch_spikes(pv1_plan *p, uint64_t step0, uint32_t n, float *out) {
    if (!p || !out) return PV1_E_ARG;
    if (!(p->recFlags & PV1_REC_SPIKES)) return fail(p, PV1_E_STATE, "spike recording is off");
    if (step0 + n > (uint64_t)p->step) return fail(p, PV1_E_ARG, "records not produced yet");
    if ((uint64_t)p->step - step0 > (uint64_t)p->recSlots) return fail(p, PV1_E_ARG, "records already overwritten");
    const size_t nV1 = p->nV1;
    // contiguous slot ranges, one or two copies
    uint32_t done = 0;
    while (done < n) {
        const uint64_t t = step0 + done;
        const uint32_t slot = (uint32_t)(t % p->recSlots);
        const uint32_t cnt = std::min<uint32_t>(n - done, (uint32_t)p->recSlots - slot);
        PV1_CUDA(p, cudaMemcpyAsync(out + (size_t)done * nV1, p->vp.recSpk + (size_t)slot * nV1,
                                    (size_t)cnt * nV1 * sizeof(float), cudaMemcpyDeviceToHost, p->stream));
        done += cnt;
    }
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    return PV1_OK;
}

int pv1_run_timed(pv1_plan *p, uint32_t nsteps, uint64_t flush_bytes, float *ms) {
    if (!p || !ms) return PV1_E_ARG;
    if (flush_bytes > p->flushSize) {
        if (p->flushBuf) free_one(p, p->flushBuf);
        p->flushBuf = nullptr;
        p->flushSize = 0;
        unsigned char *buf = nullptr;
        int r = dev_alloc(p, &buf, flush_bytes);
        if (r) return r;
        p->flushBuf = buf;
        p->flushSize = flush_bytes;
    }
    cudaEvent_t e0, e1;
    PV1_CUDA(p, cudaEventCreate(&e0));
    PV1_CUDA(p, cudaEventCreate(&e1));
    if (flush_bytes) PV1_CUDA(p, cudaMemsetAsync(p->flushBuf, (int)(p->step & 0xff), flush_bytes, p->stream));
    PV1_CUDA(p, cudaEventRecord(e0, p->stream));
    int r = pv1_run(p, nsteps, 0);
    if (r) return r;
    PV1_CUDA(p, cudaEventRecord(e1, p->stream));
    PV1_CUDA(p, cudaEventSynchronize(e1));
    PV1_CUDA(p, cudaEventElapsedTime(ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return check_device_error(p);
}

int pv1_time_kernels(pv1_plan *p, uint32_t nsteps, float *v1_ms, float *lgn_ms, int *chunk) {
    if (!p || !v1_ms || !lgn_ms) return PV1_E_ARG;
    if (p->extLgn) return fail(p, PV1_E_STATE, "pv1_time_kernels times the plan's own LGN stage");
    if (p->lgnOnly) return fail(p, PV1_E_STATE, "the plan was stepped by pv1_lgn_spikes_noalloc (LGN only)");
    if (!p->lgnReady || !p->stimReady || !p->haveState || !p->haveRng || !p->haveNear || !p->haveLGNsyn)
        return fail(p, PV1_E_STATE, "plan not ready");
    int r = choose_mode(p);
    if (r) return r;
    const int K = p->K;
    const uint32_t nchunk = nsteps / K;
    if (nchunk == 0) return fail(p, PV1_E_ARG, "nsteps < chunk");
    r = ensure_frames(p, p->step + (long long)nchunk * K - 1);
    if (r) return r;
    std::vector<cudaEvent_t> ev(3 * nchunk);
    for (auto &e : ev) PV1_CUDA(p, cudaEventCreate(&e));
    PV1_CUDA(p, cudaMemcpyAsync(p->d_stepBase, &p->step, sizeof(long long), cudaMemcpyHostToDevice, p->stream));
    for (uint32_t c = 0; c < nchunk; c++) {
        const int deliverFirst = (c == 0) ? (p->pending ? 1 : 0) : 1;
        PV1_CUDA(p, cudaEventRecord(ev[3 * c], p->stream));
        PV1_CUDA(p, launch_lgn_step(p->lp, p->d_stepBase, K, p->stream));
        PV1_CUDA(p, cudaEventRecord(ev[3 * c + 1], p->stream));
        if (p->persistent) {
            PV1_CUDA(p, launch_v1_persistent(p->vp, p->d_stepBase, K, p->d_lgnRing, p->lgnSlots, deliverFirst,
                                             p->d_barrier, p->stream));
        } else {
            for (int s = 0; s < K; s++)
                PV1_CUDA(p, launch_v1_step(p->vp, p->d_stepBase, s, p->d_lgnRing, p->lgnSlots,
                                           s == 0 ? deliverFirst : 1, 1, p->stream));
        }
        PV1_CUDA(p, cudaEventRecord(ev[3 * c + 2], p->stream));
        PV1_CUDA(p, launch_advance_step(p->d_stepBase, K, p->stream));
    }
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    double tl = 0, tv = 0;
    for (uint32_t c = 0; c < nchunk; c++) {
        float a, b;
        PV1_CUDA(p, cudaEventElapsedTime(&a, ev[3 * c], ev[3 * c + 1]));
        PV1_CUDA(p, cudaEventElapsedTime(&b, ev[3 * c + 1], ev[3 * c + 2]));
        tl += a;
        tv += b;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    p->step += (long long)nchunk * K;
    p->pending = true;
    *v1_ms = (float)(tv / ((double)nchunk * K));
    *lgn_ms = (float)(tl / nchunk);
    if (chunk) *chunk = K;
    return check_device_error(p);
}

int pv1_persistent_mode(pv1_plan *p, int allow) {
    if (!p) return PV1_E_ARG;
    if (allow >= 0) {
        p->allowPersistent = allow != 0;
        p->modeChosen = false;
        drop_graph(p);
    }
    int r = choose_mode(p);
    if (r) return r;
    return p->persistent ? 1 : 0;
}

// Applies the delivery of the last step's spikes (kept pending so that the next step can
// fuse it), so that g/h and the last record are complete.
static int flush_delivery(pv1_plan *p) {
    if (!p->pending) return PV1_OK;
    PV1_CUDA(p, cudaMemcpyAsync(p->d_stepBase, &p->step, sizeof(long long), cudaMemcpyHostToDevice, p->stream));
    PV1_CUDA(p, launch_v1_step(p->vp, p->d_stepBase, 0, p->d_lgnRing, p->lgnSlots, 1, 0, p->stream));
    p->pending = false;
    return check_device_error(p);
}

// ---- minimal output ----
int pv1_sample_ids(uint64_t seed, uint32_t nblock, uint32_t blockSize, uint32_t nE, uint32_t sampleSize,
                   uint32_t *out, uint32_t *nOut) {
    if (!out || !nOut || nE > blockSize) return PV1_E_ARG;
    std::vector<unsigned> exc;
    for (uint32_t i = 0; i < nblock; i++)
        for (uint32_t j = 0; j < nE; j++) exc.push_back(i * blockSize + j);
    std::vector<unsigned> ids;
    if ((uint64_t)sampleSize > exc.size()) {
        ids = exc;
    } else {
        std::default_random_engine gen(seed);
        std::sample(exc.begin(), exc.end(), std::back_inserter(ids), sampleSize, gen);
    }
    std::copy(ids.begin(), ids.end(), out);
    *nOut = (uint32_t)ids.size();
    return PV1_OK;
}

// ---- framed output ----
int pv1_frames_setup(pv1_plan *p, uint32_t nPixel, uint32_t nSpikePixel, const uint32_t *pixOff,
                     const uint32_t *pixIds, uint32_t ot, float odt) {
    if (!p || !nPixel || nSpikePixel > nPixel || !pixOff || ot < 1 || !(odt > 0)) return PV1_E_ARG;
    const uint32_t nIds = pixOff[nPixel];
    if (nIds && !pixIds) return PV1_E_ARG;
    for (uint32_t q = 0; q < nPixel; q++) {
        if (pixOff[q + 1] < pixOff[q]) return fail(p, PV1_E_ARG, "pixel offsets must not decrease");
        const uint32_t lim = q < nSpikePixel ? (uint32_t)p->nV1 : (uint32_t)p->nLGN;
        for (uint32_t j = pixOff[q]; j < pixOff[q + 1]; j++)
            if (pixIds[j] >= lim) return fail(p, PV1_E_ARG, "pixel cell id out of range");
    }
    for (void *q : {(void *)p->d_pixOff, (void *)p->d_pixIds, (void *)p->d_frameAcc, (void *)p->d_frameOut})
        if (q) free_one(p, q);
    p->d_frameOut = nullptr;
    p->frameOutCap = 0;
    int r = dev_upload(p, &p->d_pixOff, pixOff, (size_t)nPixel + 1);
    if (!r) r = dev_upload(p, &p->d_pixIds, nIds ? pixIds : pixOff, nIds ? nIds : 1);
    if (!r) r = dev_alloc(p, &p->d_frameAcc, nPixel);
    if (r) return r;
    p->nPixel = (int)nPixel;
    p->nSpikePixel = (int)nSpikePixel;
    p->frameOt = (int)ot;
    p->frameOdt = odt;
    p->frameT0 = p->step;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    return PV1_OK;
}

int pv1_frames_collect(pv1_plan *p, uint64_t step0, uint32_t n, float *frames, uint32_t *nFrames) {
    if (!p || !nFrames) return PV1_E_ARG;
    if (!p->d_pixOff) return fail(p, PV1_E_STATE, "call pv1_frames_setup first");
    if (p->nSpikePixel > 0 && !p->vp.recSpk) return fail(p, PV1_E_STATE, "V1 frames read the PV1_REC_SPIKES record");
    if (p->nPixel > p->nSpikePixel && !p->d_lgnFr) return fail(p, PV1_E_STATE, "LGN frames read the PV1_REC_LGN_FR record");
    if (step0 + n > (uint64_t)p->step) return fail(p, PV1_E_ARG, "steps not run yet");
    if ((uint64_t)p->step - step0 > (uint64_t)p->recSlots) return fail(p, PV1_E_ARG, "spike records already overwritten");
    uint32_t k = 0;
    for (uint32_t s = 0; s < n; s++)
        if (((long long)(step0 + s) - p->frameT0 + 1) % p->frameOt == 0) k++;
    if (k > 0 && !frames) return PV1_E_ARG;
    if ((int)k > p->frameOutCap) {
        if (p->d_frameOut) free_one(p, p->d_frameOut);
        int r = dev_alloc(p, &p->d_frameOut, (size_t)k * p->nPixel);
        if (r) return r;
        p->frameOutCap = (int)k;
    }
    PV1_CUDA(p, launch_frames(p->vp.recSpk, p->vp.recSlots, p->nV1, p->d_lgnFr, p->lgnSlots, p->nLGN, (long long)step0,
                              (int)n, p->frameOt, p->frameT0, p->d_pixOff, p->d_pixIds, p->nPixel, p->nSpikePixel,
                              p->frameOdt, p->d_frameAcc, p->d_frameOut ? p->d_frameOut : p->d_frameAcc, p->stream));
    if (k) PV1_CUDA(p, cudaMemcpyAsync(frames, p->d_frameOut, (size_t)k * p->nPixel * sizeof(float),
                                       cudaMemcpyDeviceToHost, p->stream));
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    *nFrames = k;
    return PV1_OK;
}

// ---- checkpoints ----
// Everything that a step reads from the steps before it: the neuron state and generators,
// the last two spike-word rows, the delayed-event rings with their spiker lists and flags,
// the far-failure ring and engines, and the LGN cells' integrals and generators.  The
// delivery of the last step is applied first, so a checkpoint never holds a pending one.
namespace {

struct CkptHeader {
    char magic[8];
    uint32_t version, nV1, nLGN, ngFF, ngE, ngI;
    int32_t farDepth, sDepth, farOn, farPullOn, nItems, pad;
    int64_t step;
    uint64_t cfgHash, bytes;
};
static_assert(offsetof(CkptHeader, step) == 56, "the step field sits at byte 56 of a checkpoint");

uint64_t fnv1a(const void *data, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char *b = (const unsigned char *)data;
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

void ckpt_items(pv1_plan *p, std::vector<std::pair<void *, size_t>> &items) {
    const pv1_v1_config &c = p->cfg;
    V1Params &v = p->vp;
    const size_t n = p->nV1, f = sizeof(float);
    items.clear();
    auto add = [&](void *ptr, size_t bytes) {
        if (ptr && bytes) items.emplace_back(ptr, bytes);
    };
    add(v.v, n * f);
    add(v.w, n * f);
    add(v.tBack, n * f);
    add(v.dep, n * f);
    add(v.gFF, c.ngFF * n * f);
    add(v.hFF, c.ngFF * n * f);
    add(v.gE, c.ngE * n * f);
    add(v.hE, c.ngE * n * f);
    add(v.gI, c.ngI * n * f);
    add(v.hI, c.ngI * n * f);
    add(v.lastNoise, n * f);
    add(v.rGenCond, n * sizeof(curandStateMRG32k3a));
    add(v.rNoisy, n * sizeof(curandStateMRG32k3a));
    add(v.sInfo, 2 * n * f);
    const size_t ring = (size_t)v.farDepth * (c.ngE + c.ngI) * 2 * n * sizeof(unsigned long long);
    if (v.farOn) {
        add(v.farAcc, ring);
        if (v.nearOn) add(v.nearAcc, ring);
        add(v.farFlag, 3 * sizeof(int));
        add(v.farList, 3 * n * sizeof(int4));
        add(v.farCount, 3 * sizeof(unsigned long long));
    }
    if (v.nearPullOn && !v.farPullOn) add(v.sRing, (size_t)v.sDepth * n * f);
    if (v.farPullOn) {
        add(v.sRing, (size_t)v.sDepth * n * f);
        add(v.eng, n * sizeof(unsigned));
        add(v.farPull, (size_t)(c.ngE + c.ngI) * 2 * n * f);
        add(v.pullFlag, 3 * sizeof(int));
    }
    add(p->lp.leftTimeRate, p->nLGN * f);
    add(p->lp.lastNegLogRand, p->nLGN * f);
    add(p->lp.state, p->nLGN * sizeof(curandStateMRG32k3a));
    if (v.ffMode) {
        add(v.sLGNw, (size_t)v.maxLGN * n * f);
        add(v.ffPost, ff_post_floats(p) * f);
        add(v.totalFF, 2 * n * f);
        add(p->lp.ffPre, (size_t)p->lp.nFF * p->nLGN * f);
    }
}

CkptHeader ckpt_header(pv1_plan *p, const std::vector<std::pair<void *, size_t>> &items) {
    CkptHeader h{};
    memcpy(h.magic, "PV1CKPT", 8);
    h.version = 1;
    h.nV1 = (uint32_t)p->nV1;
    h.nLGN = (uint32_t)p->nLGN;
    h.ngFF = p->cfg.ngFF;
    h.ngE = p->cfg.ngE;
    h.ngI = p->cfg.ngI;
    h.farDepth = p->vp.farOn ? p->vp.farDepth : 0;
    h.sDepth = (p->vp.farPullOn || p->vp.nearPullOn) ? p->vp.sDepth : 0;
    h.farOn = p->vp.farOn;
    h.farPullOn = p->vp.farPullOn;
    h.nItems = (int32_t)items.size();
    h.step = p->step;
    h.cfgHash = fnv1a(&p->cfg, sizeof(p->cfg));
    uint64_t bytes = sizeof(CkptHeader);
    for (auto &it : items) bytes += it.second;
    h.bytes = bytes;
    return h;
}

}  // namespace

int pv1_checkpoint_size(pv1_plan *p, uint64_t *bytes) {
    if (!p || !bytes) return PV1_E_ARG;
    if (!p->haveState || !p->haveRng || !p->lgnReady) return fail(p, PV1_E_STATE, "plan not initialised");
    std::vector<std::pair<void *, size_t>> items;
    ckpt_items(p, items);
    *bytes = ckpt_header(p, items).bytes;
    return PV1_OK;
}

int pv1_checkpoint_save(pv1_plan *p, void *buf, uint64_t bytes) {
    if (!p || !buf) return PV1_E_ARG;
    if (p->lgnOnly) return fail(p, PV1_E_STATE, "the plan was stepped by pv1_lgn_spikes_noalloc (LGN only)");
    if (!p->haveState || !p->haveRng || !p->lgnReady) return fail(p, PV1_E_STATE, "plan not initialised");
    int r = flush_delivery(p);
    if (r) return r;
    std::vector<std::pair<void *, size_t>> items;
    ckpt_items(p, items);
    const CkptHeader h = ckpt_header(p, items);
    if (bytes < h.bytes) return fail(p, PV1_E_ARG, "checkpoint buffer too small (pv1_checkpoint_size)");
    char *out = (char *)buf;
    memcpy(out, &h, sizeof(h));
    size_t off = sizeof(h);
    for (auto &it : items) {
        PV1_CUDA(p, cudaMemcpyAsync(out + off, it.first, it.second, cudaMemcpyDeviceToHost, p->stream));
        off += it.second;
    }
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    return PV1_OK;
}

int pv1_set_step(pv1_plan *p, int64_t step) {
    if (!p || step < 0) return PV1_E_ARG;
    if (!p->haveState || !p->haveRng || !p->lgnReady) return fail(p, PV1_E_STATE, "plan not initialised");
    if (p->lgnOnly) return fail(p, PV1_E_STATE, "the plan was stepped by pv1_lgn_spikes_noalloc (LGN only)");
    if (!p->cfg.noDelay)
        return fail(p, PV1_E_UNSUPPORTED,
                    "state loaded array by array with distance-delayed near synapses (noDelay = 0): the "
                    "events in flight would need the spike-word history");
    V1Params &v = p->vp;
    const size_t n = p->nV1, ns = p->cfg.ngE + p->cfg.ngI;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    auto zero = [&](void *ptr, size_t bytes) {
        return ptr ? cudaMemsetAsync(ptr, 0, bytes, p->stream) : cudaSuccess;
    };
    if (v.farOn) {
        const size_t ring = (size_t)v.farDepth * ns * 2 * n * sizeof(unsigned long long);
        PV1_CUDA(p, zero(v.farAcc, ring));
        PV1_CUDA(p, zero(v.nearAcc, ring));
        PV1_CUDA(p, zero(v.farCount, 3 * sizeof(unsigned long long)));
        PV1_CUDA(p, zero(v.farFlag, 3 * sizeof(int)));
    }
    if (v.farPullOn) {
        PV1_CUDA(p, zero(v.farPull, ns * 2 * n * sizeof(float)));
        PV1_CUDA(p, zero(v.pullFlag, 3 * sizeof(int)));
    }
    PV1_CUDA(p, zero(v.sRing, (size_t)v.sDepth * n * sizeof(float)));
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    p->step = step;
    p->pending = false;
    drop_graph(p);
    return PV1_OK;
}

int pv1_checkpoint_load(pv1_plan *p, const void *buf, uint64_t bytes) {
    if (!p || !buf || bytes < sizeof(CkptHeader)) return PV1_E_ARG;
    if (!p->haveState || !p->haveRng || !p->lgnReady) return fail(p, PV1_E_STATE, "plan not initialised");
    CkptHeader h;
    memcpy(&h, buf, sizeof(h));
    std::vector<std::pair<void *, size_t>> items;
    ckpt_items(p, items);
    CkptHeader mine = ckpt_header(p, items);
    if (memcmp(h.magic, "PV1CKPT", 8) != 0 || h.version != 1) return fail(p, PV1_E_ARG, "not a checkpoint");
    if (h.cfgHash != mine.cfgHash || h.nV1 != mine.nV1 || h.nLGN != mine.nLGN || h.farDepth != mine.farDepth ||
        h.sDepth != mine.sDepth || h.farOn != mine.farOn || h.farPullOn != mine.farPullOn ||
        h.nItems != mine.nItems || h.bytes != mine.bytes || bytes < h.bytes)
        return fail(p, PV1_E_ARG, "checkpoint of a different configuration or network");
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    const char *in = (const char *)buf;
    size_t off = sizeof(h);
    for (auto &it : items) {
        PV1_CUDA(p, cudaMemcpyAsync(it.first, in + off, it.second, cudaMemcpyHostToDevice, p->stream));
        off += it.second;
    }
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    p->step = h.step;
    p->pending = false;
    drop_graph(p);
    return PV1_OK;
}

int pv1_fetch_records(pv1_plan *p, uint64_t step0, uint32_t n, float *raw, float *lgn_sp, float *lgn_fr) {
    if (!p) return PV1_E_ARG;
    if (!p->recFlags) return fail(p, PV1_E_STATE, "recording is off");
    if (step0 + n > (uint64_t)p->step) return fail(p, PV1_E_ARG, "records not produced yet");
    if ((uint64_t)p->step - step0 > (uint64_t)p->recSlots) return fail(p, PV1_E_ARG, "records already overwritten");
    if (step0 + n == (uint64_t)p->step) {
        int r = flush_delivery(p);  // completes the g/h of the last record
        if (r) return r;
    }
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    for (uint32_t s = 0; s < n; s++) {
        const uint64_t t = step0 + s;
        if (raw && (p->recFlags & PV1_REC_RAW)) {
            const size_t slot = t % p->recSlots;
            PV1_CUDA(p, cudaMemcpy(raw + (size_t)s * p->recStride, p->d_rec + slot * p->recStride,
                                   (p->recStride - (long long)p->nI * p->cfg.nblock) * sizeof(float),
                                   cudaMemcpyDeviceToHost));
            // gap junction values (InhGap is not built): zero
            std::fill(raw + (size_t)s * p->recStride + (p->recStride - (long long)p->nI * p->cfg.nblock),
                      raw + (size_t)(s + 1) * p->recStride, 0.0f);
        }
        const size_t lrow = t % p->lgnSlots;
        if (lgn_sp && (p->recFlags & PV1_REC_LGN_SP))
            PV1_CUDA(p, cudaMemcpy(lgn_sp + (size_t)s * p->nLGN, p->d_lgnRing + lrow * p->nLGN,
                                   p->nLGN * sizeof(float), cudaMemcpyDeviceToHost));
        if (lgn_fr && (p->recFlags & PV1_REC_LGN_FR))
            PV1_CUDA(p, cudaMemcpy(lgn_fr + (size_t)s * p->nLGN, p->d_lgnFr + lrow * p->nLGN,
                                   p->nLGN * sizeof(float), cudaMemcpyDeviceToHost));
    }
    return PV1_OK;
}

int pv1_get_state(pv1_plan *p, int which, float *out) {
    if (!p || !out) return PV1_E_ARG;
    int r = flush_delivery(p);
    if (r) return r;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    const size_t n = p->nV1;
    const pv1_v1_config &c = p->cfg;
    const V1Params &v = p->vp;
    const void *src = nullptr;
    size_t cnt = n;
    switch (which) {
        case PV1_ST_V: src = v.v; break;
        case PV1_ST_W: src = v.w; break;
        case PV1_ST_TBACK: src = v.tBack; break;
        case PV1_ST_DEP: src = v.dep; break;
        case PV1_ST_GFF: src = v.gFF; cnt = c.ngFF * n; break;
        case PV1_ST_HFF: src = v.hFF; cnt = c.ngFF * n; break;
        case PV1_ST_GE: src = v.gE; cnt = c.ngE * n; break;
        case PV1_ST_HE: src = v.hE; cnt = c.ngE * n; break;
        case PV1_ST_GI: src = v.gI; cnt = c.ngI * n; break;
        case PV1_ST_HI: src = v.hI; cnt = c.ngI * n; break;
        case PV1_ST_SINFO:
            if (p->step == 0) return fail(p, PV1_E_STATE, "no step run yet");
            src = v.sInfo + (size_t)((p->step - 1) & 1) * n;
            break;
        case PV1_ST_LGN_LTR: src = p->lp.leftTimeRate; cnt = p->nLGN; break;
        case PV1_ST_LGN_LNL: src = p->lp.lastNegLogRand; cnt = p->nLGN; break;
        case PV1_ST_LGN_SINFO:
            if (p->step == 0) return fail(p, PV1_E_STATE, "no step run yet");
            src = p->d_lgnRing + (size_t)((p->step - 1) % p->lgnSlots) * p->nLGN;
            cnt = p->nLGN;
            break;
        case PV1_ST_FAR_PULL:
            if (!v.farPullOn) return fail(p, PV1_E_STATE, "no far synaptic failure in this plan");
            src = v.farPull;
            cnt = (size_t)(c.ngE + c.ngI) * 2 * n;
            break;
        case PV1_ST_LGN_RNG: src = p->lp.state; cnt = p->nLGN * (sizeof(curandStateMRG32k3a) / sizeof(float)); break;
        case PV1_ST_V1_RNG_COND: src = v.rGenCond; cnt = n * (sizeof(curandStateMRG32k3a) / sizeof(float)); break;
        case PV1_ST_V1_RNG_NOISY: src = v.rNoisy; cnt = n * (sizeof(curandStateMRG32k3a) / sizeof(float)); break;
        case PV1_ST_SLGN: src = v.sLGN; cnt = (size_t)v.maxLGN * n; break;
        case PV1_ST_FF_POST: src = v.ffPost; cnt = ff_post_floats(p); break;
        case PV1_ST_FF_PRE: src = p->lp.ffPre; cnt = (size_t)p->lp.nFF * p->nLGN; break;
        case PV1_ST_TOTAL_FF: src = v.totalFF; cnt = 2 * n; break;
        default: return fail(p, PV1_E_ARG, "unknown state id");
    }
    if (!src) return fail(p, PV1_E_STATE, "state not allocated");
    PV1_CUDA(p, cudaMemcpy(out, src, cnt * sizeof(float), cudaMemcpyDeviceToHost));
    return PV1_OK;
}

int pv1_put_state(pv1_plan *p, int which, const float *in) {
    if (!p || !in) return PV1_E_ARG;
    int r = flush_delivery(p);
    if (r) return r;
    const size_t n = p->nV1;
    const pv1_v1_config &c = p->cfg;
    const V1Params &v = p->vp;
    void *dst = nullptr;
    size_t cnt = n;
    switch (which) {
        case PV1_ST_V: dst = v.v; break;
        case PV1_ST_W: dst = v.w; break;
        case PV1_ST_TBACK: dst = v.tBack; break;
        case PV1_ST_GFF: dst = v.gFF; cnt = c.ngFF * n; break;
        case PV1_ST_HFF: dst = v.hFF; cnt = c.ngFF * n; break;
        case PV1_ST_GE: dst = v.gE; cnt = c.ngE * n; break;
        case PV1_ST_HE: dst = v.hE; cnt = c.ngE * n; break;
        case PV1_ST_GI: dst = v.gI; cnt = c.ngI * n; break;
        case PV1_ST_HI: dst = v.hI; cnt = c.ngI * n; break;
        case PV1_ST_DEP: dst = v.dep; break;
        case PV1_ST_LGN_LTR: dst = p->lp.leftTimeRate; cnt = p->nLGN; break;
        case PV1_ST_LGN_LNL: dst = p->lp.lastNegLogRand; cnt = p->nLGN; break;
        case PV1_ST_LGN_RNG: dst = p->lp.state; cnt = p->nLGN * (sizeof(curandStateMRG32k3a) / sizeof(float)); break;
        case PV1_ST_V1_RNG_COND: dst = v.rGenCond; cnt = n * (sizeof(curandStateMRG32k3a) / sizeof(float)); break;
        case PV1_ST_V1_RNG_NOISY: dst = v.rNoisy; cnt = n * (sizeof(curandStateMRG32k3a) / sizeof(float)); break;
        case PV1_ST_SLGN: dst = v.sLGNw; cnt = (size_t)v.maxLGN * n; break;
        case PV1_ST_FF_POST: dst = v.ffPost; cnt = ff_post_floats(p); break;
        case PV1_ST_FF_PRE: dst = p->lp.ffPre; cnt = (size_t)p->lp.nFF * p->nLGN; break;
        case PV1_ST_TOTAL_FF: dst = v.totalFF; cnt = 2 * n; break;
        default: return fail(p, PV1_E_ARG, "state id cannot be written");
    }
    if (!dst) return fail(p, PV1_E_STATE, "state not allocated");
    PV1_CUDA(p, cudaMemcpy(dst, in, cnt * sizeof(float), cudaMemcpyHostToDevice));
    return PV1_OK;
}

int pv1_set_draw_record(pv1_plan *p, uint32_t steps, uint32_t cap) {
    if (!p) return PV1_E_ARG;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    V1Params &v = p->vp;
    LgnParams &L = p->lp;
    void *old[] = {L.recU, L.recUCount, v.recNoise, v.recFF, v.recFFCount, v.recNear, v.recNearCount};
    for (void *o : old)
        if (o) free_one(p, o);
    L.recU = nullptr; L.recUCount = nullptr;
    v.recNoise = v.recFF = v.recNear = nullptr;
    v.recFFCount = v.recNearCount = nullptr;
    if (steps == 0 || cap == 0) {
        drop_graph(p);
        return PV1_OK;
    }
    int r = 0;
    const size_t nV1 = p->nV1, nLGN = std::max(p->nLGN, 1);
    r |= dev_alloc(p, &L.recU, steps * nLGN * cap);
    r |= dev_alloc(p, &L.recUCount, steps * nLGN);
    r |= dev_alloc(p, &v.recNoise, steps * nV1);
    r |= dev_alloc(p, &v.recFF, steps * nV1 * cap);
    r |= dev_alloc(p, &v.recFFCount, steps * nV1);
    r |= dev_alloc(p, &v.recNear, steps * nV1 * cap);
    r |= dev_alloc(p, &v.recNearCount, steps * nV1);
    if (r) return r;
    L.recCap = v.recCap = (int)cap;
    L.recSteps = v.recSteps = (int)steps;
    L.recStep0 = v.recStep0 = p->step;
    drop_graph(p);
    return PV1_OK;
}

int pv1_fetch_draws(pv1_plan *p, int kind, float *draws, int32_t *counts) {
    if (!p) return PV1_E_ARG;
    int r = flush_delivery(p);
    if (r) return r;
    PV1_CUDA(p, cudaStreamSynchronize(p->stream));
    const V1Params &v = p->vp;
    const LgnParams &L = p->lp;
    if (!v.recNoise) return fail(p, PV1_E_STATE, "draw recording is off");
    const size_t steps = v.recSteps, cap = v.recCap, nV1 = p->nV1, nLGN = std::max(p->nLGN, 1);
    const void *src = nullptr, *csrc = nullptr;
    size_t cnt = 0, ccnt = 0;
    switch (kind) {
        case 0: src = L.recU; cnt = steps * nLGN * cap; csrc = L.recUCount; ccnt = steps * nLGN; break;
        case 1: src = v.recNoise; cnt = steps * nV1; break;
        case 2: src = v.recFF; cnt = steps * nV1 * cap; csrc = v.recFFCount; ccnt = steps * nV1; break;
        case 3: src = v.recNear; cnt = steps * nV1 * cap; csrc = v.recNearCount; ccnt = steps * nV1; break;
        default: return fail(p, PV1_E_ARG, "unknown draw kind");
    }
    if (draws) PV1_CUDA(p, cudaMemcpy(draws, src, cnt * sizeof(float), cudaMemcpyDeviceToHost));
    if (counts && csrc) PV1_CUDA(p, cudaMemcpy(counts, csrc, ccnt * sizeof(int), cudaMemcpyDeviceToHost));
    return PV1_OK;
}

// ---- host initial state (src/patch.cu:4405-4560) -----------------------------------------
int pv1_host_init_state(const pv1_v1_config *cfg, uint64_t seed, const float *tonicDep,
                        const uint32_t *nLGNperV1, int use_v0, float tonicMax, const float *w0,
                        const float *gFF0, const float *gE0, const float *gI0, float *v, float *w,
                        float *gFF, float *hFF, float *gE, float *hE, float *gI, float *hI) {
    if (!cfg || !tonicDep || !nLGNperV1 || !v || !gFF || !hFF || !gE || !hE || !gI || !hI || !gFF0 ||
        !gE0 || !gI0)
        return PV1_E_ARG;
    const pv1_v1_config &c = *cfg;
    const size_t bs = c.blockSize, nblock = c.nblock, nV1 = bs * nblock;
    const int nType = (int)c.nType;
    std::vector<size_t> acc(nType + 1, 0);
    for (int j = 0; j < nType; j++) acc[j + 1] = c.typeAcc[j];
    std::default_random_engine rGen((std::default_random_engine::result_type)seed);
    // one normal distribution object shared by every draw, as the reference's function-local
    // static inside its sampling lambda is (src/patch.cu:4417-4429)
    std::normal_distribution<float> norm(0.0f, 1.0f);
    auto sampler = [&](float mean, float std, bool nonNeg) {
        return [&rGen, &norm, mean, std, nonNeg]() {
            float r;
            do {
                r = norm(rGen) * std + mean;
            } while (nonNeg && r < 0.0f);
            return r;
        };
    };
    for (int i = 0; i < nType; i++) {
        if (c.iModel == 1) {
            if (!w0 || !w) return PV1_E_ARG;
            auto get = sampler(w0[i * 2 + 0], w0[i * 2 + 1], false);
            for (size_t b = 0; b < nblock; b++)
                std::generate(w + b * bs + acc[i], w + b * bs + acc[i + 1], get);
        }
        if (use_v0 || tonicMax > 1.0f) {
            std::uniform_real_distribution<float> uni(c.vR[i], c.vT[i]);
            for (size_t b = 0; b < nblock; b++)
                std::generate(v + b * bs + acc[i], v + b * bs + acc[i + 1], [&]() { return uni(rGen); });
        } else {
            for (size_t b = 0; b < nblock; b++)
                for (size_t j = acc[i]; j < acc[i + 1]; j++)
                    v[b * bs + j] = c.vR[i] + (c.vT[i] - c.vR[i]) * tonicDep[b * bs + j];
        }
    }
    if (c.iModel != 1 && w) std::fill(w, w + nV1, 0.0f);
    const int ngFF = (int)c.ngFF, ngE = (int)c.ngE, ngI = (int)c.ngI;
    for (int i = 0; i < nType; i++) {
        for (int k = 0; k < ngFF; k++) {
            const float *q = gFF0 + (size_t)i * ngFF * 4 + k * 4;
            auto gg = sampler(q[0], q[0] * q[1], true);
            auto gh = sampler(q[2], q[2] * q[3], true);
            for (size_t b = 0; b < nblock; b++) {
                size_t ind = k * nV1 + b * bs;
                std::generate(gFF + ind + acc[i], gFF + ind + acc[i + 1], gg);
                std::generate(hFF + ind + acc[i], hFF + ind + acc[i + 1], gh);
                for (size_t j = acc[i]; j < acc[i + 1]; j++) {
                    if (nLGNperV1[b * bs + j] == 0) {
                        gFF[k * nV1 + b * bs + j] = 0;
                        hFF[k * nV1 + b * bs + j] = 0;
                    }
                }
            }
        }
    }
    for (int i = 0; i < nType; i++) {
        for (int k = 0; k < ngE; k++) {
            const float *q = gE0 + (size_t)i * ngE * 4 + k * 4;
            auto gg = sampler(q[0], q[0] * q[1], true);
            auto gh = sampler(q[2], q[2] * q[3], true);
            for (size_t b = 0; b < nblock; b++) {
                size_t off = k * nV1 + b * bs;
                std::generate(gE + off + acc[i], gE + off + acc[i + 1], gg);
                std::generate(hE + off + acc[i], hE + off + acc[i + 1], gh);
            }
        }
        for (int k = 0; k < ngI; k++) {
            const float *q = gI0 + (size_t)i * ngI * 4 + k * 4;
            auto gg = sampler(q[0], q[0] * q[1], true);
            auto gh = sampler(q[2], q[2] * q[3], true);
            for (size_t b = 0; b < nblock; b++) {
                size_t off = k * nV1 + b * bs;
                std::generate(gI + off + acc[i], gI + off + acc[i + 1], gg);
                std::generate(hI + off + acc[i], hI + off + acc[i + 1], gh);
            }
        }
    }
    return PV1_OK;
}

}  // extern "C"
