// Batched trials behind the C ABI (pv1_batch_*): many independent patches stepped by the
// same launches, replacing the reference's one-process-per-trial sweeps (src/ori.sh).
//
// Per chunk of K steps: one batched LGN launch (grid = cell CTAs x trials), then either one
// cooperative V1 launch that runs the K steps of every active trial with the trials' state in
// registers (slots of CTAs taking the trials in turn, a barrier per trial between steps) or K
// batched per-step V1 launches (grid = the active (trial, CTA) tiles of all trials), and one
// advance launch, captured once per (K, V1 variant) as a CUDA graph.  Every trial keeps its own device step counter;
// chunks run as a graph only while every active trial has K or more steps left, otherwise as
// direct launches of the smallest remainder, so no kernel steps a trial past its end and each
// trial computes exactly what pv1_run computes for it alone.  The tile list is rebuilt on the
// host when a trial ends (the V1 grid is sized for all tiles; CTAs past the list return).
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "pv1_internal.cuh"

using namespace pv1;

constexpr int kCandidates = 12;

struct pv1_batch {
    std::string err;
    int n = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<pv1_plan *> plans;
    std::vector<PlanBatchView> views;
    std::vector<BatchTrial> hT;
    std::vector<BatchLgn> hL;
    BatchTrial *dT = nullptr;
    BatchLgn *dL = nullptr;
    int2 *dTiles = nullptr;
    int *dNTiles = nullptr;
    int *dActive = nullptr, *dNActive = nullptr;   // active trial list (persistent variant)
    unsigned *dBar = nullptr;                      // per-trial barrier counters
    int slotCtas = 0, nSlots = 0;                  // persistent variant: CTAs per slot, slots
    int totalTiles = 0;
    int maxCellCtas = 0;
    bool allClass = true;
    bool rng = false;
    unsigned *dCounts = nullptr;
    long long *dCountOff = nullptr;
    std::vector<long long> countOff;
    double *dSimTime = nullptr;
    double *dMean = nullptr;
    std::vector<long long> step, end;
    std::vector<char> activeSet;
    std::vector<int2> hTiles;
    int hNTiles = 0;
    std::vector<int> hActive;
    int hNActive = 0;
    int K = 64, minB = 1;                    // minB 0: persistent variant, 1-3: per-step kernels
    bool tune = false;
    int nextCandidate = 0;
    float times[kCandidates];
    std::map<int, cudaGraphExec_t> graphs;   // key K*4 + minB
    long long launches = 0;
    std::vector<void *> allocs;
};

namespace {

const int kCandK[3] = {16, 32, 64};
// candidate c: chunk length kCandK[c / 4], V1 variant c % 4 (0: persistent, 1-3: minB)

int bfail(pv1_batch *b, int code, const std::string &m) {
    if (b) b->err = m;
    return code;
}

#define PV1_BCUDA(b, call)                                                                      \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return bfail((b), PV1_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
    } while (0)

template <class T>
int balloc(pv1_batch *b, T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) return bfail(b, PV1_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    b->allocs.push_back(*p);
    e = cudaMemsetAsync(*p, 0, n * sizeof(T), b->stream);
    if (e != cudaSuccess) return bfail(b, PV1_E_CUDA, cudaGetErrorString(e));
    return PV1_OK;
}

// Rebuilds the (trial, CTA) tile list of the trials that still have steps to run.
int refresh_tiles(pv1_batch *b) {
    std::vector<char> act(b->n);
    for (int q = 0; q < b->n; q++) act[q] = b->step[q] < b->end[q];
    if (act == b->activeSet) return PV1_OK;
    b->activeSet = act;
    b->hTiles.clear();
    for (int q = 0; q < b->n; q++)
        if (act[q])
            for (int c = 0; c < b->hT[q].nCta; c++) b->hTiles.push_back(make_int2(q, c));
    b->hNTiles = (int)b->hTiles.size();
    if (b->hNTiles)
        PV1_BCUDA(b, cudaMemcpyAsync(b->dTiles, b->hTiles.data(), b->hTiles.size() * sizeof(int2),
                                     cudaMemcpyHostToDevice, b->stream));
    PV1_BCUDA(b, cudaMemcpyAsync(b->dNTiles, &b->hNTiles, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    b->hActive.clear();
    for (int q = 0; q < b->n; q++)
        if (act[q]) b->hActive.push_back(q);
    b->hNActive = (int)b->hActive.size();
    if (b->hNActive)
        PV1_BCUDA(b, cudaMemcpyAsync(b->dActive, b->hActive.data(), b->hActive.size() * sizeof(int),
                                     cudaMemcpyHostToDevice, b->stream));
    PV1_BCUDA(b, cudaMemcpyAsync(b->dNActive, &b->hNActive, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    // the host vectors are reused by the next refresh: wait for the copies
    PV1_BCUDA(b, cudaStreamSynchronize(b->stream));
    return PV1_OK;
}

// One chunk of k steps for every active trial, on the batch stream (direct or under capture).
int issue(pv1_batch *b, int k, int minB, long long *launches) {
    long long n = 0;
    cudaError_t e;
    if (b->allClass) {
        e = launch_lgn_class_batch(b->dL, b->n, b->maxCellCtas, k, b->stream);
        if (e != cudaSuccess) return bfail(b, PV1_E_CUDA, std::string("lgn batch: ") + cudaGetErrorString(e));
        n += 1;
    } else {
        for (int q = 0; q < b->n; q++) {
            if (!b->activeSet[q]) continue;
            e = launch_lgn_step(b->views[q].lp, b->views[q].d_stepBase, k, b->stream);
            if (e != cudaSuccess) return bfail(b, PV1_E_CUDA, std::string("lgn step: ") + cudaGetErrorString(e));
            n += lgn_step_launches(b->views[q].lp, k);
        }
    }
    if (minB == 0) {
        e = launch_v1_batch_persistent(b->dT, b->dActive, b->dNActive, b->slotCtas, b->nSlots, k, b->dBar, b->n,
                                       b->rng, b->stream);
        if (e != cudaSuccess) return bfail(b, PV1_E_CUDA, std::string("v1 batch persistent: ") + cudaGetErrorString(e));
        n += 1;
    } else {
        for (int s = 0; s < k; s++) {
            e = launch_v1_batch_step(b->dT, b->dTiles, b->dNTiles, b->totalTiles, s, b->rng, minB, b->stream);
            if (e != cudaSuccess) return bfail(b, PV1_E_CUDA, std::string("v1 batch: ") + cudaGetErrorString(e));
        }
        n += k;
    }
    e = launch_batch_advance(b->dT, b->n, k, b->dSimTime, b->stream);
    if (e != cudaSuccess) return bfail(b, PV1_E_CUDA, cudaGetErrorString(e));
    n += 1;
    if (launches) *launches += n;
    return PV1_OK;
}

int graph_for(pv1_batch *b, int K, int minB, cudaGraphExec_t *out) {
    const int key = K * 4 + minB;
    auto it = b->graphs.find(key);
    if (it != b->graphs.end()) {
        *out = it->second;
        return PV1_OK;
    }
    cudaGraph_t g;
    PV1_BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int r = issue(b, K, minB, nullptr);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (r) return r;
    if (e2 != cudaSuccess) return bfail(b, PV1_E_CUDA, std::string("capture: ") + cudaGetErrorString(e2));
    cudaGraphExec_t ex;
    cudaError_t e3 = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return bfail(b, PV1_E_CUDA, std::string("instantiate: ") + cudaGetErrorString(e3));
    b->graphs[key] = ex;
    *out = ex;
    return PV1_OK;
}

int check_errors(pv1_batch *b) {
    for (int q = 0; q < b->n; q++) {
        int h = 0;
        PV1_BCUDA(b, cudaMemcpy(&h, b->hT[q].v.err, sizeof(int), cudaMemcpyDeviceToHost));
        if (h) return bfail(b, PV1_E_DEVICE, "device error word 0x" + std::to_string(h) + " in trial " +
                                                 std::to_string(q));
    }
    return PV1_OK;
}

}  // namespace

extern "C" {

int pv1_batch_create(pv1_plan *const *plans, uint32_t nTrials, const uint64_t *trialSteps, pv1_batch **out) {
    if (!plans || !trialSteps || !out || nTrials == 0) return PV1_E_ARG;
    *out = nullptr;
    pv1_batch *b = new pv1_batch();
    *out = b;
    b->n = (int)nTrials;
    for (float &t : b->times) t = -1.f;
    if (cudaGetDevice(&b->device) != cudaSuccess) return bfail(b, PV1_E_CUDA, "cudaGetDevice");
    PV1_BCUDA(b, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    PV1_BCUDA(b, cudaEventCreate(&b->ev0));
    PV1_BCUDA(b, cudaEventCreate(&b->ev1));
    b->plans.assign(plans, plans + nTrials);
    b->views.resize(nTrials);
    b->hT.resize(nTrials);
    b->hL.resize(nTrials);
    b->step.resize(nTrials);
    b->end.resize(nTrials);
    b->countOff.resize(nTrials + 1, 0);
    for (int q = 0; q < b->n; q++) {
        if (!plans[q]) return bfail(b, PV1_E_ARG, "null plan");
        for (int r = 0; r < q; r++)
            if (plans[r] == plans[q]) return bfail(b, PV1_E_ARG, "a plan appears twice in the batch");
        int r = plan_batch_view(plans[q], &b->views[q]);
        if (r) return bfail(b, r, "trial " + std::to_string(q) + ": " + pv1_last_error(plans[q]));
        if (b->views[q].device != b->device) return bfail(b, PV1_E_ARG, "plans on different devices");
        PV1_BCUDA(b, cudaStreamSynchronize(b->views[q].stream));
        b->countOff[q + 1] = b->countOff[q] + b->views[q].vp.nV1;
    }
    int r = 0;
    r |= balloc(b, &b->dT, nTrials);
    r |= balloc(b, &b->dL, nTrials);
    r |= balloc(b, &b->dCounts, (size_t)b->countOff[nTrials]);
    r |= balloc(b, &b->dCountOff, nTrials + 1);
    r |= balloc(b, &b->dSimTime, nTrials);
    r |= balloc(b, &b->dMean, 1);
    if (r) return r;
    b->totalTiles = 0;
    for (int q = 0; q < b->n; q++) {
        const PlanBatchView &v = b->views[q];
        BatchTrial &T = b->hT[q];
        T.v = v.vp;
        T.v.spikeCount = b->dCounts + b->countOff[q];
        T.lgnRing = v.lgnRing;
        T.lgnSlots = v.lgnSlots;
        T.nCta = v.vp.nblock * ((v.vp.blockSize + 255) / 256);
        T.step = v.d_stepBase;
        T.tEnd = v.step + (long long)trialSteps[q];
        T.tDeliverFrom = v.pending ? v.step : v.step + 1;
        T.dt = (double)v.vp.dt;
        BatchLgn &L = b->hL[q];
        L.p = v.lp;
        L.step = v.d_stepBase;
        L.tEnd = T.tEnd;
        b->step[q] = v.step;
        b->end[q] = T.tEnd;
        b->totalTiles += T.nCta;
        b->maxCellCtas = std::max(b->maxCellCtas, (v.lp.nMagno + 127) / 128);
        if (!v.lp.classCtw) b->allClass = false;
        if (v.vp.condRng || v.vp.noiseRng) b->rng = true;
        if (v.lgnSlots < 64) b->allClass = false;
        PV1_BCUDA(b, cudaMemcpyAsync(v.d_stepBase, &b->step[q], sizeof(long long), cudaMemcpyHostToDevice,
                                     b->stream));
    }
    PV1_BCUDA(b, cudaMemcpyAsync(b->dT, b->hT.data(), nTrials * sizeof(BatchTrial), cudaMemcpyHostToDevice,
                                 b->stream));
    PV1_BCUDA(b, cudaMemcpyAsync(b->dL, b->hL.data(), nTrials * sizeof(BatchLgn), cudaMemcpyHostToDevice,
                                 b->stream));
    PV1_BCUDA(b, cudaMemcpyAsync(b->dCountOff, b->countOff.data(), (nTrials + 1) * sizeof(long long),
                                 cudaMemcpyHostToDevice, b->stream));
    r = balloc(b, &b->dTiles, (size_t)b->totalTiles);
    r |= balloc(b, &b->dNTiles, 1);
    r |= balloc(b, &b->dActive, nTrials);
    r |= balloc(b, &b->dNActive, 1);
    r |= balloc(b, &b->dBar, nTrials);
    if (r) return r;
    // persistent variant: slots as large as the largest trial, as many as stay co-resident
    for (int q = 0; q < b->n; q++) b->slotCtas = std::max(b->slotCtas, b->hT[q].nCta);
    const int cap = v1_batch_persistent_capacity(b->rng, b->device);
    b->nSlots = b->slotCtas > 0 ? std::min(cap / b->slotCtas, b->n) : 0;
    if (b->nSlots > 0) b->minB = 0;
    PV1_BCUDA(b, cudaStreamSynchronize(b->stream));
    return refresh_tiles(b);
}

void pv1_batch_destroy(pv1_batch *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
    for (void *p : b->allocs) cudaFree(p);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

const char *pv1_batch_last_error(const pv1_batch *b) { return b ? b->err.c_str() : "null batch"; }

int pv1_batch_autotune(pv1_batch *b, int enable) {
    if (!b) return PV1_E_ARG;
    b->tune = enable != 0;
    b->nextCandidate = 0;
    if (!b->tune) {
        b->K = 64;
        b->minB = b->nSlots > 0 ? 0 : 1;
    }
    return PV1_OK;
}

int pv1_batch_tuning(const pv1_batch *b, int *K, int *minB, float *times) {
    if (!b) return PV1_E_ARG;
    if (K) *K = b->K;
    if (minB) *minB = b->minB;
    if (times) std::memcpy(times, b->times, sizeof(b->times));
    return PV1_OK;
}

int64_t pv1_batch_run(pv1_batch *b, uint64_t maxSteps, float *ms) {
    if (!b) return PV1_E_ARG;
    b->launches = 0;
    uint64_t done = 0;
    PV1_BCUDA(b, cudaEventRecord(b->ev0, b->stream));
    while (true) {
        long long left = 0, minLeft = -1;
        for (int q = 0; q < b->n; q++) {
            const long long l = b->end[q] - b->step[q];
            if (l <= 0) continue;
            left = std::max(left, l);
            minLeft = minLeft < 0 ? l : std::min(minLeft, l);
        }
        if (left == 0 || (maxSteps && done >= maxSteps)) break;
        int r = refresh_tiles(b);
        if (r) return r;
        // tuning visits the candidates forward then backward (2 * kCandidates chunks) and
        // averages the two per-step times of each, so that the drift of the activity over the
        // first chunks (onset transient) does not favour the candidates tried first
        auto cand_of = [](int idx) { return idx < kCandidates ? idx : 2 * kCandidates - 1 - idx; };
        while (b->tune && b->nextCandidate < 2 * kCandidates && cand_of(b->nextCandidate) % 4 == 0 && b->nSlots == 0)
            b->nextCandidate++;   // no persistent variant on this device / for these trial sizes
        const bool tuning = b->tune && b->nextCandidate < 2 * kCandidates;
        const int cand = tuning ? cand_of(b->nextCandidate) : 0;
        const int K = tuning ? kCandK[cand / 4] : b->K;
        const int minB = tuning ? cand % 4 : b->minB;
        long long k = std::min<long long>(K, minLeft);
        if (maxSteps) k = std::min<long long>(k, (long long)(maxSteps - done));
        if (b->allClass && k == K) {
            cudaGraphExec_t g;
            r = graph_for(b, K, minB, &g);
            if (r) return r;
            if (tuning) {
                cudaEvent_t t0, t1;
                PV1_BCUDA(b, cudaEventCreate(&t0));
                PV1_BCUDA(b, cudaEventCreate(&t1));
                PV1_BCUDA(b, cudaEventRecord(t0, b->stream));
                PV1_BCUDA(b, cudaGraphLaunch(g, b->stream));
                PV1_BCUDA(b, cudaEventRecord(t1, b->stream));
                PV1_BCUDA(b, cudaEventSynchronize(t1));
                float t = 0.f;
                PV1_BCUDA(b, cudaEventElapsedTime(&t, t0, t1));
                cudaEventDestroy(t0);
                cudaEventDestroy(t1);
                b->times[cand] = b->nextCandidate < kCandidates ? t : 0.5f * (b->times[cand] + t);
                b->nextCandidate++;
                while (b->nextCandidate < 2 * kCandidates && cand_of(b->nextCandidate) % 4 == 0 && b->nSlots == 0)
                    b->nextCandidate++;
                if (b->nextCandidate >= 2 * kCandidates) {
                    // fastest per step; a longer chunk is kept unless a shorter one is more than
                    // 10% faster (one tuning chunk underestimates the per-chunk costs -- LGN
                    // launch, host loop, partial chunks at trial ends -- that longer chunks
                    // amortise over the whole sweep)
                    int best = -1;
                    for (int c = kCandidates - 1; c >= 0; c--) {
                        if (b->times[c] <= 0) continue;
                        const float per = b->times[c] / kCandK[c / 4];
                        const float bestPer = best < 0 ? 0.f : b->times[best] / kCandK[best / 4];
                        const bool shorter = best >= 0 && kCandK[c / 4] < kCandK[best / 4];
                        if (best < 0 || (shorter ? per < 0.9f * bestPer : per < bestPer)) best = c;
                    }
                    if (best >= 0) {
                        b->K = kCandK[best / 4];
                        b->minB = best % 4;
                    }
                }
            } else {
                PV1_BCUDA(b, cudaGraphLaunch(g, b->stream));
            }
            b->launches += (minB == 0 ? 1 : K) + 2;
        } else {
            r = issue(b, (int)k, minB, &b->launches);
            if (r) return r;
        }
        for (int q = 0; q < b->n; q++)
            if (b->step[q] < b->end[q]) b->step[q] = std::min(b->end[q], b->step[q] + k);
        done += (uint64_t)k;
    }
    PV1_BCUDA(b, cudaEventRecord(b->ev1, b->stream));
    PV1_BCUDA(b, cudaEventSynchronize(b->ev1));
    if (ms) PV1_BCUDA(b, cudaEventElapsedTime(ms, b->ev0, b->ev1));
    int r = check_errors(b);
    if (r) return r;
    for (int q = 0; q < b->n; q++) plan_batch_finish(b->plans[q], b->step[q]);
    long long left = 0;
    for (int q = 0; q < b->n; q++) left = std::max(left, b->end[q] - b->step[q]);
    return left;
}

int pv1_batch_sweep(pv1_batch *b, float *ms) {
    if (!b) return PV1_E_ARG;
    if (!b->allClass || b->nSlots <= 0)
        return bfail(b, PV1_E_UNSUPPORTED,
                     "the one-launch sweep needs single-class LGN cells and every trial co-resident in a slot");
    std::vector<long long> left(b->n);
    long long maxLeft = 0;
    for (int q = 0; q < b->n; q++) {
        left[q] = std::max(0LL, b->end[q] - b->step[q]);
        maxLeft = std::max(maxLeft, left[q]);
    }
    b->launches = 0;
    if (maxLeft == 0) {
        if (ms) *ms = 0.f;
        return 0;
    }
    if (maxLeft > (1LL << 30)) return bfail(b, PV1_E_ARG, "too many steps for one launch");
    // per-trial LGN buffers of one row per remaining step (row = step mod rows, distinct for the
    // trial's remaining steps), in copies of the trial blocks
    std::vector<BatchTrial> T = b->hT;
    std::vector<BatchLgn> L = b->hL;
    std::vector<void *> bufs;
    auto release = [&]() {
        for (void *ptr : bufs) cudaFree(ptr);
        bufs.clear();
    };
    auto fresh = [&](float **ptr, size_t n) {
        if (cudaMalloc((void **)ptr, n * sizeof(float)) != cudaSuccess) return false;
        bufs.push_back(*ptr);
        return true;
    };
    for (int q = 0; q < b->n; q++) {
        if (!left[q]) continue;
        const int rows = (int)left[q];
        const size_t cells = (size_t)L[q].p.nLGN;
        float *sp = nullptr, *fr = nullptr;
        if (!fresh(&sp, (size_t)rows * cells) || (L[q].p.outFr && !fresh(&fr, (size_t)rows * cells))) {
            release();
            return bfail(b, PV1_E_NOMEM, "cudaMalloc of the sweep's LGN buffers");
        }
        L[q].p.outSInfo = sp;
        if (L[q].p.outFr) L[q].p.outFr = fr;
        L[q].p.outSlots = rows;
        T[q].lgnRing = sp;
        T[q].lgnSlots = rows;
    }
    // slot schedule: longest trial first, each to the least loaded slot; the kernel's slot s
    // takes list entries s, s + nSlots, ... (-1: nothing)
    std::vector<int> order(b->n);
    for (int q = 0; q < b->n; q++) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return left[x] > left[y]; });
    std::vector<std::vector<int>> per(b->nSlots);
    std::vector<long long> load(b->nSlots, 0);
    for (int q : order) {
        if (!left[q]) continue;
        const int sl = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        per[sl].push_back(q);
        load[sl] += left[q];
    }
    size_t depth = 0;
    for (auto &v : per) depth = std::max(depth, v.size());
    std::vector<int> list(depth * b->nSlots, -1);
    for (int sl = 0; sl < b->nSlots; sl++)
        for (size_t k = 0; k < per[sl].size(); k++) list[k * b->nSlots + sl] = per[sl][k];
    const int nList = (int)list.size();
    BatchTrial *dTs = nullptr;
    BatchLgn *dLs = nullptr;
    int *dList = nullptr, *dNList = nullptr;
    bool ok = cudaMalloc((void **)&dTs, b->n * sizeof(BatchTrial)) == cudaSuccess;
    if (ok) bufs.push_back(dTs);
    ok = ok && cudaMalloc((void **)&dLs, b->n * sizeof(BatchLgn)) == cudaSuccess;
    if (ok) bufs.push_back(dLs);
    ok = ok && cudaMalloc((void **)&dList, list.size() * sizeof(int)) == cudaSuccess;
    if (ok) bufs.push_back(dList);
    ok = ok && cudaMalloc((void **)&dNList, sizeof(int)) == cudaSuccess;
    if (ok) bufs.push_back(dNList);
    if (!ok) {
        release();
        return bfail(b, PV1_E_NOMEM, "cudaMalloc of the sweep's tables");
    }
    cudaError_t e = cudaMemcpyAsync(dTs, T.data(), b->n * sizeof(BatchTrial), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dLs, L.data(), b->n * sizeof(BatchLgn), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dList, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dNList, &nList, sizeof(int), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    // the sweep as one graph: LGN stage, one cooperative V1 launch, advance
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e1 = launch_lgn_class_batch(dLs, b->n, b->maxCellCtas, (int)maxLeft, b->stream);
        if (e1 == cudaSuccess)
            e1 = launch_v1_batch_persistent(dTs, dList, dNList, b->slotCtas, b->nSlots, (int)maxLeft, b->dBar, b->n,
                                            b->rng, b->stream);
        if (e1 == cudaSuccess) e1 = launch_batch_advance(dTs, b->n, (int)maxLeft, b->dSimTime, b->stream);
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        e = e1 != cudaSuccess ? e1 : e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev0, b->stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(ex, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev1, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b->ev1);
    if (ex) cudaGraphExecDestroy(ex);
    if (e == cudaSuccess && ms) e = cudaEventElapsedTime(ms, b->ev0, b->ev1);
    release();
    if (e != cudaSuccess) return bfail(b, PV1_E_CUDA, std::string("sweep: ") + cudaGetErrorString(e));
    b->launches = 3;
    int r = check_errors(b);
    if (r) return r;
    for (int q = 0; q < b->n; q++) {
        b->step[q] = b->end[q];
        plan_batch_finish(b->plans[q], b->step[q]);
    }
    return 0;
}

int pv1_batch_stats(pv1_batch *b, uint32_t trial, double *simTimeMs, double *rates, double *meanRate) {
    if (!b || trial >= (uint32_t)b->n) return PV1_E_ARG;
    const int nV1 = b->hT[trial].v.nV1;
    double *dRates = nullptr;
    if (rates) PV1_BCUDA(b, cudaMalloc((void **)&dRates, nV1 * sizeof(double)));
    cudaError_t e = launch_batch_rates(b->dT, b->dCounts, b->countOff.data(), b->dSimTime, (int)trial, nV1, dRates,
                                       b->dMean, b->stream);
    if (e == cudaSuccess && rates)
        e = cudaMemcpyAsync(rates, dRates, nV1 * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess && meanRate)
        e = cudaMemcpyAsync(meanRate, b->dMean, sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess && simTimeMs)
        e = cudaMemcpyAsync(simTimeMs, b->dSimTime + trial, sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (dRates) cudaFree(dRates);
    if (e != cudaSuccess) return bfail(b, PV1_E_CUDA, cudaGetErrorString(e));
    return PV1_OK;
}

int64_t pv1_batch_launch_count(const pv1_batch *b) { return b ? b->launches : -1; }

}  // extern "C"
