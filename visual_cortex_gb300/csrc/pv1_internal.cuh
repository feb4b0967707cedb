// Internal definitions shared by the patchV1 GB300 kernels and the host runtime.
//
// Device state is structure-of-arrays in HBM: every per-neuron quantity is a contiguous
// [nV1] float array (conductance species as [ng][nV1]), so a warp touches 128 contiguous
// bytes per quantity.  All arithmetic is fp32 as in the reference (Float = float,
// src/types.h:6) and uses the same CUDA math calls (expf, logf, lgammaf, sqrtf).
#pragma once

#include <cuda_runtime.h>
#include <curand_kernel.h>
#include <stdint.h>
#include "patchv1_gb300.h"   // include/ (on the include path)

namespace pv1 {

constexpr int kMaxType = PV1_MAX_NTYPE;
constexpr int kMaxNG = PV1_MAX_NG;
constexpr int kMaxSeg = 255;   // frames one temporal window may span (segments per step)
// single-temporal-class LGN kernel limits: steps per chunk, segments per step, frames per chunk
constexpr int kClassMaxK = 64;
constexpr int kClassMaxSeg = 48;
constexpr int kClassMaxSlots = 64;

// Error word bits raised by kernels (never trap).
constexpr int kMaxLgnMulti = 64;       // LGN synapses per neuron in the multi-spike step
constexpr int kMaxSpikePasses = 64;    // integration passes per step in the multi-spike step
constexpr int kErrRecordOverflow = 1;   // a draw record ran out of capacity
constexpr int kErrNegTsp = 2;           // interpolated spike time < 0 or NaN
constexpr int kErrFarOverflow = 4;      // far event beyond the delay ring
constexpr int kErrBounds = 8;           // an index failed its bounds check
constexpr int kErrBarrier = 16;         // a grid barrier gave up waiting
// Polls of a grid or trial barrier before it gives up (about 1 s); pv1_set_wait_limit
// changes it per plan.
constexpr long long kDefaultWaitSpins = 20000000;

// Two-state (g, h) conductance kernel with rise and decay times: the kinetics of the
// reference's ConductanceShape (src/condShape.h:13-41).  dod = tr/(td - tr).
struct Cond {
    float rise[kMaxNG], decay[kMaxNG], dod[kMaxNG];
};

__host__ inline Cond make_cond(const float *rt, const float *dc, int n) {
    Cond c{};
    for (int i = 0; i < n; i++) {
        c.rise[i] = rt[i];
        c.decay[i] = dc[i];
        c.dod[i] = rt[i] / (dc[i] - rt[i]);
    }
    return c;
}

// Unit input of strength f arriving `dt` before the end of the interval
// (compute_single_input_conductance, src/condShape.h:27-32).
__device__ __forceinline__ void cond_input(const Cond &c, float &g, float &h, float f, float dt,
                                           int ig) {
    float etr = expf(-dt / c.rise[ig]);
    g += f * c.dod[ig] * (expf(-dt / c.decay[ig]) - etr);
    h += f * etr;
}

// The same input with the kernel's constants passed as values (lets a caller choose between
// two kernels without taking the address of a kernel parameter).
__device__ __forceinline__ void cond_input_v(float rise, float decay, float dod, float &g, float &h, float f,
                                             float dt) {
    float etr = expf(-dt / rise);
    g += f * dod * (expf(-dt / decay) - etr);
    h += f * etr;
}

// Exact exponential decay of (g, h) over dt (decay_conductance, src/condShape.h:34-40).
__device__ __forceinline__ void cond_decay(const Cond &c, float &g, float &h, float dt, int ig) {
    float etr = expf(-dt / c.rise[ig]);
    float etd = expf(-dt / c.decay[ig]);
    g = g * etd + h * c.dod[ig] * (etd - etr);
    h *= etr;
}

// Decay factors over one full step, exp(-dt/decay) and exp(-dt/rise) per species: constant
// for a run, computed once on the device with the same expression cond_decay evaluates, so
// using them gives the same values as evaluating the exponentials every step.
struct StepDecay {
    float etd[kMaxNG], etr[kMaxNG];
};

__device__ __forceinline__ void cond_decay_step(const Cond &c, const StepDecay &e, float &g, float &h, int ig) {
    g = g * e.etd[ig] + h * c.dod[ig] * (e.etd[ig] - e.etr[ig]);
    h *= e.etr[ig];
}

// Frame bookkeeping of the magno temporal window, shared by host and device.
struct FrameSched {
    int denorm, ntPerFrame, maxFrame, magnoComp, frameOffset;
    int nFrame;        // frames in the movie (loops)
    int initRow;       // row of S holding the initial-luminance frame
};

// Segments of the temporal kernel per frame phase: for phase p (0 <= p < ntPerFrame),
// segment s covers samples [j0, j1) that all read the frame `rel` layers after the tail.
struct SegTable {
    int nPhase, maxSeg;
    const int *nseg;     // [nPhase]
    const int *rel;      // [nPhase][maxSeg]
    const int *j0;       // [nPhase][maxSeg+1] (j0[s+1] = end of segment s)
};

// Number of stimulus frames read once step `it` has started.
__host__ __device__ __forceinline__ int frames_read_after_step(const FrameSched &fs, long long it) {
    // frames are read while (it+1)*denorm > currentFrame*ntPerFrame (src/patch.cu:5969)
    long long num = (it + 1) * (long long)fs.denorm;
    return (int)((num + fs.ntPerFrame - 1) / fs.ntPerFrame);
}

struct LgnParams {
    int nMagno, nLGN;
    int nParvo_I, nMagno_I, nParvo_C;
    int nKS;                 // temporal samples
    float dt, convolRatio, frRatio;
    FrameSched fs;
    SegTable seg;
    int iKernelSampleT0, interval;
    const double *ctw;       // [nKS+1][nMagno] cumulative temporal weights
    const double *classCtw;  // [nKS+1] when every magno cell has the same temporal weights, else null
    const float *S;          // [nFrame+1][nMagno] spatial stage per frame
    const float *absk;       // [nMagno] |k| of the center
    const float *maxConvol;  // [nLGN]
    const float *c50, *sharp, *la, *lb;  // logistic per LGN id [nLGN]
    float *leftTimeRate, *lastNegLogRand;  // [nLGN]
    curandStateMRG32k3a *state;            // [nLGN]
    float *rate;             // [K][nLGN] rates of the chunk being computed
    float *outSInfo;         // [outSlots][nLGN] spike words, row = step % outSlots
    float *outFr;            // [outSlots][nLGN] rates (may be null)
    int outSlots;
    float *recU; int *recUCount; int recCap; long long recStep0; int recSteps;
    int *err;
    // parvocellular cells (nParvo = 0: none); parvo cell c is LGN id c or c + nMagno_I
    int nParvo;
    int pKS, pT0, pInterval;   // their kernel sampling
    int parvoComp, pFrameOffset;
    SegTable pseg;
    const double *pctw;        // [2][pKS+1][nParvo] cumulative temporal weights (centre, surround)
    const float *pS;           // [nFrame+1][2][nParvo] spatial stage per frame
    const float *pk;           // [2][nParvo] amplitude k of centre and surround
    // LGN->V1 plasticity: presynaptic LTP traces per cell (FF->E type first; 0 types: none)
    int nFF;
    float tauLTP[2];
    float *ffPre;              // [nFF][nLGN] traces at the end of the last computed step
    float *outPre;             // [outSlots][nFF][2][nLGN] traces at the start of the step, right after its spikes
};

// One LGN->V1 learning type (learnFF_pre/learnFF_post, src/condShape.h:85-152, derived).
struct FFType {
    float tauLTP, tauLTD, tauTrip, tauAvg, targetFR, A_LTP, A_ratio, gmax, gmin;
};

struct V1Params {
    int nV1, blockSize, nblock, nE, nI, nType, nTypeE;
    int typeAcc[kMaxType];
    int ngFF, ngE, ngI;
    float dt;
    Cond condFF, condE, condI;
    StepDecay decFF, decE, decI;   // full-step decay factors (filled by launch_step_decay)
    float vE, vI, vL;
    float vR[kMaxType], vThres[kMaxType], gL[kMaxType], C[kMaxType], tRef[kMaxType];
    float vT[kMaxType], deltaT[kMaxType], tau_w[kMaxType], a[kMaxType], b[kMaxType];
    float pFF[kMaxType * kMaxNG], pE[kMaxType * kMaxNG], pI[kMaxType * kMaxNG];
    float synFail[kMaxType * kMaxType], synPerCon[kMaxType * kMaxType];
    float synFailFF[kMaxType], synPerConFF[kMaxType], noisyDep[kMaxType];
    float tau_noise;
    int noiseOnTonic, iModel;
    int multiSpike;     // dt > min tRef: several spikes per step (compute_V_collect_spike_learnFF)
    int condRng;        // rGenCond draws can change results (some failure rate > 0)
    int noiseRng;       // some noisyDep > 0
    long long waitSpins;   // polls of a barrier wait before it gives up and raises kErrBarrier
    int pushCta;           // far-push CTAs appended to the persistent grid (0: the neuron CTAs push)
    // LGN->V1 plasticity (the reference's learning 1-4): triplet rule on the LGN->E synapses
    // (type 0) and, with learning 2, on the LGN->I synapses (type 1)
    int ffMode;            // the reference's `learning` (0: off)
    int ffLearn;           // the V1 step runs the learning block (learning 1-3)
    int ffTypes;           // traces the LGN stage keeps (FF->E, then FF->I)
    int ffI;               // FF->I learning on
    FFType ffT[2];         // FF->E, FF->I
    int applyHomeo, symmetricHomeo, rebound;
    float expHomeo;
    float tauAvgCortical;  // vAvgE through the delivery (learning 1, 2, 4)
    float *ffPost;         // learnVar's FF block: vLTD_FF_E, vTrip_FF_E, vLTD_FF_I, vTrip_FF_I, vAvgE[2], vAvgI
    int ffOffI, ffOffAvgE, ffOffAvgI;   // offsets of vLTD_FF_I, vAvgE and vAvgI in it
    float *totalFF;        // [2][nV1] total LGN weight and its target
    float *sLGNw;          // the weights, written by the learning (same array as sLGN)
    const float *ffPreRing;  // the LGN stage's outPre ring (row = step % lgn slots)
    // state [nV1] / [ng][nV1]
    float *v, *w, *tBack, *dep, *gFF, *hFF, *gE, *hE, *gI, *hI, *tonicDep, *lastNoise;
    curandStateMRG32k3a *rGenCond, *rNoisy;
    float *sInfo;       // [2][nV1], slot = step & 1
    // LGN -> V1
    int maxLGN;
    int lgnN;                  // row length of the LGN spike ring (nLGN)
    const int *nLGNperV1;      // [nV1]
    const int *lgnId;          // [maxLGN][nV1]
    const float *sLGN;         // [maxLGN][nV1]
    // near delivery
    int nnbMax;
    const int *nNearNB;        // [nblock]
    const int *nbId;           // [nblock][nnbMax]
    const float *conMat;       // [nblock][nnbMax][bs][bs]
    const int *nearRevOff;     // [nblock+1] near tiles that read block b's rows: nearRev[off[b]..off[b+1])
    const int *nearRev;        //            tile index (post block * nnbMax + position in its list)
    // far delivery (outgoing lists by pre-neuron)
    int farOn;                 // 0: no far input at all (noFarDelay=1 or no far synapses)
    const int *farOff;         // [nV1+1]
    const int *farPost;        // [nnz]
    const float *farStr;       // [nnz]
    const int *farSteps;       // [nnz] it2post
    const float *farFrac;      // [nnz] it2post*dt - delay/speed
    const int4 *farRec;        // [nnz] the four above in one record: post, str, steps, frac
    const unsigned char *farPre;  // [nV1] 1 if the neuron is a far presynaptic partner
    unsigned long long *farAcc;   // [farDepth][ngE+ngI][2][nV1] fixed-point g,h
    int farDepth;
    int *farFlag;              // [3] any far-pre spike (sInfo > 1) in step t%3
    const int *farN1;          // [nV1] leading synapses of each list with whole-step delay <= 1
    int4 *farList;             // [3][nV1] step t%3's far spikers: (pre, first synapse, count, sInfo bits)
    unsigned long long *farCount;  // [3] each list's spikers (high 32 bits) and synapses (low 32 bits)
    unsigned *spikeCount;      // [nV1] spikes per neuron since the counters were cleared (may be null)
    int noDelay;               // 1: near delivery from this step's spikes (conMat); 0: delayed events
    int nearOn;                // near-class (delayed) events exist: nearAcc is used
    int farClass;              // far-class events exist: farAcc is used
    unsigned long long *nearAcc;  // [farDepth][ngE+ngI][2][nV1] fixed-point g,h of near-class events
    // far synapses pulled by post in the reference's vec order (far synaptic failure: recal_G_vec's
    // per-post host engines and one normal_distribution per chunk of blocks)
    int farPullOn;
    const int *pullOff;        // [nV1+1]
    const int *pullPre;        // [nnz]
    const float *pullStr;      // [nnz]
    const int *pullSteps;      // [nnz] it2post
    const float *pullFrac;     // [nnz] it2post*dt - delay/speed
    const float *pullP;        // [nnz] failure rate of the (pre type, post type) pair
    const float *pullStd;      // [nnz] sqrt(p(1-p)/synPerCon)
    const unsigned char *pullIsPre;  // [nV1] 1 if the neuron is a far presynaptic partner
    float *sRing; int sDepth;  // [sDepth][nV1] spike words of the last sDepth steps (row = step mod sDepth)
    // distance-delayed near synapses with synaptic failure (noDelay = 0, some synFail > 0),
    // pulled by post in recal_G_mat's order: near blocks, then pre neurons by index
    int nearPullOn;
    const int *npOff;          // [nV1+1]
    const int *npPre;          // [nnz]
    const int *npSteps;        // [nnz] it2post
    const float *npStr;        // [nnz]
    const float *npFrac;       // [nnz] it2post*dt - delay/speed
    const float *npP;          // [nnz] failure rate of the (pre type, post type) pair
    const float *npStd;        // [nnz] sqrt(p(1-p)/synPerCon)
    unsigned *eng;             // [nV1] minstd_rand0 states
    int *pullCount, *pullStart, *pullPrev;  // [nV1] draws this step, first draw's index in the chunk, previous drawer
    float *pullCarry;          // [nV1] the unused second value of a post's last pair
    float *farPull;            // [ngE+ngI][2][nV1] far sums of the last step (consumed by the next delivery)
    int *pullFlag;             // [3] some far presynaptic spike (sInfo > 1) in step t%3
    const int *chunkStart;     // [nChunk+1] first neuron of each chunk
    int nChunk;
    // records
    float *rec; long long recStride; int recSlots; int hWrite;
    float *recSpk;             // [recSlots][nV1] spike words (PV1_REC_SPIKES)
    float *recNoise; float *recFF; int *recFFCount; float *recNear; int *recNearCount;
    int recCap; long long recStep0; int recSteps;
    int *err;
};

// Arguments of the LGN setup kernel (one CTA per magno cell).
struct SetupArgs {
    int nMagno, nLGN, nParvo_I, nMagno_I, nParvo_C;
    int nSample, nSample1D, nKS;
    float kernelSampleDt, kernelSampleT0;
    float normViewDistance, L_x0, L_y0, R_x0, R_y0, nsig;
    int flat;
    const float *polar, *ecc, *rw, *rh, *orient, *k;
    const float *ratio, *tauR, *tauD, *nR, *nD, *delay;
    float *TW, *SW, *SC, *maxConvol, *absk;
    double *ctw;
    int *err;
};

// Parvo store_PM + parvo_maxConvol arguments.
struct ParvoSetupArgs {
    int nParvo, nLGN, nParvo_I, nMagno_I;
    int flat;                  // 1: flat retina, 0: curved (sphere projected to the plane)
    int nSample, nSample1D, nKS;
    float kernelSampleDt, kernelSampleT0;
    float normViewDistance, L_x0, L_y0, R_x0, R_y0, nsig;
    const float *polar, *ecc, *rw, *rh, *orient, *k;
    const float *ratio, *tauR, *tauD, *nR, *nD, *delay;
    const float *covariant;
    int maxSample1D;           // parvo_maxConvol sample grid (src/patch.cu:5299-5312)
    float *TW;                 // [nParvo][2][nKS]
    float *SW;                 // [nSample]
    float *SC;                 // [2][nParvo][2][nSample]
    float *maxConvol;          // [nLGN]
    float *pk;                 // [2][nParvo]
    double *pctw;              // [2][nKS+1][nParvo]
    int *err;
};

// Launchers (defined next to their kernels).
cudaError_t launch_lgn_setup(const SetupArgs &a, int blockThreads, cudaStream_t st);
cudaError_t launch_parvo_setup(const ParvoSetupArgs &a, cudaStream_t st);
cudaError_t launch_parvo_spatial(cudaTextureObject_t L, cudaTextureObject_t M, cudaTextureObject_t S,
                                 const float *SW, const float *SC, const int *coneType, int nParvo,
                                 int nSample, int layer0, int nLayer, int row0, float *out, cudaStream_t st);
// Kernel launches one launch_lgn_step of K steps issues.
int lgn_step_launches(const LgnParams &p, int K);
cudaError_t launch_lgn_rng_init(curandStateMRG32k3a *state, float *lnl, float *ltr,
                                unsigned long long seed, int n, cudaStream_t st);
cudaError_t launch_lgn_spatial(cudaTextureObject_t L, cudaTextureObject_t M, cudaTextureObject_t S,
                               const float *SW, const float *SC, const int *coneType, int nMagno,
                               int nSample, int layer0, int nLayer, int row0, float *out,
                               cudaStream_t st);
cudaError_t launch_lgn_step(const LgnParams &p, const long long *stepBase, int K, cudaStream_t st);
cudaError_t launch_lgn_rate_only(const LgnParams &p, const long long *stepBase, int K, cudaStream_t st);

// What the allocation-free LGN entry point needs from a plan (defined in pv1_plan.cu).
struct PlanLgnView {
    LgnParams lp;
    cudaStream_t stream;
    long long step;
    int device;
    bool v1Stepped;   // pv1_run or a batch has stepped the plan (or left a delivery pending)
};
int plan_lgn_view(pv1_plan *p, PlanLgnView *out);
void plan_advance_steps(pv1_plan *p, long long n);
void plan_mark_lgn_only(pv1_plan *p);
int plan_fail(pv1_plan *p, int code, const char *msg);
cudaError_t launch_v1_step(const V1Params &p, const long long *stepBase, int stepOffset,
                           const float *lgnSInfo, int lgnSlots, int deliverPrev, int doStep,
                           cudaStream_t st);
cudaError_t launch_v1_rng_init(curandStateMRG32k3a *cond, curandStateMRG32k3a *noisy,
                               unsigned long long seed, int nV1, int trainDepth, cudaStream_t st);
// Initial spikes: per-step spike chance of each type, [type][0] for neurons with more than
// SCsplit LGN synapses and [type][1] for the rest.
struct Sp0 { float c[2 * kMaxType]; };
// rand_spInit with initial spikes (ogTab/ohTab may be null: no output_g/h table).
cudaError_t launch_v1_sp_init(const V1Params &p, unsigned long long seed, int depth, const Sp0 &sp0, int SCsplit,
                              float *H, float *ogTab, float *ohTab, float *recU, unsigned *recNU, cudaStream_t st);
// The near delivery before the first step (noDelay = 1).
cudaError_t launch_v1_sp_near(const V1Params &p, const float *Hlast, const float *ogTab, const float *ohTab,
                              float *recZ, unsigned *recNZ, int cap, cudaStream_t st);
// The delayed events of the history and the delivery of those arriving before the first step.
cudaError_t launch_v1_sp_events(const V1Params &p, const float *H, int depth, cudaStream_t st);
// Far delivery with synaptic failure for step *stepBase + off (stepBase may be null: step off),
// after that step's V1 kernel: four launches (count, chunk scan, carries, sums).
cudaError_t launch_far_pull(const V1Params &p, const long long *stepBase, long long off, cudaStream_t st);
constexpr int kFarPullLaunches = 4;
// Framed output over steps [step0, step0 + n): pixels below nSpikePixel from the V1 spike
// record ring, the others from the LGN firing-rate ring.
cudaError_t launch_frames(const float *recSpk, int recSlots, int nV1, const float *lgnFr, int lgnSlots, int nLGN,
                          long long step0, int n, int ot, long long tStart, const unsigned *pixOff,
                          const unsigned *pixIds, int nPixel, int nSpikePixel, float odt, float *acc, float *out,
                          cudaStream_t st);
// Adds farPull to the E/I conductances (the far part of the delivery before the first step).
cudaError_t launch_far_pull_apply(const V1Params &p, cudaStream_t st);
// Neuron CTAs of the persistent kernel; *fits: all can be resident at once; *pushCtas: the
// far-push CTAs that fit beside them on the device (0 without far synapses).
int v1_persistent_ctas(const V1Params &p, int device, bool *fits, int *pushCtas);
// Evaluates the full-step decay factors of the three conductance kernels on the device and
// stores them into p (synchronous).
cudaError_t compute_step_decay(V1Params &p, cudaStream_t st);
cudaError_t launch_v1_persistent(const V1Params &p, const long long *stepBase, int K, const float *lgnRing,
                                 int lgnSlots, int deliverFirst, unsigned *barrier, cudaStream_t st);
cudaError_t launch_advance_step(long long *stepBase, int k, cudaStream_t st);

// ---- batched trials: many independent patches stepped by the same launches ----
// One trial of a batch as the V1 kernel sees it (copied to shared memory by each CTA).
struct BatchTrial {
    V1Params v;
    const float *lgnRing;
    int lgnSlots;
    int nCta;                  // CTAs of this patch (nblock * ceil(blockSize / 256))
    long long *step;           // the trial's device step counter (its plan's)
    long long tEnd;            // first step the trial does not run
    long long tDeliverFrom;    // steps t >= this deliver the spikes of step t-1 first
    double dt;
};
// One trial as the LGN kernel sees it.
struct BatchLgn {
    LgnParams p;
    long long *step;
    long long tEnd;
};
// What the batch needs from a plan (defined in pv1_plan.cu).
struct PlanBatchView {
    V1Params vp;
    LgnParams lp;
    const float *lgnRing;
    int lgnSlots;
    long long *d_stepBase;
    long long step;
    bool pending;
    int device;
    cudaStream_t stream;
};
int plan_batch_view(pv1_plan *p, PlanBatchView *out);
void plan_batch_finish(pv1_plan *p, long long step);
// minB selects the __launch_bounds__ variant (1, 2 or 3 resident CTAs per SM).
cudaError_t launch_v1_batch_step(const BatchTrial *trials, const int2 *tiles, const int *nTiles,
                                 int gridTiles, int stepOffset, bool rng, int minB, cudaStream_t st);
cudaError_t launch_lgn_class_batch(const BatchLgn *trials, int nTrials, int maxCellCtas, int K,
                                   cudaStream_t st);
cudaError_t launch_batch_advance(BatchTrial *trials, int nTrials, int K, double *simTime,
                                 cudaStream_t st);
cudaError_t launch_batch_rates(const BatchTrial *trials, const unsigned *counts, const long long *countOff,
                               const double *simTime, int trial, int nV1, double *rates,
                               double *meanRate, cudaStream_t st);
int v1_batch_regs(int minB, bool rng);
// Batched trials in one cooperative launch per chunk (slots of slotCtas CTAs, per-trial barriers).
int v1_batch_persistent_capacity(bool rng, int device);
cudaError_t launch_v1_batch_persistent(const BatchTrial *trials, const int *activeList, const int *nActive,
                                       int slotCtas, int nSlots, int K, unsigned *barriers, int nTrials, bool rng,
                                       cudaStream_t st);

// Fixed-point scale for far-delivery accumulation: integer adds are associative, so the
// sum of events does not depend on their order and runs are reproducible.
constexpr double kFarScale = 4294967296.0;  // 2^32

// Float <-> fixed-point conversions of the far ring.  Scaling by 2^32 is exact in float (no
// overflow or underflow in range), so these give the same integers and floats as the
// corresponding double-precision expressions, without FP64 work (GB300's FP64 rate is low).
__device__ __forceinline__ long long far_to_fixed(float x) { return __float2ll_rn(x * 4294967296.0f); }
__device__ __forceinline__ float far_from_fixed(unsigned long long u) {
    return __ll2float_rn((long long)u) * 2.3283064365386963e-10f;  // 2^-32
}

}  // namespace pv1
