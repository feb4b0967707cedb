/*
 * patchv1_gb300.h -- C ABI of the GB300 (sm_103a) simulation hot path of patchV1.
 *
 * The reference (`patch`, src/patch.cu) has no library interface: its hot path is a set of
 * CUDA kernels and one host function driven from main().  Each entry point below replaces
 * one of those pieces; the comment on each cites the reference code it stands in for
 * (paths relative to the reference project root).
 *
 * Conventions
 *   - Every function returns 0 on success and a negative PV1_E* code on failure; the text of
 *     the last failure of a plan is returned by pv1_last_error().  Nothing here calls exit()
 *     or traps the GPU (the reference exits on any CUDA error, src/CUDA_MACRO.h:23-31).
 *   - All arrays are host arrays owned by the caller and copied; the plan owns every device
 *     buffer and its CUDA stream.  Calls on one plan are not thread safe; plans are
 *     independent of each other.
 *   - Float is 32-bit IEEE (the reference's Float, src/types.h:6), Size is uint32_t.
 *   - Neuron ids are block-major (id = block*blockSize + local), excitatory types first within
 *     a block (typeAcc), exactly as in the reference's files.
 */
#ifndef PATCHV1_GB300_H
#define PATCHV1_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PV1_OK              0
#define PV1_E_ARG          -1   /* bad argument / inconsistent sizes            */
#define PV1_E_CUDA         -2   /* a CUDA runtime call failed                    */
#define PV1_E_STATE        -3   /* call out of order (e.g. run before setup)     */
#define PV1_E_UNSUPPORTED  -4   /* option of the reference not built here        */
#define PV1_E_DEVICE       -5   /* a kernel raised its error word                */
#define PV1_E_NOMEM        -6   /* device allocation failed                      */

#define PV1_MAX_NTYPE 2         /* reference MAX_NTYPE, src/CONST.h:12            */
#define PV1_MAX_NG    2         /* reference MAX_NGTYPE_*, src/CONST.h:24-28      */

typedef struct pv1_plan pv1_plan;

/* V1 model description: the option table entries of src/patch.cu:181-288 that the step,
 * the delivery and the conductance kinetics read, after the per-type expansion done in
 * src/patch.cu:890-1000 (size-1 vectors broadcast to nType; vT := vThres for iModel 0). */
typedef struct pv1_v1_config {
    uint32_t nblock, blockSize;             /* V1_allpos header, src/patch.cu:697-703     */
    uint32_t nType, nTypeE;                 /* connectome_cfg, src/patch.cu:636-645       */
    uint32_t typeAcc[PV1_MAX_NTYPE];        /* typeAccCount (cumulative, last == blockSize)*/
    uint32_t ngFF, ngE, ngI;                /* sizes of riseTime{FF,E,I}                  */
    float dt;                               /* ms                                         */
    float riseFF[PV1_MAX_NG], decayFF[PV1_MAX_NG];
    float riseE[PV1_MAX_NG],  decayE[PV1_MAX_NG];
    float riseI[PV1_MAX_NG],  decayI[PV1_MAX_NG];
    float vE, vI, vL;                       /* reversal potentials; the reference fixes them
                                               at compile time to 0, -75, -65 (src/CONST.h:7-9) */
    float vR[PV1_MAX_NTYPE], vThres[PV1_MAX_NTYPE], gL[PV1_MAX_NTYPE], C[PV1_MAX_NTYPE];
    float tRef[PV1_MAX_NTYPE], vT[PV1_MAX_NTYPE], deltaT[PV1_MAX_NTYPE];
    float tau_w[PV1_MAX_NTYPE], a[PV1_MAX_NTYPE], b[PV1_MAX_NTYPE];
    float pFF[PV1_MAX_NTYPE * PV1_MAX_NG];  /* [nType][ngFF]                               */
    float pE[PV1_MAX_NTYPE * PV1_MAX_NG];   /* [nType][ngE]                                */
    float pI[PV1_MAX_NTYPE * PV1_MAX_NG];   /* [nType][ngI]                                */
    float synFail[PV1_MAX_NTYPE * PV1_MAX_NTYPE];    /* [pre type][post type]              */
    float synPerCon[PV1_MAX_NTYPE * PV1_MAX_NTYPE];
    float synFailFF[PV1_MAX_NTYPE], synPerConFF[PV1_MAX_NTYPE];
    float noisyDep[PV1_MAX_NTYPE];
    float tau_noise;
    int32_t noiseOnTonic;
    int32_t iModel;                         /* 0: LIF (w held at 0), 1: AdEx              */
    int32_t noDelay;                        /* 1: near delivery without distance delay;
                                               0: delayed (pv1_v1_set_near_delayed)       */
    int32_t noFarDelay;                     /* 0: delayed far delivery; 1: reference drops
                                               far input (src/coredynamics.cu:218-220)    */
    float speedOfThought;                   /* mm/ms                                      */
    int32_t hWrite;                         /* rawData carries h as well as g             */
} pv1_v1_config;

/* Magnocellular (ON/OFF DoG) LGN description: the stimulus/kernel-sampling bookkeeping of
 * src/patch.cu:4950-5030 and 5395-5412 and the geometry of src/patch.cu:1604-1630. */
typedef struct pv1_lgn_config {
    uint32_t nLGN;              /* all LGN cells (parvo + magno); V1 synapses index these */
    uint32_t nParvo_I, nMagno_I, nParvo_C, nMagno_C;  /* cell order in the LGN files      */
    uint32_t mSample1D;         /* mSpatialSample1D (<= 32)                                */
    uint32_t nKernelSample;     /* mKernelSample                                           */
    uint32_t kernelSampleInterval, iKernelSampleT0;   /* in steps                          */
    uint32_t denorm, ntPerFrame, maxFrame;            /* frame phase bookkeeping           */
    uint32_t magnoComp, frameOffset;  /* frameOffset = pLongerThanM*dFrame                  */
    float dt;
    float kernelSampleDt, kernelSampleT0;             /* ms                                */
    float convolRatio, frRatio;
    float normViewDistance, L_x0, L_y0, R_x0, R_y0;
    float nsig;
    int32_t flat_retina;
} pv1_lgn_config;

/* Per-cell LGN parameters as stored in the `LGN` file (src/patch.cu:2505-2534): arrays of
 * 2*nLGN hold [center][nLGN] then [surround][nLGN]. */
typedef struct pv1_lgn_params {
    const float *polar, *ecc, *rw, *rh, *orient, *k;        /* 2*nLGN each */
    const float *ratio, *tauR, *tauD, *nR, *nD, *delay;     /* 2*nLGN each */
    const float *spont, *c50, *sharpness;                   /* nLGN each   */
    const uint32_t *coneType;                               /* 2*nLGN      */
} pv1_lgn_params;

/* ---- plan lifetime ------------------------------------------------------------------ */

/* Page-locked host memory for the buffers a caller streams through the library (stimulus
 * frames in, records out): copies from and to it run at the full host-link bandwidth and
 * asynchronously.  Free with pv1_host_free. */
int pv1_host_alloc(uint64_t bytes, void **out);
void pv1_host_free(void *ptr);

/* Makes `device` the current CUDA device of the calling thread for this library (the
 * reference picks the device with the most free memory, src/patch.cu:9-24; here the caller
 * chooses).  Plans are created on the current device. */
int pv1_set_device(int device);

/* Creates a plan on the current CUDA device.  Replaces the allocation part of main()
 * (src/patch.cu:3898-4070). */
int pv1_plan_create(const pv1_v1_config *cfg, pv1_plan **out);
void pv1_plan_destroy(pv1_plan *plan);
const char *pv1_last_error(const pv1_plan *plan);
/* ABI version of this header (bumped on any signature change). */
int pv1_abi_version(void);

/* ---- LGN -------------------------------------------------------------------------- */

/* Builds the temporal weights (time reversed, L1 normalised), the DoG spatial weights, the
 * texture coordinates and max_convol of every magno cell on the device, and seeds the LGN
 * Poisson generators.  Replaces store_PM(PM=1) (src/discrete_input_convol.cu:427-744, with
 * store_temporalWeight :230-305), hStatic_nonlinear (src/LGN_props.h:143-170) and
 * logRand_init (src/coredynamics.cu:148-177) called with `seed` (src/patch.cu:2685). */
int pv1_lgn_setup(pv1_plan *plan, const pv1_lgn_config *lcfg, const pv1_lgn_params *p,
                  uint64_t seed);

/* Copies the setup tables back: TW [nMagno][nKernelSample], SW [nMagno][mSample],
 * SC [2][nMagno][mSample], maxConvol [nLGN].  Any pointer may be NULL. */
int pv1_lgn_get_tables(pv1_plan *plan, float *TW, float *SW, float *SC, float *maxConvol);

/* Loads the stimulus movie (stimulus.bin body: nFrame frames of L,M,S planes [h][w]) and the
 * initial luminance (init_L,M,S of the stimulus header), and runs the per-frame spatial stage
 * of LGN_convol_magno (src/discrete_input_convol.cu:1474-1532) once per distinct frame.
 * Frames loop at the end of the movie as in src/patch.cu:5987-5993. */
int pv1_stimulus_load(pv1_plan *plan, uint32_t nFrame, uint32_t height, uint32_t width,
                      const float init_LMS[3], const float *frames);

/* Reads the spatial-stage table S [nFrame+1][nMagno] (row nFrame: the initial luminance). */
int pv1_lgn_get_spatial(pv1_plan *plan, float *S);

/* Parvocellular cells: centre and surround are separate Gaussians of their own cone types
 * (L/M opponent or L+M), each with its own temporal kernel, sampled on their own kernel
 * grid (nKernelSample over tau) and their own frame-phase tail (parvoComp). */
typedef struct pv1_lgn_parvo_config {
    uint32_t nSample1D;          /* nSpatialSample1D (<= 32)                                  */
    uint32_t nKernelSample;      /* nKernelSample                                             */
    uint32_t kernelSampleInterval, iKernelSampleT0;   /* in steps                             */
    uint32_t parvoComp, frameOffset;  /* frameOffset = (1-pLongerThanM)*dFrame               */
    float kernelSampleDt, kernelSampleT0;             /* ms                                   */
} pv1_lgn_parvo_config;

/* pv1_lgn_setup for an LGN with parvocellular cells (nParvo_I + nParvo_C > 0): the magno part
 * as pv1_lgn_setup, plus store_PM(PM=0) (src/discrete_input_convol.cu:427-520 with
 * store_temporalWeight :230-305 and store_spatialWeight :309-425, flat retina) and
 * parvo_maxConvol (:748-883) with the sample-grid size rule of src/patch.cu:5266-5312.
 * covariant [nLGN] as stored in the `LGN` file.  pv1_lgn_setup is this call with pcfg = NULL
 * and rejects parvo cells. */
int pv1_lgn_setup_parvo(pv1_plan *plan, const pv1_lgn_config *lcfg, const pv1_lgn_parvo_config *pcfg,
                        const pv1_lgn_params *p, const float *covariant, uint64_t seed);

/* Parvo setup tables: TW [nParvo][2][nKernelSample] (centre, surround; time reversed, L1
 * normalised), SW [nSample] (the normalised Gaussian every parvo cell shares), SC
 * [2][nParvo][2][nSample] (x then y texture coordinates per cell and component).  Parvo cell
 * c is LGN id c (c < nParvo_I) or c + nMagno_I.  Any pointer may be NULL. */
int pv1_lgn_get_parvo_tables(pv1_plan *plan, float *TW, float *SW, float *SC);

/* Parvo spatial stage PS [nFrame+1][2][nParvo]: per frame the centre and surround contrast
 * sums of LGN_convol_parvo (src/discrete_input_convol.cu:1032-1062, 1151-1218). */
int pv1_lgn_get_parvo_spatial(pv1_plan *plan, float *PS);

/* ---- V1 --------------------------------------------------------------------------- */

/* LGN->V1 feed-forward synapses, transposed [maxLGN][nV1] as the reference keeps them in
 * device memory (read_LGN, src/patch.h:30-77; getLGN_V1_surface, src/stats.cu:99-112).
 * sLGN already carries sRatioLGN. */
int pv1_v1_set_lgn_synapses(pv1_plan *plan, uint32_t maxLGN, const uint32_t *nLGNperV1,
                            const uint32_t *lgnId, const float *sLGN);

/* Near-neighbour connectivity: conMat [nblock][nearNeighborBlock][blockSize pre][blockSize
 * post], neighborBlockId [nblock][nearNeighborBlock], nNearNeighborBlock [nblock]
 * (src/patch.cu:3442-3497).  Strengths already carry sRatioV1. */
int pv1_v1_set_near(pv1_plan *plan, uint32_t nearNeighborBlock, const uint32_t *nNearNB,
                    const uint32_t *neighborBlockId, const float *conMat);

/* Far connectivity as read from V1_vec (src/patch.cu:3313-3352): for post neuron i, nVec[i]
 * entries of (vecID, conVec, delayVec) stored back to back.  Strengths already carry
 * sRatioV1.  Builds the outgoing (by pre-neuron) event lists used on the device; replaces
 * the host loop recal_G_vec (src/coredynamics.cu:181-372) with fill_fSpikeTrain
 * (src/stats.cu:114-126) and sum_G (src/coredynamics.cu:2312-2349).  With synaptic failure
 * (some synFail > 0) the far synapses are instead kept by post in vec order and delivered by
 * the failure path, which then needs pv1_v1_far_failure_engines. */
int pv1_v1_set_far(pv1_plan *plan, const uint32_t *nVec, const uint32_t *vecID,
                   const float *conVec, const float *delayVec);

/* Host engines of the far synaptic failure (plans with noFarDelay = 0, far synapses and some
 * synFail > 0): engine i is default_random_engine seeded with seed + i (src/patch.cu:4224-4228,
 * seed = the logRand_init seed + 1), and the far delivery runs per chunk of blocks (nChunk of
 * the cfg, split as src/patch.cu:3430-3437), each chunk sharing one normal_distribution as
 * recal_G_vec does (src/coredynamics.cu:181-372).  Call after pv1_v1_set_far; a no-op for
 * plans without far failure. */
int pv1_v1_far_failure_engines(pv1_plan *plan, uint64_t seed, uint32_t nChunk);

/* Near-neighbour connectivity with distance delays, for plans with noDelay = 0: conMat as for
 * pv1_v1_set_near and delayMat of the same layout (distances in mm, src/patch.cu:3450-3460,
 * 3685).  Replaces recal_G_mat (src/coredynamics.cu:2063-2309): every non-zero entry becomes a
 * delayed event of the same device event lists as the far synapses.  Synaptic failure is not
 * supported with delays (PV1_E_UNSUPPORTED). */
int pv1_v1_set_near_delayed(pv1_plan *plan, uint32_t nearNeighborBlock, const uint32_t *nNearNB,
                            const uint32_t *neighborBlockId, const float *conMat, const float *delayMat);

/* Initial state (host-generated as in src/patch.cu:4405-4560).  Layouts: [nV1] or
 * [ng][nV1]; w may be NULL for iModel 0. */
int pv1_v1_set_state(pv1_plan *plan, const float *v, const float *w, const float *gFF,
                     const float *hFF, const float *gE, const float *hE, const float *gI,
                     const float *hI, const float *tonicDep);

/* Seeds the per-neuron device generators and advances them as rand_spInit does
 * (src/coredynamics.cu:5-146) for a network without initial spikes (spE0 = spI0 = 0). */
int pv1_v1_init_rng(pv1_plan *plan, uint64_t seed, uint32_t trainDepth);

/* What pv1_v1_init_spikes drew and built, for checking it against a restatement.  Host
 * arrays; any pointer may be NULL. */
typedef struct pv1_init_record {
    float *uniforms;     /* [nV1][2*trainDepth] the uniforms each neuron drew, in order */
    uint32_t *nUniform;  /* [nV1] how many */
    float *normals;      /* [nV1][normalCap] failure draws of the near delivery before the first step */
    uint32_t *nNormal;   /* [nV1] how many (more than normalCap: PV1_E_DEVICE) */
    uint32_t normalCap;
    float *history;      /* [trainDepth][nV1] spike-word ring after rand_spInit (slot 0: initial spikes) */
} pv1_init_record;

/* rand_spInit with initial spikes (src/coredynamics.cu:5-146, launched at src/patch.cu:4580)
 * and the delivery that the reference runs once before its step loop when some spE0/spI0 > 0
 * (src/patch.cu:5687-5888): replaces pv1_v1_init_rng.  sp0 [nType][2] holds the per-step
 * spike chances (spE0 then spI0 of the cfg, each times dt/1000: [t][0] for neurons with more
 * than SCsplit LGN synapses, [t][1] for the rest).  Changes v, w, tBack and the E/I
 * conductances set by pv1_v1_set_state, so call it after that and after every connectivity
 * call (pv1_v1_set_near / _near_delayed / _far), before the first step.  Quirks of the
 * reference that are kept: the initial spike words themselves are never delivered (the first
 * step overwrites their ring slot); the delivery before the loop takes the history slot
 * trainDepth-1 as the previous step's spikes and, with noDelay = 1, reads the initial
 * spikers' compacted output_g/h table at per-neuron offsets (recal_G_mat_nd,
 * src/coredynamics.cu:2497-2510, after rand_spInit wrote it at :85-116); with noDelay = 0 it
 * reads the ring with slot 0 as the newest (src/patch.cu:5760-5770) while the loop takes slot
 * trainDepth-1 as the step before the first.  The reference numbers the initial spikers of a
 * block in the order of its atomicAdd_block returns; this library numbers them by thread index.
 * rec may be NULL. */
int pv1_v1_init_spikes(pv1_plan *plan, uint64_t seed, uint32_t trainDepth, const float *sp0,
                       uint32_t SCsplit, pv1_init_record *rec);

/* Host initial-state generator of src/patch.cu:4405-4560 (libstdc++ default_random_engine
 * and normal/uniform distributions, same call order).  v0/w0/g0 arrays as in the cfg:
 * v0 [nType][2], w0 [nType][2], gFF0 [nType][ngFF][4], gE0 [nType][ngE][4],
 * gI0 [nType][ngI][4].  Outputs [nV1] / [ng][nV1]. */
int pv1_host_init_state(const pv1_v1_config *cfg, uint64_t seed, const float *tonicDep,
                        const uint32_t *nLGNperV1, int use_v0, float tonicMax,
                        const float *w0, const float *gFF0, const float *gE0,
                        const float *gI0, float *v, float *w, float *gFF, float *hFF,
                        float *gE, float *hE, float *gI, float *hI);

/* ---- stepping --------------------------------------------------------------------- */

#define PV1_REC_RAW    1   /* rawData records (src/patch.cu:6138-6165, 6255-6261)        */
#define PV1_REC_LGN_SP 2   /* LGN_sp records (src/patch.cu:6423)                         */
#define PV1_REC_LGN_FR 4   /* LGN_fr records                                             */
#define PV1_REC_SPIKES 8   /* spike words only: the first field of each rawData record   */

/* Sets which per-step records the device keeps, in a ring of `slots` steps. */
int pv1_set_record(pv1_plan *plan, int flags, uint32_t slots);
/* Bytes of one rawData record (after the file header). */
int64_t pv1_raw_record_floats(const pv1_plan *plan);

/* Runs `nsteps` steps of the hot loop (src/patch.cu:5966-6880): LGN convolution, LGN spikes,
 * V1 step, near and far delivery.  Work is issued as CUDA graphs on the plan's stream.
 * Returns after the work is queued when `sync` is 0. */
int pv1_run(pv1_plan *plan, uint32_t nsteps, int sync);

/* Feeds the V1 steps [step0, step0 + nsteps) from LGN spike words the caller computed
 * (d_sInfo: device memory of the plan's device, [nsteps][nLGN] rows in the plan's LGN cell
 * order, spike words nsp + tsp/dt as LGN_nonlinear writes them, src/discrete_input_convol.cu:
 * 1766-1771) instead of the plan's own LGN stage; each run copies the rows of its steps into
 * the LGN ring, and a run outside the range fails.  The buffer must stay valid while it is
 * set; d_sInfo = NULL returns to the plan's own LGN stage.  Not with plasticity
 * (PV1_E_UNSUPPORTED).  For instance the BF16 tensor-core LGN stage below
 * (pv1_lgn_tc_device_spikes) can drive a simulation this way. */
int pv1_set_lgn_source(pv1_plan *plan, const float *d_sInfo, int64_t step0, int64_t nsteps);

/* Copies finished records [step0, step0+n) to host buffers (any may be NULL):
 * raw: n * pv1_raw_record_floats floats; lgn_sp, lgn_fr: n * nLGN floats. */
int pv1_fetch_records(pv1_plan *plan, uint64_t step0, uint32_t n, float *raw,
                      float *lgn_sp, float *lgn_fr);

#define PV1_ST_V      0
#define PV1_ST_W      1
#define PV1_ST_TBACK  2
#define PV1_ST_DEP    3
#define PV1_ST_GFF    4   /* [ngFF][nV1] */
#define PV1_ST_HFF    5
#define PV1_ST_GE     6   /* [ngE][nV1], after the last step's delivery */
#define PV1_ST_HE     7
#define PV1_ST_GI     8
#define PV1_ST_HI     9
#define PV1_ST_SINFO 10   /* last step's spike word per neuron */
#define PV1_ST_LGN_LTR 11 /* [nLGN] leftTimeRate  */
#define PV1_ST_LGN_LNL 12 /* [nLGN] lastNegLogRand */
#define PV1_ST_LGN_SINFO 13 /* [nLGN] last step's LGN spike word */
#define PV1_ST_FAR_PULL 14  /* [ngE+ngI][2][nV1] far g, h sums of the last step (far synaptic
                               failure plans; read only), added at the next step's delivery */
/* Random generators, read only, as raw bytes: 48 bytes (one curandStateMRG32k3a) per cell or
 * neuron, so `out` must hold 12 floats' worth per entry.  LGN: one per LGN cell, set up by
 * logRand_init's curand_init(seed, id, 0) (src/coredynamics.cu:148-177); V1: rGenCond and
 * rNoisy, curand_init(seed, id, 0) and curand_init(seed, nV1 + id, 0) (:5-146). */
#define PV1_ST_LGN_RNG 15   /* [nLGN][48 B] */
#define PV1_ST_V1_RNG_COND 16  /* [nV1][48 B] */
#define PV1_ST_V1_RNG_NOISY 17 /* [nV1][48 B] */
/* Copies one state array to the host (waits for queued work). */
int pv1_get_state(pv1_plan *plan, int which, float *out);
/* The excitatory neurons sampled by minimal output (src/patch.cu:4922-4937): all of them in
 * order when sampleSize exceeds their number, else std::sample over them (block-major) with a
 * default_random_engine seeded `seed` (the rand_spInit seed + 1).  out holds
 * min(sampleSize, nblock*nE) ids, the count in *nOut. */
int pv1_sample_ids(uint64_t seed, uint32_t nblock, uint32_t blockSize, uint32_t nE, uint32_t sampleSize,
                   uint32_t *out, uint32_t *nOut);

/* Framed output (framePhyV1output, frameVisV1output, frameVisLGNoutput): pixelizeOutput
 * (src/stats.cu:4-36) as the step loop runs it (src/patch.cu:6727-6790).  Pixel q holds the
 * cells pixIds[pixOff[q] .. pixOff[q+1]) (getUnderlyingID's order, src/stats.cuh:26-60): V1
 * neurons for q < nSpikePixel (each step adds the sum of their spike counts floor(sInfo),
 * sInfo >= 0), LGN cells after that (the sum of their firing rates); the sum is divided by
 * m odt and accumulated over frames of ot steps counted from the plan's step at setup.  V1
 * pixels need the PV1_REC_SPIKES record, LGN pixels PV1_REC_LGN_FR.  collect processes steps
 * [step0, step0+n) in order, continuing the previous call, and writes the frames completed
 * among them to frames [k][nPixel], k in *nFrames. */
int pv1_frames_setup(pv1_plan *plan, uint32_t nPixel, uint32_t nSpikePixel, const uint32_t *pixOff,
                     const uint32_t *pixIds, uint32_t ot, float odt);
int pv1_frames_collect(pv1_plan *plan, uint64_t step0, uint32_t n, float *frames, uint32_t *nFrames);

/* Checkpoints: the plan's whole evolving state (neuron state and generators, spike-word
 * rows, delayed-event rings, far-failure engines, LGN integrals and generators) with the step
 * count, so that a plan of the same configuration and network that loads it continues bit
 * for bit (the reference's snapshot, src/patch.cu:6793-6912, also holds the state needed to
 * resume; its far rings, kept on the host, are not in it).  The last step's delivery is
 * applied before saving.  size -> save into a host buffer of that size -> load. */
int pv1_checkpoint_size(pv1_plan *plan, uint64_t *bytes);
int pv1_checkpoint_save(pv1_plan *plan, void *buf, uint64_t bytes);
int pv1_checkpoint_load(pv1_plan *plan, const void *buf, uint64_t bytes);
/* The step count of a plan whose state was loaded array by array (pv1_put_state), as a
 * snapshot in the reference's layout is (src/patch.cu:5489-5685): sets it, drops the pending
 * delivery (the loaded conductances already hold it) and empties the delayed-event rings and
 * far spiker lists -- the reference's snapshot holds no far events in flight, its far rings
 * being host vectors it does not save.  noDelay = 0 plans: PV1_E_UNSUPPORTED. */
int pv1_set_step(pv1_plan *plan, int64_t step);

/* LGN->V1 plasticity, the reference's learning modes 1-4 (src/patch.cu:1160-1175): the
 * triplet rule on the LGN->excitatory synapses (learning 1, 2, 3) and on the LGN->inhibitory
 * ones (learning 2) inside the V1 step (compute_V_collect_spike_learnFF_fast,
 * src/coredynamics.cu:1631-1993: LTD at each LGN spike from the post LTD trace, LTP at each V1
 * spike from the presynaptic trace and the post triplet trace, weights clipped to
 * [gmin, gmax], the filtered post rate scaling LTD when targetFR > 0, optional homeostasis of
 * each neuron's total LGN weight), the presynaptic LTP traces in the LGN stage (LGN_nonlinear,
 * src/discrete_input_convol.cu:1774-1820), and, with learning 1, 2 and 4, the excitatory
 * filtered rate vAvgE taken through the near delivery with the cortical E types' tauAvg
 * (recal_G_mat_nd_fast, src/coredynamics.cu:2866-2890) instead of inside the V1 step.  The
 * reference keeps cortical E->E and I->E learning variables as well, but no kernel of it
 * changes a cortical weight with them and none of its outputs holds them; they are not kept.
 * The fields are the cfg values the reference reads (src/patch.cu:221-256): the FF->E type's
 * tauLTP..sRatioLGN (element [0] of the arrays; sRatioLGN[0]), the FF->I type's (element
 * [nLearnTypeFF_E]; tauAvg[1], targetFR[1], sRatioLGN[1]) and the cortical E types' tauAvg
 * (tauAvg[0] when nLearnTypeE > 0; 0 reproduces the zeroed struct the reference passes
 * otherwise).  Derived rates as learnFF_post computes them (src/condShape.h:137-152),
 * exp_homeo = expf(-dt / decayTimeHomeoFF) (src/patch.cu:1330); the homeostasis totals start
 * from the current weights (src/patch.cu:4335-4352).  Plans with learning run one launch per
 * step (no persistent kernel, no batches) and one spike per step at most;
 * PV1_E_UNSUPPORTED otherwise. */
typedef struct pv1_ff_learning {
    int32_t learning;            /* 1, 2, 3 or 4 */
    float tauLTP, tauLTD, tauTrip, tauAvg, targetFR;    /* FF->E type */
    float A_LGN, r_LTD, gmaxLGN, gminLGN, sRatioLGN;
    float decayTimeHomeoFF, FF_InfRatio;
    int32_t applyHomeo;          /* 0 none, 1 multiplicative, 2 additive */
    int32_t symmetricHomeo, rebound;
    int32_t nLearnTypeFF_E;      /* 0 or 1; 0 with learning 4 */
    int32_t nLearnTypeFF_I;      /* 0 or 1; 1 only with learning 2 */
    float tauLTP_I, tauLTD_I, tauTrip_I, tauAvg_I, targetFR_I;   /* FF->I type */
    float A_LGN_I, r_LTD_I, gmaxLGN_I, gminLGN_I, sRatioLGN_I;
    float tauAvgCortical;        /* vAvgE's time constant in the delivery (learning 1, 2, 4) */
} pv1_ff_learning;
int pv1_set_ff_learning(pv1_plan *plan, const pv1_ff_learning *cfg);
/* The derived constants pv1_set_ff_learning uses for the FF->E type, for a step dt (host only,
 * no device work): out[0] A_LTP = A_LGN * sRatioLGN, out[1] A_ratio (the LTD rate; with
 * targetFR > 0 scaled by tauTrip / (tauLTD tauAvg_s^2) / 1000 / targetFR), out[2] gmax and
 * out[3] gmin scaled by sRatioLGN, out[4] exp_homeo -- learnFF_post (src/condShape.h:137-152)
 * and src/patch.cu:1330.  The FF->I type's come from the same function given its values in
 * the FF->E fields. */
int pv1_ff_learning_rates(const pv1_ff_learning *cfg, float dt, float *out5);

/* Learning state (plans with learning): the LGN->V1 weights [maxLGN][nV1] (the reference's
 * LGN_V1_s, synapse-major), the post variables in the reference's learnVar FF layout
 * (src/patch.cu:4365-4385: vLTD_FF_E [nE types][nblock*nE], vTrip_FF_E, vLTD_FF_I
 * [nI types][nblock*nI], vTrip_FF_I, vAvgE [nblock*nE][2], vAvgI [nblock*nI]), the presynaptic
 * LTP traces of each LGN cell at the end of the last step [nLearnTypeFF_E + nLearnTypeFF_I][nLGN],
 * and the homeostasis totals [2][nV1] (total, target). */
#define PV1_ST_SLGN     18
#define PV1_ST_FF_POST  19
#define PV1_ST_FF_PRE   20
#define PV1_ST_TOTAL_FF 21

/* Overwrites one state array (PV1_ST_* above; the generators as the raw bytes get_state
 * gives, which is how a snapshot in the reference's layout, src/patch.cu:6793-6912, is loaded;
 * not the spike words or the far sums). */
int pv1_put_state(pv1_plan *plan, int which, const float *in);

/* Draw recording for parity tests: when enabled, every uniform/normal the kernels draw is
 * written to per-step buffers so that a CPU restatement can consume the same draws.
 * capacity = draws kept per entity per step (LGN Poisson, V1 noise, FF failure, near
 * failure).  0 disables. */
int pv1_set_draw_record(pv1_plan *plan, uint32_t steps, uint32_t capacity);
/* kind: 0 LGN uniforms [steps][nLGN][cap], 1 V1 noise normals [steps][nV1],
 * 2 FF-failure normals [steps][nV1][cap], 3 near-failure normals [steps][nV1][cap]
 * (indexed by the step whose spikes were delivered).  counts (may be NULL) receives
 * the number of draws per entity per step, same leading shape. */
int pv1_fetch_draws(pv1_plan *plan, int kind, float *draws, int32_t *counts);

/* Spike words of steps [step0, step0+n) into out [n][nV1] (PV1_REC_SPIKES ring). */
int pv1_fetch_spikes(pv1_plan *plan, uint64_t step0, uint32_t n, float *out);

/* pv1_run(plan, nsteps, 1) that also writes the spike words of those steps into out
 * [nsteps][nV1]: each chunk's rows are copied on a copy stream while the next chunks run (the
 * reference overlaps its device-to-host copies of V1 data with the LGN convolution,
 * src/patch.cu:6120-6160).  out should be page-locked (pv1_host_alloc) for the copies to
 * overlap; PV1_REC_SPIKES must be on with a ring of at least nsteps + 1 rows. */
int pv1_run_spikes_to_host(pv1_plan *plan, uint32_t nsteps, float *out);

/* Number of kernel launches issued by the last pv1_run (for launch accounting). */
int64_t pv1_last_launch_count(const pv1_plan *plan);

/* ---- measurement (no counterpart in the reference, which has no timers) ------------- */

/* Writes flush_bytes of a scratch buffer (to evict L2), then runs nsteps between two CUDA
 * events on the plan's stream; *ms receives the device time of the run alone. */
int pv1_run_timed(pv1_plan *plan, uint32_t nsteps, uint64_t flush_bytes, float *ms);

/* Runs nsteps (rounded down to whole chunks of `chunk` steps) with direct launches, CUDA
 * events on the plan's stream around the LGN rate+spike pair and around the V1 work of each
 * chunk; returns the mean V1 device time per simulation step and the mean LGN time per
 * chunk. */
int pv1_time_kernels(pv1_plan *plan, uint32_t nsteps, float *v1_ms, float *lgn_ms, int *chunk);

/* Allocation-free LGN stepping (no counterpart in the reference).  For callers that cannot
 * allocate device memory when they step the LGN stage (a host loop under a fixed device
 * memory budget, or a framework that owns every allocation): runs the LGN rate and spike
 * kernels for the plan's next nsteps steps and writes the spike words, and the rates if d_fr
 * is not NULL, to the caller's device buffers [nsteps][nLGN] (magno cells; other entries are
 * left untouched).  The only scratch, the rates passed between the two kernels, lives in a
 * fixed 4 MiB device array of the library: nsteps * nLGN must not exceed 1048576 and nsteps
 * must not exceed 65535, otherwise PV1_E_ARG.  It calls no cudaMalloc/cudaFree.  Work is queued on the plan's stream.  The
 * first call on a device looks up the array's device address (cudaGetSymbolAddress): make
 * that first call before any stream capture.  Calls share the array, so calls that overlap on
 * the GPU race.  It advances the plan's LGN generators and step counter: a plan stepped this
 * way is an LGN-only plan, and pv1_run, pv1_time_kernels, pv1_checkpoint_save and
 * pv1_batch_create then return PV1_E_STATE; a plan already stepped by pv1_run or a batch is
 * refused here with PV1_E_STATE. */
int pv1_lgn_spikes_noalloc(pv1_plan *plan, uint32_t nsteps, float *d_sinfo, float *d_fr);

/* Polls of a barrier wait (the persistent kernel's grid barrier between steps, the batched
 * kernel's per-trial barrier) before it gives up; spins < 0 restores the default (2e7 polls,
 * about a second).  A wait that gives up releases every other waiter, the kernel returns, and
 * the run reports PV1_E_DEVICE ("a barrier wait gave up") instead of hanging: the GPU context
 * stays usable.  No counterpart in the reference (its kernels never wait on one another). */
int pv1_set_wait_limit(pv1_plan *plan, int64_t spins);

/* allow = 1/0 enables/disables the persistent cooperative V1 kernel (one launch per chunk of
 * steps, state in registers, bounded grid barrier between steps); allow = -1 only queries.
 * Returns 1 if the plan steps with the persistent kernel, 0 if with one launch per step. */
int pv1_persistent_mode(pv1_plan *plan, int allow);

/* ---- Batched trials ------------------------------------------------------------------
 * Replaces the reference's one-process-per-trial sweep (src/ori.sh runs `patch -c cfg` once
 * per orientation/seed): many fully set-up plans (each a trial with its own stimulus, seeds,
 * state and connectivity) are stepped together, every step of every trial in the same
 * launches: one batched LGN launch and K batched V1 launches per chunk of K steps, captured
 * once as a CUDA graph.  Trials may differ in duration (trialSteps) and size (nblock).  Each
 * trial computes exactly what pv1_run would compute for it alone.  The plans must live on
 * the current device and stay alive until pv1_batch_destroy. */
typedef struct pv1_batch pv1_batch;

int pv1_batch_create(pv1_plan *const *plans, uint32_t nTrials, const uint64_t *trialSteps,
                     pv1_batch **out);
void pv1_batch_destroy(pv1_batch *batch);
const char *pv1_batch_last_error(const pv1_batch *batch);
/* Runs every trial until its end (trialSteps after create), or at most maxSteps more steps
 * (0 = no limit).  Returns the number of steps of the longest trial still to run (0: all
 * done), or a negative error code.  *ms (may be null) receives the device time of the call
 * (CUDA events on the batch stream). */
int64_t pv1_batch_run(pv1_batch *batch, uint64_t maxSteps, float *ms);
/* V1 variants: 0 = one cooperative launch per chunk that runs every trial's K steps with its
 * state in registers (slots of CTAs take the trials in turn; a barrier among a trial's own
 * CTAs between steps), available when the largest trial fits the co-resident grid;
 * 1, 2, 3 = one launch per step with 1, 2 or 3 resident CTAs per SM.
 * Autotuner: tries each chunk length in {16, 32, 64} with each variant for one chunk of the
 * real run, in forward then in backward order, and keeps the fastest average per step (a
 * shorter chunk only if more than 10% faster); the tuning chunks are ordinary steps of the
 * simulation.  enable = 0 fixes K = 64 and variant 0 (1 where 0 is not available). */
int pv1_batch_autotune(pv1_batch *batch, int enable);
/* Chosen chunk length, V1 variant (minB) and the measured ms per chunk of every candidate
 * tried (times[i] for candidate i = kIndex*4 + variant; 12 entries, -1 where not tried). */
int pv1_batch_tuning(const pv1_batch *batch, int *K, int *minB, float *times);
/* FP64 statistics of one trial: simulated time (ms), per-neuron firing rates (Hz, may be
 * null) and their mean, from spike counters kept by the V1 kernel since pv1_batch_create. */
int pv1_batch_stats(pv1_batch *batch, uint32_t trial, double *simTimeMs, double *rates,
                    double *meanRate);
/* Kernel launches issued by the last pv1_batch_run or pv1_batch_sweep. */
int64_t pv1_batch_launch_count(const pv1_batch *batch);
/* Runs the rest of every trial as one CUDA graph of three launches: the LGN stage of every
 * remaining step of every trial (into per-trial buffers of one row per step, allocated for
 * the call: remaining steps x nLGN floats per trial), ONE cooperative V1 launch in which each
 * slot of CTAs runs its trials one after the other, each for all its remaining steps (trials
 * assigned to slots longest first, each to the least loaded slot), and the advance.  Each
 * trial computes exactly what pv1_run computes for it alone.  Needs the persistent variant
 * (the largest trial co-resident) and single-class LGN cells; otherwise PV1_E_UNSUPPORTED.
 * Returns 0 (every trial done) or a negative error code; *ms (may be null) receives the
 * device time of the graph. */
int pv1_batch_sweep(pv1_batch *batch, float *ms);

/* ---- Surrogate-gradient adjoint ----------------------------------------------------------
 * No counterpart in the reference (it has no gradient code).  The differentiable form of the
 * V1 step: conductance-based LIF, RK2 membrane step, two-state AMPA (from the LGN) and GABA
 * (from the block's I neurons) kernels with the conductance-shape constants of
 * src/condShape.h:13-51 passed in as (Ed, Er, dod) = (e^{-dt/td}, e^{-dt/tr}, tr/(td-tr)),
 * spikes with a fast-sigmoid surrogate derivative, step-granular delivery, B independent
 * trials.  All pointers are device pointers owned by the caller (torch tensors); work goes on
 * `stream` (a cudaStream_t, 0 = legacy default).  Sizes: N = nblock*blockSize, nI = blockSize-nE,
 * nWin = T/win, nSeg = ceil(T/seg). */
typedef struct {
    uint32_t B, nblock, blockSize, nE, nLGN, K, T, seg, win;
    float dt, vL, vE, vI, vR, vThres, gL, slope;  /* slope of the surrogate, 1/mV */
    uint32_t tRefE, tRefI;                          /* refractory steps */
    float EdE, ErE, dodE, EdI, ErI, dodI;           /* AMPA and GABA kernel constants */
    uint32_t recGrad;   /* 1: the gradient flows through the recurrent I spikes too; 0: the
                         * recurrent spike input is held constant in the backward (stop-gradient),
                         * the usual cure for the exploding recurrent surrogate gradient */
    uint32_t ctaSplit;  /* CTAs per (trial, block), joined in a thread-block cluster: 1 or 2;
                         * 0 = 2 when blockSize is a multiple of 64 and B * nblock * 2 CTAs fit
                         * the SMs, else 1.  Results do not depend on it (up to the order of the
                         * FP64 atomic sums of dL/d(kernel constants)). */
} pv1_adj_problem;

typedef struct {
    const int32_t *ids;   /* [K][N] LGN id of synapse k of neuron n */
    const float *W;       /* [K][N] LGN->V1 weights */
    const uint8_t *X;     /* [B][T][nLGN] LGN spike counts per step */
    const float *Crec;    /* [nblock][nI][blockSize] I -> block GABA weights (pre row, post column) */
    const float *I0;      /* [N] constant drive */
    const float *v0;      /* [B][N] initial v (conductances start at 0) */
    float *rates;         /* out [B][nWin][N] spike rate per window (Hz) */
    float *vbar;          /* out [B][nWin][N] mean v per window (mV) */
    float *ck;            /* [nSeg][6][B][N] checkpoints, written by forward, read by backward */
    const float *gR;      /* [B][nWin][N] dL/drates (may be null) */
    const float *gV;      /* [B][nWin][N] dL/dvbar (may be null) */
    float *gW;            /* out [K][N] dL/dW, accumulated (zero it first) */
    double *gC;           /* out [6] dL/d(EdE, ErE, dodE, EdI, ErI, dodI), accumulated */
    float *scratch;       /* [B*nblock][seg][6][blockSize] recompute buffer */
} pv1_adj_buffers;

uint64_t pv1_adj_checkpoint_floats(const pv1_adj_problem *p);
uint64_t pv1_adj_scratch_floats(const pv1_adj_problem *p);
int pv1_adj_forward(const pv1_adj_problem *p, const pv1_adj_buffers *b, void *stream);
int pv1_adj_backward(const pv1_adj_problem *p, const pv1_adj_buffers *b, void *stream);
const char *pv1_adj_last_error(void);

/* ---- LGN stage at scale on BF16 tensor cores -------------------------------------------
 * Replaces LGN_convol_magno + LGN_nonlinear (src/discrete_input_convol.cu:1342-1730) for cells
 * that share one temporal kernel, over a whole movie at once: convol[cell][t] =
 * sum_f S[cell][f] W[t][f] as tcgen05 BF16 MMAs with FP32 accumulation in tensor memory (or the
 * same tiles on CUDA cores in FP32), followed per step by the logistic rate and the
 * exact-time Poisson generator.  The spatial stage is computed on the device from the movie:
 * S[cell][pad + f] = sum over a side x side pixel footprint of SW * clamp(L/meanLum - 1, -1, 1).
 * W comes as tiles: Wtiles[i][s][k] = weight of frame column f0[i] + k for step 128*i + s
 * (f0[i] a multiple of 8; columns count frames from -pad). */
typedef struct {
    uint32_t nCells, nFrame, height, width, side, nFext, pad, T, frEvery, recordRates;
    float dt, convolRatio, frRatio, meanLum;
} pv1_lgn_tc_config;
typedef struct pv1_lgn_tc pv1_lgn_tc;

int pv1_lgn_tc_create(const pv1_lgn_tc_config *cfg, const float *frames /* [nFrame][height][width] */,
                      const float *SW /* [nCells][side*side] */, const int32_t *cx, const int32_t *cy,
                      const float *Wtiles /* [ceil(T/128)][128][64] */, const int32_t *f0,
                      const float *absk, const float *maxConvol, const float *c50, const float *sharp,
                      const float *la, const float *lb, pv1_lgn_tc **out);
/* Runs all T steps from a fresh generator state (curand_init(seed, cell, 0), one uniform
 * discarded as logRand_init does); tensorCores = 1: BF16 tcgen05 kernel, 0: FP32 CUDA cores.
 * *ms: device time of the stepping kernel (CUDA events). */
int pv1_lgn_tc_run(pv1_lgn_tc *p, int tensorCores, uint64_t seed, float *ms);
/* S [nCells][nFext] (FP32 spatial stage), spike words [T][nCells], rates
 * [ceil(T/frEvery)][nCells]; any may be null. */
int pv1_lgn_tc_fetch(pv1_lgn_tc *p, float *S, float *sInfo, float *fr);
/* The device array of the spike words [T][nCells] the last run wrote (valid until destroy). */
const float *pv1_lgn_tc_device_spikes(const pv1_lgn_tc *p);
void pv1_lgn_tc_destroy(pv1_lgn_tc *p);
const char *pv1_lgn_tc_last_error(const pv1_lgn_tc *p);

#ifdef __cplusplus
}
#endif
#endif /* PATCHV1_GB300_H */
