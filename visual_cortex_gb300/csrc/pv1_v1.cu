// V1 stage of the patchV1 hot path on GB300 (sm_103a).
//
// The reference runs, per step, compute_V_collect_spike_learnFF_fast (src/coredynamics.cu:
// 1235-2059), then recal_G_mat_nd_fast for the near-neighbour blocks (:2609-2922), then a
// single-threaded host loop for the far synapses (recal_G_vec :181-372, fill_fSpikeTrain
// src/stats.cu:114-126) whose result is copied back and added by sum_G (:2312-2349).
//
// Here every simulation step has three phases, one thread per neuron:
//   A. deliver the previous step's spikes: every CTA compacts the spikers of its neighbour
//      blocks with warp ballots (ascending neuron order, E before I), stages their unit
//      conductance (og/oh) in shared memory and reads one coalesced conMat row per spiker;
//      far events that arrive in the previous step come from a fixed-point ring filled by
//      phase C.  The sum is added to g/h exactly where the reference's delivery adds it.
//   B. the V1 membrane step (conductance decay, LGN input, RK2 AdEx/LIF, spike-time
//      interpolation, refractoriness), with the float operations of the reference's kernel.
//   C. push this step's spikes into the far-delivery ring: one event per (spike, far
//      synapse), with the reference's delay arithmetic deciding the arrival step.
// Adding the previous step's delivery before this step's decay is the same sequence of
// float operations as the reference's separate kernels.
//
// Two kernels run these phases: v1_step_kernel does one step per launch (state in HBM), and
// v1_persistent_kernel runs K steps in one cooperative launch with the neuron state, the
// LGN synapse ids and the generators held in registers and a bounded grid barrier between
// steps.  Both are instantiated with and without the random-number paths (noise, synaptic
// failure); the host picks the variant.  Per-species arrays use compile-time indices so that
// they stay in registers.
#include <algorithm>
#include "pv1_internal.cuh"

namespace pv1 {

constexpr int kCta = 256;
constexpr int kWarps = kCta / 32;
constexpr int kMaxBS = 1024;
constexpr int kLgnBatch = 8;
constexpr int kMaxLgnReg = 32;        // LGN synapses kept in shared memory by the persistent kernel
constexpr int kBatchLgn = 24;         // the same in the batched persistent kernel (two blocks per SM)
constexpr int kConBatch = 8;          // conMat rows fetched together

__device__ __forceinline__ int type_of(const V1Params &P, int local) {
    int t = P.nType - 1;
#pragma unroll
    for (int j = kMaxType - 1; j >= 0; j--) {
        if (j < P.nType && local < P.typeAcc[j]) t = j;
    }
    return t;
}

// Record offsets inside one rawData record (src/patch.cu:6138-6165, src/stats.cu:39-97).
struct RecOff {
    long long sinfo, dep, w, v, gFF, hFF, gE, gI, hE, hI;
};
__device__ __forceinline__ RecOff rec_off(const V1Params &P) {
    RecOff o;
    long long n = P.nV1;
    o.sinfo = 0;
    o.dep = n;
    o.w = 2 * n;
    o.v = (2 + (P.iModel == 1)) * n;
    o.gFF = o.v + n;
    o.hFF = o.gFF + P.ngFF * n;
    o.gE = o.hFF + (P.hWrite ? P.ngFF * n : 0);
    o.gI = o.gE + P.ngE * n;
    o.hE = o.gI + P.ngI * n;
    o.hI = o.hE + P.ngE * n;
    return o;
}

// Per-neuron dynamic state (registers).
// LGN input of the next step fetched ahead by the persistent kernel: the synapses that
// received spikes (bit mask, synapse order) and the spike word and weight of the first one.
struct LgnPre {
    unsigned mask;
    float s0, f0;
};

// Starts the copies of one step's LGN spike words of a neuron's m synapses into shared memory
// (ids and destinations [synapse][kCta] from this thread's column); lgn_words_wait completes
// them.  Each thread reads back only what it copied, so no CTA barrier is needed.
__device__ __forceinline__ void lgn_words_async(const float *__restrict__ ring, const int *ids, float *dst, int m) {
    for (int q = 0; q < m; q++) {
        const unsigned d = (unsigned)__cvta_generic_to_shared(dst + q * kCta);
        const float *src = ring + ids[q * kCta];
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void lgn_words_wait() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Fetches the spike words of a neuron's (at most kMaxLgnReg) LGN synapses for one step: ids
// at ids[q * Stride] (registers: Stride 1; shared memory: Stride kCta).
template <int Stride>
__device__ __forceinline__ LgnPre lgn_prefetch(const V1Params &P, const float *__restrict__ ring, const int *ids,
                                               int m, int i) {
    LgnPre pre{0u, 0.f, 0.f};
    float sp[kMaxLgnReg];
#pragma unroll
    for (int q = 0; q < kMaxLgnReg; q++) sp[q] = q < m ? __ldcg(ring + ids[q * Stride]) : 0.f;
#pragma unroll
    for (int q = kMaxLgnReg - 1; q >= 0; q--) {
        const bool hit = sp[q] >= 1.0f;
        pre.mask |= (hit ? 1u : 0u) << q;
        if (hit) pre.s0 = sp[q];
    }
    if (pre.mask) pre.f0 = __ldg(P.sLGN + (size_t)(__ffs(pre.mask) - 1) * P.nV1 + i);
    return pre;
}

struct NState {
    float v, w, tBack, lastNoise;
    float gE[kMaxNG], hE[kMaxNG], gI[kMaxNG], hI[kMaxNG], gFF[kMaxNG], hFF[kMaxNG];
};

struct Smem {
    int pre[kMaxBS];
    float val[kMaxBS];
    float og[kMaxNG][kMaxBS];
    float oh[kMaxNG][kMaxBS];
    unsigned ball[kMaxBS / 32];
    int pref[kMaxBS / 32];
    int total, below;
    unsigned fball[kWarps];
    int fpre[kCta], fe0[kCta], fdeg[kCta], fpref[kCta + 1];
    float fsi[kCta];
};

__device__ __forceinline__ void load_state(const V1Params &P, int i, NState &s) {
    const int nV1 = P.nV1;
    s.v = P.v[i];
    s.w = P.iModel == 1 ? P.w[i] : 0.0f;
    s.tBack = P.tBack[i];
    s.lastNoise = P.tau_noise > 0 ? P.lastNoise[i] : 0.f;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        s.gE[ig] = ig < P.ngE ? P.gE[ig * nV1 + i] : 0.f;
        s.hE[ig] = ig < P.ngE ? P.hE[ig * nV1 + i] : 0.f;
        s.gI[ig] = ig < P.ngI ? P.gI[ig * nV1 + i] : 0.f;
        s.hI[ig] = ig < P.ngI ? P.hI[ig * nV1 + i] : 0.f;
        s.gFF[ig] = ig < P.ngFF ? P.gFF[ig * nV1 + i] : 0.f;
        s.hFF[ig] = ig < P.ngFF ? P.hFF[ig * nV1 + i] : 0.f;
    }
}

__device__ __forceinline__ void store_state(const V1Params &P, int i, const NState &s) {
    const int nV1 = P.nV1;
    P.v[i] = s.v;
    if (P.iModel == 1) P.w[i] = s.w;
    P.tBack[i] = s.tBack;
    if (P.tau_noise > 0) P.lastNoise[i] = s.lastNoise;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        if (ig < P.ngE) { P.gE[ig * nV1 + i] = s.gE[ig]; P.hE[ig * nV1 + i] = s.hE[ig]; }
        if (ig < P.ngI) { P.gI[ig * nV1 + i] = s.gI[ig]; P.hI[ig * nV1 + i] = s.hI[ig]; }
        if (ig < P.ngFF) { P.gFF[ig * nV1 + i] = s.gFF[ig]; P.hFF[ig * nV1 + i] = s.hFF[ig]; }
    }
}

// Compacts the spike words blk[0..bs) that are >= 1 into sm.pre[] (ascending index) and
// stages the unit conductance of each (output_g/h of compute_V, src/coredynamics.cu:
// 2008-2041) in sm.og/sm.oh.  Returns the count; *cntE receives the number of excitatory
// spikers (index < nE), which come first.  Three CTA barriers when there are spikers, two
// otherwise.
__device__ __forceinline__ int compact_spikers(const V1Params &P, const float *__restrict__ blk, Smem &sm,
                                               int *cntE) {
    const int bs = P.blockSize, nE = P.nE;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (bs + 31) >> 5;
    const float dt = P.dt;
    float vals[kMaxBS / kCta];
#pragma unroll
    for (int k = 0; k < kMaxBS / kCta; k++) {
        const int j = k * kCta + threadIdx.x;
        vals[k] = j < bs ? __ldcg(blk + j) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kMaxBS / kCta; k++) {
        const int j = k * kCta + threadIdx.x;
        const bool f = j < bs && vals[k] >= 1.0f;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (k * kCta < bs && lane == 0) sm.ball[k * kWarps + warp] = bal;
    }
    __syncthreads();
    // every warp scans the block's ballot words itself (no second barrier): lane l holds word l
    const unsigned wb = lane < nw ? sm.ball[lane] : 0u;
    const int c = __popc(wb);
    int below = 0;
    if ((lane + 1) * 32 <= nE) below = c;
    else if (lane * 32 < nE) below = __popc(wb & ((1u << (nE - lane * 32)) - 1u));
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) below += __shfl_xor_sync(0xffffffffu, below, o);
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    *cntE = below;
    if (total == 0) return 0;
    const int excl = incl - c;
#pragma unroll
    for (int k = 0; k < kMaxBS / kCta; k++) {
        const int j = k * kCta + threadIdx.x;
        // word k * kWarps + warp holds this warp's lanes for pass k (j >> 5)
        const int wbase = __shfl_sync(0xffffffffu, excl, (k * kWarps + warp) & 31);
        const unsigned wbits = __shfl_sync(0xffffffffu, wb, (k * kWarps + warp) & 31);
        if (j < bs && vals[k] >= 1.0f) {
            const int pos = wbase + __popc(wbits & ((1u << lane) - 1u));
            sm.pre[pos] = j;
            const float sI = vals[k];
            const float nsp = floorf(sI);
            const float tsp = (sI - nsp) * dt;
            const bool isE = j < nE;
#pragma unroll
            for (int ig = 0; ig < kMaxNG; ig++) {
                if (ig < (isE ? P.ngE : P.ngI)) {
                    float g = 0.f, h = 0.f;
                    cond_input_v(isE ? P.condE.rise[ig] : P.condI.rise[ig], isE ? P.condE.decay[ig] : P.condI.decay[ig],
                                 isE ? P.condE.dod[ig] : P.condI.dod[ig], g, h, nsp, dt - tsp);
                    sm.og[ig][pos] = g;
                    sm.oh[ig][pos] = h;
                }
            }
        }
    }
    __syncthreads();
    return total;
}

// Sends to L2 what the next step reads because neuron i (local index `local` of block b)
// spiked: its rows of the near tiles that list block b (read by the delivery, whole 16-byte
// aligned rows), and the whole 16-byte chunks of its far synapse list (read by the push).
// Hints only: nothing waits on them.
__device__ __forceinline__ void prefetch_spiker(const V1Params &P, int b, int local, int farE0, int farDeg) {
    if (P.noDelay && P.nearRevOff && (P.blockSize & 3) == 0) {
        const unsigned bytes = (unsigned)P.blockSize * 4u;
        for (int e = __ldg(P.nearRevOff + b); e < __ldg(P.nearRevOff + b + 1); e++) {
            const float *row = P.conMat + ((size_t)__ldg(P.nearRev + e) * P.blockSize + local) * P.blockSize;
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(row), "r"(bytes) : "memory");
        }
    }
    if (farDeg > 0) {
        const unsigned bytes = (unsigned)farDeg * 16u;
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(P.farRec + farE0), "r"(bytes) : "memory");
    }
}

// The excitatory filtered rate of learning 1, 2 and 4, advanced over step tp in the near
// delivery as recal_G_mat_nd_fast does (src/coredynamics.cu:2866-2890): from the value stored
// at the spike time when the neuron spiked (slot 1), else the step start (slot 0), plus the
// spike count, decayed over the rest of the step with the cortical E types' tauAvg.
__device__ __forceinline__ void learn_avg_delivery(const V1Params &P, float postSInfo, int b, int local) {
    const float dt = P.dt;
    const float postNsp = floorf(postSInfo);
    const float postTsp = postSInfo > 0 ? postSInfo - postNsp : 1.f;
    const int cPick = postNsp > 0 ? 1 : 0;
    float *vAvg = P.ffPost + P.ffOffAvgE + 2 * (b * P.nE + local);
    float lAvgE = vAvg[cPick];
    float delta_t = dt;
    if (postNsp > 0) delta_t = dt * (1 - postTsp);
    lAvgE += postNsp;
    lAvgE *= expf(-delta_t / P.tauAvgCortical);
    vAvg[0] = lAvgE;
}

__device__ __forceinline__ int far_ring_slot(const V1Params &P, long long t);

// Phase A: delivery of step tp's spikes to this thread's neuron (all threads of the CTA
// must call it; `active` masks the neuron work).
template <bool Rng>
__device__ __forceinline__ void deliver_prev(const V1Params &P, long long tp, int b, int local, int i,
                                             bool active, int itype, NState &st,
                                             curandStateMRG32k3a &condState, Smem &sm, int farSlot = -1) {
    const int bs = P.blockSize, nV1 = P.nV1;
    // the far ring slot of step tp (tp mod farDepth; passed in by the persistent kernel)
    if (farSlot < 0) farSlot = far_ring_slot(P, tp);
    const int ngE = P.ngE, ngI = P.ngI;
    const float *sPrev = P.sInfo + (size_t)(tp & 1) * nV1;
    float lgE[kMaxNG], lhE[kMaxNG], lgI[kMaxNG], lhI[kMaxNG], ipE[kMaxNG], ipI[kMaxNG];
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        lgE[ig] = lhE[ig] = lgI[ig] = lhI[ig] = 0.f;
        ipE[ig] = ig < ngE ? P.pE[itype * ngE + ig] : 0.f;
        ipI[ig] = ig < ngI ? P.pI[itype * ngI + ig] : 0.f;
    }
    // far events arriving in step tp, fetched early so that the loads overlap the compaction
    const int ns = ngE + ngI;
    unsigned long long farG[2 * kMaxNG], farH[2 * kMaxNG];
    unsigned long long *acc = nullptr;
    bool farSpiked = false;
    if (P.farClass && active) {
        acc = P.farAcc + (size_t)farSlot * ns * 2 * nV1;
        farSpiked = __ldcg(P.farFlag + tp % 3) != 0;
#pragma unroll
        for (int q = 0; q < 2 * kMaxNG; q++) {
            farG[q] = q < ns ? __ldcg(acc + (size_t)(2 * q) * nV1 + i) : 0ull;
            farH[q] = q < ns ? __ldcg(acc + (size_t)(2 * q + 1) * nV1 + i) : 0ull;
        }
    }
    float *recNear = nullptr;
    int nNearDraw = 0;
    if (Rng && P.recNear && active) {
        long long rs = tp - P.recStep0;
        if (rs >= 0 && rs < P.recSteps) recNear = P.recNear + ((size_t)rs * nV1 + i) * P.recCap;
    }
    // delayed near events with synaptic failure: recal_G_mat (src/coredynamics.cu:2138-2224)
    // restated per post -- its near synapses in the reference's order, the two spike-word
    // slots that can deliver in step tp, a normal draw from the post's generator for each
    // arriving event of a pair with failure rate p > 0, float sums in that order
    if constexpr (Rng) {
        if (P.nearPullOn && active) {
            const float dt = P.dt;
            for (int e = P.npOff[i]; e < P.npOff[i + 1]; e++) {
                const int pre = P.npPre[e];
                const int steps = P.npSteps[e];
                const float frac = P.npFrac[e];
                const bool preE = (pre % bs) < P.nE;
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    const long long ts = tp - steps + k;
                    const long long row = ((ts % P.sDepth) + P.sDepth) % P.sDepth;
                    const float sI = __ldcg(P.sRing + (size_t)row * nV1 + pre);
                    if (!(sI >= 1.0f)) continue;
                    const float nsp = floorf(sI);
                    const float dtsp = (sI - nsp + (float)k) * dt - frac;
                    if (!(dtsp < dt && dtsp >= 0)) continue;
                    float f = P.npStr[e];
                    const float pf = P.npP[e];
                    if (pf > 0) {
                        const float rnd = curand_normal(&condState);
                        if (recNear) {
                            if (nNearDraw < P.recCap) recNear[nNearDraw] = rnd;
                            else atomicOr(P.err, kErrRecordOverflow);
                        }
                        nNearDraw++;
                        f *= 1 - pf + P.npStd[e] * rnd;
                    }
                    if (f > 0) {
                        const float delta = dt - dtsp;
#pragma unroll
                        for (int ig = 0; ig < kMaxNG; ig++) {
                            if (preE && ig < ngE)
                                cond_input_v(P.condE.rise[ig], P.condE.decay[ig], P.condE.dod[ig], lgE[ig], lhE[ig],
                                             nsp * f * ipE[ig], delta);
                            if (!preE && ig < ngI)
                                cond_input_v(P.condI.rise[ig], P.condI.decay[ig], P.condI.dod[ig], lgI[ig], lhI[ig],
                                             nsp * f * ipI[ig], delta);
                        }
                    }
                }
            }
        }
    }
    // delayed near events (noDelay = 0): recal_G_mat sums them into the same step's
    // conductance update; here they were pushed into their own ring
    if (!P.noDelay) {
        if (P.nearOn && active) {
            unsigned long long *nacc = P.nearAcc + (size_t)farSlot * ns * 2 * nV1;
#pragma unroll
            for (int q = 0; q < 2 * kMaxNG; q++) {
                if (q < ns) {
                    unsigned long long *pg = nacc + (size_t)(2 * q) * nV1 + i;
                    unsigned long long *ph = nacc + (size_t)(2 * q + 1) * nV1 + i;
                    const unsigned long long ug = __ldcg(pg), uh = __ldcg(ph);
                    if (ug | uh) {
                        *pg = 0ull;
                        *ph = 0ull;
                        const float fg = far_from_fixed(ug), fh = far_from_fixed(uh);
#pragma unroll
                        for (int ig = 0; ig < kMaxNG; ig++) {
                            if (q < ngE && ig == q) { lgE[ig] = fg; lhE[ig] = fh; }
                            if (q >= ngE && ig == q - ngE) { lgI[ig] = fg; lhI[ig] = fh; }
                        }
                    }
                }
            }
        }
    }
    const int nnb = P.noDelay ? P.nNearNB[b] : 0;
    for (int ib = 0; ib < nnb; ib++) {
        const int nb = P.nbId[b * P.nnbMax + ib];
        int cntE;
        const int cnt = compact_spikers(P, sPrev + (size_t)nb * bs, sm, &cntE);
        if (cnt == 0) continue;
        if (active) {
            const float *col = P.conMat + ((size_t)(b * P.nnbMax + ib) * bs) * bs + local;
            for (int r0 = 0; r0 < cnt; r0 += kConBatch) {
                float sv[kConBatch];
#pragma unroll
                for (int k = 0; k < kConBatch; k++)
                    sv[k] = r0 + k < cnt ? __ldg(col + (size_t)sm.pre[r0 + k] * bs) : 0.f;
#pragma unroll
                for (int k = 0; k < kConBatch; k++) {
                    const int r = r0 + k;
                    float strength = sv[k];
                    if (r < cnt && strength > 0) {
                        const bool isE = r < cntE;
                        if constexpr (Rng) {
                            if (P.condRng) {
                                // pre type from the spiker's rank, as the reference does
                                // (src/coredynamics.cu:2760-2766, 2815-2821)
                                const int rank = isE ? r : r - cntE;
                                const int ja = isE ? 0 : P.nTypeE, jb = isE ? P.nTypeE : P.nType;
                                int jtype = ja;
                                for (int jj = ja; jj < jb; jj++) {
                                    if (rank < P.typeAcc[jj]) { jtype = jj; break; }
                                }
                                const int idx = jtype * P.nType + itype;
                                const float lp = P.synFail[idx];
                                const float normed_std = sqrtf(lp * (1 - lp) / P.synPerCon[idx]);
                                const float rnd = curand_normal(&condState);
                                if (recNear) {
                                    if (nNearDraw < P.recCap) recNear[nNearDraw] = rnd;
                                    else atomicOr(P.err, kErrRecordOverflow);
                                }
                                nNearDraw++;
                                strength *= 1 - lp + normed_std * rnd;
                            }
                        }
                        if (strength > 0) {
                            if (isE) {
#pragma unroll
                                for (int ig = 0; ig < kMaxNG; ig++) {
                                    if (ig < ngE) {
                                        const float str = strength * ipE[ig];
                                        lgE[ig] += str * sm.og[ig][r];
                                        lhE[ig] += str * sm.oh[ig][r];
                                    }
                                }
                            } else {
#pragma unroll
                                for (int ig = 0; ig < kMaxNG; ig++) {
                                    if (ig < ngI) {
                                        const float str = strength * ipI[ig];
                                        lgI[ig] += str * sm.og[ig][r];
                                        lhI[ig] += str * sm.oh[ig][r];
                                    }
                                }
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
    if (recNear) P.recNearCount[(size_t)(tp - P.recStep0) * nV1 + i] = nNearDraw;
    if (P.ffMode && P.ffMode != 3 && active && local < P.nE) learn_avg_delivery(P, __ldcg(sPrev + i), b, local);
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        st.gE[ig] += lgE[ig]; st.hE[ig] += lhE[ig];
        st.gI[ig] += lgI[ig]; st.hI[ig] += lhI[ig];
    }
    // far sums of the failure path (already zero when no far presynaptic neuron spiked)
    if (P.farPullOn && active) {
#pragma unroll
        for (int q = 0; q < 2 * kMaxNG; q++) {
            if (q < ns) {
                const float fg = __ldcg(P.farPull + (size_t)(2 * q) * nV1 + i);
                const float fh = __ldcg(P.farPull + (size_t)(2 * q + 1) * nV1 + i);
#pragma unroll
                for (int ig = 0; ig < kMaxNG; ig++) {
                    if (q < ngE && ig == q) { st.gE[ig] += fg; st.hE[ig] += fh; }
                    if (q >= ngE && ig == q - ngE) { st.gI[ig] += fg; st.hI[ig] += fh; }
                }
            }
        }
    }
    // far events (sum_G adds them after the near delivery); the ring slot is cleared
    if (acc) {
#pragma unroll
        for (int q = 0; q < 2 * kMaxNG; q++) {
            if (q < ns) {
                if (farG[q] | farH[q]) {
                    acc[(size_t)(2 * q) * nV1 + i] = 0ull;
                    acc[(size_t)(2 * q + 1) * nV1 + i] = 0ull;
                }
                if (farSpiked) {
                    const float fg = far_from_fixed(farG[q]);
                    const float fh = far_from_fixed(farH[q]);
#pragma unroll
                    for (int ig = 0; ig < kMaxNG; ig++) {
                        if (q < ngE && ig == q) { st.gE[ig] += fg; st.hE[ig] += fh; }
                        if (q >= ngE && ig == q - ngE) { st.gI[ig] += fg; st.hI[ig] += fh; }
                    }
                }
            }
        }
    }
    if (P.rec && active) {
        const long long slot = tp % P.recSlots;
        float *r = P.rec + slot * P.recStride;
        const RecOff o = rec_off(P);
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            if (ig < ngE) r[o.gE + ig * nV1 + i] = st.gE[ig];
            if (ig < ngI) r[o.gI + ig * nV1 + i] = st.gI[ig];
            if (P.hWrite) {
                if (ig < ngE) r[o.hE + ig * nV1 + i] = st.hE[ig];
                if (ig < ngI) r[o.hI + ig * nV1 + i] = st.hI[ig];
            }
        }
    }
}

// The tonic drive of the AdEx constructor (src/coredynamics.cuh:41-49).
__device__ __forceinline__ float tonic_current(const V1Params &P, int itype, float tonic) {
    const float vT = P.vT[itype], gL = P.gL[itype], aa = P.a[itype], deltaT = P.deltaT[itype];
    const float targetV = P.vL + (vT - P.vL) * tonic;
    if (targetV > vT) return (gL + aa) * (targetV - P.vL) - gL * deltaT;
    return (gL + aa) * (targetV - P.vL) - gL * deltaT * expf((targetV - vT) / deltaT);
}

// One LGN synapse with spike word sFF and weight f (src/coredynamics.cu:1476-1500).
template <bool Rng>
__device__ __forceinline__ void lgn_input(const V1Params &P, int itype, float sFF, float f, bool backingUp,
                                          float tBack, float pf, float nSynFF, float *g0, float *h0,
                                          float *g1, float *h1, curandStateMRG32k3a &condState,
                                          float *recFF, int &nFF) {
    const float dt = P.dt;
    const unsigned nspFF = (unsigned)floorf(sFF);
    if (nspFF == 0) return;
    const float tspFF = (sFF - nspFF) * dt;
    if constexpr (Rng) {
        if (pf > 0) {
            const float normed_std = sqrtf(pf * (1 - pf) / nSynFF);
            const float rnd = curand_normal(&condState);
            if (recFF) {
                if (nFF < P.recCap) recFF[nFF] = rnd;
                else atomicOr(P.err, kErrRecordOverflow);
            }
            nFF++;
            f *= 1 - pf + normed_std * rnd;
        }
    }
    if (f > 0) {
        const float ddt = backingUp ? tBack - tspFF : 0.f;
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            if (ig < P.ngFF) {
                const float str = f * P.pFF[itype * P.ngFF + ig];
                if (backingUp && ddt > 0) cond_input(P.condFF, g0[ig], h0[ig], str * nspFF, ddt, ig);
                cond_input(P.condFF, g1[ig], h1[ig], str * nspFF, dt - tspFF, ig);
            }
        }
    }
}

// Phase B: one membrane step of neuron i.  With SmemSyn the spike words and weights of the
// neuron's synapses are in shared memory (smS, smW: [synapse][kCta] from the thread's column);
// with RegSyn the synapse ids are the register array lgnIds (up to kMaxLgnReg of them) and
// the weights are read only for synapses that received a spike; otherwise ids and weights are
// loaded batch by batch.  Returns the spike word.
template <bool Rng, bool RegSyn, bool SmemSyn = false>
__device__ __forceinline__ float step_neuron(const V1Params &P, long long t, int i, int itype,
                                             float tonic, float depC, int m, const int *lgnIds,
                                             const float *__restrict__ lgnSInfo,
                                             NState &st, curandStateMRG32k3a &condState,
                                             curandStateMRG32k3a &noisyState,
                                             const LgnPre *pre = nullptr, const float *smW = nullptr,
                                             const float *smS = nullptr) {
    const int nV1 = P.nV1;
    const float dt = P.dt;
    const int ngE = P.ngE, ngI = P.ngI, ngFF = P.ngFF;
    // spike words of this neuron's LGN inputs, gathered first so that they overlap the decay
    // (unless the caller fetched them already: pre)
    float spReg[RegSyn ? kMaxLgnReg : 1];
    if constexpr (RegSyn) {
        if (!pre) {
#pragma unroll
            for (int q = 0; q < kMaxLgnReg; q++) spReg[q] = q < m ? __ldcg(lgnSInfo + lgnIds[q]) : 0.f;
        }
    }
    const float vR = P.vR[itype], vThres = P.vThres[itype], gL = P.gL[itype];
    const float Cm = P.C[itype], tRef = P.tRef[itype], vT = P.vT[itype];
    const float deltaT = P.deltaT[itype], tau_w = P.tau_w[itype], aa = P.a[itype];
    const float bb = P.b[itype];
    const float v0 = st.v;
    float w0 = st.w;
    float tBack = st.tBack;
    const float noise0 = st.lastNoise;

    // cortical conductances: keep the start-of-step value, decay to the end
    float ge[kMaxNG], he[kMaxNG], gi[kMaxNG], hi[kMaxNG];
    float gE_t1 = 0.0f, gI_t1 = 0.0f;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        ge[ig] = st.gE[ig]; he[ig] = st.hE[ig];
        if (ig < ngE) {
            cond_decay_step(P.condE, P.decE, st.gE[ig], st.hE[ig], ig);
            gE_t1 += st.gE[ig];
        }
    }
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        gi[ig] = st.gI[ig]; hi[ig] = st.hI[ig];
        if (ig < ngI) {
            cond_decay_step(P.condI, P.decI, st.gI[ig], st.hI[ig], ig);
            gI_t1 += st.gI[ig];
        }
    }
    float g0[kMaxNG], h0[kMaxNG], g1[kMaxNG], h1[kMaxNG];
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        g1[ig] = st.gFF[ig];
        h1[ig] = st.hFF[ig];
        g0[ig] = g1[ig];
        h0[ig] = h1[ig];
        if (ig < ngFF) cond_decay_step(P.condFF, P.decFF, g1[ig], h1[ig], ig);
    }
    // noise (src/coredynamics.cu:1422-1440)
    float noise1 = 0.f;
    if constexpr (Rng) {
        const float noiseRatio = P.noiseOnTonic ? tonic : 1.0f;
        noise1 = sqrtf(2 * P.noisyDep[itype] * (vT - vR) * noiseRatio * dt);
        if (noise1 > 0) {
            const float rnd = curand_normal(&noisyState);
            if (P.recNoise) {
                long long rs = t - P.recStep0;
                if (rs >= 0 && rs < P.recSteps) P.recNoise[(size_t)rs * nV1 + i] = rnd;
            }
            noise1 *= rnd;
            if (P.tau_noise > 0) {
                noise1 /= P.tau_noise;
                const float hk1 = -noise0 / P.tau_noise;
                const float hk2 = -(noise0 + dt * hk1 + noise1) / P.tau_noise;
                noise1 += noise0 + dt * (hk1 + hk2) / 2;
                st.lastNoise = noise1;
            }
        }
    }
    const float pf = Rng ? P.synFailFF[itype] : 0.f;
    const float nSynFF = P.synPerConFF[itype];
    const bool backingUp = tBack < dt && tBack > 0;
    const float depOut = depC + noise1;
    P.dep[i] = depOut;
    if (backingUp) {
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++)
            if (ig < ngFF) cond_decay(P.condFF, g0[ig], h0[ig], tBack, ig);
    }
    // LGN input (src/coredynamics.cu:1466-1502), synapse order kept
    float *recFF = nullptr;
    int nFF = 0;
    if (Rng && P.recFF) {
        long long rs = t - P.recStep0;
        if (rs >= 0 && rs < P.recSteps) recFF = P.recFF + ((size_t)rs * nV1 + i) * P.recCap;
    }
    if constexpr (SmemSyn) {
        // the step's spike words (copied in by lgn_words_async) and the weights in shared
        // memory, [synapse][kCta] from this thread's column: no global load
        unsigned mask = 0u;
#pragma unroll
        for (int q = 0; q < kMaxLgnReg; q++)
            if (q < m) mask |= (smS[q * kCta] >= 1.0f ? 1u : 0u) << q;
        while (mask) {
            const int q = __ffs(mask) - 1;
            mask &= mask - 1;
            lgn_input<Rng>(P, itype, smS[q * kCta], smW[q * kCta], backingUp, tBack, pf, nSynFF, g0, h0, g1, h1,
                           condState, recFF, nFF);
        }
    } else if constexpr (RegSyn) {
        // synapses that received a spike, as a bit mask; they are visited in synapse order
        unsigned mask = 0u;
        if (pre) {
            mask = pre->mask;
            if (mask) {  // the first spiking synapse comes with its spike word and weight
                lgn_input<Rng>(P, itype, pre->s0, pre->f0, backingUp, tBack, pf, nSynFF, g0, h0, g1, h1, condState,
                               recFF, nFF);
                mask &= mask - 1;
            }
        } else {
#pragma unroll
            for (int q = 0; q < kMaxLgnReg; q++) mask |= (spReg[q] >= 1.0f ? 1u : 0u) << q;
        }
        while (mask) {
            const int q = __ffs(mask) - 1;
            mask &= mask - 1;
            const size_t lid = (size_t)q * nV1 + i;
            const float sFF = __ldcg(lgnSInfo + __ldg(P.lgnId + lid));
            const float f = __ldg(P.sLGN + lid);
            lgn_input<Rng>(P, itype, sFF, f, backingUp, tBack, pf, nSynFF, g0, h0, g1, h1, condState, recFF,
                           nFF);
        }
    } else if (m <= kMaxLgnReg) {
        // ids and spike words in chunks of 16 (all loads of a chunk in flight together); the
        // weight is read only for synapses that received a spike, in synapse order
        unsigned mask = 0u;
#pragma unroll
        for (int c = 0; c < kMaxLgnReg; c += 16) {
            if (c < m) {
                int ids[16];
#pragma unroll
                for (int k = 0; k < 16; k++) ids[k] = c + k < m ? __ldg(P.lgnId + (size_t)(c + k) * nV1 + i) : 0;
#pragma unroll
                for (int k = 0; k < 16; k++)
                    mask |= ((c + k < m && __ldcg(lgnSInfo + ids[k]) >= 1.0f) ? 1u : 0u) << (c + k);
            }
        }
        while (mask) {
            const int q = __ffs(mask) - 1;
            mask &= mask - 1;
            const size_t lid = (size_t)q * nV1 + i;
            const float sFF = __ldcg(lgnSInfo + __ldg(P.lgnId + lid));
            const float f = __ldg(P.sLGN + lid);
            lgn_input<Rng>(P, itype, sFF, f, backingUp, tBack, pf, nSynFF, g0, h0, g1, h1, condState, recFF,
                           nFF);
        }
    } else {
        for (int q0 = 0; q0 < m; q0 += kLgnBatch) {
            int ids[kLgnBatch];
            float fs[kLgnBatch], sp[kLgnBatch];
#pragma unroll
            for (int k = 0; k < kLgnBatch; k++) {
                const size_t lid = (size_t)(q0 + k) * nV1 + i;
                ids[k] = q0 + k < m ? __ldg(P.lgnId + lid) : 0;
                fs[k] = q0 + k < m ? __ldg(P.sLGN + lid) : 0.f;
            }
#pragma unroll
            for (int k = 0; k < kLgnBatch; k++) sp[k] = q0 + k < m ? __ldcg(lgnSInfo + ids[k]) : 0.f;
#pragma unroll
            for (int k = 0; k < kLgnBatch; k++) {
                if (q0 + k < m)
                    lgn_input<Rng>(P, itype, sp[k], fs[k], backingUp, tBack, pf, nSynFF, g0, h0, g1, h1, condState,
                                   recFF, nFF);
            }
        }
    }
    if (recFF) P.recFFCount[(size_t)(t - P.recStep0) * nV1 + i] = nFF;
    float gE_t0 = 0.0f;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        if (ig < ngFF) {
            gE_t0 += g0[ig];
            gE_t1 += g1[ig];
        }
        st.gFF[ig] = g1[ig];
        st.hFF[ig] = h1[ig];
    }
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        if (ig < ngE) {
            if (backingUp) cond_decay(P.condE, ge[ig], he[ig], tBack, ig);
            gE_t0 += ge[ig];
        }
    }
    float gI_t0 = 0.0f;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        if (ig < ngI) {
            if (backingUp) cond_decay(P.condI, gi[ig], hi[ig], tBack, ig);
            gI_t0 += gi[ig];
        }
    }
    // stepping (src/coredynamics.cu:1546-1590; AdEx src/coredynamics.cuh:27-118)
    float v = v0, w = w0, tsp = 0.f;
    int spikeCount = 0;
    if (tBack < dt) {
        const float a0 = gE_t0 + gI_t0 + gL;
        const float b0 = gE_t0 * P.vE + gI_t0 * P.vI + gL * P.vL + depC;
        const float a1 = gE_t1 + gI_t1 + gL;
        const float b1 = gE_t1 * P.vE + gI_t1 * P.vI + gL * P.vL + depC;
        const float new_dt = dt - tBack;
        if (backingUp) {
            const float A = aa * (v0 - P.vL);
            w0 = (w0 - A) * expf(-tBack / tau_w) + A;
        }
        float nz0, nz1;
        if (P.tau_noise > 0) { nz0 = noise0; nz1 = noise1; }
        else { noise1 /= dt; nz0 = noise1; nz1 = noise1; }
        {
            const float dTgL = deltaT * gL;
            const float fk1 = (-a0 * v0 + b0 + dTgL * expf((v0 - vT) / deltaT) - w0) / Cm + nz0;
            const float gk1 = (aa * (v0 - P.vL) - w0) / tau_w;
            const float v1 = v0 + new_dt * fk1;
            const float w1 = w0 + new_dt * gk1;
            const float fk2 = (-a1 * v1 + b1 + dTgL * expf((v1 - vT) / deltaT) - w1) / Cm + nz1;
            const float gk2 = (aa * (v1 - P.vL) - w1) / tau_w;
            w = w0 + new_dt * (gk1 + gk2) / 2;
            v = v0 + new_dt * (fk1 + fk2) / 2;
        }
        if (v > vThres) {
            const float ratio = (vThres - v0) / (v - v0);
            tsp = tBack + ratio * new_dt;
            w0 += ratio * (w - w0) + bb;
            if (!(tsp >= 0)) atomicOr(P.err, kErrNegTsp);
            spikeCount = 1;
            tBack = tsp + tRef;
            v = vR;
        } else {
            if (tBack > 0) tBack = 0;
        }
    }
    if (tBack >= dt) {
        v = vR;
        const float A = aa * (v - P.vL);
        w = (w0 - A) * expf(-(dt - tsp) / tau_w) + A;
        tBack -= dt;
    }
    const float sInfo = spikeCount > 0 ? 1.0f + tsp / dt : v;
    st.v = v;
    if (P.iModel == 1) st.w = w;
    st.tBack = tBack;
    __stcg(P.sInfo + (size_t)(t & 1) * nV1 + i, sInfo);
    if (P.recSpk) P.recSpk[(size_t)(t % P.recSlots) * nV1 + i] = sInfo;
    if (P.rec) {
        const long long slot = t % P.recSlots;
        float *r = P.rec + slot * P.recStride;
        const RecOff o = rec_off(P);
        r[o.sinfo + i] = sInfo;
        r[o.dep + i] = depOut;
        if (P.iModel == 1) r[o.w + i] = w;
        r[o.v + i] = v;
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            if (ig < ngFF) r[o.gFF + ig * nV1 + i] = g1[ig];
            if (P.hWrite && ig < ngFF) r[o.hFF + ig * nV1 + i] = h1[ig];
        }
    }
    return sInfo;
}

// LGN->V1 plasticity after the membrane step of neuron i (learning 1-3): the learning block
// of compute_V_collect_spike_learnFF_fast (src/coredynamics.cu:1631-1993) with one FF->E type
// for excitatory posts and, with learning 2, one FF->I type for inhibitory posts.  The post
// LTD and triplet traces and the filtered rate are read at the step start and, when the neuron
// spiked, decayed to its spike time tsp; each LGN synapse (in synapse order) takes the
// homeostatic factor, LTD when its LGN cell spiked (from the post LTD trace at the earlier of
// the two spike times, scaled by the squared filtered rate when targetFR > 0), LTP when the
// neuron spiked (the presynaptic trace at the step start or right after the LGN spike,
// whichever precedes tsp, decayed to tsp, times the post triplet trace), and is clipped to
// [gmin, gmax]; the post traces then take the spike count and decay to the end of the step.
// The reference's choices kept: with learning != 3 the excitatory filtered rate is not
// advanced here but stored at tsp into its second slot for the delivery to advance
// (vAvgE[2*eid+1], src/coredynamics.cu:1746-1748); the inhibitory posts' LTP reads
// presynaptic trace 0 (layer 1 + 3j of the LGN surface with j counting from 0,
// src/coredynamics.cu:1905-1912), which is the FF->E type's trace when both types learn.
// Float arithmetic in the reference's order.
__device__ __noinline__ void learn_ff(const V1Params &P, long long t, int i, int local, int m, float sInfo,
                                      const float *__restrict__ lgnSInfo, const float *__restrict__ preRow,
                                      int nLGN) {
    const bool isE = local < P.nE;
    if (!isE && !P.ffI) return;
    const FFType &T = P.ffT[isE ? 0 : 1];
    const float dt = P.dt;
    float nsp, tsp;
    if (sInfo > 0) {
        nsp = floorf(sInfo);
        tsp = (sInfo - nsp) * dt;
    } else {
        nsp = 0;
        tsp = dt;
    }
    const int nV1 = P.nV1;
    const int nEt = P.nE * P.nblock, nIt = P.nI * P.nblock;
    const int b = i / P.blockSize;
    const int id = isE ? b * P.nE + local : b * P.nI + (local - P.nE);   // eid / iid
    float *vLTD = isE ? P.ffPost : P.ffPost + P.ffOffI;
    float *vTrip = isE ? P.ffPost + nEt : P.ffPost + P.ffOffI + nIt;
    float *vAvg = isE ? P.ffPost + P.ffOffAvgE + 2 * id : P.ffPost + P.ffOffAvgI + id;
    // row 0: the step start; row 1: the spike time
    float lLTD[2], lTrip[2], lAvg[2];
    lLTD[0] = vLTD[id];
    lTrip[0] = vTrip[id];
    lAvg[0] = vAvg[0];
    lLTD[1] = lTrip[1] = lAvg[1] = 0.f;
    if (nsp > 0) {
        lLTD[1] = lLTD[0];
        lTrip[1] = lTrip[0];
        lLTD[1] *= expf(-tsp / T.tauLTD);
        lTrip[1] *= expf(-tsp / T.tauTrip);
        lAvg[1] = lAvg[0];
        lAvg[1] *= expf(-tsp / T.tauAvg);
        if (isE && P.ffMode != 3) vAvg[1] = lAvg[1];
    }
    float new0 = 0.f, change = 0.f, delta_f = 0.f;
    if (P.applyHomeo) {
        const float f0 = P.totalFF[i];
        const float finf = P.totalFF[nV1 + i];
        const float d = f0 - finf;
        if (d > 0 || P.symmetricHomeo) {
            new0 = d * P.expHomeo + finf;
            change = P.applyHomeo == 1 ? new0 / f0 : (new0 - f0) / (float)m;
        } else {
            new0 = f0;
            change = P.applyHomeo == 1 ? 1.f : 0.f;
        }
    }
    for (int q = 0; q < m; q++) {
        const size_t lid = (size_t)q * nV1 + i;
        float f = P.sLGNw[lid];
        if (f == 0 && !P.rebound) continue;
        if (P.applyHomeo == 1) f *= change;
        else if (P.applyHomeo == 2) f += change;
        const int cell = __ldg(P.lgnId + lid);
        const float sFF = __ldcg(lgnSInfo + cell);
        const unsigned nspFF = (unsigned)floorf(sFF);
        const float tspFF = (sFF > 0 ? sFF - (float)nspFF : 1.f) * dt;
        if (nspFF > 0) {  // LTD, whether or not the neuron spiked
            int cPick;
            float delta_t;
            if (tspFF < tsp) {
                cPick = 0;
                delta_t = tspFF;
            } else {
                cPick = 1;
                delta_t = tspFF - tsp;
            }
            float A_LTD = T.A_ratio;
            if (T.targetFR > 0) A_LTD *= T.tauLTP * lAvg[cPick] * lAvg[cPick];
            const float df = lLTD[cPick] * expf(-delta_t / T.tauLTD) * A_LTD;
            f -= df;
            if (P.applyHomeo) delta_f -= df;
        }
        if (nsp > 0) {  // LTP, whether or not the LGN cell spiked
            float lpre, delta_t;
            if (tspFF < tsp) {
                lpre = __ldcg(preRow + nLGN + cell);
                delta_t = tsp - tspFF;
            } else {
                lpre = __ldcg(preRow + cell);
                delta_t = tsp;
            }
            const float df = lpre * expf(-delta_t / T.tauLTP) * lTrip[1] * T.A_LTP;
            if (P.applyHomeo) delta_f += df;
            f += df;
        }
        if (f < T.gmin) {
            if (P.applyHomeo) delta_f += T.gmin - f;
            f = T.gmin;
        }
        if (f > T.gmax) {
            if (P.applyHomeo) delta_f -= f - T.gmax;
            f = T.gmax;
        }
        P.sLGNw[lid] = f;
    }
    if (P.applyHomeo) P.totalFF[i] = new0 + delta_f;
    // the post traces take this step's spikes and decay to its end
    float delta_t = dt;
    const int cPick = nsp > 0 ? 1 : 0;
    if (nsp > 0) delta_t -= tsp;
    lLTD[cPick] += nsp;
    lTrip[cPick] += nsp;
    lLTD[cPick] *= expf(-delta_t / T.tauLTD);
    lTrip[cPick] *= expf(-delta_t / T.tauTrip);
    vLTD[id] = lLTD[cPick];
    vTrip[id] = lTrip[cPick];
    if (!isE || P.ffMode == 3) {
        lAvg[cPick] += nsp;
        lAvg[cPick] *= expf(-delta_t / T.tauAvg);
        vAvg[0] = lAvg[cPick];
    }
}

// Phase B when dt exceeds the shortest refractory period: a neuron may fire several times in
// one step (compute_V_collect_spike_learnFF, src/coredynamics.cu:427-845, without learning).
// After each spike whose refractory period ends inside the step the membrane is integrated
// again from the end of that period (tBack): the feed-forward and cortical conductances at
// tBack are advanced from the previous interval start, inputs arriving after the interval
// start and before tBack are added, w is carried with v held at vR, and RK2 runs over the rest
// of the step.  The end-of-step conductances (g1) and the failure draws come from the first
// pass only.  Kept from the reference: with tau_noise = 0 the noise term is divided by dt once
// more on every pass (src/coredynamics.cu:758-759).  The spike word is
// nsp + mean(tsp)/dt.  m <= kMaxLgnMulti (checked by the host).
template <bool Rng>
__device__ __noinline__ float step_neuron_multi(const V1Params &P, long long t, int i, int itype, float tonic, float depC,
                                   int m, const float *__restrict__ lgnSInfo, NState &st,
                                   curandStateMRG32k3a &condState, curandStateMRG32k3a &noisyState) {
    const int nV1 = P.nV1;
    const float dt = P.dt;
    const int ngE = P.ngE, ngI = P.ngI, ngFF = P.ngFF;
    const float vR = P.vR[itype], vThres = P.vThres[itype], gL = P.gL[itype];
    const float Cm = P.C[itype], tRef = P.tRef[itype], vT = P.vT[itype];
    const float deltaT = P.deltaT[itype], tau_w = P.tau_w[itype], aa = P.a[itype];
    const float bb = P.b[itype];
    float v0 = st.v;
    float w0 = st.w;
    float tBack = st.tBack;
    const float noise0 = st.lastNoise;
    float ge[kMaxNG], he[kMaxNG], gi[kMaxNG], hi[kMaxNG];
    float gE_t1 = 0.0f, gI_t1 = 0.0f;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        ge[ig] = st.gE[ig]; he[ig] = st.hE[ig];
        if (ig < ngE) {
            cond_decay_step(P.condE, P.decE, st.gE[ig], st.hE[ig], ig);
            gE_t1 += st.gE[ig];
        }
    }
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        gi[ig] = st.gI[ig]; hi[ig] = st.hI[ig];
        if (ig < ngI) {
            cond_decay_step(P.condI, P.decI, st.gI[ig], st.hI[ig], ig);
            gI_t1 += st.gI[ig];
        }
    }
    float g0[kMaxNG], h0[kMaxNG], g1[kMaxNG], h1[kMaxNG];
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        g1[ig] = st.gFF[ig];
        h1[ig] = st.hFF[ig];
        g0[ig] = g1[ig];
        h0[ig] = h1[ig];
        if (ig < ngFF) cond_decay_step(P.condFF, P.decFF, g1[ig], h1[ig], ig);
    }
    float noise1 = 0.f;
    if constexpr (Rng) {
        const float noiseRatio = P.noiseOnTonic ? tonic : 1.0f;
        noise1 = sqrtf(2 * P.noisyDep[itype] * (vT - vR) * noiseRatio * dt);
        if (noise1 > 0) {
            const float rnd = curand_normal(&noisyState);
            if (P.recNoise) {
                long long rs = t - P.recStep0;
                if (rs >= 0 && rs < P.recSteps) P.recNoise[(size_t)rs * nV1 + i] = rnd;
            }
            noise1 *= rnd;
            if (P.tau_noise > 0) {
                noise1 /= P.tau_noise;
                const float hk1 = -noise0 / P.tau_noise;
                const float hk2 = -(noise0 + dt * hk1 + noise1) / P.tau_noise;
                noise1 += noise0 + dt * (hk1 + hk2) / 2;
                st.lastNoise = noise1;
            }
        }
    }
    const float pf = Rng ? P.synFailFF[itype] : 0.f;
    const float nSynFF = P.synPerConFF[itype];
    const float depOut = depC + noise1;
    P.dep[i] = depOut;
    float *recFF = nullptr;
    int nFF = 0;
    if (Rng && P.recFF) {
        long long rs = t - P.recStep0;
        if (rs >= 0 && rs < P.recSteps) recFF = P.recFF + ((size_t)rs * nV1 + i) * P.recCap;
    }
    float fmod[kMaxLgnMulti];
    const int mm = m < kMaxLgnMulti ? m : kMaxLgnMulti;
    bool backingUp = tBack < dt && tBack > 0;
    float new_t0 = 0.f, tspSum = 0.f, v = v0, w = w0, tsp = 0.f;
    float a1 = 0.f, b1 = 0.f;
    int spikeCount = 0, pass = 0;
    do {
        const float dtBack = backingUp ? tBack - new_t0 : 0.f;
        if (backingUp) {
#pragma unroll
            for (int ig = 0; ig < kMaxNG; ig++)
                if (ig < ngFF) cond_decay(P.condFF, g0[ig], h0[ig], dtBack, ig);
        }
        for (int q = 0; q < mm; q++) {
            const size_t lid = (size_t)q * nV1 + i;
            if (spikeCount == 0) fmod[q] = __ldg(P.sLGN + lid);
            const float sFF = __ldcg(lgnSInfo + __ldg(P.lgnId + lid));
            const unsigned nspFF = (unsigned)floorf(sFF);
            const float tspFF = (sFF - nspFF) * dt;
            if (nspFF > 0 && tspFF >= new_t0) {
                if constexpr (Rng) {
                    if (spikeCount == 0 && pf > 0) {
                        const float normed_std = sqrtf(pf * (1 - pf) / nSynFF);
                        const float rnd = curand_normal(&condState);
                        if (recFF) {
                            if (nFF < P.recCap) recFF[nFF] = rnd;
                            else atomicOr(P.err, kErrRecordOverflow);
                        }
                        nFF++;
                        fmod[q] *= 1 - pf + normed_std * rnd;
                    }
                }
                if (fmod[q] > 0) {
                    const float ddt = backingUp ? tBack - tspFF : 0.f;
#pragma unroll
                    for (int ig = 0; ig < kMaxNG; ig++) {
                        if (ig < ngFF) {
                            const float str = fmod[q] * P.pFF[itype * ngFF + ig];
                            if (backingUp && ddt > 0) cond_input(P.condFF, g0[ig], h0[ig], str * nspFF, ddt, ig);
                            if (spikeCount == 0) cond_input(P.condFF, g1[ig], h1[ig], str * nspFF, dt - tspFF, ig);
                        }
                    }
                }
            }
        }
        float gE_t0 = 0.0f;
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            if (ig < ngFF) {
                gE_t0 += g0[ig];
                if (spikeCount == 0) gE_t1 += g1[ig];
            }
        }
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            if (ig < ngE) {
                if (backingUp) cond_decay(P.condE, ge[ig], he[ig], dtBack, ig);
                gE_t0 += ge[ig];
            }
        }
        float gI_t0 = 0.0f;
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            if (ig < ngI) {
                if (backingUp) cond_decay(P.condI, gi[ig], hi[ig], dtBack, ig);
                gI_t0 += gi[ig];
            }
        }
        tsp = 0.f;
        if (tBack < dt) {
            const float a0 = gE_t0 + gI_t0 + gL;
            const float b0 = gE_t0 * P.vE + gI_t0 * P.vI + gL * P.vL + depC;
            if (spikeCount == 0) {
                a1 = gE_t1 + gI_t1 + gL;
                b1 = gE_t1 * P.vE + gI_t1 * P.vI + gL * P.vL + depC;
            }
            const float new_dt = dt - tBack;
            if (backingUp) {
                const float A = aa * (v0 - P.vL);
                w0 = (w0 - A) * expf(-dtBack / tau_w) + A;
            }
            float nz0, nz1;
            if (P.tau_noise > 0) { nz0 = noise0; nz1 = noise1; }
            else { noise1 /= dt; nz0 = noise1; nz1 = noise1; }
            const float dTgL = deltaT * gL;
            const float fk1 = (-a0 * v0 + b0 + dTgL * expf((v0 - vT) / deltaT) - w0) / Cm + nz0;
            const float gk1 = (aa * (v0 - P.vL) - w0) / tau_w;
            const float v1 = v0 + new_dt * fk1;
            const float w1 = w0 + new_dt * gk1;
            const float fk2 = (-a1 * v1 + b1 + dTgL * expf((v1 - vT) / deltaT) - w1) / Cm + nz1;
            const float gk2 = (aa * (v1 - P.vL) - w1) / tau_w;
            w = w0 + new_dt * (gk1 + gk2) / 2;
            v = v0 + new_dt * (fk1 + fk2) / 2;
            if (v > vThres) {
                new_t0 = tBack;
                const float ratio = (vThres - v0) / (v - v0);
                tsp = new_t0 + ratio * new_dt;
                w0 += ratio * (w - w0) + bb;
                if (!(tsp >= 0)) atomicOr(P.err, kErrNegTsp);
                tspSum += tsp;
                spikeCount++;
                tBack = tsp + tRef;
                backingUp = tBack < dt;
                if (backingUp) v0 = vR;
                else v = vR;
            } else {
                if (tBack > 0) tBack = 0;
                backingUp = false;
            }
        }
        if (tBack >= dt) {
            v = vR;
            const float A = aa * (v - P.vL);
            w = (w0 - A) * expf(-(dt - tsp) / tau_w) + A;
            tBack -= dt;
        }
        if (++pass >= kMaxSpikePasses && backingUp) {
            atomicOr(P.err, kErrBounds);   // more passes than the refractory periods allow
            break;
        }
    } while (backingUp);
    if (recFF) P.recFFCount[(size_t)(t - P.recStep0) * nV1 + i] = nFF;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        st.gFF[ig] = g1[ig];
        st.hFF[ig] = h1[ig];
    }
    const float sInfo = spikeCount > 0 ? tspSum / (spikeCount * dt) + spikeCount : v;
    st.v = v;
    if (P.iModel == 1) st.w = w;
    st.tBack = tBack;
    __stcg(P.sInfo + (size_t)(t & 1) * nV1 + i, sInfo);
    if (P.recSpk) P.recSpk[(size_t)(t % P.recSlots) * nV1 + i] = sInfo;
    if (P.rec) {
        const long long slot = t % P.recSlots;
        float *r = P.rec + slot * P.recStride;
        const RecOff o = rec_off(P);
        r[o.sinfo + i] = sInfo;
        r[o.dep + i] = depOut;
        if (P.iModel == 1) r[o.w + i] = w;
        r[o.v + i] = v;
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            if (ig < ngFF) r[o.gFF + ig * nV1 + i] = g1[ig];
            if (P.hWrite && ig < ngFF) r[o.hFF + ig * nV1 + i] = h1[ig];
        }
    }
    return sInfo;
}

// One delayed event: the spike of `pre` at step t (spike word sI) through delayed synapse e,
// in its k-th arrival slot; arrival step and offset as recal_G_vec (src/coredynamics.cu:282-333)
// and recal_G_mat (2163-2200) compute them, with explicitly rounded operations.  `code` is the
// synapse's packed word: post type in bits 16-23, class in bit 24 (1: near block, delivered
// through nearAcc; 0: far, through farAcc).
__device__ __forceinline__ void far_event(const V1Params &P, long long t, int tSlot, int pre, float sI, int post,
                                          float f, int steps, int code, float frac, int kk) {
    const int ptype = (code >> 16) & 0xff;
    const bool nearClass = (code >> 24) & 1;
    const float dt = P.dt;
    const unsigned nsp = (unsigned)floorf(sI);
    // dtsp = (sInfo - nsp + k)*dt - time2post, rounded step by step
    const float x = __fadd_rn(__fsub_rn(sI, (float)nsp), (float)kk);
    const float dtsp = __fsub_rn(__fmul_rn(x, dt), frac);
    if (!(dtsp < dt && dtsp >= 0 && f > 0)) return;
    const long long tArr = t + steps - kk;
    if (tArr < t || tArr - t >= P.farDepth - 1) {
        atomicOr(P.err, kErrFarOverflow);
        return;
    }
    const int nV1 = P.nV1;
    const int ns = P.ngE + P.ngI;
    const bool preE = (pre % P.blockSize) < P.nE;
    const int ng = preE ? P.ngE : P.ngI;
    const int qoff = preE ? 0 : P.ngE;
    const float delta = __fsub_rn(dt, dtsp);
    // ring slot of tArr: tSlot is step t's (t mod farDepth, in [0, farDepth)) and 0 <= tArr - t
    // < farDepth - 1 (the only arrival before step 0 is the delivery that precedes the first
    // step when there are initial spikes: step -1, slot farDepth - 1)
    int aSlot = tSlot + (int)(tArr - t);
    if (aSlot >= P.farDepth) aSlot -= P.farDepth;
    unsigned long long *acc = (nearClass ? P.nearAcc : P.farAcc) + (size_t)aSlot * ns * 2 * nV1;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        if (ig < ng) {
            const float ip = preE ? P.pE[ptype * P.ngE + ig] : P.pI[ptype * P.ngI + ig];
            const float fv = __fmul_rn(__fmul_rn((float)nsp, f), ip);
            // conductance input of the arrival (cond_input of src/condShape.h:42-51) with the
            // hardware exponential and division (within a few ulp): the reference computes far
            // arrivals on the host, so no device expression reproduces its bits, and the
            // fixed-point ring already sums delayed near events in another order than its
            // recal_G_mat; the precise forms cost 14% of the step here
            const float rise = preE ? P.condE.rise[ig] : P.condI.rise[ig];
            const float dec = preE ? P.condE.decay[ig] : P.condI.decay[ig];
            const float dod = preE ? P.condE.dod[ig] : P.condI.dod[ig];
            const float etr = __expf(-__fdividef(delta, rise));
            const float g = fv * dod * (__expf(-__fdividef(delta, dec)) - etr);
            const float h = fv * etr;
            atomicAdd(&acc[(size_t)(2 * (qoff + ig)) * nV1 + post], (unsigned long long)far_to_fixed(g));
            atomicAdd(&acc[(size_t)(2 * (qoff + ig) + 1) * nV1 + post], (unsigned long long)far_to_fixed(h));
        }
    }
}

// Exclusive prefix of sm.fdeg[0..cnt) into sm.fpref (warp 0), total in sm.fpref[cnt].
__device__ __forceinline__ void scan_degrees(Smem &sm, int cnt) {
    const int lane = threadIdx.x & 31;
    if ((threadIdx.x >> 5) == 0) {
        int run = 0;
        for (int base = 0; base < cnt; base += 32) {
            const int r = base + lane;
            const int d = r < cnt ? sm.fdeg[r] : 0;
            int incl = d;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            if (r < cnt) sm.fpref[r] = run + incl - d;
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) sm.fpref[cnt] = run;
    }
}

// Entry r of the chunk in shared memory that owns flattened work item w: the last r with
// fpref[r] <= w.
__device__ __forceinline__ int owner_of(const Smem &sm, int cnt, int w) {
    int lo = 0, hi = cnt - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sm.fpref[mid] <= w) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Ring slot of step t in the far/near event rings.
__device__ __forceinline__ int far_ring_slot(const V1Params &P, long long t) {
    const long long r = t % P.farDepth;
    return (int)(r < 0 ? r + P.farDepth : r);
}

// Spiker count (high 32 bits) and synapse work (low 32 bits) of step tl's far list.
__device__ __forceinline__ unsigned long long far_list_size(const V1Params &P, long long tl) {
    return __ldcg(P.farCount + (int)((tl + 3) % 3));
}

// Phase C, part 1 (runs in step tl + 1): the far events of step tl's spikes that arrive after
// step tl, from the step's global spiker list.  The (spiker, synapse) work items are numbered
// in list order; the items [lo, hi) are shared by the nCta CTAs given, thread gt of them
// taking lo + gt, lo + gt + G, ... (G their threads), U items per pass with their synapse
// loads issued together.  The fixed-point ring makes the sums independent of which thread
// appends which event, and in which order.
template <int U = 1>
__device__ __forceinline__ void far_push_range(const V1Params &P, long long tl, Smem &sm, int cta, int nCta,
                                               unsigned long long size, int lo, int hi, int tSlot = -1) {
    const int n = (int)(size >> 32);
    if (n == 0 || lo >= hi) return;
    const int slot = (int)((tl + 3) % 3);  // tl >= -1
    const int4 *list = P.farList + (size_t)slot * P.nV1;
    if (tSlot < 0) tSlot = far_ring_slot(P, tl);
    const int G = nCta * kCta;
    const int gt = cta * kCta + threadIdx.x;
    int base = 0;  // items of the earlier chunks
    for (int c0 = 0; c0 < n && base < hi; c0 += kCta) {
        const int cnt = min(kCta, n - c0);
        __syncthreads();
        if (threadIdx.x < cnt) {
            const int4 e = __ldcg(list + c0 + threadIdx.x);
            sm.fpre[threadIdx.x] = e.x;
            sm.fe0[threadIdx.x] = e.y;
            sm.fdeg[threadIdx.x] = e.z;
            sm.fsi[threadIdx.x] = __int_as_float(e.w);
        }
        __syncthreads();
        scan_degrees(sm, cnt);
        __syncthreads();
        const int work = sm.fpref[cnt];
        // this chunk's items [base, base + work) within [lo, hi): the first of this thread's
        // items at or after max(base, lo)
        const int a = max(base, lo), z = min(base + work, hi);
        int w = lo + gt;
        if (w < a) w += (a - w + G - 1) / G * G;
        for (; w < z; w += U * G) {
            int rr[U], post[U], sp[U];
            float f[U], frac[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int wu = w + u * G - base;
                rr[u] = -1;
                if (w + u * G < z) {
                    const int r = owner_of(sm, cnt, wu);
                    const int e = sm.fe0[r] + (wu - sm.fpref[r]);
                    rr[u] = r;
                    const int4 rc = __ldg(P.farRec + e);
                    post[u] = rc.x;
                    f[u] = __int_as_float(rc.y);
                    sp[u] = rc.z;
                    frac[u] = __int_as_float(rc.w);
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (rr[u] < 0) continue;
                const int steps = sp[u] & 0xffff;
                const int pre = sm.fpre[rr[u]];
                const float sI = sm.fsi[rr[u]];
                // the slot arriving in step tl itself (steps == k) was pushed in step tl
                if (steps != 0) far_event(P, tl, tSlot, pre, sI, post[u], f[u], steps, sp[u], frac[u], 0);
                if (steps != 1) far_event(P, tl, tSlot, pre, sI, post[u], f[u], steps, sp[u], frac[u], 1);
            }
        }
        base += work;
    }
}

// All of step tl's far push, shared by nCta CTAs.
template <int U = 1>
__device__ __forceinline__ void far_push_list(const V1Params &P, long long tl, Smem &sm, int cta, int nCta,
                                              int tSlot = -1) {
    const unsigned long long size = far_list_size(P, tl);
    far_push_range<U>(P, tl, sm, cta, nCta, size, 0, (int)(size & 0xffffffffu), tSlot);
}

// Phase C, part 2 (runs in step t): appends this CTA's far presynaptic spikers to step t's
// global list (one atomic per warp), and pushes the events that arrive within step t itself
// (whole-step delay 0 or 1: the first n1 synapses of each list), which must be in the ring
// before the next step delivers it.  All threads of the CTA call it.
__device__ __forceinline__ void far_phase(const V1Params &P, long long t, int i, bool active, float sInfo,
                                          bool isFarPre, int e0, int deg, int n1, Smem &sm, int cta,
                                          int tSlot = -1) {
    if (cta == 0 && threadIdx.x == 0) {
        P.farFlag[(t + 1) % 3] = 0;
        P.farCount[(t + 1) % 3] = 0ull;
    }
    if (active && sInfo > 1.0f && isFarPre) P.farFlag[t % 3] = 1;
    const bool spk = active && sInfo >= 1.0f;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool app = spk && deg > 0;
    const unsigned ab = __ballot_sync(0xffffffffu, app);
    if (ab) {
        const int leader = __ffs(ab) - 1;
        // one atomic per warp adds its spikers (high half) and their synapses (low half)
        const unsigned wsum = __reduce_add_sync(0xffffffffu, app ? (unsigned)deg : 0u);
        int base = 0;
        if (lane == leader)
            base = (int)(atomicAdd(P.farCount + t % 3, ((unsigned long long)__popc(ab) << 32) | wsum) >> 32);
        base = __shfl_sync(0xffffffffu, base, leader);
        if (app)
            P.farList[(size_t)(t % 3) * P.nV1 + base + __popc(ab & ((1u << lane) - 1u))] =
                make_int4(i, e0, deg, __float_as_int(sInfo));
    }
    const bool push = spk && n1 > 0;
    const unsigned bal = __ballot_sync(0xffffffffu, push);
    if (lane == 0) sm.fball[warp] = bal;
    __syncthreads();
    // list of this CTA's neurons with same-step events (ascending) and their counts
    int cnt = 0, pos = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
        const int c = __popc(sm.fball[w]);
        if (w < warp) pos += c;
        cnt += c;
    }
    if (cnt == 0) return;
    if (push) {
        pos += __popc(bal & ((1u << lane) - 1u));
        sm.fpre[pos] = i;
        sm.fsi[pos] = sInfo;
        sm.fe0[pos] = e0;
        sm.fdeg[pos] = n1;
    }
    __syncthreads();
    scan_degrees(sm, cnt);
    __syncthreads();
    const int work = sm.fpref[cnt];
    if (tSlot < 0) tSlot = far_ring_slot(P, t);
    for (int w = threadIdx.x; w < work; w += kCta) {
        const int r = owner_of(sm, cnt, w);
        const int e = sm.fe0[r] + (w - sm.fpref[r]);
        const int4 rc = __ldg(P.farRec + e);
        const int post = rc.x;
        const float f = __int_as_float(rc.y);
        const int sp = rc.z;
        const float frac = __int_as_float(rc.w);
        const int steps = sp & 0xffff;
        // steps is 0 or 1 here: the slot with tArr == t
        far_event(P, t, tSlot, sm.fpre[r], sm.fsi[r], post, f, steps, sp, frac, steps);
    }
}

// One V1 step (with the delivery of the previous step first) for CTA `cta` of the nCta CTAs
// that hold one patch: the per-step kernel and the batched kernel run this body.
template <bool Rng>
__device__ __forceinline__ void v1_step_body(const V1Params &P, long long t, int cta, int nCta,
                                             const float *__restrict__ lgnRing, int lgnSlots,
                                             int deliverPrev, int doStep, Smem &sm) {
    const int bs = P.blockSize;
    const int nq = (bs + kCta - 1) / kCta;
    const int b = cta / nq;
    const int local = (cta % nq) * kCta + threadIdx.x;
    const bool active = local < bs;
    const int i = b * bs + (active ? local : 0);
    const int itype = type_of(P, active ? local : 0);

    NState st;
    load_state(P, i, st);
    curandStateMRG32k3a condState, noisyState;
    if (Rng && P.condRng && active) condState = P.rGenCond[i];
    if (Rng && P.noiseRng && active) noisyState = P.rNoisy[i];

    if (deliverPrev) deliver_prev<Rng>(P, t - 1, b, local, i, active, itype, st, condState, sm);
    if (!doStep) {
        if (active) {
            store_state(P, i, st);
            if (Rng && P.condRng) P.rGenCond[i] = condState;
        }
        return;
    }
    float sInfo = 0.f;
    if (active) {
        const float tonic = P.tonicDep[i];
        const float depC = tonic_current(P, itype, tonic);
        const float *lgnSInfo = lgnRing + (size_t)(t % lgnSlots) * P.lgnN;
        if (P.multiSpike)
            sInfo = step_neuron_multi<Rng>(P, t, i, itype, tonic, depC, P.nLGNperV1[i], lgnSInfo, st, condState,
                                           noisyState);
        else
            sInfo = step_neuron<Rng, false>(P, t, i, itype, tonic, depC, P.nLGNperV1[i], nullptr, lgnSInfo, st,
                                        condState, noisyState);
        store_state(P, i, st);
        if (Rng && P.condRng) P.rGenCond[i] = condState;
        if (Rng && P.noiseRng) P.rNoisy[i] = noisyState;
        if (P.spikeCount && sInfo >= 1.0f) P.spikeCount[i] += (unsigned)floorf(sInfo);
        if (P.farPullOn || P.nearPullOn) P.sRing[(size_t)(t % P.sDepth) * P.nV1 + i] = sInfo;
        if (P.ffLearn)
            learn_ff(P, t, i, local, P.nLGNperV1[i], sInfo, lgnSInfo,
                     P.ffPreRing + (size_t)(t % lgnSlots) * P.ffTypes * 2 * P.lgnN, P.lgnN);
    }
    if (P.farOn) {
        const int e0 = active ? P.farOff[i] : 0;
        const int deg = active ? P.farOff[i + 1] - e0 : 0;
        const int n1 = active ? P.farN1[i] : 0;
        const bool isFarPre = active && P.farPre[i];
        far_push_list(P, t - 1, sm, cta, nCta);
        far_phase(P, t, i, active, sInfo, isFarPre, e0, deg, n1, sm, cta);
    }
}

template <bool Rng>
__global__ void __launch_bounds__(kCta) v1_step_kernel(V1Params P, const long long *stepBase,
                                                       int stepOffset,
                                                       const float *__restrict__ lgnRing,
                                                       int lgnSlots, int deliverPrev,
                                                       int doStep) {
    __shared__ Smem sm;
    const long long t = *stepBase + stepOffset;
    v1_step_body<Rng>(P, t, blockIdx.x, gridDim.x, lgnRing, lgnSlots, deliverPrev, doStep, sm);
}

// Split grid barrier of the persistent kernel on a monotonic arrival counter (zeroed before
// each launch): the barrier after step s completes when the counter reaches nCTA * (s + 1).
// arrive() publishes this CTA's writes and counts it in; wait() polls the counter with a
// bounded number of attempts.  A CTA that gives up sets kErrBarrier and the abort bit of the
// counter, which releases and fails every other waiter.  Work placed between the two calls
// must not read what other CTAs write in the step (the next step's LGN spike words are
// written before the launch).
constexpr unsigned kBarrierAbort = 0x80000000u;
constexpr int kPushBatch = 8;   // far-push items per thread and pass of a far-push CTA

__device__ __forceinline__ void barrier_arrive(unsigned *count, unsigned *s_arrived) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        *s_arrived = atomicAdd(count, 1u) + 1u;
    }
}

__device__ __forceinline__ bool barrier_wait(unsigned *count, unsigned target, const unsigned *s_arrived,
                                             int *err, long long limit) {
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        unsigned c = *s_arrived;
        long long spins = 0;
        while ((c & ~kBarrierAbort) < target && !(c & kBarrierAbort)) {
            if (++spins > limit) {
                atomicOr(err, kErrBarrier);
                atomicOr(count, kBarrierAbort);
                c = kBarrierAbort;
                break;
            }
            if (spins > 64) __nanosleep(32);
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(count) : "memory");
        }
        __threadfence();
        s_ok = (c & kBarrierAbort) ? 0 : 1;
    }
    __syncthreads();
    return s_ok != 0;
}

// K steps in one cooperative launch.  Neuron state and generators stay in registers, the LGN
// synapses of each thread's neuron (up to kMaxLgnReg: ids, weights, the step's spike words) in
// shared memory; one grid barrier separates consecutive steps, and while a CTA waits at it the
// spike words of its neurons' LGN synapses for the next step are copied in.
template <bool Rng>
__global__ void __launch_bounds__(kCta, 1) v1_persistent_kernel(V1Params P, const long long *stepBase,
                                                                 int K, const float *__restrict__ lgnRing,
                                                                 int lgnSlots, int deliverFirst,
                                                                 unsigned *barrier) {
    __shared__ Smem sm;
    __shared__ unsigned s_arrived;
    const long long t0 = *stepBase;
    const int bs = P.blockSize;
    const int nq = (bs + kCta - 1) / kCta;
    const int nNeuron = (int)gridDim.x - P.pushCta;
    // the far-push CTAs take the first items of each step's push (one batch per thread), the
    // neuron CTAs the rest after their own step work
    const int pushShare = P.pushCta * kCta * kPushBatch;
    if ((int)blockIdx.x >= nNeuron) {
        // far-push CTA: in step t it pushes the far events of step t - 1's spikers (those that
        // arrive after step t - 1) while the neuron CTAs deliver and step; the grid barrier
        // that ends step t orders them before the delivery that reads them
        int fsPrev = far_ring_slot(P, t0 - 1);  // far ring slot of step t0 + s - 1
        for (int s = 0; s < K; s++) {
            if (P.farOn) {
                const unsigned long long size = far_list_size(P, t0 + s - 1);
                far_push_range<kPushBatch>(P, t0 + s - 1, sm, (int)blockIdx.x - nNeuron, P.pushCta, size, 0,
                                           min((int)(size & 0xffffffffu), pushShare), fsPrev);
            }
            if (++fsPrev == P.farDepth) fsPrev = 0;
            if (s + 1 < K) {
                barrier_arrive(barrier, &s_arrived);
                if (!barrier_wait(barrier, (unsigned)gridDim.x * (unsigned)(s + 1), &s_arrived, P.err, P.waitSpins))
                    break;
            }
        }
        return;
    }
    const int b = blockIdx.x / nq;
    const int local = (blockIdx.x % nq) * kCta + threadIdx.x;
    const bool active = local < bs;
    const int i = b * bs + (active ? local : 0);
    const int itype = type_of(P, active ? local : 0);

    NState st;
    load_state(P, i, st);
    curandStateMRG32k3a condState, noisyState;
    if (Rng && P.condRng && active) condState = P.rGenCond[i];
    if (Rng && P.noiseRng && active) noisyState = P.rNoisy[i];
    const float tonic = active ? P.tonicDep[i] : 0.f;
    const float depC = tonic_current(P, itype, tonic);
    const int m = active ? P.nLGNperV1[i] : 0;
    // this neuron's LGN synapses in shared memory, [synapse][kCta] per array: weights, the
    // current step's spike words (copied in asynchronously a step ahead), cell ids
    extern __shared__ __align__(16) float lgnSm[];
    const int mx = P.maxLGN;
    float *smW = lgnSm + threadIdx.x;
    float *smS = lgnSm + (size_t)mx * kCta + threadIdx.x;
    int *smI = reinterpret_cast<int *>(lgnSm + (size_t)2 * mx * kCta) + threadIdx.x;
    for (int q = 0; q < m; q++) {
        smI[q * kCta] = __ldg(P.lgnId + (size_t)q * P.nV1 + i);
        smW[q * kCta] = __ldg(P.sLGN + (size_t)q * P.nV1 + i);
    }
    // ring slots kept incrementally (t mod lgnSlots, t mod farDepth)
    int lgnSlot = (int)(t0 % lgnSlots);
    int fsT = far_ring_slot(P, t0), fsPrev = far_ring_slot(P, t0 - 1);
    if (active) lgn_words_async(lgnRing + (size_t)lgnSlot * P.lgnN, smI, smS, m);
    // this neuron's outgoing far list (static for the run)
    const int farE0 = (P.farOn && active) ? P.farOff[i] : 0;
    const int farDeg = (P.farOn && active) ? P.farOff[i + 1] - farE0 : 0;
    const int farN1 = (P.farOn && active) ? P.farN1[i] : 0;
    const bool isFarPre = P.farOn && active && P.farPre[i];
    for (int s = 0; s < K; s++) {
        const long long t = t0 + s;
        const unsigned long long farSize = P.farOn ? far_list_size(P, t - 1) : 0ull;
        if (s > 0 || deliverFirst) deliver_prev<Rng>(P, t - 1, b, local, i, active, itype, st, condState, sm, fsPrev);
        const int lgnNext = lgnSlot + 1 == lgnSlots ? 0 : lgnSlot + 1;
        float sInfo = 0.f;
        if (active) {
            const float *lgnSInfo = lgnRing + (size_t)lgnSlot * P.lgnN;
            lgn_words_wait();
            sInfo = step_neuron<Rng, false, true>(P, t, i, itype, tonic, depC, m, nullptr, lgnSInfo, st, condState,
                                                  noisyState, nullptr, smW, smS);
            if (P.spikeCount && sInfo >= 1.0f) P.spikeCount[i] += (unsigned)floorf(sInfo);
            if (sInfo >= 1.0f) prefetch_spiker(P, b, local, farE0, farDeg);
        }
        if (P.farOn) {
            far_push_range(P, t - 1, sm, blockIdx.x, nNeuron, farSize, pushShare, (int)(farSize & 0xffffffffu),
                           fsPrev);
            far_phase(P, t, i, active, sInfo, isFarPre, farE0, farDeg, farN1, sm, blockIdx.x, fsT);
        }
        fsPrev = fsT;
        if (++fsT == P.farDepth) fsT = 0;
        if (s + 1 < K) {
            barrier_arrive(barrier, &s_arrived);
            // the next step's LGN rows are complete before the launch: their copies run while
            // this CTA waits at the barrier
            if (active) lgn_words_async(lgnRing + (size_t)lgnNext * P.lgnN, smI, smS, m);
            if (!barrier_wait(barrier, (unsigned)gridDim.x * (unsigned)(s + 1), &s_arrived, P.err, P.waitSpins))
                break;
        }
        lgnSlot = lgnNext;
    }
    lgn_words_wait();
    if (active) {
        store_state(P, i, st);
        if (Rng && P.condRng) P.rGenCond[i] = condState;
        if (Rng && P.noiseRng) P.rNoisy[i] = noisyState;
    }
}

// rand_spInit (src/coredynamics.cu:5-146) for a network without initial spikes: seeds the
// two per-neuron generators and consumes the uniforms the reference draws while it fills
// the spike history (one, then one per older slot).
__global__ void v1_rng_init_kernel(curandStateMRG32k3a *cond, curandStateMRG32k3a *noisy,
                                   unsigned long long seed, int nV1, int trainDepth) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nV1) return;
    curandStateMRG32k3a a, b;
    curand_init(seed, id, 0, &a);
    curand_init(seed, (unsigned long long)nV1 + id, 0, &b);
    (void)curand_uniform(&a);
    for (int q = trainDepth - 1; q > 0; q--) (void)curand_uniform(&a);
    cond[id] = a;
    noisy[id] = b;
}

// ---- initial spikes (spE0/spI0 > 0) ----
// rand_spInit (src/coredynamics.cu:5-146) with initial spikes, one CTA per block of neurons:
// neuron id spikes with chance sp0[type][nLGN > SCsplit ? 0 : 1] at a uniform time tsp of the
// step before the first (v = vR, tBack and the AdEx w advanced over the rest of that step),
// then the history slots depth-1 .. 1 of the spike-word ring are filled with spikes of the
// same chance outside the refractory period.  H [depth][nV1] receives the spike words (slot 0:
// the initial ones).  ogTab/ohTab [nblock][nE*ngE + nI*ngI] receive output_g/h of the initial
// spikers as the reference writes them for the step's compacted spiker list (E then I, each
// numbered within its block); the reference numbers them in the order its atomicAdd_block
// calls return, which the hardware does not fix, and this kernel numbers them by thread index.
__global__ void __launch_bounds__(1024) v1_sp_init_kernel(V1Params P, unsigned long long seed, int depth, Sp0 sp0,
                                                          int SCsplit, float *H, float *ogTab, float *ohTab,
                                                          float *recU, unsigned *recNU) {
    __shared__ int sCnt[2][32];
    const int bs = P.blockSize, nV1 = P.nV1;
    const int b = blockIdx.x, local = threadIdx.x;
    const bool active = local < bs;
    const int id = b * bs + (active ? local : 0);
    const int itype = type_of(P, active ? local : 0);
    const float dt = P.dt;
    float sInfo = -1.f;
    if (active) {
        curandStateMRG32k3a a, nz;
        curand_init(seed, id, 0, &a);
        curand_init(seed, (unsigned long long)nV1 + id, 0, &nz);
        float *ru = recU ? recU + (size_t)id * 2 * depth : nullptr;
        int nu = 0;
        auto draw = [&]() {
            const float u = curand_uniform(&a);
            if (ru) ru[nu] = u;
            nu++;
            return u;
        };
        const float r0 = draw();
        const float chance = sp0.c[itype * 2 + (P.nLGNperV1[id] > SCsplit ? 0 : 1)];
        const float tRef = P.tRef[itype];
        float v = P.v[id];
        float ref = 0.f;
        sInfo = v;
        if (chance > 0 && r0 < chance) {
            const float tsp = draw();
            sInfo = 1.0f + tsp;
            const float tb = tRef - (1 - tsp) * dt;
            if (tb > 0) P.tBack[id] = tb;
            const float v0 = P.vR[itype];
            v = v0;
            P.v[id] = v0;
            if (P.iModel == 1) {
                const float tw = P.tau_w[itype];
                const float A = P.a[itype] * (v0 - P.vL) * tw;
                const float w0 = P.w[id] + P.b[itype];
                P.w[id] = (w0 - A) * expf(-dt * (1 - tsp) / tw) + A;
            }
            ref = (1 - tsp) * dt + tRef - dt;
        }
        H[id] = sInfo;
        for (int q = depth - 1; q > 0; q--) {
            float word;
            if (ref < dt) {
                if (ref < 0) ref = 0;
                if (draw() < chance * (dt - ref) / dt) {
                    const float tsp = draw() * (dt - ref) / dt;
                    word = 1.0f + tsp;
                    ref = tRef + (1 - tsp) * dt;
                } else {
                    word = v;
                }
            } else {
                word = P.vR[itype];
            }
            H[(size_t)q * nV1 + id] = word;
            ref -= dt;
        }
        P.rGenCond[id] = a;
        P.rNoisy[id] = nz;
        if (recNU) recNU[id] = (unsigned)nu;
    }
    if (!ogTab) return;
    // block-wide numbering of the initial E and I spikers in thread order
    const bool isE = local < P.nE;
    const bool spk = active && sInfo >= 1.0f;
    const int lane = local & 31, warp = local >> 5, nw = (blockDim.x + 31) >> 5;
    const unsigned bE = __ballot_sync(0xffffffffu, spk && isE);
    const unsigned bI = __ballot_sync(0xffffffffu, spk && !isE);
    if (lane == 0) {
        sCnt[0][warp] = __popc(bE);
        sCnt[1][warp] = __popc(bI);
    }
    __syncthreads();
    int before = 0, nE = 0, nI = 0;
    for (int w2 = 0; w2 < nw; w2++) {
        if (w2 < warp) before += isE ? sCnt[0][w2] : sCnt[1][w2];
        nE += sCnt[0][w2];
        nI += sCnt[1][w2];
    }
    if (!spk) return;
    const int sid = before + __popc((isE ? bE : bI) & ((1u << lane) - 1u));
    const size_t base = (size_t)b * (P.nE * P.ngE + P.nI * P.ngI);
    const float tsp = (sInfo - 1) * dt;
    const int ng = isE ? P.ngE : P.ngI;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        if (ig < ng) {
            float g = 0.f, h = 0.f;
            if (isE) cond_input_v(P.condE.rise[ig], P.condE.decay[ig], P.condE.dod[ig], g, h, 1.f, dt - tsp);
            else cond_input_v(P.condI.rise[ig], P.condI.decay[ig], P.condI.dod[ig], g, h, 1.f, dt - tsp);
            const size_t r = isE ? (size_t)ig * nE + sid : (size_t)ig * nI + (size_t)nE * P.ngE + sid;
            ogTab[base + r] = g;
            ohTab[base + r] = h;
        }
    }
}

// The near delivery that runs once before the first step when there are initial spikes
// (noDelay = 1): recal_G_mat_nd (src/coredynamics.cu:2366-2608) as src/patch.cu:5750-5758
// launches it, on the history slot depth-1 of the spike-word ring, reading output_g/h at
// the per-neuron offsets (block, E: i*ngE, I: nE*ngE + (i-nE)*ngI) of the table that
// v1_sp_init_kernel wrote in the compacted layout; the sums are added to gE/hE/gI/hI.
__global__ void __launch_bounds__(1024) v1_sp_near_kernel(V1Params P, const float *Hlast, const float *ogTab,
                                                          const float *ohTab, float *recZ, unsigned *recNZ,
                                                          int cap) {
    const int bs = P.blockSize, nV1 = P.nV1;
    const int b = blockIdx.x, local = threadIdx.x;
    if (local >= bs) return;
    const int ipost = b * bs + local;
    const int itype = type_of(P, local);
    const int ngE = P.ngE, ngI = P.ngI;
    const int ncb = P.nE * ngE + P.nI * ngI;
    float lgE[kMaxNG], lhE[kMaxNG], lgI[kMaxNG], lhI[kMaxNG], ipE[kMaxNG], ipI[kMaxNG];
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        lgE[ig] = lhE[ig] = lgI[ig] = lhI[ig] = 0.f;
        ipE[ig] = ig < ngE ? P.pE[itype * ngE + ig] : 0.f;
        ipI[ig] = ig < ngI ? P.pI[itype * ngI + ig] : 0.f;
    }
    curandStateMRG32k3a cs = P.rGenCond[ipost];
    int nz = 0;
    for (int ib = 0; ib < P.nNearNB[b]; ib++) {
        const int bid = P.nbId[b * P.nnbMax + ib];
        const float *col = P.conMat + ((size_t)(b * P.nnbMax + ib) * bs) * bs + local;
        for (int i = 0; i < bs; i++) {
            float strength = col[(size_t)i * bs];
            if (!(strength != 0 && Hlast[(size_t)bid * bs + i] > 0)) continue;
            const int jtype = type_of(P, i);
            const float p = P.synFail[jtype * P.nType + itype];
            if (p > 0) {
                const float normed_std = sqrtf(p * (1 - p) / P.synPerCon[jtype * P.nType + itype]);
                const float rnd = curand_normal(&cs);
                if (recZ) {
                    if (nz < cap) recZ[(size_t)ipost * cap + nz] = rnd;
                    else atomicOr(P.err, kErrRecordOverflow);
                }
                nz++;
                strength *= 1 - p + normed_std * rnd;
            }
            if (strength > 0) {
                const bool isE = i < P.nE;
                const size_t base = (size_t)bid * ncb + (isE ? (size_t)i * ngE : (size_t)P.nE * ngE + (size_t)(i - P.nE) * ngI);
#pragma unroll
                for (int ig = 0; ig < kMaxNG; ig++) {
                    if (isE && ig < ngE) {
                        const float str = strength * ipE[ig];
                        lgE[ig] += str * ogTab[base + ig];
                        lhE[ig] += str * ohTab[base + ig];
                    }
                    if (!isE && ig < ngI) {
                        const float str = strength * ipI[ig];
                        lgI[ig] += str * ogTab[base + ig];
                        lhI[ig] += str * ohTab[base + ig];
                    }
                }
            }
        }
    }
    P.rGenCond[ipost] = cs;
    if (recNZ) recNZ[ipost] = (unsigned)nz;
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        if (ig < ngE) { P.gE[(size_t)ig * nV1 + ipost] += lgE[ig]; P.hE[(size_t)ig * nV1 + ipost] += lhE[ig]; }
        if (ig < ngI) { P.gI[(size_t)ig * nV1 + ipost] += lgI[ig]; P.hI[(size_t)ig * nV1 + ipost] += lhI[ig]; }
    }
}

// Delayed events of the history, one thread per presynaptic neuron.  Far synapses
// (fill_fSpikeTrain before the loop, src/patch.cu:5806-5846) see the history slot depth-1 as
// step -1: its events arriving in step -1 go to ring slot farDepth-1 (delivered before the
// first step), and the neuron joins step -1's far spiker list, from which step 0 pushes the
// later arrivals.  Delayed near synapses (noDelay = 0) follow recal_G_mat's reads of the
// ring: before the loop (current slot 0, src/patch.cu:5760-5770) slot 0 is step -1 and slot
// s >= 1 step s-depth-1, and only arrivals in step -1 count; in the loop slot s is step
// s-depth until it is overwritten, so slots 1 .. depth-2 push their arrivals in steps >= 0
// here (slot depth-1's come from step -1's list as above).
__global__ void v1_sp_push_kernel(V1Params P, const float *H, int depth) {
    const int nV1 = P.nV1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV1) return;
    const float sLast = H[(size_t)(depth - 1) * nV1 + i];
    const int e0 = P.farOff[i], deg = P.farOff[i + 1] - e0;
    if (sLast > 1.0f && P.farPre[i]) P.farFlag[2] = 1;
    if (sLast >= 1.0f && deg > 0) {
        const int pos = (int)(atomicAdd(P.farCount + 2, (1ull << 32) | (unsigned)deg) >> 32);
        P.farList[(size_t)2 * nV1 + pos] = make_int4(i, e0, deg, __float_as_int(sLast));
    }
    for (int e = e0; e < e0 + deg; e++) {
        const int post = P.farPost[e];
        const float f = P.farStr[e];
        const int sp = P.farSteps[e];
        const float frac = P.farFrac[e];
        const int steps = sp & 0xffff;
        if (!((sp >> 24) & 1)) {
            if (sLast >= 1.0f && steps <= 1) far_event(P, -1, far_ring_slot(P, -1), i, sLast, post, f, steps, sp, frac, steps);
            continue;
        }
        for (int q = 0; q < depth; q++) {
            const float w = H[(size_t)q * nV1 + i];
            if (w < 1.0f) continue;
            const long long th = q == 0 ? -1 : (long long)q - depth - 1;
            const long long k = th + steps + 1;
            if (k == 0 || k == 1) far_event(P, th, far_ring_slot(P, th), i, w, post, f, steps, sp, frac, (int)k);
        }
        for (int q = 1; q < depth - 1; q++) {
            const float w = H[(size_t)q * nV1 + i];
            if (w < 1.0f) continue;
            const long long th = (long long)q - depth;
            for (int k = 0; k < 2; k++)
                if (k <= steps && th + steps - k >= 0) far_event(P, th, far_ring_slot(P, th), i, w, post, f, steps, sp, frac, k);
        }
    }
}

// Adds ring slot farDepth-1 (arrivals in step -1) to the conductances and clears it: delayed
// near events as recal_G_mat adds them, then the far events as sum_G does when some far
// presynaptic neuron spiked in step -1 (src/patch.cu:5806-5846).
__global__ void v1_sp_consume_kernel(V1Params P) {
    const int nV1 = P.nV1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV1) return;
    const int ngE = P.ngE, ns = P.ngE + P.ngI;
    const size_t slot = (size_t)(P.farDepth - 1) * ns * 2 * nV1;
    for (int pass = 0; pass < 2; pass++) {
        unsigned long long *acc = pass == 0 ? (P.nearOn ? P.nearAcc : nullptr) : (P.farClass ? P.farAcc : nullptr);
        if (!acc) continue;
        const bool add = pass == 0 || P.farFlag[2] != 0;
        acc += slot;
        for (int q = 0; q < ns; q++) {
            unsigned long long *pg = acc + (size_t)(2 * q) * nV1 + i;
            unsigned long long *ph = acc + (size_t)(2 * q + 1) * nV1 + i;
            const unsigned long long ug = *pg, uh = *ph;
            *pg = 0ull;
            *ph = 0ull;
            if (!add) continue;
            const float fg = far_from_fixed(ug), fh = far_from_fixed(uh);
            if (q < ngE) {
                P.gE[(size_t)q * nV1 + i] += fg;
                P.hE[(size_t)q * nV1 + i] += fh;
            } else {
                P.gI[(size_t)(q - ngE) * nV1 + i] += fg;
                P.hI[(size_t)(q - ngE) * nV1 + i] += fh;
            }
        }
    }
}

__global__ void advance_step_kernel(long long *stepBase, int k) { *stepBase += k; }

// Full-step decay factors, evaluated with the same expressions as cond_decay (one thread).
__global__ void step_decay_kernel(Cond cFF, Cond cE, Cond cI, float dt, StepDecay *out) {
    if (threadIdx.x != 0) return;
    const Cond *cs[3] = {&cFF, &cE, &cI};
    for (int k = 0; k < 3; k++) {
        for (int ig = 0; ig < kMaxNG; ig++) {
            out[k].etr[ig] = expf(-dt / cs[k]->rise[ig]);
            out[k].etd[ig] = expf(-dt / cs[k]->decay[ig]);
        }
    }
}

cudaError_t compute_step_decay(V1Params &p, cudaStream_t st) {
    StepDecay *d = nullptr;
    cudaError_t e = cudaMalloc(&d, 3 * sizeof(StepDecay));
    if (e != cudaSuccess) return e;
    step_decay_kernel<<<1, 32, 0, st>>>(p.condFF, p.condE, p.condI, p.dt, d);
    StepDecay h[3];
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) return e;
    p.decFF = h[0];
    p.decE = h[1];
    p.decI = h[2];
    return cudaSuccess;
}

// The random-number paths are needed when a draw can change a result (the draws are then
// also recorded when recording is on).
static bool needs_rng(const V1Params &p) { return p.condRng || p.noiseRng; }

cudaError_t launch_v1_step(const V1Params &p, const long long *stepBase, int stepOffset,
                           const float *lgnSInfo, int lgnSlots, int deliverPrev, int doStep,
                           cudaStream_t st) {
    const int nq = (p.blockSize + kCta - 1) / kCta;
    if (needs_rng(p))
        v1_step_kernel<true><<<p.nblock * nq, kCta, 0, st>>>(p, stepBase, stepOffset, lgnSInfo, lgnSlots,
                                                             deliverPrev, doStep);
    else
        v1_step_kernel<false><<<p.nblock * nq, kCta, 0, st>>>(p, stepBase, stepOffset, lgnSInfo, lgnSlots,
                                                              deliverPrev, doStep);
    return cudaGetLastError();
}

// Number of CTAs of the persistent kernel and whether they can all be resident at once.
// Dynamic shared memory of the persistent kernel: weights, spike words and ids of up to maxLGN
// LGN synapses per thread.
static size_t v1_persistent_smem(const V1Params &p) {
    return (size_t)3 * std::max(p.maxLGN, 1) * kCta * sizeof(float);
}

int v1_persistent_ctas(const V1Params &p, int device, bool *fits, int *pushCtas) {
    const int nq = (p.blockSize + kCta - 1) / kCta;
    const int n = p.nblock * nq;
    *pushCtas = 0;
    int perSM = 0, sms = 0;
    const int maxDyn = (int)((size_t)3 * kMaxLgnReg * kCta * sizeof(float));
    cudaFuncSetAttribute(v1_persistent_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxDyn);
    cudaFuncSetAttribute(v1_persistent_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxDyn);
    const size_t dyn = v1_persistent_smem(p);
    if (needs_rng(p))
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, v1_persistent_kernel<true>, kCta, dyn);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, v1_persistent_kernel<false>, kCta, dyn);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    *fits = coop && perSM > 0 && n <= perSM * sms && p.maxLGN <= kMaxLgnReg;
    // far-push CTAs on the SMs the neuron CTAs leave free (at most a quarter of the neuron
    // CTAs, at least 8 when that many are free: each one more CTA at every grid barrier)
    if (*fits && p.farOn) *pushCtas = std::min(perSM * sms - n, std::max(8, n / 4));
    return n;
}

cudaError_t launch_v1_persistent(const V1Params &p, const long long *stepBase, int K, const float *lgnRing,
                                 int lgnSlots, int deliverFirst, unsigned *barrier, cudaStream_t st) {
    const int nq = (p.blockSize + kCta - 1) / kCta;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.nblock * nq + p.pushCta);
    cfg.blockDim = dim3(kCta);
    cfg.dynamicSmemBytes = v1_persistent_smem(p);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaMemsetAsync(barrier, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (needs_rng(p))
        return cudaLaunchKernelEx(&cfg, v1_persistent_kernel<true>, p, stepBase, K, lgnRing, lgnSlots,
                                  deliverFirst, barrier);
    return cudaLaunchKernelEx(&cfg, v1_persistent_kernel<false>, p, stepBase, K, lgnRing, lgnSlots,
                              deliverFirst, barrier);
}

cudaError_t launch_v1_rng_init(curandStateMRG32k3a *cond, curandStateMRG32k3a *noisy,
                               unsigned long long seed, int nV1, int trainDepth, cudaStream_t st) {
    v1_rng_init_kernel<<<(nV1 + 127) / 128, 128, 0, st>>>(cond, noisy, seed, nV1, trainDepth);
    return cudaGetLastError();
}

cudaError_t launch_v1_sp_init(const V1Params &p, unsigned long long seed, int depth, const Sp0 &sp0, int SCsplit,
                              float *H, float *ogTab, float *ohTab, float *recU, unsigned *recNU, cudaStream_t st) {
    const int threads = (p.blockSize + 31) / 32 * 32;
    v1_sp_init_kernel<<<p.nblock, threads, 0, st>>>(p, seed, depth, sp0, SCsplit, H, ogTab, ohTab, recU, recNU);
    return cudaGetLastError();
}

cudaError_t launch_v1_sp_near(const V1Params &p, const float *Hlast, const float *ogTab, const float *ohTab,
                              float *recZ, unsigned *recNZ, int cap, cudaStream_t st) {
    const int threads = (p.blockSize + 31) / 32 * 32;
    v1_sp_near_kernel<<<p.nblock, threads, 0, st>>>(p, Hlast, ogTab, ohTab, recZ, recNZ, cap);
    return cudaGetLastError();
}

cudaError_t launch_v1_sp_events(const V1Params &p, const float *H, int depth, cudaStream_t st) {
    const int n = (p.nV1 + 255) / 256;
    v1_sp_push_kernel<<<n, 256, 0, st>>>(p, H, depth);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    v1_sp_consume_kernel<<<n, 256, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_advance_step(long long *stepBase, int k, cudaStream_t st) {
    advance_step_kernel<<<1, 1, 0, st>>>(stepBase, k);
    return cudaGetLastError();
}

// ---- batched trials ----
// One step of every active (trial, CTA) tile of a batch.  Each CTA copies its trial's
// parameter block to shared memory and runs the same step body as the per-step kernel with
// the trial's own CTA index and count, so each trial computes exactly what it would alone.
// Finished trials have no tiles in the list (the host rebuilds it between chunks); a tile
// whose trial ends inside the chunk returns at its last step.
template <bool Rng, int MinB>
__global__ void __launch_bounds__(kCta, MinB) v1_batch_step_kernel(const BatchTrial *__restrict__ trials,
                                                                   const int2 *__restrict__ tiles,
                                                                   const int *__restrict__ nTiles,
                                                                   int stepOffset) {
    __shared__ Smem sm;
    __shared__ __align__(16) BatchTrial sT;
    if ((int)blockIdx.x >= *nTiles) return;
    const int2 tile = tiles[blockIdx.x];
    const int *src = reinterpret_cast<const int *>(trials + tile.x);
    int *dst = reinterpret_cast<int *>(&sT);
    for (int w = threadIdx.x; w < (int)(sizeof(BatchTrial) / sizeof(int)); w += kCta) dst[w] = src[w];
    __syncthreads();
    const long long t = *sT.step + stepOffset;
    if (t >= sT.tEnd) return;
    v1_step_body<Rng>(sT.v, t, tile.y, sT.nCta, sT.lgnRing, sT.lgnSlots, t >= sT.tDeliverFrom ? 1 : 0, 1, sm);
}

// Batched trials in one cooperative launch per chunk: the grid is split into slots of
// slotCtas CTAs (the largest trial's CTA count); slot s runs active trials s, s + nSlots, ...
// one after the other, each for its steps of the chunk, with the trial's state in registers
// and a barrier among the trial's own CTAs between steps (no grid-wide barrier: trials are
// independent).  The step is the per-step kernels' (same delivery order, same arithmetic), so
// every trial computes what the per-step batch and pv1_run compute for it.
template <bool Rng>
__device__ __forceinline__ void batch_trial_steps(const V1Params &P, long long t0, int steps, int cta, int nCta,
                                                  const float *__restrict__ lgnRing, int lgnSlots, bool deliverFirst,
                                                  unsigned *barrier, Smem &sm, unsigned *s_arrived,
                                                  float *dyn) {
    const int bs = P.blockSize;
    const int nq = (bs + kCta - 1) / kCta;
    const int b = cta / nq;
    const int local = (cta % nq) * kCta + threadIdx.x;
    const bool active = local < bs;
    const int i = b * bs + (active ? local : 0);
    const int itype = type_of(P, active ? local : 0);
    NState st;
    load_state(P, i, st);
    curandStateMRG32k3a condState, noisyState;
    if (Rng && P.condRng && active) condState = P.rGenCond[i];
    if (Rng && P.noiseRng && active) noisyState = P.rNoisy[i];
    const float tonic = active ? P.tonicDep[i] : 0.f;
    const float depC = tonic_current(P, itype, tonic);
    const int m = active ? P.nLGNperV1[i] : 0;
    const int farE0 = (P.farOn && active) ? P.farOff[i] : 0;
    const int farDeg = (P.farOn && active) ? P.farOff[i + 1] - farE0 : 0;
    const int farN1 = (P.farOn && active) ? P.farN1[i] : 0;
    const bool isFarPre = P.farOn && active && P.farPre[i];
    // short LGN lists: ids, weights and the step's spike words in shared memory ([synapse][kCta]
    // from the thread's column), the next step's words copied in while the trial's CTAs meet at
    // the barrier -- as the single-patch persistent kernel does
    const bool smemSyn = dyn && P.maxLGN <= kBatchLgn && !P.multiSpike;
    float *smW = dyn + threadIdx.x;
    float *smS = dyn + (size_t)kBatchLgn * kCta + threadIdx.x;
    int *smI = reinterpret_cast<int *>(dyn + (size_t)2 * kBatchLgn * kCta) + threadIdx.x;
    // ring slots kept incrementally (t mod lgnSlots, t mod farDepth)
    int lgnSlot = (int)(t0 % lgnSlots);
    int fsT = P.farOn ? far_ring_slot(P, t0) : 0, fsPrev = P.farOn ? far_ring_slot(P, t0 - 1) : 0;
    if (smemSyn) {
        for (int q = 0; q < m; q++) {
            smI[q * kCta] = __ldg(P.lgnId + (size_t)q * P.nV1 + i);
            smW[q * kCta] = __ldg(P.sLGN + (size_t)q * P.nV1 + i);
        }
        if (active) lgn_words_async(lgnRing + (size_t)lgnSlot * P.lgnN, smI, smS, m);
    }
    for (int s = 0; s < steps; s++) {
        const long long t = t0 + s;
        if (s > 0 || deliverFirst)
            deliver_prev<Rng>(P, t - 1, b, local, i, active, itype, st, condState, sm, P.farOn ? fsPrev : -1);
        const int lgnNext = lgnSlot + 1 == lgnSlots ? 0 : lgnSlot + 1;
        float sInfo = 0.f;
        if (active) {
            const float *lgnSInfo = lgnRing + (size_t)lgnSlot * P.lgnN;
            if (P.multiSpike) {
                sInfo = step_neuron_multi<Rng>(P, t, i, itype, tonic, depC, m, lgnSInfo, st, condState, noisyState);
            } else if (smemSyn) {
                lgn_words_wait();
                sInfo = step_neuron<Rng, false, true>(P, t, i, itype, tonic, depC, m, nullptr, lgnSInfo, st,
                                                      condState, noisyState, nullptr, smW, smS);
            } else {
                sInfo = step_neuron<Rng, false>(P, t, i, itype, tonic, depC, m, nullptr, lgnSInfo, st, condState,
                                                noisyState);
            }
            if (P.spikeCount && sInfo >= 1.0f) P.spikeCount[i] += (unsigned)floorf(sInfo);
        }
        if (P.farOn) {
            far_push_list(P, t - 1, sm, cta, nCta, fsPrev);
            far_phase(P, t, i, active, sInfo, isFarPre, farE0, farDeg, farN1, sm, cta, fsT);
            fsPrev = fsT;
            if (++fsT == P.farDepth) fsT = 0;
        }
        if (s + 1 < steps) {
            barrier_arrive(barrier, s_arrived);
            if (smemSyn && active) lgn_words_async(lgnRing + (size_t)lgnNext * P.lgnN, smI, smS, m);
            if (!barrier_wait(barrier, (unsigned)nCta * (unsigned)(s + 1), s_arrived, P.err, P.waitSpins)) break;
        }
        lgnSlot = lgnNext;
    }
    if (smemSyn) lgn_words_wait();
    if (active) {
        store_state(P, i, st);
        if (Rng && P.condRng) P.rGenCond[i] = condState;
        if (Rng && P.noiseRng) P.rNoisy[i] = noisyState;
    }
}

template <bool Rng>
__global__ void __launch_bounds__(kCta, 2) v1_batch_persistent_kernel(const BatchTrial *__restrict__ trials,
                                                                     const int *__restrict__ activeList,
                                                                     const int *__restrict__ nActive, int slotCtas,
                                                                     int nSlots, int K, unsigned *barriers) {
    __shared__ Smem sm;
    __shared__ __align__(16) BatchTrial sT;
    __shared__ unsigned s_arrived;
    extern __shared__ __align__(16) float dyn[];   // LGN synapses: weights, words, ids [kBatchLgn][kCta] each
    const int slot = blockIdx.x / slotCtas, c = blockIdx.x % slotCtas;
    const int na = *nActive;
    for (int j = slot; j < na; j += nSlots) {
        const int q = activeList[j];
        if (q < 0) continue;  // a slot's schedule ended (one-launch sweep)
        __syncthreads();
        const int *src = reinterpret_cast<const int *>(trials + q);
        int *dst = reinterpret_cast<int *>(&sT);
        for (int w = threadIdx.x; w < (int)(sizeof(BatchTrial) / sizeof(int)); w += kCta) dst[w] = src[w];
        __syncthreads();
        if (c >= sT.nCta) continue;
        const long long t0 = *sT.step;
        const long long left = sT.tEnd - t0;
        const int steps = left < K ? (int)left : K;
        if (steps <= 0) continue;
        batch_trial_steps<Rng>(sT.v, t0, steps, c, sT.nCta, sT.lgnRing, sT.lgnSlots, t0 >= sT.tDeliverFrom,
                               barriers + q, sm, &s_arrived, dyn);
    }
}

// The kernel's shared memory (Smem, the trial block and 72 KB of LGN synapses) passes the
// 48 KB a block gets without opting in; two blocks still fit an SM.
constexpr size_t kBatchDyn = (size_t)3 * kBatchLgn * kCta * sizeof(float);
static cudaError_t batch_persistent_smem_optin() {
    static cudaError_t done = cudaErrorNotReady;
    if (done == cudaErrorNotReady) {
        const int dyn = (int)kBatchDyn;
        done = cudaFuncSetAttribute(v1_batch_persistent_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
        if (done == cudaSuccess)
            done = cudaFuncSetAttribute(v1_batch_persistent_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        dyn);
    }
    return done;
}

int v1_batch_persistent_capacity(bool rng, int device) {
    int perSM = 0, sms = 0;
    if (batch_persistent_smem_optin() != cudaSuccess) return 0;
    const size_t dyn = kBatchDyn;
    cudaError_t e = rng ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, v1_batch_persistent_kernel<true>, kCta, dyn)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, v1_batch_persistent_kernel<false>, kCta, dyn);
    if (e != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    return perSM * sms;
}

cudaError_t launch_v1_batch_persistent(const BatchTrial *trials, const int *activeList, const int *nActive,
                                       int slotCtas, int nSlots, int K, unsigned *barriers, int nTrials, bool rng,
                                       cudaStream_t st) {
    if (nSlots <= 0 || slotCtas <= 0) return cudaErrorInvalidValue;
    cudaError_t e = batch_persistent_smem_optin();
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(barriers, 0, (size_t)nTrials * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nSlots * slotCtas);
    cfg.blockDim = dim3(kCta);
    cfg.dynamicSmemBytes = kBatchDyn;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (rng)
        return cudaLaunchKernelEx(&cfg, v1_batch_persistent_kernel<true>, trials, activeList, nActive, slotCtas,
                                  nSlots, K, barriers);
    return cudaLaunchKernelEx(&cfg, v1_batch_persistent_kernel<false>, trials, activeList, nActive, slotCtas, nSlots,
                              K, barriers);
}

template <bool Rng>
static cudaError_t launch_batch_variant(int minB, const BatchTrial *trials, const int2 *tiles,
                                        const int *nTiles, int grid, int stepOffset, cudaStream_t st) {
    switch (minB) {
    case 1: v1_batch_step_kernel<Rng, 1><<<grid, kCta, 0, st>>>(trials, tiles, nTiles, stepOffset); break;
    case 2: v1_batch_step_kernel<Rng, 2><<<grid, kCta, 0, st>>>(trials, tiles, nTiles, stepOffset); break;
    case 3: v1_batch_step_kernel<Rng, 3><<<grid, kCta, 0, st>>>(trials, tiles, nTiles, stepOffset); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_v1_batch_step(const BatchTrial *trials, const int2 *tiles, const int *nTiles,
                                 int gridTiles, int stepOffset, bool rng, int minB, cudaStream_t st) {
    if (gridTiles <= 0) return cudaSuccess;
    return rng ? launch_batch_variant<true>(minB, trials, tiles, nTiles, gridTiles, stepOffset, st)
               : launch_batch_variant<false>(minB, trials, tiles, nTiles, gridTiles, stepOffset, st);
}

int v1_batch_regs(int minB, bool rng) {
    cudaFuncAttributes a{};
    cudaError_t e = cudaErrorInvalidValue;
    if (rng) {
        if (minB == 1) e = cudaFuncGetAttributes(&a, v1_batch_step_kernel<true, 1>);
        if (minB == 2) e = cudaFuncGetAttributes(&a, v1_batch_step_kernel<true, 2>);
        if (minB == 3) e = cudaFuncGetAttributes(&a, v1_batch_step_kernel<true, 3>);
    } else {
        if (minB == 1) e = cudaFuncGetAttributes(&a, v1_batch_step_kernel<false, 1>);
        if (minB == 2) e = cudaFuncGetAttributes(&a, v1_batch_step_kernel<false, 2>);
        if (minB == 3) e = cudaFuncGetAttributes(&a, v1_batch_step_kernel<false, 3>);
    }
    return e == cudaSuccess ? a.numRegs : -1;
}

// Per trial: step += the steps it ran in the chunk (K, or fewer at its end), and its FP64
// simulated-time accumulator += those steps * dt.
__global__ void batch_advance_kernel(BatchTrial *trials, int nTrials, int K, double *simTime) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nTrials) return;
    const long long s = *trials[q].step;
    long long k = trials[q].tEnd - s;
    k = k < 0 ? 0 : (k > K ? K : k);
    *trials[q].step = s + k;
    simTime[q] += (double)k * trials[q].dt;
}

cudaError_t launch_batch_advance(BatchTrial *trials, int nTrials, int K, double *simTime, cudaStream_t st) {
    batch_advance_kernel<<<(nTrials + 127) / 128, 128, 0, st>>>(trials, nTrials, K, simTime);
    return cudaGetLastError();
}

// FP64 firing rates of one trial: rate[i] = count[i] / simulated seconds, and the mean over
// its neurons (one CTA, double-precision tree reduction).
__global__ void __launch_bounds__(1024) batch_rates_kernel(const unsigned *counts, int nV1, const double *simTime,
                                                           double *rates, double *meanRate) {
    __shared__ double red[32];
    const double sec = *simTime * 1e-3;
    double acc = 0.0;
    for (int i = threadIdx.x; i < nV1; i += blockDim.x) {
        const double r = sec > 0 ? (double)counts[i] / sec : 0.0;
        if (rates) rates[i] = r;
        acc += r;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) *meanRate = acc / (double)nV1;
    }
}

cudaError_t launch_batch_rates(const BatchTrial *, const unsigned *counts, const long long *countOff,
                               const double *simTime, int trial, int nV1, double *rates, double *meanRate,
                               cudaStream_t st) {
    batch_rates_kernel<<<1, 1024, 0, st>>>(counts + countOff[trial], nV1, simTime + trial, rates, meanRate);
    return cudaGetLastError();
}

}  // namespace pv1
