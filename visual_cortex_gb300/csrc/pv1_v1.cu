// V1 stage of the patchV1 hot path on GB300 (sm_103a): one kernel per simulation step.
//
// The reference runs, per step, compute_V_collect_spike_learnFF_fast (src/coredynamics.cu:
// 1235-2059), then recal_G_mat_nd_fast for the near-neighbour blocks (:2609-2922), then a
// single-threaded host loop for the far synapses (recal_G_vec :181-372, fill_fSpikeTrain
// src/stats.cu:114-126) whose result is copied back and added by sum_G (:2312-2349).
//
// Here one launch per step does three phases:
//   A. deliver the previous step's spikes: every CTA compacts the spikers of its neighbour
//      blocks with warp ballots (ascending neuron order, E before I), stages their unit
//      conductance (og/oh) in shared memory and reads one coalesced conMat row per spiker;
//      far events that arrive in the previous step come from a fixed-point ring filled by
//      phase C.  The sum is added to g/h exactly where the reference's delivery adds it.
//   B. the V1 membrane step of this step (conductance decay, LGN input, RK2 AdEx/LIF,
//      spike-time interpolation, refractoriness), same float operation order as the
//      reference's kernel.
//   C. push this step's spikes into the far-delivery ring: one event per (spike, far
//      synapse), with the reference's delay arithmetic deciding the arrival step.
// Adding the previous step's delivery before this step's decay is the same sequence of
// float operations as the reference's separate kernels.
//
// All per-species arrays are indexed with compile-time indices (loops over kMaxNG with a
// runtime guard) so that they live in registers.
#include "pv1_internal.cuh"

namespace pv1 {

constexpr int kCta = 256;
constexpr int kWarps = kCta / 32;
constexpr int kMaxBS = 1024;
constexpr int kLgnBatch = 8;

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

// Compacts the spike words blk[0..n) that are >= 1 into list[] (ascending index) using one
// ballot word per 32 entries.  Returns the count (all threads); *below receives the number
// of listed entries with index < split.  vals[j] keeps the word of every listed j.
__device__ __forceinline__ int compact_spikers(const float *__restrict__ blk, int n, int split,
                                               int *list, float *vals, unsigned *s_ball,
                                               int *below) {
    const int lane = threadIdx.x & 31;
    const int nw = (n + 31) >> 5;
    for (int j0 = threadIdx.x & ~31; j0 < n; j0 += kCta) {
        const int j = j0 + lane;
        const float v = j < n ? blk[j] : 0.f;
        const bool f = j < n && v >= 1.0f;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_ball[j0 >> 5] = bal;
        if (f) vals[j] = v;
    }
    __syncthreads();
    int total = 0, nb = 0;
    for (int w = 0; w < nw; w++) {
        const unsigned bal = s_ball[w];
        const int c = __popc(bal);
        if ((w + 1) * 32 <= split) nb += c;
        else if (w * 32 < split) nb += __popc(bal & ((1u << (split - w * 32)) - 1u));
        total += c;
    }
    if (total > 0) {
        for (int j0 = threadIdx.x & ~31; j0 < n; j0 += kCta) {
            const int w = j0 >> 5;
            const unsigned bal = s_ball[w];
            if ((bal >> lane) & 1u) {
                int pos = __popc(bal & ((1u << lane) - 1u));
                for (int q = 0; q < w; q++) pos += __popc(s_ball[q]);
                list[pos] = j0 + lane;
            }
        }
        __syncthreads();
    }
    *below = nb;
    return total;
}

// Phase C: one event per (spike, far synapse), arrival step and offset as recal_G_vec
// computes them (src/coredynamics.cu:282-333).  The arithmetic deciding the arrival is done
// with explicitly rounded operations, as on the reference's host.
__device__ __forceinline__ void far_push(const V1Params &P, long long t, int i, bool push,
                                         float sInfo, int *s_list, float *s_si, unsigned *s_ball) {
    const int nV1 = P.nV1, bs = P.blockSize;
    const float dt = P.dt;
    const unsigned bal = __ballot_sync(0xffffffffu, push);
    if ((threadIdx.x & 31) == 0) s_ball[threadIdx.x >> 5] = bal;
    __syncthreads();
    int cnt = 0, pos = 0;
    for (int w = 0; w < kWarps; w++) {
        const int c = __popc(s_ball[w]);
        if (w < (int)(threadIdx.x >> 5)) pos += c;
        cnt += c;
    }
    if (push) {
        pos += __popc(bal & ((1u << (threadIdx.x & 31)) - 1u));
        s_list[pos] = i;
        s_si[pos] = sInfo;
    }
    __syncthreads();
    const int ns = P.ngE + P.ngI;
    for (int r = 0; r < cnt; r++) {
        const int pre = s_list[r];
        const float sI = s_si[r];
        const unsigned nsp = (unsigned)floorf(sI);
        const bool preE = (pre % bs) < P.nE;
        const int ng = preE ? P.ngE : P.ngI;
        const int qoff = preE ? 0 : P.ngE;
        const int e1 = P.farOff[pre + 1];
        for (int e = P.farOff[pre] + threadIdx.x; e < e1; e += kCta) {
            const int post = P.farPost[e];
            const float f = P.farStr[e];
            const int steps = P.farSteps[e];
            const float frac = P.farFrac[e];
            const int ptype = type_of(P, post % bs);
#pragma unroll
            for (int kk = 0; kk < 2; kk++) {
                // dtsp = (sInfo - nsp + k)*dt - time2post, rounded step by step
                const float x = __fadd_rn(__fsub_rn(sI, (float)nsp), (float)kk);
                const float dtsp = __fsub_rn(__fmul_rn(x, dt), frac);
                if (dtsp < dt && dtsp >= 0 && f > 0) {
                    const long long tArr = t + steps - kk;
                    if (tArr < t || tArr - t >= P.farDepth - 1) {
                        atomicOr(P.err, kErrFarOverflow);
                        continue;
                    }
                    const float delta = __fsub_rn(dt, dtsp);
                    unsigned long long *acc = P.farAcc + (size_t)(tArr % P.farDepth) * ns * 2 * nV1;
#pragma unroll
                    for (int ig = 0; ig < kMaxNG; ig++) {
                        if (ig < ng) {
                            const float ip = preE ? P.pE[ptype * P.ngE + ig] : P.pI[ptype * P.ngI + ig];
                            const float fv = __fmul_rn(__fmul_rn((float)nsp, f), ip);
                            float g = 0.f, h = 0.f;
                            cond_input(preE ? P.condE : P.condI, g, h, fv, delta, ig);
                            const long long qg = __double2ll_rn((double)g * kFarScale);
                            const long long qh = __double2ll_rn((double)h * kFarScale);
                            atomicAdd(&acc[(size_t)(2 * (qoff + ig)) * nV1 + post], (unsigned long long)qg);
                            atomicAdd(&acc[(size_t)(2 * (qoff + ig) + 1) * nV1 + post], (unsigned long long)qh);
                        }
                    }
                }
            }
        }
    }
}

__global__ void __launch_bounds__(kCta) v1_step_kernel(V1Params P, const long long *stepBase,
                                                       int stepOffset,
                                                       const float *__restrict__ lgnRing,
                                                       int lgnSlots, int deliverPrev,
                                                       int doStep) {
    __shared__ int s_pre[kMaxBS];
    __shared__ float s_val[kMaxBS];
    __shared__ float s_og[kMaxNG][kMaxBS];
    __shared__ float s_oh[kMaxNG][kMaxBS];
    __shared__ unsigned s_ball[kMaxBS / 32];

    const long long t = *stepBase + stepOffset;
    const float *__restrict__ lgnSInfo = lgnRing + (size_t)(t % lgnSlots) * P.lgnN;
    const int bs = P.blockSize;
    const int nq = (bs + kCta - 1) / kCta;
    const int b = blockIdx.x / nq;
    const int local = (blockIdx.x % nq) * kCta + threadIdx.x;
    const bool active = local < bs;
    const int i = b * bs + (active ? local : 0);
    const int itype = type_of(P, active ? local : 0);
    const int nV1 = P.nV1;
    const float dt = P.dt;
    const int ngE = P.ngE, ngI = P.ngI, ngFF = P.ngFF;

    // conductances after delivery of the previous step (registers)
    float gE[kMaxNG], hE[kMaxNG], gI[kMaxNG], hI[kMaxNG];
#pragma unroll
    for (int ig = 0; ig < kMaxNG; ig++) {
        gE[ig] = hE[ig] = gI[ig] = hI[ig] = 0.f;
        if (ig < ngE) { gE[ig] = P.gE[ig * nV1 + i]; hE[ig] = P.hE[ig * nV1 + i]; }
        if (ig < ngI) { gI[ig] = P.gI[ig * nV1 + i]; hI[ig] = P.hI[ig * nV1 + i]; }
    }
    curandStateMRG32k3a condState;
    if (P.condRng && active) condState = P.rGenCond[i];

    // ------------------------------------------------------------------ phase A
    if (deliverPrev) {
        const long long tp = t - 1;
        const float *sPrev = P.sInfo + (size_t)(tp & 1) * nV1;
        float lgE[kMaxNG], lhE[kMaxNG], lgI[kMaxNG], lhI[kMaxNG], ipE[kMaxNG], ipI[kMaxNG];
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            lgE[ig] = lhE[ig] = lgI[ig] = lhI[ig] = 0.f;
            ipE[ig] = ig < ngE ? P.pE[itype * ngE + ig] : 0.f;
            ipI[ig] = ig < ngI ? P.pI[itype * ngI + ig] : 0.f;
        }
        const int nnb = P.nNearNB[b];
        float *recNear = nullptr;
        int nNearDraw = 0;
        if (P.recNear && active) {
            long long rs = tp - P.recStep0;
            if (rs >= 0 && rs < P.recSteps) recNear = P.recNear + ((size_t)rs * nV1 + i) * P.recCap;
        }
        for (int ib = 0; ib < nnb; ib++) {
            const int nb = P.nbId[b * P.nnbMax + ib];
            int cntE;
            const int cnt = compact_spikers(sPrev + (size_t)nb * bs, bs, P.nE, s_pre, s_val, s_ball, &cntE);
            if (cnt == 0) continue;
            // unit conductance of each spiker (output_g/h of compute_V, :2008-2041)
            for (int r = threadIdx.x; r < cnt; r += kCta) {
                const float sI = s_val[s_pre[r]];
                const float nsp = floorf(sI);
                const float tsp = (sI - nsp) * dt;
                const bool isE = r < cntE;
#pragma unroll
                for (int ig = 0; ig < kMaxNG; ig++) {
                    if (ig < (isE ? ngE : ngI)) {
                        float g = 0.f, h = 0.f;
                        cond_input(isE ? P.condE : P.condI, g, h, nsp, dt - tsp, ig);
                        s_og[ig][r] = g;
                        s_oh[ig][r] = h;
                    }
                }
            }
            __syncthreads();
            if (active) {
                const float *col = P.conMat + ((size_t)(b * P.nnbMax + ib) * bs) * bs + local;
                for (int r = 0; r < cnt; r++) {
                    float strength = col[(size_t)s_pre[r] * bs];
                    if (strength > 0) {
                        const bool isE = r < cntE;
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
                        if (strength > 0) {
                            if (isE) {
#pragma unroll
                                for (int ig = 0; ig < kMaxNG; ig++) {
                                    if (ig < ngE) {
                                        const float str = strength * ipE[ig];
                                        lgE[ig] += str * s_og[ig][r];
                                        lhE[ig] += str * s_oh[ig][r];
                                    }
                                }
                            } else {
#pragma unroll
                                for (int ig = 0; ig < kMaxNG; ig++) {
                                    if (ig < ngI) {
                                        const float str = strength * ipI[ig];
                                        lgI[ig] += str * s_og[ig][r];
                                        lhI[ig] += str * s_oh[ig][r];
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
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            gE[ig] += lgE[ig]; hE[ig] += lhE[ig];
            gI[ig] += lgI[ig]; hI[ig] += lhI[ig];
        }
        // far events arriving in step tp (sum_G adds them after the near delivery)
        if (P.farOn && active) {
            const int ns = ngE + ngI;
            unsigned long long *acc = P.farAcc + (size_t)(tp % P.farDepth) * ns * 2 * nV1;
            const bool farSpiked = P.farFlag[tp % 3] != 0;
#pragma unroll
            for (int q = 0; q < 2 * kMaxNG; q++) {
                if (q < ns) {
                    const unsigned long long ug = acc[(size_t)(2 * q) * nV1 + i];
                    const unsigned long long uh = acc[(size_t)(2 * q + 1) * nV1 + i];
                    if (ug | uh) {
                        acc[(size_t)(2 * q) * nV1 + i] = 0ull;
                        acc[(size_t)(2 * q + 1) * nV1 + i] = 0ull;
                    }
                    if (farSpiked) {
                        const float fg = (float)((double)(long long)ug / kFarScale);
                        const float fh = (float)((double)(long long)uh / kFarScale);
#pragma unroll
                        for (int ig = 0; ig < kMaxNG; ig++) {
                            if (q < ngE && ig == q) { gE[ig] += fg; hE[ig] += fh; }
                            if (q >= ngE && ig == q - ngE) { gI[ig] += fg; hI[ig] += fh; }
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
                if (ig < ngE) r[o.gE + ig * nV1 + i] = gE[ig];
                if (ig < ngI) r[o.gI + ig * nV1 + i] = gI[ig];
                if (P.hWrite) {
                    if (ig < ngE) r[o.hE + ig * nV1 + i] = hE[ig];
                    if (ig < ngI) r[o.hI + ig * nV1 + i] = hI[ig];
                }
            }
        }
    }

    if (!doStep) {
        // delivery only (end of a run): store the delivered conductances
        if (active) {
#pragma unroll
            for (int ig = 0; ig < kMaxNG; ig++) {
                if (ig < ngE) { P.gE[ig * nV1 + i] = gE[ig]; P.hE[ig * nV1 + i] = hE[ig]; }
                if (ig < ngI) { P.gI[ig * nV1 + i] = gI[ig]; P.hI[ig * nV1 + i] = hI[ig]; }
            }
            if (P.condRng) P.rGenCond[i] = condState;
        }
        return;
    }

    // ------------------------------------------------------------------ phase B
    float sInfo = 0.f;
    if (active) {
        const float vR = P.vR[itype], vThres = P.vThres[itype], gL = P.gL[itype];
        const float Cm = P.C[itype], tRef = P.tRef[itype], vT = P.vT[itype];
        const float deltaT = P.deltaT[itype], tau_w = P.tau_w[itype], aa = P.a[itype];
        const float bb = P.b[itype];
        const float tonic = P.tonicDep[i];
        float v0 = P.v[i];
        float w0 = P.iModel == 1 ? P.w[i] : 0.0f;
        float tBack = P.tBack[i];
        float g1[kMaxNG], h1[kMaxNG];
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            g1[ig] = ig < ngFF ? P.gFF[ig * nV1 + i] : 0.f;
            h1[ig] = ig < ngFF ? P.hFF[ig * nV1 + i] : 0.f;
        }
        const int m = P.nLGNperV1[i];
        // tonic drive (AdEx constructor, src/coredynamics.cuh:41-49)
        float depC;
        {
            const float targetV = P.vL + (vT - P.vL) * tonic;
            if (targetV > vT) depC = (gL + aa) * (targetV - P.vL) - gL * deltaT;
            else depC = (gL + aa) * (targetV - P.vL) - gL * deltaT * expf((targetV - vT) / deltaT);
        }
        float noise0 = 0.f;
        if (P.tau_noise > 0) noise0 = P.lastNoise[i];

        // cortical conductances: keep the start-of-step value, decay to the end
        float ge[kMaxNG], he[kMaxNG], gi[kMaxNG], hi[kMaxNG];
        float gE_t1 = 0.0f, gI_t1 = 0.0f;
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            ge[ig] = gE[ig]; he[ig] = hE[ig];
            if (ig < ngE) {
                float g = gE[ig], h = hE[ig];
                cond_decay(P.condE, g, h, dt, ig);
                P.gE[ig * nV1 + i] = g;
                P.hE[ig * nV1 + i] = h;
                gE_t1 += g;
            }
        }
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            gi[ig] = gI[ig]; hi[ig] = hI[ig];
            if (ig < ngI) {
                float g = gI[ig], h = hI[ig];
                cond_decay(P.condI, g, h, dt, ig);
                P.gI[ig * nV1 + i] = g;
                P.hI[ig * nV1 + i] = h;
                gI_t1 += g;
            }
        }
        float g0[kMaxNG], h0[kMaxNG];
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            g0[ig] = g1[ig];
            h0[ig] = h1[ig];
            if (ig < ngFF) cond_decay(P.condFF, g1[ig], h1[ig], dt, ig);
        }
        // noise (src/coredynamics.cu:1422-1440)
        const float noiseRatio = P.noiseOnTonic ? tonic : 1.0f;
        float noise1 = sqrtf(2 * P.noisyDep[itype] * (vT - vR) * noiseRatio * dt);
        const float pf = P.synFailFF[itype];
        const float nSynFF = P.synPerConFF[itype];
        if (noise1 > 0) {
            curandStateMRG32k3a ns = P.rNoisy[i];
            const float rnd = curand_normal(&ns);
            P.rNoisy[i] = ns;
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
                P.lastNoise[i] = noise1;
            }
        }
        const bool backingUp = tBack < dt && tBack > 0;
        const float depOut = depC + noise1;
        P.dep[i] = depOut;
        if (backingUp) {
#pragma unroll
            for (int ig = 0; ig < kMaxNG; ig++)
                if (ig < ngFF) cond_decay(P.condFF, g0[ig], h0[ig], tBack, ig);
        }
        // LGN input (src/coredynamics.cu:1466-1502), synapse order kept; the ids and spike
        // words are gathered in batches so that the loads overlap
        float *recFF = nullptr;
        int nFF = 0;
        if (P.recFF) {
            long long rs = t - P.recStep0;
            if (rs >= 0 && rs < P.recSteps) recFF = P.recFF + ((size_t)rs * nV1 + i) * P.recCap;
        }
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
            for (int k = 0; k < kLgnBatch; k++) sp[k] = q0 + k < m ? lgnSInfo[ids[k]] : 0.f;
#pragma unroll
            for (int k = 0; k < kLgnBatch; k++) {
                const float sFF = sp[k];
                const unsigned nspFF = (unsigned)floorf(sFF);
                if (q0 + k < m && nspFF > 0) {
                    float f = fs[k];
                    const float tspFF = (sFF - nspFF) * dt;
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
                    if (f > 0) {
                        const float ddt = backingUp ? tBack - tspFF : 0.f;
#pragma unroll
                        for (int ig = 0; ig < kMaxNG; ig++) {
                            if (ig < ngFF) {
                                const float str = f * P.pFF[itype * ngFF + ig];
                                if (backingUp && ddt > 0) cond_input(P.condFF, g0[ig], h0[ig], str * nspFF, ddt, ig);
                                cond_input(P.condFF, g1[ig], h1[ig], str * nspFF, dt - tspFF, ig);
                            }
                        }
                    }
                }
            }
        }
        if (recFF) P.recFFCount[(size_t)(t - P.recStep0) * nV1 + i] = nFF;
        if (P.condRng) P.rGenCond[i] = condState;
        float gE_t0 = 0.0f;
#pragma unroll
        for (int ig = 0; ig < kMaxNG; ig++) {
            if (ig < ngFF) {
                gE_t0 += g0[ig];
                gE_t1 += g1[ig];
                P.gFF[ig * nV1 + i] = g1[ig];
                P.hFF[ig * nV1 + i] = h1[ig];
            }
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
        sInfo = spikeCount > 0 ? 1.0f + tsp / dt : v;
        P.sInfo[(size_t)(t & 1) * nV1 + i] = sInfo;
        if (P.recSpk) P.recSpk[(size_t)(t % P.recSlots) * nV1 + i] = sInfo;
        P.v[i] = v;
        if (P.iModel == 1) P.w[i] = w;
        P.tBack[i] = tBack;
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
    }

    // ------------------------------------------------------------------ phase C
    if (!P.farOn) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) P.farFlag[(t + 1) % 3] = 0;
    if (active && sInfo > 1.0f && P.farPre[i]) P.farFlag[t % 3] = 1;
    const bool push = active && sInfo >= 1.0f && P.farOff[i + 1] > P.farOff[i];
    if (__syncthreads_or(push) == 0) return;
    far_push(P, t, i, push, sInfo, s_pre, s_val, s_ball);
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

__global__ void advance_step_kernel(long long *stepBase, int k) { *stepBase += k; }

cudaError_t launch_v1_step(const V1Params &p, const long long *stepBase, int stepOffset,
                           const float *lgnSInfo, int lgnSlots, int deliverPrev, int doStep,
                           cudaStream_t st) {
    const int nq = (p.blockSize + kCta - 1) / kCta;
    v1_step_kernel<<<p.nblock * nq, kCta, 0, st>>>(p, stepBase, stepOffset, lgnSInfo, lgnSlots,
                                                   deliverPrev, doStep);
    return cudaGetLastError();
}

cudaError_t launch_v1_rng_init(curandStateMRG32k3a *cond, curandStateMRG32k3a *noisy,
                               unsigned long long seed, int nV1, int trainDepth, cudaStream_t st) {
    v1_rng_init_kernel<<<(nV1 + 127) / 128, 128, 0, st>>>(cond, noisy, seed, nV1, trainDepth);
    return cudaGetLastError();
}

cudaError_t launch_advance_step(long long *stepBase, int k, cudaStream_t st) {
    advance_step_kernel<<<1, 1, 0, st>>>(stepBase, k);
    return cudaGetLastError();
}

}  // namespace pv1
