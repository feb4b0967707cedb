// Surrogate-gradient adjoint of a conductance-based LIF patch (the differentiable form).
//
// The reference has no gradient code; this is the differentiable counterpart of its V1 step
// (src/coredynamics.cu:1235-2059 with the two-state conductance kernel of
// src/condShape.h:13-51), on batches of trials:
//   conductances  g' = g*Ed + h*dod*(Ed - Er),  h' = h*Er   (Ed = e^{-dt/td}, Er = e^{-dt/tr},
//                 dod = tr/(td - tr)), AMPA from the LGN, GABA from the block's I neurons;
//   membrane      RK2 (Heun) of dv/dt = -gL(v-vL) - gE(v-vE) - gI(v-vI) + I0 with the
//                 conductances of the start and of the end of the step, as the reference;
//   spikes        s = H(vn - vThres) forward, ds/dvn = 1/(1 + slope|vn - vThres|)^2 (fast
//                 sigmoid) backward; reset to vR with the reset gate held constant; refractory
//                 steps hold v at vR;
//   inputs        end of step t: hE += sum_k W[k][n] X[t][id[k][n]] (k ascending),
//                 hI += sum of C[p][n] over the I neurons p of the block that spiked (ascending);
//   outputs       per window of `win` steps: spike rate (Hz) and mean membrane potential.
// Spikes are delivered at step granularity (no sub-step spike-time offsets).
//
// One CTA (or a cluster of ctaSplit CTAs sharing the block's spike ballots and adjoints through
// distributed shared memory) holds one (trial, block) pair, one thread per neuron; blocks do
// not interact.  The
// forward stores a checkpoint of (v, gE, hE, gI, hI, refractory count) every `seg` steps; the
// backward walks the segments from the last one, recomputes each forward from its checkpoint
// into a per-CTA scratch, then runs the adjoint backwards through it.  The recurrent term of
// the adjoint (sum over posts of C[p][n] * lambda_hI[n] for every I neuron p) is a
// warp-cooperative mat-vec over the block's C rows per step.  Gradients: dL/dW by atomic adds
// at the (sparse) LGN events, dL/d(EdE, ErE, dodE, EdI, ErI, dodI) reduced in FP64.
#include <cmath>
#include <cstdint>
#include <string>

#include <cooperative_groups.h>

#include "pv1_internal.cuh"

namespace cg = cooperative_groups;

namespace {

thread_local std::string g_adjErr;

struct AdjArgs {
    pv1_adj_problem p;
    pv1_adj_buffers b;
    int N, nI, nWin, nSeg;
    int split;   // CTAs per (trial, block)
    int xBytes;  // dynamic shared memory of the LGN count stage (16-byte multiple)
    int synSmem; // 1: the synapse ids and weights are copied to dynamic shared memory after it
};

// Block-wide exchange between the CTAs of a (trial, block): stores go to every CTA of the
// cluster (split > 1) or to this CTA's shared memory only.
__device__ __forceinline__ void share_word(unsigned *addr, unsigned v, int split) {
    if (split == 1) {
        *addr = v;
        return;
    }
    cg::cluster_group cl = cg::this_cluster();
    for (int r = 0; r < split; r++) *cl.map_shared_rank(addr, r) = v;
}

__device__ __forceinline__ void share_float(float *addr, float v, int split) {
    if (split == 1) {
        *addr = v;
        return;
    }
    cg::cluster_group cl = cg::this_cluster();
    for (int r = 0; r < split; r++) *cl.map_shared_rank(addr, r) = v;
}

__device__ __forceinline__ void store_at_rank(float *addr, float v, int rank, int split) {
    if (split == 1) {
        *addr = v;
        return;
    }
    *cg::this_cluster().map_shared_rank(addr, rank) = v;
}

// Barrier over the (trial, block)'s CTAs (with the memory ordering of their shared writes).
__device__ __forceinline__ void block_sync(int split) {
    if (split == 1) __syncthreads();
    else cg::this_cluster().sync();
}

constexpr int kAdjMaxK = 32;

struct AState {
    float v, gE, hE, gI, hI;
    int ref;
};

__device__ __forceinline__ float adj_f(float v, float gE, float gI, float gL, float vL, float vE, float vI,
                                       float I0) {
    return -gL * (v - vL) - gE * (v - vE) - gI * (v - vI) + I0;
}

// Forward step of one neuron up to the spike decision; returns v_next, sets spk, refr and the
// decayed conductances.  Shared by the forward and the recompute of the backward.
__device__ __forceinline__ float adj_neuron_step(const pv1_adj_problem &P, AState &s, float I0, bool isE,
                                                 bool &spk, bool &refr, float &gE1, float &hE1, float &gI1,
                                                 float &hI1) {
    gE1 = s.gE * P.EdE + s.hE * P.dodE * (P.EdE - P.ErE);
    hE1 = s.hE * P.ErE;
    gI1 = s.gI * P.EdI + s.hI * P.dodI * (P.EdI - P.ErI);
    hI1 = s.hI * P.ErI;
    refr = s.ref > 0;
    spk = false;
    if (refr) {
        s.ref -= 1;
        return P.vR;
    }
    const float k1 = adj_f(s.v, s.gE, s.gI, P.gL, P.vL, P.vE, P.vI, I0);
    const float v1 = s.v + P.dt * k1;
    const float k2 = adj_f(v1, gE1, gI1, P.gL, P.vL, P.vE, P.vI, I0);
    const float vn = s.v + (P.dt * 0.5f) * (k1 + k2);
    spk = vn > P.vThres;
    if (spk) {
        s.ref = (int)(isE ? P.tRefE : P.tRefI);
        return P.vR;
    }
    return vn;
}

// The end-of-step inputs: LGN events into hE (synapse order), spiking I neurons of the block
// into hI (ascending).  ball[] holds this step's spike ballots of the CTA's warps; x is the
// step's row of LGN counts (shared-memory stage or global).  Returns the mask of the synapses
// that carried an event.
// The neuron's LGN synapse ids and weights: synapse k at ids[k * stride], W[k * stride] (the
// global [K][N] arrays with stride N, or the CTA's shared-memory copy with stride blockDim.x).
struct SynView {
    const int32_t *ids;
    const float *W;
    int stride;
};

__device__ __forceinline__ unsigned adj_inputs(const AdjArgs &A, const uint8_t *x, int n, int local,
                                               float &hE, float &hI, const unsigned *ball, SynView sv) {
    const pv1_adj_problem &P = A.p;
    unsigned mask = 0u;
    // LGN synapses in chunks of 8: the id and count loads of a chunk are in flight together;
    // the additions stay in synapse order
    for (int k0 = 0; k0 < (int)P.K; k0 += 8) {
        int id[8];
        unsigned c[8];
#pragma unroll
        for (int j = 0; j < 8; j++) id[j] = k0 + j < (int)P.K ? sv.ids[(k0 + j) * sv.stride] : 0;
#pragma unroll
        // x may be the shared-memory stage: a generic load, not the global-only __ldg
        for (int j = 0; j < 8; j++) c[j] = k0 + j < (int)P.K ? x[id[j]] : 0u;
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (c[j]) {
                hE = hE + sv.W[(k0 + j) * sv.stride] * (float)c[j];
                mask |= 1u << (k0 + j);
            }
    }
    // spiking I neurons of the block, ascending, up to 8 weight loads in flight
    const int blk = n / (int)P.blockSize;
    const float *C = A.b.Crec + (size_t)blk * A.nI * P.blockSize;
    const int nWarp = ((int)P.blockSize + 31) / 32;
    int w = (int)P.nE / 32;
    unsigned bits = w < nWarp ? ball[w] : 0u;
    while (true) {
        int pre[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            while (!bits && w < nWarp) {
                if (++w < nWarp) bits = ball[w];
            }
            pre[j] = -1;
            if (w < nWarp) {
                const int lane = __ffs(bits) - 1;
                bits &= bits - 1;
                pre[j] = w * 32 + lane - (int)P.nE;
            }
        }
        if (pre[0] < 0) break;
        float cv[8];
#pragma unroll
        for (int j = 0; j < 8; j++) cv[j] = pre[j] >= 0 ? __ldg(C + (size_t)pre[j] * P.blockSize + local) : 0.f;
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (pre[j] >= 0) hI = hI + cv[j];
        if (pre[7] < 0) break;
    }
    return mask;
}

// Copies the neuron's synapse ids and weights into the CTA's shared memory (column per
// thread) when the caller gave room for them, else views the global arrays.
__device__ __forceinline__ SynView stage_synapses(const AdjArgs &A, uint8_t *room, int n, bool on) {
    if (!room) return SynView{A.b.ids + n, A.b.W + n, A.N};
    int32_t *sIds = reinterpret_cast<int32_t *>(room);
    float *sW = reinterpret_cast<float *>(room + (size_t)A.p.K * blockDim.x * sizeof(int32_t));
    for (int k = 0; k < (int)A.p.K; k++) {
        sIds[k * blockDim.x + threadIdx.x] = on ? __ldg(A.b.ids + (size_t)k * A.N + n) : 0;
        sW[k * blockDim.x + threadIdx.x] = on ? __ldg(A.b.W + (size_t)k * A.N + n) : 0.f;
    }
    return SynView{sIds + threadIdx.x, sW + threadIdx.x, (int)blockDim.x};
}

// ---- LGN count rows staged into shared memory by the bulk-copy (TMA) engine ----
// Three buffers of one row (nLGN bytes) each with an mbarrier; the copy of the row two steps
// ahead is issued by thread 0 while the CTA works on the current one.  A wait gives
// up after a bounded number of polls and the step reads the row from global memory instead
// (same bytes), so a copy that never lands can slow a step but never hang it.
struct XStage {
    uint8_t *buf0, *buf1, *buf2;
    uint64_t *bar;                 // [3]
    unsigned uses0, uses1, uses2;  // copies issued into each buffer (uniform across the CTA)
    int row0, row1, row2;          // step held by each buffer (-1: none)
    bool on;
};

template <class T>
__device__ __forceinline__ T sel3(int k, T a, T b, T c) { return k == 0 ? a : (k == 1 ? b : c); }

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void xs_init(XStage &s, uint8_t *buf, uint64_t *bar, int nLGN, bool on) {
    s.buf0 = buf;
    s.buf1 = buf + nLGN;
    s.buf2 = buf + 2 * nLGN;
    s.bar = bar;
    s.uses0 = s.uses1 = s.uses2 = 0;
    s.row0 = s.row1 = s.row2 = -1;
    s.on = on;
    if (on && threadIdx.x == 0) {
        for (int k = 0; k < 3; k++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar + k)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
}

// Issue the copy of row t into buffer t % 3 (two rows ahead of use, so the copy has a whole
// step to land).  Call from all threads at a point where every thread is done with the
// buffer's previous row (after a __syncthreads of a later step).
__device__ __forceinline__ void xs_issue(XStage &s, const uint8_t *row, int t, int nLGN) {
    if (!s.on) return;
    const int k = t % 3;
    if (threadIdx.x == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(s.bar + k)),
                     "r"(nLGN)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(sel3(k, s.buf0, s.buf1, s.buf2))),
            "l"(row), "r"(nLGN), "r"(smem_u32(s.bar + k))
            : "memory");
    }
    if (k == 0) {
        s.uses0++;
        s.row0 = t;
    } else if (k == 1) {
        s.uses1++;
        s.row1 = t;
    } else {
        s.uses2++;
        s.row2 = t;
    }
}

// Row t: the staged copy once its mbarrier phase completed, else the global row.
__device__ __forceinline__ const uint8_t *xs_get(XStage &s, const uint8_t *row, int t) {
    if (!s.on) return row;
    const int k = t % 3;
    if (sel3(k, s.row0, s.row1, s.row2) != t) return row;
    const unsigned parity = (sel3(k, s.uses0, s.uses1, s.uses2) - 1) & 1;
    for (int i = 0; i < (1 << 20); i++) {
        unsigned ok;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(ok)
            : "r"(smem_u32(s.bar + k)), "r"(parity)
            : "memory");
        if (ok) return sel3(k, s.buf0, s.buf1, s.buf2);
        if (i > 8) __nanosleep(256);
    }
    return row;
}

template <int MaxThreads>
__global__ void __launch_bounds__(MaxThreads) adj_forward_kernel(AdjArgs A, int stage) {
    __shared__ unsigned ball[2][32];   // double buffered: step t uses ball[t & 1]
    __shared__ __align__(8) uint64_t xbar[3];
    extern __shared__ __align__(16) uint8_t xbuf[];
    const pv1_adj_problem &P = A.p;
    const int split = A.split;
    const int blk = blockIdx.x / split, b = blockIdx.y;
    const int local = (blockIdx.x % split) * blockDim.x + threadIdx.x;
    const bool on = local < (int)P.blockSize;
    const int n = blk * (int)P.blockSize + (on ? local : 0);
    const size_t bn = (size_t)b * A.N + n;
    const bool isE = local < (int)P.nE;
    const float I0 = on ? A.b.I0[n] : 0.f;
    AState s{on ? A.b.v0[bn] : P.vR, 0.f, 0.f, 0.f, 0.f, 0};
    float cnt = 0.f, vsum = 0.f;
    const size_t BN = (size_t)P.B * A.N;
    const uint8_t *Xb = A.b.X + (size_t)b * P.T * P.nLGN;
    XStage xs;
    xs_init(xs, xbuf, xbar, (int)P.nLGN, stage != 0);
    const SynView sv = stage_synapses(A, A.synSmem ? xbuf + A.xBytes : nullptr, n, on);
    if (split > 1) cg::this_cluster().sync();   // every CTA of the cluster runs before remote stores
    xs_issue(xs, Xb, 0, (int)P.nLGN);
    if (P.T > 1) xs_issue(xs, Xb + P.nLGN, 1, (int)P.nLGN);
    for (int t = 0; t < (int)P.T; t++) {
        if (t % (int)P.seg == 0 && on) {
            float *ck = A.b.ck + (size_t)(t / P.seg) * 6 * BN + bn;
            ck[0] = s.v; ck[BN] = s.gE; ck[2 * BN] = s.hE; ck[3 * BN] = s.gI; ck[4 * BN] = s.hI;
            ck[5 * BN] = (float)s.ref;
        }
        bool spk = false, refr = false;
        float gE1 = 0.f, hE1 = 0.f, gI1 = 0.f, hI1 = 0.f, vnext = 0.f;
        if (on) vnext = adj_neuron_step(P, s, I0, isE, spk, refr, gE1, hE1, gI1, hI1);
        const unsigned bal = __ballot_sync(0xffffffffu, on && spk);
        // the readers of ball[t & 1] (step t - 2) and of the count row t - 1 finished before the
        // previous step's barrier
        if ((local & 31) == 0) share_word(&ball[t & 1][local >> 5], bal, split);
        block_sync(split);
        if (t + 2 < (int)P.T) xs_issue(xs, Xb + (size_t)(t + 2) * P.nLGN, t + 2, (int)P.nLGN);
        const uint8_t *x = xs_get(xs, Xb + (size_t)t * P.nLGN, t);
        if (on) {
            adj_inputs(A, x, n, local, hE1, hI1, ball[t & 1], sv);
            s.v = vnext;
            s.gE = gE1; s.hE = hE1; s.gI = gI1; s.hI = hI1;
            cnt += spk ? 1.f : 0.f;
            vsum += vnext;
            if ((t + 1) % (int)P.win == 0) {
                const size_t o = ((size_t)b * A.nWin + t / P.win) * A.N + n;
                A.b.rates[o] = cnt / ((float)P.win * P.dt * 1e-3f);
                A.b.vbar[o] = vsum / (float)P.win;
                cnt = 0.f;
                vsum = 0.f;
            }
        }
    }
}

__device__ __forceinline__ void block_add_double(double v, double *out, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) atomicAdd(out, v);
    }
}

constexpr int kScrWords = 7;   // v, gE, hE, gI, hI, flags, LGN event mask per neuron and step

template <int MaxThreads>
__global__ void __launch_bounds__(MaxThreads) adj_backward_kernel(AdjArgs A, int stage) {
    __shared__ unsigned ball[2][32];
    __shared__ float lam[1024];
    __shared__ float dS[1024];
    __shared__ double red[32];
    __shared__ __align__(8) uint64_t xbar[3];
    extern __shared__ __align__(16) uint8_t xbuf[];
    const pv1_adj_problem &P = A.p;
    const int split = A.split;
    const int ctaN = (int)blockDim.x;
    const int blk = blockIdx.x / split, b = blockIdx.y;
    const int local = (blockIdx.x % split) * ctaN + threadIdx.x;
    const int bs = (int)P.blockSize;
    const bool on = local < bs;
    const int n = blk * bs + (on ? local : 0);
    const size_t bn = (size_t)b * A.N + n;
    const bool isE = local < (int)P.nE;
    const float I0 = on ? A.b.I0[n] : 0.f;
    const size_t BN = (size_t)P.B * A.N;
    float *scr = A.b.scratch + (size_t)(b * (int)P.nblock + blk) * P.seg * kScrWords * bs;
    const float *C = A.b.Crec + (size_t)blk * A.nI * bs;
    const float rateScale = 1.f / ((float)P.win * P.dt * 1e-3f);
    const float invWin = 1.f / (float)P.win;
    const int warp = local >> 5, lane = local & 31, nWarp = (bs + 31) / 32;
    const uint8_t *Xb = A.b.X + (size_t)b * P.T * P.nLGN;
    XStage xs;
    xs_init(xs, xbuf, xbar, (int)P.nLGN, stage != 0);
    const SynView sv = stage_synapses(A, A.synSmem ? xbuf + A.xBytes : nullptr, n, on);
    if (split > 1) cg::this_cluster().sync();   // every CTA of the cluster runs before remote stores
    // adjoints of the state after the current step
    float lv = 0.f, lgE = 0.f, lhE = 0.f, lgI = 0.f, lhI = 0.f;
    float dEdE = 0.f, dErE = 0.f, ddodE = 0.f, dEdI = 0.f, dErI = 0.f, ddodI = 0.f;
    for (int sg = A.nSeg - 1; sg >= 0; sg--) {
        const int t0 = sg * (int)P.seg;
        const int t1 = min((int)P.T, t0 + (int)P.seg);
        // recompute the segment forward from its checkpoint
        AState s{};
        if (on) {
            const float *ck = A.b.ck + (size_t)sg * 6 * BN + bn;
            s = AState{ck[0], ck[BN], ck[2 * BN], ck[3 * BN], ck[4 * BN], (int)ck[5 * BN]};
        }
        __syncthreads();
        xs_issue(xs, Xb + (size_t)t0 * P.nLGN, t0, (int)P.nLGN);
        if (t0 + 1 < t1) xs_issue(xs, Xb + (size_t)(t0 + 1) * P.nLGN, t0 + 1, (int)P.nLGN);
        for (int t = t0; t < t1; t++) {
            bool spk = false, refr = false;
            float gE1 = 0.f, hE1 = 0.f, gI1 = 0.f, hI1 = 0.f, vnext = 0.f;
            float *o = scr + (size_t)(t - t0) * kScrWords * bs + local;
            if (on) {
                o[0] = s.v; o[bs] = s.gE; o[2 * bs] = s.hE; o[3 * bs] = s.gI; o[4 * bs] = s.hI;
                vnext = adj_neuron_step(P, s, I0, isE, spk, refr, gE1, hE1, gI1, hI1);
                o[5 * bs] = (float)((refr ? 1 : 0) | (spk ? 2 : 0));
            }
            const unsigned bal = __ballot_sync(0xffffffffu, on && spk);
            if (lane == 0) share_word(&ball[t & 1][warp], bal, split);
            block_sync(split);
            if (t + 2 < t1) xs_issue(xs, Xb + (size_t)(t + 2) * P.nLGN, t + 2, (int)P.nLGN);
            const uint8_t *x = xs_get(xs, Xb + (size_t)t * P.nLGN, t);
            if (on) {
                const unsigned mask = adj_inputs(A, x, n, local, hE1, hI1, ball[t & 1], sv);
                o[6 * bs] = __uint_as_float(mask);
                s.v = vnext;
                s.gE = gE1; s.hE = hE1; s.gI = gI1; s.hI = hI1;
            }
        }
        // adjoint backwards through the segment
        for (int t = t1 - 1; t >= t0; t--) {
            // recurrent term: dS[p] = sum_n C[p][n] * lambda_hI(t+1)[n] for the I neurons p
            if (P.recGrad) {
                block_sync(split);   // the readers of lam[] and dS[] of the previous step are done
                share_float(&lam[local], on ? lhI : 0.f, split);
                block_sync(split);
                for (int p = warp; p < A.nI; p += nWarp) {
                    const float *row = C + (size_t)p * bs;
                    float acc = 0.f;
                    for (int j = lane; j < bs; j += 32) acc += __ldg(row + j) * lam[j];
                    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
                    // into the CTA that holds I neuron p
                    if (lane == 0) store_at_rank(&dS[p], acc, ((int)P.nE + p) / ctaN, split);
                }
                block_sync(split);
            }
            if (!on) continue;
            const float *o = scr + (size_t)(t - t0) * kScrWords * bs + local;
            const float v = o[0], gE = o[bs], hE = o[2 * bs], gI = o[3 * bs], hI = o[4 * bs];
            const int fl = (int)o[5 * bs];
            unsigned mask = __float_as_uint(o[6 * bs]);
            const int win = t / (int)P.win;
            const size_t oo = ((size_t)b * A.nWin + win) * A.N + n;
            float dLds = A.b.gR ? A.b.gR[oo] * rateScale : 0.f;
            if (!isE && P.recGrad) dLds += dS[local - (int)P.nE];
            float lvn_next = lv + (A.b.gV ? A.b.gV[oo] * invWin : 0.f);   // adjoint of v(t+1)
            // LGN weight gradients at this step's events (the recompute recorded which synapses)
            while (mask) {
                const int k = __ffs(mask) - 1;
                mask &= mask - 1;
                const int id = sv.ids[k * sv.stride];
                const float c = (float)__ldg(Xb + (size_t)t * P.nLGN + id);
                atomicAdd(A.b.gW + (size_t)k * A.N + n, lhE * c);
            }
            const bool refr = fl & 1, spk = fl & 2;
            const float gE1 = gE * P.EdE + hE * P.dodE * (P.EdE - P.ErE);
            const float gI1 = gI * P.EdI + hI * P.dodI * (P.EdI - P.ErI);
            float lgE1 = lgE, lgI1 = lgI;
            const float lhE1 = lhE, lhI1 = lhI;
            float lvt = 0.f, lgE0 = 0.f, lgI0 = 0.f;
            if (!refr) {
                const float k1 = adj_f(v, gE, gI, P.gL, P.vL, P.vE, P.vI, I0);
                const float v1 = v + P.dt * k1;
                const float k2 = adj_f(v1, gE1, gI1, P.gL, P.vL, P.vE, P.vI, I0);
                const float vn = v + (P.dt * 0.5f) * (k1 + k2);
                const float xsv = vn - P.vThres;
                const float den = 1.f + P.slope * fabsf(xsv);
                const float lvn = (spk ? 0.f : lvn_next) + dLds / (den * den);
                const float lk2 = lvn * (P.dt * 0.5f);
                const float a1 = -P.gL - gE1 - gI1;
                const float lv1 = lk2 * a1;
                const float lk1 = lvn * (P.dt * 0.5f) + lv1 * P.dt;
                const float a0 = -P.gL - gE - gI;
                lvt = lvn + lk1 * a0 + lv1;
                lgE0 = -lk1 * (v - P.vE);
                lgI0 = -lk1 * (v - P.vI);
                lgE1 += -lk2 * (v1 - P.vE);
                lgI1 += -lk2 * (v1 - P.vI);
            }
            dEdE += lgE1 * (gE + hE * P.dodE);
            ddodE += lgE1 * hE * (P.EdE - P.ErE);
            dErE += lhE1 * hE - lgE1 * hE * P.dodE;
            dEdI += lgI1 * (gI + hI * P.dodI);
            ddodI += lgI1 * hI * (P.EdI - P.ErI);
            dErI += lhI1 * hI - lgI1 * hI * P.dodI;
            lgE = lgE1 * P.EdE + lgE0;
            lhE = lgE1 * P.dodE * (P.EdE - P.ErE) + lhE1 * P.ErE;
            lgI = lgI1 * P.EdI + lgI0;
            lhI = lgI1 * P.dodI * (P.EdI - P.ErI) + lhI1 * P.ErI;
            lv = lvt;
        }
    }
    if (!on) dEdE = dErE = ddodE = dEdI = dErI = ddodI = 0.f;
    block_add_double(dEdE, A.b.gC + 0, red);
    block_add_double(dErE, A.b.gC + 1, red);
    block_add_double(ddodE, A.b.gC + 2, red);
    block_add_double(dEdI, A.b.gC + 3, red);
    block_add_double(dErI, A.b.gC + 4, red);
    block_add_double(ddodI, A.b.gC + 5, red);
}

int adj_check(const pv1_adj_problem *p, const pv1_adj_buffers *b, AdjArgs *A, bool backward) {
    if (!p || !b) return PV1_E_ARG;
    if (p->blockSize < 32 || p->blockSize > 1024 || p->blockSize % 32 || p->nE % 32 || p->nE >= p->blockSize ||
        p->B < 1 || p->nblock < 1 || p->K < 1 || p->K > kAdjMaxK || p->T < 1 || p->seg < 1 || p->win < 1 ||
        p->T % p->win || p->nLGN < 1 || !(p->dt > 0)) {
        g_adjErr = "bad problem sizes (blockSize multiple of 32 up to 1024, nE multiple of 32, K <= 32, "
                   "T a multiple of win)";
        return PV1_E_ARG;
    }
    if (!b->ids || !b->W || !b->X || !b->Crec || !b->I0 || !b->v0 || !b->ck) {
        g_adjErr = "missing input buffer";
        return PV1_E_ARG;
    }
    if (!backward && (!b->rates || !b->vbar)) {
        g_adjErr = "missing output buffer";
        return PV1_E_ARG;
    }
    if (backward && (!b->gW || !b->gC || !b->scratch)) {
        g_adjErr = "missing gradient or scratch buffer";
        return PV1_E_ARG;
    }
    A->p = *p;
    A->b = *b;
    A->N = (int)(p->nblock * p->blockSize);
    A->nI = (int)(p->blockSize - p->nE);
    A->nWin = (int)(p->T / p->win);
    A->nSeg = (int)((p->T + p->seg - 1) / p->seg);
    int split = (int)p->ctaSplit;
    if (split == 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        split = (p->blockSize % 64 == 0 && (long long)p->B * p->nblock * 2 <= sms) ? 2 : 1;
    }
    if (split != 1 && (split != 2 || p->blockSize % 64)) {
        g_adjErr = "ctaSplit must be 0, 1 or 2 (2 needs blockSize a multiple of 64)";
        return PV1_E_ARG;
    }
    A->split = split;
    return PV1_OK;
}

// Dynamic shared memory: the LGN count stage (3 rows) and, when it fits, the CTA's synapse
// ids and weights (K x threads each).
void adj_smem_plan(AdjArgs &A, int stage) {
    const int threads = (int)(A.p.blockSize / A.split);
    A.xBytes = stage ? (int)((3 * A.p.nLGN + 15) / 16 * 16) : 0;
    const size_t syn = (size_t)A.p.K * threads * 8;
    A.synSmem = A.xBytes + syn <= 160 * 1024 ? 1 : 0;
}

template <class Kern>
cudaError_t adj_launch(Kern kern, const AdjArgs &A, int stage, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(A.p.nblock * A.split, A.p.B);
    cfg.blockDim = dim3(A.p.blockSize / A.split);
    cfg.dynamicSmemBytes = (size_t)A.xBytes + (A.synSmem ? (size_t)A.p.K * cfg.blockDim.x * 8 : 0);
    if (cfg.dynamicSmemBytes > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)cfg.dynamicSmemBytes);
        if (e != cudaSuccess) return e;
    }
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = A.split;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = A.split > 1 ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, A, stage);
}

// Count rows go through the bulk-copy stage when their size and offsets are multiples of 16
// bytes and two of them fit the default dynamic shared memory.
int adj_stage(const pv1_adj_problem *p) { return (p->nLGN % 16 == 0 && 3 * p->nLGN <= 32768) ? 1 : 0; }

}  // namespace

extern "C" {

const char *pv1_adj_last_error(void) { return g_adjErr.c_str(); }

uint64_t pv1_adj_checkpoint_floats(const pv1_adj_problem *p) {
    if (!p) return 0;
    return (uint64_t)((p->T + p->seg - 1) / p->seg) * 6 * p->B * p->nblock * p->blockSize;
}

uint64_t pv1_adj_scratch_floats(const pv1_adj_problem *p) {
    if (!p) return 0;
    return (uint64_t)p->B * p->nblock * p->seg * kScrWords * p->blockSize;
}

int pv1_adj_forward(const pv1_adj_problem *p, const pv1_adj_buffers *b, void *stream) {
    AdjArgs A;
    int r = adj_check(p, b, &A, false);
    if (r) return r;
    const int stage = adj_stage(p);
    adj_smem_plan(A, stage);
    cudaError_t e = A.p.blockSize / A.split <= 512 ? adj_launch(adj_forward_kernel<512>, A, stage, (cudaStream_t)stream)
                                                   : adj_launch(adj_forward_kernel<1024>, A, stage, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        g_adjErr = cudaGetErrorString(e);
        return PV1_E_CUDA;
    }
    return PV1_OK;
}

int pv1_adj_backward(const pv1_adj_problem *p, const pv1_adj_buffers *b, void *stream) {
    AdjArgs A;
    int r = adj_check(p, b, &A, true);
    if (r) return r;
    const int stage = adj_stage(p);
    adj_smem_plan(A, stage);
    cudaError_t e = A.p.blockSize / A.split <= 512
                        ? adj_launch(adj_backward_kernel<512>, A, stage, (cudaStream_t)stream)
                        : adj_launch(adj_backward_kernel<1024>, A, stage, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        g_adjErr = cudaGetErrorString(e);
        return PV1_E_CUDA;
    }
    return PV1_OK;
}

}  // extern "C"
