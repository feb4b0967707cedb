// Far delivery with synaptic failure.
//
// The reference delivers far synapses on the host (recal_G_vec, src/coredynamics.cu:181-372):
// post by post in each chunk of blocks, synapse by synapse in the post's vec order, two ring
// slots per synapse; a delivered event of a pair with failure rate p > 0 scales its strength
// by 1 - p + sqrt(p(1-p)/synPerCon) * z, z drawn from the post's own default_random_engine
// (seeded seed+i, src/patch.cu:4224-4228) through one normal_distribution<float> shared by
// the whole chunk call.  That distribution keeps the second value of each polar-method pair
// for its next call, whichever engine the call passes, so the draws of a chunk form one
// sequence: the draw at an even index of the chunk's sequence generates a pair from its
// post's engine, the draw at the next (odd) index takes that pair's second value.
//
// Here the same sequence is computed in parallel, one thread per post, in four launches per
// step: (1) each post counts its draws (the same window tests as the delivery); (2) one CTA
// per chunk scans the counts into each post's first index and finds the previous post that
// drew; (3) posts whose last draw sits at an even index run their engines to publish the
// unused second value (their carry); (4) each post runs its engine again, taking a leading
// odd-index draw from the previous drawer's carry, and sums its far input in vec order into
// farPull, which the next step's delivery adds after the near input (sum_G).  With no far
// presynaptic spike in the step (fill_fSpikeTrain found none) nothing is drawn or added.
//
// libstdc++'s pieces restated: minstd_rand0 (x <- 16807 x mod 2^31-1), generate_canonical
// <float, 24> with one engine call ((x-1) as float / 2^31 as float, clamped below 1), and the
// Marsaglia polar method with the second value kept.  logf may differ from the host's by an
// ulp, so the draws agree with the host's to float rounding.
#include "pv1_internal.cuh"

namespace pv1 {
namespace {

constexpr int kPolarTries = 1000;   // acceptance is pi/4 per try

__device__ __forceinline__ int type_in_block(const V1Params &P, int local) {
    int t = P.nType - 1;
#pragma unroll
    for (int j = kMaxType - 1; j >= 0; j--)
        if (j < P.nType && local < P.typeAcc[j]) t = j;
    return t;
}

__device__ __forceinline__ unsigned minstd_next(unsigned &x) {
    x = (unsigned)(((unsigned long long)x * 16807ull) % 2147483647ull);
    return x;
}

__device__ __forceinline__ float std_canonical(unsigned &x) {
    const float r = __fdiv_rn(__uint2float_rn(minstd_next(x) - 1u), 2147483648.0f);
    return r >= 1.0f ? 0x1.fffffep-1f : r;
}

// One polar-method pair from engine x: returns the first value handed out, keeps the other.
__device__ __forceinline__ float std_pair(unsigned &x, float &saved, int *err) {
    float a = 0.f, b = 0.f, r2 = 2.f;
    for (int k = 0; k < kPolarTries; k++) {
        a = __double2float_rn(__dsub_rn((double)__fmul_rn(2.0f, std_canonical(x)), 1.0));
        b = __double2float_rn(__dsub_rn((double)__fmul_rn(2.0f, std_canonical(x)), 1.0));
        r2 = __fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b));
        if (!(r2 > 1.0f || r2 == 0.0f)) break;
    }
    if (r2 > 1.0f || r2 == 0.0f) {
        atomicOr(err, kErrBounds);
        saved = 0.f;
        return 0.f;
    }
    const float mult = sqrtf(__fdiv_rn(__fmul_rn(-2.0f, logf(r2)), r2));
    saved = __fmul_rn(a, mult);
    return __fmul_rn(b, mult);
}

__device__ __forceinline__ long long ring_row(long long ts, int D) { return ((ts % D) + D) % D; }

// Whether synapse e's k-th ring slot delivers at step t: its spike word sI and the offset
// dtsp = (sInfo - nsp + k)*dt - time2post in [0, dt) (src/coredynamics.cu:316-320).
__device__ __forceinline__ bool pull_arrival(const V1Params &P, long long t, int e, int k, float &sI,
                                             float &dtsp) {
    const int steps = P.pullSteps[e];
    const long long ts = t - steps + k;
    sI = P.sRing[(size_t)ring_row(ts, P.sDepth) * P.nV1 + P.pullPre[e]];
    if (!(sI >= 1.0f)) return false;
    const float nsp = floorf(sI);
    dtsp = __fsub_rn(__fmul_rn(__fadd_rn(__fsub_rn(sI, nsp), (float)k), P.dt), P.pullFrac[e]);
    return dtsp < P.dt && dtsp >= 0;
}

__device__ __forceinline__ long long step_of(const long long *stepBase, long long off) {
    return (stepBase ? *stepBase : 0) + off;
}

__global__ void far_pull_count_kernel(V1Params P, const long long *stepBase, long long off) {
    const long long t = step_of(stepBase, off);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) P.pullFlag[(t + 4) % 3] = 0;   // step t+1's flag (t >= -1)
    if (i >= P.nV1) return;
    const float own = P.sRing[(size_t)ring_row(t, P.sDepth) * P.nV1 + i];
    if (own > 1.0f && P.pullIsPre[i]) P.pullFlag[(t + 3) % 3] = 1;
    int c = 0;
    for (int e = P.pullOff[i]; e < P.pullOff[i + 1]; e++) {
        if (!(P.pullP[e] > 0)) continue;
        for (int k = 0; k < 2; k++) {
            float sI, dtsp;
            if (pull_arrival(P, t, e, k, sI, dtsp)) c++;
        }
    }
    P.pullCount[i] = c;
}

// One CTA per chunk: exclusive scan of the counts and the last earlier post with draws.
__global__ void __launch_bounds__(1024) far_pull_scan_kernel(V1Params P, const long long *stepBase, long long off) {
    const long long t = step_of(stepBase, off);
    if (!P.pullFlag[(t + 3) % 3]) return;
    __shared__ int sSum[32], sMax[32];
    __shared__ int carrySum, carryPrev;
    const int c0 = P.chunkStart[blockIdx.x], c1 = P.chunkStart[blockIdx.x + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) {
        carrySum = 0;
        carryPrev = -1;
    }
    __syncthreads();
    for (int base = c0; base < c1; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int cnt = i < c1 ? P.pullCount[i] : 0;
        const int me = cnt > 0 ? i : -1;
        int incl = cnt, mx = me;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            const int z = __shfl_up_sync(0xffffffffu, mx, o);
            if (lane >= o) {
                incl += y;
                mx = max(mx, z);
            }
        }
        if (lane == 31) {
            sSum[warp] = incl;
            sMax[warp] = mx;
        }
        __syncthreads();
        int wSum = 0, wMax = -1;
        for (int w = 0; w < warp; w++) {
            wSum += sSum[w];
            wMax = max(wMax, sMax[w]);
        }
        // previous drawer: the last post with draws strictly before i
        int before = __shfl_up_sync(0xffffffffu, mx, 1);
        if (lane == 0) before = -1;
        const int exclMax = max(max(carryPrev, wMax), before);
        if (i < c1) {
            P.pullStart[i] = carrySum + wSum + incl - cnt;
            P.pullPrev[i] = exclMax;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int s = 0, m = -1;
            for (int w = 0; w < nw; w++) {
                s += sSum[w];
                m = max(m, sMax[w]);
            }
            carrySum += s;
            carryPrev = max(carryPrev, m);
        }
        __syncthreads();
    }
}

// Posts whose last draw has an even index publish the second value of that pair.
__global__ void far_pull_carry_kernel(V1Params P, const long long *stepBase, long long off) {
    const long long t = step_of(stepBase, off);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nV1 || !P.pullFlag[(t + 3) % 3]) return;
    const int cnt = P.pullCount[i];
    if (cnt == 0) return;
    const int s0 = P.pullStart[i];
    if (((s0 + cnt - 1) & 1) != 0) return;
    unsigned x = P.eng[i];
    float saved = 0.f;
    for (int r = 0; r < cnt; r++)
        if (((s0 + r) & 1) == 0) (void)std_pair(x, saved, P.err);
    P.pullCarry[i] = saved;
}

__global__ void far_pull_sum_kernel(V1Params P, const long long *stepBase, long long off) {
    const long long t = step_of(stepBase, off);
    const int nV1 = P.nV1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV1) return;
    const int ngE = P.ngE, ngI = P.ngI, ns = ngE + ngI;
    float lg[2 * kMaxNG], lh[2 * kMaxNG];
#pragma unroll
    for (int q = 0; q < 2 * kMaxNG; q++) lg[q] = lh[q] = 0.f;
    if (P.pullFlag[(t + 3) % 3]) {
        const int itype = type_in_block(P, i % P.blockSize);
        const int cnt = P.pullCount[i];
        const int s0 = P.pullStart[i];
        const float carryIn = (cnt > 0 && (s0 & 1)) ? P.pullCarry[P.pullPrev[i]] : 0.f;
        unsigned x = P.eng[i];
        float saved = 0.f;
        int r = 0;
        for (int e = P.pullOff[i]; e < P.pullOff[i + 1]; e++) {
            const int pre = P.pullPre[e];
            const bool preE = (pre % P.blockSize) < P.nE;
            const float p = P.pullP[e];
            for (int k = 0; k < 2; k++) {
                float sI, dtsp;
                if (!pull_arrival(P, t, e, k, sI, dtsp)) continue;
                float f = P.pullStr[e];
                if (p > 0) {
                    float z;
                    if (((s0 + r) & 1) == 0) z = std_pair(x, saved, P.err);
                    else z = r == 0 ? carryIn : saved;
                    r++;
                    f = __fmul_rn(f, __fadd_rn(1 - p, __fmul_rn(P.pullStd[e], z)));
                }
                if (f > 0) {
                    const float nsp = floorf(sI);
                    const float delta = __fsub_rn(P.dt, dtsp);
#pragma unroll
                    for (int ig = 0; ig < kMaxNG; ig++) {
                        if (preE && ig < ngE) {
                            const float fv = __fmul_rn(__fmul_rn(nsp, f), P.pE[itype * ngE + ig]);
                            cond_input_v(P.condE.rise[ig], P.condE.decay[ig], P.condE.dod[ig], lg[ig], lh[ig], fv, delta);
                        }
                        if (!preE && ig < ngI) {
                            const float fv = __fmul_rn(__fmul_rn(nsp, f), P.pI[itype * ngI + ig]);
                            cond_input_v(P.condI.rise[ig], P.condI.decay[ig], P.condI.dod[ig], lg[ngE + ig],
                                         lh[ngE + ig], fv, delta);
                        }
                    }
                }
            }
        }
        P.eng[i] = x;
    }
#pragma unroll
    for (int q = 0; q < 2 * kMaxNG; q++) {
        if (q < ns) {
            P.farPull[(size_t)(2 * q) * nV1 + i] = lg[q];
            P.farPull[(size_t)(2 * q + 1) * nV1 + i] = lh[q];
        }
    }
}

__global__ void far_pull_apply_kernel(V1Params P) {
    const int nV1 = P.nV1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV1) return;
    const int ngE = P.ngE, ns = P.ngE + P.ngI;
    for (int q = 0; q < ns; q++) {
        const float g = P.farPull[(size_t)(2 * q) * nV1 + i], h = P.farPull[(size_t)(2 * q + 1) * nV1 + i];
        if (q < ngE) {
            P.gE[(size_t)q * nV1 + i] += g;
            P.hE[(size_t)q * nV1 + i] += h;
        } else {
            P.gI[(size_t)(q - ngE) * nV1 + i] += g;
            P.hI[(size_t)(q - ngE) * nV1 + i] += h;
        }
    }
}

}  // namespace

cudaError_t launch_far_pull(const V1Params &p, const long long *stepBase, long long off, cudaStream_t st) {
    const int n = (p.nV1 + 255) / 256;
    far_pull_count_kernel<<<n, 256, 0, st>>>(p, stepBase, off);
    far_pull_scan_kernel<<<p.nChunk, 1024, 0, st>>>(p, stepBase, off);
    far_pull_carry_kernel<<<n, 256, 0, st>>>(p, stepBase, off);
    far_pull_sum_kernel<<<n, 256, 0, st>>>(p, stepBase, off);
    return cudaGetLastError();
}

cudaError_t launch_far_pull_apply(const V1Params &p, cudaStream_t st) {
    far_pull_apply_kernel<<<(p.nV1 + 255) / 256, 256, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace pv1
