// LGN stage of the patchV1 hot path on GB300 (sm_103a).
//
// The reference re-walks the whole temporal window every step: for each of ~32 frames it
// re-samples the stimulus texture and block-reduces the spatial contrast of every cell
// (LGN_convol_magno, src/discrete_input_convol.cu:1342-1585).  The spatial contrast of a
// cell depends only on (cell, frame), so here it is computed once per distinct frame of the
// movie (lgn_spatial_kernel) and the per-step work reduces to a short contraction over the
// frames of the window with per-frame sums of the temporal weights (lgn_step_kernel), fused
// with the logistic rate and the exact-time Poisson generator (LGN_nonlinear + get_spike,
// src/discrete_input_convol.cu:1587-1821).
#include "pv1_internal.cuh"

namespace pv1 {

// Gaussian spatial kernel of the reference (spatialKernel, src/discrete_input_convol.cu:8-12).
__device__ __forceinline__ float gauss2(float x, float y, float rx, float ry) {
    return expf(-x * x / (rx * rx) - y * y / (ry * ry));
}

// Biphasic gamma-shaped temporal kernel (temporalKernel, src/discrete_input_convol.cu:14-33).
__device__ __forceinline__ float temporal_kernel(float tau, float tauR, float tauD, float nR,
                                                 float nD, float ratio, float lfac1,
                                                 float lfac2) {
    float tau1 = tau / tauR;
    float tau2 = tau / tauD;
    float A1 = (nR - 1) * logf(tau1);
    float A2 = (nD - 1) * logf(tau2);
    float tpR = expf(A1 - tau1 - lfac1) / tauR;
    float tpD = expf(A2 - tau2 - lfac2) / tauD;
    return tpR - ratio * tpD;
}

// Block-wide sum (any block size up to 1024); every thread gets the total.
__device__ float block_sum(float v, float *scratch) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int nwarp = (blockDim.x + 31) >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    float t = 0.f;
    if (warp == 0) {
        t = lane < nwarp ? scratch[lane] : 0.f;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) scratch[32] = t;
    }
    __syncthreads();
    return scratch[32];
}



// One CTA per magno cell, one thread per spatial sample (store_PM with PM=1,
// src/discrete_input_convol.cu:427-744, store_temporalWeight :230-305).
__global__ void __launch_bounds__(1024) lgn_setup_kernel(SetupArgs A) {
    __shared__ float scratch[33];
    const int cell = blockIdx.x;
    const int tid = threadIdx.x;
    const int nSample = A.nSample;
    int id = A.nParvo_I + cell;
    if (cell >= A.nMagno_I) id += A.nParvo_C;
    const int lid = id;  // center entry; surround at nLGN + id

    // ---- temporal weights, time reversed: TW[j] = K(t_{nKS-1-j}), normalised by sum|K| ----
    {
        const float tauR = A.tauR[lid], tauD = A.tauD[lid], nR = A.nR[lid], nD = A.nD[lid];
        const float ratio = A.ratio[lid];
        const float lfac1 = lgammaf(nR), lfac2 = lgammaf(nD);
        const float t0 = A.kernelSampleT0 - A.delay[lid];
        float local = 0.f;
        for (int j = tid; j < A.nKS; j += blockDim.x) {
            int twid = A.nKS - 1 - j;
            float t = twid * A.kernelSampleDt + t0;
            float tw = t < 0 ? 0.0f : temporal_kernel(t, tauR, tauD, nR, nD, ratio, lfac1, lfac2);
            A.TW[(size_t)cell * A.nKS + j] = tw;
            local += fabsf(tw);
        }
        float total = block_sum(local, scratch);
        for (int j = tid; j < A.nKS; j += blockDim.x) {
            A.TW[(size_t)cell * A.nKS + j] /= total;
        }
        __syncthreads();
        if (tid == 0) {
            // cumulative sums in double so per-frame segment sums lose nothing
            double acc = 0.0;
            A.ctw[cell] = 0.0;
            for (int j = 0; j < A.nKS; j++) {
                acc += (double)A.TW[(size_t)cell * A.nKS + j];
                A.ctw[(size_t)(j + 1) * A.nMagno + cell] = acc;
            }
        }
    }

    // ---- DoG spatial weights and sample coordinates (magno branch) ----
    const float cPolar = A.polar[lid], cEcc = A.ecc[lid];
    const float c_rx = A.rw[lid], c_ry = A.rh[lid];
    const float c_orient = A.orient[lid];
    const float k = A.k[lid];
    const int sid = A.nLGN + lid;
    const float sPolar = A.polar[sid], sEcc = A.ecc[sid];
    const float s_rx = A.rw[sid], s_ry = A.rh[sid];
    const float s_orient = A.orient[sid];
    // center -> surround offset in visual-field coordinates
    const float ox = sEcc * cosf(sPolar) - cEcc * cosf(cPolar);
    const float oy = sEcc * sinf(sPolar) - cEcc * sinf(cPolar);
    float d_orient = c_orient - s_orient;
    if (fabsf(d_orient) > (float)(M_PI / 2)) d_orient -= copysignf((float)M_PI, d_orient);
    const float rcos = cosf(d_orient), rsin = sinf(d_orient);
    const float rs = s_rx > s_ry ? s_rx : s_ry;
    const float span = A.nsig * rs + sqrtf(ox * ox + oy * oy);
    const float ds = 2 * span / A.nSample1D;
    const int tx = tid % A.nSample1D, ty = tid / A.nSample1D;
    const bool active = tid < nSample;
    float cx = (tx + 0.5f) * ds - span;
    float cy = (ty + 0.5f) * ds - span;
    float ttx = cx - ox, tty = cy - oy;
    float sx = ttx * rcos - tty * rsin;
    float sy = ttx * rsin + tty * rcos;
    float cw = active ? gauss2(cx, cy, c_rx, c_ry) : 0.f;
    float csum = block_sum(cw, scratch);
    cw /= csum;
    float sw = active ? gauss2(sx, sy, s_rx, s_ry) : 0.f;
    float ssum = block_sum(sw, scratch);
    sw /= ssum;
    float w = active ? copysignf(cw, k) - copysignf(sw, k) : 0.f;
    float wsum = block_sum(fabsf(w), scratch);
    if (active) A.SW[(size_t)cell * nSample + tid] = w / wsum;
    if (tid == 0) {
        A.maxConvol[id] = fabsf(k) * wsum;
        A.absk[cell] = fabsf(k);
    }
    // texture coordinates, center orientation
    const float coso = cosf(c_orient), sino = sinf(c_orient);
    const bool left = cell < A.nMagno_I;
    const float x0 = left ? A.L_x0 : A.R_x0;
    const float y0 = left ? A.L_y0 : A.R_y0;
    if (A.flat) {
        float x = x0 + (cEcc * cosf(cPolar) + cx * coso - cy * sino) * A.normViewDistance;
        float y = y0 + (cEcc * sinf(cPolar) + cx * sino + cy * coso) * A.normViewDistance;
        if (active) {
            A.SC[(size_t)cell * nSample + tid] = x;
            A.SC[(size_t)A.nMagno * nSample + (size_t)cell * nSample + tid] = y;
        }
    } else if (tid == 0) {
        atomicOr(A.err, kErrBounds);  // curved-retina geometry is not built (host rejects it)
    }
}

// LGN generator seeding (logRand_init, src/coredynamics.cu:148-177): sequence id per cell,
// one discarded uniform, then the first -log(U).
__global__ void lgn_rng_init_kernel(curandStateMRG32k3a *state, float *lnl, float *ltr,
                                    unsigned long long seed, int n) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    curandStateMRG32k3a s;
    curand_init(seed, id, 0, &s);
    (void)curand_uniform(&s);
    lnl[id] = -logf(curand_uniform(&s));
    ltr[id] = 0.0f;
    state[id] = s;
}

// Intensity of one sample for a cone type (get_intensity, src/discrete_input_convol.cu:35-76).
__device__ __forceinline__ float intensity(int coneType, float x, float y, int layer,
                                           cudaTextureObject_t L, cudaTextureObject_t M,
                                           cudaTextureObject_t S) {
    switch (coneType) {
        case 0: return tex2DLayered<float>(L, x, y, layer);
        case 1: return tex2DLayered<float>(M, x, y, layer);
        case 2: return tex2DLayered<float>(S, x, y, layer);
        case 3: return (tex2DLayered<float>(L, x, y, layer) + tex2DLayered<float>(M, x, y, layer)) / 2.0f;
        case 4:
            return tex2DLayered<float>(L, x, y, layer) * 0.45436904f +
                   tex2DLayered<float>(M, x, y, layer) * 0.47353315f +
                   tex2DLayered<float>(S, x, y, layer) * 0.0720978f;
        default: return 0.0f;
    }
}

// Spatial stage, once per (frame, cell): mean luminance of the cell's samples (cone type 3),
// local contrast clip(I/mean - 1, +-1) and its DoG-weighted sum
// (src/discrete_input_convol.cu:1474-1532).  One warp per (cell, frame); the layered
// textures use hardware bilinear filtering, normalised coordinates and border addressing
// exactly as the reference's (src/patch.h:95-109).
__global__ void __launch_bounds__(256) lgn_spatial_kernel(
    cudaTextureObject_t texL, cudaTextureObject_t texM, cudaTextureObject_t texS,
    const float *__restrict__ SW, const float *__restrict__ SC, const int *__restrict__ coneType,
    int nMagno, int nSample, int layer0, int nLayer, int row0, float *__restrict__ S) {
    const int lane = threadIdx.x & 31;
    const int cell = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int li = blockIdx.y;
    if (cell >= nMagno || li >= nLayer) return;
    const int layer = layer0 + li;
    const float *sc_x = SC + (size_t)cell * nSample;
    const float *sc_y = SC + (size_t)nMagno * nSample + (size_t)cell * nSample;
    float sum = 0.f;
    for (int s = lane; s < nSample; s += 32) sum += intensity(3, sc_x[s], sc_y[s], layer, texL, texM, texS);
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    const float mean = sum / nSample;
    const int type = coneType[cell];
    float acc = 0.f;
    for (int s = lane; s < nSample; s += 32) {
        float I = intensity(type, sc_x[s], sc_y[s], layer, texL, texM, texS);
        float c;
        if (mean > 0) c = I / mean - 1.0f;
        else c = I;
        if (fabsf(c) > 1.0f) c = copysignf(1.0f, c);
        acc += SW[(size_t)cell * nSample + s] * c;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) S[(size_t)(row0 + li) * nMagno + cell] = acc;
}

// Row of S held by the texture layer `x` positions after the newest frame's layer at step it.
// The reference keeps the last maxFrame frames in a layered texture (frame F in layer
// F % maxFrame, never-written layers hold the initial luminance) and indexes it from the
// window tail (src/patch.cu:5395-5412, 6052-6104).
__device__ __forceinline__ int frame_row(const FrameSched &fs, int currentFrame, int x) {
    int back = (fs.maxFrame - (x % fs.maxFrame)) % fs.maxFrame;
    int F = currentFrame - 1 - back;
    if (F < 0) return fs.initRow;
    return F % fs.nFrame;
}

// Number of the stimulus frame held by that layer (negative: the initial luminance).
__device__ __forceinline__ int frame_number(const FrameSched &fs, int currentFrame, int x) {
    int back = (fs.maxFrame - (x % fs.maxFrame)) % fs.maxFrame;
    return currentFrame - 1 - back;
}

constexpr int kClassCta = 128;

// The whole LGN step for a chunk of K steps when every magno cell has the same temporal
// weights (one temporal kernel class): the window segment weights W[s][q] (differences of the
// shared cumulative weights) and the frame slot of every segment are computed once per CTA;
// each thread (one cell) stages the S values of the chunk's frames in shared memory, then for
// each step contracts them with W, applies the logistic rate and draws the Poisson spikes.
// The arithmetic per (cell, step) is the one of lgn_rate_kernel + lgn_spike_kernel: same
// segment weights, same summation order, same generator calls.
__device__ __forceinline__ void lgn_class_body(const LgnParams &P, long long t0, int K, int cellBase) {
    extern __shared__ float sS[];                       // [kClassMaxSlots][kClassCta]
    __shared__ float sW[kClassMaxK][kClassMaxSeg];
    __shared__ unsigned char sSlot[kClassMaxK][kClassMaxSeg];
    __shared__ int sNseg[kClassMaxK];
    __shared__ int sFlo, sNU;
    const FrameSched fs = P.fs;
    if (threadIdx.x == 0) {
        const int cf0 = frames_read_after_step(fs, t0);
        const int ph0 = (int)((fs.magnoComp + (t0 + 1) * (long long)fs.denorm) % fs.ntPerFrame);
        const int te0 = fs.frameOffset + (ph0 <= fs.magnoComp ? 2 : 1);
        sFlo = frame_number(fs, cf0, te0 + P.seg.rel[(size_t)ph0 * P.seg.maxSeg]);
        const long long t1 = t0 + K - 1;
        const int cf1 = frames_read_after_step(fs, t1);
        const int ph1 = (int)((fs.magnoComp + (t1 + 1) * (long long)fs.denorm) % fs.ntPerFrame);
        const int te1 = fs.frameOffset + (ph1 <= fs.magnoComp ? 2 : 1);
        const int n1 = P.seg.nseg[ph1];
        const int Fhi = frame_number(fs, cf1, te1 + P.seg.rel[(size_t)ph1 * P.seg.maxSeg + n1 - 1]);
        sNU = Fhi - sFlo + 1;
        if (sNU > kClassMaxSlots || sNU < 1) atomicOr(P.err, kErrBounds);
    }
    __syncthreads();
    const int Flo = sFlo, nU = min(max(sNU, 1), kClassMaxSlots);
    for (int s = threadIdx.x; s < K; s += blockDim.x) {
        const long long it = t0 + s;
        const int cf = frames_read_after_step(fs, it);
        const int phase = (int)((fs.magnoComp + (it + 1) * (long long)fs.denorm) % fs.ntPerFrame);
        const int te = fs.frameOffset + (phase <= fs.magnoComp ? 2 : 1);
        const int nseg = P.seg.nseg[phase];
        sNseg[s] = nseg;
        const int *rel = P.seg.rel + (size_t)phase * P.seg.maxSeg;
        const int *j0 = P.seg.j0 + (size_t)phase * (P.seg.maxSeg + 1);
        double ca = P.classCtw[j0[0]];
        for (int q = 0; q < nseg; q++) {
            const double cb = P.classCtw[j0[q + 1]];
            sW[s][q] = (float)(cb - ca);
            ca = cb;
            const int slot = frame_number(fs, cf, te + rel[q]) - Flo;
            sSlot[s][q] = (unsigned char)min(max(slot, 0), kClassMaxSlots - 1);
        }
    }
    const int cell = cellBase + threadIdx.x;
    const bool on = cell < P.nMagno;
    if (on) {
        for (int u = 0; u < nU; u++) {
            const int F = Flo + u;
            const int row = F < 0 ? fs.initRow : F % fs.nFrame;
            sS[u * kClassCta + threadIdx.x] = __ldg(P.S + (size_t)row * P.nMagno + cell);
        }
    }
    __syncthreads();
    if (!on) return;
    int id = P.nParvo_I + cell;
    if (cell >= P.nMagno_I) id += P.nParvo_C;
    const float absk = P.absk[cell];
    const float mx = P.maxConvol[id];
    const float C50 = P.c50[id], Kc = P.sharp[id], LA = P.la[id], LB = P.lb[id];
    float ltr = P.leftTimeRate[id];
    float lnl = P.lastNegLogRand[id];
    curandStateMRG32k3a st = P.state[id];
    const float dt = P.dt;
    for (int s = 0; s < K; s++) {
        const long long it = t0 + s;
        float convol = 0.f;
        const int nseg = sNseg[s];
        for (int q = 0; q < nseg; q++) convol += sS[sSlot[s][q] * kClassCta + threadIdx.x] * sW[s][q];
        // LGN_nonlinear (src/discrete_input_convol.cu:1660-1730)
        float current = (convol * absk) * P.convolRatio;
        if (current < 0) current = 0;
        const float X = (float)(1.0 / (double)(1 + expf(Kc * (C50 - current / mx))));
        const float fr = P.frRatio * mx * (LA * X + LB);
        if (P.outFr) P.outFr[(size_t)(it % P.outSlots) * P.nLGN + id] = fr;
        // get_spike (src/discrete_input_convol.cu:1589-1619)
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
                if (P.recU) {
                    const long long rs = it - P.recStep0;
                    if (rs >= 0 && rs < P.recSteps) {
                        const size_t base = (size_t)rs * P.nLGN + id;
                        if ((int)nsp < P.recCap) P.recU[base * P.recCap + nsp] = u;
                        else atomicOr(P.err, kErrRecordOverflow);
                        P.recUCount[base] = nsp + 1;
                    }
                }
                lnl = fmaxf(-logf(u), 0.0f * rate);
                old_rT = next_rT;
                next_rT += lnl;
                nsp++;
            } while (next_rT <= rT);
            ltr = rT - old_rT;
            tsp = old_rT / (rate * nsp);
        }
        P.outSInfo[(size_t)(it % P.outSlots) * P.nLGN + id] = nsp + tsp / dt;
    }
    P.leftTimeRate[id] = ltr;
    P.lastNegLogRand[id] = lnl;
    P.state[id] = st;
}

__global__ void __launch_bounds__(kClassCta) lgn_class_kernel(LgnParams P, const long long *stepBase, int K) {
    lgn_class_body(P, *stepBase, K, blockIdx.x * kClassCta);
}

// The single-class LGN chunk for every trial of a batch: grid (cell CTAs, trials); each CTA
// copies its trial's parameters to shared memory and runs the same body for the steps the
// trial still has in this chunk.
__global__ void __launch_bounds__(kClassCta) lgn_class_batch_kernel(const BatchLgn *__restrict__ trials, int K) {
    __shared__ __align__(16) BatchLgn sT;
    const int *src = reinterpret_cast<const int *>(trials + blockIdx.y);
    int *dst = reinterpret_cast<int *>(&sT);
    for (int w = threadIdx.x; w < (int)(sizeof(BatchLgn) / sizeof(int)); w += kClassCta) dst[w] = src[w];
    __syncthreads();
    const long long t0 = *sT.step;
    const long long left = sT.tEnd - t0;
    const int k = left < K ? (int)left : K;
    if (k <= 0 || (int)blockIdx.x * kClassCta >= sT.p.nMagno) return;
    lgn_class_body(sT.p, t0, k, blockIdx.x * kClassCta);
}

// Temporal contraction and logistic rate for (cell, step) pairs of a chunk of K steps: grid
// (cells/256, K).  The frame rows and sample ranges of the step's window segments are
// computed once per CTA into shared memory; each thread then sums, over ~33 segments,
// S[row][cell] times the segment's sum of temporal weights (a difference of the cumulative
// weights), reading both tables cell-contiguously.  Rates go to rate[s][cell].
__global__ void __launch_bounds__(256) lgn_rate_kernel(LgnParams P, const long long *stepBase) {
    __shared__ int s_row[kMaxSeg];
    __shared__ int s_j[kMaxSeg + 1];
    const int s = blockIdx.y;
    const long long it = *stepBase + s;
    const FrameSched fs = P.fs;
    // window tail for step it (phases advance before the convolution, src/patch.cu:6052-6055)
    const int currentFrame = frames_read_after_step(fs, it);
    const int phase = (int)((fs.magnoComp + (it + 1) * (long long)fs.denorm) % fs.ntPerFrame);
    const int tailExtra = fs.frameOffset + (phase <= fs.magnoComp ? 2 : 1);
    const int nseg = P.seg.nseg[phase];
    if (threadIdx.x < nseg) {
        s_row[threadIdx.x] = frame_row(fs, currentFrame, tailExtra + P.seg.rel[(size_t)phase * P.seg.maxSeg + threadIdx.x]);
    }
    if (threadIdx.x <= nseg) s_j[threadIdx.x] = P.seg.j0[(size_t)phase * (P.seg.maxSeg + 1) + threadIdx.x];
    __syncthreads();
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= P.nMagno) return;
    int id = P.nParvo_I + cell;
    if (cell >= P.nMagno_I) id += P.nParvo_C;
    const double *__restrict__ ctw = P.ctw + cell;
    const float *__restrict__ S = P.S + cell;
    const size_t nm = P.nMagno;
    float convol = 0.f;
    double ca = ctw[(size_t)s_j[0] * nm];
#pragma unroll 4
    for (int q = 0; q < nseg; q++) {
        const double cb = ctw[(size_t)s_j[q + 1] * nm];
        const float wseg = (float)(cb - ca);
        convol += S[(size_t)s_row[q] * nm] * wseg;
        ca = cb;
    }
    // LGN_nonlinear (src/discrete_input_convol.cu:1660-1730)
    const float mx = P.maxConvol[id];
    float current = (convol * P.absk[cell]) * P.convolRatio;
    if (current < 0) current = 0;
    const float X = (float)(1.0 / (double)(1 + expf(P.sharp[id] * (P.c50[id] - current / mx))));
    const float fr = P.frRatio * mx * (P.la[id] * X + P.lb[id]);
    P.rate[(size_t)s * P.nLGN + id] = fr;
    if (P.outFr) P.outFr[(size_t)(it % P.outSlots) * P.nLGN + id] = fr;
}

// Exact-time Poisson spikes for K consecutive steps; one thread per magno cell carries the
// rate integral and its generator across the steps in registers (get_spike,
// src/discrete_input_convol.cu:1589-1619, and the write-back of :1750-1771).
__global__ void __launch_bounds__(256) lgn_spike_kernel(LgnParams P, const long long *stepBase, int K) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= P.nMagno) return;
    int id = P.nParvo_I + cell;
    if (cell >= P.nMagno_I) id += P.nParvo_C;
    float ltr = P.leftTimeRate[id];
    float lnl = P.lastNegLogRand[id];
    curandStateMRG32k3a st = P.state[id];
    const float dt = P.dt;
    const long long step0 = *stepBase;
    for (int s = 0; s < K; s++) {
        const long long it = step0 + s;
        const float fr = P.rate[(size_t)s * P.nLGN + id];
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
                float u = curand_uniform(&st);
                if (P.recU) {
                    long long rs = it - P.recStep0;
                    if (rs >= 0 && rs < P.recSteps) {
                        size_t base = (size_t)rs * P.nLGN + id;
                        if ((int)nsp < P.recCap) P.recU[base * P.recCap + nsp] = u;
                        else atomicOr(P.err, kErrRecordOverflow);
                        P.recUCount[base] = nsp + 1;
                    }
                }
                lnl = fmaxf(-logf(u), 0.0f * rate);
                old_rT = next_rT;
                next_rT += lnl;
                nsp++;
            } while (next_rT <= rT);
            ltr = rT - old_rT;
            tsp = old_rT / (rate * nsp);
        }
        const float sInfo = nsp + tsp / dt;
        P.outSInfo[(size_t)(it % P.outSlots) * P.nLGN + id] = sInfo;
    }
    P.leftTimeRate[id] = ltr;
    P.lastNegLogRand[id] = lnl;
    P.state[id] = st;
}

}  // namespace pv1

// ---- launchers used by the host runtime ---------------------------------------------
namespace pv1 {

cudaError_t launch_lgn_setup(const SetupArgs &a, int blockThreads, cudaStream_t st) {
    lgn_setup_kernel<<<a.nMagno, blockThreads, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_lgn_rng_init(curandStateMRG32k3a *state, float *lnl, float *ltr,
                                unsigned long long seed, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    lgn_rng_init_kernel<<<(n + 255) / 256, 256, 0, st>>>(state, lnl, ltr, seed, n);
    return cudaGetLastError();
}

cudaError_t launch_lgn_spatial(cudaTextureObject_t L, cudaTextureObject_t M, cudaTextureObject_t S,
                               const float *SW, const float *SC, const int *coneType, int nMagno,
                               int nSample, int layer0, int nLayer, int row0, float *out,
                               cudaStream_t st) {
    dim3 grid((nMagno + 7) / 8, nLayer);
    lgn_spatial_kernel<<<grid, 256, 0, st>>>(L, M, S, SW, SC, coneType, nMagno, nSample, layer0,
                                             nLayer, row0, out);
    return cudaGetLastError();
}

cudaError_t launch_lgn_rate_only(const LgnParams &p, const long long *stepBase, int K, cudaStream_t st) {
    if (p.nMagno <= 0) return cudaSuccess;
    dim3 grid((p.nMagno + 255) / 256, K);
    lgn_rate_kernel<<<grid, 256, 0, st>>>(p, stepBase);
    return cudaGetLastError();
}

cudaError_t launch_lgn_step(const LgnParams &p, const long long *stepBase, int K, cudaStream_t st) {
    if (p.nMagno <= 0) return cudaSuccess;
    if (p.classCtw && K <= kClassMaxK) {
        const size_t smem = (size_t)kClassMaxSlots * kClassCta * sizeof(float);
        static bool attrSet = false;
        if (!attrSet) {
            cudaError_t e = cudaFuncSetAttribute(lgn_class_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            attrSet = true;
        }
        lgn_class_kernel<<<(p.nMagno + kClassCta - 1) / kClassCta, kClassCta, smem, st>>>(p, stepBase, K);
        return cudaGetLastError();
    }
    dim3 grid((p.nMagno + 255) / 256, K);
    lgn_rate_kernel<<<grid, 256, 0, st>>>(p, stepBase);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    lgn_spike_kernel<<<(p.nMagno + 255) / 256, 256, 0, st>>>(p, stepBase, K);
    return cudaGetLastError();
}

cudaError_t launch_lgn_class_batch(const BatchLgn *trials, int nTrials, int maxCellCtas, int K, cudaStream_t st) {
    if (nTrials <= 0 || maxCellCtas <= 0) return cudaSuccess;
    if (K > kClassMaxK) return cudaErrorInvalidValue;
    const size_t smem = (size_t)kClassMaxSlots * kClassCta * sizeof(float);
    static bool attrSet = false;
    if (!attrSet) {
        cudaError_t e = cudaFuncSetAttribute(lgn_class_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        attrSet = true;
    }
    lgn_class_batch_kernel<<<dim3(maxCellCtas, nTrials), kClassCta, smem, st>>>(trials, K);
    return cudaGetLastError();
}

}  // namespace pv1
