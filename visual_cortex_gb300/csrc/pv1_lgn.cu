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


constexpr double kSqrt2 = 1.4142135623730951;   // SQRT2 of src/CONST.h:30

// Span of a Gaussian's sample grid: nsig * r / SQRT2 with the float product promoted to double
// for the division, as the reference's expression evaluates.
__device__ __forceinline__ float sample_span(float nsig, float r) {
    return (float)((double)(nsig * r) / kSqrt2);
}

// Sample coordinate (i + 0.5) * d - span, evaluated in double as the reference's
// `(threadIdx.x + 0.5)*dw - wSpan` is, then rounded once.
__device__ __forceinline__ float grid_coord(int i, float d, float span) {
    return (float)(((double)i + 0.5) * (double)d - (double)span);
}



// ---- curved-retina geometry (flat_retina = 0): sample points on the eye's sphere projected
// to the stimulus plane, as orthPhiRotate3D, axisRotate3D and retina_to_plane
// (src/discrete_input_convol.cuh:200-326) compute them in single precision ----

// The point at angle eta off the meridian through (theta, phi), orthogonal to it: its polar
// angle (cos, sin) and its eccentricity (cos, sin).
__device__ __forceinline__ void orth_phi_rotate(float theta, float phi, float eta, float &cost, float &sint,
                                                float &cosPhi, float &sinPhi) {
    const float tan_eta = tanf(eta);
    const float sin_phi = sinf(phi);
    const float r = sqrtf(tan_eta * tan_eta + sin_phi * sin_phi);
    cosPhi = cosf(eta) * cosf(phi);
    sinPhi = r;
    float cost1 = sin_phi / r, sint1 = tan_eta / r;
    if (fabsf(sint1) > 1.0f) sint1 = copysignf(sqrtf(1 - cost1 * cost1), sint1);
    if (fabsf(cost1) > 1.0f) cost1 = copysignf(sqrtf(1 - sint1 * sint1), cost1);
    const float cost0 = cosf(theta), sint0 = sinf(theta);
    cost = cost0 * cost1 - sint0 * sint1;
    sint = sint0 * cost1 + cost0 * sint1;
    if (fabsf(sint) > 1.0f) sint = copysignf(sqrtf(1 - cost * cost), sint);
    if (fabsf(cost) > 1.0f) cost = copysignf(sqrtf(1 - sint * sint), cost);
}

// Rotation of the point (polar cos/sin, eccentricity cos/sin) by (ceta, seta) about the axis
// through (theta0, phi0); returns the new polar angle's cos/sin and tan(eccentricity).
__device__ __forceinline__ void axis_rotate(float theta0, float phi0, float ceta, float seta, float &cost, float &sint,
                                            float cosPhi, float sinPhi, float &tanPhi) {
    const float sinPhi0 = sinf(phi0);
    const float x_rot = sinPhi0 * sinf(theta0);
    const float y_rot = sinPhi0 * cosf(theta0);
    const float z_rot = cosf(phi0);
    const float x = sinPhi * sint, y = sinPhi * cost, z = cosPhi;
    const float z_prime = (z_rot * x_rot * (1 - ceta) + y_rot * seta) * x + (z_rot * y_rot * (1 - ceta) - x_rot * seta) * y +
                          (z_rot * z_rot * (1 - ceta) + ceta) * z;
    const float y_prime = (y_rot * x_rot * (1 - ceta) - z_rot * seta) * x + (y_rot * y_rot * (1 - ceta) + ceta) * y +
                          (y_rot * z_rot * (1 - ceta) + x_rot * seta) * z;
    const float x_prime = (x_rot * x_rot * (1 - ceta) + ceta) * x + (x_rot * y_rot * (1 - ceta) + z_rot * seta) * y +
                          (x_rot * z_rot * (1 - ceta) - y_rot * seta) * z;
    tanPhi = sqrtf(x_prime * x_prime + y_prime * y_prime) / z_prime;
    const float theta = atan2f(x_prime, y_prime);
    cost = cosf(theta);
    sint = sinf(theta);
}

// Texture coordinates of the sample at (w, h) in the frame of a Gaussian centred at
// (polar, ecc) with orientation (coso, sino) on a curved retina.
__device__ __forceinline__ void curved_sample(float polar, float ecc, float w, float h, float coso, float sino,
                                              float nvd, float x0, float y0, float &x, float &y) {
    float cosp, sinp, cosEcc, sinEcc, tanEcc;
    orth_phi_rotate(polar, ecc + h, w, cosp, sinp, cosEcc, sinEcc);
    axis_rotate(polar, ecc, coso, sino, cosp, sinp, cosEcc, sinEcc, tanEcc);
    const float r = tanEcc * nvd;
    x = x0 + r * cosp;
    y = y0 + r * sinp;
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
    float cx = grid_coord(tx, ds, span);
    float cy = grid_coord(ty, ds, span);
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
    float x, y;
    if (A.flat) {
        x = x0 + (cEcc * cosf(cPolar) + cx * coso - cy * sino) * A.normViewDistance;
        y = y0 + (cEcc * sinf(cPolar) + cx * sino + cy * coso) * A.normViewDistance;
    } else {
        curved_sample(cPolar, cEcc, cx, cy, coso, sino, A.normViewDistance, x0, y0, x, y);
    }
    if (active) {
        A.SC[(size_t)cell * nSample + tid] = x;
        A.SC[(size_t)A.nMagno * nSample + (size_t)cell * nSample + tid] = y;
    }
}

// ---- parvocellular cells ---------------------------------------------------------------

// One CTA per (parvo cell, component), one thread per spatial sample: store_PM with PM = 0
// (src/discrete_input_convol.cu:427-520) -- the component's temporal weights
// (store_temporalWeight :230-305, time reversed, L1 normalised), its texture coordinates on a
// (2 nsig r/sqrt2)^2 grid around its own centre (store_spatialWeight :309-425, flat retina)
// and, from the first cell's centre only, the normalised Gaussian SW every parvo cell shares.
__global__ void __launch_bounds__(1024) lgn_parvo_setup_kernel(ParvoSetupArgs A) {
    __shared__ float scratch[33];
    const int cell = blockIdx.x, type = blockIdx.y;
    const int tid = threadIdx.x;
    const int nSample = A.nSample, n1 = A.nSample1D, nKS = A.nKS;
    const int id = cell < A.nParvo_I ? cell : cell + A.nMagno_I;
    const int lid = type * A.nLGN + id;
    {
        const float tauR = A.tauR[lid], tauD = A.tauD[lid], nR = A.nR[lid], nD = A.nD[lid];
        const float ratio = A.ratio[lid];
        const float lfac1 = lgammaf(nR), lfac2 = lgammaf(nD);
        const float t0 = A.kernelSampleT0 - A.delay[lid];
        float *tw_row = A.TW + ((size_t)cell * 2 + type) * nKS;
        float local = 0.f;
        for (int j = tid; j < nKS; j += blockDim.x) {
            const int twid = nKS - 1 - j;
            const float t = twid * A.kernelSampleDt + t0;
            const float tw = t < 0 ? 0.0f : temporal_kernel(t, tauR, tauD, nR, nD, ratio, lfac1, lfac2);
            tw_row[j] = tw;
            local += fabsf(tw);
        }
        const float total = block_sum(local, scratch);
        for (int j = tid; j < nKS; j += blockDim.x) tw_row[j] /= total;
        __syncthreads();
        if (tid == 0) {
            double *c = A.pctw + (size_t)type * (nKS + 1) * A.nParvo + cell;
            double acc = 0.0;
            c[0] = 0.0;
            for (int j = 0; j < nKS; j++) {
                acc += (double)tw_row[j];
                c[(size_t)(j + 1) * A.nParvo] = acc;
            }
            A.pk[type * A.nParvo + cell] = A.k[lid];
        }
    }
    const float polar = A.polar[lid], ecc = A.ecc[lid];
    const float rx = A.rw[lid], ry = A.rh[lid];
    const float wSpan = sample_span(A.nsig, rx), hSpan = sample_span(A.nsig, ry);
    const float dw = 2 * wSpan / n1, dh = 2 * hSpan / n1;
    const bool active = tid < nSample;
    const int tx = tid % n1, ty = tid / n1;
    const float w = grid_coord(tx, dw, wSpan), h = grid_coord(ty, dh, hSpan);
    if (cell == 0 && type == 0) {
        const float sw = active ? gauss2(w, h, rx, ry) : 0.f;
        const float sum = block_sum(sw, scratch);
        if (active) A.SW[tid] = sw / sum;
    }
    const float coso = cosf(A.orient[lid]), sino = sinf(A.orient[lid]);
    const bool left = cell < A.nParvo_I;
    const float x0 = left ? A.L_x0 : A.R_x0, y0 = left ? A.L_y0 : A.R_y0;
    if (active) {
        float x, y;
        if (A.flat) {
            x = x0 + (ecc * cosf(polar) + w * coso - h * sino) * A.normViewDistance;
            y = y0 + (ecc * sinf(polar) + w * sino + h * coso) * A.normViewDistance;
        } else {
            curved_sample(polar, ecc, w, h, coso, sino, A.normViewDistance, x0, y0, x, y);
        }
        const size_t sid = ((size_t)cell * 2 + type) * nSample + tid;
        A.SC[sid] = x;
        A.SC[(size_t)A.nParvo * 2 * nSample + sid] = y;
    }
}

// max_convol of a parvo cell (parvo_maxConvol, src/discrete_input_convol.cu:748-883): centre
// and surround Gaussians sampled on one maxSample1D^2 grid around the surround, each
// normalised to unit sum, and the largest response a stimulus can drive through them, summed
// over the temporal samples: at every (sample, tap) the dominant component at full contrast
// plus the other one at the covariant fraction of it.  One CTA of 1024 threads per cell;
// (maxSample1D^2 / 1024) * 1024 samples take part, as in the reference.  The sum is kept in
// double per thread over the taps and reduced once (the reference reduces per tap in float).
__global__ void __launch_bounds__(1024) lgn_parvo_maxconvol_kernel(ParvoSetupArgs A) {
    extern __shared__ float swC[];
    __shared__ double dscratch[33];
    __shared__ float scratch[33];
    const int cell = blockIdx.x;
    const int id = cell < A.nParvo_I ? cell : cell + A.nMagno_I;
    const int sid = A.nLGN + id;
    const int n1 = A.maxSample1D;
    const int nPatch = (n1 * n1) / (int)blockDim.x;
    float *swS = swC + nPatch * blockDim.x;
    const float rxs = A.rw[sid], rys = A.rh[sid], xs = A.polar[sid], ys = A.ecc[sid];
    float wSpan = sample_span(A.nsig, rxs), hSpan = sample_span(A.nsig, rys);
    const float rxc = A.rw[id], ryc = A.rh[id];
    float R = wSpan > hSpan ? wSpan : hSpan;
    const float xc = A.polar[id], yc = A.ecc[id];
    wSpan = sample_span(A.nsig, rxc);
    hSpan = sample_span(A.nsig, ryc);
    const float dx = yc * cosf(xc) - ys * cosf(xs);
    const float dy = yc * sinf(xc) - ys * sinf(xs);
    float r = sqrtf(dx * dx + dy * dy);
    const float cov = A.covariant[id];
    r += wSpan > hSpan ? wSpan : hSpan;
    R = r > R ? r : R;
    const float coss = cosf(A.orient[sid]), sins = sinf(A.orient[sid]);
    const float cosc = cosf(A.orient[id]), sinc = sinf(A.orient[id]);
    const float ks = A.k[sid], kc = A.k[id];
    const float ds = 2 * R / n1;
    float sumC = 0.f, sumS = 0.f;
    for (int ip = 0; ip < nPatch; ip++) {
        const int pid = ip * blockDim.x + threadIdx.x;
        const float lx = grid_coord(pid % n1, ds, R), ly = grid_coord(pid / n1, ds, R);
        float x = cosc * (lx - dx) + sinc * (ly - dy);
        float y = -sinc * (lx - dx) + cosc * (ly - dy);
        const float c = gauss2(x, y, rxc, ryc);
        swC[pid] = c;
        sumC += block_sum(c, scratch);
        x = coss * lx + sins * ly;
        y = -sins * lx + coss * ly;
        const float s = gauss2(x, y, rxs, rys);
        swS[pid] = s;
        sumS += block_sum(s, scratch);
    }
    __syncthreads();
    for (int ip = 0; ip < nPatch; ip++) {
        const int pid = ip * blockDim.x + threadIdx.x;
        swC[pid] /= sumC;
        swS[pid] /= sumS;
    }
    __syncthreads();
    const float *twC = A.TW + (size_t)cell * 2 * A.nKS, *twS = twC + A.nKS;
    double acc = 0.0;
    for (int it = 0; it < A.nKS; it++) {
        const float tc = twC[it], ts = twS[it];
        for (int ip = 0; ip < nPatch; ip++) {
            const int pid = ip * blockDim.x + threadIdx.x;
            const float lc = swC[pid] * tc * kc;
            const float ls = swS[pid] * ts * ks;
            float decide;
            if (fabsf(lc) > fabsf(ls)) decide = fabsf(lc) + ls * copysignf(cov, lc);
            else decide = fabsf(ls) + lc * copysignf(cov, ls);
            acc += (double)decide;
        }
    }
    // block sum in double
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) dscratch[warp] = acc;
    __syncthreads();
    if (warp == 0) {
        double t = lane < (int)(blockDim.x >> 5) ? dscratch[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) A.maxConvol[id] = (float)t;
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

constexpr int kSpatialReg = 8;   // samples per lane held in registers by the spatial stage

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
    if (cell >= nMagno) return;
    const float *sc_x = SC + (size_t)cell * nSample;
    const float *sc_y = SC + (size_t)nMagno * nSample + (size_t)cell * nSample;
    const int type = coneType[cell];
    // the cell's sample coordinates and weights, loaded once for all the layers of the launch
    float X[kSpatialReg], Y[kSpatialReg], Wt[kSpatialReg];
    if (nSample <= 32 * kSpatialReg) {
#pragma unroll
        for (int k = 0; k < kSpatialReg; k++) {
            const int s = lane + 32 * k;
            X[k] = s < nSample ? sc_x[s] : 0.f;
            Y[k] = s < nSample ? sc_y[s] : 0.f;
            Wt[k] = s < nSample ? SW[(size_t)cell * nSample + s] : 0.f;
        }
    }
    for (int li = blockIdx.y; li < nLayer; li += gridDim.y) {
    const int layer = layer0 + li;
    float sum = 0.f, acc = 0.f;
    if (nSample <= 32 * kSpatialReg) {
        // each texel is fetched once: the cell's intensities stay in registers between the mean
        // and the contrast pass (same values as fetching them twice)
        float Iv[kSpatialReg];
#pragma unroll
        for (int k = 0; k < kSpatialReg; k++) {
            const int s = lane + 32 * k;
            Iv[k] = 0.f;
            if (s < nSample) {
                const float x = X[k], y = Y[k];
                const float L = tex2DLayered<float>(texL, x, y, layer), M = tex2DLayered<float>(texM, x, y, layer);
                sum += (L + M) / 2.0f;
                if (type == 3) Iv[k] = (L + M) / 2.0f;
                else if (type == 0) Iv[k] = L;
                else if (type == 1) Iv[k] = M;
                else if (type == 2) Iv[k] = tex2DLayered<float>(texS, x, y, layer);
                else if (type == 4) Iv[k] = L * 0.45436904f + M * 0.47353315f + tex2DLayered<float>(texS, x, y, layer) * 0.0720978f;
            }
        }
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        const float mean = sum / nSample;
#pragma unroll
        for (int k = 0; k < kSpatialReg; k++) {
            const int s = lane + 32 * k;
            if (s < nSample) {
                float c;
                if (mean > 0) c = Iv[k] / mean - 1.0f;
                else c = Iv[k];
                if (fabsf(c) > 1.0f) c = copysignf(1.0f, c);
                acc += Wt[k] * c;
            }
        }
    } else {
        for (int s = lane; s < nSample; s += 32) sum += intensity(3, sc_x[s], sc_y[s], layer, texL, texM, texS);
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        const float mean = sum / nSample;
        for (int s = lane; s < nSample; s += 32) {
            float I = intensity(type, sc_x[s], sc_y[s], layer, texL, texM, texS);
            float c;
            if (mean > 0) c = I / mean - 1.0f;
            else c = I;
            if (fabsf(c) > 1.0f) c = copysignf(1.0f, c);
            acc += SW[(size_t)cell * nSample + s] * c;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) S[(size_t)(row0 + li) * nMagno + cell] = acc;
    }
}

// Parvo spatial stage, once per (frame, cell): the mean luminances of the centre and the
// surround cone types -- both sampled at the surround's coordinates, as
// src/discrete_input_convol.cu:1034-1035 reads them -- then the clipped local contrast of
// each component at its own coordinates, weighted by the shared Gaussian SW and summed
// (:1151-1209).  One warp per (cell, frame).  PS [row][2][nParvo].
__global__ void __launch_bounds__(256) lgn_parvo_spatial_kernel(
    cudaTextureObject_t texL, cudaTextureObject_t texM, cudaTextureObject_t texS,
    const float *__restrict__ SW, const float *__restrict__ SC, const int *__restrict__ coneType,
    int nParvo, int nSample, int layer0, int nLayer, int row0, float *__restrict__ PS) {
    const int lane = threadIdx.x & 31;
    const int cell = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int li = blockIdx.y;
    if (cell >= nParvo || li >= nLayer) return;
    const int layer = layer0 + li;
    const size_t yOff = (size_t)nParvo * 2 * nSample;
    const float *xC = SC + (size_t)cell * 2 * nSample, *yC = xC + yOff;
    const float *xS = xC + nSample, *yS = xS + yOff;
    const int typeC = coneType[cell], typeS = coneType[nParvo + cell];
    // the surround's intensities at its own coordinates serve its mean and its contrast: kept
    // in registers between the two passes when the sample grid is small enough
    const bool keep = nSample <= 32 * kSpatialReg;
    float IS[kSpatialReg];
    float sumC = 0.f, sumS = 0.f;
#pragma unroll
    for (int k = 0; k < kSpatialReg; k++) IS[k] = 0.f;
    for (int s = lane, k = 0; s < nSample; s += 32, k++) {
        sumC += intensity(typeC, xS[s], yS[s], layer, texL, texM, texS);
        const float I = intensity(typeS, xS[s], yS[s], layer, texL, texM, texS);
        sumS += I;
        if (keep) {
#pragma unroll
            for (int q = 0; q < kSpatialReg; q++)
                if (q == k) IS[q] = I;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        sumC += __shfl_xor_sync(0xffffffffu, sumC, o);
        sumS += __shfl_xor_sync(0xffffffffu, sumS, o);
    }
    const float meanC = sumC / nSample, meanS = sumS / nSample;
    float accC = 0.f, accS = 0.f;
    for (int s = lane, k = 0; s < nSample; s += 32, k++) {
        const float sw = SW[s];
        float I = intensity(typeC, xC[s], yC[s], layer, texL, texM, texS);
        float c = meanC > 0 ? I / meanC - 1.0f : I;
        if (fabsf(c) > 1.0f) c = copysignf(1.0f, c);
        accC += sw * c;
        if (keep) {
            I = 0.f;
#pragma unroll
            for (int q = 0; q < kSpatialReg; q++)
                if (q == k) I = IS[q];
        } else {
            I = intensity(typeS, xS[s], yS[s], layer, texL, texM, texS);
        }
        c = meanS > 0 ? I / meanS - 1.0f : I;
        if (fabsf(c) > 1.0f) c = copysignf(1.0f, c);
        accS += sw * c;
    }
    for (int o = 16; o > 0; o >>= 1) {
        accC += __shfl_xor_sync(0xffffffffu, accC, o);
        accS += __shfl_xor_sync(0xffffffffu, accS, o);
    }
    if (lane == 0) {
        PS[((size_t)(row0 + li) * 2 + 0) * nParvo + cell] = accC;
        PS[((size_t)(row0 + li) * 2 + 1) * nParvo + cell] = accS;
    }
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

// Presynaptic LTP traces of LGN cell id over step it (LGN_nonlinear with learning 1-3,
// src/discrete_input_convol.cu:1774-1808), one per learning type (FF->E, then FF->I), each with
// its own tauLTP: the value at the start of the step and, when the cell spiked, the value right
// after its spikes (the spike count added, then decayed from the step start to the spike time
// tsp) go to the step's row of outPre; var leaves decayed to the end of the step.
__device__ __forceinline__ void ff_pre_step(const LgnParams &P, long long it, int id, unsigned nsp, float tsp,
                                            float sInfo, float *var) {
    float *row = P.outPre + (size_t)(it % P.outSlots) * P.nFF * 2 * P.nLGN;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        if (k < P.nFF) {
            float *r = row + (size_t)k * 2 * P.nLGN;
            r[id] = var[k];
            float delta_t;
            if (sInfo > 0) {
                delta_t = tsp;
                var[k] += (float)nsp;
                var[k] *= expf(-delta_t / P.tauLTP[k]);
                r[P.nLGN + id] = var[k];
                delta_t = P.dt - delta_t;
            } else {
                delta_t = P.dt;
            }
            var[k] *= expf(-delta_t / P.tauLTP[k]);
        }
    }
}



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
    float ffVar[2] = {P.nFF > 0 ? P.ffPre[id] : 0.f, P.nFF > 1 ? P.ffPre[(size_t)P.nLGN + id] : 0.f};
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
        const float sInfo = nsp + tsp / dt;
        P.outSInfo[(size_t)(it % P.outSlots) * P.nLGN + id] = sInfo;
        if (P.nFF) ff_pre_step(P, it, id, nsp, tsp, sInfo, ffVar);
    }
    P.leftTimeRate[id] = ltr;
    P.lastNegLogRand[id] = lnl;
    P.state[id] = st;
    if (P.nFF > 0) P.ffPre[id] = ffVar[0];
    if (P.nFF > 1) P.ffPre[(size_t)P.nLGN + id] = ffVar[1];
}

__global__ void __launch_bounds__(kClassCta) lgn_class_kernel(LgnParams P, const long long *stepBase, int K) {
    lgn_class_body(P, *stepBase, K, blockIdx.x * kClassCta);
}

// The single-class LGN stage for every trial of a batch: grid (cell CTAs, trials); each CTA
// copies its trial's parameters to shared memory and runs the same body for the steps the
// trial still has among the next K (in pieces of at most kClassMaxK steps).
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
    // chunks of at most kClassMaxK steps (the shared tables of one chunk's frames); the cells'
    // carried state passes from one chunk to the next through global memory
    for (int off = 0; off < k; off += kClassMaxK) {
        if (off) __syncthreads();
        lgn_class_body(sT.p, t0 + off, min(kClassMaxK, k - off), blockIdx.x * kClassCta);
    }
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

// Parvo temporal contraction and logistic rate for (cell, step) pairs of a chunk of K steps:
// LGN_convol_parvo's sum over the window's samples of (centre contrast x centre weight) and
// (surround contrast x surround weight), times k of each (src/discrete_input_convol.cu:
// 1143-1327), on the parvo kernel grid (nKernelSample, interval, T0) and the parvo frame tail
// (getTail with parvoComp and (1-pLongerThanM)*dFrame, src/patch.cu:5399-5422, 6068), then
// LGN_nonlinear's rate.  Same segment form as lgn_rate_kernel.
__global__ void __launch_bounds__(256) lgn_parvo_rate_kernel(LgnParams P, const long long *stepBase) {
    __shared__ int s_row[kMaxSeg];
    __shared__ int s_j[kMaxSeg + 1];
    const int s = blockIdx.y;
    const long long it = *stepBase + s;
    const FrameSched fs = P.fs;
    const int currentFrame = frames_read_after_step(fs, it);
    const int phase = (int)((P.parvoComp + (it + 1) * (long long)fs.denorm) % fs.ntPerFrame);
    const int tailExtra = P.pFrameOffset + (phase <= P.parvoComp ? 2 : 1);
    const int nseg = P.pseg.nseg[phase];
    if (threadIdx.x < nseg)
        s_row[threadIdx.x] = frame_row(fs, currentFrame, tailExtra + P.pseg.rel[(size_t)phase * P.pseg.maxSeg + threadIdx.x]);
    if (threadIdx.x <= nseg) s_j[threadIdx.x] = P.pseg.j0[(size_t)phase * (P.pseg.maxSeg + 1) + threadIdx.x];
    __syncthreads();
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= P.nParvo) return;
    const int id = cell < P.nParvo_I ? cell : cell + P.nMagno_I;
    const size_t np = P.nParvo;
    const double *__restrict__ ctwC = P.pctw + cell;
    const double *__restrict__ ctwS = ctwC + (size_t)(P.pKS + 1) * np;
    const float *__restrict__ S = P.pS + cell;
    float convolC = 0.f, convolS = 0.f;
    double caC = ctwC[(size_t)s_j[0] * np], caS = ctwS[(size_t)s_j[0] * np];
#pragma unroll 2
    for (int q = 0; q < nseg; q++) {
        const double cbC = ctwC[(size_t)s_j[q + 1] * np], cbS = ctwS[(size_t)s_j[q + 1] * np];
        const size_t row = (size_t)s_row[q] * 2 * np;
        convolC += S[row] * (float)(cbC - caC);
        convolS += S[row + np] * (float)(cbS - caS);
        caC = cbC;
        caS = cbS;
    }
    const float convol = convolC * P.pk[cell] + convolS * P.pk[np + cell];
    // LGN_nonlinear (src/discrete_input_convol.cu:1660-1730)
    const float mx = P.maxConvol[id];
    float current = convol * P.convolRatio;
    if (current < 0) current = 0;
    const float X = (float)(1.0 / (double)(1 + expf(P.sharp[id] * (P.c50[id] - current / mx))));
    const float fr = P.frRatio * mx * (P.la[id] * X + P.lb[id]);
    P.rate[(size_t)s * P.nLGN + id] = fr;
    if (P.outFr) P.outFr[(size_t)(it % P.outSlots) * P.nLGN + id] = fr;
}

// Exact-time Poisson spikes for K consecutive steps; one thread per cell carries the rate
// integral and its generator across the steps in registers (get_spike,
// src/discrete_input_convol.cu:1589-1619, and the write-back of :1750-1771).  blockIdx.y = 0:
// magno cells, 1: parvo cells.
__global__ void __launch_bounds__(256) lgn_spike_kernel(LgnParams P, const long long *stepBase, int K) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    int id;
    if (blockIdx.y == 0) {
        if (cell >= P.nMagno) return;
        id = P.nParvo_I + cell;
        if (cell >= P.nMagno_I) id += P.nParvo_C;
    } else {
        if (cell >= P.nParvo) return;
        id = cell < P.nParvo_I ? cell : cell + P.nMagno_I;
    }
    float ltr = P.leftTimeRate[id];
    float lnl = P.lastNegLogRand[id];
    curandStateMRG32k3a st = P.state[id];
    float ffVar[2] = {P.nFF > 0 ? P.ffPre[id] : 0.f, P.nFF > 1 ? P.ffPre[(size_t)P.nLGN + id] : 0.f};
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
        if (P.nFF) ff_pre_step(P, it, id, nsp, tsp, sInfo, ffVar);
    }
    P.leftTimeRate[id] = ltr;
    P.lastNegLogRand[id] = lnl;
    P.state[id] = st;
    if (P.nFF > 0) P.ffPre[id] = ffVar[0];
    if (P.nFF > 1) P.ffPre[(size_t)P.nLGN + id] = ffVar[1];
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
    // each warp runs its cell over up to 8 layers (the cell's coordinates and weights loaded once)
    dim3 grid((nMagno + 7) / 8, (nLayer + 7) / 8);
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

cudaError_t launch_parvo_setup(const ParvoSetupArgs &a, cudaStream_t st) {
    if (a.nParvo <= 0) return cudaSuccess;
    const int threads = ((a.nSample + 31) / 32) * 32;
    lgn_parvo_setup_kernel<<<dim3(a.nParvo, 2), threads, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int nPatch = a.maxSample1D * a.maxSample1D / 1024;
    const size_t smem = (size_t)2 * nPatch * 1024 * sizeof(float);
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(lgn_parvo_maxconvol_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    lgn_parvo_maxconvol_kernel<<<a.nParvo, 1024, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_parvo_spatial(cudaTextureObject_t L, cudaTextureObject_t M, cudaTextureObject_t S,
                                 const float *SW, const float *SC, const int *coneType, int nParvo,
                                 int nSample, int layer0, int nLayer, int row0, float *out, cudaStream_t st) {
    if (nParvo <= 0 || nLayer <= 0) return cudaSuccess;
    dim3 grid((nParvo + 7) / 8, nLayer);
    lgn_parvo_spatial_kernel<<<grid, 256, 0, st>>>(L, M, S, SW, SC, coneType, nParvo, nSample, layer0, nLayer, row0,
                                                   out);
    return cudaGetLastError();
}

int lgn_step_launches(const LgnParams &p, int K) {
    if (p.nParvo == 0) {
        if (p.nMagno <= 0) return 0;
        if (p.classCtw && K <= kClassMaxK) return 1;
        return 2;
    }
    return (p.nMagno > 0) + 2;
}

cudaError_t launch_lgn_step(const LgnParams &p, const long long *stepBase, int K, cudaStream_t st) {
    if (p.nParvo > 0) {
        cudaError_t e;
        if (p.nMagno > 0) {
            lgn_rate_kernel<<<dim3((p.nMagno + 255) / 256, K), 256, 0, st>>>(p, stepBase);
            e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        lgn_parvo_rate_kernel<<<dim3((p.nParvo + 255) / 256, K), 256, 0, st>>>(p, stepBase);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        const int n = std::max(p.nMagno, p.nParvo);
        lgn_spike_kernel<<<dim3((n + 255) / 256, 2), 256, 0, st>>>(p, stepBase, K);
        return cudaGetLastError();
    }
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
    if (K <= 0) return cudaErrorInvalidValue;
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
