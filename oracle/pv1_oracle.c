/*
 * pv1_oracle.c -- CPU restatement of the patchV1 simulation hot path.
 *
 * TEST INFRASTRUCTURE: this file is the oracle of the GPU library.  Only the tests, the
 * smoke check and the CPU-baseline leg of the benchmark load it; the product path never
 * does.  It follows the reference's own structure (one pass per kernel, per-synapse delay
 * rings for the far synapses, the sample-by-sample temporal convolution) rather than the GPU
 * design, so that agreement between the two is evidence about the algorithm and not about a
 * shared implementation.
 *
 * Reference files followed (paths relative to the reference project root):
 *   ConductanceShape               src/condShape.h:13-41
 *   AdEx / get_a / get_b           src/coredynamics.cuh:15-118
 *   compute_V_..._fast             src/coredynamics.cu:1235-2059
 *   recal_G_mat_nd_fast            src/coredynamics.cu:2609-2922
 *   recal_G_vec + fill_fSpikeTrain src/coredynamics.cu:181-372, src/stats.cu:114-126
 *   sum_G                          src/coredynamics.cu:2312-2349
 *   store_PM (magno) / TW          src/discrete_input_convol.cu:230-305, 427-744
 *   LGN_convol_magno               src/discrete_input_convol.cu:1342-1585
 *   store_PM (parvo), parvo_maxConvol, LGN_convol_parvo
 *                                  src/discrete_input_convol.cu:309-520, 748-883, 886-1340;
 *                                  sample-grid rule src/patch.cu:5266-5312
 *   LGN_nonlinear / get_spike      src/discrete_input_convol.cu:1587-1821
 *   transform / hStatic_nonlinear  src/LGN_props.cuh:94-100, src/LGN_props.h:143-170
 *   texture sampling               src/patch.h:95-109 (bilinear, normalised, border)
 *
 * Random numbers: the reference draws from cuRAND on the device.  This file does not
 * re-derive cuRAND; every draw it needs is passed in (recorded by the GPU run under test).
 * Build with -ffp-contract=off so the float arithmetic is the same on every host.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/patchv1_gb300.h"

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    float rise[PV1_MAX_NG], decay[PV1_MAX_NG], dod[PV1_MAX_NG];
} ocond;

static ocond ocond_make(const float *rt, const float *dc, int n) {
    ocond c;
    memset(&c, 0, sizeof(c));
    for (int i = 0; i < n; i++) {
        c.rise[i] = rt[i];
        c.decay[i] = dc[i];
        c.dod[i] = rt[i] / (dc[i] - rt[i]);
    }
    return c;
}

static inline void ocond_input(const ocond *c, float *g, float *h, float f, float dt, int ig) {
    float etr = expf(-dt / c->rise[ig]);
    *g += f * c->dod[ig] * (expf(-dt / c->decay[ig]) - etr);
    *h += f * etr;
}

static inline void ocond_decay(const ocond *c, float *g, float *h, float dt, int ig) {
    float etr = expf(-dt / c->rise[ig]);
    float etd = expf(-dt / c->decay[ig]);
    *g = *g * etd + *h * c->dod[ig] * (etd - etr);
    *h *= etr;
}

int orc_version(void) { return 1; }

/* ================================================================== LGN ============ */

static float gauss2(float x, float y, float rx, float ry) {
    return expf(-x * x / (rx * rx) - y * y / (ry * ry));
}

/* Curved retina (flat_retina = 0): orthPhiRotate3D, axisRotate3D and retina_to_plane of
 * src/discrete_input_convol.cuh:200-326, in single precision. */
static void orth_phi_rotate(float theta, float phi, float eta, float *cost, float *sint, float *cosPhi,
                            float *sinPhi) {
    const float tan_eta = tanf(eta), sin_phi = sinf(phi);
    const float r = sqrtf(tan_eta * tan_eta + sin_phi * sin_phi);
    *cosPhi = cosf(eta) * cosf(phi);
    *sinPhi = r;
    float cost1 = sin_phi / r, sint1 = tan_eta / r;
    if (fabsf(sint1) > 1.0f) sint1 = copysignf(sqrtf(1 - cost1 * cost1), sint1);
    if (fabsf(cost1) > 1.0f) cost1 = copysignf(sqrtf(1 - sint1 * sint1), cost1);
    const float cost0 = cosf(theta), sint0 = sinf(theta);
    float c = cost0 * cost1 - sint0 * sint1, sn = sint0 * cost1 + cost0 * sint1;
    if (fabsf(sn) > 1.0f) sn = copysignf(sqrtf(1 - c * c), sn);
    if (fabsf(c) > 1.0f) c = copysignf(sqrtf(1 - sn * sn), c);
    *cost = c;
    *sint = sn;
}

static void axis_rotate(float theta0, float phi0, float ceta, float seta, float *cost, float *sint, float cosPhi,
                        float sinPhi, float *tanPhi) {
    const float sinPhi0 = sinf(phi0);
    const float xr = sinPhi0 * sinf(theta0), yr = sinPhi0 * cosf(theta0), zr = cosf(phi0);
    const float x = sinPhi * *sint, y = sinPhi * *cost, z = cosPhi;
    const float zp = (zr * xr * (1 - ceta) + yr * seta) * x + (zr * yr * (1 - ceta) - xr * seta) * y +
                     (zr * zr * (1 - ceta) + ceta) * z;
    const float yp = (yr * xr * (1 - ceta) - zr * seta) * x + (yr * yr * (1 - ceta) + ceta) * y +
                     (yr * zr * (1 - ceta) + xr * seta) * z;
    const float xp = (xr * xr * (1 - ceta) + ceta) * x + (xr * yr * (1 - ceta) + zr * seta) * y +
                     (xr * zr * (1 - ceta) - yr * seta) * z;
    *tanPhi = sqrtf(xp * xp + yp * yp) / zp;
    const float theta = atan2f(xp, yp);
    *cost = cosf(theta);
    *sint = sinf(theta);
}

/* Texture coordinates of the sample (w, h) of a Gaussian centred at (polar, ecc) with
 * orientation (coso, sino): flat (a scaled plane) or curved (the sphere projected). */
static void sample_xy(int flat, float polar, float ecc, float w, float h, float coso, float sino, float nvd, float x0,
                      float y0, float *x, float *y) {
    if (flat) {
        *x = x0 + (ecc * cosf(polar) + w * coso - h * sino) * nvd;
        *y = y0 + (ecc * sinf(polar) + w * sino + h * coso) * nvd;
        return;
    }
    float cosp, sinp, cosEcc, sinEcc, tanEcc;
    orth_phi_rotate(polar, ecc + h, w, &cosp, &sinp, &cosEcc, &sinEcc);
    axis_rotate(polar, ecc, coso, sino, &cosp, &sinp, cosEcc, sinEcc, &tanEcc);
    const float r = tanEcc * nvd;
    *x = x0 + r * cosp;
    *y = y0 + r * sinp;
}

/* nsig * r / SQRT2: the float product divided in double (SQRT2, src/CONST.h:30). */
static float parvo_span(float nsig, float r) { return (float)((double)(nsig * r) / 1.4142135623730951); }
/* Sample coordinate (i + 0.5) * d - span in double, rounded once to float, as the
 * reference's `(threadIdx.x + 0.5)*ds - span` evaluates. */
static float grid_at(int i, float d, float span) { return (float)(((double)i + 0.5) * (double)d - (double)span); }

static float temporal_kernel(float tau, float tauR, float tauD, float nR, float nD, float ratio,
                             float lfac1, float lfac2) {
    float tau1 = tau / tauR, tau2 = tau / tauD;
    float A1 = (nR - 1) * logf(tau1);
    float A2 = (nD - 1) * logf(tau2);
    float tpR = expf(A1 - tau1 - lfac1) / tauR;
    float tpD = expf(A2 - tau2 - lfac2) / tauD;
    return tpR - ratio * tpD;
}

/* hStatic_nonlinear's logistic a and b (src/LGN_props.h:159-169), in float. */
void orc_logistic_ab(const float *spont, const float *c50, const float *sharp, int n, float *a, float *b) {
    for (int i = 0; i < n; i++) {
        const float e_kc50 = expf(sharp[i] * c50[i]);
        const float e_kc50_k = expf(sharp[i] * c50[i] - sharp[i]);
        a[i] = (1 - spont[i]) * (1 + e_kc50) * (1 + e_kc50_k) / (e_kc50 - e_kc50_k);
        b[i] = 1 - a[i] / (1 + e_kc50_k);
    }
}

/* store_PM for magno cells: TW [nMagno][nKS], SW [nMagno][nSample], SC [2][nMagno][nSample],
 * maxConvol [nLGN], absk [nMagno]; logistic la/lb [nLGN]. */
int orc_lgn_setup(const pv1_lgn_config *c, const pv1_lgn_params *p, float *TW, float *SW,
                  float *SC, float *maxConvol, float *absk, float *la, float *lb) {
    const int nLGN = (int)c->nLGN;
    const int nMagno = (int)(c->nMagno_I + c->nMagno_C);
    const int n1 = (int)c->mSample1D, nS = n1 * n1, nKS = (int)c->nKernelSample;
    orc_logistic_ab(p->spont, p->c50, p->sharpness, nLGN, la, lb);
    float *cw = (float *)malloc(sizeof(float) * nS), *sw = (float *)malloc(sizeof(float) * nS);
    for (int m = 0; m < nMagno; m++) {
        int id = (int)c->nParvo_I + m;
        if (m >= (int)c->nMagno_I) id += (int)c->nParvo_C;
        /* temporal weights, time reversed and L1 normalised */
        const float lfac1 = lgammaf(p->nR[id]), lfac2 = lgammaf(p->nD[id]);
        const float t0 = c->kernelSampleT0 - p->delay[id];
        float tot = 0.f;
        for (int j = 0; j < nKS; j++) {
            int twid = nKS - 1 - j;
            float t = twid * c->kernelSampleDt + t0;
            float tw = t < 0 ? 0.0f
                             : temporal_kernel(t, p->tauR[id], p->tauD[id], p->nR[id], p->nD[id],
                                               p->ratio[id], lfac1, lfac2);
            TW[(size_t)m * nKS + j] = tw;
            tot += fabsf(tw);
        }
        for (int j = 0; j < nKS; j++) TW[(size_t)m * nKS + j] /= tot;
        /* DoG weights */
        const int sid = nLGN + id;
        const float ox = p->ecc[sid] * cosf(p->polar[sid]) - p->ecc[id] * cosf(p->polar[id]);
        const float oy = p->ecc[sid] * sinf(p->polar[sid]) - p->ecc[id] * sinf(p->polar[id]);
        float d_orient = p->orient[id] - p->orient[sid];
        if (fabsf(d_orient) > (float)(M_PI / 2)) d_orient -= copysignf((float)M_PI, d_orient);
        const float rc = cosf(d_orient), rsn = sinf(d_orient);
        const float rs = p->rw[sid] > p->rh[sid] ? p->rw[sid] : p->rh[sid];
        const float span = c->nsig * rs + sqrtf(ox * ox + oy * oy);
        const float ds = 2 * span / n1;
        float csum = 0.f, ssum = 0.f;
        for (int s = 0; s < nS; s++) {
            const int tx = s % n1, ty = s / n1;
            const float cx = grid_at(tx, ds, span), cy = grid_at(ty, ds, span);
            const float ttx = cx - ox, tty = cy - oy;
            const float sx = ttx * rc - tty * rsn, sy = ttx * rsn + tty * rc;
            cw[s] = gauss2(cx, cy, p->rw[id], p->rh[id]);
            sw[s] = gauss2(sx, sy, p->rw[sid], p->rh[sid]);
            csum += cw[s];
            ssum += sw[s];
        }
        const float k = p->k[id];
        float wsum = 0.f;
        for (int s = 0; s < nS; s++) {
            float w = copysignf(cw[s] / csum, k) - copysignf(sw[s] / ssum, k);
            SW[(size_t)m * nS + s] = w;
            wsum += fabsf(w);
        }
        for (int s = 0; s < nS; s++) SW[(size_t)m * nS + s] /= wsum;
        maxConvol[id] = fabsf(k) * wsum;
        absk[m] = fabsf(k);
        /* texture coordinates (flat retina) */
        const int left = m < (int)c->nMagno_I;
        const float x0 = left ? c->L_x0 : c->R_x0, y0 = left ? c->L_y0 : c->R_y0;
        const float coso = cosf(p->orient[id]), sino = sinf(p->orient[id]);
        for (int s = 0; s < nS; s++) {
            const int tx = s % n1, ty = s / n1;
            const float cx = grid_at(tx, ds, span), cy = grid_at(ty, ds, span);
            sample_xy(c->flat_retina, p->polar[id], p->ecc[id], cx, cy, coso, sino, c->normViewDistance, x0, y0,
                      &SC[(size_t)m * nS + s], &SC[(size_t)nMagno * nS + (size_t)m * nS + s]);
        }
    }
    free(cw);
    free(sw);
    return 0;
}

/* Bilinear texture fetch with normalised coordinates and border addressing: the filtering
 * the CUDA programming guide documents for linear texture filtering, with the fractional
 * weights held in 9-bit fixed point (8 fractional bits). */
static float tex_fetch(const float *plane, int w, int h, float x, float y, int wbits) {
    float xb = x * w - 0.5f, yb = y * h - 0.5f;
    float fi = floorf(xb), fj = floorf(yb);
    float a = xb - fi, b = yb - fj;
    if (wbits > 0) {
        const float q = (float)(1 << wbits);
        a = rintf(a * q) / q;
        b = rintf(b * q) / q;
    }
    int i = (int)fi, j = (int)fj;
    float t00 = (i >= 0 && i < w && j >= 0 && j < h) ? plane[(size_t)j * w + i] : 0.f;
    float t10 = (i + 1 >= 0 && i + 1 < w && j >= 0 && j < h) ? plane[(size_t)j * w + i + 1] : 0.f;
    float t01 = (i >= 0 && i < w && j + 1 >= 0 && j + 1 < h) ? plane[(size_t)(j + 1) * w + i] : 0.f;
    float t11 = (i + 1 >= 0 && i + 1 < w && j + 1 >= 0 && j + 1 < h) ? plane[(size_t)(j + 1) * w + i + 1] : 0.f;
    return (1 - a) * (1 - b) * t00 + a * (1 - b) * t10 + (1 - a) * b * t01 + a * b * t11;
}

static float intensity(int cone, const float *L, const float *M, const float *S, int w, int h,
                       float x, float y, int wbits) {
    switch (cone) {
        case 0: return tex_fetch(L, w, h, x, y, wbits);
        case 1: return tex_fetch(M, w, h, x, y, wbits);
        case 2: return tex_fetch(S, w, h, x, y, wbits);
        case 3: return (tex_fetch(L, w, h, x, y, wbits) + tex_fetch(M, w, h, x, y, wbits)) / 2.0f;
        case 4:
            return tex_fetch(L, w, h, x, y, wbits) * 0.45436904f + tex_fetch(M, w, h, x, y, wbits) * 0.47353315f +
                   tex_fetch(S, w, h, x, y, wbits) * 0.0720978f;
        default: return 0.f;
    }
}

/* Spatial contrast of every (frame, cell): layers [nLayer][3][h][w] (the last layer may be
 * the initial luminance).  S [nLayer][nMagno]. */
int orc_lgn_spatial(int nMagno, int nSample, const float *SW, const float *SC,
                    const uint32_t *coneType, const float *layers, int nLayer, int h, int w,
                    int wbits, float *S) {
    const size_t npix = (size_t)w * h;
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nLayer; f++) {
        const float *L = layers + (size_t)f * 3 * npix, *M = L + npix, *Sp = M + npix;
        for (int m = 0; m < nMagno; m++) {
            const float *sx = SC + (size_t)m * nSample, *sy = SC + (size_t)nMagno * nSample + (size_t)m * nSample;
            float sum = 0.f;
            for (int s = 0; s < nSample; s++) sum += intensity(3, L, M, Sp, w, h, sx[s], sy[s], wbits);
            const float mean = sum / nSample;
            float acc = 0.f;
            for (int s = 0; s < nSample; s++) {
                float I = intensity((int)coneType[m], L, M, Sp, w, h, sx[s], sy[s], wbits);
                float cc = mean > 0 ? I / mean - 1.0f : I;
                if (fabsf(cc) > 1.0f) cc = copysignf(1.0f, cc);
                acc += SW[(size_t)m * nSample + s] * cc;
            }
            S[(size_t)f * nMagno + m] = acc;
        }
    }
    return 0;
}

/* Temporal convolution of step `it`, sample by sample as LGN_convol_magno walks it:
 * sample j of the window reads the texture layer tail + ((T0 + j*interval)*denorm +
 * phase)/ntPerFrame; the layer holds the newest frame with that residue mod maxFrame, or the
 * initial luminance if no frame was loaded there yet.  convol_out[m] = convol * |k|. */
/* Row of the spatial table read by sample j of step it's window: sample j sits
 * (T0 + j*interval)*denorm + phase units after the window tail layer
 * (oldFrameHead + frameOffset + (phase <= comp ? 2 : 1), getTail of src/patch.cu:5413-5422);
 * the layer holds the newest loaded frame with that residue mod maxFrame, or the initial
 * luminance (row nFrame) if no frame was loaded there yet. */
static void window_rows(const pv1_lgn_config *c, int nKS, int T0, int interval, int comp, int frameOffset,
                        int nFrame, long long it, int *rowOf) {
    const long long num = (it + 1) * (long long)c->denorm;
    const int currentFrame = (int)((num + c->ntPerFrame - 1) / c->ntPerFrame);
    const int oldFrameHead = (currentFrame - 1) % (int)c->maxFrame;
    const int phase = (int)((comp + (it + 1) * (long long)c->denorm) % c->ntPerFrame);
    const int tail = oldFrameHead + frameOffset + (phase <= comp ? 2 : 1);
    for (int j = 0; j < nKS; j++) {
        long long o = (long long)(T0 + (long long)j * interval) * c->denorm + phase;
        int layer = (int)((tail + o / c->ntPerFrame) % c->maxFrame);
        int Fnew = currentFrame - 1;
        int back = ((Fnew % (int)c->maxFrame) - layer + (int)c->maxFrame) % (int)c->maxFrame;
        int F = Fnew - back;
        rowOf[j] = F < 0 ? nFrame : F % nFrame;
    }
}

/* Temporal convolution of step `it` for the magno cells, sample by sample as
 * LGN_convol_magno walks it.  convol_out[m] = convol * |k|. */
int orc_lgn_convol(const pv1_lgn_config *c, int nMagno, int nFrame, long long it, const float *TW,
                   const float *S, const float *absk, float *convol_out) {
    const int nKS = (int)c->nKernelSample;
    int *rowOf = (int *)malloc(sizeof(int) * nKS);
    window_rows(c, nKS, (int)c->iKernelSampleT0, (int)c->kernelSampleInterval, (int)c->magnoComp,
                (int)c->frameOffset, nFrame, it, rowOf);
    for (int m = 0; m < nMagno; m++) {
        float conv = 0.f;
        for (int j = 0; j < nKS; j++) conv += S[(size_t)rowOf[j] * nMagno + m] * TW[(size_t)m * nKS + j];
        convol_out[m] = conv * absk[m];
    }
    free(rowOf);
    return 0;
}

/* ---- parvocellular cells (store_PM with PM = 0, parvo_maxConvol, LGN_convol_parvo) ---- */

/* Side of parvo_maxConvol's sample grid, src/patch.cu:5266-5312: round(mean over cone
 * type < 4 cells of sqrt(R^2 / (wSpan hSpan)), divided by nParvo) * nSpatialSample1D, at least
 * 32, and at most what 48 KB - 128 B of shared memory holds for two float arrays. */
int orc_parvo_max_sample1d(const pv1_lgn_config *c, const pv1_lgn_params *p, int n1) {
    const int nLGN = (int)c->nLGN, nParvo = (int)(c->nParvo_I + c->nParvo_C);
    const float nsig = fabsf(c->nsig);
    float meanRatio = 0.f;
    for (int i = 0; i < nLGN; i++) {
        if (p->coneType[i] >= 4) continue;
        float dx = p->ecc[i] * cosf(p->polar[i]) - p->ecc[nLGN + i] * cosf(p->polar[nLGN + i]);
        float dy = p->ecc[i] * sinf(p->polar[i]) - p->ecc[nLGN + i] * sinf(p->polar[nLGN + i]);
        float r = sqrtf(dx * dx + dy * dy);
        float wSpan = parvo_span(nsig, p->rw[nLGN + i]), hSpan = parvo_span(nsig, p->rh[nLGN + i]);
        float R = wSpan > hSpan ? wSpan : hSpan;
        wSpan = parvo_span(nsig, p->rw[i]);
        hSpan = parvo_span(nsig, p->rh[i]);
        r += wSpan > hSpan ? wSpan : hSpan;
        R = r > R ? r : R;
        meanRatio += sqrtf(R * R / wSpan / hSpan);
    }
    meanRatio /= nParvo;
    long long m1 = (long long)roundf(meanRatio) * n1;
    if (m1 * m1 < 1024) return 32;
    const size_t avail = 48 * 1024 - 32 * sizeof(float);
    if ((size_t)(m1 * m1) * 2 * sizeof(float) > avail)
        m1 = (long long)floor(sqrt((double)(avail / sizeof(float) / 2 / (size_t)(n1 * n1)))) * n1;
    return (int)m1;
}

/* TW [nParvo][2][nKS], SW [nSample], SC [2][nParvo][2][nSample], maxConvol at parvo ids. */
int orc_lgn_parvo_setup(const pv1_lgn_config *c, const pv1_lgn_parvo_config *q, const pv1_lgn_params *p,
                        const float *covariant, float *TW, float *SW, float *SC, float *maxConvol) {
    const int nLGN = (int)c->nLGN, nParvo = (int)(c->nParvo_I + c->nParvo_C);
    const int n1 = (int)q->nSample1D, nS = n1 * n1, nKS = (int)q->nKernelSample;
    for (int cell = 0; cell < nParvo; cell++) {
        const int id = cell < (int)c->nParvo_I ? cell : cell + (int)c->nMagno_I;
        for (int type = 0; type < 2; type++) {
            const int lid = type * nLGN + id;
            /* store_temporalWeight (src/discrete_input_convol.cu:230-305) */
            const float lfac1 = lgammaf(p->nR[lid]), lfac2 = lgammaf(p->nD[lid]);
            const float t0 = q->kernelSampleT0 - p->delay[lid];
            float *tw = TW + ((size_t)cell * 2 + type) * nKS;
            float tot = 0.f;
            for (int j = 0; j < nKS; j++) {
                float t = (nKS - 1 - j) * q->kernelSampleDt + t0;
                tw[j] = t < 0 ? 0.0f
                              : temporal_kernel(t, p->tauR[lid], p->tauD[lid], p->nR[lid], p->nD[lid],
                                                p->ratio[lid], lfac1, lfac2);
                tot += fabsf(tw[j]);
            }
            for (int j = 0; j < nKS; j++) tw[j] /= tot;
            /* store_spatialWeight (:309-425), flat retina */
            const float rx = p->rw[lid], ry = p->rh[lid];
            const float wSpan = parvo_span(c->nsig, rx), hSpan = parvo_span(c->nsig, ry);
            const float dw = 2 * wSpan / n1, dh = 2 * hSpan / n1;
            if (cell == 0 && type == 0) {
                float sum = 0.f;
                for (int s = 0; s < nS; s++) {
                    SW[s] = gauss2(grid_at(s % n1, dw, wSpan), grid_at(s / n1, dh, hSpan), rx, ry);
                    sum += SW[s];
                }
                for (int s = 0; s < nS; s++) SW[s] /= sum;
            }
            const int left = cell < (int)c->nParvo_I;
            const float x0 = left ? c->L_x0 : c->R_x0, y0 = left ? c->L_y0 : c->R_y0;
            const float coso = cosf(p->orient[lid]), sino = sinf(p->orient[lid]);
            const float ce = p->ecc[lid], cp = p->polar[lid];
            for (int s = 0; s < nS; s++) {
                const float w = grid_at(s % n1, dw, wSpan), h = grid_at(s / n1, dh, hSpan);
                const size_t sid = ((size_t)cell * 2 + type) * nS + s;
                sample_xy(c->flat_retina, cp, ce, w, h, coso, sino, c->normViewDistance, x0, y0, &SC[sid],
                          &SC[(size_t)nParvo * 2 * nS + sid]);
            }
        }
    }
    /* parvo_maxConvol (:748-883) */
    const int m1 = orc_parvo_max_sample1d(c, p, n1);
    const int nUse = (m1 * m1 / 1024) * 1024;
    float *swC = (float *)malloc(sizeof(float) * (size_t)(nUse > 0 ? nUse : 1));
    float *swS = (float *)malloc(sizeof(float) * (size_t)(nUse > 0 ? nUse : 1));
    for (int cell = 0; cell < nParvo; cell++) {
        const int id = cell < (int)c->nParvo_I ? cell : cell + (int)c->nMagno_I;
        const int sid = nLGN + id;
        float wSpan = parvo_span(c->nsig, p->rw[sid]), hSpan = parvo_span(c->nsig, p->rh[sid]);
        float R = wSpan > hSpan ? wSpan : hSpan;
        wSpan = parvo_span(c->nsig, p->rw[id]);
        hSpan = parvo_span(c->nsig, p->rh[id]);
        const float dx = p->ecc[id] * cosf(p->polar[id]) - p->ecc[sid] * cosf(p->polar[sid]);
        const float dy = p->ecc[id] * sinf(p->polar[id]) - p->ecc[sid] * sinf(p->polar[sid]);
        float r = sqrtf(dx * dx + dy * dy);
        r += wSpan > hSpan ? wSpan : hSpan;
        R = r > R ? r : R;
        const float coss = cosf(p->orient[sid]), sins = sinf(p->orient[sid]);
        const float cosc = cosf(p->orient[id]), sinc = sinf(p->orient[id]);
        const float ds = 2 * R / m1;
        float sumC = 0.f, sumS = 0.f;
        for (int s = 0; s < nUse; s++) {
            const float lx = grid_at(s % m1, ds, R), ly = grid_at(s / m1, ds, R);
            float x = cosc * (lx - dx) + sinc * (ly - dy), y = -sinc * (lx - dx) + cosc * (ly - dy);
            swC[s] = gauss2(x, y, p->rw[id], p->rh[id]);
            x = coss * lx + sins * ly;
            y = -sins * lx + coss * ly;
            swS[s] = gauss2(x, y, p->rw[sid], p->rh[sid]);
            sumC += swC[s];
            sumS += swS[s];
        }
        for (int s = 0; s < nUse; s++) {
            swC[s] /= sumC;
            swS[s] /= sumS;
        }
        const float *twC = TW + (size_t)cell * 2 * nKS, *twS = twC + nKS;
        const float kc = p->k[id], ks = p->k[sid], cov = covariant[id];
        double conv = 0.0;
        for (int it = 0; it < nKS; it++) {
            for (int s = 0; s < nUse; s++) {
                const float lc = swC[s] * twC[it] * kc, ls = swS[s] * twS[it] * ks;
                float decide;
                if (fabsf(lc) > fabsf(ls)) decide = fabsf(lc) + ls * copysignf(cov, lc);
                else decide = fabsf(ls) + lc * copysignf(cov, ls);
                conv += decide;
            }
        }
        maxConvol[id] = (float)conv;
    }
    free(swC);
    free(swS);
    return 0;
}

/* Per-frame centre and surround contrast sums of the parvo cells: layers [nLayer][3][h][w];
 * cone [2][nParvo]; PS [nLayer][2][nParvo].  Both means are taken at the surround's
 * coordinates, as src/discrete_input_convol.cu:1034-1035 samples them. */
int orc_lgn_parvo_spatial(int nParvo, int nSample, const float *SW, const float *SC, const uint32_t *cone,
                          const float *layers, int nLayer, int h, int w, int wbits, float *PS) {
    const size_t npix = (size_t)w * h;
    const size_t yOff = (size_t)nParvo * 2 * nSample;
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nLayer; f++) {
        const float *L = layers + (size_t)f * 3 * npix, *M = L + npix, *Sp = M + npix;
        for (int cell = 0; cell < nParvo; cell++) {
            const float *xC = SC + (size_t)cell * 2 * nSample, *yC = xC + yOff;
            const float *xS = xC + nSample, *yS = xS + yOff;
            const int tC = (int)cone[cell], tS = (int)cone[nParvo + cell];
            float sumC = 0.f, sumS = 0.f;
            for (int s = 0; s < nSample; s++) {
                sumC += intensity(tC, L, M, Sp, w, h, xS[s], yS[s], wbits);
                sumS += intensity(tS, L, M, Sp, w, h, xS[s], yS[s], wbits);
            }
            const float meanC = sumC / nSample, meanS = sumS / nSample;
            float accC = 0.f, accS = 0.f;
            for (int s = 0; s < nSample; s++) {
                float I = intensity(tC, L, M, Sp, w, h, xC[s], yC[s], wbits);
                float cc = meanC > 0 ? I / meanC - 1.0f : I;
                if (fabsf(cc) > 1.0f) cc = copysignf(1.0f, cc);
                accC += SW[s] * cc;
                I = intensity(tS, L, M, Sp, w, h, xS[s], yS[s], wbits);
                cc = meanS > 0 ? I / meanS - 1.0f : I;
                if (fabsf(cc) > 1.0f) cc = copysignf(1.0f, cc);
                accS += SW[s] * cc;
            }
            PS[((size_t)f * 2 + 0) * nParvo + cell] = accC;
            PS[((size_t)f * 2 + 1) * nParvo + cell] = accS;
        }
    }
    return 0;
}

/* LGN_convol_parvo for step it: sum over samples of (centre contrast x centre weight) and
 * (surround contrast x surround weight), each times its k.  out [nParvo]. */
int orc_lgn_parvo_convol(const pv1_lgn_config *c, const pv1_lgn_parvo_config *q, const pv1_lgn_params *p,
                         int nFrame, long long it, const float *TW, const float *PS, float *out) {
    const int nLGN = (int)c->nLGN, nParvo = (int)(c->nParvo_I + c->nParvo_C);
    const int nKS = (int)q->nKernelSample;
    int *rowOf = (int *)malloc(sizeof(int) * nKS);
    window_rows(c, nKS, (int)q->iKernelSampleT0, (int)q->kernelSampleInterval, (int)q->parvoComp,
                (int)q->frameOffset, nFrame, it, rowOf);
    for (int cell = 0; cell < nParvo; cell++) {
        const int id = cell < (int)c->nParvo_I ? cell : cell + (int)c->nMagno_I;
        const float *twC = TW + (size_t)cell * 2 * nKS, *twS = twC + nKS;
        float convC = 0.f, convS = 0.f;
        for (int j = 0; j < nKS; j++) {
            const size_t row = (size_t)rowOf[j] * 2 * nParvo;
            convC += PS[row + cell] * twC[j];
            convS += PS[row + nParvo + cell] * twS[j];
        }
        out[cell] = convC * p->k[id] + convS * p->k[nLGN + id];
    }
    free(rowOf);
    return 0;
}

/* LGN_nonlinear + get_spike for every LGN cell of one step; convol [nLGN] by LGN id (magno
 * entries already times |k|).  u: recorded uniforms [nLGN][cap] of this step, ucount [nLGN].
 * Returns the number of cells whose draw count disagrees with the record (0 when the CPU and
 * GPU took the same branches). */
/* LGN_nonlinear (src/discrete_input_convol.cu:1637-1821): logistic rate and get_spike on
 * the given uniforms; nsp_out/tsp_out (may be NULL) receive the spike count and mean spike
 * time the presynaptic learning trace uses. */
int orc_lgn_nonlinear_ex(const pv1_lgn_config *c, const float *convol, const float *maxConvol,
                         const float *c50, const float *sharp, const float *la, const float *lb,
                         float *ltr, float *lnl, const float *u, const int32_t *ucount, int cap,
                         float *sInfo_out, float *fr_out, uint32_t *nsp_out, float *tsp_out) {
    int mismatch = 0;
    for (int id = 0; id < (int)c->nLGN; id++) {
        const float mx = maxConvol[id];
        float current = convol[id] * c->convolRatio;
        if (current < 0) current = 0;
        float X = (float)(1.0 / (double)(1 + expf(sharp[id] * (c50[id] - current / mx))));
        float fr = c->frRatio * mx * (la[id] * X + lb[id]);
        const float dt = c->dt;
        const float rate = fr / 1000.0f;
        const float rT = dt * rate;
        float next_rT = lnl[id] - ltr[id];
        unsigned nsp = 0;
        float tsp = 0.f;
        if (next_rT > rT) {
            ltr[id] += rT;
        } else {
            float old_rT = 0.f;
            do {
                float rnd = (int)nsp < cap ? u[(size_t)id * cap + nsp] : 0.5f;
                lnl[id] = fmaxf(-logf(rnd), 0.0f * rate);
                old_rT = next_rT;
                next_rT += lnl[id];
                nsp++;
            } while (next_rT <= rT);
            ltr[id] = rT - old_rT;
            tsp = old_rT / (rate * nsp);
        }
        if (ucount && (int)nsp != ucount[id]) mismatch++;
        sInfo_out[id] = nsp + tsp / dt;
        if (fr_out) fr_out[id] = fr;
        if (nsp_out) nsp_out[id] = nsp;
        if (tsp_out) tsp_out[id] = tsp;
    }
    return mismatch;
}

int orc_lgn_nonlinear(const pv1_lgn_config *c, const float *convol, const float *maxConvol,
                      const float *c50, const float *sharp, const float *la, const float *lb,
                      float *ltr, float *lnl, const float *u, const int32_t *ucount, int cap,
                      float *sInfo_out, float *fr_out) {
    return orc_lgn_nonlinear_ex(c, convol, maxConvol, c50, sharp, la, lb, ltr, lnl, u, ucount, cap, sInfo_out,
                                fr_out, NULL, NULL);
}

/* The presynaptic LTP trace of each LGN cell over one step (the learning block of
 * LGN_nonlinear, src/discrete_input_convol.cu:1774-1808, one learning type): `start` gets the
 * trace at the step start; a cell that spiked adds its spike count, decays to the spike time
 * tsp and leaves that value in `at_spike`; every trace then decays to the step end. */
void orc_lgn_ff_pre(int nLGN, float dt, float tauLTP, const uint32_t *nsp, const float *tsp, const float *sInfo,
                    float *var, float *start, float *at_spike) {
    for (int id = 0; id < nLGN; id++) {
        float x = var[id];
        start[id] = x;
        float delta_t = dt;
        if (sInfo[id] > 0) {
            x += (float)nsp[id];
            x *= expf(-tsp[id] / tauLTP);
            at_spike[id] = x;
            delta_t = dt - tsp[id];
        } else {
            at_spike[id] = 0.f;
        }
        x *= expf(-delta_t / tauLTP);
        var[id] = x;
    }
}

/* ================================================================== V1 ============= */

typedef struct orc_v1 {
    pv1_v1_config c;
    int nV1, nE, nI, bs, nblock;
    ocond cFF, cE, cI;
    float *v, *w, *tBack, *dep, *gFF, *hFF, *gE, *hE, *gI, *hI, *tonic, *lastNoise, *sInfo;
    /* LGN synapses */
    int maxLGN;
    uint32_t *nLGN, *lgnId;
    float *sLGN;
    /* near */
    int nnb;
    uint32_t *nNearNB, *nbId;
    const float *conMat; /* borrowed */
    /* far: per-(post, j) spike rings (fSpikeTrain) */
    size_t nFar;
    uint32_t *nVec, *vecID;
    size_t *vecOff;
    float *conVec, *delayVec;
    float *ring;
    size_t *ringOff;
    uint32_t *depth, *slot;
    int anyFar;
    /* delayed near delivery (noDelay = 0): the spike-word ring spikeTrain[trainDepth][nV1] */
    const float *delayMat; /* borrowed, conMat layout */
    float *spikeRing;
    int trainDepth, curSlot;
    /* far synaptic failure: libstdc++ minstd_rand0 states per post, chunks of blocks */
    uint32_t *farEng;
    int nChunk;
    /* LGN->V1 plasticity (learning 1-4) */
    int learn;       /* the reference's `learning` (0: off) */
    int ffI;         /* FF->I type on (learning 2) */
    float lt[2][9];  /* per type (FF->E, FF->I): tauLTP, tauLTD, tauTrip, tauAvg, targetFR, A_LTP, A_ratio, gmax, gmin */
    float lExpHomeo, tauAvgCortical;
    int applyHomeo, symmetricHomeo, rebound;
    float *ffPost;   /* vLTD_FF_E, vTrip_FF_E [nblock*nE], vLTD_FF_I, vTrip_FF_I [nblock*nI] (with FF->I),
                        vAvgE [nblock*nE][2], vAvgI [nblock*nI] */
    size_t offI, offAvgE, offAvgI;
    float *totalFF;  /* [2][nV1] */
} orc_v1;

static int otype(const orc_v1 *o, int local) {
    for (uint32_t j = 0; j < o->c.nType; j++)
        if ((uint32_t)local < o->c.typeAcc[j]) return (int)j;
    return (int)o->c.nType - 1;
}

void orc_v1_destroy(orc_v1 *o);

orc_v1 *orc_v1_create(const pv1_v1_config *cfg, uint32_t maxLGN, const uint32_t *nLGN,
                      const uint32_t *lgnId, const float *sLGN, uint32_t nnb,
                      const uint32_t *nNearNB, const uint32_t *nbId, const float *conMat,
                      const uint32_t *nVec, const uint32_t *vecID, const float *conVec,
                      const float *delayVec, const float *tonicDep) {
    orc_v1 *o = (orc_v1 *)calloc(1, sizeof(orc_v1));
    o->c = *cfg;
    o->bs = (int)cfg->blockSize;
    o->nblock = (int)cfg->nblock;
    o->nV1 = o->bs * o->nblock;
    o->nE = (int)cfg->typeAcc[cfg->nTypeE - 1];
    o->nI = o->bs - o->nE;
    o->cFF = ocond_make(cfg->riseFF, cfg->decayFF, (int)cfg->ngFF);
    o->cE = ocond_make(cfg->riseE, cfg->decayE, (int)cfg->ngE);
    o->cI = ocond_make(cfg->riseI, cfg->decayI, (int)cfg->ngI);
    const size_t n = (size_t)o->nV1;
#define OALLOC(f, cnt) o->f = (float *)calloc((cnt), sizeof(float))
    OALLOC(v, n); OALLOC(w, n); OALLOC(tBack, n); OALLOC(dep, n);
    OALLOC(gFF, cfg->ngFF * n); OALLOC(hFF, cfg->ngFF * n);
    OALLOC(gE, cfg->ngE * n); OALLOC(hE, cfg->ngE * n);
    OALLOC(gI, cfg->ngI * n); OALLOC(hI, cfg->ngI * n);
    OALLOC(tonic, n); OALLOC(lastNoise, n); OALLOC(sInfo, n);
#undef OALLOC
    memcpy(o->tonic, tonicDep, n * sizeof(float));
    o->maxLGN = (int)maxLGN;
    o->nLGN = (uint32_t *)malloc(n * sizeof(uint32_t));
    memcpy(o->nLGN, nLGN, n * sizeof(uint32_t));
    o->lgnId = (uint32_t *)malloc((size_t)maxLGN * n * sizeof(uint32_t) + 4);
    memcpy(o->lgnId, lgnId, (size_t)maxLGN * n * sizeof(uint32_t));
    o->sLGN = (float *)malloc((size_t)maxLGN * n * sizeof(float) + 4);
    memcpy(o->sLGN, sLGN, (size_t)maxLGN * n * sizeof(float));
    o->nnb = (int)nnb;
    o->nNearNB = (uint32_t *)malloc(o->nblock * sizeof(uint32_t));
    memcpy(o->nNearNB, nNearNB, o->nblock * sizeof(uint32_t));
    o->nbId = (uint32_t *)malloc((size_t)o->nblock * nnb * sizeof(uint32_t));
    memcpy(o->nbId, nbId, (size_t)o->nblock * nnb * sizeof(uint32_t));
    o->conMat = conMat;
    /* far rings: depth = ceil(delay/speed/dt) + 1, initialised to -1 (src/patch.cu:3838-3864) */
    o->nVec = (uint32_t *)malloc(n * sizeof(uint32_t));
    memcpy(o->nVec, nVec, n * sizeof(uint32_t));
    o->vecOff = (size_t *)malloc((n + 1) * sizeof(size_t));
    o->vecOff[0] = 0;
    for (size_t i = 0; i < n; i++) o->vecOff[i + 1] = o->vecOff[i] + nVec[i];
    o->nFar = o->vecOff[n];
    o->vecID = (uint32_t *)malloc(o->nFar * sizeof(uint32_t) + 4);
    o->conVec = (float *)malloc(o->nFar * sizeof(float) + 4);
    o->delayVec = (float *)malloc(o->nFar * sizeof(float) + 4);
    if (o->nFar) {
        memcpy(o->vecID, vecID, o->nFar * sizeof(uint32_t));
        memcpy(o->conVec, conVec, o->nFar * sizeof(float));
        memcpy(o->delayVec, delayVec, o->nFar * sizeof(float));
    }
    o->depth = (uint32_t *)malloc(o->nFar * sizeof(uint32_t) + 4);
    o->slot = (uint32_t *)calloc(o->nFar + 1, sizeof(uint32_t));
    o->ringOff = (size_t *)malloc((o->nFar + 1) * sizeof(size_t));
    o->ringOff[0] = 0;
    for (size_t e = 0; e < o->nFar; e++) {
        o->depth[e] = (uint32_t)ceilf((o->delayVec[e] / cfg->speedOfThought) / cfg->dt) + 1;
        o->ringOff[e + 1] = o->ringOff[e] + o->depth[e];
    }
    o->ring = (float *)malloc(o->ringOff[o->nFar] * sizeof(float) + 4);
    for (size_t q = 0; q < o->ringOff[o->nFar]; q++) o->ring[q] = -1.0f;
    o->anyFar = o->nFar > 0;
    return o;
}

void orc_v1_destroy(orc_v1 *o) {
    if (!o) return;
    free(o->v); free(o->w); free(o->tBack); free(o->dep); free(o->gFF); free(o->hFF);
    free(o->gE); free(o->hE); free(o->gI); free(o->hI); free(o->tonic); free(o->lastNoise);
    free(o->sInfo); free(o->nLGN); free(o->lgnId); free(o->sLGN); free(o->nNearNB);
    free(o->nbId); free(o->nVec); free(o->vecOff); free(o->vecID); free(o->conVec);
    free(o->delayVec); free(o->ring); free(o->ringOff); free(o->depth); free(o->slot);
    free(o->spikeRing);
    free(o->farEng);
    free(o->ffPost);
    free(o->totalFF);
    free(o);
}

/* which: same ids as PV1_ST_*. */
static float *oarr(orc_v1 *o, int which, size_t *cnt) {
    const size_t n = (size_t)o->nV1;
    *cnt = n;
    switch (which) {
        case PV1_ST_V: return o->v;
        case PV1_ST_W: return o->w;
        case PV1_ST_TBACK: return o->tBack;
        case PV1_ST_DEP: return o->dep;
        case PV1_ST_GFF: *cnt = o->c.ngFF * n; return o->gFF;
        case PV1_ST_HFF: *cnt = o->c.ngFF * n; return o->hFF;
        case PV1_ST_GE: *cnt = o->c.ngE * n; return o->gE;
        case PV1_ST_HE: *cnt = o->c.ngE * n; return o->hE;
        case PV1_ST_GI: *cnt = o->c.ngI * n; return o->gI;
        case PV1_ST_HI: *cnt = o->c.ngI * n; return o->hI;
        case PV1_ST_SINFO: return o->sInfo;
        case PV1_ST_SLGN: *cnt = (size_t)o->maxLGN * n; return o->sLGN;
        case PV1_ST_FF_POST: *cnt = o->offAvgI + (size_t)o->nI * o->nblock; return o->ffPost;
        case PV1_ST_TOTAL_FF: *cnt = 2 * n; return o->totalFF;
        default: return NULL;
    }
}

int orc_v1_get(orc_v1 *o, int which, float *out) {
    size_t cnt;
    float *a = oarr(o, which, &cnt);
    if (!a) return -1;
    memcpy(out, a, cnt * sizeof(float));
    return 0;
}

int orc_v1_put(orc_v1 *o, int which, const float *in) {
    size_t cnt;
    float *a = oarr(o, which, &cnt);
    if (!a) return -1;
    memcpy(a, in, cnt * sizeof(float));
    return 0;
}

/* The AdEx pieces of src/coredynamics.cuh:27-118, as compute_v uses them (exported so that
 * they can be checked against the reference's own struct compiled on the host). */
float orc_adex_depc(float vL, float vT, float gL, float a, float deltaT, float dep) {
    const float targetV = vL + (vT - vL) * dep;
    if (targetV > vT) return (gL + a) * (targetV - vL) - gL * deltaT;
    return (gL + a) * (targetV - vL) - gL * deltaT * expf((targetV - vT) / deltaT);
}

/* set_p0 / set_p1 (get_a, get_b, depC, no gap junction) then rk2 over dt */
void orc_adex_rk2(float vE, float vI, float vL, float gE0, float gI0, float gE1, float gI1, float depC,
                  float gL, float vT, float deltaT, float Cm, float a, float tau_w, float v0, float w0, float dt,
                  float n0, float n1, float *v, float *w) {
    const float a0 = gE0 + gI0 + gL, b0 = gE0 * vE + gI0 * vI + gL * vL + depC;
    const float a1 = gE1 + gI1 + gL, b1 = gE1 * vE + gI1 * vI + gL * vL + depC;
    const float dTgL = deltaT * gL;
    const float fk1 = (-a0 * v0 + b0 + dTgL * expf((v0 - vT) / deltaT) - w0) / Cm + n0;
    const float gk1 = (a * (v0 - vL) - w0) / tau_w;
    const float v1 = v0 + dt * fk1;
    const float w1 = w0 + dt * gk1;
    const float fk2 = (-a1 * v1 + b1 + dTgL * expf((v1 - vT) / deltaT) - w1) / Cm + n1;
    const float gk2 = (a * (v1 - vL) - w1) / tau_w;
    *w = w0 + dt * (gk1 + gk2) / 2;
    *v = v0 + dt * (fk1 + fk2) / 2;
}

/* compute_spike_time: the threshold-crossing fraction of the step and w0's jump */
void orc_adex_spike(float vThres, float v0, float v, float w, float b, float *ratio, float *w0) {
    *ratio = (vThres - v0) / (v - v0);
    *w0 += *ratio * (w - *w0) + b;
}

/* ConductanceShape (src/condShape.h:13-41) for one species: out = {g, h after
 * decay_conductance(dt), g, h after compute_single_input_conductance(f, dt)} from (g, h). */
void orc_cond_eval(float rise, float decay, float g, float h, float f, float dt, float *out) {
    ocond c = ocond_make(&rise, &decay, 1);
    float g1 = g, h1 = h, g2 = g, h2 = h;
    ocond_decay(&c, &g1, &h1, dt, 0);
    ocond_input(&c, &g2, &h2, f, dt, 0);
    out[0] = g1; out[1] = h1; out[2] = g2; out[3] = h2;
}

/* compute_V_collect_spike_learnFF_fast for every neuron (learning off, no gap junctions).
 * noise: normals [nV1] of this step (NULL if no noise); ff: normals [nV1][cap] for the
 * feed-forward failure draws.  Writes sInfo (the step's spike word). */
/* compute_V_collect_spike_learnFF (src/coredynamics.cu:427-845, learning off): the step taken
 * when dt exceeds the shortest refractory period, several spikes per step.  Pass after pass:
 * conductances at tBack from the previous interval start (new_t0), inputs after new_t0 and
 * before tBack into g0, end-of-step inputs into g1 on the first pass only, RK2 over dt - tBack,
 * spike -> tBack = tsp + tRef and another pass while tBack < dt.  With tau_noise = 0 the noise
 * is divided by dt on every pass, as the reference does. */
static int compute_v_multi(orc_v1 *o, const float *lgnSInfo, const float *noise, const float *ff, int cap) {
    const pv1_v1_config *c = &o->c;
    const int nV1 = o->nV1;
    const float dt = c->dt;
    int nerr = 0;
#pragma omp parallel for schedule(static) reduction(+ : nerr)
    for (int i = 0; i < nV1; i++) {
        const int it = otype(o, i % o->bs);
        const float vR = c->vR[it], vThres = c->vThres[it], gL = c->gL[it], Cm = c->C[it];
        const float tRef = c->tRef[it], vT = c->vT[it], deltaT = c->deltaT[it];
        const float tau_w = c->tau_w[it], aa = c->a[it], bb = c->b[it];
        const float tonic = o->tonic[i];
        float v0 = o->v[i];
        float w0 = c->iModel == 1 ? o->w[i] : 0.0f;
        float tBack = o->tBack[i];
        const float depC = orc_adex_depc(c->vL, vT, gL, aa, deltaT, tonic);
        const float noise0 = c->tau_noise > 0 ? o->lastNoise[i] : 0.f;
        float ge[PV1_MAX_NG], he[PV1_MAX_NG], gi[PV1_MAX_NG], hi[PV1_MAX_NG];
        float gE_t1 = 0.0f, gI_t1 = 0.0f;
        for (uint32_t ig = 0; ig < c->ngE; ig++) {
            float g = o->gE[ig * nV1 + i], h = o->hE[ig * nV1 + i];
            ge[ig] = g;
            he[ig] = h;
            ocond_decay(&o->cE, &g, &h, dt, (int)ig);
            o->gE[ig * nV1 + i] = g;
            o->hE[ig * nV1 + i] = h;
            gE_t1 += g;
        }
        for (uint32_t ig = 0; ig < c->ngI; ig++) {
            float g = o->gI[ig * nV1 + i], h = o->hI[ig * nV1 + i];
            gi[ig] = g;
            hi[ig] = h;
            ocond_decay(&o->cI, &g, &h, dt, (int)ig);
            o->gI[ig * nV1 + i] = g;
            o->hI[ig * nV1 + i] = h;
            gI_t1 += g;
        }
        float g0[PV1_MAX_NG], h0[PV1_MAX_NG], g1[PV1_MAX_NG], h1[PV1_MAX_NG];
        for (uint32_t ig = 0; ig < c->ngFF; ig++) {
            g1[ig] = o->gFF[ig * nV1 + i];
            h1[ig] = o->hFF[ig * nV1 + i];
            g0[ig] = g1[ig];
            h0[ig] = h1[ig];
            ocond_decay(&o->cFF, &g1[ig], &h1[ig], dt, (int)ig);
        }
        const float noiseRatio = c->noiseOnTonic ? tonic : 1.0f;
        float noise1 = sqrtf(2 * c->noisyDep[it] * (vT - vR) * noiseRatio * dt);
        const float pf = c->synFailFF[it], nSyn = c->synPerConFF[it];
        if (noise1 > 0) {
            noise1 *= noise ? noise[i] : 0.f;
            if (c->tau_noise > 0) {
                noise1 /= c->tau_noise;
                float hk1 = -noise0 / c->tau_noise;
                float hk2 = -(noise0 + dt * hk1 + noise1) / c->tau_noise;
                noise1 += noise0 + dt * (hk1 + hk2) / 2;
                o->lastNoise[i] = noise1;
            }
        }
        int backingUp = tBack < dt && tBack > 0;
        float new_t0 = 0.f, sInfo = 0.f, v = v0, w = w0, tsp = 0.f;
        unsigned spikeCount = 0;
        const uint32_t m = o->nLGN[i];
        float *f = (float *)malloc(sizeof(float) * (m ? m : 1));
        int nff = 0, pass = 0;
        o->dep[i] = depC + noise1;
        do {
            const float dtBack = backingUp ? tBack - new_t0 : 0.f;
            if (backingUp)
                for (uint32_t ig = 0; ig < c->ngFF; ig++) ocond_decay(&o->cFF, &g0[ig], &h0[ig], dtBack, (int)ig);
            for (uint32_t q = 0; q < m; q++) {
                const size_t lid = (size_t)q * nV1 + i;
                if (spikeCount == 0) f[q] = o->sLGN[lid];
                const float sFF = lgnSInfo[o->lgnId[lid]];
                const unsigned nspFF = (unsigned)floorf(sFF);
                const float tspFF = (sFF - nspFF) * dt;
                if (nspFF > 0 && tspFF >= new_t0) {
                    if (spikeCount == 0 && pf > 0) {
                        const float nstd = sqrtf(pf * (1 - pf) / nSyn);
                        const float rnd = (ff && nff < cap) ? ff[(size_t)i * cap + nff] : 0.f;
                        nff++;
                        f[q] *= 1 - pf + nstd * rnd;
                    }
                    if (f[q] > 0) {
                        const float ddt = backingUp ? tBack - tspFF : 0.f;
                        for (uint32_t ig = 0; ig < c->ngFF; ig++) {
                            const float str = f[q] * c->pFF[it * c->ngFF + ig];
                            if (backingUp && ddt > 0) ocond_input(&o->cFF, &g0[ig], &h0[ig], str * nspFF, ddt, (int)ig);
                            if (spikeCount == 0) ocond_input(&o->cFF, &g1[ig], &h1[ig], str * nspFF, dt - tspFF, (int)ig);
                        }
                    }
                }
            }
            float gE_t0 = 0.0f;
            for (uint32_t ig = 0; ig < c->ngFF; ig++) {
                gE_t0 += g0[ig];
                if (spikeCount == 0) {
                    gE_t1 += g1[ig];
                    o->gFF[ig * nV1 + i] = g1[ig];
                    o->hFF[ig * nV1 + i] = h1[ig];
                }
            }
            for (uint32_t ig = 0; ig < c->ngE; ig++) {
                if (backingUp) ocond_decay(&o->cE, &ge[ig], &he[ig], dtBack, (int)ig);
                gE_t0 += ge[ig];
            }
            float gI_t0 = 0.0f;
            for (uint32_t ig = 0; ig < c->ngI; ig++) {
                if (backingUp) ocond_decay(&o->cI, &gi[ig], &hi[ig], dtBack, (int)ig);
                gI_t0 += gi[ig];
            }
            tsp = 0.f;
            if (tBack < dt) {
                const float new_dt = dt - tBack;
                if (backingUp) { /* rk2_vFixedBefore */
                    const float A = aa * (v0 - c->vL);
                    w0 = (w0 - A) * expf(-dtBack / tau_w) + A;
                }
                float n0, n1;
                if (c->tau_noise > 0) { n0 = noise0; n1 = noise1; }
                else { noise1 /= dt; n0 = noise1; n1 = noise1; }
                orc_adex_rk2(c->vE, c->vI, c->vL, gE_t0, gI_t0, gE_t1, gI_t1, depC, gL, vT, deltaT, Cm, aa, tau_w,
                             v0, w0, new_dt, n0, n1, &v, &w);
                if (v > vThres) {
                    new_t0 = tBack;
                    float ratio;
                    orc_adex_spike(vThres, v0, v, w, bb, &ratio, &w0);
                    tsp = new_t0 + ratio * new_dt;
                    if (!(tsp >= 0)) nerr++;
                    sInfo += tsp;
                    spikeCount++;
                    tBack = tsp + tRef;
                    backingUp = tBack < dt;
                    if (backingUp) v0 = vR; /* reset */
                    else v = vR;
                } else {
                    if (tBack > 0) tBack = 0;
                    backingUp = 0;
                }
            }
            if (tBack >= dt) { /* rk2_vFixedAfter */
                v = vR;
                const float A = aa * (v - c->vL);
                w = (w0 - A) * expf(-(dt - tsp) / tau_w) + A;
                tBack -= dt;
            }
            if (++pass >= 64 && backingUp) {
                nerr++;
                break;
            }
        } while (backingUp);
        free(f);
        if (spikeCount > 0) {
            sInfo /= spikeCount * dt;
            sInfo += spikeCount;
        } else {
            sInfo = v;
        }
        o->sInfo[i] = sInfo;
        o->v[i] = v;
        if (c->iModel == 1) o->w[i] = w;
        o->tBack[i] = tBack;
    }
    return nerr;
}

int orc_v1_compute_v(orc_v1 *o, const float *lgnSInfo, const float *noise, const float *ff, int cap) {
    const pv1_v1_config *c = &o->c;
    const int nV1 = o->nV1;
    const float dt = c->dt;
    int nerr = 0;
    {
        float minTRef = c->tRef[0];
        for (uint32_t j = 1; j < c->nType; j++) minTRef = c->tRef[j] < minTRef ? c->tRef[j] : minTRef;
        if (dt > minTRef) return compute_v_multi(o, lgnSInfo, noise, ff, cap);
    }
#pragma omp parallel for schedule(static) reduction(+ : nerr)
    for (int i = 0; i < nV1; i++) {
        const int local = i % o->bs;
        const int it = otype(o, local);
        const float vR = c->vR[it], vThres = c->vThres[it], gL = c->gL[it], Cm = c->C[it];
        const float tRef = c->tRef[it], vT = c->vT[it], deltaT = c->deltaT[it];
        const float tau_w = c->tau_w[it], aa = c->a[it], bb = c->b[it];
        const float tonic = o->tonic[i];
        float v0 = o->v[i];
        float w0 = c->iModel == 1 ? o->w[i] : 0.0f;
        float tBack = o->tBack[i];
        const float depC = orc_adex_depc(c->vL, vT, gL, aa, deltaT, tonic);
        float noise0 = c->tau_noise > 0 ? o->lastNoise[i] : 0.f;
        float ge[PV1_MAX_NG], he[PV1_MAX_NG], gi[PV1_MAX_NG], hi[PV1_MAX_NG];
        float gE_t1 = 0.0f, gI_t1 = 0.0f;
        for (uint32_t ig = 0; ig < c->ngE; ig++) {
            float g = o->gE[ig * nV1 + i], h = o->hE[ig * nV1 + i];
            ge[ig] = g;
            he[ig] = h;
            ocond_decay(&o->cE, &g, &h, dt, (int)ig);
            o->gE[ig * nV1 + i] = g;
            o->hE[ig * nV1 + i] = h;
            gE_t1 += g;
        }
        for (uint32_t ig = 0; ig < c->ngI; ig++) {
            float g = o->gI[ig * nV1 + i], h = o->hI[ig * nV1 + i];
            gi[ig] = g;
            hi[ig] = h;
            ocond_decay(&o->cI, &g, &h, dt, (int)ig);
            o->gI[ig * nV1 + i] = g;
            o->hI[ig * nV1 + i] = h;
            gI_t1 += g;
        }
        float g0[PV1_MAX_NG], h0[PV1_MAX_NG], g1[PV1_MAX_NG], h1[PV1_MAX_NG];
        for (uint32_t ig = 0; ig < c->ngFF; ig++) {
            g1[ig] = o->gFF[ig * nV1 + i];
            h1[ig] = o->hFF[ig * nV1 + i];
            g0[ig] = g1[ig];
            h0[ig] = h1[ig];
            ocond_decay(&o->cFF, &g1[ig], &h1[ig], dt, (int)ig);
        }
        const float noiseRatio = c->noiseOnTonic ? tonic : 1.0f;
        float noise1 = sqrtf(2 * c->noisyDep[it] * (vT - vR) * noiseRatio * dt);
        const float pf = c->synFailFF[it], nSyn = c->synPerConFF[it];
        if (noise1 > 0) {
            noise1 *= noise ? noise[i] : 0.f;
            if (c->tau_noise > 0) {
                noise1 /= c->tau_noise;
                float hk1 = -noise0 / c->tau_noise;
                float hk2 = -(noise0 + dt * hk1 + noise1) / c->tau_noise;
                noise1 += noise0 + dt * (hk1 + hk2) / 2;
                o->lastNoise[i] = noise1;
            }
        }
        const int backingUp = tBack < dt && tBack > 0;
        o->dep[i] = depC + noise1;
        if (backingUp)
            for (uint32_t ig = 0; ig < c->ngFF; ig++) ocond_decay(&o->cFF, &g0[ig], &h0[ig], tBack, (int)ig);
        int nff = 0;
        for (uint32_t q = 0; q < o->nLGN[i]; q++) {
            const size_t lid = (size_t)q * nV1 + i;
            float f = o->sLGN[lid];
            const float sFF = lgnSInfo[o->lgnId[lid]];
            const unsigned nspFF = (unsigned)floorf(sFF);
            if (nspFF > 0) {
                const float tspFF = (sFF - nspFF) * dt;
                if (pf > 0) {
                    const float nstd = sqrtf(pf * (1 - pf) / nSyn);
                    const float rnd = (ff && nff < cap) ? ff[(size_t)i * cap + nff] : 0.f;
                    nff++;
                    f *= 1 - pf + nstd * rnd;
                }
                if (f > 0) {
                    float ddt = backingUp ? tBack - tspFF : 0.f;
                    for (uint32_t ig = 0; ig < c->ngFF; ig++) {
                        const float str = f * c->pFF[it * c->ngFF + ig];
                        if (backingUp && ddt > 0) ocond_input(&o->cFF, &g0[ig], &h0[ig], str * nspFF, ddt, (int)ig);
                        ocond_input(&o->cFF, &g1[ig], &h1[ig], str * nspFF, dt - tspFF, (int)ig);
                    }
                }
            }
        }
        float gE_t0 = 0.0f;
        for (uint32_t ig = 0; ig < c->ngFF; ig++) {
            gE_t0 += g0[ig];
            gE_t1 += g1[ig];
            o->gFF[ig * nV1 + i] = g1[ig];
            o->hFF[ig * nV1 + i] = h1[ig];
        }
        for (uint32_t ig = 0; ig < c->ngE; ig++) {
            if (backingUp) ocond_decay(&o->cE, &ge[ig], &he[ig], tBack, (int)ig);
            gE_t0 += ge[ig];
        }
        float gI_t0 = 0.0f;
        for (uint32_t ig = 0; ig < c->ngI; ig++) {
            if (backingUp) ocond_decay(&o->cI, &gi[ig], &hi[ig], tBack, (int)ig);
            gI_t0 += gi[ig];
        }
        /* AdEx: set_p0/set_p1, rk2_vFixedBefore, rk2, compute_spike_time, reset, rk2_vFixedAfter */
        float v = v0, w = w0, tsp = 0.f;
        int spiked = 0;
        if (tBack < dt) {
            const float new_dt = dt - tBack;
            if (backingUp) {
                float A = aa * (v0 - c->vL);
                w0 = (w0 - A) * expf(-tBack / tau_w) + A;
            }
            float n0, n1;
            if (c->tau_noise > 0) { n0 = noise0; n1 = noise1; }
            else { noise1 /= dt; n0 = noise1; n1 = noise1; }
            orc_adex_rk2(c->vE, c->vI, c->vL, gE_t0, gI_t0, gE_t1, gI_t1, depC, gL, vT, deltaT, Cm, aa, tau_w,
                         v0, w0, new_dt, n0, n1, &v, &w);
            if (v > vThres) {
                float ratio;
                orc_adex_spike(vThres, v0, v, w, bb, &ratio, &w0);
                tsp = tBack + ratio * new_dt;
                if (!(tsp >= 0)) nerr++;
                spiked = 1;
                tBack = tsp + tRef;
                v = vR;
            } else if (tBack > 0) {
                tBack = 0;
            }
        }
        if (tBack >= dt) {
            v = vR;
            const float A = aa * (v - c->vL);
            w = (w0 - A) * expf(-(dt - tsp) / tau_w) + A;
            tBack -= dt;
        }
        o->sInfo[i] = spiked ? 1.0f + tsp / dt : v;
        o->v[i] = v;
        if (c->iModel == 1) o->w[i] = w;
        o->tBack[i] = tBack;
    }
    return nerr;
}

/* recal_G_mat_nd_fast: near-neighbour delivery of this step's spikes.  Spikers of a block
 * are taken in ascending neuron order (E before I).  near: normals [nV1][cap] for the
 * failure draws (consumed only when some failure rate > 0). */
int orc_v1_deliver_near(orc_v1 *o, const float *near, int cap) {
    const pv1_v1_config *c = &o->c;
    const int nV1 = o->nV1, bs = o->bs;
    const float dt = c->dt;
    int condRng = 0;
    for (uint32_t q = 0; q < c->nType * c->nType; q++) if (c->synFail[q] > 0) condRng = 1;
    for (uint32_t q = 0; q < c->nType; q++) if (c->synFailFF[q] > 0) condRng = 1;
    /* unit conductances of every spiker (output_g/h of compute_V) */
    float *og = (float *)calloc((size_t)nV1 * PV1_MAX_NG, sizeof(float));
    float *oh = (float *)calloc((size_t)nV1 * PV1_MAX_NG, sizeof(float));
    for (int i = 0; i < nV1; i++) {
        const float sI = o->sInfo[i];
        if (sI >= 1) {
            const float nsp = floorf(sI), tsp = (sI - nsp) * dt;
            const int isE = (i % bs) < o->nE;
            const int ng = isE ? (int)c->ngE : (int)c->ngI;
            for (int ig = 0; ig < ng; ig++) {
                float g = 0.f, h = 0.f;
                ocond_input(isE ? &o->cE : &o->cI, &g, &h, nsp, dt - tsp, ig);
                og[(size_t)i * PV1_MAX_NG + ig] = g;
                oh[(size_t)i * PV1_MAX_NG + ig] = h;
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nV1; i++) {
        const int b = i / bs, local = i % bs;
        const int it = otype(o, local);
        float lgE[PV1_MAX_NG] = {0, 0}, lhE[PV1_MAX_NG] = {0, 0}, lgI[PV1_MAX_NG] = {0, 0}, lhI[PV1_MAX_NG] = {0, 0};
        int ndraw = 0;
        for (uint32_t ib = 0; ib < o->nNearNB[b]; ib++) {
            const int nb = (int)o->nbId[(size_t)b * o->nnb + ib];
            const float *colbase = o->conMat + ((size_t)(b * o->nnb + ib) * bs) * bs + local;
            for (int pass = 0; pass < 2; pass++) {
                int rank = 0;
                const int j0 = pass == 0 ? 0 : o->nE, j1 = pass == 0 ? o->nE : bs;
                for (int j = j0; j < j1; j++) {
                    const int pre = nb * bs + j;
                    if (!(o->sInfo[pre] >= 1)) continue;
                    float strength = colbase[(size_t)j * bs];
                    if (strength > 0) {
                        if (condRng) {
                            int jtype = pass == 0 ? 0 : (int)c->nTypeE;
                            const int ja = pass == 0 ? 0 : (int)c->nTypeE, jb = pass == 0 ? (int)c->nTypeE : (int)c->nType;
                            for (int jj = ja; jj < jb; jj++)
                                if ((uint32_t)rank < c->typeAcc[jj]) { jtype = jj; break; }
                            const int idx = jtype * (int)c->nType + it;
                            const float lp = c->synFail[idx];
                            const float nstd = sqrtf(lp * (1 - lp) / c->synPerCon[idx]);
                            const float rnd = (near && ndraw < cap) ? near[(size_t)i * cap + ndraw] : 0.f;
                            ndraw++;
                            strength *= 1 - lp + nstd * rnd;
                        }
                        if (strength > 0) {
                            if (pass == 0) {
                                for (uint32_t ig = 0; ig < c->ngE; ig++) {
                                    const float str = strength * c->pE[it * c->ngE + ig];
                                    lgE[ig] += str * og[(size_t)pre * PV1_MAX_NG + ig];
                                    lhE[ig] += str * oh[(size_t)pre * PV1_MAX_NG + ig];
                                }
                            } else {
                                for (uint32_t ig = 0; ig < c->ngI; ig++) {
                                    const float str = strength * c->pI[it * c->ngI + ig];
                                    lgI[ig] += str * og[(size_t)pre * PV1_MAX_NG + ig];
                                    lhI[ig] += str * oh[(size_t)pre * PV1_MAX_NG + ig];
                                }
                            }
                        }
                    }
                    rank++;
                }
            }
        }
        for (uint32_t ig = 0; ig < c->ngE; ig++) { o->gE[ig * nV1 + i] += lgE[ig]; o->hE[ig * nV1 + i] += lhE[ig]; }
        for (uint32_t ig = 0; ig < c->ngI; ig++) { o->gI[ig * nV1 + i] += lgI[ig]; o->hI[ig * nV1 + i] += lhI[ig]; }
    }
    free(og);
    free(oh);
    return 0;
}

/* Delayed near delivery (noDelay = 0): the spike-word ring of depth trainDepth
 * (src/patch.cu:3813) and recal_G_mat (src/coredynamics.cu:2063-2309), without learning, gap
 * junctions or synaptic failure. */
int orc_v1_set_delays(orc_v1 *o, const float *delayMat, int trainDepth) {
    o->delayMat = delayMat;
    o->trainDepth = trainDepth;
    o->curSlot = 0;
    free(o->spikeRing);
    o->spikeRing = (float *)calloc((size_t)trainDepth * o->nV1, sizeof(float));
    return 0;
}

/* recal_G_mat (src/coredynamics.cu:2063-2309): each post neuron walks its near blocks, every
 * pre neuron of a block in index order and the two spike-word slots that can hold an event
 * arriving in this step; with a failure rate p > 0 for the (pre type, post type) pair --
 * the pre type from the pre neuron's index -- each arriving event scales its strength by
 * 1 - p + sqrt(p (1-p)/synPerCon) z with z the post's next normal draw (`near`: this step's
 * recorded draws [nV1][cap], in that order). */
int orc_v1_deliver_near_delayed(orc_v1 *o, const float *near, int cap) {
    const pv1_v1_config *c = &o->c;
    const int nV1 = o->nV1, bs = o->bs, depth = o->trainDepth;
    const float dt = c->dt;
    /* this step's spike words into the current slot */
    memcpy(o->spikeRing + (size_t)o->curSlot * nV1, o->sInfo, (size_t)nV1 * sizeof(float));
#pragma omp parallel for schedule(static)
    for (int ipost = 0; ipost < nV1; ipost++) {
        const int b = ipost / bs, local = ipost % bs;
        const int it = otype(o, local);
        float lgE[PV1_MAX_NG] = {0, 0}, lhE[PV1_MAX_NG] = {0, 0}, lgI[PV1_MAX_NG] = {0, 0}, lhI[PV1_MAX_NG] = {0, 0};
        int ndraw = 0;
        for (uint32_t ib = 0; ib < o->nNearNB[b]; ib++) {
            const size_t local_bid = (size_t)b * o->nnb + ib;
            const int bid = (int)o->nbId[local_bid];
            for (int i = 0; i < bs; i++) {
                const int ipre = bid * bs + i;
                const size_t mid = (local_bid * bs + i) * bs + local;
                const float strength = o->conMat[mid];
                if (strength == 0) continue;
                const int jtype = otype(o, i);
                const float p = c->synFail[jtype * c->nType + it];
                const float nSyn = c->synPerCon[jtype * c->nType + it];
                float time2post = o->delayMat[mid] / c->speedOfThought;
                const unsigned it2post = (unsigned)ceilf(time2post / dt);
                time2post = it2post * dt - time2post;
                int j0 = o->curSlot - (int)it2post;
                if (j0 < 0) j0 += depth;
                const int isE = i < o->nE;
                for (int j = 0; j < 2; j++) {
                    float dtsp = o->spikeRing[(size_t)((j0 + j) % depth) * nV1 + ipre];
                    if (dtsp >= 1.0f) {
                        const float nsp = floorf(dtsp);
                        dtsp = (dtsp - nsp + j) * dt - time2post;
                        if (dtsp < dt && dtsp >= 0) {
                            float f = strength;
                            if (p > 0) {
                                const float normed_std = sqrtf(p * (1 - p) / nSyn);
                                const float rnd = (near && ndraw < cap) ? near[(size_t)ipost * cap + ndraw] : 0.f;
                                ndraw++;
                                f *= 1 - p + normed_std * rnd;
                            }
                            if (f > 0) {
                                dtsp = dt - dtsp;
                                if (isE) {
                                    for (uint32_t ig = 0; ig < c->ngE; ig++)
                                        ocond_input(&o->cE, &lgE[ig], &lhE[ig], nsp * f * c->pE[it * c->ngE + ig], dtsp, (int)ig);
                                } else {
                                    for (uint32_t ig = 0; ig < c->ngI; ig++)
                                        ocond_input(&o->cI, &lgI[ig], &lhI[ig], nsp * f * c->pI[it * c->ngI + ig], dtsp, (int)ig);
                                }
                            }
                        }
                    }
                }
            }
        }
        for (uint32_t ig = 0; ig < c->ngE; ig++) { o->gE[ig * nV1 + ipost] += lgE[ig]; o->hE[ig * nV1 + ipost] += lhE[ig]; }
        for (uint32_t ig = 0; ig < c->ngI; ig++) { o->gI[ig * nV1 + ipost] += lgI[ig]; o->hI[ig * nV1 + ipost] += lhI[ig]; }
    }
    o->curSlot = (o->curSlot + 1) % depth;
    return 0;
}

/* libstdc++'s <random> as the reference's host code uses it for far synaptic failure
 * (src/coredynamics.cu:195, 319): default_random_engine is minstd_rand0 (Park-Miller,
 * x <- 16807 x mod 2^31-1, seeded with s mod m, 0 -> 1); normal_distribution<float> draws
 * uniforms through generate_canonical<float, 24> (one engine call: (x - 1) / 2^31 as float,
 * clamped below 1) and uses the Marsaglia polar method, keeping the second value of each pair
 * for its next call, whichever engine that call is given. */
typedef struct { int avail; float saved; } onormal;

static uint32_t ostd_seed(uint64_t s) {
    const uint64_t x = s % 2147483647ull;
    return x == 0 ? 1u : (uint32_t)x;
}

static uint32_t ostd_next(uint32_t *x) {
    *x = (uint32_t)(((uint64_t)*x * 16807ull) % 2147483647ull);
    return *x;
}

static float ostd_canonical(uint32_t *x) {
    const float r = (float)(ostd_next(x) - 1u) / 2147483648.0f;
    return r >= 1.0f ? nextafterf(1.0f, 0.0f) : r;
}

static float ostd_normal(onormal *d, uint32_t *x) {
    if (d->avail) {
        d->avail = 0;
        return d->saved;
    }
    float a, b, r2;
    do {
        a = (float)((double)(2.0f * ostd_canonical(x)) - 1.0);
        b = (float)((double)(2.0f * ostd_canonical(x)) - 1.0);
        r2 = a * a + b * b;
    } while (r2 > 1.0f || r2 == 0.0f);
    const float mult = sqrtf(-2.0f * logf(r2) / r2);
    d->saved = a * mult;
    d->avail = 1;
    return b * mult * 1.0f + 0.0f;
}

/* n draws from one shared normal_distribution<float>, draw q from engine who[q] (engines
 * seeded with seeds[]); for checking the restatement against libstdc++ itself. */
int orc_std_normal_draws(const uint64_t *seeds, int nEng, const int *who, int n, float *out) {
    uint32_t *x = (uint32_t *)malloc((size_t)(nEng > 0 ? nEng : 1) * sizeof(uint32_t));
    for (int q = 0; q < nEng; q++) x[q] = ostd_seed(seeds[q]);
    onormal d = {0, 0.f};
    for (int q = 0; q < n; q++) out[q] = ostd_normal(&d, &x[who[q]]);
    free(x);
    return 0;
}

/* uniform_real_distribution<float>(a, b) of libstdc++: one generate_canonical<float, 24>
 * draw u, then u * (b - a) + a in float. */
static float ostd_uniform(uint32_t *x, float a, float b) {
    const float u = ostd_canonical(x);
    return u * (b - a) + a;
}

/* normal_distribution draw * std + mean, redrawn while below 0 when nonNeg (the sampling
 * lambda of src/patch.cu:4416-4428 with get_incLowBound(0) or no bound). */
static float ostd_sample(onormal *d, uint32_t *x, float mean, float sd, int nonNeg) {
    float r;
    do {
        r = ostd_normal(d, x) * sd + mean;
    } while (nonNeg && r < 0.0f);
    return r;
}

/* The initial V1 state the reference draws on the host (src/patch.cu:4405-4540), on one
 * default_random_engine seeded with seed and one normal_distribution<float> shared by every
 * draw (the sampling lambda's function-local static): per type, w0 (iModel = 1) then v0
 * (uniform in [vR, vT) when use_v0 or tonicMax > 1, else vR + (vT - vR) tonicDep), block by
 * block; then per type and feed-forward species the block's g then its h (zeroed for neurons
 * without LGN input); then per type the cortical E species and the I species, block by block,
 * g then h.  Layouts: gFF/hFF [ngFF][nV1], gE/hE [ngE][nV1], gI/hI [ngI][nV1]; w0 [nType][2]
 * (mean, std), gFF0/gE0/gI0 [nType][ng][4] (g mean, g rel. std, h mean, h rel. std). */
int orc_host_init_state(const pv1_v1_config *c, uint64_t seed, const float *tonicDep, const uint32_t *nLGNperV1,
                        int use_v0, float tonicMax, const float *w0, const float *gFF0, const float *gE0,
                        const float *gI0, float *v, float *w, float *gFF, float *hFF, float *gE, float *hE,
                        float *gI, float *hI) {
    const size_t bs = c->blockSize, nblock = c->nblock, nV1 = bs * nblock;
    const int nType = (int)c->nType;
    size_t acc[PV1_MAX_NTYPE + 1];
    acc[0] = 0;
    for (int j = 0; j < nType; j++) acc[j + 1] = c->typeAcc[j];
    uint32_t x = ostd_seed(seed);
    onormal d = {0, 0.f};
    for (int i = 0; i < nType; i++) {
        if (c->iModel == 1) {
            for (size_t b = 0; b < nblock; b++)
                for (size_t j = acc[i]; j < acc[i + 1]; j++)
                    w[b * bs + j] = ostd_sample(&d, &x, w0[i * 2 + 0], w0[i * 2 + 1], 0);
        }
        if (use_v0 || tonicMax > 1.0f) {
            for (size_t b = 0; b < nblock; b++)
                for (size_t j = acc[i]; j < acc[i + 1]; j++) v[b * bs + j] = ostd_uniform(&x, c->vR[i], c->vT[i]);
        } else {
            for (size_t b = 0; b < nblock; b++)
                for (size_t j = acc[i]; j < acc[i + 1]; j++)
                    v[b * bs + j] = c->vR[i] + (c->vT[i] - c->vR[i]) * tonicDep[b * bs + j];
        }
    }
    if (c->iModel != 1 && w)
        for (size_t q = 0; q < nV1; q++) w[q] = 0.0f;
    for (int i = 0; i < nType; i++)
        for (uint32_t k = 0; k < c->ngFF; k++) {
            const float *q = gFF0 + ((size_t)i * c->ngFF + k) * 4;
            for (size_t b = 0; b < nblock; b++) {
                const size_t off = k * nV1 + b * bs;
                for (size_t j = acc[i]; j < acc[i + 1]; j++) gFF[off + j] = ostd_sample(&d, &x, q[0], q[0] * q[1], 1);
                for (size_t j = acc[i]; j < acc[i + 1]; j++) hFF[off + j] = ostd_sample(&d, &x, q[2], q[2] * q[3], 1);
                for (size_t j = acc[i]; j < acc[i + 1]; j++)
                    if (nLGNperV1[b * bs + j] == 0) gFF[off + j] = hFF[off + j] = 0.0f;
            }
        }
    for (int i = 0; i < nType; i++) {
        for (uint32_t k = 0; k < c->ngE; k++) {
            const float *q = gE0 + ((size_t)i * c->ngE + k) * 4;
            for (size_t b = 0; b < nblock; b++) {
                const size_t off = k * nV1 + b * bs;
                for (size_t j = acc[i]; j < acc[i + 1]; j++) gE[off + j] = ostd_sample(&d, &x, q[0], q[0] * q[1], 1);
                for (size_t j = acc[i]; j < acc[i + 1]; j++) hE[off + j] = ostd_sample(&d, &x, q[2], q[2] * q[3], 1);
            }
        }
        for (uint32_t k = 0; k < c->ngI; k++) {
            const float *q = gI0 + ((size_t)i * c->ngI + k) * 4;
            for (size_t b = 0; b < nblock; b++) {
                const size_t off = k * nV1 + b * bs;
                for (size_t j = acc[i]; j < acc[i + 1]; j++) gI[off + j] = ostd_sample(&d, &x, q[0], q[0] * q[1], 1);
                for (size_t j = acc[i]; j < acc[i + 1]; j++) hI[off + j] = ostd_sample(&d, &x, q[2], q[2] * q[3], 1);
            }
        }
    }
    return 0;
}

/* Host engines of the far synaptic failure: engine i seeded with seed + i
 * (src/patch.cu:4224-4228); the far delivery runs per chunk of blocks (nChunk as
 * src/patch.cu:3430-3437 splits them), each with its own normal_distribution. */
int orc_v1_set_far_failure(orc_v1 *o, uint64_t seed, int nChunk) {
    free(o->farEng);
    o->farEng = (uint32_t *)malloc((size_t)o->nV1 * sizeof(uint32_t));
    for (int i = 0; i < o->nV1; i++) o->farEng[i] = ostd_seed(seed + (uint64_t)i);
    o->nChunk = nChunk < 1 ? 1 : nChunk;
    return 0;
}

/* recal_G_vec for post neuron i (src/coredynamics.cu:276-333): advance its synapses' ring
 * slots and, when deliver, add the arrivals (sum_G); dist: the chunk's normal_distribution
 * (used when some failure rate > 0). */
static void ofar_post(orc_v1 *o, int i, int deliver, onormal *dist) {
    const pv1_v1_config *c = &o->c;
    const int nV1 = o->nV1, bs = o->bs;
    const float dt = c->dt;
    const int itype = otype(o, i % bs);
    float lgE[PV1_MAX_NG] = {0, 0}, lhE[PV1_MAX_NG] = {0, 0}, lgI[PV1_MAX_NG] = {0, 0}, lhI[PV1_MAX_NG] = {0, 0};
    for (size_t e = o->vecOff[i]; e < o->vecOff[i + 1]; e++) {
        const uint32_t pre = o->vecID[e];
        const int tid = (int)(pre % bs);
        const float strength = o->conVec[e];
        float time2post = o->delayVec[e] / c->speedOfThought;
        const int preE = tid < o->nE;
        const ocond *cd = preE ? &o->cE : &o->cI;
        const int ng = preE ? (int)c->ngE : (int)c->ngI;
        float *lg = preE ? lgE : lgI, *lh = preE ? lhE : lhI;
        const int jtype = otype(o, tid);
        const float p = c->synFail[jtype * c->nType + itype];
        const float nSyn = c->synPerCon[jtype * c->nType + itype];
        const unsigned it2post = (unsigned)ceilf(time2post / dt);
        time2post = it2post * dt - time2post;
        int k0 = (int)o->slot[e] - (int)it2post;
        if (k0 < 0) k0 += (int)o->depth[e];
        o->slot[e] = (o->slot[e] + 1) % o->depth[e];
        if (!deliver || c->noFarDelay) continue;
        for (int k = 0; k < 2; k++) {
            float dtsp = o->ring[o->ringOff[e] + (size_t)((k0 + k) % (int)o->depth[e])];
            if (dtsp >= 1.0f) {
                const unsigned nsp = (unsigned)floorf(dtsp);
                dtsp = (dtsp - nsp + k) * dt - time2post;
                if (dtsp < dt && dtsp >= 0) {
                    float f = strength;
                    if (p > 0) {
                        const float normed_std = sqrtf(p * (1 - p) / nSyn);
                        const float rnd = ostd_normal(dist, &o->farEng[i]);
                        f *= 1 - p + normed_std * rnd;
                    }
                    if (f > 0) {
                        dtsp = dt - dtsp;
                        for (int ig = 0; ig < ng; ig++) {
                            const float ip = preE ? c->pE[itype * c->ngE + ig] : c->pI[itype * c->ngI + ig];
                            ocond_input(cd, &lg[ig], &lh[ig], nsp * f * ip, dtsp, ig);
                        }
                    }
                }
            }
        }
    }
    if (deliver && o->vecOff[i + 1] > o->vecOff[i] && !c->noFarDelay) {
        for (uint32_t ig = 0; ig < c->ngE; ig++) { o->gE[ig * nV1 + i] += lgE[ig]; o->hE[ig * nV1 + i] += lhE[ig]; }
        for (uint32_t ig = 0; ig < c->ngI; ig++) { o->gI[ig * nV1 + i] += lgI[ig]; o->hI[ig * nV1 + i] += lhI[ig]; }
    }
}

/* Far delivery: fill_fSpikeTrain, then recal_G_vec + sum_G when some far presynaptic neuron
 * spiked (sInfo > 1) this step, else only the ring slots advance (src/patch.cu:6596-6648).
 * noFarDelay = 1 reproduces the reference's empty loop (far input dropped).  With far
 * synaptic failure each chunk's posts run in order, sharing the chunk's normal_distribution. */
int orc_v1_deliver_far(orc_v1 *o) {
    if (!o->anyFar) return 0;
    const pv1_v1_config *c = &o->c;
    const int nV1 = o->nV1, bs = o->bs;
    int farSpiked = 0;
    for (int i = 0; i < nV1; i++)
        for (size_t e = o->vecOff[i]; e < o->vecOff[i + 1]; e++) {
            const float sI = o->sInfo[o->vecID[e]];
            if (sI > 1.0f) farSpiked = 1;
            o->ring[o->ringOff[e] + o->slot[e]] = sI;
        }
    if (!farSpiked) {
        for (size_t e = 0; e < o->nFar; e++) o->slot[e] = (o->slot[e] + 1) % o->depth[e];
        return 0;
    }
    int fail = 0;
    for (uint32_t q = 0; q < c->nType * c->nType; q++) if (c->synFail[q] > 0) fail = 1;
    if (!fail || c->noFarDelay) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nV1; i++) ofar_post(o, i, 1, NULL);
        return 0;
    }
    if (!o->farEng) return -1;
    const int nCh = o->nChunk > o->nblock ? o->nblock : o->nChunk;
    const int split = o->nblock % nCh, rem = o->nblock / nCh, maxC = rem + (split > 0);
#pragma omp parallel for schedule(dynamic)
    for (int q = 0; q < nCh; q++) {
        const int b0 = q < split ? q * maxC : split * maxC + (q - split) * rem;
        const int nb = q < split ? maxC : rem;
        onormal dist = {0, 0.f};
        for (int i = b0 * bs; i < (b0 + nb) * bs; i++) ofar_post(o, i, 1, &dist);
    }
    return 0;
}

/* rand_spInit with initial spikes (src/coredynamics.cu:5-146) and the delivery before the
 * step loop (src/patch.cu:5687-5888), consuming the uniforms u [nV1][capU] (nu [nV1] of them
 * each) and the near failure normals z [nV1][capZ] the device drew.  The initial spikers of a
 * block are numbered by thread index (the device's order).  Writes the spike-word history
 * [depth][nV1] to H (may be NULL); returns the number of neurons whose draw counts differ. */
int orc_v1_init_spikes(orc_v1 *o, const float *sp0, uint32_t SCsplit, int depth, const float *u,
                       const uint32_t *nu, uint32_t capU, const float *z, const uint32_t *nz,
                       uint32_t capZ, float *Hout) {
    const pv1_v1_config *c = &o->c;
    const int nV1 = o->nV1, bs = o->bs, nE = o->nE, nI = o->nI;
    const float dt = c->dt;
    int has = 0, mism = 0;
    for (uint32_t q = 0; q < 2 * c->nType; q++) if (sp0[q] > 0) has = 1;
    float *H = (float *)calloc((size_t)depth * nV1, sizeof(float));
    for (int id = 0; id < nV1; id++) {
        const int itype = otype(o, id % bs);
        const float *ui = u + (size_t)id * capU;
        uint32_t k = 0;
#define ODRAW() (k < nu[id] && k < capU ? ui[k++] : (k++, 2.0f))
        const float r0 = ODRAW();
        const float chance = sp0[itype * 2 + (o->nLGN[id] > SCsplit ? 0 : 1)];
        const float tRef = c->tRef[itype];
        float v = o->v[id], ref = 0.f, sInfo = v;
        if (chance > 0 && r0 < chance) {
            const float tsp = ODRAW();
            sInfo = 1.0f + tsp;
            const float tb = tRef - (1 - tsp) * dt;
            if (tb > 0) o->tBack[id] = tb;
            const float v0 = c->vR[itype];
            v = v0;
            o->v[id] = v0;
            if (c->iModel == 1) {
                const float tw = c->tau_w[itype];
                const float A = c->a[itype] * (v0 - c->vL) * tw;
                const float w0 = o->w[id] + c->b[itype];
                o->w[id] = (w0 - A) * expf(-dt * (1 - tsp) / tw) + A;
            }
            ref = (1 - tsp) * dt + tRef - dt;
        }
        H[id] = sInfo;
        for (int q = depth - 1; q > 0; q--) {
            float word;
            if (ref < dt) {
                if (ref < 0) ref = 0;
                if (ODRAW() < chance * (dt - ref) / dt) {
                    const float tsp = ODRAW() * (dt - ref) / dt;
                    word = 1.0f + tsp;
                    ref = tRef + (1 - tsp) * dt;
                } else {
                    word = v;
                }
            } else {
                word = c->vR[itype];
            }
            H[(size_t)q * nV1 + id] = word;
            ref -= dt;
        }
#undef ODRAW
        if (k != nu[id]) mism++;
    }
    if (Hout) memcpy(Hout, H, (size_t)depth * nV1 * sizeof(float));
    if (!has) {
        free(H);
        return mism;
    }
    const float *Hlast = H + (size_t)(depth - 1) * nV1;
    if (c->noDelay) {
        /* output_g/h of the initial spikers, compacted per block (rand_spInit :85-116) */
        const size_t ncb = (size_t)nE * c->ngE + (size_t)nI * c->ngI;
        float *og = (float *)calloc(ncb * o->nblock, sizeof(float));
        float *oh = (float *)calloc(ncb * o->nblock, sizeof(float));
        for (int b = 0; b < o->nblock; b++) {
            int npE = 0, npI = 0;
            for (int l = 0; l < bs; l++)
                if (H[b * bs + l] >= 1) { if (l < nE) npE++; else npI++; }
            int sE = 0, sI = 0;
            for (int l = 0; l < bs; l++) {
                const float w = H[b * bs + l];
                if (!(w >= 1)) continue;
                const float tsp = (w - 1) * dt;
                const int isE = l < nE;
                const int ng = isE ? (int)c->ngE : (int)c->ngI;
                const int sid = isE ? sE++ : sI++;
                for (int ig = 0; ig < ng; ig++) {
                    float g = 0.f, h = 0.f;
                    ocond_input(isE ? &o->cE : &o->cI, &g, &h, 1.f, dt - tsp, ig);
                    const size_t r = isE ? (size_t)ig * npE + sid : (size_t)ig * npI + (size_t)npE * c->ngE + sid;
                    og[b * ncb + r] = g;
                    oh[b * ncb + r] = h;
                }
            }
        }
        /* recal_G_mat_nd on the history slot depth-1 (:2366-2608) */
        for (int ipost = 0; ipost < nV1; ipost++) {
            const int b = ipost / bs, local = ipost % bs, itype = otype(o, local);
            float lgE[PV1_MAX_NG] = {0, 0}, lhE[PV1_MAX_NG] = {0, 0}, lgI[PV1_MAX_NG] = {0, 0}, lhI[PV1_MAX_NG] = {0, 0};
            uint32_t kz = 0;
            for (uint32_t ib = 0; ib < o->nNearNB[b]; ib++) {
                const int bid = (int)o->nbId[(size_t)b * o->nnb + ib];
                const float *col = o->conMat + ((size_t)(b * o->nnb + ib) * bs) * bs + local;
                for (int i = 0; i < bs; i++) {
                    float strength = col[(size_t)i * bs];
                    if (!(strength != 0 && Hlast[bid * bs + i] > 0)) continue;
                    const int jtype = otype(o, i);
                    const float p = c->synFail[jtype * c->nType + itype];
                    if (p > 0) {
                        const float nstd = sqrtf(p * (1 - p) / c->synPerCon[jtype * c->nType + itype]);
                        const float rnd = (z && kz < nz[ipost] && kz < capZ) ? z[(size_t)ipost * capZ + kz] : 0.f;
                        kz++;
                        strength *= 1 - p + nstd * rnd;
                    }
                    if (strength > 0) {
                        const int isE = i < nE;
                        const size_t base = (size_t)bid * ncb + (isE ? (size_t)i * c->ngE : (size_t)nE * c->ngE + (size_t)(i - nE) * c->ngI);
                        if (isE) {
                            for (uint32_t ig = 0; ig < c->ngE; ig++) {
                                const float str = strength * c->pE[itype * c->ngE + ig];
                                lgE[ig] += str * og[base + ig];
                                lhE[ig] += str * oh[base + ig];
                            }
                        } else {
                            for (uint32_t ig = 0; ig < c->ngI; ig++) {
                                const float str = strength * c->pI[itype * c->ngI + ig];
                                lgI[ig] += str * og[base + ig];
                                lhI[ig] += str * oh[base + ig];
                            }
                        }
                    }
                }
            }
            if (nz && kz != nz[ipost]) mism++;
            for (uint32_t ig = 0; ig < c->ngE; ig++) { o->gE[ig * nV1 + ipost] += lgE[ig]; o->hE[ig * nV1 + ipost] += lhE[ig]; }
            for (uint32_t ig = 0; ig < c->ngI; ig++) { o->gI[ig * nV1 + ipost] += lgI[ig]; o->hI[ig * nV1 + ipost] += lhI[ig]; }
        }
        free(og);
        free(oh);
    } else {
        /* recal_G_mat with the ring's current slot 0 (src/patch.cu:5760-5770); the loop then
         * starts again at slot 0 */
        if (!o->spikeRing || o->trainDepth != depth) {
            free(H);
            return -1;
        }
        memcpy(o->spikeRing, H, (size_t)depth * nV1 * sizeof(float));
        memcpy(o->sInfo, H, (size_t)nV1 * sizeof(float));
        o->curSlot = 0;
        orc_v1_deliver_near_delayed(o, z, (int)capZ);
        o->curSlot = 0;
    }
    /* far: fill_fSpikeTrain with the history slot depth-1, recal_G_vec + sum_G */
    memcpy(o->sInfo, Hlast, (size_t)nV1 * sizeof(float));
    orc_v1_deliver_far(o);
    free(H);
    return mism;
}

/* LGN->V1 plasticity, learning 1-4.  Derived rates of one FF type as learnFF_post computes
 * them (src/condShape.h:137-152; Float = float with its double literals) and exp_homeo =
 * exp(-dt/decayTimeHomeoFF) (src/patch.cu:1330); orc_v1_set_ff_learning below takes the
 * homeostasis totals from the current weights (src/patch.cu:4335-4352) and returns -1 for
 * modes outside 1-4 or type counts the reference does not allow. */
void orc_ff_learning_rates(const pv1_ff_learning *l, float dt, float *out) {
    const float ALTP = l->A_LGN * l->sRatioLGN;
    const float tas = (float)((double)l->tauAvg / 1000.0);
    float Ar = l->r_LTD * ALTP;
    if (l->targetFR > 0) {
        const float q = l->tauTrip / (l->tauLTD * (tas * tas));
        Ar = (float)((double)Ar * ((double)q / 1000.0 / (double)l->targetFR));
    }
    out[0] = ALTP;
    out[1] = Ar;
    out[2] = l->gmaxLGN * l->sRatioLGN;
    out[3] = l->gminLGN * l->sRatioLGN;
    out[4] = expf(-dt / l->decayTimeHomeoFF);
}

int orc_v1_set_ff_learning(orc_v1 *o, const pv1_ff_learning *l) {
    if (l->learning < 1 || l->learning > 4) return -1;
    const int nE_ = l->learning == 4 ? 0 : l->nLearnTypeFF_E;
    const int nI_ = l->learning == 2 ? l->nLearnTypeFF_I : 0;
    if (l->learning != 4 && nE_ != 1) return -1;
    for (int k = 0; k < 2; k++) {
        pv1_ff_learning q = *l;
        if (k) {
            q.tauLTP = l->tauLTP_I; q.tauLTD = l->tauLTD_I; q.tauTrip = l->tauTrip_I; q.tauAvg = l->tauAvg_I;
            q.targetFR = l->targetFR_I; q.A_LGN = l->A_LGN_I; q.r_LTD = l->r_LTD_I; q.gmaxLGN = l->gmaxLGN_I;
            q.gminLGN = l->gminLGN_I; q.sRatioLGN = l->sRatioLGN_I;
        }
        float r[5];
        orc_ff_learning_rates(&q, o->c.dt, r);
        const float t[9] = {q.tauLTP, q.tauLTD, q.tauTrip, q.tauAvg, q.targetFR, r[0], r[1], r[2], r[3]};
        memcpy(o->lt[k], t, sizeof(t));
        if (!k) o->lExpHomeo = r[4];
    }
    o->learn = l->learning;
    o->ffI = nI_;
    o->tauAvgCortical = l->tauAvgCortical;
    o->applyHomeo = l->applyHomeo; o->symmetricHomeo = l->symmetricHomeo != 0; o->rebound = l->rebound != 0;
    const size_t n = (size_t)o->nV1, nEt = (size_t)o->nE * o->nblock, nIt = (size_t)o->nI * o->nblock;
    /* learnVar's FF block (src/patch.cu:4367-4392): learning 4 has no FF->E traces */
    o->offI = l->learning == 4 ? 0 : 2 * nEt;
    o->offAvgE = o->offI + 2 * (size_t)nI_ * nIt;
    o->offAvgI = o->offAvgE + 2 * nEt;
    free(o->ffPost);
    free(o->totalFF);
    o->ffPost = (float *)calloc(o->offAvgI + nIt + 1, sizeof(float));
    o->totalFF = (float *)calloc(2 * n, sizeof(float));
    for (size_t i = 0; i < n; i++) {
        float t = 0.f;
        for (uint32_t j = 0; j < o->nLGN[i]; j++) t += o->sLGN[(size_t)j * n + i];
        o->totalFF[i] = t;
        o->totalFF[n + i] = t * l->FF_InfRatio;
    }
    return 0;
}

static inline float odecay(float x, float tau, float dt) { return x * expf(-dt / tau); }

/* The learning block of compute_V_collect_spike_learnFF_fast (src/coredynamics.cu:1631-1993)
 * for learning 1-3, after orc_v1_compute_v (whose spike words it reads): every excitatory
 * neuron with the FF->E type, and with learning 2 every inhibitory neuron with the FF->I type.
 * lgnSInfo are the step's LGN spike words, pre_start / pre_spike presynaptic trace 0 at the
 * step start and right after each LGN cell's spikes (orc_lgn_ff_pre): the inhibitory posts'
 * LTP reads trace 0 as the reference's does (its surface layer 1 + 3j with j from 0).  With
 * learning != 3 the excitatory filtered rate is left to orc_v1_learn_avg, its value at the
 * spike time stored in the second slot. */
int orc_v1_learn_ff(orc_v1 *o, const float *lgnSInfo, const float *pre_start, const float *pre_spike) {
    if (!o->learn || o->learn == 4) return -1;
    const size_t n = (size_t)o->nV1;
    const float dt = o->c.dt;
    const size_t nEt = (size_t)o->nE * o->nblock, nIt = (size_t)o->nI * o->nblock;
    for (int b = 0; b < o->nblock; b++) {
        for (int j = 0; j < o->bs; j++) {
            const int isE = j < o->nE;
            if (!isE && !o->ffI) continue;
            const float *T = o->lt[isE ? 0 : 1];
            const float tLTP = T[0], tLTD = T[1], tTrip = T[2], tAvg = T[3], tFR = T[4], ALTP = T[5], Ar = T[6];
            const float gmax = T[7], gmin = T[8];
            const size_t i = (size_t)b * o->bs + j;
            const size_t id = isE ? (size_t)b * o->nE + j : (size_t)b * o->nI + (j - o->nE);
            float *vLTD = isE ? o->ffPost : o->ffPost + o->offI;
            float *vTrip = isE ? o->ffPost + nEt : o->ffPost + o->offI + nIt;
            float *vAvg = isE ? o->ffPost + o->offAvgE + 2 * id : o->ffPost + o->offAvgI + id;
            const float sI = o->sInfo[i];
            float nsp, tsp;
            if (sI > 0) { nsp = floorf(sI); tsp = (sI - nsp) * dt; }
            else { nsp = 0; tsp = dt; }
            float LTD[2] = {vLTD[id], 0.f}, Trip[2] = {vTrip[id], 0.f}, Avg[2] = {vAvg[0], 0.f};
            if (nsp > 0) {
                LTD[1] = odecay(LTD[0], tLTD, tsp);
                Trip[1] = odecay(Trip[0], tTrip, tsp);
                Avg[1] = odecay(Avg[0], tAvg, tsp);
                if (isE && o->learn != 3) vAvg[1] = Avg[1];
            }
            const uint32_t m = o->nLGN[i];
            float new0 = 0.f, ch = 0.f, dsum = 0.f;
            if (o->applyHomeo) {
                const float f0 = o->totalFF[i], finf = o->totalFF[n + i];
                const float d = f0 - finf;
                if (d > 0 || o->symmetricHomeo) {
                    new0 = d * o->lExpHomeo + finf;
                    ch = o->applyHomeo == 1 ? new0 / f0 : (new0 - f0) / (float)m;
                } else {
                    new0 = f0;
                    ch = o->applyHomeo == 1 ? 1.f : 0.f;
                }
            }
            for (uint32_t q = 0; q < m; q++) {
                const size_t lid = (size_t)q * n + i;
                float f = o->sLGN[lid];
                if (f == 0 && !o->rebound) continue;
                if (o->applyHomeo == 1) f *= ch;
                else if (o->applyHomeo == 2) f += ch;
                const uint32_t cell = o->lgnId[lid];
                const float sFF = lgnSInfo[cell];
                const uint32_t nspFF = (uint32_t)floorf(sFF);
                const float tspFF = (sFF > 0 ? sFF - (float)nspFF : 1.f) * dt;
                if (nspFF > 0) {
                    const int c = tspFF < tsp ? 0 : 1;
                    const float delta_t = c == 0 ? tspFF : tspFF - tsp;
                    float A = Ar;
                    if (tFR > 0) A *= tLTP * Avg[c] * Avg[c];
                    const float df = odecay(LTD[c], tLTD, delta_t) * A;
                    f -= df;
                    if (o->applyHomeo) dsum -= df;
                }
                if (nsp > 0) {
                    const int early = tspFF < tsp;
                    const float lpre = early ? pre_spike[cell] : pre_start[cell];
                    const float delta_t = early ? tsp - tspFF : tsp;
                    const float df = odecay(lpre, tLTP, delta_t) * Trip[1] * ALTP;
                    if (o->applyHomeo) dsum += df;
                    f += df;
                }
                if (f < gmin) { if (o->applyHomeo) dsum += gmin - f; f = gmin; }
                if (f > gmax) { if (o->applyHomeo) dsum -= f - gmax; f = gmax; }
                o->sLGN[lid] = f;
            }
            if (o->applyHomeo) o->totalFF[i] = new0 + dsum;
            const int c = nsp > 0 ? 1 : 0;
            float delta_t = dt;
            if (nsp > 0) delta_t -= tsp;
            vLTD[id] = odecay(LTD[c] + nsp, tLTD, delta_t);
            vTrip[id] = odecay(Trip[c] + nsp, tTrip, delta_t);
            if (!isE || o->learn == 3) vAvg[0] = odecay(Avg[c] + nsp, tAvg, delta_t);
        }
    }
    return 0;
}

/* The excitatory filtered rate of learning 1, 2 and 4 advanced over the step just computed,
 * as recal_G_mat_nd_fast does after its conductance sums (src/coredynamics.cu:2866-2890): from
 * the spike-time value (second slot) when the neuron spiked, else the step start value, plus
 * the spike count, decayed by dt (1 - tsp/dt) or dt with the cortical E types' tauAvg. */
int orc_v1_learn_avg(orc_v1 *o) {
    if (!o->learn || o->learn == 3) return -1;
    const float dt = o->c.dt;
    for (int b = 0; b < o->nblock; b++) {
        for (int j = 0; j < o->nE; j++) {
            const float ps = o->sInfo[(size_t)b * o->bs + j];
            const float postNsp = floorf(ps);
            const float postTsp = ps > 0 ? ps - postNsp : 1.f;
            const int c = postNsp > 0 ? 1 : 0;
            float *vAvg = o->ffPost + o->offAvgE + 2 * ((size_t)b * o->nE + j);
            float delta_t = dt;
            if (postNsp > 0) delta_t = dt * (1 - postTsp);
            vAvg[0] = odecay(vAvg[c] + postNsp, o->tauAvgCortical, delta_t);
        }
    }
    return 0;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
