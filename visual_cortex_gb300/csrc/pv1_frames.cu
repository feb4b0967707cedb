// Framed output: pixelizeOutput (src/stats.cu:4-36) as the step loop runs it
// (src/patch.cu:6727-6790), from the record rings.  One thread per pixel walks the steps in
// order: at the first step of every ot-step frame the pixel's sum restarts, each step adds
// (sum over the pixel's m cells of floor(sInfo) -- V1 pixels, spike counts -- or of the LGN
// firing rate -- LGN pixels -- for values >= 0) / (m odt), and the sum is emitted after the
// frame's last step.
#include "pv1_internal.cuh"

namespace pv1 {
namespace {

__global__ void frames_kernel(const float *__restrict__ recSpk, int recSlots, int nV1, const float *__restrict__ lgnFr,
                              int lgnSlots, int nLGN, long long step0, int n, int ot, long long tStart,
                              const unsigned *__restrict__ pixOff, const unsigned *__restrict__ pixIds, int nPixel,
                              int nSpikePixel, float odt, float *acc, float *out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nPixel) return;
    const unsigned b = pixOff[q], m = pixOff[q + 1] - b;
    const bool isSpike = q < nSpikePixel;   // V1 spike counts; the rest LGN firing rates
    float a = acc[q];
    int k = 0;
    for (int s = 0; s < n; s++) {
        const long long t = step0 + s, it = t - tStart;
        if (it % ot == 0) a = 0.f;
        float value = 0.f;
        if (m > 0) {
            const float *row = isSpike ? recSpk + (size_t)(t % recSlots) * nV1 : lgnFr + (size_t)(t % lgnSlots) * nLGN;
            for (unsigned j = 0; j < m; j++) {
                const float sI = row[pixIds[b + j]];
                if (sI >= 0) value += isSpike ? floorf(sI) : sI;
            }
            value = __fdiv_rn(value, __fmul_rn((float)m, odt));
        }
        a = __fadd_rn(a, value);
        if ((it + 1) % ot == 0) out[(size_t)k++ * nPixel + q] = a;
    }
    acc[q] = a;
}

}  // namespace

cudaError_t launch_frames(const float *recSpk, int recSlots, int nV1, const float *lgnFr, int lgnSlots, int nLGN,
                          long long step0, int n, int ot, long long tStart, const unsigned *pixOff,
                          const unsigned *pixIds, int nPixel, int nSpikePixel, float odt, float *acc, float *out,
                          cudaStream_t st) {
    frames_kernel<<<(nPixel + 255) / 256, 256, 0, st>>>(recSpk, recSlots, nV1, lgnFr, lgnSlots, nLGN, step0, n, ot,
                                                        tStart, pixOff, pixIds, nPixel, nSpikePixel, odt, acc, out);
    return cudaGetLastError();
}

}  // namespace pv1
