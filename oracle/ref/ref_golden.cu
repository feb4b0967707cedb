// Golden vectors from the reference's own code, compiled on the host from its sources
// (test infrastructure: the oracle checks itself against these).
//
//   ref_golden cond     in out   ConductanceShape::decay_conductance and
//                                compute_single_input_conductance (src/condShape.h:13-41)
//   ref_golden adex     in out   AdEx constructor (tonic drive), set_p0/set_p1, rk2 and
//                                compute_spike_time (src/coredynamics.cuh:27-118)
//   ref_golden logistic in out   hStatic_nonlinear's a and b (src/LGN_props.h:143-170)
//   ref_golden denorm   in out   find_denorm (src/util/util.h:251-279)
//   ref_golden far      in out   fill_fSpikeTrain (src/stats.cu:114-126) + recal_G_vec
//                                (src/coredynamics.cu:181-372) over a spike sequence
//   ref_golden farfail  in out   the same with synaptic failure (host engines) per chunk
//   ref_golden learnff  in out   learnFF_pre/learnFF_post (src/condShape.h:94-152) and
//                                exp_homeo (src/patch.cu:1330): LGN->V1 learning constants
// Inputs and outputs are raw little-endian arrays; tests/golden/make_golden.py writes and
// reads them.  The AdEx struct is declared __device__ in the reference; the redefinition
// below makes its members host-callable without changing their arithmetic.
#include <cuda_runtime.h>
#include <curand_kernel.h>
#undef __device__
#define __device__ __host__ __location__(device)
#include "coredynamics.cuh"
#include "stats.cuh"
#include "LGN_props.h"
#include "util/util.h"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <vector>

template <class T>
static std::vector<T> read_all(const char *fn) {
    std::ifstream f(fn, std::ios::binary);
    f.seekg(0, std::ios::end);
    const size_t n = (size_t)f.tellg() / sizeof(T);
    f.seekg(0);
    std::vector<T> v(n);
    f.read(reinterpret_cast<char *>(v.data()), n * sizeof(T));
    return v;
}

template <class T>
static void write_all(const char *fn, const std::vector<T> &v) {
    std::ofstream f(fn, std::ios::binary);
    f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
}

static int mode_cond(const char *in, const char *out) {
    // per case: rise, decay, g, h, f, dt
    auto x = read_all<float>(in);
    std::vector<float> y;
    for (size_t q = 0; q + 6 <= x.size(); q += 6) {
        Float rt[1] = {x[q]}, dc[1] = {x[q + 1]};
        ConductanceShape c(rt, dc, 1);
        Float g1 = x[q + 2], h1 = x[q + 3], g2 = x[q + 2], h2 = x[q + 3];
        c.decay_conductance(g1, h1, x[q + 5], 0);
        c.compute_single_input_conductance(g2, h2, x[q + 4], x[q + 5], 0);
        y.insert(y.end(), {g1, h1, g2, h2});
    }
    write_all(out, y);
    return 0;
}

static int mode_adex(const char *in, const char *out) {
    // per case: w0 tau_w a b v0 vR vThres gL C tRef vT deltaT dep gE0 gI0 gE1 gI1 dt
    auto x = read_all<float>(in);
    std::vector<float> y;
    for (size_t q = 0; q + 18 <= x.size(); q += 18) {
        const float *p = &x[q];
        AdEx m(p[0], p[1], p[2], p[3], p[4], 0.f, p[5], p[6], p[7], p[8], p[9], p[10], p[11], 0.f, p[12]);
        m.set_p0(p[13], p[14], 0.f);
        m.set_p1(p[15], p[16], 0.f);
        m.rk2(p[17], 0.f, 0.f);
        const float v = m.v, w = m.w;
        m.compute_spike_time(p[17], 0.f);
        y.insert(y.end(), {m.depC, v, w, m.tsp, m.w0});
    }
    write_all(out, y);
    return 0;
}

static int mode_logistic(const char *in, const char *out) {
    // spont[n], c50[n], sharp[n]
    auto x = read_all<float>(in);
    const size_t n = x.size() / 3;
    std::vector<Float> spont(x.begin(), x.begin() + n), c50(x.begin() + n, x.begin() + 2 * n),
        sharp(x.begin() + 2 * n, x.end());
    hStatic_nonlinear h((Size)n, spont, c50, sharp);
    std::vector<float> y(h.a, h.a + n);
    y.insert(y.end(), h.b, h.b + n);
    h.freeMem();
    write_all(out, y);
    return 0;
}

static int mode_denorm(const char *in, const char *out) {
    // per case: u1, u2, MorN
    auto x = read_all<uint32_t>(in);
    std::vector<uint32_t> y;
    for (size_t q = 0; q + 3 <= x.size(); q += 3) {
        PosInt norm = 0;
        const PosInt d = find_denorm(x[q], x[q + 1], x[q + 2] != 0, norm);
        y.insert(y.end(), {d, norm});
    }
    write_all(out, y);
    return 0;
}

// far: synaptic failure off, one chunk.  farfail: the header's 8th word is nChunk, followed by
// the first engine's seed (uint64, engine i seeded seed + i as src/patch.cu:4224-4228),
// synFail[4] and synPerCon[4]; recal_G_vec is called per chunk of blocks as the step loop
// does (src/patch.cu:6597-6648, chunks split as :3430-3437).
static int mode_far(const char *in, const char *out, bool failure) {
    std::ifstream f(in, std::ios::binary);
    int32_t hd[8];
    f.read(reinterpret_cast<char *>(hd), sizeof(hd));
    const Size nV1 = hd[0], bs = hd[1], nE = hd[2], ngE = hd[3], ngI = hd[4], T = hd[5];
    const size_t nnz = (size_t)hd[6];
    uint64_t seed0 = 0;
    Float synFail[4] = {0, 0, 0, 0}, synPerCon[4] = {1, 1, 1, 1};
    const Size nblock = nV1 / bs;
    Size nChunk = 1;
    if (failure) {
        nChunk = hd[7] > 0 ? (Size)hd[7] : 1;
        if (nChunk > nblock) nChunk = nblock;
        f.read(reinterpret_cast<char *>(&seed0), sizeof(seed0));
        f.read(reinterpret_cast<char *>(synFail), sizeof(synFail));
        f.read(reinterpret_cast<char *>(synPerCon), sizeof(synPerCon));
    }
    float pr[2 + 8 + 4 + 4];
    f.read(reinterpret_cast<char *>(pr), sizeof(pr));
    const Float dt = pr[0], speed = pr[1];
    Float rE[2] = {pr[2], pr[3]}, dE[2] = {pr[4], pr[5]}, rI[2] = {pr[6], pr[7]}, dI[2] = {pr[8], pr[9]};
    Float pE[4] = {pr[10], pr[11], pr[12], pr[13]}, pI[4] = {pr[14], pr[15], pr[16], pr[17]};
    std::vector<uint32_t> nVec0(nV1), id(nnz);
    std::vector<float> str(nnz), dl(nnz), sp((size_t)T * nV1);
    f.read(reinterpret_cast<char *>(nVec0.data()), nV1 * 4);
    f.read(reinterpret_cast<char *>(id.data()), nnz * 4);
    f.read(reinterpret_cast<char *>(str.data()), nnz * 4);
    f.read(reinterpret_cast<char *>(dl.data()), nnz * 4);
    f.read(reinterpret_cast<char *>(sp.data()), sp.size() * 4);
    std::vector<Size> nVec(nVec0.begin(), nVec0.end());
    std::vector<std::vector<PosInt>> vecID(nV1);
    std::vector<std::vector<Float>> conVec(nV1), delayVec(nV1);
    std::vector<std::vector<std::vector<Float>>> fsp(nV1);
    std::vector<std::vector<Size>> depth(nV1);
    std::vector<std::vector<PosInt>> slot(nV1);
    size_t e = 0;
    for (Size i = 0; i < nV1; i++)
        for (Size j = 0; j < nVec[i]; j++, e++) {
            vecID[i].push_back(id[e]);
            conVec[i].push_back(str[e]);
            delayVec[i].push_back(dl[e]);
            // ring depth and initial -1 of src/patch.cu:3838-3850
            depth[i].push_back(static_cast<Size>(ceil((dl[e] / speed) / dt)) + 1);
            slot[i].push_back(0);
            fsp[i].push_back(std::vector<Float>(depth[i].back(), -1.0));
        }
    ConductanceShape condE(rE, dE, ngE), condI(rI, dI, ngI);
    Size typeAcc[2] = {nE, bs};
    std::vector<std::default_random_engine> gen(nV1);
    if (failure)
        for (Size i = 0; i < nV1; i++) gen[i].seed(seed0 + i);
    const Size split = nblock % nChunk, rem = nblock / nChunk, maxC = rem + (split > 0 ? 1 : 0);
    std::vector<Float> og(nV1 * 2, 0.f), oh(nV1 * 2, 0.f);
    std::vector<float> y;
    std::vector<Float> gE(ngE * nV1), hE(ngE * nV1), gI(ngI * nV1), hI(ngI * nV1);
    for (Size t = 0; t < T; t++) {
        const bool farSpiked = fill_fSpikeTrain(fsp, &sp[(size_t)t * nV1], slot, vecID, nVec, nV1);
        std::fill(gE.begin(), gE.end(), 0.f);
        std::fill(hE.begin(), hE.end(), 0.f);
        std::fill(gI.begin(), gI.end(), 0.f);
        std::fill(hI.begin(), hI.end(), 0.f);
        if (farSpiked) {
            Size block_offset = 0;
            for (Size q = 0; q < nChunk; q++) {
                const Size chunkSize = q < split ? maxC : rem;
                const size_t cn = (size_t)chunkSize * bs;
                std::vector<Float> cgE(ngE * cn), chE(ngE * cn), cgI(ngI * cn), chI(ngI * cn);
                recal_G_vec(fsp, depth, slot, og.data(), oh.data(), nVec, vecID, conVec, delayVec, cgE.data(),
                            cgI.data(), chE.data(), chI.data(), pE, pI, typeAcc, gen.data(), synFail, synPerCon, dt,
                            condE, condI, ngE, ngI, block_offset, 2, nE, bs - nE, nV1, speed, chunkSize, false, t, bs);
                const size_t o = (size_t)block_offset * bs;
                for (Size ig = 0; ig < ngE; ig++)
                    for (size_t j = 0; j < cn; j++) {
                        gE[ig * nV1 + o + j] = cgE[ig * cn + j];
                        hE[ig * nV1 + o + j] = chE[ig * cn + j];
                    }
                for (Size ig = 0; ig < ngI; ig++)
                    for (size_t j = 0; j < cn; j++) {
                        gI[ig * nV1 + o + j] = cgI[ig * cn + j];
                        hI[ig * nV1 + o + j] = chI[ig * cn + j];
                    }
                block_offset += chunkSize;
            }
        } else {
            for (Size i = 0; i < nV1; i++)
                for (Size j = 0; j < nVec[i]; j++) slot[i][j] = (slot[i][j] + 1) % depth[i][j];
        }
        y.insert(y.end(), gE.begin(), gE.end());
        y.insert(y.end(), hE.begin(), hE.end());
        y.insert(y.end(), gI.begin(), gI.end());
        y.insert(y.end(), hI.begin(), hI.end());
    }
    write_all(out, y);
    return 0;
}

// learnFF_pre / learnFF_post (src/condShape.h:94-152) and exp_homeo (src/patch.cu:1330) for
// rows {tauLTP, tauLTD, tauTrip, tauAvg, targetFR, A_LGN, r_LTD, gmaxLGN, gminLGN, sRatioLGN,
// dt, decayTimeHomeoFF}; per row the bytes of LearnVarShapeFF_E_pre, of LearnVarShapeFF_E_post
// and of exp_homeo.
static int mode_learnff(const char *in, const char *out) {
    auto x = read_all<float>(in);
    std::vector<unsigned char> y;
    for (size_t r = 0; r + 12 <= x.size(); r += 12) {
        const float *q = &x[r];
        Float tauLTP[1] = {q[0]}, tauLTD[1] = {q[1]}, tauTrip[1] = {q[2]}, A[1] = {q[5]}, rLTD[1] = {q[6]};
        LearnVarShapeFF_E_pre pre = {};
        LearnVarShapeFF_E_post post = {};
        learnFF_pre<LearnVarShapeFF_E_pre>(pre, tauLTP, 1);
        learnFF_post<LearnVarShapeFF_E_post>(post, tauLTD, tauTrip, rLTD, q[3], q[4], A, q[7], q[8], 1, q[9]);
        const Float dt = q[10], hdFF = q[11];
        const Float expHomeo = exponential(-dt / hdFF);
        const unsigned char *a = reinterpret_cast<const unsigned char *>(&pre);
        const unsigned char *b = reinterpret_cast<const unsigned char *>(&post);
        const unsigned char *c = reinterpret_cast<const unsigned char *>(&expHomeo);
        y.insert(y.end(), a, a + sizeof(pre));
        y.insert(y.end(), b, b + sizeof(post));
        y.insert(y.end(), c, c + sizeof(expHomeo));
    }
    write_all(out, y);
    return 0;
}

int main(int argc, char **argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: ref_golden cond|adex|logistic|denorm|far|farfail|learnff in out\n");
        return 2;
    }
    if (!strcmp(argv[1], "cond")) return mode_cond(argv[2], argv[3]);
    if (!strcmp(argv[1], "adex")) return mode_adex(argv[2], argv[3]);
    if (!strcmp(argv[1], "logistic")) return mode_logistic(argv[2], argv[3]);
    if (!strcmp(argv[1], "denorm")) return mode_denorm(argv[2], argv[3]);
    if (!strcmp(argv[1], "far")) return mode_far(argv[2], argv[3], false);
    if (!strcmp(argv[1], "farfail")) return mode_far(argv[2], argv[3], true);
    if (!strcmp(argv[1], "learnff")) return mode_learnff(argv[2], argv[3]);
    return 2;
}
