// Runs the reference's own GPU kernels (oracle/_ref/ref_kernels.cubin, built from its sources
// by build_ref_kernels.sh) on inputs written by tests/golden/make_ref_kernel_golden.py, and
// writes their outputs: golden vectors for the oracle and the GPU tests.  Checker only.
//
//   ref_kernel_runner <ref_kernels.cubin> <mode> <in.bundle> <out.bundle>
//
// Modes (each reference kernel launched as src/patch.cu launches it):
//   lgn     logRand_init (src/coredynamics.cu:148-177) once, then K steps of LGN_nonlinear
//           (src/discrete_input_convol.cu:1637-1821) on given convolutions
//   v1init  rand_spInit (src/coredynamics.cu:5-146)
//   v1run   rand_spInit, then T steps of compute_V_collect_spike_learnFF_fast
//           (src/coredynamics.cu:1235-2059) and recal_G_mat_nd_fast (:2609-2922) with given
//           LGN spike words written to the LGN spike surface before each step
//   magno   store_PM for magno cells (src/discrete_input_convol.cu:427-744), then T steps of
//           LGN_convol_magno (:1342-1585) over a movie in layered textures
//
// The module is loaded through the driver API; kernels are found by their mangled names and
// their parameters packed at the offsets cuFuncGetParamInfo reports, so this file needs none of
// the reference's headers.  Every pointer parameter gets a valid zero-filled buffer.
// Bundles: a sequence of records {char name[32]; char type[4]; uint64 count; data}.
#include <cuda.h>
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#define CK(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) {                                                                \
            fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            exit(2);                                                                            \
        }                                                                                       \
    } while (0)
#define CU(x)                                                                         \
    do {                                                                              \
        CUresult r_ = (x);                                                            \
        if (r_ != CUDA_SUCCESS) {                                                     \
            const char *s_ = nullptr;                                                 \
            cuGetErrorString(r_, &s_);                                                \
            fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, s_ ? s_ : "?"); \
            exit(2);                                                                  \
        }                                                                             \
    } while (0)

// ---- bundles ----
struct Arr {
    std::string type;
    std::vector<char> data;
    size_t count = 0;
};
typedef std::map<std::string, Arr> Bundle;

static Bundle read_bundle(const char *fn) {
    Bundle b;
    std::ifstream f(fn, std::ios::binary);
    if (!f) {
        fprintf(stderr, "cannot read %s\n", fn);
        exit(2);
    }
    while (true) {
        char name[33] = {0}, type[5] = {0};
        uint64_t n = 0;
        if (!f.read(name, 32)) break;
        f.read(type, 4);
        f.read(reinterpret_cast<char *>(&n), 8);
        const size_t es = type[1] - '0';
        Arr a;
        a.type = std::string(type, 2);
        a.count = n;
        a.data.resize(n * es);
        f.read(a.data.data(), (std::streamsize)a.data.size());
        b[name] = a;
    }
    return b;
}

struct Writer {
    std::ofstream f;
    explicit Writer(const char *fn) : f(fn, std::ios::binary) {}
    void put(const char *name, const char *type, const void *p, size_t n) {
        char nm[32] = {0}, tp[4] = {0};
        strncpy(nm, name, 31);
        memcpy(tp, type, 2);
        uint64_t c = n;
        f.write(nm, 32);
        f.write(tp, 4);
        f.write(reinterpret_cast<const char *>(&c), 8);
        f.write(reinterpret_cast<const char *>(p), (std::streamsize)(n * (type[1] - '0')));
    }
    template <class T>
    void putv(const char *name, const char *type, const std::vector<T> &v) { put(name, type, v.data(), v.size()); }
};

template <class T>
static std::vector<T> get(const Bundle &b, const char *name) {
    auto it = b.find(name);
    if (it == b.end()) {
        fprintf(stderr, "input %s missing\n", name);
        exit(2);
    }
    std::vector<T> v(it->second.data.size() / sizeof(T));
    memcpy(v.data(), it->second.data.data(), v.size() * sizeof(T));
    return v;
}
template <class T>
static T scalar(const Bundle &b, const char *name) { return get<T>(b, name).at(0); }

// ---- device memory ----
static std::vector<void *> g_allocs;
template <class T>
static T *dev(size_t n) {
    void *p = nullptr;
    CK(cudaMalloc(&p, (n ? n : 1) * sizeof(T)));
    CK(cudaMemset(p, 0, (n ? n : 1) * sizeof(T)));
    g_allocs.push_back(p);
    return static_cast<T *>(p);
}
template <class T>
static T *dev_from(const std::vector<T> &h, size_t atLeast = 0) {
    T *p = dev<T>(h.size() > atLeast ? h.size() : atLeast);
    if (!h.empty()) CK(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return p;
}
template <class T>
static std::vector<T> host(const T *p, size_t n) {
    std::vector<T> h(n);
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost));
    return h;
}

// ---- kernels of the module ----
static CUmodule g_mod;

static CUfunction find_kernel(const char *name) {
    // Itanium-mangled C++ kernel: _Z<len><name>...; helpers are extern "C" (plain name)
    char prefix[128];
    snprintf(prefix, sizeof prefix, "_Z%zu%s", strlen(name), name);
    unsigned int n = 0;
    CU(cuModuleGetFunctionCount(&n, g_mod));
    std::vector<CUfunction> fs(n);
    CU(cuModuleEnumerateFunctions(fs.data(), n, g_mod));
    for (auto f : fs) {
        const char *nm = nullptr;
        CU(cuFuncGetName(&nm, f));
        if (!strncmp(nm, prefix, strlen(prefix)) || !strcmp(nm, name)) return f;
    }
    fprintf(stderr, "kernel %s not in the module\n", name);
    exit(2);
}

// Parameter buffer packed at the offsets and sizes the module declares.
struct Launch {
    CUfunction f;
    std::vector<unsigned char> buf;
    size_t idx = 0;
    const char *name;
    explicit Launch(const char *kname) : f(find_kernel(kname)), name(kname) {}
    Launch &raw(const void *p, size_t n) {
        size_t off = 0, sz = 0;
        if (cuFuncGetParamInfo(f, idx, &off, &sz) != CUDA_SUCCESS) {
            fprintf(stderr, "%s: more arguments than parameters (%zu)\n", name, idx);
            exit(2);
        }
        if (sz != n) {
            fprintf(stderr, "%s: parameter %zu has %zu bytes, given %zu\n", name, idx, sz, n);
            exit(2);
        }
        if (buf.size() < off + sz) buf.resize(off + sz, 0);
        memcpy(&buf[off], p, n);
        idx++;
        return *this;
    }
    template <class T>
    Launch &a(const T &v) {
        raw(&v, sizeof(T));
        return *this;
    }
    // a by-value struct of the reference passed zeroed (unused with learning = 0)
    Launch &zero() {
        size_t off = 0, sz = 0;
        CU(cuFuncGetParamInfo(f, idx, &off, &sz));
        std::vector<unsigned char> z(sz, 0);
        raw(z.data(), sz);
        return *this;
    }
    void go(unsigned gx, unsigned gy, unsigned bx, unsigned by, unsigned shmem = 0) {
        size_t off = 0, sz = 0;
        if (cuFuncGetParamInfo(f, idx, &off, &sz) == CUDA_SUCCESS) {
            fprintf(stderr, "%s: only %zu arguments given\n", name, idx);
            exit(2);
        }
        size_t n = buf.size();
        void *extra[] = {CU_LAUNCH_PARAM_BUFFER_POINTER, buf.data(), CU_LAUNCH_PARAM_BUFFER_SIZE, &n,
                         CU_LAUNCH_PARAM_END};
        if (shmem > 48 * 1024) CU(cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)shmem));
        CU(cuLaunchKernel(f, gx, gy, 1, bx, by, 1, shmem, 0, nullptr, extra));
        CK(cudaDeviceSynchronize());
    }
};

// ConductanceShape bytes from the reference's constructor (helper kernel of the module).
static std::vector<unsigned char> make_cond(const std::vector<float> &rise, const std::vector<float> &decay) {
    float *r = dev_from(rise, 2), *d = dev_from(decay, 2);
    unsigned char *out = dev<unsigned char>(256);
    Launch L("refh_make_cond");
    L.a(r).a(d).a((unsigned)rise.size()).a(out);
    L.go(1, 1, 1, 1);
    auto h = host(out, 256);
    unsigned n = 0;
    memcpy(&n, h.data(), 4);
    return std::vector<unsigned char>(h.begin() + 4, h.begin() + 4 + n);
}

// The first nu uniforms of each generator (copies; the states are not changed).
__global__ void uniforms_kernel(const curandStateMRG32k3a *st, int n, int nu, float *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    curandStateMRG32k3a s = st[i];
    for (int k = 0; k < nu; k++) out[(size_t)i * nu + k] = curand_uniform(&s);
}

// ---- LGN spike surface (src/patch.cu:2659-2675: layered float surface, x in bytes) ----
struct Surface {
    cudaArray_t arr = nullptr;
    cudaSurfaceObject_t obj = 0;
    int w = 0, h = 0, layers = 0;
    Surface(int w_, int h_, int layers_) : w(w_), h(h_), layers(layers_) {
        cudaChannelFormatDesc desc = cudaCreateChannelDesc<float>();
        CK(cudaMalloc3DArray(&arr, &desc, make_cudaExtent(w, h, layers), cudaArrayLayered | cudaArraySurfaceLoadStore));
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        CK(cudaCreateSurfaceObject(&obj, &rd));
        std::vector<float> z((size_t)w * h * layers, 0.f);
        copy_in(z);
    }
    void copy_in(const std::vector<float> &v) {
        cudaMemcpy3DParms p = {};
        p.srcPtr = make_cudaPitchedPtr((void *)v.data(), w * sizeof(float), w, h);
        p.dstArray = arr;
        p.extent = make_cudaExtent(w, h, layers);
        p.kind = cudaMemcpyHostToDevice;
        CK(cudaMemcpy3D(&p));
    }
    std::vector<float> copy_out() {
        std::vector<float> v((size_t)w * h * layers);
        cudaMemcpy3DParms p = {};
        p.srcArray = arr;
        p.dstPtr = make_cudaPitchedPtr(v.data(), w * sizeof(float), w, h);
        p.extent = make_cudaExtent(w, h, layers);
        p.kind = cudaMemcpyDeviceToHost;
        CK(cudaDeviceSynchronize());
        CK(cudaMemcpy3D(&p));
        return v;
    }
};

typedef unsigned char u8;
static const size_t kState = sizeof(curandStateMRG32k3a);

// ---- lgn: logRand_init + K steps of LGN_nonlinear ----
static void mode_lgn(const Bundle &in, Writer &out) {
    const unsigned n = scalar<unsigned>(in, "n"), K = scalar<unsigned>(in, "K"), NU = scalar<unsigned>(in, "NU");
    const unsigned nsx = scalar<unsigned>(in, "nsx"), nsy = scalar<unsigned>(in, "nsy");
    const uint64_t seed = scalar<uint64_t>(in, "seed");
    auto sx = get<int>(in, "sx"), sy = get<int>(in, "sy");
    auto convol = get<float>(in, "convol");
    Surface surf(nsx, nsy, 1);
    float *lnl = dev<float>(n), *ltr = dev<float>(n);
    int *dsx = dev_from(sx), *dsy = dev_from(sy);
    curandStateMRG32k3a *st = dev<curandStateMRG32k3a>(n);
    {
        Launch L("logRand_init");
        L.a(lnl).a(ltr).a(dsx).a(dsy).a(st).a(surf.obj).a((unsigned long)seed).a(n).a((unsigned)0);
        L.go((n + 1023) / 1024, 1, 1024, 1);
    }
    out.putv("lnl0", "f4", host(lnl, n));
    out.putv("ltr0", "f4", host(ltr, n));
    out.putv("state0", "u1", host(reinterpret_cast<u8 *>(st), n * kState));
    float *u = dev<float>((size_t)n * NU);
    uniforms_kernel<<<(n + 255) / 256, 256>>>(st, n, NU, u);
    CK(cudaGetLastError());
    out.putv("u0", "f4", host(u, (size_t)n * NU));
    // Static_nonlinear {mem_block, c50, sharpness, a, b} in device memory (LGN_props.cuh)
    auto c50 = get<float>(in, "c50"), sh = get<float>(in, "sharpness"), la = get<float>(in, "a"), lb = get<float>(in, "b");
    std::vector<float> blk;
    for (auto *v : {&c50, &sh, &la, &lb}) blk.insert(blk.end(), v->begin(), v->end());
    float *dblk = dev_from(blk);
    std::vector<float *> logi = {dblk, dblk, dblk + n, dblk + 2 * n, dblk + 3 * n};
    float **dlogi = dev_from(logi);
    float *maxc = dev_from(get<float>(in, "max_convol"));
    float *cur = dev<float>(n), *fr = dev<float>(n), *sinfo = dev<float>(n);
    float *switchv = dev<float>(n), *lvar = dev<float>(4 * n);
    int *ltype = dev<int>(n);
    const float convolRatio = scalar<float>(in, "convolRatio"), frRatio = scalar<float>(in, "frRatio");
    const float dt = scalar<float>(in, "dt");
    std::vector<float> all_fr, all_si, all_surf;
    for (unsigned k = 0; k < K; k++) {
        CK(cudaMemcpy(cur, convol.data() + (size_t)k * n, n * sizeof(float), cudaMemcpyHostToDevice));
        Launch L("LGN_nonlinear");
        L.a(n).a(dlogi).a(maxc).a(cur).a(convolRatio).a(fr).a(sinfo).a(dsx).a(dsy).a(ltr).a(lnl).a(st);
        L.a(ltype).a(switchv).zero().a(lvar).a(surf.obj).a(frRatio).a((int)0).zero().zero().a((unsigned)0).a(dt);
        L.a((int)0).a(false).a(false).a(true).a(false).a((int)0);
        L.go((n + 1023) / 1024, 1, 1024, 1);
        auto a = host(fr, n), b = host(sinfo, n);
        all_fr.insert(all_fr.end(), a.begin(), a.end());
        all_si.insert(all_si.end(), b.begin(), b.end());
        auto s = surf.copy_out();
        for (unsigned i = 0; i < n; i++) all_surf.push_back(s[(size_t)sy[i] * nsx + sx[i]]);
    }
    out.putv("fr", "f4", all_fr);
    out.putv("sInfo", "f4", all_si);
    out.putv("surf", "f4", all_surf);
    out.putv("lnl", "f4", host(lnl, n));
    out.putv("ltr", "f4", host(ltr, n));
    out.putv("state", "u1", host(reinterpret_cast<u8 *>(st), n * kState));
}

// ---- lgnlearn: logRand_init + K steps of LGN_nonlinear with learning = 3 ----
// One FF_E learning type: the surface holds the spike words (layer 0) and the presynaptic
// trace in three slots (layers 1-3: the start of the step by varSlot = k % 2, the next slot,
// and the value right after the step's spikes).  Per step: the trace at the end of the step
// (lVar, learnData_FF on) and layer 3 at each cell.
struct LearnPre {     // LearnVarShapeFF_E_pre / _I_pre with one type (src/condShape.h:85-92)
    unsigned n;
    float tauLTP[1];
};
static void mode_lgnlearn(const Bundle &in, Writer &out) {
    const unsigned n = scalar<unsigned>(in, "n"), K = scalar<unsigned>(in, "K");
    const unsigned nsx = scalar<unsigned>(in, "nsx"), nsy = scalar<unsigned>(in, "nsy");
    const uint64_t seed = scalar<uint64_t>(in, "seed");
    auto sx = get<int>(in, "sx"), sy = get<int>(in, "sy");
    auto convol = get<float>(in, "convol");
    Surface surf(nsx, nsy, 4);
    float *lnl = dev<float>(n), *ltr = dev<float>(n);
    int *dsx = dev_from(sx), *dsy = dev_from(sy);
    curandStateMRG32k3a *st = dev<curandStateMRG32k3a>(n);
    {
        Launch L("logRand_init");
        L.a(lnl).a(ltr).a(dsx).a(dsy).a(st).a(surf.obj).a((unsigned long)seed).a(n).a((unsigned)0);
        L.go((n + 1023) / 1024, 1, 1024, 1);
    }
    auto c50 = get<float>(in, "c50"), sh = get<float>(in, "sharpness"), la = get<float>(in, "a"), lb = get<float>(in, "b");
    std::vector<float> blk;
    for (auto *v : {&c50, &sh, &la, &lb}) blk.insert(blk.end(), v->begin(), v->end());
    float *dblk = dev_from(blk);
    std::vector<float *> logi = {dblk, dblk, dblk + n, dblk + 2 * n, dblk + 3 * n};
    float **dlogi = dev_from(logi);
    float *maxc = dev_from(get<float>(in, "max_convol"));
    float *cur = dev<float>(n), *fr = dev<float>(n), *sinfo = dev<float>(n);
    float *switchv = dev<float>(n), *lvar = dev<float>(4 * n);
    int *ltype = dev<int>(n);
    const float convolRatio = scalar<float>(in, "convolRatio"), frRatio = scalar<float>(in, "frRatio");
    const float dt = scalar<float>(in, "dt");
    LearnPre lE{1u, {scalar<float>(in, "tauLTP")}}, lI{0u, {0.f}};
    std::vector<float> all_si, all_var, all_spk, all_start;
    for (unsigned k = 0; k < K; k++) {
        CK(cudaMemcpy(cur, convol.data() + (size_t)k * n, n * sizeof(float), cudaMemcpyHostToDevice));
        Launch L("LGN_nonlinear");
        L.a(n).a(dlogi).a(maxc).a(cur).a(convolRatio).a(fr).a(sinfo).a(dsx).a(dsy).a(ltr).a(lnl).a(st);
        L.a(ltype).a(switchv).zero().a(lvar).a(surf.obj).a(frRatio).a((int)(k % 2)).a(lE).a(lI).a((unsigned)1).a(dt);
        L.a((int)3).a(true).a(false).a(true).a(false).a((int)0);
        L.go((n + 1023) / 1024, 1, 1024, 1);
        auto b = host(sinfo, n), v = host(lvar, n);
        all_si.insert(all_si.end(), b.begin(), b.end());
        all_var.insert(all_var.end(), v.begin(), v.end());
        auto s = surf.copy_out();
        const size_t plane = (size_t)nsx * nsy;
        for (unsigned i = 0; i < n; i++) {
            const size_t at = (size_t)sy[i] * nsx + sx[i];
            all_spk.push_back(s[3 * plane + at]);
            all_start.push_back(s[(1 + k % 2) * plane + at]);
        }
    }
    out.putv("sInfo", "f4", all_si);
    out.putv("ffvar", "f4", all_var);
    out.putv("ffspk", "f4", all_spk);
    out.putv("ffstart", "f4", all_start);
}

// ---- V1: the shared network description ----
struct V1 {
    unsigned nblock, bs, nV1, nType, nE, nI, ngFF, ngE, ngI, trainDepth, maxLGN, nnb, nLGNcells, nsx, nsy;
    float dt;
    std::vector<unsigned> typeAcc;
    std::vector<unsigned char> condFF, condE, condI;
    // device arrays
    float *v, *w, *tBack, *dep, *gapS, *gFF, *hFF, *gE, *gI, *hE, *hI, *gap;
    float **ddgE, **ddgI, **ddhE, **ddhI, **ddgap;
    float *spikeTrain, *og, *oh, *totalFF, *totalFF_inf, *last_noise;
    unsigned *ipre, *npre, *dTypeAcc, *nLGN;
    float *sLGN;
    int *lgnx, *lgny;
    float *pFF, *pE, *pI, *vR, *vThres, *gL, *C, *tRef, *tonic, *vT, *deltaT, *tau_w, *a, *b;
    float *synFailFF, *synPerConFF, *synFail, *synPerCon, *noisyDep, *sp0;
    curandStateMRG32k3a *rGenCond, *rNoisy;
    float *learn[10];
    float *conMat, *gapMat;
    unsigned *nNB, *nbId;
};

static V1 make_v1(const Bundle &in) {
    V1 m;
    m.nblock = scalar<unsigned>(in, "nblock");
    m.bs = scalar<unsigned>(in, "blockSize");
    m.nV1 = m.nblock * m.bs;
    m.nType = scalar<unsigned>(in, "nType");
    m.nE = scalar<unsigned>(in, "nE");
    m.nI = m.bs - m.nE;
    m.ngFF = scalar<unsigned>(in, "ngFF");
    m.ngE = scalar<unsigned>(in, "ngE");
    m.ngI = scalar<unsigned>(in, "ngI");
    m.trainDepth = scalar<unsigned>(in, "trainDepth");
    m.dt = scalar<float>(in, "dt");
    m.typeAcc = get<unsigned>(in, "typeAcc");
    const size_t n = m.nV1;
    m.v = dev_from(get<float>(in, "v"));
    m.w = dev_from(get<float>(in, "w"), n);
    m.tBack = dev_from(get<float>(in, "tBack"), n);
    m.dep = dev<float>(n);
    m.gapS = dev<float>(n);
    m.gap = dev<float>(n);
    m.gFF = dev<float>(2 * n);
    m.hFF = dev<float>(2 * n);
    m.gE = dev<float>(2 * n);
    m.hE = dev<float>(2 * n);
    m.gI = dev<float>(2 * n);
    m.hI = dev<float>(2 * n);
    auto put = [&](float *d, const char *name) {
        auto h = get<float>(in, name);
        CK(cudaMemcpy(d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    };
    put(m.gFF, "gFF");
    put(m.hFF, "hFF");
    put(m.gE, "gE");
    put(m.hE, "hE");
    put(m.gI, "gI");
    put(m.hI, "hI");
    // one chunk holding every block (nChunk = 1): the chunk tables point at the flat arrays
    m.ddgE = dev_from(std::vector<float *>{m.gE});
    m.ddgI = dev_from(std::vector<float *>{m.gI});
    m.ddhE = dev_from(std::vector<float *>{m.hE});
    m.ddhI = dev_from(std::vector<float *>{m.hI});
    m.ddgap = dev_from(std::vector<float *>{m.gap});
    m.spikeTrain = dev<float>((size_t)m.trainDepth * n);
    const size_t ng = (size_t)m.nblock * (m.ngE * m.nE + m.ngI * m.nI);
    m.og = dev<float>(ng);
    m.oh = dev<float>(ng);
    m.ipre = dev<unsigned>(n);
    m.npre = dev<unsigned>(2 * m.nblock);
    m.totalFF = dev<float>(n);
    m.totalFF_inf = dev<float>(n);
    m.last_noise = dev<float>(n);
    m.dTypeAcc = dev_from(m.typeAcc);
    m.pFF = dev_from(get<float>(in, "pFF"));
    m.pE = dev_from(get<float>(in, "pE"));
    m.pI = dev_from(get<float>(in, "pI"));
    m.vR = dev_from(get<float>(in, "vR"));
    m.vThres = dev_from(get<float>(in, "vThres"));
    m.gL = dev_from(get<float>(in, "gL"));
    m.C = dev_from(get<float>(in, "C"));
    m.tRef = dev_from(get<float>(in, "tRef"));
    m.vT = dev_from(get<float>(in, "vT"));
    m.deltaT = dev_from(get<float>(in, "deltaT"));
    m.tau_w = dev_from(get<float>(in, "tau_w"));
    m.a = dev_from(get<float>(in, "a"));
    m.b = dev_from(get<float>(in, "b"));
    m.synFailFF = dev_from(get<float>(in, "synFailFF"));
    m.synPerConFF = dev_from(get<float>(in, "synPerConFF"));
    m.synFail = dev_from(get<float>(in, "synFail"));
    m.synPerCon = dev_from(get<float>(in, "synPerCon"));
    m.noisyDep = dev_from(get<float>(in, "noisyDep"));
    m.sp0 = dev_from(get<float>(in, "sp0"));
    m.tonic = dev_from(get<float>(in, "tonicDep"));
    m.nLGN = dev_from(get<unsigned>(in, "nLGNperV1"));
    m.maxLGN = scalar<unsigned>(in, "maxLGN");
    m.sLGN = dev_from(get<float>(in, "sLGN"), (size_t)m.maxLGN * n);
    m.lgnx = dev_from(get<int>(in, "LGN_idx"), (size_t)m.maxLGN * n);
    m.lgny = dev_from(get<int>(in, "LGN_idy"), (size_t)m.maxLGN * n);
    m.rGenCond = dev<curandStateMRG32k3a>(n);
    m.rNoisy = dev<curandStateMRG32k3a>(n);
    // learning variables: unused with learning = 0 except vAvgE, which recal_G_mat_nd_fast
    // updates whenever learning != 3 (src/coredynamics.cu:2871-2883); zeroed, generously sized
    for (int i = 0; i < 10; i++) m.learn[i] = dev<float>((size_t)4 * m.trainDepth * n + 64);
    m.condFF = make_cond(get<float>(in, "riseFF"), get<float>(in, "decayFF"));
    m.condE = make_cond(get<float>(in, "riseE"), get<float>(in, "decayE"));
    m.condI = make_cond(get<float>(in, "riseI"), get<float>(in, "decayI"));
    return m;
}

static void rand_sp_init(V1 &m, const Bundle &in) {
    Launch L("rand_spInit");
    L.a(m.tBack).a(m.spikeTrain).a(m.ipre).a(m.npre).a(m.og).a(m.oh).a(m.v).a(m.w).a(m.nLGN).a(m.sp0);
    L.a(m.dTypeAcc).a(m.vR).a(m.tRef).a(m.tau_w).a(m.a).a(m.b).a(m.rGenCond).a(m.rNoisy);
    L.a((unsigned long)scalar<uint64_t>(in, "seed")).a(m.nV1).a(m.nType).a(scalar<unsigned>(in, "SCsplit"));
    L.a(m.trainDepth).a(m.dt);
    L.raw(m.condE.data(), m.condE.size());
    L.raw(m.condI.data(), m.condI.size());
    L.a(m.ngE).a(m.ngI).a(m.nE).a(m.nI).a(scalar<int>(in, "noDelay")).a((bool)scalar<int>(in, "iModel"));
    L.go(m.nblock, 1, m.bs, 1);
}

static void put_v1_state(const V1 &m, Writer &out, const char *suffix) {
    const size_t n = m.nV1;
    auto nm = [&](const char *b) { return std::string(b) + suffix; };
    out.putv(nm("v").c_str(), "f4", host(m.v, n));
    out.putv(nm("w").c_str(), "f4", host(m.w, n));
    out.putv(nm("tBack").c_str(), "f4", host(m.tBack, n));
    out.putv(nm("gFF").c_str(), "f4", host(m.gFF, m.ngFF * n));
    out.putv(nm("hFF").c_str(), "f4", host(m.hFF, m.ngFF * n));
    out.putv(nm("gE").c_str(), "f4", host(m.gE, m.ngE * n));
    out.putv(nm("hE").c_str(), "f4", host(m.hE, m.ngE * n));
    out.putv(nm("gI").c_str(), "f4", host(m.gI, m.ngI * n));
    out.putv(nm("hI").c_str(), "f4", host(m.hI, m.ngI * n));
}

static void mode_v1init(const Bundle &in, Writer &out) {
    V1 m = make_v1(in);
    rand_sp_init(m, in);
    const size_t n = m.nV1;
    out.putv("tBack", "f4", host(m.tBack, n));
    out.putv("v", "f4", host(m.v, n));
    out.putv("w", "f4", host(m.w, n));
    out.putv("spikeTrain", "f4", host(m.spikeTrain, (size_t)m.trainDepth * n));
    out.putv("npre", "u4", host(m.npre, 2 * m.nblock));
    out.putv("rGenCond", "u1", host(reinterpret_cast<u8 *>(m.rGenCond), n * kState));
    out.putv("rNoisy", "u1", host(reinterpret_cast<u8 *>(m.rNoisy), n * kState));
}

static void mode_v1run(const Bundle &in, Writer &out) {
    V1 m = make_v1(in);
    const size_t n = m.nV1;
    rand_sp_init(m, in);
    out.putv("rGenCond0", "u1", host(reinterpret_cast<u8 *>(m.rGenCond), n * kState));
    out.putv("rNoisy0", "u1", host(reinterpret_cast<u8 *>(m.rNoisy), n * kState));
    const unsigned T = scalar<unsigned>(in, "T"), every = scalar<unsigned>(in, "snapEvery");
    const unsigned nLGNcells = scalar<unsigned>(in, "nLGNcells");
    const unsigned nsx = scalar<unsigned>(in, "nsx"), nsy = scalar<unsigned>(in, "nsy");
    auto cx = get<int>(in, "cell_x"), cy = get<int>(in, "cell_y");
    auto lgnRows = get<float>(in, "lgnSInfo");  // [T][nLGNcells]
    Surface surf(nsx, nsy, 1);
    m.nnb = scalar<unsigned>(in, "nnb");
    m.conMat = dev_from(get<float>(in, "conMat"));
    m.gapMat = dev<float>(16);
    m.nNB = dev_from(get<unsigned>(in, "nNearNB"));
    m.nbId = dev_from(get<unsigned>(in, "nbId"));
    const int iModel = scalar<int>(in, "iModel");
    const unsigned nTypeE = scalar<unsigned>(in, "nTypeE");
    std::vector<float> raster, dep;
    std::vector<float> grid((size_t)nsx * nsy, 0.f);
    for (unsigned it = 0; it < T; it++) {
        // the LGN stage of step it writes its spike words to layer 0 (src/discrete_input_convol.cu:1810)
        for (unsigned c = 0; c < nLGNcells; c++) grid[(size_t)cy[c] * nsx + cx[c]] = lgnRows[(size_t)it * nLGNcells + c];
        surf.copy_in(grid);
        const unsigned slot = it % m.trainDepth;
        {
            Launch L("compute_V_collect_spike_learnFF_fast");
            L.a(m.v).a(m.dep).a(m.w).a(m.gapS).a(m.gFF).a(m.hFF).a(m.ddgE).a(m.ddgI).a(m.ddhE).a(m.ddhI).a(m.ddgap);
            L.a(m.nLGN).a(m.sLGN).a(m.lgnx).a(m.lgny).a(m.tBack).a(m.spikeTrain);
            for (int i = 0; i < 11; i++) L.a(m.learn[i % 10]);  // vLTD_FF_E .. vSTDP_QI
            L.a(m.pFF).a(m.vR).a(m.vThres).a(m.gL).a(m.C).a(m.tRef).a(m.tonic).a(m.vT).a(m.deltaT).a(m.tau_w);
            L.a(m.a).a(m.b).a(m.dTypeAcc).a(m.rGenCond).a(m.synFailFF).a(m.synPerConFF).a(m.rNoisy).a(m.noisyDep);
            L.a(m.last_noise).a(m.ipre).a(m.npre).a(m.og).a(m.oh).a(m.totalFF).a(m.totalFF_inf);
            L.a(0.0f).a(slot).a(m.trainDepth).a(m.maxLGN).a(m.ngFF).a(m.ngE).a(m.ngI);
            L.raw(m.condFF.data(), m.condFF.size());
            L.raw(m.condE.data(), m.condE.size());
            L.raw(m.condI.data(), m.condI.size());
            L.a(m.dt).a(m.nblock).a(m.nblock).a((unsigned)1).a((unsigned)1).a(m.nE).a(m.nI).a(m.nV1);
            L.a((int)0).a((int)(it % 2)).a(m.nType).a(surf.obj);
            L.zero().zero().zero().zero().zero().zero();
            L.a(0.0f).a(iModel).a((int)1).a((int)0).a(false).a(false).a(false).a(scalar<int>(in, "noiseOnTonic") != 0);
            L.go(m.nblock, 1, m.bs, 1);
        }
        {
            const unsigned shmem = m.nnb * 2 * 4 + std::max(m.nE, m.nI) * 4 +
                                   std::max(m.nE * m.ngE, m.nI * m.ngI) * 2 * 4;
            Launch L("recal_G_mat_nd_fast");
            L.a(m.spikeTrain + (size_t)m.nV1 * slot).a(m.ipre).a(m.npre).a(m.og).a(m.oh).a(m.conMat).a(m.gapMat);
            L.a(m.nNB).a(m.nbId).a(m.gE).a(m.gI).a(m.hE).a(m.hI).a(m.gap);
            for (int i = 0; i < 6; i++) L.a(m.learn[i]);  // vAvgE .. vSTDP_QI
            L.a(m.pE).a(m.pI).a(m.dTypeAcc).a(m.rGenCond).a(m.synFail).a(m.synPerCon).a(m.vThres);
            L.a(m.dt);
            L.raw(m.condE.data(), m.condE.size());
            L.raw(m.condI.data(), m.condI.size());
            L.a(m.ngE).a(m.ngI).a(m.nnb).a(m.nE).a(m.nI).a(m.nV1).a((int)0).a((unsigned)0).a(m.nType);
            L.a(nTypeE).a(m.nType - nTypeE).a(m.nblock).zero().zero().a((unsigned)0).a(it).a(false);
            L.go(m.nblock, 1, m.bs, 1, shmem);
        }
        auto row = host(m.spikeTrain + (size_t)m.nV1 * slot, n);
        raster.insert(raster.end(), row.begin(), row.end());
        auto dp = host(m.dep, n);
        dep.insert(dep.end(), dp.begin(), dp.end());
        if ((it + 1) % every == 0) put_v1_state(m, out, ("_" + std::to_string(it + 1)).c_str());
    }
    out.putv("raster", "f4", raster);
    out.putv("dep", "f4", dep);
    out.putv("rGenCond", "u1", host(reinterpret_cast<u8 *>(m.rGenCond), n * kState));
}

// ---- v1learn: rand_spInit, then T steps of compute_V_collect_spike_learnFF_fast with
// learning 1-3 + recal_G_mat_nd_fast, the presynaptic traces given per step (surface layer
// 1 + varSlot: the step start, layer 3: right after the LGN spikes -- the only trace layers the
// V1 kernel reads); the learning structs come as bytes in the reference's layout ("lFF_E_pre",
// "lFF_E_post", "lFF_I_pre", "lFF_I_post", "lE") ----
static void mode_v1learn(const Bundle &in, Writer &out) {
    V1 m = make_v1(in);
    const size_t n = m.nV1;
    rand_sp_init(m, in);
    const unsigned T = scalar<unsigned>(in, "T");
    const unsigned nLGNcells = scalar<unsigned>(in, "nLGNcells");
    const unsigned nsx = scalar<unsigned>(in, "nsx"), nsy = scalar<unsigned>(in, "nsy");
    auto cx = get<int>(in, "cell_x"), cy = get<int>(in, "cell_y");
    auto lgnRows = get<float>(in, "lgnSInfo");   // [T][nLGNcells]
    auto preStart = get<float>(in, "preStart");  // [T][nLGNcells]
    auto preSpk = get<float>(in, "preSpk");      // [T][nLGNcells]
    auto ePre = get<u8>(in, "lFF_E_pre"), ePost = get<u8>(in, "lFF_E_post");
    auto iPre = get<u8>(in, "lFF_I_pre"), iPost = get<u8>(in, "lFF_I_post"), lEs = get<u8>(in, "lE");
    const int learning = scalar<int>(in, "learning");
    const float expHomeo = scalar<float>(in, "expHomeo");
    const int applyHomeo = scalar<int>(in, "applyHomeo");
    const bool symmetricHomeo = scalar<int>(in, "symmetricHomeo") != 0, rebound = scalar<int>(in, "rebound") != 0;
    Surface surf(nsx, nsy, 4);
    m.nnb = scalar<unsigned>(in, "nnb");
    m.conMat = dev_from(get<float>(in, "conMat"));
    m.gapMat = dev<float>(16);
    m.nNB = dev_from(get<unsigned>(in, "nNearNB"));
    m.nbId = dev_from(get<unsigned>(in, "nbId"));
    const int iModel = scalar<int>(in, "iModel");
    const unsigned nTypeE = scalar<unsigned>(in, "nTypeE");
    const size_t nEt = (size_t)m.nE * m.nblock, nIt = (size_t)m.nI * m.nblock;
    float *vLTD = dev<float>(nEt), *vTrip = dev<float>(nEt), *vAvgE = dev<float>(2 * nEt), *vAvgI = dev<float>(nIt + 1);
    float *vLTDi = dev<float>(nIt), *vTripi = dev<float>(nIt);
    // the cortical learning variables (read and written at spikes by the V1 kernel, used by
    // nothing else): zeroed, generously sized
    float *cort = dev<float>((size_t)8 * m.trainDepth * n + 64);
    float *none = dev<float>(64);
    auto tot = get<float>(in, "totalFF");        // [2][nV1]
    CK(cudaMemcpy(m.totalFF, tot.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m.totalFF_inf, tot.data() + n, n * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<unsigned char> zQ(28, 0);
    std::vector<float> raster;
    const size_t plane = (size_t)nsx * nsy;
    std::vector<float> layers(4 * plane, 0.f);
    for (unsigned it = 0; it < T; it++) {
        const unsigned varSlot = it % 2;
        for (unsigned c = 0; c < nLGNcells; c++) {
            const size_t at = (size_t)cy[c] * nsx + cx[c], q = (size_t)it * nLGNcells + c;
            layers[at] = lgnRows[q];
            layers[(1 + varSlot) * plane + at] = preStart[q];
            layers[3 * plane + at] = preSpk[q];
        }
        surf.copy_in(layers);
        const unsigned slot = it % m.trainDepth;
        {
            Launch L("compute_V_collect_spike_learnFF_fast");
            L.a(m.v).a(m.dep).a(m.w).a(m.gapS).a(m.gFF).a(m.hFF).a(m.ddgE).a(m.ddgI).a(m.ddhE).a(m.ddhI).a(m.ddgap);
            L.a(m.nLGN).a(m.sLGN).a(m.lgnx).a(m.lgny).a(m.tBack).a(m.spikeTrain);
            L.a(vLTD).a(vTrip).a(vLTDi).a(vTripi).a(vAvgE).a(vAvgI).a(cort).a(cort).a(cort).a(cort).a(cort);
            L.a(m.pFF).a(m.vR).a(m.vThres).a(m.gL).a(m.C).a(m.tRef).a(m.tonic).a(m.vT).a(m.deltaT).a(m.tau_w);
            L.a(m.a).a(m.b).a(m.dTypeAcc).a(m.rGenCond).a(m.synFailFF).a(m.synPerConFF).a(m.rNoisy).a(m.noisyDep);
            L.a(m.last_noise).a(m.ipre).a(m.npre).a(m.og).a(m.oh).a(m.totalFF).a(m.totalFF_inf);
            L.a(0.0f).a(slot).a(m.trainDepth).a(m.maxLGN).a(m.ngFF).a(m.ngE).a(m.ngI);
            L.raw(m.condFF.data(), m.condFF.size());
            L.raw(m.condE.data(), m.condE.size());
            L.raw(m.condI.data(), m.condI.size());
            L.a(m.dt).a(m.nblock).a(m.nblock).a((unsigned)1).a((unsigned)1).a(m.nE).a(m.nI).a(m.nV1);
            L.a(learning).a((int)varSlot).a(m.nType).a(surf.obj);
            L.raw(ePre.data(), ePre.size()).raw(iPre.data(), iPre.size());
            L.raw(ePost.data(), ePost.size()).raw(iPost.data(), iPost.size());
            L.raw(lEs.data(), lEs.size()).raw(zQ.data(), zQ.size());
            L.a(expHomeo).a(iModel).a((int)1).a(applyHomeo).a(symmetricHomeo).a(false).a(rebound);
            L.a(scalar<int>(in, "noiseOnTonic") != 0);
            L.go(m.nblock, 1, m.bs, 1);
        }
        {
            const unsigned shmem = m.nnb * 2 * 4 + std::max(m.nE, m.nI) * 4 +
                                   std::max(m.nE * m.ngE, m.nI * m.ngI) * 2 * 4;
            Launch L("recal_G_mat_nd_fast");
            L.a(m.spikeTrain + (size_t)m.nV1 * slot).a(m.ipre).a(m.npre).a(m.og).a(m.oh).a(m.conMat).a(m.gapMat);
            L.a(m.nNB).a(m.nbId).a(m.gE).a(m.gI).a(m.hE).a(m.hI).a(m.gap);
            L.a(vAvgE).a(cort).a(cort).a(cort).a(cort).a(cort);
            L.a(m.pE).a(m.pI).a(m.dTypeAcc).a(m.rGenCond).a(m.synFail).a(m.synPerCon).a(m.vThres);
            L.a(m.dt);
            L.raw(m.condE.data(), m.condE.size());
            L.raw(m.condI.data(), m.condI.size());
            L.a(m.ngE).a(m.ngI).a(m.nnb).a(m.nE).a(m.nI).a(m.nV1).a(learning).a((unsigned)0).a(m.nType);
            L.a(nTypeE).a(m.nType - nTypeE).a(m.nblock).raw(lEs.data(), lEs.size()).raw(zQ.data(), zQ.size());
            L.a((unsigned)0).a(it).a(false);
            L.go(m.nblock, 1, m.bs, 1, shmem);
        }
        auto row = host(m.spikeTrain + (size_t)m.nV1 * slot, n);
        raster.insert(raster.end(), row.begin(), row.end());
    }
    out.putv("raster", "f4", raster);
    out.putv("sLGN", "f4", host(m.sLGN, (size_t)m.maxLGN * n));
    out.putv("vLTD", "f4", host(vLTD, nEt));
    out.putv("vTrip", "f4", host(vTrip, nEt));
    out.putv("vLTDi", "f4", host(vLTDi, nIt));
    out.putv("vTripi", "f4", host(vTripi, nIt));
    out.putv("vAvgE", "f4", host(vAvgE, 2 * nEt));
    out.putv("vAvgI", "f4", host(vAvgI, nIt));
    out.putv("totalFF", "f4", host(m.totalFF, n));
}

// ---- magno: store_PM (PM = 1) once, then T steps of LGN_convol_magno ----
// Stimulus textures as src/patch.h:95-109 sets them up: one layered float array per cone
// channel with maxFrame layers, border addressing, linear filtering, normalised coordinates;
// every layer starts at the initial luminance (src/patch.cu:5165-5178), and frames enter the
// layer ring one by one as the step loop reaches them (src/patch.cu:5966-6049).
struct Layers {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    int w, h, n;
    Layers(int w_, int h_, int n_, float init) : w(w_), h(h_), n(n_) {
        cudaChannelFormatDesc desc = cudaCreateChannelDesc<float>();
        CK(cudaMalloc3DArray(&arr, &desc, make_cudaExtent(w, h, n), cudaArrayLayered));
        std::vector<float> v((size_t)w * h * n, init);
        put(0, v.data(), n);
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td = {};
        td.addressMode[0] = cudaAddressModeBorder;
        td.addressMode[1] = cudaAddressModeBorder;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 1;
        CK(cudaCreateTextureObject(&tex, &rd, &td, nullptr));
    }
    void put(int layer, const float *src, int count) {
        cudaMemcpy3DParms p = {};
        p.srcPtr = make_cudaPitchedPtr((void *)src, w * sizeof(float), w, h);
        p.dstArray = arr;
        p.dstPos = make_cudaPos(0, 0, layer);
        p.extent = make_cudaExtent(w, h, count);
        p.kind = cudaMemcpyHostToDevice;
        CK(cudaMemcpy3D(&p));
    }
};

static void mode_magno(const Bundle &in, Writer &out) {
    const unsigned nLGN = scalar<unsigned>(in, "nLGN"), m1 = scalar<unsigned>(in, "mSample1D");
    const unsigned nSample = m1 * m1;
    const unsigned nKS = scalar<unsigned>(in, "mKernelSample");
    const unsigned W = scalar<unsigned>(in, "width"), H = scalar<unsigned>(in, "height");
    const unsigned nFrame = scalar<unsigned>(in, "nFrame"), maxFrame = scalar<unsigned>(in, "maxFrame");
    const unsigned ntPerFrame = scalar<unsigned>(in, "ntPerFrame"), denorm = scalar<unsigned>(in, "denorm");
    const unsigned magnoComp = scalar<unsigned>(in, "magnoComp"), frameOffset = scalar<unsigned>(in, "frameOffset");
    const unsigned ksi = scalar<unsigned>(in, "kernelSampleInterval"), ksT0 = scalar<unsigned>(in, "iKernelSampleT0");
    const unsigned T = scalar<unsigned>(in, "T"), stride = scalar<unsigned>(in, "stride");
    const float dt = scalar<float>(in, "dt");
    // Spatial_component / Temporal_component: {mem_block, 6 arrays of 2 nLGN} (LGN_props.cuh)
    float *sblk = dev_from(get<float>(in, "spatial"));      // x rx y ry orient k
    float *tblk = dev_from(get<float>(in, "temporal"));     // tauR tauD delay ratio nR nD
    std::vector<float *> sp = {sblk}, tp = {tblk};
    for (int q = 0; q < 6; q++) {
        sp.push_back(sblk + (size_t)q * 2 * nLGN);
        tp.push_back(tblk + (size_t)q * 2 * nLGN);
    }
    float **dsp = dev_from(sp), **dtp = dev_from(tp);
    unsigned *cone = dev_from(get<unsigned>(in, "coneType"));
    float *TW = dev<float>((size_t)nLGN * nKS), *SW = dev<float>((size_t)nLGN * nSample);
    float *SC = dev<float>((size_t)2 * nLGN * nSample), *maxc = dev<float>(nLGN);
    float *center = dev<float>(2 * nLGN), *smp = dev<float>(3 * nSample);
    {
        Launch L("store_PM");
        L.a(dtp).a(TW).a(nKS).a(scalar<float>(in, "kernelSampleDt")).a(scalar<float>(in, "kernelSampleT0"));
        L.a(dsp).a(SW).a(SC).a(center).a(maxc).a(smp).a(smp + nSample).a(smp + 2 * nSample);
        L.a((unsigned)0).a((unsigned)0).a(nLGN).a(nLGN);
        L.a(scalar<float>(in, "L_x0")).a(scalar<float>(in, "L_y0")).a(scalar<float>(in, "R_x0")).a(scalar<float>(in, "R_y0"));
        L.a(scalar<float>(in, "normViewDistance")).a(scalar<float>(in, "nsig")).a((int)1);
        L.a(scalar<int>(in, "flat_retina") != 0).a(false);
        L.go(nLGN, 1, m1, m1);
    }
    out.putv("TW", "f4", host(TW, (size_t)nLGN * nKS));
    out.putv("SW", "f4", host(SW, (size_t)nLGN * nSample));
    out.putv("SC", "f4", host(SC, (size_t)2 * nLGN * nSample));
    out.putv("maxConvol", "f4", host(maxc, nLGN));
    auto frames = get<float>(in, "frames");     // [nFrame][3][H][W]
    auto init = get<float>(in, "initLMS");
    Layers L0(W, H, maxFrame, init[0]), L1(W, H, maxFrame, init[1]), L2(W, H, maxFrame, init[2]);
    float *lum = dev<float>(nLGN), *conv = dev<float>(nLGN), *contrast = dev<float>(nLGN);
    unsigned currentFrame = 0, iFrameHead = 0, oldFrameHead = 0, readPos = 0;
    unsigned mPhaseTail = magnoComp;
    std::vector<float> all;
    const size_t fsz = (size_t)W * H;
    for (unsigned it = 0; it < T; it++) {
        if ((unsigned long long)(it + 1) * denorm > (unsigned long long)currentFrame * ntPerFrame) {
            const float *f = frames.data() + (size_t)readPos * 3 * fsz;
            L0.put(iFrameHead, f, 1);
            L1.put(iFrameHead, f + fsz, 1);
            L2.put(iFrameHead, f + 2 * fsz, 1);
            readPos = (readPos + 1) % nFrame;        // the stimulus file loops at its end
            currentFrame++;
            oldFrameHead = iFrameHead;
            iFrameHead = (iFrameHead + 1) % maxFrame;
        }
        mPhaseTail = (mPhaseTail + denorm) % ntPerFrame;
        const unsigned head = oldFrameHead + frameOffset;
        const unsigned mFrameTail = mPhaseTail <= magnoComp ? head + 2 : head + 1;
        Launch K("LGN_convol_magno");
        K.a(lum).a(SW).a(SC).a(TW).a(conv).a(contrast).a(cone).a(dsp).a(L0.tex).a(L1.tex).a(L2.tex);
        K.a((unsigned)0).a(nLGN).a((unsigned)0).a(scalar<float>(in, "normViewDistance"));
        K.a(mFrameTail).a(maxFrame).a(ntPerFrame).a(mPhaseTail).a(0.0f).a(ksT0).a(ksi).a(nKS).a(dt).a(denorm).a(false);
        K.go(nLGN, 1, m1, m1, (unsigned)(sizeof(float) * nSample));
        if (it % stride == 0) {
            auto c = host(conv, nLGN);
            all.insert(all.end(), c.begin(), c.end());
        }
    }
    out.putv("convol", "f4", all);
}

int main(int argc, char **argv) {
    if (argc != 5) {
        fprintf(stderr, "usage: %s <ref_kernels.cubin> <lgn|lgnlearn|v1init|v1run|v1learn|magno> <in.bundle> <out.bundle>\n", argv[0]);
        return 1;
    }
    CK(cudaFree(0));  // primary context current for the driver API too
    CU(cuModuleLoad(&g_mod, argv[1]));
    Bundle in = read_bundle(argv[3]);
    Writer out(argv[4]);
    const std::string mode = argv[2];
    if (mode == "lgn")
        mode_lgn(in, out);
    else if (mode == "v1init")
        mode_v1init(in, out);
    else if (mode == "v1run")
        mode_v1run(in, out);
    else if (mode == "magno")
        mode_magno(in, out);
    else if (mode == "lgnlearn")
        mode_lgnlearn(in, out);
    else if (mode == "v1learn")
        mode_v1learn(in, out);
    else {
        fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 1;
    }
    out.f.close();
    for (void *p : g_allocs) cudaFree(p);
    CU(cuModuleUnload(g_mod));
    printf("%s done\n", mode.c_str());
    return 0;
}
