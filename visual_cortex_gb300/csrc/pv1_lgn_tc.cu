// LGN stage at scale in BF16 on the 5th-generation tensor cores (form c), with an FP32
// CUDA-core kernel of the same formulation beside it.
//
// With one temporal kernel shared by all cells, the linear response of every cell at every
// step is a matrix product: convol[cell][t] = sum_f S[cell][f] * W[t][f], where S is the
// spatial stage (DoG-weighted contrast of frame f in the cell's footprint) and W[t][f] the
// sum of the temporal-kernel samples that read frame f at step t (src/discrete_input_convol.cu:
// 1342-1585 evaluates the same sum sample by sample every step).  A CTA owns 128 cells (the
// MMA's M); time advances in tiles of 128 steps (N); the frames a tile's steps read lie in a
// 64-frame window (K).  Per tile: TMA loads the S window (128 cells x 64 frames, bf16, 128B
// swizzle) and the tile's W (128 steps x 64 frames), one thread issues four
// tcgen05.mma.kind::f16 (K = 16 each) into an FP32 accumulator in tensor memory; two
// warpgroups read the lanes (cells) back with tcgen05.ld, 32 steps at a time, and evaluate the
// logistic rate of LGN_nonlinear (src/discrete_input_convol.cu:1637-1730) for half the steps
// each; the first group then runs the exact-time Poisson generator of get_spike (:1587-1635)
// step by step, carrying each cell's generator state across tiles, while the next tile is
// loaded and multiplied.  Every wait on an mbarrier is bounded; a timeout sets the error word and the
// CTA stops issuing work, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <curand_kernel.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "pv1_internal.cuh"

using pv1::kErrBarrier;

namespace {

constexpr int kTcM = 128;       // cells per CTA
constexpr int kTcN = 128;       // steps per tile
constexpr int kTcK = 64;        // frames per window
constexpr unsigned kTileBytes = kTcM * kTcK * 2;   // 16 KB per operand tile
constexpr long long kWaitSpins = 1LL << 24;

struct TcArgs {
    int nCells, nFext, T, nTiles, frEvery;
    float dt, convolRatio, frRatio;
    const int *f0;                      // [nTiles] first window column of each tile
    const float *absk, *maxConvol, *c50, *sharp, *la, *lb;   // [nCells]
    float *ltr, *lnl;                   // [nCells] carried generator state
    curandStateMRG32k3a *state;         // [nCells]
    float *sInfo;                       // [T][nCells]
    float *fr;                          // [ceil(T/frEvery)][nCells] (may be null)
    const float *S32;                   // [nCells][nFext] (FP32 kernel)
    const float *W32;                   // [nTiles][kTcN][kTcK] (FP32 kernel)
    int *err;
};

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// The rate of LGN_nonlinear (src/discrete_input_convol.cu:1660-1730) for this form: the same
// logistic, evaluated in single precision with the hardware exponential and reciprocal (the
// reference divides in double; this form's accuracy is stated against the FP64 oracle, and
// the BF16 operands dominate that error).  Independent across steps, so a chunk of steps is
// evaluated with full instruction-level parallelism.
__device__ __forceinline__ float lgn_rate(const TcArgs &A, float convol, float absk, float mx, float rmx, float C50,
                                          float Kc, float LA, float LB) {
    float current = (convol * absk) * A.convolRatio;
    if (current < 0) current = 0;
    const float X = __fdividef(1.0f, 1.0f + __expf(Kc * (C50 - current * rmx)));
    return A.frRatio * mx * (LA * X + LB);
}

// Steps t0..t0+n-1 of one cell through get_spike from rT values in shared memory (stride
// kTcM floats), spike words to out (stride nCells floats); four steps per pass with their
// shared-memory loads issued together.
__device__ __forceinline__ float lgn_poisson(float rT, float &ltr, float &lnl, curandStateMRG32k3a &st);
__device__ __forceinline__ void lgn_poisson_run(const float *rT, int stride, int n, float *out, size_t nCells,
                                                float &ltr, float &lnl, curandStateMRG32k3a &st) {
    int c = 0;
    for (; c + 4 <= n; c += 4) {
        const float r0 = rT[(c + 0) * stride], r1 = rT[(c + 1) * stride];
        const float r2 = rT[(c + 2) * stride], r3 = rT[(c + 3) * stride];
        out[0] = lgn_poisson(r0, ltr, lnl, st);
        out[nCells] = lgn_poisson(r1, ltr, lnl, st);
        out[2 * nCells] = lgn_poisson(r2, ltr, lnl, st);
        out[3 * nCells] = lgn_poisson(r3, ltr, lnl, st);
        out += 4 * nCells;
    }
    for (; c < n; c++) {
        out[0] = lgn_poisson(rT[c * stride], ltr, lnl, st);
        out += nCells;
    }
}

// get_spike (src/discrete_input_convol.cu:1589-1619) for one step given rT = dt * rate: the
// only sequential part of the stage (the carried integral and the generator state).
__device__ __forceinline__ float lgn_poisson(float rT, float &ltr, float &lnl, curandStateMRG32k3a &st) {
    float next_rT = lnl - ltr;
    if (next_rT > rT) {
        ltr += rT;
        return 0.f;
    }
    unsigned nsp = 0;
    float old_rT;
    do {
        const float u = curand_uniform(&st);
        lnl = fmaxf(-logf(u), 0.0f);
        old_rT = next_rT;
        next_rT += lnl;
        nsp++;
    } while (next_rT <= rT);
    ltr = rT - old_rT;
    return nsp + old_rT / (rT * nsp);   // nsp + tsp / dt
}

// Epilogue of 32 consecutive steps t0..t0+31 of one cell: rates first (independent), then the
// generator step by step.
__device__ __forceinline__ void lgn_epilogue32(const TcArgs &A, int cell, int t0, const float *conv, float absk,
                                               float mx, float rmx, float C50, float Kc, float LA, float LB,
                                               float &ltr, float &lnl, curandStateMRG32k3a &st) {
    float rT[32];
    const float scale = A.dt * 1e-3f;   // rate in spikes/ms times dt
    int ph = t0 % A.frEvery;            // steps since the last recorded rate
#pragma unroll
    for (int j = 0; j < 32; j++) {
        const float fr = lgn_rate(A, conv[j], absk, mx, rmx, C50, Kc, LA, LB);
        const int t = t0 + j;
        if (A.fr && ph == 0 && t < A.T) A.fr[(size_t)(t / A.frEvery) * A.nCells + cell] = fr;
        ph = ph + 1 == A.frEvery ? 0 : ph + 1;
        rT[j] = fr * scale;
    }
    const int n = min(32, A.T - t0);
    float *out = A.sInfo + (size_t)t0 * A.nCells + cell;
#pragma unroll
    for (int j = 0; j < 32; j++) {
        if (j < n) {
            *out = lgn_poisson(rT[j], ltr, lnl, st);
            out += A.nCells;
        }
    }
}

// ---- PTX wrappers (tcgen05, TMA, mbarrier) ----
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// Bounded wait for the phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    for (long long i = 0; i < kWaitSpins; i++) {
        unsigned ok;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        if (i > 64) __nanosleep(32);
    }
    return false;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t umma_desc_sw128(unsigned addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;               // leading byte offset (unused with K-major swizzle)
    d |= (uint64_t)(1024 >> 4) << 32;     // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;               // descriptor version
    d |= (uint64_t)2 << 61;               // 128-byte swizzle
    return d;
}
// Instruction descriptor of kind::f16: FP32 accumulate, BF16 A and B, both K-major, M x N.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                            ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ void umma_bf16(unsigned tmem, uint64_t a, uint64_t b, int accumulate) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(
            tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float *v) {
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Two warpgroups.  Per tile: the MMA result is read back by both (warp w reads the lanes of
// quadrant w % 4; the first group columns 0-63, the second 64-127), each thread turning its 64
// sums into rates (the independent part) stored to shared memory R [step][cell]; then the first
// group runs the generator of its cell through the 128 steps from R while one thread of the
// second group already loads and multiplies the next tile into the (now free) tensor memory.
constexpr int kTcThreads = 256;
constexpr unsigned kTcSmem = 1024 + 2 * kTileBytes + kTcN * kTcM * 4;   // alignment, tiles, R

__global__ void __launch_bounds__(kTcThreads, 1) lgn_tc_kernel(TcArgs A, const __grid_constant__ CUtensorMap mapS,
                                                               const __grid_constant__ CUtensorMap mapW) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t barFull, barMma;
    __shared__ unsigned tmemSlot;
    __shared__ int abortFlag;
    uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *tileS = base;
    uint8_t *tileW = base + kTileBytes;
    float *R = reinterpret_cast<float *>(base + 2 * kTileBytes);   // [kTcN][kTcM]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quad = warp & 3, half = warp >> 2;
    const int cell0 = blockIdx.x * kTcM;
    const int cl = quad * 32 + lane;   // this thread's lane of the accumulator = its cell
    const int issuer = 4 * 32;         // first thread of the second group issues the copies and MMAs
    if (threadIdx.x == 0) {
        mbar_init(&barFull, 1);
        mbar_init(&barMma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        abortFlag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemSlot)),
                     "r"(kTcN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmemSlot;
    const int cell = cell0 + cl;
    const bool on = cell < A.nCells;
    float absk = 0.f, mx = 1.f, C50 = 0.f, Kc = 0.f, LA = 0.f, LB = 0.f, ltr = 0.f, lnl = 0.f;
    curandStateMRG32k3a st;
    if (on) {
        absk = A.absk[cell]; mx = A.maxConvol[cell]; C50 = A.c50[cell]; Kc = A.sharp[cell];
        LA = A.la[cell]; LB = A.lb[cell];
        if (half == 0) {
            ltr = A.ltr[cell];
            lnl = A.lnl[cell];
            st = A.state[cell];
        }
    }
    const float rmx = 1.0f / mx;
    const float scale = A.dt * 1e-3f;   // rate in spikes/ms times dt
    // tile i: TMA of its S window and W, four MMAs into tensor memory, bounded waits
    auto load_and_multiply = [&](int i) {
        const unsigned parity = (unsigned)(i & 1);
        mbar_expect_tx(&barFull, 2 * kTileBytes);
        tma_load_2d(tileS, &mapS, A.f0[i], cell0, &barFull);
        tma_load_2d(tileW, &mapW, 0, i * kTcN, &barFull);
        if (!mbar_wait(&barFull, parity)) {
            atomicOr(A.err, kErrBarrier);
            abortFlag = 1;
            mbar_wait(&barFull, parity);   // once more, bounded: let the copies in flight land
            return;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint64_t da = umma_desc_sw128(smem_u32(tileS));
        const uint64_t db = umma_desc_sw128(smem_u32(tileW));
#pragma unroll
        for (int k = 0; k < kTcK / 16; k++)   // K = 16 per MMA: +32 bytes inside the swizzle atom
            umma_bf16(tmem, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k), k > 0);
        umma_commit(&barMma);
        if (!mbar_wait(&barMma, parity)) {
            atomicOr(A.err, kErrBarrier);
            abortFlag = 1;
            mbar_wait(&barMma, parity);    // once more, bounded, before the memory is freed
        }
    };
    if (threadIdx.x == issuer && A.nTiles > 0) load_and_multiply(0);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    for (int i = 0; i < A.nTiles; i++) {
        if (abortFlag) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // rates of this thread's cell at its group's 64 steps of the tile
        for (int c0 = half * (kTcN / 2); c0 < (half + 1) * (kTcN / 2); c0 += 32) {
            float v[32];
            tmem_ld32(tmem + ((unsigned)(quad * 32) << 16) + (unsigned)c0, v);
            if (on) {
                int ph = (i * kTcN + c0) % A.frEvery;   // steps since the last recorded rate
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const float fr = lgn_rate(A, v[j], absk, mx, rmx, C50, Kc, LA, LB);
                    const int t = i * kTcN + c0 + j;
                    if (A.fr && ph == 0 && t < A.T) A.fr[(size_t)(t / A.frEvery) * A.nCells + cell] = fr;
                    ph = ph + 1 == A.frEvery ? 0 : ph + 1;
                    R[(c0 + j) * kTcM + cl] = fr * scale;
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();   // R holds the tile; tensor memory and both tiles are free
        if (threadIdx.x == issuer && i + 1 < A.nTiles) load_and_multiply(i + 1);
        if (half == 0 && on)
            lgn_poisson_run(R + cl, kTcM, min(kTcN, A.T - i * kTcN), A.sInfo + (size_t)i * kTcN * A.nCells + cell,
                            (size_t)A.nCells, ltr, lnl, st);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();   // R is read; the next tile is in tensor memory
    }
    (void)lane;
    if (on && half == 0) {
        A.ltr[cell] = ltr;
        A.lnl[cell] = lnl;
        A.state[cell] = st;
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcN));
}

// The same tiles on CUDA cores in FP32: the thread's row of the S window in registers, the
// tile's W rows from shared memory (broadcast), a mul + add chain per step.
__global__ void __launch_bounds__(128) lgn_f32_kernel(TcArgs A) {
    __shared__ float sW[kTcN][kTcK];
    const int cell = blockIdx.x * kTcM + threadIdx.x;
    const bool on = cell < A.nCells;
    float absk = 0.f, mx = 1.f, C50 = 0.f, Kc = 0.f, LA = 0.f, LB = 0.f, ltr = 0.f, lnl = 0.f;
    curandStateMRG32k3a st;
    if (on) {
        absk = A.absk[cell]; mx = A.maxConvol[cell]; C50 = A.c50[cell]; Kc = A.sharp[cell];
        LA = A.la[cell]; LB = A.lb[cell]; ltr = A.ltr[cell]; lnl = A.lnl[cell]; st = A.state[cell];
    }
    const float rmx = 1.0f / mx;
    for (int i = 0; i < A.nTiles; i++) {
        __syncthreads();
        for (int q = threadIdx.x; q < kTcN * kTcK; q += blockDim.x)
            sW[q / kTcK][q % kTcK] = A.W32[(size_t)i * kTcN * kTcK + q];
        float s[kTcK];
        const int f0 = A.f0[i];
#pragma unroll
        for (int k = 0; k < kTcK; k++)
            s[k] = (on && f0 + k < A.nFext) ? A.S32[(size_t)cell * A.nFext + f0 + k] : 0.f;
        __syncthreads();
        if (!on) continue;
        for (int c0 = 0; c0 < kTcN; c0 += 32) {
            float conv[32];
#pragma unroll 4
            for (int c = 0; c < 32; c++) {
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < kTcK; k++) acc += s[k] * sW[c0 + c][k];
                conv[c] = acc;
            }
            lgn_epilogue32(A, cell, i * kTcN + c0, conv, absk, mx, rmx, C50, Kc, LA, LB, ltr, lnl, st);
        }
    }
    if (on) {
        A.ltr[cell] = ltr;
        A.lnl[cell] = lnl;
        A.state[cell] = st;
    }
}

// Spatial stage on a pixel grid: S[cell][PAD + f] = sum over the cell's footprint (side x side
// pixels centred on (cx, cy)) of SW * clamp(L / mean - 1, -1, 1); columns before PAD (frames
// before the movie) are zero, columns past the movie repeat it.  One warp per (cell, frame).
__global__ void __launch_bounds__(256) lgn_pixel_spatial_kernel(const float *frames, int nFrame, int H, int Wd,
                                                                const float *SW, const int *cx, const int *cy,
                                                                int side, int nCells, float mean, int pad,
                                                                int nFext, float *S32, __nv_bfloat16 *S16) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int cell = warp / nFext, col = warp % nFext;
    if (cell >= nCells) return;
    float acc = 0.f;
    if (col >= pad) {
        const int f = (col - pad) % nFrame;
        const float *img = frames + (size_t)f * H * Wd;
        const int half = side / 2;
        for (int q = lane; q < side * side; q += 32) {
            const int x = cx[cell] + q % side - half, y = cy[cell] + q / side - half;
            float c = 0.f;
            if (x >= 0 && x < Wd && y >= 0 && y < H) {
                c = img[(size_t)y * Wd + x] / mean - 1.f;
                c = fminf(fmaxf(c, -1.f), 1.f);
            }
            acc += SW[(size_t)cell * side * side + q] * c;
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    }
    if (lane == 0) {
        S32[(size_t)cell * nFext + col] = acc;
        S16[(size_t)cell * nFext + col] = __float2bfloat16_rn(acc);
    }
}

__global__ void lgn_tc_rng_init_kernel(curandStateMRG32k3a *state, float *lnl, float *ltr, unsigned long long seed,
                                       int n) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    curandStateMRG32k3a s;
    curand_init(seed, id, 0, &s);
    lnl[id] = -logf(curand_uniform(&s));
    ltr[id] = 0.f;
    state[id] = s;
}

__global__ void to_bf16_kernel(const float *in, __nv_bfloat16 *out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

}  // namespace

struct pv1_lgn_tc {
    std::string err;
    pv1_lgn_tc_config cfg{};
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    TcArgs a{};
    int nFext = 0, nTiles = 0;
    __nv_bfloat16 *S16 = nullptr, *W16 = nullptr;
    float *S32 = nullptr, *W32 = nullptr;
    CUtensorMap mapS{}, mapW{};
    int *d_err = nullptr;
};

namespace {

int tfail(pv1_lgn_tc *p, int code, const std::string &m) {
    if (p) p->err = m;
    return code;
}

#define PV1_TCUDA(p, call)                                                                      \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return tfail((p), PV1_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
    } while (0)

template <class T>
int talloc(pv1_lgn_tc *p, T **ptr, size_t n, const void *host = nullptr) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)ptr, n * sizeof(T));
    if (e != cudaSuccess) return tfail(p, PV1_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    p->allocs.push_back(*ptr);
    e = host ? cudaMemcpyAsync(*ptr, host, n * sizeof(T), cudaMemcpyHostToDevice, p->stream)
             : cudaMemsetAsync(*ptr, 0, n * sizeof(T), p->stream);
    if (e != cudaSuccess) return tfail(p, PV1_E_CUDA, cudaGetErrorString(e));
    return PV1_OK;
}

int encode_map(pv1_lgn_tc *p, CUtensorMap *map, void *base, uint64_t inner, uint64_t outer) {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || !f) return tfail(p, PV1_E_CUDA, "cuTensorMapEncodeTiled not available");
        fn = (EncodeTiledFn)f;
    }
    const cuuint64_t dims[2] = {inner, outer};
    const cuuint64_t strides[1] = {inner * 2};   // bytes, multiple of 16 (inner multiple of 8)
    const cuuint32_t box[2] = {(cuuint32_t)kTcK, (cuuint32_t)kTcM};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return tfail(p, PV1_E_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return PV1_OK;
}

}  // namespace

extern "C" {

int pv1_lgn_tc_create(const pv1_lgn_tc_config *cfg, const float *frames, const float *SW, const int32_t *cx,
                      const int32_t *cy, const float *Wtiles, const int32_t *f0, const float *absk,
                      const float *maxConvol, const float *c50, const float *sharp, const float *la,
                      const float *lb, pv1_lgn_tc **out) {
    if (!cfg || !frames || !SW || !cx || !cy || !Wtiles || !f0 || !absk || !maxConvol || !c50 || !sharp || !la ||
        !lb || !out)
        return PV1_E_ARG;
    *out = nullptr;
    pv1_lgn_tc *p = new pv1_lgn_tc();
    *out = p;
    const pv1_lgn_tc_config &c = *cfg;
    p->cfg = c;
    if (c.nCells == 0 || c.T == 0 || c.side == 0 || c.nFext % 8 || c.pad > c.nFext || c.frEvery == 0 ||
        c.nFrame == 0 || c.height == 0 || c.width == 0)
        return tfail(p, PV1_E_ARG, "bad sizes (nFext must be a multiple of 8)");
    const int nTiles = (int)((c.T + kTcN - 1) / kTcN);
    for (int i = 0; i < nTiles; i++)
        if (f0[i] % 8 || f0[i] < 0 || f0[i] >= (int)c.nFext)
            return tfail(p, PV1_E_ARG, "window start not a multiple of 8 inside the frame columns");
    PV1_TCUDA(p, cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    p->nFext = (int)c.nFext;
    p->nTiles = nTiles;
    const size_t nC = c.nCells;
    float *d_frames, *d_SW, *d_absk, *d_mx, *d_c50, *d_sharp, *d_la, *d_lb, *d_ltr, *d_lnl, *d_sInfo,
        *d_fr = nullptr;
    int *d_cx, *d_cy, *d_f0;
    curandStateMRG32k3a *d_state;
    int r = 0;
    r |= talloc(p, &d_frames, (size_t)c.nFrame * c.height * c.width, frames);
    r |= talloc(p, &d_SW, nC * c.side * c.side, SW);
    r |= talloc(p, &d_cx, nC, cx);
    r |= talloc(p, &d_cy, nC, cy);
    r |= talloc(p, &d_f0, (size_t)nTiles, f0);
    r |= talloc(p, &d_absk, nC, absk);
    r |= talloc(p, &d_mx, nC, maxConvol);
    r |= talloc(p, &d_c50, nC, c50);
    r |= talloc(p, &d_sharp, nC, sharp);
    r |= talloc(p, &d_la, nC, la);
    r |= talloc(p, &d_lb, nC, lb);
    r |= talloc(p, &d_ltr, nC);
    r |= talloc(p, &d_lnl, nC);
    r |= talloc(p, &d_state, nC);
    r |= talloc(p, &d_sInfo, (size_t)c.T * nC);
    const size_t nFr = (c.T + c.frEvery - 1) / c.frEvery;
    if (c.recordRates) r |= talloc(p, &d_fr, nFr * nC);
    r |= talloc(p, &p->S32, nC * c.nFext);
    r |= talloc(p, &p->S16, nC * c.nFext);
    r |= talloc(p, &p->W32, (size_t)nTiles * kTcN * kTcK, Wtiles);
    r |= talloc(p, &p->W16, (size_t)nTiles * kTcN * kTcK);
    r |= talloc(p, &p->d_err, 1);
    if (r) return r;
    // spatial stage and the BF16 copies
    const long long warps = (long long)nC * c.nFext;
    lgn_pixel_spatial_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, p->stream>>>(
        d_frames, (int)c.nFrame, (int)c.height, (int)c.width, d_SW, d_cx, d_cy, (int)c.side, (int)nC, c.meanLum,
        (int)c.pad, (int)c.nFext, p->S32, p->S16);
    PV1_TCUDA(p, cudaGetLastError());
    const size_t nW = (size_t)nTiles * kTcN * kTcK;
    to_bf16_kernel<<<(unsigned)((nW + 255) / 256), 256, 0, p->stream>>>(p->W32, p->W16, nW);
    PV1_TCUDA(p, cudaGetLastError());
    r = encode_map(p, &p->mapS, p->S16, c.nFext, nC);
    if (r) return r;
    r = encode_map(p, &p->mapW, p->W16, kTcK, (uint64_t)nTiles * kTcN);
    if (r) return r;
    TcArgs &a = p->a;
    a.nCells = (int)nC; a.nFext = (int)c.nFext; a.T = (int)c.T; a.nTiles = nTiles; a.frEvery = (int)c.frEvery;
    a.dt = c.dt; a.convolRatio = c.convolRatio; a.frRatio = c.frRatio;
    a.f0 = d_f0; a.absk = d_absk; a.maxConvol = d_mx; a.c50 = d_c50; a.sharp = d_sharp; a.la = d_la; a.lb = d_lb;
    a.ltr = d_ltr; a.lnl = d_lnl; a.state = d_state; a.sInfo = d_sInfo; a.fr = d_fr;
    a.S32 = p->S32; a.W32 = p->W32; a.err = p->d_err;
    PV1_TCUDA(p, cudaStreamSynchronize(p->stream));
    return PV1_OK;
}

int pv1_lgn_tc_run(pv1_lgn_tc *p, int tensorCores, uint64_t seed, float *ms) {
    if (!p) return PV1_E_ARG;
    const TcArgs &a = p->a;
    lgn_tc_rng_init_kernel<<<(a.nCells + 255) / 256, 256, 0, p->stream>>>(a.state, a.lnl, a.ltr,
                                                                        (unsigned long long)seed, a.nCells);
    PV1_TCUDA(p, cudaGetLastError());
    PV1_TCUDA(p, cudaMemsetAsync(p->d_err, 0, sizeof(int), p->stream));
    cudaEvent_t e0, e1;
    PV1_TCUDA(p, cudaEventCreate(&e0));
    PV1_TCUDA(p, cudaEventCreate(&e1));
    PV1_TCUDA(p, cudaEventRecord(e0, p->stream));
    const int grid = (a.nCells + kTcM - 1) / kTcM;
    if (tensorCores) {
        // 60 KB per CTA keeps at most 3 CTAs on an SM: 3 x 128 tensor-memory columns <= 512,
        // so no CTA ever waits in tcgen05.alloc
        const int smem = (int)kTcSmem;
        PV1_TCUDA(p, cudaFuncSetAttribute(lgn_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        lgn_tc_kernel<<<grid, kTcThreads, smem, p->stream>>>(a, p->mapS, p->mapW);
    } else {
        lgn_f32_kernel<<<grid, 128, 0, p->stream>>>(a);
    }
    PV1_TCUDA(p, cudaGetLastError());
    PV1_TCUDA(p, cudaEventRecord(e1, p->stream));
    PV1_TCUDA(p, cudaEventSynchronize(e1));
    float t = 0.f;
    PV1_TCUDA(p, cudaEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int h = 0;
    PV1_TCUDA(p, cudaMemcpy(&h, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) return tfail(p, PV1_E_DEVICE, "device error word " + std::to_string(h) + " (an mbarrier wait timed out)");
    return PV1_OK;
}

int pv1_lgn_tc_fetch(pv1_lgn_tc *p, float *S, float *sInfo, float *fr) {
    if (!p) return PV1_E_ARG;
    const TcArgs &a = p->a;
    if (S) PV1_TCUDA(p, cudaMemcpy(S, p->S32, (size_t)a.nCells * a.nFext * sizeof(float), cudaMemcpyDeviceToHost));
    if (sInfo)
        PV1_TCUDA(p, cudaMemcpy(sInfo, a.sInfo, (size_t)a.T * a.nCells * sizeof(float), cudaMemcpyDeviceToHost));
    if (fr) {
        if (!a.fr) return tfail(p, PV1_E_STATE, "rates were not recorded");
        const size_t nFr = (a.T + a.frEvery - 1) / a.frEvery;
        PV1_TCUDA(p, cudaMemcpy(fr, a.fr, nFr * a.nCells * sizeof(float), cudaMemcpyDeviceToHost));
    }
    return PV1_OK;
}

void pv1_lgn_tc_destroy(pv1_lgn_tc *p) {
    if (!p) return;
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (void *q : p->allocs) cudaFree(q);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

const char *pv1_lgn_tc_last_error(const pv1_lgn_tc *p) { return p ? p->err.c_str() : "null"; }

const float *pv1_lgn_tc_device_spikes(const pv1_lgn_tc *p) { return p ? p->a.sInfo : nullptr; }

}  // extern "C"
