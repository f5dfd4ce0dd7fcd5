#pragma once
// staged_kernels.cuh -- mixed-precision back-projection with TMA-staged raw
// windows: device code and launch templates (instantiated per chunk size in
// staged_c32.cu, staged_c64.cu, staged_c128.cu).
//
// Same decomposition and precision plan as the gather kernel
// (focus_mixed.cu, mixed_common.cuh), but each CTA stages, per STAGE-pulse
// stage (16 or 32 pulses), the range window its pixel tile can touch into
// shared memory with one 2-D tiled TMA load (box = W range bins x STAGE
// pulses of the pulse-major raw data) plus a 1-D bulk copy of the stage's
// per-pulse table.  NBUF = 64 / STAGE buffers form a ring: a warp that has
// finished a stage releases its buffer (a shared counter), and the last warp
// to release it issues the copies of the stage NBUF ahead into it.  Warps are
// never held in lock step by a CTA barrier inside a pass; a warp runs at most
// NBUF - 1 stages ahead of the slowest.
//
// The float-float reference (chunk_setup) is computed once per chunk of
// CHUNK = 32, 64 or 128 pulses (reference pulse mid-chunk), before the wait
// for the chunk's first stage; a chunk's stages sum into one FP32 partial
// that is rotated by the reference phasor and added to the Kahan accumulator
// once per chunk.  The fast path evaluates two pulses per packed f32x2
// instruction.
//
// The window of stage c is the range-bin interval every pixel of the tile can
// reach from the stage's pulses: per pixel, the distances to the stage's
// first and last pulse positions (maximum) and to the chord between them
// (minimum), widened by the stage's deviation from that chord and one bin on
// each side; reduced over the tile in a prologue.  When that interval is
// wider than W bins, or reaches outside bins 0..nra-2, the stage runs on the
// generic path, which tests every pulse's bin against the window and reads a
// bin outside it from global memory (counted as a window miss).  Only when
// the interval fits does a warp take the fast path, which reads the staged
// window without a per-pulse test (a column outside it would be clamped to
// the window's edge): its correctness rests on the prologue's bound being
// conservative, which the margins above make it (tests compare the range
// bins of rough-terrain scenes with the oracle's bit for bit).
//
// All mbarrier waits are bounded; a wait that gives up sets the CTA's stop
// flag, every warp leaves the pass, and the CTA marks the workspace status
// block and exits after the copies it issued have landed (or after a second
// bounded wait).
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "f32x2.cuh"
#include "mixed_common.cuh"
#include "tma.cuh"

namespace sarbp {

constexpr int kMaxPassStages = 128;        // stages whose windows are kept at once
constexpr int kMaxBuf = 4;                 // ring buffers (64 pulses / 16-pulse stages)
constexpr int kMaxTileThreads = 256;       // pixels (threads) per tile
constexpr uint32_t kWaitLimit = 1u << 22;  // mbarrier polls before giving up

// Compile-time shape of a staged variant.
template <int CHUNK_, int T0_, int T1_, int W_, int STAGE_, int NBUF_>
struct StagedCfg {
    static constexpr int CHUNK = CHUNK_, T0 = T0_, T1 = T1_, W = W_, STAGE = STAGE_;
    static constexpr int NBUF = NBUF_;             // ring buffers (raw windows in flight)
    static constexpr int R = CHUNK / STAGE;        // stages per chunk
    static constexpr int THREADS = T0 * T1, WARPS = THREADS / 32;
    static constexpr size_t raw_bytes = (size_t)STAGE * W * sizeof(float2);
    static constexpr size_t tab_bytes = (size_t)STAGE * sizeof(float4);
    static constexpr size_t buf_bytes = raw_bytes + tab_bytes;
    // chunk references of a pass, staged in shared memory after the ring
    // when a chunk spans several stages (the chunk set-up then reads them
    // from shared memory instead of waiting on global loads)
    static_assert(sizeof(ChunkRef) == 48, "chunk reference record");
    static constexpr bool CREF_SMEM = R > 1;
    static constexpr int PASS_CHUNKS = kMaxPassStages / R + 1;
    static constexpr size_t cref_bytes = CREF_SMEM ? PASS_CHUNKS * 48 : 0;
    static constexpr size_t smem_bytes = NBUF * buf_bytes + cref_bytes + 128;   // + alignment slack
    static_assert(STAGE == 16 || STAGE == 32, "stage");
    static_assert(NBUF >= 2 && NBUF <= kMaxBuf, "ring");
    // tile-start lane keys and the prologue's stage geometry live at the
    // start of the (then idle) ring buffers
    static_assert(NBUF * buf_bytes >= 8 * kMaxTileThreads &&
                      NBUF * buf_bytes >= 32 * kMaxPassStages,
                  "scratch aliases");
    static_assert(CHUNK % STAGE == 0 && kMaxPassStages % R == 0, "chunk");
    static_assert(buf_bytes % 128 == 0, "TMA destinations stay 128-byte aligned");
    static_assert(THREADS <= kMaxTileThreads && (THREADS & (THREADS - 1)) == 0, "tile");
};

// Ascending bitonic sort of N keys in shared memory, one key per thread of
// the CTA (N = blockDim.x, a power of two); keys must be in place and
// visible (after a barrier) on entry.
template <int N>
__device__ __forceinline__ void cta_bitonic_sort(unsigned long long *a, int t)
{
#pragma unroll 1
    for (int k = 2; k <= N; k <<= 1) {
#pragma unroll 1
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int p = t ^ j;
            if (p > t) {
                const unsigned long long x = a[t], y = a[p];
                if ((x > y) == ((t & k) == 0)) {
                    a[t] = y;
                    a[p] = x;
                }
            }
            __syncthreads();
        }
    }
}

template <int T0, int T1>
__device__ __forceinline__ void staged_tile_pixel(int t, int64_t tile0, int64_t tile1,
                                                  int64_t &i0, int64_t &i1)
{
    static_assert(T0 % 8 == 0 && T1 % 4 == 0, "tile must be a multiple of the 8x4 warp block");
    const int w = t >> 5, lane = t & 31;
    i0 = tile0 * T0 + (w % (T0 / 8)) * 8 + (lane & 7);
    i1 = tile1 * T1 + (w / (T0 / 8)) * 4 + (lane >> 3);
}

// The per-pulse coefficients of a chunk setup, each in both halves of an
// f32x2 pair: the operands of the fast path, and (low half) of the scalar
// paths, so only one copy stays live across a chunk's stages.
struct StageCoef {
    f2_t mx, my, mz, c1, c2, c3, g0, a, r0sq;
};

__device__ __forceinline__ float f2_lo(f2_t v)
{
    float lo, hi;
    f2_unpack(v, lo, hi);
    return lo;
}

__device__ __forceinline__ StageCoef stage_coef(const ChunkSetup &S)
{
    return StageCoef{f2_dup(S.mx), f2_dup(S.my), f2_dup(S.mz), f2_dup(S.c1),  f2_dup(S.c2),
                     f2_dup(S.c3), f2_dup(S.g0), f2_dup(S.a),  f2_dup(S.r0sq)};
}

// FP32 per-pulse range geometry: D = R^2 - R0^2, dR = R - R0, the window
// column of the FP32 range bin, and whether that bin is within the tie band.
__device__ __forceinline__ void pulse_eval(const StageCoef &S, float4 e, float inv_dra,
                                           int colbias, float tie, float &D, float &dR,
                                           int &col, bool &amb)
{
    D = fmaf(f2_lo(S.mx), e.x, fmaf(f2_lo(S.my), e.y, fmaf(f2_lo(S.mz), e.z, e.w)));
    dR = D * fmaf(fmaf(f2_lo(S.c3), D, f2_lo(S.c2)), D, f2_lo(S.c1));
    const float g = fmaf(dR, inv_dra, f2_lo(S.g0));
    const float t = __fadd_rn(g, 12582912.0f);
    col = __float_as_int(t) + colbias;
    amb = fabsf(__fsub_rn(g, __fsub_rn(t, 12582912.0f))) > tie;
}

// e of pulse j of a stage from the pair-interleaved per-pulse table.
__device__ __forceinline__ float4 stage_e(const float4 *stab, int j)
{
    const float *f = reinterpret_cast<const float *>(stab) + (j >> 1) * 8 + (j & 1);
    return make_float4(f[0], f[2], f[4], f[6]);
}

// R^2 * exp(-j*dphi) as (wc, ws): term = (vx + j*vy) * (wc - j*ws).
__device__ __forceinline__ void pulse_phasor(const StageCoef &S, float D, float dR, float beta,
                                             float &wc, float &ws)
{
    const float ph = dR * fmaf(beta, dR, f2_lo(S.a));
    float sn, cn;
    __sincosf(ph, &sn, &cn);
    const float w = f2_lo(S.r0sq) + D;
    wc = w * cn;
    ws = w * sn;
}

// Setup of a lane without work in this chunk: every pulse maps to column 0.
__device__ __forceinline__ void safe_setup(ChunkSetup &S, int b0)
{
    S.mx = S.my = S.mz = 0.f;
    S.c1 = S.c2 = S.c3 = 0.f;
    S.g0 = 0.f;
    S.a = 0.f;
    S.r0sq = 0.f;
    S.w0re = 1.f;
    S.w0im = 0.f;
    S.eps = 0.f;
    S.n0 = b0;
    S.exact = false;
}

// Static shared memory of a staged CTA.  It persists across the tiles a
// persistent CTA processes: the stage counter keeps the ring's mbarrier
// phases and release counts in step.
struct StagedShared {
    uint64_t full_bar[kMaxBuf];       // copy completion per buffer
    unsigned rel[kMaxBuf];            // warps done with a buffer (cumulative)
    unsigned last_parity[kMaxBuf];    // phase parity of the last copy into a buffer
    int issued[kMaxBuf];              // a copy was ever issued into the buffer
    int stop;                         // a bounded wait gave up
    int wlo[kMaxPassStages], whi[kMaxPassStages];   // range windows of a pass
    long long lo, hi;                 // tile-wide pulse range
    long long item[2];                // persistent kernels: current work item
    float2 zero;                      // read by masked-off pulses of the fast path
};

struct StagedCta {
    unsigned char *smem;       // NBUF buffers, 128-byte aligned
    StagedShared *sh;
    uint32_t it;               // stage counter (buffer = it % NBUF)
};

struct TileTables {
    const float4 *ptab;
    const PulseFF *pff;
    const ChunkRef *ctab;
    const float *sdev;
};

struct TileOutputs {
    double2 *out;
    int32_t *nvalid;
    uint64_t *checksum;
};

struct TileStats {
    unsigned ambiguous, chunks, misses;
};

// One scene of a batch, as the persistent kernel reads it from device memory.
struct BatchScene {
    CUtensorMap map;          // raw-data window tensor map (64-byte aligned)
    SceneParams P;
    TileTables tables;
    TileOutputs outputs;
    int64_t ntile0, ntiles;
};
static_assert(sizeof(BatchScene) % 16 == 0, "scene records copy as 16-byte words");

// Focus one pixel tile; false if a bounded wait gave up (the CTA must stop).
// Every thread of the CTA calls it with the same tile.
template <class Cfg, bool kChecksum>
__device__ __forceinline__ bool staged_tile(StagedCta &cta, const SceneParams &P,
                                            const CUtensorMap *raw_map, const TileTables &tb,
                                            int64_t tile0, int64_t tile1, const TileOutputs &o,
                                            TileStats &st)
{
    constexpr int W = Cfg::W, STAGE = Cfg::STAGE, NBUF = Cfg::NBUF, R = Cfg::R;
    constexpr int CHUNK = Cfg::CHUNK;
    unsigned char *smem = cta.smem;
    StagedShared &sh = *cta.sh;
    const float4 *ptab = tb.ptab;
    const PulseFF *pff = tb.pff;
    const ChunkRef *ctab = tb.ctab;
    const float *sdev = tb.sdev;

    const int t = threadIdx.x, lane = t & 31;
    int64_t i0, i1;
    staged_tile_pixel<Cfg::T0, Cfg::T1>(t, tile0, tile1, i0, i1);
    bool inside = i0 < P.dim0 && i1 < P.dim1;
    int64_t ii = inside ? i0 + P.dim0 * i1 : 0;
    int64_t lo = 0, hi = -1;
    bool active =
        inside && pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi);

    // ---- lane assignment: the tile's pixels in order of aperture midpoint.
    // Pixels without an aperture (masked, outside the DEM) gather in the last
    // warps, which then skip every stage, and each warp's apertures start and
    // end close together, so more of its stages take the fast path.
    // scratch in the ring buffers, idle between tiles (no copy in flight)
    unsigned long long *lane_key = reinterpret_cast<unsigned long long *>(smem);
    lane_key[t] = ((unsigned long long)(active ? (uint32_t)(lo + hi) : 0xffffffffu) << 16) |
                     (unsigned)t;
    __syncthreads();
    cta_bitonic_sort<Cfg::THREADS>(lane_key, t);
    {
        const int src = (int)(lane_key[t] & 0xffffu);
        __syncthreads();                       // keys read before the buffers are reused
        staged_tile_pixel<Cfg::T0, Cfg::T1>(src, tile0, tile1, i0, i1);
        inside = i0 < P.dim0 && i1 < P.dim1;
        ii = inside ? i0 + P.dim0 * i1 : 0;
        lo = 0;
        hi = -1;
        active = inside && pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi);
    }

    if (t == 0) {
        sh.lo = LLONG_MAX;
        sh.hi = -1;
    }
    __syncthreads();
    if (active) {
        atomicMin(&sh.lo, (long long)lo);
        atomicMax(&sh.hi, (long long)hi);
    }
    __syncthreads();
    const int64_t tlo = sh.lo, thi = sh.hi;

    PixelFF pf{};
    if (active) pf = pixel_ff(P.x[ii], P.y[ii], P.z[ii]);
    float acc_re = 0.f, acc_im = 0.f, cmp_re = 0.f, cmp_im = 0.f;
    int n = 0;
    uint64_t cs = 0;
    unsigned ambiguous = 0, chunks = 0, misses = 0;
    const unsigned nra_m1 = (unsigned)(P.nra - 1);
    const int pitch = (int)P.pitch;
    bool stopped = false;
    ChunkSetup S;
    safe_setup(S, 0);
    StageCoef C = stage_coef(S);
    bool gwork = false;                   // pixel has pulses in the current chunk
    int cur_chunk = -1;
    // pulse indices fit 32 bits (launches check naz < 2^31)
    const int lo32 = (int)lo, hi32 = (int)hi;
    float gre = 0.f, gim = 0.f;           // FP32 partial sum of the current chunk
    if (thi >= 0) {
        const int c_first = (int)(tlo / STAGE), c_last = (int)(thi / STAGE);
        for (int cb = c_first; cb <= c_last && !stopped; cb += kMaxPassStages) {
            const int npass = min(kMaxPassStages, c_last - cb + 1);
            // ---- window prologue: bins every pixel can reach per stage ----
            // stage geometry of the pass into shared memory (one stage per
            // thread), in the ring buffers: no copy is in flight yet
            float4 *geo = reinterpret_cast<float4 *>(smem);
            for (int q = t; q < npass; q += blockDim.x) {
                const int64_t K = (int64_t)(cb + q) * STAGE;
                const int64_t kb = min(K + STAGE - 1, P.naz - 1);
                const float4 ta = __ldg(&pff[K].hi), tb = __ldg(&pff[kb].hi);
                const float sx = tb.x - ta.x, sy = tb.y - ta.y, sz = tb.z - ta.z;
                const float ss = sx * sx + sy * sy + sz * sz;
                geo[2 * q] = make_float4(ta.x, ta.y, ta.z, ss > 0.f ? 1.0f / ss : 0.f);
                geo[2 * q + 1] = make_float4(sx, sy, sz, __ldg(&sdev[cb + q]));
                sh.wlo[q] = INT_MAX;
                sh.whi[q] = INT_MIN;
            }
            // the pass's chunk references (after the ring: no copy writes there)
            const int ch0 = (cb * STAGE) / CHUNK;
            ChunkRef *scref = reinterpret_cast<ChunkRef *>(smem + NBUF * Cfg::buf_bytes);
            if (Cfg::CREF_SMEM) {
                const int nch = ((cb + npass - 1) * STAGE) / CHUNK - ch0 + 1;
                for (int k = t; k < nch; k += blockDim.x) scref[k] = ctab[ch0 + k];
            }
            __syncthreads();
#pragma unroll 2
            for (int q = 0; q < npass; ++q) {
                const int64_t K = (cb + q) * STAGE;
                int blo = INT_MAX, bhi = INT_MIN;
                if (active && lo <= K + STAGE - 1 && hi >= K) {
                    // distances from the pixel to the stage's pulse segment:
                    // endpoints (max), closest point (min), widened by the
                    // chord deviation; approximate square roots (relative
                    // error ~1e-6, ~4 mm at 4 km) inside the 1-bin margin
                    const float4 g0 = geo[2 * q], g1 = geo[2 * q + 1];
                    const float ax = pf.xh - g0.x, ay = pf.yh - g0.y, az = pf.zh - g0.z;
                    const float a2 = ax * ax + ay * ay + az * az;
                    const float d = ax * g1.x + ay * g1.y + az * g1.z;
                    const float u = d * g0.w;
                    const float bx = ax - g1.x, by = ay - g1.y, bz = az - g1.z;
                    const float b2 = bx * bx + by * by + bz * bz;
                    const float rmin2 = (u > 0.f && u < 1.f) ? fmaf(-d, u, a2) : fminf(a2, b2);
                    const float rmax2 = fmaxf(a2, b2);
                    const float rmin = rmin2 > 0.f ? rmin2 * rsqrtf(rmin2) : 0.f;
                    const float rmax = rmax2 > 0.f ? rmax2 * rsqrtf(rmax2) : 0.f;
                    blo = (int)floorf((rmin - g1.w - P.near_hi) * P.inv_dra_f) - 1;
                    bhi = (int)ceilf((rmax + g1.w - P.near_hi) * P.inv_dra_f) + 1;
                }
                blo = __reduce_min_sync(0xffffffffu, blo);
                bhi = __reduce_max_sync(0xffffffffu, bhi);
                if (lane == 0 && blo <= bhi) {
                    atomicMin(&sh.wlo[q], blo);
                    atomicMax(&sh.whi[q], bhi);
                }
            }
            __syncthreads();
            // per stage: TMA start bin (even: 16-byte aligned x coordinate,
            // inside [0, nra]; 0 for a stage no pixel reaches) into wlo, and
            // into whi whether the window covers every reachable bin and lies
            // inside the kept bins 0..nra-2 (no per-pulse tests then)
            for (int q = t; q < npass; q += blockDim.x) {
                const int wl = sh.wlo[q], wh = sh.whi[q];
                const int b0 = wl > wh ? 0 : (int)min((int64_t)max(wl, 0), P.nra) & ~1;
                const bool ok = wl <= wh && wl >= 0 && (int64_t)wh <= P.nra - 2 && wh - b0 < W;
                sh.wlo[q] = b0;
                sh.whi[q] = ok ? 1 : 0;
            }
            __syncthreads();

            // window start of stage q: even (16-byte aligned TMA x coordinate),
            // inside [0, nra]; 0 for a stage no pixel of the tile reaches
            auto window_start = [&](int q) { return sh.wlo[q]; };
            // copies of stage q of this pass into buffer b (any single thread)
            auto issue = [&](int q, int b, uint32_t use) {
                unsigned char *base = smem + (size_t)b * Cfg::buf_bytes;
                const int64_t K = (cb + q) * STAGE;
                mbar_arrive_expect_tx(&sh.full_bar[b], (uint32_t)Cfg::buf_bytes);
                tma_load_2d(base, raw_map, &sh.full_bar[b], window_start(q), (int)K);
                bulk_load(base + Cfg::raw_bytes, ptab + K, (uint32_t)Cfg::tab_bytes,
                          &sh.full_bar[b]);
                sh.last_parity[b] = use & 1;
                sh.issued[b] = 1;
            };
            const uint32_t it0 = cta.it;
            // every buffer is free at a pass start: prime the ring (a
            // diagnostic withhold leaves stage 0 uncopied: its wait runs out);
            // the copies overwrite the scratch the barrier above retired
            if (t == 0) {
                fence_proxy_async_smem();
                for (int q = P.withhold ? 1 : 0; q < NBUF && q < npass; ++q)
                    issue(q, (int)((it0 + q) % NBUF), (it0 + q) / NBUF);
            }

            for (int q = 0; q < npass; ++q) {
                const uint32_t itq = it0 + (uint32_t)q;
                const int b = (int)(itq % NBUF);
                const uint32_t use = itq / NBUF;
                const int c = cb + q;
                const int K = c * STAGE;
                // ---- chunk reference: once per CHUNK pulses, before the wait ----
                const int chunk = c / R;
                if (chunk != cur_chunk) {
                    cur_chunk = chunk;
                    const int C0 = chunk * CHUNK;
                    gwork = active && lo32 <= C0 + CHUNK - 1 && hi32 >= C0;
                    gre = gim = 0.f;
                    if (gwork) {
                        ++chunks;
                        ChunkRef ref;
                        if (Cfg::CREF_SMEM) {
                            ref = scref[chunk - ch0];
                        } else {
                            ref.emax = __ldg(&ctab[chunk].emax);
                            ref.thi = __ldg(&ctab[chunk].thi);
                            ref.tlo = __ldg(&ctab[chunk].tlo);
                        }
                        chunk_setup(P, pf, ref, S);
                    } else {
                        safe_setup(S, 0);
                    }
                    C = stage_coef(S);
                }
                const bool ready = mbar_wait(&sh.full_bar[b], use & 1, P.wait_polls);
                if (!ready) *(volatile int *)&sh.stop = 1;
                if (__any_sync(0xffffffffu, !ready) || *(volatile int *)&sh.stop) {
                    stopped = true;
                    break;
                }
                const int jmin = lo32 > K ? lo32 - K : 0;
                const int jmax = hi32 < K + STAGE - 1 ? hi32 - K : STAGE - 1;
                const bool work = gwork && jmin <= jmax;
                const float2 *sraw =
                    reinterpret_cast<const float2 *>(smem + (size_t)b * Cfg::buf_bytes);
                const float4 *stab = reinterpret_cast<const float4 *>(
                    smem + (size_t)b * Cfg::buf_bytes + Cfg::raw_bytes);
                const int b0 = window_start(q);
                const bool win_ok = sh.whi[q] != 0;
                const bool exact = work && S.exact;
                // fast path: the window holds every bin the warp's pixels can
                // reach; pulses outside a lane's aperture are masked off
                const bool fast = __all_sync(0xffffffffu, !work || (win_ok && !exact));
                const bool whole = __all_sync(0xffffffffu,
                                              !work || (jmin == 0 && jmax == STAGE - 1));
                if (!__any_sync(0xffffffffu, work)) {
                    // no pixel of this warp has pulses in the stage
                } else if (exact) {
                    const double px = P.x[ii], py = P.y[ii], pz = P.z[ii];
                    double sre = 0.0, sim = 0.0;
                    for (int j = jmin; j <= jmax; ++j) {
                        int64_t bin;
                        double tre, tim;
                        if (exact_term(P, px, py, pz, K + j, &bin, &tre, &tim)) {
                            sre += tre;
                            sim += tim;
                            ++n;
                            if (kChecksum) cs += mix64(K + j, bin);
                        }
                    }
                    kahan_add(acc_re, cmp_re, (float)sre);
                    kahan_add(acc_im, cmp_im, (float)sim);
                } else {
                    // lanes without work use their (zero or other-chunk) setup
                    // and read column 0 or a clamped column; nothing is added
                    const int colbias = S.n0 - b0 - 0x4B400000;
                    const float tie = 0.5f - S.eps;
                    // the stage's terms (vx + j*vy)*(wc - j*ws) as four sums:
                    // (sre, sim) += v*wc and (bre, bim) += v*ws, one f32x2 FMA
                    // each per pulse (the same per-lane sequence on every path);
                    // re = sre + bim, im = sim - bre at the end of the stage
                    float sre = gre, sim = gim, bre = 0.f, bim = 0.f;
                    uint32_t amb_mask = 0, miss_mask = 0, valid_mask;
                    // pulses of the stage inside this lane's aperture
                    const uint32_t apmask =
                        work ? (((jmax == 31) ? 0xffffffffu : ((1u << (jmax + 1)) - 1u)) &
                                ~((1u << jmin) - 1u))
                             : 0u;
                    if (fast) {
                        // two pulses per f32x2 instruction, the scalar path's
                        // operation sequence per pulse (bit-identical values);
                        // MASKED reads the zero slot for pulses outside a
                        // lane's aperture
                        valid_mask = apmask;
                        const f2_t mx2 = C.mx, my2 = C.my, mz2 = C.mz;
                        const f2_t c1_2 = C.c1, c2_2 = C.c2, c3_2 = C.c3;
                        const f2_t g0_2 = C.g0, a_2 = C.a, r0sq2 = C.r0sq;
                        const f2_t idra2 = P.inv_dra_f2, beta2 = P.beta_f2, magic2 = P.magic_f2;
                        const ulonglong2 *sp = reinterpret_cast<const ulonglong2 *>(stab);
                        float rmax = 0.f;     // largest |g - rint(g)|: a tie test per stage
                        auto pulse_pairs = [&](auto masked_tag) {
                            constexpr bool MASKED = decltype(masked_tag)::value;
#pragma unroll
                            for (int p = 0; p < STAGE / 2; ++p) {
                                const ulonglong2 exy = sp[2 * p], ezw = sp[2 * p + 1];
                                f2_t D2 = f2_fma(mz2, ezw.x, ezw.y);
                                D2 = f2_fma(my2, exy.y, D2);
                                D2 = f2_fma(mx2, exy.x, D2);
                                f2_t q2 = f2_fma(c3_2, D2, c2_2);
                                q2 = f2_fma(q2, D2, c1_2);
                                const f2_t dR2 = f2_mul(D2, q2);
                                const f2_t g2 = f2_fma(dR2, idra2, g0_2);
                                const f2_t t2 = f2_add(g2, magic2);
                                const f2_t r2 = f2_sub(g2, f2_sub(t2, magic2));
                                float t0, t1, r0, r1;
                                f2_unpack(t2, t0, t1);
                                f2_unpack(r2, r0, r1);
                                rmax = fmax3(rmax, fabsf(r0), fabsf(r1));
                                const int col0 = (int)min((unsigned)(__float_as_int(t0) + colbias),
                                                          (unsigned)(W - 1));
                                const int col1 = (int)min((unsigned)(__float_as_int(t1) + colbias),
                                                          (unsigned)(W - 1));
                                const float2 *a0 = &sraw[(2 * p) * W + col0];
                                const float2 *a1 = &sraw[(2 * p + 1) * W + col1];
                                if (MASKED) {
                                    if (!((apmask >> (2 * p)) & 1u)) a0 = &sh.zero;
                                    if (!((apmask >> (2 * p + 1)) & 1u)) a1 = &sh.zero;
                                }
                                const float2 v0 = *a0, v1 = *a1;
                                const f2_t ph2 = f2_mul(dR2, f2_fma(beta2, dR2, a_2));
                                float ph0, ph1, s0, c0, s1, c1;
                                f2_unpack(ph2, ph0, ph1);
                                __sincosf(ph0, &s0, &c0);
                                __sincosf(ph1, &s1, &c1);
                                const f2_t w2 = f2_add(r0sq2, D2);
                                float wc0, wc1, ws0, ws1;
                                f2_unpack(f2_mul(w2, f2_pack(c0, c1)), wc0, wc1);
                                f2_unpack(f2_mul(w2, f2_pack(s0, s1)), ws0, ws1);
                                {
                                    f2_t A2 = f2_pack(sre, sim), B2 = f2_pack(bre, bim);
                                    const f2_t q0 = *reinterpret_cast<const f2_t *>(&v0);
                                    const f2_t q1 = *reinterpret_cast<const f2_t *>(&v1);
                                    A2 = f2_fma(q0, f2_dup(wc0), A2);
                                    B2 = f2_fma(q0, f2_dup(ws0), B2);
                                    A2 = f2_fma(q1, f2_dup(wc1), A2);
                                    B2 = f2_fma(q1, f2_dup(ws1), B2);
                                    f2_unpack(A2, sre, sim);
                                    f2_unpack(B2, bre, bim);
                                }
                                if (kChecksum) {
                                    if ((apmask >> (2 * p)) & 1u) cs += mix64(K + 2 * p, col0 + b0);
                                    if ((apmask >> (2 * p + 1)) & 1u)
                                        cs += mix64(K + 2 * p + 1, col1 + b0);
                                }
                            }
                        };
                        if (whole)
                            pulse_pairs(std::false_type{});
                        else
                            pulse_pairs(std::true_type{});
                        if (work && rmax > tie) {
                            // a pulse near a .5 tie (rare): find which
                            for (int j = 0; j < STAGE; ++j) {
                                float D, dR;
                                int col;
                                bool amb;
                                pulse_eval(C, stage_e(stab, j), P.inv_dra_f, colbias, tie, D, dR,
                                           col, amb);
                                if (amb && ((apmask >> j) & 1u)) amb_mask |= 1u << j;
                            }
                        }
                    } else {
                        valid_mask = 0;
#pragma unroll
                        for (int j = 0; j < STAGE; ++j) {
                            float D, dR;
                            int col;
                            bool amb;
                            pulse_eval(C, stage_e(stab, j), P.inv_dra_f, colbias, tie, D, dR, col, amb);
                            const bool inap = (apmask >> j) & 1u;
                            const int bin = col + b0;
                            const bool ok = inap && (unsigned)bin < nra_m1;
                            const bool inw = (unsigned)col < (unsigned)W;
                            float2 v = make_float2(0.f, 0.f);
                            if (ok && inw) v = sraw[j * W + col];
                            if (ok) valid_mask |= 1u << j;
                            if (ok && !inw) miss_mask |= 1u << j;
                            if (inap && amb) amb_mask |= 1u << j;
                            float wc, ws;
                            pulse_phasor(C, D, dR, P.beta_f, wc, ws);
                            sre = fmaf(v.x, wc, sre);
                            sim = fmaf(v.y, wc, sim);
                            bre = fmaf(v.x, ws, bre);
                            bim = fmaf(v.y, ws, bim);
                            if (kChecksum && ok) cs += mix64(K + j, bin);
                        }
                    }
                    if (work) {
                        // rare fix-ups: ties re-derived exactly, window misses from L2
                        uint32_t fix = amb_mask | miss_mask;
                        const float2 *rowc = P.raw + K * P.pitch;
                        while (fix) {
                            const int j = __ffs(fix) - 1;
                            fix &= fix - 1;
                            float D, dR;
                            int col;
                            bool amb;
                            pulse_eval(C, stage_e(stab, j), P.inv_dra_f, colbias, tie, D, dR, col, amb);
                            int bin_old = col + b0;
                            bool ok_old;
                            float2 v_old = make_float2(0.f, 0.f);
                            if (fast) {
                                col = (int)min((unsigned)col, (unsigned)(W - 1));
                                bin_old = col + b0;
                                ok_old = true;
                                v_old = sraw[j * W + col];
                            } else {
                                ok_old = (unsigned)bin_old < nra_m1;
                                if (ok_old && (unsigned)col < (unsigned)W) v_old = sraw[j * W + col];
                            }
                            int bin = bin_old;
                            if ((amb_mask >> j) & 1u) {
                                bin = resolve_bin(P, pf, ii, pff, K + j);
                                ++ambiguous;
                            }
                            const bool ok_new = bin >= 0 && (unsigned)bin < nra_m1;
                            float2 v_new = make_float2(0.f, 0.f);
                            if (ok_new) {
                                const int cn = bin - b0;
                                if ((unsigned)cn < (unsigned)W) {
                                    v_new = sraw[j * W + cn];
                                } else {
                                    v_new = __ldg(rowc + (j * pitch + bin));
                                    ++misses;
                                }
                            }
                            float wc, ws;
                            pulse_phasor(C, D, dR, P.beta_f, wc, ws);
                            const float dx = v_new.x - v_old.x, dy = v_new.y - v_old.y;
                            sre = fmaf(dx, wc, sre);
                            sim = fmaf(dy, wc, sim);
                            bre = fmaf(dx, ws, bre);
                            bim = fmaf(dy, ws, bim);
                            valid_mask = ok_new ? (valid_mask | (1u << j)) : (valid_mask & ~(1u << j));
                            if (kChecksum) {
                                if (ok_old) cs -= mix64(K + j, bin_old);
                                if (ok_new) cs += mix64(K + j, bin);
                            }
                        }
                        n += __popc(valid_mask);
                        gre = sre + bim;
                        gim = sim - bre;
                    }
                }
                // end of the chunk: rotate its partial by the reference phasor
                if (gwork && !S.exact && (c % R == R - 1 || c == c_last)) {
                    const float rre = fmaf(gre, S.w0re, -(gim * S.w0im));
                    const float rim = fmaf(gre, S.w0im, gim * S.w0re);
                    kahan_add(acc_re, cmp_re, rre);
                    kahan_add(acc_im, cmp_im, rim);
                    gre = gim = 0.f;
                }
                // release buffer b; the last warp to release it refills it
                __syncwarp();
                if (lane == 0) {
                    __threadfence_block();
                    const unsigned old = atomicAdd(&sh.rel[b], 1u);
                    if (old % Cfg::WARPS == Cfg::WARPS - 1 && q + NBUF < npass) {
                        __threadfence_block();
                        fence_proxy_async_smem();
                        issue(q + NBUF, b, use + 1);
                    }
                }
            }
            __syncthreads();                  // end of pass: every warp left the ring
            if (*(volatile int *)&sh.stop) stopped = true;
            cta.it = it0 + (uint32_t)npass;
        }
    }

    st.ambiguous += ambiguous;
    st.chunks += chunks;
    st.misses += misses;
    if (stopped) return false;
    if (inside) {
        double2 res = make_double2(0.0, 0.0);
        if (n > 0) {
            const double inv = 1.0 / (double)n;
            res = make_double2(((double)acc_re - (double)cmp_re) * inv,
                               ((double)acc_im - (double)cmp_im) * inv);
        }
        o.out[ii] = res;
        if (o.nvalid) o.nvalid[ii] = n;
        if (kChecksum) o.checksum[ii] = cs;
    }
    return true;
}

template <class Cfg>
__device__ __forceinline__ StagedCta staged_cta_init(unsigned char *smem_dyn, StagedShared &sh)
{
    StagedCta cta;
    // TMA tile loads need 128-byte aligned destinations.  The offset is
    // applied as pointer arithmetic on the __shared__ array (no integer
    // round trip), so the compiler keeps the shared address space and the
    // stage reads compile to shared-memory loads.
    cta.smem = smem_dyn + ((128u - (smem_addr(smem_dyn) & 127u)) & 127u);
    cta.sh = &sh;
    cta.it = 0;
    if (threadIdx.x == 0) {
        for (int b = 0; b < Cfg::NBUF; ++b) {
            mbar_init(&sh.full_bar[b], 1);
            sh.rel[b] = 0;
            sh.last_parity[b] = 0;
            sh.issued[b] = 0;
        }
        sh.stop = 0;
        sh.zero = make_float2(0.f, 0.f);
        mbar_fence_init();
    }
    __syncthreads();
    return cta;
}

// A bounded wait gave up: mark the status block and let the last copy issued
// into each buffer land before the CTA's shared memory goes away (at most one
// copy per buffer is ever in flight).  Called by every thread after the
// tile returned false.
template <class Cfg>
__device__ __forceinline__ void staged_abort(StagedCta &cta, StatusBlock *status,
                                             unsigned long long *counters)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        StagedShared &sh = *cta.sh;
        atomicOr(&status->error, 1u);
        atomicExch(&status->where, 1u);
        for (int b = 0; b < Cfg::NBUF; ++b)
            if (sh.issued[b]) mbar_wait(&sh.full_bar[b], sh.last_parity[b], kWaitLimit);
        if (counters) atomicAdd(counters + SARBP_CTR_TIMEOUTS, 1ull);
    }
}

__device__ __forceinline__ void flush_stats(TileStats &st, unsigned long long *counters)
{
    if (!counters) return;
    for (int o = 16; o > 0; o >>= 1) {
        st.ambiguous += __shfl_xor_sync(0xffffffffu, st.ambiguous, o);
        st.chunks += __shfl_xor_sync(0xffffffffu, st.chunks, o);
        st.misses += __shfl_xor_sync(0xffffffffu, st.misses, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (st.ambiguous)
            atomicAdd(counters + SARBP_CTR_AMBIGUOUS, (unsigned long long)st.ambiguous);
        if (st.chunks) atomicAdd(counters + SARBP_CTR_CHUNKS, (unsigned long long)st.chunks);
        if (st.misses) atomicAdd(counters + SARBP_CTR_WINDOW_MISS, (unsigned long long)st.misses);
    }
}

// At least 512 threads' worth of CTAs per SM (at most 128 registers per
// thread): two 256-thread CTAs fit the shared memory of every variant.
template <class Cfg>
constexpr int staged_min_blocks_single()
{
    return 512 / Cfg::THREADS > 2 ? 512 / Cfg::THREADS : 2;
}

// One scene: one CTA per pixel tile, tile blockIdx.x or, with a tile list,
// list[blockIdx.x] (a segment of the prepared queue).
template <class Cfg, bool kChecksum>
__global__ void __launch_bounds__(Cfg::THREADS, (staged_min_blocks_single<Cfg>()))
focus_mixed_staged_kernel(const SceneParams P, const __grid_constant__ CUtensorMap raw_map,
                          const TileTables tb, int64_t ntile0, const int32_t *__restrict__ list,
                          int64_t ntiles, const TileOutputs o,
                          unsigned long long *__restrict__ counters, StatusBlock *status)
{
    extern __shared__ unsigned char smem_dyn[];
    __shared__ StagedShared sh;
    const int64_t tile = list ? (int64_t)list[blockIdx.x] : (int64_t)blockIdx.x;
    if (tile < 0 || tile >= ntiles) return;   // a list prepared for other pixels
    StagedCta cta = staged_cta_init<Cfg>(smem_dyn, sh);
    TileStats st{0, 0, 0};
    const bool ok = staged_tile<Cfg, kChecksum>(cta, P, &raw_map, tb, tile % ntile0,
                                                tile / ntile0, o, st);
    if (!ok) {
        staged_abort<Cfg>(cta, status, counters);
        return;
    }
    flush_stats(st, counters);
}

// One scene, persistent grid: CTAs pull tiles in decreasing estimated cost
// (the order prepared in the workspace) until the queue is empty, so the
// longest tiles start first and no wave of CTAs ends half empty.
template <class Cfg, bool kChecksum>
__global__ void __launch_bounds__(Cfg::THREADS, (staged_min_blocks_single<Cfg>()))
focus_mixed_staged_queue_kernel(const SceneParams P, const __grid_constant__ CUtensorMap raw_map,
                                const TileTables tb, int64_t ntile0,
                                const int32_t *__restrict__ order, int64_t nitems,
                                int64_t ntiles, unsigned long long *cursor, const TileOutputs o,
                                unsigned long long *__restrict__ counters, StatusBlock *status)
{
    extern __shared__ unsigned char smem_dyn[];
    __shared__ StagedShared sh;
    StagedCta cta = staged_cta_init<Cfg>(smem_dyn, sh);
    TileStats st{0, 0, 0};
    for (int round = 0;; ++round) {
        if (threadIdx.x == 0) sh.item[round & 1] = (long long)atomicAdd(cursor, 1ull);
        __syncthreads();
        const long long item = sh.item[round & 1];
        if (item >= nitems) break;
        const int64_t tile = order[item];
        if (tile < 0 || tile >= ntiles) continue;   // a queue prepared for other pixels
        const bool ok = staged_tile<Cfg, kChecksum>(cta, P, &raw_map, tb, tile % ntile0,
                                                    tile / ntile0, o, st);
        if (!ok) {
            staged_abort<Cfg>(cta, status, counters);
            return;
        }
    }
    flush_stats(st, counters);
}

// CTAs per SM the shared memory of a variant allows (2 or 3): the register
// budget the batch kernel is compiled for.
template <class Cfg>
constexpr int staged_min_blocks()
{
    return (Cfg::smem_bytes + sizeof(StagedShared) + 1024) * 3 <= 228 * 1024 ? 3 : 2;
}

// Many scenes in one persistent launch: CTAs pull (scene, tile) work items
// from a device queue (a list ordered by decreasing estimated cost and an
// atomic cursor) until it is empty.
template <class Cfg, bool kChecksum>
__global__ void __launch_bounds__(Cfg::THREADS, (staged_min_blocks<Cfg>()))
focus_batch_staged_kernel(const BatchScene *__restrict__ scenes, const int2 *__restrict__ items,
                          int64_t n_items, unsigned long long *cursor,
                          unsigned long long *__restrict__ counters, StatusBlock *status)
{
    extern __shared__ unsigned char smem_dyn[];
    __shared__ StagedShared sh;
    // the current item's scene record (parameters, tables, outputs): read
    // from shared memory by the tile code instead of from global memory
    __shared__ __align__(16) unsigned char srec[sizeof(BatchScene)];
    StagedCta cta = staged_cta_init<Cfg>(smem_dyn, sh);
    TileStats st{0, 0, 0};
    for (int round = 0;; ++round) {
        if (threadIdx.x == 0) sh.item[round & 1] = (long long)atomicAdd(cursor, 1ull);
        __syncthreads();
        const long long item = sh.item[round & 1];
        if (item >= n_items) break;
        const int2 w = items[item];
        const BatchScene &G = scenes[w.x];
        {
            // every thread is past the previous tile (the barrier above)
            const uint4 *src = reinterpret_cast<const uint4 *>(&G);
            uint4 *dst = reinterpret_cast<uint4 *>(srec);
            for (int k = threadIdx.x; k < (int)(sizeof(BatchScene) / 16); k += blockDim.x)
                dst[k] = src[k];
        }
        __syncthreads();
        const BatchScene &B = *reinterpret_cast<const BatchScene *>(srec);
        const int64_t tile = w.y;
        const bool ok = staged_tile<Cfg, kChecksum>(cta, B.P, &G.map, B.tables,
                                                    tile % B.ntile0, tile / B.ntile0,
                                                    B.outputs, st);
        if (!ok) {
            staged_abort<Cfg>(cta, status, counters);
            return;
        }
    }
    flush_stats(st, counters);
}

// Batch workspace: header, scene records, work items.
struct BatchHeader {
    StatusBlock status;
    unsigned long long cursor;      // next work item
    int32_t nscenes, key;           // scene slots, tiling key of the batch
    int64_t max_items;
    unsigned char pad[256 - 8 - 8 - 8];
};

struct BatchLayout {
    size_t header, scenes, items, total;
};

inline BatchLayout batch_layout(int nscenes, int64_t max_items)
{
    BatchLayout L{};
    L.header = 0;
    L.scenes = (sizeof(BatchHeader) + 255) & ~(size_t)255;
    L.items = (L.scenes + sizeof(BatchScene) * (size_t)nscenes + 255) & ~(size_t)255;
    L.total = (L.items + sizeof(int2) * (size_t)max_items + 255) & ~(size_t)255;
    return L;
}


// 2-D tensor map over the pulse-major raw data (focus_staged.cu).
int make_raw_map(const SceneParams &P, int W, int rows, CUtensorMap *map);

template <class Cfg>
static int ensure_smem_attr()
{
    // per device: the attribute belongs to the function in each context
    static bool done[64] = {};
    int dev = 0;
    int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= 64 || done[dev]) return SARBP_OK;
    const void *ks[6] = {(const void *)focus_mixed_staged_kernel<Cfg, false>,
                         (const void *)focus_mixed_staged_kernel<Cfg, true>,
                         (const void *)focus_mixed_staged_queue_kernel<Cfg, false>,
                         (const void *)focus_mixed_staged_queue_kernel<Cfg, true>,
                         (const void *)focus_batch_staged_kernel<Cfg, false>,
                         (const void *)focus_batch_staged_kernel<Cfg, true>};
    for (const void *k : ks) {
        rc = cuda_status(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)Cfg::smem_bytes),
                         "staged smem attribute");
        if (rc) return rc;
    }
    done[dev] = true;
    return SARBP_OK;
}

inline TileTables tables_of(char *ws, const MixedLayout &L)
{
    TileTables tb;
    tb.ptab = reinterpret_cast<const float4 *>(ws + L.ptab);
    tb.pff = reinterpret_cast<const PulseFF *>(ws + L.pff);
    tb.ctab = reinterpret_cast<const ChunkRef *>(ws + L.ctab);
    tb.sdev = reinterpret_cast<const float *>(ws + L.sdev);
    return tb;
}

template <class Cfg>
int launch_staged_t(const SceneParams &P, const MixedLayout &L, char *ws, bool queued,
                    int64_t first, int64_t count, double *out, int32_t *nvalid,
                    uint64_t *checksum, uint64_t *counters, cudaStream_t stream)
{
    constexpr int T0 = Cfg::T0, T1 = Cfg::T1;
    const int64_t nt0 = (P.dim0 + T0 - 1) / T0, nt1 = (P.dim1 + T1 - 1) / T1;
    const int64_t tiles = nt0 * nt1;
    if (tiles > 0x7fffffffLL) {
        set_error("sarbp_focus_mixed: %lld tiles exceed the launch limit", (long long)tiles);
        return SARBP_ERANGE;
    }
    CUtensorMap map;
    int rc = make_raw_map(P, Cfg::W, Cfg::STAGE, &map);
    if (rc) return rc;
    rc = ensure_smem_attr<Cfg>();
    if (rc) return rc;
    const TileTables tb = tables_of(ws, L);
    const TileOutputs o{reinterpret_cast<double2 *>(out), nvalid, checksum};
    auto *status = reinterpret_cast<StatusBlock *>(ws + L.status);
    auto *ctr = reinterpret_cast<unsigned long long *>(counters);
    if (count < 0) count = tiles - first;   // the rest of the scene
    if (first < 0 || count < 0 || first + count > tiles || (queued && L.ntiles != tiles)) {
        set_error("staged launch: items [%lld, +%lld) outside the %lld-tile scene",
                  (long long)first, (long long)count, (long long)tiles);
        return SARBP_EINVAL;
    }
    if (count == 0) return SARBP_OK;
    const int32_t *order = reinterpret_cast<const int32_t *>(ws + L.vals_out);
    if (!queued || count < tiles) {
        // one CTA per tile: the whole scene in natural order, or a segment of
        // the prepared queue (tiles list[0..count))
        auto *k = checksum ? focus_mixed_staged_kernel<Cfg, true>
                           : focus_mixed_staged_kernel<Cfg, false>;
        k<<<(unsigned)count, Cfg::THREADS, Cfg::smem_bytes, stream>>>(
            P, map, tb, nt0, queued ? order + first : nullptr, tiles, o, ctr, status);
        return cuda_status(cudaGetLastError(), "focus_mixed_staged launch");
    }
    auto *k = checksum ? focus_mixed_staged_queue_kernel<Cfg, true>
                       : focus_mixed_staged_queue_kernel<Cfg, false>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, Cfg::THREADS,
                                                                   Cfg::smem_bytes),
                     "queue occupancy");
    if (rc) return rc;
    const int64_t grid = std::min<int64_t>(count, (int64_t)std::max(1, per_sm) * sms);
    auto *cursor = reinterpret_cast<unsigned long long *>(ws + L.cursor);
    rc = cuda_status(cudaMemsetAsync(cursor, 0, sizeof(*cursor), stream), "queue cursor reset");
    if (rc) return rc;
    k<<<(unsigned)grid, Cfg::THREADS, Cfg::smem_bytes, stream>>>(
        P, map, tb, nt0, order, count, tiles, cursor, o, ctr, status);
    return cuda_status(cudaGetLastError(), "focus_mixed_staged_queue launch");
}

template <class Cfg>
int launch_batch_t(char *bws, const BatchLayout &BL, int64_t n_items, bool diag,
                   uint64_t *counters, cudaStream_t stream)
{
    int rc = ensure_smem_attr<Cfg>();
    if (rc) return rc;
    auto *k = diag ? focus_batch_staged_kernel<Cfg, true> : focus_batch_staged_kernel<Cfg, false>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, Cfg::THREADS,
                                                                   Cfg::smem_bytes),
                     "batch occupancy");
    if (rc) return rc;
    const int64_t grid = std::min<int64_t>(n_items, (int64_t)std::max(1, per_sm) * sms);
    auto *hdr = reinterpret_cast<BatchHeader *>(bws);
    rc = cuda_status(cudaMemsetAsync(&hdr->cursor, 0, sizeof(hdr->cursor), stream),
                     "batch cursor reset");
    if (rc) return rc;
    k<<<(unsigned)grid, Cfg::THREADS, Cfg::smem_bytes, stream>>>(
        reinterpret_cast<const BatchScene *>(bws + BL.scenes),
        reinterpret_cast<const int2 *>(bws + BL.items), n_items, &hdr->cursor,
        reinterpret_cast<unsigned long long *>(counters), &hdr->status);
    return cuda_status(cudaGetLastError(), "focus_batch_staged launch");
}

// Per-chunk-size dispatch over the (tile, window, stage) variants;
// instantiated in staged_c32.cu / staged_c64.cu / staged_c128.cu.
// SARBP_EINVAL (with a message) for a variant that is not built.
#define SARBP_STAGED_TILES(X, C)                                                            \
    X(C, 16, 16, 160, 32, 2) X(C, 16, 16, 160, 16, 4) X(C, 16, 16, 192, 32, 2)              \
    X(C, 16, 16, 208, 32, 2) X(C, 16, 16, 128, 32, 2) X(C, 16, 8, 128, 32, 2)               \
    X(C, 16, 8, 128, 16, 4) X(C, 32, 8, 128, 32, 2) X(C, 64, 4, 128, 32, 2)

template <int C>
int launch_staged_chunk(const SceneParams &P, const sarbp_tuning &T, const MixedLayout &L,
                        char *ws, bool queued, int64_t first, int64_t count, double *out,
                        int32_t *nvalid, uint64_t *checksum, uint64_t *counters,
                        cudaStream_t stream)
{
#define X(C_, A, B, W, S, NB)                                                               \
    if (T.tile0 == A && T.tile1 == B && T.window == W && T.stage == S)                      \
        return launch_staged_t<StagedCfg<C_, A, B, W, S, NB>>(P, L, ws, queued, first, count, \
                                                          out, nvalid, checksum, counters,  \
                                                          stream);
    SARBP_STAGED_TILES(X, C)
#undef X
    set_error("staged path: unsupported tuning chunk=%d tile=%dx%d window=%d stage=%d", T.chunk,
              T.tile0, T.tile1, T.window, T.stage);
    return SARBP_EINVAL;
}

template <int C>
int launch_batch_chunk(char *bws, const BatchLayout &BL, const sarbp_tuning &T, int64_t n_items,
                       bool diag, uint64_t *counters, cudaStream_t stream)
{
#define X(C_, A, B, W, S, NB)                                                               \
    if (T.tile0 == A && T.tile1 == B && T.window == W && T.stage == S)                      \
        return launch_batch_t<StagedCfg<C_, A, B, W, S, NB>>(bws, BL, n_items, diag, counters, \
                                                         stream);
    SARBP_STAGED_TILES(X, C)
#undef X
    set_error("batch path: unsupported tuning chunk=%d tile=%dx%d window=%d stage=%d", T.chunk,
              T.tile0, T.tile1, T.window, T.stage);
    return SARBP_EINVAL;
}

#define SARBP_STAGED_CHUNK_EXTERN(EXT, C)                                                   \
    EXT template int launch_staged_chunk<C>(const SceneParams &, const sarbp_tuning &,      \
                                            const MixedLayout &, char *, bool, int64_t,     \
                                            int64_t, double *, int32_t *, uint64_t *,       \
                                            uint64_t *, cudaStream_t);                      \
    EXT template int launch_batch_chunk<C>(char *, const BatchLayout &, const sarbp_tuning &, \
                                           int64_t, bool, uint64_t *, cudaStream_t);

}  // namespace sarbp
