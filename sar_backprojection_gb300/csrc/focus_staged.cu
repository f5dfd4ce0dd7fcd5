// focus_staged.cu -- mixed-precision back-projection with TMA-staged raw
// windows.
//
// Same decomposition and precision plan as the gather kernel
// (focus_mixed.cu, mixed_common.cuh), but each CTA stages, per pulse chunk,
// the range window its pixel tile can touch into shared memory with one 2-D
// tiled TMA load (box = W range bins x CHUNK pulses of the pulse-major raw
// data) plus a 1-D bulk copy of the chunk's per-pulse table, double
// buffered: while the CTA focuses chunk c from stage c&1, the copies of chunk
// c+1 land in the other stage.  The per-pulse gathers then hit shared memory
// instead of L1/L2.
//
// The window of chunk c is the range-bin interval every pixel of the tile can
// reach from the chunk's pulses: per pixel, the distances to the chunk's
// first and last pulse positions (maximum) and to the chord between them
// (minimum), widened by the chunk's deviation from that chord and one bin on
// each side; reduced over the tile in a prologue.  A bin outside the staged
// window (a window wider than W) is read from global memory instead and
// counted as a window miss, so correctness never depends on the window.
//
// All mbarrier waits are bounded; a wait that gives up marks the workspace
// status block and the CTA leaves after its last copy lands (or after a
// second bounded wait).
#include <climits>
#include <cstdio>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "mixed_common.cuh"
#include "tma.cuh"

namespace sarbp {

constexpr int kMaxPassChunks = 128;        // chunks whose windows are kept at once
constexpr uint32_t kWaitLimit = 1u << 22;  // mbarrier polls before giving up

template <int CHUNK, int W>
struct StagedSmem {
    static constexpr size_t raw_bytes = (size_t)CHUNK * W * sizeof(float2);
    static constexpr size_t tab_bytes = (size_t)CHUNK * sizeof(float4);
    static constexpr size_t stage_bytes = raw_bytes + tab_bytes;
    static constexpr size_t bytes = 2 * stage_bytes + 1024;   // + alignment slack
};

template <int T0, int T1>
__device__ __forceinline__ void staged_tile_pixel(int t, int64_t tile0, int64_t tile1,
                                                  int64_t &i0, int64_t &i1)
{
    static_assert(T0 % 8 == 0 && T1 % 4 == 0, "tile must be a multiple of the 8x4 warp block");
    const int w = t >> 5, lane = t & 31;
    i0 = tile0 * T0 + (w % (T0 / 8)) * 8 + (lane & 7);
    i1 = tile1 * T1 + (w / (T0 / 8)) * 4 + (lane >> 3);
}

// FP32 per-pulse range geometry: D = R^2 - R0^2, dR = R - R0, the window
// column of the FP32 range bin, and whether that bin is within the tie band.
__device__ __forceinline__ void pulse_eval(const ChunkSetup &S, float4 e, float inv_dra,
                                           int colbias, float tie, float &D, float &dR,
                                           int &col, bool &amb)
{
    D = fmaf(S.mx, e.x, fmaf(S.my, e.y, fmaf(S.mz, e.z, e.w)));
    dR = D * fmaf(fmaf(S.c3, D, S.c2), D, S.c1);
    const float g = fmaf(dR, inv_dra, S.g0);
    const float t = __fadd_rn(g, 12582912.0f);
    col = __float_as_int(t) + colbias;
    amb = fabsf(__fsub_rn(g, __fsub_rn(t, 12582912.0f))) > tie;
}

// R^2 * exp(-j*dphi) as (wc, ws): term = (vx + j*vy) * (wc - j*ws).
__device__ __forceinline__ void pulse_phasor(const ChunkSetup &S, float D, float dR, float beta,
                                             float &wc, float &ws)
{
    const float ph = dR * fmaf(beta, dR, S.a);
    float sn, cn;
    __sincosf(ph, &sn, &cn);
    const float w = S.r0sq + D;
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

template <int CHUNK, int T0, int T1, int W, bool kChecksum>
__global__ void __launch_bounds__(T0 *T1)
focus_mixed_staged_kernel(const SceneParams P, const __grid_constant__ CUtensorMap raw_map,
                          const float4 *__restrict__ ptab, const PulseFF *__restrict__ pff,
                          const ChunkRef *__restrict__ ctab, int64_t ntile0,
                          double2 *__restrict__ out, int32_t *__restrict__ nvalid,
                          uint64_t *__restrict__ checksum,
                          unsigned long long *__restrict__ counters, StatusBlock *status)
{
    using SM = StagedSmem<CHUNK, W>;
    extern __shared__ unsigned char smem_dyn[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full_bar[2];
    __shared__ int s_wlo[kMaxPassChunks], s_whi[kMaxPassChunks];
    __shared__ long long s_lo, s_hi;

    const int t = threadIdx.x;
    int64_t i0, i1;
    staged_tile_pixel<T0, T1>(t, blockIdx.x % ntile0, blockIdx.x / ntile0, i0, i1);
    const bool inside = i0 < P.dim0 && i1 < P.dim1;
    const int64_t ii = inside ? i0 + P.dim0 * i1 : 0;
    int64_t lo = 0, hi = -1;
    const bool active =
        inside && pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi);

    if (t == 0) {
        s_lo = LLONG_MAX;
        s_hi = -1;
        mbar_init(&full_bar[0], 1);
        mbar_init(&full_bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (active) {
        atomicMin(&s_lo, (long long)lo);
        atomicMax(&s_hi, (long long)hi);
    }
    __syncthreads();
    const int64_t tlo = s_lo, thi = s_hi;

    PixelFF pf{};
    if (active) pf = pixel_ff(P.x[ii], P.y[ii], P.z[ii]);
    float acc_re = 0.f, acc_im = 0.f, cmp_re = 0.f, cmp_im = 0.f;
    int n = 0;
    uint64_t cs = 0;
    unsigned ambiguous = 0, chunks = 0, misses = 0;
    const unsigned nra_m1 = (unsigned)(P.nra - 1);
    const int pitch = (int)P.pitch;
    uint32_t it = 0;             // chunk iteration counter across passes (stage = it & 1)
    bool pending[2] = {false, false};     // thread 0: copies in flight per stage
    uint32_t pending_parity[2] = {0, 0};
    bool aborted = false;

    if (thi >= 0) {
        const int64_t c_first = tlo / CHUNK, c_last = thi / CHUNK;
        for (int64_t cb = c_first; cb <= c_last && !aborted; cb += kMaxPassChunks) {
            const int npass = (int)min((int64_t)kMaxPassChunks, c_last - cb + 1);
            // ---- window prologue: bins every pixel can reach per chunk ----
            for (int q = t; q < npass; q += blockDim.x) {
                s_wlo[q] = INT_MAX;
                s_whi[q] = INT_MIN;
            }
            __syncthreads();
            for (int q = 0; q < npass; ++q) {
                const int64_t K = (cb + q) * CHUNK;
                int blo = INT_MAX, bhi = INT_MIN;
                if (active && lo <= K + CHUNK - 1 && hi >= K) {
                    const int64_t ka = K, kb = min(K + CHUNK - 1, P.naz - 1);
                    const float4 ta = __ldg(&pff[ka].hi), tb = __ldg(&pff[kb].hi);
                    const float dev = __ldg(&ctab[cb + q].thi.w);
                    const float ax = pf.xh - ta.x, ay = pf.yh - ta.y, az = pf.zh - ta.z;
                    const float bx = pf.xh - tb.x, by = pf.yh - tb.y, bz = pf.zh - tb.z;
                    const float ra = sqrtf(ax * ax + ay * ay + az * az);
                    const float rb = sqrtf(bx * bx + by * by + bz * bz);
                    const float sx = tb.x - ta.x, sy = tb.y - ta.y, sz = tb.z - ta.z;
                    const float ss = sx * sx + sy * sy + sz * sz;
                    float u = ss > 0.f ? (ax * sx + ay * sy + az * sz) / ss : 0.f;
                    u = fminf(fmaxf(u, 0.f), 1.f);
                    const float cx = ax - u * sx, cy = ay - u * sy, cz = az - u * sz;
                    const float rc = sqrtf(cx * cx + cy * cy + cz * cz);
                    const float rmin = fminf(fminf(ra, rb), rc) - dev;
                    const float rmax = fmaxf(ra, rb) + dev;
                    blo = (int)floorf((rmin - P.near_hi) * P.inv_dra_f) - 1;
                    bhi = (int)ceilf((rmax - P.near_hi) * P.inv_dra_f) + 1;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    blo = min(blo, __shfl_xor_sync(0xffffffffu, blo, o));
                    bhi = max(bhi, __shfl_xor_sync(0xffffffffu, bhi, o));
                }
                if ((t & 31) == 0 && blo <= bhi) {
                    atomicMin(&s_wlo[q], blo);
                    atomicMax(&s_whi[q], bhi);
                }
            }
            __syncthreads();

            // ---- producer: stage chunk q of this pass into stage s ----
            // window start of chunk q: even (16-byte aligned TMA x coordinate),
            // inside [0, nra]; 0 for a chunk no pixel of the tile reaches
            auto window_start = [&](int q) {
                const int wl = s_wlo[q], wh = s_whi[q];
                if (wl > wh) return 0;
                return (int)min((int64_t)max(wl, 0), P.nra) & ~1;
            };
            auto issue = [&](int q, int s, uint32_t use) {
                unsigned char *base = smem + (size_t)s * SM::stage_bytes;
                const int64_t K = (cb + q) * CHUNK;
                mbar_arrive_expect_tx(&full_bar[s], (uint32_t)SM::stage_bytes);
                tma_load_2d(base, &raw_map, &full_bar[s], window_start(q), (int)K);
                bulk_load(base + SM::raw_bytes, ptab + K, (uint32_t)SM::tab_bytes, &full_bar[s]);
                pending[s] = true;
                pending_parity[s] = use & 1;
            };
            if (t == 0) issue(0, it & 1, it >> 1);

            for (int q = 0; q < npass; ++q, ++it) {
                const int s = it & 1;
                if (t == 0 && q + 1 < npass) issue(q + 1, s ^ 1, (it + 1) >> 1);
                const bool ready = mbar_wait(&full_bar[s], (it >> 1) & 1, kWaitLimit);
                if (t == 0 && ready) pending[s] = false;
                const int64_t c = cb + q;
                const int64_t K = c * CHUNK;
                const int jmin = (int)(lo > K ? lo - K : 0);
                const int jmax = (int)(hi < K + CHUNK - 1 ? hi - K : CHUNK - 1);
                const bool work = ready && active && jmin <= jmax;
                const float2 *sraw =
                    reinterpret_cast<const float2 *>(smem + (size_t)s * SM::stage_bytes);
                const float4 *stab = reinterpret_cast<const float4 *>(
                    smem + (size_t)s * SM::stage_bytes + SM::raw_bytes);
                const int b0 = window_start(q);
                // window covers every bin the tile can reach and lies inside
                // the kept bins 0..nra-2: no per-pulse validity/window tests
                const bool win_ok = s_wlo[q] >= 0 && (int64_t)s_whi[q] <= P.nra - 2 &&
                                    s_whi[q] - b0 < W;
                ChunkSetup S;
                safe_setup(S, b0);                 // lanes without work read column 0
                if (work) {
                    ++chunks;
                    ChunkRef ref;
                    ref.emax = __ldg(&ctab[c].emax);
                    ref.thi = __ldg(&ctab[c].thi);
                    ref.tlo = __ldg(&ctab[c].tlo);
                    chunk_setup(P, pf, ref, S);
                }
                const bool exact = work && S.exact;
                const bool fast = __all_sync(0xffffffffu, !work || (jmin == 0 &&
                                                                    jmax == CHUNK - 1 &&
                                                                    win_ok && !exact));
                if (exact) {
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
                    const int colbias = S.n0 - b0 - 0x4B400000;
                    const float tie = 0.5f - S.eps;
                    float sre = 0.f, sim = 0.f;
                    uint32_t amb_mask = 0, miss_mask = 0, valid_mask;
                    if (fast) {
                        valid_mask = 0xffffffffu;
#pragma unroll
                        for (int j = 0; j < CHUNK; ++j) {
                            float D, dR;
                            int col;
                            bool amb;
                            pulse_eval(S, stab[j], P.inv_dra_f, colbias, tie, D, dR, col, amb);
                            if (amb) amb_mask |= 1u << j;
                            col = (int)min((unsigned)col, (unsigned)(W - 1));
                            const float2 v = sraw[j * W + col];
                            float wc, ws;
                            pulse_phasor(S, D, dR, P.beta_f, wc, ws);
                            sre = fmaf(v.x, wc, fmaf(v.y, ws, sre));
                            sim = fmaf(v.y, wc, fmaf(-v.x, ws, sim));
                            if (kChecksum) cs += mix64(K + j, col + b0);
                        }
                    } else {
                        valid_mask = 0;
                        const uint32_t apmask =
                            work ? (((jmax == 31) ? 0xffffffffu : ((1u << (jmax + 1)) - 1u)) &
                                    ~((1u << jmin) - 1u))
                                 : 0u;
#pragma unroll
                        for (int j = 0; j < CHUNK; ++j) {
                            float D, dR;
                            int col;
                            bool amb;
                            pulse_eval(S, stab[j], P.inv_dra_f, colbias, tie, D, dR, col, amb);
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
                            pulse_phasor(S, D, dR, P.beta_f, wc, ws);
                            sre = fmaf(v.x, wc, fmaf(v.y, ws, sre));
                            sim = fmaf(v.y, wc, fmaf(-v.x, ws, sim));
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
                            pulse_eval(S, stab[j], P.inv_dra_f, colbias, tie, D, dR, col, amb);
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
                            pulse_phasor(S, D, dR, P.beta_f, wc, ws);
                            const float dx = v_new.x - v_old.x, dy = v_new.y - v_old.y;
                            sre = fmaf(dx, wc, fmaf(dy, ws, sre));
                            sim = fmaf(dy, wc, fmaf(-dx, ws, sim));
                            valid_mask = ok_new ? (valid_mask | (1u << j)) : (valid_mask & ~(1u << j));
                            if (kChecksum) {
                                if (ok_old) cs -= mix64(K + j, bin_old);
                                if (ok_new) cs += mix64(K + j, bin);
                            }
                        }
                        n += __popc(valid_mask);
                        const float rre = fmaf(sre, S.w0re, -(sim * S.w0im));
                        const float rim = fmaf(sre, S.w0im, sim * S.w0re);
                        kahan_add(acc_re, cmp_re, rre);
                        kahan_add(acc_im, cmp_im, rim);
                    }
                }
                // every thread is done with stage s before it is refilled
                if (__syncthreads_or(!ready)) {
                    aborted = true;
                    break;
                }
            }
        }
    }

    if (aborted) {
        if (t == 0) {
            atomicOr(&status->error, 1u);
            atomicExch(&status->where, 1u);
            // let copies still in flight land before the CTA's shared memory goes
            for (int s = 0; s < 2; ++s)
                if (pending[s]) mbar_wait(&full_bar[s], pending_parity[s], kWaitLimit);
            if (counters) atomicAdd(counters + SARBP_CTR_TIMEOUTS, 1ull);
        }
        return;
    }

    if (inside) {
        double2 res = make_double2(0.0, 0.0);
        if (n > 0) {
            const double inv = 1.0 / (double)n;
            res = make_double2(((double)acc_re - (double)cmp_re) * inv,
                               ((double)acc_im - (double)cmp_im) * inv);
        }
        out[ii] = res;
        if (nvalid) nvalid[ii] = n;
        if (kChecksum) checksum[ii] = cs;
    }
    if (counters) {
        for (int o = 16; o > 0; o >>= 1) {
            ambiguous += __shfl_xor_sync(0xffffffffu, ambiguous, o);
            chunks += __shfl_xor_sync(0xffffffffu, chunks, o);
            misses += __shfl_xor_sync(0xffffffffu, misses, o);
        }
        if ((t & 31) == 0) {
            if (ambiguous) atomicAdd(counters + SARBP_CTR_AMBIGUOUS, (unsigned long long)ambiguous);
            if (chunks) atomicAdd(counters + SARBP_CTR_CHUNKS, (unsigned long long)chunks);
            if (misses) atomicAdd(counters + SARBP_CTR_WINDOW_MISS, (unsigned long long)misses);
        }
    }
}

// ---------------------------------------------------------------------------
// host side

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D tensor map over the pulse-major raw data: dim0 = range bins (8-byte
// complex64 elements), dim1 = pulses; box = W bins x CHUNK pulses.
static int make_raw_map(const SceneParams &P, int W, int chunk, CUtensorMap *map)
{
    auto enc = tensor_map_encoder();
    if (!enc) {
        set_error("staged path: cuTensorMapEncodeTiled is unavailable");
        return SARBP_ECUDA;
    }
    if ((reinterpret_cast<uintptr_t>(P.raw) & 15) || (P.pitch & 1)) {
        set_error("staged path needs 16-byte aligned raw data rows (raw 16-byte aligned, "
                  "raw_pitch even); got raw=%p pitch=%lld",
                  (const void *)P.raw, (long long)P.pitch);
        return SARBP_EINVAL;
    }
    cuuint64_t dims[2] = {(cuuint64_t)P.nra, (cuuint64_t)P.naz};
    cuuint64_t strides[1] = {(cuuint64_t)P.pitch * 8};
    cuuint32_t box[2] = {(cuuint32_t)W, (cuuint32_t)chunk};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<float2 *>(P.raw), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("staged path: cuTensorMapEncodeTiled failed (%d)", (int)r);
        return SARBP_ECUDA;
    }
    return SARBP_OK;
}

template <int CHUNK, int T0, int T1, int W>
int launch_staged_t(const SceneParams &P, const MixedLayout &L, char *ws, double *out,
                    int32_t *nvalid, uint64_t *checksum, uint64_t *counters, cudaStream_t stream)
{
    using SM = StagedSmem<CHUNK, W>;
    const int64_t nt0 = (P.dim0 + T0 - 1) / T0, nt1 = (P.dim1 + T1 - 1) / T1;
    const int64_t tiles = nt0 * nt1;
    if (tiles > 0x7fffffffLL) {
        set_error("sarbp_focus_mixed: %lld tiles exceed the launch limit", (long long)tiles);
        return SARBP_ERANGE;
    }
    CUtensorMap map;
    int rc = make_raw_map(P, W, CHUNK, &map);
    if (rc) return rc;
    auto *ptab = reinterpret_cast<const float4 *>(ws + L.ptab);
    auto *pff = reinterpret_cast<const PulseFF *>(ws + L.pff);
    auto *ctab = reinterpret_cast<const ChunkRef *>(ws + L.ctab);
    auto *status = reinterpret_cast<StatusBlock *>(ws + L.status);
    auto *ctr = reinterpret_cast<unsigned long long *>(counters);
    auto *k_fast = focus_mixed_staged_kernel<CHUNK, T0, T1, W, false>;
    auto *k_diag = focus_mixed_staged_kernel<CHUNK, T0, T1, W, true>;
    static bool attr_done = false;
    if (!attr_done) {
        rc = cuda_status(cudaFuncSetAttribute(k_fast, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)SM::bytes),
                         "staged smem attribute");
        if (rc) return rc;
        rc = cuda_status(cudaFuncSetAttribute(k_diag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)SM::bytes),
                         "staged smem attribute");
        if (rc) return rc;
        attr_done = true;
    }
    auto *k = checksum ? k_diag : k_fast;
    k<<<(unsigned)tiles, T0 * T1, SM::bytes, stream>>>(
        P, map, ptab, pff, ctab, nt0, reinterpret_cast<double2 *>(out), nvalid, checksum, ctr,
        status);
    return cuda_status(cudaGetLastError(), "focus_mixed_staged launch");
}

int launch_staged(const SceneParams &P, const sarbp_tuning &T, const MixedLayout &L, char *ws,
                  double *out, int32_t *nvalid, uint64_t *checksum, uint64_t *counters,
                  cudaStream_t stream)
{
    const int key = T.chunk * 1000000 + T.tile0 * 1000 + T.tile1;
    switch (key) {
        case 32 * 1000000 + 32 * 1000 + 8:
            return launch_staged_t<32, 32, 8, 128>(P, L, ws, out, nvalid, checksum, counters,
                                                   stream);
        case 32 * 1000000 + 64 * 1000 + 4:
            return launch_staged_t<32, 64, 4, 128>(P, L, ws, out, nvalid, checksum, counters,
                                                   stream);
        case 32 * 1000000 + 16 * 1000 + 16:
            return launch_staged_t<32, 16, 16, 128>(P, L, ws, out, nvalid, checksum, counters,
                                                    stream);
        default:
            set_error("staged path: unsupported tuning chunk=%d tile=%dx%d (chunk 32 only)",
                      T.chunk, T.tile0, T.tile1);
            return SARBP_EINVAL;
    }
}

}  // namespace sarbp
