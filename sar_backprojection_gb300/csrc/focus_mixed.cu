// focus_mixed.cu -- mixed-precision pixel-tiled back-projection.
//
// Work decomposition: one CTA per pixel tile (tile0 x tile1 pixels of the
// column-major DEM grid, one thread per pixel, each warp an 8 x 4 block of
// neighbouring pixels so that its lanes share apertures and range bins); the
// union of the tile's apertures is walked in pulse chunks aligned to
// multiples of `chunk`.  Precision plan: mixed_common.cuh.  This file holds
// the chunk-table prep kernel, the L1/L2-gather main kernel and the launch
// logic.
#include <climits>
#include <cstdio>

#include "mixed_common.cuh"

namespace sarbp {

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

MixedLayout mixed_layout(const SceneParams &P, const sarbp_tuning &T)
{
    MixedLayout L{};
    const int chunk = T.chunk;
    const int64_t naz = P.naz;
    size_t off = align256(sizeof(StatusBlock));
    const int64_t nchunks = (naz + chunk - 1) / chunk;
    L.ptab = off;      // padded to whole chunks: the staged kernel copies whole chunks
    off = align256(off + sizeof(float4) * (size_t)(nchunks * chunk));
    L.pff = off;
    off = align256(off + sizeof(PulseFF) * (size_t)naz);
    L.ctab = off;
    off = align256(off + sizeof(ChunkRef) * (size_t)nchunks);
    L.sdev = off;
    off = align256(off + sizeof(float) * (size_t)(nchunks * chunk / (T.stage > 0 ? T.stage : 32)));
    L.base = off;
    if (T.staged >= 2 && T.tile0 > 0 && T.tile1 > 0) {
        const int64_t nt = ((P.dim0 + T.tile0 - 1) / T.tile0) * ((P.dim1 + T.tile1 - 1) / T.tile1);
        L.ntiles = nt;
        L.keys_in = off;
        off = align256(off + 4 * (size_t)nt);
        L.vals_in = off;
        off = align256(off + 4 * (size_t)nt);
        L.keys_out = off;
        off = align256(off + 4 * (size_t)nt);
        L.vals_out = off;
        off = align256(off + 4 * (size_t)nt);
        L.sort_tmp = off;
        L.sort_tmp_bytes = tile_sort_bytes(nt);
        off = align256(off + L.sort_tmp_bytes);
        L.cursor = off;
        off = align256(off + sizeof(unsigned long long));
    }
    L.total = off;
    return L;
}

__host__ __device__ __forceinline__ int64_t chunk_ref(int64_t c, int chunk, int64_t naz)
{
    const int64_t k0 = c * chunk + chunk / 2;
    return k0 < naz - 1 ? k0 : naz - 1;
}

// e of pulse k into the per-pulse table.  AoS: one float4 (x, y, z, |e|^2)
// per pulse.  Paired (staged kernels): pulses 2p, 2p+1 share two float4,
// (x0, x1, y0, y1) and (z0, z1, w0, w1), the operands of packed f32x2 math;
// a 32-pulse stage still occupies float4 [K, K+32).
__device__ __forceinline__ void store_e(float4 *ptab, int64_t k, float4 e, bool paired)
{
    if (!paired) {
        ptab[k] = e;
        return;
    }
    float *f = reinterpret_cast<float *>(ptab) + (k >> 1) * 8 + (k & 1);
    f[0] = e.x;
    f[2] = e.y;
    f[4] = e.z;
    f[6] = e.w;
}

// Per-pulse tables and per-chunk references: one CTA per chunk, one thread
// per pulse (blockDim = chunk).
__global__ void chunk_table_kernel(const SceneParams P, int chunk, int stage, int paired,
                                   float4 *__restrict__ ptab, PulseFF *__restrict__ pff,
                                   ChunkRef *__restrict__ ctab, float *__restrict__ sdev,
                                   int64_t nchunks)
{
    __shared__ float4 s_max[4];
    const int64_t c = blockIdx.x;
    const int j = threadIdx.x, lane = j & 31;
    if (c >= nchunks) return;
    const int64_t k0 = chunk_ref(c, chunk, P.naz);
    const double x0 = P.tx[k0], y0 = P.ty[k0], z0 = P.tz[k0];
    const int64_t k = c * chunk + j;
    float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
    if (k < P.naz) {
        const double tx = P.tx[k], ty = P.ty[k], tz = P.tz[k];
        const double ex = tx - x0, ey = ty - y0, ez = tz - z0;
        e = make_float4((float)ex, (float)ey, (float)ez, (float)(ex * ex + ey * ey + ez * ez));
        PulseFF f;
        split_ff(tx, f.hi.x, f.lo.x);
        split_ff(ty, f.hi.y, f.lo.y);
        split_ff(tz, f.hi.z, f.lo.z);
        f.hi.w = f.lo.w = 0.f;
        pff[k] = f;
    }
    // padding past the last pulse is copied with whole stages by the staged
    // kernels and must hold finite values (never a kept pulse)
    store_e(ptab, k, e, paired);

    // Largest distance of a stage's pulses from the chord between its first
    // and last pulse (bounds the staged kernels' range windows); the stage's
    // pulses are `stage` consecutive lanes of one warp.
    const int64_t sa = c * chunk + (j / stage) * stage;
    double sd = 0.0;
    if (k < P.naz) {
        const int64_t sb = min(sa + stage - 1, P.naz - 1);
        const double bx = P.tx[sa], by = P.ty[sa], bz = P.tz[sa];
        const double vx = P.tx[sb] - bx, vy = P.ty[sb] - by, vz = P.tz[sb] - bz;
        const double vv = vx * vx + vy * vy + vz * vz;
        const double qx = P.tx[k] - bx, qy = P.ty[k] - by, qz = P.tz[k] - bz;
        const double u = vv > 0.0 ? (qx * vx + qy * vy + qz * vz) / vv : 0.0;
        const double rx = qx - u * vx, ry = qy - u * vy, rz = qz - u * vz;
        sd = sqrt(rx * rx + ry * ry + rz * rz);
    }
    for (int o = stage / 2; o > 0; o >>= 1) sd = fmax(sd, __shfl_xor_sync(0xffffffffu, sd, o));
    if (j % stage == 0) sdev[c * (chunk / stage) + j / stage] = (float)sd + 1.0e-3f;  // + margin

    // |e| component bounds over the chunk, rounded up by one part in 2^20 so
    // they hold for the FP32 values
    float mx = fabsf(e.x) * 1.000001f, my = fabsf(e.y) * 1.000001f;
    float mz = fabsf(e.z) * 1.000001f, m2 = e.w * 1.000001f;
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        my = fmaxf(my, __shfl_xor_sync(0xffffffffu, my, o));
        mz = fmaxf(mz, __shfl_xor_sync(0xffffffffu, mz, o));
        m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    }
    if (lane == 0) s_max[j / 32] = make_float4(mx, my, mz, m2);
    __syncthreads();
    if (j == 0) {
        float4 m = s_max[0];
        for (int w = 1; w < chunk / 32; ++w) {
            m.x = fmaxf(m.x, s_max[w].x);
            m.y = fmaxf(m.y, s_max[w].y);
            m.z = fmaxf(m.z, s_max[w].z);
            m.w = fmaxf(m.w, s_max[w].w);
        }
        ChunkRef r;
        r.emax = m;
        split_ff(x0, r.thi.x, r.tlo.x);
        split_ff(y0, r.thi.y, r.tlo.y);
        split_ff(z0, r.thi.z, r.tlo.z);
        r.thi.w = r.tlo.w = 0.f;
        ctab[c] = r;
    }
}

// Pixel of thread t in a tile: warps are 8 (dim0) x 4 (dim1) pixel blocks.
template <int T0, int T1>
__device__ __forceinline__ void tile_pixel(int t, int64_t tile0, int64_t tile1, int64_t &i0,
                                           int64_t &i1)
{
    static_assert(T0 % 8 == 0 && T1 % 4 == 0, "tile must be a multiple of the 8x4 warp block");
    const int w = t >> 5, lane = t & 31;
    i0 = tile0 * T0 + (w % (T0 / 8)) * 8 + (lane & 7);
    i1 = tile1 * T1 + (w / (T0 / 8)) * 4 + (lane >> 3);
}

// Main kernel, raw samples gathered through L1/L2.
template <int CHUNK, int T0, int T1, bool kChecksum>
__global__ void __launch_bounds__(T0 *T1)
focus_mixed_gather_kernel(const SceneParams P, const float4 *__restrict__ ptab,
                          const PulseFF *__restrict__ pff, const ChunkRef *__restrict__ ctab,
                          int64_t ntile0, double2 *__restrict__ out, int32_t *__restrict__ nvalid,
                          uint64_t *__restrict__ checksum,
                          unsigned long long *__restrict__ counters)
{
    __shared__ long long s_lo, s_hi;
    const int t = threadIdx.x;
    int64_t i0, i1;
    tile_pixel<T0, T1>(t, blockIdx.x % ntile0, blockIdx.x / ntile0, i0, i1);
    const bool inside = i0 < P.dim0 && i1 < P.dim1;
    const int64_t ii = inside ? i0 + P.dim0 * i1 : 0;
    int64_t lo = 0, hi = -1;
    const bool active =
        inside && pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi);

    if (t == 0) {
        s_lo = LLONG_MAX;
        s_hi = -1;
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
    unsigned ambiguous = 0, chunks = 0;
    const unsigned nra_m1 = (unsigned)(P.nra - 1);
    const int pitch = (int)P.pitch;

    if (thi >= 0) {
        for (int64_t c = tlo / CHUNK; c <= thi / CHUNK; ++c) {
            const int64_t K = c * CHUNK;
            const int jmin = (int)(lo > K ? lo - K : 0);
            const int jmax = (int)(hi < K + CHUNK - 1 ? hi - K : CHUNK - 1);
            if (!active || jmin > jmax) continue;
            ++chunks;
            ChunkRef ref;
            ref.emax = __ldg(&ctab[c].emax);
            ref.thi = __ldg(&ctab[c].thi);
            ref.tlo = __ldg(&ctab[c].tlo);
            ChunkSetup S;
            chunk_setup(P, pf, ref, S);
            if (S.exact) {
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
                continue;
            }
            const float4 *ep = ptab + K;
            const float2 *rowc = P.raw + K * P.pitch;
            const float tie = 0.5f - S.eps;
            float sre = 0.f, sim = 0.f;
#pragma unroll 4
            for (int j = jmin; j <= jmax; ++j) {
                const float4 e = __ldg(ep + j);
                const float D = fmaf(S.mx, e.x, fmaf(S.my, e.y, fmaf(S.mz, e.z, e.w)));
                const float dR = D * fmaf(fmaf(S.c3, D, S.c2), D, S.c1);
                const float g = fmaf(dR, P.inv_dra_f, S.g0);
                int ib;
                const float gr = round_shift(g, ib);
                int bin = S.n0 + ib;
                if (fabsf(__fsub_rn(g, gr)) > tie) {
                    bin = resolve_bin(P, pf, ii, pff, K + j);
                    ++ambiguous;
                }
                const bool ok = (unsigned)bin < nra_m1;
                float2 v = make_float2(0.f, 0.f);
                if (ok) v = __ldg(rowc + (j * pitch + bin));
                const float ph = dR * fmaf(P.beta_f, dR, S.a);
                float sn, cn;
                __sincosf(ph, &sn, &cn);
                const float tre = fmaf(v.x, cn, v.y * sn);
                const float tim = fmaf(v.y, cn, -(v.x * sn));
                const float w = S.r0sq + D;
                sre = fmaf(w, tre, sre);
                sim = fmaf(w, tim, sim);
                n += ok ? 1 : 0;
                if (kChecksum && ok) cs += mix64(K + j, bin);
            }
            // chunk sum * exp(-j*phi0)
            const float rre = fmaf(sre, S.w0re, -(sim * S.w0im));
            const float rim = fmaf(sre, S.w0im, sim * S.w0re);
            kahan_add(acc_re, cmp_re, rre);
            kahan_add(acc_im, cmp_im, rim);
        }
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
        }
        if ((t & 31) == 0) {
            if (ambiguous) atomicAdd(counters + SARBP_CTR_AMBIGUOUS, (unsigned long long)ambiguous);
            if (chunks) atomicAdd(counters + SARBP_CTR_CHUNKS, (unsigned long long)chunks);
        }
    }
}

template <int CHUNK, int T0, int T1>
static int launch_gather(const SceneParams &P, const MixedLayout &L, char *ws, double *out,
                         int32_t *nvalid, uint64_t *checksum, uint64_t *counters,
                         cudaStream_t stream)
{
    const int64_t nt0 = (P.dim0 + T0 - 1) / T0, nt1 = (P.dim1 + T1 - 1) / T1;
    const int64_t tiles = nt0 * nt1;
    if (tiles > 0x7fffffffLL) {
        set_error("sarbp_focus_mixed: %lld tiles exceed the launch limit", (long long)tiles);
        return SARBP_ERANGE;
    }
    auto *ptab = reinterpret_cast<const float4 *>(ws + L.ptab);
    auto *pff = reinterpret_cast<const PulseFF *>(ws + L.pff);
    auto *ctab = reinterpret_cast<const ChunkRef *>(ws + L.ctab);
    auto *ctr = reinterpret_cast<unsigned long long *>(counters);
    if (checksum)
        focus_mixed_gather_kernel<CHUNK, T0, T1, true><<<(unsigned)tiles, T0 * T1, 0, stream>>>(
            P, ptab, pff, ctab, nt0, reinterpret_cast<double2 *>(out), nvalid, checksum, ctr);
    else
        focus_mixed_gather_kernel<CHUNK, T0, T1, false><<<(unsigned)tiles, T0 * T1, 0, stream>>>(
            P, ptab, pff, ctab, nt0, reinterpret_cast<double2 *>(out), nvalid, nullptr, ctr);
    return cuda_status(cudaGetLastError(), "focus_mixed_gather launch");
}

int launch_staged(const SceneParams &P, const sarbp_tuning &T, const MixedLayout &L, char *ws,
                  bool queued, int64_t first, int64_t count, double *out, int32_t *nvalid,
                  uint64_t *checksum, uint64_t *counters, cudaStream_t stream);

int launch_chunk_table(const SceneParams &P, int chunk, int stage, bool paired, char *ws,
                       const MixedLayout &L, cudaStream_t stream)
{
    const int64_t nchunks = (P.naz + chunk - 1) / chunk;
    if (nchunks > 0x7fffffffLL) {
        set_error("chunk table: %lld chunks exceed the launch limit", (long long)nchunks);
        return SARBP_ERANGE;
    }
    chunk_table_kernel<<<(unsigned)nchunks, chunk, 0, stream>>>(
        P, chunk, stage, paired ? 1 : 0, reinterpret_cast<float4 *>(ws + L.ptab),
        reinterpret_cast<PulseFF *>(ws + L.pff), reinterpret_cast<ChunkRef *>(ws + L.ctab),
        reinterpret_cast<float *>(ws + L.sdev), nchunks);
    return cuda_status(cudaGetLastError(), "chunk_table launch");
}

// Bounds of the range bins a pixel can reach over its aperture, per stage of
// `stage` pulses as in the staged kernels' window prologue, reduced to one
// [min, max] for the scene (ints in the status block).  Each block first
// stages every stage's segment geometry (first pulse, direction, 1/|s|^2,
// chord deviation) in shared memory; each thread then bounds kBinRangePix
// pixels from it.
constexpr int kBinRangePix = 4;

__global__ void raw_bin_range_kernel(const SceneParams P, const PulseFF *__restrict__ pff,
                                     const float *__restrict__ sdev, int stage, int64_t nstages,
                                     int *range)
{
    extern __shared__ float4 geo[];   // [nstages][2]
    for (int64_t c = threadIdx.x; c < nstages; c += blockDim.x) {
        const int64_t K = c * stage, kb = min(K + stage - 1, P.naz - 1);
        const float4 ta = __ldg(&pff[K].hi), tb = __ldg(&pff[kb].hi);
        const float sx = tb.x - ta.x, sy = tb.y - ta.y, sz = tb.z - ta.z;
        const float ss = sx * sx + sy * sy + sz * sz;
        geo[2 * c] = make_float4(ta.x, ta.y, ta.z, ss > 0.f ? 1.0f / ss : 0.f);
        geo[2 * c + 1] = make_float4(sx, sy, sz, __ldg(&sdev[c]));
    }
    __syncthreads();
    int blo = INT_MAX, bhi = INT_MIN;
    for (int r = 0; r < kBinRangePix; ++r) {
        const int64_t ii =
            ((int64_t)blockIdx.x * kBinRangePix + r) * blockDim.x + threadIdx.x;
        int64_t lo, hi;
        if (ii >= P.npix ||
            !pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi))
            continue;
        const PixelFF pf = pixel_ff(P.x[ii], P.y[ii], P.z[ii]);
        float rmin2 = 3.0e38f, rmax2 = 0.f, dmax = 0.f;
        for (int64_t c = lo / stage; c <= hi / stage; ++c) {
            const float4 g0 = geo[2 * c], g1 = geo[2 * c + 1];
            const float ax = pf.xh - g0.x, ay = pf.yh - g0.y, az = pf.zh - g0.z;
            const float a2 = ax * ax + ay * ay + az * az;
            const float d = ax * g1.x + ay * g1.y + az * g1.z;
            const float u = d * g0.w;
            const float bx = ax - g1.x, by = ay - g1.y, bz = az - g1.z;
            const float b2 = bx * bx + by * by + bz * bz;
            rmin2 = fminf(rmin2, (u > 0.f && u < 1.f) ? fmaf(-d, u, a2) : fminf(a2, b2));
            rmax2 = fmaxf(rmax2, fmaxf(a2, b2));
            dmax = fmaxf(dmax, g1.w);
        }
        // approximate square roots (relative error ~1e-6) inside the 1-bin margin
        rmin2 = fmaxf(rmin2, 0.f);
        const float rmin = rmin2 > 0.f ? rmin2 * rsqrtf(rmin2) : 0.f;
        const float rmax = rmax2 > 0.f ? rmax2 * rsqrtf(rmax2) : 0.f;
        blo = min(blo, (int)floorf((rmin - dmax - P.near_hi) * P.inv_dra_f) - 1);
        bhi = max(bhi, (int)ceilf((rmax + dmax - P.near_hi) * P.inv_dra_f) + 1);
    }
    blo = __reduce_min_sync(0xffffffffu, blo);
    bhi = __reduce_max_sync(0xffffffffu, bhi);
    if ((threadIdx.x & 31) == 0 && blo <= bhi) {
        atomicMin(&range[0], blo);
        atomicMax(&range[1], bhi);
    }
}

// The same bound for scenes whose stage table does not fit in shared memory:
// stage geometry read from the pulse tables, one pixel per thread.
__global__ void raw_bin_range_gmem_kernel(const SceneParams P, const PulseFF *__restrict__ pff,
                                          const float *__restrict__ sdev, int stage, int *range)
{
    const int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int blo = INT_MAX, bhi = INT_MIN;
    int64_t lo, hi;
    if (ii < P.npix && pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi)) {
        const PixelFF pf = pixel_ff(P.x[ii], P.y[ii], P.z[ii]);
        float rmin2 = 3.0e38f, rmax2 = 0.f, dmax = 0.f;
        for (int64_t c = lo / stage; c <= hi / stage; ++c) {
            const int64_t K = c * stage, kb = min(K + stage - 1, P.naz - 1);
            const float4 ta = __ldg(&pff[K].hi), tb = __ldg(&pff[kb].hi);
            const float ax = pf.xh - ta.x, ay = pf.yh - ta.y, az = pf.zh - ta.z;
            const float sx = tb.x - ta.x, sy = tb.y - ta.y, sz = tb.z - ta.z;
            const float ss = sx * sx + sy * sy + sz * sz;
            const float a2 = ax * ax + ay * ay + az * az;
            const float d = ax * sx + ay * sy + az * sz;
            const float u = ss > 0.f ? d / ss : 0.f;
            const float bx = ax - sx, by = ay - sy, bz = az - sz;
            const float b2 = bx * bx + by * by + bz * bz;
            rmin2 = fminf(rmin2, (u > 0.f && u < 1.f) ? fmaf(-d, u, a2) : fminf(a2, b2));
            rmax2 = fmaxf(rmax2, fmaxf(a2, b2));
            dmax = fmaxf(dmax, __ldg(&sdev[c]));
        }
        const float rmin = sqrtf(fmaxf(rmin2, 0.f)), rmax = sqrtf(rmax2);
        blo = (int)floorf((rmin - dmax - P.near_hi) * P.inv_dra_f) - 1;
        bhi = (int)ceilf((rmax + dmax - P.near_hi) * P.inv_dra_f) + 1;
    }
    blo = __reduce_min_sync(0xffffffffu, blo);
    bhi = __reduce_max_sync(0xffffffffu, bhi);
    if ((threadIdx.x & 31) == 0 && blo <= bhi) {
        atomicMin(&range[0], blo);
        atomicMax(&range[1], bhi);
    }
}

__global__ void range_init_kernel(int *range)
{
    range[0] = INT_MAX;
    range[1] = INT_MIN;
}

// The reduced interval as the entry points report it: [1, 0] when no pixel
// has an aperture, else clamped to the bins 0..nra-1 of a pulse row.
__global__ void range_finish_kernel(int *range, int64_t nra)
{
    const int lo = range[0], hi = range[1];
    if (lo > hi) {
        range[0] = 1;
        range[1] = 0;
    } else {
        range[0] = lo < 0 ? 0 : lo;
        range[1] = (int64_t)hi > nra - 1 ? (int)(nra - 1) : hi;
    }
}

// Enqueue the bound of the reachable bins and its copy into host[0..1]
// (int32), then clear the status block's spare words again (read by
// sarbp_mixed_status).  Nothing is synchronised.
static int raw_bin_range_enqueue(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                                 size_t ws_bytes, int32_t *host, const char *who,
                                 cudaStream_t stream)
{
    const MixedLayout L = mixed_layout(P, T);
    if (!workspace || ws_bytes < L.total || !host) {
        set_error("%s: workspace (%zu < %zu bytes) or range missing", who, ws_bytes, L.total);
        return SARBP_EWORKSPACE;
    }
    if (!T.staged) {
        set_error("%s: needs tables prepared with a staged tuning", who);
        return SARBP_EINVAL;
    }
    char *ws = static_cast<char *>(workspace);
    int *dr = reinterpret_cast<StatusBlock *>(ws + L.status)->range;
    range_init_kernel<<<1, 1, 0, stream>>>(dr);
    const int64_t per_block = 256 * kBinRangePix;
    const int64_t blocks = (P.npix + per_block - 1) / per_block;
    const int64_t nstages = (P.naz + T.stage - 1) / T.stage;
    const size_t smem = sizeof(float4) * 2 * (size_t)nstages;
    const auto *pff = reinterpret_cast<const PulseFF *>(ws + L.pff);
    const auto *sdv = reinterpret_cast<const float *>(ws + L.sdev);
    int rc = SARBP_OK;
    if (smem <= 200 * 1024) {
        rc = cuda_status(cudaFuncSetAttribute(raw_bin_range_kernel,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem),
                         "raw_bin_range smem attribute");
        if (rc) return rc;
        if (blocks > 0)
            raw_bin_range_kernel<<<(unsigned)blocks, 256, smem, stream>>>(P, pff, sdv, T.stage,
                                                                          nstages, dr);
    } else if (P.npix > 0) {
        raw_bin_range_gmem_kernel<<<(unsigned)((P.npix + 255) / 256), 256, 0, stream>>>(
            P, pff, sdv, T.stage, dr);
    }
    range_finish_kernel<<<1, 1, 0, stream>>>(dr, P.nra);
    rc = cuda_status(cudaGetLastError(), "raw_bin_range launch");
    if (rc) return rc;
    rc = cuda_status(cudaMemcpyAsync(host, dr, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                     stream),
                     "raw_bin_range read");
    if (rc) return rc;
    return cuda_status(cudaMemsetAsync(dr, 0, 2 * sizeof(int), stream), "raw_bin_range clear");
}

int raw_bin_range(const SceneParams &P, const sarbp_tuning &T, void *workspace, size_t ws_bytes,
                  int64_t *range, cudaStream_t stream)
{
    if (!range) {
        set_error("sarbp_raw_bin_range: range missing");
        return SARBP_EINVAL;
    }
    int32_t h[2];
    int rc = raw_bin_range_enqueue(P, T, workspace, ws_bytes, h, "sarbp_raw_bin_range", stream);
    if (rc) return rc;
    rc = cuda_status(cudaStreamSynchronize(stream), "raw_bin_range synchronize");
    if (rc) return rc;
    range[0] = h[0];
    range[1] = h[1];
    return SARBP_OK;
}

int raw_bin_range_async(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                        size_t ws_bytes, int32_t *host_range, cudaStream_t stream)
{
    return raw_bin_range_enqueue(P, T, workspace, ws_bytes, host_range,
                                 "sarbp_raw_bin_range_async", stream);
}

static int check_workspace(const MixedLayout &L, void *workspace, size_t ws_bytes)
{
    if (!workspace || ws_bytes < L.total) {
        set_error("sarbp mixed path: workspace of %zu bytes is smaller than the %zu required",
                  ws_bytes, L.total);
        return SARBP_EWORKSPACE;
    }
    return SARBP_OK;
}

int launch_mixed_prepare(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                         size_t ws_bytes, cudaStream_t stream)
{
    const MixedLayout L = mixed_layout(P, T);
    int rc = check_workspace(L, workspace, ws_bytes);
    if (rc) return rc;
    char *ws = static_cast<char *>(workspace);
    // the staged kernels read the pair-interleaved table (f32x2 operands)
    // a prepared workspace starts with a clear status (sarbp_mixed_status)
    rc = cuda_status(cudaMemsetAsync(ws + L.status, 0, sizeof(StatusBlock), stream),
                     "status reset");
    if (rc) return rc;
    rc = launch_chunk_table(P, T.chunk, T.stage > 0 ? T.stage : 32, T.staged != 0, ws, L, stream);
    if (rc) return rc;
    // persistent staged path: tiles in decreasing estimated cost
    if (T.staged >= 2) return tile_order(P, T, L, ws, stream);
    return SARBP_OK;
}

int launch_mixed_main(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                      size_t ws_bytes, double *out, int32_t *nvalid, uint64_t *checksum,
                      uint64_t *counters, cudaStream_t stream)
{
    const MixedLayout L = mixed_layout(P, T);
    int rc = check_workspace(L, workspace, ws_bytes);
    if (rc) return rc;
    if (P.pitch * (int64_t)T.chunk + P.nra >= (1LL << 31)) {
        set_error("sarbp mixed path: raw_pitch %lld too large for %d-pulse chunks",
                  (long long)P.pitch, T.chunk);
        return SARBP_ERANGE;
    }
    char *ws = static_cast<char *>(workspace);
    if (T.staged) {
        SceneParams Ps = P;
        Ps.wait_polls = T.wait_polls > 0 ? (uint32_t)T.wait_polls : (1u << 22);
        Ps.withhold = T.withhold;
        return launch_staged(Ps, T, L, ws, T.staged >= 2, 0, -1, out, nvalid, checksum,
                             counters, stream);
    }
    const int key = T.chunk * 1000000 + T.tile0 * 1000 + T.tile1;
    switch (key) {
        case 32 * 1000000 + 32 * 1000 + 8:
            return launch_gather<32, 32, 8>(P, L, ws, out, nvalid, checksum, counters, stream);
        case 64 * 1000000 + 32 * 1000 + 8:
            return launch_gather<64, 32, 8>(P, L, ws, out, nvalid, checksum, counters, stream);
        case 32 * 1000000 + 64 * 1000 + 4:
            return launch_gather<32, 64, 4>(P, L, ws, out, nvalid, checksum, counters, stream);
        case 64 * 1000000 + 64 * 1000 + 4:
            return launch_gather<64, 64, 4>(P, L, ws, out, nvalid, checksum, counters, stream);
        case 32 * 1000000 + 16 * 1000 + 16:
            return launch_gather<32, 16, 16>(P, L, ws, out, nvalid, checksum, counters, stream);
        case 64 * 1000000 + 16 * 1000 + 16:
            return launch_gather<64, 16, 16>(P, L, ws, out, nvalid, checksum, counters, stream);
        default:
            set_error("sarbp mixed path: unsupported tuning chunk=%d tile=%dx%d", T.chunk,
                      T.tile0, T.tile1);
            return SARBP_EINVAL;
    }
}

}  // namespace sarbp

namespace sarbp {

// Queue items [first, first + count) of a workspace prepared with staged >= 2.
int launch_mixed_range(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                       size_t ws_bytes, int64_t first, int64_t count, double *out,
                       int32_t *nvalid, uint64_t *checksum, uint64_t *counters,
                       cudaStream_t stream)
{
    if (T.staged < 2) {
        set_error("sarbp_focus_mixed_range: needs a queued tuning (staged 2 or 3)");
        return SARBP_EINVAL;
    }
    const MixedLayout L = mixed_layout(P, T);
    int rc = check_workspace(L, workspace, ws_bytes);
    if (rc) return rc;
    SceneParams Ps = P;
    Ps.wait_polls = T.wait_polls > 0 ? (uint32_t)T.wait_polls : (1u << 22);
    Ps.withhold = T.withhold;
    return launch_staged(Ps, T, L, static_cast<char *>(workspace), true, first, count, out,
                         nvalid, checksum, counters, stream);
}

// The prepared queue's sorted keys (staged=2: tile costs, staged=3: one past
// each tile's last pulse) into host memory; synchronises the stream.
int tile_queue_keys(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                    size_t ws_bytes, uint32_t *keys, int64_t n, cudaStream_t stream)
{
    const MixedLayout L = mixed_layout(P, T);
    int rc = check_workspace(L, workspace, ws_bytes);
    if (rc) return rc;
    if (T.staged < 2 || !keys || n != L.ntiles) {
        set_error("sarbp_tile_queue_keys: needs a queued tuning and %lld keys",
                  (long long)L.ntiles);
        return SARBP_EINVAL;
    }
    rc = cuda_status(cudaMemcpyAsync(keys, static_cast<char *>(workspace) + L.keys_out,
                                     sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToHost, stream),
                     "tile queue keys read");
    if (rc) return rc;
    return cuda_status(cudaStreamSynchronize(stream), "tile queue keys synchronize");
}

}  // namespace sarbp
