// focus_staged.cu -- host side of the TMA-staged kernels: tensor maps,
// per-chunk-size dispatch, batch workspaces, tile cost and queue order.
// The kernels and their launch templates are in staged_kernels.cuh.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>

#include <cub/device/device_radix_sort.cuh>

#include "staged_kernels.cuh"

namespace sarbp {

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
// complex64 elements), dim1 = pulses; box = W bins x `rows` pulses.
int make_raw_map(const SceneParams &P, int W, int rows, CUtensorMap *map)
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
    cuuint32_t box[2] = {(cuuint32_t)W, (cuuint32_t)rows};
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

// Dispatch on the chunk size; the (tile, window) variants of each chunk size
// are built in their own translation unit.
SARBP_STAGED_CHUNK_EXTERN(extern, 32)
SARBP_STAGED_CHUNK_EXTERN(extern, 64)
SARBP_STAGED_CHUNK_EXTERN(extern, 128)

int launch_staged(const SceneParams &P, const sarbp_tuning &T, const MixedLayout &L, char *ws,
                  bool queued, int64_t first, int64_t count, double *out, int32_t *nvalid,
                  uint64_t *checksum, uint64_t *counters, cudaStream_t stream)
{
    switch (T.chunk) {
        case 32:
            return launch_staged_chunk<32>(P, T, L, ws, queued, first, count, out, nvalid,
                                           checksum, counters, stream);
        case 64:
            return launch_staged_chunk<64>(P, T, L, ws, queued, first, count, out, nvalid,
                                           checksum, counters, stream);
        case 128:
            return launch_staged_chunk<128>(P, T, L, ws, queued, first, count, out, nvalid,
                                            checksum, counters, stream);
        default:
            set_error("staged path: unsupported chunk %d", T.chunk);
            return SARBP_EINVAL;
    }
}

int64_t batch_workspace_size(int nscenes, int64_t max_items)
{
    return (int64_t)batch_layout(nscenes, max_items).total;
}

static int tiling_tiles(const SceneParams &P, const sarbp_tuning &T, int64_t *nt0, int64_t *nt)
{
    if (T.tile0 <= 0 || T.tile1 <= 0) {
        set_error("tiling: tile extents must be positive");
        return SARBP_EINVAL;
    }
    *nt0 = (P.dim0 + T.tile0 - 1) / T.tile0;
    *nt = *nt0 * ((P.dim1 + T.tile1 - 1) / T.tile1);
    return SARBP_OK;
}

// Stores one batch scene descriptor.  The descriptor travels as a kernel
// parameter: the write is stream-ordered like a copy, but the host neither
// waits for the stream (a copy from pageable host memory would) nor has to
// keep a pinned copy alive until it executes.
__global__ void store_batch_scene_kernel(BatchScene *dst, const __grid_constant__ BatchScene B)
{
    if (threadIdx.x == 0) *dst = B;
}

int batch_set_scene(void *bws, size_t bytes, int slot, int nscenes, const SceneParams &P,
                    const sarbp_tuning &T, void *scene_ws, size_t scene_ws_bytes, double *out,
                    int32_t *nvalid, uint64_t *checksum, cudaStream_t stream)
{
    if (!T.staged || (T.chunk != 32 && T.chunk != 64 && T.chunk != 128)) {
        set_error("batch path: needs the staged kernel (32-, 64- or 128-pulse chunks)");
        return SARBP_EINVAL;
    }
    const BatchLayout BL = batch_layout(nscenes, 0);
    if (!bws || slot < 0 || slot >= nscenes || bytes < BL.items) {
        set_error("batch path: slot %d outside the %d-scene workspace", slot, nscenes);
        return SARBP_EINVAL;
    }
    const MixedLayout L = mixed_layout(P, T);
    if (!scene_ws || scene_ws_bytes < L.base || !out) {
        set_error("batch path: scene workspace (%zu < %zu bytes) or output missing",
                  scene_ws_bytes, L.base);
        return SARBP_EWORKSPACE;
    }
    BatchScene B;
    memset(&B, 0, sizeof(B));
    int rc = make_raw_map(P, T.window, T.stage, &B.map);
    if (rc) return rc;
    B.P = P;
    B.P.wait_polls = T.wait_polls > 0 ? (uint32_t)T.wait_polls : (1u << 22);
    B.P.withhold = T.withhold;
    B.tables = tables_of(static_cast<char *>(scene_ws), L);
    B.outputs = TileOutputs{reinterpret_cast<double2 *>(out), nvalid, checksum};
    rc = tiling_tiles(P, T, &B.ntile0, &B.ntiles);
    if (rc) return rc;
    char *dst = static_cast<char *>(bws) + BL.scenes + sizeof(BatchScene) * (size_t)slot;
    store_batch_scene_kernel<<<1, 32, 0, stream>>>(reinterpret_cast<BatchScene *>(dst), B);
    return cuda_status(cudaGetLastError(), "batch scene upload");
}

int batch_set_items(void *bws, size_t bytes, int nscenes, const int32_t *items, int64_t n,
                    cudaStream_t stream)
{
    const BatchLayout BL = batch_layout(nscenes, n);
    if (!bws || bytes < BL.total || (n > 0 && !items)) {
        set_error("batch path: workspace of %zu bytes too small for %lld items", bytes,
                  (long long)n);
        return SARBP_EWORKSPACE;
    }
    if (n == 0) return SARBP_OK;
    return cuda_status(cudaMemcpyAsync(static_cast<char *>(bws) + BL.items, items,
                                       sizeof(int2) * (size_t)n, cudaMemcpyHostToDevice, stream),
                       "batch items upload");
}

int batch_focus(void *bws, size_t bytes, int nscenes, const sarbp_tuning &T, int64_t n_items,
                bool diag, uint64_t *counters, cudaStream_t stream)
{
    const BatchLayout BL = batch_layout(nscenes, n_items);
    if (!bws || bytes < BL.total) {
        set_error("batch path: workspace of %zu bytes too small (%zu)", bytes, BL.total);
        return SARBP_EWORKSPACE;
    }
    if (n_items <= 0) return SARBP_OK;
    char *ws = static_cast<char *>(bws);
    if (!T.staged) {
        set_error("batch path: needs the staged kernel (staged > 0)");
        return SARBP_EINVAL;
    }
    switch (T.chunk) {
        case 32: return launch_batch_chunk<32>(ws, BL, T, n_items, diag, counters, stream);
        case 64: return launch_batch_chunk<64>(ws, BL, T, n_items, diag, counters, stream);
        case 128: return launch_batch_chunk<128>(ws, BL, T, n_items, diag, counters, stream);
        default:
            set_error("batch path: unsupported chunk %d", T.chunk);
            return SARBP_EINVAL;
    }
}

// Estimated cost of each tile of a scene: the sum of its pixels' kept
// aperture lengths (nominal pixel-pulses), for ordering batch work.
template <int T0, int T1>
__global__ void tile_cost_kernel(const SceneParams P, int64_t ntile0, int64_t ntiles,
                                 int64_t *__restrict__ costs)
{
    const int64_t tile = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tile >= ntiles) return;
    const int64_t t0 = tile % ntile0, t1 = tile / ntile0;
    int64_t c = 0;
    for (int b = 0; b < T1; ++b)
        for (int a = 0; a < T0; ++a) {
            const int64_t i0 = t0 * T0 + a, i1 = t1 * T1 + b;
            if (i0 >= P.dim0 || i1 >= P.dim1) continue;
            const int64_t ii = i0 + P.dim0 * i1;
            int64_t lo, hi;
            if (pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi))
                c += hi - lo + 1;
        }
    costs[tile] = c;
}

int tile_costs(const SceneParams &P, const sarbp_tuning &T, int64_t *costs, cudaStream_t stream)
{
    int64_t nt0, nt;
    int rc = tiling_tiles(P, T, &nt0, &nt);
    if (rc) return rc;
    const unsigned blocks = (unsigned)((nt + 127) / 128);
#define X(A, B)                                                                             \
    if (T.tile0 == A && T.tile1 == B) {                                                     \
        tile_cost_kernel<A, B><<<blocks, 128, 0, stream>>>(P, nt0, nt, costs);              \
        return cuda_status(cudaGetLastError(), "tile_cost launch");                         \
    }
    X(16, 16) X(16, 8) X(32, 8) X(64, 4)
#undef X
    set_error("tile costs: unsupported tile %dx%d", T.tile0, T.tile1);
    return SARBP_EINVAL;
}

// Queue key of each tile: its estimated cost (sum of its pixels' kept
// aperture lengths) or, with kEnd, one past its last kept pulse (0 for a tile
// without apertures).  One warp per tile, lanes over its pixels.
template <int T0, int T1, bool kEnd>
__global__ void tile_key_kernel(const SceneParams P, int64_t ntile0, int64_t ntiles,
                                uint32_t *__restrict__ keys, int32_t *__restrict__ ids)
{
    const int64_t tile = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (tile >= ntiles) return;              // warp-uniform
    const int64_t t0 = tile % ntile0, t1 = tile / ntile0;
    unsigned long long c = 0;
    for (int p = lane; p < T0 * T1; p += 32) {
        const int64_t i0 = t0 * T0 + p % T0, i1 = t1 * T1 + p / T0;
        if (i0 >= P.dim0 || i1 >= P.dim1) continue;
        const int64_t ii = i0 + P.dim0 * i1;
        int64_t lo, hi;
        if (pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi)) {
            if (kEnd)
                c = c > (unsigned long long)(hi + 1) ? c : (unsigned long long)(hi + 1);
            else
                c += (unsigned long long)(hi - lo + 1);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, c, o);
        c = kEnd ? (c > v ? c : v) : c + v;
    }
    if (lane == 0) {
        keys[tile] = c > 0xffffffffull ? 0xffffffffu : (uint32_t)c;
        ids[tile] = (int32_t)tile;
    }
}

size_t tile_sort_bytes(int64_t ntiles)
{
    size_t a = 0, b = 0;
    cub::DeviceRadixSort::SortPairsDescending((void *)nullptr, a, (const uint32_t *)nullptr,
                                              (uint32_t *)nullptr, (const int32_t *)nullptr,
                                              (int32_t *)nullptr, (int)ntiles);
    cub::DeviceRadixSort::SortPairs((void *)nullptr, b, (const uint32_t *)nullptr,
                                    (uint32_t *)nullptr, (const int32_t *)nullptr,
                                    (int32_t *)nullptr, (int)ntiles);
    return a > b ? a : b;
}

// The workspace tile queue: staged=2 in decreasing estimated cost (longest
// tiles first), staged=3 in increasing last pulse (a tile can run as soon as
// the raw rows up to its last pulse are resident); key kernel + device radix
// sort, stream-ordered.
int tile_order(const SceneParams &P, const sarbp_tuning &T, const MixedLayout &L, char *ws,
               cudaStream_t stream)
{
    const int64_t nt = L.ntiles;
    if (nt <= 0) return SARBP_OK;
    if (nt > 0x7fffffffLL) {
        set_error("tile order: %lld tiles exceed the queue limit", (long long)nt);
        return SARBP_ERANGE;
    }
    const int64_t nt0 = (P.dim0 + T.tile0 - 1) / T.tile0;
    auto *keys_in = reinterpret_cast<uint32_t *>(ws + L.keys_in);
    auto *vals_in = reinterpret_cast<int32_t *>(ws + L.vals_in);
    const unsigned blocks = (unsigned)((nt + 7) / 8);   // 8 warps (tiles) per block
    const bool by_end = T.staged == 3;
    bool launched = false;
#define X(A, B)                                                                             \
    if (!launched && T.tile0 == A && T.tile1 == B) {                                        \
        if (by_end)                                                                         \
            tile_key_kernel<A, B, true><<<blocks, 256, 0, stream>>>(P, nt0, nt, keys_in,    \
                                                                    vals_in);               \
        else                                                                                \
            tile_key_kernel<A, B, false><<<blocks, 256, 0, stream>>>(P, nt0, nt, keys_in,   \
                                                                     vals_in);              \
        launched = true;                                                                    \
    }
    X(16, 16) X(16, 8) X(32, 8) X(64, 4)
#undef X
    if (!launched) {
        set_error("tile order: unsupported tile %dx%d", T.tile0, T.tile1);
        return SARBP_EINVAL;
    }
    int rc = cuda_status(cudaGetLastError(), "tile_key launch");
    if (rc) return rc;
    size_t tmp = L.sort_tmp_bytes;
    auto *keys_out = reinterpret_cast<uint32_t *>(ws + L.keys_out);
    auto *vals_out = reinterpret_cast<int32_t *>(ws + L.vals_out);
    const cudaError_t e =
        by_end ? cub::DeviceRadixSort::SortPairs(ws + L.sort_tmp, tmp, keys_in, keys_out, vals_in,
                                                 vals_out, (int)nt, 0, 32, stream)
               : cub::DeviceRadixSort::SortPairsDescending(ws + L.sort_tmp, tmp, keys_in,
                                                           keys_out, vals_in, vals_out, (int)nt,
                                                           0, 32, stream);
    return cuda_status(e, "tile order sort");
}

int tile_count(const SceneParams &P, const sarbp_tuning &T, int64_t *nt)
{
    int64_t nt0;
    return tiling_tiles(P, T, &nt0, nt);
}

}  // namespace sarbp
