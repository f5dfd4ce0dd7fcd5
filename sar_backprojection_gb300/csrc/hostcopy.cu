// hostcopy.cu -- host-to-device copies done by SM loads instead of a copy
// engine.
//
// On the GB300 machines this library is measured on, copy-engine transfers from
// page-locked host memory stall for 10-100 ms every so often (about every
// 0.5 s under a steady load), while kernels reading the same memory through
// its mapped device address over the CPU-GPU link ran without a stall in
// every measurement (at 185-190 GB/s against the copy engine's ~205 GB/s).
// A caller that mostly waits on uploads rather than on kernels (the serving
// loop) gets a steadier latency from these copies.  The source must be
// page-locked host memory mapped into the device's address space (what
// cudaHostAlloc / torch pin_memory give), device memory, or -- on a device
// that reads pageable host memory through the host's page tables (the
// pageableMemoryAccessUsesHostPageTables attribute: coherent CPU-GPU
// systems such as GB300 with its NVLink-C2C link) -- any host memory, read
// in place at the link's rate instead of staged by the driver; anything
// else is rejected before any launch.
#include <algorithm>

#include <sys/mman.h>
#include <unistd.h>

#include "sarbp_internal.cuh"

namespace sarbp {

// Whether the current device loads from and stores to pageable host memory
// through the host's page tables (one query per device, cached).
static bool reads_pageable()
{
    constexpr int kMaxDev = 64;
    static int known[kMaxDev];                        // 0 unknown, 1 no, 2 yes
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
        cudaGetLastError();
        return false;
    }
    if (!known[dev]) {
        int a = 0, b = 0;
        const bool ok =
            cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                   dev) == cudaSuccess;
        if (!ok) cudaGetLastError();
        known[dev] = ok && a && b ? 2 : 1;
    }
    return known[dev] == 2;
}

// Whether the pageable host range [p, p + bytes) may be handed to a kernel:
// every page of it mapped in this process (msync fails with ENOMEM
// otherwise), and, for a range the kernel will write, every page touched
// here first (read and written back), so an unmapped or read-only
// destination fails on the host, never as a device fault.
static bool pageable_range_ok(const void *p, int64_t bytes, bool write)
{
    if (!p || bytes <= 0) return false;
    const uintptr_t pg = (uintptr_t)sysconf(_SC_PAGESIZE);
    const uintptr_t b = reinterpret_cast<uintptr_t>(p), e = b + (uintptr_t)bytes;
    if (pg == 0 || (pg & (pg - 1)) || e < b) return false;
    const uintptr_t a = b & ~(pg - 1);
    if (msync(reinterpret_cast<void *>(a), e - a, MS_ASYNC) != 0) return false;
    if (write)
        for (uintptr_t q = b; q < e; q = (q & ~(pg - 1)) + pg) {
            volatile unsigned char *c = reinterpret_cast<volatile unsigned char *>(q);
            const unsigned char v = *c;
            *c = v;
        }
    return true;
}

// Device address of host or device memory `p` for kernel loads (stores when
// `write`) over `bytes` bytes, or nullptr when a kernel cannot reach it:
// page-locked host memory through its mapping, device and managed memory as
// they are, pageable host memory as it is on a device that reads it through
// the host's page tables, once the range has been checked on the host.
static const void *device_view(const void *p, int64_t bytes, bool write = false)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();   // clear the sticky-free error of an unknown pointer
        return nullptr;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return p;
    if (at.type == cudaMemoryTypeHost) return at.devicePointer;
    if (at.type == cudaMemoryTypeUnregistered && reads_pageable() &&
        pageable_range_ok(p, bytes, write))
        return p;
    return nullptr;
}

constexpr int kCopyThreads = 256;
constexpr int kCopyUnroll = 4;

// dst[r*dpitch + lo + i] = src[r*spitch + lo + i], i < n, r < rows (complex64).
__global__ void __launch_bounds__(kCopyThreads)
gather_rows_kernel(float2 *__restrict__ dst, int64_t dpitch, const float2 *__restrict__ src,
                   int64_t spitch, int64_t lo, int64_t n, int64_t rows)
{
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const float2 *s = src + r * spitch + lo;
        float2 *d = dst + r * dpitch + lo;
        for (int64_t i = threadIdx.x; i < n; i += (int64_t)kCopyUnroll * kCopyThreads) {
            float2 v[kCopyUnroll];
#pragma unroll
            for (int u = 0; u < kCopyUnroll; ++u) {
                const int64_t k = i + (int64_t)u * kCopyThreads;
                if (k < n) v[u] = s[k];
            }
#pragma unroll
            for (int u = 0; u < kCopyUnroll; ++u) {
                const int64_t k = i + (int64_t)u * kCopyThreads;
                if (k < n) d[k] = v[u];
            }
        }
    }
}

// The same rows as 16-byte words (two complex64 samples per load) for even
// pitches and 16-byte aligned buffers: bins [lo, lo + n) split into an odd
// head bin, a body of whole pairs and an odd tail bin, so exactly those bins
// are written.  Half the load instructions for the same bytes in flight.

__global__ void __launch_bounds__(kCopyThreads)
gather_rows16_kernel(float2 *__restrict__ dst, int64_t dpitch, const float2 *__restrict__ src,
                     int64_t spitch, int64_t lo, int64_t n, int64_t rows)
{
    const int64_t lo_up = (lo + 1) & ~int64_t(1), hi = lo + n, hi_dn = hi & ~int64_t(1);
    const int64_t n2 = hi_dn > lo_up ? (hi_dn - lo_up) / 2 : 0;
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const float2 *srow = src + r * spitch;
        float2 *drow = dst + r * dpitch;
        if (threadIdx.x == 0) {
            if (lo & 1) drow[lo] = srow[lo];
            if ((hi & 1) && hi - 1 >= lo_up) drow[hi - 1] = srow[hi - 1];
        }
        const uint4 *s = reinterpret_cast<const uint4 *>(srow + lo_up);
        uint4 *d = reinterpret_cast<uint4 *>(drow + lo_up);
        for (int64_t i = threadIdx.x; i < n2; i += (int64_t)kCopyUnroll * kCopyThreads) {
            uint4 v[kCopyUnroll];
#pragma unroll
            for (int u = 0; u < kCopyUnroll; ++u) {
                const int64_t k = i + (int64_t)u * kCopyThreads;
                if (k < n2) v[u] = s[k];
            }
#pragma unroll
            for (int u = 0; u < kCopyUnroll; ++u) {
                const int64_t k = i + (int64_t)u * kCopyThreads;
                if (k < n2) d[k] = v[u];
            }
        }
    }
}

// Pulse blocks of rows copied by a persistent grid that signals each block:
// block k holds rows [ends[k-1], ends[k]); every CTA copies its share of a
// block's rows, then counts itself done with the block; the last CTA to do
// so stores `generation` into flags[k].  A stream can then be held until
// flags[k] >= generation (sarbp_stream_wait_flag), so work on block k starts
// while later blocks are still being copied, and no kernel waits on
// another.  The copy runs on a few SMs only, leaving the rest to the work
// it feeds.
constexpr int kMaxBlocks = 32;
struct BlockEnds {
    int64_t end[kMaxBlocks];
};

// kBlockRows rows at a time, each thread holding kBlockSlots 16-byte words
// of each: a CTA keeps up to 64 KB of loads from host memory in flight
// (one row at a time kept ~13 KB, so it took ~64 SMs to fill the link).
constexpr int kBlockRows = 4;
constexpr int kBlockSlots = 4;

__global__ void __launch_bounds__(kCopyThreads)
gather_blocks16_kernel(float2 *__restrict__ dst, int64_t dpitch, const float2 *__restrict__ src,
                       int64_t spitch, int64_t lo, int64_t n, const int *__restrict__ bound,
                       int64_t max_bins, const BlockEnds ends, int nblocks,
                       unsigned *__restrict__ counters, unsigned *__restrict__ flags,
                       unsigned generation)
{
    if (bound) {
        // the inclusive bin interval [bound[0], bound[1]] (empty when
        // bound[0] > bound[1]), clipped to the rows' first max_bins bins
        __shared__ int64_t sb[2];
        if (threadIdx.x == 0) {
            const int64_t b0 = bound[0], b1 = bound[1];
            const int64_t l = b0 < 0 ? 0 : b0, h = b1 > max_bins - 1 ? max_bins - 1 : b1;
            sb[0] = l;
            sb[1] = h >= l ? h - l + 1 : 0;
        }
        __syncthreads();
        lo = sb[0];
        n = sb[1];
    }
    const int64_t lo_up = (lo + 1) & ~int64_t(1), hi = lo + n, hi_dn = hi & ~int64_t(1);
    const int64_t n2 = hi_dn > lo_up ? (hi_dn - lo_up) / 2 : 0;
    constexpr int64_t kSpan = (int64_t)kBlockSlots * kCopyThreads;
    int64_t a0 = 0;
    for (int k = 0; k < nblocks; ++k) {
        const int64_t a1 = ends.end[k];
        for (int64_t r0 = a0 + (int64_t)blockIdx.x * kBlockRows; r0 < a1;
             r0 += (int64_t)gridDim.x * kBlockRows) {
            if (n > 0 && threadIdx.x < kBlockRows && r0 + threadIdx.x < a1) {
                // the odd bins at either end of the row, as single samples
                const int64_t r = r0 + threadIdx.x;
                if (lo & 1) dst[r * dpitch + lo] = src[r * spitch + lo];
                if ((hi & 1) && hi - 1 >= lo_up) dst[r * dpitch + hi - 1] = src[r * spitch + hi - 1];
            }
            for (int64_t w0 = threadIdx.x; w0 < n2; w0 += kSpan) {
                uint4 v[kBlockRows][kBlockSlots];
#pragma unroll
                for (int g = 0; g < kBlockRows; ++g) {
                    const uint4 *s4 = reinterpret_cast<const uint4 *>(src + (r0 + g) * spitch + lo_up);
#pragma unroll
                    for (int u = 0; u < kBlockSlots; ++u) {
                        const int64_t w = w0 + (int64_t)u * kCopyThreads;
                        if (r0 + g < a1 && w < n2) v[g][u] = s4[w];
                    }
                }
#pragma unroll
                for (int g = 0; g < kBlockRows; ++g) {
                    uint4 *d4 = reinterpret_cast<uint4 *>(dst + (r0 + g) * dpitch + lo_up);
#pragma unroll
                    for (int u = 0; u < kBlockSlots; ++u) {
                        const int64_t w = w0 + (int64_t)u * kCopyThreads;
                        if (r0 + g < a1 && w < n2) d4[w] = v[g][u];
                    }
                }
            }
        }
        if (counters) {
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();                  // this CTA's rows before its count
                if (atomicAdd(&counters[k], 1u) == gridDim.x - 1) {
                    __threadfence();
                    atomicExch(&flags[k], generation);
                }
            }
        }
        a0 = a1;
    }
}

// Byte copy: 16-byte words when both ends share their alignment mod 16, the
// unaligned head and the tail byte by byte.
__global__ void __launch_bounds__(kCopyThreads)
copy_bytes_kernel(unsigned char *__restrict__ dst, const unsigned char *__restrict__ src,
                  int64_t bytes, int64_t head, int64_t nvec)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src + head);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst + head);
    for (int64_t i = tid; i < nvec; i += kCopyUnroll * stride) {
        uint4 v[kCopyUnroll];
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u)
            if (i + u * stride < nvec) v[u] = s4[i + u * stride];
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u)
            if (i + u * stride < nvec) d4[i + u * stride] = v[u];
    }
    const int64_t tail = head + nvec * 16;
    for (int64_t i = tid; i < head; i += stride) dst[i] = src[i];
    for (int64_t i = tail + tid; i < bytes; i += stride) dst[i] = src[i];
}

// CTAs of a row copy: `per_sm` per SM, at most one per row.  An upload that
// shares the SMs with focusing CTAs (the drop-in call) runs best with one
// per SM: fewer, longer-lived copy CTAs measured 4 % faster calls than two
// per SM (3.89 vs 4.07 ms on the full workload; 64 CTAs the same); on an
// otherwise idle GPU (the serving queue) more CTAs keep more loads in flight.
static int row_grid(int64_t rows, int per_sm)
{
    int dev = 0, sms = 148;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t g = (int64_t)per_sm * sms;
    return (int)(rows < g ? (rows > 0 ? rows : 1) : g);
}

// Rows [0, rows) of bins [lo, lo + n): 16-byte words where pitches and
// buffers allow, complex64 words otherwise.
static void launch_rows(float2 *dst, int64_t dpitch, const float2 *sv, int64_t spitch,
                        int64_t lo, int64_t n, int64_t rows, int per_sm, cudaStream_t stream)
{
    const bool vec = !(dpitch & 1) && !(spitch & 1) &&
                     !(reinterpret_cast<uintptr_t>(dst) & 15) &&
                     !(reinterpret_cast<uintptr_t>(sv) & 15);
    if (vec)
        gather_rows16_kernel<<<row_grid(rows, per_sm), kCopyThreads, 0, stream>>>(dst, dpitch, sv,
                                                                        spitch, lo, n, rows);
    else
        gather_rows_kernel<<<row_grid(rows, per_sm), kCopyThreads, 0, stream>>>(dst, dpitch, sv, spitch,
                                                                      lo, n, rows);
}

static int copy_grid(int64_t work_units)
{
    int dev = 0, sms = 148;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t g = 2LL * sms;
    return (int)(work_units < g ? (work_units > 0 ? work_units : 1) : g);
}

static void launch_copy_bytes(void *dst, const void *sv, int64_t bytes, cudaStream_t stream)
{
    const uintptr_t sa = reinterpret_cast<uintptr_t>(sv), da = reinterpret_cast<uintptr_t>(dst);
    int64_t head = bytes, nvec = 0;               // all bytes one by one ...
    if ((sa & 15) == (da & 15)) {                 // ... unless the ends align alike
        head = (int64_t)((16 - (sa & 15)) & 15);
        if (head > bytes) head = bytes;
        nvec = (bytes - head) / 16;
    }
    // CTAs for the 16-byte words and for the bytes copied one by one (all of
    // them when the ends are not aligned alike), 16 per thread
    const int64_t singles = bytes - nvec * 16;
    const int64_t units = (nvec + kCopyThreads - 1) / kCopyThreads +
                          (singles + 16 * kCopyThreads - 1) / (16 * kCopyThreads);
    copy_bytes_kernel<<<copy_grid(units), kCopyThreads, 0, stream>>>(
        static_cast<unsigned char *>(dst), static_cast<const unsigned char *>(sv), bytes, head,
        nvec);
}

int h2d_bytes(void *dst, const void *src, int64_t bytes, cudaStream_t stream)
{
    if (bytes <= 0) return SARBP_OK;
    if (const void *sv = device_view(src, bytes)) {
        launch_copy_bytes(dst, sv, bytes, stream);
        return cuda_status(cudaGetLastError(), "host copy (SM loads)");
    }
    return cuda_status(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyHostToDevice, stream),
                       "host copy");
}

// Rows [0, rows) of the bin interval that `bound` (int32[2], inclusive;
// device or page-locked memory, written in stream order before the copy
// runs) holds, by the four-row copy kernel on `ctas` CTAs, without
// signalling.  SARBP_EINVAL (nothing enqueued) when the source, the
// destination or the pitches do not suit its 16-byte words; the caller then
// waits for the bound and uses h2d_rows.
int h2d_rows_bound(float2 *dst, int64_t dpitch, const float2 *src, int64_t spitch,
                   const int32_t *bound, int64_t rows, int ctas, cudaStream_t stream)
{
    if (rows <= 0) return SARBP_OK;
    const void *sv = device_view(src, rows * spitch * (int64_t)sizeof(float2));
    const int *bv = static_cast<const int *>(device_view(bound, 2 * sizeof(int32_t)));
    if (!sv || !bv || (reinterpret_cast<uintptr_t>(sv) & 15) ||
        (reinterpret_cast<uintptr_t>(dst) & 15) || (dpitch & 1) || (spitch & 1) || ctas <= 0)
        return SARBP_EINVAL;
    BlockEnds e{};
    e.end[0] = rows;
    const int64_t max_bins = dpitch < spitch ? dpitch : spitch;
    gather_blocks16_kernel<<<ctas, kCopyThreads, 0, stream>>>(
        dst, dpitch, static_cast<const float2 *>(sv), spitch, 0, 0, bv, max_bins, e, 1, nullptr,
        nullptr, 0);
    return cuda_status(cudaGetLastError(), "raw rows copy (SM loads, bound on the device)");
}

int d2h_bytes(void *dst, const void *src, int64_t bytes, cudaStream_t stream)
{
    if (bytes <= 0) return SARBP_OK;
    if (const void *dv = device_view(dst, bytes, true)) {
        launch_copy_bytes(const_cast<void *>(dv), src, bytes, stream);
        return cuda_status(cudaGetLastError(), "device-to-host copy (SM stores)");
    }
    return cuda_status(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost, stream),
                       "device-to-host copy");
}

int h2d_rows(float2 *dst, int64_t dpitch, const float2 *src, int64_t spitch, int64_t lo,
             int64_t n, int64_t rows, cudaStream_t stream)
{
    if (n <= 0 || rows <= 0) return SARBP_OK;
    if (const void *sv = device_view(src, rows * spitch * (int64_t)sizeof(float2))) {
        launch_rows(dst, dpitch, static_cast<const float2 *>(sv), spitch, lo, n, rows, 4,
                    stream);
        return cuda_status(cudaGetLastError(), "raw rows copy (SM loads)");
    }
    return cuda_status(cudaMemcpy2DAsync(dst + lo, (size_t)dpitch * sizeof(float2), src + lo,
                                         (size_t)spitch * sizeof(float2),
                                         (size_t)n * sizeof(float2), (size_t)rows,
                                         cudaMemcpyHostToDevice, stream),
                       "raw rows copy");
}

}  // namespace sarbp

using namespace sarbp;

extern "C" SARBP_API int sarbp_upload_raw_bins_sm(void *dst, int64_t dst_pitch, const void *src,
                                                  int64_t src_pitch, int64_t bin_lo,
                                                  int64_t nbins, int64_t npulses, void *stream)
{
    if (!dst || !src || dst_pitch <= 0 || src_pitch <= 0 || bin_lo < 0 || nbins < 0 ||
        npulses < 0 || bin_lo + nbins > dst_pitch || bin_lo + nbins > src_pitch) {
        set_error("sarbp_upload_raw_bins_sm: bad pointers or bin range [%lld, +%lld) for "
                  "pitches %lld / %lld",
                  (long long)bin_lo, (long long)nbins, (long long)dst_pitch,
                  (long long)src_pitch);
        return SARBP_EINVAL;
    }
    if (nbins == 0 || npulses == 0) return SARBP_OK;
    const void *sv = device_view(src, npulses * src_pitch * (int64_t)sizeof(float2));
    if (!sv) {
        set_error("sarbp_upload_raw_bins_sm: the source is not page-locked host memory mapped "
                  "into the device's address space (or device memory)");
        return SARBP_EINVAL;
    }
    launch_rows(static_cast<float2 *>(dst), dst_pitch, static_cast<const float2 *>(sv), src_pitch,
                bin_lo, nbins, npulses, 1, static_cast<cudaStream_t>(stream));
    return cuda_status(cudaGetLastError(), "sarbp_upload_raw_bins_sm launch");
}

extern "C" SARBP_API int sarbp_copy_to_device_sm(void *dst, const void *src, int64_t bytes,
                                                 void *stream)
{
    if (!dst || !src || bytes < 0) {
        set_error("sarbp_copy_to_device_sm: bad pointers or size %lld", (long long)bytes);
        return SARBP_EINVAL;
    }
    if (bytes == 0) return SARBP_OK;
    const void *sv = device_view(src, bytes);
    if (!sv) {
        set_error("sarbp_copy_to_device_sm: the source is not page-locked host memory mapped "
                  "into the device's address space (or device memory)");
        return SARBP_EINVAL;
    }
    launch_copy_bytes(dst, sv, bytes, static_cast<cudaStream_t>(stream));
    return cuda_status(cudaGetLastError(), "sarbp_copy_to_device_sm launch");
}

extern "C" SARBP_API int sarbp_device_reads_pageable(void)
{
    return reads_pageable() ? 1 : 0;
}

extern "C" SARBP_API int sarbp_copy_to_host_sm(void *dst, const void *src, int64_t bytes,
                                              void *stream)
{
    if (!dst || !src || bytes < 0) {
        set_error("sarbp_copy_to_host_sm: NULL pointer or %lld bytes", (long long)bytes);
        return SARBP_EINVAL;
    }
    if (bytes == 0) return SARBP_OK;
    const void *dv = device_view(dst, bytes, true);
    if (!dv) {
        set_error("sarbp_copy_to_host_sm: the destination is neither page-locked host memory "
                  "mapped into the device's address space nor host memory this device "
                  "reaches through the host's page tables");
        return SARBP_EINVAL;
    }
    const void *sv = device_view(src, bytes);
    if (!sv) {
        set_error("sarbp_copy_to_host_sm: the source is not memory the device can load from");
        return SARBP_EINVAL;
    }
    launch_copy_bytes(const_cast<void *>(dv), sv, bytes, static_cast<cudaStream_t>(stream));
    return cuda_status(cudaGetLastError(), "sarbp_copy_to_host_sm launch");
}

extern "C" SARBP_API int sarbp_upload_host_arrays(int32_t n, void *const *dst,
                                                 const void *const *src, const int64_t *bytes,
                                                 void *stream)
{
    if (n < 0 || (n > 0 && (!dst || !src || !bytes))) {
        set_error("sarbp_upload_host_arrays: %d arrays, or a NULL list", n);
        return SARBP_EINVAL;
    }
    for (int32_t i = 0; i < n; ++i) {
        if (bytes[i] < 0 || (bytes[i] > 0 && (!dst[i] || !src[i]))) {
            set_error("sarbp_upload_host_arrays: array %d: NULL pointer or %lld bytes", i,
                      (long long)bytes[i]);
            return SARBP_EINVAL;
        }
        cudaPointerAttributes at;
        if (bytes[i] > 0 && (cudaPointerGetAttributes(&at, dst[i]) != cudaSuccess ||
                             (at.type != cudaMemoryTypeDevice &&
                              at.type != cudaMemoryTypeManaged))) {
            cudaGetLastError();
            set_error("sarbp_upload_host_arrays: array %d: the destination is not device "
                      "memory", i);
            return SARBP_EINVAL;
        }
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (int32_t i = 0; i < n; ++i) {
        const int rc = h2d_bytes(dst[i], src[i], bytes[i], s);
        if (rc) return rc;
    }
    return SARBP_OK;
}

static int upload_blocks(const char *who, void *dst, int64_t dst_pitch, const void *src,
                         int64_t src_pitch, int64_t bin_lo, int64_t nbins, const int32_t *bound,
                         const int64_t *block_ends, int32_t nblocks, uint32_t *flags,
                         uint32_t *counters, uint32_t generation, int32_t ctas, void *stream)
{
    if (!dst || !src || !block_ends || !flags || !counters || dst_pitch <= 0 || src_pitch <= 0 ||
        bin_lo < 0 || nbins < 0 || bin_lo + nbins > dst_pitch || bin_lo + nbins > src_pitch ||
        nblocks <= 0 || nblocks > kMaxBlocks || ctas <= 0 || generation == 0 ||
        (dst_pitch & 1) || (src_pitch & 1) || (reinterpret_cast<uintptr_t>(dst) & 15)) {
        set_error("%s: bad pointers, bin range [%lld, +%lld), pitches %lld / %lld (both even), "
                  "%d blocks (1..%d), %d CTAs or generation 0",
                  who, (long long)bin_lo, (long long)nbins, (long long)dst_pitch,
                  (long long)src_pitch, nblocks, kMaxBlocks, ctas);
        return SARBP_EINVAL;
    }
    BlockEnds e{};
    int64_t prev = 0;
    for (int k = 0; k < nblocks; ++k) {
        if (block_ends[k] < prev) {
            set_error("%s: block ends must not decrease", who);
            return SARBP_EINVAL;
        }
        e.end[k] = prev = block_ends[k];
    }
    const void *sv = device_view(src, prev * src_pitch * (int64_t)sizeof(float2));
    if (!sv || (reinterpret_cast<uintptr_t>(sv) & 15)) {
        set_error("%s: the source is not 16-byte aligned page-locked host memory mapped into "
                  "the device's address space (or device memory)", who);
        return SARBP_EINVAL;
    }
    const int *bv = nullptr;
    if (bound) {
        bv = static_cast<const int *>(device_view(bound, 2 * sizeof(int32_t)));
        if (!bv) {
            set_error("%s: the bound is neither device memory nor page-locked host memory", who);
            return SARBP_EINVAL;
        }
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = cuda_status(cudaMemsetAsync(counters, 0, sizeof(uint32_t) * nblocks, s), who);
    if (rc) return rc;
    const int64_t max_bins = dst_pitch < src_pitch ? dst_pitch : src_pitch;
    gather_blocks16_kernel<<<ctas, kCopyThreads, 0, s>>>(
        static_cast<float2 *>(dst), dst_pitch, static_cast<const float2 *>(sv), src_pitch, bin_lo,
        nbins, bv, max_bins, e, nblocks, counters, flags, generation);
    return cuda_status(cudaGetLastError(), who);
}

extern "C" SARBP_API int sarbp_upload_raw_blocks_sm(void *dst, int64_t dst_pitch, const void *src,
                                                   int64_t src_pitch, int64_t bin_lo,
                                                   int64_t nbins, const int64_t *block_ends,
                                                   int32_t nblocks, uint32_t *flags,
                                                   uint32_t *counters, uint32_t generation,
                                                   int32_t ctas, void *stream)
{
    if (nbins <= 0) {
        set_error("sarbp_upload_raw_blocks_sm: no bins (%lld)", (long long)nbins);
        return SARBP_EINVAL;
    }
    return upload_blocks("sarbp_upload_raw_blocks_sm", dst, dst_pitch, src, src_pitch, bin_lo,
                         nbins, nullptr, block_ends, nblocks, flags, counters, generation, ctas,
                         stream);
}

extern "C" SARBP_API int sarbp_upload_raw_blocks_bound_sm(
    void *dst, int64_t dst_pitch, const void *src, int64_t src_pitch, const int32_t *bound,
    const int64_t *block_ends, int32_t nblocks, uint32_t *flags, uint32_t *counters,
    uint32_t generation, int32_t ctas, void *stream)
{
    if (!bound) {
        set_error("sarbp_upload_raw_blocks_bound_sm: bound is NULL");
        return SARBP_EINVAL;
    }
    return upload_blocks("sarbp_upload_raw_blocks_bound_sm", dst, dst_pitch, src, src_pitch, 0,
                         0, bound, block_ends, nblocks, flags, counters, generation, ctas,
                         stream);
}

namespace {
using WaitValueFn = int (*)(void *stream, unsigned long long addr, unsigned value, unsigned flags);

WaitValueFn wait_value_fn()
{
    static WaitValueFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuStreamWaitValue32", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<WaitValueFn>(p);
    }
    return fn;
}
}  // namespace

extern "C" SARBP_API int sarbp_stream_wait_supported(void)
{
    return wait_value_fn() ? 1 : 0;
}

extern "C" SARBP_API int sarbp_stream_wait_flag(void *stream, const uint32_t *flag, uint32_t value)
{
    if (!flag) {
        set_error("sarbp_stream_wait_flag: flag is NULL");
        return SARBP_EINVAL;
    }
    auto fn = wait_value_fn();
    if (!fn) {
        set_error("sarbp_stream_wait_flag: cuStreamWaitValue32 is unavailable");
        return SARBP_ECUDA;
    }
    const unsigned kWaitGeq = 0x0;   // CU_STREAM_WAIT_VALUE_GEQ
    const int r = fn(stream, reinterpret_cast<unsigned long long>(flag), value, kWaitGeq);
    if (r != 0) {
        set_error("sarbp_stream_wait_flag: cuStreamWaitValue32 failed (CUresult %d)", r);
        return SARBP_ECUDA;
    }
    return SARBP_OK;
}
