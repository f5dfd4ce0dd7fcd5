// noalloc.cu -- mixed-precision focusing for callers that cannot allocate
// device memory.
//
// sarbp_focus_mixed needs a few MB of scratch (the per-pulse chunk tables and
// a status block) that the caller passes in as `workspace`.  Some callers
// have no way to obtain that: a plugin loaded into a host application whose
// memory pool owns the whole device and forbids other allocations, a
// real-time pipeline that may not call cudaMalloc (it can synchronise the
// device and its latency is unbounded), or a thin binding that only receives
// the device pointers of its inputs and outputs.  For them this file keeps the
// scratch in one file-scope __device__ array, sized for scenes of up to
// SARBP_NOALLOC_MAX_PULSES pulses, that every GPU loading the library holds
// until the process exits.
//
// Host code must not hand the array's name to a kernel: in host code it is
// only a stand-in symbol, not a device address.  The device address is
// looked up with cudaGetSymbolAddress once per device, with that device
// current, on the first call made on it.
#include <cstring>
#include <mutex>

#include "sarbp_internal.cuh"

namespace sarbp {

// Scratch of the allocation-free entry point: the mixed path's workspace for
// up to SARBP_NOALLOC_MAX_PULSES pulses (chunk tables + status block).
constexpr size_t kNoAllocBytes = 7u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mutex;
static void *g_noalloc_ptr[kMaxDevices];

// Device address of the scratch array on the current device (looked up once).
static int noalloc_scratch(void **out)
{
    int dev = -1;
    int rc = cuda_status(cudaGetDevice(&dev), "sarbp_focus_mixed_noalloc: cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("sarbp_focus_mixed_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
        return SARBP_ERANGE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        rc = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                         "sarbp_focus_mixed_noalloc: cudaGetSymbolAddress");
        if (rc) return rc;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return SARBP_OK;
}

}  // namespace sarbp

using namespace sarbp;

extern "C" SARBP_API int sarbp_focus_mixed_noalloc(const sarbp_scene *scene,
                                                   const sarbp_tuning *tuning, double *out,
                                                   int32_t *nvalid, uint64_t *checksum,
                                                   uint64_t *counters, void *stream)
{
    sarbp_tuning T;
    if (tuning) {
        T = *tuning;
    } else {
        memset(&T, 0, sizeof(T));
    }
    if (!valid_tuning(&T)) return SARBP_EINVAL;
    SceneParams P;
    if (!build_params(scene, &P)) return SARBP_EINVAL;
    if (!out) {
        set_error("sarbp_focus_mixed_noalloc: out is NULL");
        return SARBP_EINVAL;
    }
    if (P.naz > SARBP_NOALLOC_MAX_PULSES) {
        set_error("sarbp_focus_mixed_noalloc: %lld pulses exceed the built-in scratch limit of "
                  "%d pulses; use sarbp_focus_mixed with a caller-supplied workspace",
                  (long long)P.naz, SARBP_NOALLOC_MAX_PULSES);
        return SARBP_ERANGE;
    }
    MixedLayout L = mixed_layout(P, T);
    if (T.staged >= 2 && L.total > kNoAllocBytes) {
        T.staged = 1;   // no room for the tile queue: one CTA per tile
        L = mixed_layout(P, T);
    }
    if (L.total > kNoAllocBytes) {
        set_error("sarbp_focus_mixed_noalloc: scene needs %zu bytes of scratch, %zu built in",
                  L.total, kNoAllocBytes);
        return SARBP_ERANGE;
    }
    void *ws = nullptr;
    int rc = noalloc_scratch(&ws);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The array keeps the previous call's contents: the status block must
    // start at zero; the chunk tables are rewritten by the prepare kernel.
    rc = cuda_status(cudaMemsetAsync(static_cast<char *>(ws) + L.status, 0, sizeof(StatusBlock), s),
                     "sarbp_focus_mixed_noalloc: status reset");
    if (rc) return rc;
    rc = launch_mixed_prepare(P, T, ws, kNoAllocBytes, s);
    if (rc) return rc;
    return launch_mixed_main(P, T, ws, kNoAllocBytes, out, nvalid, checksum, counters, s);
}
