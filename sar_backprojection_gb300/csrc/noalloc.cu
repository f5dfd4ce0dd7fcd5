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
// looked up with cudaGetSymbolAddress on the first call made in a device's
// CUDA context, with that device current, and kept for that context (a
// context created after cudaDeviceReset loads the module again, at an
// address of its own, and gets its own lookup).
//
// The call reads the status block back before it returns, so a bounded
// device wait that gave up (an incomplete image) is reported as
// SARBP_ETIMEOUT by this call itself: its caller has no workspace pointer to
// hand to sarbp_mixed_status.
#include <cstring>
#include <mutex>

#include "sarbp_internal.cuh"

namespace sarbp {

// Scratch of the allocation-free entry point: the mixed path's workspace for
// up to SARBP_NOALLOC_MAX_PULSES pulses (chunk tables + status block).
constexpr size_t kNoAllocBytes = 7u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// One looked-up address per (device, context) pair seen by this process.
struct ScratchAddr {
    int dev;
    void *ctx;
    void *ptr;
};
constexpr int kMaxContexts = 64;
static std::mutex g_noalloc_mutex;
static ScratchAddr g_noalloc_addr[kMaxContexts];
static int g_noalloc_n = 0;

using CtxGetCurrentFn = int (*)(void **);

// cuCtxGetCurrent from the driver, through the runtime's entry-point query
// (the library does not link libcuda).
static CtxGetCurrentFn ctx_get_current()
{
    static CtxGetCurrentFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrentFn>(p);
    }
    return fn;
}

// Device address of the scratch array in the current device's current
// context (looked up once per context).
static int noalloc_scratch(void **out)
{
    int dev = -1;
    int rc = cuda_status(cudaGetDevice(&dev), "sarbp_focus_mixed_noalloc: cudaGetDevice");
    if (rc) return rc;
    auto get = ctx_get_current();
    if (!get) {
        set_error("sarbp_focus_mixed_noalloc: cuCtxGetCurrent is unavailable");
        return SARBP_ECUDA;
    }
    void *ctx = nullptr;
    if (get(&ctx) != 0) ctx = nullptr;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (ctx) {
        for (int k = 0; k < g_noalloc_n; ++k) {
            if (g_noalloc_addr[k].dev == dev && g_noalloc_addr[k].ctx == ctx) {
                *out = g_noalloc_addr[k].ptr;
                return SARBP_OK;
            }
        }
    }
    // the lookup also creates and binds the device's primary context when no
    // context is current yet
    void *p = nullptr;
    rc = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                     "sarbp_focus_mixed_noalloc: cudaGetSymbolAddress");
    if (rc) return rc;
    if (!ctx && (get(&ctx) != 0 || !ctx)) {
        set_error("sarbp_focus_mixed_noalloc: no CUDA context is current");
        return SARBP_ECUDA;
    }
    // a full table forgets the oldest entry (that context gets a fresh lookup)
    if (g_noalloc_n == kMaxContexts) {
        memmove(g_noalloc_addr, g_noalloc_addr + 1, sizeof(ScratchAddr) * (kMaxContexts - 1));
        --g_noalloc_n;
    }
    g_noalloc_addr[g_noalloc_n++] = ScratchAddr{dev, ctx, p};
    *out = p;
    return SARBP_OK;
}

}  // namespace sarbp

using namespace sarbp;

extern "C" SARBP_API int sarbp_focus_mixed_noalloc(const sarbp_scene *scene,
                                                   const sarbp_tuning *tuning, double *out,
                                                   int32_t *nvalid, uint64_t *checksum,
                                                   uint64_t *counters, void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
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
    rc = noalloc_scratch(&ws);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The array keeps the previous call's contents: the prepare step clears
    // the status block and rewrites the chunk tables (and the tile queue).
    rc = launch_mixed_prepare(P, T, ws, kNoAllocBytes, s);
    if (rc) return rc;
    rc = launch_mixed_main(P, T, ws, kNoAllocBytes, out, nvalid, checksum, counters, s);
    if (rc) return rc;
    // The caller cannot reach the status block: read it here (into host stack
    // memory, then wait for the stream) and report a wait that gave up.
    StatusBlock st;
    rc = cuda_status(cudaMemcpyAsync(&st, static_cast<char *>(ws) + L.status, sizeof(st),
                                     cudaMemcpyDeviceToHost, s),
                     "sarbp_focus_mixed_noalloc: status read");
    if (rc) return rc;
    rc = cuda_status(cudaStreamSynchronize(s), "sarbp_focus_mixed_noalloc: synchronize");
    if (rc) return rc;
    if (st.error) {
        set_error("sarbp_focus_mixed_noalloc: a bounded device wait gave up (site %u); the "
                  "image is incomplete",
                  st.where);
        return SARBP_ETIMEOUT;
    }
    return SARBP_OK;
}
