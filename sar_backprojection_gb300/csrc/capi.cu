// capi.cu -- the extern "C" boundary: argument validation, scene constants,
// status codes and the per-thread error message.  No exception crosses it.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "sarbp_internal.cuh"

namespace sarbp {

static thread_local char g_last_error[512];

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return SARBP_OK;
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    return SARBP_ECUDA;
}

// Validate a scene and derive the kernel constants with the reference's
// evaluation order (sar_focuser_puntual_noui.py:29, :105).
bool build_params(const sarbp_scene *s, SceneParams *p)
{
    if (!s) {
        set_error("scene is NULL");
        return false;
    }
    if (s->dim0 <= 0 || s->dim1 <= 0) {
        set_error("DEM grid shape (%lld, %lld) must be positive", (long long)s->dim0,
                  (long long)s->dim1);
        return false;
    }
    if (!s->dem_x || !s->dem_y || !s->dem_z || !s->mask || !s->index || !s->sint ||
        !s->traj_x || !s->traj_y || !s->traj_z || !s->raw) {
        set_error("a scene array pointer is NULL");
        return false;
    }
    if (s->nra <= 0 || s->naz <= 0 || s->nra > 0x7fffffffLL || s->naz > 0x3fffffffLL) {
        set_error("Raw_Data shape (%lld, %lld) is outside 1..2^31-1 x 1..2^30-1",
                  (long long)s->nra, (long long)s->naz);
        return false;
    }
    if (s->raw_pitch < s->nra) {
        set_error("raw_pitch %lld is smaller than nra %lld", (long long)s->raw_pitch,
                  (long long)s->nra);
        return false;
    }
    if (!(s->delta_range != 0.0) || !(s->lambda != 0.0)) {
        set_error("delta_range and lambda must be non-zero");
        return false;
    }
    p->dim0 = s->dim0;
    p->dim1 = s->dim1;
    p->npix = s->dim0 * s->dim1;
    p->x = s->dem_x;
    p->y = s->dem_y;
    p->z = s->dem_z;
    p->mask = s->mask;
    p->index = s->index;
    p->sint = s->sint;
    p->tx = s->traj_x;
    p->ty = s->traj_y;
    p->tz = s->traj_z;
    p->raw = reinterpret_cast<const float2 *>(s->raw);
    p->nra = s->nra;
    p->naz = s->naz;
    p->pitch = s->raw_pitch;
    p->near_range = s->near_range;
    p->dra = s->delta_range;
    p->lambda = s->lambda;
    volatile double four = 4.0, pi = kPiF32, alfa = kAlfa, c = kC;
    p->beta = four * pi * alfa / (c * c);
    p->k4pl = -four * pi / s->lambda;
    p->inv_dra = 1.0 / s->delta_range;
    auto split = [](double d, float &h, float &l) {
        h = (float)d;
        l = (float)(d - (double)h);
    };
    const double two_pi = 6.283185307179586477;
    split(s->near_range, p->near_hi, p->near_lo);
    split(p->inv_dra, p->idra_hi, p->idra_lo);
    split(p->k4pl / two_pi, p->k1_hi, p->k1_lo);
    split(p->beta / two_pi, p->k2_hi, p->k2_lo);
    p->k4pl_f = (float)p->k4pl;
    p->beta_f = (float)p->beta;
    p->beta2_f = (float)(2.0 * p->beta);
    p->inv_dra_f = (float)p->inv_dra;
    auto dup = [](float v) {
        uint32_t b;
        memcpy(&b, &v, sizeof(b));
        return ((unsigned long long)b << 32) | b;
    };
    p->inv_dra_f2 = dup(p->inv_dra_f);
    p->beta_f2 = dup(p->beta_f);
    p->magic_f2 = dup(12582912.0f);   // 1.5 * 2^23: x + magic rounds x to an integer
    p->wait_polls = 1u << 22;         // staged kernels: set per launch from the tuning
    p->withhold = 0;
    return true;
}

// Library default: the TMA-staged kernel with one CTA per tile, 64-pulse
// chunks (one float-float reference per 64 pulses), 32-pulse stages, 16 x 16
// pixel tiles with a 208-bin window (two 53 KB stage buffers, still two CTAs
// per SM).  A tile whose range spread at a stage exceeds the window runs that
// stage on the scalar path with L2 reads; over rough terrain a 160-bin window
// left 2.6 % of the 4000 x 250 / 40001-pulse workload's tiles 4-7x slower
// and the whole launch 6 % slower.  On that workload 128-pulse chunks
// measure 3 % faster, but halve the pulse spacing at which the FP32 series
// gives way to the FP64 body; the cost-ordered tile queue (staged=2)
// measured slower, its order scattering neighbouring tiles in time and so
// losing the L2 reuse of their shared raw windows.
bool valid_tuning(sarbp_tuning *t)
{
    if (t->chunk == 0 && t->tile0 == 0 && t->tile1 == 0 && t->staged == 0) {
        t->chunk = 64;
        t->tile0 = 16;
        t->tile1 = 16;
        t->staged = 1;
        t->window = 208;
    }
    if (t->chunk == 0) t->chunk = 32;
    if (t->tile0 == 0 && t->tile1 == 0) {
        t->tile0 = 16;
        t->tile1 = 16;
    }
    if (t->staged && t->window == 0) t->window = (t->tile0 * t->tile1 >= 256) ? 208 : 128;
    if (t->stage == 0) t->stage = 32;
    if (t->wait_polls < 0) {
        set_error("tuning.wait_polls must be >= 0 (got %d)", t->wait_polls);
        return false;
    }
    if (t->withhold != 0 && t->withhold != 1) {
        set_error("tuning.withhold must be 0 or 1 (got %d)", t->withhold);
        return false;
    }
    if (t->stage != 16 && t->stage != 32) {
        set_error("tuning.stage must be 16 or 32 (got %d)", t->stage);
        return false;
    }
    if (t->staged < 0 || t->staged > 3) {
        set_error("tuning.staged must be 0, 1, 2 or 3 (got %d)", t->staged);
        return false;
    }
    if (t->chunk != 32 && t->chunk != 64 && !(t->staged && t->chunk == 128)) {
        set_error("tuning.chunk must be 32 or 64 (or 128 with staged > 0; got %d)", t->chunk);
        return false;
    }
    return true;
}

// Clear the thread's error, validate the scene and the tuning.
int mixed_args(const sarbp_scene *scene, const sarbp_tuning *tuning, SceneParams *P,
               sarbp_tuning *T)
{
    g_last_error[0] = 0;
    if (!build_params(scene, P)) return SARBP_EINVAL;
    *T = sarbp_tuning{};
    if (tuning) *T = *tuning;
    if (!valid_tuning(T)) return SARBP_EINVAL;
    return SARBP_OK;
}

}  // namespace sarbp

using namespace sarbp;

extern "C" {

SARBP_API int sarbp_version(void) { return 100; }

SARBP_API const char *sarbp_last_error(void) { return g_last_error; }

SARBP_API int sarbp_default_tuning(sarbp_tuning *t)
{
    if (!t) {
        set_error("tuning is NULL");
        return SARBP_EINVAL;
    }
    memset(t, 0, sizeof(*t));
    valid_tuning(t);
    return SARBP_OK;
}

SARBP_API int sarbp_focus_fp64(const sarbp_scene *scene, double *out, int32_t *nvalid,
                               uint64_t *checksum, void *stream)
{
    g_last_error[0] = 0;
    SceneParams P;
    if (!build_params(scene, &P)) return SARBP_EINVAL;
    if (!out) {
        set_error("sarbp_focus_fp64: out is NULL");
        return SARBP_EINVAL;
    }
    return launch_focus_fp64(P, out, nvalid, checksum, static_cast<cudaStream_t>(stream));
}

SARBP_API int64_t sarbp_mixed_workspace_size(const sarbp_scene *scene, const sarbp_tuning *tuning)
{
    g_last_error[0] = 0;
    SceneParams P;
    if (!build_params(scene, &P)) return SARBP_EINVAL;
    sarbp_tuning T{};
    if (tuning) T = *tuning;
    if (!valid_tuning(&T)) return SARBP_EINVAL;
    return (int64_t)mixed_layout(P, T).total;
}


SARBP_API int sarbp_mixed_prepare(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                  void *workspace, size_t workspace_bytes, void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    return launch_mixed_prepare(P, T, workspace, workspace_bytes,
                                static_cast<cudaStream_t>(stream));
}

SARBP_API int sarbp_focus_mixed_prepared(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                         double *out, int32_t *nvalid, uint64_t *checksum,
                                         uint64_t *counters, void *workspace,
                                         size_t workspace_bytes, void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    if (!out) {
        set_error("sarbp_focus_mixed: out is NULL");
        return SARBP_EINVAL;
    }
    return launch_mixed_main(P, T, workspace, workspace_bytes, out, nvalid, checksum, counters,
                             static_cast<cudaStream_t>(stream));
}

SARBP_API int sarbp_focus_mixed(const sarbp_scene *scene, const sarbp_tuning *tuning, double *out,
                                int32_t *nvalid, uint64_t *checksum, uint64_t *counters,
                                void *workspace, size_t workspace_bytes, void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    if (!out) {
        set_error("sarbp_focus_mixed: out is NULL");
        return SARBP_EINVAL;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    rc = launch_mixed_prepare(P, T, workspace, workspace_bytes, s);
    if (rc) return rc;
    return launch_mixed_main(P, T, workspace, workspace_bytes, out, nvalid, checksum, counters,
                             s);
}

SARBP_API int sarbp_mixed_status(void *workspace, size_t workspace_bytes, void *stream)
{
    if (!workspace || workspace_bytes < sizeof(StatusBlock)) {
        set_error("sarbp_mixed_status: workspace missing or too small");
        return SARBP_EWORKSPACE;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    StatusBlock st;
    int rc = cuda_status(cudaMemcpyAsync(&st, workspace, sizeof(st), cudaMemcpyDeviceToHost, s),
                         "sarbp_mixed_status: read");
    if (rc) return rc;
    rc = cuda_status(cudaStreamSynchronize(s), "sarbp_mixed_status: synchronize");
    if (rc) return rc;
    if (!st.error) return SARBP_OK;
    rc = cuda_status(cudaMemsetAsync(workspace, 0, sizeof(StatusBlock), s), "sarbp_mixed_status: clear");
    if (rc) return rc;
    set_error("mixed kernel: a bounded device wait gave up (site %u); the image is incomplete",
              st.where);
    return SARBP_ETIMEOUT;
}

SARBP_API int sarbp_raw_bin_range(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                  void *workspace, size_t workspace_bytes, int64_t *range,
                                  void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    return raw_bin_range(P, T, workspace, workspace_bytes, range,
                         static_cast<cudaStream_t>(stream));
}

SARBP_API int sarbp_raw_bin_range_async(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                        void *workspace, size_t workspace_bytes,
                                        int32_t *host_range, void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    return raw_bin_range_async(P, T, workspace, workspace_bytes, host_range,
                               static_cast<cudaStream_t>(stream));
}

SARBP_API int sarbp_upload_raw_bins(void *dst, int64_t dst_pitch, const void *src,
                                    int64_t src_pitch, int64_t bin_lo, int64_t nbins,
                                    int64_t npulses, void *stream)
{
    if (!dst || !src || dst_pitch <= 0 || src_pitch <= 0 || bin_lo < 0 || nbins < 0 ||
        npulses < 0 || bin_lo + nbins > dst_pitch || bin_lo + nbins > src_pitch) {
        set_error("sarbp_upload_raw_bins: bad pointers or bin range [%lld, +%lld) for pitches "
                  "%lld / %lld",
                  (long long)bin_lo, (long long)nbins, (long long)dst_pitch,
                  (long long)src_pitch);
        return SARBP_EINVAL;
    }
    if (nbins == 0 || npulses == 0) return SARBP_OK;
    const size_t e = 8;   // complex64
    return cuda_status(
        cudaMemcpy2DAsync(static_cast<char *>(dst) + (size_t)bin_lo * e, (size_t)dst_pitch * e,
                          static_cast<const char *>(src) + (size_t)bin_lo * e,
                          (size_t)src_pitch * e, (size_t)nbins * e, (size_t)npulses,
                          cudaMemcpyHostToDevice, static_cast<cudaStream_t>(stream)),
        "sarbp_upload_raw_bins");
}

SARBP_API int sarbp_focus_mixed_range(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                      double *out, int32_t *nvalid, uint64_t *checksum,
                                      uint64_t *counters, void *workspace,
                                      size_t workspace_bytes, int64_t first, int64_t count,
                                      void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    if (!out) {
        set_error("sarbp_focus_mixed_range: out is NULL");
        return SARBP_EINVAL;
    }
    return launch_mixed_range(P, T, workspace, workspace_bytes, first, count, out, nvalid,
                              checksum, counters, static_cast<cudaStream_t>(stream));
}

SARBP_API int sarbp_tile_queue_keys(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                    void *workspace, size_t workspace_bytes, uint32_t *keys,
                                    int64_t n, void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    return tile_queue_keys(P, T, workspace, workspace_bytes, keys, n,
                           static_cast<cudaStream_t>(stream));
}

SARBP_API int64_t sarbp_tile_count(const sarbp_scene *scene, const sarbp_tuning *tuning)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    int64_t nt = 0;
    rc = tile_count(P, T, &nt);
    return rc ? rc : nt;
}

SARBP_API int sarbp_tile_costs(const sarbp_scene *scene, const sarbp_tuning *tuning,
                               int64_t *costs, void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    if (!costs) {
        set_error("sarbp_tile_costs: costs is NULL");
        return SARBP_EINVAL;
    }
    return tile_costs(P, T, costs, static_cast<cudaStream_t>(stream));
}

SARBP_API int64_t sarbp_batch_workspace_size(int32_t nscenes, int64_t max_items)
{
    g_last_error[0] = 0;
    if (nscenes <= 0 || max_items < 0) {
        set_error("sarbp_batch_workspace_size: nscenes must be positive");
        return SARBP_EINVAL;
    }
    return batch_workspace_size(nscenes, max_items);
}

SARBP_API int sarbp_batch_set_scene(void *batch_ws, size_t batch_bytes, int32_t nscenes,
                                    int32_t slot, const sarbp_scene *scene,
                                    const sarbp_tuning *tuning, void *scene_ws,
                                    size_t scene_ws_bytes, double *out, int32_t *nvalid,
                                    uint64_t *checksum, void *stream)
{
    SceneParams P;
    sarbp_tuning T;
    int rc = mixed_args(scene, tuning, &P, &T);
    if (rc) return rc;
    return batch_set_scene(batch_ws, batch_bytes, slot, nscenes, P, T, scene_ws, scene_ws_bytes,
                           out, nvalid, checksum, static_cast<cudaStream_t>(stream));
}

SARBP_API int sarbp_batch_set_items(void *batch_ws, size_t batch_bytes, int32_t nscenes,
                                    const int32_t *items, int64_t n_items, void *stream)
{
    g_last_error[0] = 0;
    return batch_set_items(batch_ws, batch_bytes, nscenes, items, n_items,
                           static_cast<cudaStream_t>(stream));
}

SARBP_API int sarbp_batch_focus(void *batch_ws, size_t batch_bytes, int32_t nscenes,
                                const sarbp_tuning *tuning, int64_t n_items, int32_t diagnostics,
                                uint64_t *counters, void *stream)
{
    g_last_error[0] = 0;
    sarbp_tuning T{};
    if (tuning) T = *tuning;
    if (!valid_tuning(&T)) return SARBP_EINVAL;
    return batch_focus(batch_ws, batch_bytes, nscenes, T, n_items, diagnostics != 0, counters,
                       static_cast<cudaStream_t>(stream));
}

}  // extern "C"
