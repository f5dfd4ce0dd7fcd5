/*
 * bp_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle results are checked against; never the product).
 *
 * CPU FP64 restatement of the reference's per-pixel time-domain
 * back-projection.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load this library; the focusing product never does.
 *
 * Followed step by step (file:line in the reference project):
 *   sar_focuser_puntual_noui.py:24-29   physical constants, float32 pi literal
 *   sar_focuser_puntual_noui.py:35-42   mask != 1 and Sint == -9999 -> 0
 *   sar_focuser_puntual_noui.py:46-55   aperture jj_size = ceil(s/2)*2+1,
 *                                       pulse a = index + j - ceil(|s|/2),
 *                                       kept iff 0 < a < Naz-1
 *   sar_focuser_puntual_noui.py:71-90   R^2, R, bin = round_half_even((R-near)/dra)
 *   sar_focuser_puntual_noui.py:95      bin kept iff 0 <= bin < Nra-1
 *   sar_focuser_puntual_noui.py:105-110 phase = (-4*pi/lambda)*R + beta*R^2,
 *                                       filter = exp(-j*phase)
 *   sar_focuser_puntual_noui.py:125-135 sum += (R^2 * raw) * filter, n += 1
 *   sar_focuser_puntual_noui.py:139-141 result = sum / n (NumPy complex128/int:
 *                                       multiply by the rounded reciprocal)
 *   sar_focuser_puntual_noui.py:183-198 F-order flattening, Sint==-9999 masking
 *
 * Every floating-point operation is a separately rounded IEEE binary64
 * operation in the reference's evaluation order; build with
 * -ffp-contract=off so that no multiply-add is fused.  cos/sin come from the
 * C library, which is what NumPy's complex exp reaches as well.
 *
 * Beside the image, the oracle can emit per-pixel contributor counts and a
 * checksum of the (pulse, range-bin) pairs that contributed, so that range-bin
 * selection can be compared bit-exactly with any other implementation.
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API __attribute__((visibility("default")))

static const double C_F64 = 2.9979246e8;           /* :24 */
static const double ALFA_F64 = 3.335987619777693e11; /* :25 */
static const double PI_F64 = 3.141592741012573242;   /* :27, float32(pi) */

/* SplitMix64 finaliser of the key (pulse << 32 | bin). */
ORACLE_API uint64_t sarbp_oracle_mix64(int64_t pulse, int64_t bin)
{
    uint64_t z = ((uint64_t)pulse << 32) | (uint64_t)(uint32_t)bin;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    const double *x, *y, *z;
    const uint8_t *mask;
    const int32_t *index, *sint;
    const double *wx, *wy, *wz;
    const float *raw;          /* interleaved (re, im); sample (r, a) at 2*(a*pitch + r) */
    int64_t nra, naz, pitch;
    double near_range, dra, lambda;
} oracle_scene;

/* One pixel: sar_focuser_puntual_noui.py:9-144. */
static void oracle_pixel(const oracle_scene *s, int64_t ii,
                         double *out, int32_t *nvalid, uint64_t *cs)
{
    const double beta = 4.0 * PI_F64 * ALFA_F64 / (C_F64 * C_F64);   /* :29 */
    const double k4pl = -4.0 * PI_F64 / s->lambda;                     /* :105 */
    double sum_re = 0.0, sum_im = 0.0;
    int64_t n = 0;
    uint64_t check = 0;

    out[0] = 0.0;
    out[1] = 0.0;
    if (nvalid) nvalid[0] = 0;
    if (cs) cs[0] = 0;

    if (s->mask[ii] != 1) return;                                      /* :35 */
    const int32_t sint = s->sint[ii];
    if (sint == -9999) return;                                         /* :41 */

    const int64_t jj_size = (int64_t)ceil((double)sint / 2.0) * 2 + 1; /* :46 */
    const int64_t off = (int64_t)ceil(fabs((double)sint) / 2.0);      /* :51 */
    const int64_t a0 = (int64_t)s->index[ii] - off;
    const double px = s->x[ii], py = s->y[ii], pz = s->z[ii];
    const double nra_m1 = (double)(s->nra - 1);

    for (int64_t j = 0; j < jj_size; ++j) {
        const int64_t a = a0 + j;
        if (!(a < s->naz - 1 && a > 0)) continue;                      /* :55 */
        const double xc = px - s->wx[a];                               /* :71-73 */
        const double yc = py - s->wy[a];
        const double zc = pz - s->wz[a];
        const double r2 = xc * xc + yc * yc + zc * zc;                 /* :77 */
        const double r = sqrt(r2);                                     /* :83 */
        const double f = (r - s->near_range) / s->dra;                 /* :89 */
        const double fb = nearbyint(f);                                /* :90 half-even */
        if (!(fb < nra_m1 && fb >= 0.0)) continue;                     /* :95 */
        const int64_t bin = (int64_t)fb;
        const double phase = k4pl * r + beta * r2;                     /* :105 */
        const double yarg = -phase;                                    /* :110 exp(-j*phase) */
        const double fc = cos(yarg), fs = sin(yarg);
        const float *rv = s->raw + 2 * (a * s->pitch + bin);           /* :131 */
        const double A = r2 * (double)rv[0];                           /* :133 R^2 * raw */
        const double B = r2 * (double)rv[1];
        sum_re += A * fc - B * fs;                                     /* :133-134 */
        sum_im += A * fs + B * fc;
        ++n;
        if (cs) check += sarbp_oracle_mix64(a, bin);
    }
    if (n > 0) {                                                       /* :139-141 */
        const double inv = 1.0 / (double)n;
        out[0] = sum_re * inv;
        out[1] = sum_im * inv;
    }
    if (nvalid) nvalid[0] = (int32_t)n;
    if (cs) cs[0] = check;
}

/*
 * Focus a list of pixels (or all pixels when `pixels` is NULL), in parallel
 * over pixels with `nthreads` OpenMP threads (<= 0: library default).
 *
 * Inputs are already flattened in column-major order and the mask already has
 * Sint == -9999 cleared (sar_focuser_puntual_noui.py:183-198); the per-pixel
 * Sint test repeats it anyway.  Output k (complex128 as two doubles, plus
 * optional count and checksum) belongs to pixels[k] (or pixel k).
 */
ORACLE_API int sarbp_oracle_focus(
    const double *x, const double *y, const double *z,
    const uint8_t *mask, const int32_t *index, const int32_t *sint,
    const double *wx, const double *wy, const double *wz,
    const float *raw, int64_t nra, int64_t naz, int64_t pitch,
    double near_range, double dra, double lambda,
    const int64_t *pixels, int64_t count,
    double *out, int32_t *nvalid, uint64_t *checksum, int nthreads)
{
    if (!x || !y || !z || !mask || !index || !sint || !wx || !wy || !wz ||
        !raw || !out || nra <= 0 || naz <= 0 || pitch < nra || count < 0)
        return -1;
    oracle_scene s = {x, y, z, mask, index, sint, wx, wy, wz, raw,
                      nra, naz, pitch, near_range, dra, lambda};
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int64_t k;
#pragma omp parallel for schedule(dynamic, 64)
    for (k = 0; k < count; ++k) {
        const int64_t ii = pixels ? pixels[k] : k;
        oracle_pixel(&s, ii, out + 2 * k, nvalid ? nvalid + k : NULL,
                     checksum ? checksum + k : NULL);
    }
    return 0;
}

ORACLE_API int sarbp_oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
